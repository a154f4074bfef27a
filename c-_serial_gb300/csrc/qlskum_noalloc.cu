// SSPRK stage update that allocates nothing (qlskum_state_update_noalloc).
//
// Some callers of this library cannot allocate device memory while they run:
// a host CFD code that carves every device buffer out of its own
// pre-allocated arena, or a time-stepping loop that must not pay the implicit
// device synchronisation of cudaMalloc / cudaFree between its stages.  They
// already own the state (prim, prim_old, flux_res, normals, point classes)
// and only need the update and its residual.  This entry point takes those
// device buffers, runs the same per-point update as qlskum_state_update, and
// keeps the per-block residual partials in a fixed static device array
// instead of allocated scratch.
//
// Contract:
//   * Maximum cloud size kNoallocMaxPoints = 2,097,152 points (8,192 blocks
//     of 256); larger n is rejected with QLSKUM_ERR_INVALID.  The scratch
//     array is 2 x 8,192 doubles (128 KiB) and every GPU that loads the
//     library holds it until the process exits.
//   * The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current); make
//     that first call before any stream capture.  The address is kept for
//     the life of the process: a cudaDeviceReset (or anything else that
//     destroys the device's primary context) makes it stale, and later calls
//     on that device are then invalid.
//   * Errors of the launches are reported with cudaPeekAtLastError, which
//     leaves the error state as it was: an error that the caller's own work
//     left pending is reported too, and stays visible to the caller.
//   * All calls share the one array and it keeps the previous call's
//     contents.  Each call writes every partial it later reads, so nothing has
//     to start at zero, but calls that overlap on the GPU (two streams, two
//     threads) race on the array: serialise them.
#include <cmath>
#include <cstdint>
#include <mutex>

#include "qlskum.h"
#include "qlskum_math.cuh"

namespace qlskum {
namespace noalloc {

constexpr int kBlock = 256;
constexpr int kMaxBlocks = 8192;
constexpr long long kNoallocMaxPoints = (long long)kBlock * kMaxBlocks;
static_assert(kNoallocMaxPoints == QLSKUM_NOALLOC_MAX_POINTS, "header and kernel limits differ");

// [0, kMaxBlocks): partial sums of res_sqr; [kMaxBlocks, 2 kMaxBlocks): partial maxima.
static __device__ __align__(256) double g_scratch[2 * kMaxBlocks];

__global__ void __launch_bounds__(kBlock) k_update(int n, CaseConst K, const int *__restrict__ flag,
                                                   const double2 *__restrict__ nrm, double4_32a *__restrict__ prim,
                                                   const double4_32a *__restrict__ prim_old,
                                                   const double4_32a *__restrict__ flux_res, int rk,
                                                   double *__restrict__ scratch)
{
    int i = blockIdx.x * kBlock + threadIdx.x;
    double r2 = 0.0;
    if (i < n) {
        const int f = flag[i];
        const double2 nn = nrm[i];
        double P[4], F[4];
        ld4(prim[i], P);
        ld4(flux_res[i], F);
        r2 = stage_update(K, f, nn.x, nn.y, P, prim_old + i, F, rk);
        prim[i] = mk4(P);
    }
    block_sum_max<kBlock>(r2, r2, scratch + blockIdx.x, scratch + kMaxBlocks + blockIdx.x);
}

__global__ void k_finish(int nblocks, const double *__restrict__ scratch, double *__restrict__ out)
{
    __shared__ double ss[kBlock], sm[kBlock];
    double v = 0.0, m = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kBlock) {
        v += scratch[b];
        const double t = scratch[kMaxBlocks + b];
        m = t > m ? t : m;
    }
    ss[threadIdx.x] = v;
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int s = kBlock / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            ss[threadIdx.x] += ss[threadIdx.x + s];
            sm[threadIdx.x] = sm[threadIdx.x + s] > sm[threadIdx.x] ? sm[threadIdx.x + s] : sm[threadIdx.x];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = ss[0];
        out[1] = sm[0];
    }
}

// Device address of g_scratch for each device, looked up on first use.
constexpr int kMaxDevices = 64;
static double *g_addr[kMaxDevices];
static std::mutex g_addr_mu;

static cudaError_t scratch_for_current_device(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_addr_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = static_cast<double *>(p);
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

}  // namespace noalloc
}  // namespace qlskum

using namespace qlskum;

extern "C" qlskum_status qlskum_state_update_noalloc(int n, int rk, double mach, double aoa, const int *flag_1,
                                                      const double *normals, double *prim, const double *prim_old,
                                                      const double *flux_res, double *residual_out, void *stream)
{
    if (n < 1 || (long long)n > noalloc::kNoallocMaxPoints) return QLSKUM_ERR_INVALID;
    if (rk < 1 || rk > 4) return QLSKUM_ERR_INVALID;
    if (!flag_1 || !normals || !prim || !prim_old || !flux_res || !residual_out) return QLSKUM_ERR_INVALID;
    // double4_32a / double2 loads need 32- and 16-byte aligned rows; the
    // residual is two doubles, the classes int32
    if ((reinterpret_cast<uintptr_t>(prim) | reinterpret_cast<uintptr_t>(prim_old) |
         reinterpret_cast<uintptr_t>(flux_res)) & 31u)
        return QLSKUM_ERR_INVALID;
    if (reinterpret_cast<uintptr_t>(normals) & 15u) return QLSKUM_ERR_INVALID;
    if (reinterpret_cast<uintptr_t>(residual_out) & 7u) return QLSKUM_ERR_INVALID;
    if (reinterpret_cast<uintptr_t>(flag_1) & 3u) return QLSKUM_ERR_INVALID;
    double *scratch = nullptr;
    if (noalloc::scratch_for_current_device(&scratch) != cudaSuccess) return QLSKUM_ERR_CUDA;
    CaseConst K{};
    K.pi = 4 * std::atan(1.0);
    K.rho_inf = 1.0;
    K.pr_inf = 1.0 / 1.4;
    K.gamma = 1.4;
    K.mach = mach;
    K.theta = aoa * K.pi / 180;
    K.u1_inf = mach * std::cos(K.theta);
    K.u2_inf = mach * std::sin(K.theta);
    K.cfl = 0.0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int blocks = (n + noalloc::kBlock - 1) / noalloc::kBlock;
    noalloc::k_update<<<blocks, noalloc::kBlock, 0, s>>>(
        n, K, flag_1, reinterpret_cast<const double2 *>(normals), reinterpret_cast<double4_32a *>(prim),
        reinterpret_cast<const double4_32a *>(prim_old), reinterpret_cast<const double4_32a *>(flux_res), rk, scratch);
    if (cudaPeekAtLastError() != cudaSuccess) return QLSKUM_ERR_CUDA;
    noalloc::k_finish<<<1, noalloc::kBlock, 0, s>>>(blocks, scratch, residual_out);
    return cudaPeekAtLastError() == cudaSuccess ? QLSKUM_OK : QLSKUM_ERR_CUDA;
}
