// Device helpers shared by the mixed kernels and their reverse: the 256-bit
// gather load, the cp.async copies of the staged neighbour gathers (global
// -> the thread's own shared memory; 16- and 8-byte copies need 16- / 8-byte
// aligned addresses), and the state of one edge end in the mixed form, which
// the forward flux kernel and its reverse share.  (The conversions between
// FP32 and FP64 on the integer pipe are in qlskum_math.cuh.)
#pragma once

#include <cuda_runtime.h>
#include "qlskum_math.cuh"

namespace qlskum {

// Two consecutive float4 (32 bytes) in one 256-bit load through the
// read-only path (sm_100 and later); p must be 32-byte aligned and the data
// must not be written while the kernel runs.
__device__ __forceinline__ void ldg_2x4(const float4 *p, float4 &a, float4 &b)
{
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async8(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async4(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// One end of an edge in the mixed form (interior_fluxes_mod.h:50-89 with
// limiters_mod.h:64-104, q_variables_mod.h:230-253, split_fluxes_mod.h:14-26):
// the limited reconstruction q~ = q + phi dn, dn = -(delx dqx + dely dqy) / 2
// (the reference's q - 0.5 g, with q~ - q taken as dn itself), its primitive
// state and the half-range moments in the point's (t, n) frame.  The limiter
// in the branch-free form: the common factor dn of the numerator and the
// denominator cancels, the |dn| <= 1e-5 cut is a select.  The moments take
// beta and p / rho = 1 / (2 beta) from the q~ -> prim step instead of
// dividing again, and 1 / sqrt(pi beta) from the rsqrt that gives
// sqrt(beta).  The intermediates are kept for the reverse.
struct MixedEnd {
    float dn[4], dp[4], phi[4], t[4];
    float beta, tm, u1, u2, uq, rsb, sb, S1, S2;
    Kin<float> k;
};

// DQM: mx / mn hold qmax - q / qmin - q already (the owner's end, formed once per point).
template <bool DQM = false>
__device__ __forceinline__ void mixed_end(float nx, float ny, float delx, float dely, const float q[4],
                                          const float dx[4], const float dy[4], const float mx[4],
                                          const float mn[4], float e2, MixedEnd &s)
{
    // -(delx dqx + dely dqy) / 2 with the halving on the edge vector (exact: a power of two)
    const float hx = -0.5f * delx, hy = -0.5f * dely;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const float dn = fmaf(hx, dx[r], hy * dy[r]);
        const float dp = DQM ? ((dn > 0.f) ? mx[r] : mn[r]) : ((dn > 0.f) ? mx[r] : mn[r]) - q[r];
        const float base = fmaf(dp, dp, e2);
        const float num = fmaf(2.0f * dn, dp, base);
        const float den = fmaf(dn, dp, fmaf(2.0f * dn, dn, base));
        const float ph = fminf(__fdividef(num, den), 1.0f);
        s.dn[r] = dn;
        s.dp[r] = dp;
        s.phi[r] = fabsf(dn) <= 10e-6f ? 1.0f : ph;
        s.t[r] = fmaf(s.phi[r], dn, q[r]);
    }
    s.beta = -0.5f * s.t[3];
    s.tm = __fdividef(0.5f, s.beta);
    s.u1 = s.t[1] * s.tm;
    s.u2 = s.t[2] * s.tm;
    s.uq = fmaf(s.u1, s.u1, s.u2 * s.u2);
    // rho = exp(t0 + beta |u|^2 - log(beta) / (gamma - 1)), 1 / (gamma - 1) = 2.5
    s.k.rho = __expf(fmaf(s.beta, s.uq, s.t[0]) - 2.5f * __logf(s.beta));
    s.rsb = rsqrtf(s.beta);
    s.sb = s.beta * s.rsb;
    s.k.ut = s.u1 * ny - s.u2 * nx;
    s.k.un = s.u1 * nx + s.u2 * ny;
    s.S1 = s.k.ut * s.sb;
    s.S2 = s.k.un * s.sb;
    const float e1 = __expf(-s.S1 * s.S1), e2x = __expf(-s.S2 * s.S2);
    const float half_rpi = 0.28209479177387814f;  // 1 / (2 sqrt(pi))
    s.k.B1 = half_rpi * e1 * s.rsb;
    s.k.B2 = half_rpi * e2x * s.rsb;
    s.k.E1 = erf_e<float>(s.S1, e1);
    s.k.E2 = erf_e<float>(s.S2, e2x);
    s.k.pbr = s.tm;
    s.k.usq = fmaf(s.k.ut, s.k.ut, s.k.un * s.k.un);
}

}  // namespace qlskum
