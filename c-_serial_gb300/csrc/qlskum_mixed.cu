// Mixed-precision kernels: q variables, the Venkatakrishnan limiter, the
// reconstruction and the kinetic split fluxes in FP32; the 2x2
// least-squares solves in FP64 (their determinants are near-singular on
// anisotropic wall stencils), folded on the host into per-edge FP32 weights
// for the gradient and for the four directional flux solves, so the
// near-singular inverses never meet FP32 arithmetic; the state and its
// accumulation over the SSPRK stages in FP64, and the residual norm summed
// in FP64.  Same algorithm, edge order and data layout as the FP64 kernels
// (qlskum_fp64.cu); q, dq and qm are stored in FP32, which halves the bytes
// gathered per neighbour.  Built with FMA contraction and FP32
// flush-to-zero on.
//
// On GB300 FP64 runs at about 1/64 of the FP32 rate, so the O(points) FP64
// work is kept to a minimum: the kernels add weighted flux differences
// (the folded solves); an interior point's stage change is formed in FP32
// (every term a product of the state and a change, so FP32 keeps the
// change to the relative precision F has) and added to the FP64 state; the
// wall and outer points (a few thousand, in warps of their own class) take
// the reference's conserved-variable update in FP64 with no FP64 division
// (one reciprocal from an FP32 seed and two Newton steps); the local time
// step and its wave speed are FP32 (they only set the pseudo-time step, not
// the steady state).
#include "qlskum_math.cuh"
#include "qlskum_dev.cuh"

namespace qlskum {
namespace mixed {

static inline int grid_for(int n, int block) { return (n + block - 1) / block; }

// ----------------------------------------------------- lanes per point
// A point's edges can be split over L = 1, 2 or 4 adjacent lanes of a warp
// (lane s takes edges s, s + L, ...); the lanes' partial sums, maxima and
// minima are then combined with butterfly shuffles inside the aligned group
// of L lanes, and the group's first lane finishes the point.  The groups of
// a warp are independent (a group whose point is past the end skips the
// shuffles as a whole), so the shuffle mask names the group's lanes only.
template <int L> __device__ __forceinline__ unsigned group_mask()
{
    const unsigned lane = threadIdx.x & 31u;
    return L >= 32 ? 0xffffffffu : (((1u << L) - 1u) << (lane & ~(unsigned)(L - 1)));
}

template <int L> __device__ __forceinline__ float group_sum(float v, unsigned m)
{
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v += __shfl_xor_sync(m, v, o);
    return v;
}

template <int L> __device__ __forceinline__ float group_max(float v, unsigned m)
{
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(m, v, o));
    return v;
}

template <int L> __device__ __forceinline__ float group_min(float v, unsigned m)
{
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(m, v, o));
    return v;
}

__device__ __forceinline__ void q_of(const double P[4], float Q[4])
{
    prim_to_q<float>(d2f(P[0]), d2f(P[1]), d2f(P[2]), d2f(P[3]), Q);
}

// |u| + 3 sqrt(p / rho) in FP32 (state_update_mod.h:483-485)
__device__ __forceinline__ float wave_speed32(const double P[4])
{
    const float rho = d2f(P[0]), u1 = d2f(P[1]), u2 = d2f(P[2]), p = d2f(P[3]);
    return sqrtf(u1 * u1 + u2 * u2) + 3.0f * sqrtf(__fdividef(p, rho));
}

// 1 / x in FP64 without a division: FP32 seed, two Newton steps.
__device__ __forceinline__ double recip64(double x)
{
    double r = f2d(__frcp_rn(d2f(x)));
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}

// primitive_to_conserved (state_update_mod.h:18-33) rearranged for FMA and
// without the division: 0.5 (t1^2 + t2^2) / rho == 0.5 rho |u|^2.
__device__ __forceinline__ void p2c_fast(const double P[4], double nx, double ny, double U[4])
{
    const double t1 = P[0] * P[1], t2 = P[0] * P[2];
    U[0] = P[0];
    U[3] = fma(0.5, fma(t1, P[1], t2 * P[2]), 2.5 * P[3]);
    U[1] = fma(t1, ny, -t2 * nx);
    U[2] = fma(t1, nx, t2 * ny);
}

// One SSPRK stage of one point (state_update_mod.h:111-282), FP64.
__device__ __forceinline__ double stage_update_fast(const CaseConst &K, int f, double nx, double ny, double P[4],
                                                    const double4_32a *prim_old_i, const double F[4], int rk)
{
    double U[4];
    if (f == kOuter) conserved_vector_Ubar(K, P, nx, ny, U);
    else p2c_fast(P, nx, ny, U);
    const double rho0 = U[0];
    if (rk != 3) {
#pragma unroll
        for (int j = 0; j < 4; j++) U[j] = fma(-0.5, F[j], U[j]);
    } else {
        double Po[4], Uo[4];
        ld4(*prim_old_i, Po);
        if (f == kOuter) conserved_vector_Ubar(K, Po, nx, ny, Uo);
        else p2c_fast(Po, nx, ny, Uo);
#pragma unroll
        for (int j = 0; j < 4; j++) U[j] = fma(2.0 / 3.0, Uo[j], (1.0 / 3.0) * fma(-0.5, F[j], U[j]));
    }
    if (f == kWall) U[2] = 0.;
    const double U2r = U[1], U3r = U[2];
    U[1] = fma(U2r, ny, U3r * nx);
    U[2] = fma(U3r, ny, -U2r * nx);
    const double d = U[0] - rho0;
    const double res_sqr = (f == kOuter) ? 0.0 : d * d;
    const double inv = recip64(U[0]);
    P[0] = U[0];
    P[1] = U[1] * inv;
    P[2] = U[2] * inv;
    P[3] = fma(-0.2 * inv, fma(U[1], U[1], U[2] * U[2]), 0.4 * U[3]);
    return res_sqr;
}

__global__ void k_derived(int n, const double4_32a *__restrict__ prim, float4 *__restrict__ q, float *__restrict__ cs)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double P[4];
    float Q[4];
    ld4(prim[i], P);
    q_of(P, Q);
    q[i] = mk4(Q);
    cs[i] = wave_speed32(P);
}

// Edge vector and least-squares weights of edge e: {delx, dely, w delx, w dely}.
// The gradient and inner-step kernels stream their edge arrays once per
// launch: those loads are marked evict-first (__ldcs), so that L1 and L2
// keep the gathered neighbour data instead (inner step 0.059 -> 0.055 ms on
// the 1.02 M cloud).
template <bool UW>
__device__ __forceinline__ float4 edge_w(const DevCloud &c, long long e)
{
    if (UW) {
        const float2 d = __ldcs(c.e_xy32 + e);
        return make_float4(d.x, d.y, d.x, d.y);
    }
    return __ldcs(c.e_geo32 + e);
}

// ----------------------------------------------------------- point bodies
// One point's work.  Geometry (c) and state are indexed by the point i, and
// neighbour indices from the edge list address the state directly (a
// batch's concatenated cloud carries each case's indices moved by its
// offset).

// q_variables_mod.h:36-118: FP32 differences, weighted by the FP64-folded
// per-edge solve weights (DevCloud::e_gw32); with DT (the first stage) also
// the local time step (state_update_mod.h:448-496) in FP32.
template <bool DT, int L = 1>
__device__ __forceinline__ void grad_point(const DevCloud &c, int i, const float4 *__restrict__ q,
                                           float4 *__restrict__ dq, float4 *__restrict__ qm,
                                           const float *__restrict__ cs, float *__restrict__ delta, float cfl,
                                           int sub = 0)
{
    float qi[4], qmax[4], qmin[4], dx[4] = {0, 0, 0, 0}, dy[4] = {0, 0, 0, 0};
    ld4(q[i], qi);
#pragma unroll
    for (int r = 0; r < 4; r++) { qmax[r] = qi[r]; qmin[r] = qi[r]; }
    float min_dt = 1.0f;
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    // two edges per trip: their index loads and gathers are issued together
#pragma unroll 2
    for (int j = sub; j < nb; j += L) {
        const long long e = base + 32LL * j;
        const int k = __ldcs(c.e_nbr + e);
        const float2 gw = __ldcs(c.e_gw32 + e);
        float qk[4];
        ld4(q[k], qk);
#pragma unroll
        for (int r = 0; r < 4; r++) {
            qmax[r] = fmaxf(qmax[r], qk[r]);
            qmin[r] = fminf(qmin[r], qk[r]);
            const float d = qk[r] - qi[r];
            dx[r] = fmaf(gw.x, d, dx[r]);
            dy[r] = fmaf(gw.y, d, dy[r]);
        }
        if (DT) min_dt = fminf(min_dt, cfl * __fdividef(__ldcs(c.e_dist32 + e), cs[k]));
    }
    if (L > 1) {
        const unsigned m = group_mask<L>();
#pragma unroll
        for (int r = 0; r < 4; r++) {
            dx[r] = group_sum<L>(dx[r], m);
            dy[r] = group_sum<L>(dy[r], m);
            qmax[r] = group_max<L>(qmax[r], m);
            qmin[r] = group_min<L>(qmin[r], m);
        }
        if (DT) min_dt = group_min<L>(min_dt, m);
        if (sub != 0) return;
    }
    dq[2 * i] = mk4(dx);
    dq[2 * i + 1] = mk4(dy);
    qm[2 * i] = mk4(qmax);
    qm[2 * i + 1] = mk4(qmin);
    if (DT) delta[i] = min_dt;
}

// q_variables_mod.h:120-213 in the mixed form.  The reference's sums over
// w d (t_k - t_i), t = q - 0.5 d.dq, split by linearity into three parts:
// sum w d (q_k - q_i), whose solve is the stage's first-order gradient dq0;
// sum w d (0.5 d.dq_i), whose solve is 0.5 dq_i (the solve inverts exactly
// those moments); and sum w d (d.dq_k), the only part that needs the
// neighbours.  So dq_out = dq0 + 0.5 (dq_i - solve(sum w d (d.dq_k))): the
// same value up to FP32 rounding, with one gather (dq_k) per edge instead
// of two and a quarter of the arithmetic; the solve is applied through the
// folded per-edge weights (DevCloud::e_gw32): solve(sum w d (d.dq_k)) =
// sum g_e (d.dq_k).  The FP64 form keeps the reference's order of operations.
__device__ __forceinline__ void inner_finish(const float ax[4], const float ay[4], const float4 &d0x,
                                             const float4 &d0y, const float dxi[4], const float dyi[4],
                                             float4 *__restrict__ out)
{
    const float o0[4] = {d0x.x, d0x.y, d0x.z, d0x.w}, o1[4] = {d0y.x, d0y.y, d0y.z, d0y.w};
    float rx[4], ry[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        rx[r] = fmaf(0.5f, dxi[r] - ax[r], o0[r]);
        ry[r] = fmaf(0.5f, dyi[r] - ay[r], o1[r]);
    }
    out[0] = mk4(rx);
    out[1] = mk4(ry);
}

template <bool UW, int L = 1>
__device__ __forceinline__ void inner_point(const DevCloud &c, int i, const float4 *__restrict__ dq0,
                                            const float4 *__restrict__ dq_in, float4 *__restrict__ dq_out,
                                            int sub = 0)
{
    float dxi[4], dyi[4], ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0};
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
#pragma unroll 2
    for (int j = sub; j < nb; j += L) {
        const long long e = base + 32LL * j;
        const int k = __ldcs(c.e_nbr + e);
        const float4 g = edge_w<UW>(c, e);
        const float2 gw = __ldcs(c.e_gw32 + e);
        // the neighbour's gradient pair in one 32-byte load
        float4 gx, gy;
        ldg_2x4(dq_in + 2 * k, gx, gy);
        float dxk[4], dyk[4];
        ld4(gx, dxk);
        ld4(gy, dyk);
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const float u = fmaf(g.x, dxk[r], g.y * dyk[r]);
            ax[r] = fmaf(gw.x, u, ax[r]);
            ay[r] = fmaf(gw.y, u, ay[r]);
        }
    }
    if (L > 1) {
        const unsigned m = group_mask<L>();
#pragma unroll
        for (int r = 0; r < 4; r++) {
            ax[r] = group_sum<L>(ax[r], m);
            ay[r] = group_sum<L>(ay[r], m);
        }
        if (sub != 0) return;
    }
    // the point's own gradient only after the loop: fewer registers live across it
    ld4(dq_in[2 * i], dxi);
    ld4(dq_in[2 * i + 1], dyi);
    inner_finish(ax, ay, dq0[2 * i], dq0[2 * i + 1], dxi, dyi, dq_out + 2 * i);
}

// ------------------------------------------------ staged neighbour gathers
// A thread first copies its point's edge list (neighbour index and edge
// vector: one coalesced row of the sliced-ELL arrays per edge) into shared
// memory, then streams the neighbours' data through a private ring of D + 1
// shared-memory slots with cp.async, D edges ahead of the arithmetic: the
// gathers of the next edges are in flight while the current one is
// computed, instead of one exposed gather latency per edge.  Slots are
// private to their thread, so no barrier is needed (cp.async.wait_group
// orders a thread's own copies; a slot is refilled only after the registers
// read from it were consumed).  Layout per block of B threads (field-major,
// thread-minor, conflict-free): ring [D + 1][F][B] float4, then the edge
// list, neighbour index [max_nb][B] int and edge vector [max_nb][B] float2
// (unit weights) or float4.

// bytes of dynamic shared memory of a staged kernel: F float4 fields per ring slot
constexpr size_t staged_bytes(int block, int depth, int fields, int max_nb, bool uw)
{
    return (size_t)(depth + 1) * fields * block * 16 + (size_t)max_nb * block * (4 + (uw ? 8 : 16));
}

// Edge list of point i into shared memory (neighbour index, edge vector).
template <int B, bool UW>
__device__ __forceinline__ void stage_edges(const DevCloud &c, long long base, int nb, int t, int *snbr, void *sgeo)
{
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        cp_async4(snbr + j * B + t, c.e_nbr + e);
        if (UW) cp_async8(static_cast<float2 *>(sgeo) + j * B + t, c.e_xy32 + e);
        else cp_async16(static_cast<float4 *>(sgeo) + j * B + t, c.e_geo32 + e);
    }
    cp_commit();
}

template <int B, bool UW> __device__ __forceinline__ float4 staged_geo(const void *sgeo, int j, int t)
{
    if (UW) {
        const float2 d = static_cast<const float2 *>(sgeo)[j * B + t];
        return make_float4(d.x, d.y, d.x, d.y);
    }
    return static_cast<const float4 *>(sgeo)[j * B + t];
}

// The mixed inner step (inner_point) with staged gathers (dq_x, dq_y of each neighbour).
template <int B, int D, bool UW>
__global__ void __launch_bounds__(B) k_q_inner_st(DevCloud c, const float4 *__restrict__ dq0,
                                                  const float4 *__restrict__ dq_in, float4 *__restrict__ dq_out)
{
    extern __shared__ float4 smem4[];
    float4 *ring = smem4;
    int *snbr = reinterpret_cast<int *>(ring + (D + 1) * 2 * B);
    void *sgeo = snbr + c.max_nb * B;
    const int t = threadIdx.x;
    const int i = blockIdx.x * B + t;
    if (i >= c.n) return;
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    stage_edges<B, UW>(c, base, nb, t, snbr, sgeo);
    float dxi[4], dyi[4], ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0};
    ld4(dq_in[2 * i], dxi);
    ld4(dq_in[2 * i + 1], dyi);
    cp_wait<0>();
    auto issue = [&](int j) {
        const int k = snbr[j * B + t];
        float4 *slot = ring + (j % (D + 1)) * 2 * B + t;
        cp_async16(slot, dq_in + 2 * k);
        cp_async16(slot + B, dq_in + 2 * k + 1);
    };
#pragma unroll
    for (int j = 0; j < D; j++) {
        if (j < nb) issue(j);
        cp_commit();
    }
    for (int j = 0; j < nb; j++) {
        if (j + D < nb) issue(j + D);
        cp_commit();
        cp_wait<D>();
        const float4 *slot = ring + (j % (D + 1)) * 2 * B + t;
        float dxk[4], dyk[4];
        ld4(slot[0], dxk);
        ld4(slot[B], dyk);
        const float4 g = staged_geo<B, UW>(sgeo, j, t);
        const float2 gw = c.e_gw32[base + 32LL * j];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const float u = fmaf(g.x, dxk[r], g.y * dyk[r]);
            ax[r] = fmaf(gw.x, u, ax[r]);
            ay[r] = fmaf(gw.y, u, ay[r]);
        }
    }
    inner_finish(ax, ay, dq0[2 * i], dq0[2 * i + 1], dxi, dyi, dq_out + 2 * i);
}

// q_variables_mod.h:36-118 with staged gathers (q and, in the first stage,
// the wave speed of each neighbour; the edge length for the time step).
template <int B, int D, bool UW>
__global__ void __launch_bounds__(B) k_q_derivatives_st(DevCloud c, const float4 *__restrict__ q,
                                                        float4 *__restrict__ dq, float4 *__restrict__ qm,
                                                        const float *__restrict__ cs, float *__restrict__ delta,
                                                        float cfl)
{
    extern __shared__ float4 smem4[];
    float4 *ring = smem4;                                  // [D + 1][2][B]: q, {cs, dist, -, -}
    int *snbr = reinterpret_cast<int *>(ring + (D + 1) * 2 * B);
    void *sgeo = snbr + c.max_nb * B;
    const int t = threadIdx.x;
    const int i = blockIdx.x * B + t;
    if (i >= c.n) return;
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    // the edge list: neighbour index and folded gradient weights (8 B per edge whatever the weights)
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        cp_async4(snbr + j * B + t, c.e_nbr + e);
        cp_async8(static_cast<float2 *>(sgeo) + j * B + t, c.e_gw32 + e);
    }
    cp_commit();
    float qi[4], qmax[4], qmin[4], dx[4] = {0, 0, 0, 0}, dy[4] = {0, 0, 0, 0};
    ld4(q[i], qi);
#pragma unroll
    for (int r = 0; r < 4; r++) { qmax[r] = qi[r]; qmin[r] = qi[r]; }
    float min_dt = 1.0f;
    cp_wait<0>();
    auto issue = [&](int j) {
        const int k = snbr[j * B + t];
        float4 *slot = ring + (j % (D + 1)) * 2 * B + t;
        cp_async16(slot, q + k);
        if (delta) {
            float *aux = reinterpret_cast<float *>(slot + B);
            cp_async4(aux, cs + k);
            cp_async4(aux + 1, c.e_dist32 + base + 32LL * j);
        }
    };
#pragma unroll
    for (int j = 0; j < D; j++) {
        if (j < nb) issue(j);
        cp_commit();
    }
    for (int j = 0; j < nb; j++) {
        if (j + D < nb) issue(j + D);
        cp_commit();
        cp_wait<D>();
        const float4 *slot = ring + (j % (D + 1)) * 2 * B + t;
        float qk[4];
        ld4(slot[0], qk);
        const float2 gw = static_cast<const float2 *>(sgeo)[j * B + t];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            qmax[r] = fmaxf(qmax[r], qk[r]);
            qmin[r] = fminf(qmin[r], qk[r]);
            const float d = qk[r] - qi[r];
            dx[r] = fmaf(gw.x, d, dx[r]);
            dy[r] = fmaf(gw.y, d, dy[r]);
        }
        if (delta) {
            const float4 aux = slot[B];
            min_dt = fminf(min_dt, cfl * __fdividef(aux.y, aux.x));
        }
    }
    dq[2 * i] = mk4(dx);
    dq[2 * i + 1] = mk4(dy);
    qm[2 * i] = mk4(qmax);
    qm[2 * i + 1] = mk4(qmin);
    if (delta) delta[i] = min_dt;
}

// x half-range flux of one end: split flux (interior) or the class's
// quadrant flux (wall: n half-range -, outer: +), t sign s1.
__device__ __forceinline__ void x_flux(int f, const Kin<float> &k, float s1, float G[4])
{
    if (f == kInterior) flux_x(k, s1, G);
    else flux_quad(k, s1, (f == kOuter) ? 1.0f : -1.0f, G);
}

// One interior edge end's weighted pair wx Gx(s1) + wy Gy(s2) (rho = 1),
// scaled by sc and added to acc.  Both split fluxes are linear in their
// half-range moments (split_fluxes_mod.h:14-84 and :86-164):
//   Gx = A1 a + B1 b,  Gy = A2 c + B2 b,  A = (1 + s E) / 2,  B = s B,
//   a = (ut, pbr + ut^2, ut un, ut (7 pbr + usq) / 2),
//   c = (un, ut un, pbr + un^2, un (7 pbr + usq) / 2),
//   b = (1, ut, un, (6 pbr + usq) / 2),
// so the pair is three multiply-adds per component on top of the end's
// vectors a, b, c.  hs1 / hs2 = s / 2; ws1 = wx s1, ws2 = wy s2.
__device__ __forceinline__ void interior_pair(const Kin<float> &k, float hs1, float hs2, float wx, float wy,
                                              float ws1, float ws2, float sc, float acc[4])
{
    const float A1 = fmaf(hs1, k.E1, 0.5f), A2 = fmaf(hs2, k.E2, 0.5f);
    const float al = (sc * wx) * A1, ga = (sc * wy) * A2;
    const float be = sc * fmaf(ws1, k.B1, ws2 * k.B2);
    const float utun = k.ut * k.un;
    const float h7 = 0.5f * fmaf(7.0f, k.pbr, k.usq), h6 = 0.5f * fmaf(6.0f, k.pbr, k.usq);
    const float a[4] = {k.ut, fmaf(k.ut, k.ut, k.pbr), utun, k.ut * h7};
    const float c[4] = {k.un, utun, fmaf(k.un, k.un, k.pbr), k.un * h7};
    const float b[4] = {1.0f, k.ut, k.un, h6};
#pragma unroll
    for (int r = 0; r < 4; r++) acc[r] = fmaf(al, a[r], fmaf(ga, c[r], fmaf(be, b[r], acc[r])));
}

// Flux contribution of one edge (interior_fluxes_mod.h, wall_fluxes_mod.h,
// outer_fluxes_mod.h), the owner's mxi / mni given as qmax - q / qmin - q:
// reconstruction and limiter at both ends, then the
// edge's x and y half-range fluxes, each difference Gk - Gi weighted by the
// edge's folded solve weight (DevCloud::e_w32) and added to acc.  Every edge
// lies in exactly one of xpos / xneg and one of ypos / yneg, except an edge
// with dels == 0 (deln == 0), which lies in both: the sign is chosen per
// lane, so the lanes of a warp do not diverge on their edges' sub-stencils;
// the both-sides edges take one extra (rare) pass with the second weight.
// Direction bits: 1 xpos, 2 xneg, 4 ypos, 8 yneg (the wall holds only yneg,
// the outer boundary only ypos).
__device__ __forceinline__ void flux_edge(const DevCloud &c, long long e, int f, float nx, float ny,
                                          const float qi[4], const float dxi[4], const float dyi[4],
                                          const float mxi[4], const float mni[4], float e2i, float4 g, float2 w,
                                          unsigned dir, const float qk[4], const float dxk[4], const float dyk[4],
                                          const float mxk[4], const float mnk[4], float e2k, float acc[4])
{
    MixedEnd si, sk;
    mixed_end<true>(nx, ny, g.x, g.y, qi, dxi, dyi, mxi, mni, e2i, si);
    mixed_end(nx, ny, g.x, g.y, qk, dxk, dyk, mxk, mnk, e2k, sk);
    // every component of every split / quadrant flux carries the factor rho:
    // the fluxes are evaluated with rho = 1 and rho goes into the edge weight
    Kin<float> ki = si.k, kk = sk.k;
    ki.rho = 1.0f;
    kk.rho = 1.0f;
    const float ri = si.k.rho, rk = sk.k.rho;
    float Gi[4], Gk[4];
    // x: xpos (s1 = +1) when bit 1 is set, else xneg; y: ypos (s2 = +1) when bit 4 is set, else yneg
    const float s1 = (dir & kXpos) ? 1.0f : -1.0f;
    const float s2 = (dir & kYpos) ? 1.0f : -1.0f;
    if (f == kInterior) {
        // warps are class-uniform: the interior points take the combined form
        const float hs1 = 0.5f * s1, hs2 = 0.5f * s2, ws1 = w.x * s1, ws2 = w.y * s2;
        interior_pair(ki, hs1, hs2, w.x, w.y, ws1, ws2, -ri, acc);
        interior_pair(kk, hs1, hs2, w.x, w.y, ws1, ws2, rk, acc);
    } else {
        x_flux(f, ki, s1, Gi);
        x_flux(f, kk, s1, Gk);
#pragma unroll
        for (int r = 0; r < 4; r++) acc[r] = fmaf(w.x * rk, Gk[r], fmaf(-w.x * ri, Gi[r], acc[r]));
        flux_y(ki, s2, Gi);
        flux_y(kk, s2, Gk);
#pragma unroll
        for (int r = 0; r < 4; r++) acc[r] = fmaf(w.y * rk, Gk[r], fmaf(-w.y * ri, Gi[r], acc[r]));
    }
    const bool xb = (dir & (kXpos | kXneg)) == (kXpos | kXneg), yb = (dir & (kYpos | kYneg)) == (kYpos | kYneg);
    if (xb || yb) {
        const float2 w2 = c.e_w32b[e];
        if (xb) {
            x_flux(f, ki, -1.0f, Gi);
            x_flux(f, kk, -1.0f, Gk);
#pragma unroll
            for (int r = 0; r < 4; r++) acc[r] = fmaf(w2.x * rk, Gk[r], fmaf(-w2.x * ri, Gi[r], acc[r]));
        }
        if (yb) {
            flux_y(ki, -1.0f, Gi);
            flux_y(kk, -1.0f, Gk);
#pragma unroll
            for (int r = 0; r < 4; r++) acc[r] = fmaf(w2.y * rk, Gk[r], fmaf(-w2.y * ri, Gi[r], acc[r]));
        }
    }
}

// Edge vector of edge e (delx, dely) for the reconstruction, and its folded
// solve weights.
template <bool UW>
__device__ __forceinline__ void edge_geo(const DevCloud &c, long long e, float4 &g, float2 &w)
{
    if (UW) {
        const float2 d = c.e_xy32[e];
        g = make_float4(d.x, d.y, 0.f, 0.f);
    } else {
        g = c.e_geo32[e];
    }
    w = c.e_w32[e];
}

// The SSPRK stage of an interior point (state_update_mod.h:173-232) as an
// FP32 increment added to the FP64 state.  The reference turns the state
// into conserved variables in the point's (t, n) frame, subtracts F / 2
// (stage 3: 2/3 U_old + 1/3 (U - F / 2)), turns back and divides out rho.
// The same map, written for the change of the state:
//   dU = -F / 2, or 2/3 (U_old - U) - F / 6 in stage 3, F turned back to
//   (x, y) (the frame rotation is linear, so only F needs it);
//   rho' = rho + dU0,  u' = u + (dU12 - u dU0) / rho',
//   p' = p + 0.4 (dU3 - (dU0 |u'|^2 + rho (u' + u).(u' - u)) / 2),
// with U_old - U from the FP64 differences of the primitive states:
//   rho_o u_o - rho u = (rho_o - rho) u_o + rho (u_o - u),
//   E_o - E = 2.5 (p_o - p) + ((rho_o - rho) |u_o|^2 + rho (u_o + u).(u_o - u)) / 2.
// Every term is a product of a state value and a change, so FP32 carries
// the change to FP32's relative precision (the precision F itself has);
// the state accumulates in FP64 (prim + change), so changes far below the
// state's own size are not lost.  Returns res_sqr = dU0^2.
__device__ __forceinline__ float interior_stage(const float acc[4], float dl, float nx, float ny, const double P[4],
                                                const double4_32a *__restrict__ prim_old_i, int rk, double Pn[4])
{
    const float F0 = dl * acc[0], Ft = dl * acc[1], Fn = dl * acc[2], F3 = dl * acc[3];
    const float Fx = fmaf(Ft, ny, Fn * nx), Fy = fmaf(Fn, ny, -Ft * nx);
    // the state's FP32 values and the stage-3 differences rounded to nearest
    // (a truncating conversion would bias every change the same way)
    const float rho = d2f_rn(P[0]), u1 = d2f_rn(P[1]), u2 = d2f_rn(P[2]);
    float dU0, dU1, dU2, dU3;
    if (rk != 3) {
        dU0 = -0.5f * F0;
        dU1 = -0.5f * Fx;
        dU2 = -0.5f * Fy;
        dU3 = -0.5f * F3;
    } else {
        double Po[4];
        ld4(*prim_old_i, Po);
        const float dr = d2f_rn(Po[0] - P[0]), da = d2f_rn(Po[1] - P[1]), db = d2f_rn(Po[2] - P[2]),
                    dp = d2f_rn(Po[3] - P[3]);
        const float uo1 = u1 + da, uo2 = u2 + db;
        const float W1 = fmaf(dr, uo1, rho * da), W2 = fmaf(dr, uo2, rho * db);
        const float W3 = fmaf(2.5f, dp, 0.5f * fmaf(dr, fmaf(uo1, uo1, uo2 * uo2),
                                                    rho * fmaf(uo1 + u1, da, (uo2 + u2) * db)));
        const float tt = 2.0f / 3.0f, s6 = -1.0f / 6.0f;
        dU0 = fmaf(tt, dr, s6 * F0);
        dU1 = fmaf(tt, W1, s6 * Fx);
        dU2 = fmaf(tt, W2, s6 * Fy);
        dU3 = fmaf(tt, W3, s6 * F3);
    }
    const float rn = rho + dU0;
    const float ir = __fdividef(1.0f, rn);
    const float du1 = fmaf(-u1, dU0, dU1) * ir, du2 = fmaf(-u2, dU0, dU2) * ir;
    const float un1 = u1 + du1, un2 = u2 + du2;
    const float kin = fmaf(dU0, fmaf(un1, un1, un2 * un2), rho * fmaf(u1 + un1, du1, (u2 + un2) * du2));
    const float dpr = 0.4f * fmaf(-0.5f, kin, dU3);
    Pn[0] = P[0] + f2d(dU0);
    Pn[1] = P[1] + f2d(du1);
    Pn[2] = P[2] + f2d(du2);
    Pn[3] = P[3] + f2d(dpr);
    return dU0 * dU0;
}

// F = delta * acc (the weighted sum of the folded solves, flux_residual_mod.h
// with the wall's 2 delta), then the SSPRK stage, q and the wave speed of the
// new state: interior points by the increment form above; wall and outer
// points (a few thousand, in warps of their own class) in FP64 as the
// reference writes it, an outer point of a batch with its own case's
// free-stream constants.  Returns res_sqr.
__device__ __forceinline__ float flux_tail(const DevCloud &c, const CaseConst &K, int i, int f, double2 nn,
                                           float nx, float ny,
                                           const float acc[4], const float *__restrict__ delta,
                                           const double4_32a *__restrict__ prim,
                                           const double4_32a *__restrict__ prim_old,
                                           double4_32a *__restrict__ prim_next, float4 *__restrict__ q_next,
                                           float *__restrict__ cs_next, int rk, float4 *__restrict__ acc_out)
{
    if (acc_out) acc_out[i] = mk4(acc);
    double P[4];
    ld4(prim[i], P);
    float Q[4], cs, r2;
    // q and the wave speed come from the stored FP64 state, as k_derived
    // forms them, so that a run restarted from a stored state continues
    // bit for bit
    if (f == kInterior) {
        double Pn[4];
        r2 = interior_stage(acc, delta[i], nx, ny, P, prim_old + i, rk, Pn);
        prim_next[i] = mk4(Pn);
        q_of(Pn, Q);
        cs = wave_speed32(Pn);
    } else {
        const double dl = f2d(delta[i]);
        double F[4];
#pragma unroll
        for (int r = 0; r < 4; r++) F[r] = dl * f2d(acc[r]);
        // (two calls, not a reference to either: a pointer to the launch's
        // constants would copy them to the stack)
        if (c.case_k) r2 = d2f(stage_update_fast(c.case_k[c.slice_case[i >> 5]], f, nn.x, nn.y, P, prim_old + i, F, rk));
        else r2 = d2f(stage_update_fast(K, f, nn.x, nn.y, P, prim_old + i, F, rk));
        prim_next[i] = mk4(P);
        q_of(P, Q);
        cs = wave_speed32(P);
    }
    q_next[i] = mk4(Q);
    if (cs_next) cs_next[i] = cs;
    return r2;
}

// Deterministic block reduction (sum and max) of the points' res_sqr, given
// in FP32: the sum in FP64 (each value widened exactly, the warp's 32 by
// butterfly shuffles, the warps' partial sums in a fixed order by the
// block's first thread), the maximum in FP32.  Every thread of the block
// calls it.
template <int BLOCK>
__device__ __forceinline__ void block_sum_max32(float v, double *out_sum, double *out_max)
{
    __shared__ double ss[BLOCK / 32];
    __shared__ float sm[BLOCK / 32];
    double s = f2d(v);
    float m = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        ss[w] = s;
        sm[w] = m;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = ss[0];
        float mm = sm[0];
#pragma unroll
        for (int k = 1; k < BLOCK / 32; k++) {
            t += ss[k];
            mm = fmaxf(mm, sm[k]);
        }
        *out_sum = t;
        *out_max = f2d(mm);
    }
}

// Fused stage of one point: FP32 edge work with the FP64-folded solve
// weights, then the stage update (flux_tail).
// Returns the point's res_sqr.
template <bool UW, int L = 1>
__device__ __forceinline__ float flux_point(const DevCloud &c, const CaseConst &K, int i,
                                             const float4 *__restrict__ q, const float4 *__restrict__ dq,
                                             const float4 *__restrict__ qm, const float *__restrict__ delta,
                                             const double4_32a *__restrict__ prim,
                                             const double4_32a *__restrict__ prim_old,
                                             double4_32a *__restrict__ prim_next, float4 *__restrict__ q_next,
                                             float *__restrict__ cs_next, int rk, float4 *__restrict__ acc_out,
                                             int sub = 0)
{
    const int f = c.flag[i];
    const double2 nn = c.nrm[i];
    const float nx = d2f(nn.x), ny = d2f(nn.y);
    float qi[4], dxi[4], dyi[4], mxi[4], mni[4];
    ld4(q[i], qi);
    ld4(dq[2 * i], dxi);
    ld4(dq[2 * i + 1], dyi);
    ld4(qm[2 * i], mxi);
    ld4(qm[2 * i + 1], mni);
    // the owner end's limiter reads qmax - q and qmin - q (flux_edge)
#pragma unroll
    for (int r = 0; r < 4; r++) {
        mxi[r] -= qi[r];
        mni[r] -= qi[r];
    }
    const float e2i = c.eps2_32[i];
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    for (int j = sub; j < nb; j += L) {
        const long long e = base + 32LL * j;
        const int k = c.e_nbr[e];
        float4 g;
        float2 w;
        edge_geo<UW>(c, e, g, w);
        const unsigned dir = c.e_dir[e];
        float qk[4], dxk[4], dyk[4], mxk[4], mnk[4];
        ld4(q[k], qk);
        ld4(dq[2 * k], dxk);
        ld4(dq[2 * k + 1], dyk);
        ld4(qm[2 * k], mxk);
        ld4(qm[2 * k + 1], mnk);
        flux_edge(c, e, f, nx, ny, qi, dxi, dyi, mxi, mni, e2i, g, w, dir, qk, dxk, dyk, mxk, mnk, c.eps2_32[k], acc);
    }
    if (L > 1) {
        const unsigned m = group_mask<L>();
#pragma unroll
        for (int r = 0; r < 4; r++) acc[r] = group_sum<L>(acc[r], m);
        if (sub != 0) return 0.0f;
    }
    return flux_tail(c, K, i, f, nn, nx, ny, acc, delta, prim, prim_old, prim_next, q_next, cs_next, rk, acc_out);
}

// The same with the next edge's gathers in flight during the current edge's
// arithmetic: edge j + 1's neighbour data (q, dq, qm: five float4, and the
// limiter's eps^2) goes by cp.async into a two-slot ring of the thread's own
// shared memory ([2][5][B] float4 and [2][B] float), its neighbour index is
// loaded one edge earlier still, and its streamed edge data one edge ahead
// into registers.  Same arithmetic in the same edge order as flux_point.
template <int B, bool UW>
__device__ __forceinline__ float flux_point_st(const DevCloud &c, const CaseConst &K, int i, int t,
                                                float4 *ring, float *reps, const float4 *__restrict__ q,
                                                const float4 *__restrict__ dq, const float4 *__restrict__ qm,
                                                const float *__restrict__ delta,
                                                const double4_32a *__restrict__ prim,
                                                const double4_32a *__restrict__ prim_old,
                                                double4_32a *__restrict__ prim_next, float4 *__restrict__ q_next,
                                                float *__restrict__ cs_next, int rk, float4 *__restrict__ acc_out)
{
    const int f = c.flag[i];
    const double2 nn = c.nrm[i];
    const float nx = d2f(nn.x), ny = d2f(nn.y);
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    auto issue = [&](int j, int k) {
        float4 *slot = ring + (j & 1) * 5 * B + t;
        cp_async16(slot, q + k);
        cp_async16(slot + B, dq + 2 * k);
        cp_async16(slot + 2 * B, dq + 2 * k + 1);
        cp_async16(slot + 3 * B, qm + 2 * k);
        cp_async16(slot + 4 * B, qm + 2 * k + 1);
        cp_async4(reps + (j & 1) * B + t, c.eps2_32 + k);
    };
    int kn = 0;
    float4 gn = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 wn = make_float2(0.f, 0.f);
    unsigned dn = 0;
    if (nb > 0) {
        issue(0, c.e_nbr[base]);
        edge_geo<UW>(c, base, gn, wn);
        dn = c.e_dir[base];
    }
    cp_commit();
    if (nb > 1) kn = c.e_nbr[base + 32];
    float qi[4], dxi[4], dyi[4], mxi[4], mni[4];
    ld4(q[i], qi);
    ld4(dq[2 * i], dxi);
    ld4(dq[2 * i + 1], dyi);
    ld4(qm[2 * i], mxi);
    ld4(qm[2 * i + 1], mni);
    // the owner end's limiter reads qmax - q and qmin - q (flux_edge)
#pragma unroll
    for (int r = 0; r < 4; r++) {
        mxi[r] -= qi[r];
        mni[r] -= qi[r];
    }
    const float e2i = c.eps2_32[i];
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const float4 g = gn;
        const float2 w = wn;
        const unsigned dir = dn;
        if (j + 1 < nb) {
            issue(j + 1, kn);
            edge_geo<UW>(c, e + 32, gn, wn);
            dn = c.e_dir[e + 32];
        }
        cp_commit();
        if (j + 2 < nb) kn = c.e_nbr[e + 64];
        cp_wait<1>();
        const float4 *slot = ring + (j & 1) * 5 * B + t;
        float qk[4], dxk[4], dyk[4], mxk[4], mnk[4];
        ld4(slot[0], qk);
        ld4(slot[B], dxk);
        ld4(slot[2 * B], dyk);
        ld4(slot[3 * B], mxk);
        ld4(slot[4 * B], mnk);
        const float e2k = reps[(j & 1) * B + t];
        flux_edge(c, e, f, nx, ny, qi, dxi, dyi, mxi, mni, e2i, g, w, dir, qk, dxk, dyk, mxk, mnk, e2k, acc);
    }
    return flux_tail(c, K, i, f, nn, nx, ny, acc, delta, prim, prim_old, prim_next, q_next, cs_next, rk, acc_out);
}

// Neighbour data of one edge end: q, the gradient (x, y) and the neighbour
// max / min, each pair of float4 in one 32-byte load, and the limiter's eps^2.
struct NbrData {
    float4 q, dx, dy, mx, mn;
    float e2;
};

__device__ __forceinline__ void load_nbr(const DevCloud &c, int k, const float4 *__restrict__ q,
                                         const float4 *__restrict__ dq, const float4 *__restrict__ qm, NbrData &d)
{
    d.q = q[k];
    ldg_2x4(dq + 2 * k, d.dx, d.dy);
    ldg_2x4(qm + 2 * k, d.mx, d.mn);
    d.e2 = c.eps2_32[k];
}

// The same edge walk with the next edge's gathers in registers: edge j + 1's
// neighbour data (three loads: q, and the gradient and max / min as 32-byte
// pairs) and streamed edge data are loaded while edge j is evaluated, the
// neighbour index one edge earlier still.  No shared memory: the L1 data
// path carries only the gathers themselves.  Same arithmetic in the same
// edge order as flux_point.  dq and qm must be 32-byte aligned per point
// (two float4 per point from an aligned base).
template <bool UW>
__device__ __forceinline__ float flux_point_rp(const DevCloud &c, const CaseConst &K, int i,
                                               const float4 *__restrict__ q, const float4 *__restrict__ dq,
                                               const float4 *__restrict__ qm, const float *__restrict__ delta,
                                               const double4_32a *__restrict__ prim,
                                               const double4_32a *__restrict__ prim_old,
                                               double4_32a *__restrict__ prim_next, float4 *__restrict__ q_next,
                                               float *__restrict__ cs_next, int rk, float4 *__restrict__ acc_out)
{
    const int f = c.flag[i];
    const double2 nn = c.nrm[i];
    const float nx = d2f(nn.x), ny = d2f(nn.y);
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    NbrData nd;
    float4 gn = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 wn = make_float2(0.f, 0.f);
    unsigned dn = 0;
    int kn = 0;
    if (nb > 0) {
        load_nbr(c, c.e_nbr[base], q, dq, qm, nd);
        edge_geo<UW>(c, base, gn, wn);
        dn = c.e_dir[base];
    }
    if (nb > 1) kn = c.e_nbr[base + 32];
    NbrData me;
    load_nbr(c, i, q, dq, qm, me);
    float qi[4], dxi[4], dyi[4], mxi[4], mni[4];
    ld4(me.q, qi);
    ld4(me.dx, dxi);
    ld4(me.dy, dyi);
    ld4(me.mx, mxi);
    ld4(me.mn, mni);
    // the owner end's limiter reads qmax - q and qmin - q (flux_edge)
#pragma unroll
    for (int r = 0; r < 4; r++) {
        mxi[r] -= qi[r];
        mni[r] -= qi[r];
    }
    const float e2i = me.e2;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const NbrData cur = nd;
        const float4 g = gn;
        const float2 w = wn;
        const unsigned dir = dn;
        if (j + 1 < nb) {
            load_nbr(c, kn, q, dq, qm, nd);
            edge_geo<UW>(c, e + 32, gn, wn);
            dn = c.e_dir[e + 32];
        }
        if (j + 2 < nb) kn = c.e_nbr[e + 64];
        float qk[4], dxk[4], dyk[4], mxk[4], mnk[4];
        ld4(cur.q, qk);
        ld4(cur.dx, dxk);
        ld4(cur.dy, dyk);
        ld4(cur.mx, mxk);
        ld4(cur.mn, mnk);
        flux_edge(c, e, f, nx, ny, qi, dxi, dyi, mxi, mni, e2i, g, w, dir, qk, dxk, dyk, mxk, mnk, cur.e2, acc);
    }
    return flux_tail(c, K, i, f, nn, nx, ny, acc, delta, prim, prim_old, prim_next, q_next, cs_next, rk, acc_out);
}

// A float4 from shared memory, read again at every use (volatile: not
// hoisted out of the loop into registers).
__device__ __forceinline__ void lds_v4(const float4 *p, float o[4])
{
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(o[0]), "=f"(o[1]), "=f"(o[2]), "=f"(o[3])
                 : "r"(smem_addr(p)));
}

// flux_point_rp with the owner's own data (q, gradient, qmax - q, qmin - q:
// five float4) in the thread's slots of shared memory ([5][B], thread-minor,
// conflict-free), read back at every edge instead of held in 20 registers
// across the edge loop: fewer registers, so more resident warps.
// PF false: the neighbour data is loaded at its edge, only the index and the
// streamed edge data one edge ahead (fewer registers again).
template <int B, bool UW, bool PF = true>
__device__ __forceinline__ float flux_point_rps(const DevCloud &c, const CaseConst &K, int i, int t, float4 *sown,
                                                const float4 *__restrict__ q, const float4 *__restrict__ dq,
                                                const float4 *__restrict__ qm, const float *__restrict__ delta,
                                                const double4_32a *__restrict__ prim,
                                                const double4_32a *__restrict__ prim_old,
                                                double4_32a *__restrict__ prim_next, float4 *__restrict__ q_next,
                                                float *__restrict__ cs_next, int rk, float4 *__restrict__ acc_out)
{
    const int f = c.flag[i];
    const double2 nn = c.nrm[i];
    const float nx = d2f(nn.x), ny = d2f(nn.y);
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    NbrData nd;
    float4 gn = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 wn = make_float2(0.f, 0.f);
    unsigned dn = 0;
    int kn = 0;
    int kc = 0;
    if (nb > 0) {
        kc = c.e_nbr[base];
        if (PF) load_nbr(c, kc, q, dq, qm, nd);
        edge_geo<UW>(c, base, gn, wn);
        dn = c.e_dir[base];
    }
    if (nb > 1) kn = c.e_nbr[base + 32];
    {
        NbrData me;
        load_nbr(c, i, q, dq, qm, me);
        // the owner end's limiter reads qmax - q and qmin - q (flux_edge)
        sown[t] = me.q;
        sown[B + t] = me.dx;
        sown[2 * B + t] = me.dy;
        sown[3 * B + t] = make_float4(me.mx.x - me.q.x, me.mx.y - me.q.y, me.mx.z - me.q.z, me.mx.w - me.q.w);
        sown[4 * B + t] = make_float4(me.mn.x - me.q.x, me.mn.y - me.q.y, me.mn.z - me.q.z, me.mn.w - me.q.w);
    }
    const float e2i = c.eps2_32[i];
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        NbrData cur;
        if (PF) cur = nd;
        else load_nbr(c, kc, q, dq, qm, cur);
        const float4 g = gn;
        const float2 w = wn;
        const unsigned dir = dn;
        if (j + 1 < nb) {
            if (PF) load_nbr(c, kn, q, dq, qm, nd);
            else kc = kn;
            edge_geo<UW>(c, e + 32, gn, wn);
            dn = c.e_dir[e + 32];
        }
        if (j + 2 < nb) kn = c.e_nbr[e + 64];
        float qi[4], dxi[4], dyi[4], mxi[4], mni[4];
        lds_v4(sown + t, qi);
        lds_v4(sown + B + t, dxi);
        lds_v4(sown + 2 * B + t, dyi);
        lds_v4(sown + 3 * B + t, mxi);
        lds_v4(sown + 4 * B + t, mni);
        float qk[4], dxk[4], dyk[4], mxk[4], mnk[4];
        ld4(cur.q, qk);
        ld4(cur.dx, dxk);
        ld4(cur.dy, dyk);
        ld4(cur.mx, mxk);
        ld4(cur.mn, mnk);
        flux_edge(c, e, f, nx, ny, qi, dxi, dyi, mxi, mni, e2i, g, w, dir, qk, dxk, dyk, mxk, mnk, cur.e2, acc);
    }
    return flux_tail(c, K, i, f, nn, nx, ny, acc, delta, prim, prim_old, prim_next, q_next, cs_next, rk, acc_out);
}

// ---------------------------------------------------- single-case kernels

template <bool DT, int L>
__global__ void k_q_derivatives(DevCloud c, const float4 *__restrict__ q, float4 *__restrict__ dq,
                                float4 *__restrict__ qm, const float *__restrict__ cs, float *__restrict__ delta,
                                float cfl)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = g / L;
    if (i < c.n) grad_point<DT, L>(c, i, q, dq, qm, cs, delta, cfl, g % L);
}

template <bool UW, int L>
__global__ void k_q_inner(DevCloud c, const float4 *__restrict__ dq0, const float4 *__restrict__ dq_in,
                          float4 *__restrict__ dq_out)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = g / L;
    if (i < c.n) inner_point<UW, L>(c, i, dq0, dq_in, dq_out, g % L);
}

// L lanes per point: BLOCK threads hold BLOCK / L points.
template <int BLOCK, int MINB, bool UW, int L = 1>
__global__ void __launch_bounds__(BLOCK, MINB) k_flux_update(DevCloud c, CaseConst K, const float4 *__restrict__ q,
                                                       const float4 *__restrict__ dq, const float4 *__restrict__ qm,
                                                       const float *__restrict__ delta,
                                                       const double4_32a *__restrict__ prim,
                                                       const double4_32a *__restrict__ prim_old,
                                                       double4_32a *__restrict__ prim_next, float4 *__restrict__ q_next,
                                                       float *__restrict__ cs_next, int rk,
                                                       double *__restrict__ psum, double *__restrict__ pmax,
                                                       float4 *__restrict__ acc_out)
{
    const int g = blockIdx.x * BLOCK + threadIdx.x;
    const int i = g / L;
    float r2 = 0.0f;
    if (i < c.n)
        r2 = flux_point<UW, L>(c, K, i, q, dq, qm, delta, prim, prim_old, prim_next, q_next, cs_next, rk, acc_out,
                               g % L);
    if (psum) block_sum_max32<BLOCK>(r2, psum + blockIdx.x, pmax + blockIdx.x);
}

// Staged-gather form of k_flux_update; static shared ring of the block.
template <int BLOCK, int MINB, bool UW>
__global__ void __launch_bounds__(BLOCK, MINB) k_flux_update_st(DevCloud c, CaseConst K, const float4 *__restrict__ q,
                                                          const float4 *__restrict__ dq,
                                                          const float4 *__restrict__ qm,
                                                          const float *__restrict__ delta,
                                                          const double4_32a *__restrict__ prim,
                                                          const double4_32a *__restrict__ prim_old,
                                                          double4_32a *__restrict__ prim_next,
                                                          float4 *__restrict__ q_next, float *__restrict__ cs_next,
                                                          int rk, double *__restrict__ psum,
                                                          double *__restrict__ pmax, float4 *__restrict__ acc_out)
{
    __shared__ float4 ring[2 * 5 * BLOCK];
    __shared__ float reps[2 * BLOCK];
    const int t = threadIdx.x;
    const int i = blockIdx.x * BLOCK + t;
    float r2 = 0.0f;
    if (i < c.n)
        r2 = flux_point_st<BLOCK, UW>(c, K, i, t, ring, reps, q, dq, qm, delta, prim, prim_old, prim_next, q_next,
                                      cs_next, rk, acc_out);
    if (psum) block_sum_max32<BLOCK>(r2, psum + blockIdx.x, pmax + blockIdx.x);
}

// Register-prefetch form of k_flux_update (flux_point_rp).
template <int BLOCK, int MINB, bool UW>
__global__ void __launch_bounds__(BLOCK, MINB) k_flux_update_rp(DevCloud c, CaseConst K, const float4 *__restrict__ q,
                                                          const float4 *__restrict__ dq,
                                                          const float4 *__restrict__ qm,
                                                          const float *__restrict__ delta,
                                                          const double4_32a *__restrict__ prim,
                                                          const double4_32a *__restrict__ prim_old,
                                                          double4_32a *__restrict__ prim_next,
                                                          float4 *__restrict__ q_next, float *__restrict__ cs_next,
                                                          int rk, double *__restrict__ psum,
                                                          double *__restrict__ pmax, float4 *__restrict__ acc_out)
{
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    float r2 = 0.0f;
    if (i < c.n)
        r2 = flux_point_rp<UW>(c, K, i, q, dq, qm, delta, prim, prim_old, prim_next, q_next, cs_next, rk, acc_out);
    if (psum) block_sum_max32<BLOCK>(r2, psum + blockIdx.x, pmax + blockIdx.x);
}

// Register-prefetch form with the owner's data in shared memory (flux_point_rps).
template <int BLOCK, int MINB, bool UW, bool PF = true>
__global__ void __launch_bounds__(BLOCK, MINB) k_flux_update_rps(DevCloud c, CaseConst K, const float4 *__restrict__ q,
                                                           const float4 *__restrict__ dq,
                                                           const float4 *__restrict__ qm,
                                                           const float *__restrict__ delta,
                                                           const double4_32a *__restrict__ prim,
                                                           const double4_32a *__restrict__ prim_old,
                                                           double4_32a *__restrict__ prim_next,
                                                           float4 *__restrict__ q_next, float *__restrict__ cs_next,
                                                           int rk, double *__restrict__ psum,
                                                           double *__restrict__ pmax, float4 *__restrict__ acc_out)
{
    __shared__ float4 sown[5 * BLOCK];
    const int t = threadIdx.x;
    const int i = blockIdx.x * BLOCK + t;
    float r2 = 0.0f;
    if (i < c.n)
        r2 = flux_point_rps<BLOCK, UW, PF>(c, K, i, t, sown, q, dq, qm, delta, prim, prim_old, prim_next, q_next,
                                           cs_next, rk, acc_out);
    if (psum) block_sum_max32<BLOCK>(r2, psum + blockIdx.x, pmax + blockIdx.x);
}

// ------------------------------------------------------- batched kernels
// A batch is one concatenated cloud (its cases' points at offsets that are
// multiples of kBatchAlign), run by the kernels above; these build its edge
// lists and reduce its residual per case.

__global__ void k_batch_offset_nbr(const int *__restrict__ src, int *__restrict__ dst, long long ne, int off)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < ne) dst[j] = src[j] + off;
}

__global__ void k_batch_fill_normals(double2 *__restrict__ nrm, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) nrm[i] = make_double2(0.0, 1.0);
}

// Per case: res_new = sqrt(sum of its flux blocks' partials) / n, residue against
// res_old latched at iterations 1 and 2 (fpi_solver_mod.h:138-147).
__global__ void kb_reduce(const BatchCase *__restrict__ cases, int ncases, int ti, const double *__restrict__ psum,
                          const double *__restrict__ pmax, int *iter, double *res_old, double *res_new,
                          double *hist, int capacity, int *status)
{
    __shared__ double ss[256];
    const int c = blockIdx.x;
    if (c >= ncases) return;
    const BatchCase &C = cases[c];
    double v = 0.0;
    for (int t = threadIdx.x; t < C.nblk[ti]; t += 256) v += psum[C.blk0[ti] + t];
    ss[threadIdx.x] = v;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) ss[threadIdx.x] += ss[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int it = *iter + 1;
        const double r = sqrt(ss[0]) / C.n;
        if (it <= 2) res_old[c] = r;
        res_new[c] = r;
        if (it - 1 < capacity) hist[(size_t)(it - 1) * ncases + c] = r;
        if (!isfinite(r)) atomicOr(status, 1);
    }
}

__global__ void kb_count(int *iter) { *iter += 1; }

#define QLSKUM_LAUNCHED(L) \
    do { if ((L).launches) ++*(L).launches; } while (0)

void derived(const Launch &L, const DevCloud &c, const double4_32a *prim, float4 *q, float *cspeed)
{
    k_derived<<<grid_for(c.n, 256), 256, 0, L.stream>>>(c.n, prim, q, cspeed);
    QLSKUM_LAUNCHED(L);
}

// Staged variants (threads per block, gather depth D): Launch::staged = 1..4.
const int kStagedVariants = 4;

#define QLSKUM_STAGED_SWITCH(V, ...)                                                             \
    switch (V) {                                                                                 \
    case 1: { constexpr int B_ = 128, D_ = 2; __VA_ARGS__; } break;                             \
    case 2: { constexpr int B_ = 128, D_ = 4; __VA_ARGS__; } break;                             \
    case 3: { constexpr int B_ = 256, D_ = 3; __VA_ARGS__; } break;                             \
    default: { constexpr int B_ = 64, D_ = 4; __VA_ARGS__; } break;                             \
    }

int staged_block(int v)
{
    int b = 0;
    QLSKUM_STAGED_SWITCH(v, b = B_; (void)D_)
    return b;
}

int staged_depth(int v)
{
    int d = 0;
    QLSKUM_STAGED_SWITCH(v, d = D_; (void)B_)
    return d;
}

template <typename K> static bool allow_smem(K kernel, size_t bytes)
{
    if (bytes <= 48 * 1024) return true;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess;
}

int staged_variants(const DevCloud &c)
{
    int usable = 0;
    for (int v = 1; v <= kStagedVariants; v++) {
        bool ok = true;
        QLSKUM_STAGED_SWITCH(v,
            if (c.unit_w) {
                ok = allow_smem(k_q_inner_st<B_, D_, true>, staged_bytes(B_, D_, 2, c.max_nb, true)) &&
                     allow_smem(k_q_derivatives_st<B_, D_, true>, staged_bytes(B_, D_, 2, c.max_nb, true));
            } else {
                ok = allow_smem(k_q_inner_st<B_, D_, false>, staged_bytes(B_, D_, 2, c.max_nb, false)) &&
                     allow_smem(k_q_derivatives_st<B_, D_, false>, staged_bytes(B_, D_, 2, c.max_nb, true));
            })
        if (!ok) break;
        usable = v;
    }
    cudaGetLastError();  // a refused limit is not an error of the next launch
    return usable;
}

void q_derivatives(const Launch &L, const DevCloud &c, const float4 *q, float4 *dq, float4 *qm, const float *cspeed,
                   float *delta, float cfl)
{
    if (L.staged > 0) {
        QLSKUM_STAGED_SWITCH(L.staged,
            if (c.unit_w)
                k_q_derivatives_st<B_, D_, true><<<grid_for(c.n, B_), B_, staged_bytes(B_, D_, 2, c.max_nb, true),
                                                   L.stream>>>(c, q, dq, qm, cspeed, delta, cfl);
            else
                k_q_derivatives_st<B_, D_, false><<<grid_for(c.n, B_), B_, staged_bytes(B_, D_, 2, c.max_nb, true),
                                                    L.stream>>>(c, q, dq, qm, cspeed, delta, cfl))
    } else {
#define QLSKUM_GRAD(LN)                                                                                         \
    if (delta)                                                                                                  \
        k_q_derivatives<true, LN><<<grid_for(c.n * LN, L.block), L.block, 0, L.stream>>>(c, q, dq, qm, cspeed,  \
                                                                                        delta, cfl);           \
    else                                                                                                        \
        k_q_derivatives<false, LN><<<grid_for(c.n * LN, L.block), L.block, 0, L.stream>>>(c, q, dq, qm, cspeed, \
                                                                                         delta, cfl)
        if (L.lanes == 4) { QLSKUM_GRAD(4); }
        else if (L.lanes == 2) { QLSKUM_GRAD(2); }
        else { QLSKUM_GRAD(1); }
#undef QLSKUM_GRAD
    }
    QLSKUM_LAUNCHED(L);
}

void q_inner(const Launch &L, const DevCloud &c, const float4 *dq0, const float4 *dq_in, float4 *dq_out)
{
    if (L.staged > 0) {
        QLSKUM_STAGED_SWITCH(L.staged,
            if (c.unit_w)
                k_q_inner_st<B_, D_, true><<<grid_for(c.n, B_), B_, staged_bytes(B_, D_, 2, c.max_nb, true),
                                             L.stream>>>(c, dq0, dq_in, dq_out);
            else
                k_q_inner_st<B_, D_, false><<<grid_for(c.n, B_), B_, staged_bytes(B_, D_, 2, c.max_nb, false),
                                              L.stream>>>(c, dq0, dq_in, dq_out))
    } else {
#define QLSKUM_INNER(LN)                                                                                        \
    if (c.unit_w)                                                                                               \
        k_q_inner<true, LN><<<grid_for(c.n * LN, L.block), L.block, 0, L.stream>>>(c, dq0, dq_in, dq_out);      \
    else                                                                                                        \
        k_q_inner<false, LN><<<grid_for(c.n * LN, L.block), L.block, 0, L.stream>>>(c, dq0, dq_in, dq_out)
        if (L.lanes == 4) { QLSKUM_INNER(4); }
        else if (L.lanes == 2) { QLSKUM_INNER(2); }
        else { QLSKUM_INNER(1); }
#undef QLSKUM_INNER
    }
    QLSKUM_LAUNCHED(L);
}

// Launch-shape variants of the fused kernel (threads per block, minimum
// resident blocks per SM -> register cap; 4..7 the staged-gather form; 8, 9
// the per-edge gather form with 2 / 4 lanes per point; 10..13 the
// register-prefetch form; 14, 15 the same with the owner's data in shared
// memory; 16..18 that form with only the edge index and data prefetched),
// picked by the host's autotuner.
const int kFluxVariants = 19;
static const int kFluxBlock[kFluxVariants] = {128, 128, 64, 256, 128, 128, 64, 256, 128, 256,
                                              128, 128, 64, 256, 128, 128, 128, 128, 128};
static const int kFluxMinBlocks[kFluxVariants] = {4, 5, 8, 2, 4, 5, 8, 2, 4, 2, 4, 5, 6, 2, 5, 6, 6, 7, 8};
static const int kFluxLanes[kFluxVariants] = {1, 1, 1, 1, 1, 1, 1, 1, 2, 4, 1, 1, 1, 1, 1, 1, 1, 1, 1};

int flux_variants() { return kFluxVariants; }
int flux_block(int v) { return kFluxBlock[v]; }
int flux_min_blocks(int v) { return kFluxMinBlocks[v]; }
int flux_lanes(int v) { return kFluxLanes[v]; }
int flux_grid_blocks(int v, int n) { return grid_for(n * kFluxLanes[v], kFluxBlock[v]); }

void flux_update(const Launch &L, const DevCloud &c, const CaseConst &k, const float4 *q, const float4 *dq,
                 const float4 *qm, const float *delta, const double4_32a *prim, const double4_32a *prim_old,
                 double4_32a *prim_next, float4 *q_next, float *cspeed_next, int rk, const Reduce &R, int variant,
                 float4 *acc_out)
{
#define QLSKUM_FLUX_L(B, MB, LN)                                                                            \
    if (c.unit_w)                                                                                           \
        k_flux_update<B, MB, true, LN><<<grid_for(c.n * LN, B), B, 0, L.stream>>>(                          \
            c, k, q, dq, qm, delta, prim, prim_old, prim_next, q_next, cspeed_next, rk, R.partial_sum,      \
            R.partial_max, acc_out);                                                                        \
    else                                                                                                    \
        k_flux_update<B, MB, false, LN><<<grid_for(c.n * LN, B), B, 0, L.stream>>>(                         \
            c, k, q, dq, qm, delta, prim, prim_old, prim_next, q_next, cspeed_next, rk, R.partial_sum,      \
            R.partial_max, acc_out)
#define QLSKUM_FLUX(B, MB) QLSKUM_FLUX_L(B, MB, 1)
#define QLSKUM_FLUX_ST(B, MB)                                                                               \
    if (c.unit_w)                                                                                           \
        k_flux_update_st<B, MB, true><<<grid_for(c.n, B), B, 0, L.stream>>>(c, k, q, dq, qm, delta, prim,   \
                                                                         prim_old, prim_next, q_next,      \
                                                                         cspeed_next, rk, R.partial_sum,   \
                                                                         R.partial_max, acc_out);          \
    else                                                                                                    \
        k_flux_update_st<B, MB, false><<<grid_for(c.n, B), B, 0, L.stream>>>(c, k, q, dq, qm, delta, prim,  \
                                                                          prim_old, prim_next, q_next,     \
                                                                          cspeed_next, rk, R.partial_sum,  \
                                                                          R.partial_max, acc_out)
#define QLSKUM_FLUX_RP(B, MB)                                                                               \
    if (c.unit_w)                                                                                           \
        k_flux_update_rp<B, MB, true><<<grid_for(c.n, B), B, 0, L.stream>>>(c, k, q, dq, qm, delta, prim,   \
                                                                         prim_old, prim_next, q_next,      \
                                                                         cspeed_next, rk, R.partial_sum,   \
                                                                         R.partial_max, acc_out);          \
    else                                                                                                    \
        k_flux_update_rp<B, MB, false><<<grid_for(c.n, B), B, 0, L.stream>>>(c, k, q, dq, qm, delta, prim,  \
                                                                          prim_old, prim_next, q_next,     \
                                                                          cspeed_next, rk, R.partial_sum,  \
                                                                          R.partial_max, acc_out)
#define QLSKUM_FLUX_RPS(B, MB, PF)                                                                          \
    if (c.unit_w)                                                                                           \
        k_flux_update_rps<B, MB, true, PF><<<grid_for(c.n, B), B, 0, L.stream>>>(c, k, q, dq, qm, delta,     \
                                                                              prim, prim_old, prim_next,   \
                                                                              q_next, cspeed_next, rk,     \
                                                                              R.partial_sum, R.partial_max, \
                                                                              acc_out);                    \
    else                                                                                                    \
        k_flux_update_rps<B, MB, false, PF><<<grid_for(c.n, B), B, 0, L.stream>>>(c, k, q, dq, qm, delta,    \
                                                                               prim, prim_old, prim_next,  \
                                                                               q_next, cspeed_next, rk,    \
                                                                               R.partial_sum,              \
                                                                               R.partial_max, acc_out)
    switch (variant) {
    case 1: QLSKUM_FLUX(128, 5); break;
    case 2: QLSKUM_FLUX(64, 8); break;
    case 3: QLSKUM_FLUX(256, 2); break;
    case 4: QLSKUM_FLUX_ST(128, 4); break;
    case 5: QLSKUM_FLUX_ST(128, 5); break;
    case 6: QLSKUM_FLUX_ST(64, 8); break;
    case 7: QLSKUM_FLUX_ST(256, 2); break;
    case 8: QLSKUM_FLUX_L(128, 4, 2); break;
    case 9: QLSKUM_FLUX_L(256, 2, 4); break;
    case 10: QLSKUM_FLUX_RP(128, 4); break;
    case 11: QLSKUM_FLUX_RP(128, 5); break;
    case 12: QLSKUM_FLUX_RP(64, 6); break;
    case 13: QLSKUM_FLUX_RP(256, 2); break;
    case 14: QLSKUM_FLUX_RPS(128, 5, true); break;
    case 15: QLSKUM_FLUX_RPS(128, 6, true); break;
    case 16: QLSKUM_FLUX_RPS(128, 6, false); break;
    case 17: QLSKUM_FLUX_RPS(128, 7, false); break;
    case 18: QLSKUM_FLUX_RPS(128, 8, false); break;
    default: QLSKUM_FLUX(128, 4); break;
    }
#undef QLSKUM_FLUX
#undef QLSKUM_FLUX_L
#undef QLSKUM_FLUX_ST
#undef QLSKUM_FLUX_RP
#undef QLSKUM_FLUX_RPS
    QLSKUM_LAUNCHED(L);
}

// ---------------------------------------------------- batched launchers

void batch_offset_nbr(const Launch &L, const int *src, int *dst, long long ne, int off)
{
    if (ne <= 0) return;
    k_batch_offset_nbr<<<(unsigned)((ne + 255) / 256), 256, 0, L.stream>>>(src, dst, ne, off);
    QLSKUM_LAUNCHED(L);
}

void batch_fill_normals(const Launch &L, double2 *nrm, long long n)
{
    if (n <= 0) return;
    k_batch_fill_normals<<<(unsigned)((n + 255) / 256), 256, 0, L.stream>>>(nrm, n);
    QLSKUM_LAUNCHED(L);
}

void batch_reduce(const Launch &L, const BatchView &B, int points, const double *psum, const double *pmax,
                  int *iter, double *res_old, double *res_new, double *hist, int capacity, int *status)
{
    kb_reduce<<<B.ncases, 256, 0, L.stream>>>(B.cases, B.ncases, block_index(points), psum, pmax, iter, res_old,
                                              res_new, hist, capacity, status);
    kb_count<<<1, 1, 0, L.stream>>>(iter);
    if (L.launches) *L.launches += 2;
}

}  // namespace mixed
}  // namespace qlskum
