// FP64 kernels: the drop-in form of the q-LSKUM primal iteration.
//
// Every formula is the reference's, with FMA contraction on (GB300 runs FP64
// at 1/64 of the FP32 rate, and a fused multiply-add is one FP64 instruction
// instead of two), and in the edge ends' hot arithmetic a few expressions
// rewritten to use fewer FP64 instructions for the same value to a few ulps
// (edge_qtilde / venkat_r and end_kin in qlskum_math.cuh: one reciprocal
// square root for sqrt(beta), 1 / sqrt(pi beta) and beta^-2.5, reciprocals
// instead of divisions).  The results differ from the serial reference by
// those roundings and the device's exp / log / erf: 1e-10 relative after
// 1000 iterations (the parity tests).
//
// One thread per point; the point's edges are walked in the reference's
// neighbour order from the sliced-ELL edge arrays (coalesced across the warp),
// neighbour state is gathered through L1/L2 (points are Morton ordered, so
// most neighbours of a block's points are cache-resident).  All geometry that
// does not change between iterations (edge vectors, least-squares moments,
// 1/det, limiter epsilon) is precomputed on the host in the reference's
// operation order, which on this chip trades a few bytes per edge for FP64
// instructions, its scarce resource.
#include "qlskum_math.cuh"

namespace qlskum {
namespace fp64 {

static inline int grid_for(int n, int block) { return (n + block - 1) / block; }

// ----------------------------------------------------------------- q, c

// q_variables_mod.h:9-34
__global__ void k_q_variables(int n, const double4_32a *__restrict__ prim, double4_32a *__restrict__ q)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double P[4], Q[4];
    ld4(prim[i], P);
    prim_to_q(P[0], P[1], P[2], P[3], Q);
    q[i] = mk4(Q);
}

// q and the wave speed of the current state (both read by the next stage's
// gradient kernel).
__global__ void k_derived(int n, const double4_32a *__restrict__ prim, double4_32a *__restrict__ q, double *__restrict__ cs)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double P[4], Q[4];
    ld4(prim[i], P);
    prim_to_q(P[0], P[1], P[2], P[3], Q);
    q[i] = mk4(Q);
    cs[i] = wave_speed(P);
}

// ----------------------------------------------------------- gradients

// q_variables_mod.h:36-118 (+ state_update_mod.h:448-496 when delta != null):
// qm = neighbour max/min, dq = least-squares gradient with the precomputed
// moments {sxx, syy, sxy, 1/det}.
__global__ void k_q_derivatives(DevCloud c, const double4_32a *__restrict__ q, double4_32a *__restrict__ dq,
                                double4_32a *__restrict__ qm, const double *__restrict__ cs, double *__restrict__ delta,
                                double cfl)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    double qi[4], qmax[4], qmin[4], sdx[4] = {0, 0, 0, 0}, sdy[4] = {0, 0, 0, 0};
    ld4(q[i], qi);
#pragma unroll
    for (int r = 0; r < 4; r++) { qmax[r] = qi[r]; qmin[r] = qi[r]; }
    double min_delt = 1.0;
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const int k = c.e_nbr[e];
        const double4_32a g = c.e_geo[e];
        double qk[4];
        ld4(q[k], qk);
#pragma unroll
        for (int r = 0; r < 4; r++) {
            if (qk[r] > qmax[r]) qmax[r] = qk[r];
            if (qk[r] < qmin[r]) qmin[r] = qk[r];
            sdx[r] = sdx[r] + g.z * (qk[r] - qi[r]);
            sdy[r] = sdy[r] + g.w * (qk[r] - qi[r]);
        }
        if (delta) {
            double delta_t = c.e_dist[e] / cs[k];
            delta_t = cfl * delta_t;
            if (min_delt > delta_t) min_delt = delta_t;
        }
    }
    const double4_32a m = c.ggeo[i];  // sxx, syy, sxy, 1/det
    double dx[4], dy[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        dx[r] = (sdx[r] * m.y - sdy[r] * m.z) * m.w;
        dy[r] = (sdy[r] * m.x - sdx[r] * m.z) * m.w;
    }
    dq[2 * i] = mk4(dx);
    dq[2 * i + 1] = mk4(dy);
    qm[2 * i] = mk4(qmax);
    qm[2 * i + 1] = mk4(qmin);
    if (delta) delta[i] = min_delt;
}

// q_variables_mod.h:120-213: defect-corrected gradient from q shifted half an
// edge on both ends; writes to dq_out (ping-pong replaces the copy-back of
// eval_update_innerloop).
__global__ void k_q_inner(DevCloud c, const double4_32a *__restrict__ q, const double4_32a *__restrict__ dq_in,
                          double4_32a *__restrict__ dq_out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    double qi[4], dxi[4], dyi[4], sdx[4] = {0, 0, 0, 0}, sdy[4] = {0, 0, 0, 0};
    ld4(q[i], qi);
    ld4(dq_in[2 * i], dxi);
    ld4(dq_in[2 * i + 1], dyi);
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const int k = c.e_nbr[e];
        const double4_32a g = c.e_geo[e];
        double qk[4], dxk[4], dyk[4];
        ld4(q[k], qk);
        ld4(dq_in[2 * k], dxk);
        ld4(dq_in[2 * k + 1], dyk);
#pragma unroll
        for (int r = 0; r < 4; r++) {
            double temp1 = qi[r] - 0.5 * (g.x * dxi[r] + g.y * dyi[r]);
            double temp2 = qk[r] - 0.5 * (g.x * dxk[r] + g.y * dyk[r]);
            sdx[r] = sdx[r] + (g.z * (temp2 - temp1));
            sdy[r] = sdy[r] + (g.w * (temp2 - temp1));
        }
    }
    const double4_32a m = c.ggeo[i];
    double dx[4], dy[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        dx[r] = m.w * (sdx[r] * m.y - sdy[r] * m.z);
        dy[r] = m.w * (sdy[r] * m.x - sdx[r] * m.z);
    }
    dq_out[2 * i] = mk4(dx);
    dq_out[2 * i + 1] = mk4(dy);
}

// state_update_mod.h:448-496, wave speed evaluated per edge as the reference does.
__global__ void k_func_delta(DevCloud c, const double4_32a *__restrict__ prim, double *__restrict__ delta, double cfl)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    double min_delt = 1.0;
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        double P[4];
        ld4(prim[c.e_nbr[e]], P);
        double delta_t = c.e_dist[e] / wave_speed(P);
        delta_t = cfl * delta_t;
        if (min_delt > delta_t) min_delt = delta_t;
    }
    delta[i] = min_delt;
}

// ------------------------------------------------------------- flux

// The four directional flux derivatives of point i (interior_/wall_/
// outer_fluxes_mod.h), walked edge by edge: each edge's limited end states
// are reconstructed once and feed every sub-stencil the edge belongs to,
// in the reference's neighbour order, so the sums are the reference's.
// G[d] returns the solved derivative of sub-stencil d (xpos, xneg, ypos,
// yneg); unused directions are left at 0.
// sums (or NULL): the directional sums {sx[d][0..3], sy[d][0..3]} of each d,
// 32 doubles per point, kept for the reverse's moment bars.
__device__ __forceinline__ void point_flux(const DevCloud &c, int i, int f, double nx, double ny,
                                           const double4_32a *__restrict__ q, const double4_32a *__restrict__ dq,
                                           const double4_32a *__restrict__ qm, double G[4][4],
                                           double *__restrict__ sums = nullptr, double *__restrict__ ends = nullptr,
                                           long long ns = 0)
{
    double qi[4], dxi[4], dyi[4], mxi[4], mni[4];
    ld4(q[i], qi);
    ld4(dq[2 * i], dxi);
    ld4(dq[2 * i + 1], dyi);
    ld4(qm[2 * i], mxi);
    ld4(qm[2 * i + 1], mni);
    const double e2i = c.eps2[i];
    double sx[4][4], sy[4][4];
#pragma unroll
    for (int d = 0; d < 4; d++)
#pragma unroll
        for (int r = 0; r < 4; r++) { sx[d][r] = 0.0; sy[d][r] = 0.0; }

    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const int k = c.e_nbr[e];
        const double4_32a g = c.e_geo[e];
        const double2 sw = c.e_sn[e];
        const unsigned dir = c.e_dir[e];
        double qk[4], dxk[4], dyk[4], mxk[4], mnk[4];
        ld4(q[k], qk);
        ld4(dq[2 * k], dxk);
        ld4(dq[2 * k + 1], dyk);
        ld4(qm[2 * k], mxk);
        ld4(qm[2 * k + 1], mnk);
        double ti[4], tk[4];
        edge_qtilde<double>(g.x, g.y, qi, dxi, dyi, mxi, mni, e2i, qk, dxk, dyk, mxk, mnk, c.eps2[k], ti, tk);
        Kin<double> ki, kk;
        double keep_i[3], keep_k[3];
        end_kin<double>(nx, ny, ti, ki, ends ? keep_i : nullptr);
        end_kin<double>(nx, ny, tk, kk, ends ? keep_k : nullptr);
        if (ends) {
            // planes [12][ns]: per end rho, sqrt(beta), exp(-S1^2), exp(-S2^2), erf(S1), erf(S2)
            const double v[12] = {ki.rho, keep_i[0], keep_i[1], keep_i[2], ki.E1, ki.E2,
                                  kk.rho, keep_k[0], keep_k[1], keep_k[2], kk.E1, kk.E2};
#pragma unroll
            for (int w = 0; w < 12; w++) ends[w * ns + e] = v[w];
        }
#define QLSKUM_ACC(D)                                                         \
        if (dir & (1u << D)) {                                                \
            double Gi[4], Gk[4];                                              \
            dir_flux<double, D>(f, ki, Gi);                                   \
            dir_flux<double, D>(f, kk, Gk);                                   \
            _Pragma("unroll") for (int r = 0; r < 4; r++) {                   \
                sx[D][r] = sx[D][r] + (Gk[r] - Gi[r]) * sw.x;                 \
                sy[D][r] = sy[D][r] + (Gk[r] - Gi[r]) * sw.y;                 \
            }                                                                 \
        }
        QLSKUM_ACC(0)
        QLSKUM_ACC(1)
        QLSKUM_ACC(2)
        QLSKUM_ACC(3)
#undef QLSKUM_ACC
    }
    if (sums) {
        double *o = sums + 32 * (size_t)i;
#pragma unroll
        for (int d = 0; d < 4; d++)
#pragma unroll
            for (int r = 0; r < 4; r++) {
                o[8 * d + r] = sx[d][r];
                o[8 * d + 4 + r] = sy[d][r];
            }
    }
#pragma unroll
    for (int d = 0; d < 4; d++) {
        const double4_32a m = c.fgeo[4 * i + d];  // sxx, syy, sxy, 1/det
#pragma unroll
        for (int r = 0; r < 4; r++)
            G[d][r] = (d < 2) ? (sx[d][r] * m.y - sy[d][r] * m.z) * m.w
                              : (sy[d][r] * m.x - sx[d][r] * m.z) * m.w;
    }
}

// flux_residual_mod.h:18-87
__device__ __forceinline__ void combine(int f, double delta, const double G[4][4], double F[4])
{
#pragma unroll
    for (int j = 0; j < 4; j++) {
        if (f == kWall) F[j] = (2.0 * delta) * (G[0][j] + G[1][j] + G[3][j]);
        else if (f == kInterior) F[j] = delta * (G[0][j] + G[1][j] + G[2][j] + G[3][j]);
        else F[j] = delta * (G[0][j] + G[1][j] + G[2][j]);
    }
}

__global__ void __launch_bounds__(128) k_flux_residual(DevCloud c, const double4_32a *__restrict__ q,
                                                       const double4_32a *__restrict__ dq, const double4_32a *__restrict__ qm,
                                                       const double *__restrict__ delta, double4_32a *__restrict__ flux_res,
                                                       double *__restrict__ sums, double *__restrict__ ends, long long ns)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int f = c.flag[i];
    const double2 nn = c.nrm[i];
    double G[4][4], F[4];
    point_flux(c, i, f, nn.x, nn.y, q, dq, qm, G, sums, ends, ns);
    combine(f, delta[i], G, F);
    flux_res[i] = mk4(F);
}

// state_update_mod.h:92-283 over all points, prim in place, with the
// residual partial sums of each block.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_state_update(DevCloud c, CaseConst K, double4_32a *__restrict__ prim,
                                                        const double4_32a *__restrict__ prim_old,
                                                        const double4_32a *__restrict__ flux_res, int rk,
                                                        double *__restrict__ psum, double *__restrict__ pmax)
{
    int i = blockIdx.x * BLOCK + threadIdx.x;
    double r2 = 0.0;
    if (i < c.n) {
        const int f = c.flag[i];
        const double2 nn = c.nrm[i];
        double P[4], F[4];
        ld4(prim[i], P);
        ld4(flux_res[i], F);
        r2 = stage_update(K, f, nn.x, nn.y, P, prim_old + i, F, rk);
        prim[i] = mk4(P);
    }
    block_sum_max<BLOCK>(r2, r2, psum + blockIdx.x, pmax + blockIdx.x);
}

// Fused stage: flux residual + SSPRK update of point i, then q and (after the
// last stage) the wave speed of the new state for the next stage's kernels.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_flux_update(DevCloud c, CaseConst K, const double4_32a *__restrict__ q,
                                                       const double4_32a *__restrict__ dq,
                                                       const double4_32a *__restrict__ qm,
                                                       const double *__restrict__ delta,
                                                       const double4_32a *__restrict__ prim,
                                                       const double4_32a *__restrict__ prim_old,
                                                       double4_32a *__restrict__ prim_next, double4_32a *__restrict__ q_next,
                                                       double *__restrict__ cs_next, int rk,
                                                       double *__restrict__ psum, double *__restrict__ pmax)
{
    int i = blockIdx.x * BLOCK + threadIdx.x;
    double r2 = 0.0;
    if (i < c.n) {
        const int f = c.flag[i];
        const double2 nn = c.nrm[i];
        double G[4][4], F[4], P[4], Q[4];
        point_flux(c, i, f, nn.x, nn.y, q, dq, qm, G);
        combine(f, delta[i], G, F);
        ld4(prim[i], P);
        r2 = stage_update(K, f, nn.x, nn.y, P, prim_old + i, F, rk);
        prim_next[i] = mk4(P);
        prim_to_q(P[0], P[1], P[2], P[3], Q);
        q_next[i] = mk4(Q);
        if (cs_next) cs_next[i] = wave_speed(P);
    }
    if (psum) block_sum_max<BLOCK>(r2, r2, psum + blockIdx.x, pmax + blockIdx.x);
}

// fpi_solver_mod.h:138-147: res_new = sqrt(sum)/n, residue against res_old
// latched at iterations 1 and 2; one block, fixed summation order.
// One block of RB threads: each thread sums a strided share of the block
// partials with four independent accumulators (its loads in flight together
// instead of one dependent chain), then a tree over the block; the order is
// fixed, so the result is the same on every run.
constexpr int RB = 1024;
__global__ void __launch_bounds__(RB) k_reduce_residual(int nblocks, const double *__restrict__ psum,
                                                       const double *__restrict__ pmax, int n, int it_arg,
                                                       double *hist, int capacity, double *res_old, int *iter,
                                                       int *status, int latch)
{
    __shared__ double ss[RB], sm[RB];
    double v[4] = {0.0, 0.0, 0.0, 0.0}, mm[4] = {0.0, 0.0, 0.0, 0.0};
    int b = threadIdx.x;
    for (; b + 3 * RB < nblocks; b += 4 * RB) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            v[u] += psum[b + u * RB];
            const double x = pmax[b + u * RB];
            mm[u] = x > mm[u] ? x : mm[u];
        }
    }
    for (; b < nblocks; b += RB) {
        v[0] += psum[b];
        mm[0] = pmax[b] > mm[0] ? pmax[b] : mm[0];
    }
    double m = mm[0];
    for (int u = 1; u < 4; u++) m = mm[u] > m ? mm[u] : m;
    ss[threadIdx.x] = (v[0] + v[1]) + (v[2] + v[3]);
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int s = RB / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            ss[threadIdx.x] += ss[threadIdx.x + s];
            sm[threadIdx.x] = sm[threadIdx.x + s] > sm[threadIdx.x] ? sm[threadIdx.x + s] : sm[threadIdx.x];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        int it = it_arg > 0 ? it_arg : *iter + 1;
        double res_new = sqrt(ss[0]) / n;
        double residue;
        if (it <= 2 && latch) {
            *res_old = res_new;
            residue = 0;
        } else {
            residue = log10(res_new / *res_old);
        }
        if (it - 1 < capacity && it >= 1) {
            hist[3 * (it - 1)] = res_new;
            hist[3 * (it - 1) + 1] = residue;
            hist[3 * (it - 1) + 2] = sm[0];
        }
        *iter = it;
        if (!isfinite(res_new)) *status = 1;
    }
}

__global__ void k_copy(int n, const double4_32a *__restrict__ src, double4_32a *__restrict__ dst)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}

// Point states between the cloud's order and the handle's (Morton / class)
// order: dst[perm[i]] = src[i] (in) or dst[i] = src[perm[i]] (out).
__global__ void k_permute_in(int n, const int *__restrict__ perm, const double4_32a *__restrict__ src,
                             double4_32a *__restrict__ dst)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[perm[i]] = src[i];
}

__global__ void k_permute_out(int n, const int *__restrict__ perm, const double4_32a *__restrict__ src,
                              double4_32a *__restrict__ dst)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[perm[i]];
}

__global__ void k_add(int n, const double4_32a *__restrict__ src, double4_32a *__restrict__ dst)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double4_32a a = src[i], b = dst[i];
        dst[i] = make_double4_32a(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
    }
}

// compute_force_coeffs_mod.h:37-72 per shape point and compute_entropy_mod.h:
// 17-21 per point; each block writes its partial sums of H, V, pitching
// moment and entropy, k_objective_finish adds the partials in a fixed order.
// wall_geo per shape point: x = ds, y = mx - 0.25, z = my.
__global__ void __launch_bounds__(256) k_objective(DevCloud c, const double4_32a *__restrict__ prim,
                                                   const int *__restrict__ wall_perm,
                                                   const double4_32a *__restrict__ wall_geo, int n_wall,
                                                   double cp_scale, double pr_inf, double gamma,
                                                   double *__restrict__ entropy, double *__restrict__ partial)
{
    __shared__ double sh[4][256];
    const int t = blockIdx.x * 256 + threadIdx.x;
    double H = 0, V = 0, Mo = 0, E = 0;
    if (t < n_wall) {
        const int m = wall_perm[t];
        const double4_32a w = wall_geo[t];
        const double2 nn = c.nrm[m];
        double cp = prim[m].w - pr_inf;
        cp = -cp / cp_scale;
        H = cp * nn.x * w.x;
        V = cp * nn.y * w.x;
        Mo = (-cp * nn.y * w.x * w.y + cp * nn.x * w.x * w.z);
    }
    if (entropy && t < c.n) {
        const double4_32a P = prim[t];
        double temp1 = pow(P.x, gamma);
        temp1 = P.w / temp1;
        temp1 = log(temp1);
        const double s = fabs(temp1 - log(pr_inf));
        entropy[t] = s;
        E = s;
    }
    sh[0][threadIdx.x] = H;
    sh[1][threadIdx.x] = V;
    sh[2][threadIdx.x] = Mo;
    sh[3][threadIdx.x] = E;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st)
            for (int q = 0; q < 4; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x < 4) partial[4 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_objective_finish(int nblocks, const double *__restrict__ partial, double *__restrict__ out4)
{
    __shared__ double sh[4][256];
    double v[4] = {0, 0, 0, 0};
    for (int b = threadIdx.x; b < nblocks; b += 256)
        for (int q = 0; q < 4; q++) v[q] += partial[4 * b + q];
    for (int q = 0; q < 4; q++) sh[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st)
            for (int q = 0; q < 4; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x < 4) out4[threadIdx.x] = sh[threadIdx.x][0];
}

// ------------------------------------------------------------ diagnostics

// compute_enstrophy_mod.h:5-75: vorticity du2/dx - du1/dy by least squares
// over the full stencil (the gradient's weights and moments), its square, and
// per-block partial sums of the squares.
__global__ void __launch_bounds__(256) k_enstrophy(DevCloud c, const double4_32a *__restrict__ prim,
                                                   double *__restrict__ vort, double *__restrict__ partial)
{
    __shared__ double sh[256];
    const int i = blockIdx.x * 256 + threadIdx.x;
    double v2 = 0.0;
    if (i < c.n) {
        const double4_32a Pi = prim[i];
        double sx1 = 0., sx2 = 0., sy1 = 0., sy2 = 0.;
        const int nb = c.nbhs[i];
        const long long base = c.slice_base[i >> 5] + (i & 31);
        for (int j = 0; j < nb; j++) {
            const long long e = base + 32LL * j;
            const int k = c.e_nbr[e];
            const double4_32a g = c.e_geo[e];       // delx, dely, w delx, w dely
            const double4_32a Pk = prim[k];
            sx1 = sx1 + g.z * (Pk.y - Pi.y);
            sx2 = sx2 + g.z * (Pk.z - Pi.z);
            sy1 = sy1 + g.w * (Pk.y - Pi.y);
            sy2 = sy2 + g.w * (Pk.z - Pi.z);
        }
        const double4_32a m = c.ggeo[i];           // sxx, syy, sxy, 1/det
        const double du2_dx = (sx2 * m.y - sy2 * m.z) * m.w;
        const double du1_dy = (sy1 * m.x - sx1 * m.z) * m.w;
        const double t = du2_dx - du1_dy;
        vort[i] = t;
        v2 = t * t;
    }
    sh[threadIdx.x] = v2;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// Stagnation pressure p0 = p (1 + (gamma - 1)/2 M^2)^(gamma / (gamma - 1)) per
// point (stagnation_values_mod.h:9-48): per block the minimum and maximum
// (first index on ties), the sum of (p0_inf - p0)^2 (:51-80) and of p0.
// partial [blocks][6]: min, argmin, max, argmax, sum of squares, sum.
__global__ void __launch_bounds__(256) k_stagnation(int n, const double4_32a *__restrict__ prim, double gamma,
                                                    double p0_inf, double *__restrict__ partial)
{
    __shared__ double smin[256], smax[256], ssum[256], sp0[256];
    __shared__ int imin[256], imax[256];
    const int i = blockIdx.x * 256 + threadIdx.x;
    double p0 = 0.0, sq = 0.0;
    const double gp = gamma / (gamma - 1);
    if (i < n) {
        const double4_32a P = prim[i];
        const double angle = sqrt(gamma * P.w / P.x);
        const double mach_t = sqrt(pow(P.y, 2) + pow(P.z, 2)) / angle;
        p0 = P.w * pow(1 + ((gamma - 1) / 2) * mach_t * mach_t, gp);
        sq = pow(p0_inf - p0, 2);
    }
    const bool ok = i < n;
    smin[threadIdx.x] = ok ? p0 : INFINITY;
    smax[threadIdx.x] = ok ? p0 : -INFINITY;
    imin[threadIdx.x] = imax[threadIdx.x] = ok ? i : 0x7fffffff;
    ssum[threadIdx.x] = sq;
    sp0[threadIdx.x] = p0;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        const int t = threadIdx.x;
        if (t < st) {
            const int u = t + st;
            if (smin[u] < smin[t] || (smin[u] == smin[t] && imin[u] < imin[t])) { smin[t] = smin[u]; imin[t] = imin[u]; }
            if (smax[u] > smax[t] || (smax[u] == smax[t] && imax[u] < imax[t])) { smax[t] = smax[u]; imax[t] = imax[u]; }
            ssum[t] += ssum[u];
            sp0[t] += sp0[u];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double *o = partial + 6 * (size_t)blockIdx.x;
        o[0] = smin[0];
        o[1] = (double)imin[0];
        o[2] = smax[0];
        o[3] = (double)imax[0];
        o[4] = ssum[0];
        o[5] = sp0[0];
    }
}

// ------------------------------------------------------------- launchers

#define QLSKUM_LAUNCHED(L) \
    do { if ((L).launches) ++*(L).launches; } while (0)

void q_variables(const Launch &L, const DevCloud &c, const double4_32a *prim, double4_32a *q)
{
    k_q_variables<<<grid_for(c.n, 256), 256, 0, L.stream>>>(c.n, prim, q);
    QLSKUM_LAUNCHED(L);
}

void derived(const Launch &L, const DevCloud &c, const double4_32a *prim, double4_32a *q, double *cspeed)
{
    k_derived<<<grid_for(c.n, 256), 256, 0, L.stream>>>(c.n, prim, q, cspeed);
    QLSKUM_LAUNCHED(L);
}

void q_derivatives(const Launch &L, const DevCloud &c, const double4_32a *q, double4_32a *dq, double4_32a *qm,
                   const double *cspeed, double *delta, double cfl)
{
    k_q_derivatives<<<grid_for(c.n, L.block), L.block, 0, L.stream>>>(c, q, dq, qm, cspeed, delta, cfl);
    QLSKUM_LAUNCHED(L);
}

void q_inner(const Launch &L, const DevCloud &c, const double4_32a *q, const double4_32a *dq_in, double4_32a *dq_out)
{
    k_q_inner<<<grid_for(c.n, L.block), L.block, 0, L.stream>>>(c, q, dq_in, dq_out);
    QLSKUM_LAUNCHED(L);
}

void func_delta(const Launch &L, const DevCloud &c, const double4_32a *prim, double *delta, double cfl)
{
    k_func_delta<<<grid_for(c.n, L.block), L.block, 0, L.stream>>>(c, prim, delta, cfl);
    QLSKUM_LAUNCHED(L);
}

void flux_residual(const Launch &L, const DevCloud &c, const double4_32a *q, const double4_32a *dq, const double4_32a *qm,
                   const double *delta, double4_32a *flux_res, double *sums, double *ends, long long ns)
{
    k_flux_residual<<<grid_for(c.n, 128), 128, 0, L.stream>>>(c, q, dq, qm, delta, flux_res, sums, ends, ns);
    QLSKUM_LAUNCHED(L);
}

void state_update(const Launch &L, const DevCloud &c, const CaseConst &k, double4_32a *prim, const double4_32a *prim_old,
                  const double4_32a *flux_res, int rk, const Reduce &R)
{
    k_state_update<128><<<grid_for(c.n, 128), 128, 0, L.stream>>>(c, k, prim, prim_old, flux_res, rk,
                                                                   R.partial_sum, R.partial_max);
    QLSKUM_LAUNCHED(L);
}

void flux_update(const Launch &L, const DevCloud &c, const CaseConst &k, const double4_32a *q, const double4_32a *dq,
                 const double4_32a *qm, const double *delta, const double4_32a *prim, const double4_32a *prim_old,
                 double4_32a *prim_next, double4_32a *q_next, double *cspeed_next, int rk, const Reduce &R)
{
    k_flux_update<128><<<grid_for(c.n, 128), 128, 0, L.stream>>>(c, k, q, dq, qm, delta, prim, prim_old, prim_next,
                                                                  q_next, cspeed_next, rk, R.partial_sum,
                                                                  R.partial_max);
    QLSKUM_LAUNCHED(L);
}

void reduce_residual(const Launch &L, const Reduce &R, int n, int it)
{
    k_reduce_residual<<<1, RB, 0, L.stream>>>(R.blocks, R.partial_sum, R.partial_max, n, it, R.hist, R.capacity,
                                              R.res_old, R.iter, R.status, R.latch);
    QLSKUM_LAUNCHED(L);
}

void copy_prim(const Launch &L, int n, const double4_32a *src, double4_32a *dst)
{
    k_copy<<<grid_for(n, 256), 256, 0, L.stream>>>(n, src, dst);
    QLSKUM_LAUNCHED(L);
}

// out[0] = max over the n points and components of |a - b|, out[1] of |a|,
// as the bit patterns of non-negative doubles (which order like the values),
// per-warp maxima then one atomicMax per warp; out zeroed by the caller.
__global__ void k_max_change(int n, const double4_32a *__restrict__ a, const double4_32a *__restrict__ b,
                             unsigned long long *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double d = 0.0, m = 0.0;
    if (i < n) {
        const double4_32a x = a[i], y = b[i];
        d = fmax(fmax(fabs(x.x - y.x), fabs(x.y - y.y)), fmax(fabs(x.z - y.z), fabs(x.w - y.w)));
        m = fmax(fmax(fabs(x.x), fabs(x.y)), fmax(fabs(x.z), fabs(x.w)));
    }
    for (int o = 16; o > 0; o >>= 1) {
        d = fmax(d, __shfl_down_sync(0xffffffffu, d, o));
        m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, (unsigned long long)__double_as_longlong(d));
        atomicMax(out + 1, (unsigned long long)__double_as_longlong(m));
    }
}

void max_change(const Launch &L, int n, const double4_32a *a, const double4_32a *b, unsigned long long *out)
{
    k_max_change<<<grid_for(n, 256), 256, 0, L.stream>>>(n, a, b, out);
    QLSKUM_LAUNCHED(L);
}

__global__ void k_set_int(int *p, int v) { *p = v; }

void set_counter(const Launch &L, int *p, int v)
{
    k_set_int<<<1, 1, 0, L.stream>>>(p, v);
    QLSKUM_LAUNCHED(L);
}

// dst[i] = v for the n points.
__global__ void k_fill(int n, double4_32a v, double4_32a *__restrict__ dst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = v;
}

void fill_prim(const Launch &L, int n, double4_32a v, double4_32a *dst)
{
    k_fill<<<grid_for(n, 256), 256, 0, L.stream>>>(n, v, dst);
    QLSKUM_LAUNCHED(L);
}

// out[0] += sum of src.y, out[1] += sum of src.z over the n points (warp
// sums, one atomic per warp).
__global__ void k_sum_yz(int n, const double4_32a *__restrict__ src, double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0, b = 0.0;
    if (i < n) {
        const double4_32a v = src[i];
        a = v.y;
        b = v.z;
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out, a);
        atomicAdd(out + 1, b);
    }
}

void sum_yz(const Launch &L, int n, const double4_32a *src, double *out)
{
    k_sum_yz<<<grid_for(n, 256), 256, 0, L.stream>>>(n, src, out);
    QLSKUM_LAUNCHED(L);
}

void permute_in(const Launch &L, int n, const int *perm, const double4_32a *src, double4_32a *dst)
{
    k_permute_in<<<grid_for(n, 256), 256, 0, L.stream>>>(n, perm, src, dst);
    QLSKUM_LAUNCHED(L);
}

void permute_out(const Launch &L, int n, const int *perm, const double4_32a *src, double4_32a *dst)
{
    k_permute_out<<<grid_for(n, 256), 256, 0, L.stream>>>(n, perm, src, dst);
    QLSKUM_LAUNCHED(L);
}

void add_prim(const Launch &L, int n, const double4_32a *src, double4_32a *dst)
{
    k_add<<<grid_for(n, 256), 256, 0, L.stream>>>(n, src, dst);
    QLSKUM_LAUNCHED(L);
}

void enstrophy(const Launch &L, const DevCloud &c, const double4_32a *prim, double *vort, double *partial)
{
    k_enstrophy<<<grid_for(c.n, 256), 256, 0, L.stream>>>(c, prim, vort, partial);
    QLSKUM_LAUNCHED(L);
}

void stagnation(const Launch &L, int n, const double4_32a *prim, double gamma, double p0_inf, double *partial)
{
    k_stagnation<<<grid_for(n, 256), 256, 0, L.stream>>>(n, prim, gamma, p0_inf, partial);
    QLSKUM_LAUNCHED(L);
}

void objective(const Launch &L, const DevCloud &c, const double4_32a *prim, const int *wall_perm,
               const double4_32a *wall_geo, int n_wall, double cp_scale, double pr_inf, double gamma, double *entropy,
               double *out4, double *scratch)
{
    // entropy NULL: the force coefficients only (the wall points)
    const int items = (entropy && c.n > n_wall) ? c.n : n_wall;
    const int blocks = grid_for(items, 256);
    k_objective<<<blocks, 256, 0, L.stream>>>(c, prim, wall_perm, wall_geo, n_wall, cp_scale, pr_inf, gamma, entropy,
                                              scratch);
    k_objective_finish<<<1, 256, 0, L.stream>>>(blocks, scratch, out4);
    if (L.launches) *L.launches += 2;
}

}  // namespace fp64

namespace halo {

// One thread per (ghost, 16-byte word) of the element.
__global__ void k_pull16(int n, int w, const int *__restrict__ idx, const float4 *__restrict__ src,
                         float4 *__restrict__ dst)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * w) return;
    const int g = (int)(t / w), j = (int)(t - (long long)g * w);
    dst[t] = src[(long long)idx[g] * w + j];
}

template <typename T>
__global__ void k_pull(int n, const int *__restrict__ idx, const T *__restrict__ src, T *__restrict__ dst)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < n) dst[g] = src[idx[g]];
}

void pull(const Launch &L, int n, const int *idx, const void *src, void *dst, int bytes)
{
    if (n <= 0) return;
    if (bytes == 4) {
        k_pull<float><<<fp64::grid_for(n, 256), 256, 0, L.stream>>>(n, idx, static_cast<const float *>(src),
                                                             static_cast<float *>(dst));
    } else if (bytes == 8) {
        k_pull<double><<<fp64::grid_for(n, 256), 256, 0, L.stream>>>(n, idx, static_cast<const double *>(src),
                                                              static_cast<double *>(dst));
    } else {
        const int w = bytes / 16;
        const long long items = (long long)n * w;
        k_pull16<<<(int)((items + 255) / 256), 256, 0, L.stream>>>(n, w, idx, static_cast<const float4 *>(src),
                                                                    static_cast<float4 *>(dst));
    }
    if (L.launches) ++*L.launches;
}

}  // namespace halo
}  // namespace qlskum
