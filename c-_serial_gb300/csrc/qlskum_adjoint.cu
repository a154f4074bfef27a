// Discrete adjoint (reverse mode) of the FP64 q-LSKUM iteration.
//
// The reverse of one pseudo-time iteration (fpi_solver_mod.h:14-151) runs
// stage by stage from the last: the SSPRK update, the flux residual (limiter,
// reconstruction, split fluxes, least-squares solves), the inner-loop
// gradients, the least-squares gradient and neighbour min / max, the q
// variables, and finally the local time step.  The forward stage states it
// needs are recomputed by the FP64 forward kernels from the iteration's
// checkpointed state.  One thread per point; a point's contributions to its
// neighbours' adjoints are scattered with FP64 atomics (the bar of a
// neighbour's q, dq, qm, or wave speed).
//
// With GEO the kernels also accumulate the adjoints of the geometry each
// launch reads (edge vectors, rotated edge vectors, edge lengths, normals,
// least-squares moments) for the wall-displacement gradient, which the host
// finishes (qlskum_host.cpp).
#include "qlskum_adjoint.cuh"
#include "qlskum_dev.cuh"

namespace qlskum {
namespace adjk {

using adj::KinBar;

static inline int grid_for(int n, int block) { return (n + block - 1) / block; }

__device__ __forceinline__ void atomic_add4(double4_32a *p, const double v[4])
{
    double *d = reinterpret_cast<double *>(p);
    atomicAdd(d + 0, v[0]);
    atomicAdd(d + 1, v[1]);
    atomicAdd(d + 2, v[2]);
    atomicAdd(d + 3, v[3]);
}

// Reverse of the SSPRK update of every point (stage rk).  bP holds the bar of
// the stage output on entry and is overwritten with the bar of the stage
// input; bPold (stage 3) and bF receive their bars; bn / buinf the normal's
// and the free stream's (GEO / parameters).
__global__ void k_update(AdjView a, CaseConst K, const double4_32a *__restrict__ Pin,
                         const double4_32a *__restrict__ Pold, const double4_32a *__restrict__ Pout, int rk,
                         double4_32a *__restrict__ bP, double4_32a *__restrict__ bPold, double4_32a *__restrict__ bF,
                         double *__restrict__ buinf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double bu1 = 0.0, bu2 = 0.0;
    if (i < a.c.n) {
        const int f = a.c.flag[i];
        const double2 nn = a.c.nrm[i];
        double pin[4], pold[4], pout[4], bout[4], bin[4] = {0, 0, 0, 0}, bo[4] = {0, 0, 0, 0}, bf[4] = {0, 0, 0, 0};
        ld4(Pin[i], pin);
        ld4(Pold[i], pold);
        ld4(Pout[i], pout);
        ld4(bP[i], bout);
        double bnx = 0.0, bny = 0.0;
        adj::stage_update_vjp(K, f, nn.x, nn.y, pin, pold, pout, rk, bout, bin, bo, bf, bnx, bny, bu1, bu2);
        bP[i] = mk4(bin);
        bF[i] = mk4(bf);
        if (rk == 3) {
            double acc[4];
            ld4(bPold[i], acc);
            for (int r = 0; r < 4; r++) acc[r] += bo[r];
            bPold[i] = mk4(acc);
        }
        if (a.bnrm) {
            a.bnrm[i].x += bnx;
            a.bnrm[i].y += bny;
        }
    }
    // free-stream bars: warp sums, one atomic per warp
    for (int o = 16; o > 0; o >>= 1) {
        bu1 += __shfl_down_sync(0xffffffffu, bu1, o);
        bu2 += __shfl_down_sync(0xffffffffu, bu2, o);
    }
    if ((threadIdx.x & 31) == 0 && (bu1 != 0.0 || bu2 != 0.0)) {
        atomicAdd(buinf, bu1);
        atomicAdd(buinf + 1, bu2);
    }
}

// Reverse of the flux residual of every point: F_i = s delta_i sum_d G_d.
// Adds the bars of q, dq, qm (own and neighbours'), of delta, and (GEO) of the
// edge geometry, the normal and the directional moments.
template <int MODE>
__global__ void __launch_bounds__(128) k_flux(AdjView a, const double4_32a *__restrict__ q,
                                               const double4_32a *__restrict__ dq, const double4_32a *__restrict__ qm,
                                               const double *__restrict__ delta, const double4_32a *__restrict__ flux,
                                               const double *__restrict__ sums, const double *__restrict__ ends,
                                               long long ns, const double4_32a *__restrict__ bF,
                                               double4_32a *__restrict__ bq, double4_32a *__restrict__ bdq,
                                               double4_32a *__restrict__ bqm, double *__restrict__ bdelta)
{
    // MODE 0: the state bars at every point; 2: only the geometry bars, at
    // the points AdjView::geo_list names (the geometry's instantiation needs
    // far more registers, so it runs on those few points alone)
    constexpr bool GEO = MODE != 0, STATE = MODE != 2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (MODE == 2 ? a.n_geo : a.c.n)) return;
    const int i = MODE == 2 ? a.geo_list[t] : t;
    const DevCloud &c = a.c;
    const int f = c.flag[i];
    const double2 nn = c.nrm[i];
    const double nx = nn.x, ny = nn.y;
    double qi[4], dxi[4], dyi[4], mxi[4], mni[4];
    ld4(q[i], qi);
    ld4(dq[2 * i], dxi);
    ld4(dq[2 * i + 1], dyi);
    ld4(qm[2 * i], mxi);
    ld4(qm[2 * i + 1], mni);
    const double e2i = c.eps2[i];
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    const double scale = (f == kWall) ? 2.0 : 1.0;
    const bool used[4] = {true, true, f != kWall, f != kOuter};
    const bool geo = GEO;

    // forward: the directional sums, for the bars of the moments (GEO only:
    // the forward kernel's stored sums, or recomputed; without them the bar of
    // delta comes from the stage's flux residual, F = delta * scale * sum_d G_d,
    // so dF/ddelta = F / delta)
    double sx[4][4], sy[4][4];
    for (int d = 0; d < 4; d++)
        for (int r = 0; r < 4; r++) sx[d][r] = sy[d][r] = 0.0;
    if (geo && sums) {
        const double *o = sums + 32 * (size_t)i;
        for (int d = 0; d < 4; d++)
            for (int r = 0; r < 4; r++) {
                sx[d][r] = o[8 * d + r];
                sy[d][r] = o[8 * d + 4 + r];
            }
    }
    for (int j = 0; geo && !sums && j < nb; j++) {
        const long long e = base + 32LL * j;
        const int k = c.e_nbr[e];
        const double4_32a g = c.e_geo[e];
        const double2 sw = c.e_sn[e];
        const unsigned dir = c.e_dir[e];
        double qk[4], dxk[4], dyk[4], mxk[4], mnk[4], Pi[4], Pk[4];
        ld4(q[k], qk);
        ld4(dq[2 * k], dxk);
        ld4(dq[2 * k + 1], dyk);
        ld4(qm[2 * k], mxk);
        ld4(qm[2 * k + 1], mnk);
        edge_states<double>(g.x, g.y, qi, dxi, dyi, mxi, mni, e2i, qk, dxk, dyk, mxk, mnk, c.eps2[k], Pi, Pk);
        Kin<double> ki, kk;
        kin_prep<double>(nx, ny, Pi[1], Pi[2], Pi[0], Pi[3], ki);
        kin_prep<double>(nx, ny, Pk[1], Pk[2], Pk[0], Pk[3], kk);
#define QLSKUM_FWD(D)                                                                \
        if (dir & (1u << D)) {                                                       \
            double Gi[4], Gk[4];                                                     \
            dir_flux<double, D>(f, ki, Gi);                                          \
            dir_flux<double, D>(f, kk, Gk);                                          \
            for (int r = 0; r < 4; r++) {                                            \
                sx[D][r] += (Gk[r] - Gi[r]) * sw.x;                                  \
                sy[D][r] += (Gk[r] - Gi[r]) * sw.y;                                  \
            }                                                                        \
        }
        QLSKUM_FWD(0)
        QLSKUM_FWD(1)
        QLSKUM_FWD(2)
        QLSKUM_FWD(3)
#undef QLSKUM_FWD
    }
    double bFi[4];
    ld4(bF[i], bFi);
    const double dl = delta[i];
    // bars of the directional sums: the solve is linear in them, so the bar
    // of sum x (y) of half-range d, component r, is bG[r] ax[d] (bG[r] ay[d])
    // with bG = scale delta F-bar
    double bG4[4], ax[4], ay[4];
    for (int r = 0; r < 4; r++) bG4[r] = scale * dl * bFi[r];
    double bdl = 0.0;
    for (int d = 0; d < 4; d++) {
        const double4_32a m = c.fgeo[4 * i + d];
        ax[d] = ay[d] = 0.0;
        if (!used[d]) continue;
        if (d < 2) {
            ax[d] = m.y * m.w;
            ay[d] = -m.z * m.w;
        } else {
            ax[d] = -m.z * m.w;
            ay[d] = m.x * m.w;
        }
        if (!geo) continue;
        double bm[4] = {0, 0, 0, 0};
        for (int r = 0; r < 4; r++) {
            const double bG = bG4[r];
            if (d < 2) {
                const double G = (sx[d][r] * m.y - sy[d][r] * m.z) * m.w;
                bdl += scale * bFi[r] * G;
                bm[1] += bG * sx[d][r] * m.w;
                bm[2] -= bG * sy[d][r] * m.w;
                bm[3] += bG * (sx[d][r] * m.y - sy[d][r] * m.z);
            } else {
                const double G = (sy[d][r] * m.x - sx[d][r] * m.z) * m.w;
                bdl += scale * bFi[r] * G;
                bm[0] += bG * sy[d][r] * m.w;
                bm[2] -= bG * sx[d][r] * m.w;
                bm[3] += bG * (sy[d][r] * m.x - sx[d][r] * m.z);
            }
        }
        double4_32a &acc = a.bfmom[4 * i + d];
        acc.x += bm[0];
        acc.y += bm[1];
        acc.z += bm[2];
        acc.w += bm[3];
    }
    if (!geo) {
        double F[4];
        ld4(flux[i], F);
        bdl = (bFi[0] * F[0] + bFi[1] * F[1] + bFi[2] * F[2] + bFi[3] * F[3]) / dl;
    }
    if (STATE) bdelta[i] += bdl;

    // reverse over the edges, one end at a time (end64 / end64_vjp): the
    // neighbour's end first, its bars scattered, then the owner's
    double bqi[4] = {0, 0, 0, 0}, bdxi[4] = {0, 0, 0, 0}, bdyi[4] = {0, 0, 0, 0}, bmxi[4] = {0, 0, 0, 0},
           bmni[4] = {0, 0, 0, 0};
    double bnx = 0.0, bny = 0.0;
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const int k = c.e_nbr[e];
        const double4_32a g = c.e_geo[e];
        const double2 sw = c.e_sn[e];
        const unsigned dir = c.e_dir[e];
        double bdelx = 0.0, bdely = 0.0, bsw_x = 0.0, bsw_y = 0.0;
        // the bar of G_k on half-range D is bG (ax sw.x + ay sw.y), that of G_i its negative
#define QLSKUM_REV(D, SGN, KIN, KB)                                                  \
        if (dir & (1u << D)) {                                                       \
            const double fw = SGN * (ax[D] * sw.x + ay[D] * sw.y);                   \
            double bG[4];                                                            \
            for (int r = 0; r < 4; r++) bG[r] = fw * bG4[r];                         \
            adj::dir_flux_vjp<D>(f, KIN, bG, KB);                                    \
            if (geo) {                                                               \
                double G[4];                                                         \
                dir_flux<double, D>(f, KIN, G);                                      \
                const double gb = bG4[0] * G[0] + bG4[1] * G[1] + bG4[2] * G[2] + bG4[3] * G[3]; \
                bsw_x += SGN * ax[D] * gb;                                           \
                bsw_y += SGN * ay[D] * gb;                                           \
            }                                                                        \
        }
        {
            double qk[4], dxk[4], dyk[4], mxk[4], mnk[4];
            ld4(q[k], qk);
            ld4(dq[2 * k], dxk);
            ld4(dq[2 * k + 1], dyk);
            ld4(qm[2 * k], mxk);
            ld4(qm[2 * k + 1], mnk);
            adj::End64 s;
            double kept[6];
            if (ends)
                for (int w = 0; w < 6; w++) kept[w] = ends[(6 + w) * ns + e];
            adj::end64(nx, ny, g.x, g.y, qk, dxk, dyk, mxk, mnk, c.eps2[k], s, ends ? kept : nullptr);
            KinBar kb;
            QLSKUM_REV(0, 1.0, s.k, kb)
            QLSKUM_REV(1, 1.0, s.k, kb)
            QLSKUM_REV(2, 1.0, s.k, kb)
            QLSKUM_REV(3, 1.0, s.k, kb)
            double bqk[4] = {0, 0, 0, 0}, bdxk[4] = {0, 0, 0, 0}, bdyk[4] = {0, 0, 0, 0}, bmxk[4] = {0, 0, 0, 0},
                   bmnk[4] = {0, 0, 0, 0};
            adj::end64_vjp(s, nx, ny, g.x, g.y, dxk, dyk, kb, bqk, bdxk, bdyk, bmxk, bmnk, bdelx, bdely, bnx, bny);
            if (STATE) {
                atomic_add4(bq + k, bqk);
                atomic_add4(bdq + 2 * k, bdxk);
                atomic_add4(bdq + 2 * k + 1, bdyk);
                atomic_add4(bqm + 2 * k, bmxk);
                atomic_add4(bqm + 2 * k + 1, bmnk);
            }
        }
        {
            adj::End64 s;
            double kept[6];
            if (ends)
                for (int w = 0; w < 6; w++) kept[w] = ends[w * ns + e];
            adj::end64(nx, ny, g.x, g.y, qi, dxi, dyi, mxi, mni, e2i, s, ends ? kept : nullptr);
            KinBar kb;
            QLSKUM_REV(0, -1.0, s.k, kb)
            QLSKUM_REV(1, -1.0, s.k, kb)
            QLSKUM_REV(2, -1.0, s.k, kb)
            QLSKUM_REV(3, -1.0, s.k, kb)
            adj::end64_vjp(s, nx, ny, g.x, g.y, dxi, dyi, kb, bqi, bdxi, bdyi, bmxi, bmni, bdelx, bdely, bnx, bny);
        }
#undef QLSKUM_REV
        if (geo) {
            double4_32a &ge = a.bedge[e];
            ge.x += bdelx;
            ge.y += bdely;
            ge.z += bsw_x;
            ge.w += bsw_y;
        }
    }
    if (STATE) {
        atomic_add4(bq + i, bqi);
        atomic_add4(bdq + 2 * i, bdxi);
        atomic_add4(bdq + 2 * i + 1, bdyi);
        atomic_add4(bqm + 2 * i, bmxi);
        atomic_add4(bqm + 2 * i + 1, bmni);
    }
    if (geo && a.bnrm) {
        a.bnrm[i].x += bnx;
        a.bnrm[i].y += bny;
    }
}

// Reverse of one inner iteration (q_variables_mod.h:120-213): bdq_out is the
// bar of its output; adds bars of q and of its input dq.
template <int MODE>
__global__ void k_inner(AdjView a, const double4_32a *__restrict__ q, const double4_32a *__restrict__ dq_in,
                        const double4_32a *__restrict__ bdq_out, double4_32a *__restrict__ bq,
                        double4_32a *__restrict__ bdq_in)
{
    // MODE 0: state bars everywhere; 2: geometry bars only, at AdjView::geo_list
    constexpr bool STATE = MODE != 2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (MODE == 2 ? a.n_geo : a.c.n)) return;
    const int i = MODE == 2 ? a.geo_list[t] : t;
    const DevCloud &c = a.c;
    const bool geo = MODE != 0;
    const double4_32a m = c.ggeo[i];
    double bx[4], by[4];
    ld4(bdq_out[2 * i], bx);
    ld4(bdq_out[2 * i + 1], by);
    double bsdx[4], bsdy[4];
    for (int r = 0; r < 4; r++) {
        bsdx[r] = m.w * (bx[r] * m.y - by[r] * m.z);
        bsdy[r] = m.w * (by[r] * m.x - bx[r] * m.z);
    }
    double qi[4], dxi[4], dyi[4];
    ld4(q[i], qi);
    ld4(dq_in[2 * i], dxi);
    ld4(dq_in[2 * i + 1], dyi);
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    double sdx[4] = {0, 0, 0, 0}, sdy[4] = {0, 0, 0, 0};
    double bqi[4] = {0, 0, 0, 0}, bdxi[4] = {0, 0, 0, 0}, bdyi[4] = {0, 0, 0, 0};
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const int k = c.e_nbr[e];
        const double4_32a g = c.e_geo[e];
        double qk[4], dxk[4], dyk[4];
        ld4(q[k], qk);
        ld4(dq_in[2 * k], dxk);
        ld4(dq_in[2 * k + 1], dyk);
        double bqk[4], bdxk[4], bdyk[4];
        double bgx = 0.0, bgy = 0.0, bwx = 0.0, bwy = 0.0;
        for (int r = 0; r < 4; r++) {
            const double t1 = qi[r] - 0.5 * (g.x * dxi[r] + g.y * dyi[r]);
            const double t2 = qk[r] - 0.5 * (g.x * dxk[r] + g.y * dyk[r]);
            sdx[r] += g.z * (t2 - t1);
            sdy[r] += g.w * (t2 - t1);
            const double bt = g.z * bsdx[r] + g.w * bsdy[r];
            bqk[r] = bt;
            bdxk[r] = -0.5 * g.x * bt;
            bdyk[r] = -0.5 * g.y * bt;
            bqi[r] -= bt;
            bdxi[r] += 0.5 * g.x * bt;
            bdyi[r] += 0.5 * g.y * bt;
            if (geo) {
                bwx += bsdx[r] * (t2 - t1);
                bwy += bsdy[r] * (t2 - t1);
                bgx += -0.5 * bt * (dxk[r] - dxi[r]);
                bgy += -0.5 * bt * (dyk[r] - dyi[r]);
            }
        }
        if (STATE) {
            atomic_add4(bq + k, bqk);
            atomic_add4(bdq_in + 2 * k, bdxk);
            atomic_add4(bdq_in + 2 * k + 1, bdyk);
        }
        if (geo) {
            // unit weights: w delx == delx
            double4_32a &ge = a.bedge[e];
            ge.x += bgx + bwx;
            ge.y += bgy + bwy;
        }
    }
    if (STATE) {
        atomic_add4(bq + i, bqi);
        atomic_add4(bdq_in + 2 * i, bdxi);
        atomic_add4(bdq_in + 2 * i + 1, bdyi);
    }
    if (geo) {
        double bm[4] = {0, 0, 0, 0};
        for (int r = 0; r < 4; r++) {
            // dx = ood (Sx syy - Sy sxy), dy = ood (Sy sxx - Sx sxy)
            bm[1] += m.w * bx[r] * sdx[r];
            bm[2] += -m.w * (bx[r] * sdy[r] + by[r] * sdx[r]);
            bm[0] += m.w * by[r] * sdy[r];
            bm[3] += bx[r] * (sdx[r] * m.y - sdy[r] * m.z) + by[r] * (sdy[r] * m.x - sdx[r] * m.z);
        }
        double4_32a &acc = a.bgmom[i];
        acc.x += bm[0];
        acc.y += bm[1];
        acc.z += bm[2];
        acc.w += bm[3];
    }
}

// Reverse of the least-squares gradient and of the neighbour max / min
// (q_variables_mod.h:36-118).
template <int MODE>
__global__ void k_grad(AdjView a, const double4_32a *__restrict__ q, const double4_32a *__restrict__ bdq,
                       const double4_32a *__restrict__ bqm, double4_32a *__restrict__ bq)
{
    // MODE 0: state bars everywhere; 2: geometry bars only, at AdjView::geo_list
    constexpr bool STATE = MODE != 2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (MODE == 2 ? a.n_geo : a.c.n)) return;
    const int i = MODE == 2 ? a.geo_list[t] : t;
    const DevCloud &c = a.c;
    const bool geo = MODE != 0;
    const double4_32a m = c.ggeo[i];
    double bx[4], by[4], bmax[4], bmin[4];
    ld4(bdq[2 * i], bx);
    ld4(bdq[2 * i + 1], by);
    ld4(bqm[2 * i], bmax);
    ld4(bqm[2 * i + 1], bmin);
    double bsdx[4], bsdy[4];
    for (int r = 0; r < 4; r++) {
        bsdx[r] = (bx[r] * m.y - by[r] * m.z) * m.w;
        bsdy[r] = (by[r] * m.x - bx[r] * m.z) * m.w;
    }
    double qi[4];
    ld4(q[i], qi);
    double qmax[4], qmin[4];
    int amax[4], amin[4];
    for (int r = 0; r < 4; r++) {
        qmax[r] = qmin[r] = qi[r];
        amax[r] = amin[r] = i;
    }
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    double sdx[4] = {0, 0, 0, 0}, sdy[4] = {0, 0, 0, 0};
    double bqi[4] = {0, 0, 0, 0};
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const int k = c.e_nbr[e];
        const double4_32a g = c.e_geo[e];
        double qk[4], bqk[4];
        ld4(q[k], qk);
        double bwx = 0.0, bwy = 0.0;
        for (int r = 0; r < 4; r++) {
            if (qk[r] > qmax[r]) { qmax[r] = qk[r]; amax[r] = k; }
            if (qk[r] < qmin[r]) { qmin[r] = qk[r]; amin[r] = k; }
            sdx[r] += g.z * (qk[r] - qi[r]);
            sdy[r] += g.w * (qk[r] - qi[r]);
            const double bt = g.z * bsdx[r] + g.w * bsdy[r];
            bqk[r] = bt;
            bqi[r] -= bt;
            if (geo) {
                bwx += bsdx[r] * (qk[r] - qi[r]);
                bwy += bsdy[r] * (qk[r] - qi[r]);
            }
        }
        if (STATE) atomic_add4(bq + k, bqk);
        if (geo) {
            double4_32a &ge = a.bedge[e];
            ge.x += bwx;
            ge.y += bwy;
        }
    }
    if (STATE) {
        atomic_add4(bq + i, bqi);
        double *bqd = reinterpret_cast<double *>(bq);
        for (int r = 0; r < 4; r++) {
            if (bmax[r] != 0.0) atomicAdd(bqd + 4 * (size_t)amax[r] + r, bmax[r]);
            if (bmin[r] != 0.0) atomicAdd(bqd + 4 * (size_t)amin[r] + r, bmin[r]);
        }
    }
    if (geo) {
        double bm[4] = {0, 0, 0, 0};
        for (int r = 0; r < 4; r++) {
            bm[1] += m.w * bx[r] * sdx[r];
            bm[2] += -m.w * (bx[r] * sdy[r] + by[r] * sdx[r]);
            bm[0] += m.w * by[r] * sdy[r];
            bm[3] += bx[r] * (sdx[r] * m.y - sdy[r] * m.z) + by[r] * (sdy[r] * m.x - sdx[r] * m.z);
        }
        double4_32a &acc = a.bgmom[i];
        acc.x += bm[0];
        acc.y += bm[1];
        acc.z += bm[2];
        acc.w += bm[3];
    }
}

// bP += (dq/dP)^T bq  (q_variables_mod.h:19-33)
__global__ void k_q(int n, const double4_32a *__restrict__ P, const double4_32a *__restrict__ bq,
                    double4_32a *__restrict__ bP)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double p[4], b[4], acc[4];
    ld4(P[i], p);
    ld4(bq[i], b);
    ld4(bP[i], acc);
    adj::prim_to_q_vjp(p, b, acc);
    bP[i] = mk4(acc);
}

// Reverse of the local time step (state_update_mod.h:448-496): the bar of
// delta_i goes to the wave speed of the neighbour that set the minimum.
template <bool GEO>
__global__ void k_delta(AdjView a, const double4_32a *__restrict__ P, const double *__restrict__ bdelta,
                        double cfl, double *__restrict__ bc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.c.n) return;
    const DevCloud &c = a.c;
    double min_delt = 1.0;
    int arg = -1;
    long long earg = -1;
    double carg = 0.0;
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const int k = c.e_nbr[e];
        double p[4];
        ld4(P[k], p);
        const double ck = wave_speed(p);
        double dt = c.e_dist[e] / ck;
        dt = cfl * dt;
        if (min_delt > dt) {
            min_delt = dt;
            arg = k;
            earg = e;
            carg = ck;
        }
    }
    if (arg >= 0 && bdelta[i] != 0.0) {
        atomicAdd(bc + arg, -bdelta[i] * cfl * c.e_dist[earg] / (carg * carg));
        if (GEO && a.geo_pt[i]) a.bdist[earg] += bdelta[i] * cfl / carg;
    }
}

__global__ void k_wave(int n, const double4_32a *__restrict__ P, const double *__restrict__ bc,
                       double4_32a *__restrict__ bP)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || bc[i] == 0.0) return;
    double p[4], acc[4];
    ld4(P[i], p);
    ld4(bP[i], acc);
    adj::wave_speed_vjp(p, bc[i], acc);
    bP[i] = mk4(acc);
}

// bP = the bar of Cl (which = 0) or Cd (which = 1) w.r.t. the wall pressures
// (compute_force_coeffs_mod.h:37-67), added to the shape points' entries.
__global__ void k_objective(AdjView a, const int *__restrict__ wall_perm, const double4_32a *__restrict__ wall_geo,
                            int n_wall, double cp_scale, double theta, int which, double4_32a *__restrict__ bP)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_wall) return;
    const int m = wall_perm[t];
    const double ds = wall_geo[t].x;
    const double2 nn = a.c.nrm[m];
    // Cl = V cos - H sin, Cd = H cos + V sin; H = sum cp nx ds, V = sum cp ny ds, cp = -(p - p_inf) / cp_scale
    const double bH = which == 0 ? -sin(theta) : cos(theta);
    const double bV = which == 0 ? cos(theta) : sin(theta);
    bP[m].w += -(bH * nn.x + bV * nn.y) * ds / cp_scale;
}

// bP += dJ/dprim of the stagnation-pressure loss J = sum (p0_inf - p0)^2 /
// (p0_inf^2 n) (stagnation_values_mod.h:51-80), p0 = p A^g, A = 1 + (gamma-1)/2
// M^2, M^2 = rho |u|^2 / (gamma p), g = gamma / (gamma - 1).
__global__ void k_objective_J(int n, const double4_32a *__restrict__ P, double gamma, double p0_inf,
                              double4_32a *__restrict__ bP)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double4_32a p = P[i];
    const double g = gamma / (gamma - 1);
    const double u2 = p.y * p.y + p.z * p.z;
    const double M2 = p.x * u2 / (gamma * p.w);
    const double A = 1 + 0.5 * (gamma - 1) * M2;
    const double Ag = pow(A, g);
    const double p0 = p.w * Ag;
    const double bp0 = -2.0 * (p0_inf - p0) / (p0_inf * p0_inf * n);
    const double dA = p.w * g * Ag / A * 0.5 * (gamma - 1);   // dp0 / dM^2
    double4_32a b = bP[i];
    b.x += bp0 * dA * (u2 / (gamma * p.w));
    b.y += bp0 * dA * (2.0 * p.x * p.y / (gamma * p.w));
    b.z += bp0 * dA * (2.0 * p.x * p.z / (gamma * p.w));
    b.w += bp0 * (Ag - dA * M2 / p.w);
    bP[i] = b;
}

// AdjView::geo_pt: 1 for a wall point and for a point with a wall neighbour.
__global__ void k_mark_geo(DevCloud c, uint8_t *__restrict__ geo_pt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    bool g = c.flag[i] == kWall;
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    for (int j = 0; j < nb && !g; j++) g = c.flag[c.e_nbr[base + 32LL * j]] == kWall;
    geo_pt[i] = g ? 1 : 0;
}

// The geometry bars the reverse kernels accumulated (per edge: vector,
// rotated vector, length; per point: normal, gradient and directional LSQ
// moments) pulled back to the point coordinates, unit weights: each point's
// edges add to its neighbour's and its own coordinate bars (FP64 atomics),
// and the point's normal bar (the accumulated one plus its edges' rotated
// vectors') is stored for the host's normal pull-back.  bx, by zeroed first.
__global__ void k_geom_pullback(AdjView a, double *__restrict__ bx, double *__restrict__ by,
                                double2 *__restrict__ bn)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.c.n) return;
    // a point whose geometry does not depend on a wall point accumulated no
    // geometry bars (AdjView::geo_pt): nothing to pull back
    if (!a.geo_pt[i]) {
        bn[i] = a.bnrm[i];
        return;
    }
    const DevCloud &c = a.c;
    const double2 nn = c.nrm[i];
    const double nx = nn.x, ny = nn.y;
    // bars of the three sums from those of {sxx, syy, sxy, 1/det} as the kernels read them
    auto mom_bar = [](const double4_32a &m, const double4_32a &b, double &bxx, double &byy, double &bxy) {
        bxx = b.x;
        byy = b.y;
        bxy = b.z;
        if (b.w == 0.0) return;
        const double bdet = -b.w * m.w * m.w;
        bxx += bdet * m.y;
        byy += bdet * m.x;
        bxy -= 2.0 * m.z * bdet;
    };
    double gbxx, gbyy, gbxy, fbxx[4], fbyy[4], fbxy[4];
    mom_bar(c.ggeo[i], a.bgmom[i], gbxx, gbyy, gbxy);
    for (int d = 0; d < 4; d++) mom_bar(c.fgeo[4 * i + d], a.bfmom[4 * i + d], fbxx[d], fbyy[d], fbxy[d]);
    double2 bni = a.bnrm[i];
    double sx = 0.0, sy = 0.0;
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const int k = c.e_nbr[e];
        const double4_32a g = c.e_geo[e], be = a.bedge[e];
        const double2 sn = c.e_sn[e];
        const double dx = g.x, dy = g.y, ds = sn.x, dn = sn.y;
        double bdx = be.x + 2.0 * dx * gbxx + dy * gbxy;
        double bdy = be.y + 2.0 * dy * gbyy + dx * gbxy;
        double bds = be.z, bdn = be.w;
        const unsigned bits = c.e_dir[e];
        for (int d = 0; d < 4; d++)
            if (bits & (1u << d)) {
                bds += 2.0 * ds * fbxx[d] + dn * fbxy[d];
                bdn += 2.0 * dn * fbyy[d] + ds * fbxy[d];
            }
        // ds = dx ny - dy nx, dn = dx nx + dy ny
        bdx += bds * ny + bdn * nx;
        bdy += -bds * nx + bdn * ny;
        bni.x += -bds * dy + bdn * dx;
        bni.y += bds * dx + bdn * dy;
        const double bd = a.bdist[e];
        if (bd != 0.0) {
            const double dist = c.e_dist[e];
            bdx += bd * dx / dist;
            bdy += bd * dy / dist;
        }
        atomicAdd(bx + k, bdx);
        atomicAdd(by + k, bdy);
        sx += bdx;
        sy += bdy;
    }
    atomicAdd(bx + i, -sx);
    atomicAdd(by + i, -sy);
    bn[i] = bni;
}

}  // namespace adjk

// ---------------------------------------------------------------------------
// Reverse of the mixed-precision iteration (qlskum_mixed.cu): the per-edge
// work in FP32 with the FP32 instantiations of the reverse-mode functions,
// neighbour bars scattered with FP32 atomics, the stage update's reverse in
// FP64 (adjk::k_update).  Each kernel differentiates what its forward kernel
// computes: the flux kernel's folded solve weights and branch-free half-range
// selection, the gradient's FP32 sums with the FP64 solve coefficients, q of
// the FP32-rounded state, the FP32 time step and wave speed.
namespace adjm {

using adj::KinBarT;

// one 16-byte vector reduction (sm_90 and later; float4 arrays are 16-byte aligned)
__device__ __forceinline__ void atomic_add4(float4 *p, const float v[4])
{
    atomicAdd(p, make_float4(v[0], v[1], v[2], v[3]));
}

__device__ __forceinline__ void ldf4(const float4 &a, float o[4]) { o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; }

__device__ __forceinline__ void x_flux_vjp(int f, const Kin<float> &k, float s1, const float bG[4], KinBarT<float> &kb)
{
    if (f == kInterior) adj::flux_x_vjp<float>(k, s1, bG, kb);
    else adj::flux_quad_vjp<float>(k, s1, (f == kOuter) ? 1.0f : -1.0f, bG, kb);
}

// Reverse of one end of one edge of the mixed flux kernel: the end's
// reconstruction (q, dq, max / min of the point the end belongs to), its
// primitive state and half-range moments, then the bars of the x and y
// half-range fluxes it enters, weighted by the folded solve weights (bs: the
// bar of the owner's weighted sum, signed + for the neighbour end, - for the
// owner's), back to the end's q, dq and max / min (added to bq ... bmn).
// The forward quantities come from mixed_end, the forward kernel's own
// function, once, and are reused by the reverse: the limiter's dn and dp,
// the state's beta and 1 / (2 beta) (which is also the moments' p / rho),
// sqrt(beta) and the moments' exp(-S^2) (taken back from
// B = exp(-S^2) / (2 sqrt(pi beta))), so the reverse has one division per
// active limiter component and no other division, exp or log.  The same
// derivatives as the generic reverse-mode functions (qtilde_to_prim_vjp,
// kin_vjp, edge_end_vjp) up to rounding.
__device__ __forceinline__ void end_vjp(const float2 *w2p, int f, float nx, float ny, float delx,
                                        float dely, float2 w, unsigned dir, const float bs[4], const float q[4],
                                        const float dx[4], const float dy[4], const float mx[4], const float mn[4],
                                        float e2, float bq[4], float bdx[4], float bdy[4], float bmx[4], float bmn[4])
{
    // the forward state of the end (mixed_end: the forward kernel's own function)
    MixedEnd st;
    mixed_end(nx, ny, delx, dely, q, dx, dy, mx, mn, e2, st);
    const Kin<float> &k = st.k;
    const float *dn = st.dn, *dp = st.dp, *phi = st.phi, *t = st.t;
    const float beta = st.beta, tm = st.tm, u1 = st.u1, u2 = st.u2, uq = st.uq, rsb = st.rsb, sb = st.sb;
    const float S1 = st.S1, S2 = st.S2, rho = k.rho;
    // the fluxes' reverse
    KinBarT<float> kb;
    float bG[4];
#pragma unroll
    for (int r = 0; r < 4; r++) bG[r] = w.x * bs[r];
    x_flux_vjp(f, k, (dir & kXpos) ? 1.0f : -1.0f, bG, kb);
#pragma unroll
    for (int r = 0; r < 4; r++) bG[r] = w.y * bs[r];
    adj::flux_y_vjp<float>(k, (dir & kYpos) ? 1.0f : -1.0f, bG, kb);
    const bool xb = (dir & (kXpos | kXneg)) == (kXpos | kXneg), yb = (dir & (kYpos | kYneg)) == (kYpos | kYneg);
    if (xb || yb) {
        const float2 w2 = *w2p;
        if (xb) {
#pragma unroll
            for (int r = 0; r < 4; r++) bG[r] = w2.x * bs[r];
            x_flux_vjp(f, k, -1.0f, bG, kb);
        }
        if (yb) {
#pragma unroll
            for (int r = 0; r < 4; r++) bG[r] = w2.y * bs[r];
            adj::flux_y_vjp<float>(k, -1.0f, bG, kb);
        }
    }
    // moments' reverse: (2 / sqrt(pi)) exp(-S^2) = 4 sb B
    float but = fmaf(2.0f * k.ut, kb.usq, kb.ut), bun = fmaf(2.0f * k.un, kb.usq, kb.un);
    const float bS1 = k.B1 * (4.0f * sb * kb.E1 - 2.0f * S1 * kb.B1);
    const float bS2 = k.B2 * (4.0f * sb * kb.E2 - 2.0f * S2 * kb.B2);
    but = fmaf(bS1, sb, but);
    bun = fmaf(bS2, sb, bun);
    float bbeta = (bS1 * k.ut + bS2 * k.un) * 0.5f * rsb - (kb.B1 * k.B1 + kb.B2 * k.B2) * tm;
    float btm = kb.pbr;
    float bu1 = but * ny + bun * nx, bu2 = bun * ny - but * nx;
    // state's reverse: rho = exp(t0 + beta uq - 2.5 log beta), u = (t1, t2) tm, tm = 1 / (2 beta)
    const float bT = kb.rho * rho;
    bbeta = fmaf(bT, uq - 5.0f * tm, bbeta);
    bu1 = fmaf(2.0f * bT * beta, u1, bu1);
    bu2 = fmaf(2.0f * bT * beta, u2, bu2);
    btm = fmaf(bu1, t[1], fmaf(bu2, t[2], btm));
    bbeta = fmaf(-2.0f * tm * tm, btm, bbeta);
    const float bt[4] = {bT, bu1 * tm, bu2 * tm, -0.5f * bbeta};
    // reconstruction's reverse (num / den with the common factor dn cancelled)
#pragma unroll
    for (int r = 0; r < 4; r++) {
        bq[r] += bt[r];
        float bdn = phi[r] * bt[r];
        if (phi[r] < 1.0f) {
            const float bphi = dn[r] * bt[r];
            const float base = fmaf(dp[r], dp[r], e2);
            const float den = fmaf(dn[r], dp[r], fmaf(2.0f * dn[r], dn[r], base));
            const float rden = __fdividef(1.0f, den);
            const float bnum = bphi * rden, bden = -bphi * phi[r] * rden;
            bdn += bnum * 2.0f * dp[r] + bden * fmaf(4.0f, dn[r], dp[r]);
            const float bdp = bnum * 2.0f * (dp[r] + dn[r]) + bden * fmaf(2.0f, dp[r], dn[r]);
            bq[r] -= bdp;
            if (dn[r] > 0.f) bmx[r] += bdp;
            else bmn[r] += bdp;
        }
        const float bg = -0.5f * bdn;
        bdx[r] = fmaf(bg, delx, bdx[r]);
        bdy[r] = fmaf(bg, dely, bdy[r]);
    }
}

template <bool UW> __device__ __forceinline__ float2 edge_del(const DevCloud &c, long long e)
{
    if (UW) return c.e_xy32[e];
    const float4 g = c.e_geo32[e];
    return make_float2(g.x, g.y);
}

// Reverse of the flux part of the mixed flux + update kernel for stage
// state (q, dq, qm): F = delta * acc, acc = sum_e w_e (G_k - G_i) over each
// edge's x and y half-ranges.  Given the bar of acc, bs = delta * bF
// (adjm::k_update), the two ends of an edge are independent, so each point
// reverses the ends that are its own: the owner ends of its edges (bar
// -bs_i, its class and normal) and the neighbour ends of the edges that have
// it as neighbour (bar +bs of the edge's owner, the owner's class and normal),
// pulled through the transposed list T.  The point's bars stay in
// registers and are stored once (no atomics, no zeroing); the point's own
// data (q, gradient, max / min: five float4), which every end it reverses
// reads, sits in the thread's slots of shared memory and is read back per
// end instead of being held in 20 registers (4 blocks of 128 per SM instead
// of 3).
__device__ __forceinline__ void lds_f4(const float4 *p, float o[4])
{
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(o[0]), "=f"(o[1]), "=f"(o[2]), "=f"(o[3])
                 : "r"((unsigned)__cvta_generic_to_shared(p)));
}

template <bool UW>
__global__ void __launch_bounds__(128, 4) k_flux(DevCloud c, AdjT T, const float4 *__restrict__ q,
                                                    const float4 *__restrict__ dq, const float4 *__restrict__ qm,
                                                    const float4 *__restrict__ acc, const float4 *__restrict__ bF,
                                                    const float4 *__restrict__ bsum,
                                                    float4 *__restrict__ bq, float4 *__restrict__ bdq,
                                                    float4 *__restrict__ bqm, float *__restrict__ bdelta)
{
    constexpr int B = 128;
    __shared__ float4 sown[5 * B];
    const int t = threadIdx.x;
    const int i = blockIdx.x * B + t;
    if (i >= c.n) return;
    const int f = c.flag[i];
    const double2 nn = c.nrm[i];
    const float nx = d2f(nn.x), ny = d2f(nn.y);
    sown[t] = q[i];
    sown[B + t] = dq[2 * i];
    sown[2 * B + t] = dq[2 * i + 1];
    sown[3 * B + t] = qm[2 * i];
    sown[4 * B + t] = qm[2 * i + 1];
    float qi[4], dxi[4], dyi[4], mxi[4], mni[4];
    auto own = [&]() {
        lds_f4(sown + t, qi);
        lds_f4(sown + B + t, dxi);
        lds_f4(sown + 2 * B + t, dyi);
        lds_f4(sown + 3 * B + t, mxi);
        lds_f4(sown + 4 * B + t, mni);
    };
    const float e2i = c.eps2_32[i];
    const float4 bFi = bF[i], ac = acc[i], bsi = bsum[i];
    bdelta[i] += bFi.x * ac.x + bFi.y * ac.y + bFi.z * ac.z + bFi.w * ac.w;
    float bqi[4] = {0, 0, 0, 0}, bdxi[4] = {0, 0, 0, 0}, bdyi[4] = {0, 0, 0, 0}, bmxi[4] = {0, 0, 0, 0},
          bmni[4] = {0, 0, 0, 0};
    // the owner ends of the point's edges, the next edge's data one edge ahead in registers
    {
        const float bs[4] = {-bsi.x, -bsi.y, -bsi.z, -bsi.w};
        const int nb = c.nbhs[i];
        const long long base = c.slice_base[i >> 5] + (i & 31);
        float2 dn2 = make_float2(0.f, 0.f), wn = make_float2(0.f, 0.f);
        unsigned dirn = 0;
        if (nb > 0) {
            dn2 = edge_del<UW>(c, base);
            wn = c.e_w32[base];
            dirn = c.e_dir[base];
        }
        for (int j = 0; j < nb; j++) {
            const long long e = base + 32LL * j;
            const float2 d = dn2, w = wn;
            const unsigned dir = dirn;
            if (j + 1 < nb) {
                dn2 = edge_del<UW>(c, e + 32);
                wn = c.e_w32[e + 32];
                dirn = c.e_dir[e + 32];
            }
            own();
            end_vjp(c.e_w32b + e, f, nx, ny, d.x, d.y, w, dir, bs, qi, dxi, dyi, mxi, mni, e2i, bqi, bdxi, bdyi,
                    bmxi, bmni);
        }
    }
    // the neighbour ends of the edges into the point: the next slot's data and
    // its owner's bar one edge ahead in registers, the owner index two ahead
    {
        const int nb = T.nb[i];
        const long long base = T.sbase[i >> 5] + (i & 31);
        float4 bn = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 dn2 = make_float2(0.f, 0.f), wn = make_float2(0.f, 0.f), onn = make_float2(0.f, 1.f);
        unsigned dfn = 0;
        int en = 0, srcnn = 0;
        if (nb > 0) {
            bn = bsum[T.src[base]];
            dn2 = T.xy[base];
            wn = T.w[base];
            onn = T.nrm[base];
            dfn = T.df[base];
            en = T.e[base];
        }
        if (nb > 1) srcnn = T.src[base + 32];
        for (int j = 0; j < nb; j++) {
            const long long t = base + 32LL * j;
            const float bs[4] = {bn.x, bn.y, bn.z, bn.w};
            const float2 d = dn2, w = wn, on = onn;
            const unsigned df = dfn;
            const int e = en;
            if (j + 1 < nb) {
                bn = bsum[srcnn];
                dn2 = T.xy[t + 32];
                wn = T.w[t + 32];
                onn = T.nrm[t + 32];
                dfn = T.df[t + 32];
                en = T.e[t + 32];
            }
            if (j + 2 < nb) srcnn = T.src[t + 64];
            own();
            end_vjp(c.e_w32b + e, (int)(df >> 4), on.x, on.y, d.x, d.y, w, df & 15u, bs, qi, dxi, dyi, mxi, mni,
                    e2i, bqi, bdxi, bdyi, bmxi, bmni);
        }
    }
    bq[i] = mk4(bqi);
    bdq[2 * i] = mk4(bdxi);
    bdq[2 * i + 1] = mk4(bdyi);
    bqm[2 * i] = mk4(bmxi);
    bqm[2 * i + 1] = mk4(bmni);
}

// Reverse of one mixed inner step, dq_out = dq0 + 0.5 (dq_in - A),
// A = sum_e g_e (d_e.dq_in_k) with the folded solve weights g_e
// (inner_point of the mixed kernels): the bar of dq_out goes to dq0
// (accumulated over the steps in bdq0), half of it to the point's own dq_in,
// and through A of each edge's owner i to the neighbour's dq_in: the point
// pulls -0.5 d (g . bdq_out_i) over the edges into it.  Stores bdq_in.
__global__ void k_inner(DevCloud c, AdjT T, const float4 *__restrict__ bdq_out, float4 *__restrict__ bdq_in,
                        float4 *__restrict__ bdq0, int first)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    float ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0};
    const int nb = T.nb[i];
    const long long base = T.sbase[i >> 5] + (i & 31);
    // the transposed list is streamed once (evict-first), the owners' bars
    // gathered as 32-byte pairs (the forward inner step's access pattern)
#pragma unroll 2
    for (int j = 0; j < nb; j++) {
        const long long t = base + 32LL * j;
        const int src = __ldcs(T.src + t);
        const float2 d = __ldcs(T.xy + t), gw = __ldcs(T.gw + t);
        float4 b0, b1;
        ldg_2x4(bdq_out + 2 * src, b0, b1);
        float bx[4], by[4];
        ldf4(b0, bx);
        ldf4(b1, by);
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const float bu = fmaf(gw.x, bx[r], gw.y * by[r]);
            ax[r] = fmaf(d.x, bu, ax[r]);
            ay[r] = fmaf(d.y, bu, ay[r]);
        }
    }
    float bx[4], by[4];
    ldf4(bdq_out[2 * i], bx);
    ldf4(bdq_out[2 * i + 1], by);
    float a0[4] = {0, 0, 0, 0}, a1[4] = {0, 0, 0, 0};
    if (!first) {
        ldf4(bdq0[2 * i], a0);
        ldf4(bdq0[2 * i + 1], a1);
    }
    float ox[4], oy[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        a0[r] += bx[r];
        a1[r] += by[r];
        ox[r] = 0.5f * (bx[r] - ax[r]);
        oy[r] = 0.5f * (by[r] - ay[r]);
    }
    bdq0[2 * i] = mk4(a0);
    bdq0[2 * i + 1] = mk4(a1);
    bdq_in[2 * i] = mk4(ox);
    bdq_in[2 * i + 1] = mk4(oy);
}

// Reverse of the mixed gradient and neighbour max / min (q_variables_mod.h:36-118).
// The bar of the stage's first-order gradient is bdq + bdq0 (the inner
// steps' direct part; bdq0 NULL without inner steps).
template <bool UW>
__global__ void k_grad(DevCloud c, const float4 *__restrict__ q, const float4 *__restrict__ bdq,
                       const float4 *__restrict__ bdq0, const float4 *__restrict__ bqm, float4 *__restrict__ bq)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    float bx[4], by[4], bmax[4], bmin[4], qi[4], b0x[4], b0y[4];
    ldf4(bdq[2 * i], bx);
    ldf4(bdq[2 * i + 1], by);
    if (bdq0) {
        ldf4(bdq0[2 * i], b0x);
        ldf4(bdq0[2 * i + 1], b0y);
#pragma unroll
        for (int r = 0; r < 4; r++) {
            bx[r] += b0x[r];
            by[r] += b0y[r];
        }
    }
    ldf4(bqm[2 * i], bmax);
    ldf4(bqm[2 * i + 1], bmin);
    ldf4(q[i], qi);
    float qmax[4], qmin[4];
    int amax[4], amin[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        qmax[r] = qmin[r] = qi[r];
        amax[r] = amin[r] = i;
    }
    float bqi[4] = {0, 0, 0, 0};
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const int k = __ldcs(c.e_nbr + e);
        const float2 gw = __ldcs(c.e_gw32 + e);
        float qk[4], bqk[4];
        ldf4(q[k], qk);
#pragma unroll
        for (int r = 0; r < 4; r++) {
            if (qk[r] > qmax[r]) { qmax[r] = qk[r]; amax[r] = k; }
            if (qk[r] < qmin[r]) { qmin[r] = qk[r]; amin[r] = k; }
            const float bt = fmaf(gw.x, bx[r], gw.y * by[r]);
            bqk[r] = bt;
            bqi[r] -= bt;
        }
        atomic_add4(bq + k, bqk);
    }
    atomic_add4(bq + i, bqi);
    float *bqd = reinterpret_cast<float *>(bq);
#pragma unroll
    for (int r = 0; r < 4; r++) {
        if (bmax[r] != 0.f) atomicAdd(bqd + 4 * (size_t)amax[r] + r, bmax[r]);
        if (bmin[r] != 0.f) atomicAdd(bqd + 4 * (size_t)amin[r] + r, bmin[r]);
    }
}

// bP += (dq/dP)^T bq for q = prim_to_q of the FP32-rounded state.
__global__ void k_q(int n, const double4_32a *__restrict__ P, const float4 *__restrict__ bq,
                    double4_32a *__restrict__ bP)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double4_32a p = P[i];
    const float pf[4] = {d2f(p.x), d2f(p.y), d2f(p.z), d2f(p.w)};
    float b[4], g[4] = {0, 0, 0, 0};
    ldf4(bq[i], b);
    adj::prim_to_q_vjp<float>(pf, b, g);
    double4_32a acc = bP[i];
    acc.x += f2d(g[0]);
    acc.y += f2d(g[1]);
    acc.z += f2d(g[2]);
    acc.w += f2d(g[3]);
    bP[i] = acc;
}

// Reverse of the FP32 local time step min(1, min_k cfl |dr| / c_k): the bar
// goes to the wave speed of the neighbour that set the minimum.
template <bool UW>
__global__ void k_delta(DevCloud c, const float *__restrict__ cs, const float *__restrict__ bdelta, float cfl,
                        float *__restrict__ bcs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n || bdelta[i] == 0.f) return;
    float min_dt = 1.0f, carg = 0.f, darg = 0.f;
    int arg = -1;
    const int nb = c.nbhs[i];
    const long long base = c.slice_base[i >> 5] + (i & 31);
    for (int j = 0; j < nb; j++) {
        const long long e = base + 32LL * j;
        const int k = c.e_nbr[e];
        const float d = c.e_dist32[e], ck = cs[k];
        const float dt = cfl * __fdividef(d, ck);
        if (dt < min_dt) {
            min_dt = dt;
            arg = k;
            carg = ck;
            darg = d;
        }
    }
    if (arg >= 0) atomicAdd(bcs + arg, -bdelta[i] * cfl * darg / (carg * carg));
}

// bP += (dc/dP)^T bc for the FP32 wave speed |u| + 3 sqrt(p / rho).
__global__ void k_wave(int n, const double4_32a *__restrict__ P, const float *__restrict__ bc,
                       double4_32a *__restrict__ bP)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || bc[i] == 0.f) return;
    const double4_32a p = P[i];
    const float pf[4] = {d2f(p.x), d2f(p.y), d2f(p.z), d2f(p.w)};
    float g[4] = {0, 0, 0, 0};
    adj::wave_speed_vjp<float>(pf, bc[i], g);
    double4_32a acc = bP[i];
    acc.x += f2d(g[0]);
    acc.y += f2d(g[1]);
    acc.z += f2d(g[2]);
    acc.w += f2d(g[3]);
    bP[i] = acc;
}

// Reverse of one SSPRK stage update (the FP64 update of the mixed flux
// kernel), evaluated in FP32 on FP64-stored states and bars: bP (the bar of
// Pout on entry) becomes the update's part of the bar of Pin; bF the bar of
// the flux residual and bsum = delta * bF the bar of the flux kernel's
// weighted sum; stage 4 adds to bPold; outer points add the free-stream
// velocity bars (one FP64 atomic per warp).
__global__ void k_update(DevCloud c, CaseConst K, const double4_32a *__restrict__ Pin,
                         const double4_32a *__restrict__ Pold, const double4_32a *__restrict__ Pout, int rk,
                         const float *__restrict__ delta, double4_32a *__restrict__ bP,
                         double4_32a *__restrict__ bPold, float4 *__restrict__ bF, float4 *__restrict__ bsum,
                         double *__restrict__ buinf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float bu1 = 0.f, bu2 = 0.f;
    if (i < c.n) {
        const int f = c.flag[i];
        const double2 nn = c.nrm[i];
        const double4_32a a = Pin[i], b = Pold[i], o = Pout[i], g = bP[i];
        const float pin[4] = {d2f(a.x), d2f(a.y), d2f(a.z), d2f(a.w)};
        const float pold[4] = {d2f(b.x), d2f(b.y), d2f(b.z), d2f(b.w)};
        const float pout[4] = {d2f(o.x), d2f(o.y), d2f(o.z), d2f(o.w)};
        const float bout[4] = {d2f(g.x), d2f(g.y), d2f(g.z), d2f(g.w)};
        float bin[4] = {0, 0, 0, 0}, bo[4] = {0, 0, 0, 0}, bf[4] = {0, 0, 0, 0}, bnx = 0.f, bny = 0.f;
        adj::stage_update_vjp<float>(K, f, d2f(nn.x), d2f(nn.y), pin, pold, pout, rk, bout, bin, bo, bf, bnx, bny,
                                     bu1, bu2);
        bP[i] = make_double4_32a(f2d(bin[0]), f2d(bin[1]), f2d(bin[2]), f2d(bin[3]));
        bF[i] = make_float4(bf[0], bf[1], bf[2], bf[3]);
        const float dl = delta[i];
        bsum[i] = make_float4(dl * bf[0], dl * bf[1], dl * bf[2], dl * bf[3]);
        if (rk == 3) {
            double4_32a acc = bPold[i];
            acc.x += f2d(bo[0]);
            acc.y += f2d(bo[1]);
            acc.z += f2d(bo[2]);
            acc.w += f2d(bo[3]);
            bPold[i] = acc;
        }
    }
    double d1 = f2d(bu1), d2 = f2d(bu2);
    for (int o = 16; o > 0; o >>= 1) {
        d1 += __shfl_down_sync(0xffffffffu, d1, o);
        d2 += __shfl_down_sync(0xffffffffu, d2, o);
    }
    if ((threadIdx.x & 31) == 0 && (d1 != 0.0 || d2 != 0.0)) {
        atomicAdd(buinf, d1);
        atomicAdd(buinf + 1, d2);
    }
}

}  // namespace adjm

// ------------------------------------------------------------- launchers

namespace adjl {

void update(const Launch &L, const AdjView &a, const CaseConst &K, const double4_32a *Pin, const double4_32a *Pold,
            const double4_32a *Pout, int rk, double4_32a *bP, double4_32a *bPold, double4_32a *bF, double *buinf)
{
    adjk::k_update<<<adjk::grid_for(a.c.n, 128), 128, 0, L.stream>>>(a, K, Pin, Pold, Pout, rk, bP, bPold, bF, buinf);
}

void flux(const Launch &L, const AdjView &a, const double4_32a *q, const double4_32a *dq, const double4_32a *qm,
          const double *delta, const double4_32a *flux, const double *sums, const double *ends, long long ns,
          const double4_32a *bF, double4_32a *bq, double4_32a *bdq, double4_32a *bqm, double *bdelta)
{
    adjk::k_flux<0><<<adjk::grid_for(a.c.n, 128), 128, 0, L.stream>>>(a, q, dq, qm, delta, flux, nullptr, ends, ns,
                                                                       bF, bq, bdq, bqm, bdelta);
    if (a.bedge && a.n_geo > 0)
        adjk::k_flux<2><<<adjk::grid_for(a.n_geo, 128), 128, 0, L.stream>>>(a, q, dq, qm, delta, flux, sums, ends, ns,
                                                                            bF, bq, bdq, bqm, bdelta);
}

void inner(const Launch &L, const AdjView &a, const double4_32a *q, const double4_32a *dq_in,
           const double4_32a *bdq_out, double4_32a *bq, double4_32a *bdq_in)
{
    adjk::k_inner<0><<<adjk::grid_for(a.c.n, 128), 128, 0, L.stream>>>(a, q, dq_in, bdq_out, bq, bdq_in);
    if (a.bedge && a.n_geo > 0)
        adjk::k_inner<2><<<adjk::grid_for(a.n_geo, 128), 128, 0, L.stream>>>(a, q, dq_in, bdq_out, bq, bdq_in);
}

void grad(const Launch &L, const AdjView &a, const double4_32a *q, const double4_32a *bdq, const double4_32a *bqm,
          double4_32a *bq)
{
    adjk::k_grad<0><<<adjk::grid_for(a.c.n, 128), 128, 0, L.stream>>>(a, q, bdq, bqm, bq);
    if (a.bedge && a.n_geo > 0)
        adjk::k_grad<2><<<adjk::grid_for(a.n_geo, 128), 128, 0, L.stream>>>(a, q, bdq, bqm, bq);
}

void qvars(const Launch &L, int n, const double4_32a *P, const double4_32a *bq, double4_32a *bP)
{
    adjk::k_q<<<adjk::grid_for(n, 256), 256, 0, L.stream>>>(n, P, bq, bP);
}

void delta(const Launch &L, const AdjView &a, const double4_32a *P, const double *bdelta, double cfl, double *bc,
           double4_32a *bP)
{
    if (a.bdist)
        adjk::k_delta<true><<<adjk::grid_for(a.c.n, 128), 128, 0, L.stream>>>(a, P, bdelta, cfl, bc);
    else
        adjk::k_delta<false><<<adjk::grid_for(a.c.n, 128), 128, 0, L.stream>>>(a, P, bdelta, cfl, bc);
    adjk::k_wave<<<adjk::grid_for(a.c.n, 256), 256, 0, L.stream>>>(a.c.n, P, bc, bP);
}

void objective_J(const Launch &L, int n, const double4_32a *P, double gamma, double p0_inf, double4_32a *bP)
{
    adjk::k_objective_J<<<adjk::grid_for(n, 256), 256, 0, L.stream>>>(n, P, gamma, p0_inf, bP);
}

void objective(const Launch &L, const AdjView &a, const int *wall_perm, const double4_32a *wall_geo, int n_wall,
               double cp_scale, double theta, int which, double4_32a *bP)
{
    if (n_wall > 0)
        adjk::k_objective<<<adjk::grid_for(n_wall, 128), 128, 0, L.stream>>>(a, wall_perm, wall_geo, n_wall, cp_scale,
                                                                            theta, which, bP);
}

void mark_geo_points(const Launch &L, const DevCloud &c, uint8_t *geo_pt)
{
    adjk::k_mark_geo<<<adjk::grid_for(c.n, 128), 128, 0, L.stream>>>(c, geo_pt);
}

void geom_pullback(const Launch &L, const AdjView &a, double *bx, double *by, double2 *bn)
{
    adjk::k_geom_pullback<<<adjk::grid_for(a.c.n, 128), 128, 0, L.stream>>>(a, bx, by, bn);
}

}  // namespace adjl

namespace adjml {

static inline int grid_for(int n, int block) { return (n + block - 1) / block; }

void flux(const Launch &L, const DevCloud &c, const AdjT &T, const float4 *q, const float4 *dq, const float4 *qm,
          const float4 *acc, const float4 *bF, const float4 *bs, float4 *bq, float4 *bdq, float4 *bqm, float *bdelta)
{
    const int g = grid_for(c.n, 128);
    if (c.unit_w) adjm::k_flux<true><<<g, 128, 0, L.stream>>>(c, T, q, dq, qm, acc, bF, bs, bq, bdq, bqm, bdelta);
    else adjm::k_flux<false><<<g, 128, 0, L.stream>>>(c, T, q, dq, qm, acc, bF, bs, bq, bdq, bqm, bdelta);
}

void inner(const Launch &L, const DevCloud &c, const AdjT &T, const float4 *bdq_out, float4 *bdq_in, float4 *bdq0,
           bool first)
{
    adjm::k_inner<<<grid_for(c.n, 128), 128, 0, L.stream>>>(c, T, bdq_out, bdq_in, bdq0, first);
}

void grad(const Launch &L, const DevCloud &c, const float4 *q, const float4 *bdq, const float4 *bdq0,
          const float4 *bqm, float4 *bq)
{
    if (c.unit_w) adjm::k_grad<true><<<grid_for(c.n, 128), 128, 0, L.stream>>>(c, q, bdq, bdq0, bqm, bq);
    else adjm::k_grad<false><<<grid_for(c.n, 128), 128, 0, L.stream>>>(c, q, bdq, bdq0, bqm, bq);
}

void update(const Launch &L, const DevCloud &c, const CaseConst &K, const double4_32a *Pin, const double4_32a *Pold,
            const double4_32a *Pout, int rk, const float *delta, double4_32a *bP, double4_32a *bPold, float4 *bF,
            float4 *bs, double *buinf)
{
    adjm::k_update<<<grid_for(c.n, 128), 128, 0, L.stream>>>(c, K, Pin, Pold, Pout, rk, delta, bP, bPold, bF, bs,
                                                           buinf);
}

void qvars(const Launch &L, int n, const double4_32a *P, const float4 *bq, double4_32a *bP)
{
    adjm::k_q<<<grid_for(n, 256), 256, 0, L.stream>>>(n, P, bq, bP);
}

void delta(const Launch &L, const DevCloud &c, const double4_32a *P, const float *cs, const float *bdelta, float cfl,
           float *bcs, double4_32a *bP)
{
    if (c.unit_w) adjm::k_delta<true><<<grid_for(c.n, 128), 128, 0, L.stream>>>(c, cs, bdelta, cfl, bcs);
    else adjm::k_delta<false><<<grid_for(c.n, 128), 128, 0, L.stream>>>(c, cs, bdelta, cfl, bcs);
    adjm::k_wave<<<grid_for(c.n, 256), 256, 0, L.stream>>>(c.n, P, bcs, bP);
}

}  // namespace adjml
}  // namespace qlskum
