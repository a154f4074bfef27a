// Host layer of the q-LSKUM GB300 library: the C ABI declared in
// include/qlskum.h.
//
// Set-up work that the reference repeats every stage but that only depends on
// the geometry (normals, sub-stencil split, least-squares moments and their
// determinants, edge vectors, limiter epsilon) runs here once, in FP64 with
// the reference's own operation order.  This file must be compiled with
// -ffp-contract=off so that no FMA changes a rounding: the sub-stencil split
// is then bit-identical to the reference's on the same machine.
#include "qlskum.h"
#include "qlskum_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

using namespace qlskum;

namespace {

thread_local std::string g_create_error;

struct Precomp {
    // original order
    std::vector<double> nx, ny;
    std::vector<int> sub_counts;   // [n][4]
    std::vector<int> sub_lists;    // [n][4][20], 1-based
    std::vector<uint8_t> edge_dir; // [n][20]
    std::vector<double> geo;       // [n][20][4]: delx, dely, w*delx, w*dely
    std::vector<double> sn;        // [n][20][2]: dels*w, deln*w
    std::vector<double> dist;      // [n][20]
    std::vector<double> ggeo;      // [n][4]
    std::vector<double> fgeo;      // [n][4][4]
    std::vector<double> eps2;      // [n]
    // drop what only the device upload needs (keeps normals and sub-stencils)
    void release_upload_data()
    {
        for (auto *v : {&geo, &sn, &dist, &ggeo, &fgeo, &eps2}) std::vector<double>().swap(*v);
        std::vector<uint8_t>().swap(edge_dir);
    }
};

std::string fmt(const char *f, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, f);
    vsnprintf(buf, sizeof buf, f, ap);
    va_end(ap);
    return buf;
}

// Interleave the low 21 bits of x and y.
uint64_t morton2(uint32_t x, uint32_t y)
{
    auto spread = [](uint64_t v) {
        v &= 0x1fffffULL;
        v = (v | (v << 32)) & 0x1f00000000ffffULL;
        v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
        v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
        v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
        v = (v | (v << 2)) & 0x1249249249249249ULL;
        return v;
    };
    return spread(x) | (spread(y) << 1);
}

}  // namespace

struct DeviceArena {
    std::vector<void *> ptrs;
    cudaError_t err = cudaSuccess;
    template <typename T> T *alloc(size_t count)
    {
        void *p = nullptr;
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            err = e;
            return nullptr;
        }
        ptrs.push_back(p);
        return static_cast<T *>(p);
    }
    void release()
    {
        for (void *p : ptrs) cudaFree(p);
        ptrs.clear();
    }
};

struct qlskum_handle {
    qlskum_params prm{};
    int n = 0, np = 0, nslices = 0;
    int shape_points = 0;
    std::vector<int> perm, iperm;
    Precomp pc;
    DeviceArena arena;
    DevCloud dc;
    CaseConst K{};
    State64 s64;
    State32 s32;
    Reduce R;
    Launch L;
    long long launches = 0;
    int pcur = 0, pold = 1;
    int dcur = 0;
    bool inner_pending = false;
    bool derived_valid = false;  // q[0] and cspeed match prim[pcur] for the fused solver
    int it = 0;
    double *d_obj = nullptr;
    double *d_obj_partial = nullptr;
    double *d_entropy = nullptr;
    double *d_last = nullptr;
    int *d_wall_perm = nullptr;
    double4_32a *d_wall_geo = nullptr;
    cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
    // launch shape of the mixed fused kernel and of the point kernels, set by
    // tune() on the first fused iteration unless params.block_size fixes it
    int flux_variant = 0;
    bool tuned = false;
    // per-kernel event timing (qlskum_set_kernel_timing)
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    double kt_ms[4] = {0, 0, 0, 0};
    long long kt_n[4] = {0, 0, 0, 0};
    std::string err;
};

namespace {

qlskum_status fail(qlskum_handle *h, qlskum_status s, const std::string &msg)
{
    if (h) h->err = msg;
    else g_create_error = msg;
    return s;
}

qlskum_status cuda_fail(qlskum_handle *h, cudaError_t e, const char *where)
{
    return fail(h, QLSKUM_ERR_CUDA, fmt("%s: %s", where, cudaGetErrorString(e)));
}

#define CK(h, call)                                          \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
    } while (0)

qlskum_status check_launch(qlskum_handle *h, const char *where)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(h, e, where);
    return QLSKUM_OK;
}

// ------------------------------------------------------------ validation

qlskum_status validate(const qlskum_cloud *c, const qlskum_params *p, int *shape_points)
{
    if (!c || !p) return fail(nullptr, QLSKUM_ERR_INVALID, "null cloud or params");
    if (c->n < 1) return fail(nullptr, QLSKUM_ERR_INVALID, "cloud has no points");
    if (!c->x || !c->y || !c->left || !c->right || !c->flag_1 || !c->flag_2 || !c->min_dist || !c->nbhs || !c->conn)
        return fail(nullptr, QLSKUM_ERR_INVALID, "null cloud array");
    if (p->inner_iterations < 0) return fail(nullptr, QLSKUM_ERR_INVALID, "inner_iterations < 0");
    if (p->precision != QLSKUM_FP64 && p->precision != QLSKUM_MIXED)
        return fail(nullptr, QLSKUM_ERR_INVALID, fmt("unknown precision %d", p->precision));
    if (p->block_size != 0 && (p->block_size < 32 || p->block_size > 1024 || p->block_size % 32))
        return fail(nullptr, QLSKUM_ERR_INVALID, "block_size must be 0 or a multiple of 32 in [32, 1024]");
    const int n = c->n;
    int sp = 0;
    for (int i = 0; i < n; i++) {
        int f = c->flag_1[i];
        if (f < 0 || f > 2) return fail(nullptr, QLSKUM_ERR_INVALID, fmt("point %d: flag_1=%d not in 0..2", i + 1, f));
        int nb = c->nbhs[i];
        if (nb < 0 || nb > QLSKUM_MAX_NBHS)
            return fail(nullptr, QLSKUM_ERR_INVALID, fmt("point %d: nbhs=%d not in 0..20", i + 1, nb));
        for (int r = 0; r < nb; r++) {
            int k = c->conn[(size_t)i * QLSKUM_MAX_NBHS + r];
            if (k < 1 || k > n)
                return fail(nullptr, QLSKUM_ERR_INVALID, fmt("point %d: neighbour %d out of range", i + 1, k));
        }
        if (f == kWall || f == kOuter) {
            if (c->left[i] < 1 || c->left[i] > n || c->right[i] < 1 || c->right[i] > n)
                return fail(nullptr, QLSKUM_ERR_INVALID, fmt("point %d: left/right out of range", i + 1));
        }
        if (!std::isfinite(c->x[i]) || !std::isfinite(c->y[i]) || !std::isfinite(c->min_dist[i]))
            return fail(nullptr, QLSKUM_ERR_INVALID, fmt("point %d: non-finite coordinate or min_dist", i + 1));
        if (c->flag_2[i] > 0) sp++;
    }
    // compute_cl_cd_cm walks points 1..shape_points (compute_force_coeffs_mod.h:25-27)
    for (int m = 0; m < sp; m++) {
        if (c->left[m] < 1 || c->left[m] > n || c->right[m] < 1 || c->right[m] > n)
            return fail(nullptr, QLSKUM_ERR_INVALID,
                        fmt("point %d: one of the first shape_points=%d points has no valid left/right", m + 1, sp));
    }
    *shape_points = sp;
    return QLSKUM_OK;
}

// ---------------------------------------------------- geometry (host, FP64)

qlskum_status precompute(const qlskum_cloud *c, const qlskum_params *p, Precomp &P)
{
    const int n = c->n;
    const int NB = QLSKUM_MAX_NBHS;
    P.nx.assign(n, 0.0);
    P.ny.assign(n, 0.0);
    // point_normals_mod.h:17-55
    for (int i = 0; i < n; i++) {
        int f = c->flag_1[i];
        if (f == kWall || f == kOuter) {
            int l = c->left[i] - 1, r = c->right[i] - 1;
            double lx = c->x[l], ly = c->y[l], mx = c->x[i], my = c->y[i], rx = c->x[r], ry = c->y[r];
            double nx1 = my - ly, nx2 = ry - my, ny1 = mx - lx, ny2 = rx - mx;
            double nx = 0.5 * (nx1 + nx2), ny = 0.5 * (ny1 + ny2);
            double det = std::sqrt(nx * nx + ny * ny);
            P.nx[i] = -nx / det;
            P.ny[i] = ny / det;
        } else {
            P.nx[i] = 0;
            P.ny[i] = 1;
        }
    }
    P.sub_counts.assign((size_t)n * 4, 0);
    P.sub_lists.assign((size_t)n * 4 * NB, 0);
    P.edge_dir.assign((size_t)n * NB, 0);
    P.geo.assign((size_t)n * NB * 4, 0.0);
    P.sn.assign((size_t)n * NB * 2, 0.0);
    P.dist.assign((size_t)n * NB, 0.0);
    P.ggeo.assign((size_t)n * 4, 0.0);
    P.fgeo.assign((size_t)n * 16, 0.0);
    P.eps2.assign(n, 0.0);
    const double power = p->power;
    for (int i = 0; i < n; i++) {
        const int f = c->flag_1[i];
        const double xi = c->x[i], yi = c->y[i], nx = P.nx[i], ny = P.ny[i];
        const double tx = ny, ty = -nx;
        double gxx = 0., gyy = 0., gxy = 0.;
        double fxx[4] = {0, 0, 0, 0}, fyy[4] = {0, 0, 0, 0}, fxy[4] = {0, 0, 0, 0};
        for (int r = 0; r < c->nbhs[i]; r++) {
            const int k = c->conn[(size_t)i * NB + r] - 1;
            const double delx = c->x[k] - xi, dely = c->y[k] - yi;
            // generate_connectivity_mod.h:24-83 / :91-153 / :155-219
            const double dels = delx * tx + dely * ty;
            const double deln = delx * nx + dely * ny;
            unsigned bits = 0;
            if (dels <= 0.0) bits |= kXpos;
            if (dels >= 0.0) bits |= kXneg;
            if (f == kInterior) {
                if (deln <= 0.0) bits |= kYpos;
                if (deln >= 0.0) bits |= kYneg;
            } else if (f == kWall) {
                bits |= kYneg;
            } else {
                bits |= kYpos;
            }
            P.edge_dir[(size_t)i * NB + r] = (uint8_t)bits;
            for (int d = 0; d < 4; d++)
                if (bits & (1u << d)) {
                    int &cnt = P.sub_counts[(size_t)i * 4 + d];
                    P.sub_lists[((size_t)i * 4 + d) * NB + cnt] = k + 1;
                    cnt++;
                }
            // q_variables_mod.h:80-88: gradient weights and moments
            const double dist = std::sqrt(delx * delx + dely * dely);
            const double w = std::pow(dist, power);
            gxx = gxx + delx * delx * w;
            gyy = gyy + dely * dely * w;
            gxy = gxy + delx * dely * w;
            double *G = &P.geo[((size_t)i * NB + r) * 4];
            G[0] = delx;
            G[1] = dely;
            G[2] = w * delx;
            G[3] = w * dely;
            // interior_fluxes_mod.h:50-70: rotated-frame weights and moments
            const double fdist = std::sqrt(dels * dels + deln * deln);
            const double fw = std::pow(fdist, power);
            const double dels_w = dels * fw, deln_w = deln * fw;
            P.sn[((size_t)i * NB + r) * 2] = dels_w;
            P.sn[((size_t)i * NB + r) * 2 + 1] = deln_w;
            for (int d = 0; d < 4; d++)
                if (bits & (1u << d)) {
                    fxx[d] = fxx[d] + dels * dels_w;
                    fyy[d] = fyy[d] + deln * deln_w;
                    fxy[d] = fxy[d] + dels * deln_w;
                }
            // state_update_mod.h:479-481
            double dd = (c->x[k] - xi) * (c->x[k] - xi) + (c->y[k] - yi) * (c->y[k] - yi);
            P.dist[(size_t)i * NB + r] = std::sqrt(dd);
        }
        double det = gxx * gyy - gxy * gxy;
        P.ggeo[(size_t)i * 4 + 0] = gxx;
        P.ggeo[(size_t)i * 4 + 1] = gyy;
        P.ggeo[(size_t)i * 4 + 2] = gxy;
        P.ggeo[(size_t)i * 4 + 3] = 1.0 / det;
        if (!(det != 0.0) || !std::isfinite(1.0 / det))
            return fail(nullptr, QLSKUM_ERR_DEGENERATE,
                        fmt("point %d: singular least-squares matrix of its full stencil (nbhs=%d)", i + 1, c->nbhs[i]));
        const bool used[3][4] = {{true, true, false, true}, {true, true, true, true}, {true, true, true, false}};
        for (int d = 0; d < 4; d++) {
            double fd = fxx[d] * fyy[d] - fxy[d] * fxy[d];
            double *F = &P.fgeo[((size_t)i * 4 + d) * 4];
            F[0] = fxx[d];
            F[1] = fyy[d];
            F[2] = fxy[d];
            F[3] = 1.0 / fd;
            if (used[f][d] && (!(fd != 0.0) || !std::isfinite(1.0 / fd))) {
                static const char *nm[4] = {"xpos", "xneg", "ypos", "yneg"};
                return fail(nullptr, QLSKUM_ERR_DEGENERATE,
                            fmt("point %d: %s sub-stencil (%d points) has a singular least-squares matrix", i + 1,
                                nm[d], P.sub_counts[(size_t)i * 4 + d]));
            }
        }
        // limiters_mod.h:84-85
        double epsi = p->vl_const * c->min_dist[i];
        epsi = std::pow(epsi, 3);
        P.eps2[i] = epsi * epsi;
    }
    return QLSKUM_OK;
}

void set_case(qlskum_handle *h)
{
    CaseConst &K = h->K;
    K.pi = 4 * std::atan(1.0);
    K.rho_inf = 1.0;
    K.pr_inf = 1.0 / 1.4;
    K.gamma = 1.4;
    K.mach = h->prm.mach;
    K.theta = h->prm.aoa * K.pi / 180;
    K.u1_inf = h->prm.mach * std::cos(K.theta);
    K.u2_inf = h->prm.mach * std::sin(K.theta);
    K.cfl = h->prm.cfl;
}

qlskum_status ensure_hist(qlskum_handle *h, int needed)
{
    if (needed <= h->R.capacity) return QLSKUM_OK;
    int cap = std::max(1024, h->R.capacity);
    while (cap < needed) cap *= 2;
    double *nh = nullptr;
    CK(h, cudaMalloc(&nh, sizeof(double) * 3 * (size_t)cap));
    CK(h, cudaMemsetAsync(nh, 0, sizeof(double) * 3 * (size_t)cap, h->L.stream));
    if (h->R.hist) {
        CK(h, cudaMemcpyAsync(nh, h->R.hist, sizeof(double) * 3 * (size_t)h->R.capacity, cudaMemcpyDeviceToDevice,
                              h->L.stream));
        CK(h, cudaStreamSynchronize(h->L.stream));
        cudaFree(h->R.hist);
    }
    h->R.hist = nh;
    h->R.capacity = cap;
    for (auto &g : h->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    return QLSKUM_OK;
}

qlskum_status tune(qlskum_handle *h);

qlskum_status ensure_derived(qlskum_handle *h)
{
    if (h->derived_valid) return QLSKUM_OK;
    if (h->prm.precision == QLSKUM_MIXED)
        mixed::derived(h->L, h->dc, h->s64.prim[h->pcur], h->s32.q[0], h->s32.cspeed);
    else
        fp64::derived(h->L, h->dc, h->s64.prim[h->pcur], h->s64.q[0], h->s64.cspeed);
    h->derived_valid = true;
    qlskum_status st = check_launch(h, "derived");
    if (st) return st;
    return tune(h);
}

cudaEvent_t take_event(qlskum_handle *h)
{
    if (!h->ev_pool.empty()) {
        cudaEvent_t e = h->ev_pool.back();
        h->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Runs `launch` bracketed by events when kernel timing is on.
template <typename F> void timed(qlskum_handle *h, int kernel, F &&launch)
{
    if (!h->timing) {
        launch();
        return;
    }
    cudaEvent_t a = take_event(h), b = take_event(h);
    cudaEventRecord(a, h->L.stream);
    launch();
    cudaEventRecord(b, h->L.stream);
    h->ev_pending.push_back({kernel, {a, b}});
}

qlskum_status collect_timing(qlskum_handle *h)
{
    if (h->ev_pending.empty()) return QLSKUM_OK;
    CK(h, cudaStreamSynchronize(h->L.stream));
    for (auto &p : h->ev_pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.second.first, p.second.second);
        h->kt_ms[p.first] += ms;
        h->kt_n[p.first] += 1;
        h->ev_pool.push_back(p.second.first);
        h->ev_pool.push_back(p.second.second);
    }
    h->ev_pending.clear();
    return QLSKUM_OK;
}

// Autotuner of the mixed form: times each launch shape of the fused flux +
// update kernel (threads per block x register cap) and each block size of the
// gradient / inner-loop kernels on this cloud, three launches each after one
// warm-up, and keeps the fastest.  The trial launches write only buffers the
// next iteration overwrites before reading (stage-1 targets, dq, qm, delta).
qlskum_status tune(qlskum_handle *h)
{
    if (h->tuned || h->prm.precision != QLSKUM_MIXED) return QLSKUM_OK;
    h->tuned = true;
    if (h->prm.block_size != 0) return QLSKUM_OK;
    const DevCloud &c = h->dc;
    State32 &S = h->s32;
    const int o = h->pcur, x = (o + 1) % 3;
    cudaEvent_t a = take_event(h), b = take_event(h);
    auto time3 = [&](auto &&launch) -> float {
        launch();
        cudaEventRecord(a, h->L.stream);
        for (int r = 0; r < 3; r++) launch();
        cudaEventRecord(b, h->L.stream);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        return ms;
    };
    long long launches0 = h->launches;
    static const int blocks[4] = {64, 128, 256, 512};
    float best = 1e30f;
    int best_block = h->L.block;
    for (int bs : blocks) {
        Launch L = h->L;
        L.block = bs;
        float ms = time3([&] { mixed::q_inner(L, c, S.q[0], S.dq[0], S.dq[1]); });
        if (ms < best) { best = ms; best_block = bs; }
    }
    h->L.block = best_block;
    mixed::q_derivatives(h->L, c, S.q[0], S.dq[0], S.qm, S.cspeed, S.delta, (float)h->K.cfl);
    best = 1e30f;
    for (int v = 0; v < mixed::flux_variants(); v++) {
        float ms = time3([&] {
            mixed::flux_update(h->L, c, h->K, S.q[0], S.dq[0], S.qm, S.delta, h->s64.prim[o], h->s64.prim[o],
                               h->s64.prim[x], S.q[1], nullptr, 1, h->R, v);
        });
        if (ms < best) { best = ms; h->flux_variant = v; }
    }
    h->launches = launches0;
    h->ev_pool.push_back(a);
    h->ev_pool.push_back(b);
    return check_launch(h, "tune");
}

// The kernels of one fused iteration from prim buffer o (fpi_solver_mod.h:
// 14-151).  Stage buffers: o -> x -> y -> x -> y, prim_old = o throughout;
// q ping-pongs q0 -> q1 -> q0 -> q1 -> q0.
void enqueue_iteration(qlskum_handle *h, int o, int it_arg)
{
    const int x = (o + 1) % 3, y = (o + 2) % 3;
    const int dst[4] = {x, y, x, y};
    const int src[4] = {o, x, y, x};
    const int ni = h->prm.inner_iterations;
    const DevCloud &c = h->dc;
    const Launch &L = h->L;
    for (int rk = 1; rk <= 4; rk++) {
        const int qa = (rk - 1) & 1, qb = rk & 1;
        // only the last stage's residual is reported (fpi_solver_mod.h:138)
        Reduce Rk = h->R;
        if (rk != 4) Rk.partial_sum = Rk.partial_max = nullptr;
        double *dl = rk == 1 ? h->s64.delta : nullptr;
        double *cs = rk == 4 ? h->s64.cspeed : nullptr;
        const double4_32a *pin = h->s64.prim[src[rk - 1]], *pold = h->s64.prim[o];
        double4_32a *pout = h->s64.prim[dst[rk - 1]];
        if (h->prm.precision == QLSKUM_MIXED) {
            State32 &S = h->s32;
            float *dl32 = rk == 1 ? S.delta : nullptr;
            float *cs32 = rk == 4 ? S.cspeed : nullptr;
            timed(h, QLSKUM_KERNEL_GRADIENT, [&] {
                mixed::q_derivatives(L, c, S.q[qa], S.dq[0], S.qm, S.cspeed, dl32, (float)h->K.cfl);
            });
            for (int j = 0; j < ni; j++)
                timed(h, QLSKUM_KERNEL_INNER, [&] { mixed::q_inner(L, c, S.q[qa], S.dq[j & 1], S.dq[(j + 1) & 1]); });
            timed(h, QLSKUM_KERNEL_FLUX_UPDATE, [&] {
                mixed::flux_update(L, c, h->K, S.q[qa], S.dq[ni & 1], S.qm, S.delta, pin, pold, pout, S.q[qb], cs32,
                                   rk, Rk, h->flux_variant);
            });
        } else {
            State64 &S = h->s64;
            timed(h, QLSKUM_KERNEL_GRADIENT, [&] {
                fp64::q_derivatives(L, c, S.q[qa], S.dq[0], S.qm, S.cspeed, dl, h->K.cfl);
            });
            for (int j = 0; j < ni; j++)
                timed(h, QLSKUM_KERNEL_INNER, [&] { fp64::q_inner(L, c, S.q[qa], S.dq[j & 1], S.dq[(j + 1) & 1]); });
            timed(h, QLSKUM_KERNEL_FLUX_UPDATE, [&] {
                fp64::flux_update(L, c, h->K, S.q[qa], S.dq[ni & 1], S.qm, S.delta, pin, pold, pout, S.q[qb], cs, rk,
                                  Rk);
            });
        }
    }
    Reduce R = h->R;
    R.blocks = (h->n + (h->prm.precision == QLSKUM_MIXED ? mixed::flux_block(h->flux_variant) : 128) - 1) /
               (h->prm.precision == QLSKUM_MIXED ? mixed::flux_block(h->flux_variant) : 128);
    timed(h, QLSKUM_KERNEL_REDUCE, [&] { fp64::reduce_residual(L, R, h->n, it_arg); });
}

void after_iteration(qlskum_handle *h, int o)
{
    h->pold = o;
    h->pcur = (o + 2) % 3;
    h->dcur = h->prm.inner_iterations & 1;
    h->inner_pending = false;
    h->derived_valid = true;
}

template <typename T>
void unpermute(const qlskum_handle *h, const std::vector<T> &dev, T *out, int width)
{
    for (int p = 0; p < h->n; p++) {
        int i = h->iperm[p];
        std::memcpy(out + (size_t)i * width, dev.data() + (size_t)p * width, sizeof(T) * width);
    }
}

qlskum_status print_iters(qlskum_handle *h, int from, int to)
{
    std::vector<double> hist((size_t)3 * (to - from));
    if (to <= from) return QLSKUM_OK;
    CK(h, cudaMemcpyAsync(hist.data(), h->R.hist + 3 * (size_t)from, sizeof(double) * hist.size(),
                          cudaMemcpyDeviceToHost, h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    for (int t = from; t < to; t++) printf("iterations %d residue : %.13e\n", t + 1, hist[3 * (size_t)(t - from) + 1]);
    fflush(stdout);
    return QLSKUM_OK;
}

qlskum_status check_status(qlskum_handle *h)
{
    int st = 0;
    CK(h, cudaMemcpyAsync(&st, h->R.status, sizeof(int), cudaMemcpyDeviceToHost, h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    if (st) return fail(h, QLSKUM_ERR_NONFINITE, "residual became non-finite (NaN/Inf in the state)");
    return QLSKUM_OK;
}

}  // namespace

struct Geometry {
    int n = 0, np = 0, nslices = 0, shape_points = 0;
    std::vector<int> perm, iperm;
    Precomp pc;
    DevCloud dc;
    int *d_wall_perm = nullptr;
    double4_32a *d_wall_geo = nullptr;
};

namespace {

// The device geometry of one cloud: point order (class, then Morton code),
// sliced-ELL edge arrays and every per-point / per-edge quantity the kernels
// read, uploaded on `stream` into `A`.  G.pc must already hold precompute()'s
// result (done first, on the host only, so malformed clouds are reported
// before any device work).  need_fp64 / need_mixed select the arrays of the
// FP64 and the mixed kernels.  Synchronises the stream.
qlskum_status build_geometry(const qlskum_cloud *c, const qlskum_params *p, int sp, bool need_fp64, bool need_mixed,
                             DeviceArena &A, cudaStream_t stream, Geometry &G)
{
    G.n = c->n;
    G.shape_points = sp;
    const int n = c->n, NB = QLSKUM_MAX_NBHS;
    // ---- point order: class (wall, outer, interior), then Morton code
    G.iperm.resize(n);
    std::iota(G.iperm.begin(), G.iperm.end(), 0);
    if (p->reorder) {
        double x0 = c->x[0], x1 = c->x[0], y0 = c->y[0], y1 = c->y[0];
        for (int i = 0; i < n; i++) {
            x0 = std::min(x0, c->x[i]); x1 = std::max(x1, c->x[i]);
            y0 = std::min(y0, c->y[i]); y1 = std::max(y1, c->y[i]);
        }
        const double span = std::max(x1 - x0, y1 - y0) + 1e-300;
        std::vector<uint64_t> key(n);
        for (int i = 0; i < n; i++) {
            uint32_t qx = (uint32_t)std::min(2097151.0, std::floor((c->x[i] - x0) / span * 2097151.0));
            uint32_t qy = (uint32_t)std::min(2097151.0, std::floor((c->y[i] - y0) / span * 2097151.0));
            static const int rank[3] = {0, 2, 1};
            key[i] = ((uint64_t)rank[c->flag_1[i]] << 62) | morton2(qx, qy);
        }
        std::stable_sort(G.iperm.begin(), G.iperm.end(), [&](int a, int b) { return key[a] < key[b]; });
    }
    G.perm.resize(n);
    for (int p2 = 0; p2 < n; p2++) G.perm[G.iperm[p2]] = p2;

    // ---- sliced ELL
    G.np = (n + 31) / 32 * 32;
    G.nslices = G.np / 32;
    std::vector<long long> sbase(G.nslices);
    long long tot = 0;
    for (int s = 0; s < G.nslices; s++) {
        int w = 0;
        for (int l = 0; l < 32; l++) {
            int pp = s * 32 + l;
            if (pp < n) w = std::max(w, c->nbhs[G.iperm[pp]]);
        }
        sbase[s] = tot;
        tot += 32LL * w;
    }
    const size_t ne = (size_t)std::max(tot, 32LL);
    std::vector<int> e_nbr(ne, 0);
    std::vector<double4_32a> e_geo(ne, make_double4_32a(0, 0, 0, 0));
    std::vector<double2> e_sn(ne, make_double2(0, 0));
    std::vector<double> e_dist(ne, 1.0);
    std::vector<uint8_t> e_dir(ne, 0);
    std::vector<float4> e_geo32(ne, make_float4(0, 0, 0, 0));
    std::vector<float2> e_sn32(ne, make_float2(0, 0));
    std::vector<int8_t> flag(G.np, 1);
    std::vector<int> nbh(G.np, 0);
    std::vector<double2> nrm(G.np, make_double2(0, 1));
    std::vector<double> eps2(G.np, 0.0);
    std::vector<float> eps2_32(G.np, 0.0f);
    std::vector<double4_32a> ggeo(G.np, make_double4_32a(0, 0, 0, 0));
    std::vector<double4_32a> fgeo((size_t)G.np * 4, make_double4_32a(0, 0, 0, 0));
    std::vector<double2> fcoef((size_t)G.np * 4, make_double2(0, 0));
    std::vector<double4_32a> gcoef(G.np, make_double4_32a(0, 0, 0, 0));
    std::vector<float2> e_xy32(ne, make_float2(0, 0));
    const bool unit_w = p->power == 0.0;
    std::vector<float> e_dist32(ne, 1.0f);
    const Precomp &P = G.pc;
    for (int pp = 0; pp < n; pp++) {
        const int i = G.iperm[pp];
        flag[pp] = (int8_t)c->flag_1[i];
        nbh[pp] = c->nbhs[i];
        nrm[pp] = make_double2(P.nx[i], P.ny[i]);
        eps2[pp] = P.eps2[i];
        eps2_32[pp] = (float)P.eps2[i];
        ggeo[pp] = make_double4_32a(P.ggeo[4 * (size_t)i], P.ggeo[4 * (size_t)i + 1], P.ggeo[4 * (size_t)i + 2],
                                P.ggeo[4 * (size_t)i + 3]);
        // q_variables_mod.h:112-116 as coefficients: dq_x = Sx syy/det - Sy sxy/det, dq_y = Sy sxx/det - Sx sxy/det
        gcoef[pp] = make_double4_32a(P.ggeo[4 * (size_t)i + 1] * P.ggeo[4 * (size_t)i + 3],
                                     P.ggeo[4 * (size_t)i + 2] * P.ggeo[4 * (size_t)i + 3],
                                     P.ggeo[4 * (size_t)i + 0] * P.ggeo[4 * (size_t)i + 3], 0.0);
        static const bool used[3][4] = {{true, true, false, true}, {true, true, true, true}, {true, true, true, false}};
        const int fl = c->flag_1[i];
        const double scale = fl == kWall ? 2.0 : 1.0;  // flux_residual_mod.h:29
        for (int d = 0; d < 4; d++) {
            const double *F = &P.fgeo[((size_t)i * 4 + d) * 4];
            fgeo[(size_t)pp * 4 + d] = make_double4_32a(F[0], F[1], F[2], F[3]);
            // x rows (d < 2): G = (Sx syy - Sy sxy) / det;  y rows: G = (Sy sxx - Sx sxy) / det
            double a = 0.0, b = 0.0;
            if (used[fl][d]) {
                if (d < 2) { a = scale * F[1] * F[3]; b = -scale * F[2] * F[3]; }
                else { a = -scale * F[2] * F[3]; b = scale * F[0] * F[3]; }
            }
            fcoef[(size_t)pp * 4 + d] = make_double2(a, b);
        }
        for (int r = 0; r < c->nbhs[i]; r++) {
            const size_t e = (size_t)(sbase[pp >> 5] + 32LL * r + (pp & 31));
            const size_t src = (size_t)i * NB + r;
            e_nbr[e] = G.perm[c->conn[src] - 1];
            e_geo[e] = make_double4_32a(P.geo[4 * src], P.geo[4 * src + 1], P.geo[4 * src + 2], P.geo[4 * src + 3]);
            e_sn[e] = make_double2(P.sn[2 * src], P.sn[2 * src + 1]);
            e_dist[e] = P.dist[src];
            e_dist32[e] = (float)P.dist[src];
            e_xy32[e] = make_float2((float)P.geo[4 * src], (float)P.geo[4 * src + 1]);
            e_dir[e] = P.edge_dir[src];
            e_geo32[e] = make_float4((float)P.geo[4 * src], (float)P.geo[4 * src + 1], (float)P.geo[4 * src + 2],
                                     (float)P.geo[4 * src + 3]);
            e_sn32[e] = make_float2((float)P.sn[2 * src], (float)P.sn[2 * src + 1]);
        }
    }

    // ---- device
    // Host vectors must outlive the asynchronous uploads: keep them until the
    // stream is synchronised at the end of this function.
    auto up = [&](auto *dptr, const auto &vec) {
        if (dptr && !vec.empty())
            cudaMemcpyAsync(dptr, vec.data(), vec.size() * sizeof(vec[0]), cudaMemcpyHostToDevice, stream);
    };
    int8_t *d_flag = A.alloc<int8_t>(G.np);
    int *d_nb = A.alloc<int>(G.np);
    long long *d_sb = A.alloc<long long>(G.nslices);
    int *d_enbr = A.alloc<int>(ne);
    double4_32a *d_egeo = need_fp64 ? A.alloc<double4_32a>(ne) : nullptr;
    double2 *d_esn = need_fp64 ? A.alloc<double2>(ne) : nullptr;
    double *d_edist = need_fp64 ? A.alloc<double>(ne) : nullptr;
    uint8_t *d_edir = A.alloc<uint8_t>(ne);
    double2 *d_nrm = A.alloc<double2>(G.np);
    double *d_eps2 = A.alloc<double>(G.np);
    double4_32a *d_ggeo = need_fp64 ? A.alloc<double4_32a>(G.np) : nullptr;
    double4_32a *d_fgeo = need_fp64 ? A.alloc<double4_32a>((size_t)G.np * 4) : nullptr;
    float4 *d_egeo32 = nullptr;
    float2 *d_esn32 = nullptr;
    float *d_eps32 = nullptr, *d_edist32 = nullptr;
    double2 *d_fcoef = nullptr;
    double4_32a *d_gcoef = nullptr;
    float2 *d_exy32 = nullptr;
    if (need_mixed) {
        if (unit_w) {
            d_exy32 = A.alloc<float2>(ne);
        } else {
            d_egeo32 = A.alloc<float4>(ne);
            d_esn32 = A.alloc<float2>(ne);
        }
        d_eps32 = A.alloc<float>(G.np);
        d_edist32 = A.alloc<float>(ne);
        d_fcoef = A.alloc<double2>((size_t)G.np * 4);
        d_gcoef = A.alloc<double4_32a>(G.np);
    }
    up(d_flag, flag); up(d_nb, nbh); up(d_sb, sbase); up(d_enbr, e_nbr); up(d_egeo, e_geo); up(d_esn, e_sn);
    up(d_edist, e_dist); up(d_edir, e_dir); up(d_nrm, nrm); up(d_eps2, eps2); up(d_ggeo, ggeo); up(d_fgeo, fgeo);
    up(d_egeo32, e_geo32); up(d_esn32, e_sn32); up(d_eps32, eps2_32); up(d_edist32, e_dist32); up(d_fcoef, fcoef);
    up(d_gcoef, gcoef); up(d_exy32, e_xy32);
    DevCloud &dc = G.dc;
    dc.n = n; dc.np = G.np; dc.flag = d_flag; dc.nbhs = d_nb; dc.slice_base = d_sb; dc.e_nbr = d_enbr;
    dc.e_geo = d_egeo; dc.e_sn = d_esn; dc.e_dist = d_edist; dc.e_dir = d_edir; dc.nrm = d_nrm; dc.eps2 = d_eps2;
    dc.ggeo = d_ggeo; dc.fgeo = d_fgeo; dc.e_geo32 = d_egeo32; dc.e_sn32 = d_esn32; dc.eps2_32 = d_eps32;
    dc.e_dist32 = d_edist32; dc.fcoef = d_fcoef; dc.gcoef = d_gcoef; dc.unit_w = unit_w ? 1 : 0; dc.e_xy32 = d_exy32;

    G.d_wall_perm = A.alloc<int>(std::max(sp, 1));
    G.d_wall_geo = A.alloc<double4_32a>(std::max(sp, 1));
    if (A.err != cudaSuccess) return fail(nullptr, QLSKUM_ERR_CUDA, fmt("cudaMalloc: %s", cudaGetErrorString(A.err)));
    // compute_force_coeffs_mod.h:37-59 geometry of the first shape_points points
    std::vector<int> wperm(std::max(sp, 1), 0);
    std::vector<double4_32a> wgeo(std::max(sp, 1), make_double4_32a(0, 0, 0, 0));
    for (int m = 0; m < sp; m++) {
        int r = c->right[m] - 1, l = c->left[m] - 1;
        double lx = c->x[l], ly = c->y[l], mx = c->x[m], my = c->y[m], rx = c->x[r], ry = c->y[r];
        double ds1 = std::pow((mx - lx), 2) + std::pow((my - ly), 2);
        ds1 = std::sqrt(ds1);
        double ds2 = std::pow((rx - mx), 2) + std::pow((ry - my), 2);
        ds2 = std::sqrt(ds2);
        double ds = 0.5 * (ds1 + ds2);
        wperm[m] = G.perm[m];
        wgeo[m] = make_double4_32a(ds, mx - 0.25, my, 0.0);
    }
    up(G.d_wall_perm, wperm);
    up(G.d_wall_geo, wgeo);
    cudaError_t ce = cudaStreamSynchronize(stream);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    if (ce != cudaSuccess) return fail(nullptr, QLSKUM_ERR_CUDA, fmt("geometry upload: %s", cudaGetErrorString(ce)));
    if (A.err != cudaSuccess) return fail(nullptr, QLSKUM_ERR_CUDA, fmt("cudaMalloc: %s", cudaGetErrorString(A.err)));
    return QLSKUM_OK;
}

}  // namespace

// ======================================================================= C ABI

extern "C" {

int qlskum_abi_version(void) { return QLSKUM_ABI_VERSION; }

void qlskum_default_params(qlskum_params *p)
{
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->mach = 0.63;
    p->aoa = 2.0;
    p->cfl = 0.1;
    p->vl_const = 150;
    p->power = 0;
    p->inner_iterations = 3;
    p->precision = QLSKUM_FP64;
    p->block_size = 0;
    p->reorder = 1;
    p->verbose = 0;
}

const char *qlskum_last_error(const qlskum_handle *h) { return h ? h->err.c_str() : g_create_error.c_str(); }

qlskum_status qlskum_create(const qlskum_cloud *c, const qlskum_params *p, qlskum_handle **out)
{
    if (!out) return fail(nullptr, QLSKUM_ERR_INVALID, "null output handle pointer");
    *out = nullptr;
    int sp = 0;
    qlskum_status st = validate(c, p, &sp);
    if (st) return st;
    Geometry G;
    st = precompute(c, p, G.pc);
    if (st) return st;
    qlskum_handle *h = new qlskum_handle();
    h->prm = *p;
    h->n = c->n;
    h->shape_points = sp;
    set_case(h);
    cudaError_t ce = cudaStreamCreateWithFlags(&h->L.stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
        qlskum_status s2 = fail(nullptr, QLSKUM_ERR_CUDA, fmt("cudaStreamCreate: %s", cudaGetErrorString(ce)));
        delete h;
        return s2;
    }
    h->L.block = p->block_size ? p->block_size : 128;
    h->L.launches = &h->launches;
    DeviceArena &A = h->arena;
    {
        st = build_geometry(c, p, sp, true, p->precision == QLSKUM_MIXED, A, h->L.stream, G);
        if (st) {
            A.release();
            cudaStreamDestroy(h->L.stream);
            delete h;
            return st;
        }
        h->np = G.np;
        h->nslices = G.nslices;
        h->perm = std::move(G.perm);
        h->iperm = std::move(G.iperm);
        h->pc = std::move(G.pc);
        h->pc.release_upload_data();
        h->dc = G.dc;
        h->d_wall_perm = G.d_wall_perm;
        h->d_wall_geo = G.d_wall_geo;
    }
    auto up = [&](auto *dptr, const auto &vec) {
        if (dptr && !vec.empty())
            cudaMemcpyAsync(dptr, vec.data(), vec.size() * sizeof(vec[0]), cudaMemcpyHostToDevice, h->L.stream);
    };
    const int n = c->n;
    for (int b = 0; b < 3; b++) h->s64.prim[b] = A.alloc<double4_32a>(h->np);
    for (int b = 0; b < 2; b++) {
        h->s64.q[b] = A.alloc<double4_32a>(h->np);
        h->s64.dq[b] = A.alloc<double4_32a>((size_t)h->np * 2);
    }
    h->s64.qm = A.alloc<double4_32a>((size_t)h->np * 2);
    h->s64.flux_res = A.alloc<double4_32a>(h->np);
    h->s64.delta = A.alloc<double>(h->np);
    h->s64.cspeed = A.alloc<double>(h->np);
    if (p->precision == QLSKUM_MIXED) {
        for (int b = 0; b < 2; b++) {
            h->s32.q[b] = A.alloc<float4>(h->np);
            h->s32.dq[b] = A.alloc<float4>((size_t)h->np * 2);
        }
        h->s32.qm = A.alloc<float4>((size_t)h->np * 2);
        h->s32.delta = A.alloc<float>(h->np);
        h->s32.cspeed = A.alloc<float>(h->np);
    }
    h->R.blocks = (n + 127) / 128;
    h->R.max_blocks = (n + 63) / 64;
    h->R.partial_sum = A.alloc<double>(h->R.max_blocks);
    h->R.partial_max = A.alloc<double>(h->R.max_blocks);
    h->R.res_old = A.alloc<double>(1);
    h->R.iter = A.alloc<int>(1);
    h->R.status = A.alloc<int>(1);
    h->d_obj = A.alloc<double>(8);
    h->d_obj_partial = A.alloc<double>(4 * (size_t)((std::max(n, sp) + 255) / 256));
    h->d_entropy = A.alloc<double>(h->np);
    h->d_last = A.alloc<double>(2);
    if (A.err != cudaSuccess) {
        qlskum_status s2 = fail(nullptr, QLSKUM_ERR_CUDA, fmt("cudaMalloc: %s", cudaGetErrorString(A.err)));
        A.release();
        cudaStreamDestroy(h->L.stream);
        delete h;
        return s2;
    }
    // initial_conditions_mod.h:23-37
    std::vector<double4_32a> prim0(h->np, make_double4_32a(h->K.rho_inf, h->K.u1_inf, h->K.u2_inf, h->K.pr_inf));
    for (int b = 0; b < 3; b++) up(h->s64.prim[b], prim0);
    cudaMemsetAsync(h->R.iter, 0, sizeof(int), h->L.stream);
    cudaMemsetAsync(h->R.status, 0, sizeof(int), h->L.stream);
    cudaMemsetAsync(h->R.res_old, 0, sizeof(double), h->L.stream);
    cudaMemsetAsync(h->s64.delta, 0, sizeof(double) * h->np, h->L.stream);
    cudaMemsetAsync(h->s64.flux_res, 0, sizeof(double4_32a) * h->np, h->L.stream);
    cudaMemsetAsync(h->s64.q[0], 0, sizeof(double4_32a) * h->np, h->L.stream);
    cudaMemsetAsync(h->s64.qm, 0, sizeof(double4_32a) * 2 * h->np, h->L.stream);
    cudaMemsetAsync(h->s64.dq[0], 0, sizeof(double4_32a) * 2 * h->np, h->L.stream);
    cudaMemsetAsync(h->s64.dq[1], 0, sizeof(double4_32a) * 2 * h->np, h->L.stream);
    ce = cudaStreamSynchronize(h->L.stream);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    if (ce != cudaSuccess) {
        qlskum_status s2 = fail(nullptr, QLSKUM_ERR_CUDA, fmt("upload: %s", cudaGetErrorString(ce)));
        A.release();
        cudaStreamDestroy(h->L.stream);
        delete h;
        return s2;
    }
    if (ensure_hist(h, 1024) != QLSKUM_OK) {
        qlskum_status s2 = fail(nullptr, QLSKUM_ERR_CUDA, h->err);
        A.release();
        cudaStreamDestroy(h->L.stream);
        delete h;
        return s2;
    }
    *out = h;
    return QLSKUM_OK;
}

qlskum_status qlskum_destroy(qlskum_handle *h)
{
    if (!h) return QLSKUM_OK;
    if (h->L.stream) cudaStreamSynchronize(h->L.stream);
    for (auto &g : h->graph)
        if (g) cudaGraphExecDestroy(g);
    for (auto &p : h->ev_pending) {
        cudaEventDestroy(p.second.first);
        cudaEventDestroy(p.second.second);
    }
    for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
    if (h->R.hist) cudaFree(h->R.hist);
    h->arena.release();
    if (h->L.stream) cudaStreamDestroy(h->L.stream);
    delete h;
    return QLSKUM_OK;
}

#define NEED(h)                                                     \
    do {                                                            \
        if (!(h)) return fail(nullptr, QLSKUM_ERR_INVALID, "null handle"); \
    } while (0)

qlskum_status qlskum_func_delta(qlskum_handle *h)
{
    NEED(h);
    fp64::func_delta(h->L, h->dc, h->s64.prim[h->pcur], h->s64.delta, h->K.cfl);
    return check_launch(h, "func_delta");
}

qlskum_status qlskum_eval_q_variables(qlskum_handle *h)
{
    NEED(h);
    fp64::q_variables(h->L, h->dc, h->s64.prim[h->pcur], h->s64.q[0]);
    h->derived_valid = false;
    return check_launch(h, "eval_q_variables");
}

qlskum_status qlskum_eval_q_derivatives(qlskum_handle *h)
{
    NEED(h);
    fp64::q_derivatives(h->L, h->dc, h->s64.q[0], h->s64.dq[h->dcur], h->s64.qm, nullptr, nullptr, 0.0);
    h->inner_pending = false;
    return check_launch(h, "eval_q_derivatives");
}

qlskum_status qlskum_eval_q_inner_loop(qlskum_handle *h)
{
    NEED(h);
    fp64::q_inner(h->L, h->dc, h->s64.q[0], h->s64.dq[h->dcur], h->s64.dq[1 - h->dcur]);
    h->inner_pending = true;
    return check_launch(h, "eval_q_inner_loop");
}

qlskum_status qlskum_eval_update_innerloop(qlskum_handle *h)
{
    NEED(h);
    // the inner loop wrote the other buffer: make it current instead of copying
    if (h->inner_pending) h->dcur = 1 - h->dcur;
    h->inner_pending = false;
    return QLSKUM_OK;
}

qlskum_status qlskum_cal_flux_residual(qlskum_handle *h)
{
    NEED(h);
    fp64::flux_residual(h->L, h->dc, h->s64.q[0], h->s64.dq[h->dcur], h->s64.qm, h->s64.delta, h->s64.flux_res);
    return check_launch(h, "cal_flux_residual");
}

qlskum_status qlskum_state_update(qlskum_handle *h, int rk)
{
    NEED(h);
    if (rk < 1 || rk > 4) return fail(h, QLSKUM_ERR_INVALID, fmt("rk=%d not in 1..4", rk));
    fp64::state_update(h->L, h->dc, h->K, h->s64.prim[h->pcur], h->s64.prim[h->pold], h->s64.flux_res, rk, h->R);
    h->derived_valid = false;
    return check_launch(h, "state_update");
}

qlskum_status qlskum_snapshot_prim_old(qlskum_handle *h)
{
    NEED(h);
    fp64::copy_prim(h->L, h->n, h->s64.prim[h->pcur], h->s64.prim[h->pold]);
    return check_launch(h, "snapshot_prim_old");
}

qlskum_status qlskum_fpi_solver(qlskum_handle *h, int it)
{
    NEED(h);
    if (it < 1) return fail(h, QLSKUM_ERR_INVALID, "it must be >= 1");
    qlskum_status st = ensure_hist(h, std::max(it, h->it + 1));
    if (st) return st;
    st = ensure_derived(h);
    if (st) return st;
    const int o = h->pcur;
    enqueue_iteration(h, o, it);
    st = check_launch(h, "fpi_solver");
    if (st) return st;
    after_iteration(h, o);
    h->it = it;
    st = collect_timing(h);
    if (st) return st;
    if (h->prm.verbose) {
        st = print_iters(h, it - 1, it);
        if (st) return st;
    }
    return QLSKUM_OK;
}

qlskum_status qlskum_q_lskum(qlskum_handle *h, int iters)
{
    NEED(h);
    if (iters < 0) return fail(h, QLSKUM_ERR_INVALID, "iters < 0");
    qlskum_status st = ensure_hist(h, h->it + iters);
    if (st) return st;
    st = ensure_derived(h);
    if (st) return st;
    // the device counter continues from the host's
    CK(h, cudaMemcpyAsync(h->R.iter, &h->it, sizeof(int), cudaMemcpyHostToDevice, h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    // one graph per buffer-rotation phase, all three captured up front
    for (int o = 0; o < 3 && !h->timing && iters > 0; o++) {
        if (h->graph[o]) continue;
        cudaGraph_t g = nullptr;
        CK(h, cudaStreamBeginCapture(h->L.stream, cudaStreamCaptureModeThreadLocal));
        long long before = h->launches;
        enqueue_iteration(h, o, 0);
        h->launches = before;  // counted when replayed
        cudaError_t e = cudaStreamEndCapture(h->L.stream, &g);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&h->graph[o], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
    }
    for (int t = 0; t < iters; t++) {
        const int o = h->pcur;
        if (h->timing) {
            enqueue_iteration(h, o, 0);
            st = check_launch(h, "q_lskum");
            if (st) return st;
            after_iteration(h, o);
            h->it += 1;
            continue;
        }
        CK(h, cudaGraphLaunch(h->graph[o], h->L.stream));
        h->launches += 4 * (2 + h->prm.inner_iterations) + 1;
        after_iteration(h, o);
        h->it += 1;
        if (h->prm.verbose) {
            st = print_iters(h, h->it - 1, h->it);
            if (st) return st;
        }
    }
    st = collect_timing(h);
    if (st) return st;
    return check_status(h);
}

qlskum_status qlskum_objective(qlskum_handle *h, double *cl, double *cd, double *cm, double *total_entropy)
{
    NEED(h);
    const double cp_scale = 0.5 * h->K.rho_inf * h->K.mach * h->K.mach;
    fp64::objective(h->L, h->dc, h->s64.prim[h->pcur], h->d_wall_perm, h->d_wall_geo, h->shape_points, cp_scale,
                    h->K.pr_inf, h->K.gamma, h->d_entropy, h->d_obj, h->d_obj_partial);
    qlskum_status st = check_launch(h, "objective");
    if (st) return st;
    double o[4];
    CK(h, cudaMemcpyAsync(o, h->d_obj, sizeof o, cudaMemcpyDeviceToHost, h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    const double H = o[0], V = o[1];
    if (cl) *cl = V * std::cos(h->K.theta) - H * std::sin(h->K.theta);
    if (cd) *cd = H * std::cos(h->K.theta) + V * std::sin(h->K.theta);
    if (cm) *cm = o[2];
    if (total_entropy) *total_entropy = o[3];
    return QLSKUM_OK;
}

qlskum_status qlskum_get_field(qlskum_handle *h, int field, double *out)
{
    NEED(h);
    if (!out) return fail(h, QLSKUM_ERR_INVALID, "null output");
    const int n = h->n;
    if (field == QLSKUM_FIELD_NORMALS) {
        for (int i = 0; i < n; i++) {
            out[2 * (size_t)i] = h->pc.nx[i];
            out[2 * (size_t)i + 1] = h->pc.ny[i];
        }
        return QLSKUM_OK;
    }
    const void *src = nullptr;
    int width = 4;
    bool f32 = false;
    switch (field) {
    case QLSKUM_FIELD_PRIM: src = h->s64.prim[h->pcur]; break;
    case QLSKUM_FIELD_PRIM_OLD: src = h->s64.prim[h->pold]; break;
    case QLSKUM_FIELD_Q:
        if (h->prm.precision == QLSKUM_MIXED && h->derived_valid) { src = h->s32.q[0]; f32 = true; }
        else src = h->s64.q[0];
        break;
    case QLSKUM_FIELD_DQ:
        if (h->prm.precision == QLSKUM_MIXED && h->derived_valid) { src = h->s32.dq[h->dcur]; f32 = true; }
        else src = h->s64.dq[h->dcur];
        width = 8;
        break;
    case QLSKUM_FIELD_QM:
        if (h->prm.precision == QLSKUM_MIXED && h->derived_valid) { src = h->s32.qm; f32 = true; }
        else src = h->s64.qm;
        width = 8;
        break;
    case QLSKUM_FIELD_FLUX_RES: src = h->s64.flux_res; break;
    case QLSKUM_FIELD_DELTA: src = h->s64.delta; width = 1; break;
    case QLSKUM_FIELD_ENTROPY: src = h->d_entropy; width = 1; break;
    default: return fail(h, QLSKUM_ERR_INVALID, fmt("unknown field %d", field));
    }
    std::vector<double> dev((size_t)n * width);
    if (f32) {
        std::vector<float> d32((size_t)n * width);
        CK(h, cudaMemcpyAsync(d32.data(), src, sizeof(float) * d32.size(), cudaMemcpyDeviceToHost, h->L.stream));
        CK(h, cudaStreamSynchronize(h->L.stream));
        for (size_t t = 0; t < d32.size(); t++) dev[t] = d32[t];
    } else {
        CK(h, cudaMemcpyAsync(dev.data(), src, sizeof(double) * dev.size(), cudaMemcpyDeviceToHost, h->L.stream));
        CK(h, cudaStreamSynchronize(h->L.stream));
    }
    unpermute(h, dev, out, width);
    return QLSKUM_OK;
}

qlskum_status qlskum_get_prim(qlskum_handle *h, double *out) { return qlskum_get_field(h, QLSKUM_FIELD_PRIM, out); }

qlskum_status qlskum_set_prim(qlskum_handle *h, const double *prim)
{
    NEED(h);
    if (!prim) return fail(h, QLSKUM_ERR_INVALID, "null prim");
    std::vector<double4_32a> dev(h->np, make_double4_32a(1, 0, 0, 1));
    for (int i = 0; i < h->n; i++) {
        const double *s = prim + 4 * (size_t)i;
        dev[h->perm[i]] = make_double4_32a(s[0], s[1], s[2], s[3]);
    }
    CK(h, cudaMemcpyAsync(h->s64.prim[h->pcur], dev.data(), sizeof(double4_32a) * h->np, cudaMemcpyHostToDevice,
                          h->L.stream));
    // a new state clears a non-finite flag raised by the old one
    CK(h, cudaMemsetAsync(h->R.status, 0, sizeof(int), h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    h->derived_valid = false;
    return QLSKUM_OK;
}

qlskum_status qlskum_get_connectivity(qlskum_handle *h, int *counts, int *lists)
{
    NEED(h);
    if (counts) std::memcpy(counts, h->pc.sub_counts.data(), sizeof(int) * h->pc.sub_counts.size());
    if (lists) std::memcpy(lists, h->pc.sub_lists.data(), sizeof(int) * h->pc.sub_lists.size());
    return QLSKUM_OK;
}

qlskum_status qlskum_get_residual_history(qlskum_handle *h, double *out, int max_rows, int *rows)
{
    NEED(h);
    int cnt = std::min(h->it, h->R.capacity);
    if (rows) *rows = cnt;
    int m = std::min(cnt, std::max(max_rows, 0));
    if (out && m > 0) {
        CK(h, cudaMemcpyAsync(out, h->R.hist, sizeof(double) * 3 * (size_t)m, cudaMemcpyDeviceToHost, h->L.stream));
        CK(h, cudaStreamSynchronize(h->L.stream));
    }
    return QLSKUM_OK;
}

qlskum_status qlskum_get_iteration(qlskum_handle *h, int *it)
{
    NEED(h);
    if (it) *it = h->it;
    return QLSKUM_OK;
}

qlskum_status qlskum_synchronize(qlskum_handle *h)
{
    NEED(h);
    CK(h, cudaStreamSynchronize(h->L.stream));
    return QLSKUM_OK;
}

void *qlskum_stream(qlskum_handle *h) { return h ? (void *)h->L.stream : nullptr; }

long long qlskum_launch_count(const qlskum_handle *h) { return h ? h->launches : 0; }

qlskum_status qlskum_get_launch_config(qlskum_handle *h, int *flux_block, int *flux_min_blocks, int *point_block)
{
    NEED(h);
    static const int minb[4] = {4, 5, 8, 2};
    if (flux_block) *flux_block = h->prm.precision == QLSKUM_MIXED ? mixed::flux_block(h->flux_variant) : 128;
    if (flux_min_blocks) *flux_min_blocks = h->prm.precision == QLSKUM_MIXED ? minb[h->flux_variant] : 1;
    if (point_block) *point_block = h->L.block;
    return QLSKUM_OK;
}

qlskum_status qlskum_set_kernel_timing(qlskum_handle *h, int enable)
{
    NEED(h);
    qlskum_status st = collect_timing(h);
    if (st) return st;
    h->timing = enable != 0;
    for (int k = 0; k < 4; k++) {
        h->kt_ms[k] = 0;
        h->kt_n[k] = 0;
    }
    return QLSKUM_OK;
}

qlskum_status qlskum_get_kernel_timing(qlskum_handle *h, int kernel, double *ms_total, long long *launches)
{
    NEED(h);
    if (kernel < 0 || kernel > 3) return fail(h, QLSKUM_ERR_INVALID, fmt("unknown kernel id %d", kernel));
    qlskum_status st = collect_timing(h);
    if (st) return st;
    if (ms_total) *ms_total = h->kt_ms[kernel];
    if (launches) *launches = h->kt_n[kernel];
    return QLSKUM_OK;
}

}  // extern "C"

// =================================================================== batches

struct qlskum_batch {
    qlskum_params prm{};
    std::vector<Geometry> geo;                 // per cloud
    std::vector<BatchCase> cases;
    std::vector<BatchTile> tiles[3];
    DeviceArena arena;
    BatchView view;
    Launch L;
    long long launches = 0;
    long long total = 0;                       // state points over all cases
    double4_32a *prim[3] = {nullptr, nullptr, nullptr};
    float4 *q[2] = {nullptr, nullptr};
    float4 *dq[2] = {nullptr, nullptr};
    float4 *qm = nullptr;
    float *delta = nullptr, *cspeed = nullptr;
    double *psum = nullptr, *pmax = nullptr;   // per flux tile
    int *d_iter = nullptr, *d_status = nullptr;
    double *res_old = nullptr, *res_new = nullptr, *hist = nullptr;
    int capacity = 0;
    double *d_obj = nullptr, *d_obj_scratch = nullptr, *d_entropy = nullptr;
    int pcur = 0;
    int tile = 128, flux_variant = 0;
    bool tuned = false, derived_valid = false;
    int it = 0;
    float cfl = 0.f;
    cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
    std::string err;
};

namespace {

qlskum_status bfail(qlskum_batch *b, qlskum_status s, const std::string &msg)
{
    if (b) b->err = msg;
    else g_create_error = msg;
    return s;
}

#define BCK(b, call)                                                                                    \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return bfail(b, QLSKUM_ERR_CUDA, fmt("%s: %s", #call, cudaGetErrorString(e_))); \
    } while (0)

static const int kFluxTile[4] = {128, 128, 64, 256};
static const int kFluxMinB[4] = {4, 5, 8, 2};

void batch_enqueue_iteration(qlskum_batch *b, int o)
{
    const int x = (o + 1) % 3, y = (o + 2) % 3;
    const int dst[4] = {x, y, x, y};
    const int src[4] = {o, x, y, x};
    const int ni = b->prm.inner_iterations;
    for (int rk = 1; rk <= 4; rk++) {
        const int qa = (rk - 1) & 1, qb = rk & 1;
        mixed::batch_q_derivatives(b->L, b->view, b->tile, b->q[qa], b->dq[0], b->qm, b->cspeed,
                                   rk == 1 ? b->delta : nullptr, b->cfl);
        for (int j = 0; j < ni; j++) mixed::batch_q_inner(b->L, b->view, b->tile, b->q[qa], b->dq[j & 1], b->dq[(j + 1) & 1]);
        mixed::batch_flux_update(b->L, b->view, b->flux_variant, b->q[qa], b->dq[ni & 1], b->qm, b->delta,
                                 b->prim[src[rk - 1]], b->prim[o], b->prim[dst[rk - 1]], b->q[qb],
                                 rk == 4 ? b->cspeed : nullptr, rk, rk == 4 ? b->psum : nullptr,
                                 rk == 4 ? b->pmax : nullptr);
    }
    mixed::batch_reduce(b->L, b->view, kFluxTile[b->flux_variant], b->psum, b->pmax, b->d_iter, b->res_old,
                        b->res_new, b->hist, b->capacity, b->d_status);
}

qlskum_status batch_ensure_hist(qlskum_batch *b, int needed)
{
    if (needed <= b->capacity) return QLSKUM_OK;
    int cap = std::max(256, b->capacity);
    while (cap < needed) cap *= 2;
    const size_t nc = b->cases.size();
    double *nh = nullptr;
    BCK(b, cudaMalloc(&nh, sizeof(double) * nc * (size_t)cap));
    BCK(b, cudaMemsetAsync(nh, 0, sizeof(double) * nc * (size_t)cap, b->L.stream));
    if (b->hist) {
        BCK(b, cudaMemcpyAsync(nh, b->hist, sizeof(double) * nc * (size_t)b->capacity, cudaMemcpyDeviceToDevice,
                               b->L.stream));
        BCK(b, cudaStreamSynchronize(b->L.stream));
        cudaFree(b->hist);
    }
    b->hist = nh;
    b->capacity = cap;
    for (auto &g : b->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    return QLSKUM_OK;
}

// Batch autotuner: points per tile of the gradient / inner-loop kernels and
// the shape of the flux kernel, each timed over three launches on the batch.
qlskum_status batch_tune(qlskum_batch *b)
{
    if (b->tuned) return QLSKUM_OK;
    b->tuned = true;
    if (b->prm.block_size != 0) {
        b->tile = b->prm.block_size == 64 || b->prm.block_size == 256 ? b->prm.block_size : 128;
        return QLSKUM_OK;
    }
    cudaEvent_t e0, e1;
    BCK(b, cudaEventCreate(&e0));
    BCK(b, cudaEventCreate(&e1));
    auto time3 = [&](auto &&launch) -> float {
        launch();
        cudaEventRecord(e0, b->L.stream);
        for (int r = 0; r < 3; r++) launch();
        cudaEventRecord(e1, b->L.stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        return ms;
    };
    const long long l0 = b->launches;
    float best = 1e30f;
    for (int t : {64, 128, 256}) {
        float ms = time3([&] { mixed::batch_q_inner(b->L, b->view, t, b->q[0], b->dq[0], b->dq[1]); });
        if (ms < best) { best = ms; b->tile = t; }
    }
    const int o = b->pcur, x = (o + 1) % 3;
    mixed::batch_q_derivatives(b->L, b->view, b->tile, b->q[0], b->dq[0], b->qm, b->cspeed, b->delta, b->cfl);
    best = 1e30f;
    for (int v = 0; v < 4; v++) {
        float ms = time3([&] {
            mixed::batch_flux_update(b->L, b->view, v, b->q[0], b->dq[0], b->qm, b->delta, b->prim[o], b->prim[o],
                                     b->prim[x], b->q[1], nullptr, 1, nullptr, nullptr);
        });
        if (ms < best) { best = ms; b->flux_variant = v; }
    }
    b->launches = l0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return bfail(b, QLSKUM_ERR_CUDA, fmt("batch tune: %s", cudaGetErrorString(e)));
    return QLSKUM_OK;
}

}  // namespace

extern "C" {

qlskum_status qlskum_batch_create(const qlskum_cloud *clouds, int n_clouds, const int *case_cloud,
                                  const double *case_mach, const double *case_aoa, int n_cases,
                                  const qlskum_params *params, qlskum_batch **out)
{
    if (!out) return bfail(nullptr, QLSKUM_ERR_INVALID, "null output batch pointer");
    *out = nullptr;
    if (!clouds || n_clouds < 1 || !case_cloud || !case_mach || !case_aoa || n_cases < 1 || !params)
        return bfail(nullptr, QLSKUM_ERR_INVALID, "batch needs >= 1 cloud, >= 1 case and non-null arrays");
    if (params->precision != QLSKUM_MIXED)
        return bfail(nullptr, QLSKUM_ERR_UNSUPPORTED, "batched launches run the mixed-precision form only");
    for (int c = 0; c < n_cases; c++)
        if (case_cloud[c] < 0 || case_cloud[c] >= n_clouds)
            return bfail(nullptr, QLSKUM_ERR_INVALID, fmt("case %d: cloud index %d out of range", c, case_cloud[c]));
    std::vector<int> sp(n_clouds);
    std::vector<Geometry> geo(n_clouds);
    for (int k = 0; k < n_clouds; k++) {
        qlskum_status st = validate(&clouds[k], params, &sp[k]);
        if (st) return bfail(nullptr, st, fmt("cloud %d: %s", k, g_create_error.c_str()));
        st = precompute(&clouds[k], params, geo[k].pc);
        if (st) return bfail(nullptr, st, fmt("cloud %d: %s", k, g_create_error.c_str()));
    }
    qlskum_batch *b = new qlskum_batch();
    b->prm = *params;
    b->cfl = (float)params->cfl;
    b->geo = std::move(geo);
    cudaError_t ce = cudaStreamCreateWithFlags(&b->L.stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
        delete b;
        return bfail(nullptr, QLSKUM_ERR_CUDA, fmt("cudaStreamCreate: %s", cudaGetErrorString(ce)));
    }
    b->L.launches = &b->launches;
    DeviceArena &A = b->arena;
    auto cleanup = [&](qlskum_status st, const std::string &m) {
        A.release();
        cudaStreamDestroy(b->L.stream);
        delete b;
        return bfail(nullptr, st, m);
    };
    for (int k = 0; k < n_clouds; k++) {
        qlskum_status st = build_geometry(&clouds[k], params, sp[k], false, true, A, b->L.stream, b->geo[k]);
        if (st) return cleanup(st, fmt("cloud %d: %s", k, g_create_error.c_str()));
        b->geo[k].pc = Precomp();
        std::vector<int>().swap(b->geo[k].perm);
    }
    // cases, state offsets and the tile tables of the three tile sizes
    long long off = 0;
    b->cases.resize(n_cases);
    for (int c = 0; c < n_cases; c++) {
        BatchCase &C = b->cases[c];
        C.cloud = case_cloud[c];
        C.n = clouds[C.cloud].n;
        C.off = off;
        off += (C.n + 31) / 32 * 32;
        CaseConst &K = C.K;
        K.pi = 4 * std::atan(1.0);
        K.rho_inf = 1.0;
        K.pr_inf = 1.0 / 1.4;
        K.gamma = 1.4;
        K.mach = case_mach[c];
        K.theta = case_aoa[c] * K.pi / 180;
        K.u1_inf = case_mach[c] * std::cos(K.theta);
        K.u2_inf = case_mach[c] * std::sin(K.theta);
        K.cfl = params->cfl;
    }
    b->total = off;
    const int tsz[3] = {64, 128, 256};
    for (int ti = 0; ti < 3; ti++) {
        for (int c = 0; c < n_cases; c++) {
            BatchCase &C = b->cases[c];
            C.tile0[ti] = (int)b->tiles[ti].size();
            for (int f = 0; f < C.n; f += tsz[ti]) b->tiles[ti].push_back(BatchTile{c, f});
            C.ntl[ti] = (int)b->tiles[ti].size() - C.tile0[ti];
        }
    }
    std::vector<DevCloud> dcs(n_clouds);
    for (int k = 0; k < n_clouds; k++) dcs[k] = b->geo[k].dc;
    DevCloud *d_clouds = A.alloc<DevCloud>(n_clouds);
    BatchCase *d_cases = A.alloc<BatchCase>(n_cases);
    BatchTile *d_tiles[3];
    for (int ti = 0; ti < 3; ti++) d_tiles[ti] = A.alloc<BatchTile>(b->tiles[ti].size());
    const size_t T = (size_t)b->total;
    for (int k = 0; k < 3; k++) b->prim[k] = A.alloc<double4_32a>(T);
    for (int k = 0; k < 2; k++) {
        b->q[k] = A.alloc<float4>(T);
        b->dq[k] = A.alloc<float4>(2 * T);
    }
    b->qm = A.alloc<float4>(2 * T);
    b->delta = A.alloc<float>(T);
    b->cspeed = A.alloc<float>(T);
    b->psum = A.alloc<double>(b->tiles[0].size());
    b->pmax = A.alloc<double>(b->tiles[0].size());
    b->d_iter = A.alloc<int>(1);
    b->d_status = A.alloc<int>(1);
    b->res_old = A.alloc<double>(n_cases);
    b->res_new = A.alloc<double>(n_cases);
    b->d_obj = A.alloc<double>(4 * (size_t)n_cases);
    size_t maxn = 1;
    for (int k = 0; k < n_clouds; k++) maxn = std::max(maxn, (size_t)std::max(clouds[k].n, sp[k]));
    b->d_obj_scratch = A.alloc<double>(4 * ((maxn + 255) / 256));
    b->d_entropy = A.alloc<double>(T);
    if (A.err != cudaSuccess) return cleanup(QLSKUM_ERR_CUDA, fmt("cudaMalloc: %s", cudaGetErrorString(A.err)));
    cudaStream_t s = b->L.stream;
    cudaMemcpyAsync(d_clouds, dcs.data(), sizeof(DevCloud) * n_clouds, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_cases, b->cases.data(), sizeof(BatchCase) * n_cases, cudaMemcpyHostToDevice, s);
    for (int ti = 0; ti < 3; ti++)
        cudaMemcpyAsync(d_tiles[ti], b->tiles[ti].data(), sizeof(BatchTile) * b->tiles[ti].size(),
                        cudaMemcpyHostToDevice, s);
    // initial_conditions_mod.h:23-37 per case
    std::vector<double4_32a> prim0(T, make_double4_32a(1.0, 0.0, 0.0, 1.0 / 1.4));
    for (const BatchCase &C : b->cases)
        for (int i = 0; i < C.n; i++)
            prim0[C.off + i] = make_double4_32a(C.K.rho_inf, C.K.u1_inf, C.K.u2_inf, C.K.pr_inf);
    for (int k = 0; k < 3; k++)
        cudaMemcpyAsync(b->prim[k], prim0.data(), sizeof(double4_32a) * T, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(b->d_iter, 0, sizeof(int), s);
    cudaMemsetAsync(b->d_status, 0, sizeof(int), s);
    cudaMemsetAsync(b->res_old, 0, sizeof(double) * n_cases, s);
    cudaMemsetAsync(b->res_new, 0, sizeof(double) * n_cases, s);
    cudaMemsetAsync(b->dq[0], 0, sizeof(float4) * 2 * T, s);
    cudaMemsetAsync(b->dq[1], 0, sizeof(float4) * 2 * T, s);
    ce = cudaStreamSynchronize(s);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    if (ce != cudaSuccess) return cleanup(QLSKUM_ERR_CUDA, fmt("batch upload: %s", cudaGetErrorString(ce)));
    b->view.clouds = d_clouds;
    b->view.cases = d_cases;
    b->view.ncases = n_cases;
    for (int ti = 0; ti < 3; ti++) {
        b->view.tiles[ti] = d_tiles[ti];
        b->view.ntiles[ti] = (int)b->tiles[ti].size();
    }
    b->view.unit_w = params->power == 0.0 ? 1 : 0;
    if (batch_ensure_hist(b, 256) != QLSKUM_OK) return cleanup(QLSKUM_ERR_CUDA, b->err);
    *out = b;
    return QLSKUM_OK;
}

qlskum_status qlskum_batch_destroy(qlskum_batch *b)
{
    if (!b) return QLSKUM_OK;
    if (b->L.stream) cudaStreamSynchronize(b->L.stream);
    for (auto &g : b->graph)
        if (g) cudaGraphExecDestroy(g);
    if (b->hist) cudaFree(b->hist);
    b->arena.release();
    if (b->L.stream) cudaStreamDestroy(b->L.stream);
    delete b;
    return QLSKUM_OK;
}

const char *qlskum_batch_last_error(const qlskum_batch *b) { return b ? b->err.c_str() : g_create_error.c_str(); }

qlskum_status qlskum_batch_run(qlskum_batch *b, int iters)
{
    if (!b) return bfail(nullptr, QLSKUM_ERR_INVALID, "null batch");
    if (iters < 0) return bfail(b, QLSKUM_ERR_INVALID, "iters < 0");
    qlskum_status st = batch_ensure_hist(b, b->it + iters);
    if (st) return st;
    if (!b->derived_valid) {
        mixed::batch_derived(b->L, b->view, 128, b->prim[b->pcur], b->q[0], b->cspeed);
        b->derived_valid = true;
        st = batch_tune(b);
        if (st) return st;
    }
    for (int o = 0; o < 3 && iters > 0; o++) {
        if (b->graph[o]) continue;
        cudaGraph_t g = nullptr;
        BCK(b, cudaStreamBeginCapture(b->L.stream, cudaStreamCaptureModeThreadLocal));
        const long long l0 = b->launches;
        batch_enqueue_iteration(b, o);
        b->launches = l0;
        cudaError_t e = cudaStreamEndCapture(b->L.stream, &g);
        if (e != cudaSuccess) return bfail(b, QLSKUM_ERR_CUDA, fmt("batch capture: %s", cudaGetErrorString(e)));
        e = cudaGraphInstantiate(&b->graph[o], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return bfail(b, QLSKUM_ERR_CUDA, fmt("batch instantiate: %s", cudaGetErrorString(e)));
    }
    for (int t = 0; t < iters; t++) {
        const int o = b->pcur;
        BCK(b, cudaGraphLaunch(b->graph[o], b->L.stream));
        b->launches += 4 * (2 + b->prm.inner_iterations) + 2;
        b->pcur = (o + 2) % 3;
        b->it += 1;
    }
    int status = 0;
    BCK(b, cudaMemcpyAsync(&status, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, b->L.stream));
    BCK(b, cudaStreamSynchronize(b->L.stream));
    if (status) return bfail(b, QLSKUM_ERR_NONFINITE, "a case's residual became non-finite");
    return QLSKUM_OK;
}

qlskum_status qlskum_batch_objective(qlskum_batch *b, double *cl, double *cd, double *cm, double *entropy)
{
    if (!b) return bfail(nullptr, QLSKUM_ERR_INVALID, "null batch");
    const int nc = (int)b->cases.size();
    for (int c = 0; c < nc; c++) {
        const BatchCase &C = b->cases[c];
        const Geometry &G = b->geo[C.cloud];
        const double cp_scale = 0.5 * C.K.rho_inf * C.K.mach * C.K.mach;
        fp64::objective(b->L, G.dc, b->prim[b->pcur] + C.off, G.d_wall_perm, G.d_wall_geo, G.shape_points, cp_scale,
                        C.K.pr_inf, C.K.gamma, b->d_entropy + C.off, b->d_obj + 4 * c, b->d_obj_scratch);
    }
    std::vector<double> o(4 * (size_t)nc);
    BCK(b, cudaMemcpyAsync(o.data(), b->d_obj, sizeof(double) * o.size(), cudaMemcpyDeviceToHost, b->L.stream));
    BCK(b, cudaStreamSynchronize(b->L.stream));
    for (int c = 0; c < nc; c++) {
        const double H = o[4 * c], V = o[4 * c + 1], th = b->cases[c].K.theta;
        if (cl) cl[c] = V * std::cos(th) - H * std::sin(th);
        if (cd) cd[c] = H * std::cos(th) + V * std::sin(th);
        if (cm) cm[c] = o[4 * c + 2];
        if (entropy) entropy[c] = o[4 * c + 3];
    }
    return QLSKUM_OK;
}

qlskum_status qlskum_batch_get_prim(qlskum_batch *b, int case_index, double *out)
{
    if (!b) return bfail(nullptr, QLSKUM_ERR_INVALID, "null batch");
    if (case_index < 0 || case_index >= (int)b->cases.size() || !out)
        return bfail(b, QLSKUM_ERR_INVALID, "case index out of range or null output");
    const BatchCase &C = b->cases[case_index];
    const Geometry &G = b->geo[C.cloud];
    std::vector<double> dev(4 * (size_t)C.n);
    BCK(b, cudaMemcpyAsync(dev.data(), b->prim[b->pcur] + C.off, sizeof(double) * dev.size(), cudaMemcpyDeviceToHost,
                           b->L.stream));
    BCK(b, cudaStreamSynchronize(b->L.stream));
    for (int p = 0; p < C.n; p++) std::memcpy(out + 4 * (size_t)G.iperm[p], dev.data() + 4 * (size_t)p, 32);
    return QLSKUM_OK;
}

qlskum_status qlskum_batch_residual_history(qlskum_batch *b, double *out, int max_rows, int *rows)
{
    if (!b) return bfail(nullptr, QLSKUM_ERR_INVALID, "null batch");
    const int cnt = std::min(b->it, b->capacity);
    if (rows) *rows = cnt;
    const int m = std::min(cnt, std::max(0, max_rows));
    if (out && m > 0) {
        BCK(b, cudaMemcpyAsync(out, b->hist, sizeof(double) * b->cases.size() * (size_t)m, cudaMemcpyDeviceToHost,
                               b->L.stream));
        BCK(b, cudaStreamSynchronize(b->L.stream));
    }
    return QLSKUM_OK;
}

long long qlskum_batch_total_points(const qlskum_batch *b)
{
    if (!b) return 0;
    long long t = 0;
    for (const BatchCase &C : b->cases) t += C.n;
    return t;
}

long long qlskum_batch_launch_count(const qlskum_batch *b) { return b ? b->launches : 0; }

void *qlskum_batch_stream(qlskum_batch *b) { return b ? (void *)b->L.stream : nullptr; }

qlskum_status qlskum_batch_tuning(const qlskum_batch *b, int *tile, int *flux_tile, int *flux_min_blocks,
                                  int *points_per_warp)
{
    if (!b) return QLSKUM_ERR_INVALID;
    if (tile) *tile = b->tile;
    if (flux_tile) *flux_tile = kFluxTile[b->flux_variant];
    if (flux_min_blocks) *flux_min_blocks = kFluxMinB[b->flux_variant];
    if (points_per_warp) *points_per_warp = 32;
    return QLSKUM_OK;
}

}  // extern "C"
