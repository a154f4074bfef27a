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
    // drop what only the device upload needs (keeps normals, sub-stencils and
    // their membership bits)
    void release_upload_data()
    {
        for (auto *v : {&geo, &sn, &dist, &ggeo, &fgeo, &eps2}) std::vector<double>().swap(*v);
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
    double *d_vort = nullptr;     // vorticity [np] (qlskum_enstrophy)
    double *d_diag = nullptr;     // per-256-block partials of the diagnostics [6][blocks]
    bool restarted = false;       // state and res_old came from a restart file
    int *d_wall_perm = nullptr;
    double4_32a *d_wall_geo = nullptr;
    // the point permutation on the device and a staging buffer in the cloud's
    // order, for moving states across the C ABI (allocated on first use)
    int *d_perm = nullptr;
    double4_32a *d_stage = nullptr;
    cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
    // launch shape of the mixed fused kernel and of the point kernels, set by
    // tune() on the first fused iteration unless params.block_size fixes it
    int flux_variant = 0;
    bool tuned = false;
    // the cloud as given (original order), for the geometry part of the adjoint
    std::vector<double> hx, hy;
    std::vector<int> hleft, hright, hflag, hnbhs, hconn;
    // discrete adjoint buffers, allocated on first use; checkpoint stride (iterations)
    struct AdjBuf *adj = nullptr;
    int adj_stride = 1;
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

// parameter_mod.h:4-30: the free stream of a case
CaseConst case_of(const qlskum_params &p)
{
    CaseConst K{};
    K.pi = 4 * std::atan(1.0);
    K.rho_inf = 1.0;
    K.pr_inf = 1.0 / 1.4;
    K.gamma = 1.4;
    K.mach = p.mach;
    K.theta = p.aoa * K.pi / 180;
    K.u1_inf = p.mach * std::cos(K.theta);
    K.u2_inf = p.mach * std::sin(K.theta);
    K.cfl = p.cfl;
    return K;
}

void set_case(qlskum_handle *h) { h->K = case_of(h->prm); }

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
    // gradient + inner-loop kernels: one gather per edge at four block sizes,
    // then the staged forms; weighted as one iteration runs them (one
    // gradient with the time step, inner_iterations inner steps per stage)
    const int ni = std::max(1, h->prm.inner_iterations);
    auto point_kernels = [&](const Launch &L) {
        return ni * time3([&] { mixed::q_inner(L, c, S.dq[0], S.dq[0], S.dq[1]); }) +
               time3([&] { mixed::q_derivatives(L, c, S.q[0], S.dq[0], S.qm, S.cspeed, S.delta, (float)h->K.cfl); });
    };
    static const int blocks[4] = {64, 128, 256, 512};
    float best = 1e30f;
    Launch best_L = h->L;
    for (int bs : blocks)
        for (int ln : {1, 2, 4}) {
            Launch L = h->L;
            L.block = bs;
            L.staged = 0;
            L.lanes = ln;
            const float ms = point_kernels(L);
            if (ms < best) { best = ms; best_L = L; }
        }
    const int nst = mixed::staged_variants(c);
    for (int v = 1; v <= nst; v++) {
        Launch L = best_L;
        L.staged = v;
        L.lanes = 1;
        const float ms = point_kernels(L);
        if (ms < best) { best = ms; best_L = L; }
    }
    h->L.block = best_L.block;
    h->L.staged = best_L.staged;
    h->L.lanes = best_L.lanes;
    mixed::q_derivatives(h->L, c, S.q[0], S.dq[0], S.qm, S.cspeed, S.delta, (float)h->K.cfl);
    best = 1e30f;
    Reduce none = h->R;  // stage 1 writes no residual partials
    none.partial_sum = none.partial_max = nullptr;
    for (int v = 0; v < mixed::flux_variants(); v++) {
        float ms = time3([&] {
            mixed::flux_update(h->L, c, h->K, S.q[0], S.dq[0], S.qm, S.delta, h->s64.prim[o], h->s64.prim[o],
                               h->s64.prim[x], S.q[1], nullptr, 1, none, v);
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
                timed(h, QLSKUM_KERNEL_INNER,
                      [&] { mixed::q_inner(L, c, S.dq[0], S.dq[mixed_dq_in(j)], S.dq[mixed_dq_out(j)]); });
            timed(h, QLSKUM_KERNEL_FLUX_UPDATE, [&] {
                mixed::flux_update(L, c, h->K, S.q[qa], S.dq[mixed_dq_final(ni)], S.qm, S.delta, pin, pold, pout, S.q[qb], cs32,
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
    R.blocks = h->prm.precision == QLSKUM_MIXED ? mixed::flux_grid_blocks(h->flux_variant, h->n)
                                                 : (h->n + 127) / 128;
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
    if (to <= from) return QLSKUM_OK;
    std::vector<double> hist((size_t)3 * (size_t)(to - from));
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
    size_t ne = 0;                             // edge slots of the sliced-ELL arrays
    std::vector<int> perm, iperm;
    Precomp pc;
    DevCloud dc;
    int *d_wall_perm = nullptr;
    double4_32a *d_wall_geo = nullptr;
};

// One partition of a cloud in the reference's distributed layout
// (data_structure_mod.h:4-8 local_points / ghost_points / pghost,
// point_preprocessing_mod.h:124-132): the points it owns, in device order,
// then the ghost points its own points read, appended after them (slot
// n_local + g).  slot[i]: the partition's slot of global point i, -1 when it
// neither owns nor mirrors it.
struct PartSpec {
    std::vector<int> local;   // device position -> global index
    std::vector<int> ghost;   // ghost g -> global index
    std::vector<int> slot;    // global index -> slot, or -1
};

namespace {

// The device geometry of one cloud: point order (class, then Morton code),
// sliced-ELL edge arrays and every per-point / per-edge quantity the kernels
// read, uploaded on `stream` into `A`.  G.pc (or `pc`) must already hold
// precompute()'s result (done first, on the host only, so malformed clouds
// are reported before any device work).  need_fp64 / need_mixed select the arrays of the
// FP64 and the mixed kernels.  Synchronises the stream.
//
// With a partition `ps`, the device arrays are those of the partition: its
// own points (ps->local, already in device order) are the kernels' points,
// their edges address the partition's slots (ps->slot), the per-point
// arrays also hold the ghost slots (of which the kernels read only the
// limiter's eps^2, the rest is state), and the wall list holds the
// partition's own shape points.  Every per-point and per-edge value is the
// one the whole cloud's geometry has, so a partitioned solve repeats the
// single-domain arithmetic point for point.
qlskum_status build_geometry(const qlskum_cloud *c, const qlskum_params *p, int sp, bool need_fp64, bool need_mixed,
                             DeviceArena &A, cudaStream_t stream, Geometry &G, const PartSpec *ps = nullptr,
                             const Precomp *pc = nullptr)
{
    const int NB = QLSKUM_MAX_NBHS;
    const int n = ps ? (int)ps->local.size() : c->n;       // the kernels' points
    const int nslot = ps ? n + (int)ps->ghost.size() : n;  // with the ghost slots
    G.n = n;
    G.shape_points = sp;
    // ---- point order: class (wall, outer, interior), then Morton code
    G.iperm.resize(n);
    std::iota(G.iperm.begin(), G.iperm.end(), 0);
    if (ps) {
        G.iperm = ps->local;
    } else if (p->reorder) {
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
    G.perm.assign(c->n, -1);
    for (int p2 = 0; p2 < n; p2++) G.perm[G.iperm[p2]] = p2;
    // neighbour index -> the slot the kernels address
    const std::vector<int> &slot_of = ps ? ps->slot : G.perm;

    // ---- sliced ELL over the kernels' points; per-point arrays also cover the ghost slots
    G.np = (nslot + 31) / 32 * 32;
    G.nslices = (n + 31) / 32;
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
    G.ne = ne;
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
    std::vector<float2> e_w32(ne, make_float2(0, 0)), e_w32b(ne, make_float2(0, 0));
    std::vector<double4_32a> gcoef(G.np, make_double4_32a(0, 0, 0, 0));
    std::vector<float2> e_xy32(ne, make_float2(0, 0)), e_gw32(ne, make_float2(0, 0));
    const bool unit_w = p->power == 0.0;
    std::vector<float> e_dist32(ne, 1.0f);
    const Precomp &P = pc ? *pc : G.pc;
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
        // (folded into the per-edge gradient weights below)
        gcoef[pp] = make_double4_32a(P.ggeo[4 * (size_t)i + 1] * P.ggeo[4 * (size_t)i + 3],
                                     P.ggeo[4 * (size_t)i + 2] * P.ggeo[4 * (size_t)i + 3],
                                     P.ggeo[4 * (size_t)i + 0] * P.ggeo[4 * (size_t)i + 3], 0.0);
        static const bool used[3][4] = {{true, true, false, true}, {true, true, true, true}, {true, true, true, false}};
        const int fl = c->flag_1[i];
        const double scale = fl == kWall ? 2.0 : 1.0;  // flux_residual_mod.h:29
        double ca[4], cb[4];
        for (int d = 0; d < 4; d++) {
            const double *F = &P.fgeo[((size_t)i * 4 + d) * 4];
            fgeo[(size_t)pp * 4 + d] = make_double4_32a(F[0], F[1], F[2], F[3]);
            // x rows (d < 2): G = (Sx syy - Sy sxy) / det;  y rows: G = (Sy sxx - Sx sxy) / det
            double a = 0.0, b = 0.0;
            if (used[fl][d]) {
                if (d < 2) { a = scale * F[1] * F[3]; b = -scale * F[2] * F[3]; }
                else { a = -scale * F[2] * F[3]; b = scale * F[0] * F[3]; }
            }
            ca[d] = a;
            cb[d] = b;
        }
        for (int r = 0; r < c->nbhs[i]; r++) {
            const size_t e = (size_t)(sbase[pp >> 5] + 32LL * r + (pp & 31));
            const size_t src = (size_t)i * NB + r;
            e_nbr[e] = slot_of[c->conn[src] - 1];
            e_geo[e] = make_double4_32a(P.geo[4 * src], P.geo[4 * src + 1], P.geo[4 * src + 2], P.geo[4 * src + 3]);
            e_sn[e] = make_double2(P.sn[2 * src], P.sn[2 * src + 1]);
            e_dist[e] = P.dist[src];
            e_dist32[e] = (float)P.dist[src];
            e_xy32[e] = make_float2((float)P.geo[4 * src], (float)P.geo[4 * src + 1]);
            e_dir[e] = P.edge_dir[src];
            e_geo32[e] = make_float4((float)P.geo[4 * src], (float)P.geo[4 * src + 1], (float)P.geo[4 * src + 2],
                                     (float)P.geo[4 * src + 3]);
            e_sn32[e] = make_float2((float)P.sn[2 * src], (float)P.sn[2 * src + 1]);
            // per-edge gradient weights gx = a w delx - b w dely, gy = c w dely - b w delx (FP64, then FP32)
            {
                const double4_32a &gc = gcoef[pp];
                const double wx = P.geo[4 * src + 2], wy = P.geo[4 * src + 3];
                e_gw32[e] = make_float2((float)(gc.x * wx - gc.y * wy), (float)(gc.z * wy - gc.y * wx));
            }
            // per-edge solve weights c_ed = a_d dels_w + b_d deln_w (FP64, then FP32)
            {
                const unsigned bits = P.edge_dir[src];
                const double sw = P.sn[2 * src], nw = P.sn[2 * src + 1];
                auto cw = [&](int d) { return (float)(ca[d] * sw + cb[d] * nw); };
                const int dx = (bits & kXpos) ? 0 : 1, dy = (bits & kYpos) ? 2 : 3;
                e_w32[e] = make_float2(cw(dx), cw(dy));
                e_w32b[e] = make_float2((bits & (kXpos | kXneg)) == (kXpos | kXneg) ? cw(1) : 0.f,
                                        (bits & (kYpos | kYneg)) == (kYpos | kYneg) ? cw(3) : 0.f);
            }
        }
    }

    // ghost slots: the owner's limiter eps^2 (read for the neighbour end of an edge)
    if (ps)
        for (size_t g = 0; g < ps->ghost.size(); g++) {
            eps2[n + g] = P.eps2[ps->ghost[g]];
            eps2_32[n + g] = (float)P.eps2[ps->ghost[g]];
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
    float2 *d_ew32 = nullptr, *d_ew32b = nullptr;
    float2 *d_exy32 = nullptr, *d_egw32 = nullptr;
    if (need_mixed) {
        if (unit_w) {
            d_exy32 = A.alloc<float2>(ne);
        } else {
            d_egeo32 = A.alloc<float4>(ne);
            d_esn32 = A.alloc<float2>(ne);
        }
        d_eps32 = A.alloc<float>(G.np);
        d_edist32 = A.alloc<float>(ne);
        d_ew32 = A.alloc<float2>(ne);
        d_ew32b = A.alloc<float2>(ne);
        d_egw32 = A.alloc<float2>(ne);
    }
    up(d_flag, flag); up(d_nb, nbh); up(d_sb, sbase); up(d_enbr, e_nbr); up(d_egeo, e_geo); up(d_esn, e_sn);
    up(d_edist, e_dist); up(d_edir, e_dir); up(d_nrm, nrm); up(d_eps2, eps2); up(d_ggeo, ggeo); up(d_fgeo, fgeo);
    up(d_egeo32, e_geo32); up(d_esn32, e_sn32); up(d_eps32, eps2_32); up(d_edist32, e_dist32); up(d_ew32, e_w32); up(d_ew32b, e_w32b);
    up(d_exy32, e_xy32); up(d_egw32, e_gw32);
    DevCloud &dc = G.dc;
    dc.n = n; dc.np = G.np; dc.flag = d_flag; dc.nbhs = d_nb; dc.slice_base = d_sb; dc.e_nbr = d_enbr;
    dc.e_geo = d_egeo; dc.e_sn = d_esn; dc.e_dist = d_edist; dc.e_dir = d_edir; dc.nrm = d_nrm; dc.eps2 = d_eps2;
    dc.ggeo = d_ggeo; dc.fgeo = d_fgeo; dc.e_geo32 = d_egeo32; dc.e_sn32 = d_esn32; dc.eps2_32 = d_eps32;
    dc.e_dist32 = d_edist32; dc.e_w32 = d_ew32; dc.e_w32b = d_ew32b; dc.unit_w = unit_w ? 1 : 0; dc.e_xy32 = d_exy32;
    dc.e_gw32 = d_egw32;
    dc.max_nb = 0;
    for (int pp = 0; pp < n; pp++) dc.max_nb = std::max(dc.max_nb, c->nbhs[G.iperm[pp]]);

    // compute_force_coeffs_mod.h:37-59 geometry of the first shape_points
    // points (of a partition: those it owns)
    std::vector<int> wall;
    for (int m = 0; m < sp; m++)
        if (G.perm[m] >= 0) wall.push_back(m);
    const int nw = (int)wall.size();
    G.shape_points = nw;
    G.d_wall_perm = A.alloc<int>(std::max(nw, 1));
    G.d_wall_geo = A.alloc<double4_32a>(std::max(nw, 1));
    if (A.err != cudaSuccess) return fail(nullptr, QLSKUM_ERR_CUDA, fmt("cudaMalloc: %s", cudaGetErrorString(A.err)));
    std::vector<int> wperm(std::max(nw, 1), 0);
    std::vector<double4_32a> wgeo(std::max(nw, 1), make_double4_32a(0, 0, 0, 0));
    for (int t = 0; t < nw; t++) {
        const int m = wall[t];
        int r = c->right[m] - 1, l = c->left[m] - 1;
        double lx = c->x[l], ly = c->y[l], mx = c->x[m], my = c->y[m], rx = c->x[r], ry = c->y[r];
        double ds1 = std::pow((mx - lx), 2) + std::pow((my - ly), 2);
        ds1 = std::sqrt(ds1);
        double ds2 = std::pow((rx - mx), 2) + std::pow((ry - my), 2);
        ds2 = std::sqrt(ds2);
        double ds = 0.5 * (ds1 + ds2);
        wperm[t] = G.perm[m];
        wgeo[t] = make_double4_32a(ds, mx - 0.25, my, 0.0);
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

void adj_free(qlskum_handle *h);

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
    h->hx.assign(c->x, c->x + c->n);
    h->hy.assign(c->y, c->y + c->n);
    h->hleft.assign(c->left, c->left + c->n);
    h->hright.assign(c->right, c->right + c->n);
    h->hflag.assign(c->flag_1, c->flag_1 + c->n);
    h->hnbhs.assign(c->nbhs, c->nbhs + c->n);
    h->hconn.assign(c->conn, c->conn + (size_t)c->n * QLSKUM_MAX_NBHS);
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
        for (int b = 0; b < 2; b++) h->s32.q[b] = A.alloc<float4>(h->np);
        for (int b = 0; b < 3; b++) h->s32.dq[b] = A.alloc<float4>((size_t)h->np * 2);
        h->s32.qm = A.alloc<float4>((size_t)h->np * 2);
        h->s32.delta = A.alloc<float>(h->np);
        h->s32.cspeed = A.alloc<float>(h->np);
    }
    h->R.blocks = (n + 127) / 128;
    h->R.max_blocks = (n + 31) / 32;  // one partial per block of the smallest launch shape (32 threads)
    h->R.partial_sum = A.alloc<double>(h->R.max_blocks);
    h->R.partial_max = A.alloc<double>(h->R.max_blocks);
    h->R.res_old = A.alloc<double>(1);
    h->R.iter = A.alloc<int>(1);
    h->R.status = A.alloc<int>(1);
    h->d_obj = A.alloc<double>(8);
    h->d_obj_partial = A.alloc<double>(4 * (size_t)((std::max(n, sp) + 255) / 256));
    h->d_entropy = A.alloc<double>(h->np);
    h->d_last = A.alloc<double>(2);
    h->d_vort = A.alloc<double>(h->np);
    h->d_diag = A.alloc<double>(6 * (size_t)((n + 255) / 256));
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
    if (h->d_perm) cudaFree(h->d_perm);
    if (h->d_stage) cudaFree(h->d_stage);
    adj_free(h);
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

}  // extern "C"

namespace {
// One graph per buffer-rotation phase (enqueue_iteration with the device's
// iteration counter), all three captured on first use.
qlskum_status ensure_graphs(qlskum_handle *h)
{
    for (int o = 0; o < 3; o++) {
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
    return QLSKUM_OK;
}
}  // namespace

extern "C" {

qlskum_status qlskum_fpi_solver(qlskum_handle *h, int it)
{
    NEED(h);
    if (it < 1) return fail(h, QLSKUM_ERR_INVALID, "it must be >= 1");
    qlskum_status st = ensure_hist(h, std::max(it, h->it + 1));
    if (st) return st;
    st = ensure_derived(h);
    if (st) return st;
    const int o = h->pcur;
    if (h->timing) {
        enqueue_iteration(h, o, it);
    } else {
        // the captured iteration, its counter set to it - 1 on the device
        if ((st = ensure_graphs(h))) return st;
        fp64::set_counter(h->L, h->R.iter, it - 1);
        CK(h, cudaGraphLaunch(h->graph[o], h->L.stream));
        h->launches += 4 * (2 + h->prm.inner_iterations) + 1;
    }
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
    if (!h->timing && iters > 0 && (st = ensure_graphs(h))) return st;
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
        if (h->prm.precision == QLSKUM_MIXED && h->derived_valid) {
            src = h->s32.dq[mixed_dq_final(h->prm.inner_iterations)];
            f32 = true;
        }
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

namespace {
// The device copy of the permutation and the staging buffer (first use).
qlskum_status ensure_stage(qlskum_handle *h)
{
    if (h->d_stage) return QLSKUM_OK;
    cudaError_t e = cudaMalloc(&h->d_perm, sizeof(int) * (size_t)h->n);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_stage, sizeof(double4_32a) * (size_t)h->n);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->d_perm, h->perm.data(), sizeof(int) * (size_t)h->n, cudaMemcpyHostToDevice, h->L.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->L.stream);
    if (e != cudaSuccess) {
        if (h->d_perm) cudaFree(h->d_perm);
        if (h->d_stage) cudaFree(h->d_stage);
        h->d_perm = nullptr;
        h->d_stage = nullptr;
        return fail(h, QLSKUM_ERR_CUDA, fmt("state staging buffers: %s", cudaGetErrorString(e)));
    }
    return QLSKUM_OK;
}
}  // namespace

// prim in the cloud's order: one copy of [n][4] doubles from the caller's
// buffer (a DMA at the link's rate when the caller's memory is pinned), the
// reordering on the device.
qlskum_status qlskum_get_prim(qlskum_handle *h, double *out)
{
    NEED(h);
    if (!out) return fail(h, QLSKUM_ERR_INVALID, "null output");
    qlskum_status st = ensure_stage(h);
    if (st) return st;
    fp64::permute_out(h->L, h->n, h->d_perm, h->s64.prim[h->pcur], h->d_stage);
    CK(h, cudaMemcpyAsync(out, h->d_stage, sizeof(double4_32a) * (size_t)h->n, cudaMemcpyDeviceToHost, h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    return QLSKUM_OK;
}

qlskum_status qlskum_set_prim(qlskum_handle *h, const double *prim)
{
    NEED(h);
    if (!prim) return fail(h, QLSKUM_ERR_INVALID, "null prim");
    qlskum_status st = ensure_stage(h);
    if (st) return st;
    CK(h, cudaMemcpyAsync(h->d_stage, prim, sizeof(double4_32a) * (size_t)h->n, cudaMemcpyHostToDevice, h->L.stream));
    // padding rows of the state keep the finite values they were created with
    fp64::permute_in(h->L, h->n, h->d_perm, h->d_stage, h->s64.prim[h->pcur]);
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

qlskum_status qlskum_get_launch_config(qlskum_handle *h, int *flux_block, int *flux_min_blocks, int *point_block,
                                       int *gather_depth)
{
    NEED(h);
    if (flux_block) *flux_block = h->prm.precision == QLSKUM_MIXED ? mixed::flux_block(h->flux_variant) : 128;
    if (flux_min_blocks) *flux_min_blocks = h->prm.precision == QLSKUM_MIXED ? mixed::flux_min_blocks(h->flux_variant) : 1;
    if (point_block) *point_block = h->L.staged ? mixed::staged_block(h->L.staged) : h->L.block;
    if (gather_depth) *gather_depth = h->L.staged ? mixed::staged_depth(h->L.staged) : 0;
    return QLSKUM_OK;
}

int qlskum_get_flux_variant(const qlskum_handle *h)
{
    return h && h->prm.precision == QLSKUM_MIXED ? h->flux_variant : 0;
}

qlskum_status qlskum_set_launch_config(qlskum_handle *h, int flux_variant, int point_block, int staged)
{
    NEED(h);
    if (flux_variant < 0 || flux_variant >= mixed::flux_variants())
        return fail(h, QLSKUM_ERR_INVALID, fmt("flux_variant %d not in 0..%d", flux_variant, mixed::flux_variants() - 1));
    if (point_block != 64 && point_block != 128 && point_block != 256 && point_block != 512)
        return fail(h, QLSKUM_ERR_INVALID, "point_block must be 64, 128, 256 or 512");
    if (staged < 0 || staged > 4) return fail(h, QLSKUM_ERR_INVALID, "staged must be in 0..4");
    if (staged > 0 && h->prm.precision == QLSKUM_MIXED && staged > mixed::staged_variants(h->dc))
        return fail(h, QLSKUM_ERR_UNSUPPORTED, "staged variant needs more shared memory than the device allows");
    h->flux_variant = flux_variant;
    h->L.block = point_block;
    h->L.staged = h->prm.precision == QLSKUM_MIXED ? staged : 0;
    h->L.lanes = 1;
    h->tuned = true;
    // captured iterations hold the old shapes
    for (auto &g : h->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    return QLSKUM_OK;
}

qlskum_status qlskum_set_point_lanes(qlskum_handle *h, int lanes)
{
    NEED(h);
    if (lanes != 1 && lanes != 2 && lanes != 4) return fail(h, QLSKUM_ERR_INVALID, "lanes must be 1, 2 or 4");
    if (lanes > 1 && h->L.staged) return fail(h, QLSKUM_ERR_UNSUPPORTED, "the staged gather form has one lane per point");
    h->L.lanes = h->prm.precision == QLSKUM_MIXED ? lanes : 1;
    h->tuned = true;
    for (auto &g : h->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    return QLSKUM_OK;
}

qlskum_status qlskum_get_lanes(const qlskum_handle *h, int *point_lanes, int *flux_lanes)
{
    if (!h) return QLSKUM_ERR_INVALID;
    const bool mx = h->prm.precision == QLSKUM_MIXED;
    if (point_lanes) *point_lanes = mx ? h->L.lanes : 1;
    if (flux_lanes) *flux_lanes = mx ? mixed::flux_lanes(h->flux_variant) : 1;
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
    DeviceArena arena;
    DevCloud sc;                               // the cases' concatenated cloud
    BatchView view;
    Launch L;
    long long launches = 0;
    long long total = 0;                       // state points over all cases
    double4_32a *prim[3] = {nullptr, nullptr, nullptr};
    float4 *q[2] = {nullptr, nullptr};
    float4 *dq[3] = {nullptr, nullptr, nullptr};  // as State32::dq
    float4 *qm = nullptr;
    float *delta = nullptr, *cspeed = nullptr;
    double *psum = nullptr, *pmax = nullptr;   // per flux block
    int *d_iter = nullptr, *d_status = nullptr;
    double *res_old = nullptr, *res_new = nullptr, *hist = nullptr;
    int capacity = 0;
    double *d_obj = nullptr, *d_obj_scratch = nullptr, *d_entropy = nullptr;
    int pcur = 0;
    int flux_variant = 0;                      // the single-cloud flux variants (mixed::flux_update)
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


// Points of each flux block of a variant (its threads over its lanes per point).
int batch_flux_points(int v) { return mixed::flux_block(v) / mixed::flux_lanes(v); }

void batch_enqueue_iteration(qlskum_batch *b, int o)
{
    const int x = (o + 1) % 3, y = (o + 2) % 3;
    const int dst[4] = {x, y, x, y};
    const int src[4] = {o, x, y, x};
    const int ni = b->prm.inner_iterations;
    const Reduce R{b->psum, b->pmax};
    const Reduce none{nullptr, nullptr};
    for (int rk = 1; rk <= 4; rk++) {
        const int qa = (rk - 1) & 1, qb = rk & 1;
        mixed::q_derivatives(b->L, b->sc, b->q[qa], b->dq[0], b->qm, b->cspeed, rk == 1 ? b->delta : nullptr, b->cfl);
        for (int j = 0; j < ni; j++)
            mixed::q_inner(b->L, b->sc, b->dq[0], b->dq[mixed_dq_in(j)], b->dq[mixed_dq_out(j)]);
        mixed::flux_update(b->L, b->sc, b->cases[0].K, b->q[qa], b->dq[mixed_dq_final(ni)], b->qm, b->delta,
                           b->prim[src[rk - 1]], b->prim[o], b->prim[dst[rk - 1]], b->q[qb],
                           rk == 4 ? b->cspeed : nullptr, rk, rk == 4 ? R : none, b->flux_variant);
    }
    mixed::batch_reduce(b->L, b->view, batch_flux_points(b->flux_variant), b->psum, b->pmax, b->d_iter, b->res_old,
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

// Batch autotuner: threads per block and lanes per point of the gradient /
// inner-loop kernels and the shape of the flux kernel (the single-cloud
// variants), each timed over three launches on the concatenated cloud.
qlskum_status batch_tune(qlskum_batch *b)
{
    if (b->tuned) return QLSKUM_OK;
    b->tuned = true;
    if (b->prm.block_size != 0) {
        b->L.block = b->prm.block_size == 64 || b->prm.block_size == 256 ? b->prm.block_size : 128;
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
    // gradient / inner-loop kernels: threads per block x lanes per point, timed
    // as an iteration weighs them (one gradient and inner_iterations inner steps)
    float best = 1e30f;
    const int ni = std::max(1, b->prm.inner_iterations);
    for (int t : {64, 128, 256})
        for (int ln : {1, 2, 4}) {
            Launch L = b->L;
            L.block = t;
            L.lanes = ln;
            L.staged = 0;
            const float ms =
                ni * time3([&] { mixed::q_inner(L, b->sc, b->dq[0], b->dq[0], b->dq[1]); }) +
                time3([&] { mixed::q_derivatives(L, b->sc, b->q[0], b->dq[0], b->qm, b->cspeed, nullptr, b->cfl); });
            if (ms < best) { best = ms; b->L.block = t; b->L.lanes = ln; }
        }
    const int o = b->pcur, x = (o + 1) % 3;
    mixed::q_derivatives(b->L, b->sc, b->q[0], b->dq[0], b->qm, b->cspeed, b->delta, b->cfl);
    best = 1e30f;
    const Reduce none{nullptr, nullptr};
    for (int v = 0; v < mixed::flux_variants(); v++) {
        float ms = time3([&] {
            mixed::flux_update(b->L, b->sc, b->cases[0].K, b->q[0], b->dq[0], b->qm, b->delta, b->prim[o],
                               b->prim[o], b->prim[x], b->q[1], nullptr, 1, none, v);
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
    // cases and their offsets in the concatenated cloud (multiples of
    // kBatchAlign), the flux blocks of each case per block size
    long long off = 0;
    b->cases.resize(n_cases);
    for (int c = 0; c < n_cases; c++) {
        BatchCase &C = b->cases[c];
        C.cloud = case_cloud[c];
        C.n = clouds[C.cloud].n;
        C.off = off;
        off += (C.n + kBatchAlign - 1) / kBatchAlign * kBatchAlign;
        const int bsz[3] = {64, 128, 256};
        for (int t = 0; t < 3; t++) {
            C.blk0[t] = (int)(C.off / bsz[t]);
            C.nblk[t] = (C.n + bsz[t] - 1) / bsz[t];
        }
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
    if (off > 0x7fffffffLL / 4)
        return cleanup(QLSKUM_ERR_INVALID, fmt("batch of %lld points: more than the 32-bit point index allows", off));
    const bool unit_w = params->power == 0.0;
    // the concatenated cloud: per point (padding: interior, no neighbours)
    const long long T_pts = off, nsl = off / 32;
    long long ne_tot = 0;
    std::vector<long long> e_off(n_cases);
    for (int c = 0; c < n_cases; c++) {
        e_off[c] = ne_tot;
        ne_tot += (long long)b->geo[b->cases[c].cloud].ne;
    }
    int8_t *s_flag = A.alloc<int8_t>(T_pts);
    int *s_nb = A.alloc<int>(T_pts);
    double2 *s_nrm = A.alloc<double2>(T_pts);
    float *s_eps = A.alloc<float>(T_pts);
    long long *s_sb = A.alloc<long long>(nsl);
    int *s_case = A.alloc<int>(nsl);
    CaseConst *s_k = A.alloc<CaseConst>(n_cases);
    int *s_enbr = A.alloc<int>(ne_tot);
    uint8_t *s_edir = A.alloc<uint8_t>(ne_tot);
    float2 *s_exy = unit_w ? A.alloc<float2>(ne_tot) : nullptr;
    float4 *s_egeo = unit_w ? nullptr : A.alloc<float4>(ne_tot);
    float *s_edist = A.alloc<float>(ne_tot);
    float2 *s_ew = A.alloc<float2>(ne_tot), *s_ewb = A.alloc<float2>(ne_tot), *s_egw = A.alloc<float2>(ne_tot);
    if (A.err != cudaSuccess) return cleanup(QLSKUM_ERR_CUDA, fmt("cudaMalloc: %s", cudaGetErrorString(A.err)));
    {
        cudaStream_t s = b->L.stream;
        std::vector<long long> sb(nsl);
        std::vector<int> sc(nsl);
        int max_nb = 0;
        for (int c = 0; c < n_cases; c++) {
            const BatchCase &C = b->cases[c];
            const Geometry &G = b->geo[C.cloud];
            const DevCloud &d = G.dc;
            max_nb = std::max(max_nb, d.max_nb);
            std::vector<long long> csb(G.nslices);
            ce = cudaMemcpy(csb.data(), d.slice_base, sizeof(long long) * G.nslices, cudaMemcpyDeviceToHost);
            if (ce != cudaSuccess)
                return cleanup(QLSKUM_ERR_CUDA, fmt("batch cloud: slice bases of cloud %d: %s", C.cloud,
                                                    cudaGetErrorString(ce)));
            const long long s0 = C.off / 32, s1 = (C.off + (C.n + kBatchAlign - 1) / kBatchAlign * kBatchAlign) / 32;
            for (long long t = s0; t < s1; t++) {
                sb[t] = e_off[c] + (t - s0 < G.nslices ? csb[t - s0] : 0);
                sc[t] = c;
            }
        }
        cudaMemsetAsync(s_flag, kInterior, sizeof(int8_t) * T_pts, s);
        cudaMemsetAsync(s_nb, 0, sizeof(int) * T_pts, s);
        cudaMemsetAsync(s_eps, 0, sizeof(float) * T_pts, s);
        mixed::batch_fill_normals(b->L, s_nrm, T_pts);
        for (int c = 0; c < n_cases; c++) {
            const BatchCase &C = b->cases[c];
            const Geometry &G = b->geo[C.cloud];
            const DevCloud &d = G.dc;
            const size_t np = (size_t)G.n, ne = G.ne, e0 = (size_t)e_off[c], p0 = (size_t)C.off;
            auto cp = [&](auto *dst, const auto *src, size_t cnt) {
                cudaMemcpyAsync(dst, src, sizeof(*src) * cnt, cudaMemcpyDeviceToDevice, s);
            };
            cp(s_flag + p0, d.flag, np);
            cp(s_nb + p0, d.nbhs, np);
            cp(s_nrm + p0, d.nrm, np);
            cp(s_eps + p0, d.eps2_32, np);
            mixed::batch_offset_nbr(b->L, d.e_nbr, s_enbr + e0, (long long)ne, (int)C.off);
            cp(s_edir + e0, d.e_dir, ne);
            if (unit_w) cp(s_exy + e0, d.e_xy32, ne);
            else cp(s_egeo + e0, d.e_geo32, ne);
            cp(s_edist + e0, d.e_dist32, ne);
            cp(s_ew + e0, d.e_w32, ne);
            cp(s_ewb + e0, d.e_w32b, ne);
            cp(s_egw + e0, d.e_gw32, ne);
        }
        std::vector<CaseConst> ks(n_cases);
        for (int c = 0; c < n_cases; c++) ks[c] = b->cases[c].K;
        cudaMemcpyAsync(s_sb, sb.data(), sizeof(long long) * nsl, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(s_case, sc.data(), sizeof(int) * nsl, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(s_k, ks.data(), sizeof(CaseConst) * n_cases, cudaMemcpyHostToDevice, s);
        ce = cudaStreamSynchronize(s);
        if (ce == cudaSuccess) ce = cudaGetLastError();
        if (ce != cudaSuccess) return cleanup(QLSKUM_ERR_CUDA, fmt("batch cloud: %s", cudaGetErrorString(ce)));
        DevCloud &S = b->sc;
        S.n = (int)T_pts;
        S.np = (int)T_pts;
        S.flag = s_flag;
        S.nbhs = s_nb;
        S.slice_base = s_sb;
        S.e_nbr = s_enbr;
        S.e_dir = s_edir;
        S.nrm = s_nrm;
        S.eps2_32 = s_eps;
        S.e_xy32 = s_exy;
        S.e_geo32 = s_egeo;
        S.e_dist32 = s_edist;
        S.e_w32 = s_ew;
        S.e_w32b = s_ewb;
        S.e_gw32 = s_egw;
        S.unit_w = unit_w ? 1 : 0;
        S.max_nb = max_nb;
        S.case_k = s_k;
        S.slice_case = s_case;
    }
    BatchCase *d_cases = A.alloc<BatchCase>(n_cases);
    const size_t T = (size_t)b->total;
    for (int k = 0; k < 3; k++) b->prim[k] = A.alloc<double4_32a>(T);
    for (int k = 0; k < 2; k++) b->q[k] = A.alloc<float4>(T);
    for (int k = 0; k < 3; k++) b->dq[k] = A.alloc<float4>(2 * T);
    b->qm = A.alloc<float4>(2 * T);
    b->delta = A.alloc<float>(T);
    b->cspeed = A.alloc<float>(T);
    b->psum = A.alloc<double>(T / 64);
    b->pmax = A.alloc<double>(T / 64);
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
    cudaMemcpyAsync(d_cases, b->cases.data(), sizeof(BatchCase) * n_cases, cudaMemcpyHostToDevice, s);
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
    for (int k = 0; k < 3; k++) cudaMemsetAsync(b->dq[k], 0, sizeof(float4) * 2 * T, s);
    ce = cudaStreamSynchronize(s);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    if (ce != cudaSuccess) return cleanup(QLSKUM_ERR_CUDA, fmt("batch upload: %s", cudaGetErrorString(ce)));
    b->view.cases = d_cases;
    b->view.ncases = n_cases;
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
        mixed::derived(b->L, b->sc, b->prim[b->pcur], b->q[0], b->cspeed);
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

qlskum_status qlskum_batch_lanes(const qlskum_batch *b, int *point_lanes, int *flux_lanes)
{
    if (!b) return QLSKUM_ERR_INVALID;
    if (point_lanes) *point_lanes = b->L.lanes;
    if (flux_lanes) *flux_lanes = mixed::flux_lanes(b->flux_variant);
    return QLSKUM_OK;
}

qlskum_status qlskum_batch_set_launch_config(qlskum_batch *b, int tile, int point_lanes, int flux_variant)
{
    if (!b) return QLSKUM_ERR_INVALID;
    if (tile != 64 && tile != 128 && tile != 256) return bfail(b, QLSKUM_ERR_INVALID, "tile must be 64, 128 or 256");
    if (point_lanes != 1 && point_lanes != 2 && point_lanes != 4)
        return bfail(b, QLSKUM_ERR_INVALID, "point_lanes must be 1, 2 or 4");
    if (flux_variant < 0 || flux_variant >= mixed::flux_variants())
        return bfail(b, QLSKUM_ERR_INVALID, fmt("flux_variant not in 0..%d", mixed::flux_variants() - 1));
    b->L.block = tile;
    b->L.staged = 0;
    b->L.lanes = point_lanes;
    b->flux_variant = flux_variant;
    b->tuned = true;
    for (auto &g : b->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    return QLSKUM_OK;
}

void *qlskum_batch_stream(qlskum_batch *b) { return b ? (void *)b->L.stream : nullptr; }

qlskum_status qlskum_batch_tuning(const qlskum_batch *b, int *tile, int *flux_tile, int *flux_min_blocks,
                                  int *points_per_warp)
{
    if (!b) return QLSKUM_ERR_INVALID;
    if (tile) *tile = b->L.block;
    if (flux_tile) *flux_tile = batch_flux_points(b->flux_variant);
    if (flux_min_blocks) *flux_min_blocks = mixed::flux_min_blocks(b->flux_variant);
    if (points_per_warp) *points_per_warp = 32 / mixed::flux_lanes(b->flux_variant);
    return QLSKUM_OK;
}

}  // extern "C"


// ============================================================ partitions (halo exchange)
//
// The reference's distributed layout (data_structure_mod.h:4-8: local_points,
// ghost_points and pghost, the global numbers of the ghost points;
// point_preprocessing_mod.h:124-132 reads them per partition): the cloud is
// cut into partitions, each holds the points it owns followed by copies of
// the points its own points read (the ghosts), and the ghosts are refreshed
// from their owners whenever the owners' values change.  Here the partitions
// share one GPU, each with its own stream, geometry and state.  An exchange
// is an event barrier between the partitions that share ghosts followed by
// one gather launch per (partition, owner) pair and field that reads the
// owner's array (across GPUs the same lists become peer reads or NCCL send /
// receive pairs).  The residual norm and the objectives are sums over the
// partitions: the all-reduce of a distributed run.

struct PartPull {
    int owner = 0;           // the partition owning these ghosts
    int first = 0, count = 0;  // ghost range [first, first + count) of the receiving partition
    int *d_src = nullptr;    // their positions in the owner [count]
};

struct PartDev {
    PartSpec spec;
    Geometry G;
    DeviceArena A;
    Launch L;
    State64 s64;
    State32 s32;
    cudaEvent_t ev = nullptr;
    std::vector<PartPull> pulls;
    std::vector<int> peers;            // partitions it pulls from or that pull from it
    int red_off = 0, red_blocks = 0;   // its residual partials in the shared arrays
    double *d_obj = nullptr, *d_obj_partial = nullptr, *d_entropy = nullptr;
};

struct qlskum_partition {
    qlskum_params prm{};
    int n = 0, nparts = 0;
    CaseConst K{};
    std::vector<PartDev *> parts;
    std::vector<int> part_of, pos_of;  // global point -> partition, position in it
    DeviceArena A;                     // the shared residual arrays
    cudaStream_t host_stream = nullptr;
    Reduce R;
    int pcur = 0;
    bool derived_valid = false;
    int it = 0;
    int flux_variant = 5;              // mixed: the fused kernel's launch shape
    int point_block = 128, staged = 0; // mixed: gradient / inner-loop launch shape
    long long launches = 0;
    long long halo_bytes = 0;          // bytes the exchanges of one iteration move
    std::string err;
};

namespace {

qlskum_status pfail(qlskum_partition *P, qlskum_status s, const std::string &msg)
{
    if (P) P->err = msg;
    else g_create_error = msg;
    return s;
}

#define PCK(P, call)                                                                          \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return pfail(P, QLSKUM_ERR_CUDA, fmt("%s: %s", #call, cudaGetErrorString(e_))); \
    } while (0)

// Partition plan: the points sorted by the Morton code of their coordinates
// and cut into n_parts contiguous ranges of (nearly) equal size, so each
// partition is a compact region and its ghost layer a thin band; inside a
// partition its points run in the single-domain device order (class, then
// Morton code); each partition's ghosts are the points outside it that its
// own points have as neighbours, grouped by owner and in the owner's order.
void plan_partitions(const qlskum_cloud *c, int nparts, std::vector<int> &part_of, std::vector<int> &pos_of,
                     std::vector<PartSpec> &specs)
{
    const int n = c->n, NB = QLSKUM_MAX_NBHS;
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
        key[i] = morton2(qx, qy);
    }
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
    part_of.assign(n, 0);
    for (int r = 0; r < n; r++) part_of[order[r]] = (int)((long long)r * nparts / n);
    specs.assign(nparts, PartSpec());
    static const int rank[3] = {0, 2, 1};
    for (int i : order) specs[part_of[i]].local.push_back(i);
    pos_of.assign(n, 0);
    for (auto &sp : specs) {
        std::stable_sort(sp.local.begin(), sp.local.end(), [&](int a, int b) {
            const int ra = rank[c->flag_1[a]], rb = rank[c->flag_1[b]];
            return ra != rb ? ra < rb : key[a] < key[b];
        });
        for (size_t t = 0; t < sp.local.size(); t++) pos_of[sp.local[t]] = (int)t;
    }
    for (int p = 0; p < nparts; p++) {
        PartSpec &sp = specs[p];
        std::vector<int> g;
        for (int i : sp.local)
            for (int r = 0; r < c->nbhs[i]; r++) {
                const int k = c->conn[(size_t)i * NB + r] - 1;
                if (part_of[k] != p) g.push_back(k);
            }
        std::sort(g.begin(), g.end(), [&](int a, int b) {
            return part_of[a] != part_of[b] ? part_of[a] < part_of[b] : pos_of[a] < pos_of[b];
        });
        g.erase(std::unique(g.begin(), g.end()), g.end());
        sp.ghost = std::move(g);
        sp.slot.assign(n, -1);
        for (size_t t = 0; t < sp.local.size(); t++) sp.slot[sp.local[t]] = (int)t;
        for (size_t t = 0; t < sp.ghost.size(); t++) sp.slot[sp.ghost[t]] = (int)(sp.local.size() + t);
    }
}

struct FieldRef {
    void *base;
    int bytes;   // per point
};

// One exchange: every partition waits for the partitions it shares ghosts
// with to reach this point, then pulls the `nf` fields field(d, j) of its
// ghosts from their owners.
template <typename F> void part_exchange(qlskum_partition *P, int nf, F &&field)
{
    for (PartDev *d : P->parts) cudaEventRecord(d->ev, d->L.stream);
    for (PartDev *d : P->parts)
        for (int o : d->peers) cudaStreamWaitEvent(d->L.stream, P->parts[o]->ev, 0);
    for (PartDev *d : P->parts)
        for (const PartPull &pl : d->pulls)
            for (int j = 0; j < nf; j++) {
                const FieldRef src = field(*P->parts[pl.owner], j), dst = field(*d, j);
                halo::pull(d->L, pl.count, pl.d_src, src.base,
                           static_cast<char *>(dst.base) + (size_t)(d->G.n + pl.first) * dst.bytes, dst.bytes);
            }
}

// Every partition's stream waits for partition `from`'s stream.
void part_join(qlskum_partition *P, int from)
{
    PartDev *s = P->parts[from];
    cudaEventRecord(s->ev, s->L.stream);
    for (PartDev *d : P->parts)
        if (d != s) cudaStreamWaitEvent(d->L.stream, s->ev, 0);
}

// Partition 0's stream waits for every other partition's.
void part_gather(qlskum_partition *P)
{
    PartDev *z = P->parts[0];
    for (PartDev *d : P->parts)
        if (d != z) {
            cudaEventRecord(d->ev, d->L.stream);
            cudaStreamWaitEvent(z->L.stream, d->ev, 0);
        }
}

// The residual partials of each partition's fused kernel, packed back to back.
void part_reduce_layout(qlskum_partition *P)
{
    const bool mx = P->prm.precision == QLSKUM_MIXED;
    int off = 0;
    for (PartDev *d : P->parts) {
        d->red_off = off;
        d->red_blocks = mx ? mixed::flux_grid_blocks(P->flux_variant, d->G.n) : (d->G.n + 127) / 128;
        off += d->red_blocks;
    }
    P->R.blocks = off;
}

// One iteration over all partitions (the fused path of enqueue_iteration,
// stage by stage, with the ghosts refreshed before every kernel that reads
// a neighbour's value: q and, in the first stage, the wave speed before the
// gradient; dq and qm after it; dq after each inner step).
void part_iteration(qlskum_partition *P, int o)
{
    const int x = (o + 1) % 3, y = (o + 2) % 3;
    const int dst[4] = {x, y, x, y}, src[4] = {o, x, y, x};
    const int ni = P->prm.inner_iterations;
    const bool mx = P->prm.precision == QLSKUM_MIXED;
    const float cfl32 = (float)P->K.cfl;
    for (int rk = 1; rk <= 4; rk++) {
        const int qa = (rk - 1) & 1, qb = rk & 1;
        if (mx)
            part_exchange(P, rk == 1 ? 2 : 1, [&](PartDev &d, int j) {
                return j == 0 ? FieldRef{d.s32.q[qa], 16} : FieldRef{d.s32.cspeed, 4};
            });
        else
            part_exchange(P, rk == 1 ? 2 : 1, [&](PartDev &d, int j) {
                return j == 0 ? FieldRef{d.s64.q[qa], 32} : FieldRef{d.s64.cspeed, 8};
            });
        for (PartDev *d : P->parts) {
            if (mx)
                mixed::q_derivatives(d->L, d->G.dc, d->s32.q[qa], d->s32.dq[0], d->s32.qm, d->s32.cspeed,
                                     rk == 1 ? d->s32.delta : nullptr, cfl32);
            else
                fp64::q_derivatives(d->L, d->G.dc, d->s64.q[qa], d->s64.dq[0], d->s64.qm, d->s64.cspeed,
                                    rk == 1 ? d->s64.delta : nullptr, P->K.cfl);
        }
        if (mx)
            part_exchange(P, 2, [&](PartDev &d, int j) {
                return j == 0 ? FieldRef{d.s32.dq[0], 32} : FieldRef{d.s32.qm, 32};
            });
        else
            part_exchange(P, 2, [&](PartDev &d, int j) {
                return j == 0 ? FieldRef{d.s64.dq[0], 64} : FieldRef{d.s64.qm, 64};
            });
        for (int j = 0; j < ni; j++) {
            for (PartDev *d : P->parts) {
                if (mx)
                    mixed::q_inner(d->L, d->G.dc, d->s32.dq[0], d->s32.dq[mixed_dq_in(j)],
                                   d->s32.dq[mixed_dq_out(j)]);
                else
                    fp64::q_inner(d->L, d->G.dc, d->s64.q[qa], d->s64.dq[j & 1], d->s64.dq[(j + 1) & 1]);
            }
            if (mx)
                part_exchange(P, 1, [&](PartDev &d, int) { return FieldRef{d.s32.dq[mixed_dq_out(j)], 32}; });
            else
                part_exchange(P, 1, [&](PartDev &d, int) { return FieldRef{d.s64.dq[(j + 1) & 1], 64}; });
        }
        for (PartDev *d : P->parts) {
            // only the last stage's residual is reported (fpi_solver_mod.h:138)
            Reduce Rk = P->R;
            if (rk == 4) {
                Rk.partial_sum += d->red_off;
                Rk.partial_max += d->red_off;
            } else {
                Rk.partial_sum = Rk.partial_max = nullptr;
            }
            double4_32a *const *prim = d->s64.prim;
            if (mx)
                mixed::flux_update(d->L, d->G.dc, P->K, d->s32.q[qa], d->s32.dq[mixed_dq_final(ni)], d->s32.qm,
                                   d->s32.delta, prim[src[rk - 1]], prim[o], prim[dst[rk - 1]], d->s32.q[qb],
                                   rk == 4 ? d->s32.cspeed : nullptr, rk, Rk, P->flux_variant);
            else
                fp64::flux_update(d->L, d->G.dc, P->K, d->s64.q[qa], d->s64.dq[ni & 1], d->s64.qm, d->s64.delta,
                                  prim[src[rk - 1]], prim[o], prim[dst[rk - 1]], d->s64.q[qb],
                                  rk == 4 ? d->s64.cspeed : nullptr, rk, Rk);
        }
    }
    // the residual norm over all partitions (fpi_solver_mod.h:138-150)
    part_gather(P);
    fp64::reduce_residual(P->parts[0]->L, P->R, P->n, 0);
    part_join(P, 0);
}

// Bytes the ghost exchanges of one iteration move.
long long part_halo_bytes(const qlskum_partition *P)
{
    long long g = 0;
    for (const PartDev *d : P->parts) g += (long long)d->spec.ghost.size();
    const bool mx = P->prm.precision == QLSKUM_MIXED;
    const int ni = P->prm.inner_iterations;
    // per stage: q (+ the wave speed in stage 1), dq0 + qm, ni x dq
    const long long q = mx ? 16 : 32, dq = mx ? 32 : 64, cs = mx ? 4 : 8;
    return g * (4 * (q + 2 * dq + ni * dq) + cs);
}

qlskum_status part_derived(qlskum_partition *P)
{
    if (P->derived_valid) return QLSKUM_OK;
    for (PartDev *d : P->parts) {
        // over the ghost slots too: their state was written with the owners'
        DevCloud all = d->G.dc;
        all.n = d->G.n + (int)d->spec.ghost.size();
        if (P->prm.precision == QLSKUM_MIXED)
            mixed::derived(d->L, all, d->s64.prim[P->pcur], d->s32.q[0], d->s32.cspeed);
        else
            fp64::derived(d->L, all, d->s64.prim[P->pcur], d->s64.q[0], d->s64.cspeed);
    }
    P->derived_valid = true;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pfail(P, QLSKUM_ERR_CUDA, fmt("derived: %s", cudaGetErrorString(e)));
    return QLSKUM_OK;
}

qlskum_status part_sync(qlskum_partition *P)
{
    for (PartDev *d : P->parts) PCK(P, cudaStreamSynchronize(d->L.stream));
    return QLSKUM_OK;
}

qlskum_status part_ensure_hist(qlskum_partition *P, int needed)
{
    if (needed <= P->R.capacity) return QLSKUM_OK;
    int cap = std::max(1024, P->R.capacity);
    while (cap < needed) cap *= 2;
    qlskum_status st = part_sync(P);
    if (st) return st;
    double *nh = nullptr;
    PCK(P, cudaMalloc(&nh, sizeof(double) * 3 * (size_t)cap));
    PCK(P, cudaMemset(nh, 0, sizeof(double) * 3 * (size_t)cap));
    if (P->R.hist) {
        PCK(P, cudaMemcpy(nh, P->R.hist, sizeof(double) * 3 * (size_t)P->R.capacity, cudaMemcpyDeviceToDevice));
        cudaFree(P->R.hist);
    }
    // the copies above run on the legacy stream, unordered with the partitions' streams
    PCK(P, cudaDeviceSynchronize());
    P->R.hist = nh;
    P->R.capacity = cap;
    return QLSKUM_OK;
}

void part_free(qlskum_partition *P)
{
    if (!P) return;
    for (PartDev *d : P->parts) {
        if (d->L.stream) cudaStreamSynchronize(d->L.stream);
        d->A.release();
        if (d->ev) cudaEventDestroy(d->ev);
        if (d->L.stream) cudaStreamDestroy(d->L.stream);
        delete d;
    }
    P->parts.clear();
    if (P->R.hist) cudaFree(P->R.hist);
    P->R.hist = nullptr;
    P->A.release();
    delete P;
}

}  // namespace

extern "C" {

qlskum_status qlskum_partition_plan(const qlskum_cloud *c, int n_parts, int *part_of, int *n_local, int *n_ghost)
{
    qlskum_params p;
    qlskum_default_params(&p);
    int sp = 0;
    qlskum_status st = validate(c, &p, &sp);
    if (st) return st;
    if (n_parts < 1 || n_parts > c->n) return fail(nullptr, QLSKUM_ERR_INVALID, "n_parts must be in 1..n");
    std::vector<int> po, pos;
    std::vector<PartSpec> specs;
    plan_partitions(c, n_parts, po, pos, specs);
    if (part_of) std::copy(po.begin(), po.end(), part_of);
    for (int q = 0; q < n_parts; q++) {
        if (n_local) n_local[q] = (int)specs[q].local.size();
        if (n_ghost) n_ghost[q] = (int)specs[q].ghost.size();
    }
    return QLSKUM_OK;
}

qlskum_status qlskum_partition_plan_lists(const qlskum_cloud *c, int n_parts, int part, int *local_ids,
                                          int *ghost_ids)
{
    qlskum_params p;
    qlskum_default_params(&p);
    int sp = 0;
    qlskum_status st = validate(c, &p, &sp);
    if (st) return st;
    if (n_parts < 1 || n_parts > c->n || part < 0 || part >= n_parts)
        return fail(nullptr, QLSKUM_ERR_INVALID, "n_parts must be in 1..n and part in 0..n_parts-1");
    std::vector<int> po, pos;
    std::vector<PartSpec> specs;
    plan_partitions(c, n_parts, po, pos, specs);
    if (local_ids)
        for (size_t t = 0; t < specs[part].local.size(); t++) local_ids[t] = specs[part].local[t] + 1;
    if (ghost_ids)
        for (size_t t = 0; t < specs[part].ghost.size(); t++) ghost_ids[t] = specs[part].ghost[t] + 1;
    return QLSKUM_OK;
}

qlskum_status qlskum_partition_create(const qlskum_cloud *c, const qlskum_params *p, int n_parts,
                                      qlskum_partition **out)
{
    if (!out) return fail(nullptr, QLSKUM_ERR_INVALID, "null output pointer");
    *out = nullptr;
    int sp = 0;
    qlskum_status st = validate(c, p, &sp);
    if (st) return st;
    if (n_parts < 1 || n_parts > c->n) return fail(nullptr, QLSKUM_ERR_INVALID, "n_parts must be in 1..n");
    Precomp pc;
    st = precompute(c, p, pc);
    if (st) return st;
    qlskum_partition *P = new qlskum_partition();
    P->prm = *p;
    P->n = c->n;
    P->nparts = n_parts;
    P->K = case_of(*p);
    if (p->block_size) P->point_block = p->block_size;
    std::vector<PartSpec> specs;
    plan_partitions(c, n_parts, P->part_of, P->pos_of, specs);
    for (int q = 0; q < n_parts; q++)
        if (specs[q].local.empty()) {
            part_free(P);
            return fail(nullptr, QLSKUM_ERR_INVALID, fmt("partition %d has no points", q));
        }
    const bool mx = p->precision == QLSKUM_MIXED;
    const std::vector<double4_32a> free_stream(1, make_double4_32a(P->K.rho_inf, P->K.u1_inf, P->K.u2_inf,
                                                                  P->K.pr_inf));
    for (int q = 0; q < n_parts; q++) {
        PartDev *d = new PartDev();
        P->parts.push_back(d);
        d->spec = std::move(specs[q]);
        cudaError_t ce = cudaStreamCreateWithFlags(&d->L.stream, cudaStreamNonBlocking);
        if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&d->ev, cudaEventDisableTiming);
        if (ce != cudaSuccess) {
            part_free(P);
            return fail(nullptr, QLSKUM_ERR_CUDA, fmt("stream / event: %s", cudaGetErrorString(ce)));
        }
        d->L.block = P->point_block;
        d->L.staged = P->staged;
        d->L.launches = &P->launches;
        st = build_geometry(c, p, sp, true, mx, d->A, d->L.stream, d->G, &d->spec, &pc);
        if (st) {
            part_free(P);
            return st;
        }
        DeviceArena &A = d->A;
        const size_t np = d->G.np;
        for (int b = 0; b < 3; b++) d->s64.prim[b] = A.alloc<double4_32a>(np);
        for (int b = 0; b < 2; b++) {
            d->s64.q[b] = A.alloc<double4_32a>(np);
            d->s64.dq[b] = A.alloc<double4_32a>(np * 2);
        }
        d->s64.qm = A.alloc<double4_32a>(np * 2);
        d->s64.flux_res = A.alloc<double4_32a>(np);
        d->s64.delta = A.alloc<double>(np);
        d->s64.cspeed = A.alloc<double>(np);
        if (mx) {
            for (int b = 0; b < 2; b++) d->s32.q[b] = A.alloc<float4>(np);
            for (int b = 0; b < 3; b++) d->s32.dq[b] = A.alloc<float4>(np * 2);
            d->s32.qm = A.alloc<float4>(np * 2);
            d->s32.delta = A.alloc<float>(np);
            d->s32.cspeed = A.alloc<float>(np);
        }
        const int nl = d->G.n;
        d->d_obj = A.alloc<double>(8);
        d->d_obj_partial = A.alloc<double>(4 * (size_t)((std::max(nl, d->G.shape_points) + 255) / 256));
        d->d_entropy = A.alloc<double>(np);
        if (A.err != cudaSuccess) {
            part_free(P);
            return fail(nullptr, QLSKUM_ERR_CUDA, fmt("cudaMalloc: %s", cudaGetErrorString(A.err)));
        }
        // initial_conditions_mod.h:23-37 on every slot (ghosts included)
        std::vector<double4_32a> prim0(np, free_stream[0]);
        for (int b = 0; b < 3; b++)
            cudaMemcpyAsync(d->s64.prim[b], prim0.data(), np * sizeof(double4_32a), cudaMemcpyHostToDevice,
                            d->L.stream);
        cudaMemsetAsync(d->s64.dq[0], 0, sizeof(double4_32a) * 2 * np, d->L.stream);
        cudaMemsetAsync(d->s64.dq[1], 0, sizeof(double4_32a) * 2 * np, d->L.stream);
        cudaMemsetAsync(d->s64.qm, 0, sizeof(double4_32a) * 2 * np, d->L.stream);
        ce = cudaStreamSynchronize(d->L.stream);
        if (ce != cudaSuccess) {
            part_free(P);
            return fail(nullptr, QLSKUM_ERR_CUDA, fmt("upload: %s", cudaGetErrorString(ce)));
        }
    }
    // the pull lists (one per owner, ghosts grouped by owner) and the peers
    std::vector<std::vector<char>> peer(n_parts, std::vector<char>(n_parts, 0));
    for (int q = 0; q < n_parts; q++) {
        PartDev *d = P->parts[q];
        const std::vector<int> &g = d->spec.ghost;
        size_t a = 0;
        while (a < g.size()) {
            const int o = P->part_of[g[a]];
            size_t b = a;
            std::vector<int> src;
            while (b < g.size() && P->part_of[g[b]] == o) src.push_back(P->pos_of[g[b++]]);
            PartPull pl;
            pl.owner = o;
            pl.first = (int)a;
            pl.count = (int)(b - a);
            pl.d_src = d->A.alloc<int>(src.size());
            if (d->A.err != cudaSuccess) {
                part_free(P);
                return fail(nullptr, QLSKUM_ERR_CUDA, fmt("cudaMalloc: %s", cudaGetErrorString(d->A.err)));
            }
            const cudaError_t ce = cudaMemcpy(pl.d_src, src.data(), src.size() * sizeof(int),
                                              cudaMemcpyHostToDevice);
            if (ce != cudaSuccess) {
                part_free(P);
                return fail(nullptr, QLSKUM_ERR_CUDA, fmt("ghost list upload: %s", cudaGetErrorString(ce)));
            }
            d->pulls.push_back(pl);
            peer[q][o] = peer[o][q] = 1;
            a = b;
        }
    }
    for (int q = 0; q < n_parts; q++)
        for (int o = 0; o < n_parts; o++)
            if (peer[q][o] && o != q) P->parts[q]->peers.push_back(o);
    // the shared residual arrays: a partial per 32 points of each partition is enough for any launch shape
    int maxp = 0;
    for (PartDev *d : P->parts) maxp += (d->G.n + 31) / 32;
    P->R.max_blocks = maxp;
    P->R.partial_sum = P->A.alloc<double>(maxp);
    P->R.partial_max = P->A.alloc<double>(maxp);
    P->R.res_old = P->A.alloc<double>(1);
    P->R.iter = P->A.alloc<int>(1);
    P->R.status = P->A.alloc<int>(1);
    if (P->A.err != cudaSuccess) {
        part_free(P);
        return fail(nullptr, QLSKUM_ERR_CUDA, fmt("cudaMalloc: %s", cudaGetErrorString(P->A.err)));
    }
    cudaMemset(P->R.res_old, 0, sizeof(double));
    cudaMemset(P->R.iter, 0, sizeof(int));
    cudaMemset(P->R.status, 0, sizeof(int));
    part_reduce_layout(P);
    P->halo_bytes = part_halo_bytes(P);
    st = part_ensure_hist(P, 1024);
    if (st) {
        const std::string m = P->err;
        part_free(P);
        return fail(nullptr, st, m);
    }
    cudaError_t ce = cudaDeviceSynchronize();
    if (ce != cudaSuccess) {
        part_free(P);
        return fail(nullptr, QLSKUM_ERR_CUDA, fmt("partition set-up: %s", cudaGetErrorString(ce)));
    }
    *out = P;
    return QLSKUM_OK;
}

qlskum_status qlskum_partition_destroy(qlskum_partition *P)
{
    part_free(P);
    return QLSKUM_OK;
}

const char *qlskum_partition_last_error(const qlskum_partition *P)
{
    return P ? P->err.c_str() : g_create_error.c_str();
}

qlskum_status qlskum_partition_layout(const qlskum_partition *P, int part, int *n_local, int *n_ghost, int *local_ids,
                                      int *ghost_ids)
{
    if (!P || part < 0 || part >= P->nparts) return QLSKUM_ERR_INVALID;
    const PartSpec &sp = P->parts[part]->spec;
    if (n_local) *n_local = (int)sp.local.size();
    if (n_ghost) *n_ghost = (int)sp.ghost.size();
    if (local_ids)
        for (size_t t = 0; t < sp.local.size(); t++) local_ids[t] = sp.local[t] + 1;
    if (ghost_ids)
        for (size_t t = 0; t < sp.ghost.size(); t++) ghost_ids[t] = sp.ghost[t] + 1;
    return QLSKUM_OK;
}

qlskum_status qlskum_partition_set_launch_config(qlskum_partition *P, int flux_variant, int point_block, int staged)
{
    if (!P) return QLSKUM_ERR_INVALID;
    if (flux_variant < 0 || flux_variant >= mixed::flux_variants())
        return pfail(P, QLSKUM_ERR_INVALID, "flux_variant out of range");
    if (point_block != 64 && point_block != 128 && point_block != 256 && point_block != 512)
        return pfail(P, QLSKUM_ERR_INVALID, "point_block must be 64, 128, 256 or 512");
    if (staged < 0 || staged > 4) return pfail(P, QLSKUM_ERR_INVALID, "staged must be in 0..4");
    if (staged > 0 && P->prm.precision == QLSKUM_MIXED)
        for (PartDev *d : P->parts)
            if (mixed::staged_variants(d->G.dc) < staged)
                return pfail(P, QLSKUM_ERR_UNSUPPORTED, "staged variant does not fit this cloud");
    qlskum_status st = part_sync(P);
    if (st) return st;
    P->flux_variant = flux_variant;
    P->point_block = point_block;
    P->staged = staged;
    for (PartDev *d : P->parts) {
        d->L.block = point_block;
        d->L.staged = staged;
    }
    part_reduce_layout(P);
    return QLSKUM_OK;
}

qlskum_status qlskum_partition_q_lskum(qlskum_partition *P, int iters)
{
    if (!P) return fail(nullptr, QLSKUM_ERR_INVALID, "null partition");
    if (iters < 0) return pfail(P, QLSKUM_ERR_INVALID, "iters < 0");
    qlskum_status st = part_ensure_hist(P, P->it + iters);
    if (st) return st;
    st = part_derived(P);
    if (st) return st;
    // the device iteration counter continues from the host's
    PartDev *z = P->parts[0];
    PCK(P, cudaMemcpyAsync(P->R.iter, &P->it, sizeof(int), cudaMemcpyHostToDevice, z->L.stream));
    PCK(P, cudaStreamSynchronize(z->L.stream));
    for (int t = 0; t < iters; t++) {
        const int o = P->pcur;
        part_iteration(P, o);
        P->pcur = (o + 2) % 3;
        P->it += 1;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pfail(P, QLSKUM_ERR_CUDA, fmt("partition iteration: %s", cudaGetErrorString(e)));
    st = part_sync(P);
    if (st) return st;
    int bad = 0;
    PCK(P, cudaMemcpy(&bad, P->R.status, sizeof(int), cudaMemcpyDeviceToHost));
    if (bad) return pfail(P, QLSKUM_ERR_NONFINITE, "residual became non-finite (NaN/Inf in the state)");
    return QLSKUM_OK;
}

qlskum_status qlskum_partition_get_prim(qlskum_partition *P, double *out)
{
    if (!P || !out) return QLSKUM_ERR_INVALID;
    qlskum_status st = part_sync(P);
    if (st) return st;
    for (PartDev *d : P->parts) {
        const int nl = d->G.n;
        std::vector<double4_32a> h(nl);
        PCK(P, cudaMemcpy(h.data(), d->s64.prim[P->pcur], nl * sizeof(double4_32a), cudaMemcpyDeviceToHost));
        for (int t = 0; t < nl; t++) {
            double *o4 = out + 4 * (size_t)d->spec.local[t];
            o4[0] = h[t].x; o4[1] = h[t].y; o4[2] = h[t].z; o4[3] = h[t].w;
        }
    }
    return QLSKUM_OK;
}

qlskum_status qlskum_partition_set_prim(qlskum_partition *P, const double *prim)
{
    if (!P || !prim) return QLSKUM_ERR_INVALID;
    qlskum_status st = part_sync(P);
    if (st) return st;
    for (PartDev *d : P->parts) {
        const size_t ns = d->spec.local.size() + d->spec.ghost.size();
        std::vector<double4_32a> h(ns);
        for (size_t t = 0; t < ns; t++) {
            const int g = t < d->spec.local.size() ? d->spec.local[t] : d->spec.ghost[t - d->spec.local.size()];
            const double *p4 = prim + 4 * (size_t)g;
            h[t] = make_double4_32a(p4[0], p4[1], p4[2], p4[3]);
        }
        PCK(P, cudaMemcpy(d->s64.prim[P->pcur], h.data(), ns * sizeof(double4_32a), cudaMemcpyHostToDevice));
    }
    P->derived_valid = false;
    return QLSKUM_OK;
}

qlskum_status qlskum_partition_residual_history(qlskum_partition *P, double *out, int max_rows, int *rows)
{
    if (!P) return QLSKUM_ERR_INVALID;
    qlskum_status st = part_sync(P);
    if (st) return st;
    const int k = std::min(P->it, std::max(0, max_rows));
    if (rows) *rows = P->it;
    if (out && k > 0) PCK(P, cudaMemcpy(out, P->R.hist, sizeof(double) * 3 * (size_t)k, cudaMemcpyDeviceToHost));
    return QLSKUM_OK;
}

qlskum_status qlskum_partition_objective(qlskum_partition *P, double *cl, double *cd, double *cm,
                                         double *total_entropy)
{
    if (!P) return QLSKUM_ERR_INVALID;
    const double cp_scale = 0.5 * P->K.rho_inf * P->K.mach * P->K.mach;
    double sum[4] = {0, 0, 0, 0};
    for (PartDev *d : P->parts)
        fp64::objective(d->L, d->G.dc, d->s64.prim[P->pcur], d->G.d_wall_perm, d->G.d_wall_geo, d->G.shape_points,
                        cp_scale, P->K.pr_inf, P->K.gamma, d->d_entropy, d->d_obj, d->d_obj_partial);
    // the all-reduce: the partitions' sums added in partition order
    for (PartDev *d : P->parts) {
        double o[4];
        PCK(P, cudaMemcpyAsync(o, d->d_obj, sizeof o, cudaMemcpyDeviceToHost, d->L.stream));
        PCK(P, cudaStreamSynchronize(d->L.stream));
        for (int j = 0; j < 4; j++) sum[j] += o[j];
    }
    const double H = sum[0], V = sum[1];
    if (cl) *cl = V * std::cos(P->K.theta) - H * std::sin(P->K.theta);
    if (cd) *cd = H * std::cos(P->K.theta) + V * std::sin(P->K.theta);
    if (cm) *cm = sum[2];
    if (total_entropy) *total_entropy = sum[3];
    return QLSKUM_OK;
}

long long qlskum_partition_halo_bytes(const qlskum_partition *P) { return P ? P->halo_bytes : 0; }

long long qlskum_partition_launch_count(const qlskum_partition *P) { return P ? P->launches : 0; }

}  // extern "C"

// ============================================================ diagnostics and files

namespace {

struct Stagnation {
    double p0_inf, p0_min, p0_max, sum_sq, sum_p0, J;
    long long i_min, i_max;  // device order
};

// stagnation_values_mod.h at `prim`: extremes, and objective_function_J
// (:51-80) with the sum it accumulates and plen = the number of points summed
// (the reference multiplies an uninitialised total and never sets plen).
qlskum_status stagnation_values(qlskum_handle *h, const double4_32a *prim, Stagnation &sv)
{
    const double g = h->K.gamma, gp = g / (g - 1);
    sv.p0_inf = h->K.pr_inf * std::pow(1 + ((g - 1) / 2) * h->K.mach * h->K.mach, gp);
    fp64::stagnation(h->L, h->n, prim, g, sv.p0_inf, h->d_diag);
    qlskum_status st = check_launch(h, "stagnation");
    if (st) return st;
    const int blocks = (h->n + 255) / 256;
    std::vector<double> part(6 * (size_t)blocks);
    CK(h, cudaMemcpyAsync(part.data(), h->d_diag, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    sv.p0_min = part[0];
    sv.p0_max = part[2];
    sv.i_min = (long long)part[1];
    sv.i_max = (long long)part[3];
    sv.sum_sq = sv.sum_p0 = 0.0;
    for (int b = 0; b < blocks; b++) {
        const double *o = &part[6 * (size_t)b];
        if (o[0] < sv.p0_min || (o[0] == sv.p0_min && (long long)o[1] < sv.i_min)) { sv.p0_min = o[0]; sv.i_min = (long long)o[1]; }
        if (o[2] > sv.p0_max || (o[2] == sv.p0_max && (long long)o[3] < sv.i_max)) { sv.p0_max = o[2]; sv.i_max = (long long)o[3]; }
        sv.sum_sq += o[4];
        sv.sum_p0 += o[5];
    }
    sv.J = sv.sum_sq / (sv.p0_inf * sv.p0_inf * (double)h->n);
    return QLSKUM_OK;
}

qlskum_status download_prim(qlskum_handle *h, std::vector<double4_32a> &dev)
{
    dev.resize(h->np);
    CK(h, cudaMemcpyAsync(dev.data(), h->s64.prim[h->pcur], sizeof(double4_32a) * h->np, cudaMemcpyDeviceToHost,
                          h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    return QLSKUM_OK;
}

// Rows "<n> <it> <res_old>" then per point x y flag_1 and, in `order`, the
// primitive state, Mach number and entropy (compute_entropy_mod.h:5-24).
qlskum_status write_state(qlskum_handle *h, const char *path, bool restart_order)
{
    if (!path) return fail(h, QLSKUM_ERR_INVALID, "null path");
    qlskum_status st = qlskum_objective(h, nullptr, nullptr, nullptr, nullptr);  // fills the entropy field
    if (st) return st;
    std::vector<double4_32a> dev;
    if ((st = download_prim(h, dev))) return st;
    std::vector<double> ent(h->np);
    double res_old = 0.0;
    CK(h, cudaMemcpyAsync(ent.data(), h->d_entropy, sizeof(double) * h->np, cudaMemcpyDeviceToHost, h->L.stream));
    CK(h, cudaMemcpyAsync(&res_old, h->R.res_old, sizeof(double), cudaMemcpyDeviceToHost, h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    FILE *f = std::fopen(path, "w");
    if (!f) return fail(h, QLSKUM_ERR_INVALID, fmt("cannot open %s", path));
    std::fprintf(f, "%d %d %.17g\n", h->n, h->it, res_old);
    for (int i = 0; i < h->n; i++) {
        const int pp = h->perm[i];
        const double4_32a P = dev[pp];
        const double sos = std::sqrt(h->K.gamma * P.w / P.x);
        const double mach = std::sqrt(P.y * P.y + P.z * P.z) / sos;
        if (restart_order)
            std::fprintf(f, "%.17g %.17g %d %.17g %.17g %.17g %.17g %.17g %.17g\n", h->hx[i], h->hy[i], h->hflag[i],
                         mach, ent[pp], P.x, P.y, P.z, P.w);
        else
            std::fprintf(f, "%.17g %.17g %d %.17g %.17g %.17g %.17g %.17g %.17g\n", h->hx[i], h->hy[i], h->hflag[i],
                         P.x, P.y, P.z, P.w, mach, ent[pp]);
    }
    const bool ok = std::fflush(f) == 0 && !std::ferror(f);
    std::fclose(f);
    return ok ? QLSKUM_OK : fail(h, QLSKUM_ERR_INVALID, fmt("write failed: %s", path));
}

}  // namespace

extern "C" {

qlskum_status qlskum_enstrophy(qlskum_handle *h, double *total, double *vorticity)
{
    NEED(h);
    fp64::enstrophy(h->L, h->dc, h->s64.prim[h->pcur], h->d_vort, h->d_diag);
    qlskum_status st = check_launch(h, "enstrophy");
    if (st) return st;
    const int blocks = (h->n + 255) / 256;
    std::vector<double> part(blocks);
    CK(h, cudaMemcpyAsync(part.data(), h->d_diag, sizeof(double) * blocks, cudaMemcpyDeviceToHost, h->L.stream));
    std::vector<double> vort;
    if (vorticity) {
        vort.resize(h->np);
        CK(h, cudaMemcpyAsync(vort.data(), h->d_vort, sizeof(double) * h->np, cudaMemcpyDeviceToHost, h->L.stream));
    }
    CK(h, cudaStreamSynchronize(h->L.stream));
    double t = 0.0;
    for (double v : part) t += v;
    if (total) *total = t;
    if (vorticity) unpermute(h, vort, vorticity, 1);
    return QLSKUM_OK;
}

qlskum_status qlskum_stagnation(qlskum_handle *h, double *p0_min, double *p0_max, int *i_min, int *i_max, double *J)
{
    NEED(h);
    Stagnation sv;
    qlskum_status st = stagnation_values(h, h->s64.prim[h->pcur], sv);
    if (st) return st;
    if (p0_min) *p0_min = sv.p0_min;
    if (p0_max) *p0_max = sv.p0_max;
    if (i_min) *i_min = h->iperm[sv.i_min] + 1;
    if (i_max) *i_max = h->iperm[sv.i_max] + 1;
    if (J) *J = sv.J;
    return QLSKUM_OK;
}

qlskum_status qlskum_write_restart(qlskum_handle *h, const char *path)
{
    NEED(h);
    return write_state(h, path, true);
}

qlskum_status qlskum_write_output(qlskum_handle *h, const char *path)
{
    NEED(h);
    return write_state(h, path, false);
}

// restart_sol (initial_conditions_mod.h:7-21): "<nop> <itr> <res_old>", then
// per point five skipped numbers and rho u1 u2 p.
qlskum_status qlskum_read_restart(qlskum_handle *h, const char *path)
{
    NEED(h);
    if (!path) return fail(h, QLSKUM_ERR_INVALID, "null path");
    FILE *f = std::fopen(path, "r");
    if (!f) return fail(h, QLSKUM_ERR_INVALID, fmt("cannot open %s", path));
    double nop = 0, itr = 0, res_old = 0;
    if (std::fscanf(f, "%lf %lf %lf", &nop, &itr, &res_old) != 3) {
        std::fclose(f);
        return fail(h, QLSKUM_ERR_INVALID, "malformed restart header");
    }
    std::vector<double> prim((size_t)h->n * 4);
    for (int i = 0; i < h->n; i++) {
        double s5[5];
        double *p = &prim[(size_t)i * 4];
        if (std::fscanf(f, "%lf %lf %lf %lf %lf %lf %lf %lf %lf", &s5[0], &s5[1], &s5[2], &s5[3], &s5[4], &p[0], &p[1],
                        &p[2], &p[3]) != 9) {
            std::fclose(f);
            return fail(h, QLSKUM_ERR_INVALID, fmt("restart file ends before point %d of %d", i + 1, h->n));
        }
    }
    std::fclose(f);
    qlskum_status st = qlskum_set_prim(h, prim.data());
    if (st) return st;
    h->it = (int)itr;
    CK(h, cudaMemcpyAsync(h->R.res_old, &res_old, sizeof(double), cudaMemcpyHostToDevice, h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    // fpi_solver_mod.h:139: a restarted run keeps the file's res_old
    h->R.latch = 0;
    h->restarted = true;
    for (auto &g : h->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    return ensure_hist(h, h->it + 1);
}

}  // extern "C"

// ============================================================ discrete adjoint
//
// Reverse mode of the iteration (qlskum_adjoint.cu holds the kernels).
// The stage states of an iteration are recomputed from its checkpointed
// state by the module kernels of the handle's precision, whose results equal
// the fused solver's; the reverse sweep then runs stage by stage from the
// last.  FP64 handles, and wall-displacement gradients on any handle, take
// the FP64 reverse; Mach / AoA / initial-state gradients of a mixed handle
// take the reverse of the mixed iteration (FP32 edge work, FP64 update).

// One iteration's stage data of the mixed form (FP32) with its five stage
// states: what the reverse of that iteration reads.
struct Set32 {
    double4_32a *P[5] = {};
    float4 *q32[4] = {};
    std::vector<float4 *> dq32;        // [stage][inner step 0 .. ni], each [np][2]
    float4 *qm32[4] = {};
    float4 *acc32[4] = {};             // the flux kernel's weighted sums
    float *delta32 = nullptr, *cs32 = nullptr;
};

// One iteration's stage data of the FP64 form with its five stage states.
struct Set64 {
    double4_32a *P[5] = {};
    double4_32a *q[4] = {};            // q of P[0 .. 3]
    std::vector<double4_32a *> dq;     // [stage][inner step 0 .. ni], each [np][2]
    double4_32a *qm[4] = {};
    double *delta = nullptr;
    double4_32a *flux[4] = {};         // each stage's flux residual
    double *sums[4] = {};              // each stage's directional sums (wall gradients only), [n][32]
    double *ends[4] = {};              // each stage's edge-end transcendentals, [12][ne] (fp64::flux_residual)
};

struct AdjBuf {
    DeviceArena arena;
    int ni = 0;
    bool geo = false, has64 = false, has32 = false;
    size_t ne = 0;
    double4_32a *P[5] = {};            // stage states of one iteration
    Set64 set64;                       // the FP64 stage data of one iteration (its states are P)
    std::vector<Set64> sets64;         // one per iteration of a segment, on demand (set_arena)
    double4_32a *bP = nullptr, *bPacc = nullptr, *bF = nullptr, *bq = nullptr, *bdqA = nullptr, *bdqB = nullptr,
                *bqm = nullptr, *lam = nullptr, *lam_prev = nullptr, *seed = nullptr;
    double *bdelta = nullptr, *bc = nullptr, *buinf = nullptr;
    // geometry adjoints (wall-displacement gradients only)
    double4_32a *bedge = nullptr;
    double *bdist = nullptr;
    double2 *bnrm = nullptr;
    double4_32a *bgmom = nullptr, *bfmom = nullptr;
    uint8_t *geo_pt = nullptr;              // AdjView::geo_pt
    int *geo_list = nullptr;                // AdjView::geo_list
    int n_geo = 0;
    double *gbx = nullptr, *gby = nullptr;  // coordinate bars (geom_pullback)
    double2 *gbn = nullptr;                 // normal bars (geom_pullback)
    // the checkpointed primal: the state of every stride-th iteration, and
    // the states of one stride-long segment recomputed during the reverse sweep
    double4_32a *ckpt = nullptr;
    int ckpt_cap = 0;
    double4_32a *seg = nullptr;
    int seg_cap = 0;
    // the mixed iteration's stage data (FP32): set 0 (its states are P) and,
    // on demand, one set per iteration of a segment (own states, own arena)
    Set32 set0;
    std::vector<Set32> sets;
    DeviceArena set_arena;             // the on-demand sets (FP32 or FP64, one kind at a time)
    bool sets_geo = false;             // the FP64 sets carry the directional sums
    float4 *bF32 = nullptr;            // bar of the flux residual
    float4 *bs32 = nullptr;            // bar of the weighted sums (delta * bF)
    AdjT T;                            // the edge list transposed (mixed reverse)
    float4 *bq32 = nullptr, *bdqA32 = nullptr, *bdqB32 = nullptr, *bdq0_32 = nullptr, *bqm32 = nullptr;
    float *bdelta32 = nullptr, *bcs32 = nullptr;
};

void adj_free(qlskum_handle *h)
{
    if (!h->adj) return;
    if (h->adj->ckpt) cudaFree(h->adj->ckpt);
    if (h->adj->seg) cudaFree(h->adj->seg);
    h->adj->set_arena.release();
    h->adj->arena.release();
    delete h->adj;
    h->adj = nullptr;
}

namespace {

// Sliced-ELL slice bases of the handle's point order (as build_geometry lays
// them out) and the edge-slot count.
std::vector<long long> slice_bases(const qlskum_handle *h, size_t *ne)
{
    std::vector<long long> sb(h->nslices);
    long long tot = 0;
    for (int s2 = 0; s2 < h->nslices; s2++) {
        int w = 0;
        for (int l = 0; l < 32; l++) {
            const int pp = s2 * 32 + l;
            if (pp < h->n) w = std::max(w, h->hnbhs[h->iperm[pp]]);
        }
        sb[s2] = tot;
        tot += 32LL * w;
    }
    if (ne) *ne = (size_t)std::max(tot, 32LL);
    return sb;
}

qlskum_status d2h(qlskum_handle *h, void *dst, const void *src, size_t bytes)
{
    CK(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    return QLSKUM_OK;
}

void zero(qlskum_handle *h, void *p, size_t bytes) { cudaMemsetAsync(p, 0, bytes, h->L.stream); }

// The forward edge list transposed (AdjT), from the device's own copies of
// the per-edge data so that the reverse reads exactly what the forward did.
qlskum_status adj_transpose(qlskum_handle *h)
{
    AdjBuf *a = h->adj;
    const DevCloud &c = h->dc;
    const int n = h->n, np = h->np, ns = h->nslices;
    size_t ne = 0;
    slice_bases(h, &ne);
    std::vector<long long> sb(ns);
    std::vector<int> nbh(np), enbr(ne);
    std::vector<float2> exy(ne), egw(ne), ew(ne);
    std::vector<uint8_t> edir(ne);
    std::vector<double2> nrm(np);
    std::vector<int8_t> flag(np);
    qlskum_status st;
    if ((st = d2h(h, sb.data(), c.slice_base, sizeof(long long) * ns))) return st;
    if ((st = d2h(h, nbh.data(), c.nbhs, sizeof(int) * np))) return st;
    if ((st = d2h(h, enbr.data(), c.e_nbr, sizeof(int) * ne))) return st;
    if (c.unit_w) {
        if ((st = d2h(h, exy.data(), c.e_xy32, sizeof(float2) * ne))) return st;
    } else {
        std::vector<float4> g(ne);
        if ((st = d2h(h, g.data(), c.e_geo32, sizeof(float4) * ne))) return st;
        for (size_t e = 0; e < ne; e++) exy[e] = make_float2(g[e].x, g[e].y);
    }
    if ((st = d2h(h, egw.data(), c.e_gw32, sizeof(float2) * ne))) return st;
    if ((st = d2h(h, ew.data(), c.e_w32, sizeof(float2) * ne))) return st;
    if ((st = d2h(h, edir.data(), c.e_dir, ne))) return st;
    if ((st = d2h(h, nrm.data(), c.nrm, sizeof(double2) * np))) return st;
    if ((st = d2h(h, flag.data(), c.flag, np))) return st;
    // incoming counts, then the transposed slices
    std::vector<int> tnb(np, 0);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < nbh[i]; j++) tnb[enbr[(size_t)(sb[i >> 5] + 32LL * j + (i & 31))]]++;
    std::vector<long long> tsb(ns);
    long long tot = 0;
    for (int s2 = 0; s2 < ns; s2++) {
        int w = 0;
        for (int l = 0; l < 32; l++) w = std::max(w, tnb[s2 * 32 + l]);
        tsb[s2] = tot;
        tot += 32LL * w;
    }
    const size_t nt = (size_t)std::max(tot, 32LL);
    std::vector<int> tsrc(nt, 0), te(nt, 0);
    std::vector<float2> txy(nt, make_float2(0, 0)), tgw(nt, make_float2(0, 0)), tw(nt, make_float2(0, 0)),
        tnrm(nt, make_float2(0, 1));
    std::vector<uint8_t> tdf(nt, 0);
    std::vector<int> fill(np, 0);
    for (int i = 0; i < n; i++) {
        const float2 on = make_float2((float)nrm[i].x, (float)nrm[i].y);
        for (int j = 0; j < nbh[i]; j++) {
            const size_t e = (size_t)(sb[i >> 5] + 32LL * j + (i & 31));
            const int k = enbr[e];
            const size_t t = (size_t)(tsb[k >> 5] + 32LL * fill[k]++ + (k & 31));
            tsrc[t] = i;
            te[t] = (int)e;
            txy[t] = exy[e];
            tgw[t] = egw[e];
            tw[t] = ew[e];
            tnrm[t] = on;
            tdf[t] = (uint8_t)((edir[e] & 15u) | ((unsigned)flag[i] << 4));
        }
    }
    DeviceArena &A = a->arena;
    long long *d_sb = A.alloc<long long>(ns);
    int *d_nb = A.alloc<int>(np), *d_src = A.alloc<int>(nt), *d_e = A.alloc<int>(nt);
    float2 *d_xy = A.alloc<float2>(nt), *d_gw = A.alloc<float2>(nt), *d_w = A.alloc<float2>(nt),
           *d_nrm = A.alloc<float2>(nt);
    uint8_t *d_df = A.alloc<uint8_t>(nt);
    if (A.err != cudaSuccess)
        return fail(h, QLSKUM_ERR_CUDA, fmt("adjoint transposed edges: %s", cudaGetErrorString(A.err)));
    auto up = [&](void *dst, const void *src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->L.stream);
    };
    CK(h, up(d_sb, tsb.data(), sizeof(long long) * ns));
    CK(h, up(d_nb, tnb.data(), sizeof(int) * np));
    CK(h, up(d_src, tsrc.data(), sizeof(int) * nt));
    CK(h, up(d_e, te.data(), sizeof(int) * nt));
    CK(h, up(d_xy, txy.data(), sizeof(float2) * nt));
    CK(h, up(d_gw, tgw.data(), sizeof(float2) * nt));
    CK(h, up(d_w, tw.data(), sizeof(float2) * nt));
    CK(h, up(d_nrm, tnrm.data(), sizeof(float2) * nt));
    CK(h, up(d_df, tdf.data(), nt));
    CK(h, cudaStreamSynchronize(h->L.stream));
    a->T.sbase = d_sb;
    a->T.nb = d_nb;
    a->T.src = d_src;
    a->T.e = d_e;
    a->T.xy = d_xy;
    a->T.gw = d_gw;
    a->T.w = d_w;
    a->T.nrm = d_nrm;
    a->T.df = d_df;
    return QLSKUM_OK;
}

// The FP32 arrays of one stage-data set (its states are assigned by the caller).
void alloc_set32(DeviceArena &A, size_t np, int ni, Set32 &st)
{
    for (auto &p : st.q32) p = A.alloc<float4>(np);
    for (auto &p : st.qm32) p = A.alloc<float4>(2 * np);
    for (auto &p : st.acc32) p = A.alloc<float4>(np);
    st.dq32.resize(4 * (size_t)(ni + 1));
    for (auto &p : st.dq32) p = A.alloc<float4>(2 * np);
    st.delta32 = A.alloc<float>(np);
    st.cs32 = A.alloc<float>(np);
}

// The FP64 arrays of one stage-data set (its states are assigned by the
// caller); geo: also the directional sums of the wall-gradient reverse.
void alloc_set64(DeviceArena &A, size_t np, size_t ne, int ni, Set64 &st, bool geo)
{
    if (geo)
        for (auto &p : st.sums) p = A.alloc<double>(32 * np);
    for (auto &p : st.ends) p = A.alloc<double>(12 * ne);
    for (auto &p : st.q) p = A.alloc<double4_32a>(np);
    for (auto &p : st.qm) p = A.alloc<double4_32a>(2 * np);
    st.dq.resize(4 * (size_t)(ni + 1));
    for (auto &p : st.dq) p = A.alloc<double4_32a>(2 * np);
    st.delta = A.alloc<double>(np);
    for (auto &p : st.flux) p = A.alloc<double4_32a>(np);
}

size_t set64_bytes(size_t np, size_t ne, int ni, bool geo)
{
    return np * (5 * sizeof(double4_32a) + 4 * 32 + 4 * 64 + 4 * (size_t)(ni + 1) * 64 + 8 + 4 * 32 +
                 (geo ? 4 * 32 * sizeof(double) : 0)) +
           4 * 12 * ne * sizeof(double);
}

// Bytes of one set with its own states.
size_t set32_bytes(size_t np, int ni)
{
    return np * (5 * sizeof(double4_32a) + 4 * 16 + 4 * 32 + 4 * 16 + 4 * (size_t)(ni + 1) * 32 + 8);
}

// The adjoint's buffers: the FP64 stage data (need64), the mixed stage data
// (need32) and the geometry bars (geo), each kept once allocated.
qlskum_status adj_alloc(qlskum_handle *h, bool geo, bool need64, bool need32)
{
    if (h->adj && (h->adj->geo || !geo) && (h->adj->has64 || !need64) && (h->adj->has32 || !need32))
        return QLSKUM_OK;
    if (h->adj) {
        geo |= h->adj->geo;
        need64 |= h->adj->has64;
        need32 |= h->adj->has32;
    }
    adj_free(h);
    AdjBuf *a = new AdjBuf();
    h->adj = a;
    DeviceArena &A = a->arena;
    const size_t np = h->np;
    a->ni = h->prm.inner_iterations;
    a->geo = geo;
    a->has64 = need64;
    a->has32 = need32;
    for (auto &p : a->P) p = A.alloc<double4_32a>(np);
    for (auto *p : {&a->bP, &a->bPacc, &a->bF, &a->lam, &a->lam_prev, &a->seed}) *p = A.alloc<double4_32a>(np);
    a->buinf = A.alloc<double>(4);  // free-stream velocity bars, then the initial-state sums
    slice_bases(h, &a->ne);
    if (need64) {
        alloc_set64(A, np, a->ne, a->ni, a->set64, geo);
        for (int k = 0; k < 5; k++) a->set64.P[k] = a->P[k];
        a->bq = A.alloc<double4_32a>(np);
        for (auto *p : {&a->bdqA, &a->bdqB, &a->bqm}) *p = A.alloc<double4_32a>(2 * np);
        a->bdelta = A.alloc<double>(np);
        a->bc = A.alloc<double>(np);
    }
    if (need32) {
        alloc_set32(A, np, a->ni, a->set0);
        for (int k = 0; k < 5; k++) a->set0.P[k] = a->P[k];
        a->bq32 = A.alloc<float4>(np);
        a->bF32 = A.alloc<float4>(np);
        a->bs32 = A.alloc<float4>(np);
        for (auto *p : {&a->bdqA32, &a->bdqB32, &a->bdq0_32, &a->bqm32}) *p = A.alloc<float4>(2 * np);
        a->bdelta32 = A.alloc<float>(np);
        a->bcs32 = A.alloc<float>(np);
    }
    if (geo) {
        a->bedge = A.alloc<double4_32a>(a->ne);
        a->bdist = A.alloc<double>(a->ne);
        a->bnrm = A.alloc<double2>(np);
        a->bgmom = A.alloc<double4_32a>(np);
        a->gbx = A.alloc<double>(np);
        a->gby = A.alloc<double>(np);
        a->gbn = A.alloc<double2>(np);
        a->bfmom = A.alloc<double4_32a>(4 * np);
        a->geo_pt = A.alloc<uint8_t>(np);
    }
    if (A.err != cudaSuccess) {
        qlskum_status st = fail(h, QLSKUM_ERR_CUDA, fmt("adjoint cudaMalloc: %s", cudaGetErrorString(A.err)));
        adj_free(h);
        return st;
    }
    // padding rows stay zero (and finite) in every buffer
    for (auto *p : a->P) zero(h, p, sizeof(double4_32a) * np);
    if (geo) {
        // the points whose geometry depends on a wall point, marked on the
        // device and listed on the host
        adjl::mark_geo_points(h->L, h->dc, a->geo_pt);
        std::vector<uint8_t> mark(h->n);
        CK(h, cudaMemcpyAsync(mark.data(), a->geo_pt, h->n, cudaMemcpyDeviceToHost, h->L.stream));
        CK(h, cudaStreamSynchronize(h->L.stream));
        std::vector<int> list;
        for (int i = 0; i < h->n; i++)
            if (mark[i]) list.push_back(i);
        a->n_geo = (int)list.size();
        a->geo_list = a->arena.alloc<int>(std::max<size_t>(list.size(), 1));
        if (a->arena.err != cudaSuccess) {
            qlskum_status st = fail(h, QLSKUM_ERR_CUDA, fmt("adjoint cudaMalloc: %s", cudaGetErrorString(a->arena.err)));
            adj_free(h);
            return st;
        }
        if (!list.empty())
            CK(h, cudaMemcpyAsync(a->geo_list, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice,
                                  h->L.stream));
        CK(h, cudaStreamSynchronize(h->L.stream));
    }
    if (need32) {
        qlskum_status st = adj_transpose(h);
        if (st) adj_free(h);
        return st;
    }
    return QLSKUM_OK;
}

AdjView adj_view(qlskum_handle *h, bool geo)
{
    AdjView v;
    v.c = h->dc;
    AdjBuf *a = h->adj;
    if (geo && a->geo) {
        v.geo_pt = a->geo_pt;
        v.geo_list = a->geo_list;
        v.n_geo = a->n_geo;
        v.bedge = a->bedge;
        v.bdist = a->bdist;
        v.bnrm = a->bnrm;
        v.bgmom = a->bgmom;
        v.bfmom = a->bfmom;
    }
    return v;
}

void adj_zero_geometry(qlskum_handle *h)
{
    AdjBuf *a = h->adj;
    zero(h, a->buinf, 2 * sizeof(double));
    if (!a->geo) return;
    const size_t np = h->np;
    zero(h, a->bedge, sizeof(double4_32a) * a->ne);
    zero(h, a->bdist, sizeof(double) * a->ne);
    zero(h, a->bnrm, sizeof(double2) * np);
    zero(h, a->bgmom, sizeof(double4_32a) * np);
    zero(h, a->bfmom, sizeof(double4_32a) * 4 * np);
}

double4_32a *adj_dq(const Set64 &st, int ni, int s, int j) { return st.dq[(size_t)s * (ni + 1) + j]; }

// Stage s (0-based) from st.P[s]: q, the gradient and its inner-loop
// corrections, the neighbour max / min and the flux residual (into
// st.flux[s]) (fpi_solver_mod.h:20-36).
void adj_stage_forward(qlskum_handle *h, Set64 &st, int s)
{
    const int ni = h->adj->ni;
    const DevCloud &c = h->dc;
    fp64::q_variables(h->L, c, st.P[s], st.q[s]);
    fp64::q_derivatives(h->L, c, st.q[s], adj_dq(st, ni, s, 0), st.qm[s], nullptr, nullptr, 0.0);
    for (int j = 1; j <= ni; j++) fp64::q_inner(h->L, c, st.q[s], adj_dq(st, ni, s, j - 1), adj_dq(st, ni, s, j));
    fp64::flux_residual(h->L, c, st.q[s], adj_dq(st, ni, s, ni), st.qm[s], st.delta, st.flux[s], st.sums[s],
                        st.ends[s], (long long)h->adj->ne);
}

// The four stage states of one iteration from st.P[0] (fpi_solver_mod.h:14-40)
// with the module kernels, whose results equal the fused solver's bit for
// bit.  it_rec > 0: the iteration is the primal's own iteration it_rec (its
// residual row is reduced and recorded, as qlskum_fpi_solver does).
void adj_iteration_forward64(qlskum_handle *h, Set64 &st, int it_rec = 0)
{
    fp64::func_delta(h->L, h->dc, st.P[0], st.delta, h->K.cfl);
    for (int s = 0; s < 4; s++) {
        adj_stage_forward(h, st, s);
        fp64::copy_prim(h->L, h->n, st.P[s], st.P[s + 1]);
        fp64::state_update(h->L, h->dc, h->K, st.P[s + 1], st.P[0], st.flux[s], s + 1, h->R);
    }
    if (it_rec > 0) {
        Reduce R = h->R;
        R.blocks = (h->n + 127) / 128;
        fp64::reduce_residual(h->L, R, h->n, it_rec);
    }
}

// Reverse of stage s's residual chain for the bar in a->bF: adds to a->bP
// (the bar of P[s]) and to a->bdelta.
void adj_stage_reverse(qlskum_handle *h, const Set64 &st, int s, const AdjView &v)
{
    AdjBuf *a = h->adj;
    const size_t np = h->np;
    const int ni = a->ni;
    zero(h, a->bq, sizeof(double4_32a) * np);
    zero(h, a->bdqA, sizeof(double4_32a) * 2 * np);
    zero(h, a->bqm, sizeof(double4_32a) * 2 * np);
    adjl::flux(h->L, v, st.q[s], adj_dq(st, ni, s, ni), st.qm[s], st.delta, st.flux[s], st.sums[s], st.ends[s],
               (long long)a->ne, a->bF, a->bq,
               a->bdqA, a->bqm, a->bdelta);
    for (int j = ni; j >= 1; j--) {
        zero(h, a->bdqB, sizeof(double4_32a) * 2 * np);
        adjl::inner(h->L, v, st.q[s], adj_dq(st, ni, s, j - 1), a->bdqA, a->bq, a->bdqB);
        std::swap(a->bdqA, a->bdqB);
    }
    adjl::grad(h->L, v, st.q[s], a->bdqA, a->bqm, a->bq);
    adjl::qvars(h->L, h->n, st.P[s], a->bq, a->bP);
}

// Reverse of one iteration after adj_iteration_forward64: a->bP holds the
// bar of P[4] on entry and the bar of P[0] on exit.  Free-stream bars add to
// a->buinf, geometry bars to the view's accumulators.
void adj_iteration_reverse64(qlskum_handle *h, const Set64 &st, const AdjView &v)
{
    AdjBuf *a = h->adj;
    const size_t np = h->np;
    zero(h, a->bPacc, sizeof(double4_32a) * np);
    zero(h, a->bdelta, sizeof(double) * np);
    for (int s = 3; s >= 0; s--) {
        adjl::update(h->L, v, h->K, st.P[s], st.P[0], st.P[s + 1], s + 1, a->bP, a->bPacc, a->bF, a->buinf);
        adj_stage_reverse(h, st, s, v);
    }
    zero(h, a->bc, sizeof(double) * np);
    adjl::delta(h->L, v, st.P[0], a->bdelta, h->K.cfl, a->bc, a->bPacc);
    fp64::add_prim(h->L, h->n, a->bPacc, a->bP);
}

float4 *adj_dq32(const Set32 &st, int ni, int s, int j) { return st.dq32[(size_t)s * (ni + 1) + j]; }

// `count` stage-data sets with their own states (FP64 or FP32 kind; first
// use, growth and change of kind only); false when they do not fit.
bool adj_sets(qlskum_handle *h, int count, bool f64)
{
    AdjBuf *a = h->adj;
    const bool geo = f64 && a->geo;
    if ((f64 ? (int)a->sets64.size() : (int)a->sets.size()) >= count && (!geo || a->sets_geo)) return true;
    auto drop = [&]() {
        a->sets.clear();
        a->sets64.clear();
        a->set_arena.release();
        a->set_arena.err = cudaSuccess;
    };
    drop();
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return false;
    // keep a quarter of the free memory for everything else
    const size_t each = f64 ? set64_bytes(h->np, a->ne, a->ni, geo) : set32_bytes(h->np, a->ni);
    if ((double)each * count > 0.75 * (double)free_b) return false;
    std::vector<double4_32a *> p0;
    if (f64) {
        a->sets64.resize(count);
        for (auto &st : a->sets64) {
            alloc_set64(a->set_arena, h->np, a->ne, a->ni, st, geo);
            for (auto &p : st.P) p = a->set_arena.alloc<double4_32a>(h->np);
            p0.push_back(st.P[0]);
        }
    } else {
        a->sets.resize(count);
        for (auto &st : a->sets) {
            alloc_set32(a->set_arena, h->np, a->ni, st);
            for (auto &p : st.P) p = a->set_arena.alloc<double4_32a>(h->np);
            p0.push_back(st.P[0]);
        }
    }
    if (a->set_arena.err != cudaSuccess) {
        cudaGetLastError();
        drop();
        return false;
    }
    for (auto *p : p0) zero(h, p, sizeof(double4_32a) * h->np);
    a->sets_geo = geo;
    return true;
}

// The mixed iteration from st.P[0] with the solver's own kernels and launch
// shapes (enqueue_iteration), every stage's FP32 data kept in `st`: q, the
// gradient after each inner step, max / min, the flux kernel's weighted
// sums, the local time step and the wave speed it came from.  it_rec > 0:
// the iteration is the primal's own iteration it_rec (its residual row is
// reduced and recorded, as qlskum_fpi_solver does).
void adj_iteration_forward32(qlskum_handle *h, Set32 &st, int it_rec = 0)
{
    AdjBuf *a = h->adj;
    const DevCloud &c = h->dc;
    const int ni = a->ni;
    Reduce none = h->R;
    none.partial_sum = none.partial_max = nullptr;
    mixed::derived(h->L, c, st.P[0], st.q32[0], st.cs32);
    for (int s = 0; s < 4; s++) {
        mixed::q_derivatives(h->L, c, st.q32[s], adj_dq32(st, ni, s, 0), st.qm32[s], st.cs32,
                             s == 0 ? st.delta32 : nullptr, (float)h->K.cfl);
        for (int j = 1; j <= ni; j++)
            mixed::q_inner(h->L, c, adj_dq32(st, ni, s, 0), adj_dq32(st, ni, s, j - 1), adj_dq32(st, ni, s, j));
        // the last stage's q goes to the bar buffer, which the reverse overwrites
        float4 *q_next = s < 3 ? st.q32[s + 1] : a->bq32;
        mixed::flux_update(h->L, c, h->K, st.q32[s], adj_dq32(st, ni, s, ni), st.qm32[s], st.delta32, st.P[s],
                           st.P[0], st.P[s + 1], q_next, nullptr, s + 1, (it_rec > 0 && s == 3) ? h->R : none,
                           h->flux_variant, st.acc32[s]);
    }
    if (it_rec > 0) {
        Reduce R = h->R;
        R.blocks = mixed::flux_grid_blocks(h->flux_variant, h->n);
        fp64::reduce_residual(h->L, R, h->n, it_rec);
    }
}

// Reverse of adj_iteration_forward32 for the stage data in `st` (same
// contract as the FP64 reverse, without geometry bars).
void adj_iteration_reverse32(qlskum_handle *h, const Set32 &st)
{
    AdjBuf *a = h->adj;
    const size_t np = h->np;
    const int ni = a->ni;
    const DevCloud &c = h->dc;
    zero(h, a->bPacc, sizeof(double4_32a) * np);
    zero(h, a->bdelta32, sizeof(float) * np);
    for (int s = 3; s >= 0; s--) {
        adjml::update(h->L, c, h->K, st.P[s], st.P[0], st.P[s + 1], s + 1, st.delta32, a->bP, a->bPacc, a->bF32,
                      a->bs32, a->buinf);
        // the flux reverse stores every point's bars of q, dq and qm first
        adjml::flux(h->L, c, a->T, st.q32[s], adj_dq32(st, ni, s, ni), st.qm32[s], st.acc32[s], a->bF32, a->bs32,
                    a->bq32, a->bdqA32, a->bqm32, a->bdelta32);
        for (int j = ni; j >= 1; j--) {
            adjml::inner(h->L, c, a->T, a->bdqA32, a->bdqB32, a->bdq0_32, j == ni);
            std::swap(a->bdqA32, a->bdqB32);
        }
        adjml::grad(h->L, c, st.q32[s], a->bdqA32, ni > 0 ? a->bdq0_32 : nullptr, a->bqm32, a->bq32);
        adjml::qvars(h->L, h->n, st.P[s], a->bq32, a->bP);
    }
    zero(h, a->bcs32, sizeof(float) * np);
    adjml::delta(h->L, c, st.P[0], st.cs32, a->bdelta32, (float)h->K.cfl, a->bcs32, a->bPacc);
    fp64::add_prim(h->L, h->n, a->bPacc, a->bP);
}

// The reverse of a mixed handle's own iteration where no geometry bars are
// wanted, else the FP64 reverse.
bool adj_use32(const qlskum_handle *h, bool geo) { return h->prm.precision == QLSKUM_MIXED && !geo; }

void adj_iteration_forward(qlskum_handle *h, bool m32)
{
    if (m32) adj_iteration_forward32(h, h->adj->set0);
    else adj_iteration_forward64(h, h->adj->set64);
}

void adj_iteration_reverse(qlskum_handle *h, const AdjView &v, bool m32)
{
    if (m32) adj_iteration_reverse32(h, h->adj->set0);
    else adj_iteration_reverse64(h, h->adj->set64, v);
}

// Cl and Cd at `prim` (compute_force_coeffs_mod.h:37-67), and dJ/dprim of
// objective `which` (0 Cl, 1 Cd) into `bP`.
// The objective's value and its explicit dependence on Mach and AoA (the
// part not carried by the state).
struct ObjSeed {
    double J = 0.0, dM = 0.0, dth = 0.0;
};

// J at `prim` and dJ/dprim into bP: Cl / Cd (compute_force_coeffs_mod.h:37-67;
// c_p scales with 1 / M^2 and the axes rotate with theta: dCl/dtheta = -Cd,
// dCd/dtheta = Cl) or the stagnation-pressure loss (its p0_inf depends on M).
qlskum_status adj_seed(qlskum_handle *h, int which, const double4_32a *prim, double4_32a *bP, ObjSeed &o)
{
    zero(h, bP, sizeof(double4_32a) * h->np);
    qlskum_status st;
    if (which == QLSKUM_OBJECTIVE_J) {
        Stagnation sv;
        if ((st = stagnation_values(h, prim, sv))) return st;
        adjl::objective_J(h->L, h->n, prim, h->K.gamma, sv.p0_inf, bP);
        if ((st = check_launch(h, "adjoint seed"))) return st;
        const double n = (double)h->n, g = h->K.gamma, M = h->K.mach, gp = g / (g - 1);
        const double dJ_dp0inf = 2.0 * (n * sv.p0_inf - sv.sum_p0) / (sv.p0_inf * sv.p0_inf * n) -
                                 2.0 * sv.sum_sq / (sv.p0_inf * sv.p0_inf * sv.p0_inf * n);
        const double dp0inf_dM = h->K.pr_inf * gp * std::pow(1 + 0.5 * (g - 1) * M * M, gp - 1) * (g - 1) * M;
        o.J = sv.J;
        o.dM = dJ_dp0inf * dp0inf_dM;
        o.dth = 0.0;
        return QLSKUM_OK;
    }
    const double cp_scale = 0.5 * h->K.rho_inf * h->K.mach * h->K.mach;
    fp64::objective(h->L, h->dc, prim, h->d_wall_perm, h->d_wall_geo, h->shape_points, cp_scale, h->K.pr_inf,
                    h->K.gamma, nullptr, h->d_obj, h->d_obj_partial);
    adjl::objective(h->L, adj_view(h, false), h->d_wall_perm, h->d_wall_geo, h->shape_points, cp_scale, h->K.theta,
                    which, bP);
    if ((st = check_launch(h, "adjoint seed"))) return st;
    double v[4];
    if ((st = d2h(h, v, h->d_obj, sizeof v))) return st;
    const double cl = v[1] * std::cos(h->K.theta) - v[0] * std::sin(h->K.theta);
    const double cd = v[0] * std::cos(h->K.theta) + v[1] * std::sin(h->K.theta);
    o.J = which == QLSKUM_OBJECTIVE_CL ? cl : cd;
    o.dM = -2.0 * o.J / h->K.mach;
    o.dth = which == QLSKUM_OBJECTIVE_CL ? -cd : cl;
    return QLSKUM_OK;
}

// dJ/dMach and dJ/dAoA (per degree).  The free stream (u1, u2) =
// M (cos theta, sin theta) enters through the far-field states (bars in
// buinf) and, for a run from the free stream, the initial state (bars in
// binit); plus the objective's explicit terms.
void adj_params(const qlskum_handle *h, const ObjSeed &o, const double buinf[2], const double binit[2],
                double *dmach, double *daoa)
{
    const double th = h->K.theta, M = h->K.mach;
    const double b1 = buinf[0] + binit[0], b2 = buinf[1] + binit[1];
    const double dM = o.dM + b1 * std::cos(th) + b2 * std::sin(th);
    const double dth = M * (-b1 * std::sin(th) + b2 * std::cos(th)) + o.dth;
    if (dmach) *dmach = dM;
    if (daoa) *daoa = dth * h->K.pi / 180.0;
}

// Reverse of the geometry (host, FP64).  The accumulated adjoints of the edge
// vectors, rotated edge vectors, edge lengths, normals and least-squares
// moments, and the objective's own geometry (panel lengths, normals), are
// pulled back to the point coordinates, then projected on the unperturbed
// wall normals of the shape points: x_m(s) = x_m + s n_m.  Unit weights
// (power 0); the sub-stencil split and min_dist (the limiter's epsilon) are
// held at their unperturbed values.
qlskum_status adj_geometry(qlskum_handle *h, int which, const double4_32a *prim_dev, double *dJ_dwall)
{
    AdjBuf *a = h->adj;
    const int n = h->n;
    const size_t np = h->np;
    const std::vector<double> &X = h->hx, &Y = h->hy;
    // the edge and moment bars to coordinate bars on the device
    zero(h, a->gbx, sizeof(double) * np);
    zero(h, a->gby, sizeof(double) * np);
    adjl::geom_pullback(h->L, adj_view(h, true), a->gbx, a->gby, a->gbn);
    qlskum_status st;
    if ((st = check_launch(h, "geometry pull-back"))) return st;
    std::vector<double> gx(np), gy(np);
    std::vector<double2> gn(np);
    std::vector<double4_32a> prim(np);
    if ((st = d2h(h, gx.data(), a->gbx, sizeof(double) * np))) return st;
    if ((st = d2h(h, gy.data(), a->gby, sizeof(double) * np))) return st;
    if ((st = d2h(h, gn.data(), a->gbn, sizeof(double2) * np))) return st;
    if ((st = d2h(h, prim.data(), prim_dev, sizeof(double4_32a) * np))) return st;
    // in the cloud's order
    std::vector<double> bx(n), by(n), bnx(n), bny(n);
    for (int i = 0; i < n; i++) {
        const int pp = h->perm[i];
        bx[i] = gx[pp];
        by[i] = gy[pp];
        bnx[i] = gn[pp].x;
        bny[i] = gn[pp].y;
    }
    // the objective's geometry: H = sum cp nx ds, V = sum cp ny ds with
    // ds = (|x_m - x_l| + |x_r - x_m|) / 2 (compute_force_coeffs_mod.h:37-59);
    // the stagnation-pressure loss has none, nor has a residual VJP (which < 0)
    const double cp_scale = 0.5 * h->K.rho_inf * h->K.mach * h->K.mach;
    const double th = h->K.theta;
    const double bH = which == 0 ? -std::sin(th) : std::cos(th);
    const double bV = which == 0 ? std::cos(th) : std::sin(th);
    for (int m = 0; m < ((which < 0 || which == QLSKUM_OBJECTIVE_J) ? 0 : h->shape_points); m++) {
        const int l = h->hleft[m] - 1, r = h->hright[m] - 1;
        const double cp = -(prim[h->perm[m]].w - h->K.pr_inf) / cp_scale;
        const double d1x = X[m] - X[l], d1y = Y[m] - Y[l], d2x = X[r] - X[m], d2y = Y[r] - Y[m];
        const double ds1 = std::sqrt(d1x * d1x + d1y * d1y), ds2 = std::sqrt(d2x * d2x + d2y * d2y);
        const double dsm = 0.5 * (ds1 + ds2);
        bnx[m] += bH * cp * dsm;
        bny[m] += bV * cp * dsm;
        const double bds = cp * (bH * h->pc.nx[m] + bV * h->pc.ny[m]);
        bx[m] += 0.5 * bds * (d1x / ds1 - d2x / ds2);
        by[m] += 0.5 * bds * (d1y / ds1 - d2y / ds2);
        bx[l] -= 0.5 * bds * d1x / ds1;
        by[l] -= 0.5 * bds * d1y / ds1;
        bx[r] += 0.5 * bds * d2x / ds2;
        by[r] += 0.5 * bds * d2y / ds2;
    }
    // normals of wall and outer points: n = (-a, b) / |(a, b)| with
    // a = (y_r - y_l) / 2, b = (x_r - x_l) / 2 (point_normals_mod.h:17-46)
    for (int i = 0; i < n; i++) {
        if (h->hflag[i] == kInterior || (bnx[i] == 0.0 && bny[i] == 0.0)) continue;
        const int l = h->hleft[i] - 1, r = h->hright[i] - 1;
        const double av = 0.5 * (Y[r] - Y[l]), bv = 0.5 * (X[r] - X[l]);
        const double det = std::sqrt(av * av + bv * bv);
        const double bdet = (bnx[i] * av - bny[i] * bv) / (det * det);
        const double ba = -bnx[i] / det + bdet * av / det;
        const double bb = bny[i] / det + bdet * bv / det;
        by[r] += 0.5 * ba;
        by[l] -= 0.5 * ba;
        bx[r] += 0.5 * bb;
        bx[l] -= 0.5 * bb;
    }
    for (int m = 0; m < h->shape_points; m++) dJ_dwall[m] = bx[m] * h->pc.nx[m] + by[m] * h->pc.ny[m];
    return QLSKUM_OK;
}

qlskum_status upload_points(qlskum_handle *h, const double *src, double4_32a *dst, double pad)
{
    std::vector<double4_32a> dev(h->np, make_double4_32a(pad, 0, 0, pad));
    for (int i = 0; i < h->n; i++)
        dev[h->perm[i]] = make_double4_32a(src[4 * (size_t)i], src[4 * (size_t)i + 1], src[4 * (size_t)i + 2],
                                           src[4 * (size_t)i + 3]);
    CK(h, cudaMemcpyAsync(dst, dev.data(), sizeof(double4_32a) * h->np, cudaMemcpyHostToDevice, h->L.stream));
    CK(h, cudaStreamSynchronize(h->L.stream));
    return QLSKUM_OK;
}

qlskum_status download_points(qlskum_handle *h, const double4_32a *src, double *dst)
{
    std::vector<double4_32a> dev(h->np);
    qlskum_status st = d2h(h, dev.data(), src, sizeof(double4_32a) * h->np);
    if (st) return st;
    for (int i = 0; i < h->n; i++) std::memcpy(dst + 4 * (size_t)i, &dev[h->perm[i]], sizeof(double4_32a));
    return QLSKUM_OK;
}

qlskum_status adj_args(qlskum_handle *h, int objective, int count, const double *dJ_dwall)
{
    if (objective != QLSKUM_OBJECTIVE_CL && objective != QLSKUM_OBJECTIVE_CD && objective != QLSKUM_OBJECTIVE_J)
        return fail(h, QLSKUM_ERR_INVALID, fmt("unknown objective %d", objective));
    if (count < 1) return fail(h, QLSKUM_ERR_INVALID, "iteration count must be >= 1");
    if (dJ_dwall && h->prm.power != 0.0)
        return fail(h, QLSKUM_ERR_UNSUPPORTED, "wall-displacement gradients need unit least-squares weights (power 0)");
    const bool geo = dJ_dwall != nullptr;
    return adj_alloc(h, geo, !adj_use32(h, geo), adj_use32(h, geo));
}

}  // namespace

extern "C" {

qlskum_status qlskum_residual_forward(qlskum_handle *h, const double *prim, double *flux_res)
{
    NEED(h);
    if (!prim || !flux_res) return fail(h, QLSKUM_ERR_INVALID, "null prim or flux_res");
    qlskum_status st = adj_alloc(h, false, true, false);
    if (st) return st;
    AdjBuf *a = h->adj;
    if ((st = upload_points(h, prim, a->P[0], 1.0))) return st;
    fp64::func_delta(h->L, h->dc, a->P[0], a->set64.delta, h->K.cfl);
    adj_stage_forward(h, a->set64, 0);
    if ((st = check_launch(h, "residual_forward"))) return st;
    return download_points(h, a->set64.flux[0], flux_res);
}

qlskum_status qlskum_residual_vjp(qlskum_handle *h, const double *prim, const double *bar_flux_res, double *bar_prim)
{
    NEED(h);
    if (!prim || !bar_flux_res || !bar_prim) return fail(h, QLSKUM_ERR_INVALID, "null argument");
    qlskum_status st = adj_alloc(h, false, true, false);
    if (st) return st;
    AdjBuf *a = h->adj;
    if ((st = upload_points(h, prim, a->P[0], 1.0))) return st;
    if ((st = upload_points(h, bar_flux_res, a->bF, 0.0))) return st;
    fp64::func_delta(h->L, h->dc, a->P[0], a->set64.delta, h->K.cfl);
    adj_stage_forward(h, a->set64, 0);
    const AdjView v = adj_view(h, false);
    zero(h, a->bP, sizeof(double4_32a) * h->np);
    zero(h, a->bdelta, sizeof(double) * h->np);
    adj_stage_reverse(h, a->set64, 0, v);
    zero(h, a->bc, sizeof(double) * h->np);
    adjl::delta(h->L, v, a->P[0], a->bdelta, h->K.cfl, a->bc, a->bP);
    if ((st = check_launch(h, "residual_vjp"))) return st;
    return download_points(h, a->bP, bar_prim);
}

// The forward / VJP pair on device buffers in the cloud's point order, ordered
// after the caller's stream (an event it records, which the handle's stream
// waits for) and before the caller's later work (the reverse).
namespace {

qlskum_status dev_args(qlskum_handle *h, std::initializer_list<const void *> ptrs)
{
    for (const void *p : ptrs) {
        if (!p) return fail(h, QLSKUM_ERR_INVALID, "null device buffer");
        if (reinterpret_cast<uintptr_t>(p) & 31u) return fail(h, QLSKUM_ERR_INVALID, "device buffers must be 32-byte aligned");
    }
    return ensure_stage(h);
}

void wait_on(qlskum_handle *h, cudaStream_t waiter, cudaStream_t on)
{
    cudaEvent_t e = take_event(h);
    cudaEventRecord(e, on);
    cudaStreamWaitEvent(waiter, e, 0);
    h->ev_pool.push_back(e);
}

}  // namespace

qlskum_status qlskum_residual_forward_device(qlskum_handle *h, const double *prim, double *flux_res, void *stream)
{
    NEED(h);
    qlskum_status st = dev_args(h, {prim, flux_res});
    if (st) return st;
    if ((st = adj_alloc(h, false, true, false))) return st;
    AdjBuf *a = h->adj;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    wait_on(h, h->L.stream, cs);
    fp64::fill_prim(h->L, h->np, make_double4_32a(1.0, 0, 0, 1.0), a->P[0]);
    fp64::permute_in(h->L, h->n, h->d_perm, reinterpret_cast<const double4_32a *>(prim), a->P[0]);
    fp64::func_delta(h->L, h->dc, a->P[0], a->set64.delta, h->K.cfl);
    adj_stage_forward(h, a->set64, 0);
    fp64::permute_out(h->L, h->n, h->d_perm, a->set64.flux[0], reinterpret_cast<double4_32a *>(flux_res));
    wait_on(h, cs, h->L.stream);
    return check_launch(h, "residual_forward_device");
}

qlskum_status qlskum_residual_vjp_device(qlskum_handle *h, const double *prim, const double *bar_flux_res,
                                         double *bar_prim, void *stream)
{
    NEED(h);
    qlskum_status st = dev_args(h, {prim, bar_flux_res, bar_prim});
    if (st) return st;
    if ((st = adj_alloc(h, false, true, false))) return st;
    AdjBuf *a = h->adj;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    wait_on(h, h->L.stream, cs);
    fp64::fill_prim(h->L, h->np, make_double4_32a(1.0, 0, 0, 1.0), a->P[0]);
    fp64::permute_in(h->L, h->n, h->d_perm, reinterpret_cast<const double4_32a *>(prim), a->P[0]);
    zero(h, a->bF, sizeof(double4_32a) * h->np);
    fp64::permute_in(h->L, h->n, h->d_perm, reinterpret_cast<const double4_32a *>(bar_flux_res), a->bF);
    fp64::func_delta(h->L, h->dc, a->P[0], a->set64.delta, h->K.cfl);
    adj_stage_forward(h, a->set64, 0);
    const AdjView v = adj_view(h, false);
    zero(h, a->bP, sizeof(double4_32a) * h->np);
    zero(h, a->bdelta, sizeof(double) * h->np);
    adj_stage_reverse(h, a->set64, 0, v);
    zero(h, a->bc, sizeof(double) * h->np);
    adjl::delta(h->L, v, a->P[0], a->bdelta, h->K.cfl, a->bc, a->bP);
    fp64::permute_out(h->L, h->n, h->d_perm, a->bP, reinterpret_cast<double4_32a *>(bar_prim));
    wait_on(h, cs, h->L.stream);
    return check_launch(h, "residual_vjp_device");
}

qlskum_status qlskum_residual_vjp_full(qlskum_handle *h, const double *prim, const double *bar_flux_res,
                                      double *bar_prim, double *bar_params, double *bar_wall_disp)
{
    NEED(h);
    if (!prim || !bar_flux_res || !bar_prim) return fail(h, QLSKUM_ERR_INVALID, "null argument");
    if (bar_wall_disp && h->prm.power != 0.0)
        return fail(h, QLSKUM_ERR_UNSUPPORTED, "wall-displacement gradients need unit least-squares weights (power 0)");
    const bool geo = bar_wall_disp != nullptr;
    qlskum_status st = adj_alloc(h, geo, true, false);
    if (st) return st;
    AdjBuf *a = h->adj;
    if ((st = upload_points(h, prim, a->P[0], 1.0))) return st;
    if ((st = upload_points(h, bar_flux_res, a->bF, 0.0))) return st;
    fp64::func_delta(h->L, h->dc, a->P[0], a->set64.delta, h->K.cfl);
    adj_stage_forward(h, a->set64, 0);
    adj_zero_geometry(h);
    const AdjView v = adj_view(h, geo);
    zero(h, a->bP, sizeof(double4_32a) * h->np);
    zero(h, a->bdelta, sizeof(double) * h->np);
    adj_stage_reverse(h, a->set64, 0, v);
    zero(h, a->bc, sizeof(double) * h->np);
    adjl::delta(h->L, v, a->P[0], a->bdelta, h->K.cfl, a->bc, a->bP);
    if ((st = check_launch(h, "residual_vjp_full"))) return st;
    if ((st = download_points(h, a->bP, bar_prim))) return st;
    // R(prim) is the flux residual of one stage and its time step: neither
    // reads the free stream, which enters through the stage update
    if (bar_params) bar_params[0] = bar_params[1] = 0.0;
    if (geo) return adj_geometry(h, -1, a->P[0], bar_wall_disp);
    return QLSKUM_OK;
}

qlskum_status qlskum_adjoint_gradient(qlskum_handle *h, int objective, int iters, const double *prim0, double *J,
                                      double *dJ_dmach, double *dJ_daoa, double *dJ_dwall, double *dJ_dprim0)
{
    NEED(h);
    qlskum_status st = adj_args(h, objective, iters, dJ_dwall);
    if (st) return st;
    AdjBuf *a = h->adj;
    const size_t np = h->np;
    const bool m32 = adj_use32(h, dJ_dwall != nullptr);
    const int S = std::max(1, h->adj_stride);
    const int nck = (iters + S - 1) / S;
    // mixed handles keep each iteration's stage data in its own set where the
    // sets fit: with stride 1 all `iters` of them (the primal then runs as the
    // recording iteration and nothing is recomputed), with a larger stride one
    // segment's (each segment recomputed once); otherwise set 0 is refilled
    // for every iteration of the reverse sweep
    // (FP64 handles the same with FP64 stage data; a mixed handle's FP64 reverse
    // for wall gradients keeps the fused mixed primal and recomputes in FP64)
    const bool f64h = h->prm.precision == QLSKUM_FP64;
    const bool store_all = S == 1 && (m32 || f64h) && adj_sets(h, iters, !m32);
    const bool seg_sets = !store_all && S > 1 && adj_sets(h, S, !m32);
    auto set_P = [&](int t, int k) { return m32 ? a->sets[t].P[k] : a->sets64[t].P[k]; };
    auto fwd_set = [&](int t, int it_rec) {
        if (m32) adj_iteration_forward32(h, a->sets[t], it_rec);
        else adj_iteration_forward64(h, a->sets64[t], it_rec);
    };
    auto grow = [&](double4_32a *&buf, int &cap, int want, const char *what) -> qlskum_status {
        if (cap >= want) return QLSKUM_OK;
        if (buf) cudaFree(buf);
        buf = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&buf, sizeof(double4_32a) * np * (size_t)want);
        if (e != cudaSuccess)
            return fail(h, QLSKUM_ERR_CUDA, fmt("%s: %d states (%.1f GB): %s", what, want,
                                                1e-9 * sizeof(double4_32a) * np * want, cudaGetErrorString(e)));
        cap = want;
        return QLSKUM_OK;
    };
    if (!store_all && (st = grow(a->ckpt, a->ckpt_cap, nck, "adjoint checkpoints"))) return st;
    if (S > 1 && !seg_sets && (st = grow(a->seg, a->seg_cap, S, "adjoint segment"))) return st;
    // primal from prim0 or the free stream (initial_conditions_mod.h:23-37),
    // every S-th iteration's starting state kept
    if (prim0) {
        // the caller's [n][4] state reordered on the device (qlskum_set_prim's path)
        if ((st = qlskum_set_prim(h, prim0))) return st;
    } else {
        fp64::fill_prim(h->L, (int)np, make_double4_32a(h->K.rho_inf, h->K.u1_inf, h->K.u2_inf, h->K.pr_inf),
                        h->s64.prim[h->pcur]);
    }
    CK(h, cudaMemsetAsync(h->R.status, 0, sizeof(int), h->L.stream));
    h->derived_valid = false;
    h->it = 0;
    const size_t bytes = sizeof(double4_32a) * np;
    if (store_all) {
        // the primal's iterations as the recording iteration (the same kernels,
        // launch shapes and residual rows as qlskum_fpi_solver), each into its set
        if ((st = ensure_hist(h, iters))) return st;
        if ((st = ensure_derived(h))) return st;
        const int o = h->pcur;
        for (int t = 0; t < iters; t++) {
            const double4_32a *from = t == 0 ? h->s64.prim[o] : set_P(t - 1, 4);
            CK(h, cudaMemcpyAsync(set_P(t, 0), from, bytes, cudaMemcpyDeviceToDevice, h->L.stream));
            fwd_set(t, t + 1);
        }
        // the handle as after qlskum_q_lskum(iters): state and prim_old of the last iteration
        CK(h, cudaMemcpyAsync(h->s64.prim[o], set_P(iters - 1, 0), bytes, cudaMemcpyDeviceToDevice, h->L.stream));
        CK(h, cudaMemcpyAsync(h->s64.prim[(o + 2) % 3], set_P(iters - 1, 4), bytes, cudaMemcpyDeviceToDevice,
                              h->L.stream));
        after_iteration(h, o);
        h->derived_valid = false;
        h->it = iters;
        if ((st = check_launch(h, "adjoint primal"))) return st;
        if (h->prm.verbose && (st = print_iters(h, 0, iters))) return st;
    } else {
        for (int t = 0; t < iters; t++) {
            if (t % S == 0)
                CK(h, cudaMemcpyAsync(a->ckpt + np * (size_t)(t / S), h->s64.prim[h->pcur], bytes,
                                      cudaMemcpyDeviceToDevice, h->L.stream));
            if ((st = qlskum_fpi_solver(h, t + 1))) return st;
        }
    }
    if ((st = check_status(h))) return st;
    ObjSeed os;
    if ((st = adj_seed(h, objective, h->s64.prim[h->pcur], a->bP, os))) return st;
    adj_zero_geometry(h);
    // geometry bars only when this call asks for the wall gradient (the
    // buffers may exist from an earlier call)
    const AdjView v = adj_view(h, dJ_dwall != nullptr);
    for (int c0 = store_all ? -1 : nck - 1; c0 >= 0; c0--) {
        const int t0 = c0 * S, t1 = std::min(iters, t0 + S);
        // states t0 .. t1 - 1 of this segment: the checkpoint, then the reverse's own iterations from it
        const double4_32a *state_at0 = a->ckpt + np * (size_t)c0;
        if (seg_sets) {
            // the segment's iterations once, each into its set, then reversed
            for (int t = t0; t < t1; t++) {
                const double4_32a *from = t == t0 ? state_at0 : set_P(t - 1 - t0, 4);
                CK(h, cudaMemcpyAsync(set_P(t - t0, 0), from, bytes, cudaMemcpyDeviceToDevice, h->L.stream));
                fwd_set(t - t0, 0);
            }
            for (int t = t1 - 1; t >= t0; t--) {
                if (m32) adj_iteration_reverse32(h, a->sets[t - t0]);
                else adj_iteration_reverse64(h, a->sets64[t - t0], v);
            }
            continue;
        }
        if (S > 1) {
            CK(h, cudaMemcpyAsync(a->seg, state_at0, bytes, cudaMemcpyDeviceToDevice, h->L.stream));
            for (int t = t0 + 1; t < t1; t++) {
                CK(h, cudaMemcpyAsync(a->P[0], a->seg + np * (size_t)(t - 1 - t0), bytes, cudaMemcpyDeviceToDevice,
                                      h->L.stream));
                adj_iteration_forward(h, m32);
                CK(h, cudaMemcpyAsync(a->seg + np * (size_t)(t - t0), a->P[4], bytes, cudaMemcpyDeviceToDevice,
                                      h->L.stream));
            }
        }
        for (int t = t1 - 1; t >= t0; t--) {
            const double4_32a *state = S > 1 ? a->seg + np * (size_t)(t - t0) : state_at0;
            CK(h, cudaMemcpyAsync(a->P[0], state, bytes, cudaMemcpyDeviceToDevice, h->L.stream));
            adj_iteration_forward(h, m32);
            adj_iteration_reverse(h, v, m32);
        }
    }
    if (store_all)
        for (int t = iters - 1; t >= 0; t--) {
            if (m32) adj_iteration_reverse32(h, a->sets[t]);
            else adj_iteration_reverse64(h, a->sets64[t], v);
        }
    if ((st = check_launch(h, "adjoint sweep"))) return st;
    // bar of the initial state: returned for prim0, else (the free stream)
    // summed over the points into the free-stream velocity (on the device)
    double bu[2], binit[2] = {0, 0};
    if (!prim0) {
        double *d_init = a->buinf + 2;
        zero(h, d_init, 2 * sizeof(double));
        fp64::sum_yz(h->L, h->n, a->bP, d_init);
        if ((st = d2h(h, binit, d_init, sizeof binit))) return st;
    }
    if ((st = d2h(h, bu, a->buinf, sizeof bu))) return st;
    if (dJ_dprim0 && (st = download_points(h, a->bP, dJ_dprim0))) return st;
    if (J) *J = os.J;
    adj_params(h, os, bu, binit, dJ_dmach, dJ_daoa);
    if (dJ_dwall) return adj_geometry(h, objective, h->s64.prim[h->pcur], dJ_dwall);
    return QLSKUM_OK;
}

qlskum_status qlskum_set_adjoint_stride(qlskum_handle *h, int stride)
{
    NEED(h);
    if (stride < 1) return fail(h, QLSKUM_ERR_INVALID, "stride must be >= 1");
    h->adj_stride = stride;
    return QLSKUM_OK;
}

qlskum_status qlskum_adjoint_fixed_point(qlskum_handle *h, int objective, int adj_iters, double *J,
                                         double *dJ_dmach, double *dJ_daoa, double *dJ_dwall, double *adj_change)
{
    NEED(h);
    qlskum_status st = adj_args(h, objective, adj_iters, dJ_dwall);
    if (st) return st;
    AdjBuf *a = h->adj;
    const size_t np = h->np;
    const bool m32 = adj_use32(h, dJ_dwall != nullptr);
    ObjSeed os;
    if ((st = adj_seed(h, objective, h->s64.prim[h->pcur], a->seed, os))) return st;
    CK(h, cudaMemcpyAsync(a->P[0], h->s64.prim[h->pcur], sizeof(double4_32a) * np, cudaMemcpyDeviceToDevice,
                          h->L.stream));
    zero(h, a->lam, sizeof(double4_32a) * np);
    const AdjView none = adj_view(h, false);
    // the stage states of S at U, once: the reverse passes only read them
    adj_iteration_forward(h, m32);
    // lam <- S_U^T lam + J_U at the current state U (one iteration map S)
    for (int k = 0; k < adj_iters; k++) {
        if (k == adj_iters - 1)
            CK(h, cudaMemcpyAsync(a->lam_prev, a->lam, sizeof(double4_32a) * np, cudaMemcpyDeviceToDevice,
                                  h->L.stream));
        CK(h, cudaMemcpyAsync(a->bP, a->lam, sizeof(double4_32a) * np, cudaMemcpyDeviceToDevice, h->L.stream));
        zero(h, a->buinf, 2 * sizeof(double));
        adj_iteration_reverse(h, none, m32);
        CK(h, cudaMemcpyAsync(a->lam, a->seed, sizeof(double4_32a) * np, cudaMemcpyDeviceToDevice, h->L.stream));
        fp64::add_prim(h->L, h->n, a->bP, a->lam);
    }
    // lam^T dS/dalpha: one more reverse pass, accumulating the parameter bars
    adj_zero_geometry(h);
    CK(h, cudaMemcpyAsync(a->bP, a->lam, sizeof(double4_32a) * np, cudaMemcpyDeviceToDevice, h->L.stream));
    adj_iteration_reverse(h, adj_view(h, dJ_dwall != nullptr), m32);
    if ((st = check_launch(h, "fixed-point adjoint"))) return st;
    double bu[2];
    if ((st = d2h(h, bu, a->buinf, sizeof bu))) return st;
    if (adj_change) {
        // relative change of the last adjoint iteration, reduced on the device
        unsigned long long *d_mx = reinterpret_cast<unsigned long long *>(a->buinf + 2);
        zero(h, d_mx, 2 * sizeof(unsigned long long));
        fp64::max_change(h->L, h->n, a->lam, a->lam_prev, d_mx);
        unsigned long long mx[2];
        if ((st = d2h(h, mx, d_mx, sizeof mx))) return st;
        double dmax, lmax;
        std::memcpy(&dmax, &mx[0], sizeof dmax);
        std::memcpy(&lmax, &mx[1], sizeof lmax);
        *adj_change = lmax > 0.0 ? dmax / lmax : dmax;
    }
    const double binit[2] = {0, 0};
    if (J) *J = os.J;
    adj_params(h, os, bu, binit, dJ_dmach, dJ_daoa);
    if (dJ_dwall) return adj_geometry(h, objective, h->s64.prim[h->pcur], dJ_dwall);
    return QLSKUM_OK;
}

}  // extern "C"
