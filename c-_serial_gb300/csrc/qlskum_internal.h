// Internal layout shared by the host layer (qlskum_host.cpp) and the CUDA
// translation units.  Plain structs of device pointers; no torch types.
//
// Device layout (all arrays in the permuted point order, np = n rounded up to
// a multiple of 32):
//   * per point: flag (int8), nbhs (int32), normal (double2), eps^2 of the
//     Venkatakrishnan limiter (double), gradient LSQ moments
//     {sxx, syy, sxy, 1/det} (double4_32a) and the same for the four flux
//     sub-stencils (double4_32a [np][4]);
//   * per edge, in a sliced-ELL ("warp-padded CSR") layout: slice s holds 32
//     consecutive points; edge j of lane l of slice s sits at
//     slice_base[s] + 32*j + l, so the 32 threads of a warp read edge j of
//     their points with one coalesced access.  Per edge: neighbour (int32),
//     {delx, dely, w*delx, w*dely} (double4_32a), {dels*w, deln*w} of the rotated
//     frame (double2), |r_k - r_i| (double), sub-stencil membership bits
//     (uint8: 1 xpos, 2 xneg, 4 ypos, 8 yneg);
//   * state, point-major AoS per field: prim / q (double4_32a), dq and qm
//     (2 x double4_32a per point: d/dx then d/dy, max then min).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace qlskum {

enum : int { kWall = 0, kInterior = 1, kOuter = 2 };
enum : unsigned { kXpos = 1u, kXneg = 2u, kYpos = 4u, kYneg = 8u };

struct CaseConst;

struct DevCloud {
    int n = 0;
    int np = 0;
    const int8_t *flag = nullptr;
    const int *nbhs = nullptr;
    const long long *slice_base = nullptr;   // [np/32]
    const int *e_nbr = nullptr;
    const double4_32a *e_geo = nullptr;          // delx, dely, w*delx, w*dely
    const double2 *e_sn = nullptr;           // dels*w, deln*w
    const double *e_dist = nullptr;          // |r_k - r_i|
    const uint8_t *e_dir = nullptr;
    const double2 *nrm = nullptr;
    const double *eps2 = nullptr;
    const double4_32a *ggeo = nullptr;           // [np]
    const double4_32a *fgeo = nullptr;           // [np][4]
    // mixed-precision copies of the per-edge geometry (FP32)
    const float4 *e_geo32 = nullptr;         // delx, dely, w*delx, w*dely
    const float2 *e_sn32 = nullptr;          // dels*w, deln*w
    const float *e_dist32 = nullptr;         // |r_k - r_i|
    const float *eps2_32 = nullptr;
    // Mixed form: the four directional 2x2 solves and their sum into the flux
    // residual folded into per-edge weights.  With Sx_d = sum dG dels w and
    // Sy_d = sum dG deln w over the edges of sub-stencil d, the residual is
    // F = delta * sum_d (a_d Sx_d + b_d Sy_d), a_d, b_d the x / y row of the
    // inverse moment matrix (1/det included, the wall's factor 2, zero for a
    // direction the class does not use); so F = delta * sum_e sum_{d ∋ e}
    // c_ed dG_ed with c_ed = a_d dels_w + b_d deln_w, computed on the host in
    // FP64 (where the near-singular inverse meets the edge vector) and stored
    // in FP32: {c of the edge's x half-range (xpos if it lies there, else
    // xneg), c of its y half-range (ypos, else yneg)} per edge, and the same
    // for the second half-range of an edge with dels == 0 / deln == 0 (which
    // lies in both; zero otherwise).
    const float2 *e_w32 = nullptr;
    const float2 *e_w32b = nullptr;
    // Mixed form, gradient and inner loop: the 2x2 solve dq_x = Sx a - Sy b,
    // dq_y = Sy c - Sx b ({a, b, c} = {syy, sxy, sxx} / det) folded into
    // per-edge weights as for the flux: with Sx = sum w delx dq and
    // Sy = sum w dely dq, dq_x = sum_e gx_e dq_e and dq_y = sum_e gy_e dq_e,
    // gx = a w delx - b w dely, gy = c w dely - b w delx, computed on the
    // host in FP64 and stored in FP32 {gx, gy} per edge.
    const float2 *e_gw32 = nullptr;
    // power == 0 (all weights 1): the mixed kernels read only {delx, dely}
    // per edge (FP32) and rotate it by the point normal themselves.
    int unit_w = 0;
    const float2 *e_xy32 = nullptr;
    // largest neighbour count of the cloud (sizes the staged kernels' shared memory)
    int max_nb = 0;
    // A batch's concatenated cloud (several cases, each its own flight
    // condition): the free-stream constants of the case that owns slice s
    // are case_k[slice_case[s]], read by the outer points' far-field state;
    // NULL for a single case, whose constants come with the launch.
    const CaseConst *case_k = nullptr;
    const int *slice_case = nullptr;
};

// Free-stream constants of one case (parameter_mod.h:4-30).
struct CaseConst {
    double mach, theta, rho_inf, pr_inf, gamma, pi;
    double u1_inf, u2_inf;
    double cfl;
};

// ----------------------------------------------------------------- batches
// A batch runs many cases (a cloud and a flight condition each) as one
// concatenated cloud: case c owns points [off, off + n) of it, off a
// multiple of kBatchAlign, and the points up to the next case are padding
// (no neighbours, a finite state).  Its per-point and per-edge geometry is
// its cloud's, with the neighbour indices moved by off, so the single-cloud
// kernels run every case in one launch each.  Because off is a multiple of
// every flux block's point count, a block of the flux kernel never spans two
// cases and case c's residual partials are blocks [blk0, blk0 + nblk).
constexpr int kBatchAlign = 256;
constexpr int block_index(int points) { return points == 64 ? 0 : (points == 256 ? 2 : 1); }

struct BatchCase {
    int cloud;
    int n;
    long long off;
    int blk0[3], nblk[3];                    // first flux block and block count per block size (64, 128, 256 points)
    CaseConst K;
};

struct BatchView {
    const BatchCase *cases = nullptr;        // device array [ncases]
    int ncases = 0;
};

// FP64 state buffers of one handle.
struct State64 {
    double4_32a *prim[3] = {nullptr, nullptr, nullptr};
    double4_32a *q[2] = {nullptr, nullptr};
    double4_32a *dq[2] = {nullptr, nullptr};     // [np][2] each
    double4_32a *qm = nullptr;                   // [np][2]
    double4_32a *flux_res = nullptr;
    double *delta = nullptr;
    double *cspeed = nullptr;                // |u| + 3 sqrt(p/rho) of the current prim
};

// Mixed-precision state: q, dq, qm in FP32, prim in FP64; the local time step
// and the wave speed it is built from in FP32 (a pseudo-time step size: its
// rounding does not move the steady state).
struct State32 {
    float4 *q[2] = {nullptr, nullptr};
    // [np][2] each: dq[0] the stage's first-order gradient, dq[1] / dq[2]
    // the inner steps' outputs in turn (mixed_dq_in / mixed_dq_out)
    float4 *dq[3] = {nullptr, nullptr, nullptr};
    float4 *qm = nullptr;                    // [np][2]
    float *delta = nullptr;
    float *cspeed = nullptr;
};

// Buffers of the mixed inner loop: step j (0-based) reads dq[mixed_dq_in(j)]
// and writes dq[mixed_dq_out(j)]; the flux kernel reads dq[mixed_dq_final(ni)].
inline int mixed_dq_in(int j) { return j == 0 ? 0 : 1 + ((j - 1) & 1); }
inline int mixed_dq_out(int j) { return 1 + (j & 1); }
inline int mixed_dq_final(int ni) { return ni == 0 ? 0 : mixed_dq_out(ni - 1); }

// Residual reduction scratch.
struct Reduce {
    double *partial_sum = nullptr;           // [blocks]
    double *partial_max = nullptr;           // [blocks]
    double *hist = nullptr;                  // [capacity][3]: res_new, residue, max_res
    double *res_old = nullptr;               // [1]
    int *iter = nullptr;                     // [1] iterations completed
    int *status = nullptr;                   // [1] 0 ok, 1 non-finite residual
    int capacity = 0;
    int blocks = 0;                          // partials written by the last stage kernel
    int max_blocks = 0;                      // partials allocated (n / 32 rounded up)
    // res_old latches at iterations 1 and 2 unless the run continues from a
    // restart file, which carries its own (fpi_solver_mod.h:139)
    int latch = 1;
};

struct Launch {
    cudaStream_t stream = nullptr;
    int block = 128;
    long long *launches = nullptr;           // host counter
    // mixed gradient / inner-loop kernels: 0 = one gather per edge in turn,
    // v > 0 = staged variant v (edge list in shared memory, neighbour data
    // streamed with cp.async a few edges ahead); picked by the autotuner
    int staged = 0;
    // mixed gradient / inner-loop kernels of the per-edge gather form: lanes
    // per point (1, 2 or 4: a point's edges split over that many lanes)
    int lanes = 1;
};

// ---------------------------------------------------------- adjoint (qlskum_adjoint.cu)
// The geometry read by the adjoint kernels plus, when requested, the
// accumulators of the geometry's adjoints (device order): per edge
// {delx, dely, dels w, deln w} and |r_k - r_i|; per point the normal, the
// gradient moments and the four directional moment sets.
struct AdjView {
    DevCloud c;
    // with the geometry accumulators: 1 for the points whose geometry (edge
    // vectors, moments, normal) depends on a wall point's coordinates (the
    // wall points and the points with a wall neighbour), 0 elsewhere; the
    // kernels accumulate geometry bars only there
    const uint8_t *geo_pt = nullptr;
    // the same points as a list (device order indices), for the kernels
    // that accumulate geometry bars over those points alone
    const int *geo_list = nullptr;
    int n_geo = 0;
    double4_32a *bedge = nullptr;
    double *bdist = nullptr;
    double2 *bnrm = nullptr;
    double4_32a *bgmom = nullptr;
    double4_32a *bfmom = nullptr;
};

namespace adjl {
void update(const Launch &L, const AdjView &a, const CaseConst &K, const double4_32a *Pin, const double4_32a *Pold,
            const double4_32a *Pout, int rk, double4_32a *bP, double4_32a *bPold, double4_32a *bF, double *buinf);
// flux: the stage's flux residual (the bar of delta without geometry bars);
// sums: its directional sums (fp64::flux_residual) for the geometry bars, or
// NULL (recomputed); ends: the edge ends' kept transcendentals
// (fp64::flux_residual's ends, ns slots), or NULL (recomputed)
void flux(const Launch &L, const AdjView &a, const double4_32a *q, const double4_32a *dq, const double4_32a *qm,
          const double *delta, const double4_32a *flux, const double *sums, const double *ends, long long ns,
          const double4_32a *bF, double4_32a *bq, double4_32a *bdq, double4_32a *bqm, double *bdelta);
void inner(const Launch &L, const AdjView &a, const double4_32a *q, const double4_32a *dq_in,
           const double4_32a *bdq_out, double4_32a *bq, double4_32a *bdq_in);
void grad(const Launch &L, const AdjView &a, const double4_32a *q, const double4_32a *bdq, const double4_32a *bqm,
          double4_32a *bq);
void qvars(const Launch &L, int n, const double4_32a *P, const double4_32a *bq, double4_32a *bP);
void delta(const Launch &L, const AdjView &a, const double4_32a *P, const double *bdelta, double cfl, double *bc,
           double4_32a *bP);
void objective(const Launch &L, const AdjView &a, const int *wall_perm, const double4_32a *wall_geo, int n_wall,
               double cp_scale, double theta, int which, double4_32a *bP);
// bP += dJ/dprim of the stagnation-pressure loss
void objective_J(const Launch &L, int n, const double4_32a *P, double gamma, double p0_inf, double4_32a *bP);
// the geometry bars of a reverse sweep pulled back to the point coordinates
// (bx, by zeroed first; bn: each point's normal bar), unit weights
void geom_pullback(const Launch &L, const AdjView &a, double *bx, double *by, double2 *bn);
// AdjView::geo_pt of the cloud (1: a wall point or a point with a wall neighbour)
void mark_geo_points(const Launch &L, const DevCloud &c, uint8_t *geo_pt);
}  // namespace adjl

// Reverse of the mixed iteration (qlskum_adjoint.cu, FP32 edge work): bars of
// the FP32 q / dq / qm in float4 arrays (atomically accumulated), of delta in
// float, of the FP64 states in double4.
// The forward edge list transposed for the reverse of the mixed iteration:
// for each point k, the edges (i -> k) that have k as their neighbour, in a
// sliced ELL like the forward list (slot sbase[k >> 5] + 32 m + (k & 31),
// m < nb[k]), each slot carrying a copy of the forward edge's data, so a
// reverse kernel pulls its point's bars from the edges' owners instead of
// the owners scattering them with atomics.
struct AdjT {
    const long long *sbase = nullptr;  // [nslices]
    const int *nb = nullptr;           // [np] incoming edges
    const int *src = nullptr;          // the edge's owner i
    const int *e = nullptr;            // the forward slot (for the rare second flux weight)
    const float2 *xy = nullptr;        // the edge vector x_k - x_i
    const float2 *gw = nullptr;        // folded gradient weights (DevCloud::e_gw32)
    const float2 *w = nullptr;         // folded flux weights (DevCloud::e_w32)
    const float2 *nrm = nullptr;       // the owner's normal
    const uint8_t *df = nullptr;       // direction bits | the owner's class << 4
};

namespace adjml {
// reverse of the stage update (rk 1..4 as the forward), FP32 arithmetic; also
// bs = delta * bF, the bar of each point's weighted flux sum
void update(const Launch &L, const DevCloud &c, const CaseConst &K, const double4_32a *Pin, const double4_32a *Pold,
            const double4_32a *Pout, int rk, const float *delta, double4_32a *bP, double4_32a *bPold, float4 *bF,
            float4 *bs, double *buinf);
// reverse of the flux part: stores every point's bars of q, dq and qm (both
// ends of the edges it owns and the ends of the edges that have it as
// neighbour, pulled through T), adds to bdelta
void flux(const Launch &L, const DevCloud &c, const AdjT &T, const float4 *q, const float4 *dq, const float4 *qm,
          const float4 *acc, const float4 *bF, const float4 *bs, float4 *bq, float4 *bdq, float4 *bqm, float *bdelta);
// reverse of one mixed inner step: stores bdq_in, bdq0 += bdq_out (the dq0
// term; = for the stage's first reverse step)
void inner(const Launch &L, const DevCloud &c, const AdjT &T, const float4 *bdq_out, float4 *bdq_in, float4 *bdq0,
           bool first);
// reverse of the gradient and max / min; the gradient's bar is bdq + bdq0
void grad(const Launch &L, const DevCloud &c, const float4 *q, const float4 *bdq, const float4 *bdq0,
          const float4 *bqm, float4 *bq);
void qvars(const Launch &L, int n, const double4_32a *P, const float4 *bq, double4_32a *bP);
// reverse of the time step and of the wave speed it came from; bP += ...
void delta(const Launch &L, const DevCloud &c, const double4_32a *P, const float *cs, const float *bdelta, float cfl,
           float *bcs, double4_32a *bP);
}  // namespace adjml

// ---------------------------------------------------------- FP64 kernels (qlskum_fp64.cu)
namespace fp64 {
void q_variables(const Launch &L, const DevCloud &c, const double4_32a *prim, double4_32a *q);
void derived(const Launch &L, const DevCloud &c, const double4_32a *prim, double4_32a *q, double *cspeed);
void q_derivatives(const Launch &L, const DevCloud &c, const double4_32a *q, double4_32a *dq, double4_32a *qm,
                   const double *cspeed, double *delta, double cfl);
void q_inner(const Launch &L, const DevCloud &c, const double4_32a *q, const double4_32a *dq_in, double4_32a *dq_out);
void func_delta(const Launch &L, const DevCloud &c, const double4_32a *prim, double *delta, double cfl);
// sums (or NULL): each point's directional sums {sx[d][r], sy[d][r]}, [n][32] doubles.
// ends (or NULL): per edge slot of the ns slots, the owner's and the
// neighbour's end's rho, sqrt(beta), exp(-S1^2), exp(-S2^2), erf(S1),
// erf(S2), as 12 planes of ns doubles (read back by the flux reverse).
void flux_residual(const Launch &L, const DevCloud &c, const double4_32a *q, const double4_32a *dq, const double4_32a *qm,
                   const double *delta, double4_32a *flux_res, double *sums = nullptr, double *ends = nullptr,
                   long long ns = 0);
void state_update(const Launch &L, const DevCloud &c, const CaseConst &k, double4_32a *prim, const double4_32a *prim_old,
                  const double4_32a *flux_res, int rk, const Reduce &R);
void flux_update(const Launch &L, const DevCloud &c, const CaseConst &k, const double4_32a *q, const double4_32a *dq,
                 const double4_32a *qm, const double *delta, const double4_32a *prim, const double4_32a *prim_old,
                 double4_32a *prim_next, double4_32a *q_next, double *cspeed_next, int rk, const Reduce &R);
void reduce_residual(const Launch &L, const Reduce &R, int n, int it);
void copy_prim(const Launch &L, int n, const double4_32a *src, double4_32a *dst);
// dst += src over n double4 rows
void add_prim(const Launch &L, int n, const double4_32a *src, double4_32a *dst);
// dst[i] = v for i < n
void fill_prim(const Launch &L, int n, double4_32a v, double4_32a *dst);
// out[0] = max |a - b|, out[1] = max |a| over n points (as non-negative double bit patterns; out zeroed first)
void max_change(const Launch &L, int n, const double4_32a *a, const double4_32a *b, unsigned long long *out);
// *p = v on the stream (the iteration counter a captured iteration reads)
void set_counter(const Launch &L, int *p, int v);
// out[0] += sum_i src[i].y, out[1] += sum_i src[i].z
void sum_yz(const Launch &L, int n, const double4_32a *src, double *out);
// [n] point states from the cloud's order into the handle's (dst[perm[i]] = src[i]) and back
void permute_in(const Launch &L, int n, const int *perm, const double4_32a *src, double4_32a *dst);
void permute_out(const Launch &L, int n, const int *perm, const double4_32a *src, double4_32a *dst);
// diagnostics: vorticity [n] and per-256-block partial sums of its square;
// stagnation pressure per-256-block {min, argmin, max, argmax, sum (p0_inf - p0)^2, sum p0}
void enstrophy(const Launch &L, const DevCloud &c, const double4_32a *prim, double *vort, double *partial);
void stagnation(const Launch &L, int n, const double4_32a *prim, double gamma, double p0_inf, double *partial);
// objectives: per-block partial sums into scratch ([4][ceil(max(n, n_wall)/256)]), then one ordered sum;
// entropy NULL: the force sums only (wall points), the entropy sum left 0
void objective(const Launch &L, const DevCloud &c, const double4_32a *prim, const int *wall_perm, const double4_32a *wall_geo,
               int n_wall, double cp_scale, double pr_inf, double gamma, double *entropy, double *out4, double *scratch);
}  // namespace fp64

// ---------------------------------------------------------- halo exchange (qlskum_fp64.cu)
namespace halo {
// Ghost slots of a partition from their owner's arrays: dst[g] = src[idx[g]]
// for g < n, elements of `bytes` bytes (4, 8 or a multiple of 16; src, dst
// aligned to the element, 16 bytes for the multiples of 16).
void pull(const Launch &L, int n, const int *idx, const void *src, void *dst, int bytes);
}  // namespace halo

// ---------------------------------------------------------- mixed kernels (qlskum_mixed.cu)
namespace mixed {
void derived(const Launch &L, const DevCloud &c, const double4_32a *prim, float4 *q, float *cspeed);
void q_derivatives(const Launch &L, const DevCloud &c, const float4 *q, float4 *dq, float4 *qm,
                   const float *cspeed, float *delta, float cfl);
// one inner step: dq_out = dq0 + 0.5 (dq_in - solve(sum w d (d.dq_in_k))), dq0 the stage's
// first-order gradient (the reference's step, reassociated)
void q_inner(const Launch &L, const DevCloud &c, const float4 *dq0, const float4 *dq_in, float4 *dq_out);
// staged variants of the gradient / inner-loop kernels usable on this cloud
// (Launch::staged = 1 .. staged_variants()); sets their shared-memory limits
int staged_variants(const DevCloud &c);
int staged_block(int v);
int staged_depth(int v);
void flux_update(const Launch &L, const DevCloud &c, const CaseConst &k, const float4 *q, const float4 *dq,
                 const float4 *qm, const float *delta, const double4_32a *prim, const double4_32a *prim_old,
                 double4_32a *prim_next, float4 *q_next, float *cspeed_next, int rk, const Reduce &R, int variant,
                 float4 *acc_out = nullptr);  // acc_out: the point's flux accumulator (F / delta) when non-null
int flux_variants();
int flux_block(int variant);        // threads per block
int flux_min_blocks(int variant);
int flux_lanes(int variant);        // lanes per point
// blocks (residual partials) of one launch of `variant` over n points
int flux_grid_blocks(int variant, int n);
// batches: the concatenated cloud's neighbour lists (dst[j] = src[j] + off
// for j < ne) and the padding points' normals ((0, 1) for the n points)
void batch_offset_nbr(const Launch &L, const int *src, int *dst, long long ne, int off);
void batch_fill_normals(const Launch &L, double2 *nrm, long long n);
// per case: res_new from the flux kernel's block partials (`points` points per block), the residual
// history row, the non-finite flag; then the device iteration counter
void batch_reduce(const Launch &L, const BatchView &B, int points, const double *psum, const double *pmax,
                  int *iter, double *res_old, double *res_new, double *hist, int capacity, int *status);
}  // namespace mixed

}  // namespace qlskum
