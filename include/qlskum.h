/* qlskum.h -- C ABI of the GB300 (sm_103a) q-LSKUM solver core.
 *
 * Drop-in for the serial reference solver's module API (Pathlessbark8/C-_serial).
 * The reference exposes argument-less void functions over the global `point`
 * struct (data_structure_mod.h:10-49) and global knobs (data_structure_mod.h:
 * 57-121, parameter_mod.h:4-11); here the same modules are entry points on a
 * handle that owns the device-resident state.
 *
 * Conventions
 *   - Input cloud arrays are host arrays in the reference's grid-file layout
 *     (main.cpp:30-58): 1-based `left`, `right` and `conn` ([n][20], row i
 *     holding the nbhs[i] neighbours of point i+1), flag_1 0 wall / 1 interior
 *     / 2 outer, flag_2 > 0 on shape points, which must come first
 *     (compute_force_coeffs_mod.h:25-27).
 *   - Every point-valued output is in the ORIGINAL point order, 0-based rows,
 *     point-major: [n][4] for prim / q / flux_res, [n][2][4] for dq and qm
 *     (dq[i][0] = d/dx, dq[i][1] = d/dy; qm[i][0] = max, qm[i][1] = min).
 *   - All calls on one handle are stream-ordered on the handle's CUDA stream;
 *     functions that return host data synchronise that stream.  A handle is
 *     not thread-safe; distinct handles are independent.
 *   - Errors: every function returns a qlskum_status; qlskum_last_error()
 *     gives the message of the last failure on a handle (or of the last
 *     failed qlskum_create when passed NULL).
 */
#ifndef QLSKUM_H
#define QLSKUM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QLSKUM_MAX_NBHS 20
#define QLSKUM_ABI_VERSION 1

typedef enum {
    QLSKUM_OK = 0,
    QLSKUM_ERR_INVALID = 1,      /* bad argument or malformed cloud */
    QLSKUM_ERR_DEGENERATE = 2,   /* a sub-stencil has a singular 2x2 least-squares matrix */
    QLSKUM_ERR_NONFINITE = 3,    /* the state or the residual became NaN / Inf */
    QLSKUM_ERR_CUDA = 4,         /* a CUDA call failed */
    QLSKUM_ERR_UNSUPPORTED = 5   /* option not available in this build / precision */
} qlskum_status;

typedef enum {
    QLSKUM_FP64 = 0,             /* FP64 end to end: the drop-in form */
    QLSKUM_MIXED = 1             /* FP32: q, dq, qm storage, limiter, reconstruction, split fluxes,
                                    the per-point weighted sums over the edges and an interior
                                    point's stage change; FP64: the 2x2 least-squares solves (folded
                                    once per cloud into per-edge FP32 weights), prim and its
                                    accumulation over the stages (prim + change), the wall and outer
                                    points' SSPRK update, the residual norm's sum over the points */
} qlskum_precision;

/* The grid file's columns (main.cpp:32-36), host memory, 1-based indices. */
typedef struct {
    int n;
    const double *x, *y;
    const int *left, *right;
    const int *flag_1, *flag_2;
    const double *min_dist;
    const int *nbhs;
    const int *conn;              /* [n][QLSKUM_MAX_NBHS] */
} qlskum_cloud;

/* Case and solver knobs: parameter_mod.h:4-8 (mach, aoa) and
 * data_structure_mod.h:72,90,96,118 (CFL, power, VL_CONST, inner_iterations). */
typedef struct {
    double mach;
    double aoa;                   /* degrees */
    double cfl;
    double vl_const;
    double power;                 /* least-squares weights dist^power */
    int inner_iterations;
    int precision;                /* qlskum_precision */
    int block_size;               /* threads per block for the point kernels; 0 = default */
    int reorder;                  /* 1 = Morton/class reorder of points on the device (default), 0 = file order */
    int verbose;                  /* 1 = print "iterations <it> residue : <r>" per iteration like fpi_solver_mod.h:150 */
} qlskum_params;

typedef struct qlskum_handle qlskum_handle;

/* Fill `p` with the reference's defaults (parameter_mod.h / data_structure_mod.h:
 * mach 0.63, aoa 2, CFL 0.1, VL_CONST 150, power 0, inner_iterations 3), FP64. */
void qlskum_default_params(qlskum_params *p);

/* ---------------------------------------------------------------- lifetime */

/* Copies the cloud, computes normals (point_normals_mod.h:5-55) and the four
 * directional sub-stencils (generate_connectivity_mod.h:221-249) on the host
 * in FP64 with the reference's operation order (bit-exact), reorders the
 * points, uploads everything and sets the free-stream initial state
 * (initial_conditions_mod.h:23-37).  Replaces main.cpp:59-65. */
qlskum_status qlskum_create(const qlskum_cloud *cloud, const qlskum_params *params, qlskum_handle **out);
qlskum_status qlskum_destroy(qlskum_handle *h);
const char *qlskum_last_error(const qlskum_handle *h);
int qlskum_abi_version(void);

/* ------------------------------------------------ module-mirroring entry points */

/* state_update_mod.h:448-496 */
qlskum_status qlskum_func_delta(qlskum_handle *h);
/* q_variables_mod.h:9-34 */
qlskum_status qlskum_eval_q_variables(qlskum_handle *h);
/* q_variables_mod.h:36-118 */
qlskum_status qlskum_eval_q_derivatives(qlskum_handle *h);
/* q_variables_mod.h:120-213 */
qlskum_status qlskum_eval_q_inner_loop(qlskum_handle *h);
/* q_variables_mod.h:215-228 */
qlskum_status qlskum_eval_update_innerloop(qlskum_handle *h);
/* flux_residual_mod.h:10-89 with interior_/wall_/outer_fluxes_mod.h, the
 * split and quadrant fluxes and the Venkatakrishnan limiter (limiters_mod.h:55-104) */
qlskum_status qlskum_cal_flux_residual(qlskum_handle *h);
/* state_update_mod.h:92-283, rk in 1..4 */
qlskum_status qlskum_state_update(qlskum_handle *h, int rk);
/* prim_old <- prim (fpi_solver_mod.h:19-25) */
qlskum_status qlskum_snapshot_prim_old(qlskum_handle *h);
/* One pseudo-time iteration (fpi_solver_mod.h:14-151) with fused kernels.
 * `it` is the reference's iteration number (res_old latches at it <= 2). */
qlskum_status qlskum_fpi_solver(qlskum_handle *h, int it);
/* `iters` iterations continuing from the handle's iteration counter
 * (q_lskum_mod.h:13-38); replayed from a CUDA graph per iteration. */
qlskum_status qlskum_q_lskum(qlskum_handle *h, int iters);

/* compute_force_coeffs_mod.h:7-69 and compute_entropy_mod.h:5-24 (the
 * entropy total summed over all points, which the reference computes but
 * loses in a shadowing local).  Any pointer may be NULL. */
qlskum_status qlskum_objective(qlskum_handle *h, double *cl, double *cd, double *cm, double *total_entropy);

/* --------------------------------------------------------------- state I/O */

enum {
    QLSKUM_FIELD_PRIM = 0,        /* [n][4] */
    QLSKUM_FIELD_PRIM_OLD = 1,    /* [n][4] */
    QLSKUM_FIELD_Q = 2,           /* [n][4] */
    QLSKUM_FIELD_DQ = 3,          /* [n][2][4] */
    QLSKUM_FIELD_QM = 4,          /* [n][2][4] */
    QLSKUM_FIELD_FLUX_RES = 5,    /* [n][4] */
    QLSKUM_FIELD_DELTA = 6,       /* [n] */
    QLSKUM_FIELD_NORMALS = 7,     /* [n][2] */
    QLSKUM_FIELD_ENTROPY = 8      /* [n], filled by qlskum_objective */
};

/* Copy a field to host memory `out` (original point order, FP64). */
qlskum_status qlskum_get_field(qlskum_handle *h, int field, double *out);
/* Overwrite prim ([n][4], original order), e.g. from restart.dat
 * (initial_conditions_mod.h:7-21). */
qlskum_status qlskum_set_prim(qlskum_handle *h, const double *prim);
qlskum_status qlskum_get_prim(qlskum_handle *h, double *out);
/* Sub-stencils in original order: counts [n][4] (xpos, xneg, ypos, yneg) and
 * lists [n][4][20] (1-based, unused slots 0), as generate_connectivity builds them. */
qlskum_status qlskum_get_connectivity(qlskum_handle *h, int *counts, int *lists);
/* Residual history: for each completed iteration (res_new, residue, max_res)
 * as fpi_solver_mod.h:138-147 and state_update_mod.h:157-165 define them.
 * Writes min(count, max_rows) rows to out ([max_rows][3]); returns count via *rows. */
qlskum_status qlskum_get_residual_history(qlskum_handle *h, double *out, int max_rows, int *rows);
/* Iterations completed so far. */
qlskum_status qlskum_get_iteration(qlskum_handle *h, int *it);
qlskum_status qlskum_synchronize(qlskum_handle *h);
/* The CUDA stream (cudaStream_t) the handle launches on, as an opaque pointer. */
void *qlskum_stream(qlskum_handle *h);
/* Kernel launches issued by this handle so far (the benchmark's launch count). */
long long qlskum_launch_count(const qlskum_handle *h);

/* Launch shape in use: threads per block and minimum resident blocks per SM
 * (register cap) of the fused flux + update kernel, threads per block of the
 * gradient / inner-loop kernels and their gather depth (0: one neighbour
 * gather per edge in turn; D > 0: edge list staged in shared memory and the
 * neighbours' data streamed with cp.async D edges ahead).  With
 * params.block_size == 0 the mixed form picks them on its first fused
 * iteration by timing the candidates on the handle's own cloud (the
 * autotuner).  Any pointer may be NULL. */
qlskum_status qlskum_get_launch_config(qlskum_handle *h, int *flux_block, int *flux_min_blocks, int *point_block,
                                       int *gather_depth);
/* Pin the mixed form's launch shape instead of autotuning it: flux_variant in
 * 0 .. 9 (threads x min blocks 128x4, 128x5, 64x8, 256x2 with one gather per
 * edge in turn; 128x4, 128x5, 64x8, 256x2 with the next edge's neighbour data
 * in flight by cp.async; 128x4 with 2 lanes per point, 256x2 with 4 lanes per
 * point, a point's edges split over its lanes and their sums combined by
 * warp shuffles), point_block one of
 * 64 / 128 / 256 / 512 for the per-edge gather form, staged 0 (that form) or
 * 1 .. 4 (staged gathers: 128 threads depth 2, 128 / 4, 256 / 3, 64 / 4).
 * The gradient / inner-loop kernels go back to one lane per point.
 * QLSKUM_ERR_UNSUPPORTED if a staged variant does not fit the device's
 * shared memory for this cloud's neighbour count. */
qlskum_status qlskum_set_launch_config(qlskum_handle *h, int flux_variant, int point_block, int staged);
/* Lanes per point (1, 2 or 4) of the mixed gradient / inner-loop kernels in
 * the per-edge gather form (staged 0): a point's edges split over adjacent
 * lanes, their sums, maxima and minima combined with warp shuffles.  The
 * autotuner picks it together with point_block unless it is set. */
qlskum_status qlskum_set_point_lanes(qlskum_handle *h, int lanes);
/* Lanes per point in use: gradient / inner-loop kernels and the fused flux kernel. */
qlskum_status qlskum_get_lanes(const qlskum_handle *h, int *point_lanes, int *flux_lanes);
/* The flux_variant in use (as qlskum_set_launch_config numbers them; 0 for FP64 handles). */
int qlskum_get_flux_variant(const qlskum_handle *h);

/* Per-kernel device time from CUDA events recorded on the handle's stream.
 * While enabled, qlskum_q_lskum launches each iteration's kernels one by one
 * (no CUDA graph) so that every launch is bracketed by events.
 * kernel: 0 gradient + min/max (q_derivatives), 1 inner loop, 2 fused flux +
 * state update, 3 residual reduction.  Enabling resets the totals. */
enum { QLSKUM_KERNEL_GRADIENT = 0, QLSKUM_KERNEL_INNER = 1, QLSKUM_KERNEL_FLUX_UPDATE = 2, QLSKUM_KERNEL_REDUCE = 3 };
qlskum_status qlskum_set_kernel_timing(qlskum_handle *h, int enable);
qlskum_status qlskum_get_kernel_timing(qlskum_handle *h, int kernel, double *ms_total, long long *launches);

/* ------------------------------------------------------- batched launches */

/* Many flight conditions over many clouds of uneven size, solved together:
 * the cases form one concatenated cloud (each case's points from a multiple
 * of 256 on, its neighbour lists moved by that offset, its free-stream
 * constants looked up by its outer points), so every kernel of an iteration
 * is one launch of the single-cloud kernel over all cases; each iteration's
 * four SSPRK stages are captured once per buffer phase as a CUDA graph and
 * replayed, and the block size of the gradient / inner-loop kernels and the
 * flux kernel's variant are picked by timing the candidates on the batch
 * (autotuner).  The
 * q-LSKUM iteration per case is fpi_solver_mod.h:14-151 in the mixed
 * precision form (params->precision must be QLSKUM_MIXED).
 * Case c solves cloud case_cloud[c] at Mach case_mach[c], AoA case_aoa[c]
 * (degrees); cfl, vl_const, power and inner_iterations come from params. */
typedef struct qlskum_batch qlskum_batch;
qlskum_status qlskum_batch_create(const qlskum_cloud *clouds, int n_clouds, const int *case_cloud,
                                  const double *case_mach, const double *case_aoa, int n_cases,
                                  const qlskum_params *params, qlskum_batch **out);
qlskum_status qlskum_batch_destroy(qlskum_batch *b);
const char *qlskum_batch_last_error(const qlskum_batch *b);
/* `iters` iterations of every case. */
qlskum_status qlskum_batch_run(qlskum_batch *b, int iters);
/* Per-case Cl, Cd, Cm and total entropy ([n_cases] each; any may be NULL). */
qlskum_status qlskum_batch_objective(qlskum_batch *b, double *cl, double *cd, double *cm, double *entropy);
/* prim of one case, [n][4] in its cloud's original point order. */
qlskum_status qlskum_batch_get_prim(qlskum_batch *b, int case_index, double *out);
/* res_new of every case per completed iteration: out [rows][n_cases]. */
qlskum_status qlskum_batch_residual_history(qlskum_batch *b, double *out, int max_rows, int *rows);
long long qlskum_batch_total_points(const qlskum_batch *b);
long long qlskum_batch_launch_count(const qlskum_batch *b);
void *qlskum_batch_stream(qlskum_batch *b);
/* The autotuned launch shape: threads per block of the gradient / inner-loop
 * kernels, points per block and minimum resident blocks per SM of the flux
 * kernel, points per warp of the flux kernel (32 / its lanes per point). */
qlskum_status qlskum_batch_tuning(const qlskum_batch *b, int *tile, int *flux_tile, int *flux_min_blocks,
                                  int *points_per_warp);
/* Lanes per point (1, 2 or 4) of the gradient / inner-loop kernels and of the flux kernel. */
qlskum_status qlskum_batch_lanes(const qlskum_batch *b, int *point_lanes, int *flux_lanes);
/* Pin the batch's launch shape instead of autotuning it: threads per block
 * (64, 128, 256) and lanes per point of the gradient / inner-loop kernels,
 * and the flux variant (0 .. 18, the numbering of qlskum_set_launch_config). */
qlskum_status qlskum_batch_set_launch_config(qlskum_batch *b, int tile, int point_lanes, int flux_variant);

/* ------------------------------------------- partitions with a ghost-point halo */

/* The solve split into partitions in the reference's distributed layout
 * (data_structure_mod.h:4-8: local_points, ghost_points and pghost, the
 * global numbers of a partition's ghost points; point_preprocessing_mod.h:
 * 124-132 reads them per partition): each partition owns a compact range of
 * the points (the cloud sorted by the Morton code of its coordinates and cut
 * into n_parts ranges of nearly equal size) and keeps copies of the points
 * outside it that its own points read (its ghosts: 1-based global numbers,
 * grouped by owning partition, in the owner's order).  Every kernel that
 * reads a neighbour's value is preceded by an exchange that refreshes the
 * ghosts from their owners: per stage q (and the wave speed of the time
 * step in the first stage), dq and qm after the gradient, dq after each
 * inner step.  The residual norm and the objectives are sums over the
 * partitions.  All partitions run on the current GPU, each on its own
 * stream; the point arithmetic is the single-domain solve's, so the state
 * equals qlskum_q_lskum's on the whole cloud (bit for bit in FP64, and in
 * the mixed form with the same launch shape), and only the order of the
 * residual and objective sums differs.  No counterpart in the serial
 * reference, whose ghost arrays are never filled. */
typedef struct qlskum_partition qlskum_partition;
/* The plan without a GPU: part_of [n] (0-based partition of each point),
 * n_local / n_ghost [n_parts]; any pointer may be NULL. */
qlskum_status qlskum_partition_plan(const qlskum_cloud *cloud, int n_parts, int *part_of, int *n_local,
                                    int *n_ghost);
/* One partition's points (1-based, in its device order) and ghosts (1-based,
 * as pghost holds them), without a GPU; either pointer may be NULL. */
qlskum_status qlskum_partition_plan_lists(const qlskum_cloud *cloud, int n_parts, int part, int *local_ids,
                                          int *ghost_ids);
qlskum_status qlskum_partition_create(const qlskum_cloud *cloud, const qlskum_params *params, int n_parts,
                                      qlskum_partition **out);
qlskum_status qlskum_partition_destroy(qlskum_partition *p);
const char *qlskum_partition_last_error(const qlskum_partition *p);
/* Sizes and point lists of partition `part` (as qlskum_partition_plan_lists). */
qlskum_status qlskum_partition_layout(const qlskum_partition *p, int part, int *n_local, int *n_ghost,
                                      int *local_ids, int *ghost_ids);
/* Mixed form: the launch shape (numbered as qlskum_set_launch_config;
 * default flux_variant 5, point_block 128 or params.block_size, staged 0). */
qlskum_status qlskum_partition_set_launch_config(qlskum_partition *p, int flux_variant, int point_block, int staged);
/* `iters` iterations (q_lskum_mod.h:13-38) of the partitioned solve. */
qlskum_status qlskum_partition_q_lskum(qlskum_partition *p, int iters);
/* The state [n][4] in the cloud's point order, gathered from the owners /
 * written to owners and ghosts alike. */
qlskum_status qlskum_partition_get_prim(qlskum_partition *p, double *out);
qlskum_status qlskum_partition_set_prim(qlskum_partition *p, const double *prim);
/* As qlskum_get_residual_history. */
qlskum_status qlskum_partition_residual_history(qlskum_partition *p, double *out, int max_rows, int *rows);
/* As qlskum_objective, the partitions' sums added in partition order. */
qlskum_status qlskum_partition_objective(qlskum_partition *p, double *cl, double *cd, double *cm,
                                         double *total_entropy);
/* Bytes the ghost exchanges of one iteration move, and the kernel launches so far. */
long long qlskum_partition_halo_bytes(const qlskum_partition *p);
long long qlskum_partition_launch_count(const qlskum_partition *p);

/* ------------------------------------------------- diagnostics and state files */

/* compute_enstrophy_mod.h:5-75 on the device (FP64): vorticity
 * du2/dx - du1/dy of every point by least squares over its full stencil, and
 * total = the sum of its squares.  vorticity (or NULL): double [n]. */
qlskum_status qlskum_enstrophy(qlskum_handle *h, double *total, double *vorticity);
/* stagnation_values_mod.h: the smallest and largest stagnation pressure
 * p0 = p (1 + (gamma-1)/2 M^2)^(gamma/(gamma-1)) over the points and their
 * 1-based point numbers (stagnation_pressure, :9-48), and the objective
 * J = sum (p0_inf - p0)^2 / (p0_inf^2 n) (objective_function_J, :51-80, with
 * the sum it accumulates and plen = n: the reference multiplies an
 * uninitialised total and never sets plen).  Any pointer may be NULL. */
qlskum_status qlskum_stagnation(qlskum_handle *h, double *p0_min, double *p0_max, int *i_min, int *i_max,
                                double *J);
/* restart.dat as restart_sol reads it (initial_conditions_mod.h:7-21): a line
 * "<n> <it> <res_old>", then per point "x y flag_1 mach entropy rho u1 u2 p"
 * (five columns restart_sol skips, then the state), 17 significant digits. */
qlskum_status qlskum_write_restart(qlskum_handle *h, const char *path);
/* Continue from a restart file: the state, the iteration count (the next
 * iteration is it + 1, q_lskum_mod.h:31-35) and res_old, which the run then
 * keeps instead of latching it at iterations 1-2 (fpi_solver_mod.h:139). */
qlskum_status qlskum_read_restart(qlskum_handle *h, const char *path);
/* print_primal_output (post_processing_mod.h:7-26) with one point per line
 * and the Mach number |u| / sqrt(gamma p / rho) (the reference writes no line
 * breaks and takes a square root of |u|^2 / c): "<n> <it> <res_old>", then
 * "x y flag_1 rho u1 u2 p mach entropy". */
qlskum_status qlskum_write_output(qlskum_handle *h, const char *path);

/* --------------------------------------------------- cloud files (no GPU needed) */

/* The partGrid text file main.cpp:16-58 reads.  qlskum_partgrid_read
 * allocates the cloud's arrays (release with qlskum_partgrid_free); errors
 * leave a message for qlskum_io_last_error(). */
qlskum_status qlskum_partgrid_read(const char *path, qlskum_cloud *out);
void qlskum_partgrid_free(qlskum_cloud *cloud);
qlskum_status qlskum_partgrid_write(const char *path, const qlskum_cloud *cloud);
const char *qlskum_io_last_error(void);
/* The sub-stencil quality check the reference leaves as a stub
 * (check_condition_number, generate_connectivity_mod.h:84-89): for every
 * point and direction (xpos, xneg, ypos, yneg) the reciprocal condition number
 * of its weighted 2x2 least-squares matrix, split as generate_connectivity
 * does (1 for a direction the point's class does not use, 0 below two
 * members); *n_bad = points with a used direction below min_rcond.
 * rcond: double [n][4] or NULL. */
qlskum_status qlskum_check_stencils(const qlskum_cloud *cloud, double power, double min_rcond, double *rcond,
                                    int *n_bad);

/* ------------------------------------------------------------ discrete adjoint */

/* Reverse mode of the iteration, for gradients of the force coefficients.
 * No counterpart in the reference (which has no adjoint); the functions
 * differentiate exactly what q_lskum / fpi_solver compute
 * (fpi_solver_mod.h:14-151).  On an FP64 handle that is the FP64 iteration.
 * On a MIXED handle the Mach / AoA / initial-state gradients differentiate
 * the mixed iteration along the mixed trajectory (FP32 edge work, FP64
 * stage update, as the forward); its wall-displacement gradients take the
 * FP64 reverse at the mixed trajectory's states.  qlskum_residual_forward
 * and qlskum_residual_vjp are FP64 on either handle.  Arrays are in the
 * cloud's point order. */
#define QLSKUM_OBJECTIVE_CL 0
#define QLSKUM_OBJECTIVE_CD 1
/* the stagnation-pressure loss J of qlskum_stagnation */
#define QLSKUM_OBJECTIVE_J 2

/* flux_res = R(prim): the local time step of prim (state_update_mod.h:448-496)
 * and the flux residual of the first stage (q_variables, q_derivatives, the
 * inner loop, flux_residual).  prim and flux_res double [n][4].  Leaves the
 * handle's own state alone. */
qlskum_status qlskum_residual_forward(qlskum_handle *h, const double *prim, double *flux_res);
/* bar_prim = (dR/dprim)^T bar_flux_res at prim: the vector-Jacobian product
 * of qlskum_residual_forward, for an autograd.Function's backward. */
qlskum_status qlskum_residual_vjp(qlskum_handle *h, const double *prim, const double *bar_flux_res,
                                  double *bar_prim);
/* The same pair on device buffers (double [n][4] in the cloud's point order,
 * 32-byte aligned), for callers whose state already lives on the GPU (a
 * PyTorch graph): the work is ordered after what `stream` (a cudaStream_t, or
 * NULL for the legacy stream) has queued, and the results are ready for what
 * `stream` queues next; no host copy, no host synchronisation. */
qlskum_status qlskum_residual_forward_device(qlskum_handle *h, const double *prim, double *flux_res, void *stream);
qlskum_status qlskum_residual_vjp_device(qlskum_handle *h, const double *prim, const double *bar_flux_res,
                                         double *bar_prim, void *stream);
/* The same VJP with the bars of the case parameters and of the geometry:
 * bar_params (double [2] or NULL) = d/dMach, d/dAoA of bar_flux_res . R,
 * which are zero (R reads no free-stream quantity; Mach and AoA enter the
 * iteration through the stage update's far-field state), and bar_wall_disp
 * (double [shape_points] or NULL) = its derivative w.r.t. the normal
 * displacement of each shape point (edge vectors, least-squares moments,
 * lengths and normals pulled back to the coordinates; the sub-stencil split
 * and min_dist held; unit weights, params.power 0, else
 * QLSKUM_ERR_UNSUPPORTED). */
qlskum_status qlskum_residual_vjp_full(qlskum_handle *h, const double *prim, const double *bar_flux_res,
                                      double *bar_prim, double *bar_params, double *bar_wall_disp);
/* Runs `iters` iterations (as qlskum_q_lskum would; the handle holds the
 * final state afterwards) from prim0 (double [n][4]) or, when prim0 is NULL,
 * from the free stream, keeping each iteration's state, then sweeps the
 * iterations in reverse.  J: the objective (Cl, Cd or the stagnation loss)
 * at the final state;
 * dJ_dmach, dJ_daoa (per degree): its exact derivatives through all `iters`
 * iterations (from the free stream these include the initial state's
 * dependence on Mach and AoA; a given prim0 is held fixed); dJ_dwall (or
 * NULL): double [shape_points], the derivative w.r.t. moving wall point m
 * along its unit normal, with the connectivity, the sub-stencil split and
 * min_dist held fixed (power 0 only); dJ_dprim0 (or NULL): double [n][4],
 * the derivative w.r.t. the initial state.  Device memory: 32 bytes per
 * point per kept state (every stride-th iteration, qlskum_set_adjoint_stride).
 * Each iteration's stage data is also kept where it fits in three quarters
 * of the free device memory (FP64 handles about 1.7 KB per point plus 384
 * bytes per edge slot for the edge ends' kept transcendentals, about 5.5 KB
 * per point at 10 neighbours; MIXED handles without dJ_dwall about 1 KB per
 * point; per iteration at 3 inner steps): with stride 1
 * for all `iters` iterations (the primal then runs as the recording
 * iteration, with the same state, prim_old and residual history as
 * qlskum_q_lskum, and the reverse recomputes nothing), with a larger stride
 * for one stride-long segment (each segment recomputed once); otherwise every
 * iteration's stage data is recomputed from its state during the reverse
 * sweep. */
qlskum_status qlskum_adjoint_gradient(qlskum_handle *h, int objective, int iters, const double *prim0, double *J,
                                      double *dJ_dmach, double *dJ_daoa, double *dJ_dwall, double *dJ_dprim0);
/* Keep the state of every stride-th iteration only (default 1: every
 * iteration); the reverse sweep recomputes the others segment by segment in
 * FP64, trading one extra forward iteration per stored one for device memory:
 * ceil(iters / stride) + stride states instead of iters. */
qlskum_status qlskum_set_adjoint_stride(qlskum_handle *h, int stride);
/* The steady-state adjoint at the handle's current state U (a converged
 * solution): lam = S_U^T lam + J_U iterated `adj_iters` times from 0, S the
 * map of one iteration, then dJ/dalpha = J_alpha + lam^T S_alpha.
 * adj_change (or NULL): max |lam_k - lam_{k-1}| / max |lam_k| of the last
 * adjoint iteration. */
qlskum_status qlskum_adjoint_fixed_point(qlskum_handle *h, int objective, int adj_iters, double *J,
                                         double *dJ_dmach, double *dJ_daoa, double *dJ_dwall, double *adj_change);

/* ------------------------------------------- stage update without allocation */

/* One SSPRK stage update (the arithmetic of qlskum_state_update) over device
 * buffers the caller owns, allocating nothing.  No counterpart in the
 * reference.  It is for callers that cannot allocate device memory while they
 * run: a host code that hands out every device buffer from its own
 * pre-allocated arena, or a time-stepping loop that must not take the device
 * synchronisation of cudaMalloc / cudaFree between its stages.
 *   flag_1 int32 [n], normals double [n][2] (16-byte aligned), prim (updated
 *   in place), prim_old and flux_res double [n][4] (32-byte aligned), all in
 *   the caller's point order; residual_out: device double[2] receiving the
 *   sum and the maximum of res_sqr over wall and interior points
 *   (state_update_mod.h:157-165).  stream: a cudaStream_t or NULL.
 * At most QLSKUM_NOALLOC_MAX_POINTS points; larger n returns
 * QLSKUM_ERR_INVALID, as are misaligned buffers (residual_out 8 bytes,
 * flag_1 4 bytes).  The per-block partial sums live in one 128 KiB static
 * device array that every GPU loading the library keeps until the process
 * exits.  The first call on a device looks up that array's address; make it
 * before any stream capture.  The address is kept for the process's life: a
 * cudaDeviceReset makes later calls on that device invalid.  Every call
 * reuses the array: calls that overlap on the GPU race and must be
 * serialised by the caller.  Launch errors are read with
 * cudaPeekAtLastError (the error state is left as it was). */
#define QLSKUM_NOALLOC_MAX_POINTS 2097152
qlskum_status qlskum_state_update_noalloc(int n, int rk, double mach, double aoa, const int *flag_1,
                                          const double *normals, double *prim, const double *prim_old,
                                          const double *flux_res, double *residual_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
