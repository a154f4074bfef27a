/* CPU restatement of the reference q-LSKUM solver (Pathlessbark8/C-_serial).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU library is checked
 * against, and the CPU baseline that the benchmark times beside it.  The
 * product (the CUDA library in c-_serial_gb300/) never links or calls it.
 *
 * Parity pin: every function here is compared against the reference's own
 * code compiled from its sources (oracle/build_ref.sh + oracle/ref_harness.cpp)
 * and against the golden fixtures in tests/golden/ written from that build.
 *
 * Conventions: 0-based point indices; point-major arrays ([n][4] for prim, q,
 * flux_res; [n][2][4] for dq, qm); input connectivity is 1-based as in the
 * reference's grid file.  All arithmetic is FP64 with the reference's own
 * operation order; build with -ffp-contract=off so that no FMA changes the
 * rounding sequence.
 */
#ifndef QLSKUM_ORACLE_H
#define QLSKUM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define QO_MAX_NBHS 20

typedef struct {
    int n;
    const double *x, *y;          /* [n] */
    const int *left, *right;      /* [n], 1-based (wall / outer only) */
    const int *flag_1, *flag_2;   /* [n] */
    const double *min_dist;       /* [n] */
    const int *nbhs;              /* [n] */
    const int *conn;              /* [n][20], 1-based */
} qo_cloud;

typedef struct {
    double mach, aoa, cfl, vl_const, power;
    int inner_iterations;
    int threads;                  /* OpenMP threads for the per-point loops (<=0: library default) */
} qo_params;

typedef struct qo_solver qo_solver;

qo_solver *qo_create(const qo_cloud *c, const qo_params *p);
void qo_destroy(qo_solver *s);

/* Module entry points (same meaning as the reference's functions). */
void qo_func_delta(qo_solver *s);
void qo_eval_q_variables(qo_solver *s);
void qo_eval_q_derivatives(qo_solver *s);
void qo_eval_q_inner_loop(qo_solver *s);
void qo_eval_update_innerloop(qo_solver *s);
void qo_cal_flux_residual(qo_solver *s);
void qo_state_update(qo_solver *s, int rk);
/* One pseudo-time iteration; returns res_new, writes residue / max_res. */
double qo_fpi_solver(qo_solver *s, int it, double *residue, double *max_res);
void qo_objective(qo_solver *s, double *cl, double *cd, double *cm, double *total_entropy);
double qo_enstrophy(qo_solver *s, double *vort);
void qo_stagnation(qo_solver *s, double *p_min, double *p_max, int *i_min, int *i_max, double *J);

/* Direct access to the state (point-major, 0-based). */
double *qo_prim(qo_solver *s);       /* [n][4] */
double *qo_prim_old(qo_solver *s);   /* [n][4] */
double *qo_q(qo_solver *s);          /* [n][4] */
double *qo_dq(qo_solver *s);         /* [n][2][4] */
double *qo_qm(qo_solver *s);         /* [n][2][4] */
double *qo_flux_res(qo_solver *s);   /* [n][4] */
double *qo_delta(qo_solver *s);      /* [n] */
double *qo_normals(qo_solver *s);    /* [n][2] */
double *qo_entropy(qo_solver *s);    /* [n] */
/* Sub-stencils: counts [n][4] (xpos, xneg, ypos, yneg) and lists [n][4][20] (1-based). */
const int *qo_sub_counts(qo_solver *s);
const int *qo_sub_lists(qo_solver *s);
double qo_sum_res_sqr(qo_solver *s);

/* Known-answer helpers. kind: 0 Gxp 1 Gxn 2 Gyp 3 Gyn 4 GxI 5 GxII 6 GxIII 7 GxIV */
void qo_flux(int kind, double nx, double ny, double u1, double u2, double rho, double pr, double G[4]);
void qo_qtilde_to_primitive(const double qt[4], double *u1, double *u2, double *rho, double *pr);

#ifdef __cplusplus
}
#endif
#endif
