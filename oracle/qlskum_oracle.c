/* CPU restatement of the reference q-LSKUM solver -- TEST INFRASTRUCTURE ONLY.
 *
 * This is the oracle: tests, the smoke check and the benchmark's CPU-baseline
 * leg call it as the checker; the product never does.  It restates, in plain
 * C, the reference's serial FP64 algorithm (Pathlessbark8/C-_serial), keeping
 * the reference's operation order so that results match its own build bit for
 * bit on the same machine (pinned by tests/test_oracle_pin.py against
 * oracle/_ref and tests/golden/).  Each function names the reference lines it
 * follows.  Per-point loops may run under OpenMP: every point's value is
 * computed independently and the residual sum is taken afterwards in point
 * order, so the thread count never changes a result.
 */
#include "qlskum_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NB QO_MAX_NBHS

struct qo_solver {
    int n;
    qo_params p;
    double theta, pi, rho_inf, pr_inf, gamma;
    double q_inf[4];
    /* cloud */
    double *x, *y, *min_dist, *nx, *ny;
    int *left, *right, *flag1, *flag2, *nbhs, *conn; /* conn 0-based [n][20] */
    int shape_points;
    /* sub-stencils, 0-based [n][4][20] and counts [n][4] */
    int *sub, *subn;
    int *sub1; /* 1-based copy for export */
    /* state */
    double *prim, *prim_old, *q, *dq, *qm, *temp, *flux_res, *delta, *entropy, *res_sqr, *nrm;
    double sum_res_sqr, max_res, res_old;
};

/* ------------------------------------------------------------------ setup */

/* point_normals_mod.h:17-55: wall/outer normal = rot90 of the left->right
 * chord, interior points (0, 1). */
static void compute_normals(qo_solver *s)
{
    for (int i = 0; i < s->n; i++) {
        if (s->flag1[i] == 0 || s->flag1[i] == 2) {
            int l = s->left[i] - 1, r = s->right[i] - 1;
            double lx = s->x[l], ly = s->y[l], mx = s->x[i], my = s->y[i], rx = s->x[r], ry = s->y[r];
            double nx1 = my - ly, nx2 = ry - my, ny1 = mx - lx, ny2 = rx - mx;
            double nx = 0.5 * (nx1 + nx2), ny = 0.5 * (ny1 + ny2);
            double det = sqrt(nx * nx + ny * ny);
            s->nx[i] = -nx / det;
            s->ny[i] = ny / det;
        } else {
            s->nx[i] = 0;
            s->ny[i] = 1;
        }
    }
}

/* generate_connectivity_mod.h:5-83 (interior), :91-153 (wall), :155-219
 * (outer), dispatched as at :221-249. */
static void generate_connectivity(qo_solver *s)
{
    for (int i = 0; i < s->n; i++) {
        double nx = s->nx[i], ny = s->ny[i];
        double xi = s->x[i], yi = s->y[i];
        double tx = ny, ty = -nx;
        int *c = s->subn + 4 * i;
        int *L = s->sub + (size_t)i * 4 * NB;
        c[0] = c[1] = c[2] = c[3] = 0;
        int f = s->flag1[i];
        for (int r = 0; r < s->nbhs[i]; r++) {
            int nbh = s->conn[i * NB + r];
            double delx = s->x[nbh] - xi, dely = s->y[nbh] - yi;
            double dels = delx * tx + dely * ty;
            double deln = delx * nx + dely * ny;
            if (dels <= 0.0) L[0 * NB + c[0]++] = nbh;
            if (dels >= 0.0) L[1 * NB + c[1]++] = nbh;
            if (f == 1) {
                if (deln <= 0.0) L[2 * NB + c[2]++] = nbh;
                if (deln >= 0.0) L[3 * NB + c[3]++] = nbh;
            } else if (f == 0) {
                L[3 * NB + c[3]++] = nbh;
            } else {
                L[2 * NB + c[2]++] = nbh;
            }
        }
    }
}

qo_solver *qo_create(const qo_cloud *c, const qo_params *p)
{
    qo_solver *s = (qo_solver *)calloc(1, sizeof(qo_solver));
    int n = c->n;
    s->n = n;
    s->p = *p;
#ifdef _OPENMP
    if (p->threads > 0) omp_set_num_threads(p->threads);
#endif
    /* parameter_mod.h:4-30 */
    s->pi = 4 * atan(1.0);
    s->rho_inf = 1.0;
    s->pr_inf = 1.0 / 1.4;
    s->gamma = 1.4;
    s->theta = p->aoa * s->pi / 180;
    s->q_inf[0] = s->rho_inf;
    s->q_inf[1] = p->mach * cos(s->theta);
    s->q_inf[2] = p->mach * sin(s->theta);
    s->q_inf[3] = s->pr_inf;

    s->x = (double *)malloc(sizeof(double) * n);
    s->y = (double *)malloc(sizeof(double) * n);
    s->min_dist = (double *)malloc(sizeof(double) * n);
    s->nx = (double *)malloc(sizeof(double) * n);
    s->ny = (double *)malloc(sizeof(double) * n);
    s->left = (int *)malloc(sizeof(int) * n);
    s->right = (int *)malloc(sizeof(int) * n);
    s->flag1 = (int *)malloc(sizeof(int) * n);
    s->flag2 = (int *)malloc(sizeof(int) * n);
    s->nbhs = (int *)malloc(sizeof(int) * n);
    s->conn = (int *)malloc(sizeof(int) * (size_t)n * NB);
    memcpy(s->x, c->x, sizeof(double) * n);
    memcpy(s->y, c->y, sizeof(double) * n);
    memcpy(s->min_dist, c->min_dist, sizeof(double) * n);
    memcpy(s->left, c->left, sizeof(int) * n);
    memcpy(s->right, c->right, sizeof(int) * n);
    memcpy(s->flag1, c->flag_1, sizeof(int) * n);
    memcpy(s->flag2, c->flag_2, sizeof(int) * n);
    memcpy(s->nbhs, c->nbhs, sizeof(int) * n);
    for (size_t k = 0; k < (size_t)n * NB; k++) s->conn[k] = c->conn[k] - 1;
    s->shape_points = 0;
    for (int i = 0; i < n; i++)
        if (s->flag2[i] > 0) s->shape_points++;

    s->sub = (int *)calloc((size_t)n * 4 * NB, sizeof(int));
    s->sub1 = (int *)calloc((size_t)n * 4 * NB, sizeof(int));
    s->subn = (int *)calloc((size_t)n * 4, sizeof(int));
    s->prim = (double *)calloc((size_t)n * 4, sizeof(double));
    s->prim_old = (double *)calloc((size_t)n * 4, sizeof(double));
    s->q = (double *)calloc((size_t)n * 4, sizeof(double));
    s->dq = (double *)calloc((size_t)n * 8, sizeof(double));
    s->qm = (double *)calloc((size_t)n * 8, sizeof(double));
    s->temp = (double *)calloc((size_t)n * 8, sizeof(double));
    s->flux_res = (double *)calloc((size_t)n * 4, sizeof(double));
    s->delta = (double *)calloc((size_t)n, sizeof(double));
    s->entropy = (double *)calloc((size_t)n, sizeof(double));
    s->res_sqr = (double *)calloc((size_t)n, sizeof(double));
    s->nrm = (double *)calloc((size_t)n * 2, sizeof(double));

    compute_normals(s);
    generate_connectivity(s);
    for (size_t k = 0; k < (size_t)n * 4 * NB; k++) s->sub1[k] = s->sub[k] + 1;
    for (int i = 0; i < n; i++) { s->nrm[2 * i] = s->nx[i]; s->nrm[2 * i + 1] = s->ny[i]; }
    /* initial_conditions_mod.h:23-37: uniform free stream */
    for (int k = 0; k < n; k++)
        for (int r = 0; r < 4; r++) s->prim[4 * k + r] = s->q_inf[r];
    return s;
}

void qo_destroy(qo_solver *s)
{
    if (!s) return;
    free(s->x); free(s->y); free(s->min_dist); free(s->nx); free(s->ny);
    free(s->left); free(s->right); free(s->flag1); free(s->flag2); free(s->nbhs); free(s->conn);
    free(s->sub); free(s->sub1); free(s->subn);
    free(s->prim); free(s->prim_old); free(s->q); free(s->dq); free(s->qm); free(s->temp);
    free(s->flux_res); free(s->delta); free(s->entropy); free(s->res_sqr); free(s->nrm);
    free(s);
}

/* ------------------------------------------------------- q and gradients */

/* q_variables_mod.h:9-34 */
void qo_eval_q_variables(qo_solver *s)
{
    int n = s->n;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; k++) {
        const double *P = s->prim + 4 * k;
        double rho = P[0], u1 = P[1], u2 = P[2], pr = P[3];
        double beta = 0.5 * rho / pr;
        double *Q = s->q + 4 * k;
        Q[0] = log(rho) + (log(beta) * 2.5) - beta * (u1 * u1 + u2 * u2);
        double two_times_beta = 2.0 * beta;
        Q[1] = two_times_beta * u1;
        Q[2] = two_times_beta * u2;
        Q[3] = -two_times_beta;
    }
}

/* q_variables_mod.h:36-118: neighbour min/max of q into qm, least-squares
 * gradient over the full connectivity with weights dist^power. */
void qo_eval_q_derivatives(qo_solver *s)
{
    int n = s->n;
    double power = s->p.power;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        double xi = s->x[i], yi = s->y[i];
        double sxx = 0., syy = 0., sxy = 0.;
        const double *Qi = s->q + 4 * i;
        double *qmax = s->qm + 8 * i, *qmin = qmax + 4;
        double sdx[4] = {0, 0, 0, 0}, sdy[4] = {0, 0, 0, 0};
        for (int r = 0; r < 4; r++) { qmax[r] = Qi[r]; qmin[r] = Qi[r]; }
        for (int kk = 0; kk < s->nbhs[i]; kk++) {
            int nbh = s->conn[i * NB + kk];
            const double *Qk = s->q + 4 * nbh;
            for (int r = 0; r < 4; r++) {
                if (Qk[r] > qmax[r]) qmax[r] = Qk[r];
                if (Qk[r] < qmin[r]) qmin[r] = Qk[r];
            }
            double delx = s->x[nbh] - xi, dely = s->y[nbh] - yi;
            double dist = sqrt(delx * delx + dely * dely);
            double w = pow(dist, power);
            sxx = sxx + delx * delx * w;
            syy = syy + dely * dely * w;
            sxy = sxy + delx * dely * w;
            for (int r = 0; r < 4; r++) {
                sdx[r] = sdx[r] + w * delx * (Qk[r] - Qi[r]);
                sdy[r] = sdy[r] + w * dely * (Qk[r] - Qi[r]);
            }
        }
        double det = sxx * syy - sxy * sxy;
        double one_by_det = 1.0 / det;
        double *D = s->dq + 8 * i;
        for (int r = 0; r < 4; r++) {
            D[r] = (sdx[r] * syy - sdy[r] * sxy) * one_by_det;
            D[4 + r] = (sdy[r] * sxx - sdx[r] * sxy) * one_by_det;
        }
    }
}

/* q_variables_mod.h:120-213: defect-corrected gradient, q shifted half-way
 * along each edge on both ends, written to temp. */
void qo_eval_q_inner_loop(qo_solver *s)
{
    int n = s->n;
    double power = s->p.power;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        double xi = s->x[i], yi = s->y[i];
        double sxx = 0., syy = 0., sxy = 0.;
        double sdx[4] = {0, 0, 0, 0}, sdy[4] = {0, 0, 0, 0};
        const double *Qi = s->q + 4 * i, *Di = s->dq + 8 * i;
        for (int kk = 0; kk < s->nbhs[i]; kk++) {
            int nbh = s->conn[i * NB + kk];
            const double *Qk = s->q + 4 * nbh, *Dk = s->dq + 8 * nbh;
            double delx = s->x[nbh] - xi, dely = s->y[nbh] - yi;
            double dist = sqrt(delx * delx + dely * dely);
            double w = pow(dist, power);
            sxx = sxx + delx * delx * w;
            syy = syy + dely * dely * w;
            sxy = sxy + delx * dely * w;
            for (int r = 0; r < 4; r++) {
                double t1 = Qi[r] - 0.5 * (delx * Di[r] + dely * Di[4 + r]);
                double t2 = Qk[r] - 0.5 * (delx * Dk[r] + dely * Dk[4 + r]);
                sdx[r] = sdx[r] + (w * delx * (t2 - t1));
                sdy[r] = sdy[r] + (w * dely * (t2 - t1));
            }
        }
        double det = sxx * syy - sxy * sxy;
        double one_by_det = 1.0 / det;
        double *T = s->temp + 8 * i;
        for (int r = 0; r < 4; r++) {
            T[r] = one_by_det * (sdx[r] * syy - sdy[r] * sxy);
            T[4 + r] = one_by_det * (sdy[r] * sxx - sdx[r] * sxy);
        }
    }
}

/* q_variables_mod.h:215-228 */
void qo_eval_update_innerloop(qo_solver *s)
{
    memcpy(s->dq, s->temp, sizeof(double) * 8 * (size_t)s->n);
}

/* q_variables_mod.h:230-253 */
void qo_qtilde_to_primitive(const double qt[4], double *u1, double *u2, double *rho, double *pr)
{
    double q1 = qt[0], q2 = qt[1], q3 = qt[2], q4 = qt[3];
    double beta = -q4 * 0.5;
    double temp = 0.5 / beta;
    *u1 = q2 * temp;
    *u2 = q3 * temp;
    double temp1 = q1 + beta * (*u1 * *u1 + *u2 * *u2);
    double temp2 = temp1 - (log(beta) / (1.4 - 1));
    *rho = exp(temp2);
    *pr = *rho * temp;
}

/* ----------------------------------------------------------- split fluxes */

/* split_fluxes_mod.h:6-164 (kind 0..3) and quadrant_fluxes_mod.h:6-211
 * (kind 4..7).  Components are in the (t, n) frame of the point. */
void qo_flux(int kind, double nx, double ny, double u1, double u2, double rho, double pr, double G[4])
{
    const double pi = 4 * atan(1.0);
    double tx = ny, ty = -nx;
    double ut = u1 * tx + u2 * ty;
    double un = u1 * nx + u2 * ny;
    double beta = 0.5 * rho / pr;
    double pr_by_rho, u_sqr, temp1, temp2, temp3, temp4;
    if (kind <= 1) {
        double S1 = ut * sqrt(beta);
        double B1 = 0.5 * exp(-S1 * S1) / sqrt(pi * beta);
        pr_by_rho = pr / rho;
        u_sqr = ut * ut + un * un;
        if (kind == 0) {
            double A1pos = 0.5 * (1.0 + erf(S1));
            G[0] = rho * (ut * A1pos + B1);
            temp1 = pr_by_rho + ut * ut;
            temp2 = temp1 * A1pos + ut * B1;
            G[1] = rho * temp2;
            temp1 = ut * un * A1pos + un * B1;
            G[2] = rho * temp1;
            temp1 = (7.0 * pr_by_rho) + u_sqr;
            temp2 = 0.5 * ut * temp1 * A1pos;
            temp1 = (6.0 * pr_by_rho) + u_sqr;
            G[3] = rho * (temp2 + 0.5 * temp1 * B1);
        } else {
            double A1neg = 0.5 * (1.0 - erf(S1));
            G[0] = rho * (ut * A1neg - B1);
            temp1 = pr_by_rho + ut * ut;
            temp2 = temp1 * A1neg - ut * B1;
            G[1] = rho * temp2;
            temp1 = ut * un * A1neg - un * B1;
            G[2] = rho * temp1;
            temp1 = (7.0 * pr_by_rho) + u_sqr;
            temp2 = 0.5 * ut * temp1 * A1neg;
            temp1 = (6.0 * pr_by_rho) + u_sqr;
            G[3] = rho * (temp2 - 0.5 * temp1 * B1);
        }
        return;
    }
    if (kind <= 3) {
        double S2 = un * sqrt(beta);
        double B2 = 0.5 * exp(-S2 * S2) / sqrt(pi * beta);
        pr_by_rho = pr / rho;
        u_sqr = ut * ut + un * un;
        if (kind == 2) {
            double A2pos = 0.5 * (1.0 + erf(S2));
            G[0] = rho * (un * A2pos + B2);
            temp1 = pr_by_rho + un * un;
            temp2 = temp1 * A2pos + un * B2;
            G[2] = rho * temp2;
            temp1 = ut * un * A2pos + ut * B2;
            G[1] = rho * temp1;
            temp1 = (7.0 * pr_by_rho) + u_sqr;
            temp2 = 0.5 * un * temp1 * A2pos;
            temp1 = (6.0 * pr_by_rho) + u_sqr;
            G[3] = rho * (temp2 + 0.5 * temp1 * B2);
        } else {
            double A2neg = 0.5 * (1.0 - erf(S2));
            G[0] = rho * (un * A2neg - B2);
            temp1 = pr_by_rho + un * un;
            temp2 = temp1 * A2neg - un * B2;
            G[2] = rho * temp2;
            temp1 = ut * un * A2neg - ut * B2;
            G[1] = rho * temp1;
            temp1 = (7.0 * pr_by_rho) + u_sqr;
            temp2 = 0.5 * un * temp1 * A2neg;
            temp1 = (6.0 * pr_by_rho) + u_sqr;
            G[3] = rho * (temp2 - 0.5 * temp1 * B2);
        }
        return;
    }
    /* quadrant fluxes: I (A1-, A2-), II (A1+, A2-), III (A1+, A2+), IV (A1-, A2+) */
    double S1 = ut * sqrt(beta);
    double S2 = un * sqrt(beta);
    double B1 = 0.5 * exp(-S1 * S1) / sqrt(pi * beta);
    double B2 = 0.5 * exp(-S2 * S2) / sqrt(pi * beta);
    int t_pos = (kind == 5 || kind == 6);
    int n_pos = (kind == 6 || kind == 7);
    double A1 = t_pos ? 0.5 * (1.0 + erf(S1)) : 0.5 * (1.0 - erf(S1));
    double A2 = n_pos ? 0.5 * (1.0 + erf(S2)) : 0.5 * (1.0 - erf(S2));
    pr_by_rho = pr / rho;
    u_sqr = ut * ut + un * un;
    double f1 = t_pos ? ut * A1 + B1 : ut * A1 - B1; /* recurring t-half-range factor */
    G[0] = rho * A2 * f1;
    temp1 = pr_by_rho + ut * ut;
    temp2 = t_pos ? temp1 * A1 + ut * B1 : temp1 * A1 - ut * B1;
    G[1] = rho * A2 * temp2;
    temp1 = f1;
    temp2 = n_pos ? un * A2 + B2 : un * A2 - B2;
    G[2] = rho * temp1 * temp2;
    temp1 = (7.0 * pr_by_rho) + u_sqr;
    temp2 = 0.5 * ut * temp1 * A1;
    temp1 = (6.0 * pr_by_rho) + u_sqr;
    temp3 = 0.5 * B1 * temp1;
    temp1 = f1;
    temp4 = 0.5 * rho * un * B2 * temp1;
    if (t_pos) {
        G[3] = n_pos ? rho * A2 * (temp2 + temp3) + temp4 : rho * A2 * (temp2 + temp3) - temp4;
    } else {
        G[3] = n_pos ? rho * A2 * (temp2 - temp3) + temp4 : rho * A2 * (temp2 - temp3) - temp4;
    }
}

/* ------------------------------------------------------------- limiter */

/* limiters_mod.h:55-104: Venkatakrishnan limiter of qtilde about point k. */
static void venkat_limiter(const qo_solver *s, const double qt[4], double phi[4], int k)
{
    for (int r = 0; r < 4; r++) {
        double q = s->q[4 * k + r];
        double del_neg = qt[r] - q, del_pos;
        if (fabs(del_neg) <= 10e-6) {
            phi[r] = 1.0;
        } else if (fabs(del_neg) > 10e-6) {
            if (del_neg > 0) del_pos = s->qm[8 * k + r] - q;
            else del_pos = s->qm[8 * k + 4 + r] - q;
            double epsi = s->p.vl_const * s->min_dist[k];
            epsi = pow(epsi, 3);
            double num = (del_pos * del_pos) + (epsi * epsi);
            num = num * del_neg + 2.0 * del_neg * del_neg * del_pos;
            double den = del_pos * del_pos + 2.0 * del_neg * del_neg;
            den = den + del_neg * del_pos + epsi * epsi;
            den = den * del_neg;
            double temp = num / den;
            phi[r] = temp < 1 ? temp : 1;
        }
    }
}

/* --------------------------------------------------------- flux residual */

/* One directional flux derivative: interior_fluxes_mod.h:12-423,
 * wall_fluxes_mod.h:11-285, outer_fluxes_mod.h:11-287 share this body and
 * differ only in the sub-stencil walked, the split flux evaluated and
 * whether the x row (yrow = 0) or the y row (yrow = 1) of the 2x2 solve is
 * used. */
static void dir_flux(const qo_solver *s, int i, int list, int kind, int yrow, double G[4])
{
    double power = s->p.power;
    double sxx = 0.0, syy = 0.0, sxy = 0.0;
    double sdf_x[4] = {0, 0, 0, 0}, sdf_y[4] = {0, 0, 0, 0};
    double xi = s->x[i], yi = s->y[i], nx = s->nx[i], ny = s->ny[i];
    double tx = ny, ty = -nx;
    double qti[4], qtk[4], phi_i[4] = {0, 0, 0, 0}, phi_k[4] = {0, 0, 0, 0}, Gi[4], Gk[4];
    const double *Qi = s->q + 4 * i, *Di = s->dq + 8 * i;
    int cnt = s->subn[4 * i + list];
    const int *L = s->sub + (size_t)i * 4 * NB + list * NB;
    for (int j = 0; j < cnt; j++) {
        int k = L[j];
        const double *Qk = s->q + 4 * k, *Dk = s->dq + 8 * k;
        double delx = s->x[k] - xi, dely = s->y[k] - yi;
        double dels = delx * tx + dely * ty;
        double deln = delx * nx + dely * ny;
        double dist = sqrt(dels * dels + deln * deln);
        double w = pow(dist, power);
        double dels_w = dels * w, deln_w = deln * w;
        sxx = sxx + dels * dels_w;
        syy = syy + deln * deln_w;
        sxy = sxy + dels * deln_w;
        for (int r = 0; r < 4; r++) {
            qti[r] = Qi[r] - 0.5 * (delx * Di[r] + dely * Di[4 + r]);
            qtk[r] = Qk[r] - 0.5 * (delx * Dk[r] + dely * Dk[4 + r]);
        }
        venkat_limiter(s, qti, phi_i, i);
        venkat_limiter(s, qtk, phi_k, k);
        for (int r = 0; r < 4; r++) {
            qti[r] = Qi[r] - 0.5 * phi_i[r] * (delx * Di[r] + dely * Di[4 + r]);
            qtk[r] = Qk[r] - 0.5 * phi_k[r] * (delx * Dk[r] + dely * Dk[4 + r]);
        }
        double u1, u2, rho, pr;
        qo_qtilde_to_primitive(qti, &u1, &u2, &rho, &pr);
        qo_flux(kind, nx, ny, u1, u2, rho, pr, Gi);
        qo_qtilde_to_primitive(qtk, &u1, &u2, &rho, &pr);
        qo_flux(kind, nx, ny, u1, u2, rho, pr, Gk);
        for (int r = 0; r < 4; r++) {
            sdf_x[r] = sdf_x[r] + (Gk[r] - Gi[r]) * dels_w;
            sdf_y[r] = sdf_y[r] + (Gk[r] - Gi[r]) * deln_w;
        }
    }
    double det = sxx * syy - sxy * sxy;
    double one_by_det = 1.0 / det;
    for (int r = 0; r < 4; r++)
        G[r] = yrow ? (sdf_y[r] * sxx - sdf_x[r] * sxy) * one_by_det
                    : (sdf_x[r] * syy - sdf_y[r] * sxy) * one_by_det;
}

/* flux_residual_mod.h:10-89 */
void qo_cal_flux_residual(qo_solver *s)
{
    int n = s->n;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        double Gxp[4], Gxn[4], Gyp[4], Gyn[4];
        double *F = s->flux_res + 4 * i;
        if (s->flag1[i] == 0) {
            dir_flux(s, i, 0, 5, 0, Gxp); /* wall_dGx_pos: GxII */
            dir_flux(s, i, 1, 4, 0, Gxn); /* wall_dGx_neg: GxI  */
            dir_flux(s, i, 3, 3, 1, Gyn); /* wall_dGy_neg: Gyn  */
            for (int j = 0; j < 4; j++) F[j] = (2.0 * s->delta[i]) * (Gxp[j] + Gxn[j] + Gyn[j]);
        } else if (s->flag1[i] == 1) {
            dir_flux(s, i, 0, 0, 0, Gxp);
            dir_flux(s, i, 1, 1, 0, Gxn);
            dir_flux(s, i, 2, 2, 1, Gyp);
            dir_flux(s, i, 3, 3, 1, Gyn);
            for (int j = 0; j < 4; j++) F[j] = s->delta[i] * (Gxp[j] + Gxn[j] + Gyp[j] + Gyn[j]);
        } else {
            dir_flux(s, i, 0, 6, 0, Gxp); /* outer_dGx_pos: GxIII */
            dir_flux(s, i, 1, 7, 0, Gxn); /* outer_dGx_neg: GxIV  */
            dir_flux(s, i, 2, 2, 1, Gyp); /* outer_dGy_pos: Gyp   */
            for (int j = 0; j < 4; j++) F[j] = s->delta[i] * (Gxp[j] + Gxn[j] + Gyp[j]);
        }
    }
}

/* ---------------------------------------------------------- state update */

/* state_update_mod.h:18-33 */
static void primitive_to_conserved(const double *prim, double nx, double ny, double U[4])
{
    double rho = prim[0];
    U[0] = rho;
    double temp1 = rho * prim[1];
    double temp2 = rho * prim[2];
    U[3] = 2.5 * prim[3] + 0.5 * (temp1 * temp1 + temp2 * temp2) / rho;
    U[1] = temp1 * ny - temp2 * nx;
    U[2] = temp1 * nx + temp2 * ny;
}

/* state_update_mod.h:35-90: kinetic far-field state, half-range mix of the
 * free stream and the point's own state across the outward normal. */
static void conserved_vector_Ubar(const qo_solver *s, const double *prim, double Ubar[4], double nx, double ny)
{
    const double gamma_new = s->gamma, rho_inf = s->rho_inf, pr_inf = s->pr_inf, pi = s->pi;
    double u1_inf = s->q_inf[1], u2_inf = s->q_inf[2];
    double tx = ny, ty = -nx;
    double u1_inf_rot = u1_inf * tx + u2_inf * ty;
    double u2_inf_rot = u1_inf * nx + u2_inf * ny;
    double temp1 = (u1_inf_rot * u1_inf_rot + u2_inf_rot * u2_inf_rot);
    double e_inf = pr_inf / (rho_inf * (gamma_new - 1.0)) + 0.5 * (temp1);
    double beta = (0.5 * rho_inf) / pr_inf;
    double S2 = u2_inf_rot * sqrt(beta);
    double B2_inf = exp(-S2 * S2) / (2.0 * sqrt(pi * beta));
    double A2n_inf = 0.5 * (1.0 - erf(S2));
    double rho = prim[0], u1 = prim[1], u2 = prim[2], pr = prim[3];
    double u1_rot = u1 * tx + u2 * ty;
    double u2_rot = u1 * nx + u2 * ny;
    temp1 = (u1_rot * u1_rot + u2_rot * u2_rot);
    double e = pr / (rho * (gamma_new - 1.0)) + 0.5 * (temp1);
    beta = (rho) / (2.0 * pr);
    S2 = u2_rot * sqrt(beta);
    double B2 = exp(-S2 * S2) / (2.0 * sqrt(pi * beta));
    double A2p = 0.5 * (1.0 + erf(S2));
    Ubar[0] = (rho_inf * A2n_inf) + (rho * A2p);
    Ubar[1] = (rho_inf * u1_inf_rot * A2n_inf) + (rho * u1_rot * A2p);
    temp1 = rho_inf * (u2_inf_rot * A2n_inf - B2_inf);
    double temp2 = rho * (u2_rot * A2p + B2);
    Ubar[2] = temp1 + temp2;
    temp1 = (rho_inf * A2n_inf * e_inf - 0.5 * rho_inf * u2_inf_rot * B2_inf);
    temp2 = (rho * A2p * e + 0.5 * rho * u2_rot * B2);
    Ubar[3] = temp1 + temp2;
}

/* state_update_mod.h:92-283: one SSPRK stage; the residual sum and maximum
 * run over wall and interior points in point order (:157-165, :215-223). */
void qo_state_update(qo_solver *s, int rk)
{
    int n = s->n;
    const double obt = 1.0 / 3.0, tbt = 2.0 / 3.0, euler = 1.0;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; k++) {
        double U[4], U_old[4];
        double nx = s->nx[k], ny = s->ny[k];
        const double *F = s->flux_res + 4 * k;
        double *P = s->prim + 4 * k;
        int f = s->flag1[k];
        if (f == 2) {
            conserved_vector_Ubar(s, P, U, nx, ny);
            conserved_vector_Ubar(s, s->prim_old + 4 * k, U_old, nx, ny);
        } else {
            primitive_to_conserved(P, nx, ny, U);
            primitive_to_conserved(s->prim_old + 4 * k, nx, ny, U_old);
        }
        double temp = U[0];
        if (rk != 3) {
            for (int j = 0; j < 4; j++) U[j] = U[j] - (0.5 * euler * F[j]);
        } else {
            for (int j = 0; j < 4; j++) U[j] = tbt * U_old[j] + obt * (U[j] - 0.5 * F[j]);
        }
        if (f == 0) U[2] = 0.;
        double U2_rot = U[1], U3_rot = U[2];
        U[1] = U2_rot * ny + U3_rot * nx;
        U[2] = U3_rot * ny - U2_rot * nx;
        s->res_sqr[k] = (f == 2) ? 0.0 : (U[0] - temp) * (U[0] - temp);
        P[0] = U[0];
        temp = 1.0 / U[0];
        P[1] = U[1] * temp;
        P[2] = U[2] * temp;
        P[3] = 0.4 * U[3] - (0.2 * temp) * (U[1] * U[1] + U[2] * U[2]);
    }
    double sum = 0.0, mx = 0.0;
    for (int k = 0; k < n; k++) {
        if (s->flag1[k] == 2) continue;
        double r = s->res_sqr[k];
        if (r > mx) mx = r;
        sum = sum + r;
    }
    s->sum_res_sqr = sum;
    s->max_res = mx;
}

/* state_update_mod.h:448-496: local time step
 * delta_i = min(1, min_k CFL |r_k - r_i| / (|u_k| + 3 sqrt(p_k / rho_k))). */
void qo_func_delta(qo_solver *s)
{
    int n = s->n;
    double CFL = s->p.cfl;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        double min_delt = 1.0;
        for (int r = 0; r < s->nbhs[i]; r++) {
            int k = s->conn[i * NB + r];
            const double *P = s->prim + 4 * k;
            double rho = P[0], u1 = P[1], u2 = P[2], pr = P[3];
            double x_i = s->x[i], y_i = s->y[i], x_k = s->x[k], y_k = s->y[k];
            double dist = (x_k - x_i) * (x_k - x_i) + (y_k - y_i) * (y_k - y_i);
            dist = sqrt(dist);
            double mod_u = sqrt(u1 * u1 + u2 * u2);
            double delta_t = dist / (mod_u + 3.0 * sqrt(pr / rho));
            delta_t = CFL * delta_t;
            if (min_delt > delta_t) min_delt = delta_t;
        }
        s->delta[i] = min_delt;
    }
}

/* fpi_solver_mod.h:14-151 */
double qo_fpi_solver(qo_solver *s, int it, double *residue, double *max_res)
{
    memcpy(s->prim_old, s->prim, sizeof(double) * 4 * (size_t)s->n);
    qo_func_delta(s);
    for (int rk = 1; rk <= 4; rk++) {
        qo_eval_q_variables(s);
        qo_eval_q_derivatives(s);
        for (int i = 1; i <= s->p.inner_iterations; i++) {
            qo_eval_q_inner_loop(s);
            qo_eval_update_innerloop(s);
        }
        qo_cal_flux_residual(s);
        qo_state_update(s, rk);
    }
    double res_new = sqrt(s->sum_res_sqr) / s->n;
    double r;
    if (it <= 2) {
        s->res_old = res_new;
        r = 0;
    } else {
        r = log10(res_new / s->res_old);
    }
    if (residue) *residue = r;
    if (max_res) *max_res = s->max_res;
    return res_new;
}

/* compute_force_coeffs_mod.h:7-69 (points 1..shape_points, shape 1) and
 * compute_entropy_mod.h:5-24 (the total re-summed in point order). */
void qo_objective(qo_solver *s, double *cl, double *cd, double *cm, double *total_entropy)
{
    double H = 0, V = 0, pitch_mom = 0;
    double temp = 0.5 * s->rho_inf * s->p.mach * s->p.mach;
    for (int m = 0; m < s->shape_points; m++) {
        int r = s->right[m] - 1, l = s->left[m] - 1;
        double lx = s->x[l], ly = s->y[l], mx = s->x[m], my = s->y[m], rx = s->x[r], ry = s->y[r];
        double ds1 = pow((mx - lx), 2) + pow((my - ly), 2);
        ds1 = sqrt(ds1);
        double ds2 = pow((rx - mx), 2) + pow((ry - my), 2);
        ds2 = sqrt(ds2);
        double ds = 0.5 * (ds1 + ds2);
        double nx = s->nx[m], ny = s->ny[m];
        double cp = s->prim[4 * m + 3] - s->pr_inf;
        cp = -cp / temp;
        H = H + cp * nx * ds;
        V = V + cp * ny * ds;
        pitch_mom = pitch_mom + (-cp * ny * ds * (mx - 0.25) + cp * nx * ds * (my));
    }
    *cl = V * cos(s->theta) - H * sin(s->theta);
    *cd = H * cos(s->theta) + V * sin(s->theta);
    *cm = pitch_mom;
    double temp2 = log(s->pr_inf), tot = 0.0;
    for (int k = 0; k < s->n; k++) {
        double temp1 = pow((s->prim[4 * k]), s->gamma);
        temp1 = s->prim[4 * k + 3] / temp1;
        temp1 = log(temp1);
        s->entropy[k] = fabs(temp1 - temp2);
        tot = tot + s->entropy[k];
    }
    *total_entropy = tot;
}

/* compute_enstrophy_mod.h:5-75: vorticity du2/dx - du1/dy by weighted least
 * squares over the full stencil; vort [n] (may be NULL); returns the sum of
 * its squares in point order. */
double qo_enstrophy(qo_solver *s, double *vort)
{
    double total = 0.0;
    for (int i = 0; i < s->n; i++) {
        double x_i = s->x[i], y_i = s->y[i];
        double sum_delx_sqr = 0., sum_dely_sqr = 0., sum_delx_dely = 0.;
        double sum_delx_delu1 = 0., sum_dely_delu1 = 0., sum_delx_delu2 = 0., sum_dely_delu2 = 0.;
        for (int k = 0; k < s->nbhs[i]; k++) {
            int nbh = s->conn[i * NB + k];
            double delx = s->x[nbh] - x_i, dely = s->y[nbh] - y_i;
            double dist = sqrt(delx * delx + dely * dely);
            double weights = pow(dist, s->p.power);
            sum_delx_sqr = sum_delx_sqr + delx * delx * weights;
            sum_dely_sqr = sum_dely_sqr + dely * dely * weights;
            sum_delx_dely = sum_delx_dely + delx * dely * weights;
            sum_delx_delu1 = sum_delx_delu1 + weights * delx * (s->prim[4 * nbh + 1] - s->prim[4 * i + 1]);
            sum_delx_delu2 = sum_delx_delu2 + weights * delx * (s->prim[4 * nbh + 2] - s->prim[4 * i + 2]);
            sum_dely_delu1 = sum_dely_delu1 + weights * dely * (s->prim[4 * nbh + 1] - s->prim[4 * i + 1]);
            sum_dely_delu2 = sum_dely_delu2 + weights * dely * (s->prim[4 * nbh + 2] - s->prim[4 * i + 2]);
        }
        double det = sum_delx_sqr * sum_dely_sqr - sum_delx_dely * sum_delx_dely;
        double one_by_det = 1.0 / det;
        double du2_dx = (sum_delx_delu2 * sum_dely_sqr - sum_dely_delu2 * sum_delx_dely) * one_by_det;
        double du1_dy = (sum_dely_delu1 * sum_delx_sqr - sum_delx_delu1 * sum_delx_dely) * one_by_det;
        double temp = du2_dx - du1_dy;
        if (vort) vort[i] = temp;
        total = total + temp * temp;
    }
    return total;
}

/* stagnation_values_mod.h:9-48 (extremes of p0 and their 1-based point
 * numbers) and :51-80 (J, with the sum it accumulates and plen = n). */
void qo_stagnation(qo_solver *s, double *p_min, double *p_max, int *i_min, int *i_max, double *J)
{
    double g = s->gamma, gammaPower = g / (g - 1);
    double p0_inf = s->pr_inf * (pow((1 + ((g - 1) / 2) * s->p.mach * s->p.mach), gammaPower));
    double pMin = 0, pMax = 0, p0_sum = 0.0;
    int indexMin = 1, indexMax = 1;
    for (int i = 0; i < s->n; i++) {
        const double *prim = s->prim + 4 * i;
        double angle = sqrt(g * prim[3] / prim[0]);
        double mach_t = sqrt(pow(prim[1], 2) + pow(prim[2], 2)) / angle;
        double p0 = prim[3] * (pow((1 + ((g - 1) / 2) * mach_t * mach_t), gammaPower));
        if (i == 0) {
            pMin = p0;
            pMax = p0;
            indexMin = indexMax = 1;
        } else if (p0 < pMin) {
            pMin = p0;
            indexMin = i + 1;
        } else if (p0 > pMax) {
            pMax = p0;
            indexMax = i + 1;
        }
        p0_sum = p0_sum + pow((p0_inf - p0), 2);
    }
    *p_min = pMin;
    *p_max = pMax;
    *i_min = indexMin;
    *i_max = indexMax;
    *J = p0_sum * (1 / (pow(p0_inf, 2) * s->n));
}

double *qo_prim(qo_solver *s) { return s->prim; }
double *qo_prim_old(qo_solver *s) { return s->prim_old; }
double *qo_q(qo_solver *s) { return s->q; }
double *qo_dq(qo_solver *s) { return s->dq; }
double *qo_qm(qo_solver *s) { return s->qm; }
double *qo_flux_res(qo_solver *s) { return s->flux_res; }
double *qo_delta(qo_solver *s) { return s->delta; }
double *qo_normals(qo_solver *s) { return s->nrm; }
double *qo_entropy(qo_solver *s) { return s->entropy; }
const int *qo_sub_counts(qo_solver *s) { return s->subn; }
const int *qo_sub_lists(qo_solver *s) { return s->sub1; }
double qo_sum_res_sqr(qo_solver *s) { return s->sum_res_sqr; }
