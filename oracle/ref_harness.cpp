// Test-infrastructure only: a driver around the UNMODIFIED reference headers
// (Pathlessbark8/C-_serial), compiled straight from where they lie by
// oracle/build_ref.sh into oracle/_ref/ref_harness.  Nothing in the product
// links or runs this; it exists to pin the C restatement in oracle/qlskum_oracle.c
// and to generate the golden fixtures under tests/golden/.
//
// What this file adds around the reference:
//   * the grid path comes from argv instead of the hard-coded path at
//     main.cpp:17; the per-line parse follows main.cpp:30-58;
//   * the free-stream Mach/AoA are `const` at parameter_mod.h:4-5, so the
//     reference header is included with `const` defined away (the header text
//     itself is untouched) and the values are set before
//     setup_case_parameters() runs (parameter_mod.h:13-30);
//   * CFL, VL_CONST, inner_iterations, power and the iteration count are the
//     reference's own mutable globals (data_structure_mod.h:72-118);
//   * after the iterations, compute_cl_cd_cm() and compute_entropy() are called
//     explicitly (the reference's call at fpi_solver_mod.h:136 is commented
//     out) and the entropy total, which the reference accumulates into a
//     shadowing local (compute_entropy_mod.h:10,23), is re-summed from
//     point.entropy in point order.
//
// Output is raw little-endian float64 / int32 files in an output directory.
#include <cmath>
#include <math.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <iostream>
#include <fstream>
#include <iomanip>

#define const
#include "parameter_mod.h"
#undef const

#include "data_structure_mod.h"
#include "q_lskum_mod.h"          // pulls in fpi_solver, fluxes, limiter, state update, objectives
#include "compute_enstrophy_mod.h"
#include "split_fluxes_mod.h"
#include "quadrant_fluxes_mod.h"

static std::string g_out;

static void write_f64(const char *name, const std::vector<double> &v)
{
    std::string p = g_out + "/" + name;
    FILE *f = fopen(p.c_str(), "wb");
    if (!f) { perror(p.c_str()); exit(2); }
    fwrite(v.data(), sizeof(double), v.size(), f);
    fclose(f);
}

static void write_i32(const char *name, const std::vector<int> &v)
{
    std::string p = g_out + "/" + name;
    FILE *f = fopen(p.c_str(), "wb");
    if (!f) { perror(p.c_str()); exit(2); }
    fwrite(v.data(), sizeof(int), v.size(), f);
    fclose(f);
}

// Point-major [N][4] dump of a reference [5][N+1] field (rows 1..4, points 1..N).
static std::vector<double> pm4(const std::vector<std::vector<double>> &a)
{
    std::vector<double> o((size_t)max_points * 4);
    for (int i = 1; i <= max_points; i++)
        for (int r = 1; r <= 4; r++)
            o[(size_t)(i - 1) * 4 + (r - 1)] = a[r][i];
    return o;
}

// [N][2][4] dump of dq / qm (index 1..2, comp 1..4).
static std::vector<double> pm24(const std::vector<std::vector<std::vector<double>>> &a)
{
    std::vector<double> o((size_t)max_points * 8);
    for (int i = 1; i <= max_points; i++)
        for (int d = 1; d <= 2; d++)
            for (int r = 1; r <= 4; r++)
                o[(size_t)(i - 1) * 8 + (d - 1) * 4 + (r - 1)] = a[d][r][i];
    return o;
}

static void read_grid(const char *path)
{
    std::ifstream fin(path);
    if (!fin) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    fin >> max_points;
    point.x = std::vector<double>(max_points + 1);
    point.y = std::vector<double>(max_points + 1);
    point.left = std::vector<int>(max_points + 1);
    point.right = std::vector<int>(max_points + 1);
    point.flag_1 = std::vector<int>(max_points + 1);
    point.flag_2 = std::vector<int>(max_points + 1);
    point.nbhs = std::vector<int>(max_points + 1);
    point.min_dist = std::vector<double>(max_points + 1);
    point.conn = std::vector<std::vector<int>>(max_points + 1, std::vector<int>(20 + 1));
    point.nx = std::vector<double>(max_points + 1);
    point.ny = std::vector<double>(max_points + 1);
    for (int i = 1; i <= max_points; i++) {
        fin >> point.x[i] >> point.y[i] >> point.left[i] >> point.right[i] >> point.flag_1[i] >> point.flag_2[i] >> point.min_dist[i] >> point.nbhs[i];
        if (point.nbhs[i] < 0 || point.nbhs[i] > 20) { fprintf(stderr, "nbhs out of range at %d\n", i); exit(2); }
        for (int r = 1; r <= point.nbhs[i]; r++) fin >> point.conn[i][r];
        if (point.flag_1[i] == 0) { wall_points++; wall_points_index.push_back(i); }
        else if (point.flag_1[i] == 1) { interior_points++; interior_points_index.push_back(i); }
        else if (point.flag_1[i] == 2) { outer_points++; outer_points_index.push_back(i); }
        if (point.flag_2[i] > 0) shape_points++;
    }
    if (!fin) { fprintf(stderr, "short read in %s\n", path); exit(2); }
}

static void dump_connectivity()
{
    // nbhs per sub-stencil and the lists themselves, flattened in point order.
    std::vector<int> counts((size_t)max_points * 4), lists;
    for (int i = 1; i <= max_points; i++) {
        int c[4] = {point.xpos_nbhs[i], point.xneg_nbhs[i], point.ypos_nbhs[i], point.yneg_nbhs[i]};
        // The reference leaves ypos (wall) / yneg (outer) counts at their
        // allocation value 0; record them as such.
        for (int d = 0; d < 4; d++) counts[(size_t)(i - 1) * 4 + d] = c[d];
        const std::vector<int> *L[4] = {&point.xpos_conn[i], &point.xneg_conn[i], &point.ypos_conn[i], &point.yneg_conn[i]};
        for (int d = 0; d < 4; d++)
            for (int j = 1; j <= c[d]; j++) lists.push_back((*L[d])[j]);
    }
    write_i32("sub_counts.i32", counts);
    write_i32("sub_lists.i32", lists);
    std::vector<double> nrm((size_t)max_points * 2);
    for (int i = 1; i <= max_points; i++) { nrm[(size_t)(i - 1) * 2] = point.nx[i]; nrm[(size_t)(i - 1) * 2 + 1] = point.ny[i]; }
    write_f64("normals.f64", nrm);
}

static double objective_dump()
{
    compute_cl_cd_cm();
    compute_entropy();
    double tot = 0.0;
    for (int k = 1; k <= max_points; k++) tot = tot + point.entropy[k];
    std::vector<double> o = {Cl[1], Cd[1], Cm[1], tot};
    write_f64("objectives.f64", o);
    return tot;
}

static void usage()
{
    fprintf(stderr,
            "usage: ref_harness run   GRID OUTDIR [mach= aoa= cfl= vl= inner= power= iters=]\n"
            "       ref_harness stage GRID OUTDIR [same keys; iters = full iterations before the dumped one]\n"
            "       ref_harness flux  DATA OUTFILE   (8 split/quadrant fluxes per data.dat row)\n");
    exit(2);
}

int main(int argc, char **argv)
{
    if (argc < 4) usage();
    std::string mode = argv[1];

    if (mode == "flux") {
        // Rows: q1..q4 (ignored by the flux functions) nx ny u1 u2 rho pr, the
        // column meaning of the commented harness at main.cpp:72-100.
        std::ifstream fin(argv[2]);
        FILE *fo = fopen(argv[3], "wb");
        if (!fin || !fo) usage();
        double a[4], nx, ny, u1, u2, rho, pr;
        std::vector<double> G(5);
        while (fin >> a[0] >> a[1] >> a[2] >> a[3] >> nx >> ny >> u1 >> u2 >> rho >> pr) {
            void (*fns[8])(std::vector<double> &, double, double, double, double, double, double) = {
                flux_Gxp, flux_Gxn, flux_Gyp, flux_Gyn, flux_quad_GxI, flux_quad_GxII, flux_quad_GxIII, flux_quad_GxIV};
            for (int f = 0; f < 8; f++) {
                fns[f](G, nx, ny, u1, u2, rho, pr);
                fwrite(&G[1], sizeof(double), 4, fo);
            }
        }
        fclose(fo);
        return 0;
    }

    if (mode != "run" && mode != "stage") usage();
    read_grid(argv[2]);
    g_out = argv[3];
    int iters = 10;
    for (int a = 4; a < argc; a++) {
        const char *kv = argv[a];
        const char *eq = strchr(kv, '=');
        if (!eq) usage();
        std::string k(kv, eq - kv);
        double v = atof(eq + 1);
        if (k == "mach") mach = v;
        else if (k == "aoa") aoa = v;
        else if (k == "cfl") CFL = v;
        else if (k == "vl") VL_CONST = v;
        else if (k == "inner") inner_iterations = (int)v;
        else if (k == "power") power = v;
        else if (k == "iters") iters = (int)v;
        else usage();
    }

    allocate_soln();
    local_points = max_points;
    compute_normals();
    generate_connectivity();
    initial_conditions();
    dump_connectivity();

    // q_lskum_mod.h:20-26 bookkeeping, then the loop of q_lskum_mod.h:33-37
    // run one call at a time so each iteration's residual can be recorded.
    for (int i = 1; i <= local_points; i++) {
        point.U_old[1][i] = point.prim[1][i];
        point.U_old[2][i] = point.prim[1][i] * point.prim[2][i];
        point.U_old[3][i] = point.prim[1][i] * point.prim[3][i];
        point.U_old[4][i] = 2.5 * point.prim[4][i] + 0.5 * point.prim[1][i] * (point.prim[2][i] * point.prim[2][i] + point.prim[3][i] * point.prim[3][i]);
    }
    itr = 0;
    std::vector<double> hist;
    for (it = itr + 1; it <= itr + iters; it++) {
        fpi_solver(it);
        hist.push_back(res_new);
        hist.push_back(residue);
        hist.push_back(max_res);
    }
    write_f64("residuals.f64", hist);

    if (mode == "run") {
        write_f64("prim.f64", pm4(point.prim));
        objective_dump();
        // compute_enstrophy_mod.h:5-75 (never called by the reference's driver)
        compute_enstrophy();
        std::vector<double> ens(1, total_enstrophy);
        for (int i = 1; i <= max_points; i++) ens.push_back(point.vorticity[i]);
        write_f64("enstrophy.f64", ens);
        return 0;
    }

    // stage mode: one more iteration, dumped piece by piece (fpi_solver_mod.h:19-61, rk = 1).
    write_f64("prim_in.f64", pm4(point.prim));
    for (int i = 1; i <= max_points; i++)
        for (int j = 1; j <= 4; j++) point.prim_old[j][i] = point.prim[j][i];
    func_delta();
    write_f64("delta.f64", std::vector<double>(point.delta.begin() + 1, point.delta.end()));
    eval_q_variables();
    write_f64("q.f64", pm4(point.q));
    eval_q_derivatives();
    write_f64("dq0.f64", pm24(point.dq));
    write_f64("qm.f64", pm24(point.qm));
    for (int n = 1; n <= inner_iterations; n++) {
        eval_q_inner_loop();
        eval_update_innerloop();
    }
    write_f64("dq.f64", pm24(point.dq));
    cal_flux_residual();
    write_f64("flux_res.f64", pm4(point.flux_res));
    state_update(1);
    write_f64("prim_out.f64", pm4(point.prim));
    std::vector<double> s = {sum_res_sqr, max_res};
    write_f64("stage_res.f64", s);
    return 0;
}
