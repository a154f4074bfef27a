// Host-only utilities of the C ABI that need no GPU: the partGrid cloud file
// (read / write, main.cpp:16-58) and the sub-stencil quality check that the
// reference leaves as an empty stub (generate_connectivity_mod.h:84-89).
// Compiled with -ffp-contract=off like the rest of the host layer.
#include "qlskum.h"
#include "qlskum_internal.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

using namespace qlskum;

namespace {
thread_local std::string g_io_error;

qlskum_status io_fail(qlskum_status s, const std::string &msg)
{
    g_io_error = msg;
    return s;
}
}  // namespace

extern "C" {

const char *qlskum_io_last_error(void) { return g_io_error.c_str(); }

// main.cpp:18-36: the point count, then per point x y left right flag_1 flag_2
// min_dist nbhs conn[1..nbhs].
qlskum_status qlskum_partgrid_read(const char *path, qlskum_cloud *out)
{
    if (!path || !out) return io_fail(QLSKUM_ERR_INVALID, "null path or output");
    std::memset(out, 0, sizeof *out);
    FILE *f = std::fopen(path, "r");
    if (!f) return io_fail(QLSKUM_ERR_INVALID, std::string("cannot open ") + path + ": " + std::strerror(errno));
    int n = 0;
    if (std::fscanf(f, "%d", &n) != 1 || n < 1) {
        std::fclose(f);
        return io_fail(QLSKUM_ERR_INVALID, "bad point count in the header");
    }
    const size_t N = (size_t)n;
    double *x = (double *)std::calloc(N, sizeof(double)), *y = (double *)std::calloc(N, sizeof(double));
    double *md = (double *)std::calloc(N, sizeof(double));
    int *left = (int *)std::calloc(N, sizeof(int)), *right = (int *)std::calloc(N, sizeof(int));
    int *f1 = (int *)std::calloc(N, sizeof(int)), *f2 = (int *)std::calloc(N, sizeof(int));
    int *nb = (int *)std::calloc(N, sizeof(int));
    int *conn = (int *)std::calloc(N * QLSKUM_MAX_NBHS, sizeof(int));
    qlskum_cloud c = {n, x, y, left, right, f1, f2, md, nb, conn};
    if (!x || !y || !md || !left || !right || !f1 || !f2 || !nb || !conn) {
        std::fclose(f);
        qlskum_partgrid_free(&c);
        return io_fail(QLSKUM_ERR_INVALID, "out of host memory");
    }
    for (int i = 0; i < n; i++) {
        int k = 0;
        if (std::fscanf(f, "%lf %lf %d %d %d %d %lf %d", &x[i], &y[i], &left[i], &right[i], &f1[i], &f2[i], &md[i],
                        &k) != 8 ||
            k < 0 || k > QLSKUM_MAX_NBHS) {
            std::fclose(f);
            qlskum_partgrid_free(&c);
            return io_fail(QLSKUM_ERR_INVALID, "point " + std::to_string(i + 1) + ": malformed row or nbhs outside 0..20");
        }
        nb[i] = k;
        for (int r = 0; r < k; r++)
            if (std::fscanf(f, "%d", &conn[(size_t)i * QLSKUM_MAX_NBHS + r]) != 1) {
                std::fclose(f);
                qlskum_partgrid_free(&c);
                return io_fail(QLSKUM_ERR_INVALID, "point " + std::to_string(i + 1) + ": truncated neighbour list");
            }
    }
    std::fclose(f);
    *out = c;
    return QLSKUM_OK;
}

void qlskum_partgrid_free(qlskum_cloud *c)
{
    if (!c) return;
    std::free((void *)c->x);
    std::free((void *)c->y);
    std::free((void *)c->left);
    std::free((void *)c->right);
    std::free((void *)c->flag_1);
    std::free((void *)c->flag_2);
    std::free((void *)c->min_dist);
    std::free((void *)c->nbhs);
    std::free((void *)c->conn);
    std::memset(c, 0, sizeof *c);
}

qlskum_status qlskum_partgrid_write(const char *path, const qlskum_cloud *c)
{
    if (!path || !c || c->n < 1) return io_fail(QLSKUM_ERR_INVALID, "null path or empty cloud");
    FILE *f = std::fopen(path, "w");
    if (!f) return io_fail(QLSKUM_ERR_INVALID, std::string("cannot open ") + path + ": " + std::strerror(errno));
    std::fprintf(f, "%d\n", c->n);
    for (int i = 0; i < c->n; i++) {
        std::fprintf(f, "%.17g %.17g %d %d %d %d %.17g %d", c->x[i], c->y[i], c->left[i], c->right[i], c->flag_1[i],
                     c->flag_2[i], c->min_dist[i], c->nbhs[i]);
        for (int r = 0; r < c->nbhs[i]; r++) std::fprintf(f, " %d", c->conn[(size_t)i * QLSKUM_MAX_NBHS + r]);
        std::fputc('\n', f);
    }
    const bool ok = std::fflush(f) == 0 && !std::ferror(f);
    std::fclose(f);
    return ok ? QLSKUM_OK : io_fail(QLSKUM_ERR_INVALID, std::string("write failed: ") + path);
}

// Reciprocal condition number (smallest / largest eigenvalue) of the 2x2
// least-squares matrix of each directional sub-stencil, split and weighted as
// generate_connectivity_mod.h:24-219 and interior_fluxes_mod.h:50-70 do it
// (normals from point_normals_mod.h:17-55).  rcond [n][4] (xpos, xneg, ypos,
// yneg; 1 for a direction the point's class does not use, 0 for one with
// fewer than two points); *n_bad = points with a used direction below
// min_rcond.  Either output may be NULL.
qlskum_status qlskum_check_stencils(const qlskum_cloud *c, double power, double min_rcond, double *rcond,
                                    int *n_bad)
{
    if (!c || c->n < 1 || !c->x || !c->y || !c->left || !c->right || !c->flag_1 || !c->nbhs || !c->conn)
        return io_fail(QLSKUM_ERR_INVALID, "null or empty cloud");
    const int n = c->n, NB = QLSKUM_MAX_NBHS;
    static const bool used[3][4] = {{true, true, false, true}, {true, true, true, true}, {true, true, true, false}};
    int bad = 0;
    for (int i = 0; i < n; i++) {
        const int f = c->flag_1[i];
        if (f < 0 || f > 2) return io_fail(QLSKUM_ERR_INVALID, "point " + std::to_string(i + 1) + ": flag_1 not in 0..2");
        double nx = 0.0, ny = 1.0;
        if (f != kInterior) {
            const int l = c->left[i] - 1, r = c->right[i] - 1;
            if (l < 0 || l >= n || r < 0 || r >= n)
                return io_fail(QLSKUM_ERR_INVALID, "point " + std::to_string(i + 1) + ": left/right out of range");
            const double a = 0.5 * ((c->y[i] - c->y[l]) + (c->y[r] - c->y[i]));
            const double b = 0.5 * ((c->x[i] - c->x[l]) + (c->x[r] - c->x[i]));
            const double det = std::sqrt(a * a + b * b);
            nx = -a / det;
            ny = b / det;
        }
        double sxx[4] = {0, 0, 0, 0}, syy[4] = {0, 0, 0, 0}, sxy[4] = {0, 0, 0, 0};
        int cnt[4] = {0, 0, 0, 0};
        const int k_n = c->nbhs[i];
        if (k_n < 0 || k_n > NB) return io_fail(QLSKUM_ERR_INVALID, "point " + std::to_string(i + 1) + ": nbhs outside 0..20");
        for (int r = 0; r < k_n; r++) {
            const int k = c->conn[(size_t)i * NB + r] - 1;
            if (k < 0 || k >= n)
                return io_fail(QLSKUM_ERR_INVALID, "point " + std::to_string(i + 1) + ": neighbour out of range");
            const double dx = c->x[k] - c->x[i], dy = c->y[k] - c->y[i];
            const double ds = dx * ny + dy * (-nx), dn = dx * nx + dy * ny;
            const double w = std::pow(std::sqrt(ds * ds + dn * dn), power);
            bool in[4] = {ds <= 0.0, ds >= 0.0, false, false};
            if (f == kInterior) {
                in[2] = dn <= 0.0;
                in[3] = dn >= 0.0;
            } else if (f == kWall) {
                in[3] = true;
            } else {
                in[2] = true;
            }
            for (int d = 0; d < 4; d++)
                if (in[d]) {
                    sxx[d] += ds * ds * w;
                    syy[d] += dn * dn * w;
                    sxy[d] += ds * dn * w;
                    cnt[d]++;
                }
        }
        bool point_bad = false;
        for (int d = 0; d < 4; d++) {
            double rc = 1.0;
            if (used[f][d]) {
                const double tr = sxx[d] + syy[d], det = sxx[d] * syy[d] - sxy[d] * sxy[d];
                const double disc = std::sqrt(std::fmax(tr * tr * 0.25 - det, 0.0));
                const double lmax = tr * 0.5 + disc;
                rc = (cnt[d] < 2 || lmax <= 0.0) ? 0.0 : (tr * 0.5 - disc) / lmax;
                if (rc < min_rcond) point_bad = true;
            }
            if (rcond) rcond[(size_t)i * 4 + d] = rc;
        }
        bad += point_bad ? 1 : 0;
    }
    if (n_bad) *n_bad = bad;
    return QLSKUM_OK;
}

}  // extern "C"
