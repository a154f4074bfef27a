// Host entry points to the per-point arithmetic and its reverse mode, for
// checking the hand-written derivatives against finite differences on a
// machine without a GPU (tests/test_adjoint_math.py).  Same source as the
// device code (qlskum_math.cuh, qlskum_adjoint.cuh), compiled for the host.
#include <cmath>

#include "qlskum_adjoint.cuh"

using namespace qlskum;

namespace {
CaseConst make_case(double mach, double aoa)
{
    CaseConst K{};
    K.pi = 4 * std::atan(1.0);
    K.rho_inf = 1.0;
    K.pr_inf = 1.0 / 1.4;
    K.gamma = 1.4;
    K.mach = mach;
    K.theta = aoa * K.pi / 180;
    K.u1_inf = mach * std::cos(K.theta);
    K.u2_inf = mach * std::sin(K.theta);
    return K;
}
}  // namespace

extern "C" {

void qlskum_dbg_prim_to_q(const double *P, double *q) { prim_to_q<double>(P[0], P[1], P[2], P[3], q); }

void qlskum_dbg_prim_to_q_vjp(const double *P, const double *bq, double *bP)
{
    for (int r = 0; r < 4; r++) bP[r] = 0;
    adj::prim_to_q_vjp(P, bq, bP);
}

double qlskum_dbg_venkat(double qt, double q, double qmax, double qmin, double e2)
{
    return venkat<double>(qt, q, qmax, qmin, e2);
}

// out: [bqt, bq, bqmax, bqmin]
void qlskum_dbg_venkat_vjp(double qt, double q, double qmax, double qmin, double e2, double bphi, double *out)
{
    out[0] = out[1] = out[2] = out[3] = 0;
    adj::venkat_vjp(qt, q, qmax, qmin, e2, bphi, out[0], out[1], out[2], out[3]);
}

void qlskum_dbg_qtilde_to_prim(const double *qt, double *P) { qtilde_to_prim<double>(qt, P[1], P[2], P[0], P[3]); }

void qlskum_dbg_qtilde_to_prim_vjp(const double *qt, const double *bP, double *bqt)
{
    for (int r = 0; r < 4; r++) bqt[r] = 0;
    adj::qtilde_to_prim_vjp(qt, bP, bqt);
}

// G = dir_flux<D>(class f) of state P = (rho, u1, u2, p) in the frame of (nx, ny)
void qlskum_dbg_dir_flux(int f, int D, double nx, double ny, const double *P, double *G)
{
    Kin<double> k;
    kin_prep<double>(nx, ny, P[1], P[2], P[0], P[3], k);
    switch (D) {
    case 0: dir_flux<double, 0>(f, k, G); break;
    case 1: dir_flux<double, 1>(f, k, G); break;
    case 2: dir_flux<double, 2>(f, k, G); break;
    default: dir_flux<double, 3>(f, k, G); break;
    }
}

// out: bP[4], bnx, bny
void qlskum_dbg_dir_flux_vjp(int f, int D, double nx, double ny, const double *P, const double *bG, double *out)
{
    Kin<double> k;
    kin_prep<double>(nx, ny, P[1], P[2], P[0], P[3], k);
    adj::KinBar kb;
    switch (D) {
    case 0: adj::dir_flux_vjp<0>(f, k, bG, kb); break;
    case 1: adj::dir_flux_vjp<1>(f, k, bG, kb); break;
    case 2: adj::dir_flux_vjp<2>(f, k, bG, kb); break;
    default: adj::dir_flux_vjp<3>(f, k, bG, kb); break;
    }
    for (int r = 0; r < 6; r++) out[r] = 0;
    adj::kin_vjp(nx, ny, P, k, kb, out, out[4], out[5]);
}

// in: [q4 dx4 dy4 mx4 mn4] (20), e2, delx, dely -> q~ (4)
void qlskum_dbg_edge_end(const double *in, double e2, double delx, double dely, double *qt)
{
    double ph[4], gi[4];
    for (int r = 0; r < 4; r++) {
        gi[r] = delx * in[4 + r] + dely * in[8 + r];
        ph[r] = venkat<double>(in[r] - 0.5 * gi[r], in[r], in[12 + r], in[16 + r], e2);
        qt[r] = in[r] - 0.5 * ph[r] * gi[r];
    }
}

// out: bars of the 20 inputs, then bdelx, bdely
void qlskum_dbg_edge_end_vjp(const double *in, double e2, double delx, double dely, const double *bqt, double *out)
{
    for (int r = 0; r < 22; r++) out[r] = 0;
    adj::edge_end_vjp(delx, dely, in, in + 4, in + 8, in + 12, in + 16, e2, bqt, out, out + 4, out + 8, out + 12,
                      out + 16, out[20], out[21]);
}

// One edge end as the FP64 solver evaluates it: the limited reconstruction,
// q~ -> prim and the flux of half-range D of a class-f point in the frame of
// (nx, ny).  in: [q4 dx4 dy4 mx4 mn4] (20), e2, delx, dely -> G (4)
void qlskum_dbg_end_flux(int f, int D, const double *in, double e2, double delx, double dely, double nx, double ny,
                         double *G)
{
    double qt[4], P[4];
    qlskum_dbg_edge_end(in, e2, delx, dely, qt);
    qtilde_to_prim<double>(qt, P[1], P[2], P[0], P[3]);
    qlskum_dbg_dir_flux(f, D, nx, ny, P, G);
}

namespace {
adj::End64 end64_of(const double *in, double e2, double delx, double dely, double nx, double ny)
{
    adj::End64 s;
    adj::end64(nx, ny, delx, dely, in, in + 4, in + 8, in + 12, in + 16, e2, s);
    return s;
}
}  // namespace

// The same flux from the FP64 reverse's kept edge-end state (adj::end64).
void qlskum_dbg_end64_flux(int f, int D, const double *in, double e2, double delx, double dely, double nx, double ny,
                           double *G)
{
    const adj::End64 s = end64_of(in, e2, delx, dely, nx, ny);
    switch (D) {
    case 0: dir_flux<double, 0>(f, s.k, G); break;
    case 1: dir_flux<double, 1>(f, s.k, G); break;
    case 2: dir_flux<double, 2>(f, s.k, G); break;
    default: dir_flux<double, 3>(f, s.k, G); break;
    }
}

// Reverse of qlskum_dbg_end_flux by end64 / end64_vjp.  out: bars of the 20
// inputs, then bdelx, bdely, bnx, bny
void qlskum_dbg_end64_flux_vjp(int f, int D, const double *in, double e2, double delx, double dely, double nx,
                               double ny, const double *bG, double *out)
{
    const adj::End64 s = end64_of(in, e2, delx, dely, nx, ny);
    adj::KinBar kb;
    switch (D) {
    case 0: adj::dir_flux_vjp<0>(f, s.k, bG, kb); break;
    case 1: adj::dir_flux_vjp<1>(f, s.k, bG, kb); break;
    case 2: adj::dir_flux_vjp<2>(f, s.k, bG, kb); break;
    default: adj::dir_flux_vjp<3>(f, s.k, bG, kb); break;
    }
    for (int r = 0; r < 24; r++) out[r] = 0;
    adj::end64_vjp(s, nx, ny, delx, dely, in + 4, in + 8, kb, out, out + 4, out + 8, out + 12, out + 16, out[20],
                   out[21], out[22], out[23]);
}

// The same reverse with the transcendentals taken from the forward's own
// evaluation (edge_end, qtilde_to_prim, kin_prep with keep), as the FP64
// flux reverse reads them from the recording forward.
void qlskum_dbg_end64_flux_vjp_kept(int f, int D, const double *in, double e2, double delx, double dely, double nx,
                                    double ny, const double *bG, double *out)
{
    double qt[4], P[4], keep[3];
    qlskum_dbg_edge_end(in, e2, delx, dely, qt);
    qtilde_to_prim<double>(qt, P[1], P[2], P[0], P[3]);
    Kin<double> k;
    kin_prep<double>(nx, ny, P[1], P[2], P[0], P[3], k, keep);
    const double kept[6] = {k.rho, keep[0], keep[1], keep[2], k.E1, k.E2};
    adj::End64 s;
    adj::end64(nx, ny, delx, dely, in, in + 4, in + 8, in + 12, in + 16, e2, s, kept);
    adj::KinBar kb;
    switch (D) {
    case 0: adj::dir_flux_vjp<0>(f, s.k, bG, kb); break;
    case 1: adj::dir_flux_vjp<1>(f, s.k, bG, kb); break;
    case 2: adj::dir_flux_vjp<2>(f, s.k, bG, kb); break;
    default: adj::dir_flux_vjp<3>(f, s.k, bG, kb); break;
    }
    for (int r = 0; r < 24; r++) out[r] = 0;
    adj::end64_vjp(s, nx, ny, delx, dely, in + 4, in + 8, kb, out, out + 4, out + 8, out + 12, out + 16, out[20],
                   out[21], out[22], out[23]);
}

void qlskum_dbg_stage_update(int f, double nx, double ny, const double *Pin, const double *Pold, const double *F,
                             int rk, double mach, double aoa, double *Pout)
{
    const CaseConst K = make_case(mach, aoa);
    double P[4] = {Pin[0], Pin[1], Pin[2], Pin[3]};
    double4_32a old = make_double4_32a(Pold[0], Pold[1], Pold[2], Pold[3]);
    stage_update(K, f, nx, ny, P, &old, F, rk);
    for (int r = 0; r < 4; r++) Pout[r] = P[r];
}

// out: bPin[4], bPold[4], bF[4], bnx, bny, bu1_inf, bu2_inf
void qlskum_dbg_stage_update_vjp(int f, double nx, double ny, const double *Pin, const double *Pold, const double *F,
                                 int rk, double mach, double aoa, const double *bPout, double *out)
{
    const CaseConst K = make_case(mach, aoa);
    double P[4] = {Pin[0], Pin[1], Pin[2], Pin[3]};
    double4_32a old = make_double4_32a(Pold[0], Pold[1], Pold[2], Pold[3]);
    stage_update(K, f, nx, ny, P, &old, F, rk);
    for (int r = 0; r < 16; r++) out[r] = 0;
    adj::stage_update_vjp(K, f, nx, ny, Pin, Pold, P, rk, bPout, out, out + 4, out + 8, out[12], out[13], out[14],
                          out[15]);
}

// the FP32 erf of the mixed form's kinetic moments (host build of the same source)
float qlskum_dbg_erf32(float x) { return erf_e<float>(x, std::exp(-x * x)); }

double qlskum_dbg_wave_speed(const double *P) { return wave_speed(P); }

void qlskum_dbg_wave_speed_vjp(const double *P, double bc, double *bP)
{
    for (int r = 0; r < 4; r++) bP[r] = 0;
    adj::wave_speed_vjp(P, bc, bP);
}

}  // extern "C"

// FP32 instantiations of the same reverse-mode functions (the adjoint of the
// mixed form), for comparison with the FP64 ones on the CPU.
extern "C" {

void qlskum_dbg_prim_to_q_vjp32(const float *P, const float *bq, float *bP)
{
    for (int r = 0; r < 4; r++) bP[r] = 0;
    adj::prim_to_q_vjp<float>(P, bq, bP);
}

void qlskum_dbg_qtilde_to_prim_vjp32(const float *qt, const float *bP, float *bqt)
{
    for (int r = 0; r < 4; r++) bqt[r] = 0;
    adj::qtilde_to_prim_vjp<float>(qt, bP, bqt);
}

// out: bP[4], bnx, bny; kind 0 x split, 1 y split, 2 quadrant (s2 = -1)
void qlskum_dbg_flux_vjp32(int kind, float s, float nx, float ny, const float *P, const float *bG, float *out)
{
    Kin<float> k;
    kin_prep<float>(nx, ny, P[1], P[2], P[0], P[3], k);
    adj::KinBarT<float> kb;
    if (kind == 0) adj::flux_x_vjp<float>(k, s, bG, kb);
    else if (kind == 1) adj::flux_y_vjp<float>(k, s, bG, kb);
    else adj::flux_quad_vjp<float>(k, s, -1.0f, bG, kb);
    for (int r = 0; r < 6; r++) out[r] = 0;
    adj::kin_vjp<float>(nx, ny, P, k, kb, out, out[4], out[5]);
}

void qlskum_dbg_flux_vjp64(int kind, double s, double nx, double ny, const double *P, const double *bG, double *out)
{
    Kin<double> k;
    kin_prep<double>(nx, ny, P[1], P[2], P[0], P[3], k);
    adj::KinBar kb;
    if (kind == 0) adj::flux_x_vjp<double>(k, s, bG, kb);
    else if (kind == 1) adj::flux_y_vjp<double>(k, s, bG, kb);
    else adj::flux_quad_vjp<double>(k, s, -1.0, bG, kb);
    for (int r = 0; r < 6; r++) out[r] = 0;
    adj::kin_vjp<double>(nx, ny, P, k, kb, out, out[4], out[5]);
}

void qlskum_dbg_edge_end_vjp32(const float *in, float e2, float delx, float dely, const float *bqt, float *out)
{
    for (int r = 0; r < 22; r++) out[r] = 0;
    adj::edge_end_vjp<float>(delx, dely, in, in + 4, in + 8, in + 12, in + 16, e2, bqt, out, out + 4, out + 8,
                             out + 12, out + 16, out[20], out[21]);
}

void qlskum_dbg_wave_speed_vjp32(const float *P, float bc, float *bP)
{
    for (int r = 0; r < 4; r++) bP[r] = 0;
    adj::wave_speed_vjp<float>(P, bc, bP);
}

}  // extern "C"
