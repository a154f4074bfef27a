// Reverse mode (vector-Jacobian products) of the per-point and per-edge
// arithmetic of qlskum_math.cuh, host + device.  The per-edge functions are
// templates on the real type: FP64 for the adjoint of the drop-in form, FP32
// for the adjoint of the mixed form (with its SFU exp / log); the boundary
// update stays FP64 in both.
//
// Each *_vjp function takes the forward inputs (it recomputes what it needs)
// and the bar (adjoint) of the forward outputs, and ADDS the bars of the
// inputs into the caller's accumulators.  Non-smooth points follow the
// branch the forward pass took: the limiter's |dq-| <= 1e-5 and phi >= 1
// cases have zero derivative, neighbour max / min and the local time step's
// min pass the bar to the selected entry.  The derivatives are written out
// by hand from the formulas of the reference (split_fluxes_mod.h,
// quadrant_fluxes_mod.h, limiters_mod.h, q_variables_mod.h,
// state_update_mod.h) and each is checked against central differences
// (tests/test_adjoint_math.py).
#pragma once
#include "qlskum_math.cuh"

namespace qlskum {
namespace adj {

// q_variables_mod.h:19-33
template <typename R> QLSKUM_HD void prim_to_q_vjp(const R P[4], const R bq[4], R bP[4])
{
    const R rho = P[0], u1 = P[1], u2 = P[2], p = P[3];
    const R beta = M<R>::div(R(0.5) * rho, p);
    const R usq = u1 * u1 + u2 * u2;
    const R bbeta = bq[0] * (M<R>::div(R(2.5), beta) - usq) + bq[1] * R(2.0) * u1 + bq[2] * R(2.0) * u2 - R(2.0) * bq[3];
    bP[0] += M<R>::div(bq[0], rho) + M<R>::div(bbeta * R(0.5), p);
    bP[1] += -bq[0] * R(2.0) * beta * u1 + bq[1] * R(2.0) * beta;
    bP[2] += -bq[0] * R(2.0) * beta * u2 + bq[2] * R(2.0) * beta;
    bP[3] += -M<R>::div(bbeta * beta, p);
}

// limiters_mod.h:64-104 for one component.
template <typename R> QLSKUM_HD void venkat_vjp(R qt, R q, R qmax, R qmin, R eps2, R bphi, R &bqt,
                          R &bq, R &bqmax, R &bqmin)
{
    const R dn = qt - q;
    if (M<R>::ab(dn) <= R(10e-6)) return;
    const bool up = dn > 0;
    const R dp = (up ? qmax : qmin) - q;
    const R num = (dp * dp + eps2) * dn + R(2.0) * dn * dn * dp;
    const R den = (dp * dp + R(2.0) * dn * dn + dn * dp + eps2) * dn;
    const R rden = M<R>::div(R(1.0), den);
    const R t = num * rden;
    if (!(t < R(1.0))) return;
    const R bnum = bphi * rden, bden = -bphi * t * rden;
    const R bdn = bnum * (dp * dp + eps2 + R(4.0) * dn * dp) +
                       bden * ((dp * dp + R(2.0) * dn * dn + dn * dp + eps2) + dn * (R(4.0) * dn + dp));
    const R bdp = bnum * (R(2.0) * dp * dn + R(2.0) * dn * dn) + bden * (dn * (R(2.0) * dp + dn));
    bqt += bdn;
    bq -= bdn + bdp;
    if (up) bqmax += bdp;
    else bqmin += bdp;
}

// q_variables_mod.h:230-253; P = (rho, u1, u2, p).
template <typename R> QLSKUM_HD void qtilde_to_prim_vjp(const R qt[4], const R bP[4], R bqt[4])
{
    const R gm1 = R(1.4) - R(1.0);
    const R beta = -qt[3] * R(0.5);
    const R t = M<R>::div(R(0.5), beta);
    const R u1 = qt[1] * t, u2 = qt[2] * t;
    const R T1 = qt[0] + beta * (u1 * u1 + u2 * u2);
    const R rho = M<R>::ex(T1 - M<R>::div(M<R>::lg(beta), gm1));
    const R brho = bP[0] + bP[3] * t;
    const R bT2 = brho * rho, bT1 = bT2;
    const R bu1 = bP[1] + bT1 * R(2.0) * beta * u1;
    const R bu2 = bP[2] + bT1 * R(2.0) * beta * u2;
    const R bt = bP[3] * rho + bu1 * qt[1] + bu2 * qt[2];
    const R bbeta = bT1 * (u1 * u1 + u2 * u2) - M<R>::div(bT2, gm1 * beta) - M<R>::div(bt * R(0.5), beta * beta);
    bqt[0] += bT1;
    bqt[1] += bu1 * t;
    bqt[2] += bu2 * t;
    bqt[3] += -R(0.5) * bbeta;
}

// Bars of the fields of Kin<R>.
template <typename R> struct KinBarT {
    R rho = 0, ut = 0, un = 0, pbr = 0, usq = 0, B1 = 0, B2 = 0, E1 = 0, E2 = 0;
};
using KinBar = KinBarT<double>;

// kin_prep (split_fluxes_mod.h:14-26): bars of (u1, u2, rho, p) and of the normal.
template <typename R> QLSKUM_HD void kin_vjp(R nx, R ny, const R P[4], const Kin<R> &k, const KinBarT<R> &kb, R bP[4],
                       R &bnx, R &bny)
{
    const R rho = P[0], u1 = P[1], u2 = P[2], p = P[3];
    const R beta = M<R>::div(R(0.5) * rho, p);
    const R sb = M<R>::sq(beta);
    const R S1 = k.ut * sb, S2 = k.un * sb;
    const R two_over_sqrtpi = R(1.1283791670955126);
    R but = kb.ut + R(2.0) * k.ut * kb.usq;
    R bun = kb.un + R(2.0) * k.un * kb.usq;
    const R bS1 = kb.E1 * two_over_sqrtpi * M<R>::ex(-S1 * S1) + kb.B1 * k.B1 * (-R(2.0) * S1);
    const R bS2 = kb.E2 * two_over_sqrtpi * M<R>::ex(-S2 * S2) + kb.B2 * k.B2 * (-R(2.0) * S2);
    but += bS1 * sb;
    bun += bS2 * sb;
    const R bsb = bS1 * k.ut + bS2 * k.un;
    const R bbeta = M<R>::div(bsb * R(0.5), sb) - M<R>::div((kb.B1 * k.B1 + kb.B2 * k.B2) * R(0.5), beta);
    bP[0] += kb.rho + M<R>::div(bbeta * R(0.5), p) - M<R>::div(kb.pbr * p, rho * rho);
    bP[3] += -M<R>::div(bbeta * beta, p) + M<R>::div(kb.pbr, rho);
    bP[1] += but * ny + bun * nx;
    bP[2] += -but * nx + bun * ny;
    bnx += -but * u2 + bun * u1;
    bny += but * u1 + bun * u2;
}

// flux_Gxp / flux_Gxn
template <typename R> QLSKUM_HD void flux_x_vjp(const Kin<R> &k, R s1, const R bG[4], KinBarT<R> &kb)
{
    const R A1 = R(0.5) * (R(1.0) + s1 * k.E1), B1s = s1 * k.B1;
    const R ut = k.ut, un = k.un, pbr = k.pbr, usq = k.usq, rho = k.rho;
    const R a0 = ut * A1 + B1s, a1 = (pbr + ut * ut) * A1 + ut * B1s, a2 = ut * un * A1 + un * B1s;
    const R a3 = R(0.5) * ut * (R(7.0) * pbr + usq) * A1 + R(0.5) * (R(6.0) * pbr + usq) * B1s;
    kb.rho += bG[0] * a0 + bG[1] * a1 + bG[2] * a2 + bG[3] * a3;
    const R b0 = rho * bG[0], b1 = rho * bG[1], b2 = rho * bG[2], b3 = rho * bG[3];
    const R bA1 = b0 * ut + b1 * (pbr + ut * ut) + b2 * ut * un + b3 * R(0.5) * ut * (R(7.0) * pbr + usq);
    const R bB1s = b0 + b1 * ut + b2 * un + b3 * R(0.5) * (R(6.0) * pbr + usq);
    kb.ut += b0 * A1 + b1 * (R(2.0) * ut * A1 + B1s) + b2 * un * A1 + b3 * R(0.5) * (R(7.0) * pbr + usq) * A1;
    kb.un += b2 * (ut * A1 + B1s);
    kb.pbr += b1 * A1 + b3 * (R(3.5) * ut * A1 + R(3.0) * B1s);
    kb.usq += b3 * (R(0.5) * ut * A1 + R(0.5) * B1s);
    kb.E1 += R(0.5) * s1 * bA1;
    kb.B1 += s1 * bB1s;
}

// flux_Gyp / flux_Gyn
template <typename R> QLSKUM_HD void flux_y_vjp(const Kin<R> &k, R s2, const R bG[4], KinBarT<R> &kb)
{
    const R A2 = R(0.5) * (R(1.0) + s2 * k.E2), B2s = s2 * k.B2;
    const R ut = k.ut, un = k.un, pbr = k.pbr, usq = k.usq, rho = k.rho;
    const R a0 = un * A2 + B2s, a2 = (pbr + un * un) * A2 + un * B2s, a1 = ut * un * A2 + ut * B2s;
    const R a3 = R(0.5) * un * (R(7.0) * pbr + usq) * A2 + R(0.5) * (R(6.0) * pbr + usq) * B2s;
    kb.rho += bG[0] * a0 + bG[1] * a1 + bG[2] * a2 + bG[3] * a3;
    const R b0 = rho * bG[0], b1 = rho * bG[1], b2 = rho * bG[2], b3 = rho * bG[3];
    const R bA2 = b0 * un + b2 * (pbr + un * un) + b1 * ut * un + b3 * R(0.5) * un * (R(7.0) * pbr + usq);
    const R bB2s = b0 + b2 * un + b1 * ut + b3 * R(0.5) * (R(6.0) * pbr + usq);
    kb.un += b0 * A2 + b2 * (R(2.0) * un * A2 + B2s) + b1 * ut * A2 + b3 * R(0.5) * (R(7.0) * pbr + usq) * A2;
    kb.ut += b1 * (un * A2 + B2s);
    kb.pbr += b2 * A2 + b3 * (R(3.5) * un * A2 + R(3.0) * B2s);
    kb.usq += b3 * (R(0.5) * un * A2 + R(0.5) * B2s);
    kb.E2 += R(0.5) * s2 * bA2;
    kb.B2 += s2 * bB2s;
}

// flux_quad_GxI..IV
template <typename R> QLSKUM_HD void flux_quad_vjp(const Kin<R> &k, R s1, R s2, const R bG[4], KinBarT<R> &kb)
{
    const R ut = k.ut, un = k.un, pbr = k.pbr, usq = k.usq, rho = k.rho;
    const R A1 = R(0.5) * (R(1.0) + s1 * k.E1), A2 = R(0.5) * (R(1.0) + s2 * k.E2), B1s = s1 * k.B1;
    const R f1 = ut * A1 + B1s;
    const R h = (pbr + ut * ut) * A1 + ut * B1s;
    const R m = un * A2 + s2 * k.B2;
    const R t2 = R(0.5) * ut * (R(7.0) * pbr + usq) * A1, t3 = R(0.5) * k.B1 * (R(6.0) * pbr + usq);
    const R bt4 = s2 * bG[3];
    kb.rho += bG[0] * A2 * f1 + bG[1] * A2 * h + bG[2] * f1 * m + bG[3] * A2 * (t2 + s1 * t3) +
              bt4 * R(0.5) * un * k.B2 * f1;
    R bA2 = rho * (bG[0] * f1 + bG[1] * h + bG[3] * (t2 + s1 * t3));
    R bf1 = rho * (bG[0] * A2 + bG[2] * m) + bt4 * R(0.5) * rho * un * k.B2;
    const R bh = rho * A2 * bG[1];
    const R bm = rho * f1 * bG[2];
    const R bt2 = rho * A2 * bG[3], bt3 = rho * A2 * s1 * bG[3];
    kb.un += bt4 * R(0.5) * rho * k.B2 * f1 + bm * A2;
    kb.B2 += bt4 * R(0.5) * rho * un * f1 + bm * s2;
    bA2 += bm * un;
    kb.pbr += bh * A1 + bt2 * R(3.5) * ut * A1 + bt3 * R(3.0) * k.B1;
    kb.ut += bh * (R(2.0) * ut * A1 + B1s) + bf1 * A1 + bt2 * R(0.5) * (R(7.0) * pbr + usq) * A1;
    R bA1 = bh * (pbr + ut * ut) + bf1 * ut + bt2 * R(0.5) * ut * (R(7.0) * pbr + usq);
    const R bB1s = bh * ut + bf1;
    kb.usq += bt2 * R(0.5) * ut * A1 + bt3 * R(0.5) * k.B1;
    kb.B1 += bt3 * R(0.5) * (R(6.0) * pbr + usq) + s1 * bB1s;
    kb.E1 += R(0.5) * s1 * bA1;
    kb.E2 += R(0.5) * s2 * bA2;
}

template <int D> QLSKUM_HD void dir_flux_vjp(int f, const Kin<double> &k, const double bG[4], KinBar &kb)
{
    if (D <= 1) {
        const double s1 = (D == 0) ? 1.0 : -1.0;
        if (f == kInterior) flux_x_vjp(k, s1, bG, kb);
        else flux_quad_vjp(k, s1, (f == kOuter) ? 1.0 : -1.0, bG, kb);
    } else {
        flux_y_vjp(k, (D == 2) ? 1.0 : -1.0, bG, kb);
    }
}

// Reconstruction of one edge end (interior_fluxes_mod.h:72-83) for all four
// components: q~ = q - 0.5 phi(q - 0.5 g) g with g = delx dqx + dely dqy.
// Adds bars of q, dq (x, y), qm (max, min) and of the edge vector.
template <typename R> QLSKUM_HD void edge_end_vjp(R delx, R dely, const R q[4], const R dx[4], const R dy[4],
                            const R mx[4], const R mn[4], R e2, const R bqt[4], R bq[4],
                            R bdx[4], R bdy[4], R bmx[4], R bmn[4], R &bdelx, R &bdely)
{
    for (int r = 0; r < 4; r++) {
        const R g = delx * dx[r] + dely * dy[r];
        const R qtu = q[r] - R(0.5) * g;
        const R phi = venkat<R>(qtu, q[r], mx[r], mn[r], e2);
        bq[r] += bqt[r];
        const R bphi = -R(0.5) * g * bqt[r];
        R bg = -R(0.5) * phi * bqt[r];
        R bqtu = R(0.0);
        venkat_vjp(qtu, q[r], mx[r], mn[r], e2, bphi, bqtu, bq[r], bmx[r], bmn[r]);
        bq[r] += bqtu;
        bg += -R(0.5) * bqtu;
        bdx[r] += bg * delx;
        bdy[r] += bg * dely;
        bdelx += bg * dx[r];
        bdely += bg * dy[r];
    }
}

// One edge end of the FP64 reverse, evaluated once per edge and end: the
// limited reconstruction (interior_fluxes_mod.h:72-83, limiters_mod.h:64-104),
// q~ -> prim (q_variables_mod.h:230-253) and the half-range moments
// (split_fluxes_mod.h:14-26), keeping what end64_vjp reads.  The functions
// above recompute each quantity they need (an edge end then costs 33 FP64
// divisions, 6 exps and 2 logs); here one end costs 7 reciprocals (rcp64 on
// the device: an FP32 seed and two Newton steps, no FP64 division), 3 exps
// and 1 log.  The forward values are those of edge_states / kin_prep up to
// last-bit roundings: the limiter's ratio is num * (1 / den), whose
// reciprocal the VJP reads too; kin_prep's beta = rho / (2 p) and
// p / rho are the q~ -> prim step's beta and 1 / (2 beta); 1 / (gamma - 1)
// and 1 / sqrt(pi beta) are multiplications.  The reverse is the derivative
// at that state, along the branches it took.
struct End64 {
    double g[4], dn[4], dp[4], rden[4], t[4];  // per component: g, q~u - q, qmax|qmin - q, 1 / den, num / den
    double eps2, qt1, qt2, beta, tm, u1, u2, rho, sb, rsb, e1, e2;
    Kin<double> k;
};

// kept (or NULL): the forward flux kernel's {rho, sqrt(beta), exp(-S1^2),
// exp(-S2^2), erf(S1), erf(S2)} of this end (fp64::flux_residual's ends),
// taken instead of recomputing the log, the exps, the square root and the
// erfs.
QLSKUM_HD void end64(double nx, double ny, double delx, double dely, const double q[4], const double dx[4],
                     const double dy[4], const double mx[4], const double mn[4], double e2, End64 &s,
                     const double *kept = nullptr)
{
    constexpr double inv_gm1 = 1.0 / (1.4 - 1.0);
    double qt[4];
    for (int r = 0; r < 4; r++) {
        const double g = delx * dx[r] + dely * dy[r];
        const double dn = (q[r] - 0.5 * g) - q[r];
        const double dp = ((dn > 0.0) ? mx[r] : mn[r]) - q[r];
        const double num = (dp * dp + e2) * dn + 2.0 * dn * dn * dp;
        const double den = ((dp * dp + 2.0 * dn * dn) + dn * dp + e2) * dn;
        const bool cut = fabs(dn) <= 10e-6;
        const double rden = M<double>::rcp(cut ? 1.0 : den);
        const double t = num * rden;
        const double phi = (cut || !(t < 1.0)) ? 1.0 : t;
        s.g[r] = g;
        s.dn[r] = dn;
        s.dp[r] = dp;
        s.rden[r] = rden;
        s.t[r] = cut ? 1.0 : t;
        qt[r] = q[r] - 0.5 * phi * g;
    }
    s.eps2 = e2;
    s.qt1 = qt[1];
    s.qt2 = qt[2];
    s.beta = -qt[3] * 0.5;
    s.tm = 0.5 * M<double>::rcp(s.beta);
    s.u1 = qt[1] * s.tm;
    s.u2 = qt[2] * s.tm;
    s.k.ut = s.u1 * ny - s.u2 * nx;
    s.k.un = s.u1 * nx + s.u2 * ny;
    if (kept) {
        s.rho = kept[0];
        s.sb = kept[1];
        s.e1 = kept[2];
        s.e2 = kept[3];
        s.k.E1 = kept[4];
        s.k.E2 = kept[5];
    } else {
        s.rho = M<double>::ex(qt[0] + s.beta * (s.u1 * s.u1 + s.u2 * s.u2) - M<double>::lg(s.beta) * inv_gm1);
        s.sb = M<double>::sq(s.beta);
        const double S1 = s.k.ut * s.sb, S2 = s.k.un * s.sb;
        s.e1 = M<double>::ex(-S1 * S1);
        s.e2 = M<double>::ex(-S2 * S2);
        s.k.E1 = erf_e<double>(S1, s.e1);
        s.k.E2 = erf_e<double>(S2, s.e2);
    }
    s.k.rho = s.rho;
    s.rsb = M<double>::rcp(s.sb);
    const double half_rpi = 0.28209479177387814;  // 1 / (2 sqrt(pi))
    s.k.B1 = half_rpi * s.e1 * s.rsb;
    s.k.B2 = half_rpi * s.e2 * s.rsb;
    s.k.pbr = s.tm;
    s.k.usq = s.k.ut * s.k.ut + s.k.un * s.k.un;
}

// Reverse of end64 for the bar kb of its moments (the sum of dir_flux_vjp
// over the edge's half-ranges): kin_vjp, qtilde_to_prim_vjp and edge_end_vjp
// on the kept intermediates.  Adds the bars of the end's q, dq (x, y), qm
// (max, min), of the edge vector and of the normal.
QLSKUM_HD void end64_vjp(const End64 &s, double nx, double ny, double delx, double dely, const double dx[4],
                         const double dy[4], const KinBar &kb, double bq[4], double bdx[4], double bdy[4],
                         double bmx[4], double bmn[4], double &bdelx, double &bdely, double &bnx, double &bny)
{
    constexpr double inv_gm1 = 1.0 / (1.4 - 1.0);
    const double two_over_sqrtpi = 1.1283791670955126;
    // kin_prep of P = (rho, u1, u2, p), p = rho tm, beta = rho / (2 p)
    const double ut = s.k.ut, un = s.k.un;
    const double S1 = ut * s.sb, S2 = un * s.sb;
    double but = kb.ut + 2.0 * ut * kb.usq;
    double bun = kb.un + 2.0 * un * kb.usq;
    const double bS1 = kb.E1 * two_over_sqrtpi * s.e1 + kb.B1 * s.k.B1 * (-2.0 * S1);
    const double bS2 = kb.E2 * two_over_sqrtpi * s.e2 + kb.B2 * s.k.B2 * (-2.0 * S2);
    but += bS1 * s.sb;
    bun += bS2 * s.sb;
    const double bsb = bS1 * ut + bS2 * un;
    const double bbk = 0.5 * bsb * s.rsb - (kb.B1 * s.k.B1 + kb.B2 * s.k.B2) * s.tm;  // 0.5 / beta = tm
    const double irho = M<double>::rcp(s.rho);
    // 0.5 / p = beta / rho, p / rho^2 = tm / rho, beta / p = 2 beta^2 / rho
    const double bP0 = kb.rho + bbk * s.beta * irho - kb.pbr * s.tm * irho;
    const double bP3 = -bbk * 2.0 * s.beta * s.beta * irho + kb.pbr * irho;
    const double bP1 = but * ny + bun * nx;
    const double bP2 = -but * nx + bun * ny;
    bnx += -but * s.u2 + bun * s.u1;
    bny += but * s.u1 + bun * s.u2;
    // q~ -> prim: rho = exp(q0 + beta |u|^2 - log(beta) / (gamma - 1)), u = q~(1:2) tm, p = rho tm
    const double brho = bP0 + bP3 * s.tm;
    const double bT1 = brho * s.rho;
    const double bu1 = bP1 + bT1 * 2.0 * s.beta * s.u1;
    const double bu2 = bP2 + bT1 * 2.0 * s.beta * s.u2;
    const double bt = bP3 * s.rho + bu1 * s.qt1 + bu2 * s.qt2;
    // 1 / beta = 2 tm, 0.5 / beta^2 = 2 tm^2
    const double bbeta = bT1 * (s.u1 * s.u1 + s.u2 * s.u2) - bT1 * inv_gm1 * 2.0 * s.tm - bt * 2.0 * s.tm * s.tm;
    const double bqt[4] = {bT1, bu1 * s.tm, bu2 * s.tm, -0.5 * bbeta};
    // the limited reconstruction q~ = q - phi g / 2, phi = num / den of
    // dn = (q - g / 2) - q and dp = qmax - q (dn > 0) or qmin - q
    for (int r = 0; r < 4; r++) {
        const double dn = s.dn[r], dp = s.dp[r], t = s.t[r];
        const bool lim = fabs(dn) > 10e-6 && t < 1.0;
        double bg = -0.5 * (lim ? t : 1.0) * bqt[r];
        double bdp = 0.0;
        if (lim) {
            const double bphi = -0.5 * s.g[r] * bqt[r];
            const double bnum = bphi * s.rden[r], bden = -bphi * t * s.rden[r];
            const double bdn = bnum * (dp * dp + s.eps2 + 4.0 * dn * dp) +
                               bden * ((dp * dp + 2.0 * dn * dn + dn * dp + s.eps2) + dn * (4.0 * dn + dp));
            bdp = bnum * (2.0 * dp * dn + 2.0 * dn * dn) + bden * (dn * (2.0 * dp + dn));
            bg += -0.5 * bdn;
            if (dn > 0.0) bmx[r] += bdp;
            else bmn[r] += bdp;
        }
        // q enters q~ directly and through dp (dn - its own rounding aside - is -g / 2)
        bq[r] += bqt[r] - bdp;
        bdx[r] += bg * delx;
        bdy[r] += bg * dely;
        bdelx += bg * dx[r];
        bdely += bg * dy[r];
    }
}

// primitive_to_conserved (state_update_mod.h:18-33)
template <typename R>
QLSKUM_HD void p2c_vjp(const R P[4], R nx, R ny, const R bU[4], R bP[4], R &bnx, R &bny)
{
    const R rho = P[0], t1 = rho * P[1], t2 = rho * P[2];
    const R bt1 = M<R>::div(bU[3] * t1, rho) + bU[1] * ny + bU[2] * nx;
    const R bt2 = M<R>::div(bU[3] * t2, rho) - bU[1] * nx + bU[2] * ny;
    bP[0] += bU[0] - M<R>::div(bU[3] * R(0.5) * (t1 * t1 + t2 * t2), rho * rho) + bt1 * P[1] + bt2 * P[2];
    bP[1] += bt1 * rho;
    bP[2] += bt2 * rho;
    bP[3] += R(2.5) * bU[3];
    bnx += -bU[1] * t2 + bU[2] * t1;
    bny += bU[1] * t1 + bU[2] * t2;
}

// conserved_vector_Ubar (state_update_mod.h:35-90): bars of the point's
// state, of the normal and of the free-stream velocity (u1_inf, u2_inf).
template <typename R>
QLSKUM_HD void ubar_vjp(const CaseConst &K, const R P[4], R nx, R ny, const R bU[4], R bP[4], R &bnx, R &bny,
                        R &bu1i, R &bu2i)
{
    const R g1 = R(K.gamma) - R(1.0), pi = R(K.pi), rhoi = R(K.rho_inf), pri = R(K.pr_inf);
    const R u1inf = R(K.u1_inf), u2inf = R(K.u2_inf);
    const R tx = ny, ty = -nx;
    const R inv_sqrtpi = R(0.5641895835477563);
    // free-stream half
    const R u1ri = u1inf * tx + u2inf * ty, u2ri = u1inf * nx + u2inf * ny;
    const R einf = M<R>::div(pri, rhoi * g1) + R(0.5) * (u1ri * u1ri + u2ri * u2ri);
    const R bi = M<R>::div(R(0.5) * rhoi, pri), sbi = M<R>::sq(bi);
    const R Si = u2ri * sbi;
    const R ei = M<R>::ex(-Si * Si);
    const R Bi = M<R>::div(ei, R(2.0) * M<R>::sq(pi * bi));
    const R Ai = R(0.5) * (R(1.0) - erf_e<R>(Si, ei));
    const R bAi = bU[0] * rhoi + bU[1] * rhoi * u1ri + bU[2] * rhoi * u2ri + bU[3] * rhoi * einf;
    const R bBi = -bU[2] * rhoi - bU[3] * R(0.5) * rhoi * u2ri;
    const R bei = bU[3] * rhoi * Ai;
    const R bSi = -bAi * inv_sqrtpi * ei + bBi * Bi * (R(-2.0) * Si);
    const R bu1ri = bU[1] * rhoi * Ai + bei * u1ri;
    const R bu2ri = bU[2] * rhoi * Ai - bU[3] * R(0.5) * rhoi * Bi + bei * u2ri + bSi * sbi;
    bu1i += bu1ri * tx + bu2ri * nx;
    bu2i += bu1ri * ty + bu2ri * ny;
    bnx += -bu1ri * u2inf + bu2ri * u1inf;
    bny += bu1ri * u1inf + bu2ri * u2inf;
    // the point's half
    const R rho = P[0], u1 = P[1], u2 = P[2], p = P[3];
    const R u1r = u1 * tx + u2 * ty, u2r = u1 * nx + u2 * ny;
    const R e = M<R>::div(p, rho * g1) + R(0.5) * (u1r * u1r + u2r * u2r);
    const R beta = M<R>::div(rho, R(2.0) * p), sb = M<R>::sq(beta);
    const R S = u2r * sb;
    const R es = M<R>::ex(-S * S);
    const R B = M<R>::div(es, R(2.0) * M<R>::sq(pi * beta));
    const R A = R(0.5) * (R(1.0) + erf_e<R>(S, es));
    const R bA = bU[0] * rho + bU[1] * rho * u1r + bU[2] * rho * u2r + bU[3] * rho * e;
    const R bB = bU[2] * rho + bU[3] * R(0.5) * rho * u2r;
    const R be = bU[3] * rho * A;
    R brho = bU[0] * A + bU[1] * u1r * A + bU[2] * (u2r * A + B) + bU[3] * (A * e + R(0.5) * u2r * B);
    const R bS = bA * inv_sqrtpi * es + bB * B * (R(-2.0) * S);
    const R bu1r = bU[1] * rho * A + be * u1r;
    const R bu2r = bU[2] * rho * A + bU[3] * R(0.5) * rho * B + be * u2r + bS * sb;
    const R bbeta = M<R>::div(bS * u2r * R(0.5), sb) - M<R>::div(bB * B * R(0.5), beta);
    R bp = M<R>::div(be, rho * g1);
    brho += -M<R>::div(be * p, rho * rho * g1);
    brho += M<R>::div(bbeta, R(2.0) * p);
    bp += -M<R>::div(bbeta * beta, p);
    bP[0] += brho;
    bP[1] += bu1r * tx + bu2r * nx;
    bP[2] += bu1r * ty + bu2r * ny;
    bP[3] += bp;
    bnx += -bu1r * u2 + bu2r * u1;
    bny += bu1r * u1 + bu2r * u2;
}

// One SSPRK stage of one point (state_update_mod.h:111-282) in reverse.
// Pout is the stage's output state (it carries U' and 1/U'0).  Adds the bars
// of the input state, of prim_old (stage 3), of the flux residual, of the
// normal and of the free-stream velocity (outer points).  R = double for the
// FP64 iteration; float for the reverse of the mixed one (whose forward
// update is FP64: its reverse needs only the bars' relative accuracy).
template <typename R>
QLSKUM_HD void stage_update_vjp(const CaseConst &K, int f, R nx, R ny, const R Pin[4], const R Pold[4],
                                const R Pout[4], int rk, const R bPout[4], R bPin[4], R bPold[4], R bF[4], R &bnx,
                                R &bny, R &bu1i, R &bu2i)
{
    const R obt = R(1.0) / R(3.0), tbt = R(2.0) / R(3.0);
    const R U0 = Pout[0], inv = M<R>::div(R(1.0), U0);
    const R V1 = Pout[1] * U0, V2 = Pout[2] * U0;  // rotated-back momentum
    R bU[4];
    R binv = bPout[1] * V1 + bPout[2] * V2 - R(0.2) * bPout[3] * (V1 * V1 + V2 * V2);
    const R bV1 = bPout[1] * inv - R(0.4) * bPout[3] * inv * V1;
    const R bV2 = bPout[2] * inv - R(0.4) * bPout[3] * inv * V2;
    bU[0] = bPout[0] - binv * inv * inv;
    bU[3] = R(0.4) * bPout[3];
    // V1 = U1 ny + U2 nx, V2 = U2 ny - U1 nx (U in the (t, n) frame)
    bU[1] = bV1 * ny - bV2 * nx;
    bU[2] = bV1 * nx + bV2 * ny;
    // the frame of the output: U1 = V1 ny - V2 nx, U2 = V1 nx + V2 ny
    const R U1 = V1 * ny - V2 * nx, U2 = V1 * nx + V2 * ny;
    bny += bV1 * U1 + bV2 * U2;
    bnx += bV1 * U2 - bV2 * U1;
    if (f == kWall) bU[2] = R(0.0);
    R bUin[4], bUold[4];
    for (int j = 0; j < 4; j++) {
        if (rk != 3) {
            bUin[j] = bU[j];
            bF[j] += R(-0.5) * bU[j];
            bUold[j] = R(0.0);
        } else {
            bUold[j] = tbt * bU[j];
            bUin[j] = obt * bU[j];
            bF[j] += R(-0.5) * obt * bU[j];
        }
    }
    if (f == kOuter) {
        ubar_vjp<R>(K, Pin, nx, ny, bUin, bPin, bnx, bny, bu1i, bu2i);
        if (rk == 3) ubar_vjp<R>(K, Pold, nx, ny, bUold, bPold, bnx, bny, bu1i, bu2i);
    } else {
        p2c_vjp<R>(Pin, nx, ny, bUin, bPin, bnx, bny);
        if (rk == 3) p2c_vjp<R>(Pold, nx, ny, bUold, bPold, bnx, bny);
    }
}

// |u| + 3 sqrt(p / rho) (state_update_mod.h:483-485)
template <typename R> QLSKUM_HD void wave_speed_vjp(const R P[4], R bc, R bP[4])
{
    const R usq = P[1] * P[1] + P[2] * P[2];
    const R mod_u = usq > R(0.0) ? M<R>::sq(usq) : R(0.0);
    if (mod_u > R(0.0)) {
        bP[1] += M<R>::div(bc * P[1], mod_u);
        bP[2] += M<R>::div(bc * P[2], mod_u);
    }
    const R a = M<R>::div(P[3], P[0]), sa = M<R>::sq(a);
    const R ba = M<R>::div(bc * R(1.5), sa);
    bP[3] += M<R>::div(ba, P[0]);
    bP[0] += -M<R>::div(ba * P[3], P[0] * P[0]);
}

}  // namespace adj
}  // namespace qlskum
