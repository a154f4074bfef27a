// Per-point and per-edge arithmetic of the q-LSKUM scheme, templated on the
// real type R so the FP64 translation unit, the mixed-precision unit (FP32),
// the reverse-mode unit and the host build of the reverse arithmetic share
// one source.
//
// Each function names the reference lines it restates, in the reference's
// operation order.  Where the reference writes `a - b` for the negative
// half-range we write `a + s*b` with s = -1: IEEE subtraction is addition of
// the negation and s*b is exact.  Compiled without FMA contraction (the host
// build, the noalloc unit) the FP64 results are the reference's bit for bit
// apart from libm; the FP64 device unit contracts multiply-adds and takes
// the faster, equivalent forms venkat_r / end_kin for the edge ends.
#pragma once
#include <cmath>
#include <cuda_runtime.h>
#include "qlskum_internal.h"

// Host + device: the per-point arithmetic is also compiled for the host so
// that its derivatives can be checked on the CPU.
#ifdef __CUDACC__
#define QLSKUM_HD __host__ __device__ __forceinline__
#else
#define QLSKUM_HD inline
#endif

namespace qlskum {

#ifdef __CUDACC__
// Conversions between FP32 and FP64 on the integer pipe (the hardware
// conversion issues on the FP64 pipe, which on this chip is the scarce one).
// float -> double: exact for normal numbers and zero, flushes subnormals to
// zero and keeps Inf / NaN.
__device__ __forceinline__ double f2d(float x)
{
    const unsigned b = __float_as_uint(x);
    const unsigned mag = b & 0x7fffffffu;
    const unsigned sign = b & 0x80000000u;
    unsigned hi = sign | (((mag >> 23) + 896u) << 20) | ((mag & 0x7fffffu) >> 3);
    unsigned lo = b << 29;
    if (mag < 0x00800000u) { hi = sign; lo = 0u; }
    if (mag >= 0x7f800000u) hi = sign | 0x7ff00000u | ((mag & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)lo);
}

// double -> float on the integer pipe, truncating the mantissa (< 1 ulp);
// underflow goes to zero, overflow and Inf to Inf, NaN stays NaN.
__device__ __forceinline__ float d2f(double x)
{
    const unsigned h = (unsigned)__double2hiint(x), l = (unsigned)__double2loint(x);
    const unsigned mag = h & 0x7fffffffu;
    const unsigned sign = h & 0x80000000u;
    const int e = (int)(mag >> 20) - 896;
    const unsigned m = ((mag & 0xfffffu) << 3) | (l >> 29);
    unsigned b = sign | ((unsigned)e << 23) | m;
    if (e <= 0) b = sign;
    if (e >= 255) b = sign | 0x7f800000u | ((mag >= 0x7ff00000u && (m | (mag & 0xfffffu) | l)) ? 0x400000u : 0u);
    return __uint_as_float(b);
}

// double -> float rounded to nearest (ties away from zero) on the integer
// pipe: half an FP32 ulp (bit 28 of the FP64 pattern) added to the
// magnitude, then d2f's truncation; a carry out of the mantissa moves into
// the exponent as it should.  (An infinity comes out as NaN.)
__device__ __forceinline__ float d2f_rn(double x)
{
    return d2f(__longlong_as_double(__double_as_longlong(x) + (1LL << 28)));
}

// 1 / x in FP64 from the FP32 reciprocal refined by two Newton steps (about
// an ulp; no FP64 division).  Where x is outside the normal FP32 range the
// seed is not usable and the division is taken instead.
__device__ __forceinline__ double rcp64(double x)
{
    const float s = __frcp_rn(d2f(x));
    if (!(fabsf(s) > 1e-37f && fabsf(s) < 1e37f)) return 1.0 / x;
    double r = f2d(s);
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}
#endif

// Elementary operations per real type.  For double they are exactly the
// reference's: IEEE division and square root, libm-style exp / log / erf.
// For float (mixed form only) the device uses the special-function unit:
// divisions and square roots through the reciprocal / reciprocal-square-root
// approximations (2 ulp), exp and log through ex2 / lg2 (relative error
// about 2^-21 over the arguments met here); erf comes from erf_e below.
template <typename R> struct M;
template <> struct M<double> {
    static QLSKUM_HD double ex(double x) { return exp(x); }
    static QLSKUM_HD double lg(double x) { return log(x); }
    static QLSKUM_HD double ef(double x) { return erf(x); }
    static QLSKUM_HD double sq(double x) { return sqrt(x); }
    static QLSKUM_HD double ab(double x) { return fabs(x); }
    static QLSKUM_HD double div(double a, double b) { return a / b; }
    // a / sqrt(x)
    static QLSKUM_HD double rdsq(double a, double x) { return a / sqrt(x); }
    // 1 / sqrt(x) (the device's rsqrt: 1 ulp) and 1 / x (rcp64: about an ulp)
#ifdef __CUDA_ARCH__
    static QLSKUM_HD double rsq(double x) { return rsqrt(x); }
    static QLSKUM_HD double rcp(double x) { return rcp64(x); }
#else
    static QLSKUM_HD double rsq(double x) { return 1.0 / std::sqrt(x); }
    static QLSKUM_HD double rcp(double x) { return 1.0 / x; }
#endif
};
template <> struct M<float> {
    static QLSKUM_HD float ef(float x) { return erff(x); }
    static QLSKUM_HD float ab(float x) { return fabsf(x); }
#ifdef __CUDA_ARCH__
    static QLSKUM_HD float ex(float x) { return __expf(x); }
    static QLSKUM_HD float lg(float x) { return __logf(x); }
    static QLSKUM_HD float sq(float x) { return x * rsqrtf(x); }
    static QLSKUM_HD float div(float a, float b) { return __fdividef(a, b); }
    static QLSKUM_HD float rdsq(float a, float x) { return a * rsqrtf(x); }
#else
    static QLSKUM_HD float ex(float x) { return std::exp(x); }
    static QLSKUM_HD float lg(float x) { return std::log(x); }
    static QLSKUM_HD float sq(float x) { return std::sqrt(x); }
    static QLSKUM_HD float div(float a, float b) { return a / b; }
    static QLSKUM_HD float rdsq(float a, float x) { return a / std::sqrt(x); }
#endif
};

// erf(x) given e = exp(-x^2), which the kinetic moments compute anyway.
// double: the libm erf (the reference's; e unused).  float: Abramowitz &
// Stegun 7.1.26, C. Hastings' approximation
//   erf(x) = 1 - (a1 t + a2 t^2 + a3 t^3 + a4 t^4 + a5 t^5) exp(-x^2),
//   t = 1 / (1 + p x),  x >= 0, odd extension,
// absolute error <= 1.5e-7 for every x: one reciprocal and five FMAs in
// place of a separate erf evaluation.
template <typename R> QLSKUM_HD R erf_e(R x, R e);
template <> QLSKUM_HD double erf_e<double>(double x, double) { return erf(x); }
template <> QLSKUM_HD float erf_e<float>(float x, float e)
{
    const float t = M<float>::div(1.0f, fmaf(0.3275911f, fabsf(x), 1.0f));
    float p = fmaf(1.061405429f, t, -1.453152027f);
    p = fmaf(p, t, 1.421413741f);
    p = fmaf(p, t, -0.284496736f);
    p = fmaf(p, t, 0.254829592f);
    return copysignf(fmaf(-p * t, e, 1.0f), x);
}

// 4 * atan(1.0) of parameter_mod.h:10, as a literal.
#define QLSKUM_PI 3.141592653589793

template <typename R> struct V4 { R v[4]; };

QLSKUM_HD void ld4(const double4_32a &a, double o[4]) { o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; }
QLSKUM_HD void ld4(const float4 &a, float o[4]) { o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; }
QLSKUM_HD double4_32a mk4(const double o[4]) { return make_double4_32a(o[0], o[1], o[2], o[3]); }
QLSKUM_HD float4 mk4(const float o[4]) { return make_float4(o[0], o[1], o[2], o[3]); }

// q_variables_mod.h:19-33: q from (rho, u1, u2, p).
template <typename R>
QLSKUM_HD void prim_to_q(R rho, R u1, R u2, R pr, R q[4])
{
    R beta = M<R>::div(R(0.5) * rho, pr);
    q[0] = M<R>::lg(rho) + (M<R>::lg(beta) * R(2.5)) - beta * (u1 * u1 + u2 * u2);
    R two_times_beta = R(2.0) * beta;
    q[1] = two_times_beta * u1;
    q[2] = two_times_beta * u2;
    q[3] = -two_times_beta;
}

// limiters_mod.h:64-104: Venkatakrishnan limiter of one component.
// `eps2` is (pow(VL_CONST * min_dist, 3))^2 of the point the state belongs to.
template <typename R>
QLSKUM_HD R venkat(R qt, R q, R qmax, R qmin, R eps2)
{
    R del_neg = qt - q;
    if (M<R>::ab(del_neg) <= R(10e-6)) return R(1.0);
    R del_pos = (del_neg > R(0)) ? qmax - q : qmin - q;
    R num = (del_pos * del_pos) + eps2;
    num = num * del_neg + R(2.0) * del_neg * del_neg * del_pos;
    R den = del_pos * del_pos + R(2.0) * del_neg * del_neg;
    den = den + del_neg * del_pos + eps2;
    den = den * del_neg;
    R temp = M<R>::div(num, den);
    return temp < R(1) ? temp : R(1);
}

// q_variables_mod.h:230-253
template <typename R>
QLSKUM_HD void qtilde_to_prim(const R qt[4], R &u1, R &u2, R &rho, R &pr)
{
    R beta = -qt[3] * R(0.5);
    R temp = M<R>::div(R(0.5), beta);
    u1 = qt[1] * temp;
    u2 = qt[2] * temp;
    R temp1 = qt[0] + beta * (u1 * u1 + u2 * u2);
    R temp2 = temp1 - M<R>::div(M<R>::lg(beta), R(1.4) - R(1));
    rho = M<R>::ex(temp2);
    pr = rho * temp;
}

// Half-range moments of one state in the point's (t, n) frame, shared by all
// split and quadrant fluxes that state enters (split_fluxes_mod.h:14-26,
// quadrant_fluxes_mod.h:14-29).
template <typename R> struct Kin {
    R rho, ut, un, pbr, usq, B1, B2, E1, E2;
};

// keep != nullptr: also {sqrt(beta), exp(-S1^2), exp(-S2^2)}, which the
// FP64 reverse reads back instead of recomputing them.
template <typename R>
QLSKUM_HD void kin_prep(R nx, R ny, R u1, R u2, R rho, R pr, Kin<R> &k, R *keep = nullptr)
{
    R tx = ny, ty = -nx;
    k.ut = u1 * tx + u2 * ty;
    k.un = u1 * nx + u2 * ny;
    R beta = M<R>::div(R(0.5) * rho, pr);
    R sb = M<R>::sq(beta);
    R S1 = k.ut * sb;
    R S2 = k.un * sb;
    const R e1 = M<R>::ex(-S1 * S1), e2 = M<R>::ex(-S2 * S2);
    if (keep) {
        keep[0] = sb;
        keep[1] = e1;
        keep[2] = e2;
    }
    k.B1 = M<R>::rdsq(R(0.5) * e1, R(QLSKUM_PI) * beta);
    k.B2 = M<R>::rdsq(R(0.5) * e2, R(QLSKUM_PI) * beta);
    k.E1 = erf_e<R>(S1, e1);
    k.E2 = erf_e<R>(S2, e2);
    k.pbr = M<R>::div(pr, rho);
    k.usq = k.ut * k.ut + k.un * k.un;
    k.rho = rho;
}

// One edge end's q~ -> prim step (q_variables_mod.h:230-253) and its
// half-range moments (kin_prep) in one pass, for the FP64 drop-in's
// forward: the moments take beta and p / rho = 0.5 / beta from the q~ ->
// prim step (split_fluxes_mod.h:17-19 forms both again from rho and p, two
// more divisions that give the same values to an ulp); sqrt(beta),
// 1 / sqrt(pi beta) and beta^-2.5 = exp(-log(beta) / (gamma - 1)) come from
// one reciprocal square root (split_fluxes_mod.h:20-26 takes three square
// roots and two divisions, q_variables_mod.h:246-249 a log); 0.5 / beta is
// a reciprocal (rcp64) instead of a division.  Each replacement agrees with
// the reference's expression to a few ulps.  keep as kin_prep.
template <typename R>
QLSKUM_HD void end_kin(R nx, R ny, const R qt[4], Kin<R> &k, R *keep = nullptr)
{
    const R beta = -qt[3] * R(0.5);
    const R temp = R(0.5) * M<R>::rcp(beta);
    const R u1 = qt[1] * temp, u2 = qt[2] * temp;
    const R temp1 = qt[0] + beta * (u1 * u1 + u2 * u2);
    const R rsb = M<R>::rsq(beta);
    // exp(temp1 - log(beta) / (gamma - 1)) = exp(temp1) beta^-2.5, gamma = 1.4
    const R rsb2 = rsb * rsb;
    k.rho = M<R>::ex(temp1) * (rsb2 * rsb2 * rsb);
    const R tx = ny, ty = -nx;
    k.ut = u1 * tx + u2 * ty;
    k.un = u1 * nx + u2 * ny;
    const R sb = beta * rsb;
    const R S1 = k.ut * sb;
    const R S2 = k.un * sb;
    const R e1 = M<R>::ex(-S1 * S1), e2 = M<R>::ex(-S2 * S2);
    if (keep) {
        keep[0] = sb;
        keep[1] = e1;
        keep[2] = e2;
    }
    // 0.5 / sqrt(pi beta) = (0.5 / sqrt(pi)) / sqrt(beta)
    const R hrs = R(0.28209479177387814) * rsb;
    k.B1 = hrs * e1;
    k.B2 = hrs * e2;
    k.E1 = erf_e<R>(S1, e1);
    k.E2 = erf_e<R>(S2, e2);
    k.pbr = temp;
    k.usq = k.ut * k.ut + k.un * k.un;
}

// flux_Gxp (s1 = +1) / flux_Gxn (s1 = -1): split_fluxes_mod.h:6-84
template <typename R>
QLSKUM_HD void flux_x(const Kin<R> &k, R s1, R G[4])
{
    R A1 = R(0.5) * (R(1.0) + s1 * k.E1);
    R B1 = s1 * k.B1;
    G[0] = k.rho * (k.ut * A1 + B1);
    R temp1 = k.pbr + k.ut * k.ut;
    R temp2 = temp1 * A1 + k.ut * B1;
    G[1] = k.rho * temp2;
    temp1 = k.ut * k.un * A1 + k.un * B1;
    G[2] = k.rho * temp1;
    temp1 = (R(7.0) * k.pbr) + k.usq;
    temp2 = R(0.5) * k.ut * temp1 * A1;
    temp1 = (R(6.0) * k.pbr) + k.usq;
    G[3] = k.rho * (temp2 + R(0.5) * temp1 * B1);
}

// flux_Gyp (s2 = +1) / flux_Gyn (s2 = -1): split_fluxes_mod.h:86-164
template <typename R>
QLSKUM_HD void flux_y(const Kin<R> &k, R s2, R G[4])
{
    R A2 = R(0.5) * (R(1.0) + s2 * k.E2);
    R B2 = s2 * k.B2;
    G[0] = k.rho * (k.un * A2 + B2);
    R temp1 = k.pbr + k.un * k.un;
    R temp2 = temp1 * A2 + k.un * B2;
    G[2] = k.rho * temp2;
    temp1 = k.ut * k.un * A2 + k.ut * B2;
    G[1] = k.rho * temp1;
    temp1 = (R(7.0) * k.pbr) + k.usq;
    temp2 = R(0.5) * k.un * temp1 * A2;
    temp1 = (R(6.0) * k.pbr) + k.usq;
    G[3] = k.rho * (temp2 + R(0.5) * temp1 * B2);
}

// flux_quad_GxI (-,-), GxII (+,-), GxIII (+,+), GxIV (-,+):
// quadrant_fluxes_mod.h:6-211, s1 the t half-range sign, s2 the n one.
template <typename R>
QLSKUM_HD void flux_quad(const Kin<R> &k, R s1, R s2, R G[4])
{
    R A1 = R(0.5) * (R(1.0) + s1 * k.E1);
    R A2 = R(0.5) * (R(1.0) + s2 * k.E2);
    R B1 = s1 * k.B1;
    R f1 = k.ut * A1 + B1;
    G[0] = k.rho * A2 * f1;
    R temp1 = k.pbr + k.ut * k.ut;
    R temp2 = temp1 * A1 + k.ut * B1;
    G[1] = k.rho * A2 * temp2;
    temp2 = k.un * A2 + s2 * k.B2;
    G[2] = k.rho * f1 * temp2;
    temp1 = (R(7.0) * k.pbr) + k.usq;
    temp2 = R(0.5) * k.ut * temp1 * A1;
    temp1 = (R(6.0) * k.pbr) + k.usq;
    R temp3 = R(0.5) * k.B1 * temp1;
    R temp4 = R(0.5) * k.rho * k.un * k.B2 * f1;
    G[3] = k.rho * A2 * (temp2 + s1 * temp3) + s2 * temp4;
}

// Flux at one end of an edge for sub-stencil d of a point of class f
// (flux_residual_mod.h:18-87 picks the function per class and direction).
template <typename R, int D>
QLSKUM_HD void dir_flux(int f, const Kin<R> &k, R G[4])
{
    if (D <= 1) {
        const R s1 = (D == 0) ? R(1) : R(-1);
        if (f == kInterior) flux_x(k, s1, G);
        else flux_quad(k, s1, (f == kOuter) ? R(1) : R(-1), G);
    } else {
        flux_y(k, (D == 2) ? R(1) : R(-1), G);
    }
}

// Limited reconstruction of both ends of edge (i, k) and their primitive
// states (interior_fluxes_mod.h:50-89 and the identical blocks of the wall
// and outer modules).  g = (delx, dely).
template <typename R>
QLSKUM_HD void edge_states(R delx, R dely, const R qi[4], const R dxi[4], const R dyi[4],
                                            const R mxi[4], const R mni[4], R e2i, const R qk[4],
                                            const R dxk[4], const R dyk[4], const R mxk[4], const R mnk[4],
                                            R e2k, R pi_[4], R pk_[4])
{
    R ti[4], tk[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        R gi = delx * dxi[r] + dely * dyi[r];
        R gk = delx * dxk[r] + dely * dyk[r];
        R phi_i = venkat(qi[r] - R(0.5) * gi, qi[r], mxi[r], mni[r], e2i);
        R phi_k = venkat(qk[r] - R(0.5) * gk, qk[r], mxk[r], mnk[r], e2k);
        ti[r] = qi[r] - R(0.5) * phi_i * gi;
        tk[r] = qk[r] - R(0.5) * phi_k * gk;
    }
    qtilde_to_prim(ti, pi_[1], pi_[2], pi_[0], pi_[3]);
    qtilde_to_prim(tk, pk_[1], pk_[2], pk_[0], pk_[3]);
}

// venkat() with the common factor del_neg of the numerator and the
// denominator cancelled (both are multiplied by it in limiters_mod.h:93-97)
// and the quotient taken through a reciprocal: the same value to a few ulps.
template <typename R>
QLSKUM_HD R venkat_r(R qt, R q, R qmax, R qmin, R eps2)
{
    const R dn = qt - q;
    if (M<R>::ab(dn) <= R(10e-6)) return R(1.0);
    const R dp = (dn > R(0)) ? qmax - q : qmin - q;
    const R base = dp * dp + eps2;
    const R num = base + R(2.0) * dn * dp;
    const R den = base + dn * (R(2.0) * dn + dp);
    const R t = num * M<R>::rcp(den);
    return t < R(1) ? t : R(1);
}

// The limited reconstruction of edge_states, each end's q~ returned.
template <typename R>
QLSKUM_HD void edge_qtilde(R delx, R dely, const R qi[4], const R dxi[4], const R dyi[4], const R mxi[4],
                           const R mni[4], R e2i, const R qk[4], const R dxk[4], const R dyk[4], const R mxk[4],
                           const R mnk[4], R e2k, R ti[4], R tk[4])
{
#pragma unroll
    for (int r = 0; r < 4; r++) {
        R gi = delx * dxi[r] + dely * dyi[r];
        R gk = delx * dxk[r] + dely * dyk[r];
        R phi_i = venkat_r(qi[r] - R(0.5) * gi, qi[r], mxi[r], mni[r], e2i);
        R phi_k = venkat_r(qk[r] - R(0.5) * gk, qk[r], mxk[r], mnk[r], e2k);
        ti[r] = qi[r] - R(0.5) * phi_i * gi;
        tk[r] = qk[r] - R(0.5) * phi_k * gk;
    }
}

// state_update_mod.h:18-33
QLSKUM_HD void primitive_to_conserved(const double P[4], double nx, double ny, double U[4])
{
    double rho = P[0];
    U[0] = rho;
    double temp1 = rho * P[1];
    double temp2 = rho * P[2];
    U[3] = 2.5 * P[3] + 0.5 * (temp1 * temp1 + temp2 * temp2) / rho;
    U[1] = temp1 * ny - temp2 * nx;
    U[2] = temp1 * nx + temp2 * ny;
}

// state_update_mod.h:35-90
QLSKUM_HD void conserved_vector_Ubar(const CaseConst &K, const double P[4], double nx, double ny,
                                                      double Ubar[4])
{
    const double gamma_new = K.gamma, rho_inf = K.rho_inf, pr_inf = K.pr_inf, pi = K.pi;
    double tx = ny, ty = -nx;
    double u1_inf_rot = K.u1_inf * tx + K.u2_inf * ty;
    double u2_inf_rot = K.u1_inf * nx + K.u2_inf * ny;
    double temp1 = (u1_inf_rot * u1_inf_rot + u2_inf_rot * u2_inf_rot);
    double e_inf = pr_inf / (rho_inf * (gamma_new - 1.0)) + 0.5 * (temp1);
    double beta = (0.5 * rho_inf) / pr_inf;
    double S2 = u2_inf_rot * sqrt(beta);
    double B2_inf = exp(-S2 * S2) / (2.0 * sqrt(pi * beta));
    double A2n_inf = 0.5 * (1.0 - erf(S2));
    double rho = P[0], u1 = P[1], u2 = P[2], pr = P[3];
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

// One SSPRK stage of one point (state_update_mod.h:111-282).  P is updated in
// place; returns the point's res_sqr (0 on outer points, which the reference
// leaves out of the residual).
QLSKUM_HD double stage_update(const CaseConst &K, int f, double nx, double ny, double P[4],
                                               const double4_32a *prim_old_i, const double F[4], int rk)
{
    const double obt = 1.0 / 3.0, tbt = 2.0 / 3.0, euler = 1.0;
    double U[4], U_old[4];
    if (f == kOuter) conserved_vector_Ubar(K, P, nx, ny, U);
    else primitive_to_conserved(P, nx, ny, U);
    double temp = U[0];
    if (rk != 3) {
#pragma unroll
        for (int j = 0; j < 4; j++) U[j] = U[j] - (0.5 * euler * F[j]);
    } else {
        double Po[4];
        ld4(*prim_old_i, Po);
        if (f == kOuter) conserved_vector_Ubar(K, Po, nx, ny, U_old);
        else primitive_to_conserved(Po, nx, ny, U_old);
#pragma unroll
        for (int j = 0; j < 4; j++) U[j] = tbt * U_old[j] + obt * (U[j] - 0.5 * F[j]);
    }
    if (f == kWall) U[2] = 0.;
    double U2_rot = U[1], U3_rot = U[2];
    U[1] = U2_rot * ny + U3_rot * nx;
    U[2] = U3_rot * ny - U2_rot * nx;
    double res_sqr = (f == kOuter) ? 0.0 : (U[0] - temp) * (U[0] - temp);
    P[0] = U[0];
    temp = 1.0 / U[0];
    P[1] = U[1] * temp;
    P[2] = U[2] * temp;
    P[3] = 0.4 * U[3] - (0.2 * temp) * (U[1] * U[1] + U[2] * U[2]);
    return res_sqr;
}

// |u| + 3 sqrt(p / rho) of state_update_mod.h:483-485, the denominator of the
// local time step a neighbour contributes.
QLSKUM_HD double wave_speed(const double P[4])
{
    double mod_u = sqrt(P[1] * P[1] + P[2] * P[2]);
    return mod_u + 3.0 * sqrt(P[3] / P[0]);
}

#ifdef __CUDACC__
// Deterministic block reduction (sum and max) of one value per thread.
template <int BLOCK>
__device__ __forceinline__ void block_sum_max(double v, double m, double *out_sum, double *out_max)
{
    __shared__ double ss[BLOCK / 32], sm[BLOCK / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_down_sync(0xffffffffu, v, o);
        double t = __shfl_down_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { ss[w] = v; sm[w] = m; }
    __syncthreads();
    if (w == 0) {
        v = (l < BLOCK / 32) ? ss[l] : 0.0;
        m = (l < BLOCK / 32) ? sm[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            v += __shfl_down_sync(0xffffffffu, v, o);
            double t = __shfl_down_sync(0xffffffffu, m, o);
            m = t > m ? t : m;
        }
        if (l == 0) { *out_sum = v; *out_max = m; }
    }
}

__device__ __forceinline__ long long ell(const DevCloud &c, int i, int j)
{
    return c.slice_base[i >> 5] + 32LL * j + (i & 31);
}

#endif  // __CUDACC__

}  // namespace qlskum
