"""Hand-written reverse mode of the per-point / per-edge arithmetic, checked on
the CPU against central finite differences of the forward functions (the
same source compiled for the host).  For a random direction v and a random
output weight w:  w . (f(x + h v) - f(x - h v)) / 2h  ==  vjp(x, w) . v.
Relative tolerance 1e-6 (h ~ 1e-6 relative; FP64)."""
import ctypes as C

import numpy as np
import pytest

dp = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def L():
    """The test-only host build of the per-point arithmetic (not part of libqlskum.so)."""
    from qlskum import build
    lib = C.CDLL(build.build_vjp_host())
    sig = {
        "qlskum_dbg_prim_to_q": [dp, dp], "qlskum_dbg_prim_to_q_vjp": [dp, dp, dp],
        "qlskum_dbg_qtilde_to_prim": [dp, dp], "qlskum_dbg_qtilde_to_prim_vjp": [dp, dp, dp],
        "qlskum_dbg_dir_flux": [C.c_int, C.c_int, C.c_double, C.c_double, dp, dp],
        "qlskum_dbg_dir_flux_vjp": [C.c_int, C.c_int, C.c_double, C.c_double, dp, dp, dp],
        "qlskum_dbg_edge_end": [dp, C.c_double, C.c_double, C.c_double, dp],
        "qlskum_dbg_edge_end_vjp": [dp, C.c_double, C.c_double, C.c_double, dp, dp],
        "qlskum_dbg_stage_update": [C.c_int, C.c_double, C.c_double, dp, dp, dp, C.c_int, C.c_double, C.c_double, dp],
        "qlskum_dbg_stage_update_vjp": [C.c_int, C.c_double, C.c_double, dp, dp, dp, C.c_int, C.c_double, C.c_double,
                                        dp, dp],
        "qlskum_dbg_wave_speed_vjp": [dp, C.c_double, dp],
        "qlskum_dbg_venkat_vjp": [C.c_double] * 6 + [dp],
    }
    for k, a in sig.items():
        getattr(lib, k).argtypes = a
        getattr(lib, k).restype = None
    lib.qlskum_dbg_wave_speed.argtypes = [dp]
    lib.qlskum_dbg_wave_speed.restype = C.c_double
    lib.qlskum_dbg_venkat.argtypes = [C.c_double] * 5
    lib.qlskum_dbg_venkat.restype = C.c_double
    return lib


def P(a):
    return np.ascontiguousarray(a, np.float64).ctypes.data_as(dp)


def check(fwd, vjp, x, nout, rng, h=1e-6, rtol=1e-6, trials=4):
    """Dot-product test of vjp against central differences of fwd."""
    for _ in range(trials):
        v = rng.standard_normal(x.shape)
        w = rng.standard_normal(nout)
        fp = fwd(x + h * v)
        fm = fwd(x - h * v)
        lhs = float(w @ (fp - fm) / (2 * h))
        rhs = float(vjp(x, w) @ v)
        assert abs(lhs - rhs) <= rtol * max(1.0, abs(lhs), abs(rhs)), (lhs, rhs)


def state(rng):
    return np.array([rng.uniform(0.7, 1.3), rng.uniform(-0.9, 0.9), rng.uniform(-0.5, 0.5), rng.uniform(0.5, 0.9)])


def test_prim_to_q(L):
    rng = np.random.default_rng(1)
    for _ in range(10):
        x = state(rng)

        def f(z):
            o = np.zeros(4)
            L.qlskum_dbg_prim_to_q(P(z), P(o))
            return o

        def vj(z, w):
            o = np.zeros(4)
            L.qlskum_dbg_prim_to_q_vjp(P(z), P(w), P(o))
            return o
        check(f, vj, x, 4, rng)


def test_qtilde_to_prim(L):
    rng = np.random.default_rng(2)
    for _ in range(10):
        pr = state(rng)
        q = np.zeros(4)
        L.qlskum_dbg_prim_to_q(P(pr), P(q))

        def f(z):
            o = np.zeros(4)
            L.qlskum_dbg_qtilde_to_prim(P(z), P(o))
            return o

        def vj(z, w):
            o = np.zeros(4)
            L.qlskum_dbg_qtilde_to_prim_vjp(P(z), P(w), P(o))
            return o
        check(f, vj, q, 4, rng)


@pytest.mark.parametrize("f,D", [(1, 0), (1, 1), (1, 2), (1, 3), (0, 0), (0, 1), (0, 3), (2, 0), (2, 1), (2, 2)])
def test_dir_flux_state_and_normal(L, f, D):
    """Split (interior) and quadrant (wall / outer) fluxes, w.r.t. state and normal."""
    rng = np.random.default_rng(10 * f + D)
    for _ in range(6):
        th = rng.uniform(0, 2 * np.pi)
        x = np.concatenate([state(rng), [np.cos(th), np.sin(th)]])

        def fw(z):
            o = np.zeros(4)
            L.qlskum_dbg_dir_flux(f, D, z[4], z[5], P(z[:4]), P(o))
            return o

        def vj(z, w):
            o = np.zeros(6)
            L.qlskum_dbg_dir_flux_vjp(f, D, z[4], z[5], P(z[:4]), P(w), P(o))
            return o
        check(fw, vj, x, 4, rng)


def test_venkat_limiter(L):
    rng = np.random.default_rng(3)
    n = 0
    while n < 20:
        q = rng.uniform(-1, 1)
        qmax = q + rng.uniform(1e-3, 0.1)
        qmin = q - rng.uniform(1e-3, 0.1)
        qt = q + rng.uniform(-0.2, 0.2)
        e2 = rng.uniform(1e-8, 1e-4)
        if abs(qt - q) < 1e-4:
            continue
        phi = L.qlskum_dbg_venkat(qt, q, qmax, qmin, e2)
        if phi >= 1.0 - 1e-6:
            continue
        n += 1
        x = np.array([qt, q, qmax, qmin])

        def f(z):
            return np.array([L.qlskum_dbg_venkat(z[0], z[1], z[2], z[3], e2)])

        def vj(z, w):
            o = np.zeros(4)
            L.qlskum_dbg_venkat_vjp(z[0], z[1], z[2], z[3], e2, float(w[0]), P(o))
            return o
        check(f, vj, x, 1, rng, h=1e-8)


def test_edge_end_reconstruction(L):
    """q~ = q - 0.5 phi g over 4 components: bars of q, dq, qm and the edge vector."""
    rng = np.random.default_rng(4)
    for _ in range(8):
        q = rng.uniform(-1, 1, 4)
        x = np.concatenate([q, rng.uniform(-5, 5, 8), q + rng.uniform(1e-3, 0.05, 4), q - rng.uniform(1e-3, 0.05, 4),
                            rng.uniform(-0.01, 0.01, 2)])
        e2 = 1e-7

        def f(z):
            o = np.zeros(4)
            L.qlskum_dbg_edge_end(P(z[:20]), e2, z[20], z[21], P(o))
            return o

        def vj(z, w):
            o = np.zeros(22)
            L.qlskum_dbg_edge_end_vjp(P(z[:20]), e2, z[20], z[21], P(w), P(o))
            return o
        check(f, vj, x, 4, rng, h=1e-8)


@pytest.mark.parametrize("f,D", [(1, 0), (1, 1), (1, 2), (1, 3), (0, 0), (0, 1), (0, 3), (2, 0), (2, 1), (2, 2)])
def test_fp64_edge_end_reverse(L, f, D):
    """The FP64 flux reverse's unit (adj::end64 + end64_vjp): limited
    reconstruction, q~ -> prim and the half-range flux of one edge end,
    w.r.t. q, dq, qm, the edge vector and the normal, against central
    differences of the solver's own forward functions; its kept forward
    state gives the solver's flux to rounding, and the reverse from the
    forward's kept transcendentals equals it to rounding."""
    sig = [C.c_int, C.c_int, dp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]
    L.qlskum_dbg_end_flux.argtypes = sig + [dp]
    L.qlskum_dbg_end64_flux.argtypes = sig + [dp]
    L.qlskum_dbg_end64_flux_vjp.argtypes = sig + [dp, dp]
    L.qlskum_dbg_end64_flux_vjp_kept.argtypes = sig + [dp, dp]
    for fn in ("qlskum_dbg_end_flux", "qlskum_dbg_end64_flux", "qlskum_dbg_end64_flux_vjp",
               "qlskum_dbg_end64_flux_vjp_kept"):
        getattr(L, fn).restype = None
    rng = np.random.default_rng(50 + 10 * f + D)
    e2 = 1e-7
    n_lim = 0
    for _ in range(8):
        q = np.zeros(4)
        L.qlskum_dbg_prim_to_q(P(state(rng)), P(q))
        scale = np.abs(q) + 0.1
        dq = rng.uniform(-2, 2, 8) * np.tile(scale, 2)
        th = rng.uniform(0, 2 * np.pi)
        x = np.concatenate([q, dq, q + rng.uniform(1e-4, 0.02, 4) * scale, q - rng.uniform(1e-4, 0.02, 4) * scale,
                            rng.uniform(-0.01, 0.01, 2), [np.cos(th), np.sin(th)]])
        g = x[20] * x[4:8] + x[21] * x[8:12]
        n_lim += sum(L.qlskum_dbg_venkat(q[r] - 0.5 * g[r], q[r], x[12 + r], x[16 + r], e2) < 1.0 for r in range(4))

        def fwd(z, fn=L.qlskum_dbg_end_flux):
            o = np.zeros(4)
            fn(f, D, P(z[:20]), e2, z[20], z[21], z[22], z[23], P(o))
            return o

        def vj(z, w):
            o = np.zeros(24)
            L.qlskum_dbg_end64_flux_vjp(f, D, P(z[:20]), e2, z[20], z[21], z[22], z[23], P(w), P(o))
            return o
        check(fwd, vj, x, 4, rng, h=1e-8, rtol=2e-6)
        np.testing.assert_allclose(fwd(x, L.qlskum_dbg_end64_flux), fwd(x), rtol=1e-13, atol=1e-15)
        # with the transcendentals the forward kept (the recording forward's path)
        w = rng.standard_normal(4)
        kept = np.zeros(24)
        L.qlskum_dbg_end64_flux_vjp_kept(f, D, P(x[:20]), e2, x[20], x[21], x[22], x[23], P(w), P(kept))
        np.testing.assert_allclose(kept, vj(x, w), rtol=1e-10, atol=1e-12 * np.abs(vj(x, w)).max())
    assert n_lim >= 4   # the limiter's phi < 1 branch is exercised


@pytest.mark.parametrize("flag", [0, 1, 2])
@pytest.mark.parametrize("rk", [1, 3])
def test_stage_update(L, flag, rk):
    """SSPRK stage incl. the wall's no-penetration and the far-field mix: bars of
    the state, prim_old, flux residual, normal and free-stream velocity (via
    Mach and AoA)."""
    rng = np.random.default_rng(100 * flag + rk)
    for _ in range(5):
        th = rng.uniform(0, 2 * np.pi)
        mach, aoa = rng.uniform(0.4, 0.85), rng.uniform(-3, 4)
        x = np.concatenate([state(rng), state(rng), rng.uniform(-1e-2, 1e-2, 4), [np.cos(th), np.sin(th)]])

        def f(z, mach=mach, aoa=aoa):
            o = np.zeros(4)
            L.qlskum_dbg_stage_update(flag, z[12], z[13], P(z[:4]), P(z[4:8]), P(z[8:12]), rk, mach, aoa, P(o))
            return o

        def vj(z, w, mach=mach, aoa=aoa):
            o = np.zeros(16)
            L.qlskum_dbg_stage_update_vjp(flag, z[12], z[13], P(z[:4]), P(z[4:8]), P(z[8:12]), rk, mach, aoa, P(w),
                                          P(o))
            return o[:14]
        check(f, vj, x, 4, rng)
        if flag == 2:
            # free-stream velocity through Mach and AoA
            w = rng.standard_normal(4)
            h = 1e-6
            o = np.zeros(16)
            L.qlskum_dbg_stage_update_vjp(flag, x[12], x[13], P(x[:4]), P(x[4:8]), P(x[8:12]), rk, mach, aoa, P(w),
                                          P(o))
            th = np.deg2rad(aoa)
            dmach = o[14] * np.cos(th) + o[15] * np.sin(th)
            fd = w @ (f(x, mach + h, aoa) - f(x, mach - h, aoa)) / (2 * h)
            assert abs(fd - dmach) <= 1e-6 * max(1, abs(fd))


def test_wave_speed(L):
    rng = np.random.default_rng(5)
    for _ in range(10):
        x = state(rng)

        def f(z):
            return np.array([L.qlskum_dbg_wave_speed(P(z))])

        def vj(z, w):
            o = np.zeros(4)
            L.qlskum_dbg_wave_speed_vjp(P(z), float(w[0]), P(o))
            return o
        check(f, vj, x, 1, rng)


def test_fp32_erf_error_bound(L):
    """The mixed form's erf (Abramowitz & Stegun 7.1.26 from the exp(-x^2) the
    kinetic moments already hold): within its published 1.5e-7 absolute bound
    plus FP32 rounding of the evaluation, over the whole real line."""
    import math
    L.qlskum_dbg_erf32.argtypes = [C.c_float]
    L.qlskum_dbg_erf32.restype = C.c_float
    xs = np.concatenate([np.linspace(-6, 6, 4001), np.geomspace(1e-8, 1, 200), -np.geomspace(1e-8, 1, 200)])
    err = max(abs(L.qlskum_dbg_erf32(float(x)) - math.erf(float(np.float32(x)))) for x in xs)
    assert err < 1.5e-7 + 2.4e-7, err
    assert L.qlskum_dbg_erf32(0.0) == 0.0


fp = C.POINTER(C.c_float)


def F32(a):
    return np.ascontiguousarray(a, np.float32).ctypes.data_as(fp)


def test_fp32_instantiations_match_fp64(L):
    """The adjoint of the mixed form runs the same reverse-mode functions in
    FP32: they agree with the FP64 ones to FP32 accuracy (1e-4 of the
    result's scale; the host build uses the libm float functions)."""
    for nm, a in (("qlskum_dbg_prim_to_q_vjp32", [fp] * 3), ("qlskum_dbg_qtilde_to_prim_vjp32", [fp] * 3),
                  ("qlskum_dbg_flux_vjp32", [C.c_int, C.c_float, C.c_float, C.c_float, fp, fp, fp]),
                  ("qlskum_dbg_flux_vjp64", [C.c_int, C.c_double, C.c_double, C.c_double, dp, dp, dp]),
                  ("qlskum_dbg_edge_end_vjp32", [fp, C.c_float, C.c_float, C.c_float, fp, fp]),
                  ("qlskum_dbg_wave_speed_vjp32", [fp, C.c_float, fp])):
        getattr(L, nm).argtypes = a
        getattr(L, nm).restype = None
    rng = np.random.default_rng(9)

    def close(a, b):
        a, b = np.asarray(a, float), np.asarray(b, float)
        assert np.abs(a - b).max() <= 1e-4 * max(1.0, np.abs(b).max()), (a, b)

    for _ in range(20):
        Pst = state(rng)
        bq = rng.standard_normal(4)
        o32, o64 = np.zeros(4, np.float32), np.zeros(4)
        L.qlskum_dbg_prim_to_q_vjp32(F32(Pst), F32(bq), F32(o32))
        L.qlskum_dbg_prim_to_q_vjp(P(Pst), P(bq), P(o64))
        close(o32, o64)
        q = np.zeros(4)
        L.qlskum_dbg_prim_to_q(P(Pst), P(q))
        L.qlskum_dbg_qtilde_to_prim_vjp32(F32(q), F32(bq), F32(o32))
        L.qlskum_dbg_qtilde_to_prim_vjp(P(q), P(bq), P(o64))
        close(o32, o64)
        th = rng.uniform(0, 2 * np.pi)
        for kind in (0, 1, 2):
            s = float(rng.choice([-1.0, 1.0]))
            f32, f64 = np.zeros(6, np.float32), np.zeros(6)
            L.qlskum_dbg_flux_vjp32(kind, s, np.cos(th), np.sin(th), F32(Pst), F32(bq), F32(f32))
            L.qlskum_dbg_flux_vjp64(kind, s, np.cos(th), np.sin(th), P(Pst), P(bq), P(f64))
            close(f32, f64)
        o32 = np.zeros(4, np.float32)
        L.qlskum_dbg_wave_speed_vjp32(F32(Pst), 0.7, F32(o32))
        L.qlskum_dbg_wave_speed_vjp(P(Pst), 0.7, P(o64))
        close(o32, o64)
    for _ in range(10):
        qv = rng.uniform(-1, 1, 4)
        x = np.concatenate([qv, rng.uniform(-5, 5, 8), qv + rng.uniform(1e-2, 0.05, 4), qv - rng.uniform(1e-2, 0.05, 4)])
        bqt = rng.standard_normal(4)
        d = rng.uniform(-0.01, 0.01, 2)
        o32, o64 = np.zeros(22, np.float32), np.zeros(22)
        L.qlskum_dbg_edge_end_vjp32(F32(x), 1e-7, float(d[0]), float(d[1]), F32(bqt), F32(o32))
        L.qlskum_dbg_edge_end_vjp(P(x), 1e-7, float(d[0]), float(d[1]), P(bqt), P(o64))
        close(o32, o64)
