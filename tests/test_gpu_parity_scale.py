"""Oracle parity at the benchmark workloads' scale, through the C ABI.

* The FP64 drop-in on the 1,024,000-point transonic cloud (1024 wall points
  x 1000 rings, M 0.85, AoA 1, CFL 0.2, VL_CONST 50, 3 inner iterations)
  against the C restatement of the reference's serial path on all host
  threads: 1e-10 relative in the primitive state, the residual history,
  Cl / Cd / Cm and the total entropy after 5 iterations; sub-stencil
  classification bit-exact.  The mixed form on the same cloud against the
  same oracle run, at the mixed form's tolerance.
* A reduced two-element cloud (NACA 0012 main element and a 30%-chord flap
  at 20 deg, 1.5%-chord slot, 4096 + 1024 wall points, about 100 k points),
  M 0.2, AoA 8: FP64 against the oracle at 1e-10 over 10 iterations.
* Batched cases (several NACA 4-digit clouds of uneven size and flight
  conditions in one batch, mixed precision, 3 inner iterations) against the
  oracle run of each case.

The mixed form's tolerance (as in the mixed-vs-FP64 tests): |dCl|, |dCd|
<= 1e-5; the state within 1e-4 of each component's largest magnitude; the
residual norm of every iteration within 1e-3 relative.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = max(1, os.cpu_count() or 1)


def rel_err(a, b):
    a = np.asarray(a, np.float64).reshape(len(a), -1)
    b = np.asarray(b, np.float64).reshape(len(b), -1)
    scale = np.maximum(np.abs(b).max(axis=0, keepdims=True), 1e-300)
    return float((np.abs(a - b) / scale).max())


@pytest.fixture(scope="module")
def qlskum():
    import qlskum as q
    q.load()
    return q


def check_fp64(s, o, hist_o):
    """The FP64 bar: prim, residual history, objectives at 1e-10 relative."""
    h = s.residual_history()
    assert h.shape == hist_o.shape
    np.testing.assert_allclose(h[:, 0], hist_o[:, 0], rtol=1e-10)
    np.testing.assert_allclose(h[:, 2], hist_o[:, 2], rtol=1e-10)
    assert rel_err(s.prim, o.prim) < 1e-10
    np.testing.assert_allclose(s.objective(), o.objective(), rtol=1e-10)


def check_mixed(prim, hist, obj, o, hist_o):
    """The mixed form's bar against the FP64 oracle."""
    assert np.isfinite(prim).all()
    assert rel_err(prim, o.prim) < 1e-4
    np.testing.assert_allclose(hist, hist_o[:, 0], rtol=1e-3)
    cl, cd = obj[:2]
    ocl, ocd = o.objective()[:2]
    assert abs(cl - ocl) <= 1e-5 and abs(cd - ocd) <= 1e-5, (cl, ocl, cd, ocd)


def test_fp64_full_size_transonic_vs_oracle(qlskum, oracle_mod):
    from qlskum import cloudgen
    c = cloudgen.config2_cloud()
    assert c.n == 1024000
    kw = dict(mach=0.85, aoa=1.0, cfl=0.2, vl_const=50.0, power=0.0, inner_iterations=3)
    iters = 5
    o = oracle_mod.Oracle(c, threads=THREADS, **kw)
    s = qlskum.Solver(c, precision=qlskum.FP64, **kw)
    counts, lists = s.connectivity()
    assert np.array_equal(counts, o.sub_counts())
    used = np.arange(lists.shape[2])[None, None, :] < counts[:, :, None]
    assert np.array_equal(lists[used], o.sub_lists()[used])
    hist_o = o.run(iters)
    s.q_lskum(iters)
    check_fp64(s, o, hist_o)
    s.close()
    m = qlskum.Solver(c, precision=qlskum.MIXED, **kw)
    m.q_lskum(iters)
    check_mixed(m.prim, m.residual_history()[:, 0], m.objective(), o, hist_o)


def test_two_element_reduced_fp64_vs_oracle(qlskum, oracle_mod):
    from qlskum import cloudgen
    c = cloudgen.two_element_cloud(h0=1e-3, growth=0.15)
    assert 50_000 < c.n < 200_000
    assert int((c.flag_2 == 1).sum()) == 4096 and int((c.flag_2 == 2).sum()) == 1024
    kw = dict(mach=0.2, aoa=8.0, cfl=0.2, vl_const=50.0, power=0.0, inner_iterations=0)
    iters = 10
    o = oracle_mod.Oracle(c, threads=THREADS, **kw)
    s = qlskum.Solver(c, precision=qlskum.FP64, **kw)
    counts, _ = s.connectivity()
    assert np.array_equal(counts, o.sub_counts())
    hist_o = o.run(iters)
    s.q_lskum(iters)
    check_fp64(s, o, hist_o)


def test_batched_cases_vs_oracle(qlskum, oracle_mod):
    """Three NACA 4-digit clouds of uneven size (thickness 9-15%, camber
    0-4%), five flight conditions in M 0.5-0.85, AoA -2..4 deg, solved in
    one batch; every case against the oracle's run of that case."""
    from qlskum import cloudgen
    clouds = [cloudgen.make_cloud(n_wall=128, n_layers=160, first_spacing=2e-3, radius=20.0, seed=101,
                                  m=0.03, p=0.35, t=0.15),
              cloudgen.make_cloud(n_wall=96, n_layers=110, first_spacing=2e-3, radius=20.0, seed=102,
                                  m=0.0, p=0.4, t=0.09),
              cloudgen.make_cloud(n_wall=160, n_layers=200, first_spacing=2e-3, radius=20.0, seed=103,
                                  m=0.04, p=0.5, t=0.12)]
    cases = [(0, 0.52, 3.5), (1, 0.78, -1.5), (2, 0.66, 2.0), (0, 0.84, 0.5), (2, 0.71, -2.0)]
    kw = dict(cfl=0.2, vl_const=50.0, power=0.0, inner_iterations=3)
    iters = 10
    b = qlskum.Batch(clouds, cases, **kw)
    b.run(iters)
    cl, cd, cm, ent = b.objective()
    hist = b.residual_history()
    assert hist.shape == (iters, len(cases))
    for k, (ci, mach, aoa) in enumerate(cases):
        o = oracle_mod.Oracle(clouds[ci], mach=mach, aoa=aoa, threads=THREADS, **kw)
        hist_o = o.run(iters)
        check_mixed(b.prim(k), hist[:, k], (cl[k], cd[k]), o, hist_o)
        o.close()
