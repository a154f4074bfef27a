"""Pins the C restatement oracle to the reference's own code.

Two anchors:
* the golden fixtures in tests/golden/, written from the reference compiled
  from its sources (tests/golden/make_golden.py); these travel with the repo;
* when the reference sources are present, the reference itself, rebuilt here
  and run on a freshly generated cloud with other knobs.

On the machine that wrote the fixtures (x86-64, glibc libm) the oracle is
bit-identical to the reference; elsewhere libm may round exp / log / erf /
pow differently by an ulp, so floating-point checks use a relative tolerance
of 1e-12 per stage and 1e-10 after many iterations (the parity bar of the GPU
form).  Sub-stencil classification is integer work and must match exactly.
"""
import os
import platform
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, golden_cloud

EXACT = platform.machine() in ("x86_64", "AMD64")


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.maximum(np.abs(b).max(axis=0, keepdims=True) if b.ndim > 1 else np.abs(b).max(), 1e-300)
    return float((np.abs(a - b) / scale).max())


def test_flux_kat(oracle_mod):
    z = np.load(os.path.join(GOLDEN, "flux_kat.npz"))
    inp, out = z["inputs"], z["outputs"]
    got = np.array([[oracle_mod.flux(k, *row) for k in range(8)] for row in inp])
    if EXACT:
        assert np.array_equal(got, out)
    np.testing.assert_allclose(got, out, rtol=1e-13, atol=0)


def _stage(oracle_mod, inner):
    c = golden_cloud("cloud_trans")
    z = np.load(os.path.join(GOLDEN, "ref_trans_stage.npz"))
    o = oracle_mod.Oracle(c, mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, inner_iterations=inner, threads=2)
    return c, z, o


def test_connectivity_and_normals_exact(oracle_mod):
    c, z, o = _stage(oracle_mod, 2)
    assert np.array_equal(o.sub_counts(), z["sub_counts"])
    cnt = o.sub_counts()
    lists = o.sub_lists()
    flat = np.concatenate([lists[i, d, :cnt[i, d]] for i in range(c.n) for d in range(4)])
    assert np.array_equal(flat, z["sub_lists"])
    if EXACT:
        assert np.array_equal(o.normals, z["normals"])
    np.testing.assert_allclose(o.normals, z["normals"], rtol=0, atol=1e-15)


def test_stage_fields(oracle_mod):
    c, z, o = _stage(oracle_mod, 2)
    hist = o.run(5)
    np.testing.assert_allclose(hist, z["residuals"], rtol=1e-12, atol=1e-300)
    assert rel_err(o.prim, z["prim_in"]) < 1e-12
    o.snapshot_prim_old()
    o.func_delta()
    o.eval_q_variables()
    o.eval_q_derivatives()
    dq0, qm = o.dq, o.qm
    for _ in range(2):
        o.eval_q_inner_loop()
        o.eval_update_innerloop()
    o.cal_flux_residual()
    fr = o.flux_res
    o.state_update(1)
    checks = dict(delta=(o.delta, z["delta"]), q=(o.q, z["q"]), dq0=(dq0, z["dq0"]), qm=(qm, z["qm"]),
                  dq=(o.dq, z["dq"]), flux_res=(fr, z["flux_res"]), prim_out=(o.prim, z["prim_out"]))
    for name, (a, b) in checks.items():
        if EXACT:
            assert np.array_equal(a, b), name
        assert rel_err(a.reshape(c.n, -1), b.reshape(c.n, -1)) < 1e-12, name
    assert abs(o.sum_res_sqr - z["stage_res"][0]) <= 1e-12 * abs(z["stage_res"][0])


def test_small_run(oracle_mod):
    c = golden_cloud("cloud_small")
    z = np.load(os.path.join(GOLDEN, "ref_small_run.npz"))
    o = oracle_mod.Oracle(c, mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, inner_iterations=0, threads=2)
    hist = o.run(50)
    obj = o.objective()
    if EXACT:
        assert np.array_equal(hist, z["residuals"])
        assert np.array_equal(o.prim, z["prim"])
        assert np.array_equal(np.array(obj), z["objectives"])
    np.testing.assert_allclose(hist[:, 0], z["residuals"][:, 0], rtol=1e-10)
    assert rel_err(o.prim, z["prim"]) < 1e-10
    np.testing.assert_allclose(obj, z["objectives"], rtol=1e-10)


def test_threads_do_not_change_results(oracle_mod):
    c = golden_cloud("cloud_trans")
    a = oracle_mod.Oracle(c, mach=0.8, aoa=1.0, cfl=0.2, vl_const=50.0, inner_iterations=1, threads=1)
    b = oracle_mod.Oracle(c, mach=0.8, aoa=1.0, cfl=0.2, vl_const=50.0, inner_iterations=1, threads=4)
    ha, hb = a.run(8), b.run(8)
    assert np.array_equal(ha, hb)
    assert np.array_equal(a.prim, b.prim)


def test_against_reference_build(oracle_mod):
    """Oracle vs the reference compiled here, on a cloud and knobs no fixture uses."""
    from qlskum import cloudgen
    ref = oracle_mod.build_reference()
    if ref is None:
        pytest.skip("reference sources not present (oracle/build_ref.sh built nothing)")
    c = cloudgen.make_cloud(n_wall=48, n_layers=24, first_spacing=5e-3, radius=3.0, seed=23, m=0.02, p=0.4, t=0.1)
    tmp = tempfile.mkdtemp()
    grid = os.path.join(tmp, "g")
    cloudgen.write_partgrid(c, grid)
    kw = dict(mach=0.7, aoa=-1.5, cfl=0.15, vl=80, inner=1, power=-2, iters=12)
    subprocess.check_call([ref, "run", grid, tmp] + [f"{k}={v}" for k, v in kw.items()], cwd=tmp,
                          stdout=subprocess.DEVNULL)
    o = oracle_mod.Oracle(c, mach=0.7, aoa=-1.5, cfl=0.15, vl_const=80.0, power=-2.0, inner_iterations=1, threads=3)
    hist = o.run(12)
    rh = np.fromfile(os.path.join(tmp, "residuals.f64")).reshape(-1, 3)
    rp = np.fromfile(os.path.join(tmp, "prim.f64")).reshape(-1, 4)
    ro = np.fromfile(os.path.join(tmp, "objectives.f64"))
    assert np.isfinite(rh).all()
    assert np.array_equal(hist, rh)
    assert np.array_equal(o.prim, rp)
    assert np.array_equal(np.array(o.objective()), ro)
    # enstrophy of the final state (compute_enstrophy_mod.h), bit for bit
    re = np.fromfile(os.path.join(tmp, "enstrophy.f64"))
    tot, vort = o.enstrophy()
    assert tot == re[0] and np.array_equal(vort, re[1:])
