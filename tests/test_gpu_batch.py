"""Batched launches: several flight conditions over clouds of different size
run as one concatenated cloud by the single-cloud kernels, graph-captured.
Each case must give what a single-case mixed-precision solve of the same
cloud and condition gives: with the same launch shape bit for bit (the same
kernels on the same per-point data, and each case starts on a flux block
boundary); with the shapes each autotuner picks, to FP32 rounding.  The
per-case residual sums the same block partials in another order."""
import numpy as np
import pytest

from conftest import golden_cloud, small_cloud

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def qlskum():
    import qlskum as q
    q.load()
    return q


def _clouds():
    return [golden_cloud("cloud_trans"),
            small_cloud(n_wall=48, n_layers=24, first_spacing=5e-3, radius=3.0, seed=5, m=0.03, p=0.4, t=0.14)]


def _close(a, b, tol):
    scale = np.maximum(np.abs(b).max(axis=0), 1e-300)
    return float((np.abs(a - b) / scale).max()) <= tol


CASES = [(0, 0.63, 2.0), (1, 0.70, 3.0), (0, 0.80, -1.0), (1, 0.55, 0.5), (0, 0.85, 1.0)]
KW = dict(cfl=0.2, vl_const=50.0, power=0.0, inner_iterations=1)


def test_batch_matches_single_case_solves(qlskum):
    clouds = _clouds()
    b = qlskum.Batch(clouds, CASES, **KW)
    assert b.total_points == sum(clouds[c].n for c, _, _ in CASES)
    b.run(8)
    cl, cd, cm, ent = b.objective()
    hist = b.residual_history()
    assert hist.shape == (8, len(CASES))
    for k, (ci, mach, aoa) in enumerate(CASES):
        s = qlskum.Solver(clouds[ci], mach=mach, aoa=aoa, precision=qlskum.MIXED, **KW)
        s.q_lskum(8)
        assert _close(b.prim(k), s.prim, 1e-5), k
        np.testing.assert_allclose(hist[:, k], s.residual_history()[:, 0], rtol=1e-3)
        np.testing.assert_allclose([cl[k], cd[k], cm[k], ent[k]], s.objective(), rtol=1e-4, atol=1e-6)


def test_batch_tuning_and_graph_replay(qlskum):
    clouds = _clouds()
    b = qlskum.Batch(clouds, CASES[:3], **KW)
    b.run(2)
    t = b.tuning()
    assert t["tile"] in (64, 128, 256) and t["flux_tile"] in (64, 128, 256)
    assert t["points_per_warp"] == 32 // t["flux_lanes"] and t["point_lanes"] in (1, 2, 4)
    l0 = b.launches
    b.run(3)
    # per iteration: 4 x (gradient + 1 inner + flux) + reduce + counter
    assert b.launches - l0 == 3 * (4 * 3 + 2)
    fixed = qlskum.Batch(clouds, CASES[:3], block_size=128, **KW)
    fixed.run(5)
    for k in range(3):
        assert _close(b.prim(k), fixed.prim(k), 1e-5)


def test_batch_rejects_fp64_and_bad_case(qlskum):
    import ctypes as C
    L = qlskum.load()
    clouds = _clouds()
    s, keep = qlskum.cloud_struct(clouds[0])
    arr = (qlskum.CloudStruct * 1)(s)
    cc = np.array([1], np.int32)
    mm = np.array([0.6])
    aa = np.array([1.0])
    p = qlskum.ParamsStruct(0, 0, 0.2, 50, 0, 1, qlskum.MIXED, 0, 1, 0)
    h = C.c_void_p()
    assert L.qlskum_batch_create(arr, 1, qlskum._ip(cc), qlskum._dp(mm), qlskum._dp(aa), 1, C.byref(p),
                                 C.byref(h)) == 1
    cc[0] = 0
    p.precision = qlskum.FP64
    assert L.qlskum_batch_create(arr, 1, qlskum._ip(cc), qlskum._dp(mm), qlskum._dp(aa), 1, C.byref(p),
                                 C.byref(h)) == 5
    _ = keep


@pytest.mark.parametrize("variant", [17, 8, 4])
def test_batch_is_the_single_cloud_iteration(qlskum, variant):
    """With the same launch shape (the owner-in-shared-memory flux form, the
    2-lanes-per-point form, the staged form) every case's state after 6
    iterations equals the single-case solve's bit for bit."""
    clouds = _clouds()
    b = qlskum.Batch(clouds, CASES, **KW)
    b.set_launch_config(128, 1, variant)
    b.run(6)
    for k, (ci, mach, aoa) in enumerate(CASES):
        s = qlskum.Solver(clouds[ci], mach=mach, aoa=aoa, precision=qlskum.MIXED, **KW)
        s.set_launch_config(variant, 128, 0)
        s.q_lskum(6)
        assert np.array_equal(b.prim(k), s.prim), (variant, k)
        np.testing.assert_allclose(b.residual_history()[:, k], s.residual_history()[:, 0], rtol=1e-12)


def test_batch_weighted_least_squares_is_the_single_cloud_iteration(qlskum):
    """Distance-weighted least squares (power -2: the kernels read the
    weighted edge vectors instead of rotating {delx, dely}), three inner
    steps: every case equals its single-case solve bit for bit."""
    clouds = _clouds()
    kw = dict(KW, power=-2.0, inner_iterations=3)
    b = qlskum.Batch(clouds, CASES[:3], **kw)
    b.set_launch_config(128, 1, 17)
    b.run(5)
    for k, (ci, mach, aoa) in enumerate(CASES[:3]):
        s = qlskum.Solver(clouds[ci], mach=mach, aoa=aoa, precision=qlskum.MIXED, **kw)
        s.set_launch_config(17, 128, 0)
        s.q_lskum(5)
        assert np.array_equal(b.prim(k), s.prim), k


@pytest.mark.parametrize("tile,point_lanes,flux_variant", [(64, 2, 8), (128, 4, 9), (256, 2, 0), (64, 4, 1),
                                                          (128, 1, 5), (128, 2, 11), (64, 1, 17), (256, 1, 14)])
def test_batch_lanes_per_point_match_one_lane(qlskum, tile, point_lanes, flux_variant):
    """Gradient / inner-loop kernels with 2 or 4 lanes per point, and the flux
    variants (2 and 4 lanes per point, the staged, register-prefetch and
    owner-in-shared-memory forms), against the one-lane batch: the same
    state to FP32 rounding."""
    clouds = _clouds()
    a = qlskum.Batch(clouds, CASES[:3], **KW)
    a.set_launch_config(128, 1, 0)
    a.run(5)
    b = qlskum.Batch(clouds, CASES[:3], **KW)
    b.set_launch_config(tile, point_lanes, flux_variant)
    b.run(5)
    t = b.tuning()
    assert t["point_lanes"] == point_lanes and t["tile"] == tile
    assert t["points_per_warp"] == 32 // {8: 2, 9: 4}.get(flux_variant, 1)
    for k in range(3):
        assert _close(b.prim(k), a.prim(k), 1e-5), k
    np.testing.assert_allclose(b.residual_history(), a.residual_history(), rtol=1e-3)
