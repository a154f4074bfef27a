"""Runtime behaviour on the GPU: failure detection, the autotuner, the
objectives reduction, and the error path of the module API."""
import numpy as np
import pytest

from conftest import golden_cloud

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def qlskum():
    import qlskum as q
    q.load()
    return q


def test_nonfinite_state_is_reported_and_recoverable(qlskum):
    """A NaN planted in the state on the host ends the solve with
    QLSKUM_ERR_NONFINITE (the reference would print `nan` and carry on); the
    handle stays usable once a finite state is set again."""
    c = golden_cloud("cloud_small")
    s = qlskum.Solver(c, mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, inner_iterations=0)
    good = s.prim
    bad = good.copy()
    bad[123, 3] = np.nan
    s.set_prim(bad)
    with pytest.raises(qlskum.QlskumError) as e:
        s.q_lskum(2)
    assert e.value.status == 3
    s.set_prim(good)
    s.q_lskum(2)
    assert np.isfinite(s.prim).all()


def test_invalid_stage_number(qlskum):
    s = qlskum.Solver(golden_cloud("cloud_small"), inner_iterations=0)
    with pytest.raises(qlskum.QlskumError) as e:
        s.state_update(5)
    assert e.value.status == 1


def _close(a, b, tol):
    scale = np.maximum(np.abs(b).max(axis=0), 1e-300)
    return float((np.abs(a - b) / scale).max()) <= tol


def test_autotuner_shape_and_result(qlskum):
    """The tuned launch shape changes only roundings: the compiler may fuse an
    FP32 multiply and add differently under another register budget, and the
    residual sum runs in another order.  The state agrees with a fixed
    128-thread launch to FP32 rounding; a pinned shape reproduces itself bit
    for bit."""
    c = golden_cloud("cloud_c1")
    kw = dict(mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, inner_iterations=1, precision=qlskum.MIXED)
    a = qlskum.Solver(c, **kw)
    a.q_lskum(3)
    cfg = a.launch_config()
    assert cfg["flux_block"] in (64, 128, 256) and cfg["point_block"] in (64, 128, 256, 512)
    assert cfg["gather_depth"] in (0, 2, 3, 4)
    b = qlskum.Solver(c, block_size=128, **kw)
    b.q_lskum(3)
    assert b.launch_config() == {"flux_block": 128, "flux_min_blocks": 4, "point_block": 128, "gather_depth": 0,
                                 "flux_variant": 0, "point_lanes": 1, "flux_lanes": 1}
    assert cfg["point_lanes"] in (1, 2, 4) and cfg["flux_lanes"] in (1, 2, 4)
    assert _close(a.prim, b.prim, 1e-5)
    np.testing.assert_allclose(a.residual_history(), b.residual_history(), rtol=1e-3)
    c2 = qlskum.Solver(c, block_size=128, **kw)
    c2.q_lskum(3)
    assert np.array_equal(c2.prim, b.prim)


@pytest.mark.parametrize("flux_variant,staged", [(0, 1), (0, 2), (1, 3), (2, 4), (4, 0), (5, 0), (6, 2), (7, 0)])
def test_staged_gathers_bit_identical(qlskum, flux_variant, staged):
    """The staged kernels (gradient / inner loop: edge list in shared memory;
    flux: next edge's neighbour data in flight by cp.async) do the same
    arithmetic in the same edge order as the per-edge form: the same state to
    FP32 rounding (the compiler's multiply-add fusion may differ between
    launch shapes), with and without unit weights."""
    c = golden_cloud("cloud_c1")
    for power in (0.0, 1.0):
        kw = dict(mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, power=power, inner_iterations=2,
                  precision=qlskum.MIXED)
        a = qlskum.Solver(c, **kw)
        a.set_launch_config(0, 128, 0)
        a.q_lskum(4)
        b = qlskum.Solver(c, **kw)
        b.set_launch_config(flux_variant, 128, staged)
        b.q_lskum(4)
        assert (b.launch_config()["gather_depth"] > 0) == (staged > 0)
        assert _close(b.prim, a.prim, 1e-5), power
        np.testing.assert_allclose(a.residual_history(), b.residual_history(), rtol=1e-3)


@pytest.mark.parametrize("flux_variant,point_lanes", [(8, 1), (9, 1), (0, 2), (0, 4), (8, 2), (9, 4)])
def test_lanes_per_point_match_one_lane(qlskum, flux_variant, point_lanes):
    """2 or 4 lanes per point (a point's edges split over adjacent lanes,
    their sums, maxima and minima combined with warp shuffles) give the
    one-lane state to FP32 rounding (the sums run in another order), in the
    flux kernel (variants 8, 9) and in the gradient / inner-loop kernels,
    with and without unit weights."""
    c = golden_cloud("cloud_c1")
    for power in (0.0, 1.0):
        kw = dict(mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, power=power, inner_iterations=2,
                  precision=qlskum.MIXED)
        a = qlskum.Solver(c, **kw)
        a.set_launch_config(0, 128, 0)
        a.q_lskum(4)
        b = qlskum.Solver(c, **kw)
        b.set_launch_config(flux_variant, 128, 0, point_lanes=point_lanes)
        b.q_lskum(4)
        cfg = b.launch_config()
        assert cfg["point_lanes"] == point_lanes and cfg["flux_lanes"] == {8: 2, 9: 4}.get(flux_variant, 1)
        assert _close(b.prim, a.prim, 1e-5), power
        np.testing.assert_allclose(a.residual_history(), b.residual_history(), rtol=1e-3)


@pytest.mark.parametrize("flux_variant", [10, 13, 14, 16, 17, 18])
def test_flux_forms_match_per_edge_form(qlskum, flux_variant):
    """The register-prefetch forms of the flux kernel (10..13: the next
    edge's neighbour data in registers, 256-bit gathers; 14..18: the owner's
    data in shared memory, with or without the neighbour data prefetched)
    give the per-edge form's state to FP32 rounding, with and without unit
    weights."""
    c = golden_cloud("cloud_c1")
    for power in (0.0, 1.0):
        kw = dict(mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, power=power, inner_iterations=2,
                  precision=qlskum.MIXED)
        a = qlskum.Solver(c, **kw)
        a.set_launch_config(0, 128, 0)
        a.q_lskum(4)
        b = qlskum.Solver(c, **kw)
        b.set_launch_config(flux_variant, 128, 0)
        b.q_lskum(4)
        assert b.launch_config()["flux_variant"] == flux_variant
        assert _close(b.prim, a.prim, 1e-5), power
        np.testing.assert_allclose(a.residual_history(), b.residual_history(), rtol=1e-3)


def test_objective_matches_host_sum(qlskum, oracle_mod):
    """Cl / Cd / Cm / entropy of the same state from the device reduction and
    from the oracle (compute_force_coeffs_mod.h, compute_entropy_mod.h)."""
    c = golden_cloud("cloud_c1")
    s = qlskum.Solver(c, mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, inner_iterations=0)
    s.q_lskum(20)
    o = oracle_mod.Oracle(c, mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, inner_iterations=0, threads=8)
    o.set_prim(s.prim)
    np.testing.assert_allclose(s.objective(), o.objective(), rtol=1e-12)
    ent = s.field(qlskum.FIELD_ENTROPY)
    assert np.isfinite(ent).all() and (ent >= 0).all()


def test_fpi_solver_verbose_line(qlskum, capfd):
    """verbose=1 prints fpi_solver_mod.h:150's line for each iteration."""
    s = qlskum.Solver(golden_cloud("cloud_small"), mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, inner_iterations=0,
                      verbose=True)
    for it in range(1, 4):
        s.fpi_solver(it)
    out = capfd.readouterr().out.strip().splitlines()
    assert out[0] == "iterations 1 residue : 0.0000000000000e+00"
    assert out[2].startswith("iterations 3 residue : ")
    r3 = s.residual_history()[2, 1]
    assert float(out[2].split(":")[1]) == pytest.approx(r3, rel=1e-12)
