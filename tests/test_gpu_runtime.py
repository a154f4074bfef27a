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


def test_autotuner_shape_and_result(qlskum):
    """The tuned launch shape changes only the order of the residual sum:
    the state is bit-identical to a fixed 128-thread launch."""
    c = golden_cloud("cloud_c1")
    kw = dict(mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, inner_iterations=1, precision=qlskum.MIXED)
    a = qlskum.Solver(c, **kw)
    a.q_lskum(3)
    cfg = a.launch_config()
    assert cfg["flux_block"] in (64, 128, 256) and cfg["point_block"] in (64, 128, 256, 512)
    b = qlskum.Solver(c, block_size=128, **kw)
    b.q_lskum(3)
    assert b.launch_config() == {"flux_block": 128, "flux_min_blocks": 4, "point_block": 128}
    assert np.array_equal(a.prim, b.prim)
    np.testing.assert_allclose(a.residual_history(), b.residual_history(), rtol=1e-13)


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
