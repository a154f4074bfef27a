"""Discrete adjoint of the iteration (FP64, and the mixed form), through the C ABI.

* qlskum_residual_forward reproduces the reference's first-stage flux
  residual (golden fixture, 1e-12 like the stage parity test), and its VJP
  passes the dot-product test against central differences of the forward.
* qlskum_adjoint_gradient differentiates Cl / Cd after N iterations from the
  free stream; its derivatives w.r.t. Mach, AoA and wall-point normal
  displacements are checked against central finite differences of the oracle
  (the reference's algorithm in C), step 1e-6 (Mach), 1e-5 degrees (AoA),
  3e-8 (wall coordinates).  Bar: 1e-5 relative to the derivative's scale
  (FD truncation ~h^2 and rounding ~1e-16 / h are both far below it).  The
  same from a given initial state, with dJ/dprim0.
* The fixed-point adjoint contracts at a partly converged state; the torch
  autograd.Function wrapper reproduces the raw VJP.
* On a mixed handle the reverse of the mixed iteration (FP32 edge work)
  agrees with the FP64 reverse at the same state to the FP32 rounding.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cloud, small_cloud

pytestmark = pytest.mark.gpu

KW = dict(cfl=0.2, vl_const=50.0, power=0.0)
MACH, AOA, N, INNER = 0.8, 1.5, 12, 2


@pytest.fixture(scope="module")
def qlskum():
    import qlskum as q
    q.load()
    return q


def _cloud():
    return golden_cloud("cloud_trans")


def _oracle_J(oracle_mod, cloud, which, mach=MACH, aoa=AOA, iters=N, prim0=None):
    o = oracle_mod.Oracle(cloud, mach=mach, aoa=aoa, inner_iterations=INNER, threads=4, **KW)
    if prim0 is not None:
        o.set_prim(prim0)
    o.run(iters)
    cl, cd, _, _ = o.objective()
    o.close()
    return cl if which == "cl" else cd


def test_residual_forward_matches_reference_stage(qlskum):
    c = golden_cloud("cloud_trans")
    z = np.load(os.path.join(GOLDEN, "ref_trans_stage.npz"))
    s = qlskum.Solver(c, mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, inner_iterations=2)
    R = s.residual(z["prim_in"])
    scale = np.abs(z["flux_res"]).max(axis=0)
    assert (np.abs(R - z["flux_res"]) / scale).max() < 1e-12
    # the handle's own state is untouched
    s.q_lskum(1)
    assert np.isfinite(s.prim).all()


@pytest.mark.parametrize("inner", [0, 2])
def test_residual_vjp_dot_product(qlskum, inner):
    c = _cloud()
    s = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=inner, **KW)
    s.q_lskum(20)
    rng = np.random.default_rng(3 + inner)
    # The map is piecewise smooth: the neighbour max / min, the limiter's
    # branches and the time step's minimum switch where two values cross.  1%
    # noise keeps such pairs apart (no exact ties) and a step of 1e-8 makes a
    # swap of order rare; measured mismatches at this step are <= 1e-6
    # relative and <= 5e-10 of the Cauchy-Schwarz bound, against ~1e-2 for a
    # missing term.
    p = s.prim * (1.0 + 1e-2 * rng.standard_normal((c.n, 4)))
    h = 1e-8
    for _ in range(3):
        v = rng.standard_normal((c.n, 4)) * np.array([1.0, 0.5, 0.5, 0.7])
        w = rng.standard_normal((c.n, 4))
        fd = float(np.sum(w * (s.residual(p + h * v) - s.residual(p - h * v))) / (2 * h))
        g = s.residual_vjp(p, w)
        ad = float(np.sum(g * v))
        assert abs(fd - ad) <= 1e-8 * np.linalg.norm(g) * np.linalg.norm(v), (fd, ad)
        assert abs(fd - ad) <= 1e-5 * abs(ad), (fd, ad)


def test_residual_vjp_wall_displacement_vs_fd(qlskum):
    """qlskum_residual_vjp_full: the prim bar equals qlskum_residual_vjp's,
    the parameter bars are zero, and the wall-displacement bar of eight
    seeded wall points (away from the trailing edge) matches central
    differences of the residual on the moved clouds (step 3e-8, 1e-5)."""
    c = _cloud()
    s = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **KW)
    s.q_lskum(10)
    U = s.prim
    rng = np.random.default_rng(11)
    rbar = rng.standard_normal((c.n, 4))
    bprim, bp, bw = s.residual_vjp(U, rbar, wall=True)
    assert bp.tolist() == [0.0, 0.0]
    ref = s.residual_vjp(U, rbar)
    np.testing.assert_allclose(bprim, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())
    assert bw.shape == (s.shape_points,) and np.isfinite(bw).all()
    nrm = s.field(qlskum.FIELD_NORMALS)
    te = {0, int(c.left[0]) - 1, int(c.right[0]) - 1}
    pts = rng.choice(sorted(set(range(s.shape_points)) - te), size=8, replace=False)
    scale = np.abs(bw).max()
    h = 3e-8
    for m in pts:
        Rp = qlskum.Solver(_moved(c, m, h * nrm[m]), mach=MACH, aoa=AOA, inner_iterations=INNER, **KW).residual(U)
        Rm = qlskum.Solver(_moved(c, m, -h * nrm[m]), mach=MACH, aoa=AOA, inner_iterations=INNER, **KW).residual(U)
        fd = float(np.sum((Rp - Rm) * rbar)) / (2 * h)
        assert abs(bw[m] - fd) <= 1e-5 * max(abs(fd), 1e-2 * scale), (m, bw[m], fd)


def test_autograd_function_matches_vjp(qlskum):
    torch = pytest.importorskip("torch")
    from qlskum.autograd import flux_residual
    c = _cloud()
    s = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=1, **KW)
    s.q_lskum(5)
    p = torch.tensor(s.prim, dtype=torch.float64, requires_grad=True)
    w = torch.randn(c.n, 4, dtype=torch.float64, generator=torch.Generator().manual_seed(0))
    R = flux_residual(p, s)
    np.testing.assert_array_equal(R.detach().numpy(), s.residual(s.prim))
    (R * w).sum().backward()
    # the VJP scatters to neighbours with FP64 atomics: the order of the sums,
    # hence the last bits, varies between calls
    ref = s.residual_vjp(s.prim, w.numpy())
    np.testing.assert_allclose(p.grad.numpy(), ref, rtol=0, atol=1e-13 * np.abs(ref).max())


def test_autograd_function_on_cuda_tensors(qlskum):
    """CUDA tensors take the device-buffer pair (no host copy, ordered on the
    current torch stream) and give what the host-buffer pair gives."""
    torch = pytest.importorskip("torch")
    from qlskum.autograd import flux_residual
    c = _cloud()
    s = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=1, **KW)
    s.q_lskum(5)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        p = torch.tensor(s.prim, dtype=torch.float64, device="cuda", requires_grad=True)
        w = torch.randn(c.n, 4, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(0))
        R = flux_residual(p, s)
        (R * w).sum().backward()
        got_R, got_g = R.detach().cpu().numpy(), p.grad.cpu().numpy()
    np.testing.assert_array_equal(got_R, s.residual(s.prim))
    ref = s.residual_vjp(s.prim, w.cpu().numpy())
    np.testing.assert_allclose(got_g, ref, rtol=0, atol=1e-13 * np.abs(ref).max())


@pytest.mark.parametrize("which", ["cl", "cd"])
def test_adjoint_mach_aoa_vs_oracle_fd(qlskum, oracle_mod, which):
    c = _cloud()
    s = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **KW)
    g = s.adjoint_gradient(which, iters=N)
    J0 = _oracle_J(oracle_mod, c, which)
    assert abs(g["J"] - J0) <= 1e-10 * max(1.0, abs(J0))
    # the handle holds the final state, as after q_lskum(N)
    assert s.iteration == N
    hm, ha = 1e-6, 1e-5
    fd_m = (_oracle_J(oracle_mod, c, which, mach=MACH + hm) - _oracle_J(oracle_mod, c, which, mach=MACH - hm)) / (2 * hm)
    fd_a = (_oracle_J(oracle_mod, c, which, aoa=AOA + ha) - _oracle_J(oracle_mod, c, which, aoa=AOA - ha)) / (2 * ha)
    assert abs(g["dmach"] - fd_m) <= 1e-5 * max(abs(fd_m), 1e-3), (g["dmach"], fd_m)
    assert abs(g["daoa"] - fd_a) <= 1e-5 * max(abs(fd_a), 1e-3), (g["daoa"], fd_a)


def _moved(c, m, d):
    from qlskum.cloudgen import Cloud
    x = c.x.copy()
    y = c.y.copy()
    x[m] += d[0]
    y[m] += d[1]
    return Cloud(x, y, c.left, c.right, c.flag_1, c.flag_2, c.min_dist, c.nbhs, c.conn)


def test_adjoint_wall_displacement_vs_oracle_fd(qlskum, oracle_mod):
    """16 seeded wall points away from the trailing edge at 1e-5; the trailing
    edge and its two neighbours at 1e-3: the edge point's normal comes from
    two points 7e-4 apart, so J is non-smooth there on the FD step's scale
    (the FD converges to the adjoint value as the step shrinks)."""
    c = _cloud()
    s = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **KW)
    g = s.adjoint_gradient("cl", iters=N, wall=True)
    dw = g["dwall"]
    assert dw.shape == (s.shape_points,) and np.isfinite(dw).all()
    nrm = s.field(qlskum.FIELD_NORMALS)
    te = {0, int(c.left[0]) - 1, int(c.right[0]) - 1}
    rng = np.random.default_rng(16)
    pts = rng.choice(sorted(set(range(s.shape_points)) - te), size=16, replace=False)
    scale = np.abs(dw).max()
    for m, h, tol in [(m, 3e-8, 1e-5) for m in pts] + [(m, 1e-8, 1e-3) for m in sorted(te)]:
        Jp = _oracle_J(oracle_mod, _moved(c, m, h * nrm[m]), "cl")
        Jm = _oracle_J(oracle_mod, _moved(c, m, -h * nrm[m]), "cl")
        fd = (Jp - Jm) / (2 * h)
        assert abs(dw[m] - fd) <= tol * max(abs(fd), 1e-2 * scale), (m, dw[m], fd)


def test_adjoint_from_given_state_vs_oracle_fd(qlskum, oracle_mod):
    """prim0 held fixed: Mach / AoA by central differences of the oracle started
    from the same state, dJ/dprim0 by a directional difference."""
    c = _cloud()
    s = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **KW)
    s.q_lskum(10)
    rng = np.random.default_rng(7)
    U0 = s.prim * (1.0 + 1e-2 * rng.standard_normal((c.n, 4)))
    iters = 3
    g = s.adjoint_gradient("cd", iters=iters, prim0=U0)
    J0 = _oracle_J(oracle_mod, c, "cd", iters=iters, prim0=U0)
    assert abs(g["J"] - J0) <= 1e-10 * max(1.0, abs(J0))
    hm, ha = 1e-6, 1e-5
    fd_m = (_oracle_J(oracle_mod, c, "cd", mach=MACH + hm, iters=iters, prim0=U0)
            - _oracle_J(oracle_mod, c, "cd", mach=MACH - hm, iters=iters, prim0=U0)) / (2 * hm)
    fd_a = (_oracle_J(oracle_mod, c, "cd", aoa=AOA + ha, iters=iters, prim0=U0)
            - _oracle_J(oracle_mod, c, "cd", aoa=AOA - ha, iters=iters, prim0=U0)) / (2 * ha)
    assert abs(g["dmach"] - fd_m) <= 1e-5 * max(abs(fd_m), 1e-3), (g["dmach"], fd_m)
    assert abs(g["daoa"] - fd_a) <= 1e-5 * max(abs(fd_a), 1e-3), (g["daoa"], fd_a)
    v = rng.standard_normal((c.n, 4)) * np.array([1.0, 0.5, 0.5, 0.7])
    h = 1e-8
    fd = (_oracle_J(oracle_mod, c, "cd", iters=iters, prim0=U0 + h * v)
          - _oracle_J(oracle_mod, c, "cd", iters=iters, prim0=U0 - h * v)) / (2 * h)
    ad = float(np.sum(g["dprim0"] * v))
    assert abs(fd - ad) <= 1e-4 * abs(ad), (fd, ad)


def test_checkpoint_stride_same_gradient(qlskum):
    """Keeping every 2nd / 3rd state and recomputing the rest in FP64 gives the
    same gradient (the recomputed states equal the fused solver's bit for bit)."""
    c = _cloud()
    s = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **KW)
    g1 = s.adjoint_gradient("cd", iters=7, wall=True)
    for stride in (2, 3):
        g = s.adjoint_gradient("cd", iters=7, wall=True, stride=stride)
        assert g["J"] == g1["J"]
        np.testing.assert_allclose([g["dmach"], g["daoa"]], [g1["dmach"], g1["daoa"]], rtol=1e-11)
        np.testing.assert_allclose(g["dwall"], g1["dwall"], rtol=1e-9, atol=1e-12 * np.abs(g1["dwall"]).max())


def test_adjoint_of_mixed_run_close_to_fp64(qlskum):
    """On a mixed handle the reverse sweep differentiates the mixed iteration
    (FP32 edge work, FP64 update) along its own trajectory: the gradient
    agrees with the FP64 one to the mixed form's rounding.  Recomputing the
    segment states (stride 2) gives the same gradient up to the order of
    the FP32 atomic sums; the wall gradient on a mixed handle takes the FP64
    reverse."""
    c = _cloud()
    f = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **KW).adjoint_gradient("cl", iters=N)
    ms = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, precision=qlskum.MIXED, **KW)
    m = ms.adjoint_gradient("cl", iters=N)
    assert abs(m["J"] - f["J"]) < 1e-6
    np.testing.assert_allclose([m["dmach"], m["daoa"]], [f["dmach"], f["daoa"]], rtol=1e-4)
    m2 = ms.adjoint_gradient("cl", iters=N, stride=2)
    assert m2["J"] == m["J"]
    np.testing.assert_allclose([m2["dmach"], m2["daoa"]], [m["dmach"], m["daoa"]], rtol=1e-5)
    mw = ms.adjoint_gradient("cl", iters=N, wall=True)
    np.testing.assert_allclose([mw["dmach"], mw["daoa"]], [f["dmach"], f["daoa"]], rtol=1e-4)
    assert np.isfinite(mw["dwall"]).all()


@pytest.mark.parametrize("iters", [1, 3])
def test_mixed_reverse_matches_fp64_reverse_at_same_state(qlskum, iters):
    """From one partly converged state, the mixed handle's dJ/dprim0 (reverse
    of the mixed iteration) against the FP64 handle's (reverse of the FP64
    iteration): the two iterations are the same map up to FP32 rounding, so
    their transposed Jacobians applied to the same seed agree to ~1e-5 in
    norm (points where a limiter or half-range switch falls on the other
    side in FP32 are the few local exceptions)."""
    c = _cloud()
    f = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **KW)
    f.q_lskum(10)
    U0 = f.prim
    m = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, precision=qlskum.MIXED, **KW)
    for which in ("cl", "cd", "j"):
        gf = f.adjoint_gradient(which, iters=iters, prim0=U0)
        gm = m.adjoint_gradient(which, iters=iters, prim0=U0)
        assert abs(gm["J"] - gf["J"]) <= 1e-5 * max(abs(gf["J"]), 1e-3)
        d = gm["dprim0"] - gf["dprim0"]
        assert np.linalg.norm(d) <= 1e-4 * np.linalg.norm(gf["dprim0"]), (which, np.linalg.norm(d))
        np.testing.assert_allclose([gm["dmach"], gm["daoa"]], [gf["dmach"], gf["daoa"]], rtol=1e-4,
                                   atol=1e-6 * abs(gf["dmach"]))


def test_mixed_adjoint_primal_is_the_solver_run(qlskum):
    """On a mixed handle the adjoint's primal iterations (run by the recording
    kernels, which keep every stage's data for the reverse) leave the same
    state, prim_old and residual history as qlskum_q_lskum, bit for bit; the
    stride-2 sweep (each segment recomputed once) gives the same gradient up
    to the FP32 atomic sums of the gradient reverse."""
    c = _cloud()
    kw = dict(mach=MACH, aoa=AOA, inner_iterations=INNER, precision=qlskum.MIXED, **KW)
    a = qlskum.Solver(c, **kw)
    a.set_launch_config(0, 128, 0)
    g1 = a.adjoint_gradient("cl", iters=5)
    b = qlskum.Solver(c, **kw)
    b.set_launch_config(0, 128, 0)
    b.q_lskum(5)
    assert a.iteration == b.iteration == 5
    assert np.array_equal(a.prim, b.prim)
    assert np.array_equal(a.field(qlskum.FIELD_PRIM_OLD), b.field(qlskum.FIELD_PRIM_OLD))
    np.testing.assert_array_equal(a.residual_history(), b.residual_history())
    g2 = a.adjoint_gradient("cl", iters=5, stride=2)
    assert g2["J"] == g1["J"]
    np.testing.assert_allclose([g2["dmach"], g2["daoa"]], [g1["dmach"], g1["daoa"]], rtol=1e-5)


def test_mixed_reverse_weighted_stencils(qlskum):
    """The mixed reverse with distance-weighted least squares (power 1: the
    edge vectors and the folded weights are the weighted ones) against the
    FP64 reverse at the same state."""
    c = _cloud()
    kw = dict(KW, power=1.0)
    f = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **kw)
    f.q_lskum(5)
    U0 = f.prim
    m = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, precision=qlskum.MIXED, **kw)
    gf = f.adjoint_gradient("cd", iters=2, prim0=U0)
    gm = m.adjoint_gradient("cd", iters=2, prim0=U0)
    d = gm["dprim0"] - gf["dprim0"]
    assert np.linalg.norm(d) <= 1e-4 * np.linalg.norm(gf["dprim0"])
    np.testing.assert_allclose([gm["dmach"], gm["daoa"]], [gf["dmach"], gf["daoa"]], rtol=1e-4,
                               atol=1e-6 * abs(gf["dmach"]))


def test_fp64_adjoint_primal_is_the_solver_run(qlskum):
    """On an FP64 handle the adjoint's primal iterations run as the recording
    iteration (module kernels, every stage's data kept): the same state and
    residual history as qlskum_q_lskum, bit for bit."""
    c = _cloud()
    a = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **KW)
    a.adjoint_gradient("cd", iters=4)
    b = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **KW)
    b.q_lskum(4)
    assert a.iteration == b.iteration == 4
    assert np.array_equal(a.prim, b.prim)
    np.testing.assert_array_equal(a.residual_history(), b.residual_history())


def test_mixed_fixed_point_one_step_identity(qlskum):
    """The one-step identity of the fixed-point adjoint on a mixed handle
    (both sides run the mixed reverse; the FP32 atomic sums leave ~1e-7 of
    the derivative's scale)."""
    c = _cloud()
    s = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, precision=qlskum.MIXED, **KW)
    s.q_lskum(10)
    U = s.prim
    cd0 = s.objective()[1]
    fp = s.adjoint_fixed_point("cl", adj_iters=1)
    ag = s.adjoint_gradient("cl", iters=1, prim0=U)
    cd1 = s.objective()[1]
    np.testing.assert_allclose(fp["dmach"] - ag["dmach"], -2.0 * (fp["J"] - ag["J"]) / MACH, rtol=0,
                               atol=1e-5 * abs(fp["dmach"]))
    np.testing.assert_allclose(fp["daoa"] - ag["daoa"], -(cd0 - cd1) * np.pi / 180, rtol=0,
                               atol=1e-5 * abs(fp["daoa"]))
    r = s.adjoint_fixed_point("cd", adj_iters=20)
    assert np.isfinite([r["J"], r["dmach"], r["daoa"], r["adj_change"]]).all()


def test_adjoint_rejects_weighted_wall_gradient(qlskum):
    w = qlskum.Solver(_cloud(), power=1.0, inner_iterations=0, **{k: v for k, v in KW.items() if k != "power"})
    with pytest.raises(qlskum.QlskumError, match="unsupported"):
        w.adjoint_gradient("cl", iters=2, wall=True)
    # weighted stencils still give the parameter derivatives
    assert np.isfinite(w.adjoint_gradient("cd", iters=2)["dmach"])


def test_fixed_point_adjoint_one_step_identity(qlskum):
    """With one adjoint iteration, lam = dJ/dU and the fixed-point derivative is
    J_alpha(U) + lam^T dS/dalpha(U); the one-iteration adjoint from the same
    state held fixed gives J_alpha(S(U)) + lam^T dS/dalpha(U) (J is linear in
    the wall pressures, so lam is the same).  The two differ only by the
    objective's explicit terms: dCl/dM = -2 Cl / M and dCl/dtheta = -Cd."""
    c = _cloud()
    s = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **KW)
    s.q_lskum(10)
    U = s.prim
    cd0 = s.objective()[1]
    fp = s.adjoint_fixed_point("cl", adj_iters=1)
    ag = s.adjoint_gradient("cl", iters=1, prim0=U)
    cd1 = s.objective()[1]
    dm = fp["dmach"] - ag["dmach"]
    da = fp["daoa"] - ag["daoa"]
    np.testing.assert_allclose(dm, -2.0 * (fp["J"] - ag["J"]) / MACH, rtol=1e-9, atol=1e-12 * abs(fp["dmach"]))
    np.testing.assert_allclose(da, -(cd0 - cd1) * np.pi / 180, rtol=1e-9, atol=1e-12 * abs(fp["daoa"]))
    # more adjoint iterations and the wall gradient run through the same path
    r = s.adjoint_fixed_point("cd", adj_iters=20, wall=True)
    assert np.isfinite([r["J"], r["dmach"], r["daoa"], r["adj_change"]]).all() and np.isfinite(r["dwall"]).all()


def _oracle_stag_J(oracle_mod, cloud, mach=MACH, aoa=AOA, iters=N):
    o = oracle_mod.Oracle(cloud, mach=mach, aoa=aoa, inner_iterations=INNER, threads=4, **KW)
    o.run(iters)
    J = o.stagnation()[4]
    o.close()
    return J


def test_adjoint_stagnation_loss_vs_oracle_fd(qlskum, oracle_mod):
    """The stagnation-pressure loss J (qlskum_stagnation) as the adjoint's
    objective: Mach (incl. p0_inf's own dependence), AoA and wall points."""
    c = _cloud()
    s = qlskum.Solver(c, mach=MACH, aoa=AOA, inner_iterations=INNER, **KW)
    g = s.adjoint_gradient("j", iters=N, wall=True)
    J0 = _oracle_stag_J(oracle_mod, c)
    assert abs(g["J"] - J0) <= 1e-10 * abs(J0)
    hm, ha = 1e-6, 1e-5
    fd_m = (_oracle_stag_J(oracle_mod, c, mach=MACH + hm) - _oracle_stag_J(oracle_mod, c, mach=MACH - hm)) / (2 * hm)
    fd_a = (_oracle_stag_J(oracle_mod, c, aoa=AOA + ha) - _oracle_stag_J(oracle_mod, c, aoa=AOA - ha)) / (2 * ha)
    assert abs(g["dmach"] - fd_m) <= 1e-5 * abs(fd_m), (g["dmach"], fd_m)
    assert abs(g["daoa"] - fd_a) <= 1e-5 * max(abs(fd_a), 1e-3 * abs(fd_m)), (g["daoa"], fd_a)
    nrm = s.field(qlskum.FIELD_NORMALS)
    dw = g["dwall"]
    scale = np.abs(dw).max()
    # point 5 sits near the trailing edge: its difference quotient moves with
    # the step there (1e-7: 9.32820e-4, 3e-9: 9.32890e-4), so a smaller step
    for m, h, tol in ((17, 3e-8, 1e-5), (40, 3e-8, 1e-5), (25, 3e-8, 1e-5), (5, 3e-9, 1e-4)):
        fd = (_oracle_stag_J(oracle_mod, _moved(c, m, h * nrm[m])) -
              _oracle_stag_J(oracle_mod, _moved(c, m, -h * nrm[m]))) / (2 * h)
        assert abs(dw[m] - fd) <= tol * max(abs(fd), 1e-2 * scale), (m, dw[m], fd)
