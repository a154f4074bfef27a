"""The partitioned solve (ghost points refreshed from their owners before
every kernel that reads a neighbour) against the single-domain solve on the
same GPU, through the C ABI.

The per-point arithmetic of a partition is the single-domain solve's, with
the same neighbour values in the same order, so the state must agree bit
for bit: in FP64, and in the mixed form at the same launch shape.  Only the
residual norm's and the objectives' sums run in another order (per
partition, then over the partitions): 1e-13 relative.  The FP64 partitioned
solve is also held to the reference's own golden run (1e-10).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cloud

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    scale = np.maximum(np.abs(b).max(axis=0, keepdims=True), 1e-300)
    return float((np.abs(a - b) / scale).max())


@pytest.fixture(scope="module")
def qlskum():
    import qlskum as q
    q.load()
    return q


@pytest.mark.parametrize("parts", [2, 3])
def test_fp64_partitions_equal_single_domain(qlskum, parts):
    c = golden_cloud("cloud_trans")
    kw = dict(mach=0.85, aoa=1.0, cfl=0.2, vl_const=50.0, inner_iterations=3)
    s = qlskum.Solver(c, **kw)
    p = qlskum.Partition(c, parts, **kw)
    s.q_lskum(12)
    p.q_lskum(12)
    assert np.array_equal(p.prim, s.prim)
    np.testing.assert_allclose(p.residual_history(), s.residual_history(), rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(p.objective(), s.objective(), rtol=1e-13)
    # each partition's ghosts are exactly the outside neighbours of its points
    seen = np.zeros(c.n, int)
    for q in range(parts):
        loc, gh = p.layout(q)
        seen[loc - 1] += 1
        nb = np.concatenate([c.conn[i, :c.nbhs[i]] for i in loc - 1])
        assert np.array_equal(np.sort(gh), np.setdiff1d(nb, loc))
    assert (seen == 1).all()
    assert p.halo_bytes > 0


def test_fp64_partitions_vs_reference_golden(qlskum):
    """4 partitions of the 2,560-point cloud, 30 transonic iterations with 3
    inner iterations, against the reference build's run (the FP64 bar)."""
    c = golden_cloud("cloud_trans")
    z = np.load(os.path.join(GOLDEN, "ref_trans_run.npz"))
    p = qlskum.Partition(c, 4, mach=0.85, aoa=1.0, cfl=0.2, vl_const=50.0, inner_iterations=3)
    p.q_lskum(30)
    np.testing.assert_allclose(p.residual_history()[:, 0], z["residuals"][:, 0], rtol=1e-10)
    assert rel_err(p.prim, z["prim"]) < 1e-10
    np.testing.assert_allclose(p.objective(), z["objectives"], rtol=1e-10)


def test_fp64_partitions_config1_cloud(qlskum):
    """The 9,600-point config-1 cloud in 5 partitions, 100 iterations, inner 0."""
    c = golden_cloud("cloud_c1")
    kw = dict(mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, inner_iterations=0)
    s = qlskum.Solver(c, **kw)
    p = qlskum.Partition(c, 5, **kw)
    s.q_lskum(100)
    p.q_lskum(60)
    p.q_lskum(40)            # continuing across calls
    assert np.array_equal(p.prim, s.prim)
    np.testing.assert_allclose(p.residual_history(), s.residual_history(), rtol=1e-13, atol=1e-300)


def test_mixed_partitions_equal_single_domain_same_shape(qlskum):
    c = golden_cloud("cloud_trans")
    kw = dict(mach=0.8, aoa=1.5, cfl=0.2, vl_const=50.0, inner_iterations=2, precision=qlskum.MIXED)
    s = qlskum.Solver(c, **kw)
    s.set_launch_config(5, 128, 0)
    p = qlskum.Partition(c, 2, **kw)
    p.set_launch_config(5, 128, 0)
    s.q_lskum(10)
    p.q_lskum(10)
    assert np.array_equal(p.prim, s.prim)
    np.testing.assert_allclose(p.residual_history()[:, 0], s.residual_history()[:, 0], rtol=1e-13)


def test_partition_set_prim_continues_like_single_domain(qlskum):
    """A state written to owners and ghosts alike (qlskum_partition_set_prim)
    continues exactly like the single-domain solve from the same state."""
    c = golden_cloud("cloud_trans")
    kw = dict(mach=0.7, aoa=2.5, cfl=0.2, vl_const=50.0, inner_iterations=1)
    s = qlskum.Solver(c, **kw)
    s.q_lskum(4)
    start = s.prim
    t = qlskum.Solver(c, **kw)
    t.set_prim(start)
    t.q_lskum(5)
    p = qlskum.Partition(c, 3, **kw)
    p.set_prim(start)
    p.q_lskum(5)
    assert np.array_equal(p.prim, t.prim)
