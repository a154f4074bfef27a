"""Cloud files and the sub-stencil quality check through the C ABI (no GPU).

* qlskum_partgrid_write / _read round-trip a cloud exactly and agree with the
  Python reader / writer of the same format (main.cpp:16-58);
* qlskum_check_stencils restates generate_connectivity's split and the
  flux sub-stencils' weighted moments; it is checked against numpy on a
  generated cloud, and flags points whose sub-stencils are emptied.
"""
import os
import tempfile

import numpy as np
import pytest

from conftest import golden_cloud, small_cloud


@pytest.fixture(scope="module")
def q():
    import qlskum
    qlskum.load()
    return qlskum


def _same(a, b):
    for f in ("x", "y", "left", "right", "flag_1", "flag_2", "min_dist", "nbhs", "conn"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def test_partgrid_c_round_trip_and_python_agree(q):
    from qlskum import cloudgen
    c = golden_cloud("cloud_trans")
    d = tempfile.mkdtemp()
    pc, pp = os.path.join(d, "c"), os.path.join(d, "p")
    q.partgrid_write(c, pc)
    cloudgen.write_partgrid(c, pp)
    _same(q.partgrid_read(pc), c)
    _same(q.partgrid_read(pp), c)
    _same(cloudgen.read_partgrid(pc), c)


def test_partgrid_rejects_bad_files(q):
    d = tempfile.mkdtemp()
    bad = os.path.join(d, "bad")
    with open(bad, "w") as f:
        f.write("2\n0 0 1 2 0 1 0.1 21 " + " ".join(["1"] * 21) + "\n")
    with pytest.raises(q.QlskumError, match="nbhs"):
        q.partgrid_read(bad)
    with open(bad, "w") as f:
        f.write("3\n0 0 1 2 0 1 0.1 2 2 3\n")
    with pytest.raises(q.QlskumError, match="point 2"):
        q.partgrid_read(bad)
    with pytest.raises(q.QlskumError, match="cannot open"):
        q.partgrid_read(os.path.join(d, "missing"))


def _rcond_numpy(c, power):
    n = c.n
    out = np.ones((n, 4))
    for i in range(n):
        f = c.flag_1[i]
        if f != 1:
            l, r = c.left[i] - 1, c.right[i] - 1
            a = 0.5 * ((c.y[i] - c.y[l]) + (c.y[r] - c.y[i]))
            b = 0.5 * ((c.x[i] - c.x[l]) + (c.x[r] - c.x[i]))
            dd = np.sqrt(a * a + b * b)
            nx, ny = -a / dd, b / dd
        else:
            nx, ny = 0.0, 1.0
        k = c.conn[i, :c.nbhs[i]] - 1
        dx, dy = c.x[k] - c.x[i], c.y[k] - c.y[i]
        ds, dn = dx * ny - dy * nx, dx * nx + dy * ny
        w = np.sqrt(ds * ds + dn * dn) ** power
        masks = [ds <= 0, ds >= 0, dn <= 0 if f == 1 else np.full(ds.shape, f == 2),
                 dn >= 0 if f == 1 else np.full(ds.shape, f == 0)]
        used = [True, True, f != 0, f != 2]
        for d in range(4):
            if not used[d]:
                continue
            m = masks[d]
            if m.sum() < 2:
                out[i, d] = 0.0
                continue
            M = np.array([[np.sum(ds[m] ** 2 * w[m]), np.sum(ds[m] * dn[m] * w[m])],
                          [np.sum(ds[m] * dn[m] * w[m]), np.sum(dn[m] ** 2 * w[m])]])
            ev = np.linalg.eigvalsh(M)
            out[i, d] = ev[0] / ev[1] if ev[1] > 0 else 0.0
    return out


@pytest.mark.parametrize("power", [0.0, -2.0])
def test_check_stencils_matches_numpy(q, power):
    c = small_cloud()
    rc, bad = q.check_stencils(c, power=power, min_rcond=1e-3)
    ref = _rcond_numpy(c, power)
    np.testing.assert_allclose(rc, ref, rtol=1e-9, atol=1e-12)
    assert bad == int(((ref < 1e-3)).any(1).sum())
    assert bad == 0   # the generator repairs every ill-posed stencil


def test_check_stencils_flags_emptied_substencils(q):
    c = small_cloud()
    conn = c.conn.copy()
    nbhs = c.nbhs.copy()
    i = int(np.nonzero(c.flag_1 == 1)[0][5])
    nbhs[i] = 1                              # one neighbour left: every sub-stencil short
    from qlskum.cloudgen import Cloud
    c2 = Cloud(c.x, c.y, c.left, c.right, c.flag_1, c.flag_2, c.min_dist, nbhs, conn)
    rc, bad = q.check_stencils(c2)
    assert bad == 1 and (rc[i] == 0.0).sum() >= 2
