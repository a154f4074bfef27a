"""The seeded cloud generator and the partGrid text I/O (main.cpp:16-58 format)."""
import os
import tempfile

import numpy as np

from conftest import small_cloud


def test_partgrid_round_trip_exact():
    from qlskum import cloudgen
    c = small_cloud()
    path = os.path.join(tempfile.mkdtemp(), "g")
    cloudgen.write_partgrid(c, path)
    r = cloudgen.read_partgrid(path)
    for f in ("x", "y", "left", "right", "flag_1", "flag_2", "min_dist", "nbhs", "conn"):
        assert np.array_equal(getattr(r, f), getattr(c, f)), f


def test_partgrid_rejects_too_many_neighbours():
    from qlskum import cloudgen
    path = os.path.join(tempfile.mkdtemp(), "g")
    with open(path, "w") as f:
        f.write("1\n0 0 0 0 1 0 0.1 21 " + " ".join(["1"] * 21) + "\n")
    try:
        cloudgen.read_partgrid(path)
    except ValueError as e:
        assert "nbhs=21" in str(e)
    else:
        raise AssertionError("nbhs > 20 accepted")


def test_layout_invariants():
    c = small_cloud(n_wall=48, n_layers=16, first_spacing=5e-3, radius=3.0, seed=3)
    W = 48
    assert c.counts() == {"points": 48 * 16, "wall": W, "interior": 48 * 14, "outer": W, "shape": W}
    # wall points first, shape points are the wall (compute_force_coeffs_mod.h:25-27)
    assert (c.flag_1[:W] == 0).all() and (c.flag_2[:W] == 1).all() and (c.flag_2[W:] == 0).all()
    # 10 nearest as a rule; points at the trailing edge lose neighbours that
    # only see them through the body, others gain some to keep sub-stencils posed
    assert (c.nbhs >= 4).all() and (c.nbhs <= 20).all() and np.median(c.nbhs) == 10
    for i in range(c.n):
        nb = c.conn[i, :c.nbhs[i]]
        assert (nb >= 1).all() and (nb <= c.n).all() and (nb != i + 1).all()
        assert (c.conn[i, c.nbhs[i]:] == 0).all()
    # min_dist is the shortest edge of the point's stencil
    for i in range(0, c.n, 37):
        nb = c.conn[i, :c.nbhs[i]] - 1
        dx, dy = c.x[nb] - c.x[i], c.y[nb] - c.y[i]
        assert np.sqrt(dx * dx + dy * dy).min() == c.min_dist[i]


def test_normals_point_into_the_fluid():
    """n = rot90(right - left) (point_normals_mod.h:34-46) points away from the
    body on the wall and away from the domain on the far-field circle."""
    c = small_cloud(n_wall=48, n_layers=16, first_spacing=5e-3, radius=3.0, seed=3)
    for sl, sign in ((slice(0, 48), 1.0), (slice(c.n - 48, c.n), 1.0)):
        idx = np.arange(c.n)[sl]
        l, r = c.left[idx] - 1, c.right[idx] - 1
        nx = -0.5 * (c.y[r] - c.y[l])
        ny = 0.5 * (c.x[r] - c.x[l])
        cx, cy = c.x[idx] - 0.5, c.y[idx]
        assert (sign * (nx * cx + ny * cy) > 0).mean() > 0.95


def test_seeded_and_deterministic():
    from qlskum import cloudgen
    a = cloudgen.make_cloud(n_wall=32, n_layers=10, first_spacing=1e-2, radius=3.0, seed=9)
    b = cloudgen.make_cloud(n_wall=32, n_layers=10, first_spacing=1e-2, radius=3.0, seed=9)
    c = cloudgen.make_cloud(n_wall=32, n_layers=10, first_spacing=1e-2, radius=3.0, seed=10)
    assert np.array_equal(a.x, b.x) and np.array_equal(a.conn, b.conn)
    assert not np.array_equal(a.x, c.x)


def _weight_bounds(cloudgen, oracle_mod, c):
    """Per sub-stencil d: (count, rcond, weight bound, wrong-sign weight, used)
    of every point, split as the reference splits it (the oracle's normals)."""
    o = oracle_mod.Oracle(c, threads=2)
    nrm = o.normals
    valid = np.arange(20)[None, :] < c.nbhs[:, None]
    idx = np.where(valid, c.conn - 1, 0)
    dx = np.where(valid, c.x[idx] - c.x[:, None], 0.0)
    dy = np.where(valid, c.y[idx] - c.y[:, None], 0.0)
    nx, ny = nrm[:, :1], nrm[:, 1:]
    dels, deln = dx * ny - dy * nx, dx * nx + dy * ny
    dmin = cloudgen._nearest(dels, deln, valid)
    masks = cloudgen._classify_masks(dels, deln, c.flag_1)
    used = [np.ones(c.n, bool), np.ones(c.n, bool), c.flag_1 != 0, c.flag_1 != 2]
    return [cloudgen._sub_stats(dels, deln, masks[d] & valid, d < 2, dmin, cloudgen._half_sign(d, c.flag_1)[:, None])
            + (used[d],) for d in range(4)]


def test_substencils_upwind_and_bounded(oracle_mod):
    """Every sub-stencil of a generated cloud, split as the reference splits it,
    meets the generator's bounds on its least-squares derivative weights:
    their magnitude sum times the nearest-neighbour distance <= 2.5 and the
    weight of the wrong (downwind) sign <= 0.3 (points at the 20-neighbour
    cap, where the repair stops, excepted).  The same cloud without the
    bounds has wake-line stencils outside them: on the 1.02 M-point cloud
    those reached 18 and 9, and the unlimited update grew there by 1.4x per
    iteration."""
    from qlskum import cloudgen
    kw = dict(n_wall=256, n_layers=120, first_spacing=2e-3, radius=20.0, seed=3)
    c = small_cloud(**kw)
    capped = c.nbhs >= 20
    assert capped.sum() < 0.01 * c.n
    for cnt, rc, bound, wrong, used in _weight_bounds(cloudgen, oracle_mod, c):
        chk = used & ~capped
        assert (cnt[chk] >= 2).all() and (rc[chk] >= 1e-3).all()
        assert bound[chk].max() <= 2.5 + 1e-9, bound[chk].max()
        assert wrong[chk].max() <= 0.3 + 1e-9, wrong[chk].max()
    u = cloudgen.make_cloud(**kw, max_weight=np.inf, max_wrong=np.inf)
    worst = max(float(np.max(np.where(used, wrong, 0.0))) for _, _, _, wrong, used in _weight_bounds(cloudgen, oracle_mod, u))
    assert worst > 0.3, worst


def test_substencils_well_posed(oracle_mod):
    """Every sub-stencil a point's class uses has >= 2 members (the generator's
    check_condition_number job, generate_connectivity_mod.h:84-89)."""
    c = small_cloud(n_wall=48, n_layers=16, first_spacing=5e-3, radius=3.0, seed=3, m=0.04, p=0.3, t=0.16)
    o = oracle_mod.Oracle(c, threads=2)
    cnt = o.sub_counts()
    used = {0: [0, 1, 3], 1: [0, 1, 2, 3], 2: [0, 1, 2]}
    for i in range(c.n):
        for d in used[int(c.flag_1[i])]:
            assert cnt[i, d] >= 2, (i, d)
