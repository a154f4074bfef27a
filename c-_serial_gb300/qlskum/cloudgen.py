"""Seeded point-cloud generator and `partGrid` text I/O for q-LSKUM.

The file format is the one the reference reads (main.cpp:16-58): a header line
holding the number of points, then one line per point

    x y left right flag_1 flag_2 min_dist nbhs conn[1..nbhs]

1-based indices, flag_1 = 0 wall / 1 interior / 2 outer, flag_2 > 0 marks a
shape (surface) point, at most 20 neighbours (main.cpp:27).  Wall points come
first because compute_cl_cd_cm walks points 1..shape_points
(compute_force_coeffs_mod.h:25-27).

Layout of a generated cloud
---------------------------
* Body: NACA 4-digit section of chord 1 with a closed trailing edge, wall
  points cosine-spaced in the surface parameter theta (x = (1 + cos theta)/2).
  Point 1 is the trailing edge; theta runs counter-clockwise (upper surface
  first).  `left` is the next point counter-clockwise and `right` the previous
  one, so the reference's normal formula (point_normals_mod.h:17-49,
  n = rot90(r - l)) points into the fluid on the wall and away from the body
  on the far-field circle.
* Layers: `n_layers` rings; ring 0 is the wall, the last ring is the far-field
  circle of radius `radius` centred at mid-chord.  Ring offsets grow
  geometrically from `first_spacing`; the growth ratio is solved so that the
  rings reach the circle (with the literal 2e-3 / 1.1 / 60-layer recipe the
  rings would stop near 6 chords).  Near the wall a ring point sits on the
  wall normal; further out it blends to the straight line towards the circle.
* Jitter: interior points move by a seeded uniform offset of up to `jitter`
  of the local tangential / normal spacing.
* Neighbours: the `n_nbrs` nearest candidates within `nbr_radius` x the local
  spacing, "nearest" being measured in the local (tangential, normal) spacing
  units so that anisotropic near-wall rings still give every directional
  sub-stencil points on both sides.  Points whose sub-stencils (split the way
  generate_connectivity_mod.h:5-219 splits them) are empty, nearly
  collinear, or whose least-squares derivative weights are too large or
  not upwind (`_sub_stats`: weight sum times the nearest-neighbour distance
  above `max_weight`, downwind-signed weight above `max_wrong`) get further
  candidates, up to 20 neighbours.  This is the job of the empty
  `check_condition_number` stub at generate_connectivity_mod.h:84-89.  The
  weight bounds matter on the O-grid's wake line behind the trailing edge,
  where the rings are sheared: without them some stencils there are
  one-sided, and the unlimited update (small perturbations pass the
  limiter's 1e-5 cut) grows at those points by a fixed factor per
  iteration, in FP64 as in the mixed form.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

MAX_NBHS = 20


@dataclasses.dataclass
class Cloud:
    """A point cloud in the reference's layout (1-based indices in left/right/conn)."""

    x: np.ndarray          # float64 [N]
    y: np.ndarray          # float64 [N]
    left: np.ndarray       # int32 [N] (1-based, 0 for interior points)
    right: np.ndarray      # int32 [N]
    flag_1: np.ndarray     # int32 [N]: 0 wall, 1 interior, 2 outer
    flag_2: np.ndarray     # int32 [N]: shape id (>0) on wall points, else 0
    min_dist: np.ndarray   # float64 [N]
    nbhs: np.ndarray       # int32 [N]
    conn: np.ndarray       # int32 [N, 20] (1-based; unused slots 0)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    def counts(self) -> dict:
        return {
            "points": self.n,
            "wall": int((self.flag_1 == 0).sum()),
            "interior": int((self.flag_1 == 1).sum()),
            "outer": int((self.flag_1 == 2).sum()),
            "shape": int((self.flag_2 > 0).sum()),
        }


# ---------------------------------------------------------------------------
# partGrid text I/O
# ---------------------------------------------------------------------------

def write_partgrid(cloud: Cloud, path: str) -> None:
    """Write `cloud` in the reference's partGrid text format (main.cpp:18,32-36).

    Coordinates and min_dist are written with 17 significant digits so the
    file reads back to the identical doubles.
    """
    n = cloud.n
    lines = [f"{n}\n"]
    xs = [repr(float(v)) for v in cloud.x]
    ys = [repr(float(v)) for v in cloud.y]
    md = [repr(float(v)) for v in cloud.min_dist]
    for i in range(n):
        k = int(cloud.nbhs[i])
        c = " ".join(str(int(v)) for v in cloud.conn[i, :k])
        lines.append(
            f"{xs[i]} {ys[i]} {int(cloud.left[i])} {int(cloud.right[i])} "
            f"{int(cloud.flag_1[i])} {int(cloud.flag_2[i])} {md[i]} {k} {c}\n"
        )
    with open(path, "w") as f:
        f.writelines(lines)


def read_partgrid(path: str) -> Cloud:
    """Read a partGrid text file (main.cpp:16-58).  Rejects nbhs outside 0..20."""
    with open(path) as f:
        tok = f.read().split()
    n = int(tok[0])
    x = np.empty(n)
    y = np.empty(n)
    left = np.empty(n, np.int32)
    right = np.empty(n, np.int32)
    f1 = np.empty(n, np.int32)
    f2 = np.empty(n, np.int32)
    md = np.empty(n)
    nb = np.empty(n, np.int32)
    conn = np.zeros((n, MAX_NBHS), np.int32)
    p = 1
    for i in range(n):
        x[i] = float(tok[p]); y[i] = float(tok[p + 1])
        left[i] = int(tok[p + 2]); right[i] = int(tok[p + 3])
        f1[i] = int(tok[p + 4]); f2[i] = int(tok[p + 5])
        md[i] = float(tok[p + 6]); k = int(tok[p + 7])
        if k < 0 or k > MAX_NBHS:
            raise ValueError(f"point {i + 1}: nbhs={k} outside 0..{MAX_NBHS}")
        nb[i] = k
        conn[i, :k] = [int(t) for t in tok[p + 8:p + 8 + k]]
        p += 8 + k
    return Cloud(x, y, left, right, f1, f2, md, nb, conn)


# ---------------------------------------------------------------------------
# Geometry
# ---------------------------------------------------------------------------

def naca4_surface(theta: np.ndarray, m: float = 0.0, p: float = 0.4, t: float = 0.12, te_spread: float = 0.0):
    """NACA 4-digit surface at parameter theta in [0, 2 pi).

    x_c = (1 + cos theta)/2; theta in [0, pi] is the upper surface (trailing
    edge to leading edge), (pi, 2 pi) the lower one.  Closed trailing edge
    (-0.1036 x^4 coefficient).  m = max camber, p = its chord position,
    t = thickness, all as fractions of the chord.

    te_spread = w > 0 moves x_c away from the trailing edge by
    w |sin theta| (1 + cos theta) / 2: the cosine law's spacing at the
    trailing edge, which shrinks as 1 / n^2 with the number of wall points,
    becomes w times the parameter step there, while the leading edge keeps
    the cosine law (the added term vanishes to third order at theta = pi);
    the map stays monotone for w < 0.8.
    """
    xc = 0.5 * (1.0 + np.cos(theta)) - te_spread * np.abs(np.sin(theta)) * 0.5 * (1.0 + np.cos(theta))
    yt = 5.0 * t * (0.2969 * np.sqrt(xc) - 0.1260 * xc - 0.3516 * xc**2 + 0.2843 * xc**3 - 0.1036 * xc**4)
    if m > 0.0:
        fore = xc < p
        yc = np.where(fore, m / p**2 * (2 * p * xc - xc**2), m / (1 - p) ** 2 * ((1 - 2 * p) + 2 * p * xc - xc**2))
        dyc = np.where(fore, 2 * m / p**2 * (p - xc), 2 * m / (1 - p) ** 2 * (p - xc))
    else:
        yc = np.zeros_like(xc)
        dyc = np.zeros_like(xc)
    th = np.arctan(dyc)
    upper = np.sin(theta) >= 0.0
    sgn = np.where(upper, 1.0, -1.0)
    x = xc - sgn * yt * np.sin(th)
    y = yc + sgn * yt * np.cos(th)
    return x, y


def _rot_normals(px: np.ndarray, py: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Normals of a closed ring ordered counter-clockwise: rot90(prev - next)/|.|.

    The same construction as point_normals_mod.h:34-46 with l = next, r = prev.
    """
    lx, ly = np.roll(px, -1), np.roll(py, -1)
    rx, ry = np.roll(px, 1), np.roll(py, 1)
    nx = -0.5 * (ry - ly)
    ny = 0.5 * (rx - lx)
    d = np.sqrt(nx * nx + ny * ny)
    return nx / d, ny / d


def solve_growth(first: float, steps: int, total: float) -> float:
    """Ratio r with first*(r^steps - 1)/(r - 1) == total (bisection)."""
    if first * steps >= total:
        return 1.0
    lo, hi = 1.0 + 1e-12, 2.0
    while first * (hi**steps - 1.0) / (hi - 1.0) < total:
        hi *= 1.5
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if first * (mid**steps - 1.0) / (mid - 1.0) < total:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def make_layers(n_wall: int, n_layers: int, first_spacing: float, radius: float,
                m: float = 0.0, p: float = 0.4, t: float = 0.12,
                center=(0.5, 0.0), blend_len: float = 1.0, smooth: int = 0, te_spread: float = 0.0):
    """Ring points [n_layers, n_wall] (x, y) and the ring offsets d_j."""
    theta = 2.0 * np.pi * np.arange(n_wall) / n_wall
    wx, wy = naca4_surface(theta, m, p, t, te_spread)
    nx, ny = _rot_normals(wx, wy)
    # Spread the ray fan at the sharp trailing edge: smooth the ray directions
    # along the ring so that the wake behind the edge is not left empty.
    for _ in range(smooth):
        sx = np.roll(nx, 1) + 2.0 * nx + np.roll(nx, -1)
        sy = np.roll(ny, 1) + 2.0 * ny + np.roll(ny, -1)
        ln = np.sqrt(sx * sx + sy * sy)
        nx, ny = sx / ln, sy / ln
    cx = center[0] + radius * np.cos(theta)
    cy = center[1] + radius * np.sin(theta)
    span = np.sqrt((cx - wx) ** 2 + (cy - wy) ** 2)       # wall -> circle distance per ray
    steps = n_layers - 1
    g = solve_growth(first_spacing, steps, float(span.min()))
    j = np.arange(n_layers, dtype=np.float64)
    d = first_spacing * j if g == 1.0 else first_spacing * (g**j - 1.0) / (g - 1.0)
    f = d / d[-1]                                          # 0 at wall, 1 at circle
    beta = np.clip(d / blend_len, 0.0, 1.0) ** 2
    beta[-1] = 1.0
    X = np.empty((n_layers, n_wall))
    Y = np.empty((n_layers, n_wall))
    for jj in range(n_layers):
        ox = wx + d[jj] * nx
        oy = wy + d[jj] * ny
        lx = (1.0 - f[jj]) * wx + f[jj] * cx
        ly = (1.0 - f[jj]) * wy + f[jj] * cy
        X[jj] = (1.0 - beta[jj]) * ox + beta[jj] * lx
        Y[jj] = (1.0 - beta[jj]) * oy + beta[jj] * ly
    X[-1], Y[-1] = cx, cy
    return X, Y, g


# ---------------------------------------------------------------------------
# Connectivity
# ---------------------------------------------------------------------------

def _classify_masks(dels: np.ndarray, deln: np.ndarray, flag: np.ndarray):
    """Sub-stencil membership as generate_connectivity_mod.h:5-219 decides it.

    Returns four bool arrays (xpos, xneg, ypos, yneg) shaped like dels.
    Interior: by sign of dels / deln, ties in both.  Wall: x by dels, yneg all.
    Outer: x by dels, ypos all.
    """
    f = flag[:, None]
    xpos = dels <= 0.0
    xneg = dels >= 0.0
    ypos = np.where(f == 1, deln <= 0.0, f == 2)
    yneg = np.where(f == 1, deln >= 0.0, f == 0)
    return xpos, xneg, ypos, yneg


def _sub_stats(dels, deln, w, along_s, dmin, sign=0.0):
    """Per row, for the sub-stencil mask w: member count, reciprocal condition
    number of its 2x2 least-squares matrix, its weight bound and its
    wrong-sign weight.

    The weights are those of the least-squares derivative (along s for the x
    sub-stencils, along n for the y ones), in units of one over the row's
    nearest-neighbour distance.  The explicit update moves a point by about
    delta times their sum times the wave speed, and delta is CFL times the
    nearest-neighbour distance over the wave speed (func_delta), so the
    bound (the sum of their magnitudes) is the point's effective CFL number
    per unit CFL.  A half-range stencil (sign -1: members with d <= 0, +1:
    d >= 0) is upwind when every weight has that sign; the wrong-sign weight
    is the sum of the magnitudes of those that do not.  Skewed, one-sided
    stencils (on a generated cloud: the O-grid's wake line behind the
    trailing edge) reach a bound of 10 and a wrong-sign weight of several
    units where a well-shaped stencil has about 1 and 0.01; the unlimited
    update (the limiter's |dq| <= 1e-5 cut) then grows there by a fixed
    factor per iteration, in FP64 as in the mixed form."""
    cnt = w.sum(1)
    sxx = np.where(w, dels * dels, 0.0).sum(1)
    syy = np.where(w, deln * deln, 0.0).sum(1)
    sxy = np.where(w, dels * deln, 0.0).sum(1)
    tr = sxx + syy
    det = sxx * syy - sxy * sxy
    disc = np.sqrt(np.maximum(tr * tr * 0.25 - det, 0.0))
    lmax = tr * 0.5 + disc
    lmin = tr * 0.5 - disc
    rc = np.where(lmax > 0, lmin / np.where(lmax > 0, lmax, 1.0), 0.0)
    pos = det > 0
    inv = np.where(pos, 1.0 / np.where(pos, det, 1.0), 0.0)
    if along_s:
        cw = (syy[:, None] * dels - sxy[:, None] * deln) * inv[:, None]
    else:
        cw = (sxx[:, None] * deln - sxy[:, None] * dels) * inv[:, None]
    bound = np.where(pos, np.where(w, np.abs(cw), 0.0).sum(1) * dmin, np.inf)
    wrong = np.where(pos, np.where(w, np.maximum(-sign * cw, 0.0), 0.0).sum(1) * dmin, np.inf)
    return cnt, rc, bound, wrong


def _nearest(dels, deln, valid):
    return np.where(valid, np.sqrt(dels * dels + deln * deln), np.inf).min(1)


# sign of the half-range of the sub-stencils xpos, xneg, ypos, yneg of an
# interior point (members with dels <= 0, dels >= 0, deln <= 0, deln >= 0)
_HALF_SIGN = (-1.0, 1.0, -1.0, 1.0)


def _half_sign(d, flag):
    """Per row: the half-range sign of sub-stencil d, 0 where the class takes
    the whole stencil (the wall's yneg, the outer boundary's ypos)."""
    if d < 2:
        return np.full(flag.shape, _HALF_SIGN[d])
    return np.where(flag == 1, _HALF_SIGN[d], 0.0)


def _stencil_ok(dels, deln, valid, flag, min_count=2, min_rcond=1e-3, max_weight=np.inf, max_wrong=np.inf):
    """Per point: every sub-stencil the point's class uses is well posed.

    A sub-stencil passes when it has >= min_count members, the reciprocal
    condition number of its 2x2 least-squares matrix is >= min_rcond, its
    weight bound is <= max_weight and its wrong-sign weight <= max_wrong
    (`_sub_stats`).
    """
    masks = _classify_masks(dels, deln, flag)
    need = [np.ones_like(flag, bool), np.ones_like(flag, bool), flag != 0, flag != 2]
    dmin = _nearest(dels, deln, valid)
    ok = np.ones(flag.shape[0], bool)
    for d, (mk, nd) in enumerate(zip(masks, need)):
        cnt, rc, bound, wrong = _sub_stats(dels, deln, mk & valid, d < 2, dmin, _half_sign(d, flag)[:, None])
        good = (cnt >= min_count) & (rc >= min_rcond) & (bound <= max_weight) & (wrong <= max_wrong)
        ok &= np.where(nd, good, True)
    return ok


def _visible(x, y, nx, ny, flag, rows, idx, dx, dy, dist, wall, cache=None):
    """Mask of candidate neighbours that see the point through the fluid.

    `wall` is a list of closed polygons (0-based point indices, in ring order).
    A candidate is rejected when the segment to it crosses a wall edge not
    touching either end, and, for a wall point, when it lies behind the wall's
    tangent line by more than a quarter of its distance (a point on the far
    side of a thin trailing edge).
    """
    from scipy.spatial import cKDTree

    rows = np.atleast_1d(np.arange(x.shape[0]) if rows is None else rows)
    n, k = idx.shape
    ok = np.ones((n, k), bool)
    wmask = flag[rows] == 0
    deln = dx * nx[rows][:, None] + dy * ny[rows][:, None]
    ok &= ~(wmask[:, None] & (deln < -0.25 * dist))
    if cache is None:
        cache = {}
    if "dw" not in cache:
        ea = np.concatenate([np.asarray(w) for w in wall])
        eb = np.concatenate([np.roll(np.asarray(w), -1) for w in wall])
        mids = np.stack([(x[ea] + x[eb]) * 0.5, (y[ea] + y[eb]) * 0.5], 1)
        wpts = np.unique(ea)
        dw, _ = cKDTree(np.stack([x[wpts], y[wpts]], 1)).query(np.stack([x, y], 1), workers=-1)
        cache.update(ea=ea, eb=eb, mids=mids, etree=cKDTree(mids), dw=dw)
    ea, eb, mids, etree, dw = cache["ea"], cache["eb"], cache["mids"], cache["etree"], cache["dw"]
    need = (np.minimum(dw[rows][:, None], dw[idx]) <= dist) & np.isfinite(dist)
    rr, jj = np.nonzero(need)
    if rr.size == 0:
        return ok
    ii = rows[rr]
    kk = idx[rr, jj]
    ax, ay, bx, by = x[ii], y[ii], x[kk], y[kk]
    _, near = etree.query(np.stack([(ax + bx) * 0.5, (ay + by) * 0.5], 1), k=min(8, len(mids)), workers=-1)
    cross = np.zeros(ii.size, bool)

    def orient(px, py, qx, qy, rx, ry):
        return (qx - px) * (ry - py) - (qy - py) * (rx - px)

    for c in range(near.shape[1]):
        e0 = ea[near[:, c]]
        e1 = eb[near[:, c]]
        touch = (e0 == ii) | (e0 == kk) | (e1 == ii) | (e1 == kk)
        cx0, cy0, cx1, cy1 = x[e0], y[e0], x[e1], y[e1]
        o1 = orient(ax, ay, bx, by, cx0, cy0)
        o2 = orient(ax, ay, bx, by, cx1, cy1)
        o3 = orient(cx0, cy0, cx1, cy1, ax, ay)
        o4 = orient(cx0, cy0, cx1, cy1, bx, by)
        cross |= (~touch) & (o1 * o2 < 0) & (o3 * o4 < 0)
    ok[rr[cross], jj[cross]] = False
    return ok


def build_connectivity(x, y, nx, ny, flag, ht, hn, tx_, ty_, n_nbrs=10, nbr_radius=2.5,
                       n_cand=32, min_rcond=1e-3, wall=None, chunk=1 << 20, max_weight=np.inf, max_wrong=np.inf):
    """conn [N, 20] (0-based, -1 padded) and counts.

    Candidates come from a k-d tree; they are ranked by distance in the local
    spacing frame (tangent (tx_, ty_) scaled by ht, normal scaled by hn), kept
    within nbr_radius * max(ht, hn), and the first n_nbrs are taken.  Points
    whose sub-stencils fail `_stencil_ok` take further candidates one by one.
    Rows are processed `chunk` at a time to bound memory on large clouds.
    """
    from scipy.spatial import cKDTree

    n = x.shape[0]
    pts = np.stack([x, y], 1)
    tree = cKDTree(pts)
    hmax = np.maximum(ht, hn)
    k = min(n_cand + 1, n)
    conn = np.full((n, MAX_NBHS), -1, np.int64)
    cnt = np.zeros(n, np.int64)
    bad_all = []
    vis_cache = {}
    for r0 in range(0, n, chunk):
        rows = np.arange(r0, min(n, r0 + chunk))
        _, idx = tree.query(pts[rows], k=k, workers=-1)
        idx = idx[:, 1:]                                   # drop self
        dx = x[idx] - x[rows, None]
        dy = y[idx] - y[rows, None]
        dist = np.sqrt(dx * dx + dy * dy)
        st = (dx * tx_[rows, None] + dy * ty_[rows, None]) / ht[rows, None]
        sn = (dx * (-ty_)[rows, None] + dy * tx_[rows, None]) / hn[rows, None]
        sd = np.sqrt(st * st + sn * sn)
        del st, sn
        inside = dist <= nbr_radius * hmax[rows, None]
        if wall is not None:
            inside &= _visible(x, y, nx, ny, flag, rows, idx, dx, dy, dist, wall, vis_cache)
        sd = np.where(inside, sd, np.inf)
        order = np.argsort(sd, axis=1, kind="stable")
        idx = np.take_along_axis(idx, order, 1)
        sd = np.take_along_axis(sd, order, 1)
        dx = np.take_along_axis(dx, order, 1)
        dy = np.take_along_axis(dy, order, 1)
        finite = np.isfinite(sd)
        # reference split frame: t = (ny, -nx), n = (nx, ny)
        dels_all = dx * ny[rows, None] - dy * nx[rows, None]
        deln_all = dx * nx[rows, None] + dy * ny[rows, None]
        take = np.minimum(n_nbrs, finite.sum(1))
        kk = np.arange(idx.shape[1])[None, :]
        valid = (kk < take[:, None]) & finite
        fl = flag[rows]
        ok = _stencil_ok(dels_all, deln_all, valid, fl, min_rcond=min_rcond, max_weight=max_weight,
                         max_wrong=max_wrong)
        bad = np.nonzero(~ok)[0]
        # grow failing stencils one candidate at a time, up to MAX_NBHS
        for extra in range(MAX_NBHS - n_nbrs):
            if bad.size == 0:
                break
            take[bad] = np.minimum(take[bad] + 1, np.minimum(MAX_NBHS, finite[bad].sum(1)))
            vb = (kk < take[bad][:, None]) & finite[bad]
            okb = _stencil_ok(dels_all[bad], deln_all[bad], vb, fl[bad], min_rcond=min_rcond,
                              max_weight=max_weight, max_wrong=max_wrong)
            bad = bad[~okb]
        valid = (kk < take[:, None]) & finite
        conn[rows] = np.where(valid, idx, -1)[:, :MAX_NBHS]
        cnt[rows] = valid.sum(1)
        bad_all.append(rows[bad])
    bad = np.concatenate(bad_all) if bad_all else np.zeros(0, np.int64)
    if bad.size:
        conn, cnt, bad = _repair(conn, cnt, bad, x, y, nx, ny, flag, hmax, tree, n_nbrs, min_rcond, wall, vis_cache,
                                 max_weight, max_wrong)
    return conn, cnt, bad


def _rcond(dels, deln):
    """Reciprocal condition number of the 2x2 LSQ matrix of one sub-stencil."""
    sxx = float((dels * dels).sum())
    syy = float((deln * deln).sum())
    sxy = float((dels * deln).sum())
    tr = sxx + syy
    det = sxx * syy - sxy * sxy
    disc = math.sqrt(max(tr * tr * 0.25 - det, 0.0))
    lmax = tr * 0.5 + disc
    return (tr * 0.5 - disc) / lmax if lmax > 0 else 0.0


def _score(rc, bound, wrong, min_rcond, max_weight, max_wrong):
    return np.maximum(np.maximum(np.where(rc > 0, min_rcond / np.where(rc > 0, rc, 1.0), np.inf), bound / max_weight),
                      wrong / max_wrong)


def _badness(dels, deln, along_s, dmin, sign, min_rcond, max_weight, max_wrong):
    """> 1 when one sub-stencil fails: fewer than 2 members, reciprocal
    condition number below min_rcond, weight bound above max_weight or
    wrong-sign weight above max_wrong."""
    if dels.size < 2:
        return np.inf
    _, rc, bound, wrong = _sub_stats(dels[None, :], deln[None, :], np.ones((1, dels.size), bool), along_s,
                                     np.array([dmin]), sign)
    return float(_score(rc, bound, wrong, min_rcond, max_weight, max_wrong)[0])


def _repair(conn, cnt, bad, x, y, nx, ny, flag, hmax, tree, n_nbrs, min_rcond, wall=None, vis_cache=None,
            max_weight=np.inf, max_wrong=np.inf):
    """Fix the few stencils the ranked selection leaves ill-posed.

    For each such point: restart from its n_nbrs nearest (Euclidean) points
    and, while some sub-stencil its class uses fails (`_badness`), add the
    point in that sub-stencil's half-plane (among the 256 nearest) that leaves
    the sub-stencil the least bad.
    """
    still = []
    for i in bad:
        _, cand = tree.query([x[i], y[i]], k=min(257, x.shape[0]))
        cand = np.array([int(c) for c in cand if c != i])
        dx = x[cand] - x[i]
        dy = y[cand] - y[i]
        if wall is not None:
            vis = _visible(x, y, nx, ny, flag, i, cand[None, :], dx[None, :], dy[None, :],
                           np.sqrt(dx * dx + dy * dy)[None, :], wall, vis_cache)[0]
            cand, dx, dy = cand[vis], dx[vis], dy[vis]
        dist = np.sqrt(dx * dx + dy * dy)
        dels = dx * ny[i] - dy * nx[i]
        deln = dx * nx[i] + dy * ny[i]
        allm = np.ones(len(cand), bool)
        want = [dels <= 0.0, dels >= 0.0,
                (deln <= 0.0) if flag[i] == 1 else (allm if flag[i] == 2 else None),
                (deln >= 0.0) if flag[i] == 1 else (allm if flag[i] == 0 else None)]
        sel = np.zeros(len(cand), bool)
        sel[:n_nbrs] = True

        sgn = [(_HALF_SIGN[d] if (d < 2 or flag[i] == 1) else 0.0) for d in range(4)]

        def failing(d, dmin, strict=True):
            w = sel & want[d]
            return _badness(dels[w], deln[w], d < 2, dmin, sgn[d], min_rcond, max_weight if strict else np.inf,
                            max_wrong if strict else np.inf) > 1.0

        while sel.sum() < MAX_NBHS:
            dmin = dist[sel].min()
            worst = next((d for d in range(4) if want[d] is not None and failing(d, dmin)), None)
            if worst is None:
                break
            cands = np.nonzero(want[worst] & ~sel)[0]
            if cands.size == 0:
                break
            m = np.nonzero(sel & want[worst])[0]
            ds = np.concatenate([np.broadcast_to(dels[m], (cands.size, m.size)), dels[cands][:, None]], 1)
            dn = np.concatenate([np.broadcast_to(deln[m], (cands.size, m.size)), deln[cands][:, None]], 1)
            cnt_c, rc_c, bound_c, wrong_c = _sub_stats(ds, dn, np.ones(ds.shape, bool), worst < 2,
                                                       np.minimum(dmin, dist[cands]), sgn[worst])
            score = np.where(cnt_c >= 2, _score(rc_c, bound_c, wrong_c, min_rcond, max_weight, max_wrong), np.inf)
            sel[cands[int(np.argmin(score))]] = True
        chosen = np.nonzero(sel)[0]
        # degenerate stencils are errors; a weight bound that 20 neighbours
        # cannot meet is left at the best stencil found
        dmin = dist[sel].min()
        if any(want[d] is not None and failing(d, dmin, strict=False) for d in range(4)):
            still.append(i)
        conn[i, :] = -1
        conn[i, :len(chosen)] = cand[chosen]
        cnt[i] = len(chosen)
    return conn, cnt, np.array(still, dtype=np.int64)


def make_cloud(n_wall: int = 160, n_layers: int = 60, first_spacing: float = 2e-3,
               radius: float = 20.0, seed: int = 0, jitter: float = 0.1,
               n_nbrs: int = 10, nbr_radius: float = 2.5,
               m: float = 0.0, p: float = 0.4, t: float = 0.12,
               min_rcond: float = 1e-3, smooth: int = 30, max_weight: float = 2.5,
               max_wrong: float = 0.3, te_spread: float = 0.0) -> Cloud:
    """Generate a seeded NACA 4-digit O-type point cloud (see module docstring).

    Point order: wall ring (flag_1 0, flag_2 1), interior rings (flag_1 1),
    far-field ring (flag_1 2); inside a ring, counter-clockwise from the
    trailing edge.
    """
    X, Y, _ = make_layers(n_wall, n_layers, first_spacing, radius, m, p, t, smooth=smooth, te_spread=te_spread)
    L, W = X.shape
    # local spacing: half the central difference along / across rings
    Xp, Xm = np.roll(X, -1, 1), np.roll(X, 1, 1)
    Yp, Ym = np.roll(Y, -1, 1), np.roll(Y, 1, 1)
    tx = Xp - Xm
    ty = Yp - Ym
    ht = 0.5 * np.sqrt(tx * tx + ty * ty)
    tl = np.sqrt(tx * tx + ty * ty)
    tx, ty = tx / tl, ty / tl
    dxn = np.empty_like(X)
    dyn = np.empty_like(Y)
    dxn[1:-1] = X[2:] - X[:-2]; dyn[1:-1] = Y[2:] - Y[:-2]
    dxn[0] = 2 * (X[1] - X[0]); dyn[0] = 2 * (Y[1] - Y[0])
    dxn[-1] = 2 * (X[-1] - X[-2]); dyn[-1] = 2 * (Y[-1] - Y[-2])
    hn = 0.5 * np.sqrt(dxn * dxn + dyn * dyn)

    rng = np.random.default_rng(seed)
    u = rng.uniform(-1.0, 1.0, size=(2, L, W))
    jx = jitter * (u[0] * ht * tx + u[1] * hn * (-ty))
    jy = jitter * (u[0] * ht * ty + u[1] * hn * tx)
    jx[0] = jx[-1] = 0.0
    jy[0] = jy[-1] = 0.0
    X = X + jx
    Y = Y + jy

    n = L * W
    x = X.reshape(-1).copy()
    y = Y.reshape(-1).copy()
    flag = np.ones(n, np.int32)
    flag[:W] = 0
    flag[-W:] = 2
    ring = np.arange(W)
    left = np.zeros(n, np.int32)
    right = np.zeros(n, np.int32)
    # 1-based; left = next CCW, right = previous CCW (normals into the fluid)
    left[:W] = (ring + 1) % W + 1
    right[:W] = (ring - 1) % W + 1
    left[-W:] = (n - W) + (ring + 1) % W + 1
    right[-W:] = (n - W) + (ring - 1) % W + 1
    f2 = np.zeros(n, np.int32)
    f2[:W] = 1

    # normals exactly as the reference computes them (for the split checks)
    nx = np.zeros(n)
    ny = np.ones(n)
    for sl, lo in ((slice(0, W), 0), (slice(n - W, n), n - W)):
        li = left[sl] - 1
        ri = right[sl] - 1
        nxx = 0.5 * ((y[sl] - y[li]) + (y[ri] - y[sl]))
        nyy = 0.5 * ((x[sl] - x[li]) + (x[ri] - x[sl]))
        d = np.sqrt(nxx * nxx + nyy * nyy)
        nx[sl] = -nxx / d
        ny[sl] = nyy / d

    conn0, cnt, bad = build_connectivity(
        x, y, nx, ny, flag, ht.reshape(-1), hn.reshape(-1), tx.reshape(-1), ty.reshape(-1),
        n_nbrs=n_nbrs, nbr_radius=nbr_radius, min_rcond=min_rcond, wall=[np.arange(W)], max_weight=max_weight,
        max_wrong=max_wrong)
    if bad.size:
        raise RuntimeError(f"{bad.size} points have degenerate sub-stencils even with {MAX_NBHS} neighbours")
    conn = np.zeros((n, MAX_NBHS), np.int32)
    valid = conn0 >= 0
    conn[valid] = (conn0[valid] + 1).astype(np.int32)
    dxs = np.where(valid, x[np.maximum(conn0, 0)] - x[:, None], np.inf)
    dys = np.where(valid, y[np.maximum(conn0, 0)] - y[:, None], np.inf)
    md = np.sqrt(dxs * dxs + dys * dys).min(1)
    return Cloud(x, y, left, right, flag, f2, md, cnt.astype(np.int32), conn)


def config1_cloud(seed: int = 1) -> Cloud:
    """NACA 0012, 160 cosine-spaced wall points x 60 rings = 9,600 points."""
    return make_cloud(n_wall=160, n_layers=60, first_spacing=2e-3, radius=20.0, seed=seed)


def config2_cloud(seed: int = 2) -> Cloud:
    """NACA 0012, 1024 wall points x 1000 rings = 1,024,000 points, the
    trailing-edge wall spacing spread to the 160-point ring's (te_spread)."""
    return make_cloud(n_wall=1024, n_layers=1000, first_spacing=2e-3, radius=20.0, seed=seed, te_spread=0.064)


# ---------------------------------------------------------------------------
# Two-element (main element + slotted flap) clouds
# ---------------------------------------------------------------------------

def _naca_thickness(xc: np.ndarray, t: float) -> np.ndarray:
    xc = np.clip(xc, 0.0, 1.0)
    return 5.0 * t * (0.2969 * np.sqrt(xc) - 0.1260 * xc - 0.3516 * xc**2 + 0.2843 * xc**3 - 0.1036 * xc**4)


@dataclasses.dataclass
class _Body:
    """A symmetric NACA 00tt section of chord `chord`, leading edge at `le`,
    chord line turned by `deflect` degrees (positive: trailing edge down)."""

    chord: float
    le: tuple
    deflect: float = 0.0
    t: float = 0.12

    def _frame(self):
        d = math.radians(self.deflect)
        return math.cos(d), math.sin(d)

    def surface(self, theta):
        """Points at surface parameter theta (naca4_surface), counter-clockwise."""
        u, v = naca4_surface(theta, 0.0, 0.4, self.t)
        c, s = self._frame()
        u = u * self.chord
        v = v * self.chord
        return self.le[0] + u * c + v * s, self.le[1] - u * s + v * c

    def inside(self, x, y):
        c, s = self._frame()
        dx, dy = x - self.le[0], y - self.le[1]
        u = (dx * c - dy * s) / self.chord
        v = (dx * s + dy * c) / self.chord
        return (u >= 0.0) & (u <= 1.0) & (np.abs(v) <= _naca_thickness(u, self.t))


def _offset_rings(wx, wy, first, thickness, n_layers, smooth):
    """Rings 1..n_layers-1 off a closed wall ring along smoothed normals, offsets
    growing geometrically from `first` to `thickness`; returns X, Y [L, W], d."""
    nx, ny = _rot_normals(wx, wy)
    for _ in range(smooth):
        sx = np.roll(nx, 1) + 2.0 * nx + np.roll(nx, -1)
        sy = np.roll(ny, 1) + 2.0 * ny + np.roll(ny, -1)
        ln = np.sqrt(sx * sx + sy * sy)
        nx, ny = sx / ln, sy / ln
    g = solve_growth(first, n_layers - 1, thickness)
    j = np.arange(n_layers, dtype=np.float64)
    d = first * j if g == 1.0 else first * (g**j - 1.0) / (g - 1.0)
    return wx[None, :] + d[:, None] * nx[None, :], wy[None, :] + d[:, None] * ny[None, :], d


def _ring_frame(X, Y, d):
    """Tangent, tangential and normal spacing of ring points [L, W]."""
    tx = np.roll(X, -1, 1) - np.roll(X, 1, 1)
    ty = np.roll(Y, -1, 1) - np.roll(Y, 1, 1)
    tl = np.sqrt(tx * tx + ty * ty)
    ht = 0.5 * tl
    dd = np.gradient(d)
    hn = np.broadcast_to(dd[:, None], X.shape).copy()
    return tx / tl, ty / tl, ht, hn


def two_element_cloud(n_main: int = 4096, n_flap: int = 1024, flap_chord: float = 0.3, deflect: float = 20.0,
                      gap: float = 0.015, overlap: float = 0.01, n_layers: int = 12, first_spacing: float = 1e-4,
                      h0: float = 1.5e-4, growth: float = 0.0033, radius: float = 20.0, seed: int = 5,
                      jitter: float = 0.1, n_nbrs: int = 10, nbr_radius: float = 2.5,
                      min_rcond: float = 1e-3, smooth: int = 30, max_weight: float = 2.5,
               max_wrong: float = 0.3) -> Cloud:
    """Seeded two-element cloud: NACA 0012 main element (chord 1, leading edge
    at the origin) and a NACA 0012 flap of chord `flap_chord` turned by
    `deflect` degrees whose leading edge sits `overlap` ahead of the main
    trailing edge, lowered until the closest distance between the two
    surfaces is `gap` (the slot).

    * Walls: `n_main` and `n_flap` cosine-spaced points (flag_2 1 and 2, both
      rings first, main then flap; ring order and left / right as in
      make_cloud, so the reference's normals point into the fluid).
    * Layers: `n_layers` - 1 geometric rings off each wall up to a thickness
      of 0.4 gap (so the two stacks never meet in the slot), rays smoothed
      along the ring at the sharp trailing edges.
    * Background: Poisson-like jittered points from nested grids whose spacing
      h = h0 + growth * (distance beyond the layers) doubles from one grid to
      the next, a grid keeping the points whose h falls in its octave;
      points inside a body or closer to a wall than the layers' edge are
      dropped.  h0 and growth set the size (about 16M points by default).
    * Far field: a ring of radius `radius` about mid-chord at the local h.
    """
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    main = _Body(1.0, (0.0, 0.0))
    th = lambda n: 2.0 * np.pi * np.arange(n) / n
    mx, my = main.surface(th(n_main))
    # slot: lower the flap until the closest surface distance is `gap`
    dense_m = np.stack(main.surface(th(20000)), 1)
    tm = cKDTree(dense_m)

    def slot(yoff):
        fb = _Body(flap_chord, (1.0 - overlap, yoff), deflect)
        return float(tm.query(np.stack(fb.surface(th(8000)), 1))[0].min())

    lo, hi = -0.3, 0.0
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        lo, hi = (lo, mid) if slot(mid) < gap else (mid, hi)
    flap = _Body(flap_chord, (1.0 - overlap, lo), deflect)
    fx, fy = flap.surface(th(n_flap))
    thick = 0.4 * gap
    Xm, Ym, dm = _offset_rings(mx, my, first_spacing, thick, n_layers, smooth)
    Xf, Yf, df = _offset_rings(fx, fy, first_spacing, thick, n_layers, smooth)
    tmx, tmy, htm, hnm = _ring_frame(Xm, Ym, dm)
    tfx, tfy, htf, hnf = _ring_frame(Xf, Yf, df)

    # layer jitter (not on the walls)
    def jit(X, Y, tx, ty, ht, hn):
        u = rng.uniform(-1.0, 1.0, size=(2,) + X.shape) * 0.1
        jx = u[0] * ht * tx - u[1] * hn * ty
        jy = u[0] * ht * ty + u[1] * hn * tx
        jx[0] = jy[0] = 0.0
        return X + jx, Y + jy

    Xm, Ym = jit(Xm, Ym, tmx, tmy, htm, hnm)
    Xf, Yf = jit(Xf, Yf, tfx, tfy, htf, hnf)

    # distance to the bodies from dense surface samples
    dense = np.concatenate([dense_m, np.stack(flap.surface(th(20000)), 1)])
    tb = cKDTree(dense)
    center = np.array([0.5, 0.0])
    h_of = lambda dist: h0 + growth * np.maximum(dist - thick, 0.0)
    r_far = radius
    h_far = float(h_of(np.array([r_far - 0.5]))[0])

    bx0, bx1 = float(dense[:, 0].min()), float(dense[:, 0].max())
    by0, by1 = float(dense[:, 1].min()), float(dense[:, 1].max())
    pts_bg, h_bg = [], []
    level = 0
    while True:
        s_l = h0 * 2.0**level
        lo_d = thick + (s_l - h0) / growth if level > 0 else 0.0
        hi_d = thick + (2.0 * s_l - h0) / growth
        m = min(hi_d, r_far + 1.0)
        x0, x1 = max(bx0 - m, center[0] - r_far), min(bx1 + m, center[0] + r_far)
        y0, y1 = max(by0 - m, -r_far), min(by1 + m, r_far)
        # coarse cells that can hold points of this octave
        cs = 32.0 * s_l
        cxs = np.arange(x0, x1, cs) + 0.5 * cs
        cys = np.arange(y0, y1, cs) + 0.5 * cs
        CX, CY = np.meshgrid(cxs, cys, indexing="xy")
        cc = np.stack([CX.ravel(), CY.ravel()], 1)
        cd, _ = tb.query(cc, workers=-1)
        rad = np.sqrt(((cc - center) ** 2).sum(1))
        half = 0.75 * cs
        keep = (cd + half >= lo_d) & (cd - half < hi_d) & (rad - half < r_far)
        cc = cc[keep]
        nper = int(round(cs / s_l))
        if cc.size:
            g = (np.arange(nper) + 0.5) * s_l - 0.5 * cs
            GX, GY = np.meshgrid(g, g, indexing="xy")
            for c0 in range(0, cc.shape[0], 2048):
                blk = cc[c0:c0 + 2048]
                px = (blk[:, 0:1] + GX.ravel()[None, :]).ravel()
                py = (blk[:, 1:2] + GY.ravel()[None, :]).ravel()
                u = rng.uniform(-0.5, 0.5, size=(2, px.size)) * jitter * s_l
                px += u[0]
                py += u[1]
                dd, _ = tb.query(np.stack([px, py], 1), workers=-1)
                rr = np.sqrt((px - center[0]) ** 2 + (py - center[1]) ** 2)
                ok = (dd >= max(lo_d, thick + 0.5 * s_l)) & (dd < hi_d) & (rr < r_far - 0.5 * h_far)
                ok &= ~main.inside(px, py) & ~flap.inside(px, py)
                pts_bg.append(np.stack([px[ok], py[ok]], 1))
                h_bg.append(np.full(int(ok.sum()), s_l))
        if hi_d > r_far + 2.0 * (bx1 - bx0) or s_l > h_far * 2.0:
            break
        level += 1
    bg = np.concatenate(pts_bg) if pts_bg else np.zeros((0, 2))
    hb = np.concatenate(h_bg) if h_bg else np.zeros(0)

    n_out = max(64, int(round(2.0 * np.pi * r_far / h_far)))
    tho = th(n_out)
    ox = center[0] + r_far * np.cos(tho)
    oy = center[1] + r_far * np.sin(tho)

    # assemble: main wall, flap wall, layers, background, outer ring
    Wm, Wf = n_main, n_flap
    x = np.concatenate([Xm[0], Xf[0], Xm[1:].ravel(), Xf[1:].ravel(), bg[:, 0], ox])
    y = np.concatenate([Ym[0], Yf[0], Ym[1:].ravel(), Yf[1:].ravel(), bg[:, 1], oy])
    ht = np.concatenate([htm[0], htf[0], htm[1:].ravel(), htf[1:].ravel(), hb, np.full(n_out, h_far)])
    hn = np.concatenate([hnm[0], hnf[0], hnm[1:].ravel(), hnf[1:].ravel(), hb, np.full(n_out, h_far)])
    tx_ = np.concatenate([tmx[0], tfx[0], tmx[1:].ravel(), tfx[1:].ravel(), np.ones(hb.size), -np.sin(tho)])
    ty_ = np.concatenate([tmy[0], tfy[0], tmy[1:].ravel(), tfy[1:].ravel(), np.zeros(hb.size), np.cos(tho)])
    n = x.size
    flag = np.ones(n, np.int32)
    flag[:Wm + Wf] = 0
    flag[-n_out:] = 2
    f2 = np.zeros(n, np.int32)
    f2[:Wm] = 1
    f2[Wm:Wm + Wf] = 2
    left = np.zeros(n, np.int32)
    right = np.zeros(n, np.int32)
    for start, w in ((0, Wm), (Wm, Wf), (n - n_out, n_out)):
        ring = np.arange(w)
        left[start:start + w] = start + (ring + 1) % w + 1
        right[start:start + w] = start + (ring - 1) % w + 1
    nx = np.zeros(n)
    ny = np.ones(n)
    for sl in (slice(0, Wm + Wf), slice(n - n_out, n)):
        li = left[sl] - 1
        ri = right[sl] - 1
        nxx = 0.5 * ((y[sl] - y[li]) + (y[ri] - y[sl]))
        nyy = 0.5 * ((x[sl] - x[li]) + (x[ri] - x[sl]))
        d = np.sqrt(nxx * nxx + nyy * nyy)
        nx[sl] = -nxx / d
        ny[sl] = nyy / d
    conn0, cnt, bad = build_connectivity(x, y, nx, ny, flag, ht, hn, tx_, ty_, n_nbrs=n_nbrs,
                                         nbr_radius=nbr_radius, min_rcond=min_rcond,
                                         wall=[np.arange(Wm), Wm + np.arange(Wf)], max_weight=max_weight,
                                         max_wrong=max_wrong)
    if bad.size:
        raise RuntimeError(f"{bad.size} points have degenerate sub-stencils even with {MAX_NBHS} neighbours")
    conn = np.zeros((n, MAX_NBHS), np.int32)
    valid = conn0 >= 0
    conn[valid] = (conn0[valid] + 1).astype(np.int32)
    md = np.full(n, np.inf)
    for r0 in range(0, n, 1 << 20):
        sl = slice(r0, min(n, r0 + (1 << 20)))
        v = valid[sl]
        c0 = np.maximum(conn0[sl], 0)
        dxs = np.where(v, x[c0] - x[sl, None], np.inf)
        dys = np.where(v, y[c0] - y[sl, None], np.inf)
        md[sl] = np.sqrt(dxs * dxs + dys * dys).min(1)
    return Cloud(x, y, left, right, flag, f2, md, cnt.astype(np.int32), conn)
