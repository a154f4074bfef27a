"""Partitions with ghost points on the CPU (no GPU): the plan the library
computes (qlskum_partition_plan / _plan_lists, the reference's local_points /
ghost_points / pghost layout) and the ghost exchange it implies, run by two
gloo ranks that each hold one partition.

The exchange test applies a neighbour stencil three times in a row (as the
inner iterations do), refreshing the ghosts over gloo before every
application, and must reproduce the single-domain result bit for bit: every
point's arithmetic reads the same values in the same order.
"""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import REPO, golden_cloud


def _stencil(u, conn, nbhs):
    """out_i = u_i + sum_j (u_k - u_i) / nbhs_i over the listed neighbours, in list order."""
    out = u.copy()
    acc = np.zeros_like(u)
    for j in range(conn.shape[1]):
        use = j < nbhs
        k = np.where(use, conn[:, j], 0)
        acc += np.where(use[:, None], (u[k] - u) / nbhs[:, None], 0.0)
    return out + acc


def _field(n, seed=3):
    return np.random.default_rng(seed).standard_normal((n, 4))


def test_plan_covers_cloud_and_closes_stencils():
    import qlskum
    c = golden_cloud("cloud_trans")
    for parts in (2, 3, 5):
        part_of, lists = qlskum.partition_plan(c, parts)
        assert part_of.min() == 0 and part_of.max() == parts - 1
        sizes = np.bincount(part_of, minlength=parts)
        assert sizes.max() - sizes.min() <= 1
        seen = np.zeros(c.n, bool)
        for p, (loc, gh) in enumerate(lists):
            loc0, gh0 = loc - 1, gh - 1
            assert len(loc0) == sizes[p] and np.all(part_of[loc0] == p)
            assert not seen[loc0].any()
            seen[loc0] = True
            # ghosts: unique, owned elsewhere, grouped by owner
            assert len(np.unique(gh0)) == len(gh0)
            assert np.all(part_of[gh0] != p)
            assert np.all(np.diff(part_of[gh0]) >= 0)
            # every neighbour of an owned point is owned or a ghost, and every ghost is needed
            nb = np.concatenate([c.conn[i, :c.nbhs[i]] - 1 for i in loc0])
            outside = np.unique(nb[part_of[nb] != p])
            assert np.array_equal(np.sort(gh0), outside)
        assert seen.all()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, results):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    for p in (os.path.join(REPO, "c-_serial_gb300"), os.path.join(REPO, "tests")):
        sys.path.insert(0, p)
    import torch
    import torch.distributed as dist
    import qlskum
    from conftest import golden_cloud as gc
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        c = gc("cloud_trans")
        part_of, lists = qlskum.partition_plan(c, world)
        loc, gh = (lists[rank][0] - 1, lists[rank][1] - 1)
        slots = np.concatenate([loc, gh])
        slot_of = np.full(c.n, -1)
        slot_of[slots] = np.arange(len(slots))
        conn = np.where(np.arange(20)[None, :] < c.nbhs[loc][:, None], slot_of[np.maximum(c.conn[loc] - 1, 0)], 0)
        assert (conn[np.arange(20)[None, :] < c.nbhs[loc][:, None]] >= 0).all()
        u = np.zeros((len(slots), 4))
        u[:len(loc)] = _field(c.n)[loc]
        pos = {g: t for t, g in enumerate(loc)}

        def exchange():
            reqs, recv = [], {}
            for o in range(world):
                if o == rank:
                    continue
                # what o mirrors of ours, in o's ghost order; what we mirror of o's
                theirs = lists[o][1] - 1
                send = theirs[part_of[theirs] == rank]
                buf = torch.from_numpy(np.ascontiguousarray(u[[pos[g] for g in send]]))
                reqs.append(dist.isend(buf, dst=o))
                mine = np.nonzero(part_of[gh] == o)[0]
                recv[o] = (mine, torch.empty((len(mine), 4), dtype=torch.float64))
                reqs.append(dist.irecv(recv[o][1], src=o))
            for r in reqs:
                r.wait()
            for o, (mine, t) in recv.items():
                u[len(loc) + mine] = t.numpy()

        for _ in range(3):
            exchange()
            u[:len(loc)] = _apply(u, conn, c.nbhs[loc])
        results[rank] = (loc, u[:len(loc)].copy())
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _apply(u, conn, nbhs):
    """The stencil on the owned points, reading owned and ghost slots."""
    n = len(nbhs)
    acc = np.zeros((n, 4))
    for j in range(conn.shape[1]):
        use = j < nbhs
        k = np.where(use, conn[:, j], 0)
        acc += np.where(use[:, None], (u[k] - u[:n]) / nbhs[:, None], 0.0)
    return u[:n] + acc


def test_ghost_exchange_world2_matches_single_domain():
    torch = pytest.importorskip("torch")
    c = golden_cloud("cloud_trans")
    ref = _field(c.n)
    conn0 = np.maximum(c.conn - 1, 0)
    for _ in range(3):
        ref = _stencil(ref, conn0, c.nbhs)
    mp = torch.multiprocessing.get_context("spawn")
    mgr = mp.Manager()
    results = mgr.dict()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
        assert p.exitcode == 0
    got = np.full_like(ref, np.nan)
    for r in range(2):
        loc, vals = results[r]
        got[loc] = vals
    assert np.array_equal(got, ref)
