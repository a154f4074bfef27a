"""Diagnostics and state files through the C ABI on the GPU.

* enstrophy (compute_enstrophy_mod.h) and the stagnation-pressure extremes
  and objective J (stagnation_values_mod.h, with the reference's two defects
  fixed as the header states) against the oracle, FP64 (1e-12);
* restart: writing restart.dat after N iterations and continuing a fresh
  handle from it reproduces the uninterrupted run bit for bit, including the
  residual history (res_old from the file, iteration numbers continued);
* the fixed print_primal_output columns.
"""
import os
import tempfile

import numpy as np
import pytest

from conftest import golden_cloud

pytestmark = pytest.mark.gpu

KW = dict(mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, power=0.0, inner_iterations=1)


@pytest.fixture(scope="module")
def qlskum():
    import qlskum as q
    q.load()
    return q


def test_enstrophy_and_stagnation_vs_oracle(qlskum, oracle_mod):
    c = golden_cloud("cloud_trans")
    s = qlskum.Solver(c, **KW)
    s.q_lskum(15)
    o = oracle_mod.Oracle(c, threads=4, **KW)
    o.run(15)
    tot, vort = s.enstrophy()
    otot, ovort = o.enstrophy()
    scale = np.abs(ovort).max()
    assert np.abs(vort - ovort).max() <= 1e-10 * scale
    assert abs(tot - otot) <= 1e-10 * otot
    g = s.stagnation()
    r = o.stagnation()
    np.testing.assert_allclose([g[0], g[1], g[4]], [r[0], r[1], r[4]], rtol=1e-12)
    assert (g[2], g[3]) == (r[2], r[3])


def test_restart_continues_bit_for_bit(qlskum):
    c = golden_cloud("cloud_trans")
    d = tempfile.mkdtemp()
    a = qlskum.Solver(c, **KW)
    a.q_lskum(10)
    b = qlskum.Solver(c, **KW)
    b.q_lskum(6)
    path = os.path.join(d, "restart.dat")
    b.write_restart(path)
    r = qlskum.Solver(c, **KW)
    r.read_restart(path)
    assert r.iteration == 6
    r.q_lskum(4)
    assert r.iteration == 10
    assert np.array_equal(r.prim, a.prim)
    ha, hr = a.residual_history(), r.residual_history()
    assert np.array_equal(hr[6:10], ha[6:10])
    # restart_sol's layout: header n it res_old, five skipped columns, then the state
    tok = open(path).read().split()
    assert int(tok[0]) == c.n and int(tok[1]) == 6
    rows = np.array(tok[3:], float).reshape(c.n, 9)
    np.testing.assert_array_equal(rows[:, 5:9], b.prim)


def test_output_file_columns(qlskum):
    c = golden_cloud("cloud_trans")
    s = qlskum.Solver(c, **KW)
    s.q_lskum(3)
    path = os.path.join(tempfile.mkdtemp(), "output.dat")
    s.write_output(path)
    lines = open(path).read().splitlines()
    assert len(lines) == c.n + 1
    rows = np.array([l.split() for l in lines[1:]], float)
    np.testing.assert_array_equal(rows[:, 0], c.x)
    np.testing.assert_array_equal(rows[:, 3:7], s.prim)
    p = s.prim
    mach = np.sqrt(p[:, 1] ** 2 + p[:, 2] ** 2) / np.sqrt(1.4 * p[:, 3] / p[:, 0])
    np.testing.assert_allclose(rows[:, 7], mach, rtol=1e-14)
    np.testing.assert_allclose(rows[:, 8], s.field(qlskum.FIELD_ENTROPY), rtol=1e-14)
