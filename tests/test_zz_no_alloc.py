"""qlskum_state_update_noalloc: the stage update for callers that cannot
allocate device memory while they run (their device memory comes from their
own pre-allocated arena, or their stage loop must not take cudaMalloc's
synchronisation).  The entry point keeps its residual partials in a static
device array instead of allocated scratch.

Checked through the C ABI against the existing entry point
(qlskum_state_update on a handle) on every call of a full SSPRK iteration
(four calls in a row, stage 3 reading prim_old), then on two calls over a
smaller cloud, whose residual must not pick up the partials the larger
cloud's calls left in the shared array.  The buffers are allocated by the test (torch), never
by the entry point.  Tolerance: the 1e-12 per-stage relative bar of the GPU
parity tests.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_cloud

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a = np.asarray(a, np.float64).reshape(len(a), -1)
    b = np.asarray(b, np.float64).reshape(len(b), -1)
    return float((np.abs(a - b) / np.maximum(np.abs(b).max(axis=0, keepdims=True), 1e-300)).max())


def _entry():
    import qlskum
    L = qlskum.load()
    fn = L.qlskum_state_update_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double] + [C.c_void_p] * 7
    return qlskum, fn


def _stage_inputs(s, qlskum, inner):
    """Run the module pieces up to the flux residual; return what state_update reads."""
    s.eval_q_variables()
    s.eval_q_derivatives()
    for _ in range(inner):
        s.eval_q_inner_loop()
        s.eval_update_innerloop()
    s.cal_flux_residual()
    return s.prim, s.field(qlskum.FIELD_PRIM_OLD), s.field(qlskum.FIELD_FLUX_RES)


def _host_residual(before, after, flag):
    keep = flag != 2
    r2 = (after[keep, 0] - before[keep, 0]) ** 2
    return r2.sum(), r2.max()


def _run_stages(fn, qlskum, torch, c, mach, aoa, inner, stages, pre_iters):
    """Stages `stages` of one iteration on cloud c, each through
    qlskum_state_update_noalloc on torch-owned device buffers and through
    qlskum_state_update on a handle at the same inputs; both results are
    compared after every call (two calls or more in a row)."""
    s = qlskum.Solver(c, mach=mach, aoa=aoa, cfl=0.2, vl_const=50.0, inner_iterations=inner)
    s.q_lskum(pre_iters)
    s.snapshot_prim_old()
    s.func_delta()
    nrm = s.field(qlskum.FIELD_NORMALS)
    dev = torch.device("cuda:0")
    d_flag = torch.tensor(np.asarray(c.flag_1, np.int32), device=dev)
    d_nrm = torch.tensor(nrm, dtype=torch.float64, device=dev)
    d_res = torch.zeros(2, dtype=torch.float64, device=dev)
    d_prim = d_old = None
    for call, rk in enumerate(stages):
        prim_in, prim_old, fr = _stage_inputs(s, qlskum, inner)
        if call == 0:
            d_prim = torch.tensor(prim_in, device=dev)
            d_old = torch.tensor(prim_old, device=dev)
        else:
            # the previous call's output is this stage's input
            assert rel_err(d_prim.cpu().numpy(), prim_in) < 1e-12, f"call {call + 1}: input"
        s.state_update(rk)
        expect = s.prim
        d_fr = torch.tensor(fr, device=dev)
        torch.cuda.synchronize()
        st = fn(c.n, rk, mach, aoa, d_flag.data_ptr(), d_nrm.data_ptr(), d_prim.data_ptr(), d_old.data_ptr(),
                d_fr.data_ptr(), d_res.data_ptr(), None)
        torch.cuda.synchronize()
        assert st == 0, f"call {call + 1} (rk {rk}): status {st}"
        got = d_prim.cpu().numpy()
        assert rel_err(got, expect) < 1e-12, f"call {call + 1} (rk {rk})"
        hs, hm = _host_residual(prim_in, expect, np.asarray(c.flag_1))
        res = d_res.cpu().numpy()
        assert abs(res[0] - hs) <= 1e-12 * hs, (call, rk, res[0], hs)
        assert abs(res[1] - hm) <= 1e-12 * hm, (call, rk, res[1], hm)
    s.close()


def test_noalloc_matches_state_update_full_iteration_then_smaller_cloud():
    """All four SSPRK stages of one iteration (stage 3 is the one that reads
    prim_old, with the far-field points' conserved_vector_Ubar), on a
    2,560-point cloud (10 blocks of partials), then two stages on a 480-point
    cloud (2 blocks): the second run finds the first run's partials still in
    the shared array past its own blocks, and its residual must not see them."""
    import torch
    qlskum, fn = _entry()
    _run_stages(fn, qlskum, torch, golden_cloud("cloud_trans"), 0.63, 2.0, 2, (1, 2, 3, 4), pre_iters=3)
    _run_stages(fn, qlskum, torch, golden_cloud("cloud_small"), 0.7, 1.0, 0, (1, 2), pre_iters=2)


def test_noalloc_rejects_oversize_and_bad_stage():
    """Sizes past the static scratch and bad stage numbers are refused on the
    host before anything is launched (no buffers are passed)."""
    _, fn = _entry()
    limit = 2097152
    invalid = 1
    assert fn(limit + 1, 1, 0.63, 2.0, None, None, None, None, None, None, None) == invalid
    assert fn(10, 5, 0.63, 2.0, None, None, None, None, None, None, None) == invalid
    assert fn(0, 1, 0.63, 2.0, None, None, None, None, None, None, None) == invalid
