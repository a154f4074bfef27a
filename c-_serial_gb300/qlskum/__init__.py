"""Python front end of the GB300 q-LSKUM library (ctypes over include/qlskum.h).

`Solver` mirrors the reference's module API (Pathlessbark8/C-_serial): one
method per module function, with the state resident on the GPU.  The CUDA
library is built in-tree (qlskum.build) and loaded from
c-_serial_gb300/_build/libqlskum.so; there is no CPU fallback -- importing a
missing or unbuildable library raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

FP64 = 0
MIXED = 1

OBJECTIVE_CL = 0
OBJECTIVE_CD = 1
OBJECTIVE_J = 2

FIELD_PRIM, FIELD_PRIM_OLD, FIELD_Q, FIELD_DQ, FIELD_QM, FIELD_FLUX_RES, FIELD_DELTA, FIELD_NORMALS, FIELD_ENTROPY = range(9)
_FIELD_SHAPE = {FIELD_PRIM: (4,), FIELD_PRIM_OLD: (4,), FIELD_Q: (4,), FIELD_DQ: (2, 4), FIELD_QM: (2, 4),
                FIELD_FLUX_RES: (4,), FIELD_DELTA: (), FIELD_NORMALS: (2,), FIELD_ENTROPY: ()}

STATUS = {0: "ok", 1: "invalid", 2: "degenerate stencil", 3: "non-finite state", 4: "CUDA error", 5: "unsupported"}


class QlskumError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"qlskum {STATUS.get(status, status)}: {msg}")
        self.status = status


class CloudStruct(C.Structure):
    _fields_ = [("n", C.c_int),
                ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)),
                ("left", C.POINTER(C.c_int)), ("right", C.POINTER(C.c_int)),
                ("flag_1", C.POINTER(C.c_int)), ("flag_2", C.POINTER(C.c_int)),
                ("min_dist", C.POINTER(C.c_double)),
                ("nbhs", C.POINTER(C.c_int)), ("conn", C.POINTER(C.c_int))]


class ParamsStruct(C.Structure):
    _fields_ = [("mach", C.c_double), ("aoa", C.c_double), ("cfl", C.c_double), ("vl_const", C.c_double),
                ("power", C.c_double), ("inner_iterations", C.c_int), ("precision", C.c_int),
                ("block_size", C.c_int), ("reorder", C.c_int), ("verbose", C.c_int)]


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_needed: bool = True):
    """Load libqlskum.so (building it first if missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build_if_needed else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"libqlskum.so not found at {path}; run qlskum.build.build()")
    L = C.CDLL(path)
    H = C.c_void_p
    i = C.c_int
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    sig = {
        "qlskum_abi_version": (i, []),
        "qlskum_default_params": (None, [C.POINTER(ParamsStruct)]),
        "qlskum_create": (i, [C.POINTER(CloudStruct), C.POINTER(ParamsStruct), C.POINTER(H)]),
        "qlskum_destroy": (i, [H]),
        "qlskum_last_error": (C.c_char_p, [H]),
        "qlskum_func_delta": (i, [H]),
        "qlskum_eval_q_variables": (i, [H]),
        "qlskum_eval_q_derivatives": (i, [H]),
        "qlskum_eval_q_inner_loop": (i, [H]),
        "qlskum_eval_update_innerloop": (i, [H]),
        "qlskum_cal_flux_residual": (i, [H]),
        "qlskum_state_update": (i, [H, i]),
        "qlskum_snapshot_prim_old": (i, [H]),
        "qlskum_fpi_solver": (i, [H, i]),
        "qlskum_q_lskum": (i, [H, i]),
        "qlskum_objective": (i, [H, dp, dp, dp, dp]),
        "qlskum_get_field": (i, [H, i, dp]),
        "qlskum_set_prim": (i, [H, dp]),
        "qlskum_get_prim": (i, [H, dp]),
        "qlskum_get_connectivity": (i, [H, ip, ip]),
        "qlskum_get_residual_history": (i, [H, dp, i, ip]),
        "qlskum_get_iteration": (i, [H, ip]),
        "qlskum_synchronize": (i, [H]),
        "qlskum_stream": (C.c_void_p, [H]),
        "qlskum_launch_count": (C.c_longlong, [H]),
        "qlskum_get_launch_config": (i, [H, ip, ip, ip, ip]),
        "qlskum_set_launch_config": (i, [H, i, i, i]),
        "qlskum_get_flux_variant": (i, [H]),
        "qlskum_batch_create": (i, [C.POINTER(CloudStruct), i, ip, dp, dp, i, C.POINTER(ParamsStruct), C.POINTER(H)]),
        "qlskum_batch_destroy": (i, [H]),
        "qlskum_batch_last_error": (C.c_char_p, [H]),
        "qlskum_batch_run": (i, [H, i]),
        "qlskum_batch_objective": (i, [H, dp, dp, dp, dp]),
        "qlskum_batch_get_prim": (i, [H, i, dp]),
        "qlskum_batch_residual_history": (i, [H, dp, i, ip]),
        "qlskum_batch_total_points": (C.c_longlong, [H]),
        "qlskum_batch_launch_count": (C.c_longlong, [H]),
        "qlskum_batch_stream": (C.c_void_p, [H]),
        "qlskum_batch_tuning": (i, [H, ip, ip, ip, ip]),
        "qlskum_state_update_noalloc": (i, [i, i, C.c_double, C.c_double] + [C.c_void_p] * 7),
        "qlskum_set_kernel_timing": (i, [H, i]),
        "qlskum_get_kernel_timing": (i, [H, i, dp, C.POINTER(C.c_longlong)]),
        "qlskum_residual_forward": (i, [H, dp, dp]),
        "qlskum_residual_vjp": (i, [H, dp, dp, dp]),
        "qlskum_residual_vjp_full": (i, [H, dp, dp, dp, dp, dp]),
        "qlskum_adjoint_gradient": (i, [H, i, i, dp, dp, dp, dp, dp, dp]),
        "qlskum_adjoint_fixed_point": (i, [H, i, i, dp, dp, dp, dp, dp]),
        "qlskum_set_adjoint_stride": (i, [H, i]),
        "qlskum_enstrophy": (i, [H, dp, dp]),
        "qlskum_stagnation": (i, [H, dp, dp, ip, ip, dp]),
        "qlskum_write_restart": (i, [H, C.c_char_p]),
        "qlskum_read_restart": (i, [H, C.c_char_p]),
        "qlskum_write_output": (i, [H, C.c_char_p]),
        "qlskum_partgrid_read": (i, [C.c_char_p, C.POINTER(CloudStruct)]),
        "qlskum_partgrid_free": (None, [C.POINTER(CloudStruct)]),
        "qlskum_partgrid_write": (i, [C.c_char_p, C.POINTER(CloudStruct)]),
        "qlskum_io_last_error": (C.c_char_p, []),
        "qlskum_check_stencils": (i, [C.POINTER(CloudStruct), C.c_double, C.c_double, dp, ip]),
        "qlskum_residual_forward_device": (i, [H, C.c_void_p, C.c_void_p, C.c_void_p]),
        "qlskum_residual_vjp_device": (i, [H, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
        "qlskum_set_point_lanes": (i, [H, i]),
        "qlskum_get_lanes": (i, [H, ip, ip]),
        "qlskum_batch_lanes": (i, [H, ip, ip]),
        "qlskum_batch_set_launch_config": (i, [H, i, i, i]),
        "qlskum_partition_plan": (i, [C.POINTER(CloudStruct), i, ip, ip, ip]),
        "qlskum_partition_plan_lists": (i, [C.POINTER(CloudStruct), i, i, ip, ip]),
        "qlskum_partition_create": (i, [C.POINTER(CloudStruct), C.POINTER(ParamsStruct), i, C.POINTER(H)]),
        "qlskum_partition_destroy": (i, [H]),
        "qlskum_partition_last_error": (C.c_char_p, [H]),
        "qlskum_partition_layout": (i, [H, i, ip, ip, ip, ip]),
        "qlskum_partition_set_launch_config": (i, [H, i, i, i]),
        "qlskum_partition_q_lskum": (i, [H, i]),
        "qlskum_partition_get_prim": (i, [H, dp]),
        "qlskum_partition_set_prim": (i, [H, dp]),
        "qlskum_partition_residual_history": (i, [H, dp, i, ip]),
        "qlskum_partition_objective": (i, [H, dp, dp, dp, dp]),
        "qlskum_partition_halo_bytes": (C.c_longlong, [H]),
        "qlskum_partition_launch_count": (C.c_longlong, [H]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def cloud_struct(cloud):
    """ctypes view of a cloudgen.Cloud (keeps the backing arrays alive)."""
    keep = dict(
        x=np.ascontiguousarray(cloud.x, np.float64), y=np.ascontiguousarray(cloud.y, np.float64),
        left=np.ascontiguousarray(cloud.left, np.int32), right=np.ascontiguousarray(cloud.right, np.int32),
        f1=np.ascontiguousarray(cloud.flag_1, np.int32), f2=np.ascontiguousarray(cloud.flag_2, np.int32),
        md=np.ascontiguousarray(cloud.min_dist, np.float64), nb=np.ascontiguousarray(cloud.nbhs, np.int32),
        conn=np.ascontiguousarray(cloud.conn, np.int32))
    if keep["conn"].shape != (cloud.n, 20):
        raise ValueError("conn must be [n, 20]")
    s = CloudStruct(cloud.n, _dp(keep["x"]), _dp(keep["y"]), _ip(keep["left"]), _ip(keep["right"]),
                    _ip(keep["f1"]), _ip(keep["f2"]), _dp(keep["md"]), _ip(keep["nb"]), _ip(keep["conn"]))
    return s, keep


def _io_ck(L, st):
    if st != 0:
        raise QlskumError(st, L.qlskum_io_last_error().decode())


def partgrid_read(path):
    """Read a partGrid file with the library's C reader (main.cpp:16-58) into a cloudgen.Cloud."""
    from .cloudgen import Cloud
    L = load()
    c = CloudStruct()
    _io_ck(L, L.qlskum_partgrid_read(os.fsencode(path), C.byref(c)))
    try:
        n = c.n
        arr = lambda ptr, shape, dt: np.ctypeslib.as_array(ptr, shape=shape).astype(dt).copy()
        cloud = Cloud(arr(c.x, (n,), np.float64), arr(c.y, (n,), np.float64), arr(c.left, (n,), np.int32),
                      arr(c.right, (n,), np.int32), arr(c.flag_1, (n,), np.int32), arr(c.flag_2, (n,), np.int32),
                      arr(c.min_dist, (n,), np.float64), arr(c.nbhs, (n,), np.int32),
                      arr(c.conn, (n, 20), np.int32))
    finally:
        L.qlskum_partgrid_free(C.byref(c))
    return cloud


def partgrid_write(cloud, path):
    """Write a cloud with the library's C writer."""
    L = load()
    s, keep = cloud_struct(cloud)
    _io_ck(L, L.qlskum_partgrid_write(os.fsencode(path), C.byref(s)))


def check_stencils(cloud, power=0.0, min_rcond=1e-3):
    """(rcond [n, 4], number of points with a used sub-stencil below min_rcond)."""
    L = load()
    s, keep = cloud_struct(cloud)
    rc = np.empty((cloud.n, 4))
    bad = C.c_int()
    _io_ck(L, L.qlskum_check_stencils(C.byref(s), float(power), float(min_rcond), _dp(rc), C.byref(bad)))
    return rc, bad.value


class Solver:
    """The q-LSKUM solver on one GPU, with the reference's module functions as methods.

    Parameters follow the reference's globals: mach, aoa (degrees), cfl,
    vl_const (VL_CONST), power, inner_iterations; precision FP64 (drop-in) or
    MIXED.  Fields come back in the cloud's original point order.
    """

    def __init__(self, cloud, mach=0.63, aoa=2.0, cfl=0.1, vl_const=150.0, power=0.0, inner_iterations=3,
                 precision=FP64, block_size=0, reorder=True, verbose=False):
        L = load()
        self._L = L
        s, self._keep = cloud_struct(cloud)
        p = ParamsStruct(mach, aoa, cfl, vl_const, power, inner_iterations, precision, block_size,
                         1 if reorder else 0, 1 if verbose else 0)
        h = C.c_void_p()
        st = L.qlskum_create(C.byref(s), C.byref(p), C.byref(h))
        if st != 0:
            raise QlskumError(st, L.qlskum_last_error(None).decode())
        self._h = h
        self.n = cloud.n
        self.shape_points = int((np.asarray(cloud.flag_2) > 0).sum())
        self.params = p

    # ---------------------------------------------------------------- plumbing
    def _ck(self, st):
        if st != 0:
            raise QlskumError(st, self._L.qlskum_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.qlskum_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------- module functions
    def func_delta(self): self._ck(self._L.qlskum_func_delta(self._h))
    def eval_q_variables(self): self._ck(self._L.qlskum_eval_q_variables(self._h))
    def eval_q_derivatives(self): self._ck(self._L.qlskum_eval_q_derivatives(self._h))
    def eval_q_inner_loop(self): self._ck(self._L.qlskum_eval_q_inner_loop(self._h))
    def eval_update_innerloop(self): self._ck(self._L.qlskum_eval_update_innerloop(self._h))
    def cal_flux_residual(self): self._ck(self._L.qlskum_cal_flux_residual(self._h))
    def state_update(self, rk): self._ck(self._L.qlskum_state_update(self._h, int(rk)))
    def snapshot_prim_old(self): self._ck(self._L.qlskum_snapshot_prim_old(self._h))
    def fpi_solver(self, it): self._ck(self._L.qlskum_fpi_solver(self._h, int(it)))
    def q_lskum(self, iters): self._ck(self._L.qlskum_q_lskum(self._h, int(iters)))
    def synchronize(self): self._ck(self._L.qlskum_synchronize(self._h))

    def objective(self):
        """(Cl, Cd, Cm, total entropy)."""
        v = [C.c_double() for _ in range(4)]
        self._ck(self._L.qlskum_objective(self._h, *[C.byref(t) for t in v]))
        return tuple(t.value for t in v)

    # ------------------------------------------------------------- state I/O
    def field(self, which: int) -> np.ndarray:
        out = np.empty((self.n,) + _FIELD_SHAPE[which])
        self._ck(self._L.qlskum_get_field(self._h, which, _dp(out)))
        return out

    @property
    def prim(self): return self.field(FIELD_PRIM)

    def set_prim(self, prim):
        a = np.ascontiguousarray(prim, np.float64)
        if a.shape != (self.n, 4):
            raise ValueError("prim must be [n, 4]")
        self._ck(self._L.qlskum_set_prim(self._h, _dp(a)))

    def connectivity(self):
        counts = np.empty((self.n, 4), np.int32)
        lists = np.empty((self.n, 4, 20), np.int32)
        self._ck(self._L.qlskum_get_connectivity(self._h, _ip(counts), _ip(lists)))
        return counts, lists

    def residual_history(self) -> np.ndarray:
        rows = C.c_int()
        self._ck(self._L.qlskum_get_residual_history(self._h, None, 0, C.byref(rows)))
        out = np.empty((rows.value, 3))
        if rows.value:
            self._ck(self._L.qlskum_get_residual_history(self._h, _dp(out), rows.value, C.byref(rows)))
        return out

    @property
    def iteration(self) -> int:
        it = C.c_int()
        self._ck(self._L.qlskum_get_iteration(self._h, C.byref(it)))
        return it.value

    @property
    def launches(self) -> int:
        return int(self._L.qlskum_launch_count(self._h))

    def launch_config(self) -> dict:
        v = [C.c_int() for _ in range(4)]
        self._ck(self._L.qlskum_get_launch_config(self._h, *[C.byref(t) for t in v]))
        ln = [C.c_int() for _ in range(2)]
        self._ck(self._L.qlskum_get_lanes(self._h, C.byref(ln[0]), C.byref(ln[1])))
        return {"flux_block": v[0].value, "flux_min_blocks": v[1].value, "point_block": v[2].value,
                "gather_depth": v[3].value, "flux_variant": int(self._L.qlskum_get_flux_variant(self._h)),
                "point_lanes": ln[0].value, "flux_lanes": ln[1].value}

    def set_launch_config(self, flux_variant=0, point_block=128, staged=0, point_lanes=1):
        """Pin the mixed form's launch shape (no autotuning)."""
        self._ck(self._L.qlskum_set_launch_config(self._h, int(flux_variant), int(point_block), int(staged)))
        if point_lanes != 1:
            self._ck(self._L.qlskum_set_point_lanes(self._h, int(point_lanes)))

    KERNELS = ("gradient", "inner", "flux_update", "reduce")

    def set_kernel_timing(self, enable: bool):
        self._ck(self._L.qlskum_set_kernel_timing(self._h, 1 if enable else 0))

    def kernel_timing(self) -> dict:
        """{kernel name: (total ms, launches)} recorded while kernel timing was on."""
        out = {}
        for k, name in enumerate(self.KERNELS):
            ms = C.c_double()
            n = C.c_longlong()
            self._ck(self._L.qlskum_get_kernel_timing(self._h, k, C.byref(ms), C.byref(n)))
            out[name] = (ms.value, n.value)
        return out

    @property
    def stream(self) -> int:
        return int(self._L.qlskum_stream(self._h) or 0)

    # ------------------------------------------------ diagnostics and state files
    def enstrophy(self):
        """(total enstrophy, vorticity [n]) of the current state (compute_enstrophy)."""
        t = C.c_double()
        v = np.empty(self.n)
        self._ck(self._L.qlskum_enstrophy(self._h, C.byref(t), _dp(v)))
        return t.value, v

    def stagnation(self):
        """(p0 min, p0 max, 1-based point of the min, of the max, J)."""
        d = [C.c_double() for _ in range(3)]
        ii = [C.c_int() for _ in range(2)]
        self._ck(self._L.qlskum_stagnation(self._h, C.byref(d[0]), C.byref(d[1]), C.byref(ii[0]), C.byref(ii[1]),
                                           C.byref(d[2])))
        return d[0].value, d[1].value, ii[0].value, ii[1].value, d[2].value

    def write_restart(self, path):
        self._ck(self._L.qlskum_write_restart(self._h, os.fsencode(path)))

    def read_restart(self, path):
        self._ck(self._L.qlskum_read_restart(self._h, os.fsencode(path)))

    def write_output(self, path):
        self._ck(self._L.qlskum_write_output(self._h, os.fsencode(path)))

    # ------------------------------------------------------- discrete adjoint
    def _state(self, a, name):
        a = np.ascontiguousarray(a, np.float64)
        if a.shape != (self.n, 4):
            raise ValueError(f"{name} must be [n, 4]")
        return a

    def residual(self, prim) -> np.ndarray:
        """Flux residual R(prim) of one stage, with the local time step of prim (FP64 handles)."""
        a = self._state(prim, "prim")
        out = np.empty((self.n, 4))
        self._ck(self._L.qlskum_residual_forward(self._h, _dp(a), _dp(out)))
        return out

    def residual_device(self, prim_ptr: int, out_ptr: int, stream: int = 0):
        """R(prim) on device buffers (double [n, 4], cloud order), ordered on `stream`."""
        self._ck(self._L.qlskum_residual_forward_device(self._h, prim_ptr, out_ptr, stream or None))

    def residual_vjp_device(self, prim_ptr: int, bar_ptr: int, out_ptr: int, stream: int = 0):
        """(dR/dprim)^T bar on device buffers (double [n, 4], cloud order), ordered on `stream`."""
        self._ck(self._L.qlskum_residual_vjp_device(self._h, prim_ptr, bar_ptr, out_ptr, stream or None))

    def residual_vjp(self, prim, bar_res, wall=False):
        """(dR/dprim)^T bar_res at prim; with wall=True also
        (bar_params [d/dMach, d/dAoA] (zero: R reads no free stream),
        bar_wall [shape_points] normal displacements) as a tuple."""
        a = self._state(prim, "prim")
        b = self._state(bar_res, "bar_res")
        out = np.empty((self.n, 4))
        if not wall:
            self._ck(self._L.qlskum_residual_vjp(self._h, _dp(a), _dp(b), _dp(out)))
            return out
        bp = np.empty(2)
        bw = np.empty(self.shape_points)
        self._ck(self._L.qlskum_residual_vjp_full(self._h, _dp(a), _dp(b), _dp(out), _dp(bp), _dp(bw)))
        return out, bp, bw

    def _adjoint_out(self, objective, wall):
        obj = {"cl": OBJECTIVE_CL, "cd": OBJECTIVE_CD, "j": OBJECTIVE_J}.get(objective, objective)
        vals = [C.c_double() for _ in range(4)]
        dw = np.zeros(self.shape_points) if wall else None
        return obj, vals, dw

    def adjoint_gradient(self, objective="cl", iters=100, wall=False, prim0=None, stride=1) -> dict:
        """Runs `iters` iterations from prim0 (held fixed) or the free stream and
        differentiates the objective ("cl" / "cd") at the end through all of
        them: {"J", "dmach", "daoa" (per degree), "dwall" ([shape_points]
        normal displacements) or None, "dprim0" ([n, 4]) or None}.  stride:
        keep every stride-th iteration's state and recompute the rest.  A
        mixed handle differentiates the mixed iteration (the wall gradient:
        the FP64 iteration at the mixed states)."""
        self._ck(self._L.qlskum_set_adjoint_stride(self._h, int(stride)))
        obj, v, dw = self._adjoint_out(objective, wall)
        p0 = None if prim0 is None else self._state(prim0, "prim0")
        dp0 = None if prim0 is None else np.empty((self.n, 4))
        self._ck(self._L.qlskum_adjoint_gradient(self._h, int(obj), int(iters), None if p0 is None else _dp(p0),
                                                 C.byref(v[0]), C.byref(v[1]), C.byref(v[2]),
                                                 _dp(dw) if wall else None, None if dp0 is None else _dp(dp0)))
        return {"J": v[0].value, "dmach": v[1].value, "daoa": v[2].value, "dwall": dw, "dprim0": dp0}

    def adjoint_fixed_point(self, objective="cl", adj_iters=500, wall=False) -> dict:
        """Steady-state adjoint at the current state; adds "adj_change", the
        relative change of the adjoint in its last iteration."""
        obj, v, dw = self._adjoint_out(objective, wall)
        self._ck(self._L.qlskum_adjoint_fixed_point(self._h, int(obj), int(adj_iters), C.byref(v[0]),
                                                    C.byref(v[1]), C.byref(v[2]), _dp(dw) if wall else None,
                                                    C.byref(v[3])))
        return {"J": v[0].value, "dmach": v[1].value, "daoa": v[2].value, "dwall": dw, "adj_change": v[3].value}


class Batch:
    """Many flight conditions over many clouds as one concatenated cloud,
    each kernel one launch over every case, graph-captured (mixed
    precision).  cases: list of (cloud index, mach, aoa)."""

    def __init__(self, clouds, cases, cfl=0.2, vl_const=50.0, power=0.0, inner_iterations=3, block_size=0):
        L = load()
        self._L = L
        structs, self._keep = [], []
        for c in clouds:
            s, keep = cloud_struct(c)
            structs.append(s)
            self._keep.append(keep)
        arr = (CloudStruct * len(structs))(*structs)
        self._arr = arr
        cc = np.ascontiguousarray([int(c[0]) for c in cases], np.int32)
        mm = np.ascontiguousarray([float(c[1]) for c in cases], np.float64)
        aa = np.ascontiguousarray([float(c[2]) for c in cases], np.float64)
        p = ParamsStruct(0.0, 0.0, cfl, vl_const, power, inner_iterations, MIXED, block_size, 1, 0)
        h = C.c_void_p()
        st = L.qlskum_batch_create(arr, len(structs), _ip(cc), _dp(mm), _dp(aa), len(cases), C.byref(p),
                                   C.byref(h))
        if st != 0:
            raise QlskumError(st, L.qlskum_batch_last_error(None).decode())
        self._h = h
        self.cases = list(cases)
        self.sizes = [clouds[int(c[0])].n for c in cases]

    def _ck(self, st):
        if st != 0:
            raise QlskumError(st, self._L.qlskum_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.qlskum_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, iters):
        self._ck(self._L.qlskum_batch_run(self._h, int(iters)))

    def objective(self):
        n = len(self.cases)
        out = [np.empty(n) for _ in range(4)]
        self._ck(self._L.qlskum_batch_objective(self._h, *[_dp(o) for o in out]))
        return out

    def prim(self, case):
        out = np.empty((self.sizes[case], 4))
        self._ck(self._L.qlskum_batch_get_prim(self._h, int(case), _dp(out)))
        return out

    def residual_history(self):
        rows = C.c_int()
        self._ck(self._L.qlskum_batch_residual_history(self._h, None, 0, C.byref(rows)))
        out = np.empty((rows.value, len(self.cases)))
        if rows.value:
            self._ck(self._L.qlskum_batch_residual_history(self._h, _dp(out), rows.value, C.byref(rows)))
        return out

    @property
    def total_points(self) -> int:
        return int(self._L.qlskum_batch_total_points(self._h))

    @property
    def launches(self) -> int:
        return int(self._L.qlskum_batch_launch_count(self._h))

    @property
    def stream(self) -> int:
        return int(self._L.qlskum_batch_stream(self._h) or 0)

    def tuning(self) -> dict:
        v = [C.c_int() for _ in range(4)]
        self._ck(self._L.qlskum_batch_tuning(self._h, *[C.byref(t) for t in v]))
        ln = [C.c_int() for _ in range(2)]
        self._ck(self._L.qlskum_batch_lanes(self._h, C.byref(ln[0]), C.byref(ln[1])))
        return {"tile": v[0].value, "flux_tile": v[1].value, "flux_min_blocks": v[2].value,
                "points_per_warp": v[3].value, "point_lanes": ln[0].value, "flux_lanes": ln[1].value}

    def set_launch_config(self, tile, point_lanes, flux_variant):
        """Pin the launch shape: threads per block (64, 128, 256) and lanes
        per point of the gradient / inner-loop kernels, and the flux variant
        (Solver.set_launch_config's numbering)."""
        self._ck(self._L.qlskum_batch_set_launch_config(self._h, int(tile), int(point_lanes), int(flux_variant)))


def partition_plan(cloud, n_parts):
    """The partition plan without a GPU: (part_of [n], per partition
    (local ids, ghost ids), 1-based global point numbers as pghost holds them)."""
    L = load()
    s, keep = cloud_struct(cloud)
    part_of = np.empty(cloud.n, np.int32)
    nl = np.empty(n_parts, np.int32)
    ng = np.empty(n_parts, np.int32)
    st = L.qlskum_partition_plan(C.byref(s), int(n_parts), _ip(part_of), _ip(nl), _ip(ng))
    if st != 0:
        raise QlskumError(st, L.qlskum_last_error(None).decode())
    lists = []
    for p in range(n_parts):
        loc = np.empty(max(1, nl[p]), np.int32)
        gh = np.empty(max(1, ng[p]), np.int32)
        st = L.qlskum_partition_plan_lists(C.byref(s), int(n_parts), p, _ip(loc), _ip(gh))
        if st != 0:
            raise QlskumError(st, L.qlskum_last_error(None).decode())
        lists.append((loc[:nl[p]].copy(), gh[:ng[p]].copy()))
    return part_of, lists


class Partition:
    """The solve split into n_parts partitions with ghost points refreshed
    from their owners before every kernel that reads them (the reference's
    local / ghost point layout), all on the current GPU."""

    def __init__(self, cloud, n_parts, mach=0.63, aoa=2.0, cfl=0.1, vl_const=150.0, power=0.0, inner_iterations=3,
                 precision=FP64, block_size=0):
        L = load()
        self._L = L
        s, self._keep = cloud_struct(cloud)
        p = ParamsStruct(mach, aoa, cfl, vl_const, power, inner_iterations, precision, block_size, 1, 0)
        h = C.c_void_p()
        st = L.qlskum_partition_create(C.byref(s), C.byref(p), int(n_parts), C.byref(h))
        if st != 0:
            raise QlskumError(st, L.qlskum_partition_last_error(None).decode())
        self._h = h
        self.n = cloud.n
        self.n_parts = n_parts

    def _ck(self, st):
        if st != 0:
            raise QlskumError(st, self._L.qlskum_partition_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.qlskum_partition_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def layout(self, part):
        """(local ids, ghost ids) of one partition, 1-based global point numbers."""
        nl, ng = C.c_int(), C.c_int()
        self._ck(self._L.qlskum_partition_layout(self._h, int(part), C.byref(nl), C.byref(ng), None, None))
        loc = np.empty(max(1, nl.value), np.int32)
        gh = np.empty(max(1, ng.value), np.int32)
        self._ck(self._L.qlskum_partition_layout(self._h, int(part), None, None, _ip(loc), _ip(gh)))
        return loc[:nl.value].copy(), gh[:ng.value].copy()

    def set_launch_config(self, flux_variant, point_block, staged):
        self._ck(self._L.qlskum_partition_set_launch_config(self._h, int(flux_variant), int(point_block),
                                                            int(staged)))

    def q_lskum(self, iters):
        self._ck(self._L.qlskum_partition_q_lskum(self._h, int(iters)))

    @property
    def prim(self):
        out = np.empty((self.n, 4))
        self._ck(self._L.qlskum_partition_get_prim(self._h, _dp(out)))
        return out

    def set_prim(self, prim):
        a = np.ascontiguousarray(prim, np.float64)
        self._ck(self._L.qlskum_partition_set_prim(self._h, _dp(a)))

    def residual_history(self):
        rows = C.c_int()
        self._ck(self._L.qlskum_partition_residual_history(self._h, None, 0, C.byref(rows)))
        out = np.empty((rows.value, 3))
        if rows.value:
            self._ck(self._L.qlskum_partition_residual_history(self._h, _dp(out), rows.value, C.byref(rows)))
        return out

    def objective(self):
        v = [C.c_double() for _ in range(4)]
        self._ck(self._L.qlskum_partition_objective(self._h, *[C.byref(t) for t in v]))
        return tuple(t.value for t in v)

    @property
    def halo_bytes(self) -> int:
        return int(self._L.qlskum_partition_halo_bytes(self._h))

    @property
    def launches(self) -> int:
        return int(self._L.qlskum_partition_launch_count(self._h))
