"""ctypes front end of the C restatement oracle (oracle/qlskum_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
benchmark's CPU-baseline leg, always as the checker or the timed CPU
baseline, never as part of the product path.

`build()` compiles the C file into oracle/_build/libqlskum_oracle.so with
-ffp-contract=off (no FMA contraction on either x86-64 or aarch64) and
OpenMP; `build_reference()` runs oracle/build_ref.sh, which compiles the
reference's own sources into oracle/_ref/ when they are present.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libqlskum_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")

FLUX_KINDS = ("Gxp", "Gxn", "Gyp", "Gyn", "GxI", "GxII", "GxIII", "GxIV")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "qlskum_oracle.c")
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "qlskum_oracle.h"))):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off",
                               "-fopenmp", src, "-o", tmp, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def build_reference() -> str | None:
    """Compile the reference via oracle/build_ref.sh; None when its sources are absent."""
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])
    return REF_BIN if os.path.exists(REF_BIN) else None


def reference_dir() -> str | None:
    """The reference source directory oracle/build_ref.sh last built from, or None."""
    p = os.path.join(os.path.dirname(REF_BIN), "source_dir")
    if not (os.path.exists(REF_BIN) and os.path.exists(p)):
        return None
    d = open(p).read().strip()
    return d if os.path.isdir(d) else None


class _Cloud(C.Structure):
    _fields_ = [("n", C.c_int),
                ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)),
                ("left", C.POINTER(C.c_int)), ("right", C.POINTER(C.c_int)),
                ("flag_1", C.POINTER(C.c_int)), ("flag_2", C.POINTER(C.c_int)),
                ("min_dist", C.POINTER(C.c_double)),
                ("nbhs", C.POINTER(C.c_int)), ("conn", C.POINTER(C.c_int))]


class _Params(C.Structure):
    _fields_ = [("mach", C.c_double), ("aoa", C.c_double), ("cfl", C.c_double),
                ("vl_const", C.c_double), ("power", C.c_double),
                ("inner_iterations", C.c_int), ("threads", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        P = C.c_void_p
        L.qo_create.restype = P
        L.qo_create.argtypes = [C.POINTER(_Cloud), C.POINTER(_Params)]
        L.qo_destroy.argtypes = [P]
        for name in ("qo_func_delta", "qo_eval_q_variables", "qo_eval_q_derivatives",
                     "qo_eval_q_inner_loop", "qo_eval_update_innerloop", "qo_cal_flux_residual"):
            getattr(L, name).argtypes = [P]
        L.qo_state_update.argtypes = [P, C.c_int]
        L.qo_fpi_solver.restype = C.c_double
        L.qo_fpi_solver.argtypes = [P, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        dp = C.POINTER(C.c_double)
        L.qo_objective.argtypes = [P, dp, dp, dp, dp]
        L.qo_enstrophy.restype = C.c_double
        L.qo_enstrophy.argtypes = [P, dp]
        ip = C.POINTER(C.c_int)
        L.qo_stagnation.argtypes = [P, dp, dp, ip, ip, dp]
        for name in ("qo_prim", "qo_prim_old", "qo_q", "qo_dq", "qo_qm", "qo_flux_res", "qo_delta",
                     "qo_normals", "qo_entropy"):
            getattr(L, name).restype = dp
            getattr(L, name).argtypes = [P]
        L.qo_sub_counts.restype = C.POINTER(C.c_int)
        L.qo_sub_counts.argtypes = [P]
        L.qo_sub_lists.restype = C.POINTER(C.c_int)
        L.qo_sub_lists.argtypes = [P]
        L.qo_sum_res_sqr.restype = C.c_double
        L.qo_sum_res_sqr.argtypes = [P]
        L.qo_flux.argtypes = [C.c_int] + [C.c_double] * 6 + [dp]
        L.qo_qtilde_to_primitive.argtypes = [dp, dp, dp, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class Oracle:
    """The reference solver restated in C, driven function by function.

    Arrays returned by the accessors are copies, point-major and 0-based:
    prim/q/flux_res [n, 4]; dq/qm [n, 2, 4] (dq[:, 0] = d/dx, qm[:, 0] = max).
    """

    def __init__(self, cloud, mach=0.63, aoa=2.0, cfl=0.2, vl_const=50.0, power=0.0,
                 inner_iterations=0, threads=1):
        self._keep = dict(
            x=np.ascontiguousarray(cloud.x, np.float64), y=np.ascontiguousarray(cloud.y, np.float64),
            left=np.ascontiguousarray(cloud.left, np.int32), right=np.ascontiguousarray(cloud.right, np.int32),
            f1=np.ascontiguousarray(cloud.flag_1, np.int32), f2=np.ascontiguousarray(cloud.flag_2, np.int32),
            md=np.ascontiguousarray(cloud.min_dist, np.float64), nb=np.ascontiguousarray(cloud.nbhs, np.int32),
            conn=np.ascontiguousarray(cloud.conn, np.int32))
        k = self._keep
        assert k["conn"].shape == (cloud.n, 20)
        c = _Cloud(cloud.n, _dp(k["x"]), _dp(k["y"]), _ip(k["left"]), _ip(k["right"]), _ip(k["f1"]),
                   _ip(k["f2"]), _dp(k["md"]), _ip(k["nb"]), _ip(k["conn"]))
        p = _Params(mach, aoa, cfl, vl_const, power, inner_iterations, threads)
        self.n = cloud.n
        self.inner_iterations = inner_iterations
        self._h = lib().qo_create(C.byref(c), C.byref(p))
        self.it = 0

    def close(self):
        if self._h:
            lib().qo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _arr(self, fn, shape):
        ptr = getattr(lib(), fn)(self._h)
        return np.ctypeslib.as_array(ptr, shape=shape).copy()

    # module entry points
    def func_delta(self): lib().qo_func_delta(self._h)
    def eval_q_variables(self): lib().qo_eval_q_variables(self._h)
    def eval_q_derivatives(self): lib().qo_eval_q_derivatives(self._h)
    def eval_q_inner_loop(self): lib().qo_eval_q_inner_loop(self._h)
    def eval_update_innerloop(self): lib().qo_eval_update_innerloop(self._h)
    def cal_flux_residual(self): lib().qo_cal_flux_residual(self._h)
    def state_update(self, rk): lib().qo_state_update(self._h, rk)

    def snapshot_prim_old(self):
        """prim_old <- prim (fpi_solver_mod.h:19-25)."""
        self.set_prim_old(self.prim)

    def set_prim(self, prim):
        dst = np.ctypeslib.as_array(lib().qo_prim(self._h), shape=(self.n, 4))
        dst[:] = prim

    def set_prim_old(self, prim):
        dst = np.ctypeslib.as_array(lib().qo_prim_old(self._h), shape=(self.n, 4))
        dst[:] = prim

    def fpi_solver(self):
        """One iteration; returns (res_new, residue, max_res)."""
        self.it += 1
        r = C.c_double()
        m = C.c_double()
        res = lib().qo_fpi_solver(self._h, self.it, C.byref(r), C.byref(m))
        return res, r.value, m.value

    def run(self, iters):
        return np.array([self.fpi_solver() for _ in range(iters)])

    def objective(self):
        v = [C.c_double() for _ in range(4)]
        lib().qo_objective(self._h, *[C.byref(t) for t in v])
        return tuple(t.value for t in v)

    def enstrophy(self):
        """(total enstrophy, vorticity [n]) of the current state."""
        v = np.zeros(self.n)
        t = lib().qo_enstrophy(self._h, v.ctypes.data_as(C.POINTER(C.c_double)))
        return t, v

    def stagnation(self):
        """(p0 min, p0 max, 1-based point of the min, of the max, J)."""
        d = [C.c_double() for _ in range(3)]
        ii = [C.c_int() for _ in range(2)]
        lib().qo_stagnation(self._h, C.byref(d[0]), C.byref(d[1]), C.byref(ii[0]), C.byref(ii[1]), C.byref(d[2]))
        return d[0].value, d[1].value, ii[0].value, ii[1].value, d[2].value

    @property
    def prim(self): return self._arr("qo_prim", (self.n, 4))
    @property
    def q(self): return self._arr("qo_q", (self.n, 4))
    @property
    def dq(self): return self._arr("qo_dq", (self.n, 2, 4))
    @property
    def qm(self): return self._arr("qo_qm", (self.n, 2, 4))
    @property
    def flux_res(self): return self._arr("qo_flux_res", (self.n, 4))
    @property
    def delta(self): return self._arr("qo_delta", (self.n,))
    @property
    def normals(self): return self._arr("qo_normals", (self.n, 2))
    @property
    def sum_res_sqr(self): return lib().qo_sum_res_sqr(self._h)

    def sub_counts(self):
        return np.ctypeslib.as_array(lib().qo_sub_counts(self._h), shape=(self.n, 4)).copy()

    def sub_lists(self):
        return np.ctypeslib.as_array(lib().qo_sub_lists(self._h), shape=(self.n, 4, 20)).copy()


def flux(kind: int, nx, ny, u1, u2, rho, pr) -> np.ndarray:
    g = np.zeros(4)
    lib().qo_flux(int(kind), float(nx), float(ny), float(u1), float(u2), float(rho), float(pr), _dp(g))
    return g


def qtilde_to_primitive(qt) -> tuple:
    q = np.ascontiguousarray(qt, np.float64)
    v = [C.c_double() for _ in range(4)]
    lib().qo_qtilde_to_primitive(_dp(q), *[C.byref(t) for t in v])
    return tuple(t.value for t in v)
