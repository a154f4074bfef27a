"""The C ABI library: builds for sm_103a, loads, exports every symbol
include/qlskum.h declares, and rejects malformed clouds on the host before any
device work (these checks need no GPU)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import REPO, has_gpu, small_cloud

HEADER = os.path.join(REPO, "include", "qlskum.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qlskum_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import qlskum
    return qlskum.load()


def test_library_exports_every_declared_symbol(lib):
    import qlskum
    names = declared_functions()
    assert len(names) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", qlskum.library_path()], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (qlskum_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        getattr(lib, n)


def test_library_is_built_for_sm103a(lib):
    """The build recipe compiles every CUDA unit for sm_103a only (one
    -gencode, no PTX for other targets)."""
    from qlskum import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert all(f.endswith((".cu", ".cpp")) for f in build.sources())


def test_default_params(lib):
    import qlskum
    p = qlskum.ParamsStruct()
    lib.qlskum_default_params(C.byref(p))
    # the reference's globals: parameter_mod.h:4-5, data_structure_mod.h:72,90,96,118
    assert (p.mach, p.aoa, p.cfl, p.vl_const, p.power, p.inner_iterations) == (0.63, 2.0, 0.1, 150.0, 0.0, 3)
    assert p.precision == qlskum.FP64 and p.reorder == 1
    assert lib.qlskum_abi_version() == 1


def _create(lib, cloud, **kw):
    import qlskum
    s, keep = qlskum.cloud_struct(cloud)
    p = qlskum.ParamsStruct()
    lib.qlskum_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    h = C.c_void_p()
    st = lib.qlskum_create(C.byref(s), C.byref(p), C.byref(h))
    msg = lib.qlskum_last_error(None).decode()
    if st == 0:
        lib.qlskum_destroy(h)
    return st, msg


def _copy(c):
    from qlskum.cloudgen import Cloud
    return Cloud(*(np.array(getattr(c, f)) for f in ("x", "y", "left", "right", "flag_1", "flag_2", "min_dist",
                                                        "nbhs", "conn")))


def test_rejects_malformed_clouds(lib):
    base = small_cloud()
    bad = _copy(base)
    bad.nbhs[5] = 21
    assert _create(lib, bad)[0] == 1
    bad = _copy(base)
    bad.conn[7, 0] = base.n + 1
    st, msg = _create(lib, bad)
    assert st == 1 and "out of range" in msg
    bad = _copy(base)
    bad.flag_1[3] = 3
    assert _create(lib, bad)[0] == 1
    bad = _copy(base)
    bad.x[9] = np.nan
    assert _create(lib, bad)[0] == 1
    bad = _copy(base)
    bad.left[0] = 0
    assert _create(lib, bad)[0] == 1
    assert _create(lib, base, inner_iterations=-1)[0] == 1
    assert _create(lib, base, precision=7)[0] == 1
    assert _create(lib, base, block_size=100)[0] == 1


def test_rejects_degenerate_stencil(lib):
    """A point whose neighbours are collinear has a singular LSQ matrix
    (the reference would divide by det = 0)."""
    bad = _copy(small_cloud())
    i = 200  # an interior point
    assert bad.flag_1[i] == 1
    j = bad.conn[i, 0] - 1
    bad.nbhs[i] = 1
    st, msg = _create(lib, bad)
    assert st == 2, msg
    assert f"point {i + 1}" in msg
    _ = j


@pytest.mark.skipif(has_gpu(), reason="checks the error path of a machine without a GPU")
def test_valid_cloud_without_gpu_reports_cuda_error(lib):
    st, msg = _create(lib, small_cloud())
    assert st == 4 and msg
