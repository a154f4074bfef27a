"""Build recipe of the in-tree CUDA library (libqlskum.so) for sm_103a.

Six translation units compiled in parallel and linked into one shared
library with a C ABI (include/qlskum.h):

* csrc/qlskum_fp64.cu  -- FP64 drop-in kernels, FMA contraction on (one
  FP64 instruction per multiply-add; 1e-10 parity with the reference);
* csrc/qlskum_mixed.cu -- mixed-precision kernels (FP32 edge work, FMA and
  FP32 flush-to-zero on);
* csrc/qlskum_adjoint.cu -- reverse-mode kernels of the FP64 and the mixed
  iterations (FP32 flush-to-zero on, as in the mixed forward);
* csrc/qlskum_noalloc.cu -- the stage update over caller buffers that
  allocates nothing (static device scratch), -fmad=false (the reference's
  rounding sequence of the update);
* csrc/qlskum_host.cpp -- host layer, g++ -ffp-contract=off (bit-exact
  sub-stencil classification on x86-64 and aarch64 alike);
* csrc/qlskum_io.cpp -- partGrid file I/O and the sub-stencil quality check
  (host only, no GPU needed).

`build_vjp_host()` compiles a separate, test-only library
(tests/vjp_host/qlskum_vjp_host.cpp -> tests/_build/libqlskum_vjp_host.so):
the per-point arithmetic and its reverse mode compiled for the host, for
derivative checks without a GPU.  It is not part of libqlskum.so.

Output: c-_serial_gb300/_build/libqlskum.so (git-ignored; rebuilt on the GPU
machine because binaries do not travel between architectures).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                       # c-_serial_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(BUILD, "libqlskum.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the q-LSKUM library needs the CUDA toolkit to build")


def _cuda_include(nvcc: str) -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


def sources():
    return {
        "qlskum_fp64.cu": ["-fmad=true"],
        "qlskum_mixed.cu": ["-fmad=true", "-ftz=true"],
        "qlskum_noalloc.cu": ["-fmad=false"],
        "qlskum_adjoint.cu": ["-ftz=true"],
        "qlskum_host.cpp": [],
        "qlskum_io.cpp": [],
    }


def _deps():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    out += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    out.append(os.path.abspath(__file__))
    return out


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps())


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile and link libqlskum.so if it is missing or stale; return its path."""
    if not force and not needs_build():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I", INCLUDE, "-I", CSRC]
    procs = []
    objs = []
    for src, extra in sources().items():
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if src.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *extra, *inc,
                   "-c", path, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                   *inc, "-I", _cuda_include(nvcc), "-c", path, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append(f"{src}: {' '.join(cmd)}\n{out}")
        elif out.strip() and (verbose or ptxas_info):
            print(out, file=sys.stderr)
    if failed:
        raise RuntimeError("building libqlskum failed:\n" + "\n".join(failed))
    tmp = LIB + f".tmp{os.getpid()}"
    link = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("linking libqlskum failed:\n" + " ".join(link) + "\n" + r.stdout)
    os.replace(tmp, LIB)
    return LIB


VJP_SRC = os.path.join(REPO, "tests", "vjp_host", "qlskum_vjp_host.cpp")
VJP_LIB = os.path.join(REPO, "tests", "_build", "libqlskum_vjp_host.so")


def build_vjp_host() -> str:
    """Compile the test-only host build of the per-point reverse arithmetic
    (g++, no GPU needed) if missing or stale; return its path."""
    deps = [VJP_SRC] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    if os.path.exists(VJP_LIB) and all(os.path.getmtime(p) <= os.path.getmtime(VJP_LIB) for p in deps):
        return VJP_LIB
    os.makedirs(os.path.dirname(VJP_LIB), exist_ok=True)
    tmp = VJP_LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
           "-I", INCLUDE, "-I", CSRC, "-I", _cuda_include(_nvcc()), VJP_SRC, "-o", tmp]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the host VJP test library failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    os.replace(tmp, VJP_LIB)
    return VJP_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
