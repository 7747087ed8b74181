"""Build recipe of the CUDA library libadpres_gb300.so (sm_103a only).

The translation units are compiled in parallel with nvcc and linked into a
shared library inside the package directory, so the library that runs is
the in-tree one.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libadpres_gb300.so")
SOURCES = ["batch_k32.cu", "batch_k64.cu", "cmfd.cu", "nodal.cu", "capi.cu", "noalloc.cu", "adjoint.cu", "batch.cu", "edits.cu", "reactivity.cu", "transfer.cu", "trans.cu", "nodal_adj.cu"]
HEADERS = ["adp_device.cuh", "ff.cuh", "adp_kernels.h", "outer_body.cuh", "nodal_body.cuh", "cmfd_items.cuh", "host_geom.h", "handle.h", "batch_kernel.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build adpres_gb300")
    return exe


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


# Variants for tests and measurements: "nofmad" compiles with -fmad=false
# (no contraction of a separate multiply and add into an FMA by the
# compiler; the kernels' explicit fma() calls stay); "bounds" compiles the
# range checks of device indices (ADP_BOUNDS: a bad index is reported as
# ADP_ERR_BOUNDS and its item skipped, nothing traps).  A variant builds
# under _build/<variant>/ and is loaded by setting ADPRES_LIB to its library.
VARIANTS = {"default": [], "nofmad": ["-fmad=false"], "bounds": ["-DADP_BOUNDS"]}


def build(force: bool = False, verbose: bool = False, variant: str = "default") -> str:
    extra = VARIANTS[variant]
    build_dir = BUILD if variant == "default" else os.path.join(BUILD, variant)
    lib = LIB if variant == "default" else os.path.join(build_dir, "libadpres_gb300.so")
    os.makedirs(build_dir, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "adpres_gb300.h")]
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(build_dir, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [nvcc()] + ARCH + FLAGS + extra + ["-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(" ".join(cmd))
        return r

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(lib, objs):
        tmp = lib + ".tmp.%d" % os.getpid()
        run([nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs)
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    import sys
    print(build(verbose=True, variant=sys.argv[1] if len(sys.argv) > 1 else "default"))
