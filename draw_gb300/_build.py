"""Builds the in-tree CUDA library for sm_103a: draw_gb300/_lib/libdrawgpu.so
(what the Python package and the tests load) and draw_gb300/_lib/libdrawgpu.a
(the same objects as a static archive, for a host program that links the
library statically, e.g. a Rust crate's build.rs). build(checked=True) makes
draw_gb300/_lib/libdrawgpu_checked.so instead: compiled with DRAW_CHECKED, its
kernels test the indices of their gathers and scatters against the buffers'
sizes and record DG_E_CUDA in the error word, skipping the access, where one is
out of range. build(timeline=True) makes draw_gb300/_lib/libdrawgpu_timeline.so:
compiled with DRAW_TIMELINE, its kernels record their block start, wait and end
times for dg_timeline_read (python -m draw_gb300.timeline prints them).

Floating-point flags are part of the contract with the reference's Rust
semantics: -fmad=false (no FMA contraction on the device), IEEE division and
square root, no flush-to-zero, and -ffp-contract=off for the host code (GCC
contracts by default on aarch64). The kernels also use explicit __f*_rn
intrinsics on every exact path.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libdrawgpu.so")
ARCHIVE = os.path.join(LIBDIR, "libdrawgpu.a")
CHECKED_LIB = os.path.join(LIBDIR, "libdrawgpu_checked.so")
TIMELINE_LIB = os.path.join(LIBDIR, "libdrawgpu_timeline.so")
SOURCES = ["dg_kernels.cu", "dg_api.cu", "dg_server.cu", "dg_noalloc.cu", "dg_batch.cu", "dg_transparent.cu",
           "dg_selfcheck.cu", "dg_loader.cpp"]
HEADERS = ["dg_internal.cuh", "dg_host.h", "dg_device.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "--expt-relaxed-constexpr",
]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the draw_gb300 CUDA library cannot be built")


def _stale(lib: str = LIB) -> bool:
    if not os.path.exists(lib) or (lib == LIB and not os.path.exists(ARCHIVE)):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, s) for s in SOURCES + HEADERS]
    deps.append(os.path.join(HERE, "..", "include", "draw_gpu.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra: list | None = None, checked: bool = False,
          timeline: bool = False) -> str:
    lib = CHECKED_LIB if checked else TIMELINE_LIB if timeline else LIB
    if not force and not _stale(lib):
        return lib
    os.makedirs(LIBDIR, exist_ok=True)
    tag = f"{os.getpid()}{'c' if checked else ''}{'t' if timeline else ''}"
    extra = list(extra or []) + (["-DDRAW_CHECKED"] if checked else []) + (["-DDRAW_TIMELINE"] if timeline else [])
    objs = []
    cmds = []
    for s in SOURCES:
        obj = os.path.join(LIBDIR, os.path.splitext(s)[0] + f".{tag}.o")
        objs.append(obj)
        cmds.append([nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, s), "-o", obj])
    with cf.ThreadPoolExecutor(len(cmds)) as ex:
        res = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), cmds))
    for c, r in zip(cmds, res):
        if verbose or r.returncode:
            sys.stderr.write(" ".join(c) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError(f"nvcc failed on {c[-3]}")
    tmp = lib + f".{tag}.tmp"
    link = [nvcc(), *ARCH, "-shared", *objs, "-o", tmp]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode:
        sys.stderr.write(" ".join(link) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("nvcc link failed")
    if lib == LIB:
        atmp = ARCHIVE + f".{tag}.tmp.a"
        r = subprocess.run(["ar", "rcs", atmp, *objs], capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("ar failed")
        os.replace(atmp, ARCHIVE)
    os.replace(tmp, lib)
    for o in objs:
        try:
            os.remove(o)
        except OSError:
            pass
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None, checked="--checked" in sys.argv,
                timeline="--timeline" in sys.argv))
