"""Build libzosimos_gb300.so in-tree with nvcc for sm_103a (no cmake, no torch).

Each kernel file (csrc/*.cu) is its own translation unit without relocatable device
code: the few device variables they share (the sRGB tables, the status word) are
per-file copies that csrc/zs_tables.cu fills and reads through per-file host hooks.
The host side (csrc/host/*.cpp) is plain C++17 compiled by nvcc's host compiler.
Objects are compiled in parallel and linked against the CUDA runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libzosimos_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build zosimos_gb300")


def _sources():
    cu = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    host = sorted(os.path.join(CSRC, "host", f) for f in os.listdir(os.path.join(CSRC, "host")) if f.endswith(".cpp"))
    return cu, host


def _deps():
    out = []
    for root, _, files in os.walk(CSRC):
        out += [os.path.join(root, f) for f in files if f.endswith((".cu", ".cuh", ".h", ".hpp", ".cpp"))]
    out.append(os.path.join(HERE, "..", "include", "zosimos.h"))
    return out


SYNTH_SRC = os.path.join(HERE, "synth", "zs_synth.c")
SYNTH_LIB = os.path.join(BUILD, "libzs_synth.so")


def build_synth() -> str:
    """The host-side generator of seeded synthetic inputs (bench and tests only)."""
    if os.path.exists(SYNTH_LIB) and os.path.getmtime(SYNTH_LIB) >= os.path.getmtime(SYNTH_SRC):
        return SYNTH_LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the synthetic-input generator")
    tmp = SYNTH_LIB + ".tmp"
    r = subprocess.run([cc, "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp, SYNTH_SRC, "-lm"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("synthetic generator build failed\n" + r.stdout + r.stderr)
    os.replace(tmp, SYNTH_LIB)
    return SYNTH_LIB


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    build_synth()
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    cu, host = _sources()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(HERE, "..", "include")]
    jobs = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        jobs.append([nvcc, *ARCH, *common, "-lineinfo", "-Xptxas", "-v" if verbose else "-O3", "-c", src, "-o", obj])
    for src in host:
        obj = os.path.join(BUILD, "host_" + os.path.basename(src) + ".o")
        jobs.append([nvcc, *common, "-x", "cu", *ARCH, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    # An object is rebuilt when it is missing or older than its source or any header.
    headers = [p for p in _deps() if not p.endswith((".cu", ".cpp"))]
    newest_header = max(os.path.getmtime(p) for p in headers)

    def stale(cmd):
        src, obj = cmd[-3], cmd[-1]
        if force or verbose or not os.path.exists(obj):
            return True
        t = os.path.getmtime(obj)
        return os.path.getmtime(src) > t or newest_header > t

    todo = [c for c in jobs if stale(c)]
    # The slowest object (k_raster.cu) goes first so that it overlaps the rest.
    todo.sort(key=lambda c: not c[-3].endswith("k_raster.cu"))
    logs = []
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), max(4, os.cpu_count() or 4))) as ex:
            logs = list(ex.map(run, todo))
    if verbose:
        for log in logs:
            sys.stdout.write(log)
    objs = [c[-1] for c in jobs]
    tmp = LIB + ".tmp"
    run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
