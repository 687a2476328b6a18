"""Build libmyqc.so (all CUDA sources, sm_103a) and the drop-in executables.

    python -m myqc_gb300.build        # or myqc_gb300.build.build()

Each translation unit compiles in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo``; objects go to
``myqc_gb300/_build/`` and the library to ``myqc_gb300/lib/libmyqc.so``.
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
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libmyqc.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                     "-I" + os.path.join(HERE, "..", "include")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src: str, extra) -> str:
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [nvcc()] + NVCC_FLAGS + list(extra) + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "myqc.h"))
    todo = [s for s in srcs
            if force or _stale(os.path.join(BUILD, s.replace(".cu", ".o")), [os.path.join(CSRC, s)] + headers)]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda s: _compile(s, extra), todo))
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in srcs]
    if force or todo or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    build_stages(force)
    if verbose:
        print(LIB)
    return LIB


STAGES = ("parse", "int1e", "int2e", "scf", "ao2mo", "mp2", "int1p", "cphf", "props")
BINDIR = os.path.join(HERE, "bin")
STAGE_BIN = os.path.join(BINDIR, "myqc-stage")


def build_stages(force: bool = False) -> str:
    """The drop-in stage executables: one C++ program on the C ABI, linked to
    lib/libmyqc.so (found through its run path), with a link per stage name."""
    src = os.path.join(HERE, "dropin", "stages.cpp")
    os.makedirs(BINDIR, exist_ok=True)
    if force or _stale(STAGE_BIN, [src, LIB, os.path.join(HERE, "..", "include", "myqc.h")]):
        cxx = shutil.which("g++") or shutil.which("c++")
        if not cxx:
            raise RuntimeError("no C++ compiler for the stage executables")
        cmd = [cxx, "-O2", "-std=c++17", "-o", STAGE_BIN, src, "-L" + LIBDIR, "-lmyqc", "-Wl,-rpath,$ORIGIN/../lib"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"stage executables failed to build:\n{r.stderr}")
    for st in STAGES:
        link = os.path.join(BINDIR, st)
        if os.path.lexists(link):
            os.remove(link)
        os.symlink("myqc-stage", link)
    return STAGE_BIN


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
