"""Builds the engine's shared libraries in-tree for sm_103a.

    python -m komd_gb300.build          # or __graft_entry__.build()

* komd_gb300/_build/libkomd_gpu.so  -- CUDA engine behind include/komd_gpu.h
* komd_gb300/_build/libkomd_host.so and komd_gb300/_build/komd -- the C++
  host layer (Registry / plugin interfaces, input parser, checkpoint IO)
  linked against the engine

Translation units are compiled in parallel with one -gencode (sm_103a).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(CSRC, "host")
OUT = os.path.join(HERE, "_build")
INC = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I" + INC, "-I" + CSRC]
GPU_SOURCES = ["kernels.cu", "pair_tile.cu", "surrogate.cu", "sur_train.cu", "capi.cu", "noalloc.cu"]

LIB_GPU = os.path.join(OUT, "libkomd_gpu.so")
LIB_HOST = os.path.join(OUT, "libkomd_host.so")
EXE = os.path.join(OUT, "komd")


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build komd_gb300")


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _deps_common():
    out = [os.path.join(INC, "komd_gpu.h")]
    for f in os.listdir(CSRC):
        if f.endswith((".cuh", ".h")):
            out.append(os.path.join(CSRC, f))
    return out


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    common = _deps_common()
    jobs = []
    objs = []
    for src in GPU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + common):
            jobs.append([cc] + NVCC_FLAGS + ARCH + ["-c", s, "-o", o])
    host_srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp")) if os.path.isdir(HOST) else []
    host_objs = []
    for s in host_srcs:
        o = os.path.join(OUT, "host_" + os.path.basename(s).replace(".cpp", ".o"))
        host_objs.append(o)
        if force or _stale(o, [s] + common + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I" + INC, "-I" + HOST,
                         "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, len(jobs)))) as ex:
        for res in ex.map(_run, jobs):
            if verbose and (res.stdout or res.stderr):
                print(res.stdout + res.stderr)
    if force or _stale(LIB_GPU, objs):
        _run([cc, "-shared", "-o", LIB_GPU] + objs + ARCH + ["-cudart", "static"])
    main_obj = [o for o in host_objs if o.endswith("host_main.o")]
    lib_objs = [o for o in host_objs if not o.endswith("host_main.o")]
    if lib_objs and (force or _stale(LIB_HOST, lib_objs + [LIB_GPU])):
        _run(["g++", "-shared", "-o", LIB_HOST] + lib_objs + ["-L" + OUT, "-lkomd_gpu", "-Wl,-rpath,$ORIGIN"])
    if main_obj and (force or _stale(EXE, main_obj + [LIB_HOST])):
        _run(["g++", "-o", EXE] + main_obj + ["-L" + OUT, "-lkomd_host", "-lkomd_gpu", "-Wl,-rpath,$ORIGIN"])
    return LIB_GPU


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print("built", LIB_GPU)
