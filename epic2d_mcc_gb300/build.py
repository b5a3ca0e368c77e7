"""Builds the in-tree CUDA library ``epic2d_mcc_gb300/libepic2d_gb300.so``.

sm_103a only: every .cu file is compiled with one ``-gencode
arch=compute_103a,code=sm_103a``; host C++ with ``-ffp-contract=off`` so the
start-up arithmetic rounds the same on x86 and aarch64.  The FP64 kernels are
compiled with ``-fmad=false`` (no contracted multiply-adds), which is what lets
them reproduce the reference's arithmetic bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libepic2d_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

CU_FP64 = ["epic_particles.cu", "epic_field.cu", "epic_mcc.cu", "epic_capi.cu", "epic_noalloc.cu", "epic_sort.cu", "epic_load.cu",
           "epic_batch_grid.cu"]
CU_FAST = ["epic_mixed.cu", "epic_spectral.cu", "epic_batch.cu"]
CPP = ["epic_host.cpp", "epic_server.cpp"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout[-4000:], r.stderr[-8000:]))
    return r.stdout + r.stderr


def sources():
    out = []
    for f in CU_FP64 + CU_FAST + CPP:
        p = os.path.join(CSRC, f)
        if os.path.exists(p):
            out.append(p)
    return out


def _deps():
    d = sources()
    for f in os.listdir(CSRC):
        if f.endswith((".cuh", ".h")):
            d.append(os.path.join(CSRC, f))
    d.append(os.path.join(INCLUDE, "epic2d.h"))
    d.append(os.path.join(INCLUDE, "epic2d_serve.h"))
    d.append(os.path.join(INCLUDE, "epic2d_batch.h"))
    return d


def is_stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not is_stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for f in CU_FP64 + CU_FAST:
        src = os.path.join(CSRC, f)
        if not os.path.exists(src):
            continue
        obj = os.path.join(OUT, f.replace(".cu", ".o"))
        fmad = ["-fmad=false"] if f in CU_FP64 else []
        jobs.append([nvcc] + GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                        "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v",
                                        "-I", INCLUDE, "-c", src, "-o", obj] + fmad)
        objs.append(obj)
    for f in CPP:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f.replace(".cpp", ".o"))
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE,
                     "-I", "/usr/local/cuda/include", "-c", src, "-o", obj])
        objs.append(obj)
    with ThreadPoolExecutor(max_workers=max(2, min(len(jobs), os.cpu_count() or 4))) as ex:
        logs = list(ex.map(_run, jobs))
    tmp = LIB + ".tmp%d" % os.getpid()
    _run([nvcc] + GENCODE + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"])
    os.replace(tmp, LIB)
    with open(os.path.join(OUT, "ptxas.log"), "w") as f:
        f.write("\n".join(logs))
    if verbose:
        print("\n".join(logs))
    build_driver()
    return LIB


DRIVER = os.path.join(HERE, "epic2d")


def build_driver() -> str:
    """The `epic2d` command-line driver (host/main.cpp) over the C++ mirror of
    the reference classes (host/epic2d.hpp), linked to the library."""
    src = os.path.join(HERE, "host", "main.cpp")
    hdrs = [os.path.join(HERE, "host", h) for h in ("epic2d.hpp", "epic2d_output.hpp")]
    if os.path.exists(DRIVER) and all(os.path.getmtime(DRIVER) >= os.path.getmtime(p) for p in [src, LIB] + hdrs):
        return DRIVER
    tmp = DRIVER + ".tmp%d" % os.getpid()
    _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, "-o", tmp, src, LIB, "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
