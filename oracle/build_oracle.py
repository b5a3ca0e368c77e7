"""Build recipe for the oracle (test infrastructure only).

Two artefacts:

* ``oracle/_build/libepic_oracle.so`` — the plain-C restatement of the
  reference's time-step loop (``oracle/epic_oracle.c``).  Built on every
  machine, with ``-ffp-contract=off`` so that GCC on aarch64 does not fuse
  multiply-adds the reference (built on x86 without FMA) does not fuse.
* ``oracle/_ref/libepic_ref.so`` — the reference's own ``src/*.cpp`` physics
  objects, compiled from where they lie under the reference checkout, plus
  ``oracle/ref_harness.cpp``.  Built only where the reference checkout exists.
  ``main.cpp`` and ``output.cpp`` need HDF5 and are replaced by the harness;
  ``output.h`` is satisfied by the H5Cpp stub in ``oracle/stub`` and by the
  system Python and NumPy headers (pulled in by ``matplotlibcpp.h``).
"""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# The reference checkout: EPIC_REFERENCE_DIR, else a "reference" directory
# beside this repository's root.
REFERENCE = os.environ.get("EPIC_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
REF_SOURCES = ["domain", "species", "field", "collision", "cross_section", "init",
               "grid", "electrode", "iniparser", "emitter"]

ORACLE_LIB = os.path.join(BUILD, "libepic_oracle.so")
REF_LIB = os.path.join(REF_OUT, "libepic_ref.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_restatement(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "epic_oracle.c")
    hdr = os.path.join(HERE, "epic_oracle.h")
    if force or _stale(ORACLE_LIB, [src, hdr]):
        tmp = ORACLE_LIB + ".tmp%d" % os.getpid()
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
              "-o", tmp, src, "-lm"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REFERENCE, "src", "species.cpp"))


def build_reference(force: bool = False) -> str | None:
    """Compile the reference's physics objects + harness into oracle/_ref."""
    if not reference_available():
        return REF_LIB if os.path.exists(REF_LIB) else None
    os.makedirs(REF_OUT, exist_ok=True)
    srcs = [os.path.join(REFERENCE, "src", s + ".cpp") for s in REF_SOURCES]
    harness = os.path.join(HERE, "ref_harness.cpp")
    if not force and not _stale(REF_LIB, srcs + [harness]):
        return REF_LIB
    py_inc = sysconfig.get_paths()["include"]
    import numpy
    flags = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-w",
             "-I", numpy.get_include(),
             "-I", os.path.join(HERE, "stub"),
             "-idirafter", os.path.join(REFERENCE, "include"),
             "-idirafter", os.path.join(REFERENCE, "linearalgebra"),
             "-I", py_inc]
    objs = []
    jobs = []
    for s in srcs + [harness]:
        o = os.path.join(REF_OUT, os.path.basename(s).replace(".cpp", ".o"))
        objs.append(o)
        jobs.append(flags + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    tmp = REF_LIB + ".tmp%d" % os.getpid()
    _run(["g++", "-shared", "-o", tmp] + objs + ["-lpthread"])
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build_restatement(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
