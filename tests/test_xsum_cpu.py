"""The exact fixed-point summation the PCG kernel reduces its dot products
with (epic2d_mcc_gb300/csrc/epic_xsum.cuh), compiled for the host with g++
and checked against math.fsum (a correctly rounded sum): one anchored block
of terms, blocks re-anchored to a common exponent as the grid total does, the
exact order independence that makes the solver deterministic, and the stop
threshold that replaces sqrt(r.r) < tol by an integer compare."""
import ctypes
import math
import os
import random
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "epic2d_mcc_gb300", "csrc", "epic_xsum.cuh")

HARNESS = r"""
#include "epic_xsum.cuh"
using namespace epic;
extern "C" {
// sum of x[0..n) split into blocks of bs terms, each anchored on its own
// largest exponent, then re-anchored to the largest block anchor and added
double xs_sum_blocks(const double* x, int n, int bs) {
  int nb = (n + bs - 1) / bs;
  xs_int V[4096]; int A[4096];
  int Ag = 0;
  for (int b = 0; b < nb; b++) {
    int a = 0;
    for (int k = b * bs; k < n && k < (b + 1) * bs; k++) a = a > xs_exponent(x[k]) ? a : xs_exponent(x[k]);
    xs_int v = 0;
    for (int k = b * bs; k < n && k < (b + 1) * bs; k++) v += xs_from_double(x[k], a);
    V[b] = v; A[b] = a; Ag = Ag > a ? Ag : a;
  }
  xs_int s = 0;
  for (int b = 0; b < nb; b++) s += xs_realign(V[b], A[b], Ag);
  return xs_to_double(s, Ag);
}
double xs_threshold(double tol) { return xs_sqrt_threshold(tol); }
}
"""


@pytest.fixture(scope="module")
def X(tmp_path_factory):
    d = tmp_path_factory.mktemp("xsum")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    so = d / "libxsum.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-I", os.path.dirname(HEADER), str(src), "-o", str(so)], check=True)
    L = ctypes.CDLL(str(so))
    L.xs_sum_blocks.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    L.xs_sum_blocks.restype = ctypes.c_double
    L.xs_threshold.argtypes = [ctypes.c_double]
    L.xs_threshold.restype = ctypes.c_double
    return L


def xsum(L, x, bs):
    x = np.ascontiguousarray(x, dtype=np.float64)
    return L.xs_sum_blocks(x.ctypes.data, len(x), bs)


def test_dot_product_terms_sum_correctly_rounded(X):
    rng = np.random.default_rng(0)
    for trial in range(200):
        n = int(rng.integers(1, 3000))
        a = rng.standard_normal(n) * 10.0 ** rng.uniform(-20, 5)
        b = rng.standard_normal(n) * 10.0 ** rng.uniform(-20, 5)
        terms = a * b if trial % 2 else a * a
        for bs in (1, 7, 256, 2048):
            assert xsum(X, terms, bs) == math.fsum(terms), (trial, bs)


def test_wide_exponent_ranges_and_signs(X):
    rng = random.Random(1)
    for trial in range(300):
        n = rng.randint(1, 500)
        e0 = rng.randint(-300, 300)
        terms = [rng.choice([-1, 1]) * rng.random() * 2.0 ** (e0 + rng.randint(-50, 0)) for _ in range(n)]
        got = xsum(X, terms, 64)
        assert got == math.fsum(terms), trial


def test_order_independent(X):
    rng = np.random.default_rng(2)
    terms = rng.standard_normal(4000) * np.exp(rng.uniform(-30, 30, 4000))
    ref = xsum(X, terms, 256)
    for _ in range(5):
        perm = rng.permutation(len(terms))
        assert xsum(X, terms[perm], 256) == ref
        assert xsum(X, terms[perm], 160) == ref


def test_edge_values(X):
    assert xsum(X, [0.0], 1) == 0.0
    assert xsum(X, [0.0, -0.0], 2) == 0.0
    assert xsum(X, [1.0, -1.0], 2) == 0.0
    sub = struct.unpack("<d", struct.pack("<Q", 1))[0]  # smallest subnormal
    # exact cancellation within the 2^54 window below the largest term ...
    assert xsum(X, [2.0 ** 50, 1.0, -(2.0 ** 50)], 3) == 1.0
    # ... and the documented truncation of terms further below it
    assert xsum(X, [2.0 ** 1000, 1.0, -(2.0 ** 1000)], 3) == 0.0
    assert xsum(X, [1e300, 1e300], 1) == 2e300
    assert xsum(X, [sub] * 4, 4) == 0.0  # below the normal range: flushed
    assert xsum(X, [2.0 ** -1000, 2.0 ** -1000], 2) == 2.0 ** -999


def test_sqrt_stop_threshold(X):
    rng = random.Random(3)
    for tol in [1e-10, 1e-8, 1.0, 3.0, 1e-300, 1e150] + [10 ** rng.uniform(-150, 150) for _ in range(200)]:
        T = X.xs_threshold(tol)
        assert math.sqrt(T) >= tol
        below = math.nextafter(T, 0.0)
        assert math.sqrt(below) < tol
    assert X.xs_threshold(0.0) == 0.0

