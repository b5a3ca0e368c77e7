"""epic_pcg_solve_static: the PCG solve for callers that may not allocate GPU
memory (all scratch lives in a static device array of the library).

Checked through the C ABI on the largest grid the static scratch allows
(257 x 257 nodes), on two calls in a row, each starting from a different
garbage phi: against the oracle's PCG (the same iteration count, phi within
1e-12 relative, as the other parity tests) and against the regular solver
(epic_potential_solver, same kernel and launch shape).  A second test runs
the entry point as the first call into the library in a fresh process, and a
third makes its grid barrier give up (a one-poll limit) and checks the
timeout status and a clean call after it.  This file is collected last so
that a failure here stops a run only after every other test has run.
"""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N = 256  # 257 x 257 nodes: the static scratch limit


def _fn(E):
    fn = E.lib().epic_pcg_solve_static
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                   ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                   ctypes.POINTER(ctypes.c_double)]
    fn.restype = ctypes.c_int
    return fn


def _case(tmp_path):
    ini = decks.write(decks.deck(nx=N, ny=N, ne=N * N * 4, ni=N * N * 4, solver="cg", tol="1e-10", maxit=100000),
                      str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    orc.scatter_all()
    s = orc.s
    K = (s.L * s.L) / (s.LDe * s.LDe)
    phi_o, err_o, it_o, conv_o = orc.R.pcg_solve(orc.rho)
    assert conv_o
    return ini, orc, K, phi_o, err_o, it_o


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _call(fn, rho_d, phi_d, s, K):
    it = ctypes.c_int()
    err = ctypes.c_double()
    st = fn(rho_d.data_ptr(), phi_d.data_ptr(), s.nx, s.ny, s.dx, K, s.tolerance, s.max_iteration, None,
            ctypes.byref(it), ctypes.byref(err))
    return st, it.value, err.value


def test_static_scratch_pcg_matches_oracle_and_regular_solver(gpu_lib, tmp_path):
    import torch

    E = gpu_lib
    ini, orc, K, phi_o, err_o, it_o = _case(tmp_path)
    sim = E.Simulation.from_ini(ini)
    sim.set_grid("rho", orc.rho)
    it_ref, err_ref, conv = sim.potential_solver()
    assert conv and it_ref == it_o, (it_ref, it_o)
    phi_ref = sim.grid("phi")
    fn = _fn(E)
    rho_d = torch.tensor(orc.rho, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        phi_d = torch.full_like(rho_d, float(call + 7))  # garbage the solve must overwrite
        torch.cuda.synchronize()
        st, it, err = _call(fn, rho_d, phi_d, orc.s, K)
        assert st == 0, E.lib().epic_last_error()
        assert it == it_o, "iteration count %d, oracle %d" % (it, it_o)
        phi = phi_d.cpu().numpy()
        assert _rel(phi, phi_o) <= 1e-12
        assert np.max(np.abs(phi - phi_ref)) <= 1e-12 * np.max(np.abs(phi_ref))
        assert abs(err - err_ref) <= 1e-9 * err_ref


def test_static_scratch_first_call_in_a_fresh_process(gpu_lib, tmp_path):
    """No other entry point of the library runs before this one in the child process."""
    ini, orc, K, phi_o, err_o, it_o = _case(tmp_path)
    np.save(str(tmp_path / "rho.npy"), orc.rho)
    s = orc.s
    child = textwrap.dedent("""
        import ctypes, sys
        import numpy as np
        import torch
        sys.path.insert(0, %r)
        from epic2d_mcc_gb300 import api
        rho = torch.tensor(np.load(%r), dtype=torch.float64, device="cuda")
        phi = torch.zeros_like(rho)
        torch.cuda.synchronize()
        L = ctypes.CDLL(api.LIB_PATH)
        fn = L.epic_pcg_solve_static
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                       ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                       ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
        fn.restype = ctypes.c_int
        it = ctypes.c_int()
        err = ctypes.c_double()
        st = fn(rho.data_ptr(), phi.data_ptr(), %d, %d, %r, %r, %r, %d, None, ctypes.byref(it), ctypes.byref(err))
        np.save(%r, phi.cpu().numpy())
        print("status", st, "iterations", it.value)
        sys.exit(st)
    """) % (ROOT, str(tmp_path / "rho.npy"), s.nx, s.ny, s.dx, K, s.tolerance, s.max_iteration,
            str(tmp_path / "phi.npy"))
    r = subprocess.run([sys.executable, "-c", child], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert ("iterations %d" % it_o) in r.stdout, r.stdout
    assert _rel(np.load(str(tmp_path / "phi.npy")), phi_o) <= 1e-12


def test_static_scratch_barrier_timeout_then_clean_call(gpu_lib, tmp_path):
    import torch

    E = gpu_lib
    ini, orc, K, phi_o, err_o, it_o = _case(tmp_path)
    fn = _fn(E)
    spin = E.lib().epic_set_spin_limit
    spin.argtypes = [ctypes.c_longlong]
    rho_d = torch.tensor(orc.rho, dtype=torch.float64, device="cuda")
    phi_d = torch.zeros_like(rho_d)
    torch.cuda.synchronize()
    try:
        spin(1)
        st, _, _ = _call(fn, rho_d, phi_d, orc.s, K)
        assert st == 7, E.lib().epic_last_error()  # EPIC_ERR_TIMEOUT
    finally:
        spin(0)
    st, it, _ = _call(fn, rho_d, phi_d, orc.s, K)
    assert st == 0, E.lib().epic_last_error()
    assert it == it_o
    assert _rel(phi_d.cpu().numpy(), phi_o) <= 1e-12


def test_static_scratch_rejects_grids_over_the_limit(gpu_lib):
    import torch

    fn = _fn(gpu_lib)
    big = torch.zeros(258 * 258, dtype=torch.float64, device="cuda")
    it = ctypes.c_int()
    err = ctypes.c_double()
    st = fn(big.data_ptr(), big.data_ptr(), 258, 258, 1.0, 1.0, 1e-10, 100, None, ctypes.byref(it),
            ctypes.byref(err))
    assert st == 4  # EPIC_ERR_CAPACITY
    assert b"257 x 257" in gpu_lib.lib().epic_last_error()
