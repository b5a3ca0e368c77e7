"""epic_pcg_solve_static: the PCG solve for callers that may not allocate GPU
memory (all scratch lives in a static device array of the library).

Checked through the C ABI against the regular solver (epic_potential_solver,
same kernel and launch shape) on the largest grid the static scratch allows,
on two calls in a row, each starting from a different garbage phi: same
iteration count and phi within 1e-12 relative, as the other parity tests.
This file is collected last so that a failure here stops a run only after
every other test has run.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu


def _fn(E):
    fn = E.lib().epic_pcg_solve_static
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                   ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                   ctypes.POINTER(ctypes.c_double)]
    fn.restype = ctypes.c_int
    return fn


def test_static_scratch_pcg_matches_regular_solver(gpu_lib, tmp_path):
    import torch

    E = gpu_lib
    n = 256  # 257 x 257 nodes: the static scratch limit
    ini = decks.write(decks.deck(nx=n, ny=n, ne=n * n * 4, ni=n * n * 4, solver="cg", tol="1e-10", maxit=100000),
                      str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    orc.scatter_all()
    sim = E.Simulation.from_ini(ini)
    sim.set_grid("rho", orc.rho)
    it_ref, err_ref, conv = sim.potential_solver()
    assert conv
    phi_ref = sim.grid("phi")
    s = orc.s
    K = (s.L * s.L) / (s.LDe * s.LDe)
    fn = _fn(E)
    rho_d = torch.tensor(orc.rho, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        phi_d = torch.full_like(rho_d, float(call + 7))  # garbage the solve must overwrite
        torch.cuda.synchronize()
        it = ctypes.c_int()
        err = ctypes.c_double()
        st = fn(rho_d.data_ptr(), phi_d.data_ptr(), s.nx, s.ny, s.dx, K, s.tolerance, s.max_iteration, None,
                ctypes.byref(it), ctypes.byref(err))
        assert st == 0, E.lib().epic_last_error()
        assert it.value == it_ref
        phi = phi_d.cpu().numpy()
        assert np.max(np.abs(phi - phi_ref)) <= 1e-12 * np.max(np.abs(phi_ref))
        assert abs(err.value - err_ref) <= 1e-9 * err_ref


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
