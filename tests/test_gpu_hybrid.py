"""Boltzmann-electron field solvers on the GPU against the oracle (pinned to
the reference live and by tests/golden/{gshybrid,hybrid}_pbc.npz):
gsfluidsolver ("gshybrid", src/field.cpp:7-68: the SOR sweep with source
(rho - exp(phi)) K, rho's edges overwritten, residual every 50 sweeps) and
nrpcgsolver ("hybrid", src/field.cpp:141-210: ten Newton steps, each a dense
CG to 1e-4; the oracle sums its dot products in the reference's order, the
GPU exactly).  The device exp and the host library's may differ in the last
bit, hence 1e-12 rather than bit equality.  The smallest grids (6 cells
across: too few node rows or nodes for a thread-block cluster) take the
one-CTA kernels, the others the clustered ones."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)) if b.size else 0.0


@pytest.mark.parametrize("solver,nx,ny", [("gshybrid", 20, 14), ("gshybrid", 24, 24), ("gshybrid", 6, 16),
                                          ("hybrid", 14, 10), ("hybrid", 16, 16), ("hybrid", 6, 8)])
def test_boltzmann_solvers_track_oracle(gpu_lib, tmp_path, solver, nx, ny):
    ini = decks.write(decks.deck(nx=nx, ny=ny, ne=1500, ni=1500, te=2, solver=solver, tol="1e-6"), str(tmp_path))
    orc = O.OracleSim(ini)
    sim = gpu_lib.Simulation.from_ini(ini)
    sim.load_particles(0)
    sim.initial_field()
    assert rel(sim.grid("phi"), orc.phi) < TOL
    assert rel(sim.grid("rho"), orc.rho) < TOL
    for _ in range(3):
        orc.step()
        sim.step()
        assert rel(sim.grid("rho"), orc.rho) < TOL
        assert rel(sim.grid("phi"), orc.phi) < TOL
        for s in range(2):
            assert rel(sim.particles(s), orc.parts[s]) < TOL
    if solver == "gshybrid":  # the top edge carries the reference's 10000
        rho = sim.grid("rho").reshape(nx + 1, ny + 1)
        assert np.all(rho[1:-1, -1] == 10000.0) and np.all(rho[:, 0] == 0) and np.all(rho[0, :] == 0)
    sim.close()
