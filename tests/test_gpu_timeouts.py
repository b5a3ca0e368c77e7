"""The bounded device-side waits, made to give up on purpose.

Every wait inside a kernel (the grid barriers of the PCG solve, the ordered
tile look-back of the compacting push) polls at most a limited number of
times and then reports EPIC_ERR_TIMEOUT instead of waiting on.  The limit is
settable (epic_set_spin_limit); with a limit of one poll, healthy waits that
are not already complete on their first poll give up, which is the only way
to reach the timeout path without faulting or hanging a GPU.  Each test checks
that the call reports the timeout, that nothing hangs, and that the next call
with the default limit restored is clean and matches the oracle.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def set_spin(E, polls):
    fn = E.lib().epic_set_spin_limit
    fn.argtypes = [ctypes.c_longlong]
    fn.restype = ctypes.c_int
    assert fn(polls) == 0


def test_pcg_barrier_gives_up_and_the_next_solve_is_clean(gpu_lib, tmp_path):
    E = gpu_lib
    ini = decks.write(decks.deck(nx=96, ny=96, ne=40000, ni=40000, solver="cg", tol="1e-10", maxit=20000),
                      str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    orc.scatter_all()
    sim = E.Simulation.from_ini(ini)
    sim.set_grid("rho", orc.rho)
    try:
        set_spin(E, 1)
        with pytest.raises(E.EpicError) as ei:
            sim.potential_solver()
        assert ei.value.status == 7, ei.value  # EPIC_ERR_TIMEOUT
    finally:
        set_spin(E, 0)
    it, err, conv = sim.potential_solver()
    phi_o, _, it_o, conv_o = orc.R.pcg_solve(orc.rho)
    assert conv and conv_o and it == it_o
    assert rel(sim.grid("phi"), phi_o) < 1e-12


@pytest.mark.parametrize("precision", [0, 1])
def test_push_lookback_gives_up_and_the_next_push_is_clean(gpu_lib, tmp_path, precision):
    """Open walls: the push compacts the survivors in order through a tile look-back.  After the
    timeout the particles are reloaded; the next push equals the oracle's (FP64 form) or a run that
    never timed out, bit for bit (mixed form)."""
    E = gpu_lib
    ini = decks.write(decks.deck(nx=64, ny=48, ne=600000, ni=600000, bc="open", te=20, dt=0.05), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    rng = np.random.default_rng(7)
    ex, ey = rng.normal(size=orc.efx.shape) * 5, rng.normal(size=orc.efy.shape) * 5

    def fresh():
        sim = E.Simulation.from_ini(ini, precision=precision)
        sim.set_particles(0, orc.parts[0])
        sim.set_grid("efx", ex)
        sim.set_grid("efy", ey)
        return sim

    sim = fresh()
    try:
        set_spin(E, 1)
        with pytest.raises(E.EpicError) as ei:
            sim.push_species(0)
            sim.sync()
        assert ei.value.status == 7, ei.value
    finally:
        set_spin(E, 0)
    sim.set_particles(0, orc.parts[0])
    sim.push_species(0)
    got = sim.particles(0)
    if precision == 0:
        ref = orc.R.push(orc.s.species[0], orc.parts[0], ex, ey)
        assert len(ref) < len(orc.parts[0]), "electrons should leave through the open walls"
        assert got.shape == ref.shape
        for c in range(5):
            assert rel(got[:, c], ref[:, c]) < 1e-14
    else:
        other = fresh()
        other.push_species(0)
        want = other.particles(0)
        assert len(want) < len(orc.parts[0])
        assert np.array_equal(got, want)
