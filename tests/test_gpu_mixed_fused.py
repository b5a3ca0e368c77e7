"""The mixed form's fused step (CIC, periodic or reflective walls): the push
deposits every particle at its new position and, with collisions, selects the
MCC's candidates on the pushed velocities; the MCC's ionisation products are
deposited after it.  Checked bit for bit against the same steps composed of
the single-phase calls, which deposit in a separate pass over the positions
(epic_scatter_species) and select in the MCC's own pass
(epic_handle_collisions):

* particles, densities, rho and phi are equal, step after step;
* the collision counts are equal;
* a graph-replayed run (the captured step takes the accumulators the previous
  step's push left) equals the same steps launched one by one.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu

STEPS = 4


def _deck(tmp_path, bc, collisions, n=60000):
    kw = dict(nx=48, ny=40, ne=n, ni=n, bc=bc, solver="cg", tol="1e-10", maxit=100000)
    if collisions:
        kw.update(te=30, ion_mass="6.63352090e-26", collisions=True, gas="1e22", dt=0.05)
    return decks.write(decks.deck(**kw), str(tmp_path))


def _sim(E, ini, orc, collisions, **over):
    sim = E.Simulation.from_ini(ini, precision=1, capacity=4 * len(orc.parts[0]), **over)
    if collisions:
        sim.set_reference_cross_sections()
    for s in range(2):
        sim.set_particles(s, orc.parts[s])
    sim.initial_field()
    return sim


def _state(sim):
    return ([sim.particles(s) for s in range(2)], [sim.den(s) for s in range(2)], sim.grid("rho"),
            sim.grid("phi"))


def _same(a, b):
    (pa, da, ra, fa), (pb, db, rb, fb) = a, b
    for s in range(2):
        assert pa[s].shape == pb[s].shape
        assert np.array_equal(pa[s], pb[s])
        assert np.array_equal(da[s], db[s])
    assert np.array_equal(ra, rb) and np.array_equal(fa, fb)


@pytest.mark.parametrize("bc", ["pbc", "reflective"])
@pytest.mark.parametrize("collisions", [False, True])
def test_fused_step_equals_phase_calls(gpu_lib, tmp_path, bc, collisions):
    E = gpu_lib
    ini = _deck(tmp_path, bc, collisions)
    orc = O.OracleSim(ini, initial_field=False)
    fused = _sim(E, ini, orc, collisions)
    split = _sim(E, ini, orc, collisions)
    n_fused = n_split = 0
    for _ in range(STEPS):
        fused.step(collisions=collisions)
        for s in range(2):
            split.scatter_species(s)
        split.compute_rho()
        split.potential_solver()
        split.calculate_efield()
        for s in range(2):
            split.push_species(s)
        if collisions:
            n_split += split.handle_collisions(0, 1)
        # densities, rho and phi of this step: the fused run's from the accumulators the previous step's push
        # (and range deposit) left, the split run's from its own deposit pass
        _same(_state(fused), _state(split))
    if collisions:
        n_fused = fused.num_particles(0) - len(orc.parts[0])
        assert n_split > 100
        assert fused.num_particles(0) == split.num_particles(0)
        assert n_fused > 0  # ionisation appended electrons, deposited by the range pass


def test_fused_graph_replay_equals_steps(gpu_lib, tmp_path):
    E = gpu_lib
    ini = _deck(tmp_path, "pbc", True)
    orc = O.OracleSim(ini, initial_field=False)
    out = []
    for graph in (False, True):
        sim = _sim(E, ini, orc, True, sort_every=2)
        sim.run(6, collisions=True, graph=graph)
        out.append(_state(sim))
    _same(out[0], out[1])
