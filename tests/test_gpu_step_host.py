"""epic_step_host: one loop iteration for particles held in host memory, as
the reference holds part_list (src/main.cpp:405-423).  With pinned buffers the
kernels read and write them directly; with pageable ones the same step runs
through the staging copies.  Both must give the device-resident loop's
particles bit for bit, MCC (appended electrons and ions) included."""
import numpy as np
import pytest

from tests import decks

pytestmark = pytest.mark.gpu


def _deck(tmp_path, bc="pbc", collisions=True):
    return decks.write(decks.deck(nx=32, ny=32, ne=40000, ni=40000, te=30, ion_mass="6.63352090e-26", bc=bc,
                                  collisions=collisions, gas="1e22", solver="cg", tol="1e-10",
                                  beam=dict(n=4000, t=1, frac=0.1, vx=5, vy=0)), str(tmp_path))


def _pair(E, ini):
    sims = []
    for _ in range(2):
        s = E.Simulation.from_ini(ini, capacity=200000)
        s.set_reference_cross_sections()
        s.load_particles(0)
        s.initial_field()
        sims.append(s)
    return sims


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("bc,collisions", [("pbc", True), ("reflective", False)])
def test_step_host_equals_device_loop(gpu_lib, tmp_path, pinned, bc, collisions):
    import torch

    ini = _deck(tmp_path, bc, collisions)
    host_sim, dev_sim = _pair(gpu_lib, ini)
    nsp = len(host_sim.species)
    cap = 200000
    if pinned:
        bufs = [torch.zeros((cap, 5), dtype=torch.float64, pin_memory=True).numpy() for _ in range(nsp)]
    else:
        bufs = [np.zeros((cap, 5)) for _ in range(nsp)]
    counts = [host_sim.particles_into(k, bufs[k]) for k in range(nsp)]
    grew = False
    for step in range(4):
        before = list(counts)
        counts = host_sim.step_host(bufs, counts, collisions=collisions)
        dev_sim.step(collisions=collisions)
        grew |= counts[0] > before[0]
        for k in range(nsp):
            ref = dev_sim.particles(k)
            assert counts[k] == len(ref), (step, k)
            assert np.array_equal(bufs[k][:counts[k]], ref), (step, k)
    if collisions:
        assert grew  # ionisation appended electrons (and ions) through the host path
    host_sim.close()
    dev_sim.close()


def test_step_host_capacity_error(gpu_lib, tmp_path):
    ini = _deck(tmp_path)
    sim = gpu_lib.Simulation.from_ini(ini, capacity=200000)
    sim.set_reference_cross_sections()
    sim.load_particles(0)
    sim.initial_field()
    n = [sim.num_particles(k) for k in range(3)]
    bufs = [np.zeros((max(c - 1, 1), 5)) for c in n]  # one record short
    with pytest.raises(gpu_lib.EpicError):
        sim.step_host(bufs, n, collisions=True)
    sim.close()
