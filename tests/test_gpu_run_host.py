"""epic_run_host: several steps of particles held in host memory, every step's
records going to the caller's buffers and back (device-to-host after the
step, host-to-device before the next push), on copy engines beside the next
step's solve.  The result must equal the same steps run on the device
(epic_run without a graph) bit for bit: particles, counts and phi, with and
without the MCC's ionisation appends, and through the step-by-step fallback
(absorbing walls)."""
import numpy as np
import pytest

from tests import decks

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["pbc_mcc", "reflective", "open_fallback"])
def test_run_host_equals_device_run(gpu_lib, tmp_path, case):
    import torch

    E = gpu_lib
    bc = {"pbc_mcc": "pbc", "reflective": "reflective", "open_fallback": "open"}[case]
    coll = case == "pbc_mcc"
    ini = decks.write(decks.deck(nx=48, ny=40, ne=120000, ni=120000, solver="cg", tol="1e-10", bc=bc, te=30,
                                 collisions=coll, gas="1e22", ion_mass="6.63352090e-26"), str(tmp_path))
    sims = []
    for _ in range(2):
        sim = E.Simulation.from_ini(ini)
        if coll:
            sim.set_reference_cross_sections()
        sim.load_particles(0)
        sim.initial_field()
        sims.append(sim)
    a, b = sims
    a.run(5, collisions=coll, graph=False)
    nsp = len(b.species)
    caps = [b.species[s].capacity or (b.species[s].numparticle * 3 // 2 + 4096) for s in range(nsp)]
    bufs = [torch.empty((int(c), 5), dtype=torch.float64, pin_memory=True).numpy() for c in caps]
    counts = [b.particles_into(s, bufs[s]) for s in range(nsp)]
    counts = b.run_host(bufs, counts, 5, collisions=coll)
    if coll:
        assert counts[1] > 120000, "the MCC should ionise"
    for s in range(nsp):
        want = a.particles(s)
        assert counts[s] == len(want)
        assert np.array_equal(bufs[s][:counts[s]], want), "species %d" % s
        assert np.array_equal(b.particles(s), want)
    assert np.array_equal(a.grid("phi"), b.grid("phi"))
