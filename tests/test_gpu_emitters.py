"""Emitters (Emitter::inject, src/emitter.cpp:5-36) on the GPU: with caller
uniforms the appended particles equal the oracle's restatement (pinned
against the reference in test_oracle_pins) bit for bit; on the Philox stream
the positions and velocities have the reference's distributions, the counts
grow by numparticle per step, and graph replay equals stepping."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu

EMITTERS = [dict(x0=1, y0=4, x1=1, y1=12, temp=0.5, numparticle=7, vdx=0.5, vdy=0, species_idx1=0, species_idx2=1),
            dict(x0=5, y0=5, x1=9, y1=9, temp=0.02, numparticle=3, vdx=0, vdy=0.2, species_idx1=1, species_idx2=1)]


def test_inject_with_uniforms_matches_oracle(gpu_lib, tmp_path):
    ini = decks.write(decks.deck(nx=16, ny=16, ne=500, ni=500, emitters=EMITTERS), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    sim = gpu_lib.Simulation.from_ini(ini)
    sim.load_particles(0)
    rng = np.random.default_rng(3)
    parts = list(orc.parts)
    for _ in range(2):
        U = rng.random((7 + 3, 14))
        sim.inject(U)
        parts = orc.R.inject(orc.s.emitters[0], parts, None, U[:7, :2].reshape(-1), U[:7, 2:])
        parts = orc.R.inject(orc.s.emitters[1], parts, None, U[7:, :2].reshape(-1), U[7:, 2:])
    for s in range(2):
        got = sim.particles(s)
        assert got.shape == parts[s].shape
        assert np.array_equal(got, parts[s])
    sim.close()


def test_inject_philox_distribution(gpu_lib, tmp_path):
    em = [dict(x0=2, y0=3, x1=10, y1=7, temp=2.0, numparticle=200000, vdx=1.5, vdy=-0.5, species_idx1=0,
               species_idx2=1)]
    ini = decks.write(decks.deck(nx=16, ny=16, ne=100, ni=100, emitters=em), str(tmp_path))
    sims = []
    for _ in range(2):
        s = gpu_lib.Simulation.from_ini(ini, capacity=500000)
        s.load_particles(0)
        s.inject()
        sims.append(s)
    e = sims[0].particles(0)[100:]
    i = sims[0].particles(1)[100:]
    assert len(e) == 200000 and len(i) == 200000
    assert np.array_equal(e[:, :2], i[:, :2])  # the pair shares its position
    assert np.all((e[:, 0] >= 2) & (e[:, 0] < 10) & (e[:, 1] >= 3) & (e[:, 1] < 7))
    assert abs(e[:, 0].mean() - 6) < 0.05 and abs(e[:, 1].mean() - 5) < 0.05
    s = O.setup(ini)
    for sp, arr in ((s.species[0], e), (s.species[1], i)):
        vth = np.sqrt(2 * O.K_B * 2.0 * O.EV_TO_K / sp.mass)
        sd = vth * np.sqrt(2) * 0.5 / s.vel_norm  # the sum of three uniforms has variance 1/4
        for c, vd in ((2, 1.5), (3, -0.5)):
            assert abs(arr[:, c].mean() - vd) < 5 * sd / np.sqrt(len(arr)) + 1e-12
            assert abs(arr[:, c].std() / sd - 1) < 0.01
        assert np.all(arr[:, 4] == 0)
    assert np.array_equal(sims[0].particles(0), sims[1].particles(0))  # same seed, same draws
    for x in sims:
        x.close()


def test_emitters_in_the_loop(gpu_lib, tmp_path):
    grids = [dict(type="reactconduct", min_x=0, max_x=6, min_y=10, max_y=11, grid_voltage=50),
             dict(type="reactconduct", min_x=0, max_x=6, min_y=5, max_y=6, grid_voltage=50)]
    em = [dict(x0=1, y0=7, x1=1, y1=9, temp=0.1, numparticle=50, vdx=0.2, vdy=0, species_idx1=0, species_idx2=1)]
    ini = decks.write(decks.deck(nx=32, ny=16, ne=2000, ni=2000, te=1, bc="open", solver="gs", tol="1e-6",
                                 grids=grids, emitters=em), str(tmp_path))
    a, b = (gpu_lib.Simulation.from_ini(ini) for _ in range(2))
    for s_ in (a, b):
        s_.load_particles(0)
        s_.initial_field()
    n0 = [a.num_particles(k) for k in range(2)]
    a.run(6, graph=True)
    for _ in range(6):
        b.step()
    for k in range(2):
        assert np.array_equal(a.particles(k), b.particles(k))
    # 6 injections of 50 per species, minus what the walls and conductors took
    n1 = [a.num_particles(k) for k in range(2)]
    assert all(n1[k] <= n0[k] + 300 for k in range(2)) and n1[1] > n0[1]
    a.close()
    b.close()
