"""The MCC early-out by speed bin (epic_mcc.cu k_mcc_select): an electron is
dropped before its collision test only when its first draw is above a bound
of the collision probability of every speed in its bin, so it can never drop
one that the reference's test p_coll > u0 (src/collision.cpp:85-97) would
collide.  Checked adversarially: every electron's injected first draw sits
just below its own p_coll, over energies from 1e-4 eV to 1e4 eV, so nearly
every electron must collide, exactly as the oracle says."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _speeds(sim, n, rng):
    """Velocities (vel_norm units) with energies log-uniform on [1e-4, 1e4] eV."""
    vn = sim.cfg.vel_norm
    energy = 10.0 ** rng.uniform(-4, 4, n)
    speed = np.sqrt(2 * energy * O.EV / O.ME) / vn
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    return speed[:, None] * d


def _p_coll(v, vn, dt, table):
    """The reference's collision probability of velocities v (vel_norm units)."""
    v2 = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2]) * vn * vn
    energy = 0.5 * O.ME * v2 / O.EV
    return 1 - np.exp(-table(energy) * np.sqrt(v2) * dt)


def _setup(gpu_lib, tmp_path, log_table, precision=0, n=20000):
    from epic2d_mcc_gb300 import workloads

    kw = dict(nx=32, ny=32, ne=n, ni=n, te=10, ion_mass="6.63352090e-26", collisions=True, gas="1e22")
    ini = decks.write(decks.deck(**kw), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    sim = gpu_lib.Simulation.from_ini(ini, mcc_mode=1, precision=precision, capacity=4 * n)
    s = orc.s
    if log_table:
        e_grid, ela, exc, ion = workloads.synthetic_table()
        orc.R.set_log_table(ela, exc, ion, e_grid[0], e_grid[-1])
        sim.set_log_cross_sections(ela, exc, ion, e_grid[0], e_grid[-1])
        tot = (ela + exc + ion) * s.gas_density
        lg = np.log(e_grid)

        def table(energy):
            e = np.clip(energy, e_grid[0], e_grid[-1])
            return np.interp(np.log(e), lg, tot)
    else:
        sim.set_reference_cross_sections()
        tot = orc.R.cs_tables()[0]

        def table(energy):
            return tot[np.minimum((energy / 0.005 + 0.5).astype(np.int64), O.CS_RANGES - 1)]
    return ini, orc, sim, table


@pytest.mark.parametrize("log_table", [False, True])
def test_speed_bins_keep_every_collision_fp64(gpu_lib, tmp_path, log_table):
    ini, orc, sim, table = _setup(gpu_lib, tmp_path, log_table)
    rng = np.random.default_rng(21)
    e = orc.parts[0].copy()
    e[:, 2:5] = _speeds(sim, len(e), rng)
    s = orc.s
    p = _p_coll(e[:, 2:5], s.vel_norm, s.DT / s.W, table)
    assert p.max() > 1e3 * p.min()  # the bins from rarely to often
    U = rng.random((len(e), 16))
    U[:, 0] = p * (1 - 1e-3)
    sim.set_particles(0, e)
    sim.set_particles(1, orc.parts[1])
    ee, ii, nc, kinds = orc.R.mcc(e, orc.parts[1], orc.s.species[1], uniforms=U)
    assert nc == np.count_nonzero(p > 0) and nc > 0.99 * len(e)
    got = sim.handle_collisions(0, 1, uniforms=U)
    assert got == nc
    ge, gi = sim.particles(0), sim.particles(1)
    assert len(ge) == len(ee) and len(gi) == len(ii)
    assert max(np.max(np.abs(ge[:, c] - ee[:, c])) / max(np.max(np.abs(ee[:, c])), 1e-300) for c in range(5)) < TOL


@pytest.mark.parametrize("log_table", [False, True])
def test_speed_bins_keep_every_collision_mixed(gpu_lib, tmp_path, log_table):
    """Mixed form: FP32 velocities, so p_coll is taken from the stored floats."""
    ini, orc, sim, table = _setup(gpu_lib, tmp_path, log_table, precision=1)
    rng = np.random.default_rng(22)
    e = orc.parts[0].copy()
    e[:, 2:5] = _speeds(sim, len(e), rng).astype(np.float32).astype(np.float64)
    s = orc.s
    p = _p_coll(e[:, 2:5], s.vel_norm, s.DT / s.W, table)
    U = rng.random((len(e), 16))
    U[:, 0] = p * (1 - 1e-3)
    sim.set_particles(0, e)
    sim.set_particles(1, orc.parts[1])
    got = sim.handle_collisions(0, 1, uniforms=U)
    assert got == np.count_nonzero(p > 0)
