"""The null-collision MCC (mcc_mode 2, no reference counterpart): a first draw
against the constant null-collision probability P = 1 - exp(-nu_max dt)
selects the candidates, a second accepts one with nu(E) / nu_max, and the
accepted collision is the direct MCC's (src/collision.cpp:60-188).  The
synthetic log-spaced table is staged in shared memory by the collision
kernels.  nu_max bounds sigma_tot(E) v(E) over the table and speeds up to
twice that of its last energy (the set-up in epic_set_log_cross_sections).

On the same 30 eV electrons, with the direct MCC beside it:
* each method's number of collisions within 6 sigma of its own expectation
  from the table (host side): sum_i (1 - exp(-nu_i dt)) for the direct MCC,
  sum_i P nu_i / nu_max for the null-collision MCC (the two differ by the
  method's O(nu_max dt) discretisation);
* the ionisations in the same proportion, within 6 sigma;
* the energies of the scattered electrons and of the ionisation electrons
  (two-sample KS tests; a thin gas, so that the methods' energy weighting of
  the colliders differs by at most nu_max dt / 2, about 2 %).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu

KS_P_MIN = 1e-4


def _energy(v, vel_norm):
    return 0.5 * O.ME * np.sum((v * vel_norm) ** 2, axis=1) / O.EV


def _nu_max(eg, tot):
    """The null-collision bound of the table (as the library's set-up forms it)."""
    n = len(eg)
    inv_dlog = (n - 1) / (np.log(eg[-1]) - np.log(eg[0]))
    e1 = np.exp(np.log(eg[0]) + np.arange(1, n) / inv_dlog)
    mx = np.max(np.maximum(tot[:-1], tot[1:]) * np.sqrt(2.0 * e1 * O.EV / O.ME))
    return max(mx, tot[-1] * np.sqrt(2.0 * 4 * eg[-1] * O.EV / O.ME))


def test_null_collision_mcc_matches_its_expectation_and_the_direct_mcc(gpu_lib, tmp_path):
    from scipy import stats

    from epic2d_mcc_gb300 import workloads

    E = gpu_lib
    ini = decks.write(decks.deck(nx=32, ny=32, ne=400000, ni=400000, te=30, ion_mass="6.63352090e-26",
                                 collisions=True, gas="2e20"), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    s = orc.s
    e0, i0 = orc.parts[0].copy(), orc.parts[1].copy()
    eg, ela, exc, ion = workloads.synthetic_table()
    runs = {}
    for mode in (0, 2):
        sim = E.Simulation.from_ini(ini, mcc_mode=mode, seed=11)
        sim.set_log_cross_sections(ela, exc, ion, eg[0], eg[-1])
        sim.set_particles(0, e0)
        sim.set_particles(1, i0)
        n = sim.handle_collisions(0, 1)
        runs[mode] = (n, sim.particles(0), sim.particles(1))
        sim.close()
    # expectations from the table
    dt = s.DT / s.W
    v = e0[:, 2:5] * s.vel_norm
    speed = np.sqrt(np.sum(v * v, axis=1))
    energy = np.clip(0.5 * O.ME * speed ** 2 / O.EV, eg[0], eg[-1])
    tot = (ela + exc + ion) * s.gas_density
    nu = np.interp(np.log(energy), np.log(eg), tot) * speed
    numax = _nu_max(eg, tot)
    assert np.all(nu <= numax) and numax * dt < 0.1
    p_direct = 1 - np.exp(-nu * dt)
    p_null = (1 - np.exp(-numax * dt)) * nu / numax
    n_direct, ge_d, gi_d = runs[0]
    n_null, ge_n, gi_n = runs[2]
    for n, p in ((n_direct, p_direct), (n_null, p_null)):
        assert p.sum() > 1000
        assert abs(n - p.sum()) < 6 * np.sqrt((p * (1 - p)).sum()), (n, p.sum())
    ne = len(e0)
    new_d, new_n = len(ge_d) - ne, len(ge_n) - ne
    assert len(gi_d) - len(i0) == new_d and len(gi_n) - len(i0) == new_n
    ratio = p_null.sum() / p_direct.sum()
    assert new_d > 50 and abs(new_n - ratio * new_d) < 6 * np.sqrt(new_n + ratio * ratio * new_d) + 1
    hit_d = np.any(ge_d[:ne, 2:5] != e0[:, 2:5], axis=1)
    hit_n = np.any(ge_n[:ne, 2:5] != e0[:, 2:5], axis=1)
    pk = stats.ks_2samp(_energy(ge_d[:ne][hit_d, 2:5], s.vel_norm), _energy(ge_n[:ne][hit_n, 2:5], s.vel_norm))
    assert pk.pvalue > KS_P_MIN, "scattered-electron energies differ (KS p = %g)" % pk.pvalue
    pk2 = stats.ks_2samp(_energy(ge_d[ne:, 2:5], s.vel_norm), _energy(ge_n[ne:, 2:5], s.vel_norm))
    assert pk2.pvalue > KS_P_MIN, "ionisation-electron energies differ (KS p = %g)" % pk2.pvalue
