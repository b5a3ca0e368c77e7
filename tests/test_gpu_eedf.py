"""MCC statistics beyond collision counts: the electron energy distribution
after one collision step.

The GPU's direct MCC draws from a counter-based Philox stream; the oracle's
restatement draws from the reference's sequential mt19937 stream
(src/collision.cpp:60-207).  Started from the same 30 eV electrons in a dense
gas (about one in twenty-five collides), the two must agree in distribution:

* the energies of the electrons that collided (elastic, excitation and
  ionisation scattering, src/collision.cpp:60-188), two-sample KS test;
* the energies of the electrons created by ionisation, KS test;
* the number of collisions and of ionisations within 6 sigma of the oracle's
  expectation (binomial counts);
* the velocity directions after scattering: mean cosine with the incoming
  direction, within 6 standard errors.

Both the reference's analytic Ar cross sections on its linear table and the
synthetic log-spaced table are checked.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu

KS_P_MIN = 1e-4  # fail only on a clear difference of distributions


def _energy(v, vel_norm):
    return 0.5 * O.ME * np.sum((v * vel_norm) ** 2, axis=1) / O.EV


@pytest.mark.parametrize("table", ["reference", "log"])
def test_post_collision_energy_distributions_match_oracle(gpu_lib, tmp_path, table):
    from scipy import stats

    from epic2d_mcc_gb300 import workloads

    E = gpu_lib
    ini = decks.write(decks.deck(nx=32, ny=32, ne=400000, ni=400000, te=30, ion_mass="6.63352090e-26",
                                 collisions=True, gas="5e21"), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    s = orc.s
    e0, i0 = orc.parts[0].copy(), orc.parts[1].copy()
    sim = E.Simulation.from_ini(ini, mcc_mode=0, seed=7)
    if table == "log":
        eg, ela, exc, ion = workloads.synthetic_table()
        orc.R.set_log_table(ela, exc, ion, eg[0], eg[-1])
        sim.set_log_cross_sections(ela, exc, ion, eg[0], eg[-1])
    else:
        sim.set_reference_cross_sections()
    sim.set_particles(0, e0)
    sim.set_particles(1, i0)
    n_gpu = sim.handle_collisions(0, 1)
    ge, gi = sim.particles(0), sim.particles(1)
    oe, oi, n_orc, kinds = orc.R.mcc(e0, i0, s.species[1], rng=O.Rng(0))
    ne = len(e0)
    # the electrons that collided: velocity changed (their positions are untouched)
    g_hit = np.any(ge[:ne, 2:5] != e0[:, 2:5], axis=1)
    o_hit = kinds > 0
    assert g_hit.sum() > 10000 and o_hit.sum() > 10000
    # counts: binomial around the oracle's (same per-electron probabilities)
    sd = np.sqrt(n_orc * (1 - n_orc / ne))
    assert abs(n_gpu - n_orc) < 6 * np.sqrt(2) * sd + 1
    g_new, o_new = len(ge) - ne, len(oe) - ne
    assert len(gi) - len(i0) == g_new and len(oi) - len(i0) == o_new
    if o_new > 100:
        assert abs(g_new - o_new) < 6 * np.sqrt(2 * o_new) + 1
    # energies of the scattered electrons
    eg_hit = _energy(ge[:ne][g_hit, 2:5], s.vel_norm)
    eo_hit = _energy(oe[:ne][o_hit, 2:5], s.vel_norm)
    p = stats.ks_2samp(eg_hit, eo_hit).pvalue
    assert p > KS_P_MIN, "scattered-electron energies differ (KS p = %g)" % p
    # energies of the ionisation electrons
    if o_new > 200 and g_new > 200:
        p2 = stats.ks_2samp(_energy(ge[ne:, 2:5], s.vel_norm), _energy(oe[ne:, 2:5], s.vel_norm)).pvalue
        assert p2 > KS_P_MIN, "ionisation-electron energies differ (KS p = %g)" % p2
    # scattering angle: cosine between the incoming and outgoing directions
    def mean_cos(before, after):
        a = before / np.linalg.norm(before, axis=1, keepdims=True)
        b = after / np.linalg.norm(after, axis=1, keepdims=True)
        c = np.sum(a * b, axis=1)
        return c.mean(), c.std() / np.sqrt(len(c))

    mg, sg = mean_cos(e0[g_hit, 2:5], ge[:ne][g_hit, 2:5])
    mo, so = mean_cos(e0[o_hit, 2:5], oe[:ne][o_hit, 2:5])
    assert abs(mg - mo) < 6 * np.hypot(sg, so)
