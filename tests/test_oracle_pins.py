"""Pins the oracle's restatement to the reference.

* against tests/golden/*.npz (outputs of the reference's own objects), on any
  machine: bit-exact for every array of every phase;
* against the reference objects live (oracle/_ref), where the reference checkout
  was available to compile them: more decks, bit-exact;
* the MT19937 known answer of the C++ standard ([rand.predef]: the 10000th
  output of a default-seeded mt19937 is 4123659995).
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def _compare_snapshot(sim: O.OracleSim, g, prefix: str):
    for k in ("phi", "rho", "efx", "efy"):
        assert np.array_equal(getattr(sim, k), g[prefix + k]), prefix + k
    for s in range(len(sim.s.species)):
        assert np.array_equal(sim.den[s], g[prefix + "den%d" % s]), prefix + "den%d" % s
        assert np.array_equal(sim.parts[s], g[prefix + "part%d" % s]), prefix + "part%d" % s
    assert sim.error == g[prefix + "error"][0]


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_restatement_matches_reference_golden(path, tmp_path):
    g = np.load(path)
    ini = str(tmp_path / "deck.ini")
    with open(ini, "w") as f:
        f.write(str(g["ini"]))
    sim = O.OracleSim(ini, load=True, initial_field=False)
    for s in range(len(sim.s.species)):
        assert np.array_equal(sim.parts[s], g["load_part%d" % s])
    sim.initial_field()
    _compare_snapshot(sim, g, "init_")
    coll = bool(g["collisions"][0])
    for k in range(int(g["steps"][0])):
        sim.step(collisions=coll)
        _compare_snapshot(sim, g, "step%d_" % (k + 1))


def test_mt19937_known_answer():
    r = O.Rng(5489)
    for _ in range(9999):
        r.u32()
    assert r.u32() == 4123659995


def test_generate_canonical_range():
    r = O.Rng(0)
    u = np.array([r.uniform() for _ in range(20000)])
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01


def test_mcc_injected_mode_replays_sequential_stream(tmp_path):
    """Mode 1 (per-electron uniforms) equals mode 0 when fed the draws mode 0 consumed."""
    ini = decks.write(decks.deck(nx=24, ny=24, ne=300, ni=300, te=30, ion_mass="6.63352090e-26", collisions=True,
                                 gas="1e23", solver="gs", tol="1e-6"), str(tmp_path))
    a = O.OracleSim(ini)
    b = O.OracleSim(ini)
    a.step()
    b.step()
    # Record the draws mode 0 makes, electron by electron, by replaying the RNG.
    R = a.R
    tot, ela, exc, ion = R.cs_tables()
    rng_copy = O.Rng(0)
    rng_copy.s = type(a.rng.s).from_buffer_copy(a.rng.s)
    e0, i0, nc0, kinds0 = R.mcc(a.parts[0], a.parts[1], a.s.species[1], rng=a.rng)
    # draws per electron: 1 (no collision), 3 (elastic/excitation: test, type, 2 angles -> 4 or 5), ...
    counts = {0: 1, 1: 4, 2: 5, 3: 14}
    U = np.zeros((len(kinds0), 16))
    for p, k in enumerate(kinds0):
        for j in range(counts[int(k)]):
            U[p, j] = rng_copy.uniform()
    e1, i1, nc1, kinds1 = R.mcc(b.parts[0], b.parts[1], b.s.species[1], uniforms=U)
    assert nc0 == nc1 and nc0 > 0
    assert np.array_equal(kinds0, kinds1)
    assert np.array_equal(e0, e1)
    assert np.array_equal(i0, i1)


needs_ref = pytest.mark.skipif(not O.Reference.available(), reason="reference checkout not available here")

# Two conductors: a rectangle (ReactConductorGrid) and a ring of six circular
# electrodes (CircularGrid), src/grid.cpp, src/electrode.cpp.
CONDUCTORS = [dict(type="reactconduct", min_x=10, max_x=12, min_y=4, max_y=16, grid_voltage=10),
              dict(type="circular", x_center=22, y_center=12, electrode_number=6, grid_radius=5,
                   electrod_radius=1.5, electrode_voltage=-5)]

LIVE = {
    "gs_open_conductors": dict(nx=32, ny=24, ne=2000, ni=2000, te=4, solver="gs", tol="1e-8", bc="open",
                               grids=CONDUCTORS),
    "gs_reflective_conductors": dict(nx=32, ny=24, ne=2000, ni=2000, te=4, solver="gs", tol="1e-8",
                                     bc="reflective", grids=CONDUCTORS),
    "pcg_pbc_conductors": dict(nx=32, ny=24, ne=2000, ni=2000, te=4, solver="cg", tol="1e-10", grids=CONDUCTORS),
    # Boltzmann-electron solvers (src/field.cpp:7-68, 141-210)
    "gshybrid_pbc": dict(nx=20, ny=14, ne=1500, ni=1500, solver="gshybrid", tol="1e-6", te=2),
    "hybrid_pbc": dict(nx=14, ny=10, ne=800, ni=800, solver="hybrid", tol="1e-6", te=2),
    "gs_pbc_cic_rect": dict(nx=20, ny=14, ne=1500, ni=1500, solver="gs", tol="1e-9"),
    "gs_open_ngp": dict(nx=16, ny=16, ne=1500, ni=1500, solver="gs", tol="1e-8", bc="open", shape="NGP", te=6),
    "pcg_reflective_cic": dict(nx=18, ny=18, ne=1500, ni=1500, solver="cg", tol="1e-10", bc="reflective"),
    "pcg_pbc_rect": dict(nx=16, ny=12, ne=1000, ni=1000, solver="cg", tol="1e-10"),
    "gs_ionscale_norm2": dict(nx=16, ny=16, ne=1000, ni=1000, solver="gs", tol="1e-7", norm=2, dt=0.001),
    "gs_maxit_cap": dict(nx=16, ny=16, ne=1000, ni=1000, solver="gs", tol="1e-14", maxit=37),
    "pcg_maxit_cap": dict(nx=16, ny=16, ne=1000, ni=1000, solver="cg", tol="1e-16", maxit=9),
}


@needs_ref
@pytest.mark.parametrize("name", sorted(LIVE))
def test_restatement_matches_reference_live(name, tmp_path):
    ini = decks.write(decks.deck(**LIVE[name]), str(tmp_path))
    ref = O.Reference(ini)
    sim = O.OracleSim(ini)
    for _ in range(3):
        ref.step(0)
        sim.step()
    for k in ("phi", "rho", "efx", "efy"):
        assert np.array_equal(ref.grid(k), getattr(sim, k)), k
    for s in range(2):
        assert np.array_equal(ref.particles(s), sim.parts[s]), s
    assert ref.solver_error() == sim.error


@needs_ref
def test_diagnostics_match_reference_live(tmp_path):
    ini = decks.write(decks.deck(nx=16, ny=16, ne=1000, ni=1000, beam=dict(n=300, t=1, frac=0.3, vx=3, vy=1)),
                      str(tmp_path))
    ref = O.Reference(ini)
    sim = O.OracleSim(ini)
    ref.step(0)
    sim.step()
    for s in range(3):
        out = np.zeros(3)
        ref.ke(s, 0, O._p(out))
        assert np.array_equal(out, sim.R.ke(sim.s.species[s], sim.parts[s], sim.s.species[0]))
        ref.momentum(s, 0, O._p(out))
        assert np.array_equal(out, sim.R.momentum(sim.s.species[s], sim.parts[s], sim.s.species[0]))
    assert ref.pe(0) == sim.R.pe(sim.efx, sim.efy, sim.s.species[0])


@needs_ref
def test_setup_matches_reference_live(tmp_path):
    for kw in (dict(), dict(norm=2, dt=0.001), dict(norm=4), dict(beam=dict(n=300, t=2, frac=0.5, vx=1, vy=2))):
        ini = decks.write(decks.deck(**kw), str(tmp_path))
        ref = O.Reference(ini, load=False, initial_field=False)
        s = O.setup(ini)
        p = ref.params
        got = [s.nx, s.ny, s.x0, s.y0, s.dx, s.dy, s.Lx, s.Ly, s.DT, s.L, s.W, s.vel_norm, s.LDe, s.wpe, s.LDi,
               s.wpi, s.density]
        assert list(p[:17]) == got
        for k, sp in enumerate(s.species):
            rp = ref.species_params(k)
            assert [rp[0], rp[1], rp[2]] == [sp.mass, sp.charge, sp.spwt]


EMITTERS = [dict(x0=1, y0=4, x1=1, y1=12, temp=0.5, numparticle=7, vdx=0.5, vdy=0, species_idx1=0, species_idx2=1),
            dict(x0=5, y0=5, x1=9, y1=9, temp=0.02, numparticle=3, vdx=0, vdy=0.2, species_idx1=1, species_idx2=1)]


@needs_ref
def test_emitters_match_reference_live(tmp_path):
    """Emitter::inject (src/emitter.cpp:5-36): counts, append order and velocities (the global mt19937
    stream) bit for bit; positions come from a std::random_device-seeded generator in the reference, so
    only their range is checked."""
    ini = decks.write(decks.deck(nx=16, ny=16, ne=500, ni=500, emitters=EMITTERS), str(tmp_path))
    ref = O.Reference(ini)
    orc = O.OracleSim(ini)
    loaded = [len(orc.parts[s]) for s in range(2)]
    for _ in range(3):
        n0 = [len(orc.parts[s]) for s in range(2)]
        ref.inject()
        orc.inject()
        for s in range(2):
            got, want = ref.particles(s), orc.parts[s]
            assert len(got) == len(want)
            assert np.array_equal(got[:loaded[s]], want[:loaded[s]])
            assert np.array_equal(got[:, 2:], want[:, 2:])
        new_e = ref.particles(0)[n0[0]:]
        assert np.all(new_e[:, 0] == 1.0) and np.all((new_e[:, 1] >= 4) & (new_e[:, 1] < 12))
        new_i = ref.particles(1)[n0[1]:]
        assert len(new_i) == 7 + 3 and np.all(new_i[:7, 0] == 1.0)
        assert np.all((new_i[7:, :2] >= 5) & (new_i[7:, :2] < 9))
