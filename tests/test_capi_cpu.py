"""The C ABI without a GPU: the library builds and loads, exports every entry
point include/*.h declares, and its host-side set-up (INI parsing and
normalisation, src/main.cpp:34-261) agrees with the oracle bit for bit."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def E():
    from epic2d_mcc_gb300 import build as B

    B.build()
    import epic2d_mcc_gb300 as E

    return E


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(epic_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(E):
    L = E.lib()
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


DECKS = [dict(), dict(nx=20, ny=14, bc="open", shape="NGP", solver="cg", tol="1e-10"),
         dict(norm=2, dt=0.001), dict(norm=4, te=3, ti=0.1),
         dict(beam=dict(n=300, t=2, frac=0.5, vx=1, vy=2), collisions=True, gas="5e19")]


@pytest.mark.parametrize("kw", DECKS)
def test_config_from_ini_matches_oracle_setup(E, kw, tmp_path):
    ini = decks.write(decks.deck(**kw), str(tmp_path))
    cfg, descs, ts = E.config_from_ini(ini)
    s = O.setup(ini)
    assert (cfg.nx, cfg.ny) == (s.nx, s.ny)
    for f in ("x0", "y0", "dx", "dy", "DT", "L", "W", "vel_norm", "LDe", "wpe", "LDi", "wpi", "density", "tolerance",
              "gas_density"):
        assert getattr(cfg, f) == getattr(s, f), f
    assert cfg.max_iteration == s.max_iteration
    assert cfg.bc == O.BC_CODES[s.bc] and cfg.shape == O.SHAPE_CODES[s.shape]
    assert (cfg.elastic, cfg.excitation, cfg.ionization) == (s.elastic, s.excitation, s.ionization)
    assert ts == s.num_ts
    assert len(descs) == len(s.species)
    for d, sp in zip(descs, s.species):
        assert d.name.decode() == sp.name
        assert (d.mass, d.charge, d.spwt, d.temp, d.numparticle, d.vsx, d.vsy) == (
            sp.mass, sp.charge, sp.spwt, sp.temp, sp.numparticle, sp.vsx, sp.vsy)


def test_config_defaults_are_reference_behaviour(E):
    c = E.default_config()
    assert c.sor_omega == 1.4  # src/field.cpp:114
    assert c.sor_mode == 0 and c.warm_start == 0


def test_optional_keys(E, tmp_path):
    ini = decks.write(decks.deck(solver_extra="sor_omega = 1.8\nsor_mode = redblack\nwarm_start = true\n",
                                 sim_extra="deposit_mode = fp64\n", coll_extra="mcc_mode = null\nseed = 7\n"),
                      str(tmp_path))
    cfg, _, _ = E.config_from_ini(ini)
    assert cfg.sor_omega == 1.8 and cfg.sor_mode == 1 and cfg.warm_start == 1
    assert cfg.deposit_mode == 1 and cfg.mcc_mode == 2 and cfg.seed == 7


def test_errors_do_not_throw(E, tmp_path):
    with pytest.raises(E.EpicError) as ei:
        E.config_from_ini(str(tmp_path / "missing.ini"))
    assert ei.value.status == 9  # EPIC_ERR_IO
    text = decks.deck().replace("Ny       = 16\n", "")
    with pytest.raises(E.EpicError) as ei:
        E.config_from_ini(decks.write(text, str(tmp_path)))
    assert ei.value.status == 1 and "Ny" in str(ei.value)
    bad = decks.deck().replace("solvertype = gs", "solvertype = multigrid")
    with pytest.raises(E.EpicError) as ei:
        E.config_from_ini(decks.write(bad, str(tmp_path)))
    assert "multigrid" in str(ei.value)
    for name, code in (("gshybrid", 2), ("hybrid", 3)):  # the Boltzmann-electron solvers
        cfg, _, _ = E.config_from_ini(decks.write(decks.deck().replace("solvertype = gs", "solvertype = " + name),
                                                  str(tmp_path)))
        assert cfg.solver == code


def test_reference_input_deck_parses(E):
    # The repository's example deck format (three species, conductor section
    # present but grid_count = 0).
    text = decks.deck(beam=dict(n=1000, t=1, frac=1, vx=10, vy=10))
    cfg, descs, _ = E.config_from_ini(decks.write(text))
    assert [d.name.decode() for d in descs] == ["electron", "ion", "beam"]
    k = 2.0  # sum of -sign*frac = 1 + 0 + 1
    assert descs[0].spwt == pytest.approx(1e13 / k * cfg.L ** 2 * 16 * 16 / 2000)


def test_null_handle_is_rejected(E):
    L = E.lib()
    assert L.epic_step(None, 0) == 1
    assert b"null" in L.epic_last_error()


def test_conductors_from_ini_cpu(tmp_path):
    """[Grids] as src/main.cpp:284-327 reads it (no GPU needed)."""
    import epic2d_mcc_gb300 as E
    from tests import decks
    g = [dict(type="reactconduct", min_x=0, max_x=22, min_y=30, max_y=31, grid_voltage=100),
         dict(type="circular", x_center=22, y_center=12, electrode_number=6, grid_radius=5, electrod_radius=1.5,
              electrode_voltage=-5),
         dict(type="unknown_kind")]
    ini = decks.write(decks.deck(nx=32, ny=24, grids=g), str(tmp_path))
    cs = E.conductors_from_ini(ini)
    assert [c.type for c in cs] == [0, 1]  # other types are ignored, as in the reference
    assert (cs[0].min_x, cs[0].max_x, cs[0].min_y, cs[0].max_y) == (0, 22, 30, 31)
    assert (cs[1].x_center, cs[1].y_center, cs[1].electrode_number) == (22, 12, 6)
    assert (cs[1].grid_radius, cs[1].electrode_radius) == (5.0, 1.5)
    # voltages scaled as the reference does: eV / (k_B * EV_to_K) * V
    from oracle import oracle as O
    s = O.setup(ini)
    assert cs[0].voltage == s.grids[0][7] and cs[1].voltage == s.grids[1][7]


def test_emitters_from_ini_cpu(tmp_path):
    """[Emitters] as src/main.cpp:330-355 reads it (no GPU needed)."""
    import epic2d_mcc_gb300 as E
    from tests import decks
    em = [dict(x0=1, y0=20, x1=1, y1=30, temp=0, numparticle=5, vdx=0.0, vdy=0.0, species_idx1=0, species_idx2=1)]
    ini = decks.write(decks.deck(nx=32, ny=32, emitters=em), str(tmp_path))
    es = E.emitters_from_ini(ini)
    assert len(es) == 1
    e = es[0]
    assert (e.x0, e.y0, e.x1, e.y1, e.temp, e.numparticle) == (1, 20, 1, 30, 0, 5)
    assert (e.species_idx1, e.species_idx2) == (0, 1)


@pytest.mark.parametrize("name", ["conductors_64", "emitters_128", "gshybrid_64", "hybrid_24"])
def test_row_decks_parse(E, name, tmp_path):
    """The extension decks bench.py measures parse as the reference reads them, with the solver, walls,
    conductors and emitters they are meant to exercise, and agree with the oracle's set-up."""
    from epic2d_mcc_gb300 import workloads

    ini = decks.write(workloads.deck(name), str(tmp_path))
    cfg, descs, _ = E.config_from_ini(ini)
    s = O.setup(ini)
    assert (cfg.nx, cfg.ny) == (s.nx, s.ny) and cfg.DT == s.DT and len(descs) == 2
    gs, pcg, gshybrid, hybrid = 0, 1, 2, 3  # EPIC_SOLVER_* (include/epic2d.h)
    pbc, open_ = 0, 1                       # EPIC_PBC, EPIC_OPEN
    want = {"conductors_64": (gs, open_, 2, 0), "emitters_128": (pcg, open_, 0, 2),
            "gshybrid_64": (gshybrid, pbc, 0, 0), "hybrid_24": (hybrid, pbc, 0, 0)}[name]
    assert (cfg.solver, cfg.bc, len(E.conductors_from_ini(ini)), len(E.emitters_from_ini(ini))) == want
