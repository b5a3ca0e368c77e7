"""Conductors (the reference's Grid objects: ReactConductorGrid rectangles and
CircularGrid rings of electrodes, src/grid.cpp, src/electrode.cpp) on the GPU
against the oracle: Init's rejection of positions inside a conductor
(src/init.cpp:71-86), the rho override before every SOR solve
(src/field.cpp:100-103), and the ordered erasure of particles that end a push
inside one (src/species.cpp:80-165).  tests/golden/conductors_gs_pbc.npz pins
the same against the reference's own outputs (test_gpu_parity)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu

TOL = 1e-12
GRIDS = [dict(type="reactconduct", min_x=10, max_x=12, min_y=4, max_y=16, grid_voltage=10),
         dict(type="circular", x_center=22, y_center=12, electrode_number=6, grid_radius=5, electrod_radius=1.5,
              electrode_voltage=-5)]


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)) if b.size else 0.0


@pytest.mark.parametrize("bc,solver", [("pbc", "gs"), ("open", "gs"), ("reflective", "gs"), ("pbc", "cg")])
def test_conductors_track_oracle(gpu_lib, tmp_path, bc, solver):
    tol = "1e-8" if solver == "gs" else "1e-10"
    ini = decks.write(decks.deck(nx=32, ny=24, ne=3000, ni=3000, te=4, bc=bc, solver=solver, tol=tol, grids=GRIDS),
                      str(tmp_path))
    orc = O.OracleSim(ini)
    sim = gpu_lib.Simulation.from_ini(ini)
    sim.load_particles(0)
    sim.initial_field()
    for s in range(2):
        assert rel(sim.particles(s), orc.parts[s]) < TOL
    assert rel(sim.grid("rho"), orc.rho) < TOL
    for _ in range(4):
        orc.step()
        sim.step()
        for s in range(2):
            got = sim.particles(s)
            assert len(got) == len(orc.parts[s])
            assert rel(got, orc.parts[s]) < TOL
        assert rel(sim.grid("rho"), orc.rho) < TOL
        assert rel(sim.grid("phi"), orc.phi) < TOL
    assert len(orc.parts[0]) < 3000  # particles were erased
    # graph replay of further steps equals step-by-step
    sim2 = gpu_lib.Simulation.from_ini(ini)
    sim2.load_particles(0)
    sim2.initial_field()
    for _ in range(4):
        sim2.step()
    sim.run(3, graph=True)
    for _ in range(3):
        sim2.step()
    for s in range(2):
        assert np.array_equal(sim.particles(s), sim2.particles(s))
    sim.close()
    sim2.close()


def test_conductors_rules(gpu_lib, tmp_path):
    # the device loader keeps particles out of the conductor rectangles as Init does (src/init.cpp:71-86: a
    # random position inside one is drawn again; the rings have no electrodes before the first SOR solve)
    ini = decks.write(decks.deck(nx=32, ny=24, ne=4000, ni=4000, grids=GRIDS), str(tmp_path))
    r = GRIDS[0]
    sims = []
    for seed in (1, 1, 2):
        sim0 = gpu_lib.Simulation.from_ini(ini)
        sim0.load_particles_device(seed)
        sim0.initial_field()
        p = [sim0.particles(s) for s in range(2)]
        for q in p:
            assert len(q) == 4000
            inside = (q[:, 0] >= r["min_x"]) & (q[:, 0] <= r["max_x"]) & (q[:, 1] >= r["min_y"]) & (q[:, 1] <= r["max_y"])
            assert not inside.any()
        sims.append(p)
        sim0.close()
    assert all(np.array_equal(a, b) for a, b in zip(sims[0], sims[1]))  # same seed, same particles
    assert not np.array_equal(sims[0][0], sims[2][0])
    # a deterministic load type that puts a particle inside a conductor (the reference loops forever): both
    # loaders refuse it
    text = decks.deck(nx=32, ny=24, ne=1024, ni=1024, grids=GRIDS).replace(",random", ",uniform")
    ini2 = decks.write(text, str(tmp_path))
    sim = gpu_lib.Simulation.from_ini(ini2)
    with pytest.raises(gpu_lib.EpicError):
        sim.load_particles(0)
    sim.close()
    sim = gpu_lib.Simulation.from_ini(ini2)
    with pytest.raises(gpu_lib.EpicError) as ei:  # from the load itself or the next synchronising call
        sim.load_particles_device(0)
        sim.initial_field()
    assert ei.value.status == 1  # EPIC_ERR_INVALID
    sim.close()


def test_step_host_with_conductors(gpu_lib, tmp_path):
    ini = decks.write(decks.deck(nx=32, ny=24, ne=3000, ni=3000, te=4, solver="gs", tol="1e-8", grids=GRIDS),
                      str(tmp_path))
    a, b = (gpu_lib.Simulation.from_ini(ini) for _ in range(2))
    for s_ in (a, b):
        s_.load_particles(0)
        s_.initial_field()
    bufs = [np.zeros((4000, 5)) for _ in range(2)]
    counts = [a.particles_into(k, bufs[k]) for k in range(2)]
    for _ in range(3):
        counts = a.step_host(bufs, counts)
        b.step()
    for k in range(2):
        assert np.array_equal(bufs[k][:counts[k]], b.particles(k))
    a.close()
    b.close()
