"""Batched runs (include/epic2d_batch.h): every run of a batch gives the same
particles and potential, bit for bit, as the same run alone in the mixed form
(same configuration, sort period and device-loader seed) — on square and
non-square grids, periodic, reflective and absorbing walls, pcgsolver and
gssolver, conductors and emitters, with the step replayed from a graph or
launched directly, whatever launch shapes the autotuner chose for the GEMM
tiles and the particle passes."""
import numpy as np
import pytest

from tests import decks

pytestmark = pytest.mark.gpu

SPECS = [dict(nx=64, ny=64, ne=60000, ni=60000, solver="cg", tol="1e-10", maxit=100000, bc="pbc", te=1),
         dict(nx=48, ny=80, ne=50000, ni=40000, solver="cg", tol="1e-10", maxit=100000, bc="reflective", te=3),
         dict(nx=96, ny=40, ne=70000, ni=70000, solver="gs", tol="1e-8", bc="pbc", te=0.5),
         dict(nx=33, ny=33, ne=20000, ni=25000, solver="cg", tol="1e-10", maxit=100000, bc="pbc", te=2)]


def _requests(A, d, sort_every):
    out = []
    for k, sp in enumerate(SPECS):
        ini = decks.write(decks.deck(**sp), d)
        out.append((ini, A.make_request(ini, steps=0, seed=50 + k, precision=1, sort_every=sort_every)))
    return out


@pytest.mark.parametrize("graph", [True, False])
def test_batch_runs_equal_single_runs(gpu_lib, tmp_path, graph):
    A = gpu_lib.api
    sort_every, steps = 4, 10
    reqs = _requests(A, str(tmp_path), sort_every)
    b = A.Batch([r for _, r in reqs], sort_every=sort_every)
    assert all(t in (16, 32, 64) for t in b.tuning())
    b.initial_field()
    # the particle passes' launch shapes were timed on a sample and one kept
    sh = b.particle_tuning()
    assert sh["push_threads"] in (128, 256) and sh["deposit_threads"] in (128, 256)
    assert sh["push_blocks"] > 0 and sh["deposit_blocks"] > 0
    assert all(v > 0 for v in sh["push_ms_by_shape"].values())
    assert all(v > 0 for v in sh["deposit_ms_by_shape"].values())
    if not graph:  # the phase timers of directly launched steps (they change no result)
        b.set_profiling(True)
        b.profile()
    b.run(steps, graph=graph)
    if not graph:
        prof = b.profile()
        assert prof["push"][1] == steps and prof["solve"][1] == steps and prof["sort"][1] == (steps + 3) // 4
        assert all(prof[k][0] > 0 for k in ("push", "solve", "sort"))
    for k, (ini, r) in enumerate(reqs):
        sim = A.Simulation.from_ini(ini, precision=1, sort_every=sort_every)
        sim.load_particles_device(50 + k)
        sim.initial_field()
        sim.run(steps, graph=True)
        assert np.array_equal(b.grid(k, "phi"), sim.grid("phi")), k
        assert np.array_equal(b.grid(k, "rho"), sim.grid("rho")), k
        for s in range(2):
            assert np.array_equal(b.particles(k, s), sim.particles(s)), (k, s)
        sim.close()
    b.close()


def test_batch_rejects_unsupported_runs(gpu_lib, tmp_path):
    A = gpu_lib.api
    d = str(tmp_path)
    ok = A.make_request(decks.write(decks.deck(nx=32, ny=32, ne=1000, ni=1000), d), 0, precision=1)
    fp64 = A.make_request(decks.write(decks.deck(nx=32, ny=32, ne=1000, ni=1000), d), 0)
    with pytest.raises(A.EpicError):
        A.Batch([ok, fp64])


OPEN_SPECS = [dict(nx=48, ny=48, ne=50000, ni=50000, solver="cg", tol="1e-10", maxit=100000, bc="open", te=6),
              dict(nx=64, ny=40, ne=40000, ni=40000, solver="cg", tol="1e-10", maxit=100000, bc="pbc", te=2),
              dict(nx=40, ny=56, ne=30000, ni=30000, solver="gs", tol="1e-8", bc="open", te=4),
              dict(nx=32, ny=32, ne=20000, ni=20000, solver="cg", tol="1e-10", maxit=100000, bc="reflective", te=3)]


@pytest.mark.parametrize("graph", [True, False])
def test_batch_with_absorbing_walls_equals_single_runs(gpu_lib, tmp_path, graph):
    """Absorbing walls in a batch (src/species.cpp:100-112): the ordered compaction of the shared arrays keeps
    every run's survivors in their order, so each run — absorbing, periodic or reflective beside them — equals
    the same run alone bit for bit (particles, counts, rho, phi), with the cell sort on."""
    A = gpu_lib.api
    sort_every, steps = 4, 12
    d = str(tmp_path)
    reqs = []
    for k, sp in enumerate(OPEN_SPECS):
        ini = decks.write(decks.deck(**sp), d)
        reqs.append((ini, A.make_request(ini, steps=0, seed=70 + k, precision=1, sort_every=sort_every)))
    b = A.Batch([r for _, r in reqs], sort_every=sort_every)
    b.initial_field()
    n0 = b.num_particles()
    b.run(steps, graph=graph)
    assert b.num_particles() < n0  # particles left through the absorbing walls
    for k, (ini, r) in enumerate(reqs):
        sim = A.Simulation.from_ini(ini, precision=1, sort_every=sort_every)
        sim.load_particles_device(70 + k)
        sim.initial_field()
        sim.run(steps, graph=True)
        assert np.array_equal(b.grid(k, "phi"), sim.grid("phi")), k
        assert np.array_equal(b.grid(k, "rho"), sim.grid("rho")), k
        for s in range(2):
            assert np.array_equal(b.particles(k, s), sim.particles(s)), (k, s)
        sim.close()
    b.close()


EMIT_A = [dict(x0=1, y0=7, x1=1, y1=9, temp=0.1, numparticle=50, vdx=0.2, vdy=0, species_idx1=0, species_idx2=1),
          dict(x0=20, y0=3, x1=26, y1=12, temp=0.5, numparticle=40, vdx=0, vdy=0.1, species_idx1=1, species_idx2=1)]
EMIT_B = [dict(x0=30, y0=20, x1=34, y1=28, temp=1, numparticle=300, vdx=0, vdy=0, species_idx1=0, species_idx2=0)]


@pytest.mark.parametrize("walls", ["closed", "with_absorbing"])
@pytest.mark.parametrize("graph", [True, False])
def test_batch_with_emitters_equals_single_runs(gpu_lib, tmp_path, walls, graph):
    """Emitters in a batch (src/emitter.cpp:5-36, first in every step as src/main.cpp:397-403): each run's
    injections are the run alone's Philox draws (keyed by its own seed), appended after its other particles in
    its emitters' order, so every run — emitting or not — equals the same run alone bit for bit (particles,
    counts, rho, phi), with the cell sort on; with closed walls the injected particles are deposited into the
    accumulators the push left, beside an absorbing run the step deposits everything."""
    A = gpu_lib.api
    sort_every, steps = 4, 10
    open_bc = "open" if walls == "with_absorbing" else "pbc"
    specs = [(dict(nx=48, ny=32, ne=30000, ni=30000, solver="cg", tol="1e-10", maxit=100000, bc=open_bc, te=2),
              EMIT_A),
             (dict(nx=40, ny=40, ne=20000, ni=20000, solver="cg", tol="1e-10", maxit=100000, bc="pbc", te=1), []),
             (dict(nx=64, ny=48, ne=40000, ni=40000, solver="gs", tol="1e-8", bc="reflective", te=3), EMIT_B)]
    d = str(tmp_path)
    reqs = []
    for k, (sp, em) in enumerate(specs):
        ini = decks.write(decks.deck(emitters=em, **sp), d)
        reqs.append((ini, A.make_request(ini, steps=steps, seed=90 + k, precision=1, sort_every=sort_every)))
    assert [r.num_emitters for _, r in reqs] == [2, 0, 1]
    b = A.Batch([r for _, r in reqs], sort_every=sort_every)
    b.initial_field()
    n0 = b.num_particles()
    b.run(steps, graph=graph)
    if walls == "closed":  # 50 pairs + 40 ions + 300 electrons a step
        assert b.num_particles() == n0 + steps * (100 + 40 + 300)
    for k, (ini, r) in enumerate(reqs):
        sim = A.Simulation.from_ini(ini, precision=1, sort_every=sort_every)
        sim.load_particles_device(90 + k)
        sim.initial_field()
        sim.run(steps, graph=True)
        assert np.array_equal(b.grid(k, "phi"), sim.grid("phi")), k
        assert np.array_equal(b.grid(k, "rho"), sim.grid("rho")), k
        for s in range(2):
            assert np.array_equal(b.particles(k, s), sim.particles(s)), (k, s)
        sim.close()
    b.close()


GRIDS = [dict(type="reactconduct", min_x=10, max_x=12, min_y=4, max_y=16, grid_voltage=10),
         dict(type="circular", x_center=22, y_center=12, electrode_number=6, grid_radius=5, electrod_radius=1.5,
              electrode_voltage=-5)]


@pytest.mark.parametrize("graph", [True, False])
def test_batch_with_conductors_equals_single_runs(gpu_lib, tmp_path, graph):
    """Conductors in a batch (src/grid.cpp, src/electrode.cpp): a run with conductors is loaded by the host
    loader (positions inside a conductor drawn again, as the run alone with the same seed); its SOR solves get
    Grid::initialize's rho override (src/field.cpp:100-103), which also brings its electrodes into existence, its
    PCG solves do not; and the push erases, in order, the particles that end inside one. Every run (SOR and PCG
    with a rectangle and a ring, periodic, reflective and absorbing walls, one also emitting, and a plain run
    beside them) equals the same run alone bit for bit (particles, counts, rho, phi), with the cell sort on."""
    A = gpu_lib.api
    sort_every, steps = 4, 8
    specs = [(dict(nx=32, ny=24, ne=20000, ni=20000, solver="gs", tol="1e-6", bc="pbc", te=2, grids=GRIDS), []),
             (dict(nx=40, ny=40, ne=20000, ni=20000, solver="cg", tol="1e-10", maxit=100000, bc="pbc", te=1), []),
             (dict(nx=32, ny=24, ne=20000, ni=20000, solver="cg", tol="1e-10", maxit=100000, bc="reflective", te=2,
                   grids=GRIDS), []),
             (dict(nx=32, ny=24, ne=15000, ni=15000, solver="gs", tol="1e-6", bc="open", te=1, grids=GRIDS[:1]),
              EMIT_A)]
    d = str(tmp_path)
    reqs = []
    for k, (sp, em) in enumerate(specs):
        ini = decks.write(decks.deck(emitters=em, **sp), d)
        reqs.append((ini, A.make_request(ini, steps=steps, seed=110 + k, precision=1, sort_every=sort_every)))
    assert [r.num_conductors for _, r in reqs] == [2, 0, 2, 1]
    b = A.Batch([r for _, r in reqs], sort_every=sort_every)
    b.initial_field()
    b.run(steps, graph=graph)
    assert len(b.particles(0, 0)) < 20000  # electrons ended inside run 0's conductors
    for k, (ini, r) in enumerate(reqs):
        sim = A.Simulation.from_ini(ini, precision=1, sort_every=sort_every)
        if r.num_conductors:
            sim.load_particles(110 + k)
        else:
            sim.load_particles_device(110 + k)
        sim.initial_field()
        sim.run(steps, graph=True)
        assert np.array_equal(b.grid(k, "phi"), sim.grid("phi")), k
        assert np.array_equal(b.grid(k, "rho"), sim.grid("rho")), k
        for s in range(2):
            assert np.array_equal(b.particles(k, s), sim.particles(s)), (k, s)
        sim.close()
    b.close()


def test_batch_emitter_room_is_the_request_steps(gpu_lib, tmp_path):
    """A run's injections get room for its request's steps; running past it raises EPIC_ERR_CAPACITY (as a
    single run outgrowing its capacity) rather than writing past the arrays."""
    A = gpu_lib.api
    d = str(tmp_path)
    ini = decks.write(decks.deck(nx=32, ny=32, ne=2000, ni=2000, emitters=EMIT_A), d)
    b = A.Batch([A.make_request(ini, steps=2, seed=3, precision=1, sort_every=0)], sort_every=0)
    b.initial_field()
    with pytest.raises(A.EpicError) as ei:
        b.run(400, graph=False)
    assert ei.value.status == 4  # EPIC_ERR_CAPACITY
    b.close()


def _table():
    from epic2d_mcc_gb300 import workloads

    e, ela, exc, ion = workloads.synthetic_table()
    return ela, exc, ion, e[0], e[-1]


def test_batch_with_collisions(gpu_lib, tmp_path):
    # Colliding runs share the batch's launches: the collisionless runs of the
    # same batch stay bitwise equal to their single runs, and a colliding run
    # ionises at the single run's rate (statistically: its draws are keyed by
    # its place in the batch's array).
    A = gpu_lib.api
    d = str(tmp_path)
    sort_every, steps = 8, 24
    plain = dict(nx=64, ny=48, ne=50000, ni=50000, solver="cg", tol="1e-10", maxit=100000)
    hot = dict(nx=64, ny=64, ne=200000, ni=200000, solver="cg", tol="1e-10", maxit=100000, te=30, gas="1e22")
    ini_p = decks.write(decks.deck(**plain), d)
    ini_h = decks.write(decks.deck(collisions=True, **hot), d)
    reqs = [A.make_request(ini_p, 0, seed=7, precision=1, sort_every=sort_every),
            A.make_request(ini_h, 0, collisions=True, seed=8, precision=1, sort_every=sort_every)]
    b = A.Batch(reqs, sort_every=sort_every)
    b.set_log_cross_sections(*_table())
    b.initial_field()
    b.run(steps, graph=True)
    sim = A.Simulation.from_ini(ini_p, precision=1, sort_every=sort_every)
    sim.load_particles_device(7)
    sim.initial_field()
    sim.run(steps, graph=True)
    for s in range(2):
        assert np.array_equal(b.particles(0, s), sim.particles(s))
    sim.close()
    n0 = 200000
    grown_batch = len(b.particles(1, 0)) - n0
    assert len(b.particles(1, 1)) - n0 == grown_batch  # one ion per new electron
    grown = []
    for seed in (8, 9, 10):
        sim = A.Simulation.from_ini(ini_h, precision=1, sort_every=sort_every)
        sim.set_log_cross_sections(*_table())
        sim.load_particles_device(seed)
        sim.initial_field()
        sim.run(steps, collisions=True, graph=True)
        grown.append(sim.num_particles(0) - n0)
        sim.close()
    mean = float(np.mean(grown))
    assert mean > 20  # the deck ionises
    assert abs(grown_batch - mean) <= 6 * np.sqrt(mean) + 6
    b.close()
