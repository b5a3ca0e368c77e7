"""The serving loop and its building blocks on the GPU, through the C ABI.

* The device loader places particles inside the domain with the velocity
  moments of the reference's formula (v_th*sqrt(2)*(u1+u2+u3-1.5) + drift).
* A run's final state (epic_digest: phi and every particle array, bit for bit)
  and energies are the same when it is served alone and when it is served
  beside other runs that arrive while it is in flight.
* Admission keeps the resident estimate within the budget, rejects a run that
  can never fit, and runs a grid-barrier (FP64 PCG) run alone.
"""
import numpy as np
import pytest

from tests import decks

pytestmark = pytest.mark.gpu


def test_device_loader_moments(gpu_lib, tmp_path):
    A = gpu_lib.api
    ini = decks.write(decks.deck(nx=64, ny=48, ne=400000, ni=400000, te=2, vdrift=(0.5, -0.25)), str(tmp_path))
    for precision in (0, 1):
        sim = A.Simulation.from_ini(ini, precision=precision)
        sim.load_particles_device(7)
        cfg = sim.cfg
        for sp, d in enumerate(sim.species):
            p = sim.particles(sp)
            assert len(p) == d.numparticle
            Lx, Ly = (cfg.nx - 1) * cfg.dx, (cfg.ny - 1) * cfg.dy
            assert p[:, 0].min() >= cfg.x0 and p[:, 0].max() < cfg.x0 + Lx
            assert p[:, 1].min() >= cfg.y0 and p[:, 1].max() < cfg.y0 + Ly
            # uniform positions: mean L/2, variance L^2/12
            assert abs(p[:, 0].mean() - (cfg.x0 + Lx / 2)) < 5 * Lx / np.sqrt(12 * len(p))
            v_th = np.sqrt(2 * 1.380648e-23 * d.temp * (1.602176565e-19 / 1.380648e-23) / d.mass)
            sd = v_th / np.sqrt(2) / cfg.vel_norm  # sqrt(2 * 3/12) * v_th
            for c, drift in ((2, d.vsx), (3, d.vsy)):
                v = p[:, c]
                assert abs(v.mean() - drift) < 5 * sd / np.sqrt(len(v))
                assert abs(v.std() / sd - 1) < 0.01
            assert np.all(p[:, 4] == 0)
        sim.close()


def _requests(A, d, arrivals):
    reqs = []
    specs = [dict(nx=64, ny=64, ne=60000, ni=60000, solver="cg", tol="1e-10", maxit=100000, coll=True),
             dict(nx=48, ny=48, ne=40000, ni=40000, solver="gs", tol="1e-8", coll=False),
             dict(nx=96, ny=96, ne=90000, ni=90000, solver="cg", tol="1e-10", maxit=100000, coll=True, bc="open"),
             dict(nx=32, ny=32, ne=30000, ni=30000, solver="cg", tol="1e-10", maxit=100000, coll=False)]
    for k, t in enumerate(arrivals):
        s = dict(specs[k % len(specs)])
        coll = s.pop("coll")
        ini = decks.write(decks.deck(collisions=coll, **s), d)
        reqs.append(A.make_request(ini, steps=24 + 8 * k, collisions=coll, seed=100 + k, arrival_s=t,
                                   precision=1, sort_every=8))
    return reqs


def _table():
    from epic2d_mcc_gb300 import workloads

    e, ela, exc, ion = workloads.synthetic_table()
    return ela, exc, ion, e[0], e[-1]


def test_same_result_alone_and_in_the_mix(gpu_lib, tmp_path):
    A = gpu_lib.api
    d = str(tmp_path)
    reqs = _requests(A, d, [0.0, 0.002, 0.004, 0.006, 0.008, 0.010])
    srv = A.Server(budget_bytes=8 << 30, max_inflight=4, chunk_steps=8)
    srv.set_log_cross_sections(*_table())
    ids = [srv.submit(r) for r in reqs]
    srv.start()
    srv.wait(300)
    mix = [srv.result(i) for i in ids]
    st = srv.stats()
    srv.close()
    assert st.completed == len(reqs) and st.failed == 0
    assert st.peak_inflight >= 2  # runs overlapped
    assert 0 < st.p50_latency_s <= st.p99_latency_s
    for k, r in enumerate(reqs):
        alone = A.Server(budget_bytes=8 << 30, max_inflight=1, chunk_steps=5)
        alone.set_log_cross_sections(*_table())
        r.arrival_s = 0.0
        i = alone.submit(r)
        alone.start()
        alone.wait(300)
        a = alone.result(i)
        alone.close()
        assert mix[k].status == 0 and a.status == 0
        assert tuple(a.digest) == tuple(mix[k].digest), k
        assert a.kinetic_energy == mix[k].kinetic_energy and a.potential_energy == mix[k].potential_energy


def test_served_run_equals_the_plain_api(gpu_lib, tmp_path):
    A = gpu_lib.api
    ini = decks.write(decks.deck(nx=64, ny=64, ne=60000, ni=60000, solver="cg", tol="1e-10", maxit=100000,
                                 collisions=True), str(tmp_path))
    req = A.make_request(ini, steps=30, collisions=True, seed=5, precision=1, sort_every=8)
    srv = A.Server(budget_bytes=4 << 30, max_inflight=2, chunk_steps=7)
    srv.set_log_cross_sections(*_table())
    i = srv.submit(req)
    srv.start()
    srv.wait(300)
    res = srv.result(i)
    srv.close()
    sim = A.Simulation.from_ini(ini, precision=1, sort_every=8)
    ela, exc, ion, e0, e1 = _table()
    sim.set_log_cross_sections(ela, exc, ion, e0, e1)
    sim.load_particles_device(5)
    sim.initial_field()
    sim.run(30, collisions=True, graph=True)
    assert sim.digest() == tuple(res.digest)


@pytest.mark.parametrize("precision", [0, 1])
def test_served_conductors_and_emitters_equal_the_plain_api(gpu_lib, tmp_path, precision):
    """A request carries its deck's [Grids] and [Emitters]: loaded on the host
    around the conductors, with room for the injections, and stepped in chunks
    beside another run, it ends bit for bit where the plain API ends."""
    A = gpu_lib.api
    grids = [dict(type="reactconduct", min_x=10, max_x=12, min_y=4, max_y=16, grid_voltage=10),
             dict(type="circular", x_center=40, y_center=30, electrode_number=6, grid_radius=6,
                  electrod_radius=1.5, electrode_voltage=-5)]
    em = [dict(x0=2, y0=20, x1=2, y1=30, temp=0.5, numparticle=400, vdx=0.2, vdy=0, species_idx1=0,
               species_idx2=1)]
    ini = decks.write(decks.deck(nx=64, ny=48, ne=20000, ni=20000, te=1, bc="open", solver="gs", tol="1e-8",
                                 grids=grids, emitters=em), str(tmp_path))
    steps = 40
    req = A.make_request(ini, steps=steps, seed=9, precision=precision)
    assert req.num_conductors == 2 and req.num_emitters == 1
    other = A.make_request(ini, steps=12, seed=3, precision=1)
    other.num_conductors = other.num_emitters = 0
    srv = A.Server(budget_bytes=4 << 30, max_inflight=2, chunk_steps=7)
    i = srv.submit(req)
    srv.submit(other)
    srv.start()
    srv.wait(300)
    res = srv.result(i)
    srv.close()
    assert res.status == 0
    # the server's capacity: the default plus the emitter's particles over the run
    sim = A.Simulation.from_ini(ini, precision=precision, capacity=20000 + 10000 + 4096 + 400 * steps)
    sim.load_particles(9)
    sim.initial_field()
    sim.run(steps, graph=True)
    assert sim.num_particles(1) > 20000 + 400 * steps // 2  # the emitter fed the ions
    assert sim.digest() == tuple(res.digest)


def test_admission_budget_exclusive_and_rejection(gpu_lib, tmp_path):
    A = gpu_lib.api
    d = str(tmp_path)
    ini = decks.write(decks.deck(nx=64, ny=64, ne=100000, ni=100000, solver="cg", tol="1e-10", maxit=100000), d)
    r = A.make_request(ini, steps=20, precision=1, sort_every=8)
    est = A.estimate_bytes(r)
    budget = int(2.5 * est)
    srv = A.Server(budget_bytes=budget, max_inflight=8, chunk_steps=4)
    ids = []
    for k in range(5):
        r.arrival_s = 0.001 * k
        r.load_seed = k
        ids.append(srv.submit(r))
    # FP64 PCG: grid-wide barriers, so it must run alone
    excl = A.make_request(ini, steps=10, arrival_s=0.0025)
    ids.append(srv.submit(excl))
    # larger than the whole budget: rejected
    huge_ini = decks.write(decks.deck(nx=64, ny=64, ne=3000000, ni=3000000), d)
    huge = A.make_request(huge_ini, steps=1, precision=1, arrival_s=0.01)
    assert A.estimate_bytes(huge) > budget
    hid = srv.submit(huge)
    srv.start()
    srv.wait(300)
    st = srv.stats()
    res = [srv.result(i) for i in ids]
    hres = srv.result(hid)
    srv.close()
    assert st.peak_bytes <= budget and st.peak_inflight <= 2
    assert all(x.status == 0 for x in res)
    assert hres.status == 8  # EPIC_ERR_BUDGET
    ex = res[-1]
    for x in res[:-1]:
        # no overlap with the exclusive run
        assert x.finish_s <= ex.admit_s or x.admit_s >= ex.finish_s
