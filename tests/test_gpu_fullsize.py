"""Parity at the sizes the benchmarks run, through the C ABI, against the oracle.

* beam_mcc_256 (257 x 257 nodes, 13.1 M particles in three species, PCG to
  1e-10, MCC with the synthetic 1000-point log table): the loader, the
  prologue and one loop iteration, phase by phase.  Each phase gets the same
  inputs on both sides (the oracle's), so each comparison isolates one kernel:
  densities and rho within 1e-12 relative; the PCG iteration count equal to
  the oracle's and phi within 1e-12 (no relaxation when the counts differ:
  the test fails and reports both counts); rho within 1e-12 of the largest
  sum of |charge density| it is formed from (rho nearly cancels); the
  E-field bit for bit; the
  rewound and pushed particles within 1e-12; the MCC draw for draw on
  injected uniforms (same collision count, particles within 1e-12, appended
  ions in the same order).
* periodic_64 (64 x 64 cells, 409,600 particles, SOR with omega 1.8 to 1e-8,
  CIC, periodic): 50 free-running loop iterations on both sides; every SOR
  solve takes the oracle's iteration count, and after 50 steps phi and the
  particles still agree within 1e-10 relative (the two runs differ only in
  the rounding of the fixed-point deposit, ~2^-38 of a particle's weight, and
  the contracted push, a few ulps, so the trajectories separate slowly).
* the lexicographic SOR on 200^2 and 256^2 cells (the clustered wavefront,
  undrained with snapshots and drained): the oracle's iterates bit for bit.
"""
import os

import numpy as np
import pytest

from epic2d_mcc_gb300 import workloads
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def parts_rel(a, b):
    assert a.shape == b.shape, (a.shape, b.shape)
    return max(rel(a[:, c], b[:, c]) for c in range(5)) if len(b) else 0.0


def _deck(tmp_path, name):
    path = os.path.join(str(tmp_path), name + ".ini")
    with open(path, "w") as f:
        f.write(workloads.deck(name))
    return path


def test_beam_mcc_256_one_iteration_matches_oracle(gpu_lib, tmp_path):
    E = gpu_lib
    ini = _deck(tmp_path, "beam_mcc_256")
    orc = O.OracleSim(ini, initial_field=False)
    e_grid, ela, exc, ion = workloads.synthetic_table()
    orc.R.set_log_table(ela, exc, ion, e_grid[0], e_grid[-1])
    sim = E.Simulation.from_ini(ini, mcc_mode=1)
    sim.set_log_cross_sections(ela, exc, ion, e_grid[0], e_grid[-1])
    sim.load_particles(0)
    nsp = len(orc.parts)
    assert nsp == 3 and sum(len(p) for p in orc.parts) == 13107200
    for s in range(nsp):
        assert np.array_equal(sim.particles(s), orc.parts[s]), "the loader reproduces Init exactly"
    sp = orc.s.species

    def field_phase(label):
        # scatter + rho
        orc.scatter_all()
        for s in range(nsp):
            sim.scatter_species(s)
            assert rel(sim.den(s), orc.den[s]) < TOL, "%s den%d" % (label, s)
        sim.compute_rho()
        # rho is a near-cancelling sum of the species' charge densities (max |rho| ~ 0.15 of a
        # density): its error is measured against the size of the terms it is summed from.
        terms = sum(np.abs(orc.den[s] * (sp[s].charge / O.QE)) for s in range(nsp))
        assert np.max(np.abs(sim.grid("rho") - orc.rho)) < TOL * np.max(terms), label + " rho"
        # PCG on the same rho
        sim.set_grid("rho", orc.rho)
        it, err, conv = sim.potential_solver()
        phi_o, err_o, it_o, conv_o = orc.R.pcg_solve(orc.rho)
        orc.phi, orc.error, orc.iters = phi_o, err_o, it_o
        assert conv and conv_o
        assert it == it_o, "%s: PCG took %d iterations, the oracle %d" % (label, it, it_o)
        assert rel(sim.grid("phi"), phi_o) < TOL, label + " phi"
        # E-field of the same phi, bit for bit
        sim.set_grid("phi", phi_o)
        sim.calculate_efield()
        orc.efx, orc.efy = orc.R.efield(phi_o)
        assert np.array_equal(sim.grid("efx"), orc.efx) and np.array_equal(sim.grid("efy"), orc.efy), label + " E"

    field_phase("prologue")
    for s in range(nsp):
        sim.rewind_species(s)
        orc.parts[s] = orc.R.rewind(sp[s], orc.parts[s], orc.efx, orc.efy)
        assert parts_rel(sim.particles(s), orc.parts[s]) < TOL, "rewind %d" % s
        sim.set_particles(s, orc.parts[s])
    field_phase("step 1")
    for s in range(nsp):
        sim.push_species(s)
        orc.parts[s] = orc.R.push(sp[s], orc.parts[s], orc.efx, orc.efy)
        got = sim.particles(s)
        assert parts_rel(got, orc.parts[s]) < TOL, "push %d" % s
        sim.set_particles(s, orc.parts[s])  # same inputs for the MCC
    U = np.random.default_rng(11).random((len(orc.parts[0]), 16))
    e, i, nc, kinds = orc.R.mcc(orc.parts[0], orc.parts[1], sp[1], uniforms=U)
    got = sim.handle_collisions(0, 1, uniforms=U)
    assert nc > 1000 and got == nc, (got, nc)
    ge, gi = sim.particles(0), sim.particles(1)
    assert len(ge) == len(e) and len(gi) == len(i)
    assert parts_rel(ge, e) < TOL
    assert parts_rel(gi, i) < TOL


def test_periodic_64_sor_omega_18_fifty_steps_track_oracle(gpu_lib, tmp_path):
    E = gpu_lib
    ini = _deck(tmp_path, "periodic_64")
    orc = O.OracleSim(ini)
    assert orc.s.sor_omega == 1.8 and orc.s.tolerance == 1e-8 and orc.s.solver == "gs"
    sim = E.Simulation.from_ini(ini)
    sim.load_particles(0)
    sim.initial_field()
    assert rel(sim.grid("phi"), orc.phi) < TOL
    nsp = len(orc.parts)
    iters = []
    for k in range(50):
        orc.scatter_all()
        orc.field()
        orc.push_all()
        for s in range(nsp):
            sim.scatter_species(s)
        sim.compute_rho()
        it, err, conv = sim.potential_solver()
        assert conv and it == orc.iters, "step %d: SOR took %d sweeps, the oracle %d" % (k + 1, it, orc.iters)
        iters.append(it)
        sim.calculate_efield()
        for s in range(nsp):
            sim.push_species(s)
    assert min(iters) > 25
    assert rel(sim.grid("phi"), orc.phi) < 1e-10
    for s in range(nsp):
        assert parts_rel(sim.particles(s), orc.parts[s]) < 1e-10


@pytest.mark.parametrize("n", [200, 256])
def test_large_lattice_sor_is_iterate_exact(gpu_lib, tmp_path, n):
    """The clustered lexicographic SOR on large lattices: 200^2 cells runs the
    undrained wavefront with eight snapshot bands per CTA (rho K read from
    global memory to make room), 256^2 (whose snapshots do not fit) drains at
    every check.  Capped at 60 sweeps, and
    converging at the check after sweep 275 (a tolerance just above the
    oracle's residual there): the oracle's iteration count and phi bit for
    bit."""
    from tests import decks

    d = str(tmp_path)
    ini = decks.write(decks.deck(nx=n, ny=n, ne=n * n * 4, ni=n * n * 4, solver="gs", tol="1e-30", maxit=276), d)
    orc = O.OracleSim(ini, initial_field=False)
    orc.scatter_all()
    phi275, err275, it_o, conv_o = orc.R.gs_solve(orc.rho)
    assert it_o == 276 and not conv_o
    cases = [("1e-30", 60, 60, False), (repr(err275 * 1.0001), 400, 276, True)]
    for tol, maxit, it_want, conv_want in cases:
        ini = decks.write(decks.deck(nx=n, ny=n, ne=n * n * 4, ni=n * n * 4, solver="gs", tol=tol, maxit=maxit), d)
        o = O.OracleSim(ini, initial_field=False)
        o.scatter_all()
        phi_o, err_o, it_o, conv_o = o.R.gs_solve(o.rho)
        assert it_o == it_want and bool(conv_o) == conv_want
        sim = gpu_lib.Simulation.from_ini(ini)
        sim.set_grid("rho", o.rho)
        it, err, conv = sim.potential_solver()
        assert it == it_o and bool(conv) == conv_want
        assert np.array_equal(sim.grid("phi"), phi_o)
        if conv_want:
            assert np.array_equal(phi_o, phi275)
        sim.close()
