"""Mixed-precision form against the FP64 oracle.

Stated errors (relative, max |a-b| / max |b|):
* layout round trip: positions to FP32 in-cell resolution (<= 2^-23 cell),
  velocities to FP32 rounding (<= 2^-24);
* density: <= 1e-5 (offsets quantised to 2^-20 of a cell for the integer weights);
* potential from the FP64-refined solve: <= 1e-5 against a tightly converged
  FP64 solution, with the reference's own stopping norm below its tolerance;
* one full step and ten steps: potential <= 1e-5, total energy <= 1e-5.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    assert a.shape == b.shape
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def mixed_sim(E, ini, **over):
    return E.Simulation.from_ini(ini, precision=1, **over)


def test_mixed_layout_round_trip(gpu_lib, tmp_path):
    ini = decks.write(decks.deck(nx=64, ny=48, ne=50000, ni=50000, te=4), str(tmp_path))
    orc = O.OracleSim(ini)
    sim = mixed_sim(gpu_lib, ini)
    for s in range(2):
        sim.set_particles(s, orc.parts[s])
        got = sim.particles(s)
        assert np.max(np.abs(got[:, 0] - orc.parts[s][:, 0])) <= 2.0 ** -23 * orc.s.dx
        assert np.max(np.abs(got[:, 1] - orc.parts[s][:, 1])) <= 2.0 ** -23 * orc.s.dy
        assert rel(got[:, 2:], orc.parts[s][:, 2:]) <= 2.0 ** -24


@pytest.mark.parametrize("bc", ["pbc", "open", "reflective"])
@pytest.mark.parametrize("shape", ["CIC", "NGP"])
def test_mixed_deposit(gpu_lib, tmp_path, bc, shape):
    ini = decks.write(decks.deck(nx=48, ny=40, ne=60000, ni=60000, bc=bc, shape=shape), str(tmp_path))
    orc = O.OracleSim(ini)
    sim = mixed_sim(gpu_lib, ini)
    for s in range(2):
        sim.set_particles(s, orc.parts[s])
    dens = [orc.R.scatter(orc.parts[s], orc.s.species[s].spwt) for s in range(2)]
    for s in range(2):
        sim.scatter_species(s)
        assert rel(sim.den(s), dens[s]) < 1e-5
    sim.compute_rho()
    rho = orc.R.compute_rho(dens, [sp.charge for sp in orc.s.species])
    assert np.max(np.abs(sim.grid("rho") - rho)) < 1e-5 * np.max(np.abs(dens[0]))


@pytest.mark.parametrize("solver", ["cg", "gs"])
@pytest.mark.parametrize("n", [32, 64, 128])
def test_mixed_spectral_solve(gpu_lib, tmp_path, solver, n):
    ini = decks.write(decks.deck(nx=n, ny=n, ne=n * n * 4, ni=n * n * 4, solver=solver, tol="1e-10",
                                 maxit=200000), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    orc.scatter_all()
    sim = mixed_sim(gpu_lib, ini)
    sim.set_grid("rho", orc.rho)
    it, err, conv = sim.potential_solver()
    assert conv and 1 <= it <= 5
    if solver == "cg":
        d = orc.R.d
        d.tolerance = 1e-13
        exact, _, _, _ = orc.R.pcg_solve(orc.rho)
        assert err * (n + 1) ** 2 < 1e-10  # |Ax - b| / n, the reference's error figure
    else:
        d = orc.R.d
        d.tolerance = 1e-13
        exact, _, _, _ = orc.R.gs_solve(orc.rho, 1.9)
        assert err < 1e-10  # SOR residual L2
    assert rel(sim.grid("phi"), exact) < 1e-5


@pytest.mark.parametrize("n, bc", [(833, "dirichlet"), (803, "dirichlet"), (833, "periodic")])
def test_mixed_spectral_solve_large_lattice(gpu_lib, tmp_path, n, bc):
    """Lattices with a 64 x 64 output tile for every SM take the register-blocked products (803: lengths
    that are not multiples of 4, the guarded scalar loads): the solve converges within a few stages and its
    FP64 residual meets the tolerance.  On the periodic lattice phi also agrees with a tightly converged
    FP64 PCG solve of the same rho (on the reference's flattened lattice the PCG's iteration cap, n * n in
    32-bit arithmetic as in the reference, wraps at this size)."""
    E = gpu_lib
    extra = "" if bc == "dirichlet" else "poisson_bc = periodic\n"
    ini = decks.write(decks.deck(nx=n, ny=n, ne=1000, ni=1000, solver="cg", tol="1", maxit=1000000,
                                 solver_extra=extra), str(tmp_path))
    s = O.setup(ini)
    N = s.nx  # nodes per side (the deck counts cells)
    x = np.linspace(0, 1, N)
    rho = (np.sin(3 * np.pi * x)[:, None] * np.cos(2 * np.pi * x)[None, :]).ravel()
    rho += 0.1 * np.random.default_rng(5).normal(size=N * N)
    bnorm = np.linalg.norm(rho) * s.dx * s.dx * (s.L / s.LDe) ** 2
    tol = 1e-9 * bnorm  # relative 1e-9: well above the FP64 rounding floor of |b - A x| at this size
    mx = mixed_sim(E, ini, tolerance=tol)
    mx.set_grid("rho", rho)
    it, err, conv = mx.potential_solver()
    assert conv and 1 <= it <= 4, (it, err * N * N / bnorm)
    assert err * N * N < tol  # |b - A x|_2 (the reported error is that over nx ny)
    if bc == "periodic":
        ref = E.Simulation.from_ini(ini, tolerance=0.05 * tol)
        ref.set_grid("rho", rho)
        assert ref.potential_solver()[2]
        assert rel(mx.grid("phi"), ref.grid("phi")) < 1e-5


@pytest.mark.parametrize("n, bc, solver", [(1024, "periodic", "cg"), (512, "dirichlet_x", "cg"), (512, "dirichlet", "gs"),
                                           (510, "dirichlet", "cg")])
def test_mixed_spectral_solve_fft_lattice(gpu_lib, tmp_path, n, bc, solver):
    """Lattices with a side of 512 or more unknowns whose sides allow it take FFT passes instead of the
    dense products: the Hartley transform of a periodic direction (1024 or 512 points), the sine transform
    of a Dirichlet one by the odd extension (2 x 512 points; pcgsolver's flattened lattice of all 511 x 511
    nodes included).  The solve converges within a few stages to the reference's stopping norm, and phi
    agrees within 1e-6 with the FP64 solution of the same rho: a tightly converged FP64 PCG on the periodic
    and x-Dirichlet lattices, the exact discrete solution by orthonormal DST-I in FP64 (scipy) on the
    Dirichlet lattices (pcgsolver's own iteration cap, n * n in 32-bit arithmetic, wraps at that size)."""
    E = gpu_lib
    extra = "" if bc == "dirichlet" else "poisson_bc = %s\n" % bc
    ini = decks.write(decks.deck(nx=n, ny=n, ne=1000, ni=1000, solver=solver, tol="1", maxit=1000000,
                                 solver_extra=extra), str(tmp_path))
    s = O.setup(ini)
    N = s.nx
    x = np.linspace(0, 1, N)
    rho = (np.sin(3 * np.pi * x)[:, None] * np.cos(2 * np.pi * x)[None, :]).ravel()
    rho += 0.1 * np.random.default_rng(7).normal(size=N * N)
    K = (s.L / s.LDe) ** 2
    if solver == "cg":
        bnorm = np.linalg.norm(rho) * s.dx * s.dx * K
        tol = 1e-9 * bnorm
    else:
        tol = 1e-9 * np.sqrt(np.sum((rho * K) ** 2) / (N * N))  # the SOR residual's norm, relative 1e-9
    mx = mixed_sim(E, ini, tolerance=tol)
    mx.set_grid("rho", rho)
    it, err, conv = mx.potential_solver()
    assert conv and 1 <= it <= 4, (it, err)
    phi = mx.grid("phi")
    if solver == "cg" and bc != "dirichlet":
        ref = E.Simulation.from_ini(ini, tolerance=0.05 * tol)
        ref.set_grid("rho", rho)
        assert ref.potential_solver()[2]
        want = ref.grid("phi")
    else:
        from scipy import fft as sfft

        # A phi = b with b = -rho K dx^2 (dx = dy): on the interior with phi = 0 on the edges (gssolver), or
        # on every node of the flattened lattice with b zero on the grid edges (pcgsolver, src/field.cpp:240-251)
        rr = rho.reshape(N, N)
        if solver == "gs":
            b = -(rr[1:-1, 1:-1] * K) * s.dx * s.dx
        else:
            b = -(rr * K) * s.dx * s.dx
            b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = 0.0
        m = b.shape[0]
        lam = -4.0 * np.sin(np.pi * np.arange(1, m + 1) / (2.0 * (m + 1))) ** 2
        inner = sfft.dstn(sfft.dstn(b, type=1, norm="ortho") / (lam[:, None] + lam[None, :]), type=1, norm="ortho")
        if solver == "gs":
            want = np.zeros((N, N))
            want[1:-1, 1:-1] = inner
            want = want.ravel()
        else:
            want = inner.ravel()
    assert rel(phi, want) < 1e-6


@pytest.mark.parametrize("solver", ["cg", "gs"])
@pytest.mark.parametrize("shape", [(64, 40), (40, 72), (97, 33)])
def test_mixed_spectral_solve_rectangular(gpu_lib, tmp_path, solver, shape):
    # Non-square grids: pcgsolver's lattice is the flattened vector in rows of nx
    # (not the physical grid); gssolver's is the physical interior.
    nx, ny = shape
    ini = decks.write(decks.deck(nx=nx, ny=ny, ne=nx * ny * 4, ni=nx * ny * 4, solver=solver, tol="1e-10",
                                 maxit=400000), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    orc.scatter_all()
    sim = mixed_sim(gpu_lib, ini)
    sim.set_grid("rho", orc.rho)
    it, err, conv = sim.potential_solver()
    assert conv and 1 <= it <= 5
    orc.R.d.tolerance = 1e-13
    exact = orc.R.pcg_solve(orc.rho)[0] if solver == "cg" else orc.R.gs_solve(orc.rho, 1.9)[0]
    assert rel(sim.grid("phi"), exact) < 1e-5


def test_mixed_one_step_vs_fp64(gpu_lib, tmp_path):
    ini = decks.write(decks.deck(nx=64, ny=64, ne=100000, ni=100000, solver="cg", tol="1e-10"), str(tmp_path))
    orc = O.OracleSim(ini)
    sim = mixed_sim(gpu_lib, ini)
    for s in range(2):
        sim.set_particles(s, orc.parts[s])
    orc.step()
    sim.step()
    assert rel(sim.grid("phi"), orc.phi) < 1e-5
    assert rel(sim.grid("efx"), orc.efx) < 1e-4
    for s in range(2):
        got = sim.particles(s)
        assert np.max(np.abs(got[:, 0] - orc.parts[s][:, 0])) < 1e-5
        assert rel(got[:, 2:4], orc.parts[s][:, 2:4]) < 1e-5


def test_mixed_energy_tracks_fp64(gpu_lib, tmp_path):
    """Ten loop iterations from the same start: total energy within 1e-5."""
    ini = decks.write(decks.deck(nx=64, ny=64, ne=100000, ni=100000, solver="cg", tol="1e-10"), str(tmp_path))
    orc = O.OracleSim(ini)
    sim = mixed_sim(gpu_lib, ini)
    sim.load_particles(0)
    sim.initial_field()
    for _ in range(10):
        orc.step()
        sim.step()
    norm = orc.s.species[0]
    ke_o = sum(orc.R.ke(sp, orc.parts[k], norm).sum() for k, sp in enumerate(orc.s.species))
    pe_o = orc.R.pe(orc.efx, orc.efy, norm)
    ke_g = sum(sim.compute_ke(k, 0).sum() for k in range(2))
    pe_g = sim.compute_pe(0)
    assert abs((ke_g + pe_g) - (ke_o + pe_o)) < 1e-5 * (ke_o + pe_o)
    assert rel(sim.grid("phi"), orc.phi) < 1e-4


def test_mixed_open_boundary_and_mcc(gpu_lib, tmp_path):
    kw = dict(nx=32, ny=32, ne=30000, ni=30000, te=30, ion_mass="6.63352090e-26", collisions=True, gas="1e22",
              bc="open", dt=0.05)
    ini = decks.write(decks.deck(**kw), str(tmp_path))
    orc = O.OracleSim(ini)
    orc.step()
    sim = mixed_sim(gpu_lib, ini, mcc_mode=1)
    sim.set_reference_cross_sections()
    for s in range(2):
        sim.set_particles(s, orc.parts[s])
    U = np.random.default_rng(7).random((len(orc.parts[0]), 16))
    e, i, nc, kinds = orc.R.mcc(orc.parts[0], orc.parts[1], orc.s.species[1], uniforms=U)
    got = sim.handle_collisions(0, 1, uniforms=U)
    assert abs(got - nc) <= 2 and nc > 100
    ge = sim.particles(0)
    assert abs(len(ge) - len(e)) <= 2
    # push with open walls: same survivors as the FP64 oracle
    ex = np.random.default_rng(8).normal(size=orc.efx.shape)
    sim.set_grid("efx", ex)
    sim.set_grid("efy", ex)
    ref = orc.R.push(orc.s.species[1], i, ex, ex)
    sim.push_species(1)
    assert abs(sim.num_particles(1) - len(ref)) <= 2


def test_mixed_upload_keeps_particles_by_the_far_walls(gpu_lib, tmp_path):
    """A particle a hair inside the far walls, whose FP32 offset in the last cell rounds up to 1, stays in the
    last cell at the largest offset below 1 (2^-24 cell from the wall); one on the wall itself is outside the
    grid, as for the reference's deposit."""
    E = gpu_lib
    ini = decks.write(decks.deck(nx=32, ny=24, ne=100, ni=100), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    s = orc.s
    sim = mixed_sim(E, ini)
    e = orc.parts[0].copy()
    far_x, far_y = s.x0 + s.Lx * (1 - 2.0 ** -40), s.y0 + s.Ly * (1 - 2.0 ** -40)
    e[0, :2] = far_x, far_y
    e[1, 0] = far_x
    e[2, 1] = far_y
    sim.set_particles(0, e)
    got = sim.particles(0)
    for k, c, far, L in ((0, 0, far_x, s.Lx), (0, 1, far_y, s.Ly), (1, 0, far_x, s.Lx), (2, 1, far_y, s.Ly)):
        d = s.dx if c == 0 else s.dy
        assert s.x0 + L - 2.0 ** -23 * d < got[k, c] < s.x0 + L, (k, c)
    sim.set_particles(1, orc.parts[1])
    sim.scatter_species(0)
    assert rel(sim.den(0), orc.R.scatter(e, s.species[0].spwt)) < 1e-5
    e[3, 0] = s.x0 + s.Lx
    with pytest.raises(E.EpicError) as ei:
        sim.set_particles(0, e)
    assert ei.value.status == 6  # EPIC_ERR_DOMAIN


def test_set_grid_refuses_arrays_of_another_size(gpu_lib, tmp_path):
    """The C entry point copies nx * ny values: the Python API refuses an array of another size (a deck's Nx
    counts cells, the grids hold Nx + 1 nodes per side)."""
    ini = decks.write(decks.deck(nx=32, ny=24, ne=100, ni=100), str(tmp_path))
    sim = mixed_sim(gpu_lib, ini)
    with pytest.raises(ValueError):
        sim.set_grid("rho", np.zeros(32 * 24))
    sim.set_grid("rho", np.zeros(33 * 25))
