"""The oracle's restatement of the Poisson extensions (no reference
counterpart), pinned against direct solves of the same discrete problems.

* periodic:    unknowns i in [0, nx-2], j in [0, ny-2], both directions
               periodic; right-hand side projected onto zero mean, phi with
               zero mean.  Direct solve: 2-D FFT.
* dirichlet_x: unknowns i in [1, nx-2], j in [0, ny-2]; phi = 0 on the x walls,
               periodic in y.  Direct solve: DST-I along x, FFT along y.

Both the PCG and the lexicographic SOR restatements must land on the direct
solution (to what their stopping tolerance allows), fill the duplicated
nodes, and the E-field must use the periodic / one-sided edge formulas of
the field's boundary.  Also: the correctly rounded sum the mean projections
use, and the 3V loading extension.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from tests import decks


def _setup(tmp_path, bc, solver="cg", tol="1e-12", nx=32, ny=24, extra=""):
    ini = decks.write(decks.deck(nx=nx, ny=ny, ne=20000, ni=20000, solver=solver, tol=tol, maxit=200000,
                                 solver_extra="poisson_bc = %s\n%s" % (bc, extra)), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    orc.scatter_all()
    return orc


def _direct(orc):
    """phi of the extension problem from the FFT / DST-I solve: -(A phi) = rho K dx^2 on the unknowns,
    A the 5-point operator (diagonal -4) with the boundary of the extension."""
    import scipy.fft as F

    s = orc.s
    nx, ny = s.nx, s.ny
    K = (s.L * s.L) / (s.LDe * s.LDe)
    rho = orc.rho.reshape(nx, ny)
    periodic = s.poisson_bc == "periodic"
    i0 = 0 if periodic else 1
    R, C = nx - 1 - i0, ny - 1
    b = -rho[i0:i0 + R, :C] * s.dx * s.dx * K
    q = np.arange(C)
    mu = 2 * np.cos(2 * np.pi * q / C) - 2
    if periodic:
        b = b - b.mean()
        p = np.arange(R)
        lam = (2 * np.cos(2 * np.pi * p / R) - 2)[:, None] + mu[None, :]
        bh = np.fft.fft2(b)
        lam[0, 0] = 1.0
        xh = bh / lam
        xh[0, 0] = 0.0
        x = np.real(np.fft.ifft2(xh))
    else:
        p = np.arange(1, R + 1)
        lam = (2 * np.cos(np.pi * p / (R + 1)) - 2)[:, None] + mu[None, :]
        bh = np.fft.fft(F.dst(b, type=1, axis=0, norm="ortho"), axis=1)
        x = F.idst(np.real(np.fft.ifft(bh / lam, axis=1)), type=1, axis=0, norm="ortho")
    phi = np.zeros((nx, ny))
    phi[i0:i0 + R, :C] = x
    if periodic:
        phi[nx - 1, :C] = phi[0, :C]
    phi[:, ny - 1] = phi[:, 0]
    if not periodic:
        phi[0, :] = phi[nx - 1, :] = 0
    return phi.reshape(-1)


def test_exact_sum_is_correctly_rounded():
    L = O.restatement_lib()
    rng = np.random.default_rng(0)
    for trial in range(300):
        n = int(rng.integers(1, 2000))
        kind = trial % 4
        if kind == 0:
            x = rng.normal(size=n)
        elif kind == 1:
            x = rng.normal(size=n) * 10.0 ** rng.integers(-300, 300, size=n)
        elif kind == 2:
            x = rng.normal(size=n)
            x = np.concatenate([x, -x, [1e-300, 1e300, -1e300, 5e-320]])
        else:
            x = (rng.random(n) - 0.5) * 2.0 ** rng.integers(-60, 60, size=n)
        x = np.ascontiguousarray(x)
        assert L.or_exact_sum(x.ctypes.data, len(x)) == math.fsum(x.tolist()), trial


@pytest.mark.parametrize("bc", ["periodic", "dirichlet_x"])
@pytest.mark.parametrize("nxy", [(32, 24), (20, 33)])
def test_pcg_extension_matches_direct_solve(tmp_path, bc, nxy):
    orc = _setup(tmp_path, bc, nx=nxy[0], ny=nxy[1])
    phi, err, it, conv = orc.R.pcg_solve(orc.rho)
    want = _direct(orc)
    assert conv and it > 10
    # |phi - phi*| <= |A^-1| |r| with |r| < 1e-12 and |A^-1| <= 1/lambda_min ~ (n/2pi)^2
    assert np.max(np.abs(phi - want)) < 1e-8 * np.max(np.abs(want))
    if bc == "periodic":
        nx, ny = orc.s.nx, orc.s.ny
        assert abs(phi.reshape(nx, ny)[:-1, :-1].mean()) < 1e-14 * np.max(np.abs(phi))


@pytest.mark.parametrize("bc", ["periodic", "dirichlet_x"])
def test_sor_extension_matches_direct_solve(tmp_path, bc):
    orc = _setup(tmp_path, bc, solver="gs", tol="1e-11", nx=24, ny=20, extra="sor_omega = 1.8\n")
    phi, err, it, conv = orc.R.gs_solve(orc.rho, 1.8)
    want = _direct(orc)
    assert conv and it > 25 and err < 1e-11
    assert np.max(np.abs(phi - want)) < 1e-6 * np.max(np.abs(want))


@pytest.mark.parametrize("bc", ["periodic", "dirichlet_x"])
def test_efield_follows_the_field_boundary(tmp_path, bc):
    orc = _setup(tmp_path, bc, nx=16, ny=12)
    nx, ny = orc.s.nx, orc.s.ny
    phi = np.random.default_rng(3).normal(size=nx * ny)
    ex, ey = orc.R.efield(phi)
    P = phi.reshape(nx, ny)
    EX, EY = ex.reshape(nx, ny), ey.reshape(nx, ny)
    assert np.array_equal(EY[:, 0], -(P[:, 1] - P[:, ny - 2]) / 2) and np.array_equal(EY[:, ny - 1], EY[:, 0])
    if bc == "periodic":
        assert np.array_equal(EX[0], -(P[1] - P[nx - 2]) / 2) and np.array_equal(EX[nx - 1], EX[0])
    else:
        assert np.array_equal(EX[0], -(P[1] - P[0])) and np.array_equal(EX[nx - 1], -(P[nx - 1] - P[nx - 2]))
    assert np.array_equal(EX[1:-1], -(P[2:] - P[:-2]) / 2)


def test_load_3v_draws_vz_like_vx(tmp_path):
    ini = decks.write(decks.deck(nx=16, ny=16, ne=200000, ni=200000, te=2, sim_extra="load_3v = true\n"),
                      str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    e = orc.parts[0]
    sx, sz = e[:, 2].std(), e[:, 4].std()
    assert abs(sz / sx - 1) < 0.01 and abs(e[:, 4].mean()) < 5 * sz / math.sqrt(len(e))
    plain = O.OracleSim(decks.write(decks.deck(nx=16, ny=16, ne=2000, ni=2000, te=2), str(tmp_path)),
                        initial_field=False)
    assert np.all(plain.parts[0][:, 4] == 0)
