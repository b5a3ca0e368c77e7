"""Conductors and emitters in the mixed form, against the FP64 form on the
same deck and the same loaded particles.

* Conductors (src/grid.cpp, src/electrode.cpp): the mixed push erases the
  particles that end inside one (its FP64 position rebuilt from cell and
  offset), in order, and the SOR's rho override (src/field.cpp:100-103)
  precedes the mixed solve.  Over a few steps the mixed run erases the same
  particles as the FP64 run (equal counts), its particles stay within the
  mixed form's tolerance of the FP64 ones (positions 2e-5 of a cell,
  velocities 1e-4 relative), and phi within 1e-4.
* Emitters (src/emitter.cpp:5-36): the mixed form's injection writes the same
  Philox draws into its layout: equal counts step by step, the injected
  particles within FP32 rounding of the FP64 run's, and graph replay equal to
  stepping.
"""
import numpy as np
import pytest

from tests import decks

pytestmark = pytest.mark.gpu

GRIDS = [dict(type="reactconduct", min_x=10, max_x=12, min_y=4, max_y=16, grid_voltage=10),
         dict(type="circular", x_center=22, y_center=12, electrode_number=6, grid_radius=5, electrod_radius=1.5,
              electrode_voltage=-5)]


def _pair(E, ini):
    fp = E.Simulation.from_ini(ini)
    mx = E.Simulation.from_ini(ini, precision=1)
    for s in (fp, mx):
        s.load_particles(0)
        s.initial_field()
    return fp, mx


def _close(fp, mx, cell_tol, v_tol):
    for k in range(2):
        a, b = fp.particles(k), mx.particles(k)
        assert a.shape == b.shape, (k, a.shape, b.shape)
        if len(a):
            assert np.max(np.abs(a[:, :2] - b[:, :2])) < cell_tol
            vs = max(np.max(np.abs(a[:, 2:4])), 1e-300)
            assert np.max(np.abs(a[:, 2:4] - b[:, 2:4])) < v_tol * vs


@pytest.mark.parametrize("bc", ["pbc", "open", "reflective"])
def test_mixed_conductors_track_fp64(gpu_lib, tmp_path, bc):
    E = gpu_lib
    ini = decks.write(decks.deck(nx=32, ny=24, ne=3000, ni=3000, te=4, bc=bc, solver="gs", tol="1e-8", grids=GRIDS),
                      str(tmp_path))
    fp, mx = _pair(E, ini)
    n0 = fp.num_particles(0)
    for _ in range(4):
        fp.step()
        mx.step()
        _close(fp, mx, 2e-5, 1e-4)
        phi = fp.grid("phi")
        assert np.max(np.abs(mx.grid("phi") - phi)) < 1e-4 * np.max(np.abs(phi))
    assert fp.num_particles(0) < n0  # the conductors (and walls) took particles
    # graph replay equals stepping in the mixed form too
    mx2 = E.Simulation.from_ini(ini, precision=1)
    mx2.load_particles(0)
    mx2.initial_field()
    for _ in range(4):
        mx2.step()
    mx.run(3, graph=True)
    for _ in range(3):
        mx2.step()
    for k in range(2):
        assert np.array_equal(mx.particles(k), mx2.particles(k))


def test_mixed_emitters_track_fp64(gpu_lib, tmp_path):
    E = gpu_lib
    grids = [dict(type="reactconduct", min_x=0, max_x=6, min_y=10, max_y=11, grid_voltage=50),
             dict(type="reactconduct", min_x=0, max_x=6, min_y=5, max_y=6, grid_voltage=50)]
    em = [dict(x0=1, y0=7, x1=1, y1=9, temp=0.1, numparticle=50, vdx=0.2, vdy=0, species_idx1=0, species_idx2=1),
          dict(x0=20, y0=3, x1=26, y1=12, temp=0.5, numparticle=40, vdx=0, vdy=0.1, species_idx1=1, species_idx2=1)]
    ini = decks.write(decks.deck(nx=32, ny=16, ne=2000, ni=2000, te=1, bc="open", solver="gs", tol="1e-6",
                                 grids=grids, emitters=em), str(tmp_path))
    fp, mx = _pair(E, ini)
    n0 = [mx.num_particles(k) for k in range(2)]
    for _ in range(5):
        fp.step()
        mx.step()
        _close(fp, mx, 2e-5, 1e-4)
    assert mx.num_particles(1) > n0[1]
    mx2 = E.Simulation.from_ini(ini, precision=1)
    mx2.load_particles(0)
    mx2.initial_field()
    mx2.run(5, graph=True)
    for k in range(2):
        assert np.array_equal(mx.particles(k), mx2.particles(k))
