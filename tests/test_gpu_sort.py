"""Cell sort (no counterpart in the reference) through the C ABI.

* FP64 form: the sorted particle array equals the input permuted by a stable
  argsort of the keys i*ny + j, i = (int)((x - x0)/dx), j = (int)((y - y0)/dy)
  — bit for bit (records are moved, never recomputed).
* Mixed form: the same, with the mixed form's own cell as the key.
* Sorting changes nothing a step computes from the particles: the int64
  fixed-point deposit is exact, so density, potential and the pushed
  particles (compared as sets) are identical with and without sorting, for
  the shared-memory-tile deposit of the mixed form too.
* A graph-replayed run with sorting every k steps matches the same steps
  launched one by one, bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import decks

pytestmark = pytest.mark.gpu


def keys_of(parts, s):
    i = np.trunc((parts[:, 0] - s.x0) / s.dx).astype(np.int64)
    j = np.trunc((parts[:, 1] - s.y0) / s.dy).astype(np.int64)
    i = np.clip(i, 0, s.nx - 1)
    j = np.clip(j, 0, s.ny - 1)
    return i * s.ny + j


def canon(parts):
    return parts[np.lexsort(parts.T[::-1])]


@pytest.mark.parametrize("n", [1, 4095, 4097, 60000])
def test_sort_fp64_is_stable_argsort(gpu_lib, tmp_path, n):
    ini = decks.write(decks.deck(nx=64, ny=48, ne=max(n, 2), ni=max(n, 2)), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    sim = gpu_lib.Simulation.from_ini(ini)
    for sp in range(2):
        parts = orc.parts[sp][:n]
        sim.set_particles(sp, parts)
        sim.sort_species(sp)
        got = sim.particles(sp)
        perm = np.argsort(keys_of(parts, orc.s), kind="stable")
        assert np.array_equal(got, parts[perm])


def test_sort_large_grid_three_passes(gpu_lib, tmp_path):
    # 1025 x 1025 nodes: keys need 21 bits, three 9-bit digit passes.
    ini = decks.write(decks.deck(nx=1024, ny=1024, ne=300000, ni=1000), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    sim = gpu_lib.Simulation.from_ini(ini)
    parts = orc.parts[0]
    sim.set_particles(0, parts)
    sim.sort_species(0)
    perm = np.argsort(keys_of(parts, orc.s), kind="stable")
    assert np.array_equal(sim.particles(0), parts[perm])


def test_sort_mixed_is_stable_argsort(gpu_lib, tmp_path):
    ini = decks.write(decks.deck(nx=64, ny=48, ne=50000, ni=50000), str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    s = orc.s
    assert s.dx == 1.0 and s.dy == 1.0 and s.x0 == 0.0 and s.y0 == 0.0  # positions map to cells exactly
    sim = gpu_lib.Simulation.from_ini(ini, precision=1, sort_every=0)
    for sp in range(2):
        sim.set_particles(sp, orc.parts[sp])
        before = sim.particles(sp)
        sim.sort_species(sp)
        got = sim.particles(sp)
        perm = np.argsort(keys_of(before, s), kind="stable")
        assert np.array_equal(got, before[perm])


@pytest.mark.parametrize("precision", [0, 1])
def test_sorting_changes_no_step_result(gpu_lib, tmp_path, precision):
    ini = decks.write(decks.deck(nx=64, ny=64, ne=200000, ni=200000, solver="cg", tol="1e-10", maxit=100000),
                      str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    runs = []
    for sort_every in (0, 1):
        sim = gpu_lib.Simulation.from_ini(ini, precision=precision, sort_every=sort_every)
        for sp in range(2):
            sim.set_particles(sp, orc.parts[sp])
        sim.initial_field()
        for _ in range(3):
            sim.step(collisions=False)
        runs.append((sim.grid("rho"), sim.grid("phi"), [canon(sim.particles(sp)) for sp in range(2)],
                     [sim.den(sp) for sp in range(2)]))
    (r0, p0, q0, d0), (r1, p1, q1, d1) = runs
    assert np.array_equal(r0, r1) and np.array_equal(p0, p1)
    for sp in range(2):
        assert np.array_equal(d0[sp], d1[sp])
        assert np.array_equal(q0[sp], q1[sp])


def test_graph_replay_with_sorting(gpu_lib, tmp_path):
    ini = decks.write(decks.deck(nx=64, ny=64, ne=100000, ni=100000, solver="cg", tol="1e-10", maxit=100000),
                      str(tmp_path))
    orc = O.OracleSim(ini, initial_field=False)
    out = []
    for graph in (False, True):
        sim = gpu_lib.Simulation.from_ini(ini, precision=1, sort_every=2)
        for sp in range(2):
            sim.set_particles(sp, orc.parts[sp])
        sim.initial_field()
        sim.run(5, collisions=False, graph=graph)
        out.append((sim.grid("phi"), [sim.particles(sp) for sp in range(2)]))
    assert np.array_equal(out[0][0], out[1][0])
    for sp in range(2):
        assert np.array_equal(out[0][1][sp], out[1][1][sp])
