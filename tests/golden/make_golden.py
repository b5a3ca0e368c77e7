"""Generates the golden fixtures of tests/golden/*.npz from the reference itself.

The reference's own physics objects (src/*.cpp, compiled into oracle/_ref by
oracle/build_oracle.py) run each deck below through the set-up of
src/main.cpp (particle loading from mt19937 seed 0, initial field, rewind)
and a few loop iterations; every array is saved after each phase.  The
fixtures let machines without the reference checkout (the GPU machine) pin the
restatement and the GPU kernels to the reference's outputs.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402
import decks  # noqa: E402

CASES = {
    # name: (deck kwargs, steps, collisions)
    "pbc_gs_cic": (dict(nx=12, ny=12, ne=600, ni=600, solver="gs", tol="1e-8"), 2, False),
    "reflective_gs_ngp_rect": (dict(nx=14, ny=10, ne=500, ni=500, solver="gs", tol="1e-7", bc="reflective",
                                    shape="NGP"), 2, False),
    "open_pcg_cic": (dict(nx=12, ny=12, ne=600, ni=600, solver="cg", tol="1e-9", bc="open", te=4), 3, False),
    "pbc_pcg_beam": (dict(nx=12, ny=12, ne=500, ni=600, solver="cg", tol="1e-10",
                          beam=dict(n=100, t=1, frac=0.2, vx=5, vy=0)), 2, False),
    "mcc_ionizing": (dict(nx=24, ny=24, ne=500, ni=500, solver="gs", tol="1e-6", te=30,
                          ion_mass="6.63352090e-26", collisions=True, gas="1e23"), 2, True),
    # Boltzmann-electron solvers (src/field.cpp:7-68, 141-210)
    "gshybrid_pbc": (dict(nx=16, ny=12, ne=600, ni=600, solver="gshybrid", tol="1e-6", te=2), 2, False),
    "hybrid_pbc": (dict(nx=12, ny=10, ne=500, ni=500, solver="hybrid", tol="1e-6", te=2), 2, False),
    # a rectangular conductor and a ring of circular electrodes (src/grid.cpp, src/electrode.cpp)
    "conductors_gs_pbc": (dict(nx=24, ny=16, ne=800, ni=800, solver="gs", tol="1e-8", te=4,
                               grids=[dict(type="reactconduct", min_x=6, max_x=8, min_y=3, max_y=11, grid_voltage=10),
                                      dict(type="circular", x_center=16, y_center=8, electrode_number=5,
                                           grid_radius=4, electrod_radius=1.2, electrode_voltage=-5)]), 3, False),
}


def snapshot(ref: O.Reference, prefix: str, out: dict):
    for k in ("phi", "rho", "efx", "efy"):
        out[prefix + k] = ref.grid(k)
    for s in range(ref.nsp):
        out[prefix + "den%d" % s] = ref.den(s)
        out[prefix + "part%d" % s] = ref.particles(s)
    out[prefix + "error"] = np.array([ref.solver_error()])


def make(name: str, kw: dict, steps: int, collisions: bool):
    text = decks.deck(**kw)
    path = decks.write(text)
    out = {"ini": np.array(text)}
    ref = O.Reference(path, load=True, initial_field=False)
    for s in range(ref.nsp):
        out["load_part%d" % s] = ref.particles(s)
    del ref
    ref = O.Reference(path, load=True, initial_field=True)
    snapshot(ref, "init_", out)
    if collisions:
        ref.init_collisions()
    for k in range(steps):
        ref.step(1 if collisions else 0)
        snapshot(ref, "step%d_" % (k + 1), out)
    out["steps"] = np.array([steps])
    out["collisions"] = np.array([int(collisions)])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    os.remove(path)


if __name__ == "__main__":
    for name, (kw, steps, coll) in CASES.items():
        make(name, kw, steps, coll)
        print("wrote", name)
