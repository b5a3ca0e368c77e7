"""The C++ seam (epic2d_mcc_gb300/host/epic2d.hpp) takes a main written in the
reference's style: tests/dropin/reference_loop.cpp uses the reference's
classes, constructors and method signatures (Domain(x0, y0, dx, dy, nx, ny)
and its member assignments, Species(name, mass, ..., initialization, domain),
Create_Grid, Emitter(params, domain), Init(species, domain, grids),
FieldSolve(domain, grids), Push_species_serial(1, grids), CollisionHandler(domain),
handle_collisions(electrons, ions)) in the call order of the reference's main.

CPU: it compiles against the shim and links against the library.
GPU: its particles and potential after NUM_TS + 1 loop iterations equal, bit
for bit, the same deck run through the Python API (Simulation.from_ini,
load_particles(0), initial_field, step), for a beam/MCC/PCG deck and a
conductor/emitter/SOR deck with absorbing walls.
"""
import os
import subprocess

import numpy as np
import pytest

from tests import decks

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "dropin", "reference_loop.cpp")
HOST = os.path.join(ROOT, "epic2d_mcc_gb300", "host")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(ROOT, "epic2d_mcc_gb300", "libepic2d_gb300.so")


def _compile(out_dir):
    from epic2d_mcc_gb300 import build as B

    B.build()
    exe = os.path.join(str(out_dir), "reference_loop")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-I", HOST, "-I", INCLUDE, "-o", exe, SRC, LIB,
                        "-Wl,-rpath," + os.path.dirname(LIB)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


def test_reference_style_main_compiles_against_the_shim(tmp_path):
    assert os.access(_compile(tmp_path), os.X_OK)


def _beam_deck():
    return decks.deck(nx=32, ny=32, ne=40000, ni=40000, solver="cg", tol="1e-10", te=30, collisions=True,
                      gas="1e22", ion_mass="6.63352090e-26", beam=dict(n=4000, t=1, frac=0.1, vx=5, vy=0), num_ts=3)


def _conductor_deck():
    grids = [dict(type="reactconduct", min_x=8, max_x=10, min_y=6, max_y=26, grid_voltage=10),
             dict(type="circular", x_center=22, y_center=16, electrode_number=4, grid_radius=5,
                  electrod_radius=1.5, electrode_voltage=-5)]
    emitters = [dict(x0=1, y0=4, x1=1, y1=28, temp=0.5, numparticle=300, vdx=0.5, vdy=0, species_idx1=0,
                     species_idx2=1),
                dict(x0=14, y0=14, x1=18, y1=18, temp=0.02, numparticle=100, vdx=0, vdy=0.2, species_idx1=1,
                     species_idx2=1)]
    # no sor_omega key: the reference's main knows only its hard-coded 1.4
    return decks.deck(nx=32, ny=32, ne=20000, ni=20000, solver="gs", tol="1e-6", te=2, bc="open", num_ts=3,
                      grids=grids, emitters=emitters)


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["beam_mcc_pcg", "conductors_emitters_sor"])
def test_reference_style_main_equals_the_api_run(gpu_lib, tmp_path, which):
    E = gpu_lib
    text = _beam_deck() if which == "beam_mcc_pcg" else _conductor_deck()
    ini = decks.write(text, str(tmp_path))
    exe = _compile(tmp_path)
    prefix = str(tmp_path / "out")
    r = subprocess.run([exe, ini, prefix], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    steps = int(r.stdout.split()[1])
    sim = E.Simulation.from_ini(ini)
    coll = which == "beam_mcc_pcg"
    if coll:
        sim.set_reference_cross_sections()
    sim.load_particles(0)
    sim.initial_field()
    for _ in range(steps):
        sim.step(collisions=coll)
    for s in range(len(sim.species)):
        got = np.fromfile(prefix + "_part%d.bin" % s, dtype=np.float64).reshape(-1, 5)
        assert np.array_equal(got, sim.particles(s)), "species %d" % s
    assert np.array_equal(np.fromfile(prefix + "_phi.bin", dtype=np.float64), sim.grid("phi"))
