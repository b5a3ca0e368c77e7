"""The command-line driver's result tree (host/main.cpp --output, the
reference's result.h5 layout of src/output.cpp:4-287 written as NPY files on
the cadence of src/main.cpp:426-455), checked against the same run through the
Python API: the written potential, fields, densities, particles and energy
history are the run's own, bit for bit."""
import json
import os
import subprocess

import numpy as np
import pytest

from tests import decks

pytestmark = pytest.mark.gpu


def test_driver_writes_the_result_tree(gpu_lib, tmp_path):
    from epic2d_mcc_gb300 import build as B

    drv = B.build_driver()
    nx = ny = 33  # nodes: Nx + 1
    ini = decks.write(decks.deck(nx=nx - 1, ny=ny - 1, ne=20000, ni=20000, solver="cg", num_ts=20,
                                 beam=dict(n=2000, t=1, frac=0.1, vx=5, vy=0)), str(tmp_path))
    out = tmp_path / "out"
    energy = tmp_path / "energy.csv"
    subprocess.run([drv, ini, "--output", str(out), "--energy", str(energy), "--quiet"], check=True,
                   stdout=subprocess.DEVNULL)
    res = out / "result"

    meta = json.loads((res / "metadata.json").read_text())
    assert meta["NC"] == nx and meta["NUM_TS"] == 20 and meta["write_int"] == 10 and meta["write_int_phase"] == 100
    assert meta["spno"] == 3 and meta["GAS_DENSITY"] == 0 and meta["DT_coeff"] == 0.01
    for name in ("electron", "ion", "beam"):
        sm = json.loads((res / "metadata_species" / (name + ".json")).read_text())
        assert sm["name"] == name
    assert json.loads((res / "metadata_species" / "beam.json").read_text())["streaming_velocity"] == 5

    # the same run through the API: initial field, then ts = 0 .. 20
    sim = gpu_lib.Simulation.from_ini(ini)
    sim.load_particles(0)
    sim.initial_field()
    ke_rows = []
    for ts in range(21):
        sim.step()
        if ts % 10:
            continue
        for g, which in (("pot", "phi"), ("efieldx", "efx"), ("efieldy", "efy")):
            f = np.load(res / "fielddata" / g / ("%d.npy" % ts))
            assert f.shape == (nx, ny)
            # buffer element j*nx + i holds node (i, j)
            assert np.array_equal(f.reshape(-1), sim.grid(which).reshape(nx, ny).T.reshape(-1)), (g, ts)
        for s, name in ((0, "electron"), (1, "ion")):
            f = np.load(res / "fielddata" / ("den_" + name) / ("%d.npy" % ts))
            assert np.array_equal(f.reshape(-1), sim.den(s).reshape(nx, ny).T.reshape(-1))
        assert not (res / "fielddata" / "den_beam").exists()
        row = [ts * sim.cfg.DT]
        for s in range(3):
            row += list(sim.compute_ke(s, 0))
        row.append(sim.compute_pe(0))
        ke_rows.append(row)
        # particle data only where ts is a multiple of write_interval_phase (100)
        for name in ("electron", "ion", "beam"):
            assert (res / ("particle_" + name) / ("pos%d.npy" % ts)).exists() == (ts == 0)
        if ts == 0:
            for s, name in enumerate(("electron", "ion", "beam")):
                p = sim.particles(s)
                pos = np.load(res / ("particle_" + name) / "pos0.npy")
                vel = np.load(res / ("particle_" + name) / "vel0.npy")
                assert pos.shape == (len(p), 2) and vel.shape == (len(p), 2)
                assert np.array_equal(pos, p[:, 0:2]) and np.array_equal(vel, p[:, 2:4])
    ke = np.load(res / "time_var" / "kinetic_energy.npy")
    assert ke.shape == (3, 3 * 3 + 2)
    assert np.array_equal(ke, np.array(ke_rows))
    csv = np.loadtxt(energy, delimiter=",")
    assert csv.shape == ke.shape
    np.testing.assert_allclose(csv, ke, rtol=1e-5, atol=0)  # the CSV carries 6 significant digits
    sim.close()
