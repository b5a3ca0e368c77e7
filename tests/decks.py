"""input.ini decks for the tests, in the reference's format (input.ini:1-166)."""
from __future__ import annotations

import os
import tempfile

TEMPLATE = """[file]
output = data/

[time]
NUM_TS = {num_ts}
DT_coeff = {dt}

[diagnostics]
write_interval = 10
write_interval_phase = 100
write_diagnostics = 50
write_flag = 1
save_fig   = 1
sub_cycle_interval = 20
precision = 4

[PlotFlags]
phase_space     = 0
config_space    = 0
electric_field  = 0
potential_field = 0
density_contour = 0
ke_components   = 1
total_energy    = 1
species_index   = 0

[domain]
Nx       = {nx}
Ny       = {ny}
x0       = {x0}
y0       = {x0}

[Grids]
{grids}

[Emitters]
{emitters}

[normalization]
norm_scheme = {norm}
vel_norm_scheme = 1
lenght_scale = 0.005
time_scale = omegape
energy_scale = 1

[solver]
solvertype = {solver}
tolerance = {tol}
max_iteration = {maxit}
{solver_extra}
[simulation]
shapefunction = {shape}
push_parallal  = false
deposit_parallal = false
density = {density}
bc = {bc}
ionfixed = {ionfixed}
{sim_extra}
[collision]
elastic    = {el}
excitation = {ex}
ionization = {io}
GAS_DENSITY = {gas}
{coll_extra}
[species]
{species}
"""

ELECTRON = "electron,9.10938215E-31,{n},{t},-1,1,{vx},{vy},random"
ION = "ion,{m},{n},{t},1,0,0,0,random"
BEAM = "beam,9.10938215E-31,{n},{t},-1,{frac},{vx},{vy},random"


def deck(nx=16, ny=16, ne=2000, ni=2000, te=1, ti=0.026, ion_mass="1.6726219e-27", solver="gs", tol="1e-8",
         maxit=20000, bc="pbc", shape="CIC", dt=0.01, norm=1, density="1E13", collisions=False, gas="1e20",
         ionfixed=0, beam=None, vdrift=(0, 0), solver_extra="", sim_extra="", coll_extra="", num_ts=10, grids=None,
         emitters=None, x0=0):
    sp = [ELECTRON.format(n=ne, t=te, vx=vdrift[0], vy=vdrift[1]), ION.format(m=ion_mass, n=ni, t=ti)]
    if beam:
        sp.append(BEAM.format(**beam))
    flag = "true" if collisions else "false"
    return TEMPLATE.format(num_ts=num_ts, dt=dt, nx=nx, ny=ny, norm=norm, solver=solver, tol=tol, maxit=maxit,
                           shape=shape, density=density, bc=bc, ionfixed=ionfixed, el=flag, ex=flag, io=flag,
                           gas=gas, species="\n".join(sp), solver_extra=solver_extra, sim_extra=sim_extra,
                           coll_extra=coll_extra, grids=grid_section(grids or []),
                           emitters=emitter_section(emitters or []), x0=x0)


def grid_section(grids) -> str:
    """[Grids] lines in the reference's keys (src/main.cpp:284-327) from dicts with a "type" of
    "reactconduct" (min_x, max_x, min_y, max_y, grid_voltage) or "circular" (x_center, y_center,
    electrode_number, grid_radius, electrod_radius, electrode_voltage)."""
    lines = ["grid_count = %d" % len(grids)]
    for i, g in enumerate(grids):
        for k, v in g.items():
            lines.append("grid_%d.%s = %s" % (i, k, v))
    return "\n".join(lines)


def write(text: str, directory: str | None = None) -> str:
    d = directory or tempfile.mkdtemp(prefix="epic_deck_")
    fd, path = tempfile.mkstemp(suffix=".ini", dir=d)
    with os.fdopen(fd, "w") as f:
        f.write(text)
    return path


def emitter_section(emitters) -> str:
    """[Emitters] lines in the reference's keys (src/main.cpp:330-355) from dicts of x0, y0, x1, y1,
    temp, numparticle, vdx, vdy, species_idx1, species_idx2."""
    lines = ["count = %d" % len(emitters)]
    for i, e in enumerate(emitters):
        for k, v in e.items():
            lines.append("emitter_%d.%s = %s" % (i, k, v))
    return "\n".join(lines)
