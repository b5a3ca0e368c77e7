"""Benchmark workloads as input.ini decks, and the synthetic cross-section table.

Each workload is a deck in the reference's input.ini format.  Sizes follow the
configurations the project is measured on:

* ``periodic_64`` — 64x64 cells, 50 particles per cell per species
  (204,800 electrons + 204,800 ions), Te 1 eV, Ti 0.026 eV, ion mass 1836 m_e,
  n0 1e13 m^-3, dt 0.01/wpe, CIC, SOR (omega 1.8, tolerance 1e-8), no
  collisions; periodic particles and a periodic Poisson problem
  (poisson_bc = periodic), velocities drawn in 3V (load_3v).
* ``beam_mcc_256`` — 256x256 cells, 100 particles per cell: 6,553,600 ions
  (40 amu) and 6,553,600 electrons of which 10 % are a beam drifting at 5 v_th,e,
  PCG to 1e-10, MCC against 1e20 m^-3 neutrals with the synthetic 1000-point
  log-spaced table below; phi = 0 on the x walls and periodic in y
  (poisson_bc = dirichlet_x), particles periodic.
* ``periodic_1024`` — 1024x1024 cells, 100 particles per cell per species.
* ``conductors_64``, ``emitters_128``, ``gshybrid_64``, ``hybrid_24`` — one deck
  per extension of the loop (conductors with the SOR solver and absorbing walls,
  emitters with absorbing walls and PCG, the two Boltzmann-electron solvers),
  for their per-step measurements (``bench.py --rows``).
* ``twostream_1024`` — the precision form's plasma: 1024x1024 periodic cells,
  100 particles per cell per species (1.05e8 ions of 1836 m_e at 0.05 eV,
  1.05e8 electrons at 2 eV in two halves drifting at +-3 v_th,e), dt 0.05/wpe,
  PCG to 1e-10 on a periodic Poisson problem, no collisions (``twostream_256``
  is the same on 256x256 cells).

Inputs are seeded synthetic plasmas (the reference loads positions and
velocities from mt19937 seed 0; so do these decks).
"""
from __future__ import annotations

import numpy as np

AMU = 1.660538921e-27
ME = 9.10938215e-31

_TEMPLATE = """[file]
output = data/

[time]
NUM_TS = {num_ts}
DT_coeff = {dt}

[diagnostics]
write_interval = 10
write_interval_phase = 100
write_diagnostics = 50
write_flag = 0
save_fig   = 0
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
Nx       = {n}
Ny       = {n}
x0       = 0
y0       = 0

[Grids]
grid_count = 0

[Emitters]
count = 0

[normalization]
norm_scheme = 1
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
shapefunction = CIC
push_parallal  = false
deposit_parallal = false
density = 1E13
bc = {bc}
ionfixed = 0

[collision]
elastic    = {coll}
excitation = {coll}
ionization = {coll}
GAS_DENSITY = {gas}

[species]
{species}
"""


def deck(name: str) -> str:
    if name == "periodic_64":
        n, ppc = 64, 50
        sp = ["electron,%.8E,%d,1,-1,1,0,0,random" % (ME, n * n * ppc),
              "ion,%.8E,%d,0.026,1,0,0,0,random" % (1836 * ME, n * n * ppc)]
        text = _TEMPLATE.format(num_ts=1000, dt=0.01, n=n, solver="gs", tol="1e-8", maxit=200000,
                                solver_extra="sor_omega = 1.8\npoisson_bc = periodic\n", bc="pbc", coll="false",
                                gas="1e20", species="\n".join(sp))
        return text.replace("ionfixed = 0\n", "ionfixed = 0\nload_3v = true\n")
    if name in ("beam_mcc_256", "beam_mcc_160"):
        # beam_mcc_160 is the same plasma on 160x160 cells (5.1 M particles,
        # 205 MB: still larger than L2) for profiler captures.
        n, ppc = (256, 100) if name == "beam_mcc_256" else (160, 100)
        total_e = n * n * ppc
        beam = total_e // 10
        # fract_den is relative to the first species: 0.1/0.9 of the bulk.
        sp = ["electron,%.8E,%d,1,-1,1,0,0,random" % (ME, total_e - beam),
              "ion,%.8E,%d,0.026,1,0,0,0,random" % (40 * AMU, total_e),
              "beam,%.8E,%d,1,-1,%.17g,5,0,random" % (ME, beam, 1.0 / 9.0)]
        return _TEMPLATE.format(num_ts=2000, dt=0.01, n=n, solver="cg", tol="1e-10", maxit=100000,
                                solver_extra="poisson_bc = dirichlet_x\n", bc="pbc", coll="true", gas="1e20",
                                species="\n".join(sp))
    if name in ("twostream_1024", "twostream_256"):
        # two counter-streaming electron populations at +-3 v_th,e (v_th = sqrt(2 e Te / m_e));
        # velocities are in units of vel_norm = LDe * wpe = sqrt(e Te / m_e) (norm_scheme 1), so
        # 3 v_th,e = 3 sqrt(2) vel_norm.  Electron halves: fract_den 1 relative to the first.
        n = 1024 if name == "twostream_1024" else 256
        ppc = 100
        half = n * n * ppc // 2
        vs = 3.0 * np.sqrt(2.0)
        sp = ["electron,%.8E,%d,2,-1,1,%.17g,0,random" % (ME, half, vs),
              "ion,%.8E,%d,0.05,1,0,0,0,random" % (1836 * ME, n * n * ppc),
              "beam,%.8E,%d,2,-1,1,%.17g,0,random" % (ME, half, -vs)]
        return _TEMPLATE.format(num_ts=500, dt=0.05, n=n, solver="cg", tol="1e-10", maxit=100000,
                                solver_extra="poisson_bc = periodic\n", bc="pbc", coll="false", gas="1e20",
                                species="\n".join(sp))
    if name == "periodic_1024":
        n, ppc = 1024, 100
        sp = ["electron,%.8E,%d,2,-1,1,0,0,random" % (ME, n * n * ppc),
              "ion,%.8E,%d,0.05,1,0,0,0,random" % (1836 * ME, n * n * ppc)]
        return _TEMPLATE.format(num_ts=500, dt=0.05, n=n, solver="cg", tol="1e-10", maxit=100000,
                                solver_extra="", bc="pbc", coll="false", gas="1e20", species="\n".join(sp))
    if name in ROW_DECKS:
        return row_deck(name)
    raise KeyError(name)


def _sections(text: str, grids=(), emitters=()) -> str:
    """[Grids] and [Emitters] entries in the reference's keys (src/main.cpp:284-355)."""
    g = ["grid_count = %d" % len(grids)]
    for i, d in enumerate(grids):
        g += ["grid_%d.%s = %s" % (i, k, v) for k, v in d.items()]
    e = ["count = %d" % len(emitters)]
    for i, d in enumerate(emitters):
        e += ["emitter_%d.%s = %s" % (i, k, v) for k, v in d.items()]
    text = text.replace("[Grids]\ngrid_count = 0", "[Grids]\n" + "\n".join(g))
    return text.replace("[Emitters]\ncount = 0", "[Emitters]\n" + "\n".join(e))


ROW_DECKS = ("conductors_64", "emitters_128", "gshybrid_64", "hybrid_24")


def row_deck(name: str) -> str:
    def plasma(n, ppc, te=1.0):
        return ["electron,%.8E,%d,%g,-1,1,0,0,random" % (ME, n * n * ppc, te),
                "ion,%.8E,%d,0.026,1,0,0,0,random" % (1836 * ME, n * n * ppc)]
    if name == "conductors_64":
        # a biased plate and a ring of six electrodes; SOR (the solver the
        # conductors act on), absorbing walls
        n = 64
        grids = [dict(type="reactconduct", min_x=18, max_x=21, min_y=12, max_y=52, grid_voltage=10),
                 dict(type="circular", x_center=42, y_center=32, electrode_number=6, grid_radius=10,
                      electrod_radius=2, electrode_voltage=-5)]
        text = _TEMPLATE.format(num_ts=1000, dt=0.01, n=n, solver="gs", tol="1e-6", maxit=200000,
                                solver_extra="sor_omega = 1.8\n", bc="open", coll="false", gas="1e20",
                                species="\n".join(plasma(n, 100, 2.0)))
        return _sections(text, grids=grids)
    if name == "emitters_128":
        # an electron-ion source on the left wall and an ion source in the
        # middle, 2,000 + 500 points a step; absorbing walls, PCG
        n = 128
        em = [dict(x0=1, y0=16, x1=1, y1=112, temp=0.5, numparticle=2000, vdx=0.5, vdy=0, species_idx1=0,
                   species_idx2=1),
              dict(x0=60, y0=60, x1=68, y1=68, temp=0.02, numparticle=500, vdx=0, vdy=0.2, species_idx1=1,
                   species_idx2=1)]
        text = _TEMPLATE.format(num_ts=1000, dt=0.01, n=n, solver="cg", tol="1e-10", maxit=100000,
                                solver_extra="", bc="open", coll="false", gas="1e20",
                                species="\n".join(plasma(n, 50)))
        return _sections(text, emitters=em)
    if name == "gshybrid_64":
        n = 64
        return _TEMPLATE.format(num_ts=1000, dt=0.01, n=n, solver="gshybrid", tol="1e-6", maxit=200000,
                                solver_extra="sor_omega = 1.8\n", bc="pbc", coll="false", gas="1e20",
                                species="\n".join(plasma(n, 50, 2.0)))
    if name == "hybrid_24":
        # nrpcgsolver builds dense n x n matrices in the reference: small grids only
        n = 24
        return _TEMPLATE.format(num_ts=1000, dt=0.01, n=n, solver="hybrid", tol="1e-6", maxit=100000,
                                solver_extra="", bc="pbc", coll="false", gas="1e20",
                                species="\n".join(plasma(n, 50, 2.0)))
    raise KeyError(name)


def synthetic_table(n: int = 1000, e_min: float = 0.01, e_max: float = 1000.0):
    """Synthetic e-/neutral cross sections [m^2] on n log-spaced energies [eV]:
    elastic 1e-19 flat; excitation zero below 11.5 eV, rising linearly to
    2e-20 at 50 eV and falling as 1/E above; ionisation zero below 15.8 eV,
    x*exp(1-x) with x = (E-15.8)/(100-15.8), i.e. a 3e-20 peak at 100 eV."""
    e = e_min * (e_max / e_min) ** (np.arange(n) / (n - 1))
    ela = np.full(n, 1e-19)
    exc = np.where(e < 11.5, 0.0, np.where(e < 50.0, 2e-20 * (e - 11.5) / (50.0 - 11.5), 2e-20 * 50.0 / e))
    x = (e - 15.8) / (100.0 - 15.8)
    ion = np.where(e < 15.8, 0.0, 3e-20 * x * np.exp(1.0 - x))
    return e, ela, exc, ion


def serving_requests(seed: int = 0, rate_per_s: float = 50.0, window_s: float = 60.0, sides=(64, 128, 256, 512),
                     ppc=(25, 100), steps=(500, 5000), step_scale: float = 1.0, p_mcc: float = 0.5):
    """Requests of the serving workload: Poisson arrivals at `rate_per_s` over
    `window_s` seconds; per request a square grid side drawn from `sides`,
    particles per cell per species drawn from `ppc`, a step count drawn from
    `steps` and multiplied by `step_scale`, MCC with probability `p_mcc`
    (synthetic table), and a periodic system (periodic walls and Poisson
    problem) or a Dirichlet one (phi = 0 on the edges, absorbing walls), each
    with probability 0.5.  Electrons Te = 1 eV, ions 40 amu at 0.026 eV, PCG
    to 1e-10.  Returns a list of dicts {ini, steps, collisions, seed,
    arrival_s, side, particles}."""
    rng = np.random.default_rng(seed)
    out = []
    t = float(rng.exponential(1.0 / rate_per_s))
    k = 0
    while t < window_s:
        n = int(rng.choice(sides))
        pe, pi = (int(rng.integers(ppc[0], ppc[1] + 1)) for _ in range(2))
        st = max(1, int(round(int(rng.integers(steps[0], steps[1] + 1)) * step_scale)))
        coll = bool(rng.random() < p_mcc)
        periodic = rng.random() < 0.5
        bc = "pbc" if periodic else "open"
        sp = ["electron,%.8E,%d,1,-1,1,0,0,random" % (ME, n * n * pe),
              "ion,%.8E,%d,0.026,1,0,0,0,random" % (40 * AMU, n * n * pi)]
        ini = _TEMPLATE.format(num_ts=st, dt=0.01, n=n, solver="cg", tol="1e-10", maxit=100000,
                               solver_extra="poisson_bc = periodic\n" if periodic else "", bc=bc,
                               coll="true" if coll else "false", gas="1e20", species="\n".join(sp))
        out.append({"ini": ini, "steps": st, "collisions": coll, "seed": 1000 + k, "arrival_s": t, "side": n,
                    "particles": n * n * (pe + pi)})
        k += 1
        t += float(rng.exponential(1.0 / rate_per_s))
    return out


def batching_requests(seed: int = 0, nruns: int = 512, sides=tuple(range(32, 257, 16)), ppc=(20, 200),
                      te=(0.5, 5.0), p_mcc: float = 0.5):
    """Runs of the batching workload: per run the cell counts along x and y
    drawn independently from `sides`, particles per cell from `ppc` (both
    species), Te from `te` (eV; ions 1836 m_e at 0.026 eV), MCC with
    probability `p_mcc`, periodic walls, PCG to 1e-10.  Returns a list of dicts
    {ini, collisions, seed, nx, ny, particles}."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nruns):
        nx, ny = (int(rng.choice(sides)) for _ in range(2))
        p = int(rng.integers(ppc[0], ppc[1] + 1))
        t = float(rng.uniform(te[0], te[1]))
        coll = bool(rng.random() < p_mcc)
        sp = ["electron,%.8E,%d,%.6g,-1,1,0,0,random" % (ME, nx * ny * p, t),
              "ion,%.8E,%d,0.026,1,0,0,0,random" % (1836 * ME, nx * ny * p)]
        ini = _TEMPLATE.format(num_ts=1000, dt=0.01, n=nx, solver="cg", tol="1e-10", maxit=100000, solver_extra="",
                               bc="pbc", coll="true" if coll else "false", gas="1e20", species="\n".join(sp))
        ini = ini.replace("Ny       = %d" % nx, "Ny       = %d" % ny, 1)
        out.append({"ini": ini, "collisions": coll, "seed": 2000 + k, "nx": nx, "ny": ny,
                    "particles": 2 * nx * ny * p})
    return out
