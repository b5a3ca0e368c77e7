"""ORACLE TEST INFRASTRUCTURE — not part of the product.

Python face of the oracle:

* :func:`parse_ini` / :func:`setup` restate the reference's INI parser
  (src/iniparser.cpp:4-113) and the set-up arithmetic of src/main.cpp:42-261
  with Domain::set_normscheme (src/domain.cpp:123-183), keeping the
  reference's operation order.
* :class:`Restatement` binds the plain-C restatement (oracle/epic_oracle.c).
* :class:`Reference` binds the reference's own objects (oracle/_ref), which
  exist only where the reference checkout was available to compile them.
* :class:`OracleSim` runs the time-step loop of src/main.cpp:359-423 on the
  restatement.

Only tests/, the smoke check and bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import build_oracle

EPS_0 = 8.85418782e-12
QE = 1.602176565e-19
AMU = 1.660538921e-27
ME = 9.10938215e-31
K_B = 1.380648e-23
EV_TO_K = QE / K_B
EV = 1.602176565e-19
CS_RANGES = 5_000_000

BC_CODES = {"pbc": 0, "open": 1, "reflective": 2}
# [solver] poisson_bc (extension): the reference's zero edges, periodic, or
# zero on the x walls and periodic in y
POISSON_BC_CODES = {"dirichlet": 0, "periodic": 1, "dirichlet_x": 2}
SHAPE_CODES = {"CIC": 0, "NGP": 1}


# ----------------------------------------------------------------- INI ---
def _trim(s: str) -> str:
    return s.strip(" \t")


def parse_ini(path: str) -> dict:
    """src/iniparser.cpp:4-49: sections of key=value; [species] lines are kept
    raw under keys "0", "1", ...; lines starting with ';' or '#' are skipped."""
    sections: dict = {}
    cur = ""
    with open(path) as f:
        for line in f.read().split("\n"):
            if not line or line[0] in ";#":
                continue
            if line[0] == "[" and line[-1] == "]":
                cur = line[1:-1]
                sections.setdefault(cur, {})
                continue
            sec = sections.setdefault(cur, {})
            if cur == "species":
                sec[str(len(sec))] = line
            elif "=" in line:
                k, v = line.split("=", 1)
                sec[_trim(k)] = _trim(v)
    return sections


def _stoi(s: str) -> int:
    s = s.strip()
    i = 0
    if i < len(s) and s[i] in "+-":
        i += 1
    while i < len(s) and s[i].isdigit():
        i += 1
    return int(s[:i])


def _stod(s: str) -> float:
    s = s.strip()
    best = None
    for j in range(len(s), 0, -1):
        try:
            best = float(s[:j])
            break
        except ValueError:
            continue
    if best is None:
        raise ValueError("stod: no conversion for %r" % s)
    return best


def string_to_bool(s: str) -> bool:
    """include/extrafun.h:6-17."""
    return s in ("true", "True", "T", "t", "1", "yes", "Yes", "Y", "y")


@dataclass
class SpeciesDesc:
    name: str
    mass: float
    numparticle: int
    temp: float
    charge_sign: int
    frac: float
    vsx: float
    vsy: float
    load: str
    charge: float = 0.0
    spwt: float = 0.0


@dataclass
class Setup:
    nx: int
    ny: int
    x0: float
    y0: float
    dx: float
    dy: float
    Lx: float
    Ly: float
    DT: float
    L: float
    W: float
    vel_norm: float
    LDe: float
    wpe: float
    LDi: float
    wpi: float
    density: float
    shape: str
    bc: str
    solver: str
    tolerance: float
    max_iteration: int
    gas_density: float
    elastic: bool
    excitation: bool
    ionization: bool
    num_ts: int
    ionfixed: int
    normscheme: int
    species: list = field(default_factory=list)
    sor_omega: float = 1.4  # optional [solver] sor_omega; 1.4 is hard-coded in src/field.cpp:114
    poisson_bc: str = "dirichlet"  # optional [solver] poisson_bc (extension)
    load_3v: bool = False  # optional [simulation] load_3v: vz drawn like vx, vy (the reference loads 0)
    # [Grids] (src/main.cpp:284-327) as rows of 8 doubles: {0, min_x, max_x, min_y, max_y, 0, 0, V}
    # (reactconduct) or {1, x_center, y_center, electrode_number, grid_radius, electrod_radius, 0, V}
    grids: np.ndarray = field(default_factory=lambda: np.zeros((0, 8)))
    # [Emitters] (src/main.cpp:330-355) as rows {x0, y0, x1, y1, temp, numparticle, vdx, vdy, idx1, idx2}
    emitters: np.ndarray = field(default_factory=lambda: np.zeros((0, 10)))


def setup(path: str) -> Setup:
    """src/main.cpp:42-261 plus Domain::set_normscheme (src/domain.cpp:123-183)."""
    ini = parse_ini(path)
    sp_lines = ini["species"]
    Nx = _stoi(ini["domain"]["Nx"])
    Ny = _stoi(ini["domain"]["Ny"])
    x0 = _stod(ini["domain"]["x0"])
    col = ini["collision"]
    num_ts = _stoi(ini["time"]["NUM_TS"])
    DT_coeff = _stod(ini["time"]["DT_coeff"])
    sim = ini["simulation"]
    den = _stod(sim["density"])
    norm_scheme = _stoi(ini["normalization"]["norm_scheme"])
    L_scale = _stod(ini["normalization"]["lenght_scale"])
    T_scale = ini["normalization"]["time_scale"]
    solver = ini["solver"]
    species = []
    for k in sorted(sp_lines, key=int):
        t = sp_lines[k].split(",")
        if len(t) == 9:
            species.append(SpeciesDesc(t[0], _stod(t[1]), _stoi(t[2]), _stod(t[3]), _stoi(t[4]), _stod(t[5]),
                                       _stod(t[6]), _stod(t[7]), t[8]))
    n = len(species)
    k = 0.0
    for s in species:
        k += float(-s.charge_sign) * s.frac
    normden = [0.0] * n
    normden[1] = den
    normden[0] = den / k
    for i in range(2, n):
        normden[i] = species[i].frac * normden[0]
    t0, t1 = species[0].temp, species[1].temp
    LDe = math.sqrt((EPS_0 * K_B * t0 * EV_TO_K) / (normden[0] * QE * QE))
    wpe = math.sqrt((normden[0] * QE * QE) / (species[0].mass * EPS_0))
    wpi = math.sqrt((normden[1] * QE * QE) / (species[1].mass * EPS_0))
    LDi = math.sqrt((EPS_0 * K_B * t1 * EV_TO_K) / (normden[1] * QE * QE))
    if T_scale == "omegape":
        time_scale = wpe
    elif T_scale == "omegapi":
        time_scale = wpi
    else:
        time_scale = _stod(T_scale)
    dx = dy = DT = 0.0
    if norm_scheme in (2, 4):
        step = LDi
        dx = step / LDi
        dy = step / LDi
        DT = DT_coeff * (1.0 / wpi)
        DT = wpi * DT
    if norm_scheme in (1, 3):
        step = LDe
        dx = step / LDe
        dy = step / LDe
        DT = DT_coeff * (1.0 / wpe)
        DT = wpe * DT
    if norm_scheme == 5:
        step = L_scale
        dx = step / L_scale
        dy = step / L_scale
        DT = DT_coeff * (1.0 / time_scale)
        DT = time_scale * DT
    nx, ny = Nx + 1, Ny + 1
    Lx = (nx - 1) * dx
    Ly = (ny - 1) * dy
    if norm_scheme in (1, 3):
        L, W = LDe, wpe
    elif norm_scheme in (2, 4):
        L, W = LDi, (wpi if norm_scheme == 2 else wpe)
    elif norm_scheme == 5:
        L, W = L_scale, time_scale
        LDe, wpe = L, W
    else:
        raise ValueError("Invalid normscheme flag")
    vel_norm = L * W
    for i, s in enumerate(species):
        s.charge = s.charge_sign * QE
        s.spwt = normden[i] * Lx * Ly * L * L / s.numparticle
    return Setup(nx=nx, ny=ny, x0=x0, y0=x0, dx=dx, dy=dy, Lx=Lx, Ly=Ly, DT=DT, L=L, W=W, vel_norm=vel_norm,
                 LDe=LDe, wpe=wpe, LDi=LDi, wpi=wpi, density=den, shape=sim["shapefunction"], bc=sim["bc"],
                 solver=solver["solvertype"], tolerance=_stod(solver["tolerance"]),
                 max_iteration=_stoi(solver["max_iteration"]), gas_density=_stod(col["GAS_DENSITY"]),
                 elastic=string_to_bool(col["elastic"]), excitation=string_to_bool(col["excitation"]),
                 ionization=string_to_bool(col["ionization"]), num_ts=num_ts, ionfixed=_stoi(sim["ionfixed"]),
                 normscheme=norm_scheme, species=species, sor_omega=_stod(solver.get("sor_omega", "1.4")),
                 poisson_bc=solver.get("poisson_bc", "dirichlet"),
                 load_3v=string_to_bool(sim.get("load_3v", "false")),
                 grids=conductors(ini), emitters=emitters(ini))


def emitters(ini) -> np.ndarray:
    """The [Emitters] section as src/main.cpp:330-355 reads it."""
    e = ini.get("Emitters", {})
    rows = []
    for i in range(_stoi(e.get("count", "0"))):
        pre = "emitter_%d." % i
        rows.append([_stod(e[pre + "x0"]), _stod(e[pre + "y0"]), _stod(e[pre + "x1"]), _stod(e[pre + "y1"]),
                     _stod(e[pre + "temp"]), _stoi(e[pre + "numparticle"]), _stod(e[pre + "vdx"]),
                     _stod(e[pre + "vdy"]), _stoi(e[pre + "species_idx1"]), _stoi(e[pre + "species_idx2"])])
    return np.array(rows, dtype=np.float64).reshape(-1, 10)


def conductors(ini) -> np.ndarray:
    """The [Grids] section as src/main.cpp:284-327 reads it (voltages scaled by eV/(k_B EV_to_K))."""
    g = ini.get("Grids", {})
    rows = []
    vscale = EV / (K_B * EV_TO_K)
    for i in range(_stoi(g.get("grid_count", "0"))):
        pre = "grid_%d." % i
        t = g[pre + "type"]
        if t == "circular":
            rows.append([1, _stoi(g[pre + "x_center"]), _stoi(g[pre + "y_center"]), _stoi(g[pre + "electrode_number"]),
                         _stod(g[pre + "grid_radius"]), _stod(g[pre + "electrod_radius"]), 0,
                         vscale * _stod(g[pre + "electrode_voltage"])])
        elif t == "reactconduct":
            rows.append([0, _stoi(g[pre + "min_x"]), _stoi(g[pre + "max_x"]), _stoi(g[pre + "min_y"]),
                         _stoi(g[pre + "max_y"]), 0, 0, vscale * _stod(g[pre + "grid_voltage"])])
    return np.array(rows, dtype=np.float64).reshape(-1, 8)


def load_type(s: str):
    """INIParser::loadtypeextract (src/iniparser.cpp:100-113): "sin(3)" -> ("sin", 3)."""
    if "(" in s and ")" in s.split("(", 1)[1]:
        a, b = s.split("(", 1)
        return a, _stoi(b.split(")", 1)[0])
    return s, 0


# -------------------------------------------------------------- binding ---
class _Domain(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("x0", ctypes.c_double), ("y0", ctypes.c_double), ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("Lx", ctypes.c_double), ("Ly", ctypes.c_double),
                ("DT", ctypes.c_double), ("L", ctypes.c_double), ("W", ctypes.c_double),
                ("vel_norm", ctypes.c_double), ("LDe", ctypes.c_double), ("wpe", ctypes.c_double),
                ("density", ctypes.c_double),
                ("shape", ctypes.c_int), ("bc", ctypes.c_int),
                ("tolerance", ctypes.c_double), ("max_iteration", ctypes.c_int),
                ("gas_density", ctypes.c_double),
                ("elastic", ctypes.c_int), ("excitation", ctypes.c_int), ("ionization", ctypes.c_int),
                ("poisson_bc", ctypes.c_int), ("load_3v", ctypes.c_int)]


class _Rng(ctypes.Structure):
    _fields_ = [("mt", ctypes.c_uint32 * 624), ("mti", ctypes.c_int)]


class _Table(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("n", ctypes.c_long), ("de", ctypes.c_double),
                ("e_min", ctypes.c_double), ("e_max", ctypes.c_double), ("log_emin", ctypes.c_double),
                ("inv_dlog", ctypes.c_double), ("tot", ctypes.c_void_p), ("ela", ctypes.c_void_p),
                ("exc", ctypes.c_void_p), ("ion", ctypes.c_void_p)]


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def domain_struct(s: Setup) -> _Domain:
    return _Domain(s.nx, s.ny, s.x0, s.y0, s.dx, s.dy, s.Lx, s.Ly, s.DT, s.L, s.W, s.vel_norm, s.LDe, s.wpe,
                   s.density, SHAPE_CODES[s.shape], BC_CODES.get(s.bc, -1), s.tolerance, s.max_iteration,
                   s.gas_density, int(s.elastic), int(s.excitation), int(s.ionization),
                   POISSON_BC_CODES[s.poisson_bc], int(s.load_3v))


_LIB = None


def restatement_lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build_restatement()
        L = ctypes.CDLL(path)
        vp, i, l, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_double
        L.or_rng_seed.argtypes = [vp, ctypes.c_uint32]
        L.or_rng_uniform.argtypes = [vp]
        L.or_rng_uniform.restype = d
        L.or_rng_u32.argtypes = [vp]
        L.or_rng_u32.restype = ctypes.c_uint32
        L.or_load.argtypes = [vp, vp, ctypes.c_char_p, i, d, d, d, d, l, vp]
        L.or_load_c.argtypes = [vp, vp, ctypes.c_char_p, i, d, d, d, d, l, vp, vp, i]
        L.or_push_c.argtypes = [vp, d, d, i, vp, l, vp, vp, vp, i, i]
        L.or_push_c.restype = l
        L.or_conductor_rho.argtypes = [vp, vp, i, vp]
        L.or_in_conductors.argtypes = [vp, i, i, d, d]
        L.or_in_conductors.restype = i
        L.or_inject.argtypes = [vp, vp, d, d, vp, vp, vp, vp, vp, l, vp, vp, l]
        L.or_gsfluid_solve.argtypes = [vp, vp, vp, vp, vp]
        L.or_nrpcg_solve.argtypes = [vp, vp, vp, vp]
        L.or_nrpcg_solve.restype = l
        L.or_inject.restype = i
        L.or_scatter.argtypes = [vp, vp, l, d, vp]
        L.or_scatter.restype = l
        L.or_compute_rho.argtypes = [vp, i, vp, vp, vp]
        L.or_gs_solve.argtypes = [vp, d, vp, vp, vp, vp]
        L.or_pcg_solve.argtypes = [vp, vp, vp, vp, vp]
        L.or_efield.argtypes = [vp, vp, vp, vp]
        L.or_exact_sum.argtypes = [vp, l]
        L.or_exact_sum.restype = d
        L.or_push.argtypes = [vp, d, d, i, vp, l, vp, vp]
        L.or_push.restype = l
        L.or_rewind.argtypes = [vp, d, d, vp, l, vp, vp]
        L.or_cs_tables.argtypes = [vp, vp, vp, vp, vp]
        L.or_mcc.argtypes = [vp, vp, vp, vp, vp, vp, vp, l, d, d, vp, vp, l, i, vp, vp, i, vp]
        L.or_mcc.restype = l
        L.or_table_log.argtypes = [vp, l, d, d]
        L.or_mcc_table.argtypes = [vp, vp, vp, vp, l, d, d, vp, vp, l, i, vp, vp, i, vp]
        L.or_mcc_table.restype = l
        L.or_ke.argtypes = [vp, vp, l, d, d, d, d, i, vp]
        L.or_momentum.argtypes = [vp, vp, l, d, d, d, d, i, vp]
        L.or_pe.argtypes = [vp, vp, vp, d, d, i]
        L.or_pe.restype = d
        _LIB = L
    return _LIB


class Rng:
    def __init__(self, seed: int = 0):
        self.s = _Rng()
        restatement_lib().or_rng_seed(ctypes.byref(self.s), seed)

    def uniform(self) -> float:
        return restatement_lib().or_rng_uniform(ctypes.byref(self.s))

    def u32(self) -> int:
        return restatement_lib().or_rng_u32(ctypes.byref(self.s))


class Restatement:
    """Thin wrappers over oracle/epic_oracle.c for one Setup."""

    def __init__(self, s: Setup):
        self.s = s
        self.d = domain_struct(s)
        self.L = restatement_lib()
        self._cs = None

    def grid(self):
        return np.zeros(self.s.nx * self.s.ny)

    def load(self, rng: Rng, sp: SpeciesDesc) -> np.ndarray:
        t, n = load_type(sp.load)
        out = np.zeros((sp.numparticle, 5))
        g = np.ascontiguousarray(self.s.grids)
        rc = self.L.or_load_c(ctypes.byref(self.d), ctypes.byref(rng.s), t.encode(), n, sp.mass, sp.temp, sp.vsx,
                              sp.vsy, sp.numparticle, _p(out), _p(g), len(g))
        if rc == -2:
            raise ValueError("load type %r puts a particle inside a conductor (the reference loops forever)" % sp.load)
        if rc != 0:
            raise ValueError("unsupported load type %r" % sp.load)
        return out

    def inject(self, em, parts, rng, pos_u, vel_u=None):
        """Emitter::inject of one emitter row (src/emitter.cpp:5-36) appending to parts[idx1] (and
        parts[idx2]); pos_u: 2 uniforms per point; vel_u: 12 per point, else the stream rng."""
        i1, i2 = int(em[8]), int(em[9])
        num = int(em[5])
        sp = self.s.species
        out1 = np.zeros((len(parts[i1]) + num, 5))
        out1[:len(parts[i1])] = parts[i1]
        n1 = ctypes.c_long(len(parts[i1]))
        out2 = np.zeros((len(parts[i2]) + num, 5))
        out2[:len(parts[i2])] = parts[i2]
        n2 = ctypes.c_long(len(parts[i2]))
        em = np.ascontiguousarray(em, dtype=np.float64)
        pos_u = np.ascontiguousarray(pos_u, dtype=np.float64)
        vu = None if vel_u is None else np.ascontiguousarray(vel_u, dtype=np.float64)
        rc = self.L.or_inject(ctypes.byref(self.d), _p(em), sp[i1].mass, sp[i2].mass,
                              None if rng is None else ctypes.byref(rng.s), _p(pos_u), None if vu is None else _p(vu),
                              _p(out1), ctypes.byref(n1), len(out1), _p(out2), ctypes.byref(n2), len(out2))
        assert rc == 0
        parts = list(parts)
        parts[i1] = out1[:n1.value]
        if i2 != i1:
            parts[i2] = out2[:n2.value]
        return parts

    def conductor_rho(self, rho):
        """Grid::initialize of every conductor, as gssolver runs it (src/field.cpp:100-103)."""
        rho = np.ascontiguousarray(rho).copy()
        g = np.ascontiguousarray(self.s.grids)
        self.L.or_conductor_rho(ctypes.byref(self.d), _p(g), len(g), _p(rho))
        return rho

    def scatter(self, part: np.ndarray, spwt: float) -> np.ndarray:
        den = self.grid()
        part = np.ascontiguousarray(part)
        bad = self.L.or_scatter(ctypes.byref(self.d), _p(part), len(part), spwt, _p(den))
        if bad:
            raise IndexError("%d particles outside the grid" % bad)
        return den

    def compute_rho(self, dens, charges) -> np.ndarray:
        rho = self.grid()
        dens = [np.ascontiguousarray(x) for x in dens]
        ptrs = (ctypes.c_void_p * len(dens))(*[x.ctypes.data for x in dens])
        ch = np.asarray(charges, dtype=np.float64)
        self.L.or_compute_rho(ctypes.byref(self.d), len(dens), ptrs, _p(ch), _p(rho))
        return rho

    def gs_solve(self, rho, omega=1.4):
        phi = self.grid()
        err = ctypes.c_double()
        it = ctypes.c_int()
        conv = self.L.or_gs_solve(ctypes.byref(self.d), omega, _p(np.ascontiguousarray(rho)), _p(phi),
                                  ctypes.byref(err), ctypes.byref(it))
        return phi, err.value, it.value, bool(conv)

    def pcg_solve(self, rho):
        phi = self.grid()
        err = ctypes.c_double()
        it = ctypes.c_int()
        conv = self.L.or_pcg_solve(ctypes.byref(self.d), _p(np.ascontiguousarray(rho)), _p(phi), ctypes.byref(err),
                                   ctypes.byref(it))
        return phi, err.value, it.value, bool(conv)

    def gsfluid_solve(self, rho):
        """gsfluidsolver; returns (phi, error, iterations, converged, rho with its edge values)."""
        phi = self.grid()
        rho = np.ascontiguousarray(rho).copy()
        err = ctypes.c_double()
        it = ctypes.c_int()
        conv = self.L.or_gsfluid_solve(ctypes.byref(self.d), _p(rho), _p(phi), ctypes.byref(err), ctypes.byref(it))
        return phi, err.value, it.value, bool(conv), rho

    def nrpcg_solve(self, rho):
        phi = self.grid()
        err = ctypes.c_double()
        it = self.L.or_nrpcg_solve(ctypes.byref(self.d), _p(np.ascontiguousarray(rho)), _p(phi), ctypes.byref(err))
        return phi, err.value, it, True

    def solve(self, rho):
        if self.s.solver == "gs":
            return self.gs_solve(rho, self.s.sor_omega)
        if self.s.solver in ("cg", "iter", "iterative"):
            return self.pcg_solve(rho)
        if self.s.solver == "hybrid":
            return self.nrpcg_solve(rho)
        raise ValueError("solver %r not restated" % self.s.solver)

    def efield(self, phi):
        efx, efy = self.grid(), self.grid()
        self.L.or_efield(ctypes.byref(self.d), _p(np.ascontiguousarray(phi)), _p(efx), _p(efy))
        return efx, efy

    def push(self, sp: SpeciesDesc, part, efx, efy, sub_cycle=1, circles_live=False):
        part = np.ascontiguousarray(part).copy()
        g = np.ascontiguousarray(self.s.grids)
        n = self.L.or_push_c(ctypes.byref(self.d), sp.mass, sp.charge, sub_cycle, _p(part), len(part), _p(efx),
                             _p(efy), _p(g), len(g), int(circles_live))
        return part[:n]

    def rewind(self, sp: SpeciesDesc, part, efx, efy):
        part = np.ascontiguousarray(part).copy()
        self.L.or_rewind(ctypes.byref(self.d), sp.mass, sp.charge, _p(part), len(part), _p(efx), _p(efy))
        return part

    def cs_tables(self):
        if self._cs is None:
            t = [np.zeros(CS_RANGES) for _ in range(4)]
            self.L.or_cs_tables(ctypes.byref(self.d), *[_p(x) for x in t])
            self._cs = t
        return self._cs

    def set_log_table(self, ela, exc, ion, e_min, e_max):
        """Logarithmic cross-section table (extension); tot is formed as the
        C ABI forms it: (ela + exc + ion) * gas density."""
        ela, exc, ion = [np.ascontiguousarray(a, dtype=np.float64) for a in (ela, exc, ion)]
        tot = np.array([(a + b + c) * self.s.gas_density for a, b, c in zip(ela, exc, ion)])
        t = _Table()
        self.L.or_table_log(ctypes.byref(t), len(ela), e_min, e_max)
        t.tot, t.ela, t.exc, t.ion = tot.ctypes.data, ela.ctypes.data, exc.ctypes.data, ion.ctypes.data
        self._log = (t, tot, ela, exc, ion)

    def mcc(self, electrons, ions, ion_sp: SpeciesDesc, rng: Rng | None = None, uniforms=None, ustride=16):
        """Returns (electrons, ions, ncoll, kinds)."""
        if getattr(self, "_log", None) is None:
            tot, ela, exc, ion = self.cs_tables()
        ne, ni = len(electrons), len(ions)
        ecap, icap = 2 * ne + 16, ni + ne + 16
        e = np.zeros((ecap, 5))
        e[:ne] = electrons
        i_ = np.zeros((icap, 5))
        i_[:ni] = ions
        kinds = np.zeros(ne, dtype=np.int32)
        n_e = ctypes.c_long(ne)
        n_i = ctypes.c_long(ni)
        mode = 0 if rng is not None else 1
        u = None if uniforms is None else np.ascontiguousarray(uniforms, dtype=np.float64)
        if getattr(self, "_log", None) is not None:
            nc = self.L.or_mcc_table(ctypes.byref(self.d), ctypes.byref(self._log[0]), _p(e), ctypes.byref(n_e), ecap,
                                     ion_sp.mass, ion_sp.temp, _p(i_), ctypes.byref(n_i), icap, mode,
                                     ctypes.byref(rng.s) if rng is not None else None, _p(u), ustride, _p(kinds))
        else:
            nc = self.L.or_mcc(ctypes.byref(self.d), _p(tot), _p(ela), _p(exc), _p(ion), _p(e), ctypes.byref(n_e),
                               ecap, ion_sp.mass, ion_sp.temp, _p(i_), ctypes.byref(n_i), icap, mode,
                               ctypes.byref(rng.s) if rng is not None else None, _p(u), ustride, _p(kinds))
        if nc < 0:
            raise RuntimeError("capacity exceeded")
        return e[:n_e.value].copy(), i_[:n_i.value].copy(), nc, kinds

    def ke(self, sp: SpeciesDesc, part, norm: SpeciesDesc):
        out = np.zeros(3)
        self.L.or_ke(ctypes.byref(self.d), _p(np.ascontiguousarray(part)), len(part), sp.mass, sp.spwt, norm.temp,
                     norm.spwt, norm.numparticle, _p(out))
        return out

    def momentum(self, sp: SpeciesDesc, part, norm: SpeciesDesc):
        out = np.zeros(3)
        self.L.or_momentum(ctypes.byref(self.d), _p(np.ascontiguousarray(part)), len(part), sp.mass, sp.spwt,
                           norm.temp, norm.spwt, norm.numparticle, _p(out))
        return out

    def pe(self, efx, efy, norm: SpeciesDesc):
        return self.L.or_pe(ctypes.byref(self.d), _p(efx), _p(efy), norm.temp, norm.spwt, norm.numparticle)


class OracleSim:
    """The loop of src/main.cpp:359-423 on the restatement, conductors
    included (no emitters).  State: parts[s] (n,5) arrays, den[s], rho, phi,
    efx, efy."""

    def __init__(self, ini_path: str, load: bool = True, initial_field: bool = True, rng: Rng | None = None):
        self.s = setup(ini_path)
        self.R = Restatement(self.s)
        self.rng = rng or Rng(0)
        self.parts = [np.zeros((0, 5)) for _ in self.s.species]
        self.den = [self.R.grid() for _ in self.s.species]
        self.rho = self.R.grid()
        self.phi = self.R.grid()
        self.efx = self.R.grid()
        self.efy = self.R.grid()
        self.error = 0.0
        self.iters = 0
        self.circles_live = False  # circular grids have electrodes after the first gssolver call
        # positions of emitted particles: the reference seeds their generator from std::random_device
        self.pos_rng = np.random.default_rng(12345)
        if load:
            self.parts = [self.R.load(self.rng, sp) for sp in self.s.species]
        if initial_field:
            self.initial_field()

    def scatter_all(self):
        self.den = [self.R.scatter(p, sp.spwt) for p, sp in zip(self.parts, self.s.species)]
        self.rho = self.R.compute_rho(self.den, [sp.charge for sp in self.s.species])

    def field(self):
        if self.s.solver == "gs" and len(self.s.grids):
            self.rho = self.R.conductor_rho(self.rho)
            self.circles_live = True
        if self.s.solver == "gshybrid":  # gsfluidsolver edits domain.rho's edges
            self.phi, self.error, self.iters, _, self.rho = self.R.gsfluid_solve(self.rho)
        else:
            self.phi, self.error, self.iters, _ = self.R.solve(self.rho)
        self.efx, self.efy = self.R.efield(self.phi)

    def initial_field(self):
        self.scatter_all()
        self.field()
        self.parts = [self.R.rewind(sp, p, self.efx, self.efy) for p, sp in zip(self.parts, self.s.species)]

    def push_all(self):
        for k, sp in enumerate(self.s.species):
            if sp.name == "ion" and self.s.ionfixed == 1:
                continue
            self.parts[k] = self.R.push(sp, self.parts[k], self.efx, self.efy, circles_live=self.circles_live)

    def collide(self, uniforms=None):
        e, i, nc, kinds = self.R.mcc(self.parts[0], self.parts[1], self.s.species[1],
                                     rng=self.rng if uniforms is None else None, uniforms=uniforms)
        self.parts[0], self.parts[1] = e, i
        return nc, kinds

    def inject(self, pos_u=None, vel_u=None):
        """Every emitter, in order (src/main.cpp:397-403); pos_u / vel_u: one array per emitter."""
        for k, em in enumerate(self.s.emitters):
            pu = pos_u[k] if pos_u is not None else self.pos_rng.random(2 * int(em[5]))
            self.parts = self.R.inject(em, self.parts, self.rng, pu, None if vel_u is None else vel_u[k])

    def step(self, collisions=False, uniforms=None):
        if len(self.s.emitters):
            self.inject()
        self.scatter_all()
        self.field()
        self.push_all()
        if collisions:
            return self.collide(uniforms)
        return None


# --------------------------------------------------------- reference ---
class Reference:
    """The reference's own objects (oracle/_ref/libepic_ref.so)."""

    _lib = None

    @classmethod
    def available(cls) -> bool:
        try:
            cls.lib()
            return True
        except OSError:
            return False

    @classmethod
    def lib(cls):
        if cls._lib is None:
            path = build_oracle.build_reference()
            if path is None or not os.path.exists(path):
                raise OSError("reference objects not built (no reference checkout)")
            L = ctypes.CDLL(path)
            vp, i, l, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_double
            L.ref_create.restype = vp
            L.ref_create.argtypes = [ctypes.c_char_p, i, i]
            L.ref_error.restype = ctypes.c_char_p
            L.ref_error.argtypes = [vp]
            for nm, args in [("ref_destroy", [vp]), ("ref_params", [vp, vp]), ("ref_species_params", [vp, i, vp]),
                             ("ref_get_particles", [vp, i, vp]), ("ref_set_particles", [vp, i, vp, l]),
                             ("ref_get_grid", [vp, i, vp]), ("ref_set_grid", [vp, i, vp]),
                             ("ref_compute_rho", [vp]), ("ref_efield", [vp]),
                             ("ref_init_collisions", [vp]), ("ref_ke", [vp, i, i, vp]),
                             ("ref_momentum", [vp, i, i, vp]), ("ref_reset_rng", [])]:
                getattr(L, nm).argtypes = args
                getattr(L, nm).restype = None
            for nm, args in [("ref_scatter", [vp, i]), ("ref_solve", [vp]), ("ref_push", [vp, i, i]), ("ref_inject", [vp]),
                             ("ref_rewind", [vp, i]), ("ref_collide", [vp]), ("ref_step", [vp, i])]:
                getattr(L, nm).argtypes = args
                getattr(L, nm).restype = i
            L.ref_num_particles.argtypes = [vp, i]
            L.ref_num_particles.restype = l
            L.ref_solver_error.argtypes = [vp]
            L.ref_solver_error.restype = d
            L.ref_pe.argtypes = [vp, i]
            L.ref_pe.restype = d
            L.ref_rnd.restype = d
            cls._lib = L
        return cls._lib

    def __init__(self, ini_path: str, load: bool = True, initial_field: bool = True, reset_rng: bool = True):
        L = self.lib()
        if reset_rng:
            L.ref_reset_rng()
        self.h = L.ref_create(ini_path.encode(), int(load), int(initial_field))
        err = L.ref_error(self.h)
        if err:
            raise RuntimeError(err.decode())
        p = np.zeros(20)
        L.ref_params(self.h, _p(p))
        self.nx, self.ny = int(p[0]), int(p[1])
        self.params = p
        self.nsp = int(p[17])

    def __del__(self):
        if getattr(self, "h", None) and self._lib is not None:
            self._lib.ref_destroy(self.h)
            self.h = None

    def particles(self, sp: int) -> np.ndarray:
        n = self._lib.ref_num_particles(self.h, sp)
        out = np.zeros((n, 5))
        if n:
            self._lib.ref_get_particles(self.h, sp, _p(out))
        return out

    def set_particles(self, sp: int, part: np.ndarray):
        part = np.ascontiguousarray(part, dtype=np.float64)
        self._lib.ref_set_particles(self.h, sp, _p(part), len(part))

    def grid(self, which) -> np.ndarray:
        code = {"phi": 0, "rho": 1, "efx": 2, "efy": 3}.get(which, which)
        out = np.zeros(self.nx * self.ny)
        self._lib.ref_get_grid(self.h, code, _p(out))
        return out

    def set_grid(self, which, arr):
        code = {"phi": 0, "rho": 1, "efx": 2, "efy": 3}.get(which, which)
        self._lib.ref_set_grid(self.h, code, _p(np.ascontiguousarray(arr, dtype=np.float64)))

    def den(self, sp: int) -> np.ndarray:
        return self.grid(10 + sp)

    def species_params(self, sp: int) -> np.ndarray:
        out = np.zeros(8)
        self._lib.ref_species_params(self.h, sp, _p(out))
        return out

    _CHECKED = ("scatter", "solve", "push", "rewind", "collide", "step", "inject")

    def __getattr__(self, name):
        fn = getattr(self.lib(), "ref_" + name)
        if name in self._CHECKED:
            def call(*a):
                if fn(self.h, *a) != 0:
                    raise IndexError("reference raised: " + self._lib.ref_error(self.h).decode())
            return call
        return lambda *a: fn(self.h, *a)
