"""ctypes binding of the C ABI (include/epic2d.h).

:class:`Simulation` mirrors the reference's per-step interface — the methods of
Species, Domain, FieldSolve and CollisionHandler that src/main.cpp calls — over
one GPU-resident simulation.  There is no CPU implementation behind it: if the
CUDA library is missing the import fails.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libepic2d_gb300.so")

EPIC_OK = 0
EPIC_WARN_NOT_CONVERGED = 5
STATUS = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "CAPACITY", 5: "NOT_CONVERGED", 6: "DOMAIN",
          7: "TIMEOUT", 8: "BUDGET", 9: "IO"}
CIC, NGP = 0, 1
PBC, OPEN, REFLECTIVE = 0, 1, 2
SOLVER_GS, SOLVER_PCG = 0, 1
SOR_LEXICOGRAPHIC, SOR_REDBLACK = 0, 1
POISSON_DIRICHLET, POISSON_PERIODIC, POISSON_DIRICHLET_X = 0, 1, 2
DEPOSIT_FIXED, DEPOSIT_FP64 = 0, 1
MCC_PHILOX, MCC_INJECTED, MCC_NULL = 0, 1, 2
GRID = {"phi": 0, "rho": 1, "efx": 2, "efy": 3}


class EpicError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("x0", ctypes.c_double), ("y0", ctypes.c_double), ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("DT", ctypes.c_double), ("L", ctypes.c_double), ("W", ctypes.c_double),
                ("vel_norm", ctypes.c_double), ("LDe", ctypes.c_double), ("wpe", ctypes.c_double),
                ("LDi", ctypes.c_double), ("wpi", ctypes.c_double), ("density", ctypes.c_double),
                ("shape", ctypes.c_int), ("bc", ctypes.c_int), ("solver", ctypes.c_int),
                ("tolerance", ctypes.c_double), ("max_iteration", ctypes.c_int), ("ionfixed", ctypes.c_int),
                ("normscheme", ctypes.c_int), ("gas_density", ctypes.c_double),
                ("elastic", ctypes.c_int), ("excitation", ctypes.c_int), ("ionization", ctypes.c_int),
                ("sor_omega", ctypes.c_double), ("sor_mode", ctypes.c_int), ("deposit_mode", ctypes.c_int),
                ("mcc_mode", ctypes.c_int), ("seed", ctypes.c_uint64), ("warm_start", ctypes.c_int),
                ("solver_blocks", ctypes.c_int), ("precision", ctypes.c_int), ("sort_every", ctypes.c_int),
                ("push_order", ctypes.c_int), ("poisson_bc", ctypes.c_int), ("load_3v", ctypes.c_int),
                ("reserved", ctypes.c_int * 10)]


class SpeciesDesc(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("mass", ctypes.c_double), ("charge", ctypes.c_double),
                ("spwt", ctypes.c_double), ("temp", ctypes.c_double), ("numparticle", ctypes.c_int),
                ("vsx", ctypes.c_double), ("vsy", ctypes.c_double), ("fract_den", ctypes.c_double),
                ("load", ctypes.c_char * 32), ("capacity", ctypes.c_int64)]


class Conductor(ctypes.Structure):
    """epic_conductor: a ReactConductorGrid (type 0) or a CircularGrid (type 1), src/grid.cpp."""
    _fields_ = [("type", ctypes.c_int), ("min_x", ctypes.c_int), ("max_x", ctypes.c_int), ("min_y", ctypes.c_int),
                ("max_y", ctypes.c_int), ("x_center", ctypes.c_int), ("y_center", ctypes.c_int),
                ("electrode_number", ctypes.c_int), ("grid_radius", ctypes.c_double),
                ("electrode_radius", ctypes.c_double), ("voltage", ctypes.c_double), ("reserved", ctypes.c_int * 4)]


class Emitter(ctypes.Structure):
    """epic_emitter (src/emitter.cpp, include/emitter.h EmitterParams)."""
    _fields_ = [("x0", ctypes.c_double), ("y0", ctypes.c_double), ("x1", ctypes.c_double), ("y1", ctypes.c_double),
                ("temp", ctypes.c_double), ("numparticle", ctypes.c_int), ("vdx", ctypes.c_double),
                ("vdy", ctypes.c_double), ("species_idx1", ctypes.c_int), ("species_idx2", ctypes.c_int),
                ("reserved", ctypes.c_int * 4)]


def emitters_from_ini(path: str):
    """The [Emitters] section as epic_emitter records (src/main.cpp:330-355)."""
    n = ctypes.c_int()
    _check(lib().epic_emitters_from_ini(path.encode(), None, 0, ctypes.byref(n)))
    out = (Emitter * max(n.value, 1))()
    _check(lib().epic_emitters_from_ini(path.encode(), out, n.value, ctypes.byref(n)))
    return list(out)[:n.value]


def conductors_from_ini(path: str):
    """The [Grids] section as epic_conductor records (src/main.cpp:284-327)."""
    n = ctypes.c_int()
    _check(lib().epic_conductors_from_ini(path.encode(), None, 0, ctypes.byref(n)))
    out = (Conductor * max(n.value, 1))()
    _check(lib().epic_conductors_from_ini(path.encode(), out, n.value, ctypes.byref(n)))
    return list(out)[:n.value]


_lib = None


def lib() -> ctypes.CDLL:
    """Load the CUDA library (built by epic2d_mcc_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libepic2d_gb300.so is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(LIB_PATH)
    vp, i, i64, d, st = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_int
    pd = ctypes.POINTER(ctypes.c_double)
    sigs = {
        "epic_last_error": ([], ctypes.c_char_p),
        "epic_config_defaults": ([vp], None),
        "epic_config_from_ini": ([ctypes.c_char_p, vp, vp, i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)], st),
        "epic_create": ([vp, ctypes.POINTER(vp)], st),
        "epic_destroy": ([vp], None),
        "epic_add_species": ([vp, vp, ctypes.POINTER(ctypes.c_int)], st),
        "epic_load_particles": ([vp, ctypes.c_uint32], st),
        "epic_set_particles": ([vp, i, vp, i64], st),
        "epic_get_particles": ([vp, i, vp, i64, ctypes.POINTER(ctypes.c_int64)], st),
        "epic_num_particles": ([vp, i, ctypes.POINTER(ctypes.c_int64)], st),
        "epic_scatter_species": ([vp, i], st),
        "epic_compute_rho": ([vp], st),
        "epic_potential_solver": ([vp, ctypes.POINTER(ctypes.c_int), pd], st),
        "epic_calculate_efield": ([vp], st),
        "epic_push_species": ([vp, i, i], st),
        "epic_rewind_species": ([vp, i], st),
        "epic_sort_species": ([vp, i], st),
        "epic_initial_field_async": ([vp], st),
        "epic_run_async": ([vp, i, i], st),
        "epic_poll": ([vp, ctypes.POINTER(ctypes.c_int)], st),
        "epic_load_particles_device": ([vp, ctypes.c_uint64], st),
        "epic_digest": ([vp, vp], st),
        "epic_set_cross_sections": ([vp, vp, vp, vp, vp, i64, d], st),
        "epic_set_reference_cross_sections": ([vp], st),
        "epic_set_log_cross_sections": ([vp, vp, vp, vp, i64, d, d], st),
        "epic_handle_collisions": ([vp, i, i, vp, i, ctypes.POINTER(ctypes.c_int64)], st),
        "epic_step": ([vp, i], st),
        "epic_conductors_from_ini": ([ctypes.c_char_p, vp, i, ctypes.POINTER(ctypes.c_int)], st),
        "epic_add_conductor": ([vp, vp], st),
        "epic_emitters_from_ini": ([ctypes.c_char_p, vp, i, ctypes.POINTER(ctypes.c_int)], st),
        "epic_add_emitter": ([vp, vp], st),
        "epic_inject": ([vp, vp], st),
        "epic_step_host": ([vp, i, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)],
                           st),
        "epic_initial_field": ([vp], st),
        "epic_run_host": ([vp, i, i, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)],
                          st),
        "epic_init_species": ([vp, i], st),
        "epic_inject_emitter": ([vp, i, vp], st),
        "epic_set_spin_limit": ([ctypes.c_longlong], st),
        "epic_run": ([vp, i, i, i], st),
        "epic_compute_ke": ([vp, i, i, vp], st),
        "epic_compute_momentum": ([vp, i, i, vp], st),
        "epic_compute_pe": ([vp, i, pd], st),
        "epic_delta_phi": ([vp, pd], st),
        "epic_get_grid": ([vp, i, vp], st),
        "epic_set_grid": ([vp, i, vp], st),
        "epic_sync": ([vp], st),
        "epic_kernel_launches": ([vp], i64),
        "epic_stream": ([vp], vp),
        "epic_set_profiling": ([vp, i], st),
        "epic_get_profile": ([vp, vp, vp, ctypes.POINTER(ctypes.c_int64)], st),
        "epic_estimate_bytes": ([vp, vp, i, i], i64),
        "epic_server_create": ([i64, i, i, ctypes.POINTER(vp)], st),
        "epic_server_destroy": ([vp], None),
        "epic_server_set_log_cross_sections": ([vp, vp, vp, vp, i64, d, d], st),
        "epic_server_submit": ([vp, vp, ctypes.POINTER(ctypes.c_int64)], st),
        "epic_server_start": ([vp], st),
        "epic_server_wait": ([vp, d], st),
        "epic_server_result": ([vp, i64, vp], st),
        "epic_server_get_stats": ([vp, vp], st),
        "epic_batch_create": ([vp, i, i, ctypes.POINTER(vp)], st),
        "epic_batch_destroy": ([vp], None),
        "epic_batch_initial_field": ([vp], st),
        "epic_batch_run": ([vp, i, i], st),
        "epic_batch_get_particles": ([vp, i, i, vp, i64, ctypes.POINTER(ctypes.c_int64)], st),
        "epic_batch_get_grid": ([vp, i, i, vp], st),
        "epic_batch_num_particles": ([vp, ctypes.POINTER(ctypes.c_int64)], st),
        "epic_batch_tuning": ([vp, vp], st),
        "epic_batch_particle_tuning": ([vp, vp, vp, vp], st),
        "epic_batch_set_profiling": ([vp, i], st),
        "epic_batch_get_profile": ([vp, vp, vp], st),
        "epic_batch_stream": ([vp], vp),
        "epic_batch_set_log_cross_sections": ([vp, vp, vp, vp, i64, d, d], st),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _check(status: int, allow=(EPIC_OK,)):
    if status not in allow:
        raise EpicError(status, lib().epic_last_error().decode())
    return status


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def default_config() -> Config:
    c = Config()
    lib().epic_config_defaults(ctypes.byref(c))
    return c


def config_from_ini(path: str):
    """INIParser::parse + src/main.cpp set-up: returns (Config, [SpeciesDesc], NUM_TS)."""
    cfg = Config()
    descs = (SpeciesDesc * 8)()
    n = ctypes.c_int()
    ts = ctypes.c_int()
    _check(lib().epic_config_from_ini(path.encode(), ctypes.byref(cfg), descs, 8, ctypes.byref(n), ctypes.byref(ts)))
    return cfg, [descs[k] for k in range(min(n.value, 8))], ts.value


class Simulation:
    """One simulation resident on the GPU (Domain + species + FieldSolve + CollisionHandler)."""

    def __init__(self, cfg: Config, species):
        self._h = ctypes.c_void_p()
        _check(lib().epic_create(ctypes.byref(cfg), ctypes.byref(self._h)))
        self.cfg = cfg
        self.species = []
        for d in species:
            idx = ctypes.c_int()
            _check(lib().epic_add_species(self._h, ctypes.byref(d), ctypes.byref(idx)))
            self.species.append(d)
        self.nx, self.ny = cfg.nx, cfg.ny

    @classmethod
    def from_ini(cls, path: str, **overrides):
        """Config, species and the [Grids] conductors of an input.ini."""
        cfg, descs, _ = config_from_ini(path)
        for k, v in overrides.items():
            if k == "capacity":
                for d in descs:
                    d.capacity = int(v)
            else:
                setattr(cfg, k, v)
        sim = cls(cfg, descs)
        for c in conductors_from_ini(path):
            sim.add_conductor(c)
        for e in emitters_from_ini(path):
            sim.add_emitter(e)
        return sim

    def add_emitter(self, e: Emitter):
        _check(lib().epic_add_emitter(self._h, ctypes.byref(e)))

    def inject(self, uniforms: np.ndarray | None = None):
        """Emitter::inject of every emitter (epic_inject); uniforms: rows of 14 per emitted point."""
        u = None if uniforms is None else np.ascontiguousarray(uniforms, dtype=np.float64)
        _check(lib().epic_inject(self._h, None if u is None else _ptr(u)))

    def add_conductor(self, c: Conductor):
        _check(lib().epic_add_conductor(self._h, ctypes.byref(c)))

    def close(self):
        if self._h:
            lib().epic_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- particles ---
    def load_particles(self, seed: int = 0):
        _check(lib().epic_load_particles(self._h, seed))

    def set_particles(self, sp: int, parts: np.ndarray):
        parts = np.ascontiguousarray(parts, dtype=np.float64).reshape(-1, 5)
        _check(lib().epic_set_particles(self._h, sp, _ptr(parts), len(parts)))

    def num_particles(self, sp: int) -> int:
        n = ctypes.c_int64()
        _check(lib().epic_num_particles(self._h, sp, ctypes.byref(n)))
        return n.value

    def particles_into(self, sp: int, out: np.ndarray) -> int:
        """Download species `sp` into a caller-owned (capacity, 5) float64 array; returns the count."""
        got = ctypes.c_int64()
        _check(lib().epic_get_particles(self._h, sp, _ptr(out), len(out), ctypes.byref(got)))
        return got.value

    def particles(self, sp: int) -> np.ndarray:
        n = self.num_particles(sp)
        out = np.zeros((max(n, 1), 5))
        got = ctypes.c_int64()
        _check(lib().epic_get_particles(self._h, sp, _ptr(out), len(out), ctypes.byref(got)))
        return out[:got.value]

    # --- the loop, phase by phase ---
    def scatter_species(self, sp: int):
        _check(lib().epic_scatter_species(self._h, sp))

    def compute_rho(self):
        _check(lib().epic_compute_rho(self._h))

    def potential_solver(self):
        it = ctypes.c_int()
        err = ctypes.c_double()
        st = _check(lib().epic_potential_solver(self._h, ctypes.byref(it), ctypes.byref(err)),
                    allow=(EPIC_OK, EPIC_WARN_NOT_CONVERGED))
        return it.value, err.value, st == EPIC_OK

    def calculate_efield(self):
        _check(lib().epic_calculate_efield(self._h))

    def push_species(self, sp: int, sub_cycle: int = 1):
        _check(lib().epic_push_species(self._h, sp, sub_cycle))

    def rewind_species(self, sp: int):
        _check(lib().epic_rewind_species(self._h, sp))

    def load_particles_device(self, seed: int = 0):
        """Loads every species on the GPU (Philox uniforms, the reference's placement and velocity formula)."""
        _check(lib().epic_load_particles_device(self._h, seed))
        self.sync()

    def digest(self):
        """(phi hash, particles hash): order-independent 64-bit digests of the run's state."""
        out = np.zeros(2, dtype=np.uint64)
        _check(lib().epic_digest(self._h, _ptr(out)))
        return int(out[0]), int(out[1])

    def sort_species(self, sp: int):
        """Stable sort of the species' particles by cell (i*ny + j)."""
        _check(lib().epic_sort_species(self._h, sp))

    def set_reference_cross_sections(self):
        _check(lib().epic_set_reference_cross_sections(self._h))

    def set_cross_sections(self, tot, ela, exc, ion, de):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (tot, ela, exc, ion)]
        _check(lib().epic_set_cross_sections(self._h, *[_ptr(a) for a in arrs], len(arrs[0]), de))

    def set_log_cross_sections(self, ela, exc, ion, e_min, e_max):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (ela, exc, ion)]
        _check(lib().epic_set_log_cross_sections(self._h, *[_ptr(a) for a in arrs], len(arrs[0]), e_min, e_max))

    def handle_collisions(self, electrons: int = 0, ions: int = 1, uniforms: np.ndarray | None = None,
                          ustride: int = 16) -> int:
        nc = ctypes.c_int64()
        u = None if uniforms is None else np.ascontiguousarray(uniforms, dtype=np.float64)
        _check(lib().epic_handle_collisions(self._h, electrons, ions, None if u is None else _ptr(u), ustride,
                                            ctypes.byref(nc)))
        return nc.value

    def step(self, collisions: bool = False):
        _check(lib().epic_step(self._h, int(collisions)))

    def step_host(self, bufs, counts, collisions: bool = False):
        """One step of particles held in host arrays (epic_step_host): bufs[s] is a (capacity, 5)
        float64 array whose first counts[s] rows are species s; returns the new counts.  Pinned
        arrays (e.g. torch pin_memory) take the direct path."""
        nsp = len(self.species)
        for b in bufs:
            if b.dtype != np.float64 or not b.flags["C_CONTIGUOUS"] or b.ndim != 2 or b.shape[1] != 5:
                raise ValueError("each buffer must be a C-contiguous (capacity, 5) float64 array")
        ptrs = (ctypes.c_void_p * nsp)(*[b.ctypes.data for b in bufs])
        n = (ctypes.c_int64 * nsp)(*[int(c) for c in counts])
        cap = (ctypes.c_int64 * nsp)(*[len(b) for b in bufs])
        _check(lib().epic_step_host(self._h, int(collisions), ptrs, n, cap))
        return [int(v) for v in n]

    def run_host(self, bufs, counts, steps: int, collisions: bool = False):
        """`steps` steps of particles held in host arrays (epic_run_host): bufs[s] is a (capacity, 5)
        float64 array whose first counts[s] rows are species s; every step's records go to the
        arrays and back; returns the final counts.  Pinned arrays take the copy-engine path."""
        nsp = len(self.species)
        for b in bufs:
            if b.dtype != np.float64 or not b.flags["C_CONTIGUOUS"] or b.ndim != 2 or b.shape[1] != 5:
                raise ValueError("each buffer must be a C-contiguous (capacity, 5) float64 array")
        ptrs = (ctypes.c_void_p * nsp)(*[b.ctypes.data for b in bufs])
        n = (ctypes.c_int64 * nsp)(*[int(c) for c in counts])
        cap = (ctypes.c_int64 * nsp)(*[len(b) for b in bufs])
        _check(lib().epic_run_host(self._h, int(steps), int(collisions), ptrs, n, cap))
        return [int(v) for v in n]

    def init_species(self, sp: int):
        """Init of one species from the handle's copy of the reference's generator (epic_init_species)."""
        _check(lib().epic_init_species(self._h, sp))

    def initial_field(self):
        _check(lib().epic_initial_field(self._h))

    def run(self, steps: int, collisions: bool = False, graph: bool = True):
        _check(lib().epic_run(self._h, steps, int(collisions), int(graph)))

    # --- diagnostics ---
    def compute_ke(self, sp: int, norm: int = 0) -> np.ndarray:
        out = np.zeros(3)
        _check(lib().epic_compute_ke(self._h, sp, norm, _ptr(out)))
        return out

    def compute_momentum(self, sp: int, norm: int = 0) -> np.ndarray:
        out = np.zeros(3)
        _check(lib().epic_compute_momentum(self._h, sp, norm, _ptr(out)))
        return out

    def compute_pe(self, norm: int = 0) -> float:
        v = ctypes.c_double()
        _check(lib().epic_compute_pe(self._h, norm, ctypes.byref(v)))
        return v.value

    def delta_phi(self) -> float:
        v = ctypes.c_double()
        _check(lib().epic_delta_phi(self._h, ctypes.byref(v)))
        return v.value

    def grid(self, which) -> np.ndarray:
        code = GRID.get(which, which)
        out = np.zeros(self.nx * self.ny)
        _check(lib().epic_get_grid(self._h, code, _ptr(out)))
        return out

    def den(self, sp: int) -> np.ndarray:
        return self.grid(10 + sp)

    def set_grid(self, which, arr):
        """Sets a node grid (nx * ny values, i-major) from the host; an array of another size is refused (the C
        entry point copies nx * ny values)."""
        code = GRID.get(which, which)
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
        if a.size != self.cfg.nx * self.cfg.ny:
            raise ValueError("grid %r needs %d x %d = %d values, got %d" % (which, self.cfg.nx, self.cfg.ny,
                                                                        self.cfg.nx * self.cfg.ny, a.size))
        _check(lib().epic_set_grid(self._h, code, _ptr(a)))

    def sync(self):
        _check(lib().epic_sync(self._h))

    @property
    def launches(self) -> int:
        return lib().epic_kernel_launches(self._h)

    @property
    def stream(self) -> int:
        return lib().epic_stream(self._h) or 0

    PHASES = ("deposit", "finalize", "solve", "efield", "push", "mcc", "sort")

    def set_profiling(self, on: bool = True):
        _check(lib().epic_set_profiling(self._h, int(on)))

    def profile(self):
        """{phase: (ms, launches)} accumulated since the last call, plus solver iterations."""
        ms = np.zeros(len(self.PHASES))
        cnt = np.zeros(len(self.PHASES), dtype=np.int64)
        it = ctypes.c_int64()
        _check(lib().epic_get_profile(self._h, _ptr(ms), _ptr(cnt), ctypes.byref(it)))
        return {p: (float(ms[k]), int(cnt[k])) for k, p in enumerate(self.PHASES)}, it.value


# ------------------------------------------------------------------ serving ---
REQUEST_MAX_CONDUCTORS = REQUEST_MAX_EMITTERS = 8


class Request(ctypes.Structure):
    _fields_ = [("cfg", Config), ("species", SpeciesDesc * 8), ("num_species", ctypes.c_int),
                ("steps", ctypes.c_int), ("collisions", ctypes.c_int), ("load_seed", ctypes.c_uint64),
                ("arrival_s", ctypes.c_double), ("num_conductors", ctypes.c_int),
                ("conductors", Conductor * REQUEST_MAX_CONDUCTORS), ("num_emitters", ctypes.c_int),
                ("emitters", Emitter * REQUEST_MAX_EMITTERS)]


class Result(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("status", ctypes.c_int), ("arrival_s", ctypes.c_double),
                ("admit_s", ctypes.c_double), ("finish_s", ctypes.c_double), ("particle_steps", ctypes.c_int64),
                ("bytes", ctypes.c_int64), ("digest", ctypes.c_uint64 * 2), ("kinetic_energy", ctypes.c_double),
                ("potential_energy", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("failed", ctypes.c_int64),
                ("p50_latency_s", ctypes.c_double), ("p99_latency_s", ctypes.c_double),
                ("mean_latency_s", ctypes.c_double), ("max_latency_s", ctypes.c_double),
                ("makespan_s", ctypes.c_double), ("particle_steps_per_s", ctypes.c_double),
                ("peak_bytes", ctypes.c_int64), ("peak_inflight", ctypes.c_int)]


def make_request(path: str, steps: int, collisions: bool = False, seed: int = 0, arrival_s: float = 0.0,
                 **overrides) -> Request:
    """A serving request from an input deck (config overrides as in Simulation.from_ini)."""
    cfg, descs, _ = config_from_ini(path)
    for k, v in overrides.items():
        if k == "capacity":
            for d in descs:
                d.capacity = int(v)
        else:
            setattr(cfg, k, v)
    r = Request()
    r.cfg = cfg
    for k, d in enumerate(descs):
        r.species[k] = d
    r.num_species = len(descs)
    r.steps = int(steps)
    r.collisions = int(bool(collisions))
    r.load_seed = int(seed)
    r.arrival_s = float(arrival_s)
    conds, ems = conductors_from_ini(path), emitters_from_ini(path)
    if len(conds) > REQUEST_MAX_CONDUCTORS or len(ems) > REQUEST_MAX_EMITTERS:
        raise ValueError("a request carries at most %d conductors and %d emitters" % (REQUEST_MAX_CONDUCTORS,
                                                                                     REQUEST_MAX_EMITTERS))
    r.num_conductors = len(conds)
    for k, c in enumerate(conds):
        r.conductors[k] = c
    r.num_emitters = len(ems)
    for k, e in enumerate(ems):
        r.emitters[k] = e
    return r


def estimate_bytes(req: Request) -> int:
    return lib().epic_estimate_bytes(ctypes.byref(req.cfg), req.species, req.num_species, req.collisions)


class Server:
    """Continuous-batching serving loop (include/epic2d_serve.h)."""

    def __init__(self, budget_bytes: int, max_inflight: int = 8, chunk_steps: int = 16):
        self._h = ctypes.c_void_p()
        _check(lib().epic_server_create(int(budget_bytes), int(max_inflight), int(chunk_steps), ctypes.byref(self._h)))

    def set_log_cross_sections(self, ela, exc, ion, e_min, e_max):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (ela, exc, ion)]
        _check(lib().epic_server_set_log_cross_sections(self._h, *[_ptr(a) for a in arrs], len(arrs[0]),
                                                        e_min, e_max))

    def submit(self, req: Request) -> int:
        i = ctypes.c_int64()
        _check(lib().epic_server_submit(self._h, ctypes.byref(req), ctypes.byref(i)))
        return i.value

    def start(self):
        _check(lib().epic_server_start(self._h))

    def wait(self, timeout_s: float = 600.0):
        _check(lib().epic_server_wait(self._h, timeout_s))

    def result(self, rid: int) -> Result:
        r = Result()
        _check(lib().epic_server_result(self._h, rid, ctypes.byref(r)))
        return r

    def stats(self) -> ServerStats:
        s = ServerStats()
        _check(lib().epic_server_get_stats(self._h, ctypes.byref(s)))
        return s

    def close(self):
        if self._h:
            lib().epic_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ batching ---
class Batch:
    """Many runs advanced together, one launch per phase (include/epic2d_batch.h)."""

    def __init__(self, requests, sort_every: int = 16):
        arr = (Request * len(requests))(*requests)
        self._h = ctypes.c_void_p()
        self.requests = list(requests)
        _check(lib().epic_batch_create(arr, len(requests), int(sort_every), ctypes.byref(self._h)))

    def set_log_cross_sections(self, ela, exc, ion, e_min, e_max):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (ela, exc, ion)]
        _check(lib().epic_batch_set_log_cross_sections(self._h, *[_ptr(a) for a in arrs], len(arrs[0]), e_min, e_max))

    def initial_field(self):
        _check(lib().epic_batch_initial_field(self._h))

    def run(self, steps: int, graph: bool = True):
        _check(lib().epic_batch_run(self._h, int(steps), int(graph)))

    def particles(self, run: int, sp: int) -> np.ndarray:
        n = self.requests[run].species[sp].numparticle
        if self.requests[run].collisions:
            n = 2 * n + 8192  # ionisation adds particles
        while True:
            out = np.empty((max(n, 1), 5), dtype=np.float64)
            got = ctypes.c_int64()
            st = lib().epic_batch_get_particles(self._h, run, sp, _ptr(out), len(out), ctypes.byref(got))
            if st == 4 and got.value > len(out):  # CAPACITY: emitters added more; the count came back
                n = got.value
                continue
            _check(st)
            return out[:got.value]

    def grid(self, run: int, which: str = "phi") -> np.ndarray:
        c = self.requests[run].cfg
        out = np.empty(c.nx * c.ny, dtype=np.float64)  # node (i, j) at i*ny + j, as Simulation.grid
        _check(lib().epic_batch_get_grid(self._h, run, GRID[which], _ptr(out)))
        return out

    def num_particles(self) -> int:
        n = ctypes.c_int64()
        _check(lib().epic_batch_num_particles(self._h, ctypes.byref(n)))
        return n.value

    def tuning(self):
        t = np.zeros(4, dtype=np.int32)
        _check(lib().epic_batch_tuning(self._h, _ptr(t)))
        return [int(x) for x in t]

    def set_profiling(self, on: bool = True):
        _check(lib().epic_batch_set_profiling(self._h, 1 if on else 0))

    def profile(self):
        """{phase: (ms, count)} accumulated since the last call (directly launched steps only)."""
        ms = np.zeros(7, dtype=np.float64)
        cnt = np.zeros(7, dtype=np.int64)
        _check(lib().epic_batch_get_profile(self._h, _ptr(ms), _ptr(cnt)))
        return {name: (float(ms[k]), int(cnt[k])) for k, name in enumerate(Simulation.PHASES)}

    def particle_tuning(self):
        """The autotuner's launch shapes of the fused push and the deposit pass, with the timings behind them."""
        sh = np.zeros(4, dtype=np.int32)
        pm = np.zeros(5, dtype=np.float32)
        dm = np.zeros(6, dtype=np.float32)
        _check(lib().epic_batch_particle_tuning(self._h, _ptr(sh), _ptr(pm), _ptr(dm)))
        return {"push_threads": int(sh[0]), "push_blocks": int(sh[1]), "deposit_threads": int(sh[2]),
                "deposit_blocks": int(sh[3]),
                "push_ms_by_shape": dict(zip(["128 resident", "256 resident", "256 x 1/SM", "256 x 2/SM",
                                              "128 x 3/SM"], [round(float(x), 4) for x in pm])),
                "deposit_ms_by_shape": dict(zip(["128 resident", "256 resident", "256 x 4/SM", "256 x 8/SM",
                                                 "256 x 16/SM", "128 x 8/SM"], [round(float(x), 4) for x in dm]))}

    @property
    def stream(self) -> int:
        return lib().epic_batch_stream(self._h) or 0

    def close(self):
        if self._h:
            lib().epic_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
