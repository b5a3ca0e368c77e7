#!/usr/bin/env python3
"""Benchmark of the ePIC2D time-step loop on GB300.

One "step" is one iteration of the loop body of the reference (deposit of all
species, charge density, Poisson solve, E-field, push of all species, MCC) on
the GPU-resident workload.  Prints one JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

* value      — particle-steps/s with all state resident in HBM (CUDA events on
               the simulation's stream around K steps).
* e2e        — the same metric through the public API with host-owned
               particles: every step's input records are copied from pinned
               host memory and its stepped records copied back to it
               (epic_run_host: copy engines carry both directions at once
               while the SMs run the next step's solve).
* roofline   — the dominant phase's algorithmic bytes per launch over its
               measured average launch time, against the measured HBM copy
               bandwidth.
* cpu_baseline — the oracle's C restatement of the reference loop timed on
               this host for a bounded sample of the same workload.
* extension_rows — conductors, emitters and the two Boltzmann-electron
               solvers, each on its own deck (10 steps after 3 warm-up), with
               the oracle on one host core beside them (--no-rows skips;
               --rows runs only these).
* --impl reference — the reference's CPU implementation of the loop (the
               restatement, or the reference's own objects where they were
               compiled on this machine) on the same workload, one full loop
               iteration per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "beam_mcc_256"
METRIC = "particle-steps/s on 1 GB300 (plain FP64 time-step loop)"
UNIT = "particle-steps/s"
SORT_EVERY = 16  # cell-sort period of the mixed form (the mixed decks' default)
REF_BUDGET_S = 150.0  # bound on the reference arm's timed CPU loop

# Algorithmic bytes per unit of each phase (FP64 plain form).
BYTES = {
    "push": 64,       # per particle: x, y, vx, vy read + written
    "deposit": 16,    # per particle: x, y read (accumulation stays in L2)
    "mcc": 24,        # per electron: vx, vy, vz read (collided ones also written)
    "solve": 88,      # per node per PCG iteration (11 FP64 words)
    "finalize": 24,   # per node per species: accumulator read + density write + rho share
    "efield": 40,     # per node: phi read, efx, efy, (efx, efy) written
}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            # the sampler is up (its first sample written) before the timed region starts
            t0 = time.time()
            while time.time() - t0 < 5 and os.path.getsize(self.path) == 0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.remove(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, r in rows for k in range(4) if r[k].lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def write_deck(name):
    from epic2d_mcc_gb300 import workloads

    d = tempfile.mkdtemp(prefix="epic_bench_")
    path = os.path.join(d, name + ".ini")
    with open(path, "w") as f:
        f.write(workloads.deck(name))
    return path


def collisions_on(ini):
    from oracle import oracle as O

    s = O.setup(ini)
    return s.elastic or s.excitation or s.ionization


# ------------------------------------------------------------ CPU arm ---
def cpu_port_run(ini, steps, warmup, budget_s=None):
    """The oracle restatement of the reference loop (single thread, as the
    reference).  Returns (particle-steps/s, steps timed, particles, kind)."""
    from epic2d_mcc_gb300 import workloads
    from oracle import oracle as O

    coll = collisions_on(ini)
    sim = O.OracleSim(ini)
    if coll:
        e, ela, exc, ion = workloads.synthetic_table()
        sim.R.set_log_table(ela, exc, ion, e[0], e[-1])
    for _ in range(warmup):
        sim.step(collisions=coll)
    done, n_acc = 0, 0
    t0 = time.perf_counter()
    while True:
        n_acc += sum(len(p) for p in sim.parts)
        sim.step(collisions=coll)
        done += 1
        el = time.perf_counter() - t0
        if steps is not None and done >= steps:
            break
        if budget_s is not None and el >= budget_s:
            break
    el = time.perf_counter() - t0
    return n_acc / el, done, n_acc // done, "port"


def workload_config(ini, name, world=1):
    """The workload as both arms report it (from the deck: the same dict for
    the GPU arm and the reference arm)."""
    from oracle import oracle as O

    s = O.setup(ini)
    coll = bool(s.elastic or s.excitation or s.ionization)
    solver = {"cg": "PCG", "gs": "SOR"}.get(s.solver, s.solver)
    n = int(sum(sp.numparticle for sp in s.species))
    return {"workload": name, "particles": n, "grid": [s.nx, s.ny],
            "solver": "%s tol %g (cold start, as the reference)" % (solver, s.tolerance),
            "field_bc": {"dirichlet": "phi = 0 on all edges (the reference's)", "periodic": "periodic",
                         "dirichlet_x": "phi = 0 on the x walls, periodic in y"}.get(s.poisson_bc, s.poisson_bc),
            "particle_bc": {"pbc": "periodic", "open": "absorbing", "reflective": "reflecting"}.get(s.bc, s.bc),
            "mcc": "direct MCC, 1000-point log table" if coll else "off",
            "l2": "inputs larger than L2 (particles %.0f MB)" % (n * 40 / 1e6),
            "parallelism": "replicas" if world > 1 else "single run"}


def _cpu_run_worker(job):
    """One reference loop (oracle restatement, one thread) on one deck for
    budget_s seconds after its load and initial field: (particle-steps, s)."""
    ini, coll, budget_s = job
    from epic2d_mcc_gb300 import workloads
    from oracle import oracle as O

    sim = O.OracleSim(ini)
    if coll:
        e, ela, exc, ion = workloads.synthetic_table()
        sim.R.set_log_table(ela, exc, ion, e[0], e[-1])
    n_acc, t0 = 0, time.perf_counter()
    while True:
        n_acc += sum(len(p) for p in sim.parts)
        sim.step(collisions=coll)
        if time.perf_counter() - t0 >= budget_s:
            break
    return n_acc, time.perf_counter() - t0


def cpu_multi_run(jobs, budget_s):
    """Many runs on the host cores at once, one reference loop per core (the
    reference is serial, so concurrent runs are how a CPU serves many):
    aggregate particle-steps/s of len(jobs) concurrent processes.  A spawned
    pool (this process has already used the GPU)."""
    import multiprocessing as mp

    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        res = pool.map(_cpu_run_worker, [(ini, coll, budget_s) for ini, coll in jobs])
    return sum(r[0] / r[1] for r in res)


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


CPU_MULTI_SECONDS = 8.0  # per process, after its load and initial field


def run_reference(args, rank, world):
    if rank != 0:
        return
    ini = write_deck(args.workload)
    # One loop iteration of the reference takes ~1 s on this workload: at most
    # one warm-up iteration, and the timed iterations stop at REF_BUDGET_S.
    value, done, n, kind = cpu_port_run(ini, args.steps, min(args.warmup, 1), budget_s=REF_BUDGET_S)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": done, "warmup": min(args.warmup, 1), "ms_per_step": n / value * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (particles loaded from mt19937 seed 0, as the reference's Init)",
            "config": workload_config(ini, args.workload),
            "particles_stepped": n,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": kind,
                             "sample": "%d full loop iterations of %s (%d particles), single thread; the "
                                       "reference loop is serial" % (done, args.workload, n)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ GPU arm ---
def over_ranks(x, op, dist, device):
    """x reduced over the ranks of a replica run (max of times, sum of work);
    x itself on a single rank.  No data-path collective: one scalar per run."""
    if not dist:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def replica_value(particle_steps_rank, ms_rank, dist=None, device="cuda"):
    """Whole-job particle-steps/s of N replicas: all ranks' particle-steps over
    the slowest rank's time."""
    ms_max = over_ranks(ms_rank, "max", dist, device)
    return over_ranks(particle_steps_rank, "sum", dist, device) / (ms_max / 1e3), ms_max


def run_ours(args, rank, world):
    import numpy as np
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    import epic2d_mcc_gb300 as E
    from epic2d_mcc_gb300 import build as B
    from epic2d_mcc_gb300 import workloads

    B.build()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()

    def max_over_ranks(x):
        return over_ranks(x, "max", dist, "cuda")

    def sum_over_ranks(x):
        return over_ranks(x, "sum", dist, "cuda")

    ini = write_deck(args.workload)
    coll = collisions_on(ini)
    sim = E.Simulation.from_ini(ini)
    if coll:
        e, ela, exc, ion = workloads.synthetic_table()
        sim.set_log_cross_sections(ela, exc, ion, e[0], e[-1])
    sim.load_particles(0)
    sim.initial_field()
    nsp = len(sim.species)
    # warm-up by graph replay (the step graph is captured in the first call)
    for _ in range(args.warmup):
        sim.run(1, collisions=coll, graph=True)
    stream = torch.cuda.ExternalStream(sim.stream)
    n_before = sum(sim.num_particles(s) for s in range(nsp))
    launches0 = sim.launches
    clocks = Clocks(local)
    barrier()
    torch.cuda.synchronize()
    sim.sync()
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    sim.run(args.steps, collisions=coll, graph=True)  # the loop as epic_run runs it: the step graph replayed
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    launches = sim.launches - launches0
    n_after = sum(sim.num_particles(s) for s in range(nsp))
    pst_rank = 0.5 * (n_before + n_after) * args.steps
    value, ms_max = replica_value(pst_rank, ms, dist, "cuda")
    # phase split: as many more steps launched directly with the phase timers on
    sim.set_profiling(True)
    sim.profile()
    sim.run(args.steps, collisions=coll, graph=False)
    prof, iters = sim.profile()
    sim.set_profiling(False)

    # roofline of the dominant phase
    g = sim.cfg
    nodes = g.nx * g.ny
    n_e = sim.num_particles(0)
    dom = max(prof, key=lambda k: prof[k][0])
    d_ms, d_launch = prof[dom]
    if dom == "solve":
        per_step_bytes = BYTES["solve"] * nodes * (iters / max(d_launch, 1))
    elif dom in ("push", "deposit"):
        per_step_bytes = BYTES[dom] * 0.5 * (n_before + n_after) / nsp
    elif dom == "mcc":
        per_step_bytes = BYTES["mcc"] * n_e
    else:
        per_step_bytes = BYTES[dom] * nodes * (nsp if dom == "finalize" else 1)
    achieved = per_step_bytes / (d_ms / max(d_launch, 1) / 1e3) / 1e9
    peak, peak_kind = load_peaks()
    traffic = TRAFFIC.get(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": per_step_bytes, "avg_launch_ms": d_ms / max(d_launch, 1),
                "phases_ms_per_step": {k: v[0] / args.steps for k, v in prof.items()},
                "solver_iterations_per_step": iters / args.steps}

    # e2e through the public API with host-owned particles
    caps = [sim.species[s].capacity or (sim.species[s].numparticle * 3 // 2 + 4096) for s in range(nsp)]
    bufs = [torch.empty((int(c), 5), dtype=torch.float64, pin_memory=True).numpy() for c in caps]
    counts = [sim.particles_into(s, bufs[s]) for s in range(nsp)]
    counts = sim.run_host(bufs, counts, 1, collisions=coll)  # warm-up: streams, events, staging
    e2e_steps = max(1, min(args.steps, 20))
    n_in = sum(counts)
    barrier()
    t0 = time.perf_counter()
    # epic_run_host: every step's input records are copied from the pinned host
    # arrays and its stepped records copied back into them (copy engines,
    # beside the next step's solve); the counts come back at the end.
    counts = sim.run_host(bufs, counts, e2e_steps, collisions=coll)
    el = time.perf_counter() - t0
    el = max_over_ranks(el)
    n_out = sum(counts)
    h2d = d2h = int(0.5 * (n_in + n_out) * 40 * e2e_steps)
    e2e_value = sum_over_ranks(0.5 * (n_in + n_out) * e2e_steps) / el

    # The mixed-precision form on the same workload from the same start (the
    # FP64 run above advanced warmup + steps + e2e steps; compare at equal steps).
    mixed = None
    if not args.no_mixed:
        total_steps = args.warmup + 2 * args.steps + 1 + e2e_steps
        # The mixed form sorts particles by cell every SORT_EVERY steps: warm up
        # and time whole sort periods so the sort's cost is in the timed steps.
        # The FP64 comparison run sorts on the same steps: MCC draws are keyed by
        # a particle's position in the array, so both runs must order their
        # particles alike to draw the same collisions.
        ref = E.Simulation.from_ini(ini, sort_every=SORT_EVERY)
        mx = E.Simulation.from_ini(ini, precision=1, sort_every=SORT_EVERY)
        for s_ in (ref, mx):
            if coll:
                s_.set_log_cross_sections(ela, exc, ion, e[0], e[-1])
            s_.load_particles(0)
            s_.initial_field()
        del sim

        def energy(sm):
            return sum(sm.compute_ke(k, 0).sum() for k in range(nsp)) + sm.compute_pe(0)

        def errors(a, b):
            pa = a.grid("phi")
            return (abs(energy(b) - energy(a)) / abs(energy(a)),
                    float(np.max(np.abs(b.grid("phi") - pa)) / np.max(np.abs(pa))))

        # Accuracy: one sort period of both forms from the same start.  Later
        # differences grow by trajectory divergence (the beam instability and
        # the MCC decisions amplify rounding differences), reported separately.
        for s_ in (ref, mx):
            s_.run(SORT_EVERY, collisions=coll, graph=False)
        acc_e, acc_phi = errors(ref, mx)
        mwarm = SORT_EVERY * -(-args.warmup // SORT_EVERY)
        msteps = SORT_EVERY * -(-args.steps // SORT_EVERY)
        mx.run(mwarm, collisions=coll, graph=True)  # warm-up: the step graphs are captured here
        mstream = torch.cuda.ExternalStream(mx.stream)
        m0 = torch.cuda.Event(enable_timing=True)
        m1 = torch.cuda.Event(enable_timing=True)
        nb = sum(mx.num_particles(s_) for s_ in range(nsp))
        m0.record(mstream)
        mx.run(msteps, collisions=coll, graph=True)
        m1.record(mstream)
        m1.synchronize()
        mms = max_over_ranks(m0.elapsed_time(m1))
        na = sum(mx.num_particles(s_) for s_ in range(nsp))
        # phase split: one more sort period launched directly with the phase timers on
        mx.set_profiling(True)
        mx.profile()
        mx.run(SORT_EVERY, collisions=coll, graph=False)
        mprof, miters = mx.profile()
        mx.set_profiling(False)
        mvalue = sum_over_ranks(0.5 * (nb + na) * msteps) / (mms / 1e3)
        ref.run(mwarm + msteps + SORT_EVERY, collisions=coll, graph=False)
        div_e, div_phi = errors(ref, mx)
        # HBM roofline of the mixed particle pass: the push deposits each particle
        # at its new position in the same pass (the accumulators stay in L2) and
        # selects the MCC's candidates, so its algorithmic bytes are the push's
        # 40 B per particle (cell, offsets, vx, vy read and written; the
        # electrons' vz read for the selection is not counted).  The "deposit"
        # phase is left with the accumulators' clearing and the MCC products.
        npart = 0.5 * (nb + na)
        mroof = {}
        t_ms = mprof["push"][0] / SORT_EVERY
        if t_ms > 0:
            gbs = 40 * npart / (t_ms / 1e3) / 1e9
            mroof["push_deposit_select"] = {"achieved_gbs": gbs, "frac": gbs / load_peaks()[0],
                                            "bytes_per_particle": 40}
        mixed = {"value": mvalue, "unit": UNIT, "ms_per_step": mms / msteps, "steps": msteps,
                 "roofline_particle_phases": mroof,
                 "speedup_vs_fp64": mvalue / value, "dtype": "f32 particles/inner solve + f64 refinement",
                 "sort_every": SORT_EVERY,
                 "phases_ms_per_step": {k: v[0] / SORT_EVERY for k, v in mprof.items()},
                 "phases_note": "one sort period launched directly with the phase timers on, after the timed "
                                "steps (graph replay)",
                 "solver_refinements_per_step": miters / SORT_EVERY,
                 "after_steps": SORT_EVERY,
                 "total_energy_rel_err_vs_fp64": acc_e,
                 "phi_rel_err_vs_fp64": acc_phi,
                 "divergence_after_steps": 2 * SORT_EVERY + mwarm + msteps,
                 "total_energy_rel_diff_after": div_e,
                 "phi_rel_diff_after": div_phi}
        ref.close()
        mx.close()

    serving = None
    if not args.no_serve:
        serving = run_serving(E, workloads, args.serve_scale)
    batching = None
    if not args.no_batch:
        batching = run_batching(E, workloads)
    precision_form = None
    if not args.no_precision_form:
        precision_form = run_precision_form(E, PRECISION_WORKLOAD, PRECISION_STEPS)

    rows = None
    if rank == 0 and world == 1 and not args.no_rows:
        try:  # the extensions on their own decks (10 steps each), the oracle beside them
            rows = measure_rows(10, 3, 12.0)
        except Exception as exc:  # recorded, not fatal to the headline line
            rows = {"error": repr(exc)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, done, n, kind = cpu_port_run(ini, None, 0, budget_s=args.cpu_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": kind,
               "sample": "%d full loop iterations of %s (%d particles) on one host core after load + initial "
                         "field (the reference loop is serial)" % (done, args.workload, n)}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (particles loaded from mt19937 seed 0, as the reference's Init)",
                "config": workload_config(ini, args.workload, world),
                "particles_stepped": int(0.5 * (n_before + n_after)),
                "push": "FP64, contracted (multiply-adds; within a few ulps of the reference's order)",
                "mcc_uniforms": "Philox" if coll else None,
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d // e2e_steps,
                        "d2h_bytes_per_step": d2h // e2e_steps, "steps": e2e_steps},
                "gpu_launches": int(launches), "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
                "mixed_precision": mixed, "serving": serving, "batching": batching,
                "precision_form": precision_form, "extension_rows": rows}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


PRECISION_WORKLOAD = "twostream_1024"
PRECISION_STEPS = 32      # one sort period of the mixed form (PRECISION_SORT_EVERY)


# The precision form's plasma moves about 0.15 cells per step, so its mixed run
# sorts every 32 steps (measured on GB300: 3.08 ms per step against 3.47 with
# a sort every 16 and 4.42 every 8; every 64, 3.08).  Without collisions the
# sort period changes only the order of the particles, not the physics: the
# deposit is an exact integer sum.
PRECISION_SORT_EVERY = 32
PRECISION_WARMUP = 2  # the sorting step and a plain one: both step graphs captured


def run_precision_form(E, name, steps):
    """The precision form's plasma (2.1e8 particles on 1024^2 periodic cells,
    two electron streams) in the plain FP64 form and the mixed form from the
    same particles (device loader, one seed): throughput of each over `steps`
    steps (CUDA events, graph replay), and the mixed form's density, potential
    and total-energy errors against the FP64 run after those steps."""
    import numpy as np
    import torch

    A = E.api
    ini = write_deck(name)
    out = {"workload": name, "steps": steps, "warmup": PRECISION_WARMUP, "mixed_sort_every": PRECISION_SORT_EVERY}
    sims = {}
    for form, kw in (("fp64", {}), ("mixed", {"precision": 1, "sort_every": PRECISION_SORT_EVERY})):
        sim = A.Simulation.from_ini(ini, **kw)
        sim.load_particles_device(11)
        sim.initial_field()
        n = sum(sim.num_particles(k) for k in range(len(sim.species)))
        # warm-up: the step graphs (plain and sorting) are captured here, not in the timed region
        sim.run(PRECISION_WARMUP, collisions=False, graph=True)
        st = torch.cuda.ExternalStream(sim.stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        sim.run(steps, collisions=False, graph=True)
        e1.record(st)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out[form + "_particle_steps_per_s"] = n * steps / (ms / 1e3)
        out[form + "_ms_per_step"] = ms / steps
        out["particles"] = n
        sims[form] = sim
    fp, mx = sims["fp64"], sims["mixed"]

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

    def energy(sm):
        return sum(sm.compute_ke(k, 0).sum() for k in range(len(sm.species))) + sm.compute_pe(0)

    out["rho_rel_err_vs_fp64"] = rel(mx.grid("rho"), fp.grid("rho"))
    out["phi_rel_err_vs_fp64"] = rel(mx.grid("phi"), fp.grid("phi"))
    ef, em = energy(fp), energy(mx)
    out["total_energy_rel_err_vs_fp64"] = abs(em - ef) / abs(ef)
    out["speedup_vs_fp64"] = out["mixed_particle_steps_per_s"] / out["fp64_particle_steps_per_s"]
    # Phase split of each form: one more sort period, launched step by step
    # with the phase timers on (after the comparison above).
    for form, sim in (("fp64", fp), ("mixed", mx)):
        sim.set_profiling(True)
        sim.profile()
        sim.run(PRECISION_SORT_EVERY, collisions=False, graph=False)
        prof, iters = sim.profile()
        sim.set_profiling(False)
        out[form + "_phases_ms_per_step"] = {k: v[0] / PRECISION_SORT_EVERY for k, v in prof.items()}
        out[form + ("_pcg_iterations_per_step" if form == "fp64" else "_solve_stages_per_step")] = \
            iters / PRECISION_SORT_EVERY
    fp.close()
    mx.close()
    return out


# The batch sorts every 32 steps (measured on GB300: 51.9 ms per step against
# 57.3 sorting every 16; the particles of these runs move well under a cell per
# step).  The sort period changes only the particles' order: collisionless
# runs are unchanged bit for bit, colliding ones draw other (equally
# distributed) Philox numbers.  The runs timed alone use the same period.
BATCH_SORT_EVERY = 32
BATCH_STEPS = 64          # timed steps of the batch (two sort periods)
BATCH_SAMPLE = 4          # runs timed one at a time for comparison


def run_batching(E, workloads):
    """The batching workload (512 runs, cells {32..256} per axis, 20-200
    particles per cell, Te 0.5-5 eV, MCC on half) as one batch in the mixed
    form: every phase one launch for all runs, graph-replayed steps, tuned GEMM
    tiles.  Compared with a sample of the same runs advanced one at a time."""
    import torch

    A = E.api
    reqs = workloads.batching_requests(seed=0)
    e, ela, exc, ion = workloads.synthetic_table()
    d = tempfile.mkdtemp(prefix="epic_batch_")
    rq, paths = [], []
    for k, q in enumerate(reqs):
        path = os.path.join(d, "run%03d.ini" % k)
        with open(path, "w") as f:
            f.write(q["ini"])
        paths.append(path)
        rq.append(A.make_request(path, 0, q["collisions"], q["seed"], 0.0, precision=1,
                                 sort_every=BATCH_SORT_EVERY))
    t0 = time.perf_counter()
    b = A.Batch(rq, sort_every=BATCH_SORT_EVERY)
    b.set_log_cross_sections(ela, exc, ion, e[0], e[-1])
    b.initial_field()
    setup_s = time.perf_counter() - t0
    b.run(BATCH_SORT_EVERY, graph=True)  # warm-up: one sort period
    n = b.num_particles()
    st = torch.cuda.ExternalStream(b.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    b.run(BATCH_STEPS, graph=True)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    tiles = b.tuning()
    shapes = b.particle_tuning()
    # phase split: one more sort period launched step by step with the phase timers on
    b.set_profiling(True)
    b.profile()
    b.run(BATCH_SORT_EVERY, graph=False)
    phases = {k: v[0] / BATCH_SORT_EVERY for k, v in b.profile().items()}
    b.set_profiling(False)
    b.close()
    rate = n * BATCH_STEPS / (ms / 1e3)
    # the same runs one at a time (mixed form, graph replay)
    sample = list(range(0, len(reqs), max(1, len(reqs) // BATCH_SAMPLE)))[:BATCH_SAMPLE]
    pst, t_ms = 0.0, 0.0
    for k in sample:
        coll = reqs[k]["collisions"]
        sim = A.Simulation.from_ini(paths[k], precision=1, sort_every=BATCH_SORT_EVERY)
        if coll:
            sim.set_log_cross_sections(ela, exc, ion, e[0], e[-1])
        sim.load_particles_device(reqs[k]["seed"])
        sim.initial_field()
        sim.run(BATCH_SORT_EVERY, collisions=coll, graph=True)
        s2 = torch.cuda.ExternalStream(sim.stream)
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(s2)
        sim.run(BATCH_STEPS, collisions=coll, graph=True)
        a1.record(s2)
        a1.synchronize()
        t_ms += a0.elapsed_time(a1)
        pst += reqs[k]["particles"] * BATCH_STEPS
        sim.close()
    single = pst / (t_ms / 1e3)
    procs = min(cpu_cores(), len(reqs), 16)
    cpu_sample = list(range(0, len(reqs), max(1, len(reqs) // procs)))[:procs]
    cpu_rate = cpu_multi_run([(paths[k], reqs[k]["collisions"]) for k in cpu_sample], CPU_MULTI_SECONDS)
    return {"workload": "batching: 512 runs (cells {32,...,256} per axis, 20-200 ppc per species, Te 0.5-5 eV, "
                        "MCC on %d, periodic) as one batch, mixed form" % sum(q["collisions"] for q in reqs),
            "runs": len(reqs), "particles": n, "steps": BATCH_STEPS, "sort_every": BATCH_SORT_EVERY,
            "ms_per_step": ms / BATCH_STEPS,
            "particle_steps_per_s": rate, "setup_s": setup_s, "gemm_tiles_by_size_class": tiles,
            "particle_launch_shapes": shapes, "phases_ms_per_step": phases,
            "one_at_a_time_particle_steps_per_s": single,
            "one_at_a_time_sample": "%d of the runs, each alone (mixed form, graph replay)" % len(sample),
            "speedup_vs_one_at_a_time": rate / single,
            "cpu_baseline": {"value": cpu_rate, "unit": "particle-steps/s", "cores": procs, "kind": "port",
                             "sample": "%d of the runs at once, one reference loop (oracle restatement) per host "
                                       "core, %g s each after load and initial field" % (procs, CPU_MULTI_SECONDS)},
            "speedup_vs_cpu_cores": rate / cpu_rate if cpu_rate else None}


SERVE_BUDGET = 150e9      # device bytes the serving loop may admit
SERVE_STEP_SCALE = 0.01   # step counts 500-5000 scaled to 5-50: the arrivals then offer ~60 % of the GPU's rate
SERVE_FP64_SAMPLE = 6     # requests timed one at a time in the plain FP64 form


def run_serving(E, workloads, step_scale=SERVE_STEP_SCALE):
    """The serving workload (Poisson arrivals at 50 runs/s for 60 s; grids
    {64..512}^2; 25-100 particles per cell per species; MCC on half the runs;
    periodic or Dirichlet systems; step counts 500-5000 times step_scale)
    through the continuous-batching server in the mixed form, against a sample
    of the same requests run one at a time in the plain FP64 form.  Also
    reported: the particle-steps per second the arrivals offer, scaled and
    unscaled."""
    import torch

    A = E.api
    reqs = workloads.serving_requests(seed=0, step_scale=step_scale)
    unscaled = workloads.serving_requests(seed=0, step_scale=1.0)
    window = 60.0
    e, ela, exc, ion = workloads.synthetic_table()
    d = tempfile.mkdtemp(prefix="epic_serve_")
    paths = []
    for k, q in enumerate(reqs):
        path = os.path.join(d, "req%03d.ini" % k)
        with open(path, "w") as f:
            f.write(q["ini"])
        paths.append(path)
    srv = A.Server(SERVE_BUDGET, max_inflight=16, chunk_steps=16)
    srv.set_log_cross_sections(ela, exc, ion, e[0], e[-1])
    ids = [srv.submit(A.make_request(paths[k], q["steps"], q["collisions"], q["seed"], q["arrival_s"],
                                     precision=1, sort_every=SORT_EVERY)) for k, q in enumerate(reqs)]
    torch.cuda.synchronize()
    srv.start()
    srv.wait(1800)
    st = srv.stats()
    failed = []
    for k, i in enumerate(ids):
        r = srv.result(i)
        if r.status != 0:
            q = reqs[k]
            failed.append({"request": k, "status": int(r.status), "side": q["side"], "steps": q["steps"],
                           "collisions": q["collisions"], "particles": q["particles"],
                           "periodic": "poisson_bc = periodic" in q["ini"]})
    fails = len(failed)
    srv.close()
    # the plain FP64 form, one request at a time (wall time from creation to the end of the last step)
    sample = list(range(0, len(reqs), max(1, len(reqs) // SERVE_FP64_SAMPLE)))[:SERVE_FP64_SAMPLE]
    pst, wall = 0.0, 0.0
    for k in sample:
        q = reqs[k]
        t0 = time.perf_counter()
        sim = A.Simulation.from_ini(paths[k])
        if q["collisions"]:
            sim.set_log_cross_sections(ela, exc, ion, e[0], e[-1])
        sim.load_particles_device(q["seed"])
        sim.initial_field()
        sim.run(q["steps"], collisions=q["collisions"], graph=True)
        wall += time.perf_counter() - t0
        pst += q["particles"] * q["steps"]
        sim.close()
    fp64_rate = pst / wall if wall > 0 else None
    procs = min(cpu_cores(), len(reqs), 16)
    cpu_sample = list(range(0, len(reqs), max(1, len(reqs) // procs)))[:procs]
    cpu_rate = cpu_multi_run([(paths[k], reqs[k]["collisions"]) for k in cpu_sample], CPU_MULTI_SECONDS)
    offered = sum(q["particles"] * q["steps"] for q in reqs) / window
    offered_unscaled = sum(q["particles"] * q["steps"] for q in unscaled) / window
    return {"workload": "serving: Poisson arrivals 50/s for 60 s, grids {64,128,256,512}^2, 25-100 ppc per species, "
                        "steps 500-5000 x %g, MCC p=0.5, periodic or Dirichlet systems, %.0f GB budget, mixed form"
                        % (step_scale, SERVE_BUDGET / 1e9),
            "step_scale": step_scale,
            "offered_particle_steps_per_s": offered,
            "offered_particle_steps_per_s_unscaled": offered_unscaled,
            "unscaled_load_over_served_rate": offered_unscaled / st.particle_steps_per_s if st.particle_steps_per_s else None,
            "requests": len(reqs), "completed": int(st.completed), "failed": fails, "failures": failed[:16],
            "p50_latency_s": st.p50_latency_s, "p99_latency_s": st.p99_latency_s,
            "mean_latency_s": st.mean_latency_s, "max_latency_s": st.max_latency_s,
            "makespan_s": st.makespan_s, "particle_steps_per_s": st.particle_steps_per_s,
            "peak_inflight": int(st.peak_inflight), "peak_bytes": int(st.peak_bytes),
            "fp64_one_at_a_time_particle_steps_per_s": fp64_rate,
            "fp64_sample": "%d of the %d requests, each created, loaded, initialised and run alone" % (len(sample), len(reqs)),
            "speedup_vs_fp64_one_at_a_time": (st.particle_steps_per_s / fp64_rate) if fp64_rate else None,
            "cpu_baseline": {"value": cpu_rate, "unit": "particle-steps/s", "cores": procs, "kind": "port",
                             "sample": "%d of the requests at once, one reference loop (oracle restatement) per "
                                       "host core, %g s each after load and initial field" % (procs, CPU_MULTI_SECONDS)},
            "speedup_vs_cpu_cores": (st.particle_steps_per_s / cpu_rate) if cpu_rate else None}


# Per-launch DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of each
# phase's kernel from the ncu captures summarised under profiles/ (beam_mcc_256);
# absent where no capture of that phase's average launch exists.  The solve's
# vectors stay in registers and L2, so its traffic is ~0.7 MB against 5.5 GB of
# algorithmic (memory-streamed) bytes.
TRAFFIC = {"solve": 0.631296e6 + 0.080384e6}


# ------------------------------------------------ extension-row measurements ---
ROWS = (("conductors (SOR, absorbing walls, erase on hit)", "conductors_64"),
        ("emitters (injection every step, absorbing walls, PCG)", "emitters_128"),
        ("gsfluidsolver (solvertype = gshybrid)", "gshybrid_64"),
        ("nrpcgsolver (solvertype = hybrid)", "hybrid_24"))


def measure_rows(steps, warmup, cpu_seconds):
    """Per-step throughput of each extension of the loop on its own deck: the
    GPU loop (CUDA events on the handle's stream, FP64 form) and the oracle
    restatement on one host core beside it (cpu_seconds over all rows)."""
    import torch

    import epic2d_mcc_gb300 as E
    from epic2d_mcc_gb300 import build as B

    B.build()
    out = []
    for label, name in ROWS:
        ini = write_deck(name)
        sim = E.Simulation.from_ini(ini)
        sim.load_particles(0)
        sim.initial_field()
        nsp = len(sim.species)
        for _ in range(warmup):
            sim.run(1, collisions=False, graph=False)
        stream = torch.cuda.ExternalStream(sim.stream)
        n0 = sum(sim.num_particles(s) for s in range(nsp))
        sim.sync()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        sim.run(steps, collisions=False, graph=False)
        ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1)
        n1 = sum(sim.num_particles(s) for s in range(nsp))
        gpu = 0.5 * (n0 + n1) * steps / (ms * 1e-3)
        cpu, done, n, _ = cpu_port_run(ini, None, 1, budget_s=cpu_seconds / len(ROWS))
        out.append({"row": label, "workload": name, "particles": int(0.5 * (n0 + n1)), "gpu_ms_per_step": ms / steps,
                    "gpu_particle_steps_per_s": gpu, "cpu_particle_steps_per_s": cpu, "cpu_steps_timed": done,
                    "cpu_cores": 1, "speedup": gpu / cpu})
        del sim
    return out


def run_serving_unscaled(cutoff_s):
    """The serving configuration as stated: Poisson arrivals at 50 runs/s for
    60 s with the unscaled step counts (500-5000).  The arrivals offer about
    100 times the particle-steps per second the GPU serves, so the queue grows
    without bound; the server runs until cutoff_s after its start and is then
    stopped.  Reported: what arrived, completed and was still queued or in
    service at the cutoff; the latencies of the completed requests; and the
    latencies of every request that had arrived, an unfinished one counted as
    (cutoff - arrival), i.e. lower bounds."""
    import ctypes

    import numpy as np
    import torch

    import epic2d_mcc_gb300 as E
    from epic2d_mcc_gb300 import build as B
    from epic2d_mcc_gb300 import workloads

    B.build()
    A = E.api
    reqs = workloads.serving_requests(seed=0, step_scale=1.0)
    e, ela, exc, ion = workloads.synthetic_table()
    d = tempfile.mkdtemp(prefix="epic_serve_full_")
    srv = A.Server(SERVE_BUDGET, max_inflight=16, chunk_steps=16)
    srv.set_log_cross_sections(ela, exc, ion, e[0], e[-1])
    ids = []
    for k, q in enumerate(reqs):
        path = os.path.join(d, "req%03d.ini" % k)
        with open(path, "w") as f:
            f.write(q["ini"])
        ids.append(srv.submit(A.make_request(path, q["steps"], q["collisions"], q["seed"], q["arrival_s"],
                                             precision=1, sort_every=SORT_EVERY)))
    torch.cuda.synchronize()
    srv.start()
    t0 = time.perf_counter()
    try:
        srv.wait(cutoff_s)
    except E.EpicError:
        pass  # the cutoff came first (the expected outcome at this load)
    cutoff = time.perf_counter() - t0
    done_lat, all_lat, work, failed = [], [], 0.0, 0
    arrived = 0
    for k, i in enumerate(ids):
        q = reqs[k]
        if q["arrival_s"] > cutoff:
            continue
        arrived += 1
        r = A.Result()
        ok = A.lib().epic_server_result(srv._h, i, ctypes.byref(r)) == 0
        if ok and r.status == 0:
            lat = r.finish_s - r.arrival_s
            done_lat.append(lat)
            all_lat.append(lat)
            work += q["particles"] * q["steps"]
        else:
            failed += int(ok)
            all_lat.append(cutoff - q["arrival_s"])
    srv.close()
    offered = sum(q["particles"] * q["steps"] for q in reqs) / 60.0
    pct = lambda v, p: float(np.percentile(v, p)) if v else None
    print(json.dumps({
        "workload": "serving as configured: Poisson arrivals 50/s for 60 s, grids {64,128,256,512}^2, 25-100 ppc "
                    "per species, steps 500-5000 (unscaled), MCC p=0.5, periodic or Dirichlet systems, mixed form",
        "requests": len(reqs), "cutoff_s": cutoff, "arrived_by_cutoff": arrived, "completed": len(done_lat),
        "failed": failed, "queued_or_in_service_at_cutoff": arrived - len(done_lat) - failed,
        "completed_p50_latency_s": pct(done_lat, 50), "completed_p99_latency_s": pct(done_lat, 99),
        "arrived_p50_latency_s_lower_bound": pct(all_lat, 50), "arrived_p99_latency_s_lower_bound": pct(all_lat, 99),
        "offered_particle_steps_per_s": offered,
        "completed_particle_steps_per_s_lower_bound": work / cutoff,
        "note": "unfinished requests count as (cutoff - arrival); work of runs still in service is not counted"}),
        flush=True)


def run_rows(args):
    out = measure_rows(args.steps, args.warmup, args.cpu_seconds)
    print(json.dumps({"rows": out, "steps": args.steps, "warmup": args.warmup, "dtype": "f64",
                      "data": "synthetic (particles loaded from mt19937 seed 0, as the reference's Init)"}),
          flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--serve-scale", type=float, default=SERVE_STEP_SCALE,
                    help="factor on the serving requests' step counts (1 = the configuration's 500-5000)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batching measurement")
    ap.add_argument("--no-precision-form", action="store_true", help="skip the 1024^2 precision-form measurement")
    ap.add_argument("--no-rows", action="store_true", help="skip the extension-row measurements")
    ap.add_argument("--rows", action="store_true",
                    help="measure the loop's extensions (conductors, emitters, Boltzmann solvers) instead")
    ap.add_argument("--serve-unscaled", type=float, default=0.0, metavar="SECONDS",
                    help="run the serving configuration with unscaled step counts for SECONDS, then stop it "
                         "and report the queue (instead of the default measurements)")
    args = ap.parse_args()
    if args.rows:
        run_rows(args)
        return
    if args.serve_unscaled > 0:
        run_serving_unscaled(args.serve_unscaled)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)


if __name__ == "__main__":
    main()
