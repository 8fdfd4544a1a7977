#!/usr/bin/env python3
"""Throughput of the MITHRA FdTd time-marching loop on GB300.

Metric: cell+particle updates per second, i.e. (mesh nodes + particle pushes) per field step
divided by the step time, where particle pushes = particles x bunch substeps.  The default
workload is the 128 x 128 x 2048-cell job (130 x 130 x 2050 nodes, ~8.1e6 macro-particles,
two bunch substeps per field step) in the plain FP64 form; --precision fp32 selects the mixed
form.  Inputs are seeded synthetic bunches (Halton sequence) built by the reference's own
initialisation restated on the host; the field state (3.4 GB) exceeds the 129 MB L2, so no L2
flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU (the path is a
single domain per GPU); the value is the sum over ranks and the time the maximum over ranks.
`--impl reference` times the reference algorithm on the host cores instead: the C restatement
in oracle/ (the reference tree itself is not present on the GPU host), with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOADS = {
    "fel-130x130x2050": "fel-130x130x2050.job",
    "fel-ir-48x48x384": "fel-ir-48x48x384.job",
    "fel-98x98x1026": "fel-98x98x1026.job",  # profiling case (about 1 GB on the device)
}
METRIC = "cell+particle updates/s"
FP64_NOMINAL_TFLOPS = 1.25  # GB300 dense FP64, nominal

# Algorithmic bytes per unit (each array element counted once, halo re-reads free).
# Units: interior node for the field kernels, particle for the particle kernels.
ALGO_BYTES = {
    "fp64": {"potential_interior_fd": 96, "potential_interior_nsfd": 96, "eval_eb": 72, "push": 96 + 1,
             "deposit": 48 + 8, "erase": 8 + 1},
    "fp32": {"potential_interior_fd": 48, "potential_interior_nsfd": 48, "eval_eb": 48, "push": 56 + 1,
             "deposit": 24 + 4 + 20, "erase": 12 + 1},
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--workload", default="fel-130x130x2050", choices=sorted(WORKLOADS) + ["sweep-192"])
    ap.add_argument("--autotune-steps", type=int, default=0,
                    help="sweep-192: autotune every instance on this many steps per candidate shape")
    ap.add_argument("--cpu-sample-seconds", type=float, default=15.0)
    ap.add_argument("--sweep-designs", type=int, default=384,
                    help="sweep-192: designs marched to their exits through a refilled queue (0: skip)")
    ap.add_argument("--sweep-leg-designs", type=int, default=192,
                    help="default workload: sweep-family designs marched through the refilled queue for the "
                         "FEL runs/h figure (0: skip the sweep leg)")
    ap.add_argument("--sweep-leg-slots", type=int, default=96)
    ap.add_argument("--sweep-check-designs", type=int, default=8,
                    help="designs marched in both forms for the P_sat error of the sweep leg")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp32-compare", action="store_true",
                    help="with --precision fp64, skip the mixed-form run reported under fp32_form")
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3)
    return a


class Dist:
    def __init__(self, want_gpus: int):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = dist
            self.torch = torch
            self.backend = backend

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = self.torch.tensor([v], dtype=self.torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = self.torch.tensor([v], dtype=self.torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi samples of the SM clock and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_table():
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


STATE_DIR = os.path.join(REPO, "oracle", "_build", "state")


def initial_state_dir(jobpath):
    return os.path.join(STATE_DIR, os.path.splitext(os.path.basename(jobpath))[0])


def oracle_run_for(jobpath):
    """The CPU restatement (oracle/) started from the job's seeded initial state, read from the
    file that build() (or a child process) wrote: this process does not load the CUDA library."""
    from oracle import initial_state
    from oracle import pyoracle as po
    d = initial_state.ensure(jobpath, initial_state_dir(jobpath))
    m, anp1, an, anm1, parts, solver, order, _ = initial_state.load(d)
    return po, po.OracleRun(m, an, anm1, anp1, parts, solver=solver, order=order), m


def units_per_step(meta, n_particles):
    nsub = 0
    t = 0.0
    while t < meta["nUpdateBunch"]:
        nsub += 1
        t += 1.0
    nodes = int(meta["N0"]) * int(meta["N1"]) * int(meta["N2"])
    return nodes, n_particles * nsub, nsub


def run_config(workload, nodes, particles, nsub, precision, world):
    """The `config` object both arms print for one workload."""
    return {"workload": workload, "nodes": nodes, "particles": particles, "substeps": nsub, "precision": precision,
            "parallelism": "replicas" if world > 1 else "single-gpu",
            "l2": "inputs larger than L2 (%.1f GB of field state)" % (nodes * 3 * 3 * 8 / 1e9)}


def host_cpu():
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k = line.split(":")[0].strip().lower()
                if k in ("model name", "cpu model"):
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if model is None:
        import platform
        model = platform.machine()
    return {"model": model, "logical_cpus": os.cpu_count(), "threads_available": cpu_threads()}


def time_oracle(run, po, threads, min_seconds, max_steps):
    """Steps of the oracle at `threads` OpenMP threads until `min_seconds` or `max_steps`."""
    po.set_threads(threads)
    steps, t0 = 0, time.perf_counter()
    while True:
        run.step()
        steps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or steps >= max_steps:
            break
    po.set_threads(1)
    return steps, el


def cpu_baseline(jobpath, sample_seconds):
    po, run, m = oracle_run_for(jobpath)
    threads = cpu_threads()
    nodes, pushes, _ = units_per_step(m, run.n)
    po.set_threads(threads)
    run.step()  # first-touch of the arrays
    steps, el = time_oracle(run, po, threads, sample_seconds, 200)
    return {"value": (nodes + pushes) * steps / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": "%d field steps of the same job (after one untimed step), C restatement of the "
                      "reference with OpenMP over %d host threads, %.1f s" % (steps, threads, el)}


def run_reference(args, dist):
    """The reference algorithm on the host cores: the oracle's C restatement (pinned bit for bit
    to the reference in the container that has the reference tree; that tree is not on the GPU
    host, so its binary cannot be built here), all host threads, then one thread."""
    jobpath = os.path.join(REPO, "mithra_gb300", "jobs", WORKLOADS[args.workload])
    if dist.rank != 0:
        return
    po, run, m = oracle_run_for(jobpath)
    threads = cpu_threads()
    nodes, pushes, nsub = units_per_step(m, run.n)
    po.set_threads(threads)
    for _ in range(args.warmup):
        run.step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run.step()
    el = time.perf_counter() - t0
    value = (nodes + pushes) * args.steps / el
    # one thread on a bounded sample of the same march (continues from the state reached)
    s1, el1 = time_oracle(run, po, 1, args.cpu_sample_seconds, 3)
    po.set_threads(1)
    v1 = (nodes + pushes) * s1 / el1
    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Halton bunch of the job file)",
        "config": run_config(args.workload, nodes, run.n, nsub, "fp64", dist.world),
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": "%d timed field steps after %d warm-up steps, C restatement of the reference "
                                   "(oracle/) with OpenMP over %d host threads, one process (the reference's "
                                   "MPI decomposition is not used: a single domain)" % (args.steps, args.warmup, threads)},
        "one_thread": {"value": v1, "unit": METRIC, "cores": 1, "threads": 1, "ms_per_step": 1e3 * el1 / s1,
                       "sample": "%d further field steps of the same march on one thread" % s1,
                       "threads_speedup": value / v1},
        "host": host_cpu(),
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def measure_form(mg, setup, prec_name, args, dist, units, interior, clocks=True):
    """One precision form on the workload: K timed graph-replayed steps (CUDA events on the context
    stream), the per-kernel breakdown and roofline of an instrumented pass over K more steps, and
    the end-to-end rate through the public API with host buffers."""
    prec = mg.FP64 if prec_name == "fp64" else mg.FP32
    ctx = mg.Context.from_setup(setup, prec, device=dist.local)
    n_part = ctx.particle_count()
    ctx.run_prelude()
    ctx.run(args.warmup)
    ctx.synchronize()
    dist.barrier()
    with ClockSampler(dist.local) as clk:
        ms = ctx.run_timed(args.steps)
    dist.barrier()
    ms_max = dist.max(ms)
    out = {"ms_total": ms_max, "ms_per_step": ms_max / args.steps,
           "value": dist.world * units * args.steps / (ms_max / 1e3), "clocks": clk.summary()}

    # Per-kernel device times: the same K steps again, each kernel bracketed by CUDA events on
    # the context stream (direct launches instead of the step graph).
    ctx.enable_timing(True)
    ctx.run(args.steps)
    kt = ctx.kernel_times()
    ctx.enable_timing(False)
    total_k = sum(v[0] for v in kt.values())
    dominant = max(kt.items(), key=lambda kv: kv[1][0])[0]
    dom_ms, dom_launches = kt[dominant]
    unit_count = n_part if dominant in ("push", "deposit", "erase", "tile_scatter") else interior
    per_unit = ALGO_BYTES[prec_name].get(dominant)
    peak, peak_kind = measured_peaks()
    roof = None
    if per_unit:
        avg_s = dom_ms / dom_launches / 1e3
        achieved = per_unit * unit_count / avg_s / 1e9
        tr = traffic_table().get(prec_name, {}).get(dominant)
        roof = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": per_unit * unit_count,
                "traffic": (tr * unit_count if tr else None),
                "avg_launch_ms": dom_ms / dom_launches, "share": dom_ms / total_k}
    out["roofline"] = roof
    out["dominant"] = (dominant, dom_ms / dom_launches, unit_count)
    out["kernels"] = {k: {"ms_per_launch": v[0] / v[1], "launches": v[1], "share": v[0] / total_k}
                      for k, v in kt.items()}
    # per-kernel HBM fractions for the kernels with an algorithmic byte count
    for k, v in out["kernels"].items():
        pu = ALGO_BYTES[prec_name].get(k)
        if pu:
            cnt = n_part if k in ("push", "deposit", "erase") else interior
            v["hbm_frac"] = pu * cnt / (v["ms_per_launch"] / 1e3) / 1e9 / peak

    # End to end through the public API with host buffers: upload the initial state from pinned
    # host memory, march K steps, read the power rows back.
    e2e = None
    if not args.no_e2e:
        anp1, an, anm1 = setup.fields()
        parts = setup.particles()
        bufs = [mg.PinnedArray(anp1.shape), mg.PinnedArray(an.shape), mg.PinnedArray(anm1.shape),
                mg.PinnedArray(parts.shape)]
        for b, src in zip(bufs, (anp1, an, anm1, parts)):
            b.array[...] = src
        t0_state = setup.time()
        h2d = sum(b.array.nbytes for b in bufs)
        dist.barrier()
        t0 = time.perf_counter()
        ctx.upload_fields(bufs[0].array, bufs[1].array, bufs[2].array)
        ctx.upload_particles(bufs[3].array)
        ctx.set_time(t0_state)
        ctx.run(args.steps)
        rows = ctx.power_rows()
        el = time.perf_counter() - t0
        el = dist.max(el)
        e2e = {"value": dist.world * units * args.steps / el, "unit": METRIC,
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": rows.nbytes / args.steps,
               "ms_per_step": 1e3 * el / args.steps}
        for b in bufs:
            b.free()
    out["e2e"] = e2e
    out["launches"] = ctx.launches_per_step() * args.steps
    out["n_part"] = n_part
    ctx.close()
    return out


def sweep_leg(args, dist):
    """FEL runs per hour of the sweep family (C4 designs, mixed form) measured through the
    refilled queue, and the mixed form's P_sat error against the FP64 form on a fixed subset."""
    import tempfile

    import mithra_gb300 as mg
    from mithra_gb300 import sweep
    params = sweep.sweep_parameters(args.sweep_leg_designs, seed=20261205)
    done, wall, rebuilds = sweep.run_queue(params, tempfile.mkdtemp(prefix="mithra-leg-"), slots=args.sweep_leg_slots,
                                           device=dist.local)
    runs_h = dist.sum(len(done) * 3600.0 / wall)
    # P_sat of a fixed subset of the family in both forms, each design marched to its exit
    sub = sweep.sweep_parameters(args.sweep_check_designs, seed=20261206)
    psat = {}
    for prec in (mg.FP64, mg.FP32):
        d, _, _ = sweep.run_queue(sub, tempfile.mkdtemp(prefix="mithra-chk-"), slots=len(sub), precision=prec,
                                  device=dist.local)
        psat[prec] = {i: float(r.reshape(-1, 2)[:, 1].max()) for i, r in d.items()}
    ok = [i for i in psat[mg.FP64] if np.isfinite(psat[mg.FP64][i]) and psat[mg.FP64][i] > 0.0]
    errs = sorted(abs(psat[mg.FP32][i] - psat[mg.FP64][i]) / psat[mg.FP64][i] for i in ok) or [float("nan")]
    return {"value": runs_h, "unit": "FEL runs/h", "designs": len(done), "slots": args.sweep_leg_slots,
            "wall_s": wall, "batch_rebuilds": rebuilds, "precision": "fp32",
            "how": "designs of the sweep family (gamma 80-400, K 0.8-2, lambda_u 1.5-3 cm, 50-500 pC, "
                   "32-96 x 32-96 x 128-768 cells, 5e4-1e6 particles) marched to their undulator exits "
                   "through a queue of slots refilled as designs exit; device set-up, prelude and batch "
                   "rebuilds inside the clock",
            "psat_error_vs_fp64": {"designs": len(ok), "max": errs[-1], "median": errs[len(errs) // 2],
                                   "bound": 0.02, "within_bound": bool(errs[-1] <= 0.02),
                                   "excluded": {"no_power": sum(1 for i in psat[mg.FP64] if psat[mg.FP64][i] == 0.0),
                                                "non_finite": sum(1 for i in psat[mg.FP64]
                                                                  if not np.isfinite(psat[mg.FP64][i]))},
                                   "psat_fp64": [psat[mg.FP64][i] for i in sorted(psat[mg.FP64])],
                                   "psat_fp32": [psat[mg.FP32][i] for i in sorted(psat[mg.FP32])]}}


def run_gpu(args, dist):
    import mithra_gb300 as mg
    jobpath = os.path.join(REPO, "mithra_gb300", "jobs", WORKLOADS[args.workload])
    setup = mg.Setup.from_job(jobpath)
    meta = setup.meta()
    g = setup.grid()
    interior = (g.N0 - 2) * (g.N1 - 2) * (g.N2 - 2)
    n_part = setup.particles().shape[0]
    nodes, pushes, nsub = units_per_step(meta, n_part)
    units = nodes + pushes
    main = measure_form(mg, setup, args.precision, args, dist, units, interior)
    ms_max = main["ms_total"]
    value = main["value"]

    # The FP64 form is bound by GB300's FP64 pipe, not by HBM: its dominant kernel is also placed
    # against the FP64 rate measured on this device (FLOPs per unit counted by ncu on the
    # profiling case, FMA = 2).
    fp64_pipe = None
    dominant, dom_ms, unit_count = main["dominant"]
    flop = traffic_table().get("fp64_flop_per_unit", {}).get(dominant) if args.precision == "fp64" else None
    if flop:
        peak = mg.probe_fp64_tflops(dist.local)
        tflops = flop * unit_count / (dom_ms / 1e3) / 1e12
        fp64_pipe = {"kernel": dominant, "flop_per_unit": flop, "achieved": tflops, "peak": peak,
                     "unit": "TFLOP/s", "frac": tflops / peak,
                     "peak_source": "measured in this run (mithra_probe_fp64_tflops: independent DFMA chains on "
                                    "every SM); nominal %.2f" % FP64_NOMINAL_TFLOPS}

    # "FP32 vs FP64": the mixed form on the same workload and step count, measured the same way.
    fp32_form = None
    if args.precision == "fp64" and not args.no_fp32_compare:
        f = measure_form(mg, setup, "fp32", args, dist, units, interior)
        fp32_form = {"value": f["value"], "unit": METRIC, "ms_per_step": f["ms_per_step"],
                     "speedup_vs_fp64": f["value"] / value, "roofline": f["roofline"], "kernels": f["kernels"],
                     "e2e": f["e2e"], "clocks": f["clocks"], "gpu_launches": f["launches"]}

    runs = None
    if args.workload == "fel-130x130x2050" and args.sweep_leg_designs > 0:
        runs = sweep_leg(args, dist)

    if dist.rank != 0:
        return
    cpu = None
    if dist.world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(jobpath, args.cpu_sample_seconds)
    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
        "data": "synthetic (seeded Halton bunch of the job file)",
        "config": run_config(args.workload, nodes, n_part, nsub, args.precision, dist.world),
        "cell_updates_per_s": dist.world * nodes * args.steps / (ms_max / 1e3),
        "particle_pushes_per_s": dist.world * pushes * args.steps / (ms_max / 1e3),
        "roofline": main["roofline"],
        "fp64_pipe": fp64_pipe,
        "fp32_form": fp32_form,
        "fel_runs_per_hour": runs,
        "kernels": main["kernels"],
        "gpu_launches": main["launches"],
        "clocks": main["clocks"],
        "e2e": main["e2e"],
        "cpu_baseline": cpu,
    }
    print(json.dumps(out), flush=True)


def run_sweep(args, dist):
    """192 seeded FEL designs (mixed form) stepped as one batch: one graph launch per field step."""
    import tempfile

    import mithra_gb300 as mg
    from mithra_gb300 import sweep
    params = sweep.sweep_parameters(192)
    setups = sweep.make_setups(params, tempfile.mkdtemp(prefix="mithra-sweep-"))
    batch, ctxs, tuned = sweep.make_batch(setups, mg.FP32, dist.local, args.autotune_steps)
    units, steps_to_end, total_nodes, total_particles = 0, [], 0, 0
    for s, c in zip(setups, ctxs):
        npart = c.particle_count()
        nodes, pushes, _ = units_per_step(s.meta(), npart)
        units += nodes + pushes
        total_nodes += nodes
        total_particles += npart
        steps_to_end.append(sweep.steps_to_exit(s, c))
    batch.run(args.warmup)
    dist.barrier()
    with ClockSampler(dist.local) as clk:
        ms = batch.run_timed(args.steps)
    dist.barrier()
    ms_max = dist.max(ms)
    step_s = ms_max / 1e3 / args.steps
    value = dist.world * units / step_s
    # FEL runs per hour: every design marched to its undulator exit.  Lock-step: the batch runs
    # until its longest design ends; refilled: finished slots take new designs at once.
    runs_lockstep = dist.world * len(ctxs) * 3600.0 / (max(steps_to_end) * step_s)
    runs_refill = dist.world * len(ctxs) * 3600.0 / (float(np.mean(steps_to_end)) * step_s)
    # The same instances and step count one at a time, each from its own captured step graphs (a
    # queue of single-instance launches with nothing overlapping), against the batch's one launch.
    for c in ctxs:
        c.run(6)  # one cycle of step phases: every step graph of the instance captured
    ms_seq = sum(c.run_timed(args.steps) for c in ctxs)
    sequential = {"ms_per_step": ms_seq / args.steps, "batch_speedup": ms_seq / ms_max,
                  "how": "each instance's own step graphs launched alone, instance after instance"}
    batch.close()
    for c in ctxs:
        c.close()
    measured = None
    if args.sweep_designs > 0:
        # measured: that many further designs of the family marched to their exits through a
        # refilled queue of 192 slots (device set-up, prelude and batch rebuilds included)
        extra = sweep.sweep_parameters(192 + args.sweep_designs)[192:]
        done, wall, rebuilds = sweep.run_queue(extra, tempfile.mkdtemp(prefix="mithra-queue-"), slots=192,
                                               device=dist.local)
        measured = {"designs": len(done), "wall_s": wall, "runs_per_hour": dist.world * len(done) * 3600.0 / wall,
                    "batch_rebuilds": rebuilds}
    if dist.rank != 0:
        return
    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (192 seeded designs, Halton bunches)",
        "config": {"workload": "sweep-192", "instances": len(ctxs), "precision": "fp32",
                   "nodes": total_nodes, "particles": total_particles,
                   "autotune_steps": args.autotune_steps, "parallelism": "one graph launch per step for all instances",
                   "l2": "inputs larger than L2"},
        "fel_runs_per_hour": {"lockstep": runs_lockstep, "refilled": runs_refill, "measured_queue": measured,
                              "steps_to_exit": {"min": min(steps_to_end), "mean": float(np.mean(steps_to_end)),
                                                "max": max(steps_to_end)}},
        "sequential": sequential,
        "tuning": [[t.blocks_per_sm, t.slab_planes, ms] for t, ms in tuned][:8],
        "clocks": clk.summary(),
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    dist = Dist(args.gpus)
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        elif args.workload == "sweep-192":
            run_sweep(args, dist)
        else:
            run_gpu(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
