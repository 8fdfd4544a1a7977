#!/usr/bin/env python3
"""Throughput of the MITHRA FdTd time-marching loop on GB300.

Metric: cell+particle updates per second, i.e. (mesh nodes + particle pushes) per field step
divided by the step time, where particle pushes = particles x bunch substeps.  The default
workload is the 128 x 128 x 2048-cell job (130 x 130 x 2050 nodes, ~8.1e6 macro-particles,
two bunch substeps per field step) in the plain FP64 form; --precision fp32 selects the mixed
form.  Inputs are seeded synthetic bunches (Halton sequence) built by the reference's own
initialisation restated on the host; the march state (2.5 GB of potentials, 3.2 GB with the
particles) exceeds the 129 MB L2, so no L2 flush is needed between steps.

The timed window lies in the part of the march where the whole bunch is inside the undulator
(every particle gathers E and B and feels the undulator field): the march is run from its start
to 90 % of its steps, then W warm-up and K timed steps follow.  The whole march (start to
undulator exit) is timed beside it.  The CPU legs start the oracle from a snapshot of the same
march at the window's first step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU (the path is a
single domain per GPU); the value is the sum over ranks and the time the maximum over ranks.
`--impl reference` times the reference algorithm on the host cores instead: the C restatement
in oracle/ (the reference tree itself is not present on the GPU host), with all host threads.

Other workloads: `--workload sweep-192` (192 sweep-family designs stepped by one graph launch
per field step, FEL runs/h through a refilled queue) and `--workload surrogate` (FEL designs/h
with surrogate screening against the batched full solver, with the held-out P_sat error).
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
# First step of the timed window, as a fraction of the march (see window_start).
WINDOW_AT = 0.9
DEFAULT_STEPS, DEFAULT_WARMUP = 10, 3
# Timed repetitions of the e2e leg (restore, K steps, power rows): the host link's upload time
# varies between repetitions on the GB300 host (16-60 ms for the same 3.2 GB), so the median is
# reported with every repetition beside it.
E2E_REPEATS = 3
FP64_NOMINAL_TFLOPS = 1.25  # GB300 dense FP64, nominal

# Algorithmic bytes per unit (each array element counted once, halo re-reads free).
# Units: interior node for the stencils, interior node of the particle slab for E/B (read A^n and
# A^{n+1}, write E and B: doubles in the FP64 form, floats in the mixed form), particle for the
# particle kernels (plus the gathered E/B nodes for the push, GATHER_BYTES).
ALGO_BYTES = {
    "fp64": {"potential_interior_fd": 96, "potential_interior_nsfd": 96, "eval_eb": 96, "push": 96 + 1,
             "deposit": 48 + 8, "erase": 8 + 1},
    "fp32": {"potential_interior_fd": 48, "potential_interior_nsfd": 48, "eval_eb": 48, "push": 56 + 1,
             "deposit": 24 + 4 + 20, "erase": 12 + 1},
}


# Bytes of E and B per node that a push's gathers read: six doubles (FP64 form), six floats (mixed).
GATHER_BYTES = {"fp64": 48, "fp32": 24}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=DEFAULT_STEPS)
    ap.add_argument("--warmup", type=int, default=DEFAULT_WARMUP)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--workload", default="fel-130x130x2050", choices=sorted(WORKLOADS) + ["sweep-192", "surrogate"])
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
    ap.add_argument("--surrogate-designs", type=int, default=16384,
                    help="surrogate: designs solved by the full solver (training + held-out)")
    ap.add_argument("--surrogate-held-out", type=int, default=1024)
    ap.add_argument("--surrogate-threshold", type=float, default=0.1,
                    help="surrogate: ensemble spread of P_sat above which a design goes to the full solver")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp32-compare", action="store_true",
                    help="with --precision fp64, skip the mixed-form run reported under fp32_form")
    ap.add_argument("--snapshot-fd", type=int, default=None, help=argparse.SUPPRESS)
    ap.add_argument("--write-snapshot", default=None, metavar="DIR",
                    help="write the workload's march state at the timed window's first step (FP64 form) to "
                         "DIR and exit (nothing to do when DIR holds it already); `python -m "
                         "mithra_gb300.snapshot <job> --resume DIR` marches on from it")
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


def march_steps(setup, ctx) -> int:
    """Field steps of the march (`while (time_ < mesh_.totalTime_)`, src/solver.cpp:1300) from
    the context's time, which run_prelude has brought to the march's start."""
    t, total, dt = ctx.get_time().time, setup.total_time(), setup.meta()["dt"]
    n = 0
    while t < total:
        t += dt
        n += 1
    return n


def window_start(total: int, warmup: int, steps: int) -> int:
    """First step of the timed window.  Particles gather E and B and feel the undulator only once
    they have passed its entrance (the e flag, src/solver.cpp:1509-1514); the bunch of the default
    workload is wholly inside by 85 % of its march (step 1623 of 1905), so the window starts at 90 %,
    or earlier if the window and the legs after it would run past the undulator exit."""
    return max(warmup, min(int(WINDOW_AT * total), total - warmup - 3 * steps - 3))


def oracle_run_for(snap_info, snap):
    """The CPU restatement (oracle/) started from a snapshot of the march."""
    from oracle import pyoracle as po
    a = snap.fields
    return po, po.OracleRun(snap_info["meta"], a[1], a[2], a[0], snap.particles, solver=snap_info["solver"],
                            order=snap_info["order"])


STATE_DIR = os.path.join(REPO, "oracle", "_build", "state")


def window_snapshot_dir(workload):
    """Where build() leaves the workload's window snapshot (on a machine with a GPU)."""
    return os.path.join(STATE_DIR, os.path.splitext(WORKLOADS[workload])[0] + "-window")


def window_snapshot_ready(d, args, jobpath):
    """`d` holds the snapshot of the job file as it is now at the window's first step for these
    --steps/--warmup (checked from meta.json alone, without the CUDA library)."""
    from mithra_gb300 import snapshot
    try:
        with open(os.path.join(d, "meta.json")) as f:
            info = json.load(f)
    except (OSError, ValueError):
        return False
    total = info.get("march_steps")
    return total is not None and snapshot.current(d, jobpath, window_start(int(total), args.warmup, args.steps))


def window_snapshot_file(args, jobpath):
    """(info, snapshot) of the window's first step from the snapshot build() wrote, or None when
    it is absent or was taken at another step (read without the CUDA library)."""
    from mithra_gb300 import snapshot
    d = window_snapshot_dir(args.workload)
    if not window_snapshot_ready(d, args, jobpath):
        return None
    with open(os.path.join(d, "meta.json")) as f:
        info = json.load(f)
    return info, snapshot.load(d)


def window_snapshot_child(args, jobpath):
    """(info, snapshot) of the job at the window's first step, marched by the FP64 form in a child
    process (this process never loads the CUDA library) and streamed back through a pipe."""
    from mithra_gb300 import snapshot
    r, w = os.pipe()
    cmd = [sys.executable, os.path.abspath(__file__), "--snapshot-fd", str(w), "--workload", args.workload,
           "--steps", str(args.steps), "--warmup", str(args.warmup)]
    p = subprocess.Popen(cmd, cwd=REPO, pass_fds=(w,), stdout=sys.stderr)
    os.close(w)
    try:
        with os.fdopen(r, "rb") as f:
            info, snap = snapshot.read_stream(f)
    finally:
        rc = p.wait()
    if rc != 0:
        raise RuntimeError("window snapshot process exited with status %d" % rc)
    return info, snap


def write_window_snapshot(args):
    """--snapshot-fd / --write-snapshot: march the workload (FP64 form) to the window's first step
    and stream the snapshot to the descriptor or write it to the directory."""
    jobpath = os.path.join(REPO, "mithra_gb300", "jobs", WORKLOADS[args.workload])
    if args.write_snapshot and window_snapshot_ready(args.write_snapshot, args, jobpath):
        print("window snapshot in %s is current" % args.write_snapshot, file=sys.stderr)
        return
    import mithra_gb300 as mg
    from mithra_gb300 import snapshot
    setup = mg.Setup.from_job(jobpath)
    with mg.Context.from_setup(setup, mg.FP64) as ctx:
        ctx.run_prelude()
        total = march_steps(setup, ctx)
        start = window_start(total, args.warmup, args.steps)
        ctx.run(start)
        snap = snapshot.take(ctx)
    extra = {"march_steps": total}
    if args.write_snapshot:
        snapshot.save(snap, args.write_snapshot, jobpath, setup, start, extra)
        return
    with os.fdopen(args.snapshot_fd, "wb") as f:
        snapshot.write_stream(snap, f, jobpath, setup, start, extra)


def snapshot_info(setup, jobpath, snap, step):
    from mithra_gb300 import snapshot
    return snapshot._info(snap, jobpath, setup, step)


def touched_nodes(parts, meta) -> int:
    """Mesh nodes whose E and B the particles' gathers read: the 8 corners of each occupied cell
    (x index i < N0, y index j < N1, z plane k < np)."""
    lo = np.array([meta["xmin"], meta["ymin"], meta["zmin"]])
    h = np.array([meta["dx"], meta["dy"], meta["dz"]])
    ext = np.array([int(meta["N0"]), int(meta["N1"]), int(meta["np"])], dtype=np.int64)
    c = np.floor((parts[:, 1:4] - lo) / h).astype(np.int64)
    c = c[np.all((c >= 0) & (c < ext - 1), axis=1)]
    cells = np.unique((c[:, 2] * ext[1] + c[:, 1]) * ext[0] + c[:, 0])
    i, j, k = cells % ext[0], (cells // ext[0]) % ext[1], cells // (ext[0] * ext[1])
    corners = [((k + dk) * ext[1] + j + dj) * ext[0] + i + di for dk in (0, 1) for dj in (0, 1) for di in (0, 1)]
    return int(np.unique(np.concatenate(corners)).size)


def slab_nodes(parts, meta) -> int:
    """Interior nodes on the planes the E/B evaluation covers: the particles' cell planes with two
    planes of margin below and three above (eb_plane_wanted in the kernels)."""
    ext = int(meta["np"])
    k = np.floor((parts[:, 3] - meta["zmin"]) / meta["dz"]).astype(np.int64)
    k = k[(k >= 0) & (k < ext - 1)]
    if k.size == 0:
        return 0
    lo, hi = max(1, int(k.min()) - 2), min(ext - 2, int(k.max()) + 3)
    return (hi - lo + 1) * (int(meta["N0"]) - 2) * (int(meta["N1"]) - 2)


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


def cpu_baseline(snap_info, snap, sample_seconds):
    po, run = oracle_run_for(snap_info, snap)
    threads = cpu_threads()
    nodes, pushes, _ = units_per_step(snap_info["meta"], run.n)
    po.set_threads(threads)
    run.step()  # first-touch of the arrays
    steps, el = time_oracle(run, po, threads, sample_seconds, 200)
    return {"value": (nodes + pushes) * steps / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": "%d field steps from step %d of the same march (after one untimed step; the "
                      "bench window's part of the march, every particle inside the undulator), C "
                      "restatement of the reference with OpenMP over %d host threads, %.1f s"
                      % (steps, snap_info["step"], threads, el)}


def run_reference(args, dist):
    """The reference algorithm on the host cores: the oracle's C restatement (pinned bit for bit
    to the reference in the container that has the reference tree; that tree is not on the GPU
    host, so its binary cannot be built here), all host threads, then one thread.  It starts from
    the march state at the window's first step, computed by the FP64 form (the CPU would take
    about 15 minutes to march there): the snapshot build() writes on a machine with a GPU, or,
    when that is absent, one a child process marches and streams back.  This process loads no
    CUDA library either way."""
    jobpath = os.path.join(REPO, "mithra_gb300", "jobs", WORKLOADS[args.workload])
    if dist.rank != 0:
        return
    got = window_snapshot_file(args, jobpath)
    source = "written by build()"
    if got is None:
        got = window_snapshot_child(args, jobpath)
        source = "marched by a child process and streamed through a pipe"
    info, snap = got
    po, run = oracle_run_for(info, snap)
    del snap
    threads = cpu_threads()
    nodes, pushes, nsub = units_per_step(info["meta"], run.n)
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
    entered = float(np.mean(run.particles[:, 10] > 0.5))
    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Halton bunch of the job file)",
        "config": run_config(args.workload, nodes, run.n, nsub, "fp64", dist.world),
        "window": {"first_step": info["step"] + args.warmup, "steps": args.steps, "entered_fraction": entered,
                   "how": "the march state of step %d (FP64 form on the GPU, %s), W warm-up and K timed "
                          "steps on the host" % (info["step"], source)},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": "%d timed field steps after %d warm-up steps from step %d of the march, C "
                                   "restatement of the reference (oracle/) with OpenMP over %d host threads, one "
                                   "process (the reference's MPI decomposition is not used: a single domain)"
                                   % (args.steps, args.warmup, info["step"], threads)},
        "one_thread": {"value": v1, "unit": METRIC, "cores": 1, "threads": 1, "ms_per_step": 1e3 * el1 / s1,
                       "sample": "%d further field steps of the same march on one thread" % s1,
                       "threads_speedup": value / v1},
        "host": host_cpu(),
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def measure_form(mg, setup, prec_name, args, dist, units, interior, keep_snapshot=False):
    """One precision form on the workload, march order:

    steps 0..W        untimed (every step graph captured)
    steps W..S        timed: the entry phase of the march
    step S            snapshot of the state into page-locked host memory
    S..S+W            warm-up at the window
    S+W..S+W+K        timed: the headline window (CUDA events on the context stream)
    S+W+K..S+W+2K     per-kernel times (each kernel bracketed by CUDA events)
    e2e               the step-S snapshot uploaded from host memory, K steps, power rows read
    S+K..exit         timed: the rest of the march

    The whole march's device time is the timed parts plus steps 0..W at the entry phase's rate
    and S..S+K at the window's."""
    from mithra_gb300 import snapshot
    prec = mg.FP64 if prec_name == "fp64" else mg.FP32
    ctx = mg.Context.from_setup(setup, prec, device=dist.local)
    n_part = ctx.particle_count()
    ctx.run_prelude()
    total = march_steps(setup, ctx)
    start = window_start(total, args.warmup, args.steps)
    ctx.run(args.warmup)
    ms_entry = ctx.run_timed(start - args.warmup)
    snap = snapshot.take(ctx, pinned=True)
    entered = float(np.mean(snap.particles[:, 10] > 0.5))
    ctx.run(args.warmup)
    ctx.synchronize()
    dist.barrier()
    with ClockSampler(dist.local) as clk:
        ms = ctx.run_timed(args.steps)
    dist.barrier()
    ms_max = dist.max(ms)
    out = {"ms_total": ms_max, "ms_per_step": ms_max / args.steps,
           "value": dist.world * units * args.steps / (ms_max / 1e3), "clocks": clk.summary()}
    window = {"first_step": start + args.warmup, "steps": args.steps, "march_steps": total,
              "entered_fraction": entered,
              "how": "K timed steps after W warm-up steps from step %d of the %d-step march, where "
                     "%.4f of the particles are inside the undulator" % (start, total, entered)}

    # Per-kernel device times: the same K steps again, each kernel bracketed by CUDA events on
    # the context stream (direct launches instead of the step graph).
    ctx.enable_timing(True)
    ctx.run(args.steps)
    kt = ctx.kernel_times()
    ctx.enable_timing(False)
    total_k = sum(v[0] for v in kt.values())
    dominant = max(kt.items(), key=lambda kv: kv[1][0])[0]
    dom_ms, dom_launches = kt[dominant]
    particle_kernels = ("push", "deposit", "erase", "tile_scatter")
    # the push's gathers read E and B of every node around an occupied cell once per launch
    gather = touched_nodes(snap.particles, setup.meta()) if entered > 0.0 else 0
    window["gather_nodes"] = gather
    # E and B are evaluated on the particles' planes only
    eb_nodes = slab_nodes(snap.particles, setup.meta())
    window["eb_slab_nodes"] = eb_nodes

    def units_of(k):
        if k in particle_kernels:
            return n_part
        return eb_nodes if k == "eval_eb" else interior

    def algo_bytes(k, count):
        pu = ALGO_BYTES[prec_name].get(k)
        if not pu:
            return None
        return pu * count + (GATHER_BYTES[prec_name] * gather if k == "push" else 0)

    unit_count = units_of(dominant)
    peak, peak_kind = measured_peaks()
    roof = None
    ab = algo_bytes(dominant, unit_count)
    if ab:
        avg_s = dom_ms / dom_launches / 1e3
        achieved = ab / avg_s / 1e9
        tr = traffic_table().get(prec_name, {}).get(dominant)
        roof = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "algorithmic_bytes_per_launch": ab,
                "traffic": (tr * unit_count if tr else None),
                "avg_launch_ms": dom_ms / dom_launches, "share": dom_ms / total_k}
    out["roofline"] = roof
    out["dominant"] = (dominant, dom_ms / dom_launches, unit_count)
    out["kernels"] = {k: {"ms_per_launch": v[0] / v[1], "launches": v[1], "share": v[0] / total_k}
                      for k, v in kt.items()}
    for k, v in out["kernels"].items():
        ab = algo_bytes(k, units_of(k))
        if ab:
            v["hbm_frac"] = ab / (v["ms_per_launch"] / 1e3) / 1e9 / peak
            v["units"] = units_of(k)

    # End to end through the public API with host buffers: the step-S state uploaded from
    # page-locked host memory (a resumed march), K steps, the power rows read back.  One untimed
    # restore of the same buffers first, as the warm-up steps precede the device timing: the
    # first upload after the snapshot was written runs 4-10x slower than the later ones on the
    # GB300 host (reported as first_restore_ms).
    e2e = None
    if not args.no_e2e:
        ctx.synchronize()
        tw = time.perf_counter()
        snapshot.restore(ctx, snap)
        first_restore_ms = 1e3 * (time.perf_counter() - tw)
        ctx.power_rows()  # the rows logged so far, so that each repetition reads its own K rows
        reps = []
        for _ in range(E2E_REPEATS):
            dist.barrier()
            t0 = time.perf_counter()
            snapshot.restore(ctx, snap)
            t1 = time.perf_counter()
            ctx.run(args.steps)
            rows = ctx.power_rows()
            t2 = time.perf_counter()
            reps.append((dist.max(t2 - t0), 1e3 * (t1 - t0), 1e3 * (t2 - t1), rows.nbytes))
        el, up_ms, march_ms, row_bytes = sorted(reps)[len(reps) // 2]  # the median repetition
        e2e = {"value": dist.world * units * args.steps / el, "unit": METRIC,
               "h2d_bytes_per_step": snap.nbytes / args.steps, "d2h_bytes_per_step": row_bytes / args.steps,
               "ms_per_step": 1e3 * el / args.steps, "upload_ms": up_ms, "march_ms": march_ms,
               "repeats_ms_per_step": [1e3 * r[0] / args.steps for r in reps],
               "first_restore_ms": first_restore_ms,
               "warmup": "one untimed restore of the same host buffers; the median of %d timed repetitions" % E2E_REPEATS,
               "how": "march state of step %d (fields, particles, time) uploaded from page-locked host "
                      "memory, K steps, the K power rows read back" % start}
        rest_from = start + args.steps
    else:
        rest_from = start + args.warmup + 2 * args.steps
    ms_rest = ctx.run_timed(total - rest_from) if total > rest_from else 0.0
    march_ms = (args.warmup * ms_entry / max(start - args.warmup, 1) + ms_entry
                + (rest_from - start) * ms / args.steps + ms_rest)
    window["march"] = {"steps": total, "device_s": march_ms / 1e3,
                       "value": dist.world * units * total / (march_ms / 1e3), "unit": METRIC,
                       "entry_phase_ms_per_step": ms_entry / max(start - args.warmup, 1),
                       "rest_ms_per_step": ms_rest / max(total - rest_from, 1),
                       "how": "device time of the whole march from its start to the undulator exit: steps "
                              "%d..%d and %d..%d timed, the %d steps before and the %d at the window at "
                              "their phase's rate" % (args.warmup, start, rest_from, total, args.warmup,
                                                      rest_from - start)}
    out["window"] = window
    out["e2e"] = e2e
    out["launches"] = ctx.launches_per_step() * args.steps
    out["n_part"] = n_part
    ctx.close()
    if keep_snapshot:
        out["snapshot"] = (snapshot_info(setup, os.path.join(REPO, "mithra_gb300", "jobs", WORKLOADS[args.workload]),
                                         snap, start), snap)
    else:
        snap.free()
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
    want_cpu = dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline
    main = measure_form(mg, setup, args.precision, args, dist, units, interior, keep_snapshot=want_cpu)
    ms_max = main["ms_total"]
    value = main["value"]
    cpu = None
    if want_cpu:  # the oracle from the same march state as the window, on the host cores
        info, snap = main.pop("snapshot")
        try:
            cpu = cpu_baseline(info, snap, args.cpu_sample_seconds)
        finally:
            snap.free()

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
                     "e2e": f["e2e"], "clocks": f["clocks"], "gpu_launches": f["launches"], "window": f["window"],
                     "march_speedup_vs_fp64": f["window"]["march"]["value"] / main["window"]["march"]["value"]}

    runs = None
    if args.workload == "fel-130x130x2050" and args.sweep_leg_designs > 0:
        runs = sweep_leg(args, dist)

    if dist.rank != 0:
        return
    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
        "data": "synthetic (seeded Halton bunch of the job file)",
        "config": run_config(args.workload, nodes, n_part, nsub, args.precision, dist.world),
        "cell_updates_per_s": dist.world * nodes * args.steps / (ms_max / 1e3),
        "particle_pushes_per_s": dist.world * pushes * args.steps / (ms_max / 1e3),
        "window": main["window"],
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


def run_surrogate(args, dist):
    """FEL designs per hour with surrogate screening, against the batched full solver: seeded designs
    of the surrogate family (48x48x384 cells, 131,072 particles, NSFD, mixed form) solved in batches,
    an ensemble trained on all but the held-out designs by the library's tcgen05 GEMMs, and the
    held-out designs screened at the spread threshold (the full solver takes those above it).  A
    screened design costs the ensemble's inference plus, for the fallback fraction, a full solve."""
    import tempfile

    from mithra_gb300 import surrogate as sg
    if dist.rank != 0:
        return
    n, held, thr = args.surrogate_designs, args.surrogate_held_out, args.surrogate_threshold
    ps = sg.design_parameters(n, 7)
    with ClockSampler(dist.local) as clk:
        curves, spectra, psat, host_s, dev_s = sg.solve_designs(ps, 128, tempfile.mkdtemp(prefix="mithra-surrogate-"),
                                                                device=dist.local)
        out = sg.train_and_screen(sg.features(ps), curves, spectra, psat, host_s, dev_s, held, 128,
                                  thresholds=sorted({0.02, 0.05, 0.1, 0.2, thr}))
    print(json.dumps(surrogate_line(out, n, held, thr, clk.summary())), flush=True)


def surrogate_line(out: dict, n: int, held: int, thr: float, clocks: dict) -> dict:
    """The bench line of the surrogate workload from `surrogate.train_and_screen`'s result: the
    screened designs per hour at threshold `thr` (inference for every design plus a full solve for
    the fallback fraction), the batched full solver's designs per hour and the held-out error."""
    row = next(r for r in out["screening"] if r["threshold"] == thr)
    solve_s = out["solve_s_per_design"]
    screened_s = out["infer_s_per_design"] + row["fallback"] * solve_s
    return {
        "metric": "FEL designs/h (surrogate-screened)", "value": 3600.0 / screened_s, "unit": "designs/h",
        "n_gpus": 1, "steps": out["train_steps"], "warmup": 0, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16", "data": "synthetic (seeded designs, Halton bunches)",
        "config": {"workload": "surrogate-48x48x384", "designs": n, "held_out": held, "threshold": thr,
                   "precision": "fp32 (mixed form) solves, bf16 network with fp32 accumulation",
                   "parallelism": "single-gpu"},
        "full_solve_designs_per_hour": 3600.0 / solve_s,
        "speedup_vs_full_solve": row["speedup"],
        "held_out_psat_error": {"median": out["median_err"], "p90": out["p90_err"],
                                "accepted_median": row["accepted_median_err"], "accepted_p90": row["accepted_p90_err"],
                                "fallback": row["fallback"], "trivial_median": out["baseline_median_err"]},
        "train_s": out["train_s"], "infer_s_per_design": out["infer_s_per_design"], "screening": out["screening"],
        "clocks": clocks,
    }


def main():
    args = parse_args()
    if args.snapshot_fd is not None or args.write_snapshot:
        write_window_snapshot(args)
        return
    dist = Dist(args.gpus)
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        elif args.workload == "sweep-192":
            run_sweep(args, dist)
        elif args.workload == "surrogate":
            run_surrogate(args, dist)
        else:
            run_gpu(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
