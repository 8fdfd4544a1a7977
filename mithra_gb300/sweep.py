"""Parameter sweeps of FEL designs run as one batch of independent instances.

Each instance is a job of the 48x48x384 FEL family with its own undulator, bunch and mesh,
drawn from fixed ranges with a seeded generator:

    gamma 80 .. 400, undulator parameter K 0.8 .. 2.0, period 1.5 .. 3 cm (30 periods),
    charge 50 .. 500 pC, relative energy spread 1e-5 .. 1e-3,
    transverse cells 32 .. 96, longitudinal cells 128 .. 768, macro-particles 5e4 .. 1e6.

The mesh length along z follows each design's resonant wavelength (4.8 cells per wavelength, as
in the 48x48x384 job) and the solver is NSFD, which may widen the transverse cells.

The jobs are ordinary job files (written to a work directory), set up on the host in parallel
and stepped together on one device by `mithra_gb300.Batch`.
"""
from __future__ import annotations

import math
import os
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import FP32, Batch, Context, Setup

ELECTRONS_PER_PC = 1.0 / 1.602e-7
PERIODS = 30


def sweep_parameters(n: int = 192, seed: int = 20261204) -> list[dict]:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        out.append(dict(
            index=i,
            gamma=float(rng.uniform(80.0, 400.0)),
            K=float(rng.uniform(0.8, 2.0)),
            lambda_u=float(rng.uniform(1.5e4, 3.0e4)),           # um
            charge_pc=float(rng.uniform(50.0, 500.0)),
            energy_spread=float(10.0 ** rng.uniform(-5.0, -3.0)),
            n_transverse=int(rng.integers(32, 97)),
            n_longitudinal=int(rng.integers(128, 769)),
            particles=int(rng.integers(50_000, 1_000_001)),
            solver="NSFD",
        ))
    return out


def job_text(p: dict, spectrum_points: int = 0) -> str:
    """Job file of one sweep instance (the 48x48x384 FEL job with the instance's parameters).
    p may set "periods" (default 30), "sigma_r" (transverse rms size in um, default 200),
    "lz" (mesh length along z in um; the bunch's rms length is lz / 6, truncated at lz / 3, and
    the power is sampled at z = lz / 3) and "solver" ("FD" or "NSFD", default FD; the sweep family
    uses NSFD, the reference's solver for FEL runs: with FD, low-gamma designs of the family can
    diverge in both precision forms).  The default
    lz follows the radiation as the 48x48x384 FEL job does (80 resonant wavelengths on 384 cells):
    4.8 cells per resonant wavelength lambda_u (1 + K^2 / 2) / (2 gamma^2) along z, so that every
    design resolves its own radiation; a fixed lz leaves the radiation of high-gamma designs
    below one cell per wavelength, and such marches diverge;
    spectrum_points > 0 samples the power at that many normalized frequencies in 0.89 .. 1.11
    (centred on 1.0) instead of at 1.0 only.  p["seed_a0"] > 0 adds a continuous gaussian-beam seed at the
    resonant wavelength lambda_u (1 + K^2/2) / (2 gamma^2), polarised along y, focused at the
    undulator start with a waist of 2 sigma_r and that strength parameter."""
    lam = p["lambda_u"] * (1.0 + 0.5 * p["K"] ** 2) / (2.0 * p["gamma"] ** 2)
    lx, lz = 2400.0, float(p.get("lz", p["n_longitudinal"] / 4.8 * lam))
    dx, dz = lx / p["n_transverse"], lz / p["n_longitudinal"]
    # the reference counts cells as int(L / d) + 1 (src/solver.cpp:610-612): a length a hair above
    # the whole number of cells keeps that count from losing one to rounding
    lz = dz * p["n_longitudinal"] * (1.0 + 1e-12)
    periods = int(p.get("periods", PERIODS))
    sr = float(p.get("sigma_r", 200.0))
    solver = p.get("solver", "FD")
    # march from the bunch's start to the undulator exit (plus the 2-period default gap)
    total_time = (periods + 2) * p["lambda_u"] / 299.792458 * 1.05
    if spectrum_points > 0:
        # The DFT window of the power sampling is Nf = int(3 T / dt) samples, T the period of the
        # lowest frequency (src/radiation.cpp:88-93); this family's time step is T_1.0 / 9.6, so a band
        # starting at 0.9 puts 3 T / dt at exactly 32 and rounding picks Nf = 31 or 32 (a jump of
        # several percent in the sampled power) from design to design.  0.89 gives 32.36: Nf = 32.
        freq = ("minimum-normalized-frequency = 0.89\n    maximum-normalized-frequency = 1.11\n"
                "    number-of-frequency-points   = %d" % spectrum_points)
    else:
        freq = "normalized-frequency    = 1.0"
    a0 = float(p.get("seed_a0", 0.0))
    field = ""
    if a0 > 0.0:
        lam = p["lambda_u"] * (1.0 + 0.5 * p["K"] ** 2) / (2.0 * p["gamma"] ** 2)
        field = f"""
FIELD
{{
  field-initialization
  {{
    type                    = gaussian-beam
    position                = ( 0.0, 0.0, 0.0 )
    direction               = ( 0.0, 0.0, 1.0 )
    polarization            = ( 0.0, 1.0, 0.0 )
    radius-parallel         = {2.0 * sr!r}
    radius-perpendicular    = {2.0 * sr!r}
    strength-parameter      = {a0!r}
    signal-type             = gaussian
    offset                  = 0.0
    pulse-length            = 1.0e12
    wavelength              = {lam!r}
    CEP                     = 0.0
  }}
}}
"""
    return f"""# sweep instance {p['index']}
MESH
{{
  length-scale              = MICROMETER
  time-scale                = PICOSECOND
  mesh-lengths              = ( {lx}, {lx}, {lz} )
  mesh-resolution           = ( {dx!r}, {dx!r}, {dz!r} )
  mesh-center               = ( 0.0, 0.0, 0.0 )
  total-time                = {total_time!r}
  bunch-time-step           = 1.6
  mesh-truncation-order     = 2
  space-charge              = false
  solver                    = {solver}
}}

BUNCH
{{
  bunch-initialization
  {{
    type                    = ellipsoid
    distribution            = uniform
    charge                  = {p['charge_pc'] * ELECTRONS_PER_PC!r}
    number-of-particles     = {p['particles']}
    gamma                   = {p['gamma']!r}
    direction               = ( 0.0, 0.0, 1.0 )
    position                = ( 0.0, 0.0, 0.0 )
    sigma-position          = ( {sr!r}, {sr!r}, {lz / 6.0!r} )
    sigma-momentum          = ( 0.005, 0.005, {p['energy_spread'] * p['gamma']!r} )
    transverse-truncation   = {4.0 * sr!r}
    longitudinal-truncation = {lz / 3.0!r}
    shot-noise              = true
  }}
}}

{field}
UNDULATOR
{{
  static-undulator
  {{
    undulator-parameter     = {p['K']!r}
    period                  = {p['lambda_u']!r}
    length                  = {periods}
    polarization-angle      = 0.0
  }}
}}

FEL-OUTPUT
{{
  radiation-power
  {{
    sample                  = true
    type                    = at-point
    directory               = ./
    base-name               = power-sampling/power
    plane-position          = {lz / 3.0!r}
    {freq}
  }}
}}
"""


def make_setups(params: list[dict], workdir: str, threads: int | None = None, spectrum_points: int = 0) -> list[Setup]:
    """Writes the job files and runs the host initialisation of every instance in parallel."""
    os.makedirs(workdir, exist_ok=True)
    paths = []
    for p in params:
        path = os.path.join(workdir, "sweep-%03d.job" % p["index"])
        with open(path, "w") as f:
            f.write(job_text(p, spectrum_points))
        paths.append(path)
    with ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 4) as ex:
        return list(ex.map(Setup.from_job, paths))


def make_batch(setups: list[Setup], precision: int = FP32, device: int = 0, autotune_steps: int = 0):
    """Contexts for every instance (prelude marched), optionally autotuned, and their batch."""
    contexts = []
    for s in setups:
        c = Context.from_setup(s, precision, device)
        c.run_prelude()
        contexts.append(c)
    tuned = []
    if autotune_steps > 0:
        for c in contexts:
            tuned.append(c.autotune(autotune_steps))
    # tuning marches each instance by the same number of steps, so they stay in one step phase
    return Batch(contexts), contexts, tuned


def steps_to_exit(setup: Setup, ctx: Context) -> int:
    """Field steps left until the job's total time (the reference's `while (time_ < totalTime)`)."""
    t = ctx.get_time()
    total, dt = setup.total_time(), setup.meta()["dt"]
    time, n = t.time, 0
    while time < total:
        time += dt
        n += 1
    return n


def run_queue(params: list[dict], workdir: str, slots: int = 192, precision: int = FP32, device: int = 0,
              device_init: bool = True, min_chunk: int = 30, spectrum_points: int = 0):
    """Marches every design to its undulator exit with at most `slots` instances on the device:
    the batch runs until its earliest design exits (at least `min_chunk` steps, a multiple of six
    so that every instance stays in the same step phase), finished designs leave with their
    power rows and new designs take their slots (set up on the device when `device_init`).
    Returns ({index: power rows}, wall seconds, batch rebuilds)."""
    from . import Batch, Context, Setup
    os.makedirs(workdir, exist_ok=True)
    queue = list(params)
    active = []  # [params, context, field steps left]
    done = {}
    rebuilds = 0
    t0 = time.perf_counter()

    def admit():
        while queue and len(active) < slots:
            p = queue.pop(0)
            path = os.path.join(workdir, "queue-%06d.job" % p["index"])
            with open(path, "w") as f:
                f.write(job_text(p, spectrum_points))
            s = Setup.from_job(path, device_init=device_init, device=device)
            c = Context.from_setup(s, precision, device)
            c.run_prelude()
            active.append([p, c, steps_to_exit(s, c)])

    admit()
    while active:
        n = max(min_chunk, min(a[2] for a in active))
        n = 6 * math.ceil(n / 6)
        batch = Batch([a[1] for a in active])
        batch.run(n)
        batch.close()
        rebuilds += 1
        keep = []
        for a in active:
            a[2] -= n
            if a[2] <= 0:
                done[a[0]["index"]] = a[1].power_rows()
                a[1].close()
            else:
                keep.append(a)
        active[:] = keep
        admit()
    return done, time.perf_counter() - t0, rebuilds
