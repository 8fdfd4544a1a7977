"""March state snapshots: checkpoint and resume of a solve through the C ABI.

A snapshot is everything a field step reads from the previous one: the vector-potential levels
(anp1_, which holds the current J between steps, an_ and anm1_; src/solver.h:231-233), the
scalar levels of an FdTdSC solve (src/solver.h:236-238), the particle records chargeVectorn_
(q, rnp, rnm, gb, e; src/stdinclude.h:130-144) and the time state (time_, timeBunch_, nTime_,
nTimeBunch_; src/solver.h:266-275).  The device keeps nothing else that a step depends on: the
tile sort is rebuilt from the particle records, E and B from the potentials, and the undulator
phases from the time.  Power-sampling sums stay with the context they were taken in.

The reference writes bunch and field profiles as text but reads neither back
(src/solver.cpp:1763-1792, src/fdtd.cpp:1546-1594), so it has no resume path to match; the
FP64 form resumed from a snapshot continues the march up to the rounding of the current
deposition's atomic sums.

On disk a snapshot is a directory: meta.json (job file, step, time state, and the job's meta
values with the time state of the snapshot), fields.npz, scalar.npz (FdTdSC) and
particles.npy.

    python -m mithra_gb300.snapshot <job file> (<output directory> | --fd N) --step S [--precision fp64|fp32]
    python -m mithra_gb300.snapshot <job file> --resume <directory> --run N [--precision fp64|fp32]

The first marches the job S field steps on the GPU and writes the snapshot to the directory, or
as a stream (write_stream) to file descriptor N; the second puts a snapshot of the job into a
fresh context and marches N field steps from it (a profiler's view of one part of a march).
"""
from __future__ import annotations

import argparse
import json
import os
from dataclasses import dataclass

import numpy as np

from . import FP32, FP64, Context, PinnedArray, Setup, TimeState

FORMAT = 1


@dataclass
class Snapshot:
    fields: tuple            # (anp1, an, anm1), FP64, nodes x 3 each
    scalar: tuple | None     # (fnp1, fn, fnm1) for FdTdSC, else None
    particles: np.ndarray    # rows of 11 doubles
    time: tuple              # (time, time_bunch, n_time, n_time_bunch)
    _pinned: list | None = None

    @property
    def step(self) -> int:
        return int(self.time[2])

    @property
    def nbytes(self) -> int:
        n = sum(a.nbytes for a in self.fields) + self.particles.nbytes
        if self.scalar is not None:
            n += sum(a.nbytes for a in self.scalar)
        return n

    def free(self):
        """Releases the page-locked buffers of a snapshot taken with pinned=True."""
        for b in self._pinned or []:
            b.free()
        self._pinned = None
        self.fields = self.scalar = self.particles = None


def take(ctx: Context, pinned: bool = False) -> Snapshot:
    """The state of `ctx` between two field steps.  With `pinned`, the arrays live in
    page-locked host memory (freed by Snapshot.free), so that restoring them runs at the
    host link's full rate."""
    n = ctx.nodes * 3
    npart = ctx.particle_count()
    bufs = []

    def alloc(shape):
        if pinned:
            b = PinnedArray(shape)
            bufs.append(b)
            return b.array
        return np.empty(shape)

    fields = ctx.download_fields(out=(alloc(n), alloc(n), alloc(n)))
    scalar = None
    if ctx.grid.space_charge:
        m = ctx.nodes
        scalar = ctx.download_scalar(out=(alloc(m), alloc(m), alloc(m)))
    parts = ctx.download_particles(out=alloc((max(npart, 1), 11)))
    t = ctx.get_time()
    return Snapshot(tuple(fields), None if scalar is None else tuple(scalar), parts,
                    (t.time, t.time_bunch, int(t.n_time), int(t.n_time_bunch)), bufs or None)


def restore(ctx: Context, snap: Snapshot):
    """Puts a snapshot into `ctx` (a context of the same job and mesh, either precision)."""
    if snap.fields[0].size != ctx.nodes * 3:
        raise ValueError("snapshot of %d nodes, context of %d" % (snap.fields[0].size // 3, ctx.nodes))
    if bool(ctx.grid.space_charge) != (snap.scalar is not None):
        raise ValueError("snapshot and context differ in the scalar potential (FdTd vs FdTdSC)")
    ctx.upload_fields(*snap.fields)
    if snap.scalar is not None:
        ctx.upload_scalar(*snap.scalar)
    ctx.upload_particles(snap.particles)
    ctx.set_time(TimeState(snap.time[0], snap.time[1], snap.time[2], snap.time[3]))


def save(snap: Snapshot, out_dir: str, job_path: str, setup: Setup, step: int | None = None,
         extra: dict | None = None):
    """Writes `snap` of `job_path` (initialised as `setup`) to `out_dir`; `step`: the field steps
    marched since the job's start (default: the snapshot's nTime); `extra`: more keys for
    meta.json."""
    os.makedirs(out_dir, exist_ok=True)
    if os.path.exists(os.path.join(out_dir, "meta.json")):  # no stale marker while the arrays change
        os.remove(os.path.join(out_dir, "meta.json"))
    anp1, an, anm1 = snap.fields
    np.savez(os.path.join(out_dir, "fields.npz"), anp1=anp1, an=an, anm1=anm1)
    if snap.scalar is not None:
        fnp1, fn, fnm1 = snap.scalar
        np.savez(os.path.join(out_dir, "scalar.npz"), fnp1=fnp1, fn=fn, fnm1=fnm1)
    np.save(os.path.join(out_dir, "particles.npy"), np.ascontiguousarray(snap.particles))
    info = _info(snap, job_path, setup, step, extra)
    tmp = os.path.join(out_dir, "meta.json.tmp")
    with open(tmp, "w") as f:
        json.dump(info, f)
    os.replace(tmp, os.path.join(out_dir, "meta.json"))  # written last: marks the snapshot complete


def load(in_dir: str) -> Snapshot:
    with open(os.path.join(in_dir, "meta.json")) as f:
        info = json.load(f)
    if info.get("format") != FORMAT:
        raise ValueError("%s: snapshot format %r, expected %d" % (in_dir, info.get("format"), FORMAT))
    z = np.load(os.path.join(in_dir, "fields.npz"))
    scalar = None
    if os.path.exists(os.path.join(in_dir, "scalar.npz")):
        s = np.load(os.path.join(in_dir, "scalar.npz"))
        scalar = (s["fnp1"], s["fn"], s["fnm1"])
    t = info["time"]
    return Snapshot((z["anp1"], z["an"], z["anm1"]), scalar, np.load(os.path.join(in_dir, "particles.npy")),
                    (float(t[0]), float(t[1]), int(t[2]), int(t[3])))


def _info(snap: Snapshot, job_path: str, setup: Setup, step: int | None, extra: dict | None = None) -> dict:
    g = setup.grid()
    meta = dict(setup.meta())
    meta.update({"time": snap.time[0], "timeBunch": snap.time[1], "nTime": snap.time[2],
                 "nTimeBunch": snap.time[3]})
    info = {"format": FORMAT, "job": os.path.abspath(job_path), "job_mtime": os.path.getmtime(job_path),
            "step": snap.step if step is None else int(step), "solver": int(g.solver),
            "order": int(g.truncation_order), "total_time": setup.total_time(),
            "n_particles": int(snap.particles.shape[0]), "time": list(snap.time), "meta": meta}
    info.update(extra or {})
    return info


class _Pipe:
    """A file object that numpy's .npy reader and writer treat as a plain stream (chunked reads
    and writes, no seek or tell, which a pipe does not have)."""

    def __init__(self, f):
        self._f = f

    def read(self, n=-1):
        return self._f.read(n)

    def readline(self):
        return self._f.readline()

    def write(self, b):
        return self._f.write(b)

    def flush(self):
        self._f.flush()


def write_stream(snap: Snapshot, f, job_path: str, setup: Setup, step: int | None = None, extra: dict | None = None):
    """Writes `snap` to the binary stream `f` (a pipe, say): one JSON line as in meta.json (plus
    `extra`) with the names of the arrays, then each array in .npy format."""
    names = ["anp1", "an", "anm1"] + (["fnp1", "fn", "fnm1"] if snap.scalar is not None else []) + ["particles"]
    arrays = list(snap.fields) + (list(snap.scalar) if snap.scalar is not None else []) + [snap.particles]
    info = _info(snap, job_path, setup, step, extra)
    info["arrays"] = names
    f = _Pipe(f)
    f.write((json.dumps(info) + "\n").encode())
    for a in arrays:
        np.lib.format.write_array(f, np.ascontiguousarray(a), allow_pickle=False)
    f.flush()


def read_stream(f):
    """(info, Snapshot) from a stream written by write_stream; needs no GPU and no library."""
    f = _Pipe(f)
    info = json.loads(f.readline().decode())
    if info.get("format") != FORMAT:
        raise ValueError("snapshot stream format %r, expected %d" % (info.get("format"), FORMAT))
    arr = {n: np.lib.format.read_array(f, allow_pickle=False) for n in info["arrays"]}
    scalar = (arr["fnp1"], arr["fn"], arr["fnm1"]) if "fnp1" in arr else None
    t = info["time"]
    return info, Snapshot((arr["anp1"], arr["an"], arr["anm1"]), scalar, arr["particles"],
                          (float(t[0]), float(t[1]), int(t[2]), int(t[3])))


def current(in_dir: str, job_path: str, step: int) -> bool:
    """`in_dir` holds the snapshot of this job file, as it is now, `step` field steps in."""
    try:
        with open(os.path.join(in_dir, "meta.json")) as f:
            info = json.load(f)
    except (OSError, ValueError):
        return False
    return (info.get("format") == FORMAT and info.get("job") == os.path.abspath(job_path)
            and info.get("job_mtime") == os.path.getmtime(job_path) and info.get("step") == step
            and os.path.exists(os.path.join(in_dir, "particles.npy")))


def march(job_path: str, step: int, precision: int = FP64, device: int = 0):
    """(setup, snapshot) of the job after `step` field steps from its initial state."""
    setup = Setup.from_job(job_path, device=device)
    with Context.from_setup(setup, precision, device=device) as ctx:
        ctx.run_prelude()
        ctx.run(step)
        return setup, take(ctx)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("job")
    ap.add_argument("out_dir", nargs="?", help="directory to write (or --fd)")
    ap.add_argument("--fd", type=int, help="write the snapshot as a stream to this file descriptor")
    ap.add_argument("--step", type=int)
    ap.add_argument("--resume", metavar="DIR", help="march on from the snapshot in DIR")
    ap.add_argument("--run", type=int, default=0, help="with --resume: field steps to march")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args()
    prec = FP64 if a.precision == "fp64" else FP32
    if a.resume:
        setup = Setup.from_job(a.job, device=a.device)
        with Context.from_setup(setup, prec, device=a.device) as ctx:
            restore(ctx, load(a.resume))
            ctx.run(a.run)
            ctx.synchronize()
        return
    if (a.out_dir is None) == (a.fd is None) or a.step is None:
        ap.error("give --step and an output directory or --fd")
    setup, snap = march(a.job, a.step, prec, a.device)
    if a.fd is not None:
        with os.fdopen(a.fd, "wb") as f:
            write_stream(snap, f, a.job, setup, a.step)
    else:
        save(snap, a.out_dir, a.job, setup, a.step)


if __name__ == "__main__":
    main()
