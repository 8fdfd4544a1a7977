"""Seeded initial state of a job for the oracle, written to disk by one process, read by another.

TEST INFRASTRUCTURE ONLY (like the rest of oracle/): the CPU timing legs of bench.py start the
oracle from this file, so that a process timing the oracle never loads the CUDA library.

The state is what Solver::initialize produces (src/solver.cpp:547-595): the meta values the
oracle reads (mesh, coefficients, frame, power-sampling planes and twiddles, time state), the
three initial vector-potential levels and the particle records.  It is computed by the host
initialisation of mithra_gb300 (libmithra_gb300.so), which tests/test_host_setup.py checks bit
for bit against the reference's own initialisation.

    python -m oracle.initial_state <job file> <output directory>

writes meta.json, particles.npy and, when any is non-zero, fields.npz.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

FORMAT = 1


def write(job_path: str, out_dir: str) -> str:
    """Runs the host initialisation of `job_path` in this process and writes its state."""
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if here not in sys.path:
        sys.path.insert(0, here)
    import mithra_gb300 as mg

    s = mg.Setup.from_job(job_path)
    g = s.grid()
    os.makedirs(out_dir, exist_ok=True)
    anp1, an, anm1 = s.fields()
    if anp1.any() or an.any() or anm1.any():
        np.savez(os.path.join(out_dir, "fields.npz"), anp1=anp1, an=an, anm1=anm1)
    elif os.path.exists(os.path.join(out_dir, "fields.npz")):
        os.remove(os.path.join(out_dir, "fields.npz"))
    parts = s.particles()
    tmp = os.path.join(out_dir, "particles.tmp.npy")
    np.save(tmp, parts)
    os.replace(tmp, os.path.join(out_dir, "particles.npy"))
    info = {"format": FORMAT, "job": os.path.abspath(job_path), "job_mtime": os.path.getmtime(job_path),
            "solver": int(g.solver), "order": int(g.truncation_order), "total_time": s.total_time(),
            "n_particles": int(parts.shape[0]), "meta": s.meta()}
    with open(os.path.join(out_dir, "meta.json.tmp"), "w") as f:
        json.dump(info, f)
    os.replace(os.path.join(out_dir, "meta.json.tmp"), os.path.join(out_dir, "meta.json"))
    return out_dir


def current(job_path: str, out_dir: str) -> bool:
    """The directory holds the state of this job file as it is now."""
    try:
        with open(os.path.join(out_dir, "meta.json")) as f:
            info = json.load(f)
    except (OSError, ValueError):
        return False
    return (info.get("format") == FORMAT and info.get("job") == os.path.abspath(job_path)
            and info.get("job_mtime") == os.path.getmtime(job_path)
            and os.path.exists(os.path.join(out_dir, "particles.npy")))


def ensure(job_path: str, out_dir: str) -> str:
    """The state of `job_path` in `out_dir`, computed by a child process when absent or stale, so
    that the calling process does not load the CUDA library."""
    if not current(job_path, out_dir):
        import subprocess
        root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        subprocess.run([sys.executable, "-m", "oracle.initial_state", job_path, out_dir], cwd=root, check=True)
    return out_dir


def load(out_dir: str):
    """(meta dict, anp1, an, anm1, particles, solver, order, total_time)."""
    with open(os.path.join(out_dir, "meta.json")) as f:
        info = json.load(f)
    m = info["meta"]
    nodes = int(m["N0"]) * int(m["N1"]) * int(m["np"])
    fp = os.path.join(out_dir, "fields.npz")
    if os.path.exists(fp):
        z = np.load(fp)
        anp1, an, anm1 = z["anp1"], z["an"], z["anm1"]
    else:
        anp1, an, anm1 = (np.zeros(nodes * 3) for _ in range(3))
    parts = np.load(os.path.join(out_dir, "particles.npy"))
    return m, anp1, an, anm1, parts, info["solver"], info["order"], info["total_time"]


if __name__ == "__main__":
    if len(sys.argv) != 3:
        sys.exit("usage: python -m oracle.initial_state <job file> <output directory>")
    write(sys.argv[1], sys.argv[2])
