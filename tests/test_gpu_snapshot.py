"""Checkpoint and resume through the C ABI (mithra_gb300.snapshot).

A march resumed from a snapshot, in a fresh context, continues as the march it was taken from:
in the FP64 form to 1e-10 relative L2 on the potentials after 12 more steps (the deposit's atomic
sums may round in another order), with the same particles; in the mixed form a snapshot taken
again right after a restore holds the same state.  The bunch of the first case is partly inside
the undulator, so the gathers and the undulator field run on both sides of the snapshot."""
import os
import threading

import numpy as np
import pytest

import mithra_gb300 as mg
from mithra_gb300 import snapshot as sn
from tests.conftest import job

pytestmark = pytest.mark.gpu

RESUME_RTOL = 1e-10


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_fp64_resume_continues_the_march(gpu_available):
    s = mg.Setup.from_job(job("fel-ir-48x48x384.job"))
    with mg.Context.from_setup(s, mg.FP64) as a:
        a.run_prelude()
        a.run(450)
        snap = sn.take(a, pinned=True)
        entered = float(np.mean(snap.particles[:, 10] > 0.5))
        a.run(12)
        fa = a.download_fields()
        pa = a.download_particles()
        ta = a.get_time()
    assert 0.0 < entered
    with mg.Context.from_setup(s, mg.FP64) as b:
        sn.restore(b, snap)
        b.run(12)
        fb = b.download_fields()
        pb = b.download_particles()
        tb = b.get_time()
    snap.free()
    assert (ta.time, ta.n_time, ta.n_time_bunch) == (tb.time, tb.n_time, tb.n_time_bunch)
    for x, y in zip(fb, fa):
        assert _rel(x, y) <= RESUME_RTOL
    assert pa.shape == pb.shape
    ka, kb = np.lexsort(pa[:, 1:4].T), np.lexsort(pb[:, 1:4].T)
    assert _rel(pb[kb], pa[ka]) <= RESUME_RTOL


def test_fp32_restore_then_take_is_the_same_state(gpu_available):
    s = mg.Setup.from_job(job("fel-ir-48x48x384.job"))
    with mg.Context.from_setup(s, mg.FP32) as a:
        a.run_prelude()
        a.run(301)  # not a multiple of the sort period
        snap = sn.take(a)
    with mg.Context.from_setup(s, mg.FP32) as b:
        sn.restore(b, snap)
        again = sn.take(b)
        b.run(6)  # the restored (unsorted) particles march and sort
        t = b.get_time()
    assert again.time == snap.time
    for x, y in zip(again.fields, snap.fields):
        assert np.array_equal(x, y)
    ka, kb = np.lexsort(snap.particles[:, 1:4].T), np.lexsort(again.particles[:, 1:4].T)
    assert np.allclose(again.particles[kb], snap.particles[ka], rtol=1e-6, atol=1e-9)
    assert t.n_time == snap.time[2] + 6


def test_snapshot_streams_from_a_child_process(gpu_available, tmp_path):
    """The CLI writes the snapshot through a pipe; the parent reads it without the library."""
    import subprocess
    import sys
    jf = job("fel-ir-48x48x384.job")
    r, w = os.pipe()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    p = subprocess.Popen([sys.executable, "-m", "mithra_gb300.snapshot", jf, "--fd", str(w), "--step", "40"],
                         cwd=root, pass_fds=(w,))
    os.close(w)
    with os.fdopen(r, "rb") as f:
        info, snap = sn.read_stream(f)
    assert p.wait() == 0
    assert info["step"] == 40 and info["meta"]["nTime"] == snap.time[2]
    # the same march in this process reaches the same state
    s = mg.Setup.from_job(jf)
    with mg.Context.from_setup(s, mg.FP64) as c:
        c.run_prelude()
        c.run(40)
        mine = sn.take(c)
    assert mine.time == snap.time
    for x, y in zip(snap.fields, mine.fields):
        assert _rel(x, y) <= RESUME_RTOL
