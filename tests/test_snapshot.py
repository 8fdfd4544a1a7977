"""March-state snapshots on the host: the stream written through a pipe and the directory form
read back exactly (no GPU: the snapshot arrays are made up)."""
import os
import threading

import numpy as np

from mithra_gb300 import snapshot as sn
from tests.conftest import job


class _Grid:
    solver = 0
    truncation_order = 2


class _Setup:
    def grid(self):
        return _Grid()

    def meta(self):
        return {"N0": 4, "N1": 3, "np": 5, "time": -1.0, "timeBunch": -1.0, "nTime": 0, "nTimeBunch": 0}

    def total_time(self):
        return 12.5


def _snap(rng, scalar):
    n = 4 * 3 * 5
    f = tuple(rng.standard_normal(3 * n) for _ in range(3))
    s = tuple(rng.standard_normal(n) for _ in range(3)) if scalar else None
    return sn.Snapshot(f, s, rng.standard_normal((17, 11)), (3.25, 3.5, 13, 26))


def _same(a, b):
    assert a.time == b.time
    for x, y in zip(a.fields, b.fields):
        assert np.array_equal(x, y)
    assert (a.scalar is None) == (b.scalar is None)
    if a.scalar is not None:
        for x, y in zip(a.scalar, b.scalar):
            assert np.array_equal(x, y)
    assert np.array_equal(a.particles, b.particles)


def test_stream_round_trip_through_a_pipe():
    rng = np.random.default_rng(7)
    jf = job("kat-small.job")
    for scalar in (False, True):
        snap = _snap(rng, scalar)
        r, w = os.pipe()

        def writer():
            with os.fdopen(w, "wb") as f:
                sn.write_stream(snap, f, jf, _Setup(), 13)

        t = threading.Thread(target=writer)
        t.start()
        with os.fdopen(r, "rb") as f:
            info, back = sn.read_stream(f)
        t.join()
        _same(snap, back)
        assert info["step"] == 13 and info["total_time"] == 12.5
        # the meta values carry the snapshot's time state, the rest as the job's
        assert (info["meta"]["time"], info["meta"]["timeBunch"], info["meta"]["nTime"],
                info["meta"]["nTimeBunch"]) == (3.25, 3.5, 13, 26)
        assert info["meta"]["N0"] == 4


def test_directory_round_trip(tmp_path):
    rng = np.random.default_rng(8)
    jf = job("kat-small.job")
    snap = _snap(rng, True)
    d = str(tmp_path / "snap")
    sn.save(snap, d, jf, _Setup(), 13)
    assert sn.current(d, jf, 13)
    assert not sn.current(d, jf, 14)
    _same(snap, sn.load(d))
