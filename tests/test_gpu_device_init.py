"""Device initialisation of ellipsoid bunches (Halton generation, boost, back-propagation,
distribution, time shift on the GPU) against the host initialisation, which is bit-identical to
the reference: same particles in the same order; values equal except where the device's
log/sin/cos round differently from the host C library (a few units in the last place)."""
import time

import numpy as np
import pytest

import mithra_gb300 as mg
from tests.conftest import job, rel_l2

pytestmark = pytest.mark.gpu

JOBS = ["kat-small.job", "kat-small-screen.job", "kat-small-nsfd.job", "fel-ir-48x48x384.job"]


@pytest.mark.parametrize("name", JOBS)
def test_device_init_matches_host(gpu_available, name):
    host = mg.Setup.from_job(job(name))
    dev = mg.Setup.from_job(job(name), device_init=True)
    a, b = host.particles(), dev.particles()
    assert a.shape == b.shape, "particle count"
    scale = np.abs(a).max(axis=0) + 1e-300
    err = (np.abs(a - b) / scale).max()
    assert err <= 1e-13, "max column-relative difference %.2e" % err
    ma, mb = host.meta(), dev.meta()
    for k in ("dt_shift", "timeBunch", "time", "totalTime", "n_particles"):
        assert mb[k] == pytest.approx(ma[k], rel=1e-14, abs=1e-300), k


def test_device_init_context_marches_like_host(gpu_available):
    """A context created from the device records marches like one created from the host's."""
    runs = []
    for device_init in (False, True):
        s = mg.Setup.from_job(job("kat-small-screen.job"), device_init=device_init)
        ctx = mg.Context.from_setup(s, mg.FP64)
        ctx.run_prelude()
        ctx.run(12)
        runs.append(ctx.download_fields()[1])
    assert rel_l2(runs[1], runs[0]) <= 1e-9


def test_device_init_is_faster_on_the_large_bunch(gpu_available):
    """8.1 M particles (128x128x2048 job): host and device initialisation times (printed)."""
    t0 = time.perf_counter()
    mg.Setup.from_job(job("fel-130x130x2050.job"), device_init=True)
    t1 = time.perf_counter()
    mg.Setup.from_job(job("fel-130x130x2050.job"))
    t2 = time.perf_counter()
    print("setup of the 128x128x2048 job: device initialisation %.3f s, host %.3f s" % (t1 - t0, t2 - t1))
    assert t1 - t0 < t2 - t1


def test_device_init_refuses_other_bunch_types(gpu_available, tmp_path):
    text = open(job("kat-small.job")).read().replace("type                    = ellipsoid", "type                    = 3D-crystal")
    p = tmp_path / "c.job"
    p.write_text(text)
    with pytest.raises(mg.MithraError, match="ellipsoid"):
        mg.Setup.from_job(str(p), device_init=True)
