"""Batched instances (one graph launch per step for several contexts) and launch-shape tuning."""
import numpy as np
import pytest

import mithra_gb300 as mg
from tests._golden import BEAM_TAGS, TAGS, load
from tests.conftest import job, rel_l2

pytestmark = pytest.mark.gpu

MARCH_RTOL = 1e-10
ALL = {**TAGS, **BEAM_TAGS}


def test_batch_matches_reference_per_instance(gpu_available):
    """Four different jobs (FD, NSFD, TF/SF seed, external fields) stepped as one batch: each
    instance against the reference's own 12-step run."""
    tags = ["kat-small-fd", "kat-small-nsfd", "kat-small-seed", "kat-small-ext"]
    ctxs = []
    for t in tags:
        c = mg.Context.from_setup(mg.Setup.from_job(job(ALL[t][0])))
        c.run_prelude()
        ctxs.append(c)
    b = mg.Batch(ctxs)
    b.run(5)
    b.run(7)
    for t, c in zip(tags, ctxs):
        run = load(t, "run")
        anp1, an, anm1 = c.download_fields()
        assert rel_l2(an, run["an12"]) <= MARCH_RTOL, t
        assert rel_l2(anm1, run["anm1_12"]) <= MARCH_RTOL, t
        assert c.download_particles().shape == run["particles12"].shape, t
        rows = c.power_rows().reshape(12, -1)
        assert np.abs(rows - run["power"]).max() <= 1e-9 * np.abs(run["power"]).max(), t
    b.close()


def test_batch_mixed_form_matches_individual_runs(gpu_available):
    tags = ["kat-small-fd", "kat-small-optical"]
    single, batched = [], []
    for t in tags:
        s = mg.Setup.from_job(job(ALL[t][0]))
        a = mg.Context.from_setup(s, mg.FP32)
        a.run_prelude()
        a.run(12)
        single.append(a.download_fields()[1])
        c = mg.Context.from_setup(s, mg.FP32)
        c.run_prelude()
        batched.append(c)
    b = mg.Batch(batched)
    b.run(12)
    for t, a_n, c in zip(tags, single, batched):
        assert rel_l2(c.download_fields()[1], a_n) <= 1e-5, t   # FP32 atomics add in any order
    b.close()


def test_batch_refuses_instances_out_of_phase(gpu_available):
    a = mg.Context.from_setup(mg.Setup.from_job(job("kat-small.job")))
    c = mg.Context.from_setup(mg.Setup.from_job(job("kat-small.job")))
    a.run(1)
    with pytest.raises(mg.MithraError):
        mg.Batch([a, c])


def test_autotune_steps_are_part_of_the_march(gpu_available):
    """The FP64 autotuner times 4 shapes x (1 + 2) real steps: 12 steps that must equal the
    reference's 12-step run, whatever shape it keeps."""
    c = mg.Context.from_setup(mg.Setup.from_job(job("kat-small.job")))
    c.run_prelude()
    t, ms = c.autotune(2)
    assert t.blocks_per_sm in (4, 8, 16, 32) and ms > 0
    run = load("kat-small-fd", "run")
    assert rel_l2(c.download_fields()[1], run["an12"]) <= MARCH_RTOL
    assert c.tuning().blocks_per_sm == t.blocks_per_sm


def test_refilled_queue_matches_standalone_runs(gpu_available, tmp_path):
    """sweep.run_queue: six designs through four slots (two refills); every design's power rows
    equal those of its own standalone march to the undulator exit."""
    from mithra_gb300 import surrogate, sweep
    ps = surrogate.design_parameters(6, 11, small=True)
    done, wall, rebuilds = sweep.run_queue(ps, str(tmp_path / "q"), slots=4, min_chunk=12)
    assert sorted(done) == [p["index"] for p in ps] and rebuilds >= 2
    for p in ps[:2] + ps[-1:]:
        path = tmp_path / ("alone-%d.job" % p["index"])
        path.write_text(sweep.job_text(p))
        s = mg.Setup.from_job(str(path), device_init=True)
        c = mg.Context.from_setup(s, mg.FP32)
        c.run_prelude()
        n = sweep.steps_to_exit(s, c)
        c.run(n)
        alone = c.power_rows().reshape(n, -1)
        queued = done[p["index"]].reshape(-1, alone.shape[1])[:n]
        np.testing.assert_allclose(queued, alone, rtol=1e-4, atol=1e-6 * np.abs(alone).max())
        c.close()
