"""Parity of the FP64 CUDA path with the reference (golden vectors) and the C oracle.

Tolerances: the device kernels use FMA contraction and reciprocal multiplies and the deposit
sums with atomics in any order, so single-stage results agree to a few ulp rather than bit for
bit.  Stage tolerances are relative to the largest magnitude of the compared array; the march
gate is the relative L2 norm on the potentials, <= 1e-10, as required for 100 steps."""
import numpy as np
import pytest

import mithra_gb300 as mg
from oracle import pyoracle as po
from tests._golden import BEAM_TAGS, TAGS, load, meta
from tests.conftest import job, rel_l2

pytestmark = pytest.mark.gpu

STAGE_RTOL = 1e-13      # potentials after one field update, relative to max |A|
EB_RTOL = 3e-7          # E/B are stored in float (1-2 float ulp from the reciprocal multiply)
PUSH_RTOL = 1e-12       # particle coordinates and momenta after one push
DEPOSIT_RTOL = 1e-13    # current density, relative L2
MARCH_RTOL = 1e-10      # potentials after a march, relative L2


def ctx_for(tag, precision=mg.FP64):
    s = mg.Setup.from_job(job(TAGS[tag][0]))
    return s, mg.Context.from_setup(s, precision)


def interior_mask(m):
    N0, N1, N2 = int(m["N0"]), int(m["N1"]), int(m["np"])
    sel = np.zeros((N2, N0, N1), dtype=bool)
    sel[:, 1:-1, 1:-1] = True
    return np.repeat(sel.ravel(), 3)


def assert_close_scaled(a, b, rtol, what):
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64)).max() / scale
    assert err <= rtol, "%s: max error %.3e relative to max |ref| (tolerance %.1e)" % (what, err, rtol)


@pytest.mark.parametrize("tag", sorted(TAGS))
def test_field_update_matches_reference(gpu_available, tag):
    f = load(tag, "field")
    _, ctx = ctx_for(tag)
    ctx.upload_fields(f["anp1"], f["an"], f["anm1"])
    ctx.field_update()
    anp1, _, _ = ctx.download_fields()
    assert_close_scaled(anp1, f["out_anp1"], STAGE_RTOL, "A^{n+1}")
    en, bn = ctx.download_eb()
    sel = interior_mask(meta(tag))
    assert_close_scaled(en[sel], f["en"][sel], EB_RTOL, "E")
    assert_close_scaled(bn[sel], f["bn"][sel], EB_RTOL, "B")


def test_push_matches_reference(gpu_available):
    tag = "kat-small-fd"
    p = load(tag, "push")
    _, ctx = ctx_for(tag)
    ctx.upload_fields(p["anp1"], p["an"], None)
    ctx.field_evaluate()
    ctx.upload_particles(p["particles"])
    t = ctx.get_time()
    t.time_bunch = float(p["time_bunch"][0])
    ctx.set_time(t)
    ctx.bunch_update()
    out = ctx.download_particles()
    ref = p["out"]
    assert out.shape == ref.shape
    for col in range(11):
        assert_close_scaled(out[:, col], ref[:, col], PUSH_RTOL, "particle column %d" % col)


def test_deposit_matches_reference(gpu_available):
    tag = "kat-small-fd"
    d = load(tag, "deposit")
    _, ctx = ctx_for(tag)
    ctx.upload_particles(d["particles"])
    ctx.current_update()
    J, _, _ = ctx.download_fields()
    assert rel_l2(J, d["J"]) <= DEPOSIT_RTOL


@pytest.mark.parametrize("tag", sorted(TAGS))
def test_march_matches_reference(gpu_available, tag):
    """12 graph-replayed field steps against the reference's own 12 steps."""
    run = load(tag, "run")
    _, ctx = ctx_for(tag)
    ctx.run_prelude()
    ctx.run(12)
    anp1, an, anm1 = ctx.download_fields()
    assert rel_l2(an, run["an12"]) <= MARCH_RTOL
    assert rel_l2(anm1, run["anm1_12"]) <= MARCH_RTOL
    assert rel_l2(anp1, run["anp1_12"]) <= MARCH_RTOL
    parts = ctx.download_particles()
    ref = run["particles12"]
    assert parts.shape == ref.shape, "particle count incl. z-face copies"
    for col in range(11):
        assert_close_scaled(parts[:, col], ref[:, col], 1e-10, "particle column %d" % col)
    rows = ctx.power_rows().reshape(12, -1)
    assert_close_scaled(rows, run["power"], 1e-9, "power rows")


def test_stagewise_equals_graph_march(gpu_available):
    """The per-stage entry points reproduce what the captured step graph computes."""
    tag = "kat-small-fd"
    _, g = ctx_for(tag)
    g.run(5)
    _, s = ctx_for(tag)
    for _ in range(5):
        s.field_update()
        s.save_positions()
        t, nsub = 0.0, 0
        while t < meta(tag)["nUpdateBunch"]:
            s.bunch_update()
            t += 1.0
        s.recycle()
        s.power_sample()
        s.field_shift()
        s.current_update()
        s.advance_time()
    a, b = g.download_fields(), s.download_fields()
    for x, y in zip(a, b):
        assert rel_l2(x, y) <= 1e-13
    assert np.allclose(g.power_rows(), s.power_rows(), rtol=1e-12, atol=0)
    tg, ts = g.get_time(), s.get_time()
    assert (tg.time, tg.time_bunch, tg.n_time, tg.n_time_bunch) == (ts.time, ts.time_bunch, ts.n_time, ts.n_time_bunch)


def test_config1_100_steps_against_oracle(gpu_available):
    """The plain-form gate: 48x48x384 cells, 237,572 particles, 100 field steps, relative L2 on A
    <= 1e-10 against the CPU oracle started from the same seeded (Halton) bunch."""
    s = mg.Setup.from_job(job("fel-ir-48x48x384.job"))
    m = s.meta()
    anp1, an, anm1 = s.fields()
    o = po.OracleRun(m, an, anm1, anp1, s.particles(), solver=0, order=2)
    po.set_threads(16)
    try:
        for _ in range(100):
            o.step()
    finally:
        po.set_threads(1)
    ctx = mg.Context.from_setup(s)
    ctx.run_prelude()
    ctx.run(100)
    g_anp1, g_an, g_anm1 = ctx.download_fields()
    assert rel_l2(g_an, o.an) <= MARCH_RTOL
    assert rel_l2(g_anm1, o.anm1) <= MARCH_RTOL
    parts = ctx.download_particles()
    assert parts.shape == o.particles.shape
    assert np.abs(parts[:, 1:4] - o.particles[:, 1:4]).max() <= 1e-9 * np.abs(o.particles[:, 1:4]).max()
    rows = ctx.power_rows().reshape(100, -1)
    ref = np.array([np.ravel(np.column_stack([zl, pg.reshape(len(zl), -1)])) for zl, pg in o.power_rows])
    assert_close_scaled(rows, ref, 1e-8, "power rows")


def test_space_charge_march_matches_reference(gpu_available):
    """FdTdSC on the device: A and phi after 12 steps against the reference's own run."""
    run = load("kat-small-sc", "run")
    s = mg.Setup.from_job(job("kat-small-sc.job"))
    ctx = mg.Context.from_setup(s)
    ctx.run_prelude()
    ctx.run(12)
    anp1, an, anm1 = ctx.download_fields()
    fnp1, fn, fnm1 = ctx.download_scalar()
    assert rel_l2(an, run["an12"]) <= MARCH_RTOL
    assert rel_l2(anm1, run["anm1_12"]) <= MARCH_RTOL
    assert rel_l2(fn, run["fn12"]) <= MARCH_RTOL
    assert rel_l2(fnm1, run["fnm1_12"]) <= MARCH_RTOL
    assert rel_l2(fnp1, run["fnp1_12"]) <= MARCH_RTOL
    assert np.abs(run["fn12"]).max() > 0
    rows = ctx.power_rows().reshape(12, -1)
    assert_close_scaled(rows, run["power"], 1e-9, "power rows")


@pytest.mark.parametrize("tag", sorted(BEAM_TAGS))
def test_beam_march_matches_reference(gpu_available, tag):
    """TF/SF seed injection, external laser fields and the optical undulator on the device:
    12 graph-replayed steps against the reference's own run."""
    run = load(tag, "run")
    ctx = mg.Context.from_setup(mg.Setup.from_job(job(BEAM_TAGS[tag][0])))
    ctx.run_prelude()
    ctx.run(12)
    anp1, an, anm1 = ctx.download_fields()
    assert rel_l2(an, run["an12"]) <= MARCH_RTOL
    assert rel_l2(anm1, run["anm1_12"]) <= MARCH_RTOL
    assert rel_l2(anp1, run["anp1_12"]) <= MARCH_RTOL
    parts = ctx.download_particles()
    ref = run["particles12"]
    assert parts.shape == ref.shape
    for col in range(11):
        assert_close_scaled(parts[:, col], ref[:, col], 1e-10, "particle column %d" % col)
    rows = ctx.power_rows().reshape(12, -1)
    assert_close_scaled(rows, run["power"], 1e-9, "power rows")


@pytest.mark.parametrize("tag", sorted(TAGS))
def test_bunch_diagnostics(gpu_available, tag):
    """Device bunch moments against the reference's Solver::bunchSample, and the bunching factor
    against the oracle, on the reference's step-12 particles (compensated device sums agree with
    the reference's ordered sums to rounding)."""
    b, m = load(tag, "bunch"), meta(tag)
    _, ctx = ctx_for(tag)
    ctx.upload_particles(b["particles"])
    row = ctx.bunch_sample()
    np.testing.assert_allclose(row[1:], b["moments"], rtol=1e-12, atol=1e-12 * np.abs(b["moments"]).max())
    k = 2 * np.pi * m["gamma"] / m["und0_lu"]
    ref = po.bunching_factor(m, b["particles"], k)
    assert abs(ctx.bunching_factor(k) - ref) <= 1e-11 * ref


@pytest.mark.parametrize("tag", sorted(TAGS))
def test_field_sample_matches_reference(gpu_available, tag):
    """Device field sampling (E, B, A^n at 24 points) against the reference's FdTd::fieldSample."""
    fs = load(tag, "fieldsample")
    _, ctx = ctx_for(tag)
    ctx.upload_fields(fs["anp1"], fs["an"], None)
    out = ctx.field_sample(fs["points"])
    for c in range(9):
        assert_close_scaled(out[:, c], fs["sample"][:, c], EB_RTOL, "sample column %d" % c)
