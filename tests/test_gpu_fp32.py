"""The mixed-precision form against the FP64 form and the reference's golden vectors.

The mixed form stores fields, currents and particle coordinates in FP32 (particle position as
integer cell + FP32 offset) and keeps FP64 for the undulator phase and the time state.  Its
errors against FP64 are stated per quantity; the bounds below are the ones the tests enforce."""
import numpy as np
import pytest

import mithra_gb300 as mg
from oracle import pyoracle as po
from tests._golden import BEAM_TAGS, TAGS, load, meta
from tests.conftest import job, rel_l2

pytestmark = pytest.mark.gpu

FIELD_STAGE_RTOL = 2e-6   # one field update in FP32, relative to max |A|
PUSH_RTOL = 2e-5          # one push: E = (A^n - A^{n+1})/dt loses digits to cancellation in FP32
DEPOSIT_RTOL = 5e-6       # relative L2 of J
# Full-march bounds against the FP64 form: about ten times the largest errors measured on the
# 48x48x384 job (P_sat 4.1e-5 .. 2.5e-4 over repeated runs, whose atomic order differs; P(z)
# curve 2.3e-4; spectrum 6.5e-5; bunching factor 4.2e-6), so that a regression shows; the
# target itself is 1 % on P_sat.
PSAT_RTOL = 2.5e-3        # saturated (peak) radiated power
CURVE_RTOL = 2.5e-3       # largest P(z) difference / peak power
SPECTRUM_RTOL = 1e-3      # final spectrum, relative L2
BUNCHING_RTOL = 5e-5      # bunching factor at the ponderomotive wavenumber
BEAM_MARCH_RTOL = 2e-4    # A after 12 steps with seed / laser fields, relative L2 vs the reference


def interior_mask(m):
    N0, N1, N2 = int(m["N0"]), int(m["N1"]), int(m["np"])
    sel = np.zeros((N2, N0, N1), dtype=bool)
    sel[:, 1:-1, 1:-1] = True
    return np.repeat(sel.ravel(), 3)


def scaled_err(a, b):
    return float(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64)).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("tag", sorted(TAGS))
def test_fp32_field_update(gpu_available, tag):
    f = load(tag, "field")
    s = mg.Setup.from_job(job(TAGS[tag][0]))
    ctx = mg.Context.from_setup(s, mg.FP32)
    ctx.upload_fields(f["anp1"], f["an"], f["anm1"])
    ctx.field_update()
    anp1, _, _ = ctx.download_fields()
    assert scaled_err(anp1, f["out_anp1"]) <= FIELD_STAGE_RTOL
    en, bn = ctx.download_eb()
    sel = interior_mask(meta(tag))
    assert scaled_err(en[sel], f["en"][sel]) <= 1e-5
    assert scaled_err(bn[sel], f["bn"][sel]) <= 1e-5


def test_fp32_push(gpu_available):
    tag = "kat-small-fd"
    p = load(tag, "push")
    s = mg.Setup.from_job(job(TAGS[tag][0]))
    ctx = mg.Context.from_setup(s, mg.FP32)
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
    for col in (1, 2, 3, 7, 8, 9):
        assert scaled_err(out[:, col], ref[:, col]) <= PUSH_RTOL, col


def test_fp32_deposit(gpu_available):
    tag = "kat-small-fd"
    d = load(tag, "deposit")
    s = mg.Setup.from_job(job(TAGS[tag][0]))
    ctx = mg.Context.from_setup(s, mg.FP32)
    ctx.upload_particles(d["particles"])
    ctx.current_update()
    J, _, _ = ctx.download_fields()
    assert rel_l2(J, d["J"]) <= DEPOSIT_RTOL


def full_march_power(precision, jobname="fel-ir-48x48x384.job"):
    s = mg.Setup.from_job(job(jobname))
    fd = mg.FdTd(s, precision=precision, write_files=False)
    rows = fd.solve()
    return rows.reshape(-1, 2)


@pytest.mark.slow
def test_fp32_saturation_power_within_one_percent(gpu_available):
    """Full march of the 48x48x384 job (to the undulator exit) in both forms."""
    p64 = full_march_power(mg.FP64)
    p32 = full_march_power(mg.FP32)
    assert p64.shape == p32.shape
    P64, P32 = p64[:, 1], p32[:, 1]
    psat64, psat32 = P64.max(), P32.max()
    assert psat64 > 0
    assert abs(psat32 - psat64) / psat64 <= PSAT_RTOL


@pytest.mark.parametrize("tag", sorted(BEAM_TAGS))
def test_fp32_beam_march(gpu_available, tag):
    """Seed, external fields and optical undulator in the mixed form: laser phases in FP64,
    fields in FP32; 12 steps against the reference's FP64 run."""
    run = load(tag, "run")
    ctx = mg.Context.from_setup(mg.Setup.from_job(job(BEAM_TAGS[tag][0])), mg.FP32)
    ctx.run_prelude()
    ctx.run(12)
    anp1, an, anm1 = ctx.download_fields()
    err = rel_l2(an, run["an12"])
    print("%s: FP32 A relative L2 after 12 steps %.3e" % (tag, err))
    assert err <= BEAM_MARCH_RTOL
    assert ctx.download_particles().shape == run["particles12"].shape


def test_fp32_bunch_diagnostics(gpu_available):
    """Moments and bunching factor from the mixed form's cell + FP32 offset positions."""
    tag = "kat-small-fd"
    b, m = load(tag, "bunch"), meta(tag)
    ctx = mg.Context.from_setup(mg.Setup.from_job(job(TAGS[tag][0])), mg.FP32)
    ctx.upload_particles(b["particles"])
    row = ctx.bunch_sample()
    np.testing.assert_allclose(row[1:], b["moments"], rtol=1e-5, atol=1e-6 * np.abs(b["moments"]).max())
    k = 2 * np.pi * m["gamma"] / m["und0_lu"]
    ref = po.bunching_factor(m, b["particles"], k)
    assert abs(ctx.bunching_factor(k) - ref) <= 1e-4 * ref


def test_fp32_error_statement_p_spectrum_bunching(gpu_available):
    """The mixed form against the FP64 form over the full 48x48x384 march (20-point spectrum at
    the power plane): saturated power, the P(z) curve at the resonant frequency, the final
    spectrum and the final bunching factor at the ponderomotive bunch-frame wavenumber."""
    s = mg.Setup.from_job(job("fel-ir-48x48x384-spectrum.job"))
    m = s.meta()
    nl = int(m["rp0_Nl"])
    w = np.array([m["rp0_w%d" % i] for i in range(nl)])
    # ponderomotive bunching in the moving frame: period lambda_u / (2 gamma)
    k = 4 * np.pi * m["gamma"] / m["und0_lu"]
    res = {}
    for prec in (mg.FP64, mg.FP32):
        fd = mg.FdTd(s, precision=prec, write_files=False)
        rows = fd.solve().reshape(-1, 1 + nl)
        res[prec] = (rows[:, 1:], fd.ctx.bunching_factor(k))
        fd.ctx.close()
    (p64, b64), (p32, b32) = res[mg.FP64], res[mg.FP32]
    assert p64.shape == p32.shape and np.isfinite(p32).all()
    ir = int(np.argmin(np.abs(w - w.mean())))   # centre of the 0.9 .. 1.1 sweep
    psat = abs(p32[:, ir].max() - p64[:, ir].max()) / p64[:, ir].max()
    curve = np.abs(p32[:, ir] - p64[:, ir]).max() / np.abs(p64[:, ir]).max()
    spec = np.linalg.norm(p32[-1] - p64[-1]) / np.linalg.norm(p64[-1])
    bunch = abs(b32 - b64) / b64
    print("mixed vs FP64 form: P_sat %.2e, P(z) curve %.2e (max abs diff / max P), final spectrum %.2e "
          "(relative L2), bunching factor %.2e (%.4g vs %.4g)" % (psat, curve, spec, bunch, b32, b64))
    assert psat <= PSAT_RTOL
    assert curve <= CURVE_RTOL and spec <= SPECTRUM_RTOL and bunch <= BUNCHING_RTOL


def test_fp32_space_charge_march(gpu_available):
    """FdTdSC in the mixed form: A and phi after 12 steps against the reference's own FP64 run."""
    run = load("kat-small-sc", "run")
    ctx = mg.Context.from_setup(mg.Setup.from_job(job("kat-small-sc.job")), mg.FP32)
    ctx.run_prelude()
    ctx.run(12)
    _, an, _ = ctx.download_fields()
    _, fn, _ = ctx.download_scalar()
    ea, ef = rel_l2(an, run["an12"]), rel_l2(fn, run["fn12"])
    print("kat-small-sc: FP32 relative L2 after 12 steps: A %.3e, phi %.3e" % (ea, ef))
    assert ea <= BEAM_MARCH_RTOL and ef <= BEAM_MARCH_RTOL
    assert ctx.download_particles().shape == run["particles12"].shape


def test_fp32_particle_rows_follow_the_list_order_across_sorts(gpu_available):
    """Nine field steps (three tile sorts) with z-face copies: the mixed form's download lists the
    particles, copies included, in the FP64 form's (the reference's) list order."""
    s = mg.Setup.from_job(job(TAGS["kat-small-fd"][0]))
    rows = {}
    for prec in (mg.FP64, mg.FP32):
        ctx = mg.Context.from_setup(s, prec)
        ctx.run_prelude()
        ctx.run(9)
        rows[prec] = ctx.download_particles()
    a, b = rows[mg.FP32], rows[mg.FP64]
    assert a.shape == b.shape
    for col in (1, 2, 3):  # positions, relative to their range
        span = b[:, col].max() - b[:, col].min()
        assert np.abs(a[:, col] - b[:, col]).max() <= 1e-3 * span, col
