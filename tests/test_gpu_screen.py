"""Lab-frame screens (Solver::screenProfile) and the negative-time prelude on the device, against
the reference's own run of the same job (kat-small shifted back in time by 40 ps, three
screens): the prelude's end state, the 12-step march, and every screen record."""
import numpy as np
import pytest

import mithra_gb300 as mg
from tests._golden import load
from tests.conftest import job, rel_l2

pytestmark = pytest.mark.gpu

TAG, JOB = "kat-small-screen", "kat-small-screen.job"


def golden():
    z = load(TAG, "screen")
    texts, start = [], 0
    for size in z["text_sizes"]:
        texts.append(bytes(z["text"][start:start + size]).decode())
        start += size
    return z, texts


def march(precision):
    s = mg.Setup.from_job(job(JOB))
    ctx = mg.Context.from_setup(s, precision)
    ctx.set_screens(s.screens())
    ctx.run_prelude()
    n0 = ctx.get_time().n_time
    after_prelude = ctx.download_particles()
    ctx.run(12)
    return s, ctx, n0, after_prelude


def per_step(rows, n0, nsteps=12):
    """Golden step index of device rows: 0 = prelude, k = k-th field step."""
    return np.where(rows[:, 6] < n0, 0, rows[:, 6] - n0 + 1).astype(int)


def test_fp64_prelude_march_and_screens_match_reference():
    init, run = load(TAG, "init"), load(TAG, "run")
    z, _ = golden()
    s, ctx, n0, after = march(mg.FP64)
    # the prelude (about six negative-time steps of the bunch alone) ends where the reference's does
    assert after.shape == init["particles"].shape
    scale = np.abs(init["particles"]).max(axis=0) + 1e-300
    assert np.all(np.abs(after - init["particles"]).max(axis=0) <= 1e-12 * scale)
    anp1, an, anm1 = ctx.download_fields()
    assert rel_l2(an, run["an12"]) <= 1e-10
    for i in range(3):
        rows = ctx.screen_records(i)
        ref = z["rows"][z["screen"] == i]
        assert rows.shape[0] == ref.shape[0], "screen %d: %d records, reference %d" % (i, rows.shape[0], ref.shape[0])
        np.testing.assert_array_equal(per_step(rows, n0), z["step"][z["screen"] == i])
        err = np.abs(rows[:, :6] - ref) / (np.abs(ref).max(axis=0) + 1e-300)
        assert err.max() <= 1e-11, "screen %d: max error %.2e" % (i, err.max())
    assert int(np.sum(z["step"][z["screen"] == 0] == 0)) > 0, "the job crosses a screen during the prelude"


def test_screen_files_have_reference_layout(tmp_path):
    z, texts = golden()
    s, ctx, n0, _ = march(mg.FP64)
    names = ctx.write_screen_files(str(tmp_path / "screen" / "scr"))
    assert [n.rsplit("/", 1)[-1] for n in names] == list(z["names"])
    for name, ref in zip(names, texts):
        mine = open(name).read()
        a, b = mine.splitlines(), ref.splitlines()
        assert len(a) == len(b)
        assert len(a[0].split("\t")[0]) == len(b[0].split("\t")[0]) == 40  # one-shot stream width
        va = np.array([[float(x) for x in l.split()] for l in a])
        vb = np.array([[float(x) for x in l.split()] for l in b])
        assert np.all(np.abs(va - vb) <= 1e-11 * (np.abs(vb).max(axis=0) + 1e-300))


def test_fp32_screens_against_reference():
    """Mixed form: crossings decided from FP32 cell offsets, values to FP32 accuracy."""
    z, _ = golden()
    s, ctx, n0, _ = march(mg.FP32)
    for i in range(3):
        rows = ctx.screen_records(i)
        sel = z["screen"] == i
        ref, ref_step = z["rows"][sel], z["step"][sel]
        steps = per_step(rows, n0)
        assert abs(rows.shape[0] - ref.shape[0]) <= max(2, ref.shape[0] // 100)
        for k in range(13):
            a, b = rows[steps == k, :6], ref[ref_step == k]
            if a.shape != b.shape:
                continue  # a particle within FP32 rounding of the screen moved to a neighbouring step
            scale = np.abs(ref).max(axis=0) + 1e-300
            assert np.all(np.abs(a - b) <= 2e-5 * scale), "screen %d step %d" % (i, k)


def test_screens_off_and_capacity():
    s = mg.Setup.from_job(job(JOB))
    ctx = mg.Context.from_setup(s, mg.FP64)
    ctx.set_screens(s.screens(), capacity=4)
    ctx.run_prelude()
    ctx.run(12)
    with pytest.raises(mg.MithraError):
        ctx.screen_records(0)        # more crossings than the 4 records kept
    ctx.set_screens([])              # no screens: the step graphs drop the kernel
    ctx.run(2)
    assert ctx.n_screens == 0


def test_solve_writes_screen_and_bunch_sample_files(tmp_path, monkeypatch):
    """FdTd.solve() writes the screen files (screen/scr-p0-screen<i>.txt) and the bunch-sampling
    file (bunch-sampling/bunch.txt, prelude and field steps) where the reference does."""
    monkeypatch.chdir(tmp_path)
    z, texts = golden()
    mg.FdTd(mg.Setup.from_job(job(JOB))).solve(max_steps=12)
    bref = bytes(z["bunch_text"]).decode().splitlines()
    bmine = (tmp_path / "bunch-sampling" / "bunch.txt").read_text().splitlines()
    assert len(bmine) == len(bref)
    A = np.array([[float(x) for x in l.split()] for l in bmine])
    B = np.array([[float(x) for x in l.split()] for l in bref])
    assert np.all(np.abs(A - B) <= 2e-4 * np.abs(B) + 1e-12 * np.abs(B).max(axis=0))
    # bunch-profile dumps (prelude and field steps): same files, same particles, values to 1e-11
    start = 0
    for name, size in zip(z["profile_names"], z["profile_sizes"]):
        ref = bytes(z["profile_text"][start:start + size]).decode().splitlines()
        start += size
        mine = (tmp_path / "bunch-profile" / str(name)).read_text().splitlines()
        assert len(mine) == len(ref) and len(mine[0]) == 40
        A = np.array([[float(x) for x in l.split()] for l in mine[1:]])
        B = np.array([[float(x) for x in l.split()] for l in ref[1:]])
        assert float(mine[0]) == pytest.approx(float(ref[0]), rel=1e-13)
        assert np.all(np.abs(A - B) <= 1e-11 * (np.abs(B).max(axis=0) + 1e-300))
    for name, ref in zip(z["names"], texts):
        mine = (tmp_path / "screen" / str(name)).read_text().splitlines()
        b = ref.splitlines()
        assert len(mine) == len(b)
        A = np.array([[float(x) for x in l.split()] for l in mine])
        B = np.array([[float(x) for x in l.split()] for l in b])
        assert np.all(np.abs(A - B) <= 1e-11 * (np.abs(B).max(axis=0) + 1e-300))
