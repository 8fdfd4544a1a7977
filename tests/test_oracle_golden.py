"""The C oracle against the reference's own outputs (golden vectors from oracle/_ref).

Bit-exact: the oracle restates the reference's arithmetic in the same order and is built with
-ffp-contract=off, so every comparison here is array_equal."""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests._golden import BEAM_TAGS, TAGS, load, meta


@pytest.mark.parametrize("tag", sorted(TAGS))
def test_oracle_march_matches_reference(tag):
    m = meta(tag)
    init, run = load(tag, "init"), load(tag, "run")
    solver = TAGS[tag][1]
    r = po.OracleRun(m, init["an"], init["anm1"], init["anp1"], init["particles"], solver=solver, order=2)
    for step in range(1, 13):
        r.step()
        zl, pg = r.power_rows[-1]
        row = np.ravel(np.column_stack([zl, pg.reshape(len(zl), -1)]))
        assert np.array_equal(row, run["power"][step - 1]), "power row %d" % step
        if step == 6:
            assert np.array_equal(r.an, run["an6"])
            assert np.array_equal(r.anp1, run["anp1_6"])
            assert np.array_equal(r.particles, run["particles6"])
    assert np.array_equal(r.an, run["an12"])
    assert np.array_equal(r.anm1, run["anm1_12"])
    assert np.array_equal(r.anp1, run["anp1_12"])
    assert np.array_equal(r.particles, run["particles12"])


@pytest.mark.parametrize("tag", sorted(TAGS))
def test_oracle_field_update_matches_reference(tag):
    m = meta(tag)
    f = load(tag, "field")
    fp = po.field_params(m, TAGS[tag][1], 2)
    anp1 = f["anp1"].copy()
    po.lib().mo_field_update(po.C.byref(fp), po.dptr(anp1), po.dptr(f["an"].copy()), po.dptr(f["anm1"].copy()))
    assert np.array_equal(anp1, f["out_anp1"])
    nodes = anp1.size // 3
    en = np.zeros(nodes * 3, dtype=np.float32)
    bn = np.zeros(nodes * 3, dtype=np.float32)
    po.lib().mo_eval_eb(po.C.byref(fp), po.dptr(anp1), po.dptr(f["an"].copy()), None, po.fptr(en), po.fptr(bn))
    N0, N1, N2 = int(m["N0"]), int(m["N1"]), int(m["np"])
    sel = np.zeros((N2, N0, N1), dtype=bool)
    sel[:, 1:-1, 1:-1] = True
    sel = np.repeat(sel.ravel(), 3)
    assert np.array_equal(en[sel], f["en"][sel])
    assert np.array_equal(bn[sel], f["bn"][sel])


def test_oracle_push_matches_reference():
    tag = "kat-small-fd"
    m = meta(tag)
    p = load(tag, "push")
    fp = po.field_params(m, 0, 2)
    nodes = p["an"].size // 3
    en = np.zeros(nodes * 3, dtype=np.float32)
    bn = np.zeros(nodes * 3, dtype=np.float32)
    po.lib().mo_eval_eb(po.C.byref(fp), po.dptr(p["anp1"].copy()), po.dptr(p["an"].copy()), None, po.fptr(en), po.fptr(bn))
    rec = np.zeros((p["out"].shape[0] + 16, 11))
    n = p["particles"].shape[0]
    rec[:n] = p["particles"]
    pp = po.push_params(m)
    nt = po.C.c_long(0)
    n2 = po.lib().mo_push_substep(po.C.byref(pp), float(p["time_bunch"][0]), po.dptr(rec), n, rec.shape[0],
                                  po.fptr(en), po.fptr(bn), po.C.byref(nt))
    assert n2 == p["out"].shape[0]
    assert np.array_equal(rec[:n2], p["out"])


def test_oracle_deposit_matches_reference():
    tag = "kat-small-fd"
    m = meta(tag)
    d = load(tag, "deposit")
    dp = po.deposit_params(m)
    J = np.zeros_like(d["J"])
    po.lib().mo_deposit_current(po.C.byref(dp), po.dptr(np.ascontiguousarray(d["particles"])), d["particles"].shape[0],
                                po.dptr(J), None)
    assert np.array_equal(J, d["J"])
    assert np.count_nonzero(J) > 0


def test_oracle_space_charge_march_matches_reference():
    """FdTdSC: scalar potential leapfrog, rho deposit and -grad(phi) in E, 12 steps."""
    tag = "kat-small-sc"
    z = load(tag, "init")
    m = {str(k): float(v) for k, v in zip(z["meta_keys"], z["meta_vals"])}
    run = load(tag, "run")
    r = po.OracleRun(m, z["an"], z["anm1"], z["anp1"], z["particles"], solver=0, order=2,
                     fn=z["fn"], fnm1=z["fnm1"], fnp1=z["fnp1"])
    for step in range(1, 13):
        r.step()
        zl, pg = r.power_rows[-1]
        row = np.ravel(np.column_stack([zl, pg.reshape(len(zl), -1)]))
        assert np.array_equal(row, run["power"][step - 1]), "power row %d" % step
    for a, b in ((r.an, "an12"), (r.anm1, "anm1_12"), (r.anp1, "anp1_12"), (r.fn, "fn12"), (r.fnm1, "fnm1_12"),
                 (r.fnp1, "fnp1_12"), (r.particles, "particles12")):
        assert np.array_equal(a, run[b]), b
    assert np.abs(r.fn).max() > 0


@pytest.mark.parametrize("tag", sorted(BEAM_TAGS))
def test_oracle_beam_march_matches_reference(tag):
    """Seed injection through the TF/SF planes, external laser fields and the optical undulator:
    12 steps against the reference's own run, bit for bit."""
    m = meta(tag)
    init, run = load(tag, "init"), load(tag, "run")
    r = po.OracleRun(m, init["an"], init["anm1"], init["anp1"], init["particles"], solver=BEAM_TAGS[tag][1], order=2)
    for step in range(1, 13):
        r.step()
        zl, pg = r.power_rows[-1]
        row = np.ravel(np.column_stack([zl, pg.reshape(len(zl), -1)]))
        assert np.array_equal(row, run["power"][step - 1]), "power row %d" % step
    for a, b in ((r.an, "an12"), (r.anm1, "anm1_12"), (r.anp1, "anp1_12"), (r.particles, "particles12")):
        assert np.array_equal(a, run[b]), b


def test_oracle_seed_injection_is_active():
    """The seed job's march differs from the same march without the injection."""
    tag = "kat-small-seed"
    m = meta(tag)
    init, run = load(tag, "init"), load(tag, "run")
    r = po.OracleRun(m, init["an"], init["anm1"], init["anp1"], init["particles"], solver=1, order=2)
    r.seed = None
    for _ in range(12):
        r.step()
    assert not np.array_equal(r.an, run["an12"])


@pytest.mark.parametrize("tag", sorted(TAGS))
def test_oracle_bunch_sample_matches_reference(tag):
    """Solver::bunchSample moments of the step-12 particles, bit for bit."""
    b = load(tag, "bunch")
    assert np.array_equal(po.bunch_sample(meta(tag), b["particles"]), b["moments"])


def test_oracle_bunching_factor_formula():
    """The bunching factor restated with numpy (complex sum over the particles in the domain)."""
    tag = "kat-small-fd"
    m, p = meta(tag), load(tag, "bunch")["particles"]
    k = 2 * np.pi * m["gamma"] / m["und0_lu"]
    zr = np.fmod(p[:, 3] - m["zmin"], m["Lz"])
    zr = np.where(zr < 0, zr + m["Lz"], zr) + m["zmin"]
    sel = (zr >= m["zp0"]) & (zr < m["zp1"])
    ref = abs(np.sum(p[sel, 0] * np.exp(1j * k * p[sel, 3]))) / p[sel, 0].sum()
    assert abs(po.bunching_factor(m, p, k) - ref) <= 1e-12 * ref


@pytest.mark.parametrize("tag", sorted(TAGS))
def test_oracle_field_sample_matches_reference(tag):
    """FdTd::fieldSample at 24 points on random potentials, bit for bit."""
    m, fs = meta(tag), load(tag, "fieldsample")
    nodes = fs["an"].size // 3
    en = np.zeros(nodes * 3, dtype=np.float32)
    bn = np.zeros(nodes * 3, dtype=np.float32)
    fp = po.field_params(m, TAGS[tag][1], 2)
    po.lib().mo_eval_eb(po.C.byref(fp), po.dptr(fs["anp1"].copy()), po.dptr(fs["an"].copy()), None, po.fptr(en),
                        po.fptr(bn))
    assert np.array_equal(po.field_sample(m, fs["an"], en, bn, fs["points"], TAGS[tag][1]), fs["sample"])


def _screen_golden():
    z = load("kat-small-screen", "screen")
    texts, start = [], 0
    for size in z["text_sizes"]:
        texts.append(bytes(z["text"][start:start + size]).decode())
        start += size
    return z, texts


def test_oracle_screen_profile_matches_reference():
    """Solver::screenProfile rows of the 12 field steps against the reference's own screen files
    (16 significant digits in the files)."""
    m = meta("kat-small-screen")
    init = load("kat-small-screen", "init")
    z, _ = _screen_golden()
    lz = np.sort([-35000.0, -65000.0, -50000.0])
    r = po.OracleRun(m, init["an"], init["anm1"], init["anp1"], init["particles"], solver=0, order=2)
    r.set_screens(lz)
    for _ in range(12):
        r.step()
    for step in range(1, 13):
        got = r.screen_rows[step - 1]
        for i in range(3):
            g = got[got[:, 7] == i][:, :6]
            ref = z["rows"][(z["step"] == step) & (z["screen"] == i)]
            assert g.shape == ref.shape, (step, i)
            assert np.all(np.abs(g - ref) <= 1e-15 * np.abs(ref) + 1e-300)
    assert sum(len(x) for x in r.screen_rows) == int(np.sum(z["step"] > 0))


def test_screen_file_format_matches_reference():
    """The writer of mithra_gb300 reproduces the reference's screen files byte for byte from the
    oracle's rows (screens without prelude crossings: the whole file; the first screen: the part
    written by the field steps)."""
    import mithra_gb300 as mg
    m = meta("kat-small-screen")
    init = load("kat-small-screen", "init")
    z, texts = _screen_golden()
    r = po.OracleRun(m, init["an"], init["anm1"], init["anp1"], init["particles"], solver=0, order=2)
    r.set_screens(np.sort([-35000.0, -65000.0, -50000.0]))
    for _ in range(12):
        r.step()
    rows = np.concatenate(r.screen_rows)
    for i in range(3):
        mine = rows[rows[:, 7] == i][:, :6]
        prelude = int(z["offsets"][0, i])
        assert mg.format_screen_text(mine, first_in_file=prelude == 0) == texts[i][prelude:]


def test_field_vtk_files_match_reference(tmp_path):
    """The field-visualization writer (all-domain and the three in-plane orientations) reproduces
    the reference's .vts and .pvts files byte for byte from the oracle's E, B and A^n at the
    steps where Solver::solve writes them."""
    import mithra_gb300 as mg
    m = meta("kat-small-vtk")
    init = load("kat-small-vtk", "init")
    z = load("kat-small-vtk", "vtk")
    setup = mg.Setup.from_job(__import__("tests.conftest", fromlist=["job"]).job("kat-small-vtk.job"))
    sm = setup.meta()
    names = [setup.vtk_basename(i).split("/")[-1] for i in range(int(sm["n_vtk"]))]
    r = po.OracleRun(m, init["an"], init["anm1"], init["anp1"], init["particles"], solver=0, order=2)

    def write(run):
        for i, name in enumerate(names):
            if mg.vtk_due(sm, i, run.time):
                mg.write_field_vtk(sm, i, str(tmp_path / name), run.n_time, run.en, run.bn, run.an)

    r.after_recycle = write
    for _ in range(12):
        r.step()
    ref, start = {}, 0
    for name, size in zip(z["names"], z["text_sizes"]):
        ref[str(name)] = bytes(z["text"][start:start + size])
        start += size
    mine = {p.name: p.read_bytes() for p in tmp_path.iterdir()}
    assert sorted(mine) == sorted(ref)
    for name in ref:
        assert mine[name] == ref[name], name


def test_oracle_ragged_mesh_march_matches_reference():
    """10 x 13 transverse nodes centred off axis: 12 steps bit for bit against the reference."""
    from tests._golden import LAYOUT_TAGS
    tag = "kat-small-ragged"
    m = meta(tag)
    init, run = load(tag, "init"), load(tag, "run")
    r = po.OracleRun(m, init["an"], init["anm1"], init["anp1"], init["particles"], solver=LAYOUT_TAGS[tag][1], order=2)
    for step in range(1, 13):
        r.step()
        zl, pg = r.power_rows[-1]
        assert np.array_equal(np.ravel(np.column_stack([zl, pg.reshape(len(zl), -1)])), run["power"][step - 1])
    assert np.array_equal(r.an, run["an12"]) and np.array_equal(r.anm1, run["anm1_12"])
    assert np.array_equal(r.particles, run["particles12"])


def test_power_file_format_matches_reference():
    """The power-file writer reproduces the reference's power-sampling file byte for byte from
    the oracle's power rows (12 steps of kat-small-vtk, one plane, one frequency)."""
    import mithra_gb300 as mg
    m = meta("kat-small-vtk")
    init = load("kat-small-vtk", "init")
    z = load("kat-small-vtk", "vtk")
    r = po.OracleRun(m, init["an"], init["anm1"], init["anp1"], init["particles"], solver=0, order=2)
    for _ in range(12):
        r.step()
    rows = np.array([np.ravel(np.column_stack([zl, pg.reshape(len(zl), -1)])) for zl, pg in r.power_rows])
    N, nl = int(m["rp0_N"]), int(m["rp0_Nl"])
    ref = bytes(z["power_text"][:int(z["power_sizes"][0])]).decode()
    assert mg.format_power_text(rows, N, nl, 0) == ref


def test_bunch_sample_file_matches_reference():
    """Solver::bunchSample lines of the field steps (the last lines of the reference's file; the
    first come from the prelude) byte for byte from the oracle's moments and format_bunch_sample."""
    import mithra_gb300 as mg
    from tests.conftest import job
    m = meta("kat-small-screen")
    sm = mg.Setup.from_job(job("kat-small-screen.job")).meta()
    init = load("kat-small-screen", "init")
    ref = bytes(load("kat-small-screen", "screen")["bunch_text"]).decode().splitlines(keepends=True)
    r = po.OracleRun(m, init["an"], init["anm1"], init["anp1"], init["particles"], solver=0, order=2)
    lines = []

    def sample(run):
        if mg.bunch_sample_due(sm, run.time):
            lines.append(mg.format_bunch_sample(np.concatenate([[run.time_bunch], po.bunch_sample(m, run.particles)])))

    r.after_recycle = sample
    for _ in range(12):
        r.step()
    assert 0 < len(lines) < len(ref)
    assert lines == ref[len(ref) - len(lines):]


def test_field_sample_file_matches_reference():
    """FdTd::fieldSample rows (over-line points, six components, lab transform and units) byte for
    byte from the oracle's E, B, A^n and format_field_sample."""
    import mithra_gb300 as mg
    from tests.conftest import job
    m = meta("kat-small-vtk")
    sm = mg.Setup.from_job(job("kat-small-vtk.job")).meta()
    pts = mg.field_sample_points(sm)
    assert pts.shape == (5, 3)
    init = load("kat-small-vtk", "init")
    ref = bytes(load("kat-small-vtk", "vtk")["field_sample_text"]).decode().splitlines(keepends=True)
    r = po.OracleRun(m, init["an"], init["anm1"], init["anp1"], init["particles"], solver=0, order=2)
    lines = []

    def sample(run):
        if mg.field_sample_due(sm, run.time):
            lines.append(mg.format_field_sample(sm, run.time, pts, po.field_sample(m, run.an, run.en, run.bn, pts)))

    r.after_recycle = sample
    for _ in range(12):
        r.step()
    assert len(lines) == len(ref) > 0
    assert lines == ref


def test_bunch_profile_dumps_match_reference():
    """Solver::bunchProfile dumps written during the field steps (listed time and rhythm) byte for
    byte from the oracle's particles and format_bunch_profile."""
    import mithra_gb300 as mg
    from tests.conftest import job
    m = meta("kat-small-screen")
    sm = mg.Setup.from_job(job("kat-small-screen.job")).meta()
    init = load("kat-small-screen", "init")
    z = load("kat-small-screen", "screen")
    ref, start = {}, 0
    for name, size in zip(z["profile_names"], z["profile_sizes"]):
        ref[str(name)] = bytes(z["profile_text"][start:start + size]).decode()
        start += size
    r = po.OracleRun(m, init["an"], init["anm1"], init["anp1"], init["particles"], solver=0, order=2)
    mine = {}

    def dump(run):
        if mg.bunch_profile_due(sm, run.time):
            mine["prof-p0-%d.txt" % run.n_time] = mg.format_bunch_profile(run.time * m["gamma"], run.particles)

    r.after_recycle = dump
    for _ in range(12):
        r.step()
    assert len(mine) >= 2 and set(mine) <= set(ref)
    for name, text in mine.items():
        assert text == ref[name], name
