"""Generates the golden vectors under tests/golden/ from the reference itself.

Runs oracle/_ref/ref_harness (the unmodified reference sources built by oracle/Makefile.ref
against the single-rank MPI stand-in) on the small known-answer jobs and stores inputs and
outputs as compressed .npz files.  Run from the repository root in a checkout that has the
reference tree:

    python tests/golden/make_golden.py [REF_SRC] [--only=screen|--only=vtk|--only=ragged]

REF_SRC defaults to $MITHRA_REFERENCE_SRC.

Seeded random inputs (numpy default_rng) make every fixture reproducible.
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, REPO)
from oracle import pyoracle  # noqa: E402

OUT = os.path.join(REPO, "tests", "golden")
JOBS = os.path.join(REPO, "mithra_gb300", "jobs")


def meta_arrays(path):
    m = pyoracle.read_meta(path)
    keys = sorted(m)
    return np.array(keys), np.array([m[k] for k in keys])


def run(harness, *args, cwd):
    subprocess.run([harness] + [str(a) for a in args], check=True, cwd=cwd,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


def bunch_fixture(harness, job, dst, tmp, parts):
    """Solver::bunchSample moments of the step-12 particles of the march."""
    bin_ = os.path.join(tmp, "bunch_in")
    os.makedirs(bin_, exist_ok=True)
    parts.tofile(os.path.join(bin_, "particles.bin"))
    run(harness, "bunch", job, bin_, os.path.join(tmp, "bunch_out"), cwd=tmp)
    np.savez_compressed(os.path.join(dst, "bunch.npz"), particles=parts,
                        moments=np.fromfile(os.path.join(tmp, "bunch_out", "bunch.bin")))


def field_sample_fixture(harness, job, dst, tmp, an, anp1, meta, rng):
    """FdTd::fieldSample at 24 random points inside the interior cells, on random potentials."""
    fin = os.path.join(tmp, "fs_in")
    os.makedirs(fin, exist_ok=True)
    lo = np.array([meta["xmin"] + meta["dx"], meta["ymin"] + meta["dy"], meta["zmin"] + meta["dz"]])
    hi = np.array([meta["xmax"] - meta["dx"], meta["ymax"] - meta["dy"], meta["zmax"] - meta["dz"]])
    pts = lo + (hi - lo) * rng.uniform(0, 1, size=(24, 3))
    an.tofile(os.path.join(fin, "an.bin"))
    anp1.tofile(os.path.join(fin, "anp1.bin"))
    pts.tofile(os.path.join(fin, "points.bin"))
    run(harness, "fieldsample", job, fin, os.path.join(tmp, "fs_out"), cwd=tmp)
    np.savez_compressed(os.path.join(dst, "fieldsample.npz"), an=an, anp1=anp1, points=pts,
                        sample=np.fromfile(os.path.join(tmp, "fs_out", "sample.bin")).reshape(-1, 9))


def screen_fixture(harness, jobname, tag, nsteps=12):
    """Solver::screenProfile through the prelude and nsteps field steps: the screen files the
    reference writes (text as written) and each file's size after the prelude and every step."""
    job = os.path.join(JOBS, jobname)
    dst = os.path.join(OUT, tag)
    os.makedirs(dst, exist_ok=True)
    tmp = tempfile.mkdtemp()
    try:
        run(harness, "screen", job, nsteps, os.path.join(tmp, "screen_out"), cwd=tmp)
        offsets = np.fromfile(os.path.join(tmp, "screen_out", "offsets.bin"))
        files = sorted(f for f in os.listdir(os.path.join(tmp, "screen")) if f.endswith(".txt"))
        offsets = offsets.reshape(nsteps + 1, len(files))
        texts = [open(os.path.join(tmp, "screen", f), "rb").read() for f in files]
        rows, screen, step = [], [], []
        for i, t in enumerate(texts):
            start = 0
            for n in range(nsteps + 1):
                end = int(offsets[n, i])
                for line in t[start:end].decode().splitlines():
                    rows.append([float(x) for x in line.split()])
                    screen.append(i)
                    step.append(n)
                start = end
        pdir = os.path.join(tmp, "bunch-profile")
        pnames = sorted(os.listdir(pdir)) if os.path.isdir(pdir) else []
        ptexts = [open(os.path.join(pdir, f), "rb").read() for f in pnames]
        bfile = os.path.join(tmp, "bunch-sampling", "bunch.txt")
        btext = open(bfile, "rb").read() if os.path.exists(bfile) else b""
        np.savez_compressed(os.path.join(dst, "screen.npz"), names=np.array(files), offsets=offsets,
                            bunch_text=np.frombuffer(btext, dtype=np.uint8),
                            profile_names=np.array(pnames), profile_sizes=np.array([len(t) for t in ptexts]),
                            profile_text=np.frombuffer(b"".join(ptexts), dtype=np.uint8),
                            text=np.frombuffer(b"".join(texts), dtype=np.uint8),
                            text_sizes=np.array([len(t) for t in texts]),
                            rows=np.array(rows).reshape(-1, 6), screen=np.array(screen), step=np.array(step))
    finally:
        shutil.rmtree(tmp)


def vtk_fixture(harness, jobname, tag, nsteps=12):
    """FdTd::fieldVisualize* through nsteps field steps: every .vts/.pvts file the reference
    writes (text as written) and the nTime_ of each step."""
    job = os.path.join(JOBS, jobname)
    dst = os.path.join(OUT, tag)
    os.makedirs(dst, exist_ok=True)
    tmp = tempfile.mkdtemp()
    try:
        run(harness, "vtk", job, nsteps, os.path.join(tmp, "vtk_out"), cwd=tmp)
        files = sorted(os.listdir(os.path.join(tmp, "vtk")))
        texts = [open(os.path.join(tmp, "vtk", f), "rb").read() for f in files]
        # the power files Solver::powerSample writes in the same run
        pfiles = sorted(os.listdir(os.path.join(tmp, "power-sampling")))
        ptexts = [open(os.path.join(tmp, "power-sampling", f), "rb").read() for f in pfiles]
        np.savez_compressed(os.path.join(dst, "vtk.npz"), names=np.array(files),
                            text=np.frombuffer(b"".join(texts), dtype=np.uint8),
                            text_sizes=np.array([len(t) for t in texts]),
                            steps=np.fromfile(os.path.join(tmp, "vtk_out", "steps.bin")),
                            field_sample_text=np.frombuffer(
                                open(os.path.join(tmp, "field-sampling", "field-0.txt"), "rb").read()
                                if os.path.exists(os.path.join(tmp, "field-sampling", "field-0.txt")) else b"",
                                dtype=np.uint8),
                            power_names=np.array(pfiles),
                            power_text=np.frombuffer(b"".join(ptexts), dtype=np.uint8),
                            power_sizes=np.array([len(t) for t in ptexts]))
    finally:
        shutil.rmtree(tmp)


def fixtures_for(harness, jobname, tag, with_kats=True):
    job = os.path.join(JOBS, jobname)
    dst = os.path.join(OUT, tag)
    os.makedirs(dst, exist_ok=True)
    tmp = tempfile.mkdtemp()
    try:
        # Initial state and a 12-step march, dumped at steps 6 and 12.
        run(harness, "run", job, 12, os.path.join(tmp, "run"), 6, cwd=tmp)
        r = os.path.join(tmp, "run")
        ld = lambda s, n: np.fromfile(os.path.join(r, "step%d" % s, n + ".bin"))
        keys, vals = meta_arrays(os.path.join(r, "step0", "meta.txt"))
        sc = os.path.exists(os.path.join(r, "step0", "fn.bin"))
        extra0 = dict(fn=ld(0, "fn"), fnm1=ld(0, "fnm1"), fnp1=ld(0, "fnp1")) if sc else {}
        np.savez_compressed(os.path.join(dst, "init.npz"), meta_keys=keys, meta_vals=vals,
                            particles=ld(0, "particles").reshape(-1, 11), an=ld(0, "an"), anm1=ld(0, "anm1"),
                            anp1=ld(0, "anp1"), **extra0)
        extra = dict(fn12=ld(12, "fn"), fnm1_12=ld(12, "fnm1"), fnp1_12=ld(12, "fnp1")) if sc else {}
        np.savez_compressed(os.path.join(dst, "run.npz"),
                            an6=ld(6, "an"), anp1_6=ld(6, "anp1"), particles6=ld(6, "particles").reshape(-1, 11),
                            an12=ld(12, "an"), anm1_12=ld(12, "anm1"), anp1_12=ld(12, "anp1"),
                            particles12=ld(12, "particles").reshape(-1, 11),
                            power=np.fromfile(os.path.join(r, "power.bin")).reshape(12, -1), **extra)
        if not with_kats:
            return
        meta = pyoracle.read_meta(os.path.join(r, "step0", "meta.txt"))
        nodes = int(meta["N0"]) * int(meta["N1"]) * int(meta["np"])
        rng = np.random.default_rng(20261203)

        # Field update with random potentials and current.
        fin = os.path.join(tmp, "field_in")
        os.makedirs(fin)
        an, anm1, anp1 = (rng.standard_normal(nodes * 3) for _ in range(3))
        an.tofile(os.path.join(fin, "an.bin"))
        anm1.tofile(os.path.join(fin, "anm1.bin"))
        anp1.tofile(os.path.join(fin, "anp1.bin"))
        run(harness, "field", job, fin, os.path.join(tmp, "field_out"), cwd=tmp)
        fo = os.path.join(tmp, "field_out")
        np.savez_compressed(os.path.join(dst, "field.npz"), an=an, anm1=anm1, anp1=anp1,
                            out_anp1=np.fromfile(os.path.join(fo, "anp1.bin")),
                            en=np.fromfile(os.path.join(fo, "en.bin"), dtype=np.float32),
                            bn=np.fromfile(os.path.join(fo, "bn.bin"), dtype=np.float32))

        # One push of the initial bunch with all particles past the entrance, inside the
        # undulator (lz about 10.3 periods), in random radiation fields.
        parts = ld(0, "particles").reshape(-1, 11).copy()
        parts[:, 10] = 1.0
        lu = meta["und0_lu"]
        tb = -meta["dt_shift"] + 10.3 * lu / (meta["gamma"] * meta["beta"] * meta["c0"])
        pin = os.path.join(tmp, "push_in")
        os.makedirs(pin)
        a_n = 1e-3 * rng.standard_normal(nodes * 3)
        a_np1 = a_n + 1e-5 * rng.standard_normal(nodes * 3)
        a_n.tofile(os.path.join(pin, "an.bin"))
        a_np1.tofile(os.path.join(pin, "anp1.bin"))
        parts.tofile(os.path.join(pin, "particles.bin"))
        np.array([tb]).tofile(os.path.join(pin, "timebunch.bin"))
        run(harness, "push", job, pin, os.path.join(tmp, "push_out"), cwd=tmp)
        np.savez_compressed(os.path.join(dst, "push.npz"), an=a_n, anp1=a_np1, particles=parts,
                            time_bunch=np.array([tb]),
                            out=np.fromfile(os.path.join(tmp, "push_out", "particles.bin")).reshape(-1, 11))

        # Deposit of particles that moved by a random sub-cell step.
        dep = ld(0, "particles").reshape(-1, 11).copy()
        dep[:, 4:7] = dep[:, 1:4]
        step = np.array([meta["dx"], meta["dy"], meta["dz"]]) * 0.7
        dep[:, 1:4] += step * rng.uniform(-1, 1, size=(dep.shape[0], 3))
        din = os.path.join(tmp, "dep_in")
        os.makedirs(din)
        dep.tofile(os.path.join(din, "particles.bin"))
        run(harness, "deposit", job, din, os.path.join(tmp, "dep_out"), cwd=tmp)
        np.savez_compressed(os.path.join(dst, "deposit.npz"), particles=dep,
                            J=np.fromfile(os.path.join(tmp, "dep_out", "anp1.bin")))
        bunch_fixture(harness, job, dst, tmp, ld(12, "particles").reshape(-1, 11))
        field_sample_fixture(harness, job, dst, tmp, a_n, a_np1, meta, rng)
    finally:
        shutil.rmtree(tmp)


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--only=")]
    only = [a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--only=")]
    ref_src = args[0] if args else pyoracle.reference_src()
    if not ref_src:
        sys.exit("give the reference's src/ directory as the first argument or in $MITHRA_REFERENCE_SRC")
    harness = pyoracle.build_reference(ref_src)
    if harness is None:
        sys.exit("reference sources not found at %s" % ref_src)
    harness = os.path.abspath(harness)
    if only == ["screen"]:  # the lab-frame screen fixtures alone
        fixtures_for(harness, "kat-small-screen.job", "kat-small-screen", with_kats=False)
        screen_fixture(harness, "kat-small-screen.job", "kat-small-screen")
        print("golden vectors written to", OUT)
        return
    if only == ["ragged"]:  # the ragged-mesh march alone
        fixtures_for(harness, "kat-small-ragged.job", "kat-small-ragged", with_kats=False)
        print("golden vectors written to", OUT)
        return
    if only == ["vtk"]:  # the field visualization fixtures alone
        fixtures_for(harness, "kat-small-vtk.job", "kat-small-vtk", with_kats=False)
        vtk_fixture(harness, "kat-small-vtk.job", "kat-small-vtk")
        print("golden vectors written to", OUT)
        return
    fixtures_for(harness, "kat-small.job", "kat-small-fd")
    fixtures_for(harness, "kat-small-nsfd.job", "kat-small-nsfd")
    fixtures_for(harness, "kat-small-sc.job", "kat-small-sc", with_kats=False)
    fixtures_for(harness, "kat-small-seed.job", "kat-small-seed", with_kats=False)
    fixtures_for(harness, "kat-small-ext.job", "kat-small-ext", with_kats=False)
    fixtures_for(harness, "kat-small-optical.job", "kat-small-optical", with_kats=False)
    fixtures_for(harness, "kat-small-screen.job", "kat-small-screen", with_kats=False)
    screen_fixture(harness, "kat-small-screen.job", "kat-small-screen")
    fixtures_for(harness, "kat-small-vtk.job", "kat-small-vtk", with_kats=False)
    vtk_fixture(harness, "kat-small-vtk.job", "kat-small-vtk")
    fixtures_for(harness, "kat-small-ragged.job", "kat-small-ragged", with_kats=False)
    print("golden vectors written to", OUT)


if __name__ == "__main__":
    main()
