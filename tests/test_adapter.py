"""The reference-side adapter (mithra_gb300/adapter/gpu_fdtd.cpp) builds, from the reference's own
initialised Solver, the same descriptors as the library's host set-up, bit for bit.

The adapter is compiled against the reference's headers and linked with the reference's objects
(oracle/Makefile.ref, target `adapter`); the test program oracle/adapter_check.cpp parses each job as
the reference's main does, runs Solver::initialize through the adapter's solver class and writes
what describe_for_gpu() returns, stopping before any device call.  Skipped where the reference
tree is absent."""
import ctypes as C
import os
import struct
import subprocess

import numpy as np
import pytest

import mithra_gb300 as mg
from tests.conftest import JOBS, REPO

JOBS_CHECKED = ["kat-small.job", "kat-small-nsfd.job", "kat-small-sc.job", "kat-small-seed.job",
                "kat-small-ext.job", "kat-small-optical.job", "kat-small-ragged.job", "kat-small-screen.job",
                "kat-small-vtk.job", "fel-ir-48x48x384.job", "fel-ir-48x48x384-spectrum.job"]
CHECK = os.path.join(REPO, "oracle", "_ref", "adapter_check")


@pytest.fixture(scope="module")
def adapter_check():
    mg.lib()  # the library the test program links against
    cmd = ["make", "-s", "-f", os.path.join(REPO, "oracle", "Makefile.ref"), "adapter", "-j8"]
    ref = os.environ.get("MITHRA_REFERENCE_SRC")
    if ref:
        cmd.append("REF_SRC=" + ref)
    subprocess.run(cmd, cwd=REPO, check=True, capture_output=True)
    if not os.path.exists(CHECK):
        pytest.skip("reference tree absent: the adapter cannot be compiled here")
    return CHECK


def same_bits(a, b, where):
    if isinstance(a, C.Structure):
        for name, _ in a._fields_:
            same_bits(getattr(a, name), getattr(b, name), where + "." + name)
    elif isinstance(a, C.Array):
        for i in range(len(a)):
            same_bits(a[i], b[i], "%s[%d]" % (where, i))
    elif isinstance(a, float):
        assert struct.pack("<d", a) == struct.pack("<d", b), "%s: %r != %r" % (where, a, b)
    else:
        assert a == b, "%s: %r != %r" % (where, a, b)


def read_struct(path, typ):
    return typ.from_buffer_copy(open(path, "rb").read())


def read_array(path, typ):
    raw = open(path, "rb").read()
    n = len(raw) // C.sizeof(typ)
    return [typ.from_buffer_copy(raw, i * C.sizeof(typ)) for i in range(n)]


@pytest.mark.parametrize("jobname", JOBS_CHECKED)
def test_adapter_descriptors_equal_library_setup(adapter_check, jobname, tmp_path):
    job = os.path.join(JOBS, jobname)
    out = tmp_path / "desc"
    out.mkdir()
    r = subprocess.run([adapter_check, job, str(out)], cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    s = mg.Setup.from_job(job)
    same_bits(read_struct(out / "grid.bin", mg.GridDesc), s.grid(), "grid")
    same_bits(read_struct(out / "push.bin", mg.PushDesc), s.push(), "push")
    same_bits(read_struct(out / "seed.bin", mg.SeedDesc), s.seed(), "seed")
    same_bits(read_struct(out / "time.bin", mg.TimeState), s.time(), "time")
    und, ref_und = read_array(out / "undulators.bin", mg.UndulatorDesc), s.undulators()
    assert len(und) == len(ref_und)
    for i, (a, b) in enumerate(zip(und, ref_und)):
        if a.type == 0:  # a static undulator's laser-beam members are not used: compare the rest
            for name in ("type", "k", "lu", "rb", "length", "dist", "theta"):
                same_bits(getattr(a, name), getattr(b, name), "undulator%d.%s" % (i, name))
        else:
            same_bits(a, b, "undulator%d" % i)
    ext, ref_ext = read_array(out / "ext.bin", mg.BeamDesc), s.external_fields()
    assert len(ext) == len(ref_ext)
    for i, (a, b) in enumerate(zip(ext, ref_ext)):
        same_bits(a, b, "ext%d" % i)
    total, n_particles, n_power = open(out / "scalars.txt").read().split()
    assert float(total) == s.total_time()
    assert int(n_particles) == s.particles().shape[0]
    outputs = s.power_outputs()
    assert int(n_power) == len(outputs)
    for o, p in enumerate(outputs):
        raw = open(out / ("power%d.bin" % o), "rb").read()
        N, Nl, Nf = struct.unpack_from("<3i", raw, 0)
        pc = struct.unpack_from("<d", raw, 12)[0]
        arr = np.frombuffer(raw, dtype="<f8", offset=20)
        assert (N, Nl, Nf) == (p["N"], p["Nl"], p["Nf"])
        same_bits(pc, p["pc"], "power%d.pc" % o)
        k = Nl * Nf
        for name, got in (("z", arr[:N]), ("re", arr[N:N + k]), ("im", arr[N + k:N + 2 * k])):
            assert got.tobytes() == p[name].tobytes(), "power%d.%s" % (o, name)
