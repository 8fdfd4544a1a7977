"""Field visualization from the device (FdTd.solve writes the reference's .vts/.pvts files at the
steps Solver::solve does) against the reference's own files for the same job."""
import numpy as np
import pytest

import mithra_gb300 as mg
from tests._golden import load
from tests.conftest import job

pytestmark = pytest.mark.gpu


def reference_files():
    z = load("kat-small-vtk", "vtk")
    ref, start = {}, 0
    for name, size in zip(z["names"], z["text_sizes"]):
        ref[str(name)] = bytes(z["text"][start:start + size]).decode()
        start += size
    return ref


def numbers(line):
    out = []
    for tok in line.split():
        try:
            out.append(float(tok))
        except ValueError:
            return None
    return out


@pytest.mark.parametrize("precision,rtol", [(mg.FP64, 1e-9), (mg.FP32, 2e-3)])
def test_solve_writes_reference_vtk(gpu_available, tmp_path, monkeypatch, precision, rtol):
    monkeypatch.chdir(tmp_path)        # the job writes to ./vtk/ like the reference
    setup = mg.Setup.from_job(job("kat-small-vtk.job"))
    mg.FdTd(setup, precision=precision).solve(max_steps=12)
    # the power file written at the end of solve()
    z = load("kat-small-vtk", "vtk")
    pref = bytes(z["power_text"][:int(z["power_sizes"][0])]).decode().splitlines()
    pmine = (tmp_path / "power-sampling" / str(z["power_names"][0])).read_text().splitlines()
    assert len(pmine) == len(pref) and len(pmine[0].split("\t")[0]) == 40
    A = np.array([[float(x) for x in l.split()] for l in pmine])
    B = np.array([[float(x) for x in l.split()] for l in pref])
    assert np.all(np.abs(A - B) <= max(rtol, 1e-9) * 10 * (np.abs(B).max(axis=0) + 1e-300))
    # the field-sampling file (over-line points, lab-frame fields)
    fref = bytes(z["field_sample_text"]).decode().splitlines()
    fmine = (tmp_path / "field-sampling" / "field-0.txt").read_text().splitlines()
    assert len(fmine) == len(fref) > 0
    A = np.array([[float(x) for x in l.split()] for l in fmine])
    B = np.array([[float(x) for x in l.split()] for l in fref])
    assert np.all(np.abs(A - B) <= np.maximum(rtol, 1.01e-4) * (np.abs(B).max(axis=0) + 1e-300))
    ref = reference_files()
    mine = {p.name: p.read_text() for p in (tmp_path / "vtk").iterdir()}
    assert sorted(mine) == sorted(ref)
    for name, text in ref.items():
        a, b = mine[name].splitlines(), text.splitlines()
        assert len(a) == len(b), name
        groups = {}                            # numeric rows by column count: points, values
        for la, lb in zip(a, b):
            na, nb = numbers(la), numbers(lb)
            if nb is None or not nb:
                assert la == lb, (name, la, lb)      # header and tag lines are identical
            else:
                assert na is not None and len(na) == len(nb), (name, la, lb)
                groups.setdefault(len(nb), ([], []))
                groups[len(nb)][0].append(na)
                groups[len(nb)][1].append(nb)
        for rows_a, rows_b in groups.values():
            A, B = np.array(rows_a), np.array(rows_b)
            # coordinates to print precision; field values to the form's accuracy (4 printed
            # decimals: one unit in the last place is 1e-4 of the value)
            scale = np.abs(B).max(axis=0) + 1e-300
            assert np.all(np.abs(A - B) <= np.maximum(rtol, 1.01e-4) * scale), name
