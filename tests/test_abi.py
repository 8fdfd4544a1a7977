"""The C-ABI library loads and exports every function that include/*.h declares."""
import glob
import os
import re
import subprocess

import mithra_gb300 as mg

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"^\s*int\s+(mithra_\w+)\s*\(", src, flags=re.M))
    return names


def test_library_exports_every_declared_symbol():
    path = mg.lib_path()
    mg.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(mithra_\w+)", out))
    declared = declared_functions()
    assert declared, "no declarations found"
    missing = declared - exported
    assert not missing, sorted(missing)


def test_setup_entry_points_run_without_gpu():
    s = mg.Setup.from_job(os.path.join(REPO, "mithra_gb300", "jobs", "kat-small.job"))
    g = s.grid()
    assert g.N0 == 10 and g.N2 == 42
    anp1, an, anm1 = s.fields()
    assert anp1.size == 10 * 10 * 42 * 3 and not an.any()
