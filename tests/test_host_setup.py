"""Host parser + FP64 initialisation against the reference's initial state (golden vectors)."""
import numpy as np
import pytest

import mithra_gb300 as mg
from tests._golden import BEAM_TAGS, LAYOUT_TAGS, TAGS, load, meta
from tests.conftest import job


@pytest.mark.parametrize("tag", sorted(TAGS) + sorted(BEAM_TAGS) + sorted(LAYOUT_TAGS))
def test_setup_matches_reference(tag):
    ref = meta(tag)
    s = mg.Setup.from_job(job({**TAGS, **BEAM_TAGS, **LAYOUT_TAGS}[tag][0]))
    m = s.meta()
    for k, v in ref.items():
        assert k in m, k
        assert m[k] == v, (k, m[k], v)
    assert np.array_equal(s.particles(), load(tag, "init")["particles"])


def test_config1_setup_particle_count():
    s = mg.Setup.from_job(job("fel-ir-48x48x384.job"))
    g = s.grid()
    assert (g.N0, g.N1, g.N2) == (50, 50, 386)
    assert s.particles().shape == (237572, 11)   # 2e5 requested, beamlets of 4 + taper
    assert s.meta()["nUpdateBunch"] > 4.9


def test_parse_errors_are_reported(tmp_path):
    bad = tmp_path / "bad.job"
    bad.write_text("MESH\n{\n  no-such-key = 1\n}\n")
    with pytest.raises(mg.MithraError, match="not defined in solver group"):
        mg.Setup.from_job(str(bad))
    bad.write_text("WRONGGROUP\n{\n}\n")
    with pytest.raises(mg.MithraError, match="is not a defined group"):
        mg.Setup.from_job(str(bad))
    with pytest.raises(mg.MithraError, match="Unable to open file"):
        mg.Setup.from_job(str(tmp_path / "missing.job"))


def test_comment_and_whitespace_rules(tmp_path):
    text = open(job("kat-small.job")).read()
    mangled = "\n".join(("\t" + l.replace(" ", "  ") + "   # trailing comment") if l.strip() and not l.startswith("#")
                        else l for l in text.splitlines())
    p = tmp_path / "m.job"
    p.write_text(mangled)
    a = mg.Setup.from_job(job("kat-small.job")).particles()
    b = mg.Setup.from_job(str(p)).particles()
    assert np.array_equal(a, b)


def test_space_charge_setup_matches_reference():
    z = load("kat-small-sc", "init")
    ref = {str(k): float(v) for k, v in zip(z["meta_keys"], z["meta_vals"])}
    s = mg.Setup.from_job(job("kat-small-sc.job"))
    m = s.meta()
    for k, v in ref.items():
        assert m[k] == v, k
    assert s.grid().space_charge == 1
    assert np.array_equal(s.particles(), z["particles"])


def test_seed_fill_matches_reference():
    """Initial seed fill of A^n and A^{n-1} (src/solver.cpp:828-839) from the host set-up."""
    z = load("kat-small-seed", "init")
    anp1, an, anm1 = mg.Setup.from_job(job("kat-small-seed.job")).fields()
    assert np.abs(z["an"]).max() > 0
    assert np.array_equal(an, z["an"]) and np.array_equal(anm1, z["anm1"])


def test_screen_positions_parsed_and_sorted(tmp_path):
    """bunch-profile-lab-frame (src/datainput.cpp:726-745) and initializeScreenProfile
    (src/solver.cpp:2145-2199): positions sorted, a rhythm adds 0, r, 2r, ... to the undulator end,
    unknown keys and screens without positions are errors with the reference's messages."""
    s = mg.Setup.from_job(job("kat-small-screen.job"))
    assert list(s.screens()) == [-65000.0, -50000.0, -35000.0]
    text = open(job("kat-small-screen.job")).read()
    m = s.meta()
    end = m["und0_rb"] + m["und0_length"] * m["und0_lu"]
    rhythm = text.replace("    position                = -50000.0\n", "    rhythm                  = 400000.0\n")
    p = tmp_path / "r.job"
    p.write_text(rhythm)
    z = list(mg.Setup.from_job(str(p)).screens())
    assert z == sorted([-65000.0, -35000.0] + list(np.arange(0.0, end, 400000.0)))
    p.write_text(text.replace("    position                = -50000.0\n", "    no-such-key             = 1\n"))
    with pytest.raises(mg.MithraError, match="not defined in the bunch-profile-lab-frame group"):
        mg.Setup.from_job(str(p))
    nopos = "\n".join(l for l in text.splitlines() if "position                = -" not in l)
    p.write_text(nopos)
    with pytest.raises(mg.MithraError, match="No position is set for the screen"):
        mg.Setup.from_job(str(p))
