"""The parameter-sweep generator: seeded, inside its ranges, and every job parses and initialises."""
import tempfile

from mithra_gb300 import sweep


def test_sweep_parameters_are_seeded_and_in_range():
    a, b = sweep.sweep_parameters(192), sweep.sweep_parameters(192)
    assert a == b and len(a) == 192
    for p in a:
        assert 80 <= p["gamma"] <= 400 and 0.8 <= p["K"] <= 2.0 and 1.5e4 <= p["lambda_u"] <= 3e4
        assert 50 <= p["charge_pc"] <= 500 and 1e-5 <= p["energy_spread"] <= 1e-3
        assert 32 <= p["n_transverse"] <= 96 and 128 <= p["n_longitudinal"] <= 768
        assert 50_000 <= p["particles"] <= 1_000_000


def test_sweep_jobs_initialise():
    ps = sweep.sweep_parameters(192)[:4]
    setups = sweep.make_setups(ps, tempfile.mkdtemp(), threads=4)
    for p, s in zip(ps, setups):
        g = s.grid()
        # NSFD may widen the transverse cells (src/solver.cpp:237-245), never narrow them
        assert g.N2 == p["n_longitudinal"] + 2 and 34 <= g.N0 <= p["n_transverse"] + 2
        assert s.particles().shape[0] >= p["particles"]
