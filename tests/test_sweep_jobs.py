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


def test_surrogate_family_keeps_one_dft_window_length():
    """The power band of the surrogate's designs keeps the DFT window (Nf = int(3 T / dt) samples,
    T the period of the band's lowest frequency, src/radiation.cpp:88-93) at one length: with the
    family's time step T_1.0 / 9.6 a band starting at 0.9 put 3 T / dt at exactly 32, where
    rounding chose 31 or 32 from design to design; the central frequency stays at 1.0."""
    import numpy as np

    from mithra_gb300 import surrogate
    for small in (False, True):
        ps = surrogate.design_parameters(48, 7, small=small)
        setups = sweep.make_setups(ps, tempfile.mkdtemp(), threads=4, spectrum_points=128)
        metas = [s.meta() for s in setups]
        assert {m["rp0_Nf"] for m in metas} == {32.0}
        for m in metas:
            w1 = 2.0 * np.pi / (9.6 * m["dt"])
            assert abs(m["rp0_w64"] / w1 - 1.0) < 1e-9
