"""The FEL surrogate end to end on small designs: batched solves give finite, positive P(z),
the trained ensemble beats the trivial predictor on held-out designs, and the screened
evaluation returns the full solver's result for every design it hands back."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fel_data(gpu_available, tmp_path_factory):
    from mithra_gb300 import surrogate as S
    ps = S.design_parameters(448, 3, small=True)
    curves, spectra, psat, host_s, dev_s = S.solve_designs(ps, 16, str(tmp_path_factory.mktemp("fel")))
    return S, ps, curves, spectra, psat


def test_batched_solves_give_finite_growing_power(fel_data):
    S, ps, curves, spectra, psat = fel_data
    assert np.isfinite(curves).all() and np.isfinite(spectra).all()
    assert (psat > 0).all()
    # the power grows along the undulator: the last quarter is above the first quarter
    q = curves.shape[1] // 4
    assert np.median(curves[:, -q:].mean(1) / np.maximum(curves[:, :q].mean(1), 1e-300)) > 10.0


def test_ensemble_beats_trivial_predictor_and_falls_back(fel_data, tmp_path):
    S, ps, curves, spectra, psat = fel_data
    X = S.features(ps)
    ntr = 384
    model = S.FelSurrogate(16, ensemble=3, seed=2)
    loss = model.fit(X[:ntr], curves[:ntr], spectra[:ntr], psat[:ntr], steps=1500)
    assert np.all(loss[-50:].mean(0) < 0.2 * loss[:10].mean(0))
    held = ps[ntr:]
    mean, fb = S.screen(model, X[ntr:], threshold=1e9)
    assert not fb.any()
    err = np.abs(mean - psat[ntr:]) / psat[ntr:]
    geo = 10.0 ** np.mean(np.log10(psat[:ntr]))
    base = np.abs(geo - psat[ntr:]) / psat[ntr:]
    assert np.median(err) < 0.5 * np.median(base)
    # threshold 0: every design goes back to the solver, whose answer is returned
    out, fb, _ = S.evaluate(model, held[:8], str(tmp_path), threshold=0.0)
    assert fb.all()
    np.testing.assert_allclose(out, psat[ntr:ntr + 8], rtol=2e-3)
