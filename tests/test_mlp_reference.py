"""The CPU MLP reference that checks the device gradients: its backward pass against central
finite differences (float64, no rounding)."""
import numpy as np

from tests import _mlp_reference as R


def test_reference_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    n_in, h, nl, n_out = 3, 5, 2, 4
    dims = [n_in] + [h] * nl + [n_out]
    flat = np.concatenate([np.concatenate([rng.standard_normal(dims[l + 1] * dims[l]) * 0.5,
                                           rng.standard_normal(dims[l + 1]) * 0.1]) for l in range(nl + 1)])
    X, Y = rng.standard_normal((7, n_in)), rng.standard_normal((7, n_out))
    loss = lambda f: R.loss_and_grads(R.unpack(f, n_in, h, nl, n_out), X, Y, exact=True)[0]
    g = R.loss_and_grads(R.unpack(flat, n_in, h, nl, n_out), X, Y, exact=True)[1]
    eps, eye = 1e-6, np.eye(flat.size)
    fd = np.array([(loss(flat + eps * eye[i]) - loss(flat - eps * eye[i])) / (2 * eps) for i in range(flat.size)])
    assert np.linalg.norm(fd - g) / np.linalg.norm(g) < 1e-7


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e38], dtype=np.float32)
    r = R.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and r[3] == -2.5
