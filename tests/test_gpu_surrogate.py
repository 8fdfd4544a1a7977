"""Tensor-core GEMM and the device MLP of the surrogate: products against FP32, gradients against
the CPU reference with the same rounding points, and training progress."""
import numpy as np
import pytest

from tests._mlp_reference import bf16, loss_and_grads, unpack

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(gpu_available):
    import torch
    return torch


def test_tc_gemm_matches_fp32(torch_cuda):
    from mithra_gb300 import surrogate
    torch = torch_cuda
    g = torch.Generator(device="cuda").manual_seed(3)
    # K >= 256 runs the pipelined TMA kernel (ring of 4 stages; K = 2048 wraps it 8 times), with
    # 128 x 256 tiles when N is a multiple of 256 and 128 x 128 tiles otherwise
    for M, N, K in ((128, 128, 64), (256, 384, 192), (256, 384, 512), (512, 256, 512), (1024, 512, 2048)):
        A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
        B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
        bias = torch.randn(N, device="cuda", generator=g)
        ref = A.double() @ B.double().T + bias.double()
        out = surrogate.tc_gemm(A, B, bias)
        assert (out.double() - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()
        out = surrogate.tc_gemm(A, B, bias, relu=True)
        assert (out.double() - ref.clamp(min=0)).abs().max().item() <= 1e-5 * ref.abs().max().item()


def test_mlp_gradients_match_cpu_reference(torch_cuda):
    from mithra_gb300 import surrogate
    torch = torch_cuda
    n_in, n_out, hidden, nl = 8, 384, 512, 4
    m = surrogate.MLP(n_in, n_out, hidden, nl, ensemble=2, seed=5)
    rng = np.random.default_rng(11)
    X = rng.standard_normal((200, n_in)).astype(np.float32)
    Y = rng.standard_normal((200, n_out)).astype(np.float32)
    Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    for member in (0, 1):
        g_dev, loss_dev = m.gradients(member, Xd, Yd)
        layers = unpack(m.weights(member), n_in, hidden, nl, n_out)
        loss_ref, g_ref = loss_and_grads(layers, X.astype(np.float64), Y.astype(np.float64))
        assert abs(loss_dev - loss_ref) <= 1e-4 * loss_ref
        err = np.linalg.norm(g_dev - g_ref) / np.linalg.norm(g_ref)
        assert err <= 2e-3, "gradient relative L2 %.3e" % err
    m.close()


def test_mlp_training_reduces_loss(torch_cuda):
    from mithra_gb300 import surrogate
    torch = torch_cuda
    rng = np.random.default_rng(2)
    n_in, n_out = 8, 128
    P = rng.standard_normal((n_in, n_out)) / np.sqrt(n_in)
    X = rng.uniform(-1, 1, (512, n_in))
    Y = np.sin(X @ P)
    Xd = torch.tensor(X, dtype=torch.float32, device="cuda")
    Yd = torch.tensor(Y, dtype=torch.float32, device="cuda")
    m = surrogate.MLP(n_in, n_out, 512, 4, ensemble=3, seed=9)
    first = m.train_step(Xd, Yd, 1e-3)
    for _ in range(300):
        last = m.train_step(Xd, Yd, 1e-3)
    assert (last < 0.05 * first).all(), (first, last)
    pred = m.predict(Xd).cpu().numpy()
    assert pred.shape == (3, 512, n_out)
    assert np.mean((pred.mean(axis=0) - Y) ** 2) < 0.05 * np.mean(Y ** 2)
    m.close()
