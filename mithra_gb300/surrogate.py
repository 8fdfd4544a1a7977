"""MLP surrogate of FEL runs, trained on the device with the library's tensor-core kernels.

The network maps design parameters (gamma, K, lambda_u, periods, charge, sigma_r, energy spread,
seed power) to the radiated power along the undulator, log10 P(z) at 256 points, and the final
spectrum, log10 P at the sampled frequencies.  An ensemble of members is trained on runs of the
full solver (batched sweeps); a design whose ensemble spread of predicted saturation power
exceeds a threshold is handed back to the full solver.

Device buffers are torch CUDA tensors (plumbing only); every product, activation, loss and Adam
step runs in `libmithra_gb300.so` (`mithra_mlp_*`, `mithra_tc_gemm`).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import MithraError, lib

_vp, _dp = C.c_void_p, C.POINTER(C.c_double)
_SIGS = {
    "mithra_tc_gemm": [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp],
    "mithra_mlp_create": [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.c_int, C.POINTER(_vp)],
    "mithra_mlp_destroy": [_vp],
    "mithra_mlp_train_step": [_vp, _vp, _vp, C.c_int, C.c_float, _dp],
    "mithra_mlp_predict": [_vp, _vp, C.c_int, _vp],
    "mithra_mlp_gradients": [_vp, C.c_int, _vp, _vp, C.c_int, C.POINTER(C.c_float), _dp],
    "mithra_mlp_weights": [_vp, C.c_int, C.POINTER(C.c_float), C.c_int],
    "mithra_mlp_param_count": [_vp],
}
_bound = False


def _lib():
    global _bound
    L = lib()
    if not _bound:
        for name, args in _SIGS.items():
            getattr(L, name).argtypes = args
            getattr(L, name).restype = C.c_longlong if name == "mithra_mlp_param_count" else C.c_int
        _bound = True
    return L


def _ck(r, what):
    if r != 0:
        raise MithraError("%s failed with status %d" % (what, r))


def tc_gemm(A, B, bias=None, relu=False):
    """C = A B^T (+ bias) (ReLU) on the tensor cores; A [M x K], B [N x K] bf16 CUDA tensors."""
    import torch
    M, K = A.shape
    N = B.shape[0]
    out = torch.empty((M, N), dtype=torch.float32, device=A.device)
    err = torch.zeros(1, dtype=torch.int32, device=A.device)
    _ck(_lib().mithra_tc_gemm(A.data_ptr(), B.data_ptr(), out.data_ptr(), None,
                              bias.data_ptr() if bias is not None else None, M, N, K, 1 if relu else 0, None,
                              err.data_ptr()), "mithra_tc_gemm")
    torch.cuda.synchronize()
    if int(err.item()):
        raise MithraError("mithra_tc_gemm: a bounded wait gave up")
    return out


class MLP:
    """Ensemble of ReLU networks n_in -> n_hidden x n_layers -> n_out on one device."""

    def __init__(self, n_in: int, n_out: int, n_hidden: int = 512, n_layers: int = 4, ensemble: int = 5,
                 seed: int = 1, device: int = 0):
        self.n_in, self.n_out, self.ensemble = n_in, n_out, ensemble
        self._h = _vp()
        _ck(_lib().mithra_mlp_create(n_in, n_hidden, n_layers, n_out, ensemble, seed, device, C.byref(self._h)),
            "mithra_mlp_create")

    def close(self):
        if self._h:
            _lib().mithra_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_params(self) -> int:
        return int(_lib().mithra_mlp_param_count(self._h))

    def train_step(self, X, Y, lr: float) -> np.ndarray:
        """One Adam step of every member on the batch (X [B x n_in], Y [B x n_out] FP32 CUDA)."""
        loss = np.zeros(self.ensemble)
        _ck(_lib().mithra_mlp_train_step(self._h, X.data_ptr(), Y.data_ptr(), X.shape[0], float(lr),
                                         loss.ctypes.data_as(_dp)), "mithra_mlp_train_step")
        return loss

    def predict(self, X):
        """Predictions of every member: [ensemble x B x n_out] FP32 CUDA tensor."""
        import torch
        out = torch.empty((self.ensemble, X.shape[0], self.n_out), dtype=torch.float32, device=X.device)
        _ck(_lib().mithra_mlp_predict(self._h, X.data_ptr(), X.shape[0], out.data_ptr()), "mithra_mlp_predict")
        return out

    def gradients(self, member: int, X, Y):
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = np.zeros(1)
        _ck(_lib().mithra_mlp_gradients(self._h, member, X.data_ptr(), Y.data_ptr(), X.shape[0],
                                        g.ctypes.data_as(C.POINTER(C.c_float)), loss.ctypes.data_as(_dp)),
            "mithra_mlp_gradients")
        return g, float(loss[0])

    def weights(self, member: int) -> np.ndarray:
        w = np.zeros(self.n_params, dtype=np.float32)
        _ck(_lib().mithra_mlp_weights(self._h, member, w.ctypes.data_as(C.POINTER(C.c_float)), 0), "weights")
        return w

    def set_weights(self, member: int, w: np.ndarray):
        w = np.ascontiguousarray(w, dtype=np.float32)
        _ck(_lib().mithra_mlp_weights(self._h, member, w.ctypes.data_as(C.POINTER(C.c_float)), 1), "set_weights")
