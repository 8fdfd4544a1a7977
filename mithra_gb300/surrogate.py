"""MLP surrogate of FEL runs, trained on the device with the library's tensor-core kernels.

The network maps design parameters (gamma, K, lambda_u, periods, charge, sigma_r, energy spread,
seed power) to the radiated power along the undulator, log10 P(z) at 256 points, the final
spectrum, log10 P at the sampled frequencies, and the saturation power.  An ensemble of members is trained on runs of the
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


# ---- FEL designs: data from the full solver, training, screening ------------------------------

FEATURES = ("gamma", "K", "lambda_u", "periods", "charge_pc", "sigma_r", "energy_spread", "seed_power")
N_Z = 256                 # points of log10 P(z) along the undulator
FLOOR = 1e-12             # powers below FLOOR x (largest power of the data) are clipped in log space
PSAT_COLS = 128           # output columns that carry log10 P_sat (its share of the loss)


def resonant_wavelength(p: dict) -> float:
    """Lab-frame FEL wavelength lambda_u (1 + K^2 / 2) / (2 gamma^2), in um."""
    return p["lambda_u"] * (1.0 + 0.5 * p["K"] ** 2) / (2.0 * p["gamma"] ** 2)


def design_parameters(n: int, seed: int, small: bool = False, seeded: bool = False) -> list[dict]:
    """Seeded FEL designs for the surrogate: the sweep family's undulator and bunch ranges
    (gamma 100 .. 250) with the undulator length (periods) and the bunch radius varied as well.
    The mesh follows the radiation as the 48x48x384 FEL job does: 80 resonant wavelengths along
    z at 4.8 cells per wavelength (384 cells), the bunch's rms length 1/6 of that, so every design
    marches about 14 (periods + 2) steps; the solver is NSFD.  The macro-particle count is fixed:
    the power varies by several percent, irregularly, with the number of macro-particles (their
    sampling noise seeds the radiation), which is a numerical parameter and not a design input.
    small=True: 40 wavelengths on 192 cells, a 32x32 transverse mesh, 32768 particles and short
    undulators (fast runs for tests).  seeded=True adds a resonant continuous seed with strength
    parameter a0 drawn log-uniformly in 1e-6 .. 3e-5 (seed_power = a0^2); otherwise the
    radiation starts from the bunch's noise (seed_power = 0)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        p = dict(
            index=i,
            gamma=float(rng.uniform(100.0, 250.0)),
            K=float(rng.uniform(0.8, 2.0)),
            lambda_u=float(rng.uniform(1.5e4, 3.0e4)),
            charge_pc=float(rng.uniform(50.0, 500.0)),
            energy_spread=float(10.0 ** rng.uniform(-5.0, -3.0)),
            sigma_r=float(rng.uniform(150.0, 250.0)),
            seed_power=0.0,
            solver="NSFD",
        )
        if seeded:
            p["seed_a0"] = float(10.0 ** rng.uniform(-6.0, np.log10(3e-5)))
            p["seed_power"] = p["seed_a0"] ** 2
        lam = resonant_wavelength(p)
        if small:
            p.update(periods=int(rng.integers(6, 13)), n_transverse=32, n_longitudinal=192, lz=40.0 * lam,
                     particles=32768)
        else:
            p.update(periods=int(rng.integers(10, 31)), n_transverse=48, n_longitudinal=384, lz=80.0 * lam,
                     particles=131072)
        out.append(p)
    return out


def features(ps: list[dict]) -> np.ndarray:
    return np.array([[p["gamma"] / 100.0, p["K"], p["lambda_u"] / 1e4, p["periods"] / 10.0, np.log10(p["charge_pc"]),
                      p["sigma_r"] / 100.0, np.log10(p["energy_spread"]),
                      np.log10(p["seed_power"]) if p["seed_power"] > 0 else -20.0] for p in ps])


def solve_designs(ps: list[dict], spectrum_points: int, workdir: str, device: int = 0, chunk: int = 256):
    """Runs every design to its undulator exit with the full solver (mixed form, batches of
    `chunk` designs, one graph launch per step).  Designs are grouped by undulator length so that
    the instances of a batch need about the same number of steps.  Returns (curves [n x N_Z] of P
    at the central frequency along the undulator, spectra [n x spectrum_points] at the exit,
    saturation powers, seconds of host setup, seconds of device solves)."""
    import time as _time

    from . import FP32, sweep
    n = len(ps)
    curves = np.zeros((n, N_Z))
    spectra = np.zeros((n, spectrum_points))
    psat = np.zeros(n)
    host = wall = 0.0
    order = sorted(range(n), key=lambda i: (ps[i].get("periods", sweep.PERIODS), ps[i]["lambda_u"]))
    for c0 in range(0, n, chunk):
        part = order[c0:c0 + chunk]
        t0 = _time.perf_counter()
        setups = sweep.make_setups([ps[i] for i in part], workdir, spectrum_points=spectrum_points)
        t1 = _time.perf_counter()
        batch, ctxs, _ = sweep.make_batch(setups, FP32, device)
        steps = [sweep.steps_to_exit(s, c) for s, c in zip(setups, ctxs)]
        batch.run(max(steps))
        t2 = _time.perf_counter()
        host += t1 - t0
        wall += t2 - t1
        for i, s, c, m in zip(part, setups, ctxs, steps):
            # the reference's frequency loop (rw += dl while rw < max) may add one point
            nl = int(s.meta()["rp0_Nl"])
            rows = c.power_rows().reshape(-1, 1 + nl)[:m]
            z, P = rows[:, 0], rows[:, 1:1 + spectrum_points]
            pc = P[:, spectrum_points // 2]
            u = (z - z[0]) / max(z[-1] - z[0], 1e-300)
            curves[i] = np.interp(np.linspace(0.0, 1.0, N_Z), u, pc)
            spectra[i] = P[-1]
            psat[i] = float(pc.max())
            c.close()
        batch.close()
    return curves, spectra, psat, host, wall


def noise_floor(ps: list[dict], n_perturb: int, spectrum_points: int, workdir: str, device: int = 0,
                step: float = 4):
    """The full solver's own repeatability of P_sat: every design solved `n_perturb` times with
    only the macro-particle count changed (the bunch's charge, size and energy, the undulator and
    the mesh unchanged), which changes only the sampling noise that seeds the radiation.  step >= 1:
    the count moves by that many particles per solve (4 = one beamlet group: the quasi-random
    sequence keeps its points and gains one group); step < 1: by that fraction per solve, rounded
    to whole groups (the sequence is then truncated elsewhere, a different sampling of the same
    bunch).  Returns (P_sat [n_designs x n_perturb], the spread per design: relative standard
    deviation and median relative deviation from the design's mean)."""
    runs = []
    for p in ps:
        for j in range(n_perturb):
            q = dict(p)
            if step >= 1:
                q["particles"] = int(p["particles"]) + int(step) * j
            else:
                q["particles"] = 4 * int(round(int(p["particles"]) * (1.0 + step * j) / 4.0))
            q["index"] = len(runs)
            runs.append(q)
    _, _, psat, _, _ = solve_designs(runs, spectrum_points, workdir, device)
    P = psat.reshape(len(ps), n_perturb)
    mean = P.mean(axis=1, keepdims=True)
    rel_sd = P.std(axis=1) / mean[:, 0]
    rel_dev = np.median(np.abs(P - mean) / mean, axis=1)
    return P, rel_sd, rel_dev


ROUGH_INPUTS = ("gamma", "K", "lambda_u", "charge_pc", "sigma_r", "energy_spread")


def roughness(ps: list[dict], deltas, spectrum_points: int, workdir: str, device: int = 0):
    """How far P_sat moves when one design input moves by a small relative step: every design
    solved as drawn and with each input of ROUGH_INPUTS multiplied by (1 + delta), one input at a
    time, for every delta.  A smooth map of the inputs changes P_sat by about its logarithmic
    slope times delta; a change far above that at small delta is the roughness that limits any
    regressor trained on a feasible number of designs.  Returns {delta: |P_sat(moved) / P_sat - 1|
    as an array [n_designs x len(ROUGH_INPUTS)]}."""
    runs = []
    for p in ps:
        runs.append(dict(p))
        for d in deltas:
            for k in ROUGH_INPUTS:
                q = dict(p)
                q[k] = p[k] * (1.0 + d)
                runs.append(q)
    for j, q in enumerate(runs):
        q["index"] = j
    _, _, psat, _, _ = solve_designs(runs, spectrum_points, workdir, device)
    per = 1 + len(deltas) * len(ROUGH_INPUTS)
    P = psat.reshape(len(ps), per)
    out = {}
    for a, d in enumerate(deltas):
        moved = P[:, 1 + a * len(ROUGH_INPUTS):1 + (a + 1) * len(ROUGH_INPUTS)]
        out[d] = np.abs(moved / P[:, :1] - 1.0)
    return out


def to_log(x: np.ndarray, scale: float) -> np.ndarray:
    return np.log10(np.maximum(x, FLOOR * scale))


class FelSurrogate:
    """Ensemble MLP: design features -> [log10 P(z) at N_Z points, log10 spectrum, log10 P_sat].

    The saturation power (the largest sampled P along the undulator) is its own target: the
    sampled P(z) jumps by tens of percent from step to step, so the maximum of a smooth
    predicted curve sits well below the solver's maximum.  It fills PSAT_COLS output columns,
    which gives it that share of the squared-error loss; its prediction is their mean."""

    def __init__(self, n_spectrum: int, hidden: int = 512, layers: int = 4, ensemble: int = 5, seed: int = 1,
                 device: int = 0):
        self.n_spectrum = n_spectrum
        self.net = MLP(len(FEATURES), N_Z + n_spectrum + PSAT_COLS, hidden, layers, ensemble, seed, device)

    def fit(self, X: np.ndarray, curves: np.ndarray, spectra: np.ndarray, psat: np.ndarray, steps: int = 3000,
            batch: int = 128, lr: float = 1e-3, seed: int = 0):
        """Adam with a cosine learning-rate decay over `steps` mini-batches; returns the losses
        [steps x ensemble]."""
        import torch
        self.scale = float(max(curves.max(), spectra.max()))
        T = np.concatenate([to_log(curves, self.scale), to_log(spectra, self.scale),
                            np.repeat(np.log10(np.maximum(psat, FLOOR * self.scale))[:, None], PSAT_COLS, 1)], axis=1)
        self.x_mu, self.x_sd = X.mean(0), X.std(0) + 1e-12
        self.t_mu, self.t_sd = T.mean(0), T.std(0) + 1e-6
        Xn = torch.tensor((X - self.x_mu) / self.x_sd, dtype=torch.float32, device="cuda")
        Tn = torch.tensor((T - self.t_mu) / self.t_sd, dtype=torch.float32, device="cuda")
        rng = np.random.default_rng(seed)
        n = X.shape[0]
        losses = []
        for it in range(steps):
            idx = torch.tensor(rng.choice(n, size=min(batch, n), replace=False), device="cuda")
            lr_t = lr * 0.5 * (1.0 + np.cos(np.pi * it / steps))
            losses.append(self.net.train_step(Xn[idx].contiguous(), Tn[idx].contiguous(), lr_t))
        return np.array(losses)

    def predict(self, X: np.ndarray):
        """Per-member predictions in linear power: curves [E x n x N_Z], spectra
        [E x n x n_spectrum] and saturation powers [E x n]."""
        import torch
        Xn = torch.tensor((X - self.x_mu) / self.x_sd, dtype=torch.float32, device="cuda")
        T = self.net.predict(Xn).cpu().numpy() * self.t_sd + self.t_mu
        ns = N_Z + self.n_spectrum
        return 10.0 ** T[:, :, :N_Z], 10.0 ** T[:, :, N_Z:ns], 10.0 ** T[:, :, ns:].mean(axis=2)


def screen(model: FelSurrogate, X: np.ndarray, threshold: float = 0.05):
    """Ensemble prediction of the saturation power and whether to fall back to the full solver
    (relative ensemble spread above `threshold`)."""
    _, _, ps = model.predict(X)                  # [E x n]
    mean, sd = ps.mean(0), ps.std(0)
    return mean, sd / np.maximum(mean, 1e-300) > threshold


def evaluate(model: FelSurrogate, ps: list[dict], workdir: str, threshold: float = 0.05, device: int = 0):
    """Saturation powers of designs: the ensemble mean where the members agree to `threshold`,
    the full solver's result where they do not.  Returns (P_sat, fallback mask, seconds)."""
    import time as _time
    t0 = _time.perf_counter()
    psat, fb = screen(model, features(ps), threshold)
    psat = psat.copy()
    if fb.any():
        idx = np.flatnonzero(fb)
        _, _, solved, _, _ = solve_designs([ps[i] for i in idx], model.n_spectrum, workdir, device)
        psat[idx] = solved
    return psat, fb, _time.perf_counter() - t0


def gemm_bench(sizes=((512, 512, 512), (4096, 4096, 4096), (8192, 8192, 8192)), reps: int = 10) -> list[dict]:
    """Throughput of mithra_tc_gemm (BF16 in, FP32 out) on random operands, CUDA-event timed on
    the default stream after three warm-up calls, with the largest error against a float64 product."""
    import torch
    out = []
    g = torch.Generator(device="cuda").manual_seed(0)
    for M, N, K in sizes:
        A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
        B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
        C = torch.empty(M, N, device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")

        def call():
            _ck(_lib().mithra_tc_gemm(A.data_ptr(), B.data_ptr(), C.data_ptr(), None, None, M, N, K, 0, None,
                                      err.data_ptr()), "mithra_tc_gemm")
        for _ in range(3):
            call()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            call()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        ref = A.double() @ B.double().T
        rel = float(((C.double() - ref).abs().max() / ref.abs().max()).item())
        out.append(dict(M=M, N=N, K=K, ms=ms, tflops=2.0 * M * N * K / ms / 1e9, max_rel_err=rel,
                        wait_error=int(err.item())))
    return out


def main(argv=None):
    """Dataset from batched solves, ensemble training, and screening of held-out designs against
    the full solver; prints one JSON line with the errors, fallback fractions and speed-up."""
    import argparse
    import json
    import tempfile

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--designs", type=int, default=2304, help="solved designs (training + held-out)")
    ap.add_argument("--held-out", type=int, default=256)
    ap.add_argument("--small", action="store_true", help="32x32x192 meshes, short undulators")
    ap.add_argument("--seeded", action="store_true", help="designs with a resonant seed of varied power")
    ap.add_argument("--spectrum", type=int, default=128, help="frequency points of the spectrum")
    ap.add_argument("--steps", type=int, default=3000, help="Adam steps")
    ap.add_argument("--batch", type=int, default=128, help="mini-batch size")
    ap.add_argument("--lr", type=float, default=1e-3, help="initial Adam learning rate (cosine decay)")
    ap.add_argument("--ensemble", type=int, default=5)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--save", default="", help="npz file for the dataset")
    ap.add_argument("--load", default="", help="npz dataset written by --save (no solves)")
    ap.add_argument("--gemm-bench", action="store_true", help="time mithra_tc_gemm and exit")
    ap.add_argument("--noise-floor", type=int, default=0, metavar="N",
                    help="measure the solver's P_sat repeatability on N designs and exit")
    ap.add_argument("--perturb", type=int, default=8, help="--noise-floor: solves per design")
    ap.add_argument("--perturb-step", type=float, default=4,
                    help="--noise-floor: particles added per solve (>= 1) or fraction of the count (< 1)")
    ap.add_argument("--roughness", type=int, default=0, metavar="N",
                    help="measure how far P_sat moves under small relative input steps on N designs and exit")
    ap.add_argument("--deltas", default="1e-4,1e-3,1e-2", help="--roughness: relative input steps")
    a = ap.parse_args(argv)

    if a.gemm_bench:
        print(json.dumps(gemm_bench()))
        return
    if a.noise_floor:
        ps = design_parameters(a.noise_floor, a.seed, small=a.small, seeded=a.seeded)
        P, sd, dev = noise_floor(ps, a.perturb, a.spectrum, tempfile.mkdtemp(prefix="mithra-floor-"),
                                 step=a.perturb_step)
        print(json.dumps(dict(designs=a.noise_floor, perturb=a.perturb, step=a.perturb_step, small=a.small,
                              seeded=a.seeded,
                              median_rel_sd=float(np.median(sd)), p90_rel_sd=float(np.quantile(sd, 0.9)),
                              median_rel_dev=float(np.median(dev)), p90_rel_dev=float(np.quantile(dev, 0.9)),
                              rel_sd=[float(x) for x in sd], psat=P.tolist())))
        return
    if a.roughness:
        ps = design_parameters(a.roughness, a.seed, small=a.small, seeded=a.seeded)
        deltas = [float(x) for x in a.deltas.split(",")]
        r = roughness(ps, deltas, a.spectrum, tempfile.mkdtemp(prefix="mithra-rough-"))
        print(json.dumps(dict(designs=a.roughness, small=a.small, seeded=a.seeded, inputs=list(ROUGH_INPUTS),
                              steps=[dict(delta=d, median=float(np.median(v)), p90=float(np.quantile(v, 0.9)),
                                          median_per_input={k: float(np.median(v[:, i]))
                                                            for i, k in enumerate(ROUGH_INPUTS)})
                                     for d, v in r.items()])))
        return
    if a.load:
        d = np.load(a.load)
        X, curves, spectra, psat = (d[k].astype(np.float64) for k in ("X", "curves", "spectra", "psat"))
        host_s, dev_s = float(d["host_s"]), float(d["dev_s"])
        a.designs, a.spectrum = X.shape[0], spectra.shape[1]
    else:
        ps = design_parameters(a.designs, a.seed, small=a.small, seeded=a.seeded)
        work = tempfile.mkdtemp(prefix="mithra-surrogate-")
        curves, spectra, psat, host_s, dev_s = solve_designs(ps, a.spectrum, work)
        X = features(ps)
    if a.save:
        np.savez(a.save, X=X.astype(np.float32), curves=curves.astype(np.float32),
                 spectra=spectra.astype(np.float32), psat=psat, host_s=host_s, dev_s=dev_s)
    out = train_and_screen(X, curves, spectra, psat, host_s, dev_s, a.held_out, a.spectrum, steps=a.steps,
                           batch=a.batch, lr=a.lr, ensemble=a.ensemble)
    print(json.dumps(dict(designs=a.designs, held_out=a.held_out, small=a.small, seeded=a.seeded,
                          spectrum=a.spectrum, **out)))


def train_and_screen(X, curves, spectra, psat, host_s: float, dev_s: float, held_out: int, spectrum: int,
                     steps: int = 6000, batch: int = 512, lr: float = 2e-3, ensemble: int = 5,
                     thresholds=(0.02, 0.05, 0.1, 0.2, 0.5)) -> dict:
    """Trains the ensemble on all designs but the last `held_out` and screens those: the held-out
    P_sat error of the ensemble mean and, per spread threshold, the fallback fraction, the error of
    the accepted designs and the speed-up over solving every design (full-solve time per design
    from the dataset's own solves, host setup included)."""
    import time as _time
    n = X.shape[0]
    ntr = n - held_out
    tr, te = slice(0, ntr), slice(ntr, n)
    model = FelSurrogate(spectrum, ensemble=ensemble)
    t0 = _time.perf_counter()
    loss = model.fit(X[tr], curves[tr], spectra[tr], psat[tr], steps=steps, batch=batch, lr=lr)
    train_s = _time.perf_counter() - t0
    t0 = _time.perf_counter()
    reps = 10
    for _ in range(reps):
        mean, _ = screen(model, X[te])
    infer_s = (_time.perf_counter() - t0) / reps / held_out
    err = np.abs(mean - psat[te]) / psat[te]
    geo = 10.0 ** np.mean(np.log10(psat[tr]))
    solve_s = (host_s + dev_s) / n
    rows = []
    for thr in thresholds:
        _, fb = screen(model, X[te], thr)
        acc = ~fb
        f = float(fb.mean())
        rows.append(dict(threshold=thr, fallback=f,
                         accepted_median_err=float(np.median(err[acc])) if acc.any() else None,
                         accepted_p90_err=float(np.quantile(err[acc], 0.9)) if acc.any() else None,
                         speedup=solve_s / (infer_s + f * solve_s)))
    return dict(solve_s_per_design=solve_s, host_s_per_design=host_s / n, device_s_per_design=dev_s / n,
                train_s=train_s, train_steps=steps, final_loss=[float(x) for x in loss[-100:].mean(0)],
                infer_s_per_design=infer_s, median_err=float(np.median(err)), p90_err=float(np.quantile(err, 0.9)),
                baseline_median_err=float(np.median(np.abs(geo - psat[te]) / psat[te])), screening=rows)

if __name__ == "__main__":
    main()
