"""Python binding of the C oracle (oracle/mithra_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU-baseline
legs of bench.py, never by the product package.

The state layout is the reference's: vector fields are (N1N0*np, 3) float64 arrays in node
order m = N1N0*k + N1*i + j, particles are (n, 11) float64 records
q, rnp[3], rnm[3], gb[3], e.  `OracleRun.step()` performs one field step in the order of
Solver::solve (src/solver.cpp:1300-1399).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "libmithra_oracle.so")
MO_MAX_UND = 64
_lock = threading.Lock()


def build_oracle(force: bool = False) -> str:
    """Compile the C restatement into oracle/_build/libmithra_oracle.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "mithra_oracle.c")
    hdr = os.path.join(HERE, "mithra_oracle.h")
    with _lock:
        if (not force and os.path.exists(LIB_PATH)
                and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
            return LIB_PATH
        os.makedirs(BUILD, exist_ok=True)
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", src, "-o", tmp, "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def reference_src() -> str | None:
    """The reference's src/ directory: $MITHRA_REFERENCE_SRC, or None when it is not set."""
    return os.environ.get("MITHRA_REFERENCE_SRC") or None


def build_reference(ref_src: str | None = None, jobs: int = 8) -> str | None:
    """Build oracle/_ref/ref_harness from the reference sources (`ref_src`, else
    $MITHRA_REFERENCE_SRC, else the default of oracle/Makefile.ref) when they are present;
    returns its path, or None when no reference tree was found."""
    ref_src = ref_src or reference_src()
    if ref_src and not os.path.isdir(ref_src):
        return None
    repo = os.path.dirname(HERE)
    # without REF_SRC the recipe's own default applies (and it builds nothing where that is absent)
    cmd = ["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"), "-j%d" % jobs]
    if ref_src:
        cmd.append("REF_SRC=" + ref_src)
    subprocess.run(cmd, cwd=repo, check=True)
    harness = os.path.join(HERE, "_ref", "ref_harness")
    return harness if os.path.exists(harness) else None


MO_MAX_EXT = 16


class MoSignal(C.Structure):
    _fields_ = [("type", C.c_int), ("t0", C.c_double), ("s", C.c_double), ("f0", C.c_double),
                ("cep", C.c_double), ("nR", C.c_double), ("sig0", C.c_double), ("sig1", C.c_double)]


class MoBeam(C.Structure):
    _fields_ = [("type", C.c_int), ("position", C.c_double * 3), ("direction", C.c_double * 3),
                ("polarization", C.c_double * 3), ("amplitude", C.c_double), ("radius", C.c_double * 2),
                ("order", C.c_int * 2), ("l", C.c_double), ("zR", C.c_double * 2), ("signal", MoSignal)]


class MoSeed(C.Structure):
    _fields_ = [("beam", MoBeam), ("gamma", C.c_double), ("beta", C.c_double), ("c0", C.c_double),
                ("dt", C.c_double)]


class MoField(C.Structure):
    _fields_ = [("N0", C.c_int), ("N1", C.c_int), ("np", C.c_int), ("k0", C.c_int),
                ("solver", C.c_int), ("order", C.c_int), ("space_charge", C.c_int),
                ("a", C.c_double * 6), ("nsfd_alpha", C.c_double), ("nsfd_beta", C.c_double),
                ("bB", C.c_double * 5), ("cB", C.c_double * 5), ("dB", C.c_double * 5),
                ("eE", C.c_double * 5), ("fE", C.c_double * 5), ("gE", C.c_double * 5),
                ("hC", C.c_double * 17),
                ("dt", C.c_double), ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("xmin", C.c_double), ("ymin", C.c_double), ("zmin", C.c_double)]


class MoUndulator(C.Structure):
    _fields_ = [("type", C.c_int), ("k", C.c_double), ("lu", C.c_double), ("rb", C.c_double),
                ("length", C.c_double), ("dist", C.c_double), ("theta", C.c_double), ("beam", MoBeam)]


class MoPush(C.Structure):
    _fields_ = [("N0", C.c_int), ("N1", C.c_int), ("np", C.c_int), ("k0", C.c_int),
                ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double), ("ymax", C.c_double),
                ("zmin", C.c_double), ("zmax", C.c_double), ("zp0", C.c_double), ("zp1", C.c_double),
                ("Lz", C.c_double), ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("dtb", C.c_double), ("r1", C.c_double), ("r2", C.c_double),
                ("gamma", C.c_double), ("beta", C.c_double), ("c0", C.c_double), ("dt_shift", C.c_double),
                ("n_und", C.c_int), ("und", MoUndulator * MO_MAX_UND),
                ("n_ext", C.c_int), ("ext", MoBeam * MO_MAX_EXT)]


class MoDeposit(C.Structure):
    _fields_ = [("N0", C.c_int), ("N1", C.c_int), ("np", C.c_int), ("k0", C.c_int),
                ("xmin", C.c_double), ("ymin", C.c_double), ("zmin", C.c_double),
                ("xmax", C.c_double), ("ymax", C.c_double),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("dv", C.c_double), ("rc", C.c_double),
                ("zp0", C.c_double), ("zp1", C.c_double), ("Lz", C.c_double)]


class MoPower(C.Structure):
    _fields_ = [("N0", C.c_int), ("N1", C.c_int), ("np", C.c_int), ("k0", C.c_int),
                ("N", C.c_int), ("Nl", C.c_int), ("Nf", C.c_int),
                ("zmin", C.c_double), ("dz", C.c_double), ("zp0", C.c_double), ("zp1", C.c_double),
                ("gamma", C.c_double), ("beta", C.c_double), ("c0", C.c_double), ("pc", C.c_double),
                ("z", C.POINTER(C.c_double)), ("ep_re", C.POINTER(C.c_double)),
                ("ep_im", C.POINTER(C.c_double)), ("fdt", C.POINTER(C.c_double))]


class MoScreen(C.Structure):
    _fields_ = [("gamma", C.c_double), ("beta", C.c_double), ("c0", C.c_double), ("dt_shift", C.c_double),
                ("dt", C.c_double), ("zmin", C.c_double), ("Lz", C.c_double), ("zp0", C.c_double),
                ("zp1", C.c_double)]


def screen_params(m: dict) -> MoScreen:
    return MoScreen(m["gamma"], m["beta"], m["c0"], m["dt_shift"], m["dt"], m["zmin"], m["Lz"], m["zp0"], m["zp1"])


def screen_profile(m: dict, lz_screens, time_bunch: float, rec) -> np.ndarray:
    """Solver::screenProfile rows (x, y, t, gbx, gby, gbz_lab, list index) of one step, screens
    in the given order, particles in list order."""
    rec = np.ascontiguousarray(rec, dtype=np.float64)
    lz = np.ascontiguousarray(lz_screens, dtype=np.float64)
    sp = screen_params(m)
    n = lib().mo_screen_profile(C.byref(sp), dptr(lz), len(lz), float(time_bunch), dptr(rec), rec.shape[0], None, 0)
    out = np.zeros((max(n, 1), 7))
    lib().mo_screen_profile(C.byref(sp), dptr(lz), len(lz), float(time_bunch), dptr(rec), rec.shape[0], dptr(out), n)
    return out[:n]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_oracle())
        P = C.POINTER
        d, f, l = P(C.c_double), P(C.c_float), C.c_long
        _lib.mo_field_update.argtypes = [P(MoField), d, d, d]
        _lib.mo_field_update_seeded.argtypes = [P(MoField), P(MoSeed), C.c_double, d, d, d]
        _lib.mo_seed_fields.argtypes = [P(MoSeed), d, C.c_double, d]
        _lib.mo_scalar_update.argtypes = [P(MoField), d, d, d]
        _lib.mo_eval_eb.argtypes = [P(MoField), d, d, d, f, f]
        _lib.mo_push_substep.argtypes = [P(MoPush), C.c_double, d, l, l, f, f, P(C.c_long)]
        _lib.mo_push_substep.restype = l
        _lib.mo_deposit_current.argtypes = [P(MoDeposit), d, l, d, d]
        _lib.mo_erase_outside.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, d, l]
        _lib.mo_erase_outside.restype = l
        _lib.mo_power_sample.argtypes = [P(MoPower), C.c_uint, f, f, d]
        _lib.mo_set_threads.argtypes = [C.c_int]
        dd = C.c_double
        _lib.mo_bunch_sample.argtypes = [dd, dd, dd, dd, d, l, d]
        _lib.mo_field_sample.argtypes = [P(MoField), d, f, f, d, l, d]
        _lib.mo_bunching_factor.argtypes = [dd, dd, dd, dd, d, l, dd]
        _lib.mo_bunching_factor.restype = dd
        _lib.mo_screen_profile.argtypes = [P(MoScreen), d, C.c_int, dd, d, l, d, l]
        _lib.mo_screen_profile.restype = l
    return _lib


def set_threads(n: int) -> None:
    lib().mo_set_threads(int(n))


def dptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def fptr(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_float))


def read_meta(path: str) -> dict:
    out = {}
    with open(path) as fh:
        for line in fh:
            k, v = line.split()
            out[k] = float(v)
    return out


def beam_params(m: dict, prefix: str, out: MoBeam) -> MoBeam:
    """A laser beam (seed, optical undulator or external field) from the meta keys `prefix*`."""
    g = lambda k: m.get(prefix + k, 0.0)
    out.type = int(g("type"))
    for c in range(3):
        out.position[c], out.direction[c], out.polarization[c] = g("pos%d" % c), g("dir%d" % c), g("pol%d" % c)
    out.amplitude = g("amp")
    out.radius[0], out.radius[1] = g("r0"), g("r1")
    out.order[0], out.order[1] = int(g("o0")), int(g("o1"))
    out.l, out.zR[0], out.zR[1] = g("l"), g("zR0"), g("zR1")
    sg = out.signal
    sg.type = int(g("sig_type"))
    sg.t0, sg.s, sg.f0, sg.cep, sg.nR = g("sig_t0"), g("sig_s"), g("sig_f0"), g("sig_cep"), g("sig_nR")
    sg.sig0, sg.sig1 = g("sig_g0"), g("sig_g1")
    return out


def seed_params(m: dict) -> MoSeed | None:
    """The seed, or None when it injects nothing (|amplitude| <= 1e-50, src/fdtd.cpp:307)."""
    if abs(m.get("seed_amp", 0.0)) <= 1.0e-50:
        return None
    sd = MoSeed()
    beam_params(m, "seed_", sd.beam)
    sd.gamma, sd.beta, sd.c0, sd.dt = m["seed_gamma"], m["seed_beta"], m["seed_c0"], m["seed_dt"]
    return sd


def field_params(m: dict, solver: int, order: int, space_charge: int = 0) -> MoField:
    f = MoField()
    f.N0, f.N1, f.np, f.k0 = int(m["N0"]), int(m["N1"]), int(m["np"]), int(m.get("k0", 0))
    f.solver, f.order, f.space_charge = solver, order, space_charge
    for i in range(6):
        f.a[i] = m["a%d" % i]
    f.nsfd_alpha, f.nsfd_beta = m["nsfd_alpha"], m["nsfd_beta"]
    for name in ("bB", "cB", "dB", "eE", "fE", "gE"):
        arr = getattr(f, name)
        for i in range(5):
            arr[i] = m["%s%d" % (name, i)]
    for i in range(17):
        f.hC[i] = m["hC%d" % i]
    f.dt, f.dx, f.dy, f.dz = m["dt"], m["dx"], m["dy"], m["dz"]
    f.xmin, f.ymin, f.zmin = m["xmin"], m["ymin"], m["zmin"]
    return f


def push_params(m: dict) -> MoPush:
    p = MoPush()
    p.N0, p.N1, p.np, p.k0 = int(m["N0"]), int(m["N1"]), int(m["np"]), int(m.get("k0", 0))
    for k in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax", "zp0", "zp1", "dx", "dy", "dz"):
        setattr(p, k, m[k])
    p.Lz = m["Lz"]
    p.dtb, p.r1, p.r2 = m["ub_dtb"], m["ub_r1"], m["ub_r2"]
    p.gamma, p.beta, p.c0, p.dt_shift = m["gamma"], m["beta"], m["c0"], m["dt_shift"]
    n = int(m.get("n_undulator", 0))
    p.n_und = n
    for u in range(n):
        U = p.und[u]
        U.type = int(m["und%d_type" % u])
        U.k, U.lu, U.rb = m["und%d_k" % u], m["und%d_lu" % u], m["und%d_rb" % u]
        U.length, U.dist, U.theta = m["und%d_length" % u], m["und%d_dist" % u], m["und%d_theta" % u]
        if U.type == 1:
            beam_params(m, "und%d_beam_" % u, U.beam)
    p.n_ext = int(m.get("n_ext", 0))
    if p.n_ext > MO_MAX_EXT:
        raise ValueError("at most %d external fields" % MO_MAX_EXT)
    for x in range(p.n_ext):
        beam_params(m, "ext%d_" % x, p.ext[x])
    return p


def deposit_params(m: dict) -> MoDeposit:
    d = MoDeposit()
    d.N0, d.N1, d.np, d.k0 = int(m["N0"]), int(m["N1"]), int(m["np"]), int(m.get("k0", 0))
    for k in ("xmin", "ymin", "zmin", "xmax", "ymax", "dx", "dy", "dz", "zp0", "zp1"):
        setattr(d, k, m[k])
    d.Lz = m["Lz"]
    d.dv, d.rc = m.get("uc_dv", 0.0), m.get("uc_rc", 0.0)
    return d


class PowerSampler:
    """State of Solver::powerSample for one FEL output (src/radiation.cpp:18-232)."""

    def __init__(self, m: dict, jf: int = 0):
        self.N = int(m["rp%d_N" % jf])
        self.Nl = int(m["rp%d_Nl" % jf])
        self.Nf = int(m["rp%d_Nf" % jf])
        self.z = np.array([m["rp%d_z%d" % (jf, i)] for i in range(self.N)], dtype=np.float64)
        w = np.array([m["rp%d_w%d" % (jf, i)] for i in range(self.Nl)], dtype=np.float64)
        dt = m["dt"]
        import math
        re = np.empty((self.Nl, self.Nf))
        im = np.empty((self.Nl, self.Nf))
        for l in range(self.Nl):
            for j in range(self.Nf):
                arg = w[l] * j * dt
                re[l, j] = math.cos(arg)
                im[l, j] = math.sin(arg)
        self.ep_re, self.ep_im = re.ravel().copy(), im.ravel().copy()
        N1N0 = int(m["N0"]) * int(m["N1"])
        self.fdt = np.zeros(self.Nf * self.N * N1N0 * 4)
        p = MoPower()
        p.N0, p.N1, p.np, p.k0 = int(m["N0"]), int(m["N1"]), int(m["np"]), int(m.get("k0", 0))
        p.N, p.Nl, p.Nf = self.N, self.Nl, self.Nf
        p.zmin, p.dz, p.zp0, p.zp1 = m["zmin"], m["dz"], m["zp0"], m["zp1"]
        p.gamma, p.beta, p.c0, p.pc = m["gamma"], m["beta"], m["c0"], m["rp%d_pc" % jf]
        p.z, p.ep_re, p.ep_im, p.fdt = dptr(self.z), dptr(self.ep_re), dptr(self.ep_im), dptr(self.fdt)
        self.p = p

    def sample(self, n_time: int, en, bn) -> np.ndarray:
        out = np.zeros(self.N * self.Nl)
        lib().mo_power_sample(C.byref(self.p), n_time, fptr(en), fptr(bn), dptr(out))
        return out


class OracleRun:
    """One single-rank FdTd march on the CPU, state initialised from a meta dict and arrays."""

    def __init__(self, meta: dict, an, anm1, anp1, particles, solver: int, order: int,
                 cap_factor: float = 2.0, fn=None, fnm1=None, fnp1=None):
        self.m = dict(meta)
        self.sc = fn is not None
        self.f = field_params(meta, solver, order, 1 if self.sc else 0)
        self.seed = seed_params(meta)
        self.p = push_params(meta)
        self.d = deposit_params(meta)
        nodes = int(meta["N0"]) * int(meta["N1"]) * int(meta["np"])
        self.an = np.ascontiguousarray(an, dtype=np.float64).reshape(nodes * 3).copy()
        self.anm1 = np.ascontiguousarray(anm1, dtype=np.float64).reshape(nodes * 3).copy()
        self.anp1 = np.ascontiguousarray(anp1, dtype=np.float64).reshape(nodes * 3).copy()
        if self.sc:
            self.fn = np.ascontiguousarray(fn, dtype=np.float64).reshape(nodes).copy()
            self.fnm1 = np.ascontiguousarray(fnm1, dtype=np.float64).reshape(nodes).copy()
            self.fnp1 = np.ascontiguousarray(fnp1, dtype=np.float64).reshape(nodes).copy()
        self.en = np.zeros(nodes * 3, dtype=np.float32)
        self.bn = np.zeros(nodes * 3, dtype=np.float32)
        parts = np.ascontiguousarray(particles, dtype=np.float64).reshape(-1, 11)
        self.n = parts.shape[0]
        self.cap = max(16, int(self.n * cap_factor) + 16)
        self.rec = np.zeros((self.cap, 11))
        self.rec[: self.n] = parts
        self.time = meta["time"]
        self.time_bunch = meta["timeBunch"]
        self.n_time = int(meta["nTime"])
        self.n_time_bunch = int(meta["nTimeBunch"])
        self.n_update_bunch = meta["nUpdateBunch"]
        self.dt = meta["dt"]
        self.dtb_time = meta["dtb"]
        self.power = PowerSampler(meta) if int(meta.get("n_fel", 0)) > 0 and "rp0_N" in meta else None
        self.power_rows = []
        self.screens = None        # lab z of the screens (set_screens)
        self.screen_rows = []      # per step: rows of screen_profile with the screen index in column 7
        self.after_recycle = None  # called as f(run) where Solver::solve writes its field diagnostics

    @property
    def particles(self):
        return self.rec[: self.n]

    def field_update(self):
        if self.seed is not None:
            lib().mo_field_update_seeded(C.byref(self.f), C.byref(self.seed), self.time, dptr(self.anp1),
                                         dptr(self.an), dptr(self.anm1))
        else:
            lib().mo_field_update(C.byref(self.f), dptr(self.anp1), dptr(self.an), dptr(self.anm1))
        if self.sc:
            lib().mo_scalar_update(C.byref(self.f), dptr(self.fnp1), dptr(self.fn), dptr(self.fnm1))

    def eval_eb(self):
        lib().mo_eval_eb(C.byref(self.f), dptr(self.anp1), dptr(self.an), dptr(self.fn) if self.sc else None,
                         fptr(self.en), fptr(self.bn))

    def push(self):
        nt = C.c_long(0)
        n = lib().mo_push_substep(C.byref(self.p), self.time_bunch, dptr(self.rec), self.n, self.cap,
                                  fptr(self.en), fptr(self.bn), C.byref(nt))
        if n < 0:
            raise RuntimeError("particle capacity exceeded")
        self.n = n

    def erase(self):
        m = self.m
        self.n = lib().mo_erase_outside(m["zmin"], m["Lz"], m["zp0"], m["zp1"], dptr(self.rec), self.n)

    def deposit(self):
        self.anp1[:] = 0.0
        if self.sc:
            self.fnp1[:] = 0.0
        lib().mo_deposit_current(C.byref(self.d), dptr(self.rec), self.n, dptr(self.anp1),
                                 dptr(self.fnp1) if self.sc else None)

    def set_screens(self, lz_screens):
        """Record Solver::screenProfile rows every step (screens in the given order)."""
        self.screens = np.ascontiguousarray(lz_screens, dtype=np.float64)

    def _screen(self):
        rows = []
        for i, lz in enumerate(self.screens):
            r = screen_profile(self.m, [lz], self.time_bunch, self.particles)
            rows.append(np.column_stack([r, np.full(len(r), float(i))]))
        self.screen_rows.append(np.concatenate(rows) if rows else np.zeros((0, 8)))

    def step(self):
        """One field step, src/solver.cpp:1300-1399 (diagnostic file writers omitted)."""
        self.field_update()
        self.eval_eb()
        self.rec[: self.n, 4:7] = self.rec[: self.n, 1:4]
        t = 0.0
        while t < self.n_update_bunch:
            self.push()
            self.time_bunch += self.dtb_time
            self.n_time_bunch += 1
            t += 1.0
        self.erase()
        if self.after_recycle is not None:
            self.after_recycle(self)
        if self.screens is not None:
            self._screen()
        if self.power is not None:
            pg = self.power.sample(self.n_time, self.en, self.bn)
            m = self.m
            zl = m["gamma"] * (self.power.z + m["beta"] * m["c0"] * (self.time_bunch + m["dt_shift"]))
            self.power_rows.append((zl, pg))
        self.anm1, self.an, self.anp1 = self.an, self.anp1, self.anm1
        if self.sc:
            self.fnm1, self.fn, self.fnp1 = self.fn, self.fnp1, self.fnm1
        self.deposit()
        self.erase()
        self.time += self.dt
        self.n_time += 1


def bunch_sample(m: dict, rec) -> np.ndarray:
    """Solver::bunchSample moments (12 values) of particle records in the reference's order."""
    rec = np.ascontiguousarray(rec, dtype=np.float64)
    out = np.zeros(12)
    lib().mo_bunch_sample(m["zmin"], m["Lz"], m["zp0"], m["zp1"], dptr(rec), rec.shape[0], dptr(out))
    return out


def bunching_factor(m: dict, rec, k: float) -> float:
    rec = np.ascontiguousarray(rec, dtype=np.float64)
    return lib().mo_bunching_factor(m["zmin"], m["Lz"], m["zp0"], m["zp1"], dptr(rec), rec.shape[0], float(k))


def field_sample(m: dict, an, en, bn, pts, solver: int = 0) -> np.ndarray:
    """FdTd::fieldSample interpolation (E, B, A^n) at points, as (n, 9)."""
    fp = field_params(m, solver, 2)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros((pts.shape[0], 9))
    lib().mo_field_sample(C.byref(fp), dptr(np.ascontiguousarray(an, dtype=np.float64)), fptr(en), fptr(bn),
                          dptr(pts), pts.shape[0], dptr(out))
    return out
