"""GB300-native FdTd/FdTdSC time-marching loop of MITHRA.

The compute path is libmithra_gb300.so (hand-written sm_103a CUDA kernels behind the C ABI of
include/mithra_gpu.h).  This module binds that ABI with ctypes and mirrors the reference's
solver interface (src/solver.h:20-345, src/fdtd.h:15-66):

    job = Setup.from_job("run.job")            # parse + FP64 initialisation (host)
    s = FdTd(job)                              # `new FdTd(...)`, src/mithra.cpp:86-90
    s.solve()                                  # Solver::solve, src/solver.cpp:1212-1418

Importing never falls back to a CPU implementation: if the library is missing it is built
with nvcc, and if that is impossible the import raises.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import build as _build

__all__ = ["Setup", "Context", "Batch", "FdTd", "FdTdSC", "MithraError", "PinnedArray", "lib", "FP64", "FP32"]

FP64 = 0
FP32 = 1
MAX_UND = 64
MAX_EXT = 16


class MithraError(RuntimeError):
    pass


class GridDesc(C.Structure):
    _fields_ = [("N0", C.c_int32), ("N1", C.c_int32), ("N2", C.c_int32), ("solver", C.c_int32),
                ("truncation_order", C.c_int32), ("space_charge", C.c_int32),
                ("a", C.c_double * 6), ("nsfd_alpha", C.c_double), ("nsfd_beta", C.c_double),
                ("bB", C.c_double * 5), ("cB", C.c_double * 5), ("dB", C.c_double * 5),
                ("eE", C.c_double * 5), ("fE", C.c_double * 5), ("gE", C.c_double * 5),
                ("hC", C.c_double * 17),
                ("dt", C.c_double), ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double), ("ymax", C.c_double),
                ("zmin", C.c_double), ("zmax", C.c_double), ("zp0", C.c_double), ("zp1", C.c_double),
                ("Lz", C.c_double)]


class PushDesc(C.Structure):
    _fields_ = [("dtb", C.c_double), ("bunch_time_step", C.c_double), ("r1", C.c_double), ("r2", C.c_double),
                ("gamma", C.c_double), ("beta", C.c_double), ("c0", C.c_double), ("dt_shift", C.c_double),
                ("n_update_bunch", C.c_double)]


class BeamDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("position", C.c_double * 3), ("direction", C.c_double * 3),
                ("polarization", C.c_double * 3), ("amplitude", C.c_double), ("radius", C.c_double * 2),
                ("order", C.c_int32 * 2), ("wavelength", C.c_double), ("rayleigh", C.c_double * 2),
                ("signal_type", C.c_int32), ("signal_t0", C.c_double), ("signal_s", C.c_double),
                ("signal_f0", C.c_double), ("signal_cep", C.c_double), ("signal_nr", C.c_double),
                ("signal_sigma", C.c_double * 2)]


class SeedDesc(C.Structure):
    _fields_ = [("beam", BeamDesc), ("gamma", C.c_double), ("beta", C.c_double), ("c0", C.c_double),
                ("dt", C.c_double)]


class UndulatorDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("k", C.c_double), ("lu", C.c_double), ("rb", C.c_double),
                ("length", C.c_double), ("dist", C.c_double), ("theta", C.c_double), ("beam", BeamDesc)]


class Tuning(C.Structure):
    _fields_ = [("blocks_per_sm", C.c_int32), ("slab_planes", C.c_int32)]


class PowerDesc(C.Structure):
    _fields_ = [("N", C.c_int32), ("Nl", C.c_int32), ("Nf", C.c_int32), ("pc", C.c_double),
                ("z", C.POINTER(C.c_double)), ("twiddle_re", C.POINTER(C.c_double)),
                ("twiddle_im", C.POINTER(C.c_double))]


class VtkDesc(C.Structure):
    _fields_ = [("N0", C.c_int), ("N1", C.c_int), ("N2", C.c_int), ("np", C.c_int), ("k0", C.c_int),
                ("xmin", C.c_double), ("ymin", C.c_double), ("zmin", C.c_double), ("dx", C.c_double),
                ("dy", C.c_double), ("dz", C.c_double), ("type", C.c_int), ("plane", C.c_int),
                ("position", C.c_double * 3), ("nfield", C.c_int), ("field", C.c_int * 16)]


class TimeState(C.Structure):
    _fields_ = [("time", C.c_double), ("time_bunch", C.c_double), ("n_time", C.c_int64),
                ("n_time_bunch", C.c_int64)]


_lib = None
_P = C.POINTER
_dp, _fp, _vp = _P(C.c_double), _P(C.c_float), C.c_void_p

_SIGS = {
    "mithra_gpu_create": [_P(GridDesc), _P(PushDesc), C.c_int, C.c_int, C.c_size_t, _P(_vp)],
    "mithra_gpu_destroy": [_vp],
    "mithra_gpu_last_error": [_vp, C.c_char_p, C.c_size_t],
    "mithra_gpu_synchronize": [_vp],
    "mithra_gpu_set_undulators": [_vp, _P(UndulatorDesc), C.c_int],
    "mithra_gpu_set_seed": [_vp, C.c_void_p],
    "mithra_gpu_set_external_fields": [_vp, _P(BeamDesc), C.c_int],
    "mithra_gpu_set_power": [_vp, _P(PowerDesc), C.c_int],
    "mithra_gpu_upload_fields": [_vp, _dp, _dp, _dp],
    "mithra_gpu_download_fields": [_vp, _dp, _dp, _dp],
    "mithra_gpu_upload_scalar": [_vp, _dp, _dp, _dp],
    "mithra_gpu_download_scalar": [_vp, _dp, _dp, _dp],
    "mithra_gpu_download_eb": [_vp, _fp, _fp],
    "mithra_gpu_upload_particles": [_vp, _dp, C.c_size_t],
    "mithra_gpu_download_particles": [_vp, _dp, C.c_size_t, _P(C.c_size_t)],
    "mithra_gpu_particle_count": [_vp, _P(C.c_size_t)],
    "mithra_gpu_set_time": [_vp, _P(TimeState)],
    "mithra_gpu_get_time": [_vp, _P(TimeState)],
    "mithra_gpu_field_update": [_vp],
    "mithra_gpu_field_evaluate": [_vp],
    "mithra_gpu_save_positions": [_vp],
    "mithra_gpu_bunch_update": [_vp],
    "mithra_gpu_recycle": [_vp],
    "mithra_gpu_power_sample": [_vp],
    "mithra_gpu_power_sample_noalloc": [_vp],
    "mithra_gpu_bunch_sample": [_vp, _dp],
    "mithra_gpu_set_tuning": [_vp, _P(Tuning)],
    "mithra_gpu_set_wait_limit": [_vp, C.c_int64],
    "mithra_gpu_get_tuning": [_vp, _P(Tuning)],
    "mithra_gpu_autotune": [_vp, C.c_int, _P(Tuning), _dp],
    "mithra_batch_create": [_P(_vp), C.c_int, _P(_vp)],
    "mithra_batch_run": [_vp, C.c_int64],
    "mithra_batch_run_timed": [_vp, C.c_int64, _dp],
    "mithra_batch_destroy": [_vp],
    "mithra_gpu_field_sample": [_vp, _dp, C.c_size_t, _dp],
    "mithra_gpu_bunching_factor": [_vp, C.c_double, _dp],
    "mithra_gpu_set_screens": [_vp, _dp, C.c_int, C.c_longlong],
    "mithra_gpu_screen_clear": [_vp],
    "mithra_gpu_screen_records": [_vp, C.c_int, _dp, C.c_longlong, C.POINTER(C.c_longlong)],
    "mithra_gpu_field_shift": [_vp],
    "mithra_gpu_current_update": [_vp],
    "mithra_gpu_advance_time": [_vp],
    "mithra_gpu_run": [_vp, C.c_int64],
    "mithra_gpu_run_prelude": [_vp],
    "mithra_gpu_run_timed": [_vp, C.c_int64, _dp],
    "mithra_gpu_launches_per_step": [_vp, _P(C.c_int)],
    "mithra_host_alloc": [C.c_size_t, _P(_vp)],
    "mithra_host_free": [_vp],
    "mithra_probe_fp64_tflops": [C.c_int, _dp],
    "mithra_gpu_power_rows": [_vp, _dp, C.c_size_t, _P(C.c_size_t)],
    "mithra_gpu_kernel_times": [_vp, C.c_char_p, C.c_size_t, _dp, C.c_int, _P(C.c_int)],
    "mithra_gpu_enable_timing": [_vp, C.c_int],
    "mithra_setup_from_job": [C.c_char_p, _P(_vp), C.c_char_p, C.c_size_t],
    "mithra_setup_destroy": [_vp],
    "mithra_setup_grid": [_vp, _P(GridDesc)],
    "mithra_setup_push": [_vp, _P(PushDesc)],
    "mithra_setup_undulators": [_vp, _P(UndulatorDesc), C.c_int, _P(C.c_int)],
    "mithra_setup_seed": [_vp, _P(SeedDesc)],
    "mithra_setup_external_fields": [_vp, _P(BeamDesc), C.c_int, _P(C.c_int)],
    "mithra_setup_time": [_vp, _P(TimeState)],
    "mithra_setup_power": [_vp, C.c_int, _P(PowerDesc), _P(C.c_int)],
    "mithra_setup_particles": [_vp, _dp, C.c_size_t, _P(C.c_size_t)],
    "mithra_setup_fields": [_vp, _dp, _dp, _dp],
    "mithra_setup_total_time": [_vp, _dp],
    "mithra_setup_meta": [_vp, C.c_char_p, C.c_size_t, _P(C.c_size_t)],
    "mithra_setup_vtk_basename": [_vp, C.c_int, C.c_char_p, C.c_size_t, _P(C.c_size_t)],
    "mithra_setup_power_basename": [_vp, C.c_int, C.c_char_p, C.c_size_t, _P(C.c_size_t)],
    "mithra_setup_screen_basename": [_vp, C.c_int, C.c_char_p, C.c_size_t, _P(C.c_size_t)],
    "mithra_setup_bunch_sample_file": [_vp, C.c_char_p, C.c_size_t, _P(C.c_size_t)],
    "mithra_setup_field_sample_file": [_vp, C.c_char_p, C.c_size_t, _P(C.c_size_t)],
    "mithra_setup_bunch_profile_basename": [_vp, C.c_char_p, C.c_size_t, _P(C.c_size_t)],
    "mithra_setup_from_job_device": [C.c_char_p, C.c_int, _P(_vp), C.c_char_p, C.c_size_t],
    "mithra_gpu_upload_particles_device": [_vp, _vp, C.c_size_t],
    "mithra_vtk_write_field": [_vp, C.c_char_p, C.c_longlong, _fp, _fp, _dp, _dp],
    "mithra_gpu_screen_profile": [_vp],
    "mithra_gpu_create_from_setup": [_vp, C.c_int, C.c_int, C.c_double, _P(_vp)],
}


def lib_path() -> str:
    return _build.LIB


def lib():
    """Loads libmithra_gb300.so, building it first when it is absent or stale."""
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        for name, args in _SIGS.items():
            fn = getattr(_lib, name)
            fn.argtypes = args
            fn.restype = C.c_int
    return _lib


def dptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous, "float64 C-contiguous array expected"
    return a.ctypes.data_as(_dp)


def fptr(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous, "float32 C-contiguous array expected"
    return a.ctypes.data_as(_fp)


def probe_fp64_tflops(device: int = 0) -> float:
    """The device's measured FP64 FMA rate in TFLOP/s (mithra_probe_fp64_tflops)."""
    out = np.zeros(1)
    r = lib().mithra_probe_fp64_tflops(int(device), dptr(out))
    if r != 0:
        raise MithraError("mithra_probe_fp64_tflops: status %d" % r)
    return float(out[0])


def _check_out(a, n):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or a.size != n or not a.flags.c_contiguous:
        raise MithraError("output buffer must be a C-contiguous float64 array of %d elements" % n)


class PinnedArray:
    """A page-locked host buffer (cudaMallocHost) exposed as a numpy array."""

    def __init__(self, shape, dtype=np.float64):
        self.dtype = np.dtype(dtype)
        n = int(np.prod(shape))
        self._p = _vp()
        r = lib().mithra_host_alloc(max(n, 1) * self.dtype.itemsize, C.byref(self._p))
        if r != 0:
            raise MithraError("mithra_host_alloc failed with status %d" % r)
        buf = (C.c_char * (max(n, 1) * self.dtype.itemsize)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=n).reshape(shape)

    def free(self):
        if getattr(self, "_p", None) and self._p.value and _lib is not None:
            self.array = None
            _lib.mithra_host_free(self._p)
            self._p = None

    def __del__(self):
        self.free()


class Setup:
    """Parsed job plus the reference's FP64 host initialisation (Solver::initialize)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def from_job(cls, path: str, device_init: bool = False, device: int = 0) -> "Setup":
        """Parses the job and runs Solver::initialize.  device_init=True runs the particle phase
        (ellipsoid bunch generation, boost, distribution, time shift) as kernels on `device`,
        and the particles stay there for Context.from_setup."""
        h = _vp()
        err = C.create_string_buffer(1024)
        if device_init:
            r = lib().mithra_setup_from_job_device(os.fsencode(path), int(device), C.byref(h), err, len(err))
        else:
            r = lib().mithra_setup_from_job(os.fsencode(path), C.byref(h), err, len(err))
        if r != 0:
            raise MithraError("job %s: %s (status %d)" % (path, err.value.decode(errors="replace"), r))
        return cls(h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mithra_setup_destroy(self._h)
            self._h = None

    def grid(self) -> GridDesc:
        g = GridDesc()
        lib().mithra_setup_grid(self._h, C.byref(g))
        return g

    def push(self) -> PushDesc:
        p = PushDesc()
        lib().mithra_setup_push(self._h, C.byref(p))
        return p

    def seed(self) -> "SeedDesc":
        sd = SeedDesc()
        lib().mithra_setup_seed(self._h, C.byref(sd))
        return sd

    def external_fields(self):
        arr = (BeamDesc * MAX_EXT)()
        n = C.c_int()
        lib().mithra_setup_external_fields(self._h, arr, MAX_EXT, C.byref(n))
        return [arr[i] for i in range(n.value)]

    def undulators(self):
        arr = (UndulatorDesc * MAX_UND)()
        n = C.c_int()
        lib().mithra_setup_undulators(self._h, arr, MAX_UND, C.byref(n))
        return [arr[i] for i in range(n.value)]

    def time(self) -> TimeState:
        t = TimeState()
        lib().mithra_setup_time(self._h, C.byref(t))
        return t

    def power_outputs(self) -> list:
        """The radiation-power outputs as mithra_gpu_set_power takes them: dicts of N, Nl, Nf, pc
        and copies of the plane positions z and the twiddles re, im (Nl * Nf each)."""
        n = C.c_int()
        lib().mithra_setup_power(self._h, 0, None, C.byref(n))
        out = []
        for o in range(n.value):
            d = PowerDesc()
            lib().mithra_setup_power(self._h, o, C.byref(d), C.byref(n))
            k = d.Nl * d.Nf
            out.append({"N": d.N, "Nl": d.Nl, "Nf": d.Nf, "pc": d.pc,
                        "z": np.ctypeslib.as_array(d.z, (d.N,)).copy() if d.N else np.zeros(0),
                        "re": np.ctypeslib.as_array(d.twiddle_re, (k,)).copy() if k else np.zeros(0),
                        "im": np.ctypeslib.as_array(d.twiddle_im, (k,)).copy() if k else np.zeros(0)})
        return out

    def total_time(self) -> float:
        v = C.c_double()
        lib().mithra_setup_total_time(self._h, C.byref(v))
        return v.value

    def particles(self) -> np.ndarray:
        n = C.c_size_t()
        lib().mithra_setup_particles(self._h, None, 0, C.byref(n))
        out = np.zeros((n.value, 11))
        lib().mithra_setup_particles(self._h, dptr(out), n.value, C.byref(n))
        return out

    def fields(self):
        g = self.grid()
        n = g.N0 * g.N1 * g.N2 * 3
        anp1, an, anm1 = np.zeros(n), np.zeros(n), np.zeros(n)
        lib().mithra_setup_fields(self._h, dptr(anp1), dptr(an), dptr(anm1))
        return anp1, an, anm1

    def _string(self, fn: str, i: int) -> str:
        need = C.c_size_t()
        if getattr(lib(), fn)(self._h, int(i), None, 0, C.byref(need)) != 0:
            raise MithraError("%s: no entry %d" % (fn, i))
        buf = C.create_string_buffer(need.value)
        getattr(lib(), fn)(self._h, int(i), buf, need.value, C.byref(need))
        return buf.value.decode()

    def _file(self, fn: str, what: str) -> str:
        need = C.c_size_t()
        if getattr(lib(), fn)(self._h, None, 0, C.byref(need)) != 0:
            raise MithraError("the job does not %s" % what)
        buf = C.create_string_buffer(need.value)
        getattr(lib(), fn)(self._h, buf, need.value, C.byref(need))
        return buf.value.decode()

    def bunch_sample_file(self) -> str:
        """File of the bunch-sampling group (directory prefixed, .txt)."""
        return self._file("mithra_setup_bunch_sample_file", "sample the bunch")

    def field_sample_file(self) -> str:
        """File of the field-sampling group (directory prefixed, -0.txt)."""
        return self._file("mithra_setup_field_sample_file", "sample the field")

    def bunch_profile_basename(self) -> str:
        """Base name of the bunch-profile dumps (directory prefixed)."""
        return self._file("mithra_setup_bunch_profile_basename", "dump bunch profiles")

    def screen_basename(self, jf: int) -> str:
        """Base name of the screens of FEL-OUTPUT entry jf (directory prefixed)."""
        return self._string("mithra_setup_screen_basename", jf)

    def power_basename(self, o: int) -> str:
        """Base name of radiation-power output o (directory prefixed); files <base>-<l>.txt."""
        need = C.c_size_t()
        if lib().mithra_setup_power_basename(self._h, int(o), None, 0, C.byref(need)) != 0:
            raise MithraError("no radiation-power output %d" % o)
        buf = C.create_string_buffer(need.value)
        lib().mithra_setup_power_basename(self._h, int(o), buf, need.value, C.byref(need))
        return buf.value.decode()

    def vtk_basename(self, i: int) -> str:
        """Base name of field-visualization output i (directory prefixed)."""
        need = C.c_size_t()
        if lib().mithra_setup_vtk_basename(self._h, int(i), None, 0, C.byref(need)) != 0:
            raise MithraError("no field-visualization output %d" % i)
        buf = C.create_string_buffer(need.value)
        lib().mithra_setup_vtk_basename(self._h, int(i), buf, need.value, C.byref(need))
        return buf.value.decode()

    def screens(self) -> np.ndarray:
        """Lab z of the job's screens (bunch-profile-lab-frame groups), in the reference's
        order: FEL-OUTPUT entries in order, each entry's positions sorted."""
        m = self.meta()
        return np.array([m["scr%d_z" % i] for i in range(int(m.get("n_screens", 0)))])

    def meta(self) -> dict:
        need = C.c_size_t()
        lib().mithra_setup_meta(self._h, None, 0, C.byref(need))
        buf = C.create_string_buffer(need.value)
        lib().mithra_setup_meta(self._h, buf, need.value, C.byref(need))
        out = {}
        for line in buf.value.decode().splitlines():
            k, v = line.split()
            out[k] = float(v)
        return out


def vtk_desc(meta: dict, i: int) -> VtkDesc:
    """The i-th field-visualization output of a job (meta of Setup.meta) as the writer's
    descriptor: one domain, bunch-frame geometry, field codes Ex..Az = 0..8, F = 9."""
    p = "vtk%d_" % i
    d = VtkDesc()
    d.N0, d.N1, d.N2 = int(meta["N0"]), int(meta["N1"]), int(meta["N2"])
    d.np, d.k0 = int(meta["np"]), int(meta["k0"])
    d.xmin, d.ymin, d.zmin = meta["xmin"], meta["ymin"], meta["zmin"]
    d.dx, d.dy, d.dz = meta["dx"], meta["dy"], meta["dz"]
    d.type, d.plane = int(meta[p + "type"]), int(meta[p + "plane"])
    for q in range(3):
        d.position[q] = meta[p + "pos%d" % q]
    d.nfield = int(meta[p + "nfield"])
    for l in range(d.nfield):
        d.field[l] = int(meta[p + "f%d" % l])
    return d


def vtk_due(meta: dict, i: int, time: float) -> bool:
    """Solver::solve's condition for writing output i at field time `time` (src/solver.cpp:1328-1340)."""
    p = "vtk%d_" % i
    return bool(meta[p + "sample"]) and float(np.fmod(time, meta[p + "rhythm"])) < meta["dt"] and time > 0.0


def write_field_vtk(meta: dict, i: int, basename: str, n_time: int, en, bn, an, fn=None):
    """Writes output i (FdTd::fieldVisualize*, the reference's file layout) from host arrays: E, B
    float32 and A^n float64 with 3 values per node, phi^n float64 or None."""
    d = os.path.dirname(basename)
    if d:
        os.makedirs(d, exist_ok=True)
    en = np.ascontiguousarray(en, dtype=np.float32)
    bn = np.ascontiguousarray(bn, dtype=np.float32)
    an = np.ascontiguousarray(an, dtype=np.float64)
    fn = None if fn is None else np.ascontiguousarray(fn, dtype=np.float64)
    r = lib().mithra_vtk_write_field(C.byref(vtk_desc(meta, i)), basename.encode(), int(n_time), fptr(en), fptr(bn),
                                     dptr(an), dptr(fn))
    if r != 0:
        raise MithraError("mithra_vtk_write_field failed with status %d (output %d)" % (r, i))


def format_bunch_sample(row) -> str:
    """One line of the bunch-sampling file (Solver::bunchSample, src/solver.cpp:1623-1635):
    timeBunch, <r>, <gb>, rms r, rms gb in %.4e, tab-separated."""
    return "\t".join("%.4e" % v for v in np.asarray(row, dtype=np.float64)[:13]) + "\n"


def field_sample_points(meta: dict) -> np.ndarray:
    """The field-sampling points of a job (bunch frame, inside the mesh), (n, 3)."""
    return np.array([[meta["fs_p%d_%d" % (i, d)] for d in range(3)] for i in range(int(meta.get("fs_n", 0)))])


def field_sample_due(meta: dict, time: float) -> bool:
    """Solver::solve's condition for a field sample at field time `time` (src/solver.cpp:1329)."""
    return bool(meta.get("fs_sampling", 0)) and float(np.fmod(time, meta["fs_rhythm"])) < meta["dt"] and time > 0.0


def format_field_sample(meta: dict, time: float, points, samples) -> str:
    """One row of the field-sampling file (FdTd::fieldSample, src/fdtd.cpp:851-950): time_ gamma_,
    then per point its position and the requested fields transformed to the lab frame and the
    file's units, %.4e, tab-separated.  samples: (n, 9) E, B, A^n of Context.field_sample."""
    g, c0 = meta["gamma"], meta["c0"]
    Ce, Cb, Ca = meta["fs_Ce"], meta["fs_Cb"], meta["fs_Ca"]
    gb = math.sqrt(math.pow(g, 2) - 1)
    fields = [int(meta["fs_f%d" % l]) for l in range(int(meta.get("fs_nfield", 0)))]
    out = ["%.4e" % (time * g)]
    for p, v in zip(np.asarray(points, dtype=np.float64), np.asarray(samples, dtype=np.float64)):
        e, b, a = v[0:3], v[3:6], v[6:9]
        out += ["%.4e" % p[0], "%.4e" % p[1], "%.4e" % p[2]]
        for f in fields:
            if f == 0: x = (g * e[0] + c0 * gb * b[1]) * Ce
            elif f == 1: x = (g * e[1] - c0 * gb * b[0]) * Ce
            elif f == 2: x = e[2] * Ce
            elif f == 3: x = (g * b[0] - gb / c0 * e[1]) * Cb
            elif f == 4: x = (g * b[1] + gb / c0 * e[0]) * Cb
            elif f == 5: x = b[2] * Cb
            elif f < 9: x = a[f - 6] * Ca
            else: continue  # FdTd writes nothing for the scalar potential
            out.append("%.4e" % x)
    return "\t".join(out) + "\t\n"


def bunch_profile_due(meta: dict, time: float) -> int:
    """How many times Solver::solve writes a bunch profile at field time `time`
    (src/solver.cpp:1258-1266, :1362-1370): once per listed time just passed, once on the rhythm."""
    if not meta.get("bunch_profile", 0):
        return 0
    n, dt = 0, meta["dt"]
    for i in range(int(meta.get("bunch_profile_ntime", 0))):
        t = meta["bunch_profile_t%d" % i]
        if time - t < dt and time > t:
            n += 1
    r, ts = meta["bunch_profile_rhythm"], time + meta["time_shift"]
    if r != 0.0 and float(np.fmod(ts, r)) < dt and ts > 0.0:
        n += 1
    return n


def format_bunch_profile(time_lab: float, rec) -> str:
    """A bunch-profile dump (Solver::bunchProfile, src/solver.cpp:1763-1792): time_ gamma_ on the
    first line (width 40), then q, rnp, gb of every particle, %.15e, tab-separated.  rec: particle
    records (q, rnp, rnm, gb, e) in list order."""
    rec = np.asarray(rec, dtype=np.float64).reshape(-1, 11)
    out = [("%.15e" % time_lab).rjust(40) + "\n"]
    cols = rec[:, [0, 1, 2, 3, 7, 8, 9]]
    out += ["\t".join("%.15e" % v for v in row) + "\n" for row in cols]
    return "".join(out)


def bunch_sample_due(meta: dict, time: float) -> bool:
    """Solver::solve's condition for a bunch sample at field time `time` (src/solver.cpp:1252, :1356)."""
    t = time + meta["time_shift"]
    return bool(meta.get("bunch_sampling", 0)) and float(np.fmod(t, meta["bunch_rhythm"])) < meta["dt"] and t > 0.0


def format_power_text(rows, n_planes: int, n_freq: int, freq: int, first_in_file: bool = True) -> str:
    """One frequency's power file as the reference writes it (src/radiation.cpp:80-82, :222-229):
    per step, for each sampling plane, z_lab and P tab-terminated, in %.15e, the stream's width of
    40 applying once, to the first value of the file.  rows: the row log of one power output,
    steps x (n_planes x (1 + n_freq)) as mithra_gpu_power_rows returns it."""
    rows = np.asarray(rows, dtype=np.float64).reshape(-1, n_planes, 1 + n_freq)
    out = []
    for r, step in enumerate(rows):
        vals = []
        for k in range(n_planes):
            vals += ["%.15e" % step[k, 0], "%.15e" % step[k, 1 + freq]]
        if r == 0 and first_in_file:
            vals[0] = vals[0].rjust(40)
        out.append("\t".join(vals) + "\t\n")
    return "".join(out)


def format_screen_text(rows, first_in_file: bool = True) -> str:
    """Screen rows (x, y, t, gbx, gby, gbz) as the reference writes them
    (src/solver.cpp:2186-2191, :2230-2252): scientific with 15 decimals, tab-separated, one
    crossing per line; the stream's width of 40 applies once, to the first value of the file."""
    out = []
    for r, row in enumerate(np.asarray(rows, dtype=np.float64).reshape(-1, 6)):
        vals = ["%.15e" % v for v in row]
        if r == 0 and first_in_file:
            vals[0] = vals[0].rjust(40)
        out.append("\t".join(vals) + "\n")
    return "".join(out)


class Context:
    """One GPU domain: owns every device buffer of a FdTd/FdTdSC solve."""

    def __init__(self, handle, grid: GridDesc):
        self._h = handle
        self.grid = grid
        self.nodes = grid.N0 * grid.N1 * grid.N2

    @classmethod
    def create(cls, grid: GridDesc, push: PushDesc, precision: int = FP64, device: int = 0,
               capacity: int = 1 << 20) -> "Context":
        h = _vp()
        r = lib().mithra_gpu_create(C.byref(grid), C.byref(push), precision, device, capacity, C.byref(h))
        if r != 0:
            raise MithraError("mithra_gpu_create failed with status %d" % r)
        return cls(h, grid)

    @classmethod
    def from_setup(cls, setup: Setup, precision: int = FP64, device: int = 0,
                   capacity_factor: float = 1.25) -> "Context":
        h = _vp()
        r = lib().mithra_gpu_create_from_setup(setup._h, precision, device, capacity_factor, C.byref(h))
        if r != 0:
            raise MithraError("mithra_gpu_create_from_setup failed with status %d" % r)
        return cls(h, setup.grid())

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.mithra_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _ck(self, r, what):
        if r != 0:
            buf = C.create_string_buffer(1024)
            lib().mithra_gpu_last_error(self._h, buf, len(buf))
            raise MithraError("%s: %s (status %d)" % (what, buf.value.decode(errors="replace"), r))

    def call(self, name, *args):
        self._ck(getattr(lib(), name)(self._h, *args), name)

    def set_undulators(self, und):
        arr = (UndulatorDesc * max(1, len(und)))(*und)
        self.call("mithra_gpu_set_undulators", arr, len(und))

    def set_seed(self, seed):
        """The TF/SF seed (a SeedDesc), or None for none."""
        self.call("mithra_gpu_set_seed", C.byref(seed) if seed is not None else None)

    def set_external_fields(self, fields):
        arr = (BeamDesc * max(1, len(fields)))(*fields)
        self.call("mithra_gpu_set_external_fields", arr, len(fields))

    def set_power(self, outputs):
        """outputs: list of dicts with N, Nl, Nf, pc, z, tw_re, tw_im (numpy float64)."""
        self._power_keep = []
        descs = (PowerDesc * max(1, len(outputs)))()
        for i, o in enumerate(outputs):
            z = np.ascontiguousarray(o["z"], dtype=np.float64)
            re = np.ascontiguousarray(o["tw_re"], dtype=np.float64)
            im = np.ascontiguousarray(o["tw_im"], dtype=np.float64)
            self._power_keep += [z, re, im]
            descs[i] = PowerDesc(int(o["N"]), int(o["Nl"]), int(o["Nf"]), float(o["pc"]), dptr(z), dptr(re), dptr(im))
        self.call("mithra_gpu_set_power", descs, len(outputs))

    def upload_fields(self, anp1=None, an=None, anm1=None):
        conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        a, b, c = conv(anp1), conv(an), conv(anm1)
        self.call("mithra_gpu_upload_fields", dptr(a), dptr(b), dptr(c))

    def download_fields(self, out=None):
        """(anp1_, an_, anm1_) as FP64 arrays of nodes x 3; `out`: three such arrays to fill
        (pinned host buffers, say)."""
        n = self.nodes * 3
        anp1, an, anm1 = out if out is not None else (np.empty(n), np.empty(n), np.empty(n))
        for a in (anp1, an, anm1):
            _check_out(a, n)
        self.call("mithra_gpu_download_fields", dptr(anp1), dptr(an), dptr(anm1))
        return anp1, an, anm1

    def upload_scalar(self, fnp1=None, fn=None, fnm1=None):
        conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        self.call("mithra_gpu_upload_scalar", dptr(conv(fnp1)), dptr(conv(fn)), dptr(conv(fnm1)))

    def download_scalar(self, out=None):
        n = self.nodes
        a, b, c = out if out is not None else (np.empty(n), np.empty(n), np.empty(n))
        for x in (a, b, c):
            _check_out(x, n)
        self.call("mithra_gpu_download_scalar", dptr(a), dptr(b), dptr(c))
        return a, b, c

    def download_eb(self):
        en = np.empty(self.nodes * 3, dtype=np.float32)
        bn = np.empty(self.nodes * 3, dtype=np.float32)
        self.call("mithra_gpu_download_eb", fptr(en), fptr(bn))
        return en, bn

    def upload_particles(self, rec):
        rec = np.ascontiguousarray(rec, dtype=np.float64).reshape(-1, 11)
        self.call("mithra_gpu_upload_particles", dptr(rec), rec.shape[0])

    def particle_count(self) -> int:
        n = C.c_size_t()
        self.call("mithra_gpu_particle_count", C.byref(n))
        return n.value

    def download_particles(self, out=None) -> np.ndarray:
        """The particle records (rows of 11 doubles); `out`: an array of at least
        particle_count() such rows to fill.  Returns the filled rows."""
        cap = self.particle_count()
        if out is None:
            out = np.zeros((max(cap, 1), 11))
        elif out.dtype != np.float64 or out.ndim != 2 or out.shape[1] != 11 or out.shape[0] < cap \
                or not out.flags.c_contiguous:
            raise MithraError("download_particles: out must be a C-contiguous float64 array of at least "
                              "%d x 11" % cap)
        n = C.c_size_t()
        self.call("mithra_gpu_download_particles", dptr(out), cap, C.byref(n))
        return out[: n.value]

    def set_time(self, t: TimeState):
        self.call("mithra_gpu_set_time", C.byref(t))

    def get_time(self) -> TimeState:
        t = TimeState()
        self.call("mithra_gpu_get_time", C.byref(t))
        return t

    def power_rows(self) -> np.ndarray:
        n = C.c_size_t()
        self.call("mithra_gpu_power_rows", None, 0, C.byref(n))
        out = np.zeros(n.value)
        self.call("mithra_gpu_power_rows", dptr(out), n.value, C.byref(n))
        return out

    def enable_timing(self, on: bool = True):
        self.call("mithra_gpu_enable_timing", 1 if on else 0)

    def kernel_times(self) -> dict:
        n = C.c_int()
        self.call("mithra_gpu_kernel_times", None, 0, None, 0, C.byref(n))
        cnt = n.value
        names = C.create_string_buffer(64 * max(cnt, 1))
        ms = np.zeros(2 * max(cnt, 1))
        self.call("mithra_gpu_kernel_times", names, 64, dptr(ms), cnt, C.byref(n))
        out = {}
        for i in range(cnt):
            nm = names.raw[64 * i: 64 * (i + 1)].split(b"\0", 1)[0].decode()
            out[nm] = (ms[2 * i], int(ms[2 * i + 1]))
        return out

    # Stages, one per reference member function.
    def field_update(self):
        self.call("mithra_gpu_field_update")

    def field_evaluate(self):
        self.call("mithra_gpu_field_evaluate")

    def save_positions(self):
        self.call("mithra_gpu_save_positions")

    def bunch_update(self):
        self.call("mithra_gpu_bunch_update")

    def recycle(self):
        self.call("mithra_gpu_recycle")

    def power_sample(self):
        self.call("mithra_gpu_power_sample")

    def set_tuning(self, blocks_per_sm: int = 16, slab_planes: int = 64):
        self.call("mithra_gpu_set_tuning", C.byref(Tuning(blocks_per_sm, slab_planes)))

    def set_wait_limit(self, iterations: int = -1):
        """Attempts of each bounded barrier wait in the mixed form's stencil (negative: default;
        0: every wait gives up at once)."""
        self.call("mithra_gpu_set_wait_limit", int(iterations))

    def tuning(self) -> Tuning:
        t = Tuning()
        self.call("mithra_gpu_get_tuning", C.byref(t))
        return t

    def autotune(self, steps_per_trial: int = 2):
        """Times the candidate launch shapes on real steps of the march; keeps the fastest.
        Returns (Tuning, ms per step)."""
        t = Tuning()
        ms = np.zeros(1)
        self.call("mithra_gpu_autotune", int(steps_per_trial), C.byref(t), dptr(ms))
        return t, float(ms[0])

    def bunch_sample(self) -> np.ndarray:
        """Solver::bunchSample row: timeBunch, <r>(3), <gb>(3), rms r(3), rms gb(3)."""
        row = np.zeros(13)
        self.call("mithra_gpu_bunch_sample", dptr(row))
        return row

    def field_sample(self, points) -> np.ndarray:
        """FdTd::fieldSample: E, B, A^n at each point (n, 3) -> (n, 9)."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((pts.shape[0], 9))
        self.call("mithra_gpu_field_sample", dptr(pts), pts.shape[0], dptr(out))
        return out

    def bunching_factor(self, k: float) -> float:
        """|sum q exp(i k z)| / sum q over the particles of the domain (bunch-frame z)."""
        b = np.zeros(1)
        self.call("mithra_gpu_bunching_factor", float(k), dptr(b))
        return float(b[0])

    def set_screens(self, lz, capacity: int = 0):
        """Lab-frame screens (Solver::screenProfile): every following step, and every step of
        run_prelude, records the particles whose lab z passes a screen.  lz in um from the
        undulator start; capacity = records kept per screen (0: the particle capacity)."""
        z = np.ascontiguousarray(lz, dtype=np.float64)
        self.n_screens = len(z)
        self.call("mithra_gpu_set_screens", dptr(z) if len(z) else None, len(z), int(capacity))

    def screen_clear(self):
        self.call("mithra_gpu_screen_clear")

    def screen_records(self, screen: int) -> np.ndarray:
        """Records of one screen in the reference's file order: (n, 7) rows of x, y, t, gbx,
        gby, gbz (lab) and the step's nTime_."""
        n = C.c_longlong(0)
        self.call("mithra_gpu_screen_records", int(screen), None, 0, C.byref(n))
        out = np.zeros((n.value, 7))
        if n.value:
            self.call("mithra_gpu_screen_records", int(screen), dptr(out), n.value, C.byref(n))
        return out

    def write_screen_files(self, base: str) -> list:
        """The reference's screen files, base + "-p0-screen<i>.txt" (src/solver.cpp:2186-2191,
        :2230-2252): per crossing x, y, t, gbx, gby, gbz tab-separated in %.15e, the first value
        of a file right-aligned in 40 characters (the stream's one-shot width).  Returns the
        file names."""
        names = []
        d = os.path.dirname(base)
        if d:
            os.makedirs(d, exist_ok=True)
        for i in range(getattr(self, "n_screens", 0)):
            name = "%s-p0-screen%d.txt" % (base, i)
            with open(name, "w") as f:
                f.write(format_screen_text(self.screen_records(i)[:, :6]))
            names.append(name)
        return names

    def power_sample_noalloc(self):
        """power_sample with no device allocation: partial sums in a fixed per-device array."""
        self.call("mithra_gpu_power_sample_noalloc")

    def field_shift(self):
        self.call("mithra_gpu_field_shift")

    def current_update(self):
        self.call("mithra_gpu_current_update")

    def advance_time(self):
        self.call("mithra_gpu_advance_time")

    def run(self, nsteps: int):
        self.call("mithra_gpu_run", int(nsteps))

    def run_timed(self, nsteps: int) -> float:
        """Runs `nsteps` steps; returns their device time in ms (CUDA events on the context stream)."""
        ms = C.c_double()
        self.call("mithra_gpu_run_timed", int(nsteps), C.byref(ms))
        return ms.value

    def launches_per_step(self) -> int:
        n = C.c_int()
        self.call("mithra_gpu_launches_per_step", C.byref(n))
        return n.value

    def run_prelude(self):
        self.call("mithra_gpu_run_prelude")

    def synchronize(self):
        self.call("mithra_gpu_synchronize")


class Batch:
    """Independent contexts on one device stepped together: one graph launch per field step
    advances every instance (a parameter sweep)."""

    def __init__(self, contexts):
        self.contexts = list(contexts)
        arr = (_vp * len(self.contexts))(*[c._h for c in self.contexts])
        self._h = _vp()
        r = lib().mithra_batch_create(arr, len(self.contexts), C.byref(self._h))
        if r != 0:
            raise MithraError("mithra_batch_create failed with status %d" % r)

    def _ck(self, r, what):
        if r != 0:
            for c in self.contexts:   # a failing instance reports through its own context
                buf = C.create_string_buffer(1024)
                lib().mithra_gpu_last_error(c._h, buf, len(buf))
                if buf.value:
                    raise MithraError("%s: %s (status %d)" % (what, buf.value.decode(errors="replace"), r))
            raise MithraError("%s failed with status %d" % (what, r))

    def run(self, nsteps: int):
        self._ck(lib().mithra_batch_run(self._h, int(nsteps)), "mithra_batch_run")

    def run_timed(self, nsteps: int) -> float:
        ms = np.zeros(1)
        self._ck(lib().mithra_batch_run_timed(self._h, int(nsteps), dptr(ms)), "mithra_batch_run_timed")
        return float(ms[0])

    def close(self):
        if self._h:
            lib().mithra_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FdTd:
    """Drop-in for the reference's FdTd (src/fdtd.h:15-66) driven by a GPU context.

    The member functions keep the reference's names; `solve()` marches to mesh.totalTime_ like
    Solver::solve and returns the power rows (z_lab, P...) that the reference writes to its
    power-sampling files."""

    precision = FP64

    def __init__(self, setup: Setup, precision: int | None = None, device: int = 0, capacity_factor: float = 1.25,
                 write_files: bool = True):
        """write_files: solve() writes the job's output files where the reference does (power
        per frequency, field visualization, lab-frame screens), relative to the working
        directory for relative names."""
        self.setup = setup
        self.write_files = write_files
        self.meta = setup.meta()
        self.ctx = Context.from_setup(setup, self.precision if precision is None else precision, device, capacity_factor)
        screens = setup.screens()
        if len(screens):  # Solver::initializeScreenProfile: record crossings from the start
            self.ctx.set_screens(screens)

    def currentReset(self):  # noqa: N802 - reference name
        pass  # folded into currentUpdate, as the reference calls them back to back

    def currentUpdate(self):  # noqa: N802
        self.ctx.current_update()

    def currentCommunicate(self):  # noqa: N802
        pass  # one domain: nothing to exchange; the erasure is part of currentUpdate

    def fieldUpdate(self):  # noqa: N802
        self.ctx.field_update()

    def fieldShift(self):  # noqa: N802
        self.ctx.field_shift()

    def bunchUpdate(self):  # noqa: N802
        self.ctx.bunch_update()

    def powerSample(self):  # noqa: N802
        self.ctx.power_sample()

    def steps_to_total_time(self) -> int:
        t = self.ctx.get_time()
        total = self.setup.total_time()
        time, dt, n = t.time, self.meta["dt"], 0
        while time < total:
            time += dt
            n += 1
        return n

    def solve(self, max_steps: int | None = None):
        """Solver::solve: the prelude, then field steps to the total time.  Steps at which a
        field-visualization output or a bunch sample is due (src/solver.cpp:1252, :1328-1356) run
        stage by stage and write their files where the reference does; all others replay the
        captured step graph."""
        m = self.meta
        c = self.ctx
        sampling = self.write_files and (bool(m.get("bunch_sampling", 0)) or bool(m.get("bunch_profile", 0)))
        fsampling = self.write_files and int(m.get("fs_n", 0)) > 0
        self._bunch_lines = []
        self._field_lines = []
        self._fs_points = field_sample_points(m) if fsampling else None
        if sampling:
            self._prelude_with_samples()
        else:
            c.run_prelude()
        n = self.steps_to_total_time()
        if max_steps is not None:
            n = min(n, max_steps)
        nv = int(m.get("n_vtk", 0)) if self.write_files else 0
        due = []
        if nv or sampling or fsampling:
            t, dt = c.get_time().time, m["dt"]
            for s in range(n):
                outs = [i for i in range(nv) if vtk_due(m, i, t)]
                bs = sampling and (bunch_sample_due(m, t) or bunch_profile_due(m, t) > 0)
                fs = fsampling and field_sample_due(m, t)
                if outs or bs or fs:
                    due.append((s, outs, bs, fs))
                t += dt
        done = 0
        for s, outs, bs, fs in due:
            c.run(s - done)
            self._step_with_outputs(outs, bs, fs)
            done = s + 1
        c.run(n - done)
        rows = c.power_rows()
        if self.write_files:
            self.write_power_files(rows)
            self.write_screen_files()
            for on, getter, lines in ((bool(m.get("bunch_sampling", 0)), "bunch_sample_file", self._bunch_lines),
                                      (fsampling, "field_sample_file", self._field_lines)):
                if not on:
                    continue
                path = getattr(self.setup, getter)()
                d = os.path.dirname(path)
                if d:
                    os.makedirs(d, exist_ok=True)
                with open(path, "w") as f:
                    f.write("".join(lines))
        return rows

    def _substeps(self):
        t = 0.0
        while t < self.meta["nUpdateBunch"]:
            self.ctx.bunch_update()
            t += 1.0

    def _prelude_with_samples(self):
        """The time_ < 0 loop of Solver::solve (src/solver.cpp:1232-1291) stage by stage, with its
        screen profile and bunch samples."""
        c = self.ctx
        if not c.get_time().time < 0.0:
            return
        c.field_evaluate()  # no field update before time zero: E/B of the initial potentials
        while True:
            t = c.get_time()
            if not t.time < 0.0:
                break
            c.save_positions()
            self._substeps()
            if getattr(c, "n_screens", 0):
                c.call("mithra_gpu_screen_profile")
            self._bunch_outputs(t)
            c.recycle()
            c.advance_time()

    def _bunch_outputs(self, t):
        """bunchSample and bunchProfile where Solver::solve calls them (t: the step's time state)."""
        m, c = self.meta, self.ctx
        if self.write_files and m.get("bunch_sampling", 0) and bunch_sample_due(m, t.time):
            self._bunch_lines.append(format_bunch_sample(c.bunch_sample()))
        if self.write_files and bunch_profile_due(m, t.time):
            base = self.setup.bunch_profile_basename()
            d = os.path.dirname(base)
            if d:
                os.makedirs(d, exist_ok=True)
            with open("%s-p0-%d.txt" % (base, t.n_time), "w") as f:
                f.write(format_bunch_profile(t.time * m["gamma"], c.download_particles()))

    def _step_with_outputs(self, outs, bunch_sample: bool, field_sample: bool = False):
        c = self.ctx
        tm = c.get_time()
        n_time = tm.n_time
        c.field_update()
        c.save_positions()
        self._substeps()
        c.recycle()
        if field_sample:
            self._field_lines.append(format_field_sample(self.meta, tm.time, self._fs_points,
                                                         c.field_sample(self._fs_points)))
        if outs:
            c.field_evaluate()
            en, bn = c.download_eb()
            _, an, _ = c.download_fields()
            fn = c.download_scalar()[1] if isinstance(self, FdTdSC) else None
            for i in outs:
                write_field_vtk(self.meta, i, self.setup.vtk_basename(i), n_time, en, bn, an, fn)
        if bunch_sample:
            self._bunch_outputs(tm)
        if getattr(c, "n_screens", 0):
            c.call("mithra_gpu_screen_profile")
        c.power_sample()
        c.field_shift()
        c.current_update()
        c.advance_time()

    def write_power_files(self, rows=None):
        """<base>-<l>.txt for every radiation-power output and frequency, in the reference's
        layout (Solver::powerSample, src/radiation.cpp:222-229)."""
        m = self.meta
        jfs = [jf for jf in range(int(m.get("n_fel", 0))) if "rp%d_N" % jf in m]
        if not jfs:
            return []
        shape = [(int(m["rp%d_N" % jf]), int(m["rp%d_Nl" % jf])) for jf in jfs]
        per_step = sum(N * (1 + nl) for N, nl in shape)
        rows = (self.ctx.power_rows() if rows is None else np.asarray(rows)).reshape(-1, per_step)
        names, off = [], 0
        for o, (N, nl) in enumerate(shape):
            block = rows[:, off:off + N * (1 + nl)]
            off += N * (1 + nl)
            base = self.setup.power_basename(o)
            d = os.path.dirname(base)
            if d:
                os.makedirs(d, exist_ok=True)
            for l in range(nl):
                name = "%s-%d.txt" % (base, l)
                with open(name, "w") as f:
                    f.write(format_power_text(block, N, nl, l))
                names.append(name)
        return names

    def write_screen_files(self):
        """<base>-p0-screen<i>.txt per FEL-OUTPUT entry with screens (src/solver.cpp:2186-2252)."""
        m = self.meta
        n = int(m.get("n_screens", 0))
        names, i = [], 0
        while i < n:
            jf = int(m["scr%d_fel" % i])
            base = self.setup.screen_basename(jf)
            d = os.path.dirname(base)
            if d:
                os.makedirs(d, exist_ok=True)
            local = 0
            while i < n and int(m["scr%d_fel" % i]) == jf:
                name = "%s-p0-screen%d.txt" % (base, local)
                with open(name, "w") as f:
                    f.write(format_screen_text(self.ctx.screen_records(i)[:, :6]))
                names.append(name)
                i += 1
                local += 1
        return names

class FdTdSC(FdTd):
    """Drop-in for FdTdSC (src/fdtdSC.h): the same loop with the scalar potential."""
