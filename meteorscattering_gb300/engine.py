"""ctypes binding of the C ABI in ``include/mfdtd.h``.

This is the Python face of the engine.  It mirrors the reference's interface
for the path: :func:`run_rundir` is the reference executable run in a run
directory (``source/meteor-2.1.cpp:42``); :class:`Problem` and
:class:`Simulation` expose the same stages for callers that keep data in
memory.  There is no CPU fallback: if ``libmfdtd.so`` has not been built, or a
call needs a GPU and none is present, the call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmfdtd.so")
EXE_PATH = os.path.join(_HERE, "_lib", "meteor")

FORM_FP64_PLAIN = 0
FORM_FP32_FUSED = 1

STATUS = {0: "OK", -1: "EINVAL", -2: "EIO", -3: "ECUDA", -4: "ENOMEM", -5: "ETIMEOUT",
          -6: "ENUMERIC", -7: "ESTATE", -8: "ECANCELED"}

# Every entry point declared in include/mfdtd.h.
EXPORTS = (
    "mfdtd_run_rundir", "mfdtd_problem_from_rundir", "mfdtd_problem_create",
    "mfdtd_problem_destroy", "mfdtd_problem_dims", "mfdtd_problem_footprint",
    "mfdtd_sim_create", "mfdtd_sim_destroy", "mfdtd_sim_advance", "mfdtd_sim_sync",
    "mfdtd_sim_step_index", "mfdtd_sim_ntf_size", "mfdtd_sim_read_ntf",
    "mfdtd_sim_read_probes", "mfdtd_sim_read_field", "mfdtd_sim_write_outputs",
    "mfdtd_sim_last_timing", "mfdtd_sim_kernel_stats", "mfdtd_sim_far_field",
    "mfdtd_far_field_static", "mfdtd_last_error", "mfdtd_version", "mfdtd_ext_defaults",
    "mfdtd_problem_set_ext", "mfdtd_problem_set_trail", "mfdtd_batch_capacity",
    "mfdtd_batch_create", "mfdtd_batch_destroy", "mfdtd_batch_add", "mfdtd_batch_remove",
    "mfdtd_batch_run", "mfdtd_batch_sync", "mfdtd_batch_tune", "mfdtd_server_create",
    "mfdtd_server_destroy", "mfdtd_server_submit", "mfdtd_server_poll", "mfdtd_server_stats",
    "mfdtd_server_cancel", "mfdtd_sim_read_slices", "mfdtd_sim_plasma_fraction",
    "mfdtd_batch_tile_shape",
)


class MfdtdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class RunOpts(C.Structure):
    _fields_ = [("form", C.c_int32), ("device", C.c_int32), ("guard_period", C.c_int32),
                ("quiet", C.c_int32), ("timeout_s", C.c_double), ("profile", C.c_int32)]


class Params(C.Structure):
    """``mfdtd_params`` -- the fields of inputs.dat in file order."""
    _fields_ = [
        ("dopml", C.c_int32), ("savefields", C.c_int32), ("f0", C.c_double), ("fsig", C.c_double),
        ("sourcetype", C.c_int32), ("sourcepol", C.c_int32), ("gridfactor", C.c_double),
        ("dt", C.c_double), ("tsteps", C.c_int32), ("Nx", C.c_int32), ("Ny", C.c_int32),
        ("Nz", C.c_int32), ("metsize", C.c_double * 2), ("wpmax", C.c_double),
        ("numax", C.c_double), ("metloc", C.c_double * 3), ("metangle", C.c_double),
        ("mettype", C.c_int32), ("numfiles", C.c_int32), ("nprobes", C.c_int32),
        ("probex", C.POINTER(C.c_int32)), ("probey", C.POINTER(C.c_int32)),
        ("probez", C.POINTER(C.c_int32)), ("nntf", C.c_int32), ("fntf", C.POINTER(C.c_double)),
        ("doplate", C.c_int32), ("platesize", C.c_double), ("doB0", C.c_int32),
    ]


class Ext(C.Structure):
    """``mfdtd_ext`` -- extended inputs (reference values from mfdtd_ext_defaults)."""
    _fields_ = [
        ("pmllen", C.c_int32), ("tfsf_gap", C.c_int32), ("ntf_gap", C.c_int32),
        ("oblique", C.c_int32), ("exact_coords", C.c_int32), ("lk_colocated", C.c_int32),
        ("pml_m", C.c_double), ("kappa_max", C.c_double), ("alpha_max", C.c_double),
        ("inc_theta", C.c_double), ("inc_phi", C.c_double), ("inc_psi", C.c_double),
    ]


class Trail(C.Structure):
    """``mfdtd_trail`` -- parametric trail."""
    _fields_ = [("centre", C.c_double * 3), ("axis", C.c_double * 3), ("r0", C.c_double),
                ("log10n_lo", C.c_double), ("log10n_hi", C.c_double), ("s_half", C.c_double)]


_lib: Optional[C.CDLL] = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load ``libmfdtd.so`` (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run meteorscattering_gb300.build.build() "
                           "(or __graft_entry__.build()) first; there is no CPU fallback")
    lib = C.CDLL(path)
    vp, i32, i64, dp = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)
    sig = {
        "mfdtd_run_rundir": (C.c_int, [C.c_char_p, C.POINTER(RunOpts)]),
        "mfdtd_problem_from_rundir": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
        "mfdtd_problem_create": (C.c_int, [C.POINTER(Params), dp, dp, dp, C.POINTER(vp)]),
        "mfdtd_problem_destroy": (None, [vp]),
        "mfdtd_problem_dims": (C.c_int, [vp, C.POINTER(i64)]),
        "mfdtd_problem_footprint": (C.c_int, [vp, i32, C.POINTER(i64)]),
        "mfdtd_sim_create": (C.c_int, [vp, C.POINTER(RunOpts), C.POINTER(vp)]),
        "mfdtd_sim_destroy": (None, [vp]),
        "mfdtd_sim_advance": (C.c_int, [vp, i32, i32]),
        "mfdtd_sim_sync": (C.c_int, [vp]),
        "mfdtd_sim_step_index": (C.c_int, [vp, C.POINTER(i32)]),
        "mfdtd_sim_ntf_size": (i64, [vp]),
        "mfdtd_sim_read_ntf": (C.c_int, [vp, dp, i64]),
        "mfdtd_sim_read_probes": (C.c_int, [vp, dp, i64]),
        "mfdtd_sim_read_field": (C.c_int, [vp, i32, dp, i64]),
        "mfdtd_sim_write_outputs": (C.c_int, [vp, C.c_char_p]),
        "mfdtd_sim_last_timing": (C.c_int, [vp, dp, C.POINTER(i64)]),
        "mfdtd_sim_kernel_stats": (C.c_int, [vp, i32, C.c_char_p, C.c_size_t, dp,
                                             C.POINTER(i64)]),
        "mfdtd_sim_far_field": (C.c_int, [vp, i32, dp, dp, i32, dp]),
        "mfdtd_far_field_static": (C.c_int, [C.POINTER(C.c_void_p), i32, i32, i32, i32, i32, dp,
                                             C.c_double, C.c_double, C.c_double, dp, i32, dp, dp,
                                             dp, vp]),
        "mfdtd_ext_defaults": (None, [C.POINTER(Ext)]),
        "mfdtd_problem_set_ext": (C.c_int, [vp, C.POINTER(Ext), dp, dp]),
        "mfdtd_problem_set_trail": (C.c_int, [vp, C.POINTER(Trail)]),
        "mfdtd_batch_capacity": (C.c_int, []),
        "mfdtd_batch_create": (C.c_int, [i32, C.POINTER(vp)]),
        "mfdtd_batch_destroy": (None, [vp]),
        "mfdtd_batch_add": (C.c_int, [vp, vp]),
        "mfdtd_batch_remove": (C.c_int, [vp, vp]),
        "mfdtd_batch_run": (C.c_int, [vp, i32]),
        "mfdtd_batch_sync": (C.c_int, [vp]),
        "mfdtd_batch_tune": (C.c_int, [vp, C.POINTER(i32), i32, C.POINTER(i32), i32,
                                       C.POINTER(i32), C.POINTER(i32)]),
        "mfdtd_batch_tile_shape": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i32)]),
        "mfdtd_server_create": (C.c_int, [i32, i64, i32, C.POINTER(vp)]),
        "mfdtd_server_destroy": (None, [vp]),
        "mfdtd_server_submit": (C.c_int, [vp, vp, i32, dp, dp, C.POINTER(i64)]),
        "mfdtd_server_poll": (C.c_int, [vp, i64, i32, dp, i64, dp, C.POINTER(i32)]),
        "mfdtd_server_stats": (C.c_int, [vp, C.POINTER(i64)]),
        "mfdtd_server_cancel": (C.c_int, [vp, i64]),
        "mfdtd_sim_read_slices": (C.c_int, [vp, i32, dp, dp, i64]),
        "mfdtd_sim_plasma_fraction": (C.c_int, [vp, dp]),
        "mfdtd_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
        "mfdtd_version": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    buf = C.create_string_buffer(4096)
    load_library().mfdtd_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def _check(rc: int) -> None:
    if rc != 0:
        raise MfdtdError(rc, last_error())


def _opts(form: int = FORM_FP64_PLAIN, device: int = 0, guard_period: int = 0,
          quiet: bool = True, timeout_s: float = 0.0, profile: bool = False) -> RunOpts:
    return RunOpts(form, device, guard_period, 1 if quiet else 0, timeout_s, 1 if profile else 0)


def run_rundir(path: str, form: int = FORM_FP64_PLAIN, device: int = 0,
               quiet: bool = True, timeout_s: float = 0.0) -> None:
    """Run the whole solver in run directory ``path`` (the reference's
    ``meteor`` executable contract)."""
    lib = load_library()
    o = _opts(form, device, 0, quiet, timeout_s)
    _check(lib.mfdtd_run_rundir(os.fsencode(path), C.byref(o)))


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Problem:
    """Parsed inputs (host only; no GPU needed)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle

    @classmethod
    def from_rundir(cls, path: str) -> "Problem":
        lib = load_library()
        h = C.c_void_p()
        _check(lib.mfdtd_problem_from_rundir(os.fsencode(path), C.byref(h)))
        return cls(h)

    @classmethod
    def from_params(cls, p, wp2_c: np.ndarray, nu2_c: np.ndarray,
                    B0: Sequence[float] = (0.0, 0.0, 0.0)) -> "Problem":
        """``p`` is a :class:`meteorscattering_gb300.rundir.RunParams`;
        ``wp2_c``/``nu2_c`` are ``[Nx][Ny]`` C-order arrays (wp.dat byte order)."""
        lib = load_library()
        px = np.ascontiguousarray(p.probex, dtype=np.int32)
        py = np.ascontiguousarray(p.probey, dtype=np.int32)
        pz = np.ascontiguousarray(p.probez, dtype=np.int32)
        ff = np.ascontiguousarray(p.fntf, dtype=np.float64)
        i32p = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
        prm = Params(p.dopml, p.savefields, p.f0, p.fsig, p.sourcetype, p.sourcepol,
                     p.gridfactor, p.dt, p.tsteps, p.Nx, p.Ny, p.Nz,
                     (C.c_double * 2)(*p.metsize), p.wpmax, p.numax,
                     (C.c_double * 3)(*p.metloc), p.metangle, p.mettype, p.numfiles,
                     len(px), i32p(px), i32p(py), i32p(pz), len(ff), _dp(ff), p.doplate,
                     p.platesize, int(p.doB0 or 0))
        w = np.ascontiguousarray(wp2_c, dtype=np.float64)
        n = np.ascontiguousarray(nu2_c, dtype=np.float64)
        b = np.ascontiguousarray(B0, dtype=np.float64)
        h = C.c_void_p()
        _check(lib.mfdtd_problem_create(C.byref(prm), _dp(w), _dp(n), _dp(b), C.byref(h)))
        return cls(h)

    def set_ext(self, ext=None, wp3: Optional[np.ndarray] = None,
                nu3: Optional[np.ndarray] = None) -> "Problem":
        """Apply extended inputs (a :class:`rundir.ExtParams`, or None for the
        reference values) and optional per-cell ``[Nx][Ny][Nz]`` maps."""
        lib = load_library()
        e = Ext()
        lib.mfdtd_ext_defaults(C.byref(e))
        if ext is not None:
            for f, _ in Ext._fields_:
                setattr(e, f, getattr(ext, f))
        Nx, Ny, Nz = self.dims()[:3]
        keep = []

        def arr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            if a.shape != (Nx, Ny, Nz):
                raise ValueError(f"per-cell maps must be (Nx, Ny, Nz) = ({Nx}, {Ny}, {Nz})")
            keep.append(a)
            return _dp(a)

        _check(lib.mfdtd_problem_set_ext(self._h, C.byref(e), arr(wp3), arr(nu3)))
        return self

    def set_trail(self, trail=None) -> "Problem":
        """Parametric trail (a :class:`rundir.TrailParams`) for the plasma
        frequency, evaluated on the device; None removes it."""
        lib = load_library()
        if trail is None:
            _check(lib.mfdtd_problem_set_trail(self._h, None))
            return self
        t = Trail((C.c_double * 3)(*trail.centre), (C.c_double * 3)(*trail.axis), trail.r0,
                  trail.log10n_lo, trail.log10n_hi, trail.s_half)
        _check(lib.mfdtd_problem_set_trail(self._h, C.byref(t)))
        return self

    def dims(self):
        out = (C.c_int64 * 6)()
        _check(load_library().mfdtd_problem_dims(self._h, out))
        return tuple(out)

    def footprint(self, form: int = FORM_FP64_PLAIN) -> int:
        v = C.c_int64()
        _check(load_library().mfdtd_problem_footprint(self._h, form, C.byref(v)))
        return v.value

    def close(self):
        if self._h:
            load_library().mfdtd_problem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Simulation:
    """Device-resident state of one run."""

    def __init__(self, problem: Problem, form: int = FORM_FP64_PLAIN, device: int = 0,
                 guard_period: int = 0, timeout_s: float = 0.0, profile: bool = False):
        lib = load_library()
        self.dims = problem.dims()
        o = _opts(form, device, guard_period, True, timeout_s, profile)
        h = C.c_void_p()
        _check(lib.mfdtd_sim_create(problem._h, C.byref(o), C.byref(h)))
        self._h = h

    def advance(self, nsteps: int, collect_records: bool = False) -> None:
        _check(load_library().mfdtd_sim_advance(self._h, nsteps, 1 if collect_records else 0))

    def sync(self) -> None:
        _check(load_library().mfdtd_sim_sync(self._h))

    @property
    def step_index(self) -> int:
        v = C.c_int32()
        _check(load_library().mfdtd_sim_step_index(self._h, C.byref(v)))
        return v.value

    def read_ntf(self) -> np.ndarray:
        lib = load_library()
        n = lib.mfdtd_sim_ntf_size(self._h)
        out = np.empty(n, dtype=np.float64)
        _check(lib.mfdtd_sim_read_ntf(self._h, _dp(out), n))
        return out

    def read_probes(self) -> np.ndarray:
        Nx, Ny, Nz, T, nf, npb = self.dims
        out = np.empty((6, T, npb), dtype=np.float64)
        _check(load_library().mfdtd_sim_read_probes(self._h, _dp(out), out.size))
        return out

    def read_field(self, comp: int) -> np.ndarray:
        Nx, Ny, Nz = self.dims[:3]
        out = np.empty((Nx, Ny, Nz), dtype=np.float64)
        _check(load_library().mfdtd_sim_read_field(self._h, comp, _dp(out), out.size))
        return out

    def plasma_fraction(self) -> float:
        """Share of the FP32 pass's (plane, tile) blocks that hold plasma (J is
        loaded and stored there only); 1 for the FP64 plain form."""
        f = C.c_double()
        _check(load_library().mfdtd_sim_plasma_fraction(self._h, C.byref(f)))
        return f.value

    def read_slices(self, scattered: bool = False):
        """(E, H) record slices of the current state, each a dict of planes
        {"z": [2][Nx][Ny], "y": [2][Nx][Nz], "x": [2][Ny][Nz]} (y and z
        components), total or scattered field."""
        Nx, Ny, Nz = self.dims[:3]
        n = 2 * (Nx * Ny + Nx * Nz + Ny * Nz)
        E = np.empty(n, dtype=np.float64)
        H = np.empty(n, dtype=np.float64)
        _check(load_library().mfdtd_sim_read_slices(self._h, int(bool(scattered)), _dp(E), _dp(H), n))

        def planes(v):
            a, b = 2 * Nx * Ny, 2 * Nx * Nz
            return {"z": v[:a].reshape(2, Nx, Ny), "y": v[a:a + b].reshape(2, Nx, Nz),
                    "x": v[a + b:].reshape(2, Ny, Nz)}
        return planes(E), planes(H)

    def write_outputs(self, path: str) -> None:
        _check(load_library().mfdtd_sim_write_outputs(self._h, os.fsencode(path)))

    def last_timing(self):
        ms, n = C.c_double(), C.c_int64()
        _check(load_library().mfdtd_sim_last_timing(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def far_field(self, theta, phi, method: int = 0) -> np.ndarray:
        """sigma[nntf, ndir, 3] (total, and the two polarisation parts) in m^2."""
        th = np.ascontiguousarray(theta, dtype=np.float64)
        ph = np.ascontiguousarray(phi, dtype=np.float64)
        if th.shape != ph.shape:
            raise ValueError("theta and phi must have the same shape")
        nf = self.dims[4]
        out = np.empty((nf, th.size, 3), dtype=np.float64)
        _check(load_library().mfdtd_sim_far_field(self._h, th.size, _dp(th), _dp(ph), method,
                                                  _dp(out)))
        return out

    def kernel_stats(self):
        """[(name, mean ms per launch, launches)] of the last advance (profile=True)."""
        lib, out, q = load_library(), [], 0
        while True:
            name = C.create_string_buffer(128)
            ms, n = C.c_double(), C.c_int64()
            if lib.mfdtd_sim_kernel_stats(self._h, q, name, 128, C.byref(ms), C.byref(n)) != 0:
                break
            out.append((name.value.decode(), ms.value, n.value))
            q += 1
        return out

    def close(self):
        if self._h:
            load_library().mfdtd_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """FP32 simulations advanced together by the persistent kernel (see
    ``mfdtd_batch_*`` in include/mfdtd.h)."""

    def __init__(self, device: int = 0):
        lib = load_library()
        h = C.c_void_p()
        _check(lib.mfdtd_batch_create(device, C.byref(h)))
        self._h = h
        self._members = []

    @staticmethod
    def capacity() -> int:
        return load_library().mfdtd_batch_capacity()

    def add(self, sim: "Simulation") -> None:
        _check(load_library().mfdtd_batch_add(self._h, sim._h))
        self._members.append(sim)

    def remove(self, sim: "Simulation") -> None:
        _check(load_library().mfdtd_batch_remove(self._h, sim._h))
        self._members.remove(sim)

    def run(self, nsteps: int) -> None:
        _check(load_library().mfdtd_batch_run(self._h, nsteps))

    def sync(self) -> None:
        _check(load_library().mfdtd_batch_sync(self._h))

    def tune(self, slab_depths=(16, 32, 64, 128), ctas_per_sm=(2, 3)):
        """Try every (tile shape, slab depth, CTAs per SM); returns the chosen
        (slab depth, CTAs per SM).  tile_shape() gives the chosen shape."""
        d = (C.c_int32 * len(slab_depths))(*slab_depths)
        c = (C.c_int32 * len(ctas_per_sm))(*ctas_per_sm)
        bd, bc = C.c_int32(), C.c_int32()
        _check(load_library().mfdtd_batch_tune(self._h, d, len(slab_depths), c, len(ctas_per_sm),
                                               C.byref(bd), C.byref(bc)))
        return bd.value, bc.value

    def tile_shape(self):
        """(rows, cols) of the (j, k) tiles the batch runs its interior on."""
        r, c = C.c_int32(), C.c_int32()
        _check(load_library().mfdtd_batch_tile_shape(self._h, C.byref(r), C.byref(c)))
        return r.value, c.value

    def close(self):
        if self._h:
            load_library().mfdtd_batch_destroy(self._h)
            self._h = None
            self._members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The native serving loop (``mfdtd_server_*``): submit problems with the
    radar directions wanted, poll for their cross sections."""

    def __init__(self, device: int = 0, hbm_cap_bytes: int = 150 * 10 ** 9,
                 steps_per_round: int = 100):
        lib = load_library()
        h = C.c_void_p()
        _check(lib.mfdtd_server_create(device, int(hbm_cap_bytes), steps_per_round, C.byref(h)))
        self._h = h
        self._nf = {}

    def submit(self, problem: Problem, theta, phi) -> int:
        th = np.ascontiguousarray(theta, dtype=np.float64)
        ph = np.ascontiguousarray(phi, dtype=np.float64)
        jid = C.c_int64()
        _check(load_library().mfdtd_server_submit(self._h, problem._h, th.size, _dp(th), _dp(ph),
                                                  C.byref(jid)))
        self._nf[jid.value] = (problem.dims()[4], th.size)
        return jid.value

    def poll(self, job_id: int, wait_ms: int = 0):
        """(done, sigma[nntf, ndir, 3] or None, (to_admission_s, to_done_s))."""
        nf, nd = self._nf.get(job_id, (0, 0))   # a canceled job has no result
        out = np.empty((nf, nd, 3), dtype=np.float64)
        times = np.zeros(3)
        done = C.c_int32()
        try:
            _check(load_library().mfdtd_server_poll(self._h, job_id, wait_ms, _dp(out), out.size,
                                                    _dp(times), C.byref(done)))
        except MfdtdError:
            self._nf.pop(job_id, None)   # the native record is released with the error
            raise
        if not done.value:
            return False, None, None
        self._nf.pop(job_id, None)
        return True, out, (times[0], times[1])

    def cancel(self, job_id: int) -> None:
        """Cancel a queued or running job (or drop a finished one's result).
        Polling a canceled job raises MfdtdError with code ECANCELED."""
        _check(load_library().mfdtd_server_cancel(self._h, job_id))
        self._nf.pop(job_id, None)

    def stats(self):
        out = (C.c_int64 * 5)()
        _check(load_library().mfdtd_server_stats(self._h, out))
        return dict(zip(("submitted", "queued", "running", "retired", "device_bytes"), out))

    def close(self):
        if self._h:
            load_library().mfdtd_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
