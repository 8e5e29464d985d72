"""Run-directory file formats of the meteor FDTD solver.

The solver's whole external interface is a directory: four binary input files
written by the MATLAB setup scripts and five output files read by the MATLAB
analysis scripts.  This module writes the inputs and parses the outputs with
exactly the reference byte layouts, so tests and tools can drive either the
reference executable or this engine and compare the files they produce.

Byte layouts (little-endian; MATLAB 'int' = int32, 'double' = float64):

* ``inputs.dat`` -- positional record written by ``setup/meteorrun.m:44-70`` and
  read by ``source/meteor-2.1.cpp:84-112``; the magnetized solver
  ``source/meteor-fork.cpp:115`` reads one more int, ``doB0``, after
  ``platesize``.  MATLAB never writes it, so both lengths are accepted.
* ``B0.dat`` -- three doubles Bx, By, Bz in tesla (``setup/meteorrun.m:74-78``,
  ``source/meteor-fork.cpp:219-224``).
* ``wp.dat`` / ``nu.dat`` -- an Nx-by-Ny MATLAB matrix written column-major
  (``setup/meteorrun.m:106-112``) and read back as a C ``[Nx][Ny]`` array
  (``source/meteor-2.1.cpp:301-315``).  The writer here takes the MATLAB-shaped
  matrix and writes it in Fortran order, so the solver sees the same bytes.
* ``output_{E,H,J}.dat`` -- one record per record step, appended
  (``source/meteor-2.1.cpp:1545-1568``; reader ``analysis/plotMresults.m:179-208``).
* ``output_NTF.dat`` -- ``source/meteor-2.1.cpp:1579-1620``; reader
  ``analysis/meteorNTF.m:12-57``.
* ``Probe.dat`` -- ``source/meteor-2.1.cpp:1624-1636``.
"""
from __future__ import annotations

import dataclasses
import math
import os
import struct
from typing import Dict, List, Optional, Sequence

import numpy as np

# Solver constants (source/meteor-2.1.cpp:12-18).  These differ from the
# analysis constants in analysis/loadconstants.m on purpose: the solver uses
# U0 = 1.2566e-6 and E0 = 8.85419e-12.
PI = 3.141592653589793
QE = 1.602177e-19
E0 = 8.85419e-12
U0 = 1.2566e-6
ME = 9.10939e-31
C0 = 3.0e8

NTF_FACE_ORDER = (
    # (name, face-kind) in the order output_NTF.dat stores them
    # (source/meteor-2.1.cpp:1591-1620)
    ("My_front", "fb"), ("Mz_front", "fb"), ("Jy_front", "fb"), ("Jz_front", "fb"),
    ("My_back", "fb"), ("Mz_back", "fb"), ("Jy_back", "fb"), ("Jz_back", "fb"),
    ("Mx_top", "tb"), ("Mz_top", "tb"), ("Jx_top", "tb"), ("Jz_top", "tb"),
    ("Mx_bot", "tb"), ("Mz_bot", "tb"), ("Jx_bot", "tb"), ("Jz_bot", "tb"),
    ("Mx_left", "lr"), ("My_left", "lr"), ("Jx_left", "lr"), ("Jy_left", "lr"),
    ("Mx_right", "lr"), ("My_right", "lr"), ("Jx_right", "lr"), ("Jy_right", "lr"),
)


@dataclasses.dataclass
class RunParams:
    """Fields of ``inputs.dat`` in file order (``source/meteor-2.1.cpp:84-112``)."""

    Nx: int
    Ny: int
    Nz: int
    tsteps: int
    dt: float
    f0: float = 50e6
    fsig: float = 20.0
    gridfactor: float = 24.0
    dopml: int = 1
    savefields: int = 1
    sourcetype: int = 2
    sourcepol: int = 1
    metsize: Sequence[float] = (1.0, 1.0)
    wpmax: float = 1.0
    numax: float = 0.0
    metloc: Sequence[float] = (0.0, 0.0, 0.0)
    metangle: float = 0.0
    mettype: int = 0
    numfiles: int = 1
    probex: Sequence[int] = ()
    probey: Sequence[int] = ()
    probez: Sequence[int] = ()
    fntf: Sequence[float] = (50e6,)
    doplate: int = 0
    platesize: float = 1.0
    doB0: Optional[int] = None  # None: omit the field, as MATLAB does

    @property
    def nprobes(self) -> int:
        return len(self.probex)

    @property
    def nntf(self) -> int:
        return len(self.fntf)

    @property
    def dx(self) -> float:
        return (C0 / self.f0) / self.gridfactor

    def record_steps(self) -> List[int]:
        """Steps at which slices and the max|Ex| line are written
        (``source/meteor-2.1.cpp:1523``: ``t % (tsteps/numfiles) == 0``)."""
        period = self.tsteps // self.numfiles
        return [t for t in range(self.tsteps) if t % period == 0]


def pack_inputs(p: RunParams) -> bytes:
    """Serialise ``p`` exactly as ``setup/meteorrun.m:44-70`` does."""
    if not (len(p.probex) == len(p.probey) == len(p.probez)):
        raise ValueError("probex/probey/probez must have equal length")
    out = bytearray()
    i32 = lambda v: out.extend(struct.pack("<i", int(v)))
    f64 = lambda v: out.extend(struct.pack("<d", float(v)))
    i32(p.dopml); i32(p.savefields)
    f64(p.f0); f64(p.fsig)
    i32(p.sourcetype); i32(p.sourcepol)
    f64(p.gridfactor); f64(p.dt)
    i32(p.tsteps); i32(p.Nx); i32(p.Ny); i32(p.Nz)
    for v in p.metsize:
        f64(v)
    f64(p.wpmax); f64(p.numax)
    for v in p.metloc:
        f64(v)
    f64(p.metangle)
    i32(p.mettype); i32(p.numfiles); i32(p.nprobes)
    for arr in (p.probex, p.probey, p.probez):
        for v in arr:
            i32(v)
    i32(p.nntf)
    for v in p.fntf:
        f64(v)
    i32(p.doplate); f64(p.platesize)
    if p.doB0 is not None:
        i32(p.doB0)
    return bytes(out)


def unpack_inputs(buf: bytes) -> RunParams:
    """Parse an ``inputs.dat`` record (either length)."""
    off = 0

    def take(fmt):
        nonlocal off
        vals = struct.unpack_from("<" + fmt, buf, off)
        off += struct.calcsize("<" + fmt)
        return vals

    dopml, savefields = take("ii")
    f0, fsig = take("dd")
    sourcetype, sourcepol = take("ii")
    gridfactor, dt = take("dd")
    tsteps, Nx, Ny, Nz = take("iiii")
    metsize = take("dd")
    wpmax, numax = take("dd")
    metloc = take("ddd")
    (metangle,) = take("d")
    mettype, numfiles, nprobes = take("iii")
    probex = take("i" * nprobes)
    probey = take("i" * nprobes)
    probez = take("i" * nprobes)
    (nntf,) = take("i")
    fntf = take("d" * nntf)
    (doplate,) = take("i")
    (platesize,) = take("d")
    doB0 = None
    if len(buf) - off >= 4:
        (doB0,) = take("i")
    return RunParams(Nx=Nx, Ny=Ny, Nz=Nz, tsteps=tsteps, dt=dt, f0=f0, fsig=fsig,
                     gridfactor=gridfactor, dopml=dopml, savefields=savefields,
                     sourcetype=sourcetype, sourcepol=sourcepol, metsize=metsize,
                     wpmax=wpmax, numax=numax, metloc=metloc, metangle=metangle,
                     mettype=mettype, numfiles=numfiles, probex=list(probex),
                     probey=list(probey), probez=list(probez), fntf=list(fntf), doplate=doplate, platesize=platesize,
                     doB0=doB0)


def write_rundir(path: str, p: RunParams, wp: np.ndarray, nu: np.ndarray,
                 B0: Sequence[float] = (0.0, 0.0, 0.0)) -> None:
    """Write ``inputs.dat``, ``B0.dat``, ``wp.dat``, ``nu.dat`` into ``path``.

    ``wp`` and ``nu`` are MATLAB-shaped ``(Nx, Ny)`` matrices (rad/s and 1/s);
    they are written column-major like MATLAB's ``fwrite``
    (``setup/meteorrun.m:106-112``).  Stale appended outputs are removed first,
    which is what ``setup/writepbsfile.m:10-13`` does before each run.
    """
    os.makedirs(path, exist_ok=True)
    wp = np.asarray(wp, dtype=np.float64)
    nu = np.asarray(nu, dtype=np.float64)
    if wp.shape != (p.Nx, p.Ny) or nu.shape != (p.Nx, p.Ny):
        raise ValueError(f"wp/nu must be (Nx, Ny) = ({p.Nx}, {p.Ny})")
    with open(os.path.join(path, "inputs.dat"), "wb") as f:
        f.write(pack_inputs(p))
    with open(os.path.join(path, "B0.dat"), "wb") as f:
        f.write(struct.pack("<ddd", *[float(b) for b in B0]))
    with open(os.path.join(path, "wp.dat"), "wb") as f:
        f.write(wp.tobytes(order="F"))
    with open(os.path.join(path, "nu.dat"), "wb") as f:
        f.write(nu.tobytes(order="F"))
    for name in ("output_E.dat", "output_H.dat", "output_J.dat", "Probe.dat",
                 "output_NTF.dat", "log.txt", "ext.dat", "wp3.dat", "nu3.dat", "trail.dat"):
        fp = os.path.join(path, name)
        if os.path.exists(fp):
            os.remove(fp)


# --------------------------------------------------------------------------
# Extended inputs (no counterpart in the reference, which hard-codes them)

EXT_MAGIC = b"MFDTDX01"


@dataclasses.dataclass
class ExtParams:
    """``mfdtd_ext`` of ``include/mfdtd.h``.  The defaults are the values the
    reference hard-codes (``source/meteor-2.1.cpp:343, 413-415, 539-552``) and
    its +x plane wave."""

    pmllen: int = 10
    tfsf_gap: int = 10
    ntf_gap: int = 5
    oblique: int = 0
    exact_coords: int = 0
    lk_colocated: int = 0
    pml_m: float = 4.0
    kappa_max: float = 1.0
    alpha_max: float = 0.0
    inc_theta: float = math.pi / 2
    inc_phi: float = 0.0
    inc_psi: float = 0.0

    def k_hat(self) -> np.ndarray:
        th, ph = self.inc_theta, self.inc_phi
        return np.array([math.sin(th) * math.cos(ph), math.sin(th) * math.sin(ph), math.cos(th)])


def pack_ext(e: ExtParams, has_wp3: bool, has_nu3: bool) -> bytes:
    """``ext.dat``: 8-byte magic, 8 int32 (pmllen, tfsf_gap, ntf_gap, oblique,
    exact_coords, has_wp3, has_nu3, lk_colocated), 6 float64 (pml_m, kappa_max, alpha_max,
    inc_theta, inc_phi, inc_psi); 88 bytes."""
    return (EXT_MAGIC
            + struct.pack("<8i", e.pmllen, e.tfsf_gap, e.ntf_gap, e.oblique, e.exact_coords,
                          1 if has_wp3 else 0, 1 if has_nu3 else 0, e.lk_colocated)
            + struct.pack("<6d", e.pml_m, e.kappa_max, e.alpha_max, e.inc_theta, e.inc_phi,
                          e.inc_psi))


def unpack_ext(buf: bytes):
    if buf[:8] != EXT_MAGIC or len(buf) < 88:
        raise ValueError("not an ext.dat record")
    iv = struct.unpack_from("<8i", buf, 8)
    dv = struct.unpack_from("<6d", buf, 40)
    e = ExtParams(pmllen=iv[0], tfsf_gap=iv[1], ntf_gap=iv[2], oblique=iv[3],
                  exact_coords=iv[4], lk_colocated=iv[7], pml_m=dv[0], kappa_max=dv[1], alpha_max=dv[2],
                  inc_theta=dv[3], inc_phi=dv[4], inc_psi=dv[5])
    return e, bool(iv[5]), bool(iv[6])


def write_ext(path: str, e: ExtParams, wp3: Optional[np.ndarray] = None,
              nu3: Optional[np.ndarray] = None) -> None:
    """Write ``ext.dat`` and, when given, the per-cell maps ``wp3.dat`` /
    ``nu3.dat`` (``[Nx][Ny][Nz]`` float64, C order: these files are this
    engine's own, so no MATLAB transposition applies)."""
    with open(os.path.join(path, "ext.dat"), "wb") as f:
        f.write(pack_ext(e, wp3 is not None, nu3 is not None))
    for name, arr in (("wp3.dat", wp3), ("nu3.dat", nu3)):
        fp = os.path.join(path, name)
        if arr is not None:
            np.ascontiguousarray(arr, dtype="<f8").tofile(fp)
        elif os.path.exists(fp):
            os.remove(fp)


@dataclasses.dataclass
class TrailParams:
    """``mfdtd_trail`` of ``include/mfdtd.h``: n = n0(s) exp(-d^2/r0^2) about
    an axis through ``centre`` along ``axis``; log10 n0 linear in s from
    ``log10n_lo`` at s = -s_half to ``log10n_hi`` at s = +s_half, held beyond."""

    centre: Sequence[float] = (0.0, 0.0, 0.0)
    axis: Sequence[float] = (0.0, 0.0, 1.0)
    r0: float = 1.0
    log10n_lo: float = 14.0
    log10n_hi: float = 14.0
    s_half: float = 1.0

    @classmethod
    def tilted(cls, tilt_deg: float, r0: float, log10n_lo: float, log10n_hi: float,
               s_half: float, centre=(0.0, 0.0, 0.0)) -> "TrailParams":
        """Axis tilted ``tilt_deg`` from +z toward +x."""
        t = math.radians(tilt_deg)
        return cls(tuple(centre), (math.sin(t), 0.0, math.cos(t)), r0, log10n_lo, log10n_hi, s_half)


TRAIL_MAGIC = b"MFDTDT01"


def write_trail(path: str, t: Optional[TrailParams]) -> None:
    """``trail.dat``: 8-byte magic and 12 float64 (centre, axis, r0, log10n_lo,
    log10n_hi, s_half, 0, 0); ``None`` removes the file."""
    fp = os.path.join(path, "trail.dat")
    if t is None:
        if os.path.exists(fp):
            os.remove(fp)
        return
    with open(fp, "wb") as f:
        f.write(TRAIL_MAGIC + struct.pack("<12d", *t.centre, *t.axis, t.r0, t.log10n_lo,
                                          t.log10n_hi, t.s_half, 0.0, 0.0))


def trail_wp3(Nx: int, Ny: int, Nz: int, dx: float, t: TrailParams) -> np.ndarray:
    """The per-cell plasma frequency the engine evaluates for trail ``t``
    (exact cell coordinates), as an ``[Nx][Ny][Nz]`` array."""
    a = np.asarray(t.axis, dtype=np.float64)
    a = a / math.sqrt(float(a @ a))
    x = grid_coords(Nx, dx)[:, None, None] - t.centre[0]
    y = grid_coords(Ny, dx)[None, :, None] - t.centre[1]
    z = grid_coords(Nz, dx)[None, None, :] - t.centre[2]
    out = np.empty((Nx, Ny, Nz))
    for i in range(Nx):  # plane by plane keeps the temporaries small
        xi = x[i]
        s = xi * a[0] + y * a[1] + z * a[2]
        d2 = np.maximum(xi * xi + y * y + z * z - s * s, 0.0)
        frac = np.clip((s + t.s_half) / (2 * t.s_half), 0.0, 1.0)
        n0 = 10.0 ** (t.log10n_lo + (t.log10n_hi - t.log10n_lo) * frac)
        out[i] = plasma_frequency(n0 * np.exp(-d2 / (t.r0 * t.r0)))
    return out


def tilted_trail_wp3(Nx: int, Ny: int, Nz: int, dx: float, tilt_deg: float, r0: float,
                     log10n_lo: float, log10n_hi: float, centre=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Per-cell plasma frequency of a straight trail tilted ``tilt_deg`` from +z
    toward +x whose log10 density runs from ``log10n_lo`` at the bottom of the
    grid to ``log10n_hi`` at the top."""
    t = TrailParams.tilted(tilt_deg, r0, log10n_lo, log10n_hi, 0.5 * (Nz - 1) * dx, centre)
    return trail_wp3(Nx, Ny, Nz, dx, t)


def plasma_sphere_wp3(Nx: int, Ny: int, Nz: int, dx: float, radius: float,
                      n_e: float) -> np.ndarray:
    """Per-cell plasma frequency of a homogeneous sphere of ``radius`` (m)
    and density ``n_e`` (m^-3) at the grid centre (cell-centred exact
    coordinates, staircased)."""
    x = grid_coords(Nx, dx)[:, None, None]
    y = grid_coords(Ny, dx)[None, :, None]
    z = grid_coords(Nz, dx)[None, None, :]
    inside = (x * x + y * y + z * z) < radius * radius
    return np.where(inside, plasma_frequency(n_e), 0.0)


# --------------------------------------------------------------------------
# Physical set-up helpers (restating the trail model of setup/meteorrun.m:83-104
# and the synthetic trail used by the benchmarks)

def stable_dt(dx: float, courant: float = 0.5) -> float:
    """dt = courant * dx / (c * sqrt(3)) with the solver's c."""
    return courant * dx / (C0 * math.sqrt(3.0))


def plasma_frequency(n_e: np.ndarray) -> np.ndarray:
    """omega_p = sqrt(n e^2 / (eps0 m_e)) with the solver's constants."""
    return np.sqrt(np.asarray(n_e, dtype=np.float64) * QE * QE / (E0 * ME))


def grid_coords(n: int, dx: float) -> np.ndarray:
    """MATLAB grid coordinates ``-(N-1)/2*dx + dx*(0:N-1)`` (setup/meteorrun.m:27-29)."""
    return -(n - 1) / 2.0 * dx + dx * np.arange(n)


def gaussian_trail_wp(p: RunParams, n0: float, r0: float,
                      centre=(0.0, 0.0)) -> np.ndarray:
    """Plasma-frequency map of a straight trail along z with
    n(r) = n0 exp(-r^2 / r0^2), as an (Nx, Ny) MATLAB-shaped matrix."""
    x = grid_coords(p.Nx, p.dx)[:, None]
    y = grid_coords(p.Ny, p.dx)[None, :]
    r2 = (x - centre[0]) ** 2 + (y - centre[1]) ** 2
    return plasma_frequency(n0 * np.exp(-r2 / (r0 * r0)))


def meteorrun_wp(p: RunParams) -> np.ndarray:
    """Trail map of ``setup/meteorrun.m:86-96`` for ``metangle == 0``
    (``imrotate(wp, 0, 'crop')`` is the identity).  ``p.wpmax`` is in units
    of the radar angular frequency, ``metsize`` = (size, size*metshape)."""
    if p.metangle != 0:
        raise NotImplementedError("only metangle == 0 is restated")
    x = grid_coords(p.Nx, p.dx)
    y = grid_coords(p.Ny, p.dx)
    w0 = p.wpmax * (2 * math.pi * p.f0)
    wp = np.zeros((p.Nx, p.Ny))
    for i in range(p.Nx):
        s = p.metsize[0] if x[i] < p.metloc[0] else p.metsize[1]
        wp[i, :] = (w0 * np.exp(-(x[i] - p.metloc[0]) ** 2 / s ** 2)
                    * np.exp(-(y - p.metloc[1]) ** 2 / p.metsize[0] ** 2))
    return wp


# --------------------------------------------------------------------------
# Output readers

def read_ntf(path: str, p: RunParams) -> Dict[str, np.ndarray]:
    """Parse ``output_NTF.dat``.  Face arrays come back C-shaped
    ``[a][b][2*nntf]`` with (sin, cos) interleaved on the last axis."""
    with open(path, "rb") as f:
        buf = f.read()
    nntf, ntfb = struct.unpack_from("<ii", buf, 0)
    off = 8
    arr = lambda n: np.frombuffer(buf, dtype="<f8", count=n, offset=off)
    out: Dict[str, np.ndarray] = {"nntf": nntf, "ntfb": ntfb}
    out["fntf"] = arr(nntf).copy(); off += 8 * nntf
    out["Eydft"] = arr(2 * nntf).copy(); off += 16 * nntf
    out["Ezdft"] = arr(2 * nntf).copy(); off += 16 * nntf
    shapes = {"fb": (p.Ny, p.Nz), "tb": (p.Nx, p.Nz), "lr": (p.Nx, p.Ny)}
    for name, kind in NTF_FACE_ORDER:
        a, b = shapes[kind]
        n = a * b * 2 * nntf
        out[name] = arr(n).reshape(a, b, 2 * nntf).copy()
        off += 8 * n
    if off != len(buf):
        raise ValueError(f"output_NTF.dat: {len(buf) - off} trailing bytes")
    return out


def read_probes(path: str, tsteps: int) -> Dict[str, np.ndarray]:
    with open(path, "rb") as f:
        buf = f.read()
    (n,) = struct.unpack_from("<i", buf, 0)
    off = 4
    out: Dict[str, np.ndarray] = {"nprobes": n}
    for key in ("probex", "probey", "probez"):
        out[key] = np.frombuffer(buf, dtype="<i4", count=n, offset=off).copy()
        off += 4 * n
    for key in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        out[key] = np.frombuffer(buf, dtype="<f8", count=tsteps * n,
                                 offset=off).reshape(tsteps, n).copy()
        off += 8 * tsteps * n
    if off != len(buf):
        raise ValueError(f"Probe.dat: {len(buf) - off} trailing bytes")
    return out


def read_slices(path: str, p: RunParams, with_inc: bool) -> List[Dict[str, np.ndarray]]:
    """Parse one of ``output_{E,H,J}.dat`` into a list of records.  Each record
    holds C-shaped slices ``z [2][Nx][Ny]``, ``y [2][Nx][Nz]``, ``x [2][Ny][Nz]``
    and, for E and H, the two 1-D incident arrays."""
    data = np.fromfile(path, dtype="<f8")
    per = 2 * (p.Nx * p.Ny + p.Nx * p.Nz + p.Ny * p.Nz) + (2 * p.Nx if with_inc else 0)
    if data.size % per:
        raise ValueError(f"{path}: size {data.size} not a multiple of record {per}")
    recs = []
    for r in range(data.size // per):
        d = data[r * per:(r + 1) * per]
        o = 0
        rec = {}
        for key, (a, b) in (("z", (p.Nx, p.Ny)), ("y", (p.Nx, p.Nz)), ("x", (p.Ny, p.Nz))):
            rec[key] = d[o:o + 2 * a * b].reshape(2, a, b)
            o += 2 * a * b
        if with_inc:
            rec["inc0"] = d[o:o + p.Nx]; o += p.Nx
            rec["inc1"] = d[o:o + p.Nx]; o += p.Nx
        recs.append(rec)
    return recs


def read_log_maxima(path: str) -> List[str]:
    """The ``Maximum abs(Ex) is ...`` values of ``log.txt`` as printed."""
    out = []
    with open(path) as f:
        for line in f:
            key = "Maximum abs(Ex) is "
            if key in line:
                out.append(line.split(key, 1)[1].strip())
    return out
