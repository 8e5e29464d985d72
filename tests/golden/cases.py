"""Parity cases shared by the golden-vector generator and the tests.

Each case is a complete run directory for the reference solver: a
:class:`RunParams`, MATLAB-shaped ``wp``/``nu`` maps and a ``B0`` vector.  They
are small (seconds on one CPU core for the reference) but together reach every
code path of the time loop: both J updates (Young DI and Lee-Kalluri), all
source types and polarisations, the plate and the conducting sphere, CPML on
and off, record steps and probes, non-cubic grids, and every way the collision
frequency can vary (uniform, per column, per cell).
"""
from __future__ import annotations

import math
from typing import Dict, Tuple

import numpy as np

from meteorscattering_gb300 import rundir as rd

# B0 = 5e-5 T dipped 60 degrees in the x-z plane.
B0_DIP60 = (5e-5 * math.cos(math.pi / 3), 0.0, -5e-5 * math.sin(math.pi / 3))


def _mk(N=(48, 48, 48), n0=1e14, r0=1.0, nu=5e4, B0=B0_DIP60, **kw):
    Nx, Ny, Nz = N
    d = dict(Nx=Nx, Ny=Ny, Nz=Nz, tsteps=40, dt=rd.stable_dt(0.25), f0=50e6, fsig=8.0,
             gridfactor=24.0, numfiles=4, probex=[Nx // 2, 23], probey=[Ny // 2, 21],
             probez=[Nz // 2, 25], fntf=[45e6, 50e6], metsize=(2.0, 2.0), doB0=0)
    d.update(kw)
    p = rd.RunParams(**d)
    wp = rd.gaussian_trail_wp(p, n0, r0)
    nuarr = nu if isinstance(nu, np.ndarray) else np.full((Nx, Ny), float(nu))
    return p, wp, nuarr, B0


def _nu_map(N, seed=7):
    rng = np.random.default_rng(seed)
    return 3e4 + 4e4 * rng.random((N[0], N[1]))


def cases() -> Dict[str, Tuple[rd.RunParams, np.ndarray, np.ndarray, tuple]]:
    return {
        # magnetized trail, LK table per k (uniform nu, z-Gaussian active)
        "lk_trail": _mk(doB0=1, sourcepol=4),
        # isotropic trail, sinusoid source, Ey polarisation
        "di_sine_ey": _mk(sourcetype=1, sourcepol=2, fntf=[50e6]),
        # Ricker source, 45-degree polarisation, MATLAB-length inputs.dat (no doB0)
        "ricker_matlab": _mk(sourcetype=3, sourcepol=3, doB0=None),
        # flat plate scatterer (doplate=1), LHCP
        "plate": _mk(doplate=1, platesize=3.0, sourcepol=5),
        # conducting sphere (doplate=2)
        "sphere": _mk(doplate=2, platesize=2.0, fntf=[40e6, 50e6, 60e6]),
        # no CPML
        "nopml": _mk(dopml=0, doB0=1),
        # non-cubic grid, Nz < Nx (coordinate quirks stay harmless)
        "rect": _mk(N=(52, 52, 40), doB0=1, numfiles=40),
        # collision frequency varies per column, z-uniform trail: LK table per (i,j)
        "lk_numap": _mk(doB0=1, nu=_nu_map((48, 48)), metsize=(1e200, 1e200)),
        # collision frequency varies per cell: LK table per cell
        "lk_general": _mk(N=(44, 44, 44), doB0=1, nu=_nu_map((44, 44), 3)),
        # no probes, no saved fields, one record step
        "quiet": _mk(probex=[], probey=[], probez=[], savefields=0, numfiles=1, doB0=1),
    }


# ---------------------------------------------------------------------------
# Extended inputs (ext.dat; no counterpart in the reference).  Each case is
# (RunParams, wp, nu, B0, ExtParams, wp3 or None, nu3 or None).  The oracle is
# the checker for these; its extensions are validated by physics tests
# (TF/SF leakage, normal incidence through the oblique path, Mie series).

def _ext_mk(N=(48, 48, 48), **kw):
    # Courant 0.9 and 160+ steps: the pulse crosses the Huygens surface.
    d = dict(dt=rd.stable_dt(0.25, 0.9), tsteps=160, fsig=20.0, numfiles=8)
    d.update(kw)
    return _mk(N=N, **d)


def ext_cases():
    out = {}
    # CPML of the 96x96x192 benchmark configuration: m = 3, kappa_max = 5,
    # alpha_max = 0.05, 12 cells; TF/SF box 8 cells and Huygens surface 4 cells
    # inside the CPML; reference +x plane wave.
    p, wp, nu, B0 = _ext_mk(doB0=1)
    out["ext_cpml"] = (p, wp, nu, B0,
                       rd.ExtParams(pmllen=12, tfsf_gap=8, ntf_gap=4, pml_m=3.0, kappa_max=5.0,
                                    alpha_max=0.05), None, None)
    # Tilted trail with log-varying density, magnetized (L&K, uniform nu), oblique
    # TM incidence at theta = 70, phi = 20 degrees: the 768x768x1536 set-up in small.
    p, wp, nu, B0 = _ext_mk(doB0=1, nu=3e4, metsize=(1e200, 1e200))
    wp3 = rd.tilted_trail_wp3(p.Nx, p.Ny, p.Nz, p.dx, 30.0, 0.8, 13.0, 15.0)
    out["ext_oblique_trail"] = (p, wp * 0, nu, B0,
                                rd.ExtParams(pmllen=8, tfsf_gap=6, ntf_gap=3, pml_m=3.0,
                                             kappa_max=5.0, alpha_max=0.05, oblique=1,
                                             exact_coords=1, lk_colocated=1,
                                             inc_theta=math.radians(70),
                                             inc_phi=math.radians(20)), wp3, None)
    # Unmagnetized collisional plasma sphere (per-cell maps), oblique TE incidence.
    p, wp, nu, B0 = _ext_mk(doB0=0, fntf=[40e6, 50e6, 60e6], metsize=(1e200, 1e200))
    wp3 = rd.plasma_sphere_wp3(p.Nx, p.Ny, p.Nz, p.dx, 2.0, 5e13)
    nu3 = np.full((p.Nx, p.Ny, p.Nz), 1e5)
    out["ext_sphere"] = (p, wp * 0, nu, (0.0, 0.0, 0.0),
                         rd.ExtParams(oblique=1, exact_coords=1, inc_theta=math.radians(30),
                                      inc_phi=math.radians(60), inc_psi=math.pi / 2),
                         wp3, nu3)
    # Collision frequency per cell with L&K (one matrix pair per cell), oblique.
    p, wp, nu, B0 = _ext_mk(N=(44, 44, 44), doB0=1, tsteps=120, metsize=(1e200, 1e200))
    rng = np.random.default_rng(11)
    nu3 = 2e4 + 6e4 * rng.random((p.Nx, p.Ny, p.Nz))
    wp3 = rd.tilted_trail_wp3(p.Nx, p.Ny, p.Nz, p.dx, 45.0, 1.0, 14.0, 15.0)
    out["ext_lk_cell"] = (p, wp * 0, nu, B0,
                          rd.ExtParams(oblique=1, inc_theta=math.radians(120),
                                       inc_phi=math.radians(-35), inc_psi=0.3), wp3, nu3)
    return out


def write_ext_case(d, case):
    """Write a full run directory (inputs + ext.dat + maps) for an ext case."""
    p, wp, nu, B0, ext, wp3, nu3 = case
    rd.write_rundir(d, p, wp, nu, B0)
    rd.write_ext(d, ext, wp3, nu3)


def trail_case(N=(48, 48, 48), steps=160):
    """Parametric trail (trail.dat): tilted 30 degrees, log10 n0 from 13 to 15,
    magnetized with the co-located Lee-Kalluri update, oblique incidence, the
    benchmark's CPML grading.  Returns (RunParams, wp, nu, B0, ExtParams,
    TrailParams)."""
    p, wp, nu, B0 = _ext_mk(N=N, doB0=1, nu=3e4, metsize=(1e200, 1e200), tsteps=steps)
    ext = rd.ExtParams(pmllen=8, tfsf_gap=6, ntf_gap=3, pml_m=3.0, kappa_max=5.0, alpha_max=0.05,
                       oblique=1, exact_coords=1, lk_colocated=1, inc_theta=math.radians(70),
                       inc_phi=math.radians(20))
    tr = rd.TrailParams.tilted(30.0, 0.8, 13.0, 15.0, 0.5 * (N[2] - 1) * p.dx)
    return p, wp * 0, nu, B0, ext, tr


def write_trail_case(d, case):
    p, wp, nu, B0, ext, tr = case
    rd.write_rundir(d, p, wp, nu, B0)
    rd.write_ext(d, ext)
    rd.write_trail(d, tr)


def plate_case(N=128, plate_wavelengths=3.0, steps=2000):
    """The reference's far-field calibration run (doplate = 1,
    analysis/meteorNTF.m:346-349) in reference-format inputs: a square PEC
    plate of side `plate_wavelengths` wavelengths at f0 = 100 MHz, 24 cells
    per wavelength, a Gaussian-modulated pulse along +x (E along z) of
    bandwidth f0 / 4, DFT at 0.8, 0.9, 1.0, 1.1 and 1.2 f0."""
    f0, gf = 100e6, 24.0
    lam = rd.C0 / f0
    dt = rd.stable_dt(lam / gf)
    fntf = list(np.array([0.8, 0.9, 1.0, 1.1, 1.2]) * f0)
    p = rd.RunParams(Nx=N, Ny=N, Nz=N, tsteps=steps, dt=dt, f0=f0,
                     fsig=1 / (2 * math.pi * 0.25 * f0 * dt), gridfactor=gf, numfiles=1,
                     savefields=0, fntf=fntf, doplate=1, platesize=plate_wavelengths * lam,
                     metsize=(1e200, 1e200), doB0=0, probex=[], probey=[], probez=[])
    return p, np.zeros((N, N)), np.zeros((N, N)), (0.0, 0.0, 0.0)


def plate_physical_optics(p):
    """sigma = 4 pi a^4 f^2 / vp^2, analysis/meteorNTF.m:347 (vp = 3e8 of the
    analysis constants)."""
    f = np.asarray(p.fntf, dtype=np.float64)
    return 4 * math.pi * p.platesize ** 4 * f ** 2 / 3e8 ** 2


def pec_sphere_case(N=128, radius=2.0, steps=2500):
    """The reference's sphere calibration run (doplate = 2: a sigma = 1e7
    conductor, source/meteor-2.1.cpp:200-206; compared with
    analysis/sphereRCSvsFreq.m by analysis/meteorNTF.m:350-352 and
    analysis/spherescattering.m) in reference-format inputs: radius 2 m at
    dx = 0.1 m (20 cells), a Gaussian-modulated pulse centred at 30 MHz with a
    10 MHz bandwidth, DFT at 20, 25, 30 and 35 MHz (ka from 0.84 to 1.47)."""
    f0, dx = 30e6, 0.1
    dt = rd.stable_dt(dx)
    p = rd.RunParams(Nx=N, Ny=N, Nz=N, tsteps=steps, dt=dt, f0=f0,
                     fsig=1 / (2 * math.pi * 10e6 * dt), gridfactor=(rd.C0 / f0) / dx, numfiles=1,
                     savefields=0, fntf=[20e6, 25e6, 30e6, 35e6], doplate=2, platesize=radius,
                     metsize=(1e200, 1e200), doB0=0, probex=[], probey=[], probez=[])
    return p, np.zeros((N, N)), np.zeros((N, N)), (0.0, 0.0, 0.0)

