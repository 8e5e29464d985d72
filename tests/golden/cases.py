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
