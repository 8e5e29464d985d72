"""Random trail populations for batched sweeps and serving streams.

The reference fans trail studies out as independent PBS jobs generated by
MATLAB (setup/meteorbatch.m, setup/meteorrandom.m); here a population is a
list of in-memory problems drawn from one seed, with the distributions of the
batched-sweep configuration:

* grid nx = ny in {64, 80, ..., 256}, nz in {128, 160, ..., 512};
* radar frequency U(30, 60) MHz, dx = lambda / 20;
* density n0 log-uniform in [1e12, 1e16] m^-3, radius r0 U(0.3, 3) m,
  collision frequency log-uniform in [1e4, 1e6] 1/s;
* trail axis and incidence direction uniform on the upper hemisphere,
  polarisation angle U(0, pi);
* B0 = 5e-5 T dipped U(30, 80) degrees in the x-z plane;
* 10-cell CPML, 2500 steps.

The time step is the Courant step 0.5 dx / (c sqrt 3), shortened where the
densest plasma of the trail would make the explicit plasma update unstable
(omega_p dt must stay below 2; it is held at 1.2).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

from . import rundir as rd


@dataclasses.dataclass
class TrailJob:
    params: rd.RunParams
    ext: rd.ExtParams
    trail: rd.TrailParams
    B0: tuple
    nu: float

    @property
    def cells(self) -> int:
        p = self.params
        return p.Nx * p.Ny * p.Nz

    def problem(self, E):
        """Build the engine problem (``E`` = meteorscattering_gb300.engine)."""
        p = self.params
        wp2 = np.zeros((p.Nx, p.Ny))
        nu2 = np.full((p.Nx, p.Ny), self.nu)
        return E.Problem.from_params(p, wp2, nu2, self.B0).set_ext(self.ext).set_trail(self.trail)


def _hemisphere(rng) -> tuple:
    """Uniform direction with a non-negative z component: (theta, phi)."""
    cz = rng.uniform(0.0, 1.0)
    return math.acos(cz), rng.uniform(-math.pi, math.pi)


def random_trail(rng, steps: int = 2500, size: Optional[tuple] = None, pmllen: int = 10) -> TrailJob:
    if size is None:
        n = int(rng.choice(np.arange(64, 257, 16)))
        nz = int(rng.choice(np.arange(128, 513, 32)))
        size = (n, n, nz)
    Nx, Ny, Nz = size
    f0 = rng.uniform(30e6, 60e6)
    gf = 20.0
    dx = rd.C0 / f0 / gf
    log_n0 = rng.uniform(12.0, 16.0)
    r0 = rng.uniform(0.3, 3.0)
    nu = 10 ** rng.uniform(4.0, 6.0)
    ath, aph = _hemisphere(rng)
    ith, iph = _hemisphere(rng)
    psi = rng.uniform(0.0, math.pi)
    dip = math.radians(rng.uniform(30.0, 80.0))
    B0 = (5e-5 * math.cos(dip), 0.0, -5e-5 * math.sin(dip))
    wp_max = float(rd.plasma_frequency(10 ** log_n0))
    dt = min(rd.stable_dt(dx), 1.2 / wp_max)
    axis = (math.sin(ath) * math.cos(aph), math.sin(ath) * math.sin(aph), math.cos(ath))
    trail = rd.TrailParams(centre=(0.0, 0.0, 0.0), axis=axis, r0=r0, log10n_lo=log_n0,
                           log10n_hi=log_n0, s_half=1.0)
    ext = rd.ExtParams(pmllen=pmllen, oblique=1, exact_coords=1, lk_colocated=1, inc_theta=ith,
                       inc_phi=iph, inc_psi=psi)
    p = rd.RunParams(Nx=Nx, Ny=Ny, Nz=Nz, tsteps=steps, dt=dt, f0=f0, fsig=20.0, gridfactor=gf,
                     numfiles=1, savefields=0, probex=[], probey=[], probez=[], fntf=[f0],
                     metsize=(1e200, 1e200), doB0=1)
    return TrailJob(p, ext, trail, B0, nu)


def population(n: int, seed: int = 0, steps: int = 2500, big_fraction: float = 0.0,
               big_size=(384, 384, 768)) -> List[TrailJob]:
    """`n` trails from one seed; a fraction `big_fraction` of them on the large
    grid `big_size` (the serving-stream mix)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        big = rng.uniform() < big_fraction
        out.append(random_trail(rng, steps, big_size if big else None))
    return out


def direction_grid(step_deg: float):
    """theta in [0, 180], phi in [0, 360) on a regular grid (radians)."""
    th = np.radians(np.arange(0.0, 180.0 + 1e-9, step_deg))
    ph = np.radians(np.arange(0.0, 360.0, step_deg))
    T, P = np.meshgrid(th, ph, indexing="ij")
    return T.ravel(), P.ravel()
