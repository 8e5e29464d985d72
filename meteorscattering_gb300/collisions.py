"""Collision frequencies of the trail plasma, restating ``setup/meteorCollisions.m``.

The reference builds ``nu.dat`` (``setup/meteorrun.m:101-112``) as the sum of
three collision frequencies per column of the trail map:

* electron-neutral, from the electron mobility at sea level scaled by the
  neutral number density at the altitude (``meteorCollisions.m:11-19``);
* electron-ion and electron-electron (Coulomb) collisions, from the electron
  density the plasma frequency implies and the neutral temperature at the
  altitude, with a Coulomb logarithm of 20 (``meteorCollisions.m:22-47``).

The neutral atmosphere is an input.  The reference reads it from an MSIS-E-90
profile table embedded in ``setup/MSISatmosphere1.m``, interpolated with
MATLAB's ``interp1(..., 'cubic')`` (``MSISatmosphere1.m:238-250``).  Here the
profile is the caller's: :class:`AtmosphereProfile` takes the same ten columns
(the layout of an MSIS-E-90 model output) from arrays or a text file and
interpolates them the same way (piecewise cubic Hermite, shape preserving:
MATLAB's ``'cubic'`` is its ``'pchip'``, which ``scipy.interpolate.
PchipInterpolator`` implements with the same one-sided end slopes).

Constants are the set-up scripts' own (``setup/loadconstants.m:3-10``), which
differ from the solver's (``source/meteor-2.1.cpp:12-18``).
"""
from __future__ import annotations

import dataclasses
from typing import Dict, Sequence

import numpy as np

# setup/loadconstants.m
E0_SETUP = 8.845e-12
QE_SETUP = 1.6e-19
ME_SETUP = 9.11e-31
MI_SETUP = 5.0e-26      # NO+ ion
KB_SETUP = 1.38065e-23

# meteorCollisions.m
SEA_LEVEL_MOBILITY = 1.4856   # electron mobility at the ground, m^2 / (V s)
COULOMB_LOG = 20.0
CALLEN_COEFF = 6.6e-11        # J. D. Callen, Fundamentals of Plasma Physics (2006), eq. 2.86

# Column order of an MSIS-E-90 profile (MSISatmosphere1.m:13-22).
COLUMNS = ("height_km", "o", "n2", "o2", "mass", "temp", "he", "ar", "h", "n")
SPECIES = ("o", "n2", "o2", "he", "ar", "h", "n")   # the number densities summed into "total"


@dataclasses.dataclass
class AtmosphereProfile:
    """Neutral atmosphere versus height: number densities in cm^-3, mass
    density in g cm^-3, temperature in K, heights in km (strictly increasing)."""

    table: np.ndarray   # [rows][10] in COLUMNS order

    def __post_init__(self):
        t = np.asarray(self.table, dtype=np.float64)
        if t.ndim != 2 or t.shape[1] != len(COLUMNS) or t.shape[0] < 2:
            raise ValueError(f"an atmosphere table has {len(COLUMNS)} columns {COLUMNS} and >= 2 rows")
        if np.any(np.diff(t[:, 0]) <= 0):
            raise ValueError("heights must be strictly increasing")
        self.table = t

    @classmethod
    def from_file(cls, path: str) -> "AtmosphereProfile":
        """Whitespace-separated rows in COLUMNS order; lines starting with
        '%' or '#' are comments (an MSIS-E-90 text output pasted as is)."""
        rows = []
        with open(path) as f:
            for line in f:
                s = line.strip().rstrip(";")
                if not s or s[0] in "%#":
                    continue
                rows.append([float(v) for v in s.replace(";", " ").split()])
        return cls(np.array(rows))

    def at(self, height_km) -> Dict[str, np.ndarray]:
        """Every column interpolated at ``height_km`` (MSISatmosphere1.m:238-248),
        plus ``total`` = the sum of the species number densities (:250)."""
        from scipy.interpolate import PchipInterpolator
        h = self.table[:, 0]
        x = np.asarray(height_km, dtype=np.float64)
        out = {}
        for c, name in enumerate(COLUMNS[1:], start=1):
            out[name] = PchipInterpolator(h, self.table[:, c], extrapolate=True)(x)
        out["total"] = sum(out[s] for s in SPECIES)
        return out


def electron_density(wp: np.ndarray) -> np.ndarray:
    """n_e = wp^2 ME e0 / QE^2 in m^-3 (meteorCollisions.m:24)."""
    wp = np.asarray(wp, dtype=np.float64)
    return wp * wp * ME_SETUP * E0_SETUP / QE_SETUP ** 2


def collision_frequencies(wp: np.ndarray, altitude_m: float,
                          atmosphere: AtmosphereProfile) -> Dict[str, np.ndarray]:
    """Electron-neutral (``en``, a scalar), electron-ion (``ei``) and
    electron-electron (``ee``) collision frequencies in 1/s for the plasma
    frequency map ``wp`` (rad/s) at ``altitude_m``, and the electron
    temperature ``Te`` in eV (meteorCollisions.m:4-47).  Products are taken
    in the reference's order."""
    n0 = atmosphere.at(0.0)
    nd = atmosphere.at(altitude_m / 1e3)
    mobility = SEA_LEVEL_MOBILITY * n0["total"] / nd["total"]
    en = QE_SETUP / (ME_SETUP * mobility)
    ni = electron_density(wp)          # singly charged ions, quasi-neutral
    te = nd["temp"] * KB_SETUP / QE_SETUP
    z = 1.0
    ei = CALLEN_COEFF * ni * z ** 2 * (MI_SETUP / ME_SETUP) ** -0.5 * te ** -1.5 * (COULOMB_LOG / 17.0)
    ee = CALLEN_COEFF * ni * z ** 2 * (ME_SETUP / ME_SETUP) ** -0.5 * te ** -1.5 * (COULOMB_LOG / 17.0)
    return {"en": float(en), "ei": ei, "ee": ee, "Te": float(te)}


def collision_map(wp: np.ndarray, altitude_m: float, atmosphere: AtmosphereProfile) -> np.ndarray:
    """The ``nu`` map ``meteorrun.m`` writes to nu.dat: en + ee + ei per
    entry of ``wp`` (setup/meteorrun.m:105-106), same shape as ``wp``."""
    c = collision_frequencies(wp, altitude_m, atmosphere)
    return c["en"] + c["ee"] + c["ei"]


def isothermal_profile(heights_km: Sequence[float], n_ground_cm3: float = 2.55e19,
                       scale_height_km: float = 7.0, temp_k: float = 250.0) -> AtmosphereProfile:
    """A synthetic exponential atmosphere (all neutrals as N2), for tests and
    for runs without a measured profile."""
    h = np.asarray(heights_km, dtype=np.float64)
    t = np.zeros((h.size, len(COLUMNS)))
    t[:, 0] = h
    t[:, 2] = n_ground_cm3 * np.exp(-h / scale_height_km)
    t[:, 4] = t[:, 2] * 28 * 1.6605e-24
    t[:, 5] = temp_k
    return AtmosphereProfile(t)
