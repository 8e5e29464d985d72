"""Far-field (near-to-far-field) projection oracle -- TEST INFRASTRUCTURE ONLY.

FP64 numpy restatements used to check the engine's far-field projection:

* :func:`meteorntf_backscatter` restates ``analysis/meteorNTF.m`` line by line
  (read-out of output_NTF.dat :12-57, trimming and edge halving :66-196,
  phasors ``1i*sin + cos`` :202-230, x-only distances :236-246, face integrals
  :253-304, theta/phi components :311-314, cross sections :319-332).  Like the
  MATLAB it uses ``in.Nx`` for every trim, so it is only meaningful on cubic
  grids, and it uses the analysis constants of ``analysis/loadconstants.m``
  (eps0 = 8.845e-12, mu0 = 4e-7*pi), not the solver's.
* :func:`bistatic` generalises it to any direction (theta from +z, phi from +x)
  and any grid shape: every tangential current sample sits at its Yee position
  (half-cell offsets as in the MATLAB distances), with the MATLAB's trapezoid
  edge weights, and the phase factor is exp(-j k r_hat . r').  At
  theta = 90 deg, phi = 180 deg (observer along -x) it reduces to the MATLAB
  backscatter result.
"""
from __future__ import annotations

import math
from typing import Dict, Sequence

import numpy as np

# analysis/loadconstants.m:3-10
U0_ANALYSIS = 4 * math.pi * 1e-7
E0_ANALYSIS = 8.845e-12
VP = math.sqrt(1.0 / (U0_ANALYSIS * E0_ANALYSIS))
ETA0 = math.sqrt(U0_ANALYSIS / E0_ANALYSIS)


def _phasor(X: np.ndarray) -> np.ndarray:
    """[..., 2*nntf] interleaved (sin, cos) -> complex [nntf, ...] = 1i*sin + cos."""
    Z = 1j * X[..., 0::2] + X[..., 1::2]
    return np.moveaxis(Z, -1, 0)


def _trim(X: np.ndarray, N: int, ntfb: int, kind: str) -> np.ndarray:
    """Apply the MATLAB trim + edge halving to a C-shaped [a][b][2n] array.

    kind 'A': b in [ntfb, N-ntfb-1], a in [ntfb, N-ntfb], halve a-edges
              (MATLAB X(:, ntfb+1:N-ntfb, ntfb+1:N-ntfb+1), dim-3 ends).
    kind 'B': b in [ntfb, N-ntfb],   a in [ntfb, N-ntfb-1], halve b-edges.
    Returns complex [nntf, a, b]."""
    if kind == "A":
        Y = X[ntfb:N - ntfb + 1, ntfb:N - ntfb, :].copy()
        Y[0] *= 0.5
        Y[-1] *= 0.5
    else:
        Y = X[ntfb:N - ntfb, ntfb:N - ntfb + 1, :].copy()
        Y[:, 0] *= 0.5
        Y[:, -1] *= 0.5
    return _phasor(Y)


def meteorntf_backscatter(ntf: Dict[str, np.ndarray], Nx: int, dx: float,
                          dy: float = None, dz: float = None) -> Dict[str, np.ndarray]:
    """Backscatter cross sections exactly as analysis/meteorNTF.m computes them."""
    dy = dx if dy is None else dy
    dz = dx if dz is None else dz
    N, ntfb, nntf = Nx, int(ntf["ntfb"]), int(ntf["nntf"])
    fntf = np.asarray(ntf["fntf"], dtype=np.float64)
    T = {}
    for name, kind in (("My_front", "A"), ("My_back", "A"), ("Jz_front", "A"), ("Jz_back", "A"),
                       ("Mz_front", "B"), ("Mz_back", "B"), ("Jy_front", "B"), ("Jy_back", "B"),
                       ("Mx_top", "A"), ("Mx_bot", "A"), ("Jz_top", "A"), ("Jz_bot", "A"),
                       ("Mz_top", "B"), ("Mz_bot", "B"), ("Jx_top", "B"), ("Jx_bot", "B"),
                       ("Mx_left", "A"), ("Mx_right", "A"), ("Jy_left", "A"), ("Jy_right", "A"),
                       ("My_left", "B"), ("My_right", "B"), ("Jx_left", "B"), ("Jx_right", "B")):
        T[name] = _trim(ntf[name], N, ntfb, kind)
    Ez_src = 1j * ntf["Ezdft"][0::2] + ntf["Ezdft"][1::2]
    Ey_src = 1j * ntf["Eydft"][0::2] + ntf["Eydft"][1::2]

    # distances (x only), analysis/meteorNTF.m:236-246; [a] index along x
    d_front, d_back = ntfb * dx, (N - ntfb) * dx
    x1 = np.arange(ntfb, N - ntfb + 1) * dx          # top1/left1 (type A, a = i)
    x2 = np.arange(ntfb, N - ntfb) * dx + dx / 2     # top2/left2 (type B, a = i)

    out = {k: np.zeros(nntf, dtype=complex) for k in ("Lx", "Ly", "Lz", "Nx", "Ny", "Nz")}
    for m in range(nntf):
        k = 2 * math.pi * fntf[m] / VP
        e1 = np.exp(1j * k * x1)[:, None]   # broadcast over b
        e2 = np.exp(1j * k * x2)[:, None]
        ef, eb = np.exp(1j * k * d_front), np.exp(1j * k * d_back)
        s = lambda X, e, area: np.sum(X[m] * area * e)
        out["Lx"][m] = (s(T["Mx_top"], e1, dx * dz) + s(T["Mx_bot"], e1, dx * dz) +
                        s(T["Mx_left"], e1, dx * dy) + s(T["Mx_right"], e1, dx * dy))
        out["Ly"][m] = (s(T["My_front"], ef, dy * dz) + s(T["My_back"], eb, dy * dz) +
                        s(T["My_left"], e2, dx * dy) + s(T["My_right"], e2, dx * dy))
        out["Lz"][m] = (s(T["Mz_front"], ef, dy * dz) + s(T["Mz_back"], eb, dy * dz) +
                        s(T["Mz_top"], e2, dx * dz) + s(T["Mz_bot"], e2, dx * dz))
        out["Nx"][m] = (s(T["Jx_top"], e2, dx * dz) + s(T["Jx_bot"], e2, dx * dz) +
                        s(T["Jx_left"], e2, dx * dy) + s(T["Jx_right"], e2, dx * dy))
        out["Ny"][m] = (s(T["Jy_front"], ef, dy * dz) + s(T["Jy_back"], eb, dy * dz) +
                        s(T["Jy_left"], e1, dx * dy) + s(T["Jy_right"], e1, dx * dy))
        out["Nz"][m] = (s(T["Jz_front"], ef, dy * dz) + s(T["Jz_back"], eb, dy * dz) +
                        s(T["Jz_top"], e1, dx * dz) + s(T["Jz_bot"], e1, dx * dz))
    Lth, Lph, Nth, Nph = -out["Lz"], -out["Ly"], -out["Nz"], -out["Ny"]
    Eth, Eph = -Ez_src, -Ey_src
    Pinc = (np.abs(Eth) ** 2 + np.abs(Eph) ** 2) / 2 / ETA0
    kk = 2 * math.pi * fntf / VP
    with np.errstate(divide="ignore", invalid="ignore"):
        sig = {
            "thth": kk ** 2 / (4 * math.pi) * np.abs(Lph + ETA0 * Nth) ** 2 / np.abs(Eth) ** 2,
            "phth": kk ** 2 / (4 * math.pi) * np.abs(Lth - ETA0 * Nph) ** 2 / np.abs(Eth) ** 2,
            "phph": kk ** 2 / (4 * math.pi) * np.abs(Lth - ETA0 * Nph) ** 2 / np.abs(Eph) ** 2,
            "thph": kk ** 2 / (4 * math.pi) * np.abs(Lph + ETA0 * Nth) ** 2 / np.abs(Eph) ** 2,
            "sig": kk ** 2 / (8 * math.pi * ETA0) * (np.abs(Lph + ETA0 * Nth) ** 2 +
                                                     np.abs(Lth - ETA0 * Nph) ** 2) / np.abs(Pinc),
        }
    sig.update(out)
    return sig


# --------------------------------------------------------------------------
# Bistatic generalisation

# (face, component, kind, position offsets of the sample in cells along
# (a, b), the fixed coordinate of the face) -- a/b axes per face:
# front/back: a = j (y), b = k (z); top/bot: a = i (x), b = k (z);
# left/right: a = i (x), b = j (y).
_FACES = {
    "front": ("x", "y", "z"), "back": ("x", "y", "z"),
    "top": ("y", "x", "z"), "bot": ("y", "x", "z"),
    "left": ("z", "x", "y"), "right": ("z", "x", "y"),
}
# component -> (vector kind 'M' or 'J', axis, trim kind); half offsets follow
# the trim kind: type A samples sit at integer a and half-integer b, type B at
# half-integer a and integer b.
_COMPS = {
    "front": (("My", "A"), ("Mz", "B"), ("Jy", "B"), ("Jz", "A")),
    "back": (("My", "A"), ("Mz", "B"), ("Jy", "B"), ("Jz", "A")),
    "top": (("Mx", "A"), ("Mz", "B"), ("Jx", "B"), ("Jz", "A")),
    "bot": (("Mx", "A"), ("Mz", "B"), ("Jx", "B"), ("Jz", "A")),
    "left": (("Mx", "A"), ("My", "B"), ("Jx", "B"), ("Jy", "A")),
    "right": (("Mx", "A"), ("My", "B"), ("Jx", "B"), ("Jy", "A")),
}


def face_samples(ntf: Dict[str, np.ndarray], Nx: int, Ny: int, Nz: int, dx: float, dy: float,
                 dz: float):
    """Yield (vec 'M'/'J', axis 'x'/'y'/'z', complex values [nntf, A, B] with
    area and edge weights applied, coordinates (X, Y, Z) each broadcastable
    to [A, B]) for the 24 face arrays, trimmed on the true grid extents."""
    ntfb = int(ntf["ntfb"])
    dims = {"x": Nx, "y": Ny, "z": Nz}
    h = {"x": dx, "y": dy, "z": dz}
    for face, (n_ax, a_ax, b_ax) in _FACES.items():
        Na, Nb = dims[a_ax], dims[b_ax]
        high = face in ("back", "top", "right")
        n_pos = ((dims[n_ax] - ntfb) if high else ntfb) * h[n_ax]
        area = h[a_ax] * h[b_ax]
        for comp, kind in _COMPS[face]:
            X = ntf[f"{comp}_{face}"]
            if kind == "A":
                ar = np.arange(ntfb, Na - ntfb + 1)
                br = np.arange(ntfb, Nb - ntfb)
                Y = X[ntfb:Na - ntfb + 1, ntfb:Nb - ntfb, :].copy()
                Y[0] *= 0.5
                Y[-1] *= 0.5
                apos, bpos = ar * h[a_ax], (br + 0.5) * h[b_ax]
            else:
                ar = np.arange(ntfb, Na - ntfb)
                br = np.arange(ntfb, Nb - ntfb + 1)
                Y = X[ntfb:Na - ntfb, ntfb:Nb - ntfb + 1, :].copy()
                Y[:, 0] *= 0.5
                Y[:, -1] *= 0.5
                apos, bpos = (ar + 0.5) * h[a_ax], br * h[b_ax]
            coords = {n_ax: np.full((1, 1), n_pos), a_ax: apos[:, None], b_ax: bpos[None, :]}
            yield comp[0], comp[1].lower(), _phasor(Y) * area, (coords["x"], coords["y"], coords["z"])


def bistatic(ntf: Dict[str, np.ndarray], Nx: int, Ny: int, Nz: int, dx: float,
             theta: Sequence[float], phi: Sequence[float], dy: float = None,
             dz: float = None) -> Dict[str, np.ndarray]:
    """Bistatic cross sections sigma[nntf, ndir] (m^2) for directions
    (theta[d], phi[d]) in radians, with the MATLAB's normalisation by the
    source-DFT incident power."""
    dy = dx if dy is None else dy
    dz = dx if dz is None else dz
    th = np.asarray(theta, dtype=np.float64)
    ph = np.asarray(phi, dtype=np.float64)
    rx, ry, rz = np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)
    fntf = np.asarray(ntf["fntf"], dtype=np.float64)
    nntf, nd = len(fntf), len(th)
    acc = {v + a: np.zeros((nntf, nd), dtype=complex) for v in "LN" for a in "xyz"}
    key = {"M": "L", "J": "N"}
    for vec, ax, vals, (X, Y, Z) in face_samples(ntf, Nx, Ny, Nz, dx, dy, dz):
        for m in range(nntf):
            k = 2 * math.pi * fntf[m] / VP
            for d in range(nd):
                phase = np.exp(-1j * k * (rx[d] * X + ry[d] * Y + rz[d] * Z))
                acc[key[vec] + ax][m, d] += np.sum(vals[m] * phase)
    ct, st, cp, sp = np.cos(th), np.sin(th), np.cos(ph), np.sin(ph)
    Lth = acc["Lx"] * ct * cp + acc["Ly"] * ct * sp - acc["Lz"] * st
    Lph = -acc["Lx"] * sp + acc["Ly"] * cp
    Nth = acc["Nx"] * ct * cp + acc["Ny"] * ct * sp - acc["Nz"] * st
    Nph = -acc["Nx"] * sp + acc["Ny"] * cp
    Ez_src = 1j * ntf["Ezdft"][0::2] + ntf["Ezdft"][1::2]
    Ey_src = 1j * ntf["Eydft"][0::2] + ntf["Eydft"][1::2]
    Pinc = (np.abs(Ez_src) ** 2 + np.abs(Ey_src) ** 2) / 2 / ETA0
    kk = (2 * math.pi * fntf / VP)[:, None]
    c = kk ** 2 / (8 * math.pi * ETA0) / np.abs(Pinc)[:, None]
    A = c * np.abs(Lph + ETA0 * Nth) ** 2
    B = c * np.abs(Lth - ETA0 * Nph) ** 2
    return {"sig": A + B, "sig_a": A, "sig_b": B, "Lth": Lth, "Lph": Lph, "Nth": Nth, "Nph": Nph}
