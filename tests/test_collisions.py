"""CPU: the collision-frequency model of the input generator
(meteorscattering_gb300/collisions.py, restating setup/meteorCollisions.m).

There is no MATLAB here to produce known answers, so the checks are closed
forms: on an exponential atmosphere sampled every 2 km, heights on a sample
need no interpolation, and every term is a one-line formula of the sample.
Between samples the interpolation must stay between its neighbours (the
shape-preserving property of MATLAB's 'cubic'/'pchip')."""
import math

import numpy as np
import pytest

from meteorscattering_gb300 import collisions as C

H_KM = np.arange(0.0, 202.0, 2.0)


def test_electron_neutral_closed_form():
    atm = C.isothermal_profile(H_KM, n_ground_cm3=2.5e19, scale_height_km=7.0, temp_k=250.0)
    for alt_km in (80.0, 100.0, 120.0):
        got = C.collision_frequencies(np.zeros(1), alt_km * 1e3, atm)["en"]
        mobility = C.SEA_LEVEL_MOBILITY * math.exp(alt_km / 7.0)    # n(0) / n(alt)
        want = C.QE_SETUP / (C.ME_SETUP * mobility)
        assert got == pytest.approx(want, rel=1e-12)


def test_coulomb_terms_closed_form():
    atm = C.isothermal_profile(H_KM, temp_k=200.0)
    wp = np.array([[0.0, 1e8], [3e8, 2e9]])
    c = C.collision_frequencies(wp, 100e3, atm)
    te = 200.0 * C.KB_SETUP / C.QE_SETUP
    ne = wp ** 2 * C.ME_SETUP * C.E0_SETUP / C.QE_SETUP ** 2
    base = 6.6e-11 * ne * te ** -1.5 * (20.0 / 17.0)
    np.testing.assert_allclose(c["ee"], base, rtol=1e-12)
    np.testing.assert_allclose(c["ei"], base * math.sqrt(C.ME_SETUP / C.MI_SETUP), rtol=1e-12)
    assert c["Te"] == pytest.approx(te, rel=1e-15)
    # nu.dat = en + ee + ei, element by element, same shape as the map
    nu = C.collision_map(wp, 100e3, atm)
    assert nu.shape == wp.shape
    np.testing.assert_allclose(nu, c["en"] + c["ee"] + c["ei"], rtol=1e-15)
    assert nu[0, 0] == pytest.approx(c["en"], rel=1e-15)   # no plasma: neutral collisions only


def test_interpolation_is_shape_preserving():
    rng = np.random.default_rng(3)
    t = np.zeros((H_KM.size, len(C.COLUMNS)))
    t[:, 0] = H_KM
    t[:, 1:] = np.exp(rng.normal(size=(H_KM.size, 9)).cumsum(axis=0) * 0.3)   # positive, wiggly
    atm = C.AtmosphereProfile(t)
    x = H_KM[:-1] + rng.random(H_KM.size - 1) * 2.0
    got = atm.at(x)
    for c, name in enumerate(C.COLUMNS[1:], start=1):
        lo = np.minimum(t[:-1, c], t[1:, c])
        hi = np.maximum(t[:-1, c], t[1:, c])
        assert np.all(got[name] >= lo * (1 - 1e-12)) and np.all(got[name] <= hi * (1 + 1e-12)), name
    np.testing.assert_allclose(atm.at(H_KM)["o"], t[:, 1], rtol=1e-14)   # exact on the samples
    assert np.allclose(got["total"], sum(got[s] for s in C.SPECIES))


def test_profile_from_matlab_style_text(tmp_path):
    atm = C.isothermal_profile(H_KM[:6])
    lines = ["% height O N2 O2 mass T He Ar H N", ""]
    for row in atm.table:
        lines.append("  " + "  ".join(f"{v:.6e}" for v in row) + ";")
    p = tmp_path / "msis.txt"
    p.write_text("\n".join(lines) + "\n")
    back = C.AtmosphereProfile.from_file(str(p))
    np.testing.assert_allclose(back.table, atm.table, rtol=1e-6)


def test_profile_validation():
    with pytest.raises(ValueError):
        C.AtmosphereProfile(np.zeros((3, 4)))
    t = C.isothermal_profile(H_KM[:4]).table.copy()
    t[2, 0] = t[1, 0]
    with pytest.raises(ValueError):
        C.AtmosphereProfile(t)
