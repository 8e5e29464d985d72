"""GPU: record slices read from the device state, total and scattered
(mfdtd_sim_read_slices; the subtraction analysis/plotMresults.m:210-234 does
on the host).

* Layout: the total-field slices equal the matching planes of the full
  field components, value for value.
* With no scatterer the scattered field is what the TF/SF surface leaks: at
  normal incidence in FP64 that is round-off (the 1-D line and the grid run
  the same update), so any node placed on the wrong side of the box would
  show the full incident amplitude; at oblique incidence it is the
  interpolated line's leakage (-57 to -63 dB on this grid, below 1e-2 of the
  amplitude).
* FP32 and FP64 slices of a plasma case agree to 1e-3 relative L2.
"""
import dataclasses
import math

import numpy as np
import pytest

import cases as golden_cases
import helpers as H
from meteorscattering_gb300 import engine as E
from meteorscattering_gb300 import rundir as rd

pytestmark = pytest.mark.gpu


# The 48^3 grid's TF/SF box is 8 cells wide (10-cell CPML and gap); a pulse
# of fsig = 15 steps, delayed 45 steps, is over the box centre around step 90
# at normal incidence and step 120 at (60, 25) degrees, when the slices are read.
STEPS = {False: 90, True: 120}


def _empty(oblique):
    p, wp, nu, B0 = golden_cases._mk(n0=0.0, doB0=0)
    p = dataclasses.replace(p, dt=rd.stable_dt(p.dx, 0.9), tsteps=STEPS[oblique], numfiles=1, fsig=15.0)
    pb = E.Problem.from_params(p, np.zeros((p.Nx, p.Ny)), np.full((p.Nx, p.Ny), 5e4), B0)
    if oblique:
        pb.set_ext(rd.ExtParams(oblique=1, inc_theta=math.radians(60), inc_phi=math.radians(25)))
    return p, pb


def _run(pb, form, steps):
    s = E.Simulation(pb, form=form)
    s.advance(steps)
    return s


def _amax(planes):
    return max(np.abs(v).max() for v in planes.values())


@pytest.mark.parametrize("form", [E.FORM_FP64_PLAIN, E.FORM_FP32_FUSED])
def test_slices_are_the_field_planes(built, form):
    p, pb = _empty(False)
    s = _run(pb, form, STEPS[False])
    Et, Ht = s.read_slices()
    ssx, ssy, ssz = (p.Nx + 1) // 2, (p.Ny + 1) // 2, (p.Nz + 1) // 2
    ey, ez, hy, hz = (s.read_field(c) for c in (1, 2, 4, 5))
    assert np.array_equal(Et["z"][0], ey[:, :, ssz]) and np.array_equal(Et["z"][1], ez[:, :, ssz])
    assert np.array_equal(Et["y"][0], ey[:, ssy, :]) and np.array_equal(Et["x"][1], ez[ssx, :, :])
    assert np.array_equal(Ht["z"][0][:, :-1], hy[:, :-1, ssz]) and np.all(Ht["z"][0][:, -1] == 0)
    assert np.array_equal(Ht["x"][1][:-1, :-1], hz[ssx, :-1, :-1])
    assert _amax(Et) > 0.1      # the pulse is in the grid
    s.close()


def test_scattered_field_of_an_empty_grid_is_round_off(built):
    p, pb = _empty(False)
    s = _run(pb, E.FORM_FP64_PLAIN, STEPS[False])
    Et, Ht = s.read_slices()
    Es, Hs = s.read_slices(scattered=True)
    assert _amax(Et) > 0.1 and _amax(Ht) > 1e-4
    assert _amax(Es) < 1e-10 * _amax(Et), _amax(Es)
    assert _amax(Hs) < 1e-10 * _amax(Ht), _amax(Hs)
    s.close()


@pytest.mark.parametrize("form", [E.FORM_FP64_PLAIN, E.FORM_FP32_FUSED])
def test_scattered_field_of_an_empty_grid_oblique(built, form):
    p, pb = _empty(True)
    s = _run(pb, form, STEPS[True])
    Et, Ht = s.read_slices()
    Es, Hs = s.read_slices(scattered=True)
    assert _amax(Et) > 0.1
    assert _amax(Es) < 1e-2 * _amax(Et), _amax(Es) / _amax(Et)
    assert _amax(Hs) < 1e-2 * _amax(Ht), _amax(Hs) / _amax(Ht)
    s.close()


def test_fp32_slices_match_fp64(built):
    p, wp, nu, B0 = golden_cases.cases()["di_sine_ey"]
    p = dataclasses.replace(p, dt=rd.stable_dt(p.dx, 0.9), tsteps=120, numfiles=1)
    wp2 = np.asarray(wp).reshape(-1, order="F").reshape(p.Nx, p.Ny)
    nu2 = np.asarray(nu).reshape(-1, order="F").reshape(p.Nx, p.Ny)
    out = {}
    for form in (E.FORM_FP64_PLAIN, E.FORM_FP32_FUSED):
        s = _run(E.Problem.from_params(p, wp2, nu2, B0), form, 120)
        out[form] = [np.concatenate([v.ravel() for v in d.values()]) for sc in (False, True)
                     for d in s.read_slices(scattered=sc)]
        s.close()
    for a, b in zip(out[E.FORM_FP32_FUSED], out[E.FORM_FP64_PLAIN]):
        assert np.abs(b).max() > 0
        assert H.rel_l2(a, b) < 1e-3
