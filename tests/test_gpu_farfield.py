"""GPU far-field projection against the FP64 numpy restatement of
analysis/meteorNTF.m and its bistatic generalisation (oracle/ntf_oracle.py)."""
import dataclasses
import math
import os
import sys

import numpy as np
import pytest

import cases as golden_cases
import helpers as H
from meteorscattering_gb300 import engine as E
from meteorscattering_gb300 import rundir as rd

sys.path.insert(0, os.path.join(H.ROOT, "oracle"))
import ntf_oracle as NO  # noqa: E402

pytestmark = pytest.mark.gpu


def _sim_for(case, form):
    p, wp, nu, B0 = case
    wp2 = np.asarray(wp).reshape(-1, order="F").reshape(p.Nx, p.Ny)
    nu2 = np.asarray(nu).reshape(-1, order="F").reshape(p.Nx, p.Ny)
    sim = E.Simulation(E.Problem.from_params(p, wp2, nu2, B0), form=form)
    sim.advance(p.tsteps)
    return sim


def _ntf_dict(sim, p):
    flat = sim.read_ntf()
    out = {"nntf": p.nntf, "ntfb": 15, "fntf": np.asarray(p.fntf, dtype=float)}
    nf2 = 2 * p.nntf
    out["Eydft"], out["Ezdft"] = flat[:nf2], flat[nf2:2 * nf2]
    o = 2 * nf2
    shapes = {"fb": (p.Ny, p.Nz), "tb": (p.Nx, p.Nz), "lr": (p.Nx, p.Ny)}
    for name, kind in rd.NTF_FACE_ORDER:
        a, b = shapes[kind]
        out[name] = flat[o:o + a * b * nf2].reshape(a, b, nf2)
        o += a * b * nf2
    return out


@pytest.mark.parametrize("name", ["sphere", "lk_trail", "rect"])
def test_far_field_fp64_matches_oracle(built, name):
    case = golden_cases.cases()[name]
    p = case[0]
    sim = _sim_for(case, E.FORM_FP64_PLAIN)
    rng = np.random.default_rng(3)
    th = np.concatenate([[math.pi / 2], rng.uniform(0, math.pi, 40)])
    ph = np.concatenate([[math.pi], rng.uniform(-math.pi, math.pi, 40)])
    got = sim.far_field(th, ph)
    want = NO.bistatic(_ntf_dict(sim, p), p.Nx, p.Ny, p.Nz, p.dx, th, ph)
    # relative L2 over every direction and frequency (the FP64 tolerance on
    # fields and RCS), and element-wise
    assert H.rel_l2(got[..., 0], want["sig"]) < 1e-12
    assert H.rel_l2(got[..., 1], want["sig_a"]) < 1e-12
    np.testing.assert_allclose(got[..., 0], want["sig"], rtol=1e-10)
    np.testing.assert_allclose(got[..., 1], want["sig_a"], rtol=1e-10, atol=1e-300)
    if p.Nx == p.Ny == p.Nz:  # the MATLAB itself assumes a cubic grid
        back = NO.meteorntf_backscatter(_ntf_dict(sim, p), p.Nx, p.dx)
        assert H.rel_l2(got[:, 0, 0], back["sig"]) < 1e-12
        np.testing.assert_allclose(got[:, 0, 0], back["sig"], rtol=1e-10)
    sim.close()


def test_far_field_theta_phi_grid_fp32_within_tenth_db(built):
    """FP32 fields + FP64 sums: RCS on a 10-degree theta/phi grid within 0.1 dB
    of the FP64 plain form wherever sigma is within 30 dB of its peak."""
    p, wp, nu, B0 = golden_cases.cases()["sphere"]
    p = dataclasses.replace(p, dt=rd.stable_dt(p.dx, 0.9), tsteps=240)
    case = (p, wp, nu, B0)
    th, ph = np.meshgrid(np.radians(np.arange(0, 181, 10)), np.radians(np.arange(0, 360, 10)),
                         indexing="ij")
    th, ph = th.ravel(), ph.ravel()
    s64 = _sim_for(case, E.FORM_FP64_PLAIN).far_field(th, ph)[..., 0]
    s32 = _sim_for(case, E.FORM_FP32_FUSED).far_field(th, ph)[..., 0]
    mask = s64 > s64.max() * 1e-3
    err_db = np.abs(10 * np.log10(s32[mask] / s64[mask]))
    assert err_db.max() < 0.1, err_db.max()


@pytest.mark.parametrize("name", ["sphere", "di_sine_ey"])
def test_far_field_tensor_cores_match_fp64(built, name):
    """Method 1 (stage 1 on the tensor cores, TF32 three-term split, FP32
    accumulation) against method 0 (FP64): within 0.01 dB wherever sigma is
    within 30 dB of its peak, on a theta/phi grid that makes the z faces a full
    GEMM (one distinct direction cosine per direction)."""
    p, wp, nu, B0 = golden_cases.cases()[name]
    p = dataclasses.replace(p, dt=rd.stable_dt(p.dx, 0.9), tsteps=240)
    sim = _sim_for((p, wp, nu, B0), E.FORM_FP64_PLAIN)
    th, ph = np.meshgrid(np.radians(np.arange(1, 180, 4)), np.radians(np.arange(0, 360, 4)),
                         indexing="ij")
    th, ph = th.ravel(), ph.ravel()
    s0 = sim.far_field(th, ph, method=0)[..., 0]
    s1 = sim.far_field(th, ph, method=1)[..., 0]
    mask = s0 > s0.max(axis=1, keepdims=True) * 1e-3
    err_db = np.abs(10 * np.log10(s1[mask] / s0[mask]))
    assert err_db.max() < 0.01, err_db.max()
    sim.close()


def test_far_field_tensor_cores_large_projection(built):
    """A large tensor-core projection: 20,000 random directions make every
    direction cosine distinct, so each face of a 96^3 grid gives a GEMM of
    about 470 128 x 128 tiles (more than two CTAs per SM).  Method 1 stays
    within 0.01 dB of method 0."""
    p, wp, nu, B0 = golden_cases._mk(N=(96, 96, 96), doplate=2, platesize=2.0, fntf=[50e6])
    p = dataclasses.replace(p, dt=rd.stable_dt(p.dx, 0.9), tsteps=320, numfiles=1, savefields=0)
    sim = _sim_for((p, wp, nu, B0), E.FORM_FP32_FUSED)
    rng = np.random.default_rng(17)
    th = np.arccos(rng.uniform(-1.0, 1.0, 20000))
    ph = rng.uniform(0.0, 2 * math.pi, 20000)
    s0 = sim.far_field(th, ph, method=0)[..., 0]
    s1 = sim.far_field(th, ph, method=1)[..., 0]
    mask = s0 > s0.max(axis=1, keepdims=True) * 1e-3
    assert mask.sum() > 1000
    err_db = np.abs(10 * np.log10(s1[mask] / s0[mask]))
    assert err_db.max() < 0.01, err_db.max()
    sim.close()
