"""Extended inputs (ext.dat): the oracle's extensions checked by physics, and
the host-side handling of the new inputs (no GPU).

The reference cannot express these inputs (configurable CPML, TF/SF and
Huygens offsets, oblique incidence, per-cell plasma maps), so the oracle's
extension is validated by properties instead of golden vectors:
  * an ext.dat holding the reference's values changes no output byte;
  * a plane wave injected obliquely through the total-field/scattered-field
    box leaves the scattered-field region empty (leakage below -50 dB);
  * at normal incidence the oblique machinery reproduces the reference's own
    x-directed line;
  * the reference's Lee-Kalluri update grows without bound in a magnetized
    trail, while the co-located variant stays bounded.
"""
import dataclasses
import math
import os
import shutil

import numpy as np
import pytest

import cases as golden_cases
import helpers as H
from meteorscattering_gb300 import engine as E
from meteorscattering_gb300 import rundir as rd


def _run(tmp_path, name, p, wp, nu, B0, ext=None, wp3=None, nu3=None):
    d = os.path.join(str(tmp_path), name)
    shutil.rmtree(d, ignore_errors=True)
    rd.write_rundir(d, p, wp, nu, B0)
    if ext is not None:
        rd.write_ext(d, ext, wp3, nu3)
    H.run_oracle(d)
    return d


def test_ext_with_reference_values_changes_nothing(built, tmp_path):
    p, wp, nu, B0 = golden_cases.cases()["lk_trail"]
    da = _run(tmp_path, "plain", p, wp, nu, B0)
    db = _run(tmp_path, "ext", p, wp, nu, B0, rd.ExtParams())
    assert H.diff_outputs(da, db, p.nntf) == []


def _leakage_db(tmp_path, ext, N=56, steps=260):
    p, wp, nu, B0 = golden_cases._mk(N=(N, N, N), doB0=0, fsig=20.0, tsteps=steps,
                                     numfiles=steps // 4, metsize=(1e200, 1e200),
                                     dt=rd.stable_dt(0.25, 0.9), savefields=1)
    d = _run(tmp_path, "leak", p, wp * 0, nu, B0, ext)
    recs = rd.read_slices(os.path.join(d, "output_E.dat"), p, True)
    L, g = ext.pmllen, ext.tfsf_gap
    b1, b2 = L + g, N - L - g
    tf = np.zeros((N, N), bool)
    tf[b1 + 1:b2 - 1, b1 + 1:b2 - 1] = True
    sf = np.zeros((N, N), bool)
    sf[L + 2:N - L - 2, L + 2:N - L - 2] = True
    sf[b1 - 2:b2 + 2, b1 - 2:b2 + 2] = False
    mt = max(np.abs(r["z"][c][tf]).max() for r in recs for c in (0, 1))
    ms = max(np.abs(r["z"][c][sf]).max() for r in recs for c in (0, 1))
    assert mt > 0.3  # the incident pulse is inside the box
    return 20 * math.log10(ms / mt)


@pytest.mark.parametrize("theta,phi,psi", [(70, 20, 0), (30, 60, 90), (120, -35, 17), (45, 45, 45)])
def test_oblique_plane_wave_stays_inside_the_box(built, tmp_path, theta, phi, psi):
    ext = rd.ExtParams(pmllen=10, tfsf_gap=6, ntf_gap=3, oblique=1, inc_theta=math.radians(theta),
                       inc_phi=math.radians(phi), inc_psi=math.radians(psi))
    assert _leakage_db(tmp_path, ext) < -50.0  # measured -57 to -63 dB


def test_normal_incidence_through_the_oblique_line_matches_reference_line(built, tmp_path):
    """A plasma sphere well inside the box, lit along +x: the generic TF/SF
    corrections fed by the dispersion-matched auxiliary line give the same
    near-to-far-field sums as the reference's x-directed line (the two lines
    differ only in how their far ends are terminated)."""
    N = 64
    p, wp, nu, B0 = golden_cases._mk(N=(N, N, N), doB0=0, fsig=20.0, tsteps=300, numfiles=4,
                                     dt=rd.stable_dt(0.25, 0.9), metsize=(1e200, 1e200),
                                     sourcepol=1, nu=1e5)
    wp3 = rd.plasma_sphere_wp3(N, N, N, p.dx, 2.0, 5e13)
    ntf = {}
    for tag, obl in (("ref", 0), ("obl", 1)):
        d = _run(tmp_path, tag, p, wp * 0, nu, B0, rd.ExtParams(oblique=obl, exact_coords=1), wp3)
        ntf[tag] = rd.read_ntf(os.path.join(d, "output_NTF.dat"), p)
    a = np.concatenate([ntf["ref"][k].ravel() for k, _ in rd.NTF_FACE_ORDER])
    b = np.concatenate([ntf["obl"][k].ravel() for k, _ in rd.NTF_FACE_ORDER])
    assert np.abs(a).max() > 1.0
    assert H.rel_l2(b, a) < 1e-4  # measured 2.3e-5


def test_reference_lee_kalluri_grows_colocated_stays_bounded(built, tmp_path):
    """Magnetized trail (B0 dipped 60 degrees, n0 = 1e15, Courant 0.9): the
    reference's update (E averaged over two nodes, J applied at one) grows by
    orders of magnitude within 900 steps; with E taken at the current's own
    node the same run stays at the incident amplitude."""
    p, wp, nu, B0 = golden_cases._mk(doB0=1, n0=1e15, nu=3e4, metsize=(1e200, 1e200),
                                     fsig=20.0, dt=rd.stable_dt(0.25, 0.9), tsteps=900,
                                     numfiles=6)
    d = _run(tmp_path, "ref", p, wp, nu, B0)
    m_ref = [float(v) for v in rd.read_log_maxima(os.path.join(d, "log.txt"))]
    d = _run(tmp_path, "colo", p, wp, nu, B0, rd.ExtParams(lk_colocated=1))
    m_col = [float(v) for v in rd.read_log_maxima(os.path.join(d, "log.txt"))]
    assert m_ref[-1] > 1e3 * max(m_ref[1:3])
    assert max(m_col) < 5.0 and np.isfinite(m_col).all()


@pytest.mark.parametrize("name", sorted(golden_cases.ext_cases()))
def test_ext_cases_run_finite_in_the_oracle(built, tmp_path, name):
    case = golden_cases.ext_cases()[name]
    d = os.path.join(str(tmp_path), name)
    golden_cases.write_ext_case(d, case)
    H.run_oracle(d)
    ntf = rd.read_ntf(os.path.join(d, "output_NTF.dat"), case[0])
    v = np.concatenate([ntf[k].ravel() for k, _ in rd.NTF_FACE_ORDER])
    assert np.isfinite(v).all() and np.abs(v).max() > 0


def test_oracle_trail_matches_the_map_generator(built, tmp_path):
    """The oracle's parametric-trail evaluation (trail.dat) and the numpy map
    generator (rundir.trail_wp3 written as wp3.dat) describe the same plasma:
    the runs agree to rounding of the transcendental functions."""
    case = golden_cases.trail_case()
    p, wp, nu, B0, ext, tr = case
    da = os.path.join(str(tmp_path), "trail")
    golden_cases.write_trail_case(da, case)
    H.run_oracle(da)
    db = _run(tmp_path, "map", p, wp, nu, B0, ext, rd.trail_wp3(p.Nx, p.Ny, p.Nz, p.dx, tr))
    A = rd.read_ntf(os.path.join(da, "output_NTF.dat"), p)
    B = rd.read_ntf(os.path.join(db, "output_NTF.dat"), p)
    a = np.concatenate([A[k].ravel() for k, _ in rd.NTF_FACE_ORDER])
    b = np.concatenate([B[k].ravel() for k, _ in rd.NTF_FACE_ORDER])
    assert np.abs(a).max() > 1.0 and H.rel_l2(a, b) < 1e-10


# ---- host logic of the extended inputs (library, no GPU) ----------------------

def test_ext_file_roundtrip(tmp_path):
    e = rd.ExtParams(pmllen=12, tfsf_gap=8, ntf_gap=4, oblique=1, exact_coords=1, lk_colocated=1,
                     pml_m=3.0, kappa_max=5.0, alpha_max=0.05, inc_theta=1.2, inc_phi=0.3,
                     inc_psi=0.1)
    b = rd.pack_ext(e, True, False)
    assert len(b) == 88
    e2, w3, n3 = rd.unpack_ext(b)
    assert e2 == e and w3 and not n3


def test_problem_reads_ext_dat_and_maps(built, tmp_path):
    case = golden_cases.ext_cases()["ext_sphere"]
    d = os.path.join(str(tmp_path), "r")
    golden_cases.write_ext_case(d, case)
    pb = E.Problem.from_rundir(d)
    p = case[0]
    assert pb.dims()[:3] == (p.Nx, p.Ny, p.Nz)
    # per-cell maps are resident on the device: the FP64 footprint grows by two maps
    plain = E.Problem.from_rundir(d)
    assert pb.footprint(E.FORM_FP32_FUSED) > 0 and plain.footprint(E.FORM_FP64_PLAIN) > 0
    os.remove(os.path.join(d, "nu3.dat"))
    with pytest.raises(E.MfdtdError) as ei:
        E.Problem.from_rundir(d)
    assert E.STATUS[ei.value.code] == "EIO" and "nu3.dat" in E.last_error()


@pytest.mark.parametrize("bad", [dict(pmllen=40), dict(tfsf_gap=6, ntf_gap=5), dict(kappa_max=0.5),
                                 dict(pmllen=12, tfsf_gap=12)])
def test_set_ext_rejects_bad_values(built, bad):
    p, wp, nu, B0 = golden_cases.cases()["lk_trail"]
    pb = E.Problem.from_params(p, np.asarray(wp), np.asarray(nu), B0)
    with pytest.raises(E.MfdtdError) as ei:
        pb.set_ext(rd.ExtParams(**bad))
    assert E.STATUS[ei.value.code] == "EINVAL"
    pb.set_ext(rd.ExtParams())  # a rejected call leaves the problem usable


def test_set_ext_checks_map_shape(built):
    p, wp, nu, B0 = golden_cases.cases()["lk_trail"]
    pb = E.Problem.from_params(p, np.asarray(wp), np.asarray(nu), B0)
    with pytest.raises(ValueError):
        pb.set_ext(rd.ExtParams(), wp3=np.zeros((p.Nx, p.Ny, p.Nz + 1)))


def test_trail_rejects_bad_parameters(built):
    p, wp, nu, B0 = golden_cases.cases()["lk_trail"]
    pb = E.Problem.from_params(p, np.asarray(wp), np.asarray(nu), B0)
    for bad in (dict(r0=0.0), dict(axis=(0.0, 0.0, 0.0)), dict(s_half=-1.0), dict(log10n_hi=40.0)):
        with pytest.raises(E.MfdtdError) as ei:
            pb.set_trail(rd.TrailParams(**bad))
        assert E.STATUS[ei.value.code] == "EINVAL"
    pb.set_trail(rd.TrailParams())
    pb.set_trail(None)
