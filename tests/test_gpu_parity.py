"""GPU parity: the FP64 plain form against the CPU oracle, through the C ABI.

The plain form must reproduce the reference bit for bit on every output file
(indices, masks, step counts, fields, DFT sums, probes, slices), so these tests
compare file bytes, not tolerances.  The oracle runs on the same machine, so
libm differences between hosts do not enter.
"""
import dataclasses
import os
import subprocess

import numpy as np
import pytest

import cases as golden_cases
import helpers as H
from meteorscattering_gb300 import engine as E
from meteorscattering_gb300 import rundir as rd

pytestmark = pytest.mark.gpu
CASES = golden_cases.cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_plain_rundir_bit_exact(built, tmp_path, name):
    case = CASES[name]
    da = H.fresh_dir(tmp_path, name + "_gpu", case)
    db = H.fresh_dir(tmp_path, name + "_orc", case)
    E.run_rundir(da)
    H.run_oracle(db)
    assert H.diff_outputs(da, db, case[0].nntf) == []


def test_drop_in_executable(built, tmp_path):
    case = CASES["lk_trail"]
    da = H.fresh_dir(tmp_path, "exe", case)
    db = H.fresh_dir(tmp_path, "orc", case)
    r = subprocess.run([E.EXE_PATH], cwd=da, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    H.run_oracle(db)
    assert H.diff_outputs(da, db, case[0].nntf) == []


def test_in_memory_api_chunked_advance(built, tmp_path):
    """Advancing in uneven chunks gives the same NTF sums and probes as one run."""
    p, wp, nu, B0 = CASES["lk_trail"]
    d = H.fresh_dir(tmp_path, "orc", CASES["lk_trail"])
    H.run_oracle(d)
    wp2 = np.asarray(wp).reshape(-1, order="F").reshape(p.Nx, p.Ny)
    nu2 = np.asarray(nu).reshape(-1, order="F").reshape(p.Nx, p.Ny)
    pb = E.Problem.from_params(p, wp2, nu2, B0)
    sim = E.Simulation(pb)
    for n in (1, 7, 13, p.tsteps - 21):
        sim.advance(n)
    assert sim.step_index == p.tsteps
    ntf = sim.read_ntf()
    with open(os.path.join(d, "output_NTF.dat"), "rb") as f:
        raw = f.read()
    ref = np.frombuffer(raw, dtype="<f8", offset=8 + 8 * p.nntf)
    assert np.array_equal(ntf.view(np.uint64), ref.view(np.uint64))
    pr = sim.read_probes()
    want = rd.read_probes(os.path.join(d, "Probe.dat"), p.tsteps)
    for q, key in enumerate(("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")):
        assert np.array_equal(pr[q], want[key]), key
    ms, launches = sim.last_timing()
    assert ms > 0 and launches >= 2
    sim.close()


def test_every_step_is_a_record_step(built, tmp_path):
    p, wp, nu, B0 = CASES["rect"]  # numfiles = tsteps
    assert p.numfiles == p.tsteps
    da = H.fresh_dir(tmp_path, "g", CASES["rect"])
    db = H.fresh_dir(tmp_path, "o", CASES["rect"])
    E.run_rundir(da)
    H.run_oracle(db)
    assert H.diff_outputs(da, db, p.nntf) == []
    assert len(rd.read_slices(os.path.join(da, "output_E.dat"), p, True)) == p.tsteps


def test_single_step_and_many_frequencies(built, tmp_path):
    p, wp, nu, B0 = CASES["lk_trail"]
    p = dataclasses.replace(p, tsteps=1, numfiles=1, fntf=list(np.linspace(30e6, 70e6, 11)))
    case = (p, wp, nu, B0)
    da = H.fresh_dir(tmp_path, "g", case)
    db = H.fresh_dir(tmp_path, "o", case)
    E.run_rundir(da)
    H.run_oracle(db)
    assert H.diff_outputs(da, db, p.nntf) == []


def test_cfg1_sized_grid_bit_exact(built, tmp_path):
    """96x96x192 (the reference-runnable configuration's grid), z-uniform
    magnetized trail, 120 steps: every output byte equal."""
    p = rd.RunParams(Nx=96, Ny=96, Nz=192, tsteps=120, dt=rd.stable_dt(0.25), f0=50e6,
                     fsig=20.0, gridfactor=24.0, numfiles=4, probex=[48], probey=[48],
                     probez=[96], fntf=[50e6], metsize=(1e200, 1e200), doB0=1)
    wp = rd.gaussian_trail_wp(p, 1e14, 1.0)
    nu = np.full((96, 96), 5e4)
    case = (p, wp, nu, golden_cases.B0_DIP60)
    da = H.fresh_dir(tmp_path, "g", case)
    db = H.fresh_dir(tmp_path, "o", case)
    E.run_rundir(da)
    H.run_oracle(db)
    assert H.diff_outputs(da, db, p.nntf) == []


def test_guard_catches_nonfinite(built, tmp_path):
    """A NaN planted in the input maps is caught by the field guard on the
    host side as MFDTD_ENUMERIC, and the context stays usable."""
    p, wp, nu, B0 = CASES["lk_trail"]
    wp2 = np.asarray(wp).reshape(-1, order="F").reshape(p.Nx, p.Ny).copy()
    nu2 = np.asarray(nu).reshape(-1, order="F").reshape(p.Nx, p.Ny).copy()
    wp2[24, 24] = np.inf
    pb = E.Problem.from_params(p, wp2, nu2, B0)
    sim = E.Simulation(pb, guard_period=5)
    with pytest.raises(E.MfdtdError) as ei:
        sim.advance(p.tsteps)
    assert E.STATUS[ei.value.code] == "ENUMERIC"
    sim.close()
    # the device is still usable
    good = E.Simulation(E.Problem.from_params(p, np.abs(wp2.clip(0, 1e9)), nu2, B0))
    good.advance(3)
    good.close()
