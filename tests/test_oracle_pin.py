"""Pin the CPU oracle (oracle/fdtd_oracle.c) to the reference solver.

* Against the committed golden vectors (tests/golden/*.json, produced by the
  reference binary built from source/meteor-fork.cpp): exact SHA-256 of every
  output file on the machine type that generated them, sampled values within
  1e-12 relative elsewhere (libm may round transcendentals differently there).
* Against the reference binary itself when it has been built here
  (oracle/_ref): byte-identical output files on every case.
* The reference's uninitialised source-DFT sums are excluded from byte
  comparisons and checked against an independent numpy sum instead.
"""
import json
import os
import platform

import numpy as np
import pytest

import cases as golden_cases
import helpers as H
from meteorscattering_gb300 import rundir as rd

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = golden_cases.cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_golden(built, tmp_path, name):
    with open(os.path.join(GOLDEN, f"{name}.json")) as f:
        gold = json.load(f)
    p = CASES[name][0]
    d = H.fresh_dir(tmp_path, name, CASES[name])
    H.run_oracle(d)
    exact = gold["machine"] == platform.machine()
    for fname, g in gold["outputs"].items():
        if fname == "log_maxima":
            got = rd.read_log_maxima(os.path.join(d, "log.txt"))
            if exact:
                assert got == g
            else:
                assert np.allclose([float(v) for v in got], [float(v) for v in g], rtol=1e-9)
            continue
        path = os.path.join(d, fname)
        if g is None:
            assert not os.path.exists(path), fname
            continue
        b = H.comparable_bytes(path, fname, p.nntf, skip_srcdft=True)
        assert len(b) == g["size"], fname
        if exact:
            assert H.sha256_file_bytes(b) == g["sha256"], fname
        vals = np.array([float.fromhex(v) for v in g["values"]])
        got = np.array([np.frombuffer(b, dtype="<f8", count=1, offset=g["header"] + 8 * o)[0]
                        for o in g["offsets"]])
        if exact:
            assert np.array_equal(got.view(np.uint64), vals.view(np.uint64)), fname
        else:
            np.testing.assert_allclose(got, vals, rtol=1e-12, atol=1e-300)


def _have_reference():
    return os.path.exists(H.REF_FORK)


@pytest.mark.skipif(not _have_reference(), reason="reference binary not built here")
@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_live(built, tmp_path, name):
    case = CASES[name]
    da = H.fresh_dir(tmp_path, name + "_ref", case)
    db = H.fresh_dir(tmp_path, name + "_orc", case)
    H.run_reference(da)
    H.run_oracle(db)
    assert H.diff_outputs(da, db, case[0].nntf, skip_srcdft=True) == []


@pytest.mark.skipif(not os.path.exists(H.REF_21), reason="reference binary not built here")
def test_v21_equals_fork_without_b0(built, tmp_path):
    """source/meteor-2.1.cpp and the fork agree when doB0=0 (the fork is a superset)."""
    case = CASES["di_sine_ey"]
    da = H.fresh_dir(tmp_path, "v21", case)
    db = H.fresh_dir(tmp_path, "fork", case)
    H.run_reference(da, H.REF_21)
    H.run_reference(db, H.REF_FORK)
    assert H.diff_outputs(da, db, case[0].nntf, skip_srcdft=True) == []


def test_oracle_source_dft(built, tmp_path):
    """Eydft/Ezdft = sum_t Einc0(t) * (sin, cos)(2 pi f t dt), t integer
    (source/meteor-2.1.cpp:1378-1383; (t+1/2) is integer division)."""
    case = CASES["lk_trail"]  # RHCP: both components driven
    p = case[0]
    d = H.fresh_dir(tmp_path, "srcdft", case)
    H.run_oracle(d)
    ntf = rd.read_ntf(os.path.join(d, "output_NTF.dat"), p)
    t = np.arange(p.tsteps, dtype=np.float64)
    tt = t - 3 * p.fsig
    env = np.exp(-tt * tt / (2 * p.fsig * p.fsig))
    A = np.sin(2 * np.pi * p.f0 * tt * p.dt) * env
    B = np.cos(2 * np.pi * p.f0 * tt * p.dt) * env
    for m, f in enumerate(p.fntf):
        s, c = np.sin(2 * np.pi * f * t * p.dt), np.cos(2 * np.pi * f * t * p.dt)
        np.testing.assert_allclose(ntf["Ezdft"][2 * m:2 * m + 2], [A @ s, A @ c], rtol=1e-12)
        np.testing.assert_allclose(ntf["Eydft"][2 * m:2 * m + 2], [B @ s, B @ c], rtol=1e-12)


def test_oracle_rejects_bad_sizes(built, tmp_path):
    p, wp, nu, B0 = CASES["quiet"]
    import dataclasses
    bad = dataclasses.replace(p, numfiles=p.tsteps + 1)  # reference: SIGFPE
    d = os.path.join(str(tmp_path), "bad")
    rd.write_rundir(d, bad, wp, nu, B0)
    with pytest.raises(RuntimeError):
        H.run_oracle(d)
