"""C-ABI library: loads, exports what include/mfdtd.h declares, and its host
logic (input parsing, validation, error reporting) behaves without a GPU."""
import dataclasses
import os
import re
import struct

import numpy as np
import pytest

import cases as golden_cases
from meteorscattering_gb300 import engine as E
from meteorscattering_gb300 import rundir as rd

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mfdtd.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mfdtd_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built):
    lib = E.load_library()
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(E.EXPORTS)
    assert b"mfdtd" in lib.mfdtd_version()


def _dir(tmp_path, case="lk_trail", **repl):
    p, wp, nu, B0 = golden_cases.cases()[case]
    if repl:
        p = dataclasses.replace(p, **repl)
    d = os.path.join(str(tmp_path), "r")
    rd.write_rundir(d, p, wp, nu, B0)
    return d, p


def test_problem_from_rundir_reads_both_input_lengths(built, tmp_path):
    d, p = _dir(tmp_path)
    pb = E.Problem.from_rundir(d)
    assert pb.dims() == (p.Nx, p.Ny, p.Nz, p.tsteps, p.nntf, p.nprobes)
    d2, p2 = _dir(tmp_path / "m", "ricker_matlab")  # no doB0 field
    assert E.Problem.from_rundir(d2).dims()[0] == p2.Nx


def test_problem_from_params_matches_rundir(built, tmp_path):
    d, p = _dir(tmp_path)
    p_, wp, nu, B0 = golden_cases.cases()["lk_trail"]
    wp2 = np.asarray(wp).reshape(-1, order="F").reshape(p.Nx, p.Ny)  # wp.dat byte order
    nu2 = np.asarray(nu).reshape(-1, order="F").reshape(p.Nx, p.Ny)
    pb = E.Problem.from_params(p, wp2, nu2, B0)
    assert pb.dims() == E.Problem.from_rundir(d).dims()
    assert pb.footprint(E.FORM_FP64_PLAIN) == E.Problem.from_rundir(d).footprint(E.FORM_FP64_PLAIN)


@pytest.mark.parametrize("repl,code", [
    (dict(numfiles=1000), "EINVAL"),          # reference: t % 0 -> SIGFPE
    (dict(Nx=20), "EINVAL"),                  # CPML slabs overlap
    (dict(probex=[0], probey=[5], probez=[5]), "EINVAL"),  # stencil reads index -1
    (dict(tsteps=0, numfiles=1), "EINVAL"),
    (dict(doplate=1, platesize=1e3), "EINVAL"),  # plate outside the grid
])
def test_invalid_inputs_are_rejected(built, tmp_path, repl, code):
    p, wp, nu, B0 = golden_cases.cases()["lk_trail"]
    p = dataclasses.replace(p, **repl)
    if p.Nx != wp.shape[0]:
        wp = np.zeros((p.Nx, p.Ny)); nu = np.zeros((p.Nx, p.Ny))
    d = os.path.join(str(tmp_path), "bad")
    rd.write_rundir(d, p, wp, nu, B0)
    with pytest.raises(E.MfdtdError) as ei:
        E.Problem.from_rundir(d)
    assert E.STATUS[ei.value.code] == code


@pytest.mark.parametrize("victim", ["inputs.dat", "wp.dat", "nu.dat", "B0.dat"])
def test_missing_or_short_files_are_io_errors(built, tmp_path, victim):
    d, p = _dir(tmp_path)
    path = os.path.join(d, victim)
    with open(path, "rb") as f:
        b = f.read()
    with open(path, "wb") as f:
        f.write(b[: len(b) // 2])
    with pytest.raises(E.MfdtdError) as ei:
        E.Problem.from_rundir(d)
    assert ei.value.code == -2
    os.remove(path)
    with pytest.raises(E.MfdtdError) as ei:
        E.Problem.from_rundir(d)
    assert ei.value.code == -2
    assert victim in E.last_error()


def test_drop_in_executable_reports_errors(built, tmp_path):
    import subprocess
    r = subprocess.run([E.EXE_PATH], cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 1 and "inputs.dat" in r.stderr


def test_static_far_field_rejects_oversize_faces(built):
    """The allocation-free far field refuses faces larger than its fixed
    working array before touching the device."""
    import ctypes as C
    lib = E.load_library()
    fake = (C.c_void_p * 24)(*range(4096, 4096 + 24 * 64, 64))
    one = np.ones(4)
    dp = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))
    out = np.zeros(3)
    rc = lib.mfdtd_far_field_static(fake, 3000, 64, 64, 15, 1, dp(one), 0.2, 0.2, 0.2, dp(one), 1,
                                    dp(one), dp(one), dp(out), None)
    assert E.STATUS[rc] == "EINVAL"
    assert "2048" in E.last_error()
    # a negative Huygens offset would place the faces before the arrays' start
    rc = lib.mfdtd_far_field_static(fake, 64, 64, 64, -1, 1, dp(one), 0.2, 0.2, 0.2, dp(one), 1,
                                    dp(one), dp(one), dp(out), None)
    assert E.STATUS[rc] == "EINVAL"
    assert "ntfb" in E.last_error()
