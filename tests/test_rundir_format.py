"""Run-directory byte layouts (setup/meteorrun.m:44-114, source/meteor-2.1.cpp:84-112)."""
import os
import struct

import numpy as np

import cases as golden_cases
from meteorscattering_gb300 import rundir as rd


def test_inputs_round_trip_both_lengths():
    p = golden_cases.cases()["lk_trail"][0]
    b = rd.pack_inputs(p)
    assert rd.unpack_inputs(b) == p
    q = golden_cases.cases()["ricker_matlab"][0]
    bq = rd.pack_inputs(q)
    assert len(bq) == len(b) - 4  # MATLAB never writes doB0
    assert rd.unpack_inputs(bq).doB0 is None


def test_inputs_field_offsets():
    p = rd.RunParams(Nx=30, Ny=31, Nz=32, tsteps=7, dt=1e-9, probex=[3], probey=[4],
                     probez=[5], fntf=[1.0, 2.0], doB0=1)
    b = rd.pack_inputs(p)
    assert struct.unpack_from("<ii", b, 0) == (p.dopml, p.savefields)
    assert struct.unpack_from("<iiii", b, 48) == (7, 30, 31, 32)
    # 2+2(d)+2+2(d)+4 ints, metsize 2d, wpmax, numax, metloc 3d, metangle, 3 ints
    off = 8 + 16 + 8 + 16 + 16 + 16 + 16 + 24 + 8 + 12
    assert struct.unpack_from("<iii", b, off) == (3, 4, 5)
    assert struct.unpack_from("<i", b, off + 12)[0] == 2
    assert len(b) == off + 12 + 4 + 16 + 4 + 8 + 4


def test_maps_are_written_column_major(tmp_path):
    p = rd.RunParams(Nx=3, Ny=2, Nz=22, tsteps=1, dt=1e-9)
    wp = np.arange(6, dtype=float).reshape(3, 2)  # MATLAB wp(i,j)
    rd.write_rundir(str(tmp_path), p, wp, wp * 0, (0, 0, 0))
    raw = np.fromfile(os.path.join(str(tmp_path), "wp.dat"))
    # MATLAB column-major: wp(1,1), wp(2,1), wp(3,1), wp(1,2), ...
    assert list(raw) == [0, 2, 4, 1, 3, 5]
    # the solver reads C [Nx][Ny]: wp2[i][j] = raw[i*Ny + j]
    assert raw.reshape(3, 2)[1, 0] == wp.reshape(-1, order="F")[2]


def test_record_steps():
    p = rd.RunParams(Nx=30, Ny=30, Nz=30, tsteps=10, dt=1e-9, numfiles=3)
    assert p.record_steps() == [0, 3, 6, 9]  # tsteps/numfiles = 3, includes t=0


def test_meteorrun_trail_shape():
    p = rd.RunParams(Nx=41, Ny=41, Nz=22, tsteps=1, dt=1e-9, metsize=(1.0, 2.0), wpmax=2.0)
    wp = rd.meteorrun_wp(p)
    assert wp.shape == (41, 41)
    i0 = int(np.argmax(wp.max(axis=1)))
    assert abs(i0 - 20) <= 1
    assert np.isclose(wp.max(), 2.0 * 2 * np.pi * p.f0, rtol=1e-2)
