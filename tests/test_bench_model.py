"""CPU: the byte counts bench.py reports for the FP32 step.

The compulsory bytes follow the per-cell-update figures of the step (E, H and
J read and written, plus the plasma map where the plasma is 3-D), and the
DRAM traffic estimate scales the ncu capture of the 128 x 384 x 1024
profiling case to other grids: the pass's bytes per own byte of the cells it
marches, and the CPML band kernels' bytes per band cell.  On the captured
grid the estimate must give back the captured bytes.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

# The profiling capture: the pass read + written, the H and E band kernels.
CAPTURED_PASS = 1.060137e9 + 0.903979e9
CAPTURED_BAND = 0.791891e9 + 0.796273e9
CAPTURED_PLASMA = 0.0368245


def test_band_and_marched_cells():
    p, *_ = bench.workload("trailprof", 10)
    w = 13  # 12-cell CPML + 1
    assert bench.band_cells(p, 12) == p.Nx * p.Ny * p.Nz - (p.Nx - 2 * w) * (p.Ny - 2 * w) * (p.Nz - 2 * w)
    # planes 13..114; rows 8..375 (tile rows 0-7 and 376-383 lie in the band)
    assert bench.marched_cells(p, 12) == (p.Nx - 2 * w) * (p.Ny - 16) * p.Nz
    q, *_ = bench.workload("trail768", 10)
    assert bench.marched_cells(q, 12) == (768 - 26) * (768 - 16) * 1536


def test_traffic_reproduces_the_capture():
    p, *_ = bench.workload("trailprof", 10)
    t = bench.traffic_per_launch("fp32", "trailprof", "k_fp32_step", p, 12, CAPTURED_PLASMA, True)
    assert t == pytest.approx(CAPTURED_PASS + CAPTURED_BAND, rel=1e-4)


def test_traffic_at_full_size_is_near_the_compulsory_bytes():
    p, *_ = bench.workload("trail768", 10)
    own = bench.algorithmic_bytes("fp32", "k_fp32_step", p, 12, True, 0.0118)
    t = bench.traffic_per_launch("fp32", "trail768", "k_fp32_step", p, 12, 0.0118, True)
    # halo re-reads and the band recomputation: a little above the compulsory bytes
    assert 1.0 < t / own < 1.25
    assert bench.traffic_per_launch("fp32", "cfg1", "k_fp32_step", p, 12, 0.0118, True) is None


def test_per_cell_update_figure():
    p, *_ = bench.workload("trail768", 10)
    cells = p.Nx * p.Ny * p.Nz
    psi = 2 * (2 * 12 * p.Ny * p.Nz + p.Nx * 2 * 12 * p.Nz + p.Nx * p.Ny * 2 * 12)
    # 76 B per cell-update with a per-cell plasma map and plasma everywhere
    assert bench.algorithmic_bytes("fp32", "k_fp32_step", p, 12, True) == cells * 76 + 2 * psi * 8
    # J and the map only in the blocks holding plasma
    assert bench.algorithmic_bytes("fp32", "k_fp32_step", p, 12, True, 0.0) == cells * 48 + 2 * psi * 8
