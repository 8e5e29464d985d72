"""CPU: the byte counts bench.py reports for the FP32 step.

The compulsory bytes follow the per-cell-update figures of the step (E, H and
J read and written, plus the plasma map where the plasma is 3-D), and the
DRAM traffic estimate scales the ncu captures of the 128 x 384 x 1024
profiling case to other grids: the wide interior pass's bytes per own byte of
the cells it marches, and the slab march's bytes per cell.  On the captured
grid the estimate must give back the captured bytes.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

# The profiling captures: the wide pass over every plane, the slab march,
# read + written.
CAPTURED_WIDE = 1.372194e9 + 1.150718e9
CAPTURED_SLAB = 0.340058e9 + 0.213999e9
CAPTURED_PLASMA = 0.0368245


def test_pass_cells():
    p, *_ = bench.workload("trailprof", 10)
    w = 13  # 12-cell CPML + 1
    inner, xslab, slab = bench.pass_cells(p, 12)
    # tiles interior in j: rows 16..363 (44 tile rows); in k: 32..991 (30 tiles, 15 pairs)
    assert inner == 44 * 15 * 512 * (p.Nx - 2 * w)
    assert xslab == 44 * 15 * 512 * 2 * w
    assert inner + xslab + slab == p.Nx * p.Ny * p.Nz  # every cell once (Ny, Nz tile-aligned)
    q, *_ = bench.workload("trail768", 10)
    inner, xslab, slab = bench.pass_cells(q, 12)
    assert inner + xslab == 92 * 23 * 512 * 768
    assert inner + xslab + slab == 768 * 768 * 1536


def test_traffic_reproduces_the_capture():
    p, *_ = bench.workload("trailprof", 10)
    t = bench.traffic_per_launch("fp32", "trailprof", "k_fp32_step_wide+k_fp32_slab", p, 12, CAPTURED_PLASMA,
                                 True)
    assert t == pytest.approx(CAPTURED_WIDE + CAPTURED_SLAB, rel=1e-4)


def test_traffic_at_full_size_is_near_the_compulsory_bytes():
    p, *_ = bench.workload("trail768", 10)
    own = bench.algorithmic_bytes("fp32", "k_fp32_step_wide", p, 12, True, 0.0118)
    t = bench.traffic_per_launch("fp32", "trail768", "k_fp32_step_wide+k_fp32_slab", p, 12, 0.0118, True)
    # halo re-reads and the slab march's psi: a little above the compulsory bytes
    assert 1.0 < t / own < 1.25
    assert bench.traffic_per_launch("fp32", "cfg1", "k_fp32_step_wide", p, 12, 0.0118, True) is None


def test_per_cell_update_figure():
    p, *_ = bench.workload("trail768", 10)
    cells = p.Nx * p.Ny * p.Nz
    psi = 2 * (2 * 12 * p.Ny * p.Nz + p.Nx * 2 * 12 * p.Nz + p.Nx * p.Ny * 2 * 12)
    # 76 B per cell-update with a per-cell plasma map and plasma everywhere
    assert bench.algorithmic_bytes("fp32", "k_fp32_step", p, 12, True) == cells * 76 + 2 * psi * 8
    # J and the map only in the blocks holding plasma
    assert bench.algorithmic_bytes("fp32", "k_fp32_step", p, 12, True, 0.0) == cells * 48 + 2 * psi * 8
