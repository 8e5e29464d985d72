"""GPU: the benchmark's pass kernels against the FP64 plain form.

The large-trail workload's physics at 96 x 96 x 192 cells (bench.py workload
``trail96``; the same code path as the 768 x 768 x 1536 benchmark):
* 12-cell CPML graded m = 3, kappa_max = 5, alpha_max = 0.05;
* trail axis tilted 30 degrees from z, log10 n0 from 13 to 16 along it,
  r0 = 0.8 m, evaluated on the device;
* uniform nu = 3e4 and B0 = 5e-5 T dipped 60 degrees, so one Lee-Kalluri
  matrix pair serves the whole grid, with the current driven by E at its own
  node;
* oblique TM plane wave at theta = 70, phi = 20 degrees.

Every step of the FP32 form (no records are taken, so step 0 is an ordinary
step too) runs the interior pass with two cells per thread
(k_fp32_step_wide) and, on a second stream, the march over the CPML slabs
and domain edges (k_fp32_slab), then the oblique TF/SF corrections and the
Huygens-surface DFT kernels; the test checks that these are the kernels that
ran.  The FP64 plain form runs the same inputs; on
extended inputs it is byte-identical to the CPU oracle (tests/test_gpu_ext.py).

Tolerances (FP32 fields against FP64 after 1200 steps):
* E and H, each component: relative L2 below 1e-3;
* the 24 Huygens-surface DFT arrays: relative L2 below 1e-3;
* bistatic RCS on the 2-degree theta/phi grid (91 x 180 directions): within
  0.1 dB wherever sigma is within 30 dB of its peak.
"""
import os
import sys

import numpy as np
import pytest

import helpers as H
from meteorscattering_gb300 import engine as E
from meteorscattering_gb300 import sweep

sys.path.insert(0, H.ROOT)
import bench  # noqa: E402

pytestmark = pytest.mark.gpu

STEPS = 1200


def _run(form):
    p, wp2, nu2, B0, _, _, ext, trail = bench.workload("trail96", STEPS)
    sim = E.Simulation(bench.make_problem(E, p, wp2, nu2, B0, ext, trail), form=form, profile=True)
    sim.advance(STEPS)
    return p, sim


@pytest.fixture(scope="module")
def runs(built):
    p, s64 = _run(E.FORM_FP64_PLAIN)
    _, s32 = _run(E.FORM_FP32_FUSED)
    yield p, s64, s32
    s64.close()
    s32.close()


def test_benchmark_pass_kernels_ran(runs):
    _, _, s32 = runs
    name = s32.kernel_stats()[0][0]
    # the interior pass with the slab march on every step, t = 0 included
    assert name == "k_fp32_step_wide+k_fp32_slab", name


def test_fields_close_to_plain(runs):
    _, s64, s32 = runs
    for comp in range(6):  # Ex Ey Ez Hx Hy Hz
        a, b = s32.read_field(comp), s64.read_field(comp)
        assert np.abs(b).max() > 0
        err = H.rel_l2(a, b)
        assert err < 1e-3, ("EH"[comp // 3] + "xyz"[comp % 3], err)


def test_dft_sums_close_to_plain(runs):
    p, s64, s32 = runs
    a, b = s32.read_ntf()[4 * p.nntf:], s64.read_ntf()[4 * p.nntf:]
    assert np.abs(b).max() > 0
    assert H.rel_l2(a, b) < 1e-3


def test_rcs_within_tenth_db_on_two_degree_grid(runs):
    _, s64, s32 = runs
    th, ph = sweep.direction_grid(2.0)
    r64 = s64.far_field(th, ph)[..., 0]
    r32 = s32.far_field(th, ph)[..., 0]
    mask = r64 > r64.max(axis=1, keepdims=True) * 1e-3
    err = np.abs(10 * np.log10(r32[mask] / r64[mask]))
    assert mask.sum() > 1000
    assert err.max() < 0.1, (err.max(), np.percentile(err, 99))
