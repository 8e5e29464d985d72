"""GPU: the FP32 form's CPML band kernels with plasma inside the band.

Under oblique incidence the FP32 pass treats the CPML slabs and the domain
edges like interior cells and leaves them, together with the band's x planes
and the tile rows wholly inside its y rows, to two band kernels that
recompute them with the CPML corrections; the E band kernel also advances J
where the pass did not march.  A wide trail whose plasma fills the band must
then give the same physics as the FP64 plain form (itself byte-identical to
the CPU oracle): the near-to-far-field sums, the fields and the probe series
within 1e-3 relative L2, for both current models (Young's DI update and the
node-averaged Lee-Kalluri update).
"""
import dataclasses
import math

import numpy as np
import pytest

import helpers as H
from meteorscattering_gb300 import engine as E
from meteorscattering_gb300 import rundir as rd

pytestmark = pytest.mark.gpu

B0 = (5e-5 * math.cos(math.pi / 3), 0.0, -5e-5 * math.sin(math.pi / 3))


def _case(doB0):
    N = (50, 53, 61)
    p = rd.RunParams(Nx=N[0], Ny=N[1], Nz=N[2], tsteps=80, dt=rd.stable_dt(0.25, 0.9), f0=50e6, fsig=8.0,
                     gridfactor=24.0, numfiles=4, savefields=1, probex=[4, 25], probey=[26, 3],
                     probez=[30, 30], fntf=[50e6, 60e6], metsize=(2.0, 2.0), doB0=doB0, sourcepol=4)
    ext = rd.ExtParams(pmllen=8, tfsf_gap=4, ntf_gap=2, oblique=1, lk_colocated=0, pml_m=3.0, kappa_max=4.0,
                       alpha_max=0.05, inc_theta=math.radians(60), inc_phi=math.radians(25))
    wp = rd.gaussian_trail_wp(p, 1e13, 5.0)  # r0 = 20 cells: the column reaches every face's band
    return p, ext, wp


@pytest.mark.parametrize("doB0", [0, 1], ids=["young", "lee_kalluri_avg"])
def test_fp32_band_with_plasma_close_to_plain(built, tmp_path, doB0):
    p, ext, wp = _case(doB0)
    w = ext.pmllen + 1
    assert wp[:w, :].max() > 0.3 * wp.max() and wp[:, :w].max() > 0.3 * wp.max()
    nu = np.full((p.Nx, p.Ny), 5e4)
    d = str(tmp_path)
    rd.write_rundir(d, p, wp, nu, B0 if doB0 else (0.0, 0.0, 0.0))
    rd.write_ext(d, ext)
    pb = E.Problem.from_rundir(d)
    sims = {}
    for form in (E.FORM_FP64_PLAIN, E.FORM_FP32_FUSED):
        s = E.Simulation(pb, form=form)
        s.advance(p.tsteps)
        sims[form] = s
    a, b = sims[E.FORM_FP64_PLAIN], sims[E.FORM_FP32_FUSED]
    na, nb = a.read_ntf()[4 * p.nntf:], b.read_ntf()[4 * p.nntf:]
    assert np.abs(na).max() > 0
    assert H.rel_l2(nb, na) < 1e-3
    for c in range(9):
        fa, fb = a.read_field(c), b.read_field(c)
        if np.abs(fa).max() > 0:
            assert H.rel_l2(fb, fa) < 1e-3, (c, H.rel_l2(fb, fa))
    # J inside the x band (advanced by the E band kernel) is not zero
    jy = b.read_field(7)
    assert np.abs(jy[:w]).max() > 1e-3 * np.abs(jy).max()
    assert H.rel_l2(b.read_probes(), a.read_probes()) < 1e-3
    for s in sims.values():
        s.close()
