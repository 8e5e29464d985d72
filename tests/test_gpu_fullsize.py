"""GPU: the FP32 form at the full 768 x 768 x 1536 size of the large-trail
configuration, checked through a size-independent property.

With no scatterer, the field inside the TF/SF box is the incident wave and
the field outside is what the box surface leaks.  After the oblique front has
swept over the grid's centre planes, the scattered-field slices (total minus
incident inside the total-field region) stay at the leakage level of the
interpolated auxiliary line while the total field is of order one.  That
checks, at the size the benchmark runs, every tile class of the step kernel
(interior, CPML, domain edges), its x-chunks, the TF/SF pass and the state
hand-over between passes.  62 GB of device memory, about 700 steps.
"""
import math

import numpy as np
import pytest

from meteorscattering_gb300 import engine as E
from meteorscattering_gb300 import rundir as rd

pytestmark = pytest.mark.gpu


def test_full_size_empty_grid_scatters_nothing(built):
    N = (768, 768, 1536)
    f0, gf = 50e6, 30.0
    dx = rd.C0 / f0 / gf
    steps = 700
    p = rd.RunParams(Nx=N[0], Ny=N[1], Nz=N[2], tsteps=steps, dt=rd.stable_dt(dx, 0.9), f0=f0,
                     fsig=20.0, gridfactor=gf, numfiles=1, savefields=0, probex=[], probey=[],
                     probez=[], fntf=[f0], metsize=(1e200, 1e200), doB0=0)
    pb = E.Problem.from_params(p, np.zeros((N[0], N[1])), np.full((N[0], N[1]), 3e4))
    pb.set_ext(rd.ExtParams(pmllen=12, pml_m=3.0, kappa_max=5.0, alpha_max=0.05, oblique=1,
                            exact_coords=1, inc_theta=math.radians(70), inc_phi=math.radians(20)))
    sim = E.Simulation(pb, form=E.FORM_FP32_FUSED)
    sim.advance(steps)
    Et, Ht = sim.read_slices()
    Es, Hs = sim.read_slices(scattered=True)
    sim.close()
    amax = lambda d: max(float(np.abs(v).max()) for v in d.values())
    assert all(np.isfinite(v).all() for d in (Et, Ht) for v in d.values())
    assert amax(Et) > 0.1, amax(Et)
    assert amax(Es) < 1e-2 * amax(Et), amax(Es) / amax(Et)
    assert amax(Hs) < 1e-2 * amax(Ht), amax(Hs) / amax(Ht)
