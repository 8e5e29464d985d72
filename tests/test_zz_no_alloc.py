"""The far field computed without any device allocation (GPU).

mfdtd_far_field_static serves callers that must not call cudaMalloc while
they run -- a plugin whose host application owns all device memory, or a
service that reserves its memory once and forbids allocation on the request
path.  It keeps its working memory in one fixed array inside the library.
This test feeds it DFT sums held in device buffers owned by the caller, calls
it twice in a row (the second call sees the array as the first left it), and
requires both results to equal the allocating mfdtd_sim_far_field within
1e-9 relative.  The first call may load the library's far-field module on
the device (CUDA loads modules lazily), which creates the fixed array; the
second call must leave the device's free memory exactly as it found it.  It
is collected last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes as C
import math

import numpy as np
import pytest

import cases as golden_cases
from meteorscattering_gb300 import engine as E
from meteorscattering_gb300 import rundir as rd

pytestmark = pytest.mark.gpu


def test_static_far_field_matches_allocating_far_field(built):
    torch = pytest.importorskip("torch")
    p, wp, nu, B0 = golden_cases.cases()["sphere"]
    wp2 = np.asarray(wp).reshape(-1, order="F").reshape(p.Nx, p.Ny)
    nu2 = np.asarray(nu).reshape(-1, order="F").reshape(p.Nx, p.Ny)
    sim = E.Simulation(E.Problem.from_params(p, wp2, nu2, B0))
    sim.advance(p.tsteps)
    # 10-degree theta/phi grid: 684 directions, more than one 256-direction pass
    th, ph = np.meshgrid(np.radians(np.arange(0, 181, 10)), np.radians(np.arange(0, 360, 10)),
                         indexing="ij")
    th, ph = np.ascontiguousarray(th.ravel()), np.ascontiguousarray(ph.ravel())
    want = sim.far_field(th, ph)

    flat = sim.read_ntf()
    sim.close()
    nf2 = 2 * p.nntf
    srcdft = np.ascontiguousarray(flat[:2 * nf2])
    shapes = {"fb": (p.Ny, p.Nz), "tb": (p.Nx, p.Nz), "lr": (p.Nx, p.Ny)}
    o, dev = 2 * nf2, []
    for _, kind in rd.NTF_FACE_ORDER:
        a, b = shapes[kind]
        n = a * b * nf2
        dev.append(torch.from_numpy(flat[o:o + n].copy()).to("cuda:0"))
        o += n
    torch.cuda.synchronize()
    ptrs = (C.c_void_p * 24)(*[t.data_ptr() for t in dev])
    fntf = np.ascontiguousarray(p.fntf, dtype=np.float64)
    lib = E.load_library()
    dp = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))
    for call in range(2):
        out = np.full((p.nntf, th.size, 3), np.nan)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(0)[0]
        rc = lib.mfdtd_far_field_static(ptrs, p.Nx, p.Ny, p.Nz, 15, p.nntf, dp(fntf), p.dx, p.dx,
                                        p.dx, dp(srcdft), th.size, dp(th), dp(ph), dp(out), None)
        assert rc == 0, E.last_error()
        free_after = torch.cuda.mem_get_info(0)[0]
        np.testing.assert_allclose(out, want, rtol=1e-9, atol=1e-300, err_msg=f"call {call}")
        if call == 1:  # the module (and its array) exists now: nothing may be allocated
            assert free_after == free_before, (free_before, free_after)
