"""GPU: batched FP32 simulations (one persistent kernel per step, device work
queue, CUDA graph) give each member the result it gets alone.

Tolerance: the batched and the single-simulation kernels compile the same
arithmetic but the compiler may contract multiply-adds differently in each,
so results agree to FP32 rounding: the near-to-far-field sums (integrated over
the surface and the run) to 1e-6 relative L2, the probe series (point values)
to 2e-5 (measured 5.8e-6 after 200 steps).  Members of different sizes and
step counts share the batch; one joins at an odd tick; one finishes early and
idles while the rest continue.

The non-cubic member is a 52 x 56 x 64 magnetized trail.  (The golden
"rect" case is 52 x 52 x 40: with the default 10-cell TF/SF gap its box is
empty along z, so no incident field enters and its FP32 fields are only the
rounding residue of the two coinciding face corrections, about 1e-9; a
relative comparison of two such residues says nothing.)
"""
import dataclasses
import os

import numpy as np
import pytest

import cases as golden_cases
import helpers as H
from meteorscattering_gb300 import engine as E
from meteorscattering_gb300 import rundir as rd

pytestmark = pytest.mark.gpu
TOL = 1e-6        # near-to-far-field sums
TOL_PROBE = 2e-5  # probe series


def _problem(case):
    p, wp, nu, B0 = case
    wp2 = np.asarray(wp).reshape(-1, order="F").reshape(p.Nx, p.Ny)
    nu2 = np.asarray(nu).reshape(-1, order="F").reshape(p.Nx, p.Ny)
    return E.Problem.from_params(p, wp2, nu2, B0)


def _long(name, steps):
    p, wp, nu, B0 = golden_cases.cases()[name]
    return dataclasses.replace(p, dt=rd.stable_dt(p.dx, 0.9), tsteps=steps, numfiles=1), wp, nu, B0


def _noncubic(steps):
    p, wp, nu, B0 = golden_cases._mk(N=(52, 56, 64), doB0=1)
    return dataclasses.replace(p, dt=rd.stable_dt(p.dx, 0.9), tsteps=steps, numfiles=1), wp, nu, B0


def _alone(pb):
    s = E.Simulation(pb, form=E.FORM_FP32_FUSED)
    s.advance(s.dims[3])
    out = s.read_ntf(), s.read_probes()
    s.close()
    return out


def test_batch_members_match_their_single_runs(built):
    cases = [_long("lk_trail", 240), _noncubic(200), _long("lk_numap", 240)]
    pbs = [_problem(c) for c in cases]
    want = [_alone(pb) for pb in pbs]
    b = E.Batch()
    sims = [E.Simulation(pb, form=E.FORM_FP32_FUSED) for pb in pbs]
    b.add(sims[0])
    b.add(sims[1])
    b.run(7)                    # the third member joins at an odd tick
    b.add(sims[2])
    b.run(240)                  # the non-cubic member finishes at 200 and idles
    b.sync()
    for s, c, (ntf, prb) in zip(sims, cases, want):
        assert s.step_index == c[0].tsteps
        got = s.read_ntf()
        assert np.abs(ntf).max() > 0
        assert H.rel_l2(got, ntf) < TOL
        assert H.rel_l2(s.read_probes(), prb) < TOL_PROBE
    b.close()


def test_batch_trails_with_uniform_lee_kalluri_and_autotuner(built):
    """Parametric trails of two sizes (uniform Lee-Kalluri matrices, oblique
    incidence, graded CPML): the autotuner tries slab depths and CTAs per SM
    on the live batch, and the results still match the single runs."""
    cases = []
    for N, steps in (((48, 48, 48), 160), ((40, 56, 64), 150)):
        p, wp, nu, B0, ext, tr = golden_cases.trail_case(N=N, steps=steps)
        cases.append((p, wp, nu, B0, ext, tr))

    def problem(c):
        p, wp, nu, B0, ext, tr = c
        pb = E.Problem.from_params(p, np.asarray(wp).reshape(-1, order="F").reshape(p.Nx, p.Ny),
                                   np.asarray(nu).reshape(-1, order="F").reshape(p.Nx, p.Ny), B0)
        return pb.set_ext(ext).set_trail(tr)

    want = [_alone(problem(c)) for c in cases]
    b = E.Batch()
    sims = [E.Simulation(problem(c), form=E.FORM_FP32_FUSED) for c in cases]
    for s in sims:
        b.add(s)
    depth, ctas = b.tune((8, 16, 48), (2, 3))
    assert depth in (8, 16, 48) and ctas in (2, 3)
    b.run(200)
    b.sync()
    for s, c, (ntf, _) in zip(sims, cases, want):
        assert s.step_index == c[0].tsteps
        assert H.rel_l2(s.read_ntf(), ntf) < TOL
    b.close()


def test_batch_membership_rules(built):
    pb = _problem(_long("lk_trail", 20))
    b = E.Batch()
    s = E.Simulation(pb, form=E.FORM_FP32_FUSED)
    b.add(s)
    with pytest.raises(E.MfdtdError) as ei:
        s.advance(1)             # members are advanced by the batch only
    assert E.STATUS[ei.value.code] == "ESTATE"
    di = E.Simulation(_problem(_long("di_sine_ey", 20)), form=E.FORM_FP32_FUSED)
    with pytest.raises(E.MfdtdError) as ei:
        b.add(di)                # another current update than the batch's
    assert E.STATUS[ei.value.code] == "EINVAL"
    plain = E.Simulation(pb, form=E.FORM_FP64_PLAIN)
    with pytest.raises(E.MfdtdError):
        b.add(plain)
    b.run(5)
    b.sync()
    b.remove(s)
    assert s.step_index == 5
    s.advance(15)                # on its own again
    assert s.step_index == 20
    b.close()


def test_member_removed_between_dft_ring_flushes_keeps_its_sums(built):
    """The running DFT of a member goes through a ring of 8 steps that its
    batch flushes into the sums every 8 ticks.  A member leaving the batch
    off a ring boundary (101 steps: 96 flushed, 5 still in the ring) has the
    pending steps added on removal: continued alone to its end, it matches
    the stand-alone run."""
    pb = _problem(_long("lk_trail", 160))
    ntf, _ = _alone(pb)
    b = E.Batch()
    s = E.Simulation(pb, form=E.FORM_FP32_FUSED)
    b.add(s)
    b.run(101)
    b.sync()
    b.remove(s)
    assert s.step_index == 101
    s.advance(59)
    assert np.abs(ntf).max() > 0
    assert H.rel_l2(s.read_ntf(), ntf) < TOL
    b.close()
    s.close()


def test_two_batches_on_one_device_keep_their_members_apart(built):
    """Batches of different current updates (Lee-Kalluri, Young DI) run side by
    side on one device, as a server with several batch keys runs them.  The
    members' kernel arguments live in constant-memory slots that every batch
    on the device draws from, so each member must still get its stand-alone
    result, and the slots must come back when the batches close."""
    cases = [_long("lk_trail", 60), _long("di_sine_ey", 60)]
    pbs = [_problem(c) for c in cases]
    want = [_alone(pb) for pb in pbs]
    cap = E.Batch.capacity()
    batches, sims = [], []
    for pb in pbs:
        b = E.Batch()
        s = E.Simulation(pb, form=E.FORM_FP32_FUSED)
        b.add(s)
        batches.append(b)
        sims.append(s)
    for b in batches:
        b.run(60)               # both enqueued before either is synchronised
    for b in batches:
        b.sync()
    for s, (ntf, prb) in zip(sims, want):
        assert np.abs(ntf).max() > 0
        assert H.rel_l2(s.read_ntf(), ntf) < TOL
        assert H.rel_l2(s.read_probes(), prb) < TOL_PROBE
    for b in batches:
        b.close()
    # every slot is free again: a batch can take the whole capacity
    b = E.Batch()
    full = [E.Simulation(pbs[0], form=E.FORM_FP32_FUSED) for _ in range(cap)]
    for s in full:
        b.add(s)
    b.close()
    for s in full:
        s.close()


def test_batch_tile_shapes_under_the_autotuner(built):
    """Members that qualify for the CPML slab march (oblique trails with a pair
    of interior 8 x 32 tiles along k): the autotuner times 8 x 32 tiles (fast
    path) and 8 x 64 tiles (wide path, two cells per thread) on the live batch,
    so the members advance under both shapes while it tunes, and the results
    still match the stand-alone runs."""
    cases = []
    for N, steps in (((40, 48, 128), 140), ((48, 40, 128), 130)):
        cases.append(golden_cases.trail_case(N=N, steps=steps))

    def problem(c):
        p, wp, nu, B0, ext, tr = c
        pb = E.Problem.from_params(p, np.asarray(wp).reshape(-1, order="F").reshape(p.Nx, p.Ny),
                                   np.asarray(nu).reshape(-1, order="F").reshape(p.Nx, p.Ny), B0)
        return pb.set_ext(ext).set_trail(tr)

    want = [_alone(problem(c)) for c in cases]
    b = E.Batch()
    sims = [E.Simulation(problem(c), form=E.FORM_FP32_FUSED) for c in cases]
    for s in sims:
        b.add(s)
    depth, ctas = b.tune((16, 48), (2, 3))   # 2 shapes x 2 depths, 4 steps each
    assert b.tile_shape() in ((8, 32), (8, 64))
    b.run(200)
    b.sync()
    for s, c, (ntf, prb) in zip(sims, cases, want):
        assert s.step_index == c[0].tsteps
        assert np.abs(ntf).max() > 0
        assert H.rel_l2(s.read_ntf(), ntf) < TOL
        assert H.rel_l2(s.read_probes(), prb) < TOL_PROBE
    b.close()
