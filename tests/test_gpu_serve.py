"""GPU: the serving loop (continuous batching under an HBM cap).

* Jobs submitted while others run are admitted as memory frees up, share
  batches with them, and each result equals the job's stand-alone FP32 result
  (relative difference of the cross sections below 1e-5 wherever sigma is
  within 30 dB of its peak: the batched follow-up kernel and the stand-alone
  one may round differently, which deep nulls of the pattern magnify) and
  lies within 0.1 dB of the FP64 plain form there.
* The device memory of admitted jobs never exceeds the cap.
* A job larger than the cap is refused at submission.
* Queued and running jobs can be canceled.
* A job of at least 2^25 cells marches alone, beside the batches, and its
  result is the stand-alone run's bit for bit.
"""
import time

import numpy as np
import pytest

from meteorscattering_gb300 import engine as E
from meteorscattering_gb300 import sweep

pytestmark = pytest.mark.gpu


def _jobs(n, steps, seed=5):
    rng = np.random.default_rng(seed)
    sizes = [(48, 48, 64), (48, 48, 48), (56, 56, 64), (48, 48, 96), (52, 48, 56)]
    return [sweep.random_trail(rng, steps, sizes[q % len(sizes)]) for q in range(n)]


def _standalone(job, form, th, ph, method=0):
    s = E.Simulation(job.problem(E), form=form)
    s.advance(s.dims[3])
    out = s.far_field(th, ph, method=method)
    s.close()
    return out


def test_served_results_match_standalone_runs(built):
    th, ph = sweep.direction_grid(15.0)
    jobs = _jobs(5, 180)
    srv = E.Server(hbm_cap_bytes=8 * 10 ** 9, steps_per_round=40)
    ids = [srv.submit(j.problem(E), th, ph) for j in jobs[:3]]
    time.sleep(0.05)
    ids += [srv.submit(j.problem(E), th, ph) for j in jobs[3:]]  # arrive while others run
    got = {}
    deadline = time.time() + 120
    while len(got) < len(ids) and time.time() < deadline:
        for jid in ids:
            if jid in got:
                continue
            done, sig, times = srv.poll(jid, 50)
            if done:
                assert times[1] >= times[0] >= 0
                got[jid] = sig
    srv.close()
    assert len(got) == len(ids)
    for jid, job in zip(ids, jobs):
        # the server projects on the tensor cores (far-field method 1)
        s32 = _standalone(job, E.FORM_FP32_FUSED, th, ph, method=1)[..., 0]
        s64 = _standalone(job, E.FORM_FP64_PLAIN, th, ph)[..., 0]
        served = got[jid][..., 0]
        m32 = s32 > s32.max() * 1e-3
        assert np.max(np.abs(served - s32)[m32] / s32[m32]) < 1e-5
        mask = s64 > s64.max() * 1e-3
        assert np.abs(10 * np.log10(served[mask] / s64[mask])).max() < 0.1


def test_large_job_marches_alone_beside_the_batches(built):
    th, ph = sweep.direction_grid(15.0)
    rng = np.random.default_rng(21)
    big = sweep.random_trail(rng, 120, (256, 256, 512))  # 2^25 cells: the solo lane
    small = _jobs(2, 120, seed=22)
    srv = E.Server(hbm_cap_bytes=16 * 10 ** 9, steps_per_round=40)
    ids = [srv.submit(j.problem(E), th, ph) for j in [small[0], big, small[1]]]
    got = {}
    deadline = time.time() + 180
    while len(got) < len(ids) and time.time() < deadline:
        for jid in ids:
            if jid not in got:
                done, sig, _ = srv.poll(jid, 50)
                if done:
                    got[jid] = sig
    srv.close()
    assert len(got) == len(ids)
    want = _standalone(big, E.FORM_FP32_FUSED, th, ph, method=1)
    assert np.array_equal(got[ids[1]], want)
    for jid, job in ((ids[0], small[0]), (ids[2], small[1])):
        s32 = _standalone(job, E.FORM_FP32_FUSED, th, ph, method=1)[..., 0]
        m32 = s32 > s32.max() * 1e-3
        assert np.max(np.abs(got[jid][..., 0] - s32)[m32] / s32[m32]) < 1e-5


def test_admission_respects_the_device_cap(built):
    th, ph = sweep.direction_grid(30.0)
    jobs = _jobs(4, 120, seed=9)
    one = max(E.Problem.footprint(j.problem(E), E.FORM_FP32_FUSED) for j in jobs)
    cap = int(one * 1.5)                     # room for one job at a time
    srv = E.Server(hbm_cap_bytes=cap, steps_per_round=30)
    ids = [srv.submit(j.problem(E), th, ph) for j in jobs]
    peak_running, peak_bytes, done = 0, 0, set()
    deadline = time.time() + 120
    while len(done) < len(ids) and time.time() < deadline:
        st = srv.stats()
        peak_running = max(peak_running, st["running"])
        peak_bytes = max(peak_bytes, st["device_bytes"])
        for jid in ids:
            if jid not in done and srv.poll(jid, 10)[0]:
                done.add(jid)
    srv.close()
    assert len(done) == len(ids)
    assert peak_bytes <= cap and peak_running <= 1


def test_oversize_job_is_refused(built):
    th, ph = sweep.direction_grid(45.0)
    job = _jobs(1, 50)[0]
    srv = E.Server(hbm_cap_bytes=10 ** 6, steps_per_round=10)
    with pytest.raises(E.MfdtdError) as ei:
        srv.submit(job.problem(E), th, ph)
    assert E.STATUS[ei.value.code] == "ENOMEM"
    srv.close()


def test_cancel_queued_and_running_jobs(built):
    """With room for one job at a time: a canceled queued job fails its poll
    with ECANCELED at once; a canceled running job leaves its batch after the
    current round and its memory admits the next job, which completes with
    the same cross sections as its stand-alone run; an unknown id is EINVAL."""
    th, ph = sweep.direction_grid(30.0)
    jobs = _jobs(3, 3000, seed=11)
    one = max(E.Problem.footprint(j.problem(E), E.FORM_FP32_FUSED) for j in jobs)
    srv = E.Server(hbm_cap_bytes=int(one * 1.5), steps_per_round=10)
    a, b, c = (srv.submit(j.problem(E), th, ph) for j in jobs)
    deadline = time.time() + 60
    while srv.stats()["running"] < 1 and time.time() < deadline:
        time.sleep(0.005)
    assert srv.stats()["running"] == 1 and srv.stats()["queued"] == 2
    srv.cancel(c)                       # queued
    with pytest.raises(E.MfdtdError) as ei:
        srv.poll(c, 0)
    assert E.STATUS[ei.value.code] == "ECANCELED"
    srv.cancel(a)                       # running
    with pytest.raises(E.MfdtdError) as ei:
        srv.poll(a, 10000)
    assert E.STATUS[ei.value.code] == "ECANCELED"
    done, sig = False, None
    while not done and time.time() < deadline + 120:
        done, sig, _ = srv.poll(b, 100)
    assert done
    st = srv.stats()
    assert st["device_bytes"] == 0 and st["running"] == 0 and st["queued"] == 0
    with pytest.raises(E.MfdtdError) as ei:
        srv.cancel(12345)
    assert E.STATUS[ei.value.code] == "EINVAL"
    srv.close()
    want = _standalone(jobs[1], E.FORM_FP32_FUSED, th, ph, method=1)[..., 0]
    assert np.max(np.abs(sig[..., 0] - want) / np.maximum(want, 1e-300)) < 1e-5
