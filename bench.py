#!/usr/bin/env python
"""Benchmark of the FDTD time-stepping path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--form fp32|fp64]
                    [--workload NAME] [--impl reference]

A "step" is one FDTD time step (H half-step, E half-step, plasma current J,
CPML, TF/SF, running DFT) over the whole grid.  ``value`` is whole-job
Gcell-updates/s = cells * K * N / (max over ranks of the device time of the K
timed steps), measured with CUDA events on the simulation's stream between a
barrier + synchronize on both sides.  The state of every workload is far larger
than the 129 MB L2, so no flush is needed between steps.

``e2e`` is the same metric through the public API from host buffers: problem
creation from host arrays, device allocation and upload, K steps, and the
device-to-host read of the near-to-far-field sums, timed by the host clock.

Beside the headline, the default line carries (one GPU only; ``--no-plain``,
``--no-sweep`` skip them):

* ``plain_fp64``: the FP64 plain form on the same workload (device time of 3
  steps after a warm-up step) and the FP32/FP64 speed ratio;
* ``sweep``: the batched sweep of 128 random trails from one seed (2500 steps
  each, bistatic RCS on a 5-degree grid) through the serving loop: solves/hour,
  latency p50/p99, and two sequential baselines of the same jobs, FP64 plain
  and single-simulation FP32 (``run_population``).

``--impl reference`` times the reference's CPU implementation of the path on
this host's cores (the reference binary built from its sources when present,
else the C restatement of it in oracle/) on a bounded slab of the same
workload, and prints the same JSON line with ``"impl": "reference"``.

N > 1 runs independent replicas, one per GPU (the path has no data exchange
between jobs); rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import resource
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from meteorscattering_gb300 import rundir as rd  # noqa: E402

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0

# --------------------------------------------------------------------------
# Workloads


TRAIL_GRIDS = {"trail768": (768, 768, 1536), "trailprof": (128, 384, 1024),
               "trail384": (384, 384, 768), "trail96": (96, 96, 192),
               "trail768_nodeavg": (768, 768, 1536)}


def workload(name: str, steps_total: int):
    """(RunParams, wp2 [Nx][Ny] C-order, nu2, B0, description, MATLAB-shaped wp,
    ExtParams or None, TrailParams or None)."""
    B0 = (5e-5 * math.cos(math.pi / 3), 0.0, -5e-5 * math.sin(math.pi / 3))  # 60 deg dip
    ext = trail = None
    if name in TRAIL_GRIDS:
        # Large single trail: 768 x 768 x 1536 cells (trailprof: 128 x 384 x 1024,
        # the profiling-size case; trail384: 384 x 384 x 768, the precision
        # check; trail96: 96 x 96 x 192, the parity test; all with the same
        # physics), dx = 0.2 m (50 MHz radar, gridfactor 30), 12-cell CPML
        # graded m = 3, kappa_max = 5, alpha_max = 0.05; trail axis tilted 30
        # degrees from z in the x-z plane, log10 n0 rising linearly from 13 to
        # 16 along it, r0 = 0.8 m; nu = 3e4; B0 = 5e-5 T dipped 60 degrees;
        # oblique TM plane wave along (theta, phi) = (70, 20) degrees;
        # Lee-Kalluri current driven by E at the current's node (the
        # reference's two-node average diverges here; trail768_nodeavg runs
        # it anyway, for its speed over a few steps).
        N = TRAIL_GRIDS[name]
        f0, gf, nu = 50e6, 30.0, 3e4
        desc = (f"{N[0]}x{N[1]}x{N[2]} tilted magnetized trail, dx=0.2 m, 12-cell CPML "
                "(m=3, kappa_max=5, alpha_max=0.05), trail axis 30 deg from z in x-z, "
                "log10 n0 13..16 along the axis, r0=0.8 m, nu=3e4, B0=5e-5 T at 60 deg dip, "
                "oblique TM plane wave theta=70 phi=20 deg, Lee-Kalluri J (E at the J node)")
        nodeavg = name.endswith("_nodeavg")
        if nodeavg:
            desc = desc.replace("Lee-Kalluri J (E at the J node)", "Lee-Kalluri J (E averaged over two nodes)")
        ext = rd.ExtParams(pmllen=12, pml_m=3.0, kappa_max=5.0, alpha_max=0.05, oblique=1,
                           exact_coords=1, lk_colocated=0 if nodeavg else 1, inc_theta=math.radians(70),
                           inc_phi=math.radians(20), inc_psi=0.0)
        dx = rd.C0 / f0 / gf
        trail = rd.TrailParams.tilted(30.0, 0.8, 13.0, 16.0, 0.5 * (N[2] - 1) * dx)
        n0, r0 = 0.0, 0.8
    elif name == "trail768_refinputs":
        # What the reference's own input format can express at the same size:
        # 10-cell CPML, plane wave along +x, z-uniform Gaussian trail.
        N = (768, 768, 1536)
        f0, gf = 50e6, 30.0
        desc = ("768x768x1536 magnetized trail, dx=0.2 m, Lee-Kalluri J, 10-cell CPML, "
                "plane wave along +x (Ez), z-uniform Gaussian trail n0=1e15 r0=0.8 m, "
                "nu=3e4, B0=5e-5 T at 60 deg dip")
        n0, r0, nu = 1e15, 0.8, 3e4
    elif name == "cfg1":
        # 96 x 96 x 192, dx = 0.25 m, 10-cell CPML graded m = 3, kappa_max = 5,
        # alpha_max = 0.05, TF/SF box 8 and Huygens surface 4 cells inside it,
        # plane wave along +x with E along z, overdense Gaussian trail along z.
        N = (96, 96, 192)
        f0, gf = 50e6, 24.0
        desc = ("96x96x192 magnetized trail, dx=0.25 m, CPML m=3 kappa_max=5 alpha_max=0.05, "
                "TF/SF gap 8, NTF gap 4, Lee-Kalluri J, n0=1e14 r0=1 m, nu=5e4, "
                "B0=5e-5 T at 60 deg dip")
        n0, r0, nu = 1e14, 1.0, 5e4
        ext = rd.ExtParams(pmllen=10, tfsf_gap=8, ntf_gap=4, pml_m=3.0, kappa_max=5.0,
                           alpha_max=0.05)
    else:
        raise SystemExit(f"unknown workload {name}")
    Nx, Ny, Nz = N
    dx = rd.C0 / f0 / gf
    p = rd.RunParams(Nx=Nx, Ny=Ny, Nz=Nz, tsteps=steps_total, dt=rd.stable_dt(dx), f0=f0,
                     fsig=20.0, gridfactor=gf, numfiles=1, savefields=0, probex=[Nx // 2],
                     probey=[Ny // 2], probez=[Nz // 2], fntf=[f0], metsize=(1e200, 1e200),
                     doB0=1)
    wp = rd.gaussian_trail_wp(p, n0, r0) if n0 > 0 else np.zeros((Nx, Ny))
    nu2 = np.full((Nx, Ny), nu)
    wp2 = np.asarray(wp).reshape(-1, order="F").reshape(Nx, Ny)
    return p, wp2, nu2, B0, desc, wp, ext, trail


def make_problem(E, p, wp2, nu2, B0, ext, trail):
    """The public-API call sequence a user makes for this workload."""
    pb = E.Problem.from_params(p, wp2, nu2, B0)
    if ext is not None:
        pb.set_ext(ext)
    if trail is not None:
        pb.set_trail(trail)
    return pb


def algorithmic_bytes(form: str, kernel: str, p: rd.RunParams, L: int = 10,
                      per_cell_map: bool = False, plasma: float = 1.0) -> float:
    """Compulsory DRAM bytes of one launch of `kernel` (per cell-update figure
    x cells, plus the CPML psi slabs each launch reads and writes).  `plasma`
    is the share of the FP32 pass's (plane, tile) blocks holding plasma: J
    (and the per-cell plasma map) are read and written there only, since J is
    identically zero where omega_p is."""
    cells = p.Nx * p.Ny * p.Nz
    psi = 2 * (2 * L * p.Ny * p.Nz + p.Nx * 2 * L * p.Nz + p.Nx * p.Ny * 2 * L)  # one half-step
    if form == "fp64":
        m = 8 if per_cell_map else 0
        if kernel == "k_plain_h":   # E r(3), H r/w(6), J r/w(6) ; psi r/w ; omega_p map
            return cells * (15 * 8 + m) + psi * 16
        if kernel == "k_plain_e":   # H r(3), E r/w(6), J r(3) ; psi r/w
            return cells * 12 * 8 + psi * 16
    else:
        # FP32 single pass: E and H read and written (12 x 4 B) everywhere; J
        # read and written (6 x 4 B) plus the per-cell E0 wp^2 map when the
        # plasma is 3-D (4 B) in the blocks holding plasma; every psi cell of
        # both half-steps read and written once.
        return cells * (12 * 4 + plasma * (6 * 4 + (4 if per_cell_map else 0))) + 2 * psi * 8
    raise KeyError(kernel)


# DRAM traffic of one FP32 step's pass (the wide interior pass and the CPML
# slab march), measured by ncu on the 128 x 384 x 1024 profiling case of the
# large-trail workload (profiles/k_fp32_step_wide_trailprof_full.md,
# profiles/k_fp32_slab_trailprof_full.md); the full-size grid is too large for
# a multi-pass capture.  Three parts scale to a full launch:
#   * the wide pass over the interior planes moves a fixed multiple of its own
#     bytes (E and H, plus J and the plasma map in plasma blocks; the excess
#     is the tile boxes' halo rows and columns, a property of the tile shape):
#     1.077, from a capture of the pass over the interior planes only;
#   * its cells on the x-slab planes move a fixed number of bytes each (the
#     same capture of the pass over every plane, less the first part);
#   * the slab march moves a fixed number of bytes per cell it marches.
TILE_J, TILE_K = 8, 32     # rows and columns of an 8 x 32 tile (the wide pass pairs two)
PROFILE_PLASMA = 0.0368245  # share of plasma blocks in the profiling case
PROFILE_OWN = 48 + PROFILE_PLASMA * 28
WIDE_TRAFFIC_RATIO = (1.011269e9 + 0.809244e9) / (660 * 512 * 102 * PROFILE_OWN)
WIDE_XSLAB_BYTES_PER_CELL = ((1.372194e9 + 1.150718e9) - WIDE_TRAFFIC_RATIO * 660 * 512 * 102 * PROFILE_OWN) / (
    660 * 512 * 26)
SLAB_BYTES_PER_CELL = (0.340058e9 + 0.213999e9) / (216 * 256 * 128)
TRAFFIC_WORKLOADS = ("trail768", "trailprof")


def pass_cells(p: rd.RunParams, L: int):
    """(cells of the wide pass over the interior planes, its cells on the
    x-slab planes, cells of the slab march) of a non-record step, with the
    host's tile classification: 8 x 32 tiles whose cells are all interior in
    j and k (w = L + 1 from every face) pair up along k into 8 x 64 tiles that
    the wide pass marches over every plane (the 2 w x-slab planes with their
    x-normal CPML terms); every other tile goes to the slab march, over every
    plane."""
    w = L + 1
    nzp = -(-p.Nz // TILE_K) * TILE_K
    ntk, nty = nzp // TILE_K, -(-p.Ny // TILE_J)
    pairs = 0
    for ty in range(nty):
        j0 = ty * TILE_J
        if not (j0 >= w and j0 + TILE_J <= p.Ny - w):
            continue
        run = 0
        for tk in range(ntk):
            k0 = tk * TILE_K
            if k0 >= w and k0 + TILE_K <= p.Nz - w:
                run += 1
            else:
                pairs += run // 2
                run = 0
        pairs += run // 2
    cells_tile = TILE_J * TILE_K
    wide_inner = pairs * 2 * cells_tile * (p.Nx - 2 * w)
    wide_xslab = pairs * 2 * cells_tile * 2 * w
    slab = (ntk * nty - 2 * pairs) * p.Nx * cells_tile
    return wide_inner, wide_xslab, slab


def traffic_per_launch(form: str, workload: str, kernel: str, p: rd.RunParams, L: int, plasma: float,
                       per_cell_map: bool):
    """DRAM traffic (read + write bytes) of one step's pass, or None when no
    ncu capture of this workload's kernels is recorded."""
    if form == "fp32" and kernel.startswith("k_fp32_step_wide") and workload in TRAFFIC_WORKLOADS:
        inner, xslab, slab = pass_cells(p, L)
        own = inner * (48 + plasma * (24 + (4 if per_cell_map else 0)))
        return WIDE_TRAFFIC_RATIO * own + WIDE_XSLAB_BYTES_PER_CELL * xslab + SLAB_BYTES_PER_CELL * slab
    return None


# --------------------------------------------------------------------------
# Clock sampling (nvidia-smi during the timed region)


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        if shutil.which("nvidia-smi") is None:
            return
        self.proc = subprocess.Popen(
            ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
             "--format=csv,noheader,nounits", "-lms", "200"],
            stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------
# CPU baseline: the reference implementation on the host cores


def _unlimited_stack():
    resource.setrlimit(resource.RLIMIT_STACK, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))


def cpu_baseline(name: str, steps: int, budget_s: float = 20.0):
    """Time the reference CPU path on a slab of the workload (full Nx x Ny,
    reduced Nz) for a few steps; returns a cpu_baseline dict.  Workloads the
    reference's input format cannot express (extended inputs) run in the C
    restatement, which implements them; the rest run in the reference binary
    where it was built from source on this host."""
    p, wp2, nu2, B0, desc, wp, ext, trail = workload(name, 4)
    threads = os.cpu_count() or 1
    nz = min(p.Nz, max(24, int(4e7 // (p.Nx * p.Ny))))
    ref_exe = os.path.join(ROOT, "oracle", "_ref", "meteor_fork")
    use_ref = (os.path.exists(ref_exe) and os.access(ref_exe, os.X_OK) and ext is None
               and trail is None)
    oracle_so = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
    if not use_ref and not os.path.exists(oracle_so):
        from meteorscattering_gb300 import build as B
        B.build_oracle(with_reference=False)
    import dataclasses
    d = tempfile.mkdtemp(prefix="mfdtd_cpu_")
    try:
        def run(nsteps):
            q = dataclasses.replace(p, Nz=nz, tsteps=nsteps, numfiles=1, savefields=0,
                                    probez=[nz // 2])
            shutil.rmtree(d, ignore_errors=True)
            rd.write_rundir(d, q, wp, np.full((p.Nx, p.Ny), nu2.flat[0]), B0)
            if ext is not None:
                rd.write_ext(d, ext)
            rd.write_trail(d, trail)
            env = dict(os.environ, OMP_NUM_THREADS=str(threads))
            if use_ref:
                t0 = time.perf_counter()
                r = subprocess.run([ref_exe], cwd=d, preexec_fn=_unlimited_stack, env=env,
                                   capture_output=True, text=True)
                if r.returncode != 0:
                    raise RuntimeError(r.stderr)
                return time.perf_counter() - t0
            lib = ctypes.CDLL(oracle_so)
            lib.oracle_run_dir.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
            secs = ctypes.c_double()
            rc = lib.oracle_run_dir(os.fsencode(d), -1, threads, 1, ctypes.byref(secs))
            if rc != 0:
                raise RuntimeError(f"oracle error {rc}")
            return secs.value
        # A one-step run sizes the sample; the reference binary's set-up time is
        # removed by differencing two runs (the port reports its loop time).
        t1 = run(1)
        n = max(2, min(max(steps, 2), int(budget_s / max(t1, 1e-3))))
        t_run = run(n + 1) - t1 if use_ref else run(n)
        cells = p.Nx * p.Ny * nz
        return {"value": cells * n / t_run / 1e9, "unit": "Gcell-updates/s", "cores": threads,
                "kind": "reference" if use_ref else "port",
                "note": None if use_ref else
                ("the C restatement; on an 8-thread x86 host, on the 768x768x67 slab of the "
                 "reference-format workload, it runs at 0.68x the reference binary built from source "
                 "(0.0298 against 0.0436 Gcell/s), so ratios against it overstate the reference-relative "
                 "speed-up by up to 1.46x"),
                "sample": f"{p.Nx}x{p.Ny}x{nz} slab of the workload, {n} steps, "
                          f"{'reference binary (source/meteor-fork.cpp)' if use_ref else 'oracle/fdtd_oracle.c'} "
                          f"with {threads} OpenMP threads; time-loop seconds"}
    finally:
        shutil.rmtree(d, ignore_errors=True)


# --------------------------------------------------------------------------


def dist_setup(n_gpus: int):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def load_peaks():
    try:
        with open(PEAKS_FILE) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def run_population(kind: str, n: int = 0, capacity_gcells: float = 44.0):
    """Batched sweep ("sweep": 128 random trails submitted together) or serving
    stream ("serve": Poisson arrivals, 90 % sweep-distribution trails and 10 %
    384 x 384 x 768 trails, offered at 80 % of `capacity_gcells`, the
    Gcell-updates/s the batched sweep measures):
    every trail runs its full 2500 steps through the native serving loop and
    returns its bistatic RCS on a 5-degree grid.  Returns solves/hour, the
    latency distribution, Gcell-updates/s, and two sequential baselines of the
    same jobs: FP64 plain solves (device time per cell-update measured on the
    smallest and largest job, scaled to every job) and single-simulation FP32
    solves (the whole solve -- set-up, 2500 steps, far field -- timed on the
    smallest and largest job, interpolated in cell count), the latter being
    what batching and serving gain over running the same fused kernels one
    job at a time."""
    from meteorscattering_gb300 import build as B
    B.build()
    from meteorscattering_gb300 import engine as E
    from meteorscattering_gb300 import sweep
    steps = 2500
    if kind == "sweep":
        n = n or 128
        jobs = sweep.population(n, seed=4, steps=steps)
    else:
        n = n or 32
        jobs = sweep.population(n, seed=5, steps=steps, big_fraction=0.1)
    th, ph = sweep.direction_grid(5.0)
    cells = np.array([j.cells for j in jobs], dtype=np.float64)
    work = float(cells.sum()) * steps
    srv = E.Server(hbm_cap_bytes=150 * 10 ** 9, steps_per_round=100)
    clk = ClockSampler(0)
    clk.start()
    rng = np.random.default_rng(11)
    lat, adm, pending = [], [], {}
    t0 = time.perf_counter()
    if kind == "sweep":
        for j in jobs:
            pending[srv.submit(j.problem(E), th, ph)] = j
    else:
        # offered load: 80 % of the capacity measured by the batched sweep
        rate_cells = capacity_gcells * 1e9 * 0.8
        mean_job = float(cells.mean()) * steps / rate_cells
        arrivals = np.cumsum(rng.exponential(mean_job, size=n))
        arrivals -= arrivals[0]
    submitted = 0
    while len(lat) < n:
        now = time.perf_counter() - t0
        if kind == "serve":
            while submitted < n and arrivals[submitted] <= now:
                pending[srv.submit(jobs[submitted].problem(E), th, ph)] = jobs[submitted]
                submitted += 1
        for jid in list(pending):
            done, sig, times = srv.poll(jid, 0)
            if done:
                lat.append(times[1])
                adm.append(times[0])
                del pending[jid]
        time.sleep(0.005)
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    srv.close()
    order = sorted(range(n), key=lambda q: cells[q])
    sample = [order[0], order[-1]]
    # sequential FP64 plain solves: device time per cell-update, interpolated in cell count
    rate = []
    for q in sample:
        s = E.Simulation(jobs[q].problem(E), form=E.FORM_FP64_PLAIN)
        s.advance(10)
        s.advance(40)
        ms, _ = s.last_timing()
        s.close()
        rate.append((cells[q], cells[q] / (ms * 1e-3)))
    (c0, r0), (c1, r1) = rate
    per_cell = np.interp(cells, [c0, c1], [1 / r0, 1 / r1]) if c1 > c0 else np.full_like(cells, 1 / r0)
    plain_s = float((cells * steps * per_cell).sum())
    # sequential single-simulation FP32 solves: the whole solve, timed
    solve = []
    for q in sample:
        ts = time.perf_counter()
        s = E.Simulation(jobs[q].problem(E), form=E.FORM_FP32_FUSED)
        s.advance(steps)
        s.far_field(th, ph, method=1)
        s.close()
        solve.append((cells[q], time.perf_counter() - ts))
    (c0, t0s), (c1, t1s) = solve
    single_s = float(np.interp(cells, [c0, c1], [t0s, t1s]).sum()) if c1 > c0 else t0s * n
    lat = np.array(lat)
    return {"kind": kind, "jobs": n, "steps_per_job": steps, "wall_s": wall,
            "solves_per_hour": n / wall * 3600,
            "gcell_updates_per_s": work / wall / 1e9,
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max())},
            "admission_wait_s": {"p50": float(np.percentile(adm, 50)),
                                 "p99": float(np.percentile(adm, 99))},
            "plain_fp64_sequential": {"solves_per_hour": n / plain_s * 3600, "seconds": plain_s,
                                      "method": "device time per cell-update of FP64 plain measured "
                                                "on the smallest and largest job, scaled to every job"},
            "fp32_single_sequential": {"solves_per_hour": n / single_s * 3600, "seconds": single_s,
                                       "method": "whole FP32 solve (set-up, all steps, far field) timed "
                                                 "on the smallest and largest job, interpolated in cell "
                                                 "count over every job"},
            "speedup_vs_plain_sequential": plain_s / wall,
            "speedup_vs_fp32_single_sequential": single_s / wall,
            "clocks": clocks}


def population_bench(args):
    r = run_population(args.workload, args.jobs, args.capacity)
    n = r["jobs"]
    line = {"metric": "RCS solves/hour", "value": r["solves_per_hour"], "unit": "solves/hour",
            "n_gpus": 1, "steps": r["steps_per_job"], "warmup": 0, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": (f"{n} random trails submitted together (batched sweep)"
                                    if args.workload == "sweep" else
                                    f"{n}-job Poisson stream at ~80% load, 10% 384x384x768 trails"),
                       "jobs": n, "steps_per_job": r["steps_per_job"], "rcs_grid_deg": 5,
                       "hbm_cap_gb": 150, "steps_per_round": 100,
                       "offered_gcell_updates_per_s": (0.8 * args.capacity if args.workload == "serve" else None),
                       "l2": "inputs far larger than L2 on the large jobs; small jobs are "
                             "L2-resident between steps (reported as is)"},
            "e2e": {"value": r["solves_per_hour"], "unit": "solves/hour", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0,
                    "includes": "problem set-up from host parameters, admission, all steps, "
                                "far field on the device, D2H of the cross sections"}}
    line.update({k: v for k, v in r.items() if k not in ("kind", "jobs", "steps_per_job")})
    print(json.dumps(line), flush=True)


def plain_fp64_rate(p, wp2, nu2, B0, ext, trail, steps: int = 3):
    """Device time per step of the FP64 plain form on the same workload (one
    warm-up step, then `steps` timed with CUDA events)."""
    from meteorscattering_gb300 import engine as E
    sim = E.Simulation(make_problem(E, p, wp2, nu2, B0, ext, trail), form=E.FORM_FP64_PLAIN)
    sim.advance(1)
    sim.advance(steps)
    ms, _ = sim.last_timing()
    sim.close()
    return ms


def farfield_bench(args):
    """Far-field projection (bistatic RCS on the 2-degree theta/phi grid,
    16380 directions) of a 384^3 FP32 simulation advanced 20 steps: method 1
    (dense stage on the tensor cores) against method 0 (FP64 CUDA cores)."""
    from meteorscattering_gb300 import build as B
    B.build()
    from meteorscattering_gb300 import engine as E
    from meteorscattering_gb300 import sweep
    N, dx, f0 = 384, 0.15, 50e6
    p = rd.RunParams(Nx=N, Ny=N, Nz=N, tsteps=20, dt=rd.stable_dt(dx), f0=f0, fsig=20.0,
                     gridfactor=(rd.C0 / f0) / dx, numfiles=1, savefields=0, fntf=[f0],
                     metsize=(1e200, 1e200), doB0=0, probex=[], probey=[], probez=[])
    pb = E.Problem.from_params(p, np.zeros((N, N)), np.full((N, N), 1e5), (0.0, 0.0, 0.0))
    sim = E.Simulation(pb, form=E.FORM_FP32_FUSED)
    sim.advance(20)
    th, ph = sweep.direction_grid(2.0)
    times = {}
    for m in ([1] if args.steps <= 1 else [1, 0, 1]):
        t0 = time.perf_counter()
        sim.far_field(th, ph, method=m)
        times.setdefault(m, []).append(time.perf_counter() - t0)
    line = {"metric": "far-field projections/s", "value": 1.0 / min(times[1]), "unit": "1/s",
            "n_gpus": 1, "higher_is_better": True, "dtype": "tf32x3/f64",
            "config": {"workload": f"{N}^3 FP32 simulation, bistatic RCS at {th.size} directions, "
                                   "1 frequency"},
            "ms": {"tensor_cores": 1e3 * min(times[1]),
                   "fp64_cuda_cores": 1e3 * times[0][0] if 0 in times else None}}
    print(json.dumps(line), flush=True)


def mie_bench(args, steps: int = 4000, courant: float = 0.5):
    """Precision check on the 128^3 plasma sphere: homogeneous unmagnetized
    collisional plasma sphere (radius 2 m, n = 5e13 m^-3, nu = 1e5 1/s),
    dx = 0.15 m, 10-cell CPML, 4000 steps, a Gaussian-modulated pulse covering
    30-70 MHz along +x (E along z), RCS at 11 frequencies on the 2-degree
    theta/phi grid.  Reports, for the FP32 fused form against the FP64 plain
    form: field relative L2 after the last step and the RCS dB error per
    angle; for both forms: the backscatter error against the FP64 Mie
    series (oracle/mie.py; the test-infrastructure oracle is used here as the
    checker only)."""
    from meteorscattering_gb300 import build as B
    B.build()
    from meteorscattering_gb300 import engine as E
    from meteorscattering_gb300 import sweep
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import mie
    N, dx, f0 = 128, 0.15, 50e6
    dt = rd.stable_dt(dx, courant)
    freqs = list(np.linspace(30e6, 70e6, 11))
    p = rd.RunParams(Nx=N, Ny=N, Nz=N, tsteps=steps, dt=dt, f0=f0,
                     fsig=1 / (2 * math.pi * 15e6 * dt), gridfactor=(rd.C0 / f0) / dx,
                     numfiles=1, savefields=0, fntf=freqs, metsize=(1e200, 1e200), doB0=0,
                     probex=[], probey=[], probez=[], sourcepol=1)
    n_e, nu, R = 5e13, 1e5, 2.0
    wp3 = rd.plasma_sphere_wp3(N, N, N, dx, R, n_e)
    th, ph = sweep.direction_grid(2.0)
    res, fields, times = {}, {}, {}
    for form in (E.FORM_FP64_PLAIN, E.FORM_FP32_FUSED):
        pb = E.Problem.from_params(p, np.zeros((N, N)), np.full((N, N), nu), (0.0, 0.0, 0.0))
        pb.set_ext(rd.ExtParams(exact_coords=1), wp3=wp3)
        sim = E.Simulation(pb, form=form)
        t0 = time.perf_counter()
        sim.advance(steps)
        sim.sync()
        times[form] = time.perf_counter() - t0
        t1 = time.perf_counter()
        res[form] = sim.far_field(th, ph, method=0)[..., 0]
        times[(form, "ff0")] = time.perf_counter() - t1
        if form == E.FORM_FP32_FUSED:   # the same projection on the tensor cores
            sim.far_field(th, ph, method=1)
            t1 = time.perf_counter()
            res["tc"] = sim.far_field(th, ph, method=1)[..., 0]
            times["ff1"] = time.perf_counter() - t1
        fields[form] = sim.read_field(2)  # Ez after the last step
        back = sim.far_field(np.array([math.pi / 2]), np.array([math.pi]), method=0)[:, 0, 0]
        res[(form, "back")] = back
        sim.close()
    s64, s32 = res[E.FORM_FP64_PLAIN], res[E.FORM_FP32_FUSED]
    mask = s64 > s64.max(axis=1, keepdims=True) * 1e-3
    db = np.abs(10 * np.log10(s32 / s64))
    want = mie.sphere_backscatter(freqs, R, mie.plasma_eps(freqs, float(rd.plasma_frequency(n_e)), nu))
    mie64 = 10 * np.log10(res[(E.FORM_FP64_PLAIN, "back")] / want)
    mie32 = 10 * np.log10(res[(E.FORM_FP32_FUSED, "back")] / want)
    e64, e32 = fields[E.FORM_FP64_PLAIN].ravel(), fields[E.FORM_FP32_FUSED].ravel()
    line = {"metric": "RCS error vs FP64 plain and vs Mie", "value": float(db[mask].max()),
            "unit": "dB (FP32 vs FP64, max over angles within 30 dB of the peak)",
            "higher_is_better": False, "n_gpus": 1, "steps": steps, "dtype": "f32 vs f64",
            "data": "synthetic",
            "config": {"workload": "128^3 plasma sphere r=2 m n=5e13 nu=1e5, dx=0.15 m, "
                                   "10-cell CPML, 30-70 MHz pulse along +x, 11 frequencies, "
                                   "2-degree theta/phi grid",
                       "dt_s": dt, "courant": courant},
            "fp32_vs_fp64": {"field_rel_l2_Ez_final": float(np.linalg.norm(e32 - e64) / np.linalg.norm(e64)),
                             "rcs_db_max": float(db[mask].max()),
                             "rcs_db_p99": float(np.percentile(db[mask], 99)),
                             "rcs_db_max_per_freq": [float(db[m][mask[m]].max()) for m in range(len(freqs))]},
            "vs_mie_backscatter_db": {"freqs_mhz": [f / 1e6 for f in freqs],
                                      "fp64_plain": [float(v) for v in mie64],
                                      "fp32_fused": [float(v) for v in mie32]},
            "seconds": {"fp64_plain": times[E.FORM_FP64_PLAIN], "fp32_fused": times[E.FORM_FP32_FUSED]},
            "far_field": {"ms_fp64": 1e3 * times[(E.FORM_FP32_FUSED, "ff0")],
                          "ms_tensor_cores": 1e3 * times["ff1"],
                          "max_db_tensor_cores_vs_fp64": float(
                              np.abs(10 * np.log10(res["tc"] / s32))[s32 > s32.max(axis=1, keepdims=True) * 1e-3].max())}}
    print(json.dumps(line), flush=True)


def precision_bench(args, steps: int = 4000):
    """FP32 fused against FP64 plain on the large-trail physics at 384 x 384 x
    768 cells (half the 768 x 768 x 1536 benchmark grid along each axis; the
    full size in FP64 would take about 37 minutes), 4000 steps: relative L2 of
    every field component after the last step and of the DFT sums, and the
    bistatic RCS dB error on the 2-degree theta/phi grid (max and p99 over the
    directions within 30 dB of the peak)."""
    from meteorscattering_gb300 import build as B
    B.build()
    from meteorscattering_gb300 import engine as E
    from meteorscattering_gb300 import sweep
    steps = args.steps if args.steps > 100 else steps
    p, wp2, nu2, B0, desc, _, ext, trail = workload("trail384", steps)
    th, ph = sweep.direction_grid(2.0)
    res, secs = {}, {}
    for form in (E.FORM_FP32_FUSED, E.FORM_FP64_PLAIN):
        sim = E.Simulation(make_problem(E, p, wp2, nu2, B0, ext, trail), form=form)
        t0 = time.perf_counter()
        sim.advance(steps)
        sim.sync()
        secs[form] = time.perf_counter() - t0
        res[form] = {"rcs": sim.far_field(th, ph, method=0)[..., 0],
                     "ntf": sim.read_ntf()[4 * p.nntf:]}
        if form == E.FORM_FP32_FUSED:
            res[form]["fields"] = [sim.read_field(c) for c in range(6)]
        else:  # compared one component at a time (each is 0.9 GB in FP64)
            res["field_rel_l2"] = {}
            for c, n in enumerate(("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")):
                y = sim.read_field(c)
                x = res[E.FORM_FP32_FUSED]["fields"][c]
                res["field_rel_l2"][n] = float(np.linalg.norm((x - y).ravel()) / np.linalg.norm(y.ravel()))
                res[E.FORM_FP32_FUSED]["fields"][c] = None
        if form == E.FORM_FP32_FUSED:
            res["tc"] = sim.far_field(th, ph, method=1)[..., 0]
        sim.close()
    a, b = res[E.FORM_FP32_FUSED], res[E.FORM_FP64_PLAIN]

    def rel(x, y):
        return float(np.linalg.norm((x - y).ravel()) / np.linalg.norm(y.ravel()))

    mask = b["rcs"] > b["rcs"].max(axis=1, keepdims=True) * 1e-3
    db = np.abs(10 * np.log10(a["rcs"][mask] / b["rcs"][mask]))
    dbtc = np.abs(10 * np.log10(res["tc"][mask] / b["rcs"][mask]))
    line = {"metric": "RCS error, FP32 fused vs FP64 plain", "value": float(db.max()),
            "unit": "dB (max over the 2-degree directions within 30 dB of the peak)",
            "higher_is_better": False, "n_gpus": 1, "steps": steps, "dtype": "f32 vs f64",
            "data": "synthetic",
            "config": {"workload": desc, "grid": [p.Nx, p.Ny, p.Nz], "directions": int(th.size)},
            "rcs_db_max": float(db.max()), "rcs_db_p99": float(np.percentile(db, 99)),
            "rcs_db_max_tensor_cores_vs_fp64_plain": float(dbtc.max()),
            "directions_within_30db": int(mask.sum()),
            "field_rel_l2": res["field_rel_l2"],
            "dft_sums_rel_l2": rel(a["ntf"], b["ntf"]),
            "seconds": {"fp32_fused": secs[E.FORM_FP32_FUSED], "fp64_plain": secs[E.FORM_FP64_PLAIN]},
            "ms_per_step": {"fp32_fused": 1e3 * secs[E.FORM_FP32_FUSED] / steps,
                            "fp64_plain": 1e3 * secs[E.FORM_FP64_PLAIN] / steps}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default="fp32", choices=["fp64", "fp32"])
    ap.add_argument("--workload", default="trail768")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 plain comparison")
    ap.add_argument("--no-sweep", action="store_true", help="skip the 128-trail batched sweep")
    ap.add_argument("--jobs", type=int, default=0, help="sweep/serve: number of trails")
    ap.add_argument("--capacity", type=float, default=44.0,
                    help="serve: Gcell-updates/s the batched sweep measured; the stream offers 80 %% of it")
    args = ap.parse_args()
    if args.workload in ("sweep", "serve") and args.impl == "gb300":
        population_bench(args)
        return
    if args.workload == "farfield" and args.impl == "gb300":
        farfield_bench(args)
        return
    if args.workload == "mie" and args.impl == "gb300":
        mie_bench(args)
        return
    if args.workload == "precision384" and args.impl == "gb300":
        precision_bench(args)
        return
    K, W = args.steps, max(args.warmup, 0)

    rank, world, local, pg = dist_setup(args.gpus)
    p, wp2, nu2, B0, desc, _, ext, trail = workload(args.workload, K + W + 1)
    L = ext.pmllen if ext is not None else 10
    per_cell = trail is not None
    cells = p.Nx * p.Ny * p.Nz

    if args.impl == "reference":
        if rank != 0:
            return
        cb = cpu_baseline(args.workload, K + W)
        line = {"impl": "reference", "metric": "Gcell-updates/s", "value": cb["value"],
                "unit": "Gcell-updates/s", "n_gpus": args.gpus, "steps": K, "warmup": W,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic",
                "config": {"workload": desc, "grid": [p.Nx, p.Ny, p.Nz]},
                "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "Gcell-updates/s",
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    from meteorscattering_gb300 import build as B
    B.build()
    from meteorscattering_gb300 import engine as E

    form = E.FORM_FP32_FUSED if args.form == "fp32" else E.FORM_FP64_PLAIN
    device = local
    pb = make_problem(E, p, wp2, nu2, B0, ext, trail)
    sim = E.Simulation(pb, form=form, device=device, profile=True)
    plasma = sim.plasma_fraction()
    if W:
        sim.advance(W)
    sim.sync()
    clk = ClockSampler(device)
    clk.start()
    barrier(pg)
    t0 = time.perf_counter()
    sim.advance(K)  # events around the K steps on the simulation's stream
    sim.sync()
    wall = time.perf_counter() - t0
    barrier(pg)
    clocks = clk.stop()
    ms_step, launches = sim.last_timing()
    kstats = sim.kernel_stats()
    sim.close()
    ms_step = max_over_ranks(pg, ms_step)
    value = cells * world / (ms_step * 1e-3) / 1e9

    # dominant kernel roofline
    dom = max(kstats, key=lambda r: r[1] * r[2]) if kstats else None
    peak, peak_kind = load_peaks()
    roof = None
    if dom:
        # achieved / frac: the bytes this step must move (E and H read and
        # written everywhere; J and the per-cell plasma map read and written in
        # the (plane, tile) blocks holding plasma only, since J is identically
        # zero elsewhere; every psi cell of both half-steps read and written)
        # over the dominant launch's time.  per_cell_update: the same launch
        # against the per-cell-update figure of the hot-path table (76 B for
        # the FP32 pass with J and the map counted in every cell), which counts
        # J traffic the pass does not have and so is not a DRAM efficiency.
        alg76 = algorithmic_bytes(args.form, dom[0], p, L, per_cell)
        alg_own = algorithmic_bytes(args.form, dom[0], p, L, per_cell, plasma)
        secs = dom[1] * 1e-3
        ach = alg_own / secs / 1e9
        traffic = traffic_per_launch(args.form, args.workload, dom[0], p, L, plasma, per_cell)
        roof = {"kernel": dom[0], "bound": "hbm", "achieved": ach, "peak": peak,
                "unit": "GB/s", "frac": ach / peak, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": alg_own, "avg_launch_ms": dom[1],
                "plasma_block_fraction": plasma,
                "traffic": traffic,
                "traffic_over_algorithmic": traffic / alg_own if traffic else None,
                "per_cell_update": {"bytes_per_launch": alg76, "achieved": alg76 / secs / 1e9,
                                    "frac": alg76 / secs / 1e9 / peak},
                "kernel_times_ms": {n: m for n, m, c in kstats},
                # the same compulsory bytes over the whole step (every kernel of it)
                "step_achieved": alg_own / (ms_step * 1e-3) / 1e9,
                "step_frac": alg_own / (ms_step * 1e-3) / 1e9 / peak}

    # end to end through the public API from host buffers
    e2e = None
    if not args.no_e2e:
        barrier(pg)
        t0 = time.perf_counter()
        pb2 = make_problem(E, p, wp2, nu2, B0, ext, trail)
        s2 = E.Simulation(pb2, form=form, device=device)
        s2.advance(K)
        ntf = s2.read_ntf()
        s2.close()
        pb2.close()
        t_e2e = max_over_ranks(pg, time.perf_counter() - t0)
        h2d = (wp2.nbytes + nu2.nbytes) / K
        e2e = {"value": cells * world * K / t_e2e / 1e9, "unit": "Gcell-updates/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": ntf.nbytes / K,
               "wall_s": t_e2e,
               "includes": "problem set-up from host arrays, device allocation + upload, "
                           "K steps, D2H of the near-to-far-field sums"}

    # The FP64 plain form on the same workload (the FP32 form's comparison
    # target), and the batched sweep of 128 random trails, on one GPU.
    plain = None
    if rank == 0 and world == 1 and args.form == "fp32" and not args.no_plain:
        pm = plain_fp64_rate(p, wp2, nu2, B0, ext, trail, steps=min(3, K))
        plain = {"ms_per_step": pm, "gcell_updates_per_s": cells / (pm * 1e-3) / 1e9,
                 "fp32_over_fp64": pm / ms_step, "steps": min(3, K),
                 "how": "same workload and API, FP64 plain form, one warm-up step then CUDA-event "
                        "device time of the timed steps"}
    sweep_summary = None
    if rank == 0 and world == 1 and args.form == "fp32" and not args.no_sweep:
        sweep_summary = run_population("sweep")

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(args.workload, K)
        except Exception as ex:  # report, never fake
            cpu = {"value": None, "error": str(ex)[:200]}

    if rank == 0:
        line = {"metric": "Gcell-updates/s", "value": value, "unit": "Gcell-updates/s",
                "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32" if args.form == "fp32" else "f64", "data": "synthetic",
                "config": {"workload": desc, "grid": [p.Nx, p.Ny, p.Nz],
                           "form": "fp32_fused" if args.form == "fp32" else "fp64_plain",
                           "parallelism": f"replicas x{world}",
                           "l2": "state larger than L2 (no flush needed)"},
                "hbm_gbs": roof["achieved"] if roof else None,
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
                "gpu_launches": launches, "host_wall_s": wall,
                "plain_fp64": plain, "sweep": sweep_summary}
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
