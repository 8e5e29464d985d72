"""CPU: the N > 1 path of bench.py, world size 2 over gloo.

The path has no data exchange: each rank runs an independent replica, the
ranks meet at a barrier around the timed region, and the job's time is the
slowest rank's (max over ranks).  The reference arm runs on rank 0 alone; the
other ranks exit 0 without work.  Ranks are separate processes that find each
other through MASTER_ADDR/MASTER_PORT on 127.0.0.1, as under torchrun.
"""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_CODE = """
import json, sys
sys.path.insert(0, {root!r})
import bench
rank, world, local, pg = bench.dist_setup(2)
bench.barrier(pg)
v = bench.max_over_ranks(pg, 1.0 + 2.5 * rank)
bench.barrier(pg)
print(json.dumps({{"rank": rank, "world": world, "local": local, "max": v}}), flush=True)
pg.destroy_process_group()
"""


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _run_ranks(argv, timeout=240):
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(r), WORLD_SIZE="2",
                   LOCAL_RANK=str(r))
        procs.append(subprocess.Popen(argv, cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                      text=True))
    outs = []
    try:
        for p in procs:
            outs.append(p.communicate(timeout=timeout))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
                p.wait()
    return procs, outs


def _json_lines(text):
    return [json.loads(ln) for ln in text.splitlines() if ln.startswith("{")]


def test_replica_barrier_and_max_over_ranks():
    procs, outs = _run_ranks([sys.executable, "-c", RANK_CODE.format(root=ROOT)])
    assert [p.returncode for p in procs] == [0, 0], [o[1][-2000:] for o in outs]
    got = sorted((d for o in outs for d in _json_lines(o[0])), key=lambda d: d["rank"])
    assert [d["rank"] for d in got] == [0, 1]
    assert all(d["world"] == 2 and d["local"] == d["rank"] and d["max"] == 3.5 for d in got)


def test_reference_arm_runs_on_rank_zero_only():
    argv = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "cfg1",
            "--gpus", "2", "--steps", "2", "--warmup", "1"]
    procs, outs = _run_ranks(argv)
    assert [p.returncode for p in procs] == [0, 0], [o[1][-2000:] for o in outs]
    rank0, rank1 = _json_lines(outs[0][0]), _json_lines(outs[1][0])
    assert len(rank0) == 1 and rank1 == []
    line = rank0[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["cores"] >= 1
