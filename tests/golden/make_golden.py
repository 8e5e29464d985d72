"""Generate the golden vectors of tests/golden/*.json from the reference solver.

Runs the reference executable built by ``make -C oracle ref`` (from
``source/meteor-fork.cpp``, or ``source/meteor-2.1.cpp`` with ``--v21``) on
every case of ``cases.py`` and stores, per output file:

* its size and SHA-256 (``output_NTF.dat`` without the 4*nntf source-DFT
  doubles, which the reference never initialises -- source/meteor-2.1.cpp:555-556);
* 64 sampled doubles at seeded offsets, as exact hex floats;
* the ``Maximum abs(Ex)`` strings of log.txt.

Usage:  python tests/golden/make_golden.py  (needs oracle/_ref/meteor_fork)
"""
from __future__ import annotations

import hashlib
import json
import os
import platform
import resource
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

from meteorscattering_gb300 import rundir as rd  # noqa: E402
import cases as golden_cases  # noqa: E402

OUTPUTS = ("output_E.dat", "output_H.dat", "output_J.dat", "output_NTF.dat", "Probe.dat")
NSAMPLE = 64


def comparable_bytes(path: str, name: str, nntf: int) -> bytes:
    """File bytes with the uninitialised source-DFT block of output_NTF.dat removed."""
    with open(path, "rb") as f:
        b = f.read()
    if name == "output_NTF.dat":
        o = 8 + 8 * nntf
        b = b[:o] + b[o + 32 * nntf:]
    return b


def sample_offsets(nbytes: int, header: int, seed: int) -> list:
    n = (nbytes - header) // 8
    if n <= 0:
        return []
    rng = np.random.default_rng(seed)
    return sorted(int(v) for v in rng.choice(n, size=min(NSAMPLE, n), replace=False))


def header_bytes(name: str, p: rd.RunParams) -> int:
    if name == "Probe.dat":
        return 4 + 12 * p.nprobes
    if name == "output_NTF.dat":
        return 8 + 8 * p.nntf + 32 * p.nntf
    return 0


def describe_run(d: str, p: rd.RunParams) -> dict:
    out = {}
    for name in OUTPUTS:
        path = os.path.join(d, name)
        if not os.path.exists(path):
            out[name] = None
            continue
        b = comparable_bytes(path, name, p.nntf)
        hdr = header_bytes(name, p) - (32 * p.nntf if name == "output_NTF.dat" else 0)
        offs = sample_offsets(len(b), hdr, seed=len(b))
        vals = [float(np.frombuffer(b, dtype="<f8", count=1, offset=hdr + 8 * o)[0]).hex()
                for o in offs]
        out[name] = {"size": len(b), "sha256": hashlib.sha256(b).hexdigest(),
                     "header": hdr, "offsets": offs, "values": vals}
    out["log_maxima"] = rd.read_log_maxima(os.path.join(d, "log.txt"))
    return out


def _unlimited_stack():
    resource.setrlimit(resource.RLIMIT_STACK, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))


def run_reference(exe: str, d: str) -> None:
    r = subprocess.run([exe], cwd=d, preexec_fn=_unlimited_stack, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference failed in {d}: {r.stderr}")


def main() -> None:
    exe = os.path.join(ROOT, "oracle", "_ref", "meteor_fork")
    if not os.path.exists(exe):
        raise SystemExit("build the reference first: make -C oracle ref")
    for name, (p, wp, nu, B0) in golden_cases.cases().items():
        d = tempfile.mkdtemp(prefix=f"golden_{name}_")
        try:
            rd.write_rundir(d, p, wp, nu, B0)
            run_reference(exe, d)
            rec = {"case": name, "machine": platform.machine(),
                   "generator": "oracle/_ref/meteor_fork (source/meteor-fork.cpp, "
                                "g++ -O2 -fopenmp -ffp-contract=off)",
                   "outputs": describe_run(d, p)}
            with open(os.path.join(HERE, f"{name}.json"), "w") as f:
                json.dump(rec, f, indent=1)
            print("wrote", name)
        finally:
            shutil.rmtree(d, ignore_errors=True)


if __name__ == "__main__":
    main()
