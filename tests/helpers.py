"""Test helpers: run the oracle / reference / engine on run directories and
compare their output files."""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import resource
import shutil
import subprocess
import tempfile

import numpy as np

from meteorscattering_gb300 import rundir as rd

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
REF_FORK = os.path.join(ROOT, "oracle", "_ref", "meteor_fork")
REF_21 = os.path.join(ROOT, "oracle", "_ref", "meteor_21")
OUTPUTS = ("output_E.dat", "output_H.dat", "output_J.dat", "output_NTF.dat", "Probe.dat")

_oracle = None


def oracle_lib():
    global _oracle
    if _oracle is None:
        lib = C.CDLL(ORACLE_SO)
        lib.oracle_run_dir.restype = C.c_int
        lib.oracle_run_dir.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int,
                                       C.POINTER(C.c_double)]
        _oracle = lib
    return _oracle


def run_oracle(d: str, max_steps: int = -1, nthreads: int = 0) -> float:
    secs = C.c_double()
    rc = oracle_lib().oracle_run_dir(os.fsencode(d), max_steps, nthreads, 0, C.byref(secs))
    if rc != 0:
        raise RuntimeError(f"oracle failed in {d}: {rc}")
    return secs.value


def _unlimited_stack():
    resource.setrlimit(resource.RLIMIT_STACK, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))


def run_reference(d: str, exe: str = REF_FORK) -> None:
    r = subprocess.run([exe], cwd=d, preexec_fn=_unlimited_stack, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference failed in {d}: {r.stderr}")


def fresh_dir(tmp_path, name, case) -> str:
    p, wp, nu, B0 = case
    d = os.path.join(str(tmp_path), name)
    shutil.rmtree(d, ignore_errors=True)
    rd.write_rundir(d, p, wp, nu, B0)
    return d


def comparable_bytes(path: str, name: str, nntf: int, skip_srcdft: bool) -> bytes:
    with open(path, "rb") as f:
        b = f.read()
    if skip_srcdft and name == "output_NTF.dat":
        o = 8 + 8 * nntf
        b = b[:o] + b[o + 32 * nntf:]
    return b


def diff_outputs(da: str, db: str, nntf: int, skip_srcdft: bool = False):
    """Names of output files whose bytes differ (missing on one side counts)."""
    bad = []
    for name in OUTPUTS:
        pa, pb = os.path.join(da, name), os.path.join(db, name)
        ea, eb = os.path.exists(pa), os.path.exists(pb)
        if ea != eb:
            bad.append(name + " (missing)")
            continue
        if ea and comparable_bytes(pa, name, nntf, skip_srcdft) != \
                comparable_bytes(pb, name, nntf, skip_srcdft):
            bad.append(name)
    if rd.read_log_maxima(os.path.join(da, "log.txt")) != \
            rd.read_log_maxima(os.path.join(db, "log.txt")):
        bad.append("log.txt maxima")
    return bad


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def sha256_file_bytes(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()
