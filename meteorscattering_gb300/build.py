"""In-tree build of the engine: CUDA kernels for sm_103a plus the C++ host.

Produces, under ``meteorscattering_gb300/_lib/``:

* ``libmfdtd.so`` -- the C-ABI library declared in ``include/mfdtd.h``;
* ``meteor``      -- the drop-in replacement of the reference executable.

Translation units compile in parallel; only ``-gencode
arch=compute_103a,code=sm_103a`` is generated.  The FP64 plain-form kernels and
the host set-up code are compiled without FMA contraction (``-fmad=false`` /
``-ffp-contract=off``) because they reproduce the reference's rounding.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "_lib")
OBJ = os.path.join(LIB, "obj")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-Xptxas", "-v"] + ARCH
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-result",
            "-ffp-contract=off", f"-I{CUDA_HOME}/include"]

# (source, extra flags)
CUDA_UNITS = [
    ("plain_fp64.cu", ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]),
    ("fp32_fused.cu", []),
    ("farfield.cu", []),
]
CXX_UNITS = ["problem.cpp", "sim.cpp"]


def _run(cmd, log):
    r = subprocess.run(cmd, capture_output=True, text=True)
    log.append((cmd, r.returncode, r.stdout + r.stderr))
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile everything; return the path of ``libmfdtd.so``."""
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".hpp", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "mfdtd.h"))
    jobs, objs, log = [], [], []
    for src, extra in CUDA_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([NVCC, "-c", s, "-o", o] + NVFLAGS + extra)
    for src in CXX_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append(["g++", "-c", s, "-o", o] + CXXFLAGS)
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        list(ex.map(lambda c: _run(c, log), jobs))
    so = os.path.join(LIB, "libmfdtd.so")
    if force or jobs or not os.path.exists(so):
        _run([NVCC, "-shared", "-o", so] + objs + ARCH + ["-Xcompiler", "-fPIC"], log)
    exe = os.path.join(LIB, "meteor")
    main_src = os.path.join(CSRC, "meteor_main.cpp")
    if force or jobs or not _newer(exe, [main_src, so]):
        _run(["g++", "-O2", "-std=c++17", "-o", exe, main_src, f"-L{LIB}", "-lmfdtd",
              "-Wl,-rpath,$ORIGIN"], log)
    if verbose:
        for cmd, rc, out in log:
            print(" ".join(cmd))
            if out.strip():
                print(out)
    return so


def build_oracle(with_reference: bool = True) -> None:
    """Build the CPU oracle (test infrastructure) and, where the reference
    sources are present, the reference binaries."""
    make = shutil.which("make")
    if make is None:
        raise RuntimeError("make not found")
    subprocess.run([make, "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    if with_reference:
        # The recipe knows where the reference sources lie (REFSRC, or the
        # MFDTD_REFSRC environment variable) and skips them when absent.
        subprocess.run([make, "-s", "-C", os.path.join(ROOT, "oracle"), "ref-if-present"], check=True)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    build_oracle()
