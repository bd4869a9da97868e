"""Build the GB300 library (sm_103a) and the CPU oracle, in place.

    python hr-weno_gb300/build.py            # library + oracle
    python hr-weno_gb300/build.py --lib      # library only

Outputs (git-ignored):
    hr-weno_gb300/hrweno/_lib/libhrweno_gb300.so   the product: CUDA kernels + C ABI
    oracle/_build/libhrweno_oracle.so              the test oracle (CPU restatement)

Translation units compile in parallel with one -gencode each; no cmake.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "hrweno" / "_lib"
LIB = LIBDIR / "libhrweno_gb300.so"
ORACLE_SRC = ROOT / "oracle" / "hrweno_oracle.cpp"
ORACLE_LIB = ROOT / "oracle" / "_build" / "libhrweno_oracle.so"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# the oracle: no fused multiply-add (the reference's operation order), OpenMP over the 1D
# cell loops for the multi-core CPU baseline (results are bit-identical for any thread count)
ORACLE_FLAGS = ["-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-std=c++17"]
# the CPU baseline's build of the same source: -O3 and the compiler's default contraction (as
# a gfortran -O3 build of the reference would be); it only times the baseline.  No
# -march=native: the same flags build on the x86-64 host and the aarch64 GPU host.
ORACLE_BASELINE_LIB = ROOT / "oracle" / "_build" / "libhrweno_oracle_o3.so"
ORACLE_BASELINE_FLAGS = ["-O3", "-fopenmp", "-fPIC", "-shared", "-std=c++17"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# sources whose kernel instantiations are split over several objects, each compiled with
# -DHRW_PART=i, so that the longest translation units build in parallel
PARTS = {"stage2d.cu": 9, "batch.cu": 3, "stage2d_f32c.cu": 2}
# the slowest units first, so that they do not start last
SLOW_FIRST = ["stage2d.cu", "batch.cu", "stage1d_f32c.cu", "stage2d_f32c.cu", "stage1d.cu"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_lib(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"),
                     key=lambda p: (SLOW_FIRST.index(p.name) if p.name in SLOW_FIRST else len(SLOW_FIRST), p.name))
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "hrweno_gpu.h"]
    jobs = []
    objs = []
    for src in sources:
        n = PARTS.get(src.name, 0)
        for part in range(n) if n else [None]:
            obj = BUILD / (src.stem + (f".p{part}" if part is not None else "") + ".o")
            objs.append(obj)
            if force or _stale(obj, [src] + headers):
                extra = [f"-DHRW_PART={part}"] if part is not None else []
                jobs.append([NVCC, *ARCH, *NVFLAGS, *extra, "-c", str(src), "-o", str(obj)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    return LIB


def build_oracle(force: bool = False) -> Path:
    """The parity build of the oracle, and its -O3 build that times the CPU baseline."""
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    deps = [ORACLE_SRC, ROOT / "include" / "hrweno_gpu.h"]
    if force or _stale(ORACLE_LIB, deps):
        _run(["g++", *ORACLE_FLAGS, "-o", str(ORACLE_LIB), str(ORACLE_SRC)])
    if force or _stale(ORACLE_BASELINE_LIB, deps):
        _run(["g++", *ORACLE_BASELINE_FLAGS, "-o", str(ORACLE_BASELINE_LIB), str(ORACLE_SRC)])
    return ORACLE_LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_lib(force))
    if "--lib" not in sys.argv:
        print(build_oracle(force))
