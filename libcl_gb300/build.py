"""Builds the CUDA library (sm_103a) and the CPU oracle, in tree.

`python -m libcl_gb300.build` compiles `libcl_gb300/csrc/*.cu` into
`libcl_gb300/_lib/libgbsph.so` with one nvcc process per translation unit (in parallel)
and a final link; no cmake. `build_oracle()` compiles `oracle/*.cpp` into
`oracle/_build/liboracle.so` (test infrastructure: used only by tests, smoke and the
bench's CPU-baseline leg).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "libcl_gb300"
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libgbsph.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# No fast-math: keys need IEEE division, the exact kernels IEEE sqrt/division.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler",
              "-fPIC,-fvisibility=hidden,-O2", "-I", str(ROOT / "include")]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compiles every .cu for sm_103a and links libgbsph.so."""
    LIBDIR.mkdir(parents=True, exist_ok=True)
    objdir = LIBDIR / "obj"
    objdir.mkdir(exist_ok=True)
    srcs, hdrs = _sources(), _headers()
    jobs = []
    for s in srcs:
        o = objdir / (s.stem + ".o")
        if force or _stale(o, [s] + hdrs):
            jobs.append([NVCC, *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd in jobs:
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
            list(ex.map(_run, jobs))
    objs = [objdir / (s.stem + ".o") for s in srcs]
    if force or jobs or _stale(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcuda"])
    return LIB


def build_oracle(force: bool = False) -> Path:
    """Compiles the CPU restatement (test infrastructure) into oracle/_build/liboracle.so."""
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    srcs = sorted(ORACLE_DIR.glob("*.cpp"))
    if force or _stale(ORACLE_LIB, srcs + [ROOT / "include" / "gbsph.h"]):
        _run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
              "-shared", "-fPIC", "-o", str(ORACLE_LIB), *map(str, srcs)])
    return ORACLE_LIB


def build(force: bool = False, verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, force, verbose)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
