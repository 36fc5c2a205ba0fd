"""Recipe that builds the reference's own kernels for the host cores (TEST INFRASTRUCTURE).

    python -m oracle.ref.build [--force]

1. Reads libCL/phys/oclFluid3D.cl, libCL/phys/oclFluid2D.cl, libCL/sort/oclRadixSort.cl,
   libCL/geom/oclBvhTrimesh.cl and libCL/geom/oclBvhLines.cl from the reference checkout
   (LIBCL_REFERENCE, default /root/reference) and writes their C++ translations
   (oracle/ref/rewrite.py: comments blanked, vector literals, __local, barrier kernels as
   coroutines, lockstep butterfly steps) to oracle/_ref/gen/. Nothing from the reference is
   copied into the repository: oracle/_ref/ is git-ignored.
2. Compiles the translations with the shim (oracle/ref/clshim.h) and the drivers
   (oracle/ref/ref3d.cpp, ref2d.cpp, refsort.cpp, refbvh.cpp, which enqueue the kernels as
   the reference's host classes do) into oracle/_ref/libclref.so with g++ (C++20, OpenMP,
   -ffp-contract=off so that x86 and Arm give the same bits).

Where the reference checkout is absent (a machine that only received a copy of this tree),
step 1 is skipped and step 2 uses the translations already in oracle/_ref/gen/, if any.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
GEN = OUT / "gen"
LIB = OUT / "libclref.so"
REFERENCE = Path(os.environ.get("LIBCL_REFERENCE", "/root/reference")) / "libCL"
SOURCES = {
    "oclFluid3D.cl.inc": "phys/oclFluid3D.cl",
    "oclFluid2D.cl.inc": "phys/oclFluid2D.cl",
    "oclRadixSort.cl.inc": "sort/oclRadixSort.cl",
    "oclBvhTrimesh.cl.inc": "geom/oclBvhTrimesh.cl",
    "oclBvhLines.cl.inc": "geom/oclBvhLines.cl",
}
DRIVERS = ["ref3d.cpp", "ref2d.cpp", "refsort.cpp", "refbvh.cpp"]


def generate() -> bool:
    """Writes the translations when the reference checkout is present. Returns whether
    every translation exists afterwards."""
    if REFERENCE.is_dir():
        sys.path.insert(0, str(ORACLE.parent))
        from oracle.ref.rewrite import rewrite
        GEN.mkdir(parents=True, exist_ok=True)
        for out, rel in SOURCES.items():
            text = rewrite((REFERENCE / rel).read_text(), f"libCL/{rel}")
            target = GEN / out
            if not target.exists() or target.read_text() != text:
                target.write_text(text)
    return all((GEN / o).exists() for o in SOURCES)


def build(force: bool = False) -> Path | None:
    """Builds oracle/_ref/libclref.so; returns its path, or None when neither the reference
    checkout nor earlier translations are available."""
    if not generate():
        return None
    deps = [GEN / o for o in SOURCES] + [HERE / d for d in DRIVERS] + [HERE / "clshim.h"]
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    cmd = ["g++", "-O2", "-std=c++20", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
           "-w", "-I", str(HERE), "-I", str(GEN), "-o", str(LIB), *[str(HERE / d) for d in DRIVERS]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the reference kernels failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
