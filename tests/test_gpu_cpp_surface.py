"""Builds and runs the C++ drop-in smoke program (tests/cpp/class_surface_smoke.cpp): the
reference's own driver sequence through the header-only class surface over the C ABI."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
pytestmark = pytest.mark.gpu


def test_cpp_class_surface_runs(cuda, tmp_path):
    exe = tmp_path / "class_surface_smoke"
    lib = ROOT / "libcl_gb300" / "_lib"
    cmd = ["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), "-I", "/usr/local/cuda/include",
           str(ROOT / "tests" / "cpp" / "class_surface_smoke.cpp"), "-o", str(exe), "-L", str(lib), "-lgbsph",
           "-L", "/usr/local/cuda/lib64", "-lcudart", f"-Wl,-rpath,{lib}:/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr
