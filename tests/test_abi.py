"""CPU checks of the C ABI boundary: the library loads without a GPU, exports every symbol
include/gbsph.h declares, host-only entry points behave, null handles are rejected, and the
C++ class surface header compiles against the C header."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

import libcl_gb300 as gb

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"GBSPH_API\s+[^;(]*?\b(gbsph_\w+)\s*\(", text, re.S))
    return names


def test_library_exports_every_declared_symbol():
    lib = gb.load_library()
    names = declared_symbols()
    assert len(names) >= 28
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python bindings know every one of them
    assert not (names - set(gb.SIGNATURES)), names - set(gb.SIGNATURES)


def test_only_abi_symbols_are_exported():
    out = subprocess.run(["nm", "-D", "--defined-only", str(gb.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    ours = {s for s in exported if s.startswith("gbsph_")}
    assert ours == declared_symbols()


def test_status_strings_and_version():
    lib = gb.load_library()
    assert lib.gbsph_status_string(gb.OK) == b"GBSPH_OK"
    assert lib.gbsph_status_string(gb.ERR_DEVICE_TIMEOUT) == b"GBSPH_ERR_DEVICE_TIMEOUT"
    assert lib.gbsph_status_string(12345) == b"GBSPH_ERR_UNKNOWN"
    assert lib.gbsph_version() >= 10000


def test_null_handles_are_rejected_without_a_device():
    lib = gb.load_library()
    n = None
    assert lib.gbsph_radix_sort_destroy(n) == gb.ERR_ARGUMENT
    assert lib.gbsph_radix_sort_compute(n, n, n, 1, 1, 0, 32, n) == gb.ERR_ARGUMENT
    assert lib.gbsph_fluid3d_compute(n, n) == gb.ERR_ARGUMENT
    assert lib.gbsph_fluid3d_stage(n, 0, n) == gb.ERR_ARGUMENT
    assert lib.gbsph_fluid3d_set_buffer(n, 0, n, 0) == gb.ERR_ARGUMENT
    assert lib.gbsph_fluid3d_get_particle_count(n) == 0
    assert not lib.gbsph_fluid3d_get_params(n)
    assert lib.gbsph_radix_sort_create(None) == gb.ERR_ARGUMENT
    assert lib.gbsph_fluid3d_create(None) == gb.ERR_ARGUMENT


def test_default_params_match_the_restated_clInitFluid(olib):
    p = gb.default_params()
    q = gb.Fluid3DParams()
    olib.init_fluid_params(q)
    for name, _ in gb.Fluid3DParams._fields_[:13]:
        assert getattr(p, name) == getattr(q, name), name
    import numpy as np
    assert np.array_equal(np.array(list(p.gravity), np.float32), np.float32(-9.8) * np.array([0, 0, 1, 0], np.float32))
    assert list(p.boxMin)[:3] == [-1, -1, -1] and list(p.boxMax)[:3] == [1, 1, 1]
    assert p.keyMode == gb.KEY_REFERENCE_HASH and p.dims == 3


def test_params_derive_3d_and_2d():
    import math
    p = gb.Fluid3DParams()
    p.cellSize, p.viscosity, p.dims = 0.02, 0.05, 3
    gb.params_derive(p)
    h = 0.02
    assert math.isclose(p.kernelConstant, 315 / (64 * math.pi * h ** 9), rel_tol=1e-6)
    assert math.isclose(p.pressureConstant, 45 / (math.pi * h ** 6), rel_tol=1e-6)
    assert math.isclose(p.viscosityConstant, 0.05 * 45 / (math.pi * h ** 6), rel_tol=1e-6)
    p.dims, p.cellSize, p.viscosity = 2, 0.01, 0.1
    gb.params_derive(p)
    h = 0.01
    assert math.isclose(p.kernelConstant, 4 / (math.pi * h ** 8), rel_tol=1e-6)
    assert math.isclose(p.pressureConstant, 30 / (math.pi * h ** 5), rel_tol=1e-6)
    assert math.isclose(p.viscosityConstant, 0.1 * 40 / (math.pi * h ** 5), rel_tol=1e-6)


def test_2d_kernel_normalisations_integrate_to_one():
    """The 2D constants used by params_derive: poly6 4/(pi h^8)(h^2-r^2)^3 and spiky
    10/(pi h^5)(h-r)^3 integrate to 1 over the disc (the spiky gradient and viscosity
    Laplacian constants 30/(pi h^5) and 40/(pi h^5) derive from them)."""
    import numpy as np
    h = 0.01
    r = np.linspace(0, h, 200001)
    dr = r[1] - r[0]
    poly6 = 4 / (np.pi * h ** 8) * (h * h - r * r) ** 3
    spiky = 10 / (np.pi * h ** 5) * (h - r) ** 3
    for w in (poly6, spiky):
        assert abs(np.trapezoid(2 * np.pi * r * w, dx=dr) - 1.0) < 1e-6


def test_struct_layout_matches_header():
    assert ctypes.sizeof(gb.Fluid3DParams) == 13 * 4 + 4 * 16 + 16 + 4 * 4
    assert gb.Fluid3DParams.gravity.offset == 52
    assert gb.Fluid3DParams.keyMode.offset == 52 + 64 + 16


def test_cpp_class_surface_compiles(tmp_path):
    """The header-only C++ mirror of oclFluid3D / oclRadixSort builds against the C ABI."""
    src = tmp_path / "t.cpp"
    src.write_text('#include "gbFluid3D.hpp"\nint main(){ return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", str(ROOT / "include"),
                        "-I", "/usr/local/cuda/include", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
