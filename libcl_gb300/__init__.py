"""GB300 (sm_103a) SPH fluid step and radix sort: Python mirror of the C ABI in include/gbsph.h.

The classes keep the names and method names of the reference's C++ classes
(jochenstier/libcl): `RadixSort` <-> `oclRadixSort` (libCL/sort/oclRadixSort.h:22-49),
`Fluid3D` <-> `oclFluid3D` (libCL/phys/oclFluid3D.h:21-123). Device memory and streams come
from PyTorch (plumbing only); every computation runs in the CUDA library `libgbsph.so`,
loaded with ctypes. There is no fallback: if the library is missing, importing the
bindings raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_lib" / "libgbsph.so"

# status codes (include/gbsph.h)
OK = 0
ERR_ARGUMENT = -1
ERR_SIZE_MISMATCH = -2
ERR_TOO_LARGE = -3
ERR_BIT_RANGE = -4
ERR_CUDA = -5
ERR_DEVICE_TIMEOUT = -6
ERR_NOT_COMPILED = -7
ERR_OUT_OF_MEMORY = -8
ERR_DEVICE_RANGE = -9
ERR_STATE = -10

KEY_REFERENCE_HASH = 0
KEY_LINEAR_GRID = 1

BUF_POSITION, BUF_VELOCITY, BUF_FORCE, BUF_SORTED_POSITION, BUF_SORTED_VELOCITY, BUF_INDEX, BUF_CELL, BUF_PARAMS = range(8)
(STAGE_HASH, STAGE_SORT, STAGE_REORDER, STAGE_BOUNDS, STAGE_DENSITY, STAGE_FORCES, STAGE_CLIP_BOX,
 STAGE_INTEGRATE_FORCE, STAGE_GRAVITY, STAGE_INTEGRATE_VELOCITY) = range(10)
OPT_FUSED, OPT_CUDA_GRAPH, OPT_BRICK_WIDTH, OPT_PROFILE, OPT_RADIX_BITS, OPT_SORT_TILE, OPT_PERSISTENT = range(7)
STAGE_TIME_NAMES = ("front_end", "sort", "bounds", "density", "forces")

REF_BUCKETS = 262144  # cBucketCount, libCL/phys/oclFluid3D.cpp:17


class Fluid3DParams(C.Structure):
    """gbsph_fluid3d_params: oclFluid3D::Params (libCL/phys/oclFluid3D.h:48-63) + extensions."""
    _fields_ = [(n, C.c_float) for n in (
        "deltaTime", "particleRadius", "cellSize", "mass", "viscosity", "pressure", "density",
        "spacing", "stiffness", "viscosityConstant", "pressureConstant", "kernelConstant",
        "velocitylimit")] + [
        ("gravity", C.c_float * 4), ("boxMin", C.c_float * 4), ("boxMax", C.c_float * 4),
        ("gridOrigin", C.c_float * 4), ("gridDim", C.c_int32 * 4), ("keyMode", C.c_int32),
        ("dims", C.c_int32), ("reserved", C.c_int32 * 2)]


class Fluid2DParams(C.Structure):
    """gbsph_fluid2d_params: oclFluid2D::Params (libCL/phys/oclFluid2D.h:42-60)."""
    _fields_ = [("dT", C.c_float), ("h", C.c_float), ("containerW", C.c_float), ("containerH", C.c_float),
                ("cellSize", C.c_float), ("cellCountX", C.c_int32), ("cellCountY", C.c_int32),
                ("particleSize", C.c_float), ("particleMass", C.c_float), ("p0", C.c_float), ("vmax", C.c_float),
                ("B", C.c_float)]


(BUF2D_STATE, BUF2D_SORTED_STATE, BUF2D_INDEX, BUF2D_CELL, BUF2D_PRESSURE, BUF2D_RELAXED, BUF2D_PREVIOUS,
 BUF2D_BORDER_STATE, BUF2D_BORDER_VECTOR) = range(9)

class SceneDesc(C.Structure):
    """gbsph_scene3d_desc: one scene of a batch."""
    _fields_ = [("n_particles", C.c_uint32), ("stiffness", C.c_float), ("viscosity", C.c_float),
                ("boxMin", C.c_float * 3), ("boxMax", C.c_float * 3), ("gridOrigin", C.c_float * 3),
                ("gridDim", C.c_int32 * 3)]


HOOK_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p)
LOG_FN = C.CFUNCTYPE(None, C.c_int, C.c_char_p, C.c_void_p)

# name -> (restype, argtypes); every symbol declared in include/gbsph.h
_P, _I, _SZ, _U32P = C.c_void_p, C.c_int, C.c_size_t, C.POINTER(C.c_uint32)
SIGNATURES = {
    "gbsph_status_string": (C.c_char_p, [_I]),
    "gbsph_version": (_I, []),
    "gbsph_set_logger": (None, [LOG_FN, _P]),
    "gbsph_radix_sort_create": (_I, [C.POINTER(_P)]),
    "gbsph_radix_sort_destroy": (_I, [_P]),
    "gbsph_radix_sort_compute": (_I, [_P, _P, _P, _SZ, _SZ, _I, _I, _P]),
    "gbsph_radix_sort_cell_bounds": (_I, [_P, _P, _SZ, _P, _P, _SZ, _P]),
    "gbsph_radix_sort_sync_status": (_I, [_P, _P]),
    "gbsph_radix_sort_last_error": (C.c_char_p, [_P]),
    "gbsph_radix_sort_noalloc": (_I, [_P, _P, _SZ, _SZ, _I, _I, _P]),
    "gbsph_radix_sort_noalloc_status": (_I, [_P]),
    "gbsph_fluid3d_create": (_I, [C.POINTER(_P)]),
    "gbsph_fluid3d_destroy": (_I, [_P]),
    "gbsph_fluid3d_compile": (_I, [_P]),
    "gbsph_fluid3d_set_particle_count": (_I, [_P, _SZ]),
    "gbsph_fluid3d_get_particle_count": (_SZ, [_P]),
    "gbsph_fluid3d_set_buffer": (_I, [_P, _I, _P, _SZ]),
    "gbsph_fluid3d_get_buffer": (_P, [_P, _I, C.POINTER(_SZ)]),
    "gbsph_fluid3d_get_params": (C.POINTER(Fluid3DParams), [_P]),
    "gbsph_fluid3d_params_derive": (_I, [C.POINTER(Fluid3DParams)]),
    "gbsph_fluid3d_default_params": (_I, [C.POINTER(Fluid3DParams)]),
    "gbsph_fluid3d_set_integrate_hook": (_I, [_P, HOOK_FN, _P]),
    "gbsph_fluid3d_set_option": (_I, [_P, _I, _I]),
    "gbsph_fluid3d_compute": (_I, [_P, _P]),
    "gbsph_fluid3d_compute_host": (_I, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "gbsph_fluid3d_stage": (_I, [_P, _I, _P]),
    "gbsph_fluid3d_get_cell_bounds": (_I, [_P, _P, _P, _SZ, _P]),
    "gbsph_fluid3d_sync_status": (_I, [_P, _P]),
    "gbsph_fluid3d_last_error": (C.c_char_p, [_P]),
    "gbsph_fluid3d_stage_times": (_I, [_P, C.POINTER(C.c_float), _I]),
    "gbsph_batch3d_create": (_I, [C.POINTER(_P)]),
    "gbsph_batch3d_destroy": (_I, [_P]),
    "gbsph_batch3d_set_scenes": (_I, [_P, C.POINTER(Fluid3DParams), C.POINTER(SceneDesc), _I]),
    "gbsph_batch3d_get_buffer": (_P, [_P, _I, C.POINTER(_SZ)]),
    "gbsph_batch3d_scene_range": (_I, [_P, _I, C.POINTER(_SZ), C.POINTER(_SZ)]),
    "gbsph_batch3d_set_option": (_I, [_P, _I, _I]),
    "gbsph_batch3d_get_option": (_I, [_P, _I, C.POINTER(_I)]),
    "gbsph_batch3d_compute": (_I, [_P, _P]),
    "gbsph_batch3d_autotune": (_I, [_P, _P, C.POINTER(_I)]),
    "gbsph_batch3d_sync_status": (_I, [_P, _P]),
    "gbsph_batch3d_last_error": (C.c_char_p, [_P]),
    "gbsph_fluid2d_create": (_I, [C.POINTER(_P)]),
    "gbsph_fluid2d_destroy": (_I, [_P]),
    "gbsph_fluid2d_compile": (_I, [_P]),
    "gbsph_fluid2d_default_params": (_I, [C.POINTER(Fluid2DParams)]),
    "gbsph_fluid2d_set_particle_count": (_I, [_P, _SZ]),
    "gbsph_fluid2d_get_particle_count": (_SZ, [_P]),
    "gbsph_fluid2d_set_state_buffer": (_I, [_P, _P, _SZ]),
    "gbsph_fluid2d_get_buffer": (_P, [_P, _I, C.POINTER(_SZ)]),
    "gbsph_fluid2d_get_params": (C.POINTER(Fluid2DParams), [_P]),
    "gbsph_fluid2d_compute_border": (_I, [_P, _P, _I, _I, _P]),
    "gbsph_fluid2d_compute": (_I, [_P, _P]),
    "gbsph_fluid2d_get_cell_bounds": (_I, [_P, _P, _P, _SZ, _P]),
    "gbsph_fluid2d_sync_status": (_I, [_P, _P]),
    "gbsph_fluid2d_last_error": (C.c_char_p, [_P]),
    "gbsph_fluid2d_emit": (_I, [_P, C.c_uint32, _P]),
    "gbsph_fluid3d_emit": (_I, [_P, C.c_uint32, C.c_float, _P]),
    "gbsph_bvh_create": (_I, [C.POINTER(_P)]),
    "gbsph_bvh_destroy": (_I, [_P]),
    "gbsph_bvh_compute": (_I, [_P, _P, _SZ, _P, _SZ, _P]),
    "gbsph_bvh_get_node_buffer": (_P, [_P, C.POINTER(_SZ)]),
    "gbsph_bvh_get_node_count": (_SZ, [_P]),
    "gbsph_bvh_get_root_node": (_I, [_P, C.POINTER(C.c_uint32), _P]),
    "gbsph_bvh_get_bounds": (_I, [_P, C.POINTER(C.c_float), _P]),
    "gbsph_bvh_sync_status": (_I, [_P, _P]),
    "gbsph_bvh_last_error": (C.c_char_p, [_P]),
    "gbsph_bvh_collide": (_I, [_P, C.POINTER(Fluid3DParams), _P, _P, _P, _SZ, _P, _SZ, _P, _P]),
    "gbsph_selftest_bounded_wait": (_I, [_I, _P]),
    "gbsph_bvh_lines_create": (_I, [C.POINTER(_P)]),
    "gbsph_bvh_lines_destroy": (_I, [_P]),
    "gbsph_bvh_lines_compute": (_I, [_P, _P, _SZ, _P]),
    "gbsph_bvh_lines_get_node_buffer": (_P, [_P, C.POINTER(_SZ)]),
    "gbsph_bvh_lines_get_node_count": (_SZ, [_P]),
    "gbsph_bvh_lines_get_root_node": (_I, [_P, C.POINTER(C.c_uint32), _P]),
    "gbsph_bvh_lines_sync_status": (_I, [_P, _P]),
    "gbsph_bvh_lines_last_error": (C.c_char_p, [_P]),
    "gbsph_adjoint3d_create": (_I, [C.POINTER(_P), _P, C.c_uint32, C.c_uint32]),
    "gbsph_adjoint3d_destroy": (_I, [_P]),
    "gbsph_adjoint3d_forward": (_I, [_P, _P]),
    "gbsph_adjoint3d_backward": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "gbsph_adjoint3d_last_error": (C.c_char_p, [_P]),
}

_lib = None


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads libgbsph.so (building nothing). Raises if it is missing: there is no fallback."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} not found: build it with `python -m libcl_gb300.build`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class GbsphError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        lib = load_library()
        super().__init__(f"{lib.gbsph_status_string(status).decode()}: {message}")


def status_name(status: int) -> str:
    return load_library().gbsph_status_string(status).decode()


def _ptr(t) -> int:
    return 0 if t is None else int(t.data_ptr())


def _host_ptr(a) -> int:
    """Address of a contiguous float32 host tensor or numpy array."""
    if hasattr(a, "data_ptr"):
        assert not a.is_cuda and a.is_contiguous() and a.element_size() == 4, "a contiguous float32 CPU tensor"
        return a.data_ptr()
    assert a.flags["C_CONTIGUOUS"] and a.dtype.itemsize == 4, "a contiguous float32 array"
    return a.ctypes.data


def _stream(stream) -> int:
    if stream is None:
        import torch
        return int(torch.cuda.current_stream().cuda_stream)
    return int(getattr(stream, "cuda_stream", stream))


class RadixSort:
    """oclRadixSort: stable LSD sort of uint32 (key, value) pairs in place on key bits
    [start_bit, end_bit) (libCL/sort/oclRadixSort.cpp:62-144)."""

    def __init__(self):
        self._lib = load_library()
        h = C.c_void_p()
        rc = self._lib.gbsph_radix_sort_create(C.byref(h))
        if rc:
            raise GbsphError(rc, "gbsph_radix_sort_create")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.gbsph_radix_sort_destroy(self._h)
            self._h = None

    def last_error(self) -> str:
        return self._lib.gbsph_radix_sort_last_error(self._h).decode()

    def compute_raw(self, keys, values, start_bit: int, end_bit: int, stream=None) -> int:
        """Returns the status code (no raise); keys/values are int32/uint32 CUDA tensors."""
        return self._lib.gbsph_radix_sort_compute(self._h, _ptr(keys), _ptr(values), keys.numel(),
                                                  values.numel(), start_bit, end_bit, _stream(stream))

    def compute(self, keys, values, start_bit: int = 0, end_bit: int = 32, stream=None) -> None:
        rc = self.compute_raw(keys, values, start_bit, end_bit, stream)
        if rc:
            raise GbsphError(rc, self.last_error())

    def cell_bounds(self, sorted_keys, cell_start, cell_end, stream=None) -> None:
        rc = self._lib.gbsph_radix_sort_cell_bounds(self._h, _ptr(sorted_keys), sorted_keys.numel(),
                                                    _ptr(cell_start), _ptr(cell_end), cell_start.numel(),
                                                    _stream(stream))
        if rc:
            raise GbsphError(rc, self.last_error())

    def sync_status(self, stream=None) -> int:
        return self._lib.gbsph_radix_sort_sync_status(self._h, _stream(stream))


class Fluid3D:
    """oclFluid3D (libCL/phys/oclFluid3D.h:21-123): construct, compile(), set buffers,
    compute(), read position/velocity and the sorted buffers (.w = density / pressure)."""

    EVT_INTEGRATE = "OnIntegrate"
    cLocalSize = 256
    cBucketCount = REF_BUCKETS

    def __init__(self):
        self._lib = load_library()
        h = C.c_void_p()
        rc = self._lib.gbsph_fluid3d_create(C.byref(h))
        if rc:
            raise GbsphError(rc, "gbsph_fluid3d_create")
        self._h = h
        self._hook = None
        self._borrowed = {}

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.gbsph_fluid3d_destroy(self._h)
            self._h = None

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def _check(self, rc: int) -> None:
        if rc:
            raise GbsphError(rc, self._lib.gbsph_fluid3d_last_error(self._h).decode())

    def last_error(self) -> str:
        return self._lib.gbsph_fluid3d_last_error(self._h).decode()

    def compile(self) -> None:
        self._check(self._lib.gbsph_fluid3d_compile(self._h))

    def compute(self, stream=None) -> None:
        self._check(self._lib.gbsph_fluid3d_compute(self._h, _stream(stream)))

    def compute_raw(self, stream=None) -> int:
        return self._lib.gbsph_fluid3d_compute(self._h, _stream(stream))

    def compute_host(self, position, velocity, force, position_out=None, velocity_out=None, force_out=None,
                     stream=None) -> None:
        """One step on host-resident state (gbsph_fluid3d_compute_host): CPU float32 tensors or
        arrays [N, 4] (page-locked tensors give the overlapped path); the outputs default to
        the inputs. Asynchronous on `stream`: synchronise before reading the outputs."""
        outs = [position if position_out is None else position_out, velocity if velocity_out is None else velocity_out,
                force if force_out is None else force_out]
        self._check(self._lib.gbsph_fluid3d_compute_host(self._h, _host_ptr(position), _host_ptr(velocity),
                                                         _host_ptr(force), *(_host_ptr(o) for o in outs),
                                                         _stream(stream)))

    def stage(self, stage: int, stream=None) -> None:
        self._check(self._lib.gbsph_fluid3d_stage(self._h, stage, _stream(stream)))

    def setParticleCount(self, n: int) -> None:
        self._check(self._lib.gbsph_fluid3d_set_particle_count(self._h, n))

    def getParticleCount(self) -> int:
        return int(self._lib.gbsph_fluid3d_get_particle_count(self._h))

    def getParameters(self) -> Fluid3DParams:
        return self._lib.gbsph_fluid3d_get_params(self._h).contents

    def set_option(self, option: int, value: int) -> None:
        self._check(self._lib.gbsph_fluid3d_set_option(self._h, option, value))

    def _set(self, which: int, tensor) -> int:
        rc = self._lib.gbsph_fluid3d_set_buffer(self._h, which, _ptr(tensor), tensor.numel() // 4)
        if rc == 0:
            self._borrowed[which] = tensor  # keep the borrowed memory alive
        return rc

    def setPositionBuffer(self, t) -> None:
        self._check(self._set(BUF_POSITION, t))

    def setVelocityBuffer(self, t) -> None:
        self._check(self._set(BUF_VELOCITY, t))

    def setForceBuffer(self, t) -> None:
        self._check(self._set(BUF_FORCE, t))

    def buffer(self, which: int):
        """A torch view of one of the library's device buffers (no copy)."""
        import torch
        count = C.c_size_t()
        p = self._lib.gbsph_fluid3d_get_buffer(self._h, which, C.byref(count))
        if not p:
            raise GbsphError(ERR_ARGUMENT, f"no buffer {which}")
        if which in self._borrowed:
            return self._borrowed[which]
        n = count.value
        if which == BUF_PARAMS:  # one gbsph_fluid3d_params record, as float32 words
            words = C.sizeof(Fluid3DParams) // 4
            return _device_view(p, words, torch.float32, (words,))
        is_f4 = which in (BUF_POSITION, BUF_VELOCITY, BUF_FORCE, BUF_SORTED_POSITION, BUF_SORTED_VELOCITY)
        return _device_view(p, n * 4 if is_f4 else n, torch.float32 if is_f4 else torch.int32,
                            (n, 4) if is_f4 else (n,))

    def getPositionBuffer(self):
        return self.buffer(BUF_POSITION)

    def getVelocityBuffer(self):
        return self.buffer(BUF_VELOCITY)

    def getForceBuffer(self):
        return self.buffer(BUF_FORCE)

    def getSortedPositionBuffer(self):
        return self.buffer(BUF_SORTED_POSITION)

    def getSortedVelocityBuffer(self):
        return self.buffer(BUF_SORTED_VELOCITY)

    def getIndexBuffer(self):
        return self.buffer(BUF_INDEX)

    def getCellBuffer(self):
        return self.buffer(BUF_CELL)

    def getParamBuffer(self):
        """getParamBuffer (libCL/phys/oclFluid3D.cpp:198-201): a float32 view of the device copy
        of getParameters() (first 13 words: the kernels' System block), brought up to date by
        this call and by every compute() whose parameters changed."""
        return self.buffer(BUF_PARAMS)

    def cell_bounds(self, n_cells: int, stream=None):
        import torch
        cs = torch.empty(n_cells, dtype=torch.int32, device="cuda")
        ce = torch.empty(n_cells, dtype=torch.int32, device="cuda")
        self._check(self._lib.gbsph_fluid3d_get_cell_bounds(self._h, _ptr(cs), _ptr(ce), n_cells, _stream(stream)))
        return cs, ce

    def addEventHandler(self, fn) -> None:
        """EVT_INTEGRATE hook: fn(fluid, stream_handle) runs in place of the clip/integrate
        stages (libCL/phys/oclFluid3D.cpp:287-291,325-328); return 0 on success."""
        if fn is None:
            self._hook = None
            self._check(self._lib.gbsph_fluid3d_set_integrate_hook(self._h, HOOK_FN(), None))
            return

        def tramp(_h, stream, _user):
            try:
                return int(fn(self, stream) or 0)
            except Exception:  # an exception must not unwind through C
                return -1

        self._hook = HOOK_FN(tramp)
        self._check(self._lib.gbsph_fluid3d_set_integrate_hook(self._h, self._hook, None))

    def sync_status(self, stream=None) -> int:
        return self._lib.gbsph_fluid3d_sync_status(self._h, _stream(stream))

    def emit(self, emit: int, emit_speed: float, stream=None) -> None:
        """clEmitter: particles emit+1 .. emit+99 start on a sheet at y = 0.6."""
        self._check(self._lib.gbsph_fluid3d_emit(self._h, emit, emit_speed, _stream(stream)))

    def stage_times(self) -> dict:
        """Per-stage milliseconds of the last compute() run with OPT_PROFILE on."""
        buf = (C.c_float * 5)()
        n = self._lib.gbsph_fluid3d_stage_times(self._h, buf, 5)
        if n < 0:
            raise GbsphError(n, self.last_error())
        return {STAGE_TIME_NAMES[i]: float(buf[i]) for i in range(n)}


class Adjoint3D:
    """Reverse-mode gradients of `steps` Fluid3D.compute() calls (gbsph_adjoint3d_*):
    forward() advances the fluid keeping a checkpoint every `checkpoint_every` steps;
    backward(dL/dpos, dL/dvel) returns (dL/dpos0, dL/dvel0, dL/dstiffness, dL/dviscosity)."""

    def __init__(self, fluid: Fluid3D, steps: int, checkpoint_every: int = 20):
        self._lib = load_library()
        self.fluid = fluid  # the fluid must outlive the adjoint
        self.steps = steps
        h = C.c_void_p()
        rc = self._lib.gbsph_adjoint3d_create(C.byref(h), fluid.handle, steps, checkpoint_every)
        if rc:
            raise GbsphError(rc, "gbsph_adjoint3d_create")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.gbsph_adjoint3d_destroy(self._h)
            self._h = None

    def _check(self, rc: int) -> None:
        if rc:
            raise GbsphError(rc, self._lib.gbsph_adjoint3d_last_error(self._h).decode())

    def last_error(self) -> str:
        return self._lib.gbsph_adjoint3d_last_error(self._h).decode()

    def forward(self, stream=None) -> None:
        self._check(self._lib.gbsph_adjoint3d_forward(self._h, _stream(stream)))

    def backward_raw(self, grad_pos, grad_vel=None, grad_pos0=None, grad_vel0=None, grad_params=None,
                     stream=None) -> int:
        return self._lib.gbsph_adjoint3d_backward(self._h, _ptr(grad_pos), _ptr(grad_vel), _ptr(grad_pos0),
                                                  _ptr(grad_vel0), _ptr(grad_params), _stream(stream))

    def backward(self, grad_pos, grad_vel=None, stream=None):
        """grad_pos / grad_vel: float32 CUDA tensors [N, 4] (.w ignored). Returns
        (grad_pos0 [N, 4], grad_vel0 [N, 4], grad_params float64 [2] = (d/dstiffness,
        d/dviscosity)), all on the device."""
        import torch
        gp0 = torch.empty_like(grad_pos)
        gv0 = torch.empty_like(grad_pos)
        gpar = torch.empty(2, dtype=torch.float64, device=grad_pos.device)
        self._check(self.backward_raw(grad_pos.contiguous(), None if grad_vel is None else grad_vel.contiguous(),
                                      gp0, gv0, gpar, stream))
        return gp0, gv0, gpar


class BvhTrimesh:
    """oclBvhTrimesh (libCL/geom/oclBvhTrimesh.h:20-84): compute(vertex, index) builds the
    BVH of a triangle mesh; getNodeBuffer / getNodeCount / getRootNode read it. Nodes are
    48-byte records (bbMin[4], bbMax[4], left, right, bit, trav) returned as an int32 tensor
    view [count, 12] (use .view(torch.float32) for the boxes)."""

    NODE_WORDS = 12

    def __init__(self):
        self._lib = load_library()
        h = C.c_void_p()
        rc = self._lib.gbsph_bvh_create(C.byref(h))
        if rc:
            raise GbsphError(rc, "gbsph_bvh_create")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.gbsph_bvh_destroy(self._h)
            self._h = None

    def _check(self, rc: int) -> None:
        if rc:
            raise GbsphError(rc, self._lib.gbsph_bvh_last_error(self._h).decode())

    def compute_raw(self, vertex, index, stream=None) -> int:
        return self._lib.gbsph_bvh_compute(self._h, _ptr(vertex), vertex.numel() // 4, _ptr(index), index.numel(),
                                           _stream(stream))

    def compute(self, vertex, index, stream=None) -> None:
        """vertex: float32 CUDA tensor [V, 4]; index: int32/uint32 CUDA tensor [3 n]."""
        self._check(self.compute_raw(vertex, index, stream))

    def getNodeCount(self) -> int:
        return int(self._lib.gbsph_bvh_get_node_count(self._h))

    def getNodeBuffer(self):
        import torch
        count = C.c_size_t()
        p = self._lib.gbsph_bvh_get_node_buffer(self._h, C.byref(count))
        return _device_view(p, count.value * self.NODE_WORDS, torch.int32, (count.value, self.NODE_WORDS))

    def getRootNode(self, stream=None) -> int:
        r = C.c_uint32()
        self._check(self._lib.gbsph_bvh_get_root_node(self._h, C.byref(r), _stream(stream)))
        return r.value

    def bounds(self, stream=None):
        b = (C.c_float * 8)()
        self._check(self._lib.gbsph_bvh_get_bounds(self._h, b, _stream(stream)))
        return list(b)

    def sync_status(self, stream=None) -> int:
        return self._lib.gbsph_bvh_sync_status(self._h, _stream(stream))

    def collide(self, params: Fluid3DParams, position, velocity, force, vertex, index, stream=None) -> None:
        """clCollideBVH on particle float4 tensors [N, 4] (updated in place) against the mesh
        (vertex [V, 4], index [3 n]) this BVH was last built from."""
        self._check(self._lib.gbsph_bvh_collide(self._h, C.byref(params), _ptr(position), _ptr(velocity), _ptr(force),
                                                position.numel() // 4, _ptr(vertex), vertex.numel() // 4, _ptr(index),
                                                _stream(stream)))


class BvhLines:
    """oclBvhLines (libCL/geom/oclBvhLines.h:20-77): compute(vertex) builds the BVH of 2D line
    segments (two float2 vertices each); getNodeBuffer / getNodeCount / getRootNode read it.
    Nodes are 32-byte records (bbMin[2], bbMax[2], left, right, bit, trav) returned as an int32
    tensor view [count, 8] (use .view(torch.float32) for the boxes)."""

    NODE_WORDS = 8

    def __init__(self):
        self._lib = load_library()
        h = C.c_void_p()
        rc = self._lib.gbsph_bvh_lines_create(C.byref(h))
        if rc:
            raise GbsphError(rc, "gbsph_bvh_lines_create")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.gbsph_bvh_lines_destroy(self._h)
            self._h = None

    def _check(self, rc: int) -> None:
        if rc:
            raise GbsphError(rc, self._lib.gbsph_bvh_lines_last_error(self._h).decode())

    def compute_raw(self, vertex, stream=None) -> int:
        return self._lib.gbsph_bvh_lines_compute(self._h, _ptr(vertex), vertex.numel() // 2, _stream(stream))

    def compute(self, vertex, stream=None) -> None:
        """vertex: float32 CUDA tensor [V, 2], two vertices per segment."""
        self._check(self.compute_raw(vertex, stream))

    def getNodeCount(self) -> int:
        return int(self._lib.gbsph_bvh_lines_get_node_count(self._h))

    def getNodeBuffer(self):
        import torch
        count = C.c_size_t()
        p = self._lib.gbsph_bvh_lines_get_node_buffer(self._h, C.byref(count))
        return _device_view(p, count.value * self.NODE_WORDS, torch.int32, (count.value, self.NODE_WORDS))

    def getRootNode(self, stream=None) -> int:
        r = C.c_uint32()
        self._check(self._lib.gbsph_bvh_lines_get_root_node(self._h, C.byref(r), _stream(stream)))
        return r.value

    def sync_status(self, stream=None) -> int:
        return self._lib.gbsph_bvh_lines_sync_status(self._h, _stream(stream))


class Batch3D:
    """Many independent 3D scenes advanced together (gbsph_batch3d_*)."""

    def __init__(self):
        self._lib = load_library()
        h = C.c_void_p()
        rc = self._lib.gbsph_batch3d_create(C.byref(h))
        if rc:
            raise GbsphError(rc, "gbsph_batch3d_create")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.gbsph_batch3d_destroy(self._h)
            self._h = None

    def _check(self, rc: int) -> None:
        if rc:
            raise GbsphError(rc, self._lib.gbsph_batch3d_last_error(self._h).decode())

    def set_scenes(self, shared: Fluid3DParams, scenes) -> None:
        arr = (SceneDesc * len(scenes))(*scenes)
        self._check(self._lib.gbsph_batch3d_set_scenes(self._h, C.byref(shared), arr, len(scenes)))

    def scene_range(self, s: int):
        first, count = C.c_size_t(), C.c_size_t()
        self._check(self._lib.gbsph_batch3d_scene_range(self._h, s, C.byref(first), C.byref(count)))
        return first.value, count.value

    def buffer(self, which: int):
        import torch
        count = C.c_size_t()
        p = self._lib.gbsph_batch3d_get_buffer(self._h, which, C.byref(count))
        if not p:
            raise GbsphError(ERR_ARGUMENT, f"no buffer {which}")
        n = count.value
        if which in (BUF_INDEX, BUF_CELL):
            return _device_view(p, n, torch.int32, (n,))
        return _device_view(p, n * 4, torch.float32, (n, 4))

    def set_option(self, option: int, value: int) -> None:
        self._check(self._lib.gbsph_batch3d_set_option(self._h, option, value))

    def get_option(self, option: int) -> int:
        v = C.c_int()
        self._check(self._lib.gbsph_batch3d_get_option(self._h, option, C.byref(v)))
        return v.value

    def config(self) -> dict:
        """The step's current launch configuration (what autotune() chose)."""
        return {"brick_width": self.get_option(OPT_BRICK_WIDTH),
                "radix_bits": self.get_option(OPT_RADIX_BITS),
                "sort_tile_items": self.get_option(OPT_SORT_TILE),
                "cuda_graph": self.get_option(OPT_CUDA_GRAPH),
                "persistent": self.get_option(OPT_PERSISTENT)}

    def compute(self, stream=None) -> None:
        self._check(self._lib.gbsph_batch3d_compute(self._h, _stream(stream)))

    def autotune(self, stream=None) -> int:
        best = C.c_int()
        self._check(self._lib.gbsph_batch3d_autotune(self._h, _stream(stream), C.byref(best)))
        return best.value

    def sync_status(self, stream=None) -> int:
        return self._lib.gbsph_batch3d_sync_status(self._h, _stream(stream))


class Fluid2D:
    """oclFluid2D (libCL/phys/oclFluid2D.h:22-138): the reference's 2D double-density
    relaxation model. State is gbsph_particle2d (pos.xy, vel.xy, mass, unused) per particle."""

    cLocalSize = 256

    def __init__(self):
        self._lib = load_library()
        h = C.c_void_p()
        rc = self._lib.gbsph_fluid2d_create(C.byref(h))
        if rc:
            raise GbsphError(rc, "gbsph_fluid2d_create")
        self._h = h
        self._borrowed = None

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.gbsph_fluid2d_destroy(self._h)
            self._h = None

    def _check(self, rc: int) -> None:
        if rc:
            raise GbsphError(rc, self._lib.gbsph_fluid2d_last_error(self._h).decode())

    def compile(self) -> None:
        self._check(self._lib.gbsph_fluid2d_compile(self._h))

    def compute(self, stream=None) -> None:
        self._check(self._lib.gbsph_fluid2d_compute(self._h, _stream(stream)))

    def setParticleCount(self, n: int) -> None:
        self._check(self._lib.gbsph_fluid2d_set_particle_count(self._h, n))

    def getParticleCount(self) -> int:
        return int(self._lib.gbsph_fluid2d_get_particle_count(self._h))

    def getParameters(self) -> Fluid2DParams:
        return self._lib.gbsph_fluid2d_get_params(self._h).contents

    def setStateBuffer(self, t) -> None:
        self._check(self._lib.gbsph_fluid2d_set_state_buffer(self._h, _ptr(t), t.numel() // 6))
        self._borrowed = t

    def computeBorder(self, mask, stream=None) -> None:
        """mask: CUDA float32 tensor [H, W, 4]; .w == 1 marks wall pixels."""
        h, w = mask.shape[0], mask.shape[1]
        self._check(self._lib.gbsph_fluid2d_compute_border(self._h, _ptr(mask), w, h, _stream(stream)))

    def buffer(self, which: int):
        import torch
        count = C.c_size_t()
        p = self._lib.gbsph_fluid2d_get_buffer(self._h, which, C.byref(count))
        if not p:
            raise GbsphError(ERR_ARGUMENT, f"no buffer {which}")
        if which == BUF2D_STATE and self._borrowed is not None:
            return self._borrowed
        n = count.value
        cols = {BUF2D_STATE: 6, BUF2D_SORTED_STATE: 6, BUF2D_PRESSURE: 4, BUF2D_RELAXED: 2, BUF2D_PREVIOUS: 2,
                BUF2D_BORDER_STATE: 4, BUF2D_BORDER_VECTOR: 4}.get(which)
        if cols is None:
            return _device_view(p, n, torch.int32, (n,))
        return _device_view(p, n * cols, torch.float32, (n, cols))

    def getStateBuffer(self):
        return self.buffer(BUF2D_STATE)

    def cell_bounds(self, n_cells: int, stream=None):
        import torch
        cs = torch.empty(n_cells, dtype=torch.int32, device="cuda")
        ce = torch.empty(n_cells, dtype=torch.int32, device="cuda")
        self._check(self._lib.gbsph_fluid2d_get_cell_bounds(self._h, _ptr(cs), _ptr(ce), n_cells, _stream(stream)))
        return cs, ce

    def sync_status(self, stream=None) -> int:
        return self._lib.gbsph_fluid2d_sync_status(self._h, _stream(stream))

    def emit(self, emit: int, stream=None) -> None:
        """clEmitter: particle emit+1 enters at x = 1 with velocity (25, 1)."""
        self._check(self._lib.gbsph_fluid2d_emit(self._h, emit, _stream(stream)))


def default_params_2d() -> Fluid2DParams:
    p = Fluid2DParams()
    rc = load_library().gbsph_fluid2d_default_params(C.byref(p))
    if rc:
        raise GbsphError(rc, "default_params_2d")
    return p


def params_derive(p: Fluid3DParams) -> None:
    rc = load_library().gbsph_fluid3d_params_derive(C.byref(p))
    if rc:
        raise GbsphError(rc, "params_derive")


def default_params() -> Fluid3DParams:
    """The parameters compile() loads (clInitFluid, libCL/phys/oclFluid3D.cl:130-148)."""
    p = Fluid3DParams()
    rc = load_library().gbsph_fluid3d_default_params(C.byref(p))
    if rc:
        raise GbsphError(rc, "default_params")
    return p


class _CudaArrayView:
    """Minimal __cuda_array_interface__ provider to wrap library-owned device memory."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3, "strides": None}


def _device_view(ptr: int, numel: int, dtype, shape):
    import torch
    typestr = "<f4" if dtype == torch.float32 else "<i4"
    return torch.as_tensor(_CudaArrayView(ptr, shape, typestr), device="cuda")
