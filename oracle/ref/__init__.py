"""The reference's own kernels on the host cores -- TEST INFRASTRUCTURE ONLY.

ctypes bindings to oracle/_ref/libclref.so, which oracle/ref/build.py compiles from the
reference's OpenCL C sources (libCL/phys/oclFluid3D.cl, libCL/phys/oclFluid2D.cl,
libCL/sort/oclRadixSort.cl, libCL/geom/oclBvhTrimesh.cl, libCL/geom/oclBvhLines.cl) through an
OpenCL C shim (oracle/ref/clshim.h). Each entry point
enqueues the kernels in the order the reference's host class does. Used by the tests to pin
the oracle restatement (oracle/*.cpp) to the reference, and by bench.py's reference arm as
the reference's CPU implementation of the step. The product library never loads it.

`available()` is False where the library cannot be built (no reference checkout and no
earlier translation in oracle/_ref/gen/); callers skip in that case.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

POW_LIBM = 0
POW_INTEGER_CUBE = 1
BUCKETS = 262144
LOCAL_SIZE = 256

_lib = None
_tried = False


def _load():
    global _lib, _tried
    if _tried:
        return _lib
    _tried = True
    from oracle.ref.build import build
    path = build()
    if path is None:
        return None
    lib = C.CDLL(str(path))
    P, U, F, I = C.c_void_p, C.c_uint32, C.c_float, C.c_int
    sig = {
        "clref_radix_sort": (I, [P, P, U, I, I]),
        "clref_set_pow_mode": (None, [I]),
        "clref_set_num_threads": (I, [I]),
        "clref3d_init_fluid": (None, [P]),
        "clref3d_kernel_constants": (None, [F, F, P]),
        "clref3d_step": (I, [P, P, P, U, P, P, P, P, P, P, P, P, P, P, P]),
        "clref3d_emit": (None, [P, P, U, U, F, P]),
        "clref3d_collide_bvh": (None, [P, P, P, U, P, P, U, U, P, P, U]),
        "clref2d_init_fluid": (None, [P]),
        "clref2d_table_size": (U, [P]),
        "clref2d_compute_border": (None, [P, I, I, P, P, P]),
        "clref2d_step": (I, [P, U, P, P, P, I, I, P, P, P, P, P, P, P, P]),
        "clref2d_emit": (None, [P, U, U, P]),
        "clref_bvh_build": (I, [P, U, P, U, P, P, P, P, P]),
        "clref_bvh_lines_build": (I, [P, U, P, P, P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args
    _lib = lib
    return _lib


def available() -> bool:
    return _load() is not None


def lib():
    lb = _load()
    if lb is None:
        raise RuntimeError("the reference kernels are not built (no reference checkout, no translation)")
    return lb


def _p(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def set_pow_mode(mode: int) -> None:
    lib().clref_set_pow_mode(mode)


def set_num_threads(n: int) -> int:
    return int(lib().clref_set_num_threads(n))


def radix_sort(keys: np.ndarray, vals: np.ndarray, start: int, end: int) -> int:
    """oclRadixSort::compute in place on uint32 arrays of equal size; 0 or the reference's
    refusal code (-3 too large, -4 bit range not a multiple of 4)."""
    assert keys.dtype == np.uint32 and vals.dtype == np.uint32 and keys.size == vals.size
    return int(lib().clref_radix_sort(_p(keys), _p(vals), keys.size, start, end))


def system13(params) -> np.ndarray:
    """The reference's 13-float System block: the first 13 fields of a params struct."""
    return np.frombuffer(bytes(params)[:52], np.float32).copy()


def init_fluid3d() -> np.ndarray:
    s = np.zeros(13, np.float32)
    lib().clref3d_init_fluid(_p(s))
    return s


def kernel_constants(cell_size: float, viscosity: float) -> np.ndarray:
    """(kernelConstant, viscosityConstant, pressureConstant) as clInitFluid forms them."""
    out = np.zeros(3, np.float32)
    lib().clref3d_kernel_constants(cell_size, viscosity, _p(out))
    return out


class Step3D:
    def __init__(self, n: int):
        self.cell = np.empty(n, np.uint32)
        self.index = np.empty(n, np.uint32)
        self.spos = np.empty((n, 4), np.float32)
        self.svel = np.empty((n, 4), np.float32)
        self.cell_start = np.empty(BUCKETS, np.uint32)
        self.cell_end = np.empty(BUCKETS, np.uint32)
        self.force_pre = np.empty((n, 4), np.float32)


def step3d(pos, vel, force, system, gravity_arg, box_min, box_max) -> Step3D:
    """One oclFluid3D::compute with the reference's kernels; pos/vel/force float32 [N, 4]
    updated in place (N a multiple of 256). `gravity_arg` is clGravity's float4 argument
    (the stage writes -9.8f * gravity_arg)."""
    n = pos.shape[0]
    r = Step3D(n)
    f4 = lambda v: np.ascontiguousarray(np.asarray(v, np.float32).reshape(4))
    g, lo, hi = f4(gravity_arg), f4(box_min), f4(box_max)
    sysa = np.ascontiguousarray(system, np.float32)
    rc = lib().clref3d_step(_p(pos), _p(vel), _p(force), n, _p(sysa), _p(g), _p(lo), _p(hi), _p(r.cell),
                            _p(r.index), _p(r.spos), _p(r.svel), _p(r.cell_start), _p(r.cell_end), _p(r.force_pre))
    if rc != 0:
        raise ValueError(f"clref3d_step returned {rc}")
    return r


def emit3d(pos, vel, emit: int, speed: float, system) -> None:
    sysa = np.ascontiguousarray(system, np.float32)
    lib().clref3d_emit(_p(pos), _p(vel), pos.shape[0], emit, speed, _p(sysa))


def collide_bvh3d(force, pos, vel, system, nodes, root: int, triangle, vertex) -> None:
    sysa = np.ascontiguousarray(system, np.float32)
    nodes = np.ascontiguousarray(nodes)
    assert nodes.dtype.itemsize == 48
    tri = np.ascontiguousarray(triangle, np.uint32)
    vtx = np.ascontiguousarray(vertex, np.float32)
    lib().clref3d_collide_bvh(_p(force), _p(pos), _p(vel), pos.shape[0], _p(sysa), _p(nodes), nodes.size, root,
                              _p(tri), _p(vtx), vtx.shape[0])


def init_fluid2d(params) -> None:
    """clInitFluid (2D) into a 48-byte params struct (ctypes)."""
    buf = (C.c_char * 48)()
    lib().clref2d_init_fluid(C.addressof(buf))
    C.memmove(C.addressof(params), buf, 48)


def table_size_2d(params) -> int:
    return int(lib().clref2d_table_size(C.addressof(params)))


def compute_border_2d(mask: np.ndarray, params):
    h, w = mask.shape[:2]
    vec = np.empty((h, w, 4), np.float32)
    st = np.empty((h, w, 4), np.float32)
    lib().clref2d_compute_border(_p(np.ascontiguousarray(mask, np.float32)), w, h, C.addressof(params), _p(vec),
                                 _p(st))
    return vec, st


class Step2D:
    def __init__(self, n: int, table: int):
        self.cell = np.empty(n, np.uint32)
        self.index = np.empty(n, np.uint32)
        self.sorted = np.empty((n, 6), np.float32)
        self.pstate = np.empty((n, 4), np.float32)
        self.relaxed = np.empty((n, 2), np.float32)
        self.prev = np.empty((n, 2), np.float32)
        self.cell_start = np.empty(table, np.uint32)
        self.cell_end = np.empty(table, np.uint32)


def step_2d(state: np.ndarray, params, border_state: np.ndarray, border_vec: np.ndarray) -> Step2D:
    """One oclFluid2D::compute with the reference's kernels; state float32 [N, 6] in place."""
    n = state.shape[0]
    h, w = border_state.shape[:2]
    r = Step2D(n, table_size_2d(params))
    rc = lib().clref2d_step(_p(state), n, C.addressof(params), _p(np.ascontiguousarray(border_state, np.float32)),
                            _p(np.ascontiguousarray(border_vec, np.float32)), w, h, _p(r.cell), _p(r.index),
                            _p(r.sorted), _p(r.pstate), _p(r.relaxed), _p(r.prev), _p(r.cell_start),
                            _p(r.cell_end))
    if rc != 0:
        raise ValueError(f"clref2d_step returned {rc}")
    return r


def emit2d(state: np.ndarray, emit: int, params) -> None:
    lib().clref2d_emit(_p(state), state.shape[0], emit, C.addressof(params))


def bvh_build(vertex: np.ndarray, index: np.ndarray, box: np.ndarray, root: int = 0):
    """oclBvhTrimesh::compute through the reference's kernels: vertex float32 [V, 4], index
    uint32 [3 n], box float32 [8] updated in place (bfAABB, kept across builds). Returns (rc,
    nodes [2n - 1], root, sorted keys, sorted triangle ids); rc -5 means two Morton keys are
    equal (the reference's linking races on them) and nothing else is returned."""
    from oracle import BVH_NODE_DTYPE
    vertex = np.ascontiguousarray(vertex, np.float32)
    index = np.ascontiguousarray(index, np.uint32)
    n = index.size // 3
    nodes = np.zeros(2 * n - 1, BVH_NODE_DTYPE)
    r = np.array([root], np.uint32)
    sk = np.empty(n, np.uint32)
    sv = np.empty(n, np.uint32)
    rc = int(lib().clref_bvh_build(_p(vertex), vertex.shape[0], _p(index), n, _p(box), _p(nodes), _p(r), _p(sk),
                                   _p(sv)))
    return rc, nodes, int(r[0]), sk, sv


def bvh_lines_build(vertex: np.ndarray, root: int = 0):
    """oclBvhLines::compute through the reference's kernels on float32 [V, 2] (two vertices per
    segment). Returns (rc, nodes [2n - 1], root, sorted keys, sorted segment ids), rc as in
    bvh_build."""
    from oracle import BVH2D_NODE_DTYPE
    vertex = np.ascontiguousarray(vertex, np.float32)
    n = vertex.shape[0] // 2
    vertex = np.ascontiguousarray(vertex[:2 * n])
    nodes = np.zeros(2 * n - 1, BVH2D_NODE_DTYPE)
    r = np.array([root], np.uint32)
    sk = np.empty(n, np.uint32)
    sv = np.empty(n, np.uint32)
    rc = int(lib().clref_bvh_lines_build(_p(vertex), n, _p(nodes), _p(r), _p(sk), _p(sv)))
    return rc, nodes, int(r[0]), sk, sv
