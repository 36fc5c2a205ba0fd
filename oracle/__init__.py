"""CPU oracle for the SPH step and radix sort -- TEST INFRASTRUCTURE ONLY.

ctypes bindings to `oracle/_build/liboracle.so`, the C++ restatement of the reference's
OpenCL kernels (oracle/oracle3d.cpp; each function there cites the libCL file:line it
follows). Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
package, as the checker or the timed CPU baseline; the product library never does.

Parity status: unpinned against executed reference output (the reference's OpenCL kernels
cannot run in this environment and its tests hold no golden vectors); see the header of
oracle3d.cpp.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_build" / "liboracle.so"
_lib = None


def _ensure_built() -> None:
    if not LIB_PATH.exists():
        import sys
        sys.path.insert(0, str(_HERE.parent))
        from libcl_gb300.build import build_oracle
        build_oracle()


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _ensure_built()
        _lib = C.CDLL(str(LIB_PATH))
        P = C.c_void_p
        U = C.c_uint32
        sig = {
            "orc_radix_sort_reference": (C.c_int, [P, P, U, U, C.c_int, C.c_int]),
            "orc_stable_sort": (C.c_int, [P, P, U, C.c_int, C.c_int]),
            "orc_find_bounds": (C.c_int, [P, U, P, P, U]),
            "orc_init_fluid_params": (None, [P]),
            "orc_kernel_constants": (None, [C.c_float, C.c_float, P]),
            "orc_hash": (None, [P, U, P, P, P]),
            "orc_reorder": (None, [P, P, P, P, P, U]),
            "orc_density": (None, [P, P, P, P, U, P]),
            "orc_forces": (None, [P, P, P, P, P, P, U, P]),
            "orc_clip_box": (None, [P, P, P, P, U, P]),
            "orc_integrate_force": (None, [P, P, U, P]),
            "orc_gravity": (None, [P, U, P]),
            "orc_integrate_velocity": (None, [P, P, U, P]),
            "orc_density_f64": (None, [P, P, P, P, P, U, P]),
            "orc_forces_f64": (None, [P, P, P, P, P, P, P, U, P]),
            "orc_step": (C.c_int, [P, P, P, U, P, P, P, P, P, P, P, C.c_int]),
            "orc_step_f64": (C.c_int, [P, P, P, P, U, P, P, P, P, P, P, P]),
            "orc_num_threads": (C.c_int, []),
            "orc2d_default_params": (None, [P]),
            "orc2d_table_size": (U, [P]),
            "orc2d_compute_border": (None, [P, C.c_int, C.c_int, P, P, P]),
            "orc2d_step": (None, [P, U, P, P, P, C.c_int, C.c_int, P, P, P, P, P, P, P, P]),
            "orc_set_num_threads": (None, [C.c_int]),
            "orc_run_f64": (C.c_int, [P, P, P, U, P, U]),
            "orc_adjoint_f64": (C.c_int, [P, P, P, U, P, U, U, P, P, P, P, P]),
            "orc_adjoint_states_f64": (C.c_int, [P, P, P, U, P, U, P, P, P, P, P]),
            "orc_bvh_build": (C.c_int, [P, U, P, U, P, P, P, P, P]),
            "orc_bvh_lines_build": (C.c_int, [P, U, P, P, P, P]),
            "orc_bvh_collide": (None, [P, P, P, P, U, P, U, P, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(_lib, name)
            f.restype, f.argtypes = res, args
    return _lib


def _p(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _pp(params) -> int:
    return C.addressof(params)


def radix_sort_reference(keys: np.ndarray, vals: np.ndarray, start: int, end: int) -> int:
    """Restated oclRadixSort (4-bit passes of 256-item blocks), in place on uint32 arrays."""
    return lib().orc_radix_sort_reference(_p(keys), _p(vals), keys.size, vals.size, start, end)


def stable_sort(keys: np.ndarray, vals: np.ndarray, start: int, end: int) -> None:
    rc = lib().orc_stable_sort(_p(keys), _p(vals), keys.size, start, end)
    assert rc == 0


def find_bounds(sorted_keys: np.ndarray, n_cells: int):
    cs = np.empty(n_cells, dtype=np.uint32)
    ce = np.empty(n_cells, dtype=np.uint32)
    lib().orc_find_bounds(_p(sorted_keys), sorted_keys.size, _p(cs), _p(ce), n_cells)
    return cs, ce


def init_fluid_params(params) -> None:
    lib().orc_init_fluid_params(_pp(params))


def kernel_constants(cell_size: float, viscosity: float) -> np.ndarray:
    """(kernelConstant, viscosityConstant, pressureConstant) by clInitFluid's formulas."""
    out = np.zeros(3, np.float32)
    lib().orc_kernel_constants(cell_size, viscosity, _p(out))
    return out


def table_cells(params) -> int:
    if params.keyMode == 1:
        return params.gridDim[0] * params.gridDim[1] * (1 if params.dims == 2 else params.gridDim[2])
    return 262144


class StepResult:
    """Everything one reference step leaves behind."""

    def __init__(self, n: int, cells: int):
        self.cell = np.empty(n, np.uint32)
        self.index = np.empty(n, np.uint32)
        self.spos = np.empty((n, 4), np.float32)
        self.svel = np.empty((n, 4), np.float32)
        self.cell_start = np.empty(cells, np.uint32)
        self.cell_end = np.empty(cells, np.uint32)


def step(pos: np.ndarray, vel: np.ndarray, force: np.ndarray, params, ref_sort: bool = False) -> StepResult:
    """One FP32 step of oclFluid3D::compute on host arrays (pos/vel/force updated in place)."""
    n = pos.shape[0]
    r = StepResult(n, table_cells(params))
    rc = lib().orc_step(_p(pos), _p(vel), _p(force), n, _pp(params), _p(r.cell), _p(r.index),
                        _p(r.spos), _p(r.svel), _p(r.cell_start), _p(r.cell_end), int(ref_sort))
    assert rc == 0, rc
    return r


def step_f64(pos64: np.ndarray, vel64: np.ndarray, force64: np.ndarray, params):
    """One FP64 step; keys from the positions rounded to FP32 (shared permutation)."""
    n = pos64.shape[0]
    fpos = pos64.astype(np.float32)
    r = StepResult(n, table_cells(params))
    r.spos = np.empty((n, 4), np.float64)
    r.svel = np.empty((n, 4), np.float64)
    rc = lib().orc_step_f64(_p(pos64), _p(vel64), _p(force64), _p(fpos), n, _pp(params), _p(r.cell),
                            _p(r.index), _p(r.spos), _p(r.svel), _p(r.cell_start), _p(r.cell_end))
    assert rc == 0, rc
    return r


def density(spos, svel, cs, ce, params):
    lib().orc_density(_p(spos), _p(svel), _p(cs), _p(ce), spos.shape[0], _pp(params))


def forces(spos, svel, force, index, cs, ce, params):
    lib().orc_forces(_p(spos), _p(svel), _p(force), _p(index), _p(cs), _p(ce), spos.shape[0], _pp(params))


def density_f64(spos64, svel64, fspos, cs, ce, params):
    lib().orc_density_f64(_p(spos64), _p(svel64), _p(fspos), _p(cs), _p(ce), spos64.shape[0], _pp(params))


def forces_f64(spos64, svel64, force64, index, fspos, cs, ce, params):
    lib().orc_forces_f64(_p(spos64), _p(svel64), _p(force64), _p(index), _p(fspos), _p(cs), _p(ce),
                         spos64.shape[0], _pp(params))


def num_threads() -> int:
    return lib().orc_num_threads()


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(n)


def hash(pos, params):
    n = pos.shape[0]
    cell = np.empty(n, np.uint32)
    index = np.empty(n, np.uint32)
    lib().orc_hash(_p(pos), n, _pp(params), _p(cell), _p(index))
    return cell, index


def reorder(index, pos, vel):
    n = pos.shape[0]
    spos = np.empty_like(pos)
    svel = np.empty_like(vel)
    lib().orc_reorder(_p(index), _p(pos), _p(vel), _p(spos), _p(svel), n)
    return spos, svel


def clip_box(spos, svel, force, index, params):
    lib().orc_clip_box(_p(spos), _p(svel), _p(force), _p(index), spos.shape[0], _pp(params))


def integrate_force(vel, force, params):
    lib().orc_integrate_force(_p(vel), _p(force), vel.shape[0], _pp(params))


def gravity(force, params):
    lib().orc_gravity(_p(force), force.shape[0], _pp(params))


def integrate_velocity(pos, vel, params):
    lib().orc_integrate_velocity(_p(pos), _p(vel), pos.shape[0], _pp(params))


def front_end(pos, vel, params):
    """hash -> stable sort on bits [0,24) -> reorder -> fill + find bounds."""
    cell, index = hash(pos, params)
    stable_sort(cell, index, 0, 24)
    spos, svel = reorder(index, pos, vel)
    cs, ce = find_bounds(cell, table_cells(params))
    return cell, index, spos, svel, cs, ce


class Step2D:
    """Everything one oclFluid2D::compute leaves behind."""

    def __init__(self, n: int, table: int):
        self.cell = np.empty(n, np.uint32)
        self.index = np.empty(n, np.uint32)
        self.sorted = np.empty((n, 6), np.float32)
        self.pstate = np.empty((n, 4), np.float32)
        self.relaxed = np.empty((n, 2), np.float32)
        self.prev = np.empty((n, 2), np.float32)
        self.cell_start = np.empty(table, np.uint32)
        self.cell_end = np.empty(table, np.uint32)


def default_params_2d(p) -> None:
    lib().orc2d_default_params(_pp(p))


def table_size_2d(p) -> int:
    return int(lib().orc2d_table_size(_pp(p)))


def compute_border_2d(mask: np.ndarray, p):
    """clComputeBorder on a [H, W, 4] float32 mask; returns (vector, state) [H, W, 4]."""
    h, w = mask.shape[:2]
    vec = np.empty((h, w, 4), np.float32)
    st = np.empty((h, w, 4), np.float32)
    lib().orc2d_compute_border(_p(np.ascontiguousarray(mask, np.float32)), w, h, _pp(p), _p(vec), _p(st))
    return vec, st


def step_2d(state: np.ndarray, p, border_state: np.ndarray, border_vec: np.ndarray) -> Step2D:
    """One FP32 step of oclFluid2D::compute; state is float32 [N, 6] (updated in place)."""
    n = state.shape[0]
    h, w = border_state.shape[:2]
    r = Step2D(n, table_size_2d(p))
    lib().orc2d_step(_p(state), n, _pp(p), _p(border_state), _p(border_vec), w, h, _p(r.cell), _p(r.index),
                     _p(r.sorted), _p(r.pstate), _p(r.relaxed), _p(r.prev), _p(r.cell_start), _p(r.cell_end))
    return r


def run_f64(pos64: np.ndarray, vel64: np.ndarray, force64: np.ndarray, params, steps: int) -> None:
    """`steps` FP64 steps in place (keys from the positions rounded to FP32)."""
    rc = lib().orc_run_f64(_p(pos64), _p(vel64), _p(force64), pos64.shape[0], _pp(params), steps)
    assert rc == 0, rc


def adjoint_f64(pos0, vel0, force0, params, steps: int, every: int, gpos, gvel=None):
    """FP64 adjoint of `steps` steps (LINEAR_GRID, 3D): returns (dL/dpos0, dL/dvel0,
    dL/dstiffness, dL/dviscosity) for the final-state gradients gpos, gvel (float64 [N, 4])."""
    n = pos0.shape[0]
    gp0 = np.empty((n, 4), np.float64)
    gv0 = np.empty((n, 4), np.float64)
    gpar = np.empty(2, np.float64)
    rc = lib().orc_adjoint_f64(_p(pos0), _p(vel0), _p(force0), n, _pp(params), steps, every, _p(gpos),
                               None if gvel is None else _p(gvel), _p(gp0), _p(gv0), _p(gpar))
    assert rc == 0, rc
    return gp0, gv0, float(gpar[0]), float(gpar[1])


def adjoint_states_f64(states_pos, states_vel, force0, params, gpos, gvel=None):
    """FP64 adjoint along a given trajectory: states_pos / states_vel float32 [steps, N, 4]
    (the state before each step), force0 float64 [N, 4]. Returns like adjoint_f64."""
    steps, n = states_pos.shape[:2]
    sp = np.ascontiguousarray(states_pos, np.float32)
    sv = np.ascontiguousarray(states_vel, np.float32)
    gp0 = np.empty((n, 4), np.float64)
    gv0 = np.empty((n, 4), np.float64)
    gpar = np.empty(2, np.float64)
    rc = lib().orc_adjoint_states_f64(_p(sp), _p(sv), _p(force0), n, _pp(params), steps, _p(gpos),
                                      None if gvel is None else _p(gvel), _p(gp0), _p(gv0), _p(gpar))
    assert rc == 0, rc
    return gp0, gv0, float(gpar[0]), float(gpar[1])


BVH_NODE_DTYPE = np.dtype([("bbMin", np.float32, 4), ("bbMax", np.float32, 4), ("left", np.int32),
                           ("right", np.int32), ("bit", np.uint32), ("trav", np.uint32)])


def bvh_build(vertex: np.ndarray, index: np.ndarray, box: np.ndarray, root: int = 0):
    """The reference's BVH build (oclBvhTrimesh::compute) on host arrays: vertex float32
    [V, 4], index uint32 [3 n], box float32 [8] updated in place (the persistent global box).
    Returns (nodes [2n - 1] structured array, root, sorted keys, sorted triangle ids)."""
    vertex = np.ascontiguousarray(vertex, np.float32)
    index = np.ascontiguousarray(index, np.uint32)
    n = index.size // 3
    nodes = np.zeros(2 * n - 1, BVH_NODE_DTYPE)
    r = np.array([root], np.uint32)
    sk = np.empty(n, np.uint32)
    sv = np.empty(n, np.uint32)
    rc = lib().orc_bvh_build(_p(vertex), vertex.shape[0], _p(index), n, _p(box), _p(nodes), _p(r), _p(sk), _p(sv))
    assert rc == 0, rc
    return nodes, int(r[0]), sk, sv


BVH2D_NODE_DTYPE = np.dtype([("bbMin", np.float32, 2), ("bbMax", np.float32, 2), ("left", np.int32),
                             ("right", np.int32), ("bit", np.uint32), ("trav", np.uint32)])


def bvh_lines_build(vertex: np.ndarray, root: int = 0):
    """The reference's 2D segment BVH build (oclBvhLines::compute) on a host float32 [V, 2]
    array (two vertices per segment). Returns (nodes [2n - 1], root, sorted keys, sorted
    segment ids)."""
    vertex = np.ascontiguousarray(vertex, np.float32)
    n = vertex.shape[0] // 2
    vertex = np.ascontiguousarray(vertex[:2 * n])
    nodes = np.zeros(2 * n - 1, BVH2D_NODE_DTYPE)
    r = np.array([root], np.uint32)
    sk = np.empty(n, np.uint32)
    sv = np.empty(n, np.uint32)
    rc = lib().orc_bvh_lines_build(_p(vertex), n, _p(nodes), _p(r), _p(sk), _p(sv))
    assert rc == 0, rc
    return nodes, int(r[0]), sk, sv


def bvh_collide(params, position, velocity, force, nodes, root, index, vertex) -> None:
    """clCollideBVH on host float32 [N, 4] arrays (updated in place)."""
    lib().orc_bvh_collide(_pp(params), _p(position), _p(velocity), _p(force), position.shape[0], _p(nodes), root,
                          _p(np.ascontiguousarray(index, np.uint32)), _p(np.ascontiguousarray(vertex, np.float32)))
