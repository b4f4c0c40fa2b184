"""numpy front end for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Wraps ``libnbody_oracle.so`` (the C restatement of the reference CPU path) and, when it
was built, ``oracle/_ref/libnbody_ref.so`` (the reference's own CPU solvers compiled from
its sources). Only ``tests/``, ``__graft_entry__.smoke`` and ``bench.py``'s CPU-baseline
leg may import this module; the product never does.

Bodies are ``float32`` arrays of shape ``(n, 12)`` in the reference's ``Body`` layout
(include/nbody/body.h:6-19): pos xyz, radius, vel xyz, mass, acc xyz, pad.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build_oracle

_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_U64 = C.POINTER(C.c_uint64)
_U32 = C.POINTER(C.c_uint32)
_SZ = C.c_size_t

NODE_DTYPE = np.dtype([("center", "<f4", 3), ("size", "<f4"), ("com", "<f4", 3), ("mass", "<f4"),
                       ("next", "<u4"), ("children", "<u4"), ("pad", "<u4", 2)])
assert NODE_DTYPE.itemsize == 48

LAW_CUTOFF = 0
LAW_SOFTENED = 1

_lib = None
_timing = None
_ref = None
_ref_timing = None


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def lib(timing: bool = False):
    """The oracle library; timing=True gives the same source built for speed (the CPU
    baselines only: its last bits are not the checked ones)."""
    global _lib, _timing
    if timing:
        if _timing is None:
            _timing = _bind(C.CDLL(str(build_oracle.build_oracle_timing())))
        return _timing
    if _lib is None:
        _lib = _bind(C.CDLL(str(build_oracle.build_oracle())))
    return _lib


def _bind(L):
    """Argument and result types of every oracle entry point."""
    L.orc_gravity.argtypes = [_F, C.c_float, _F, C.c_float, C.c_float, _F]
    L.orc_wrap.argtypes = [C.c_float, C.c_float]
    L.orc_wrap.restype = C.c_float
    L.orc_integrate.argtypes = [_F, _SZ, C.c_float, C.c_float, C.c_int]
    L.orc_brute_force.argtypes = [_F, _SZ, C.c_float, C.c_int]
    L.orc_brute_force_targets.argtypes = [_F, _SZ, C.c_float, _I64, _SZ, _F, C.c_int]
    L.orc_barnes_hut.argtypes = [_F, _SZ, C.c_float, C.c_float, C.c_float, C.c_int, _U64]
    L.orc_gravity_softened.argtypes = [_F, _F, C.c_float, C.c_float, C.c_float, _F]
    L.orc_brute_force_targets_law.argtypes = [_F, _SZ, C.c_float, C.c_int, C.c_float, _I64, _SZ, _F, C.c_int]
    L.orc_barnes_hut_law.argtypes = [_F, _SZ, C.c_float, C.c_float, C.c_float, C.c_int, C.c_float, C.c_int,
                                     _U64]
    L.orc_tree_accel_law.argtypes = [C.c_void_p, _F, _SZ, _I64, _SZ, C.c_float, C.c_float, C.c_int, C.c_float,
                                     _F, _U64, C.c_int]
    L.orc_nodes_accel_law.argtypes = [C.c_void_p, _SZ, _F, _SZ, _I64, _SZ, C.c_float, C.c_float, C.c_int,
                                      C.c_float, _F, _U64, C.c_int]
    L.orc_tree_new.argtypes = [C.c_float]
    L.orc_tree_new.restype = C.c_void_p
    L.orc_tree_free.argtypes = [C.c_void_p]
    L.orc_tree_clear.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float]
    L.orc_tree_insert.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float]
    L.orc_tree_build.argtypes = [C.c_void_p, _F, _SZ, C.c_float]
    L.orc_tree_build_box.argtypes = [C.c_void_p, _F, _SZ, C.c_float, C.c_float, C.c_float, C.c_float]
    L.orc_tree_exact_moments.argtypes = [C.c_void_p, _F, _SZ]
    L.orc_tree_exact_moments.restype = C.c_int
    L.orc_tree_size.argtypes = [C.c_void_p]
    L.orc_tree_size.restype = _SZ
    L.orc_tree_nodes.argtypes = [C.c_void_p]
    L.orc_tree_nodes.restype = C.c_void_p
    L.orc_tree_accel.argtypes = [C.c_void_p, _F, _SZ, _I64, _SZ, C.c_float, C.c_float, _F, _U64, C.c_int]
    L.orc_nodes_accel.argtypes = [C.c_void_p, _SZ, _F, _SZ, _I64, _SZ, C.c_float, C.c_float, _F, _U64, C.c_int]
    L.orc_direct_f64.argtypes = [_F, _F, _SZ, C.c_double, C.c_double, C.c_int, _I64, _SZ, _D, _D, C.c_int]
    L.orc_direct_f64_pos.argtypes = [_D, _D, _SZ, C.c_double, C.c_double, _I64, _SZ, _D, C.c_int]
    L.orc_energy_f64.argtypes = [_D, _D, _D, _SZ, C.c_double, C.c_double, _D, _D, _D, C.c_int]
    L.orc_morton63.argtypes = [_F, _SZ, _SZ, _D, C.c_double, _U64]
    L.orc_sort_order.argtypes = [_U64, _SZ, _U32]
    L.orc_default_threads.restype = C.c_int
    L.orc_minstd_value.argtypes = [C.c_uint64]
    L.orc_minstd_value.restype = C.c_uint32
    L.orc_compute_radius.argtypes = [C.c_float, C.c_float]
    L.orc_compute_radius.restype = C.c_float
    L.orc_disk.argtypes = [_F, _SZ, _F]
    L.orc_cube.argtypes = [_F, _SZ, _F]
    L.orc_disk_positions.argtypes = [_F, _SZ, _F, _SZ, _SZ]
    L.orc_tree_query.argtypes = [C.c_void_p, _SZ, _F, C.c_int, _U32, _SZ, C.POINTER(C.c_int)]
    L.orc_tree_query.restype = _SZ
    return L


def ref_lib(timing: bool = False):
    """The reference's own CPU solvers, or None where they could not be built; timing=True
    gives them built with the timing flags."""
    global _ref, _ref_timing
    if (_ref_timing if timing else _ref) is None:
        path = build_oracle.REF_TIMING_LIB if timing else build_oracle.REF_LIB
        if not path.exists():
            try:
                path = build_oracle.build_ref(timing=timing)
            except RuntimeError:
                path = None
        if path is None or not Path(path).exists():
            return None
        try:
            L = C.CDLL(str(path))
        except OSError:     # e.g. a library built for another architecture
            return None
        L.ref_hardware_threads.restype = C.c_int
        L.ref_brute_force.argtypes = [_F, _SZ, C.c_float, C.c_float, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int]
        L.ref_barnes_hut.argtypes = [_F, _SZ, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int]
        L.ref_integrate.argtypes = [_F, _SZ, C.c_float, C.c_float, C.c_int]
        L.ref_build_tree.argtypes = [_F, _SZ, C.c_float, C.c_void_p, _SZ]
        L.ref_build_tree.restype = _SZ
        L.ref_insert_points.argtypes = [_F, _SZ, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p, _SZ]
        L.ref_insert_points.restype = _SZ
        L.ref_disk.argtypes = [_F, _SZ, C.c_float, C.c_float, C.c_float, C.c_float]
        L.ref_cube.argtypes = [_F, _SZ]
        L.ref_disk_args.argtypes = [_F, _SZ, _SZ, _SZ, _F]
        L.ref_tree_query.argtypes = [_F, _SZ, C.c_float, _F, C.c_int, _U32, _SZ]
        L.ref_tree_query.restype = _SZ
        L.ref_cube_args.argtypes = [_F, _SZ, _SZ, _SZ, _F]
        if timing:
            _ref_timing = L
        else:
            _ref = L
    return _ref_timing if timing else _ref


def threads() -> int:
    return int(lib().orc_default_threads())


def _bodies(b):
    b = np.ascontiguousarray(b, dtype=np.float32)
    assert b.ndim == 2 and b.shape[1] == 12
    return b


# --- restatement ---------------------------------------------------------------------

def gravity(pos, radius, src, src_mass, G):
    out = np.zeros(3, np.float32)
    lib().orc_gravity(_p(np.ascontiguousarray(pos, np.float32), _F), radius,
                      _p(np.ascontiguousarray(src, np.float32), _F), src_mass, G, _p(out, _F))
    return out


def wrap(x, size):
    return lib().orc_wrap(x, size)


def integrate(bodies, dt, size, do_wrap):
    b = _bodies(bodies).copy()
    lib().orc_integrate(_p(b, _F), len(b), dt, size, int(do_wrap))
    return b


def brute_force(bodies, G, nthreads=0):
    """CpuBruteForceSolver::accelerate restated; returns a copy with acc filled in."""
    b = _bodies(bodies).copy()
    lib().orc_brute_force(_p(b, _F), len(b), G, nthreads)
    return b


def gravity_softened(pos, src, src_mass, G, eps2):
    out = np.zeros(3, np.float32)
    lib().orc_gravity_softened(_p(np.ascontiguousarray(pos, np.float32), _F),
                               _p(np.ascontiguousarray(src, np.float32), _F), src_mass, G, eps2, _p(out, _F))
    return out


def brute_force_targets(bodies, G, targets, nthreads=0, law=LAW_CUTOFF, eps2=0.0, timing=False):
    """CpuBruteForceSolver::accelerate (cpu_brute_force.h:17-43) for the listed targets, with
    the reference's cutoff law or the softened law (eps2); timing=True runs the speed build."""
    b = _bodies(bodies)
    t = np.ascontiguousarray(targets, np.int64)
    out = np.zeros((len(t), 3), np.float32)
    lib(timing).orc_brute_force_targets_law(_p(b, _F), len(b), G, law, eps2, _p(t, _I64), len(t), _p(out, _F),
                                            nthreads)
    return out


def barnes_hut(bodies, size, theta, G, nthreads=0, law=LAW_CUTOFF, eps2=0.0, timing=False):
    """CpuBarnesHutSolver::accelerate restated; returns (bodies with acc, interactions).
    law/eps2 choose the visitor's force law (the reference's cutoff law by default);
    timing=True runs the speed build."""
    b = _bodies(bodies).copy()
    inter = np.zeros(1, np.uint64)
    lib(timing).orc_barnes_hut_law(_p(b, _F), len(b), size, theta, G, law, eps2, nthreads, _p(inter, _U64))
    return b, int(inter[0])


class Tree:
    """bh::Tree restated (source/bhtree.cpp)."""

    def __init__(self, size=1.0, center=(0.0, 0.0, 0.0)):
        self._t = lib().orc_tree_new(size)
        lib().orc_tree_clear(self._t, float(center[0]), float(center[1]), float(center[2]), size)

    def __del__(self):
        if getattr(self, "_t", None):
            lib().orc_tree_free(self._t)
            self._t = None

    def insert(self, pos, mass):
        lib().orc_tree_insert(self._t, float(pos[0]), float(pos[1]), float(pos[2]), float(mass))

    def build(self, bodies, size):
        b = _bodies(bodies)
        lib().orc_tree_build(self._t, _p(b, _F), len(b), size)

    def build_on_box(self, bodies, box):
        """Insert every body, in index order, under a root box given as (lower corner xyz,
        edge), as the device tree's root box is reported (nbody_cuda_morton)."""
        b = _bodies(bodies)
        e = float(box[3])
        lib().orc_tree_build_box(self._t, _p(b, _F), len(b), float(box[0]) + 0.5 * e, float(box[1]) + 0.5 * e,
                                 float(box[2]) + 0.5 * e, e)

    def exact_moments(self, bodies):
        """Replace every node's mass and centre of mass by exact (FP64-summed) values over
        its bodies, keeping the reference's cells: the reference tree without the FP32
        running mean's drift (bhtree.cpp:87-95)."""
        b = _bodies(bodies)
        if lib().orc_tree_exact_moments(self._t, _p(b, _F), len(b)) != 0:
            raise MemoryError("orc_tree_exact_moments: no scratch")

    def nodes(self):
        n = lib().orc_tree_size(self._t)
        ptr = lib().orc_tree_nodes(self._t)
        buf = (C.c_char * (48 * n)).from_address(ptr)
        return np.frombuffer(bytes(buf), dtype=NODE_DTYPE).copy()

    def accel(self, bodies, theta, G, targets=None, nthreads=0, law=LAW_CUTOFF, eps2=0.0):
        """Tree::apply (bhtree.cpp:97-138) with the gravity visitor of cpu_barnes_hut.h:31-41
        for the listed targets; law/eps2 choose the visitor's force law."""
        b = _bodies(bodies)
        t = None if targets is None else np.ascontiguousarray(targets, np.int64)
        nt = len(b) if t is None else len(t)
        out = np.zeros((nt, 3), np.float32)
        inter = np.zeros(1, np.uint64)
        lib().orc_tree_accel_law(self._t, _p(b, _F), len(b), _p(t, _I64), 0 if t is None else len(t),
                                 theta, G, law, eps2, _p(out, _F), _p(inter, _U64), nthreads)
        return out, int(inter[0])


def tree_nodes(bodies, size):
    """detail::build_tree (tree.h:14-29) restated: the node array of the reference tree."""
    t = Tree(size)
    t.build(bodies, size)
    return t.nodes()


def nodes_accel(nodes, bodies, theta, G, targets=None, nthreads=0, law=LAW_CUTOFF, eps2=0.0):
    """Tree::apply (bhtree.cpp:97-138) over a node array in the reference layout."""
    nd = np.ascontiguousarray(nodes)
    assert nd.dtype == NODE_DTYPE
    b = _bodies(bodies)
    t = None if targets is None else np.ascontiguousarray(targets, np.int64)
    nt = len(b) if t is None else len(t)
    out = np.zeros((nt, 3), np.float32)
    inter = np.zeros(1, np.uint64)
    lib().orc_nodes_accel_law(nd.ctypes.data_as(C.c_void_p), len(nd), _p(b, _F), len(b), _p(t, _I64),
                              0 if t is None else len(t), theta, G, law, eps2, _p(out, _F), _p(inter, _U64),
                              nthreads)
    return out, int(inter[0])


def direct_f64(pos_mass, G, eps2=0.0, law=LAW_SOFTENED, radius=None, targets=None, nthreads=0,
               with_scale=False):
    """FP64 direct sum for the given targets (all when None). Returns acc (and scale)."""
    pm = np.ascontiguousarray(pos_mass, np.float32)
    assert pm.ndim == 2 and pm.shape[1] == 4
    r = None if radius is None else np.ascontiguousarray(radius, np.float32)
    t = None if targets is None else np.ascontiguousarray(targets, np.int64)
    nt = len(pm) if t is None else len(t)
    acc = np.zeros((nt, 3), np.float64)
    scale = np.zeros(nt, np.float64) if with_scale else None
    lib().orc_direct_f64(_p(pm, _F), _p(r, _F), len(pm), G, eps2, law, _p(t, _I64),
                         0 if t is None else len(t), _p(acc, _D), _p(scale, _D), nthreads)
    return (acc, scale) if with_scale else acc


def direct_f64_pos(pos, mass, G, eps2, targets=None, nthreads=0):
    p = np.ascontiguousarray(pos, np.float64)
    m = np.ascontiguousarray(mass, np.float64)
    t = None if targets is None else np.ascontiguousarray(targets, np.int64)
    nt = len(p) if t is None else len(t)
    acc = np.zeros((nt, 3), np.float64)
    lib().orc_direct_f64_pos(_p(p, _D), _p(m, _D), len(p), G, eps2, _p(t, _I64),
                             0 if t is None else len(t), _p(acc, _D), nthreads)
    return acc


def energy_f64(pos, vel, mass, G, eps2, nthreads=0):
    p = np.ascontiguousarray(pos, np.float64)
    v = np.ascontiguousarray(vel, np.float64)
    m = np.ascontiguousarray(mass, np.float64)
    ke = np.zeros(1)
    pe = np.zeros(1)
    mom = np.zeros(3)
    lib().orc_energy_f64(_p(p, _D), _p(v, _D), _p(m, _D), len(m), G, eps2, _p(ke, _D), _p(pe, _D),
                         _p(mom, _D), nthreads)
    return float(ke[0]), float(pe[0]), mom


def morton63(xyz, lo, inv_cell, stride=None):
    a = np.ascontiguousarray(xyz, np.float32)
    s = stride if stride is not None else a.shape[1]
    lo = np.ascontiguousarray(lo, np.float64)
    out = np.zeros(len(a), np.uint64)
    lib().orc_morton63(_p(a, _F), s, len(a), _p(lo, _D), inv_cell, _p(out, _U64))
    return out


def sort_order(codes):
    c = np.ascontiguousarray(codes, np.uint64)
    out = np.zeros(len(c), np.uint32)
    lib().orc_sort_order(_p(c, _U64), len(c), _p(out, _U32))
    return out


# --- the reference itself (where it was built) ---------------------------------------

def ref_available() -> bool:
    return ref_lib() is not None


def ref_brute_force(bodies, G, steps=0, dt=0.0, size=10000.0, do_wrap=False, nthreads=0):
    b = _bodies(bodies).copy()
    ref_lib().ref_brute_force(_p(b, _F), len(b), G, dt, steps, int(steps == 0), size, int(do_wrap), nthreads)
    return b


def ref_barnes_hut(bodies, size, theta, G, steps=0, dt=0.0, do_wrap=False, nthreads=0):
    b = _bodies(bodies).copy()
    ref_lib().ref_barnes_hut(_p(b, _F), len(b), size, theta, G, dt, steps, int(steps == 0), int(do_wrap), nthreads)
    return b


def ref_integrate(bodies, dt, size, do_wrap):
    b = _bodies(bodies).copy()
    ref_lib().ref_integrate(_p(b, _F), len(b), dt, size, int(do_wrap))
    return b


def ref_build_tree(bodies, size):
    b = _bodies(bodies)
    n = ref_lib().ref_build_tree(_p(b, _F), len(b), size, None, 0)
    out = np.zeros(n, NODE_DTYPE)
    ref_lib().ref_build_tree(_p(b, _F), len(b), size, out.ctypes.data_as(C.c_void_p), n)
    return out


def ref_insert_points(points, center, size):
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    n = ref_lib().ref_insert_points(_p(pts, _F), len(pts), *map(float, center), size, None, 0)
    out = np.zeros(n, NODE_DTYPE)
    ref_lib().ref_insert_points(_p(pts, _F), len(pts), *map(float, center), size,
                                out.ctypes.data_as(C.c_void_p), n)
    return out


def ref_disk(n, center=(0.0, 0.0, 0.0), outer_radius=100.0):
    b = np.zeros((n, 12), np.float32)
    ref_lib().ref_disk(_p(b, _F), n, *map(float, center), outer_radius)
    return b


def ref_cube(n):
    b = np.zeros((n, 12), np.float32)
    ref_lib().ref_cube(_p(b, _F), n)
    return b


# --- scene generators (source/util.cpp) ---------------------------------------------------

DISK_DEFAULTS = dict(center=(0.0, 0.0, 0.0), vel=(0.0, 0.0, 0.0), axis=(0.0, 0.0, 1.0), inner_radius=0.0,
                     outer_radius=250.0, thickness=1.0, central_mass=4.1e6, star_mass=1.0)
CUBE_DEFAULTS = dict(center=(0.0, 0.0, 0.0), size=500.0, vel=(0.0, 0.0, 0.0), star_mass=1.0)


def disk_arg_array(**kw):
    """util::DiskArgs as the 14 floats the oracle and the reference driver take."""
    a = dict(DISK_DEFAULTS, **kw)
    return np.array([*a["center"], *a["vel"], *a["axis"], a["inner_radius"], a["outer_radius"],
                     a["thickness"], a["central_mass"], a["star_mass"]], np.float32)


def cube_arg_array(**kw):
    a = dict(CUBE_DEFAULTS, **kw)
    return np.array([*a["center"], a["size"], *a["vel"], a["star_mass"]], np.float32)


def minstd_value(j: int) -> int:
    return int(lib().orc_minstd_value(j))


def disk(num: int, **kw) -> np.ndarray:
    """The oracle's util::disk over a fresh array of num bodies."""
    b = np.zeros((num, 12), np.float32)
    lib().orc_disk(_p(b, _F), num, _p(disk_arg_array(**kw), _F))
    return b


def disk_positions(num: int, first: int, last: int, **kw) -> np.ndarray:
    """Bodies [first, last) of util::disk(num) without the velocity pass: positions,
    radius and mass as the reference writes them, velocity the unit direction."""
    b = np.zeros((num, 12), np.float32)
    lib().orc_disk_positions(_p(b, _F), num, _p(disk_arg_array(**kw), _F), first, last)
    return b[first:last]


def cube(num: int, **kw) -> np.ndarray:
    b = np.zeros((num, 12), np.float32)
    lib().orc_cube(_p(b, _F), num, _p(cube_arg_array(**kw), _F))
    return b


def ref_disk_range(bodies: np.ndarray, begin: int, num: int, **kw) -> np.ndarray:
    """The reference's util::disk over bodies[begin, begin + num) of a copy of `bodies`."""
    b = np.ascontiguousarray(bodies, np.float32).copy()
    ref_lib().ref_disk_args(_p(b, _F), len(b), begin, num, _p(disk_arg_array(**kw), _F))
    return b


def ref_cube_range(bodies: np.ndarray, begin: int, num: int, **kw) -> np.ndarray:
    b = np.ascontiguousarray(bodies, np.float32).copy()
    ref_lib().ref_cube_args(_p(b, _F), len(b), begin, num, _p(cube_arg_array(**kw), _F))
    return b


# --- ray query (source/bhtree.cpp:153-173) -------------------------------------------------

def tree_query(nodes: np.ndarray, ray, stop: int = 0, max_hits: int = 1 << 16):
    """Tree::query over a node array (NODE_DTYPE) for one ray: (visited indices, visited
    count, whether the walk passed a node the ray misses)."""
    nodes = np.ascontiguousarray(nodes)
    r = np.ascontiguousarray(ray, np.float32)
    hits = np.zeros(max_hits, np.uint32)
    missed = C.c_int()
    cnt = lib().orc_tree_query(nodes.ctypes.data_as(C.c_void_p), len(nodes), _p(r, _F), stop, _p(hits, _U32),
                               max_hits, C.byref(missed))
    return hits[:min(cnt, max_hits)], int(cnt), bool(missed.value)


def ref_tree_query(bodies: np.ndarray, size: float, ray, stop: int = 0, max_hits: int = 1 << 16):
    """The reference's Tree::query over detail::build_tree(bodies, size). Only for rays
    that meet every node the walk reaches: elsewhere the reference's loop never ends."""
    b = np.ascontiguousarray(bodies, np.float32)
    r = np.ascontiguousarray(ray, np.float32)
    hits = np.zeros(max_hits, np.uint32)
    cnt = ref_lib().ref_tree_query(_p(b, _F), len(b), size, _p(r, _F), stop, _p(hits, _U32), max_hits)
    return hits[:min(cnt, max_hits)], int(cnt)
