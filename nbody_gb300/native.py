"""ctypes binding of the C ABI in ``include/nbody_cuda.h``.

This is how Python (tests, bench) reaches the CUDA library; it adds no behaviour of its
own. The library is loaded from ``nbody_gb300/lib/libnbody_cuda.so`` (built in-tree by
``nbody_gb300/build.py``); if it is missing, :func:`lib` raises -- there is no fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libnbody_cuda.so"

# status codes (nbody_status)
OK, ERR_INVALID, ERR_NO_DEVICE, ERR_CUDA, ERR_ALLOC, ERR_TIMEOUT, ERR_UNSUPPORTED = range(7)
MODE_N2, MODE_NLOGN, MODE_BATCHED = 0, 1, 2
LAW_CUTOFF, LAW_SOFTENED = 0, 1
PREC_FP32, PREC_COMPENSATED, PREC_FP64 = 0, 1, 2
LAYOUT_SOA, LAYOUT_AOS = 0, 1
READ_POSITIONS, READ_VELOCITIES, READ_ACCELERATIONS, READ_ALL = 1, 2, 4, 7
QUERY_ALL, QUERY_FIRST_BODY = 0, 1
TRANSFER_AUTO, TRANSFER_STAGED, TRANSFER_MAPPED, TRANSFER_DIRECT = 0, 1, 2, 3
WALK_TARGET, WALK_GROUP = 0, 1

# bh::Node (include/nbody/bhtree.h of the reference): bounds centre, size, com, mass, links
NODE_DTYPE = np.dtype([("center", "<f4", 3), ("size", "<f4"), ("com", "<f4", 3), ("mass", "<f4"),
                       ("next", "<u4"), ("children", "<u4"), ("pad", "<u4", 2)])

# Every symbol include/nbody_cuda.h declares (checked by tests/test_boundary.py).
EXPORTS = (
    "nbody_cuda_probe", "nbody_cuda_create", "nbody_cuda_destroy", "nbody_cuda_last_error",
    "nbody_cuda_set_stream", "nbody_cuda_stream", "nbody_cuda_layout", "nbody_cuda_reserve",
    "nbody_cuda_count", "nbody_cuda_upload_bodies", "nbody_cuda_download_bodies",
    "nbody_cuda_upload_soa", "nbody_cuda_download_soa", "nbody_cuda_accelerate",
    "nbody_cuda_integrate", "nbody_cuda_update", "nbody_cuda_synchronize",
    "nbody_cuda_dev_accel_soa", "nbody_cuda_dev_accel_aos", "nbody_cuda_dev_integrate_soa",
    "nbody_cuda_launch_count", "nbody_cuda_last_direct_config", "nbody_cuda_calibrate_fp32",
    "nbody_cuda_dev_accel_soa_noalloc", "nbody_cuda_bh_stats", "nbody_cuda_bh_stage_ms", "nbody_cuda_morton",
    "nbody_cuda_accel_sampled", "nbody_cuda_split_origin", "nbody_cuda_calibrate_fp64",
    "nbody_cuda_tree_export", "nbody_cuda_set_systems", "nbody_cuda_batch_autotune",
    "nbody_cuda_batch_config_count", "nbody_cuda_batch_config", "nbody_cuda_batch_set_config",
    "nbody_cuda_system_energy", "nbody_cuda_update_graph", "nbody_cuda_direct_variant_count",
    "nbody_cuda_direct_variant", "nbody_cuda_set_direct_variant", "nbody_cuda_direct_autotune",
    "nbody_cuda_selftest_wait", "nbody_cuda_set_transfer", "nbody_cuda_transfer_info",
    "nbody_cuda_prefetch", "nbody_cuda_scene_disk", "nbody_cuda_scene_cube", "nbody_cuda_tree_query",
    "nbody_cuda_energy",
)


class StepParams(C.Structure):
    """nbody_step_params."""
    _fields_ = [("dt", C.c_float), ("theta", C.c_float), ("G", C.c_float), ("eps2", C.c_float),
                ("size", C.c_float), ("wrap", C.c_int32), ("mode", C.c_int32), ("law", C.c_int32),
                ("precision", C.c_int32), ("tree_box", C.c_int32), ("walk", C.c_int32), ("reserved", C.c_int32)]


class DiskArgs(C.Structure):
    """nbody_disk_args: util::DiskArgs (include/nbody/util.h of the reference)."""
    _fields_ = [("center", C.c_float * 3), ("vel", C.c_float * 3), ("axis", C.c_float * 3),
                ("inner_radius", C.c_float), ("outer_radius", C.c_float), ("thickness", C.c_float),
                ("central_mass", C.c_float), ("star_mass", C.c_float)]


class CubeArgs(C.Structure):
    """nbody_cube_args: util::CubeArgs."""
    _fields_ = [("center", C.c_float * 3), ("size", C.c_float), ("vel", C.c_float * 3), ("star_mass", C.c_float)]


def disk_args(center=(0.0, 0.0, 0.0), vel=(0.0, 0.0, 0.0), axis=(0.0, 0.0, 1.0), inner_radius=0.0,
              outer_radius=250.0, thickness=1.0, central_mass=4.1e6, star_mass=1.0) -> DiskArgs:
    """The reference's defaults (util.h: DiskArgs; sagittarius_mass, solar_mass)."""
    f3 = C.c_float * 3
    return DiskArgs(f3(*center), f3(*vel), f3(*axis), inner_radius, outer_radius, thickness, central_mass,
                    star_mass)


def cube_args(center=(0.0, 0.0, 0.0), size=500.0, vel=(0.0, 0.0, 0.0), star_mass=1.0) -> CubeArgs:
    f3 = C.c_float * 3
    return CubeArgs(f3(*center), size, f3(*vel), star_mass)


def params(dt=0.0, theta=0.5, G=1.0, eps2=0.0, size=10000.0, wrap=False, mode=MODE_N2,
           law=LAW_CUTOFF, precision=PREC_FP32, tree_box=0, walk=WALK_TARGET) -> StepParams:
    return StepParams(dt, theta, G, eps2, size, int(bool(wrap)), mode, law, precision, tree_box, walk, 0)


class NbodyError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"nbody_cuda status {status}: {message}")
        self.status = status


_lib = None


def lib() -> C.CDLL:
    """The loaded library; raises if it was not built (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with nbody_gb300.build.build()")
    L = C.CDLL(str(LIB_PATH))
    vp, sz, u = C.c_void_p, C.c_size_t, C.c_uint
    P = C.POINTER(StepParams)
    sig = {
        "nbody_cuda_probe": ([C.c_char_p, sz], C.c_int),
        "nbody_cuda_create": ([C.POINTER(vp), C.c_int], C.c_int),
        "nbody_cuda_destroy": ([vp], None),
        "nbody_cuda_last_error": ([vp, C.c_char_p, sz], C.c_int),
        "nbody_cuda_set_stream": ([vp, vp], C.c_int),
        "nbody_cuda_stream": ([vp], vp),
        "nbody_cuda_layout": ([vp], C.c_int),
        "nbody_cuda_reserve": ([vp, sz], C.c_int),
        "nbody_cuda_count": ([vp], sz),
        "nbody_cuda_upload_bodies": ([vp, vp, sz], C.c_int),
        "nbody_cuda_download_bodies": ([vp, vp, sz, u], C.c_int),
        "nbody_cuda_upload_soa": ([vp, vp, vp, vp, sz], C.c_int),
        "nbody_cuda_download_soa": ([vp, vp, vp, vp, sz], C.c_int),
        "nbody_cuda_accelerate": ([vp, P], C.c_int),
        "nbody_cuda_integrate": ([vp, P], C.c_int),
        "nbody_cuda_update": ([vp, P, C.c_int], C.c_int),
        "nbody_cuda_synchronize": ([vp], C.c_int),
        "nbody_cuda_dev_accel_soa": ([vp, vp, vp, vp, sz, P], C.c_int),
        "nbody_cuda_dev_accel_aos": ([vp, vp, sz, P], C.c_int),
        "nbody_cuda_dev_integrate_soa": ([vp, vp, vp, vp, sz, P], C.c_int),
        "nbody_cuda_launch_count": ([vp], C.c_uint64),
        "nbody_cuda_last_direct_config": ([vp] + [C.POINTER(C.c_int)] * 5, C.c_int),
        "nbody_cuda_calibrate_fp32": ([vp, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
        "nbody_cuda_dev_accel_soa_noalloc": ([vp, vp, vp, sz, P, vp], C.c_int),
        "nbody_cuda_bh_stats": ([vp, C.POINTER(C.c_uint64)], C.c_int),
        "nbody_cuda_bh_stage_ms": ([vp, C.POINTER(C.c_float)], C.c_int),
        "nbody_cuda_morton": ([vp, P, vp, vp, C.POINTER(C.c_double)], C.c_int),
        "nbody_cuda_accel_sampled": ([vp, P, vp, sz, vp], C.c_int),
        "nbody_cuda_split_origin": ([vp, C.POINTER(C.c_double)], C.c_int),
        "nbody_cuda_calibrate_fp64": ([vp, C.POINTER(C.c_double)], C.c_int),
        "nbody_cuda_tree_export": ([vp, vp, sz, C.POINTER(sz)], C.c_int),
        "nbody_cuda_set_systems": ([vp, vp, sz], C.c_int),
        "nbody_cuda_batch_autotune": ([vp, P, vp, sz, C.POINTER(C.c_int)], C.c_int),
        "nbody_cuda_batch_config_count": ([], C.c_int),
        "nbody_cuda_batch_config": ([vp, C.c_int] + [C.POINTER(C.c_int)] * 3, C.c_int),
        "nbody_cuda_batch_set_config": ([vp, C.c_int], C.c_int),
        "nbody_cuda_system_energy": ([vp, P, vp, sz], C.c_int),
        "nbody_cuda_energy": ([vp, P, C.POINTER(C.c_double)], C.c_int),
        "nbody_cuda_update_graph": ([vp, P, C.c_int], C.c_int),
        "nbody_cuda_direct_variant_count": ([], C.c_int),
        "nbody_cuda_direct_variant": ([C.c_int] + [C.POINTER(C.c_int)] * 3, C.c_int),
        "nbody_cuda_set_direct_variant": ([vp, C.c_int], C.c_int),
        "nbody_cuda_direct_autotune": ([vp, P, vp, sz, C.POINTER(C.c_int)], C.c_int),
        "nbody_cuda_selftest_wait": ([vp, C.c_uint64], C.c_int),
        "nbody_cuda_set_transfer": ([vp, C.c_int], C.c_int),
        "nbody_cuda_transfer_info": ([vp] + [C.POINTER(C.c_int)] * 3 + [C.POINTER(C.c_uint64)], C.c_int),
        "nbody_cuda_prefetch": ([vp, u], C.c_int),
        "nbody_cuda_scene_disk": ([vp, C.POINTER(DiskArgs), sz, sz], C.c_int),
        "nbody_cuda_scene_cube": ([vp, C.POINTER(CubeArgs), sz, sz], C.c_int),
        "nbody_cuda_tree_query": ([vp, vp, sz, vp, sz, C.c_int, vp, sz, vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def probe() -> tuple[int, str]:
    buf = C.create_string_buffer(512)
    st = lib().nbody_cuda_probe(buf, len(buf))
    return st, buf.value.decode()


def _ptr(a: np.ndarray | None):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Context:
    """One nbody_cuda context (device bodies in one layout + stream + scratch)."""

    def __init__(self, layout: int = LAYOUT_SOA):
        h = C.c_void_p()
        st = lib().nbody_cuda_create(C.byref(h), layout)
        if st != OK:
            buf = C.create_string_buffer(512)
            lib().nbody_cuda_last_error(None, buf, len(buf))
            raise NbodyError(st, buf.value.decode())
        self.h = h
        self.layout = layout

    def close(self):
        if getattr(self, "h", None):
            lib().nbody_cuda_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def error(self) -> str:
        buf = C.create_string_buffer(512)
        lib().nbody_cuda_last_error(self.h, buf, len(buf))
        return buf.value.decode()

    def check(self, st: int):
        if st != OK:
            raise NbodyError(st, self.error())

    # --- bodies -----------------------------------------------------------------
    def upload_bodies(self, bodies: np.ndarray):
        b = np.ascontiguousarray(bodies, np.float32)
        assert b.ndim == 2 and b.shape[1] == 12
        self.check(lib().nbody_cuda_upload_bodies(self.h, _ptr(b), len(b)))

    def download_bodies(self, n: int | None = None, mask: int = READ_ALL, into: np.ndarray | None = None):
        n = self.count() if n is None else n
        out = np.zeros((n, 12), np.float32) if into is None else into
        self.check(lib().nbody_cuda_download_bodies(self.h, _ptr(out), n, mask))
        return out

    def upload_soa(self, pos_mass, vel_radius=None, acc=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (pos_mass, vel_radius, acc)]
        n = len(arrs[0])
        self.check(lib().nbody_cuda_upload_soa(self.h, *map(_ptr, arrs), n))

    def download_soa(self, n: int | None = None):
        n = self.count() if n is None else n
        out = [np.zeros((n, 4), np.float32) for _ in range(3)]
        self.check(lib().nbody_cuda_download_soa(self.h, *map(_ptr, out), n))
        return out

    def count(self) -> int:
        return int(lib().nbody_cuda_count(self.h))

    # --- transfer policy ---------------------------------------------------------
    def set_transfer(self, policy: int):
        self.check(lib().nbody_cuda_set_transfer(self.h, policy))

    def transfer_info(self) -> dict:
        pol, res, pg = C.c_int(), C.c_int(), C.c_int()
        hits = C.c_uint64()
        self.check(lib().nbody_cuda_transfer_info(self.h, C.byref(pol), C.byref(res), C.byref(pg), C.byref(hits)))
        return {"policy": pol.value, "resolved": res.value, "pageable": pg.value, "readback_hits": hits.value}

    def prefetch(self, mask: int = READ_ALL):
        self.check(lib().nbody_cuda_prefetch(self.h, mask))

    # --- ray query ---------------------------------------------------------------
    def tree_query(self, rays: np.ndarray, stop: int = QUERY_ALL, max_hits: int = 64,
                   nodes: np.ndarray | None = None):
        """Tree::query for every ray (rows of origin xyz, direction xyz) over `nodes`
        (NODE_DTYPE) or the last Barnes-Hut tree: (hits (nrays, max_hits), counts)."""
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        hits = np.zeros((len(r), max_hits), np.uint32)
        counts = np.zeros(len(r), np.uint32)
        nd = None if nodes is None else np.ascontiguousarray(nodes)
        self.check(lib().nbody_cuda_tree_query(self.h, None if nd is None else C.c_void_p(nd.ctypes.data),
                                               0 if nd is None else len(nd), _ptr(r), len(r), stop,
                                               _ptr(hits), max_hits, _ptr(counts)))
        return hits, counts

    # --- scene generators --------------------------------------------------------
    def scene_disk(self, num: int, begin: int = 0, **kw):
        """util::disk on the device over bodies [begin, begin + num); kw as disk_args."""
        a = disk_args(**kw)
        self.check(lib().nbody_cuda_scene_disk(self.h, C.byref(a), begin, num))

    def scene_cube(self, num: int, begin: int = 0, **kw):
        a = cube_args(**kw)
        self.check(lib().nbody_cuda_scene_cube(self.h, C.byref(a), begin, num))

    def reserve(self, n: int):
        self.check(lib().nbody_cuda_reserve(self.h, n))

    # --- stepping -------------------------------------------------------------------
    def accelerate(self, p: StepParams):
        self.check(lib().nbody_cuda_accelerate(self.h, C.byref(p)))

    def integrate(self, p: StepParams):
        self.check(lib().nbody_cuda_integrate(self.h, C.byref(p)))

    def update(self, p: StepParams, steps: int = 1):
        self.check(lib().nbody_cuda_update(self.h, C.byref(p), steps))

    def synchronize(self):
        self.check(lib().nbody_cuda_synchronize(self.h))

    def set_stream(self, stream: int | None):
        self.check(lib().nbody_cuda_set_stream(self.h, None if not stream else C.c_void_p(stream)))

    # --- caller-owned device buffers (integer device pointers) -------------------------------
    def dev_accel_soa(self, pos_mass: int, vel_radius: int | None, acc: int, n: int, p: StepParams):
        self.check(lib().nbody_cuda_dev_accel_soa(self.h, C.c_void_p(pos_mass),
                                                  C.c_void_p(vel_radius) if vel_radius else None,
                                                  C.c_void_p(acc), n, C.byref(p)))

    def dev_accel_aos(self, bodies: int, n: int, p: StepParams):
        self.check(lib().nbody_cuda_dev_accel_aos(self.h, C.c_void_p(bodies), n, C.byref(p)))

    def dev_integrate_soa(self, pos_mass: int, vel_radius: int, acc: int, n: int, p: StepParams):
        self.check(lib().nbody_cuda_dev_integrate_soa(self.h, C.c_void_p(pos_mass), C.c_void_p(vel_radius),
                                                      C.c_void_p(acc), n, C.byref(p)))

    # --- introspection -------------------------------------------------------------------------
    def launches(self) -> int:
        return int(lib().nbody_cuda_launch_count(self.h))

    def bh_stats(self) -> dict:
        out = (C.c_uint64 * 3)()
        self.check(lib().nbody_cuda_bh_stats(self.h, out))
        return {"interactions": int(out[0]), "visits": int(out[1]), "cells": int(out[2])}

    def bh_stage_ms(self) -> tuple[float, float]:
        """(tree build, traversal) device milliseconds of the last Barnes-Hut accelerate."""
        out = (C.c_float * 2)()
        self.check(lib().nbody_cuda_bh_stage_ms(self.h, out))
        return float(out[0]), float(out[1])

    def morton(self, p: StepParams):
        n = self.count()
        codes = np.zeros(n, np.uint64)
        order = np.zeros(n, np.uint32)
        box = (C.c_double * 4)()
        self.check(lib().nbody_cuda_morton(self.h, C.byref(p), _ptr(codes), _ptr(order), box))
        return codes, order, np.array(box[:])

    def accel_sampled(self, p: StepParams, targets) -> np.ndarray:
        t = np.ascontiguousarray(targets, np.int64)
        out = np.zeros((len(t), 3), np.float64)
        self.check(lib().nbody_cuda_accel_sampled(self.h, C.byref(p), _ptr(t), len(t), _ptr(out)))
        return out

    # --- batched systems and graphs ------------------------------------------------------------
    def set_systems(self, offsets):
        o = np.ascontiguousarray(offsets, np.int64)
        self.nsys = len(o) - 1
        self.check(lib().nbody_cuda_set_systems(self.h, _ptr(o), len(o) - 1))

    def batch_autotune(self, p: StepParams):
        n = int(lib().nbody_cuda_batch_config_count())
        times = np.zeros(n, np.float64)
        best = C.c_int()
        self.check(lib().nbody_cuda_batch_autotune(self.h, C.byref(p), _ptr(times), n, C.byref(best)))
        return best.value, times

    def batch_config(self, index: int = -1) -> dict:
        v = [C.c_int() for _ in range(3)]
        self.check(lib().nbody_cuda_batch_config(self.h, index, *[C.byref(x) for x in v]))
        return dict(zip(("threads_per_cta", "targets_per_thread", "sources_per_chunk"), (x.value for x in v)))

    def batch_set_config(self, index: int):
        self.check(lib().nbody_cuda_batch_set_config(self.h, index))

    def energy(self, p: StepParams) -> dict:
        """nbody_cuda_energy: kinetic and potential energy and momentum of all bodies."""
        out = (C.c_double * 5)()
        self.check(lib().nbody_cuda_energy(self.h, C.byref(p), out))
        return {"kinetic": out[0], "potential": out[1], "momentum": np.array(out[2:5])}

    def system_energy(self, p: StepParams, nsys: int | None = None) -> np.ndarray:
        n = nsys or getattr(self, "nsys", 1) or 1
        out = np.zeros((n, 5), np.float64)
        self.check(lib().nbody_cuda_system_energy(self.h, C.byref(p), _ptr(out), n))
        return out

    # --- direct-sum kernel shapes ----------------------------------------------------------
    @staticmethod
    def direct_variant(index: int) -> dict:
        v = [C.c_int() for _ in range(3)]
        st = lib().nbody_cuda_direct_variant(index, *[C.byref(x) for x in v])
        if st != OK:
            raise NbodyError(st, f"no direct-sum kernel shape {index}")
        return dict(zip(("targets_per_thread", "block", "packed"), (x.value for x in v)))

    @staticmethod
    def direct_variant_count() -> int:
        return int(lib().nbody_cuda_direct_variant_count())

    def set_direct_variant(self, index: int):
        self.check(lib().nbody_cuda_set_direct_variant(self.h, index))

    def direct_autotune(self, p: StepParams):
        n = int(lib().nbody_cuda_direct_variant_count())
        times = np.zeros(n, np.float64)
        best = C.c_int()
        self.check(lib().nbody_cuda_direct_autotune(self.h, C.byref(p), _ptr(times), n, C.byref(best)))
        return best.value, times

    def update_graph(self, p: StepParams, steps: int):
        self.check(lib().nbody_cuda_update_graph(self.h, C.byref(p), steps))

    def tree_export(self) -> np.ndarray:
        """The last Barnes-Hut tree as reference-layout nodes (48-byte records)."""
        n = C.c_size_t()
        self.check(lib().nbody_cuda_tree_export(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value, NODE_DTYPE)
        self.check(lib().nbody_cuda_tree_export(self.h, _ptr(out), n.value, C.byref(n)))
        return out

    def split_origin(self) -> np.ndarray:
        out = (C.c_double * 4)()
        self.check(lib().nbody_cuda_split_origin(self.h, out))
        return np.array(out[:])

    def calibrate_fp64(self) -> float:
        v = C.c_double()
        self.check(lib().nbody_cuda_calibrate_fp64(self.h, C.byref(v)))
        return v.value

    def calibrate_fp32(self) -> tuple[float, float]:
        s, p = C.c_double(), C.c_double()
        self.check(lib().nbody_cuda_calibrate_fp32(self.h, C.byref(s), C.byref(p)))
        return s.value, p.value

    def last_direct_config(self) -> dict:
        v = [C.c_int() for _ in range(5)]
        self.check(lib().nbody_cuda_last_direct_config(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("targets_per_thread", "block", "tile", "jsplit", "grid"), (x.value for x in v)))
