"""ctypes binding of the oracle — TEST INFRASTRUCTURE ONLY.

The oracle (``cde_oracle.cpp``) is a C++ restatement of the reference's f32 collision detection
engine.  Only the test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
load it, as the reference the product's results are compared with.  Parity of the oracle itself is UNPINNED (the reference is Rust and
cannot be built here, and it ships no golden vectors); see the header of ``cde_oracle.cpp``.

The classes mirror the duck-typed backend interface of ``jcde.workload`` so that the same seeded
workload generator can drive the oracle or the GPU engine.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

QUERY_DTYPE = np.dtype([("item", "<u4"), ("cos", "<f4"), ("sin", "<f4"), ("tx", "<f4"), ("ty", "<f4")])

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, -ffp-contract=off)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
        os.path.join(HERE, "cde_oracle.cpp")
    ):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        f32p = C.POINTER(C.c_float)
        u32p = C.POINTER(C.c_uint32)
        u64p = C.POINTER(C.c_uint64)
        u8p = C.POINTER(C.c_uint8)
        sig = {
            "or_engine_new": (P, [C.c_uint8, C.c_uint8, f32p]),
            "or_engine_free": (None, [P]),
            "or_register_hazard": (C.c_int32, [P, C.c_int32, C.c_int32, f32p, C.c_uint32, f32p]),
            "or_deregister_hazard": (C.c_int32, [P, C.c_uint32]),
            "or_add_item": (C.c_int32, [P, f32p, C.c_uint32, f32p, f32p, C.c_uint32, C.c_uint32, f32p, C.c_uint32]),
            "or_detect_batch": (None, [P, P, C.c_uint64, u32p, C.c_uint32, u8p, C.c_int32, u64p, C.c_int32]),
            "or_collect_poly": (C.c_int32, [P, f32p, C.c_uint32, f32p, u32p, C.c_uint32, u32p, C.c_uint32]),
            "or_collect_surrogate": (C.c_int32, [P, C.c_uint32, f32p, u32p, C.c_uint32, u32p, C.c_uint32]),
            "or_collect_batch": (C.c_int64, [P, P, C.c_uint64, u32p, C.c_uint32, u32p, u32p, C.c_uint64, C.c_int32]),
            "or_detect_poly": (C.c_int32, [P, f32p, C.c_uint32, f32p, u32p, C.c_uint32]),
            "or_detect_surrogate": (C.c_int32, [P, C.c_uint32, f32p, u32p, C.c_uint32]),
            "or_spolygon_new": (C.c_int32, [f32p, C.c_uint32, f32p, f32p, f32p, f32p]),
            "or_surrogate_poles": (C.c_int32, [f32p, C.c_uint32, C.c_float, f32p, u32p, f32p, C.c_int32, f32p, C.c_uint32, u32p]),
            "or_centroid": (None, [f32p, C.c_uint32, C.c_float, f32p]),
            "or_simplify_shape": (C.c_int32, [f32p, C.c_uint32, C.c_float, C.c_int32, C.c_float, f32p, u32p]),
            "or_close_concavities": (C.c_int32, [f32p, C.c_uint32, C.c_int32, C.c_float, f32p, u32p]),
            "or_fpa_eq": (C.c_int32, [C.c_float, C.c_float]),
            "or_edge_intersection": (C.c_int32, [f32p, f32p]),
            "or_rect_collides_edge": (C.c_int32, [f32p, f32p]),
            "or_point_in_poly": (C.c_int32, [f32p, C.c_uint32, C.c_float, C.c_float]),
            "or_almost_relation": (C.c_int32, [f32p, f32p]),
            "or_edge_quadrants": (None, [f32p, f32p, u8p]),
            "or_tree_dump": (C.c_uint64, [P, u32p, C.c_uint64]),
            "or_n_slots": (C.c_uint32, [P]),
            "or_proxy_f64": (None, [C.c_uint64, C.POINTER(C.c_double), u32p, u32p, f32p, f32p, C.c_uint64, u32p, C.c_uint32,
                                     C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _filter_arr(ignored):
    ids = np.ascontiguousarray(np.asarray(list(ignored) if ignored is not None else [], dtype=np.uint32))
    return ids, len(ids)


class OracleEngine:
    """CPU restatement of ``CDEngine`` (cd_engine.rs:22-341) with dense hazard keys."""

    def __init__(self, depth: int, cd_threshold: int, bbox):
        self._bbox = _f32(bbox)
        self.h = lib().or_engine_new(depth, cd_threshold, _ptr(self._bbox, C.c_float))
        self.n_items = 0

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_engine_free(self.h)
            self.h = None

    def bbox(self):
        return tuple(float(v) for v in self._bbox)

    def register_hazard(self, kind: int, dynamic: bool, xy, poi, tag: int = 0) -> int:
        xy = _f32(xy)
        poi = _f32(poi)
        k = lib().or_register_hazard(self.h, kind, int(dynamic), _ptr(xy, C.c_float), len(xy), _ptr(poi, C.c_float))
        return int(k)

    def deregister_hazard(self, key: int) -> None:
        if lib().or_deregister_hazard(self.h, key) != 0:
            raise KeyError(key)

    def add_item(self, xy, poi, poles, n_ff_poles: int, piers=None) -> int:
        xy, poi, poles = _f32(xy), _f32(poi), _f32(np.asarray(poles).reshape(-1, 3))
        piers = _f32(np.zeros((0, 4)) if piers is None else np.asarray(piers).reshape(-1, 4))
        r = lib().or_add_item(self.h, _ptr(xy, C.c_float), len(xy), _ptr(poi, C.c_float), _ptr(poles, C.c_float),
                              len(poles), n_ff_poles, _ptr(piers, C.c_float), len(piers))
        self.n_items += 1
        return int(r)

    def detect_batch(self, queries: np.ndarray, ignored=None, n_threads: int = 0, counts=None, mode: int = 3) -> np.ndarray:
        """mode 3: surrogate || polygon (ci_bench.rs:111-119); 1: surrogate only; 2: polygon only;
        4: as 3, with 1 for collisions the surrogate found and 3 for those the polygon pass found."""
        q = np.ascontiguousarray(queries, dtype=QUERY_DTYPE)
        out = np.zeros(len(q), dtype=np.uint8)
        ids, nf = _filter_arr(ignored)
        nt = n_threads or (os.cpu_count() or 1)
        cnt = counts if counts is not None else None
        lib().or_detect_batch(self.h, q.ctypes.data, len(q), _ptr(ids, C.c_uint32), nf, _ptr(out, C.c_uint8), nt,
                              _ptr(cnt, C.c_uint64) if cnt is not None else None, mode)
        return out

    def detect_with_surrogate(self, queries: np.ndarray, ignored=None):
        """(verdicts, number of queries the surrogate pass left undecided) in one pass."""
        v = self.detect_batch(queries, ignored, mode=4)
        return np.where(v == 3, 1, v).astype(np.uint8), int(((v == 0) | (v == 3)).sum())

    def collect_batch(self, queries: np.ndarray, ignored=None, n_threads: int = 0):
        """Returns (counts, ids): CSR of the sorted colliding hazard keys per query."""
        q = np.ascontiguousarray(queries, dtype=QUERY_DTYPE)
        ids, nf = _filter_arr(ignored)
        counts = np.zeros(len(q), dtype=np.uint32)
        nt = n_threads or (os.cpu_count() or 1)
        cap = max(16, 8 * len(q))
        while True:
            out = np.zeros(cap, dtype=np.uint32)
            r = lib().or_collect_batch(self.h, q.ctypes.data, len(q), _ptr(ids, C.c_uint32), nf,
                                       _ptr(counts, C.c_uint32), _ptr(out, C.c_uint32), cap, nt)
            if r >= 0:
                return counts, out[:r]
            cap = -r

    def detect_poly(self, xy, poi, ignored=None) -> bool:
        xy, poi = _f32(xy), _f32(poi)
        ids, nf = _filter_arr(ignored)
        return bool(lib().or_detect_poly(self.h, _ptr(xy, C.c_float), len(xy), _ptr(poi, C.c_float),
                                         _ptr(ids, C.c_uint32), nf))

    def collect_poly(self, xy, poi, ignored=None) -> list:
        xy, poi = _f32(xy), _f32(poi)
        ids, nf = _filter_arr(ignored)
        keys = np.zeros(4096, np.uint32)
        n = lib().or_collect_poly(self.h, _ptr(xy, C.c_float), len(xy), _ptr(poi, C.c_float), _ptr(ids, C.c_uint32),
                                  nf, _ptr(keys, C.c_uint32), len(keys))
        return [int(k) for k in keys[:n]]

    def collect_surrogate(self, item: int, transform, ignored=None) -> list:
        t = _f32(transform)
        ids, nf = _filter_arr(ignored)
        keys = np.zeros(4096, np.uint32)
        n = lib().or_collect_surrogate(self.h, item, _ptr(t, C.c_float), _ptr(ids, C.c_uint32), nf,
                                       _ptr(keys, C.c_uint32), len(keys))
        return [int(k) for k in keys[:n]]

    def detect_surrogate(self, item: int, transform, ignored=None) -> bool:
        t = _f32(transform)
        ids, nf = _filter_arr(ignored)
        return bool(lib().or_detect_surrogate(self.h, item, _ptr(t, C.c_float), _ptr(ids, C.c_uint32), nf))

    def tree_dump(self) -> np.ndarray:
        n = lib().or_tree_dump(self.h, None, 0)
        out = np.zeros(n, dtype=np.uint32)
        lib().or_tree_dump(self.h, _ptr(out, C.c_uint32), n)
        return out


class OracleBackend:
    """Backend for ``jcde.workload``: host prep + engines from the oracle."""

    name = "oracle"

    @staticmethod
    def spolygon_new(xy):
        xy = _f32(xy)
        n = len(xy)
        xy_out = np.zeros_like(xy)
        bbox = np.zeros(4, np.float32)
        stats = np.zeros(2, np.float32)
        poi = np.zeros(3, np.float32)
        r = lib().or_spolygon_new(_ptr(xy, C.c_float), n, _ptr(xy_out, C.c_float), _ptr(bbox, C.c_float),
                                  _ptr(stats, C.c_float), _ptr(poi, C.c_float))
        if r != 0:
            raise ValueError("invalid simple polygon")
        return xy_out, bbox, stats[0], stats[1], poi

    @staticmethod
    def simplify_shape(xy, area, deflate, tolerance):
        """simplify_shape (shape_modification.rs:48-144) before its final SPolygon::new."""
        xy = _f32(xy)
        out = np.zeros_like(xy)
        n = np.zeros(1, np.uint32)
        lib().or_simplify_shape(_ptr(xy, C.c_float), len(xy), np.float32(area), int(bool(deflate)), np.float32(tolerance),
                                _ptr(out, C.c_float), _ptr(n, C.c_uint32))
        return out[: int(n[0])].copy()

    @staticmethod
    def close_concavities(xy, deflate, ratio):
        """close_narrow_concavities (shape_modification.rs:374-478), after SPolygon::new of xy."""
        xy = _f32(xy)
        out = np.zeros_like(xy)
        n = np.zeros(1, np.uint32)
        lib().or_close_concavities(_ptr(xy, C.c_float), len(xy), int(bool(deflate)), np.float32(ratio),
                                   _ptr(out, C.c_float), _ptr(n, C.c_uint32))
        return out[: int(n[0])].copy()

    @staticmethod
    def surrogate_poles(xy, area, poi, limits):
        xy, poi = _f32(xy), _f32(poi)
        ln = np.ascontiguousarray([l[0] for l in limits], dtype=np.uint32)
        lc = np.ascontiguousarray([l[1] for l in limits], dtype=np.float32)
        cap = 1024
        out = np.zeros((cap, 3), np.float32)
        n = np.zeros(1, np.uint32)
        r = lib().or_surrogate_poles(_ptr(xy, C.c_float), len(xy), np.float32(area), _ptr(poi, C.c_float),
                                     _ptr(ln, C.c_uint32), _ptr(lc, C.c_float), len(limits), _ptr(out, C.c_float),
                                     cap, _ptr(n, C.c_uint32))
        if r != 0:
            raise ValueError("pole generation failed")
        return out[: int(n[0])].copy()

    @staticmethod
    def new_engine(depth: int, cd_threshold: int, bbox):
        return OracleEngine(depth, cd_threshold, bbox)


def centroid(xy, area) -> np.ndarray:
    xy = _f32(xy)
    out = np.zeros(2, np.float32)
    lib().or_centroid(_ptr(xy, C.c_float), len(xy), np.float32(area), _ptr(out, C.c_float))
    return out


def fpa_eq(a, b) -> bool:
    return bool(lib().or_fpa_eq(np.float32(a), np.float32(b)))


def edge_intersection(e1, e2) -> bool:
    a, b = _f32(e1), _f32(e2)
    return bool(lib().or_edge_intersection(_ptr(a, C.c_float), _ptr(b, C.c_float)))


def rect_collides_edge(r, e) -> bool:
    a, b = _f32(r), _f32(e)
    return bool(lib().or_rect_collides_edge(_ptr(a, C.c_float), _ptr(b, C.c_float)))


def point_in_poly(xy, p) -> bool:
    xy = _f32(xy)
    return bool(lib().or_point_in_poly(_ptr(xy, C.c_float), len(xy), np.float32(p[0]), np.float32(p[1])))


def almost_relation(a, b) -> int:
    """0 Intersecting, 1 Enclosed, 2 Surrounding, 3 Disjoint (geo_enums.rs:10-19)."""
    x, y = _f32(a), _f32(b)
    return int(lib().or_almost_relation(_ptr(x, C.c_float), _ptr(y, C.c_float)))


def edge_quadrants(e, r):
    a, b = _f32(e), _f32(r)
    out = np.zeros(4, np.uint8)
    lib().or_edge_quadrants(_ptr(a, C.c_float), _ptr(b, C.c_float), _ptr(out, C.c_uint8))
    return [bool(v) for v in out]


def proxy_f64(params, items, item_poles, hazard_poles, ignored=None, n_threads=0):
    """FP64 pole-overlap proxy and gradient (theta, tx, ty) — the tolerance reference.

    params [n, 3] (float32 values are taken exactly; float64 allowed for finite differences),
    items [n], item_poles: list of (k, 3) arrays per item type,
    hazard_poles [m, 4] float32 (x, y, r, key as uint32 bits)."""
    params = np.ascontiguousarray(params, dtype=np.float64).reshape(-1, 3)
    items = np.ascontiguousarray(items, dtype=np.uint32)
    offs = np.zeros(len(item_poles) + 1, np.uint32)
    offs[1:] = np.cumsum([len(p) for p in item_poles])
    ip = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float32).reshape(-1, 3) for p in item_poles]))
    hp = np.ascontiguousarray(hazard_poles, dtype=np.float32).reshape(-1, 4)
    ids, nf = _filter_arr(ignored)
    val = np.zeros(len(params), np.float64)
    grad = np.zeros((len(params), 3), np.float64)
    lib().or_proxy_f64(len(params), params.ctypes.data_as(C.POINTER(C.c_double)), _ptr(items, C.c_uint32),
                       _ptr(offs, C.c_uint32),
                       _ptr(ip, C.c_float), _ptr(hp, C.c_float), len(hp), _ptr(ids, C.c_uint32), nf,
                       val.ctypes.data_as(C.POINTER(C.c_double)), grad.ctypes.data_as(C.POINTER(C.c_double)),
                       n_threads or (os.cpu_count() or 1))
    return val, grad
