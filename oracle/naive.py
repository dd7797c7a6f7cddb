"""ctypes binding of the naive checker — TEST INFRASTRUCTURE ONLY.

``naive.cpp`` decides the same verdicts and collected hazard sets as the reference's collision
detection engine without any quadtree: every query is tested against every edge of every relevant
hazard, plus the containment rule.  It shares no code with the oracle (``cde_oracle.cpp``) or the
product, so it cross-checks the quadtree reading both of them rely on.  Only the test-suite loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnaive.so")
QUERY_DTYPE = np.dtype([("item", "<u4"), ("cos", "<f4"), ("sin", "<f4"), ("tx", "<f4"), ("ty", "<f4")])

_lib = None


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(HERE, "naive.cpp")
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
            subprocess.run(["make", "-s", "-C", HERE], check=True)
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        f32p = C.POINTER(C.c_float)
        u32p = C.POINTER(C.c_uint32)
        u8p = C.POINTER(C.c_uint8)
        sig = {
            "nv_new": (P, [f32p]),
            "nv_free": (None, [P]),
            "nv_set_hazard": (C.c_int32, [P, C.c_uint32, C.c_int32, C.c_int32, f32p, C.c_uint32, f32p]),
            "nv_add_item": (C.c_int32, [P, f32p, C.c_uint32, f32p, f32p, C.c_uint32, f32p, C.c_uint32]),
            "nv_detect_batch": (None, [P, P, C.c_uint64, u32p, C.c_uint32, u8p, C.c_int32]),
            "nv_collect_batch": (C.c_int64, [P, P, C.c_uint64, u32p, C.c_uint32, u32p, u32p, C.c_uint64, C.c_int32]),
            "nv_explain": (C.c_int32, [P, P, C.c_uint32]),
            "nv_fpa_eq": (C.c_int32, [C.c_float, C.c_float]),
            "nv_seg_cross": (C.c_int32, [f32p, f32p]),
            "nv_inside": (C.c_int32, [f32p, C.c_uint32, C.c_float, C.c_float]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _p(a, ct=C.c_float):
    return a.ctypes.data_as(C.POINTER(ct))


def _ids(ignored):
    return np.ascontiguousarray(np.asarray(list(ignored) if ignored is not None else [], dtype=np.uint32))


class NaiveChecker:
    """Every item type and live hazard of a layout, with no spatial index."""

    def __init__(self, cde_bbox):
        self._bbox = _f32(cde_bbox)
        self.h = lib().nv_new(_p(self._bbox))

    def __del__(self):
        if getattr(self, "h", None):
            lib().nv_free(self.h)
            self.h = None

    @classmethod
    def from_layout(cls, lay):
        """Items and hazards of a ``jcde.workload.Layout`` (hazard keys as registered)."""
        nc = cls(lay.cde_bbox)
        for it in lay.items:
            nc.add_item(it.xy, it.poi, np.asarray(it.poles)[: it.n_ff_poles])
        for i, hz in enumerate(lay.hazards):
            nc.set_hazard(hz.key if hz.key >= 0 else i, hz.kind, hz.xy, hz.poi)
        return nc

    def set_hazard(self, key: int, kind: int, xy, poi, live: bool = True) -> None:
        xy, poi = _f32(xy), _f32(poi)
        lib().nv_set_hazard(self.h, key, kind, int(live), _p(xy), len(xy), _p(poi))

    def add_item(self, xy, poi, ff_poles, piers=None) -> int:
        xy, poi = _f32(xy), _f32(poi)
        ff = _f32(np.asarray(ff_poles).reshape(-1, 3))
        pr = _f32(np.zeros((0, 4)) if piers is None else np.asarray(piers).reshape(-1, 4))
        return int(lib().nv_add_item(self.h, _p(xy), len(xy), _p(poi), _p(ff), len(ff), _p(pr), len(pr)))

    def detect_batch(self, queries, ignored=None, n_threads: int = 0) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=QUERY_DTYPE)
        ids = _ids(ignored)
        out = np.zeros(len(q), np.uint8)
        lib().nv_detect_batch(self.h, q.ctypes.data, len(q), _p(ids, C.c_uint32), len(ids), _p(out, C.c_uint8),
                              n_threads or (os.cpu_count() or 1))
        return out

    def explain(self, query, key: int) -> int:
        """Clause flags for one query against one hazard (see nv_explain in naive.cpp)."""
        q = np.ascontiguousarray(np.asarray(query, dtype=QUERY_DTYPE).reshape(1))
        return int(lib().nv_explain(self.h, q.ctypes.data, int(key)))

    def collect_batch(self, queries, ignored=None, n_threads: int = 0):
        """(counts, ids): CSR of the ascending colliding hazard keys per query."""
        q = np.ascontiguousarray(queries, dtype=QUERY_DTYPE)
        ids = _ids(ignored)
        counts = np.zeros(len(q), np.uint32)
        cap = max(16, 8 * len(q))
        while True:
            out = np.zeros(cap, np.uint32)
            r = lib().nv_collect_batch(self.h, q.ctypes.data, len(q), _p(ids, C.c_uint32), len(ids),
                                       _p(counts, C.c_uint32), _p(out, C.c_uint32), cap,
                                       n_threads or (os.cpu_count() or 1))
            if r >= 0:
                return counts, out[:r]
            cap = -r


def fpa_eq(a, b) -> bool:
    return bool(lib().nv_fpa_eq(np.float32(a), np.float32(b)))


def seg_cross(e1, e2) -> bool:
    a, b = _f32(e1), _f32(e2)
    return bool(lib().nv_seg_cross(_p(a), _p(b)))


def inside(xy, p) -> bool:
    xy = _f32(xy)
    return bool(lib().nv_inside(_p(xy), len(xy), np.float32(p[0]), np.float32(p[1])))
