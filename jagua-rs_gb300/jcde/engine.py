"""Python mirror of the reference's ``CDEngine`` over the jcde C ABI.

The method names, argument meanings and failure behaviour follow
jagua-rs/src/collision_detection/cd_engine.rs: ``register_hazard`` / ``deregister_hazard_by_key`` /
``deregister_hazard_by_entity`` / ``detect_poly_collision`` / ``detect_surrogate_collision`` /
``collect_poly_collisions`` / ``collect_surrogate_collisions`` / ``save`` / ``restore`` / ``bbox``.
Where the reference panics (unknown key, cd_engine.rs:78 and :91) these raise ``KeyError``.

Every query runs on the GPU through libjcde.so; nothing here answers a query on the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _ffi
from ._ffi import (check, jcde_config, jcde_filter, jcde_hazard, jcde_lbf_params, jcde_rect, jcde_resident_config,
                   jcde_tuning, lib)
from .workload import QUERY_DTYPE

PLACED_ITEM, EXTERIOR, HOLE, QUALITY_ZONE = 0, 1, 2, 3


@dataclass
class CDEConfig:
    """CDEConfig (cd_engine.rs:346-353) with its SPSurrogateConfig (sp_surrogate.rs:120-131)."""

    quadtree_depth: int = 5
    cd_threshold: int = 16
    n_pole_limits: tuple = ((100, 0.0), (20, 0.75), (10, 0.90))
    n_ff_poles: int = 2
    n_ff_piers: int = 0

    def to_c(self) -> jcde_config:
        c = jcde_config()
        c.quadtree_depth = self.quadtree_depth
        c.cd_threshold = self.cd_threshold
        c.n_pole_limits = len(self.n_pole_limits)
        for i, (n, cov) in enumerate(self.n_pole_limits):
            c.pole_limit_n[i] = n
            c.pole_limit_coverage[i] = cov
        c.n_ff_poles = self.n_ff_poles
        c.n_ff_piers = self.n_ff_piers
        return c


@dataclass
class Hazard:
    """Hazard (hazards/hazard.rs:16-23): entity kind + tag, final shape (vertices + poi), dynamic."""

    kind: int
    xy: np.ndarray
    poi: np.ndarray
    dynamic: bool = False
    tag: int = 0


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _c_hazard(h: Hazard, keep: list) -> jcde_hazard:
    xy = _f32(h.xy).reshape(-1, 2)
    keep.append(xy)
    ch = jcde_hazard()
    ch.kind = int(h.kind)
    ch.dynamic = int(bool(h.dynamic))
    ch.xy = _fp(xy)
    ch.n_vertices = len(xy)
    for i in range(3):
        ch.poi[i] = float(h.poi[i])
    ch.tag = int(h.tag)
    return ch


class _Filter:
    """HazardFilter as a jcde_filter: None/empty = NoFilter, else a HazKeyFilter of keys."""

    def __init__(self, ignored):
        keys = [] if ignored is None else [int(k) for k in (ignored if hasattr(ignored, "__iter__") else [ignored])]
        self.arr = np.ascontiguousarray(np.asarray(keys, dtype=np.uint32))
        self.c = jcde_filter()
        self.c.ignored = self.arr.ctypes.data_as(C.POINTER(C.c_uint32))
        self.c.n_ignored = len(self.arr)

    @property
    def ref(self):
        return C.byref(self.c)


def _stream_handle(stream) -> int | None:
    if stream is None:
        try:
            import torch

            return torch.cuda.current_stream().cuda_stream
        except Exception:
            return None
    return int(getattr(stream, "cuda_stream", stream))


class CDEngine:
    """GPU collision detection engine with the reference's query surface (cd_engine.rs:22-341)."""

    def __init__(self, bbox, static_hazards=(), config: CDEConfig | None = None):
        self.config = config or CDEConfig()
        self._cfg = self.config.to_c()
        keep: list = []
        arr = (jcde_hazard * max(1, len(static_hazards)))()
        for i, h in enumerate(static_hazards):
            arr[i] = _c_hazard(h, keep)
        handle = C.c_void_p()
        check(lib().jcde_create(C.byref(self._cfg), jcde_rect(*[float(v) for v in bbox]), arr, len(static_hazards),
                                C.byref(handle)), "jcde_create")
        self.h = handle
        self.n_items = 0

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            try:
                lib().jcde_destroy(h)
            except Exception:
                pass
            self.h = None

    # --- hazards -------------------------------------------------------------------------------
    def register_hazard(self, hazard: Hazard) -> int:
        keep: list = []
        ch = _c_hazard(hazard, keep)
        k = C.c_uint32()
        check(lib().jcde_register_hazard(self.h, C.byref(ch), C.byref(k)), "register_hazard")
        return k.value

    def deregister_hazard_by_key(self, key: int) -> None:
        st = lib().jcde_deregister_hazard(self.h, int(key))
        if st == _ffi.ERR_NOT_FOUND:
            raise KeyError(f"Cannot deregister hazard that is not registered: {key}")
        check(st, "deregister_hazard_by_key")

    def deregister_hazard_by_entity(self, kind: int, tag: int) -> int:
        k = C.c_uint32()
        st = lib().jcde_deregister_hazard_by_entity(self.h, int(kind), int(tag), C.byref(k))
        if st == _ffi.ERR_NOT_FOUND:
            raise KeyError(f"Cannot deregister hazard that is not registered: kind {kind} tag {tag}")
        check(st, "deregister_hazard_by_entity")
        return k.value

    def n_hazard_slots(self) -> int:
        n = C.c_uint32()
        check(lib().jcde_n_hazard_slots(self.h, C.byref(n)), "n_hazard_slots")
        return n.value

    def bbox(self):
        r = jcde_rect()
        check(lib().jcde_bbox(self.h, C.byref(r)), "bbox")
        return (r.x_min, r.y_min, r.x_max, r.y_max)

    # --- items ---------------------------------------------------------------------------------
    def register_item(self, xy, poi, poles, piers=None) -> int:
        xy, poi = _f32(xy).reshape(-1, 2), _f32(poi)
        poles = _f32(np.asarray(poles).reshape(-1, 3))
        piers = _f32(np.zeros((0, 4)) if piers is None else np.asarray(piers).reshape(-1, 4))
        out = C.c_uint32()
        check(lib().jcde_register_item(self.h, _fp(xy), len(xy), _fp(poi), _fp(poles), len(poles),
                                       _fp(piers) if len(piers) else None, len(piers), C.byref(out)), "register_item")
        self.n_items += 1
        return out.value

    # --- single queries (reference signatures) ---------------------------------------------------
    def detect_poly_collision(self, xy, poi, filter=None) -> bool:
        xy, poi = _f32(xy).reshape(-1, 2), _f32(poi)
        f = _Filter(filter)
        out = C.c_uint8()
        check(lib().jcde_detect_poly(self.h, _fp(xy), len(xy), _fp(poi), f.ref, C.byref(out)), "detect_poly_collision")
        return bool(out.value)

    def detect_surrogate_collision(self, item: int, transform, filter=None) -> bool:
        t = _f32(transform)
        f = _Filter(filter)
        out = C.c_uint8()
        st = lib().jcde_detect_surrogate(self.h, int(item), _fp(t), f.ref, C.byref(out))
        if st == _ffi.ERR_NOT_FOUND:
            raise KeyError(f"unknown item {item}")
        check(st, "detect_surrogate_collision")
        return bool(out.value)

    def collect_poly_collisions(self, xy, poi, filter=None) -> list:
        xy, poi = _f32(xy).reshape(-1, 2), _f32(poi)
        f = _Filter(filter)
        cap = max(1, self.n_hazard_slots())
        keys = np.zeros(cap, np.uint32)
        n = C.c_uint32()
        check(lib().jcde_collect_poly(self.h, _fp(xy), len(xy), _fp(poi), f.ref,
                                      keys.ctypes.data_as(C.POINTER(C.c_uint32)), cap, C.byref(n)), "collect_poly")
        return [int(k) for k in keys[: n.value]]

    def collect_surrogate_collisions(self, item: int, transform, filter=None) -> list:
        t = _f32(transform)
        f = _Filter(filter)
        cap = max(1, self.n_hazard_slots())
        keys = np.zeros(cap, np.uint32)
        n = C.c_uint32()
        check(lib().jcde_collect_surrogate(self.h, int(item), _fp(t), f.ref,
                                           keys.ctypes.data_as(C.POINTER(C.c_uint32)), cap, C.byref(n)),
              "collect_surrogate")
        return [int(k) for k in keys[: n.value]]

    # --- batched queries -----------------------------------------------------------------------
    def detect_batch(self, queries, filter=None, out=None, stream=None, mode: str = "both"):
        """Verdicts of a query batch.

        ``queries`` is either a numpy array of QUERY_DTYPE (host path: copies in, kernel, copies
        out) or a CUDA torch uint8/int tensor holding packed 20-byte queries (device path, stream
        ordered; ``out`` must then be a CUDA uint8 tensor).
        """
        f = _Filter(filter)
        if isinstance(queries, np.ndarray):
            q = np.ascontiguousarray(queries, dtype=QUERY_DTYPE)
            res = np.zeros(len(q), np.uint8) if out is None else out
            if mode != "both":
                raise ValueError("host path supports mode='both' only")
            check(lib().jcde_detect_batch_host(self.h, q.ctypes.data, len(q), f.ref, res.ctypes.data), "detect_batch")
            return res
        n = queries.numel() * queries.element_size() // QUERY_DTYPE.itemsize
        if out is None:
            import torch

            out = torch.empty(n, dtype=torch.uint8, device=queries.device)
        fn = {"both": lib().jcde_detect_batch, "surrogate": lib().jcde_detect_surrogate_batch,
              "poly": lib().jcde_detect_poly_batch}[mode]
        check(fn(self.h, queries.data_ptr(), n, f.ref, out.data_ptr(), _stream_handle(stream)), "detect_batch")
        return out

    def collect_batch(self, queries, filter=None, ids_cap: int | None = None, stream=None):
        """Colliding hazard keys per query as (offsets, counts, ids) CUDA tensors (device path)."""
        import torch

        f = _Filter(filter)
        if isinstance(queries, np.ndarray):
            q = torch.from_numpy(np.ascontiguousarray(queries, dtype=QUERY_DTYPE).view(np.uint8)).cuda()
        else:
            q = queries
        n = q.numel() * q.element_size() // QUERY_DTYPE.itemsize
        dev = q.device
        cap = ids_cap if ids_cap is not None else max(1024, 4 * n)
        while True:
            offsets = torch.empty(n, dtype=torch.int32, device=dev)
            counts = torch.empty(n, dtype=torch.int32, device=dev)
            ids = torch.empty(max(1, cap), dtype=torch.int32, device=dev)
            total = torch.zeros(1, dtype=torch.int32, device=dev)
            check(lib().jcde_collect_batch(self.h, q.data_ptr(), n, f.ref, offsets.data_ptr(), counts.data_ptr(),
                                           ids.data_ptr(), cap, total.data_ptr(), _stream_handle(stream)),
                  "collect_batch")
            t = int(total.item())
            if t <= cap:
                return offsets, counts, ids[:t], t
            cap = t

    # --- pole-overlap proxy ---------------------------------------------------------------------
    def set_hazard_poles(self, key: int, poles) -> None:
        """Surrogate poles (x, y, r) of hazard `key`, used by the overlap proxy."""
        p = _f32(np.asarray(poles).reshape(-1, 3))
        st = lib().jcde_set_hazard_poles(self.h, int(key), _fp(p) if len(p) else None, len(p))
        if st == _ffi.ERR_NOT_FOUND:
            raise KeyError(key)
        check(st, "set_hazard_poles")

    def proxy_batch(self, params, items, filter=None, stream=None, out=None):
        """(value, grad) CUDA tensors of the proxy for (theta, tx, ty) params [n, 3] and items [n];
        `out` = (value [n], grad [n, 3]) float32 tensors to write into."""
        import torch

        f = _Filter(filter)
        n = items.numel()
        if out is not None:
            val, grad = out
        else:
            val = torch.empty(n, dtype=torch.float32, device=params.device)
            grad = torch.empty((n, 3), dtype=torch.float32, device=params.device)
        check(lib().jcde_proxy_batch(self.h, params.data_ptr(), items.data_ptr(), n, f.ref, val.data_ptr(),
                                     grad.data_ptr(), _stream_handle(stream)), "proxy_batch")
        return val, grad

    def proxy_forward(self, params, items, filter=None, stream=None):
        import torch

        f = _Filter(filter)
        n = items.numel()
        val = torch.empty(n, dtype=torch.float32, device=params.device)
        check(lib().jcde_proxy_forward(self.h, params.data_ptr(), items.data_ptr(), n, f.ref, val.data_ptr(),
                                       _stream_handle(stream)), "proxy_forward")
        return val

    def proxy_backward(self, params, items, grad_value=None, filter=None, stream=None):
        import torch

        f = _Filter(filter)
        n = items.numel()
        grad = torch.empty((n, 3), dtype=torch.float32, device=params.device)
        gv = None if grad_value is None else grad_value.contiguous()
        check(lib().jcde_proxy_backward(self.h, params.data_ptr(), items.data_ptr(), n, f.ref,
                                        None if gv is None else gv.data_ptr(), grad.data_ptr(),
                                        _stream_handle(stream)), "proxy_backward")
        return grad

    def separate_batch(self, params, items, steps=20, step_t=0.25, step_th=0.25, clearance=0.0, filter=None,
                       stream=None):
        """Gradient-descent separation in place on params [n, 3]; returns (packed queries, final P)."""
        import torch

        f = _Filter(filter)
        n = items.numel()
        q = torch.empty(n * QUERY_DTYPE.itemsize, dtype=torch.uint8, device=params.device)
        val = torch.empty(n, dtype=torch.float32, device=params.device)
        check(lib().jcde_separate_batch(self.h, params.data_ptr(), items.data_ptr(), n, steps, step_t, step_th,
                                        clearance, f.ref, q.data_ptr(), val.data_ptr(), _stream_handle(stream)),
              "separate_batch")
        return q, val

    def resample_batch(self, params, items, k=20, sigma_t=10.0, sigma_th=0.2, seed=1, stream=None):
        """k random perturbations per candidate as packed queries [n * k]."""
        import torch

        n = items.numel()
        q = torch.empty(n * k * QUERY_DTYPE.itemsize, dtype=torch.uint8, device=params.device)
        check(lib().jcde_resample_batch(self.h, params.data_ptr(), items.data_ptr(), n, k, sigma_t, sigma_th, seed,
                                        q.data_ptr(), _stream_handle(stream)), "resample_batch")
        return q

    # --- snapshots -----------------------------------------------------------------------------
    def save(self):
        s = C.c_void_p()
        check(lib().jcde_save(self.h, C.byref(s)), "save")
        return _Snapshot(s)

    def restore(self, snap) -> None:
        check(lib().jcde_restore(self.h, snap.h), "restore")

    # --- introspection -------------------------------------------------------------------------
    def tree_dump(self) -> np.ndarray:
        n = C.c_uint64()
        check(lib().jcde_tree_dump(self.h, None, 0, C.byref(n)), "tree_dump")
        out = np.zeros(n.value, np.uint32)
        check(lib().jcde_tree_dump(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32)), n.value, C.byref(n)), "tree_dump")
        return out

    def device_stats(self) -> dict:
        a = (C.c_uint64 * 5)()
        check(lib().jcde_device_stats(self.h, a), "device_stats")
        return dict(nodes=a[0], entries=a[1], edges=a[2], hazard_vertices=a[3], item_vertices=a[4])

    def kernel_launches(self) -> int:
        return int(lib().jcde_kernel_launches(self.h))

    TUNING_FIELDS = ("surrogate_warp_max", "leaf_table_max", "poly_chunk", "order_min_batch", "surrogate_lanes",
                     "edge_tile", "staging_depth")

    def get_tuning(self) -> dict:
        t = jcde_tuning()
        check(lib().jcde_get_tuning(self.h, C.byref(t)), "get_tuning")
        return {k: int(getattr(t, k)) for k in self.TUNING_FIELDS}

    def set_tuning(self, **fields) -> None:
        cur = self.get_tuning()
        cur.update(fields)
        t = jcde_tuning(*[int(cur[k]) for k in self.TUNING_FIELDS])
        check(lib().jcde_set_tuning(self.h, C.byref(t)), "set_tuning")

    def autotune(self, queries, filter=None, stream=None) -> tuple:
        """jcde_autotune on a CUDA batch: (chosen tuning, its median ms)."""
        f = _Filter(filter)
        n = queries.numel() * queries.element_size() // QUERY_DTYPE.itemsize
        t = jcde_tuning()
        ms = C.c_double()
        check(lib().jcde_autotune(self.h, queries.data_ptr(), n, f.ref, _stream_handle(stream), C.byref(t),
                                  C.byref(ms)), "autotune")
        return {k: int(getattr(t, k)) for k in self.TUNING_FIELDS}, float(ms.value)

    PROFILE_KINDS = ("surrogate", "poly", "collect", "order", "filter", "proxy", "update", "lbf")

    def profile(self, enable: bool = True) -> None:
        """Bracket every kernel launch with CUDA events (jcde_profile_enable)."""
        check(lib().jcde_profile_enable(self.h, int(enable)), "profile_enable")

    def profile_read(self, reset: bool = True) -> dict:
        """{kind: (total_ms, launches)} of the profiled launches since the last reset."""
        ms = (C.c_double * len(self.PROFILE_KINDS))()
        n = (C.c_uint64 * len(self.PROFILE_KINDS))()
        check(lib().jcde_profile_read(self.h, ms, n, int(reset)), "profile_read")
        return {k: (ms[i], int(n[i])) for i, k in enumerate(self.PROFILE_KINDS)}


class _Snapshot:
    def __init__(self, h):
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            try:
                lib().jcde_snapshot_free(self.h)
            except Exception:
                pass
            self.h = None


def spolygon_new(xy):
    """SPolygon::new (simple_polygon.rs:41-71): (xy_ccw, bbox, area, diameter, poi)."""
    xy = _f32(xy).reshape(-1, 2)
    xo = np.zeros_like(xy)
    bbox = np.zeros(4, np.float32)
    ad = np.zeros(2, np.float32)
    poi = np.zeros(3, np.float32)
    check(lib().jcde_spolygon_new(_fp(xy), len(xy), _fp(xo), _fp(bbox), _fp(ad), _fp(poi)), "spolygon_new")
    return xo, bbox, ad[0], ad[1], poi


def surrogate_poles(xy, area, poi, limits) -> np.ndarray:
    """generate_surrogate_poles (pole.rs:12-47) of an internal shape: (k, 3) array, [0] = poi."""
    xy, poi = _f32(xy).reshape(-1, 2), _f32(poi)
    cfg = CDEConfig(n_pole_limits=tuple(limits)).to_c()
    cap = 1024
    out = np.zeros((cap, 3), np.float32)
    n = C.c_uint32()
    check(lib().jcde_surrogate_poles(_fp(xy), len(xy), np.float32(area), _fp(poi), C.byref(cfg), _fp(out), cap,
                                     C.byref(n)), "surrogate_poles")
    return out[: n.value].copy()


class GpuEngine:
    """Adapter of CDEngine to the workload generator's engine interface."""

    def __init__(self, depth: int, cd_threshold: int, bbox):
        self.eng = CDEngine(bbox, (), CDEConfig(quadtree_depth=depth, cd_threshold=cd_threshold))

    def register_hazard(self, kind, dynamic, xy, poi, tag: int = 0) -> int:
        return self.eng.register_hazard(Hazard(kind, xy, poi, dynamic, tag))

    def deregister_hazard(self, key) -> None:
        self.eng.deregister_hazard_by_key(key)

    def add_item(self, xy, poi, poles, n_ff_poles, piers=None) -> int:
        return self.eng.register_item(xy, poi, poles, piers)

    def detect_batch(self, queries, ignored=None):
        return self.eng.detect_batch(np.ascontiguousarray(queries, dtype=QUERY_DTYPE), filter=ignored)

    def detect_with_surrogate(self, queries, ignored=None):
        """(verdicts, number of queries the surrogate pass left undecided)."""
        import torch

        q = np.ascontiguousarray(queries, dtype=QUERY_DTYPE)
        dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
        sv = self.eng.detect_batch(dq, filter=ignored, mode="surrogate").cpu().numpy()
        return self.detect_batch(q, ignored), int((sv == 0).sum())

    def tree_dump(self):
        return self.eng.tree_dump()


class GpuBackend:
    """Backend for jcde.workload: host preparation and engines from libjcde."""

    name = "gpu"
    spolygon_new = staticmethod(spolygon_new)
    surrogate_poles = staticmethod(surrogate_poles)

    @staticmethod
    def simplify_shape(xy, area, deflate, tolerance):
        """simplify_shape before its final SPolygon::new, on the device (jcde_simplify_batch)."""
        from . import prep

        return prep.simplify_batch([xy], [area], deflate, tolerance)[0]

    @staticmethod
    def close_concavities(xy, deflate, ratio):
        """close_narrow_concavities after SPolygon::new (jcde_close_concavities, host)."""
        from . import prep

        return prep.close_concavities(xy, deflate, ratio)

    @staticmethod
    def new_engine(depth: int, cd_threshold: int, bbox):
        return GpuEngine(depth, cd_threshold, bbox)


class MultiEngine:
    """Several engines (layouts) answered by one launch sequence (jcde_multi_*)."""

    def __init__(self, engines):
        self.engines = list(engines)   # keep the engines alive as long as the group
        arr = (C.c_void_p * len(self.engines))(*[e.h.value if hasattr(e.h, "value") else e.h for e in self.engines])
        h = C.c_void_p()
        check(lib().jcde_multi_create(arr, len(self.engines), C.byref(h)), "jcde_multi_create")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            try:
                lib().jcde_multi_destroy(self.h)
            except Exception:
                pass
            self.h = None

    def _filters(self, filters):
        if filters is None:
            return None, []
        fs = [_Filter(f) for f in filters]
        arr = (jcde_filter * len(fs))(*[f.c for f in fs])
        return arr, fs

    def detect(self, queries, offsets, filters=None, out=None, stream=None, graph: bool = False):
        """Verdicts of all layouts' queries; `queries` is a CUDA uint8 tensor of packed queries with
        layout l's at [offsets[l], offsets[l+1])."""
        import torch

        offs = np.ascontiguousarray(offsets, dtype=np.uint32)
        n = int(offs[-1])
        if out is None:
            out = torch.empty(n, dtype=torch.uint8, device=queries.device)
        farr, keep = self._filters(filters)
        fn = lib().jcde_multi_detect_graph if graph else lib().jcde_multi_detect
        sh = _stream_handle(stream)
        check(fn(self.h, queries.data_ptr(), offs.ctypes.data_as(C.POINTER(C.c_uint32)), farr, out.data_ptr(), sh),
              "multi_detect")
        return out

    def kernel_launches(self) -> int:
        return int(lib().jcde_multi_kernel_launches(self.h))

    def autotune(self, queries, offsets, filters=None, stream=None) -> tuple:
        """jcde_multi_autotune: ({"poly_chunk", "ordered", "edge_tile"}, median ms of the choice)."""
        import torch

        offs = np.ascontiguousarray(offsets, dtype=np.uint32)
        out = torch.empty(int(offs[-1]), dtype=torch.uint8, device=queries.device)
        farr, keep = self._filters(filters)
        o3 = (C.c_uint32 * 3)()
        ms = C.c_double()
        check(lib().jcde_multi_autotune(self.h, queries.data_ptr(), offs.ctypes.data_as(C.POINTER(C.c_uint32)), farr,
                                        out.data_ptr(), _stream_handle(stream), o3, C.byref(ms)), "multi_autotune")
        return {"poly_chunk": int(o3[0]), "ordered": bool(o3[1]), "edge_tile": int(o3[2])}, float(ms.value)



class ResidentEngine:
    """An engine's quadtree resident in device memory, updated by register / deregister kernels
    (jcde_resident_*), plus the on-device LBF-style build that runs on it (jcde_lbf_*)."""

    def __init__(self, engine: CDEngine, **capacities):
        cfg = jcde_resident_config()
        lib().jcde_resident_default_config(C.byref(cfg))
        for k, v in capacities.items():
            setattr(cfg, k, int(v))
        h = C.c_void_p()
        check(lib().jcde_resident_create(engine.h, C.byref(cfg), C.byref(h)), "resident_create")
        self.h = h
        self.engine = engine   # items and staging are shared with the engine

    def __del__(self):
        if getattr(self, "h", None):
            try:
                lib().jcde_resident_destroy(self.h)
            except Exception:
                pass
            self.h = None

    def reset(self) -> int:
        """Back to a copy of the engine's current hazards; returns the bytes uploaded."""
        n = C.c_uint64()
        check(lib().jcde_resident_reset(self.h, C.byref(n)), "resident_reset")
        return int(n.value)

    def register_placed(self, query, key_out=None, stream=None) -> None:
        """query: CUDA uint8 tensor holding one packed query; key_out: CUDA int32 tensor of 1 or None."""
        check(lib().jcde_resident_register_placed(self.h, query.data_ptr(),
                                                  None if key_out is None else key_out.data_ptr(),
                                                  _stream_handle(stream)), "resident_register_placed")

    def deregister(self, key, stream=None) -> None:
        """key: CUDA int32 tensor of 1."""
        check(lib().jcde_resident_deregister(self.h, key.data_ptr(), _stream_handle(stream)), "resident_deregister")

    def detect_batch(self, queries, out=None, stream=None):
        import torch

        n = queries.numel() // QUERY_DTYPE.itemsize
        if out is None:
            out = torch.empty(n, dtype=torch.uint8, device=queries.device)
        check(lib().jcde_resident_detect_batch(self.h, queries.data_ptr(), n, out.data_ptr(), _stream_handle(stream)),
              "resident_detect_batch")
        return out

    def status(self) -> dict:
        a = (C.c_uint32 * 8)()
        st = lib().jcde_resident_status(self.h, a)
        names = ("error", "not_found", "n_live", "n_slots", "n_nodes", "entries", "edges", "hazard_vertices")
        d = dict(zip(names, (int(x) for x in a)))
        d["status"] = int(st)
        return d

    def tree_dump(self) -> np.ndarray:
        n = C.c_uint64()
        check(lib().jcde_resident_tree_dump(self.h, None, 0, C.byref(n)), "resident_tree_dump")
        out = np.zeros(n.value, dtype=np.uint32)
        check(lib().jcde_resident_tree_dump(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32)), n.value, C.byref(n)),
              "resident_tree_dump")
        return out

    def kernel_launches(self) -> int:
        return int(lib().jcde_resident_kernel_launches(self.h))

    def lbf_begin(self, seed, n_candidates, n_types, remove_every, max_steps, sample_box, verdict_log_steps=0,
                  ls_rounds=0, ls_candidates=0, ls_sigmas=(), uniform_rounds=1, item_sequence=None,
                  orientations=None):
        """ls_sigmas: per local round (translation deviation, rotation deviation in turns);
        orientations: per engine item a float32 [k, 2] (cos, sin) table, or None for continuous rotation."""
        p = jcde_lbf_params()
        keep = []
        if item_sequence is not None:
            seq = np.ascontiguousarray(item_sequence, dtype=np.uint32)
            keep.append(seq)
            p.item_sequence = seq.ctypes.data_as(C.POINTER(C.c_uint32))
            p.n_sequence = len(seq)
        if orientations is not None:
            offs = np.zeros(len(orientations) + 1, dtype=np.uint32)
            for i, o in enumerate(orientations):
                offs[i + 1] = offs[i] + (0 if o is None else len(o))
            cs = np.concatenate([np.asarray(o, np.float32).reshape(-1, 2) for o in orientations if o is not None]
                                or [np.zeros((0, 2), np.float32)]).astype(np.float32)
            cs = np.ascontiguousarray(cs if len(cs) else np.zeros((1, 2), np.float32))
            keep += [offs, cs]
            p.n_orientation_items = len(orientations)
            p.orientation_offsets = offs.ctypes.data_as(C.POINTER(C.c_uint32))
            p.orientation_cs = cs.ctypes.data_as(C.POINTER(C.c_float))
        p.ls_rounds = int(ls_rounds)
        p.ls_candidates = int(ls_candidates)
        for k, (sg, sth) in enumerate(ls_sigmas):
            p.ls_sigma_t[k] = float(np.float32(sg))
            p.ls_sigma_turns[k] = float(sth)
        p.uniform_rounds = int(uniform_rounds)
        p.seed = int(seed)
        p.n_candidates = int(n_candidates)
        p.n_types = int(n_types)
        p.remove_every = int(remove_every)
        p.max_steps = int(max_steps)
        p.verdict_log_steps = int(verdict_log_steps)
        b = np.asarray(sample_box, dtype=np.float32)
        p.sample_box = jcde_rect(*[float(x) for x in b])
        self._lbf = p
        check(lib().jcde_lbf_begin(self.h, C.byref(p)), "lbf_begin")
        del keep   # the arrays are copied by jcde_lbf_begin

    def lbf_steps(self, n_steps, steps_per_graph=0, stream=None) -> None:
        check(lib().jcde_lbf_steps(self.h, int(n_steps), int(steps_per_graph), _stream_handle(stream)), "lbf_steps")

    def lbf_read(self) -> dict:
        p = self._lbf
        counts = np.zeros(4, dtype=np.uint32)
        u32 = C.POINTER(C.c_uint32)
        pl = np.zeros((p.max_steps, 8), dtype=np.uint32)
        rm = np.zeros((p.max_steps, 2), dtype=np.uint32)
        fc = np.zeros(p.max_steps, dtype=np.uint32)
        vl = np.zeros(max(1, p.verdict_log_steps * p.n_candidates), dtype=np.uint8)
        check(lib().jcde_lbf_read(self.h, counts.ctypes.data_as(u32), pl.ctypes.data_as(u32), p.max_steps,
                                  rm.ctypes.data_as(u32), p.max_steps, fc.ctypes.data_as(u32), p.max_steps,
                                  vl.ctypes.data, vl.size if p.verdict_log_steps else 0), "lbf_read")
        steps, n_pl, n_rm = int(counts[0]), int(counts[1]), int(counts[2])
        nv = min(steps, p.verdict_log_steps)
        return {"steps": steps, "placements": pl[:n_pl], "removals": rm[:n_rm], "free_counts": fc[:steps],
                "n_live": int(counts[3]), "verdicts": vl[: nv * p.n_candidates].reshape(nv, p.n_candidates)}


def lbf_select(eng: "GpuEngine", q, verdicts) -> int:
    """The LBF choice of a candidate batch on the device (jcde_lbf_select): index or -1."""
    import torch

    dq = torch.from_numpy(np.ascontiguousarray(q, dtype=QUERY_DTYPE).view(np.uint8).copy()).cuda()
    dv = torch.from_numpy(np.ascontiguousarray(verdicts, dtype=np.uint8)).cuda()
    best = torch.empty(1, dtype=torch.int64, device="cuda")
    check(lib().jcde_lbf_select(eng.eng.h, dq.data_ptr(), dv.data_ptr(), len(q), best.data_ptr(),
                                _stream_handle(None)), "lbf_select")
    b = int(best.item()) & 0xFFFFFFFFFFFFFFFF
    return -1 if b == 0xFFFFFFFFFFFFFFFF else int(b & 0xFFFFFFFF)



def pole_overlap(engine: CDEngine, params, items, filter=None):
    """The pole-overlap proxy P per candidate as a differentiable torch function of params [n, 3]
    (theta, tx, ty; float32, CUDA): forward is jcde_proxy_forward, backward jcde_proxy_backward."""
    import torch

    class _PoleOverlap(torch.autograd.Function):
        @staticmethod
        def forward(ctx, p):
            p = p.detach().contiguous()
            ctx.save_for_backward(p)
            return engine.proxy_forward(p, items, filter=filter)

        @staticmethod
        def backward(ctx, grad_value):
            (p,) = ctx.saved_tensors
            return engine.proxy_backward(p, items, grad_value=grad_value.contiguous().float(), filter=filter)

    return _PoleOverlap.apply(params)
