"""Shape preparation on the device: the poles of many shapes per launch.

The reference prepares every item with Item::new (entities/item.rs:27-48): SPolygon::new, whose
pole of inaccessibility is compute_pole without earlier poles (simple_polygon.rs:152-171), then
generate_surrogate_poles (fail_fast/pole.rs:12-47), one shape at a time on the host.  Here the cheap
parts of SPolygon::new (orientation, area, diameter) stay on the host and both pole searches run as
one kernel launch per batch (jcde_poi_batch, jcde_surrogate_poles_batch), each shape's poles bit for
bit those of the host preparation.  `import_items` is Importer::import_item (io/import.rs:47-98,
without simplification) for a whole list of shapes.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import workload as W
from ._ffi import JcdeError, check, lib
from .engine import CDEConfig

STATUS = {1: "invalid shape", 2: "no pole found", 3: "a thousand poles reached", 4: "cell-tree level too wide",
          5: "more poles than the output holds"}


def _torch():
    import torch

    return torch


def _stream_ptr(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def pack(shapes):
    """Shapes back to back: ((V, 2) float32 vertices, (n + 1,) uint32 offsets)."""
    xy = [np.ascontiguousarray(s, np.float32).reshape(-1, 2) for s in shapes]
    off = np.zeros(len(xy) + 1, np.uint32)
    off[1:] = np.cumsum([len(s) for s in xy])
    return (np.concatenate(xy) if xy else np.zeros((0, 2), np.float32)), off


class ShapeBatch:
    """Shapes packed for the device: every shape's (x, y) vertices back to back and their offsets,
    plus the workspaces of the two pole searches (kept for repeated calls)."""

    def __init__(self, shapes=None, device="cuda", packed=None):
        torch = _torch()
        if packed is None:
            flat, off = pack(shapes)
        else:
            flat, off = packed
        self.n = len(off) - 1
        self.vmax = max(int(np.diff(off).max()) if self.n else 3, 3)
        self.xy = torch.from_numpy(np.ascontiguousarray(flat, np.float32).reshape(-1)).to(device)
        self.voff = torch.from_numpy(np.ascontiguousarray(off, np.uint32).view(np.int32)).to(device)
        self.device = self.xy.device
        # larger shapes first (descending vertex count, stable): the last shapes a batch hands out
        # are small, so CTAs finish together
        order = np.argsort(-np.diff(np.asarray(off, np.int64)), kind="stable").astype(np.uint32)
        self.order = torch.from_numpy(order.view(np.int32)).to(device)
        self._ws = {}

    def workspace(self, with_poles: bool):
        torch = _torch()
        key = bool(with_poles)
        if key not in self._ws:
            nb = int(lib().jcde_poles_workspace_bytes(self.n, self.vmax, int(key))) if self.n else 0
            self._ws[key] = torch.empty(max(nb, 1), dtype=torch.uint8, device=self.device)
        return self._ws[key]

    def poi(self, out=None, status=None, stream=None):
        """Launch jcde_poi_batch: (n, 3) float32 poi and (n,) int32 status device tensors."""
        torch = _torch()
        out = torch.empty((self.n, 3), dtype=torch.float32, device=self.device) if out is None else out
        status = torch.empty(self.n, dtype=torch.int32, device=self.device) if status is None else status
        ws = self.workspace(False)
        check(lib().jcde_poi_batch(C.c_void_p(self.xy.data_ptr()), C.c_void_p(self.voff.data_ptr()), self.n,
                                   self.vmax, C.c_void_p(out.data_ptr()), C.c_void_p(status.data_ptr()),
                                   C.c_void_p(self.order.data_ptr()), C.c_void_p(ws.data_ptr()), ws.numel(),
                                   _stream_ptr(stream)), "poi_batch")
        return out, status

    def poles(self, area, poi, limits=W.DEFAULT_POLE_LIMITS, cap=128, out=None, counts=None, status=None,
              stream=None):
        """Launch jcde_surrogate_poles_batch: area (n,) and poi (n, 3) float32 device tensors in;
        (n, cap, 3) poles, (n,) counts and (n,) status device tensors out."""
        torch = _torch()
        cfg = CDEConfig(n_pole_limits=tuple(limits)).to_c()
        out = torch.empty((self.n, cap, 3), dtype=torch.float32, device=self.device) if out is None else out
        counts = torch.empty(self.n, dtype=torch.int32, device=self.device) if counts is None else counts
        status = torch.empty(self.n, dtype=torch.int32, device=self.device) if status is None else status
        ws = self.workspace(True)
        check(lib().jcde_surrogate_poles_batch(C.c_void_p(self.xy.data_ptr()), C.c_void_p(self.voff.data_ptr()),
                                               self.n, self.vmax, C.c_void_p(area.data_ptr()),
                                               C.c_void_p(poi.data_ptr()), C.byref(cfg), C.c_void_p(out.data_ptr()),
                                               cap, C.c_void_p(counts.data_ptr()), C.c_void_p(status.data_ptr()),
                                               C.c_void_p(self.order.data_ptr()), C.c_void_p(ws.data_ptr()),
                                               ws.numel(), _stream_ptr(stream)),
              "surrogate_poles_batch")
        return out, counts, status


def simplify_device(batch: "ShapeBatch", area, deflate: bool, tolerance: float, stream=None):
    """Launch jcde_simplify_batch on a packed batch: area (n,) float32 device tensor in; the
    simplified vertices (same layout as the batch), counts and statuses as device tensors out."""
    torch = _torch()
    out = torch.empty_like(batch.xy)
    cnt = torch.empty(batch.n, dtype=torch.int32, device=batch.device)
    st = torch.empty(batch.n, dtype=torch.int32, device=batch.device)
    check(lib().jcde_simplify_batch(C.c_void_p(batch.xy.data_ptr()), C.c_void_p(batch.voff.data_ptr()), batch.n,
                                    batch.vmax, C.c_void_p(area.data_ptr()), int(bool(deflate)), float(tolerance),
                                    C.c_void_p(out.data_ptr()), C.c_void_p(cnt.data_ptr()), C.c_void_p(st.data_ptr()),
                                    _stream_ptr(stream)), "simplify_batch")
    return out, cnt, st


def simplify_batch(shapes, areas, deflate: bool, tolerance: float) -> list:
    """simplify_shape (shape_modification.rs:48-144, before its final SPolygon::new) of each internal
    shape on the device: a list of (k, 2) float32 vertex arrays."""
    torch = _torch()
    if not len(shapes):
        return []
    flat, off = pack(shapes)
    b = ShapeBatch(packed=(flat, off))
    area = torch.from_numpy(np.ascontiguousarray(areas, np.float32)).to(b.device)
    out, cnt, st = simplify_device(b, area, deflate, tolerance)
    _raise_on(st.cpu().numpy(), "simplify_batch")
    o, c = out.view(-1, 2).cpu().numpy(), cnt.cpu().numpy()
    return [o[off[i]: off[i] + int(c[i])].copy() for i in range(b.n)]


def close_concavities(xy, deflate: bool, ratio: float) -> np.ndarray:
    """close_narrow_concavities (shape_modification.rs:374-478) of one shape, on the host
    (jcde_close_concavities): a pairwise search over the shape's vertices, run between two
    simplification passes."""
    xy = np.ascontiguousarray(xy, np.float32).reshape(-1, 2)
    out = np.zeros_like(xy)
    n = np.zeros(1, np.uint32)
    f32p = C.POINTER(C.c_float)
    check(lib().jcde_close_concavities(xy.ctypes.data_as(f32p), len(xy), int(bool(deflate)), float(np.float32(ratio)),
                                       out.ctypes.data_as(f32p), n.ctypes.data_as(C.POINTER(C.c_uint32))),
          "close_concavities")
    return out[: int(n[0])].copy()


def _raise_on(status: np.ndarray, what: str, allow=()):
    bad = [(i, int(s)) for i, s in enumerate(status) if s != 0 and s not in allow]
    if bad:
        i, s = bad[0]
        raise JcdeError(-1, f"{what}: shape {i}: {STATUS.get(s, s)} ({len(bad)} shapes failed)")


def poi_batch(shapes) -> np.ndarray:
    """The pole of inaccessibility of each internal (counter-clockwise) shape, computed on the device."""
    if not len(shapes):
        return np.zeros((0, 3), np.float32)
    b = ShapeBatch(shapes)
    poi, st = b.poi()
    _raise_on(st.cpu().numpy(), "poi_batch")
    return poi.cpu().numpy()


def surrogate_poles_batch(shapes, areas, pois, limits=W.DEFAULT_POLE_LIMITS, cap=128) -> list:
    """generate_surrogate_poles of each internal shape on the device: a list of (k, 3) arrays, [0] = poi."""
    torch = _torch()
    if not len(shapes):
        return []
    b = ShapeBatch(shapes)
    area = torch.from_numpy(np.ascontiguousarray(areas, np.float32)).to(b.device)
    poi = torch.from_numpy(np.ascontiguousarray(pois, np.float32).reshape(-1, 3)).to(b.device)
    out, cnt, st = b.poles(area, poi, limits, cap)
    st_h = st.cpu().numpy()
    if (st_h == 5).any():   # more poles than `cap`: once more with room for the bound of 1000
        out, cnt, st = b.poles(area, poi, limits, 1000)
        st_h = st.cpu().numpy()
    _raise_on(st_h, "surrogate_poles_batch")
    o, c = out.cpu().numpy(), cnt.cpu().numpy()
    return [o[i, : int(c[i])].copy() for i in range(b.n)]


def spolygon_shape(raw_xy):
    """SPolygon::new without its poi (simple_polygon.rs:41-71): (xy_ccw, bbox, area, diameter)."""
    xy = np.ascontiguousarray(raw_xy, np.float32).reshape(-1, 2)
    xo = np.zeros_like(xy)
    bbox = np.zeros(4, np.float32)
    ad = np.zeros(2, np.float32)
    f32p = C.POINTER(C.c_float)
    check(lib().jcde_spolygon_new(xy.ctypes.data_as(f32p), len(xy), xo.ctypes.data_as(f32p),
                                  bbox.ctypes.data_as(f32p), ad.ctypes.data_as(f32p), None), "spolygon_new")
    return xo, bbox, ad[0], ad[1]


def spolygon_batch(raw_shapes, n_threads: int = 0, centroids: bool = False):
    """spolygon_shape of every shape in one call (host threads): packed internal vertices and
    offsets, (n, 4) bboxes, (n, 2) area / diameter, and with `centroids` the (n, 2) centroids
    (SPolygon::centroid, the same float32 sums as workload.centroid_f32)."""
    flat, off = pack(raw_shapes)
    n = len(off) - 1
    xo = np.empty_like(flat)
    bbox = np.empty((n, 4), np.float32)
    ad = np.empty((n, 2), np.float32)
    cen = np.empty((n, 2), np.float32) if centroids else None
    st = np.empty(n, np.int32)
    f32p, u32p = C.POINTER(C.c_float), C.POINTER(C.c_uint32)
    check(lib().jcde_spolygon_batch(flat.ctypes.data_as(f32p), off.ctypes.data_as(u32p), n, xo.ctypes.data_as(f32p),
                                    bbox.ctypes.data_as(f32p), ad.ctypes.data_as(f32p),
                                    None if cen is None else C.c_void_p(cen.ctypes.data), C.c_void_p(st.ctypes.data),
                                    n_threads), "spolygon_batch")
    if (st != 0).any():
        raise JcdeError(-1, f"spolygon_batch: shape {int(np.flatnonzero(st)[0])} is not a valid simple polygon")
    return (xo, off, bbox, ad, cen) if centroids else (xo, off, bbox, ad)


def import_items(raw_shapes, pole_limits=W.DEFAULT_POLE_LIMITS, n_ff_poles=W.DEFAULT_N_FF_POLES,
                 simplify_tolerance=None, narrow_concavity_ratio=None) -> list:
    """Importer::import_item (io/import.rs:47-98) for every shape of the list, the poi and surrogate
    poles searched on the device: the same Items as workload.import_item.  With a
    `simplify_tolerance` the centred shapes are simplified on the device (ShapeModifyMode::Inflate,
    original_shape.rs:23-50), with `narrow_concavity_ratio` their narrow concavities are then closed
    (host) and the shapes simplified again at a tenth of the tolerance, and the poi is that of the
    final shape."""
    torch = _torch()
    n = len(raw_shapes)
    if n == 0:
        return []
    flat, off, _, ad, cent = spolygon_batch(raw_shapes, centroids=True)
    if simplify_tolerance is None:
        b = ShapeBatch(packed=(flat, off))
        poi_d, st = b.poi()
    # centering_transformation (io/import.rs:214-217) as in workload.import_item, every shape at once
    reps = np.diff(off).astype(np.int64)
    cxy = W.transform_points(flat, 1.0, 0.0, np.repeat(-cent[:, 0], reps), np.repeat(-cent[:, 1], reps))
    area_int = ad[:, 0]
    diam_int = ad[:, 1]
    if simplify_tolerance is None:
        _raise_on(st.cpu().numpy(), "poi_batch")
        poi = poi_d.cpu().numpy()
        ipoi = np.concatenate([W.transform_points(poi[:, :2], 1.0, 0.0, -cent[:, 0], -cent[:, 1]), poi[:, 2:3]],
                              axis=1).astype(np.float32)
        bc = ShapeBatch(packed=(cxy, off))
    else:
        # simplify_shape, then its SPolygon::new: orientation, area, diameter on the host, poi on the device
        simp = simplify_batch([cxy[off[i]: off[i + 1]] for i in range(n)], area_int, False, simplify_tolerance)
        if narrow_concavity_ratio is not None:
            # close_narrow_concavities (host), then simplify_shape at a tenth of the tolerance
            closed = [close_concavities(s_, False, narrow_concavity_ratio) for s_ in simp]
            cflat, coff, _, cad = spolygon_batch(closed)
            simp = simplify_batch([cflat[coff[i]: coff[i + 1]] for i in range(n)], cad[:, 0], False,
                                  float(np.float32(simplify_tolerance) / np.float32(10.0)))
        cxy, off, _, ad2 = spolygon_batch(simp)
        area_int, diam_int = ad2[:, 0], ad2[:, 1]
        bc = ShapeBatch(packed=(cxy, off))
        poi_d, st = bc.poi()
        _raise_on(st.cpu().numpy(), "poi_batch")
        ipoi = poi_d.cpu().numpy()
    area_d = torch.from_numpy(np.ascontiguousarray(area_int, np.float32)).to(bc.device)
    cap = 128
    out, cnt, sp = bc.poles(area_d, torch.from_numpy(ipoi).to(bc.device), pole_limits, cap)
    sp_h = sp.cpu().numpy()
    if (sp_h == 5).any():   # more poles than `cap`: once more with room for the bound of 1000
        cap = 1000
        out, cnt, sp = bc.poles(area_d, torch.from_numpy(ipoi).to(bc.device), pole_limits, cap)
        sp_h = sp.cpu().numpy()
    _raise_on(sp_h, "surrogate_poles_batch")
    o, c = out.cpu().numpy(), cnt.cpu().numpy()
    items = []
    for i in range(n):
        p = o[i, : int(c[i])].copy()
        items.append(W.Item(cxy[off[i]: off[i + 1]].copy(), ipoi[i].copy(), p, min(n_ff_poles, len(p)),
                            float(ad[i, 0]), float(diam_int[i]), (float(cent[i, 0]), float(cent[i, 1]))))
    return items
