"""Bin packing (probs/bpp) driven by the LBF optimizer of lbf/src/opt/lbf_bpp.rs on the engine.

Instances are the reference's ExtBPInstance JSON (probs/bpp/io/ext_repr.rs): items with a demand
(and an optional min_quality), bins (ExtContainer: an outer shape, holes, quality zones) with a
stock and a cost.  Import follows probs/bpp/io/import.rs (items and bins sorted by id, zero demand /
stock dropped, ids must then be 0..n-1) and io/import.rs's import_container: the outer boundary is
the Exterior hazard; holes join the quality-0 zones; every zone shape is an InferiorQualityZone
hazard, registered after the Exterior in quality order (entities/container.rs:55-69).

The optimizer (LBFOptimizerBP::solve, lbf_bpp.rs:40-79): item types in item_placement_order
(descending internal diameter, search.rs:108-115), each copy placed by `search_layouts`
(lbf_bpp.rs:98-140): the open layouts in the order they were opened, then every bin with stock
left, and the first layout where the search finds a collision-free candidate takes the item (a
closed bin opens a new layout); when no layout fits a copy, the remaining copies of that type are
skipped.  Items with a min_quality see the quality zones through
HazKeyFilter::from_irrelevant_qzones (hazards/filter.rs:21-41), which deems irrelevant the zones
whose quality is below the item's min_quality (the code's condition; its doc comment words it the
other way round).

The search in each layout is this package's LBF round (jcde.lbf): candidates from a seeded stream
over the bin's bounding box, the free one of least LBFLoss cost, then optional local-search rounds.
Every layout of a search draws its own stream (keyed by attempt and layout), so evaluating all
of them at once — one jcde_multi launch sequence over the open layouts and the unopened bins on
the GPU — chooses exactly what the sequential search of the reference's loop would.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field

import numpy as np

from . import instance as I
from . import lbf
from . import workload as W

BPP_SID_BASE = 2_000_000   # attempt a, layout slot s: stream BPP_SID_BASE + 4096 a + s
CLOSED_SLOT = 2048         # slot of an unopened bin b: CLOSED_SLOT + b
BPP_LS_STEP = 10_000_000   # local-search rounds of attempt a use lbf's streams of step BPP_LS_STEP + a


@dataclass
class BppItem:
    id: int
    demand: int
    orientations: list | None   # degrees; None = continuous, [] = none
    xy: np.ndarray
    min_quality: int | None = None


@dataclass
class BppBin:
    id: int
    stock: int
    cost: int
    outer: np.ndarray
    zones: list = field(default_factory=list)   # [(quality, xy)]; holes are quality-0 zones


@dataclass
class BppInstance:
    name: str
    items: list
    bins: list


def _orientations(it):
    ao = it.get("allowed_orientations")
    if ao is not None and (len(ao) == 0 or (len(ao) == 1 and float(ao[0]) == 0.0)):
        return []
    return None if ao is None else [float(a) for a in ao]


def _zone_xy(shape):
    if shape["type"] == "polygon":
        raise ValueError("quality zones of polygon shape are not supported (as in io/import.rs:156-158)")
    return I._shape_xy(shape)


def load_bpp(src) -> BppInstance:
    """A bin-packing instance from a JSON file path, a JSON string or an already parsed dict."""
    if isinstance(src, dict):
        d = src
    elif isinstance(src, str) and src.lstrip().startswith("{"):
        d = json.loads(src)
    else:
        with open(src) as f:
            d = json.load(f)
    items = [BppItem(int(it["id"]), int(it["demand"]), _orientations(it), I._shape_xy(it["shape"]),
                     None if it.get("min_quality") is None else int(it["min_quality"])) for it in d["items"]]
    items.sort(key=lambda it: it.id)
    items = [it for it in items if it.demand > 0]
    if [it.id for it in items] != list(range(len(items))) or not items:
        raise ValueError("items with positive demand must have ids 0..n-1 (probs/bpp/io/import.rs:25-34)")
    bins = []
    for b in d["bins"]:
        shape = b["shape"]
        if shape["type"] == "polygon":
            outer = I.import_simple_polygon(shape["data"]["outer"])
            holes = [I.import_simple_polygon(h) for h in shape["data"].get("inner", [])]
        else:
            outer, holes = I._shape_xy(shape), []
        by_q = {}
        for z in b.get("zones", []):
            by_q.setdefault(int(z["quality"]), []).append(_zone_xy(z["shape"]))
        by_q.setdefault(0, []).extend(holes)   # holes join the quality-0 zones (io/import.rs:168-169)
        zones = [(q, xy) for q in sorted(by_q) for xy in by_q[q]]
        bins.append(BppBin(int(b["id"]), int(b["stock"]), int(b["cost"]), outer, zones))
    bins.sort(key=lambda b: b.id)
    bins = [b for b in bins if b.stock > 0]
    if [b.id for b in bins] != list(range(len(bins))) or not bins:
        raise ValueError("bins with positive stock must have ids 0..n-1 (probs/bpp/io/import.rs:47-56)")
    return BppInstance(str(d.get("name", "")), items, bins)


def synthetic_instance(seed: int = 0xB1, n_types: int = 30, v_range=(8, 60), r_range=(20.0, 60.0),
                       demand_range=(1, 5), n_bins: int = 4) -> dict:
    """A seeded bin-packing instance in the reference's JSON format: star items (every fifth needs
    quality 1, every seventh turns by multiples of 90 degrees only) and bins that are rectangles or
    rectangle polygons with rectangular holes, with quality-1 and quality-2 star zones."""
    st = W.Stream(seed, 1)
    items = []
    for i in range(n_types):
        nv = int(st.randint(v_range[0], v_range[1], 1)[0])
        xy = W.star_polygon(st, nv, *r_range)
        it = {"id": i, "demand": int(st.randint(demand_range[0], demand_range[1], 1)[0]),
              "shape": {"type": "simple_polygon", "data": xy.astype(float).tolist()}}
        if i % 5 == 4:
            it["min_quality"] = 1
        if i % 7 == 6:
            it["allowed_orientations"] = [0.0, 90.0, 180.0, 270.0]
        items.append(it)
    bins = []
    for b in range(n_bins):
        w = float(np.float32(600 + 200 * b))
        h = float(np.float32(500 + 100 * (b % 2)))
        zones = []
        for q in (1, 2):
            cx, cy = float(w * (0.3 + 0.4 * (q - 1))), float(h * 0.5)
            zones.append({"quality": q, "shape": {"type": "simple_polygon", "data":
                          W.star_polygon(st, 12, 40.0, 70.0, center=(cx, cy)).astype(float).tolist()}})
        if b % 2 == 0:
            shape = {"type": "rectangle", "data": {"x_min": 0.0, "y_min": 0.0, "width": w, "height": h}}
        else:
            holes = [W.rect_polygon(w * 0.45, h * 0.1, w * 0.45 + 60.0, h * 0.1 + 40.0).astype(float).tolist()]
            shape = {"type": "polygon", "data": {"outer": W.rect_polygon(0.0, 0.0, w, h).astype(float).tolist(),
                                                 "inner": holes}}
        bins.append({"id": b, "stock": 1 + b % 3, "cost": int(w * h // 1000), "shape": shape, "zones": zones})
    return {"name": f"bpp-synthetic-{seed:x}", "items": items, "bins": bins}


@dataclass
class BinSetup:
    hazards: list         # HazardSpec: the Exterior, then the zones in quality order
    qualities: list       # per hazard: None (Exterior) or the zone's quality
    cde_bbox: np.ndarray
    box: np.ndarray       # the sampling box: the outer shape's bounding box
    area: float           # Container::area: outer minus the quality-0 zones (container.rs:82-84)


@dataclass
class BppSetup:
    instance: BppInstance
    items: list            # W.Item per instance item
    bins: list             # BinSetup per bin
    order: list            # item ids in placement order
    orient: list           # per item: float32 (cos, sin) table or None
    depth: int
    cd_threshold: int


def setup_bpp(backend, inst: BppInstance, simplify_tolerance=None, depth: int = W.DEFAULT_DEPTH,
              cd_threshold: int = W.DEFAULT_CD_THRESHOLD, device_prep: bool = False,
              narrow_concavity_ratio=None) -> BppSetup:
    """Items and bins imported (see the module notes); `device_prep` imports the items in one
    jcde.prep batch with the pole searches on the GPU (the same items)."""
    items = I.import_items(backend, [it.xy for it in inst.items], simplify_tolerance, device_prep,
                           narrow_concavity_ratio)
    bins = []
    for b in inst.bins:
        outer = W.import_static(backend, b.outer, W.EXTERIOR, simplify_tolerance, narrow_concavity_ratio)
        hz, qs = [outer], [None]
        q0_area = 0.0
        for q, xy in b.zones:
            hz.append(W.import_static(backend, xy, W.QUALITY_ZONE, simplify_tolerance, narrow_concavity_ratio))
            qs.append(q)
            if q == 0:
                q0_area += float(backend.spolygon_new(xy)[2])
        bins.append(BinSetup(hz, qs, W.inflate_to_square(W.bbox_of(outer.xy)), W.bbox_of(outer.xy),
                             float(backend.spolygon_new(b.outer)[2]) - q0_area))
    order = sorted(range(len(items)), key=lambda i: -float(np.float32(items[i].diameter)))
    orient = []
    for it in inst.items:
        if it.orientations is None:
            orient.append(None)
        elif len(it.orientations) == 0:
            orient.append(I.orientation_cs([0.0]))
        else:
            orient.append(I.orientation_cs(it.orientations))
    return BppSetup(inst, items, bins, order, orient, depth, cd_threshold)


def _bin_engine(backend, su: BppSetup, b: int):
    """A fresh engine of bin b: the Container's base CDE (entities/container.rs:55-69)."""
    bs = su.bins[b]
    eng = backend.new_engine(su.depth, su.cd_threshold, bs.cde_bbox)
    for it in su.items:
        eng.add_item(it.xy, it.poi, it.poles, it.n_ff_poles)
    keys = [eng.register_hazard(hz.kind, hz.dynamic, hz.xy, hz.poi, i + 1) for i, hz in enumerate(bs.hazards)]
    return eng, keys


def quality_filter(bs: BinSetup, keys: list, min_quality) -> list | None:
    """HazKeyFilter::from_irrelevant_qzones (hazards/filter.rs:21-41) for an item's min_quality:
    the keys of the zones whose quality is below it; None (NoFilter) without a min_quality."""
    if min_quality is None:
        return None
    return [k for k, q in zip(keys, bs.qualities) if q is not None and q < min_quality]


@dataclass
class BppSpec:
    seed: int = 0xB1
    n_cand: int = 4096
    ls_rounds: int = 0   # local-search rounds after a layout's uniform round (lbf's deviations)
    ls_cand: int = 0


@dataclass
class Layout:
    bin: int
    engine: object
    keys: list                                    # the bin's hazard keys (Exterior, zones)
    placed: list = field(default_factory=list)    # (item, cos, sin, tx, ty) float32


@dataclass
class BppLog:
    placements: np.ndarray   # (n, 9) uint32: attempt, layout, bin, item, candidate, cos, sin, tx, ty (f32 bits)
    layouts: list            # bin id per opened layout, in opening order
    unplaced: dict           # item id -> copies left when no layout fitted
    layout_objs: list = field(default_factory=list)   # the opened Layouts (engines and placed items)
    judged: int = 0          # candidates judged (all layouts of a batched search, else up to the chosen one)

    def same_as(self, other: "BppLog") -> bool:
        return (np.array_equal(self.placements, other.placements) and self.layouts == other.layouts
                and self.unplaced == other.unplaced)


def _round(spec: BppSpec, attempt: int, slot: int, t: int, box, orient):
    """The uniform round of one layout's search: lbf's round over the bin's box with this layout's stream."""
    q = W.make_queries(W.Stream(spec.seed, BPP_SID_BASE + 4096 * attempt + slot), spec.n_cand, 1, box)
    st = W.Stream(spec.seed, BPP_SID_BASE + 4096 * attempt + slot)
    st.pos = spec.n_cand
    if orient is None:
        u = st.f64(spec.n_cand)
    else:
        k = (st.u64(spec.n_cand) % np.uint64(len(orient))).astype(np.int64)
        q["cos"] = orient[k, 0]
        q["sin"] = orient[k, 1]
        u = np.zeros(spec.n_cand)
    q["item"] = t
    return q, u


def _local_search(spec: BppSpec, su: BppSetup, eng, filt, attempt: int, t: int, rec, box):
    """lbf's local-search rounds around a layout's best (strict improvement), on that layout's engine;
    the deviations scale with the bin's CDE box (its box inflated to a square)."""
    box = np.asarray(box, dtype=np.float64)
    ls = lbf.LbfSpec(seed=spec.seed, ls_rounds=spec.ls_rounds, ls_cand=spec.ls_cand, orient=su.orient,
                     ls_max_dim=max(box[2] - box[0], box[3] - box[1]))
    for r, (sg, sth) in enumerate(ls.ls_sigmas(), start=1):
        # the rounds of attempt a draw lbf's local-search streams of step BPP_LS_STEP + a
        ql, ul = lbf._local_round(ls, BPP_LS_STEP + attempt, r, t, rec[1], rec[2], sg, sth)
        vl = eng.detect_batch(ql, filt)
        b, cb = lbf.select_host_cost(su.items, ql, vl)
        if b >= 0 and cb < rec[0]:
            rec = (cb, float(ul[b]), ql[b].copy(), (r << 24) | b)
    return rec


def run_bpp(backend, su: BppSetup, spec: BppSpec, batched: bool = True) -> BppLog:
    """LBFOptimizerBP::solve.  With the GPU backend and `batched`, every search evaluates all of its
    layouts in one jcde_multi launch sequence; otherwise layout by layout, as the reference does."""
    use_multi = batched and getattr(backend, "name", "") == "gpu"
    stock = [b.stock for b in su.instance.bins]
    demand = [it.demand for it in su.instance.items]
    base = [_bin_engine(backend, su, b) for b in range(len(su.bins))]   # the bins' unopened CDEs
    layouts: list[Layout] = []
    placements, unplaced = [], {}
    attempt = 0
    judged = 0
    gpu = _GpuSearch(su, spec) if use_multi else None
    for t in su.order:
        while demand[t] > 0:
            # search_layouts (lbf_bpp.rs:98-140): open layouts, then bins with stock
            slots = [(li, layouts[li].engine, layouts[li].keys, layouts[li].bin) for li in range(len(layouts))]
            slots += [(CLOSED_SLOT + b, base[b][0], base[b][1], b) for b in range(len(su.bins)) if stock[b] > 0]
            mq = su.instance.items[t].min_quality
            filts = [quality_filter(su.bins[b], keys, mq) for _, _, keys, b in slots]
            found = None
            if use_multi and slots:
                found = gpu.search(su, spec, slots, filts, attempt, t)
                judged += len(slots) * spec.n_cand
            else:
                for j, (s, eng, keys, b) in enumerate(slots):
                    q, u = _round(spec, attempt, s, t, su.bins[b].box, su.orient[t])
                    v = eng.detect_batch(q, filts[j])
                    judged += len(q)
                    best, cost = lbf.select_host_cost(su.items, q, v)
                    if best >= 0:
                        found = (j, (cost, float(u[best]), q[best].copy(), best))
                        break
            if found is None:
                unplaced[su.instance.items[t].id] = demand[t]   # this type fits nowhere (lbf_bpp.rs:70)
                break
            j, rec = found
            s, eng, keys, b = slots[j]
            if spec.ls_rounds:
                rec = _local_search(spec, su, eng, filts[j], attempt, t, rec, su.bins[b].box)
                judged += spec.ls_rounds * spec.ls_cand
            if s >= CLOSED_SLOT:   # BPProblem::place_item opens a new layout (problem.rs:44-66)
                eng, keys = _bin_engine(backend, su, b)
                layouts.append(Layout(b, eng, keys))
                stock[b] -= 1
                li = len(layouts) - 1
            else:
                li = s
            r_q = rec[2]
            hz = W.placed_hazard(su.items[t], t, r_q["cos"], r_q["sin"], r_q["tx"], r_q["ty"])
            layouts[li].engine.register_hazard(hz.kind, hz.dynamic, hz.xy, hz.poi, 1_000_000 + attempt)
            layouts[li].placed.append((t, r_q["cos"], r_q["sin"], r_q["tx"], r_q["ty"]))
            placements.append([attempt, li, b, t, rec[3]] +
                              [int(np.float32(r_q[f]).view(np.uint32)) for f in ("cos", "sin", "tx", "ty")])
            demand[t] -= 1
            attempt += 1
    return BppLog(np.array(placements, dtype=np.uint32).reshape(-1, 9), [l.bin for l in layouts], unplaced, layouts,
                  judged)


class _GpuSearch:
    """One search over several layouts on the GPU: every layout's uniform round drawn on the device
    (jcde_gen_candidates, the same stream as the host round), all judged by one jcde_multi launch
    sequence, each layout's LBF choice made on the device (jcde_lbf_select); the host reads one
    64-bit result per layout and the chosen candidate."""

    def __init__(self, su: BppSetup, spec: BppSpec):
        import torch

        n_slots = len(su.bins) + sum(b.stock for b in su.instance.bins)
        self.n = spec.n_cand
        self.dq = torch.empty(n_slots * self.n * W.QUERY_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        self.du = torch.empty(n_slots * self.n, dtype=torch.float64, device="cuda")
        self.best = torch.empty(n_slots, dtype=torch.int64, device="cuda")
        self.dv = torch.empty(n_slots * self.n, dtype=torch.uint8, device="cuda")
        self.orient = [None if o is None else torch.from_numpy(np.ascontiguousarray(o, np.float32)).cuda()
                       for o in su.orient]
        self.multi = {}

    def _group(self, engines):
        from .engine import MultiEngine

        key = tuple(id(e) for e in engines)
        m = self.multi.get(key)
        if m is None:
            self.multi.clear()   # the set of layouts changed (a bin was opened): regroup
            m = self.multi[key] = MultiEngine(engines)
        return m

    def search(self, su: BppSetup, spec: BppSpec, slots, filts, attempt: int, t: int):
        import ctypes as C

        from ._ffi import check, jcde_rect, lib
        from .engine import _stream_handle

        L, n, qs = len(slots), self.n, W.QUERY_DTYPE.itemsize
        sh = _stream_handle(None)
        o = self.orient[t]
        sids = (C.c_uint64 * L)(*[BPP_SID_BASE + 4096 * attempt + slot for slot, _, _, _ in slots])
        rects = (jcde_rect * L)(*[jcde_rect(*[float(x) for x in su.bins[b].box]) for _, _, _, b in slots])
        check(lib().jcde_gen_candidates_segments(spec.seed, sids, rects, L, n, t, None if o is None else o.data_ptr(),
                                                 0 if o is None else len(o), self.dq.data_ptr(), self.du.data_ptr(),
                                                 sh), "gen_candidates_segments")
        cdes = [e.eng for _, e, _, _ in slots]
        offs = np.arange(L + 1, dtype=np.uint32) * np.uint32(n)
        self._group(cdes).detect(self.dq[: L * n * qs], offs, filters=[list(f) if f else [] for f in filts],
                                 out=self.dv[: L * n])
        # every engine holds the same items: one of them serves the choice of all segments
        check(lib().jcde_lbf_select_segments(cdes[0].h, self.dq.data_ptr(), self.dv.data_ptr(), n, L,
                                             self.best.data_ptr(), sh), "lbf_select_segments")
        best = self.best[:L].cpu().numpy().view(np.uint64)
        for j in range(L):
            if best[j] != np.uint64(0xFFFFFFFFFFFFFFFF):
                i = int(best[j] & np.uint64(0xFFFFFFFF))
                row = self.dq[(j * n + i) * qs: (j * n + i + 1) * qs].cpu().numpy().view(W.QUERY_DTYPE)[0].copy()
                u = float(self.du[j * n + i].item())
                xy = W.transform_points(su.items[t].xy, row["cos"], row["sin"], row["tx"], row["ty"])
                return j, (lbf.lbf_cost(xy), u, row, i)
        return None


def export_solution(su: BppSetup, log: BppLog) -> dict:
    """ExtBPSolution (probs/bpp/io/ext_repr.rs:34-47): cost, the layouts as ExtLayout with their
    placed items (rotation in degrees as the reference's ExtTransformation conversion writes it),
    and the density (item area over container area, solution.rs:17-31)."""
    lays, tot_items, tot_bins, cost = [], 0.0, 0.0, 0
    for lay in log.layout_objs:
        placed, a = [], 0.0
        for t, c, s, tx, ty in lay.placed:
            c, s, tx, ty = float(c), float(s), float(tx), float(ty)
            cx, cy = su.items[t].centroid
            placed.append({"item_id": su.instance.items[t].id,
                           "transformation": {"rotation": float(np.degrees(np.arctan2(s, c))),
                                              "translation": [tx - (c * cx - s * cy), ty - (s * cx + c * cy)]}})
            a += su.items[t].area
        area = su.bins[lay.bin].area
        lays.append({"container_id": su.instance.bins[lay.bin].id, "placed_items": placed,
                     "density": a / area if area else 0.0})
        tot_items += a
        tot_bins += area
        cost += su.instance.bins[lay.bin].cost
    return {"cost": cost, "layouts": lays, "density": tot_items / tot_bins if tot_bins else 0.0, "run_time_sec": 0}
