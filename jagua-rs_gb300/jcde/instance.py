"""Strip-packing instances in the reference's JSON format, imported for the engine.

The format is the strip-packing problem's external representation (probs/spp/io/ext_repr.rs with
io/ext_repr.rs): {"name", "items": [{"id", "demand", "allowed_orientations"?, "shape"}],
"strip_height"}.  Shapes are ExtShape values: "rectangle" {x_min, y_min, width, height},
"simple_polygon" [[x, y], ...], "polygon" {"outer", "inner"} (items keep the outer boundary, as
Importer::import_item does, io/import.rs:64-67); "multi_polygon" is refused like the reference does.
Items are imported by the engine's importer without shape simplification (poly_simpl_tolerance
off); allowed orientations follow io/import.rs:78-88 (absent: continuous rotation; empty or [0]:
no rotation; otherwise the listed angles in degrees).

The LBF placement order is lbf's item_placement_order (lbf/src/opt/search.rs:108-115): item types by
descending diameter, each repeated `demand` times.  An angle's (cos, sin) is evaluated by the
workload generator's float64 Taylor evaluation (sincos_turns) of angle/360 turns and rounded to
float32, so the GPU and the oracle see the same matrix.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field

import numpy as np

from . import workload as W


@dataclass
class SppItem:
    id: int
    demand: int
    orientations: list | None   # degrees; None = continuous, [] = none
    xy: np.ndarray               # raw outer boundary, float32 [n, 2]


@dataclass
class SppInstance:
    name: str
    items: list = field(default_factory=list)
    strip_height: float = 0.0


def fpa_eq32(a, b) -> bool:
    """float-cmp's approx_eq!(f32) with the default margin (util/fpa.rs): equal, within f32::EPSILON,
    or at most 4 ULPs apart."""
    a, b = np.float32(a), np.float32(b)
    if a == b or abs(float(a) - float(b)) <= float(np.finfo(np.float32).eps):
        return True
    ia, ib = int(a.view(np.int32)), int(b.view(np.int32))
    return abs(((ia - ib + 2**31) % 2**32) - 2**31) <= 4


def import_simple_polygon(data) -> np.ndarray:
    """import_simple_polygon (io/import.rs:198-211): the closing duplicate dropped, consecutive
    (approximately) equal vertices eliminated (eliminate_degenerate_vertices, io/import.rs:236-260),
    other duplicates refused."""
    pts = [(np.float32(x), np.float32(y)) for x, y in data]
    if len(pts) > 1 and pts[0] == pts[-1]:
        pts.pop()
    n = len(pts)
    drop = [i for i in range(n) if fpa_eq32(pts[i][0], pts[(i + 1) % n][0]) and fpa_eq32(pts[i][1], pts[(i + 1) % n][1])]
    for i in sorted(drop, reverse=True):
        if i < len(pts):
            pts.pop(i)
    if len(set(pts)) != len(pts):
        raise ValueError("simple polygon has non-consecutive duplicate vertices")
    return np.array(pts, dtype=np.float32).reshape(-1, 2)


def _shape_xy(shape) -> np.ndarray:
    kind, data = shape["type"], shape["data"]
    if kind == "rectangle":
        x0, y0 = np.float32(data["x_min"]), np.float32(data["y_min"])
        return W.rect_polygon(x0, y0, np.float32(x0 + np.float32(data["width"])), np.float32(y0 + np.float32(data["height"])))
    if kind == "simple_polygon":
        return import_simple_polygon(data)
    if kind == "polygon":
        return import_simple_polygon(data["outer"])
    raise ValueError(f"unsupported item shape: {kind}")


def load_spp(src) -> SppInstance:
    """A strip-packing instance from a JSON file path, a JSON string or an already parsed dict."""
    if isinstance(src, dict):
        d = src
    elif isinstance(src, str) and src.lstrip().startswith("{"):
        d = json.loads(src)
    else:
        with open(src) as f:
            d = json.load(f)
    inst = SppInstance(str(d.get("name", "")), [], float(d["strip_height"]))
    for it in d["items"]:
        ao = it.get("allowed_orientations")
        if ao is not None and (len(ao) == 0 or (len(ao) == 1 and float(ao[0]) == 0.0)):
            ao = []
        inst.items.append(SppItem(int(it["id"]), int(it.get("demand", 1)),
                                  None if ao is None else [float(a) for a in ao], _shape_xy(it["shape"])))
    return inst


def orientation_cs(degrees) -> np.ndarray:
    """(cos, sin) float32 pairs of angles given in degrees."""
    u = np.asarray(degrees, dtype=np.float64) / 360.0
    u = u - np.floor(u)
    c, s = W.sincos_turns(u)
    return np.stack([c.astype(np.float32), s.astype(np.float32)], axis=1)


def import_items(backend, raws, simplify_tolerance=None, device_prep: bool = False,
                 narrow_concavity_ratio=None) -> list:
    """workload.import_item for every shape, or with `device_prep` one jcde.prep batch (GPU)."""
    if device_prep:
        from . import prep

        return prep.import_items(raws, simplify_tolerance=simplify_tolerance,
                                 narrow_concavity_ratio=narrow_concavity_ratio)
    return [W.import_item(backend, xy, simplify_tolerance=simplify_tolerance,
                          narrow_concavity_ratio=narrow_concavity_ratio) for xy in raws]


@dataclass
class SppSetup:
    layout: W.Layout
    engine: object
    sequence: np.ndarray     # item index per LBF step (placement order, demand expanded)
    orient: list             # per item: float32 [k, 2] (cos, sin) table, or None for continuous
    width: float


def setup_spp(backend, inst: SppInstance, strip_width: float, depth: int = W.DEFAULT_DEPTH,
              cd_threshold: int = W.DEFAULT_CD_THRESHOLD, simplify_tolerance=None, device_prep: bool = False,
              narrow_concavity_ratio=None) -> SppSetup:
    """Items imported, a strip of `strip_width` x strip_height as the container, a fresh engine.
    `simplify_tolerance` simplifies the items as lbf's importer does (its default config: 0.001);
    `device_prep` imports all items in one batch with the pole searches on the GPU (jcde.prep,
    the same items)."""
    items = import_items(backend, [it.xy for it in inst.items], simplify_tolerance, device_prep, narrow_concavity_ratio)
    outer = W.import_static(backend, W.rect_polygon(0.0, 0.0, strip_width, inst.strip_height), W.EXTERIOR)
    lay = W.Layout(inst.name or "spp", depth, cd_threshold, W.inflate_to_square(W.bbox_of(outer.xy)), items=items)
    lay.hazards.append(outer)
    eng = W._new_layout_engine(backend, lay)
    # item_placement_order: descending diameter, stable on the instance order
    order = sorted(range(len(items)), key=lambda i: -float(np.float32(items[i].diameter)))
    seq = np.array([i for i in order for _ in range(inst.items[i].demand)], dtype=np.uint32)
    orient = []
    for it in inst.items:
        if it.orientations is None:
            orient.append(None)
        elif len(it.orientations) == 0:
            orient.append(orientation_cs([0.0]))
        else:
            orient.append(orientation_cs(it.orientations))
    return SppSetup(lay, eng, seq, orient, float(strip_width))


def export_solution(setup: SppSetup, inst: SppInstance, placements: np.ndarray, removals=None) -> dict:
    """The placed items as the reference's external layout (io/ext_repr.rs ExtLayout / ExtPlacedItem):
    per item its instance id and the transformation of its original shape, rotation in degrees (as
    From<DTransformation> for ExtTransformation writes it) and translation.  The internal placement
    (c, s, tx, ty) acts on the centred shape, so the original shape moves by t - R * centroid."""
    gone = set() if removals is None else {int(k) for _, k in np.asarray(removals).reshape(-1, 2)}
    placed, area = [], 0.0
    for p in np.asarray(placements).reshape(-1, 8):
        if int(p[1]) in gone:
            continue
        t = int(p[3])
        c, s, tx, ty = (float(np.uint32(v).view(np.float32)) for v in p[4:8])
        cx, cy = setup.layout.items[t].centroid
        placed.append({"item_id": inst.items[t].id,
                       "transformation": {"rotation": float(np.degrees(np.arctan2(s, c))),
                                          "translation": [tx - (c * cx - s * cy), ty - (s * cx + c * cy)]}})
        area += setup.layout.items[t].area
    return {"container_id": 0, "placed_items": placed,
            "density": float(area / (setup.width * inst.strip_height)) if placed else 0.0}
