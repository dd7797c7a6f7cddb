"""Seeded synthetic layouts and query batches for the CDE query path.

The reference benchmarks its CDE on a nested instance (lbf/benches/ci_bench.rs:79-126): a dense
layout, then uniform (item, rotation, translation) samples over the CDE's bounding box, each
checked with ``detect_surrogate_collision`` then ``detect_poly_collision``.  The generators here
build layouts of the same kind from star-shaped polygons, so that no dataset is needed:

* every random number comes from a counter-based SplitMix64 stream (bit-identical on x86 and Arm);
* rotations are given as ``(cos, sin)`` pairs computed by a fixed Taylor polynomial in float64 and
  rounded once to float32, so no libm routine decides a single bit of the workload;
* items go through the reference importer pipeline without simplification
  (io/import.rs:47-98 -> SPolygon::new simple_polygon.rs:41-71 -> centering pre-transform
  io/import.rs:214-217 -> SPSurrogate::new sp_surrogate.rs:33-53);
* containers follow Container::new (entities/container.rs:29-79): the Exterior hazard first, then
  holes (quality 0) and inferior-quality zones by ascending quality; the CDE box is the
  container's bounding box inflated to a square (container.rs:68);
* items are placed by seeded rejection sampling: candidates are drawn in a fixed order and the
  first one the engine reports collision-free is registered, so any engine that answers like the
  reference produces the same layout.

The generator needs a *backend* for host preparation and for the engine used while placing; the
GPU engine (``jcde.engine.GpuBackend``) and the test-suite's oracle both provide one.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

QUERY_DTYPE = np.dtype([("item", "<u4"), ("cos", "<f4"), ("sin", "<f4"), ("tx", "<f4"), ("ty", "<f4")])

# HazardEntity kinds (collision_detection/hazards/hazard.rs:38-51)
PLACED_ITEM, EXTERIOR, HOLE, QUALITY_ZONE = 0, 1, 2, 3

# CDEConfig defaults used by lbf (lbf/src/config.rs:37-45)
DEFAULT_DEPTH = 5
DEFAULT_CD_THRESHOLD = 16
DEFAULT_POLE_LIMITS = ((100, 0.0), (20, 0.75), (10, 0.90))
DEFAULT_N_FF_POLES = 2

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 output function on a uint64 array (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        x = np.asarray(x, dtype=np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


class Stream:
    """Counter-based random stream: draw i of stream (seed, sid) is mix(key ^ mix(i))."""

    def __init__(self, seed: int, sid: int):
        k = (int(seed) * 0x100000001B3 + int(sid) * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        self.key = _mix64(np.array([k], dtype=np.uint64))[0]
        self.pos = 0

    def u64(self, n: int) -> np.ndarray:
        idx = np.arange(self.pos, self.pos + n, dtype=np.uint64)
        self.pos += n
        return _mix64(_mix64(idx) ^ self.key)

    def f32(self, n: int) -> np.ndarray:
        """Uniform [0, 1) with 24 random bits, exact in float32."""
        return (self.u64(n) >> np.uint64(40)).astype(np.float32) * np.float32(2.0**-24)

    def f64(self, n: int) -> np.ndarray:
        return (self.u64(n) >> np.uint64(11)).astype(np.float64) * (2.0**-53)

    def uniform_f32(self, lo, hi, n: int) -> np.ndarray:
        lo, hi = np.float32(lo), np.float32(hi)
        v = lo + self.f32(n) * (hi - lo)
        return np.minimum(v, np.nextafter(hi, lo)).astype(np.float32)

    def randint(self, lo: int, hi: int, n: int) -> np.ndarray:
        """Uniform integers in [lo, hi] inclusive."""
        span = np.uint64(hi - lo + 1)
        return (self.u64(n) % span).astype(np.int64) + lo


_SIN_C = [(-1.0) ** k / math.factorial(2 * k + 1) for k in range(13)]
_COS_C = [(-1.0) ** k / math.factorial(2 * k) for k in range(13)]


def sincos_turns(u: np.ndarray):
    """(cos, sin) of 2*pi*u for u in [0, 1), float64, by quadrant reduction + Taylor (Horner).

    Only IEEE float64 additions and multiplications are used, so the result is the same on every
    platform; accuracy is ~1e-15, far below the float32 rounding applied afterwards.
    """
    u = np.asarray(u, dtype=np.float64)
    q = u * 4.0
    k = np.floor(q)
    r = q - k
    phi = r * (math.pi / 2.0)
    p2 = phi * phi
    s = np.full_like(phi, _SIN_C[-1])
    c = np.full_like(phi, _COS_C[-1])
    for a in reversed(_SIN_C[:-1]):
        s = s * p2 + a
    for a in reversed(_COS_C[:-1]):
        c = c * p2 + a
    s = s * phi
    k = k.astype(np.int64) & 3
    cos = np.where(k == 0, c, np.where(k == 1, -s, np.where(k == 2, -c, s)))
    sin = np.where(k == 0, s, np.where(k == 1, c, np.where(k == 2, -s, -c)))
    return cos, sin


# 1 / (2k + 1), k = 0..12, and ln 2 split into two doubles (hi + lo)
_ATANH_C = [float.fromhex(h) for h in (
    "0x1.0000000000000p+0", "0x1.5555555555555p-2", "0x1.999999999999ap-3", "0x1.2492492492492p-3",
    "0x1.c71c71c71c71cp-4", "0x1.745d1745d1746p-4", "0x1.3b13b13b13b14p-4", "0x1.1111111111111p-4",
    "0x1.e1e1e1e1e1e1ep-5", "0x1.af286bca1af28p-5", "0x1.8618618618618p-5", "0x1.642c8590b2164p-5",
    "0x1.47ae147ae147bp-5")]
_LN2_HI = float.fromhex("0x1.62e42fefa39efp-1")
_LN2_LO = float.fromhex("0x1.abc9e3b39803fp-56")
_SQRT_HALF = float.fromhex("0x1.6a09e667f3bcdp-1")


def ln_f64(x: np.ndarray) -> np.ndarray:
    """Natural logarithm of positive normal float64 values using only IEEE additions, multiplications
    and divisions (bit-identical on every platform, and restated in the device generator): x = m 2^e
    with m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh(z) = 2 (z + z^3/3 + ...) with z = (m-1)/(m+1),
    |z| <= 0.172, 13 terms of the series (Horner form)."""
    x = np.asarray(x, dtype=np.float64)
    bits = x.view(np.uint64)
    e = ((bits >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64) - 1022
    m = ((bits & np.uint64((1 << 52) - 1)) | np.uint64(1022 << 52)).view(np.float64)   # [0.5, 1)
    low = m < _SQRT_HALF
    m = np.where(low, m * 2.0, m)
    e = np.where(low, e - 1, e).astype(np.float64)
    z = (m - 1.0) / (m + 1.0)
    z2 = z * z
    s = np.full_like(z, _ATANH_C[-1])
    for c in reversed(_ATANH_C[:-1]):
        s = s * z2 + c
    t = (2.0 * z) * s
    return e * _LN2_HI + (e * _LN2_LO + t)


def normal_pair(u1: np.ndarray, u2: np.ndarray):
    """Two standard normal float64 draws from uniforms u1 in (0, 1] and u2 in [0, 1) by the
    Box-Muller transform (G. E. P. Box and M. E. Muller, 1958): r = sqrt(-2 ln u1), (r cos 2 pi u2,
    r sin 2 pi u2), with ln_f64 and the Taylor sin/cos of sincos_turns (every step an IEEE operation)."""
    r = np.sqrt(-2.0 * ln_f64(u1))
    c, s = sincos_turns(u2)
    return r * c, r * s


def transform_points(xy: np.ndarray, cos, sin, tx, ty) -> np.ndarray:
    """TRANSFORM_FORMULA (geometry/primitives/point.rs:259-264) in float32, no fused multiply-add.

    The matrix is rot_transl_m (geometry/transformation.rs:475-483): [[c, -s, tx], [s, c, ty]].
    """
    xy = np.asarray(xy, dtype=np.float32)
    c, s = np.float32(cos), np.float32(sin)
    ms = np.float32(-s)
    x, y = xy[:, 0], xy[:, 1]
    one = np.float32(1.0)
    tx_ = np.float32(tx) * one
    ty_ = np.float32(ty) * one
    ox = (c * x + ms * y) + tx_
    oy = (s * x + c * y) + ty_
    return np.stack([ox, oy], axis=1).astype(np.float32)


def centroid_f32(xy: np.ndarray, area) -> tuple:
    """SPolygon::centroid (simple_polygon.rs:173-192), sequential float32 accumulation."""
    xy = np.asarray(xy, dtype=np.float32)
    n = len(xy)
    cx = np.float32(0.0)
    cy = np.float32(0.0)
    for i in range(n):
        j = 0 if i == n - 1 else i + 1
        xi, yi = xy[i, 0], xy[i, 1]
        xj, yj = xy[j, 0], xy[j, 1]
        cr = xi * yj - xj * yi
        cx = np.float32(cx + (xi + xj) * cr)
        cy = np.float32(cy + (yi + yj) * cr)
    six_a = np.float32(6.0) * np.float32(area)
    return np.float32(cx / six_a), np.float32(cy / six_a)


def centroids_f32(shapes, areas) -> np.ndarray:
    """centroid_f32 of many shapes at once: the same sequential float32 accumulation per shape,
    vectorised across shapes (vertex i of every shape per numpy step).  Returns (n, 2) float32."""
    n = len(shapes)
    nv = np.array([len(s) for s in shapes], dtype=np.int64)
    m = int(nv.max()) if n else 0
    X = np.zeros((n, m + 1), np.float32)
    Y = np.zeros((n, m + 1), np.float32)
    for k, s in enumerate(shapes):
        s = np.asarray(s, dtype=np.float32)
        X[k, : len(s)] = s[:, 0]
        Y[k, : len(s)] = s[:, 1]
        X[k, len(s)] = s[0, 0]   # the closing edge (i = n-1, j = 0)
        Y[k, len(s)] = s[0, 1]
    cx = np.zeros(n, np.float32)
    cy = np.zeros(n, np.float32)
    for i in range(m):
        live = i < nv
        xi, yi, xj, yj = X[:, i], Y[:, i], X[:, i + 1], Y[:, i + 1]
        # a shape's last vertex pairs with its first
        last = i == nv - 1
        xj = np.where(last, X[:, 0], xj)
        yj = np.where(last, Y[:, 0], yj)
        cr = xi * yj - xj * yi
        cx = np.where(live, (cx + (xi + xj) * cr).astype(np.float32), cx)
        cy = np.where(live, (cy + (yi + yj) * cr).astype(np.float32), cy)
    six_a = np.float32(6.0) * np.asarray(areas, dtype=np.float32)
    return np.stack([cx / six_a, cy / six_a], axis=1).astype(np.float32)


def star_polygon(st: Stream, nv: int, r_lo: float, r_hi: float, center=(0.0, 0.0)) -> np.ndarray:
    """Star-shaped simple polygon: sorted uniform angles, radii R*U[0.6, 1.0], R ~ U[r_lo, r_hi]."""
    R = r_lo + st.f64(1)[0] * (r_hi - r_lo)
    while True:
        u = np.sort(st.f64(nv))
        rad = R * (0.6 + 0.4 * st.f64(nv))
        c, s = sincos_turns(u)
        x = (center[0] + rad * c).astype(np.float32)
        y = (center[1] + rad * s).astype(np.float32)
        xy = np.stack([x, y], axis=1)
        if len(np.unique(xy, axis=0)) == nv and len(np.unique(u)) == nv:
            return xy


def rect_polygon(x_min, y_min, x_max, y_max) -> np.ndarray:
    """SPolygon::from(Rect) vertex order (simple_polygon.rs:330-343)."""
    return np.array([[x_min, y_min], [x_max, y_min], [x_max, y_max], [x_min, y_max]], dtype=np.float32)


@dataclass
class Item:
    xy: np.ndarray          # internal shape (centered), counter-clockwise
    poi: np.ndarray         # (x, y, r)
    poles: np.ndarray       # (k, 3) surrogate poles, poles[0] is the poi
    n_ff_poles: int
    area: float
    diameter: float
    centroid: tuple = (0.0, 0.0)   # of the imported shape: the centering pre-transform moved it to the origin


@dataclass
class HazardSpec:
    kind: int
    dynamic: bool
    xy: np.ndarray
    poi: np.ndarray
    key: int = -1
    placement: tuple | None = None   # (item, cos, sin, tx, ty) for placed items
    tag: int = 0                     # unique entity identity (HazardEntity equality, hazard.rs:38-51)


@dataclass
class Layout:
    name: str
    depth: int
    cd_threshold: int
    cde_bbox: np.ndarray
    items: list = field(default_factory=list)
    hazards: list = field(default_factory=list)      # registration order (static first)
    filter_keys: list = field(default_factory=list)
    n_failed_placements: int = 0


def modify_shape(backend, xy, area, deflate: bool, simplify_tolerance, narrow_concavity_ratio=None):
    """The shape modification of OriginalShape::convert_to_internal (original_shape.rs:33-42):
    simplify_shape at the tolerance, then — with a narrow-concavity cutoff — close_narrow_concavities
    and simplify_shape at a tenth of the tolerance.  Returns the vertices before the final
    SPolygon::new."""
    xy = backend.simplify_shape(xy, area, deflate, simplify_tolerance)
    if narrow_concavity_ratio is not None:
        xy = backend.close_concavities(xy, deflate, narrow_concavity_ratio)
        cxy, _, carea, _, _ = backend.spolygon_new(xy)
        xy = backend.simplify_shape(cxy, carea, deflate, np.float32(simplify_tolerance) / np.float32(10.0))
    return xy


def import_item(backend, raw_xy, pole_limits=DEFAULT_POLE_LIMITS, n_ff_poles=DEFAULT_N_FF_POLES,
                simplify_tolerance=None, narrow_concavity_ratio=None) -> Item:
    """Importer::import_item (io/import.rs:47-98, entities/item.rs:27-48) with
    OriginalShape::convert_to_internal (original_shape.rs:23-50): the centred shape, simplified
    (ShapeModifyMode::Inflate) when a tolerance is given — lbf's default config uses 0.001
    (lbf/src/config.rs:42), with narrow concavities closed when a cutoff is given as well (lbf's
    default: 0.01, config.rs:43).  Item.area is the original shape's (Item::area), the diameter that
    of the internal shape (the one item_placement_order sorts by)."""
    xy, bbox, area, diam, poi = backend.spolygon_new(raw_xy)
    cx, cy = centroid_f32(xy, area)
    # centering_transformation (io/import.rs:214-217): DTransformation(0, (-cx, -cy)); sin_cos(0) = (0, 1)
    ixy = transform_points(xy, 1.0, 0.0, -cx, -cy)
    ipoi = np.concatenate([transform_points(poi[None, :2], 1.0, 0.0, -cx, -cy)[0], poi[2:3]]).astype(np.float32)
    iarea, idiam = area, diam
    if simplify_tolerance is not None:
        # simplify_shape ends in SPolygon::new: new area, diameter and poi for the internal shape
        simp = modify_shape(backend, ixy, area, False, simplify_tolerance, narrow_concavity_ratio)
        ixy, _, iarea, idiam, ipoi = backend.spolygon_new(simp)
    poles = backend.surrogate_poles(ixy, iarea, ipoi, pole_limits)
    return Item(ixy, ipoi, poles, min(n_ff_poles, len(poles)), float(area), float(idiam), (float(cx), float(cy)))


def import_static(backend, raw_xy, kind, simplify_tolerance=None, narrow_concavity_ratio=None) -> HazardSpec:
    """Container outer / hole / zone: SPolygon::new then the empty pre-transform (io/import.rs:119-124);
    with a tolerance simplified as OriginalShape::convert_to_internal does (original_shape.rs:23-50):
    the outer with ShapeModifyMode::Deflate (io/import.rs:123), holes and zones with Inflate
    (io/import.rs:181)."""
    xy, bbox, area, diam, poi = backend.spolygon_new(raw_xy)
    ixy = transform_points(xy, 1.0, 0.0, 0.0, 0.0)
    ipoi = np.concatenate([transform_points(poi[None, :2], 1.0, 0.0, 0.0, 0.0)[0], poi[2:3]]).astype(np.float32)
    if simplify_tolerance is not None:
        simp = modify_shape(backend, ixy, area, kind == EXTERIOR, simplify_tolerance, narrow_concavity_ratio)
        ixy, _, _, _, ipoi = backend.spolygon_new(simp)
    return HazardSpec(kind, False, ixy, ipoi)


def inflate_to_square(b) -> np.ndarray:
    """Rect::inflate_to_square (rect.rs:93-109) in float32."""
    x0, y0, x1, y1 = (np.float32(v) for v in b)
    w = np.float32(x1 - x0)
    h = np.float32(y1 - y0)
    dx = dy = np.float32(0.0)
    if h < w:
        dy = np.float32((w - h) / np.float32(2.0))
    elif w < h:
        dx = np.float32((h - w) / np.float32(2.0))
    return np.array([x0 - dx, y0 - dy, x1 + dx, y1 + dy], dtype=np.float32)


def bbox_of(xy) -> np.ndarray:
    xy = np.asarray(xy, dtype=np.float32)
    return np.array([xy[:, 0].min(), xy[:, 1].min(), xy[:, 0].max(), xy[:, 1].max()], dtype=np.float32)


def placed_hazard(item: Item, item_id: int, cos, sin, tx, ty) -> HazardSpec:
    """PlacedItem::new (entities/placed_item.rs:27-36): the item shape and poi, transformed."""
    xy = transform_points(item.xy, cos, sin, tx, ty)
    p = transform_points(item.poi[None, :2], cos, sin, tx, ty)[0]
    poi = np.array([p[0], p[1], item.poi[2]], dtype=np.float32)
    return HazardSpec(PLACED_ITEM, True, xy, poi, placement=(item_id, float(cos), float(sin), float(tx), float(ty)))


def _tag_of(lay: "Layout") -> int:
    return len(lay.hazards) + 1


def make_queries(st: Stream, n: int, n_item_types: int, bbox) -> np.ndarray:
    """Uniform queries: item ~ U{0..T-1}, rotation ~ U[0, 2pi), translation ~ U(bbox)."""
    q = np.zeros(n, dtype=QUERY_DTYPE)
    q["item"] = st.randint(0, n_item_types - 1, n).astype(np.uint32)
    c, s = sincos_turns(st.f64(n))
    q["cos"] = c.astype(np.float32)
    q["sin"] = s.astype(np.float32)
    q["tx"] = st.uniform_f32(bbox[0], bbox[2], n)
    q["ty"] = st.uniform_f32(bbox[1], bbox[3], n)
    return q


def _place_items(backend, lay: Layout, eng, seed: int, n_place: int, chunk: int, max_attempts: int):
    """Seeded rejection sampling: place item p at the first collision-free candidate of its stream."""
    st_types = Stream(seed, 7)
    types = st_types.randint(0, len(lay.items) - 1, n_place)
    for p in range(n_place):
        t = int(types[p])
        st = Stream(seed, 1000 + p)
        placed = False
        tried = 0
        while tried < max_attempts and not placed:
            q = make_queries(st, chunk, 1, lay.cde_bbox)
            q["item"] = t
            v = eng.detect_batch(q)
            free = np.flatnonzero(v == 0)
            if len(free):
                j = int(free[0])
                hz = placed_hazard(lay.items[t], t, q["cos"][j], q["sin"][j], q["tx"][j], q["ty"][j])
                hz.tag = _tag_of(lay)
                hz.key = eng.register_hazard(hz.kind, hz.dynamic, hz.xy, hz.poi, hz.tag)
                lay.hazards.append(hz)
                placed = True
            tried += chunk
        if not placed:
            lay.n_failed_placements += 1


def _new_layout_engine(backend, lay: Layout):
    eng = backend.new_engine(lay.depth, lay.cd_threshold, lay.cde_bbox)
    for it in lay.items:
        eng.add_item(it.xy, it.poi, it.poles, it.n_ff_poles)
    for i, hz in enumerate(lay.hazards):
        hz.tag = hz.tag or i + 1
        hz.key = eng.register_hazard(hz.kind, hz.dynamic, hz.xy, hz.poi, hz.tag)
    return eng


def replay(backend, lay: Layout):
    """A fresh engine of `backend` holding exactly the layout's items and hazards."""
    eng = backend.new_engine(lay.depth, lay.cd_threshold, lay.cde_bbox)
    for it in lay.items:
        eng.add_item(it.xy, it.poi, it.poles, it.n_ff_poles)
    for hz in lay.hazards:
        k = eng.register_hazard(hz.kind, hz.dynamic, hz.xy, hz.poi, hz.tag)
        if hz.key >= 0 and k != hz.key:
            raise RuntimeError(f"hazard key mismatch on replay: {k} != {hz.key}")
    return eng


def strip_layout(backend, seed=0xC0, n_types=10, v_range=(8, 24), r_range=(20.0, 60.0), width=1000.0,
                 height=500.0, n_place=40, depth=DEFAULT_DEPTH, cd_threshold=DEFAULT_CD_THRESHOLD,
                 chunk=256, max_attempts=1 << 16, name="strip", import_many=None):
    """Rectangular strip container with star items (the small CPU-runnable layout).  `import_many`
    (a list of raw shapes -> a list of Items, e.g. ``jcde.prep.import_items``) imports the item
    types in one batch instead of one ``import_item`` call each; the Items must be the same."""
    st = Stream(seed, 1)
    raws = []
    for _ in range(n_types):
        nv = int(st.randint(v_range[0], v_range[1], 1)[0])
        raws.append(star_polygon(st, nv, *r_range))
    items = import_many(raws) if import_many is not None else [import_item(backend, r) for r in raws]
    outer = import_static(backend, rect_polygon(0.0, 0.0, width, height), EXTERIOR)
    lay = Layout(name, depth, cd_threshold, inflate_to_square(bbox_of(outer.xy)), items=items)
    lay.hazards.append(outer)
    eng = _new_layout_engine(backend, lay)
    _place_items(backend, lay, eng, seed, n_place, chunk, max_attempts)
    return lay, eng


def star_container_layout(backend, seed=0xC1, n_types=40, v_range=(8, 200), r_range=(20.0, 60.0),
                          container_r=2000.0, container_nv=64, n_holes=4, hole_side=(100.0, 300.0),
                          zone_qualities=(1, 2), zone_r=(150.0, 300.0), n_place=300, depth=DEFAULT_DEPTH,
                          cd_threshold=DEFAULT_CD_THRESHOLD, chunk=256, max_attempts=1 << 16, name="star"):
    """Star container with rectangular holes and inferior-quality zones (the large collect layout)."""
    st = Stream(seed, 1)
    items = []
    for _ in range(n_types):
        nv = int(st.randint(v_range[0], v_range[1], 1)[0])
        items.append(import_item(backend, star_polygon(st, nv, *r_range)))
    sc = Stream(seed, 2)
    outer = import_static(backend, star_polygon(sc, container_nv, container_r, container_r), EXTERIOR)
    statics = [outer]
    inner = 0.35 * container_r
    for _ in range(n_holes):            # quality 0 zones are holes (entities/container.rs:124-126)
        w, h = sc.f64(2) * (hole_side[1] - hole_side[0]) + hole_side[0]
        cx, cy = (sc.f64(2) * 2.0 - 1.0) * inner
        statics.append(import_static(backend, rect_polygon(np.float32(cx - w / 2), np.float32(cy - h / 2),
                                                            np.float32(cx + w / 2), np.float32(cy + h / 2)), HOLE))
    for q in zone_qualities:
        cx, cy = (sc.f64(2) * 2.0 - 1.0) * inner
        nv = int(sc.randint(8, 24, 1)[0])
        z = import_static(backend, star_polygon(sc, nv, zone_r[0], zone_r[1], center=(cx, cy)), QUALITY_ZONE)
        z.placement = ("quality", q)
        statics.append(z)
    lay = Layout(name, depth, cd_threshold, inflate_to_square(bbox_of(outer.xy)), items=items)
    lay.hazards.extend(statics)
    eng = _new_layout_engine(backend, lay)
    # HazKeyFilter::from_irrelevant_qzones(2) (hazards/filter.rs:21-41) ignores the quality-1 zone
    lay.filter_keys = [hz.key for hz in lay.hazards if hz.kind == QUALITY_ZONE and hz.placement == ("quality", 1)]
    _place_items(backend, lay, eng, seed, n_place, chunk, max_attempts)
    return lay, eng


def queries_for(lay: Layout, n: int, seed: int, sid: int = 3) -> np.ndarray:
    return make_queries(Stream(seed, sid), n, len(lay.items), lay.cde_bbox)


_RIGHT_COS = np.array([1, 0, -1, 0], np.float32)
_RIGHT_SIN = np.array([0, 1, 0, -1], np.float32)


def boundary_queries(lay: Layout, n: int, seed: int) -> np.ndarray:
    """Queries on the quadtree's split lines at right-angle rotations (cos / sin exactly 0 or +-1),
    a third of them nudged by one ULP: the closed-interval, half-intersection and FPA cases."""
    st = Stream(seed, 1)
    b = np.asarray(lay.cde_bbox, dtype=np.float32)
    lines_x = b[0] + (b[2] - b[0]) * np.arange(33, dtype=np.float32) / np.float32(32)
    lines_y = b[1] + (b[3] - b[1]) * np.arange(33, dtype=np.float32) / np.float32(32)
    q = np.zeros(n, dtype=QUERY_DTYPE)
    q["item"] = st.randint(0, len(lay.items) - 1, n).astype(np.uint32)
    rot = st.randint(0, 3, n)
    q["cos"] = _RIGHT_COS[rot]
    q["sin"] = _RIGHT_SIN[rot]
    ix, iy = st.randint(0, 32, n), st.randint(0, 32, n)
    tx, ty = lines_x[ix], lines_y[iy]
    free_x = st.f32(n) < 0.3   # a coordinate off the lines keeps the other one on a line
    tx = np.where(free_x, st.uniform_f32(b[0], b[2], n), tx).astype(np.float32)
    nudge = st.randint(0, 2, n) - 1   # -1, 0, +1 ULP
    q["tx"] = np.where(nudge < 0, np.nextafter(tx, np.float32(-np.inf)),
                       np.where(nudge > 0, np.nextafter(tx, np.float32(np.inf)), tx))
    q["ty"] = ty
    return q


def touch_queries(lay: Layout, n: int, seed: int) -> np.ndarray:
    """Queries whose item touches a hazard: at a right-angle rotation, one item vertex is put on a
    hazard vertex, on a hazard edge's midpoint or at a random point of a hazard edge (up to the
    rounding of the translation), and half of them are moved one ULP in x or y.  These are the
    exact-touch cases of edge_intersection (edge.rs:180-228), of the closed box tests and of the
    FPA vertex guard."""
    st = Stream(seed, 1)
    hz = lay.hazards
    hi = st.randint(0, len(hz) - 1, n)
    it = st.randint(0, len(lay.items) - 1, n)
    rot = st.randint(0, 3, n)
    mode = st.randint(0, 2, n)          # 0: on a vertex, 1: on an edge midpoint, 2: on an edge at random t
    tt = st.f32(n)
    r1, r2 = st.u64(n), st.u64(n)
    nudge = st.randint(0, 7, n)         # 1-4: one ULP in +x, -x, +y, -y
    hv_n = np.array([len(h.xy) for h in hz], np.uint64)
    iv_n = np.array([len(i.xy) for i in lay.items], np.uint64)
    hoff = np.concatenate([[0], np.cumsum(hv_n)]).astype(np.int64)
    ioff = np.concatenate([[0], np.cumsum(iv_n)]).astype(np.int64)
    hxy = np.concatenate([h.xy for h in hz]).astype(np.float32)
    ixy = np.concatenate([i.xy for i in lay.items]).astype(np.float32)
    a = (r1 % hv_n[hi]).astype(np.int64)
    b = np.where(a + 1 == hv_n[hi].astype(np.int64), 0, a + 1)
    pa, pb = hxy[hoff[hi] + a], hxy[hoff[hi] + b]
    t = np.where(mode == 1, np.float32(0.5), tt).astype(np.float32)[:, None]
    p = np.where((mode == 0)[:, None], pa, (pa + t * (pb - pa)).astype(np.float32)).astype(np.float32)
    v = ixy[ioff[it] + (r2 % iv_n[it]).astype(np.int64)]
    c, s = _RIGHT_COS[rot], _RIGHT_SIN[rot]
    px = (c * v[:, 0]).astype(np.float32) + (-s * v[:, 1]).astype(np.float32)
    py = (s * v[:, 0]).astype(np.float32) + (c * v[:, 1]).astype(np.float32)
    tx = (p[:, 0] - px).astype(np.float32)
    ty = (p[:, 1] - py).astype(np.float32)
    up, dn = np.float32(np.inf), np.float32(-np.inf)
    tx = np.where(nudge == 1, np.nextafter(tx, up), np.where(nudge == 2, np.nextafter(tx, dn), tx))
    ty = np.where(nudge == 3, np.nextafter(ty, up), np.where(nudge == 4, np.nextafter(ty, dn), ty))
    q = np.zeros(n, dtype=QUERY_DTYPE)
    q["item"] = it.astype(np.uint32)
    q["cos"], q["sin"], q["tx"], q["ty"] = c, s, tx, ty
    return q


def multi_layouts(backend, seed=0xC2, n_layouts=64, n_types=40, v_range=(8, 200), r_range=(20.0, 60.0),
                  items_range=(20, 400), container_v=(32, 128), radius_per_sqrt_item=70.0, depth=DEFAULT_DEPTH,
                  cd_threshold=DEFAULT_CD_THRESHOLD, chunk=256, max_attempts=1 << 14, item_pool=None):
    """Independent bin layouts (the batched multi-layout workload): star containers of 32-128
    vertices, each holding a log-uniform 20-400 items drawn from one shared pool of star item types
    (8-200 vertices).  Returns [(layout, engine)]."""
    st = Stream(seed, 1)
    if item_pool is None:
        item_pool = []
        for _ in range(n_types):
            nv = int(st.randint(v_range[0], v_range[1], 1)[0])
            item_pool.append(import_item(backend, star_polygon(st, nv, *r_range)))
    sl = Stream(seed, 2)
    out = []
    for l in range(n_layouts):
        n_items = int(round(math.exp(math.log(items_range[0]) + sl.f64(1)[0] *
                                     (math.log(items_range[1]) - math.log(items_range[0])))))
        nv = int(sl.randint(container_v[0], container_v[1], 1)[0])
        R = radius_per_sqrt_item * math.sqrt(n_items)
        outer = import_static(backend, star_polygon(sl, nv, R, R), EXTERIOR)
        lay = Layout(f"bin{l}", depth, cd_threshold, inflate_to_square(bbox_of(outer.xy)), items=item_pool)
        lay.hazards.append(outer)
        eng = _new_layout_engine(backend, lay)
        _place_items(backend, lay, eng, seed * 1000 + l, n_items, chunk, max_attempts)
        out.append((lay, eng))
    return out


def multi_queries(layouts, seed=0xC2, q_range=(4096, 262144)):
    """Per-layout uniform query batches with log-uniform sizes; returns (queries, offsets)."""
    sq = Stream(seed, 3)
    parts, offs = [], [0]
    for l, (lay, _) in enumerate(layouts):
        n = int(round(math.exp(math.log(q_range[0]) + sq.f64(1)[0] * (math.log(q_range[1]) - math.log(q_range[0])))))
        parts.append(make_queries(Stream(seed, 100 + l), n, len(lay.items), lay.cde_bbox))
        offs.append(offs[-1] + n)
    return np.concatenate(parts), np.array(offs, dtype=np.uint32)


def exterior_ring(xy, radius: float) -> np.ndarray:
    """Circles just outside a counter-clockwise container, tangent to each edge from outside and
    spaced one radius apart: the exterior hazard's stand-in for poles (the region outside a polygon
    has no inscribed circles of its own)."""
    xy = np.asarray(xy, dtype=np.float64)
    out = []
    for i in range(len(xy)):
        a, b = xy[i], xy[(i + 1) % len(xy)]
        d = b - a
        L = float(np.hypot(d[0], d[1]))
        if L == 0.0:
            continue
        nrm = np.array([d[1], -d[0]]) / L   # outward for counter-clockwise vertices
        k = max(1, int(math.ceil(L / radius)))
        for j in range(k):
            c = a + d * ((j + 0.5) / k) + nrm * radius
            out.append((c[0], c[1], radius))
    return np.asarray(out, dtype=np.float32)


def hazard_poles(backend, lay: Layout, pole_limits=DEFAULT_POLE_LIMITS, ring_radius=40.0) -> np.ndarray:
    """Poles of every hazard, as rows (x, y, r, key bits) — the pole sets the overlap proxy measures
    against.  A placed item's are its item's surrogate poles under its placement (SPolygon::transform
    moves the surrogate with the shape, simple_polygon.rs:195-224); holes and zones get poles
    generated on their own shapes; the exterior gets a ring of tangent circles outside the container."""
    rows = []
    for hz in lay.hazards:
        if hz.kind == EXTERIOR:
            poles = exterior_ring(hz.xy, ring_radius)
        elif hz.placement is not None and hz.kind == PLACED_ITEM:
            t, c, s, tx, ty = hz.placement
            it = lay.items[t]
            ctr = transform_points(it.poles[:, :2], c, s, tx, ty)
            poles = np.concatenate([ctr, it.poles[:, 2:3]], axis=1)
        else:
            _, _, area, _, _ = backend.spolygon_new(hz.xy)
            poles = backend.surrogate_poles(hz.xy, area, hz.poi, pole_limits)
        key = np.full((len(poles), 1), hz.key, dtype=np.uint32).view(np.float32)
        rows.append(np.concatenate([poles.astype(np.float32), key], axis=1))
    return np.ascontiguousarray(np.concatenate(rows).astype(np.float32))


def random_params(st: Stream, n: int, n_item_types: int, bbox):
    """Uniform candidate placements as (theta, tx, ty) float32 rows + item types."""
    items = st.randint(0, n_item_types - 1, n).astype(np.uint32)
    th = (st.f64(n) * (2.0 * math.pi)).astype(np.float32)
    tx = st.uniform_f32(bbox[0], bbox[2], n)
    ty = st.uniform_f32(bbox[1], bbox[3], n)
    return np.ascontiguousarray(np.stack([th, tx, ty], axis=1).astype(np.float32)), items
