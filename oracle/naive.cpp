// NAIVE CHECKER — TEST INFRASTRUCTURE ONLY.
//
// A tree-free statement of what jagua-rs's collision detection engine decides, written apart from
// the oracle (cde_oracle.cpp) and from the product so that a misreading of the quadtree code
// (register / constrict / collides_with_quadrants / collect_collisions) shared by those two cannot
// go unnoticed.  It keeps no quadtree, no presence inference, no clipped edge lists and no virtual
// root: every query is tested against every edge of every relevant hazard, as the reference's
// README describes the engine's intent ("designed to mimic a naive trigonometric approach",
// README.md:53).  The primitives below are a separate reading of the reference's Rust sources
// (file:line at each); nothing is shared with cde_oracle.cpp.
//
// What it decides for a query (item, transformation) against hazard h (not ignored by the filter):
//   * bbox rule (cd_engine.rs:161-163, :261-263): the CDE box does not surround the shape's box;
//   * surrogate half (cd_engine.rs:204-223): a fail-fast pole touches an edge of h
//     (circle.rs:109-113, edge.rs:152-159) or its centre lies in h's forbidden region (inside h for
//     interior-scope hazards, outside for the exterior), or a pier crosses an edge of h or starts in
//     that region;
//   * polygon half (cd_engine.rs:160-197): an edge of the transformed shape crosses an edge of h
//     (edge.rs:180-228), or the containment rule holds (cd_engine.rs:231-255 with the ray-cast
//     point-in-polygon of simple_polygon.rs:255-292).
// The engine reaches the same answers through its quadtree; the two can differ only where
// floating-point rounding puts a touch exactly on a quadtree boundary (an FPA-tolerance corner).
// The surrogate half's "centre in the forbidden region" clause is geometric, not the engine's
// rule (the engine only sees the region through Entire nodes), but wherever it fires the item
// itself overlaps h, so the combined verdict and the combined collected set are unchanged.
//
// Build with -ffp-contract=off and without fast-math (Rust never fuses a*b+c).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

namespace naive {

struct V2 { float x, y; };
struct Seg { V2 a, b; };
struct Box { float x0, y0, x1, y1; };
struct Disc { V2 c; float r; };

// float-cmp 0.10, `approx_eq!(f32, a, b)` with the default F32Margin (epsilon = f32::EPSILON,
// ulps = 4), as used by FPA's PartialEq (util/fpa.rs:18-23): exact equality, then an absolute
// epsilon, then the i32 distance of the bit patterns (wrapping subtraction, saturating absolute
// value).
static inline bool approx(float a, float b) {
    if (a == b) return true;
    if (std::fabs(a - b) <= FLT_EPSILON) return true;
    uint32_t ua, ub;
    std::memcpy(&ua, &a, 4);
    std::memcpy(&ub, &b, 4);
    int32_t d = (int32_t)(ua - ub);
    int64_t ad = d < 0 ? -(int64_t)d : (int64_t)d;
    if (ad > INT32_MAX) ad = INT32_MAX;
    return ad <= 4;
}
// FPA's PartialOrd (util/fpa.rs:25-31): Equal when approx-equal, otherwise f32's own order.
static inline bool a_le(float a, float b) { return approx(a, b) || a < b; }
static inline bool a_ge(float a, float b) { return approx(a, b) || a > b; }
static inline bool a_lt(float a, float b) { return !approx(a, b) && a < b; }
static inline bool a_gt(float a, float b) { return !approx(a, b) && a > b; }

enum Rel { R_INTERSECTING, R_ENCLOSED, R_SURROUNDING, R_DISJOINT };

// rect.rs:268-271
static inline bool box_overlap(const Box& p, const Box& q) {
    return std::fmax(p.x0, q.x0) <= std::fmin(p.x1, q.x1) && std::fmax(p.y0, q.y0) <= std::fmin(p.y1, q.y1);
}
// rect.rs:46-65
static Rel relation(const Box& s, const Box& o) {
    if (!box_overlap(s, o)) return R_DISJOINT;
    if (s.x0 <= o.x0 && s.y0 <= o.y0 && s.x1 >= o.x1 && s.y1 >= o.y1) return R_SURROUNDING;
    if (s.x0 >= o.x0 && s.y0 >= o.y0 && s.x1 <= o.x1 && s.y1 <= o.y1) return R_ENCLOSED;
    return R_INTERSECTING;
}
// rect.rs:70-89 with rect.rs:274-279
static Rel almost_relation(const Box& s, const Box& o) {
    if (!(a_le(std::fmax(s.x0, o.x0), std::fmin(s.x1, o.x1)) && a_le(std::fmax(s.y0, o.y0), std::fmin(s.y1, o.y1))))
        return R_DISJOINT;
    if (a_le(s.x0, o.x0) && a_le(s.y0, o.y0) && a_ge(s.x1, o.x1) && a_ge(s.y1, o.y1)) return R_SURROUNDING;
    if (a_ge(s.x0, o.x0) && a_ge(s.y0, o.y0) && a_le(s.x1, o.x1) && a_le(s.y1, o.y1)) return R_ENCLOSED;
    return R_INTERSECTING;
}
// rect.rs:282-288
static inline bool box_has(const Box& r, V2 p) { return p.x >= r.x0 && p.x <= r.x1 && p.y >= r.y0 && p.y <= r.y1; }

// edge.rs:180-228 (edge_intersection without the intersection point)
static bool seg_cross(const Seg& e1, const Seg& e2) {
    const float x1 = e1.a.x, y1 = e1.a.y, x2 = e1.b.x, y2 = e1.b.y;
    const float x3 = e2.a.x, y3 = e2.a.y, x4 = e2.b.x, y4 = e2.b.y;
    if (std::fmax(std::fmin(x1, x2), std::fmin(x3, x4)) > std::fmin(std::fmax(x1, x2), std::fmax(x3, x4))) return false;
    if (std::fmax(std::fmin(y1, y2), std::fmin(y3, y4)) > std::fmin(std::fmax(y1, y2), std::fmax(y3, y4))) return false;
    const float tn = (x2 - x4) * (y4 - y3) - (y2 - y4) * (x4 - x3);
    const float td = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    const float un = (x2 - x4) * (y2 - y1) - (y2 - y4) * (x2 - x1);
    const float ud = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    if (td == 0.0f || ud == 0.0f) return false;
    const float t = tn / td, u = un / ud;
    return t >= 0.0f && t <= 1.0f && u >= 0.0f && u <= 1.0f;
}
// edge.rs:63-87 (closest_point_on_edge) and edge.rs:152-159 (sq_distance_to)
static float seg_sq_dist(const Seg& e, V2 p) {
    const float a = p.x - e.a.x, b = p.y - e.a.y, c = e.b.x - e.a.x, d = e.b.y - e.a.y;
    const float dot = a * c + b * d;
    const float len_sq = c * c + d * d;
    float param = -1.0f;
    if (len_sq != 0.0f) param = dot / len_sq;
    float qx, qy;
    if (param < 0.0f) { qx = e.a.x; qy = e.a.y; }
    else if (param > 1.0f) { qx = e.b.x; qy = e.b.y; }
    else { qx = e.a.x + param * c; qy = e.a.y + param * d; }
    const float dx = p.x - qx, dy = p.y - qy;
    return dx * dx + dy * dy;
}
// circle.rs:109-113
static inline bool disc_touches(const Disc& c, const Seg& e) { return seg_sq_dist(e, c.c) <= c.r * c.r; }

struct Shape {
    std::vector<V2> v;
    Box bb;
    Disc poi;
    Seg edge(size_t i) const { return Seg{v[i], v[i + 1 == v.size() ? 0 : i + 1]}; }  // simple_polygon.rs:86-93
};
// simple_polygon.rs:122-133 (starts at f32::MAX / f32::MIN)
static Box bounds(const std::vector<V2>& v) {
    Box b{FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (const V2& p : v) {
        b.x0 = std::fmin(b.x0, p.x);
        b.y0 = std::fmin(b.y0, p.y);
        b.x1 = std::fmax(b.x1, p.x);
        b.y1 = std::fmax(b.y1, p.y);
    }
    return b;
}
// simple_polygon.rs:255-292: ray to the right, vertex guard by FPA
static bool inside(const Shape& s, V2 p) {
    if (!box_has(s.bb, p)) return false;
    const Seg ray{p, V2{s.bb.x1 + (s.bb.x1 - s.bb.x0), p.y}};
    unsigned n = 0;
    for (size_t i = 0; i < s.v.size(); i++) {
        const Seg e = s.edge(i);
        if ((approx(e.a.y, p.y) && a_gt(e.a.x, p.x)) || (approx(e.b.y, p.y) && a_gt(e.b.x, p.x))) {
            if (a_lt(e.a.y, p.y) || a_lt(e.b.y, p.y)) n++;
        } else if (seg_cross(ray, e)) {
            n++;
        }
    }
    return (n & 1u) == 1u;
}
// point.rs:26-31 with the rot_transl_m matrix [[c, -s, tx], [s, c, ty]] (transformation.rs:131-139)
static inline V2 move(float c, float s, float tx, float ty, V2 p) {
    const float ns = -s;
    return V2{c * p.x + ns * p.y + tx * 1.0f, s * p.x + c * p.y + ty * 1.0f};
}

enum Kind { PLACED = 0, EXTERIOR = 1, HOLE = 2, ZONE = 3 };

struct Haz {
    int kind;
    bool live;
    Shape s;
};
struct ItemT {
    Shape s;
    std::vector<Disc> ff;
    std::vector<Seg> piers;
};

struct Ctx {
    Box cde;
    std::vector<Haz> hz;
    std::vector<ItemT> items;
    int32_t exterior = -1;
};

// the hazard's forbidden region holds p: interior scope = inside, exterior scope = outside
// (hazard.rs scope: only the Exterior entity has exterior scope)
static inline bool in_region(const Haz& h, V2 p) {
    const bool in = inside(h.s, p);
    return h.kind == EXTERIOR ? !in : in;
}

// can a disc at c with radius r touch anything of box b?  Conservative in double, with a margin far
// above f32 rounding of the distance test, so it never hides a touch seg_sq_dist would report.
static inline bool disc_near_box(const Disc& d, const Box& b) {
    const double dx = std::max({(double)b.x0 - d.c.x, 0.0, (double)d.c.x - b.x1});
    const double dy = std::max({(double)b.y0 - d.c.y, 0.0, (double)d.c.y - b.y1});
    const double m = (double)d.r + 1e-3 * (std::fabs((double)d.c.x) + std::fabs((double)d.c.y) + d.r) + 1e-3;
    return dx * dx + dy * dy <= m * m;
}

static bool surrogate_hits(const Ctx& x, const ItemT& it, const float t[4], const Haz& h) {
    for (const Disc& p0 : it.ff) {
        const Disc p{move(t[0], t[1], t[2], t[3], p0.c), p0.r};
        if (in_region(h, p.c)) return true;
        if (h.kind != EXTERIOR && !disc_near_box(p, h.s.bb)) continue;
        for (size_t i = 0; i < h.s.v.size(); i++)
            if (disc_touches(p, h.s.edge(i))) return true;
    }
    for (const Seg& q0 : it.piers) {
        const Seg q{move(t[0], t[1], t[2], t[3], q0.a), move(t[0], t[1], t[2], t[3], q0.b)};
        if (in_region(h, q.a)) return true;
        for (size_t i = 0; i < h.s.v.size(); i++)
            if (seg_cross(q, h.s.edge(i))) return true;
    }
    return false;
}

// cd_engine.rs:231-255
static bool contained_hit(const Shape& s, const Haz& h) {
    const Rel rel = almost_relation(h.s.bb, s.bb);
    bool c = false;
    if (rel == R_SURROUNDING) c = inside(h.s, s.poi.c);
    else if (rel == R_ENCLOSED) c = inside(s, h.s.poi.c);
    return h.kind == EXTERIOR ? !c : c;
}

static bool poly_hits(const Shape& s, const Haz& h) {
    if (box_overlap(s.bb, h.s.bb)) {  // exact prune: seg_cross rejects on box overlap first
        for (size_t i = 0; i < s.v.size(); i++) {
            const Seg q = s.edge(i);
            const Box qb{std::fmin(q.a.x, q.b.x), std::fmin(q.a.y, q.b.y), std::fmax(q.a.x, q.b.x), std::fmax(q.a.y, q.b.y)};
            if (!box_overlap(qb, h.s.bb)) continue;
            for (size_t j = 0; j < h.s.v.size(); j++)
                if (seg_cross(q, h.s.edge(j))) return true;
        }
    }
    return contained_hit(s, h);
}

static void place(const ItemT& it, const float t[4], Shape& out) {
    out.v.resize(it.s.v.size());
    for (size_t i = 0; i < it.s.v.size(); i++) out.v[i] = move(t[0], t[1], t[2], t[3], it.s.v[i]);
    out.bb = bounds(out.v);
    out.poi = Disc{move(t[0], t[1], t[2], t[3], it.s.poi.c), it.s.poi.r};
}

static inline bool ignored(const std::vector<uint8_t>& f, size_t k) { return k < f.size() && f[k]; }

// 1 = collision (bbox rule, surrogate, polygon), 0 = free
static bool detect(const Ctx& x, uint32_t item, const float t[4], const std::vector<uint8_t>& f, Shape& buf) {
    const ItemT& it = x.items[item];
    place(it, t, buf);
    if (relation(x.cde, buf.bb) != R_SURROUNDING) return true;
    for (size_t k = 0; k < x.hz.size(); k++)
        if (x.hz[k].live && !ignored(f, k) && surrogate_hits(x, it, t, x.hz[k])) return true;
    for (size_t k = 0; k < x.hz.size(); k++)
        if (x.hz[k].live && !ignored(f, k) && poly_hits(buf, x.hz[k])) return true;
    return false;
}

static void collect(const Ctx& x, uint32_t item, const float t[4], const std::vector<uint8_t>& f, Shape& buf,
                    std::vector<uint32_t>& keys) {
    keys.clear();
    const ItemT& it = x.items[item];
    place(it, t, buf);
    const bool outside = relation(x.cde, buf.bb) != R_SURROUNDING;
    for (size_t k = 0; k < x.hz.size(); k++) {
        const Haz& h = x.hz[k];
        if (!h.live || ignored(f, k)) continue;
        if ((outside && (int32_t)k == x.exterior) || surrogate_hits(x, it, t, h) || poly_hits(buf, h))
            keys.push_back((uint32_t)k);
    }
}

static void parallel(uint64_t n, int nt, const std::function<void(uint64_t, uint64_t)>& fn) {
    if (nt <= 1 || n < 256) { fn(0, n); return; }
    std::vector<std::thread> th;
    for (int i = 0; i < nt; i++) th.emplace_back(fn, n * i / nt, n * (i + 1) / nt);
    for (auto& t : th) t.join();
}

static std::vector<uint8_t> mask(const uint32_t* ids, uint32_t n) {
    std::vector<uint8_t> m;
    for (uint32_t i = 0; i < n; i++) {
        if (ids[i] >= m.size()) m.resize(ids[i] + 1, 0);
        m[ids[i]] = 1;
    }
    return m;
}

}  // namespace naive

extern "C" {
using namespace naive;

#pragma pack(push, 1)
struct nv_query { uint32_t item; float cos, sin, tx, ty; };
#pragma pack(pop)

void* nv_new(const float* bbox4) {
    Ctx* c = new Ctx();
    c->cde = Box{bbox4[0], bbox4[1], bbox4[2], bbox4[3]};
    return c;
}
void nv_free(void* p) { delete (Ctx*)p; }

// Hazard with key = slot (the engine's dense key); a slot may be left dead with live = 0.
int32_t nv_set_hazard(void* p, uint32_t key, int32_t kind, int32_t live, const float* xy, uint32_t nv, const float* poi3) {
    Ctx* c = (Ctx*)p;
    if (key >= c->hz.size()) c->hz.resize(key + 1, Haz{0, false, Shape{}});
    Haz& h = c->hz[key];
    h.kind = kind;
    h.live = live != 0;
    h.s.v.resize(nv);
    for (uint32_t i = 0; i < nv; i++) h.s.v[i] = V2{xy[2 * i], xy[2 * i + 1]};
    h.s.bb = bounds(h.s.v);
    h.s.poi = Disc{V2{poi3[0], poi3[1]}, poi3[2]};
    if (kind == EXTERIOR && h.live && c->exterior < 0) c->exterior = (int32_t)key;
    return 0;
}

int32_t nv_add_item(void* p, const float* xy, uint32_t nv, const float* poi3, const float* ff_xyr, uint32_t n_ff,
                    const float* piers4, uint32_t n_piers) {
    Ctx* c = (Ctx*)p;
    ItemT it;
    it.s.v.resize(nv);
    for (uint32_t i = 0; i < nv; i++) it.s.v[i] = V2{xy[2 * i], xy[2 * i + 1]};
    it.s.bb = bounds(it.s.v);
    it.s.poi = Disc{V2{poi3[0], poi3[1]}, poi3[2]};
    for (uint32_t i = 0; i < n_ff; i++) it.ff.push_back(Disc{V2{ff_xyr[3 * i], ff_xyr[3 * i + 1]}, ff_xyr[3 * i + 2]});
    for (uint32_t i = 0; i < n_piers; i++)
        it.piers.push_back(Seg{V2{piers4[4 * i], piers4[4 * i + 1]}, V2{piers4[4 * i + 2], piers4[4 * i + 3]}});
    c->items.push_back(std::move(it));
    return (int32_t)c->items.size() - 1;
}

void nv_detect_batch(void* p, const nv_query* q, uint64_t n, const uint32_t* filt, uint32_t n_filt, uint8_t* out,
                     int32_t n_threads) {
    const Ctx& c = *(Ctx*)p;
    const std::vector<uint8_t> f = mask(filt, n_filt);
    parallel(n, n_threads, [&](uint64_t a, uint64_t b) {
        Shape buf;
        for (uint64_t i = a; i < b; i++) {
            const float t[4] = {q[i].cos, q[i].sin, q[i].tx, q[i].ty};
            out[i] = q[i].item < c.items.size() ? (detect(c, q[i].item, t, f, buf) ? 1 : 0) : 2;
        }
    });
}

// CSR of the ascending colliding keys per query; returns the total, or -(needed) if ids_cap is short.
int64_t nv_collect_batch(void* p, const nv_query* q, uint64_t n, const uint32_t* filt, uint32_t n_filt,
                         uint32_t* counts, uint32_t* ids, uint64_t ids_cap, int32_t n_threads) {
    const Ctx& c = *(Ctx*)p;
    const std::vector<uint8_t> f = mask(filt, n_filt);
    std::vector<std::vector<uint32_t>> per(n);
    parallel(n, n_threads, [&](uint64_t a, uint64_t b) {
        Shape buf;
        std::vector<uint32_t> keys;
        for (uint64_t i = a; i < b; i++) {
            const float t[4] = {q[i].cos, q[i].sin, q[i].tx, q[i].ty};
            if (q[i].item < c.items.size()) collect(c, q[i].item, t, f, buf, keys);
            else keys.clear();
            per[i] = keys;
        }
    });
    uint64_t total = 0;
    for (auto& v : per) total += v.size();
    if (total > ids_cap) return -(int64_t)total;
    uint64_t o = 0;
    for (uint64_t i = 0; i < n; i++) {
        counts[i] = (uint32_t)per[i].size();
        for (uint32_t k : per[i]) ids[o++] = k;
    }
    return (int64_t)total;
}

// Which clauses make query q collide with hazard `key` (0 when none does):
//   1  the bbox rule names this hazard (it is the exterior and the CDE box misses part of the shape)
//   2  a fail-fast pole or pier touches the hazard or lies in its forbidden region
//   4  a shape edge crosses a hazard edge, and the closed box of that hazard edge meets the shape
//      edge (rect.rs:301-345)
//   8  a shape edge crosses a hazard edge by edge_intersection's rounding only: the box of that
//      hazard edge rejects the shape edge (the engine meets hazard edges only through such boxes,
//      qt_partial_hazard.rs:67-71)
//   16 the containment rule (cd_engine.rs:231-255)
int32_t nv_explain(void* p, const nv_query* q, uint32_t key) {
    const Ctx& c = *(Ctx*)p;
    if (q->item >= c.items.size() || key >= c.hz.size() || !c.hz[key].live) return -1;
    const ItemT& it = c.items[q->item];
    const Haz& h = c.hz[key];
    const float t[4] = {q->cos, q->sin, q->tx, q->ty};
    Shape s;
    place(it, t, s);
    int32_t f = 0;
    if ((int32_t)key == c.exterior && relation(c.cde, s.bb) != R_SURROUNDING) f |= 1;
    if (surrogate_hits(c, it, t, h)) f |= 2;
    for (size_t i = 0; i < s.v.size(); i++)
        for (size_t j = 0; j < h.s.v.size(); j++) {
            const Seg a = s.edge(i), b = h.s.edge(j);
            if (!seg_cross(a, b)) continue;
            const Box eb{std::fmin(b.a.x, b.b.x), std::fmin(b.a.y, b.b.y), std::fmax(b.a.x, b.b.x), std::fmax(b.a.y, b.b.y)};
            // rect.rs:301-345 against the hazard edge's box
            const bool x_no = std::fmax(std::fmin(a.a.x, a.b.x), eb.x0) > std::fmin(std::fmax(a.a.x, a.b.x), eb.x1);
            const bool y_no = std::fmax(std::fmin(a.a.y, a.b.y), eb.y0) > std::fmin(std::fmax(a.a.y, a.b.y), eb.y1);
            bool meets = false;
            if (!(x_no || y_no)) {
                if (box_has(eb, a.a) || box_has(eb, a.b)) {
                    meets = true;
                } else {
                    const float dx = a.b.x - a.a.x, dy = a.b.y - a.a.y;
                    const V2 cs[4] = {{eb.x1, eb.y1}, {eb.x0, eb.y1}, {eb.x0, eb.y0}, {eb.x1, eb.y0}};
                    bool pos = true, neg = true;
                    for (const V2& k : cs) {
                        const float sd = (k.x - a.a.x) * dy - (k.y - a.a.y) * dx;
                        pos = pos && sd > 0.0f;
                        neg = neg && sd < 0.0f;
                    }
                    meets = !(pos || neg);
                }
            }
            f |= meets ? 4 : 8;
        }
    if (contained_hit(s, h)) f |= 16;
    return f;
}

// primitives, for known-answer tests
int32_t nv_fpa_eq(float a, float b) { return approx(a, b) ? 1 : 0; }
int32_t nv_seg_cross(const float* e1, const float* e2) {
    return seg_cross(Seg{V2{e1[0], e1[1]}, V2{e1[2], e1[3]}}, Seg{V2{e2[0], e2[1]}, V2{e2[2], e2[3]}}) ? 1 : 0;
}
int32_t nv_inside(const float* xy, uint32_t nv, float px, float py) {
    Shape s;
    s.v.resize(nv);
    for (uint32_t i = 0; i < nv; i++) s.v[i] = V2{xy[2 * i], xy[2 * i + 1]};
    s.bb = bounds(s.v);
    return inside(s, V2{px, py}) ? 1 : 0;
}

}  // extern "C"
