// Host preparation of item and container shapes: SPolygon::new and the surrogate poles.
//
// These run once per item type (the reference does them in Item::new / Container::new), never per
// query.  Compiled with -ffp-contract=off so that every pole is bit-identical to the reference's.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <deque>
#include <vector>

#include "prep.hpp"
#include "qtree.hpp"

namespace jcde {

static const float PI_F32 = 3.14159265358979323846f;

// simple_polygon.rs:137-150 (shoelace, counter-clockwise positive)
float polygon_area(const Pt* v, size_t n) {
    float sigma = 0.0f;
    for (size_t i = 0; i < n; i++) {
        size_t j = (i + 1) % n;
        sigma += (v[i].y + v[j].y) * (v[i].x - v[j].x);
    }
    return 0.5f * sigma;
}

// convex_hull.rs:31-64 — monotone chain over points stably sorted by x
static float cross3(Pt a, Pt b, Pt c) { return (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x); }
static std::vector<Pt> convex_hull(std::vector<Pt> p) {
    std::stable_sort(p.begin(), p.end(), [](const Pt& a, const Pt& b) { return a.x < b.x; });
    std::vector<Pt> lo, up;
    auto grow = [](std::vector<Pt>& h, Pt q) {
        while (h.size() >= 2 && cross3(h[h.size() - 2], h[h.size() - 1], q) <= 0.0f) h.pop_back();
        h.push_back(q);
    };
    for (const Pt& q : p) grow(lo, q);
    for (auto it = p.rbegin(); it != p.rend(); ++it) grow(up, *it);
    up.pop_back();
    lo.pop_back();
    lo.insert(lo.end(), up.begin(), up.end());
    return lo;
}
// simple_polygon.rs:107-120
static float polygon_diameter(const std::vector<Pt>& v) {
    std::vector<Pt> ch = convex_hull(v);
    float best = 0.0f;
    bool have = false;
    for (size_t i = 0; i < ch.size(); i++)
        for (size_t j = i + 1; j < ch.size(); j++) {
            float dx = ch[i].x - ch[j].x, dy = ch[i].y - ch[j].y;
            float sq = dx * dx + dy * dy;
            if (!have || sq >= best) {
                best = sq;
                have = true;
            }
        }
    return sqrtf(best);
}

namespace {
struct PoiCell {
    int level;
    Box box;
    float radius;
    float distance;
};
}  // namespace

// pole.rs:90-120 (POINode::new)
static PoiCell poi_cell(const Box& b, int level, const Polygon& poly, const std::vector<Disk>& poles) {
    PoiCell n;
    n.box = b;
    n.level = level;
    n.radius = box_diameter(b) / 2.0f;
    Pt c = box_mid(b);
    bool inside = polygon_contains(poly, c);
    if (inside)
        for (const Disk& d : poles)
            if (disk_hits_pt(d, c)) {
                inside = false;
                break;
            }
    float dist = FLT_MAX;
    size_t nv = poly.v.size();
    for (size_t i = 0; i < nv; i++) dist = fmn(dist, sqrtf(seg_sq_dist(Seg{poly.v[i], poly.v[i + 1 == nv ? 0 : i + 1]}, c)));
    for (const Disk& d : poles) dist = fmn(dist, disk_sep_dist(d, c));
    n.distance = inside ? dist : -dist;
    return n;
}

// pole.rs:52-77 (compute_pole): breadth-first branch and bound over a 10-level cell tree
static bool compute_pole(const Polygon& poly, const std::vector<Disk>& poles, Disk* out) {
    std::deque<PoiCell> queue;
    queue.push_back(poi_cell(box_square(poly.bbox), 10, poly, poles));
    bool have = false;
    Disk best{};
    while (!queue.empty()) {
        PoiCell n = queue.front();
        queue.pop_front();
        if (n.distance > (have ? best.r : 0.0f)) {
            best = Disk{box_mid(n.box), n.distance};
            have = true;
        }
        if (n.radius + n.distance > (have ? best.r : 0.0f) && n.level != 0)
            for (int i = 0; i < 4; i++) queue.push_back(poi_cell(box_quadrant(n.box, i), n.level - 1, poly, poles));
    }
    if (have) *out = best;
    return have;
}

int spolygon_new(std::vector<Pt> pts, PreparedPolygon* out, bool with_poi) {
    if (pts.size() < 3) return -1;
    for (size_t i = 0; i < pts.size(); i++)
        for (size_t j = i + 1; j < pts.size(); j++)
            if (pts[i].x == pts[j].x && pts[i].y == pts[j].y) return -1;
    float area = polygon_area(pts.data(), pts.size());
    if (area == 0.0f) return -1;
    if (area < 0.0f) {
        std::reverse(pts.begin(), pts.end());
        area = -area;
    }
    out->diameter = polygon_diameter(pts);
    out->area = area;
    Polygon p;
    p.v = pts;
    p.bbox = bounding_box(pts.data(), pts.size());
    Disk poi{Pt{0.0f, 0.0f}, 0.0f};
    if (with_poi && !compute_pole(p, {}, &poi)) return -1;   // calculate_poi (simple_polygon.rs:152-171)
    out->v = std::move(pts);
    out->bbox = p.bbox;
    out->poi = poi;
    return 0;
}

// close_narrow_concavities (shape_modification.rs:374-478), on the host: each round bridges the
// pair of non-adjacent vertices that eliminates the most vertices among those whose connecting
// edge, shrunk by Edge::scale(0.9999) (edge.rs:39-46), is at most ratio x diameter long, lies
// outside the shape (inflate) or inside it (deflate) at both ends, crosses none of its edges and cuts
// off a chain of negative area; ties keep the first pair in (i, j) order.  The shape is rebuilt by
// SPolygon::new after every bridge (its diameter bounds the next round).
int close_concavities(std::vector<Pt> pts, bool deflate, float ratio, std::vector<Pt>* out) {
    PreparedPolygon shape;
    if (spolygon_new(std::move(pts), &shape, false)) return -1;
    const size_t rounds = shape.v.size();
    for (size_t it = 0; it < rounds; it++) {
        const size_t n = shape.v.size();
        Polygon poly;
        poly.v = shape.v;
        poly.bbox = shape.bbox;
        const float f = 0.9999f;
        size_t best_i = 0, best_j = 0, best_elim = 0;
        bool found = false;
        for (size_t i = 0; i < n; i++) {
            for (size_t j = 0; j < n; j++) {
                if (i == j || (i + 1) % n == j || (j + 1) % n == i) continue;
                const Pt a = shape.v[i], b = shape.v[j];
                const float dx = b.x - a.x, dy = b.y - a.y;
                const Seg c{Pt{a.x - dx * (f - 1.0f) / 2.0f, a.y - dy * (f - 1.0f) / 2.0f},
                            Pt{b.x + dx * (f - 1.0f) / 2.0f, b.y + dy * (f - 1.0f) / 2.0f}};
                const float lx = c.s.x - c.e.x, ly = c.s.y - c.e.y;
                if (sqrtf(lx * lx + ly * ly) > ratio * shape.diameter) continue;
                const bool in_s = polygon_contains(poly, c.s), in_e = polygon_contains(poly, c.e);
                if (deflate ? !(in_s && in_e) : (in_s || in_e)) continue;
                bool crossing = false;
                for (size_t k = 0; k < n && !crossing; k++)
                    crossing = seg_hits_seg(Seg{shape.v[k], shape.v[k + 1 == n ? 0 : k + 1]}, c);
                if (crossing) continue;
                // the chain from i up to (not including) j
                std::vector<Pt> chain;
                for (size_t k = i; k != j; k = k + 1 == n ? 0 : k + 1) chain.push_back(shape.v[k]);
                if (polygon_area(chain.data(), chain.size()) >= 0.0f) continue;
                const size_t elim = j > i ? j - i - 1 : n - i + j - 1;
                if (!found || elim > best_elim) {
                    found = true;
                    best_i = i;
                    best_j = j;
                    best_elim = elim;
                }
            }
        }
        if (!found) break;
        // drop the vertices strictly between best_i and best_j (wrapping), keeping the list's order
        std::vector<Pt> next;
        for (size_t k = 0; k < n; k++) {
            const bool gone = best_j > best_i ? (k > best_i && k < best_j) : (k > best_i || k < best_j);
            if (!gone) next.push_back(shape.v[k]);
        }
        PreparedPolygon rebuilt;
        if (spolygon_new(std::move(next), &rebuilt, false)) return -2;   // the reference panics here
        shape = std::move(rebuilt);
    }
    *out = shape.v;
    return 0;
}

int surrogate_poles(const std::vector<Pt>& v, float area, Disk poi, const PoleLimit* lim, int n_lim,
                    std::vector<Disk>* poles) {
    Polygon p;
    p.v = v;
    p.bbox = bounding_box(v.data(), v.size());
    std::vector<Disk>& all = *poles;
    all.clear();
    all.push_back(poi);
    float total = poi.r * poi.r * PI_F32;
    for (;;) {   // pole.rs:12-47
        Disk next;
        if (!compute_pole(p, all, &next)) return -1;
        total += next.r * next.r * PI_F32;
        all.push_back(next);
        float coverage = total / area;
        bool found = false;
        uint32_t cap = 0;
        for (int i = 0; i < n_lim; i++)
            if (coverage > lim[i].coverage && (!found || lim[i].n < cap)) {
                cap = lim[i].n;
                found = true;
            }
        if (found && all.size() >= cap) break;
        if (all.size() >= 1000) return -2;
    }
    return 0;
}

}  // namespace jcde
