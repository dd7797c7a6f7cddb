// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// A plain C++ restatement of jagua-rs's f32 collision detection engine (crate jagua-rs 0.6.4),
// used by the test-suite, by smoke() and by the CPU-baseline leg of bench.py as the reference the
// product's results are compared with.
// Nothing in the product library links, loads or calls this file.
//
// PARITY UNPINNED: the reference is Rust, no Rust toolchain exists where this is built, and the
// reference ships no golden vectors or known-answer tests for the CDE.  The restatement follows
// the reference line by line (file:line cited at every function) and is itself checked by
// hand-derived known-answer tests (tests/test_oracle_kat.py, tests/test_naive_crosscheck.py) and
// by a tree-free brute-force checker written apart from this file (naive.cpp: every query against
// every hazard edge, no quadtree), which must report the same verdicts and collected sets.
// The FPA tolerance comes from the float-cmp 0.10 crate (not vendored in the reference tree);
// its documented default margin (epsilon = f32::EPSILON, 4 ULPs) is restated in fpa_eq().
//
// Build with -ffp-contract=off and without fast-math: Rust never fuses a*b+c, so neither may we.
#include <algorithm>
#include <array>
#include <functional>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <memory>
#include <thread>
#include <vector>

namespace oracle {

// ------------------------------------------------------------------------------------------
// geometry primitives  (jagua-rs/src/geometry/primitives/*.rs)
// ------------------------------------------------------------------------------------------
struct Point { float x, y; };
struct Edge { Point s, e; };
struct Rect { float x_min, y_min, x_max, y_max; };
struct Circle { Point c; float r; };

static const float PI_F32 = 3.14159265358979323846f;

// util/fpa.rs:18-31 + float-cmp 0.10 `approx_eq!(f32, a, b)` with F32Margin::default()
static inline bool fpa_eq(float a, float b) {
    if (a == b) return true;
    float d = std::fabs(a - b);
    if (d <= FLT_EPSILON) return true;
    int32_t ai, bi;
    std::memcpy(&ai, &a, 4);
    std::memcpy(&bi, &b, 4);
    int32_t diff = (int32_t)((uint32_t)ai - (uint32_t)bi);  // i32::wrapping_sub
    int32_t ad = diff < 0 ? (diff == INT32_MIN ? INT32_MAX : -diff) : diff;  // saturating abs
    return ad <= 4;
}
// FPA's PartialOrd (fpa.rs:25-31): Equal when approx-equal, else the plain f32 ordering.
static inline bool fpa_le(float a, float b) { return fpa_eq(a, b) || a < b; }
static inline bool fpa_ge(float a, float b) { return fpa_eq(a, b) || a > b; }
static inline bool fpa_lt(float a, float b) { return !fpa_eq(a, b) && a < b; }
static inline bool fpa_gt(float a, float b) { return !fpa_eq(a, b) && a > b; }

// Rust f32::min / f32::max ignore a NaN operand, like fminf/fmaxf.
static inline float fmin_(float a, float b) { return std::fmin(a, b); }
static inline float fmax_(float a, float b) { return std::fmax(a, b); }

enum Relation { INTERSECTING = 0, ENCLOSED = 1, SURROUNDING = 2, DISJOINT = 3 };  // geo_enums.rs:10-19

// rect.rs:266-271
static inline bool rect_collides_rect(const Rect& a, const Rect& b) {
    return fmax_(a.x_min, b.x_min) <= fmin_(a.x_max, b.x_max) &&
           fmax_(a.y_min, b.y_min) <= fmin_(a.y_max, b.y_max);
}
// rect.rs:274-279
static inline bool rect_almost_collides_rect(const Rect& a, const Rect& b) {
    return fpa_le(fmax_(a.x_min, b.x_min), fmin_(a.x_max, b.x_max)) &&
           fpa_le(fmax_(a.y_min, b.y_min), fmin_(a.y_max, b.y_max));
}
// rect.rs:46-65
static inline Relation rect_relation_to(const Rect& s, const Rect& o) {
    if (!rect_collides_rect(s, o)) return DISJOINT;
    if (s.x_min <= o.x_min && s.y_min <= o.y_min && s.x_max >= o.x_max && s.y_max >= o.y_max)
        return SURROUNDING;
    if (s.x_min >= o.x_min && s.y_min >= o.y_min && s.x_max <= o.x_max && s.y_max <= o.y_max)
        return ENCLOSED;
    return INTERSECTING;
}
// rect.rs:70-89
static inline Relation rect_almost_relation_to(const Rect& s, const Rect& o) {
    if (!rect_almost_collides_rect(s, o)) return DISJOINT;
    if (fpa_le(s.x_min, o.x_min) && fpa_le(s.y_min, o.y_min) && fpa_ge(s.x_max, o.x_max) &&
        fpa_ge(s.y_max, o.y_max))
        return SURROUNDING;
    if (fpa_ge(s.x_min, o.x_min) && fpa_ge(s.y_min, o.y_min) && fpa_le(s.x_max, o.x_max) &&
        fpa_le(s.y_max, o.y_max))
        return ENCLOSED;
    return INTERSECTING;
}
// rect.rs:282-288
static inline bool rect_collides_point(const Rect& r, Point p) {
    return p.x >= r.x_min && p.x <= r.x_max && p.y >= r.y_min && p.y <= r.y_max;
}
// rect.rs:248-253
static inline Point rect_centroid(const Rect& r) {
    return Point{(r.x_min + r.x_max) / 2.0f, (r.y_min + r.y_max) / 2.0f};
}
static inline float rect_width(const Rect& r) { return r.x_max - r.x_min; }
static inline float rect_height(const Rect& r) { return r.y_max - r.y_min; }
// rect.rs:259-263
static inline float rect_diameter(const Rect& r) {
    float dx = r.x_max - r.x_min;
    float dy = r.y_max - r.y_min;
    return std::sqrt(dx * dx + dy * dy);
}
// rect.rs:93-109
static inline Rect rect_inflate_to_square(const Rect& r) {
    float width = r.x_max - r.x_min;
    float height = r.y_max - r.y_min;
    float dx = 0.0f, dy = 0.0f;
    if (height < width) dy = (width - height) / 2.0f;
    else if (width < height) dx = (height - width) / 2.0f;
    return Rect{r.x_min - dx, r.y_min - dy, r.x_max + dx, r.y_max + dy};
}
// rect.rs:154-161
static inline void rect_corners(const Rect& r, Point c[4]) {
    c[0] = Point{r.x_max, r.y_max};
    c[1] = Point{r.x_min, r.y_max};
    c[2] = Point{r.x_min, r.y_min};
    c[3] = Point{r.x_max, r.y_min};
}
// rect.rs:35-41 (from_diagonal_corners) and rect.rs:141-151 (quadrants)
static inline Rect rect_from_diag(Point a, Point b) {
    return Rect{fmin_(a.x, b.x), fmin_(a.y, b.y), fmax_(a.x, b.x), fmax_(a.y, b.y)};
}
static inline void rect_quadrants(const Rect& r, Rect q[4]) {
    Point mid = rect_centroid(r);
    Point c[4];
    rect_corners(r, c);
    for (int i = 0; i < 4; i++) q[i] = rect_from_diag(c[i], mid);
}
// rect.rs:164-184
static inline void rect_sides(const Rect& r, Edge s[4]) {
    Point c[4];
    rect_corners(r, c);
    s[0] = Edge{c[0], c[1]};
    s[1] = Edge{c[1], c[2]};
    s[2] = Edge{c[2], c[3]};
    s[3] = Edge{c[3], c[0]};
}

// edge.rs:89-103
static inline float edge_x_min(const Edge& e) { return fmin_(e.s.x, e.e.x); }
static inline float edge_y_min(const Edge& e) { return fmin_(e.s.y, e.e.y); }
static inline float edge_x_max(const Edge& e) { return fmax_(e.s.x, e.e.x); }
static inline float edge_y_max(const Edge& e) { return fmax_(e.s.y, e.e.y); }

// rect.rs:301-345  (Rect collides with Edge)
static inline bool rect_collides_edge(const Rect& r, const Edge& e) {
    float e_x_min = edge_x_min(e), e_x_max = edge_x_max(e);
    float e_y_min = edge_y_min(e), e_y_max = edge_y_max(e);
    bool x_no = fmax_(e_x_min, r.x_min) > fmin_(e_x_max, r.x_max);
    bool y_no = fmax_(e_y_min, r.y_min) > fmin_(e_y_max, r.y_max);
    if (x_no || y_no) return false;
    if (rect_collides_point(r, e.s) || rect_collides_point(r, e.e)) return true;
    float s_x = e.s.x, s_y = e.s.y;
    float edge_dx = e.e.x - s_x;
    float edge_dy = e.e.y - s_y;
    Point c[4];
    rect_corners(r, c);
    float sides[4];
    for (int i = 0; i < 4; i++) sides[i] = (c[i].x - s_x) * edge_dy - (c[i].y - s_y) * edge_dx;
    bool all_pos = true, all_neg = true;
    for (int i = 0; i < 4; i++) {
        all_pos = all_pos && (sides[i] > 0.0f);
        all_neg = all_neg && (sides[i] < 0.0f);
    }
    return !(all_pos || all_neg);
}

// edge.rs:63-87
static inline Point closest_point_on_edge(const Edge& e, Point p) {
    float x1 = e.s.x, y1 = e.s.y, x2 = e.e.x, y2 = e.e.y;
    float a = p.x - x1;
    float b = p.y - y1;
    float c = x2 - x1;
    float d = y2 - y1;
    float dot = a * c + b * d;
    float len_sq = c * c + d * d;
    float param = -1.0f;
    if (len_sq != 0.0f) param = dot / len_sq;
    if (param < 0.0f) return Point{x1, y1};
    if (param > 1.0f) return Point{x2, y2};
    return Point{x1 + param * c, y1 + param * d};
}
// edge.rs:152-159
static inline float edge_sq_distance_to_point(const Edge& e, Point p) {
    Point q = closest_point_on_edge(e, p);
    float dx = p.x - q.x, dy = p.y - q.y;
    return dx * dx + dy * dy;
}
// edge.rs:147-150
static inline float edge_distance_to_point(const Edge& e, Point p) {
    return std::sqrt(edge_sq_distance_to_point(e, p));
}

// edge.rs:180-228 (calc_loc = false)
static inline bool edge_intersection(const Edge& e1, const Edge& e2) {
    float x1 = e1.s.x, y1 = e1.s.y, x2 = e1.e.x, y2 = e1.e.y;
    float x3 = e2.s.x, y3 = e2.s.y, x4 = e2.e.x, y4 = e2.e.y;
    {
        float x_min_e1 = fmin_(x1, x2), x_max_e1 = fmax_(x1, x2);
        float y_min_e1 = fmin_(y1, y2), y_max_e1 = fmax_(y1, y2);
        float x_min_e2 = fmin_(x3, x4), x_max_e2 = fmax_(x3, x4);
        float y_min_e2 = fmin_(y3, y4), y_max_e2 = fmax_(y3, y4);
        bool x_no = fmax_(x_min_e1, x_min_e2) > fmin_(x_max_e1, x_max_e2);
        bool y_no = fmax_(y_min_e1, y_min_e2) > fmin_(y_max_e1, y_max_e2);
        if (x_no || y_no) return false;
    }
    float t_nom = (x2 - x4) * (y4 - y3) - (y2 - y4) * (x4 - x3);
    float t_denom = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    float u_nom = (x2 - x4) * (y2 - y1) - (y2 - y4) * (x2 - x1);
    float u_denom = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    if (t_denom == 0.0f || u_denom == 0.0f) return false;
    float t = t_nom / t_denom;
    float u = u_nom / u_denom;
    return (0.0f <= t && t <= 1.0f) && (0.0f <= u && u <= 1.0f);
}

// circle.rs:506-510
static inline bool circle_collides_edge(const Circle& c, const Edge& e) {
    return edge_sq_distance_to_point(e, c.c) <= c.r * c.r;
}
// circle.rs:512-525
static inline bool circle_collides_rect(const Circle& c, const Rect& r) {
    float nx = fmax_(r.x_min, fmin_(c.c.x, r.x_max));
    float ny = fmax_(r.y_min, fmin_(c.c.y, r.y_max));
    float dx = nx - c.c.x, dy = ny - c.c.y;
    return dx * dx + dy * dy <= c.r * c.r;
}
// circle.rs:527-531 with point.rs:282-285 (point.sq_distance_to(center))
static inline bool circle_collides_point(const Circle& c, Point p) {
    float dx = p.x - c.c.x, dy = p.y - c.c.y;
    return dx * dx + dy * dy <= c.r * c.r;
}
// circle.rs:551-560
static inline float circle_separation_distance_point(const Circle& c, Point p) {
    float dx = p.x - c.c.x, dy = p.y - c.c.y;
    float d_center = std::sqrt(dx * dx + dy * dy);
    if (d_center <= c.r) return c.r - d_center;
    return d_center - c.r;
}
// circle.rs:457-459
static inline float circle_area(const Circle& c) { return c.r * c.r * PI_F32; }

// transformation.rs:475-483 (rot_transl_m) + point.rs:259-264 (TRANSFORM_FORMULA).
// The matrix is [[cos, -sin, tx], [sin, cos, ty], [0, 0, 1]].
struct Transform { float cos, sin, tx, ty; };
static inline Point transform_point(const Transform& t, Point p) {
    float m00 = t.cos, m01 = -t.sin, m02 = t.tx;
    float m10 = t.sin, m11 = t.cos, m12 = t.ty;
    float x = m00 * p.x + m01 * p.y + m02 * 1.0f;
    float y = m10 * p.x + m11 * p.y + m12 * 1.0f;
    return Point{x, y};
}

// ------------------------------------------------------------------------------------------
// simple polygon  (simple_polygon.rs)
// ------------------------------------------------------------------------------------------
struct SPolygon {
    std::vector<Point> v;
    Rect bbox;
    float area = 0.0f;
    float diameter = 0.0f;
    Circle poi{};
    size_t n() const { return v.size(); }
    Edge edge(size_t i) const {
        size_t j = (i == v.size() - 1) ? 0 : i + 1;  // simple_polygon.rs:86-93
        return Edge{v[i], v[j]};
    }
};

// simple_polygon.rs:122-133
static Rect generate_bounding_box(const std::vector<Point>& pts) {
    float x_min = FLT_MAX, y_min = FLT_MAX, x_max = -FLT_MAX, y_max = -FLT_MAX;
    for (const Point& p : pts) {
        x_min = fmin_(x_min, p.x);
        y_min = fmin_(y_min, p.y);
        x_max = fmax_(x_max, p.x);
        y_max = fmax_(y_max, p.y);
    }
    return Rect{x_min, y_min, x_max, y_max};
}
// simple_polygon.rs:137-150
static float calculate_area(const std::vector<Point>& pts) {
    float sigma = 0.0f;
    for (size_t i = 0; i < pts.size(); i++) {
        size_t j = (i + 1) % pts.size();
        sigma += (pts[i].y + pts[j].y) * (pts[i].x - pts[j].x);
    }
    return 0.5f * sigma;
}

// simple_polygon.rs:255-292  (ray-cast point in polygon with FPA vertex guard)
struct Counters {
    uint64_t nodes = 0, entries = 0, edge_tests = 0, pip_edges = 0;
};
static thread_local Counters* tl_cnt = nullptr;

static bool poly_collides_point(const SPolygon& poly, Point p) {
    if (!rect_collides_point(poly.bbox, p)) return false;
    Point outside{poly.bbox.x_max + rect_width(poly.bbox), p.y};
    Edge ray{p, outside};
    int n_int = 0;
    for (size_t i = 0; i < poly.n(); i++) {
        Edge e = poly.edge(i);
        if (tl_cnt) tl_cnt->pip_edges++;
        if ((fpa_eq(e.s.y, p.y) && fpa_gt(e.s.x, p.x)) || (fpa_eq(e.e.y, p.y) && fpa_gt(e.e.x, p.x))) {
            if (fpa_lt(e.s.y, p.y) || fpa_lt(e.e.y, p.y)) n_int++;
        } else if (edge_intersection(ray, e)) {
            n_int++;
        }
    }
    return n_int % 2 == 1;
}

// convex_hull.rs:31-64 (monotone chain)
static float cross3(Point a, Point b, Point c) {
    return (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);
}
static void grow_hull(std::vector<Point>& h, Point next) {
    while (h.size() >= 2 && cross3(h[h.size() - 2], h[h.size() - 1], next) <= 0.0f) h.pop_back();
    h.push_back(next);
}
static std::vector<Point> convex_hull_from_points(std::vector<Point> pts) {
    std::stable_sort(pts.begin(), pts.end(), [](const Point& a, const Point& b) { return a.x < b.x; });
    std::vector<Point> lower, upper;
    for (const Point& p : pts) grow_hull(lower, p);
    for (auto it = pts.rbegin(); it != pts.rend(); ++it) grow_hull(upper, *it);
    upper.pop_back();
    lower.pop_back();
    lower.insert(lower.end(), upper.begin(), upper.end());
    return lower;
}
// simple_polygon.rs:107-120
static float calculate_diameter(const std::vector<Point>& pts) {
    std::vector<Point> ch = convex_hull_from_points(pts);
    float best = -1.0f;
    bool have = false;
    for (size_t i = 0; i < ch.size(); i++)
        for (size_t j = i + 1; j < ch.size(); j++) {
            float dx = ch[i].x - ch[j].x, dy = ch[i].y - ch[j].y;
            float sq = dx * dx + dy * dy;
            if (!have || sq >= best) { best = sq; have = true; }
        }
    return std::sqrt(best);
}

// ------------------------------------------------------------------------------------------
// poles  (geometry/fail_fast/pole.rs)
// ------------------------------------------------------------------------------------------
static const int MAX_POI_TREE_DEPTH = 10;  // pole.rs:80

struct POINode {
    int level;
    Rect bbox;
    float radius;
    float distance;
};
// pole.rs:90-120
static POINode poi_node_new(const Rect& bbox, int level, const SPolygon& poly,
                            const std::vector<Circle>& poles) {
    POINode n;
    n.bbox = bbox;
    n.level = level;
    n.radius = rect_diameter(bbox) / 2.0f;
    Point c = rect_centroid(bbox);
    bool inside = poly_collides_point(poly, c);
    if (inside)
        for (const Circle& p : poles)
            if (circle_collides_point(p, c)) { inside = false; break; }
    float d = FLT_MAX;
    for (size_t i = 0; i < poly.n(); i++) d = fmin_(d, edge_distance_to_point(poly.edge(i), c));
    for (const Circle& p : poles) d = fmin_(d, circle_separation_distance_point(p, c));
    n.distance = inside ? d : -d;
    return n;
}
// pole.rs:52-77
static bool compute_pole(const SPolygon& shape, const std::vector<Circle>& poles, Circle* out) {
    Rect sq = rect_inflate_to_square(shape.bbox);
    std::deque<POINode> queue;
    queue.push_back(poi_node_new(sq, MAX_POI_TREE_DEPTH, shape, poles));
    bool have = false;
    Circle best{};
    while (!queue.empty()) {
        POINode node = queue.front();
        queue.pop_front();
        float bd = have ? best.r : 0.0f;
        if (node.distance > bd) {
            best = Circle{rect_centroid(node.bbox), node.distance};
            have = true;
        }
        bd = have ? best.r : 0.0f;
        if (node.radius + node.distance > bd && node.level != 0) {
            Rect q[4];
            rect_quadrants(node.bbox, q);
            for (int i = 0; i < 4; i++) queue.push_back(poi_node_new(q[i], node.level - 1, shape, poles));
        }
    }
    if (have) *out = best;
    return have;
}

struct PoleLimit { uint32_t n; float coverage; };

// pole.rs:12-47
static bool generate_surrogate_poles(const SPolygon& shape, const PoleLimit* limits, int n_limits,
                                     std::vector<Circle>& all) {
    all.clear();
    all.push_back(shape.poi);
    float total = circle_area(shape.poi);
    for (;;) {
        Circle next;
        if (!compute_pole(shape, all, &next)) return false;
        total += circle_area(next);
        all.push_back(next);
        float coverage = total / shape.area;
        bool found = false;
        uint32_t lim = 0;
        for (int i = 0; i < n_limits; i++)
            if (coverage > limits[i].coverage && (!found || limits[i].n < lim)) { lim = limits[i].n; found = true; }
        if (found && all.size() >= lim) break;
        if (all.size() >= 1000) return false;
    }
    return true;
}

// simple_polygon.rs:41-71 (SPolygon::new) including calculate_poi (simple_polygon.rs:152-171)
static bool spolygon_new(std::vector<Point> pts, SPolygon* out) {
    if (pts.size() < 3) return false;
    for (size_t i = 0; i < pts.size(); i++)
        for (size_t j = i + 1; j < pts.size(); j++)
            if (pts[i].x == pts[j].x && pts[i].y == pts[j].y) return false;
    float area = calculate_area(pts);
    if (area == 0.0f) return false;
    if (area < 0.0f) {
        std::reverse(pts.begin(), pts.end());
        area = -area;
    }
    SPolygon sp;
    sp.diameter = calculate_diameter(pts);
    sp.bbox = generate_bounding_box(pts);
    sp.area = area;
    sp.v = pts;
    SPolygon dummy = sp;
    dummy.area = calculate_area(pts);
    dummy.poi = Circle{Point{FLT_MAX, FLT_MAX}, FLT_MAX};
    std::vector<Circle> none;
    if (!compute_pole(dummy, none, &sp.poi)) return false;
    *out = sp;
    return true;
}

// ------------------------------------------------------------------------------------------
// hazards + quadtree  (collision_detection/hazards/*.rs, collision_detection/quadtree/*.rs)
// ------------------------------------------------------------------------------------------
enum EntityKind { PLACED_ITEM = 0, EXTERIOR = 1, HOLE = 2, QUALITY_ZONE = 3 };
enum Scope { SCOPE_INTERIOR = 0, SCOPE_EXTERIOR = 1 };
// hazard.rs:55-62
static inline Scope entity_scope(int kind) { return kind == EXTERIOR ? SCOPE_EXTERIOR : SCOPE_INTERIOR; }

struct Hazard {
    int kind;
    bool dynamic;
    SPolygon shape;
};

enum Presence { P_NONE = 0, P_PARTIAL = 1, P_ENTIRE = 2 };

struct QTHazPartial {
    std::vector<Edge> edges;
    Rect ff_bbox;
};

struct QTHazard {
    Rect qt_bbox;
    uint32_t hkey;
    int kind;
    Presence presence;
    std::shared_ptr<const QTHazPartial> partial;
    size_t n_edges() const { return presence == P_PARTIAL ? partial->edges.size() : 0; }
};

// Filter: HazKeyFilter (filter.rs:13-48) over dense hazard keys; an empty filter is NoFilter.
struct Filter {
    std::vector<uint8_t> ignored;
    bool irrelevant(uint32_t k) const { return k < ignored.size() && ignored[k]; }
};

// Collector: BasicHazardCollector (collector.rs:45-67) keyed by dense hazard keys.
struct Collector {
    std::vector<uint8_t> in;
    std::vector<uint32_t> keys;
    void reset(size_t n) {
        in.assign(n, 0);
        keys.clear();
    }
    bool contains(uint32_t k) const { return in[k] != 0; }
    void insert(uint32_t k) {
        if (!in[k]) {
            in[k] = 1;
            keys.push_back(k);
        }
    }
};

// qt_partial_hazard.rs:20-24
static std::shared_ptr<const QTHazPartial> partial_from_shape(const SPolygon& s) {
    auto p = std::make_shared<QTHazPartial>();
    for (size_t i = 0; i < s.n(); i++) p->edges.push_back(s.edge(i));
    p->ff_bbox = s.bbox;
    return p;
}
// qt_partial_hazard.rs:25-59
static std::shared_ptr<const QTHazPartial> partial_from_parent(const QTHazPartial& parent,
                                                               std::vector<Edge> edges) {
    auto p = std::make_shared<QTHazPartial>();
    if (parent.edges.size() == edges.size()) {
        p->ff_bbox = parent.ff_bbox;
    } else {
        float x_min = INFINITY, y_min = INFINITY, x_max = -INFINITY, y_max = -INFINITY;
        for (const Edge& e : edges) {
            x_min = fmin_(fmin_(x_min, e.s.x), e.e.x);
            y_min = fmin_(fmin_(y_min, e.s.y), e.e.y);
            x_max = fmax_(fmax_(x_max, e.s.x), e.e.x);
            y_max = fmax_(fmax_(y_max, e.s.y), e.e.y);
        }
        if (x_min < x_max && y_min < y_max) p->ff_bbox = Rect{x_min, y_min, x_max, y_max};
        else p->ff_bbox = parent.ff_bbox;
    }
    p->edges = std::move(edges);
    return p;
}

// rect.rs:136
static const int QUADRANT_NEIGHBOR_LAYOUT[4][2] = {{1, 3}, {0, 2}, {1, 3}, {0, 2}};

// qt_hazard.rs:48-167
static void constrict(const QTHazard& h, const Rect quads[4], const std::vector<Hazard*>& hmap,
                      QTHazard out[4]) {
    if (h.presence == P_ENTIRE) {
        for (int i = 0; i < 4; i++) out[i] = h;
        return;
    }
    const SPolygon& shape = hmap[h.hkey]->shape;
    int enclosed = -1;
    for (int i = 0; i < 4; i++)
        if (rect_relation_to(shape.bbox, quads[i]) == ENCLOSED) { enclosed = i; break; }
    if (enclosed >= 0) {
        for (int i = 0; i < 4; i++) {
            out[i] = h;
            out[i].qt_bbox = quads[i];
            if (i != enclosed) { out[i].presence = P_NONE; out[i].partial.reset(); }
        }
        return;
    }
    bool resolved[4] = {false, false, false, false};
    for (int i = 0; i < 4; i++) {
        std::vector<Edge> col;
        for (const Edge& e : h.partial->edges)
            if (rect_collides_edge(quads[i], e)) col.push_back(e);
        if (!col.empty()) {
            out[i] = QTHazard{quads[i], h.hkey, h.kind, P_PARTIAL, partial_from_parent(*h.partial, std::move(col))};
            resolved[i] = true;
        }
    }
    for (int i = 0; i < 4; i++) {
        if (resolved[i]) continue;
        bool none_nb = false, entire_nb = false;
        for (int k = 0; k < 2; k++) {
            int nb = QUADRANT_NEIGHBOR_LAYOUT[i][k];
            if (!resolved[nb]) continue;
            if (out[nb].presence == P_NONE) none_nb = true;
            if (out[nb].presence == P_ENTIRE) entire_nb = true;
        }
        Presence pr;
        if (none_nb && !entire_nb) pr = P_NONE;
        else if (!none_nb && entire_nb) pr = P_ENTIRE;
        else {
            // (true, true) is unreachable in the reference; the neighbour-free case tests the centroid
            bool colliding = poly_collides_point(shape, rect_centroid(quads[i]));
            Scope sc = entity_scope(h.kind);
            if (sc == SCOPE_INTERIOR && colliding) pr = P_ENTIRE;
            else if (sc == SCOPE_EXTERIOR && !colliding) pr = P_ENTIRE;
            else pr = P_NONE;
        }
        out[i] = QTHazard{quads[i], h.hkey, h.kind, pr, nullptr};
        resolved[i] = true;
    }
}

// qt_hazard_vec.rs: vector kept sorted by presence, Entire > Partial > None
struct QTHazardVec {
    std::vector<QTHazard> hz;
    size_t n_active_edges = 0;
    void add(QTHazard h) {
        // qt_hazard_vec.rs:24-43: insertion point from a binary search on descending strength
        size_t pos = 0;
        while (pos < hz.size() && hz[pos].presence >= h.presence) pos++;
        n_active_edges += h.n_edges();
        hz.insert(hz.begin() + pos, std::move(h));
    }
    bool remove(uint32_t k) {
        for (size_t i = 0; i < hz.size(); i++)
            if (hz[i].hkey == k) {
                n_active_edges -= hz[i].n_edges();
                hz.erase(hz.begin() + i);
                return true;
            }
        return false;
    }
    const QTHazard* strongest(const Filter& f) const {
        for (const QTHazard& h : hz) {
            if (tl_cnt) tl_cnt->entries++;
            if (!f.irrelevant(h.hkey)) return &h;
        }
        return nullptr;
    }
    bool no_partial() const {
        for (const QTHazard& h : hz) if (h.presence == P_PARTIAL) return false;
        return true;
    }
};

// qt_traits.rs:144-177 ; returns -1 for no intersection, else the half of e2: 0 first, 1 halfway, 2 second
static inline int edge_intersection_half_e2(const Edge& e1, const Edge& e2) {
    float x1 = e1.s.x, y1 = e1.s.y, x2 = e1.e.x, y2 = e1.e.y;
    float x3 = e2.s.x, y3 = e2.s.y, x4 = e2.e.x, y4 = e2.e.y;
    float t_nom = (x2 - x4) * (y4 - y3) - (y2 - y4) * (x4 - x3);
    float t_denom = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    float u_nom = (x2 - x4) * (y2 - y1) - (y2 - y4) * (x2 - x1);
    float u_denom = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    if (t_denom == 0.0f || u_denom == 0.0f) return -1;
    float t = t_nom / t_denom;
    float u = u_nom / u_denom;
    if ((0.0f <= t && t <= 1.0f) && (0.0f <= u && u <= 1.0f)) {
        if (u > 0.5f) return 0;
        if (u < 0.5f) return 2;
        return 1;
    }
    return -1;
}
// qt_traits.rs:110-140 ; state per quadrant: -1 = undetermined, 0 = false, 1 = true
static inline void half_intersect(const Edge& e1, const Edge& e2, int* const* fst, int nf,
                                  int* const* sec, int ns) {
    bool any_undet = false;
    for (int i = 0; i < nf; i++) any_undet |= (*fst[i] < 0);
    for (int i = 0; i < ns; i++) any_undet |= (*sec[i] < 0);
    if (!any_undet) return;
    int h = edge_intersection_half_e2(e1, e2);
    if (h == 0 || h == 1) for (int i = 0; i < nf; i++) *fst[i] = 1;
    if (h == 1 || h == 2) for (int i = 0; i < ns; i++) *sec[i] = 1;
}
// qt_traits.rs:19-106
static void edge_collides_with_quadrants(const Edge& e, const Rect& r, const Rect* qs, bool out[4]) {
    float e_x_min = edge_x_min(e), e_x_max = edge_x_max(e);
    float e_y_min = edge_y_min(e), e_y_max = edge_y_max(e);
    int c[4];
    for (int i = 0; i < 4; i++) {
        const Rect& q = qs[i];
        bool x_no = fmax_(e_x_min, q.x_min) > fmin_(e_x_max, q.x_max);
        bool y_no = fmax_(e_y_min, q.y_min) > fmin_(e_y_max, q.y_max);
        if (x_no || y_no) c[i] = 0;
        else if (rect_collides_point(q, e.s) || rect_collides_point(q, e.e)) c[i] = 1;
        else c[i] = -1;
    }
    if (c[0] >= 0 && c[1] >= 0 && c[2] >= 0 && c[3] >= 0) {
        for (int i = 0; i < 4; i++) out[i] = c[i] == 1;
        return;
    }
    Point ctr = rect_centroid(r);
    Edge sides[4];
    rect_sides(r, sides);
    const Edge& top = sides[0];
    const Edge& left = sides[1];
    const Edge& bottom = sides[2];
    const Edge& right = sides[3];
    Edge h_bisect{Point{r.x_min, ctr.y}, Point{r.x_max, ctr.y}};
    Edge v_bisect{Point{ctr.x, r.y_min}, Point{ctr.x, r.y_max}};
    {
        int* f[1] = {&c[1]}; int* s[1] = {&c[2]};
        half_intersect(e, left, f, 1, s, 1);
    }
    {
        int* f[1] = {&c[3]}; int* s[1] = {&c[0]};
        half_intersect(e, right, f, 1, s, 1);
    }
    {
        int* f[1] = {&c[0]}; int* s[1] = {&c[1]};
        half_intersect(e, top, f, 1, s, 1);
    }
    {
        int* f[1] = {&c[2]}; int* s[1] = {&c[3]};
        half_intersect(e, bottom, f, 1, s, 1);
    }
    {
        int* f[2] = {&c[1], &c[2]}; int* s[2] = {&c[0], &c[3]};
        half_intersect(e, h_bisect, f, 2, s, 2);
    }
    {
        int* f[2] = {&c[2], &c[3]}; int* s[2] = {&c[0], &c[1]};
        half_intersect(e, v_bisect, f, 2, s, 2);
    }
    for (int i = 0; i < 4; i++) out[i] = c[i] == 1;
}

// Queryable entities: Edge and Circle (qt_traits.rs:9-13, 280-283)
static inline bool q_collides_edge(const Edge& q, const Edge& e) { return edge_intersection(q, e); }
static inline bool q_collides_edge(const Circle& q, const Edge& e) { return circle_collides_edge(q, e); }
static inline bool q_collides_rect(const Edge& q, const Rect& r) { return rect_collides_edge(r, q); }
static inline bool q_collides_rect(const Circle& q, const Rect& r) { return circle_collides_rect(q, r); }
static inline void q_quadrants(const Edge& q, const Rect& r, const Rect* qs, bool out[4]) {
    edge_collides_with_quadrants(q, r, qs, out);
}
static inline void q_quadrants(const Circle& q, const Rect&, const Rect* qs, bool out[4]) {
    for (int i = 0; i < 4; i++) out[i] = circle_collides_rect(q, qs[i]);
}

// qt_partial_hazard.rs:67-71
template <class T>
static bool partial_collides(const QTHazPartial& p, const T& q) {
    if (!q_collides_rect(q, p.ff_bbox)) return false;
    for (const Edge& e : p.edges) {
        if (tl_cnt) tl_cnt->edge_tests++;
        if (q_collides_edge(q, e)) return true;
    }
    return false;
}

struct QTNode {
    uint8_t level;
    Rect bbox;
    std::unique_ptr<QTNode[]> children;  // 4 children or null
    QTHazardVec hazards;
    uint8_t cd_threshold;

    QTNode(uint8_t lvl, Rect b, uint8_t cdt) : level(lvl), bbox(b), cd_threshold(cdt) {}
    QTNode() : level(0), bbox{0, 0, 0, 0}, cd_threshold(0) {}

    void register_to_children(const QTHazard& h, const std::vector<Hazard*>& hmap) {
        Rect qb[4];
        for (int i = 0; i < 4; i++) qb[i] = children[i].bbox;
        QTHazard ch[4];
        constrict(h, qb, hmap, ch);
        for (int i = 0; i < 4; i++)
            if (ch[i].presence != P_NONE) children[i].register_hazard(ch[i], hmap);
    }

    // qt_node.rs:38-81
    void register_hazard(const QTHazard& h, const std::vector<Hazard*>& hmap) {
        if (!children && level > 0 && h.presence == P_PARTIAL) {
            Rect q[4];
            rect_quadrants(bbox, q);
            children.reset(new QTNode[4]);
            for (int i = 0; i < 4; i++) {
                children[i].level = level - 1;
                children[i].bbox = q[i];
                children[i].cd_threshold = cd_threshold;
            }
            for (const QTHazard& old : hazards.hz) register_to_children(old, hmap);
        }
        if (children) register_to_children(h, hmap);
        hazards.add(h);
    }

    // qt_node.rs:83-94
    void deregister_hazard(uint32_t k) {
        bool modified = hazards.remove(k);
        if (modified) {
            if (hazards.no_partial()) children.reset();
            else if (children)
                for (int i = 0; i < 4; i++) children[i].deregister_hazard(k);
        }
    }

    // qt_node.rs:99-147
    template <class T>
    bool collides(const T& q, const Filter& f) const {
        if (tl_cnt) tl_cnt->nodes++;
        const QTHazard* s = hazards.strongest(f);
        if (!s) return false;
        if (s->presence == P_NONE) return false;
        if (s->presence == P_ENTIRE) return true;
        if (children) {
            Rect qs[4];
            for (int i = 0; i < 4; i++) qs[i] = children[i].bbox;
            bool cq[4];
            q_quadrants(q, bbox, qs, cq);
            for (int i = 0; i < 4; i++)
                if (cq[i] && children[i].collides(q, f)) return true;
            return false;
        }
        for (const QTHazard& h : hazards.hz) {
            if (tl_cnt) tl_cnt->entries++;
            if (f.irrelevant(h.hkey)) continue;
            if (h.presence == P_PARTIAL && partial_collides(*h.partial, q)) return true;
        }
        return false;
    }

    // qt_node.rs:151-191
    template <class T>
    void collect_collisions(const T& q, Collector& c) const {
        if (tl_cnt) tl_cnt->nodes++;
        bool now = hazards.n_active_edges <= (size_t)cd_threshold;
        if (children && !now) {
            Rect qs[4];
            for (int i = 0; i < 4; i++) qs[i] = children[i].bbox;
            bool cq[4];
            q_quadrants(q, bbox, qs, cq);
            for (int i = 0; i < 4; i++)
                if (cq[i]) children[i].collect_collisions(q, c);
        } else {
            for (const QTHazard& h : hazards.hz) {
                if (tl_cnt) tl_cnt->entries++;
                if (c.contains(h.hkey)) continue;
                if (h.presence == P_ENTIRE) c.insert(h.hkey);
                else if (h.presence == P_PARTIAL && partial_collides(*h.partial, q)) c.insert(h.hkey);
            }
        }
    }
};

// ------------------------------------------------------------------------------------------
// items (entities/item.rs) — shape + surrogate (fail_fast/sp_surrogate.rs)
// ------------------------------------------------------------------------------------------
struct Item {
    SPolygon shape;
    std::vector<Circle> poles;  // all surrogate poles
    uint32_t n_ff_poles;
    std::vector<Edge> piers;    // ff piers
};

// ------------------------------------------------------------------------------------------
// CDEngine  (collision_detection/cd_engine.rs)
// ------------------------------------------------------------------------------------------
struct Engine {
    QTNode root;
    std::vector<Hazard*> hmap;          // slot -> hazard (null when free)
    std::vector<uint32_t> free_slots;   // LIFO free list (slotmap reuses the last freed slot)
    std::vector<Item> items;
    int32_t hkey_exterior = -1;

    Engine(uint8_t depth, uint8_t cdt, Rect bbox) : root(depth, bbox, cdt) {}
    ~Engine() {
        for (Hazard* h : hmap) delete h;
    }

    // cd_engine.rs:59-70 (and the static-hazard loop of cd_engine.rs:34-56)
    uint32_t register_hazard(Hazard* hz) {
        uint32_t k;
        if (!free_slots.empty()) {
            k = free_slots.back();
            free_slots.pop_back();
            hmap[k] = hz;
        } else {
            k = (uint32_t)hmap.size();
            hmap.push_back(hz);
        }
        if (hz->kind == EXTERIOR && hkey_exterior < 0) hkey_exterior = (int32_t)k;
        QTHazard qh{root.bbox, k, hz->kind, P_PARTIAL, partial_from_shape(hz->shape)};  // qt_hazard.rs:36-43
        root.register_hazard(qh, hmap);
        return k;
    }
    // cd_engine.rs:87-96
    bool deregister_hazard(uint32_t k) {
        if (k >= hmap.size() || !hmap[k]) return false;
        root.deregister_hazard(k);
        if ((int32_t)k == hkey_exterior) hkey_exterior = -1;
        delete hmap[k];
        hmap[k] = nullptr;
        free_slots.push_back(k);
        return true;
    }

    Rect bbox() const { return root.bbox; }

    // cd_engine.rs:314-327
    const QTNode* get_virtual_root(const Rect& b) const {
        const QTNode* v = &root;
        while (v->children) {
            const QTNode* next = nullptr;
            for (int i = 0; i < 4; i++)
                if (rect_relation_to(v->children[i].bbox, b) == SURROUNDING) { next = &v->children[i]; break; }
            if (!next) break;
            v = next;
        }
        return v;
    }

    // cd_engine.rs:231-255
    bool detect_containment_collision(const SPolygon& shape, const SPolygon& haz_shape, int kind) const {
        Relation rel = rect_almost_relation_to(haz_shape.bbox, shape.bbox);
        bool contained = false;
        if (rel == SURROUNDING) contained = poly_collides_point(haz_shape, shape.poi.c);
        else if (rel == ENCLOSED) contained = poly_collides_point(shape, haz_shape.poi.c);
        Scope sc = entity_scope(kind);
        return (sc == SCOPE_INTERIOR && contained) || (sc == SCOPE_EXTERIOR && !contained);
    }

    // cd_engine.rs:160-197
    bool detect_poly_collision(const SPolygon& shape, const Filter& f) const {
        if (rect_relation_to(bbox(), shape.bbox) != SURROUNDING) return true;
        const QTNode* v = get_virtual_root(shape.bbox);
        for (size_t i = 0; i < shape.n(); i++)
            if (v->collides(shape.edge(i), f)) return true;
        for (const QTHazard& h : v->hazards.hz) {
            // None is never stored.  An Entire entry can only survive the edge loop when the filter
            // ignores it; the reference then hits `unreachable!` (cd_engine.rs:179) before its own
            // filter check — here the ignored hazard is skipped, which is what the filter asks for.
            if (h.presence != P_PARTIAL) continue;
            if (f.irrelevant(h.hkey)) continue;
            if (detect_containment_collision(shape, hmap[h.hkey]->shape, h.kind)) return true;
        }
        return false;
    }

    // cd_engine.rs:204-223
    bool detect_surrogate_collision(const Item& it, const Transform& t, const Filter& f) const {
        for (uint32_t i = 0; i < it.n_ff_poles; i++) {
            Circle c{transform_point(t, it.poles[i].c), it.poles[i].r};
            if (root.collides(c, f)) return true;
        }
        for (const Edge& p : it.piers) {
            Edge e{transform_point(t, p.s), transform_point(t, p.e)};
            if (root.collides(e, f)) return true;
        }
        return false;
    }

    // cd_engine.rs:261-289
    void collect_poly_collisions(const SPolygon& shape, Collector& c) const {
        if (rect_relation_to(bbox(), shape.bbox) != SURROUNDING && hkey_exterior >= 0)
            c.insert((uint32_t)hkey_exterior);
        const QTNode* v = get_virtual_root(shape.bbox);
        for (size_t i = 0; i < shape.n(); i++) v->collect_collisions(shape.edge(i), c);
        for (const QTHazard& h : v->hazards.hz) {
            if (h.presence != P_PARTIAL) continue;
            if (c.contains(h.hkey)) continue;
            if (detect_containment_collision(shape, hmap[h.hkey]->shape, h.kind)) c.insert(h.hkey);
        }
    }

    // cd_engine.rs:296-310
    void collect_surrogate_collisions(const Item& it, const Transform& t, Collector& c) const {
        for (uint32_t i = 0; i < it.n_ff_poles; i++) {
            Circle cc{transform_point(t, it.poles[i].c), it.poles[i].r};
            root.collect_collisions(cc, c);
        }
        for (const Edge& p : it.piers) {
            Edge e{transform_point(t, p.s), transform_point(t, p.e)};
            root.collect_collisions(e, c);
        }
    }

    // simple_polygon.rs:226-253 (transform_from): vertices, poi, bbox
    void transform_item(const Item& it, const Transform& t, SPolygon& buf) const {
        buf.v.resize(it.shape.n());
        for (size_t i = 0; i < it.shape.n(); i++) buf.v[i] = transform_point(t, it.shape.v[i]);
        buf.poi = Circle{transform_point(t, it.shape.poi.c), it.shape.poi.r};
        buf.bbox = generate_bounding_box(buf.v);
        buf.area = it.shape.area;
        buf.diameter = it.shape.diameter;
    }

    // lbf/benches/ci_bench.rs:111-119 : collision = surrogate hit || polygon hit
    bool detect_query(uint32_t item, const Transform& t, const Filter& f, SPolygon& buf) const {
        const Item& it = items[item];
        if (detect_surrogate_collision(it, t, f)) return true;
        transform_item(it, t, buf);
        return detect_poly_collision(buf, f);
    }
    // lbf/benches/ci_bench.rs:56-68 : surrogate collect, then polygon collect, same collector.
    // A user filter is applied as the reference's collector-as-filter (filter.rs:69-76): keys are
    // pre-seeded into the collector and stripped from the result.
    void collect_query(uint32_t item, const Transform& t, const Filter& f, SPolygon& buf, Collector& c) const {
        const Item& it = items[item];
        c.reset(hmap.size());
        for (size_t k = 0; k < f.ignored.size() && k < hmap.size(); k++)
            if (f.ignored[k]) c.in[k] = 1;
        collect_surrogate_collisions(it, t, c);
        transform_item(it, t, buf);
        collect_poly_collisions(buf, c);
        std::sort(c.keys.begin(), c.keys.end());
    }
};

// ------------------------------------------------------------------------------------------
// canonical tree dump (test helper): DFS pre-order, hazards sorted by key, edges sorted
// ------------------------------------------------------------------------------------------
static inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static void dump_rect(std::vector<uint32_t>& o, const Rect& r) {
    o.push_back(fbits(r.x_min)); o.push_back(fbits(r.y_min));
    o.push_back(fbits(r.x_max)); o.push_back(fbits(r.y_max));
}
static void dump_node(const QTNode& n, std::vector<uint32_t>& o) {
    o.push_back(n.level);
    o.push_back(n.children ? 1u : 0u);
    o.push_back((uint32_t)n.hazards.hz.size());
    o.push_back((uint32_t)n.hazards.n_active_edges);
    dump_rect(o, n.bbox);
    std::vector<const QTHazard*> hs;
    for (const QTHazard& h : n.hazards.hz) hs.push_back(&h);
    std::sort(hs.begin(), hs.end(), [](const QTHazard* a, const QTHazard* b) { return a->hkey < b->hkey; });
    for (const QTHazard* h : hs) {
        o.push_back(h->hkey);
        o.push_back((uint32_t)h->presence);
        if (h->presence == P_PARTIAL) {
            dump_rect(o, h->partial->ff_bbox);
            std::vector<std::array<uint32_t, 4>> es;
            for (const Edge& e : h->partial->edges)
                es.push_back({fbits(e.s.x), fbits(e.s.y), fbits(e.e.x), fbits(e.e.y)});
            std::sort(es.begin(), es.end());
            o.push_back((uint32_t)es.size());
            for (auto& e : es) o.insert(o.end(), e.begin(), e.end());
        }
    }
    if (n.children)
        for (int i = 0; i < 4; i++) dump_node(n.children[i], o);
}

// ------------------------------------------------------------------------------------------
// shape simplification  (geometry/shape_modification.rs:48-328)
// ------------------------------------------------------------------------------------------
enum CornerType { CORNER_CONCAVE, CORNER_COLLINEAR, CORNER_CONVEX };
struct Corner { size_t a, b, c; };   // shape_modification.rs:296-308 (left-hand side of a-b-c)
enum CandKind { CAND_CONCAVE, CAND_CONVEX_CONVEX, CAND_COLLINEAR };
struct Candidate { CandKind kind; Corner c1, c2; };

// shape_modification.rs:317-327
static CornerType corner_type(Point p1, Point p2, Point p3) {
    float ax = p2.x - p1.x, ay = p2.y - p1.y;
    float bx = p3.x - p1.x, by = p3.y - p1.y;
    float cross = ax * by - ay * bx;
    if (cross < 0.0f) return CORNER_CONCAVE;
    if (cross == 0.0f) return CORNER_COLLINEAR;
    return CORNER_CONVEX;   // NaN panics in the reference (`expect`); not reached for valid shapes
}

// shape_modification.rs:248-283 (calculate_intersection_in_front)
static bool intersection_in_front(const Edge& l1, const Edge& l2, Point* out) {
    float x1 = l1.s.x, y1 = l1.s.y, x2 = l1.e.x, y2 = l1.e.y;
    float x3 = l2.s.x, y3 = l2.s.y, x4 = l2.e.x, y4 = l2.e.y;
    float t_nom = (x2 - x4) * (y4 - y3) - (y2 - y4) * (x4 - x3);
    float t_denom = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    float u_nom = (x2 - x4) * (y2 - y1) - (y2 - y4) * (x2 - x1);
    float u_denom = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    float t = t_denom != 0.0f ? t_nom / t_denom : 0.0f;
    float u = u_denom != 0.0f ? u_nom / u_denom : 0.0f;
    if (t < 0.0f && u < 0.0f) {
        *out = Point{x2 + t * (x1 - x2), y2 + t * (y1 - y2)};
        return true;
    }
    return false;
}

// shape_modification.rs:234-246
static bool replacing_vertex(const std::vector<Point>& s, const Corner& c1, const Corner& c2, Point* out) {
    return intersection_in_front(Edge{s[c1.a], s[c1.b]}, Edge{s[c2.c], s[c2.b]}, out);
}

static float triangle_area_abs(Point p0, Point p1, Point p2) {
    float x0 = p0.x, y0 = p0.y, x1 = p1.x, y1 = p1.y, x2 = p2.x, y2 = p2.y;
    float area = (x0 * y1 + x1 * y2 + x2 * y0 - x0 * y2 - x1 * y0 - x2 * y1) / 2.0f;
    return std::fabs(area);
}

// shape_modification.rs:146-174 — INFINITY stands for the Err of an invalid convex-convex candidate
static float area_delta(const std::vector<Point>& s, const Candidate& c) {
    switch (c.kind) {
        case CAND_COLLINEAR: return 0.0f;
        case CAND_CONCAVE: return triangle_area_abs(s[c.c1.a], s[c.c1.b], s[c.c1.c]);
        default: {
            Point v;
            if (!replacing_vertex(s, c.c1, c.c2, &v)) return INFINITY;
            return triangle_area_abs(s[c.c1.b], v, s[c.c2.b]);
        }
    }
}

static bool same_point(Point a, Point b) { return a.x == b.x && a.y == b.y; }

// shape_modification.rs:176-207
static bool candidate_valid(const std::vector<Point>& s, const Candidate& c) {
    const size_t n = s.size();
    if (c.kind == CAND_COLLINEAR) return true;
    std::vector<Edge> news;
    std::vector<Point> affected;
    if (c.kind == CAND_CONCAVE) {
        news.push_back(Edge{s[c.c1.a], s[c.c1.c]});
        affected = {s[c.c1.a], s[c.c1.b], s[c.c1.c]};
    } else {
        Point v;
        if (!replacing_vertex(s, c.c1, c.c2, &v)) return false;
        news.push_back(Edge{s[c.c1.a], v});
        news.push_back(Edge{v, s[c.c2.c]});
        affected = {s[c.c1.b], s[c.c1.a], s[c.c2.b], s[c.c2.c]};
    }
    for (size_t i = 0; i < n; i++) {
        Edge l{s[i], s[(i + 1) % n]};
        bool touches = false;
        for (const Point& p : affected) touches = touches || same_point(p, l.s) || same_point(p, l.e);
        if (touches) continue;
        for (const Edge& ne : news)
            if (edge_intersection(l, ne)) return false;
    }
    return true;
}

// shape_modification.rs:217-232
static std::vector<Point> execute_candidate(const std::vector<Point>& s, const Candidate& c) {
    std::vector<Point> p = s;
    if (c.kind != CAND_CONVEX_CONVEX) {
        p.erase(p.begin() + c.c1.b);
    } else {
        Point v;
        replacing_vertex(s, c.c1, c.c2, &v);
        p.erase(p.begin() + c.c1.b);
        size_t other = c.c1.b < c.c2.b ? c.c2.b - 1 : c.c2.b;
        p.erase(p.begin() + other);
        p.insert(p.begin() + other, v);
    }
    return p;
}

// simplify_shape (shape_modification.rs:48-144) up to its final SPolygon::new: the simplified
// vertices.  deflate selects ShapeModifyMode::Deflate.
static std::vector<Point> simplify_shape(const std::vector<Point>& shape, float shape_area, bool deflate,
                                         float max_area_change_ratio) {
    std::vector<Point> ref = shape;
    for (size_t it = 0; it < shape.size(); it++) {
        const size_t n = ref.size();
        if (n < 4) break;
        std::vector<Corner> corners(n);
        for (size_t i = 0; i < n; i++) corners[i] = Corner{(i + n - 1) % n, i, (i + 1) % n};
        if (deflate) {
            std::reverse(corners.begin(), corners.end());
            for (Corner& c : corners) std::swap(c.a, c.c);
        }
        auto type_of = [&](const Corner& c) { return corner_type(ref[c.a], ref[c.b], ref[c.c]); };
        std::vector<Candidate> cands;
        Corner prev = corners.back();
        CornerType prev_t = type_of(prev);
        for (const Corner& c : corners) {
            CornerType t = type_of(c);
            if (t == CORNER_CONCAVE) cands.push_back(Candidate{CAND_CONCAVE, c, c});
            else if (t == CORNER_COLLINEAR) cands.push_back(Candidate{CAND_COLLINEAR, c, c});
            else if (prev_t == CORNER_CONVEX) cands.push_back(Candidate{CAND_CONVEX_CONVEX, prev, c});
            prev = c;
            prev_t = t;
        }
        // sorted_by_cached_key(OrderedFloat(delta)) is a stable sort; OrderedFloat puts NaN last
        std::vector<std::pair<float, size_t>> keyed(cands.size());
        for (size_t k = 0; k < cands.size(); k++) keyed[k] = {area_delta(ref, cands[k]), k};
        auto key_less = [](float a, float b) {
            if (std::isnan(a)) return false;
            if (std::isnan(b)) return true;
            return a < b;
        };
        std::stable_sort(keyed.begin(), keyed.end(),
                         [&](const std::pair<float, size_t>& x, const std::pair<float, size_t>& y) { return key_less(x.first, y.first); });
        const Candidate* best = nullptr;
        for (const auto& kk : keyed)
            if (candidate_valid(ref, cands[kk.second])) {
                best = &cands[kk.second];
                break;
            }
        if (!best) break;
        std::vector<Point> next = execute_candidate(ref, *best);
        float next_area = calculate_area(next);
        float delta = std::fabs(next_area - shape_area) / shape_area;
        if (delta <= max_area_change_ratio) ref = next;
        else break;
    }
    return ref;
}

// close_narrow_concavities (shape_modification.rs:374-478): repeatedly bridge the pair of
// non-adjacent vertices whose (0.9999-scaled) connecting edge is shorter than ratio x diameter,
// stays outside (Inflate) or inside (Deflate) the shape, crosses none of its edges and cuts off a
// negative-area chain; the pair eliminating the most vertices wins (the first on ties).
static std::vector<Point> close_narrow_concavities(std::vector<Point> pts, bool deflate, float ratio) {
    SPolygon shape;
    if (!spolygon_new(pts, &shape)) return pts;
    const size_t rounds = shape.v.size();
    for (size_t it = 0; it < rounds; it++) {
        const size_t n = shape.v.size();
        auto elim = [n](size_t i, size_t j) { return j > i ? j - i - 1 : n - i + j - 1; };
        bool have = false;
        size_t bi = 0, bj = 0;
        for (size_t i = 0; i < n; i++) {
            for (size_t j = 0; j < n; j++) {
                if (i == j || (i + 1) % n == j || (j + 1) % n == i) continue;
                const Point a = shape.v[i], b = shape.v[j];
                // Edge::scale(0.9999) (edge.rs:39-46)
                const float f = 0.9999f;
                const float dx = b.x - a.x, dy = b.y - a.y;
                const Point s{a.x - dx * (f - 1.0f) / 2.0f, a.y - dy * (f - 1.0f) / 2.0f};
                const Point e{b.x + dx * (f - 1.0f) / 2.0f, b.y + dy * (f - 1.0f) / 2.0f};
                const float ex = s.x - e.x, ey = s.y - e.y;
                const float len = std::sqrt(ex * ex + ey * ey);   // Point::distance_to (point.rs:45-47)
                if (len > ratio * shape.diameter) continue;
                const bool s_in = poly_collides_point(shape, s), e_in = poly_collides_point(shape, e);
                if (!deflate && (s_in || e_in)) continue;
                if (deflate && !(s_in && e_in)) continue;
                const Edge c{s, e};
                bool crosses = false;
                for (size_t k = 0; k < n && !crosses; k++) crosses = edge_intersection(shape.edge(k), c);
                if (crosses) continue;
                std::vector<Point> sub;
                if (j > i) sub.assign(shape.v.begin() + i, shape.v.begin() + j);
                else {
                    sub.assign(shape.v.begin() + i, shape.v.end());
                    sub.insert(sub.end(), shape.v.begin(), shape.v.begin() + j);
                }
                if (calculate_area(sub) >= 0.0f) continue;
                if (!have || elim(i, j) > elim(bi, bj)) {
                    have = true;
                    bi = i;
                    bj = j;
                }
            }
        }
        if (!have) break;
        std::vector<Point> r = shape.v;
        const long start = (long)bi + 1, end = (long)bj - 1;
        if (start <= end) {
            r.erase(r.begin() + start, r.begin() + end + 1);
        } else {
            if ((size_t)start < n) r.erase(r.begin() + start, r.end());
            if (end >= 0) r.erase(r.begin(), r.begin() + end + 1);
        }
        SPolygon next;
        if (!spolygon_new(r, &next)) break;   // the reference panics here (expect)
        shape = next;
    }
    return shape.v;
}

}  // namespace oracle

// ==========================================================================================
// C API for the test-suite (ctypes)
// ==========================================================================================
using namespace oracle;

extern "C" {

#pragma pack(push, 1)
struct or_query { uint32_t item; float cos, sin, tx, ty; };
#pragma pack(pop)

void* or_engine_new(uint8_t depth, uint8_t cd_threshold, const float* bbox4) {
    return new Engine(depth, cd_threshold, Rect{bbox4[0], bbox4[1], bbox4[2], bbox4[3]});
}
void or_engine_free(void* e) { delete (Engine*)e; }

static Filter make_filter(const uint32_t* ids, uint32_t n, size_t cap) {
    Filter f;
    if (n) {
        size_t m = cap;
        for (uint32_t i = 0; i < n; i++) m = std::max<size_t>(m, ids[i] + 1);
        f.ignored.assign(m, 0);
        for (uint32_t i = 0; i < n; i++) f.ignored[ids[i]] = 1;
    }
    return f;
}

// Registers a hazard whose shape (vertices in the given order, poi) is already final.
// bbox is recomputed from the vertices (simple_polygon.rs:122-133). Returns the hazard key.
int32_t or_register_hazard(void* ep, int32_t kind, int32_t dynamic, const float* xy, uint32_t nv,
                           const float* poi3) {
    Engine* e = (Engine*)ep;
    Hazard* h = new Hazard();
    h->kind = kind;
    h->dynamic = dynamic != 0;
    h->shape.v.resize(nv);
    for (uint32_t i = 0; i < nv; i++) h->shape.v[i] = Point{xy[2 * i], xy[2 * i + 1]};
    h->shape.bbox = generate_bounding_box(h->shape.v);
    h->shape.poi = Circle{Point{poi3[0], poi3[1]}, poi3[2]};
    h->shape.area = calculate_area(h->shape.v);
    return (int32_t)e->register_hazard(h);
}
int32_t or_deregister_hazard(void* ep, uint32_t k) { return ((Engine*)ep)->deregister_hazard(k) ? 0 : -1; }

int32_t or_add_item(void* ep, const float* xy, uint32_t nv, const float* poi3, const float* poles_xyr,
                    uint32_t n_poles, uint32_t n_ff_poles, const float* piers4, uint32_t n_piers) {
    Engine* e = (Engine*)ep;
    Item it;
    it.shape.v.resize(nv);
    for (uint32_t i = 0; i < nv; i++) it.shape.v[i] = Point{xy[2 * i], xy[2 * i + 1]};
    it.shape.bbox = generate_bounding_box(it.shape.v);
    it.shape.poi = Circle{Point{poi3[0], poi3[1]}, poi3[2]};
    it.shape.area = calculate_area(it.shape.v);
    for (uint32_t i = 0; i < n_poles; i++)
        it.poles.push_back(Circle{Point{poles_xyr[3 * i], poles_xyr[3 * i + 1]}, poles_xyr[3 * i + 2]});
    it.n_ff_poles = std::min(n_ff_poles, n_poles);
    for (uint32_t i = 0; i < n_piers; i++)
        it.piers.push_back(Edge{Point{piers4[4 * i], piers4[4 * i + 1]}, Point{piers4[4 * i + 2], piers4[4 * i + 3]}});
    e->items.push_back(std::move(it));
    return (int32_t)e->items.size() - 1;
}

static void run_threads(uint64_t n, int n_threads, const std::function<void(uint64_t, uint64_t, int)>& fn) {
    if (n_threads <= 1 || n < 64) {
        fn(0, n, 0);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; t++) {
        uint64_t a = n * t / n_threads, b = n * (t + 1) / n_threads;
        th.emplace_back(fn, a, b, t);
    }
    for (auto& x : th) x.join();
}

// Batch detect: verdict[i] = 1 when query i collides (surrogate || polygon).  When counts is
// non-null, the algorithmic work per query is accumulated into counts[0..4) (nodes visited,
// node-hazard entries scanned, hazard edges tested, PIP edges) — used for the roofline bytes.
void or_detect_batch(void* ep, const or_query* q, uint64_t n, const uint32_t* filt, uint32_t n_filt,
                     uint8_t* out, int32_t n_threads, uint64_t* counts, int32_t mode) {
    Engine* e = (Engine*)ep;
    Filter f = make_filter(filt, n_filt, e->hmap.size());
    std::vector<Counters> cs(std::max(1, n_threads));
    run_threads(n, n_threads, [&](uint64_t a, uint64_t b, int tid) {
        SPolygon buf;
        tl_cnt = counts ? &cs[tid] : nullptr;
        for (uint64_t i = a; i < b; i++) {
            Transform t{q[i].cos, q[i].sin, q[i].tx, q[i].ty};
            if (q[i].item >= e->items.size()) { out[i] = 2; continue; }
            if (mode == 1) out[i] = e->detect_surrogate_collision(e->items[q[i].item], t, f) ? 1 : 0;
            else if (mode == 4) {   // the verdict with the pass that decided it: 1 surrogate, 3 polygon, 0 free
                const Item& it = e->items[q[i].item];
                if (e->detect_surrogate_collision(it, t, f)) {
                    out[i] = 1;
                } else {
                    e->transform_item(it, t, buf);
                    out[i] = e->detect_poly_collision(buf, f) ? 3 : 0;
                }
            } else if (mode == 2) {
                e->transform_item(e->items[q[i].item], t, buf);
                out[i] = e->detect_poly_collision(buf, f) ? 1 : 0;
            } else out[i] = e->detect_query(q[i].item, t, f, buf) ? 1 : 0;
        }
        tl_cnt = nullptr;
    });
    if (counts) {
        for (auto& c : cs) {
            counts[0] += c.nodes; counts[1] += c.entries; counts[2] += c.edge_tests; counts[3] += c.pip_edges;
        }
    }
}

// Batch collect: counts[i] = number of colliding hazards of query i; ids holds the sorted keys
// of each query back to back (CSR, offsets = exclusive prefix sum of counts).  Returns the total
// number of ids, or -(needed) when ids_cap is too small (nothing written to ids then).
int64_t or_collect_batch(void* ep, const or_query* q, uint64_t n, const uint32_t* filt, uint32_t n_filt,
                         uint32_t* counts, uint32_t* ids, uint64_t ids_cap, int32_t n_threads) {
    Engine* e = (Engine*)ep;
    Filter f = make_filter(filt, n_filt, e->hmap.size());
    std::vector<std::vector<uint32_t>> per(n);
    run_threads(n, n_threads, [&](uint64_t a, uint64_t b, int) {
        SPolygon buf;
        Collector c;
        for (uint64_t i = a; i < b; i++) {
            Transform t{q[i].cos, q[i].sin, q[i].tx, q[i].ty};
            e->collect_query(q[i].item, t, f, buf, c);
            per[i] = c.keys;
        }
    });
    uint64_t total = 0;
    for (uint64_t i = 0; i < n; i++) total += per[i].size();
    if (total > ids_cap) return -(int64_t)total;
    uint64_t off = 0;
    for (uint64_t i = 0; i < n; i++) {
        counts[i] = (uint32_t)per[i].size();
        for (uint32_t k : per[i]) ids[off++] = k;
    }
    return (int64_t)total;
}

// Single polygon detect (cd_engine.rs:160) for an already transformed shape with its poi.
int32_t or_detect_poly(void* ep, const float* xy, uint32_t nv, const float* poi3, const uint32_t* filt,
                       uint32_t n_filt) {
    Engine* e = (Engine*)ep;
    Filter f = make_filter(filt, n_filt, e->hmap.size());
    SPolygon s;
    s.v.resize(nv);
    for (uint32_t i = 0; i < nv; i++) s.v[i] = Point{xy[2 * i], xy[2 * i + 1]};
    s.bbox = generate_bounding_box(s.v);
    s.poi = Circle{Point{poi3[0], poi3[1]}, poi3[2]};
    return e->detect_poly_collision(s, f) ? 1 : 0;
}
// Single polygon collect (cd_engine.rs:261) with the filter as pre-seeded collector keys.
int32_t or_collect_poly(void* ep, const float* xy, uint32_t nv, const float* poi3, const uint32_t* filt,
                        uint32_t n_filt, uint32_t* keys, uint32_t cap) {
    Engine* e = (Engine*)ep;
    Filter f = make_filter(filt, n_filt, e->hmap.size());
    SPolygon s;
    s.v.resize(nv);
    for (uint32_t i = 0; i < nv; i++) s.v[i] = Point{xy[2 * i], xy[2 * i + 1]};
    s.bbox = generate_bounding_box(s.v);
    s.poi = Circle{Point{poi3[0], poi3[1]}, poi3[2]};
    Collector c;
    c.reset(e->hmap.size());
    for (size_t k = 0; k < f.ignored.size() && k < e->hmap.size(); k++) if (f.ignored[k]) c.in[k] = 1;
    e->collect_poly_collisions(s, c);
    std::sort(c.keys.begin(), c.keys.end());
    for (size_t i = 0; i < c.keys.size() && i < cap; i++) keys[i] = c.keys[i];
    return (int32_t)c.keys.size();
}
// Single surrogate collect (cd_engine.rs:296).
int32_t or_collect_surrogate(void* ep, uint32_t item, const float* t4, const uint32_t* filt, uint32_t n_filt,
                             uint32_t* keys, uint32_t cap) {
    Engine* e = (Engine*)ep;
    Filter f = make_filter(filt, n_filt, e->hmap.size());
    Transform t{t4[0], t4[1], t4[2], t4[3]};
    Collector c;
    c.reset(e->hmap.size());
    for (size_t k = 0; k < f.ignored.size() && k < e->hmap.size(); k++) if (f.ignored[k]) c.in[k] = 1;
    e->collect_surrogate_collisions(e->items[item], t, c);
    std::sort(c.keys.begin(), c.keys.end());
    for (size_t i = 0; i < c.keys.size() && i < cap; i++) keys[i] = c.keys[i];
    return (int32_t)c.keys.size();
}
// Single surrogate detect (cd_engine.rs:204).
int32_t or_detect_surrogate(void* ep, uint32_t item, const float* t4, const uint32_t* filt, uint32_t n_filt) {
    Engine* e = (Engine*)ep;
    Filter f = make_filter(filt, n_filt, e->hmap.size());
    Transform t{t4[0], t4[1], t4[2], t4[3]};
    return e->detect_surrogate_collision(e->items[item], t, f) ? 1 : 0;
}

// SPolygon::new (simple_polygon.rs:41-71, including calculate_poi :152-171) on raw vertices.
// xy_out receives the vertices in internal (counter-clockwise) order; stats = {area, diameter}.
int32_t or_spolygon_new(const float* xy, uint32_t nv, float* xy_out, float* bbox_out, float* stats_out,
                        float* poi_out) {
    std::vector<Point> pts(nv);
    for (uint32_t i = 0; i < nv; i++) pts[i] = Point{xy[2 * i], xy[2 * i + 1]};
    SPolygon sp;
    if (!spolygon_new(pts, &sp)) return -1;
    for (uint32_t i = 0; i < nv; i++) { xy_out[2 * i] = sp.v[i].x; xy_out[2 * i + 1] = sp.v[i].y; }
    bbox_out[0] = sp.bbox.x_min; bbox_out[1] = sp.bbox.y_min; bbox_out[2] = sp.bbox.x_max; bbox_out[3] = sp.bbox.y_max;
    stats_out[0] = sp.area;
    stats_out[1] = sp.diameter;
    poi_out[0] = sp.poi.c.x; poi_out[1] = sp.poi.c.y; poi_out[2] = sp.poi.r;
    return 0;
}

// Surrogate poles (sp_surrogate.rs:33-53 -> pole.rs:12-47) of an internal shape whose poi and
// area are given (SPolygon::transform keeps area and moves the poi, simple_polygon.rs:195-224).
// poles_out receives (x, y, r) per pole, the first being the poi.  Returns 0, -1 (no pole) or
// -2 (capacity).
int32_t or_surrogate_poles(const float* xy, uint32_t nv, float area, const float* poi3, const uint32_t* lim_n,
                           const float* lim_cov, int32_t n_limits, float* poles_out, uint32_t poles_cap,
                           uint32_t* n_poles) {
    SPolygon sp;
    sp.v.resize(nv);
    for (uint32_t i = 0; i < nv; i++) sp.v[i] = Point{xy[2 * i], xy[2 * i + 1]};
    sp.bbox = generate_bounding_box(sp.v);
    sp.area = area;
    sp.poi = Circle{Point{poi3[0], poi3[1]}, poi3[2]};
    std::vector<PoleLimit> lims(n_limits);
    for (int i = 0; i < n_limits; i++) lims[i] = PoleLimit{lim_n[i], lim_cov[i]};
    std::vector<Circle> poles;
    if (!generate_surrogate_poles(sp, lims.data(), n_limits, poles)) return -1;
    *n_poles = (uint32_t)poles.size();
    if (poles.size() > poles_cap) return -2;
    for (size_t i = 0; i < poles.size(); i++) {
        poles_out[3 * i] = poles[i].c.x; poles_out[3 * i + 1] = poles[i].c.y; poles_out[3 * i + 2] = poles[i].r;
    }
    return 0;
}

// Polygon centroid (simple_polygon.rs:173-192) — used for the importer's centering pre-transform.
void or_centroid(const float* xy, uint32_t nv, float area, float* out2) {
    float cx = 0.0f, cy = 0.0f;
    for (uint32_t i = 0; i < nv; i++) {
        uint32_t j = (i == nv - 1) ? 0 : i + 1;
        float xi = xy[2 * i], yi = xy[2 * i + 1], xj = xy[2 * j], yj = xy[2 * j + 1];
        cx += (xi + xj) * (xi * yj - xj * yi);
        cy += (yi + yj) * (xi * yj - xj * yi);
    }
    cx /= 6.0f * area;
    cy /= 6.0f * area;
    out2[0] = cx;
    out2[1] = cy;
}

// simplify_shape (shape_modification.rs:48-144) of an internal shape with the given area, without
// the final SPolygon::new: *n_out receives the simplified vertex count.  deflate: 0 Inflate, 1 Deflate.
int32_t or_simplify_shape(const float* xy, uint32_t nv, float area, int32_t deflate, float tolerance, float* xy_out,
                          uint32_t* n_out) {
    std::vector<Point> pts(nv);
    for (uint32_t i = 0; i < nv; i++) pts[i] = Point{xy[2 * i], xy[2 * i + 1]};
    std::vector<Point> r = simplify_shape(pts, area, deflate != 0, tolerance);
    *n_out = (uint32_t)r.size();
    for (size_t i = 0; i < r.size(); i++) { xy_out[2 * i] = r[i].x; xy_out[2 * i + 1] = r[i].y; }
    return 0;
}

// close_narrow_concavities (shape_modification.rs:374-478) of a shape (SPolygon::new is applied
// first, as the reference's input is an SPolygon); *n_out receives the resulting vertex count.
int32_t or_close_concavities(const float* xy, uint32_t nv, int32_t deflate, float ratio, float* xy_out,
                             uint32_t* n_out) {
    std::vector<Point> pts(nv);
    for (uint32_t i = 0; i < nv; i++) pts[i] = Point{xy[2 * i], xy[2 * i + 1]};
    std::vector<Point> r = close_narrow_concavities(pts, deflate != 0, ratio);
    *n_out = (uint32_t)r.size();
    for (size_t i = 0; i < r.size(); i++) { xy_out[2 * i] = r[i].x; xy_out[2 * i + 1] = r[i].y; }
    return 0;
}

// Primitive probes for known-answer tests.
int32_t or_fpa_eq(float a, float b) { return fpa_eq(a, b); }
int32_t or_edge_intersection(const float* e1, const float* e2) {
    return edge_intersection(Edge{{e1[0], e1[1]}, {e1[2], e1[3]}}, Edge{{e2[0], e2[1]}, {e2[2], e2[3]}});
}
int32_t or_rect_collides_edge(const float* r, const float* e) {
    return rect_collides_edge(Rect{r[0], r[1], r[2], r[3]}, Edge{{e[0], e[1]}, {e[2], e[3]}});
}
int32_t or_point_in_poly(const float* xy, uint32_t nv, float px, float py) {
    SPolygon s;
    s.v.resize(nv);
    for (uint32_t i = 0; i < nv; i++) s.v[i] = Point{xy[2 * i], xy[2 * i + 1]};
    s.bbox = generate_bounding_box(s.v);
    return poly_collides_point(s, Point{px, py});
}
int32_t or_almost_relation(const float* a, const float* b) {
    return rect_almost_relation_to(Rect{a[0], a[1], a[2], a[3]}, Rect{b[0], b[1], b[2], b[3]});
}
void or_edge_quadrants(const float* e, const float* r, uint8_t* out4) {
    Rect rr{r[0], r[1], r[2], r[3]};
    Rect q[4];
    rect_quadrants(rr, q);
    bool o[4];
    edge_collides_with_quadrants(Edge{{e[0], e[1]}, {e[2], e[3]}}, rr, q, o);
    for (int i = 0; i < 4; i++) out4[i] = o[i];
}

// Canonical dump of the quadtree; returns the number of words (writes only if cap suffices).
uint64_t or_tree_dump(void* ep, uint32_t* out, uint64_t cap) {
    std::vector<uint32_t> o;
    dump_node(((Engine*)ep)->root, o);
    if (o.size() <= cap) std::memcpy(out, o.data(), o.size() * 4);
    return o.size();
}
uint32_t or_n_slots(void* ep) { return (uint32_t)((Engine*)ep)->hmap.size(); }

}  // extern "C"

// ------------------------------------------------------------------------------------------
// FP64 oracle of the pole-overlap proxy (test infrastructure): for each candidate (theta, tx, ty)
// of item `items[i]` whose poles are item_poles[pole_off[item] .. pole_off[item+1]) (x, y, r),
//   P = sum_ij max(0, r_i + r_j - |R(theta) p_i + t - c_j|)^2
// over every hazard pole (x, y, r, key) whose key is not ignored, evaluated in double precision
// from the float32 inputs, with its analytic gradient d/d(theta, tx, ty).
// ------------------------------------------------------------------------------------------
extern "C" void or_proxy_f64(uint64_t n, const double* params, const uint32_t* items, const uint32_t* pole_off,
                             const float* item_poles, const float* hpoles, uint64_t n_hpoles,
                             const uint32_t* ignored, uint32_t n_ignored, double* value, double* grad,
                             int32_t n_threads) {
    std::vector<uint8_t> ign;
    for (uint32_t i = 0; i < n_ignored; i++) {
        if (ignored[i] >= ign.size()) ign.resize(ignored[i] + 1, 0);
        ign[ignored[i]] = 1;
    }
    // A uniform grid over the hazard poles' centres only prunes pairs that cannot overlap (centres
    // further apart than r_i + r_max + 1); the pairs that remain are summed in ascending pole order,
    // the order of a plain loop over every hazard pole.
    double x0 = 1e300, y0 = 1e300, x1 = -1e300, y1 = -1e300, rmax = 0;
    for (uint64_t j = 0; j < n_hpoles; j++) {
        x0 = std::min(x0, (double)hpoles[4 * j]); x1 = std::max(x1, (double)hpoles[4 * j]);
        y0 = std::min(y0, (double)hpoles[4 * j + 1]); y1 = std::max(y1, (double)hpoles[4 * j + 1]);
        rmax = std::max(rmax, (double)hpoles[4 * j + 2]);
    }
    const double cs = std::max(1.0, 2.0 * rmax);
    const int64_t gx_n = n_hpoles ? std::min<int64_t>(4096, (int64_t)((x1 - x0) / cs) + 1) : 1;
    const int64_t gy_n = n_hpoles ? std::min<int64_t>(4096, (int64_t)((y1 - y0) / cs) + 1) : 1;
    const double csx = n_hpoles ? std::max(cs, (x1 - x0) / (double)gx_n + 1e-9) : 1.0;
    const double csy = n_hpoles ? std::max(cs, (y1 - y0) / (double)gy_n + 1e-9) : 1.0;
    std::vector<uint32_t> start((size_t)(gx_n * gy_n + 1), 0), idx(n_hpoles);
    auto cell_of = [&](double v, double o, double w, int64_t g) {
        int64_t c = (int64_t)std::floor((v - o) / w);
        return std::max<int64_t>(0, std::min<int64_t>(g - 1, c));
    };
    for (uint64_t j = 0; j < n_hpoles; j++)
        start[cell_of(hpoles[4 * j + 1], y0, csy, gy_n) * gx_n + cell_of(hpoles[4 * j], x0, csx, gx_n) + 1]++;
    for (size_t c = 1; c < start.size(); c++) start[c] += start[c - 1];
    {
        std::vector<uint32_t> fill(start.begin(), start.end() - 1);
        for (uint64_t j = 0; j < n_hpoles; j++)
            idx[fill[cell_of(hpoles[4 * j + 1], y0, csy, gy_n) * gx_n + cell_of(hpoles[4 * j], x0, csx, gx_n)]++] = (uint32_t)j;
    }
    run_threads(n, n_threads, [&](uint64_t a, uint64_t b, int) {
        std::vector<uint32_t> near;
        for (uint64_t i = a; i < b; i++) {
            const double th = params[3 * i], tx = params[3 * i + 1], ty = params[3 * i + 2];
            const double c = std::cos(th), s = std::sin(th);
            double P = 0, gt = 0, gx = 0, gy = 0;
            const uint32_t it = items[i];
            for (uint32_t k = pole_off[it]; k < pole_off[it + 1]; k++) {
                const double px = item_poles[3 * k], py = item_poles[3 * k + 1], r = item_poles[3 * k + 2];
                const double rx = c * px - s * py, ry = s * px + c * py;
                const double cx = rx + tx, cy = ry + ty, reach = r + rmax + 1.0;
                near.clear();
                if (n_hpoles) {
                    const int64_t ax = cell_of(cx - reach, x0, csx, gx_n), bx = cell_of(cx + reach, x0, csx, gx_n);
                    const int64_t ay = cell_of(cy - reach, y0, csy, gy_n), by = cell_of(cy + reach, y0, csy, gy_n);
                    for (int64_t yy = ay; yy <= by; yy++)
                        for (int64_t xx = ax; xx <= bx; xx++)
                            for (uint32_t q = start[yy * gx_n + xx]; q < start[yy * gx_n + xx + 1]; q++) near.push_back(idx[q]);
                    std::sort(near.begin(), near.end());
                }
                for (uint32_t j : near) {
                    uint32_t key;
                    std::memcpy(&key, &hpoles[4 * j + 3], 4);
                    if (key < ign.size() && ign[key]) continue;
                    const double dx = (tx - (double)hpoles[4 * j]) + rx, dy = (ty - (double)hpoles[4 * j + 1]) + ry;
                    const double d = std::sqrt(dx * dx + dy * dy);
                    const double pen = r + (double)hpoles[4 * j + 2] - d;
                    if (pen <= 0) continue;
                    P += pen * pen;
                    if (d > 0) {
                        const double f = -2.0 * pen / d;
                        gx += f * dx;
                        gy += f * dy;
                        gt += f * (dy * rx - dx * ry);
                    }
                }
            }
            value[i] = P;
            grad[3 * i] = gt;
            grad[3 * i + 1] = gx;
            grad[3 * i + 2] = gy;
        }
    });
}
