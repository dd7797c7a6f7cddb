// Geometry predicates of the CDE query path, compiled both for the host (quadtree builder, pole
// generation) and for sm_103a kernels, so that both sides round every operation identically.
//
// Every function restates an f32 routine of jagua-rs (path:line in the comment).  Rules that keep
// the device bit-identical with the reference's f32 arithmetic:
//   * device code is compiled with -fmad=false -prec-div=true -prec-sqrt=true -ftz=false, host code
//     with -ffp-contract=off: Rust never contracts a*b+c into a fused multiply-add;
//   * expressions keep the reference's evaluation order ((a*b) - (c*d), left-to-right sums);
//   * f32::min / f32::max are fminf / fmaxf (a NaN operand is ignored);
//   * sin/cos are never evaluated here: transforms arrive as matrix entries.
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>

#ifdef __CUDACC__
#define JHD __host__ __device__ __forceinline__
#define JCDE_UNROLL _Pragma("unroll")
#else
#define JHD inline
#define JCDE_UNROLL
#endif

namespace jcde {

#ifdef __CUDACC__
// Programmatic dependent launch: a grid launched with the programmatic stream-serialization
// attribute may be scheduled as soon as every block of the grid before it on the stream has
// exited, ahead of that grid's completion and the launch processing that would otherwise follow
// it.  pdl_wait() returns once that grid has completed and its memory writes are visible (at once
// when there is none, or when the grid was launched without the attribute), so a kernel that calls
// it before its first global memory access gives the same results launched either way.  (Letting
// the successor be scheduled earlier still, with griddepcontrol.launch_dependents at the start of
// the predecessor, made the LBF build slower: its blocks sit waiting on SMs the predecessor uses.)
__device__ __forceinline__ void pdl_wait() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}
#endif

struct Pt { float x, y; };
struct Seg { Pt s, e; };
struct Box { float x0, y0, x1, y1; };
struct Disk { Pt c; float r; };

enum Rel : int { REL_INTERSECTING = 0, REL_ENCLOSED = 1, REL_SURROUNDING = 2, REL_DISJOINT = 3 };

JHD float fmn(float a, float b) { return fminf(a, b); }
JHD float fmx(float a, float b) { return fmaxf(a, b); }

JHD int32_t f2i(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_int(f);
#else
    int32_t i;
    std::memcpy(&i, &f, 4);
    return i;
#endif
}

// util/fpa.rs:18-31 — FPA equality is float-cmp's approx_eq!(f32) with the default margin:
// exactly equal, or |a-b| <= f32::EPSILON, or at most 4 ULPs apart (bit patterns as i32).
JHD bool fpa_eq(float a, float b) {
    if (a == b) return true;
    if (fabsf(a - b) <= 1.1920928955078125e-07f) return true;
    int32_t d = (int32_t)((uint32_t)f2i(a) - (uint32_t)f2i(b));
    int32_t ad = d < 0 ? (d == INT32_MIN ? INT32_MAX : -d) : d;
    return ad <= 4;
}
// FPA's PartialOrd (util/fpa.rs:25-31): Equal when approx-equal, else the f32 order.  The plain
// comparison is tested first: the boolean is the same (both terms are pure), and it usually
// decides without the approximate-equality test.
JHD bool fpa_le(float a, float b) { return a < b || fpa_eq(a, b); }
JHD bool fpa_ge(float a, float b) { return a > b || fpa_eq(a, b); }
JHD bool fpa_lt(float a, float b) { return a < b && !fpa_eq(a, b); }
JHD bool fpa_gt(float a, float b) { return a > b && !fpa_eq(a, b); }

// rect.rs:266-271
JHD bool box_hits_box(const Box& a, const Box& b) {
    return fmx(a.x0, b.x0) <= fmn(a.x1, b.x1) && fmx(a.y0, b.y0) <= fmn(a.y1, b.y1);
}
// rect.rs:46-65 — relation of `s` to `o`
JHD int box_relation(const Box& s, const Box& o) {
    if (!box_hits_box(s, o)) return REL_DISJOINT;
    if (s.x0 <= o.x0 && s.y0 <= o.y0 && s.x1 >= o.x1 && s.y1 >= o.y1) return REL_SURROUNDING;
    if (s.x0 >= o.x0 && s.y0 >= o.y0 && s.x1 <= o.x1 && s.y1 <= o.y1) return REL_ENCLOSED;
    return REL_INTERSECTING;
}
// rect.rs:46-65 restricted to the Surrounding answer (get_virtual_root, detect_poly_collision)
JHD bool box_surrounds(const Box& s, const Box& o) {
    return box_hits_box(s, o) && s.x0 <= o.x0 && s.y0 <= o.y0 && s.x1 >= o.x1 && s.y1 >= o.y1;
}
// rect.rs:70-89 + rect.rs:274-279
JHD int box_almost_relation(const Box& s, const Box& o) {
    bool hit = fpa_le(fmx(s.x0, o.x0), fmn(s.x1, o.x1)) && fpa_le(fmx(s.y0, o.y0), fmn(s.y1, o.y1));
    if (!hit) return REL_DISJOINT;
    if (fpa_le(s.x0, o.x0) && fpa_le(s.y0, o.y0) && fpa_ge(s.x1, o.x1) && fpa_ge(s.y1, o.y1))
        return REL_SURROUNDING;
    if (fpa_ge(s.x0, o.x0) && fpa_ge(s.y0, o.y0) && fpa_le(s.x1, o.x1) && fpa_le(s.y1, o.y1))
        return REL_ENCLOSED;
    return REL_INTERSECTING;
}
// rect.rs:282-288
JHD bool box_hits_pt(const Box& r, Pt p) { return p.x >= r.x0 && p.x <= r.x1 && p.y >= r.y0 && p.y <= r.y1; }
// rect.rs:248-253
// x / 2 and x * 0.5 are the same correctly rounded value of the same real number
JHD Pt box_mid(const Box& r) { return Pt{(r.x0 + r.x1) * 0.5f, (r.y0 + r.y1) * 0.5f}; }
// rect.rs:259-263
JHD float box_diameter(const Box& r) {
    float dx = r.x1 - r.x0;
    float dy = r.y1 - r.y0;
    return sqrtf(dx * dx + dy * dy);
}
// rect.rs:93-109
JHD Box box_square(const Box& r) {
    float w = r.x1 - r.x0, h = r.y1 - r.y0;
    float dx = 0.0f, dy = 0.0f;
    if (h < w) dy = (w - h) / 2.0f;
    else if (w < h) dx = (h - w) / 2.0f;
    return Box{r.x0 - dx, r.y0 - dy, r.x1 + dx, r.y1 + dy};
}
// rect.rs:154-161 corner i (quadrant order: ++, -+, --, +-)
JHD Pt box_corner(const Box& r, int i) {
    return Pt{(i == 0 || i == 3) ? r.x1 : r.x0, (i == 0 || i == 1) ? r.y1 : r.y0};
}
// rect.rs:141-151 with rect.rs:35-41 — quadrant i of r (from_diagonal_corners(corner_i, mid))
JHD Box box_quadrant(const Box& r, int i) {
    Pt m = box_mid(r);
    Pt c = box_corner(r, i);
    return Box{fmn(c.x, m.x), fmn(c.y, m.y), fmx(c.x, m.x), fmx(c.y, m.y)};
}
// The same four boxes given the midpoint: the midpoint of a valid box lies between its bounds, so
// from_diagonal_corners(corner_i, mid) reduces to picking bounds (q0 = ++, q1 = -+, q2 = --, q3 = +-).
JHD Box quad_box(const Box& r, Pt m, int i) {
    return Box{(i == 0 || i == 3) ? m.x : r.x0, (i == 0 || i == 1) ? m.y : r.y0,
               (i == 0 || i == 3) ? r.x1 : m.x, (i == 0 || i == 1) ? r.y1 : m.y};
}

// rect.rs:301-345 — Rect collides with Edge
JHD bool box_hits_seg(const Box& r, const Seg& e) {
    float ex0 = fmn(e.s.x, e.e.x), ex1 = fmx(e.s.x, e.e.x);
    float ey0 = fmn(e.s.y, e.e.y), ey1 = fmx(e.s.y, e.e.y);
    if (fmx(ex0, r.x0) > fmn(ex1, r.x1) || fmx(ey0, r.y0) > fmn(ey1, r.y1)) return false;
    if (box_hits_pt(r, e.s) || box_hits_pt(r, e.e)) return true;
    float sx = e.s.x, sy = e.s.y;
    float dx = e.e.x - sx, dy = e.e.y - sy;
    bool all_pos = true, all_neg = true;
JCDE_UNROLL
    for (int i = 0; i < 4; i++) {
        Pt c = box_corner(r, i);
        float side = (c.x - sx) * dy - (c.y - sy) * dx;
        all_pos = all_pos && side > 0.0f;
        all_neg = all_neg && side < 0.0f;
    }
    return !(all_pos || all_neg);
}

// edge.rs:180-228 (location not requested) — e1 is the querying edge, e2 the hazard edge.
// The reference divides (t = t_nom / t_den, u = u_nom / t_den) and tests 0 <= t, u <= 1.  With
// the denominator's sign moved into the numerators (a / d with d = |t_den| > 0, negation is exact),
// the rounded quotient is decided by comparisons in most cases:
//   * RN(a / d) <= 1 exactly when a <= d: a float above d is at least d's successor, and the
//     quotient of the two exceeds 1 + 2^-24, the midpoint that rounds to 1 (true for every d > 0);
//   * RN(a / d) >= 0 exactly when a >= 0, unless a < 0 is so small against d that the quotient
//     rounds to -0; with a <= -2^-60 and d <= 2^60 the quotient is at most -2^-120, so it cannot.
// Outside those ranges (and for NaN or infinite terms) the divisions are done as the reference does.
JHD bool seg_hits_seg(const Seg& e1, const Seg& e2) {
    float x1 = e1.s.x, y1 = e1.s.y, x2 = e1.e.x, y2 = e1.e.y;
    float x3 = e2.s.x, y3 = e2.s.y, x4 = e2.e.x, y4 = e2.e.y;
    if (fmx(fmn(x1, x2), fmn(x3, x4)) > fmn(fmx(x1, x2), fmx(x3, x4))) return false;
    if (fmx(fmn(y1, y2), fmn(y3, y4)) > fmn(fmx(y1, y2), fmx(y3, y4))) return false;
    float t_nom = (x2 - x4) * (y4 - y3) - (y2 - y4) * (x4 - x3);
    float t_den = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    float u_nom = (x2 - x4) * (y2 - y1) - (y2 - y4) * (x2 - x1);
    // u's denominator (edge.rs:210) is the same expression as t's (edge.rs:208)
    if (t_den == 0.0f) return false;
    const bool neg = t_den < 0.0f;
    const float a = neg ? -t_nom : t_nom, b = neg ? -u_nom : u_nom, d = neg ? -t_den : t_den;
    if (d <= 0x1p60f && (a >= 0.0f || a <= -0x1p-60f) && (b >= 0.0f || b <= -0x1p-60f))
        return a >= 0.0f && a <= d && b >= 0.0f && b <= d;
    float t = t_nom / t_den;
    float u = u_nom / t_den;
    return 0.0f <= t && t <= 1.0f && 0.0f <= u && u <= 1.0f;
}
// The same test with the reference's two divisions always done (kept for the equivalence test).
JHD bool seg_hits_seg_div(const Seg& e1, const Seg& e2) {
    float x1 = e1.s.x, y1 = e1.s.y, x2 = e1.e.x, y2 = e1.e.y;
    float x3 = e2.s.x, y3 = e2.s.y, x4 = e2.e.x, y4 = e2.e.y;
    if (fmx(fmn(x1, x2), fmn(x3, x4)) > fmn(fmx(x1, x2), fmx(x3, x4))) return false;
    if (fmx(fmn(y1, y2), fmn(y3, y4)) > fmn(fmx(y1, y2), fmx(y3, y4))) return false;
    float t_nom = (x2 - x4) * (y4 - y3) - (y2 - y4) * (x4 - x3);
    float t_den = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    float u_nom = (x2 - x4) * (y2 - y1) - (y2 - y4) * (x2 - x1);
    if (t_den == 0.0f) return false;
    float t = t_nom / t_den;
    float u = u_nom / t_den;
    return 0.0f <= t && t <= 1.0f && 0.0f <= u && u <= 1.0f;
}

// qt_traits.rs:144-177 — half of e2 hit by e1: -1 none, 0 first half, 1 halfway, 2 second half
JHD int seg_hit_half(const Seg& e1, const Seg& e2) {
    float x1 = e1.s.x, y1 = e1.s.y, x2 = e1.e.x, y2 = e1.e.y;
    float x3 = e2.s.x, y3 = e2.s.y, x4 = e2.e.x, y4 = e2.e.y;
    float t_nom = (x2 - x4) * (y4 - y3) - (y2 - y4) * (x4 - x3);
    float t_den = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    float u_nom = (x2 - x4) * (y2 - y1) - (y2 - y4) * (x2 - x1);
    if (t_den == 0.0f) return -1;
    float t = t_nom / t_den;
    float u = u_nom / t_den;
    if (0.0f <= t && t <= 1.0f && 0.0f <= u && u <= 1.0f) return u > 0.5f ? 0 : (u < 0.5f ? 2 : 1);
    return -1;
}

// qt_traits.rs:19-106 — which of the 4 quadrants of node box r the edge touches (bit i = quadrant i)
JHD uint32_t seg_quadrant_mask(const Seg& e, const Box& r) {
    float ex0 = fmn(e.s.x, e.e.x), ex1 = fmx(e.s.x, e.e.x);
    float ey0 = fmn(e.s.y, e.e.y), ey1 = fmx(e.s.y, e.e.y);
    const Pt c = box_mid(r);
    // per-quadrant overlap tests of qt_traits.rs:29-31; quadrants share their x (or y) extents in
    // pairs, so each distinct expression is evaluated once
    const bool xr = !(fmx(ex0, c.x) > fmn(ex1, r.x1)), xl = !(fmx(ex0, r.x0) > fmn(ex1, c.x));
    const bool yt = !(fmx(ey0, c.y) > fmn(ey1, r.y1)), yb = !(fmx(ey0, r.y0) > fmn(ey1, c.y));
    const uint32_t ov = (xr && yt ? 1u : 0u) | (xl && yt ? 2u : 0u) | (xl && yb ? 4u : 0u) | (xr && yb ? 8u : 0u);
    // end points inside quadrants (rect.rs:282-288 per quadrant box)
    auto pt_mask = [&](Pt p) -> uint32_t {
        const bool R = p.x >= c.x && p.x <= r.x1, L = p.x >= r.x0 && p.x <= c.x;
        const bool T = p.y >= c.y && p.y <= r.y1, B = p.y >= r.y0 && p.y <= c.y;
        return (R && T ? 1u : 0u) | (L && T ? 2u : 0u) | (L && B ? 4u : 0u) | (R && B ? 8u : 0u);
    };
    uint32_t hit = ov & (pt_mask(e.s) | pt_mask(e.e));
    uint32_t undet = ov & ~hit;
    if (!undet) return hit;
    // sides (rect.rs:164-184): top c0->c1, left c1->c2, bottom c2->c3, right c3->c0; bisectors
    // (qt_traits.rs:123-130).  half_intersect (qt_traits.rs:110-140) runs only while a quadrant it
    // could set is undetermined, and sets the quadrants of the half of the side that was hit.
    const Seg sides[6] = {
        Seg{Pt{r.x0, r.y1}, Pt{r.x0, r.y0}},  // left:   first half -> q1, second -> q2
        Seg{Pt{r.x1, r.y0}, Pt{r.x1, r.y1}},  // right:  q3 | q0
        Seg{Pt{r.x1, r.y1}, Pt{r.x0, r.y1}},  // top:    q0 | q1
        Seg{Pt{r.x0, r.y0}, Pt{r.x1, r.y0}},  // bottom: q2 | q3
        Seg{Pt{r.x0, c.y}, Pt{r.x1, c.y}},    // h-bisector: q1,q2 | q0,q3
        Seg{Pt{c.x, r.y0}, Pt{c.x, r.y1}},    // v-bisector: q2,q3 | q0,q1
    };
    const uint32_t fst[6] = {0x2, 0x8, 0x1, 0x4, 0x6, 0xC};
    const uint32_t sec[6] = {0x4, 0x1, 0x2, 0x8, 0x9, 0x3};
JCDE_UNROLL
    for (int k = 0; k < 6; k++) {
        if ((fst[k] | sec[k]) & undet) {
            int h = seg_hit_half(e, sides[k]);
            uint32_t set = (h == 0 ? fst[k] : 0u) | (h == 2 ? sec[k] : 0u) | (h == 1 ? (fst[k] | sec[k]) : 0u);
            hit |= set;
            undet &= ~set;
        }
    }
    return hit;
}
// The same mask, first for an edge that lies strictly on one side of both bisectors: its extent
// then misses the other three quadrants' extents (their overlap tests compare a bound beyond the
// bisector with one short of it), so only quadrant i can be set, by the very tests the full form
// makes for it; an edge whose quadrant is then still undetermined (it overlaps the quadrant with
// neither end point inside) takes the full form.  A NaN coordinate fails the strict comparisons,
// so such an edge takes the full form too.  (Faster in the collect walks, where every lane walks its
// own edge to the end; slower in the polygon pass's lockstep walk, which keeps the full form.)
JHD uint32_t seg_quadrant_mask_short(const Seg& e, const Box& r) {
    const float ex0 = fmn(e.s.x, e.e.x), ex1 = fmx(e.s.x, e.e.x);
    const float ey0 = fmn(e.s.y, e.e.y), ey1 = fmx(e.s.y, e.e.y);
    const Pt c = box_mid(r);
    const bool lft = ex1 < c.x, rgt = ex0 > c.x, bot = ey1 < c.y, top = ey0 > c.y;
    if ((lft || rgt) && (bot || top)) {
        const int i = rgt ? (top ? 0 : 3) : (top ? 1 : 2);
        const float qx0 = rgt ? c.x : r.x0, qx1 = rgt ? r.x1 : c.x;
        const float qy0 = top ? c.y : r.y0, qy1 = top ? r.y1 : c.y;
        const bool ov = !(fmx(ex0, qx0) > fmn(ex1, qx1)) && !(fmx(ey0, qy0) > fmn(ey1, qy1));
        if (!ov) return 0u;
        const bool in_s = e.s.x >= qx0 && e.s.x <= qx1 && e.s.y >= qy0 && e.s.y <= qy1;
        const bool in_e = e.e.x >= qx0 && e.e.x <= qx1 && e.e.y >= qy0 && e.e.y <= qy1;
        if (in_s || in_e) return 1u << i;
    }
    return seg_quadrant_mask(e, r);
}

// edge.rs:63-87 + edge.rs:152-159 — squared distance from p to the segment
JHD float seg_sq_dist(const Seg& e, Pt p) {
    float x1 = e.s.x, y1 = e.s.y, x2 = e.e.x, y2 = e.e.y;
    float a = p.x - x1, b = p.y - y1, c = x2 - x1, d = y2 - y1;
    float dot = a * c + b * d;
    float len_sq = c * c + d * d;
    float param = -1.0f;
    if (len_sq != 0.0f) param = dot / len_sq;
    float xx, yy;
    if (param < 0.0f) { xx = x1; yy = y1; }
    else if (param > 1.0f) { xx = x2; yy = y2; }
    else { xx = x1 + param * c; yy = y1 + param * d; }
    float dx = p.x - xx, dy = p.y - yy;
    return dx * dx + dy * dy;
}
// The same squared distance with the end-point cases decided without the division: for a finite
// len_sq > 0, RN(dot / len_sq) > 1 exactly when dot > len_sq (a float above len_sq is at least its
// successor, whose quotient exceeds the midpoint 1 + 2^-24), and dot < 0 gives a negative quotient
// or -0, whose projection x1 + (-0) c is x1 again (c finite), so both pick the first end point.
// The division stays for the projection itself and for a non-finite len_sq.
JHD float seg_sq_dist_ep(const Seg& e, Pt p) {
    float x1 = e.s.x, y1 = e.s.y, x2 = e.e.x, y2 = e.e.y;
    float a = p.x - x1, b = p.y - y1, c = x2 - x1, d = y2 - y1;
    float dot = a * c + b * d;
    float len_sq = c * c + d * d;
    float xx, yy;
    const bool fin = len_sq <= 3.40282347e+38f;
    if (len_sq == 0.0f || (fin && dot < 0.0f)) {
        xx = x1;
        yy = y1;
    } else if (fin && dot > len_sq) {
        xx = x2;
        yy = y2;
    } else {
        float param = -1.0f;
        if (len_sq != 0.0f) param = dot / len_sq;
        if (param < 0.0f) { xx = x1; yy = y1; }
        else if (param > 1.0f) { xx = x2; yy = y2; }
        else { xx = x1 + param * c; yy = y1 + param * d; }
    }
    float dx = p.x - xx, dy = p.y - yy;
    return dx * dx + dy * dy;
}
// circle.rs:506-510
JHD bool disk_hits_seg(const Disk& c, const Seg& e) { return seg_sq_dist_ep(e, c.c) <= c.r * c.r; }
// ... with the reference's division always done (the lane-group surrogate pass, the equivalence test)
JHD bool disk_hits_seg_div(const Disk& c, const Seg& e) { return seg_sq_dist(e, c.c) <= c.r * c.r; }
// circle.rs:512-525
JHD bool disk_hits_box(const Disk& c, const Box& r) {
    float nx = fmx(r.x0, fmn(c.c.x, r.x1));
    float ny = fmx(r.y0, fmn(c.c.y, r.y1));
    float dx = nx - c.c.x, dy = ny - c.c.y;
    return dx * dx + dy * dy <= c.r * c.r;
}
// circle.rs:527-531 (point.sq_distance_to(center) <= r^2)
JHD bool disk_hits_pt(const Disk& c, Pt p) {
    float dx = p.x - c.c.x, dy = p.y - c.c.y;
    return dx * dx + dy * dy <= c.r * c.r;
}
// circle.rs:551-560 — separation distance (either side) from the circle to p
JHD float disk_sep_dist(const Disk& c, Pt p) {
    float dx = p.x - c.c.x, dy = p.y - c.c.y;
    float d = sqrtf(dx * dx + dy * dy);
    return d <= c.r ? c.r - d : d - c.r;
}
// qt_traits.rs:9-13 default: Circle collides with each quadrant box (circle.rs:512-525); the
// nearest-point terms are shared by the quadrants that share an extent
JHD uint32_t disk_quadrant_mask(const Disk& c, const Box& r) {
    const Pt m = box_mid(r);
    const float nxr = fmx(m.x, fmn(c.c.x, r.x1)) - c.c.x, nxl = fmx(r.x0, fmn(c.c.x, m.x)) - c.c.x;
    const float nyt = fmx(m.y, fmn(c.c.y, r.y1)) - c.c.y, nyb = fmx(r.y0, fmn(c.c.y, m.y)) - c.c.y;
    const float dxr = nxr * nxr, dxl = nxl * nxl, dyt = nyt * nyt, dyb = nyb * nyb;
    const float rr = c.r * c.r;
    return (dxr + dyt <= rr ? 1u : 0u) | (dxl + dyt <= rr ? 2u : 0u) | (dxl + dyb <= rr ? 4u : 0u) |
           (dxr + dyb <= rr ? 8u : 0u);
}

// point.rs:259-264 with the rot_transl_m matrix [[c, -s, tx], [s, c, ty]] (transformation.rs:475-483)
JHD Pt xform(Pt p, float c, float s, float tx, float ty) {
    float ms = -s;
    return Pt{c * p.x + ms * p.y + tx * 1.0f, s * p.x + c * p.y + ty * 1.0f};
}

// One edge's contribution to the ray-cast point-in-polygon test of simple_polygon.rs:255-292.
// `ray` runs from p to the right, past the polygon's bbox; returns 1 when the edge counts.
JHD int pip_edge_term(const Seg& ray, const Seg& e, Pt p) {
    if ((fpa_eq(e.s.y, p.y) && fpa_gt(e.s.x, p.x)) || (fpa_eq(e.e.y, p.y) && fpa_gt(e.e.x, p.x)))
        return (fpa_lt(e.s.y, p.y) || fpa_lt(e.e.y, p.y)) ? 1 : 0;
    return seg_hits_seg(ray, e) ? 1 : 0;
}
JHD Seg pip_ray(const Box& bbox, Pt p) { return Seg{p, Pt{bbox.x1 + (bbox.x1 - bbox.x0), p.y}}; }

}  // namespace jcde
