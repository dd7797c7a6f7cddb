"""The division-free form of the edge crossing test (geom.cuh `seg_hits_seg`) against the
reference's form with its two divisions (edge.rs:180-228, kept as `seg_hits_seg_div`), and the
quadrant mask's one-quadrant shortcut (`seg_quadrant_mask_short`) against its full form
(qt_traits.rs:19-106, `seg_quadrant_mask`), on tens of millions of cases: random coordinates
over many magnitudes, shared and nearly shared end points (quotients of exactly 0 and 1, and their
neighbours), integer grids (exact collinear and touching cases), tiny and huge coordinates (the
fallback ranges), random bit patterns (NaN, infinities, subnormals), and for the mask node boxes of
many scales and of zero width with edges on, one ulp off and across the bisectors; and the pole-edge
distance with its end-point branches decided without the division (`seg_sq_dist_ep`) against the
reference form (`seg_sq_dist`, edge.rs:63-87), bit for bit.  The header is compiled for the host here, with the flags of the library's
host code; the device compiles the same source with IEEE division and no contraction, so both
round every operation alike.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "jagua-rs_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <cmath>
#include "geom.cuh"
using namespace jcde;
static uint64_t s = 0x9E3779B97F4A7C15ull;
static inline uint64_t nx() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static inline float unif(float lo, float hi) { return lo + (hi - lo) * (float)((nx() >> 40) * 0x1p-24); }
static inline float bits() { uint32_t u = (uint32_t)nx(); float f; std::memcpy(&f, &u, 4); return f; }
static inline float nudge(float f, int k) {   // k ulps up (k > 0) or down
    for (; k > 0; k--) f = std::nextafter(f, INFINITY);
    for (; k < 0; k++) f = std::nextafter(f, -INFINITY);
    return f;
}
static long long n_pairs = 0, n_bad = 0, n_hits = 0;
static void check(const Seg& a, const Seg& b) {
    const bool x = seg_hits_seg(a, b), y = seg_hits_seg_div(a, b);
    n_pairs++;
    n_hits += y;
    if (x != y && n_bad++ < 5)
        std::printf("mismatch %a %a %a %a | %a %a %a %a: %d vs %d\n", a.s.x, a.s.y, a.e.x, a.e.y, b.s.x, b.s.y,
                    b.e.x, b.e.y, (int)x, (int)y);
}
int main(int argc, char** argv) {
    const long long N = argc > 1 ? atoll(argv[1]) : 4000000;
    const float mags[] = {1e-30f, 1e-6f, 1e-3f, 1.0f, 100.0f, 2000.0f, 1e5f, 1e9f, 1e18f, 1e30f};
    for (long long i = 0; i < N; i++) {
        const float m = mags[nx() % 10];
        Seg a{{unif(-m, m), unif(-m, m)}, {unif(-m, m), unif(-m, m)}};
        Seg b{{unif(-m, m), unif(-m, m)}, {unif(-m, m), unif(-m, m)}};
        check(a, b);
        // b through an end point of a, or a point of a, nudged by a few ulps
        const int k = (int)(nx() % 7) - 3;
        Pt p = (nx() & 1) ? a.s : a.e;
        if (nx() % 3 == 0) {
            const float t = unif(0.0f, 1.0f);
            p = Pt{a.s.x + t * (a.e.x - a.s.x), a.s.y + t * (a.e.y - a.s.y)};
        }
        Seg c{{nudge(p.x, k), nudge(p.y, (int)(nx() % 7) - 3)}, {unif(-m, m), unif(-m, m)}};
        check(a, c);
        check(c, a);
        Seg c2{b.s, {nudge(p.x, -k), p.y}};
        check(a, c2);
        // shared end points, either orientation
        check(a, Seg{a.e, b.e});
        check(a, Seg{b.s, a.s});
        // integer grid (exact ties, collinear overlaps)
        Seg g{{(float)(nx() % 9), (float)(nx() % 9)}, {(float)(nx() % 9), (float)(nx() % 9)}};
        Seg h{{(float)(nx() % 9), (float)(nx() % 9)}, {(float)(nx() % 9), (float)(nx() % 9)}};
        check(g, h);
        // raw bit patterns (NaN, infinities, subnormals)
        if ((i & 7) == 0) {
            check(Seg{{bits(), bits()}, {bits(), bits()}}, Seg{{bits(), bits()}, {bits(), bits()}});
            Seg d{{bits(), bits()}, {bits(), bits()}};
            check(d, Seg{d.e, {bits(), bits()}});
        }
    }
    // the quadrant mask's one-quadrant shortcut against its full form: node boxes of many scales and
    // of zero width, edges inside, across and beyond them, on and one ulp off the bisectors, NaN
    long long n_masks = 0, n_mask_bad = 0, n_short = 0;
    for (long long i = 0; i < N; i++) {
        const float m = mags[nx() % 10];
        const float x0 = unif(-m, m), y0 = unif(-m, m);
        const float w = (nx() % 16 == 0) ? 0.0f : unif(0.0f, m), h = (nx() % 16 == 0) ? 0.0f : unif(0.0f, m);
        const Box r{x0, y0, x0 + w, y0 + h};
        const Pt c = box_mid(r);
        for (int k = 0; k < 6; k++) {
            auto coord = [&](float lo, float hi, float mid) {
                switch (nx() % 6) {
                    case 0: return nudge(mid, (int)(nx() % 5) - 2);
                    case 1: return nudge(nx() & 1 ? lo : hi, (int)(nx() % 5) - 2);
                    case 2: return unif(lo - (hi - lo), hi + (hi - lo));
                    case 3: return (nx() % 64 == 0) ? NAN : unif(lo, hi);
                    default: return unif(lo, hi);
                }
            };
            Seg e{{coord(r.x0, r.x1, c.x), coord(r.y0, r.y1, c.y)}, {coord(r.x0, r.x1, c.x), coord(r.y0, r.y1, c.y)}};
            if (k == 5) e.e = Pt{nudge(e.s.x, (int)(nx() % 3) - 1), nudge(e.s.y, (int)(nx() % 3) - 1)};
            const uint32_t a = seg_quadrant_mask_short(e, r), b = seg_quadrant_mask(e, r);
            n_masks++;
            n_short += (a != 0 && (a & (a - 1)) == 0);
            if (a != b && n_mask_bad++ < 5)
                std::printf("mask mismatch %a %a %a %a | %a %a %a %a: %u vs %u\n", e.s.x, e.s.y, e.e.x, e.e.y, r.x0,
                            r.y0, r.x1, r.y1, a, b);
        }
    }
    // the pole-edge test with its end-point cases decided without the division, against the reference
    // form: the squared distances must be the same bits, and so the verdicts
    long long n_disks = 0, n_disk_bad = 0;
    for (long long i = 0; i < N; i++) {
        const float m = mags[nx() % 10];
        Seg e{{unif(-m, m), unif(-m, m)}, {unif(-m, m), unif(-m, m)}};
        if (nx() % 8 == 0) e.e = e.s;                                              // zero length
        if (nx() % 8 == 0) e.e = Pt{nudge(e.s.x, (int)(nx() % 3) - 1), e.s.y};   // nearly zero
        Pt p{unif(-m, m), unif(-m, m)};
        switch (nx() % 5) {
            case 0: p = Pt{nudge(e.s.x, (int)(nx() % 5) - 2), nudge(e.s.y, (int)(nx() % 5) - 2)}; break;
            case 1: p = Pt{nudge(e.e.x, (int)(nx() % 5) - 2), nudge(e.e.y, (int)(nx() % 5) - 2)}; break;
            case 2: {   // on the perpendicular through an end point (dot ~ 0 or ~ len_sq)
                const Pt q = nx() & 1 ? e.s : e.e;
                const float t = unif(-1.0f, 1.0f);
                p = Pt{q.x - t * (e.e.y - e.s.y), q.y + t * (e.e.x - e.s.x)};
                break;
            }
            default: break;
        }
        if ((i & 15) == 0) { e = Seg{{bits(), bits()}, {bits(), bits()}}; p = Pt{bits(), bits()}; }
        const Disk dk{p, unif(0.0f, m)};
        const float a = seg_sq_dist_ep(e, p), b = seg_sq_dist(e, p);
        uint32_t ua, ub;
        std::memcpy(&ua, &a, 4);
        std::memcpy(&ub, &b, 4);
        n_disks++;
        if ((ua != ub && !(a != a && b != b)) || disk_hits_seg(dk, e) != disk_hits_seg_div(dk, e))
            if (n_disk_bad++ < 5)
                std::printf("disk mismatch %a %a %a %a | %a %a: %a vs %a\n", e.s.x, e.s.y, e.e.x, e.e.y, p.x, p.y, a, b);
    }
    std::printf("pairs %lld hits %lld mismatches %lld masks %lld single %lld mask_mismatches %lld disks %lld "
                "disk_mismatches %lld\n", n_pairs, n_hits, n_bad, n_masks, n_short, n_mask_bad, n_disks, n_disk_bad);
    return (n_bad || n_mask_bad || n_disk_bad) ? 1 : 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_division_free_edge_crossing_equals_reference_form(tmp_path):
    src = tmp_path / "seg.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "seg"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-I", CSRC, str(src), "-o",
                    str(exe)], check=True)
    r = subprocess.run([str(exe), "3000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    tok = r.stdout.split()
    pairs, hits, masks, single = int(tok[1]), int(tok[3]), int(tok[7]), int(tok[9])
    assert pairs > 2e7 and hits > 1e6, r.stdout
    assert masks > 1e7 and single > 1e6, r.stdout
    assert int(tok[13]) >= 3e6 and int(tok[15]) == 0, r.stdout
