// Host-side quadtree of the CDE (see qtree.hpp).  Compiled with -ffp-contract=off.
#include "qtree.hpp"

#include <algorithm>
#include <cmath>
#include <array>
#include <cfloat>
#include <cstring>
#include <deque>

namespace jcde {

Box bounding_box(const Pt* v, size_t n) {
    float x0 = FLT_MAX, y0 = FLT_MAX, x1 = -FLT_MAX, y1 = -FLT_MAX;
    for (size_t i = 0; i < n; i++) {
        x0 = fmn(x0, v[i].x);
        y0 = fmn(y0, v[i].y);
        x1 = fmx(x1, v[i].x);
        y1 = fmx(y1, v[i].y);
    }
    return Box{x0, y0, x1, y1};
}

bool polygon_contains(const Polygon& poly, Pt p) {
    if (!box_hits_pt(poly.bbox, p)) return false;
    Seg ray = pip_ray(poly.bbox, p);
    int n = 0;
    size_t nv = poly.v.size();
    for (size_t i = 0; i < nv; i++) {
        Seg e{poly.v[i], poly.v[i + 1 == nv ? 0 : i + 1]};
        n += pip_edge_term(ray, e, p);
    }
    return (n & 1) == 1;
}

QuadTree::QuadTree(uint8_t depth, uint8_t cdt, Box bbox) : cdt_(cdt) {
    HNode root;
    root.bbox = bbox;
    root.level = depth;
    nodes_.push_back(std::move(root));
}

int32_t QuadTree::alloc_quartet(int32_t parent) {
    int32_t c;
    if (!free_quartets_.empty()) {
        c = free_quartets_.back();
        free_quartets_.pop_back();
    } else {
        c = (int32_t)nodes_.size();
        nodes_.resize(nodes_.size() + 4);
    }
    const Box pb = nodes_[parent].bbox;
    for (int i = 0; i < 4; i++) {
        HNode& n = nodes_[c + i];
        n.bbox = box_quadrant(pb, i);   // Rect::quadrants (rect.rs:141-151)
        n.level = (uint8_t)(nodes_[parent].level - 1);
        n.child = -1;
        n.parent = parent;
        n.hz.clear();
        n.n_active_edges = 0;
    }
    return c;
}

void QuadTree::free_subtree(int32_t c) {
    for (int i = 0; i < 4; i++) {
        HNode& n = nodes_[c + i];
        if (n.child >= 0) free_subtree(n.child);
        n.child = -1;
        n.hz.clear();
        n.n_active_edges = 0;
    }
    free_quartets_.push_back(c);
}

// QTHazPartial::from_parent (qt_partial_hazard.rs:25-59): the ff_bbox of a clipped edge set
static Box ff_from_parent(const NodeHaz& parent, const std::vector<Seg>& edges) {
    if (parent.edges->size() == edges.size()) return parent.ff;
    float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
    for (const Seg& e : edges) {
        x0 = fmn(fmn(x0, e.s.x), e.e.x);
        y0 = fmn(fmn(y0, e.s.y), e.e.y);
        x1 = fmx(fmx(x1, e.s.x), e.e.x);
        y1 = fmx(fmx(y1, e.s.y), e.e.y);
    }
    if (x0 < x1 && y0 < y1) return Box{x0, y0, x1, y1};
    return parent.ff;
}

// QTHazard::constrict (qt_hazard.rs:48-167)
void QuadTree::constrict(const NodeHaz& h, const Box q[4], NodeHaz out[4]) const {
    if (h.presence == PRES_ENTIRE) {
        for (int i = 0; i < 4; i++) out[i] = h;
        return;
    }
    const Polygon& shape = haz_[h.hkey].shape;
    for (int i = 0; i < 4; i++) {
        if (box_relation(shape.bbox, q[i]) == REL_ENCLOSED) {
            for (int k = 0; k < 4; k++) {
                out[k] = h;
                if (k != i) {
                    out[k].presence = PRES_NONE;
                    out[k].edges.reset();
                }
            }
            return;
        }
    }
    bool resolved[4] = {false, false, false, false};
    for (int i = 0; i < 4; i++) {
        std::vector<Seg> clipped;
        for (const Seg& e : *h.edges)
            if (box_hits_seg(q[i], e)) clipped.push_back(e);
        if (!clipped.empty()) {
            Box ff = ff_from_parent(h, clipped);
            out[i] = NodeHaz{h.hkey, PRES_PARTIAL, h.kind, ff,
                             std::make_shared<const std::vector<Seg>>(std::move(clipped))};
            resolved[i] = true;
        }
    }
    static const int NEIGHBOR[4][2] = {{1, 3}, {0, 2}, {1, 3}, {0, 2}};  // rect.rs:136
    for (int i = 0; i < 4; i++) {
        if (resolved[i]) continue;
        bool none_nb = false, entire_nb = false;
        for (int k = 0; k < 2; k++) {
            int nb = NEIGHBOR[i][k];
            if (!resolved[nb]) continue;
            none_nb |= out[nb].presence == PRES_NONE;
            entire_nb |= out[nb].presence == PRES_ENTIRE;
        }
        Presence p;
        if (none_nb && !entire_nb) p = PRES_NONE;
        else if (entire_nb && !none_nb) p = PRES_ENTIRE;
        else {
            bool inside = polygon_contains(shape, box_mid(q[i]));
            bool ext = kind_is_exterior(h.kind);
            p = (!ext && inside) || (ext && !inside) ? PRES_ENTIRE : PRES_NONE;
        }
        out[i] = NodeHaz{h.hkey, p, h.kind, Box{0, 0, 0, 0}, nullptr};
        resolved[i] = true;
    }
}

void QuadTree::reg_children(int32_t n, const NodeHaz& h) {
    const int32_t c = nodes_[n].child;
    Box q[4];
    for (int i = 0; i < 4; i++) q[i] = nodes_[c + i].bbox;
    NodeHaz ch[4];
    constrict(h, q, ch);
    for (int i = 0; i < 4; i++)
        if (ch[i].presence != PRES_NONE) reg(c + i, ch[i]);
}

// QTNode::register_hazard (qt_node.rs:38-81)
void QuadTree::reg(int32_t n, const NodeHaz& h) {
    if (nodes_[n].child < 0 && nodes_[n].level > 0 && h.presence == PRES_PARTIAL) {
        int32_t c = alloc_quartet(n);
        nodes_[n].child = c;
        std::vector<NodeHaz> old = nodes_[n].hz;
        for (const NodeHaz& o : old) reg_children(n, o);
    }
    if (nodes_[n].child >= 0) reg_children(n, h);
    // QTHazardVec::add (qt_hazard_vec.rs:24-43): kept sorted Entire before Partial
    std::vector<NodeHaz>& v = nodes_[n].hz;
    size_t pos = 0;
    while (pos < v.size() && v[pos].presence >= h.presence) pos++;
    v.insert(v.begin() + pos, h);
    nodes_[n].n_active_edges += h.n_edges();
}

// QTNode::deregister_hazard (qt_node.rs:83-94)
void QuadTree::dereg(int32_t n, uint32_t key) {
    std::vector<NodeHaz>& v = nodes_[n].hz;
    bool modified = false;
    for (size_t i = 0; i < v.size(); i++) {
        if (v[i].hkey == key) {
            nodes_[n].n_active_edges -= v[i].n_edges();
            v.erase(v.begin() + i);
            modified = true;
            break;
        }
    }
    if (!modified) return;
    bool any_partial = false;
    for (const NodeHaz& h : nodes_[n].hz) any_partial |= h.presence == PRES_PARTIAL;
    if (!any_partial) {
        if (nodes_[n].child >= 0) {
            free_subtree(nodes_[n].child);
            nodes_[n].child = -1;
        }
    } else if (nodes_[n].child >= 0) {
        int32_t c = nodes_[n].child;
        for (int i = 0; i < 4; i++) dereg(c + i, key);
    }
}

// CDEngine::register_hazard (cd_engine.rs:59-70) with QTHazard::from_root (qt_hazard.rs:36-43)
uint32_t QuadTree::insert(HazardRec&& h) {
    uint32_t k;
    if (!free_keys_.empty()) {   // a freed key is reused last-in first-out, like slotmap
        k = free_keys_.back();
        free_keys_.pop_back();
    } else {
        k = (uint32_t)haz_.size();
        haz_.emplace_back();
    }
    h.alive = true;
    h.shape.bbox = bounding_box(h.shape.v.data(), h.shape.v.size());
    haz_[k] = std::move(h);
    if (haz_[k].kind == KIND_EXTERIOR && exterior_ < 0) exterior_ = (int32_t)k;
    const Polygon& s = haz_[k].shape;
    auto edges = std::make_shared<std::vector<Seg>>();
    size_t nv = s.v.size();
    edges->reserve(nv);
    for (size_t i = 0; i < nv; i++) edges->push_back(Seg{s.v[i], s.v[i + 1 == nv ? 0 : i + 1]});
    NodeHaz root_h{k, PRES_PARTIAL, haz_[k].kind, s.bbox, std::move(edges)};
    reg(0, root_h);
    version_++;
    return k;
}

// CDEngine::deregister_hazard_by_key (cd_engine.rs:87-96)
bool QuadTree::remove(uint32_t k) {
    if (k >= haz_.size() || !haz_[k].alive) return false;
    dereg(0, k);
    haz_[k].alive = false;
    haz_[k].shape = Polygon{};
    haz_[k].poles.clear();
    if ((int32_t)k == exterior_) exterior_ = -1;
    free_keys_.push_back(k);
    version_++;
    return true;
}

void QuadTree::flatten(FlatTree& out) const {
    out.nodes.clear();
    out.nedges.clear();
    out.strength.clear();
    out.entries.clear();
    out.edges.clear();
    for (auto& c : out.cbox) c.clear();
    // breadth-first so that every quartet of children stays contiguous
    std::vector<int32_t> order{0};
    std::vector<int32_t> newid(nodes_.size(), -1);
    newid[0] = 0;
    for (size_t i = 0; i < order.size(); i++) {
        const HNode& n = nodes_[order[i]];
        if (n.child >= 0)
            for (int k = 0; k < 4; k++) {
                newid[n.child + k] = (int32_t)order.size();
                order.push_back(n.child + k);
            }
    }
    out.nodes.resize(order.size());
    out.nedges.resize(order.size());
    out.strength.resize(order.size());
    for (size_t i = 0; i < order.size(); i++) {
        const HNode& n = nodes_[order[i]];
        DNode& d = out.nodes[i];
        d.box = n.bbox;
        d.child = n.child >= 0 ? newid[n.child] : -1;
        d.parent = n.parent >= 0 ? newid[n.parent] : -1;
        d.hz_off = (uint32_t)out.entries.size();
        d.hz_cnt = (uint32_t)n.hz.size();
        out.nedges[i] = n.n_active_edges;
        out.strength[i] = n.hz.empty() ? 0 : (uint8_t)n.hz[0].presence;
        // edges are only read at nodes where a probe can test them: leaves (detect and collect)
        // and nodes at or under the cd_threshold (collect tests hazards there, qt_node.rs:157)
        bool keep_edges = n.child < 0 || n.n_active_edges <= cdt_;
        for (const NodeHaz& h : n.hz) {
            DEntry e;
            e.ff = h.ff;
            e.hkey = h.hkey;
            e.presence = h.presence;
            e.edge_off = (uint32_t)(out.edges.size() / 4);
            e.edge_cnt = 0;
            if (h.presence == PRES_PARTIAL && keep_edges) {
                while ((out.edges.size() / 4) % EDGE_ALIGN) out.edges.push_back(0.0f);   // lists start on a tile
                e.edge_off = (uint32_t)(out.edges.size() / 4);
                for (size_t j = 0; j < h.edges->size(); j++) {
                    const Seg& s = (*h.edges)[j];
                    out.edges.push_back(s.s.x);
                    out.edges.push_back(s.s.y);
                    out.edges.push_back(s.e.x);
                    out.edges.push_back(s.e.y);
                    const Box b{fmn(s.s.x, s.e.x), fmn(s.s.y, s.e.y), fmx(s.s.x, s.e.x), fmx(s.s.y, s.e.y)};
                    for (int t = 0; t < EDGE_TILES; t++) {
                        const size_t g = (e.edge_off + j) >> (2 + t);
                        std::vector<Box>& cb = out.cbox[t];
                        if (cb.size() <= g) cb.resize(g + 1, Box{INFINITY, INFINITY, -INFINITY, -INFINITY});
                        Box& c = cb[g];
                        c = Box{fmn(c.x0, b.x0), fmn(c.y0, b.y0), fmx(c.x1, b.x1), fmx(c.y1, b.y1)};
                    }
                }
                e.edge_cnt = (uint32_t)h.edges->size();
            }
            out.entries.push_back(e);
        }
    }
}

static inline uint32_t fb(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
static void dump_box(std::vector<uint32_t>& o, const Box& b) {
    o.push_back(fb(b.x0));
    o.push_back(fb(b.y0));
    o.push_back(fb(b.x1));
    o.push_back(fb(b.y1));
}

void QuadTree::dump_node(int32_t ni, std::vector<uint32_t>& o) const {
    const HNode& n = nodes_[ni];
    o.push_back(n.level);
    o.push_back(n.child >= 0 ? 1u : 0u);
    o.push_back((uint32_t)n.hz.size());
    o.push_back(n.n_active_edges);
    dump_box(o, n.bbox);
    std::vector<const NodeHaz*> hs;
    for (const NodeHaz& h : n.hz) hs.push_back(&h);
    std::sort(hs.begin(), hs.end(), [](const NodeHaz* a, const NodeHaz* b) { return a->hkey < b->hkey; });
    for (const NodeHaz* h : hs) {
        o.push_back(h->hkey);
        o.push_back(h->presence);
        if (h->presence == PRES_PARTIAL) {
            dump_box(o, h->ff);
            std::vector<std::array<uint32_t, 4>> es;
            for (const Seg& s : *h->edges) es.push_back({fb(s.s.x), fb(s.s.y), fb(s.e.x), fb(s.e.y)});
            std::sort(es.begin(), es.end());
            o.push_back((uint32_t)es.size());
            for (auto& e : es) o.insert(o.end(), e.begin(), e.end());
        }
    }
    if (n.child >= 0)
        for (int i = 0; i < 4; i++) dump_node(n.child + i, o);
}

void QuadTree::dump(std::vector<uint32_t>& out) const {
    out.clear();
    dump_node(0, out);
}

}  // namespace jcde
