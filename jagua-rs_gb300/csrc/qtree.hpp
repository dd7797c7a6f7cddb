// Host-side quadtree of the CDE: hazard registry, incremental register / deregister, and the
// flattening into the structure-of-arrays image that the sm_103a kernels walk.
//
// The tree follows collision_detection/quadtree/ of jagua-rs: a node holds the hazards present in
// it (Entire before Partial, qt_hazard_vec.rs:24-63), grows four children the first time a Partial
// hazard reaches it (qt_node.rs:38-81) and drops them when its last Partial hazard leaves
// (qt_node.rs:83-94).  Its shape is therefore a function of the registered hazard set only.
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

#include "geom.cuh"

namespace jcde {

enum Presence : uint32_t { PRES_NONE = 0, PRES_PARTIAL = 1, PRES_ENTIRE = 2 };

// Edge tiles: the edge list of every entry starts on a multiple of EDGE_ALIGN edges, and for each
// tile size 4 << t (t = 0, 1, 2) every tile of consecutive edges of a list has a bounding box
// (FlatTree::cbox[t]); the query kernels use one of the three (jcde_tuning.edge_tile).
constexpr uint32_t EDGE_ALIGN = 16;
constexpr int EDGE_TILES = 3;
constexpr uint32_t EDGE_TILE_DEFAULT = 8;
enum Kind : int32_t { KIND_PLACED_ITEM = 0, KIND_EXTERIOR = 1, KIND_HOLE = 2, KIND_QUALITY_ZONE = 3 };
inline bool kind_is_exterior(int32_t k) { return k == KIND_EXTERIOR; }  // hazard.rs:55-62

struct Polygon {
    std::vector<Pt> v;
    Box bbox;
    Disk poi;
};

struct HazardRec {
    int32_t kind = 0;
    bool dynamic = false;
    bool alive = false;
    uint64_t tag = 0;   // caller's entity identity (placed-item key, zone index, ...)
    Polygon shape;
    std::vector<Disk> poles;   // surrogate poles of the shape (SPolygon::surrogate), optional
};

struct NodeHaz {
    uint32_t hkey;
    Presence presence;
    int32_t kind;
    Box ff;                                          // QTHazPartial::ff_bbox
    std::shared_ptr<const std::vector<Seg>> edges;   // QTHazPartial::edges (shared with parents)
    uint32_t n_edges() const { return presence == PRES_PARTIAL ? (uint32_t)edges->size() : 0u; }
};

struct HNode {
    Box bbox;
    uint8_t level = 0;
    int32_t child = -1;   // first of four consecutive children in the pool, -1 for none
    int32_t parent = -1;
    std::vector<NodeHaz> hz;
    uint32_t n_active_edges = 0;
};

// Flattened image (device layout; see kernels.cuh for the readers).
struct alignas(16) DNode {
    Box box;
    int32_t child, parent;
    uint32_t hz_off, hz_cnt;
};
struct alignas(16) DEntry {
    Box ff;
    uint32_t hkey, edge_off, edge_cnt, presence;
};
struct alignas(16) DHaz {
    Box box;
    float poi_x, poi_y;
    uint32_t v_off;
    uint32_t v_cnt_scope;   // vertex count, bit 31 set for an exterior-scoped hazard
};
struct alignas(16) DItem {
    uint32_t v_off, v_cnt, pole_off, n_ff_poles;
    uint32_t pier_off, n_piers;
    float poi_x, poi_y;
    uint32_t n_poles;       // all surrogate poles (the proxy uses every pole, probes only the ff ones)
    float pole_r2max;       // largest squared distance of a pole centre from the item origin
    float pole_bound;       // radius around the item origin that holds every pole
    uint32_t pad0;
};

struct FlatTree {
    std::vector<DNode> nodes;
    std::vector<uint32_t> nedges;   // n_active_edges per node (collect's cd_threshold rule)
    std::vector<uint8_t> strength;  // strongest presence per node with no filter
    std::vector<DEntry> entries;
    std::vector<float> edges;       // 4 floats per edge (x1, y1, x2, y2); every list starts at a group boundary
    std::vector<Box> cbox[EDGE_TILES];   // bounding box of each tile of 4 << t edges of one list
};

class QuadTree {
  public:
    QuadTree(uint8_t depth, uint8_t cd_threshold, Box bbox);

    uint32_t insert(HazardRec&& h);          // registry insert + quadtree registration -> key
    bool remove(uint32_t key);               // quadtree deregistration + registry removal
    const HazardRec* hazard(uint32_t key) const {
        return key < haz_.size() && haz_[key].alive ? &haz_[key] : nullptr;
    }
    uint32_t n_slots() const { return (uint32_t)haz_.size(); }
    const std::vector<uint32_t>& free_keys() const { return free_keys_; }   // next reused key last
    const std::vector<HazardRec>& hazards() const { return haz_; }
    int32_t exterior_key() const { return exterior_; }
    Box bbox() const { return nodes_[0].bbox; }
    uint8_t cd_threshold() const { return cdt_; }

    void flatten(FlatTree& out) const;                 // breadth-first, quartets contiguous
    void dump(std::vector<uint32_t>& out) const;       // canonical form (tests)
    uint64_t version() const { return version_; }
    // surrogate poles of a registered hazard (used by the overlap proxy); false for an unknown key
    bool set_poles(uint32_t key, std::vector<Disk>&& poles) {
        if (key >= haz_.size() || !haz_[key].alive) return false;
        haz_[key].poles = std::move(poles);
        pole_version_++;
        return true;
    }
    uint64_t pole_version() const { return pole_version_ + version_; }

  private:
    int32_t alloc_quartet(int32_t parent);
    void free_subtree(int32_t first_child);
    void reg(int32_t n, const NodeHaz& h);
    void reg_children(int32_t n, const NodeHaz& h);
    void dereg(int32_t n, uint32_t key);
    void constrict(const NodeHaz& h, const Box q[4], NodeHaz out[4]) const;
    void dump_node(int32_t n, std::vector<uint32_t>& out) const;

    std::vector<HNode> nodes_;
    std::vector<int32_t> free_quartets_;
    std::vector<HazardRec> haz_;
    std::vector<uint32_t> free_keys_;
    uint8_t cdt_;
    int32_t exterior_ = -1;
    uint64_t version_ = 0;
    uint64_t pole_version_ = 0;
};

// simple_polygon.rs:255-292 — ray-cast point in polygon with the FPA vertex guard
bool polygon_contains(const Polygon& poly, Pt p);
// simple_polygon.rs:122-133
Box bounding_box(const Pt* v, size_t n);

}  // namespace jcde
