// Host preparation of shapes (see prep.cpp).
#pragma once
#include <cstdint>
#include <vector>

#include "geom.cuh"

namespace jcde {

struct PreparedPolygon {
    std::vector<Pt> v;   // counter-clockwise
    Box bbox;
    float area;
    float diameter;
    Disk poi;            // pole of inaccessibility
};

struct PoleLimit {
    uint32_t n;
    float coverage;
};

float polygon_area(const Pt* v, size_t n);
// SPolygon::new (simple_polygon.rs:41-71): 0 on success, -1 for an invalid polygon; without
// `with_poi` the poi is left zero (computed elsewhere, e.g. by the device batch)
int spolygon_new(std::vector<Pt> pts, PreparedPolygon* out, bool with_poi = true);
// close_narrow_concavities (shape_modification.rs:374-478) after SPolygon::new of pts: 0, -1 for
// an invalid input polygon, -2 when a bridge leaves an invalid polygon (the reference panics)
int close_concavities(std::vector<Pt> pts, bool deflate, float ratio, std::vector<Pt>* out);
// generate_surrogate_poles (pole.rs:12-47) of an internal shape with the given area and poi
int surrogate_poles(const std::vector<Pt>& v, float area, Disk poi, const PoleLimit* lim, int n_lim,
                    std::vector<Disk>* poles);

}  // namespace jcde
