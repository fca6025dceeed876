// cmg/core/plc.hpp — the piecewise-linear complex handed to voxelize.
//
// Replaces include/cmg/core/plc.hpp of the reference for the voxelization path, with
// the same members in the same order. The voxelizer reads `points` and the polygons
// of every facet (each polygon fan-triangulated, hole polygons included, as the
// reference's boundary_triangles does); holes, regions and markers are carried but
// not read.
#pragma once

#include <vector>

#include "cmg/core/geometry.hpp"

namespace cmg {

struct Polygon {
    std::vector<Index> vertices;  // a closed loop of point indices
};

struct Facet {
    std::vector<Polygon> polygons;
    std::vector<Point3> holes;
    int marker = 0;
};

struct Region {
    Point3 seed;
    Real attribute = 0;
    Real max_volume = -1;  // negative: unconstrained
};

class PLC {
public:
    std::vector<Point3> points;
    std::vector<Facet> facets;
    std::vector<Point3> holes;
    std::vector<Region> regions;
    IndexBase index_base = IndexBase::Zero;

    bool empty() const noexcept { return points.empty() && facets.empty(); }
};

}  // namespace cmg
