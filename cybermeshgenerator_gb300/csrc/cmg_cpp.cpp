// cmg_cpp.cpp — the C++ surface of libcmg_c.so: cmg::voxelize::voxelize
// (include/cmg/voxelize/voxelize.hpp), the drop-in for the reference's
// cmg::voxelize::voxelize (include/cmg/voxelize/voxelize.hpp:63 of the reference).
//
// The PLC's facets are fan-triangulated here as the reference's boundary_triangles
// does (src/voxelize/voxelize.cpp:29-38: every polygon of every facet, in order,
// (v0, v[i-1], v[i])); its points are read in place (Point3 is three packed doubles).
// Validation, grid and GPU pipeline are those of cmg_plc_voxelize. Built with
// -std=c++20, as the reference is, so that cmg::expected has the reference's layout.
#include "cmg/voxelize/voxelize.hpp"

#include <cstring>
#include <exception>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/cmg_c/cmg_c.h"

static_assert(std::is_same_v<cmg::Real, double>, "FP64 coordinates");
static_assert(std::is_standard_layout_v<cmg::Point3> && sizeof(cmg::Point3) == 24,
              "Point3 is three packed doubles");

namespace cmg::gpu {
cmg_status voxelize_host(const double* pts, int64_t npts, const int* tris, int64_t ntris,
                         int resolution, int pad, int mode, cmg_voxels** out, std::string* msg);
}

namespace cmg::voxelize {

namespace {

MeshErrorCode to_code(cmg_status st) {
    switch (st) {
        case CMG_ERR_INVALID_INPUT: return MeshErrorCode::InvalidInput;
        case CMG_ERR_SELF_INTERSECTION: return MeshErrorCode::SelfIntersection;
        case CMG_ERR_UNSUPPORTED_OPTION: return MeshErrorCode::UnsupportedOption;
        case CMG_ERR_QUALITY_NOT_MET: return MeshErrorCode::QualityNotMet;
        case CMG_ERR_NOT_IMPLEMENTED: return MeshErrorCode::NotImplemented;
        default: return MeshErrorCode::Internal;
    }
}

// Owns a cmg_voxels handle for the duration of the copy-out.
struct Handle {
    cmg_voxels* h = nullptr;
    ~Handle() { cmg_voxels_destroy(h); }
};

}  // namespace

expected<VoxelGrid, MeshError> voxelize(const PLC& plc, const VoxelOptions& opts) {
    try {
        std::vector<int> tris;
        size_t n = 0;
        for (const Facet& f : plc.facets)
            for (const Polygon& poly : f.polygons)
                if (poly.vertices.size() >= 3) n += 3 * (poly.vertices.size() - 2);
        tris.reserve(n);
        for (const Facet& f : plc.facets)
            for (const Polygon& poly : f.polygons) {
                const std::vector<Index>& v = poly.vertices;
                for (size_t i = 2; i < v.size(); ++i) {
                    tris.push_back(v[0]);
                    tris.push_back(v[i - 1]);
                    tris.push_back(v[i]);
                }
            }
        const int mode = opts.mode == VoxelMode::SignedDistance ? 1 : 0;
        Handle g;
        std::string msg;
        const cmg_status st = cmg::gpu::voxelize_host(
            plc.points.empty() ? nullptr : &plc.points[0].x, static_cast<int64_t>(plc.points.size()),
            tris.data(), static_cast<int64_t>(tris.size() / 3), opts.resolution, opts.pad, mode,
            &g.h, &msg);
        if (st != CMG_OK) return unexpected<MeshError>(MeshError{to_code(st), msg});
        VoxelGrid out;
        cmg_voxels_dims(g.h, &out.nx, &out.ny, &out.nz);
        cmg_voxels_origin(g.h, &out.origin.x, &out.origin.y, &out.origin.z);
        out.spacing = cmg_voxels_spacing(g.h);
        const size_t cells = out.cell_count();
        if (mode == 1) {
            const float* d = cmg_voxels_distance(g.h);
            out.distance.assign(d, d + cells);
        } else {
            const unsigned char* o = cmg_voxels_occupancy(g.h);
            out.occupancy.assign(o, o + cells);
        }
        return out;
    } catch (const std::exception& e) {
        return unexpected<MeshError>(MeshError{MeshErrorCode::Internal, e.what()});
    } catch (...) {
        return unexpected<MeshError>(MeshError{MeshErrorCode::Internal, "unknown error"});
    }
}

}  // namespace cmg::voxelize
