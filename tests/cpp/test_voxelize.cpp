// C++ surface test: cmg::voxelize::voxelize from libcmg_c.so, written as a program
// that uses the reference's C++ API would be (include/cmg/voxelize/voxelize.hpp).
//
//   test_voxelize validate          checks the InvalidInput answers (no GPU call)
//   test_voxelize run IN OUT        voxelizes the mesh in IN (see read_case) in both
//                                   modes and writes OUT (see write_grid)
//
// Exit status 0 when every check passes.
#include <cmg/voxelize/voxelize.hpp>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

namespace {

int failures = 0;

void check(bool ok, const std::string& what) {
    if (!ok) {
        std::fprintf(stderr, "FAIL: %s\n", what.c_str());
        ++failures;
    }
}

cmg::PLC tetra() {
    cmg::PLC p;
    p.points = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (auto t : {std::vector<int>{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}}) {
        cmg::Facet f;
        f.polygons.push_back(cmg::Polygon{t});
        p.facets.push_back(f);
    }
    return p;
}

void expect_invalid(const cmg::PLC& p, const cmg::voxelize::VoxelOptions& o, const char* msg) {
    auto r = cmg::voxelize::voxelize(p, o);
    check(!r.has_value(), std::string("rejected: ") + msg);
    if (!r) {
        check(r.error().code == cmg::MeshErrorCode::InvalidInput, std::string("InvalidInput: ") + msg);
        check(r.error().message == msg, "message '" + r.error().message + "' == '" + msg + "'");
    }
}

int validate() {
    cmg::voxelize::VoxelOptions o;
    o.resolution = 0;
    expect_invalid(tetra(), o, "voxelize: resolution must be >= 1");
    o.resolution = 8;
    expect_invalid(cmg::PLC{}, o, "voxelize: PLC has no points");
    cmg::PLC pts_only = tetra();
    pts_only.facets.clear();
    expect_invalid(pts_only, o, "voxelize: PLC has no boundary triangles");
    cmg::PLC two = tetra();  // facets of fewer than three corners fan to nothing
    two.facets.clear();
    two.facets.push_back(cmg::Facet{{cmg::Polygon{{0, 1}}}, {}, 0});
    expect_invalid(two, o, "voxelize: PLC has no boundary triangles");
    cmg::PLC flat;
    flat.points = {{1, 1, 1}, {1, 1, 1}, {1, 1, 1}};
    flat.facets.push_back(cmg::Facet{{cmg::Polygon{{0, 1, 2}}}, {}, 0});
    expect_invalid(flat, o, "voxelize: degenerate (zero-extent) PLC");
    cmg::PLC bad = tetra();
    bad.facets[2].polygons[0].vertices[1] = 4;
    expect_invalid(bad, o, "voxelize: facet vertex index out of range");
    // defaults of the options, as the reference's
    cmg::voxelize::VoxelOptions d;
    check(d.resolution == 64 && d.pad == 1 && d.mode == cmg::voxelize::VoxelMode::Occupancy,
          "VoxelOptions defaults");
    cmg::voxelize::VoxelGrid g;
    g.nx = 3, g.ny = 4, g.nz = 5;
    check(g.index(2, 3, 4) == (4 * 4 + 3) * 3 + 2 && g.cell_count() == 60, "index layout");
    return failures;
}

// IN: int64 npoints, npoints*3 doubles, int64 nfacets, per facet int64 ncorners and
// that many int32 indices, int32 resolution, int32 pad.
bool read_case(const char* path, cmg::PLC& p, cmg::voxelize::VoxelOptions& o) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    auto get = [&](void* dst, size_t n) { f.read(static_cast<char*>(dst), static_cast<std::streamsize>(n)); };
    int64_t np = 0, nf = 0;
    get(&np, 8);
    p.points.resize(static_cast<size_t>(np));
    get(p.points.data(), 24 * static_cast<size_t>(np));
    get(&nf, 8);
    for (int64_t i = 0; i < nf; ++i) {
        int64_t k = 0;
        get(&k, 8);
        cmg::Polygon poly;
        poly.vertices.resize(static_cast<size_t>(k));
        get(poly.vertices.data(), 4 * static_cast<size_t>(k));
        cmg::Facet fa;
        fa.polygons.push_back(std::move(poly));
        p.facets.push_back(std::move(fa));
    }
    get(&o.resolution, 4);
    get(&o.pad, 4);
    return static_cast<bool>(f);
}

// OUT: int32 nx ny nz, double origin[3], double spacing, then nx*ny*nz occupancy bytes
// and nx*ny*nz floats of the signed distance.
int run(const char* in, const char* out) {
    cmg::PLC p;
    cmg::voxelize::VoxelOptions o;
    if (!read_case(in, p, o)) {
        std::fprintf(stderr, "cannot read %s\n", in);
        return 2;
    }
    auto occ = cmg::voxelize::voxelize(p, o);
    o.mode = cmg::voxelize::VoxelMode::SignedDistance;
    auto sdf = cmg::voxelize::voxelize(p, o);
    check(occ.has_value(), "occupancy call: " + (occ ? std::string() : occ.error().message));
    check(sdf.has_value(), "distance call: " + (sdf ? std::string() : sdf.error().message));
    if (!occ || !sdf) return 1;
    const cmg::voxelize::VoxelGrid& a = *occ;
    const cmg::voxelize::VoxelGrid& b = sdf.value();
    check(a.distance.empty() && a.occupancy.size() == a.cell_count(), "occupancy mode: one output");
    check(b.occupancy.empty() && b.distance.size() == b.cell_count(), "distance mode: one output");
    check(a.nx == b.nx && a.ny == b.ny && a.nz == b.nz && a.origin == b.origin &&
              a.spacing == b.spacing, "same grid in both modes");
    std::ofstream f(out, std::ios::binary);
    int32_t dims[3] = {a.nx, a.ny, a.nz};
    f.write(reinterpret_cast<const char*>(dims), sizeof(dims));
    f.write(reinterpret_cast<const char*>(&a.origin.x), 24);
    f.write(reinterpret_cast<const char*>(&a.spacing), 8);
    f.write(reinterpret_cast<const char*>(a.occupancy.data()), static_cast<std::streamsize>(a.occupancy.size()));
    f.write(reinterpret_cast<const char*>(b.distance.data()),
            static_cast<std::streamsize>(4 * b.distance.size()));
    return failures;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc >= 2 && std::strcmp(argv[1], "validate") == 0) return validate() ? 1 : 0;
    if (argc >= 4 && std::strcmp(argv[1], "run") == 0) return run(argv[2], argv[3]) ? 1 : 0;
    std::fprintf(stderr, "usage: %s validate | run IN OUT\n", argv[0]);
    return 2;
}
