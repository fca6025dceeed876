// ref_harness.cpp — exposes the reference's own voxelizer and predicates as C
// functions, for pinning the oracle restatement (TEST INFRASTRUCTURE ONLY).
//
// Built by oracle/Makefile into oracle/_ref/ from the reference sources where they
// lie (REF_ROOT). The reference's voxelize.cpp is #included so that its internal
// functions (make_grid, build_xy_buckets, classify_occupancy, point_tri_dist2,
// fill_distance) can be driven on explicit grids; src/predicates/predicates.cpp
// (at -O0, as the reference ships it) and src/predicates/robust.cpp are linked.
#include "src/voxelize/voxelize.cpp"

#include <cstdint>
#include <cstring>
#include <limits>

namespace cmg::predicates {
REAL orient3dexact(REAL* pa, REAL* pb, REAL* pc, REAL* pd);
REAL insphereexact(REAL* pa, REAL* pb, REAL* pc, REAL* pd, REAL* pe);
} // namespace cmg::predicates

namespace {

cmg::PLC make_plc(const double* pts, int64_t npts, const int* idx,
                  const int64_t* off, int64_t nfacets) {
    cmg::PLC p;
    for (int64_t i = 0; i < npts; ++i)
        p.points.push_back({pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]});
    for (int64_t f = 0; f < nfacets; ++f) {
        cmg::Facet fa;
        cmg::Polygon poly;
        for (int64_t k = off[f]; k < off[f + 1]; ++k) poly.vertices.push_back(idx[k]);
        fa.polygons.push_back(std::move(poly));
        p.facets.push_back(std::move(fa));
    }
    return p;
}

cmg::voxelize::Grid to_grid(const double* corner, double spacing, const int* dims) {
    cmg::voxelize::Grid g;
    for (int a = 0; a < 3; ++a) g.corner[a] = corner[a];
    g.spacing = spacing;
    g.nx = dims[0];
    g.ny = dims[1];
    g.nz = dims[2];
    return g;
}

std::vector<cmg::Point3> to_points(const double* pts, int64_t npts) {
    std::vector<cmg::Point3> v;
    v.reserve(static_cast<std::size_t>(npts));
    for (int64_t i = 0; i < npts; ++i) v.push_back({pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]});
    return v;
}

std::vector<cmg::voxelize::Tri> to_tris(const int* tris, int64_t ntris) {
    std::vector<cmg::voxelize::Tri> v(static_cast<std::size_t>(ntris));
    for (int64_t t = 0; t < ntris; ++t) v[t] = {tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]};
    return v;
}

} // namespace

extern "C" {

// make_grid over the point set: corner[3], spacing, dims[3]. Returns 0 or -1.
int ref_make_grid(const double* pts, int64_t npts, int resolution, int pad,
                  double* corner, double* spacing, int* dims) {
    cmg::voxelize::VoxelOptions o;
    o.resolution = resolution;
    o.pad = pad;
    auto g = cmg::voxelize::make_grid(to_points(pts, npts), o);
    for (int a = 0; a < 3; ++a) corner[a] = g.corner[a];
    *spacing = g.spacing;
    dims[0] = g.nx;
    dims[1] = g.ny;
    dims[2] = g.nz;
    return g.spacing > 0 ? 0 : -1;
}

// The public entry point cmg::voxelize::voxelize on a PLC of polygon facets.
// Writes origin[3], spacing, dims[3]; copies occupancy (mode 0) or float distance
// (mode 1) into out when out_cap (in cells) is large enough. Returns 0 on success,
// 1 + MeshErrorCode on a voxelize error, -2 if out_cap is too small.
int ref_voxelize(const double* pts, int64_t npts, const int* idx, const int64_t* off,
                 int64_t nfacets, int resolution, int pad, int mode, double* origin,
                 double* spacing, int* dims, void* out, int64_t out_cap) {
    cmg::voxelize::VoxelOptions o;
    o.resolution = resolution;
    o.pad = pad;
    o.mode = mode == 1 ? cmg::voxelize::VoxelMode::SignedDistance
                       : cmg::voxelize::VoxelMode::Occupancy;
    auto r = cmg::voxelize::voxelize(make_plc(pts, npts, idx, off, nfacets), o);
    if (!r) return 1 + static_cast<int>(r.error().code);
    origin[0] = r->origin.x;
    origin[1] = r->origin.y;
    origin[2] = r->origin.z;
    *spacing = r->spacing;
    dims[0] = r->nx;
    dims[1] = r->ny;
    dims[2] = r->nz;
    int64_t n = static_cast<int64_t>(r->cell_count());
    if (out_cap < n) return -2;
    if (mode == 1)
        std::memcpy(out, r->distance.data(), sizeof(float) * n);
    else
        std::memcpy(out, r->occupancy.data(), n);
    return 0;
}

// classify_occupancy on an explicit grid.
void ref_occupancy_grid(const double* pts, int64_t npts, const int* tris, int64_t ntris,
                        const double* corner, double spacing, const int* dims,
                        uint8_t* occ) {
    cmg::robust::ensure_initialized();
    auto g = to_grid(corner, spacing, dims);
    auto P = to_points(pts, npts);
    auto T = to_tris(tris, ntris);
    auto buckets = cmg::voxelize::build_xy_buckets(g, P, T);
    auto o = cmg::voxelize::classify_occupancy(g, P, T, buckets);
    std::memcpy(occ, o.data(), o.size());
}

// fill_distance (ring search, float output) on an explicit grid.
void ref_fill_distance(const double* pts, int64_t npts, const int* tris, int64_t ntris,
                       const double* corner, double spacing, const int* dims,
                       const uint8_t* occ, float* dist) {
    auto g = to_grid(corner, spacing, dims);
    auto P = to_points(pts, npts);
    auto T = to_tris(tris, ntris);
    std::vector<std::uint8_t> o(occ, occ + static_cast<std::size_t>(dims[0]) * dims[1] * dims[2]);
    auto d = cmg::voxelize::fill_distance(g, P, T, o);
    std::memcpy(dist, d.data(), sizeof(float) * d.size());
}

// Brute-force minimum of the reference's point_tri_dist2 at the listed voxel
// centres (the FP64 SDF magnitude squared before the float cast).
void ref_dist2_brute(const double* pts, int64_t npts, const int* tris, int64_t ntris,
                     const double* corner, double spacing, const int* dims,
                     const int64_t* vox, int64_t nq, double* d2) {
    (void)npts;
    const int64_t nxy = static_cast<int64_t>(dims[0]) * dims[1];
    for (int64_t q = 0; q < nq; ++q) {
        int64_t idx = vox[q];
        int k = static_cast<int>(idx / nxy);
        int j = static_cast<int>((idx % nxy) / dims[0]);
        int i = static_cast<int>(idx % dims[0]);
        double p[3] = {corner[0] + (i + 0.5) * spacing, corner[1] + (j + 0.5) * spacing,
                       corner[2] + (k + 0.5) * spacing};
        double best = std::numeric_limits<double>::max();
        for (int64_t t = 0; t < ntris; ++t) {
            double a[3], b[3], c[3];
            for (int x = 0; x < 3; ++x) {
                a[x] = pts[3 * tris[3 * t] + x];
                b[x] = pts[3 * tris[3 * t + 1] + x];
                c[x] = pts[3 * tris[3 * t + 2] + x];
            }
            best = std::min(best, cmg::voxelize::point_tri_dist2(p, a, b, c));
        }
        d2[q] = best;
    }
}

// The reference ring search for the listed voxels, including the 3-D bucket
// build (for timing a bounded sample). Returns the squared distances.
void ref_ring_sample(const double* pts, int64_t npts, const int* tris, int64_t ntris,
                     const double* corner, double spacing, const int* dims,
                     const int64_t* vox, int64_t nq, double* d2) {
    auto g = to_grid(corner, spacing, dims);
    auto P = to_points(pts, npts);
    auto T = to_tris(tris, ntris);
    std::vector<std::array<double, 3>> tri_pts(T.size() * 3);
    for (std::size_t t = 0; t < T.size(); ++t)
        for (int v = 0; v < 3; ++v) {
            const auto& p = P[T[t][v]];
            tri_pts[t * 3 + v] = {p.x, p.y, p.z};
        }
    const auto buckets = cmg::voxelize::build_xyz_buckets(g, P, T);
    std::vector<int> seen(T.size(), -1);
    const int64_t nxy = static_cast<int64_t>(dims[0]) * dims[1];
    for (int64_t q = 0; q < nq; ++q) {
        int64_t idx = vox[q];
        int k = static_cast<int>(idx / nxy);
        int j = static_cast<int>((idx % nxy) / dims[0]);
        int i = static_cast<int>(idx % dims[0]);
        double p[3] = {corner[0] + (i + 0.5) * spacing, corner[1] + (j + 0.5) * spacing,
                       corner[2] + (k + 0.5) * spacing};
        d2[q] = cmg::voxelize::nearest_tri_dist2(g, i, j, k, p, buckets, tri_pts, seen,
                                                 static_cast<int>(q));
    }
}

double ref_orient3d(const double* a, const double* b, const double* c, const double* d) {
    return cmg::robust::orient3d({a[0], a[1], a[2]}, {b[0], b[1], b[2]},
                                 {c[0], c[1], c[2]}, {d[0], d[1], d[2]});
}

double ref_insphere(const double* a, const double* b, const double* c, const double* d,
                    const double* e) {
    return cmg::robust::insphere({a[0], a[1], a[2]}, {b[0], b[1], b[2]},
                                 {c[0], c[1], c[2]}, {d[0], d[1], d[2]},
                                 {e[0], e[1], e[2]});
}

double ref_orient3dexact(const double* a, const double* b, const double* c,
                         const double* d) {
    cmg::robust::ensure_initialized();
    double pa[3] = {a[0], a[1], a[2]}, pb[3] = {b[0], b[1], b[2]};
    double pc[3] = {c[0], c[1], c[2]}, pd[3] = {d[0], d[1], d[2]};
    return cmg::predicates::orient3dexact(pa, pb, pc, pd);
}

double ref_insphereexact(const double* a, const double* b, const double* c,
                         const double* d, const double* e) {
    cmg::robust::ensure_initialized();
    double pa[3] = {a[0], a[1], a[2]}, pb[3] = {b[0], b[1], b[2]};
    double pc[3] = {c[0], c[1], c[2]}, pd[3] = {d[0], d[1], d[2]};
    double pe[3] = {e[0], e[1], e[2]};
    return cmg::predicates::insphereexact(pa, pb, pc, pd, pe);
}

} // extern "C"
