// ref_simplify.cpp — exposes the reference's own grid vertex clustering
// (src/simplify/simplify.cpp, compiled from its sources where they lie) to the oracle
// tests and the fixture generator. Test infrastructure only; built into oracle/_ref by
// `make ref`.
#include "src/simplify/simplify.cpp"

#include <cstring>

// Returns the number of output points (out_pts: 3 per point, out_tris: 3 per kept
// triangle, *nout_tris of them; capacities in points / triangles), or -1 with the
// reference's message in err.
extern "C" long long ref_simplify(const double* pts, long long npts, const int* tris,
                                  long long ntris, int grid, double* out_pts, long long pcap,
                                  int* out_tris, long long tcap, long long* nout_tris, char* err,
                                  long long errlen) {
    cmg::PLC plc;
    plc.index_base = cmg::IndexBase::Zero;
    for (long long i = 0; i < npts; ++i)
        plc.points.push_back(cmg::Point3{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]});
    for (long long t = 0; t < ntris; ++t) {
        cmg::Facet f;
        cmg::Polygon p;
        p.vertices = {tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]};
        f.polygons.push_back(p);
        plc.facets.push_back(f);
    }
    cmg::simplify::SimplifyOptions o;
    o.grid = grid;
    auto r = cmg::simplify::simplify(plc, o);
    *nout_tris = 0;
    if (!r) {
        std::strncpy(err, r.error().message.c_str(), static_cast<size_t>(errlen - 1));
        err[errlen - 1] = '\0';
        return -1;
    }
    const long long np = static_cast<long long>(r->points.size());
    for (long long i = 0; i < np && i < pcap; ++i) {
        out_pts[3 * i] = r->points[i].x;
        out_pts[3 * i + 1] = r->points[i].y;
        out_pts[3 * i + 2] = r->points[i].z;
    }
    long long m = 0;
    for (const auto& f : r->facets)
        for (const auto& p : f.polygons) {
            if (m < tcap)
                for (int c = 0; c < 3; ++c) out_tris[3 * m + c] = p.vertices[c];
            ++m;
        }
    *nout_tris = m;
    return np;
}
