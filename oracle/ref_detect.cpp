// ref_detect.cpp — exposes the reference's own self-intersection detector
// (src/detect/self_intersection.cpp, compiled from its sources where they lie) to the
// oracle tests and the fixture generator. Test infrastructure only; built into
// oracle/_ref by `make ref`.
#include "src/detect/self_intersection.cpp"

#include <vector>

extern "C" long long ref_self_intersections(const double* pts, long long npts, const int* tris,
                                            long long ntris, int* out, long long cap) {
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
    const auto hits = cmg::detect::self_intersections(plc);
    long long n = 0;
    for (const auto& h : hits) {
        if (n < cap) {
            int* o = out + 8 * n;
            o[0] = h.facet_a;
            o[1] = h.facet_b;
            for (int k = 0; k < 3; ++k) {
                o[2 + k] = h.tri_a[k];
                o[5 + k] = h.tri_b[k];
            }
        }
        ++n;
    }
    return n;
}
