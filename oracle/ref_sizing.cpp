// ref_sizing.cpp — exposes the reference's own background sizing field
// (src/sizing/background.cpp, compiled from its sources where they lie) to the oracle
// tests and the fixture generator. Test infrastructure only; built into oracle/_ref by
// `make ref`.
#include "src/sizing/background.cpp"

#include <span>

// Evaluates the closure from_background(mesh, sizes, scale) at each query.
extern "C" void ref_sizing_eval(const double* pts, long long npts, const int* tets, long long ntets,
                                const double* sizes, long long nsizes, double scale,
                                const double* queries, long long nq, double* out) {
    cmg::Mesh m;
    for (long long i = 0; i < npts; ++i)
        m.points.push_back(cmg::Point3{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]});
    for (long long t = 0; t < ntets; ++t)
        m.tetrahedra.push_back(
            cmg::Tetrahedron{tets[4 * t], tets[4 * t + 1], tets[4 * t + 2], tets[4 * t + 3]});
    auto f = cmg::sizing::from_background(
        m, std::span<const double>(sizes, static_cast<size_t>(nsizes)), scale);
    for (long long q = 0; q < nq; ++q)
        out[q] = f(cmg::Point3{queries[3 * q], queries[3 * q + 1], queries[3 * q + 2]});
}
