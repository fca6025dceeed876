// ref_stl.cpp — exposes the reference's own STL reader (src/io/stl.cpp, compiled from
// its sources where they lie) to the oracle tests and the fixture generator.
// Test infrastructure only; built into oracle/_ref by `make ref`.
#include "src/io/stl.cpp"

#include <string>
#include <vector>

namespace {
struct RefStl {
    std::vector<double> pts;
    std::vector<int> tris;
    std::string err;
};
}  // namespace

extern "C" {

void* ref_stl_read(const char* path) {
    RefStl* o = new RefStl;
    auto r = cmg::io::read_stl(path);
    if (!r) {
        o->err = r.error().message;
        return o;
    }
    for (const auto& p : r->points) o->pts.insert(o->pts.end(), {p.x, p.y, p.z});
    for (const auto& f : r->facets)
        for (int v : f.polygons[0].vertices) o->tris.push_back(v);
    return o;
}
const char* ref_stl_error(void* h) { return static_cast<RefStl*>(h)->err.c_str(); }
long long ref_stl_num_points(void* h) { return static_cast<long long>(static_cast<RefStl*>(h)->pts.size() / 3); }
long long ref_stl_num_triangles(void* h) { return static_cast<long long>(static_cast<RefStl*>(h)->tris.size() / 3); }
const double* ref_stl_points(void* h) { return static_cast<RefStl*>(h)->pts.data(); }
const int* ref_stl_triangles(void* h) { return static_cast<RefStl*>(h)->tris.data(); }
void ref_stl_free(void* h) { delete static_cast<RefStl*>(h); }

}  // extern "C"
