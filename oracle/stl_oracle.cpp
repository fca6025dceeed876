// stl_oracle.cpp — CPU restatement of the reference's STL reader (test infrastructure).
//
// Follows src/io/stl.cpp: binary when the image size is exactly 84 + 50 n (n the
// little-endian u32 at byte 80; :163-168), each record's three float32 vertices after
// its normal (:96-110), widened to double; otherwise ASCII (:112-129): lines split on
// '\n', '#' comments removed, blank lines skipped, tokens separated by whitespace or
// ',' (include/cmg/io/detail.hpp:22-55), records whose first token is "vertex" or
// "VERTEX" must have three more tokens that std::stod converts whole
// (detail.hpp:57-60). Coincident vertices are merged on their exact coordinate
// triple in order of first occurrence (:26-65). One deliberate difference: a NaN
// coordinate is rejected (the reference's ordered map has no defined behaviour for it).
//
// Used only by tests/, the fixture generator and bench.py's CPU legs, as the checker
// and the timed CPU baseline; never by the product path.
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

namespace {

struct Stl {
    std::vector<double> pts;  // 3 per point
    std::vector<int> tris;    // 3 per facet
    std::string err;
};

bool is_space(unsigned char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// std::stod's acceptance: strtod converts the whole token without ERANGE.
bool to_real(const std::string& s, double& out) {
    if (s.empty()) return false;
    errno = 0;
    char* end = nullptr;
    const double v = std::strtod(s.c_str(), &end);
    if (end == s.c_str() || errno == ERANGE) return false;
    if (static_cast<size_t>(end - s.c_str()) != s.size()) return false;
    out = v;
    return true;
}

bool weld(const std::vector<double>& v, Stl& o) {
    if (v.empty() || (v.size() / 3) % 3 != 0) {
        o.err = ".stl: vertex count is not a positive multiple of 3";
        return false;
    }
    for (double x : v)
        if (std::isnan(x)) {
            o.err = ".stl: NaN vertex coordinate";
            return false;
        }
    // exact coordinate triples; +0 and -0 compare equal as doubles, so the key is
    // canonicalised (x + 0.0) while the stored point keeps the first occurrence's bits
    std::map<std::tuple<double, double, double>, int> seen;
    const size_t nv = v.size() / 3;
    o.tris.resize(nv);
    for (size_t i = 0; i < nv; ++i) {
        const auto key = std::make_tuple(v[3 * i] + 0.0, v[3 * i + 1] + 0.0, v[3 * i + 2] + 0.0);
        auto it = seen.find(key);
        int idx;
        if (it != seen.end()) {
            idx = it->second;
        } else {
            idx = static_cast<int>(o.pts.size() / 3);
            o.pts.insert(o.pts.end(), {v[3 * i], v[3 * i + 1], v[3 * i + 2]});
            seen.emplace(key, idx);
        }
        o.tris[i] = idx;
    }
    return true;
}

bool parse_ascii(const char* b, size_t len, std::vector<double>& v, std::string& err) {
    size_t pos = 0;
    std::vector<std::string> tok;
    while (pos < len) {
        size_t e = pos;
        while (e < len && b[e] != '\n') ++e;
        std::string line(b + pos, e - pos);
        pos = e + 1;
        const size_t h = line.find('#');
        if (h != std::string::npos) line.erase(h);
        tok.clear();
        std::string cur;
        for (char c : line) {
            if (is_space(static_cast<unsigned char>(c)) || c == ',') {
                if (!cur.empty()) {
                    tok.push_back(cur);
                    cur.clear();
                }
            } else {
                cur.push_back(c);
            }
        }
        if (!cur.empty()) tok.push_back(cur);
        if (tok.empty()) continue;
        if (tok[0] == "vertex" || tok[0] == "VERTEX") {
            if (tok.size() < 4) {
                err = ".stl: short vertex record";
                return false;
            }
            double x, y, z;
            if (!to_real(tok[1], x) || !to_real(tok[2], y) || !to_real(tok[3], z)) {
                err = ".stl: non-numeric vertex coordinate";
                return false;
            }
            v.insert(v.end(), {x, y, z});
        }
    }
    return true;
}

}  // namespace

extern "C" {

// Reads an STL image; returns a handle (never NULL) whose error text is empty on success.
void* orc_stl_read(const char* bytes, size_t len) {
    Stl* o = new Stl;
    std::vector<double> v;
    bool binary = false;
    if (len >= 84) {
        uint32_t n;
        std::memcpy(&n, bytes + 80, 4);
        binary = len == 84u + 50ull * n;
        if (binary) {
            v.reserve(9ull * n);
            for (uint32_t t = 0; t < n; ++t) {
                const char* rec = bytes + 84 + 50ull * t + 12;
                for (int k = 0; k < 9; ++k) {
                    float f;
                    std::memcpy(&f, rec + 4 * k, 4);
                    v.push_back(static_cast<double>(f));
                }
            }
        }
    }
    if (!binary && !parse_ascii(bytes, len, v, o->err)) return o;
    weld(v, *o);
    return o;
}

const char* orc_stl_error(void* h) { return static_cast<Stl*>(h)->err.c_str(); }
int64_t orc_stl_num_points(void* h) { return static_cast<int64_t>(static_cast<Stl*>(h)->pts.size() / 3); }
int64_t orc_stl_num_triangles(void* h) { return static_cast<int64_t>(static_cast<Stl*>(h)->tris.size() / 3); }
const double* orc_stl_points(void* h) { return static_cast<Stl*>(h)->pts.data(); }
const int* orc_stl_triangles(void* h) { return static_cast<Stl*>(h)->tris.data(); }
void orc_stl_free(void* h) { delete static_cast<Stl*>(h); }

}  // extern "C"
