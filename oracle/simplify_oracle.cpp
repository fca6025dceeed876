// simplify_oracle.cpp — CPU restatement of the reference's grid vertex clustering
// (src/simplify/simplify.cpp), test infrastructure only.
//
// The reference (:48-112): bounding box of the points (:57-62), longest extent `ext`
// (:63-64; error when it is not positive, :65-67), inv = grid / ext (:68); each vertex
// goes to the cell ((p - lo) * inv truncated to int and clamped to [0, grid - 1] per
// axis, key (ix * grid + iy) * grid + iz, :21-32); cells become representatives in
// order of their first vertex (:71-88), a representative's point is the sum of its
// vertices' coordinates taken in vertex order from 0, divided by their count
// (:83-97); fan triangles of every facet (:35-44) are re-emitted over
// representatives in fan order, skipping those with two equal corners and those whose
// sorted corner triple was already emitted (:100-110).
//
// This restatement reaches the same result by sorting instead of ordered maps: the
// vertices sorted by (key, index) give each cell's members in vertex order and its
// first vertex; the non-degenerate triangles sorted by (sorted triple, position) give
// each triple's first occurrence. Deliberate differences: a non-finite coordinate and
// a facet index outside the points are errors here (the reference's behaviour is
// undefined for both). Keys wrap modulo 2^64 as the reference's 64-bit products do.
//
// Used only by tests/, the fixture generator and bench.py's CPU legs, as the checker;
// never by the product path.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

namespace {

void put_err(char* buf, size_t len, const char* msg) {
    if (buf && len) {
        std::strncpy(buf, msg, len - 1);
        buf[len - 1] = '\0';
    }
}

int cell_coord(double p, double lo, double inv, int grid) {
    const double f = (p - lo) * inv;
    int i = static_cast<int>(f);
    return i < 0 ? 0 : (i >= grid ? grid - 1 : i);
}

}  // namespace

extern "C" {

// Simplifies the triangle set (pts: npts x 3, tris: ntris x 3 fan triangles in facet
// order). out_pts must hold 3 * npts doubles, out_tris 3 * ntris ints. Returns the
// number of representative points (the first *nout_tris rows of out_tris are the kept
// triangles), or -1 with the message in err.
int64_t orc_simplify(const double* pts, int64_t npts, const int* tris, int64_t ntris, int grid,
                     double* out_pts, int* out_tris, int64_t* nout_tris, char* err, size_t errlen) {
    *nout_tris = 0;
    if (npts <= 0) {
        put_err(err, errlen, "simplify: PLC has no points");
        return -1;
    }
    if (grid < 1) {
        put_err(err, errlen, "simplify: grid must be >= 1");
        return -1;
    }
    for (int64_t i = 0; i < 3 * npts; ++i)
        if (!std::isfinite(pts[i])) {
            put_err(err, errlen, "simplify: non-finite point coordinate");
            return -1;
        }
    double lo[3], hi[3];
    for (int a = 0; a < 3; ++a) lo[a] = hi[a] = pts[a];
    for (int64_t i = 1; i < npts; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], pts[3 * i + a]);
            hi[a] = std::max(hi[a], pts[3 * i + a]);
        }
    double ext = 0.0;
    for (int a = 0; a < 3; ++a) ext = std::max(ext, hi[a] - lo[a]);
    if (!(ext > 0.0)) {
        put_err(err, errlen, "simplify: degenerate (zero-extent) surface");
        return -1;
    }
    for (int64_t k = 0; k < 3 * ntris; ++k)
        if (tris[k] < 0 || tris[k] >= npts) {
            put_err(err, errlen, "simplify: facet vertex index out of range");
            return -1;
        }
    const double inv = static_cast<double>(grid) / ext;
    const uint64_t g = static_cast<uint64_t>(grid);
    std::vector<uint64_t> key(static_cast<size_t>(npts));
    for (int64_t i = 0; i < npts; ++i) {
        const uint64_t ix = static_cast<uint64_t>(cell_coord(pts[3 * i], lo[0], inv, grid));
        const uint64_t iy = static_cast<uint64_t>(cell_coord(pts[3 * i + 1], lo[1], inv, grid));
        const uint64_t iz = static_cast<uint64_t>(cell_coord(pts[3 * i + 2], lo[2], inv, grid));
        key[i] = (ix * g + iy) * g + iz;
    }

    // cells: members in vertex order, numbered by their first member
    std::vector<int64_t> order(static_cast<size_t>(npts));
    std::iota(order.begin(), order.end(), int64_t(0));
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        return key[a] != key[b] ? key[a] < key[b] : a < b;
    });
    std::vector<int64_t> first_of(static_cast<size_t>(npts));  // per vertex: its cell's first member
    std::vector<std::pair<int64_t, int64_t>> groups;              // [begin, end) in `order`
    for (int64_t s = 0; s < npts;) {
        int64_t e = s + 1;
        while (e < npts && key[order[e]] == key[order[s]]) ++e;
        for (int64_t k = s; k < e; ++k) first_of[order[k]] = order[s];
        groups.emplace_back(s, e);
        s = e;
    }
    std::vector<int64_t> number(static_cast<size_t>(npts), -1);  // per first member
    int64_t nrep = 0;
    for (int64_t i = 0; i < npts; ++i)
        if (first_of[i] == i) number[i] = nrep++;
    std::vector<int> rep(static_cast<size_t>(npts));
    for (int64_t i = 0; i < npts; ++i) rep[i] = static_cast<int>(number[first_of[i]]);
    for (const auto& gr : groups) {
        const int64_t r = number[order[gr.first]];
        double s[3] = {0.0, 0.0, 0.0};
        for (int64_t k = gr.first; k < gr.second; ++k)
            for (int a = 0; a < 3; ++a) s[a] += pts[3 * order[k] + a];
        const double n = static_cast<double>(gr.second - gr.first);
        for (int a = 0; a < 3; ++a) out_pts[3 * r + a] = s[a] / n;
    }

    // triangles: first occurrence of each sorted representative triple
    std::vector<std::array<int, 3>> sk(static_cast<size_t>(ntris));
    std::vector<int64_t> live;
    for (int64_t t = 0; t < ntris; ++t) {
        const int a = rep[tris[3 * t]], b = rep[tris[3 * t + 1]], c = rep[tris[3 * t + 2]];
        if (a == b || b == c || a == c) continue;
        sk[t] = {a, b, c};
        std::sort(sk[t].begin(), sk[t].end());
        live.push_back(t);
    }
    std::vector<int64_t> by_key(live);
    std::sort(by_key.begin(), by_key.end(), [&](int64_t a, int64_t b) {
        return sk[a] != sk[b] ? sk[a] < sk[b] : a < b;
    });
    std::vector<char> keep(static_cast<size_t>(ntris), 0);
    for (size_t k = 0; k < by_key.size(); ++k)
        if (k == 0 || sk[by_key[k]] != sk[by_key[k - 1]]) keep[by_key[k]] = 1;
    int64_t m = 0;
    for (int64_t t = 0; t < ntris; ++t)
        if (keep[t]) {
            for (int c = 0; c < 3; ++c) out_tris[3 * m + c] = rep[tris[3 * t + c]];
            ++m;
        }
    *nout_tris = m;
    return nrep;
}

}  // extern "C"
