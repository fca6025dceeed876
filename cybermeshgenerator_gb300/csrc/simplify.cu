// simplify.cu — surface simplification by grid vertex clustering on the device.
//
// Semantics of the reference (src/simplify/simplify.cpp:48-112): the points'
// bounding box and its longest extent `ext` (an error when not positive); inv =
// grid / ext; a vertex p falls in the cell ((p - lo) * inv truncated toward zero,
// clamped to [0, grid - 1]) per axis, key (ix * grid + iy) * grid + iz in 64-bit
// wrapping arithmetic (:21-32); cells become representative points numbered in order
// of their first vertex, each the sum of its vertices' coordinates taken in vertex
// order from 0.0 divided by their count (:71-97); the fan triangles of the facets
// (:35-44) are re-emitted over representatives in fan order, without those having two
// equal corners and without repeats of an already emitted sorted corner triple
// (:100-110). A non-finite coordinate and a facet index outside the points are errors
// here (the reference's behaviour is undefined for both).
//
// Device plan, every step deterministic and every result bit-identical to the
// sequential definition:
//   points    bounding box by order-preserving integer atomics (min / max commute);
//             cell keys with the reference's rounded FP64 subtract and multiply;
//             first vertex of each cell from an open-addressing table whose slot
//             keeps the smallest vertex index with that key (atomicMin; keys compared
//             through the key array, written by the previous kernel); the exclusive
//             scan of "is first" flags numbers the representatives; a stable radix
//             sort of (representative, vertex) lists each cell's vertices in vertex
//             order, and one thread per representative adds them in that order.
//   triangles fan triangulation from the facet offsets (scan of per-facet counts);
//             representatives substituted; the first occurrence of each sorted triple
//             found by a second min-index table; the scan of kept flags places them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "cmg_util.h"
#include "engine_kernels.h"

namespace cmg::gpu {

namespace {

constexpr int kEmpty = -1;
constexpr int kThreads = 256;

enum : int { kFlagNonFinite = 0, kFlagDegenerate = 1, kFlagRange = 2, kFlagOverflow = 3, kNumFlags = 4 };

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

// Total order of doubles as unsigned integers (negative values reversed), so that
// integer min / max atomics give the coordinate min / max.
__device__ __forceinline__ unsigned long long ord_of(double x) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_ord(unsigned long long o) {
    return __longlong_as_double(static_cast<long long>((o >> 63) ? (o & 0x7fffffffffffffffull) : ~o));
}

// Inserts idx under hash h; the slot ends holding the smallest index whose key
// equals idx's (same(o) compares o's key with idx's). Returns the slot.
template <typename Same>
__device__ __forceinline__ int insert_min(int* tab, uint64_t mask, uint64_t h, int idx, Same same,
                                          int* flags) {
    for (uint64_t probe = 0; probe <= mask; ++probe) {
        int o = tab[h];
        if (o == kEmpty) {
            o = atomicCAS(&tab[h], kEmpty, idx);
            if (o == kEmpty) return static_cast<int>(h);
        }
        if (same(o)) {
            atomicMin(&tab[h], idx);
            return static_cast<int>(h);
        }
        h = (h + 1) & mask;
    }
    atomicExch(&flags[kFlagOverflow], 1);  // unreachable: tables hold twice the entries
    return -1;
}

// ---------------------------------------------------------------- points

// box[0..2] min, box[3..5] max (ord_of encoding).
__global__ void __launch_bounds__(kThreads) k_bbox(const double* __restrict__ p, int64_t n,
                                                   unsigned long long* __restrict__ box,
                                                   int* __restrict__ flags) {
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
    bool bad = false;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double x = p[3 * i + a];
            bad |= !isfinite(x);
            const unsigned long long o = ord_of(x);
            lo[a] = o < lo[a] ? o : lo[a];
            hi[a] = o > hi[a] ? o : hi[a];
        }
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const unsigned long long l = __shfl_xor_sync(0xffffffffu, lo[a], s);
            const unsigned long long h = __shfl_xor_sync(0xffffffffu, hi[a], s);
            lo[a] = l < lo[a] ? l : lo[a];
            hi[a] = h > hi[a] ? h : hi[a];
        }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicExch(&flags[kFlagNonFinite], 1);
    if ((threadIdx.x & 31) == 0)
        for (int a = 0; a < 3; ++a) {
            atomicMin(&box[a], lo[a]);
            atomicMax(&box[3 + a], hi[a]);
        }
}

// prm[0..2] = lo, prm[3] = inv (0 when the extent is not positive, which is flagged).
__global__ void k_params(const unsigned long long* __restrict__ box, int grid, double* __restrict__ prm,
                         int* __restrict__ flags) {
    double ext = 0.0;
    for (int a = 0; a < 3; ++a) {
        const double d = __dsub_rn(from_ord(box[3 + a]), from_ord(box[a]));
        ext = ext < d ? d : ext;
        prm[a] = from_ord(box[a]);
    }
    if (ext > 0.0) {
        prm[3] = __ddiv_rn(static_cast<double>(grid), ext);
    } else {
        prm[3] = 0.0;
        flags[kFlagDegenerate] = 1;
    }
}

__device__ __forceinline__ uint64_t cell_coord(double p, double lo, double inv, int grid) {
    // static_cast<int> truncates toward zero; the product stays below 2^31 for finite input
    int i = __double2int_rz(__dmul_rn(__dsub_rn(p, lo), inv));
    i = i < 0 ? 0 : (i >= grid ? grid - 1 : i);
    return static_cast<uint64_t>(i);
}

__global__ void __launch_bounds__(kThreads) k_cell_keys(const double* __restrict__ p, int64_t n,
                                                        const double* __restrict__ prm, int grid,
                                                        uint64_t* __restrict__ key) {
    const int64_t v = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const double inv = prm[3];
    const uint64_t g = static_cast<uint64_t>(grid);
    const uint64_t ix = cell_coord(p[3 * v], prm[0], inv, grid);
    const uint64_t iy = cell_coord(p[3 * v + 1], prm[1], inv, grid);
    const uint64_t iz = cell_coord(p[3 * v + 2], prm[2], inv, grid);
    key[v] = (ix * g + iy) * g + iz;
}

__global__ void __launch_bounds__(kThreads) k_cell_insert(const uint64_t* __restrict__ key, int64_t n,
                                                          int* __restrict__ tab, uint64_t mask,
                                                          int* __restrict__ slot, int* __restrict__ flags) {
    const int64_t v = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint64_t k = key[v];
    slot[v] = insert_min(tab, mask, mix64(k) & mask, static_cast<int>(v),
                         [&](int o) { return key[o] == k; }, flags);
}

__global__ void __launch_bounds__(kThreads) k_first_flags(int64_t n, const int* __restrict__ slot,
                                                          const int* __restrict__ tab,
                                                          int* __restrict__ flag) {
    const int64_t v = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int s = slot[v];
    flag[v] = s >= 0 && tab[s] == static_cast<int>(v) ? 1 : 0;
}

// rep[v]: the representative of vertex v; (sort_key, sort_val) = (rep, v) for the sort.
__global__ void __launch_bounds__(kThreads) k_rep_of(int64_t n, const int* __restrict__ slot,
                                                     const int* __restrict__ tab,
                                                     const int64_t* __restrict__ rank,
                                                     int* __restrict__ rep, uint32_t* __restrict__ sk,
                                                     uint32_t* __restrict__ sv) {
    const int64_t v = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int s = slot[v];
    const int r = s >= 0 ? static_cast<int>(rank[tab[s]]) : 0;
    rep[v] = r;
    sk[v] = static_cast<uint32_t>(r);
    sv[v] = static_cast<uint32_t>(v);
}

// off[r] = first sorted position of representative r; off[nrep] = n.
__global__ void __launch_bounds__(kThreads) k_rep_heads(int64_t n, const uint32_t* __restrict__ sk,
                                                        int* __restrict__ off) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t r = sk[i];
    if (i == 0 || sk[i - 1] != r) off[r] = static_cast<int>(i);
    if (i == n - 1) off[r + 1] = static_cast<int>(n);
}

// One thread per representative: its vertices' coordinates added in vertex order
// from 0.0 (three independent chains), then divided by their count.
__global__ void __launch_bounds__(kThreads) k_rep_sum(const int64_t* __restrict__ nrep_p,
                                                      const int* __restrict__ off,
                                                      const uint32_t* __restrict__ member,
                                                      const double* __restrict__ p,
                                                      double* __restrict__ out) {
    const int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= *nrep_p) return;
    const int b = off[r], e = off[r + 1];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    int k = b;
    for (; k + 4 <= e; k += 4) {
        double x[4], y[4], z[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t v = member[k + j];
            x[j] = p[3 * v];
            y[j] = p[3 * v + 1];
            z[j] = p[3 * v + 2];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            sx = __dadd_rn(sx, x[j]);
            sy = __dadd_rn(sy, y[j]);
            sz = __dadd_rn(sz, z[j]);
        }
    }
    for (; k < e; ++k) {
        const int64_t v = member[k];
        sx = __dadd_rn(sx, p[3 * v]);
        sy = __dadd_rn(sy, p[3 * v + 1]);
        sz = __dadd_rn(sz, p[3 * v + 2]);
    }
    const double c = static_cast<double>(e - b);
    out[3 * r] = __ddiv_rn(sx, c);
    out[3 * r + 1] = __ddiv_rn(sy, c);
    out[3 * r + 2] = __ddiv_rn(sz, c);
}

// ---------------------------------------------------------------- triangles

__global__ void __launch_bounds__(kThreads) k_fan_count(const size_t* __restrict__ foff, int64_t nf,
                                                        int64_t* __restrict__ cnt) {
    const int64_t f = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int64_t n = static_cast<int64_t>(foff[f + 1] - foff[f]);
    cnt[f] = n >= 3 ? n - 2 : 0;
}

// Fan triangles (v0, v[i-1], v[i]) of facet f at positions toff[f] + i - 2, over
// representatives: rt = corners in fan order, skey = sorted corners (x = -1 for a
// triangle with two equal corners or an index outside the points).
__global__ void __launch_bounds__(kThreads) k_fan_emit(const size_t* __restrict__ foff,
                                                       const int* __restrict__ fidx, int64_t nf,
                                                       const int64_t* __restrict__ toff,
                                                       const int* __restrict__ rep, int64_t npts,
                                                       int4* __restrict__ rt, int4* __restrict__ skey,
                                                       int* __restrict__ flags) {
    const int64_t f = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const size_t o = foff[f];
    const int64_t n = static_cast<int64_t>(foff[f + 1] - o);
    const int v0 = fidx[o];
    for (int64_t i = 2; i < n; ++i) {
        const int64_t t = toff[f] + i - 2;
        const int v1 = fidx[o + i - 1], v2 = fidx[o + i];
        if (v0 < 0 || v0 >= npts || v1 < 0 || v1 >= npts || v2 < 0 || v2 >= npts) {
            atomicExch(&flags[kFlagRange], 1);
            skey[t] = make_int4(-1, -1, -1, -1);
            continue;
        }
        const int a = rep[v0], b = rep[v1], c = rep[v2];
        rt[t] = make_int4(a, b, c, 0);
        if (a == b || b == c || a == c) {
            skey[t] = make_int4(-1, -1, -1, -1);
            continue;
        }
        const int lo = min(a, min(b, c)), hi = max(a, max(b, c));
        skey[t] = make_int4(lo, a + b + c - lo - hi, hi, 0);
    }
}

__device__ __forceinline__ uint64_t triple_hash(int4 k) {
    return mix64(mix64((static_cast<uint64_t>(static_cast<uint32_t>(k.x)) << 32) |
                       static_cast<uint32_t>(k.y)) ^
                 static_cast<uint32_t>(k.z));
}

__global__ void __launch_bounds__(kThreads) k_tri_insert(const int4* __restrict__ skey, int64_t m,
                                                         int* __restrict__ tab, uint64_t mask,
                                                         int* __restrict__ slot,
                                                         int* __restrict__ flags) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= m) return;
    const int4 k = skey[t];
    if (k.x < 0) {
        slot[t] = -1;
        return;
    }
    slot[t] = insert_min(tab, mask, triple_hash(k) & mask, static_cast<int>(t),
                         [&](int o) {
                             const int4 q = skey[o];
                             return q.x == k.x && q.y == k.y && q.z == k.z;
                         },
                         flags);
}

__global__ void __launch_bounds__(kThreads) k_tri_keep(int64_t m, const int* __restrict__ slot,
                                                       const int* __restrict__ tab,
                                                       int* __restrict__ keep) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= m) return;
    const int s = slot[t];
    keep[t] = s >= 0 && tab[s] == static_cast<int>(t) ? 1 : 0;
}

__global__ void __launch_bounds__(kThreads) k_tri_out(int64_t m, const int* __restrict__ keep,
                                                      const int64_t* __restrict__ pos,
                                                      const int4* __restrict__ rt,
                                                      int* __restrict__ out) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= m || !keep[t]) return;
    const int4 r = rt[t];
    const int64_t q = pos[t];
    out[3 * q] = r.x;
    out[3 * q + 1] = r.y;
    out[3 * q + 2] = r.z;
}

unsigned blocks(int64_t n) { return static_cast<unsigned>((n + kThreads - 1) / kThreads); }

uint64_t table_size(int64_t n) {
    uint64_t s = 2;
    while (s < 2 * static_cast<uint64_t>(n)) s <<= 1;
    return s;
}

struct SimplifyWork {
    Arena pa, ta;  // point phase (and the facet scan); triangle phase
    std::mutex mu;
    int64_t* pinned = nullptr;  // [0] triangles, [1] representatives, [2] kept, [3..6] flags
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    float ms[3] = {0.f, 0.f, 0.f};  // last call: upload, clustering, download
};
SimplifyWork& simplify_work() {
    static SimplifyWork w[64];
    int dev = 0;
    CMG_CUDA(cudaGetDevice(&dev));
    return w[dev & 63];
}

}  // namespace

void simplify(const double* pts, int64_t npts, const int* fidx, int64_t nidx, const size_t* foff,
              int64_t nfacets, int grid, HostVec<double>& out_pts, HostVec<int>& out_tris,
              cudaStream_t st) {
    if (npts <= 0) throw std::invalid_argument("simplify: PLC has no points");
    if (grid < 1) throw std::invalid_argument("simplify: grid must be >= 1");
    if (npts >= (int64_t(1) << 30)) throw std::invalid_argument("simplify: too many points");
    if (nidx >= (int64_t(1) << 30)) throw std::invalid_argument("simplify: too many facet vertices");

    SimplifyWork& W = simplify_work();
    std::lock_guard<std::mutex> lk(W.mu);
    if (!W.pinned) CMG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&W.pinned), 8 * sizeof(int64_t),
                                          cudaHostAllocDefault));
    if (!W.ev[0])
        for (cudaEvent_t& e : W.ev) CMG_CUDA(cudaEventCreate(&e));
    const uint64_t S1 = table_size(npts);
    int bits = 1;
    while ((int64_t(1) << bits) < npts) ++bits;

    struct P {
        double *p, *prm, *outp;
        int *fidx, *tab, *slot, *flag, *rep, *off, *flags;
        size_t* foff;
        uint64_t* key;
        unsigned long long* box;
        int64_t *rank, *cnt, *toff, *stmp;
        uint32_t *sk, *sv;
        void* sort_tmp;
    } a{};
    const int64_t nf = nfacets;
    auto plan_points = [&]() {
        Arena& A = W.pa;
        A.reset();
        a.p = A.take<double>(3 * npts);
        a.fidx = A.take<int>(nidx > 0 ? nidx : 1);
        a.foff = A.take<size_t>(nf + 1);
        a.prm = A.take<double>(4);
        a.box = A.take<unsigned long long>(6);
        a.flags = A.take<int>(kNumFlags);
        a.key = A.take<uint64_t>(npts);
        a.tab = A.take<int>(S1);
        a.slot = A.take<int>(npts);
        a.flag = A.take<int>(npts);
        a.rank = A.take<int64_t>(npts + 1);
        a.rep = A.take<int>(npts);
        a.sk = A.take<uint32_t>(npts);
        a.sv = A.take<uint32_t>(npts);
        a.off = A.take<int>(npts + 1);
        a.outp = A.take<double>(3 * npts);
        a.cnt = A.take<int64_t>(nf > 0 ? nf : 1);
        a.toff = A.take<int64_t>(nf + 1);
        a.stmp = A.take<int64_t>(scan_tmp_elems(npts > nf ? npts : nf));
        a.sort_tmp = A.take<char>(radix_sort_tmp_bytes(npts));
    };
    W.pa.clear_need();
    plan_points();
    if (W.pa.overflowed()) {
        W.pa.reserve(W.pa.need());
        plan_points();
    }

    CMG_CUDA(cudaEventRecord(W.ev[0], st));
    CMG_CUDA(cudaMemcpyAsync(a.p, pts, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice, st));
    if (nidx > 0) CMG_CUDA(cudaMemcpyAsync(a.fidx, fidx, sizeof(int) * nidx, cudaMemcpyHostToDevice, st));
    CMG_CUDA(cudaMemcpyAsync(a.foff, foff, sizeof(size_t) * (nf + 1), cudaMemcpyHostToDevice, st));
    CMG_CUDA(cudaEventRecord(W.ev[1], st));

    // facet scan first, so that the triangle count reaches the host while the
    // point phase runs
    W.pinned[0] = 0;
    if (nf > 0) {
        k_fan_count<<<blocks(nf), kThreads, 0, st>>>(a.foff, nf, a.cnt);
        CMG_LAUNCH();
        exclusive_scan(a.cnt, a.toff, nf, a.stmp, st);
        CMG_CUDA(cudaMemcpyAsync(W.pinned, a.toff + nf, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    }
    CMG_CUDA(cudaEventRecord(W.ev[4], st));

    CMG_CUDA(cudaMemsetAsync(a.box, 0xff, 3 * sizeof(unsigned long long), st));  // minima
    CMG_CUDA(cudaMemsetAsync(a.box + 3, 0, 3 * sizeof(unsigned long long), st));  // maxima
    CMG_CUDA(cudaMemsetAsync(a.flags, 0, sizeof(int) * kNumFlags, st));
    CMG_CUDA(cudaMemsetAsync(a.tab, 0xff, sizeof(int) * S1, st));  // kEmpty
    const unsigned bb = std::min<unsigned>(blocks(npts), 152u * 8u);
    k_bbox<<<bb, kThreads, 0, st>>>(a.p, npts, a.box, a.flags);
    CMG_LAUNCH();
    k_params<<<1, 1, 0, st>>>(a.box, grid, a.prm, a.flags);
    CMG_LAUNCH();
    k_cell_keys<<<blocks(npts), kThreads, 0, st>>>(a.p, npts, a.prm, grid, a.key);
    CMG_LAUNCH();
    k_cell_insert<<<blocks(npts), kThreads, 0, st>>>(a.key, npts, a.tab, S1 - 1, a.slot, a.flags);
    CMG_LAUNCH();
    k_first_flags<<<blocks(npts), kThreads, 0, st>>>(npts, a.slot, a.tab, a.flag);
    CMG_LAUNCH();
    exclusive_scan(a.flag, a.rank, npts, a.stmp, st);
    k_rep_of<<<blocks(npts), kThreads, 0, st>>>(npts, a.slot, a.tab, a.rank, a.rep, a.sk, a.sv);
    CMG_LAUNCH();
    radix_sort_pairs(a.sk, a.sv, npts, bits, a.sort_tmp, st);
    k_rep_heads<<<blocks(npts), kThreads, 0, st>>>(npts, a.sk, a.off);
    CMG_LAUNCH();
    k_rep_sum<<<blocks(npts), kThreads, 0, st>>>(a.rank + npts, a.off, a.sv, a.p, a.outp);
    CMG_LAUNCH();

    CMG_CUDA(cudaEventSynchronize(W.ev[4]));
    const int64_t m = W.pinned[0];
    if (m >= (int64_t(1) << 30)) throw std::invalid_argument("simplify: too many triangles");
    int* outt = nullptr;
    int64_t* tpos = nullptr;
    if (m > 0) {
        const uint64_t S2 = table_size(m);
        struct T {
            int4 *rt, *skey;
            int *tab, *slot, *keep, *out;
            int64_t *pos, *stmp;
        } b{};
        auto plan_tris = [&]() {
            Arena& A = W.ta;
            A.reset();
            b.rt = A.take<int4>(m);
            b.skey = A.take<int4>(m);
            b.tab = A.take<int>(S2);
            b.slot = A.take<int>(m);
            b.keep = A.take<int>(m);
            b.pos = A.take<int64_t>(m + 1);
            b.stmp = A.take<int64_t>(scan_tmp_elems(m));
            b.out = A.take<int>(3 * m);
        };
        W.ta.clear_need();
        plan_tris();
        if (W.ta.overflowed()) {
            W.ta.reserve(W.ta.need());
            plan_tris();
        }
        CMG_CUDA(cudaMemsetAsync(b.tab, 0xff, sizeof(int) * S2, st));
        k_fan_emit<<<blocks(nf), kThreads, 0, st>>>(a.foff, a.fidx, nf, a.toff, a.rep, npts, b.rt,
                                                    b.skey, a.flags);
        CMG_LAUNCH();
        k_tri_insert<<<blocks(m), kThreads, 0, st>>>(b.skey, m, b.tab, S2 - 1, b.slot, a.flags);
        CMG_LAUNCH();
        k_tri_keep<<<blocks(m), kThreads, 0, st>>>(m, b.slot, b.tab, b.keep);
        CMG_LAUNCH();
        exclusive_scan(b.keep, b.pos, m, b.stmp, st);
        k_tri_out<<<blocks(m), kThreads, 0, st>>>(m, b.keep, b.pos, b.rt, b.out);
        CMG_LAUNCH();
        outt = b.out;
        tpos = b.pos + m;
    }
    CMG_CUDA(cudaEventRecord(W.ev[2], st));
    CMG_CUDA(cudaMemcpyAsync(W.pinned + 1, a.rank + npts, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    W.pinned[2] = 0;
    if (tpos) CMG_CUDA(cudaMemcpyAsync(W.pinned + 2, tpos, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    int* hflags = reinterpret_cast<int*>(W.pinned + 3);
    CMG_CUDA(cudaMemcpyAsync(hflags, a.flags, sizeof(int) * kNumFlags, cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaStreamSynchronize(st));
    if (hflags[kFlagNonFinite]) throw std::invalid_argument("simplify: non-finite point coordinate");
    if (hflags[kFlagDegenerate])
        throw std::invalid_argument("simplify: degenerate (zero-extent) surface");
    if (hflags[kFlagRange]) throw std::invalid_argument("simplify: facet vertex index out of range");
    if (hflags[kFlagOverflow]) throw std::runtime_error("simplify: hash table overflow");
    const int64_t nrep = W.pinned[1], mout = W.pinned[2];
    out_pts.resize(static_cast<size_t>(3 * nrep));
    out_tris.resize(static_cast<size_t>(3 * mout));
    CMG_CUDA(cudaMemcpyAsync(out_pts.data(), a.outp, sizeof(double) * 3 * nrep, cudaMemcpyDeviceToHost, st));
    if (mout > 0)
        CMG_CUDA(cudaMemcpyAsync(out_tris.data(), outt, sizeof(int) * 3 * mout, cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaEventRecord(W.ev[3], st));
    CMG_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < 3; ++k) CMG_CUDA(cudaEventElapsedTime(&W.ms[k], W.ev[k], W.ev[k + 1]));
}

void simplify_last_timing(float* upload_ms, float* cluster_ms, float* download_ms) {
    SimplifyWork& W = simplify_work();
    std::lock_guard<std::mutex> lk(W.mu);
    *upload_ms = W.ms[0];
    *cluster_ms = W.ms[1];
    *download_ms = W.ms[2];
}

}  // namespace cmg::gpu
