// sdf_sub.cu — distance per cell, evaluated in 4^3 sub-bricks of the 16^3 candidate bricks.
//
// The brick candidate lists (k_brick_walk at brick edge 16) hold every triangle
// that can be nearest to some cell of the brick. One 64-thread CTA per 4^3
// sub-brick (a persistent kernel over an LPT-ordered queue of sub-bricks):
//   1. probe: an upper bound U on the distance from the sub-brick centre c to the
//      surface (FP32 point-triangle distance with its error bound, over the brick
//      list, each thread skipping triangles whose bounding sphere is beyond its
//      own bound so far);
//   2. filter: the brick list is compacted in shared memory to the triangles whose
//      bounding sphere can reach U + 2 r (r the sub-brick radius) — in rounds of at
//      most kCap entries;
//   3. cells, one per thread: a bounding-sphere test per listed triangle, and the
//      distance only when some lane of the warp needs it; FP64 Ericson in the
//      reference order (plain) or the FP32 record distance (mixed);
//   4. mixed only: cells within `band` cells of the surface are re-evaluated in FP64
//      over the triangles whose FP32 distance is within twice the stated bound of
//      the FP32 best, which gives the FP64 minimum exactly there.
// The exact FP64 path (kPrecExact) is the mixed kernel with bounds widened to every
// such near-tie, the near-ties kept per cell as the FP32 pass meets them, and the FP64
// distance over them for every cell (step 4 only for cells with too many near-ties).
// Centroids are stored as FP32 hi + lo pairs relative to the grid corner, so the
// centroid-to-centre differences are formed in FP32 without losing the low bits
// (the sub-brick recentring).
#include <cuda_runtime.h>

#include <cfloat>
#include <climits>

#include "cmg_device.cuh"
#include "cmg_sdf.cuh"
#include "cmg_seg.cuh"
#include "cmg_types.h"
#include "cmg_util.h"
#include "engine_kernels.h"

namespace cmg::gpu {

namespace {

using namespace sdf;

constexpr int kSub = 4;          // sub-brick edge (cells)
constexpr int kSubThreads = 64;  // one cell per thread
// filtered candidates per round in shared memory (STAGE: their records as well; the
// exact path, whose near-tie slots take 3 KB, 256). The mixed path's 296 keeps its
// shared memory (13.3 KB, plus the 1 KB the SM reserves per CTA) within 1/16 of the
// SM's 228 KB, so that 16 CTAs are resident; at least one filter step (kBatch x 64).
template <int PREC, bool STAGE>
struct Cap {
    static constexpr int value = STAGE || PREC == kPrecExact ? 256 : 296;
};
// mixed path: filtered entries per need-mask chunk (one bit per entry); the records a
// warp needs in a chunk are staged in its own shared-memory slots
constexpr int kChunk = 32;
// a chunk whose warp pre-test passes at least this many entries tests all of them
// unrolled, else only those that passed
constexpr int kDenseChunk = 20;
// kPrecExact, the exact FP64 path: the mixed kernel's FP32 pass with its bounds widened
// to admit every triangle whose FP32 distance is within twice the stated error of the
// cell's FP32 minimum, those near-ties kept per cell (kNear slots), and the FP64 distance
// in the reference's order over them, which is the FP64 minimum over all triangles (a
// cell with more near-ties takes the band pass).
constexpr int kNear = 6;
constexpr int kBatch = 4;  // candidates per thread per probe/filter step (loads in flight)
constexpr int kProbe = 1024;  // default head of the brick list the mixed probe scans

// Reach of a cell's sphere test against one filtered triangle (mixed path): the cell
// may need the triangle when |cell - centroid| <= lim, lim = (b + w)(1 + 16u) + 16u r
// (b the cell's bound, w the triangle's radius, r the sub-brick radius; the margins
// cover the FP32 rounding of the centroids, cell offsets and bound). Evaluated as
//   reach_term(w, r) = RU(w (1 + 20u) + RU(17u r))     once per triangle, and
//   reach(b, term)   = RU(b (1 + 20u) + term)           per cell,
// which is at least (b + w)(1 + 20u) + 17u r. The same expression rounded to nearest
// step by step is at most (b + w)(1 + 16u)(1 + u)^3 + 16u r (1 + u)^2, which is smaller,
// so this test admits every triangle the step-by-step form admits.
__device__ __forceinline__ float reach_term(float w, float r) {
    return __fmaf_ru(w, 1.f + 20.f * kU32, __fmul_ru(17.f * kU32, r));
}
__device__ __forceinline__ float reach(float b, float term) {
    return __fmaf_ru(b, 1.f + 20.f * kU32, term);
}

// The mixed path's sphere test in expanded form: 4 FMAs and a compare per entry. For a
// cell p (|p| <= r (1 + 2u), r the sub-brick radius) and an entry c with the reach L = reach(b,
// term) above, let
//   T = RU(term (1 + 51u) + RU(0.002 r + 1e-18))   per entry (exp_term),
//   G = RN(|c|^2 - T^2)                             per entry (exp_g),
//   B = RU(b (1 + 71u)), K = RN(B^2 - |p|^2)        per cell and chunk,
// so that B + T >= L (1 + 50u) + 0.002 r. The test
//   fma(-2p, c) + (-2B) T + G <= K,               i.e. |p - c|^2 <= (B + T)^2 expanded,
// is passed by every entry with |p - c| <= L: its rounding error (four FMA roundings,
// G's and K's) is at most 20.1u (R + r)^2 <= 40.2u (R^2 + r^2), R = B + T, while
// R^2 - L^2 >= (R - L) R >= (50u R^2 + 0.002 r R) / (1 + 50u), which exceeds it because
// R >= 0.002 r and 0.002^2 > 40.2u (the 1e-18 keeps R^2 above FP32's underflow error).
// The entries store c' = -2c (exact), so the dot product is fma(p, c') and the offsets
// p - c and w - c are fma(0.5, c', p), bit for bit the subtractions. Conversely an
// entry that passes has |p - c| <= (R + 0.00155 r)(1 + 21u) (exp_pass_reach).
__device__ __forceinline__ float exp_term(float term, float sr) {
    return __fmaf_ru(term, 1.f + 51.f * kU32, sr);
}
__device__ __forceinline__ float exp_sr(float r) { return __fmaf_ru(0.002f, r, 1e-18f); }
__device__ __forceinline__ float exp_g(float cx, float cy, float cz, float t) {
    return fmaf(-t, t, fmaf(cx, cx, fmaf(cy, cy, cz * cz)));
}
__device__ __forceinline__ float exp_b(float b) { return __fmul_ru(b, 1.f + 71.f * kU32); }
// Largest distance from the centroid of a cell whose expanded test passes, for the
// cell's B (at most bmax's) and the entry's T; sw = RU(0.0016 r).
__device__ __forceinline__ float exp_pass_reach(float bb, float t, float sw) {
    return __fmaf_ru(__fadd_ru(bb, t), 1.f + 21.f * kU32, sw);
}

// A cell's bound in the mixed path, from its smallest FP32 squared distance so far, d2:
// sqrt(d2) rounded (1 + 8u) plus the stated FP32 error of a distance of that size,
// 48u (d + 2 e + 2 r) with d <= sqrt(d2) + the error itself (kap = 98u (e + r)). A
// triangle whose FP32 distance can still be at most the current minimum lies within
// this bound, so its sphere test passes whatever order the candidates come in: the
// cell ends with the exact (FP32 distance, triangle id) minimum over all triangles,
// independent of the order of the filtered list (which the warps' scheduling sets).
__device__ __forceinline__ float cell_bound(float d2, float kap) {
    return __fmaf_ru(sqrtf(d2), 1.f + 58.f * kU32, kap);
}

// The exact path's bound: a near-tie's FP32 distance is within two stated errors of the
// cell's FP32 minimum m = sqrt(d2) and its true distance d one more, so d <= m + 3 E(d),
// E(d) = 48u (d + 2e + 2r), which gives 3 E(d) <= 144.1u m + 288.2u (e + r); with the
// square root's rounding, sqrt(d2)(1 + 160u) + kapx, kapx = RU(300u (e + r)), covers it.
__device__ __forceinline__ float cell_bound_x(float d2, float kapx) {
    return __fmaf_ru(sqrtf(d2), 1.f + 160.f * kU32, kapx);
}

// The near-tie threshold of a cell whose FP32 minimum is sqrt(d2), squared and rounded
// up: at least (m + 2 eb)^2, eb = 48u (m + 2e + 2r) the band pass's stated bound, so the
// kept triangles include every one the band pass would refine (kap = 98u (e + r)).
__device__ __forceinline__ float near_thr2(float d2, float kap) {
    const float thr = __fmaf_ru(sqrtf(d2), 1.f + 100.f * kU32, __fmul_ru(2.f, kap));
    return __fmul_ru(thr, thr);
}

// Largest computed plane distance |n . (cell - a)| of a triangle that can still reach
// the cell's FP32 minimum, for a cell bound b (cell_bound): such a triangle is within b
// of the cell, so |cell - a| <= b + 2e (a a vertex, e the mesh's largest
// centroid-to-vertex distance), and the FP32 plane distance errs by at most
// nerr |cell - a| (nerr bounds the FP32 unit normal's error, TriRec::nerr) plus the
// rounding of the recentred offsets and the dot product, all within
// (nerr + 64u)(b + 4e + 4r) (ebr4 = 4(e + r), rounded up).
__device__ __forceinline__ float plane_reach(float b, float nerr, float ebr4) {
    return __fmaf_ru(__fadd_ru(b, ebr4), __fadd_ru(nerr, 64.f * kU32), b);
}

// Reach of the warp pre-test: the warp's cells lie within wr of its sphere's centre
// (wr an upper bound, rounded up), and a cell's test passes only when the cell is
// within lim (1 + 4u) of the centroid (the test's own rounding), lim = reach(b, term) at
// most lim_max = reach(bmax, term) for the warp's largest bound bmax (reach grows with
// b); in the expanded form only within lim_max = exp_pass_reach(exp_b(bmax), T, sw).
// So the centre is within (lim_max + wr)(1 + 4u) of the centroid, and the squared
// distance computed from the centre (relative rounding within 7u) stays below the
// square of RU(RU(lim_max + wr)(1 + 16u)) rounded to nearest.
__device__ __forceinline__ float warp_reach(float lim_max, float wr) {
    return __fmul_ru(__fadd_ru(lim_max, wr), 1.f + 16.f * kU32);
}

// 16-byte asynchronous global -> shared copy (cp.async, L2 only) and its wait.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_all;\n" ::: "memory");
}

struct SubGeo {
    int x0, y0, z0, x1, y1, z1;
    bool empty;
};

__device__ __forceinline__ SubGeo sub_geo(const MeshSeg& s, int64_t lb, int sub) {
    SubGeo q;
    const int bx = static_cast<int>(lb % s.bnx);
    const int by = static_cast<int>((lb / s.bnx) % s.bny);
    const int bz = static_cast<int>(lb / (static_cast<int64_t>(s.bnx) * s.bny));
    const int per = s.brick / kSub;
    const int sx = sub % per, sy = (sub / per) % per, sz = sub / (per * per);
    q.x0 = bx * s.brick + sx * kSub;
    q.y0 = by * s.brick + sy * kSub;
    q.z0 = (bz + s.bzo) * s.brick + sz * kSub;  // bz counts from the slab's first brick
    q.x1 = min(q.x0 + kSub, s.g.nx);
    q.y1 = min(q.y0 + kSub, s.g.ny);
    q.z1 = min(q.z0 + kSub, s.g.nz);
    // the sub-brick keeps the whole grid's geometry; only its cells inside the slab
    // [z0, z1) are evaluated (none: nothing to do)
    q.empty = q.x0 >= s.g.nx || q.y0 >= s.g.ny || q.z0 >= s.g.nz || q.z1 <= s.g.z0 ||
              q.z0 >= s.g.z1;
    return q;
}

// PREC: kPrecMixed, kPrecExact or kPrecFP64. STAGE (mixed only): copy the records of the
// filtered candidates into shared memory (cp.async) instead of reading them
// from L1/L2 at evaluation time. MINB: resident CTAs per SM the registers are
// budgeted for (12: 80 registers; 16: 64). grab: consecutive sub-bricks taken from
// the queue at once (a divisor of 64: they share one brick list). probe_n: entries
// of the brick list head the mixed probe scans.
template <int PREC, bool STAGE, int MINB>
__global__ void __launch_bounds__(kSubThreads, MINB)
k_sdf_sub(const MeshSeg* __restrict__ segs, int nseg, const uint32_t* __restrict__ work,
          int64_t nwork, int grab_n, int probe_n, unsigned long long* __restrict__ queue,
          const double* __restrict__ soup,
          const float4* __restrict__ tinfo, const float4* __restrict__ tinfo_lo,
          const TriRec* __restrict__ trec, const float4* __restrict__ tnorm,
          const int64_t* __restrict__ cand_off,
          const int* __restrict__ cand, const float* __restrict__ brick_emax, float band_cells,
          Out o, Stats* __restrict__ st) {
    constexpr bool MIX = PREC != kPrecFP64;     // the FP32 pass (mixed or exact)
    constexpr bool EXACT = PREC == kPrecExact;  // ... refined to the FP64 minimum everywhere
    constexpr bool EXPAND = PREC == kPrecMixed && !STAGE;  // expanded sphere tests (exp_*)
    constexpr int kCap = Cap<PREC, STAGE>::value;
    static_assert(kCap >= kBatch * kSubThreads, "a round must hold one filter step");
    // exact path: per cell, its near-ties (triangle, FP32 squared distance), slot-major
    __shared__ int2 s_near[EXACT ? kNear : 1][kSubThreads];
    __shared__ float4 s_c[kCap];  // centroid relative to the sub-brick centre, radius
    __shared__ float s_g[EXPAND ? kCap : 1];  // EXPAND: exp_g of the entry
    // FP64 path: unit normal and plane offset n . centroid, and a bound on the error of
    // the plane distances computed from them
    __shared__ float4 s_nrm[PREC == kPrecFP64 ? kCap : 1];
    __shared__ float s_pe[PREC == kPrecFP64 ? kCap : 1];
    __shared__ int s_t[kCap];
    __shared__ TriRec s_rec[STAGE ? kCap : 1];
    __shared__ TriRec s_wrec[MIX && !STAGE ? (kSubThreads / 32) * kChunk : 1];
    __shared__ float4 s_wsph[MIX && !STAGE ? kSubThreads / 32 : 1];  // per warp
    __shared__ int s_n;
    __shared__ long long s_item;
    __shared__ unsigned long long s_red[kSubThreads / 32];
    __shared__ int s_band;
    __shared__ unsigned s_rmax;  // largest band reach of the CTA (FP32 bits)
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned long long evals = 0, evals64 = 0, bandc = 0;

    for (;;) {
        if (tid == 0) s_item = static_cast<long long>(atomicAdd(queue, 1ull));
        __syncthreads();
        const int64_t grab = s_item;
        __syncthreads();
        if (grab * grab_n >= nwork) break;
      for (int gi = 0; gi < grab_n; ++gi) {
        const int64_t item = grab * grab_n + gi;
        if (item >= nwork) break;
        if (tid == 0) s_band = 0;
        const uint32_t w = work[item];
        const int64_t gb = static_cast<int64_t>(w >> 6);
        const int sub = static_cast<int>(w & 63u);
        const MeshSeg& s = segs[find_seg<&MeshSeg::brick_begin>(segs, nseg, gb)];
        const GridDesc g = s.g;
        const SubGeo q = sub_geo(s, gb - s.brick_begin, sub);
        if (q.empty) continue;
        // sub-brick centre relative to the grid corner, as an FP32 hi + lo pair
        const double ckx = 0.5 * (q.x0 + q.x1) * g.h, cky = 0.5 * (q.y0 + q.y1) * g.h,
                     ckz = 0.5 * (q.z0 + q.z1) * g.h;
        float chx, clx, chy, cly, chz, clz;
        split2(ckx, chx, clx);
        split2(cky, chy, cly);
        split2(ckz, chz, clz);
        const double hx = 0.5 * (q.x1 - q.x0 - 1) * g.h, hy = 0.5 * (q.y1 - q.y0 - 1) * g.h,
                     hz = 0.5 * (q.z1 - q.z0 - 1) * g.h;
        const float r4 = __double2float_ru(sqrt(hx * hx + hy * hy + hz * hz) * (1.0 + 1e-9));
        // this thread's cell
        const int x = q.x0 + (tid & 3), y = q.y0 + ((tid >> 2) & 3), z = q.z0 + (tid >> 4);
        const bool valid = x < q.x1 && y < q.y1 && z < q.z1 && z >= g.z0 && z < g.z1;
        const float px = static_cast<float>((x + 0.5) * g.h - ckx);
        const float py = static_cast<float>((y + 0.5) * g.h - cky);
        const float pz = static_cast<float>((z + 0.5) * g.h - ckz);
        // EXPAND: |p|^2, the entries' radius margin (exp_sr) and the warp test's (exp_pass_reach)
        const float p2 = EXPAND ? fmaf(px, px, fmaf(py, py, pz * pz)) : 0.f;
        const float sr = EXPAND ? exp_sr(r4) : 0.f, sw = EXPAND ? __fmul_ru(0.0016f, r4) : 0.f;
        const int64_t c0 = cand_off[gb], c1 = cand_off[gb + 1];
        if (MIX && !STAGE) {
            // the warp's sphere for the chunk pre-test: centre at the middle of the box of
            // its valid cells, radius an upper bound on their distances from it (none
            // valid: radius 0, and no cell tests anything)
            float lox = valid ? px : FLT_MAX, loy = valid ? py : FLT_MAX, loz = valid ? pz : FLT_MAX;
            float hix = valid ? px : -FLT_MAX, hiy = valid ? py : -FLT_MAX, hiz = valid ? pz : -FLT_MAX;
#pragma unroll
            for (int sh = 16; sh > 0; sh >>= 1) {
                lox = fminf(lox, __shfl_xor_sync(0xffffffffu, lox, sh));
                loy = fminf(loy, __shfl_xor_sync(0xffffffffu, loy, sh));
                loz = fminf(loz, __shfl_xor_sync(0xffffffffu, loz, sh));
                hix = fmaxf(hix, __shfl_xor_sync(0xffffffffu, hix, sh));
                hiy = fmaxf(hiy, __shfl_xor_sync(0xffffffffu, hiy, sh));
                hiz = fmaxf(hiz, __shfl_xor_sync(0xffffffffu, hiz, sh));
            }
            const float wcx = 0.5f * (lox + hix), wcy = 0.5f * (loy + hiy), wcz = 0.5f * (loz + hiz);
            const float ox = px - wcx, oy = py - wcy, oz = pz - wcz;
            const float dw = valid ? sqrtf(ox * ox + oy * oy + oz * oz) : 0.f;
            const float wr =
                __fmul_ru(__uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(dw))), 1.f + 16.f * kU32);
            if (lane == 0) s_wsph[warp] = make_float4(wcx, wcy, wcz, wr);
        }

        // ---- 1. probe: upper bound on the distance from the centre to the surface,
        //         and the triangle that gives it (the seed of every cell below)
        float tb = FLT_MAX;
        int tseed = INT_MAX;
        // any bound is valid; the brick list runs from the brick centre outwards (large
        // triangles, then bins ring by ring), so its head holds the centre's nearest. The
        // mixed path scans only the head (a looser U lengthens the filtered lists a
        // little, which the cheap FP32 distances absorb); the FP64 path scans it all
        const int64_t cp = MIX && c1 - c0 > probe_n ? c0 + probe_n : c1;
        for (int64_t k0 = c0 + tid; k0 < cp; k0 += kBatch * kSubThreads) {
            // loads of kBatch candidates in flight before any of them is used
            int tt[kBatch];
            float4 hh[kBatch], ll[kBatch];
#pragma unroll
            for (int i = 0; i < kBatch; ++i) {
                const int64_t k = k0 + i * kSubThreads;
                tt[i] = k < cp ? cand[k] : -1;
            }
#pragma unroll
            for (int i = 0; i < kBatch; ++i)
                if (tt[i] >= 0) { hh[i] = tinfo[tt[i]]; ll[i] = tinfo_lo[tt[i]]; }
#pragma unroll
            for (int i = 0; i < kBatch; ++i) {
                if (tt[i] < 0) continue;
                const int t = tt[i];
                const float4 hi = hh[i], lo = ll[i];
                const float rx = (hi.x - chx) + (lo.x - clx);
                const float ry = (hi.y - chy) + (lo.y - cly);
                const float rz = (hi.z - chz) + (lo.z - clz);
                const float dc = sqrtf(rx * rx + ry * ry + rz * rz);
                const float sb = (dc + hi.w) * (1.f + 8.f * kU32);  // bounding-sphere bound
                if (sb < tb) { tb = sb; tseed = t; }
                if (dc - hi.w < tb) {
                    TriRec r;
                    load_rec(trec, t, r);
                    const float d = sqrtf(dist_rec_val(r, -rx, -ry, -rz));
                    const float ub = d * (1.f + 32.f * kU32) + 32.f * kU32 * (dc + 2.f * hi.w);
                    if (ub < tb || (ub == tb && t < tseed)) { tb = ub; tseed = t; }
                }
            }
        }
        // block argmin of (bound, triangle): bound bits first, then the id
        unsigned long long key =
            (static_cast<unsigned long long>(__float_as_uint(tb)) << 32) | static_cast<unsigned>(tseed);
#pragma unroll
        for (int sh = 16; sh > 0; sh >>= 1) {
            const unsigned long long k2 = __shfl_xor_sync(0xffffffffu, key, sh);
            key = k2 < key ? k2 : key;
        }
        if (lane == 0) s_red[warp] = key;
        __syncthreads();
        unsigned long long kmin = s_red[0];
#pragma unroll
        for (int i = 1; i < kSubThreads / 32; ++i) kmin = s_red[i] < kmin ? s_red[i] : kmin;
        const float U = __uint_as_float(static_cast<unsigned>(kmin >> 32));
        const int seed = static_cast<int>(static_cast<unsigned>(kmin & 0xffffffffull));
        // mixed: the stated FP32 error of a distance near d is 48u (d + 2 e + 2 r) (e the
        // mesh's largest centroid-to-vertex distance); kap carries its constant part
        const float kap = MIX ? __fmul_ru(98.f * kU32, __fadd_ru(s.emax_all, r4)) : 0.f;
        // the cells' pruning bound's constant: one stated error (mixed), three (exact)
        const float kapb = EXACT ? __fmul_ru(300.f * kU32, __fadd_ru(s.emax_all, r4)) : kap;
        const float ebr4 = MIX ? __fmul_ru(4.f, __fadd_ru(s.emax_all, r4)) : 0.f;
        // a triangle can be nearest to a cell only if its sphere reaches U + 2 r; in the
        // mixed path, also any triangle whose FP32 distance can undercut the nearest
        // one's (two stated errors more), so the filtered list holds every triangle the
        // FP32 minimum can come from; in the exact path every near-tie too (four)
        const float limf = (U + 2.f * r4) * (1.f + 32.f * kU32) + 32.f * kU32 * (U + r4) +
                           (EXACT ? __fmaf_ru(200.f * kU32, U + 4.f * r4, 4.f * kap)
                                  : MIX ? __fmaf_ru(100.f * kU32, U + 4.f * r4, 2.f * kap) : 0.f);

        // ---- 2+3. rounds: filter into shared memory, then evaluate the cells
        float best = FLT_MAX, bestd = FLT_MAX;  // FP32 path
        double best64 = DBL_MAX;                // FP64 path
        int bt = INT_MAX, br = 0;
        // exact path: the near-ties kept (s_near[0 .. nnear)), whether more were met, and
        // the squared threshold that keeps them (near_thr2 of the current minimum)
        int nnear = 0;
        bool over = false;
        float thr2 = 0.f;
        d3 P{0, 0, 0};
        if (PREC == kPrecFP64)
            P = {cell_center(g.corner[0], x, g.h), cell_center(g.corner[1], y, g.h),
                 cell_center(g.corner[2], z, g.h)};
        if (seed != INT_MAX && valid) {
            // the centre's nearest triangle: a tight start for every cell's bound
            const float4 hi = tinfo[seed], lo = tinfo_lo[seed];
            const float dx = px - ((hi.x - chx) + (lo.x - clx));
            const float dy = py - ((hi.y - chy) + (lo.y - cly));
            const float dz = pz - ((hi.z - chz) + (lo.z - clz));
            if (MIX) {
                TriRec r;
                load_rec(trec, seed, r);
                int reg;
                best = dist_rec(r, dx, dy, dz, &reg);
                ++evals;
                bt = seed;
                br = reg;
                bestd = EXACT ? cell_bound_x(best, kapb) : cell_bound(best, kap);
                if (EXACT) {
                    thr2 = near_thr2(best, kap);
                    s_near[0][tid] = make_int2(seed, __float_as_int(best));
                    nnear = 1;
                }
            } else {
                d3 a, b, c;
                load_soup(soup, seed, a, b, c);
                int reg;
                best64 = ericson(P, a, b, c, &reg);
                ++evals;
                bt = seed;
                br = reg;
                bestd = __double2float_ru(sqrt(best64)) * (1.f + 8.f * kU32);
            }
        }
        int64_t cursor = c0;
        while (cursor < c1) {
            if (tid == 0) s_n = 0;
            __syncthreads();
            int n = 0;
            while (cursor < c1 && n <= kCap - kBatch * kSubThreads) {
                int tt[kBatch];
                float4 hh[kBatch], ll[kBatch];
#pragma unroll
                for (int i = 0; i < kBatch; ++i) {
                    const int64_t k = cursor + tid + i * kSubThreads;
                    tt[i] = k < c1 ? cand[k] : -1;
                }
#pragma unroll
                for (int i = 0; i < kBatch; ++i)
                    if (tt[i] >= 0) { hh[i] = tinfo[tt[i]]; ll[i] = tinfo_lo[tt[i]]; }
#pragma unroll
                for (int i = 0; i < kBatch; ++i) {
                    bool take = false;
                    float4 e = make_float4(0.f, 0.f, 0.f, 0.f), nv = e;
                    float pe = 0.f;
                    const int t = tt[i];
                    if (t >= 0) {
                        e.x = (hh[i].x - chx) + (ll[i].x - clx);
                        e.y = (hh[i].y - chy) + (ll[i].y - cly);
                        e.z = (hh[i].z - chz) + (ll[i].z - clz);
                        e.w = hh[i].w;
                        const float dc = sqrtf(e.x * e.x + e.y * e.y + e.z * e.z);
                        // FP64 cells: the plane's distance from a cell is at most its
                        // distance from the triangle, so a triangle whose plane stays
                        // beyond every cell's reach (U + r from the centre) cannot be
                        // nearest to any of them. pe bounds the plane distances' error
                        // at any cell of the sub-brick (normal error n.w; rounding of the
                        // FP32 centroid, cell offsets and dot products). In the mixed
                        // path an FP32 distance costs about as much as this test, which
                        // is left out there.
                        take = dc - e.w <= limf;
                        if (PREC == kPrecFP64 && take) {
                            nv = tnorm[t];
                            pe = (nv.w + 12.f * kU32) * (dc + r4) * 1.1f + 1e-30f;
                            nv.w = fmaf(nv.x, e.x, fmaf(nv.y, e.y, nv.z * e.z));
                            take = fabsf(nv.w) - pe <= limf;
                        }
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, take);
                    int base = 0;
                    if (lane == 0 && m) base = atomicAdd(&s_n, __popc(m));
                    base = __shfl_sync(0xffffffffu, base, 0);
                    if (take) {
                        const int pos = base + __popc(m & ((1u << lane) - 1u));
                        if (EXPAND) {
                            e.w = exp_term(reach_term(e.w, r4), sr);
                            s_g[pos] = exp_g(e.x, e.y, e.z, e.w);
                            e.x *= -2.f;
                            e.y *= -2.f;
                            e.z *= -2.f;
                        } else if (MIX && !STAGE) {
                            e.w = reach_term(e.w, r4);
                        }
                        s_c[pos] = e;
                        if (PREC == kPrecFP64) {
                            s_nrm[pos] = nv;
                            s_pe[pos] = pe;
                        }
                        s_t[pos] = t;
                        if (STAGE) {
                            const float4* src = reinterpret_cast<const float4*>(trec + t);
                            float4* dst = reinterpret_cast<float4*>(&s_rec[pos]);
#pragma unroll
                            for (int q2 = 0; q2 < kRecVec; ++q2) cp_async16(dst + q2, src + q2);
                        }
                    }
                }
                cursor += kBatch * kSubThreads;
                if (STAGE) cp_async_wait_all();
                __syncthreads();
                n = s_n;
            }
            if (tid == 0 && n) atomicAdd(&st->filtered, static_cast<unsigned long long>(n));
            if (MIX && !STAGE) {
                // In chunks of kChunk entries: each lane marks the entries its cell may
                // need under its bound at the start of the chunk (s_c[].w holds the
                // radius term of the reach, see reach_term; EXPAND: the widened term T of
                // the expanded test, with -2 x the centroid in s_c[].xyz and exp_g in
                // s_g, see exp_term); the warp stages the records
                // of the union into its shared slots (lane k loads entry k's record:
                // every load of the chunk in flight at once) and evaluates every marked
                // entry. The bound only shrinks and the test admits at least what the
                // one-by-one test with the running bound admits, so every triangle that
                // can be nearest is evaluated; the running minimum is of (distance,
                // triangle id) pairs, so the extra evaluations change nothing.
                // Before the cells' tests, lane k tests entry k of the chunk once against
                // the warp's sphere (s_wsph) with the largest bound of its cells: the
                // entries that fail are beyond every cell's reach and skip the cells'
                // tests (see warp_reach).
                TriRec* wrec = s_wrec + warp * kChunk;
                for (int j0 = 0; j0 < n; j0 += kChunk) {
                    const int cnt = min(kChunk, n - j0);
                    const float bmax =
                        __uint_as_float(__reduce_max_sync(0xffffffffu, valid ? __float_as_uint(bestd) : 0u));
                    bool pass = false;
                    if (lane < cnt) {
                        const float4 ws = s_wsph[warp];
                        const float4 e = s_c[j0 + lane];
                        float dx, dy, dz, lw;
                        if (EXPAND) {
                            dx = fmaf(0.5f, e.x, ws.x);
                            dy = fmaf(0.5f, e.y, ws.y);
                            dz = fmaf(0.5f, e.z, ws.z);
                            lw = warp_reach(exp_pass_reach(exp_b(bmax), e.w, sw), ws.w);
                        } else {
                            dx = ws.x - e.x;
                            dy = ws.y - e.y;
                            dz = ws.z - e.z;
                            lw = warp_reach(reach(bmax, e.w), ws.w);
                        }
                        pass = dx * dx + dy * dy + dz * dz <= lw * lw;
                    }
                    const unsigned cand = __ballot_sync(0xffffffffu, pass);
                    unsigned mine = 0;
                    if (valid && EXPAND) {
                        const float bb = exp_b(bestd);
                        const float kk = fmaf(bb, bb, -p2), mb = -2.f * bb;
                        if (cnt == kChunk && __popc(cand) >= kDenseChunk) {
#pragma unroll
                            for (int k = 0; k < kChunk; ++k) {
                                const float4 e = s_c[j0 + k];
                                const float a = fmaf(px, e.x, fmaf(py, e.y, fmaf(pz, e.z, fmaf(mb, e.w, s_g[j0 + k]))));
                                if (a <= kk) mine |= 1u << k;
                            }
                        } else {
                            for (unsigned m = cand; m; m &= m - 1u) {
                                const int k = __ffs(m) - 1;
                                const float4 e = s_c[j0 + k];
                                const float a = fmaf(px, e.x, fmaf(py, e.y, fmaf(pz, e.z, fmaf(mb, e.w, s_g[j0 + k]))));
                                if (a <= kk) mine |= 1u << k;
                            }
                        }
                    } else if (valid) {
                        const float bl = bestd;
                        if (cnt == kChunk && __popc(cand) >= kDenseChunk) {
                            // most entries passed: every entry, unrolled (the entries that
                            // failed the warp test fail here too)
#pragma unroll
                            for (int k = 0; k < kChunk; ++k) {
                                const float4 e = s_c[j0 + k];
                                const float dx = px - e.x, dy = py - e.y, dz = pz - e.z;
                                const float lim = reach(bl, e.w);
                                if (dx * dx + dy * dy + dz * dz <= lim * lim) mine |= 1u << k;
                            }
                        } else {
                            for (unsigned m = cand; m; m &= m - 1u) {
                                const int k = __ffs(m) - 1;
                                const float4 e = s_c[j0 + k];
                                const float dx = px - e.x, dy = py - e.y, dz = pz - e.z;
                                const float lim = reach(bl, e.w);
                                if (dx * dx + dy * dy + dz * dz <= lim * lim) mine |= 1u << k;
                            }
                        }
                    }
                    const unsigned any = __reduce_or_sync(0xffffffffu, mine);
                    if (!any) continue;
                    if ((any >> lane) & 1u) {
                        const int slot = __popc(any & ((1u << lane) - 1u));
                        const float4* src = reinterpret_cast<const float4*>(trec + s_t[j0 + lane]);
                        float4* dst = reinterpret_cast<float4*>(wrec + slot);
                        float4 v[kRecVec];
#pragma unroll
                        for (int q2 = 0; q2 < kRecVec; ++q2) v[q2] = __ldg(src + q2);
#pragma unroll
                        for (int q2 = 0; q2 < kRecVec; ++q2) dst[q2] = v[q2];
                    }
                    __syncwarp();
                    unsigned m = any;
                    for (int slot = 0; m; ++slot) {
                        const int k = __ffs(m) - 1;
                        m &= m - 1u;
                        const float4 e = s_c[j0 + k];
                        const float dx = EXPAND ? fmaf(0.5f, e.x, px) : px - e.x;
                        const float dy = EXPAND ? fmaf(0.5f, e.y, py) : py - e.y;
                        const float dz = EXPAND ? fmaf(0.5f, e.z, pz) : pz - e.z;
                        // the plane: a triangle is no nearer than the plane of its frame
                        // (every triangle, degenerate or not, lies in one), so a marked
                        // triangle whose plane lies beyond every lane's bound is skipped
                        // (see plane_reach); its n component is the distance's first step
                        const TriRec& R = wrec[slot];
                        const PaN pn = pa_n(R, dx, dy, dz);
                        if (!__any_sync(0xffffffffu, valid && fabsf(pn.n) <= plane_reach(bestd, R.nerr, ebr4)))
                            continue;
                        if (valid) {
                            const float d2 = dist_rec_t<false>(R, pn, nullptr);
                            ++evals;
                            const int t = s_t[j0 + k];
                            if (d2 < best || (d2 == best && t < bt)) {
                                best = d2;
                                bt = t;
                                br = -1;  // the region of the final triangle is found below
                                bestd = EXACT ? cell_bound_x(d2, kapb) : cell_bound(d2, kap);
                                if (EXACT) {
                                    // a new minimum: drop the kept near-ties beyond its
                                    // (smaller) threshold
                                    thr2 = near_thr2(d2, kap);
                                    int kept = 0;
                                    for (int q = 0; q < nnear; ++q) {
                                        const int2 nt = s_near[q][tid];
                                        if (__int_as_float(nt.y) <= thr2) s_near[kept++][tid] = nt;
                                    }
                                    nnear = kept;
                                }
                            }
                            // every triangle within the threshold when evaluated is kept
                            // (the threshold only shrinks; the seed is kept already)
                            if (EXACT && d2 <= thr2 && t != seed) {
                                if (nnear < kNear) s_near[nnear++][tid] = make_int2(t, __float_as_int(d2));
                                else over = true;
                            }
                        }
                    }
                    __syncwarp();
                }
            } else
            for (int j = 0; j < n; ++j) {
                const float4 e = s_c[j];
                const float dx = px - e.x, dy = py - e.y, dz = pz - e.z;
                const float lim = (bestd + e.w) * (1.f + 16.f * kU32) + 16.f * kU32 * r4;
                bool need = valid && dx * dx + dy * dy + dz * dz <= lim * lim;
                if (!__any_sync(0xffffffffu, need)) continue;
                if (PREC == kPrecFP64) {
                    // and the plane: its distance from the cell bounds the triangle's below
                    const float4 nv = s_nrm[j];
                    const float pd = fabsf(fmaf(nv.x, px, fmaf(nv.y, py, fmaf(nv.z, pz, -nv.w))));
                    need = need && pd - s_pe[j] <= bestd * (1.f + 16.f * kU32) + 16.f * kU32 * r4;
                    if (!__any_sync(0xffffffffu, need)) continue;
                }
                const int t = s_t[j];
                if (MIX) {
                    TriRec rr;
                    if (!STAGE) load_rec(trec, t, rr);
                    const TriRec& r = STAGE ? s_rec[j] : rr;
                    if (valid) {
                        int reg;
                        const float d2 = dist_rec(r, dx, dy, dz, &reg);
                        ++evals;
                        if (d2 < best || (d2 == best && t < bt)) {
                            best = d2;
                            bt = t;
                            br = reg;
                            bestd = cell_bound(d2, kap);
                        }
                    }
                } else {
                    d3 a, b, c;
                    load_soup(soup, t, a, b, c);
                    if (valid) {
                        int reg;
                        const double d2 = ericson(P, a, b, c, &reg);
                        ++evals;
                        if (d2 < best64 || (d2 == best64 && t < bt)) {
                            best64 = d2;
                            bt = t;
                            br = reg;
                            bestd = __double2float_ru(sqrt(d2)) * (1.f + 8.f * kU32);
                        }
                    }
                }
            }
            __syncthreads();
        }

        // ---- 4. mixed: FP64 band
        float eb = 0.f;
        bool inband = false;
        double best_band = DBL_MAX;
        int bt64 = INT_MAX, br64 = 0;
        if (MIX) {
            const float d32 = sqrtf(best);
            // the mesh's largest triangle radius (not the brick's candidates', which
            // depend on the candidate walk): the bound, and the band it selects, are
            // the same whatever slab of the grid is evaluated
            eb = 48.f * kU32 * (d32 + 2.f * s.emax_all + 2.f * r4) + 1e-30f;
            if (EXACT) {
                // the FP64 distance, in the reference's order, of every kept near-tie: the
                // FP64 minimum over all triangles (lowest index on ties). A cell that met
                // more near-ties than it could keep, or none, takes the band pass below.
                if (valid && !over) {
                    const d3 Pc{cell_center(g.corner[0], x, g.h), cell_center(g.corner[1], y, g.h),
                                cell_center(g.corner[2], z, g.h)};
                    for (int q = 0; q < nnear; ++q) {
                        const int2 nt = s_near[q][tid];
                        d3 a, b, c;
                        load_soup(soup, nt.x, a, b, c);
                        int r64;
                        const double e2 = ericson(Pc, a, b, c, &r64);
                        ++evals64;
                        if (e2 < best_band || (e2 == best_band && nt.x < bt64)) {
                            best_band = e2;
                            bt64 = nt.x;
                            br64 = r64;
                        }
                    }
                }
                inband = valid && (over || nnear == 0);
            } else {
                inband = valid && d32 <= band_cells * static_cast<float>(g.h) + eb;
            }
            if (__any_sync(0xffffffffu, inband) && lane == 0) s_band = 1;
            __syncthreads();
            if (s_band) {
                const float reach = d32 + 2.f * eb;
                const d3 Pc{cell_center(g.corner[0], x, g.h), cell_center(g.corner[1], y, g.h),
                            cell_center(g.corner[2], z, g.h)};
                // the CTA's largest band reach: a triangle passes some band cell's test
                // below only if its sphere comes within that reach plus the sub-brick
                // radius of the centre, so the brick list is compacted to those first
                // (one cooperative pass) instead of every cell testing all of it
                {
                    const unsigned rbits = __reduce_max_sync(0xffffffffu, inband ? __float_as_uint(reach) : 0u);
                    if (tid == 0) s_rmax = 0u;
                    __syncthreads();
                    if (lane == 0) atomicMax(&s_rmax, rbits);
                    __syncthreads();
                }
                const float Rb = __uint_as_float(s_rmax);
                int64_t bcur = c0;
                while (bcur < c1) {
                    if (tid == 0) s_n = 0;
                    __syncthreads();
                    int n = 0;
                    while (bcur < c1 && n <= kCap - kSubThreads) {
                        const int64_t k = bcur + tid;
                        bool take = false;
                        float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
                        int t = -1;
                        if (k < c1) {
                            t = cand[k];
                            const float4 hi = tinfo[t], lo = tinfo_lo[t];
                            e = make_float4((hi.x - chx) + (lo.x - clx), (hi.y - chy) + (lo.y - cly),
                                            (hi.z - chz) + (lo.z - clz), hi.w);
                            const float limb = ((Rb + e.w) * (1.f + 16.f * kU32) + r4 * (1.f + 17.f * kU32)) *
                                               (1.f + 8.f * kU32);
                            take = sqrtf(e.x * e.x + e.y * e.y + e.z * e.z) <= limb;
                        }
                        const unsigned m = __ballot_sync(0xffffffffu, take);
                        int base = 0;
                        if (lane == 0 && m) base = atomicAdd(&s_n, __popc(m));
                        base = __shfl_sync(0xffffffffu, base, 0);
                        if (take) {
                            const int pos = base + __popc(m & ((1u << lane) - 1u));
                            s_c[pos] = e;
                            s_t[pos] = t;
                        }
                        bcur += kSubThreads;
                        __syncthreads();
                        n = s_n;
                    }
                    for (int j = 0; j < n; ++j) {
                        const float4 e = s_c[j];
                        const float dx = px - e.x, dy = py - e.y, dz = pz - e.z;
                        const float lim = (reach + e.w) * (1.f + 16.f * kU32) + 16.f * kU32 * r4;
                        const bool need = inband && dx * dx + dy * dy + dz * dz <= lim * lim;
                        if (!__any_sync(0xffffffffu, need)) continue;
                        const int t = s_t[j];
                        TriRec r;
                        load_rec(trec, t, r);
                        if (!need) continue;
                        const float d = sqrtf(dist_rec_val(r, dx, dy, dz));
                        if (d > reach * (1.f + 1e-6f)) continue;
                        d3 a, b, c;
                        load_soup(soup, t, a, b, c);
                        int r64;
                        const double e2 = ericson(Pc, a, b, c, &r64);
                        ++evals64;
                        if (e2 < best_band || (e2 == best_band && t < bt64)) {
                            best_band = e2;
                            bt64 = t;
                            br64 = r64;
                        }
                    }
                    __syncthreads();
                }
            }
        }
        if (valid) {
            const int64_t idx = s.vox_begin + (static_cast<int64_t>(z - g.z0) * g.ny + y) * g.nx + x;
            if (PREC == kPrecFP64) {
                write_cell(o, idx, __dsqrt_rn(best64), bt, br);
            } else if (EXACT) {
                if (inband) ++bandc;
                write_cell(o, idx, __dsqrt_rn(best_band), bt64, br64);
            } else if (inband) {
                ++bandc;
                write_cell(o, idx, __dsqrt_rn(best_band), bt64, br64);
                if (o.errbound) o.errbound[idx] = 0.f;
            } else {
                if (MIX && !STAGE && br < 0 && o.near_reg) {
                    // the region of the nearest triangle: its distance again, recentred
                    // exactly as the filter recentred it (the same value, now with the
                    // region)
                    const float4 hi = tinfo[bt], lo = tinfo_lo[bt];
                    const float ex = (hi.x - chx) + (lo.x - clx), ey = (hi.y - chy) + (lo.y - cly),
                                ez = (hi.z - chz) + (lo.z - clz);
                    TriRec r;
                    load_rec(trec, bt, r);
                    dist_rec(r, px - ex, py - ey, pz - ez, &br);
                }
                write_cell(o, idx, static_cast<double>(sqrtf(best)), bt, br);
                if (o.errbound) o.errbound[idx] = eb;
            }
        }
        __syncthreads();
      }
    }
    long long ev = warp_sum(static_cast<long long>(evals));
    long long ev64 = warp_sum(static_cast<long long>(evals64));
    long long bc = warp_sum(static_cast<long long>(bandc));
    if (lane == 0) {
        if (ev) atomicAdd(&st->evaluations, static_cast<unsigned long long>(ev));
        const long long f64 = PREC == kPrecFP64 ? ev : ev64;
        if (f64) atomicAdd(&st->fp64_evaluations, static_cast<unsigned long long>(f64));
        if (bc) atomicAdd(&st->band_voxels, static_cast<unsigned long long>(bc));
    }
}

// Work ids of the sub-bricks (brick * 64 + sub) in LPT order: key = ~brick count.
__global__ void k_sub_work_keys(const int* __restrict__ cand_cnt, int64_t nbricks,
                                uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    int64_t w = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (w >= nbricks * 64) return;
    keys[w] = ~static_cast<uint32_t>(cand_cnt[w >> 6]);
    vals[w] = static_cast<uint32_t>(w);
}

}  // namespace

void launch_sub_work_keys(const int* cand_cnt, int64_t nbricks, uint32_t* keys, uint32_t* vals,
                          cudaStream_t st) {
    if (nbricks == 0) return;
    const int64_t n = nbricks * 64;
    k_sub_work_keys<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(cand_cnt, nbricks, keys,
                                                                           vals);
    CMG_LAUNCH();
}

namespace {
template <int PREC, bool STAGE, int MINB>
int resident_ctas() {
    int per = 0;
    CMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sdf_sub<PREC, STAGE, MINB>,
                                                           kSubThreads, 0));
    return per > 0 ? per : 1;
}
}  // namespace

// Resident CTAs per SM targeted by the evaluation kernel: 16 when asked for, else 12.
int sdf_sub_minb(int ctas) { return ctas == 16 ? 16 : 12; }

int sdf_sub_grid(int precision, bool stage, int ctas) {
    const int sms = device_sms();
    const bool hi = sdf_sub_minb(ctas) == 16;
    int per;
    if (precision == kPrecMixed && stage) per = resident_ctas<kPrecMixed, true, 12>();
    else if (precision == kPrecMixed) per = hi ? resident_ctas<kPrecMixed, false, 16>()
                                               : resident_ctas<kPrecMixed, false, 12>();
    else if (precision == kPrecExact) per = hi ? resident_ctas<kPrecExact, false, 16>()
                                               : resident_ctas<kPrecExact, false, 12>();
    else per = hi ? resident_ctas<kPrecFP64, false, 16>() : resident_ctas<kPrecFP64, false, 12>();
    return sms * per;
}

void launch_sdf_sub(int precision, bool stage, int grab, int probe, int ctas, const MeshSeg* segs,
                    int nseg, const uint32_t* work, int64_t nwork, unsigned long long* queue,
                    const double* soup, const float4* tinfo, const float4* tinfo_lo, const void* trec,
                    const float4* tnorm, const int64_t* cand_off, const int* cand, const float* brick_emax,
                    float band_cells, const uint8_t* occ, float* sdf32, double* sdf64,
                    int* near_tri, uint8_t* near_reg, float* errbound, Stats* stats, int grid,
                    cudaStream_t st) {
    if (nwork == 0) return;
    Out o{occ, sdf32, sdf64, near_tri, near_reg, errbound};
    const TriRec* r = static_cast<const TriRec*>(trec);
    if (grab != 1 && grab != 2 && grab != 4 && grab != 8) grab = 1;
    if (probe <= 0) probe = kProbe;
    const bool hi = sdf_sub_minb(ctas) == 16;
    auto go = [&](auto kernel) {
        kernel<<<grid, kSubThreads, 0, st>>>(segs, nseg, work, nwork, grab, probe, queue, soup, tinfo,
                                            tinfo_lo, r, tnorm, cand_off, cand, brick_emax, band_cells,
                                            o, stats);
    };
    if (precision == kPrecMixed && stage) go(k_sdf_sub<kPrecMixed, true, 12>);
    else if (precision == kPrecMixed) hi ? go(k_sdf_sub<kPrecMixed, false, 16>) : go(k_sdf_sub<kPrecMixed, false, 12>);
    else if (precision == kPrecExact) hi ? go(k_sdf_sub<kPrecExact, false, 16>) : go(k_sdf_sub<kPrecExact, false, 12>);
    else hi ? go(k_sdf_sub<kPrecFP64, false, 16>) : go(k_sdf_sub<kPrecFP64, false, 12>);
    CMG_LAUNCH();
}

}  // namespace cmg::gpu
