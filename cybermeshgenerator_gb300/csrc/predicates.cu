// predicates.cu — batched orient3d / insphere sign streams.
//
// Semantics per query (src/predicates/robust.cpp:36-50 as initialised by :28-34):
//   COMPAT: sign of the rounded determinant in Shewchuk's operation order
//           (predicates.cpp:2201-2222, 4067-4110) unless it is exactly zero, then
//           the exact sign (the reference's orient3dadapt / insphereadapt result);
//   EXACT:  the sign of the exact determinant.
// Three passes, each over a compacted list of the queries the previous pass could
// not decide, so that divergent work never holds back a full warp:
//   k_pred_fp32   one thread per query, coordinates streamed from HBM (SoA) into
//                 shared memory by the TMA engine (bulk copies, mbarrier pipeline;
//                 per-thread loads for unaligned columns and the tail), the
//                 queries it leaves listed per CTA with their coordinates (see
//                 Seg), the determinant in FP32 with a rigorous bound that
//                 covers the rounding of the inputs to FP32 and of every FP32
//                 operation, plus the FP64 filter bound of the reference: a sign it
//                 certifies is the exact sign and also the sign of the FP64 rounded
//                 determinant, so it serves both modes;
//   k_pred_fp64   the reference's rounded determinant (and, in EXACT mode, its
//                 permanent bound); when that does not decide, an evaluation with
//                 exactness tracking (cmg_exact.cuh): if no operation rounded, its
//                 value is the exact determinant;
//   k_pred_exact  expansion arithmetic (cmg_exact.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/cmg_c/cmg_gpu.h"
#include "cmg_device.cuh"
#include "cmg_exact.cuh"
#include "cmg_types.h"
#include "cmg_util.h"
#include "engine.h"

namespace cmg::gpu {

namespace {

constexpr float kU = 5.9604645e-8f;  // 2^-24
constexpr int kThreads = 256;
constexpr int kTile = 256;  // queries per tile of the FP32 pass: one per thread

struct Soa {
    const double* c[15];
};

// The list of the queries the FP32 pass leaves, in segments: CTA b of the pass (of
// nseg, b = tile % nseg) appends the queries of its tiles to segment b, entries
// [b * segcap, b * segcap + cnt[b]), counting them in shared memory, so no global
// atomic sits between a tile's certification and the release of its stage. Entry j of
// segment b with j < ccap also has its coordinates at cc[.][b * ccap + j], copied by
// the FP32 pass from the tile it holds, so that the FP64 pass reads them contiguously
// instead of gathering each from its own column at a scattered index (a whole DRAM
// access per 8-byte value); entries at j >= ccap are gathered.
constexpr int kMaxSeg = 2048;
struct Seg {
    int64_t* list;
    unsigned long long* cnt;  // [nseg]
    int nseg;
    int64_t segcap, ccap;
    double* cc[15];
};

__device__ __forceinline__ float amax3(float a, float b, float c) {
    return fmaxf(fabsf(a), fmaxf(fabsf(b), fabsf(c)));
}

// FP64 -> FP32 by truncating the significand, on the integer pipe (the hardware
// conversion is far slower on this part): |f - x| < 2^-23 |x|. Zero maps to zero;
// values outside the FP32 normal range, subnormals, infinities and NaN set ok = false.
// The FP64 fields shifted left by 3 (a funnel shift of hi:lo) put the exponent's low 9
// bits over the FP32 exponent and the top 23 significand bits over the FP32 significand;
// adding 128 to that 9-bit field turns e64 mod 512 into e64 - 896 = e32 for every
// exponent of the FP32 normal range (e64 in [897, 1150]), with the 9th bit clear.
__device__ __forceinline__ float trunc32(double x, bool& ok) {
    const unsigned hi = static_cast<unsigned>(__double2hiint(x));
    const unsigned lo = static_cast<unsigned>(__double2loint(x));
    const unsigned e = (hi >> 20) & 0x7ffu;
    const bool zero = ((hi << 1) | lo) == 0u;
    ok = ok && (zero || e - 897u <= 253u);
    const unsigned r = __funnelshift_l(lo, hi, 3) + (128u << 23);
    return __uint_as_float(zero ? (hi & 0x80000000u) : (r | (hi & 0x80000000u)));
}

// FP32 orient3d: certified sign (+1/-1) or 0 when the bound does not decide.
// Inputs truncated to FP32 are off by less than 2 u |v|, so the FP32 differences
// (|difference| <= 2A, A the largest magnitude) are off by at most eta = 6 u A; the
// determinant (six products of three differences, at most five roundings deep) then
// errs by at most 72 eta A^2 + 5 u 48 A^3 = 672 u A^3 to first order; 1024 u A^3 is
// used. The reference's FP64 bound o3derrboundA * permanent is at most
// 7.8e-16 * 48 A^3 and is added, so a certified sign is the sign of the FP64 rounded
// determinant as well.
__device__ __forceinline__ int o3d_fp32(const double* v) {
    float f[12];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 12; ++i) f[i] = trunc32(v[i], ok);
    if (!ok) return 0;
    float A = 0.f;
#pragma unroll
    for (int i = 0; i < 12; i += 3) A = fmaxf(A, amax3(f[i], f[i + 1], f[i + 2]));
    const float adx = f[0] - f[9], ady = f[1] - f[10], adz = f[2] - f[11];
    const float bdx = f[3] - f[9], bdy = f[4] - f[10], bdz = f[5] - f[11];
    const float cdx = f[6] - f[9], cdy = f[7] - f[10], cdz = f[8] - f[11];
    const float det = adz * (bdx * cdy - cdx * bdy) + bdz * (cdx * ady - adx * cdy) +
                      cdz * (adx * bdy - bdx * ady);
    const float A3 = A * A * A * (1.f + 8.f * kU);
    const float bound = 1024.f * kU * A3 + 4e-14f * A3 + 1e-36f;
    if (!(A3 < 1e30f)) return 0;  // overflow / non-finite: no certificate
    return det > bound ? 1 : (det < -bound ? -1 : 0);
}

// The lifted insphere determinant (e as origin) of 12 differences, and the same
// expression over absolute values (every monomial counted with its magnitude).
__device__ __forceinline__ float isp_lifted(const float* x) {
    const float aex = x[0], aey = x[1], aez = x[2], bex = x[3], bey = x[4], bez = x[5];
    const float cex = x[6], cey = x[7], cez = x[8], dex = x[9], dey = x[10], dez = x[11];
    const float ab = aex * bey - bex * aey, bc = bex * cey - cex * bey;
    const float cd = cex * dey - dex * cey, da = dex * aey - aex * dey;
    const float ac = aex * cey - cex * aey, bd = bex * dey - dex * bey;
    const float abc = aez * bc - bez * ac + cez * ab;
    const float bcd = bez * cd - cez * bd + dez * bc;
    const float cda = cez * da + dez * ac + aez * cd;
    const float dab = dez * ab + aez * bd + bez * da;
    const float al = aex * aex + aey * aey + aez * aez;
    const float bl = bex * bex + bey * bey + bez * bez;
    const float cl = cex * cex + cey * cey + cez * cez;
    const float dl = dex * dex + dey * dey + dez * dez;
    return (dl * abc - cl * dab) + (bl * cda - al * bcd);
}
__device__ __forceinline__ float isp_absolute(const float* x) {  // x >= 0
    const float aex = x[0], aey = x[1], aez = x[2], bex = x[3], bey = x[4], bez = x[5];
    const float cex = x[6], cey = x[7], cez = x[8], dex = x[9], dey = x[10], dez = x[11];
    const float ab = aex * bey + bex * aey, bc = bex * cey + cex * bey;
    const float cd = cex * dey + dex * cey, da = dex * aey + aex * dey;
    const float ac = aex * cey + cex * aey, bd = bex * dey + dex * bey;
    const float abc = aez * bc + bez * ac + cez * ab;
    const float bcd = bez * cd + cez * bd + dez * bc;
    const float cda = cez * da + dez * ac + aez * cd;
    const float dab = dez * ab + aez * bd + bez * da;
    const float al = aex * aex + aey * aey + aez * aez;
    const float bl = bex * bex + bey * bey + bez * bez;
    const float cl = cex * cex + cey * cey + cez * cez;
    const float dl = dex * dex + dey * dey + dez * dez;
    return (dl * abc + cl * dab) + (bl * cda + al * bcd);
}

// FP32 insphere with a permanent-style bound. Inputs truncated to FP32
// (|f - v| < 2 u |v|) and differences D = fl(f_a - f_e) satisfy
// |D - d| <= 1.01 u |D| + 4.02 u A (A = max |f|). The lifted determinant is a sum of degree-5 monomials, so
//   |det(D) - det(d)| <= P(|D| + |D - d|) - P(|D|) <= P2 - P1,
// P the absolute-value polynomial, P1 = P(|D|), P2 = P(|D| (1 + 1.01 u) + 4.02 u A)
// (entries inflated once more by 4 u for their own rounding); the FP32 evaluation
// of det(D) (at most eight roundings deep) errs by at most 8.1 u P(|D|); P1 and P2
// are themselves computed in FP32 (relative error <= 9 u each). Bound:
//   (P2 - P1) + 20 u (P1 + P2) + 1e-36,
// which also covers the reference's FP64 bound isperrboundA * permanent (~16e-16
// relative): a certified sign is exact and is the sign of the FP64 rounded
// determinant. The additive term covers FP32 underflow (< 1e-43 over the whole
// evaluation); no certificate on overflow or when A < 1e-30.
__device__ __forceinline__ int isp_fp32(const double* v) {
    float f[15];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 15; ++i) f[i] = trunc32(v[i], ok);
    if (!ok) return 0;
    float A = 0.f;
#pragma unroll
    for (int i = 0; i < 15; i += 3) A = fmaxf(A, amax3(f[i], f[i + 1], f[i + 2]));
    float D[12], X[12], Y[12];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int q = 0; q < 3; ++q) D[3 * k + q] = f[3 * k + q] - f[12 + q];
    const float eta = 4.02f * kU * A * (1.f + 4.f * kU);
#pragma unroll
    for (int i = 0; i < 12; ++i) {
        X[i] = fabsf(D[i]);
        Y[i] = (X[i] * (1.f + 1.01f * kU) + eta) * (1.f + 4.f * kU);
    }
    const float det = isp_lifted(D);
    const float p1 = isp_absolute(X), p2 = isp_absolute(Y);
    if (!(p2 < 1e30f) || !(A >= 1e-30f)) return 0;  // overflow, non-finite or tiny
    const float bound = (p2 - p1) + 20.f * kU * (p1 + p2) + 1e-36f;
    return det > bound ? 1 : (det < -bound ? -1 : 0);
}

template <int NPT>
__device__ __forceinline__ void load_query(const Soa& s, int64_t i, double* v) {
#pragma unroll
    for (int k = 0; k < 3 * NPT; ++k) v[k] = __ldg(s.c[k] + i);
}

// Appends the lanes with `flag` to list (warp-aggregated).
__device__ __forceinline__ void push(bool flag, int64_t i, int64_t* list,
                                     unsigned long long* count) {
    const unsigned m = __ballot_sync(0xffffffffu, flag);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == __ffs(m) - 1) base = atomicAdd(count, static_cast<unsigned long long>(__popc(m)));
    base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
    if (flag) list[base + __popc(m & ((1u << lane) - 1u))] = i;
}

// Position of the lanes with `flag` in this CTA's segment (warp-aggregated on the
// CTA's shared count); -1 without flag.
__device__ __forceinline__ int64_t seg_pos(bool flag, unsigned long long* s_cnt) {
    const unsigned m = __ballot_sync(0xffffffffu, flag);
    if (!m) return -1;
    const int lane = threadIdx.x & 31, lead = __ffs(m) - 1;
    unsigned long long base = 0;
    if (lane == lead) base = atomicAdd(s_cnt, static_cast<unsigned long long>(__popc(m)));
    base = __shfl_sync(0xffffffffu, base, lead);
    return flag ? static_cast<int64_t>(base + __popc(m & ((1u << lane) - 1u))) : -1;
}

// The FP32 pass with per-thread loads over tiles [t0, t1) (queries below n): CTA b of
// the grid (gridDim.x == L.nseg) takes the tiles t with t % nseg == b and appends to
// segment b, after what an earlier launch left there. Serves the tail tile and
// columns the bulk copies cannot take, the rerun after a TMA wait ran out, and (PULL)
// host memory the device reads through the host's page tables: each query is then
// loaded once over the host link and its coordinates stored to the device columns
// `dst` that the FP64 and exact passes read.
template <int NPT, bool PULL>
__global__ void __launch_bounds__(kThreads, 4) k_pred_fp32_seg(Soa src, Soa dst, int64_t t0, int64_t t1,
                                                               int64_t n, int8_t* __restrict__ out, Seg L) {
    __shared__ unsigned long long s_cnt;
    const int b = blockIdx.x, G = gridDim.x;
    if (threadIdx.x == 0) s_cnt = L.cnt[b];
    __syncthreads();
    int64_t* seg = L.list + static_cast<int64_t>(b) * L.segcap;
    // the device copy of the coordinates (PULL: the columns written here)
    const Soa& dev = PULL ? dst : src;
    for (int64_t t = t0 + ((b - t0 % G) % G + G) % G; t < t1; t += G) {
        const int64_t i = t * kTile + threadIdx.x;
        const bool live = i < n;
        int sg = 0;
        if (live) {
            double v[3 * NPT];
#pragma unroll
            for (int k = 0; k < 3 * NPT; ++k) v[k] = PULL ? src.c[k][i] : __ldg(src.c[k] + i);
            if (PULL) {
#pragma unroll
                for (int k = 0; k < 3 * NPT; ++k) const_cast<double*>(dst.c[k])[i] = v[k];
            }
            sg = NPT == 4 ? o3d_fp32(v) : isp_fp32(v);
            out[i] = static_cast<int8_t>(sg);
        }
        const int64_t pos = seg_pos(live && sg == 0, &s_cnt);
        if (pos >= 0) {
            seg[pos] = i;
            if (pos < L.ccap) {
                // read again from device memory (this thread's own loads or stores, in
                // L1 / L2), which keeps the values out of registers across the append
#pragma unroll
                for (int k = 0; k < 3 * NPT; ++k) L.cc[k][b * L.ccap + pos] = dev.c[k][i];
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) L.cnt[b] = s_cnt;
}

// Bytes [0, n) of src to dst (host memory written by the device): 16-byte words
// when dst is 16-byte aligned (src always is), single bytes otherwise and for the
// tail.
__global__ void k_put_bytes(const int8_t* __restrict__ src, int8_t* __restrict__ dst, int64_t n) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const int64_t t0 = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
        const int64_t nw = n / 16;
        for (int64_t w = t0; w < nw; w += stride)
            reinterpret_cast<uint4*>(dst)[w] = reinterpret_cast<const uint4*>(src)[w];
        done = nw * 16;
    }
    for (int64_t i = done + t0; i < n; i += stride) dst[i] = src[i];
}

// ---- the FP32 pass with the columns moved by the TMA engine ----------------------
// A persistent CTA streams tiles of kTile queries: per tile one bulk copy per
// coordinate column (cp.async.bulk, global -> shared, completion counted on an
// mbarrier), kStages tiles in flight, one thread per query computing from shared
// memory, the queries left appended to the CTA's own list segment (a shared-memory
// count); a producer warp refills a stage once every consumer warp has arrived on the
// stage's `empty` mbarrier. Every wait is bounded: a wait that runs out (it never
// should) stops every warp of the CTA (a shared flag the other waits watch), the CTA
// drains the last copy issued into each stage, and sets `fault`, on which the host
// reruns the pass with the per-thread loads. When the drain's own bounded waits run out
// as well, the CTA sets `drain_fault` too: copies may still have been writing its
// shared memory, and the host reports an error instead of rerunning.
template <int NPT>
struct Tma {
    static constexpr int kCols = 3 * NPT;
    static constexpr int kStages = NPT == 4 ? 4 : 3;
    static constexpr unsigned kStageBytes = kCols * kTile * 8u;
    static constexpr size_t kSmem = static_cast<size_t>(kStages) * kStageBytes;
};

__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, unsigned bytes,
                                          unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase with the given parity for at most about a second of clocks.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > (1ll << 31)) return false;
    return true;
}
// The same, giving up at once when *abort is set (another warp's wait ran out).
__device__ __forceinline__ bool mbar_wait_or_abort(unsigned long long* bar, unsigned parity,
                                                   const volatile int* abort) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (*abort || clock64() - t0 > (1ll << 31)) return false;
    return true;
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Warp kConsumers of the CTA (thread kThreads on) issues the copies; warps 0 ..
// kConsumers - 1 certify, one query per thread. A stage is refilled when its consumer
// warps have each arrived on its `empty` mbarrier, so no warp waits for the others
// between tiles.
constexpr int kConsumers = kThreads / 32;
constexpr int kTmaThreads = kThreads + 32;

// fail_at >= 0 (tests): consumer warp 0 of CTA 0 takes its wait for tile fail_at as
// having run out, which drives the abort, the drain and the host's rerun without a
// wait that really runs out.
template <int NPT>
__global__ void __launch_bounds__(kTmaThreads) k_pred_fp32_tma(Soa s, int64_t ntiles,
                                                               int8_t* __restrict__ out, Seg L,
                                                               unsigned long long* __restrict__ fault,
                                                               unsigned long long* __restrict__ drain_fault,
                                                               int64_t fail_at) {
    using T = Tma<NPT>;
    constexpr int C = T::kCols, S = T::kStages;
    extern __shared__ __align__(128) unsigned char smem[];
    double* buf = reinterpret_cast<double*>(smem);  // [S][C][kTile]
    __shared__ __align__(8) unsigned long long full[S], empty[S];
    __shared__ unsigned long long s_cnt;  // entries of this CTA's segment so far
    __shared__ long long s_last[S];       // the last tile issued into each stage (-1: none)
    __shared__ int s_abort;               // a wait ran out: every warp stops
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, b = blockIdx.x;
    const int64_t K = ntiles > b ? (ntiles - 1 - b) / gridDim.x + 1 : 0;
    int64_t* seg = L.list + static_cast<int64_t>(b) * L.segcap;
    const int64_t cbase = static_cast<int64_t>(b) * L.ccap;
    if (tid == 0) {
        s_cnt = 0;
        s_abort = 0;
        for (int st = 0; st < S; ++st) {
            mbar_init(&full[st], 1);
            mbar_init(&empty[st], kConsumers);
            s_last[st] = -1;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (warp == kConsumers) {
        if (lane == 0) {
            for (int64_t k = 0; k < K; ++k) {
                const int st = static_cast<int>(k % S);
                // tile k - S has been read by every consumer warp (its phase of `empty`)
                if (k >= S &&
                    !mbar_wait_or_abort(&empty[st], static_cast<unsigned>((k / S - 1) & 1), &s_abort)) {
                    if (atomicExch(&s_abort, 1) == 0) atomicExch(fault, 1ull);
                    break;
                }
                // the copy into the stage follows the consumers' generic reads of it
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                const int64_t tile = b + k * gridDim.x;
                mbar_expect_tx(&full[st], T::kStageBytes);
#pragma unroll
                for (int c = 0; c < C; ++c)
                    bulk_copy(buf + (static_cast<size_t>(st) * C + c) * kTile, s.c[c] + tile * kTile,
                              kTile * 8u, &full[st]);
                s_last[st] = k;
            }
        }
    } else {
        for (int64_t k = 0; k < K; ++k) {
            const int st = static_cast<int>(k % S);
            const bool ok =
                __all_sync(0xffffffffu,
                           mbar_wait_or_abort(&full[st], static_cast<unsigned>((k / S) & 1), &s_abort) &&
                               !(b == 0 && warp == 0 && k == fail_at));
            if (!ok) {
                if (lane == 0 && atomicExch(&s_abort, 1) == 0) atomicExch(fault, 1ull);
                break;
            }
            const int64_t i = (b + k * gridDim.x) * kTile + tid;
            const double* sb = buf + static_cast<size_t>(st) * C * kTile;
            int sg;
            {
                double v[C];
#pragma unroll
                for (int c = 0; c < C; ++c) v[c] = sb[c * kTile + tid];
                sg = NPT == 4 ? o3d_fp32(v) : isp_fp32(v);
                out[i] = static_cast<int8_t>(sg);
            }
            // a query left goes to this CTA's segment, and its coordinates, read again
            // from the stage (still held; reading them again keeps the values out of
            // registers across the append), to the segment's compact slots
            const int64_t pos = seg_pos(sg == 0, &s_cnt);
            if (pos >= 0) {
                seg[pos] = i;
                if (pos < L.ccap) {
                    const volatile double* vb = sb;
#pragma unroll
                    for (int c = 0; c < C; ++c) L.cc[c][cbase + pos] = vb[c * kTile + tid];
                }
            }
            // this warp is done with the stage
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
        }
    }
    __syncthreads();
    if (s_abort) {
        // a wait ran out: drain the last copy issued into each stage (bounded), then stop
        if (tid == 0) {
            bool drained = true;
            for (int st = 0; st < S; ++st)
                if (s_last[st] >= 0)
                    drained = mbar_wait(&full[st], static_cast<unsigned>((s_last[st] / S) & 1)) && drained;
            if (!drained) atomicExch(drain_fault, 1ull);
        }
        return;
    }
    if (tid == 0) L.cnt[b] = s_cnt;
}

// Exclusive prefix of the segment counts into pre[0..nseg] (pre[nseg] = the total), by
// the whole CTA (kThreads threads, at most kMaxSeg segments).
__device__ __forceinline__ void seg_prefix(const Seg& L, unsigned long long* pre) {
    constexpr int kPer = kMaxSeg / kThreads;
    __shared__ unsigned long long s_w[kThreads / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned long long loc[kPer], sum = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const int b = tid * kPer + j;
        loc[j] = b < L.nseg ? L.cnt[b] : 0ull;
        sum += loc[j];
    }
    unsigned long long x = sum;  // inclusive scan over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    unsigned long long before = x - sum;
    for (int w = 0; w < warp; ++w) before += s_w[w];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const int b = tid * kPer + j;
        if (b <= L.nseg) pre[b] = before;
        before += loc[j];
    }
    __syncthreads();
}

// The FP64 pass over the segmented list of the FP32 pass (list position k counts
// through the segments in order); writes the list's length to *n32.
template <int NPT, int MODE>
__global__ void __launch_bounds__(kThreads) k_pred_fp64(Soa s, Seg L,
                                                        unsigned long long* __restrict__ n32,
                                                        int8_t* __restrict__ out,
                                                        int64_t* __restrict__ list,
                                                        unsigned long long* __restrict__ count,
                                                        unsigned long long* __restrict__ ncert) {
    __shared__ unsigned long long s_pre[kMaxSeg + 1];
    seg_prefix(L, s_pre);
    const int64_t n = static_cast<int64_t>(s_pre[L.nseg]);
    if (blockIdx.x == 0 && threadIdx.x == 0) *n32 = static_cast<unsigned long long>(n);
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const int64_t n_round = (n + 31) & ~int64_t(31);
    for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < n_round;
         k += stride) {
        bool undecided = false, certified = false;
        int64_t i = 0;
        if (k < n) {
            // the segment holding position k: the last with pre[b] <= k
            int lo = 0, hi = L.nseg - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_pre[mid] <= static_cast<unsigned long long>(k)) lo = mid;
                else hi = mid - 1;
            }
            const int64_t j = k - static_cast<int64_t>(s_pre[lo]);
            i = L.list[static_cast<int64_t>(lo) * L.segcap + j];
            double v[3 * NPT];
            if (j < L.ccap) {
#pragma unroll
                for (int c = 0; c < 3 * NPT; ++c) v[c] = L.cc[c][static_cast<int64_t>(lo) * L.ccap + j];
            } else {
                load_query<NPT>(s, i, v);
            }
            const d3 a{v[0], v[1], v[2]}, b{v[3], v[4], v[5]}, c{v[6], v[7], v[8]}, d{v[9], v[10], v[11]};
            // integer coordinates first (integer pipe): in EXACT mode their sign decides;
            // in COMPAT mode too when the FP64 evaluation is provably exact there (it then
            // equals the exact determinant), which spares the narrow FP64 pipe
            int isg = 0;
            bool ic = false;
            {
                const d3 e5{NPT == 5 ? v[12] : 0.0, NPT == 5 ? v[13] : 0.0, NPT == 5 ? v[14] : 0.0};
                bool fexact = false;
                ic = NPT == 4 ? exact::orient3d_int_exact64(a, b, c, d, &isg, &fexact)
                              : exact::insphere_int_exact64(a, b, c, d, e5, &isg, &fexact);
                if (ic && (MODE == kPredExact || fexact)) {
                    out[i] = static_cast<int8_t>(isg);
                    certified = true;
                }
            }
            double perm = 0.0, det = 0.0;
            if (certified) {
            } else if (NPT == 4) {
                det = o3d_fast(a, b, c, d, MODE == kPredExact ? &perm : nullptr);
                perm *= kO3dErrA;
            } else {
                const d3 e{v[12], v[13], v[14]};
                det = isp_fast(a, b, c, d, e, MODE == kPredExact ? &perm : nullptr);
                perm *= kIspErrA;
            }
            bool decided = certified || (MODE == kPredCompat ? det != 0.0 : (det > perm || -det > perm));
            if (certified) {
            } else if (decided) {
                out[i] = static_cast<int8_t>(sgn(det));
            } else {
                // integer coordinates after a common power-of-two scaling gave the
                // exact determinant on the integer pipe above; else an FP64 evaluation
                // in which no operation rounded is the exact determinant
                const d3 e{NPT == 5 ? v[12] : 0.0, NPT == 5 ? v[13] : 0.0, NPT == 5 ? v[14] : 0.0};
                if (ic) {
                    out[i] = static_cast<int8_t>(isg);
                    decided = certified = true;
                } else {
                    double ex;
                    const bool cert = NPT == 4 ? exact::orient3d_certified(a, b, c, d, &ex)
                                               : exact::insphere_certified(a, b, c, d, e, &ex);
                    if (cert) {
                        out[i] = static_cast<int8_t>(sgn(ex));
                        decided = certified = true;
                    }
                }
            }
            undecided = !decided;
        }
        const unsigned cm = __ballot_sync(0xffffffffu, certified);
        if (cm && (threadIdx.x & 31) == 0) atomicAdd(ncert, static_cast<unsigned long long>(__popc(cm)));
        push(undecided, i, list, count);
    }
}

template <int NPT>
__global__ void __launch_bounds__(128) k_pred_exact(Soa s, const int64_t* __restrict__ in,
                                                    const unsigned long long* __restrict__ nin,
                                                    int8_t* __restrict__ out,
                                                    unsigned long long* __restrict__ overflow) {
    const int64_t n = static_cast<int64_t>(*nin);
    for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
         k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t i = in[k];
        double v[3 * NPT];
        load_query<NPT>(s, i, v);
        const d3 a{v[0], v[1], v[2]}, b{v[3], v[4], v[5]}, c{v[6], v[7], v[8]}, d{v[9], v[10], v[11]};
        int sg;
        if (NPT == 4) {
            sg = exact::orient3d_sign(a, b, c, d);
        } else {
            int of = 0;
            sg = exact::insphere_sign(a, b, c, d, {v[12], v[13], v[14]}, &of);
            if (of) atomicAdd(overflow, 1ull);
        }
        out[i] = static_cast<int8_t>(sg);
    }
}

// Gathers (xyz, tets) index-form queries into SoA for the stream kernels.
__global__ void k_gather_tets(const double* __restrict__ xyz, const int* __restrict__ tets, int64_t n,
                              double* __restrict__ soa) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int p = 0; p < 4; ++p) {
        const int64_t v = tets[4 * i + p];
        for (int a = 0; a < 3; ++a) soa[(3 * p + a) * n + i] = xyz[3 * v + a];
    }
}

__global__ void k_widen(const int8_t* __restrict__ s, int64_t n, int* __restrict__ out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = s[i];
}

// Device workspace for the stream (grows, kept per device).
struct PredWork {
    Arena arena;
    std::mutex mu;
    cudaEvent_t ev[2] = {nullptr, nullptr};  // around the FP32 pass of the last stream
    // host-resident streams: the copy stream, buffer-set events and per-chunk FP32
    // pass events
    cudaStream_t copy = nullptr;
    cudaEvent_t in[2] = {nullptr, nullptr}, done[2] = {nullptr, nullptr};
    std::vector<cudaEvent_t> chunk_ev;
    int pull = -1;  // the device reads pageable host memory (-1: not asked yet)
};
PredWork& pred_work() {
    static PredWork w[64];
    int dev = 0;
    CMG_CUDA(cudaGetDevice(&dev));
    return w[dev & 63];
}

// One-shot test knob: the next TMA-staged FP32 pass takes its wait for this tile (of
// CTA 0, warp 0) as having run out; -1 = off.
std::atomic<long long> g_fail_wait_at{-1};

struct Counters {
    unsigned long long n32;  // left by the FP32 pass
    unsigned long long n64;  // left by the FP64 pass
    unsigned long long overflow;
    unsigned long long certified;  // decided in the FP64 pass by an exact evaluation
    unsigned long long fault;      // a TMA wait of the FP32 pass ran out
    unsigned long long drain_fault;  // ... and so did the drain of the copies in flight
    unsigned long long seg[kMaxSeg];  // entries per segment of the FP32 pass's list
};

// The segmented list for streams (or chunks) of at most nmax queries: at most `per_sm`
// segments (CTAs of the FP32 pass) per SM, at most one per tile; each segment holds
// every query of its tiles, and compact slots for a quarter of them (uniform queries
// leave about a tenth to the FP64 pass; beyond the slots it gathers by index).
Seg take_seg(Arena& a, int64_t nmax, int ncol, int sms, int per_sm) {
    const int64_t tiles = std::max<int64_t>(1, (nmax + kTile - 1) / kTile);
    Seg L{};
    L.nseg = static_cast<int>(std::min<int64_t>({tiles, static_cast<int64_t>(per_sm) * sms,
                                                  static_cast<int64_t>(kMaxSeg - 1)}));
    L.segcap = (tiles + L.nseg - 1) / L.nseg * kTile;
    L.ccap = std::min<int64_t>(L.segcap, L.segcap / 4 + 64);
    L.list = a.take<int64_t>(L.nseg * L.segcap);
    for (int k = 0; k < ncol; ++k) L.cc[k] = a.take<double>(L.nseg * L.ccap);
    return L;
}

// Queries per chunk of a host-resident stream (two buffer sets of up to 15 columns:
// at most 1 GB of device memory).
constexpr int64_t kHostChunk = int64_t{1} << 22;
// Queries per chunk when the device reads host memory itself (one set of device
// columns: at most 2 GB).
constexpr int64_t kPullChunk = int64_t{1} << 24;

}  // namespace

// The FP64 pass over the queries the FP32 pass left in the segments of L (their counts
// in c->seg), then the exact pass.
static void pred_stream_finish(int npt, const Soa& s, int mode, int8_t* d_out, Seg L,
                               int64_t* list_b, Counters* c, cudaStream_t st, int sms) {
    L.cnt = c->seg;
    if (npt == 4 && mode == kPredExact)
        k_pred_fp64<4, kPredExact><<<2 * sms, kThreads, 0, st>>>(s, L, &c->n32, d_out, list_b, &c->n64,
                                                                      &c->certified);
    else if (npt == 4)
        k_pred_fp64<4, kPredCompat><<<2 * sms, kThreads, 0, st>>>(s, L, &c->n32, d_out, list_b, &c->n64,
                                                                      &c->certified);
    else if (mode == kPredExact)
        k_pred_fp64<5, kPredExact><<<2 * sms, kThreads, 0, st>>>(s, L, &c->n32, d_out, list_b, &c->n64,
                                                                      &c->certified);
    else
        k_pred_fp64<5, kPredCompat><<<2 * sms, kThreads, 0, st>>>(s, L, &c->n32, d_out, list_b, &c->n64,
                                                                      &c->certified);
    CMG_LAUNCH();
    if (npt == 4) k_pred_exact<4><<<2 * sms, 128, 0, st>>>(s, list_b, &c->n64, d_out, &c->overflow);
    else k_pred_exact<5><<<2 * sms, 128, 0, st>>>(s, list_b, &c->n64, d_out, &c->overflow);
    CMG_LAUNCH();
}

// The FP32 pass with per-thread loads over tiles [t0, t1) into the segments of L.
static void pred_fp32_loads(int npt, const Soa& s, int64_t t0, int64_t t1, int64_t n, int8_t* d_out,
                            const Seg& L, cudaStream_t st) {
    if (npt == 4) k_pred_fp32_seg<4, false><<<L.nseg, kThreads, 0, st>>>(s, s, t0, t1, n, d_out, L);
    else k_pred_fp32_seg<5, false><<<L.nseg, kThreads, 0, st>>>(s, s, t0, t1, n, d_out, L);
    CMG_LAUNCH();
}

// Runs the three passes on device-resident SoA coordinates, the FP32 pass's list in
// the segments of L (shaped for at least n queries). Returns the number of times the
// FP32 pass was rerun with per-thread loads after a TMA wait ran out (0 or 1); throws
// when copies may have outlived their CTA.
int pred_stream_device(int npt, const double* const* coords, int64_t n, int mode, int8_t* d_out,
                        Seg L, int64_t* list_b, void* counters, cudaStream_t st, int sms,
                        cudaEvent_t* fp32_events) {
    Soa s{};
    for (int k = 0; k < 3 * npt; ++k) s.c[k] = coords[k];
    Counters* c = static_cast<Counters*>(counters);
    L.cnt = c->seg;
    const int64_t T = (n + kTile - 1) / kTile;
    if ((T + L.nseg - 1) / L.nseg > L.segcap / kTile)
        throw std::logic_error("predicate stream: list segments too small for the stream");
    CMG_CUDA(cudaMemsetAsync(c, 0, sizeof(Counters), st));
    // the TMA pass takes the whole tiles when every column starts on a 16-byte boundary
    // (the bulk copies' rule); the rest, and unaligned columns, take the per-thread loads
    bool aligned = true;
    for (int k = 0; k < 3 * npt; ++k) aligned = aligned && (reinterpret_cast<uintptr_t>(coords[k]) % 16 == 0);
    const int64_t ntiles = aligned ? n / kTile : 0;
    if (fp32_events) CMG_CUDA(cudaEventRecord(fp32_events[0], st));
    if (ntiles > 0) {
        const int64_t fail_at = g_fail_wait_at.exchange(-1);
        if (npt == 4) {
            CMG_CUDA(cudaFuncSetAttribute(k_pred_fp32_tma<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(Tma<4>::kSmem)));
            k_pred_fp32_tma<4><<<L.nseg, kTmaThreads, Tma<4>::kSmem, st>>>(s, ntiles, d_out, L, &c->fault,
                                                                           &c->drain_fault, fail_at);
        } else {
            CMG_CUDA(cudaFuncSetAttribute(k_pred_fp32_tma<5>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(Tma<5>::kSmem)));
            k_pred_fp32_tma<5><<<L.nseg, kTmaThreads, Tma<5>::kSmem, st>>>(s, ntiles, d_out, L, &c->fault,
                                                                           &c->drain_fault, fail_at);
        }
        CMG_LAUNCH();
    }
    if (ntiles < T) pred_fp32_loads(npt, s, ntiles, T, n, d_out, L, st);
    if (fp32_events) CMG_CUDA(cudaEventRecord(fp32_events[1], st));
    int reruns = 0;
    if (ntiles > 0) {
        // a TMA wait that ran out (it never should) reruns the pass with per-thread loads,
        // unless the copies in flight could not be drained either
        unsigned long long fault[2] = {0, 0};
        CMG_CUDA(cudaMemcpyAsync(fault, &c->fault, sizeof(fault), cudaMemcpyDeviceToHost, st));
        CMG_CUDA(cudaStreamSynchronize(st));
        if (fault[1])
            throw std::runtime_error(
                "predicate stream: a bulk copy of the FP32 pass did not complete within its wait");
        if (fault[0]) {
            CMG_CUDA(cudaMemsetAsync(c, 0, sizeof(Counters), st));
            pred_fp32_loads(npt, s, 0, T, n, d_out, L, st);
            reruns = 1;
        }
    }
    pred_stream_finish(npt, s, mode, d_out, L, list_b, c, st, sms);
    return reruns;
}

}  // namespace cmg::gpu

namespace {

void set_err(char* buf, size_t len, const std::string& msg) {
    if (buf && len) {
        std::strncpy(buf, msg.c_str(), len - 1);
        buf[len - 1] = '\0';
    }
}

// Whether host-resident streams are read by the device directly: when the device
// accesses pageable host memory (cudaDevAttrPageableMemoryAccess), unless the
// environment variable CMG_HOST_STREAM is "copy" (copy calls through two device
// buffer sets instead; "pull" or unset: direct when supported).
bool use_pull(cmg::gpu::PredWork& w) {
    if (w.pull < 0) {
        int dev = 0, v = 0;
        CMG_CUDA(cudaGetDevice(&dev));
        CMG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev));
        w.pull = v ? 1 : 0;
    }
    const char* e = std::getenv("CMG_HOST_STREAM");
    if (e && std::strcmp(e, "copy") == 0) return false;
    return w.pull == 1;
}

cmg_status run_stream(int npt, const double* const* coords, int64_t n, int mode, int where,
                      signed char* out, cmg_pred_stats* stats, void* stream, char* errbuf,
                      size_t len) {
    using namespace cmg::gpu;
    if (!coords || !out || n < 0) return CMG_ERR_INVALID_INPUT;
    if (mode != CMG_PRED_COMPAT && mode != CMG_PRED_EXACT) {
        set_err(errbuf, len, "predicate mode must be CMG_PRED_COMPAT or CMG_PRED_EXACT");
        return CMG_ERR_UNSUPPORTED_OPTION;
    }
    if (where != CMG_MEM_HOST && where != CMG_MEM_DEVICE) {
        set_err(errbuf, len, "where must be CMG_MEM_HOST or CMG_MEM_DEVICE");
        return CMG_ERR_INVALID_INPUT;
    }
    for (int k = 0; k < 3 * npt; ++k)
        if (!coords[k] && n) return CMG_ERR_INVALID_INPUT;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (n == 0) return CMG_OK;
    try {
        PredWork& w = pred_work();
        std::lock_guard<std::mutex> lk(w.mu);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const int sms = device_sms();
        const bool host = where == CMG_MEM_HOST;
        auto plan = [&](Arena& a, Seg* la, int64_t** lb, void** cnt) {
            a.reset();
            *la = take_seg(a, n, 3 * npt, sms, 2);
            *lb = a.take<int64_t>(n);
            *cnt = a.take<Counters>(1);
        };
        if (!w.ev[0])
            for (cudaEvent_t& e : w.ev) CMG_CUDA(cudaEventCreate(&e));
        const int ncol = 3 * npt;
        Counters hc{};
        int reruns = 0;
        if (!host) {
            Seg la;
            int64_t* lb;
            void* cnt;
            w.arena.clear_need();
            plan(w.arena, &la, &lb, &cnt);
            if (w.arena.overflowed()) {
                w.arena.reserve(w.arena.need());
                plan(w.arena, &la, &lb, &cnt);
            }
            reruns += pred_stream_device(npt, coords, n, mode == CMG_PRED_EXACT ? kPredExact : kPredCompat,
                                         reinterpret_cast<int8_t*>(out), la, lb, cnt, st, sms, w.ev);
            CMG_CUDA(cudaMemcpyAsync(&hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
            CMG_CUDA(cudaStreamSynchronize(st));
            if (stats) CMG_CUDA(cudaEventElapsedTime(&stats->fp32_pass_ms, w.ev[0], w.ev[1]));
        } else if (use_pull(w)) {
            // Host arrays read by the device through the host's page tables (the GPU
            // and CPU share them over the coherent link): no copy calls. Per chunk the
            // FP32 pass pulls each query over the link once and stores it to device
            // columns for the FP64 and exact passes; the device writes the signs back.
            const int64_t chunk = std::min<int64_t>(n, kPullChunk);
            const int64_t nch = (n + chunk - 1) / chunk;
            double* col[15];
            int8_t* sg;
            Seg la;
            int64_t* lb;
            Counters* cnt;
            auto plan_pull = [&](Arena& a) {
                a.reset();
                for (int k = 0; k < ncol; ++k) col[k] = a.take<double>(chunk);
                sg = a.take<int8_t>(chunk);
                la = take_seg(a, chunk, ncol, sms, 4);  // 4 resident CTAs per SM
                lb = a.take<int64_t>(chunk);
                cnt = a.take<Counters>(nch);
            };
            w.arena.clear_need();
            plan_pull(w.arena);
            if (w.arena.overflowed()) {
                w.arena.reserve(w.arena.need());
                plan_pull(w.arena);
            }
            while (w.chunk_ev.size() < static_cast<size_t>(2 * nch)) {
                cudaEvent_t e;
                CMG_CUDA(cudaEventCreate(&e));
                w.chunk_ev.push_back(e);
            }
            CMG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(Counters) * nch, st));
            for (int64_t c = 0; c < nch; ++c) {
                const int64_t i0 = c * chunk, m = std::min(chunk, n - i0);
                Soa src{}, dst{};
                for (int k = 0; k < ncol; ++k) {
                    src.c[k] = coords[k] + i0;
                    dst.c[k] = col[k];
                }
                CMG_CUDA(cudaEventRecord(w.chunk_ev[2 * c], st));
                Seg lc = la;
                lc.cnt = cnt[c].seg;
                const int64_t T = (m + kTile - 1) / kTile;
                if (npt == 4)
                    k_pred_fp32_seg<4, true><<<lc.nseg, kThreads, 0, st>>>(src, dst, 0, T, m, sg, lc);
                else
                    k_pred_fp32_seg<5, true><<<lc.nseg, kThreads, 0, st>>>(src, dst, 0, T, m, sg, lc);
                CMG_LAUNCH();
                CMG_CUDA(cudaEventRecord(w.chunk_ev[2 * c + 1], st));
                pred_stream_finish(npt, dst, mode == CMG_PRED_EXACT ? kPredExact : kPredCompat, sg, la,
                                   lb, cnt + c, st, sms);
                k_put_bytes<<<4 * sms, 256, 0, st>>>(sg, reinterpret_cast<int8_t*>(out) + i0, m);
                CMG_LAUNCH();
            }
            std::vector<Counters> hcs(static_cast<size_t>(nch));
            CMG_CUDA(cudaMemcpyAsync(hcs.data(), cnt, sizeof(Counters) * nch, cudaMemcpyDeviceToHost, st));
            CMG_CUDA(cudaStreamSynchronize(st));
            float total = 0.f;
            for (int64_t c = 0; c < nch; ++c) {
                hc.n32 += hcs[c].n32;
                hc.n64 += hcs[c].n64;
                hc.certified += hcs[c].certified;
                hc.overflow |= hcs[c].overflow;
                float ms = 0.f;
                CMG_CUDA(cudaEventElapsedTime(&ms, w.chunk_ev[2 * c], w.chunk_ev[2 * c + 1]));
                total += ms;
            }
            if (stats) stats->fp32_pass_ms = total;
        } else {
            // Host arrays: chunks through two device buffer sets. The copy stream
            // uploads chunk c+1 while the launch stream certifies chunk c and
            // downloads its signs; the link, not the certification, sets the pace.
            const int64_t chunk = std::min<int64_t>(n, kHostChunk);
            const int64_t nch = (n + chunk - 1) / chunk;
            double* col[2][15];
            int8_t* sg[2];
            Seg la;
            int64_t* lb;
            Counters* cnt;
            auto plan_host = [&](Arena& a) {
                a.reset();
                for (int b = 0; b < 2; ++b) {
                    for (int k = 0; k < ncol; ++k) col[b][k] = a.take<double>(chunk);
                    sg[b] = a.take<int8_t>(chunk);
                }
                la = take_seg(a, chunk, ncol, sms, 2);
                lb = a.take<int64_t>(chunk);
                cnt = a.take<Counters>(nch);
            };
            w.arena.clear_need();
            plan_host(w.arena);
            if (w.arena.overflowed()) {
                w.arena.reserve(w.arena.need());
                plan_host(w.arena);
            }
            if (!w.copy) {
                CMG_CUDA(cudaStreamCreateWithFlags(&w.copy, cudaStreamNonBlocking));
                for (int b = 0; b < 2; ++b) {
                    CMG_CUDA(cudaEventCreateWithFlags(&w.in[b], cudaEventDisableTiming));
                    CMG_CUDA(cudaEventCreateWithFlags(&w.done[b], cudaEventDisableTiming));
                }
            }
            while (w.chunk_ev.size() < static_cast<size_t>(2 * nch)) {
                cudaEvent_t e;
                CMG_CUDA(cudaEventCreate(&e));
                w.chunk_ev.push_back(e);
            }
            // the launch stream's earlier work comes before the first upload
            CMG_CUDA(cudaEventRecord(w.done[1], st));
            CMG_CUDA(cudaStreamWaitEvent(w.copy, w.done[1], 0));
            auto upload = [&](int64_t c) {
                const int b = static_cast<int>(c & 1);
                const int64_t i0 = c * chunk, m = std::min(chunk, n - i0);
                if (c >= 2) CMG_CUDA(cudaStreamWaitEvent(w.copy, w.done[b], 0));
                for (int k = 0; k < ncol; ++k)
                    CMG_CUDA(cudaMemcpyAsync(col[b][k], coords[k] + i0, sizeof(double) * m,
                                             cudaMemcpyHostToDevice, w.copy));
                CMG_CUDA(cudaEventRecord(w.in[b], w.copy));
            };
            upload(0);
            for (int64_t c = 0; c < nch; ++c) {
                const int b = static_cast<int>(c & 1);
                const int64_t i0 = c * chunk, m = std::min(chunk, n - i0);
                CMG_CUDA(cudaStreamWaitEvent(st, w.in[b], 0));
                if (c + 1 < nch) upload(c + 1);
                const double* dc[15];
                for (int k = 0; k < ncol; ++k) dc[k] = col[b][k];
                reruns += pred_stream_device(npt, dc, m, mode == CMG_PRED_EXACT ? kPredExact : kPredCompat,
                                   sg[b], la, lb, cnt + c, st, sms, &w.chunk_ev[2 * c]);
                CMG_CUDA(cudaMemcpyAsync(out + i0, sg[b], m, cudaMemcpyDeviceToHost, st));
                CMG_CUDA(cudaEventRecord(w.done[b], st));
            }
            std::vector<Counters> hcs(static_cast<size_t>(nch));
            CMG_CUDA(cudaMemcpyAsync(hcs.data(), cnt, sizeof(Counters) * nch, cudaMemcpyDeviceToHost, st));
            CMG_CUDA(cudaStreamSynchronize(st));
            float total = 0.f;
            for (int64_t c = 0; c < nch; ++c) {
                hc.n32 += hcs[c].n32;
                hc.n64 += hcs[c].n64;
                hc.certified += hcs[c].certified;
                hc.overflow |= hcs[c].overflow;
                float ms = 0.f;
                CMG_CUDA(cudaEventElapsedTime(&ms, w.chunk_ev[2 * c], w.chunk_ev[2 * c + 1]));
                total += ms;
            }
            if (stats) stats->fp32_pass_ms = total;
        }
        if (stats) {
            stats->queries = n;
            stats->fp64_queries = static_cast<int64_t>(hc.n32);
            stats->exact_queries = static_cast<int64_t>(hc.n64 + hc.certified);
            stats->expansion_queries = static_cast<int64_t>(hc.n64);
            stats->tma_reruns = reruns;
        }
        if (hc.overflow) {
            set_err(errbuf, len, "insphere: exact expansion exceeded its capacity");
            return CMG_ERR_INTERNAL;
        }
        return CMG_OK;
    } catch (const std::exception& e) {
        set_err(errbuf, len, e.what());
        return CMG_ERR_INTERNAL;
    }
}

}  // namespace

extern "C" {

cmg_status cmg_orient3d_stream(const double* const* coords, int64_t n, int mode, int where,
                               signed char* out, cmg_pred_stats* stats, void* stream, char* errbuf,
                               size_t errbuf_len) {
    return run_stream(4, coords, n, mode, where, out, stats, stream, errbuf, errbuf_len);
}

cmg_status cmg_insphere_stream(const double* const* coords, int64_t n, int mode, int where,
                               signed char* out, cmg_pred_stats* stats, void* stream, char* errbuf,
                               size_t errbuf_len) {
    return run_stream(5, coords, n, mode, where, out, stats, stream, errbuf, errbuf_len);
}

cmg_status cmg_debug_fail_pred_wait(int64_t tile) {
    if (tile < -1) return CMG_ERR_INVALID_INPUT;
    cmg::gpu::g_fail_wait_at.store(tile);
    return CMG_OK;
}

cmg_status cmg_orient3d_signs(const double* xyz, int npts, const int* tets, int n, int* out_sign) {
    using namespace cmg::gpu;
    if (n <= 0) return CMG_OK;
    if (!xyz || !tets || !out_sign || npts <= 0) return CMG_ERR_INVALID_INPUT;
    for (int i = 0; i < 4 * n; ++i)
        if (tets[i] < 0 || tets[i] >= npts) return CMG_ERR_INVALID_INPUT;
    try {
        PredWork& w = pred_work();
        std::lock_guard<std::mutex> lk(w.mu);
        cudaStream_t st = nullptr;
        const int64_t N = n;
        const int sms = device_sms();
        auto plan = [&](Arena& a, double** dx, int** dt, double** soa, int8_t** d8, int** dsg,
                        Seg* la, int64_t** lb, void** cnt) {
            a.reset();
            *dx = a.take<double>(3 * static_cast<size_t>(npts));
            *dt = a.take<int>(4 * N);
            *soa = a.take<double>(12 * N);
            *d8 = a.take<int8_t>(N);
            *dsg = a.take<int>(N);
            *la = take_seg(a, N, 12, sms, 2);
            *lb = a.take<int64_t>(N);
            *cnt = a.take<Counters>(1);
        };
        double *dx, *soa;
        int *dt, *dsg;
        int8_t* d8;
        Seg la;
        int64_t* lb;
        void* cnt;
        w.arena.clear_need();
        plan(w.arena, &dx, &dt, &soa, &d8, &dsg, &la, &lb, &cnt);
        if (w.arena.overflowed()) {
            w.arena.reserve(w.arena.need());
            plan(w.arena, &dx, &dt, &soa, &d8, &dsg, &la, &lb, &cnt);
        }
        CMG_CUDA(cudaMemcpyAsync(dx, xyz, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice, st));
        CMG_CUDA(cudaMemcpyAsync(dt, tets, sizeof(int) * 4 * N, cudaMemcpyHostToDevice, st));
        k_gather_tets<<<static_cast<unsigned>((N + 255) / 256), 256, 0, st>>>(dx, dt, N, soa);
        CMG_LAUNCH();
        const double* cols[12];
        for (int k = 0; k < 12; ++k) cols[k] = soa + k * N;
        pred_stream_device(4, cols, N, kPredCompat, d8, la, lb, cnt, st, sms, nullptr);
        k_widen<<<static_cast<unsigned>((N + 255) / 256), 256, 0, st>>>(d8, N, dsg);
        CMG_LAUNCH();
        CMG_CUDA(cudaMemcpyAsync(out_sign, dsg, sizeof(int) * N, cudaMemcpyDeviceToHost, st));
        CMG_CUDA(cudaStreamSynchronize(st));
        return CMG_OK;
    } catch (const std::exception&) {
        return CMG_ERR_INTERNAL;
    }
}

}  // extern "C"
