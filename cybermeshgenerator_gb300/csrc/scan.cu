// scan.cu — exclusive prefix sums (counts -> offsets) and a stable LSD radix sort.
//
// Both are deterministic: integer arithmetic only, and the radix sort ranks
// equal keys by their input position.
#include <cuda_runtime.h>

#include <cstdint>

#include "cmg_util.h"

namespace cmg::gpu {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename T>
__device__ int64_t block_exclusive(int64_t v, int64_t* sh, int64_t* total) {
    // Hillis-Steele over a warp then across warps (blockDim == kScanThreads).
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < kScanThreads / 32 ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanThreads / 32) sh[lane] = w;
    }
    __syncthreads();
    int64_t before = (warp > 0 ? sh[warp - 1] : 0) + x - v;
    if (total) *total = sh[kScanThreads / 32 - 1];
    __syncthreads();
    return before;
}

template <typename T>
__global__ void __launch_bounds__(kScanThreads) k_tile_sums(const T* __restrict__ in, int64_t n,
                                                            int64_t* __restrict__ sums) {
    __shared__ int64_t sh[kScanThreads / 32];
    int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) s += static_cast<int64_t>(in[base + i]);
    int64_t total;
    block_exclusive<T>(s, sh, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One block scans the tile sums in place (exclusive), looping over chunks.
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int64_t* __restrict__ sums, int64_t m) {
    __shared__ int64_t sh[kScanThreads / 32];
    int64_t carry = 0;
    for (int64_t base = 0; base < m; base += kScanThreads) {
        int64_t i = base + threadIdx.x;
        int64_t v = i < m ? sums[i] : 0;
        int64_t total;
        int64_t ex = block_exclusive<int64_t>(v, sh, &total);
        if (i < m) sums[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) sums[m] = carry;
}

template <typename T>
__global__ void __launch_bounds__(kScanThreads) k_tile_scan(const T* __restrict__ in, int64_t n,
                                                            const int64_t* __restrict__ sums,
                                                            int64_t* __restrict__ out) {
    __shared__ int64_t sh[kScanThreads / 32];
    int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? static_cast<int64_t>(in[base + i]) : 0;
        s += v[i];
    }
    int64_t before = block_exclusive<T>(s, sh, nullptr) + sums[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = before;
        before += v[i];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = sums[gridDim.x];
}

template <typename T>
void exclusive_scan_impl(const T* in, int64_t* out, int64_t n, int64_t* tmp, cudaStream_t st) {
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 0) {
        cudaMemsetAsync(out, 0, sizeof(int64_t), st);
        return;
    }
    k_tile_sums<T><<<static_cast<unsigned>(tiles), kScanThreads, 0, st>>>(in, n, tmp);
    k_scan_sums<<<1, kScanThreads, 0, st>>>(tmp, tiles);
    k_tile_scan<T><<<static_cast<unsigned>(tiles), kScanThreads, 0, st>>>(in, n, tmp, out);
    note_launch(2);
    CMG_LAUNCH();
}

// ------------------------------------------------------------------ radix sort
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;  // keys per tile
constexpr int kRadix = 256;

// Per tile digit histogram: hist[digit * ntiles + tile] (digit-major, so one
// exclusive scan of the whole array gives every (digit, tile) its global start).
__global__ void __launch_bounds__(kSortThreads) k_digit_hist(const uint32_t* __restrict__ keys,
                                                             int64_t n, int shift, int64_t ntiles,
                                                             int* __restrict__ hist) {
    __shared__ int h[kRadix];
    for (int i = threadIdx.x; i < kRadix; i += kSortThreads) h[i] = 0;
    __syncthreads();
    int64_t base = static_cast<int64_t>(blockIdx.x) * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += kSortThreads)
        if (base + i < n) atomicAdd(&h[(keys[base + i] >> shift) & 0xff], 1);
    __syncthreads();
    for (int i = threadIdx.x; i < kRadix; i += kSortThreads)
        hist[static_cast<int64_t>(i) * ntiles + blockIdx.x] = h[i];
}

// Stable scatter: each tile processes its keys in order, in rounds of
// kSortThreads; within a round a key's rank among equal digits comes from
// warp match masks and per-warp digit counts, so equal keys keep input order.
__global__ void __launch_bounds__(kSortThreads) k_digit_scatter(
    const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, int64_t n, int shift,
    int64_t ntiles, const int64_t* __restrict__ start, uint32_t* __restrict__ keys_out,
    uint32_t* __restrict__ vals_out) {
    __shared__ int64_t base_of[kRadix];
    __shared__ int warp_cnt[kSortThreads / 32][kRadix];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kRadix; i += kSortThreads)
        base_of[i] = start[static_cast<int64_t>(i) * ntiles + blockIdx.x];
    __syncthreads();
    int64_t tile0 = static_cast<int64_t>(blockIdx.x) * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        for (int i = threadIdx.x; i < (kSortThreads / 32) * kRadix; i += kSortThreads)
            (&warp_cnt[0][0])[i] = 0;
        __syncthreads();
        int64_t idx = tile0 + static_cast<int64_t>(r) * kSortThreads + threadIdx.x;
        bool valid = idx < n;
        uint32_t k = valid ? keys[idx] : 0u;
        int d = valid ? static_cast<int>((k >> shift) & 0xff) : -1;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank_in_warp = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank_in_warp == 0) warp_cnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            int64_t pos = base_of[d] + rank_in_warp;
            for (int w = 0; w < warp; ++w) pos += warp_cnt[w][d];
            keys_out[pos] = k;
            vals_out[pos] = vals[idx];
        }
        __syncthreads();
        // advance the per-digit bases by this round's totals
        for (int i = threadIdx.x; i < kRadix; i += kSortThreads) {
            int s = 0;
            for (int w = 0; w < kSortThreads / 32; ++w) s += warp_cnt[w][i];
            base_of[i] += s;
        }
        __syncthreads();
    }
}

}  // namespace

void exclusive_scan(const int* in, int64_t* out, int64_t n, int64_t* tmp, cudaStream_t st) {
    exclusive_scan_impl<int>(in, out, n, tmp, st);
}
void exclusive_scan(const int64_t* in, int64_t* out, int64_t n, int64_t* tmp, cudaStream_t st) {
    exclusive_scan_impl<int64_t>(in, out, n, tmp, st);
}
size_t scan_tmp_elems(int64_t n) { return static_cast<size_t>((n + kScanTile - 1) / kScanTile + 2); }

size_t radix_sort_tmp_bytes(int64_t n) {
    int64_t ntiles = (n + kSortTile - 1) / kSortTile;
    int64_t hn = ntiles * kRadix;
    return sizeof(uint32_t) * 2 * static_cast<size_t>(n) + sizeof(int) * static_cast<size_t>(hn) +
           sizeof(int64_t) * (static_cast<size_t>(hn) + 1) +
           sizeof(int64_t) * scan_tmp_elems(hn) + 5 * 256;  // 5 sub-buffers, 256-byte aligned
}

void radix_sort_pairs(uint32_t* keys, uint32_t* vals, int64_t n, int key_bits, void* tmp,
                      cudaStream_t st) {
    if (n <= 0) return;
    int64_t ntiles = (n + kSortTile - 1) / kSortTile;
    int64_t hn = ntiles * kRadix;
    char* p = static_cast<char*>(tmp);
    auto take = [&](size_t bytes) {
        char* q = p;
        p += (bytes + 255) & ~size_t(255);
        return q;
    };
    uint32_t* k2 = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * n));
    uint32_t* v2 = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * n));
    int* hist = reinterpret_cast<int*>(take(sizeof(int) * hn));
    int64_t* start = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * (hn + 1)));
    int64_t* stmp = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * scan_tmp_elems(hn)));
    uint32_t *ka = keys, *va = vals, *kb = k2, *vb = v2;
    int passes = (key_bits + 7) / 8;
    for (int pss = 0; pss < passes; ++pss) {
        int shift = 8 * pss;
        k_digit_hist<<<static_cast<unsigned>(ntiles), kSortThreads, 0, st>>>(ka, n, shift, ntiles, hist);
        exclusive_scan(hist, start, hn, stmp, st);
        note_launch();
        k_digit_scatter<<<static_cast<unsigned>(ntiles), kSortThreads, 0, st>>>(
            ka, va, n, shift, ntiles, start, kb, vb);
        CMG_LAUNCH();
        uint32_t* t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    if (ka != keys) {
        cudaMemcpyAsync(keys, ka, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(vals, va, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
    }
}

}  // namespace cmg::gpu
