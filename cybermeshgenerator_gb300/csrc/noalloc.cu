// noalloc.cu — occupancy of one mesh without allocating any memory.
//
// Some callers cannot call cudaMalloc: code running inside a framework that owns
// the device memory through its own pool allocator (and forbids foreign
// allocations, or must not fragment its pool), real-time loops that may not
// allocate after start-up, and plugins whose host process installs a
// fixed-budget memory policy. They hand over device buffers for the inputs and the
// output, and this entry point takes its working memory (triangle records,
// per-column buckets, the exact-pass scratch) from one fixed array in device
// global memory, declared below at file scope. Every GPU that loads this library
// holds that array until the process exits.
//
// Set-up: the first call on a device resolves the array's device address with
// cudaGetSymbolAddress, with that device current. Every call reads two sizes back from
// the device and waits for `stream` to finish before it returns (it synchronises the
// stream), so no call can be captured into a CUDA graph: on a stream being captured the
// call is rejected before any device work. Calls share the
// array and it keeps the last call's contents, so each call clears what must start at
// zero; calls that overlap on the GPU (two streams, or two host threads) race on it
// and must be serialised by the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/cmg_c/cmg_gpu.h"
#include "cmg_types.h"
#include "cmg_util.h"
#include "engine.h"
#include "engine_kernels.h"

namespace cmg::gpu {

// The working memory of cmg_gpu_occupancy_static (a stated maximum of 32 MiB).
constexpr size_t kStaticScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (resolved once).
unsigned char* scratch_base(int dev) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        CMG_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    return g_scratch_addr[dev];
}

// Sets *bad when a triangle index is outside [0, npts).
__global__ void k_check_indices(const int* __restrict__ tris, int64_t n, int64_t npts,
                                int* __restrict__ bad) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int v = tris[i];
        if (v < 0 || v >= npts) atomicExch(bad, 1);
    }
}

// Bump allocation inside the static array (256-byte aligned pieces).
struct Carver {
    unsigned char* base;
    size_t used = 0;
    template <typename T>
    T* take(size_t count) {
        size_t at = used;
        used += (sizeof(T) * (count ? count : 1) + 255) & ~size_t(255);
        return reinterpret_cast<T*>(base + at);
    }
};

void set_err(char* buf, size_t len, const char* msg) {
    if (buf && len) {
        std::strncpy(buf, msg, len - 1);
        buf[len - 1] = '\0';
    }
}

// Formats the capacity message on the stack (no heap allocation on any path).
void set_capacity_err(char* buf, size_t len, size_t need) {
    char m[192];
    std::snprintf(m, sizeof(m),
                  "cmg_gpu_occupancy_static: input exceeds the static scratch (needs %zu bytes, "
                  "maximum %zu)",
                  need, kStaticScratchBytes);
    set_err(buf, len, m);
}

}  // namespace
}  // namespace cmg::gpu

extern "C" cmg_status cmg_gpu_occupancy_static(const double* d_points, int64_t npoints,
                                               const int* d_triangles, int64_t ntriangles,
                                               const double* corner, double spacing,
                                               const int* dims, int predicates,
                                               unsigned char* d_occupancy, void* stream,
                                               char* errbuf, size_t errbuf_len) {
    using namespace cmg::gpu;
    if (!d_points || !d_triangles || !corner || !dims || !d_occupancy) {
        set_err(errbuf, errbuf_len, "cmg_gpu_occupancy_static: null pointer argument");
        return CMG_ERR_INVALID_INPUT;
    }
    if (npoints < 1 || ntriangles < 1) {
        set_err(errbuf, errbuf_len, "cmg_gpu_occupancy_static: no points or no triangles");
        return CMG_ERR_INVALID_INPUT;
    }
    if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1 || !(spacing > 0)) {
        set_err(errbuf, errbuf_len, "cmg_gpu_occupancy_static: empty grid or spacing <= 0");
        return CMG_ERR_INVALID_INPUT;
    }
    if (predicates != kPredCompat && predicates != kPredExact) {
        set_err(errbuf, errbuf_len, "cmg_gpu_occupancy_static: predicates must be 0 or 1");
        return CMG_ERR_UNSUPPORTED_OPTION;
    }
    try {
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CMG_CUDA(cudaStreamIsCapturing(st, &cs));
        if (cs != cudaStreamCaptureStatusNone) {
            set_err(errbuf, errbuf_len,
                    "cmg_gpu_occupancy_static: the call synchronises its stream, which is being captured");
            return CMG_ERR_UNSUPPORTED_OPTION;
        }
        int dev = 0;
        CMG_CUDA(cudaGetDevice(&dev));
        if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("device ordinal out of range");
        const int64_t T = ntriangles;
        const int64_t ncol = static_cast<int64_t>(dims[0]) * dims[1];
        const int rc = occ_row_cols();
        const int64_t nrows = static_cast<int64_t>(dims[1]) * ((dims[0] + rc - 1) / rc);

        // sizes known before any device work: reject what cannot fit
        Carver c{scratch_base(dev)};
        MeshSeg* segs = c.take<MeshSeg>(1);
        Stats* stats = c.take<Stats>(1);
        int* bad = c.take<int>(1);
        double* soup = c.take<double>(kSoupStride * T);
        int4* xybox = c.take<int4>(T);
        int64_t* pairs_n = c.take<int64_t>(T + 1);
        int64_t* pair_off = c.take<int64_t>(T + 1);
        int* colcnt = c.take<int>(ncol);
        int64_t* col_off = c.take<int64_t>(ncol + 1);
        int64_t* flagged = c.take<int64_t>(ncol);
        int64_t* scan_tmp = c.take<int64_t>(scan_tmp_elems(std::max(T, ncol)));
        if (c.used > kStaticScratchBytes) {  // before the buckets are sized
            set_capacity_err(errbuf, errbuf_len, c.used);
            return CMG_ERR_INVALID_INPUT;
        }

        MeshSeg s{};
        for (int a = 0; a < 3; ++a) s.g.corner[a] = corner[a];
        s.g.h = spacing;
        s.g.nx = dims[0];
        s.g.ny = dims[1];
        s.g.nz = dims[2];
        s.g.z0 = 0;  // every layer
        s.g.z1 = dims[2];
        s.tri_begin = 0;
        s.tri_end = T;
        CMG_CUDA(cudaMemcpyAsync(segs, &s, sizeof(s), cudaMemcpyHostToDevice, st));
        CMG_CUDA(cudaMemsetAsync(stats, 0, sizeof(Stats), st));
        CMG_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), st));

        // every triangle index must address a point before any kernel reads one
        k_check_indices<<<256, 256, 0, st>>>(d_triangles, 3 * T, npoints, bad);
        CMG_LAUNCH();
        int h_bad = 0;
        CMG_CUDA(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
        CMG_CUDA(cudaStreamSynchronize(st));
        if (h_bad) {
            set_err(errbuf, errbuf_len, "cmg_gpu_occupancy_static: triangle index out of range");
            return CMG_ERR_INVALID_INPUT;
        }

        launch_tri_prep(segs, 1, T, d_points, d_triangles, soup, xybox, pairs_n, st);
        exclusive_scan(pairs_n, pair_off, T, scan_tmp, st);
        int64_t P = 0;
        CMG_CUDA(cudaMemcpyAsync(&P, pair_off + T, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CMG_CUDA(cudaStreamSynchronize(st));
        int* col_list = c.take<int>(P);
        double* hs = c.take<double>(P);
        uint8_t* hv = c.take<uint8_t>(P);
        if (c.used > kStaticScratchBytes) {
            set_capacity_err(errbuf, errbuf_len, c.used);
            return CMG_ERR_INVALID_INPUT;
        }

        const int grid = 4 * device_sms();
        CMG_CUDA(cudaMemsetAsync(colcnt, 0, sizeof(int) * ncol, st));
        launch_col_pairs(false, segs, 1, T, xybox, pair_off, colcnt, nullptr, nullptr, grid, st);
        exclusive_scan(colcnt, col_off, ncol, scan_tmp, st);
        CMG_CUDA(cudaMemsetAsync(colcnt, 0, sizeof(int) * ncol, st));
        launch_col_pairs(true, segs, 1, T, xybox, pair_off, colcnt, col_off, col_list, grid, st);
        launch_occ_filter(predicates, segs, 1, nrows, soup, col_off, col_list, d_occupancy, flagged,
                          stats, st);
        launch_occ_exact(predicates, segs, 1, soup, col_off, col_list, flagged, hs, hv,
                         d_occupancy, stats, 2 * device_sms(), st);
        CMG_CUDA(cudaStreamSynchronize(st));
        return CMG_OK;
    } catch (const std::exception& e) {
        set_err(errbuf, errbuf_len, e.what());
        return CMG_ERR_INTERNAL;
    }
}
