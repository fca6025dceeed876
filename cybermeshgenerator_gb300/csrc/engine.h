// engine.h — host orchestration of the voxelization pipeline on one GPU.
//
// A Batch holds one or more meshes (each with its own grid) resident on the
// device, the workspace sized for them, and the device outputs. run() enqueues
// the whole pipeline on a stream:
//   occupancy: triangle prep -> per-column buckets -> FP64 filter -> exact pass
//   SDF:       triangle bins -> brick candidate lists -> LPT work order ->
//              persistent evaluation (plain FP64 or mixed FP32 + FP64 band)
// The first run sizes the workspace (it reads two totals back from the device);
// later runs allocate nothing and synchronise nothing, so they can be captured in
// a CUDA graph and replayed.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "cmg_types.h"
#include "host_mem.h"

namespace cmg::gpu {

struct VoxOpts {
    int predicates = kPredCompat;  // kPredCompat (reference semantics) | kPredExact
    int precision = kPrecFP64;     // kPrecFP64 (bit-exact) | kPrecMixed
    bool fp64_filter = true;       // kPrecFP64 on 16^3 bricks: the FP32 pass with an FP64
                                   // refinement of each cell's near-ties (kPrecExact);
                                   // false: every candidate in FP64 (the same results)
    int brick = 0;                 // candidate brick edge: 16 (default; 4^3 sub-brick
                                   // evaluation), 8 or 4 (one CTA per brick)
    float band = 1.0f;             // mixed: FP64 refinement band, in cells
    bool want_occ = true;
    bool want_sdf32 = false;
    bool want_sdf64 = false;
    bool want_near = false;        // nearest triangle id + Ericson region per cell
    bool want_err = false;         // mixed: stated per-cell FP32 error bound
    bool autotune = false;
    int grab = 0;                  // sub-bricks per queue grab (1, 2, 4, 8); 0 = default
    int stage = -1;                // mixed: stage candidate records in shared memory
                                   // (1) or read them from L1/L2 (0); -1 = default
    int walk_warps = 0;            // warps per brick in the candidate walk (1, 2, 4); 0 =
                                   // by the brick count
    int probe = 0;                 // mixed: brick-list head the probe scans; 0 = default
    int ctas = 0;                  // evaluation CTAs per SM (12 or 16); 0 = default (12)
};

struct HostMesh {
    const double* pts = nullptr;  // 3*npts
    int64_t npts = 0;
    const int* tris = nullptr;    // 3*ntris, indices into pts
    int64_t ntris = 0;
    GridDesc g{};
};

// Host array filled by a device copy: allocated without value-initialisation, from
// the page-locked block pool.
template <typename T>
class HostBuf {
public:
    HostBuf() = default;
    ~HostBuf() { reset(); }
    HostBuf(const HostBuf&) = delete;
    HostBuf& operator=(const HostBuf&) = delete;
    HostBuf(HostBuf&& o) noexcept { take(o); }
    HostBuf& operator=(HostBuf&& o) noexcept {
        if (this != &o) {
            reset();
            take(o);
        }
        return *this;
    }
    void resize(size_t n) {
        if (n * sizeof(T) <= cap_ && n_ != 0) {
            n_ = n;
            return;
        }
        reset();
        if (n) p_ = static_cast<T*>(host_block_acquire(n * sizeof(T), &cap_, &pinned_));
        n_ = n;
    }
    T* data() { return p_; }
    const T* data() const { return p_; }
    size_t size() const { return n_; }
    bool empty() const { return n_ == 0; }
    T& operator[](size_t i) { return p_[i]; }
    const T& operator[](size_t i) const { return p_[i]; }
    const T* begin() const { return p_; }
    const T* end() const { return p_ + n_; }

private:
    void reset() {
        if (p_) host_block_release(p_, cap_, pinned_);
        p_ = nullptr;
        n_ = cap_ = 0;
        pinned_ = false;
    }
    void take(HostBuf& o) {
        p_ = o.p_; n_ = o.n_; cap_ = o.cap_; pinned_ = o.pinned_;
        o.p_ = nullptr; o.n_ = o.cap_ = 0; o.pinned_ = false;
    }
    T* p_ = nullptr;
    size_t n_ = 0, cap_ = 0;
    bool pinned_ = false;
};

struct HostResult {
    HostBuf<uint8_t> occ;
    HostBuf<float> sdf32;
    HostBuf<double> sdf64;
    HostBuf<int> near_tri;
    HostBuf<uint8_t> near_reg;
    HostBuf<float> err;
};

// Phase times of the last run(), from CUDA events on the batch's streams. The SDF
// preparation overlaps the occupancy passes (a second stream), so the phases can
// sum to more than the total.
struct Timing {
    float occupancy_ms = 0.f;  // triangle prep .. exact pass
    float sdf_prep_ms = 0.f;   // bins, candidate lists, work order
    float eval_ms = 0.f;       // the distance evaluation kernel
    float total_ms = 0.f;
};

// Cost model counts of a finished run (see k_count_K).
struct WorkModel {
    double sum_k = 0;       // sum over cells of K(v)
    double sum_k_band = 0;  // over the FP64 band cells
    double band_cells = 0;
    double orient_calls = 0;
    double crossings = 0;
};

struct RunInfo {
    Stats stats{};
    int brick = 0;
    int grab = 0;
    int walk_warps = 0;  // warps per brick of the candidate walk
    int probe = 0;       // probe head (mixed)
    int ctas = 0;        // evaluation CTAs per SM
    int64_t cells = 0;
    int64_t pairs = 0;       // (triangle, column) bucket entries
    int64_t candidates = 0;  // (brick, triangle) candidate entries
};

class Batch {
public:
    // Uploads the meshes (host buffers) and plans the workspace. Grids must be set.
    // A transient batch borrows the device's shared workspace (at most one alive
    // per device at a time); otherwise the batch owns its memory.
    Batch(const std::vector<HostMesh>& meshes, const VoxOpts& opts, cudaStream_t stream,
          bool transient = false);
    ~Batch();
    Batch(const Batch&) = delete;
    Batch& operator=(const Batch&) = delete;

    // Re-uploads point coordinates (same topology and grids), e.g. between
    // forward passes of an optimisation. Moved points change the bucket and
    // candidate list lengths, so the next run re-sizes the workspace.
    void update_points(const std::vector<HostMesh>& meshes);
    // Device-pointer form: the coordinates already live on the device
    // (concatenated, 3 doubles per point, triangle indices unchanged).
    void update_points_device(const double* d_pts);

    // Enqueues the pipeline. The first call (and the first after an update of the
    // points) sizes the workspace, synchronising twice; other calls only enqueue.
    void run();
    // Replays the pipeline as a CUDA graph. A call that must size the workspace
    // runs the pipeline eagerly instead (and drops a graph whose buffers moved);
    // the graph is captured at the next call and replayed from then on.
    void run_graph();
    // Stream for later runs (graph replays included).
    void set_stream(cudaStream_t st) { stream_ = st; }
    void synchronize();
    void download(std::vector<HostResult>& out, RunInfo* info);
    // Mesh i's outputs only.
    void download_one(int i, HostResult& out);
    RunInfo info();
    // Records CUDA events around the phases of each run() (not in graph replays).
    void set_timing(bool on) { timing_ = on; }
    Timing timing();
    // Runs the K(v) counting pass over the last run's outputs (needs an SDF output).
    WorkModel work_model();

    int nmeshes() const { return static_cast<int>(segs_.size()); }
    const std::vector<MeshSeg>& segs() const { return segs_; }
    int64_t total_cells() const { return nvox_; }
    int64_t total_points() const { return npts_; }
    int64_t total_tris() const { return ntris_; }
    const VoxOpts& opts() const { return opts_; }
    cudaStream_t stream() const { return stream_; }
    // device outputs (nullptr unless requested)
    uint8_t* d_occ() const { return occ_; }
    float* d_sdf32() const { return sdf32_; }
    double* d_sdf64() const { return sdf64_; }
    int* d_near_tri() const { return near_tri_; }
    uint8_t* d_near_reg() const { return near_reg_; }
    const double* d_points() const { return pts_; }
    const int* d_tris() const { return tris_; }
    // Bytes moved host->device by construction / update_points and device->host by
    // download (the e2e accounting).
    int64_t h2d_bytes() const { return h2d_bytes_; }
    int64_t d2h_bytes() const;

private:
    struct Impl;
    std::unique_ptr<Impl> impl_;
    VoxOpts opts_;
    cudaStream_t stream_;
    std::vector<MeshSeg> segs_;
    int64_t npts_ = 0, ntris_ = 0, ncol_ = 0, nrow_ = 0, nvox_ = 0, nbrick_ = 0, nwork_ = 0;
    int64_t pairs_cap_ = -1, cand_cap_ = -1;
    bool resize_ = false;  // points moved since the workspace was sized
    double* pts_ = nullptr;
    int* tris_ = nullptr;
    MeshSeg* dsegs_ = nullptr;
    uint8_t* occ_ = nullptr;
    float* sdf32_ = nullptr;
    double* sdf64_ = nullptr;
    int* near_tri_ = nullptr;
    uint8_t* near_reg_ = nullptr;
    float* err_ = nullptr;
    Stats* stats_ = nullptr;
    unsigned long long* queue_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;
    int64_t h2d_bytes_ = 0;
    bool timing_ = false;
    // step start, occupancy done, evaluation start, step end, SDF preparation start / end
    cudaEvent_t ev_[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // The SDF preparation needs the triangle soup but not the occupancy, so it runs on
    // a second stream beside the occupancy passes and joins before the evaluation.
    cudaStream_t side_ = nullptr;
    cudaEvent_t fork_ = nullptr, join_ = nullptr;
    // work on side_ not yet joined (a run that threw between fork and join): the next
    // run and the destructor wait for it before the buffers are used again
    bool side_open_ = false;
    void run_impl(bool sizing);
    bool needs_sizing() const { return pairs_cap_ < 0 || cand_cap_ < 0 || resize_; }
    void sized_run();
};

// Sets opts.brick, grab, walk_warps, probe and ctas for a workload by timing the
// candidates on the device (see engine.cu); the choice is cached per process by
// workload shape (precision, log2 of triangle and cell counts, number of meshes,
// whether FP64 distances are kept).
void autotune(const std::vector<HostMesh>& meshes, VoxOpts& opts, cudaStream_t stream);

// Number of SMs of the current device.
int device_sms();

}  // namespace cmg::gpu
