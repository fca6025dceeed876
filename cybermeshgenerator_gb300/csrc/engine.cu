// engine.cu — host orchestration of the voxelization pipeline (see engine.h).
#include "engine.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <tuple>

#include "cmg_util.h"
#include "engine_kernels.h"

namespace cmg::gpu {

namespace {
std::atomic<long long> g_launches{0};
}
void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches() { return g_launches.load(std::memory_order_relaxed); }

namespace {
std::mutex g_alloc_mu;
int g_alloc_skip = 0, g_alloc_fail = 0;
}  // namespace

void set_alloc_failures(int skip, int count) {
    std::lock_guard<std::mutex> lk(g_alloc_mu);
    g_alloc_skip = skip > 0 ? skip : 0;
    g_alloc_fail = count > 0 ? count : 0;
}

cudaError_t device_alloc_raw(void** p, size_t bytes) {
    {
        std::lock_guard<std::mutex> lk(g_alloc_mu);
        if (g_alloc_fail > 0) {
            if (g_alloc_skip > 0) {
                --g_alloc_skip;
            } else {
                --g_alloc_fail;
                *p = nullptr;
                return cudaErrorMemoryAllocation;  // the fake: nothing was allocated
            }
        }
    }
    return cudaMalloc(p, bytes);
}

// ------------------------------------------------------------------ host block pool
namespace {

struct HostPool {
    static constexpr size_t kCachedCap = size_t{4} << 30;  // idle pinned bytes kept
    std::mutex mu;
    std::multimap<size_t, void*> idle;                      // capacity -> block
    size_t cached = 0;
};

HostPool& host_pool() {
    static HostPool* pool = new HostPool;  // never destroyed: blocks outlive static teardown
    return *pool;
}

}  // namespace

void* host_block_acquire(size_t bytes, size_t* cap, bool* pinned) {
    HostPool& P = host_pool();
    {
        std::lock_guard<std::mutex> lk(P.mu);
        auto it = P.idle.lower_bound(bytes);
        if (it != P.idle.end() && it->first <= 2 * bytes + (size_t{1} << 20)) {
            void* p = it->second;
            *cap = it->first;
            *pinned = true;
            P.cached -= it->first;
            P.idle.erase(it);
            return p;
        }
    }
    const size_t c = (bytes + 65535) & ~size_t{65535};
    void* p = nullptr;
    if (cudaHostAlloc(&p, c, cudaHostAllocDefault) == cudaSuccess && p) {
        *cap = c;
        *pinned = true;
        return p;
    }
    cudaGetLastError();  // a failed pinning is not an error of the pipeline
    p = std::malloc(bytes);
    if (!p) throw std::bad_alloc();
    *cap = bytes;
    *pinned = false;
    return p;
}

void host_block_release(void* p, size_t cap, bool pinned) {
    if (!p) return;
    if (!pinned) {
        std::free(p);
        return;
    }
    HostPool& P = host_pool();
    {
        std::lock_guard<std::mutex> lk(P.mu);
        if (P.cached + cap <= HostPool::kCachedCap) {
            P.idle.emplace(cap, p);
            P.cached += cap;
            return;
        }
    }
    cudaFreeHost(p);
}

namespace {
constexpr size_t kLargeHost = size_t{1} << 20;
struct LargeBlocks {
    std::mutex mu;
    std::map<void*, std::pair<size_t, bool>> live;  // block -> capacity, page-locked
};
LargeBlocks& large_blocks() {
    static LargeBlocks* b = new LargeBlocks;  // never destroyed, like the pool
    return *b;
}
}  // namespace

void* host_large_alloc(size_t bytes) {
    if (bytes < kLargeHost) {
        void* p = std::malloc(bytes ? bytes : 1);
        if (!p) throw std::bad_alloc();
        return p;
    }
    size_t cap = 0;
    bool pinned = false;
    void* p = host_block_acquire(bytes, &cap, &pinned);
    LargeBlocks& L = large_blocks();
    std::lock_guard<std::mutex> lk(L.mu);
    L.live[p] = {cap, pinned};
    return p;
}

void host_large_free(void* p, size_t bytes) noexcept {
    if (!p) return;
    if (bytes < kLargeHost) {
        std::free(p);
        return;
    }
    std::pair<size_t, bool> b{0, false};
    {
        LargeBlocks& L = large_blocks();
        std::lock_guard<std::mutex> lk(L.mu);
        auto it = L.live.find(p);
        if (it == L.live.end()) return;
        b = it->second;
        L.live.erase(it);
    }
    host_block_release(p, b.first, b.second);
}

int device_sms() {
    int dev = 0, sms = 0;
    CMG_CUDA(cudaGetDevice(&dev));
    CMG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    return sms;
}

namespace {

template <typename T>
T* carve(Arena& a, size_t n) {
    T* p = a.take<T>(n ? n : 1);
    return p;
}

// 16: candidate lists per 16^3 brick, evaluation per 4^3 sub-brick (default);
// 4 or 8: one list and one evaluation CTA per brick of that edge.
int pick_brick(const VoxOpts& o) { return (o.brick == 4 || o.brick == 8) ? o.brick : 16; }

// The 4^3 sub-brick kernel's precision: mixed, exact FP64 through the FP32 pass
// (kPrecExact), or every candidate in FP64.
int sub_precision(const VoxOpts& o) {
    if (o.precision == kPrecMixed) return kPrecMixed;
    return o.fp64_filter ? kPrecExact : kPrecFP64;
}

}  // namespace

// Workspace arenas shared by transient batches on a device (one call at a time,
// serialised by the caller), so repeated single calls do not re-allocate.
struct Pool {
    Arena a[4];
};
Pool& pool_for_device() {
    static std::mutex mu;
    static std::map<int, std::unique_ptr<Pool>> pools;
    int dev = 0;
    CMG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(mu);
    auto& p = pools[dev];
    if (!p) p.reset(new Pool);
    return *p;
}

struct Batch::Impl {
    Arena own[4];
    Arena& fixed;    // inputs, sized-up-front workspace
    Arena& pairs;    // (triangle, column) bucket entries and their scratch
    Arena& cands;    // brick candidate lists
    Arena& outs;     // outputs
    // a == nullptr: the batch owns its arenas
    explicit Impl(Arena* a)
        : fixed(a ? a[0] : own[0]), pairs(a ? a[1] : own[1]), cands(a ? a[2] : own[2]),
          outs(a ? a[3] : own[3]) {}
    // workspace
    double* soup = nullptr;
    int4* xybox = nullptr;
    int64_t* pairs_n = nullptr;
    int64_t* pair_off = nullptr;
    int* colcnt = nullptr;
    int64_t* col_off = nullptr;
    int64_t* flagged = nullptr;
    int64_t* scan_tmp = nullptr;
    int64_t* scan_tmp_side = nullptr;  // the SDF preparation's, on the second stream
    uint8_t* occ_internal = nullptr;
    int* col_list = nullptr;
    double* hs = nullptr;
    uint8_t* hv = nullptr;
    // sdf
    float4* tinfo = nullptr;
    float4* tinfo_lo = nullptr;
    float4* tnorm = nullptr;  // unit normal (FP32) and its error bound
    void* trec = nullptr;
    float4* tlo = nullptr;
    float4* thi = nullptr;
    int64_t* tbin = nullptr;
    int* bincnt = nullptr;
    int64_t* bin_off = nullptr;
    int* bin_list = nullptr;
    int* large_cnt = nullptr;
    int64_t* large_off = nullptr;
    int* large_list = nullptr;
    unsigned* emax_bits = nullptr;
    float* bound = nullptr;
    int* cand_cnt = nullptr;
    int64_t* cand_off = nullptr;
    float* brick_emax = nullptr;
    uint32_t* work_keys = nullptr;
    uint32_t* work = nullptr;
    void* sort_tmp = nullptr;
    int* cand = nullptr;
    int grid_exact = 0;
    int grid_eval = 0;
    cudaGraph_t graph = nullptr;
};

Batch::Batch(const std::vector<HostMesh>& meshes, const VoxOpts& opts, cudaStream_t stream,
             bool transient)
    : opts_(opts), stream_(stream) {
    impl_.reset(new Impl(transient ? pool_for_device().a : nullptr));
    bool slab = false;
    for (const HostMesh& m : meshes)
        slab = slab || (m.g.z1 > 0 && (m.g.z0 != 0 || m.g.z1 != m.g.nz));
    // a slab is evaluated by 16^3 bricks (their 4^3 sub-bricks keep the whole grid's
    // geometry, which makes the slab's cells those of the whole grid)
    const int brick = slab ? 16 : pick_brick(opts);
    opts_.brick = brick;
    const int rc = occ_row_cols();
    int64_t tb = 0, pb = 0;
    for (const HostMesh& m : meshes) {
        if (m.g.nx <= 0 || m.g.ny <= 0 || m.g.nz <= 0)
            throw std::invalid_argument("voxelize: empty grid");
        MeshSeg s{};
        s.g = m.g;
        if (s.g.z1 <= 0) {  // the whole grid
            s.g.z0 = 0;
            s.g.z1 = s.g.nz;
        }
        if (s.g.z0 < 0 || s.g.z0 >= s.g.z1 || s.g.z1 > s.g.nz)
            throw std::invalid_argument("voxelize: cell layers outside the grid");
        s.tri_begin = tb;
        s.tri_end = tb + m.ntris;
        s.col_begin = ncol_;
        s.row_begin = nrow_;
        s.vox_begin = nvox_;
        s.brick_begin = nbrick_;
        s.brick = brick;
        s.bnx = (m.g.nx + brick - 1) / brick;
        s.bny = (m.g.ny + brick - 1) / brick;
        // along z only the bricks that overlap the slab
        s.bzo = s.g.z0 / brick;
        s.bnz = (s.g.z1 - 1) / brick + 1 - s.bzo;
        double sc = 0.0;
        for (int64_t i = 0; i < m.npts; ++i)
            for (int a = 0; a < 3; ++a) sc = std::max(sc, std::fabs(m.pts[3 * i + a] - m.g.corner[a]));
        sc = std::max(sc, m.g.h * std::max(m.g.nx, std::max(m.g.ny, m.g.nz)));
        s.scale = static_cast<float>(sc * 1.0001);
        segs_.push_back(s);
        tb += m.ntris;
        pb += m.npts;
        ncol_ += static_cast<int64_t>(m.g.nx) * m.g.ny;
        nrow_ += static_cast<int64_t>(m.g.ny) * ((m.g.nx + rc - 1) / rc);
        nvox_ += slab_cells(s.g);
        nbrick_ += static_cast<int64_t>(s.bnx) * s.bny * s.bnz;
    }
    ntris_ = tb;
    npts_ = pb;
    nwork_ = brick == 16 ? 64 * nbrick_ : nbrick_;
    if (nwork_ >= (int64_t(1) << 32)) throw std::invalid_argument("voxelize: grid too large");
    const int nseg = static_cast<int>(segs_.size());
    const bool sdf = opts_.want_sdf32 || opts_.want_sdf64 || opts_.want_near;

    // ---- fixed workspace
    Arena& A = impl_->fixed;
    auto plan = [&](bool commit) {
        A.reset();
        pts_ = carve<double>(A, 3 * npts_);
        tris_ = carve<int>(A, 3 * ntris_);
        dsegs_ = carve<MeshSeg>(A, nseg);
        stats_ = carve<Stats>(A, 1);
        queue_ = carve<unsigned long long>(A, 1);
        impl_->soup = carve<double>(A, kSoupStride * ntris_);
        impl_->xybox = carve<int4>(A, ntris_);
        impl_->pairs_n = carve<int64_t>(A, ntris_ + 1);
        impl_->pair_off = carve<int64_t>(A, ntris_ + 1);
        impl_->colcnt = carve<int>(A, ncol_);
        impl_->col_off = carve<int64_t>(A, ncol_ + 1);
        impl_->flagged = carve<int64_t>(A, ncol_);
        int64_t smax = std::max(std::max(ntris_, ncol_), std::max(nbrick_, int64_t(nseg)));
        impl_->scan_tmp = carve<int64_t>(A, scan_tmp_elems(smax));
        if (!opts_.want_occ) impl_->occ_internal = carve<uint8_t>(A, nvox_);
        if (sdf) {
            impl_->scan_tmp_side = carve<int64_t>(A, scan_tmp_elems(smax));
            impl_->tinfo = carve<float4>(A, ntris_);
            impl_->tinfo_lo = carve<float4>(A, ntris_);
            impl_->tnorm = carve<float4>(A, ntris_);
            impl_->trec = carve<char>(A, kTriRecBytes * static_cast<size_t>(ntris_));
            impl_->tlo = carve<float4>(A, ntris_);
            impl_->thi = carve<float4>(A, ntris_);
            impl_->tbin = carve<int64_t>(A, ntris_);
            impl_->bincnt = carve<int>(A, nbrick_);
            impl_->bin_off = carve<int64_t>(A, nbrick_ + 1);
            impl_->bin_list = carve<int>(A, ntris_);
            impl_->large_cnt = carve<int>(A, 2 * nseg);
            impl_->large_off = carve<int64_t>(A, nseg + 1);
            impl_->large_list = carve<int>(A, ntris_);
            impl_->emax_bits = carve<unsigned>(A, 3 * nseg);  // emax, scale, emax_all
            impl_->bound = carve<float>(A, nbrick_);
            impl_->cand_cnt = carve<int>(A, nbrick_);
            impl_->cand_off = carve<int64_t>(A, nbrick_ + 1);
            impl_->brick_emax = carve<float>(A, nbrick_);
            impl_->work_keys = carve<uint32_t>(A, nwork_);
            impl_->work = carve<uint32_t>(A, nwork_);
            impl_->sort_tmp = carve<char>(A, radix_sort_tmp_bytes(nwork_));
        }
        if (commit) return;
    };
    A.clear_need();
    plan(false);
    if (A.overflowed()) {
        A.reserve(A.need());
        plan(true);
    }
    // ---- outputs
    Arena& O = impl_->outs;
    auto plan_out = [&]() {
        O.reset();
        occ_ = opts_.want_occ ? carve<uint8_t>(O, nvox_) : nullptr;
        sdf32_ = opts_.want_sdf32 ? carve<float>(O, nvox_) : nullptr;
        sdf64_ = opts_.want_sdf64 ? carve<double>(O, nvox_) : nullptr;
        near_tri_ = opts_.want_near ? carve<int>(O, nvox_) : nullptr;
        near_reg_ = opts_.want_near ? carve<uint8_t>(O, nvox_) : nullptr;
        err_ = (opts_.want_err && opts_.precision == kPrecMixed) ? carve<float>(O, nvox_) : nullptr;
    };
    O.clear_need();
    plan_out();
    if (O.overflowed()) {
        O.reserve(O.need());
        plan_out();
    }
    if (!opts_.want_occ) occ_ = nullptr;

    // ---- upload inputs (indices rebased to the concatenated point array)
    std::vector<double> hp(static_cast<size_t>(3 * npts_));
    std::vector<int> ht(static_cast<size_t>(3 * ntris_));
    int64_t po = 0, to = 0;
    for (const HostMesh& m : meshes) {
        std::memcpy(hp.data() + 3 * po, m.pts, sizeof(double) * 3 * m.npts);
        for (int64_t i = 0; i < 3 * m.ntris; ++i) ht[3 * to + i] = m.tris[i] + static_cast<int>(po);
        po += m.npts;
        to += m.ntris;
    }
    CMG_CUDA(cudaMemcpyAsync(pts_, hp.data(), sizeof(double) * hp.size(), cudaMemcpyHostToDevice, stream_));
    CMG_CUDA(cudaMemcpyAsync(tris_, ht.data(), sizeof(int) * ht.size(), cudaMemcpyHostToDevice, stream_));
    CMG_CUDA(cudaMemcpyAsync(dsegs_, segs_.data(), sizeof(MeshSeg) * segs_.size(),
                             cudaMemcpyHostToDevice, stream_));
    CMG_CUDA(cudaStreamSynchronize(stream_));  // host vectors go out of scope
    h2d_bytes_ = static_cast<int64_t>(sizeof(double) * hp.size() + sizeof(int) * ht.size());

    const int sms = device_sms();
    impl_->grid_exact = 2 * sms;
    // persistent evaluation grid: resident CTAs per SM for the chosen kernel
    if (opts_.grab <= 0) opts_.grab = 1;
    if (opts_.stage < 0) opts_.stage = 0;
    if (brick == 16) impl_->grid_eval = sdf ? sdf_sub_grid(sub_precision(opts_), opts_.stage != 0, opts_.ctas) : sms;
    else impl_->grid_eval = (brick == 4 ? 8 : 3) * sms;
    if (sdf) {  // made here: a graph capture must not create them
        CMG_CUDA(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
        CMG_CUDA(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
        CMG_CUDA(cudaEventCreateWithFlags(&join_, cudaEventDisableTiming));
    }
}

Batch::~Batch() {
    for (cudaEvent_t& e : ev_)
        if (e) cudaEventDestroy(e);
    if (fork_) cudaEventDestroy(fork_);
    if (join_) cudaEventDestroy(join_);
    if (side_) {
        if (side_open_) cudaStreamSynchronize(side_);  // pooled arenas are reused next
        cudaStreamDestroy(side_);
    }
    if (graph_) cudaGraphExecDestroy(graph_);
    if (impl_ && impl_->graph) cudaGraphDestroy(impl_->graph);
}

void Batch::update_points(const std::vector<HostMesh>& meshes) {
    std::vector<double> hp(static_cast<size_t>(3 * npts_));
    int64_t po = 0;
    for (const HostMesh& m : meshes) {
        std::memcpy(hp.data() + 3 * po, m.pts, sizeof(double) * 3 * m.npts);
        po += m.npts;
    }
    CMG_CUDA(cudaMemcpyAsync(pts_, hp.data(), sizeof(double) * hp.size(), cudaMemcpyHostToDevice, stream_));
    CMG_CUDA(cudaStreamSynchronize(stream_));
    resize_ = true;
}

void Batch::update_points_device(const double* d_pts) {
    CMG_CUDA(cudaMemcpyAsync(pts_, d_pts, sizeof(double) * 3 * npts_, cudaMemcpyDeviceToDevice, stream_));
    resize_ = true;
}

// A sizing pass: reads the list totals back, grows the list arenas if needed and
// drops the captured graph when a grown arena moved the buffers it refers to.
void Batch::sized_run() {
    const size_t pc = impl_->pairs.capacity(), cc = impl_->cands.capacity();
    run_impl(true);
    resize_ = false;
    if ((impl_->pairs.capacity() != pc || impl_->cands.capacity() != cc) && graph_) {
        CMG_CUDA(cudaStreamSynchronize(stream_));
        CMG_CUDA(cudaGraphExecDestroy(graph_));
        graph_ = nullptr;
        CMG_CUDA(cudaGraphDestroy(impl_->graph));
        impl_->graph = nullptr;
    }
}

void Batch::run() {
    if (needs_sizing()) sized_run();
    else run_impl(false);
}

void Batch::run_graph() {
    if (needs_sizing()) {  // sizing synchronises, so it runs outside any capture
        sized_run();
        return;
    }
    if (!graph_) {
        CMG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        run_impl(false);
        CMG_CUDA(cudaStreamEndCapture(stream_, &impl_->graph));
        CMG_CUDA(cudaGraphInstantiate(&graph_, impl_->graph, 0));
    }
    CMG_CUDA(cudaGraphLaunch(graph_, stream_));
}

void Batch::synchronize() { CMG_CUDA(cudaStreamSynchronize(stream_)); }

void Batch::run_impl(bool sizing) {
    Impl& I = *impl_;
    cudaStream_t st = stream_;
    const int nseg = static_cast<int>(segs_.size());
    const bool sdf = opts_.want_sdf32 || opts_.want_sdf64 || opts_.want_near;
    uint8_t* occ = opts_.want_occ ? occ_ : I.occ_internal;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CMG_CUDA(cudaStreamIsCapturing(st, &cap));
    const bool timed = timing_ && cap == cudaStreamCaptureStatusNone;
    if (timed && !ev_[0])
        for (cudaEvent_t& e : ev_) CMG_CUDA(cudaEventCreate(&e));
    if (side_open_) {
        CMG_CUDA(cudaStreamSynchronize(side_));
        side_open_ = false;
    }
    if (timed) CMG_CUDA(cudaEventRecord(ev_[0], st));

    CMG_CUDA(cudaMemsetAsync(stats_, 0, sizeof(Stats), st));
    launch_tri_prep(dsegs_, nseg, ntris_, pts_, tris_, I.soup, I.xybox, I.pairs_n, st);

    // Ray-parity occupancy: (triangle, column) pairs, filter, exact pass. The pair count
    // sizes the pair arena in a sizing run.
    auto occ_head = [&](cudaStream_t s) {
        exclusive_scan(I.pairs_n, I.pair_off, ntris_, I.scan_tmp, s);
        if (!sizing) return;
        int64_t P = 0;
        CMG_CUDA(cudaMemcpyAsync(&P, I.pair_off + ntris_, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        CMG_CUDA(cudaStreamSynchronize(s));
        Arena& B = I.pairs;
        auto planb = [&]() {
            B.reset();
            I.col_list = carve<int>(B, P);
            I.hs = carve<double>(B, P);
            I.hv = carve<uint8_t>(B, P);
        };
        B.clear_need();
        planb();
        if (B.overflowed()) {
            B.reserve(B.need());
            planb();
        }
        pairs_cap_ = P;
    };
    auto occ_tail = [&](cudaStream_t s) {
        const int pair_grid = 4 * device_sms();
        CMG_CUDA(cudaMemsetAsync(I.colcnt, 0, sizeof(int) * std::max<int64_t>(ncol_, 1), s));
        launch_col_pairs(false, dsegs_, nseg, ntris_, I.xybox, I.pair_off, I.colcnt, nullptr, nullptr,
                         pair_grid, s);
        exclusive_scan(I.colcnt, I.col_off, ncol_, I.scan_tmp, s);
        CMG_CUDA(cudaMemsetAsync(I.colcnt, 0, sizeof(int) * std::max<int64_t>(ncol_, 1), s));
        launch_col_pairs(true, dsegs_, nseg, ntris_, I.xybox, I.pair_off, I.colcnt, I.col_off,
                         I.col_list, pair_grid, s);
        launch_occ_filter(opts_.predicates, dsegs_, nseg, nrow_, I.soup, I.col_off, I.col_list, occ,
                          I.flagged, stats_, s);
        launch_occ_exact(opts_.predicates, dsegs_, nseg, I.soup, I.col_off, I.col_list, I.flagged,
                         I.hs, I.hv, occ, stats_, I.grid_exact, s);
        if (timed) CMG_CUDA(cudaEventRecord(ev_[1], s));
    };
    if (!sdf) {
        occ_head(st);
        occ_tail(st);
        if (timed)
            for (int e : {4, 5, 2, 3}) CMG_CUDA(cudaEventRecord(ev_[e], st));
        return;
    }

    // SDF preparation: triangle bins, brick walk (candidate lists), work order. It reads
    // the soup, never the occupancy, so it runs on the second stream beside the
    // occupancy passes. The candidate count sizes the candidate arena in a sizing run.
    cudaStream_t ss = side_;
    int64_t* tmp = I.scan_tmp_side;
    auto prep_head = [&]() {
        if (timed) CMG_CUDA(cudaEventRecord(ev_[4], ss));
        CMG_CUDA(cudaMemsetAsync(I.bincnt, 0, sizeof(int) * nbrick_, ss));
        CMG_CUDA(cudaMemsetAsync(I.large_cnt, 0, sizeof(int) * 2 * nseg, ss));
        CMG_CUDA(cudaMemsetAsync(I.emax_bits, 0, sizeof(unsigned) * 3 * nseg, ss));
        launch_sdf_tri_prep(dsegs_, nseg, ntris_, I.soup, I.tinfo, I.tinfo_lo, I.trec, I.tnorm, I.tlo,
                            I.thi, I.tbin, I.bincnt, I.large_cnt, I.emax_bits, ss);
        exclusive_scan(I.bincnt, I.bin_off, nbrick_, tmp, ss);
        exclusive_scan(I.large_cnt, I.large_off, nseg, tmp, ss);
        launch_seg_finish(dsegs_, nseg, I.large_off, I.emax_bits, ss);
        CMG_CUDA(cudaMemsetAsync(I.bincnt, 0, sizeof(int) * nbrick_, ss));
        CMG_CUDA(cudaMemsetAsync(I.large_cnt + nseg, 0, sizeof(int) * nseg, ss));
        launch_bin_fill(ntris_, I.tbin, I.bin_off, I.bincnt, I.bin_list, dsegs_, nseg,
                        I.large_cnt + nseg, I.large_list, ss);
        launch_brick_walk(false, dsegs_, nseg, nbrick_, I.soup, I.tinfo, I.tlo, I.thi, I.bin_off,
                          I.bin_list, I.large_list, I.bound, I.cand_cnt, nullptr, nullptr, nullptr,
                          stats_, opts_.walk_warps, ss);
        exclusive_scan(I.cand_cnt, I.cand_off, nbrick_, tmp, ss);
    };
    auto prep_size = [&]() {
        int64_t C = 0;
        CMG_CUDA(cudaMemcpyAsync(&C, I.cand_off + nbrick_, sizeof(int64_t), cudaMemcpyDeviceToHost, ss));
        CMG_CUDA(cudaStreamSynchronize(ss));
        Arena& Cn = I.cands;
        auto planc = [&]() {
            Cn.reset();
            I.cand = carve<int>(Cn, C);
        };
        Cn.clear_need();
        planc();
        if (Cn.overflowed()) {
            Cn.reserve(Cn.need());
            planc();
        }
        cand_cap_ = C;
    };
    auto prep_tail = [&]() {
        launch_brick_walk(true, dsegs_, nseg, nbrick_, I.soup, I.tinfo, I.tlo, I.thi, I.bin_off,
                          I.bin_list, I.large_list, I.bound, I.cand_cnt, I.cand_off, I.cand,
                          I.brick_emax, stats_, opts_.walk_warps, ss);
        if (opts_.brick == 16) launch_sub_work_keys(I.cand_cnt, nbrick_, I.work_keys, I.work, ss);
        else launch_work_keys(I.cand_cnt, nbrick_, I.work_keys, I.work, ss);
        radix_sort_pairs(I.work_keys, I.work, nwork_, 32, I.sort_tmp, ss);
        CMG_CUDA(cudaMemsetAsync(queue_, 0, sizeof(unsigned long long), ss));
        if (timed) CMG_CUDA(cudaEventRecord(ev_[5], ss));
    };

    // The longer preparation is issued first. In a sizing run each arena is re-planned
    // while the other stream's passes, which do not touch it, keep the device busy.
    CMG_CUDA(cudaEventRecord(fork_, st));
    CMG_CUDA(cudaStreamWaitEvent(ss, fork_, 0));
    side_open_ = true;
    prep_head();
    occ_head(st);
    if (!sizing) prep_tail();
    occ_tail(st);
    if (sizing) {
        prep_size();
        prep_tail();
    }
    CMG_CUDA(cudaEventRecord(join_, ss));
    CMG_CUDA(cudaStreamWaitEvent(st, join_, 0));
    side_open_ = false;
    if (timed) CMG_CUDA(cudaEventRecord(ev_[2], st));
    if (opts_.brick == 16)
        launch_sdf_sub(sub_precision(opts_), opts_.stage != 0, opts_.grab, opts_.probe, opts_.ctas, dsegs_,
                       nseg, I.work, nwork_, queue_, I.soup, I.tinfo,
                       I.tinfo_lo, I.trec, I.tnorm, I.cand_off, I.cand, I.brick_emax, opts_.band, occ,
                       sdf32_, sdf64_, near_tri_, near_reg_, err_, stats_, I.grid_eval, st);
    else
        launch_sdf_eval(opts_.precision, opts_.brick, dsegs_, nseg, I.work, nbrick_, queue_,
                        I.soup, I.tinfo, I.cand_off, I.cand, I.brick_emax, opts_.band, occ,
                        sdf32_, sdf64_, near_tri_, near_reg_, err_, stats_, I.grid_eval, st);
    if (timed) CMG_CUDA(cudaEventRecord(ev_[3], st));
}

Timing Batch::timing() {
    Timing t;
    if (!ev_[0]) return t;
    CMG_CUDA(cudaEventSynchronize(ev_[3]));
    CMG_CUDA(cudaEventElapsedTime(&t.occupancy_ms, ev_[0], ev_[1]));
    CMG_CUDA(cudaEventElapsedTime(&t.sdf_prep_ms, ev_[4], ev_[5]));
    CMG_CUDA(cudaEventElapsedTime(&t.eval_ms, ev_[2], ev_[3]));
    CMG_CUDA(cudaEventElapsedTime(&t.total_ms, ev_[0], ev_[3]));
    return t;
}

WorkModel Batch::work_model() {
    WorkModel w;
    Impl& I = *impl_;
    RunInfo ri = info();
    w.orient_calls = static_cast<double>(ri.stats.orient_calls);
    w.crossings = static_cast<double>(ri.stats.crossings);
    if (!(sdf32_ || sdf64_) || !I.cand) return w;
    unsigned long long* d = nullptr;
    CMG_CUDA(device_alloc(&d, 3 * sizeof(unsigned long long)));
    CMG_CUDA(cudaMemsetAsync(d, 0, 3 * sizeof(unsigned long long), stream_));
    launch_count_K(opts_.brick, dsegs_, static_cast<int>(segs_.size()), nbrick_, I.tinfo, I.cand_off,
                   I.cand, sdf64_, sdf32_, opts_.band, d, stream_);
    unsigned long long h[3];
    CMG_CUDA(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, stream_));
    CMG_CUDA(cudaStreamSynchronize(stream_));
    cudaFree(d);
    w.sum_k = static_cast<double>(h[0]);
    w.sum_k_band = static_cast<double>(h[1]);
    w.band_cells = static_cast<double>(h[2]);
    return w;
}

int64_t Batch::d2h_bytes() const {
    int64_t b = 0;
    if (occ_) b += nvox_;
    if (sdf32_) b += 4 * nvox_;
    if (sdf64_) b += 8 * nvox_;
    if (near_tri_) b += 5 * nvox_;
    if (err_) b += 4 * nvox_;
    return b;
}

RunInfo Batch::info() {
    RunInfo r;
    CMG_CUDA(cudaMemcpyAsync(&r.stats, stats_, sizeof(Stats), cudaMemcpyDeviceToHost, stream_));
    CMG_CUDA(cudaStreamSynchronize(stream_));
    r.brick = opts_.brick;
    r.grab = opts_.brick == 16 ? opts_.grab : 0;
    r.walk_warps = brick_walk_warps(nbrick_, opts_.walk_warps);
    r.probe = sub_precision(opts_) != kPrecFP64 ? (opts_.probe > 0 ? opts_.probe : 1024) : 0;
    r.ctas = opts_.brick == 16 ? sdf_sub_minb(opts_.ctas) : 0;
    r.cells = nvox_;
    r.pairs = pairs_cap_;
    r.candidates = cand_cap_;
    return r;
}

void Batch::download_one(int m, HostResult& r) {
    const MeshSeg& s = segs_[static_cast<size_t>(m)];
    const int64_t n = slab_cells(s.g);
    auto get = [&](auto* dev, auto& vec) {
        if (!dev) return;
        vec.resize(static_cast<size_t>(n));
        CMG_CUDA(cudaMemcpyAsync(vec.data(), dev + s.vox_begin, sizeof(vec[0]) * n,
                                 cudaMemcpyDeviceToHost, stream_));
    };
    get(occ_, r.occ);
    get(sdf32_, r.sdf32);
    get(sdf64_, r.sdf64);
    get(near_tri_, r.near_tri);
    get(near_reg_, r.near_reg);
    get(err_, r.err);
    CMG_CUDA(cudaStreamSynchronize(stream_));
}

void Batch::download(std::vector<HostResult>& out, RunInfo* info) {
    out.resize(segs_.size());
    for (size_t m = 0; m < segs_.size(); ++m) download_one(static_cast<int>(m), out[m]);
    if (info) *info = this->info();
}

// ------------------------------------------------------------------ autotuner
// A coordinate search on the device, each candidate timed as a whole pipeline run
// (the better of two runs after the sizing run), in this order:
//   1. candidate brick edge and queue grab: 16^3 bricks evaluated by 4^3 sub-bricks
//      taken 1 or 2 per grab, or 8^3 bricks with one evaluation CTA each;
//   2. warps per brick of the candidate walk: 1, 2, 4 (the heaviest bricks' walks set
//      the SDF preparation time when the bricks are few);
//   3. mixed precision, 16^3 bricks: the probe head, 256 / 512 / 1024 / 2048 entries (a
//      longer head gives a tighter bound and shorter filtered lists for more loads);
//   4. 16^3 bricks: evaluation CTAs per SM, 12 (80 registers) or 16 (64 registers).
// Each step keeps the fastest value and moves on; the result is cached per process by
// workload shape.
namespace {
struct Tuned {
    int brick, grab, walk_warps, probe, ctas;
};
}  // namespace

void autotune(const std::vector<HostMesh>& meshes, VoxOpts& opts, cudaStream_t stream) {
    static std::mutex mu;
    static std::map<std::tuple<int, int, int, int, int>, Tuned> cache;
    int64_t tris = 0, cells = 0;
    for (const HostMesh& m : meshes) {
        tris += m.ntris;
        cells += m.g.z1 > 0 ? static_cast<int64_t>(m.g.nx) * m.g.ny * (m.g.z1 - m.g.z0)
                            : static_cast<int64_t>(m.g.nx) * m.g.ny * m.g.nz;
    }
    const bool sdf = opts.want_sdf32 || opts.want_sdf64 || opts.want_near;
    if (!sdf) return;  // the occupancy kernels have no tunables
    auto lg = [](int64_t v) { return v > 0 ? static_cast<int>(std::log2(static_cast<double>(v)) * 2) : 0; };
    auto key = std::make_tuple(sub_precision(opts), lg(tris), lg(cells),
                               static_cast<int>(std::min<size_t>(meshes.size(), 4)),
                               static_cast<int>(opts.want_sdf64));
    auto apply = [&](const Tuned& t) {
        opts.brick = t.brick;
        opts.grab = t.grab;
        opts.walk_warps = t.walk_warps;
        opts.probe = t.probe;
        opts.ctas = t.ctas;
    };
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = cache.find(key);
        if (it != cache.end()) {
            apply(it->second);
            return;
        }
    }
    cudaEvent_t e0, e1;
    CMG_CUDA(cudaEventCreate(&e0));
    CMG_CUDA(cudaEventCreate(&e1));
    auto time_one = [&](const Tuned& t) {
        VoxOpts o = opts;
        o.brick = t.brick;
        o.grab = t.grab;
        o.walk_warps = t.walk_warps;
        o.probe = t.probe;
        o.ctas = t.ctas;
        o.autotune = false;
        Batch bt(meshes, o, stream);
        bt.run();  // sizing run (warms up as well)
        bt.synchronize();
        float best = 0.f;
        for (int r = 0; r < 2; ++r) {
            CMG_CUDA(cudaEventRecord(e0, stream));
            bt.run();
            CMG_CUDA(cudaEventRecord(e1, stream));
            CMG_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            CMG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (r == 0 || ms < best) best = ms;
        }
        return best;
    };
    Tuned cur{16, 1, 0, 0, 0};
    float cur_ms = time_one(cur);
    auto try_set = [&](Tuned t) {
        const float ms = time_one(t);
        if (ms < cur_ms) {
            cur = t;
            cur_ms = ms;
        }
    };
    try_set({16, 2, 0, 0, 0});
    try_set({8, 1, 0, 0, 0});
    const Tuned step1 = cur;
    for (int w : {1, 2, 4}) {
        Tuned t = step1;
        t.walk_warps = w;
        try_set(t);
    }
    if (cur.brick == 16) {
        if (sub_precision(opts) != kPrecFP64) {  // the FP32 pass's probe head
            const Tuned step2 = cur;
            for (int pr : {256, 512, 2048}) {
                Tuned t = step2;
                t.probe = pr;
                try_set(t);
            }
        }
        Tuned t = cur;
        t.ctas = 16;
        try_set(t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> g(mu);
    cache[key] = cur;
    apply(cur);
}

}  // namespace cmg::gpu
