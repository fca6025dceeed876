// cmg_c.cpp — the C ABI of libcmg_c.so (include/cmg_c/cmg_c.h, cmg_gpu.h).
//
// Handle, status and error-buffer conventions follow the reference's C shim
// (bindings/c/src/cmg_c.cpp): NULL handles and arguments answer
// CMG_ERR_INVALID_INPUT, core validation errors carry the core's message, and
// every C++ exception is caught at the boundary as CMG_ERR_INTERNAL. The
// voxelization itself runs on the GPU (engine.h); there is no CPU path, and a
// host without a CUDA device gets CMG_ERR_INTERNAL with the CUDA error text.
//
// Compile with -ffp-contract=off: make_grid must round like the reference.
#include "../../include/cmg_c/cmg_c.h"
#include "../../include/cmg_c/cmg_gpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <climits>
#include <cmath>
#include <cstring>
#include <exception>
#include <fstream>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "cmg_util.h"
#include "engine.h"
#include "engine_kernels.h"

namespace {

using cmg::gpu::GridDesc;

struct Region {
    double x, y, z, attribute, max_volume;
};

}  // namespace

// Large arrays in pooled page-locked host memory (cmg::gpu::HostVec): the device
// reads and fills them without staging or first-touch faults.
struct cmg_plc {
    cmg::gpu::HostVec<double> points;      // 3 per point
    cmg::gpu::HostVec<int> fidx;           // facet polygons, concatenated
    cmg::gpu::HostVec<size_t> foff{0};     // facet f is fidx[foff[f] .. foff[f+1])
    cmg::gpu::HostVec<int> markers;
    std::vector<double> holes;
    std::vector<Region> regions;
    cmg::gpu::HostVec<double> pts_cache;
    cmg::gpu::HostVec<int> tri_cache;
};

struct cmg_options {
    int plc = 0;
    double max_volume = -1.0;
    double radius_edge = 0.0, min_dihedral = 0.0;
    int quality = 0;
    int preserve_edges = 0;
};

struct cmg_mesh {};

struct cmg_voxels {
    double corner[3] = {0, 0, 0};
    double origin[3] = {0, 0, 0};
    double spacing = 0;
    int nx = 0, ny = 0, nz = 0;   // nz: the layers held (the slab's)
    int z0 = 0, z1 = 0, nz_grid = 0;  // the slab [z0, z1) of the grid's nz_grid layers
    cmg::gpu::HostResult r;
    cmg_voxel_stats stats{};
};

struct cmg_batch {
    std::unique_ptr<cmg::gpu::Batch> batch;
    std::vector<GridDesc> grids;
    int outputs = 0;
    bool ran = false;
};

struct cmg_intersections {
    std::vector<int> rows;  // 8 per crossing pair: facet_a, facet_b, tri_a[3], tri_b[3]
};

struct cmg_sdf_plan {
    std::unique_ptr<cmg::gpu::Batch> batch;
    GridDesc g{};
    int64_t npts = 0, ntris = 0, ncell = 0;
    int64_t* voff = nullptr;  // per point: its (3 * triangle + corner) entries, ascending
    int* vinc = nullptr;
    void* tmp = nullptr;      // adjoint workspace
    bool ran = false;
    ~cmg_sdf_plan() {
        if (voff) cudaFree(voff);
        if (vinc) cudaFree(vinc);
        if (tmp) cudaFree(tmp);
    }
};

namespace {

void set_err(char* buf, size_t len, const std::string& msg) {
    if (buf && len) {
        std::strncpy(buf, msg.c_str(), len - 1);
        buf[len - 1] = '\0';
    }
}

// The GPU entry points are serialised per device (one workspace pool and one library
// stream per device), on the calling thread's current device: calls on different
// devices run concurrently. Never throws (no current device: the first lock).
std::mutex& gpu_mutex() {
    constexpr int kMaxDevices = 64;
    static std::mutex m[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        dev = 0;
    }
    return m[dev >= 0 && dev < kMaxDevices ? dev : 0];
}

// The library's own stream on the current device, created on first use and kept
// for the life of the process (one per device ordinal).
cudaStream_t gpu_stream() {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static cudaStream_t streams[kMaxDevices] = {};
    int dev = 0;
    CMG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("device ordinal out of range");
    std::lock_guard<std::mutex> g(mu);
    if (!streams[dev]) CMG_CUDA(cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking));
    return streams[dev];
}

// Fan triangulation (v0, v[i-1], v[i]) of every facet polygon
// (src/voxelize/voxelize.cpp:29-38).
cmg::gpu::HostVec<int> fan(const cmg_plc& p) {
    const size_t nf = p.foff.size() - 1;
    size_t total = 0;
    bool all3 = true;
    for (size_t f = 0; f < nf; ++f) {
        const size_t n = p.foff[f + 1] - p.foff[f];
        total += n >= 3 ? 3 * (n - 2) : 0;
        all3 = all3 && n == 3;
    }
    cmg::gpu::HostVec<int> t(total);
    if (total == 0) return t;
    if (all3 && total == p.fidx.size()) {  // every facet a triangle: as stored
        std::memcpy(t.data(), p.fidx.data(), sizeof(int) * total);
        return t;
    }
    size_t o = 0;
    for (size_t f = 0; f < nf; ++f) {
        const int* v = p.fidx.data() + p.foff[f];
        const size_t n = p.foff[f + 1] - p.foff[f];
        for (size_t i = 2; i < n; ++i) {
            t[o++] = v[0];
            t[o++] = v[i - 1];
            t[o++] = v[i];
        }
    }
    return t;
}

// make_grid (src/voxelize/voxelize.cpp:52-74), same operations in the same order;
// pts holds n points of 3 coordinates (n >= 1).
bool make_grid(const double* pts, size_t n, int resolution, int pad, GridDesc& g) {
    double lo[3] = {pts[0], pts[1], pts[2]}, hi[3] = {pts[0], pts[1], pts[2]};
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            double v = pts[3 * i + a];
            if (v < lo[a]) lo[a] = v;
            if (v > hi[a]) hi[a] = v;
        }
    double ext = 0;
    for (int a = 0; a < 3; ++a) ext = std::max(ext, hi[a] - lo[a]);
    g = GridDesc{};
    g.h = ext / resolution;
    if (!(g.h > 0)) return false;
    int* dims[3] = {&g.nx, &g.ny, &g.nz};
    for (int a = 0; a < 3; ++a) {
        double e = hi[a] - lo[a];
        int core = std::max(1, static_cast<int>(std::ceil(e / g.h)));
        double covered = core * g.h;
        g.corner[a] = lo[a] - (covered - e) / 2.0 - pad * g.h;
        *dims[a] = core + 2 * pad;
    }
    return true;
}

struct CoreError {
    cmg_status code;
    std::string msg;
};

// Validation of voxelize (src/voxelize/voxelize.cpp:362-379) plus index checks
// (an out-of-range facet index is undefined behaviour in the reference; here it
// is an InvalidInput error, since the GPU must never read outside its inputs).
void check_mesh(int64_t npts, const int* tris, int64_t ntris) {
    if (npts == 0) throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: PLC has no points"};
    if (ntris == 0)
        throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: PLC has no boundary triangles"};
    for (int64_t i = 0; i < 3 * ntris; ++i)
        if (tris[i] < 0 || tris[i] >= npts)
            throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: facet vertex index out of range"};
}

cmg::gpu::HostVec<int> checked_triangles(const cmg_plc& p) {
    if (p.points.empty()) throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: PLC has no points"};
    cmg::gpu::HostVec<int> t = fan(p);
    check_mesh(static_cast<int64_t>(p.points.size() / 3), t.data(), static_cast<int64_t>(t.size() / 3));
    return t;
}

void check_grid_size(const GridDesc& g) {
    if (g.nx <= 0 || g.ny <= 0 || g.nz <= 0)
        throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: grid has no cells (pad too negative)"};
}

cmg::gpu::VoxOpts to_vox(const cmg_voxel_opts& o, int outputs) {
    cmg::gpu::VoxOpts v;
    v.predicates = o.predicates == CMG_PRED_EXACT ? cmg::gpu::kPredExact : cmg::gpu::kPredCompat;
    v.precision = o.precision == CMG_PREC_MIXED ? cmg::gpu::kPrecMixed : cmg::gpu::kPrecFP64;
    v.fp64_filter = o.precision != CMG_PREC_FP64_PLAIN;
    v.brick = o.brick;
    v.band = static_cast<float>(o.band);
    v.want_occ = outputs & CMG_OUT_OCCUPANCY;
    v.want_sdf32 = outputs & CMG_OUT_SDF_F32;
    v.want_sdf64 = outputs & CMG_OUT_SDF_F64;
    v.want_near = outputs & CMG_OUT_NEAREST;
    v.want_err = outputs & CMG_OUT_ERROR_BOUND;
    v.autotune = o.autotune != 0;
    v.grab = o.grab;
    v.stage = o.stage;
    v.walk_warps = o.walk_warps;
    v.probe = o.probe;
    v.ctas = o.ctas;
    return v;
}

int effective_outputs(const cmg_voxel_opts& o) {
    if (o.outputs) return o.outputs;
    return o.mode == 1 ? CMG_OUT_SDF_F32 : CMG_OUT_OCCUPANCY;
}

void fill_stats(cmg_voxels* v, const cmg::gpu::RunInfo& ri) {
    cmg_voxel_stats& s = v->stats;
    s.cells = ri.cells;
    s.flagged_columns = static_cast<int64_t>(ri.stats.flagged_columns);
    s.nudged_columns = static_cast<int64_t>(ri.stats.nudged_columns);
    s.exhausted_columns = static_cast<int64_t>(ri.stats.exhausted_columns);
    s.exact_calls = static_cast<int64_t>(ri.stats.exact_calls);
    s.bucket_entries = ri.pairs;
    s.candidates = ri.candidates;
    s.evaluations = static_cast<int64_t>(ri.stats.evaluations);
    s.fp64_evaluations = static_cast<int64_t>(ri.stats.fp64_evaluations);
    s.band_cells = static_cast<int64_t>(ri.stats.band_voxels);
    s.filtered = static_cast<int64_t>(ri.stats.filtered);
    s.brick = ri.brick;
    s.grab = ri.grab;
    s.walk_warps = ri.walk_warps;
    s.probe = ri.probe;
    s.ctas = ri.ctas;
    double m = 0;
    for (float e : v->r.err) m = std::max(m, static_cast<double>(e));
    s.max_error_bound = m;
}

// The handle's geometry: the grid's corner and origin (centre of cell (0,0,0) of the
// whole grid) and, along z, the layers held (a slab's, or all).
void set_geometry(cmg_voxels* v, const GridDesc& g) {
    for (int a = 0; a < 3; ++a) {
        v->corner[a] = g.corner[a];
        v->origin[a] = g.corner[a] + 0.5 * g.h;  // voxelize.cpp:389-391
    }
    v->spacing = g.h;
    v->nx = g.nx;
    v->ny = g.ny;
    v->z0 = g.z1 > 0 ? g.z0 : 0;
    v->z1 = g.z1 > 0 ? g.z1 : g.nz;
    v->nz_grid = g.nz;
    v->nz = v->z1 - v->z0;
}

// The cell layers [z_begin, z_end) of the options (z_end 0: through the last layer),
// checked against the grid's nz layers.
void set_layers(const cmg_voxel_opts& o, GridDesc& g) {
    const int z1 = o.z_end == 0 ? g.nz : o.z_end;
    if (o.z_begin < 0 || o.z_begin >= z1 || z1 > g.nz)
        throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: cell layers [z_begin, z_end) outside the grid"};
    g.z0 = o.z_begin;
    g.z1 = z1;
}

bool has_layers(const cmg_voxel_opts& o) { return o.z_begin != 0 || o.z_end != 0; }

// One voxelization of host arrays: pts (npts points of 3 coordinates), tris (ntris
// triangles of 3 indices, already fanned and checked).
cmg_voxels* voxelize_arrays(const double* pts, int64_t npts, const int* tris, int64_t ntris,
                            const cmg_voxel_opts& o) {
    GridDesc g{};
    if (o.explicit_grid) {
        for (int a = 0; a < 3; ++a) g.corner[a] = o.corner[a];
        g.h = o.spacing;
        g.nx = o.dims[0];
        g.ny = o.dims[1];
        g.nz = o.dims[2];
        if (!(g.h > 0)) throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: spacing must be > 0"};
    } else if (!make_grid(pts, static_cast<size_t>(npts), o.resolution, o.pad, g)) {
        throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: degenerate (zero-extent) PLC"};
    }
    check_grid_size(g);
    set_layers(o, g);
    const int outputs = effective_outputs(o);
    cmg::gpu::VoxOpts vo = to_vox(o, outputs);
    cmg::gpu::HostMesh m;
    m.pts = pts;
    m.npts = npts;
    m.tris = tris;
    m.ntris = ntris;
    m.g = g;
    std::lock_guard<std::mutex> lk(gpu_mutex());
    cudaStream_t st = gpu_stream();
    if (vo.autotune && vo.brick == 0) cmg::gpu::autotune({m}, vo, st);
    std::unique_ptr<cmg_voxels> v(new cmg_voxels);
    set_geometry(v.get(), g);
    cmg::gpu::Batch b({m}, vo, st, /*transient=*/true);
    b.run();
    std::vector<cmg::gpu::HostResult> res;
    cmg::gpu::RunInfo ri;
    b.download(res, &ri);
    v->r = std::move(res[0]);
    fill_stats(v.get(), ri);
    return v.release();
}

cmg_voxels* voxelize_one(const cmg_plc& p, const cmg_voxel_opts& o) {
    if (!o.explicit_grid && o.resolution < 1)
        throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: resolution must be >= 1"};
    cmg::gpu::HostVec<int> tris = checked_triangles(p);
    return voxelize_arrays(p.points.data(), static_cast<int64_t>(p.points.size() / 3), tris.data(),
                           static_cast<int64_t>(tris.size() / 3), o);
}

template <typename F>
cmg_status guarded(char* errbuf, size_t len, F&& f) {
    try {
        f();
        return CMG_OK;
    } catch (const CoreError& e) {
        set_err(errbuf, len, e.msg);
        return e.code;
    } catch (const std::invalid_argument& e) {
        set_err(errbuf, len, e.what());
        return CMG_ERR_INVALID_INPUT;
    } catch (const std::exception& e) {
        set_err(errbuf, len, e.what());
        return CMG_ERR_INTERNAL;
    } catch (...) {
        set_err(errbuf, len, "unknown error");
        return CMG_ERR_INTERNAL;
    }
}

const char* kNotHere = "not part of the GB300 voxelization library (meshing and file I/O stay in the reference)";

}  // namespace

namespace cmg::gpu {

// The core of cmg_plc_voxelize on host arrays, for the C++ surface (cmg_cpp.cpp):
// validation in the reference's order and with its messages, then the GPU pipeline.
// pts: npts points of 3 coordinates; tris: ntris fanned triangles. Returns the
// status; on success *out holds the grid, otherwise *msg the error text.
cmg_status voxelize_host(const double* pts, int64_t npts, const int* tris, int64_t ntris,
                         int resolution, int pad, int mode, cmg_voxels** out, std::string* msg) {
    *out = nullptr;
    char buf[512] = {0};
    const cmg_status st = guarded(buf, sizeof(buf), [&] {
        if (resolution < 1)
            throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: resolution must be >= 1"};
        check_mesh(npts, tris, ntris);
        cmg_voxel_opts o;
        cmg_voxel_opts_init(&o);
        o.resolution = resolution;
        o.pad = pad;
        o.mode = mode == 1 ? 1 : 0;
        *out = voxelize_arrays(pts, npts, tris, ntris, o);
    });
    if (st != CMG_OK) *msg = buf;
    return st;
}

}  // namespace cmg::gpu

namespace {
// Blocks handed out by cmg_host_alloc: capacity and whether page-locked.
struct HostBlocks {
    std::mutex mu;
    std::unordered_map<void*, std::pair<size_t, bool>> live;
};
HostBlocks& host_blocks() {
    static HostBlocks* h = new HostBlocks;  // outlives static teardown, like the pool
    return *h;
}
}  // namespace

extern "C" {

// ------------------------------------------------------------------ PLC
cmg_plc* cmg_plc_create(void) { return new (std::nothrow) cmg_plc{}; }
void cmg_plc_destroy(cmg_plc* p) { delete p; }

cmg_status cmg_plc_set_points(cmg_plc* plc, const double* xyz, size_t count) {
    if (!plc || (!xyz && count)) return CMG_ERR_INVALID_INPUT;
    try {
        plc->points.assign(xyz, xyz + 3 * count);
    } catch (...) {
        return CMG_ERR_INTERNAL;
    }
    return CMG_OK;
}

cmg_status cmg_plc_add_facet(cmg_plc* plc, const int* idx, size_t count, int marker) {
    if (!plc || (!idx && count)) return CMG_ERR_INVALID_INPUT;
    if (count < 3) return CMG_ERR_INVALID_INPUT;
    try {
        plc->fidx.insert(plc->fidx.end(), idx, idx + count);
        plc->foff.push_back(plc->fidx.size());
        plc->markers.push_back(marker);
    } catch (...) {
        return CMG_ERR_INTERNAL;
    }
    return CMG_OK;
}

cmg_status cmg_plc_add_triangles(cmg_plc* plc, const int* idx, size_t count, int marker) {
    if (!plc || (!idx && count)) return CMG_ERR_INVALID_INPUT;
    try {
        plc->fidx.insert(plc->fidx.end(), idx, idx + 3 * count);
        const size_t base = plc->foff.back();
        plc->foff.reserve(plc->foff.size() + count);
        for (size_t f = 1; f <= count; ++f) plc->foff.push_back(base + 3 * f);
        plc->markers.insert(plc->markers.end(), count, marker);
    } catch (...) {
        return CMG_ERR_INTERNAL;
    }
    return CMG_OK;
}

cmg_status cmg_plc_add_hole(cmg_plc* plc, double x, double y, double z) {
    if (!plc) return CMG_ERR_INVALID_INPUT;
    plc->holes.insert(plc->holes.end(), {x, y, z});
    return CMG_OK;
}

cmg_status cmg_plc_add_region(cmg_plc* plc, double x, double y, double z, double attribute,
                              double max_volume) {
    if (!plc) return CMG_ERR_INVALID_INPUT;
    plc->regions.push_back({x, y, z, attribute, max_volume});
    return CMG_OK;
}

size_t cmg_plc_num_points(const cmg_plc* p) { return p ? p->points.size() / 3 : 0; }

const double* cmg_plc_points(cmg_plc* p) {
    if (!p) return nullptr;
    p->pts_cache = p->points;
    return p->pts_cache.data();
}

size_t cmg_plc_num_triangles(cmg_plc* p) {
    if (!p) return 0;
    p->tri_cache = fan(*p);
    return p->tri_cache.size() / 3;
}

const int* cmg_plc_triangles(cmg_plc* p) {
    if (!p) return nullptr;
    p->tri_cache = fan(*p);
    return p->tri_cache.data();
}

// ------------------------------------------------------------------ voxelization
void cmg_voxel_opts_init(cmg_voxel_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->resolution = 64;
    o->pad = 1;
    o->precision = CMG_PREC_FP64;
    o->predicates = CMG_PRED_COMPAT;
    o->band = 1.0;
    o->stage = -1;
}

cmg_status cmg_plc_voxelize(const cmg_plc* in, int resolution, int mode, int pad,
                            cmg_voxels** out, char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if (!in || !out) return CMG_ERR_INVALID_INPUT;
    if (resolution < 1) {
        set_err(errbuf, len, "resolution must be >= 1");
        return CMG_ERR_INVALID_INPUT;
    }
    cmg_voxel_opts o;
    cmg_voxel_opts_init(&o);
    o.resolution = resolution;
    o.pad = pad;
    o.mode = mode == 1 ? 1 : 0;
    return guarded(errbuf, len, [&] { *out = voxelize_one(*in, o); });
}

cmg_status cmg_plc_voxelize_ex(const cmg_plc* in, const cmg_voxel_opts* opts, cmg_voxels** out,
                               char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if (!in || !out || !opts) return CMG_ERR_INVALID_INPUT;
    if (!opts->explicit_grid && opts->resolution < 1) {
        set_err(errbuf, len, "resolution must be >= 1");
        return CMG_ERR_INVALID_INPUT;
    }
    if (opts->brick != 0 && opts->brick != 4 && opts->brick != 8 && opts->brick != 16) {
        set_err(errbuf, len, "brick must be 0, 4, 8 or 16");
        return CMG_ERR_UNSUPPORTED_OPTION;
    }
    return guarded(errbuf, len, [&] { *out = voxelize_one(*in, *opts); });
}

void cmg_voxels_destroy(cmg_voxels* v) { delete v; }

void cmg_voxels_dims(const cmg_voxels* v, int* nx, int* ny, int* nz) {
    if (nx) *nx = v ? v->nx : 0;
    if (ny) *ny = v ? v->ny : 0;
    if (nz) *nz = v ? v->nz : 0;
}

void cmg_voxels_origin(const cmg_voxels* v, double* x, double* y, double* z) {
    if (x) *x = v ? v->origin[0] : 0.0;
    if (y) *y = v ? v->origin[1] : 0.0;
    if (z) *z = v ? v->origin[2] : 0.0;
}

void cmg_voxels_corner(const cmg_voxels* v, double* x, double* y, double* z) {
    if (x) *x = v ? v->corner[0] : 0.0;
    if (y) *y = v ? v->corner[1] : 0.0;
    if (z) *z = v ? v->corner[2] : 0.0;
}

cmg_status cmg_plc_grid(const cmg_plc* plc, int resolution, int pad, double* corner,
                        double* spacing, int* dims, char* errbuf, size_t len) {
    if (!plc || !corner || !spacing || !dims) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        if (resolution < 1)
            throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: resolution must be >= 1"};
        if (plc->points.empty())
            throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: PLC has no points"};
        GridDesc g{};
        if (!make_grid(plc->points.data(), plc->points.size() / 3, resolution, pad, g))
            throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: degenerate (zero-extent) PLC"};
        for (int a = 0; a < 3; ++a) corner[a] = g.corner[a];
        *spacing = g.h;
        dims[0] = g.nx;
        dims[1] = g.ny;
        dims[2] = g.nz;
    });
}

cmg_status cmg_debug_fail_device_allocs(int skip, int count) {
    if (skip < 0 || count < 0) return CMG_ERR_INVALID_INPUT;
    cmg::gpu::set_alloc_failures(skip, count);
    return CMG_OK;
}

void cmg_voxels_layers(const cmg_voxels* v, int* z_begin, int* z_end, int* nz_grid) {
    if (z_begin) *z_begin = v ? v->z0 : 0;
    if (z_end) *z_end = v ? v->z1 : 0;
    if (nz_grid) *nz_grid = v ? v->nz_grid : 0;
}

double cmg_voxels_spacing(const cmg_voxels* v) { return v ? v->spacing : 0.0; }

const unsigned char* cmg_voxels_occupancy(const cmg_voxels* v) {
    return (v && !v->r.occ.empty()) ? v->r.occ.data() : nullptr;
}
const float* cmg_voxels_distance(const cmg_voxels* v) {
    return (v && !v->r.sdf32.empty()) ? v->r.sdf32.data() : nullptr;
}
const double* cmg_voxels_distance_f64(const cmg_voxels* v) {
    return (v && !v->r.sdf64.empty()) ? v->r.sdf64.data() : nullptr;
}
const int* cmg_voxels_nearest_triangle(const cmg_voxels* v) {
    return (v && !v->r.near_tri.empty()) ? v->r.near_tri.data() : nullptr;
}
const unsigned char* cmg_voxels_nearest_region(const cmg_voxels* v) {
    return (v && !v->r.near_reg.empty()) ? v->r.near_reg.data() : nullptr;
}
const float* cmg_voxels_error_bound(const cmg_voxels* v) {
    return (v && !v->r.err.empty()) ? v->r.err.data() : nullptr;
}
void cmg_voxels_stats(const cmg_voxels* v, cmg_voxel_stats* out) {
    if (!out) return;
    if (!v) {
        std::memset(out, 0, sizeof(*out));
        return;
    }
    *out = v->stats;
}

// ------------------------------------------------------------------ batches
cmg_status cmg_batch_create(const cmg_plc* const* plcs, const int* resolutions, const int* pads,
                            int n, const cmg_voxel_opts* opts, cmg_batch** out, char* errbuf,
                            size_t len) {
    if (out) *out = nullptr;
    if (!plcs || !opts || !out || n < 1) return CMG_ERR_INVALID_INPUT;
    if (!opts->explicit_grid && (!resolutions || !pads)) return CMG_ERR_INVALID_INPUT;
    if (has_layers(*opts)) {
        set_err(errbuf, len, "cmg_batch_create: a batch is split by whole meshes, not by cell layers");
        return CMG_ERR_UNSUPPORTED_OPTION;
    }
    return guarded(errbuf, len, [&] {
        std::vector<cmg::gpu::HostVec<int>> tris(static_cast<size_t>(n));
        std::vector<cmg::gpu::HostMesh> meshes(static_cast<size_t>(n));
        std::unique_ptr<cmg_batch> b(new cmg_batch);
        for (int i = 0; i < n; ++i) {
            if (!plcs[i]) throw CoreError{CMG_ERR_INVALID_INPUT, "cmg_batch_create: NULL plc"};
            const cmg_plc& p = *plcs[i];
            tris[i] = checked_triangles(p);
            GridDesc g{};
            if (opts->explicit_grid) {
                for (int a = 0; a < 3; ++a) g.corner[a] = opts->corner[a];
                g.h = opts->spacing;
                g.nx = opts->dims[0];
                g.ny = opts->dims[1];
                g.nz = opts->dims[2];
            } else {
                if (resolutions[i] < 1)
                    throw CoreError{CMG_ERR_INVALID_INPUT, "resolution must be >= 1"};
                if (!make_grid(p.points.data(), p.points.size() / 3, resolutions[i], pads[i], g))
                    throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: degenerate (zero-extent) PLC"};
            }
            check_grid_size(g);
            meshes[i].pts = p.points.data();
            meshes[i].npts = static_cast<int64_t>(p.points.size() / 3);
            meshes[i].tris = tris[i].data();
            meshes[i].ntris = static_cast<int64_t>(tris[i].size() / 3);
            meshes[i].g = g;
            b->grids.push_back(g);
        }
        b->outputs = effective_outputs(*opts);
        cmg::gpu::VoxOpts vo = to_vox(*opts, b->outputs);
        std::lock_guard<std::mutex> lk(gpu_mutex());
        cudaStream_t st = gpu_stream();
        if (vo.autotune && vo.brick == 0) cmg::gpu::autotune(meshes, vo, st);
        b->batch.reset(new cmg::gpu::Batch(meshes, vo, st, /*transient=*/false));
        *out = b.release();
    });
}

cmg_status cmg_batch_run(cmg_batch* b, int use_graph, char* errbuf, size_t len) {
    if (!b) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        if (use_graph) b->batch->run_graph();
        else b->batch->run();
        b->ran = true;
    });
}

cmg_status cmg_batch_sync(cmg_batch* b, char* errbuf, size_t len) {
    if (!b) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] { b->batch->synchronize(); });
}

cmg_status cmg_batch_get(cmg_batch* b, int i, cmg_voxels** out, char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if (!b || !out || i < 0 || i >= b->batch->nmeshes()) return CMG_ERR_INVALID_INPUT;
    if (!b->ran) {
        set_err(errbuf, len, "cmg_batch_get: the batch has not run");
        return CMG_ERR_INVALID_INPUT;
    }
    return guarded(errbuf, len, [&] {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        std::unique_ptr<cmg_voxels> v(new cmg_voxels);
        set_geometry(v.get(), b->grids[static_cast<size_t>(i)]);
        b->batch->download_one(i, v->r);
        fill_stats(v.get(), b->batch->info());
        v->stats.cells = static_cast<int64_t>(v->nx) * v->ny * v->nz;
        *out = v.release();
    });
}

int cmg_batch_size(const cmg_batch* b) { return b ? b->batch->nmeshes() : 0; }
int64_t cmg_batch_cells(const cmg_batch* b) { return b ? b->batch->total_cells() : 0; }
void cmg_batch_destroy(cmg_batch* b) {
    if (!b) return;
    std::lock_guard<std::mutex> lk(gpu_mutex());
    delete b;
}

void* cmg_batch_stream(const cmg_batch* b) { return b ? static_cast<void*>(b->batch->stream()) : nullptr; }

cmg_status cmg_batch_set_timing(cmg_batch* b, int on) {
    if (!b) return CMG_ERR_INVALID_INPUT;
    b->batch->set_timing(on != 0);
    return CMG_OK;
}

cmg_status cmg_batch_get_timing(cmg_batch* b, cmg_batch_timing* out, char* errbuf, size_t len) {
    if (!b || !out) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        cmg::gpu::Timing t = b->batch->timing();
        out->occupancy_ms = t.occupancy_ms;
        out->sdf_prep_ms = t.sdf_prep_ms;
        out->eval_ms = t.eval_ms;
        out->total_ms = t.total_ms;
    });
}

cmg_status cmg_batch_work_model(cmg_batch* b, cmg_work_model* out, char* errbuf, size_t len) {
    if (!b || !out) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        cmg::gpu::WorkModel w = b->batch->work_model();
        out->sum_k = w.sum_k;
        out->sum_k_band = w.sum_k_band;
        out->band_cells = w.band_cells;
        out->orient_calls = w.orient_calls;
        out->crossings = w.crossings;
    });
}

cmg_status cmg_batch_stats(cmg_batch* b, cmg_voxel_stats* out, char* errbuf, size_t len) {
    if (!b || !out) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        cmg_voxels v;
        fill_stats(&v, b->batch->info());
        *out = v.stats;
        out->cells = b->batch->total_cells();
    });
}

// ------------------------------------------------------------------ SDF plan (adjoint)
cmg_status cmg_sdf_plan_create(const double* points, int64_t npoints, const int* triangles,
                               int64_t ntriangles, const cmg_voxel_opts* opts, cmg_sdf_plan** out,
                               char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if (!points || !triangles || !opts || !out || npoints < 1 || ntriangles < 1)
        return CMG_ERR_INVALID_INPUT;
    if (has_layers(*opts)) {
        set_err(errbuf, len, "cmg_sdf_plan_create: a plan holds the whole grid (no cell layers)");
        return CMG_ERR_UNSUPPORTED_OPTION;
    }
    return guarded(errbuf, len, [&] {
        if (!opts->explicit_grid)
            throw CoreError{CMG_ERR_INVALID_INPUT, "cmg_sdf_plan_create: an explicit grid is required"};
        if (npoints > INT32_MAX || 3 * ntriangles > INT32_MAX)
            throw CoreError{CMG_ERR_INVALID_INPUT, "cmg_sdf_plan_create: mesh too large"};
        for (int64_t i = 0; i < 3 * ntriangles; ++i)
            if (triangles[i] < 0 || triangles[i] >= npoints)
                throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: facet vertex index out of range"};
        std::unique_ptr<cmg_sdf_plan> p(new cmg_sdf_plan);
        GridDesc g{};
        for (int a = 0; a < 3; ++a) g.corner[a] = opts->corner[a];
        g.h = opts->spacing;
        g.nx = opts->dims[0];
        g.ny = opts->dims[1];
        g.nz = opts->dims[2];
        if (!(g.h > 0)) throw CoreError{CMG_ERR_INVALID_INPUT, "voxelize: spacing must be > 0"};
        check_grid_size(g);
        p->g = g;
        p->npts = npoints;
        p->ntris = ntriangles;
        p->ncell = static_cast<int64_t>(g.nx) * g.ny * g.nz;
        if (p->ncell >= (int64_t(1) << 32))
            throw CoreError{CMG_ERR_INVALID_INPUT, "cmg_sdf_plan_create: grid too large"};
        cmg::gpu::VoxOpts vo =
            to_vox(*opts, CMG_OUT_OCCUPANCY | CMG_OUT_SDF_F64 | CMG_OUT_NEAREST);
        cmg::gpu::HostMesh m;
        m.pts = points;
        m.npts = npoints;
        m.tris = triangles;
        m.ntris = ntriangles;
        m.g = g;
        // the point -> (triangle, corner) incidence in a fixed order
        std::vector<int64_t> voff(static_cast<size_t>(npoints + 1), 0);
        for (int64_t i = 0; i < 3 * ntriangles; ++i) ++voff[static_cast<size_t>(triangles[i]) + 1];
        for (int64_t v = 0; v < npoints; ++v) voff[v + 1] += voff[v];
        std::vector<int64_t> cur(voff.begin(), voff.end() - 1);
        std::vector<int> vinc(static_cast<size_t>(3 * ntriangles));
        for (int64_t i = 0; i < 3 * ntriangles; ++i) vinc[cur[triangles[i]]++] = static_cast<int>(i);
        std::lock_guard<std::mutex> lk(gpu_mutex());
        cudaStream_t st = gpu_stream();
        if (vo.autotune && vo.brick == 0) cmg::gpu::autotune({m}, vo, st);
        p->batch.reset(new cmg::gpu::Batch({m}, vo, st, /*transient=*/false));
        CMG_CUDA(cmg::gpu::device_alloc(&p->voff, sizeof(int64_t) * voff.size()));
        CMG_CUDA(cmg::gpu::device_alloc(&p->vinc, sizeof(int) * vinc.size()));
        CMG_CUDA(cmg::gpu::device_alloc(&p->tmp, cmg::gpu::adjoint_tmp_bytes(p->ncell, ntriangles)));
        CMG_CUDA(cudaMemcpy(p->voff, voff.data(), sizeof(int64_t) * voff.size(), cudaMemcpyHostToDevice));
        CMG_CUDA(cudaMemcpy(p->vinc, vinc.data(), sizeof(int) * vinc.size(), cudaMemcpyHostToDevice));
        *out = p.release();
    });
}

cmg_status cmg_sdf_plan_forward(cmg_sdf_plan* p, const double* d_points, void* stream,
                                char* errbuf, size_t len) {
    if (!p) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the default stream
        p->batch->set_stream(st);
        if (d_points) p->batch->update_points_device(d_points);
        p->batch->run();
        p->ran = true;
    });
}

cmg_status cmg_sdf_plan_outputs(const cmg_sdf_plan* p, const unsigned char** d_occupancy,
                                const double** d_sdf, const int** d_nearest_triangle,
                                const unsigned char** d_nearest_region) {
    if (!p || !p->ran) return CMG_ERR_INVALID_INPUT;
    if (d_occupancy) *d_occupancy = p->batch->d_occ();
    if (d_sdf) *d_sdf = p->batch->d_sdf64();
    if (d_nearest_triangle) *d_nearest_triangle = p->batch->d_near_tri();
    if (d_nearest_region) *d_nearest_region = p->batch->d_near_reg();
    return CMG_OK;
}

int64_t cmg_sdf_plan_cells(const cmg_sdf_plan* p) { return p ? p->ncell : 0; }

cmg_status cmg_sdf_plan_copy_outputs(const cmg_sdf_plan* p, unsigned char* d_occupancy,
                                     double* d_sdf, int* d_nearest_triangle,
                                     unsigned char* d_nearest_region, void* stream, char* errbuf,
                                     size_t len) {
    if (!p || !p->ran) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the default stream
        const size_t n = static_cast<size_t>(p->ncell);
        const cmg::gpu::Batch& b = *p->batch;
        if (d_occupancy)
            CMG_CUDA(cudaMemcpyAsync(d_occupancy, b.d_occ(), n, cudaMemcpyDeviceToDevice, st));
        if (d_sdf)
            CMG_CUDA(cudaMemcpyAsync(d_sdf, b.d_sdf64(), 8 * n, cudaMemcpyDeviceToDevice, st));
        if (d_nearest_triangle)
            CMG_CUDA(cudaMemcpyAsync(d_nearest_triangle, b.d_near_tri(), 4 * n,
                                     cudaMemcpyDeviceToDevice, st));
        if (d_nearest_region)
            CMG_CUDA(cudaMemcpyAsync(d_nearest_region, b.d_near_reg(), n, cudaMemcpyDeviceToDevice,
                                     st));
    });
}

cmg_status cmg_sdf_plan_backward(cmg_sdf_plan* p, const double* d_points,
                                 const unsigned char* d_occupancy, const int* d_nearest_triangle,
                                 const unsigned char* d_nearest_region, const double* d_grad_sdf,
                                 double* d_grad_points, void* stream, char* errbuf, size_t len) {
    if (!p || !d_occupancy || !d_nearest_triangle || !d_nearest_region || !d_grad_sdf ||
        !d_grad_points)
        return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the default stream
        const double* pts = d_points ? d_points : p->batch->d_points();
        cmg::gpu::adjoint_backward(p->batch->opts().precision, p->g, p->ncell, pts, p->npts,
                                   p->batch->d_tris(), p->ntris,
                                   d_nearest_triangle, d_nearest_region, d_occupancy, d_grad_sdf,
                                   p->voff, p->vinc, d_grad_points, p->tmp, st);
    });
}

void cmg_sdf_plan_destroy(cmg_sdf_plan* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(gpu_mutex());
    delete p;
}

long long cmg_gpu_launches(void) { return cmg::gpu::launches(); }

cmg_status cmg_gpu_peak_flops(int fp64, double* flops, char* errbuf, size_t len) {
    if (!flops) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        *flops = cmg::gpu::peak_flops(fp64 != 0);
    });
}

const char* cmg_gpu_version(void) { return "cmg-gb300 0.1.0 sm_103a"; }

// ------------------------------------------------------------------ options
cmg_options* cmg_options_create(void) { return new (std::nothrow) cmg_options{}; }
void cmg_options_destroy(cmg_options* o) { delete o; }
cmg_status cmg_options_from_switches(cmg_options* o, const char* sw, char* errbuf, size_t len) {
    if (!o || !sw) return CMG_ERR_INVALID_INPUT;
    set_err(errbuf, len, kNotHere);
    return CMG_ERR_NOT_IMPLEMENTED;
}
cmg_status cmg_options_set_plc(cmg_options* o, int on) {
    if (!o) return CMG_ERR_INVALID_INPUT;
    o->plc = on != 0;
    return CMG_OK;
}
cmg_status cmg_options_set_max_volume(cmg_options* o, double v) {
    if (!o) return CMG_ERR_INVALID_INPUT;
    o->max_volume = v;
    return CMG_OK;
}
cmg_status cmg_options_set_quality(cmg_options* o, double radius_edge, double min_dihedral) {
    if (!o) return CMG_ERR_INVALID_INPUT;
    o->quality = 1;
    o->radius_edge = radius_edge;
    o->min_dihedral = min_dihedral;
    return CMG_OK;
}
cmg_status cmg_options_set_preserve_edges(cmg_options* o, int on) {
    if (!o) return CMG_ERR_INVALID_INPUT;
    o->preserve_edges = on != 0;
    return CMG_OK;
}

// ------------------------------------------------------------------ not in this library
void cmg_mesh_destroy(cmg_mesh* m) { delete m; }
cmg_status cmg_tetrahedralize(const cmg_plc* plc, const cmg_options* opts, cmg_mesh** out,
                              char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if (!plc || !opts || !out) return CMG_ERR_INVALID_INPUT;
    set_err(errbuf, len, kNotHere);
    return CMG_ERR_NOT_IMPLEMENTED;
}
cmg_status cmg_delaunay(const double* xyz, size_t count, const cmg_options* opts, cmg_mesh** out,
                        char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if ((!xyz && count) || !opts || !out) return CMG_ERR_INVALID_INPUT;
    set_err(errbuf, len, kNotHere);
    return CMG_ERR_NOT_IMPLEMENTED;
}
size_t cmg_mesh_num_points(const cmg_mesh*) { return 0; }
size_t cmg_mesh_num_tets(const cmg_mesh*) { return 0; }
size_t cmg_mesh_num_faces(const cmg_mesh*) { return 0; }
const double* cmg_mesh_points(const cmg_mesh*) { return nullptr; }
const int* cmg_mesh_tets(const cmg_mesh*) { return nullptr; }
const int* cmg_mesh_faces(const cmg_mesh*) { return nullptr; }
const int* cmg_mesh_tet_markers(const cmg_mesh*) { return nullptr; }
const int* cmg_mesh_face_markers(const cmg_mesh*) { return nullptr; }
// ------------------------------------------------------------------ self-intersections
cmg_status cmg_plc_self_intersections(const cmg_plc* plc, cmg_intersections** out, char* errbuf,
                                      size_t len) {
    if (out) *out = nullptr;
    if (!plc || !out) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        // fan triangles in facet order with their facet (src/detect/self_intersection.cpp:
        // 153-164), formed on the device from the facet offsets
        std::unique_ptr<cmg_intersections> r(new cmg_intersections);
        {
            std::lock_guard<std::mutex> lk(gpu_mutex());
            cmg::gpu::self_intersections(plc->points.data(),
                                         static_cast<int64_t>(plc->points.size() / 3),
                                         plc->fidx.data(), static_cast<int64_t>(plc->fidx.size()),
                                         plc->foff.data(), static_cast<int64_t>(plc->foff.size()) - 1,
                                         r->rows, gpu_stream());
        }
        *out = r.release();
    });
}
int64_t cmg_intersections_count(const cmg_intersections* r) {
    return r ? static_cast<int64_t>(r->rows.size() / 8) : 0;
}
const int* cmg_intersections_data(const cmg_intersections* r) {
    return (r && !r->rows.empty()) ? r->rows.data() : nullptr;
}
void cmg_intersections_destroy(cmg_intersections* r) { delete r; }
float cmg_self_intersections_last_ms(void) { return cmg::gpu::self_intersections_last_ms(); }

// The file extension, lower case (src/io/dispatch.cpp:19-26).
std::string lower_ext(const std::string& path) {
    const auto dot = path.rfind('.');
    if (dot == std::string::npos) return {};
    std::string e = path.substr(dot + 1);
    for (char& c : e) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return e;
}

cmg_plc* plc_from_stl(const char* bytes, size_t n) {
    cmg::gpu::HostVec<double> pts;
    cmg::gpu::HostVec<int> tris;
    {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        cmg::gpu::stl_read(bytes, n, pts, tris, gpu_stream());
    }
    std::unique_ptr<cmg_plc> p(new cmg_plc{});
    p->points = std::move(pts);
    const size_t nt = tris.size() / 3;
    p->fidx = std::move(tris);
    p->foff.resize(nt + 1);
    for (size_t f = 0; f <= nt; ++f) p->foff[f] = 3 * f;
    p->markers.assign(nt, 0);
    return p.release();
}

cmg_status cmg_plc_from_stl(const void* data, size_t n, cmg_plc** out, char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if ((!data && n) || !out) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] { *out = plc_from_stl(static_cast<const char*>(data), n); });
}

cmg_status cmg_stl_last_timing(float* upload_ms, float* merge_ms, float* download_ms) {
    if (!upload_ms || !merge_ms || !download_ms) return CMG_ERR_INVALID_INPUT;
    try {
        cmg::gpu::stl_last_timing(upload_ms, merge_ms, download_ms);
    } catch (...) {
        return CMG_ERR_INTERNAL;
    }
    return CMG_OK;
}

// read_plc (src/io/dispatch.cpp:64-74): .stl through the GPU reader; the other formats
// the reference reads are outside this library; anything else is unsupported.
cmg_status cmg_read_plc(const char* path, cmg_plc** out, char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if (!path || !out) return CMG_ERR_INVALID_INPUT;
    const std::string p(path), e = lower_ext(p);
    if (e == "poly" || e == "smesh" || e == "off" || e == "ply" || e == "obj") {
        set_err(errbuf, len, kNotHere);
        return CMG_ERR_NOT_IMPLEMENTED;
    }
    if (e != "stl") {
        set_err(errbuf, len, "unsupported file format for " + p);
        return CMG_ERR_INVALID_INPUT;
    }
    return guarded(errbuf, len, [&] {
        std::ifstream in(p, std::ios::binary | std::ios::ate);
        if (!in) throw CoreError{CMG_ERR_INVALID_INPUT, "cannot open file for reading: " + p};
        const std::streamoff sz = in.tellg();
        if (sz < 0) throw CoreError{CMG_ERR_INVALID_INPUT, "cannot open file for reading: " + p};
        std::vector<char> buf(static_cast<size_t>(sz));
        in.seekg(0);
        if (sz > 0) in.read(buf.data(), sz);
        *out = plc_from_stl(buf.data(), buf.size());
    });
}
cmg_status cmg_read_points(const char* path, cmg_plc** out, char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if (!path || !out) return CMG_ERR_INVALID_INPUT;
    set_err(errbuf, len, kNotHere);
    return CMG_ERR_NOT_IMPLEMENTED;
}
cmg_status cmg_read_mesh(const char* path, cmg_mesh** out, char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if (!path || !out) return CMG_ERR_INVALID_INPUT;
    set_err(errbuf, len, kNotHere);
    return CMG_ERR_NOT_IMPLEMENTED;
}
cmg_status cmg_write_mesh(const char* path, const cmg_mesh* m, char* errbuf, size_t len) {
    if (!path || !m) return CMG_ERR_INVALID_INPUT;
    set_err(errbuf, len, kNotHere);
    return CMG_ERR_NOT_IMPLEMENTED;
}
cmg_status cmg_write_plc(const char* path, const cmg_plc* p, char* errbuf, size_t len) {
    if (!path || !p) return CMG_ERR_INVALID_INPUT;
    set_err(errbuf, len, kNotHere);
    return CMG_ERR_NOT_IMPLEMENTED;
}
// simplify (src/simplify/simplify.cpp:48-112) on the GPU: the result holds the
// representative points and one single-triangle facet (marker 0) per kept triangle,
// with no holes or regions, as the reference's.
cmg_status cmg_plc_simplify(const cmg_plc* in, int grid, cmg_plc** out, char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if (!in || !out) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        // simplify.cpp:49-54, answered before any device is touched
        if (in->points.empty()) throw CoreError{CMG_ERR_INVALID_INPUT, "simplify: PLC has no points"};
        if (grid < 1) throw CoreError{CMG_ERR_INVALID_INPUT, "simplify: grid must be >= 1"};
        cmg::gpu::HostVec<double> pts;
        cmg::gpu::HostVec<int> tris;
        {
            std::lock_guard<std::mutex> lk(gpu_mutex());
            cmg::gpu::simplify(in->points.data(), static_cast<int64_t>(in->points.size() / 3),
                               in->fidx.data(), static_cast<int64_t>(in->fidx.size()),
                               in->foff.data(), static_cast<int64_t>(in->foff.size()) - 1, grid, pts,
                               tris, gpu_stream());
        }
        std::unique_ptr<cmg_plc> p(new cmg_plc{});
        p->points = std::move(pts);
        const size_t nt = tris.size() / 3;
        p->fidx = std::move(tris);
        p->foff.resize(nt + 1);
        for (size_t f = 0; f <= nt; ++f) p->foff[f] = 3 * f;
        p->markers.assign(nt, 0);
        *out = p.release();
    });
}

cmg_status cmg_simplify_last_timing(float* upload_ms, float* cluster_ms, float* download_ms) {
    if (!upload_ms || !cluster_ms || !download_ms) return CMG_ERR_INVALID_INPUT;
    try {
        cmg::gpu::simplify_last_timing(upload_ms, cluster_ms, download_ms);
    } catch (...) {
        return CMG_ERR_INTERNAL;
    }
    return CMG_OK;
}

// ------------------------------------------------------------------ sizing field
struct cmg_sizing {
    cmg::gpu::SizingField* f = nullptr;
    ~cmg_sizing() {
        if (f) cmg::gpu::sizing_destroy(f);
    }
};

// from_background (src/sizing/background.cpp:58-74): the closure's data moved to the
// device once; evaluations run in batches.
cmg_status cmg_sizing_create(const double* points, int64_t npoints, const int* tets, int64_t ntets,
                             const double* node_sizes, int64_t nsizes, double scale,
                             cmg_sizing** out, char* errbuf, size_t len) {
    if (out) *out = nullptr;
    if (!out || npoints < 0 || ntets < 0 || nsizes < 0 || (npoints && !points) ||
        (ntets && !tets) || (nsizes && !node_sizes))
        return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        // inputs whose behaviour is undefined in the reference, refused before any device work
        for (int64_t i = 0; i < 3 * npoints; ++i)
            if (!std::isfinite(points[i]))
                throw CoreError{CMG_ERR_INVALID_INPUT, "sizing: non-finite background point"};
        for (int64_t k = 0; k < 4 * ntets; ++k)
            if (tets[k] < 0 || tets[k] >= npoints)
                throw CoreError{CMG_ERR_INVALID_INPUT, "sizing: tetrahedron vertex index out of range"};
        std::unique_ptr<cmg_sizing> s(new cmg_sizing);
        std::lock_guard<std::mutex> lk(gpu_mutex());
        s->f = cmg::gpu::sizing_create(points, npoints, tets, ntets, node_sizes, nsizes, scale,
                                       gpu_stream());
        *out = s.release();
    });
}

cmg_status cmg_sizing_eval(cmg_sizing* s, const double* queries, int64_t n, double* out, int* which,
                           char* errbuf, size_t len) {
    if (!s || n < 0 || (n && (!queries || !out))) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        cmg::gpu::sizing_eval_host(s->f, queries, n, out, which, gpu_stream());
    });
}

cmg_status cmg_sizing_eval_device(cmg_sizing* s, const double* d_queries, int64_t n, double* d_out,
                                  int* d_which, void* stream, char* errbuf, size_t len) {
    if (!s || n < 0 || (n && (!d_queries || !d_out))) return CMG_ERR_INVALID_INPUT;
    return guarded(errbuf, len, [&] {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        cmg::gpu::sizing_eval_device(s->f, d_queries, n, d_out, d_which,
                                     static_cast<cudaStream_t>(stream));  // NULL: the default stream
    });
}

cmg_status cmg_sizing_get_stats(cmg_sizing* s, cmg_sizing_stats* out) {
    if (!s || !out) return CMG_ERR_INVALID_INPUT;
    try {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        const cmg::gpu::SizingStats r = cmg::gpu::sizing_stats(s->f, gpu_stream());
        out->binned_pairs = r.binned_pairs;
        out->global_tets = r.global_tets;
        out->far_tets = r.far_tets;
        out->inside = r.inside;
        out->nearest = r.nearest;
        out->slow = r.slow;
        out->tests = r.tests;
        out->candidates = r.candidates;
        out->upload_ms = r.upload_ms;
        out->eval_ms = r.eval_ms;
        out->download_ms = r.download_ms;
    } catch (...) {
        return CMG_ERR_INTERNAL;
    }
    return CMG_OK;
}

void cmg_sizing_destroy(cmg_sizing* s) { delete s; }

cmg_status cmg_orient3d_batch(const double* xyz, int npts, const int* tets, int n, double* out_value) {
    if (n <= 0) return CMG_OK;
    if (!xyz || !tets || !out_value || npts <= 0) return CMG_ERR_INVALID_INPUT;
    for (int64_t i = 0; i < 4 * static_cast<int64_t>(n); ++i)
        if (tets[i] < 0 || tets[i] >= npts) return CMG_ERR_INVALID_INPUT;
    try {
        std::lock_guard<std::mutex> lk(gpu_mutex());
        cmg::gpu::orient3d_batch(xyz, npts, tets, n, out_value, gpu_stream());
    } catch (...) {
        return CMG_ERR_INTERNAL;
    }
    return CMG_OK;
}

void* cmg_host_alloc(size_t bytes) {
    try {
        size_t cap = 0;
        bool pinned = false;
        void* p = cmg::gpu::host_block_acquire(bytes ? bytes : 1, &cap, &pinned);
        std::lock_guard<std::mutex> lk(host_blocks().mu);
        host_blocks().live[p] = {cap, pinned};
        return p;
    } catch (...) {
        return nullptr;
    }
}

void cmg_host_free(void* p) {
    if (!p) return;
    HostBlocks& H = host_blocks();
    std::pair<size_t, bool> b;
    {
        std::lock_guard<std::mutex> lk(H.mu);
        auto it = H.live.find(p);
        if (it == H.live.end()) return;
        b = it->second;
        H.live.erase(it);
    }
    cmg::gpu::host_block_release(p, b.first, b.second);
}

const char* cmg_version(void) { return "0.5.0"; }

}  // extern "C"
