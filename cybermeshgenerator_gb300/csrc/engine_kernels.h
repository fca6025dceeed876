// engine_kernels.h — host launchers of the device kernels (one per .cu file).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <utility>
#include <vector>

#include "cmg_types.h"
#include "host_mem.h"

namespace cmg::gpu {

// engine.cu: multiprocessors of the current device.
int device_sms();

// occupancy.cu
void launch_tri_prep(const MeshSeg* segs, int nseg, int64_t ntris, const double* pts,
                     const int* tris, double* soup, int4* xybox, int64_t* pairs, cudaStream_t st);
void launch_col_pairs(bool fill, const MeshSeg* segs, int nseg, int64_t ntris, const int4* xybox,
                      const int64_t* pair_off, int* colcnt, const int64_t* col_off, int* col_list,
                      int grid, cudaStream_t st);
void launch_occ_filter(int mode, const MeshSeg* segs, int nseg, int64_t nrows, const double* soup,
                       const int64_t* col_off, const int* col_list, uint8_t* occ, int64_t* flagged,
                       Stats* stats, cudaStream_t st);
void launch_occ_exact(int mode, const MeshSeg* segs, int nseg, const double* soup,
                      const int64_t* col_off, const int* col_list, const int64_t* flagged,
                      double* hs, uint8_t* hv, uint8_t* occ, Stats* stats, int grid,
                      cudaStream_t st);
int occ_row_cols();

// sdf.cu
// trec: one kTriRecBytes-byte translation-invariant FP32 record per triangle (sdf::TriRec,
// the triangle in its own frame).
constexpr size_t kTriRecBytes = 96;
void launch_sdf_tri_prep(const MeshSeg* segs, int nseg, int64_t ntris, const double* soup,
                         float4* tinfo, float4* tinfo_lo, void* trec, float4* tnorm, float4* tlo,
                         float4* thi,
                         int64_t* tbin, int* bincnt, int* large_cnt, unsigned* emax_bits,
                         cudaStream_t st);
void launch_bin_fill(int64_t ntris, const int64_t* tbin, const int64_t* bin_off, int* bincur,
                     int* bin_list, const MeshSeg* segs, int nseg, int* large_cur, int* large_list,
                     cudaStream_t st);
void launch_seg_finish(MeshSeg* segs, int nseg, const int64_t* large_off, const unsigned* emax_bits,
                       cudaStream_t st);
void launch_brick_walk(bool fill, const MeshSeg* segs, int nseg, int64_t nbricks, const double* soup,
                       const float4* tinfo, const float4* tlo, const float4* thi,
                       const int64_t* bin_off, const int* bin_list, const int* large_list,
                       float* bound, int* cand_cnt, const int64_t* cand_off, int* cand,
                       float* brick_emax, Stats* stats, int walk_warps, cudaStream_t st);
// Warps per brick the walk uses: walk_warps when it is 1, 2 or 4, else by the brick
// count (4 while 4-warp bricks fit about twice in the GPU, 2 up to twice that, then 1).
int brick_walk_warps(int64_t nbricks, int walk_warps);
void launch_count_K(int brick, const MeshSeg* segs, int nseg, int64_t nbricks, const float4* tinfo,
                    const int64_t* cand_off, const int* cand, const double* sdf64,
                    const float* sdf32, float band_cells, unsigned long long* out,
                    cudaStream_t st);
void launch_work_keys(const int* cand_cnt, int64_t n, uint32_t* keys, uint32_t* vals,
                      cudaStream_t st);
void launch_sdf_eval(int precision, int brick, const MeshSeg* segs, int nseg, const uint32_t* work,
                     int64_t nwork, unsigned long long* queue, const double* soup,
                     const float4* tinfo, const int64_t* cand_off, const int* cand,
                     const float* brick_emax, float band_cells, const uint8_t* occ, float* sdf32,
                     double* sdf64, int* near_tri, uint8_t* near_reg, float* errbound, Stats* stats,
                     int grid, cudaStream_t st);

// sdf_sub.cu: evaluation by 4^3 sub-bricks of 16^3 candidate bricks.
void launch_sub_work_keys(const int* cand_cnt, int64_t nbricks, uint32_t* keys, uint32_t* vals,
                          cudaStream_t st);
// ctas: resident CTAs per SM of the evaluation kernel (16, or 12 for any other value);
// probe: brick-list head scanned by the mixed probe (<= 0: the default).
int sdf_sub_minb(int ctas);
int sdf_sub_grid(int precision, bool stage, int ctas);
void launch_sdf_sub(int precision, bool stage, int grab, int probe, int ctas, const MeshSeg* segs,
                    int nseg, const uint32_t* work, int64_t nwork, unsigned long long* queue,
                    const double* soup, const float4* tinfo, const float4* tinfo_lo, const void* trec,
                    const float4* tnorm, const int64_t* cand_off, const int* cand, const float* brick_emax,
                    float band_cells, const uint8_t* occ, float* sdf32, double* sdf64,
                    int* near_tri, uint8_t* near_reg, float* errbound, Stats* stats, int grid,
                    cudaStream_t st);

// adjoint.cu: dL/d(points) of the signed distance from the nearest-feature
// checkpoint, per-cell terms in FP64 (kPrecFP64) or FP32 on triangle-recentred
// coordinates (kPrecMixed), sums in FP64 in a fixed order. voff (npts+1) / vinc: per
// point, its (3 * triangle + corner) entries in ascending order. grad (3*npts
// doubles) is overwritten; tmp holds adjoint_tmp_bytes(ncell, ntris). Synchronises
// the stream once (the number of runs sizes the sort).
size_t adjoint_tmp_bytes(int64_t ncell, int64_t ntris);
void adjoint_backward(int precision, const GridDesc& g, int64_t ncell, const double* pts,
                      int64_t npts, const int* tris, int64_t ntris, const int* near_tri,
                      const uint8_t* near_reg, const uint8_t* occ, const double* grad_sdf,
                      const int64_t* voff, const int* vinc, double* grad, void* tmp,
                      cudaStream_t st);

// stl.cu: an STL image (host bytes) -> merged points (3 doubles each, first-occurrence
// order) and triangles (3 indices each), as the reference's read_stl; throws
// std::invalid_argument with its messages.
void stl_read(const char* bytes, size_t len, HostVec<double>& pts, HostVec<int>& tris,
              cudaStream_t st);
// Phase times of the last stl_read on this device (CUDA events): upload of the
// records (or parsed coordinates), decode + merge kernels, download of the arrays.
void stl_last_timing(float* upload_ms, float* merge_ms, float* download_ms);

// detect.cu: the pairs (i, j), i < j, of fan triangles of the facets (host CSR:
// facet f's polygon is fidx[foff[f] .. foff[f+1]); a triangle with an index outside
// [0, npts) is skipped) that share no vertex index and cross, in (i, j) order, as the
// reference's self_intersections; rows gets 8 ints per pair: facet_a, facet_b,
// triangle a's corners, triangle b's.
void self_intersections(const double* pts, int64_t npts, const int* fidx, int64_t nidx,
                        const size_t* foff, int64_t nfacets, std::vector<int>& rows,
                        cudaStream_t st);
// Device time (CUDA events) of the last call's boxes, binning and pair tests.
float self_intersections_last_ms();

// simplify.cu: grid vertex clustering of the points and the fan triangles of the
// facets (fidx / foff: facet f's polygon is fidx[foff[f] .. foff[f+1]), nfacets + 1
// offsets), as the reference's cmg::simplify::simplify. Throws std::invalid_argument
// with the reference's message on invalid input.
void simplify(const double* pts, int64_t npts, const int* fidx, int64_t nidx, const size_t* foff,
              int64_t nfacets, int grid, HostVec<double>& out_pts, HostVec<int>& out_tris,
              cudaStream_t st);
// Device times of the last simplify: host-to-device copy, clustering, device-to-host copy.
void simplify_last_timing(float* upload_ms, float* cluster_ms, float* download_ms);

// sizing.cu: the background sizing field (cmg::sizing::from_background) as a device
// object evaluated for batches of queries with the reference's results bit for bit.
struct SizingField;
struct SizingStats {
    int64_t binned_pairs = 0, global_tets = 0, far_tets = 0;  // construction
    int64_t inside = 0, nearest = 0, slow = 0;           // last evaluation: answers by kind
    int64_t tests = 0, candidates = 0;                   // full tests, candidates seen
    float upload_ms = 0.f, eval_ms = 0.f, download_ms = 0.f;  // last host evaluation
};
// Throws std::invalid_argument on a non-finite node or an index outside the nodes.
SizingField* sizing_create(const double* pts, int64_t np, const int* tets, int64_t nt,
                           const double* sizes, int64_t ns, double scale, cudaStream_t st);
void sizing_destroy(SizingField* f);
// q: 3 n device doubles; out: n device doubles; which (may be null): the answering
// tetrahedron per query, or -1 for the nearest node. Asynchronous on st.
void sizing_eval_device(SizingField* f, const double* q, int64_t n, double* out, int* which,
                        cudaStream_t st);
// Host arrays: copies in, evaluates, copies out (synchronous).
void sizing_eval_host(SizingField* f, const double* q, int64_t n, double* out, int* which,
                      cudaStream_t st);
SizingStats sizing_stats(SizingField* f, cudaStream_t st);
// robust::orient3d_batch (host arrays, synchronous): the orient3d value of each of n
// candidate tetrahedra (4 indices into pts each).
void orient3d_batch(const double* pts, int64_t np, const int* tets, int64_t n, double* out,
                    cudaStream_t st);

// peak.cu: FMA throughput (FLOP/s, FMA = 2) of the current device.
double peak_flops(bool fp64);

}  // namespace cmg::gpu
