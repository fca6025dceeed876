/* cmg_gpu.h — GB300 additions to the reference C ABI (libcmg_c.so).
 *
 * None of these has a counterpart in the reference's bindings/c/include/cmg_c/
 * cmg_c.h; they expose what the GPU path adds: an explicit grid, the FP64 and
 * mixed-precision distance fields, exact-predicate occupancy, the nearest-feature
 * checkpoint used by the adjoint, run statistics, and batches of meshes.
 * cmg_plc_voxelize (cmg_c.h) keeps the reference's semantics exactly.
 */
#ifndef CMG_GPU_H
#define CMG_GPU_H

#include <stddef.h>
#include <stdint.h>

#include "cmg_c.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Output selection bits for cmg_voxel_opts.outputs. */
#define CMG_OUT_OCCUPANCY 1   /* uint8 occupancy */
#define CMG_OUT_SDF_F32 2     /* float signed distance (the reference's output) */
#define CMG_OUT_SDF_F64 4     /* double signed distance (before the float cast) */
#define CMG_OUT_NEAREST 8     /* nearest triangle id (int) + Ericson region (uint8) */
#define CMG_OUT_ERROR_BOUND 16 /* mixed precision: stated per-cell bound (float) */

/* Distance arithmetic. */
#define CMG_PREC_FP64 0   /* FP64 distances in the reference's operation order,
                             bit-identical to the reference: on 16^3 bricks an FP32 pass
                             with a stated error bound finds each cell's near-ties, whose
                             FP64 distances give the FP64 minimum */
#define CMG_PREC_MIXED 1  /* FP32 on brick-recentred coordinates + FP64 band */
#define CMG_PREC_FP64_PLAIN 2 /* the same results as CMG_PREC_FP64 with every
                                 candidate evaluated in FP64 (for comparison) */

/* Predicate semantics for occupancy. */
#define CMG_PRED_COMPAT 0 /* the reference as initialised: sign of the rounded
                             determinant unless it is exactly zero */
#define CMG_PRED_EXACT 1  /* sign of the exact determinant */

typedef struct cmg_voxel_opts {
    int resolution;      /* cells along the longest bbox axis (>= 1), as cmg_plc_voxelize */
    int pad;             /* margin cells per side */
    int mode;            /* 0 occupancy, 1 signed distance: the outputs when outputs == 0 */
    int outputs;         /* CMG_OUT_* bits; 0 = as `mode` selects */
    int precision;       /* CMG_PREC_* */
    int predicates;      /* CMG_PRED_* */
    int explicit_grid;   /* nonzero: corner/spacing/dims replace resolution/pad */
    double corner[3];    /* min corner of cell (0,0,0) */
    double spacing;      /* cubic cell edge */
    int dims[3];         /* nx, ny, nz */
    double band;         /* mixed: FP64 refinement band around the surface, in cells */
    int brick;           /* SDF candidate brick edge: 0 = default (16, evaluated by 4^3
                            sub-bricks), 8 or 4 (one evaluation CTA per brick) */
    int autotune;        /* nonzero (with brick 0): time the brick edges, queue grab sizes,
                            walk warps, probe heads and evaluation CTAs per SM on this
                            input and keep the fastest */
    int grab;            /* sub-bricks taken per work-queue grab: 0 = default, 1, 2, 4, 8 */
    int stage;           /* mixed: 1 stage candidate records in shared memory, 0 read them
                            through L1/L2, -1 = default */
    int walk_warps;      /* warps per brick of the candidate walk: 1, 2 or 4; 0 = by the
                            brick count */
    int probe;           /* mixed: brick-list head the probe scans (entries); 0 = 1024 */
    int ctas;            /* evaluation CTAs per SM the registers are budgeted for: 16, or
                            0 / 12 = 12 */
    int z_begin, z_end;  /* cell layers [z_begin, z_end) of the grid to evaluate (a z-slab,
                            e.g. one rank's share); z_end 0 = through the last layer. The
                            slab's cells equal the whole grid's bit for bit (same centres,
                            occupancy columns through the whole grid); its outputs hold
                            those layers only. cmg_plc_voxelize_ex only. */
} cmg_voxel_opts;

/* Counters of one voxelization. */
typedef struct cmg_voxel_stats {
    int64_t cells;
    int64_t flagged_columns;   /* occupancy columns resolved by the exact pass */
    int64_t nudged_columns;    /* columns whose first attempt grazed an edge/vertex */
    int64_t exhausted_columns; /* columns where every nudge grazed (partial result kept) */
    int64_t exact_calls;       /* orient3d evaluations that needed exact arithmetic */
    int64_t bucket_entries;    /* (triangle, column) pairs */
    int64_t candidates;        /* (brick, triangle) SDF candidates */
    int64_t evaluations;       /* (cell, triangle) distance evaluations */
    int64_t fp64_evaluations;  /* of which in FP64 */
    int64_t band_cells;        /* mixed: cells refined in FP64 */
    int64_t filtered;          /* SDF: sub-brick candidate entries (each tested by 64 cells) */
    int brick;                 /* brick edge used */
    int grab;                  /* sub-bricks per work-queue grab used (16^3 bricks) */
    double max_error_bound;    /* mixed: largest stated per-cell bound (0 for FP64) */
    int walk_warps;            /* warps per brick of the candidate walk used */
    int probe;                 /* probe head used (mixed; 0 for FP64) */
    int ctas;                  /* evaluation CTAs per SM used (16^3 bricks) */
} cmg_voxel_stats;

/* Defaults: resolution 64, pad 1, occupancy, FP64, compat predicates, band 1. */
void cmg_voxel_opts_init(cmg_voxel_opts* opts);

/* Appends `count` triangular facets (idx: 3*count vertex indices), each as
 * cmg_plc_add_facet(plc, idx + 3*i, 3, marker) would, in one call. No
 * counterpart in the reference; for meshes of millions of triangles. */
cmg_status cmg_plc_add_triangles(cmg_plc*, const int* idx, size_t count, int marker);

/* An STL image in memory (binary when its size is 84 + 50 n, else ASCII) read as the
 * reference's read_stl reads a file (src/io/stl.cpp): one triangular facet per STL
 * facet, coincident vertices merged on their exact coordinates in order of first
 * occurrence; records decoded and vertices merged on the GPU. Errors carry the
 * reference's messages (CMG_ERR_INVALID_INPUT); a NaN coordinate is an error. */
cmg_status cmg_plc_from_stl(const void* data, size_t size, cmg_plc** out, char* errbuf,
                            size_t errbuf_len);

/* Phase times (CUDA events) of the last STL read on the current device: upload of
 * the records (binary) or parsed coordinates (ASCII), decode + merge kernels, download
 * of the points and triangles. */
cmg_status cmg_stl_last_timing(float* upload_ms, float* merge_ms, float* download_ms);

/* Phase times (CUDA events) of the last cmg_plc_simplify on the current device:
 * upload of points and facets, clustering kernels, download of the result. */
cmg_status cmg_simplify_last_timing(float* upload_ms, float* cluster_ms, float* download_ms);

/* ---- background sizing field ------------------------------------------------- */
/* Replaces cmg::sizing::from_background (src/sizing/background.cpp:58-74), whose
 * closure scans every tetrahedron per query: the background mesh (points, 4 indices per
 * tetrahedron) and node sizes (padded with 0 or truncated to the node count) move to
 * the GPU once; each evaluation returns, per query, the reference's closure value bit
 * for bit: (w0 s0 + w1 s1 + w2 s2 + w3 s3) * scale in the first tetrahedron whose
 * orient3d weights are all >= -1e-9, else the nearest node's size * scale. `which`
 * (may be NULL) receives the answering tetrahedron or -1 (nearest node). Errors:
 * "sizing: non-finite background point", "sizing: tetrahedron vertex index out of
 * range" (undefined behaviour in the reference). */
typedef struct cmg_sizing cmg_sizing;
typedef struct cmg_sizing_stats {
    int64_t binned_pairs, global_tets;  /* construction: cell entries, tetrahedra every query tests */
    int64_t far_tets;                   /* binned tetrahedra also tested by queries far from them */
    int64_t inside, nearest, slow;      /* last evaluation: answers in a tetrahedron, by the
                                           nearest node; queries outside the binned domain */
    int64_t tests, candidates;          /* full containment tests, candidates seen */
    float upload_ms, eval_ms, download_ms;  /* last host evaluation (CUDA events) */
} cmg_sizing_stats;
cmg_status cmg_sizing_create(const double* points, int64_t npoints, const int* tets, int64_t ntets,
                             const double* node_sizes, int64_t nsizes, double scale,
                             cmg_sizing** out, char* errbuf, size_t errbuf_len);
/* Host arrays (queries: 3 n doubles; out: n doubles; which: n ints or NULL). */
cmg_status cmg_sizing_eval(cmg_sizing*, const double* queries, int64_t n, double* out, int* which,
                           char* errbuf, size_t errbuf_len);
/* Device arrays, asynchronous on `stream` (a cudaStream_t; NULL: the default stream). */
cmg_status cmg_sizing_eval_device(cmg_sizing*, const double* d_queries, int64_t n, double* d_out,
                                  int* d_which, void* stream, char* errbuf, size_t errbuf_len);
cmg_status cmg_sizing_get_stats(cmg_sizing*, cmg_sizing_stats* out);
void cmg_sizing_destroy(cmg_sizing*);

/* ---- self-intersections ------------------------------------------------------ */
/* Replaces cmg::detect::self_intersections (src/detect/self_intersection.cpp:150-188):
 * every facet polygon flattened into a fan (v0, v[i-1], v[i]) in facet order; the pairs
 * of fan triangles i < j that share no vertex index and cross (the Guigue-Devillers
 * orientation test on the reference's orient3d signs; coplanar pairs do not cross),
 * in (i, j) order. Triangles with an index outside the point range are skipped.
 * A uniform-grid broad phase on the GPU replaces the reference's all-pairs loop; the
 * result is the same list. Each row of the result holds 8 ints: facet_a, facet_b, the
 * three vertex indices of triangle i, those of triangle j. */
typedef struct cmg_intersections cmg_intersections;
cmg_status cmg_plc_self_intersections(const cmg_plc*, cmg_intersections** out, char* errbuf,
                                      size_t errbuf_len);
int64_t cmg_intersections_count(const cmg_intersections*);
const int* cmg_intersections_data(const cmg_intersections*);
void cmg_intersections_destroy(cmg_intersections*);
/* Device time in ms (CUDA events) of the last self-intersection search: boxes,
 * binning and pair tests, without the host transfers. */
float cmg_self_intersections_last_ms(void);

/* The grid cmg_plc_voxelize(plc, resolution, ., pad) lays over the PLC (the
 * reference's make_grid, src/voxelize/voxelize.cpp:52-74): corner of cell (0,0,0)
 * (3 doubles), cubic spacing, dims nx, ny, nz (3 ints). Host only, no GPU call; the
 * reference's errors for resolution < 1, no points and a zero-extent PLC. No
 * counterpart in the reference's C ABI; for choosing slabs (cmg_voxel_opts.z_begin). */
cmg_status cmg_plc_grid(const cmg_plc* plc, int resolution, int pad, double* corner,
                        double* spacing, int* dims, char* errbuf, size_t errbuf_len);

/* Voxelizes with explicit options. Same handle and error conventions as
 * cmg_plc_voxelize; the grid holds every requested output. */
cmg_status cmg_plc_voxelize_ex(const cmg_plc*, const cmg_voxel_opts* opts, cmg_voxels** out,
                               char* errbuf, size_t errbuf_len);

/* Extra views of a grid (NULL when not requested). */
const double* cmg_voxels_distance_f64(const cmg_voxels*);
const int* cmg_voxels_nearest_triangle(const cmg_voxels*);
const unsigned char* cmg_voxels_nearest_region(const cmg_voxels*);
const float* cmg_voxels_error_bound(const cmg_voxels*);
/* Corner of cell (0,0,0) (the origin is its centre). */
void cmg_voxels_corner(const cmg_voxels*, double* x, double* y, double* z);
/* The layers a grid holds: [z_begin, z_end) of the grid's nz_grid layers (0, nz, nz
 * unless cmg_voxel_opts.z_begin / z_end chose a slab). cmg_voxels_dims reports the
 * layers held; corner and origin are the whole grid's, so layer k of a slab is layer
 * z_begin + k of the grid. */
void cmg_voxels_layers(const cmg_voxels*, int* z_begin, int* z_end, int* nz_grid);
void cmg_voxels_stats(const cmg_voxels*, cmg_voxel_stats* out);

/* ---- batches: many meshes, one pipeline ---------------------------------- */
typedef struct cmg_batch cmg_batch;

/* Plans a batch of n PLCs, mesh i voxelized with resolutions[i] and pads[i] (or,
 * when opts->explicit_grid, every mesh on opts' grid). Inputs are uploaded once. */
cmg_status cmg_batch_create(const cmg_plc* const* plcs, const int* resolutions, const int* pads,
                            int n, const cmg_voxel_opts* opts, cmg_batch** out, char* errbuf,
                            size_t errbuf_len);
/* Enqueues one pass over every mesh on the batch's stream. use_graph != 0
 * captures the pass in a CUDA graph on first use and replays it afterwards. */
cmg_status cmg_batch_run(cmg_batch*, int use_graph, char* errbuf, size_t errbuf_len);
/* Waits for the batch's stream. */
cmg_status cmg_batch_sync(cmg_batch*, char* errbuf, size_t errbuf_len);
/* Copies mesh i's results into a new grid handle (cmg_voxels_destroy frees it). */
cmg_status cmg_batch_get(cmg_batch*, int i, cmg_voxels** out, char* errbuf, size_t errbuf_len);
int cmg_batch_size(const cmg_batch*);
int64_t cmg_batch_cells(const cmg_batch*);
void cmg_batch_destroy(cmg_batch*);

/* ---- measurement ---------------------------------------------------------- */
/* Phase times of a batch's last run (CUDA events on its streams), once enabled. The
   SDF preparation runs on a second stream beside the occupancy passes, so the phases
   can sum to more than total_ms. */
typedef struct cmg_batch_timing {
    float occupancy_ms; /* triangle prep .. exact pass */
    float sdf_prep_ms;  /* triangle bins, brick candidate lists, work order */
    float eval_ms;      /* distance evaluation kernel */
    float total_ms;
} cmg_batch_timing;

/* Cost-model counts of a batch's last run: sum over cells of K(v), the number of
 * triangles whose bounding sphere reaches the cell's distance sphere (the minimal
 * candidate set of a bounding-sphere-pruned exact search), the same over the
 * FP64 band, and the occupancy filter's orient3d and plane_z evaluations. */
typedef struct cmg_work_model {
    double sum_k;
    double sum_k_band;
    double band_cells;
    double orient_calls;
    double crossings;
} cmg_work_model;

/* The cudaStream_t the batch runs on (for events recorded by the caller). */
void* cmg_batch_stream(const cmg_batch*);
cmg_status cmg_batch_set_timing(cmg_batch*, int on);
cmg_status cmg_batch_get_timing(cmg_batch*, cmg_batch_timing* out, char* errbuf, size_t errbuf_len);
cmg_status cmg_batch_work_model(cmg_batch*, cmg_work_model* out, char* errbuf, size_t errbuf_len);
cmg_status cmg_batch_stats(cmg_batch*, cmg_voxel_stats* out, char* errbuf, size_t errbuf_len);
/* Kernels this library has launched in this process. */
long long cmg_gpu_launches(void);
/* Measured FMA throughput of the current GPU in FLOP/s (FMA = 2 FLOPs):
 * fp64 != 0 for DFMA, else FFMA. */
cmg_status cmg_gpu_peak_flops(int fp64, double* flops, char* errbuf, size_t errbuf_len);

/* ---- differentiable signed distance (forward + adjoint) -------------------- */
/* No counterpart in the reference (it has no SDF gradient). A plan holds one mesh
 * of fixed topology on an explicit grid for repeated forwards with moving points
 * and the adjoint dL/d(points) of the signed distance. */
typedef struct cmg_sdf_plan cmg_sdf_plan;

/* points: host, 3*npoints doubles (the first positions); triangles: host,
 * 3*ntriangles indices (fixed). opts->explicit_grid must be set (corner, spacing,
 * dims); precision, predicates, band and brick apply. Every forward produces
 * occupancy, the FP64 signed distance and the nearest-feature checkpoint. */
cmg_status cmg_sdf_plan_create(const double* points, int64_t npoints, const int* triangles,
                               int64_t ntriangles, const cmg_voxel_opts* opts,
                               cmg_sdf_plan** out, char* errbuf, size_t errbuf_len);
/* Voxelizes at the device positions d_points (3*npoints doubles; NULL keeps the
 * last ones), enqueued on `stream` (a cudaStream_t; NULL for the default stream).
 * The call synchronises that stream twice (to size the candidate lists for the
 * new positions) and returns with the evaluation enqueued. */
cmg_status cmg_sdf_plan_forward(cmg_sdf_plan*, const double* d_points, void* stream,
                                char* errbuf, size_t errbuf_len);
/* Device views of the last forward's outputs, valid until the next forward:
 * occupancy (uint8), signed distance (double), nearest triangle (int, -1 when
 * none) and its Ericson region (uint8: 0 a, 1 b, 2 ab, 3 c, 4 ac, 5 bc, 6 face);
 * cell idx = (k*ny + j)*nx + i. CMG_ERR_INVALID_INPUT before the first forward. */
cmg_status cmg_sdf_plan_outputs(const cmg_sdf_plan*, const unsigned char** d_occupancy,
                                const double** d_sdf, const int** d_nearest_triangle,
                                const unsigned char** d_nearest_region);
int64_t cmg_sdf_plan_cells(const cmg_sdf_plan*);
/* Copies the last forward's outputs (the four arrays above) into device buffers
 * the caller owns, enqueued on `stream`; a NULL destination is skipped. */
cmg_status cmg_sdf_plan_copy_outputs(const cmg_sdf_plan*, unsigned char* d_occupancy,
                                     double* d_sdf, int* d_nearest_triangle,
                                     unsigned char* d_nearest_region, void* stream,
                                     char* errbuf, size_t errbuf_len);
/* Adjoint: d_grad_points (3*npoints doubles, overwritten) = dL/d(points) given
 * d_grad_sdf = dL/d(signed distance) per cell, from a forward's checkpoint
 * (occupancy, nearest triangle, region: device copies the caller kept) and the
 * positions of that forward (d_points; NULL = the plan's last). Distances are
 * recomputed in FP64; a cell on the surface (distance 0) contributes nothing.
 * The reduction has a fixed order (no float atomics): results are bitwise
 * reproducible. Enqueued on `stream`; allocates nothing. */
cmg_status cmg_sdf_plan_backward(cmg_sdf_plan*, const double* d_points,
                                 const unsigned char* d_occupancy, const int* d_nearest_triangle,
                                 const unsigned char* d_nearest_region, const double* d_grad_sdf,
                                 double* d_grad_points, void* stream, char* errbuf,
                                 size_t errbuf_len);
void cmg_sdf_plan_destroy(cmg_sdf_plan*);

/* ---- predicate streams ------------------------------------------------------ */
/* Where stream arrays live. */
#define CMG_MEM_HOST 0
#define CMG_MEM_DEVICE 1

typedef struct cmg_pred_stats {
    int64_t queries;
    int64_t fp64_queries;      /* not certified by the FP32 filter */
    int64_t exact_queries;     /* resolved in exact arithmetic (an FP64 evaluation in
                                  which no operation rounded, or expansions) */
    int64_t expansion_queries; /* of which needed expansion arithmetic */
    float fp32_pass_ms;        /* device time of the FP32 certification pass (CUDA events) */
    int32_t tma_reruns;        /* FP32 passes rerun with per-thread loads after a bulk-copy
                                  wait ran out (expected 0) */
} cmg_pred_stats;

/* Signs (-1, 0, +1) of n orient3d(a,b,c,d) queries given as 12 SoA coordinate
 * arrays (ax ay az bx by bz cx cy cz dx dy dz). mode: CMG_PRED_COMPAT (the
 * reference's robust::orient3d as initialised: the rounded determinant's sign
 * unless it is exactly zero, src/predicates/robust.cpp:36-42) or CMG_PRED_EXACT.
 * where: CMG_MEM_HOST (arrays and out in host memory) or CMG_MEM_DEVICE (device
 * memory; stream is the cudaStream_t to use, NULL for the default). Host arrays are
 * read by the device directly where it accesses pageable host memory
 * (cudaDevAttrPageableMemoryAccess), in chunks of 2^24 queries, and otherwise copied
 * in chunks of 2^22 through two device buffer sets (the environment variable
 * CMG_HOST_STREAM=copy forces the copies). The call returns when the signs are
 * written. stats may be NULL (fp32_pass_ms: summed over the chunks). No counterpart
 * in the reference beyond the scalar predicate it applies per query. */
cmg_status cmg_orient3d_stream(const double* const* coords, int64_t n, int mode, int where,
                               signed char* out, cmg_pred_stats* stats, void* stream,
                               char* errbuf, size_t errbuf_len);
/* Same for insphere(a,b,c,d,e) with 15 SoA arrays (src/predicates/robust.cpp:44-50). */
cmg_status cmg_insphere_stream(const double* const* coords, int64_t n, int mode, int where,
                               signed char* out, cmg_pred_stats* stats, void* stream,
                               char* errbuf, size_t errbuf_len);
/* Replaces cmg::backend::cuda::orient3d_signs (src/backend/cuda/orient3d.cu:54-82)
 * together with the CPU escalation of robust::orient3d_signs
 * (src/predicates/robust.cpp:68-105): host points xyz[3*npts], candidate
 * tetrahedra tets[4*n] (indices into xyz), signs equal to the scalar
 * robust::orient3d's for every candidate, computed entirely on the GPU. */
cmg_status cmg_orient3d_signs(const double* xyz, int npts, const int* tets, int n, int* out_sign);
/* Replaces robust::orient3d_batch (src/predicates/robust.cpp:52-66): the orient3d
 * VALUE of every candidate (the rounded determinant when it is not zero, else the
 * adaptive routine's answer), bit for bit, computed on the GPU. */
cmg_status cmg_orient3d_batch(const double* xyz, int npts, const int* tets, int n, double* out_value);

/* ---- host memory ------------------------------------------------------------ */
/* No counterpart in the reference. Page-locked host memory from the library's pool
 * of reused blocks: outputs (stream signs, grids) written there skip the page
 * faults of freshly mapped memory and the copy engine's staging. At least `bytes`
 * bytes, or NULL when no memory is left. cmg_host_free returns a block to the pool
 * (NULL is ignored). */
void* cmg_host_alloc(size_t bytes);
void cmg_host_free(void* p);

/* ---- occupancy without allocation ----------------------------------------- */
/* No counterpart in the reference. For callers that cannot call cudaMalloc (a host
 * framework that owns device memory through its own pool, a loop that may not
 * allocate after start-up): occupancy of one mesh on an explicit grid, with the
 * inputs and the output in device buffers the caller owns (d_points: 3*npoints
 * doubles, d_triangles: 3*ntriangles ints, d_occupancy: dims[0]*dims[1]*dims[2]
 * bytes, idx = (k*ny + j)*nx + i) and all working memory taken from a fixed 32 MiB
 * array in device memory that the library holds on every GPU it is loaded on.
 * Allocates nothing. Inputs that need more working memory than the array holds
 * are rejected with CMG_ERR_INVALID_INPUT and a message. Calls share the array, so
 * calls that overlap on the GPU race and must be serialised.
 * `stream` is a cudaStream_t (NULL for the default stream); the call reads two
 * sizes back from the device and synchronises `stream`, so it returns after the
 * work on it has finished, and it cannot be part of a CUDA graph: on a stream that
 * is being captured it returns CMG_ERR_UNSUPPORTED_OPTION before any device work.
 * predicates: CMG_PRED_COMPAT or
 * CMG_PRED_EXACT. The result equals cmg_plc_voxelize_ex's occupancy. */
cmg_status cmg_gpu_occupancy_static(const double* d_points, int64_t npoints,
                                    const int* d_triangles, int64_t ntriangles,
                                    const double* corner, double spacing, const int* dims,
                                    int predicates, unsigned char* d_occupancy, void* stream,
                                    char* errbuf, size_t errbuf_len);

/* ---- testing the error paths ------------------------------------------------ */
/* No counterpart in the reference. After the library's next `skip` device allocations
 * succeed, the `count` after them report cudaErrorMemoryAllocation without allocating
 * (a host-side fake of a failed cudaMalloc); (0, 0) turns the failures off. Each call
 * that meets one returns CMG_ERR_INTERNAL with "out of memory" in its error buffer,
 * releases what it holds, and leaves the library usable for the next call. */
cmg_status cmg_debug_fail_device_allocs(int skip, int count);

/* Test hook, no reference counterpart: the next predicate stream whose FP32 pass is
 * TMA-staged takes the wait of its first CTA's first warp for that CTA's tile `tile`
 * as having run out (-1 = off; used once). The pass then stops every warp, drains the
 * copies in flight and is rerun with per-thread loads (cmg_pred_stats.tma_reruns = 1),
 * with the same signs. No wait runs out for real and the GPU stays usable. */
cmg_status cmg_debug_fail_pred_wait(int64_t tile);

/* Library build identification, e.g. "cmg-gb300 sm_103a". */
const char* cmg_gpu_version(void);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* CMG_GPU_H */
