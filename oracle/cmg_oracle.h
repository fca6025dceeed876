/* cmg_oracle.h — CPU restatement of CyberMeshGenerator's voxelization path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the parity checker for the GPU
 * product in cybermeshgenerator_gb300/: the test suite, the smoke check and the
 * CPU-baseline leg of bench.py load it; the product library never links it.
 *
 * It restates, in plain C compiled with -ffp-contract=off, the reference's
 *   - grid set-up            src/voxelize/voxelize.cpp:52-74   (make_grid)
 *   - xy bucket membership   src/voxelize/voxelize.cpp:78-103  (build_xy_buckets)
 *   - ray-parity occupancy   src/voxelize/voxelize.cpp:121-196 (column_crossings,
 *                            solve_column, kNudge, classify_occupancy)
 *   - Ericson distance       src/voxelize/voxelize.cpp:202-247 (point_tri_dist2)
 *   - ring-search SDF        src/voxelize/voxelize.cpp:251-358 (build_xyz_buckets,
 *                            for_shell, nearest_tri_dist2, fill_distance)
 *   - orient3d / insphere    src/predicates/predicates.cpp:2194-2243, 4050-4163 as
 *                            initialised by src/predicates/robust.cpp:28-34
 *                            (static filter threshold 0: the rounded determinant is
 *                            returned whenever it is nonzero; only an exact zero is
 *                            resolved by exact arithmetic).
 * Exact signs use expansion arithmetic after Shewchuk, "Adaptive Precision
 * Floating-Point Arithmetic and Fast Robust Geometric Predicates" (CMU-CS-96-140):
 * Two-Sum, Dekker-split Two-Product, Grow-Expansion and Scale-Expansion with zero
 * elimination, written here from that paper.
 *
 * Parity pinning: tests/golden holds outputs of the reference itself (built from
 * its own sources by oracle/Makefile into oracle/_ref/), and the CPU test suite
 * checks this restatement against them bit for bit.
 */
#ifndef CMG_ORACLE_H
#define CMG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_grid {
    double corner[3]; /* world coordinate of the MIN corner of cell (0,0,0) */
    double spacing;
    int nx, ny, nz;
} orc_grid;

/* Occupancy statistics gathered while classifying (one column = one (i,j)). */
typedef struct orc_occ_stats {
    int64_t columns;          /* nx*ny */
    int64_t nudged_columns;   /* first attempt grazed; a nudge was needed */
    int64_t exhausted_columns;/* every nudge grazed: partial heights kept */
    int64_t exact_calls;      /* orient3d evaluations that needed exact arithmetic */
    int64_t orient_calls;     /* all orient3d evaluations */
    int64_t crossings;        /* heights pushed on the successful attempts */
} orc_occ_stats;

/* Predicate modes. COMPAT = the reference as initialised (sign of the rounded
 * determinant unless it is exactly zero). EXACT = sign of the exact determinant. */
enum { ORC_COMPAT = 0, ORC_EXACT = 1 };

/* ---- predicates ---------------------------------------------------------- */
/* robust::orient3d's value (sizing_oracle.c): the rounded determinant when it is not
 * zero, else the adaptive routine's answer. */
double orc_orient3d_value(const double* pa, const double* pb, const double* pc, const double* pd);
void orc_orient3d_values(const double* const* soa, int64_t n, double* out);
/* Background sizing field (sizing_oracle.c): sizes (np entries, already padded or
 * truncated) interpolated in the first containing tetrahedron, else the nearest
 * node's; which[q] = the answering tetrahedron or -1 (may be NULL). */
void orc_sizing_eval(const double* P, int64_t np, const int* T, int64_t nt, const double* S,
                     double scale, const double* Q, int64_t nq, double* out, int64_t* which,
                     int nthreads);
double orc_orient3d_fast(const double* pa, const double* pb, const double* pc,
                         const double* pd);
double orc_insphere_fast(const double* pa, const double* pb, const double* pc,
                         const double* pd, const double* pe);
int orc_orient3d_exact_sign(const double* pa, const double* pb, const double* pc,
                            const double* pd);
int orc_insphere_exact_sign(const double* pa, const double* pb, const double* pc,
                            const double* pd, const double* pe);
int orc_orient3d_sign(const double* pa, const double* pb, const double* pc,
                      const double* pd, int mode);
int orc_insphere_sign(const double* pa, const double* pb, const double* pc,
                      const double* pd, const double* pe, int mode);
/* Stream form: n queries, coordinates in SoA (12 arrays for orient3d: ax ay az bx
 * ... dz; 15 for insphere), one int8 sign per query. */
void orc_orient3d_stream(const double* const* soa, int64_t n, int mode, int8_t* out,
                         int nthreads);
void orc_insphere_stream(const double* const* soa, int64_t n, int mode, int8_t* out,
                         int nthreads);

/* ---- grid ---------------------------------------------------------------- */
/* make_grid: returns 0, or -1 for a zero-extent point set. */
int orc_make_grid(const double* pts, int64_t npts, int resolution, int pad,
                  orc_grid* g);
/* Fan triangulation (v0, v[i-1], v[i]) of polygon facets given as a flat index
 * array with per-facet offsets (nfacets+1 entries). Returns the triangle count;
 * when tris is non-NULL writes 3 ints per triangle. */
int64_t orc_fan_triangles(const int* idx, const int64_t* off, int64_t nfacets,
                          int* tris);

/* ---- occupancy ----------------------------------------------------------- */
void orc_occupancy(const double* pts, const int* tris, int64_t ntris,
                   const orc_grid* g, int mode, uint8_t* occ, orc_occ_stats* st,
                   int nthreads);

/* ---- distance ------------------------------------------------------------ */
/* Ericson squared distance; *region gets 0..6 (vertex a, vertex b, edge ab,
 * vertex c, edge ac, edge bc, interior) when non-NULL. */
double orc_point_tri_dist2(const double* p, const double* a, const double* b,
                           const double* c, int* region);
/* Reference algorithm (3-D buckets + Chebyshev ring search). occ is required for
 * the sign. Writes the signed distance in double (before the float cast) and/or
 * float. Either output may be NULL. */
void orc_sdf_ring(const double* pts, const int* tris, int64_t ntris,
                  const orc_grid* g, const uint8_t* occ, double* sdf64, float* sdf32,
                  int nthreads);
/* Ring search restricted to the listed voxels (flat indices); unsigned distance
 * squared out. Used to time a bounded sample: times (nullable) receives the
 * seconds of the bucket build [0] and of the queries [1]. */
void orc_sdf_ring_sample(const double* pts, const int* tris, int64_t ntris,
                         const orc_grid* g, const int64_t* vox, int64_t nq,
                         double* d2, int nthreads, double* times);
/* Brute force over every triangle for the listed voxels: nearest squared distance,
 * the first triangle attaining it (ascending id) and its Ericson region. */
void orc_sdf_brute(const double* pts, const int* tris, int64_t ntris,
                   const orc_grid* g, const int64_t* vox, int64_t nq, double* d2,
                   int* tri, int* region, int nthreads);
/* Brute force at arbitrary query points (3 doubles each). */
void orc_dist2_points(const double* pts, const int* tris, int64_t ntris,
                      const double* q, int64_t nq, double* d2, int* tri, int nthreads);

/* ---- adjoint ------------------------------------------------------------- */
/* Analytic FP64 gradient of L = sum_v w_v (s_v d_v - t_v)^2 with respect to the
 * vertex positions, where d_v is the distance of voxel v to triangle tri[v] (its
 * nearest triangle; the Ericson region is recomputed), s_v = -1 for occupied
 * voxels, +1 otherwise. Voxels are all nx*ny*nz cells; tri[v] < 0 skips a voxel.
 * grad has 3*npts doubles and is overwritten. */
void orc_sdf_grad(const double* pts, int64_t npts, const int* tris,
                  const orc_grid* g, const uint8_t* occ, const int* tri,
                  const double* w, const double* t, double* grad);

/* Self-intersections (src/detect/self_intersection.cpp): the pairs (i, j), i < j, of
 * triangles sharing no vertex index that cross by the Guigue-Devillers orientation test
 * on the reference's orient3d signs; triangles with an index outside [0, npts) are
 * skipped. Writes at most cap pairs (2 int64 each) in (i, j) order; returns the count. */
int orc_tri_tri_cross(const double* p1, const double* q1, const double* r1, const double* p2,
                      const double* q2, const double* r2);
int64_t orc_self_intersections(const double* pts, int64_t npts, const int* tris, int64_t ntris,
                               int64_t* out_pairs, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
