/* cmg_c.h — C ABI of the GB300 voxelization library (libcmg_c.so).
 *
 * Drop-in for the reference's stable C ABI, bindings/c/include/cmg_c/cmg_c.h:
 * every symbol below has the reference's name, signature, status codes, ownership
 * and layout, so a program (or the reference's ctypes binding,
 * bindings/python/src/cybermesh/__init__.py:58-157, which binds all of them at
 * import) links against this library unchanged. The voxelization path runs on the
 * GPU; the meshing and file-I/O entry points exist so that such a program loads,
 * and answer CMG_ERR_NOT_IMPLEMENTED (they are not part of this library).
 *
 * GPU-specific additions are declared in cmg_c/cmg_gpu.h.
 */
#ifndef CMG_C_H
#define CMG_C_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes; values as in the reference (cmg_c.h:18-27). */
typedef enum cmg_status {
    CMG_OK = 0,
    CMG_ERR_INVALID_INPUT = 1,
    CMG_ERR_SELF_INTERSECTION = 2,
    CMG_ERR_UNSUPPORTED_OPTION = 3,
    CMG_ERR_QUALITY_NOT_MET = 4,
    CMG_ERR_NOT_IMPLEMENTED = 5,
    CMG_ERR_INTERNAL = 6,
    CMG_ERR_PARSE = 7
} cmg_status;

/* Opaque handles (cmg_c.h:30-33). */
typedef struct cmg_plc cmg_plc;
typedef struct cmg_mesh cmg_mesh;
typedef struct cmg_options cmg_options;
typedef struct cmg_voxels cmg_voxels;

/* --- PLC handles and input (cmg_c.h:36-60; cmg_c.cpp:73-125) ------------- */
cmg_plc* cmg_plc_create(void);
void cmg_plc_destroy(cmg_plc*);
/* Replaces the point set with `count` points from xyz[3*count]. */
cmg_status cmg_plc_set_points(cmg_plc*, const double* xyz, size_t count);
/* Appends a one-polygon facet (count >= 3 vertex indices); fan-triangulated as
 * (v0, v[i-1], v[i]) by voxelization. */
cmg_status cmg_plc_add_facet(cmg_plc*, const int* poly_vertex_indices, size_t count, int marker);
cmg_status cmg_plc_add_hole(cmg_plc*, double x, double y, double z);
cmg_status cmg_plc_add_region(cmg_plc*, double x, double y, double z, double attribute,
                              double max_volume);
/* Read-back (cmg_c.h:119-122; cmg_c.cpp:392-417): points as [x,y,z,...]; facets
 * fan-triangulated to [a,b,c,...]. Valid until the PLC changes or is destroyed. */
size_t cmg_plc_num_points(const cmg_plc*);
const double* cmg_plc_points(cmg_plc*);
size_t cmg_plc_num_triangles(cmg_plc*);
const int* cmg_plc_triangles(cmg_plc*);

/* --- voxelization (cmg_c.h:137-153; cmg_c.cpp:242-292) ------------------- */
/* Voxelizes a closed PLC: `resolution` (>= 1) cubic cells along the longest
 * bounding-box axis, `pad` margin cells on every side; mode 1 = signed distance
 * (float, negative inside), any other mode = occupancy bytes (1 inside). *out is
 * set to NULL first; on CMG_OK it receives a handle for cmg_voxels_destroy. */
cmg_status cmg_plc_voxelize(const cmg_plc*, int resolution, int mode, int pad, cmg_voxels** out,
                            char* errbuf, size_t errbuf_len);
void cmg_voxels_destroy(cmg_voxels*);
void cmg_voxels_dims(const cmg_voxels*, int* nx, int* ny, int* nz);
/* World coordinate of the CENTRE of cell (0,0,0). */
void cmg_voxels_origin(const cmg_voxels*, double* x, double* y, double* z);
double cmg_voxels_spacing(const cmg_voxels*);
/* Zero-copy views, idx = (k*ny + j)*nx + i; NULL when the grid holds the other
 * mode's data. Valid until the handle is destroyed. */
const unsigned char* cmg_voxels_occupancy(const cmg_voxels*);
const float* cmg_voxels_distance(const cmg_voxels*);

/* --- options (cmg_c.h:38-39, 64-77); kept so that binders load ----------- */
cmg_options* cmg_options_create(void);
void cmg_options_destroy(cmg_options*);
cmg_status cmg_options_from_switches(cmg_options*, const char* switches, char* errbuf,
                                     size_t errbuf_len);
cmg_status cmg_options_set_plc(cmg_options*, int on);
cmg_status cmg_options_set_max_volume(cmg_options*, double max_volume);
cmg_status cmg_options_set_quality(cmg_options*, double radius_edge, double min_dihedral);
cmg_status cmg_options_set_preserve_edges(cmg_options*, int on);

/* --- meshing, mesh views and file I/O (cmg_c.h:82-128): not part of this
 * library; each answers CMG_ERR_NOT_IMPLEMENTED (or 0 / NULL for getters). */
void cmg_mesh_destroy(cmg_mesh*);
cmg_status cmg_tetrahedralize(const cmg_plc*, const cmg_options*, cmg_mesh** out, char* errbuf,
                              size_t errbuf_len);
cmg_status cmg_delaunay(const double* xyz, size_t count, const cmg_options*, cmg_mesh** out,
                        char* errbuf, size_t errbuf_len);
size_t cmg_mesh_num_points(const cmg_mesh*);
size_t cmg_mesh_num_tets(const cmg_mesh*);
size_t cmg_mesh_num_faces(const cmg_mesh*);
const double* cmg_mesh_points(const cmg_mesh*);
const int* cmg_mesh_tets(const cmg_mesh*);
const int* cmg_mesh_faces(const cmg_mesh*);
const int* cmg_mesh_tet_markers(const cmg_mesh*);
const int* cmg_mesh_face_markers(const cmg_mesh*);
/* GB300 library: a .stl path is read on the GPU (the reference's read_stl semantics,
 * see cmg_plc_from_stl in cmg_gpu.h); .poly/.smesh/.off/.ply/.obj answer
 * CMG_ERR_NOT_IMPLEMENTED; any other extension is CMG_ERR_INVALID_INPUT
 * ("unsupported file format for <path>"), as in the reference. */
cmg_status cmg_read_plc(const char* path, cmg_plc** out, char* errbuf, size_t len);
cmg_status cmg_read_points(const char* path, cmg_plc** out, char* errbuf, size_t len);
cmg_status cmg_read_mesh(const char* path, cmg_mesh** out, char* errbuf, size_t len);
cmg_status cmg_write_mesh(const char* path, const cmg_mesh*, char* errbuf, size_t len);
cmg_status cmg_write_plc(const char* path, const cmg_plc*, char* errbuf, size_t len);
/* Replaces cmg_plc_simplify (bindings/c/src/cmg_c.cpp:222-240 over
 * src/simplify/simplify.cpp:48-112): grid vertex clustering on the GPU with the
 * reference's cells, representative numbering (first vertex order), centroids (sums
 * in vertex order, bit for bit) and triangle order; degenerate and repeated
 * triangles dropped. Errors as the reference's ("simplify: PLC has no points",
 * "simplify: grid must be >= 1", "simplify: degenerate (zero-extent) surface"), plus
 * "simplify: non-finite point coordinate" and "simplify: facet vertex index out of
 * range" where the reference's behaviour is undefined. */
cmg_status cmg_plc_simplify(const cmg_plc*, int grid, cmg_plc** out, char* errbuf,
                            size_t errbuf_len);

/* Library version string (cmg_c.h:156): the reference version it drops in for. */
const char* cmg_version(void);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* CMG_C_H */
