/*
 * orc.h - C interface of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a scalar C++ restatement of the
 * Vermeer hot path (QBVH build and traversal, watertight ray/triangle test,
 * motion traversal, two-level scene traversal, QMC sequences, reference-mode
 * shading).  It is the checker for the CUDA path: only the tests, the smoke
 * check and the CPU-baseline leg of the benchmark load it.  The product
 * library (libvmr) never links or calls it.
 *
 * All floating-point code is compiled with -ffp-contract=off so that every
 * a*b+c is two rounded operations, as in the reference's amd64 build (SSE
 * scalar arithmetic, no FMA).
 */
#ifndef ORC_H
#define ORC_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 128-byte node, field for field the layout of qbvh.Node (qbvh/qbvh.go:31-36). */
typedef struct {
    float boxes[24];
    uint32_t axis0, axis1, axis2;
    int32_t children[4];
    int32_t parent;
} orc_node;

/* Topology node of the motion tree (qbvh/mqbvh.go:24-29); 40 bytes, although
 * the reference comment says 32. */
typedef struct {
    int32_t axis0, axis1, axis2;
    int32_t children[4];
    int32_t parent;
    uint32_t pad[2];
} orc_mnode;

typedef struct orc_mesh orc_mesh;
typedef struct orc_scene orc_scene;

/* Rays are passed as 8 floats each: px py pz dx dy dz tmax time. */
enum { ORC_RAY_STRIDE = 8 };

/* Per-ray counters written by the trace calls (3 x uint32 per ray):
 * node visits (NodesT), leaf visits (LeafsT), triangle tests. */

/* Build a PolyMesh accelerator exactly as PolyMesh.initAccel
 * (builtin/geom/polymesh/buildqbvh.go:14-144).
 *   verts   : keys * nverts * 3 floats (key-major, PointArray layout)
 *   idxp    : ntris * 3 vertex indices in the mesh's original face order
 *   motion_fixed : 0 = faithful motion leaf test (reference behaviour),
 *                  1 = fixed (leaf position mapped through accel idx).
 * Returns NULL on error (message via orc_last_error). */
orc_mesh* orc_mesh_create(const float* verts, uint32_t nverts, uint32_t keys,
                          const uint32_t* idxp, uint32_t ntris, float ray_bias,
                          int motion_fixed);
void orc_mesh_destroy(orc_mesh* m);
const char* orc_last_error(void);

/* Sizes: number of static nodes (0 for a motion mesh), number of motion
 * nodes (0 for a static mesh), bounds (6 floats, min xyz then max xyz). */
void orc_mesh_info(const orc_mesh* m, uint32_t* n_nodes, uint32_t* n_mnodes,
                   float* bounds6);
/* Export the accelerator: static nodes, accel idx (leaf position -> original
 * face), idxp as the mesh holds it after the build (leaf order for a static
 * mesh, original order for a motion mesh), motion nodes and motion boxes
 * ([keys][n_mnodes][24]).  Any pointer may be NULL. */
void orc_mesh_export(const orc_mesh* m, orc_node* nodes, int32_t* accel_idx,
                     uint32_t* idxp_out, orc_mnode* mnodes, float* mboxes);

/* Closest-hit (shadow=0) or any-hit (shadow=1) traversal of one mesh
 * (PolyMesh.Trace, builtin/geom/polymesh/trace.go:15-102).
 * Outputs per ray: prim (ElemID or -1), t (Tclosest after the trace), u,v,w
 * (barycentrics of the accepted hit, 0 if none).  counters may be NULL.
 * status: 0 ok, -5 traversal stack (90 entries) overflowed on some ray.
 * nthreads <= 0 uses all hardware threads. */
int orc_trace_mesh(const orc_mesh* m, const float* rays, size_t n, int shadow,
                   int nthreads, int32_t* prim, float* t, float* u, float* v,
                   float* w, uint32_t* counters);

/* Two-level scene (builtin/scene/scene.go): meshes are referenced, not
 * copied, and must outlive the scene. */
orc_scene* orc_scene_create(orc_mesh* const* meshes, uint32_t n);
void orc_scene_destroy(orc_scene* s);
/* Sizes of the top level: static node count or motion node count and keys. */
void orc_scene_info(const orc_scene* s, uint32_t* n_nodes, uint32_t* n_mnodes,
                    uint32_t* keys);
/* Export top level: static nodes, geom order (leaf position -> mesh index as
 * passed to orc_scene_create), motion nodes, motion boxes. */
void orc_scene_export(const orc_scene* s, orc_node* nodes, int32_t* geom_order,
                      orc_mnode* mnodes, float* mboxes);
int orc_trace_scene(const orc_scene* s, const float* rays, size_t n, int shadow,
                    int nthreads, int32_t* prim, int32_t* geom, float* t,
                    float* u, float* v, float* w, uint32_t* counters);

/* QMC (math/ldseq).  Integer forms, bit-exact. */
uint64_t orc_vdc(uint64_t i, uint64_t scramble);     /* ldseq.go:55-75 */
uint64_t orc_sobol(uint64_t i, uint64_t scramble);   /* ldseq.go:83-96 */
/* ldseq.RasterXY (raster.go:50-57): returns index, writes rx, ry. */
uint64_t orc_raster_xy(uint32_t m, uint32_t frame, uint32_t px, uint32_t py,
                       uint64_t sx, uint64_t sy, double* rx, double* ry);
/* The m-th rows (m = 1..26) of the two Grunschloss tables, computed from the
 * generator matrices: 52 uint64 each. */
void orc_vdc_sobol_tables(uint32_t m, uint64_t* fwd52, uint64_t* inv52);

#ifdef __cplusplus
}
#endif
#endif
