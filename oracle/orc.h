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

/* ------------------------------------------------------ reference render */
/* ShaderStd parameters (builtin/shader/std.go:25-47).  A parameter the scene
 * does not set is absent (nil in the reference), which changes defaults:
 * flags say which are present. */
enum {
    ORC_SH_EMISSION_COLOUR = 1, ORC_SH_EMISSION_STRENGTH = 2,
    ORC_SH_DIFFUSE_COLOUR = 4, ORC_SH_DIFFUSE_STRENGTH = 8, ORC_SH_DIFFUSE_ROUGHNESS = 16,
    ORC_SH_SPEC1_COLOUR = 32, ORC_SH_SPEC1_STRENGTH = 64, ORC_SH_SPEC1_ROUGHNESS = 128,
    ORC_SH_FRESNEL_REFL = 256, ORC_SH_FRESNEL_EDGE = 512, ORC_SH_IOR = 1024,
    ORC_SH_DEBUG = 2048  /* DebugShader (builtin/shader/debug.go): OutRGB = diffuse_colour */
};
typedef struct {
    uint32_t flags;
    float emission_colour[3], emission_strength;
    float diffuse_colour[3], diffuse_strength, diffuse_roughness;
    float spec1_colour[3], spec1_strength, spec1_roughness;
    int spec1_fresnel; /* 0 Dielectric (also the unset default), 1 Metal */
    float spec1_fresnel_refl[3], spec1_fresnel_edge[3];
    float ior;
} orc_shader;

/* TriLight (builtin/light/triangle.go:18-28); mesh = index, among the
 * meshes given to orc_scene_create, of the light's own emissive mesh. */
typedef struct {
    float p0[3], p1[3], p2[3];
    int samples;
    uint32_t shader;
    uint32_t mesh;
} orc_trilight;

/* Camera (builtin/camera/camera.go): m = LocalToWorld, column-major. */
typedef struct {
    float m[16];
    float tan_theta_focal, aspect, focal, radius;
} orc_camera;

/* DiskLight (builtin/light/disk.go:18-31): N = normalize(LookAt - P),
 * T = normalize(N x Up), B = N x T; mesh = its emissive fan (createMesh). */
typedef struct {
    float P[3], up[3], lookat[3];
    float radius;
    int samples;
    uint32_t shader, mesh;
} orc_disklight;

/* SphereLight (builtin/light/sphere.go:14-28); mesh = its sphere geom. */
typedef struct {
    float P[3];
    float radius;
    int samples;
    uint32_t shader, mesh;
} orc_spherelight;

typedef struct orc_render orc_render;

/* Pixel filter for filter importance sampling (builtin/filter/filter.go):
 * kind 0 none (box), 1 GaussianFilter (gauss.go; defaults res 17, width 2),
 * 2 AiryFilter (airy.go; defaults res 49, width 6, peak 4). */
typedef struct {
    int kind;
    int res;
    float width;
    float peak;
} orc_pixel_filter;
/* Sampler.WarpSample (filter.go:40-80) of n sample pairs. */
int orc_filter_warp(const orc_pixel_filter* f, const double* r0, const double* r1, size_t n, double* u, double* v);
/* CreateSampler's cdfV (res) and cdfVU (res x res, row j = cdfVU[j]). */
int orc_filter_tables(const orc_pixel_filter* f, double* cdfV, double* cdfVU);

/* OutputHDR's pixel bytes (image/hdr/writer.go:58-82, convertRGBToRGBE,
 * image/hdr/hdr.go:28-55): out = w*h*4 bytes, scanline j = row h-1-j. */
int orc_encode_rgbe(const float* rgb, uint32_t w, uint32_t h, uint8_t* out);

/* An analytic sphere geom (builtin/geom/sphere): usable wherever a mesh is
 * (scenes, renders); its shader is the mesh's shader 0. */
orc_mesh* orc_sphere_create(const float center[3], float radius);

/* Per-mesh shading data: shader index per face (face order, may be NULL)
 * and per-vertex normals of key 0 (may be NULL). */
int orc_mesh_set_shading(orc_mesh* m, const uint8_t* face_shader, const float* normals);
/* Per-key normals of a motion mesh (PolyMesh.Normals with as many keys as
 * the vertices): normals[key][i][3], n_per_key >= 3 x triangles; a hit on
 * element e reads entries 3e .. 3e+2 of the two keys around the ray's time
 * (builtin/geom/polymesh/trace.go:694-712).  NULL clears them; -1 when the
 * mesh is static, keys differ or n_per_key is short. */
int orc_mesh_set_motion_normals(orc_mesh* m, const float* normals, uint32_t n_per_key, uint32_t keys);

/* shader_list[mesh_shader_offset[m] .. + mesh_shader_count[m]] are the
 * shaders of mesh m (PolyMesh.Shader). */
orc_render* orc_render_create(const orc_scene* scene, orc_mesh* const* meshes, uint32_t n_meshes,
                              const uint32_t* mesh_shader_offset, const uint32_t* mesh_shader_count,
                              const uint32_t* shader_list, const orc_shader* shaders, uint32_t n_shaders,
                              const orc_trilight* lights, uint32_t n_lights, const orc_camera* cam);
void orc_render_destroy(orc_render* r);
/* The render's pixel filter (core.Init of a PixelFilter node, core/core.go:88-89):
 * the RasterXY sample's position in its pixel is warped before the camera
 * ray is made (core/render.go:99-107).  kind 0 removes it. */
int orc_render_set_filter(orc_render* r, const orc_pixel_filter* f);
/* Append DiskLights to the light list (after the TriLights). */
int orc_render_add_disk_lights(orc_render* r, const orc_disklight* lights, uint32_t n);
/* Append SphereLights (after the DiskLights). */
int orc_render_add_sphere_lights(orc_render* r, const orc_spherelight* lights, uint32_t n);
/* Runs core.Render iterations iter_begin .. iter_begin+iter_count-1 (the
 * reference's 0-based loop variable; each renders sample iter+1 and folds
 * it into fb as buf = (buf*(iter+1) + c)/(iter+2), core/render.go:127-129).
 * fb: w*h*3 floats, in/out.  seed: per-pixel scrambles (see orc_scramble). */
int orc_render_run(orc_render* r, uint32_t w, uint32_t h, uint32_t iter_begin, uint32_t iter_count,
                   uint64_t seed, float* fb, int nthreads);
/* Rows [row0, row0 + nrows) of the w x h image only (nrows 0: all); fb holds
 * those rows.  Each pixel is sampled as in the whole render. */
int orc_render_run_rows(orc_render* r, uint32_t w, uint32_t h, uint32_t row0, uint32_t nrows, uint32_t iter_begin,
                        uint32_t iter_count, uint64_t seed, float* fb, int nthreads);
/* The scramble k (0 lensU, 1 lensV, 2 time, 3 lambda, 4 light/glossy 0,
 * 5 light/glossy 1) of pixel pix: replaces the reference's draws from
 * math/rand (core/render.go:166-176). */
uint64_t orc_scramble(uint64_t seed, uint64_t pix, uint32_t k);

/* Extended path tracer (no reference counterpart; orc_pt.cpp restates the
 * project's own estimator).  Quad light: parallelogram p0, p0+e1, p0+e1+e2,
 * p0+e2 emitting toward e1 x e2, mesh = its emissive mesh's index. */
typedef struct {
    float p0[3], e1[3], e2[3];
    uint32_t shader, mesh;
} orc_quad_light;
typedef struct {
    uint32_t width, height, iter_begin, iter_count;
    uint64_t seed;
    uint32_t max_depth, rr_depth;
    float env[3];
} orc_pt_params;
/* precision 32: float32 shading in the CUDA kernels' operation order;
 * 64: float64 shading.  fb (float, may be NULL) and fb64 (double, may be
 * NULL) both receive the running mean buf = (buf*j + L)/(j+1). */
int orc_pt_run(const orc_render* r, const orc_quad_light* quads, uint32_t n_quads, const orc_pt_params* p,
               float* fb, double* fb64, int precision, int nthreads);
/* orc_pt_run over rows [row0, row0 + nrows) only (nrows 0: all). */
int orc_pt_run_rows(const orc_render* r, const orc_quad_light* quads, uint32_t n_quads, const orc_pt_params* p,
                    uint32_t row0, uint32_t nrows, float* fb, double* fb64, int precision, int nthreads);
/* Random number `dim` of pixel sample (pix, j = iteration + 1). */
float orc_pt_rnd(uint64_t seed, uint64_t pix, uint32_t j, uint32_t dim);
/* PolyMesh.Transform of a mesh (column-major 4x4, NULL: none); scenes and
 * renders created after the call see it. */
void orc_mesh_set_transform(orc_mesh* m, const float* xf);
/* PolyMesh.Transform of n keys (16 floats each): one key is the matrix as
 * it is; two or more are decomposed and blended at each ray's time
 * (builtin/geom/polymesh/trace.go:33-48). */
void orc_mesh_set_transform_keys(orc_mesh* m, const float* keys16, uint32_t n);
/* GeomInstance (builtin/geom/instance/instance.go): a geom tracing `of`
 * through n_keys transform keys (always decomposed, TimeKey), with the given
 * bounds (BMin/BMax of key 0).  Its hits report the instance's own id. */
orc_mesh* orc_instance_create(const orc_mesh* of, const float* keys16, uint32_t n_keys, const float bmin[3],
                              const float bmax[3]);
/* Proc (builtin/geom/proc/proc.go) holding n child geoms (meshes or
 * spheres, traced in order); a hit in child i reports child_ids[i].  n_keys
 * 0 means the identity (Proc.PreRender). */
orc_mesh* orc_proc_create(orc_mesh* const* children, const int32_t* child_ids, uint32_t n, const float* keys16,
                          uint32_t n_keys, const float bmin[3], const float bmax[3]);
/* orc_scene_create whose hits report ids[i] for meshes[i] (default i). */
orc_scene* orc_scene_create_ids(orc_mesh* const* meshes, const int32_t* ids, uint32_t n);
/* TransformDecompMatrix4 of a matrix: out = T[3], R[4] (x y z w), S[16]. */
void orc_decompose(const float* m, float* trs23);
/* The keyed transform at a time (keys decomposed, blended, rebuilt);
 * blend_one: blend a single key with itself as Camera.ComputeRay does. */
int orc_keyed_matrix(const float* keys16, uint32_t n, float time, int blend_one, float* out16);
/* Camera.LocalToWorld keys of a render (decomposed; camera.go:207-236).
 * orc_render_create decomposes the camera's m as the single key. */
int orc_render_set_camera_keys(orc_render* r, const float* keys16, uint32_t n);
/* Vec3Normalize in the reference-mode renderer: 0 exact (default), 1 an
 * emulation of the RSQRTSS estimate plus Newton step of
 * math/vec3_amd64.s:11-42, the estimate's error drawn from a hash of the
 * input and seed within the documented 1.5*2^-12 bound.  Process-wide. */
void orc_set_normalize_mode(int mode, uint64_t seed);
/* sin and cos of 2*pi*u[i] (u in [0, 1)) in the float32 operations of the
 * extended path tracer's sampling. */
void orc_sincos_turns(const float* u, size_t n, float* s, float* c);

/* Path-guiding network (orc_mlp.cpp; no reference counterpart).  Weights:
 * W0 [64][80], W1..W3 [64][64], W4 [41][64] concatenated, row-major (the 41st
 * output is the guide's selection logit).
 * precision: 64, 32, or 16 (the CUDA kernels' bfloat16 roundings with
 * float32 accumulation). */
int orc_guide_n_weights(void);
void orc_guide_features(const float* pos, const float* nrm, const float* wo, const float* lo, const float* hi, int n,
                        double* feat);
void orc_guide_forward(const float* W, const double* feat, int n, int precision, double* out);
double orc_guide_pdf(const double* out41, const double* w);
void orc_guide_out_grad(const double* out41, const double* w, double weight, double pb, double amax, double* g41,
                        double* loss);
double orc_guide_loss_grad(const float* W, const double* feat, const float* omega, const float* weight,
                           const float* bsdf_pdf, double amax, int n, int precision, double* gW);

#ifdef __cplusplus
}
#endif
#endif
