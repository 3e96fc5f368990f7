/*
 * vmr.h - C ABI of libvmr, the GB300 (sm_103a) traversal and rendering path
 * for Vermeer scenes.
 *
 * The reference renderer (jamiec7919/vermeer, Go) reaches its hot path through
 * Go interfaces: core.Scene (core/scene.go:8-24) with qbvh.Trace /
 * qbvh.TraceMotion (qbvh/intersect.go:91, qbvh/motionintersect.go:22) calling
 * PolyMesh.TraceElems / TraceMotionElems (builtin/geom/polymesh/trace.go:108,
 * :520) one ray at a time, and core.Render (core/render.go:140) looping over
 * pixels.  A per-ray callback cannot cross cgo efficiently, so this ABI takes
 * whole batches: meshes with their reference-built QBVH, SoA ray streams, and
 * whole render passes.  Every function returns a vmr_status; 0 is success.
 *
 * Threading: one context per host thread (a Go caller pins its goroutine with
 * runtime.LockOSThread).  Calls on one context are serialised on its stream;
 * contexts are independent.  No call invokes a host callback.
 */
#ifndef VMR_H
#define VMR_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VMR_ABI_VERSION 1

typedef enum {
    VMR_OK = 0,
    VMR_ERR_INVALID = -1,        /* bad argument or handle */
    VMR_ERR_CUDA = -2,           /* a CUDA runtime call failed */
    VMR_ERR_OOM = -3,            /* device or host allocation failed */
    VMR_ERR_TIMEOUT = -4,        /* a device loop hit its iteration cap */
    VMR_ERR_STACK_OVERFLOW = -5, /* a ray needed more than 90 traversal stack
                                    entries (RenderTask.Traversal.Stack,
                                    core/ray.go:158) */
    VMR_ERR_QUEUE_OVERFLOW = -6, /* a wavefront queue exceeded its capacity */
    VMR_ERR_UNSUPPORTED = -7     /* input the path does not handle */
} vmr_status;

typedef struct vmr_ctx vmr_ctx;

/* ---------------------------------------------------------------- context */
/* Replaces the process-global state of core (core/core.go:10-15): a Go host
 * creates one context per render.  device < 0 creates a host-only context
 * that builds and exports accelerators but cannot trace. */
int vmr_create(int device, vmr_ctx** out);
int vmr_destroy(vmr_ctx* ctx);
/* Message of the last failing call on ctx (owned by ctx, never NULL). */
const char* vmr_last_error(const vmr_ctx* ctx);
/* Use an external CUDA stream (a cudaStream_t) for all work of ctx; NULL
 * restores the context's own stream. */
int vmr_set_stream(vmr_ctx* ctx, void* cuda_stream);
/* Wait for the context's stream and report any device-side status
 * (stack overflow, iteration caps) raised since the last call. */
int vmr_sync(vmr_ctx* ctx);
int vmr_abi_version(void);

/* Launch parameters of the traversal kernels, chosen per scene (by hand or
 * by an autotuner).  Results never depend on them: they only change how
 * rays are scheduled onto warps.  Zero block/blocks_per_sm/refill_min take
 * the defaults. */
typedef struct {
    int kernel;          /* bit 0: while-while (else step-scheduled); bit 1:
                            L1 prefetch of the next node; bit 2: register
                            cap for 7 resident 128-thread blocks per SM (5
                            for motion meshes; while-while only); bit 3:
                            reorder rays by
                            permutation class and origin cell before a mesh
                            trace of >= 65536 rays; bit 4: the top 16
                            entries of the traversal stack in shared memory
                            (while-while); bit 5: warp-cooperative leaf
                            scan (while-while, static meshes: the warp's
                            leaves tested as one list, one triangle per
                            lane).  Default 45. */
    int block;           /* threads per block, multiple of 32, <= 256 (128) */
    int blocks_per_sm;   /* resident blocks per SM (occupancy maximum) */
    int refill_min;      /* step-scheduled: idle lanes that trigger a warp
                            refill, 1..32 (4) */
    int walk_tail;       /* while-while: end a node walk early once at most
                            this many lanes still walk and a lane holds a
                            leaf for the cooperative scan (any leaf with bit
                            5, a static leaf without it), 0..31 (default 8;
                            0 = wait for every lane) */
    int sort_bits;       /* sort-key width: the ray reordering groups origins
                            in (2^b)^3 cells, b = 3, 4 or 5 (0: 4) */
} vmr_tuning;
int vmr_set_tuning(vmr_ctx* ctx, const vmr_tuning* tuning);
int vmr_get_tuning(vmr_ctx* ctx, vmr_tuning* tuning);
/* Device time of the last trace call on ctx: the ray reordering kernels and
 * the traversal kernel, in milliseconds (waits for the trace to finish). */
int vmr_trace_timing(vmr_ctx* ctx, float* sort_ms, float* traverse_ms);

/* ------------------------------------------------------------ QBVH nodes */
/* qbvh.Node (qbvh/qbvh.go:31-36), 128 bytes, identical memory layout:
 * boxes[child + 12*(0 min|1 max) + 4*axis]; children >= 0 inner node,
 * -1 empty, else leaf (1<<31)|(first<<4)|(count-1). */
typedef struct {
    float boxes[24];
    uint32_t axis0, axis1, axis2;
    int32_t children[4];
    int32_t parent;
} vmr_qbvh_node;

/* qbvh.MotionNode (qbvh/mqbvh.go:24-29), 40 bytes. */
typedef struct {
    int32_t axis0, axis1, axis2;
    int32_t children[4];
    int32_t parent;
    uint32_t pad[2];
} vmr_mqbvh_node;

typedef enum {
    VMR_MOTION_FAITHFUL = 0, /* leaf test reads idxp at the leaf position, as
                                TraceMotionElems does (trace.go:532-537) */
    VMR_MOTION_FIXED = 1     /* leaf position mapped through accel idx, the
                                face the leaf boxes were built from */
} vmr_motion_mode;

/* --------------------------------------------------------------- meshes */
/* Raw mesh input (the PolyMesh fields after init(), polymesh/init.go):
 * verts is a key-major PointArray (motion_keys * n_verts * 3 floats), idxp
 * holds 3 vertex indices per triangle in face order. */
typedef struct {
    const float* verts;
    uint32_t n_verts;
    uint32_t motion_keys;
    const uint32_t* idxp;
    uint32_t n_tris;
    float ray_bias;               /* PolyMesh.RayBias */
    int motion_mode;              /* vmr_motion_mode */
    const uint8_t* shader_idx;    /* optional, per face in face order */
} vmr_mesh_input;

/* A mesh whose QBVH was built by the caller (the reference's
 * PolyMesh.initAccel, buildqbvh.go:14-144).  Static: nodes + accel_idx and
 * idxp already permuted to leaf order.  Motion: mnodes + mboxes
 * ([keys][n_mnodes][24]) + accel_idx, idxp in face order, plus the per-key
 * bounds (PolyMesh.motionBounds) used by the top level. */
typedef struct {
    const float* verts;
    uint32_t n_verts;
    uint32_t motion_keys;
    const uint32_t* idxp;
    uint32_t n_tris;
    const int32_t* accel_idx;
    float ray_bias;
    int motion_mode;
    const vmr_qbvh_node* nodes;
    uint32_t n_nodes;
    const vmr_mqbvh_node* mnodes;
    uint32_t n_mnodes;
    const float* mboxes;
    const float* bounds;          /* 6 floats (static) or 6*motion_keys */
    const uint8_t* shader_idx;    /* optional, per face in leaf order */
} vmr_mesh_desc;

/* An analytic sphere geom (builtin/geom/sphere: Sphere.Trace with
 * raySphereIntersect; hit attributes N = normalize(P - centre), Poffset =
 * 0.001 N).  It joins scenes and renders like a mesh (its shader is the
 * first of vmr_mesh_set_shading's list); vmr_trace_mesh does not take it. */
int vmr_sphere_add(vmr_ctx* ctx, const float center[3], float radius, uint32_t* out_geom);

/* Build the mesh's QBVH on the host exactly as PolyMesh.initAccel does
 * (binned SAH, qbvh/build.go:28-307, leafMax 16) and upload it. */
int vmr_mesh_build(vmr_ctx* ctx, const vmr_mesh_input* in, uint32_t* out_geom);
/* Which builder vmr_mesh_build uses.  Both give the same node arrays, leaf
 * order and bounds, bit for bit.  AUTO (the default) builds meshes of 16384
 * or more triangles on the device and smaller ones on the host; DEVICE
 * always builds on the device (VMR_ERR_UNSUPPORTED for build geometry that
 * is not finite); HOST always on the host (threads per upper-level subtree). */
typedef enum { VMR_BUILD_AUTO = 0, VMR_BUILD_HOST = 1, VMR_BUILD_DEVICE = 2 } vmr_builder;
int vmr_set_builder(vmr_ctx* ctx, int builder);
/* Upload a caller-built (reference-built) accelerator; the data is copied. */
int vmr_mesh_upload(vmr_ctx* ctx, const vmr_mesh_desc* desc, uint32_t* out_geom);
/* Sizes of a mesh's accelerator: static node count, motion node count. */
int vmr_mesh_info(vmr_ctx* ctx, uint32_t geom, uint32_t* n_nodes, uint32_t* n_mnodes,
                  uint32_t* n_tris, uint32_t* motion_keys);
/* Copy the host-side accelerator of a mesh (what the builder produced or the
 * caller uploaded).  Any pointer may be NULL.  bounds: 6 floats per key. */
int vmr_mesh_export(vmr_ctx* ctx, uint32_t geom, vmr_qbvh_node* nodes, int32_t* accel_idx,
                    uint32_t* idxp, vmr_mqbvh_node* mnodes, float* mboxes, float* bounds);

/* ---------------------------------------------------------------- scene */
/* Two-level scene (builtin/scene/scene.go): a top-level QBVH with leafMax 1
 * over the listed geoms (Scene.initAccel, scene.go:135-203).  Replaces any
 * previous scene of ctx. */
int vmr_scene_build(vmr_ctx* ctx, const uint32_t* geoms, uint32_t n_geoms);
/* PolyMesh.Transform with one matrix (builtin/geom/polymesh/trace.go:15-101):
 * m = the 4x4 object-to-world matrix, column-major as math.Matrix4 (m[12..14]
 * the translation); NULL removes it.  A scene trace that enters the mesh
 * maps the ray into object space with Matrix4Inverse(m) (the same float32
 * cofactor expansion; a singular m gives the zero matrix, as the reference
 * ignores its ok flag), re-runs Ray.Setup, walks the mesh and restores the
 * world ray, keeping Tclosest.  As in the reference the top level keeps the
 * mesh's object-space bounds (PolyMesh.Bounds ignores the transform) and a
 * direct vmr_trace_mesh ignores the transform (qbvh.Trace).  Renders apply
 * the hit mesh's transform as core.Trace does after the trace
 * (ShaderContext.ApplyTransform over the mesh's P = M Po, N = M^-T N):
 * P = M Po, N = normalize(M^-T M^-T N), Ng = normalize(M^-T Ng),
 * dPdu/dPdv = normalize(M dPdu/dPdv); Poffset stays in object space.  Not
 * reproduced: the reference also rewrites the context with the transform
 * of every other transformed mesh the ray enters (a leak across geoms).
 * Analytic spheres take no transform.  Takes effect in the scene at once. */
int vmr_mesh_set_transform(vmr_ctx* ctx, uint32_t geom, const float* m);
/* PolyMesh.Transform with motion keys (builtin/geom/polymesh/init.go:14-16,
 * trace.go:33-48): n_keys column-major 4x4 matrices.  One key is
 * vmr_mesh_set_transform; with two or more each key is decomposed
 * (TransformDecompMatrix4, math/animdecomp.go:20-62) and a scene trace
 * entering the mesh blends the keys around the ray's time
 * (TransformDecompLerp, animdecomp.go:74-80), rebuilds the matrix
 * (TransformDecompToMatrix4) and maps the ray by its Matrix4Inverse; renders
 * take that matrix for the hit.  Scenes holding such a mesh are traced by
 * the single-loop scene kernel (both render modes); batched jobs do not
 * take them.  n_keys = 0 removes the transform. */
int vmr_mesh_set_transform_keys(vmr_ctx* ctx, uint32_t geom, const float* keys16, uint32_t n_keys);

/* GeomInstance (builtin/geom/instance/instance.go:40-160): a new geom that
 * traces geom `of` (a mesh or sphere, itself also a geom of the scene or not)
 * through n_keys transform keys.  Every key is decomposed, and a ray's
 * transform is TransformSRTArray.TimeKey's (one key as it is, else the keys
 * around the ray's time blended), rebuilt, inverted (Matrix4Inverse); the
 * ray is mapped and re-set-up, the geom traced (through its own transform
 * too), the world ray restored.  bmin/bmax: the instance's bounds at every
 * time (BMin/BMax of key 0, instance.go:64-68); its motion keys for the top
 * level are the instanced geom's (instance.go:144-148).  Hits report the
 * instance's id (vmr_trace_scene's geom) and shade as the instanced geom with
 * the instance's transform applied to the shading context (P = T Po with Po
 * the hit point in instance space, normals by T^-T, as core.Trace's
 * ApplyTransform).  Instances of instances or Procs are not supported. */
int vmr_instance_add(vmr_ctx* ctx, uint32_t of, const float* keys16, uint32_t n_keys, const float bmin[3],
                     const float bmax[3], uint32_t* out_geom);
/* Proc (builtin/geom/proc/proc.go:50-190): a new geom holding n child geoms
 * (meshes or spheres made for it: they join no scene themselves), traced in
 * order through the Proc's transform keys (n_keys 0: the identity, as
 * Proc.PreRender sets); a closest-hit ray stops at the first child that hits
 * (proc.go:117-124), a shadow ray goes on.  A hit reports the child's id.
 * Its motion keys for the top level are its transform keys. */
int vmr_proc_add(vmr_ctx* ctx, const uint32_t* children, uint32_t n, const float* keys16, uint32_t n_keys,
                 const float bmin[3], const float bmax[3], uint32_t* out_geom);
/* Caller-built top level: static nodes, or motion nodes + boxes; geom_order
 * maps leaf position -> geom id. */
int vmr_scene_upload(vmr_ctx* ctx, const vmr_qbvh_node* nodes, uint32_t n_nodes,
                     const vmr_mqbvh_node* mnodes, uint32_t n_mnodes, const float* mboxes,
                     uint32_t motion_keys, const uint32_t* geom_order, uint32_t n_geoms);
/* Top-level export: geom_order (leaf position -> geom id), nodes or motion
 * nodes + boxes.  Any pointer may be NULL. */
int vmr_scene_export(vmr_ctx* ctx, uint32_t* geom_order, vmr_qbvh_node* nodes,
                     vmr_mqbvh_node* mnodes, float* mboxes, uint32_t* n_nodes,
                     uint32_t* n_mnodes, uint32_t* motion_keys);

/* ---------------------------------------------------------------- trace */
/* Structure-of-arrays ray stream (the traversal inputs of core.Ray,
 * core/ray.go:27-51).  time may be NULL (time 0). */
typedef struct {
    const float *px, *py, *pz;
    const float *dx, *dy, *dz;
    const float *tmax;
    const float *time;
} vmr_rays;

/* Hit stream.  prim = ShaderContext.ElemID (leaf-order triangle index for
 * static meshes, -1 on a miss); geom = hit geom id (scene traces); t =
 * Ray.Tclosest after the trace; u,v,w = barycentrics of the accepted hit.
 * Any pointer may be NULL. */
typedef struct {
    int32_t* prim;
    int32_t* geom;
    float *t, *u, *v, *w;
} vmr_hits;

typedef enum {
    VMR_TRACE_CLOSEST = 0,
    VMR_TRACE_ANY_HIT = 1,   /* RayTypeShadow: stop at the first hit leaf
                                (intersect.go:231-236) */
    VMR_TRACE_DEVICE = 2,    /* ray and hit pointers are device pointers;
                                the call is asynchronous on ctx's stream */
    VMR_TRACE_COUNT = 4      /* fill the visit counters of vmr_trace_stats */
} vmr_trace_flags;

typedef struct {
    uint64_t rays;
    uint64_t node_visits;    /* Ray.NodesT summed over rays */
    uint64_t leaf_visits;    /* Ray.LeafsT summed over rays */
    uint64_t tri_tests;
    float kernel_ms;         /* device time of the traversal kernel (host-pointer
                                calls; use vmr_trace_timing for device ones) */
} vmr_trace_stats;

/* Closest-hit / any-hit traversal of one mesh (PolyMesh.Trace without a
 * transform, trace.go:57-101).  Host pointers (default): the call copies
 * rays in and hits out and returns when done.  stats may be NULL. */
int vmr_trace_mesh(vmr_ctx* ctx, uint32_t geom, const vmr_rays* rays, size_t n, int flags,
                   const vmr_hits* hits, vmr_trace_stats* stats);
/* Traversal of the two-level scene (Scene.Trace, scene.go:30-58). */
int vmr_trace_scene(vmr_ctx* ctx, const vmr_rays* rays, size_t n, int flags,
                    const vmr_hits* hits, vmr_trace_stats* stats);

/* Batched jobs (no reference counterpart: the reference renders one scene
 * per process).  Each job traces n rays against one mesh, static or motion;
 * the jobs' rays are gathered into one stream with a per-ray job index, one
 * persistent traversal launch (the scene kernel's job mode: each ray enters
 * its job's mesh directly; the context's tuning) traces them all, and the
 * hits are scattered back, so jobs of very uneven size share the GPU
 * without one launch each.  Results equal vmr_trace_mesh per job (a mesh's
 * transform is not applied, as there).  Rays and hits are device pointers
 * (the call is asynchronous unless stats is given). */
typedef struct {
    uint32_t geom;
    uint32_t pad;
    size_t n;
    vmr_rays rays;
    vmr_hits hits;
} vmr_trace_job;
int vmr_trace_jobs(vmr_ctx* ctx, const vmr_trace_job* jobs, uint32_t n_jobs, int flags, vmr_trace_stats* stats);

/* The autotuner: times every candidate launch configuration (kernel variant,
 * block size, resident blocks, walk-tail cutoff, sort-key width) on a sample
 * of rays for one mesh, keeps the fastest for that mesh (vmr_trace_mesh uses
 * it from then on instead of the context's tuning) and
 * returns it.  rays: host pointers, or device pointers with
 * VMR_TRACE_DEVICE in flags; the sample should be a few hundred thousand
 * rays of the kind the mesh will see.  best_ms (may be NULL) receives the
 * winner's traversal time; n_tried (may be NULL) the candidates timed. */
int vmr_autotune(vmr_ctx* ctx, uint32_t geom, const vmr_rays* rays, size_t n, int flags, vmr_tuning* best,
                 float* best_ms, uint32_t* n_tried);
/* Forget a mesh's own tuning (it falls back to the context's). */
int vmr_clear_tuning(vmr_ctx* ctx, uint32_t geom);

/* ----------------------------------------------------------------- render */
/* ShaderStd parameters (builtin/shader/std.go:25-47).  The reference leaves
 * an unset parameter nil, which changes its default; flags say which are
 * set.  spec1_fresnel: 0 Dielectric (also the default), 1 Metal. */
enum {
    VMR_SH_EMISSION_COLOUR = 1, VMR_SH_EMISSION_STRENGTH = 2,
    VMR_SH_DIFFUSE_COLOUR = 4, VMR_SH_DIFFUSE_STRENGTH = 8, VMR_SH_DIFFUSE_ROUGHNESS = 16,
    VMR_SH_SPEC1_COLOUR = 32, VMR_SH_SPEC1_STRENGTH = 64, VMR_SH_SPEC1_ROUGHNESS = 128,
    VMR_SH_FRESNEL_REFL = 256, VMR_SH_FRESNEL_EDGE = 512, VMR_SH_IOR = 1024,
    /* DebugShader (builtin/shader/debug.go:16-57) instead of ShaderStd: the
     * surface's colour is diffuse_colour (Colour) and nothing else (no
     * lights, no emission); reference mode (vmr_render) only */
    VMR_SH_DEBUG = 2048
};
typedef struct {
    uint32_t flags;
    float emission_colour[3], emission_strength;
    float diffuse_colour[3], diffuse_strength, diffuse_roughness;
    float spec1_colour[3], spec1_strength, spec1_roughness;
    int spec1_fresnel;
    float spec1_fresnel_refl[3], spec1_fresnel_edge[3];
    float ior;
} vmr_shader_std;

/* TriLight (builtin/light/triangle.go:18-28): geom is the light's own
 * emissive mesh (Tri.createMesh, triangle.go:537-565), which shading
 * excludes from the light list when it is the hit geom (scene.go:100-116). */
typedef struct {
    float p0[3], p1[3], p2[3];
    int samples;           /* NumSamples = 1 << samples (default 1) */
    uint32_t shader;
    uint32_t geom;
} vmr_tri_light;

/* DiskLight (builtin/light/disk.go:18-31): a disk of the given radius at P
 * facing LookAt; geom is its emissive fan mesh (Disk.createMesh, 20 segments
 * by default). */
typedef struct {
    float P[3], up[3], lookat[3];
    float radius;
    int samples;           /* NumSamples = 1 << samples (default 1) */
    uint32_t shader;
    uint32_t geom;
} vmr_disk_light;

/* SphereLight (builtin/light/sphere.go:14-28): cone sampling toward the
 * sphere (pdf q_2 of Shirley et al. 1996); geom is its sphere geom
 * (vmr_sphere_add).  Lights are used in the order TriLights, DiskLights,
 * SphereLights. */
typedef struct {
    float P[3];
    float radius;
    int samples;
    uint32_t shader;
    uint32_t geom;
} vmr_sphere_light;

/* Camera (builtin/camera/camera.go): m = LocalToWorld, column-major;
 * tan_theta_focal = tan(fov/2) * focal; radius > 0 is a thin lens sampled
 * with UniformDisk2D (math/sample/sample.go:105-129). */
typedef struct {
    float m[16];
    float tan_theta_focal, aspect, focal, radius;
} vmr_camera;

typedef struct {
    uint32_t width, height;
    uint32_t iter_begin, iter_count;  /* core.Render loop iterations */
    uint64_t seed;                    /* per-pixel scrambles */
    uint32_t max_batch_samples;       /* samples per wavefront batch (0: 4M) */
    /* A band of the image's rows: rows [row_begin, row_begin + row_count) of
     * the width x height image, fb holding just those rows; each pixel's
     * samples are the full render's, so the bands of a split render put
     * together are the one-call image bit for bit.  row_count 0: all rows. */
    uint32_t row_begin, row_count;
    uint32_t flags;                   /* VMR_RENDER_* */
} vmr_render_params;
enum {
    /* The shading's transcendentals (light and BSDF sampling, Oren-Nayar,
     * the spherical-triangle sampling) in float32 instead of the reference's
     * float64-rounded-to-float32 (math/sincos.go): off the FP64 pipe, no
     * longer bit-exact with the oracle; the image stays within the stated
     * tolerance of the float64 one. */
    VMR_RENDER_F32 = 1
};

typedef struct {
    uint64_t samples;      /* pixel samples rendered */
    uint64_t camera_rays;  /* primary rays traced */
    uint64_t shadow_rays;  /* shadow rays traced */
    float ms;              /* device time of the render */
} vmr_render_stats;

/* Material table (index = shader id). */
int vmr_set_shaders(vmr_ctx* ctx, const vmr_shader_std* shaders, uint32_t n);
/* PolyMesh.Shader (the mesh's shader ids; faces pick one through the
 * shader_idx given at build) and optional per-vertex normals (key 0) of a
 * static mesh; a motion mesh's normals go through
 * vmr_mesh_set_motion_normals (VMR_ERR_UNSUPPORTED here). */
int vmr_mesh_set_shading(vmr_ctx* ctx, uint32_t geom, const uint32_t* shaders, uint32_t n_shaders,
                         const float* normals);
/* Per-key normals of a motion mesh: PolyMesh.Normals with as many motion
 * keys as the vertices (builtin/geom/polymesh/trace.go:694-712).
 * normals[key][i] are 3 floats, n_per_key entries a key, keys = the mesh's
 * keys.  A hit on element e reads entries 3e .. 3e + 2 of the two keys
 * around the ray's time (directly, not through NormalIdx), lerps them and
 * interpolates them with the hit's barycentrics; without them a motion
 * hit's N is Ng.  n_per_key must be at least 3 x the mesh's triangles.
 * NULL removes them.  VMR_ERR_INVALID for a static mesh, another key count
 * or too few entries. */
int vmr_mesh_set_motion_normals(vmr_ctx* ctx, uint32_t geom, const float* normals, uint32_t n_per_key,
                                uint32_t keys);
int vmr_set_lights(vmr_ctx* ctx, const vmr_tri_light* lights, uint32_t n);
int vmr_set_disk_lights(vmr_ctx* ctx, const vmr_disk_light* lights, uint32_t n);
int vmr_set_sphere_lights(vmr_ctx* ctx, const vmr_sphere_light* lights, uint32_t n);
/* The camera (Camera node, builtin/camera/camera.go): m is LocalToWorld.  As
 * the reference does, the ray is made with the matrix rebuilt from m's
 * decomposition (TransformDecompMatrix4, then TransformDecompToMatrix4 of
 * TransformDecompLerp of that key with itself, camera.go:207-236), which is
 * close to m but not equal to it. */
int vmr_set_camera(vmr_ctx* ctx, const vmr_camera* camera);
/* Camera motion keys: LocalToWorld as n_keys column-major 4x4 matrices
 * (after vmr_set_camera, whose other fields stay).  Each key is decomposed;
 * a sample at time t (the VdC time of core/render.go:94) takes
 * k = t*(n-1) and blends keys floor(k), ceil(k) at k - floor(k)
 * (camera.go:223-236).  vmr_get_camera returns key 0 in m. */
int vmr_set_camera_keys(vmr_ctx* ctx, const float* keys16, uint32_t n_keys);
/* The matrix libvmr uses for n_keys transform keys at a time: each key
 * decomposed (TransformDecompMatrix4), the keys around time blended
 * (TransformDecompLerp), the matrix rebuilt (TransformDecompToMatrix4); one
 * key is rebuilt as it is unless blend_one (the camera blends it with
 * itself).  Host-side, needs no context or GPU; VMR_ERR_INVALID if time
 * falls outside the keys. */
int vmr_transform_keys_at(const float* keys16, uint32_t n_keys, float time, int blend_one, float* out16);
/* The camera's LocalToWorld keys as set or loaded: *n_keys receives their
 * number, keys16 (may be NULL) the first min(n, cap) of them. */
int vmr_get_camera_keys(vmr_ctx* ctx, float* keys16, uint32_t cap, uint32_t* n_keys);

/* Pixel filters for filter importance sampling: replaces core.Init of a
 * PixelFilter node (core/core.go:88-89, core/pixelfilter.go:8-10) with the
 * GaussianFilter and AiryFilter nodes (builtin/filter/gauss.go, airy.go).
 * The sample's position inside its pixel (the fractional part of the
 * RasterXY coordinates) is warped by the filter's tabulated distribution
 * (Sampler.WarpSample, builtin/filter/filter.go:40-80, tables built as
 * CreateSampler does, filter.go:87-166) before the camera ray is made
 * (core/render.go:99-107); the sample still lands in its own pixel's
 * running mean.  Applies to vmr_render and vmr_render_path.  res, width
 * and peak <= 0 take the nodes' defaults (Gaussian res 17, width 2; Airy
 * res 49, width 6, peak 4).  Note: the Airy filter at an odd res samples its
 * centre, where 2 J1(v)/v is 0/0; as in the reference, the table is then
 * NaN and every sample stays at its pixel's centre. */
enum {
    VMR_FILTER_BOX = 0,       /* no warp (no PixelFilter node) */
    VMR_FILTER_GAUSSIAN = 1,
    VMR_FILTER_AIRY = 2
};
typedef struct {
    int kind;
    int res;       /* table resolution (Res), >= 2 */
    float width;   /* Width */
    float peak;    /* Peak (Airy only) */
} vmr_pixel_filter;
int vmr_set_pixel_filter(vmr_ctx* ctx, const vmr_pixel_filter* filter);
/* The filter's Sampler.WarpSample (builtin/filter/filter.go:40-80,
 * core.PixelFilter.WarpSample, core/pixelfilter.go:8-10) on the host, for n
 * sample pairs (r0, r1) in [0, 1): the offsets (u, v) from the pixel centre
 * that the camera kernels apply.  Needs no context or GPU. */
int vmr_pixel_filter_warp(const vmr_pixel_filter* filter, const double* r0, const double* r1, size_t n, double* u,
                          double* v);

/* ------------------------------------------------------------ scene files */
/* A .vnf scene file into ctx: replaces nodes.Parse (nodes/lex.go,
 * nodes/parser.go) and core.PreRender (core/core.go:29-104) for the node
 * types the GPU path renders: Globals, Camera (LookAt, or LocalToWorld),
 * PolyMesh (PolyCount/FaceIdx fan triangulation, ShaderIdx, Normals and
 * NormalIdx, motion keys in Verts; polymesh/init.go), Sphere, ShaderStd
 * (rgb and float maps), TriLight, DiskLight, SphereLight, QuadLight (the
 * extended mode's quad light; the reference's panics), GaussianFilter,
 * AiryFilter, OutputHDR, OutputFloat.  Geoms are taken in file order, then
 * the lights' own meshes in light order, as the reference adds them; each
 * goes through vmr_mesh_build / vmr_sphere_add and then vmr_scene_build,
 * the material, light, camera and filter setters.  Lights are grouped by
 * kind (TriLights, DiskLights, SphereLights) in file order within a kind.
 * Errors the reference prints and skips stop the load here:
 * VMR_ERR_INVALID with "file:line: message" in vmr_last_error; DebugShader,
 * Proc, GeomInstance, rgbtex textures, non-identity PolyMesh transforms and
 * camera motion keys give VMR_ERR_UNSUPPORTED.  flags: VMR_VNF_MOTION_FIXED
 * builds motion meshes in VMR_MOTION_FIXED mode (default: faithful).
 * Works on host-only contexts too (parsing and accelerator builds). */
enum { VMR_VNF_MOTION_FIXED = 1 };
typedef struct {
    uint32_t width, height;   /* Globals XRes, YRes (1024 x 1024 without a Globals node) */
    int max_iter;             /* Globals MaxIter (16 without a Globals node; 0 = until stopped) */
    uint32_t n_geoms, n_shaders, n_lights;
    char camera[64];          /* the render's camera node */
    char output_hdr[256];     /* OutputHDR Filename ("" if none) */
    char output_float[256];   /* OutputFloat Filename ("" if none) */
} vmr_vnf_info;
int vmr_load_vnf(vmr_ctx* ctx, const char* path, int flags, vmr_vnf_info* info);
/* The camera the context renders with (as set or loaded). */
int vmr_get_camera(vmr_ctx* ctx, vmr_camera* camera);

/* ------------------------------------------------------- output drivers */
/* The OutputHDR driver's pixel bytes, encoded on the device: replaces the
 * loop of image/hdr/writer.go:58-82 (called by OutputHDR.PostRender,
 * builtin/driver/outputhdr.go:26-55) over core.FrameBuf().  rgb: the
 * width*height*3 float framebuffer (row-major, top row first, as vmr_render
 * and vmr_render_path write it); rgbe: width*height*4 bytes in the file's
 * order, scanline j = image row height-1-j, each pixel convertRGBToRGBE's
 * (r, g, b, e) (image/hdr/hdr.go:28-55, float32 arithmetic, Go's byte
 * conversions).  The caller writes the text header ("#?RADIANCE",
 * "FORMAT=32-bit_rle_rgbe", "+Y h +X w") and then these bytes.  Flags:
 * VMR_IO_DEVICE_IN / VMR_IO_DEVICE_OUT mark rgb / rgbe as device pointers
 * (otherwise host memory, copied inside the call). */
enum {
    VMR_IO_DEVICE_IN = 1,
    VMR_IO_DEVICE_OUT = 2
};
int vmr_encode_rgbe(vmr_ctx* ctx, const float* rgb, uint32_t width, uint32_t height, int flags, uint8_t* rgbe);
/* core.Render in reference mode (core/render.go:140-218 with ShaderStd's
 * direct lighting): iterations iter_begin..iter_begin+iter_count-1 of every
 * pixel, folded into fb (host, width*height*3 floats, in/out) as
 * buf = (buf*(iter+1) + c)/(iter+2).  Needs the scene (vmr_scene_build)
 * over every mesh, light meshes included. */
int vmr_render(vmr_ctx* ctx, const vmr_render_params* params, float* fb, vmr_render_stats* stats);

/* ------------------------------------------------- extended path tracing */
/* No counterpart in the reference, which renders direct light only (plus
 * mirror recursion) and has no environment light; its QuadLight panics in
 * ValidSample (builtin/light/quad.go:87-89).  The extended mode is a unidirectional
 * path tracer over the same scene, materials, TriLights and camera:
 *   - indirect bounces up to max_depth scattering events, Russian roulette
 *     from rr_depth on (survival min(0.95, max throughput));
 *   - next-event estimation with one light picked uniformly from TriLights,
 *     quad lights and the environment, combined with BSDF sampling by the
 *     power heuristic;
 *   - ShaderStd as the mixture dw*Diffuse + sw*GGX (weights normalised;
 *     diffuse roughness 0 = Lambert, else OrenNayar; GGX alpha =
 *     Spec1Roughness^4 as the reference's, sampled by the visible-normal-free
 *     D(m)cos(m) method with the correct 1/(4|wo.m|) Jacobian; roughness 0
 *     = a perfect mirror); surfaces are two-sided, emitters one-sided;
 *   - RGB throughout (no hero wavelength); camera rays equal reference mode's;
 *   - per-sample random numbers from a counter-based SplitMix64 hash of
 *     (seed, pixel, iteration, dimension).
 * A quad light is the parallelogram p0, p0+e1, p0+e1+e2, p0+e2 emitting on the
 * side of e1 x e2; geom is its emissive mesh (two triangles with that
 * winding), uploaded by the caller. */
typedef struct {
    float p0[3], e1[3], e2[3];
    uint32_t shader;
    uint32_t geom;
} vmr_quad_light;

int vmr_set_quad_lights(vmr_ctx* ctx, const vmr_quad_light* lights, uint32_t n);
/* Constant environment radiance seen by rays that leave the scene (0,0,0:
 * no environment light). */
int vmr_set_env_light(vmr_ctx* ctx, const float radiance[3]);

typedef struct {
    uint32_t width, height;
    uint32_t iter_begin, iter_count;  /* iterations (one sample per pixel each) */
    uint64_t seed;
    uint32_t max_depth;               /* scattering events per path */
    uint32_t rr_depth;                /* Russian roulette from this event on */
    uint32_t max_batch_samples;       /* paths per wavefront batch (0: the
                                         context's, vmr_set_path_batch) */
    uint32_t flags;                   /* VMR_PATH_* */
    double* fb64;                     /* optional host width*height*3: the same
                                         running mean folded in float64 */
    float guide_fraction;             /* VMR_PATH_GUIDED: alpha_max, the largest
                                         probability of sampling the guide at a
                                         vertex; each vertex's probability is
                                         alpha_max * sigmoid(the network's
                                         selection output) (0: 0.9); with
                                         VMR_PATH_FIXED_SELECTION the
                                         probability itself (0: 0.5) */
    uint32_t train_steps;             /* VMR_PATH_TRAIN: Adam steps after each
                                         batch (0: 4) */
    uint32_t train_batch;             /* training records per step (0: 65536) */
    float train_lr;                   /* Adam learning rate (0: 1e-3) */
    uint32_t guide_depth;             /* VMR_PATH_GUIDED: guide (and, with TRAIN,
                                         record) only the first guide_depth
                                         vertices of a path; deeper vertices
                                         sample the BSDF alone (0: all) */
    uint32_t row_begin, row_count;    /* a band of rows, as vmr_render_params
                                         (0: all rows); not with VMR_PATH_TRAIN
                                         (a band would train on its rows only) */
} vmr_path_params;

enum {
    VMR_PATH_NO_GRAPH = 1,  /* launch the bounce loop stage by stage instead
                               of replaying its CUDA graph */
    VMR_PATH_GUIDED = 2,    /* one-sample MIS of the guide (vmr_guide_*) and the
                               BSDF at every non-mirror vertex; the density of
                               the mixture enters the NEE and emission weights,
                               so the estimator stays unbiased */
    VMR_PATH_TRAIN = 4,     /* record (vertex, sampled direction, density,
                               incident radiance) and train the guide on them
                               after each batch (online) */
    VMR_PATH_SORT_QUEUES = 8, /* batches of >= 65,536 paths: trace each bounce
                               and shadow queue in ray-key order (direction
                               class + Morton cell of the origin, the
                               tuning's sort-key width); images unchanged */
    VMR_PATH_FIXED_SELECTION = 16, /* VMR_PATH_GUIDED: every vertex samples the
                               guide with probability guide_fraction (the
                               network's selection output unused, and with
                               TRAIN the guide is fitted to the product
                               alone, not to the vertex's full density) */
    VMR_PATH_TWO_LEVEL = 32 /* trace the two-level scene even when it can be
                               flattened: by default a scene of static,
                               untransformed triangle meshes with one ray bias
                               is traced as one mesh over all its triangles
                               (built once per scene by the device builder),
                               its hits mapped back to (geom, triangle); the
                               closest hit is the same triangle either way
                               (only exact ties in t between two triangles may
                               resolve differently) */
};

typedef struct {
    uint64_t samples;        /* pixel samples (paths) */
    uint64_t rays;           /* extension rays traced (camera rays included) */
    uint64_t shadow_rays;
    uint32_t graph_replays;  /* batches run by replaying the captured graph */
    float ms;                /* device time */
    uint64_t train_records;  /* training records collected */
    uint32_t train_steps;    /* Adam steps taken */
    float train_loss;        /* loss of the last step over its weight sum */
} vmr_path_stats;

/* Iterations iter_begin..iter_begin+iter_count-1 of every pixel folded into
 * fb (host, width*height*3 floats, in/out) as buf = (buf*i + L)/(i+1),
 * i = the 0-based iteration: the exact mean of the samples (the reference's
 * fold starts at i+1 and so counts the initial buffer as a sample, F6). */
int vmr_render_path(vmr_ctx* ctx, const vmr_path_params* params, float* fb, vmr_path_stats* stats);

/* ------------------------------------------------------- several GPUs */
/* One image over n contexts (each on its own GPU, each holding the same
 * scene, camera, lights and settings): the reference's tile split of a
 * render (core/render.go:184-204) across devices.  The rows are cut into n
 * contiguous bands (vmr_split_rows); context i renders band i
 * (row_begin/row_count) on its own host thread straight into its rows of fb
 * (width*height*3 floats, folded into as vmr_render does).  Every pixel is
 * sampled and folded by one context only, exactly as in a one-context
 * render, so the image is that render's bit for bit; no framebuffer
 * reduction is needed.  params' row_count must be 0.  Stats sum over the
 * bands; ms is the slowest band's. */
int vmr_render_split(vmr_ctx* const* ctxs, uint32_t n, const vmr_render_params* params, float* fb,
                     vmr_render_stats* stats);
/* The same for the extended path tracer (fb64 split alike); not with
 * VMR_PATH_TRAIN (each band would train its own guide on its rows); a
 * guided render needs the same guide weights in every context. */
int vmr_render_path_split(vmr_ctx* const* ctxs, uint32_t n, const vmr_path_params* params, float* fb,
                          vmr_path_stats* stats);
/* The bands of a split: height rows into n contiguous bands, the first
 * height % n of them one row taller.  Host-side, needs no context or GPU. */
int vmr_split_rows(uint32_t height, uint32_t n, uint32_t* row_begin, uint32_t* row_count);

/* Queue capacity (paths per wavefront batch, whole iterations) of the
 * context's one-scene renders when params.max_batch_samples is 0.
 * vmr_set_path_batch: set it (0: the default, 16M paths; else >= 1024).
 * vmr_autotune_path: render params' iterations (GUIDED sampled, TRAIN and
 * fb64 ignored; no framebuffer of the caller is touched) at candidate
 * capacities of 256K..32M paths, each after an untimed call, and keep the
 * fastest; candidates/ms (optional, room for 8) receive the capacities
 * timed and their device times.  A tuned capacity changes no image: any
 * batch split gives the same bits. */
int vmr_set_path_batch(vmr_ctx* ctx, uint32_t paths);
int vmr_get_path_batch(vmr_ctx* ctx, uint32_t* paths);
int vmr_autotune_path(vmr_ctx* ctx, const vmr_path_params* params, uint32_t* candidates, float* ms,
                      uint32_t* n_candidates, uint32_t* best);

/* Batched path-traced jobs (no reference counterpart: the reference renders
 * one scene per process).  Every job is its own one-mesh scene: its mesh
 * (static or motion, with its shading set by vmr_mesh_set_shading), camera
 * and image; the jobs share the material table and the environment light
 * (their only light).  The static jobs' paths run through one set of
 * wavefront launches (one per stage and bounce), the motion jobs' through a
 * second; a path's rays trace only its job's mesh.  Each job's image equals vmr_render_path of that mesh alone as the
 * scene, with the same params (seed, iterations, depths), bit for bit.
 * params: width/height are ignored (per job), GUIDED and fb64 are not
 * supported.  fb: width*height*3 floats per job (host), in/out. */
typedef struct {
    uint32_t geom;
    uint32_t width, height;
    vmr_camera camera;
    float* fb;
} vmr_path_job;
int vmr_render_path_jobs(vmr_ctx* ctx, const vmr_path_job* jobs, uint32_t n_jobs, const vmr_path_params* params,
                         vmr_path_stats* stats);

/* ------------------------------------------------------------ path guide */
/* No counterpart in the reference.  A small MLP proposes directions at path
 * vertices: inputs = the hit point normalised to the scene bounds [lo, hi]
 * encoded with 12 sin/cos frequencies per axis, the shading normal and the
 * direction toward the previous vertex (78 values, plus a constant 1);
 * 4 hidden ReLU layers of 64; 41 outputs = 8 von Mises-Fisher lobes
 * (direction, concentration, mixture logit) and the selection logit s: a
 * vertex samples the guide with probability alpha = alpha_max * sigmoid(s)
 * and its BSDF otherwise.  Weights: W0 [64][80], W1..W3 [64][64], W4 [41][64]
 * row-major, concatenated (VMR_GUIDE_WEIGHTS floats); the kernels run them
 * on the tensor cores in bf16 with float32 accumulation.  Vertex arrays are
 * host pointers to n x 3 floats. */
#define VMR_GUIDE_WEIGHTS 20032
#define VMR_GUIDE_OUTPUTS 41

typedef struct {
    float lr, beta1, beta2, eps;
} vmr_adam;

/* He-uniform initial weights from a seed (the output layer scaled by 0.1);
 * resets the optimiser. */
int vmr_guide_init(vmr_ctx* ctx, uint64_t seed);
/* Self-test of the kernels' failure path: a one-block kernel waits, with the
 * guide kernels' bounded mbarrier wait, on a barrier that nothing arrives
 * at.  The wait runs out (after one second), the kernel sets the
 * error word and returns, and the call reports VMR_ERR_TIMEOUT with the
 * kernel's duration in *ms (optional); the context stays usable.  Any other
 * status means the bound did not work as designed. */
int vmr_selftest_wait(vmr_ctx* ctx, float* ms);
int vmr_guide_set_weights(vmr_ctx* ctx, const float* weights);
int vmr_guide_get_weights(vmr_ctx* ctx, float* weights);
/* The 41 outputs of n vertices (out: n x 41 floats). */
int vmr_guide_forward(vmr_ctx* ctx, const float* pos, const float* nrm, const float* wo, size_t n,
                      const float lo[3], const float hi[3], float* out);
/* Gradient of sum_i -weight_i * log q_i(omega_i) with respect to the weights
 * (grad: VMR_GUIDE_WEIGHTS floats) and the loss itself; omega: n x 3 unit
 * directions, weight: n floats.  bsdf_pdf (n floats, optional): the BSDF's
 * density of each omega_i; with it q_i is the vertex's full sampling density
 * alpha_i p_guide + (1 - alpha_i) p_bsdf, alpha_i = alpha_max * sigmoid(s_i)
 * (alpha_max in (0, 1)), and the selection logit is trained too; without it
 * q_i is the guide's own density.  The weights are not changed. */
int vmr_guide_gradient(vmr_ctx* ctx, const float* pos, const float* nrm, const float* wo, const float* omega,
                       const float* weight, const float* bsdf_pdf, float alpha_max, size_t n, const float lo[3],
                       const float hi[3], float* grad, float* loss);
/* One Adam step on that loss divided by the sum of the weights. */
int vmr_guide_train_step(vmr_ctx* ctx, const float* pos, const float* nrm, const float* wo, const float* omega,
                         const float* weight, const float* bsdf_pdf, float alpha_max, size_t n, const float lo[3],
                         const float hi[3], const vmr_adam* opt, float* loss);

/* -------------------------------------------------------------- no-alloc */
/* No counterpart in the reference.  For callers that must not have a library
 * allocate device memory while they run (they manage the whole device
 * themselves, or cannot afford an allocation's synchronisation in their
 * loop): the same trace as vmr_trace_mesh with device pointers (the mesh's
 * own tuning, autotuned or the context's), but every scratch buffer (work
 * counter, status word, ray-reordering buffers) lives in one static device
 * array of about 11 MB that stays on the GPU until the process exits.
 * vmr_create resolves that array on its device (this is where the array is
 * loaded onto the GPU); the call itself allocates nothing.
 *   - flags must hold VMR_TRACE_DEVICE (rays and hits are device or managed
 *     memory; anything else fails with VMR_ERR_INVALID before any launch) and
 *     may add VMR_TRACE_ANY_HIT;
 *   - at most VMR_NOALLOC_MAX_RAYS rays per call (larger batches fail with
 *     VMR_ERR_INVALID);
 *   - all calls share the one array: calls that overlap on the GPU (other
 *     host threads, other streams, other contexts of the process on the same
 *     device) race and corrupt each other's results;
 *   - the call waits on the context's stream and returns when the trace has
 *     finished. */
#define VMR_NOALLOC_MAX_RAYS 262144
int vmr_trace_mesh_noalloc(vmr_ctx* ctx, uint32_t geom, const vmr_rays* rays, size_t n, int flags,
                           const vmr_hits* hits);

#ifdef __cplusplus
}
#endif
#endif
