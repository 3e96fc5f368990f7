// device.h - device-side data layout of libvmr (shared by host and kernels).
//
// HBM layout of one mesh (all arrays 128-byte aligned, resident for the
// lifetime of the context):
//   static mesh
//     GNode   nodes[n_nodes]       128 B: the 24 child-box floats of qbvh.Node
//                                  as 6 float4 (minx,miny,minz,maxx,maxy,maxz
//                                  over the 4 children), children as int4,
//                                  split axes packed in one word
//     float4  tris[3*n_tris]       leaf order: v0,v1,v2 (w unused), 48 B per
//                                  triangle, so a leaf is one contiguous run
//   motion mesh
//     MNode   mnodes[n_mnodes]     32 B: children int4 + packed axes
//     float4  mboxes[keys][n][6]   96 B per node per key
//     float4  mtris[keys][3*n]     leaf-position order, per key
//     int32   elem[n]              leaf position -> reported ElemID
#pragma once
#include <cstdint>

#include "animdecomp.h"

#ifndef __CUDACC__
struct float4_host { float x, y, z, w; };
#endif

namespace vmr {

// Leaf code in GNode/MNode children: bit 31 set, bits 4..30 first element,
// bits 0..3 count-1.  -1 is an empty child.  The reference packs the first
// element into 23 bits (LeafBase, qbvh/qbvh.go:64); the device format keeps
// 27, the upload path checks that reference trees decode unchanged.
constexpr int32_t kEmptyChild = -1;

struct alignas(128) GNode {
  float box[24];        // box[c + 4*axis] = min, box[12 + c + 4*axis] = max
  int32_t child[4];
  uint32_t axes;        // axis0 | axis1<<2 | axis2<<4
  uint32_t rank[2];     // push rank of each child per ray octant: byte o
                        // (o = sign bits of D) holds rank(c) at bits 2c
  uint32_t pad;
};
static_assert(sizeof(GNode) == 128, "GNode must be 128 bytes");

struct alignas(32) MNode {
  int32_t child[4];
  uint32_t axes;
  uint32_t rank[2];
  uint32_t pad;
};
static_assert(sizeof(MNode) == 32, "MNode must be 32 bytes");

// One mesh as the kernels see it.
struct DMesh {
  const GNode* nodes;       // static
  const void* tris;         // float4[3*n_tris] (static)
  const MNode* mnodes;      // motion
  const void* mboxes;       // float4[keys][n_mnodes][6]
  const void* mtris;        // float4[keys][3*n_tris]
  const int32_t* elem;      // motion: leaf position -> ElemID
  uint32_t n_tris;
  uint32_t n_mnodes;
  uint32_t keys;            // 1 = static
  float lower_static;       // EpsilonFloat32 + RayBias (trace.go:182)
  float ray_bias;           // motion lower bound (trace.go:612)
  uint32_t iter_cap;        // 4 * nodes + 2: a traversal pops each entry once
  uint32_t kind;            // kTriangles, kSphere, or kGroup
  float sphere[4];          // centre, radius
  uint32_t has_xf;          // PolyMesh.Transform: rays enter through xf_inv
  uint32_t xf_nkeys;        // >= 2: the transform is blended per ray from xf_keys
  uint32_t pad;
  // Matrix4Inverse of the transform, columns 0..3 rows 0..2 (column-major
  // elements 0,1,2, 4,5,6, 8,9,10, 12,13,14)
  float xf_inv[12];
  const anim::Decomp* xf_keys;  // decomposed transform keys (xf_nkeys >= 2)
  // kGroup (GeomInstance: group 1, Proc: group 2): the transform (has_xf /
  // xf_keys as above), the geoms traced in order and the geom id a hit in
  // each reports
  const uint32_t* children;
  const int32_t* child_hit;
  uint32_t n_children;
  uint32_t group;
};
enum MeshKind : uint32_t { kTriangles = 0, kSphere = 1, kGroup = 2 };

// Top level of a scene (builtin/scene): static GNodes or motion MNodes with
// boxes; leaves index geom_order (leaf position -> geom id).
struct DTop {
  const GNode* nodes;
  const MNode* mnodes;
  const void* mboxes;
  const uint32_t* geom_order;
  const DMesh* meshes;      // indexed by geom id
  uint32_t keys;
  uint32_t n_mnodes;
  uint32_t n_geoms;
  uint32_t iter_cap;
  uint32_t all_static;  // static top level and only static meshes: the
                        // while-while scene kernel applies
  uint32_t simple_only; // instances, Procs or keyed transforms: the
                        // single-loop scene kernel only
};

struct RaySoA {
  const float *px, *py, *pz, *dx, *dy, *dz, *tmax, *time;
  // If set: the rays as two 16-byte records each, (px, py, pz, dx) and
  // (dy, dz, tmax, input index as bits), the key-ordered copy of a static
  // mesh trace (the arrays above are then unused; time is 0)
  const void* rec = nullptr;
};
struct HitSoA {
  int32_t* prim;
  int32_t* geom;
  float *t, *u, *v, *w;
};

// Device scratch of one context: the persistent kernels' work counter, the
// status word and the visit counters (reset before every launch).
struct DScratch {
  unsigned long long next_ray;
  int status;
  int pad;
  unsigned long long node_visits;
  unsigned long long leaf_visits;
  unsigned long long tri_tests;
};

enum DeviceStatus : int {
  kStatusOk = 0,
  kStatusStackOverflow = 1,
  kStatusIterationCap = 2,
};

constexpr int kStackCapacity = 90;  // RenderTask.Traversal.Stack (core/ray.go:158)

// Traversal kernel variants (vmr_tuning.kernel bits).
enum TraceKernel : int {
  kKernelScheduled = 0,
  kKernelWhileWhile = 1,
  kKernelPrefetch = 2,
  kKernelRegCap = 4,
  kKernelSort = 8,
  kKernelSharedStack = 16,  // while-while: the top of the stack in shared memory
  kKernelCoopLeaf = 32,     // while-while, static meshes: warp-cooperative leaf scan
};
constexpr int kSharedStackEntries = 16;

// Ray reordering (raysort.cu): 6 permutation classes x (2^b)^3 origin cells,
// b = 3..5 (default 4: 16^3 cells).
constexpr int kSortCells = 4096;
constexpr int kSortBuckets = 6 * kSortCells;
constexpr int kSortMaxBits = 5;
constexpr int kSortBucketsMax = 6 << (3 * kSortMaxBits);
constexpr uint32_t sort_buckets(int bits) { return 6u << (3 * bits); }
constexpr uint64_t kSortMinRays = 1u << 16;  // smaller batches are traced unsorted

// Launch entry points (traverse.cu).
struct TraceLaunch {
  RaySoA rays;
  HitSoA hits;
  const uint32_t* order;  // rays[i] is input ray order[i] (nullptr: identity)
  uint64_t n;
  const unsigned long long* n_dev;  // if set, the ray count is read from device
                                    // memory when the kernel starts (wavefront
                                    // queues; n is then a capacity); scene
                                    // traces and the while-while mesh kernels
  int any_hit;
  int count;
  DScratch* scratch;
  int grid;             // resident blocks per SM wanted (0 = occupancy maximum)
  int block;
  int kernel;
  int refill_min;
  int walk_tail;
  void* stream;
  // scene traces in job mode (batched renders): no top level; ray i enters
  // mesh path_geom[ray_path[i]] directly (both set or both null)
  const uint32_t* ray_path;
  const uint32_t* path_geom;
};
int launch_trace_mesh(const DMesh& mesh, const TraceLaunch& l);
// n_dev (optional): the ray count on the device, at most n (a wavefront queue
// length); the grid is sized for n.  sorted_out.rec set: the key-ordered copy
// is written as records (RaySoA::rec, 32 bytes a ray) and order is not
// written; else as arrays, with order[i] = the input index of position i.
int launch_ray_sort(const RaySoA& rays, uint64_t n, const float bounds[6], int bits, uint32_t* keys, uint32_t* hist,
                    uint32_t* order, const RaySoA& sorted_out, void* stream,
                    const unsigned long long* n_dev = nullptr);
int launch_trace_scene(const DTop& top, const TraceLaunch& l);
int device_sm_count();

// One job of a batched trace (vmr_trace_jobs): its rays and hits (device
// SoA, its own buffers) and its first position in the gathered ray stream.
struct JobDesc {
  RaySoA rays;
  HitSoA hits;
  uint64_t n;
  uint64_t ray0;  // the job's first position in the gathered ray stream
};
// Gathered rays and hits of a batched trace, the per-ray job index and the
// job -> geom table (the scene kernel's job mode reads job_geom[ray_job[i]]).
struct JobWork {
  RaySoA rays;
  HitSoA hits;
  uint32_t* ray_job;
  uint32_t* job_geom;
};
// l: the launch settings (stream, kernel, walk tail, scratch, any_hit); top:
// the mesh table indexed by geom id (keys = 1, no top level).
int launch_trace_jobs(const JobDesc* jobs, uint32_t n_jobs, uint64_t n_rays, const DTop& top, const JobWork& w,
                      TraceLaunch l);

}  // namespace vmr
