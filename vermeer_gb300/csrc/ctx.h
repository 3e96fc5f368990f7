// ctx.h - the context record behind vmr_ctx (shared by the C-ABI sources).
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "accel.h"
#include "device.h"
#include "vmr.h"

using vmr::DMesh;
using vmr::DScratch;
using vmr::DTop;
using vmr::GNode;
using vmr::HostMesh;
using vmr::HostTop;
using vmr::MNode;

namespace vmr {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { if (p) cudaFree(p); }
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) { cudaFree(p); p = nullptr; bytes = 0; }
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

struct MeshRec {
  HostMesh host;
  DevBuf nodes, tris, mnodes, mboxes, mtris, elem;
  DMesh dmesh{};
  float bounds6[6];
  // shading (render.cu): PolyMesh.Shader, shader index and normals per
  // leaf-order triangle
  std::vector<uint32_t> shader_list;
  bool has_normals = false;
  DevBuf shlist, sidx, nrm;
  DevBuf avert, aidx;  // motion meshes: key-major vertices (float4) and face-order idxp for hit attributes
  // motion meshes: per-key corner normals (vmr_mesh_set_motion_normals),
  // float4 [keys][mnrm_n]; mnrm_n = 0: none
  DevBuf mnrm;
  uint32_t mnrm_n = 0;
  // PolyMesh.Transform (one matrix, column-major) and its Matrix4Inverse;
  // a GeomInstance's or Proc's transform when it has one key (the matrix
  // rebuilt from its decomposition, as TimeKey returns it)
  bool has_xf = false;
  float xf[16] = {}, xf_inv[16] = {};
  // Transform keys decomposed (two or more keys: blended at each ray's time)
  std::vector<anim::Decomp> xkeys;
  DevBuf dxkeys;
  // GeomInstance / Proc (host.group != 0): the geoms it traces and the id
  // a hit in each reports
  std::vector<uint32_t> children;
  std::vector<int32_t> child_hit;
  DevBuf dchildren, dchild_hit;
  // A Proc's child: the Proc's geom id (such a geom is traced only through
  // its Proc, never from the top level); -1 otherwise
  int32_t owner = -1;
  // the autotuner's choice for this mesh (vmr_autotune)
  bool tuned = false;
  vmr_tuning tuning{};
};

// The extended path tracer's captured bounce loop (pathtrace.cu): valid for
// the buffers, scene tables and launch shapes it was captured with.
struct PathGraph {
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> key;
  ~PathGraph() { if (exec) cudaGraphExecDestroy(exec); }
};

struct RenderState {
  std::vector<vmr_shader_std> shaders;
  std::vector<vmr_tri_light> lights;
  std::vector<vmr_disk_light> disks;
  std::vector<vmr_sphere_light> spheres;
  std::vector<vmr_quad_light> quads;
  float env[3] = {0.f, 0.f, 0.f};
  vmr_camera camera{};
  bool has_camera = false;
  // Camera.LocalToWorld keys decomposed (camera.go:207-236); cam_used is the
  // camera the kernels see: m rebuilt from the decomposition for one key
  // (the reference's round trip), key 0 otherwise (the kernels blend
  // dcam_keys per sample)
  std::vector<anim::Decomp> cam_keys;
  std::vector<float> cam_key_m;  // the keys as given (16 floats each)
  DevBuf dcam_keys;
  vmr_camera cam_used{};
  // pixel filter (vmr_set_pixel_filter): filter_n = 0 is none; the device
  // table holds cdfV (n) then cdfVU (n x n) as float64
  uint32_t filter_n = 0;
  double filter_w = 0.0;
  std::vector<double> filter_host;
  DevBuf filter;
  DevBuf outbuf;   // vmr_encode_rgbe staging for host framebuffers
  DevBuf jobmesh;  // batched path jobs: the mesh table the traversal reads
  DevBuf buf;      // reference mode batch buffers
  DevBuf ptbuf;    // extended mode batch buffers
  uint32_t path_batch = 0;  // paths per batch of a one-scene render when the call gives none (0: 16M)
  void* pt_host = nullptr;  // pinned per-batch parameters (extended mode)
  size_t pt_host_bytes = 0;
  PathGraph graph;
  ~RenderState() { if (pt_host) cudaFreeHost(pt_host); }
};

// The path-guiding network (guide.cu): float32 master weights with Adam
// state, bf16 forward and transposed copies, and training scratch.
struct GuideState {
  bool ready = false;
  int step = 0;
  DevBuf W, m, v, grad, wf, wb, sums, err;
  DevBuf save;          // bf16 activations and deltas, chunk-blocked (guide.cu save_vec)
  uint32_t save_rows = 0;
  DevBuf io;            // host-call staging (SoA rows, outputs)
};

struct TopRec {
  HostTop host;
  DevBuf nodes, mnodes, mboxes, order, meshes;
  DTop dtop{};
  float bounds6[6] = {0, 0, 0, 0, 0, 0};  // union of the geoms' bounds (ray reordering)
  bool valid = false;
};

// The camera the kernels see for a vmr_camera: m replaced by the matrix the
// reference rebuilds from its decomposition (render.cu).
vmr_camera camera_round_trip(const vmr_camera& c);

// A static scene flattened into one mesh for the extended path tracer's
// traces: every triangle of every top-level geom (each geom's triangles in
// its leaf order) in one QBVH, and per leaf position of that QBVH the geom
// and the geom's own leaf position the hit reports (map[e], map[n + e]).
// Built once per scene, on the first render that can use it; any change of
// the top level drops it.
struct FlatScene {
  bool tried = false;  // the current top level was examined
  std::unique_ptr<MeshRec> rec;  // nullptr: the scene does not qualify
  DevBuf map;
  uint32_t n = 0;
};

}  // namespace vmr

using vmr::DevBuf;
using vmr::MeshRec;
using vmr::TopRec;

struct vmr_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  DevBuf scratch;                 // DScratch
  DevBuf io;                      // rays + hits for host-pointer traces
  DevBuf sortbuf;                 // ray keys, bucket offsets, order, key-ordered rays
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evm = nullptr;  // start, after the sort, end
  // vmr_render's own start/end (its scene traces record ev0/ev1 themselves)
  cudaEvent_t rev0 = nullptr, rev1 = nullptr;
  std::vector<std::unique_ptr<MeshRec>> meshes;
  TopRec top;
  vmr::FlatScene flat;
  vmr::RenderState render;
  vmr::GuideState guide;
  vmr_tuning tuning{45, 0, 0, 0, 8, 0};
  int builder = VMR_BUILD_AUTO;   // vmr_set_builder
  DevBuf jobs;                    // vmr_trace_jobs tables
  // Bounds (min xyz, max xyz) of the mesh a DMesh belongs to.
  const float* mesh_bounds_of(const DMesh* d) const {
    for (const auto& m : meshes)
      if (&m->dmesh == d) return m->bounds6;
    return nullptr;
  }
  // The tuning a trace of this mesh uses: its own (autotuned) or the context's.
  const vmr_tuning& tuning_for(const DMesh* d) const {
    if (d)
      for (const auto& m : meshes)
        if (&m->dmesh == d) return m->tuned ? m->tuning : tuning;
    return tuning;
  }
};


namespace vmr {
// The context's flattened scene (capi.cpp), built on the first call that
// asks for it: the flat mesh, or nullptr when the scene does not qualify
// (a motion, transformed, sphere, instance or Proc geom, geoms with
// different ray biases, fewer than two geoms, or a build the device
// builder declines).  *map / *n: the leaf position -> (geom, leaf position)
// table on the device and its length.  Returns a VMR status in *status.
const DMesh* flat_scene(vmr_ctx* ctx, const uint32_t** map, uint32_t* n, int* status);
// Any-hit trace of n device rays against the flattened scene (capi.cpp):
// whether each ray hits something within its tmax is the same whichever
// tree holds the triangles, so shadow rays may take it wherever the scene
// flattens.  h.prim >= 0 marks a hit (a leaf position of the flat mesh).
// *used false (nothing launched): the scene does not flatten, or the
// context's kernel is not the while-while one.
int trace_flat_any_hit(vmr_ctx* ctx, const vmr_rays& r, size_t n, const vmr_hits& h, bool* used);
}  // namespace vmr
