// capi.cpp - the C ABI of libvmr (include/vmr.h).
//
// Host side of the traversal path: contexts, mesh and scene upload (the
// reference's 128-byte qbvh.Node repacked into the device GNode layout),
// batched traces with host or device buffers, and status reporting.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "accel.h"
#include "ctx.h"
#include "device.h"
#include "gpubuild.h"
#include "vmr.h"

namespace {

// Smallest mesh vmr_mesh_build builds on the device under VMR_BUILD_AUTO.
constexpr uint32_t kDeviceBuildMin = 16384;

int fail(vmr_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int cuda_fail(vmr_ctx* ctx, cudaError_t e, const char* what) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? VMR_ERR_OOM : VMR_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define VMR_CUDA(ctx, call)                                   \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);  \
  } while (0)

template <class T>
cudaError_t upload(vmr_ctx* ctx, DevBuf& buf, const std::vector<T>& v) {
  if (v.empty()) return cudaSuccess;
  cudaError_t e = buf.ensure(v.size() * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
}

// Reference leaf code -> device leaf code (see device.h).
bool repack_child(int32_t c, uint32_t n_inner, uint32_t n_elems, int32_t& out) {
  if (c >= 0) {
    if ((uint32_t)c >= n_inner) return false;
    out = c;
    return true;
  }
  if (c == -1) { out = vmr::kEmptyChild; return true; }
  uint32_t first = ((uint32_t)c & 0x7ffffffu) >> 4;  // LeafBase (qbvh/qbvh.go:64)
  uint32_t count = ((uint32_t)c & 0xfu) + 1u;         // LeafCount (qbvh.go:61)
  if ((uint64_t)first + count > n_elems) return false;
  out = (int32_t)(0x80000000u | (first << 4) | (count - 1u));
  return true;
}

uint32_t pack_axes(uint32_t a0, uint32_t a1, uint32_t a2) { return (a0 & 3u) | ((a1 & 3u) << 2) | ((a2 & 3u) << 4); }

// Push rank of each child for every ray octant (bit k of o set when D[k] < 0),
// following qbvh.Trace (qbvh/intersect.go:137-216): the pairs (0,1) and
// (2,3) are each ordered by the sign of D along their split axis and the
// pair order by D[Axis0].  Rank 0 is pushed first, so it is popped last.
void push_ranks(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t rank[2]) {
  rank[0] = rank[1] = 0;
  for (uint32_t o = 0; o < 8; ++o) {
    const uint32_t s0 = (o >> a0) & 1u, s1 = (o >> a1) & 1u, s2 = (o >> a2) & 1u;
    const uint32_t r[4] = {2u * (1u - s0) + (1u - s1), 2u * (1u - s0) + s1, 2u * s0 + (1u - s2), 2u * s0 + s2};
    uint32_t byte = r[0] | (r[1] << 2) | (r[2] << 4) | (r[3] << 6);
    rank[o >> 2] |= byte << (8u * (o & 3u));
  }
}

bool repack_nodes(const std::vector<vmr_qbvh_node>& in, uint32_t n_elems, std::vector<GNode>& out) {
  out.resize(in.size());
  for (size_t i = 0; i < in.size(); ++i) {
    GNode g;
    std::memset(&g, 0, sizeof(g));
    std::memcpy(g.box, in[i].boxes, sizeof(g.box));
    for (int c = 0; c < 4; ++c)
      if (!repack_child(in[i].children[c], (uint32_t)in.size(), n_elems, g.child[c])) return false;
    if (in[i].axis0 > 2 || in[i].axis1 > 2 || in[i].axis2 > 2) return false;
    g.axes = pack_axes(in[i].axis0, in[i].axis1, in[i].axis2);
    push_ranks(in[i].axis0, in[i].axis1, in[i].axis2, g.rank);
    out[i] = g;
  }
  return true;
}

bool repack_mnodes(const std::vector<vmr_mqbvh_node>& in, uint32_t n_elems, std::vector<MNode>& out) {
  out.resize(in.size());
  for (size_t i = 0; i < in.size(); ++i) {
    MNode g;
    std::memset(&g, 0, sizeof(g));
    for (int c = 0; c < 4; ++c)
      if (!repack_child(in[i].children[c], (uint32_t)in.size(), n_elems, g.child[c])) return false;
    if ((uint32_t)in[i].axis0 > 2 || (uint32_t)in[i].axis1 > 2 || (uint32_t)in[i].axis2 > 2) return false;
    g.axes = pack_axes((uint32_t)in[i].axis0, (uint32_t)in[i].axis1, (uint32_t)in[i].axis2);
    push_ranks((uint32_t)in[i].axis0, (uint32_t)in[i].axis1, (uint32_t)in[i].axis2, g.rank);
    out[i] = g;
  }
  return true;
}

struct F4 { float x, y, z, w; };

// The device copy of a mesh's transform (its inverse, columns 0..3 of rows 0..2).
void fill_xf(const MeshRec& rec, DMesh& d) {
  static const int kCols[12] = {0, 1, 2, 4, 5, 6, 8, 9, 10, 12, 13, 14};
  d.has_xf = rec.has_xf ? 1u : 0u;
  for (int k = 0; k < 12; ++k) d.xf_inv[k] = rec.has_xf ? rec.xf_inv[kCols[k]] : 0.0f;
  const bool keyed = rec.xkeys.size() >= 2;
  d.xf_nkeys = keyed ? (uint32_t)rec.xkeys.size() : 0u;
  d.xf_keys = keyed ? rec.dxkeys.as<vmr::anim::Decomp>() : nullptr;
}

// Host accelerator -> device arrays (layout in device.h).  tris_ready: the
// device builder already wrote the static triangle table into rec.tris.
int upload_mesh(vmr_ctx* ctx, MeshRec& rec, bool tris_ready = false) {
  HostMesh& m = rec.host;
  if (ctx->device < 0) return VMR_OK;
  DMesh d{};
  d.n_tris = m.n_tris;
  d.keys = m.motion() ? m.keys : 1u;
  d.lower_static = 1.19209290e-07f + m.ray_bias;  // EpsilonFloat32 + RayBias
  d.ray_bias = m.ray_bias;
  if (!m.motion()) {
    std::vector<GNode> g;
    if (!repack_nodes(m.nodes, m.n_tris, g)) return fail(ctx, VMR_ERR_INVALID, "malformed QBVH nodes");
    VMR_CUDA(ctx, upload(ctx, rec.nodes, g));
    if (!tris_ready) {
      std::vector<F4> tris((size_t)m.n_tris * 3);
      for (size_t i = 0; i < (size_t)m.n_tris * 3; ++i) {
        const float* v = &m.verts[(size_t)m.idxp[i] * 3];
        tris[i] = F4{v[0], v[1], v[2], 0.0f};
      }
      VMR_CUDA(ctx, upload(ctx, rec.tris, tris));
    }
    d.nodes = rec.nodes.as<GNode>();
    d.tris = rec.tris.p;
    d.iter_cap = 4u * (uint32_t)m.nodes.size() + 2u;
  } else {
    std::vector<MNode> g;
    if (!repack_mnodes(m.mnodes, m.n_tris, g)) return fail(ctx, VMR_ERR_INVALID, "malformed motion QBVH nodes");
    const bool fixed = m.motion_mode == VMR_MOTION_FIXED;
    std::vector<F4> tris((size_t)m.keys * m.n_tris * 3);
    std::vector<int32_t> elem(m.n_tris);
    for (uint32_t i = 0; i < m.n_tris; ++i) {
      // Faithful: idxp read at the leaf position (trace.go:532-537).
      // Fixed: the face the leaf boxes were built from.
      const uint32_t face = fixed ? (uint32_t)m.accel_idx[i] : i;
      elem[i] = (int32_t)face;
      for (uint32_t key = 0; key < m.keys; ++key)
        for (int j = 0; j < 3; ++j) {
          const float* v = &m.verts[((size_t)key * m.n_verts + m.idxp[(size_t)face * 3 + j]) * 3];
          tris[((size_t)key * m.n_tris + i) * 3 + j] = F4{v[0], v[1], v[2], 0.0f};
        }
    }
    VMR_CUDA(ctx, upload(ctx, rec.mnodes, g));
    VMR_CUDA(ctx, upload(ctx, rec.mboxes, m.mboxes));
    VMR_CUDA(ctx, upload(ctx, rec.mtris, tris));
    VMR_CUDA(ctx, upload(ctx, rec.elem, elem));
    d.mnodes = rec.mnodes.as<MNode>();
    d.mboxes = rec.mboxes.p;
    d.mtris = rec.mtris.p;
    d.elem = rec.elem.as<int32_t>();
    d.n_mnodes = (uint32_t)m.mnodes.size();
    d.iter_cap = 4u * (uint32_t)m.mnodes.size() + 2u;
  }
  VMR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  fill_xf(rec, d);
  rec.dmesh = d;
  for (int a = 0; a < 3; ++a) {
    rec.bounds6[a] = m.bounds.lo[a];
    rec.bounds6[3 + a] = m.bounds.hi[a];
  }
  return VMR_OK;
}

bool valid_mesh_input(const vmr_mesh_input* in, std::string& why) {
  if (!in || in->motion_keys < 1) { why = "motion_keys must be >= 1"; return false; }
  if (in->n_tris > 0 && (!in->verts || !in->idxp)) { why = "null verts or idxp"; return false; }
  if (in->n_tris >= (1u << 23)) { why = "a mesh holds at most 2^23-1 triangles (qbvh.LeafBase)"; return false; }
  for (size_t i = 0; i < (size_t)in->n_tris * 3; ++i)
    if (in->idxp[i] >= in->n_verts) { why = "vertex index out of range"; return false; }
  return true;
}

// math.Matrix4Inverse (math/matrix4.go:116-160), restated in animdecomp.h;
// a zero determinant leaves c all zero (the reference returns its zero c).
void matrix4_inverse(const float m[16], float c[16]) { vmr::anim::inverse(m, c); }

int refresh_top(vmr_ctx* ctx) {
  TopRec& t = ctx->top;
  ctx->flat.tried = false;  // a flattened copy of the old top level is stale
  ctx->flat.rec.reset();
  if (ctx->device < 0) return VMR_OK;
  // Device mesh table indexed by geom id.
  std::vector<DMesh> table(ctx->meshes.size());
  for (size_t i = 0; i < ctx->meshes.size(); ++i) table[i] = ctx->meshes[i]->dmesh;
  VMR_CUDA(ctx, upload(ctx, t.meshes, table));
  DTop d{};
  if (t.host.keys <= 1) {
    std::vector<GNode> g;
    if (!repack_nodes(t.host.nodes, (uint32_t)t.host.geom_order.size(), g))
      return fail(ctx, VMR_ERR_INVALID, "malformed top-level nodes");
    VMR_CUDA(ctx, upload(ctx, t.nodes, g));
    d.nodes = t.nodes.as<GNode>();
    d.keys = 1;
    d.iter_cap = 4u * (uint32_t)t.host.nodes.size() + 2u;
  } else {
    std::vector<MNode> g;
    if (!repack_mnodes(t.host.mnodes, (uint32_t)t.host.geom_order.size(), g))
      return fail(ctx, VMR_ERR_INVALID, "malformed top-level motion nodes");
    VMR_CUDA(ctx, upload(ctx, t.mnodes, g));
    VMR_CUDA(ctx, upload(ctx, t.mboxes, t.host.mboxes));
    d.mnodes = t.mnodes.as<MNode>();
    d.mboxes = t.mboxes.p;
    d.keys = t.host.keys;
    d.n_mnodes = (uint32_t)t.host.mnodes.size();
    d.iter_cap = 4u * (uint32_t)t.host.mnodes.size() + 2u;
  }
  VMR_CUDA(ctx, upload(ctx, t.order, t.host.geom_order));
  VMR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  d.geom_order = t.order.as<uint32_t>();
  d.meshes = t.meshes.as<DMesh>();
  d.n_geoms = (uint32_t)t.host.geom_order.size();
  d.all_static = d.keys == 1 ? 1u : 0u;
  d.simple_only = 0u;
  for (int k = 0; k < 3; ++k) {
    t.bounds6[k] = INFINITY;
    t.bounds6[3 + k] = -INFINITY;
  }
  for (uint32_t g : t.host.geom_order) {
    if (ctx->meshes[g]->host.motion() || ctx->meshes[g]->has_xf) d.all_static = 0u;
    if (ctx->meshes[g]->host.group || ctx->meshes[g]->xkeys.size() >= 2) {
      d.simple_only = 1u;
      d.all_static = 0u;
    }
    for (int k = 0; k < 3; ++k) {
      t.bounds6[k] = std::min(t.bounds6[k], ctx->meshes[g]->bounds6[k]);
      t.bounds6[3 + k] = std::max(t.bounds6[3 + k], ctx->meshes[g]->bounds6[3 + k]);
    }
  }
  t.dtop = d;
  t.valid = !t.host.geom_order.empty();
  return VMR_OK;
}

int read_status(vmr_ctx* ctx, vmr_trace_stats* stats) {
  DScratch s;
  VMR_CUDA(ctx, cudaMemcpyAsync(&s, ctx->scratch.p, sizeof(s), cudaMemcpyDeviceToHost, ctx->stream));
  VMR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (stats) {
    stats->node_visits = s.node_visits;
    stats->leaf_visits = s.leaf_visits;
    stats->tri_tests = s.tri_tests;
  }
  if (s.status == vmr::kStatusStackOverflow)
    return fail(ctx, VMR_ERR_STACK_OVERFLOW, "a ray needed more than 90 traversal stack entries");
  if (s.status == vmr::kStatusIterationCap)
    return fail(ctx, VMR_ERR_TIMEOUT, "a traversal loop hit its iteration cap");
  return VMR_OK;
}

// Sort (when the tuning asks) and traversal of n device rays, queued on
// ctx->stream.  reset: zero the whole scratch (ray counter, status, visit
// counters); otherwise only the ray counter, so consecutive launches add up
// their counters and statuses.  first/last: record the timing events (ev0,
// evm around the sort of the first launch; ev1 after the last traversal).
int launch_trace_chunk(vmr_ctx* ctx, const DMesh* mesh, const vmr_rays& r, size_t n, int flags, const vmr_hits& h,
                       bool reset, bool first, bool last) {
  vmr::TraceLaunch l{};
  l.rays = vmr::RaySoA{r.px, r.py, r.pz, r.dx, r.dy, r.dz, r.tmax, r.time};
  l.hits = vmr::HitSoA{h.prim, h.geom, h.t, h.u, h.v, h.w};
  l.n = n;
  l.any_hit = (flags & VMR_TRACE_ANY_HIT) ? 1 : 0;
  l.count = (flags & VMR_TRACE_COUNT) ? 1 : 0;
  l.scratch = ctx->scratch.as<DScratch>();
  l.stream = ctx->stream;
  const vmr_tuning& tn = ctx->tuning_for(mesh);
  l.kernel = tn.kernel;
  l.block = tn.block;
  l.grid = tn.blocks_per_sm;
  l.refill_min = tn.refill_min;
  l.walk_tail = tn.walk_tail;
  if (reset) VMR_CUDA(ctx, cudaMemsetAsync(ctx->scratch.p, 0, sizeof(DScratch), ctx->stream));
  else VMR_CUDA(ctx, cudaMemsetAsync(ctx->scratch.p, 0, sizeof(unsigned long long), ctx->stream));  // next_ray
  if (first) VMR_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  const bool scene_sort = !mesh && ctx->top.dtop.all_static && !(flags & VMR_TRACE_COUNT);
  if ((mesh || scene_sort) && (tn.kernel & vmr::kKernelSort) && n >= vmr::kSortMinRays) {
    // Key-ordered copy of the rays (raysort.cu); hits go back through order[].
    const size_t nf = ((n + 31) / 32) * 32;
    const int nfield = r.time ? 8 : 7;
    const size_t bytes = nf * 4 * (2 + nfield) + sizeof(uint32_t) * vmr::kSortBucketsMax;
    VMR_CUDA(ctx, ctx->sortbuf.ensure(bytes));
    uint32_t* keys = ctx->sortbuf.as<uint32_t>();
    uint32_t* order = keys + nf;
    float* f = reinterpret_cast<float*>(order + nf);
    uint32_t* hist = reinterpret_cast<uint32_t*>(f + nf * nfield);
    vmr::RaySoA sorted{f, f + nf, f + 2 * nf, f + 3 * nf, f + 4 * nf, f + 5 * nf, f + 6 * nf,
                       nfield == 8 ? f + 7 * nf : nullptr};
    // a context mesh's own bounds; the scene's (the flattened scene's mesh,
    // which is no context mesh, covers exactly the scene's geoms)
    const float* mb = mesh ? ctx->mesh_bounds_of(mesh) : ctx->top.bounds6;
    if (!mb) mb = ctx->top.bounds6;
    // A static mesh in the while-while kernel reads the copy as 32-byte
    // records (two 16-byte loads a ray, its input index inside), written
    // over the order and array regions (4 + 28 bytes a ray).
    const bool recs = mesh && mesh->keys <= 1 && !r.time && (tn.kernel & vmr::kKernelWhileWhile);
    if (recs) sorted = vmr::RaySoA{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, order};
    int se = vmr::launch_ray_sort(l.rays, n, mb, tn.sort_bits ? tn.sort_bits : 4, keys, hist, order, sorted,
                                  ctx->stream);
    if (se != 0) return cuda_fail(ctx, (cudaError_t)se, "ray sort launch");
    l.rays = sorted;
    l.order = recs ? nullptr : order;
  }
  if (first) VMR_CUDA(ctx, cudaEventRecord(ctx->evm, ctx->stream));
  int e = mesh ? vmr::launch_trace_mesh(*mesh, l) : vmr::launch_trace_scene(ctx->top.dtop, l);
  if (e != 0) return cuda_fail(ctx, (cudaError_t)e, "trace kernel launch");
  if (last) VMR_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  return VMR_OK;
}

// One traversal launch: rays/hits are device pointers here.
int run_trace(vmr_ctx* ctx, const DMesh* mesh, const vmr_rays& r, size_t n, int flags, const vmr_hits& h,
              vmr_trace_stats* stats) {
  int rc = launch_trace_chunk(ctx, mesh, r, n, flags, h, true, true, true);
  if (rc != VMR_OK) return rc;
  if (stats) stats->rays = n;
  if (flags & VMR_TRACE_DEVICE) return VMR_OK;
  int st = read_status(ctx, stats);
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->evm, ctx->ev1);
    stats->kernel_ms = ms;
  }
  return st;
}

// Host-pointer trace: stage rays in, sort and trace, copy hits out, all
// queued on ctx->stream; the status read after the downloads is the one
// synchronisation.  (Splitting the call into chunks whose copies overlap the
// neighbouring chunks' traversal measured slower on GB300: every persistent
// launch ends with a tail in which SMs drain, and sorting smaller batches
// groups rays less well, which cost more than the overlapped copies saved.)
int trace_host(vmr_ctx* ctx, const DMesh* mesh, const vmr_rays* rays, size_t n, int flags, const vmr_hits* hits,
               vmr_trace_stats* stats) {
  const size_t fb = n * sizeof(float);
  const int n_in = rays->time ? 8 : 7;
  const size_t bytes = fb * (size_t)n_in + fb * 6;
  VMR_CUDA(ctx, ctx->io.ensure(bytes == 0 ? 16 : bytes));
  char* base = ctx->io.as<char>();
  const float* src[8] = {rays->px, rays->py, rays->pz, rays->dx, rays->dy, rays->dz, rays->tmax, rays->time};
  float* dst[8];
  for (int k = 0; k < n_in; ++k) {
    dst[k] = reinterpret_cast<float*>(base + fb * k);
    if (!src[k]) return fail(ctx, VMR_ERR_INVALID, "null ray array");
  }
  for (int k = 0; k < n_in; ++k)
    if (n) VMR_CUDA(ctx, cudaMemcpyAsync(dst[k], src[k], fb, cudaMemcpyHostToDevice, ctx->stream));
  char* hb = base + fb * n_in;
  void* outs[6] = {hits->prim, hits->geom, hits->t, hits->u, hits->v, hits->w};
  char* douts[6];
  for (int k = 0; k < 6; ++k) douts[k] = outs[k] ? hb + (size_t)k * fb : nullptr;
  vmr_rays dr{dst[0], dst[1], dst[2], dst[3], dst[4], dst[5], dst[6], n_in == 8 ? dst[7] : nullptr};
  vmr_hits dh{reinterpret_cast<int32_t*>(douts[0]), reinterpret_cast<int32_t*>(douts[1]),
              reinterpret_cast<float*>(douts[2]), reinterpret_cast<float*>(douts[3]),
              reinterpret_cast<float*>(douts[4]), reinterpret_cast<float*>(douts[5])};
  int rc = launch_trace_chunk(ctx, mesh, dr, n, flags & ~VMR_TRACE_DEVICE, dh, true, true, true);
  if (rc != VMR_OK) {
    cudaStreamSynchronize(ctx->stream);
    return rc;
  }
  for (int k = 0; k < 6; ++k)
    if (outs[k] && n) VMR_CUDA(ctx, cudaMemcpyAsync(outs[k], douts[k], fb, cudaMemcpyDeviceToHost, ctx->stream));
  if (stats) stats->rays = n;
  const int st = read_status(ctx, stats);  // synchronises ctx->stream, hence the downloads
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->evm, ctx->ev1);
    stats->kernel_ms = ms;
  }
  return st;
}

}  // namespace

namespace vmr {
int trace_flat_any_hit(vmr_ctx* ctx, const vmr_rays& r, size_t n, const vmr_hits& h, bool* used) {
  *used = false;
  if (!(ctx->tuning.kernel & kKernelWhileWhile)) return VMR_OK;
  const uint32_t* map = nullptr;
  uint32_t nmap = 0;
  int st = VMR_OK;
  const DMesh* flat = flat_scene(ctx, &map, &nmap, &st);
  if (st != VMR_OK || !flat) return st;
  *used = true;
  return launch_trace_chunk(ctx, flat, r, n, VMR_TRACE_DEVICE | VMR_TRACE_ANY_HIT, h, true, true, true);
}

const DMesh* flat_scene(vmr_ctx* ctx, const uint32_t** map, uint32_t* n, int* status) {
  *status = VMR_OK;
  FlatScene& F = ctx->flat;
  if (F.tried) {
    if (!F.rec) return nullptr;
    *map = F.map.as<uint32_t>();
    *n = F.n;
    return &F.rec->dmesh;
  }
  F.tried = true;
  F.rec.reset();
  const TopRec& top = ctx->top;
  if (ctx->device < 0 || !top.valid || !top.dtop.all_static || top.dtop.simple_only || top.host.keys > 1) return nullptr;
  const std::vector<uint32_t>& order = top.host.geom_order;
  if (order.size() < 2) return nullptr;
  float bias = 0.0f;
  uint64_t total = 0;
  for (size_t i = 0; i < order.size(); ++i) {
    const MeshRec& r = *ctx->meshes[order[i]];
    const HostMesh& m = r.host;
    if (m.sphere || m.group || m.motion() || r.has_xf || r.xkeys.size() >= 2 || m.n_tris == 0) return nullptr;
    if (i == 0) bias = m.ray_bias;
    else if (m.ray_bias != bias) return nullptr;
    total += m.n_tris;
  }
  if (total >= (1u << 23)) return nullptr;  // a mesh's leaf base limit (qbvh.LeafBase)
  const uint32_t T = (uint32_t)total;
  auto rec = std::make_unique<MeshRec>();
  HostMesh& fm = rec->host;
  fm.keys = 1;
  fm.n_tris = T;
  fm.n_verts = 3 * T;
  fm.ray_bias = bias;
  fm.verts.resize((size_t)9 * T);
  fm.idxp.resize((size_t)3 * T);
  std::vector<uint32_t> fgeom(T), fprim(T);
  uint32_t c = 0;
  for (uint32_t g : order) {
    const HostMesh& m = ctx->meshes[g]->host;
    for (uint32_t j = 0; j < m.n_tris; ++j, ++c) {  // the geom's leaf order
      for (int k = 0; k < 3; ++k) {
        const float* v = &m.verts[(size_t)m.idxp[(size_t)3 * j + k] * 3];
        std::memcpy(&fm.verts[((size_t)3 * c + k) * 3], v, 12);
        fm.idxp[(size_t)3 * c + k] = 3 * c + (uint32_t)k;
      }
      fgeom[c] = g;
      fprim[c] = j;
    }
  }
  std::string why;
  if (vmr::device_build_mesh(fm, rec->tris, ctx->stream, why) != vmr::kBuildOk) return nullptr;
  if ((*status = upload_mesh(ctx, *rec, true)) != VMR_OK) return nullptr;
  std::vector<uint32_t> tab((size_t)2 * T);
  for (uint32_t e = 0; e < T; ++e) {
    const uint32_t f = (uint32_t)fm.accel_idx[e];
    tab[e] = fgeom[f];
    tab[(size_t)T + e] = fprim[f];
  }
  cudaError_t ce = upload(ctx, F.map, tab);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
  if (ce != cudaSuccess) {
    *status = cuda_fail(ctx, ce, "flattened scene upload");
    return nullptr;
  }
  // the host copies are not needed again
  std::vector<float>().swap(fm.verts);
  std::vector<uint32_t>().swap(fm.idxp);
  F.rec = std::move(rec);
  F.n = T;
  *map = F.map.as<uint32_t>();
  *n = T;
  return &F.rec->dmesh;
}
}  // namespace vmr

namespace vmr {
// Read-only view of a context's mesh and settings for vmr_trace_mesh_noalloc
// (noalloc.cu), which keeps its own scratch and launches the same kernels.
bool ctx_noalloc_view(vmr_ctx* ctx, uint32_t geom, const DMesh** mesh, const float** bounds, void** stream,
                      int* device, vmr_tuning* tuning) {
  if (!ctx || ctx->device < 0 || geom >= ctx->meshes.size()) return false;
  *mesh = &ctx->meshes[geom]->dmesh;
  *bounds = ctx->meshes[geom]->bounds6;
  *stream = ctx->stream;
  *device = ctx->device;
  *tuning = ctx->tuning_for(*mesh);
  return ctx->meshes[geom]->host.n_tris > 0;
}
int ctx_fail(vmr_ctx* ctx, int code, const char* msg) { return fail(ctx, code, msg); }
int noalloc_setup(int device);  // noalloc.cu
}  // namespace vmr

extern "C" {

int vmr_abi_version(void) { return VMR_ABI_VERSION; }

int vmr_create(int device, vmr_ctx** out) {
  if (!out) return VMR_ERR_INVALID;
  *out = nullptr;
  if (device < 0) {  // host-only: builds accelerators, cannot trace
    auto* ctx = new vmr_ctx();
    ctx->device = -1;
    *out = ctx;
    return VMR_OK;
  }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return VMR_ERR_CUDA;
  if (device < 0 || device >= ndev) return VMR_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return VMR_ERR_CUDA;
  auto* ctx = new vmr_ctx();
  ctx->device = device;
  if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
      cudaEventCreate(&ctx->evm) != cudaSuccess || cudaEventCreate(&ctx->rev0) != cudaSuccess ||
      cudaEventCreate(&ctx->rev1) != cudaSuccess ||
      ctx->scratch.ensure(sizeof(DScratch)) != cudaSuccess) {
    delete ctx;
    return VMR_ERR_CUDA;
  }
  ctx->stream = ctx->own_stream;
  // Load vmr_trace_mesh_noalloc's static scratch array on this device now, so
  // that the no-alloc call itself never triggers a module load.  A failure
  // here is reported by that call, not by vmr_create.
  vmr::noalloc_setup(device);
  *out = ctx;
  return VMR_OK;
}

int vmr_destroy(vmr_ctx* ctx) {
  if (!ctx) return VMR_ERR_INVALID;
  if (ctx->device < 0) { delete ctx; return VMR_OK; }
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->evm) cudaEventDestroy(ctx->evm);
  if (ctx->rev0) cudaEventDestroy(ctx->rev0);
  if (ctx->rev1) cudaEventDestroy(ctx->rev1);
  cudaStream_t s = ctx->own_stream;
  delete ctx;
  if (s) cudaStreamDestroy(s);
  return VMR_OK;
}

const char* vmr_last_error(const vmr_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int vmr_set_tuning(vmr_ctx* ctx, const vmr_tuning* t) {
  if (!ctx || !t) return VMR_ERR_INVALID;
  if (t->kernel < 0 || t->kernel > 63) return fail(ctx, VMR_ERR_INVALID, "tuning.kernel must be in [0, 63]");
  if (t->walk_tail < 0 || t->walk_tail > 31) return fail(ctx, VMR_ERR_INVALID, "tuning.walk_tail must be in [0, 31]");
  if (t->block != 0 && (t->block < 32 || t->block > 256 || t->block % 32 != 0))
    return fail(ctx, VMR_ERR_INVALID, "tuning.block must be a multiple of 32 in [32, 256]");
  if (t->blocks_per_sm < 0 || t->refill_min < 0 || t->refill_min > 32)
    return fail(ctx, VMR_ERR_INVALID, "tuning.blocks_per_sm >= 0 and refill_min in [0, 32]");
  if (t->sort_bits != 0 && (t->sort_bits < 3 || t->sort_bits > vmr::kSortMaxBits))
    return fail(ctx, VMR_ERR_INVALID, "tuning.sort_bits must be 0, 3, 4 or 5");
  ctx->tuning = *t;
  return VMR_OK;
}

int vmr_get_tuning(vmr_ctx* ctx, vmr_tuning* t) {
  if (!ctx || !t) return VMR_ERR_INVALID;
  *t = ctx->tuning;
  return VMR_OK;
}

int vmr_trace_timing(vmr_ctx* ctx, float* sort_ms, float* traverse_ms) {
  if (!ctx) return VMR_ERR_INVALID;
  if (ctx->device < 0) return fail(ctx, VMR_ERR_UNSUPPORTED, "host-only context");
  VMR_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
  float a = 0.f, b = 0.f;
  VMR_CUDA(ctx, cudaEventElapsedTime(&a, ctx->ev0, ctx->evm));
  VMR_CUDA(ctx, cudaEventElapsedTime(&b, ctx->evm, ctx->ev1));
  if (sort_ms) *sort_ms = a;
  if (traverse_ms) *traverse_ms = b;
  return VMR_OK;
}

int vmr_set_stream(vmr_ctx* ctx, void* s) {
  if (!ctx) return VMR_ERR_INVALID;
  ctx->stream = s ? (cudaStream_t)s : ctx->own_stream;
  return VMR_OK;
}

int vmr_sync(vmr_ctx* ctx) {
  if (!ctx) return VMR_ERR_INVALID;
  if (ctx->device < 0) return VMR_OK;
  cudaSetDevice(ctx->device);
  return read_status(ctx, nullptr);
}

int vmr_mesh_build(vmr_ctx* ctx, const vmr_mesh_input* in, uint32_t* out_geom) {
  if (!ctx) return VMR_ERR_INVALID;
  std::string why;
  if (!valid_mesh_input(in, why)) return fail(ctx, VMR_ERR_INVALID, why);
  if (ctx->device >= 0) cudaSetDevice(ctx->device);
  auto rec = std::make_unique<MeshRec>();
  HostMesh& m = rec->host;
  m.n_verts = in->n_verts;
  m.keys = in->motion_keys;
  m.n_tris = in->n_tris;
  m.verts.assign(in->verts, in->verts + (size_t)in->n_verts * in->motion_keys * 3);
  m.idxp.assign(in->idxp, in->idxp + (size_t)in->n_tris * 3);
  m.ray_bias = in->ray_bias;
  m.motion_mode = in->motion_mode;
  if (in->shader_idx) m.shader_idx.assign(in->shader_idx, in->shader_idx + in->n_tris);
  // The device builder gives the host builder's result; AUTO takes it for
  // meshes large enough to gain from it.
  bool on_device = false;
  const bool want_device = ctx->device >= 0 && (ctx->builder == VMR_BUILD_DEVICE ||
                                                (ctx->builder == VMR_BUILD_AUTO && in->n_tris >= kDeviceBuildMin));
  if (want_device) {
    int r = vmr::device_build_mesh(m, rec->tris, ctx->stream, why);
    if (r == vmr::kBuildError) return fail(ctx, VMR_ERR_INVALID, why);
    if (r == vmr::kBuildDeclined && ctx->builder == VMR_BUILD_DEVICE && in->n_tris > 0)
      return fail(ctx, VMR_ERR_UNSUPPORTED, "the device builder declined this mesh (non-finite build geometry)");
    on_device = r == vmr::kBuildOk;
  }
  if (!on_device && !vmr::build_mesh_accel(m, why)) return fail(ctx, VMR_ERR_INVALID, why);
  int st = upload_mesh(ctx, *rec, on_device && !m.motion());
  if (st != VMR_OK) return st;
  if (out_geom) *out_geom = (uint32_t)ctx->meshes.size();
  ctx->meshes.push_back(std::move(rec));
  return VMR_OK;
}

int vmr_set_builder(vmr_ctx* ctx, int builder) {
  if (!ctx) return VMR_ERR_INVALID;
  if (builder < VMR_BUILD_AUTO || builder > VMR_BUILD_DEVICE) return fail(ctx, VMR_ERR_INVALID, "unknown builder");
  if (builder == VMR_BUILD_DEVICE && ctx->device < 0)
    return fail(ctx, VMR_ERR_INVALID, "a host-only context has no device builder");
  ctx->builder = builder;
  return VMR_OK;
}

int vmr_sphere_add(vmr_ctx* ctx, const float center[3], float radius, uint32_t* out_geom) {
  if (!ctx || !center) return VMR_ERR_INVALID;
  if (!(radius > 0.0f) || std::isinf(radius)) return fail(ctx, VMR_ERR_INVALID, "sphere radius must be positive");
  auto rec = std::make_unique<MeshRec>();
  HostMesh& m = rec->host;
  m.sphere = true;
  for (int k = 0; k < 3; ++k) {
    m.sphere_c[k] = center[k];
    m.bounds.lo[k] = center[k] - radius;  // Sphere.Bounds (builtin/geom/sphere/sphere.go:62-72)
    m.bounds.hi[k] = center[k] + radius;
    rec->bounds6[k] = m.bounds.lo[k];
    rec->bounds6[3 + k] = m.bounds.hi[k];
  }
  m.sphere_r = radius;
  DMesh& d = rec->dmesh;
  d = DMesh{};
  d.keys = 1;
  d.kind = 1;
  for (int k = 0; k < 3; ++k) d.sphere[k] = center[k];
  d.sphere[3] = radius;
  if (out_geom) *out_geom = (uint32_t)ctx->meshes.size();
  ctx->meshes.push_back(std::move(rec));
  return VMR_OK;
}

int vmr_mesh_upload(vmr_ctx* ctx, const vmr_mesh_desc* d, uint32_t* out_geom) {
  if (!ctx || !d) return VMR_ERR_INVALID;
  if (d->motion_keys < 1 || (d->n_tris && (!d->verts || !d->idxp || !d->accel_idx)))
    return fail(ctx, VMR_ERR_INVALID, "incomplete mesh description");
  if (d->n_tris >= (1u << 23)) return fail(ctx, VMR_ERR_INVALID, "a mesh holds at most 2^23-1 triangles");
  for (size_t i = 0; i < (size_t)d->n_tris * 3; ++i)
    if (d->idxp[i] >= d->n_verts) return fail(ctx, VMR_ERR_INVALID, "vertex index out of range");
  for (size_t i = 0; i < d->n_tris; ++i)
    if (d->accel_idx[i] < 0 || (uint32_t)d->accel_idx[i] >= d->n_tris)
      return fail(ctx, VMR_ERR_INVALID, "accel_idx out of range");
  if (ctx->device >= 0) cudaSetDevice(ctx->device);
  auto rec = std::make_unique<MeshRec>();
  HostMesh& m = rec->host;
  m.n_verts = d->n_verts;
  m.keys = d->motion_keys;
  m.n_tris = d->n_tris;
  m.verts.assign(d->verts, d->verts + (size_t)d->n_verts * d->motion_keys * 3);
  m.idxp.assign(d->idxp, d->idxp + (size_t)d->n_tris * 3);
  m.accel_idx.assign(d->accel_idx, d->accel_idx + d->n_tris);
  m.ray_bias = d->ray_bias;
  m.motion_mode = d->motion_mode;
  if (d->shader_idx) m.shader_idx.assign(d->shader_idx, d->shader_idx + d->n_tris);
  if (m.motion()) {
    if (!d->mnodes || !d->mboxes || !d->bounds || d->n_mnodes == 0)
      return fail(ctx, VMR_ERR_INVALID, "motion mesh needs mnodes, mboxes and per-key bounds");
    m.mnodes.assign(d->mnodes, d->mnodes + d->n_mnodes);
    m.mboxes.assign(d->mboxes, d->mboxes + (size_t)d->motion_keys * d->n_mnodes * 24);
    m.key_bounds.resize(d->motion_keys);
    vmr::Bounds full{{__builtin_huge_valf(), __builtin_huge_valf(), __builtin_huge_valf()},
                     {-__builtin_huge_valf(), -__builtin_huge_valf(), -__builtin_huge_valf()}};
    for (uint32_t k = 0; k < d->motion_keys; ++k) {
      for (int a = 0; a < 3; ++a) {
        m.key_bounds[k].lo[a] = d->bounds[6 * k + a];
        m.key_bounds[k].hi[a] = d->bounds[6 * k + 3 + a];
        full.lo[a] = full.lo[a] < m.key_bounds[k].lo[a] ? full.lo[a] : m.key_bounds[k].lo[a];
        full.hi[a] = full.hi[a] > m.key_bounds[k].hi[a] ? full.hi[a] : m.key_bounds[k].hi[a];
      }
    }
    m.bounds = full;
  } else {
    if ((!d->nodes && d->n_tris) || !d->bounds) return fail(ctx, VMR_ERR_INVALID, "static mesh needs nodes and bounds");
    if (d->nodes) m.nodes.assign(d->nodes, d->nodes + d->n_nodes);
    for (int a = 0; a < 3; ++a) { m.bounds.lo[a] = d->bounds[a]; m.bounds.hi[a] = d->bounds[3 + a]; }
  }
  int st = upload_mesh(ctx, *rec);
  if (st != VMR_OK) return st;
  if (out_geom) *out_geom = (uint32_t)ctx->meshes.size();
  ctx->meshes.push_back(std::move(rec));
  return VMR_OK;
}

int vmr_mesh_info(vmr_ctx* ctx, uint32_t geom, uint32_t* n_nodes, uint32_t* n_mnodes, uint32_t* n_tris,
                  uint32_t* motion_keys) {
  if (!ctx || geom >= ctx->meshes.size()) return fail(ctx, VMR_ERR_INVALID, "bad geom id");
  const HostMesh& m = ctx->meshes[geom]->host;
  if (n_nodes) *n_nodes = (uint32_t)m.nodes.size();
  if (n_mnodes) *n_mnodes = (uint32_t)m.mnodes.size();
  if (n_tris) *n_tris = m.n_tris;
  if (motion_keys) *motion_keys = m.keys;
  return VMR_OK;
}

int vmr_mesh_export(vmr_ctx* ctx, uint32_t geom, vmr_qbvh_node* nodes, int32_t* accel_idx, uint32_t* idxp,
                    vmr_mqbvh_node* mnodes, float* mboxes, float* bounds) {
  if (!ctx || geom >= ctx->meshes.size()) return fail(ctx, VMR_ERR_INVALID, "bad geom id");
  const HostMesh& m = ctx->meshes[geom]->host;
  if (nodes && !m.nodes.empty()) std::memcpy(nodes, m.nodes.data(), m.nodes.size() * sizeof(vmr_qbvh_node));
  if (accel_idx && !m.accel_idx.empty()) std::memcpy(accel_idx, m.accel_idx.data(), m.accel_idx.size() * 4);
  if (idxp && !m.idxp.empty()) std::memcpy(idxp, m.idxp.data(), m.idxp.size() * 4);
  if (mnodes && !m.mnodes.empty()) std::memcpy(mnodes, m.mnodes.data(), m.mnodes.size() * sizeof(vmr_mqbvh_node));
  if (mboxes && !m.mboxes.empty()) std::memcpy(mboxes, m.mboxes.data(), m.mboxes.size() * 4);
  if (bounds) {
    if (m.motion()) {
      for (size_t k = 0; k < m.key_bounds.size(); ++k)
        for (int a = 0; a < 3; ++a) { bounds[6 * k + a] = m.key_bounds[k].lo[a]; bounds[6 * k + 3 + a] = m.key_bounds[k].hi[a]; }
    } else {
      for (int a = 0; a < 3; ++a) { bounds[a] = m.bounds.lo[a]; bounds[3 + a] = m.bounds.hi[a]; }
    }
  }
  return VMR_OK;
}

int vmr_scene_build(vmr_ctx* ctx, const uint32_t* geoms, uint32_t n) {
  if (!ctx || (n && !geoms)) return VMR_ERR_INVALID;
  std::vector<const HostMesh*> ms(n);
  std::vector<uint32_t> ids(geoms, geoms + n);
  for (uint32_t i = 0; i < n; ++i) {
    if (geoms[i] >= ctx->meshes.size()) return fail(ctx, VMR_ERR_INVALID, "bad geom id");
    if (ctx->meshes[geoms[i]]->owner >= 0)
      return fail(ctx, VMR_ERR_INVALID, "a Proc's child geom is traced through its Proc, not from the scene");
    ms[i] = &ctx->meshes[geoms[i]]->host;
  }
  if (ctx->device >= 0) cudaSetDevice(ctx->device);
  std::string why;
  HostTop top;
  if (!vmr::build_top_level(ms, ids, top, why)) return fail(ctx, VMR_ERR_INVALID, why);
  ctx->top.host = std::move(top);
  return refresh_top(ctx);
}

namespace {
// Decomposes n transform keys into rec.xkeys and uploads them (device
// contexts).  Returns a CUDA error or cudaSuccess.
cudaError_t set_keys(vmr_ctx* ctx, MeshRec& rec, const float* keys16, uint32_t n) {
  rec.xkeys.resize(n);
  for (uint32_t i = 0; i < n; ++i) vmr::anim::decompose(keys16 + 16 * i, rec.xkeys[i]);
  if (ctx->device < 0 || n < 2) return cudaSuccess;
  cudaError_t e = rec.dxkeys.ensure(sizeof(vmr::anim::Decomp) * n);
  if (e == cudaSuccess)
    e = cudaMemcpy(rec.dxkeys.p, rec.xkeys.data(), sizeof(vmr::anim::Decomp) * n, cudaMemcpyHostToDevice);
  return e;
}

// A new GeomInstance / Proc record: its transform keys (one key: the matrix
// rebuilt from the decomposition, as TimeKey returns it), the given bounds
// grown as BoundingBox.GrowVec3 does (BMin, then BMax), its children.
int add_group(vmr_ctx* ctx, int group, const uint32_t* children, uint32_t n_children, const float* keys16,
              uint32_t n_keys, const float bmin[3], const float bmax[3], int motion_keys, uint32_t* out_geom) {
  if (ctx->device >= 0) cudaSetDevice(ctx->device);
  auto rec = std::make_unique<MeshRec>();
  const uint32_t id = (uint32_t)ctx->meshes.size();
  HostMesh& h = rec->host;
  h.group = group;
  h.group_keys = motion_keys;
  for (int k = 0; k < 3; ++k) {
    float lo = INFINITY, hi = -INFINITY;
    lo = bmin[k] < lo ? bmin[k] : lo;
    hi = bmin[k] > hi ? bmin[k] : hi;
    lo = bmax[k] < lo ? bmax[k] : lo;
    hi = bmax[k] > hi ? bmax[k] : hi;
    h.bounds.lo[k] = lo;
    h.bounds.hi[k] = hi;
    rec->bounds6[k] = lo;
    rec->bounds6[3 + k] = hi;
  }
  VMR_CUDA(ctx, set_keys(ctx, *rec, keys16, n_keys));
  if (n_keys == 1) {
    rec->has_xf = true;
    vmr::anim::compose(rec->xkeys[0], rec->xf);
    vmr::anim::inverse(rec->xf, rec->xf_inv);
  }
  rec->children.assign(children, children + n_children);
  for (uint32_t i = 0; i < n_children; ++i) rec->child_hit.push_back(group == 1 ? (int32_t)id : (int32_t)children[i]);
  DMesh d{};
  d.kind = vmr::kGroup;
  d.group = (uint32_t)group;
  d.keys = 1;
  d.iter_cap = 2;
  if (ctx->device >= 0) {
    VMR_CUDA(ctx, upload(ctx, rec->dchildren, rec->children));
    VMR_CUDA(ctx, upload(ctx, rec->dchild_hit, rec->child_hit));
    VMR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    d.children = rec->dchildren.as<uint32_t>();
    d.child_hit = rec->dchild_hit.as<int32_t>();
  }
  d.n_children = n_children;
  fill_xf(*rec, d);
  rec->dmesh = d;
  ctx->meshes.push_back(std::move(rec));
  if (out_geom) *out_geom = id;
  return VMR_OK;
}
}  // namespace

int vmr_instance_add(vmr_ctx* ctx, uint32_t of, const float* keys16, uint32_t n_keys, const float bmin[3],
                     const float bmax[3], uint32_t* out_geom) {
  if (!ctx || !keys16 || n_keys < 1 || !bmin || !bmax) return VMR_ERR_INVALID;
  if (of >= ctx->meshes.size()) return fail(ctx, VMR_ERR_INVALID, "bad geom id");
  const MeshRec& c = *ctx->meshes[of];
  if (c.host.group) return fail(ctx, VMR_ERR_UNSUPPORTED, "an instance of an instance or Proc is not supported");
  if (c.owner >= 0) return fail(ctx, VMR_ERR_INVALID, "a Proc's child geom cannot be instanced");
  // Instance.MotionKeys is the instanced geom's (instance.go:144-148)
  return add_group(ctx, 1, &of, 1, keys16, n_keys, bmin, bmax, c.host.motion_keys(), out_geom);
}

int vmr_proc_add(vmr_ctx* ctx, const uint32_t* children, uint32_t n, const float* keys16, uint32_t n_keys,
                 const float bmin[3], const float bmax[3], uint32_t* out_geom) {
  if (!ctx || !children || n == 0 || (n_keys && !keys16) || !bmin || !bmax) return VMR_ERR_INVALID;
  for (uint32_t i = 0; i < n; ++i) {
    if (children[i] >= ctx->meshes.size()) return fail(ctx, VMR_ERR_INVALID, "bad geom id");
    const MeshRec& c = *ctx->meshes[children[i]];
    if (c.host.group) return fail(ctx, VMR_ERR_UNSUPPORTED, "a Proc's children are meshes or spheres");
    if (c.owner >= 0) return fail(ctx, VMR_ERR_INVALID, "a geom belongs to one Proc at most");
    for (uint32_t j = 0; j < i; ++j)
      if (children[j] == children[i]) return fail(ctx, VMR_ERR_INVALID, "a Proc lists a geom twice");
  }
  static const float kIdentity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  // Proc.PreRender: no Transform is one identity key (proc.go:157-160)
  const uint32_t nk = n_keys ? n_keys : 1u;
  int rc = add_group(ctx, 2, children, n, n_keys ? keys16 : kIdentity, nk, bmin, bmax, (int)nk, out_geom);
  if (rc != VMR_OK) return rc;
  for (uint32_t i = 0; i < n; ++i) ctx->meshes[children[i]]->owner = (int32_t)*out_geom;
  return VMR_OK;
}

int vmr_mesh_set_transform_keys(vmr_ctx* ctx, uint32_t geom, const float* keys16, uint32_t n_keys) {
  if (!ctx || (n_keys && !keys16)) return VMR_ERR_INVALID;
  if (geom >= ctx->meshes.size()) return fail(ctx, VMR_ERR_INVALID, "bad geom id");
  if (n_keys <= 1) return vmr_mesh_set_transform(ctx, geom, n_keys ? keys16 : nullptr);
  MeshRec& rec = *ctx->meshes[geom];
  if (rec.host.sphere || rec.host.group)
    return fail(ctx, VMR_ERR_UNSUPPORTED, "transform keys apply to meshes (PolyMesh.Transform)");
  if (ctx->device >= 0) cudaSetDevice(ctx->device);
  rec.has_xf = false;
  VMR_CUDA(ctx, set_keys(ctx, rec, keys16, n_keys));
  fill_xf(rec, rec.dmesh);
  if (ctx->top.valid) return refresh_top(ctx);
  return VMR_OK;
}

int vmr_mesh_set_transform(vmr_ctx* ctx, uint32_t geom, const float* m) {
  if (!ctx) return VMR_ERR_INVALID;
  if (geom >= ctx->meshes.size()) return fail(ctx, VMR_ERR_INVALID, "bad geom id");
  MeshRec& rec = *ctx->meshes[geom];
  if (m && rec.host.sphere) return fail(ctx, VMR_ERR_UNSUPPORTED, "an analytic sphere takes no transform");
  if (rec.host.group) return fail(ctx, VMR_ERR_UNSUPPORTED, "an instance or Proc takes its transform when added");
  rec.xkeys.clear();
  rec.has_xf = m != nullptr;
  if (m) {
    std::memcpy(rec.xf, m, sizeof(rec.xf));
    matrix4_inverse(rec.xf, rec.xf_inv);
  }
  fill_xf(rec, rec.dmesh);
  if (ctx->top.valid) return refresh_top(ctx);
  return VMR_OK;
}

int vmr_scene_upload(vmr_ctx* ctx, const vmr_qbvh_node* nodes, uint32_t n_nodes, const vmr_mqbvh_node* mnodes,
                     uint32_t n_mnodes, const float* mboxes, uint32_t keys, const uint32_t* order, uint32_t n_geoms) {
  if (!ctx || !order || keys < 1) return VMR_ERR_INVALID;
  for (uint32_t i = 0; i < n_geoms; ++i)
    if (order[i] >= ctx->meshes.size()) return fail(ctx, VMR_ERR_INVALID, "bad geom id in order");
  if (ctx->device >= 0) cudaSetDevice(ctx->device);
  HostTop top;
  top.keys = keys;
  top.geom_order.assign(order, order + n_geoms);
  if (keys == 1) {
    if (!nodes) return fail(ctx, VMR_ERR_INVALID, "static top level needs nodes");
    top.nodes.assign(nodes, nodes + n_nodes);
  } else {
    if (!mnodes || !mboxes) return fail(ctx, VMR_ERR_INVALID, "motion top level needs mnodes and mboxes");
    top.mnodes.assign(mnodes, mnodes + n_mnodes);
    top.mboxes.assign(mboxes, mboxes + (size_t)keys * n_mnodes * 24);
  }
  ctx->top.host = std::move(top);
  return refresh_top(ctx);
}

int vmr_scene_export(vmr_ctx* ctx, uint32_t* order, vmr_qbvh_node* nodes, vmr_mqbvh_node* mnodes, float* mboxes,
                     uint32_t* n_nodes, uint32_t* n_mnodes, uint32_t* keys) {
  if (!ctx) return VMR_ERR_INVALID;
  const HostTop& t = ctx->top.host;
  if (order && !t.geom_order.empty()) std::memcpy(order, t.geom_order.data(), t.geom_order.size() * 4);
  if (nodes && !t.nodes.empty()) std::memcpy(nodes, t.nodes.data(), t.nodes.size() * sizeof(vmr_qbvh_node));
  if (mnodes && !t.mnodes.empty()) std::memcpy(mnodes, t.mnodes.data(), t.mnodes.size() * sizeof(vmr_mqbvh_node));
  if (mboxes && !t.mboxes.empty()) std::memcpy(mboxes, t.mboxes.data(), t.mboxes.size() * 4);
  if (n_nodes) *n_nodes = (uint32_t)t.nodes.size();
  if (n_mnodes) *n_mnodes = (uint32_t)t.mnodes.size();
  if (keys) *keys = t.keys;
  return VMR_OK;
}

int vmr_trace_mesh(vmr_ctx* ctx, uint32_t geom, const vmr_rays* rays, size_t n, int flags, const vmr_hits* hits,
                   vmr_trace_stats* stats) {
  if (ctx && ctx->device < 0) return fail(ctx, VMR_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (!ctx || !rays || !hits) return VMR_ERR_INVALID;
  if (geom >= ctx->meshes.size()) return fail(ctx, VMR_ERR_INVALID, "bad geom id");
  cudaSetDevice(ctx->device);
  const DMesh* m = &ctx->meshes[geom]->dmesh;
  if (ctx->meshes[geom]->host.sphere || ctx->meshes[geom]->host.group)
    return fail(ctx, VMR_ERR_UNSUPPORTED, "sphere, instance and Proc geoms are traced through the scene (vmr_trace_scene)");
  if (ctx->meshes[geom]->host.n_tris == 0) return fail(ctx, VMR_ERR_INVALID, "empty mesh");
  if (flags & VMR_TRACE_DEVICE) return run_trace(ctx, m, *rays, n, flags, *hits, stats);
  return trace_host(ctx, m, rays, n, flags, hits, stats);
}

int vmr_trace_scene(vmr_ctx* ctx, const vmr_rays* rays, size_t n, int flags, const vmr_hits* hits,
                    vmr_trace_stats* stats) {
  if (ctx && ctx->device < 0) return fail(ctx, VMR_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (!ctx || !rays || !hits) return VMR_ERR_INVALID;
  if (!ctx->top.valid) return fail(ctx, VMR_ERR_INVALID, "no scene: call vmr_scene_build first");
  cudaSetDevice(ctx->device);
  if (flags & VMR_TRACE_DEVICE) return run_trace(ctx, nullptr, *rays, n, flags, *hits, stats);
  return trace_host(ctx, nullptr, rays, n, flags, hits, stats);
}


int vmr_clear_tuning(vmr_ctx* ctx, uint32_t geom) {
  if (!ctx || geom >= ctx->meshes.size()) return VMR_ERR_INVALID;
  ctx->meshes[geom]->tuned = false;
  return VMR_OK;
}

int vmr_autotune(vmr_ctx* ctx, uint32_t geom, const vmr_rays* rays, size_t n, int flags, vmr_tuning* best,
                 float* best_ms, uint32_t* n_tried) {
  if (!ctx || !rays || !best || n == 0) return VMR_ERR_INVALID;
  if (ctx->device < 0) return fail(ctx, VMR_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (geom >= ctx->meshes.size()) return fail(ctx, VMR_ERR_INVALID, "no such geom");
  MeshRec& mr = *ctx->meshes[geom];
  if (mr.host.group) return fail(ctx, VMR_ERR_UNSUPPORTED, "instances and Procs are not autotuned");
  if (mr.host.n_tris == 0) return fail(ctx, VMR_ERR_INVALID, "empty mesh");
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  // device copies of the sample and a hit buffer
  DevBuf buf;
  const size_t nf = (n + 63) / 64 * 64;
  VMR_CUDA(ctx, buf.ensure(nf * 4 * 13));
  float* f = buf.as<float>();
  vmr_rays dr{f, f + nf, f + 2 * nf, f + 3 * nf, f + 4 * nf, f + 5 * nf, f + 6 * nf, rays->time ? f + 7 * nf : nullptr};
  const float* src[8] = {rays->px, rays->py, rays->pz, rays->dx, rays->dy, rays->dz, rays->tmax, rays->time};
  const cudaMemcpyKind kind = (flags & VMR_TRACE_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  for (int k = 0; k < 8; ++k)
    if (src[k]) VMR_CUDA(ctx, cudaMemcpyAsync(f + k * nf, src[k], n * 4, kind, st));
  int32_t* hb = reinterpret_cast<int32_t*>(f + 8 * nf);
  vmr_hits dh{hb, nullptr, f + 9 * nf, f + 10 * nf, f + 11 * nf, f + 12 * nf};
  // candidates: while-while (with/without reordering, register cap, the
  // shared-memory stack top, tail cutoff, key width) and the step-scheduled
  // kernel
  std::vector<vmr_tuning> cands;
  for (int k : {13, 9, 29, 45, 41})
    for (int tail : {0, 2, 4, 8})
      for (int bits : {3, 4, 5}) cands.push_back(vmr_tuning{k, 0, 0, 0, tail, bits});
  for (int k : {5, 1})
    for (int tail : {0, 4}) cands.push_back(vmr_tuning{k, 0, 0, 0, tail, 0});
  for (int bits : {3, 4, 5}) cands.push_back(vmr_tuning{8, 256, 0, 4, 4, bits});
  cands.push_back(vmr_tuning{0, 256, 0, 4, 4, 0});
  const bool had = mr.tuned;
  const vmr_tuning old = mr.tuning;
  float best_t = INFINITY;
  vmr_tuning win = ctx->tuning;
  const int tflags = (flags & VMR_TRACE_ANY_HIT) | VMR_TRACE_DEVICE;
  for (const vmr_tuning& c : cands) {
    mr.tuned = true;
    mr.tuning = c;
    float tmin = INFINITY;
    for (int rep = 0; rep < 3; ++rep) {
      int rc = run_trace(ctx, &mr.dmesh, dr, n, tflags, dh, nullptr);
      if (rc != VMR_OK) {
        mr.tuned = had;
        mr.tuning = old;
        return rc;
      }
      VMR_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
      if (rep > 0) tmin = std::min(tmin, ms);
    }
    int rc = read_status(ctx, nullptr);
    if (rc != VMR_OK) {
      mr.tuned = had;
      mr.tuning = old;
      return rc;
    }
    if (tmin < best_t) {
      best_t = tmin;
      win = c;
    }
  }
  mr.tuned = true;
  mr.tuning = win;
  *best = win;
  if (best_ms) *best_ms = best_t;
  if (n_tried) *n_tried = (uint32_t)cands.size();
  return VMR_OK;
}

int vmr_trace_jobs(vmr_ctx* ctx, const vmr_trace_job* jobs, uint32_t n_jobs, int flags, vmr_trace_stats* stats) {
  if (!ctx || (n_jobs && !jobs)) return VMR_ERR_INVALID;
  if (ctx->device < 0) return fail(ctx, VMR_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (!(flags & VMR_TRACE_DEVICE)) return fail(ctx, VMR_ERR_INVALID, "vmr_trace_jobs takes device pointers");
  if (flags & VMR_TRACE_COUNT) return fail(ctx, VMR_ERR_UNSUPPORTED, "vmr_trace_jobs has no visit counters");
  cudaSetDevice(ctx->device);
  std::vector<vmr::JobDesc> t(n_jobs);
  std::vector<uint32_t> job_geom(n_jobs);
  uint64_t rays = 0;
  bool motion = false;
  for (uint32_t j = 0; j < n_jobs; ++j) {
    const vmr_trace_job& J = jobs[j];
    if (J.geom >= ctx->meshes.size()) return fail(ctx, VMR_ERR_INVALID, "job geom out of range");
    if (ctx->meshes[J.geom]->host.group || ctx->meshes[J.geom]->xkeys.size() >= 2)
      return fail(ctx, VMR_ERR_UNSUPPORTED, "job geoms are meshes (instances, Procs and keyed transforms are not)");
    const vmr_rays& r = J.rays;
    const vmr_hits& h = J.hits;
    if (J.n && (!r.px || !r.py || !r.pz || !r.dx || !r.dy || !r.dz || !r.tmax))
      return fail(ctx, VMR_ERR_INVALID, "job rays need px..tmax");
    t[j].rays = vmr::RaySoA{r.px, r.py, r.pz, r.dx, r.dy, r.dz, r.tmax, r.time};
    t[j].hits = vmr::HitSoA{h.prim, h.geom, h.t, h.u, h.v, h.w};
    t[j].n = J.n;
    t[j].ray0 = rays;
    job_geom[j] = J.geom;
    if (ctx->meshes[J.geom]->host.motion()) motion = true;
    rays += J.n;
  }
  if (stats) *stats = vmr_trace_stats{rays, 0, 0, 0, 0.f};
  if (rays == 0) return VMR_OK;
  // Each job is a mesh trace (qbvh.Trace on its mesh): the table the scene
  // kernel reads holds the meshes without their transforms.
  std::vector<DMesh> table(ctx->meshes.size());
  for (size_t g = 0; g < table.size(); ++g) {
    table[g] = ctx->meshes[g]->dmesh;
    table[g].has_xf = 0u;
  }
  // Gathered rays (8 floats) and hits (6 words) per ray, the ray -> job
  // index, the job -> geom table, the job table and the mesh table.
  const size_t nr = (size_t)rays;
  const size_t o_rays = 0, o_hits = o_rays + nr * 8 * 4, o_rj = o_hits + nr * 6 * 4, o_jg = o_rj + nr * 4,
               o_jobs = (o_jg + (size_t)n_jobs * 4 + 255) / 256 * 256,
               o_tab = (o_jobs + (size_t)n_jobs * sizeof(vmr::JobDesc) + 255) / 256 * 256,
               bytes = o_tab + table.size() * sizeof(DMesh);
  // The buffer is read by the launch; a pending launch of an earlier call may
  // still read it, so wait before overwriting it.
  VMR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  VMR_CUDA(ctx, ctx->jobs.ensure(bytes));
  char* base = ctx->jobs.as<char>();
  VMR_CUDA(ctx, cudaMemcpyAsync(base + o_jg, job_geom.data(), job_geom.size() * 4, cudaMemcpyHostToDevice,
                                ctx->stream));
  VMR_CUDA(ctx, cudaMemcpyAsync(base + o_jobs, t.data(), t.size() * sizeof(vmr::JobDesc), cudaMemcpyHostToDevice,
                                ctx->stream));
  VMR_CUDA(ctx, cudaMemcpyAsync(base + o_tab, table.data(), table.size() * sizeof(DMesh), cudaMemcpyHostToDevice,
                                ctx->stream));
  float* rf = reinterpret_cast<float*>(base + o_rays);
  float* hf = reinterpret_cast<float*>(base + o_hits);
  vmr::JobWork w;
  w.rays = vmr::RaySoA{rf, rf + nr, rf + 2 * nr, rf + 3 * nr, rf + 4 * nr, rf + 5 * nr, rf + 6 * nr, rf + 7 * nr};
  w.hits = vmr::HitSoA{reinterpret_cast<int32_t*>(hf), reinterpret_cast<int32_t*>(hf + nr), hf + 2 * nr,
                       hf + 3 * nr, hf + 4 * nr, hf + 5 * nr};
  w.ray_job = reinterpret_cast<uint32_t*>(base + o_rj);
  w.job_geom = reinterpret_cast<uint32_t*>(base + o_jg);
  DTop top{};
  top.meshes = reinterpret_cast<const DMesh*>(base + o_tab);
  top.n_geoms = (uint32_t)table.size();
  top.keys = 1;
  top.all_static = motion ? 0u : 1u;
  const vmr_tuning& tn = ctx->tuning;
  vmr::TraceLaunch l{};
  l.any_hit = (flags & VMR_TRACE_ANY_HIT) ? 1 : 0;
  l.scratch = ctx->scratch.as<DScratch>();
  l.grid = tn.blocks_per_sm;
  l.kernel = tn.kernel;
  l.walk_tail = tn.walk_tail;
  l.stream = ctx->stream;
  VMR_CUDA(ctx, cudaMemsetAsync(ctx->scratch.p, 0, sizeof(DScratch), ctx->stream));
  VMR_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  VMR_CUDA(ctx, cudaEventRecord(ctx->evm, ctx->stream));
  const int e = vmr::launch_trace_jobs(reinterpret_cast<const vmr::JobDesc*>(base + o_jobs), n_jobs, rays, top, w, l);
  if (e != 0) return cuda_fail(ctx, (cudaError_t)e, "jobs kernel launch");
  VMR_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  if (!stats) return VMR_OK;
  const int st = read_status(ctx, nullptr);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->evm, ctx->ev1);
  stats->kernel_ms = ms;
  return st;
}

}  // extern "C"
