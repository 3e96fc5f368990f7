// noalloc.cu - vmr_trace_mesh_noalloc: a mesh trace that allocates nothing.
//
// Some callers cannot let a library allocate device memory while they run: a
// host that reserves and sub-allocates the whole device itself, or a frame
// loop whose time budget has no room for cudaMalloc's synchronisation and
// latency.  vmr_trace_mesh (device pointers) may still allocate, because the
// context grows its ray-reordering buffers to the largest batch seen.  This
// entry point runs the same reordering and traversal kernels on a fixed
// scratch area instead: one file-scope device array, sized for
// VMR_NOALLOC_MAX_RAYS rays and loaded with the library on every GPU that
// uses it, where it stays until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "device.h"
#include "vmr.h"

namespace vmr {
bool ctx_noalloc_view(vmr_ctx* ctx, uint32_t geom, const DMesh** mesh, const float** bounds, void** stream,
                      int* device, vmr_tuning* tuning);
int ctx_fail(vmr_ctx* ctx, int code, const char* msg);
}  // namespace vmr

namespace {

constexpr size_t kMaxRays = VMR_NOALLOC_MAX_RAYS;
// Layout: work counter / status / visit counters, bucket histogram, ray keys,
// order, key-ordered rays (8 float fields).  Every part starts on a 256-byte
// boundary.
constexpr size_t kHeaderBytes = 256;
constexpr size_t kHistBytes = ((sizeof(uint32_t) * vmr::kSortBuckets + 255) / 256) * 256;
constexpr size_t kKeyBytes = sizeof(uint32_t) * kMaxRays;
constexpr size_t kOrderBytes = sizeof(uint32_t) * kMaxRays;
constexpr size_t kRayBytes = sizeof(float) * 8 * kMaxRays;
constexpr size_t kScratchBytes = kHeaderBytes + kHistBytes + kKeyBytes + kOrderBytes + kRayBytes;
static_assert(sizeof(vmr::DScratch) <= kHeaderBytes, "scratch header too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// The device address of g_noalloc_scratch on the current device (resolved on
// the first call for that device; host code only sees a stand-in for the
// symbol, never its device address).
cudaError_t scratch_address(int device, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_addr[device];
  return cudaSuccess;
}

}  // namespace

extern "C" int vmr_trace_mesh_noalloc(vmr_ctx* ctx, uint32_t geom, const vmr_rays* rays, size_t n, int flags,
                                      const vmr_hits* hits) {
  if (!ctx || !rays || !hits) return VMR_ERR_INVALID;
  const vmr::DMesh* mesh = nullptr;
  const float* bounds = nullptr;
  void* stream = nullptr;
  int device = -1;
  vmr_tuning tuning{};
  if (!vmr::ctx_noalloc_view(ctx, geom, &mesh, &bounds, &stream, &device, &tuning))
    return vmr::ctx_fail(ctx, VMR_ERR_INVALID, "vmr_trace_mesh_noalloc: bad geom id, empty mesh or host-only context");
  if (n > kMaxRays)
    return vmr::ctx_fail(ctx, VMR_ERR_INVALID,
                         "vmr_trace_mesh_noalloc: batch larger than VMR_NOALLOC_MAX_RAYS (262144 rays); "
                         "split it or use vmr_trace_mesh");
  if (flags & ~(VMR_TRACE_ANY_HIT | VMR_TRACE_DEVICE))
    return vmr::ctx_fail(ctx, VMR_ERR_INVALID, "vmr_trace_mesh_noalloc: only VMR_TRACE_ANY_HIT and VMR_TRACE_DEVICE");
  if (device >= kMaxDevices) return vmr::ctx_fail(ctx, VMR_ERR_UNSUPPORTED, "vmr_trace_mesh_noalloc: device >= 64");
  if (n == 0) return VMR_OK;
  cudaError_t e = cudaSetDevice(device);
  unsigned char* base = nullptr;
  if (e == cudaSuccess) e = scratch_address(device, &base);
  if (e != cudaSuccess)
    return vmr::ctx_fail(ctx, VMR_ERR_CUDA, "vmr_trace_mesh_noalloc: cannot resolve the scratch address");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto* scratch = reinterpret_cast<vmr::DScratch*>(base);
  auto* hist = reinterpret_cast<uint32_t*>(base + kHeaderBytes);
  auto* keys = reinterpret_cast<uint32_t*>(base + kHeaderBytes + kHistBytes);
  auto* order = reinterpret_cast<uint32_t*>(base + kHeaderBytes + kHistBytes + kKeyBytes);
  auto* f = reinterpret_cast<float*>(base + kHeaderBytes + kHistBytes + kKeyBytes + kOrderBytes);

  // The work counter and status word must start at zero: the last call left
  // its values behind.
  e = cudaMemsetAsync(scratch, 0, sizeof(vmr::DScratch), s);
  if (e != cudaSuccess) return vmr::ctx_fail(ctx, VMR_ERR_CUDA, "vmr_trace_mesh_noalloc: scratch reset failed");

  vmr::TraceLaunch l{};
  l.rays = vmr::RaySoA{rays->px, rays->py, rays->pz, rays->dx, rays->dy, rays->dz, rays->tmax, rays->time};
  l.hits = vmr::HitSoA{hits->prim, hits->geom, hits->t, hits->u, hits->v, hits->w};
  l.n = n;
  l.any_hit = (flags & VMR_TRACE_ANY_HIT) ? 1 : 0;
  l.scratch = scratch;
  l.stream = stream;
  l.kernel = tuning.kernel;
  l.block = tuning.block;
  l.grid = tuning.blocks_per_sm;
  l.refill_min = tuning.refill_min;
  l.walk_tail = tuning.walk_tail;
  if ((tuning.kernel & vmr::kKernelSort) && n >= vmr::kSortMinRays) {
    const vmr::RaySoA sorted{f, f + kMaxRays, f + 2 * kMaxRays, f + 3 * kMaxRays, f + 4 * kMaxRays,
                             f + 5 * kMaxRays, f + 6 * kMaxRays, rays->time ? f + 7 * kMaxRays : nullptr};
    if (vmr::launch_ray_sort(l.rays, n, bounds, 4, keys, hist, order, sorted, stream) != 0)
      return vmr::ctx_fail(ctx, VMR_ERR_CUDA, "vmr_trace_mesh_noalloc: ray reordering launch failed");
    l.rays = sorted;
    l.order = order;
  }
  if (vmr::launch_trace_mesh(*mesh, l) != 0)
    return vmr::ctx_fail(ctx, VMR_ERR_CUDA, "vmr_trace_mesh_noalloc: traversal launch failed");
  int status = 0;
  e = cudaMemcpyAsync(&status, &scratch->status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return vmr::ctx_fail(ctx, VMR_ERR_CUDA, "vmr_trace_mesh_noalloc: trace failed");
  if (status == vmr::kStatusStackOverflow)
    return vmr::ctx_fail(ctx, VMR_ERR_STACK_OVERFLOW, "a ray needed more than 90 traversal stack entries");
  if (status == vmr::kStatusIterationCap)
    return vmr::ctx_fail(ctx, VMR_ERR_TIMEOUT, "a traversal loop hit its iteration cap");
  return VMR_OK;
}
