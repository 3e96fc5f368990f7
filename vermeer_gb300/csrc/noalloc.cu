// noalloc.cu - vmr_trace_mesh_noalloc: a mesh trace that allocates nothing.
//
// Some callers cannot let a library allocate device memory while they run: a
// host that reserves and sub-allocates the whole device itself, or a frame
// loop whose time budget has no room for cudaMalloc's synchronisation and
// latency.  vmr_trace_mesh (device pointers) may still allocate, because the
// context grows its ray-reordering buffers to the largest batch seen.  This
// entry point runs the same reordering and traversal kernels on a fixed
// scratch area instead: one file-scope device array, sized for
// VMR_NOALLOC_MAX_RAYS rays and a histogram of any key width, where it stays
// until the process exits.  vmr_create resolves the array's device address
// for its device (noalloc_setup below), which is where the array is loaded
// onto that GPU; the entry point itself only reads the cached address.
#include <cuda_runtime.h>

#include <mutex>

#include "device.h"
#include "vmr.h"

namespace vmr {
bool ctx_noalloc_view(vmr_ctx* ctx, uint32_t geom, const DMesh** mesh, const float** bounds, void** stream,
                      int* device, vmr_tuning* tuning);
int ctx_fail(vmr_ctx* ctx, int code, const char* msg);
int noalloc_setup(int device);
}  // namespace vmr

namespace {

constexpr size_t kMaxRays = VMR_NOALLOC_MAX_RAYS;
// Layout: work counter / status / visit counters, bucket histogram (sized for
// the widest sort key a tuning may select), ray keys, order, key-ordered rays
// (8 float fields, or 32-byte records for static meshes).  Every part starts
// on a 256-byte boundary.
constexpr size_t kHeaderBytes = 256;
constexpr size_t kHistBytes = ((sizeof(uint32_t) * vmr::kSortBucketsMax + 255) / 256) * 256;
constexpr size_t kKeyBytes = sizeof(uint32_t) * kMaxRays;
constexpr size_t kOrderBytes = sizeof(uint32_t) * kMaxRays;
constexpr size_t kRayBytes = sizeof(float) * 8 * kMaxRays;
constexpr size_t kScratchBytes = kHeaderBytes + kHistBytes + kKeyBytes + kOrderBytes + kRayBytes;
static_assert(sizeof(vmr::DScratch) <= kHeaderBytes, "scratch header too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// The device address of g_noalloc_scratch on the current device.  Host code
// only sees a stand-in for the symbol, never its device address, so the
// address is looked up once per device with that device current.
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

unsigned char* cached_address(int device) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  return g_scratch_addr[device];
}

// True when p is memory the GPU addresses directly (device or managed).
bool device_pointer(const void* p) {
  if (!p) return true;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

namespace vmr {
// Called by vmr_create with the context's device current: resolves (and so
// loads) the scratch array on that device.  Returns the CUDA error, 0 on
// success; a failure leaves later no-alloc calls on the device to report it.
int noalloc_setup(int device) {
  if (device < 0 || device >= kMaxDevices) return 0;
  unsigned char* base = nullptr;
  const cudaError_t e = scratch_address(device, &base);
  if (e != cudaSuccess) cudaGetLastError();
  return (int)e;
}
}  // namespace vmr

extern "C" int vmr_trace_mesh_noalloc(vmr_ctx* ctx, uint32_t geom, const vmr_rays* rays, size_t n, int flags,
                                      const vmr_hits* hits) {
  if (!ctx || !rays || !hits) return VMR_ERR_INVALID;
  // Checked before anything touches the GPU: the kernels read rays and write
  // hits in place, so host arrays must never reach them.
  if (!(flags & VMR_TRACE_DEVICE))
    return vmr::ctx_fail(ctx, VMR_ERR_INVALID,
                         "vmr_trace_mesh_noalloc: rays and hits must be device pointers; set VMR_TRACE_DEVICE");
  if (flags & ~(VMR_TRACE_ANY_HIT | VMR_TRACE_DEVICE))
    return vmr::ctx_fail(ctx, VMR_ERR_INVALID, "vmr_trace_mesh_noalloc: only VMR_TRACE_ANY_HIT and VMR_TRACE_DEVICE");
  if (n > kMaxRays)
    return vmr::ctx_fail(ctx, VMR_ERR_INVALID,
                         "vmr_trace_mesh_noalloc: batch larger than VMR_NOALLOC_MAX_RAYS (262144 rays); "
                         "split it or use vmr_trace_mesh");
  const vmr::DMesh* mesh = nullptr;
  const float* bounds = nullptr;
  void* stream = nullptr;
  int device = -1;
  vmr_tuning tuning{};
  if (!vmr::ctx_noalloc_view(ctx, geom, &mesh, &bounds, &stream, &device, &tuning))
    return vmr::ctx_fail(ctx, VMR_ERR_INVALID, "vmr_trace_mesh_noalloc: bad geom id, empty mesh or host-only context");
  if (device >= kMaxDevices) return vmr::ctx_fail(ctx, VMR_ERR_UNSUPPORTED, "vmr_trace_mesh_noalloc: device >= 64");
  if (n == 0) return VMR_OK;
  if (cudaSetDevice(device) != cudaSuccess)
    return vmr::ctx_fail(ctx, VMR_ERR_CUDA, "vmr_trace_mesh_noalloc: cannot select the context's device");
  const void* ptrs[14] = {rays->px, rays->py, rays->pz, rays->dx, rays->dy, rays->dz, rays->tmax, rays->time,
                          hits->prim, hits->geom, hits->t, hits->u, hits->v, hits->w};
  for (const void* p : ptrs)
    if (!device_pointer(p))
      return vmr::ctx_fail(ctx, VMR_ERR_INVALID,
                           "vmr_trace_mesh_noalloc: a ray or hit array is not device memory");
  if (!rays->px || !rays->py || !rays->pz || !rays->dx || !rays->dy || !rays->dz || !rays->tmax)
    return vmr::ctx_fail(ctx, VMR_ERR_INVALID, "vmr_trace_mesh_noalloc: null ray array");
  unsigned char* base = cached_address(device);
  if (!base)
    return vmr::ctx_fail(ctx, VMR_ERR_CUDA,
                         "vmr_trace_mesh_noalloc: the scratch array could not be resolved when the context was created");
  cudaError_t e = cudaSuccess;
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
    // a static mesh in the while-while kernel reads the copy as 32-byte
    // records (RaySoA::rec), which fill the ray region exactly
    const bool recs = mesh->keys <= 1 && !rays->time && (tuning.kernel & vmr::kKernelWhileWhile);
    vmr::RaySoA sorted{f, f + kMaxRays, f + 2 * kMaxRays, f + 3 * kMaxRays, f + 4 * kMaxRays,
                       f + 5 * kMaxRays, f + 6 * kMaxRays, rays->time ? f + 7 * kMaxRays : nullptr};
    if (recs) sorted = vmr::RaySoA{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, f};
    const int bits = tuning.sort_bits ? tuning.sort_bits : 4;
    if (bits > vmr::kSortMaxBits)
      return vmr::ctx_fail(ctx, VMR_ERR_INVALID, "vmr_trace_mesh_noalloc: sort key wider than the histogram");
    if (vmr::launch_ray_sort(l.rays, n, bounds, bits, keys, hist, order, sorted, stream) != 0)
      return vmr::ctx_fail(ctx, VMR_ERR_CUDA, "vmr_trace_mesh_noalloc: ray reordering launch failed");
    l.rays = sorted;
    l.order = recs ? nullptr : order;
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
