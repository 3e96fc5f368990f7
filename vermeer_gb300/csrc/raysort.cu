// raysort.cu - ray reordering before traversal.
//
// Each ray gets the key  class * 2^(3b) + morton(origin),  where class =
// 2*Kz + (D[Kz] < 0) is the permutation the watertight test uses (Ray.Setup,
// core/ray.go:103-135) and morton interleaves a 2^b x 2^b x 2^b grid cell of
// the origin inside the scene bounds (b = 3, 4 or 5: the sort-key width the
// tuning chooses).  A one-pass bucket sort (histogram,
// exclusive scan, scatter) gathers the rays into key order: warps then trace
// rays that start close together and head into the same sixth of the
// sphere, and the triangle test can use one compile-time permutation per
// warp.  Inside a bucket, each warp's rays keep their input order and warps
// follow the atomics' order; every ray is traced independently, so results
// do not depend on it.
#include <cuda_runtime.h>

#include "device.h"

namespace vmr {
namespace {

__device__ __forceinline__ uint32_t spread5(uint32_t v) {  // abcde -> a..b..c..d..e
  v &= 31u;
  v = (v | (v << 8)) & 0x100fu;
  v = (v | (v << 4)) & 0x10c3u;
  v = (v | (v << 2)) & 0x1249u;
  return v;
}

__device__ __forceinline__ uint32_t cell(float p, float lo, float inv, float top) {
  const float q = fminf(fmaxf((p - lo) * inv, 0.0f), top);  // NaN -> 0
  return (uint32_t)q;
}

// The permutation class of Ray.Setup: Kz chosen by the strict |D|
// comparisons, and whether Kx/Ky were swapped because D[Kz] < 0.
__device__ __forceinline__ uint32_t ray_class(float dx, float dy, float dz) {
  const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  int kz = 0;
  if (ay > az) {
    if (ay > ax) kz = 1;
  } else {
    if (az > ax) kz = 2;
  }
  const float dkz = kz == 0 ? dx : (kz == 1 ? dy : dz);
  return 2u * (uint32_t)kz + (dkz < 0.0f ? 1u : 0u);
}

// Lanes of a warp that share a key take one atomic: the lowest such lane
// adds their count and hands each its slot in lane order (so a bucket that
// holds most rays, e.g. camera primaries from one eye, costs one atomic per
// warp rather than one per ray, and each warp's rays stay together in input
// order).  Every lane of the warp calls this; invalid lanes pass kNoKey.
constexpr uint32_t kNoKey = 0xffffffffu;
__device__ __forceinline__ uint32_t warp_bucket_add(uint32_t* counters, uint32_t key) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t peers = __match_any_sync(0xffffffffu, key);
  const uint32_t leader = (uint32_t)__ffs(peers) - 1u;
  uint32_t base = 0;
  if (lane == leader && key != kNoKey) base = atomicAdd(counters + key, (uint32_t)__popc(peers));
  base = __shfl_sync(0xffffffffu, base, (int)leader);
  return base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

// Grid-stride loops below run whole warps (blockDim.x is a multiple of 32)
// for the same number of rounds, so every lane reaches the warp collectives.
__global__ void k_ray_keys(RaySoA rays, uint64_t n, const unsigned long long* n_dev, float3 lo, float3 inv,
                           uint32_t bits, uint32_t* keys, uint32_t* hist) {
  if (n_dev && *n_dev < n) n = *n_dev;
  const float top = (float)((1u << bits) - 1u);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t rounds = (n + stride - 1) / stride;
  for (uint64_t r = 0; r < rounds; ++r) {
    const uint64_t i = r * stride + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint32_t k = kNoKey;
    if (i < n) {
      const uint32_t c = ray_class(rays.dx[i], rays.dy[i], rays.dz[i]);
      const uint32_t m = spread5(cell(rays.px[i], lo.x, inv.x, top)) << 2 |
                         spread5(cell(rays.py[i], lo.y, inv.y, top)) << 1 | spread5(cell(rays.pz[i], lo.z, inv.z, top));
      k = (c << (3 * bits)) + m;
      keys[i] = k;
    }
    warp_bucket_add(hist, k);
  }
}

// Exclusive scan of nb counters in one block of 1024 threads (each thread a
// contiguous range, read twice).
__global__ void __launch_bounds__(1024) k_bucket_scan(uint32_t* hist, uint32_t nb) {
  __shared__ uint32_t part[1024];
  const uint32_t t = threadIdx.x;
  const uint32_t per = (nb + 1023) / 1024;
  uint32_t sum = 0;
  for (uint32_t j = 0; j < per; ++j) {
    const uint32_t b = t * per + j;
    sum += b < nb ? hist[b] : 0u;
  }
  part[t] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const uint32_t v = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  uint32_t run = part[t] - sum;  // exclusive prefix of this thread's range
  for (uint32_t j = 0; j < per; ++j) {
    const uint32_t b = t * per + j;
    if (b < nb) {
      const uint32_t v = hist[b];
      hist[b] = run;
      run += v;
    }
  }
}

__global__ void k_ray_scatter(RaySoA rays, uint64_t n, const unsigned long long* n_dev, const uint32_t* keys,
                              uint32_t* offsets, uint32_t* order, RaySoA sorted_out) {
  if (n_dev && *n_dev < n) n = *n_dev;
  float* px = const_cast<float*>(sorted_out.px);
  float* py = const_cast<float*>(sorted_out.py);
  float* pz = const_cast<float*>(sorted_out.pz);
  float* dx = const_cast<float*>(sorted_out.dx);
  float* dy = const_cast<float*>(sorted_out.dy);
  float* dz = const_cast<float*>(sorted_out.dz);
  float* tm = const_cast<float*>(sorted_out.tmax);
  float* ti = const_cast<float*>(sorted_out.time);
  float4* rec = static_cast<float4*>(const_cast<void*>(sorted_out.rec));
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t rounds = (n + stride - 1) / stride;
  for (uint64_t r = 0; r < rounds; ++r) {
    const uint64_t i = r * stride + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint32_t pos = warp_bucket_add(offsets, i < n ? keys[i] : kNoKey);
    if (i >= n) continue;
    if (rec) {  // one ray = two 16-byte stores instead of eight scattered 4-byte ones
      rec[2 * (size_t)pos] = make_float4(rays.px[i], rays.py[i], rays.pz[i], rays.dx[i]);
      rec[2 * (size_t)pos + 1] = make_float4(rays.dy[i], rays.dz[i], rays.tmax[i], __uint_as_float((uint32_t)i));
      continue;
    }
    order[pos] = (uint32_t)i;
    px[pos] = rays.px[i];
    py[pos] = rays.py[i];
    pz[pos] = rays.pz[i];
    dx[pos] = rays.dx[i];
    dy[pos] = rays.dy[i];
    dz[pos] = rays.dz[i];
    tm[pos] = rays.tmax[i];
    if (ti) ti[pos] = rays.time ? rays.time[i] : 0.0f;
  }
}

}  // namespace

int launch_ray_sort(const RaySoA& rays, uint64_t n, const float bounds[6], int bits, uint32_t* keys, uint32_t* hist,
                    uint32_t* order, const RaySoA& sorted_out, void* stream, const unsigned long long* n_dev) {
  cudaStream_t s = (cudaStream_t)stream;
  if (bits < 3 || bits > kSortMaxBits) bits = 4;
  const uint32_t nb = sort_buckets(bits);
  const float side = (float)(1u << bits);
  float3 lo = make_float3(bounds[0], bounds[1], bounds[2]);
  float3 inv;
  const float ext[3] = {bounds[3] - bounds[0], bounds[4] - bounds[1], bounds[5] - bounds[2]};
  inv.x = ext[0] > 0.f ? side / ext[0] : 0.f;
  inv.y = ext[1] > 0.f ? side / ext[1] : 0.f;
  inv.z = ext[2] > 0.f ? side / ext[2] : 0.f;
  cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(uint32_t) * nb, s);
  if (e != cudaSuccess) return (int)e;
  const int block = 256;
  int grid = (int)((n + block - 1) / block);
  const int cap = device_sm_count() * 16;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  k_ray_keys<<<grid, block, 0, s>>>(rays, n, n_dev, lo, inv, (uint32_t)bits, keys, hist);
  k_bucket_scan<<<1, 1024, 0, s>>>(hist, nb);
  k_ray_scatter<<<grid, block, 0, s>>>(rays, n, n_dev, keys, hist, order, sorted_out);
  return (int)cudaGetLastError();
}

}  // namespace vmr
