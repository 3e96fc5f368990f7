// guide.cu - the path-guiding network on the 5th-generation tensor cores.
//
// No reference counterpart.  The network (80 inputs, 4 hidden ReLU layers
// of 64, 41 outputs = 8 vMF lobes and the selection logit; no biases, input
// 78 is the constant 1) runs fused per tile of 128 rows: a group of 128
// threads works on a tile with the bf16 weights in shared memory (several
// groups per CTA share one copy), thread r owns row r, and each layer is
//   A (128 x K activations, smem) * B (N x K weights, smem) -> D (TMEM, fp32)
// issued as K/16 tcgen05.mma (kind::f16, bf16 inputs, fp32 accumulate) by
// one thread and committed to the group's mbarrier; every thread then reads
// its row of D with tcgen05.ld, applies ReLU, rounds to bf16 and writes the
// next layer's input over the tile the MMA has finished reading.  Operands
// use the no-swizzle K-major canonical layout: 8-row x 16-byte core matrices
// of 128 contiguous bytes, LBO = 128 (next core matrix along K), SBO =
// (K/8)*128 (next 8-row group).
//
//   k_guide_infer   forward for path vertices (features computed in-kernel)
//   k_guide_train   forward, loss gradient at the outputs, backward-data
//                   (dH = dZ * W through transposed weight copies), storing
//                   every layer's input and output delta chunk-blocked
//   k_guide_wgrad   weight gradients dW_l = dZ_{l+1}^T H_l as M = 64
//                   tensor-core GEMMs whose K dimension is the batch; each
//                   chunk's operands are one bulk async copy each
//                   (cp.async.bulk) through a 3-stage mbarrier pipeline
//   k_guide_adam    Adam on float32 master weights, then the bf16 copies
//
// Every mbarrier wait is bounded: a wait that runs out sets the error word,
// the CTA stops issuing work, frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "guide.h"
#include "vmr.h"

namespace vmr {
namespace guide {
namespace {

// ------------------------------------------------------------- PTX glue ---
__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start >> 4 at bit 0, LBO >> 4
// at 16, SBO >> 4 at 32, the fixed 0b001 at 46, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
               : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait for the phase `parity` of an mbarrier to complete.  try_wait
// suspends the thread in hardware until the phase completes (or a short
// system time limit passes), so waiting threads take no issue slots from
// the other tile groups' epilogues; the wait gives up after one second of
// global time (or 2^24 tries, whichever comes first).
constexpr uint64_t kWaitNs = 1000000000ull;
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = saddr(bar);
  uint64_t t0 = 0;
  for (uint32_t i = 0; i < (1u << 24); ++i) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    const uint64_t t = global_ns();
    if (i == 0) t0 = t;
    else if (t - t0 > kWaitNs) return false;
  }
  return false;
}
// 16 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------ layouts ---
// Byte offset of the 16-byte chunk (row r, columns 8c..8c+7) of a K-major
// canonical tile with K columns.
__device__ __forceinline__ uint32_t chunk_off(uint32_t r, uint32_t c, uint32_t K) {
  return ((r >> 3) * (K >> 3) + c) * 128u + (r & 7u) * 16u;
}
__device__ __forceinline__ uint32_t pack2(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}
// max(a, 0) and max(b, 0) rounded to bf16 and packed (a in the low half) by
// one conversion: a negative value converts to +0, the same bits as
// rounding the ReLU's output.
__device__ __forceinline__ uint32_t pack2_relu(float a, float b) {
  uint32_t d;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(b), "f"(a));
  return d;
}
// Row r of a K-major tile from K fp32 values (rounded to bf16).
__device__ __forceinline__ void put_row(char* tile, uint32_t r, uint32_t K, const float* v) {
  for (uint32_t c = 0; c < K / 8; ++c) {
    uint4 q;
    q.x = pack2(v[8 * c + 0], v[8 * c + 1]);
    q.y = pack2(v[8 * c + 2], v[8 * c + 3]);
    q.z = pack2(v[8 * c + 4], v[8 * c + 5]);
    q.w = pack2(v[8 * c + 6], v[8 * c + 7]);
    *reinterpret_cast<uint4*>(tile + chunk_off(r, c, K)) = q;
  }
}
// A [N][K] row-major bf16 matrix from global memory into a K-major tile.
__device__ void load_tile(char* tile, const __nv_bfloat16* g, uint32_t N, uint32_t K) {
  const uint32_t chunks = N * (K / 8);
  for (uint32_t i = threadIdx.x; i < chunks; i += blockDim.x) {
    const uint32_t r = i / (K / 8), c = i % (K / 8);
    *reinterpret_cast<uint4*>(tile + chunk_off(r, c, K)) = *reinterpret_cast<const uint4*>(g + (size_t)r * K + 8 * c);
  }
}

// Issue D = A * B^T over K (one thread), commit to bar.
__device__ __forceinline__ void gemm_issue(uint32_t tmem, const char* A, const char* B, uint32_t K, uint32_t N,
                                           uint64_t* bar) {
  fence_after();
  const uint32_t a0 = saddr(A), b0 = saddr(B);
  const uint32_t sbo = (K / 8) * 128u;
  const uint32_t id = idesc(128, (int)N);
  for (uint32_t kk = 0; kk < K / 16; ++kk)
    mma(tmem, sdesc(a0 + kk * 256u, 128u, sbo), sdesc(b0 + kk * 256u, 128u, sbo), id, kk > 0 ? 1u : 0u);
  mma_commit(bar);
}

// ---------------------------------------------------------- the network ---
// Global bf16 weight copies: forward B operands [N][K] (W4 padded to 48 rows)
// and transposed backward B operands [K_in][N_out] (W4^T padded to 48 columns).
constexpr uint32_t kWf0 = 0, kWf1 = 64 * 80, kWf2 = kWf1 + 4096, kWf3 = kWf2 + 4096, kWf4 = kWf3 + 4096,
                   kWfSize = kWf4 + 48 * 64;
constexpr uint32_t kWb1 = 0, kWb2 = 4096, kWb3 = 8192, kWb4 = 12288, kWbSize = kWb4 + 64 * 48;

// Shared-memory plan (bytes; all tiles 1024-aligned): the forward weights,
// then (training) the transposed weights, then the groups' activation tiles.
constexpr uint32_t kSW0 = 0, kSW1 = kSW0 + 64 * 80 * 2, kSW2 = kSW1 + 8192, kSW3 = kSW2 + 8192, kSW4 = kSW3 + 8192,
                   kSWEnd = kSW4 + 48 * 64 * 2;  // 40960
constexpr uint32_t kSB1 = kSWEnd, kSB2 = kSB1 + 8192, kSB3 = kSB2 + 8192, kSB4 = kSB3 + 8192,
                   kSBEnd = kSB4 + 64 * 48 * 2;  // 71680

constexpr int kLobes = 8;

// Input features of a vertex (the encoding the oracle's guide_features
// restates), for the training kernel.  sin and cos of pi 2^k q are exact
// (sincospif) at k = 0 and 8 and carried to the other frequencies by the
// double-angle identities sin 2x = 2 sin x cos x, cos 2x = (cos x - sin x)
// (cos x + sin x): at most seven steps, an absolute error below 2e-5, far
// under the bf16 rounding the features then get (the inference kernel
// builds the same values in freq_words).
__device__ void features(const float* p, const float* n, const float* wo, const float* lo, const float* inv_ext,
                         float* f) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float q = (p[c] - lo[c]) * inv_ext[c];
    float s = 0.f, co = 1.f;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      if (k == 0 || k == 8) {
        sincospif(ldexpf(q, k), &s, &co);
      } else {
        const float s2 = 2.0f * s * co;
        co = (co - s) * (co + s);
        s = s2;
      }
      f[24 * c + 2 * k] = s;
      f[24 * c + 2 * k + 1] = co;
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    f[72 + c] = n[c];
    f[75 + c] = wo[c];
  }
  f[78] = 1.0f;
  f[79] = 0.0f;
}

// Mixture parameters and loss gradient at the outputs (the oracle's
// loss_grad_out in float): the lobes descend -weight * log p_guide; with a
// BSDF density (pb >= 0) the selection logit descends -weight * log q, q =
// alpha p_guide + (1 - alpha) p_bsdf, alpha = amax * sigmoid(o[40]), with
// p_guide held fixed; loss = -weight * log q (or log p_guide).
constexpr float kLogKapMin = -4.6f, kLogKapMax = 6.9f;  // kappa in [0.01, 992]
__device__ void out_grad(const float* o, const float* w, float weight, float pb, float amax, float* g, float& loss) {
  float mx = -INFINITY;
#pragma unroll
  for (int k = 0; k < kLobes; ++k) mx = fmaxf(mx, o[5 * k + 4]);
  float pi[kLobes], v[kLobes], mu[kLobes][3], rn[kLobes], kap[kLobes];
  bool cl[kLobes];
  float z = 0.f;
#pragma unroll
  for (int k = 0; k < kLobes; ++k) {
    const float* r = o + 5 * k;
    float n = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    n = n < 1e-6f ? 1e-6f : n;
    rn[k] = n;
    for (int c = 0; c < 3; ++c) mu[k][c] = r[c] / n;
    const float s = r[3];
    cl[k] = s < kLogKapMin || s > kLogKapMax;
    kap[k] = expf(fminf(fmaxf(s, kLogKapMin), kLogKapMax));
    pi[k] = expf(r[4] - mx);
    z += pi[k];
  }
  float p = 0.f;
#pragma unroll
  for (int k = 0; k < kLobes; ++k) {
    pi[k] /= z;
    const float d = mu[k][0] * w[0] + mu[k][1] * w[1] + mu[k][2] * w[2];
    const float c = kap[k] / (6.28318530718f * (-expm1f(-2.f * kap[k])));
    v[k] = c * expf(kap[k] * (d - 1.f));
    p += pi[k] * v[k];
  }
  p = fmaxf(p, 1e-30f);
  loss = -weight * logf(p);
  g[40] = 0.f;
  if (pb >= 0.f) {
    const float sg = 1.f / (1.f + expf(-o[40]));
    const float a = amax * sg;
    const float q = fmaxf(a * p + (1.f - a) * pb, 1e-30f);
    g[40] = -weight * (p - pb) / q * (amax * sg * (1.f - sg));
    loss = -weight * logf(q);
  }
#pragma unroll
  for (int k = 0; k < kLobes; ++k) {
    const float rr = pi[k] * v[k] / p;
    const float d = mu[k][0] * w[0] + mu[k][1] * w[1] + mu[k][2] * w[2];
    g[5 * k + 4] = -weight * (rr - pi[k]);
    const float dl = 1.f / kap[k] - 2.f / expm1f(2.f * kap[k]) + (d - 1.f);
    g[5 * k + 3] = cl[k] ? 0.f : -weight * rr * dl * kap[k];
    for (int c = 0; c < 3; ++c) g[5 * k + c] = -weight * rr * kap[k] * (w[c] - d * mu[k][c]) / rn[k];
  }
}

// Inference: one CTA per SM runs six tile streams.  768 threads in six
// groups of four warps share one copy of the weights; each group owns one
// 128 x 80 activation tile (a layer's MMA has completed before its epilogue
// writes the next layer's input over the same tile), an mbarrier, a named
// barrier (ids 1..6) and 64 TMEM columns (the 32x32b loads reach TMEM lanes
// 32*(warp % 4) .. +31, so every group's warps read the same 128 lanes in
// their own columns).  With six independent five-layer chains per SM the
// tensor pipe has MMAs from some group while the others run their
// epilogues (TMEM -> ReLU -> bf16 -> shared memory).  Registers stay within
// 85 per thread: the input encoding is built one 16-byte chunk (8 features)
// at a time and the epilogues run in halves of 32 columns.
constexpr uint32_t kGroups = 6;
constexpr uint32_t kInferThreads = 128 * kGroups;
// tcgen05.alloc takes a power of two of columns (>= 32): 64 a group, rounded up
constexpr uint32_t kInferTmemCols = 64 * kGroups <= 256 ? (64 * kGroups <= 128 ? 128 : 256) : 512;
static_assert(64 * kGroups <= kInferTmemCols && kInferTmemCols <= 512, "inference tensor memory");
constexpr uint32_t kSAGroup = 128 * 80 * 2;  // one group's activation tile: 20480
// Dynamic shared memory: weights, the groups' tiles, then the control block
// (kGroups mbarrier records, then the TMEM address slot).
constexpr uint32_t kInferCtl = kSWEnd + kGroups * kSAGroup;

__device__ __forceinline__ void group_sync(uint32_t id) {
  asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory");
}
// OR over the group's 128 threads (barrier.red on the group's named barrier).
__device__ __forceinline__ bool group_any(bool v, uint32_t id) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, 128, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id)
      : "memory");
  return r != 0;
}

struct GroupShared {
  uint64_t bar;
  int abort;
};
constexpr uint32_t kInferSlot = kInferCtl + kGroups * (uint32_t)sizeof(GroupShared);
constexpr uint32_t kInferSmem2 = kInferSlot + 16;
static_assert(kInferSmem2 <= 227u * 1024u, "inference shared memory");

// 32 consecutive fp32 columns of this thread's TMEM lane (one wait).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Features of one axis (chunks 3 ax .. 3 ax + 2 of a row: frequencies
// 0..11, sin then cos, 8 features a chunk) into the tile (the encoding of
// features()).  sin and cos of pi 2^k q are exact (sincospif) at k = 0 and
// 8 and carried by double-angle steps from there: at most seven steps, an
// absolute error below 2e-5, far under the bf16 rounding the features get.
__device__ __forceinline__ void put_axis_features(char* tile, uint32_t r, uint32_t ax, float qa, bool valid) {
  float s = 0.f, co = 1.f;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    if (m == 1) {  // one more step from frequency 3
      const float s2 = 2.0f * s * co;
      co = (co - s) * (co + s);
      s = s2;
    } else {
      sincospif(ldexpf(qa, 4 * m), &s, &co);
    }
    float f[8];
    f[0] = s;
    f[1] = co;
#pragma unroll
    for (int k = 1; k < 4; ++k) {
      const float s2 = 2.0f * s * co;
      co = (co - s) * (co + s);
      s = s2;
      f[2 * k] = s;
      f[2 * k + 1] = co;
    }
    uint4 w = make_uint4(0, 0, 0, 0);
    if (valid) {
      w.x = pack2(f[0], f[1]);
      w.y = pack2(f[2], f[3]);
      w.z = pack2(f[4], f[5]);
      w.w = pack2(f[6], f[7]);
    }
    *reinterpret_cast<uint4*>(tile + chunk_off(r, 3 * ax + m, 80)) = w;
  }
}
__device__ __forceinline__ void put_chunk(char* tile, uint32_t r, uint32_t c, uint32_t K, const float* v) {
  uint4 w;
  w.x = pack2(v[0], v[1]);
  w.y = pack2(v[2], v[3]);
  w.z = pack2(v[4], v[5]);
  w.w = pack2(v[6], v[7]);
  *reinterpret_cast<uint4*>(tile + chunk_off(r, c, K)) = w;
}

// The forward pass of one tile by one group (features already in its
// tile): false if a wait ran out.  The output layer ends in the group's
// TMEM columns 0..47.
__device__ bool forward_tile_group(char* sm, char* a, GroupShared& gs, uint32_t tmem, uint32_t bid, uint32_t r,
                                   uint32_t& phase) {
  const uint32_t lane_base = (r & ~31u) << 16;
#pragma unroll
  for (int l = 0; l < 5; ++l) {
    fence_async_smem();
    group_sync(bid);
    if (r == 0)
      gemm_issue(tmem, a, sm + (l == 0 ? kSW0 : (l == 1 ? kSW1 : (l == 2 ? kSW2 : (l == 3 ? kSW3 : kSW4)))),
                 l == 0 ? 80u : 64u, l == 4 ? 48u : 64u, &gs.bar);
    const bool ok = bar_wait(&gs.bar, phase);
    phase ^= 1u;
    if (group_any(!ok, bid)) {
      if (r == 0) gs.abort = 1;
      return false;
    }
    fence_after();
    if (l == 4) return true;
    // the MMA has read the tile: the next layer's input goes over it (K = 64)
#pragma unroll
    for (uint32_t hh = 0; hh < 2; ++hh) {
      float h[32];
      tmem_ld32(tmem + lane_base + 32u * hh, h);
#pragma unroll
      for (uint32_t cc = 0; cc < 4; ++cc) {
        const float* v = h + 8 * cc;
        uint4 w;
        w.x = pack2_relu(v[0], v[1]);
        w.y = pack2_relu(v[2], v[3]);
        w.z = pack2_relu(v[4], v[5]);
        w.w = pack2_relu(v[6], v[7]);
        *reinterpret_cast<uint4*>(a + chunk_off(r, 4 * hh + cc, 64)) = w;
      }
    }
    fence_before();
  }
  return true;
}

__global__ void __launch_bounds__(kInferThreads, 1) k_guide_infer(GuideRows in, const __nv_bfloat16* wf, float* out,
                                                                  int* err) {
  extern __shared__ __align__(1024) char sm[];
  GroupShared* gsh = reinterpret_cast<GroupShared*>(sm + kInferCtl);
  uint32_t& tmem_base = *reinterpret_cast<uint32_t*>(sm + kInferSlot);
  const uint32_t g = threadIdx.x / 128u, r = threadIdx.x % 128u;
  const uint32_t bid = 1u + g;
  const uint64_t n = in.n_dev ? *in.n_dev : in.n;
  if (r == 0) {
    bar_init(&gsh[g].bar);
    gsh[g].abort = 0;
  }
  load_tile(sm + kSW0, wf + kWf0, 64, 80);
  load_tile(sm + kSW1, wf + kWf1, 64, 64);
  load_tile(sm + kSW2, wf + kWf2, 64, 64);
  load_tile(sm + kSW3, wf + kWf3, 64, 64);
  load_tile(sm + kSW4, wf + kWf4, 48, 64);
  if (threadIdx.x < 32) tmem_alloc(&tmem_base, kInferTmemCols);
  fence_before();
  __syncthreads();
  fence_after();
  GroupShared& gs = gsh[g];
  char* a = sm + kSWEnd + g * kSAGroup;
  const uint32_t tmem = tmem_base + 64u * g;
  const uint32_t lane_base = (r & ~31u) << 16;
  uint32_t phase = 0;
  const uint64_t ntiles = (n + 127) / 128;
  for (uint64_t t = (uint64_t)blockIdx.x * kGroups + g; t < ntiles; t += (uint64_t)gridDim.x * kGroups) {
    const uint64_t row = t * 128 + r;
    const bool valid = row < n;
    float q[3] = {0.f, 0.f, 0.f}, nn[3] = {0.f, 0.f, 0.f}, wo[3] = {0.f, 0.f, 0.f};
    if (valid) {
      q[0] = (in.px[row] - in.lo[0]) * in.inv_ext[0];
      q[1] = (in.py[row] - in.lo[1]) * in.inv_ext[1];
      q[2] = (in.pz[row] - in.lo[2]) * in.inv_ext[2];
      nn[0] = in.nx[row]; nn[1] = in.ny[row]; nn[2] = in.nz[row];
      wo[0] = in.wx[row]; wo[1] = in.wy[row]; wo[2] = in.wz[row];
    }
#pragma unroll 1
    for (uint32_t ax = 0; ax < 3; ++ax) put_axis_features(a, r, ax, ax == 0 ? q[0] : (ax == 1 ? q[1] : q[2]), valid);
    {
      // chunk 9: normal, direction toward the previous vertex, 1, 0
      const float f[8] = {nn[0], nn[1], nn[2], wo[0], wo[1], wo[2], valid ? 1.0f : 0.0f, 0.0f};
      put_chunk(a, r, 9, 80, f);
    }
    if (!forward_tile_group(sm, a, gs, tmem, bid, r, phase)) break;
    // 44 floats per row (41 outputs; columns 41..43 of the padded layer are 0)
    float4* dst = reinterpret_cast<float4*>(out + (size_t)row * kGuideOutStride);
    {
      float o[32];
      tmem_ld32(tmem + lane_base, o);
      if (valid)
#pragma unroll
        for (int k = 0; k < 8; ++k) dst[k] = make_float4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
    }
    {
      float o[16];
      tmem_ld16(tmem + lane_base + 32u, o);
      if (valid)
#pragma unroll
        for (int k = 0; k < 3; ++k) dst[8 + k] = make_float4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
    }
    fence_before();
  }
  // a group that stopped early waits (bounded) for its MMAs still in flight
  if (gs.abort) (void)bar_wait(&gs.bar, phase ^ 1u);
  __syncthreads();
  if (r == 0 && gs.abort) atomicExch(err, 1);
  if (threadIdx.x < 32) tmem_free(tmem_base, kInferTmemCols);
}

// The saved activations and deltas, per section of R rows starting at
// row0 (X: rows 0..79; h1..h4: 80 + 64 (l - 1); dY: 336, 48 rows; dZ4..dZ1:
// 384 + 64 (4 - l)), are stored chunk-blocked: the 128 records of chunk c
// form one block of R x 128 bf16 laid out [row group (R / 8)][record (128)]
// [row % 8 (8)], a record's 8 consecutive rows in one 16-byte vector (one
// store of the training kernel, consecutive across a warp's records).  The
// block is the no-swizzle MN-major operand layout of a weight-gradient MMA
// whose M (or N) is the section's rows and K the chunk's records: core
// matrices of 8 records x 16 bytes (128 contiguous bytes), the next 8
// records 128 bytes on (LBO), the next 8 rows 2048 bytes on (SBO).  A
// chunk's operand is one contiguous block of 256 R bytes, moved by one bulk
// copy.  The record stride B is a multiple of 128.  save_vec: the element
// index of the vector holding rows 8 g .. 8 g + 7 of record b.
__device__ __forceinline__ size_t save_vec(uint32_t row0, uint32_t R, uint32_t g, uint64_t b, uint32_t B) {
  return (size_t)row0 * B + (size_t)(b >> 7) * (R * 128u) + (g * 128u + ((uint32_t)b & 127u)) * 8u;
}
// 8 fp32 values as 8 bf16 in one 16-byte store.
__device__ __forceinline__ void save8(__nv_bfloat16* save, size_t at, const float* v) {
  uint4 w;
  w.x = pack2(v[0], v[1]);
  w.y = pack2(v[2], v[3]);
  w.z = pack2(v[4], v[5]);
  w.w = pack2(v[6], v[7]);
  *reinterpret_cast<uint4*>(save + at) = w;
}

// Training: forward + loss gradient + backward-data, four tile streams per
// CTA (512 threads in groups of four warps, one CTA per SM) sharing both
// weight copies; each group owns one 128 x 80 tile that holds the current
// layer's input (forward), dY (K = 48) and then each dZ (backward), written
// over the tile once the MMA that read it has completed.  Every layer's
// input and output delta is saved chunk-blocked (save_vec).
constexpr uint32_t kTrainGroups = 4;
constexpr uint32_t kTrainThreads = 128 * kTrainGroups;
constexpr uint32_t kTrainCtl = kSBEnd + kTrainGroups * kSAGroup;
constexpr uint32_t kTrainSlot = kTrainCtl + kTrainGroups * (uint32_t)sizeof(GroupShared);
constexpr uint32_t kTrainSmem = kTrainSlot + 16;
static_assert(kTrainSmem <= 227u * 1024u, "training shared memory");

// One MMA of a group (the tile as A, K-major) and its bounded wait; false if
// the wait ran out (the group agrees; thread 0 marks the abort).
__device__ __forceinline__ bool group_gemm(uint32_t tmem, const char* A, const char* Bm, uint32_t K, uint32_t N,
                                           GroupShared& gs, uint32_t bid, uint32_t r, uint32_t& phase) {
  fence_async_smem();
  group_sync(bid);
  if (r == 0) gemm_issue(tmem, A, Bm, K, N, &gs.bar);
  const bool ok = bar_wait(&gs.bar, phase);
  phase ^= 1u;
  if (group_any(!ok, bid)) {
    if (r == 0) gs.abort = 1;
    return false;
  }
  fence_after();
  return true;
}

__global__ void __launch_bounds__(kTrainThreads, 1) k_guide_train(GuideTrain tr, const __nv_bfloat16* wf,
                                                                  const __nv_bfloat16* wb, __nv_bfloat16* save,
                                                                  float* sums, int* err) {
  extern __shared__ __align__(1024) char sm[];
  GroupShared* gsh = reinterpret_cast<GroupShared*>(sm + kTrainCtl);
  uint32_t& tmem_base = *reinterpret_cast<uint32_t*>(sm + kTrainSlot);
  const uint32_t g = threadIdx.x / 128u, r = threadIdx.x % 128u;
  const uint32_t bid = 1u + g;
  const uint64_t n = tr.rows.n_dev ? *tr.rows.n_dev : tr.rows.n;
  const uint32_t B = tr.stride;
  if (r == 0) {
    bar_init(&gsh[g].bar);
    gsh[g].abort = 0;
  }
  load_tile(sm + kSW0, wf + kWf0, 64, 80);
  load_tile(sm + kSW1, wf + kWf1, 64, 64);
  load_tile(sm + kSW2, wf + kWf2, 64, 64);
  load_tile(sm + kSW3, wf + kWf3, 64, 64);
  load_tile(sm + kSW4, wf + kWf4, 48, 64);
  load_tile(sm + kSB1, wb + kWb1, 64, 64);
  load_tile(sm + kSB2, wb + kWb2, 64, 64);
  load_tile(sm + kSB3, wb + kWb3, 64, 64);
  load_tile(sm + kSB4, wb + kWb4, 64, 48);
  if (threadIdx.x < 32) tmem_alloc(&tmem_base, 64 * kTrainGroups);
  fence_before();
  __syncthreads();
  fence_after();
  GroupShared& gs = gsh[g];
  char* a = sm + kSBEnd + g * kSAGroup;
  const uint32_t tmem = tmem_base + 64u * g;
  const uint32_t lane_base = (r & ~31u) << 16;
  uint32_t phase = 0;
  const uint64_t ntiles = (n + 127) / 128;
  float loss_acc = 0.f, w_acc = 0.f;
  for (uint64_t t = (uint64_t)blockIdx.x * kTrainGroups + g; t < ntiles; t += (uint64_t)gridDim.x * kTrainGroups) {
    const uint64_t row = t * 128 + r;
    const bool valid = row < n;
    float weight = 0.f, om[3] = {0.f, 0.f, 1.f}, pb = -1.0f;
    {
      float f[80];
      if (valid) {
        const GuideRows& in = tr.rows;
        const uint64_t e = row * in.rstride;
        const float p[3] = {in.px[e], in.py[e], in.pz[e]};
        const float nn[3] = {in.nx[e], in.ny[e], in.nz[e]};
        const float wo[3] = {in.wx[e], in.wy[e], in.wz[e]};
        features(p, nn, wo, in.lo, in.inv_ext, f);
        weight = tr.weight[e];
        om[0] = tr.ox[e];
        om[1] = tr.oy[e];
        om[2] = tr.oz[e];
        if (tr.pb) pb = tr.pb[e];
      } else {
        for (int k = 0; k < 80; ++k) f[k] = 0.f;
      }
      // every row of the tile is saved (an invalid row as zeros), so the
      // weight gradient reads whole 128-record chunks
#pragma unroll
      for (int g8 = 0; g8 < 10; ++g8) save8(save, save_vec(0, 80, g8, row, B), f + 8 * g8);
      put_row(a, r, 80, f);
    }
    // forward; mask[l] holds bit j for h_{l+1}[j] > 0 (two words a layer)
    uint32_t mask[8];
    bool ok = true;
#pragma unroll 1
    for (int l = 0; l < 5 && ok; ++l) {
      const uint32_t W = l == 0 ? kSW0 : (l == 1 ? kSW1 : (l == 2 ? kSW2 : (l == 3 ? kSW3 : kSW4)));
      if (!group_gemm(tmem, a, sm + W, l == 0 ? 80u : 64u, l == 4 ? 48u : 64u, gs, bid, r, phase)) {
        ok = false;
        break;
      }
      if (l == 4) break;
      float h[64];
#pragma unroll
      for (int q = 0; q < 4; ++q) tmem_ld16(tmem + lane_base + 16 * q, h + 16 * q);
      uint32_t m0 = 0, m1 = 0;
#pragma unroll
      for (int j = 0; j < 64; ++j) {
        h[j] = h[j] > 0.0f ? h[j] : 0.0f;
        if (h[j] > 0.0f) {
          if (j < 32) m0 |= 1u << j;
          else m1 |= 1u << (j - 32);
        }
      }
      mask[2 * l] = m0;
      mask[2 * l + 1] = m1;
      put_row(a, r, 64, h);
      fence_before();
#pragma unroll
      for (int g8 = 0; g8 < 8; ++g8)  // h_{l+1} for the weight gradient
        save8(save, save_vec(80 + 64 * l, 64, g8, row, B), h + 8 * g8);
    }
    if (!ok) break;
    {
      float o[48], gr[48];
#pragma unroll
      for (int q = 0; q < 3; ++q) tmem_ld16(tmem + lane_base + 16 * q, o + 16 * q);
      for (int k = kGuideOut; k < 48; ++k) gr[k] = 0.f;
      if (valid) {
        float loss;
        out_grad(o, om, weight, pb, tr.amax, gr, loss);
        loss_acc += loss;
        w_acc += weight;
      } else {
        for (int k = 0; k < kGuideOut; ++k) gr[k] = 0.f;
      }
      put_row(a, r, 48, gr);  // dY, K = 48
      fence_before();
#pragma unroll
      for (int g8 = 0; g8 < 6; ++g8) save8(save, save_vec(336, 48, g8, row, B), gr + 8 * g8);
    }
    // dH_l = dZ_{l+1} * W_l, masked by h_l > 0, for l = 4 .. 1
#pragma unroll 1
    for (int l = 4; l >= 1; --l) {
      const uint32_t Bt = l == 1 ? kSB1 : (l == 2 ? kSB2 : (l == 3 ? kSB3 : kSB4));
      if (!group_gemm(tmem, a, sm + Bt, l == 4 ? 48u : 64u, 64u, gs, bid, r, phase)) {
        ok = false;
        break;
      }
      float d[64];
#pragma unroll
      for (int q = 0; q < 4; ++q) tmem_ld16(tmem + lane_base + 16 * q, d + 16 * q);
      const uint32_t m0 = mask[2 * (l - 1)], m1 = mask[2 * (l - 1) + 1];
#pragma unroll
      for (int j = 0; j < 64; ++j) {
        const bool on = j < 32 ? ((m0 >> j) & 1u) : ((m1 >> (j - 32)) & 1u);
        d[j] = on ? d[j] : 0.f;
      }
      put_row(a, r, 64, d);
      fence_before();
#pragma unroll
      for (int g8 = 0; g8 < 8; ++g8) save8(save, save_vec(384 + 64 * (4 - l), 64, g8, row, B), d + 8 * g8);
    }
    if (!ok) break;
  }
  // batch sums: loss, weight
#pragma unroll
  for (int o2 = 16; o2 > 0; o2 >>= 1) {
    loss_acc += __shfl_down_sync(0xffffffffu, loss_acc, o2);
    w_acc += __shfl_down_sync(0xffffffffu, w_acc, o2);
  }
  if ((r & 31) == 0) {
    atomicAdd(&sums[0], loss_acc);
    atomicAdd(&sums[1], w_acc);
  }
  // a group that stopped early waits (bounded) for its MMAs still in flight
  if (gs.abort) (void)bar_wait(&gs.bar, phase ^ 1u);
  __syncthreads();
  if (r == 0 && gs.abort) atomicExch(err, 1);
  if (threadIdx.x < 32) tmem_free(tmem_base, 64 * kTrainGroups);
}

// Weight gradients: for layer l, D [64 x N] += A [64 x 128] * B [N x 128]^T
// over chunks of 128 records (M = 64: the layer's output deltas, the last
// layer's 48 saved dY rows read as 64 with rows 48..63 unused; N = the
// layer's 80 or 64 inputs; K = the chunk's records).  Each operand of a
// chunk is one contiguous block of the chunk-blocked save, fetched by one
// bulk async copy (cp.async.bulk, completion counted on the stage's
// mbarrier) into one of kWgStages stages; one thread issues the copies
// kWgStages chunks ahead and the MMAs, whose commit frees the stage.
// blockIdx.y = layer, blockIdx.x strides the chunks; the CTA's sum goes to
// the float32 gradient with atomics.  The M = 64 accumulator sits in TMEM
// lanes 0-15 of each 32-lane quarter (row 16q + j in lane 32q + j).
constexpr uint32_t kWgStages = 3;
constexpr uint32_t kWgStage = 64 * 128 * 2 + 80 * 128 * 2;  // A + B of one stage: 36864
constexpr uint32_t kWgCtl = kWgStages * kWgStage;
constexpr uint32_t kWgradSmem = kWgCtl + 2 * kWgStages * 8 + 16;

__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   saddr(dst)),
               "l"(src), "r"(bytes), "r"(saddr(bar))
               : "memory");
}
__device__ __forceinline__ void bar_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}

__global__ void __launch_bounds__(128) k_guide_wgrad(const __nv_bfloat16* save, uint32_t B, uint64_t n,
                                                     const unsigned long long* n_dev, float* grad, int* err) {
  extern __shared__ __align__(1024) char sm[];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + kWgCtl);
  uint64_t* empty = full + kWgStages;
  const uint32_t r = threadIdx.x;
  if (n_dev) n = *n_dev < n ? *n_dev : n;
  const int l = blockIdx.y;
  // layer l: output deltas (A, RA rows saved, 64 read) and inputs (B, N rows)
  const uint32_t RA = l == 4 ? 48u : 64u;
  const uint32_t N = l == 0 ? 80u : 64u;
  const uint32_t a_row0 = l == 4 ? 336u : 384u + 64u * (3u - (uint32_t)l);
  const uint32_t b_row0 = l == 0 ? 0u : 80u + 64u * (uint32_t)(l - 1);
  const uint32_t Mr = l == 4 ? (uint32_t)kGuideOut : 64u;
  const uint32_t goff = l == 0 ? 0u : (l == 4 ? 17408u : 5120u + 4096u * (uint32_t)(l - 1));
  const uint32_t a_bytes = RA * 256u, b_bytes = N * 256u;
  if (r == 0) {
    for (uint32_t st = 0; st < kWgStages; ++st) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(full + st)) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(empty + st)) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  // the A region of every stage is 64 rows: rows RA..63 of a 48-row block
  // read the stage's other bytes, which only reach D rows >= 48 (unused)
  for (uint32_t i = r; i < kWgStages * kWgStage / 16; i += 128) reinterpret_cast<uint4*>(sm)[i] = make_uint4(0, 0, 0, 0);
  fence_async_smem();
  if (r < 32) tmem_alloc(&tmem_slot, 128);
  fence_before();
  __syncthreads();
  fence_after();
  const uint64_t nchunks = (n + 127) / 128;
  const uint64_t first = blockIdx.x, step = gridDim.x;
  const uint64_t nloc = first < nchunks ? (nchunks - first + step - 1) / step : 0;
  const __nv_bfloat16* a_src = save + (size_t)a_row0 * B;
  const __nv_bfloat16* b_src = save + (size_t)b_row0 * B;
  uint64_t issued = 0, done_mma = 0;
  if (r == 0 && nloc > 0) {
    auto issue = [&](uint64_t i) {
      const uint32_t st = (uint32_t)(i % kWgStages);
      const uint64_t c = first + i * step;
      char* A = sm + st * kWgStage;
      char* Bt = A + 64 * 128 * 2;
      bar_expect(full + st, a_bytes + b_bytes);
      bulk_copy(A, a_src + (size_t)c * (RA * 128u), a_bytes, full + st);
      bulk_copy(Bt, b_src + (size_t)c * (N * 128u), b_bytes, full + st);
    };
    for (; issued < nloc && issued < kWgStages; ++issued) issue(issued);
    const uint32_t id = idesc(64, (int)N) | (1u << 15) | (1u << 16);  // A and B MN-major
    for (uint64_t i = 0; i < nloc; ++i) {
      const uint32_t st = (uint32_t)(i % kWgStages);
      const uint32_t par = (uint32_t)((i / kWgStages) & 1u);
      if (!bar_wait(full + st, par)) {
        abort_flag = 1;
        break;
      }
      fence_after();
      const uint32_t a0 = saddr(sm + st * kWgStage), bb = a0 + 64 * 128 * 2;
      for (uint32_t kk = 0; kk < 8; ++kk)  // K = 16: records 16 kk .. 16 kk + 15
        mma(tmem_slot, sdesc(a0 + kk * 256u, 128u, 2048u), sdesc(bb + kk * 256u, 128u, 2048u), id,
            (i > 0 || kk > 0) ? 1u : 0u);
      mma_commit(empty + st);
      done_mma = i + 1;
      if (issued < nloc) {  // refill this stage once its MMAs have read it
        if (!bar_wait(empty + st, par)) {
          abort_flag = 1;
          break;
        }
        issue(issued);
        ++issued;
      }
    }
    // the last commit of each stage still pending: wait for the final one
    if (!abort_flag && done_mma > 0) {
      const uint64_t i = done_mma - 1;
      if (!bar_wait(empty + (uint32_t)(i % kWgStages), (uint32_t)((i / kWgStages) & 1u))) abort_flag = 1;
    }
    if (abort_flag) {
      // bounded waits for the copies and MMAs still in flight
      for (uint64_t i = done_mma; i < issued; ++i)
        (void)bar_wait(full + (uint32_t)(i % kWgStages), (uint32_t)((i / kWgStages) & 1u));
      if (done_mma > 0) {
        const uint64_t i = done_mma - 1;
        (void)bar_wait(empty + (uint32_t)(i % kWgStages), (uint32_t)((i / kWgStages) & 1u));
      }
    }
  }
  __syncthreads();
  if (!abort_flag && nloc > 0) {
    fence_after();
    // every warp loads its lane quarter (warp-collective); row 16q + j is in
    // lane 32q + j for j < 16
    const uint32_t q = r >> 5, j = r & 31u;
    const uint32_t lane_base = (q * 32u) << 16;
    const uint32_t row = 16u * q + j;
    for (uint32_t c16 = 0; c16 < N / 16; ++c16) {
      float v[16];
      tmem_ld16(tmem_slot + lane_base + 16 * c16, v);
      if (j < 16 && row < Mr)
        for (int e = 0; e < 16; ++e) atomicAdd(&grad[goff + row * N + 16 * c16 + e], v[e]);
    }
  }
  fence_before();
  __syncthreads();
  if (abort_flag && r == 0) atomicExch(err, 1);
  if (r < 32) tmem_free(tmem_slot, 128);
}

// Adam on the float32 masters (gradient divided by the batch's weight sum),
// then the bf16 forward and transposed copies.  One thread per weight.
__global__ void k_guide_adam(float* W, float* m, float* v, float* grad, const float* sums, GuideAdam a,
                             __nv_bfloat16* wf, __nv_bfloat16* wb) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kGuideWeights) return;
  if (a.step > 0) {
    const float scale = sums[1] > 0.f ? 1.f / sums[1] : 0.f;
    const float g = grad[i] * scale;
    const float mi = a.beta1 * m[i] + (1.f - a.beta1) * g;
    const float vi = a.beta2 * v[i] + (1.f - a.beta2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.f - powf(a.beta1, (float)a.step));
    const float vh = vi / (1.f - powf(a.beta2, (float)a.step));
    W[i] -= a.lr * mh / (sqrtf(vh) + a.eps);
    grad[i] = 0.f;
  }
  const float w = W[i];
  const __nv_bfloat16 h = __float2bfloat16_rn(w);
  // forward copy: same row-major index except W4 rows sit in a 48-row block
  wf[i] = h;
  if (i >= 5120u) {
    uint32_t l, o, j;
    if (i < 17408u) {
      l = 1 + (i - 5120u) / 4096u;
      const uint32_t k = (i - 5120u) % 4096u;
      o = k / 64;
      j = k % 64;
      wb[(l - 1) * 4096u + j * 64 + o] = h;  // W_l^T [in][out]
    } else {
      const uint32_t k = i - 17408u;
      o = k / 64;
      j = k % 64;
      wb[kWb4 + j * 48 + o] = h;  // W4^T [64][48]
    }
  }
}

}  // namespace

void prepare_kernels() {
  cudaFuncSetAttribute(k_guide_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem2);
  cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem);
  cudaFuncSetAttribute(k_guide_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWgradSmem);
}

// The failure path of the bounded waits, exercised on purpose: one block
// waits with bar_wait on an mbarrier that nothing arrives at; the wait runs
// out after its bound (2^22 polls), the block agrees on the outcome and
// thread 0 sets the error word, as the guide kernels do before returning.
// No tensor memory is held.
__global__ void k_wait_selftest(int* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) bar_init(&bar);
  __syncthreads();
  const bool ok = bar_wait(&bar, 0u);
  if (__syncthreads_or(ok ? 0 : 1) && threadIdx.x == 0) atomicExch(err, 1);
}

// One CTA per SM at most (it holds all of the SM's tensor memory): sms = the
// device's SM count; fewer CTAs when the host knows the row count.
int launch_infer(const GuideRows& rows, const void* wf, float* out, int* err, int sms, cudaStream_t st) {
  uint64_t grid = (uint64_t)(sms > 0 ? sms : 1);
  if (!rows.n_dev) grid = std::min<uint64_t>(grid, std::max<uint64_t>(1, (rows.n + 128 * kGroups - 1) / (128 * kGroups)));
  k_guide_infer<<<(int)grid, kInferThreads, kInferSmem2, st>>>(rows, static_cast<const __nv_bfloat16*>(wf), out, err);
  return (int)cudaGetLastError();
}

// One CTA per SM at most; sms = the device's SM count (fewer CTAs for a
// small batch: rows.n bounds the device count too).
int launch_train(const GuideTrain& tr, const void* wf, const void* wb, void* save, float* sums, int* err, int sms,
                 cudaStream_t st) {
  const uint64_t per_cta = 128ull * kTrainGroups;
  const int grid = (int)std::min<uint64_t>((uint64_t)(sms > 0 ? sms : 1),
                                           std::max<uint64_t>(1, (tr.rows.n + per_cta - 1) / per_cta));
  k_guide_train<<<grid, kTrainThreads, kTrainSmem, st>>>(tr, static_cast<const __nv_bfloat16*>(wf),
                                                static_cast<const __nv_bfloat16*>(wb),
                                                static_cast<__nv_bfloat16*>(save), sums, err);
  return (int)cudaGetLastError();
}

// Two CTAs per SM (110 KB of stages each) over the five layers: about
// 2 * sms / 5 CTAs per layer, fewer for a small batch (n bounds the device
// count too).
int launch_wgrad(const void* save, uint32_t B, uint64_t n, const unsigned long long* n_dev, float* grad, int* err,
                 int sms, cudaStream_t st) {
  const uint64_t per_layer = std::max<uint64_t>(1, (uint64_t)(sms > 0 ? sms : 1) * 2 / 5);
  const uint64_t chunks = std::max<uint64_t>(1, std::min<uint64_t>(per_layer, (n + 127) / 128));
  dim3 g((unsigned)chunks, 5);
  k_guide_wgrad<<<g, 128, kWgradSmem, st>>>(static_cast<const __nv_bfloat16*>(save), B, n, n_dev, grad, err);
  return (int)cudaGetLastError();
}

int launch_adam(float* W, float* m, float* v, float* grad, const float* sums, const GuideAdam& a, void* wf, void* wb,
                cudaStream_t st) {
  k_guide_adam<<<(kGuideWeights + 255) / 256, 256, 0, st>>>(W, m, v, grad, sums, a, static_cast<__nv_bfloat16*>(wf),
                                                           static_cast<__nv_bfloat16*>(wb));
  return (int)cudaGetLastError();
}

int ensure_ready(vmr_ctx* ctx) {
  if (ctx->guide.ready) return VMR_OK;
  return vmr_guide_init(ctx, 0);
}

size_t wf_elems() { return kWfSize; }
size_t wb_elems() { return kWbSize; }

}  // namespace guide
}  // namespace vmr

// ------------------------------------------------------------------- C ABI ---
namespace {

int gfail(vmr_ctx* ctx, int code, const std::string& msg) {
  ctx->err = msg;
  return code;
}
#define GCUDA(x)                                                               \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess) return gfail(ctx, VMR_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

using vmr::guide::GuideAdam;
using vmr::guide::GuideRows;
using vmr::guide::GuideTrain;
using vmr::guide::kGuideOut;
using vmr::guide::kGuideOutStride;
using vmr::guide::kGuideWeights;

int guide_alloc(vmr_ctx* ctx) {
  auto& G = ctx->guide;
  if (G.ready) return VMR_OK;
  vmr::guide::prepare_kernels();
  const size_t nw = kGuideWeights * sizeof(float);
  GCUDA(G.W.ensure(nw));
  GCUDA(G.m.ensure(nw));
  GCUDA(G.v.ensure(nw));
  GCUDA(G.grad.ensure(nw));
  GCUDA(G.wf.ensure(vmr::guide::wf_elems() * 2));
  GCUDA(G.wb.ensure(vmr::guide::wb_elems() * 2));
  GCUDA(G.sums.ensure(16));
  GCUDA(G.err.ensure(16));
  GCUDA(cudaMemsetAsync(G.wf.p, 0, vmr::guide::wf_elems() * 2, ctx->stream));
  GCUDA(cudaMemsetAsync(G.wb.p, 0, vmr::guide::wb_elems() * 2, ctx->stream));
  GCUDA(cudaMemsetAsync(G.err.p, 0, 16, ctx->stream));
  G.ready = true;
  return VMR_OK;
}

int guide_upload(vmr_ctx* ctx, const float* w) {
  auto& G = ctx->guide;
  const size_t nw = kGuideWeights * sizeof(float);
  GCUDA(cudaMemcpyAsync(G.W.p, w, nw, cudaMemcpyHostToDevice, ctx->stream));
  GCUDA(cudaMemsetAsync(G.m.p, 0, nw, ctx->stream));
  GCUDA(cudaMemsetAsync(G.v.p, 0, nw, ctx->stream));
  GCUDA(cudaMemsetAsync(G.grad.p, 0, nw, ctx->stream));
  G.step = 0;
  GuideAdam a{0.f, 0.f, 0.f, 0.f, 0};
  if (vmr::guide::launch_adam(G.W.as<float>(), G.m.as<float>(), G.v.as<float>(), G.grad.as<float>(),
                              G.sums.as<float>(), a, G.wf.p, G.wb.p, ctx->stream) != 0)
    return gfail(ctx, VMR_ERR_CUDA, "guide weight refresh failed");
  return VMR_OK;
}

int guide_check(vmr_ctx* ctx) {
  if (!ctx) return VMR_ERR_INVALID;
  if (ctx->device < 0) return gfail(ctx, VMR_ERR_UNSUPPORTED, "host-only context has no guide");
  if (!ctx->guide.ready) return gfail(ctx, VMR_ERR_INVALID, "guide has no weights: call vmr_guide_init first");
  return VMR_OK;
}

// Host n x 3 arrays -> device SoA rows in the context's staging buffer
// (omega, weight and pb optional), followed by extra_out floats of room.
int stage_rows(vmr_ctx* ctx, const float* pos, const float* nrm, const float* wo, const float* omega,
               const float* weight, const float* pb, size_t n, const float lo[3], const float hi[3], GuideTrain& tr,
               size_t extra_out) {
  auto& G = ctx->guide;
  const size_t cols = 9 + (omega ? 3 : 0) + (weight ? 1 : 0) + (pb ? 1 : 0);
  GCUDA(G.io.ensure((cols * n + extra_out) * sizeof(float) + 256));
  std::vector<float> h(cols * n);
  for (size_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      h[c * n + i] = pos[3 * i + c];
      h[(3 + c) * n + i] = nrm[3 * i + c];
      h[(6 + c) * n + i] = wo[3 * i + c];
      if (omega) h[(9 + c) * n + i] = omega[3 * i + c];
    }
  size_t col = omega ? 12 : 9;
  const size_t wcol = col;
  if (weight) {
    for (size_t i = 0; i < n; ++i) h[col * n + i] = weight[i];
    ++col;
  }
  const size_t pcol = col;
  if (pb)
    for (size_t i = 0; i < n; ++i) h[col * n + i] = pb[i];
  float* d = G.io.as<float>();
  GCUDA(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  GCUDA(cudaStreamSynchronize(ctx->stream));  // h goes out of scope
  GuideRows& r = tr.rows;
  r.px = d; r.py = d + n; r.pz = d + 2 * n;
  r.nx = d + 3 * n; r.ny = d + 4 * n; r.nz = d + 5 * n;
  r.wx = d + 6 * n; r.wy = d + 7 * n; r.wz = d + 8 * n;
  r.n = n;
  r.n_dev = nullptr;
  for (int c = 0; c < 3; ++c) {
    r.lo[c] = lo[c];
    r.inv_ext[c] = 1.0f / (hi[c] - lo[c]);
  }
  if (omega) {
    tr.ox = d + 9 * n; tr.oy = d + 10 * n; tr.oz = d + 11 * n;
  }
  if (weight) tr.weight = d + wcol * n;
  tr.pb = pb ? d + pcol * n : nullptr;
  tr.stride = (uint32_t)n;
  return VMR_OK;
}

int guide_sms(vmr_ctx* ctx) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  return sms > 0 ? sms : 1;
}

// Forward + backward over n staged records into G.grad (summed); loss sum
// and weight sum in G.sums.  The save buffer's row stride is n rounded up to
// 128, so every 8-value chunk the weight-gradient kernel loads is 16-byte
// aligned.
int guide_backprop(vmr_ctx* ctx, const GuideTrain& tr, size_t n) {
  auto& G = ctx->guide;
  const size_t stride = (n + 127) / 128 * 128;
  if (G.save_rows < stride) {
    GCUDA(G.save.ensure((size_t)vmr::guide::kSaveRows * stride * 2));
    G.save_rows = (uint32_t)stride;
  }
  GuideTrain t = tr;
  t.stride = (uint32_t)stride;
  GCUDA(cudaMemsetAsync(G.sums.p, 0, 16, ctx->stream));
  const int sms = guide_sms(ctx);
  if (vmr::guide::launch_train(t, G.wf.p, G.wb.p, G.save.p, G.sums.as<float>(), G.err.as<int>(), sms,
                               ctx->stream) != 0)
    return gfail(ctx, VMR_ERR_CUDA, "guide training kernel launch failed");
  if (vmr::guide::launch_wgrad(G.save.p, (uint32_t)stride, n, nullptr, G.grad.as<float>(), G.err.as<int>(), sms,
                               ctx->stream) != 0)
    return gfail(ctx, VMR_ERR_CUDA, "guide weight-gradient kernel launch failed");
  return VMR_OK;
}

int guide_status(vmr_ctx* ctx) {
  int e = 0;
  GCUDA(cudaMemcpyAsync(&e, ctx->guide.err.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
  GCUDA(cudaStreamSynchronize(ctx->stream));
  if (e) {
    cudaMemsetAsync(ctx->guide.err.p, 0, 4, ctx->stream);
    return gfail(ctx, VMR_ERR_TIMEOUT, "a guide kernel's tensor-core wait ran out");
  }
  return VMR_OK;
}

uint64_t smix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

extern "C" {

int vmr_selftest_wait(vmr_ctx* ctx, float* ms) {
  if (!ctx) return VMR_ERR_INVALID;
  if (ctx->device < 0) return gfail(ctx, VMR_ERR_UNSUPPORTED, "host-only context");
  cudaSetDevice(ctx->device);
  int rc = guide_alloc(ctx);
  if (rc) return rc;
  cudaStream_t st = ctx->stream;
  GCUDA(cudaMemsetAsync(ctx->guide.err.p, 0, 4, st));
  GCUDA(cudaEventRecord(ctx->ev0, st));
  vmr::guide::k_wait_selftest<<<1, 64, 0, st>>>(ctx->guide.err.as<int>());
  GCUDA(cudaGetLastError());
  GCUDA(cudaEventRecord(ctx->ev1, st));
  int err = 0;
  GCUDA(cudaMemcpyAsync(&err, ctx->guide.err.p, 4, cudaMemcpyDeviceToHost, st));
  GCUDA(cudaStreamSynchronize(st));
  GCUDA(cudaMemsetAsync(ctx->guide.err.p, 0, 4, st));
  float t = 0.f;
  cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1);
  if (ms) *ms = t;
  return err ? VMR_ERR_TIMEOUT : VMR_OK;
}

int vmr_guide_init(vmr_ctx* ctx, uint64_t seed) {
  if (!ctx) return VMR_ERR_INVALID;
  if (ctx->device < 0) return gfail(ctx, VMR_ERR_UNSUPPORTED, "host-only context has no guide");
  cudaSetDevice(ctx->device);
  int rc = guide_alloc(ctx);
  if (rc) return rc;
  std::vector<float> w(kGuideWeights);
  const int off[6] = {0, 5120, 9216, 13312, 17408, kGuideWeights};
  const int kin[5] = {80, 64, 64, 64, 64};
  for (int l = 0; l < 5; ++l) {
    const float bound = std::sqrt(6.0f / (float)kin[l]) * (l == 4 ? 0.1f : 1.0f);
    for (int i = off[l]; i < off[l + 1]; ++i) {
      const double u = (double)(smix(seed * 0x9E3779B97F4A7C15ull + (uint64_t)i + 1) >> 11) * (1.0 / 9007199254740992.0);
      // First layer: the weights of encoding frequency 2^k start scaled by
      // 0.7^k, so the untrained network varies smoothly over the scene and
      // the high frequencies grow only where the data ask for them.
      const int col = (i - off[l]) % 80;
      const double damp = (l == 0 && col < 72) ? std::pow(0.7, (double)((col % 24) / 2)) : 1.0;
      w[i] = (float)((2.0 * u - 1.0) * bound * damp);
    }
  }
  rc = guide_upload(ctx, w.data());
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? VMR_OK : gfail(ctx, VMR_ERR_CUDA, cudaGetErrorString(e));
}

int vmr_guide_set_weights(vmr_ctx* ctx, const float* weights) {
  if (!ctx || !weights) return VMR_ERR_INVALID;
  if (ctx->device < 0) return gfail(ctx, VMR_ERR_UNSUPPORTED, "host-only context has no guide");
  cudaSetDevice(ctx->device);
  int rc = guide_alloc(ctx);
  if (rc) return rc;
  rc = guide_upload(ctx, weights);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? VMR_OK : gfail(ctx, VMR_ERR_CUDA, cudaGetErrorString(e));
}

int vmr_guide_get_weights(vmr_ctx* ctx, float* weights) {
  if (!weights) return VMR_ERR_INVALID;
  int rc = guide_check(ctx);
  if (rc) return rc;
  GCUDA(cudaMemcpyAsync(weights, ctx->guide.W.p, kGuideWeights * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  GCUDA(cudaStreamSynchronize(ctx->stream));
  return VMR_OK;
}

int vmr_guide_forward(vmr_ctx* ctx, const float* pos, const float* nrm, const float* wo, size_t n, const float lo[3],
                      const float hi[3], float* out) {
  int rc = guide_check(ctx);
  if (rc) return rc;
  if (!pos || !nrm || !wo || !lo || !hi || !out) return gfail(ctx, VMR_ERR_INVALID, "null argument");
  if (n == 0) return VMR_OK;
  cudaSetDevice(ctx->device);
  GuideTrain tr{};
  // the outputs follow the 9 input columns: 9n floats, a multiple of 16 bytes
  // when the row count is (padded below)
  const size_t n4 = (n + 3) / 4 * 4;
  rc = stage_rows(ctx, pos, nrm, wo, nullptr, nullptr, nullptr, n, lo, hi, tr, 9 * (n4 - n) + n * kGuideOutStride);
  if (rc) return rc;
  float* dout = ctx->guide.io.as<float>() + 9 * n4;
  if (vmr::guide::launch_infer(tr.rows, ctx->guide.wf.p, dout, ctx->guide.err.as<int>(), guide_sms(ctx), ctx->stream) !=
      0)
    return gfail(ctx, VMR_ERR_CUDA, "guide inference launch failed");
  std::vector<float> h(n * kGuideOutStride);
  GCUDA(cudaMemcpyAsync(h.data(), dout, h.size() * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  rc = guide_status(ctx);  // synchronises
  if (rc) return rc;
  for (size_t i = 0; i < n; ++i)
    std::memcpy(out + i * kGuideOut, h.data() + i * kGuideOutStride, kGuideOut * sizeof(float));
  return VMR_OK;
}

int vmr_guide_gradient(vmr_ctx* ctx, const float* pos, const float* nrm, const float* wo, const float* omega,
                       const float* weight, const float* bsdf_pdf, float alpha_max, size_t n, const float lo[3],
                       const float hi[3], float* grad, float* loss) {
  int rc = guide_check(ctx);
  if (rc) return rc;
  if (!pos || !nrm || !wo || !omega || !weight || !lo || !hi || !grad) return gfail(ctx, VMR_ERR_INVALID, "null argument");
  if (n == 0 || n > (1u << 24)) return gfail(ctx, VMR_ERR_INVALID, "n must be in [1, 2^24]");
  cudaSetDevice(ctx->device);
  GuideTrain tr{};
  if (bsdf_pdf && !(alpha_max > 0.0f && alpha_max < 1.0f))
    return gfail(ctx, VMR_ERR_INVALID, "alpha_max must be in (0, 1)");
  rc = stage_rows(ctx, pos, nrm, wo, omega, weight, bsdf_pdf, n, lo, hi, tr, 0);
  tr.amax = alpha_max;
  if (rc) return rc;
  GCUDA(cudaMemsetAsync(ctx->guide.grad.p, 0, kGuideWeights * sizeof(float), ctx->stream));
  rc = guide_backprop(ctx, tr, n);
  if (rc) return rc;
  float sums[2];
  GCUDA(cudaMemcpyAsync(grad, ctx->guide.grad.p, kGuideWeights * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  GCUDA(cudaMemcpyAsync(sums, ctx->guide.sums.p, 8, cudaMemcpyDeviceToHost, ctx->stream));
  GCUDA(cudaMemsetAsync(ctx->guide.grad.p, 0, kGuideWeights * sizeof(float), ctx->stream));
  rc = guide_status(ctx);
  if (rc) return rc;
  if (loss) *loss = sums[0];
  return VMR_OK;
}

int vmr_guide_train_step(vmr_ctx* ctx, const float* pos, const float* nrm, const float* wo, const float* omega,
                         const float* weight, const float* bsdf_pdf, float alpha_max, size_t n, const float lo[3],
                         const float hi[3], const vmr_adam* opt, float* loss) {
  int rc = guide_check(ctx);
  if (rc) return rc;
  if (!pos || !nrm || !wo || !omega || !weight || !lo || !hi || !opt) return gfail(ctx, VMR_ERR_INVALID, "null argument");
  if (n == 0 || n > (1u << 24)) return gfail(ctx, VMR_ERR_INVALID, "n must be in [1, 2^24]");
  cudaSetDevice(ctx->device);
  GuideTrain tr{};
  if (bsdf_pdf && !(alpha_max > 0.0f && alpha_max < 1.0f))
    return gfail(ctx, VMR_ERR_INVALID, "alpha_max must be in (0, 1)");
  rc = stage_rows(ctx, pos, nrm, wo, omega, weight, bsdf_pdf, n, lo, hi, tr, 0);
  tr.amax = alpha_max;
  if (rc) return rc;
  rc = guide_backprop(ctx, tr, n);
  if (rc) return rc;
  auto& G = ctx->guide;
  GuideAdam a{opt->lr, opt->beta1, opt->beta2, opt->eps, ++G.step};
  if (vmr::guide::launch_adam(G.W.as<float>(), G.m.as<float>(), G.v.as<float>(), G.grad.as<float>(),
                              G.sums.as<float>(), a, G.wf.p, G.wb.p, ctx->stream) != 0)
    return gfail(ctx, VMR_ERR_CUDA, "guide Adam launch failed");
  float sums[2];
  GCUDA(cudaMemcpyAsync(sums, G.sums.p, 8, cudaMemcpyDeviceToHost, ctx->stream));
  rc = guide_status(ctx);
  if (rc) return rc;
  if (loss) *loss = sums[0];
  return VMR_OK;
}

}  // extern "C"
