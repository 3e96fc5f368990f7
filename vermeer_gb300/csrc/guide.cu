// guide.cu - the path-guiding network on the 5th-generation tensor cores.
//
// No reference counterpart.  The network (80 inputs, 4 hidden ReLU layers
// of 64, 41 outputs = 8 vMF lobes and the selection logit; no biases, input
// 78 is the constant 1)
// runs fused per tile of 128 rows: a group of 128 threads works on a tile
// with the bf16 weights in shared memory (inference: two groups per CTA
// share one copy), thread r owns row r, and each layer is
//   A (128 x K activations, smem) * B (N x K weights, smem) -> D (TMEM, fp32)
// issued as K/16 tcgen05.mma (kind::f16, bf16 inputs, fp32 accumulate) by
// one thread and committed to an mbarrier; every thread then reads its row of
// D with tcgen05.ld, applies ReLU, rounds to bf16 and writes the next layer's
// A tile.  Operands use the no-swizzle K-major canonical layout: 8-row x
// 16-byte core matrices of 128 contiguous bytes, LBO = 128 (next core matrix
// along K), SBO = (K/8)*128 (next 8-row group).
//
//   k_guide_infer   forward for path vertices (features computed in-kernel)
//   k_guide_train   forward, loss gradient at the outputs, backward-data
//                   (dH = dZ * W through transposed weight copies), storing
//                   every layer's input and output delta feature-major
//   k_guide_wgrad   weight gradients dW_l = dZ_{l+1}^T H_l as a tensor-core
//                   GEMM whose K dimension is the batch (M padded to 128)
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
struct Shared {
  uint64_t bar;
  uint32_t tmem;
  int abort;
};

// Every thread waits for the commit; the outcome is agreed by a block vote so
// that all threads leave together (the loads that follow are warp-collective).
__device__ __forceinline__ bool wait_all(Shared& sh, uint32_t& phase) {
  const bool ok = bar_wait(&sh.bar, phase);
  phase ^= 1u;
  if (__syncthreads_or(ok ? 0 : 1)) {
    if (threadIdx.x == 0) sh.abort = 1;
    return false;
  }
  return true;
}

// After an abort: a second bounded wait for the MMAs still in flight, so
// that the tensor memory they write is not freed under them.
__device__ __forceinline__ void drain(Shared& sh, uint32_t phase) {
  if (sh.abort) (void)bar_wait(&sh.bar, phase ^ 1u);
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

// 64 consecutive fp32 columns of this thread's TMEM lane: both 32-column
// loads are issued before the one wait (a single asm statement, so no use of
// the registers can be scheduled before the wait).
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float* v) {
  uint32_t r[64];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%64];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%65];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr), "r"(taddr + 32u)
      : "memory");
#pragma unroll
  for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}
// 48 columns (the output layer): a 32- and a 16-column load, one wait.
__device__ __forceinline__ void tmem_ld48(uint32_t taddr, float* v) {
  uint32_t r[48];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%48];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47}, [%49];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47])
      : "r"(taddr), "r"(taddr + 32u)
      : "memory");
#pragma unroll
  for (int i = 0; i < 48; ++i) v[i] = __uint_as_float(r[i]);
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

// Shared-memory plan (bytes; all tiles 1024-aligned).
constexpr uint32_t kSW0 = 0, kSW1 = kSW0 + 64 * 80 * 2, kSW2 = kSW1 + 8192, kSW3 = kSW2 + 8192, kSW4 = kSW3 + 8192,
                   kSWEnd = kSW4 + 48 * 64 * 2;  // 40960
constexpr uint32_t kSA0 = kSWEnd, kSA1 = kSA0 + 128 * 80 * 2, kSAEnd = kSA1 + 128 * 64 * 2;  // 77824
constexpr uint32_t kSB1 = kSAEnd, kSB2 = kSB1 + 8192, kSB3 = kSB2 + 8192, kSB4 = kSB3 + 8192,
                   kSBEnd = kSB4 + 64 * 48 * 2;  // 108544
constexpr uint32_t kTrainSmem = kSBEnd + 64;

constexpr int kLobes = 8;

// Input features of a vertex (the encoding the oracle's guide_features
// restates).  sin and cos of pi 2^k q are evaluated exactly (sincospif) at
// k = 0, 4, 8 and carried to the next three frequencies by the double-angle
// identities sin 2x = 2 sin x cos x, cos 2x = (cos x - sin x)(cos x + sin x):
// nine calls instead of 36 per row, with an absolute error below 1e-6 after
// three doublings, far under the bf16 rounding the features then get.
__device__ void features(const float* p, const float* n, const float* wo, const float* lo, const float* inv_ext,
                         float* f) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float q = (p[c] - lo[c]) * inv_ext[c];
#pragma unroll
    for (int a = 0; a < 12; a += 4) {
      float s, co;
      sincospif(ldexpf(q, a), &s, &co);
      f[24 * c + 2 * a] = s;
      f[24 * c + 2 * a + 1] = co;
#pragma unroll
      for (int k = a + 1; k < a + 4; ++k) {
        const float s2 = 2.0f * s * co;
        co = (co - s) * (co + s);
        s = s2;
        f[24 * c + 2 * k] = s;
        f[24 * c + 2 * k + 1] = co;
      }
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

// The forward pass of one tile; the caller has written the input features
// into A0.  Returns false if a wait ran out.  On return the output layer
// (48 columns, 41 used) is in TMEM columns 0..47; mask[l] holds bit j for
// h_{l+1}[j] > 0 (l = 0..3, two words each).
__device__ bool forward_tile(char* sm, Shared& sh, uint32_t& phase, uint32_t* mask, bool keep_mask,
                             __nv_bfloat16* save_h, uint32_t save_stride, uint32_t row_global, bool row_valid) {
  const uint32_t r = threadIdx.x;
  const uint32_t lane_base = (r & ~31u) << 16;
  const uint32_t Ks[5] = {80, 64, 64, 64, 64};
  const uint32_t Ns[5] = {64, 64, 64, 64, 48};
  const uint32_t Ws[5] = {kSW0, kSW1, kSW2, kSW3, kSW4};
  for (int l = 0; l < 5; ++l) {
    const char* A = sm + ((l & 1) ? kSA1 : kSA0);
    fence_async_smem();
    __syncthreads();
    if (r == 0) gemm_issue(sh.tmem, A, sm + Ws[l], Ks[l], Ns[l], &sh.bar);
    if (!wait_all(sh, phase)) return false;
    fence_after();
    if (l == 4) return true;
    float h[64];
#pragma unroll
    for (int q = 0; q < 4; ++q) tmem_ld16(sh.tmem + lane_base + 16 * q, h + 16 * q);
    uint32_t m0 = 0, m1 = 0;
#pragma unroll
    for (int j = 0; j < 64; ++j) {
      h[j] = h[j] > 0.0f ? h[j] : 0.0f;
      if (h[j] > 0.0f) {
        if (j < 32) m0 |= 1u << j;
        else m1 |= 1u << (j - 32);
      }
    }
    if (keep_mask) {
      mask[2 * l] = m0;
      mask[2 * l + 1] = m1;
    }
    fence_before();
    put_row(sm + ((l & 1) ? kSA0 : kSA1), r, 64, h);
    if (save_h && row_valid) {  // feature-major copy of h_{l+1} for the weight gradient
      __nv_bfloat16* dst = save_h + (size_t)(80 + 64 * l) * save_stride + row_global;
      for (int j = 0; j < 64; ++j) dst[(size_t)j * save_stride] = __float2bfloat16_rn(h[j]);
    }
  }
  return true;
}

// Mixture parameters and loss gradient at the outputs (the oracle's
// loss_grad_out in float): the loss is -weight * log q with q the vertex's
// sampling density alpha p_guide + (1 - alpha) p_bsdf, alpha = amax *
// sigmoid(o[40]); pb < 0 (no BSDF density recorded): q = p_guide and the
// selection logit gets no gradient.
__device__ void out_grad(const float* o, const float* w, float weight, float pb, float amax, float* g, float& loss) {
  float mx = -INFINITY;
#pragma unroll
  for (int k = 0; k < kLobes; ++k) mx = fmaxf(mx, o[5 * k + 4]);
  float pi[kLobes], v[kLobes], mu[kLobes][3], rn[kLobes], kap[kLobes], sig[kLobes];
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
    const float sp = s > 20.f ? s : log1pf(expf(s));
    float kk = sp + 0.01f;
    cl[k] = kk > 1000.f;
    kap[k] = cl[k] ? 1000.f : kk;
    sig[k] = 1.f / (1.f + expf(-s));
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
  float q = p, a = 1.f;
  g[40] = 0.f;
  if (pb >= 0.f) {
    const float sg = 1.f / (1.f + expf(-o[40]));
    a = amax * sg;
    q = fmaxf(a * p + (1.f - a) * pb, 1e-30f);
    g[40] = -weight * (p - pb) / q * (amax * sg * (1.f - sg));
  }
  q = fmaxf(q, 1e-30f);
  loss = -weight * logf(q);
  const float share = a * p / q;
#pragma unroll
  for (int k = 0; k < kLobes; ++k) {
    const float rr = a * pi[k] * v[k] / q;
    const float d = mu[k][0] * w[0] + mu[k][1] * w[1] + mu[k][2] * w[2];
    g[5 * k + 4] = -weight * (rr - share * pi[k]);
    const float dl = 1.f / kap[k] - 2.f / expm1f(2.f * kap[k]) + (d - 1.f);
    g[5 * k + 3] = cl[k] ? 0.f : -weight * rr * dl * sig[k];
    for (int c = 0; c < 3; ++c) g[5 * k + c] = -weight * rr * kap[k] * (w[c] - d * mu[k][c]) / rn[k];
  }
}

// Inference runs two tile streams per CTA: 256 threads in two groups of
// four warps share one copy of the weights; each group has its own
// activation tiles, mbarrier, named barrier (ids 1 and 2) and 64 TMEM
// columns (the 32x32b loads reach TMEM lanes 32*(warp % 4) .. +31, so the
// second group's warps read the same 128 lanes in their own columns).  One
// group's epilogue (TMEM -> ReLU -> bf16 -> shared memory) overlaps the
// other group's MMAs, and the SM holds twice the warps of a one-tile CTA.
constexpr uint32_t kGroups = 2;
constexpr uint32_t kSAGroup = 128 * 80 * 2 + 128 * 64 * 2;  // A0 + A1 of one group: 36864
// Dynamic shared memory: weights, the groups' tiles, then the control block
// (no static shared memory, so two CTAs fit an SM's 228 KB).
constexpr uint32_t kInferCtl = kSWEnd + kGroups * kSAGroup;
constexpr uint32_t kInferSmem2 = kInferCtl + 64;

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

// The forward pass of one tile by one group (features already in its A0):
// false if a wait ran out.  The output layer ends in the group's TMEM
// columns 0..47.
__device__ bool forward_tile_group(char* sm, char* a0, char* a1, GroupShared& gs, uint32_t tmem, uint32_t bid,
                                   uint32_t r, uint32_t& phase) {
  const uint32_t lane_base = (r & ~31u) << 16;
  const uint32_t Ks[5] = {80, 64, 64, 64, 64};
  const uint32_t Ns[5] = {64, 64, 64, 64, 48};
  const uint32_t Ws[5] = {kSW0, kSW1, kSW2, kSW3, kSW4};
  for (int l = 0; l < 5; ++l) {
    const char* A = (l & 1) ? a1 : a0;
    fence_async_smem();
    group_sync(bid);
    if (r == 0) gemm_issue(tmem, A, sm + Ws[l], Ks[l], Ns[l], &gs.bar);
    const bool ok = bar_wait(&gs.bar, phase);
    phase ^= 1u;
    if (group_any(!ok, bid)) {
      if (r == 0) gs.abort = 1;
      return false;
    }
    fence_after();
    if (l == 4) return true;
    float h[64];
#pragma unroll
    tmem_ld64(tmem + lane_base, h);
#pragma unroll
    for (int j = 0; j < 64; ++j) h[j] = h[j] > 0.0f ? h[j] : 0.0f;
    fence_before();
    put_row((l & 1) ? a0 : a1, r, 64, h);
  }
  return true;
}

__global__ void __launch_bounds__(256) k_guide_infer(GuideRows in, const __nv_bfloat16* wf, float* out, int* err) {
  extern __shared__ __align__(1024) char sm[];
  GroupShared* gsh = reinterpret_cast<GroupShared*>(sm + kInferCtl);
  uint32_t& tmem_base = *reinterpret_cast<uint32_t*>(sm + kInferCtl + kGroups * sizeof(GroupShared));
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
  if (threadIdx.x < 32) tmem_alloc(&tmem_base, 64 * kGroups);
  fence_before();
  __syncthreads();
  fence_after();
  GroupShared& gs = gsh[g];
  char* a0 = sm + kSWEnd + g * kSAGroup;
  char* a1 = a0 + 128 * 80 * 2;
  const uint32_t tmem = tmem_base + 64u * g;
  const uint32_t lane_base = (r & ~31u) << 16;
  uint32_t phase = 0;
  const uint64_t ntiles = (n + 127) / 128;
  for (uint64_t t = (uint64_t)blockIdx.x * kGroups + g; t < ntiles; t += (uint64_t)gridDim.x * kGroups) {
    const uint64_t row = t * 128 + r;
    float f[80];
    const bool valid = row < n;
    if (valid) {
      const float p[3] = {in.px[row], in.py[row], in.pz[row]};
      const float nn[3] = {in.nx[row], in.ny[row], in.nz[row]};
      const float wo[3] = {in.wx[row], in.wy[row], in.wz[row]};
      features(p, nn, wo, in.lo, in.inv_ext, f);
    } else {
      for (int k = 0; k < 80; ++k) f[k] = 0.f;
    }
    put_row(a0, r, 80, f);
    if (!forward_tile_group(sm, a0, a1, gs, tmem, bid, r, phase)) break;
    float o[48];
#pragma unroll
    tmem_ld48(tmem + lane_base, o);
    fence_before();
    if (valid) {
      // 44 floats per row (41 outputs; columns 41..43 of the padded layer are 0)
      float4* dst = reinterpret_cast<float4*>(out + (size_t)row * kGuideOutStride);
#pragma unroll
      for (int k = 0; k < kGuideOutStride / 4; ++k)
        dst[k] = make_float4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
    }
  }
  // a group that stopped early waits (bounded) for its MMAs still in flight
  if (gs.abort) (void)bar_wait(&gs.bar, phase ^ 1u);
  __syncthreads();
  if (r == 0 && gs.abort) atomicExch(err, 1);
  if (threadIdx.x < 32) tmem_free(tmem_base, 64 * kGroups);
}

// Forward + loss gradient + backward-data over one tile per iteration.
// Saved feature-major (stride = batch size B): X rows 0..79, h1..h4 at 80 +
// 64*l, dY at 336 (48 rows), dZ4..dZ1 at 384 + 64*(4-l) (l = 4..1).
__global__ void __launch_bounds__(128) k_guide_train(GuideTrain tr, const __nv_bfloat16* wf, const __nv_bfloat16* wb,
                                                     __nv_bfloat16* save, float* sums, int* err) {
  extern __shared__ __align__(1024) char sm[];
  __shared__ Shared sh;
  const uint32_t r = threadIdx.x;
  const uint64_t n = tr.rows.n_dev ? *tr.rows.n_dev : tr.rows.n;
  const uint32_t B = tr.stride;
  if (r == 0) {
    bar_init(&sh.bar);
    sh.abort = 0;
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
  if (r < 32) tmem_alloc(&sh.tmem, 64);
  fence_before();
  __syncthreads();
  fence_after();
  uint32_t phase = 0;
  const uint32_t lane_base = (r & ~31u) << 16;
  const uint64_t ntiles = (n + 127) / 128;
  float loss_acc = 0.f, w_acc = 0.f;
  bool ok = true;
  for (uint64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const uint64_t row = t * 128 + r;
    const bool valid = row < n;
    float f[80];
    float weight = 0.f, om[3] = {0.f, 0.f, 1.f};
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
      for (int k = 0; k < 80; ++k) save[(size_t)k * B + row] = __float2bfloat16_rn(f[k]);
    } else {
      for (int k = 0; k < 80; ++k) f[k] = 0.f;
    }
    put_row(sm + kSA0, r, 80, f);
    uint32_t mask[8];
    if (!forward_tile(sm, sh, phase, mask, true, save, B, (uint32_t)row, valid)) {
      ok = false;
      break;
    }
    float o[48];
#pragma unroll
    for (int q = 0; q < 3; ++q) tmem_ld16(sh.tmem + lane_base + 16 * q, o + 16 * q);
    float g[48];
    for (int k = kGuideOut; k < 48; ++k) g[k] = 0.f;
    if (valid) {
      float loss;
      const float pb = tr.pb ? tr.pb[row * tr.rows.rstride] : -1.0f;
      out_grad(o, om, weight, pb, tr.amax, g, loss);
      loss_acc += loss;
      w_acc += weight;
    } else {
      for (int k = 0; k < kGuideOut; ++k) g[k] = 0.f;
    }
    fence_before();
    put_row(sm + kSA0, r, 48, g);  // dY, K = 48
    if (valid)
      for (int k = 0; k < 48; ++k) save[(size_t)(336 + k) * B + row] = __float2bfloat16_rn(g[k]);
    // dH_l = dZ_{l+1} * W_l, masked by h_l > 0, for l = 4 .. 1
    const uint32_t Bt[5] = {0, kSB1, kSB2, kSB3, kSB4};
    for (int l = 4; l >= 1; --l) {
      const uint32_t K = l == 4 ? 48u : 64u;
      const char* A = sm + ((l & 1) ? kSA1 : kSA0);  // l=4 reads A0 (dY), l=3 reads A1, ...
      fence_async_smem();
      __syncthreads();
      if (r == 0) gemm_issue(sh.tmem, A, sm + Bt[l], K, 64, &sh.bar);
      if (!wait_all(sh, phase)) {
        ok = false;
        break;
      }
      fence_after();
      float d[64];
#pragma unroll
      for (int q = 0; q < 4; ++q) tmem_ld16(sh.tmem + lane_base + 16 * q, d + 16 * q);
      const uint32_t m0 = mask[2 * (l - 1)], m1 = mask[2 * (l - 1) + 1];
#pragma unroll
      for (int j = 0; j < 64; ++j) {
        const bool on = j < 32 ? ((m0 >> j) & 1u) : ((m1 >> (j - 32)) & 1u);
        d[j] = on ? d[j] : 0.f;
      }
      fence_before();
      put_row(sm + ((l & 1) ? kSA0 : kSA1), r, 64, d);
      if (valid)
        for (int j = 0; j < 64; ++j) save[(size_t)(384 + 64 * (4 - l) + j) * B + row] = __float2bfloat16_rn(d[j]);
    }
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
  __syncthreads();
  drain(sh, phase);
  if (sh.abort && r == 0) atomicExch(err, 1);
  if (r < 32) tmem_free(sh.tmem, 64);
}

// Weight gradients: for layer l, D [128 x N] += A [128 x 128] * B [N x 128]^T
// over chunks of 128 batch rows, A = the output deltas of layer l (M rows of
// the feature-major save, rows M..127 zero), B = the layer's input (N rows).
// blockIdx.y = layer, blockIdx.x strides the chunks; partial sums go to the
// float32 gradient with atomics.
constexpr uint32_t kGA = 0, kGB = 128 * 128 * 2, kWgradSmem = kGB + 80 * 128 * 2 + 64;
__global__ void __launch_bounds__(128) k_guide_wgrad(const __nv_bfloat16* save, uint32_t B, uint64_t n,
                                                     const unsigned long long* n_dev, float* grad, int* err) {
  extern __shared__ __align__(1024) char sm[];
  __shared__ Shared sh;
  const uint32_t r = threadIdx.x;
  if (n_dev) n = *n_dev < n ? *n_dev : n;
  const int l = blockIdx.y;
  // layer l: output deltas at row dz0 (M of them), inputs at row in0 (N)
  const uint32_t M = l == 4 ? (uint32_t)kGuideOut : 64u;
  const uint32_t N = l == 0 ? 80u : 64u;
  const uint32_t dz0 = l == 4 ? 336u : 384u + 64u * (3u - (uint32_t)l);
  const uint32_t in0 = l == 0 ? 0u : 80u + 64u * (uint32_t)(l - 1);
  const uint32_t goff = l == 0 ? 0u : (l == 4 ? 17408u : 5120u + 4096u * (uint32_t)(l - 1));
  if (r == 0) {
    bar_init(&sh.bar);
    sh.abort = 0;
  }
  // zero the whole A tile once (rows >= M stay zero)
  for (uint32_t i = r; i < 128 * 128 * 2 / 16; i += 128) reinterpret_cast<uint4*>(sm + kGA)[i] = make_uint4(0, 0, 0, 0);
  if (r < 32) tmem_alloc(&sh.tmem, 128);
  fence_before();
  __syncthreads();
  fence_after();
  uint32_t phase = 0;
  bool any = false, ok = true;
  const uint64_t nchunks = (n + 127) / 128;
  for (uint64_t c = blockIdx.x; c < nchunks && ok; c += gridDim.x) {
    const uint64_t b0 = c * 128;
    // A rows (deltas) and B rows (inputs): 16 chunks of 8 batch values per row
    for (uint32_t i = r; i < (M + N) * 16; i += 128) {
      const uint32_t row = i / 16, ch = i % 16;
      const bool isA = row < M;
      const uint32_t src = isA ? dz0 + row : in0 + (row - M);
      uint4 q = make_uint4(0, 0, 0, 0);
      const uint64_t col = b0 + 8 * ch;
      if (col + 8 <= n) {
        q = *reinterpret_cast<const uint4*>(save + (size_t)src * B + col);
      } else if (col < n) {
        union {
          uint4 q;
          __nv_bfloat16 h[8];
        } tmp;
        for (int e = 0; e < 8; ++e)
          tmp.h[e] = col + e < n ? save[(size_t)src * B + col + e] : __float2bfloat16_rn(0.f);
        q = tmp.q;
      }
      char* dst = isA ? sm + kGA + chunk_off(row, ch, 128) : sm + kGB + chunk_off(row - M, ch, 128);
      *reinterpret_cast<uint4*>(dst) = q;
    }
    fence_async_smem();
    __syncthreads();
    if (r == 0) {
      fence_after();
      const uint32_t a0 = saddr(sm + kGA), bb = saddr(sm + kGB);
      const uint32_t id = idesc(128, (int)N);
      for (uint32_t kk = 0; kk < 8; ++kk)
        mma(sh.tmem, sdesc(a0 + kk * 256u, 128u, 16u * 128u), sdesc(bb + kk * 256u, 128u, 16u * 128u), id,
            (any || kk > 0) ? 1u : 0u);
      mma_commit(&sh.bar);
    }
    any = true;
    if (!wait_all(sh, phase)) {
      ok = false;
      break;
    }
    fence_after();  // the loop's next __syncthreads orders the operand reuse
  }
  if (any && ok) {
    // every warp loads its lane quarter (warp-collective); rows >= M are padding
    const uint32_t lane_base = (r & ~31u) << 16;
    for (uint32_t q = 0; q < N / 16; ++q) {
      float v[16];
      tmem_ld16(sh.tmem + lane_base + 16 * q, v);
      if (r < M)
        for (int e = 0; e < 16; ++e) atomicAdd(&grad[goff + r * N + 16 * q + e], v[e]);
    }
  }
  fence_before();
  __syncthreads();
  drain(sh, phase);
  if (sh.abort && r == 0) atomicExch(err, 1);
  if (r < 32) tmem_free(sh.tmem, 128);
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

int launch_infer(const GuideRows& rows, const void* wf, float* out, int* err, int grid, cudaStream_t st) {
  k_guide_infer<<<grid, 256, kInferSmem2, st>>>(rows, static_cast<const __nv_bfloat16*>(wf), out, err);
  return (int)cudaGetLastError();
}

int launch_train(const GuideTrain& tr, const void* wf, const void* wb, void* save, float* sums, int* err, int grid,
                 cudaStream_t st) {
  k_guide_train<<<grid, 128, kTrainSmem, st>>>(tr, static_cast<const __nv_bfloat16*>(wf),
                                                static_cast<const __nv_bfloat16*>(wb),
                                                static_cast<__nv_bfloat16*>(save), sums, err);
  return (int)cudaGetLastError();
}

int launch_wgrad(const void* save, uint32_t B, uint64_t n, const unsigned long long* n_dev, float* grad, int* err,
                 int chunks, cudaStream_t st) {
  dim3 g(chunks, 5);
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
  const uint64_t tiles = (n + 127) / 128;
  const int grid = (int)std::min<uint64_t>(tiles, (uint64_t)sms * 2);
  if (vmr::guide::launch_train(t, G.wf.p, G.wb.p, G.save.p, G.sums.as<float>(), G.err.as<int>(), grid,
                               ctx->stream) != 0)
    return gfail(ctx, VMR_ERR_CUDA, "guide training kernel launch failed");
  const int chunks = (int)std::min<uint64_t>(tiles, (uint64_t)sms);
  if (vmr::guide::launch_wgrad(G.save.p, (uint32_t)stride, n, nullptr, G.grad.as<float>(), G.err.as<int>(), chunks,
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
  const uint64_t tiles = (n + 127) / 128;
  const int grid = (int)std::min<uint64_t>(tiles, (uint64_t)guide_sms(ctx) * 2);
  if (vmr::guide::launch_infer(tr.rows, ctx->guide.wf.p, dout, ctx->guide.err.as<int>(), grid, ctx->stream) != 0)
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
