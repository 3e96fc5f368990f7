// pathtrace.cu - extended path tracer (vmr_render_path): indirect bounces,
// next-event estimation with the power heuristic, Russian roulette, quad and
// environment lights.  No reference counterpart (the reference renders
// direct light only); the estimator is specified in include/vmr.h and
// restated independently by the float32/float64 oracle.
//
// Wavefront per batch of whole iterations (n paths, one per (iteration,
// pixel)):
//   k_pt_generate            camera rays (the reference mode's) into queue 0
//   for d = 0 .. max_depth:
//     [ray sort]             VMR_PATH_SORT_QUEUES, d > 0: queue d in key order
//     trace                  closest hit of queue d (count read on the device)
//     [k_pt_prep, guide]     guided vertices (d < guide_depth): network rows
//                            and the tcgen05 inference over the queue
//     k_pt_shade<d>          emission / environment with MIS, light sample +
//                            shadow ray into the shadow queue, BSDF sample +
//                            continuation into queue d+1 (warp-aggregated
//                            appends), Russian roulette
//     trace (d < max_depth)  any hit of the shadow queue (sorted first with
//                            VMR_PATH_SORT_QUEUES)
//     k_pt_resolve           unoccluded shadow rays add their contribution
//   k_pt_accumulate          per pixel, the batch's iterations in order:
//                            buf = (buf*i + L)/(i+1), i the 0-based iteration
//                            (float, optional float64)
//   [k_pt_targets, training] VMR_PATH_TRAIN: the guide's records and Adam steps
// A batch holds the context's queue capacity (16M paths by default,
// vmr_set_path_batch / vmr_autotune_path).  Batched jobs put many one-mesh
// images end to end in one pixel arena; their rays enter their own mesh
// (the scene kernels' job mode).
// Every queue length lives in device memory and every kernel reads it there,
// so a batch runs without host synchronisation; the whole sequence is
// captured once as a CUDA graph and replayed per batch (the batch's first
// iteration and path count are copied in before each replay).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "device.h"
#include "guide.h"
#include "shade_common.cuh"
#include "vmr.h"

namespace vmr {
namespace {

constexpr int kPtMaxDepth = 32;
constexpr int kPtBlock = 256;

// One light of the path tracer's light list (TriLights, quad lights, the
// environment, in that order).
struct PtLight {
  int kind;  // 0 triangle (p0, a = p1, b = p2), 1 quad (p0, a = e1, b = e2), 2 environment
  float p0[3], a[3], b[3];
  float N[3];  // emitting side
  float area;
  float Le[3];
  int32_t geom;
};

// Per-batch values copied in before each replay.
struct PtIter {
  uint32_t iter0;  // first iteration of the batch
  uint32_t iters;  // iterations in the batch
  unsigned long long n;  // paths = iters * npix
};

// One job of a batched render (vmr_render_path_jobs): its mesh, camera and
// image; pix0 is the first pixel of the job in the batch's pixel arena (the
// jobs' images end to end, in job order).
struct PtJob {
  vmr_camera cam;
  uint32_t width, height, npix, geom;
  uint32_t pix0;
  uint32_t pad[3];
};

struct PtBatch {
  uint32_t width, height, npix;  // npix: the pixels of the rendered band
  // GeomInstances, Procs or keyed mesh transforms in the scene: the shading
  // kernels' GROUPS instantiation applies their transforms at each hit
  uint32_t groups;
  uint32_t pix0;                 // the band's first pixel in the image (one-scene renders)
  uint32_t nl;        // lights
  uint32_t max_depth, rr_depth;
  uint32_t has_env;
  uint32_t cap;       // path capacity of the buffers
  float env[3];
  float sel;          // 1/nl
  uint64_t seed;
  vmr_camera cam;
  const anim::Decomp* cam_keys;  // camera motion keys (cam_nkeys >= 2), else null
  uint32_t cam_nkeys;
  PixFilter filt;     // pixel filter tables (n = 0: none)
  const PtIter* it;
  const vmr_shader_std* shaders;
  const PtLight* lights;
  const RMesh* meshes;
  const int32_t* light_of_geom;
  uint32_t n_geoms;
  // per path
  float *bx, *by, *bz;   // throughput
  float *lx, *ly, *lz;   // radiance
  float* pdf;            // pdf of the last BSDF sample (0: camera or mirror)
  unsigned long long* key;
  // extension queues (ping-pong) and the hit record of the current one
  float* qray[2];        // 8 * cap floats: px py pz dx dy dz tmax time
  uint32_t* qpath[2];
  int32_t *hprim, *hgeom;
  float *ht, *hu, *hv, *hw;
  // shadow queue
  float* sray;           // 8 * cap
  uint32_t* spath;
  float* scontrib;       // 3 * cap
  int32_t* shit;
  unsigned long long* qlen;  // [kPtMaxDepth + 2]
  unsigned long long* slen;  // [kPtMaxDepth + 1]
  unsigned long long* totals;  // [2]: extension rays, shadow rays
  const DScratch* scr;         // the traversal launches' scratch, 2 per bounce
  int* status;                 // worst traversal status over all batches
  float* fb;
  double* fb64;
  // path guiding
  float alpha;                 // learned selection: the largest probability of
                               // sampling the guide at a vertex (alpha_max);
                               // fixed selection: that probability itself
  uint32_t learn_sel;          // 1: each vertex's probability is alpha_max *
                               // sigmoid(the network's selection output)
  uint32_t gdepth;             // guided vertices: the first gdepth of a path (host side)
  float glo[3];                // scene bounds for the guide's inputs
  float* grow;                 // 9 * cap: guide input rows per queue entry
  float* gout;                 // 44 * cap: guide outputs per queue entry
  float* rec;                  // kRecCols * rcap training records (SoA)
  uint32_t rcap;
  unsigned long long* rcount;  // [2]: records this batch, records in total
  uint32_t* last_rec;          // per path: its last record awaiting L_mark
  // batched jobs (n_jobs > 0): the job table and each path's mesh
  const PtJob* jobs;
  uint32_t n_jobs;
  uint32_t* pgeom;             // cap: path -> its job's geom
  float* snee;                 // 8 * cap: per shadow slot, the vertex's normal and
                               // direction toward the previous vertex, the
                               // light sample's training weight (0: no record)
                               // and the BSDF's density of its direction
};

// Training record columns: vertex (p, n, wo), sampled direction, weight
// (filled after the bounce loop), density, throughput after the vertex,
// radiance before the next vertex, path, the BSDF's density of the direction.
constexpr int kRecCols = 22;
enum RecCol {
  kRP = 0, kRN = 3, kRWo = 6, kROm = 9, kRW = 12, kRQ = 13, kRBeta = 14, kRMark = 17, kRPath = 20, kRPb = 21
};
constexpr uint32_t kNoPath = 0xffffffffu;  // path column of a light-sample record

// ------------------------------------------------------------- random ----
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
constexpr uint64_t kGold = 0x9E3779B97F4A7C15ull;
__device__ __forceinline__ uint64_t sample_key(uint64_t seed, uint64_t pix, uint64_t j) {
  return mix64(mix64(seed + kGold * (pix + 1)) + kGold * (j + 1));
}
// 24 random bits as a float in [0, 1), exact in float32.
__device__ __forceinline__ float rnd(uint64_t key, uint32_t dim) {
  // 24 bits: converted through uint32 (a 64-bit conversion would take the
  // narrow float64 pipe); the same value either way
  return (float)(uint32_t)(mix64(key + kGold * (uint64_t)(dim + 1)) >> 40) * 5.9604644775390625e-08f;
}

constexpr float kInv4Pi = 0.0795774715f;  // float32(1/(4 pi))

// sin and cos of 2*pi*u for u in [0, 1) in float32 arithmetic only (GB300's
// float64 pipe is narrow, and these sit in every bounce's sampling):
// u*4 splits exactly into a quarter turn k and a fraction f (u has 24
// fraction bits), f > 1/2 is reflected to 1-f with sin and cos swapped, and
// the remaining angle x = (pi/2)*f in [0, pi/4] goes through the Taylor
// series of sin to x^9 and of cos to x^10 (truncation below 2e-9 there);
// the quarter turn rotates the pair.  The oracle evaluates the same
// operations in the same order, so both give the same bits.
__device__ __forceinline__ void sincos_turns(float u, float& s, float& c) {
  const float q = u * 4.0f;
  int k = (int)q;
  float f = q - (float)k;
  const bool refl = f > 0.5f;
  if (refl) f = 1.0f - f;
  const float x = f * 1.57079632679f;
  const float x2 = x * x;
  const float sp = x * (1.0f + x2 * (-0.166666667f + x2 * (8.33333333e-3f + x2 * (-1.98412698e-4f +
                                                                                 x2 * 2.75573192e-6f))));
  const float cp = 1.0f + x2 * (-0.5f + x2 * (4.16666667e-2f + x2 * (-1.38888889e-3f + x2 * (2.48015873e-5f +
                                                                                            x2 * -2.75573192e-7f))));
  const float s0 = refl ? cp : sp, c0 = refl ? sp : cp;
  k &= 3;
  s = k == 0 ? s0 : (k == 1 ? c0 : (k == 2 ? -s0 : -c0));
  c = k == 0 ? c0 : (k == 1 ? -s0 : (k == 2 ? -c0 : s0));
}

// ----------------------------------------------------------- material ----
struct Mat {
  float dw, sw;
  V3 cd, cs;
  float rd, alpha;
  bool mirror;
  Fresnel fr;
};

__device__ __forceinline__ Mat material(const vmr_shader_std& s) {
  Mat m;
  const float dw = (s.flags & VMR_SH_DIFFUSE_STRENGTH) ? s.diffuse_strength : 0.0f;
  const float sw = (s.flags & VMR_SH_SPEC1_STRENGTH) ? s.spec1_strength : 0.0f;
  const float tw = dw + sw;
  m.dw = dw / tw;
  m.sw = sw / tw;
  m.cd = (s.flags & VMR_SH_DIFFUSE_COLOUR) ? v3(s.diffuse_colour[0], s.diffuse_colour[1], s.diffuse_colour[2])
                                           : v3(0, 0, 0);
  m.cs = (s.flags & VMR_SH_SPEC1_COLOUR) ? v3(s.spec1_colour[0], s.spec1_colour[1], s.spec1_colour[2]) : v3(0, 0, 0);
  m.rd = (s.flags & VMR_SH_DIFFUSE_ROUGHNESS) ? s.diffuse_roughness : 0.5f;
  const float rs = (s.flags & VMR_SH_SPEC1_ROUGHNESS) ? s.spec1_roughness : 0.5f;
  m.mirror = rs == 0.0f;
  m.alpha = sqr(rs * rs);
  m.fr = Fresnel{0, (s.flags & VMR_SH_IOR) ? s.ior : 1.7f, {}, {}};
  if (s.spec1_fresnel == 1) {
    RGB refl{{0.5f, 0.5f, 0.5f}}, edge{{0.5f, 0.5f, 0.5f}};
    if (s.flags & VMR_SH_FRESNEL_REFL) refl = RGB{{s.spec1_fresnel_refl[0], s.spec1_fresnel_refl[1], s.spec1_fresnel_refl[2]}};
    if (s.flags & VMR_SH_FRESNEL_EDGE)  // the reference's assignment (std.go:185-187)
      refl = RGB{{s.spec1_fresnel_edge[0], s.spec1_fresnel_edge[1], s.spec1_fresnel_edge[2]}};
    m.fr = Fresnel{1, 0, refl, edge};
  }
  return m;
}

__device__ __forceinline__ float ggx_d_pt(V3 m, float alpha) {
  if (m.z <= 0.0f) return 0.0f;
  if (m.z == 1.0f) return 1.0f / (kPi * alpha * alpha);
  const float denom = kPi * sqr(m.z * m.z) * sqr(alpha * alpha + ((1.0f / (m.z * m.z)) - 1));
  return (alpha * alpha) / denom;
}

// f(wi, wo)*|cos wo| in the local frame (wi.z > 0: the frame faces wi).
__device__ V3 bsdf_f(const Mat& m, V3 wi, V3 wo) {
  V3 f = v3(0, 0, 0);
  if (wo.z <= 0.0f) return f;
  if (m.dw > 0.0f) {
    float s;
    if (m.rd == 0.0f) {
      s = wo.z / kPi;
    } else {  // OrenNayar (bsdf/orennayar.go:42-73), sigma = roughness^2
      // without angles: alpha = max(theta), beta = min(theta) of the two
      // directions, so sin(alpha) = sin(theta) of the smaller cos and
      // tan(beta) = sin/cos of the larger; cos(phiO - phiI) from the
      // tangent-plane components (0 when a direction is along the normal)
      const float sigma = m.rd * m.rd;
      const float A = 1 - (0.5f * (sigma * sigma) / ((sigma * sigma) + 0.57f));
      const float B = 0.45f * (sigma * sigma) / ((sigma * sigma) + 0.09f);
      const float sI = sqrtf(fmaxf(0.0f, 1.0f - wi.z * wi.z)), sO = sqrtf(fmaxf(0.0f, 1.0f - wo.z * wo.z));
      const bool iLow = wi.z < wo.z;  // theta_i is the larger angle
      const float C = iLow ? sI * (sO / wo.z) : sO * (sI / wi.z);
      const float den = sI * sO;
      const float gm = den > 1e-6f ? (wi.x * wo.x + wi.y * wo.y) / den : 0.0f;
      s = wo.z * (A + (B * (gm > 0.0f ? gm : 0.0f) * C)) / kPi;
    }
    const float k = m.dw * s;
    f = v3(k * m.cd.x, k * m.cd.y, k * m.cd.z);
  }
  if (m.sw > 0.0f && !m.mirror) {
    const V3 h = normalize(add(wi, wo));
    const RGB F = fresnel_kr(m.fr, fabsf(dot(wi, h)));
    const float numer = ggx_g1(wi, h, m.alpha) * ggx_g1(wo, h, m.alpha) * ggx_d_pt(h, m.alpha);
    const float denom = 4 * wi.z * wo.z;
    float s = wo.z * numer / denom;
    if (!(s > 0.0f)) s = 0.0f;
    const float k = m.sw * s;
    f = add(f, v3(k * m.cs.x * F.c[0], k * m.cs.y * F.c[1], k * m.cs.z * F.c[2]));
  }
  return f;
}

__device__ float bsdf_pdf_pt(const Mat& m, V3 wi, V3 wo) {
  if (wo.z <= 0.0f) return 0.0f;
  float p = m.dw * (wo.z / kPi);
  if (m.sw > 0.0f && !m.mirror) {
    const V3 h = normalize(add(wi, wo));
    const float d = fabsf(dot(wo, h));
    if (d > 0.0f) p = p + m.sw * (ggx_d_pt(h, m.alpha) * h.z / (4 * d));
  }
  return p;
}

__device__ __forceinline__ float power_w(float a, float b) { return (a * a) / (a * a + b * b); }
__device__ __forceinline__ float tmax3(float a, float b, float c) { return a > b ? (a > c ? a : c) : (b > c ? b : c); }

// Warp-aggregated append: one atomic per warp for the lanes that want a slot.
__device__ __forceinline__ unsigned long long warp_append(unsigned long long* counter, bool want) {
  const unsigned act = __activemask();
  const unsigned m = __ballot_sync(act, want);
  if (m == 0u) return ~0ull;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(m));
  base = __shfl_sync(act, base, leader);
  return want ? base + __popc(m & ((1u << lane) - 1u)) : ~0ull;
}

__device__ __forceinline__ void put_ray(float* q, uint32_t cap, uint64_t i, const float o[3], V3 d, float tmax,
                                        float time) {
  q[i] = o[0];
  q[cap + i] = o[1];
  q[2 * (size_t)cap + i] = o[2];
  q[3 * (size_t)cap + i] = d.x;
  q[4 * (size_t)cap + i] = d.y;
  q[5 * (size_t)cap + i] = d.z;
  q[6 * (size_t)cap + i] = tmax;
  q[7 * (size_t)cap + i] = time;
}

// ------------------------------------------------------- guide mixture ---
// The network outputs 0..39 as 8 vMF lobes (the same decoding the trainer
// differentiates): mu = normalize, kappa = exp(s) with s clamped to
// [-4.6, 6.9], pi = softmax; c = kappa / (2 pi (1 - exp(-2 kappa))).  Output 40 is the
// selection logit: with learned selection the vertex samples the guide with
// probability alpha = alpha_max * sigmoid(o[40]), else with alpha_max.
struct GMix {
  float mu[8][3], kap[8], c[8], pi[8];
  float alpha;
};
__device__ void gmix_decode(const float* o, float amax, bool learned, GMix& g) {
  g.alpha = learned ? amax / (1.f + expf(-o[40])) : amax;
  float mx = -INFINITY;
  for (int k = 0; k < 8; ++k) mx = fmaxf(mx, o[5 * k + 4]);
  float z = 0.f;
  for (int k = 0; k < 8; ++k) {
    const float* r = o + 5 * k;
    float n = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    n = n < 1e-6f ? 1e-6f : n;
    for (int c = 0; c < 3; ++c) g.mu[k][c] = r[c] / n;
    g.kap[k] = expf(fminf(fmaxf(r[3], -4.6f), 6.9f));
    g.c[k] = g.kap[k] / (6.28318530718f * (-expm1f(-2.f * g.kap[k])));
    g.pi[k] = expf(r[4] - mx);
    z += g.pi[k];
  }
  for (int k = 0; k < 8; ++k) g.pi[k] /= z;
}
__device__ float gmix_pdf(const GMix& g, V3 w) {
  float p = 0.f;
  for (int k = 0; k < 8; ++k) {
    const float d = g.mu[k][0] * w.x + g.mu[k][1] * w.y + g.mu[k][2] * w.z;
    p += g.pi[k] * g.c[k] * expf(g.kap[k] * (d - 1.f));
  }
  return p;
}
// A direction from the mixture: lobe by u (cumulative pi), then the vMF
// inversion w = 1 + log(u1 + (1-u1) e^{-2 kappa}) / kappa around mu.
__device__ V3 gmix_sample(const GMix& g, float u, float u1, float u2) {
  int k = 7;
  float acc = 0.f;
  for (int j = 0; j < 8; ++j) {
    acc += g.pi[j];
    if (u < acc) {
      k = j;
      break;
    }
  }
  const float kap = g.kap[k];
  float w = 1.f + logf(u1 + (1.f - u1) * expf(-2.f * kap)) / kap;
  w = fminf(1.f, fmaxf(-1.f, w));
  const float st = sqrtf(fmaxf(0.f, 1.f - w * w));
  const float phi = 6.28318530718f * u2;
  const V3 mu = v3(g.mu[k][0], g.mu[k][1], g.mu[k][2]);
  const float sgn = mu.z >= 0.f ? 1.f : -1.f;  // orthonormal basis (Duff et al. 2017)
  const float a = -1.f / (sgn + mu.z);
  const float bb = mu.x * mu.y * a;
  const V3 t1 = v3(1.f + sgn * mu.x * mu.x * a, sgn * bb, -sgn * mu.x);
  const V3 t2 = v3(bb, sgn + mu.y * mu.y * a, -mu.y);
  const float cp = cosf(phi), sp = sinf(phi);
  return normalize(v3(w * mu.x + st * (cp * t1.x + sp * t2.x), w * mu.y + st * (cp * t1.y + sp * t2.y),
                      w * mu.z + st * (cp * t1.z + sp * t2.z)));
}

// CKEYS: the camera has motion keys (b.cam_nkeys >= 2).
template <bool CKEYS>
__global__ void __launch_bounds__(kPtBlock) k_pt_generate(PtBatch b) {
  const uint64_t n = b.it->n < b.cap ? b.it->n : b.cap;
  if (blockIdx.x == 0 && threadIdx.x == 0) b.qlen[0] = n;
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t pix = (uint32_t)(s % b.npix);
    const uint32_t j = b.it->iter0 + (uint32_t)(s / b.npix) + 1;
    V3 P, D;
    float time, lambda;
    if (b.n_jobs) {  // the job holding arena pixel pix (jobs sorted by pix0)
      uint32_t lo = 0, hi = b.n_jobs - 1;
      while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (b.jobs[mid].pix0 <= pix) lo = mid;
        else hi = mid - 1;
      }
      const PtJob& job = b.jobs[lo];
      pix -= job.pix0;
      b.pgeom[s] = job.geom;
      camera_primary<false>(job.cam, nullptr, 0, job.width, job.height, j, pix, b.seed, b.filt, P, D, time, lambda);
    } else {
      pix += b.pix0;  // the image pixel: a band samples as the whole image does
      camera_primary<CKEYS>(b.cam, b.cam_keys, b.cam_nkeys, b.width, b.height, j, pix, b.seed, b.filt, P, D,
                            time, lambda);
    }
    const float o[3] = {P.x, P.y, P.z};
    put_ray(b.qray[0], b.cap, s, o, D, __int_as_float(0x7f800000), time);
    b.qpath[0][s] = (uint32_t)s;
    b.bx[s] = 1.0f; b.by[s] = 1.0f; b.bz[s] = 1.0f;
    b.lx[s] = 0.0f; b.ly[s] = 0.0f; b.lz[s] = 0.0f;
    b.pdf[s] = 0.0f;
    b.key[s] = sample_key(b.seed, pix, j);
    if (b.last_rec) b.last_rec[s] = 0xffffffffu;
  }
}

// Guide inputs of queue d: the hit point, the shading normal facing the
// incoming ray and the direction toward the previous vertex (misses and
// faces without a shader get a placeholder row the shade kernel ignores).
template <bool GROUPS>
__global__ void __launch_bounds__(kPtBlock) k_pt_prep(PtBatch b, uint32_t d) {
  const uint64_t n = b.qlen[d] < b.cap ? b.qlen[d] : b.cap;
  const float* q = b.qray[d & 1];
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    V3 P = v3(b.glo[0], b.glo[1], b.glo[2]), N = v3(0, 0, 1), wi = v3(0, 0, 1);
    const int32_t prim = b.hprim[i];
    if (prim >= 0) {
      Ctx sc;
      uint32_t shid = 0;
      const V3 Ro = v3(q[i], q[(size_t)b.cap + i], q[2 * (size_t)b.cap + i]);
      const V3 Rd = v3(q[3 * (size_t)b.cap + i], q[4 * (size_t)b.cap + i], q[5 * (size_t)b.cap + i]);
      if (surface_attributes<GROUPS>(b.meshes[b.hgeom[i]], prim, b.hu[i], b.hv[i], b.hw[i], Ro, Rd, b.ht[i],
                             q[7 * (size_t)b.cap + i], sc, shid)) {
        wi = v3(-q[3 * (size_t)b.cap + i], -q[4 * (size_t)b.cap + i], -q[5 * (size_t)b.cap + i]);
        P = sc.P;
        N = dot(sc.Ng, wi) > 0.0f ? sc.N : v3(-sc.N.x, -sc.N.y, -sc.N.z);
      }
    }
    float* g = b.grow;
    const size_t c = b.cap;
    g[i] = P.x; g[c + i] = P.y; g[2 * c + i] = P.z;
    g[3 * c + i] = N.x; g[4 * c + i] = N.y; g[5 * c + i] = N.z;
    g[6 * c + i] = wi.x; g[7 * c + i] = wi.y; g[8 * c + i] = wi.z;
  }
}

// One bounce of every path in queue d.  GUIDED: one-sample MIS of the guide
// (probability alpha) and the BSDF at non-mirror vertices; TRAIN: training
// records of the guided continuations; GROUPS: the scene has GeomInstances,
// Procs or keyed mesh transforms (their transforms applied at each hit).
// Registers capped for 3 resident blocks per SM (2 guided): measured faster
// than the uncapped 121 (166) registers despite a few spilled words; the
// GROUPS instantiation, which holds the keyed-transform helpers' registers,
// is left uncapped.
template <bool GUIDED, bool TRAIN, bool GROUPS>
__global__ void __launch_bounds__(kPtBlock, GROUPS ? 1 : (GUIDED ? 2 : 3)) k_pt_shade(PtBatch b, uint32_t d) {
  const uint64_t n = b.qlen[d] < b.cap ? b.qlen[d] : b.cap;
  const float* q = b.qray[d & 1];
  const uint32_t* qp = b.qpath[d & 1];
  float* nq = b.qray[(d + 1) & 1];
  uint32_t* nqp = b.qpath[(d + 1) & 1];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  // Every lane of a warp runs the same number of iterations so the
  // warp-aggregated appends see whole warps.
  const uint64_t nround = (n + stride - 1) / stride;
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  for (uint64_t r = 0; r < nround; ++r) {
    const uint64_t i = r * stride + tid;
    const bool active = i < n;
    bool want_shadow = false, want_next = false;
    uint32_t p = 0;
    float so[3] = {0, 0, 0}, no[3] = {0, 0, 0};
    V3 sd = v3(0, 0, 0), nd = v3(0, 0, 0), sc3 = v3(0, 0, 0);
    float stmax = 0.f, time = 0.f;
    bool want_rec = false;
    V3 rP = v3(0, 0, 0), rN = v3(0, 0, 0), rWi = v3(0, 0, 0);
    float rQ = 0.f, rPb = 0.f;
    float nee_w = 0.f, nee_pb = 0.f;  // TRAIN: the light sample's record weight, BSDF density
    if (active) {
      p = qp[i];
      const V3 D = v3(q[3 * (size_t)b.cap + i], q[4 * (size_t)b.cap + i], q[5 * (size_t)b.cap + i]);
      time = q[7 * (size_t)b.cap + i];
      V3 beta = v3(b.bx[p], b.by[p], b.bz[p]);
      V3 L = v3(b.lx[p], b.ly[p], b.lz[p]);
      if (TRAIN) {  // the radiance before this vertex closes the previous record
        const uint32_t lr = b.last_rec[p];
        if (lr != 0xffffffffu) {
          b.rec[(size_t)(kRMark + 0) * b.rcap + lr] = L.x;
          b.rec[(size_t)(kRMark + 1) * b.rcap + lr] = L.y;
          b.rec[(size_t)(kRMark + 2) * b.rcap + lr] = L.z;
          b.last_rec[p] = 0xffffffffu;
        }
      }
      const float pdf_prev = b.pdf[p];
      const uint64_t key = b.key[p];
      const int32_t prim = b.hprim[i];
      bool cont = false;
      if (prim < 0) {
        if (b.has_env) {
          const float w = pdf_prev == 0.0f ? 1.0f : power_w(pdf_prev, b.sel * kInv4Pi);
          L = add(L, v3(beta.x * b.env[0] * w, beta.y * b.env[1] * w, beta.z * b.env[2] * w));
        }
      } else {
        const int32_t geom = b.hgeom[i];
        Ctx sc;
        uint32_t shid = 0;
        const V3 Ro = v3(q[i], q[(size_t)b.cap + i], q[2 * (size_t)b.cap + i]);
        if (surface_attributes<GROUPS>(b.meshes[geom], prim, b.hu[i], b.hv[i], b.hw[i], Ro, D, b.ht[i], time, sc, shid)) {
          const vmr_shader_std& sh = b.shaders[shid];
          const V3 wi = v3(-D.x, -D.y, -D.z);
          const bool front = dot(sc.Ng, wi) > 0.0f;
          const RGB e = emission(sh);
          const V3 Le = v3(e.c[0], e.c[1], e.c[2]);
          if (front && (Le.x != 0.0f || Le.y != 0.0f || Le.z != 0.0f)) {
            float w = 1.0f;
            const int32_t li = (uint32_t)geom < b.n_geoms ? b.light_of_geom[geom] : -1;
            if (pdf_prev != 0.0f && li >= 0) {
              const PtLight& l = b.lights[li];
              const float t = b.ht[i];
              const float pl = b.sel * (t * t) / (l.area * fabsf(dot(D, sc.Ng)));
              w = power_w(pdf_prev, pl);
            }
            L = add(L, v3(beta.x * Le.x * w, beta.y * Le.y * w, beta.z * Le.z * w));
          }
          const float tw = ((sh.flags & VMR_SH_DIFFUSE_STRENGTH) ? sh.diffuse_strength : 0.0f) +
                           ((sh.flags & VMR_SH_SPEC1_STRENGTH) ? sh.spec1_strength : 0.0f);
          if (d < b.max_depth && tw != 0.0f) {
            if (!front) {  // two-sided: face the incoming ray
              sc.N = v3(-sc.N.x, -sc.N.y, -sc.N.z);
              sc.Ng = v3(-sc.Ng.x, -sc.Ng.y, -sc.Ng.z);
              sc.Poffset = v3(-sc.Poffset.x, -sc.Poffset.y, -sc.Poffset.z);
            }
            V3 Vt = cross(sc.N, sc.DdPdu);
            if (len2(Vt) < 0.1f) Vt = cross(sc.N, sc.DdPdv);
            Vt = normalize(Vt);
            const V3 Ut = normalize(cross(sc.N, Vt));
            const Mat m = material(sh);
            const V3 wil = project(Ut, Vt, sc.N, wi);
            const uint32_t base = 8 * d;
            const int nL = (int)b.nl;
            const bool guided = GUIDED && (m.dw > 0.0f || !m.mirror);
            GMix gm;
            if (guided) gmix_decode(b.gout + i * guide::kGuideOutStride, b.alpha, b.learn_sel != 0, gm);
            // ---- next-event estimation
            if (nL > 0 && (m.dw > 0.0f || !m.mirror)) {
              const float u = rnd(key, base + 0);
              int li = (int)(u * (float)nL);
              if (li > nL - 1) li = nL - 1;
              const float u0 = rnd(key, base + 1), u1 = rnd(key, base + 2);
              const PtLight& l = b.lights[li];
              V3 Ld;
              float dist = 0.f, pl = 0.f;
              bool ok = true;
              if (l.kind == 2) {
                const float z = 1 - 2 * u0;
                const float rr = sqrtf((1 - z * z) > 0.0f ? (1 - z * z) : 0.0f);
                float sp, cp;
                sincos_turns(u1, sp, cp);
                Ld = v3(rr * cp, rr * sp, z);
                pl = b.sel * kInv4Pi;
              } else {
                const V3 p0 = v3(l.p0[0], l.p0[1], l.p0[2]), la = v3(l.a[0], l.a[1], l.a[2]),
                         lb = v3(l.b[0], l.b[1], l.b[2]);
                V3 Pl;
                if (l.kind == 0) {
                  const float su = sqrtf(u0);
                  const float b0 = 1 - su, b1 = su * (1 - u1), b2 = su * u1;
                  Pl = add(add(scale(b0, p0), scale(b1, la)), scale(b2, lb));
                } else {
                  Pl = add(add(p0, scale(u0, la)), scale(u1, lb));
                }
                const V3 Dv = sub(Pl, sc.P);
                dist = length(Dv);
                Ld = normalize(Dv);
                const float cl = dot(Ld, v3(l.N[0], l.N[1], l.N[2]));
                if (!(cl < 0.0f)) ok = false;
                else pl = b.sel * (dist * dist) / (l.area * (-cl));
              }
              if (ok && dot(Ld, sc.Ng) > 0.0f && dot(Ld, sc.N) > 0.0f && pl > 0.0f && !isinf(pl)) {
                const V3 wol = project(Ut, Vt, sc.N, Ld);
                const V3 f = bsdf_f(m, wil, wol);
                const float pbs = bsdf_pdf_pt(m, wil, wol);
                const float pb = guided ? gm.alpha * gmix_pdf(gm, Ld) + (1.0f - gm.alpha) * pbs : pbs;
                const float w = power_w(pl, pb);
                const float k = w / pl;
                const V3 c = v3(beta.x * f.x * l.Le[0] * k, beta.y * f.y * l.Le[1] * k, beta.z * f.z * l.Le[2] * k);
                if (c.x > 0.0f || c.y > 0.0f || c.z > 0.0f) {
                  const V3 o = offset_p(sc, 1);
                  so[0] = o.x; so[1] = o.y; so[2] = o.z;
                  if (l.kind == 2) {
                    sd = Ld;
                    stmax = __int_as_float(0x7f800000);
                  } else {
                    const float sl = dist * 0.9999f;
                    sd = v3(Ld.x * sl, Ld.y * sl, Ld.z * sl);
                    stmax = 1.0f;
                  }
                  sc3 = c;
                  want_shadow = true;
                  if (TRAIN && guided) {
                    // incident radiance x |cos| over the light's density, with
                    // the light's MIS weight: summed with the continuation
                    // records (whose emission carries the other weight) it
                    // estimates the product the guide is fitted to
                    const float lum = 0.2126f * l.Le[0] + 0.7152f * l.Le[1] + 0.0722f * l.Le[2];
                    const float wt = lum * w * fabsf(dot(sc.N, Ld)) / pl;
                    nee_w = isfinite(wt) ? fminf(wt, 1e4f) : 0.f;
                    rN = sc.N;
                    rWi = wi;
                    nee_pb = pbs;
                  }
                }
              }
            }
            // ---- continuation: the guide (probability alpha) or the BSDF
            const float ul = rnd(key, base + 3);
            const float r0 = rnd(key, base + 4), r1 = rnd(key, base + 5);
            V3 wol, wo;
            bool delta = false;
            const bool from_guide = guided && rnd(key, base + 7) < gm.alpha;
            if (from_guide) {
              wo = gmix_sample(gm, ul, r0, r1);
              wol = project(Ut, Vt, sc.N, wo);
            } else if (ul < m.dw) {  // CosineHemisphere (math/sample/sample.go:18-27), float32
              const float r = sqrtf(1.0f - r0);
              float sp, cp;
              sincos_turns(r1, sp, cp);
              wol = v3(r * cp, r * sp, sqrtf(r0));
            } else if (m.mirror) {
              wol = v3(-wil.x, -wil.y, wil.z);
              delta = true;
            } else {  // GGX D(m)cos(m) (microfacetggx.go:82-100): tan(theta_m) = alpha sqrt(r0) / sqrt(1-r0)
              const float a = m.alpha * sqrtf(r0), bq = sqrtf(1.0f - r0);
              const float hyp = sqrtf(a * a + bq * bq);
              const float st = a / hyp, ct = bq / hyp;
              float sp, cp;
              sincos_turns(r1, sp, cp);
              const V3 mh = v3(st * cp, st * sp, ct);
              wol = normalize(sub(scale(2 * fabsf(dot(mh, wil)), mh), wil));
            }
            if (!from_guide) wo = expand(Ut, Vt, sc.N, wol);
            if (dot(wo, sc.Ng) > 0.0f) {
              bool alive = true;
              float pb = 0.0f;
              if (delta) {
                const RGB F = fresnel_kr(m.fr, wil.z);
                beta = v3(beta.x * (m.cs.x * F.c[0]), beta.y * (m.cs.y * F.c[1]), beta.z * (m.cs.z * F.c[2]));
                if (guided) {  // the mirror lobe is taken with probability (1-alpha)*sw
                  const float inv = 1.0f / (1.0f - gm.alpha);
                  beta = v3(beta.x * inv, beta.y * inv, beta.z * inv);
                }
              } else {
                const V3 f = bsdf_f(m, wil, wol);
                pb = bsdf_pdf_pt(m, wil, wol);
                rPb = pb;
                if (guided) pb = gm.alpha * gmix_pdf(gm, wo) + (1.0f - gm.alpha) * pb;
                if (!(pb > 0.0f)) alive = false;
                else beta = v3(beta.x * (f.x / pb), beta.y * (f.y / pb), beta.z * (f.z / pb));
              }
              if (alive && d + 1 >= b.rr_depth) {  // Russian roulette
                float qq = tmax3(beta.x, beta.y, beta.z);
                if (qq > 0.95f) qq = 0.95f;
                const float ur = rnd(key, base + 6);
                if (!(ur < qq)) alive = false;
                else beta = v3(beta.x / qq, beta.y / qq, beta.z / qq);
              }
              if (alive) {
                const V3 o = offset_p(sc, 1);
                no[0] = o.x; no[1] = o.y; no[2] = o.z;
                nd = wo;
                b.pdf[p] = delta ? 0.0f : pb;
                cont = true;
                if (TRAIN && guided && !delta) {
                  want_rec = true;
                  rP = sc.P;
                  rN = sc.N;
                  rWi = wi;
                  rQ = pb;
                }
              }
            }
          }
        }
      }
      b.lx[p] = L.x; b.ly[p] = L.y; b.lz[p] = L.z;
      if (cont) {
        b.bx[p] = beta.x; b.by[p] = beta.y; b.bz[p] = beta.z;
        want_next = true;
      }
    }
    __syncwarp();
    const unsigned long long si = warp_append(&b.slen[d], want_shadow);
    if (want_shadow && si < b.cap) {
      put_ray(b.sray, b.cap, si, so, sd, stmax, time);
      b.spath[si] = p;
      b.scontrib[si] = sc3.x;
      b.scontrib[b.cap + si] = sc3.y;
      b.scontrib[2 * (size_t)b.cap + si] = sc3.z;
      if (TRAIN) {
        const size_t c = b.cap;
        b.snee[si] = rN.x; b.snee[c + si] = rN.y; b.snee[2 * c + si] = rN.z;
        b.snee[3 * c + si] = rWi.x; b.snee[4 * c + si] = rWi.y; b.snee[5 * c + si] = rWi.z;
        b.snee[6 * c + si] = nee_w;
        b.snee[7 * c + si] = nee_pb;
      }
    }
    const unsigned long long ni = warp_append(&b.qlen[d + 1], want_next);
    if (want_next && ni < b.cap) {
      put_ray(nq, b.cap, ni, no, nd, __int_as_float(0x7f800000), time);
      nqp[ni] = p;
    }
    if (TRAIN) {
      const unsigned long long ri = warp_append(&b.rcount[0], want_rec);
      if (want_rec && ri < b.rcap) {
        float* R = b.rec;
        const size_t c = b.rcap;
        const float v[20] = {rP.x, rP.y, rP.z, rN.x, rN.y, rN.z, rWi.x, rWi.y, rWi.z, nd.x, nd.y, nd.z, 0.f, rQ,
                             b.bx[p], b.by[p], b.bz[p], 0.f, 0.f, 0.f};
        for (int k = 0; k < 20; ++k) R[(size_t)k * c + ri] = v[k];
        R[(size_t)kRPath * c + ri] = __uint_as_float(p);
        R[(size_t)kRPb * c + ri] = rPb;
        b.last_rec[p] = (uint32_t)ri;
      }
    }
  }
}

// Training weights: incident radiance along the sampled direction,
// (L_final - L_mark) / beta per channel, as luminance, times |cos| with the
// shading normal, over the density it was sampled with (clamped to 1e4).
__global__ void __launch_bounds__(kPtBlock) k_pt_targets(PtBatch b) {
  const uint64_t n = b.rcount[0] < b.rcap ? b.rcount[0] : b.rcap;
  const size_t c = b.rcap;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = __float_as_uint(b.rec[(size_t)kRPath * c + i]);
    if (p == kNoPath) continue;  // a light-sample record: weight already set
    const float Lf[3] = {b.lx[p], b.ly[p], b.lz[p]};
    float lin[3];
    for (int k = 0; k < 3; ++k) {
      const float bt = b.rec[(size_t)(kRBeta + k) * c + i];
      const float v = bt > 0.f ? (Lf[k] - b.rec[(size_t)(kRMark + k) * c + i]) / bt : 0.f;
      lin[k] = v > 0.f ? v : 0.f;
    }
    const float lum = 0.2126f * lin[0] + 0.7152f * lin[1] + 0.0722f * lin[2];
    const float q = b.rec[(size_t)kRQ * c + i];
    // the product the vertex integrates: incident radiance x |cos| with the normal
    const float cs = fabsf(b.rec[(size_t)kRN * c + i] * b.rec[(size_t)kROm * c + i] +
                           b.rec[(size_t)(kRN + 1) * c + i] * b.rec[(size_t)(kROm + 1) * c + i] +
                           b.rec[(size_t)(kRN + 2) * c + i] * b.rec[(size_t)(kROm + 2) * c + i]);
    float w = q > 0.f ? lum * cs / q : 0.f;
    w = isfinite(w) ? fminf(w, 1e4f) : 0.f;
    b.rec[(size_t)kRW * c + i] = w;
  }
}

// Records of training step s: [s*B, s*B + B) clipped to the batch's count.
// Training step s of S takes records s, s + S, s + 2S, ... (every depth and
// pixel of the batch, not one block of queue order), at most B of them.
__global__ void k_pt_train_count(const unsigned long long* rcount, uint32_t rcap, uint64_t s, uint64_t S,
                                 uint64_t B, unsigned long long* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const uint64_t n = rcount[0] < rcap ? rcount[0] : rcap;
  const uint64_t m = n > s ? (n - s + S - 1) / S : 0;
  *out = m < B ? m : B;
}

// Unoccluded shadow rays add their contribution, in queue order (each path
// has at most one shadow ray per bounce, so no two threads touch one path).
// TRAIN: an unoccluded light sample of a guided vertex becomes a training
// record (direction toward the light, weight from the shade kernel; its path
// column is the marker kNoPath so the targets pass keeps the weight).
template <bool TRAIN>
__global__ void __launch_bounds__(kPtBlock) k_pt_resolve(PtBatch b, uint32_t d) {
  const uint64_t n = b.slen[d] < b.cap ? b.slen[d] : b.cap;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t nround = (n + stride - 1) / stride;
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  for (uint64_t r = 0; r < nround; ++r) {
    const uint64_t i = r * stride + tid;
    const bool lit = i < n && b.shit[i] < 0;
    if (lit) {
      const uint32_t p = b.spath[i];
      b.lx[p] = b.lx[p] + b.scontrib[i];
      b.ly[p] = b.ly[p] + b.scontrib[b.cap + i];
      b.lz[p] = b.lz[p] + b.scontrib[2 * (size_t)b.cap + i];
    }
    if (TRAIN) {
      const size_t c = b.cap;
      const float wt = lit ? b.snee[6 * c + i] : 0.f;
      const unsigned long long ri = warp_append(&b.rcount[0], wt > 0.f);
      if (wt > 0.f && ri < b.rcap) {
        const float* sr = b.sray;
        const V3 dir = normalize(v3(sr[3 * c + i], sr[4 * c + i], sr[5 * c + i]));
        const float v[13] = {sr[i], sr[c + i], sr[2 * c + i], b.snee[i], b.snee[c + i], b.snee[2 * c + i],
                             b.snee[3 * c + i], b.snee[4 * c + i], b.snee[5 * c + i], dir.x, dir.y, dir.z, wt};
        float* R = b.rec;
        const size_t rc = b.rcap;
        for (int k = 0; k < 13; ++k) R[(size_t)k * rc + ri] = v[k];
        R[(size_t)kRPath * rc + ri] = __uint_as_float(kNoPath);
        R[(size_t)kRPb * rc + ri] = b.snee[7 * c + i];
      }
    }
  }
}

__global__ void __launch_bounds__(kPtBlock) k_pt_accumulate(PtBatch b) {
  const uint32_t iters = b.it->iters;
  for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < b.npix; pix += gridDim.x * blockDim.x) {
    float f[3] = {b.fb[pix * 3], b.fb[pix * 3 + 1], b.fb[pix * 3 + 2]};
    double g[3] = {0, 0, 0};
    if (b.fb64)
      for (int k = 0; k < 3; ++k) g[k] = b.fb64[(size_t)pix * 3 + k];
    for (uint32_t t = 0; t < iters; ++t) {
      const uint64_t s = (uint64_t)t * b.npix + pix;
      const uint32_t i = b.it->iter0 + t;  // 0-based: the exact running mean
      const float L[3] = {b.lx[s], b.ly[s], b.lz[s]};
      for (int k = 0; k < 3; ++k) {
        f[k] = (f[k] * (float)i + L[k]) / (float)(i + 1);
        g[k] = (g[k] * (double)i + (double)L[k]) / (double)(i + 1);
      }
    }
    for (int k = 0; k < 3; ++k) b.fb[pix * 3 + k] = f[k];
    if (b.fb64)
      for (int k = 0; k < 3; ++k) b.fb64[(size_t)pix * 3 + k] = g[k];
  }
}

// Ray counts and traversal status of the batch, kept across batches (the
// next batch clears the per-launch scratch).
__global__ void k_pt_tally(PtBatch b) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  unsigned long long r = 0, s = 0;
  int st = *b.status;
  for (uint32_t d = 0; d <= b.max_depth; ++d) {
    r += b.qlen[d];
    s += b.slen[d];
    st = max(st, max(b.scr[2 * d].status, b.scr[2 * d + 1].status));
  }
  b.totals[0] += r;
  b.totals[1] += s;
  *b.status = st;
  if (b.rcount) b.rcount[1] += b.rcount[0] < b.rcap ? b.rcount[0] : b.rcap;
}

// ---------------------------------------------------- host: light table ---
// Host float math in the oracle's operation order (compiled without
// contraction), so the device sees the same light table as the oracle.
struct HV {
  float x, y, z;
};
inline HV hv(const float* p) { return HV{p[0], p[1], p[2]}; }
inline HV hsub(HV a, HV b) { return HV{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline HV hcross(HV a, HV b) { return HV{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float hlen(HV a) { return std::sqrt((a.x * a.x + a.y * a.y) + a.z * a.z); }
inline HV hnrm(HV a) {
  const float r = 1.0f / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return HV{a.x * r, a.y * r, a.z * r};
}
void host_emission(const vmr_shader_std& s, float out[3]) {
  out[0] = out[1] = out[2] = 0.0f;
  if (!(s.flags & VMR_SH_EMISSION_STRENGTH)) return;
  for (int k = 0; k < 3; ++k)
    out[k] = ((s.flags & VMR_SH_EMISSION_COLOUR) ? s.emission_colour[k] : 0.0f) * s.emission_strength;
}

int pfail(vmr_ctx* ctx, int code, const std::string& msg) {
  ctx->err = msg;
  return code;
}

#define PCUDA(x)                                                              \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) return pfail(ctx, VMR_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

// Launches one batch's stages on the context's stream (also used while
// capturing the graph).  Every count is read on the device.
// Reordering of the wavefront's queues before their traces
// (VMR_PATH_SORT_QUEUES, batches of at least kSortMinRays paths): the rays of
// a queue are gathered
// into a key-ordered copy (direction class + Morton cell of the origin,
// raysort.cu) and the traversal writes each hit back at its queue position,
// so nothing downstream sees the order.
struct PtSort {
  bool on = false;
  int bits = 4;
  float bounds[6] = {0, 0, 0, 0, 0, 0};
  uint32_t* keys = nullptr;
  uint32_t* order = nullptr;
  uint32_t* hist = nullptr;
  float* rays = nullptr;  // 8 * cap floats
};

// The flattened scene (vmr::flat_scene) the bounce loop traces instead of
// the two-level scene: one mesh over every triangle, its hits mapped back to
// (geom, the geom's leaf position) by k_flat_remap.
struct PtFlat {
  const DMesh* mesh = nullptr;
  const uint32_t* map = nullptr;  // [2 * n]: geom, then the geom's leaf position
  uint32_t n = 0;
};

// Closest hits of a flattened-scene trace back to the scene's ids: the flat
// mesh's leaf position e becomes geom map[e] and triangle map[n + e].
__global__ void __launch_bounds__(kPtBlock) k_flat_remap(const uint32_t* __restrict__ map, uint32_t n,
                                                          int32_t* prim, int32_t* geom,
                                                          const unsigned long long* qlen, uint64_t cap) {
  const uint64_t m = *qlen < cap ? *qlen : cap;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
    const int32_t e = prim[i];
    if (e >= 0 && (uint32_t)e < n) {
      geom[i] = (int32_t)__ldg(map + e);
      prim[i] = (int32_t)__ldg(map + n + e);
    } else {
      geom[i] = -1;
    }
  }
}

int launch_batch(vmr_ctx* ctx, const PtBatch& b, const DTop& top, DScratch* scr, int grid, bool guided, bool train,
                 const guide::GuideRows& grows, const PtSort& srt, const PtFlat& flat) {
  cudaStream_t st = ctx->stream;
  auto sort_queue = [&](TraceLaunch& l) -> int {
    const size_t c = b.cap;
    const float* f = srt.rays;
    const RaySoA sorted{f, f + c, f + 2 * c, f + 3 * c, f + 4 * c, f + 5 * c, f + 6 * c, f + 7 * c};
    const int e = launch_ray_sort(l.rays, c, srt.bounds, srt.bits, srt.keys, srt.hist, srt.order, sorted, st, l.n_dev);
    l.rays = sorted;
    l.order = srt.order;
    return e;
  };
  const size_t nq = kPtMaxDepth + 2, ns = kPtMaxDepth + 1;
  PCUDA(cudaMemsetAsync(b.qlen, 0, nq * sizeof(unsigned long long), st));
  PCUDA(cudaMemsetAsync(b.slen, 0, ns * sizeof(unsigned long long), st));
  PCUDA(cudaMemsetAsync(scr, 0, sizeof(DScratch) * 2 * (b.max_depth + 1), st));
  if (train) PCUDA(cudaMemsetAsync(b.rcount, 0, sizeof(unsigned long long), st));
  if (b.cam_nkeys >= 2) k_pt_generate<true><<<grid, kPtBlock, 0, st>>>(b);
  else k_pt_generate<false><<<grid, kPtBlock, 0, st>>>(b);
  PCUDA(cudaGetLastError());
  for (uint32_t d = 0; d <= b.max_depth; ++d) {
    TraceLaunch l{};
    l.rays = RaySoA{b.qray[d & 1], b.qray[d & 1] + b.cap, b.qray[d & 1] + 2 * (size_t)b.cap,
                    b.qray[d & 1] + 3 * (size_t)b.cap, b.qray[d & 1] + 4 * (size_t)b.cap,
                    b.qray[d & 1] + 5 * (size_t)b.cap, b.qray[d & 1] + 6 * (size_t)b.cap,
                    b.qray[d & 1] + 7 * (size_t)b.cap};
    l.hits = HitSoA{b.hprim, b.hgeom, b.ht, b.hu, b.hv, b.hw};
    l.n = b.cap;
    l.n_dev = &b.qlen[d];
    l.scratch = scr + 2 * d;
    l.stream = st;
    l.kernel = ctx->tuning.kernel;
    l.walk_tail = ctx->tuning.walk_tail;
    l.grid = ctx->tuning.blocks_per_sm;
    if (b.n_jobs) {
      l.ray_path = b.qpath[d & 1];
      l.path_geom = b.pgeom;
    }
    // camera rays are traced in pixel order (already coherent)
    if (srt.on && d > 0 && sort_queue(l) != 0) return pfail(ctx, VMR_ERR_CUDA, "ray sort launch failed");
    if (flat.mesh) {
      if (launch_trace_mesh(*flat.mesh, l) != 0) return pfail(ctx, VMR_ERR_CUDA, "trace launch failed");
      k_flat_remap<<<grid, kPtBlock, 0, st>>>(flat.map, flat.n, b.hprim, b.hgeom, &b.qlen[d], b.cap);
      PCUDA(cudaGetLastError());
    } else if (launch_trace_scene(top, l) != 0) {
      return pfail(ctx, VMR_ERR_CUDA, "trace launch failed");
    }
    // vertices past the guided depth sample the BSDF alone (and record nothing)
    const bool gd = guided && d < b.gdepth;
    if (gd) {
      if (b.groups) k_pt_prep<true><<<grid, kPtBlock, 0, st>>>(b, d);
      else k_pt_prep<false><<<grid, kPtBlock, 0, st>>>(b, d);
      PCUDA(cudaGetLastError());
      guide::GuideRows r = grows;
      r.n_dev = &b.qlen[d];
      if (guide::launch_infer(r, ctx->guide.wf.p, b.gout, ctx->guide.err.as<int>(), grid / 8, st) != 0)
        return pfail(ctx, VMR_ERR_CUDA, "guide inference launch failed");
      if (b.groups) {
        if (train) k_pt_shade<true, true, true><<<grid, kPtBlock, 0, st>>>(b, d);
        else k_pt_shade<true, false, true><<<grid, kPtBlock, 0, st>>>(b, d);
      } else {
        if (train) k_pt_shade<true, true, false><<<grid, kPtBlock, 0, st>>>(b, d);
        else k_pt_shade<true, false, false><<<grid, kPtBlock, 0, st>>>(b, d);
      }
    } else if (b.groups) {
      k_pt_shade<false, false, true><<<grid, kPtBlock, 0, st>>>(b, d);
    } else {
      k_pt_shade<false, false, false><<<grid, kPtBlock, 0, st>>>(b, d);
    }
    PCUDA(cudaGetLastError());
    if (d < b.max_depth) {
      TraceLaunch s{};
      s.rays = RaySoA{b.sray, b.sray + b.cap, b.sray + 2 * (size_t)b.cap, b.sray + 3 * (size_t)b.cap,
                      b.sray + 4 * (size_t)b.cap, b.sray + 5 * (size_t)b.cap, b.sray + 6 * (size_t)b.cap,
                      b.sray + 7 * (size_t)b.cap};
      s.hits = HitSoA{b.shit, nullptr, nullptr, nullptr, nullptr, nullptr};
      s.n = b.cap;
      s.n_dev = &b.slen[d];
      s.any_hit = 1;
      s.scratch = scr + 2 * d + 1;
      s.stream = st;
      s.kernel = ctx->tuning.kernel;
      s.walk_tail = ctx->tuning.walk_tail;
      s.grid = ctx->tuning.blocks_per_sm;
      if (b.n_jobs) {
        s.ray_path = b.spath;
        s.path_geom = b.pgeom;
      }
      if (srt.on && sort_queue(s) != 0) return pfail(ctx, VMR_ERR_CUDA, "ray sort launch failed");
      // shadow rays need hit or miss only: the flat mesh's prim is enough
      if ((flat.mesh ? launch_trace_mesh(*flat.mesh, s) : launch_trace_scene(top, s)) != 0)
        return pfail(ctx, VMR_ERR_CUDA, "trace launch failed");
      if (train && gd) k_pt_resolve<true><<<grid, kPtBlock, 0, st>>>(b, d);
      else k_pt_resolve<false><<<grid, kPtBlock, 0, st>>>(b, d);
      PCUDA(cudaGetLastError());
    }
  }
  k_pt_accumulate<<<grid, kPtBlock, 0, st>>>(b);
  PCUDA(cudaGetLastError());
  if (train) {
    k_pt_targets<<<grid, kPtBlock, 0, st>>>(b);
    PCUDA(cudaGetLastError());
  }
  k_pt_tally<<<1, 32, 0, st>>>(b);
  PCUDA(cudaGetLastError());
  return VMR_OK;
}

}  // namespace
}  // namespace vmr

extern "C" {

int vmr_set_quad_lights(vmr_ctx* ctx, const vmr_quad_light* lights, uint32_t n) {
  if (!ctx || (n && !lights)) return VMR_ERR_INVALID;
  ctx->render.quads.assign(lights, lights + n);
  return VMR_OK;
}

int vmr_set_env_light(vmr_ctx* ctx, const float radiance[3]) {
  if (!ctx || !radiance) return VMR_ERR_INVALID;
  for (int k = 0; k < 3; ++k) {
    if (!(radiance[k] >= 0.0f) || std::isinf(radiance[k]))
      return vmr::pfail(ctx, VMR_ERR_INVALID, "environment radiance must be finite and non-negative");
    ctx->render.env[k] = radiance[k];
  }
  return VMR_OK;
}

// The extended path tracer over the context's scene (jobs == nullptr) or
// over batched jobs (each path traces only its job's mesh; lights: the
// environment).  fb: the scene's image; jobs: each job's own image.
static int render_path_impl(vmr_ctx* ctx, const vmr_path_params* p, float* fb, vmr_path_stats* stats,
                            const vmr_path_job* jobs, uint32_t n_jobs) {
  using namespace vmr;
  if (!ctx || !p || (!fb && !jobs)) return VMR_ERR_INVALID;
  if (ctx->device < 0) return pfail(ctx, VMR_ERR_UNSUPPORTED, "host-only context cannot render");
  std::vector<uint32_t> used_geoms;
  uint64_t npix_jobs = 0;
  if (!jobs) {
    if (!ctx->top.valid) return pfail(ctx, VMR_ERR_INVALID, "no scene: call vmr_scene_build first");
    if (!ctx->render.has_camera) return pfail(ctx, VMR_ERR_INVALID, "no camera");
    if (p->width == 0 || p->height == 0 || p->width > 4096 || p->height > 4096)
      return pfail(ctx, VMR_ERR_INVALID, "image size must be in [1, 4096] (RasterXY uses m = 12)");
    if (p->row_count && (p->row_begin >= p->height || p->row_count > p->height - p->row_begin))
      return pfail(ctx, VMR_ERR_INVALID, "row band outside the image");
    if (!p->row_count && p->row_begin) return pfail(ctx, VMR_ERR_INVALID, "row_begin without row_count");
    if (p->row_count && (p->flags & VMR_PATH_TRAIN))
      return pfail(ctx, VMR_ERR_UNSUPPORTED, "a row band does not train the guide (it would see its rows only)");
    used_geoms = ctx->top.host.geom_order;
  } else {
    if (n_jobs == 0) return VMR_OK;
    if (p->flags & VMR_PATH_GUIDED) return pfail(ctx, VMR_ERR_UNSUPPORTED, "batched jobs render without the guide");
    if (p->fb64) return pfail(ctx, VMR_ERR_UNSUPPORTED, "batched jobs have no float64 images");
    for (uint32_t k = 0; k < n_jobs; ++k) {
      const vmr_path_job& jb = jobs[k];
      if (!jb.fb) return pfail(ctx, VMR_ERR_INVALID, "a job has no image buffer");
      if (jb.width == 0 || jb.height == 0 || jb.width > 4096 || jb.height > 4096)
        return pfail(ctx, VMR_ERR_INVALID, "job image size must be in [1, 4096] (RasterXY uses m = 12)");
      if (jb.geom >= ctx->meshes.size()) return pfail(ctx, VMR_ERR_INVALID, "job geom out of range");
      if (!(jb.camera.radius >= 0.0f)) return pfail(ctx, VMR_ERR_INVALID, "job camera radius must be >= 0");
      used_geoms.push_back(jb.geom);
      npix_jobs += (uint64_t)jb.width * jb.height;
    }
    if (npix_jobs > 0xffffffffull) return pfail(ctx, VMR_ERR_INVALID, "too many job pixels");
  }
  if (p->max_depth > (uint32_t)kPtMaxDepth) return pfail(ctx, VMR_ERR_INVALID, "max_depth must be <= 32");
  auto& R = ctx->render;
  // The geoms whose shading a hit reads: a GeomInstance shades as the geom
  // it instances, a Proc's hits report its children.
  std::vector<uint32_t> shaded;
  for (uint32_t g : used_geoms) {
    const auto& mr = ctx->meshes[g];
    if (jobs && (mr->host.group || mr->xkeys.size() >= 2))
      return pfail(ctx, VMR_ERR_UNSUPPORTED,
                   "batched path jobs take meshes, spheres and one-matrix transforms (instances, Procs and "
                   "transform keys render in one-scene calls)");
    if (mr->host.group == 1) shaded.push_back(mr->children[0]);
    else if (mr->host.group == 2) shaded.insert(shaded.end(), mr->children.begin(), mr->children.end());
    else shaded.push_back(g);
  }
  for (uint32_t g : shaded) {
    const auto& mr = ctx->meshes[g];
    if (mr->host.motion() && mr->aidx.p == nullptr)
      return pfail(ctx, VMR_ERR_INVALID, "a motion mesh in the scene has no shading (vmr_mesh_set_shading)");
    for (uint32_t sid : mr->shader_list) {
      if (sid >= R.shaders.size()) return pfail(ctx, VMR_ERR_INVALID, "mesh shader id out of range");
      if (R.shaders[sid].flags & VMR_SH_DEBUG)
        return pfail(ctx, VMR_ERR_UNSUPPORTED, "DebugShader renders in reference mode (vmr_render)");
    }
  }
  // Light list: TriLights, quad lights, environment.
  const uint32_t n_geoms = (uint32_t)ctx->meshes.size();
  std::vector<PtLight> lights;
  std::vector<int32_t> log(std::max<uint32_t>(1, n_geoms), -1);
  for (const auto& t : R.lights) {
    if (jobs) break;  // batched jobs: the environment only
    if (t.shader >= R.shaders.size()) return pfail(ctx, VMR_ERR_INVALID, "light shader out of range");
    PtLight l{};
    l.kind = 0;
    std::memcpy(l.p0, t.p0, 12);
    std::memcpy(l.a, t.p1, 12);
    std::memcpy(l.b, t.p2, 12);
    const HV c = hcross(hsub(hv(t.p1), hv(t.p0)), hsub(hv(t.p2), hv(t.p0)));
    const HV N = hnrm(c);
    l.N[0] = N.x; l.N[1] = N.y; l.N[2] = N.z;
    l.area = 0.5f * hlen(c);
    host_emission(R.shaders[t.shader], l.Le);
    l.geom = (int32_t)t.geom;
    if (t.geom < n_geoms) log[t.geom] = (int32_t)lights.size();
    lights.push_back(l);
  }
  for (const auto& qd : R.quads) {
    if (jobs) break;
    if (qd.shader >= R.shaders.size()) return pfail(ctx, VMR_ERR_INVALID, "quad light shader out of range");
    PtLight l{};
    l.kind = 1;
    std::memcpy(l.p0, qd.p0, 12);
    std::memcpy(l.a, qd.e1, 12);
    std::memcpy(l.b, qd.e2, 12);
    const HV c = hcross(hv(qd.e1), hv(qd.e2));
    const HV N = hnrm(c);
    l.N[0] = N.x; l.N[1] = N.y; l.N[2] = N.z;
    l.area = hlen(c);
    host_emission(R.shaders[qd.shader], l.Le);
    l.geom = (int32_t)qd.geom;
    if (qd.geom < n_geoms) log[qd.geom] = (int32_t)lights.size();
    lights.push_back(l);
  }
  const bool has_env = R.env[0] != 0.0f || R.env[1] != 0.0f || R.env[2] != 0.0f;
  if (has_env) {
    PtLight l{};
    l.kind = 2;
    std::memcpy(l.Le, R.env, 12);
    l.geom = -1;
    lights.push_back(l);
  }
  const uint32_t nl = (uint32_t)lights.size();
  const std::vector<RMesh> rm = rmesh_table(ctx);
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  const uint32_t band = (!jobs && p->row_count) ? p->row_count : p->height;
  const uint32_t npix = jobs ? (uint32_t)npix_jobs : p->width * band;
  // Default 16M paths per batch (about 3 GB of queues, allocated only when
  // a call has that many paths): every bounce's launches end in a tail of
  // long paths, which a larger batch amortises (sphere grid 1920x1080, 8
  // spp: 80.7 ms at 2M, 66.5 ms at 8M, 16M 3-4% faster than 8M); a one-scene
  // render uses the context's tuned capacity when it has one
  // (vmr_autotune_path, vmr_set_path_batch).
  const uint32_t per_batch = p->max_batch_samples     ? p->max_batch_samples
                             : (!jobs && ctx->render.path_batch) ? ctx->render.path_batch
                                                                 : (16u << 20);
  uint32_t ipb = std::max<uint32_t>(1, per_batch / npix);
  if (p->iter_count > 0 && ipb > p->iter_count) ipb = p->iter_count;
  const uint64_t cap = (uint64_t)ipb * npix;
  if (cap > 0xffffffffull) return pfail(ctx, VMR_ERR_INVALID, "batch too large");
  const bool guided = (p->flags & VMR_PATH_GUIDED) != 0;
  const bool train = guided && (p->flags & VMR_PATH_TRAIN) != 0;
  if (guided) {
    const int rc = guide::ensure_ready(ctx);
    if (rc != VMR_OK) return rc;
    guide::prepare_kernels();
  }
  const bool learn_sel = !(p->flags & VMR_PATH_FIXED_SELECTION);
  const float alpha = p->guide_fraction > 0.0f ? p->guide_fraction : (learn_sel ? 0.9f : 0.5f);
  if (guided && !(alpha < 1.0f)) return pfail(ctx, VMR_ERR_INVALID, "guide_fraction must be below 1");
  // continuation and light-sample records: at most two per vertex
  const uint64_t rcap = train ? std::min<uint64_t>(2 * cap * std::max<uint32_t>(1, p->max_depth), 0xffffffffull) : 0;
  const uint32_t tsteps = p->train_steps ? p->train_steps : 4;
  const uint32_t tbatch = p->train_batch ? p->train_batch : 65536;
  const float tlr = p->train_lr > 0.0f ? p->train_lr : 1e-3f;
  // scene bounds for the guide's inputs
  float glo[3] = {INFINITY, INFINITY, INFINITY}, ghi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint32_t g : ctx->top.host.geom_order)
    for (int k = 0; k < 3; ++k) {
      glo[k] = std::min(glo[k], ctx->meshes[g]->bounds6[k]);
      ghi[k] = std::max(ghi[k], ctx->meshes[g]->bounds6[3 + k]);
    }
  for (int k = 0; k < 3; ++k)
    if (!(ghi[k] > glo[k])) ghi[k] = glo[k] + 1.0f;
  // One device block, carved.
  size_t bytes = 0;
  auto carve = [&](size_t nb) { size_t o = bytes; bytes += (nb + 255) / 256 * 256; return o; };
  const size_t o_state = carve(cap * 7 * 4), o_key = carve(cap * 8), o_q0 = carve(cap * 8 * 4),
               o_q1 = carve(cap * 8 * 4), o_qp0 = carve(cap * 4), o_qp1 = carve(cap * 4), o_hit = carve(cap * 6 * 4),
               o_s = carve(cap * 8 * 4), o_sp = carve(cap * 4), o_sc = carve(cap * 3 * 4), o_sh = carve(cap * 4),
               o_cnt = carve((2 * kPtMaxDepth + 6) * 8), o_scr = carve(sizeof(DScratch) * 2 * (kPtMaxDepth + 1)),
               o_it = carve(sizeof(PtIter)), o_fb = carve((size_t)npix * 3 * 4),
               o_fb64 = carve(p->fb64 ? (size_t)npix * 3 * 8 : 0), o_mesh = carve(rm.size() * sizeof(RMesh)),
               o_light = carve(std::max<size_t>(1, lights.size()) * sizeof(PtLight)),
               o_shader = carve(std::max<size_t>(1, R.shaders.size()) * sizeof(vmr_shader_std)),
               o_log = carve(log.size() * 4), o_grow = carve(guided ? cap * 9 * 4 : 0),
               o_gout = carve(guided ? cap * guide::kGuideOutStride * 4 : 0), o_rec = carve(rcap * kRecCols * 4),
               o_last = carve(train ? cap * 4 : 0), o_rcnt = carve(32), o_snee = carve(train ? cap * 8 * 4 : 0),
               o_jobs = carve(jobs ? n_jobs * sizeof(PtJob) : 0), o_pgeom = carve(jobs ? cap * 4 : 0);
  // queue reordering (not for jobs: a key-ordered queue would mix the jobs'
  // meshes inside a warp)
  const bool sort_on = !jobs && (p->flags & VMR_PATH_SORT_QUEUES) && cap >= kSortMinRays;
  const size_t o_sort = carve(sort_on ? cap * 4 * (2 + 8) + sizeof(uint32_t) * kSortBucketsMax : 0);
  PCUDA(R.ptbuf.ensure(bytes));
  char* base = R.ptbuf.as<char>();
  uint64_t fwd[52], inv[52];
  raster_tables_m12(fwd, inv);
  PCUDA(cudaMemcpyToSymbolAsync(c_raster_fwd, fwd, sizeof(fwd), 0, cudaMemcpyHostToDevice, st));
  PCUDA(cudaMemcpyToSymbolAsync(c_raster_inv, inv, sizeof(inv), 0, cudaMemcpyHostToDevice, st));
  PCUDA(cudaMemcpyAsync(base + o_mesh, rm.data(), rm.size() * sizeof(RMesh), cudaMemcpyHostToDevice, st));
  if (!lights.empty())
    PCUDA(cudaMemcpyAsync(base + o_light, lights.data(), lights.size() * sizeof(PtLight), cudaMemcpyHostToDevice, st));
  if (!R.shaders.empty())
    PCUDA(cudaMemcpyAsync(base + o_shader, R.shaders.data(), R.shaders.size() * sizeof(vmr_shader_std),
                          cudaMemcpyHostToDevice, st));
  PCUDA(cudaMemcpyAsync(base + o_log, log.data(), log.size() * 4, cudaMemcpyHostToDevice, st));
  // batched jobs: their images end to end in the pixel arena, and the job table
  std::vector<float> arena;
  std::vector<PtJob> jtab;
  if (jobs) {
    arena.resize((size_t)npix * 3);
    uint32_t pix0 = 0;
    for (uint32_t k = 0; k < n_jobs; ++k) {
      PtJob j{};
      j.cam = camera_round_trip(jobs[k].camera);
      j.width = jobs[k].width;
      j.height = jobs[k].height;
      j.npix = j.width * j.height;
      j.geom = jobs[k].geom;
      j.pix0 = pix0;
      std::memcpy(arena.data() + (size_t)pix0 * 3, jobs[k].fb, (size_t)j.npix * 12);
      pix0 += j.npix;
      jtab.push_back(j);
    }
    PCUDA(cudaMemcpyAsync(base + o_jobs, jtab.data(), jtab.size() * sizeof(PtJob), cudaMemcpyHostToDevice, st));
    PCUDA(cudaMemcpyAsync(base + o_fb, arena.data(), arena.size() * 4, cudaMemcpyHostToDevice, st));
  } else {
    PCUDA(cudaMemcpyAsync(base + o_fb, fb, (size_t)npix * 3 * 4, cudaMemcpyHostToDevice, st));
  }
  if (p->fb64) PCUDA(cudaMemcpyAsync(base + o_fb64, p->fb64, (size_t)npix * 3 * 8, cudaMemcpyHostToDevice, st));
  PtBatch b{};
  b.width = p->width;
  b.height = p->height;
  b.npix = npix;
  b.pix0 = (!jobs && p->row_count) ? p->row_begin * p->width : 0u;
  b.nl = nl;
  b.max_depth = p->max_depth;
  b.rr_depth = p->rr_depth;
  b.has_env = has_env ? 1u : 0u;
  b.cap = (uint32_t)cap;
  std::memcpy(b.env, R.env, 12);
  b.sel = nl > 0 ? 1.0f / (float)nl : 0.0f;
  b.groups = 0u;
  for (const RMesh& r : rm) b.groups |= (r.outer_nkeys != 0 || r.xf_nkeys >= 2) ? 1u : 0u;
  b.seed = p->seed;
  b.cam = R.cam_used;
  b.cam_nkeys = R.cam_keys.size() >= 2 ? (uint32_t)R.cam_keys.size() : 0u;
  b.cam_keys = b.cam_nkeys ? R.dcam_keys.as<const anim::Decomp>() : nullptr;
  b.filt = PixFilter{R.filter_n ? R.filter.as<const double>() : nullptr, R.filter_n, R.filter_w};
  b.it = reinterpret_cast<const PtIter*>(base + o_it);
  b.shaders = reinterpret_cast<const vmr_shader_std*>(base + o_shader);
  b.lights = reinterpret_cast<const PtLight*>(base + o_light);
  b.meshes = reinterpret_cast<const RMesh*>(base + o_mesh);
  b.light_of_geom = reinterpret_cast<const int32_t*>(base + o_log);
  b.n_geoms = n_geoms;
  float* stt = reinterpret_cast<float*>(base + o_state);
  b.bx = stt; b.by = stt + cap; b.bz = stt + 2 * cap;
  b.lx = stt + 3 * cap; b.ly = stt + 4 * cap; b.lz = stt + 5 * cap;
  b.pdf = stt + 6 * cap;
  b.key = reinterpret_cast<unsigned long long*>(base + o_key);
  b.qray[0] = reinterpret_cast<float*>(base + o_q0);
  b.qray[1] = reinterpret_cast<float*>(base + o_q1);
  b.qpath[0] = reinterpret_cast<uint32_t*>(base + o_qp0);
  b.qpath[1] = reinterpret_cast<uint32_t*>(base + o_qp1);
  int32_t* hit = reinterpret_cast<int32_t*>(base + o_hit);
  b.hprim = hit;
  b.hgeom = hit + cap;
  b.ht = reinterpret_cast<float*>(hit + 2 * cap);
  b.hu = reinterpret_cast<float*>(hit + 3 * cap);
  b.hv = reinterpret_cast<float*>(hit + 4 * cap);
  b.hw = reinterpret_cast<float*>(hit + 5 * cap);
  b.sray = reinterpret_cast<float*>(base + o_s);
  b.spath = reinterpret_cast<uint32_t*>(base + o_sp);
  b.scontrib = reinterpret_cast<float*>(base + o_sc);
  b.shit = reinterpret_cast<int32_t*>(base + o_sh);
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(base + o_cnt);
  b.qlen = cnt;
  b.slen = cnt + kPtMaxDepth + 2;
  b.totals = cnt + 2 * kPtMaxDepth + 3;
  b.status = reinterpret_cast<int*>(cnt + 2 * kPtMaxDepth + 5);
  b.fb = reinterpret_cast<float*>(base + o_fb);
  b.fb64 = p->fb64 ? reinterpret_cast<double*>(base + o_fb64) : nullptr;
  DScratch* scr = reinterpret_cast<DScratch*>(base + o_scr);
  b.scr = scr;
  b.alpha = alpha;
  b.learn_sel = learn_sel ? 1u : 0u;
  b.gdepth = p->guide_depth ? p->guide_depth : 0xffffffffu;
  std::memcpy(b.glo, glo, 12);
  b.grow = guided ? reinterpret_cast<float*>(base + o_grow) : nullptr;
  b.gout = guided ? reinterpret_cast<float*>(base + o_gout) : nullptr;
  b.rec = train ? reinterpret_cast<float*>(base + o_rec) : nullptr;
  b.rcap = (uint32_t)rcap;
  b.rcount = train ? reinterpret_cast<unsigned long long*>(base + o_rcnt) : nullptr;
  b.last_rec = train ? reinterpret_cast<uint32_t*>(base + o_last) : nullptr;
  b.snee = train ? reinterpret_cast<float*>(base + o_snee) : nullptr;
  b.jobs = jobs ? reinterpret_cast<const PtJob*>(base + o_jobs) : nullptr;
  b.n_jobs = jobs ? n_jobs : 0u;
  b.pgeom = jobs ? reinterpret_cast<uint32_t*>(base + o_pgeom) : nullptr;
  PtFlat flat;
  if (!jobs && !(p->flags & VMR_PATH_TWO_LEVEL) && (ctx->tuning.kernel & kKernelWhileWhile)) {
    int fs = VMR_OK;
    flat.mesh = flat_scene(ctx, &flat.map, &flat.n, &fs);
    if (fs != VMR_OK) return fs;
  }
  PtSort srt;
  if (sort_on) {
    srt.on = true;
    srt.bits = ctx->tuning.sort_bits ? ctx->tuning.sort_bits : 4;
    for (int k = 0; k < 3; ++k) {
      srt.bounds[k] = glo[k];
      srt.bounds[3 + k] = ghi[k];
    }
    srt.keys = reinterpret_cast<uint32_t*>(base + o_sort);
    srt.order = srt.keys + cap;
    srt.rays = reinterpret_cast<float*>(srt.order + cap);
    srt.hist = reinterpret_cast<uint32_t*>(srt.rays + cap * 8);
  }
  // the traversal's view: the scene's top level, or for jobs only the mesh
  // table (each ray enters its own mesh)
  DTop top = ctx->top.dtop;
  if (jobs) {
    std::vector<DMesh> table(ctx->meshes.size());
    for (size_t g = 0; g < table.size(); ++g) table[g] = ctx->meshes[g]->dmesh;
    PCUDA(R.jobmesh.ensure(table.size() * sizeof(DMesh)));
    PCUDA(cudaMemcpyAsync(R.jobmesh.p, table.data(), table.size() * sizeof(DMesh), cudaMemcpyHostToDevice, st));
    top = DTop{};
    top.meshes = R.jobmesh.as<DMesh>();
    top.n_geoms = (uint32_t)table.size();
    top.keys = 1;
    top.all_static = 1u;
    for (uint32_t g : used_geoms)
      if (ctx->meshes[g]->host.motion() || ctx->meshes[g]->has_xf) top.all_static = 0u;
  }
  if (train) PCUDA(cudaMemsetAsync(b.rcount, 0, 32, st));
  guide::GuideRows grows{};
  if (guided) {
    const float* g = b.grow;
    grows = guide::GuideRows{g, g + cap, g + 2 * cap, g + 3 * cap, g + 4 * cap, g + 5 * cap, g + 6 * cap,
                             g + 7 * cap, g + 8 * cap, cap, nullptr, {glo[0], glo[1], glo[2]},
                             {1.0f / (ghi[0] - glo[0]), 1.0f / (ghi[1] - glo[1]), 1.0f / (ghi[2] - glo[2])}};
  }
  PCUDA(cudaMemsetAsync(b.totals, 0, 24, st));
  PCUDA(cudaMemsetAsync(scr, 0, sizeof(DScratch) * 2 * (kPtMaxDepth + 1), st));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const int grid = std::max(1, sms) * 8;
  // Per-batch parameters, pinned so that each copy has its own stable source.
  const uint32_t nbatch = p->iter_count == 0 ? 0 : (p->iter_count + ipb - 1) / ipb;
  const size_t hbytes = std::max<size_t>(1, nbatch) * sizeof(PtIter);
  if (R.pt_host_bytes < hbytes) {
    PCUDA(cudaStreamSynchronize(st));
    if (R.pt_host) cudaFreeHost(R.pt_host);
    R.pt_host = nullptr;
    R.pt_host_bytes = 0;
    PCUDA(cudaMallocHost(&R.pt_host, hbytes));
    R.pt_host_bytes = hbytes;
  }
  PtIter* batches = static_cast<PtIter*>(R.pt_host);
  for (uint32_t k = 0; k < nbatch; ++k) {
    const uint32_t it0 = k * ipb;
    batches[k].iter0 = p->iter_begin + it0;
    batches[k].iters = std::min(ipb, p->iter_count - it0);
    batches[k].n = (unsigned long long)batches[k].iters * npix;
  }
  // The captured graph depends on every pointer and launch parameter above.
  const bool use_graph = !(p->flags & VMR_PATH_NO_GRAPH);
  std::vector<uint64_t> key = {(uint64_t)(uintptr_t)base, bytes, cap, npix, p->width, p->height, nl, p->max_depth,
                               p->rr_depth, p->seed, (uint64_t)(p->fb64 != nullptr), (uint64_t)(uintptr_t)st,
                               (uint64_t)(uintptr_t)ctx->top.nodes.p, (uint64_t)grid, (uint64_t)guided,
                               (uint64_t)train, (uint64_t)(uintptr_t)ctx->guide.wf.p, rcap,
                               (uint64_t)ctx->tuning.kernel, (uint64_t)ctx->tuning.walk_tail,
                               (uint64_t)ctx->tuning.blocks_per_sm,
                               (uint64_t)ctx->tuning.sort_bits, (uint64_t)sort_on,
                               (uint64_t)(uintptr_t)flat.mesh, (uint64_t)(uintptr_t)flat.map};
  {
    uint64_t h = 1469598103934665603ull;
    auto fold = [&](const void* d, size_t nb) {
      const unsigned char* c = static_cast<const unsigned char*>(d);
      for (size_t i = 0; i < nb; ++i) h = (h ^ c[i]) * 1099511628211ull;
    };
    fold(&b.groups, sizeof(b.groups));
    fold(&b.cam, sizeof(b.cam));
    fold(&b.cam_keys, sizeof(b.cam_keys));
    fold(&b.cam_nkeys, sizeof(b.cam_nkeys));
    fold(&b.pix0, sizeof(b.pix0));
    fold(&b.filt, sizeof(b.filt));
    fold(b.env, sizeof(b.env));
    fold(&b.sel, sizeof(b.sel));
    fold(&top, sizeof(top));
    const uint64_t nj = b.n_jobs;
    fold(&nj, sizeof(nj));
    fold(&b.alpha, sizeof(b.alpha));
    fold(&b.learn_sel, sizeof(b.learn_sel));
    fold(&b.gdepth, sizeof(b.gdepth));
    fold(b.glo, sizeof(b.glo));
    fold(grows.inv_ext, sizeof(grows.inv_ext));
    key.push_back(h);
  }
  uint32_t replays = 0, tsteps_done = 0;
  if (use_graph && nbatch > 0 && !(R.graph.exec && R.graph.key == key)) {
    if (R.graph.exec) {
      cudaGraphExecDestroy(R.graph.exec);
      R.graph.exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    PCUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    const int rc = launch_batch(ctx, b, top, scr, grid, guided, train, grows, srt, flat);
    const cudaError_t ec = cudaStreamEndCapture(st, &g);
    if (rc != VMR_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    PCUDA(ec);
    const cudaError_t ei = cudaGraphInstantiate(&R.graph.exec, g, 0);
    cudaGraphDestroy(g);
    PCUDA(ei);
    R.graph.key = key;
  }
  PCUDA(cudaEventRecord(ctx->ev0, st));
  for (uint32_t k = 0; k < nbatch; ++k) {
    PCUDA(cudaMemcpyAsync((void*)b.it, &batches[k], sizeof(PtIter), cudaMemcpyHostToDevice, st));
    if (use_graph) {
      PCUDA(cudaGraphLaunch(R.graph.exec, st));
      ++replays;
    } else {
      const int rc = launch_batch(ctx, b, top, scr, grid, guided, train, grows, srt, flat);
      if (rc != VMR_OK) return rc;
    }
    if (train) {  // online training on this batch's records (device counts)
      auto& G = ctx->guide;
      const uint32_t stride = (tbatch + 127) / 128 * 128;
      if (G.save_rows < stride) {
        PCUDA(G.save.ensure((size_t)guide::kSaveRows * stride * 2));
        G.save_rows = stride;
      }
      unsigned long long* ncount = b.rcount + 2;
      for (uint32_t s = 0; s < tsteps; ++s) {
        const uint64_t off = s;
        k_pt_train_count<<<1, 32, 0, st>>>(b.rcount, b.rcap, off, tsteps, tbatch, ncount);
        PCUDA(cudaGetLastError());
        guide::GuideTrain tr{};
        tr.rows = grows;
        const float* R = b.rec;
        const size_t c = b.rcap;
        tr.rows.px = R + kRP * c + off; tr.rows.py = R + (kRP + 1) * c + off; tr.rows.pz = R + (kRP + 2) * c + off;
        tr.rows.nx = R + kRN * c + off; tr.rows.ny = R + (kRN + 1) * c + off; tr.rows.nz = R + (kRN + 2) * c + off;
        tr.rows.wx = R + kRWo * c + off; tr.rows.wy = R + (kRWo + 1) * c + off; tr.rows.wz = R + (kRWo + 2) * c + off;
        tr.rows.n = tbatch;
        tr.rows.n_dev = ncount;
        tr.rows.rstride = tsteps;
        tr.ox = R + kROm * c + off; tr.oy = R + (kROm + 1) * c + off; tr.oz = R + (kROm + 2) * c + off;
        tr.weight = R + kRW * c + off;
        tr.pb = learn_sel ? R + kRPb * c + off : nullptr;
        tr.amax = alpha;
        tr.stride = stride;
        if (off >= rcap) break;
        PCUDA(cudaMemsetAsync(G.sums.p, 0, 16, st));
        if (guide::launch_train(tr, G.wf.p, G.wb.p, G.save.p, G.sums.as<float>(), G.err.as<int>(), sms, st) != 0)
          return pfail(ctx, VMR_ERR_CUDA, "guide training launch failed");
        if (guide::launch_wgrad(G.save.p, stride, tbatch, ncount, G.grad.as<float>(), G.err.as<int>(), sms, st) !=
            0)
          return pfail(ctx, VMR_ERR_CUDA, "guide weight-gradient launch failed");
        guide::GuideAdam a{tlr, 0.9f, 0.999f, 1e-8f, ++G.step};
        if (guide::launch_adam(G.W.as<float>(), G.m.as<float>(), G.v.as<float>(), G.grad.as<float>(),
                               G.sums.as<float>(), a, G.wf.p, G.wb.p, st) != 0)
          return pfail(ctx, VMR_ERR_CUDA, "guide Adam launch failed");
        ++tsteps_done;
      }
    }
  }
  PCUDA(cudaEventRecord(ctx->ev1, st));
  PCUDA(cudaMemcpyAsync(jobs ? arena.data() : fb, b.fb, (size_t)npix * 3 * 4, cudaMemcpyDeviceToHost, st));
  if (p->fb64) PCUDA(cudaMemcpyAsync(p->fb64, b.fb64, (size_t)npix * 3 * 8, cudaMemcpyDeviceToHost, st));
  unsigned long long tot[2] = {0, 0};
  PCUDA(cudaMemcpyAsync(tot, b.totals, 16, cudaMemcpyDeviceToHost, st));
  int status = 0, gerr = 0;
  PCUDA(cudaMemcpyAsync(&status, b.status, 4, cudaMemcpyDeviceToHost, st));
  unsigned long long recs[2] = {0, 0};
  float gsums[2] = {0.f, 0.f};
  if (train) {
    PCUDA(cudaMemcpyAsync(recs, b.rcount, 16, cudaMemcpyDeviceToHost, st));
    PCUDA(cudaMemcpyAsync(gsums, ctx->guide.sums.p, 8, cudaMemcpyDeviceToHost, st));
  }
  if (guided) PCUDA(cudaMemcpyAsync(&gerr, ctx->guide.err.p, 4, cudaMemcpyDeviceToHost, st));
  PCUDA(cudaStreamSynchronize(st));
  if (status == kStatusStackOverflow) return pfail(ctx, VMR_ERR_STACK_OVERFLOW, "traversal stack overflow");
  if (status != kStatusOk) return pfail(ctx, VMR_ERR_TIMEOUT, "traversal iteration cap");
  if (gerr) {
    cudaMemsetAsync(ctx->guide.err.p, 0, 4, st);
    return pfail(ctx, VMR_ERR_TIMEOUT, "a guide kernel's tensor-core wait ran out");
  }
  if (jobs)
    for (uint32_t k = 0; k < n_jobs; ++k)
      std::memcpy(jobs[k].fb, arena.data() + (size_t)jtab[k].pix0 * 3, (size_t)jtab[k].npix * 12);
  if (stats) {
    stats->samples = (uint64_t)npix * p->iter_count;
    stats->rays = tot[0];
    stats->shadow_rays = tot[1];
    stats->graph_replays = replays;
    stats->train_records = recs[1];
    stats->train_steps = tsteps_done;
    stats->train_loss = gsums[1] > 0.f ? gsums[0] / gsums[1] : 0.f;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    stats->ms = ms;
  }
  return VMR_OK;
}

int vmr_render_path(vmr_ctx* ctx, const vmr_path_params* p, float* fb, vmr_path_stats* stats) {
  if (!fb) return VMR_ERR_INVALID;
  return render_path_impl(ctx, p, fb, stats, nullptr, 0);
}

// Static and motion jobs run as two batched renders, so that the static ones
// keep the while-while scene kernel's leaner static instantiation and only
// the motion ones pay for its motion instantiation (every job is
// independent, so the split changes no result).
int vmr_render_path_jobs(vmr_ctx* ctx, const vmr_path_job* jobs, uint32_t n_jobs, const vmr_path_params* p,
                         vmr_path_stats* stats) {
  if (!ctx || !p || (n_jobs && !jobs)) return VMR_ERR_INVALID;
  std::vector<vmr_path_job> groups[2];
  for (uint32_t k = 0; k < n_jobs; ++k) {
    if (jobs[k].geom >= ctx->meshes.size()) return vmr::pfail(ctx, VMR_ERR_INVALID, "job geom out of range");
    groups[ctx->meshes[jobs[k].geom]->host.motion() ? 1 : 0].push_back(jobs[k]);
  }
  vmr_path_stats total{};
  for (const auto& gr : groups) {
    if (gr.empty()) continue;
    vmr_path_stats st{};
    const int rc = render_path_impl(ctx, p, nullptr, &st, gr.data(), (uint32_t)gr.size());
    if (rc != VMR_OK) return rc;
    total.samples += st.samples;
    total.rays += st.rays;
    total.shadow_rays += st.shadow_rays;
    total.graph_replays += st.graph_replays;
    total.ms += st.ms;
  }
  if (stats) *stats = total;
  return VMR_OK;
}

int vmr_set_path_batch(vmr_ctx* ctx, uint32_t paths) {
  if (!ctx) return VMR_ERR_INVALID;
  if (paths != 0 && paths < 1024) return vmr::pfail(ctx, VMR_ERR_INVALID, "path batch must be 0 or >= 1024");
  ctx->render.path_batch = paths;
  return VMR_OK;
}

int vmr_get_path_batch(vmr_ctx* ctx, uint32_t* paths) {
  if (!ctx || !paths) return VMR_ERR_INVALID;
  *paths = ctx->render.path_batch;
  return VMR_OK;
}

// Queue capacity per scene: the render of p (its size, depths, flags; the
// guide is sampled but never trained here) timed at each candidate batch
// size, after one untimed call that captures that size's bounce-loop graph;
// the fastest becomes the context's default.  Candidates that round to the
// same whole number of iterations per batch are timed once.
int vmr_autotune_path(vmr_ctx* ctx, const vmr_path_params* p, uint32_t* candidates, float* ms,
                      uint32_t* n_candidates, uint32_t* best) {
  if (!ctx || !p || !p->width || !p->height || !p->iter_count) return VMR_ERR_INVALID;
  static const uint32_t kCand[] = {256u << 10, 512u << 10, 1u << 20, 2u << 20, 4u << 20, 8u << 20, 16u << 20,
                                   32u << 20};
  const uint64_t npix = (uint64_t)p->width * p->height;
  std::vector<float> fb((size_t)npix * 3);
  vmr_path_params q = *p;
  q.flags &= ~(uint32_t)VMR_PATH_TRAIN;
  q.fb64 = nullptr;
  uint32_t n = 0, win = 0, last_ipb = 0;
  float win_ms = INFINITY;
  for (uint32_t c : kCand) {
    uint64_t ipb = std::max<uint64_t>(1, c / npix);
    if (ipb > p->iter_count) ipb = p->iter_count;
    if (ipb == last_ipb) continue;
    last_ipb = (uint32_t)ipb;
    if ((uint64_t)ipb * npix > 0xffffffffull) break;
    q.max_batch_samples = (uint32_t)(ipb * npix);
    vmr_path_stats st{};
    std::fill(fb.begin(), fb.end(), 0.0f);
    int rc = render_path_impl(ctx, &q, fb.data(), &st, nullptr, 0);
    if (rc != VMR_OK) return rc;
    std::fill(fb.begin(), fb.end(), 0.0f);
    rc = render_path_impl(ctx, &q, fb.data(), &st, nullptr, 0);
    if (rc != VMR_OK) return rc;
    if (candidates) candidates[n] = q.max_batch_samples;
    if (ms) ms[n] = st.ms;
    ++n;
    if (st.ms < win_ms) {
      win_ms = st.ms;
      win = q.max_batch_samples;
    }
  }
  ctx->render.path_batch = win;
  if (n_candidates) *n_candidates = n;
  if (best) *best = win;
  return VMR_OK;
}

}  // extern "C"
