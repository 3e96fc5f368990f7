// render.cu - reference-mode render path: generate, shade, shadow, accumulate.
//
// core.Render (core/render.go:66-218) renders one sample per pixel per
// iteration: RasterXY/VdC/Sobol QMC (math/ldseq), a pinhole camera ray
// (builtin/camera/camera.go:221-323), the closest hit, ShaderStd.Eval
// (builtin/shader/std.go:77-316) with EvaluateLightSamples' MIS over TriLights
// (core/shader.go:203-402, builtin/light/triangle.go) and the hero-wavelength
// spectrum (colour/*.go), then buf = (buf*iter + c)/(iter+1).  Here a batch of
// iterations runs as a wavefront:
//   k_generate    one camera ray per (iteration, pixel), bit-identical to the
//                 oracle (IEEE float ops in the reference's order, no FMA)
//   trace         the two-level closest-hit kernel
//   k_shade       hit attributes + ShaderStd: emission, per (lobe, light,
//                 sample) a contribution slot, and a compacted shadow-ray
//                 queue filled with warp-aggregated atomics
//   trace         the any-hit kernel over the shadow queue
//   k_accumulate  per pixel, the iterations in order: slots summed in the
//                 reference's order, scaled, folded into the framebuffer
// Transcendentals are evaluated in float64 and rounded to float32, as
// math/sincos.go does; normalisation is a * (1/sqrt(a.a)) with IEEE sqrt and
// division (the reference's RSQRTSS estimate is machine-dependent).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "device.h"
#include "shade_common.cuh"
#include "vmr.h"

namespace vmr {
namespace {

// A light-sample candidate: direction, distance, pdf, spectrum.
struct Cand {
  V3 Ld;
  float Ldist;
  float pdf_own;    // light samples: ls.Pdf; BSDF samples: unused
  double pdf_bsdf;  // BSDF samples: bs.Pdf
  float pdf_light;  // BSDF samples: bs.PdfLight
  bool ok;
};

// Disk.SampleArea, sample i of n (builtin/light/disk.go:154-204).
// F32 (in this and the functions below): the VMR_RENDER_F32 precision switch
// of the transcendentals (shade_common.cuh msin etc.).
template <bool F32>
__device__ Cand disk_sample(const RLight& L, const Ctx& sc, int n, int i) {
  Cand c{};
  const uint64_t idx = sc.I * (uint64_t)n + (uint64_t)i;
  const double r0 = vdc(idx, sc.scr0), r1 = sobol(idx, sc.scr1);
  const float u = L.radius * sqrtf((float)r0) * mcos<F32>(2 * kPi * (float)r1);
  const float v = L.radius * sqrtf((float)r0) * msin<F32>(2 * kPi * (float)r1);
  const double pdf = (double)(1.0f / (kPi * L.radius * L.radius));
  const V3 LP = v3(L.P[0], L.P[1], L.P[2]), LT = v3(L.T[0], L.T[1], L.T[2]), LB = v3(L.B[0], L.B[1], L.B[2]),
           LN = v3(L.N[0], L.N[1], L.N[2]);
  const V3 P = add(add(LP, scale(u, LB)), scale(v, LT));
  const V3 V = sub(P, sc.P);
  if (!(dot(V, sc.Ng) > 0.0f && dot(V, LN) < 0.0f)) return c;
  c.Ldist = length(V);
  c.Ld = normalize(V);
  c.pdf_own = (float)pdf * (c.Ldist * c.Ldist) / fabsf(dot(c.Ld, LN));
  c.ok = true;
  return c;
}

// raySphereIntersect (builtin/light/sphere.go:96-124).
__device__ bool light_sphere_hit(V3 Ro, V3 Rd, V3 C, float radius, float& t) {
  const V3 Lv = sub(Ro, C);
  const float a = dot(Rd, Rd);
  const float b = 2 * dot(Rd, Lv);
  const float c = dot(Lv, Lv) - radius * radius;
  const float discr = b * b - 4 * a * c;
  if (discr < 0) return false;
  float x0, x1;
  if (discr == 0) {
    x1 = -0.5f * b / a;
    x0 = x1;
  } else {
    const float q = b > 0 ? -0.5f * (b + sqrtf(discr)) : -0.5f * (b - sqrtf(discr));
    x0 = q / a;
    x1 = c / q;
  }
  if (x0 > x1) { const float tt = x0; x0 = x1; x1 = tt; }
  if (x0 > x1) { const float tt = x0; x0 = x1; x1 = tt; }
  if (x0 < 0) {
    x0 = x1;
    if (x0 < 0) return false;
  }
  t = x0;
  return true;
}

// Sphere.SampleArea, sample i of n (builtin/light/sphere.go:178-254).
template <bool F32>
__device__ Cand sphere_sample(const RLight& L, const Ctx& sc, int n, int i) {
  Cand c{};
  const V3 C = v3(L.P[0], L.P[1], L.P[2]);
  const V3 V = sub(C, sc.P);
  const float l = length(V);
  const V3 w = normalize(V);
  const V3 v = normalize(cross(w, sc.Ng));
  const V3 u = cross(w, v);
  const uint64_t idx = sc.I * (uint64_t)n + (uint64_t)i;
  const double r0 = vdc(idx, sc.scr0), r1 = sobol(idx, sc.scr1);
  const float theta = macos<F32>(1 - (float)r0 + (float)r0 * sqrtf(1 - sqr(L.radius / l)));
  const float phi = 2 * kPi * (float)r1;
  const V3 a = v3(mcos<F32>(phi) * msin<F32>(theta), msin<F32>(phi) * msin<F32>(theta), mcos<F32>(theta));
  const V3 omega = expand(u, v, w, a);
  if (dot(omega, sc.Ng) < 0) return c;
  float t;
  if (!light_sphere_hit(sc.P, omega, C, L.radius, t)) return c;
  const V3 x = add(sc.P, scale(t, omega));
  const V3 D = sub(x, sc.P);
  c.Ldist = length(D);
  c.Ld = normalize(D);
  c.pdf_own = 1 / (2 * kPi * (1 - sqrtf(1 - sqr(L.radius / l))));
  c.ok = true;
  return c;
}

// Tri.SampleArea, sample i of n (triangle.go:232-343).
template <bool F32>
__device__ Cand light_sample(const RLight& L, const Ctx& sc, int n, int i) {
  if (L.kind == 1) return disk_sample<F32>(L, sc, n, i);
  if (L.kind == 2) return sphere_sample<F32>(L, sc, n, i);
  Cand c{};
  const V3 p0 = lp(L, 0), p1 = lp(L, 1), p2 = lp(L, 2);
  const V3 N = normalize(cross(sub(p1, p0), sub(p2, p0)));
  const bool area_only = dot(sc.Ng, sub(p0, sc.P)) < 0 || dot(sc.Ng, sub(p1, sc.P)) < 0 || dot(sc.Ng, sub(p2, sc.P)) < 0;
  const uint64_t idx = sc.I * (uint64_t)n + (uint64_t)i;
  const double r0 = vdc(idx, sc.scr0), r1 = sobol(idx, sc.scr1);
  if (area_only) {
    const double pdf = (double)(1 / tri_area(p0, p1, p2));
    const float a = F32 ? (float)r1 * sqrtf(1.0f - (float)r0) : (float)(r1 * sqrt(1 - r0));
    const float b = F32 ? 1.0f - sqrtf(1.0f - (float)r0) : (float)(1 - sqrt(1 - r0));
    const V3 P = add(add(p0, scale(a, sub(p1, p0))), scale(b, sub(p2, p0)));
    const V3 D = sub(P, sc.P);
    c.Ldist = length(D);
    c.Ld = normalize(D);
    if (dot(c.Ld, N) > 0 || dot(c.Ld, sc.Ng) < 0) return c;
    c.pdf_own = (float)pdf * sqr(c.Ldist) / fabsf(dot(c.Ld, N));
  } else {
    double pdf;
    const V3 x = sample_spherical<F32>(p0, p1, p2, sc.P, r0, r1, pdf);
    float t;
    ray_plane(sc.P, x, p0, N, t);
    const V3 P = add(sc.P, scale(t, x));
    const V3 D = sub(P, sc.P);
    c.Ldist = length(D);
    c.Ld = normalize(D);
    if (dot(c.Ld, N) > 0 || dot(c.Ld, sc.Ng) < 0) return c;
    c.pdf_own = (float)pdf;
  }
  c.ok = true;
  return c;
}

// BSDF sample i then Tri.ValidSample / Disk.ValidSample (core/shader.go:211-228,
// triangle.go:136-230, disk.go:119-151).
template <bool F32>
__device__ Cand bsdf_candidate(const RLight& L, const Ctx& sc, const Bsdf& bsdf, int half, int i) {
  Cand c{};
  const uint64_t idx = sc.I * (uint64_t)half + (uint64_t)i;
  const double r0 = vdc(idx, sc.scr0), r1 = sobol(idx, sc.scr1);
  const V3 D = normalize(bsdf_sample<F32>(bsdf, r0, r1));
  c.pdf_bsdf = bsdf_pdf<F32>(bsdf, D);
  if (c.pdf_bsdf <= 0) return c;
  if (L.kind == 2) {  // Sphere.ValidSample (sphere.go:126-176)
    const V3 C = v3(L.P[0], L.P[1], L.P[2]);
    float t;
    if (!light_sphere_hit(sc.P, D, C, L.radius, t)) return c;
    const V3 x = add(sc.P, scale(t, D));
    const V3 Dl = sub(x, sc.P);
    c.Ldist = length(Dl);
    c.Ld = normalize(Dl);
    const float l = length(sub(C, sc.P));
    c.pdf_light = 1 / (2 * kPi * (1 - sqrtf(1 - sqr(L.radius / l))));
    c.ok = true;
    return c;
  }
  if (L.kind == 1) {
    const double pdf = (double)(1.0f / (kPi * L.radius * L.radius));
    const V3 LP = v3(L.P[0], L.P[1], L.P[2]), LN = v3(L.N[0], L.N[1], L.N[2]);
    float t;
    if (!ray_plane(sc.P, D, LP, LN, t)) return c;  // rayDiskIntersect (disk.go:53-68)
    const V3 pp = add(sc.P, scale(t, D));
    const V3 vv = sub(pp, LP);
    if (!(sqrtf(dot(vv, vv)) <= L.radius)) return c;
    const V3 V = sub(add(sc.P, scale(t, D)), sc.P);
    if (dot(V, sc.Ng) <= 0.0f || dot(V, LN) >= 0.0f) return c;
    c.Ldist = length(V);
    c.Ld = normalize(V);
    c.pdf_light = (float)pdf * (c.Ldist * c.Ldist) / fabsf(dot(c.Ld, LN));
    c.ok = true;
    return c;
  }
  const V3 p0 = lp(L, 0), p1 = lp(L, 1), p2 = lp(L, 2);
  V3 P;
  if (!ray_tri(sc.P, D, p0, p1, p2, P)) return c;
  const V3 N = normalize(cross(sub(p1, p0), sub(p2, p0)));
  const bool area_only = dot(sc.Ng, sub(p0, P)) < 0 || dot(sc.Ng, sub(p1, P)) < 0 || dot(sc.Ng, sub(p2, P)) < 0;
  const V3 Dl = sub(P, sc.P);
  c.Ldist = length(Dl);
  c.Ld = normalize(Dl);
  if (dot(c.Ld, N) > 0 || dot(c.Ld, sc.Ng) < 0) return c;
  if (area_only) {
    const double pdf = (double)(1 / tri_area(p0, p1, p2));
    c.pdf_light = (float)pdf * sqr(c.Ldist) / fabsf(dot(c.Ld, N));
  } else {
    const V3 pa = normalize(sub(p0, sc.P)), pb = normalize(sub(p1, sc.P)), pc = normalize(sub(p2, sc.P));
    const float a = macos<F32>(dot(pb, pc)), b = macos<F32>(dot(pc, pa)), cc = macos<F32>(dot(pa, pb));
    float al, be, ga;
    sides_to_angles<F32>(a, b, cc, al, be, ga);
    const float area = al + be + ga - kPi;
    c.pdf_light = (float)(1 / (double)area);
  }
  c.ok = true;
  return c;
}

// --------------------------------------------------------------- layout ---
constexpr int kMaxHalf = 8;    // NumSamples up to 16 per light (Samples <= 4)
constexpr int kMaxLevel = 3;   // ShaderStd.Eval returns nothing above level 3 (std.go:96-98)

// One recursion level of a batch (level 0: the camera rays, one entry per
// sample; level l > 0: the mirror reflections of level l-1, one entry per
// reflection, compacted).  Per entry e: slots[e][lobe][light][k] hold a
// contribution (rgb) that counts when its shadow ray is unoccluded (k < half:
// light samples, then BSDF samples: the order EvaluateLightSamples adds
// them); lscale[e][lobe][light] = 1/float32(total), -1 when the light takes
// one sample (no MIS, no scale), 0 when nothing was taken; mw[e] = the mirror
// weight to_rgb(rho/pdf)*Spec1Colour and Spec1Weight (w = -1: not a mirror).
struct Level {
  float* ray;          // 8 * cap: px py pz dx dy dz tmax time
  uint32_t* samp;      // entry -> sample (null at level 0: the identity)
  int32_t* hit;        // 6 * cap: prim geom t u v w
  int32_t* shader;     // shader id of the hit, -1 none
  float* emis;         // 3 per entry
  float* slot_rgb;     // [cap][2][nl][ns][3]
  uint8_t* slot_live;  // [cap][2][nl][ns]
  float* lscale;       // [cap][2][nl]
  float* mw;           // 4 per entry: w.rgb, Spec1Weight (-1: not a mirror)
  int32_t* child;      // entry at level + 1, -1 none
  uint32_t ns;         // slots per (lobe, light)
  uint32_t cap;
  unsigned long long* count;  // entries (levels > 0; appended by the level below)
};

struct RenderBatch {
  uint32_t width, height, npix;  // npix: the pixels of the rendered band
  uint32_t pix0;                 // the band's first pixel in the image
  uint32_t iter0;  // first core.Render loop iteration of the batch
  uint32_t n;      // samples in the batch
  uint32_t nl;     // lights
  uint32_t levels; // levels with storage (1 + mirror depth)
  uint32_t pad;
  uint64_t seed;
  vmr_camera cam;
  const anim::Decomp* cam_keys;  // camera motion keys (cam_nkeys >= 2), else null
  uint32_t cam_nkeys;
  PixFilter filt;     // pixel filter tables (n = 0: none)
  const vmr_shader_std* shaders;
  const RLight* lights;
  const RMesh* meshes;
  float* lambda;      // per sample
  Level lv[kMaxLevel + 1];
  float *sx, *sy, *sz, *sdx, *sdy, *sdz, *stmax, *stime;
  uint32_t* sback;    // queue entry -> slot index (of the level being shaded)
  int32_t* shit;      // any-hit prim per queue entry
  unsigned long long* queue_len;
  uint32_t queue_cap;
  int* status;
  float* fb;          // framebuffer (device), w*h*3
};

__device__ __forceinline__ float* ray_f(const Level& L, int k, uint64_t e) { return L.ray + (size_t)k * L.cap + e; }

// CKEYS: the camera has motion keys (b.cam_nkeys >= 2).
template <bool CKEYS>
__global__ void k_generate(RenderBatch b) {
  const uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (s >= b.n) return;
  const uint32_t pix = b.pix0 + (uint32_t)(s % b.npix);    // the image pixel
  const uint32_t j = b.iter0 + (uint32_t)(s / b.npix) + 1;  // render(iter+1)
  V3 P, D;
  float time, lambda;
  camera_primary<CKEYS>(b.cam, b.cam_keys, b.cam_nkeys, b.width, b.height, j, pix, b.seed, b.filt, P, D, time,
                        lambda);
  const Level& L = b.lv[0];
  *ray_f(L, 0, s) = P.x; *ray_f(L, 1, s) = P.y; *ray_f(L, 2, s) = P.z;
  *ray_f(L, 3, s) = D.x; *ray_f(L, 4, s) = D.y; *ray_f(L, 5, s) = D.z;
  *ray_f(L, 6, s) = __int_as_float(0x7f800000);
  *ray_f(L, 7, s) = time;
  b.lambda[s] = lambda;
}

// Queues one shadow ray (one atomic per warp for the lanes that want one).
__device__ void emit_shadow(const RenderBatch& b, const Level& lv, const Ctx& sc, V3 Ld, float Ldist, uint32_t slot,
                            bool want) {
  const unsigned act = __activemask();
  const unsigned m = __ballot_sync(act, want);
  if (m == 0u) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(b.queue_len, (unsigned long long)__popc(m));
  base = __shfl_sync(act, base, leader);
  if (!want) return;
  const unsigned long long q = base + __popc(m & ((1u << lane) - 1u));
  if (q >= b.queue_cap) {  // counted by the host from queue_len; never written
    lv.slot_live[slot] = 0;
    return;
  }
  const V3 o = offset_p(sc, dot(Ld, sc.Ng) < 0 ? -1 : 1);
  const V3 d = scale(Ldist * 0.9999f, Ld);  // D = Ld*(Ldist*(1-ShadowRayEpsilon)), tmax 1 (shader.go:269-274)
  b.sx[q] = o.x; b.sy[q] = o.y; b.sz[q] = o.z;
  b.sdx[q] = d.x; b.sdy[q] = d.y; b.sdz[q] = d.z;
  b.stmax[q] = 1.0f;
  b.stime[q] = sc.time;
  b.sback[q] = slot;
}

// EvaluateLightSamples (core/shader.go:203-402) for one (lobe, light):
// writes the slot contributions, queues their shadow rays and returns the
// scale the accumulate pass applies.
template <bool F32>
__device__ float light_lobe(const RenderBatch& b, const Level& lv, const Ctx& sc, const RLight& L, const Bsdf& bsdf,
                            int NS, uint32_t slot0) {
  const int half = NS > 1 ? NS / 2 : 0;
  const int nls = NS > 1 ? half : NS;
  Cand cl[kMaxHalf], cb[kMaxHalf];
  int n_light = 0, n_bsdf = 0;
  for (int i = 0; i < nls; ++i) {
    cl[i] = light_sample<F32>(L, sc, nls, i);
    n_light += cl[i].ok ? 1 : 0;
  }
  for (int i = 0; i < half; ++i) {
    cb[i] = bsdf_candidate<F32>(L, sc, bsdf, half, i);
    n_bsdf += cb[i].ok ? 1 : 0;
  }
  const int nB = n_bsdf == 0 ? 0 : half;
  const int nL = n_light == 0 ? 0 : half;
  const int total = nB + nL;
  const bool mis = NS > 1;
  const Spec Liu = from_rgb(emission(b.shaders[L.shader]), sc.lambda);
  for (int pass = 0; pass < 2; ++pass) {
    const int cnt = pass == 0 ? nls : half;
    for (int i = 0; i < cnt; ++i) {
      const Cand& c = pass == 0 ? cl[i] : cb[i];
      const uint32_t slot = slot0 + (pass == 0 ? 0 : half) + i;
      const bool want = c.ok && dot(c.Ld, sc.N) > 0 && !(mis && total == 0);
      float* out = lv.slot_rgb + (size_t)slot * 3;
      out[0] = out[1] = out[2] = 0.0f;
      if (want) {
        Spec rho = bsdf_eval<F32>(bsdf, c.Ld);
        for (int k = 0; k < 4; ++k) rho.c[k] *= Liu.c[k];
        float inv;
        if (mis) {
          float p_hat;
          if (pass == 0) {
            p_hat = (float)nB * (float)bsdf_pdf<F32>(bsdf, c.Ld) / (float)total;
            p_hat += (float)nL * c.pdf_own / (float)total;
          } else {
            p_hat = (float)nB * (float)c.pdf_bsdf / (float)total;
            p_hat += (float)nL * c.pdf_light / (float)total;
          }
          inv = 1.0f / p_hat;
        } else {
          inv = 1.0f / c.pdf_own;
        }
        for (int k = 0; k < 4; ++k) rho.c[k] *= inv;
        RGB rgb = to_rgb(rho, sc.lambda);
        if (mis)
          for (float& v : rgb.c)
            if (v < 0) v = 0;
        out[0] = rgb.c[0];
        out[1] = rgb.c[1];
        out[2] = rgb.c[2];
      }
      lv.slot_live[slot] = want ? 1 : 0;
      emit_shadow(b, lv, sc, c.Ld, c.Ldist, slot, want);
    }
  }
  if (!mis) return -1.0f;
  return total == 0 ? 0.0f : 1.0f / (float)total;
}

// Hit attributes (builtin/geom/polymesh/trace.go:276-515, static meshes) and
// ShaderStd.Eval (builtin/shader/std.go:77-296) for the entries of one
// level: emission, the diffuse and glossy lobes' light samples, and the
// mirror (Spec1Roughness 0) reflection queued for the next level with the
// sample's I and scrambles (a child ShaderContext copies them).
template <bool F32, bool GROUPS>
__global__ void __launch_bounds__(128) k_shade(RenderBatch b, uint32_t level) {
  const Level& lv = b.lv[level];
  const uint64_t n = level == 0 ? (uint64_t)b.n : (*lv.count < lv.cap ? *lv.count : lv.cap);
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t s = level == 0 ? e : lv.samp[e];
    const int32_t prim = lv.hit[e];
    float* em = lv.emis + e * 3;
    em[0] = em[1] = em[2] = 0.0f;
    const size_t nslot = (size_t)2 * b.nl * lv.ns;
    for (size_t k = 0; k < nslot; ++k) lv.slot_live[e * nslot + k] = 0;
    for (size_t k = 0; k < (size_t)2 * b.nl; ++k) lv.lscale[e * 2 * b.nl + k] = 0.0f;
    lv.shader[e] = -1;
    lv.mw[e * 4 + 3] = -1.0f;
    lv.child[e] = -1;
    if (prim < 0) continue;
    const int32_t geom = lv.hit[lv.cap + e];
    const RMesh& m = b.meshes[geom];
    Ctx sc;
    uint32_t shid;
    const float* hf = reinterpret_cast<const float*>(lv.hit);
    const V3 Ro = v3(*ray_f(lv, 0, e), *ray_f(lv, 1, e), *ray_f(lv, 2, e));
    const V3 Rdir = v3(*ray_f(lv, 3, e), *ray_f(lv, 4, e), *ray_f(lv, 5, e));
    if (!surface_attributes<GROUPS>(m, prim, hf[3 * (size_t)lv.cap + e], hf[4 * (size_t)lv.cap + e],
                            hf[5 * (size_t)lv.cap + e], Ro, Rdir, hf[2 * (size_t)lv.cap + e], *ray_f(lv, 7, e), sc,
                            shid))
      continue;
    const vmr_shader_std& sh = b.shaders[shid];
    sc.Rd = v3(*ray_f(lv, 3, e), *ray_f(lv, 4, e), *ray_f(lv, 5, e));
    sc.lambda = b.lambda[s];
    sc.time = *ray_f(lv, 7, e);
    const uint32_t pix = b.pix0 + (uint32_t)(s % b.npix);
    sc.I = b.iter0 + (uint64_t)(s / b.npix) + 1;
    sc.scr0 = scramble(b.seed, pix, 4);
    sc.scr1 = scramble(b.seed, pix, 5);
    sc.geom = geom;
    lv.shader[e] = (int32_t)shid;
    if (sh.flags & VMR_SH_DEBUG) {  // Debug.Eval: OutRGB = Colour (debug.go:47-49)
      em[0] = sh.diffuse_colour[0];
      em[1] = sh.diffuse_colour[1];
      em[2] = sh.diffuse_colour[2];
      continue;
    }
    const RGB ec = emission(sh);
    em[0] = ec.c[0];
    em[1] = ec.c[1];
    em[2] = ec.c[2];
    // tangent frame (std.go:101-108)
    V3 Vt = cross(sc.N, sc.DdPdu);
    if (len2(Vt) < 0.1f) Vt = cross(sc.N, sc.DdPdv);
    Vt = normalize(Vt);
    const V3 Ut = normalize(cross(sc.N, Vt));
    const V3 wi = v3(-sc.Rd.x, -sc.Rd.y, -sc.Rd.z);
    float dw = (sh.flags & VMR_SH_DIFFUSE_STRENGTH) ? sh.diffuse_strength : 0.0f;
    float sw = (sh.flags & VMR_SH_SPEC1_STRENGTH) ? sh.spec1_strength : 0.0f;
    const float total = dw + sw;
    if (total == 0.0f) {  // the reference panics: no weight (std.go:141-143)
      atomicMax(b.status, kStatusIterationCap + 1);
      continue;
    }
    dw /= total;
    sw /= total;
    if (dw > 0.0f) {
      const float rough = (sh.flags & VMR_SH_DIFFUSE_ROUGHNESS) ? sh.diffuse_roughness : 0.5f;
      const Bsdf diff{0, sc.lambda, project(Ut, Vt, sc.N, wi), rough * rough, Fresnel{0, 0, {}, {}}, Ut, Vt, sc.N};
      for (uint32_t l = 0; l < b.nl; ++l) {
        const RLight& L = b.lights[l];
        if ((int32_t)L.geom == geom) continue;  // LightsPrepare (scene.go:100-116)
        const int NS = level > 0 ? 1 : 1 << L.samples;  // level > 0: one sample (shader.go:189-191)
        const uint32_t slot0 = (uint32_t)((e * 2 + 0) * b.nl + l) * lv.ns;
        lv.lscale[(e * 2 + 0) * b.nl + l] = light_lobe<F32>(b, lv, sc, L, diff, NS, slot0);
      }
    }
    if (sw > 0.0f) {
      const float rough = (sh.flags & VMR_SH_SPEC1_ROUGHNESS) ? sh.spec1_roughness : 0.5f;
      Fresnel fr{0, (sh.flags & VMR_SH_IOR) ? sh.ior : 1.7f, {}, {}};
      if (sh.spec1_fresnel == 1) {
        RGB refl{{0.5f, 0.5f, 0.5f}}, edge{{0.5f, 0.5f, 0.5f}};
        if (sh.flags & VMR_SH_FRESNEL_REFL) refl = RGB{{sh.spec1_fresnel_refl[0], sh.spec1_fresnel_refl[1], sh.spec1_fresnel_refl[2]}};
        if (sh.flags & VMR_SH_FRESNEL_EDGE)  // assigned to refl, as std.go:185-187 does
          refl = RGB{{sh.spec1_fresnel_edge[0], sh.spec1_fresnel_edge[1], sh.spec1_fresnel_edge[2]}};
        fr = Fresnel{1, 0, refl, edge};
      }
      if (rough > 0.0f) {
        const Bsdf spec{1, sc.lambda, project(Ut, Vt, sc.N, wi), rough * rough, fr, Ut, Vt, sc.N};
        for (uint32_t l = 0; l < b.nl; ++l) {
          const RLight& L = b.lights[l];
          if ((int32_t)L.geom == geom) continue;
          const int NS = level > 0 ? 1 : 1 << L.samples;
          const uint32_t slot0 = (uint32_t)((e * 2 + 1) * b.nl + l) * lv.ns;
          lv.lscale[(e * 2 + 1) * b.nl + l] = light_lobe<F32>(b, lv, sc, L, spec, NS, slot0);
        }
      } else {
        // the mirror: one sample at idx = I (std.go:216-259)
        const Bsdf spec{2, sc.lambda, project(Ut, Vt, sc.N, wi), rough * rough, fr, Ut, Vt, sc.N};
        const double r0 = vdc(sc.I, sc.scr0), r1 = sobol(sc.I, sc.scr1);
        const V3 wo = bsdf_sample<F32>(spec, r0, r1);
        const double pdf = bsdf_pdf<F32>(spec, wo);
        float* w = lv.mw + e * 4;
        w[0] = w[1] = w[2] = 0.0f;
        w[3] = sw;
        if (dot(wo, sc.Ng) > 0.0f) {
          Spec rho = bsdf_eval<F32>(spec, wo);
          const float inv = 1.0f / (float)pdf;
          for (int k = 0; k < 4; ++k) rho.c[k] *= inv;
          const RGB col = to_rgb(rho, sc.lambda);
          const RGB scol = (sh.flags & VMR_SH_SPEC1_COLOUR)
                               ? RGB{{sh.spec1_colour[0], sh.spec1_colour[1], sh.spec1_colour[2]}}
                               : RGB{{0, 0, 0}};
          for (int k = 0; k < 3; ++k) w[k] = col.c[k] * scol.c[k];
          // level 3's reflection reaches level 4, whose ShaderStd.Eval adds
          // nothing: it would contribute w*0, clamped to 0, so it is not traced
          if (level < (uint32_t)kMaxLevel && level + 1 < b.levels) {
            const Level& nx = b.lv[level + 1];
            const unsigned long long c = atomicAdd(nx.count, 1ull);
            if (c < nx.cap) {
              const V3 o = offset_p(sc, 1);
              *ray_f(nx, 0, c) = o.x; *ray_f(nx, 1, c) = o.y; *ray_f(nx, 2, c) = o.z;
              *ray_f(nx, 3, c) = wo.x; *ray_f(nx, 4, c) = wo.y; *ray_f(nx, 5, c) = wo.z;
              *ray_f(nx, 6, c) = __int_as_float(0x7f800000);
              *ray_f(nx, 7, c) = sc.time;
              nx.samp[c] = (uint32_t)s;
              lv.child[e] = (int32_t)c;
            }
          }
        }
      }
    }
  }
}

// Occluded shadow rays switch their slot off.
__global__ void k_resolve(RenderBatch b, uint32_t level, uint32_t nq) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq && b.shit[q] >= 0) b.lv[level].slot_live[b.sback[q]] = 0;
}

// ShaderStd.Eval's sum for one entry: ((0 + emission) + diffuse) + spec, the
// spec part being the glossy lobes' light samples or, for a mirror,
// clamp(w * child) * Spec1Weight (0 when the reflection found nothing).
__device__ RGB entry_colour(const RenderBatch& b, const Level& lv, uint64_t e, bool child_hit, RGB child) {
  RGB c{{0, 0, 0}};
  const vmr_shader_std& sh = b.shaders[lv.shader[e]];
  float dw = (sh.flags & VMR_SH_DIFFUSE_STRENGTH) ? sh.diffuse_strength : 0.0f;
  float sw = (sh.flags & VMR_SH_SPEC1_STRENGTH) ? sh.spec1_strength : 0.0f;
  const float tw = dw + sw;
  dw /= tw;
  sw /= tw;
  RGB lobe[2] = {{{0, 0, 0}}, {{0, 0, 0}}};
  const RGB colour[2] = {
      (sh.flags & VMR_SH_DIFFUSE_COLOUR) ? RGB{{sh.diffuse_colour[0], sh.diffuse_colour[1], sh.diffuse_colour[2]}} : RGB{{0, 0, 0}},
      (sh.flags & VMR_SH_SPEC1_COLOUR) ? RGB{{sh.spec1_colour[0], sh.spec1_colour[1], sh.spec1_colour[2]}} : RGB{{0, 0, 0}}};
  for (int lb = 0; lb < 2; ++lb) {
    for (uint32_t l = 0; l < b.nl; ++l) {
      const float sc = lv.lscale[(e * 2 + lb) * b.nl + l];
      if (sc == 0.0f) continue;
      RGB col{{0, 0, 0}};
      const uint32_t slot0 = (uint32_t)((e * 2 + lb) * b.nl + l) * lv.ns;
      for (uint32_t k = 0; k < lv.ns; ++k) {
        if (!lv.slot_live[slot0 + k]) continue;
        const float* v = lv.slot_rgb + (size_t)(slot0 + k) * 3;
        col.c[0] += v[0];
        col.c[1] += v[1];
        col.c[2] += v[2];
      }
      if (sc > 0.0f)
        for (float& v : col.c) v *= sc;
      for (int k = 0; k < 3; ++k) col.c[k] *= colour[lb].c[k];
      for (int k = 0; k < 3; ++k) lobe[lb].c[k] += col.c[k];
    }
    if (lb == 0 && dw > 0.0f)
      for (float& v : lobe[0].c) v *= dw;
  }
  const float* w = lv.mw + e * 4;
  if (w[3] >= 0.0f) {  // mirror
    RGB sp{{0, 0, 0}};
    if (child_hit)
      for (int k = 0; k < 3; ++k) {
        float v = w[k] * child.c[k];
        if (v < 0 || isnan(v)) v = 0;
        sp.c[k] = 0.0f + v;
      }
    for (int k = 0; k < 3; ++k) lobe[1].c[k] = sp.c[k] * (w[3] / 1.0f);
  }
  for (int k = 0; k < 3; ++k) c.c[k] = ((0.0f + lv.emis[e * 3 + k]) + lobe[0].c[k]) + lobe[1].c[k];
  return c;
}

// Per pixel, the batch's iterations in order: each sample's chain of mirror
// reflections evaluated from the deepest level up, then
// buf = (buf*iter + c)/(iter+1).
__global__ void k_accumulate(RenderBatch b, uint32_t iters) {
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= b.npix) return;
  float f0 = b.fb[pix * 3], f1 = b.fb[pix * 3 + 1], f2 = b.fb[pix * 3 + 2];
  for (uint32_t it = 0; it < iters; ++it) {
    const uint64_t s = (uint64_t)it * b.npix + pix;
    const uint32_t j = b.iter0 + it + 1;
    int64_t chain[kMaxLevel + 1];
    int depth = 0;
    chain[0] = (int64_t)s;
    while (depth < kMaxLevel && depth + 1 < (int)b.levels && b.lv[depth].shader[chain[depth]] >= 0 &&
           b.lv[depth].child[chain[depth]] >= 0) {
      chain[depth + 1] = b.lv[depth].child[chain[depth]];
      ++depth;
    }
    RGB res{{0, 0, 0}};
    bool hit = false;
    for (int l = depth; l >= 0; --l) {
      const Level& lv = b.lv[l];
      if (lv.shader[chain[l]] < 0) {  // core.Trace returned false
        hit = false;
        res = RGB{{0, 0, 0}};
        continue;
      }
      res = entry_colour(b, lv, (uint64_t)chain[l], hit, res);
      hit = true;
    }
    const RGB c = hit ? res : RGB{{0, 0, 0}};
    f0 = (f0 * (float)j + c.c[0]) / (float)(j + 1);
    f1 = (f1 * (float)j + c.c[1]) / (float)(j + 1);
    f2 = (f2 * (float)j + c.c[2]) / (float)(j + 1);
  }
  b.fb[pix * 3] = f0;
  b.fb[pix * 3 + 1] = f1;
  b.fb[pix * 3 + 2] = f2;
}

}  // namespace

// The RasterXY tables for m = 12 from the generator matrices (the same
// derivation as the oracle's; pinned against the reference's tables).
void raster_tables_m12(uint64_t fwd[52], uint64_t inv[52]) {
  const uint32_t m = 12, n = 2 * m;
  auto vdc_h = [](uint64_t i) {
    uint64_t r = 0;
    for (int k = 0; k < 64; ++k)
      if ((i >> k) & 1) r |= 1ull << (63 - k);
    return r >> 12;
  };
  auto sobol_h = [](uint64_t i) {
    uint64_t r = 0;
    for (uint64_t v = 1ull << 51; i != 0; i >>= 1) {
      if (i & 1) r ^= v;
      v ^= v >> 1;
    }
    return r;
  };
  auto bits = [&](uint64_t idx) { return ((vdc_h(idx) >> (52 - m)) << m) | (sobol_h(idx) >> (52 - m)); };
  for (int c = 0; c < 52; ++c) { fwd[c] = 0; inv[c] = 0; }
  for (uint32_t c = 0; n + c < 52; ++c) fwd[c] = bits(1ull << (n + c));
  uint64_t a[52], e[52];
  for (uint32_t r = 0; r < n; ++r) {
    a[r] = 0;
    for (uint32_t k = 0; k < n; ++k)
      if ((bits(1ull << k) >> r) & 1) a[r] |= 1ull << k;
    e[r] = 1ull << r;
  }
  for (uint32_t col = 0; col < n; ++col) {
    uint32_t p = col;
    while (p < n && !((a[p] >> col) & 1)) ++p;
    if (p == n) return;
    std::swap(a[p], a[col]);
    std::swap(e[p], e[col]);
    for (uint32_t r = 0; r < n; ++r)
      if (r != col && ((a[r] >> col) & 1)) { a[r] ^= a[col]; e[r] ^= e[col]; }
  }
  for (uint32_t c = 0; c < n; ++c) {
    uint64_t x = 0;
    for (uint32_t k = 0; k < n; ++k)
      if ((e[k] >> c) & 1) x |= 1ull << k;
    inv[c] = x;
  }
}

}  // namespace vmr

namespace {

int rfail(vmr_ctx* ctx, int code, const std::string& msg) {
  ctx->err = msg;
  return code;
}
#define RCUDA(call)                                                                  \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return rfail(ctx, e_ == cudaErrorMemoryAllocation ? VMR_ERR_OOM : VMR_ERR_CUDA, \
                   std::string(#call) + ": " + cudaGetErrorString(e_));              \
  } while (0)

}  // namespace

namespace vmr {
// The camera as the kernels see it: m replaced by the matrix the reference
// computes from it, TransformDecompToMatrix4(TransformDecompLerp(d, d, 0))
// of d = TransformDecompMatrix4(m) (camera.go:207-236), which is not m.
vmr_camera camera_round_trip(const vmr_camera& c) {
  vmr_camera o = c;
  anim::Decomp d;
  anim::decompose(c.m, d);
  anim::at_time(&d, 1, 0.0f, true, o.m);
  return o;
}
}  // namespace vmr

extern "C" {

int vmr_set_shaders(vmr_ctx* ctx, const vmr_shader_std* shaders, uint32_t n) {
  if (!ctx || (n && !shaders)) return VMR_ERR_INVALID;
  ctx->render.shaders.assign(shaders, shaders + n);
  return VMR_OK;
}

int vmr_mesh_set_shading(vmr_ctx* ctx, uint32_t geom, const uint32_t* shaders, uint32_t n_shaders, const float* normals) {
  if (!ctx || geom >= ctx->meshes.size() || (n_shaders && !shaders)) return VMR_ERR_INVALID;
  MeshRec& rec = *ctx->meshes[geom];
  if (rec.host.group) return rfail(ctx, VMR_ERR_UNSUPPORTED, "an instance or Proc shades through its geoms");
  if (rec.host.motion() && normals)
    return rfail(ctx, VMR_ERR_UNSUPPORTED,
                 "a motion mesh takes keyed normals through vmr_mesh_set_motion_normals (its hits ignore "
                 "one-key normals, trace.go:694-712)");
  rec.shader_list.assign(shaders, shaders + n_shaders);
  rec.has_normals = normals != nullptr;
  if (ctx->device < 0) return VMR_OK;
  cudaSetDevice(ctx->device);
  const HostMesh& m = rec.host;
  if (!m.shader_idx.empty()) {
    RCUDA(rec.sidx.ensure(m.shader_idx.size()));
    RCUDA(cudaMemcpy(rec.sidx.p, m.shader_idx.data(), m.shader_idx.size(), cudaMemcpyHostToDevice));
  }
  if (normals) {
    std::vector<float4> nrm((size_t)m.n_tris * 3);
    for (size_t i = 0; i < nrm.size(); ++i) {
      const float* v = normals + (size_t)m.idxp[i] * 3;
      nrm[i] = make_float4(v[0], v[1], v[2], 0.f);
    }
    RCUDA(rec.nrm.ensure(nrm.size() * sizeof(float4)));
    RCUDA(cudaMemcpy(rec.nrm.p, nrm.data(), nrm.size() * sizeof(float4), cudaMemcpyHostToDevice));
  }
  if (m.motion()) {  // vertices and face-order idxp for the hit attributes
    std::vector<float4> av((size_t)m.keys * m.n_verts);
    for (size_t i = 0; i < av.size(); ++i) av[i] = make_float4(m.verts[i * 3], m.verts[i * 3 + 1], m.verts[i * 3 + 2], 0.f);
    RCUDA(rec.avert.ensure(av.size() * sizeof(float4)));
    RCUDA(cudaMemcpy(rec.avert.p, av.data(), av.size() * sizeof(float4), cudaMemcpyHostToDevice));
    RCUDA(rec.aidx.ensure(m.idxp.size() * 4));
    RCUDA(cudaMemcpy(rec.aidx.p, m.idxp.data(), m.idxp.size() * 4, cudaMemcpyHostToDevice));
  }
  RCUDA(rec.shlist.ensure(std::max<size_t>(1, n_shaders) * 4));
  if (n_shaders) RCUDA(cudaMemcpy(rec.shlist.p, shaders, n_shaders * 4, cudaMemcpyHostToDevice));
  return VMR_OK;
}

int vmr_mesh_set_motion_normals(vmr_ctx* ctx, uint32_t geom, const float* normals, uint32_t n_per_key,
                                uint32_t keys) {
  if (!ctx || geom >= ctx->meshes.size()) return VMR_ERR_INVALID;
  MeshRec& rec = *ctx->meshes[geom];
  if (!normals) {
    rec.mnrm_n = 0;
    return VMR_OK;
  }
  const HostMesh& m = rec.host;
  if (!m.motion() || m.group || m.sphere) return rfail(ctx, VMR_ERR_INVALID, "motion normals need a motion mesh");
  if (keys != m.keys) return rfail(ctx, VMR_ERR_INVALID, "motion normals need as many keys as the mesh's vertices");
  if ((uint64_t)n_per_key < 3ull * m.n_tris)
    return rfail(ctx, VMR_ERR_INVALID, "motion normals: fewer than three entries per triangle");
  if (ctx->device < 0) {
    rec.mnrm_n = n_per_key;
    return VMR_OK;
  }
  cudaSetDevice(ctx->device);
  std::vector<float4> nv((size_t)keys * n_per_key);
  for (size_t i = 0; i < nv.size(); ++i) nv[i] = make_float4(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2], 0.f);
  RCUDA(rec.mnrm.ensure(nv.size() * sizeof(float4)));
  RCUDA(cudaMemcpy(rec.mnrm.p, nv.data(), nv.size() * sizeof(float4), cudaMemcpyHostToDevice));
  rec.mnrm_n = n_per_key;
  return VMR_OK;
}

int vmr_set_lights(vmr_ctx* ctx, const vmr_tri_light* lights, uint32_t n) {
  if (!ctx || (n && !lights)) return VMR_ERR_INVALID;
  for (uint32_t i = 0; i < n; ++i)
    if (lights[i].samples < 0 || (1 << lights[i].samples) > 2 * vmr::kMaxHalf)
      return rfail(ctx, VMR_ERR_UNSUPPORTED, "TriLight samples must be in [0, 4]");
  ctx->render.lights.assign(lights, lights + n);
  return VMR_OK;
}

int vmr_set_disk_lights(vmr_ctx* ctx, const vmr_disk_light* lights, uint32_t n) {
  if (!ctx || (n && !lights)) return VMR_ERR_INVALID;
  for (uint32_t i = 0; i < n; ++i) {
    if (lights[i].samples < 0 || (1 << lights[i].samples) > 2 * vmr::kMaxHalf)
      return rfail(ctx, VMR_ERR_UNSUPPORTED, "DiskLight samples must be in [0, 4]");
    if (!(lights[i].radius > 0.0f)) return rfail(ctx, VMR_ERR_INVALID, "DiskLight radius must be positive");
  }
  ctx->render.disks.assign(lights, lights + n);
  return VMR_OK;
}

int vmr_set_sphere_lights(vmr_ctx* ctx, const vmr_sphere_light* lights, uint32_t n) {
  if (!ctx || (n && !lights)) return VMR_ERR_INVALID;
  for (uint32_t i = 0; i < n; ++i) {
    if (lights[i].samples < 0 || (1 << lights[i].samples) > 2 * vmr::kMaxHalf)
      return rfail(ctx, VMR_ERR_UNSUPPORTED, "SphereLight samples must be in [0, 4]");
    if (!(lights[i].radius > 0.0f)) return rfail(ctx, VMR_ERR_INVALID, "SphereLight radius must be positive");
  }
  ctx->render.spheres.assign(lights, lights + n);
  return VMR_OK;
}


int vmr_set_camera(vmr_ctx* ctx, const vmr_camera* cam) {
  if (!ctx || !cam) return VMR_ERR_INVALID;
  if (!(cam->radius >= 0.0f)) return rfail(ctx, VMR_ERR_INVALID, "camera radius must be >= 0");
  auto& R = ctx->render;
  R.camera = *cam;
  R.has_camera = true;
  R.cam_keys.resize(1);
  vmr::anim::decompose(cam->m, R.cam_keys[0]);
  R.cam_key_m.assign(cam->m, cam->m + 16);
  R.cam_used = vmr::camera_round_trip(*cam);
  return VMR_OK;
}

int vmr_get_camera_keys(vmr_ctx* ctx, float* keys16, uint32_t cap, uint32_t* n_keys) {
  if (!ctx || !n_keys) return VMR_ERR_INVALID;
  const auto& R = ctx->render;
  if (!R.has_camera) return rfail(ctx, VMR_ERR_INVALID, "no camera set");
  const uint32_t n = (uint32_t)(R.cam_key_m.size() / 16);
  *n_keys = n;
  if (keys16) std::memcpy(keys16, R.cam_key_m.data(), sizeof(float) * 16 * std::min(n, cap));
  return VMR_OK;
}

int vmr_transform_keys_at(const float* keys16, uint32_t n_keys, float time, int blend_one, float* out16) {
  if (!keys16 || !out16 || n_keys < 1) return VMR_ERR_INVALID;
  std::vector<vmr::anim::Decomp> k(n_keys);
  for (uint32_t i = 0; i < n_keys; ++i) vmr::anim::decompose(keys16 + 16 * i, k[i]);
  return vmr::anim::at_time(k.data(), n_keys, time, blend_one != 0, out16) ? VMR_OK : VMR_ERR_INVALID;
}

int vmr_set_camera_keys(vmr_ctx* ctx, const float* keys16, uint32_t n_keys) {
  if (!ctx || !keys16 || n_keys < 1) return VMR_ERR_INVALID;
  auto& R = ctx->render;
  if (!R.has_camera) return rfail(ctx, VMR_ERR_INVALID, "set the camera (vmr_set_camera) before its keys");
  vmr_camera c = R.camera;
  std::memcpy(c.m, keys16, sizeof(c.m));
  int rc = vmr_set_camera(ctx, &c);
  if (rc != VMR_OK || n_keys == 1) return rc;
  R.cam_keys.resize(n_keys);
  for (uint32_t i = 0; i < n_keys; ++i) vmr::anim::decompose(keys16 + 16 * i, R.cam_keys[i]);
  R.cam_key_m.assign(keys16, keys16 + 16 * (size_t)n_keys);
  if (ctx->device >= 0) {
    cudaSetDevice(ctx->device);
    RCUDA(R.dcam_keys.ensure(sizeof(vmr::anim::Decomp) * n_keys));
    RCUDA(cudaMemcpy(R.dcam_keys.p, R.cam_keys.data(), sizeof(vmr::anim::Decomp) * n_keys, cudaMemcpyHostToDevice));
  }
  return VMR_OK;
}

int vmr_render(vmr_ctx* ctx, const vmr_render_params* p, float* fb, vmr_render_stats* stats) {
  using namespace vmr;
  if (!ctx || !p || !fb) return VMR_ERR_INVALID;
  if (ctx->device < 0) return rfail(ctx, VMR_ERR_UNSUPPORTED, "host-only context cannot render");
  if (!ctx->top.valid) return rfail(ctx, VMR_ERR_INVALID, "no scene: call vmr_scene_build first");
  if (!ctx->render.has_camera) return rfail(ctx, VMR_ERR_INVALID, "no camera");
  if (p->width == 0 || p->height == 0 || p->width > 4096 || p->height > 4096)
    return rfail(ctx, VMR_ERR_INVALID, "image size must be in [1, 4096] (RasterXY uses m = 12)");
  if (p->row_count && (p->row_begin >= p->height || p->row_count > p->height - p->row_begin))
    return rfail(ctx, VMR_ERR_INVALID, "row band outside the image");
  if (!p->row_count && p->row_begin) return rfail(ctx, VMR_ERR_INVALID, "row_begin without row_count");
  const uint32_t row0 = p->row_count ? p->row_begin : 0u, nrows = p->row_count ? p->row_count : p->height;
  if (p->flags & ~(uint32_t)VMR_RENDER_F32) return rfail(ctx, VMR_ERR_INVALID, "unknown render flags");
  const bool f32 = (p->flags & VMR_RENDER_F32) != 0;
  auto& R = ctx->render;
  for (const auto& L : R.lights)
    if (L.shader >= R.shaders.size() || L.geom >= ctx->meshes.size())
      return rfail(ctx, VMR_ERR_INVALID, "light shader or geom out of range");
  for (const auto& L : R.disks)
    if (L.shader >= R.shaders.size() || L.geom >= ctx->meshes.size())
      return rfail(ctx, VMR_ERR_INVALID, "disk light shader or geom out of range");
  for (const auto& L : R.spheres)
    if (L.shader >= R.shaders.size() || L.geom >= ctx->meshes.size())
      return rfail(ctx, VMR_ERR_INVALID, "sphere light shader or geom out of range");
  std::vector<uint32_t> shaded;  // the geoms whose shading data hits read
  for (uint32_t g : ctx->top.host.geom_order) {
    const MeshRec& gr = *ctx->meshes[g];
    if (gr.host.group == 2) shaded.insert(shaded.end(), gr.children.begin(), gr.children.end());
    else shaded.push_back(g);
  }
  for (uint32_t g : shaded) {
    const MeshRec& mr = shading_rec(ctx, g);
    if (mr.host.motion() && mr.aidx.p == nullptr)
      return rfail(ctx, VMR_ERR_INVALID, "a motion mesh in the scene has no shading (vmr_mesh_set_shading)");
    for (uint32_t sid : mr.shader_list)
      if (sid >= R.shaders.size()) return rfail(ctx, VMR_ERR_INVALID, "mesh shader id out of range");
  }
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  // Scene tables.
  const std::vector<RMesh> rm = rmesh_table(ctx);
  // Instances, Procs or keyed transforms in the scene: the shading kernel
  // with the group and keyed-transform helpers (and their registers).
  bool groups = false;
  for (const RMesh& r : rm) groups = groups || r.outer_nkeys != 0 || r.xf_nkeys >= 2;
  std::vector<RLight> rl(R.lights.size() + R.disks.size() + R.spheres.size());
  uint32_t ns = 1;
  for (size_t i = 0; i < R.lights.size(); ++i) {
    rl[i] = RLight{};
    std::memcpy(rl[i].p, R.lights[i].p0, 12);
    std::memcpy(rl[i].p + 3, R.lights[i].p1, 12);
    std::memcpy(rl[i].p + 6, R.lights[i].p2, 12);
    rl[i].samples = R.lights[i].samples;
    rl[i].shader = R.lights[i].shader;
    rl[i].geom = R.lights[i].geom;
    rl[i].kind = 0;
    ns = std::max<uint32_t>(ns, 1u << R.lights[i].samples);
  }
  for (size_t k = 0; k < R.disks.size(); ++k) {  // Disk.PreRender frame (disk.go:88-90), host float math
    const vmr_disk_light& d = R.disks[k];
    RLight& L = rl[R.lights.size() + k];
    L = RLight{};
    L.kind = 1;
    L.samples = d.samples;
    L.shader = d.shader;
    L.geom = d.geom;
    L.radius = d.radius;
    std::memcpy(L.P, d.P, 12);
    auto nrm = [](const float* a, float* o) {
      const float r = 1.0f / std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
      o[0] = a[0] * r; o[1] = a[1] * r; o[2] = a[2] * r;
    };
    auto crs = [](const float* a, const float* b, float* o) {
      o[0] = a[1] * b[2] - a[2] * b[1];
      o[1] = a[2] * b[0] - a[0] * b[2];
      o[2] = a[0] * b[1] - a[1] * b[0];
    };
    const float dn[3] = {d.lookat[0] - d.P[0], d.lookat[1] - d.P[1], d.lookat[2] - d.P[2]};
    nrm(dn, L.N);
    float t[3];
    crs(L.N, d.up, t);
    nrm(t, L.T);
    crs(L.N, L.T, L.B);
    ns = std::max<uint32_t>(ns, 1u << d.samples);
  }
  for (size_t k = 0; k < R.spheres.size(); ++k) {
    const vmr_sphere_light& d = R.spheres[k];
    RLight& L = rl[R.lights.size() + R.disks.size() + k];
    L = RLight{};
    L.kind = 2;
    L.samples = d.samples;
    L.shader = d.shader;
    L.geom = d.geom;
    L.radius = d.radius;
    std::memcpy(L.P, d.P, 12);
    ns = std::max<uint32_t>(ns, 1u << d.samples);
  }
  const uint32_t nl = (uint32_t)rl.size();
  const uint32_t npix = p->width * nrows;
  uint32_t per_batch = p->max_batch_samples ? p->max_batch_samples : (4u << 20);
  uint32_t iters_per_batch = std::max<uint32_t>(1, per_batch / npix);
  if (iters_per_batch > p->iter_count) iters_per_batch = std::max<uint32_t>(1, p->iter_count);
  const uint64_t nmax = (uint64_t)iters_per_batch * npix;
  const uint64_t nslots = nmax * 2 * nl * ns;
  // Mirror levels get storage only when a shader is a mirror.
  bool has_mirror = false;
  for (const auto& sh : R.shaders)
    if ((sh.flags & VMR_SH_SPEC1_STRENGTH) && sh.spec1_strength > 0.0f && (sh.flags & VMR_SH_SPEC1_ROUGHNESS) &&
        sh.spec1_roughness == 0.0f)
      has_mirror = true;
  const uint32_t levels = has_mirror ? (uint32_t)kMaxLevel + 1 : 1u;
  // Device buffers (one block, carved).
  const size_t fsz = 4;
  size_t bytes = 0;
  auto carve = [&](size_t nbytes) { size_t o = bytes; bytes += (nbytes + 255) / 256 * 256; return o; };
  size_t o_lv[kMaxLevel + 1][10];
  for (uint32_t l = 0; l < levels; ++l) {
    const uint64_t cap = nmax;
    const uint32_t lns = l == 0 ? ns : 1u;
    const uint64_t lslots = cap * 2 * nl * lns;
    o_lv[l][0] = carve(cap * 8 * fsz);                 // rays
    o_lv[l][1] = carve(l == 0 ? 0 : cap * 4);          // samp
    o_lv[l][2] = carve(cap * 6 * 4);                   // hits
    o_lv[l][3] = carve(cap * 4);                       // shader
    o_lv[l][4] = carve(cap * 3 * fsz);                 // emis
    o_lv[l][5] = carve(lslots * 3 * fsz);              // slot rgb
    o_lv[l][6] = carve(lslots);                        // slot live
    o_lv[l][7] = carve(cap * 2 * nl * fsz);            // lscale
    o_lv[l][8] = carve(cap * 4 * fsz);                 // mirror weight
    o_lv[l][9] = carve(cap * 4);                       // child
  }
  const size_t o_lambda = carve(nmax * fsz), o_q = carve(std::max<uint64_t>(1, nslots) * 8 * fsz),
               o_back = carve(std::max<uint64_t>(1, nslots) * 4), o_shit = carve(std::max<uint64_t>(1, nslots) * 4),
               o_cnt = carve(128), o_fb = carve((size_t)npix * 3 * fsz), o_meshes = carve(rm.size() * sizeof(RMesh)),
               o_lights = carve(std::max<size_t>(1, rl.size()) * sizeof(RLight)),
               o_shaders = carve(std::max<size_t>(1, R.shaders.size()) * sizeof(vmr_shader_std));
  RCUDA(R.buf.ensure(bytes));
  char* base = R.buf.as<char>();
  uint64_t fwd[52], inv[52];
  raster_tables_m12(fwd, inv);
  RCUDA(cudaMemcpyToSymbolAsync(c_raster_fwd, fwd, sizeof(fwd), 0, cudaMemcpyHostToDevice, st));
  RCUDA(cudaMemcpyToSymbolAsync(c_raster_inv, inv, sizeof(inv), 0, cudaMemcpyHostToDevice, st));
  RCUDA(cudaMemcpyAsync(base + o_meshes, rm.data(), rm.size() * sizeof(RMesh), cudaMemcpyHostToDevice, st));
  if (!rl.empty()) RCUDA(cudaMemcpyAsync(base + o_lights, rl.data(), rl.size() * sizeof(RLight), cudaMemcpyHostToDevice, st));
  if (!R.shaders.empty())
    RCUDA(cudaMemcpyAsync(base + o_shaders, R.shaders.data(), R.shaders.size() * sizeof(vmr_shader_std), cudaMemcpyHostToDevice, st));
  RCUDA(cudaMemcpyAsync(base + o_fb, fb, (size_t)npix * 3 * fsz, cudaMemcpyHostToDevice, st));
  RenderBatch b{};
  b.width = p->width;
  b.height = p->height;
  b.npix = npix;
  b.pix0 = row0 * p->width;
  b.nl = nl;
  b.levels = levels;
  b.seed = p->seed;
  b.cam = R.cam_used;
  b.cam_nkeys = R.cam_keys.size() >= 2 ? (uint32_t)R.cam_keys.size() : 0u;
  b.cam_keys = b.cam_nkeys ? R.dcam_keys.as<const anim::Decomp>() : nullptr;
  b.filt = PixFilter{R.filter_n ? R.filter.as<const double>() : nullptr, R.filter_n, R.filter_w};
  b.shaders = reinterpret_cast<const vmr_shader_std*>(base + o_shaders);
  b.lights = reinterpret_cast<const RLight*>(base + o_lights);
  b.meshes = reinterpret_cast<const RMesh*>(base + o_meshes);
  b.lambda = reinterpret_cast<float*>(base + o_lambda);
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(base + o_cnt);
  for (uint32_t l = 0; l < levels; ++l) {
    Level& L = b.lv[l];
    L.ray = reinterpret_cast<float*>(base + o_lv[l][0]);
    L.samp = l == 0 ? nullptr : reinterpret_cast<uint32_t*>(base + o_lv[l][1]);
    L.hit = reinterpret_cast<int32_t*>(base + o_lv[l][2]);
    L.shader = reinterpret_cast<int32_t*>(base + o_lv[l][3]);
    L.emis = reinterpret_cast<float*>(base + o_lv[l][4]);
    L.slot_rgb = reinterpret_cast<float*>(base + o_lv[l][5]);
    L.slot_live = reinterpret_cast<uint8_t*>(base + o_lv[l][6]);
    L.lscale = reinterpret_cast<float*>(base + o_lv[l][7]);
    L.mw = reinterpret_cast<float*>(base + o_lv[l][8]);
    L.child = reinterpret_cast<int32_t*>(base + o_lv[l][9]);
    L.ns = l == 0 ? ns : 1u;
    L.cap = (uint32_t)nmax;
    L.count = cnt + 2 + l;
  }
  const uint64_t qcap = std::max<uint64_t>(1, nslots);
  float* q = reinterpret_cast<float*>(base + o_q);
  b.sx = q; b.sy = q + qcap; b.sz = q + 2 * qcap; b.sdx = q + 3 * qcap; b.sdy = q + 4 * qcap;
  b.sdz = q + 5 * qcap; b.stmax = q + 6 * qcap; b.stime = q + 7 * qcap;
  b.sback = reinterpret_cast<uint32_t*>(base + o_back);
  b.shit = reinterpret_cast<int32_t*>(base + o_shit);
  b.queue_len = cnt;
  b.status = reinterpret_cast<int*>(cnt + 1);
  b.queue_cap = (uint32_t)std::min<uint64_t>(qcap, 0xffffffffu);
  b.fb = reinterpret_cast<float*>(base + o_fb);
  RCUDA(cudaMemsetAsync(b.status, 0, 4, st));
  RCUDA(cudaEventRecord(ctx->rev0, st));
  uint64_t n_shadow = 0, n_cam = 0;
  for (uint32_t it0 = 0; it0 < p->iter_count; it0 += iters_per_batch) {
    const uint32_t iters = std::min(iters_per_batch, p->iter_count - it0);
    b.iter0 = p->iter_begin + it0;
    b.n = iters * npix;
    const int blk = 128;
    const int grid = (int)((b.n + blk - 1) / blk);
    RCUDA(cudaMemsetAsync(cnt + 2, 0, sizeof(unsigned long long) * (kMaxLevel + 1), st));
    if (b.cam_nkeys >= 2) k_generate<true><<<grid, blk, 0, st>>>(b);
    else k_generate<false><<<grid, blk, 0, st>>>(b);
    RCUDA(cudaGetLastError());
    for (uint32_t l = 0; l < levels; ++l) {
      const Level& L = b.lv[l];
      uint64_t ne = b.n;
      if (l > 0) {  // mirror reflections queued by the level below
        unsigned long long c = 0;
        RCUDA(cudaMemcpyAsync(&c, L.count, 8, cudaMemcpyDeviceToHost, st));
        RCUDA(cudaStreamSynchronize(st));
        ne = std::min<uint64_t>(c, L.cap);
        if (ne == 0) break;
      }
      const uint64_t cap = L.cap;
      vmr_rays rr{L.ray, L.ray + cap, L.ray + 2 * cap, L.ray + 3 * cap, L.ray + 4 * cap, L.ray + 5 * cap,
                  L.ray + 6 * cap, L.ray + 7 * cap};
      float* hf = reinterpret_cast<float*>(L.hit);
      vmr_hits hh{L.hit, L.hit + cap, hf + 2 * cap, hf + 3 * cap, hf + 4 * cap, hf + 5 * cap};
      int rc = vmr_trace_scene(ctx, &rr, ne, VMR_TRACE_DEVICE, &hh, nullptr);
      if (rc != VMR_OK) return rc;
      RCUDA(cudaMemsetAsync(b.queue_len, 0, 8, st));
      const int nblk = (int)((ne + blk - 1) / blk);
      if (f32) {
        if (groups) k_shade<true, true><<<nblk, blk, 0, st>>>(b, l);
        else k_shade<true, false><<<nblk, blk, 0, st>>>(b, l);
      } else {
        if (groups) k_shade<false, true><<<nblk, blk, 0, st>>>(b, l);
        else k_shade<false, false><<<nblk, blk, 0, st>>>(b, l);
      }
      RCUDA(cudaGetLastError());
      unsigned long long nq = 0;
      RCUDA(cudaMemcpyAsync(&nq, b.queue_len, 8, cudaMemcpyDeviceToHost, st));
      RCUDA(cudaStreamSynchronize(st));
      if (nq > b.queue_cap) return rfail(ctx, VMR_ERR_QUEUE_OVERFLOW, "shadow-ray queue overflow");
      if (nq) {
        vmr_rays sr{b.sx, b.sy, b.sz, b.sdx, b.sdy, b.sdz, b.stmax, b.stime};
        vmr_hits sh{b.shit, nullptr, nullptr, nullptr, nullptr, nullptr};
        // EvaluateLightSamples uses only TraceProbe's yes/no for its shadow
        // rays (core/shader.go:276,317,380; core/trace.go:23-35), which does
        // not depend on the traversal order: a scene that flattens answers
        // it from one tree
        bool flat = false;
        rc = vmr::trace_flat_any_hit(ctx, sr, nq, sh, &flat);
        if (rc == VMR_OK && !flat) rc = vmr_trace_scene(ctx, &sr, nq, VMR_TRACE_DEVICE | VMR_TRACE_ANY_HIT, &sh, nullptr);
        if (rc != VMR_OK) return rc;
        k_resolve<<<(int)((nq + 255) / 256), 256, 0, st>>>(b, l, (uint32_t)nq);
        RCUDA(cudaGetLastError());
      }
      n_shadow += nq;
      if (l == 0) n_cam += ne;
    }
    k_accumulate<<<(int)((npix + 127) / 128), 128, 0, st>>>(b, iters);
    RCUDA(cudaGetLastError());
  }
  RCUDA(cudaEventRecord(ctx->rev1, st));
  RCUDA(cudaMemcpyAsync(fb, b.fb, (size_t)npix * 3 * fsz, cudaMemcpyDeviceToHost, st));
  int status = 0;
  RCUDA(cudaMemcpyAsync(&status, b.status, 4, cudaMemcpyDeviceToHost, st));
  RCUDA(cudaStreamSynchronize(st));
  if (status > kStatusIterationCap) return rfail(ctx, VMR_ERR_INVALID, "a shader has no weight (ShaderStd panics)");
  int trs = vmr_sync(ctx);
  if (trs != VMR_OK) return trs;
  if (stats) {
    stats->samples = (uint64_t)npix * p->iter_count;
    stats->camera_rays = n_cam;
    stats->shadow_rays = n_shadow;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->rev0, ctx->rev1);
    stats->ms = ms;
  }
  return VMR_OK;
}

}  // extern "C"
