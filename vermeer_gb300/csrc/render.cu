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

#include <cstring>
#include <string>
#include <vector>

#include "colour_tables.h"
#include "ctx.h"
#include "device.h"
#include "vmr.h"

namespace vmr {
namespace {

// -------------------------------------------------------------- vectors ---
struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 scale(float s, V3 a) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float len2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ V3 normalize(V3 a) {
  const float r = 1.0f / sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
  return v3(a.x * r, a.y * r, a.z * r);
}
__device__ __forceinline__ float length(V3 a) { return sqrtf((a.x * a.x + a.y * a.y) + a.z * a.z); }
__device__ __forceinline__ float gmax(float x, float y) { return x > y ? x : y; }
__device__ __forceinline__ float gmin(float x, float y) { return x < y ? x : y; }
__device__ __forceinline__ float sqr(float v) { return v * v; }
constexpr float kPi = 3.14159265358f;  // math.Pi (math/const.go:8) as float32
__device__ __forceinline__ float gsin(float x) { return (float)sin((double)x); }
__device__ __forceinline__ float gcos(float x) { return (float)cos((double)x); }
__device__ __forceinline__ float gtan(float x) { return (float)tan((double)x); }
__device__ __forceinline__ float gatan(float x) { return (float)atan((double)x); }
__device__ __forceinline__ float gatan2(float y, float x) { return (float)atan2((double)y, (double)x); }
__device__ __forceinline__ float gacos(float x) {
  return (float)acos((double)(x > 1.0f ? 1.0f : (x < -1.0f ? -1.0f : x)));
}
__device__ __forceinline__ V3 project(V3 U, V3 V, V3 W, V3 s) { return v3(dot(U, s), dot(V, s), dot(W, s)); }
__device__ __forceinline__ V3 expand(V3 U, V3 V, V3 W, V3 s) {
  return v3(U.x * s.x + V.x * s.y + W.x * s.z, U.y * s.x + V.y * s.y + W.y * s.z, U.z * s.x + V.z * s.y + W.z * s.z);
}

// ------------------------------------------------------------------ QMC ---
__device__ __forceinline__ uint64_t vdc_bits(uint64_t i, uint64_t s) { return (s ^ __brevll(i)) >> 12; }
__device__ __forceinline__ uint64_t sobol_bits(uint64_t i, uint64_t s) {
  uint64_t r = s >> 12;
  for (uint64_t v = 1ull << 51; i != 0; i >>= 1) {
    if (i & 1) r ^= v;
    v ^= v >> 1;
  }
  return r;
}
constexpr double kTwo52 = 4503599627370496.0;
__device__ __forceinline__ double vdc(uint64_t i, uint64_t s) { return (double)vdc_bits(i, s) / kTwo52; }
__device__ __forceinline__ double sobol(uint64_t i, uint64_t s) { return (double)sobol_bits(i, s) / kTwo52; }
__device__ __forceinline__ uint64_t scramble(uint64_t seed, uint64_t pix, uint32_t k) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (pix * 8ull + k + 1ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// RasterXY tables for m = 12 (the Grunschloss enumeration, computed on the
// host from the generator matrices).
__constant__ uint64_t c_raster_fwd[52];
__constant__ uint64_t c_raster_inv[52];

// ldseq.RasterXY(12, frame, px, py, 0, 0) (math/ldseq/raster.go:10-57).
__device__ void raster_xy(uint32_t frame, uint32_t px, uint32_t py, double& rx, double& ry) {
  const uint32_t m = 12;
  uint64_t index = (uint64_t)frame << (2 * m);
  uint64_t delta = 0;
  for (uint32_t c = 0; frame != 0; frame >>= 1, ++c)
    if (frame & 1) delta ^= c_raster_fwd[c];
  uint64_t b = (((uint64_t)px << m) | (uint64_t)py) ^ delta;
  for (uint32_t c = 0; b != 0; b >>= 1, ++c)
    if (b & 1) index ^= c_raster_inv[c];
  const double sc = (double)(1ull << (52 - m));
  rx = (double)vdc_bits(index, 0) / sc;
  ry = (double)sobol_bits(index, 0) / sc;
}

// ------------------------------------------------------------- spectrum ---
struct RGB {
  float c[3];
};
struct Spec {
  float c[4];
};
__device__ __forceinline__ float wavelength(float lambda, int j) {  // Spectrum.Wavelength
  float v = (lambda - 450.0f + ((float)j / 4.0f) * 300.0f);
  if (v >= 300.0f) v -= 300.0f;
  return v + 450.0f;
}
__device__ __forceinline__ float smits_eval(const float* s, float l) {
  if (l < 380.0f || l >= 720.0f) return 0.0f;
  return s[(int)(((l - 380.0f) / (720.0f - 380.0f)) * 10.0f)];
}
__device__ float smits(float r, float g, float b, float l) {  // RGBToSpectrumSmits99
  float c = 0.0f;
  if (r <= g && r <= b) {
    c += r * smits_eval(kSmitsWhite, l);
    if (g <= b) {
      c += (g - r) * smits_eval(kSmitsCyan, l);
      c += (b - g) * smits_eval(kSmitsBlue, l);
    } else {
      c += (b - r) * smits_eval(kSmitsCyan, l);
      c += (g - b) * smits_eval(kSmitsGreen, l);
    }
  } else if (g <= r && g <= b) {
    c += g * smits_eval(kSmitsWhite, l);
    if (r <= b) {
      c += (r - g) * smits_eval(kSmitsMagenta, l);
      c += (b - r) * smits_eval(kSmitsBlue, l);
    } else {
      c += (b - g) * smits_eval(kSmitsMagenta, l);
      c += (r - b) * smits_eval(kSmitsRed, l);
    }
  } else {
    c += b * smits_eval(kSmitsWhite, l);
    if (r <= g) {
      c += (r - b) * smits_eval(kSmitsYellow, l);
      c += (g - r) * smits_eval(kSmitsGreen, l);
    } else {
      c += (g - b) * smits_eval(kSmitsYellow, l);
      c += (r - g) * smits_eval(kSmitsRed, l);
    }
  }
  return c;
}
__device__ __forceinline__ Spec from_rgb(RGB rgb, float lambda) {
  Spec s;
#pragma unroll
  for (int k = 0; k < 4; ++k) s.c[k] = smits(rgb.c[0], rgb.c[1], rgb.c[2], wavelength(lambda, k));
  return s;
}
__device__ __forceinline__ float cie(const float* t, float l) {
  if (l < 360.0f || l >= 830.0f) return -1.0f;
  return t[(int)(((l - 360.0f) / (830.0f - 360.0f)) * 95.0f)];
}
__device__ RGB to_rgb(const Spec& s, float lambda) {
  float x = 0, y = 0, z = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float l = wavelength(lambda, i);
    x += s.c[i] * cie(kCieX, l);
    y += s.c[i] * cie(kCieY, l);
    z += s.c[i] * cie(kCieZ, l);
  }
  const float* m = kSrgbFromXyz;
  return RGB{{x * m[0] + y * m[1] + z * m[2], x * m[3] + y * m[4] + z * m[5], x * m[6] + y * m[7] + z * m[8]}};
}

// -------------------------------------------------------------- fresnel ---
struct Fresnel {
  int model;
  float eta;
  RGB r, g;
};
__device__ RGB fresnel_kr(const Fresnel& f, float c) {
  if (f.model == 0) {  // Dielectric.Kr (fresnel/dielectric.go:34-47)
    float g = (f.eta * f.eta) - 1 + (c * c);
    if (g < 0.0f) return RGB{{1, 1, 1}};
    g = sqrtf(g);
    const float fr = 0.5f * sqr((g - c) / (g + c)) * (1 + sqr((c * (g + c) - 1) / (c * (g - c) + 1)));
    return RGB{{fr, fr, fr}};
  }
  RGB out;  // Conductor.Kr (fresnel/conductor.go:58-89)
  for (int k = 0; k < 3; ++k) {
    const float r = gmax(0.0f, gmin(f.r.c[k], 0.99f));
    const float g = f.g.c[k];
    const float nmin = (1 - r) / (1 + r);
    const float nmax = (1 + sqrtf(r)) / (1 - sqrtf(r));
    const float n = nmin * g + (1 - g) * nmax;
    const float k2 = ((n + 1) * (n + 1) * r - (n - 1) * (n - 1)) / (1 - r);
    const float rs = (n * n + k2 - 2 * n * c + c * c) / (n * n + k2 + 2 * n * c + c * c);
    const float rp = ((n * n + k2) * c * c - 2 * n * c + 1) / ((n * n + k2) * c * c + 2 * n * c + 1);
    out.c[k] = 0.5f * (rs + rp);
  }
  return out;
}

// ---------------------------------------------------------------- BSDFs ---
struct Bsdf {
  int kind;  // 0 OrenNayar, 1 GGX
  float lambda;
  V3 wi;
  float rough;  // roughness^2 as the constructors store it
  Fresnel fr;
  V3 U, V, N;
};
__device__ __forceinline__ float chi(float x) { return x > 0.0f ? 1.0f : 0.0f; }
__device__ __forceinline__ float signf(float v) { return v < 0 ? -1.0f : 1.0f; }
__device__ float ggx_g1(V3 w, V3 m, float alpha) {
  const float odn = dot(w, m);
  const float denom = 1 + sqrtf(1 + (alpha * alpha) * ((1.0f / (w.z * w.z)) - 1));
  return chi(odn / w.z) * 2 / denom;
}
__device__ float ggx_d(V3 m, float alpha) {
  const float numer = alpha * alpha * chi(m.z);
  if (m.z == 1.0f) return 1.0f / (kPi * alpha * alpha);
  const float denom = kPi * sqr(m.z * m.z) * sqr(alpha * alpha + ((1.0f / (m.z * m.z)) - 1));
  return numer / denom;
}
__device__ V3 bsdf_sample(const Bsdf& b, double r0, double r1) {
  if (b.kind == 0) {  // CosineHemisphere (math/sample/sample.go:18-27)
    const double r = sqrt(1 - r0), th = 2 * 3.14159265358979323846 * r1;
    return expand(b.U, b.V, b.N, v3((float)(r * cos(th)), (float)(r * sin(th)), (float)sqrt(r0)));
  }
  const float alpha = sqr(b.rough);  // MicrofacetGGX.Sample
  const double thetaM = atan2((double)alpha * sqrt(r0), sqrt(1 - r0));
  const double phiM = 2.0 * 3.14159265358979323846 * r1;
  const V3 m = v3(gsin((float)thetaM) * gcos((float)phiM), gsin((float)thetaM) * gsin((float)phiM), gcos((float)thetaM));
  const V3 wo = sub(scale(2.0f * fabsf(dot(m, b.wi)), m), b.wi);
  return expand(b.U, b.V, b.N, normalize(wo));
}
__device__ double bsdf_pdf(const Bsdf& b, V3 wo_world) {
  const V3 wo = project(b.U, b.V, b.N, wo_world);
  if (b.kind == 0) return (double)gmax(0.0f, wo.z) / 3.14159265358979323846;
  const float alpha = sqr(b.rough);
  const V3 m = scale(signf(b.wi.z), normalize(add(b.wi, wo)));
  const double pdf = (double)(ggx_d(m, alpha) * m.z);
  return isnan(pdf) ? 0.0 : pdf;
}
__device__ Spec bsdf_eval(const Bsdf& b, V3 wo_world) {
  const V3 wo = project(b.U, b.V, b.N, wo_world);
  if (b.kind == 0) {  // OrenNayar.Eval (bsdf/orennayar.go:42-73)
    const float sigma = b.rough;
    const float A = 1 - (0.5f * (sigma * sigma) / ((sigma * sigma) + 0.57f));
    const float B = 0.45f * (sigma * sigma) / ((sigma * sigma) + 0.09f);
    const float phiI = gatan2(b.wi.y, b.wi.x), phiO = gatan2(wo.y, wo.x);
    const float thetaI = gacos(b.wi.z), thetaO = gacos(wo.z);
    const float alpha = gmax(thetaI, thetaO), beta = gmin(thetaI, thetaO);
    const float C = gsin(alpha) * gtan(beta);
    const float gamma = gcos(phiO - phiI);
    const float s = wo.z * (A + (B * gmax(0.0f, gamma) * C));
    Spec rho = from_rgb(RGB{{1, 1, 1}}, b.lambda);
#pragma unroll
    for (int k = 0; k < 4; ++k) rho.c[k] *= s / kPi;
    return rho;
  }
  const float alpha = sqr(b.rough);  // MicrofacetGGX.Eval (microfacetggx.go:119-145)
  const V3 h = scale(signf(b.wi.z), normalize(add(b.wi, wo)));
  const RGB f = fresnel_kr(b.fr, fabsf(dot(b.wi, h)));
  const float numer = ggx_g1(b.wi, h, alpha) * ggx_g1(wo, h, alpha) * ggx_d(h, alpha);
  const float denom = 4 * fabsf(b.wi.z) * fabsf(wo.z);
  Spec rho = from_rgb(f, b.lambda);
  const float s = fabsf(wo.z) * numer / denom;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    rho.c[k] *= s;
    if (rho.c[k] < 0 || isnan(rho.c[k])) rho.c[k] = 0;
  }
  return rho;
}

// ----------------------------------------------------------- scene data ---
struct RMesh {
  const float4* tris;      // leaf order, as the traversal holds them
  const float4* nrm;       // per corner (leaf order) or null
  const uint8_t* sidx;     // per leaf-order triangle or null
  const uint32_t* shaders; // PolyMesh.Shader
  uint32_t n_shaders;
  uint32_t pad;
};
struct RLight {
  float p[9];
  int samples;
  uint32_t shader;
  uint32_t geom;
};

struct Ctx {
  V3 P, N, Ng, Poffset, DdPdu, DdPdv, Rd;
  float lambda, time;
  uint64_t I, scr0, scr1;
  int32_t geom;
};

__device__ RGB emission(const vmr_shader_std& s) {
  if (!(s.flags & VMR_SH_EMISSION_STRENGTH)) return RGB{{0, 0, 0}};
  RGB e = (s.flags & VMR_SH_EMISSION_COLOUR) ? RGB{{s.emission_colour[0], s.emission_colour[1], s.emission_colour[2]}}
                                            : RGB{{0, 0, 0}};
  for (float& c : e.c) c *= s.emission_strength;
  return e;
}
__device__ __forceinline__ float next_up(float v) {
  if (isinf(v) && v > 0) return v;
  if (v == 0.0f) v = 0.0f;
  unsigned u = __float_as_uint(v);
  u = v >= 0.0f ? u + 1 : u - 1;
  return __uint_as_float(u);
}
__device__ __forceinline__ float next_down(float v) {
  if (isinf(v) && v < 0) return v;
  if (v == 0.0f) v = 0.0f;
  unsigned u = __float_as_uint(v);
  u = v >= 0.0f ? u - 1 : u + 1;
  return __uint_as_float(u);
}
__device__ V3 offset_p(const Ctx& sc, int dir) {  // OffsetP (core/shader.go:139-163)
  const V3 pofs = dir < 0 ? v3(-sc.Poffset.x, -sc.Poffset.y, -sc.Poffset.z) : sc.Poffset;
  V3 po = add(sc.P, pofs);
  float* p = &po.x;
  const float* o = &pofs.x;
  for (int i = 0; i < 3; ++i) {
    if (o[i] > 0) p[i] = next_up(p[i]);
    else if (o[i] < -0.0f) p[i] = next_down(p[i]);
  }
  return po;
}

__device__ __forceinline__ V3 lp(const RLight& L, int k) { return v3(L.p[3 * k], L.p[3 * k + 1], L.p[3 * k + 2]); }
__device__ __forceinline__ float tri_area(V3 p0, V3 p1, V3 p2) { return 0.5f * length(cross(sub(p1, p0), sub(p2, p0))); }
__device__ void sides_to_angles(float as, float bs, float cs, float& a, float& b, float& c) {
  const float ssu = (as + bs + cs) / 2;
  const float sa = gsin(ssu - as), sb = gsin(ssu - bs), sc2 = gsin(ssu - cs), s = gsin(ssu);
  a = 2 * gatan(sqrtf(sb * sc2 / (s * sa)));
  b = 2 * gatan(sqrtf(sa * sc2 / (s * sb)));
  c = 2 * gatan(sqrtf(sa * sb / (s * sc2)));
}
// sampleSphericalTriangle (triangle.go:474-535)
__device__ V3 sample_spherical(V3 p0, V3 p1, V3 p2, V3 p, double r0, double r1, double& pdf) {
  const V3 pa = normalize(sub(p0, p)), pb = normalize(sub(p1, p)), pc = normalize(sub(p2, p));
  const float a = gacos(dot(pb, pc)), b = gacos(dot(pc, pa)), c = gacos(dot(pa, pb));
  float alpha, beta, gamma;
  sides_to_angles(a, b, c, alpha, beta, gamma);
  const float area = alpha + beta + gamma - kPi;
  const float areaHat = (float)r0 * area;
  const float s = gsin(areaHat - alpha), t = gcos(areaHat - alpha);
  const float sinA = gsin(alpha), cosA = gcos(alpha);
  const float u = t - cosA;
  const float v = s + sinA * gcos(c);
  float q = ((v * t - u * s) * cosA - v) / ((v * s + u * t) * sinA);
  q = gmax(-1.0f, gmin(q, 1.0f));
  float w = dot(pc, pa);
  const V3 v31 = normalize(v3(pc.x - w * pa.x, pc.y - w * pa.y, pc.z - w * pa.z));
  const float sq = sqrtf(1 - q * q);
  const V3 v4 = v3(q * pa.x + sq * v31.x, q * pa.y + sq * v31.y, q * pa.z + sq * v31.z);
  const float z = 1 - (float)r1 * (1 - dot(v4, pb));
  w = dot(v4, pb);
  const V3 v42 = normalize(v3(v4.x - w * pb.x, v4.y - w * pb.y, v4.z - w * pb.z));
  pdf = 1 / (double)area;
  return add(scale(z, pb), scale(sqrtf(1 - z * z), v42));
}
__device__ bool ray_plane(V3 Ro, V3 Rd, V3 P, V3 N, float& t) {
  const float denom = dot(N, Rd);
  if (fabsf(denom) > 1e-6f) {
    t = dot(sub(P, Ro), N) / denom;
    return t >= 0;
  }
  t = 0;
  return false;
}
__device__ bool ray_tri(V3 Ro, V3 Rd, V3 P0, V3 P1, V3 P2, V3& out) {  // Moller-Trumbore
  const V3 e1 = sub(P1, P0), e2 = sub(P2, P0);
  const V3 P = cross(Rd, e2);
  const float det = dot(e1, P);
  if (det > -1e-6f && det < 1e-6f) return false;
  const float inv = 1 / det;
  const V3 T = sub(Ro, P0);
  const float u = dot(T, P) * inv;
  if (u < 0 || u > 1) return false;
  const V3 Q = cross(T, e1);
  const float v = dot(Rd, Q) * inv;
  if (v < 0 || u + v > 1) return false;
  const float t = dot(e2, Q) * inv;
  if (t > 1e-6f) {
    out = add(add(scale(1 - u - v, P0), scale(u, P1)), scale(v, P2));
    return true;
  }
  return false;
}

// A light-sample candidate: direction, distance, pdf, spectrum.
struct Cand {
  V3 Ld;
  float Ldist;
  float pdf_own;    // light samples: ls.Pdf; BSDF samples: unused
  double pdf_bsdf;  // BSDF samples: bs.Pdf
  float pdf_light;  // BSDF samples: bs.PdfLight
  bool ok;
};

// Tri.SampleArea, sample i of n (triangle.go:232-343).
__device__ Cand light_sample(const RLight& L, const Ctx& sc, int n, int i) {
  Cand c{};
  const V3 p0 = lp(L, 0), p1 = lp(L, 1), p2 = lp(L, 2);
  const V3 N = normalize(cross(sub(p1, p0), sub(p2, p0)));
  const bool area_only = dot(sc.Ng, sub(p0, sc.P)) < 0 || dot(sc.Ng, sub(p1, sc.P)) < 0 || dot(sc.Ng, sub(p2, sc.P)) < 0;
  const uint64_t idx = sc.I * (uint64_t)n + (uint64_t)i;
  const double r0 = vdc(idx, sc.scr0), r1 = sobol(idx, sc.scr1);
  if (area_only) {
    const double pdf = (double)(1 / tri_area(p0, p1, p2));
    const float a = (float)(r1 * sqrt(1 - r0)), b = (float)(1 - sqrt(1 - r0));
    const V3 P = add(add(p0, scale(a, sub(p1, p0))), scale(b, sub(p2, p0)));
    const V3 D = sub(P, sc.P);
    c.Ldist = length(D);
    c.Ld = normalize(D);
    if (dot(c.Ld, N) > 0 || dot(c.Ld, sc.Ng) < 0) return c;
    c.pdf_own = (float)pdf * sqr(c.Ldist) / fabsf(dot(c.Ld, N));
  } else {
    double pdf;
    const V3 x = sample_spherical(p0, p1, p2, sc.P, r0, r1, pdf);
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

// BSDF sample i then Tri.ValidSample (core/shader.go:211-228, triangle.go:136-230).
__device__ Cand bsdf_candidate(const RLight& L, const Ctx& sc, const Bsdf& bsdf, int half, int i) {
  Cand c{};
  const uint64_t idx = sc.I * (uint64_t)half + (uint64_t)i;
  const double r0 = vdc(idx, sc.scr0), r1 = sobol(idx, sc.scr1);
  const V3 D = normalize(bsdf_sample(bsdf, r0, r1));
  c.pdf_bsdf = bsdf_pdf(bsdf, D);
  if (c.pdf_bsdf <= 0) return c;
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
    const float a = gacos(dot(pb, pc)), b = gacos(dot(pc, pa)), cc = gacos(dot(pa, pb));
    float al, be, ga;
    sides_to_angles(a, b, cc, al, be, ga);
    const float area = al + be + ga - kPi;
    c.pdf_light = (float)(1 / (double)area);
  }
  c.ok = true;
  return c;
}

// --------------------------------------------------------------- layout ---
constexpr int kMaxHalf = 8;  // NumSamples up to 16 per light (TriLight.Samples <= 4)

// Per sample s of a batch: slots[s][lobe][light][k] hold a contribution (rgb)
// that counts when its shadow ray is unoccluded.  k < half: light samples;
// half <= k < 2*half: BSDF samples (the order EvaluateLightSamples adds
// them).  lscale[s][lobe][light] = 1/float32(total), -1 when the light takes
// one sample (no MIS, no scale), 0 when nothing was taken.
struct RenderBatch {
  uint32_t width, height, npix;
  uint32_t iter0;  // first core.Render loop iteration of the batch
  uint32_t n;      // samples in the batch
  uint32_t nl;     // lights
  uint32_t ns;     // slots per (lobe, light)
  uint32_t pad;
  uint64_t seed;
  vmr_camera cam;
  const vmr_shader_std* shaders;
  const RLight* lights;
  const RMesh* meshes;
  float *px, *py, *pz, *dx, *dy, *dz, *tmax, *time;
  float* lambda;
  int32_t *hprim, *hgeom;
  float *ht, *hu, *hv, *hw;
  int32_t* shader;    // per sample: shader id of the hit, -1 none
  float* emis;        // per sample rgb
  float* slot_rgb;    // [n][2][nl][ns][3]
  uint8_t* slot_live; // [n][2][nl][ns]
  float* lscale;      // [n][2][nl]
  float *sx, *sy, *sz, *sdx, *sdy, *sdz, *stmax, *stime;
  uint32_t* sback;    // queue entry -> slot index
  int32_t* shit;      // any-hit prim per queue entry
  unsigned long long* queue_len;
  uint32_t queue_cap;
  int* status;
  float* fb;          // framebuffer (device), w*h*3
};

__global__ void k_generate(RenderBatch b) {
  const uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (s >= b.n) return;
  const uint32_t pix = (uint32_t)(s % b.npix);
  const uint32_t j = b.iter0 + (uint32_t)(s / b.npix) + 1;  // render(iter+1)
  const uint32_t x = pix % b.width, y = pix / b.width;
  double rx, ry;
  raster_xy(j, x, y, rx, ry);
  const double time = vdc(j, scramble(b.seed, pix, 2));
  const double lambda = (720.0 - 450.0) * vdc(j, scramble(b.seed, pix, 3)) + 450.0;
  const float Sx = (float)(-1.0 + 2.0 * (rx / (double)b.width));
  const float Sy = -(float)(-1.0 + 2.0 * (ry / (double)b.height));
  const vmr_camera& c = b.cam;
  const float camu = Sx * c.tan_theta_focal;
  const float camv = Sy * (c.tan_theta_focal / c.aspect);
  const V3 s3 = sub(add(scale(camu, v3(1, 0, 0)), scale(camv, v3(0, 1, 0))), scale(c.focal, v3(0, 0, 1)));
  const float* M = c.m;
  const V3 d = v3(M[0] * s3.x + M[4] * s3.y + M[8] * s3.z, M[1] * s3.x + M[5] * s3.y + M[9] * s3.z,
                  M[2] * s3.x + M[6] * s3.y + M[10] * s3.z);
  const V3 D = normalize(d);
  const V3 P = v3(M[0] * 0.0f + M[4] * 0.0f + M[8] * 0.0f + M[12], M[1] * 0.0f + M[5] * 0.0f + M[9] * 0.0f + M[13],
                  M[2] * 0.0f + M[6] * 0.0f + M[10] * 0.0f + M[14]);
  b.px[s] = P.x; b.py[s] = P.y; b.pz[s] = P.z;
  b.dx[s] = D.x; b.dy[s] = D.y; b.dz[s] = D.z;
  b.tmax[s] = __int_as_float(0x7f800000);
  b.time[s] = (float)time;
  b.lambda[s] = (float)lambda;
}

// Queues one shadow ray (one atomic per warp for the lanes that want one).
__device__ void emit_shadow(const RenderBatch& b, const Ctx& sc, V3 Ld, float Ldist, uint32_t slot, bool want) {
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
    b.slot_live[slot] = 0;
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
__device__ float light_lobe(const RenderBatch& b, const Ctx& sc, const RLight& L, const Bsdf& bsdf, int NS,
                            uint32_t slot0) {
  const int half = NS > 1 ? NS / 2 : 0;
  const int nls = NS > 1 ? half : NS;
  Cand cl[kMaxHalf], cb[kMaxHalf];
  int n_light = 0, n_bsdf = 0;
  for (int i = 0; i < nls; ++i) {
    cl[i] = light_sample(L, sc, nls, i);
    n_light += cl[i].ok ? 1 : 0;
  }
  for (int i = 0; i < half; ++i) {
    cb[i] = bsdf_candidate(L, sc, bsdf, half, i);
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
      float* out = b.slot_rgb + (size_t)slot * 3;
      out[0] = out[1] = out[2] = 0.0f;
      if (want) {
        Spec rho = bsdf_eval(bsdf, c.Ld);
        for (int k = 0; k < 4; ++k) rho.c[k] *= Liu.c[k];
        float inv;
        if (mis) {
          float p_hat;
          if (pass == 0) {
            p_hat = (float)nB * (float)bsdf_pdf(bsdf, c.Ld) / (float)total;
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
      b.slot_live[slot] = want ? 1 : 0;
      emit_shadow(b, sc, c.Ld, c.Ldist, slot, want);
    }
  }
  if (!mis) return -1.0f;
  return total == 0 ? 0.0f : 1.0f / (float)total;
}

// Hit attributes (builtin/geom/polymesh/trace.go:276-515, static meshes) and
// ShaderStd.Eval's direct lighting (builtin/shader/std.go:77-296).
__global__ void __launch_bounds__(128) k_shade(RenderBatch b) {
  const uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (s >= b.n) return;
  const int32_t prim = b.hprim[s];
  float* em = b.emis + s * 3;
  em[0] = em[1] = em[2] = 0.0f;
  const size_t nslot = (size_t)2 * b.nl * b.ns;
  for (size_t k = 0; k < nslot; ++k) b.slot_live[s * nslot + k] = 0;
  for (size_t k = 0; k < (size_t)2 * b.nl; ++k) b.lscale[s * 2 * b.nl + k] = 0.0f;
  b.shader[s] = -1;
  if (prim < 0) return;
  const int32_t geom = b.hgeom[s];
  const RMesh& m = b.meshes[geom];
  const float U = b.hu[s], V = b.hv[s], W = b.hw[s];
  const float4 a0 = m.tris[3 * (size_t)prim], a1 = m.tris[3 * (size_t)prim + 1], a2 = m.tris[3 * (size_t)prim + 2];
  const V3 V0 = v3(a0.x, a0.y, a0.z), V1 = v3(a1.x, a1.y, a1.z), V2 = v3(a2.x, a2.y, a2.z);
  const uint32_t sidx = m.sidx ? m.sidx[prim] : 0u;
  if (sidx >= m.n_shaders) return;  // no shader: core.Trace returns false (trace.go:281-283)
  const uint32_t shid = m.shaders[sidx];
  const vmr_shader_std& sh = b.shaders[shid];
  Ctx sc;
  const float xs = fabsf(U * V0.x) + fabsf(V * V1.x) + fabsf(W * V2.x);
  const float ys = fabsf(U * V0.y) + fabsf(V * V1.y) + fabsf(W * V2.y);
  const float zs = fabsf(U * V0.z) + fabsf(V * V1.z) + fabsf(W * V2.z);
  const V3 e0 = sub(V1, V0), e1 = sub(V2, V0);
  const V3 Ng = normalize(v3(e0.y * e1.z - e0.z * e1.y, e0.z * e1.x - e0.x * e1.z, e0.x * e1.y - e0.y * e1.x));
  V3 N = Ng;
  if (m.nrm) {
    const float4 n0 = m.nrm[3 * (size_t)prim], n1 = m.nrm[3 * (size_t)prim + 1], n2 = m.nrm[3 * (size_t)prim + 2];
    N = normalize(v3(U * n0.x + V * n1.x + W * n2.x, U * n0.y + V * n1.y + W * n2.y, U * n0.z + V * n1.z + W * n2.z));
  }
  const float g7 = (7.0f * 5.96046448e-08f) / (1 - 7.0f * 5.96046448e-08f);  // Gamma(7) (math/ferror.go:22-24)
  const float d = g7 * xs * fabsf(Ng.x) + g7 * ys * fabsf(Ng.y) + g7 * zs * fabsf(Ng.z);
  sc.Poffset = scale(d, Ng);
  sc.P = v3(U * V0.x + V * V1.x + W * V2.x, U * V0.y + V * V1.y + W * V2.y, U * V0.z + V * V1.z + W * V2.z);
  V3 axisu = sub(v3(1, 0, 0), scale(dot(v3(1, 0, 0), Ng), Ng));
  if (len2(axisu) < 0.1f || fabsf(dot(axisu, Ng)) > 0.3f) axisu = sub(v3(0, 0, 1), scale(dot(v3(0, 0, 1), Ng), Ng));
  const V3 dpdu = normalize(axisu);
  const V3 dpdv = cross(Ng, dpdu);
  // ApplyTransform with the identity transform renormalises (core/shader.go:129-135)
  sc.N = normalize(N);
  sc.Ng = normalize(Ng);
  sc.DdPdu = normalize(dpdu);
  sc.DdPdv = normalize(dpdv);
  sc.Rd = v3(b.dx[s], b.dy[s], b.dz[s]);
  sc.lambda = b.lambda[s];
  sc.time = b.time[s];
  const uint32_t pix = (uint32_t)(s % b.npix);
  sc.I = b.iter0 + (uint64_t)(s / b.npix) + 1;
  sc.scr0 = scramble(b.seed, pix, 4);
  sc.scr1 = scramble(b.seed, pix, 5);
  sc.geom = geom;
  b.shader[s] = (int32_t)shid;
  const RGB e = emission(sh);
  em[0] = e.c[0];
  em[1] = e.c[1];
  em[2] = e.c[2];
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
    return;
  }
  dw /= total;
  sw /= total;
  if (dw > 0.0f) {
    const float rough = (sh.flags & VMR_SH_DIFFUSE_ROUGHNESS) ? sh.diffuse_roughness : 0.5f;
    const Bsdf diff{0, sc.lambda, project(Ut, Vt, sc.N, wi), rough * rough, Fresnel{0, 0, {}, {}}, Ut, Vt, sc.N};
    for (uint32_t l = 0; l < b.nl; ++l) {
      const RLight& L = b.lights[l];
      if ((int32_t)L.geom == geom) continue;  // LightsPrepare (scene.go:100-116)
      const int NS = 1 << L.samples;
      const uint32_t slot0 = (uint32_t)((s * 2 + 0) * b.nl + l) * b.ns;
      b.lscale[(s * 2 + 0) * b.nl + l] = light_lobe(b, sc, L, diff, NS, slot0);
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
        const int NS = 1 << L.samples;
        const uint32_t slot0 = (uint32_t)((s * 2 + 1) * b.nl + l) * b.ns;
        b.lscale[(s * 2 + 1) * b.nl + l] = light_lobe(b, sc, L, spec, NS, slot0);
      }
    }
  }
}

// Occluded shadow rays switch their slot off.
__global__ void k_resolve(RenderBatch b, uint32_t nq) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq && b.shit[q] >= 0) b.slot_live[b.sback[q]] = 0;
}

// Per pixel, the batch's iterations in order: the sample colour assembled
// as ShaderStd.Eval adds its parts, then buf = (buf*iter + c)/(iter+1).
__global__ void k_accumulate(RenderBatch b, uint32_t iters) {
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= b.npix) return;
  float f0 = b.fb[pix * 3], f1 = b.fb[pix * 3 + 1], f2 = b.fb[pix * 3 + 2];
  for (uint32_t it = 0; it < iters; ++it) {
    const uint64_t s = (uint64_t)it * b.npix + pix;
    const uint32_t j = b.iter0 + it + 1;
    RGB c{{0, 0, 0}};
    const int32_t shid = b.shader[s];
    if (shid >= 0) {
      const vmr_shader_std& sh = b.shaders[shid];
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
          const float sc = b.lscale[(s * 2 + lb) * b.nl + l];
          if (sc == 0.0f) continue;
          RGB col{{0, 0, 0}};
          const uint32_t slot0 = (uint32_t)((s * 2 + lb) * b.nl + l) * b.ns;
          for (uint32_t k = 0; k < b.ns; ++k) {
            if (!b.slot_live[slot0 + k]) continue;
            const float* v = b.slot_rgb + (size_t)(slot0 + k) * 3;
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
      for (int k = 0; k < 3; ++k) c.c[k] = ((0.0f + b.emis[s * 3 + k]) + lobe[0].c[k]) + lobe[1].c[k];
    }
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

extern "C" {

int vmr_set_shaders(vmr_ctx* ctx, const vmr_shader_std* shaders, uint32_t n) {
  if (!ctx || (n && !shaders)) return VMR_ERR_INVALID;
  ctx->render.shaders.assign(shaders, shaders + n);
  return VMR_OK;
}

int vmr_mesh_set_shading(vmr_ctx* ctx, uint32_t geom, const uint32_t* shaders, uint32_t n_shaders, const float* normals) {
  if (!ctx || geom >= ctx->meshes.size() || (n_shaders && !shaders)) return VMR_ERR_INVALID;
  MeshRec& rec = *ctx->meshes[geom];
  if (rec.host.motion()) return rfail(ctx, VMR_ERR_UNSUPPORTED, "rendering motion meshes is not supported yet");
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
  RCUDA(rec.shlist.ensure(std::max<size_t>(1, n_shaders) * 4));
  if (n_shaders) RCUDA(cudaMemcpy(rec.shlist.p, shaders, n_shaders * 4, cudaMemcpyHostToDevice));
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

int vmr_set_camera(vmr_ctx* ctx, const vmr_camera* cam) {
  if (!ctx || !cam) return VMR_ERR_INVALID;
  if (cam->radius > 0.0f) return rfail(ctx, VMR_ERR_UNSUPPORTED, "thin-lens cameras are not supported yet");
  ctx->render.camera = *cam;
  ctx->render.has_camera = true;
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
  auto& R = ctx->render;
  for (const auto& sh : R.shaders)
    if ((sh.flags & VMR_SH_SPEC1_STRENGTH) && sh.spec1_strength > 0.0f && (sh.flags & VMR_SH_SPEC1_ROUGHNESS) &&
        sh.spec1_roughness == 0.0f)
      return rfail(ctx, VMR_ERR_UNSUPPORTED, "mirror (Spec1Roughness 0) shaders are not supported yet");
  for (const auto& L : R.lights)
    if (L.shader >= R.shaders.size() || L.geom >= ctx->meshes.size())
      return rfail(ctx, VMR_ERR_INVALID, "light shader or geom out of range");
  for (uint32_t g : ctx->top.host.geom_order) {
    const auto& mr = ctx->meshes[g];
    if (mr->host.motion()) return rfail(ctx, VMR_ERR_UNSUPPORTED, "rendering motion meshes is not supported yet");
    for (uint32_t sid : mr->shader_list)
      if (sid >= R.shaders.size()) return rfail(ctx, VMR_ERR_INVALID, "mesh shader id out of range");
  }
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  // Scene tables.
  std::vector<RMesh> rm(ctx->meshes.size());
  for (size_t g = 0; g < ctx->meshes.size(); ++g) {
    MeshRec& mr = *ctx->meshes[g];
    rm[g].tris = reinterpret_cast<const float4*>(mr.tris.p);
    rm[g].nrm = mr.has_normals ? reinterpret_cast<const float4*>(mr.nrm.p) : nullptr;
    rm[g].sidx = mr.host.shader_idx.empty() ? nullptr : mr.sidx.as<uint8_t>();
    rm[g].shaders = mr.shader_list.empty() ? nullptr : mr.shlist.as<uint32_t>();
    rm[g].n_shaders = (uint32_t)mr.shader_list.size();
  }
  std::vector<RLight> rl(R.lights.size());
  uint32_t ns = 1;
  for (size_t i = 0; i < R.lights.size(); ++i) {
    std::memcpy(rl[i].p, R.lights[i].p0, 12);
    std::memcpy(rl[i].p + 3, R.lights[i].p1, 12);
    std::memcpy(rl[i].p + 6, R.lights[i].p2, 12);
    rl[i].samples = R.lights[i].samples;
    rl[i].shader = R.lights[i].shader;
    rl[i].geom = R.lights[i].geom;
    ns = std::max<uint32_t>(ns, 1u << R.lights[i].samples);
  }
  const uint32_t nl = (uint32_t)R.lights.size();
  const uint32_t npix = p->width * p->height;
  uint32_t per_batch = p->max_batch_samples ? p->max_batch_samples : (4u << 20);
  uint32_t iters_per_batch = std::max<uint32_t>(1, per_batch / npix);
  if (iters_per_batch > p->iter_count) iters_per_batch = std::max<uint32_t>(1, p->iter_count);
  const uint64_t nmax = (uint64_t)iters_per_batch * npix;
  const uint64_t nslots = nmax * 2 * nl * ns;
  // Device buffers (one block, carved).
  const size_t fsz = 4;
  size_t bytes = 0;
  auto carve = [&](size_t nbytes) { size_t o = bytes; bytes += (nbytes + 255) / 256 * 256; return o; };
  const size_t o_ray = carve(nmax * 9 * fsz), o_hit = carve(nmax * 6 * fsz), o_sh = carve(nmax * 4),
               o_em = carve(nmax * 3 * fsz), o_srgb = carve(nslots * 3 * fsz), o_live = carve(nslots),
               o_lsc = carve(nmax * 2 * nl * fsz), o_q = carve(std::max<uint64_t>(1, nslots) * 8 * fsz),
               o_back = carve(std::max<uint64_t>(1, nslots) * 4), o_shit = carve(std::max<uint64_t>(1, nslots) * 4),
               o_cnt = carve(64), o_fb = carve((size_t)npix * 3 * fsz), o_meshes = carve(rm.size() * sizeof(RMesh)),
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
  b.nl = nl;
  b.ns = ns;
  b.seed = p->seed;
  b.cam = R.camera;
  b.shaders = reinterpret_cast<const vmr_shader_std*>(base + o_shaders);
  b.lights = reinterpret_cast<const RLight*>(base + o_lights);
  b.meshes = reinterpret_cast<const RMesh*>(base + o_meshes);
  float* ray = reinterpret_cast<float*>(base + o_ray);
  b.px = ray; b.py = ray + nmax; b.pz = ray + 2 * nmax; b.dx = ray + 3 * nmax; b.dy = ray + 4 * nmax;
  b.dz = ray + 5 * nmax; b.tmax = ray + 6 * nmax; b.time = ray + 7 * nmax; b.lambda = ray + 8 * nmax;
  char* hit = base + o_hit;
  b.hprim = reinterpret_cast<int32_t*>(hit);
  b.hgeom = reinterpret_cast<int32_t*>(hit) + nmax;
  b.ht = reinterpret_cast<float*>(hit) + 2 * nmax;
  b.hu = reinterpret_cast<float*>(hit) + 3 * nmax;
  b.hv = reinterpret_cast<float*>(hit) + 4 * nmax;
  b.hw = reinterpret_cast<float*>(hit) + 5 * nmax;
  b.shader = reinterpret_cast<int32_t*>(base + o_sh);
  b.emis = reinterpret_cast<float*>(base + o_em);
  b.slot_rgb = reinterpret_cast<float*>(base + o_srgb);
  b.slot_live = reinterpret_cast<uint8_t*>(base + o_live);
  b.lscale = reinterpret_cast<float*>(base + o_lsc);
  const uint64_t qcap = std::max<uint64_t>(1, nslots);
  float* q = reinterpret_cast<float*>(base + o_q);
  b.sx = q; b.sy = q + qcap; b.sz = q + 2 * qcap; b.sdx = q + 3 * qcap; b.sdy = q + 4 * qcap;
  b.sdz = q + 5 * qcap; b.stmax = q + 6 * qcap; b.stime = q + 7 * qcap;
  b.sback = reinterpret_cast<uint32_t*>(base + o_back);
  b.shit = reinterpret_cast<int32_t*>(base + o_shit);
  b.queue_len = reinterpret_cast<unsigned long long*>(base + o_cnt);
  b.status = reinterpret_cast<int*>(base + o_cnt + 8);
  b.queue_cap = (uint32_t)std::min<uint64_t>(qcap, 0xffffffffu);
  b.fb = reinterpret_cast<float*>(base + o_fb);
  RCUDA(cudaMemsetAsync(b.status, 0, 4, st));
  RCUDA(cudaEventRecord(ctx->ev0, st));
  uint64_t n_shadow = 0, n_cam = 0;
  for (uint32_t it0 = 0; it0 < p->iter_count; it0 += iters_per_batch) {
    const uint32_t iters = std::min(iters_per_batch, p->iter_count - it0);
    b.iter0 = p->iter_begin + it0;
    b.n = iters * npix;
    const int blk = 128;
    const int grid = (int)((b.n + blk - 1) / blk);
    k_generate<<<grid, blk, 0, st>>>(b);
    RCUDA(cudaGetLastError());
    vmr_rays rr{b.px, b.py, b.pz, b.dx, b.dy, b.dz, b.tmax, b.time};
    vmr_hits hh{b.hprim, b.hgeom, b.ht, b.hu, b.hv, b.hw};
    int rc = vmr_trace_scene(ctx, &rr, b.n, VMR_TRACE_DEVICE, &hh, nullptr);
    if (rc != VMR_OK) return rc;
    RCUDA(cudaMemsetAsync(b.queue_len, 0, 8, st));
    k_shade<<<grid, blk, 0, st>>>(b);
    RCUDA(cudaGetLastError());
    unsigned long long nq = 0;
    RCUDA(cudaMemcpyAsync(&nq, b.queue_len, 8, cudaMemcpyDeviceToHost, st));
    RCUDA(cudaStreamSynchronize(st));
    if (nq > b.queue_cap) return rfail(ctx, VMR_ERR_QUEUE_OVERFLOW, "shadow-ray queue overflow");
    if (nq) {
      vmr_rays sr{b.sx, b.sy, b.sz, b.sdx, b.sdy, b.sdz, b.stmax, b.stime};
      vmr_hits sh{b.shit, nullptr, nullptr, nullptr, nullptr, nullptr};
      rc = vmr_trace_scene(ctx, &sr, nq, VMR_TRACE_DEVICE | VMR_TRACE_ANY_HIT, &sh, nullptr);
      if (rc != VMR_OK) return rc;
      k_resolve<<<(int)((nq + 255) / 256), 256, 0, st>>>(b, (uint32_t)nq);
      RCUDA(cudaGetLastError());
    }
    k_accumulate<<<(int)((npix + 127) / 128), 128, 0, st>>>(b, iters);
    RCUDA(cudaGetLastError());
    n_shadow += nq;
    n_cam += b.n;
  }
  RCUDA(cudaEventRecord(ctx->ev1, st));
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
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    stats->ms = ms;
  }
  return VMR_OK;
}

}  // extern "C"
