// shade_common.cuh - device math shared by the render paths (render.cu,
// pathtrace.cu): float vectors with the reference's operation order, the
// ldseq QMC sequences, RasterXY, the hero-wavelength spectrum, Fresnel,
// the OrenNayar and GGX BSDFs, OffsetP, triangle-light geometry and the
// static-mesh hit attributes.  Everything is in an anonymous namespace, so
// each translation unit that includes it holds its own copy (including the
// RasterXY constant tables, which each unit uploads).
//
// Transcendentals are evaluated in float64 and rounded to float32, as
// math/sincos.go does; normalisation is a * (1/sqrt(a.a)) with IEEE sqrt and
// division (the reference's RSQRTSS estimate is machine-dependent).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "animdecomp.h"
#include "colour_tables.h"
#include "ctx.h"
#include "pixfilter.h"
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
// The same functions under the reference-mode precision switch: F32 false
// is the float64 evaluation above (the reference's math/sincos.go, bit for
// bit with the oracle); F32 true is CUDA's float32 functions (within 2 ulp),
// the VMR_RENDER_F32 option, which keeps the shading off the FP64 pipe.
template <bool F32> __device__ __forceinline__ float msin(float x) { return F32 ? sinf(x) : gsin(x); }
template <bool F32> __device__ __forceinline__ float mcos(float x) { return F32 ? cosf(x) : gcos(x); }
template <bool F32> __device__ __forceinline__ float mtan(float x) { return F32 ? tanf(x) : gtan(x); }
template <bool F32> __device__ __forceinline__ float matan(float x) { return F32 ? atanf(x) : gatan(x); }
template <bool F32> __device__ __forceinline__ float matan2(float y, float x) { return F32 ? atan2f(y, x) : gatan2(y, x); }
template <bool F32> __device__ __forceinline__ float macos(float x) {
  return F32 ? acosf(x > 1.0f ? 1.0f : (x < -1.0f ? -1.0f : x)) : gacos(x);
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
  int kind;  // 0 OrenNayar, 1 GGX, 2 Specular
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
// reflect(omegaR, (0,0,1)) (bsdf/specular.go:13-19): 2*dot(N, w)*N - w.
__device__ __forceinline__ V3 reflect_z(V3 w) {
  const float d = 0.0f * w.x + 0.0f * w.y + 1.0f * w.z;
  return sub(scale(2.0f * d, v3(0, 0, 1)), w);
}
template <bool F32 = false>
__device__ V3 bsdf_sample(const Bsdf& b, double r0, double r1) {
  if (b.kind == 2) return expand(b.U, b.V, b.N, normalize(reflect_z(b.wi)));  // Specular.Sample
  if (b.kind == 0) {  // CosineHemisphere (math/sample/sample.go:18-27)
    if (F32) {
      const float r = sqrtf(1.0f - (float)r0), th = 2.0f * kPi * (float)r1;
      return expand(b.U, b.V, b.N, v3(r * cosf(th), r * sinf(th), sqrtf((float)r0)));
    }
    const double r = sqrt(1 - r0), th = 2 * 3.14159265358979323846 * r1;
    return expand(b.U, b.V, b.N, v3((float)(r * cos(th)), (float)(r * sin(th)), (float)sqrt(r0)));
  }
  const float alpha = sqr(b.rough);  // MicrofacetGGX.Sample
  float thetaM, phiM;
  if (F32) {
    thetaM = atan2f(alpha * sqrtf((float)r0), sqrtf(1.0f - (float)r0));
    phiM = 2.0f * kPi * (float)r1;
  } else {
    thetaM = (float)atan2((double)alpha * sqrt(r0), sqrt(1 - r0));
    phiM = (float)(2.0 * 3.14159265358979323846 * r1);
  }
  const V3 m = v3(msin<F32>(thetaM) * mcos<F32>(phiM), msin<F32>(thetaM) * msin<F32>(phiM), mcos<F32>(thetaM));
  const V3 wo = sub(scale(2.0f * fabsf(dot(m, b.wi)), m), b.wi);
  return expand(b.U, b.V, b.N, normalize(wo));
}
template <bool F32 = false>
__device__ double bsdf_pdf(const Bsdf& b, V3 wo_world) {
  const V3 wo = project(b.U, b.V, b.N, wo_world);
  if (b.kind == 2) return dot(wo, reflect_z(b.wi)) < 0.9999f ? 0.0 : 1.0;  // Specular.PDF
  if (b.kind == 0) return (double)gmax(0.0f, wo.z) / 3.14159265358979323846;
  const float alpha = sqr(b.rough);
  const V3 m = scale(signf(b.wi.z), normalize(add(b.wi, wo)));
  const double pdf = (double)(ggx_d(m, alpha) * m.z);
  return isnan(pdf) ? 0.0 : pdf;
}
template <bool F32 = false>
__device__ Spec bsdf_eval(const Bsdf& b, V3 wo_world) {
  const V3 wo = project(b.U, b.V, b.N, wo_world);
  if (b.kind == 2) {  // Specular.Eval (bsdf/specular.go:77-101)
    Spec rho;
    for (int k = 0; k < 4; ++k) rho.c[k] = 0.0f;
    if (dot(wo, reflect_z(b.wi)) < 0.9999f) return rho;
    rho = from_rgb(fresnel_kr(b.fr, b.wi.z), b.lambda);
    const float s = fabsf(dot(wo, v3(0, 0, 1)));
    for (int k = 0; k < 4; ++k) rho.c[k] *= s;
    return rho;
  }
  if (b.kind == 0) {  // OrenNayar.Eval (bsdf/orennayar.go:42-73)
    const float sigma = b.rough;
    const float A = 1 - (0.5f * (sigma * sigma) / ((sigma * sigma) + 0.57f));
    const float B = 0.45f * (sigma * sigma) / ((sigma * sigma) + 0.09f);
    const float phiI = matan2<F32>(b.wi.y, b.wi.x), phiO = matan2<F32>(wo.y, wo.x);
    const float thetaI = macos<F32>(b.wi.z), thetaO = macos<F32>(wo.z);
    const float alpha = gmax(thetaI, thetaO), beta = gmin(thetaI, thetaO);
    const float C = msin<F32>(alpha) * mtan<F32>(beta);
    const float gamma = mcos<F32>(phiO - phiI);
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
  const uint32_t* shaders; // PolyMesh.Shader (a sphere: its shader first)
  uint32_t n_shaders;
  uint32_t kind;           // 0 triangles, 1 analytic sphere
  float sphere[4];         // centre, radius
  // motion meshes: vertices [keys][n_verts] and idxp in face order
  const float4* mverts;
  const uint32_t* midxp;
  uint32_t keys, n_verts;
  // motion meshes: per-key corner normals [keys][mnrm_n] (entry 3e + j is
  // corner j of element e), or null
  const float4* mnrm;
  uint32_t mnrm_n;
  // PolyMesh.Transform: the matrix and its Matrix4Inverse, column-major
  uint32_t has_xf;
  float xf[16], xf_inv[16];
  // PolyMesh.Transform of two or more keys (blended at the ray's time)
  const anim::Decomp* xf_keys;
  uint32_t xf_nkeys;
  // The GeomInstance or Proc through which this geom's hits are reached:
  // on a hit its transform becomes the shading context's
  // (instance.go:105-110, proc.go:133-138).  outer_nkeys 0: none; 1: the
  // matrix and inverse below; >= 2: blended from outer_keys at the ray's time.
  uint32_t outer_nkeys;
  const anim::Decomp* outer_keys;
  float outer_xf[16], outer_inv[16];
};
struct RLight {
  float p[9];        // TriLight: p0, p1, p2
  int samples;
  uint32_t shader;
  uint32_t geom;
  int kind;          // 0 TriLight, 1 DiskLight, 2 SphereLight
  float P[3], T[3], B[3], N[3], radius;  // DiskLight frame (Disk.PreRender); SphereLight centre, radius
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
template <bool F32 = false>
__device__ void sides_to_angles(float as, float bs, float cs, float& a, float& b, float& c) {
  const float ssu = (as + bs + cs) / 2;
  const float sa = msin<F32>(ssu - as), sb = msin<F32>(ssu - bs), sc2 = msin<F32>(ssu - cs), s = msin<F32>(ssu);
  a = 2 * matan<F32>(sqrtf(sb * sc2 / (s * sa)));
  b = 2 * matan<F32>(sqrtf(sa * sc2 / (s * sb)));
  c = 2 * matan<F32>(sqrtf(sa * sb / (s * sc2)));
}
// sampleSphericalTriangle (triangle.go:474-535)
template <bool F32 = false>
__device__ V3 sample_spherical(V3 p0, V3 p1, V3 p2, V3 p, double r0, double r1, double& pdf) {
  const V3 pa = normalize(sub(p0, p)), pb = normalize(sub(p1, p)), pc = normalize(sub(p2, p));
  const float a = macos<F32>(dot(pb, pc)), b = macos<F32>(dot(pc, pa)), c = macos<F32>(dot(pa, pb));
  float alpha, beta, gamma;
  sides_to_angles<F32>(a, b, c, alpha, beta, gamma);
  const float area = alpha + beta + gamma - kPi;
  const float areaHat = (float)r0 * area;
  const float s = msin<F32>(areaHat - alpha), t = mcos<F32>(areaHat - alpha);
  const float sinA = msin<F32>(alpha), cosA = mcos<F32>(alpha);
  const float u = t - cosA;
  const float v = s + sinA * mcos<F32>(c);
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


// Hit attributes of a static mesh (builtin/geom/polymesh/trace.go:276-515)
// followed by ApplyTransform with the identity (core/shader.go:129-135):
// P, Ng, N (interpolated normals when the mesh has them), Poffset (Gamma(7)
// error bound), dPdu/dPdv.  Returns false when the face has no shader.
__device__ __forceinline__ bool hit_attributes(const RMesh& m, int32_t prim, float U, float V, float W, Ctx& sc,
                                               uint32_t& shader_id) {
  const float4 a0 = m.tris[3 * (size_t)prim], a1 = m.tris[3 * (size_t)prim + 1], a2 = m.tris[3 * (size_t)prim + 2];
  const V3 V0 = v3(a0.x, a0.y, a0.z), V1 = v3(a1.x, a1.y, a1.z), V2 = v3(a2.x, a2.y, a2.z);
  const uint32_t sidx = m.sidx ? m.sidx[prim] : 0u;
  if (sidx >= m.n_shaders) return false;  // no shader: core.Trace returns false (trace.go:281-283)
  shader_id = m.shaders[sidx];
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
  sc.N = normalize(N);
  sc.Ng = normalize(Ng);
  sc.DdPdu = normalize(dpdu);
  sc.DdPdv = normalize(dpdv);
  return true;
}

// sample.UniformDisk2D (math/sample/sample.go:105-129), concentric warp.
__device__ __forceinline__ void uniform_disk(float radius, float r0, float r1, float& xo, float& yo) {
  const float x = -1 + 2 * r0, y = -1 + 2 * r1;
  float r = 0, theta = 0;
  const float q = kPi / 4;
  if (x > -y && x > y) {
    r = x;
    theta = q * y / x;
  } else if (x > -y && x < y) {
    r = y;
    theta = q * (2 - x / y);
  } else if (x < y && x < -y) {
    r = -x;
    theta = q * (4 + y / x);
  } else if (x > y && x < -y) {
    r = -y;
    theta = q * (6 - x / y);
  }
  xo = radius * r * gcos(theta);
  yo = radius * r * gsin(theta);
}

// The camera matrix of a sample with camera motion keys
// (Camera.ComputeRay, camera.go:223-236): the keys around the sample's time
// blended and rebuilt.  Not inlined: once per camera ray.
__device__ __noinline__ void camera_keyed(const anim::Decomp* keys, uint32_t n, float time, float* M) {
  if (!anim::at_time(keys, n, time, true, M))
    for (int i = 0; i < 16; ++i) M[i] = 0.0f;
}

// core.Render's per-sample setup (core/render.go:89-120) and a pinhole
// Camera.ComputeRay (builtin/camera/camera.go:244-284) for iteration j
// (render(iter+1)) of pixel pix: RasterXY position, VdC time and hero
// wavelength with the pixel's scrambles, the ray through the camera matrix:
// c.m (the host rebuilt it from its decomposition, as the reference does
// for one key) or, with two or more keys (ckeys, cnk), the keys blended at
// the sample's time.  KEYS false: the caller has no camera keys, and the
// blend (whose registers a kernel that calls it must hold) is left out.
template <bool KEYS = true>
__device__ __forceinline__ void camera_primary(const vmr_camera& c, const anim::Decomp* ckeys, uint32_t cnk,
                                               uint32_t width, uint32_t height, uint32_t j, uint32_t pix,
                                               uint64_t seed, const PixFilter& filt, V3& P, V3& D, float& time,
                                               float& lambda) {
  const uint32_t x = pix % width, y = pix / width;
  double rx, ry;
  raster_xy(j, x, y, rx, ry);
  if (filt.n > 0) {  // filter importance sampling (core/render.go:99-107)
    const double fx = floor(rx), fy = floor(ry);
    double u, v;
    warp_sample(filt, rx - fx, ry - fy, u, v);
    rx = fx + 0.5 + u;
    ry = fy + 0.5 + v;
  }
  time = (float)vdc(j, scramble(seed, pix, 2));
  lambda = (float)((720.0 - 450.0) * vdc(j, scramble(seed, pix, 3)) + 450.0);
  const float Sx = (float)(-1.0 + 2.0 * (rx / (double)width));
  const float Sy = -(float)(-1.0 + 2.0 * (ry / (double)height));
  const float camu = Sx * c.tan_theta_focal;
  const float camv = Sy * (c.tan_theta_focal / c.aspect);
  const V3 s3 = sub(add(scale(camu, v3(1, 0, 0)), scale(camv, v3(0, 1, 0))), scale(c.focal, v3(0, 0, 1)));
  float Mk[16];
  const float* M = c.m;
  if (KEYS && cnk >= 2) {
    camera_keyed(ckeys, cnk, time, Mk);
    M = Mk;
  }
  V3 e = v3(0, 0, 0), sv = s3;
  if (c.radius > 0.0f) {  // thin lens: UniformDisk2D at (lensU, lensV)
    const double lensU = vdc(j, scramble(seed, pix, 0)), lensV = sobol(j, scramble(seed, pix, 1));
    float x, y;
    uniform_disk(c.radius, (float)lensU, (float)lensV, x, y);
    e = add(scale(x, v3(1, 0, 0)), scale(y, v3(0, 1, 0)));
    sv = sub(s3, e);
  }
  const V3 d = v3(M[0] * sv.x + M[4] * sv.y + M[8] * sv.z, M[1] * sv.x + M[5] * sv.y + M[9] * sv.z,
                  M[2] * sv.x + M[6] * sv.y + M[10] * sv.z);
  D = normalize(d);
  P = v3(M[0] * e.x + M[4] * e.y + M[8] * e.z + M[12], M[1] * e.x + M[5] * e.y + M[9] * e.z + M[13],
         M[2] * e.x + M[6] * e.y + M[10] * e.z + M[14]);
}

// Hit attributes of an analytic sphere (builtin/geom/sphere/trace.go):
// P = ray.P + t*ray.D, N = Ng = normalize(P - centre), Poffset = 0.001*N,
// dPdu = (1,0,0), dPdv = (0,0,1), then ApplyTransform's renormalisation.
__device__ __forceinline__ bool sphere_attributes(const RMesh& m, V3 Ro, V3 Rd, float t, Ctx& sc,
                                                  uint32_t& shader_id) {
  if (m.n_shaders == 0) return false;
  shader_id = m.shaders[0];
  const V3 P = add(Ro, scale(t, Rd));
  const V3 N = normalize(sub(P, v3(m.sphere[0], m.sphere[1], m.sphere[2])));
  sc.Poffset = scale(0.001f, N);
  sc.P = P;
  sc.N = normalize(N);
  sc.Ng = normalize(N);
  sc.DdPdu = normalize(v3(1, 0, 0));
  sc.DdPdv = normalize(v3(0, 0, 1));
  return true;
}

// Hit attributes of a motion mesh (TraceMotionElems, trace.go:520-719): the
// face's vertices idxp[ElemID*3 + j] lerped between the keys around the ray
// time (Vec3Lerp, math/vec3.go:52-58), dPdu/dPdv the raw edges, then
// ApplyTransform's renormalisation; N from the per-key corner normals when
// the mesh has them (trace.go:694-712), else N = Ng.
__device__ __forceinline__ bool motion_attributes(const RMesh& m, int32_t elem, float U, float V, float W, float time,
                                                  Ctx& sc, uint32_t& shader_id) {
  const uint32_t sidx = m.sidx ? m.sidx[elem] : 0u;
  if (sidx >= m.n_shaders) return false;
  shader_id = m.shaders[sidx];
  const float k = time * (float)(m.keys - 1);
  const float tm = k - floorf(k);
  const uint32_t key = (uint32_t)floorf(k), key2 = (uint32_t)ceilf(k);
  V3 Vx[3];
  for (int j = 0; j < 3; ++j) {
    const uint32_t i = m.midxp[(size_t)elem * 3 + j];
    const float4 a = m.mverts[(size_t)key * m.n_verts + i], c = m.mverts[(size_t)key2 * m.n_verts + i];
    Vx[j] = v3((1.0f - tm) * a.x + tm * c.x, (1.0f - tm) * a.y + tm * c.y, (1.0f - tm) * a.z + tm * c.z);
  }
  const V3 V0 = Vx[0], V1 = Vx[1], V2 = Vx[2];
  const float xs = fabsf(U * V0.x) + fabsf(V * V1.x) + fabsf(W * V2.x);
  const float ys = fabsf(U * V0.y) + fabsf(V * V1.y) + fabsf(W * V2.y);
  const float zs = fabsf(U * V0.z) + fabsf(V * V1.z) + fabsf(W * V2.z);
  const V3 e0 = sub(V1, V0), e1 = sub(V2, V0);
  const V3 Ng = normalize(v3(e0.y * e1.z - e0.z * e1.y, e0.z * e1.x - e0.x * e1.z, e0.x * e1.y - e0.y * e1.x));
  const float g7 = (7.0f * 5.96046448e-08f) / (1 - 7.0f * 5.96046448e-08f);  // Gamma(7)
  const float d = g7 * xs * fabsf(Ng.x) + g7 * ys * fabsf(Ng.y) + g7 * zs * fabsf(Ng.z);
  sc.Poffset = scale(d, Ng);
  sc.P = v3(U * V0.x + V * V1.x + W * V2.x, U * V0.y + V * V1.y + W * V2.y, U * V0.z + V * V1.z + W * V2.z);
  V3 N = Ng;
  if (m.mnrm) {  // the element's corner normals of the two keys, lerped, then weighted by U, V, W
    V3 Nc[3];
    for (int j = 0; j < 3; ++j) {
      const size_t c = (size_t)elem * 3 + j;
      const float4 a = m.mnrm[(size_t)key * m.mnrm_n + c], b = m.mnrm[(size_t)key2 * m.mnrm_n + c];
      Nc[j] = v3((1.0f - tm) * a.x + tm * b.x, (1.0f - tm) * a.y + tm * b.y, (1.0f - tm) * a.z + tm * b.z);
    }
    N = normalize(v3(U * Nc[0].x + V * Nc[1].x + W * Nc[2].x, U * Nc[0].y + V * Nc[1].y + W * Nc[2].y,
                     U * Nc[0].z + V * Nc[1].z + W * Nc[2].z));
  }
  sc.N = normalize(N);
  sc.Ng = normalize(Ng);
  sc.DdPdu = normalize(e0);
  sc.DdPdv = normalize(e1);
  return true;
}

// Matrix4MulPoint / Matrix4MulVec (math/matrix4.go:177-218) of a
// column-major matrix, and Matrix4MulVec of its transpose.
__device__ __forceinline__ V3 xf_point(const float* a, V3 b) {
  return v3(a[0] * b.x + a[4] * b.y + a[8] * b.z + a[12], a[1] * b.x + a[5] * b.y + a[9] * b.z + a[13],
            a[2] * b.x + a[6] * b.y + a[10] * b.z + a[14]);
}
__device__ __forceinline__ V3 xf_vec(const float* a, V3 b) {
  return v3(a[0] * b.x + a[4] * b.y + a[8] * b.z, a[1] * b.x + a[5] * b.y + a[9] * b.z,
            a[2] * b.x + a[6] * b.y + a[10] * b.z);
}
__device__ __forceinline__ V3 xf_vec_t(const float* a, V3 b) {
  return v3(a[0] * b.x + a[1] * b.y + a[2] * b.z, a[4] * b.x + a[5] * b.y + a[6] * b.z,
            a[8] * b.x + a[9] * b.y + a[10] * b.z);
}

// A keyed transform at a time and its Matrix4Inverse (not inlined: it runs
// once per shaded hit on a keyed geom).
__device__ __noinline__ void keyed_matrix(const anim::Decomp* keys, uint32_t n, float time, float* M, float* I) {
  if (!anim::at_time(keys, n, time, false, M))
    for (int i = 0; i < 16; ++i) M[i] = 0.0f;
  anim::inverse(M, I);
}

// The five vectors of a shading context that a transform changes.
struct XfFrame {
  V3 P, N, Ng, DdPdu, DdPdv;
};
__device__ __forceinline__ XfFrame frame_of(const Ctx& sc) { return XfFrame{sc.P, sc.N, sc.Ng, sc.DdPdu, sc.DdPdv}; }
__device__ __forceinline__ void set_frame(Ctx& sc, const XfFrame& f) {
  sc.P = f.P;
  sc.N = f.N;
  sc.Ng = f.Ng;
  sc.DdPdu = f.DdPdu;
  sc.DdPdv = f.DdPdv;
}

// ShaderContext.ApplyTransform (core/shader.go:129-135): f.P still holds
// Po, the hit point in the space the geom was traced in.
__device__ __forceinline__ void apply_transform(XfFrame& f, const float* T, const float* I) {
  const V3 Po = f.P;
  f.P = xf_point(T, Po);
  f.N = normalize(xf_vec_t(I, f.N));
  f.Ng = normalize(xf_vec_t(I, f.Ng));
  f.DdPdu = normalize(xf_vec(T, f.DdPdu));
  f.DdPdv = normalize(xf_vec(T, f.DdPdv));
}

// The transforms of a mesh hit: a transformed mesh's PolyMesh.Trace sets
// N = M^-T N (builtin/geom/polymesh/trace.go:67-74; its P = M Po is replaced
// by ApplyTransform) and makes M the context's transform; a GeomInstance or
// Proc around the geom makes its own transform the context's instead
// (instance.go:105-110, proc.go:133-138); core.Trace then applies the
// context's transform.  Keyed transforms are taken at the ray's time.  Not
// inlined, like the keyed matrices: the matrices live in this frame only, so
// an untransformed hit, the common case, keeps its registers.
__device__ __noinline__ XfFrame mesh_transform(const RMesh& m, float time, XfFrame f) {
  float OT[16], OI[16], MT[16], MI[16];
  const float* ot = m.outer_xf;
  const float* oi = m.outer_inv;
  if (m.outer_nkeys >= 2) {
    keyed_matrix(m.outer_keys, m.outer_nkeys, time, OT, OI);
    ot = OT;
    oi = OI;
  }
  const float* mt = m.xf;
  const float* mi = m.xf_inv;
  const bool own = m.has_xf || m.xf_nkeys >= 2;
  if (m.xf_nkeys >= 2) {
    keyed_matrix(m.xf_keys, m.xf_nkeys, time, MT, MI);
    mt = MT;
    mi = MI;
  }
  if (own) f.N = xf_vec_t(mi, f.N);
  if (m.outer_nkeys) apply_transform(f, ot, oi);
  else if (own) apply_transform(f, mt, mi);
  return f;
}

// An analytic sphere inside a GeomInstance or Proc: the ray as its group
// mapped it (instance.go:91-93), the sphere's attributes, then the group's
// transform applied.  Not inlined, for the same reason.
struct GroupSphere {
  XfFrame f;
  V3 Poffset;
  uint32_t shader_id;
  bool ok;
};
__device__ __noinline__ GroupSphere grouped_sphere_attributes(const RMesh& m, V3 Ro, V3 Rd, float t, float time) {
  float OT[16], OI[16];
  const float* ot = m.outer_xf;
  const float* oi = m.outer_inv;
  if (m.outer_nkeys >= 2) {
    keyed_matrix(m.outer_keys, m.outer_nkeys, time, OT, OI);
    ot = OT;
    oi = OI;
  }
  Ro = xf_point(oi, Ro);
  Rd = xf_vec(oi, Rd);
  Ctx sc{};
  GroupSphere g{};
  g.ok = sphere_attributes(m, Ro, Rd, t, sc, g.shader_id);
  g.f = frame_of(sc);
  g.Poffset = sc.Poffset;
  if (g.ok) apply_transform(g.f, ot, oi);
  return g;
}

// A mesh's own one-matrix PolyMesh.Transform (the reference's steps as in
// mesh_transform, inlined for the kernels that take no groups or keys).
__device__ __forceinline__ XfFrame own_transform(const RMesh& m, XfFrame f) {
  f.N = xf_vec_t(m.xf_inv, f.N);
  apply_transform(f, m.xf, m.xf_inv);
  return f;
}

// The hit attributes of any geom kind, with the transforms above applied
// (P = T Po, N = normalize(T^-T N), Ng = normalize(T^-T Ng), dPdu/dPdv =
// normalize(T dPdu/dPdv), core/shader.go:129-135).  GROUPS false: the
// caller's scenes hold no GeomInstance, Proc or keyed transform (the
// extended path tracer refuses them on the host), so only a mesh's own
// one-matrix transform is applied and the keyed and group helpers, whose
// registers a kernel that calls them must hold, are left out.
template <bool GROUPS = true>
__device__ __forceinline__ bool surface_attributes(const RMesh& m, int32_t prim, float U, float V, float W, V3 Ro,
                                                   V3 Rd, float t, float time, Ctx& sc, uint32_t& shader_id) {
  if (m.kind == 1) {
    if (GROUPS && m.outer_nkeys) {
      const GroupSphere g = grouped_sphere_attributes(m, Ro, Rd, t, time);
      if (!g.ok) return false;
      set_frame(sc, g.f);
      sc.Poffset = g.Poffset;
      shader_id = g.shader_id;
      return true;
    }
    return sphere_attributes(m, Ro, Rd, t, sc, shader_id);
  }
  const bool ok = m.keys > 1 ? motion_attributes(m, prim, U, V, W, time, sc, shader_id)
                             : hit_attributes(m, prim, U, V, W, sc, shader_id);
  if (!ok) return false;
  if (GROUPS) {
    if (m.outer_nkeys || m.has_xf || m.xf_nkeys >= 2) set_frame(sc, mesh_transform(m, time, frame_of(sc)));
  } else if (m.has_xf) {
    set_frame(sc, own_transform(m, frame_of(sc)));
  }
  return true;
}

// The shading table indexed by geom id (host side).  A GeomInstance shades
// as the geom it instances, a Proc's child as itself; both with the group's
// transform as the outer one.  Group ids never reach a shading kernel
// otherwise (a Proc's hits report its children's ids).
inline void fill_rmesh_one(const MeshRec& mr, RMesh& r) {
  r = RMesh{};
  r.tris = reinterpret_cast<const float4*>(mr.tris.p);
  r.nrm = mr.has_normals ? reinterpret_cast<const float4*>(mr.nrm.p) : nullptr;
  r.sidx = mr.host.shader_idx.empty() ? nullptr : mr.sidx.as<uint8_t>();
  r.shaders = mr.shader_list.empty() ? nullptr : mr.shlist.as<uint32_t>();
  r.n_shaders = (uint32_t)mr.shader_list.size();
  r.kind = mr.host.sphere ? 1u : 0u;
  for (int k = 0; k < 3; ++k) r.sphere[k] = mr.host.sphere_c[k];
  r.sphere[3] = mr.host.sphere_r;
  r.keys = mr.host.motion() ? mr.host.keys : 1u;
  r.n_verts = mr.host.n_verts;
  r.mverts = mr.host.motion() ? mr.avert.as<float4>() : nullptr;
  r.midxp = mr.host.motion() ? mr.aidx.as<uint32_t>() : nullptr;
  r.mnrm = mr.host.motion() && mr.mnrm_n ? mr.mnrm.as<float4>() : nullptr;
  r.mnrm_n = r.mnrm ? mr.mnrm_n : 0u;
  r.has_xf = mr.has_xf ? 1u : 0u;
  std::memcpy(r.xf, mr.xf, sizeof(mr.xf));
  std::memcpy(r.xf_inv, mr.xf_inv, sizeof(mr.xf_inv));
  r.xf_nkeys = mr.xkeys.size() >= 2 ? (uint32_t)mr.xkeys.size() : 0u;
  r.xf_keys = r.xf_nkeys ? mr.dxkeys.as<const anim::Decomp>() : nullptr;
}
inline void set_outer(const MeshRec& g, RMesh& r) {
  r.outer_nkeys = (uint32_t)g.xkeys.size();
  r.outer_keys = g.xkeys.size() >= 2 ? g.dxkeys.as<const anim::Decomp>() : nullptr;
  std::memcpy(r.outer_xf, g.xf, sizeof(g.xf));
  std::memcpy(r.outer_inv, g.xf_inv, sizeof(g.xf_inv));
}
inline std::vector<RMesh> rmesh_table(const vmr_ctx* ctx) {
  std::vector<RMesh> rm(ctx->meshes.size());
  for (size_t g = 0; g < ctx->meshes.size(); ++g) {
    const MeshRec& mr = *ctx->meshes[g];
    if (mr.host.group == 1) {
      fill_rmesh_one(*ctx->meshes[mr.children[0]], rm[g]);
      set_outer(mr, rm[g]);
    } else {
      fill_rmesh_one(mr, rm[g]);
      if (mr.owner >= 0) set_outer(*ctx->meshes[mr.owner], rm[g]);
    }
  }
  return rm;
}
// The geom whose shading data a hit on geom g reads (the instanced geom for
// an instance), for the render's input checks.
inline const MeshRec& shading_rec(const vmr_ctx* ctx, uint32_t g) {
  const MeshRec& mr = *ctx->meshes[g];
  return mr.host.group == 1 ? *ctx->meshes[mr.children[0]] : mr;
}

}  // namespace

// RasterXY tables for m = 12 (render.cu).
void raster_tables_m12(uint64_t fwd[52], uint64_t inv[52]);

}  // namespace vmr
