// orc_render.cpp - CPU oracle of the reference render path (reference mode).
//
// TEST INFRASTRUCTURE ONLY (see orc.h).  Restates core.Render / render
// (core/render.go:66-218), Camera.ComputeRay for a pinhole
// (builtin/camera/camera.go:221-323), core.Trace (core/trace.go:40-83), the
// static hit attributes of PolyMesh.TraceElems (trace.go:276-515),
// ShaderStd.Eval (builtin/shader/std.go:77-316), EvaluateLightSamples
// (core/shader.go:203-402), the OrenNayar and GGX BSDFs, the Fresnel models,
// TriLight sampling (builtin/light/triangle.go) and the hero-wavelength
// spectrum (colour/*.go).
//
// Deliberate, documented departures from the Go code (the CUDA path does the
// same, so the two agree closely):
//  * Vec3Normalize is a * (1/sqrt(a.a)) with IEEE sqrt and division; the
//    reference's RSQRTSS estimate is machine-dependent (math/vec3_amd64.s).
//    orc_set_normalize_mode(1, seed) switches to an emulation of the
//    assembly (an estimate within RSQRTSS's documented relative error of
//    1.5*2^-12, then its Newton step in its operation order) so that the
//    size of this departure can be measured on whole images.
//  * acos arguments are clamped to [-1, 1]: a normalised dot product can
//    exceed 1 by an ulp, where the reference yields NaN.
//  * per-pixel scrambles come from a hash of (seed, pixel) instead of the
//    unseeded math/rand stream (core/render.go:166-176).
// The camera goes through the reference's SRT decomposition round trip
// (TransformDecompMatrix4 of each LocalToWorld key, then per sample
// TransformDecompToMatrix4 of TransformDecompLerp; camera.go:223-236).
// Transcendentals follow math/sincos.go: evaluated in float64, rounded to
// float32.
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "orc.h"
#include "orc_colour_tables.h"
#include "orc_internal.h"

namespace {

using orc_internal::Hit;

struct V3 {
  float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 scale(float s, V3 a) { return v3(a.x * s, a.y * s, a.z * s); }  // Vec3Scale
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {  // Vec3Cross (math/vec3.go:69-74)
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float len2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline float gabs(float x) { return std::fabs(x); }
// Vec3Normalize.  Mode 0: a * (1/sqrt(a.a)).  Mode 1 emulates
// math/vec3_amd64.s:11-42: s = (x*x + y*y) + z*z; g = RSQRTSS(s), here the
// exact 1/sqrt(s) times (1 + e) with e a hash of (s, seed) uniform in
// [-1.5*2^-12, 1.5*2^-12] (the instruction's documented error bound);
// g' = (1.5 - (g*g)*(0.5*s)) * g; result a * g'.
int g_norm_mode = 0;
uint64_t g_norm_seed = 0;
inline float rsqrtss_estimate(float s) {
  uint32_t bits;
  std::memcpy(&bits, &s, 4);
  uint64_t z = g_norm_seed + 0x9E3779B97F4A7C15ull * ((uint64_t)bits + 1ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
  const double e = (2.0 * u - 1.0) * 1.5 / 4096.0;
  return (float)((1.0 / std::sqrt((double)s)) * (1.0 + e));
}
inline V3 normalize(V3 a) {
  if (g_norm_mode == 1) {
    const float s = (a.x * a.x + a.y * a.y) + a.z * a.z;
    const float g = rsqrtss_estimate(s);
    const float h = 0.5f * s;
    const float g2 = (1.5f - (g * g) * h) * g;
    return v3(a.x * g2, a.y * g2, a.z * g2);
  }
  const float r = 1.0f / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return v3(a.x * r, a.y * r, a.z * r);
}
inline float length(V3 a) { return std::sqrt((a.x * a.x + a.y * a.y) + a.z * a.z); }  // Vec3Length
inline float gmax(float x, float y) { return x > y ? x : y; }
inline float gmin(float x, float y) { return x < y ? x : y; }
const float kPi = 3.14159265358f;  // math.Pi (math/const.go:8) as float32
// math/sincos.go: float64 evaluation, float32 result.
inline float gsin(float x) { return (float)std::sin((double)x); }
inline float gcos(float x) { return (float)std::cos((double)x); }
inline float gtan(float x) { return (float)std::tan((double)x); }
inline float gatan(float x) { return (float)std::atan((double)x); }
inline float gatan2(float y, float x) { return (float)std::atan2((double)y, (double)x); }
inline float gacos(float x) { return (float)std::acos((double)(x > 1.0f ? 1.0f : (x < -1.0f ? -1.0f : x))); }
// Vec3BasisProject / Vec3BasisExpand (math/vec3.go:122-137).
inline V3 project(V3 U, V3 V, V3 W, V3 s) { return v3(dot(U, s), dot(V, s), dot(W, s)); }
inline V3 expand(V3 U, V3 V, V3 W, V3 s) {
  return v3(U.x * s.x + V.x * s.y + W.x * s.z, U.y * s.x + V.y * s.y + W.y * s.z, U.z * s.x + V.z * s.y + W.z * s.z);
}

// ---------------------------------------------------------------- QMC ----
uint64_t vdc_bits(uint64_t i, uint64_t s) {  // ldseq.vanDerCorput
  uint64_t b = (i << 32) | (i >> 32);
  b = ((b & 0x0000ffff0000ffffull) << 16) | ((b & 0xffff0000ffff0000ull) >> 16);
  b = ((b & 0x00ff00ff00ff00ffull) << 8) | ((b & 0xff00ff00ff00ff00ull) >> 8);
  b = ((b & 0x0f0f0f0f0f0f0f0full) << 4) | ((b & 0xf0f0f0f0f0f0f0f0ull) >> 4);
  b = ((b & 0x3333333333333333ull) << 2) | ((b & 0xccccccccccccccccull) >> 2);
  b = ((b & 0x5555555555555555ull) << 1) | ((b & 0xaaaaaaaaaaaaaaaaull) >> 1);
  return (s ^ b) >> 12;
}
uint64_t sobol_bits(uint64_t i, uint64_t s) {  // ldseq.sobol
  uint64_t r = s >> 12;
  for (uint64_t v = 1ull << 51; i != 0; i >>= 1) {
    if (i & 1) r ^= v;
    v ^= v >> 1;
  }
  return r;
}
const double kTwo52 = 4503599627370496.0;
inline double vdc(uint64_t i, uint64_t s) { return (double)vdc_bits(i, s) / kTwo52; }
inline double sobol(uint64_t i, uint64_t s) { return (double)sobol_bits(i, s) / kTwo52; }

// ----------------------------------------------------------- spectrum ----
struct RGB {
  float c[3];
};
struct Spectrum {
  float c[4];
  float lambda;
};
// Spectrum.Wavelength (colour/spectrum.go:102-112).
float wavelength(float lambda, int j) {
  float v = (lambda - 450.0f + ((float)j / 4.0f) * 300.0f);
  if (v >= 300.0f) v -= 300.0f;
  v += 450.0f;
  return v;
}
float smits_eval(const float* s, float lambda) {  // smitsSpectrum.eval
  if (lambda < 380.0f || lambda >= 720.0f) return 0.0f;
  int bin = (int)(((lambda - 380.0f) / (720.0f - 380.0f)) * 10.0f);
  return s[bin];
}
// RGBToSpectrumSmits99 (colour/spectrum_smits9.go:48-84).
float smits(float r, float g, float b, float l) {
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
Spectrum from_rgb(RGB rgb, float lambda) {  // Spectrum.FromRGB
  Spectrum s;
  s.lambda = lambda;
  for (int k = 0; k < 4; ++k) s.c[k] = smits(rgb.c[0], rgb.c[1], rgb.c[2], wavelength(lambda, k));
  return s;
}
float cie(const float* t, float l) {  // CieObserverData.X/Y/Z
  if (l < 360.0f || l >= 830.0f) return -1.0f;
  int bin = (int)(((l - 360.0f) / (830.0f - 360.0f)) * 95.0f);
  return t[bin];
}
RGB to_rgb(const Spectrum& s) {  // Spectrum.ToRGB + sRGB.XYZToRGB
  float x = 0, y = 0, z = 0;
  for (int i = 0; i < 4; ++i) {
    const float l = wavelength(s.lambda, i);
    x += s.c[i] * cie(kCieX, l);
    y += s.c[i] * cie(kCieY, l);
    z += s.c[i] * cie(kCieZ, l);
  }
  const float* m = kSrgbFromXyz;
  return RGB{{x * m[0] + y * m[1] + z * m[2], x * m[3] + y * m[4] + z * m[5], x * m[6] + y * m[7] + z * m[8]}};
}
inline void sscale(Spectrum& s, float f) {
  for (float& c : s.c) c *= f;
}
inline void smul(Spectrum& s, const Spectrum& o) {
  for (int k = 0; k < 4; ++k) s.c[k] *= o.c[k];
}
inline void radd(RGB& a, RGB b) {
  for (int k = 0; k < 3; ++k) a.c[k] += b.c[k];
}
inline void rmul(RGB& a, RGB b) {
  for (int k = 0; k < 3; ++k) a.c[k] *= b.c[k];
}
inline void rscale(RGB& a, float f) {
  for (float& c : a.c) c *= f;
}

// ------------------------------------------------------------ fresnel ----
struct Fresnel {
  int model;  // 0 dielectric, 1 conductor
  float eta;
  RGB r, g;
};
inline float sqr(float v) { return v * v; }
RGB fresnel_kr(const Fresnel& f, float c) {
  if (f.model == 0) {  // Dielectric.Kr (fresnel/dielectric.go:34-47)
    float g = (f.eta * f.eta) - 1 + (c * c);
    if (g < 0.0f) return RGB{{1, 1, 1}};
    g = std::sqrt(g);
    float fr = 0.5f * sqr((g - c) / (g + c)) * (1 + sqr((c * (g + c) - 1) / (c * (g - c) + 1)));
    return RGB{{fr, fr, fr}};
  }
  RGB out;  // Conductor.Kr (fresnel/conductor.go:58-89)
  for (int k = 0; k < 3; ++k) {
    const float r = gmax(0.0f, gmin(f.r.c[k], 0.99f));  // Clamp(r, 0, 0.99)
    const float g = f.g.c[k];
    const float nmin = (1 - r) / (1 + r);
    const float nmax = (1 + std::sqrt(r)) / (1 - std::sqrt(r));
    const float n = nmin * g + (1 - g) * nmax;
    const float k2 = ((n + 1) * (n + 1) * r - (n - 1) * (n - 1)) / (1 - r);
    const float rs = (n * n + k2 - 2 * n * c + c * c) / (n * n + k2 + 2 * n * c + c * c);
    const float rp = ((n * n + k2) * c * c - 2 * n * c + 1) / ((n * n + k2) * c * c + 2 * n * c + 1);
    out.c[k] = 0.5f * (rs + rp);
  }
  return out;
}

// --------------------------------------------------------------- BSDFs ----
struct Bsdf {
  int kind;  // 0 OrenNayar, 1 GGX, 2 specular
  float lambda;
  V3 wi;       // OmegaI / OmegaR in the local frame
  float rough; // roughness^2 as the constructors store it
  Fresnel fr;
  V3 U, V, N;
};
// sample.CosineHemisphere (math/sample/sample.go:18-27)
V3 cosine_hemisphere(double u0, double u1) {
  double r = std::sqrt(1 - u0);
  double th = 2 * M_PI * u1;
  return v3((float)(r * std::cos(th)), (float)(r * std::sin(th)), (float)std::sqrt(u0));
}
// sample.UniformDisk2D (math/sample/sample.go:105-129), concentric warp.
void uniform_disk(float radius, float r0, float r1, float& xo, float& yo) {
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
inline float chi(float x) { return x > 0.0f ? 1.0f : 0.0f; }
float ggx_g1(V3 w, V3 m, float alpha) {
  float odn = dot(w, m);
  float denom = 1 + std::sqrt(1 + (alpha * alpha) * ((1.0f / (w.z * w.z)) - 1));
  return chi(odn / w.z) * 2 / denom;
}
float ggx_d(V3 m, float alpha) {
  float numer = alpha * alpha * chi(m.z);
  if (m.z == 1.0f) return 1.0f / (kPi * alpha * alpha);
  float denom = kPi * sqr(m.z * m.z) * sqr(alpha * alpha + ((1.0f / (m.z * m.z)) - 1));
  return numer / denom;
}
inline float signf(float v) { return v < 0 ? -1.0f : 1.0f; }
inline V3 reflect_z(V3 w) {  // reflect(omegaR, (0,0,1)) (bsdf/specular.go:13-19)
  const float d = 0.0f * w.x + 0.0f * w.y + 1.0f * w.z;
  return sub(scale(2.0f * d, v3(0, 0, 1)), w);
}

V3 bsdf_sample(const Bsdf& b, double r0, double r1) {
  if (b.kind == 0) return expand(b.U, b.V, b.N, cosine_hemisphere(r0, r1));
  if (b.kind == 1) {  // MicrofacetGGX.Sample (bsdf/microfacetggx.go:82-100)
    const float alpha = sqr(b.rough);
    const double thetaM = std::atan2((double)alpha * std::sqrt(r0), std::sqrt(1 - r0));
    const double phiM = 2.0 * M_PI * r1;
    const V3 m = v3(gsin((float)thetaM) * gcos((float)phiM), gsin((float)thetaM) * gsin((float)phiM), gcos((float)thetaM));
    const V3 wo = sub(scale(2.0f * gabs(dot(m, b.wi)), m), b.wi);
    return expand(b.U, b.V, b.N, normalize(wo));
  }
  return expand(b.U, b.V, b.N, normalize(reflect_z(b.wi)));  // Specular.Sample
}

double bsdf_pdf(const Bsdf& b, V3 wo_world) {
  const V3 wo = project(b.U, b.V, b.N, wo_world);
  if (b.kind == 0) return (double)gmax(0.0f, wo.z) / M_PI;
  if (b.kind == 1) {
    const float alpha = sqr(b.rough);
    const V3 m = scale(signf(b.wi.z), normalize(add(b.wi, wo)));
    const double pdf = (double)(ggx_d(m, alpha) * m.z);
    return std::isnan(pdf) ? 0.0 : pdf;
  }
  return dot(wo, reflect_z(b.wi)) < 0.9999f ? 0.0 : 1.0;
}

Spectrum bsdf_eval(const Bsdf& b, V3 wo_world) {
  Spectrum rho;
  rho.lambda = b.lambda;
  for (float& c : rho.c) c = 0.0f;
  const V3 wo = project(b.U, b.V, b.N, wo_world);
  if (b.kind == 0) {  // OrenNayar.Eval (bsdf/orennayar.go:42-73)
    const float sigma = b.rough;
    const float A = 1 - (0.5f * (sigma * sigma) / ((sigma * sigma) + 0.57f));
    const float B = 0.45f * (sigma * sigma) / ((sigma * sigma) + 0.09f);
    const float phiI = gatan2(b.wi.y, b.wi.x);
    const float phiO = gatan2(wo.y, wo.x);
    const float thetaI = gacos(b.wi.z);
    const float thetaO = gacos(wo.z);
    const float alpha = gmax(thetaI, thetaO);
    const float beta = gmin(thetaI, thetaO);
    const float C = gsin(alpha) * gtan(beta);
    const float gamma = gcos(phiO - phiI);
    const float s = wo.z * (A + (B * gmax(0.0f, gamma) * C));
    rho = from_rgb(RGB{{1, 1, 1}}, b.lambda);
    sscale(rho, s / kPi);
    return rho;
  }
  if (b.kind == 1) {  // MicrofacetGGX.Eval (microfacetggx.go:119-145)
    const float alpha = sqr(b.rough);
    const V3 h = scale(signf(b.wi.z), normalize(add(b.wi, wo)));
    const RGB f = fresnel_kr(b.fr, gabs(dot(b.wi, h)));
    const float numer = ggx_g1(b.wi, h, alpha) * ggx_g1(wo, h, alpha) * ggx_d(h, alpha);
    const float denom = 4 * gabs(b.wi.z) * gabs(wo.z);
    rho = from_rgb(f, b.lambda);
    sscale(rho, gabs(wo.z) * numer / denom);
    for (float& c : rho.c)
      if (c < 0 || std::isnan(c)) c = 0;
    return rho;
  }
  if (dot(wo, reflect_z(b.wi)) < 0.9999f) return rho;  // Specular.Eval
  rho = from_rgb(fresnel_kr(b.fr, b.wi.z), b.lambda);
  sscale(rho, gabs(dot(wo, v3(0, 0, 1))));
  return rho;
}

// -------------------------------------------------------------- scene ----
struct Shader {
  orc_shader p;
  bool has(uint32_t f) const { return (p.flags & f) != 0; }
};

struct Ctx {  // the ShaderContext fields the path reads
  V3 P, N, Ng, Poffset, DdPdu, DdPdv, Rd;
  float lambda, time;
  int level;
  uint64_t I;
  uint64_t scr0, scr1;
  int32_t geom;
  const Shader* shader;
};

struct LightSample {
  V3 Ld;
  float Ldist, pdf;
  Spectrum Liu;
};
struct BsdfSample {
  V3 D, Ld;
  double pdf;
  float pdf_light, Ldist;
  Spectrum Liu;
};

// A light of the list: a TriLight (kind 0) or a DiskLight (kind 1, with its
// frame from Disk.PreRender, builtin/light/disk.go:79-104).
struct Light {
  int kind;
  orc_trilight tri;
  V3 P, T, B, N;
  float radius;
  int samples;
  uint32_t shader, mesh;
};

struct Render {
  const orc_scene* scene = nullptr;
  std::vector<orc_internal::MeshView> meshes;
  std::vector<std::vector<uint32_t>> mesh_shaders;
  std::vector<Shader> shaders;
  std::vector<orc_trilight> tri_lights;
  std::vector<Light> lights;
  orc_camera cam;
  std::vector<orc_internal::Decomp> cam_keys;  // LocalToWorld keys, decomposed
  orc_internal::FilterTable filter;
};

// EvalEmission (std.go:299-316).
RGB emission(const Shader& s) {
  if (!s.has(ORC_SH_EMISSION_STRENGTH)) return RGB{{0, 0, 0}};
  RGB e = s.has(ORC_SH_EMISSION_COLOUR) ? RGB{{s.p.emission_colour[0], s.p.emission_colour[1], s.p.emission_colour[2]}}
                                        : RGB{{0, 0, 0}};
  rscale(e, s.p.emission_strength);
  return e;
}

// OffsetP (core/shader.go:139-163).
float next_up(float v) {
  if (std::isinf(v) && v > 0) return v;
  if (v == 0.0f) v = 0.0f;
  uint32_t u;
  std::memcpy(&u, &v, 4);
  if (v >= 0.0f) ++u; else --u;
  std::memcpy(&v, &u, 4);
  return v;
}
float next_down(float v) {
  if (std::isinf(v) && v < 0) return v;
  if (v == 0.0f) v = 0.0f;
  uint32_t u;
  std::memcpy(&u, &v, 4);
  if (v >= 0.0f) --u; else ++u;
  std::memcpy(&v, &u, 4);
  return v;
}
V3 offset_p(const Ctx& sc, int dir) {
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

// Triangle-light helpers (builtin/light/triangle.go).
V3 tri_normal(const orc_trilight& L) {
  const V3 p0 = v3(L.p0[0], L.p0[1], L.p0[2]), p1 = v3(L.p1[0], L.p1[1], L.p1[2]), p2 = v3(L.p2[0], L.p2[1], L.p2[2]);
  return normalize(cross(sub(p1, p0), sub(p2, p0)));
}
float tri_area(V3 p0, V3 p1, V3 p2) { return 0.5f * length(cross(sub(p1, p0), sub(p2, p0))); }
void sides_to_angles(float as, float bs, float cs, float& a, float& b, float& c) {
  const float ssu = (as + bs + cs) / 2;
  const float sa = gsin(ssu - as), sb = gsin(ssu - bs), sc2 = gsin(ssu - cs), s = gsin(ssu);
  a = 2 * gatan(std::sqrt(sb * sc2 / (s * sa)));
  b = 2 * gatan(std::sqrt(sa * sc2 / (s * sb)));
  c = 2 * gatan(std::sqrt(sa * sb / (s * sc2)));
}
float spherical_area(V3 pa, V3 pb, V3 pc, float& a_side_c) {
  const float a = gacos(dot(pb, pc)), b = gacos(dot(pc, pa)), c = gacos(dot(pa, pb));
  float al, be, ga;
  sides_to_angles(a, b, c, al, be, ga);
  a_side_c = c;
  return al + be + ga - kPi;
}
// sampleSphericalTriangle (triangle.go:474-535), Arvo's method.
V3 sample_spherical(V3 p0, V3 p1, V3 p2, V3 p, double r0, double r1, double& pdf) {
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
  V3 v31 = normalize(v3(pc.x - w * pa.x, pc.y - w * pa.y, pc.z - w * pa.z));
  const float sq = std::sqrt(1 - q * q);
  const V3 v4 = v3(q * pa.x + sq * v31.x, q * pa.y + sq * v31.y, q * pa.z + sq * v31.z);
  const float z = 1 - (float)r1 * (1 - dot(v4, pb));
  w = dot(v4, pb);
  const V3 v42 = normalize(v3(v4.x - w * pb.x, v4.y - w * pb.y, v4.z - w * pb.z));
  pdf = 1 / (double)area;
  return add(scale(z, pb), scale(std::sqrt(1 - z * z), v42));
}
// rayPlaneIntersect (builtin/light/disk.go:38-51)
bool ray_plane(V3 Ro, V3 Rd, V3 P, V3 N, float& t) {
  const float denom = dot(N, Rd);
  if (gabs(denom) > 1e-6f) {
    t = dot(sub(P, Ro), N) / denom;
    return t >= 0;
  }
  t = 0;
  return false;
}
// rayTriangleIntersect, Moller-Trumbore (triangle.go:79-129)
bool ray_tri(V3 Ro, V3 Rd, V3 P0, V3 P1, V3 P2, V3& out) {
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

struct Renderer {
  const Render& R;

  Spectrum light_liu(const Light& L, const Ctx& sc) const {
    return from_rgb(emission(R.shaders[L.shader]), sc.lambda);
  }

  // Tri.SampleArea (triangle.go:285-343) with the area fallback (:232-282).
  // Disk.SampleArea (builtin/light/disk.go:154-204).
  void sample_area_disk(const Light& L, const Ctx& sc, int n, std::vector<LightSample>& out) const {
    for (int i = 0; i < n; ++i) {
      const uint64_t idx = sc.I * (uint64_t)n + (uint64_t)i;
      const double r0 = vdc(idx, sc.scr0), r1 = sobol(idx, sc.scr1);
      const float u = L.radius * std::sqrt((float)r0) * gcos(2 * kPi * (float)r1);
      const float v = L.radius * std::sqrt((float)r0) * gsin(2 * kPi * (float)r1);
      const double pdf = (double)(1.0f / (kPi * L.radius * L.radius));
      const V3 P = add(add(L.P, scale(u, L.B)), scale(v, L.T));  // Vec3Add3
      const V3 V = sub(P, sc.P);
      if (dot(V, sc.Ng) > 0.0f && dot(V, L.N) < 0.0f) {
        LightSample ls;
        ls.Ldist = length(V);
        ls.Ld = normalize(V);
        ls.Liu = light_liu(L, sc);
        ls.pdf = (float)pdf * (ls.Ldist * ls.Ldist) / gabs(dot(ls.Ld, L.N));
        out.push_back(ls);
      }
    }
  }

  // raySphereIntersect (builtin/light/sphere.go:96-124), the same as the geom's.
  static bool sphere_hit(V3 Ro, V3 Rd, V3 C, float radius, float& t) {
    const float ro[3] = {Ro.x, Ro.y, Ro.z}, rd[3] = {Rd.x, Rd.y, Rd.z}, c[3] = {C.x, C.y, C.z};
    const float L[3] = {ro[0] - c[0], ro[1] - c[1], ro[2] - c[2]};
    const float a = rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2];
    const float b = 2 * (rd[0] * L[0] + rd[1] * L[1] + rd[2] * L[2]);
    const float cc = (L[0] * L[0] + L[1] * L[1] + L[2] * L[2]) - radius * radius;
    float x0, x1;
    const float discr = b * b - 4 * a * cc;
    if (discr < 0) return false;
    if (discr == 0) {
      x1 = -0.5f * b / a;
      x0 = x1;
    } else {
      const float q = b > 0 ? -0.5f * (b + std::sqrt(discr)) : -0.5f * (b - std::sqrt(discr));
      x0 = q / a;
      x1 = cc / q;
    }
    if (x0 > x1) std::swap(x0, x1);
    if (x0 > x1) std::swap(x0, x1);
    if (x0 < 0) {
      x0 = x1;
      if (x0 < 0) return false;
    }
    t = x0;
    return true;
  }

  // Sphere.SampleArea (builtin/light/sphere.go:178-254): a cone toward the
  // sphere, pdf q_2 of Shirley et al. 1996.
  void sample_area_sphere(const Light& L, const Ctx& sc, int n, std::vector<LightSample>& out) const {
    const V3 V = sub(L.P, sc.P);
    const float l = length(V);
    const V3 w = normalize(V);
    const V3 v = normalize(cross(w, sc.Ng));
    const V3 u = cross(w, v);
    for (int i = 0; i < n; ++i) {
      const uint64_t idx = sc.I * (uint64_t)n + (uint64_t)i;  // + sg.Sample, which is 0
      const double r0 = vdc(idx, sc.scr0), r1 = sobol(idx, sc.scr1);
      const float theta = gacos(1 - (float)r0 + (float)r0 * std::sqrt(1 - sqr(L.radius / l)));
      const float phi = 2 * kPi * (float)r1;
      const V3 a = v3(gcos(phi) * gsin(theta), gsin(phi) * gsin(theta), gcos(theta));
      const V3 omega = expand(u, v, w, a);
      if (dot(omega, sc.Ng) < 0) continue;
      float t;
      if (!sphere_hit(sc.P, omega, L.P, L.radius, t)) continue;
      const V3 x = add(sc.P, scale(t, omega));
      const V3 D = sub(x, sc.P);
      LightSample ls;
      ls.Ldist = length(D);
      ls.Ld = normalize(D);
      ls.Liu = light_liu(L, sc);
      ls.pdf = 1 / (2 * kPi * (1 - std::sqrt(1 - sqr(L.radius / l))));
      out.push_back(ls);
    }
  }

  void sample_area(const Light& LL, const Ctx& sc, int n, std::vector<LightSample>& out) const {
    if (LL.kind == 1) {
      sample_area_disk(LL, sc, n, out);
      return;
    }
    if (LL.kind == 2) {
      sample_area_sphere(LL, sc, n, out);
      return;
    }
    const orc_trilight& L = LL.tri;
    const V3 p0 = v3(L.p0[0], L.p0[1], L.p0[2]), p1 = v3(L.p1[0], L.p1[1], L.p1[2]), p2 = v3(L.p2[0], L.p2[1], L.p2[2]);
    const V3 N = tri_normal(L);
    const bool area_only = dot(sc.Ng, sub(p0, sc.P)) < 0 || dot(sc.Ng, sub(p1, sc.P)) < 0 || dot(sc.Ng, sub(p2, sc.P)) < 0;
    for (int i = 0; i < n; ++i) {
      const uint64_t idx = sc.I * (uint64_t)n + (uint64_t)i;
      const double r0 = vdc(idx, sc.scr0), r1 = sobol(idx, sc.scr1);
      LightSample ls;
      if (area_only) {
        const double pdf = (double)(1 / tri_area(p0, p1, p2));
        const float a = (float)(r1 * std::sqrt(1 - r0)), b = (float)(1 - std::sqrt(1 - r0));
        const V3 P = add(add(p0, scale(a, sub(p1, p0))), scale(b, sub(p2, p0)));
        const V3 D = sub(P, sc.P);
        ls.Ldist = length(D);
        ls.Ld = normalize(D);
        if (dot(ls.Ld, N) > 0 || dot(ls.Ld, sc.Ng) < 0) continue;
        ls.Liu = light_liu(LL, sc);
        ls.pdf = (float)pdf * sqr(ls.Ldist) / gabs(dot(ls.Ld, N));
      } else {
        double pdf;
        const V3 x = sample_spherical(p0, p1, p2, sc.P, r0, r1, pdf);
        float t;
        ray_plane(sc.P, x, p0, N, t);
        const V3 P = add(sc.P, scale(t, x));  // Vec3Mad
        const V3 D = sub(P, sc.P);
        ls.Ldist = length(D);
        ls.Ld = normalize(D);
        if (dot(ls.Ld, N) > 0 || dot(ls.Ld, sc.Ng) < 0) continue;
        ls.Liu = light_liu(LL, sc);
        ls.pdf = (float)pdf;
      }
      out.push_back(ls);
    }
  }

  // Disk.ValidSample (disk.go:119-151) with rayDiskIntersect (disk.go:53-68).
  bool valid_sample_disk(const Light& L, const Ctx& sc, BsdfSample& s) const {
    const double pdf = (double)(1.0f / (kPi * L.radius * L.radius));
    float t;
    if (!ray_plane(sc.P, s.D, L.P, L.N, t)) return false;
    const V3 pp = add(sc.P, scale(t, s.D));  // Vec3Mad(Ro, Rd, t)
    const V3 vv = sub(pp, L.P);
    if (!(std::sqrt(dot(vv, vv)) <= L.radius)) return false;
    const V3 p = add(sc.P, scale(t, s.D));
    const V3 V = sub(p, sc.P);
    if (dot(V, sc.Ng) <= 0.0f || dot(V, L.N) >= 0.0f) return false;
    s.Ldist = length(V);
    s.Ld = normalize(V);
    s.Liu = light_liu(L, sc);
    s.pdf_light = (float)pdf * (s.Ldist * s.Ldist) / gabs(dot(s.Ld, L.N));
    return true;
  }

  // Tri.ValidSample (triangle.go:136-230).
  // Sphere.ValidSample (builtin/light/sphere.go:126-176).
  bool valid_sample_sphere(const Light& L, const Ctx& sc, BsdfSample& s) const {
    float t;
    if (!sphere_hit(sc.P, s.D, L.P, L.radius, t)) return false;
    const V3 x = add(sc.P, scale(t, s.D));
    const V3 D = sub(x, sc.P);
    s.Ldist = length(D);
    s.Ld = normalize(D);
    s.Liu = light_liu(L, sc);
    const V3 V = sub(L.P, sc.P);
    const float l = length(V);
    s.pdf_light = 1 / (2 * kPi * (1 - std::sqrt(1 - sqr(L.radius / l))));
    return true;
  }

  bool valid_sample(const Light& LL, const Ctx& sc, BsdfSample& s) const {
    if (LL.kind == 1) return valid_sample_disk(LL, sc, s);
    if (LL.kind == 2) return valid_sample_sphere(LL, sc, s);
    const orc_trilight& L = LL.tri;
    const V3 p0 = v3(L.p0[0], L.p0[1], L.p0[2]), p1 = v3(L.p1[0], L.p1[1], L.p1[2]), p2 = v3(L.p2[0], L.p2[1], L.p2[2]);
    V3 P;
    if (!ray_tri(sc.P, s.D, p0, p1, p2, P)) return false;
    const V3 N = tri_normal(L);
    const bool area_only = dot(sc.Ng, sub(p0, P)) < 0 || dot(sc.Ng, sub(p1, P)) < 0 || dot(sc.Ng, sub(p2, P)) < 0;
    const V3 D = sub(P, sc.P);
    s.Ldist = length(D);
    s.Ld = normalize(D);
    if (dot(s.Ld, N) > 0 || dot(s.Ld, sc.Ng) < 0) return false;
    s.Liu = light_liu(LL, sc);
    if (area_only) {
      const double pdf = (double)(1 / tri_area(p0, p1, p2));
      s.pdf_light = (float)pdf * sqr(s.Ldist) / gabs(dot(s.Ld, N));
    } else {
      float cside;
      const float area = spherical_area(normalize(sub(p0, sc.P)), normalize(sub(p1, sc.P)), normalize(sub(p2, sc.P)), cside);
      s.pdf_light = (float)(1 / (double)area);
    }
    return true;
  }

  bool occluded(const Ctx& sc, V3 Ld, float Ldist) const {
    const V3 o = offset_p(sc, dot(Ld, sc.Ng) < 0 ? -1 : 1);
    const V3 d = scale(Ldist * 0.9999f, Ld);  // ShadowRayEpsilon (core/ray.go:22)
    const float P[3] = {o.x, o.y, o.z}, D[3] = {d.x, d.y, d.z};
    return orc_internal::trace(R.scene, P, D, 1.0f, sc.time, true).hit;
  }

  // EvaluateLightSamples (core/shader.go:203-402).
  RGB evaluate_light_samples(const Ctx& sc, const Light& L, int NS, const Bsdf& bsdf) const {
    RGB col{{0, 0, 0}};
    if (NS > 1) {
      std::vector<BsdfSample> bsdf_samples;
      for (int i = 0; i < NS / 2; ++i) {
        const uint64_t idx = sc.I * (uint64_t)(NS / 2) + (uint64_t)i;
        const double r0 = vdc(idx, sc.scr0), r1 = sobol(idx, sc.scr1);
        BsdfSample s;
        s.D = normalize(bsdf_sample(bsdf, r0, r1));
        s.pdf = bsdf_pdf(bsdf, s.D);
        if (s.pdf <= 0) continue;
        if (valid_sample(L, sc, s)) bsdf_samples.push_back(s);
      }
      std::vector<LightSample> ls;
      sample_area(L, sc, NS / 2, ls);
      int nB = NS / 2, nL = NS / 2;
      if (ls.empty()) nL = 0;
      if (bsdf_samples.empty()) nB = 0;
      const int total = nB + nL;
      if (total == 0) return col;
      for (const LightSample& l : ls) {
        if (dot(l.Ld, sc.N) <= 0) continue;
        if (occluded(sc, l.Ld, l.Ldist)) continue;
        Spectrum rho = bsdf_eval(bsdf, l.Ld);
        smul(rho, l.Liu);
        float p_hat = (float)nB * (float)bsdf_pdf(bsdf, l.Ld) / (float)total;
        p_hat += (float)nL * l.pdf / (float)total;
        sscale(rho, 1.0f / p_hat);
        RGB rgb = to_rgb(rho);
        for (float& c : rgb.c)
          if (c < 0) c = 0;
        radd(col, rgb);
      }
      for (const BsdfSample& b : bsdf_samples) {
        if (dot(b.Ld, sc.N) <= 0) continue;
        if (occluded(sc, b.Ld, b.Ldist)) continue;
        Spectrum rho = bsdf_eval(bsdf, b.Ld);
        smul(rho, b.Liu);
        float p_hat = (float)nB * (float)b.pdf / (float)total;
        p_hat += (float)nL * b.pdf_light / (float)total;
        sscale(rho, 1.0f / p_hat);
        RGB rgb = to_rgb(rho);
        for (float& c : rgb.c)
          if (c < 0) c = 0;
        radd(col, rgb);
      }
      rscale(col, 1.0f / (float)total);
      return col;
    }
    std::vector<LightSample> ls;
    sample_area(L, sc, NS, ls);
    for (const LightSample& l : ls) {
      if (dot(l.Ld, sc.N) <= 0) continue;
      if (occluded(sc, l.Ld, l.Ldist)) continue;
      Spectrum rho = bsdf_eval(bsdf, l.Ld);
      smul(rho, l.Liu);
      sscale(rho, 1.0f / l.pdf);
      radd(col, to_rgb(rho));
    }
    return col;
  }

  // Hit attributes for a static mesh (trace.go:276-515) or an analytic sphere
  // (sphere/trace.go), then the transforms: a transformed mesh's
  // PolyMesh.Trace sets P = M Po and N = M^-T N (trace.go:67-74) and makes M
  // the context's transform; a GeomInstance or Proc around the geom makes
  // its own transform the context's on a hit (instance.go:105-110,
  // proc.go:133-138); core.Trace then calls ShaderContext.ApplyTransform with
  // the context's transform (core/shader.go:129-135; the identity when none
  // was set).  Keyed transforms are taken at the ray's time.
  bool hit_context(const Hit& h, Ctx& sc, V3 Ro, V3 Rd) const {
    const orc_internal::MeshView& m = R.meshes[h.geom];
    float OT[16], OI[16];  // the instance's / Proc's transform and inverse
    if (m.outer) {
      orc_internal::decomp_at(*m.outer, sc.time, false, OT);
      orc_internal::matrix_inverse(OT, OI);
      // the ray its children were traced with (instance.go:91-93)
      const V3 P0 = Ro, D0 = Rd;
      Ro = v3(OI[0] * P0.x + OI[4] * P0.y + OI[8] * P0.z + OI[12], OI[1] * P0.x + OI[5] * P0.y + OI[9] * P0.z + OI[13],
              OI[2] * P0.x + OI[6] * P0.y + OI[10] * P0.z + OI[14]);
      Rd = v3(OI[0] * D0.x + OI[4] * D0.y + OI[8] * D0.z, OI[1] * D0.x + OI[5] * D0.y + OI[9] * D0.z,
              OI[2] * D0.x + OI[6] * D0.y + OI[10] * D0.z);
    }
    if (m.sphere) {
      const auto& list = R.mesh_shaders[h.geom];
      if (list.empty()) return false;
      sc.shader = &R.shaders[list[0]];
      const V3 P = add(Ro, scale(h.t, Rd));  // Vec3Mad(ray.P, ray.D, t)
      const V3 N = normalize(sub(P, v3(m.sc[0], m.sc[1], m.sc[2])));
      sc.Poffset = scale(0.001f, N);
      sc.P = P;
      sc.N = normalize(N);
      sc.Ng = normalize(N);
      sc.DdPdu = normalize(v3(1, 0, 0));
      sc.DdPdv = normalize(v3(0, 0, 1));
      sc.geom = h.geom;
      if (m.outer) apply_transform(sc, OT, OI);
      return true;
    }
    const uint32_t i0 = m.idxp[h.elem * 3 + 0], i1 = m.idxp[h.elem * 3 + 1], i2 = m.idxp[h.elem * 3 + 2];
    // static: key 0; motion: the keys around the ray's time, lerped as
    // TraceMotionElems does (trace.go:520-560, Vec3Lerp math/vec3.go:52-58)
    float tm = 0.0f;
    int key = 0, key2 = 0;
    if (m.motion) {
      const float k = sc.time * (float)(m.keys - 1);
      tm = k - std::floor(k);
      key = (int)std::floor(k);
      key2 = (int)std::ceil(k);
    }
    auto vert = [&](uint32_t i) {
      const float* a = m.verts + ((size_t)key * m.nverts + i) * 3;
      if (!m.motion) return v3(a[0], a[1], a[2]);
      const float* b = m.verts + ((size_t)key2 * m.nverts + i) * 3;
      return v3((1.0f - tm) * a[0] + tm * b[0], (1.0f - tm) * a[1] + tm * b[1], (1.0f - tm) * a[2] + tm * b[2]);
    };
    const V3 V0 = vert(i0), V1 = vert(i1), V2 = vert(i2);
    const float U = h.u, V = h.v, W = h.w;
    const float xs = gabs(U * V0.x) + gabs(V * V1.x) + gabs(W * V2.x);
    const float ys = gabs(U * V0.y) + gabs(V * V1.y) + gabs(W * V2.y);
    const float zs = gabs(U * V0.z) + gabs(V * V1.z) + gabs(W * V2.z);
    const uint8_t sidx = m.shaderidx ? m.shaderidx[h.elem] : 0;
    const auto& list = R.mesh_shaders[h.geom];
    if (sidx >= list.size()) return false;
    sc.shader = &R.shaders[list[sidx]];
    const V3 e0 = sub(V1, V0), e1 = sub(V2, V0);
    V3 Ng = normalize(v3(e0.y * e1.z - e0.z * e1.y, e0.z * e1.x - e0.x * e1.z, e0.x * e1.y - e0.y * e1.x));
    V3 N;
    if (m.motion ? m.mnormals != nullptr : m.normals != nullptr) {
      // static: per-vertex normals; motion: the element's corner normals of
      // the two keys lerped at the ray's time (trace.go:694-712), N = Ng
      // when the mesh has none with as many keys as its vertices
      auto nrm = [&](uint32_t i, uint32_t j) {
        if (!m.motion) return v3(m.normals[i * 3], m.normals[i * 3 + 1], m.normals[i * 3 + 2]);
        const size_t c = (size_t)h.elem * 3 + j;
        const float* a = m.mnormals + ((size_t)key * m.mnormals_per_key + c) * 3;
        const float* b = m.mnormals + ((size_t)key2 * m.mnormals_per_key + c) * 3;
        return v3((1.0f - tm) * a[0] + tm * b[0], (1.0f - tm) * a[1] + tm * b[1], (1.0f - tm) * a[2] + tm * b[2]);
      };
      const V3 N0 = nrm(i0, 0), N1 = nrm(i1, 1), N2 = nrm(i2, 2);
      N = normalize(v3(U * N0.x + V * N1.x + W * N2.x, U * N0.y + V * N1.y + W * N2.y, U * N0.z + V * N1.z + W * N2.z));
    } else {
      N = Ng;
    }
    const float g7 = (7.0f * 5.96046448e-08f) / (1 - 7.0f * 5.96046448e-08f);  // Gamma(7)
    const float d = g7 * xs * gabs(Ng.x) + g7 * ys * gabs(Ng.y) + g7 * zs * gabs(Ng.z);
    sc.Poffset = scale(d, Ng);
    sc.P = v3(U * V0.x + V * V1.x + W * V2.x, U * V0.y + V * V1.y + W * V2.y, U * V0.z + V * V1.z + W * V2.z);
    V3 dpdu, dpdv;
    if (m.motion) {  // the motion path keeps the raw edges (trace.go:655-661)
      dpdu = e0;
      dpdv = e1;
    } else {
      V3 axisu = sub(v3(1, 0, 0), scale(dot(v3(1, 0, 0), Ng), Ng));
      if (len2(axisu) < 0.1f || gabs(dot(axisu, Ng)) > 0.3f) axisu = sub(v3(0, 0, 1), scale(dot(v3(0, 0, 1), Ng), Ng));
      dpdu = normalize(axisu);
      dpdv = cross(Ng, dpdu);
    }
    sc.N = normalize(N);
    sc.Ng = normalize(Ng);
    sc.DdPdu = normalize(dpdu);
    sc.DdPdv = normalize(dpdv);
    sc.geom = h.geom;
    float MT[16], MI[16];  // the mesh's own transform and inverse
    const bool own = m.has_xf || m.xkeys;
    if (m.xkeys) {
      orc_internal::decomp_at(*m.xkeys, sc.time, false, MT);
      orc_internal::matrix_inverse(MT, MI);
    } else if (m.has_xf) {
      for (int i = 0; i < 16; ++i) {
        MT[i] = m.xf[i];
        MI[i] = m.xinv[i];
      }
    }
    if (own) sc.N = mul_inv_t(MI, sc.N);  // PolyMesh.Trace (its P is replaced below)
    if (m.outer) apply_transform(sc, OT, OI);
    else if (own) apply_transform(sc, MT, MI);
    return true;
  }

  // Matrix4MulPoint / Matrix4MulVec (math/matrix4.go:177-218, sums left to
  // right) and Matrix4MulVec of the inverse transposed (Matrix4Transpose,
  // :100-108).
  static V3 mul_point(const float* T, V3 b) {
    return v3(T[0] * b.x + T[4] * b.y + T[8] * b.z + T[12], T[1] * b.x + T[5] * b.y + T[9] * b.z + T[13],
              T[2] * b.x + T[6] * b.y + T[10] * b.z + T[14]);
  }
  static V3 mul_vec(const float* T, V3 b) {
    return v3(T[0] * b.x + T[4] * b.y + T[8] * b.z, T[1] * b.x + T[5] * b.y + T[9] * b.z,
              T[2] * b.x + T[6] * b.y + T[10] * b.z);
  }
  static V3 mul_inv_t(const float* I, V3 b) {
    float t[16];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) t[i * 4 + j] = I[j * 4 + i];
    return v3(t[0] * b.x + t[4] * b.y + t[8] * b.z, t[1] * b.x + t[5] * b.y + t[9] * b.z,
              t[2] * b.x + t[6] * b.y + t[10] * b.z);
  }
  // ShaderContext.ApplyTransform (core/shader.go:129-135); Po is the hit
  // point in the space the geom was traced in.
  static void apply_transform(Ctx& sc, const float* T, const float* I) {
    const V3 Po = sc.P;
    sc.P = mul_point(T, Po);
    sc.N = normalize(mul_inv_t(I, sc.N));
    sc.Ng = normalize(mul_inv_t(I, sc.Ng));
    sc.DdPdu = normalize(mul_vec(T, sc.DdPdu));
    sc.DdPdv = normalize(mul_vec(T, sc.DdPdv));
  }

  // core.Trace (core/trace.go:40-83).
  bool trace(V3 P, V3 D, int level, const Ctx& parent, RGB& out) const {
    const float Pa[3] = {P.x, P.y, P.z}, Da[3] = {D.x, D.y, D.z};
    const Hit h = orc_internal::trace(R.scene, Pa, Da, INFINITY, parent.time, false);
    if (!h.hit) return false;
    Ctx sc = parent;
    sc.level = level;
    sc.Rd = D;
    if (!hit_context(h, sc, P, D)) return false;
    out = shade(sc);
    return true;
  }

  // ShaderStd.Eval (builtin/shader/std.go:77-296).
  RGB shade(const Ctx& sg) const {
    RGB zero{{0, 0, 0}};
    if (sg.level > 3) return zero;
    const Shader& sh = *sg.shader;
    if (sh.has(ORC_SH_DEBUG))  // Debug.Eval (builtin/shader/debug.go:47-49)
      return RGB{{sh.p.diffuse_colour[0], sh.p.diffuse_colour[1], sh.p.diffuse_colour[2]}};
    V3 Vt = cross(sg.N, sg.DdPdu);
    if (len2(Vt) < 0.1f) Vt = cross(sg.N, sg.DdPdv);
    Vt = normalize(Vt);
    const V3 Ut = normalize(cross(sg.N, Vt));
    const float diff_rough = sh.has(ORC_SH_DIFFUSE_ROUGHNESS) ? sh.p.diffuse_roughness : 0.5f;
    const V3 wi = v3(-sg.Rd.x, -sg.Rd.y, -sg.Rd.z);
    Bsdf diff{0, sg.lambda, project(Ut, Vt, sg.N, wi), diff_rough * diff_rough, Fresnel{}, Ut, Vt, sg.N};
    RGB diff_col = sh.has(ORC_SH_DIFFUSE_COLOUR) ? RGB{{sh.p.diffuse_colour[0], sh.p.diffuse_colour[1], sh.p.diffuse_colour[2]}} : zero;
    float dw = sh.has(ORC_SH_DIFFUSE_STRENGTH) ? sh.p.diffuse_strength : 0.0f;
    float sw = sh.has(ORC_SH_SPEC1_STRENGTH) ? sh.p.spec1_strength : 0.0f;
    const float total = dw + sw;
    dw /= total;
    sw /= total;
    RGB diff_contrib = zero;
    if (total == 0.0f) return zero;  // the reference panics ("Shader has no weight")
    if (dw > 0.0f) {
      for (const Light& L : R.lights) {
        if ((int32_t)L.mesh == sg.geom) continue;  // LightsPrepare (scene.go:100-116)
        const int NS = sg.level > 0 ? 1 : (1 << L.samples);
        RGB col = evaluate_light_samples(sg, L, NS, diff);
        rmul(col, diff_col);
        radd(diff_contrib, col);
      }
      rscale(diff_contrib, dw);
    }
    Fresnel fr{0, sh.has(ORC_SH_IOR) ? sh.p.ior : 1.7f, {}, {}};
    if (sh.p.spec1_fresnel == 1) {
      RGB refl{{0.5f, 0.5f, 0.5f}}, edge{{0.5f, 0.5f, 0.5f}};
      if (sh.has(ORC_SH_FRESNEL_REFL)) refl = RGB{{sh.p.spec1_fresnel_refl[0], sh.p.spec1_fresnel_refl[1], sh.p.spec1_fresnel_refl[2]}};
      if (sh.has(ORC_SH_FRESNEL_EDGE))  // the reference assigns the edge colour to refl (std.go:185-187)
        refl = RGB{{sh.p.spec1_fresnel_edge[0], sh.p.spec1_fresnel_edge[1], sh.p.spec1_fresnel_edge[2]}};
      fr = Fresnel{1, 0, refl, edge};
    }
    RGB spec_contrib = zero;
    if (sw > 0.0f) {
      const float rough = sh.has(ORC_SH_SPEC1_ROUGHNESS) ? sh.p.spec1_roughness : 0.5f;
      const RGB spec_col = sh.has(ORC_SH_SPEC1_COLOUR) ? RGB{{sh.p.spec1_colour[0], sh.p.spec1_colour[1], sh.p.spec1_colour[2]}} : zero;
      Bsdf spec{rough == 0.0f ? 2 : 1, sg.lambda, project(Ut, Vt, sg.N, wi), rough * rough, fr, Ut, Vt, sg.N};
      const int spec_samples = rough == 0.0f ? 1 : 0;
      for (int i = 0; i < spec_samples; ++i) {
        const uint64_t idx = sg.I * (uint64_t)spec_samples + (uint64_t)i;
        const double r0 = vdc(idx, sg.scr0), r1 = sobol(idx, sg.scr1);
        const V3 wo = bsdf_sample(spec, r0, r1);
        const double pdf = bsdf_pdf(spec, wo);
        if (dot(wo, sg.Ng) <= 0.0f) continue;
        RGB child;
        if (trace(offset_p(sg, 1), wo, sg.level + 1, sg, child)) {
          Spectrum rho = bsdf_eval(spec, wo);
          sscale(rho, 1.0f / (float)pdf);
          RGB col = to_rgb(rho);
          rmul(col, spec_col);
          rmul(col, child);
          for (float& c : col.c)
            if (c < 0 || std::isnan(c)) c = 0;
          radd(spec_contrib, col);
        }
      }
      if (spec_samples > 0) rscale(spec_contrib, sw / (float)spec_samples);
      if (rough > 0.0f) {
        for (const Light& L : R.lights) {
          if ((int32_t)L.mesh == sg.geom) continue;
          const int NS = sg.level > 0 ? 1 : (1 << L.samples);
          RGB col = evaluate_light_samples(sg, L, NS, spec);
          rmul(col, spec_col);
          radd(spec_contrib, col);
        }
      }
    }
    RGB contrib = zero;
    radd(contrib, emission(sh));
    radd(contrib, diff_contrib);
    radd(contrib, spec_contrib);
    return contrib;
  }
};

// Per-pixel scramble: SplitMix64 of (seed, pixel, k).
uint64_t scramble(uint64_t seed, uint64_t pix, uint32_t k) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (pix * 8ull + k + 1ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

struct orc_render {
  Render r;
};

namespace orc_internal {

void camera_primary(const orc_camera& c, const std::vector<Decomp>& keys, uint32_t w, uint32_t h, uint32_t j,
                    uint64_t pix, uint64_t seed, float Po[3],
                    float Do[3], float* time, const FilterTable* filt) {
  const uint32_t x = (uint32_t)(pix % w), y = (uint32_t)(pix / w);
  double rx, ry;
  orc_raster_xy(12, j, x, y, 0, 0, &rx, &ry);  // render.go:89
  *time = (float)vdc(j, scramble(seed, pix, 2));
  if (filt && filt->n > 0) {  // filter importance sampling (render.go:99-107)
    const double fx = std::floor(rx), fy = std::floor(ry);
    double u, v;
    warp_sample(*filt, rx - fx, ry - fy, u, v);
    rx = fx + 0.5 + u;
    ry = fy + 0.5 + v;
  }
  const float Sx = (float)(-1.0 + 2.0 * (rx / (double)w));
  const float Sy = -(float)(-1.0 + 2.0 * (ry / (double)h));
  // Camera.ComputeRay (camera.go:244-284): pinhole, or a thin lens of
  // radius c.radius sampled with UniformDisk2D at (lensU, lensV)
  const float camu = Sx * c.tan_theta_focal;
  const float camv = Sy * (c.tan_theta_focal / c.aspect);
  const V3 s3 = sub(add(scale(camu, v3(1, 0, 0)), scale(camv, v3(0, 1, 0))), scale(c.focal, v3(0, 0, 1)));
  float M[16];  // Matrix4Identity without keys (camera.go:223-236)
  for (int i = 0; i < 16; ++i) M[i] = (i % 5 == 0) ? 1.0f : 0.0f;
  if (!keys.empty()) decomp_at(keys, *time, true, M);
  V3 e = v3(0, 0, 0);
  V3 sv = s3;
  if (c.radius > 0.0f) {
    const double lensU = vdc(j, scramble(seed, pix, 0)), lensV = sobol(j, scramble(seed, pix, 1));
    float x, y;
    uniform_disk(c.radius, (float)lensU, (float)lensV, x, y);
    e = add(scale(x, v3(1, 0, 0)), scale(y, v3(0, 1, 0)));
    sv = sub(s3, e);
  }
  const V3 d = v3(M[0] * sv.x + M[4] * sv.y + M[8] * sv.z, M[1] * sv.x + M[5] * sv.y + M[9] * sv.z,
                  M[2] * sv.x + M[6] * sv.y + M[10] * sv.z);
  const V3 D = normalize(d);
  const V3 P = v3(M[0] * e.x + M[4] * e.y + M[8] * e.z + M[12], M[1] * e.x + M[5] * e.y + M[9] * e.z + M[13],
                  M[2] * e.x + M[6] * e.y + M[10] * e.z + M[14]);
  Po[0] = P.x; Po[1] = P.y; Po[2] = P.z;
  Do[0] = D.x; Do[1] = D.y; Do[2] = D.z;
}

RenderScene render_scene(const orc_render* o) {
  const Render& r = o->r;
  RenderScene s;
  s.scene = r.scene;
  s.meshes = r.meshes;
  s.mesh_shaders = r.mesh_shaders;
  for (const Shader& sh : r.shaders) s.shaders.push_back(sh.p);
  s.lights = r.tri_lights;
  s.cam = r.cam;
  s.cam_keys = r.cam_keys;
  s.filter = r.filter;
  return s;
}

}  // namespace orc_internal

extern "C" {

uint64_t orc_scramble(uint64_t seed, uint64_t pix, uint32_t k) { return scramble(seed, pix, k); }

int orc_render_set_filter(orc_render* r, const orc_pixel_filter* f) {
  if (!r || !f) return -1;
  if (f->kind != 0 && f->res < 2) return -1;
  r->r.filter = orc_internal::make_filter(*f);
  return 0;
}

orc_render* orc_render_create(const orc_scene* scene, orc_mesh* const* meshes, uint32_t n_meshes,
                              const uint32_t* off, const uint32_t* cnt, const uint32_t* list, const orc_shader* shaders,
                              uint32_t n_shaders, const orc_trilight* lights, uint32_t n_lights, const orc_camera* cam) {
  auto* o = new orc_render();
  Render& r = o->r;
  r.scene = scene;
  for (uint32_t i = 0; i < n_meshes; ++i) {
    r.meshes.push_back(orc_internal::mesh_view(meshes[i]));
    r.mesh_shaders.emplace_back(list + off[i], list + off[i] + cnt[i]);
  }
  for (uint32_t i = 0; i < n_shaders; ++i) r.shaders.push_back(Shader{shaders[i]});
  r.tri_lights.assign(lights, lights + n_lights);
  for (uint32_t i = 0; i < n_lights; ++i) {
    Light L{};
    L.kind = 0;
    L.tri = lights[i];
    L.samples = lights[i].samples;
    L.shader = lights[i].shader;
    L.mesh = lights[i].mesh;
    r.lights.push_back(L);
  }
  r.cam = *cam;
  r.cam_keys.resize(1);
  orc_internal::decomp_matrix(cam->m, r.cam_keys[0]);
  return o;
}

int orc_render_set_camera_keys(orc_render* o, const float* keys16, uint32_t n) {
  if (!o || (n > 0 && !keys16)) return -1;
  o->r.cam_keys.resize(n);
  for (uint32_t i = 0; i < n; ++i) orc_internal::decomp_matrix(keys16 + 16 * i, o->r.cam_keys[i]);
  return 0;
}

void orc_set_normalize_mode(int mode, uint64_t seed) {
  g_norm_mode = mode;
  g_norm_seed = seed;
}

void orc_render_destroy(orc_render* r) { delete r; }

int orc_render_run(orc_render* o, uint32_t w, uint32_t h, uint32_t iter_begin, uint32_t iter_count, uint64_t seed,
                   float* fb, int nthreads) {
  return orc_render_run_rows(o, w, h, 0, 0, iter_begin, iter_count, seed, fb, nthreads);
}

int orc_render_run_rows(orc_render* o, uint32_t w, uint32_t h, uint32_t row0, uint32_t nrows, uint32_t iter_begin,
                        uint32_t iter_count, uint64_t seed, float* fb, int nthreads) {
  if (row0 + nrows > h) return -1;
  const Render& R = o->r;
  Renderer rr{R};
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  if (nrows == 0) nrows = h;
  const size_t npix = (size_t)w * nrows, pix0 = (size_t)row0 * w;
  for (uint32_t it = iter_begin; it < iter_begin + iter_count; ++it) {
    const uint32_t j = it + 1;  // render(iter+1, ...) (core/render.go:192)
    std::atomic<size_t> next(0);
    auto work = [&]() {
      for (;;) {
        const size_t s = next.fetch_add(256);
        if (s >= npix) break;
        for (size_t lp = s; lp < std::min(npix, s + 256); ++lp) {
          const size_t pix = pix0 + lp;  // the image pixel; lp its place in the band
          float Pf[3], Df[3], tf;
          orc_internal::camera_primary(R.cam, R.cam_keys, w, h, j, pix, seed, Pf, Df, &tf, &R.filter);
          const V3 P = v3(Pf[0], Pf[1], Pf[2]), D = v3(Df[0], Df[1], Df[2]);
          const double time = (double)tf;
          const double lambda = (720.0 - 450.0) * vdc(j, scramble(seed, pix, 3)) + 450.0;
          Ctx sc{};
          sc.lambda = (float)lambda;
          sc.time = (float)time;
          sc.I = j;
          sc.scr0 = scramble(seed, pix, 4);
          sc.scr1 = scramble(seed, pix, 5);
          sc.level = 0;
          RGB col{{0, 0, 0}};
          rr.trace(P, D, 0, sc, col);
          for (int k = 0; k < 3; ++k)
            fb[lp * 3 + k] = (fb[lp * 3 + k] * (float)j + col.c[k]) / (float)(j + 1);  // render.go:127-129
        }
      }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back(work);
    for (auto& t : th) t.join();
  }
  return 0;
}

int orc_render_add_disk_lights(orc_render* o, const orc_disklight* lights, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    const orc_disklight& d = lights[i];
    Light L{};
    L.kind = 1;
    L.P = v3(d.P[0], d.P[1], d.P[2]);
    const V3 up = v3(d.up[0], d.up[1], d.up[2]), at = v3(d.lookat[0], d.lookat[1], d.lookat[2]);
    L.N = normalize(sub(at, L.P));  // Disk.PreRender (disk.go:88-90)
    L.T = normalize(cross(L.N, up));
    L.B = cross(L.N, L.T);
    L.radius = d.radius;
    L.samples = d.samples;
    L.shader = d.shader;
    L.mesh = d.mesh;
    o->r.lights.push_back(L);
  }
  return 0;
}

int orc_render_add_sphere_lights(orc_render* o, const orc_spherelight* lights, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    Light L{};
    L.kind = 2;
    L.P = v3(lights[i].P[0], lights[i].P[1], lights[i].P[2]);
    L.radius = lights[i].radius;
    L.samples = lights[i].samples;
    L.shader = lights[i].shader;
    L.mesh = lights[i].mesh;
    o->r.lights.push_back(L);
  }
  return 0;
}

}  // extern "C"
