// orc_pt.cpp - CPU oracle of the extended path tracer (vmr_render_path).
//
// TEST INFRASTRUCTURE ONLY (see orc.h).  The extended mode has no reference
// counterpart (the reference renders direct light only, core/shader.go and
// builtin/shader/std.go), so this file restates the project's own
// estimator, written independently of the CUDA code from the same
// specification (include/vmr.h, "extended path tracing"):
//
//   for each pixel sample (pixel pix, iteration j = iter+1):
//     ray = the reference-mode camera ray (RasterXY, VdC time)
//     beta = 1, L = 0, pdf_prev = 0 (0 = camera or mirror: no MIS)
//     for d = 0 .. max_depth:
//       trace; miss: L += beta*env*w(pdf_prev, sel/(4 pi)); stop
//       hit attributes; emission of a front-facing emitter:
//         L += beta*Le*w(pdf_prev, p_light(hit))
//       d == max_depth: stop
//       two-sided frame; one light picked uniformly (TriLights, quads, env),
//       a point on it, power-heuristic weight against the BSDF pdf, shadow
//       ray; unoccluded: L += beta*f*Le*(w/p_light)
//       BSDF sample (lobe by normalised weight; diffuse cosine, GGX D(m)cos(m)
//       with the 1/(4|wo.m|) Jacobian, mirror when roughness is 0);
//       beta *= f/pdf (mirror: beta *= cs*F); Russian roulette from rr_depth
//     fb = (fb*i + L)/(i+1), i = iteration (0-based): the exact mean, unlike
//     the reference's F6 fold, which counts the initial buffer as a sample
//
// Precision: the template parameter T is the arithmetic of everything but
// the traversal.  T = float restates the CUDA kernels' float32 operation
// order (no contraction; the sampling angles through sincos_turns, the same
// float32 quarter-turn reduction and Taylor series as the kernels), so the
// two agree sample for sample.  T = double is the float64 oracle the
// converged images are checked against (same random numbers, float64
// shading, float64 accumulation).  Traversal is the float32 watertight test
// of orc_core.cpp in both: ray origins and directions are rounded to float32
// before tracing.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "orc.h"
#include "orc_internal.h"

namespace {

using orc_internal::Hit;

template <class T>
struct Vec {
  T x, y, z;
};
template <class T> inline Vec<T> mk(T x, T y, T z) { return Vec<T>{x, y, z}; }
template <class T> inline Vec<T> add(Vec<T> a, Vec<T> b) { return mk<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> inline Vec<T> sub(Vec<T> a, Vec<T> b) { return mk<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> inline Vec<T> scl(T s, Vec<T> a) { return mk<T>(a.x * s, a.y * s, a.z * s); }
template <class T> inline Vec<T> neg(Vec<T> a) { return mk<T>(-a.x, -a.y, -a.z); }
template <class T> inline T dot(Vec<T> a, Vec<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline Vec<T> cross(Vec<T> a, Vec<T> b) {
  return mk<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T> inline T len2(Vec<T> a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
template <class T> inline T vlen(Vec<T> a) { return std::sqrt((a.x * a.x + a.y * a.y) + a.z * a.z); }
template <class T> inline Vec<T> nrm(Vec<T> a) {
  const T r = T(1) / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return mk<T>(a.x * r, a.y * r, a.z * r);
}
template <class T> inline Vec<T> project(Vec<T> U, Vec<T> V, Vec<T> W, Vec<T> s) {
  return mk<T>(dot(U, s), dot(V, s), dot(W, s));
}
template <class T> inline Vec<T> expand(Vec<T> U, Vec<T> V, Vec<T> W, Vec<T> s) {
  return mk<T>(U.x * s.x + V.x * s.y + W.x * s.z, U.y * s.x + V.y * s.y + W.y * s.z, U.z * s.x + V.z * s.y + W.z * s.z);
}
template <class T> inline Vec<T> fromf(const float* p) { return mk<T>((T)p[0], (T)p[1], (T)p[2]); }
template <class T> inline T tmax3(T a, T b, T c) { return a > b ? (a > c ? a : c) : (b > c ? b : c); }

// sin and cos of 2*pi*u, u in [0, 1).  float: u*4 split exactly into a
// quarter turn and a fraction f, f > 1/2 reflected (sin and cos swapped),
// x = (pi/2) f in [0, pi/4] through the Taylor series of sin to x^9 and cos
// to x^10, then the quarter-turn rotation; every operation rounds to float32
// in this order (compiled without contraction), as the CUDA kernels do.
// double: std::sin/std::cos of the float64 angle.
inline void sincos_turns_f(float u, float& s, float& c) {
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
template <class T> inline void sincos_turns(T u, T& s, T& c);
template <> inline void sincos_turns<float>(float u, float& s, float& c) { sincos_turns_f(u, s, c); }
template <> inline void sincos_turns<double>(double u, double& s, double& c) {
  const double th = 2 * 3.14159265358979323846 * u;
  s = std::sin(th);
  c = std::cos(th);
}

template <class T> struct Consts;
template <> struct Consts<float> {
  static constexpr float pi = 3.14159265358f;    // math.Pi as the reference's float32
  static constexpr float inv4pi = 0.0795774715f;  // float32(1/(4 pi))
};
template <> struct Consts<double> {
  static constexpr double pi = 3.14159265358979323846;
  static constexpr double inv4pi = 0.07957747154594767;
};

// ------------------------------------------------------------ random ----
inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
const uint64_t kGold = 0x9E3779B97F4A7C15ull;
inline uint64_t sample_key(uint64_t seed, uint64_t pix, uint64_t j) {
  return mix64(mix64(seed + kGold * (pix + 1)) + kGold * (j + 1));
}
// 24 random bits as a float in [0, 1) (exact in float32).
inline float rnd(uint64_t key, uint32_t dim) {
  return (float)(uint32_t)(mix64(key + kGold * (uint64_t)(dim + 1)) >> 40) * 5.9604644775390625e-08f;
}

// ------------------------------------------------------------ offsets ----
inline float next_up(float v) {
  if (std::isinf(v) && v > 0) return v;
  if (v == 0.0f) v = 0.0f;
  uint32_t u;
  std::memcpy(&u, &v, 4);
  if (v >= 0.0f) ++u; else --u;
  std::memcpy(&v, &u, 4);
  return v;
}
inline float next_down(float v) {
  if (std::isinf(v) && v < 0) return v;
  if (v == 0.0f) v = 0.0f;
  uint32_t u;
  std::memcpy(&u, &v, 4);
  if (v >= 0.0f) --u; else ++u;
  std::memcpy(&v, &u, 4);
  return v;
}

template <class T>
struct Surf {
  Vec<T> P, N, Ng, Poffset, dPdu, dPdv;
};

// OffsetP (core/shader.go:139-163), toward +Poffset (dir > 0) or -Poffset;
// the result is the float32 ray origin.
template <class T>
void offset_p(const Surf<T>& s, int dir, float out[3]) {
  const Vec<T> o = dir < 0 ? neg(s.Poffset) : s.Poffset;
  const Vec<T> p = add(s.P, o);
  const T oa[3] = {o.x, o.y, o.z};
  const T pa[3] = {p.x, p.y, p.z};
  for (int i = 0; i < 3; ++i) {
    float v = (float)pa[i];
    if (oa[i] > 0) v = next_up(v);
    else if (oa[i] < -T(0)) v = next_down(v);
    out[i] = v;
  }
}

// ------------------------------------------------------------ material ----
template <class T>
struct Mat {
  T dw, sw;             // normalised weights
  Vec<T> cd, cs;        // diffuse and spec1 colour
  T rd;                 // diffuse roughness (0 = Lambert)
  T alpha;              // GGX alpha = Spec1Roughness^4
  bool mirror;          // Spec1Roughness == 0
  int fresnel;          // 0 dielectric, 1 conductor
  T eta;
  Vec<T> frefl, fedge;
};

template <class T> inline T sqr(T v) { return v * v; }

template <class T>
Vec<T> fresnel(const Mat<T>& m, T c) {
  if (m.fresnel == 0) {  // Dielectric.Kr (fresnel/dielectric.go:34-47)
    T g = (m.eta * m.eta) - 1 + (c * c);
    if (g < T(0)) return mk<T>(1, 1, 1);
    g = std::sqrt(g);
    const T fr = T(0.5) * sqr((g - c) / (g + c)) * (1 + sqr((c * (g + c) - 1) / (c * (g - c) + 1)));
    return mk<T>(fr, fr, fr);
  }
  const T r3[3] = {m.frefl.x, m.frefl.y, m.frefl.z}, g3[3] = {m.fedge.x, m.fedge.y, m.fedge.z};
  T out[3];
  for (int k = 0; k < 3; ++k) {  // Conductor.Kr (fresnel/conductor.go:58-89)
    const T r = r3[k] > T(0.99) ? T(0.99) : (r3[k] < T(0) ? T(0) : r3[k]);
    const T g = g3[k];
    const T nmin = (1 - r) / (1 + r);
    const T nmax = (1 + std::sqrt(r)) / (1 - std::sqrt(r));
    const T n = nmin * g + (1 - g) * nmax;
    const T k2 = ((n + 1) * (n + 1) * r - (n - 1) * (n - 1)) / (1 - r);
    const T rs = (n * n + k2 - 2 * n * c + c * c) / (n * n + k2 + 2 * n * c + c * c);
    const T rp = ((n * n + k2) * c * c - 2 * n * c + 1) / ((n * n + k2) * c * c + 2 * n * c + 1);
    out[k] = T(0.5) * (rs + rp);
  }
  return mk<T>(out[0], out[1], out[2]);
}

template <class T> inline T chi(T x) { return x > T(0) ? T(1) : T(0); }
template <class T>
T ggx_g1(Vec<T> w, Vec<T> m, T alpha) {
  const T denom = 1 + std::sqrt(1 + (alpha * alpha) * ((T(1) / (w.z * w.z)) - 1));
  return chi(dot(w, m) / w.z) * 2 / denom;
}
template <class T>
T ggx_d(Vec<T> m, T alpha) {
  if (m.z <= T(0)) return T(0);
  const T pi = Consts<T>::pi;
  if (m.z == T(1)) return T(1) / (pi * alpha * alpha);
  const T denom = pi * sqr(m.z * m.z) * sqr(alpha * alpha + ((T(1) / (m.z * m.z)) - 1));
  return (alpha * alpha) / denom;
}

// f(wi, wo) * |cos(wo)| in the local frame (wi.z > 0 by the two-sided frame).
template <class T>
Vec<T> bsdf_f(const Mat<T>& m, Vec<T> wi, Vec<T> wo) {
  const T pi = Consts<T>::pi;
  Vec<T> f = mk<T>(0, 0, 0);
  if (wo.z <= T(0)) return f;
  if (m.dw > T(0)) {
    T s;
    if (m.rd == T(0)) {
      s = wo.z / pi;  // Lambert
    } else {  // OrenNayar (bsdf/orennayar.go:42-73), sigma = roughness^2
      // sin(max theta) * tan(min theta) and cos(phiO - phiI) from the
      // direction components (no angles)
      const T sigma = m.rd * m.rd;
      const T A = 1 - (T(0.5) * (sigma * sigma) / ((sigma * sigma) + T(0.57)));
      const T B = T(0.45) * (sigma * sigma) / ((sigma * sigma) + T(0.09));
      const T sI = std::sqrt(std::max(T(0), T(1) - wi.z * wi.z)), sO = std::sqrt(std::max(T(0), T(1) - wo.z * wo.z));
      const T C = wi.z < wo.z ? sI * (sO / wo.z) : sO * (sI / wi.z);
      const T den = sI * sO;
      const T gm = den > T(1e-6f) ? (wi.x * wo.x + wi.y * wo.y) / den : T(0);
      s = wo.z * (A + (B * (gm > T(0) ? gm : T(0)) * C)) / pi;
    }
    const T k = m.dw * s;
    f = mk<T>(k * m.cd.x, k * m.cd.y, k * m.cd.z);
  }
  if (m.sw > T(0) && !m.mirror) {
    const Vec<T> h = nrm(add(wi, wo));
    const Vec<T> F = fresnel(m, std::fabs(dot(wi, h)));
    const T numer = ggx_g1(wi, h, m.alpha) * ggx_g1(wo, h, m.alpha) * ggx_d(h, m.alpha);
    const T denom = 4 * wi.z * wo.z;
    T s = wo.z * numer / denom;
    if (!(s > T(0))) s = T(0);  // negative or NaN
    const T k = m.sw * s;
    f = add(f, mk<T>(k * m.cs.x * F.x, k * m.cs.y * F.y, k * m.cs.z * F.z));
  }
  return f;
}

// Solid-angle pdf of sampling wo from wi (the non-mirror part).
template <class T>
T bsdf_pdf(const Mat<T>& m, Vec<T> wi, Vec<T> wo) {
  const T pi = Consts<T>::pi;
  if (wo.z <= T(0)) return T(0);
  T p = m.dw * (wo.z / pi);
  if (m.sw > T(0) && !m.mirror) {
    const Vec<T> h = nrm(add(wi, wo));
    const T d = std::fabs(dot(wo, h));
    if (d > T(0)) p = p + m.sw * (ggx_d(h, m.alpha) * h.z / (4 * d));
  }
  return p;
}

// Power heuristic (beta = 2).
template <class T> inline T power_w(T a, T b) { return (a * a) / (a * a + b * b); }

// ------------------------------------------------------------- lights ----
template <class T>
struct Light {
  int kind;             // 0 triangle, 1 quad, 2 environment
  Vec<T> p0, a, b;      // triangle: p0, p1, p2; quad: p0, e1, e2
  Vec<T> N;             // emitting side
  T area;
  Vec<T> Le;
  int32_t geom;
};

template <class T>
Vec<T> emission(const orc_shader& s) {
  if (!(s.flags & ORC_SH_EMISSION_STRENGTH)) return mk<T>(0, 0, 0);
  const Vec<T> c = (s.flags & ORC_SH_EMISSION_COLOUR) ? fromf<T>(s.emission_colour) : mk<T>(0, 0, 0);
  const T k = (T)s.emission_strength;
  return mk<T>(c.x * k, c.y * k, c.z * k);
}

template <class T>
Mat<T> material(const orc_shader& s) {
  Mat<T> m{};
  T dw = (s.flags & ORC_SH_DIFFUSE_STRENGTH) ? (T)s.diffuse_strength : T(0);
  T sw = (s.flags & ORC_SH_SPEC1_STRENGTH) ? (T)s.spec1_strength : T(0);
  const T tw = dw + sw;
  m.dw = dw / tw;
  m.sw = sw / tw;
  m.cd = (s.flags & ORC_SH_DIFFUSE_COLOUR) ? fromf<T>(s.diffuse_colour) : mk<T>(0, 0, 0);
  m.cs = (s.flags & ORC_SH_SPEC1_COLOUR) ? fromf<T>(s.spec1_colour) : mk<T>(0, 0, 0);
  m.rd = (s.flags & ORC_SH_DIFFUSE_ROUGHNESS) ? (T)s.diffuse_roughness : T(0.5);
  const T rs = (s.flags & ORC_SH_SPEC1_ROUGHNESS) ? (T)s.spec1_roughness : T(0.5);
  m.mirror = rs == T(0);
  m.alpha = sqr(rs * rs);
  m.fresnel = s.spec1_fresnel;
  m.eta = (s.flags & ORC_SH_IOR) ? (T)s.ior : T(1.7);
  m.frefl = mk<T>(T(0.5), T(0.5), T(0.5));
  m.fedge = mk<T>(T(0.5), T(0.5), T(0.5));
  if (s.flags & ORC_SH_FRESNEL_REFL) m.frefl = fromf<T>(s.spec1_fresnel_refl);
  if (s.flags & ORC_SH_FRESNEL_EDGE) m.frefl = fromf<T>(s.spec1_fresnel_edge);  // the reference's assignment
  return m;
}

template <class T>
struct PT {
  orc_internal::RenderScene R;
  std::vector<Light<T>> lights;
  std::vector<int32_t> light_of_geom;
  Vec<T> env;
  bool has_env = false;
  uint32_t max_depth = 4, rr_depth = 3;

  // Matrix4MulPoint / Matrix4MulVec of a column-major matrix (sums left to
  // right) and Matrix4MulVec of the inverse transposed, in T.
  static Vec<T> xf_pt(const float* M, Vec<T> b) {
    return mk<T>((T)M[0] * b.x + (T)M[4] * b.y + (T)M[8] * b.z + (T)M[12],
                 (T)M[1] * b.x + (T)M[5] * b.y + (T)M[9] * b.z + (T)M[13],
                 (T)M[2] * b.x + (T)M[6] * b.y + (T)M[10] * b.z + (T)M[14]);
  }
  static Vec<T> xf_vec(const float* M, Vec<T> b) {
    return mk<T>((T)M[0] * b.x + (T)M[4] * b.y + (T)M[8] * b.z, (T)M[1] * b.x + (T)M[5] * b.y + (T)M[9] * b.z,
                 (T)M[2] * b.x + (T)M[6] * b.y + (T)M[10] * b.z);
  }
  static Vec<T> inv_t(const float* I, Vec<T> b) {
    return mk<T>((T)I[0] * b.x + (T)I[1] * b.y + (T)I[2] * b.z, (T)I[4] * b.x + (T)I[5] * b.y + (T)I[6] * b.z,
                 (T)I[8] * b.x + (T)I[9] * b.y + (T)I[10] * b.z);
  }
  // ShaderContext.ApplyTransform (core/shader.go:129-135); s.P holds Po.
  static void apply_transform(Surf<T>& s, const float* M, const float* I) {
    const Vec<T> Po = s.P;
    s.P = xf_pt(M, Po);
    s.N = nrm(inv_t(I, s.N));
    s.Ng = nrm(inv_t(I, s.Ng));
    s.dPdu = nrm(xf_vec(M, s.dPdu));
    s.dPdv = nrm(xf_vec(M, s.dPdv));
  }

  // Hit attributes (trace.go:276-515 and :520-719, sphere/trace.go; the
  // same expressions as the reference mode).  Returns the shader id or -1.
  int32_t attributes(const Hit& h, Surf<T>& s, const float* Ro, const float* Rd, float time) const {
    const orc_internal::MeshView& m = R.meshes[h.geom];
    const auto& list = R.mesh_shaders[h.geom];
    // the GeomInstance / Proc transform that reaches this geom, at the ray's
    // time (instance.go:105-110, proc.go:133-138); a sphere inside one takes
    // the ray as its group mapped it (instance.go:91-93), in float32 as the
    // traversal does
    float OT[16], OI[16];
    if (m.outer) {
      orc_internal::decomp_at(*m.outer, time, false, OT);
      orc_internal::matrix_inverse(OT, OI);
    }
    float Rog[3], Rdg[3];
    if (m.sphere && m.outer) {
      for (int k = 0; k < 3; ++k) {
        Rog[k] = OI[k] * Ro[0] + OI[4 + k] * Ro[1] + OI[8 + k] * Ro[2] + OI[12 + k];
        Rdg[k] = OI[k] * Rd[0] + OI[4 + k] * Rd[1] + OI[8 + k] * Rd[2];
      }
      Ro = Rog;
      Rd = Rdg;
    }
    if (m.sphere) {  // sphere/trace.go: P = ray.P + t ray.D, N = normalize(P - centre)
      if (list.empty()) return -1;
      const float P[3] = {Ro[0] + Rd[0] * h.t, Ro[1] + Rd[1] * h.t, Ro[2] + Rd[2] * h.t};  // float32, as the hit
      const Vec<T> Pv = fromf<T>(P);
      const Vec<T> N = nrm(sub(Pv, fromf<T>(m.sc)));
      s.Poffset = scl(T(0.001f), N);
      s.P = Pv;
      s.N = nrm(N);
      s.Ng = nrm(N);
      s.dPdu = mk<T>(1, 0, 0);
      s.dPdv = mk<T>(0, 0, 1);
      if (m.outer) apply_transform(s, OT, OI);
      return (int32_t)list[0];
    }
    const uint32_t i0 = m.idxp[h.elem * 3 + 0], i1 = m.idxp[h.elem * 3 + 1], i2 = m.idxp[h.elem * 3 + 2];
    float tm = 0.0f;
    int key = 0, key2 = 0;
    if (m.motion) {  // TraceMotionElems' lerped vertices (trace.go:520-560)
      const float k = time * (float)(m.keys - 1);
      tm = k - std::floor(k);
      key = (int)std::floor(k);
      key2 = (int)std::ceil(k);
    }
    auto vert = [&](uint32_t i) {
      const float* a = m.verts + ((size_t)key * m.nverts + i) * 3;
      if (!m.motion) return fromf<T>(a);
      const float* b = m.verts + ((size_t)key2 * m.nverts + i) * 3;
      const float v[3] = {(1.0f - tm) * a[0] + tm * b[0], (1.0f - tm) * a[1] + tm * b[1], (1.0f - tm) * a[2] + tm * b[2]};
      return fromf<T>(v);
    };
    const Vec<T> V0 = vert(i0), V1 = vert(i1), V2 = vert(i2);
    const uint8_t sidx = m.shaderidx ? m.shaderidx[h.elem] : 0;
    if (sidx >= list.size()) return -1;
    const T U = (T)h.u, V = (T)h.v, W = (T)h.w;
    const T xs = std::fabs(U * V0.x) + std::fabs(V * V1.x) + std::fabs(W * V2.x);
    const T ys = std::fabs(U * V0.y) + std::fabs(V * V1.y) + std::fabs(W * V2.y);
    const T zs = std::fabs(U * V0.z) + std::fabs(V * V1.z) + std::fabs(W * V2.z);
    const Vec<T> e0 = sub(V1, V0), e1 = sub(V2, V0);
    const Vec<T> Ng = nrm(mk<T>(e0.y * e1.z - e0.z * e1.y, e0.z * e1.x - e0.x * e1.z, e0.x * e1.y - e0.y * e1.x));
    Vec<T> N = Ng;
    if (m.motion ? m.mnormals != nullptr : m.normals != nullptr) {
      // static: per-vertex normals; motion: the element's corner normals of
      // the two keys lerped at the ray's time (trace.go:694-712)
      auto cn = [&](uint32_t i, uint32_t j) {
        if (!m.motion) return fromf<T>(m.normals + i * 3);
        const size_t c = (size_t)h.elem * 3 + j;
        const float* a = m.mnormals + ((size_t)key * m.mnormals_per_key + c) * 3;
        const float* b = m.mnormals + ((size_t)key2 * m.mnormals_per_key + c) * 3;
        const float v[3] = {(1.0f - tm) * a[0] + tm * b[0], (1.0f - tm) * a[1] + tm * b[1], (1.0f - tm) * a[2] + tm * b[2]};
        return fromf<T>(v);
      };
      const Vec<T> N0 = cn(i0, 0), N1 = cn(i1, 1), N2 = cn(i2, 2);
      N = nrm(mk<T>(U * N0.x + V * N1.x + W * N2.x, U * N0.y + V * N1.y + W * N2.y, U * N0.z + V * N1.z + W * N2.z));
    }
    const float g7f = (7.0f * 5.96046448e-08f) / (1 - 7.0f * 5.96046448e-08f);  // Gamma(7) of float32 data
    const T g7 = (T)g7f;
    const T d = g7 * xs * std::fabs(Ng.x) + g7 * ys * std::fabs(Ng.y) + g7 * zs * std::fabs(Ng.z);
    s.Poffset = scl(d, Ng);
    s.P = mk<T>(U * V0.x + V * V1.x + W * V2.x, U * V0.y + V * V1.y + W * V2.y, U * V0.z + V * V1.z + W * V2.z);
    Vec<T> dpdu, dpdv;
    if (m.motion) {  // raw edges (trace.go:655-661)
      dpdu = e0;
      dpdv = e1;
    } else {
      Vec<T> axisu = sub(mk<T>(1, 0, 0), scl(dot(mk<T>(1, 0, 0), Ng), Ng));
      if (len2(axisu) < T(0.1) || std::fabs(dot(axisu, Ng)) > T(0.3))
        axisu = sub(mk<T>(0, 0, 1), scl(dot(mk<T>(0, 0, 1), Ng), Ng));
      dpdu = nrm(axisu);
      dpdv = cross(Ng, dpdu);
    }
    s.N = nrm(N);
    s.Ng = nrm(Ng);
    s.dPdu = nrm(dpdu);
    s.dPdv = nrm(dpdv);
    // to world space as the reference mode does: a transformed mesh's
    // PolyMesh.Trace sets N = M^-T N (trace.go:67-74), then ApplyTransform
    // with the group's transform when one reaches the geom, else the mesh's
    // own (core/shader.go:129-135); keyed transforms at the ray's time
    float MT[16], MI[16];
    const bool own = m.has_xf || m.xkeys;
    if (m.xkeys) {
      orc_internal::decomp_at(*m.xkeys, time, false, MT);
      orc_internal::matrix_inverse(MT, MI);
    } else if (m.has_xf) {
      std::memcpy(MT, m.xf, sizeof(MT));
      std::memcpy(MI, m.xinv, sizeof(MI));
    }
    if (own) s.N = inv_t(MI, s.N);
    if (m.outer) apply_transform(s, OT, OI);
    else if (own) apply_transform(s, MT, MI);
    return (int32_t)list[sidx];
  }

  Hit trace(const float P[3], const float D[3], float tmax, float time, bool shadow) const {
    return orc_internal::trace(R.scene, P, D, tmax, time, shadow);
  }

  // One path; returns L.
  Vec<T> path(uint64_t key, const float P0[3], const float D0[3], float time) const {
    Vec<T> beta = mk<T>(1, 1, 1), L = mk<T>(0, 0, 0);
    T pdf_prev = 0;
    float Pf[3] = {P0[0], P0[1], P0[2]}, Df[3] = {D0[0], D0[1], D0[2]};
    Vec<T> D = fromf<T>(Df);
    const int nL = (int)lights.size();
    const T sel = nL > 0 ? T(1) / (T)nL : T(0);
    for (uint32_t d = 0; d <= max_depth; ++d) {
      const Hit h = trace(Pf, Df, INFINITY, time, false);
      if (!h.hit) {
        if (has_env) {
          const T w = pdf_prev == T(0) ? T(1) : power_w(pdf_prev, sel * Consts<T>::inv4pi);
          L = add(L, mk<T>(beta.x * env.x * w, beta.y * env.y * w, beta.z * env.z * w));
        }
        break;
      }
      Surf<T> s;
      const int32_t shid = attributes(h, s, Pf, Df, time);
      if (shid < 0) break;
      const orc_shader& sh = R.shaders[shid];
      const Vec<T> wi = neg(D);
      const bool front = dot(s.Ng, wi) > T(0);
      const Vec<T> Le = emission<T>(sh);
      if (front && (Le.x != T(0) || Le.y != T(0) || Le.z != T(0))) {
        T w = 1;
        const int32_t li = (size_t)h.geom < light_of_geom.size() ? light_of_geom[h.geom] : -1;
        if (pdf_prev != T(0) && li >= 0) {
          const Light<T>& l = lights[li];
          const T t = (T)h.t;
          const T pl = sel * (t * t) / (l.area * std::fabs(dot(D, s.Ng)));
          w = power_w(pdf_prev, pl);
        }
        L = add(L, mk<T>(beta.x * Le.x * w, beta.y * Le.y * w, beta.z * Le.z * w));
      }
      if (d == max_depth) break;
      const T tw = ((sh.flags & ORC_SH_DIFFUSE_STRENGTH) ? (T)sh.diffuse_strength : T(0)) +
                   ((sh.flags & ORC_SH_SPEC1_STRENGTH) ? (T)sh.spec1_strength : T(0));
      if (tw == T(0)) break;  // no weight (the reference panics)
      if (!front) {           // two-sided: face the incoming ray
        s.N = neg(s.N);
        s.Ng = neg(s.Ng);
        s.Poffset = neg(s.Poffset);
      }
      Vec<T> Vt = cross(s.N, s.dPdu);
      if (len2(Vt) < T(0.1)) Vt = cross(s.N, s.dPdv);
      Vt = nrm(Vt);
      const Vec<T> Ut = nrm(cross(s.N, Vt));
      const Mat<T> m = material<T>(sh);
      const Vec<T> wil = project(Ut, Vt, s.N, wi);
      const uint32_t base = 8 * d;
      // ---- next-event estimation
      if (nL > 0 && (m.dw > T(0) || !m.mirror)) {
        const T u = (T)rnd(key, base + 0);
        int li = (int)(u * (T)nL);
        if (li > nL - 1) li = nL - 1;
        const T u0 = (T)rnd(key, base + 1), u1 = (T)rnd(key, base + 2);
        const Light<T>& l = lights[li];
        Vec<T> Ld;
        T dist = 0, pl = 0;
        bool ok = true;
        if (l.kind == 2) {
          const T z = 1 - 2 * u0;
          const T rr = std::sqrt((1 - z * z) > T(0) ? (1 - z * z) : T(0));
          T sp, cp;
          sincos_turns(u1, sp, cp);
          Ld = mk<T>(rr * cp, rr * sp, z);
          pl = sel * Consts<T>::inv4pi;
        } else {
          Vec<T> Pl;
          if (l.kind == 0) {
            const T su = std::sqrt(u0);
            const T b0 = 1 - su, b1 = su * (1 - u1), b2 = su * u1;
            Pl = add(add(scl(b0, l.p0), scl(b1, l.a)), scl(b2, l.b));
          } else {
            Pl = add(add(l.p0, scl(u0, l.a)), scl(u1, l.b));
          }
          const Vec<T> Dv = sub(Pl, s.P);
          dist = vlen(Dv);
          Ld = nrm(Dv);
          const T cl = dot(Ld, l.N);
          if (!(cl < T(0))) ok = false;
          else pl = sel * (dist * dist) / (l.area * (-cl));
        }
        if (ok && dot(Ld, s.Ng) > T(0) && dot(Ld, s.N) > T(0) && pl > T(0) && !std::isinf(pl)) {
          const Vec<T> wol = project(Ut, Vt, s.N, Ld);
          const Vec<T> f = bsdf_f(m, wil, wol);
          const T pb = bsdf_pdf(m, wil, wol);
          const T w = power_w(pl, pb);
          const T k = w / pl;
          const Vec<T> c = mk<T>(beta.x * f.x * l.Le.x * k, beta.y * f.y * l.Le.y * k, beta.z * f.z * l.Le.z * k);
          if (c.x > T(0) || c.y > T(0) || c.z > T(0)) {
            float o[3];
            offset_p(s, 1, o);
            float sd[3];
            float stmax;
            if (l.kind == 2) {
              sd[0] = (float)Ld.x; sd[1] = (float)Ld.y; sd[2] = (float)Ld.z;
              stmax = INFINITY;
            } else {
              const T sd_len = dist * T(0.9999f);
              sd[0] = (float)(Ld.x * sd_len); sd[1] = (float)(Ld.y * sd_len); sd[2] = (float)(Ld.z * sd_len);
              stmax = 1.0f;
            }
            if (!trace(o, sd, stmax, time, true).hit) L = add(L, c);
          }
        }
      }
      // ---- BSDF sample
      const T ul = (T)rnd(key, base + 3);
      const T r0 = (T)rnd(key, base + 4), r1 = (T)rnd(key, base + 5);
      Vec<T> wol;
      bool delta = false;
      if (ul < m.dw) {  // CosineHemisphere (math/sample/sample.go:18-27)
        const T r = std::sqrt(T(1) - r0);
        T sp, cp;
        sincos_turns(r1, sp, cp);
        wol = mk<T>(r * cp, r * sp, std::sqrt(r0));
      } else if (m.mirror) {
        wol = mk<T>(-wil.x, -wil.y, wil.z);
        delta = true;
      } else {  // GGX: tan(theta_m) = alpha sqrt(r0) / sqrt(1-r0) (microfacetggx.go:82-100)
        const T a = m.alpha * std::sqrt(r0), bq = std::sqrt(T(1) - r0);
        const T hyp = std::sqrt(a * a + bq * bq);
        const T st = a / hyp, ct = bq / hyp;
        T sp, cp;
        sincos_turns(r1, sp, cp);
        const Vec<T> mh = mk<T>(st * cp, st * sp, ct);
        wol = nrm(sub(scl(2 * std::fabs(dot(mh, wil)), mh), wil));
      }
      const Vec<T> wo = expand(Ut, Vt, s.N, wol);
      if (!(dot(wo, s.Ng) > T(0))) break;
      if (delta) {
        const Vec<T> F = fresnel(m, wil.z);
        beta = mk<T>(beta.x * (m.cs.x * F.x), beta.y * (m.cs.y * F.y), beta.z * (m.cs.z * F.z));
        pdf_prev = 0;
      } else {
        const Vec<T> f = bsdf_f(m, wil, wol);
        const T pb = bsdf_pdf(m, wil, wol);
        if (!(pb > T(0))) break;
        beta = mk<T>(beta.x * (f.x / pb), beta.y * (f.y / pb), beta.z * (f.z / pb));
        pdf_prev = pb;
      }
      // ---- Russian roulette
      if (d + 1 >= rr_depth) {
        T q = tmax3(beta.x, beta.y, beta.z);
        if (q > T(0.95)) q = T(0.95);
        const T ur = (T)rnd(key, base + 6);
        if (!(ur < q)) break;
        beta = mk<T>(beta.x / q, beta.y / q, beta.z / q);
      }
      offset_p(s, 1, Pf);
      Df[0] = (float)wo.x; Df[1] = (float)wo.y; Df[2] = (float)wo.z;
      D = mk<T>((T)Df[0], (T)Df[1], (T)Df[2]);
    }
    return L;
  }
};

template <class T>
void setup(PT<T>& pt, const orc_render* r, const orc_quad_light* quads, uint32_t nq, const orc_pt_params* p) {
  pt.R = orc_internal::render_scene(r);
  pt.max_depth = p->max_depth;
  pt.rr_depth = p->rr_depth;
  pt.env = mk<T>((T)p->env[0], (T)p->env[1], (T)p->env[2]);
  pt.has_env = p->env[0] != 0.0f || p->env[1] != 0.0f || p->env[2] != 0.0f;
  pt.light_of_geom.assign(pt.R.meshes.size(), -1);
  for (const orc_trilight& t : pt.R.lights) {
    Light<T> l{};
    l.kind = 0;
    l.p0 = fromf<T>(t.p0);
    l.a = fromf<T>(t.p1);
    l.b = fromf<T>(t.p2);
    const Vec<T> c = cross(sub(l.a, l.p0), sub(l.b, l.p0));
    l.N = nrm(c);
    l.area = T(0.5) * vlen(c);
    l.Le = emission<T>(pt.R.shaders[t.shader]);
    l.geom = (int32_t)t.mesh;
    if (t.mesh < pt.light_of_geom.size()) pt.light_of_geom[t.mesh] = (int32_t)pt.lights.size();
    pt.lights.push_back(l);
  }
  for (uint32_t i = 0; i < nq; ++i) {
    const orc_quad_light& q = quads[i];
    Light<T> l{};
    l.kind = 1;
    l.p0 = fromf<T>(q.p0);
    l.a = fromf<T>(q.e1);
    l.b = fromf<T>(q.e2);
    const Vec<T> c = cross(l.a, l.b);
    l.N = nrm(c);
    l.area = vlen(c);
    l.Le = emission<T>(pt.R.shaders[q.shader]);
    l.geom = (int32_t)q.mesh;
    if (q.mesh < pt.light_of_geom.size()) pt.light_of_geom[q.mesh] = (int32_t)pt.lights.size();
    pt.lights.push_back(l);
  }
  if (pt.has_env) {
    Light<T> l{};
    l.kind = 2;
    l.Le = pt.env;
    l.geom = -1;
    pt.lights.push_back(l);
  }
}

// Rows [row0, row0 + nrows) of the image (nrows 0: all); fb and fb64 hold
// those rows only.
template <class T>
int run(const orc_render* r, const orc_quad_light* quads, uint32_t nq, const orc_pt_params* p, float* fb, double* fb64,
        int nthreads, uint32_t row0 = 0, uint32_t nrows = 0) {
  PT<T> pt;
  setup(pt, r, quads, nq, p);
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  const uint32_t w = p->width, h = p->height;
  if (nrows == 0) nrows = h;
  const size_t npix = (size_t)w * nrows, pix0 = (size_t)row0 * w;
  for (uint32_t it = p->iter_begin; it < p->iter_begin + p->iter_count; ++it) {
    const uint32_t j = it + 1;
    std::atomic<size_t> next(0);
    auto work = [&]() {
      for (;;) {
        const size_t s0 = next.fetch_add(64);
        if (s0 >= npix) break;
        for (size_t lp = s0; lp < std::min(npix, s0 + 64); ++lp) {
          const size_t gp = pix0 + lp;  // the image pixel
          const size_t pix = lp;        // its place in the band
          float P[3], D[3], time;
          orc_internal::camera_primary(pt.R.cam, pt.R.cam_keys, w, h, j, gp, p->seed, P, D, &time, &pt.R.filter);
          const Vec<T> L = pt.path(sample_key(p->seed, gp, j), P, D, time);
          const T Lc[3] = {L.x, L.y, L.z};
          for (int k = 0; k < 3; ++k) {  // exact running mean over iterations 0..it
            if (fb) fb[pix * 3 + k] = (fb[pix * 3 + k] * (float)it + (float)Lc[k]) / (float)(it + 1);
            if (fb64) fb64[pix * 3 + k] = (fb64[pix * 3 + k] * (double)it + (double)Lc[k]) / (double)(it + 1);
          }
        }
      }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back(work);
    for (auto& t : th) t.join();
  }
  return 0;
}

}  // namespace

extern "C" {

float orc_pt_rnd(uint64_t seed, uint64_t pix, uint32_t j, uint32_t dim) { return rnd(sample_key(seed, pix, j), dim); }

void orc_sincos_turns(const float* u, size_t n, float* s, float* c) {
  for (size_t i = 0; i < n; ++i) sincos_turns_f(u[i], s[i], c[i]);
}

int orc_pt_run(const orc_render* r, const orc_quad_light* quads, uint32_t n_quads, const orc_pt_params* p, float* fb,
               double* fb64, int precision, int nthreads) {
  return orc_pt_run_rows(r, quads, n_quads, p, 0, 0, fb, fb64, precision, nthreads);
}

int orc_pt_run_rows(const orc_render* r, const orc_quad_light* quads, uint32_t n_quads, const orc_pt_params* p,
                    uint32_t row0, uint32_t nrows, float* fb, double* fb64, int precision, int nthreads) {
  if (!r || !p || row0 + nrows > p->height) return -1;
  if (precision == 64) return run<double>(r, quads, n_quads, p, fb, fb64, nthreads, row0, nrows);
  return run<float>(r, quads, n_quads, p, fb, fb64, nthreads, row0, nrows);
}

}  // extern "C"
