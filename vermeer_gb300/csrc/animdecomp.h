// animdecomp.h - decomposed transforms: the camera's motion keys
// (builtin/camera/camera.go:207-236), PolyMesh transform motion keys
// (builtin/geom/polymesh/trace.go:33-48) and the GeomInstance / Proc
// transforms (builtin/geom/instance/instance.go:20-36,89,
// builtin/geom/proc/proc.go:20-36,104).
//
// The reference never uses a keyed matrix directly: each key is split into
// translation, rotation quaternion and stretch (TransformDecompMatrix4,
// math/animdecomp.go:20-62, a polar decomposition iterated with
// Matrix4Inverse), keys are blended component-wise (TransformDecompLerp,
// animdecomp.go:74-80: Vec3Lerp, QuatSlerp, Matrix4Lerp) and the matrix is
// rebuilt (TransformDecompToMatrix4, animdecomp.go:65-71).  Even one key goes
// through that round trip, which is not exact, so the functions below follow
// the reference's float32 operation order step by step (host code is built
// with -ffp-contract=off and device code with -fmad=false, so no product is
// fused).  Acos and Sin are evaluated in float64 and rounded to float32, as
// math/sincos.go does; Sqrt is the IEEE float32 square root (SQRTSS).
//
// Matrices are column-major float[16] (math/matrix4.go:7-19): element (row i,
// column j) is m[j*4+i].
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define VMR_HD __host__ __device__ __forceinline__
#else
#define VMR_HD inline
#endif

namespace vmr {
namespace anim {

struct Decomp {
  float T[3];   // translation
  float R[4];   // rotation quaternion x, y, z, w
  float S[16];  // stretch matrix
};

VMR_HD float f_sqrt(float x) {
#ifdef __CUDA_ARCH__
  return __fsqrt_rn(x);
#else
  return sqrtf(x);
#endif
}
VMR_HD float f_div(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}
VMR_HD float f_abs(float x) { return x < 0.0f ? -x : (x == 0.0f ? 0.0f : x); }  // math.Abs (math/abs.go)
// math/sincos.go: float64 evaluation rounded to float32.
VMR_HD float f_acos(float x) { return (float)acos((double)x); }
VMR_HD float f_sin(float x) { return (float)sin((double)x); }

VMR_HD void identity(float* m) {
  for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}

// Matrix4Mul (matrix4.go:87-97): c starts at zero and accumulates
// a(i,k) * b(k,j) for k = 0..3 in order.
VMR_HD void mul(const float* a, const float* b, float* c) {
  float r[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      float s = 0.0f;
      for (int k = 0; k < 4; ++k) s = s + a[k * 4 + i] * b[j * 4 + k];
      r[j * 4 + i] = s;
    }
  for (int i = 0; i < 16; ++i) c[i] = r[i];
}

VMR_HD void transpose(const float* a, float* c) {  // Matrix4Transpose (matrix4.go:100-108)
  float r[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) r[i * 4 + j] = a[j * 4 + i];
  for (int i = 0; i < 16; ++i) c[i] = r[i];
}

// The adjugate terms of Matrix4Inverse / Matrix4Det (matrix4.go:116-184):
// output element, then six (sign, a, b, c) triple products (m[a]*m[b])*m[c]
// summed left to right.  The table keeps the reference's term order, which
// fixes the rounding.
struct InvTerm {
  signed char s, a, b, c;
};
#ifdef __CUDACC__
__host__ __device__
#endif
inline void adjugate(const float* m, float* inv) {
  const signed char out[16] = {0, 4, 8, 12, 1, 5, 9, 13, 2, 6, 10, 14, 3, 7, 11, 15};
  const InvTerm t[16][6] = {
      {{1, 5, 10, 15}, {-1, 5, 11, 14}, {-1, 9, 6, 15}, {1, 9, 7, 14}, {1, 13, 6, 11}, {-1, 13, 7, 10}},
      {{-1, 4, 10, 15}, {1, 4, 11, 14}, {1, 8, 6, 15}, {-1, 8, 7, 14}, {-1, 12, 6, 11}, {1, 12, 7, 10}},
      {{1, 4, 9, 15}, {-1, 4, 11, 13}, {-1, 8, 5, 15}, {1, 8, 7, 13}, {1, 12, 5, 11}, {-1, 12, 7, 9}},
      {{-1, 4, 9, 14}, {1, 4, 10, 13}, {1, 8, 5, 14}, {-1, 8, 6, 13}, {-1, 12, 5, 10}, {1, 12, 6, 9}},
      {{-1, 1, 10, 15}, {1, 1, 11, 14}, {1, 9, 2, 15}, {-1, 9, 3, 14}, {-1, 13, 2, 11}, {1, 13, 3, 10}},
      {{1, 0, 10, 15}, {-1, 0, 11, 14}, {-1, 8, 2, 15}, {1, 8, 3, 14}, {1, 12, 2, 11}, {-1, 12, 3, 10}},
      {{-1, 0, 9, 15}, {1, 0, 11, 13}, {1, 8, 1, 15}, {-1, 8, 3, 13}, {-1, 12, 1, 11}, {1, 12, 3, 9}},
      {{1, 0, 9, 14}, {-1, 0, 10, 13}, {-1, 8, 1, 14}, {1, 8, 2, 13}, {1, 12, 1, 10}, {-1, 12, 2, 9}},
      {{1, 1, 6, 15}, {-1, 1, 7, 14}, {-1, 5, 2, 15}, {1, 5, 3, 14}, {1, 13, 2, 7}, {-1, 13, 3, 6}},
      {{-1, 0, 6, 15}, {1, 0, 7, 14}, {1, 4, 2, 15}, {-1, 4, 3, 14}, {-1, 12, 2, 7}, {1, 12, 3, 6}},
      {{1, 0, 5, 15}, {-1, 0, 7, 13}, {-1, 4, 1, 15}, {1, 4, 3, 13}, {1, 12, 1, 7}, {-1, 12, 3, 5}},
      {{-1, 0, 5, 14}, {1, 0, 6, 13}, {1, 4, 1, 14}, {-1, 4, 2, 13}, {-1, 12, 1, 6}, {1, 12, 2, 5}},
      {{-1, 1, 6, 11}, {1, 1, 7, 10}, {1, 5, 2, 11}, {-1, 5, 3, 10}, {-1, 9, 2, 7}, {1, 9, 3, 6}},
      {{1, 0, 6, 11}, {-1, 0, 7, 10}, {-1, 4, 2, 11}, {1, 4, 3, 10}, {1, 8, 2, 7}, {-1, 8, 3, 6}},
      {{-1, 0, 5, 11}, {1, 0, 7, 9}, {1, 4, 1, 11}, {-1, 4, 3, 9}, {-1, 8, 1, 7}, {1, 8, 3, 5}},
      {{1, 0, 5, 10}, {-1, 0, 6, 9}, {-1, 4, 1, 10}, {1, 4, 2, 9}, {1, 8, 1, 6}, {-1, 8, 2, 5}},
  };
  for (int e = 0; e < 16; ++e) {
    float acc = 0.0f;
    for (int k = 0; k < 6; ++k) {
      const InvTerm& q = t[e][k];
      const float v = (m[q.a] * m[q.b]) * m[q.c];
      acc = k == 0 ? (q.s > 0 ? v : -v) : (q.s > 0 ? acc + v : acc - v);
    }
    inv[out[e]] = acc;
  }
}

// Matrix4Det (matrix4.go:163-184).
VMR_HD float det(const float* m) {
  float inv[16];
  adjugate(m, inv);
  return ((m[0] * inv[0] + m[1] * inv[4]) + m[2] * inv[8]) + m[3] * inv[12];
}

// Matrix4Inverse (matrix4.go:116-160); a zero determinant gives the zero
// matrix and false.
VMR_HD bool inverse(const float* m, float* c) {
  float inv[16];
  adjugate(m, inv);
  float d = ((m[0] * inv[0] + m[1] * inv[4]) + m[2] * inv[8]) + m[3] * inv[12];
  for (int i = 0; i < 16; ++i) c[i] = 0.0f;
  if (d == 0.0f) return false;
  d = f_div(1.0f, d);
  for (int i = 0; i < 16; ++i) c[i] = inv[i] * d;
  return true;
}

VMR_HD void scale(float s, const float* m, float* x) {  // Matrix4Scale (matrix4.go:288-294)
  for (int i = 0; i < 16; ++i) x[i] = s * m[i];
}

// Matrix4PolarFactor (matrix4.go:343-363): Q <- (Q + Q^-T)/2 until no
// element decreases by more than 1e-6 (Matrix4Eq tests A-B > eps only), at
// most 10 times.
VMR_HD bool polar_factor(const float* m, float* q) {
  float Q[16], Qi[16], Qt[16], Qn[16];
  for (int i = 0; i < 16; ++i) Q[i] = m[i];
  for (int it = 0; it < 10; ++it) {
    if (!inverse(Q, Qi)) return false;
    transpose(Qi, Qt);
    for (int i = 0; i < 16; ++i) Qt[i] = Q[i] + Qt[i];  // Matrix4Add
    scale(0.5f, Qt, Qn);
    bool eq = true;
    for (int i = 0; i < 16; ++i)
      if (Qn[i] - Q[i] > 0.000001f) { eq = false; break; }
    if (eq) {
      for (int i = 0; i < 16; ++i) q[i] = Qn[i];
      return true;
    }
    for (int i = 0; i < 16; ++i) Q[i] = Qn[i];
  }
  return false;
}

// Matrix4ToQuat (math/quat.go:136-165).
VMR_HD void to_quat(const float* m, float* q) {
  const float m00 = m[0], m11 = m[5], m22 = m[10];
  const float tr = (m00 + m11) + m22;
  if (tr > 0.0f) {
    const float S = f_sqrt(tr + 1.0f) * 2.0f;
    q[3] = 0.25f * S;
    q[0] = f_div(m[6] - m[9], S);   // (Elt(2,1) - Elt(1,2)) / S
    q[1] = f_div(m[8] - m[2], S);   // (Elt(0,2) - Elt(2,0)) / S
    q[2] = f_div(m[1] - m[4], S);   // (Elt(1,0) - Elt(0,1)) / S
  } else if ((m00 > m11) && (m00 > m22)) {
    const float S = f_sqrt(((1.0f + m00) - m11) - m22) * 2.0f;
    q[3] = f_div(m[6] - m[9], S);
    q[0] = 0.25f * S;
    q[1] = f_div(m[4] + m[1], S);   // (Elt(0,1) + Elt(1,0)) / S
    q[2] = f_div(m[8] + m[2], S);   // (Elt(0,2) + Elt(2,0)) / S
  } else if (m11 > m22) {
    const float S = f_sqrt(((1.0f + m11) - m00) - m22) * 2.0f;
    q[3] = f_div(m[8] - m[2], S);
    q[0] = f_div(m[4] + m[1], S);
    q[1] = 0.25f * S;
    q[2] = f_div(m[9] + m[6], S);   // (Elt(1,2) + Elt(2,1)) / S
  } else {
    const float S = f_sqrt(((1.0f + m22) - m00) - m11) * 2.0f;
    q[3] = f_div(m[1] - m[4], S);
    q[0] = f_div(m[8] + m[2], S);
    q[1] = f_div(m[9] + m[6], S);
    q[2] = 0.25f * S;
  }
}

// QuatToMatrix4 (math/quat.go:81-104).
VMR_HD void quat_matrix(const float* q, float* m) {
  const float n = f_div(1.0f, f_sqrt(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]));
  const float X = q[0] * n, Y = q[1] * n, Z = q[2] * n, W = q[3] * n;
  for (int i = 0; i < 16; ++i) m[i] = 0.0f;
  m[0] = (1.0f - (2.0f * Y) * Y) - (2.0f * Z) * Z;
  m[4] = (2.0f * X) * Y - (2.0f * W) * Z;
  m[8] = (2.0f * X) * Z + (2.0f * W) * Y;
  m[1] = (2.0f * X) * Y + (2.0f * W) * Z;
  m[5] = (1.0f - (2.0f * X) * X) - (2.0f * Z) * Z;
  m[9] = (2.0f * Y) * Z - (2.0f * W) * X;
  m[2] = (2.0f * X) * Z - (2.0f * W) * Y;
  m[6] = (2.0f * Y) * Z + (2.0f * W) * X;
  m[10] = (1.0f - (2.0f * X) * X) - (2.0f * Y) * Y;
  m[15] = 1.0f;
}

// sign (math/octanormal.go:16-23): 1 for v >= 0, else -1 (NaN gives -1).
VMR_HD float sign_of(float v) { return v >= 0.0f ? 1.0f : -1.0f; }

// TransformDecompMatrix4 (math/animdecomp.go:20-62).
VMR_HD void decompose(const float* m_in, Decomp& d) {
  float m[16], neg[16], I[16], Q[16], Qt[16], S[16];
  for (int i = 0; i < 16; ++i) m[i] = m_in[i];
  const float sg = sign_of(det(m));
  for (int i = 0; i < 3; ++i) d.T[i] = m[12 + i];
  m[12] = 0.0f;
  m[13] = 0.0f;
  m[14] = 0.0f;
  identity(I);
  scale(-1.0f, I, neg);
  if (sg < 0.0f) mul(neg, m, m);
  if (!polar_factor(m, Q)) {
    d.R[0] = d.R[1] = d.R[2] = 0.0f;
    d.R[3] = 1.0f;
    identity(d.S);
    return;
  }
  transpose(Q, Qt);
  mul(Qt, m, S);
  to_quat(Q, d.R);
  if (sg < 0.0f) {
    mul(neg, S, d.S);
    d.S[15] = 1.0f;
  } else {
    for (int i = 0; i < 16; ++i) d.S[i] = S[i];
  }
}

// TransformDecompToMatrix4 (math/animdecomp.go:65-71): Translate(T) * (R * S).
VMR_HD void compose(const Decomp& d, float* m) {
  float R[16], RS[16], Tm[16];
  quat_matrix(d.R, R);
  mul(R, d.S, RS);
  identity(Tm);
  Tm[12] = d.T[0];
  Tm[13] = d.T[1];
  Tm[14] = d.T[2];
  mul(Tm, RS, m);
}

// QuatSlerp (math/quat.go:30-67).
VMR_HD void slerp(const float* qa, const float* qb, float t, float* qm) {
  const float c = ((qa[3] * qb[3] + qa[0] * qb[0]) + qa[1] * qb[1]) + qa[2] * qb[2];
  if (f_abs(c) >= 1.0f) {
    for (int i = 0; i < 4; ++i) qm[i] = qa[i];
    return;
  }
  const float half = f_acos(c);
  const float s = f_sqrt(1.0f - c * c);
  if (f_abs(s) < 0.001f) {
    for (int i = 0; i < 4; ++i) qm[i] = qa[i] * 0.5f + qb[i] * 0.5f;
    return;
  }
  const float ra = f_div(f_sin((1.0f - t) * half), s);
  const float rb = f_div(f_sin(t * half), s);
  for (int i = 0; i < 4; ++i) qm[i] = qa[i] * ra + qb[i] * rb;
}

// TransformDecompLerp (math/animdecomp.go:74-80): Vec3Lerp (math/vec3.go:52-58),
// QuatSlerp, Matrix4Lerp (math/matrix4.go:298-304).
VMR_HD void lerp(const Decomp& a, const Decomp& b, float t, Decomp& o) {
  for (int i = 0; i < 3; ++i) o.T[i] = (1.0f - t) * a.T[i] + t * b.T[i];
  slerp(a.R, b.R, t, o.R);
  for (int i = 0; i < 16; ++i) o.S[i] = (1.0f - t) * a.S[i] + t * b.S[i];
}

// The keyed transform at a time in [0, 1]: k = time*(n-1), frac =
// k - floor(k), keys floor(k) and ceil(k), blended by TransformDecompLerp
// and rebuilt.  One key: TransformSRTArray.TimeKey (instance.go:20-36,
// proc.go:20-36) uses it as it is (blend_one = false); Camera.ComputeRay
// (camera.go:223-236) still blends it with itself at frac 0 (blend_one =
// true), which is the identity except for a quaternion far from unit length.
// Returns false if the time falls outside the keys (the reference panics).
VMR_HD bool at_time(const Decomp* keys, unsigned n, float time, bool blend_one, float* m) {
  if (n <= 1 && !blend_one) {
    compose(keys[0], m);
    return true;
  }
  const float k = time * (float)(n - 1);
  const float fk = floorf(k);
  const float tf = k - fk;
  const int key = (int)fk, key2 = (int)ceilf(k);
  if (key < 0 || key2 < 0 || key >= (int)n || key2 >= (int)n) return false;
  Decomp d;
  lerp(keys[key], keys[key2], tf, d);
  compose(d, m);
  return true;
}

}  // namespace anim
}  // namespace vmr
