// orc_anim.cpp - CPU oracle of the reference's decomposed transforms.
//
// TEST INFRASTRUCTURE ONLY (see orc.h).  Restates math/animdecomp.go
// (TransformDecompMatrix4 :20-62, TransformDecompToMatrix4 :65-71,
// TransformDecompLerp :74-80), the matrix helpers it calls in
// math/matrix4.go (Matrix4Mul :87-97, Matrix4Transpose :100-108,
// Matrix4Inverse :116-160, Matrix4Det :163-184, Matrix4Scale :288-294,
// Matrix4Lerp :298-304, Matrix4Eq :326-336, Matrix4PolarFactor :343-363),
// math/quat.go (QuatSlerp :30-67, QuatToMatrix4 :81-104, Matrix4ToQuat
// :136-165) and Vec3Lerp (math/vec3.go:52-58), in float32 with every
// product rounded separately (built with -ffp-contract=off).  Acos and Sin
// are float64 and rounded to float32 (math/sincos.go).
#include <cmath>
#include <cstring>

#include "orc.h"
#include "orc_internal.h"

namespace orc_internal {

namespace {

typedef float M4[16];  // column-major: (row i, column j) at [j*4+i]

float elt(const M4 m, int i, int j) { return m[j * 4 + i]; }

void m4_copy(M4 d, const M4 s) { std::memcpy(d, s, sizeof(M4)); }

void m4_identity(M4 m) {
  for (int i = 0; i < 16; ++i) m[i] = 0.0f;
  m[0] = m[5] = m[10] = m[15] = 1.0f;
}

void m4_mul(const M4 a, const M4 b, M4 out) {
  M4 c;
  for (int i = 0; i < 16; ++i) c[i] = 0.0f;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      for (int k = 0; k < 4; ++k) c[(j * 4) + i] += a[(k * 4) + i] * b[(j * 4) + k];
  m4_copy(out, c);
}

void m4_transpose(const M4 a, M4 out) {
  M4 c;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) c[(i * 4) + j] = a[(j * 4) + i];
  m4_copy(out, c);
}

void m4_scale(float s, const M4 m, M4 x) {
  for (int i = 0; i < 16; ++i) x[i] = s * m[i];
}

// The sixteen cofactor expressions of Matrix4Inverse / Matrix4Det, written
// out as the reference writes them (Go evaluates a*b*c as (a*b)*c and sums
// left to right).
void cofactors(const M4 m, M4 inv) {
  inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] +
           m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
  inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] -
           m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
  inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] +
           m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
  inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] -
            m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
  inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] -
           m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
  inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] +
           m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
  inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] -
           m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
  inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] +
            m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
  inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] +
           m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
  inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] -
           m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
  inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] +
            m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
  inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] -
            m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
  inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] -
           m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
  inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] +
           m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
  inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] -
            m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
  inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] +
            m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
}

float m4_det(const M4 m) {
  M4 inv;
  cofactors(m, inv);
  return m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
}

bool m4_inverse(const M4 m, M4 c) {
  M4 inv;
  cofactors(m, inv);
  for (int i = 0; i < 16; ++i) c[i] = 0.0f;
  float det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  if (det == 0.0f) return false;
  det = 1.0f / det;
  for (int i = 0; i < 16; ++i) c[i] = inv[i] * det;
  return true;
}

bool m4_eq(const M4 A, const M4 B, float eps) {
  for (int i = 0; i < 16; ++i)
    if (A[i] - B[i] > eps) return false;
  return true;
}

bool polar_factor(const M4 m, M4 out) {
  M4 Q;
  m4_copy(Q, m);
  for (int i = 0; i < 10; ++i) {
    M4 Qinv, QinvT, sum, Qnew;
    if (!m4_inverse(Q, Qinv)) return false;
    m4_transpose(Qinv, QinvT);
    for (int k = 0; k < 16; ++k) sum[k] = Q[k] + QinvT[k];
    m4_scale(0.5f, sum, Qnew);
    if (m4_eq(Qnew, Q, 0.000001f)) {
      m4_copy(out, Qnew);
      return true;
    }
    m4_copy(Q, Qnew);
  }
  return false;
}

float go_abs(float x) {  // math.Abs (math/abs.go)
  if (x < 0) return -x;
  if (x == 0) return 0;
  return x;
}

void matrix_to_quat(const M4 m, float q[4]) {  // q = X, Y, Z, W
  float tr = elt(m, 0, 0) + elt(m, 1, 1) + elt(m, 2, 2);
  if (tr > 0.0f) {
    float S = std::sqrt(tr + 1.0f) * 2;
    q[3] = 0.25f * S;
    q[0] = (elt(m, 2, 1) - elt(m, 1, 2)) / S;
    q[1] = (elt(m, 0, 2) - elt(m, 2, 0)) / S;
    q[2] = (elt(m, 1, 0) - elt(m, 0, 1)) / S;
  } else if ((elt(m, 0, 0) > elt(m, 1, 1)) && (elt(m, 0, 0) > elt(m, 2, 2))) {
    float S = std::sqrt(1.0f + elt(m, 0, 0) - elt(m, 1, 1) - elt(m, 2, 2)) * 2;
    q[3] = (elt(m, 2, 1) - elt(m, 1, 2)) / S;
    q[0] = 0.25f * S;
    q[1] = (elt(m, 0, 1) + elt(m, 1, 0)) / S;
    q[2] = (elt(m, 0, 2) + elt(m, 2, 0)) / S;
  } else if (elt(m, 1, 1) > elt(m, 2, 2)) {
    float S = std::sqrt(1.0f + elt(m, 1, 1) - elt(m, 0, 0) - elt(m, 2, 2)) * 2;
    q[3] = (elt(m, 0, 2) - elt(m, 2, 0)) / S;
    q[0] = (elt(m, 0, 1) + elt(m, 1, 0)) / S;
    q[1] = 0.25f * S;
    q[2] = (elt(m, 1, 2) + elt(m, 2, 1)) / S;
  } else {
    float S = std::sqrt(1.0f + elt(m, 2, 2) - elt(m, 0, 0) - elt(m, 1, 1)) * 2;
    q[3] = (elt(m, 1, 0) - elt(m, 0, 1)) / S;
    q[0] = (elt(m, 0, 2) + elt(m, 2, 0)) / S;
    q[1] = (elt(m, 1, 2) + elt(m, 2, 1)) / S;
    q[2] = 0.25f * S;
  }
}

void quat_to_matrix(const float q[4], M4 m) {
  const float n = 1.0f / std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  const float qX = q[0] * n, qY = q[1] * n, qZ = q[2] * n, qW = q[3] * n;
  for (int i = 0; i < 16; ++i) m[i] = 0.0f;
  auto set = [&](int i, int j, float v) { m[j * 4 + i] = v; };
  set(0, 0, 1 - 2 * qY * qY - 2 * qZ * qZ);
  set(0, 1, 2 * qX * qY - 2 * qW * qZ);
  set(0, 2, 2 * qX * qZ + 2 * qW * qY);
  set(1, 0, 2 * qX * qY + 2 * qW * qZ);
  set(1, 1, 1 - 2 * qX * qX - 2 * qZ * qZ);
  set(1, 2, 2 * qY * qZ - 2 * qW * qX);
  set(2, 0, 2 * qX * qZ - 2 * qW * qY);
  set(2, 1, 2 * qY * qZ + 2 * qW * qX);
  set(2, 2, 1 - 2 * qX * qX - 2 * qY * qY);
  set(3, 3, 1.0f);
}

void quat_slerp(const float qa[4], const float qb[4], float t, float qm[4]) {
  const float cosHalfTheta = qa[3] * qb[3] + qa[0] * qb[0] + qa[1] * qb[1] + qa[2] * qb[2];
  if (go_abs(cosHalfTheta) >= 1.0f) {
    for (int i = 0; i < 4; ++i) qm[i] = qa[i];
    return;
  }
  const float halfTheta = (float)std::acos((double)cosHalfTheta);
  const float sinHalfTheta = std::sqrt(1.0f - cosHalfTheta * cosHalfTheta);
  if (go_abs(sinHalfTheta) < 0.001f) {
    for (int i = 0; i < 4; ++i) qm[i] = qa[i] * 0.5f + qb[i] * 0.5f;
    return;
  }
  const float ratioA = (float)std::sin((double)((1 - t) * halfTheta)) / sinHalfTheta;
  const float ratioB = (float)std::sin((double)(t * halfTheta)) / sinHalfTheta;
  for (int i = 0; i < 4; ++i) qm[i] = qa[i] * ratioA + qb[i] * ratioB;
}

}  // namespace

void decomp_matrix(const float* m_in, Decomp& d) {
  M4 m;
  m4_copy(m, m_in);
  const float sign = m4_det(m) >= 0.0f ? 1.0f : -1.0f;  // sign (math/octanormal.go:16-23)
  for (int i = 0; i < 3; ++i) d.T[i] = elt(m, i, 3);
  m[12] = 0;
  m[13] = 0;
  m[14] = 0;
  M4 I, negI;
  m4_identity(I);
  m4_scale(-1, I, negI);
  if (sign < 0.0f) m4_mul(negI, m, m);
  M4 Q;
  if (!polar_factor(m, Q)) {
    d.R[0] = d.R[1] = d.R[2] = 0;
    d.R[3] = 1;
    m4_identity(d.S);
    return;
  }
  M4 QT, S;
  m4_transpose(Q, QT);
  m4_mul(QT, m, S);
  matrix_to_quat(Q, d.R);
  if (sign < 0.0f) {
    m4_mul(negI, S, d.S);
    d.S[15] = 1;
  } else {
    m4_copy(d.S, S);
  }
}

void decomp_to_matrix(const Decomp& d, float* out) {
  M4 Tm, R, RS;
  m4_identity(Tm);
  Tm[12] = d.T[0];
  Tm[13] = d.T[1];
  Tm[14] = d.T[2];
  quat_to_matrix(d.R, R);
  m4_mul(R, d.S, RS);
  m4_mul(Tm, RS, out);
}

void decomp_lerp(const Decomp& a, const Decomp& b, float t, Decomp& o) {
  for (int i = 0; i < 3; ++i) o.T[i] = (1.0f - t) * a.T[i] + t * b.T[i];
  quat_slerp(a.R, b.R, t, o.R);
  for (int i = 0; i < 16; ++i) o.S[i] = (1.0f - t) * a.S[i] + t * b.S[i];
}

bool decomp_at(const std::vector<Decomp>& keys, float time, bool blend_one, float* m) {
  if (keys.empty()) return false;
  if (keys.size() == 1 && !blend_one) {
    decomp_to_matrix(keys[0], m);
    return true;
  }
  const float k = time * (float)(keys.size() - 1);
  const float t = k - std::floor(k);
  const int key = (int)std::floor(k), key2 = (int)std::ceil(k);
  if (key < 0 || key2 < 0 || key >= (int)keys.size() || key2 >= (int)keys.size()) return false;
  Decomp d;
  decomp_lerp(keys[key], keys[key2], t, d);
  decomp_to_matrix(d, m);
  return true;
}

bool matrix_inverse(const float* m, float* c) { return m4_inverse(m, c); }

}  // namespace orc_internal

extern "C" {

void orc_decompose(const float* m, float* trs23) {
  orc_internal::Decomp d;
  orc_internal::decomp_matrix(m, d);
  std::memcpy(trs23, d.T, 3 * 4);
  std::memcpy(trs23 + 3, d.R, 4 * 4);
  std::memcpy(trs23 + 7, d.S, 16 * 4);
}

int orc_keyed_matrix(const float* keys16, uint32_t n, float time, int blend_one, float* out16) {
  std::vector<orc_internal::Decomp> ks(n);
  for (uint32_t i = 0; i < n; ++i) orc_internal::decomp_matrix(keys16 + 16 * i, ks[i]);
  return orc_internal::decomp_at(ks, time, blend_one != 0, out16) ? 0 : -1;
}

}  // extern "C"
