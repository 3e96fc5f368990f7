// orc_mlp.cpp - CPU oracle of the path-guiding network (no reference
// counterpart; the project's own design).
//
// TEST INFRASTRUCTURE ONLY (see orc.h).
//
// Network: 80 inputs -> 4 hidden layers of 64 (ReLU, no biases; input 78 is
// the constant 1) -> 41 outputs = 8 von Mises-Fisher lobes x (direction 3,
// concentration 1, mixture logit 1), then the selection logit s.  Weights:
// W0 [64][80], W1..W3 [64][64], W4 [41][64], row-major, concatenated (20,032
// floats).
//
// Inputs of a path vertex: the hit point p normalised to the scene bounds,
// q = (p - lo)/(hi - lo); for each axis c and frequency f = 0..11,
// sin(2^f pi q_c) and cos(2^f pi q_c) at 24c + 2f (+0 sin, +1 cos); the
// shading normal at 72..74; the direction toward the previous vertex at
// 75..77; 1 at 78; 0 at 79.
//
// Lobe k: mu = normalize(o[5k..5k+2]), kappa = exp(o[5k+3]) with the
// exponent clamped to [-4.6, 6.9] (kappa in [0.01, 992]), pi = softmax over
// o[5k+4]; vMF density kappa / (2 pi (1 - exp(-2 kappa))) * exp(kappa
// (mu.w - 1)).  The vertex samples the guide with probability alpha = amax *
// sigmoid(o[40]) and its BSDF otherwise, so its sampling density is q =
// alpha p_guide + (1 - alpha) p_bsdf.
//
// Training, per record (omega_i: a direction the tracer sampled at the
// vertex; weight_i: its incident radiance (luminance) x |cos| over the
// density it was sampled with): the lobes descend -weight_i * log
// p_guide(omega_i), the guide's own fit to the product; with the BSDF's
// density p_bsdf(omega_i) recorded, the selection logit descends -weight_i *
// log q(omega_i) with p_guide held fixed (the best mixing weight for the
// current guide; the lobes do not see alpha, so a small alpha does not stop
// them from learning).  The reported loss is the sum of -weight_i * log q
// (of -weight_i * log p_guide without BSDF densities).  The gradients are
// analytic (the selection, the mixture, the lobe parameters, back through
// the ReLU layers).
//
// Precision modes: 64 and 32 compute everything in that type; 16 mirrors
// the CUDA kernels' tensor-core arithmetic: weights, layer inputs and
// back-propagated deltas rounded to bfloat16 (round to nearest even), products
// accumulated in float32.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "orc.h"

namespace {

const int kIn = 80, kHid = 64, kOut = 41, kLobes = 8;
const int kLayerIn[5] = {80, 64, 64, 64, 64};
const int kLayerOut[5] = {64, 64, 64, 64, 41};
const int kOffset[5] = {0, 5120, 9216, 13312, 17408};

float bf16(float x) {  // round to nearest even, as __float2bfloat16_rn
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;  // inf / nan unchanged
  const uint32_t lsb = (u >> 16) & 1u;
  u += 0x7fffu + lsb;
  u &= 0xffff0000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

template <class T>
T rnd_in(T v, int mode) {
  return mode == 16 ? (T)bf16((float)v) : v;
}

void features(const float* p, const float* n, const float* wo, const float* lo, const float* hi, double* f) {
  for (int c = 0; c < 3; ++c) {
    const double q = ((double)p[c] - (double)lo[c]) / ((double)hi[c] - (double)lo[c]);
    for (int k = 0; k < 12; ++k) {
      const double a = std::ldexp(q, k);  // 2^k q
      f[24 * c + 2 * k] = std::sin(M_PI * a);
      f[24 * c + 2 * k + 1] = std::cos(M_PI * a);
    }
  }
  for (int c = 0; c < 3; ++c) {
    f[72 + c] = n[c];
    f[75 + c] = wo[c];
  }
  f[78] = 1.0;
  f[79] = 0.0;
}

// Forward pass of one row; acts[l] = input of layer l (acts[0] = features).
template <class T>
void forward(const float* W, const double* feat, int mode, std::vector<std::vector<T>>& acts, T* out) {
  acts.assign(5, {});
  acts[0].resize(kIn);
  for (int i = 0; i < kIn; ++i) acts[0][i] = rnd_in((T)feat[i], mode);
  for (int l = 0; l < 5; ++l) {
    const int ni = kLayerIn[l], no = kLayerOut[l];
    std::vector<T> z(no);
    for (int o = 0; o < no; ++o) {
      T s = 0;
      for (int i = 0; i < ni; ++i) s += rnd_in((T)W[kOffset[l] + o * ni + i], mode) * acts[l][i];
      z[o] = s;
    }
    if (l < 4) {
      acts[l + 1].resize(no);
      for (int o = 0; o < no; ++o) acts[l + 1][o] = rnd_in(z[o] > T(0) ? z[o] : T(0), mode);
    } else {
      for (int o = 0; o < no; ++o) out[o] = z[o];
    }
  }
}

const double kLogKapMin = -4.6, kLogKapMax = 6.9;  // kappa in [0.01, 992]

template <class T>
struct Lobes {
  T mu[kLobes][3], rn[kLobes], kappa[kLobes], pi[kLobes];
  bool clamped[kLobes];
};

template <class T>
void lobes(const T* o, Lobes<T>& L) {
  T mx = -INFINITY;
  for (int k = 0; k < kLobes; ++k) mx = std::max(mx, o[5 * k + 4]);
  T z = 0;
  for (int k = 0; k < kLobes; ++k) {
    const T* r = o + 5 * k;
    T n = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (n < T(1e-6)) n = T(1e-6);
    L.rn[k] = n;
    for (int c = 0; c < 3; ++c) L.mu[k][c] = r[c] / n;
    const T s = r[3];
    L.clamped[k] = s < T(kLogKapMin) || s > T(kLogKapMax);
    L.kappa[k] = std::exp(std::min(std::max(s, T(kLogKapMin)), T(kLogKapMax)));
    L.pi[k] = std::exp(r[4] - mx);
    z += L.pi[k];
  }
  for (int k = 0; k < kLobes; ++k) L.pi[k] /= z;
}

// vMF density of lobe k at w (unit).
template <class T>
T vmf(const Lobes<T>& L, int k, const T* w) {
  const T kap = L.kappa[k];
  const T d = L.mu[k][0] * w[0] + L.mu[k][1] * w[1] + L.mu[k][2] * w[2];
  const T c = kap / (T(2 * M_PI) * (-std::expm1(T(-2) * kap)));
  return c * std::exp(kap * (d - T(1)));
}

template <class T>
T mixture_pdf(const Lobes<T>& L, const T* w) {
  T p = 0;
  for (int k = 0; k < kLobes; ++k) p += L.pi[k] * vmf(L, k, w);
  return p;
}

// Gradient at the outputs: lobes from -weight * log p_guide, the selection
// logit from -weight * log q with p_guide fixed (pb < 0: no BSDF density,
// no selection gradient); loss = -weight * log q (or log p_guide).
template <class T>
void loss_grad_out(const T* o, const T* w, T weight, T pb, T amax, T* g, T& loss) {
  Lobes<T> L;
  lobes(o, L);
  T v[kLobes];
  T p = 0;
  for (int k = 0; k < kLobes; ++k) {
    v[k] = vmf(L, k, w);
    p += L.pi[k] * v[k];
  }
  loss = -weight * std::log(p);
  g[40] = T(0);
  if (pb >= T(0)) {
    const T sg = T(1) / (T(1) + std::exp(-o[40]));
    const T a = amax * sg;
    const T q = a * p + (T(1) - a) * pb;
    g[40] = -weight * (p - pb) / q * (amax * sg * (T(1) - sg));
    loss = -weight * std::log(q);
  }
  for (int k = 0; k < kLobes; ++k) {
    const T r = L.pi[k] * v[k] / p;  // responsibility of lobe k
    const T d = L.mu[k][0] * w[0] + L.mu[k][1] * w[1] + L.mu[k][2] * w[2];
    const T kap = L.kappa[k];
    g[5 * k + 4] = -weight * (r - L.pi[k]);
    // d log v / d kappa, times d kappa / d s = kappa
    const T dlogv_dk = T(1) / kap - T(2) / std::expm1(T(2) * kap) + (d - T(1));
    g[5 * k + 3] = L.clamped[k] ? T(0) : -weight * r * dlogv_dk * kap;
    for (int c = 0; c < 3; ++c) g[5 * k + c] = -weight * r * kap * (w[c] - d * L.mu[k][c]) / L.rn[k];
  }
}

template <class T>
double loss_and_grad(const float* W, const double* feats, const float* omega, const float* weight, const float* pb,
                     double amax, int n, int mode, double* gW) {
  const int nw = kOffset[4] + kOut * 64;
  std::vector<double> acc(nw, 0.0);
  double total = 0;
  std::vector<std::vector<T>> acts;
  for (int i = 0; i < n; ++i) {
    T out[kOut], go[kOut], loss;
    forward<T>(W, feats + (size_t)i * kIn, mode, acts, out);
    const T w[3] = {(T)omega[3 * i], (T)omega[3 * i + 1], (T)omega[3 * i + 2]};
    loss_grad_out<T>(out, w, (T)weight[i], pb ? (T)pb[i] : T(-1), (T)amax, go, loss);
    total += (double)loss;
    // back-propagate: delta of layer l's output
    std::vector<T> delta(go, go + kOut);
    for (int k = 0; k < kOut; ++k) delta[k] = rnd_in(delta[k], mode);
    for (int l = 4; l >= 0; --l) {
      const int ni = kLayerIn[l], no = kLayerOut[l];
      for (int o = 0; o < no; ++o)
        for (int j = 0; j < ni; ++j) acc[kOffset[l] + o * ni + j] += (double)(delta[o] * acts[l][j]);
      if (l == 0) break;
      std::vector<T> prev(ni);
      for (int j = 0; j < ni; ++j) {
        T s = 0;
        for (int o = 0; o < no; ++o) s += rnd_in((T)W[kOffset[l] + o * ni + j], mode) * delta[o];
        prev[j] = acts[l][j] > T(0) ? rnd_in(s, mode) : T(0);  // ReLU' of the layer input
      }
      delta.swap(prev);
    }
  }
  for (int k = 0; k < nw; ++k) gW[k] = acc[k];
  return total;
}

}  // namespace

extern "C" {

int orc_guide_n_weights(void) { return kOffset[4] + kOut * 64; }

void orc_guide_features(const float* pos, const float* nrm, const float* wo, const float* lo, const float* hi, int n,
                        double* feat) {
  for (int i = 0; i < n; ++i) features(pos + 3 * i, nrm + 3 * i, wo + 3 * i, lo, hi, feat + (size_t)i * kIn);
}

void orc_guide_forward(const float* W, const double* feat, int n, int precision, double* out) {
  std::vector<std::vector<double>> ad;
  std::vector<std::vector<float>> af;
  for (int i = 0; i < n; ++i) {
    if (precision == 64) {
      double o[kOut];
      forward<double>(W, feat + (size_t)i * kIn, 64, ad, o);
      for (int k = 0; k < kOut; ++k) out[(size_t)i * kOut + k] = o[k];
    } else {
      float o[kOut];
      forward<float>(W, feat + (size_t)i * kIn, precision, af, o);
      for (int k = 0; k < kOut; ++k) out[(size_t)i * kOut + k] = o[k];
    }
  }
}

double orc_guide_pdf(const double* out41, const double* w) {
  Lobes<double> L;
  lobes(out41, L);
  return mixture_pdf(L, w);
}

void orc_guide_out_grad(const double* out41, const double* w, double weight, double pb, double amax, double* g41,
                        double* loss) {
  loss_grad_out<double>(out41, w, weight, pb, amax, g41, *loss);
}

double orc_guide_loss_grad(const float* W, const double* feat, const float* omega, const float* weight,
                           const float* bsdf_pdf, double amax, int n, int precision, double* gW) {
  if (precision == 64) return loss_and_grad<double>(W, feat, omega, weight, bsdf_pdf, amax, n, 64, gW);
  return loss_and_grad<float>(W, feat, omega, weight, bsdf_pdf, amax, n, precision, gW);
}

}  // extern "C"
