// orc_filter.cpp - pixel filters for filter importance sampling.
// TEST INFRASTRUCTURE ONLY (see orc.h): the checker for libvmr's filter
// tables and warps, never part of the product path.
//
// Restates builtin/filter/filter.go (Sampler, CreateSampler, WarpSample),
// builtin/filter/gauss.go (GaussianFilter.PreRender) and
// builtin/filter/airy.go (BesselJ1, AiryFilter.PreRender) in float64 with
// the reference's operation order, including its quirks:
//  * the Gaussian's exponent is (-(x^2+y^2)/2) * sigma^2 (Go precedence,
//    gauss.go:44), sigma = 1/sqrt(width);
//  * the grid coordinates are accumulated (u += du, v += dv), not computed
//    from the index (filter.go:100-113);
//  * WarpSample's first-cell branch uses du / w (filter.go:51-52,66-67),
//    u keeps 0 when r0 is not below any CDF entry, and (0, 0) is returned
//    when r1 is not below any entry of its row (filter.go:79);
//  * the Airy filter at its default resolution samples q = 0 exactly, where
//    2 J1(v)/v is 0/0: the NaN spreads through the normalisation, every
//    comparison fails and every warp returns (0, 0).
#include <cmath>
#include <cstddef>
#include <vector>

#include "orc.h"
#include "orc_internal.h"

namespace orc_internal {
namespace {

double sqr(double x) { return x * x; }

// Numerical Recipes' rational approximation of J1 (airy.go:33-66).
double bessel_j1(double x) {
  const double ax = std::fabs(x);
  if (ax < 8.0) {
    const double y = x * x;
    const double a1 = x * (72362614232.0 +
                           y * (-7895059235.0 + y * (242396853.1 + y * (-2972611.439 + y * (15704.48260 + y * (-30.16036606))))));
    const double a2 = 144725228442.0 + y * (2300535178.0 + y * (18583304.74 + y * (99447.43394 + y * (376.9991397 + y * 1.0))));
    return a1 / a2;
  }
  const double z = 8.0 / ax;
  const double y = z * z;
  const double xx = ax - 2.356194491;
  const double a1 = 1.0 + y * (0.183105e-2 + y * (-0.3516396496e-4 + y * (0.2457520174e-5 + y * (-0.240337019e-6))));
  const double a2 =
      0.04687499995 + y * (-0.2002690873e-3 + y * (0.8449199096e-5 + y * (-0.88228987e-6 + y * 0.105787412e-6)));
  double ans = std::sqrt(0.636619772 / ax) * (std::cos(xx) * a1 - z * std::sin(xx) * a2);
  if (x < 0.0) ans = -ans;
  return ans;
}

double filter_value(const orc_pixel_filter& f, double x, double y) {
  const double q = std::sqrt(x * x + y * y);
  if (q > (double)(f.width / 2.0f)) return 0.0;  // the cutoff (gauss.go:38-41, airy.go:79-82)
  if (f.kind == 1) {
    const double sigma = 1.0 / std::sqrt((double)f.width);
    const double pi = 3.141592653589793;
    const double t = (-(x * x + y * y)) / 2 * sqr(sigma);
    return (1 / (2 * pi * sqr(sigma))) * std::exp(t);
  }
  const double lambda = 550.0, N = 5.6;  // airy.go:84-85
  const double pi = 3.141592653589793;
  const double v = (20000 / (double)f.width) * (pi * q) / (lambda * N);
  return (double)f.peak * sqr(2 * bessel_j1(v) / v);
}

}  // namespace

// CreateSampler (filter.go:87-166).
FilterTable make_filter(const orc_pixel_filter& f) {
  FilterTable t;
  if (f.kind != 1 && f.kind != 2) return t;
  const int n = f.res;
  const double w = (double)f.width;
  t.n = n;
  t.w = w;
  std::vector<double> filter((size_t)n * n);
  const double du = w / (double)(n - 1);
  double u = -w / 2;
  double F = 0;
  for (int j = 0; j < n; ++j) {
    const double dv = w / (double)(n - 1);
    double v = -w / 2;
    for (int i = 0; i < n; ++i) {
      const double fuv = filter_value(f, u, v);
      filter[(size_t)j + (size_t)i * n] = fuv;
      F += fuv;
      v += dv;
    }
    u += du;
  }
  std::vector<double> pdf((size_t)n * n), pV(n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) pdf[(size_t)j * n + i] = filter[(size_t)j + (size_t)i * n] / F;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) pV[j] += pdf[(size_t)j * n + i];
  t.cdfV.assign(n, 0.0);
  t.cdfVU.assign((size_t)n * n, 0.0);
  double p = 0;
  for (int i = 0; i < n; ++i) {
    p += pV[i];
    t.cdfV[i] = p;
  }
  for (int j = 0; j < n; ++j) {
    double q = 0;
    for (int i = 0; i < n; ++i) {
      q += pdf[(size_t)j * n + i] / pV[j];
      t.cdfVU[(size_t)j * n + i] = q;
    }
  }
  return t;
}

// Sampler.WarpSample (filter.go:40-80).
void warp_sample(const FilterTable& t, double r0, double r1, double& u, double& v) {
  u = 0.0;
  v = 0.0;
  const int n = t.n;
  const double w = t.w;
  int uI = -1;
  for (int i = 0; i < n; ++i) {
    uI = i;
    if (r0 < t.cdfV[i]) {
      if (i == 0) {
        const double du = r0 / t.cdfV[i];
        u = (-w / 2) + (du / w);
      } else {
        const double du = (r0 - t.cdfV[i - 1]) / (t.cdfV[i] - t.cdfV[i - 1]);
        u = (-w / 2) + w * ((double)i + du) / (double)(n - 1);
      }
      break;
    }
  }
  const double* row = t.cdfVU.data() + (size_t)uI * n;
  for (int i = 0; i < n; ++i) {
    if (r1 < row[i]) {
      if (i == 0) {
        const double dv = r1 / row[i];
        v = (-w / 2) + (dv / w);
      } else {
        const double dv = (r1 - row[i - 1]) / (row[i] - row[i - 1]);
        v = (-w / 2) + w * ((double)i + dv) / (double)(n - 1);
      }
      return;
    }
  }
  u = 0.0;
  v = 0.0;
}

}  // namespace orc_internal

extern "C" {

int orc_filter_warp(const orc_pixel_filter* f, const double* r0, const double* r1, size_t n, double* u, double* v) {
  if (!f || f->res < 2 || (n && (!r0 || !r1 || !u || !v))) return -1;
  const orc_internal::FilterTable t = orc_internal::make_filter(*f);
  if (t.n == 0) return -1;
  for (size_t i = 0; i < n; ++i) orc_internal::warp_sample(t, r0[i], r1[i], u[i], v[i]);
  return 0;
}

int orc_filter_tables(const orc_pixel_filter* f, double* cdfV, double* cdfVU) {
  if (!f || f->res < 2 || !cdfV || !cdfVU) return -1;
  const orc_internal::FilterTable t = orc_internal::make_filter(*f);
  if (t.n == 0) return -1;
  for (int i = 0; i < t.n; ++i) cdfV[i] = t.cdfV[i];
  for (size_t i = 0; i < t.cdfVU.size(); ++i) cdfVU[i] = t.cdfVU[i];
  return 0;
}

}  // extern "C"
