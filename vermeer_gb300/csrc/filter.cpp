// filter.cpp - pixel filters for filter importance sampling (host side).
//
// vmr_set_pixel_filter tabulates a GaussianFilter or AiryFilter
// (builtin/filter/gauss.go, airy.go) the way CreateSampler does
// (builtin/filter/filter.go:87-166) and uploads the two CDFs; the camera
// kernels warp each sample inside its pixel with them (warp_sample in
// shade_common.cuh, Sampler.WarpSample filter.go:40-80).  The tables are
// float64 and built in the reference's operation order (this file is
// compiled without contraction), so the device warps equal the reference's.
#include <cmath>
#include <vector>

#include "ctx.h"
#include "pixfilter.h"
#include "vmr.h"

namespace vmr {
namespace {

inline double sq(double x) { return x * x; }

// J1 by the rational approximation of Numerical Recipes (bessj1), the
// approximation the Airy filter is defined with (airy.go:33-66).
double j1_approx(double x) {
  const double ax = std::fabs(x);
  if (ax < 8.0) {
    const double y = x * x;
    const double num = x * (72362614232.0 + y * (-7895059235.0 + y * (242396853.1 + y * (-2972611.439 +
                                                                      y * (15704.48260 + y * (-30.16036606))))));
    const double den = 144725228442.0 + y * (2300535178.0 + y * (18583304.74 + y * (99447.43394 +
                                                                 y * (376.9991397 + y * 1.0))));
    return num / den;
  }
  const double z = 8.0 / ax, y = z * z, xx = ax - 2.356194491;
  const double p = 1.0 + y * (0.183105e-2 + y * (-0.3516396496e-4 + y * (0.2457520174e-5 + y * (-0.240337019e-6))));
  const double q = 0.04687499995 + y * (-0.2002690873e-3 + y * (0.8449199096e-5 + y * (-0.88228987e-6 +
                                                                y * 0.105787412e-6)));
  const double r = std::sqrt(0.636619772 / ax) * (std::cos(xx) * p - z * std::sin(xx) * q);
  return x < 0.0 ? -r : r;
}

// The filter functions with their circular cutoff at width/2.
double eval_filter(const vmr_pixel_filter& f, double x, double y) {
  const double r = std::sqrt(x * x + y * y);
  if (r > (double)(f.width / 2.0f)) return 0.0;
  const double pi = 3.141592653589793;
  if (f.kind == VMR_FILTER_GAUSSIAN) {
    // gauss.go:43-46, including the exponent (-(x^2+y^2)/2) * sigma^2
    const double s = 1.0 / std::sqrt((double)f.width);
    const double e = (-(x * x + y * y)) / 2 * sq(s);
    return (1 / (2 * pi * sq(s))) * std::exp(e);
  }
  // airy.go:86-92: lambda 550, f-stop 5.6, the 20000 scale
  const double v = (20000 / (double)f.width) * (pi * r) / (550.0 * 5.6);
  return (double)f.peak * sq(2 * j1_approx(v) / v);
}

}  // namespace

// Tables of one filter: out[0 .. n) = cdfV, out[n + j*n + i] = cdfVU[j][i].
bool build_filter_table(const vmr_pixel_filter& f, std::vector<double>& out) {
  const int n = f.res;
  const double w = (double)f.width;
  std::vector<double> val((size_t)n * n);  // val[j + i*n] = f(u_j, v_i), grid accumulated
  const double du = w / (double)(n - 1);
  double F = 0.0, u = -w / 2;
  for (int j = 0; j < n; ++j) {
    const double dv = w / (double)(n - 1);
    double v = -w / 2;
    for (int i = 0; i < n; ++i) {
      const double x = eval_filter(f, u, v);
      val[(size_t)j + (size_t)i * n] = x;
      F += x;
      v += dv;
    }
    u += du;
  }
  out.assign((size_t)n + (size_t)n * n, 0.0);
  std::vector<double> marg(n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) marg[j] += val[(size_t)j + (size_t)i * n] / F;
  double acc = 0.0;
  for (int j = 0; j < n; ++j) {
    acc += marg[j];
    out[j] = acc;
  }
  for (int j = 0; j < n; ++j) {
    double row = 0.0;
    for (int i = 0; i < n; ++i) {
      row += (val[(size_t)j + (size_t)i * n] / F) / marg[j];
      out[(size_t)n + (size_t)j * n + i] = row;
    }
  }
  return true;
}

// The node defaults for unset fields; false (with why) if f is unusable.
bool resolve_filter(vmr_pixel_filter& f, const char** why) {
  if (f.kind != VMR_FILTER_GAUSSIAN && f.kind != VMR_FILTER_AIRY) {
    *why = "unknown pixel filter kind";
    return false;
  }
  if (f.res <= 0) f.res = f.kind == VMR_FILTER_GAUSSIAN ? 17 : 49;
  if (!(f.width > 0.0f)) f.width = f.kind == VMR_FILTER_GAUSSIAN ? 2.0f : 6.0f;
  if (f.kind == VMR_FILTER_AIRY && !(f.peak > 0.0f)) f.peak = 4.0f;
  if (f.res < 2 || f.res > 1024 || !std::isfinite(f.width)) {
    *why = "pixel filter res must be in [2, 1024] and width finite";
    return false;
  }
  return true;
}

}  // namespace vmr

extern "C" int vmr_pixel_filter_warp(const vmr_pixel_filter* filter, const double* r0, const double* r1, size_t n,
                                     double* u, double* v) {
  if (!filter || (n && (!r0 || !r1 || !u || !v))) return VMR_ERR_INVALID;
  vmr_pixel_filter f = *filter;
  const char* why = nullptr;
  if (f.kind == VMR_FILTER_BOX) {
    for (size_t i = 0; i < n; ++i) u[i] = v[i] = 0.0;
    return VMR_OK;
  }
  if (!vmr::resolve_filter(f, &why)) return VMR_ERR_INVALID;
  std::vector<double> t;
  vmr::build_filter_table(f, t);
  const vmr::PixFilter pf{t.data(), (uint32_t)f.res, (double)f.width};
  for (size_t i = 0; i < n; ++i) vmr::warp_sample(pf, r0[i], r1[i], u[i], v[i]);
  return VMR_OK;
}

extern "C" int vmr_set_pixel_filter(vmr_ctx* ctx, const vmr_pixel_filter* filter) {
  if (!ctx || !filter) return VMR_ERR_INVALID;
  vmr_pixel_filter f = *filter;
  vmr::RenderState& R = ctx->render;
  if (f.kind == VMR_FILTER_BOX) {
    R.filter_n = 0;
    return VMR_OK;
  }
  const char* why = nullptr;
  if (!vmr::resolve_filter(f, &why)) {
    ctx->err = why;
    return VMR_ERR_INVALID;
  }
  std::vector<double> t;
  vmr::build_filter_table(f, t);
  if (ctx->device >= 0) {
    cudaSetDevice(ctx->device);
    cudaError_t e = R.filter.ensure(t.size() * sizeof(double));
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(R.filter.p, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
      ctx->err = cudaGetErrorString(e);
      return e == cudaErrorMemoryAllocation ? VMR_ERR_OOM : VMR_ERR_CUDA;
    }
  }
  R.filter_host = t;
  R.filter_n = (uint32_t)f.res;
  R.filter_w = (double)f.width;
  return VMR_OK;
}
