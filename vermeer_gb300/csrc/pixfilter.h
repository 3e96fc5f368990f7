// pixfilter.h - Sampler.WarpSample (builtin/filter/filter.go:40-80) over
// the tables vmr_set_pixel_filter builds, shared by the camera kernels and
// the host entry point vmr_pixel_filter_warp.
//
// Float64 throughout, in the reference's operation order, including its
// quirks: the first cell's lerp is du / w, the lerp runs over
// (i + du) / (n - 1) (one cell past the grid point), u stays 0 when r0 is
// not below any entry of cdfV, and (0, 0) comes back when r1 is not below
// any entry of its row (so NaN tables warp nothing).
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define VMR_HD __host__ __device__ __forceinline__
#else
#define VMR_HD inline
#endif

namespace vmr {

// cdf[0 .. n) = cdfV, cdf[n + j*n + i] = cdfVU[j][i]; n = 0: no filter.
struct PixFilter {
  const double* cdf;
  uint32_t n;
  double w;
};

VMR_HD void warp_sample(const PixFilter& f, double r0, double r1, double& u, double& v) {
  const int n = (int)f.n;
  const double w = f.w;
  const double* cdfV = f.cdf;
  u = 0.0;
  v = 0.0;
  int uI = -1;
  for (int i = 0; i < n; ++i) {
    uI = i;
    if (r0 < cdfV[i]) {
      if (i == 0) {
        u = (-w / 2) + ((r0 / cdfV[0]) / w);
      } else {
        const double du = (r0 - cdfV[i - 1]) / (cdfV[i] - cdfV[i - 1]);
        u = (-w / 2) + w * ((double)i + du) / (double)(n - 1);
      }
      break;
    }
  }
  const double* row = f.cdf + n + (int64_t)uI * n;
  for (int i = 0; i < n; ++i) {
    if (r1 < row[i]) {
      if (i == 0) {
        v = (-w / 2) + ((r1 / row[0]) / w);
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

}  // namespace vmr
