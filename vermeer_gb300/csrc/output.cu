// output.cu - the OutputHDR driver's pixel encoding on the device.
//
// builtin/driver/outputhdr.go:26-55 writes core.FrameBuf() through the
// Radiance writer (image/hdr/writer.go:58-82): after a text header, one
// scanline per image row from the bottom row up (scanline j holds row
// h - j - 1), each pixel as the 4 bytes of convertRGBToRGBE
// (image/hdr/hdr.go:28-55), without run-length encoding.  k_encode_rgbe
// produces those bytes, one thread per output pixel (12 bytes read, 4
// written: a memory-bound pass), so only a quarter of the float
// framebuffer's bytes cross to the host.
//
// convertRGBToRGBE in float32 as the reference computes it:
//   d = max of r, g, b by the comparisons g > d, b > d (a NaN never wins);
//   d < 1e-6 -> (0, 0, 0, 0);
//   (m, e) = frexp(float64(d)), m in [0.5, 1); df = float32(m) * 255.999 / d;
//   bytes = byte(r*df), byte(g*df), byte(b*df), byte(e + 128).
// Go's float32 -> byte conversion on amd64 truncates to a 32-bit integer and
// keeps its low byte (a NaN or out-of-range value gives the integer
// indefinite 0x80000000, low byte 0); frexp(+Inf) and frexp(NaN) give the
// value itself and exponent 0.  Both are reproduced exactly.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#include "ctx.h"
#include "vmr.h"

namespace vmr {
namespace {

__device__ __forceinline__ uint8_t go_byte(float x) {
  if (!(x > -2147483648.0f && x < 2147483648.0f)) return 0;  // NaN, +-Inf, out of int32 range
  return (uint8_t)(uint32_t)(int32_t)x;                      // truncation toward zero, low byte
}

__global__ void k_encode_rgbe(const float* __restrict__ rgb, uint32_t w, uint32_t h, uchar4* __restrict__ out) {
  const uint64_t n = (uint64_t)w * h;
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t j = (uint32_t)(p / w), i = (uint32_t)(p % w);
    const uint64_t src = ((uint64_t)(h - j - 1) * w + i) * 3;
    const float r = rgb[src], g = rgb[src + 1], b = rgb[src + 2];
    float d = r;
    if (g > d) d = g;
    if (b > d) d = b;
    uchar4 o = make_uchar4(0, 0, 0, 0);
    if (!(d < 0.000001f)) {
      int e = 0;
      double m = (double)d;
      if (isfinite(m)) m = frexp(m, &e);
      const float df = __fdiv_rn(__fmul_rn((float)m, 255.999f), d);
      o = make_uchar4(go_byte(__fmul_rn(r, df)), go_byte(__fmul_rn(g, df)), go_byte(__fmul_rn(b, df)),
                      (uint8_t)(e + 128));
    }
    out[p] = o;
  }
}

}  // namespace
}  // namespace vmr

extern "C" int vmr_encode_rgbe(vmr_ctx* ctx, const float* rgb, uint32_t width, uint32_t height, int flags,
                               uint8_t* rgbe) {
  if (!ctx || !rgb || !rgbe) return VMR_ERR_INVALID;
  if (ctx->device < 0) {
    ctx->err = "host-only context cannot encode";
    return VMR_ERR_UNSUPPORTED;
  }
  if (width == 0 || height == 0) return VMR_OK;
  cudaSetDevice(ctx->device);
  const size_t npix = (size_t)width * height;
  const bool dev_in = (flags & VMR_IO_DEVICE_IN) != 0, dev_out = (flags & VMR_IO_DEVICE_OUT) != 0;
  cudaStream_t st = ctx->stream;
  vmr::RenderState& R = ctx->render;
  const size_t in_bytes = dev_in ? 0 : (npix * 12 + 255) / 256 * 256;
  const size_t out_bytes = dev_out ? 0 : npix * 4;
  cudaError_t e = cudaSuccess;
  if (in_bytes + out_bytes) e = R.outbuf.ensure(in_bytes + out_bytes);
  if (e != cudaSuccess) {
    ctx->err = cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? VMR_ERR_OOM : VMR_ERR_CUDA;
  }
  const float* d_in = rgb;
  if (!dev_in) {
    e = cudaMemcpyAsync(R.outbuf.p, rgb, npix * 12, cudaMemcpyHostToDevice, st);
    d_in = R.outbuf.as<const float>();
  }
  uchar4* d_out = dev_out ? reinterpret_cast<uchar4*>(rgbe)
                          : reinterpret_cast<uchar4*>(static_cast<char*>(R.outbuf.p) + in_bytes);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const uint64_t want = (npix + 255) / 256;
  const int grid = (int)(want < (uint64_t)sms * 8 ? want : (uint64_t)sms * 8);
  if (e == cudaSuccess) {
    vmr::k_encode_rgbe<<<grid > 0 ? grid : 1, 256, 0, st>>>(d_in, width, height, d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && !dev_out) e = cudaMemcpyAsync(rgbe, d_out, npix * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    ctx->err = cudaGetErrorString(e);
    return VMR_ERR_CUDA;
  }
  return VMR_OK;
}
