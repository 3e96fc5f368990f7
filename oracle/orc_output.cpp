// orc_output.cpp - the OutputHDR pixel encoding.
// TEST INFRASTRUCTURE ONLY (see orc.h): the checker for vmr_encode_rgbe.
//
// Restates image/hdr/writer.go:58-82 (scanline j = image row h-1-j, no
// run-length encoding) and convertRGBToRGBE (image/hdr/hdr.go:28-55) in
// float32: d = the largest of r, g, b by the comparisons g > d, b > d;
// d < 1e-6 gives four zero bytes; (m, e) = frexp(float64(d)) (frexp of
// +Inf or NaN returns it with exponent 0, as Go's math.Frexp does);
// df = float32(m) * 255.999 / d; the colour bytes are byte(c * df) and the
// exponent byte byte(e + 128).  byte(x) of a float32 is Go's amd64
// conversion: truncation to a 32-bit integer, low byte; a NaN or a value
// outside the 32-bit range gives the integer indefinite, low byte 0.
#include <cmath>
#include <cstdint>

#include "orc.h"

namespace {

uint8_t go_byte(float x) {
  if (!(x > -2147483648.0f && x < 2147483648.0f)) return 0;
  return (uint8_t)(uint32_t)(int32_t)x;
}

void rgbe(float r, float g, float b, uint8_t o[4]) {
  float d = r;
  if (g > d) d = g;
  if (b > d) d = b;
  if (d < 0.000001f) {
    o[0] = o[1] = o[2] = o[3] = 0;
    return;
  }
  int e = 0;
  double m = (double)d;
  if (std::isfinite(m)) m = std::frexp(m, &e);
  const float n = (float)m;
  const float df = n * 255.999f / d;
  o[0] = go_byte(r * df);
  o[1] = go_byte(g * df);
  o[2] = go_byte(b * df);
  o[3] = (uint8_t)(e + 128);
}

}  // namespace

extern "C" int orc_encode_rgbe(const float* rgb, uint32_t w, uint32_t h, uint8_t* out) {
  if ((w && h) && (!rgb || !out)) return -1;
  for (uint32_t j = 0; j < h; ++j) {
    const uint32_t k = h - j - 1;
    for (uint32_t i = 0; i < w; ++i) {
      const float* p = rgb + ((size_t)k * w + i) * 3;
      rgbe(p[0], p[1], p[2], out + ((size_t)j * w + i) * 4);
    }
  }
  return 0;
}
