// orc_ldseq.cpp - CPU oracle for the QMC sequences of math/ldseq.
//
// TEST INFRASTRUCTURE ONLY (see orc.h).  Bit-exact integer restatements of
// the scrambled Van der Corput and Sobol radical inverses and of the
// Grunschloss enumeration RasterXY.  The two enumeration tables
// (math/ldseq/vdc_sobol_matrices52.go) are not copied: they are derived here
// from the two generator matrices and Gauss-Jordan elimination over GF(2).
#include "orc.h"

#include <cstring>

namespace {

// ldseq.vanDerCorput (math/ldseq/ldseq.go:55-75): 64-bit bit reversal,
// XOR scramble, keep 52 bits.
uint64_t vdc(uint64_t i, uint64_t scramble) {
  uint64_t bits = (i << 32) | (i >> 32);
  bits = ((bits & 0x0000ffff0000ffffull) << 16) | ((bits & 0xffff0000ffff0000ull) >> 16);
  bits = ((bits & 0x00ff00ff00ff00ffull) << 8) | ((bits & 0xff00ff00ff00ff00ull) >> 8);
  bits = ((bits & 0x0f0f0f0f0f0f0f0full) << 4) | ((bits & 0xf0f0f0f0f0f0f0f0ull) >> 4);
  bits = ((bits & 0x3333333333333333ull) << 2) | ((bits & 0xccccccccccccccccull) >> 2);
  bits = ((bits & 0x5555555555555555ull) << 1) | ((bits & 0xaaaaaaaaaaaaaaaaull) >> 1);
  return (scramble ^ bits) >> (64 - 52);
}

// ldseq.sobol (ldseq.go:83-96): the second Sobol dimension, columns
// v_0 = 2^51, v_{k+1} = v_k ^ (v_k >> 1).
uint64_t sobol(uint64_t i, uint64_t scramble) {
  uint64_t r = scramble >> (64 - 52);
  for (uint64_t v = 1ull << 51; i != 0; i >>= 1) {
    if (i & 1) r ^= v;
    v ^= v >> 1;
  }
  return r;
}

// The 2m-bit image (px << m) | py of a sample index at resolution 2^m.
uint64_t raster_bits(uint32_t m, uint64_t index) {
  uint64_t px = vdc(index, 0) >> (52 - m);
  uint64_t py = sobol(index, 0) >> (52 - m);
  return (px << m) | py;
}

// fwd[c] = image of index bit 2m+c (the part of the pixel coordinates fixed
// by the frame number; only py is affected), zero once 2m+c >= 52.
// inv[c] = the low-2m-bit index whose image is the unit vector e_c.
void tables(uint32_t m, uint64_t* fwd, uint64_t* inv) {
  for (int c = 0; c < 52; ++c) { fwd[c] = 0; inv[c] = 0; }
  const uint32_t n = 2 * m;
  for (uint32_t c = 0; n + c < 52; ++c) fwd[c] = raster_bits(m, 1ull << (n + c));
  // rows[r] = (A row r over index bits, identity row r) for Gauss-Jordan.
  uint64_t a[52], e[52];
  for (uint32_t r = 0; r < n; ++r) {
    a[r] = 0;
    for (uint32_t k = 0; k < n; ++k)
      if ((raster_bits(m, 1ull << k) >> r) & 1) a[r] |= 1ull << k;
    e[r] = 1ull << r;
  }
  for (uint32_t col = 0; col < n; ++col) {
    uint32_t p = col;
    while (p < n && !((a[p] >> col) & 1)) ++p;
    if (p == n) return;  // singular: cannot happen for a (0,2)-sequence
    uint64_t t = a[p]; a[p] = a[col]; a[col] = t;
    t = e[p]; e[p] = e[col]; e[col] = t;
    for (uint32_t r = 0; r < n; ++r)
      if (r != col && ((a[r] >> col) & 1)) { a[r] ^= a[col]; e[r] ^= e[col]; }
  }
  // Now row k of e is row k of A^-1: bit c of e[k] = (A^-1)[k][c].
  for (uint32_t c = 0; c < n; ++c) {
    uint64_t x = 0;
    for (uint32_t k = 0; k < n; ++k)
      if ((e[k] >> c) & 1) x |= 1ull << k;
    inv[c] = x;
  }
}

// ldseq.lookup (math/ldseq/raster.go:10-40).
uint64_t lookup(uint32_t m, uint32_t frame, uint32_t px, uint32_t py, uint64_t sx, uint64_t sy) {
  uint64_t fwd[52], inv[52];
  tables(m, fwd, inv);
  uint32_t m2 = m << 1;
  uint64_t index = (uint64_t)frame << m2;
  uint64_t delta = 0;
  for (uint32_t c = 0; frame != 0; frame >>= 1, ++c)
    if (frame & 1) delta ^= fwd[c];
  px ^= (uint32_t)(sx >> (64 - m));
  py ^= (uint32_t)(sy >> (64 - m));
  uint64_t b = (((uint64_t)px << m) | (uint64_t)py) ^ delta;
  for (uint32_t c = 0; b != 0; b >>= 1, ++c)
    if (b & 1) index ^= inv[c];
  return index;
}

}  // namespace

extern "C" {

uint64_t orc_vdc(uint64_t i, uint64_t scramble) { return vdc(i, scramble); }
uint64_t orc_sobol(uint64_t i, uint64_t scramble) { return sobol(i, scramble); }

// ldseq.RasterXY (raster.go:50-57).
uint64_t orc_raster_xy(uint32_t m, uint32_t frame, uint32_t px, uint32_t py, uint64_t sx, uint64_t sy,
                       double* rx, double* ry) {
  uint64_t index = lookup(m, frame, px, py, sx, sy);
  const double scale = (double)(1ull << (52 - m));
  if (rx) *rx = (double)vdc(index, sx) / scale;
  if (ry) *ry = (double)sobol(index, sy) / scale;
  return index;
}

void orc_vdc_sobol_tables(uint32_t m, uint64_t* fwd52, uint64_t* inv52) {
  uint64_t f[52], v[52];
  tables(m, f, v);
  if (fwd52) std::memcpy(fwd52, f, sizeof(f));
  if (inv52) std::memcpy(inv52, v, sizeof(v));
}

}  // extern "C"
