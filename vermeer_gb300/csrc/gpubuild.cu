// gpubuild.cu - QBVH construction on the device, byte-identical to the host
// builder (accel.cpp) and so to the reference's qbvh.BuildAccel
// (qbvh/build.go:28-307) as PolyMesh.initAccel calls it
// (builtin/geom/polymesh/buildqbvh.go:14-144, leafMax 16).
//
// The reference recursion builds one QBVH node from three binary splits of
// an index range: the whole range, then its left and its right part
// (build.go:180-192).  Here the nodes of one tree level are built together,
// one CTA per node, and the tree is numbered afterwards in the reference's
// pre-order.  Every float result that reaches the output is produced by the
// same operation sequence as the reference:
//  * triangle boxes and centroids per triangle as in buildqbvh.go:19-83;
//  * centroid bounds, bin boxes and bin counts feed only comparisons and the
//    SAH costs, whose values do not depend on the fold order (min and max of
//    finite floats, integer counts; a signed zero changes no extent), so they
//    are reduced in parallel;
//  * the SAH cost of each plane in the reference's operation order;
//  * the in-place partition of build.go:111-130 (a left cursor that keeps
//    "left" elements and swaps "right" ones with the element under a right
//    cursor) as its closed form, computed with prefix counts.  With nL left
//    elements, P = nL + (element nL is "right"), the j-th "right" element of
//    [0, P) and the j-th "left" element of [P, n) counted from the end are
//    the switch points; left elements of [0, P) stay, right elements of
//    [P, n) move down by one, the j-th left switch element goes to the j-th
//    right switch position, and the j-th right switch element to position
//    n-1 (j = 0) or one below the (j-1)-th left switch element's position;
//  * stored node boxes are folded sequentially in element order (leaves) and
//    child order (inner nodes), as build.go:203-283 does, so signed zeros
//    come out as in the reference.
// Input whose build geometry is not finite is declined (the host builder
// takes it).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "gpubuild.h"

namespace vmr {
namespace {

namespace cg = cooperative_groups;

constexpr int kLeafMax = 16;
constexpr int kMaxLevels = 4096;
constexpr float kBinScale = 8.0f * 0.99994f;  // float32(nbins) * (1.0 - 0.00006), build.go:45

enum : int {
  kErrBin = 1,        // centroid bin out of range (build.go:57-62 panics)
  kErrPartition = 2,  // partition bookkeeping inconsistent
  kErrCapacity = 4,   // task table full
  kErrNonFinite = 8,  // build geometry not finite: declined
};

struct BTask {
  int first, n;
  int p0, p1, p2;  // pivots of the three splits: [0,p1) [p1,p0) [p0,p0+p2) [p0+p2,n)
  int axes;        // axis0 | axis1 << 2 | axis2 << 4
  int child[4];    // task of an inner child, -1 for a leaf or an empty child
};

struct Bufs {
  float4 *A, *B, *C;     // (box min xyz, id bits), (box max xyz, 0), (centroid xyz, 0)
  float4 *TA, *TB, *TC;  // partition targets
  int* sw;               // switch-element positions
  int* rk;               // switch-element ranks
  BTask* tasks;
  int* n_tasks;
  int* err;
  int cap;
};

__device__ __forceinline__ float gmin(float x, float y) { return x < y ? x : y; }  // math.Min
__device__ __forceinline__ float gmax(float x, float y) { return x > y ? x : y; }  // math.Max
__device__ __forceinline__ float comp(const float4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

template <int BS>
struct Smem {
  static constexpr int W = BS / 32;
  float part[W][8][6];
  int pcnt[W][8];
  float wcb[W][6];
  int wsum[W][2];
  // this CTA's partial results, read by the other CTAs of the cluster
  float cb[6];
  float bin[8][6];
  int cnt[8];
  int sw_count[2];
  float scale, origin;
  int axis, flat, plane, nL, P;
};

// The CTAs that build one node: a thread-block cluster of CL CTAs (CL = 1:
// a single CTA).  Each CTA owns a contiguous slice of every range; partial
// results are exchanged through distributed shared memory in rank order, so
// all CTAs derive identical split decisions.
template <int CL>
struct Team {
  int rank;
  __device__ Team() {
    if constexpr (CL > 1) rank = (int)cg::this_cluster().block_rank();
    else rank = 0;
  }
  __device__ __forceinline__ void sync() const {
    if constexpr (CL > 1) cg::this_cluster().sync();  // barrier.cluster arrive.release / wait.acquire
    else __syncthreads();
  }
  template <class T>
  __device__ __forceinline__ T* peer(T* p, int r) const {
    if constexpr (CL > 1) return cg::this_cluster().map_shared_rank(p, r);
    else return p;
  }
  // [lo, hi) of an n-element range owned by this CTA
  __device__ __forceinline__ void slice(int n, int& lo, int& hi) const {
    lo = (int)(((long long)n * rank) / CL);
    hi = (int)(((long long)n * (rank + 1)) / CL);
  }
};

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = gmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = gmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int BS>
__device__ void copy_range(const float4* __restrict__ SA, const float4* __restrict__ SB,
                           const float4* __restrict__ SC, float4* __restrict__ DA, float4* __restrict__ DB,
                           float4* __restrict__ DC, int f, int lo, int hi) {
  for (int i = lo + (int)threadIdx.x; i < hi; i += BS) {
    DA[f + i] = SA[f + i];
    DB[f + i] = SB[f + i];
    DC[f + i] = SC[f + i];
  }
}

__device__ __forceinline__ int bin_of(float c, float scale, float origin) {
  return __float2int_rz(__fmul_rn(scale, __fsub_rn(c, origin)));  // int(k1 * (c - k0)), build.go:55
}

// binarySplit + calcMinCost (build.go:28-178) over [f, f+n) of S, the
// partitioned range written to D.  Returns (axis, pivot) in every thread of
// every CTA of the team.
template <int BS, int CL>
__device__ int2 split(const float4* __restrict__ SA, const float4* __restrict__ SB, const float4* __restrict__ SC,
                      float4* __restrict__ DA, float4* __restrict__ DB, float4* __restrict__ DC, int* __restrict__ sw,
                      int* __restrict__ rk, int f, int n, int* err, Smem<BS>& sh, const Team<CL>& team) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int W = Smem<BS>::W;
  const float inf = __int_as_float(0x7f800000);
  int lo, hi;
  team.slice(n, lo, hi);
  team.sync();  // shared state of a previous split is no longer read, here or by peers
  if (n <= kLeafMax) {
    copy_range<BS>(SA, SB, SC, DA, DB, DC, f, lo, hi);
    return make_int2(0, n);
  }
  // Centroid bounds.
  float l0 = inf, l1 = inf, l2 = inf, h0 = -inf, h1 = -inf, h2 = -inf;
  for (int i = lo + tid; i < hi; i += BS) {
    const float4 c = SC[f + i];
    l0 = gmin(c.x, l0); l1 = gmin(c.y, l1); l2 = gmin(c.z, l2);
    h0 = gmax(c.x, h0); h1 = gmax(c.y, h1); h2 = gmax(c.z, h2);
  }
  l0 = warp_min(l0); l1 = warp_min(l1); l2 = warp_min(l2);
  h0 = warp_max(h0); h1 = warp_max(h1); h2 = warp_max(h2);
  if (lane == 0) {
    sh.wcb[warp][0] = l0; sh.wcb[warp][1] = l1; sh.wcb[warp][2] = l2;
    sh.wcb[warp][3] = h0; sh.wcb[warp][4] = h1; sh.wcb[warp][5] = h2;
  }
  __syncthreads();
  if (tid == 0) {
    float b[6] = {inf, inf, inf, -inf, -inf, -inf};
    for (int w = 0; w < W; ++w)
      for (int k = 0; k < 3; ++k) {
        b[k] = gmin(sh.wcb[w][k], b[k]);
        b[3 + k] = gmax(sh.wcb[w][3 + k], b[3 + k]);
      }
    for (int k = 0; k < 6; ++k) sh.cb[k] = b[k];
  }
  team.sync();
  if (tid == 0) {
    float b[6] = {inf, inf, inf, -inf, -inf, -inf};
    for (int r = 0; r < CL; ++r) {
      const float* pc = team.peer(sh.cb, r);
      for (int k = 0; k < 3; ++k) {
        b[k] = gmin(pc[k], b[k]);
        b[3 + k] = gmax(pc[3 + k], b[3 + k]);
      }
    }
    // BoundingBox.MaxDim (math/boundingbox.go:54-70)
    const float e0 = __fsub_rn(b[3], b[0]), e1 = __fsub_rn(b[4], b[1]), e2 = __fsub_rn(b[5], b[2]);
    int axis;
    if (e0 < e1) axis = e1 < e2 ? 2 : 1;
    else axis = e0 < e2 ? 2 : 0;
    sh.axis = axis;
    sh.flat = b[3 + axis] == b[axis];
    sh.origin = b[axis];
    sh.scale = sh.flat ? 0.0f : __fdiv_rn(kBinScale, __fsub_rn(b[3 + axis], b[axis]));
  }
  __syncthreads();
  const int axis = sh.axis;
  if (sh.flat) {  // build.go:34-43
    copy_range<BS>(SA, SB, SC, DA, DB, DC, f, lo, hi);
    return make_int2(axis, n / 2 + 1);
  }
  const float scale = sh.scale, origin = sh.origin;
  // Bin counts and boxes (build.go:52-66).
  float bl[8][3], bh[8][3];
  int bc[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    bc[k] = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) { bl[k][a] = inf; bh[k][a] = -inf; }
  }
  bool bad = false;
  for (int i = lo + tid; i < hi; i += BS) {
    const float4 c = SC[f + i], a = SA[f + i], b = SB[f + i];
    int bin = bin_of(comp(c, axis), scale, origin);
    if (bin < 0 || bin > 7) { bad = true; bin = bin < 0 ? 0 : 7; }
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (bin == k) {
        ++bc[k];
        bl[k][0] = gmin(bl[k][0], a.x); bl[k][1] = gmin(bl[k][1], a.y); bl[k][2] = gmin(bl[k][2], a.z);
        bh[k][0] = gmax(bh[k][0], b.x); bh[k][1] = gmax(bh[k][1], b.y); bh[k][2] = gmax(bh[k][2], b.z);
      }
  }
  if (bad) atomicOr(err, kErrBin);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int c = warp_sum(bc[k]);
    float v[6];
#pragma unroll
    for (int a = 0; a < 3; ++a) { v[a] = warp_min(bl[k][a]); v[3 + a] = warp_max(bh[k][a]); }
    if (lane == 0) {
      sh.pcnt[warp][k] = c;
#pragma unroll
      for (int a = 0; a < 6; ++a) sh.part[warp][k][a] = v[a];
    }
  }
  __syncthreads();
  if (tid < 8) {
    const int k = tid;
    int c = 0;
    float v[6] = {inf, inf, inf, -inf, -inf, -inf};
    for (int w = 0; w < W; ++w) {
      c += sh.pcnt[w][k];
      for (int a = 0; a < 3; ++a) {
        v[a] = gmin(v[a], sh.part[w][k][a]);
        v[3 + a] = gmax(v[3 + a], sh.part[w][k][3 + a]);
      }
    }
    sh.cnt[k] = c;
    for (int a = 0; a < 6; ++a) sh.bin[k][a] = v[a];
  }
  team.sync();
  if (tid == 0) {
    float bin[8][6];
    int cnt8[8];
    for (int k = 0; k < 8; ++k) {
      cnt8[k] = 0;
      for (int a = 0; a < 3; ++a) { bin[k][a] = inf; bin[k][3 + a] = -inf; }
    }
    for (int r = 0; r < CL; ++r) {
      const float* pb = &team.peer(&sh.bin[0][0], r)[0];
      const int* pn = team.peer(&sh.cnt[0], r);
      for (int k = 0; k < 8; ++k) {
        cnt8[k] += pn[k];
        for (int a = 0; a < 3; ++a) {
          bin[k][a] = gmin(bin[k][a], pb[k * 6 + a]);
          bin[k][3 + a] = gmax(bin[k][3 + a], pb[k * 6 + 3 + a]);
        }
      }
    }
    // Costs from the left and from the right (build.go:68-107).
    float lb[8][6], rb[8][6];
    int ln[8], rn[8];
    float acc[6];
    for (int a = 0; a < 3; ++a) { acc[a] = inf; acc[3 + a] = -inf; }
    int cnt = 0;
    for (int i = 0; i < 8; ++i) {
      for (int a = 0; a < 3; ++a) { acc[a] = gmin(acc[a], bin[i][a]); acc[3 + a] = gmax(acc[3 + a], bin[i][3 + a]); }
      cnt += cnt8[i];
      for (int a = 0; a < 6; ++a) lb[i][a] = acc[a];
      ln[i] = cnt;
    }
    for (int a = 0; a < 3; ++a) { acc[a] = inf; acc[3 + a] = -inf; }
    cnt = 0;
    for (int i = 7; i >= 0; --i) {
      for (int a = 0; a < 3; ++a) { acc[a] = gmin(acc[a], bin[i][a]); acc[3 + a] = gmax(acc[3 + a], bin[i][3 + a]); }
      cnt += cnt8[i];
      for (int a = 0; a < 6; ++a) rb[i][a] = acc[a];
      rn[i] = cnt;
    }
    int plane = -1;
    float best = inf;
    for (int i = 1; i < 8; ++i) {
      // BoundingBox.SurfaceArea (boundingbox.go:17-19) times the count
      const float le0 = __fsub_rn(lb[i - 1][3], lb[i - 1][0]), le1 = __fsub_rn(lb[i - 1][4], lb[i - 1][1]),
                  le2 = __fsub_rn(lb[i - 1][5], lb[i - 1][2]);
      const float re0 = __fsub_rn(rb[i][3], rb[i][0]), re1 = __fsub_rn(rb[i][4], rb[i][1]),
                  re2 = __fsub_rn(rb[i][5], rb[i][2]);
      const float la = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(le0, le1), 2.0f), __fmul_rn(__fmul_rn(le1, le2), 2.0f)),
                                 __fmul_rn(__fmul_rn(le0, le2), 2.0f));
      const float ra = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(re0, re1), 2.0f), __fmul_rn(__fmul_rn(re1, re2), 2.0f)),
                                 __fmul_rn(__fmul_rn(re0, re2), 2.0f));
      const float cost = __fadd_rn(__fmul_rn(la, (float)ln[i - 1]), __fmul_rn(ra, (float)rn[i]));
      if (cost < best) { best = cost; plane = i; }
    }
    int nL = 0;
    for (int k = 0; k < 8; ++k)
      if (k < plane) nL += cnt8[k];
    int P = nL;
    if (nL < n && bin_of(comp(SC[f + nL], axis), scale, origin) >= plane) P = nL + 1;
    sh.plane = plane;
    sh.nL = nL;
    sh.P = P;
  }
  __syncthreads();
  const int plane = sh.plane, nL = sh.nL, P = sh.P;
  const unsigned below = (1u << lane) - 1u;
  // Switch elements of this CTA's slice, then the slices before it.
  int baseL = 0, baseR = 0, kL = 0, kR = 0;
  if constexpr (CL > 1) {
    int cl = 0, cr = 0;
    for (int i = lo + tid; i < hi; i += BS) {
      const bool right = bin_of(comp(SC[f + i], axis), scale, origin) >= plane;
      cl += (i < P && right);
      cr += (i >= P && !right);
    }
    cl = warp_sum(cl);
    cr = warp_sum(cr);
    if (lane == 0) { sh.wsum[warp][0] = cl; sh.wsum[warp][1] = cr; }
    __syncthreads();
    if (tid == 0) {
      int a = 0, b2 = 0;
      for (int w = 0; w < W; ++w) { a += sh.wsum[w][0]; b2 += sh.wsum[w][1]; }
      sh.sw_count[0] = a;
      sh.sw_count[1] = b2;
    }
    team.sync();
    for (int r = 0; r < CL; ++r) {
      const int* pc = team.peer(sh.sw_count, r);
      if (r < team.rank) { baseL += pc[0]; baseR += pc[1]; }
      kL += pc[0];
      kR += pc[1];
    }
    __syncthreads();  // wsum is reused below
  }
  int runL = baseL, runR = baseR;
  for (int base = lo; base < hi; base += BS) {
    const int i = base + tid;
    bool fl = false, fr = false;
    if (i < hi) {
      const bool right = bin_of(comp(SC[f + i], axis), scale, origin) >= plane;
      fl = i < P && right;
      fr = i >= P && !right;
    }
    const unsigned ml = __ballot_sync(0xffffffffu, fl), mr = __ballot_sync(0xffffffffu, fr);
    if (lane == 0) { sh.wsum[warp][0] = __popc(ml); sh.wsum[warp][1] = __popc(mr); }
    __syncthreads();
    int offL = 0, offR = 0, totL = 0, totR = 0;
    for (int w = 0; w < W; ++w) {
      const int a = sh.wsum[w][0], b = sh.wsum[w][1];
      if (w < warp) { offL += a; offR += b; }
      totL += a;
      totR += b;
    }
    if (fl) {
      const int j = runL + offL + __popc(ml & below);
      sw[f + j] = i;
      rk[f + i] = j;
    }
    if (fr) {
      const int q = runR + offR + __popc(mr & below);
      sw[f + n - 1 - q] = i;
      rk[f + i] = q;
    }
    runL += totL;
    runR += totR;
    __syncthreads();
  }
  if constexpr (CL == 1) {
    kL = runL;
    kR = runR;
  }
  if (tid == 0 && team.rank == 0 && kL - kR != P - nL) atomicOr(err, kErrPartition);
  team.sync();  // every switch position of the range is written
  // Scatter to the partitioned order.
  for (int i = lo + tid; i < hi; i += BS) {
    const float4 a = SA[f + i], b = SB[f + i], c = SC[f + i];
    const bool right = bin_of(comp(c, axis), scale, origin) >= plane;
    int d;
    if (i < P) {
      if (!right) {
        d = i;
      } else {
        const int j = rk[f + i];
        d = j == 0 ? n - 1 : sw[f + n - 1 - (kR - j)] - 1;
      }
    } else if (right) {
      d = i - 1;
    } else {
      d = sw[f + (kR - 1 - rk[f + i])];
    }
    if ((unsigned)d >= (unsigned)n) {
      atomicOr(err, kErrPartition);
      continue;
    }
    DA[f + d] = a;
    DB[f + d] = b;
    DC[f + d] = c;
  }
  return make_int2(axis, nL);
}

// One tree level: each team (a CTA or a cluster) builds the node of one
// task (build.go:180-192) and appends its inner children to the next level.
template <int BS, int CL>
__global__ void __launch_bounds__(BS) k_build_level(Bufs b, int t0) {
  __shared__ Smem<BS> sh;
  const Team<CL> team;
  const int t = t0 + (int)blockIdx.x / CL;
  const int f = b.tasks[t].first, n = b.tasks[t].n;
  const int2 s0 = split<BS, CL>(b.A, b.B, b.C, b.TA, b.TB, b.TC, b.sw, b.rk, f, n, b.err, sh, team);
  // split 1 and 2 read the whole of split 0's output
  team.sync();
  const int2 s1 = split<BS, CL>(b.TA, b.TB, b.TC, b.A, b.B, b.C, b.sw, b.rk, f, s0.y, b.err, sh, team);
  const int2 s2 = split<BS, CL>(b.TA, b.TB, b.TC, b.A, b.B, b.C, b.sw, b.rk, f + s0.y, n - s0.y, b.err, sh, team);
  team.sync();  // no CTA leaves while a peer may still read its shared memory
  if (threadIdx.x == 0 && team.rank == 0) {
    BTask& T = b.tasks[t];
    T.p0 = s0.y;
    T.p1 = s1.y;
    T.p2 = s2.y;
    T.axes = s0.x | (s1.x << 2) | (s2.x << 4);
    const int beg[4] = {0, s1.y, s0.y, s0.y + s2.y};
    const int end[4] = {s1.y, s0.y, s0.y + s2.y, n};
    for (int c = 0; c < 4; ++c) {
      const int len = end[c] - beg[c];
      T.child[c] = -1;
      if (len > kLeafMax) {
        const int idx = atomicAdd(b.n_tasks, 1);
        if (idx >= b.cap) {
          atomicOr(b.err, kErrCapacity);
          continue;
        }
        BTask nt;
        nt.first = f + beg[c];
        nt.n = len;
        nt.p0 = nt.p1 = nt.p2 = nt.axes = 0;
        nt.child[0] = nt.child[1] = nt.child[2] = nt.child[3] = -1;
        b.tasks[idx] = nt;
        T.child[c] = idx;
      }
    }
  }
}

// Build geometry per triangle (buildqbvh.go:19-83): the key-0 vertices, or
// the mesh lerped to time 0.5 for a motion mesh.
__global__ void k_prep(const float* __restrict__ verts, const uint32_t* __restrict__ idxp, int n, uint32_t n_verts,
                       int motion, uint32_t ka, uint32_t kb, float tt, float4* A, float4* B, float4* C, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float v[3][3];
  bool finite = true;
  for (int j = 0; j < 3; ++j) {
    const uint32_t vi = idxp[(size_t)i * 3 + j];
    const float* a = verts + ((size_t)ka * n_verts + vi) * 3;
    if (motion) {
      const float* bb = verts + ((size_t)kb * n_verts + vi) * 3;
      const float w = __fsub_rn(1.0f, tt);
      for (int k = 0; k < 3; ++k) v[j][k] = __fadd_rn(__fmul_rn(w, a[k]), __fmul_rn(tt, bb[k]));  // Vec3Lerp
    } else {
      for (int k = 0; k < 3; ++k) v[j][k] = a[k];
    }
    for (int k = 0; k < 3; ++k) finite = finite && isfinite(v[j][k]);
  }
  if (!finite) atomicOr(err, kErrNonFinite);
  const float inf = __int_as_float(0x7f800000);
  float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
  for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 3; ++k) {  // BoundingBox.Grow: Min(point, box)
      lo[k] = gmin(v[j][k], lo[k]);
      hi[k] = gmax(v[j][k], hi[k]);
    }
  float c[3];
  for (int k = 0; k < 3; ++k) c[k] = __fdiv_rn(__fadd_rn(__fadd_rn(v[0][k], v[1][k]), v[2][k]), 3.0f);
  A[i] = make_float4(lo[0], lo[1], lo[2], __int_as_float(i));
  B[i] = make_float4(hi[0], hi[1], hi[2], 0.0f);
  C[i] = make_float4(c[0], c[1], c[2], 0.0f);
}

// Subtree node counts, deepest level first.
__global__ void k_sizes(const BTask* __restrict__ tasks, int t0, int count, int* size) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const BTask& T = tasks[t0 + i];
  int s = 1;
  for (int c = 0; c < 4; ++c)
    if (T.child[c] >= 0) s += size[T.child[c]];
  size[t0 + i] = s;
}

// Pre-order node numbers (buildAccelRec appends a node before recursing
// into children 0..3), top level first.
__global__ void k_ids(const BTask* __restrict__ tasks, int t0, int count, const int* __restrict__ size, int* id) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const BTask& T = tasks[t0 + i];
  int run = id[t0 + i] + 1;
  for (int c = 0; c < 4; ++c) {
    const int ch = T.child[c];
    if (ch >= 0) {
      id[ch] = run;
      run += size[ch];
    }
  }
}

__device__ __forceinline__ void child_range(const BTask& T, int c, int& beg, int& len) {
  const int b[5] = {0, T.p1, T.p0, T.p0 + T.p2, T.n};
  beg = b[c];
  len = b[c + 1] - b[c];
}

// Node.SetLeaf (qbvh/qbvh.go:82-93).
__device__ __forceinline__ int32_t encode_leaf(uint32_t first, uint32_t count) {
  return (int32_t)((1u << 31) | ((first << 4) & 0xfffffff0u) | ((count - 1u) & 0xfu));
}

// Static nodes, deepest level first: leaf boxes folded over the leaf's
// elements, inner boxes from the child's node union (build.go:201-283).
__global__ void k_nodes(const BTask* __restrict__ tasks, int t0, int count, const int* __restrict__ id,
                        const float4* __restrict__ A, const float4* __restrict__ B, float* nbox,
                        vmr_qbvh_node* nodes) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int t = t0 + i;
  const BTask& T = tasks[t];
  const float inf = __int_as_float(0x7f800000);
  vmr_qbvh_node nd;
  memset(&nd, 0, sizeof(nd));
  nd.axis0 = (uint32_t)(T.axes & 3);
  nd.axis1 = (uint32_t)((T.axes >> 2) & 3);
  nd.axis2 = (uint32_t)((T.axes >> 4) & 3);
  float u[6] = {inf, inf, inf, -inf, -inf, -inf};
  for (int c = 0; c < 4; ++c) {
    int beg, len;
    child_range(T, c, beg, len);
    float bx[6];
    if (len == 0) {  // SetEmptyLeaf (qbvh.go:67-79)
      nd.children[c] = -1;
      for (int k = 0; k < 6; ++k) bx[k] = inf;
    } else if (len <= kLeafMax) {
      for (int k = 0; k < 3; ++k) { bx[k] = inf; bx[3 + k] = -inf; }
      for (int e = T.first + beg; e < T.first + beg + len; ++e) {  // calcBox
        const float4 a = A[e], b = B[e];
        bx[0] = gmin(bx[0], a.x); bx[1] = gmin(bx[1], a.y); bx[2] = gmin(bx[2], a.z);
        bx[3] = gmax(bx[3], b.x); bx[4] = gmax(bx[4], b.y); bx[5] = gmax(bx[5], b.z);
      }
      nd.children[c] = encode_leaf((uint32_t)(T.first + beg), (uint32_t)len);
    } else {
      const int ch = T.child[c];
      for (int k = 0; k < 6; ++k) bx[k] = nbox[(size_t)ch * 6 + k];
      nd.children[c] = id[ch];
    }
    for (int k = 0; k < 3; ++k) {
      nd.boxes[c + 4 * k] = bx[k];
      nd.boxes[c + 12 + 4 * k] = bx[3 + k];
    }
    if (nd.children[c] != -1)
      for (int k = 0; k < 3; ++k) { u[k] = gmin(u[k], bx[k]); u[3 + k] = gmax(u[3 + k], bx[3 + k]); }
  }
  for (int k = 0; k < 6; ++k) nbox[(size_t)t * 6 + k] = u[k];
  nodes[id[t]] = nd;
}

// Motion topology (qbvh.MotionNode): axes and children; parent stays 0.
__global__ void k_mnodes(const BTask* __restrict__ tasks, int count, const int* __restrict__ id, vmr_mqbvh_node* nodes) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const BTask& T = tasks[t];
  vmr_mqbvh_node nd;
  memset(&nd, 0, sizeof(nd));
  nd.axis0 = T.axes & 3;
  nd.axis1 = (T.axes >> 2) & 3;
  nd.axis2 = (T.axes >> 4) & 3;
  for (int c = 0; c < 4; ++c) {
    int beg, len;
    child_range(T, c, beg, len);
    nd.children[c] = len == 0 ? -1 : (len <= kLeafMax ? encode_leaf((uint32_t)(T.first + beg), (uint32_t)len) : id[T.child[c]]);
  }
  nodes[id[t]] = nd;
}

// Per-key motion boxes, deepest level first (buildqbvh.go:159-212): leaf
// boxes grown over the leaf faces' vertices at the key, inner boxes the
// union of the child's children; empty children keep a zero box.
__global__ void k_mboxes(const BTask* __restrict__ tasks, int t0, int count, const int* __restrict__ id,
                         const float4* __restrict__ A, const float* __restrict__ verts,
                         const uint32_t* __restrict__ idxp, uint32_t n_verts, uint32_t key, uint32_t n_nodes,
                         float* nbox, float* mboxes) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int t = t0 + i;
  const BTask& T = tasks[t];
  const float inf = __int_as_float(0x7f800000);
  float* out = mboxes + ((size_t)key * n_nodes + id[t]) * 24;
  float u[6] = {inf, inf, inf, -inf, -inf, -inf};
  for (int c = 0; c < 4; ++c) {
    int beg, len;
    child_range(T, c, beg, len);
    if (len == 0) continue;
    float bx[6];
    if (len <= kLeafMax) {
      for (int k = 0; k < 3; ++k) { bx[k] = inf; bx[3 + k] = -inf; }
      for (int e = T.first + beg; e < T.first + beg + len; ++e) {
        const uint32_t face = (uint32_t)__float_as_int(A[e].w);
        for (int j = 0; j < 3; ++j) {
          const float* v = verts + ((size_t)key * n_verts + idxp[(size_t)face * 3 + j]) * 3;
          for (int k = 0; k < 3; ++k) { bx[k] = gmin(v[k], bx[k]); bx[3 + k] = gmax(v[k], bx[3 + k]); }
        }
      }
    } else {
      for (int k = 0; k < 6; ++k) bx[k] = nbox[(size_t)T.child[c] * 6 + k];
    }
    for (int k = 0; k < 3; ++k) {
      out[c + 4 * k] = bx[k];
      out[c + 12 + 4 * k] = bx[3 + k];
    }
    for (int k = 0; k < 3; ++k) { u[k] = gmin(u[k], bx[k]); u[3 + k] = gmax(u[3 + k], bx[3 + k]); }
  }
  for (int k = 0; k < 6; ++k) nbox[(size_t)t * 6 + k] = u[k];
}

// Leaf order: accel idx, idxp and the device triangle table of a static mesh.
__global__ void k_leaf_order(const float4* __restrict__ A, const uint32_t* __restrict__ idxp,
                             const float* __restrict__ verts, int n, int static_mesh, int32_t* accel,
                             uint32_t* leaf_idxp, float4* tris) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int face = __float_as_int(A[i].w);
  accel[i] = face;
  if (!static_mesh) return;
  for (int j = 0; j < 3; ++j) {
    const uint32_t vi = idxp[(size_t)face * 3 + j];
    leaf_idxp[(size_t)i * 3 + j] = vi;
    const float* v = verts + (size_t)vi * 3;
    tris[(size_t)i * 3 + j] = make_float4(v[0], v[1], v[2], 0.0f);
  }
}

int blocks(long n, int bs) { return (int)((n + bs - 1) / bs); }

template <int BS, int CL>
cudaError_t launch_cluster_level(const Bufs& b, int t0, int count, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(count * CL));
  cfg.blockDim = dim3(BS);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (CL > 8) {
    cudaError_t e = cudaFuncSetAttribute(k_build_level<BS, CL>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  return cudaLaunchKernelEx(&cfg, k_build_level<BS, CL>, b, t0);
}

// Team shape per level: clusters of 16 and 8 CTAs for the few large nodes of
// the upper levels, one CTA per node below.
cudaError_t launch_level(const Bufs& b, int t0, int count, cudaStream_t s) {
  if (count <= 2) {
    int clusters = 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(512);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 16;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    // 16-CTA clusters where the device schedules them, else 8
    if (cudaFuncSetAttribute(k_build_level<512, 16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess &&
        cudaOccupancyMaxActiveClusters(&clusters, k_build_level<512, 16>, &cfg) == cudaSuccess && clusters > 0)
      return launch_cluster_level<512, 16>(b, t0, count, s);
    cudaGetLastError();
    return launch_cluster_level<512, 8>(b, t0, count, s);
  }
  if (count <= 64) return launch_cluster_level<512, 8>(b, t0, count, s);
  k_build_level<128, 1><<<count, 128, 0, s>>>(b, t0);
  return cudaGetLastError();
}

}  // namespace

int device_build_mesh(HostMesh& m, DevBuf& tris_out, cudaStream_t s, std::string& err) {
  const int n = (int)m.n_tris;
  if (n == 0) return kBuildDeclined;
  const bool motion = m.keys > 1;
  const size_t nv = (size_t)m.n_verts * m.keys * 3;
  const int cap = n / 2 + 4 * kMaxLevels + 16;
  // One allocation for the build's working set.
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
  const size_t o_verts = take(nv * 4), o_idxp = take((size_t)n * 12), o_abc = take((size_t)n * 16 * 6),
               o_sw = take((size_t)n * 4), o_rk = take((size_t)n * 4), o_tasks = take((size_t)cap * sizeof(BTask)),
               o_size = take((size_t)cap * 4), o_id = take((size_t)cap * 4), o_nbox = take((size_t)cap * 24),
               o_cnt = take(8), o_accel = take((size_t)n * 4), o_lidx = take((size_t)n * 12);
  DevBuf work;
  if (work.ensure(off) != cudaSuccess) { err = "device build: out of memory"; return kBuildError; }
  char* base = work.as<char>();
  float* d_verts = (float*)(base + o_verts);
  uint32_t* d_idxp = (uint32_t*)(base + o_idxp);
  Bufs b;
  b.A = (float4*)(base + o_abc);
  b.B = b.A + n; b.C = b.B + n; b.TA = b.C + n; b.TB = b.TA + n; b.TC = b.TB + n;
  b.sw = (int*)(base + o_sw);
  b.rk = (int*)(base + o_rk);
  b.tasks = (BTask*)(base + o_tasks);
  b.n_tasks = (int*)(base + o_cnt);
  b.err = b.n_tasks + 1;
  b.cap = cap;
  int* d_size = (int*)(base + o_size);
  int* d_id = (int*)(base + o_id);
  float* d_nbox = (float*)(base + o_nbox);
  int32_t* d_accel = (int32_t*)(base + o_accel);
  uint32_t* d_lidx = (uint32_t*)(base + o_lidx);

#define VB_CHECK(call)                                                                  \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) { err = std::string("device build: ") + cudaGetErrorString(e_); return kBuildError; } \
  } while (0)

  VB_CHECK(cudaMemcpyAsync(d_verts, m.verts.data(), nv * 4, cudaMemcpyHostToDevice, s));
  VB_CHECK(cudaMemcpyAsync(d_idxp, m.idxp.data(), (size_t)n * 12, cudaMemcpyHostToDevice, s));
  BTask root{};
  root.first = 0;
  root.n = n;
  root.child[0] = root.child[1] = root.child[2] = root.child[3] = -1;
  const int init[2] = {1, 0};
  VB_CHECK(cudaMemcpyAsync(b.tasks, &root, sizeof(root), cudaMemcpyHostToDevice, s));
  VB_CHECK(cudaMemcpyAsync(b.n_tasks, init, sizeof(init), cudaMemcpyHostToDevice, s));
  const float kf = 0.5f * (float)(m.keys - 1);
  const float tt = kf - std::floor(kf);
  const uint32_t ka = (uint32_t)std::floor(kf), kb = (uint32_t)std::ceil(kf);
  k_prep<<<blocks(n, 256), 256, 0, s>>>(d_verts, d_idxp, n, m.n_verts, motion ? 1 : 0, ka, kb, tt, b.A, b.B, b.C,
                                        b.err);
  VB_CHECK(cudaGetLastError());
  int hc[2] = {0, 0};
  VB_CHECK(cudaMemcpyAsync(hc, b.n_tasks, sizeof(hc), cudaMemcpyDeviceToHost, s));
  VB_CHECK(cudaStreamSynchronize(s));
  if (hc[1] & kErrNonFinite) return kBuildDeclined;

  std::vector<std::pair<int, int>> levels;
  int lb = 0, le = 1;
  while (lb < le) {
    if ((int)levels.size() >= kMaxLevels) { err = "QBVH build recursion does not terminate"; return kBuildError; }
    const int count = le - lb;
    VB_CHECK(launch_level(b, lb, count, s));
    VB_CHECK(cudaMemcpyAsync(hc, b.n_tasks, sizeof(hc), cudaMemcpyDeviceToHost, s));
    VB_CHECK(cudaStreamSynchronize(s));
    if (hc[1] & kErrBin) { err = "QBVH build: centroid bin out of range"; return kBuildError; }
    if (hc[1] & kErrPartition) { err = "device build: partition check failed"; return kBuildError; }
    if (hc[1] & kErrCapacity) return kBuildDeclined;
    levels.emplace_back(lb, le);
    lb = le;
    le = hc[0];
  }
  const int n_nodes = le;
  // Pre-order numbering.
  for (int L = (int)levels.size() - 1; L >= 0; --L) {
    const int c = levels[L].second - levels[L].first;
    k_sizes<<<blocks(c, 128), 128, 0, s>>>(b.tasks, levels[L].first, c, d_size);
  }
  VB_CHECK(cudaMemsetAsync(d_id, 0, sizeof(int), s));
  for (size_t L = 0; L < levels.size(); ++L) {
    const int c = levels[L].second - levels[L].first;
    k_ids<<<blocks(c, 128), 128, 0, s>>>(b.tasks, levels[L].first, c, d_size, d_id);
  }
  VB_CHECK(cudaGetLastError());
  // the device triangle table of a static mesh (upload_mesh's layout) is
  // written here rather than gathered on the host
  if (!motion) VB_CHECK(tris_out.ensure((size_t)n * 3 * 16));
  k_leaf_order<<<blocks(n, 256), 256, 0, s>>>(b.A, d_idxp, d_verts, n, motion ? 0 : 1, d_accel, d_lidx,
                                              motion ? nullptr : tris_out.as<float4>());
  VB_CHECK(cudaGetLastError());
  m.accel_idx.resize(n);
  VB_CHECK(cudaMemcpyAsync(m.accel_idx.data(), d_accel, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
  const float inf = __builtin_huge_valf();
  if (!motion) {
    DevBuf dn;
    VB_CHECK(dn.ensure((size_t)n_nodes * sizeof(vmr_qbvh_node)));
    for (int L = (int)levels.size() - 1; L >= 0; --L) {
      const int c = levels[L].second - levels[L].first;
      k_nodes<<<blocks(c, 128), 128, 0, s>>>(b.tasks, levels[L].first, c, d_id, b.A, b.B, d_nbox,
                                             dn.as<vmr_qbvh_node>());
    }
    VB_CHECK(cudaGetLastError());
    m.nodes.resize(n_nodes);
    std::vector<uint32_t> lidx((size_t)n * 3);
    float rb[6];
    VB_CHECK(cudaMemcpyAsync(m.nodes.data(), dn.p, (size_t)n_nodes * sizeof(vmr_qbvh_node), cudaMemcpyDeviceToHost, s));
    VB_CHECK(cudaMemcpyAsync(lidx.data(), d_lidx, (size_t)n * 12, cudaMemcpyDeviceToHost, s));
    VB_CHECK(cudaMemcpyAsync(rb, d_nbox, sizeof(rb), cudaMemcpyDeviceToHost, s));  // the root's union
    VB_CHECK(cudaStreamSynchronize(s));
    m.idxp.swap(lidx);
    for (int k = 0; k < 3; ++k) { m.bounds.lo[k] = rb[k]; m.bounds.hi[k] = rb[3 + k]; }
    if (!m.shader_idx.empty()) {
      std::vector<uint8_t> sidx(n);
      for (int i = 0; i < n; ++i) sidx[i] = m.shader_idx[m.accel_idx[i]];
      m.shader_idx.swap(sidx);
    }
    return kBuildOk;
  }
  DevBuf dn, db;
  VB_CHECK(dn.ensure((size_t)n_nodes * sizeof(vmr_mqbvh_node)));
  VB_CHECK(db.ensure((size_t)m.keys * n_nodes * 24 * 4));
  VB_CHECK(cudaMemsetAsync(db.p, 0, (size_t)m.keys * n_nodes * 24 * 4, s));
  k_mnodes<<<blocks(n_nodes, 128), 128, 0, s>>>(b.tasks, n_nodes, d_id, dn.as<vmr_mqbvh_node>());
  m.key_bounds.assign(m.keys, Bounds{});
  std::vector<float> kbs((size_t)m.keys * 6);
  for (uint32_t key = 0; key < m.keys; ++key) {
    for (int L = (int)levels.size() - 1; L >= 0; --L) {
      const int c = levels[L].second - levels[L].first;
      k_mboxes<<<blocks(c, 128), 128, 0, s>>>(b.tasks, levels[L].first, c, d_id, b.A, d_verts, d_idxp, m.n_verts,
                                              key, (uint32_t)n_nodes, d_nbox, db.as<float>());
    }
    VB_CHECK(cudaMemcpyAsync(&kbs[(size_t)key * 6], d_nbox, 24, cudaMemcpyDeviceToHost, s));
  }
  VB_CHECK(cudaGetLastError());
  m.mnodes.resize(n_nodes);
  m.mboxes.resize((size_t)m.keys * n_nodes * 24);
  VB_CHECK(cudaMemcpyAsync(m.mnodes.data(), dn.p, (size_t)n_nodes * sizeof(vmr_mqbvh_node), cudaMemcpyDeviceToHost, s));
  VB_CHECK(cudaMemcpyAsync(m.mboxes.data(), db.p, m.mboxes.size() * 4, cudaMemcpyDeviceToHost, s));
  VB_CHECK(cudaStreamSynchronize(s));
  Bounds full{{inf, inf, inf}, {-inf, -inf, -inf}};
  for (uint32_t key = 0; key < m.keys; ++key) {
    Bounds& kb2 = m.key_bounds[key];
    for (int k = 0; k < 3; ++k) { kb2.lo[k] = kbs[key * 6 + k]; kb2.hi[k] = kbs[key * 6 + 3 + k]; }
    for (int k = 0; k < 3; ++k) {  // BoundingBox.GrowBox
      full.lo[k] = full.lo[k] < kb2.lo[k] ? full.lo[k] : kb2.lo[k];
      full.hi[k] = full.hi[k] > kb2.hi[k] ? full.hi[k] : kb2.hi[k];
    }
  }
  m.bounds = full;
  return kBuildOk;
#undef VB_CHECK
}

}  // namespace vmr
