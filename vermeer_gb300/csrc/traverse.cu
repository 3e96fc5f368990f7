// traverse.cu - QBVH traversal and watertight ray/triangle kernels (sm_103a).
//
// Bit-exactness contract: for the same QBVH and rays, the hit element id, t
// and barycentrics equal those of the reference's qbvh.Trace +
// PolyMesh.TraceElems (qbvh/intersect.go:91-246, qbvh/intersect_amd64.s,
// builtin/geom/polymesh/trace.go:108-194), motion traversal
// (qbvh/motionintersect.go:22-127, trace.go:520-719) and the two-level scene
// (builtin/scene/scene.go:30-97).  To get there:
//   * every float operation of the box and triangle tests is an explicit
//     round-to-nearest intrinsic (__fadd_rn/__fsub_rn/__fmul_rn never fuse
//     into FMA), in the reference's operation order;
//   * divisions are IEEE (__fdiv_rn/__frcp_rn), which equal the reference's
//     float32(float64(a)/float64(b));
//   * the FP64 edge fallback is kept (__dmul_rn/__dsub_rn/__double2float_rn);
//   * children are visited in the reference's order, pops are culled with
//     the reference's test (Tclosest < T), leaves are scanned in order.
// The traversal may skip work the reference does without effect: children
// that would be culled when popped are never pushed, and the child popped
// next stays in registers instead of a stack round trip.
//
// Execution model: persistent warps (grid = SMs x resident blocks) pull
// rays from a global counter with one warp-aggregated atomic per refill;
// each lane owns one ray and a private stack in local memory (L1-resident,
// interleaved per lane by the hardware so same-depth accesses coalesce).
// The while-while kernels alternate a warp-synchronous node walk with a
// leaf phase in which the warp scans all its lanes' leaves as one list of
// (ray, triangle) tests.  Kernels: k_trace_mesh_ww (one mesh, static or
// motion), k_trace_scene_ww (two-level scenes, and job mode: each ray enters
// its own mesh), k_trace_mesh_sched and k_trace_scene (the step-scheduled
// and single-loop kernels the tuning can select), k_jobs_gather and
// k_jobs_scatter (vmr_trace_jobs).
#include <cuda_runtime.h>

#include "device.h"

namespace vmr {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float pick3(float x, float y, float z, int k) {
  return k == 0 ? x : (k == 1 ? y : z);
}

// Traversal inputs of core.Ray after Ray.Setup (core/ray.go:103-148).
struct TRay {
  float ox, oy, oz;
  float dx, dy, dz;
  float ix, iy, iz;     // Dinv
  float tclosest;       // Tclosest
  float s0, s1, s2;     // S
  float pkx, pky, pkz;  // P[Kx], P[Ky], P[Kz]
  int kx, ky, kz;
  unsigned oct;         // bit k set when D[k] < 0
  int cls;              // 2*Kz + (D[Kz] < 0): selects (Kx, Ky, Kz)
  bool exact;           // a NaN can arise in the slab test
  float time;
};

__device__ __forceinline__ void ray_setup(TRay& r) {
  float ax = fabsf(r.dx), ay = fabsf(r.dy), az = fabsf(r.dz);
  int kz = 0;
  if (ay > az) {
    if (ay > ax) kz = 1;
  } else {
    if (az > ax) kz = 2;
  }
  int kx = kz + 1;
  if (kx == 3) kx = 0;
  int ky = kx + 1;
  if (ky == 3) ky = 0;
  float dkz = pick3(r.dx, r.dy, r.dz, kz);
  if (dkz < 0.0f) { int t = kx; kx = ky; ky = t; }
  r.kx = kx; r.ky = ky; r.kz = kz;
  r.cls = 2 * kz + (dkz < 0.0f ? 1 : 0);
  r.s2 = __frcp_rn(dkz);
  r.s0 = __fdiv_rn(pick3(r.dx, r.dy, r.dz, kx), dkz);
  r.s1 = __fdiv_rn(pick3(r.dx, r.dy, r.dz, ky), dkz);
  r.ix = __frcp_rn(r.dx);
  r.iy = __frcp_rn(r.dy);
  r.iz = __frcp_rn(r.dz);
  r.pkx = pick3(r.ox, r.oy, r.oz, kx);
  r.pky = pick3(r.ox, r.oy, r.oz, ky);
  r.pkz = pick3(r.ox, r.oy, r.oz, kz);
  r.oct = (r.dx < 0.0f ? 1u : 0u) | (r.dy < 0.0f ? 2u : 0u) | (r.dz < 0.0f ? 4u : 0u);
  // (b - o) * Dinv can only be NaN when Dinv is infinite or zero or an
  // input is not finite; otherwise the ternary min/max of the reference
  // and fminf/fmaxf agree (up to the sign of zero, which no comparison sees).
  r.exact = !(isfinite(r.ix) && isfinite(r.iy) && isfinite(r.iz) && r.ix != 0.0f && r.iy != 0.0f &&
              r.iz != 0.0f && isfinite(r.ox) && isfinite(r.oy) && isfinite(r.oz));
}

// Slab test of the 4 children against boxes b[6] (intersect_amd64.s).
// Returns the 4-bit hit mask, tNear per child in tn[].
template <bool EXACT>
__device__ __forceinline__ unsigned box4(const TRay& r, const float4 (&b)[6], float (&tn)[4]) {
  unsigned mask = 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float bminx = (&b[0].x)[c], bminy = (&b[1].x)[c], bminz = (&b[2].x)[c];
    const float bmaxx = (&b[3].x)[c], bmaxy = (&b[4].x)[c], bmaxz = (&b[5].x)[c];
    float x1 = __fmul_rn(__fsub_rn(bminx, r.ox), r.ix);
    float x2 = __fmul_rn(__fsub_rn(bmaxx, r.ox), r.ix);
    float y1 = __fmul_rn(__fsub_rn(bminy, r.oy), r.iy);
    float y2 = __fmul_rn(__fsub_rn(bmaxy, r.oy), r.iy);
    float z1 = __fmul_rn(__fsub_rn(bminz, r.oz), r.iz);
    float z2 = __fmul_rn(__fsub_rn(bmaxz, r.oz), r.iz);
    float lo, hi;
    if (EXACT) {
      // MINPS/MAXPS operand order: the second source wins unless the first
      // compares strictly smaller/larger, so a NaN propagates as the SSE
      // code does.
      lo = x2 < x1 ? x2 : x1;
      hi = x2 > x1 ? x2 : x1;
      float ylo = y2 < y1 ? y2 : y1, yhi = y2 > y1 ? y2 : y1;
      lo = lo > ylo ? lo : ylo;
      hi = hi < yhi ? hi : yhi;
      float zlo = z2 < z1 ? z2 : z1, zhi = z2 > z1 ? z2 : z1;
      lo = lo > zlo ? lo : zlo;
      hi = hi < zhi ? hi : zhi;
      float t = 0.0f > lo ? 0.0f : lo;
      tn[c] = t;
      if (t <= hi) mask |= 1u << c;
    } else {
      lo = fmaxf(fmaxf(fminf(x1, x2), fminf(y1, y2)), fminf(z1, z2));
      hi = fminf(fminf(fmaxf(x1, x2), fmaxf(y1, y2)), fmaxf(z1, z2));
      float t = fmaxf(0.0f, lo);
      tn[c] = t;
      if (t <= hi) mask |= 1u << c;
    }
  }
  return mask;
}

// L1 prefetch hints (no register result).  Only issued for addresses inside
// the node and triangle arrays.
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}
// The lines holding triangles [first, first+count) (48 bytes each).
__device__ __forceinline__ void prefetch_leaf(const float4* tris, uint32_t first, uint32_t count) {
  const char* a = reinterpret_cast<const char*>(tris + 3 * (size_t)first);
  const char* e = reinterpret_cast<const char*>(tris + 3 * (size_t)(first + count));
  for (const char* q = reinterpret_cast<const char*>((uintptr_t)a & ~(uintptr_t)127); q < e; q += 128) prefetch_l1(q);
}

// Result of the accepted triangle (ShaderContext fields the trace fills).
struct HitRec {
  int32_t elem;
  int32_t geom;
  float u, v, w;
};

// Component k of a vertex: compile-time for a known permutation class,
// selected at run time otherwise (C < 0).
template <int C>
struct Perm {
  static constexpr int KZ = C >> 1;
  static constexpr int KX0 = (KZ + 1) % 3;
  static constexpr int KY0 = (KX0 + 1) % 3;
  static constexpr int KX = (C & 1) ? KY0 : KX0;
  static constexpr int KY = (C & 1) ? KX0 : KY0;
};
template <int K>
__device__ __forceinline__ float comp(const float4& v) {
  return K == 0 ? v.x : (K == 1 ? v.y : v.z);
}
template <int C, int AXIS>  // AXIS: 0 = Kx, 1 = Ky, 2 = Kz
__device__ __forceinline__ float kcomp(const TRay& r, const float4& v) {
  if constexpr (C >= 0) {
    return comp<AXIS == 0 ? Perm<C>::KX : (AXIS == 1 ? Perm<C>::KY : Perm<C>::KZ)>(v);
  } else {
    return pick3(v.x, v.y, v.z, AXIS == 0 ? r.kx : (AXIS == 1 ? r.ky : r.kz));
  }
}

// The watertight test (trace.go:123-193), in two parts.  tri_prepare: the
// part that does not depend on Tclosest (edge functions with the FP64
// fallback, the sign test, det, T and the lower bound); false when the
// triangle cannot be hit at any Tclosest.  STRICT: static idxp path
// (xT < lower*xdet); otherwise the motion path (xT <= lower*xdet).
template <bool STRICT, int C = -1>
__device__ __forceinline__ bool tri_prepare(const TRay& r, float4 v0, float4 v1, float4 v2, float lower, float& fU,
                                            float& fV, float& fW, float& det, float& T) {
  const float AKz = __fsub_rn(kcomp<C, 2>(r, v0), r.pkz);
  const float BKz = __fsub_rn(kcomp<C, 2>(r, v1), r.pkz);
  const float CKz = __fsub_rn(kcomp<C, 2>(r, v2), r.pkz);
  const float Cx = __fsub_rn(__fsub_rn(kcomp<C, 0>(r, v2), r.pkx), __fmul_rn(r.s0, CKz));
  const float By = __fsub_rn(__fsub_rn(kcomp<C, 1>(r, v1), r.pky), __fmul_rn(r.s1, BKz));
  const float Cy = __fsub_rn(__fsub_rn(kcomp<C, 1>(r, v2), r.pky), __fmul_rn(r.s1, CKz));
  const float Bx = __fsub_rn(__fsub_rn(kcomp<C, 0>(r, v1), r.pkx), __fmul_rn(r.s0, BKz));
  const float Ax = __fsub_rn(__fsub_rn(kcomp<C, 0>(r, v0), r.pkx), __fmul_rn(r.s0, AKz));
  const float Ay = __fsub_rn(__fsub_rn(kcomp<C, 1>(r, v0), r.pky), __fmul_rn(r.s1, AKz));
  fU = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
  fV = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
  fW = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
  if (fU == 0.0f || fV == 0.0f || fW == 0.0f) {
    // FP64 fallback (trace.go:142-155): exact products, one rounding in the
    // double subtraction, one in the conversion.
    fU = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx)));
    fV = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx)));
    fW = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax)));
  }
  if ((fU < 0.0f || fV < 0.0f || fW < 0.0f) && (fU > 0.0f || fV > 0.0f || fW > 0.0f)) return false;
  det = __fadd_rn(__fadd_rn(fU, fV), fW);
  if (det == 0.0f) return false;
  T = __fmul_rn(r.s2, __fadd_rn(__fadd_rn(__fmul_rn(fU, AKz), __fmul_rn(fV, BKz)), __fmul_rn(fW, CKz)));
  const unsigned sgn = __float_as_uint(det) & 0x80000000u;
  const float xT = __uint_as_float(__float_as_uint(T) ^ sgn);
  const float xdet = __uint_as_float(__float_as_uint(det) ^ sgn);
  const float lo = __fmul_rn(lower, xdet);
  return !(STRICT ? (xT < lo) : (xT <= lo));
}

// The Tclosest test and the hit update of a prepared triangle.
__device__ __forceinline__ bool tri_accept(TRay& r, float fU, float fV, float fW, float det, float T, float& U,
                                           float& V, float& W) {
  const unsigned sgn = __float_as_uint(det) & 0x80000000u;
  const float xT = __uint_as_float(__float_as_uint(T) ^ sgn);
  const float xdet = __uint_as_float(__float_as_uint(det) ^ sgn);
  if (xT > __fmul_rn(r.tclosest, xdet)) return false;
  const float rcp = __frcp_rn(det);
  U = __fmul_rn(fU, rcp);
  V = __fmul_rn(fV, rcp);
  W = __fmul_rn(fW, rcp);
  r.tclosest = __fmul_rn(T, rcp);
  return true;
}

template <bool STRICT, int C = -1>
__device__ __forceinline__ bool tri_test(TRay& r, float4 v0, float4 v1, float4 v2, float lower, float& U,
                                         float& V, float& W) {
  float fU, fV, fW, det, T;
  if (!tri_prepare<STRICT, C>(r, v0, v1, v2, lower, fU, fV, fW, det, T)) return false;
  return tri_accept(r, fU, fV, fW, det, T, U, V, W);
}

struct Counters {
  uint32_t nodes, leafs, tris;
};

__device__ __forceinline__ void leaf_decode(int32_t c, uint32_t& first, uint32_t& count) {
  first = ((uint32_t)c & 0x7fffffffu) >> 4;
  count = ((uint32_t)c & 15u) + 1u;
}

// Push-order rank of each child (intersect.go:137-216): pairs (0,1) and
// (2,3) each ordered by the sign of D along their split axis, the pair
// order by the sign of D[Axis0].  Rank 0 is pushed first (popped last).
__device__ __forceinline__ void child_ranks(unsigned axes, unsigned oct, unsigned (&rk)[4]) {
  const unsigned s0 = (oct >> (axes & 3u)) & 1u;
  const unsigned s1 = (oct >> ((axes >> 2) & 3u)) & 1u;
  const unsigned s2 = (oct >> ((axes >> 4) & 3u)) & 1u;
  rk[0] = 2u * (1u - s0) + (1u - s1);
  rk[1] = 2u * (1u - s0) + s1;
  rk[2] = 2u * s0 + (1u - s2);
  rk[3] = 2u * s0 + s2;
}

// Push the hit children of a node in the reference order.  The child that
// would be popped first is returned in (next, nextT) instead of being
// stored.  Returns false when there is no child to visit.
__device__ __forceinline__ bool push_children(int2* stk, int& sp, int cap, unsigned mask, const int4& ch,
                                              const float (&tn)[4], unsigned axes, unsigned oct, int& next,
                                              float& nextT, int& status) {
  if (mask == 0) return false;
  unsigned rk[4];
  child_ranks(axes, oct, rk);
  unsigned rmask = 0;
#pragma unroll
  for (int c = 0; c < 4; ++c)
    if (mask & (1u << c)) rmask |= 1u << rk[c];
  const unsigned rtop = 31u - __clz(rmask);
  const int npush = __popc(rmask) - 1;
  if (sp + npush > cap) {
    status = kStatusStackOverflow;
    return false;
  }
  const int chv[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    if (mask & (1u << c)) {
      if (rk[c] == rtop) {
        next = chv[c];
        nextT = tn[c];
      } else {
        const int slot = sp + __popc(rmask & ((1u << rk[c]) - 1u));
        stk[slot] = make_int2(chv[c], __float_as_int(tn[c]));
      }
    }
  }
  sp += npush;
  return true;
}

// qbvh.Trace over a static mesh (intersect.go:91-246) with
// PolyMesh.TraceElems at the leaves.  Returns true if some leaf accepted a
// triangle.  stk/cap: the free part of the ray's stack.
template <bool ANY, bool COUNT>
__device__ bool trace_static(const DMesh& m, TRay& r, int2* stk, int cap, HitRec& h, Counters& cnt,
                             int& status) {
  const uint32_t CAP = m.iter_cap;
  const float4* __restrict__ tris = reinterpret_cast<const float4*>(m.tris);
  bool hit = false;
  int sp = 0;
  int node = 0;
  float nodeT = r.tclosest;
  for (uint32_t iter = 0;; ++iter) {
    if (iter >= CAP) { status = kStatusIterationCap; break; }
    if (!(r.tclosest < nodeT) && node != kEmptyChild) {
      if (node >= 0) {
        if (COUNT) cnt.nodes++;
        const float4* nb = reinterpret_cast<const float4*>(m.nodes + node);
        float4 b[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) b[k] = __ldg(nb + k);
        const int4 ch = __ldg(reinterpret_cast<const int4*>(nb + 6));
        const unsigned axes = __ldg(reinterpret_cast<const unsigned*>(nb + 7));
        float tn[4];
        unsigned mask = r.exact ? box4<true>(r, b, tn) : box4<false>(r, b, tn);
        // Children culled at pop time in the reference are dropped here.
        if (ch.x == kEmptyChild || r.tclosest < tn[0]) mask &= ~1u;
        if (ch.y == kEmptyChild || r.tclosest < tn[1]) mask &= ~2u;
        if (ch.z == kEmptyChild || r.tclosest < tn[2]) mask &= ~4u;
        if (ch.w == kEmptyChild || r.tclosest < tn[3]) mask &= ~8u;
        int next;
        float nextT;
        if (push_children(stk, sp, cap, mask, ch, tn, axes, r.oct, next, nextT, status)) {
          node = next;
          nodeT = nextT;
          continue;
        }
        if (status != kStatusOk) break;
      } else {
        uint32_t first, count;
        leaf_decode(node, first, count);
        if (COUNT) { cnt.leafs++; cnt.tris += count; }
        int32_t idx = -1;
        float U = 0.f, V = 0.f, W = 0.f;
        for (uint32_t i = first; i < first + count; ++i) {
          const float4 v0 = __ldg(tris + 3 * (size_t)i);
          const float4 v1 = __ldg(tris + 3 * (size_t)i + 1);
          const float4 v2 = __ldg(tris + 3 * (size_t)i + 2);
          if (tri_test<true>(r, v0, v1, v2, m.lower_static, U, V, W)) idx = (int32_t)i;
        }
        if (idx != -1) {
          h.elem = idx;
          h.u = U; h.v = V; h.w = W;
          hit = true;
          if (ANY) break;
        }
      }
    }
    if (sp == 0) break;
    --sp;
    const int2 e = stk[sp];
    node = e.x;
    nodeT = __int_as_float(e.y);
  }
  return hit;
}

// qbvh.TraceMotion (motionintersect.go:22-127) with TraceMotionElems
// (trace.go:520-719): per-key boxes and vertices lerped with the ray's time.
template <bool ANY, bool COUNT>
__device__ bool trace_motion(const DMesh& m, TRay& r, int2* stk, int cap, HitRec& h, Counters& cnt,
                             int& status) {
  const uint32_t CAP = m.iter_cap;
  // k = Time*float32(keys-1); time = k - Floor(k); key = Floor, key2 = Ceil
  const float k = __fmul_rn(r.time, (float)(m.keys - 1));
  const float fk = floorf(k);
  const float tm = __fsub_rn(k, fk);
  const int key = (int)fk, key2 = (int)ceilf(k);
  if (key < 0 || key2 >= (int)m.keys) return false;  // the reference indexes out of range here
  const float omt = __fsub_rn(1.0f, tm);
  const float4* __restrict__ bx0 = reinterpret_cast<const float4*>(m.mboxes) + (size_t)key * m.n_mnodes * 6;
  const float4* __restrict__ bx1 = reinterpret_cast<const float4*>(m.mboxes) + (size_t)key2 * m.n_mnodes * 6;
  const float4* __restrict__ t0 = reinterpret_cast<const float4*>(m.mtris) + (size_t)key * m.n_tris * 3;
  const float4* __restrict__ t1 = reinterpret_cast<const float4*>(m.mtris) + (size_t)key2 * m.n_tris * 3;
  bool hit = false;
  int sp = 0;
  int node = 0;
  float nodeT = r.tclosest;
  for (uint32_t iter = 0;; ++iter) {
    if (iter >= CAP) { status = kStatusIterationCap; break; }
    if (!(r.tclosest < nodeT) && node != kEmptyChild) {
      if (node >= 0) {
        if (COUNT) cnt.nodes++;
        float4 b[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          const float4 a = __ldg(bx0 + (size_t)node * 6 + q);
          const float4 c = __ldg(bx1 + (size_t)node * 6 + q);
          // (1.0-time)*Boxes[key] + time*Boxes[key2] (motionintersect.go:47-49)
          b[q].x = __fadd_rn(__fmul_rn(omt, a.x), __fmul_rn(tm, c.x));
          b[q].y = __fadd_rn(__fmul_rn(omt, a.y), __fmul_rn(tm, c.y));
          b[q].z = __fadd_rn(__fmul_rn(omt, a.z), __fmul_rn(tm, c.z));
          b[q].w = __fadd_rn(__fmul_rn(omt, a.w), __fmul_rn(tm, c.w));
        }
        const int4 ch = __ldg(reinterpret_cast<const int4*>(m.mnodes + node));
        const unsigned axes = __ldg(reinterpret_cast<const unsigned*>(m.mnodes + node) + 4);
        float tn[4];
        unsigned mask = r.exact ? box4<true>(r, b, tn) : box4<false>(r, b, tn);
        if (ch.x == kEmptyChild || r.tclosest < tn[0]) mask &= ~1u;
        if (ch.y == kEmptyChild || r.tclosest < tn[1]) mask &= ~2u;
        if (ch.z == kEmptyChild || r.tclosest < tn[2]) mask &= ~4u;
        if (ch.w == kEmptyChild || r.tclosest < tn[3]) mask &= ~8u;
        int next;
        float nextT;
        if (push_children(stk, sp, cap, mask, ch, tn, axes, r.oct, next, nextT, status)) {
          node = next;
          nodeT = nextT;
          continue;
        }
        if (status != kStatusOk) break;
      } else {
        uint32_t first, count;
        leaf_decode(node, first, count);
        if (COUNT) { cnt.leafs++; cnt.tris += count; }
        int32_t idx = -1;
        float U = 0.f, V = 0.f, W = 0.f;
        for (uint32_t i = first; i < first + count; ++i) {
          float4 v[3];
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const float4 a = __ldg(t0 + 3 * (size_t)i + j);
            const float4 c = __ldg(t1 + 3 * (size_t)i + j);
            // Vec3Lerp (math/vec3.go:52-58)
            v[j].x = __fadd_rn(__fmul_rn(omt, a.x), __fmul_rn(tm, c.x));
            v[j].y = __fadd_rn(__fmul_rn(omt, a.y), __fmul_rn(tm, c.y));
            v[j].z = __fadd_rn(__fmul_rn(omt, a.z), __fmul_rn(tm, c.z));
            v[j].w = 0.0f;
          }
          if (tri_test<false>(r, v[0], v[1], v[2], m.ray_bias, U, V, W)) idx = (int32_t)i;
        }
        if (idx != -1) {
          h.elem = __ldg(m.elem + idx);
          h.u = U; h.v = V; h.w = W;
          hit = true;
          if (ANY) break;
        }
      }
    }
    if (sp == 0) break;
    --sp;
    const int2 e = stk[sp];
    node = e.x;
    nodeT = __int_as_float(e.y);
  }
  return hit;
}

// Sphere.Trace with raySphereIntersect (builtin/geom/sphere/trace.go): the
// nearer non-negative root of the quadratic, taken if below Tclosest.
__device__ __forceinline__ bool sphere_hit(const DMesh& m, TRay& r, HitRec& h) {
  const float L[3] = {__fsub_rn(r.ox, m.sphere[0]), __fsub_rn(r.oy, m.sphere[1]), __fsub_rn(r.oz, m.sphere[2])};
  const float a = __fadd_rn(__fadd_rn(__fmul_rn(r.dx, r.dx), __fmul_rn(r.dy, r.dy)), __fmul_rn(r.dz, r.dz));
  const float b = __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(r.dx, L[0]), __fmul_rn(r.dy, L[1])),
                                           __fmul_rn(r.dz, L[2])));
  const float c = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(L[0], L[0]), __fmul_rn(L[1], L[1])), __fmul_rn(L[2], L[2])),
                            __fmul_rn(m.sphere[3], m.sphere[3]));
  const float discr = __fsub_rn(__fmul_rn(b, b), __fmul_rn(__fmul_rn(4.0f, a), c));
  if (discr < 0.0f) return false;
  float x0, x1;
  if (discr == 0.0f) {
    x1 = __fdiv_rn(__fmul_rn(-0.5f, b), a);
    x0 = x1;
  } else {
    const float sq = __fsqrt_rn(discr);
    const float q = b > 0.0f ? __fmul_rn(-0.5f, __fadd_rn(b, sq)) : __fmul_rn(-0.5f, __fsub_rn(b, sq));
    x0 = __fdiv_rn(q, a);
    x1 = __fdiv_rn(c, q);
  }
  if (x0 > x1) { const float t = x0; x0 = x1; x1 = t; }
  if (x0 > x1) { const float t = x0; x0 = x1; x1 = t; }
  if (x0 < 0.0f) {
    x0 = x1;
    if (x0 < 0.0f) return false;
  }
  if (!(x0 < r.tclosest)) return false;
  r.tclosest = x0;
  h.elem = 0;
  h.u = h.v = h.w = 0.0f;
  return true;
}

template <bool ANY, bool COUNT>
__device__ __forceinline__ bool trace_any_mesh(const DMesh& m, TRay& r, int2* stk, int cap, HitRec& h,
                                               Counters& cnt, int& status) {
  if (m.kind == 1) return sphere_hit(m, r, h);
  if (m.n_tris == 0) return false;
  if (m.keys > 1) return trace_motion<ANY, COUNT>(m, r, stk, cap, h, cnt, status);
  return trace_static<ANY, COUNT>(m, r, stk, cap, h, cnt, status);
}

// PolyMesh.Trace with a Transform (builtin/geom/polymesh/trace.go:22-55): the
// ray in object space, P' = Matrix4MulPoint(inv, P), D' = Matrix4MulVec(inv,
// D) (math/matrix4.go:177-218, sums left to right), then Ray.Setup; time and
// Tclosest stay.  x: the inverse's columns 0..3, rows 0..2.
__device__ __forceinline__ void ray_to_object(TRay& r, const float* x) {
  const float px = r.ox, py = r.oy, pz = r.oz, dx = r.dx, dy = r.dy, dz = r.dz;
  r.ox = ((x[0] * px + x[3] * py) + x[6] * pz) + x[9];
  r.oy = ((x[1] * px + x[4] * py) + x[7] * pz) + x[10];
  r.oz = ((x[2] * px + x[5] * py) + x[8] * pz) + x[11];
  r.dx = (x[0] * dx + x[3] * dy) + x[6] * dz;
  r.dy = (x[1] * dx + x[4] * dy) + x[7] * dz;
  r.dz = (x[2] * dx + x[5] * dy) + x[8] * dz;
  ray_setup(r);
}

// A transform of two or more keys at the ray's time (PolyMesh.Trace,
// builtin/geom/polymesh/trace.go:33-48; TransformSRTArray.TimeKey,
// instance.go:20-36): the keys around the time blended
// (TransformDecompLerp), the matrix rebuilt, Matrix4Inverse; x receives the
// inverse's columns 0..3, rows 0..2.  Outside the keys (the reference panics)
// x is zero and the ray misses.  Not inlined: it runs once per entry into a
// keyed geom and would otherwise bloat the walk's registers.
__device__ __noinline__ void keyed_inverse(const anim::Decomp* keys, uint32_t n, float time, float* x) {
  float m[16], inv[16];
  if (!anim::at_time(keys, n, time, false, m)) {
    for (int k = 0; k < 12; ++k) x[k] = 0.0f;
    return;
  }
  anim::inverse(m, inv);
  const int cols[12] = {0, 1, 2, 4, 5, 6, 8, 9, 10, 12, 13, 14};
  for (int k = 0; k < 12; ++k) x[k] = inv[cols[k]];
}

// The ray in a geom's object space: its one matrix's inverse or its keyed
// transform at the ray's time.
__device__ __forceinline__ void to_object(const DMesh& M, TRay& r) {
  if (M.xf_nkeys >= 2) {
    float x[12];
    keyed_inverse(M.xf_keys, M.xf_nkeys, r.time, x);
    ray_to_object(r, x);
  } else {
    ray_to_object(r, M.xf_inv);
  }
}

// Instance.Trace (builtin/geom/instance/instance.go:72-115) and Proc.Trace
// (builtin/geom/proc/proc.go:88-140): the ray mapped by the group's
// transform at its time, then its geoms in order on the same stack slice,
// each through its own PolyMesh transform; a Proc stops at the first geom
// that hits unless the ray is a shadow ray (proc.go:117-124).  A hit reports
// the group's id for an instance and the child's id for a Proc (child_hit).
template <bool ANY, bool COUNT>
__device__ bool trace_group(const DTop& top, const DMesh& G, TRay& r, int2* stk, int cap, HitRec& h, Counters& cnt,
                            int& status) {
  TRay rg = r;
  to_object(G, rg);
  bool hit = false;
  for (uint32_t c = 0; c < G.n_children; ++c) {
    const DMesh& C = top.meshes[__ldg(G.children + c)];
    HitRec hc = h;
    bool ch;
    if (C.has_xf || C.xf_nkeys >= 2) {
      TRay ro = rg;
      to_object(C, ro);
      ch = trace_any_mesh<ANY, COUNT>(C, ro, stk, cap, hc, cnt, status);
      rg.tclosest = ro.tclosest;
    } else {
      ch = trace_any_mesh<ANY, COUNT>(C, rg, stk, cap, hc, cnt, status);
    }
    if (ch) {
      h = hc;
      h.geom = __ldg(G.child_hit + c);
      hit = true;
      if (!ANY) break;
    }
    if (status != kStatusOk) break;
  }
  r.tclosest = rg.tclosest;
  return hit;
}

// The world ray again after an object-space walk: P and D from the ray
// stream and Ray.Setup, Tclosest and time kept.
__device__ __forceinline__ void load_ray_pd(const RaySoA& rs, uint64_t i, TRay& r) {
  r.ox = __ldg(rs.px + i); r.oy = __ldg(rs.py + i); r.oz = __ldg(rs.pz + i);
  r.dx = __ldg(rs.dx + i); r.dy = __ldg(rs.dy + i); r.dz = __ldg(rs.dz + i);
  ray_setup(r);
}

__device__ __forceinline__ void load_ray(const RaySoA& rs, uint64_t i, TRay& r) {
  r.ox = __ldg(rs.px + i); r.oy = __ldg(rs.py + i); r.oz = __ldg(rs.pz + i);
  r.dx = __ldg(rs.dx + i); r.dy = __ldg(rs.dy + i); r.dz = __ldg(rs.dz + i);
  r.tclosest = __ldg(rs.tmax + i);
  r.time = rs.time ? __ldg(rs.time + i) : 0.0f;
  ray_setup(r);
}

__device__ __forceinline__ void store_hit(const HitSoA& hs, uint64_t i, const TRay& r, bool hit, const HitRec& h) {
  if (hs.prim) hs.prim[i] = hit ? h.elem : -1;
  if (hs.geom) hs.geom[i] = hit ? h.geom : -1;
  if (hs.t) hs.t[i] = r.tclosest;
  if (hs.u) hs.u[i] = hit ? h.u : 0.0f;
  if (hs.v) hs.v[i] = hit ? h.v : 0.0f;
  if (hs.w) hs.w[i] = hit ? h.w : 0.0f;
}

template <bool COUNT>
__device__ __forceinline__ void flush_counters(DScratch* s, const Counters& c) {
  if (!COUNT) return;
  unsigned long long a = c.nodes, b = c.leafs, d = c.tris;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(kFull, a, o);
    b += __shfl_down_sync(kFull, b, o);
    d += __shfl_down_sync(kFull, d, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s->node_visits, a);
    atomicAdd(&s->leaf_visits, b);
    atomicAdd(&s->tri_tests, d);
  }
}

// Scene.Trace (scene.go:30-58): top-level QBVH (leafMax 1) whose leaves run
// the per-mesh traversal on the remaining part of the same stack, sharing
// Tclosest, as Scene.TraceElems calls Geom.Trace (scene.go:61-97).
template <bool ANY, bool COUNT>
__device__ bool trace_scene_ray(const DTop& top, TRay& r, int2* stk, HitRec& h, Counters& cnt, int& status) {
  const uint32_t CAP = top.iter_cap;
  bool hit = false;
  const bool motion = top.keys > 1;
  float tm = 0.f, omt = 1.f;
  int key = 0, key2 = 0;
  if (motion) {
    const float k = __fmul_rn(r.time, (float)(top.keys - 1));
    const float fk = floorf(k);
    tm = __fsub_rn(k, fk);
    omt = __fsub_rn(1.0f, tm);
    key = (int)fk;
    key2 = (int)ceilf(k);
    if (key < 0 || key2 >= (int)top.keys) return false;
  }
  int sp = 0;
  int node = 0;
  float nodeT = r.tclosest;
  for (uint32_t iter = 0;; ++iter) {
    if (iter >= CAP) { status = kStatusIterationCap; break; }
    if (!(r.tclosest < nodeT) && node != kEmptyChild) {
      if (node >= 0) {
        if (COUNT) cnt.nodes++;
        float4 b[6];
        int4 ch;
        unsigned axes;
        if (!motion) {
          const float4* nb = reinterpret_cast<const float4*>(top.nodes + node);
#pragma unroll
          for (int q = 0; q < 6; ++q) b[q] = __ldg(nb + q);
          ch = __ldg(reinterpret_cast<const int4*>(nb + 6));
          axes = __ldg(reinterpret_cast<const unsigned*>(nb + 7));
        } else {
          const float4* bk = reinterpret_cast<const float4*>(top.mboxes);
          const float4* pa = bk + ((size_t)key * top.n_mnodes + node) * 6;
          const float4* pb = bk + ((size_t)key2 * top.n_mnodes + node) * 6;
#pragma unroll
          for (int q = 0; q < 6; ++q) {
            const float4 a = __ldg(pa + q), c = __ldg(pb + q);
            b[q].x = __fadd_rn(__fmul_rn(omt, a.x), __fmul_rn(tm, c.x));
            b[q].y = __fadd_rn(__fmul_rn(omt, a.y), __fmul_rn(tm, c.y));
            b[q].z = __fadd_rn(__fmul_rn(omt, a.z), __fmul_rn(tm, c.z));
            b[q].w = __fadd_rn(__fmul_rn(omt, a.w), __fmul_rn(tm, c.w));
          }
          ch = __ldg(reinterpret_cast<const int4*>(top.mnodes + node));
          axes = __ldg(reinterpret_cast<const unsigned*>(top.mnodes + node) + 4);
        }
        float tn[4];
        unsigned mask = r.exact ? box4<true>(r, b, tn) : box4<false>(r, b, tn);
        if (ch.x == kEmptyChild || r.tclosest < tn[0]) mask &= ~1u;
        if (ch.y == kEmptyChild || r.tclosest < tn[1]) mask &= ~2u;
        if (ch.z == kEmptyChild || r.tclosest < tn[2]) mask &= ~4u;
        if (ch.w == kEmptyChild || r.tclosest < tn[3]) mask &= ~8u;
        int next;
        float nextT;
        if (push_children(stk, sp, kStackCapacity, mask, ch, tn, axes, r.oct, next, nextT, status)) {
          node = next;
          nodeT = nextT;
          continue;
        }
        if (status != kStatusOk) break;
      } else {
        uint32_t first, count;
        leaf_decode(node, first, count);
        if (COUNT) cnt.leafs++;
        bool leaf_hit = false;
        for (uint32_t i = first; i < first + count; ++i) {
          const uint32_t g = __ldg(top.geom_order + i);
          HitRec hm = h;
          // The mesh traversal starts one slot above the free stack top,
          // as Traversal.StackTop = stackTop + 1 does (intersect.go:226).
          const int base = sp + 1;
          if (base >= kStackCapacity) { status = kStatusStackOverflow; break; }
          const DMesh& M = top.meshes[g];
          bool mh;
          if (M.kind == kGroup) {
            mh = trace_group<ANY, COUNT>(top, M, r, stk + base, kStackCapacity - base, hm, cnt, status);
          } else if (M.has_xf || M.xf_nkeys >= 2) {
            // the object-space copy walks the mesh; the world ray keeps its Tclosest
            TRay ro = r;
            to_object(M, ro);
            mh = trace_any_mesh<ANY, COUNT>(M, ro, stk + base, kStackCapacity - base, hm, cnt, status);
            r.tclosest = ro.tclosest;
          } else {
            mh = trace_any_mesh<ANY, COUNT>(M, r, stk + base, kStackCapacity - base, hm, cnt, status);
          }
          if (mh) {
            h = hm;
            if (M.kind != kGroup) h.geom = (int32_t)g;
            leaf_hit = true;
            if (ANY) break;
          }
          if (status != kStatusOk) break;
        }
        if (status != kStatusOk) break;
        if (leaf_hit) {
          hit = true;
          if (ANY) break;
        }
      }
    }
    if (sp == 0) break;
    --sp;
    const int2 e = stk[sp];
    node = e.x;
    nodeT = __int_as_float(e.y);
  }
  return hit;
}

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(128) k_trace_scene(const DTop top, RaySoA rays, HitSoA hits, uint64_t n,
                                                     DScratch* scratch, const unsigned long long* n_dev,
                                                     const uint32_t* order, const uint32_t* ray_path,
                                                     const uint32_t* path_geom) {
  if (n_dev) {
    const uint64_t nd = *n_dev;
    n = nd < n ? nd : n;
  }
  int2 stk[kStackCapacity];
  Counters cnt{0, 0, 0};
  const unsigned lane = threadIdx.x & 31u;
  int status = kStatusOk;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) {
      base = atomicAdd(&scratch->next_ray, 32ull);
      // A ray that hit a bound stops the whole launch at the next fetch.
      if (*reinterpret_cast<volatile int*>(&scratch->status) != kStatusOk) base = n;
    }
    base = __shfl_sync(kFull, base, 0);
    if (base >= n) break;
    const uint64_t i = base + lane;
    if (i < n) {
      // reordered rays: position i of the sorted copy is input ray order[i]
      const uint64_t rid = order ? (uint64_t)__ldg(order + i) : i;
      TRay r;
      load_ray(rays, i, r);
      HitRec h{-1, -1, 0.f, 0.f, 0.f};
      bool hit;
      if (ray_path) {  // job mode: the ray's own mesh, one stack slot above the (absent) top level
        const uint32_t g = __ldg(path_geom + __ldg(ray_path + rid));
        HitRec hm = h;
        if (top.meshes[g].has_xf) ray_to_object(r, top.meshes[g].xf_inv);  // no world-space work follows
        hit = trace_any_mesh<ANY, COUNT>(top.meshes[g], r, stk + 1, kStackCapacity - 1, hm, cnt, status);
        if (hit) {
          h = hm;
          h.geom = (int32_t)g;
        }
      } else {
        hit = trace_scene_ray<ANY, COUNT>(top, r, stk, h, cnt, status);
      }
      store_hit(hits, rid, r, hit, h);
      if (status != kStatusOk) {
        atomicMax(&scratch->status, status);
        status = kStatusOk;
      }
    }
  }
  flush_counters<COUNT>(scratch, cnt);
}

// Batched jobs (vmr_trace_jobs): the jobs' rays are gathered into one ray
// stream with a per-ray job index, traced by the scene kernel's job mode
// (each ray enters its job's mesh directly, in the while-while schedule with
// the cooperative leaf phase), and the hits are scattered back.  The job of
// stream position g: the last job whose first ray (ray0) is <= g.
__device__ __forceinline__ uint32_t job_of(const JobDesc* jobs, uint32_t n_jobs, uint64_t g) {
  uint32_t lo = 0, hi = n_jobs - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) / 2;
    if (jobs[mid].ray0 <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void k_jobs_gather(const JobDesc* jobs, uint32_t n_jobs, uint64_t n, RaySoA out, uint32_t* ray_job) {
  float* px = const_cast<float*>(out.px);
  float* py = const_cast<float*>(out.py);
  float* pz = const_cast<float*>(out.pz);
  float* dx = const_cast<float*>(out.dx);
  float* dy = const_cast<float*>(out.dy);
  float* dz = const_cast<float*>(out.dz);
  float* tm = const_cast<float*>(out.tmax);
  float* ti = const_cast<float*>(out.time);
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < n; g += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t j = job_of(jobs, n_jobs, g);
    const JobDesc& J = jobs[j];
    const uint64_t i = g - J.ray0;
    px[g] = J.rays.px[i]; py[g] = J.rays.py[i]; pz[g] = J.rays.pz[i];
    dx[g] = J.rays.dx[i]; dy[g] = J.rays.dy[i]; dz[g] = J.rays.dz[i];
    tm[g] = J.rays.tmax[i];
    ti[g] = J.rays.time ? J.rays.time[i] : 0.0f;
    ray_job[g] = j;
  }
}

__global__ void k_jobs_scatter(const JobDesc* jobs, uint32_t n_jobs, uint64_t n, HitSoA in) {
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < n; g += (uint64_t)gridDim.x * blockDim.x) {
    const JobDesc& J = jobs[job_of(jobs, n_jobs, g)];
    const uint64_t i = g - J.ray0;
    if (J.hits.prim) J.hits.prim[i] = in.prim[g];
    if (J.hits.geom) J.hits.geom[i] = in.geom[g];
    if (J.hits.t) J.hits.t[i] = in.t[g];
    if (J.hits.u) J.hits.u[i] = in.u[g];
    if (J.hits.v) J.hits.v[i] = in.v[g];
    if (J.hits.w) J.hits.w[i] = in.w[g];
  }
}

// ------------------------------------------------------------------------
// While-while persistent kernel for one mesh (the hot path).
//
// Each lane owns one ray.  An outer iteration runs a node phase (visit
// inner nodes until the current entry is a leaf or the ray is done) and a
// leaf phase (scan the leaf's triangles in order), so the warp executes the
// two code paths one after the other instead of interleaving them per lane.
// Lanes whose ray finished are refilled at the top of the next iteration
// with one warp-aggregated atomic (ballot of idle lanes, leader adds the
// count, lanes take base + their rank among the idle lanes), which keeps the
// warp full until the ray pool runs dry.

// 32 bytes of read-only global memory (32-byte aligned) as two float4, in
// one 256-bit load: a node of 128 bytes takes four load instructions
// instead of eight, and each instruction of a warp whose lanes fetch
// different nodes costs the L1 one pass per lane either way, so the node
// fetches' share of the L1 passes halves.
__device__ __forceinline__ void ld256(const void* p, float4& a, float4& c) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(c.x), "=f"(c.y), "=f"(c.z), "=f"(c.w)
      : "l"(p));
}
// A static wide node (128-byte aligned): 6 box float4, children, meta.
__device__ __forceinline__ void ld_node(const void* p, float4 (&b)[6], int4& ch, uint4& meta) {
  const float4* q = static_cast<const float4*>(p);
  ld256(q, b[0], b[1]);
  ld256(q + 2, b[2], b[3]);
  ld256(q + 4, b[4], b[5]);
  float4 c4, m4;
  ld256(q + 6, c4, m4);
  ch = make_int4(__float_as_int(c4.x), __float_as_int(c4.y), __float_as_int(c4.z), __float_as_int(c4.w));
  meta = make_uint4(__float_as_uint(m4.x), __float_as_uint(m4.y), __float_as_uint(m4.z), __float_as_uint(m4.w));
}

// Fetch a static node: 6 box float4, children, and this octant's push ranks.
__device__ __forceinline__ void fetch_node(const DMesh& m, int node, unsigned oct, float4 (&b)[6], int4& ch,
                                           unsigned& rk) {
  uint4 meta;
  ld_node(m.nodes + node, b, ch, meta);
  rk = (((oct & 4u) ? meta.z : meta.y) >> ((oct & 3u) * 8u)) & 0xffu;
}

// Fetch a motion node: boxes of both keys lerped per float
// ((1.0-time)*Boxes[key] + time*Boxes[key2], motionintersect.go:47-49).
__device__ __forceinline__ void fetch_mnode(const MNode* mnodes, int node, unsigned oct, const float4* bx0,
                                            const float4* bx1, float tm, float omt, float4 (&b)[6], int4& ch,
                                            unsigned& rk) {
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const float4 a = __ldg(bx0 + (size_t)node * 6 + q);
    const float4 c = __ldg(bx1 + (size_t)node * 6 + q);
    b[q].x = __fadd_rn(__fmul_rn(omt, a.x), __fmul_rn(tm, c.x));
    b[q].y = __fadd_rn(__fmul_rn(omt, a.y), __fmul_rn(tm, c.y));
    b[q].z = __fadd_rn(__fmul_rn(omt, a.z), __fmul_rn(tm, c.z));
    b[q].w = __fadd_rn(__fmul_rn(omt, a.w), __fmul_rn(tm, c.w));
  }
  const uint4* mn = reinterpret_cast<const uint4*>(mnodes + node);
  const uint4 c4 = __ldg(mn);
  ch = make_int4((int)c4.x, (int)c4.y, (int)c4.z, (int)c4.w);
  const uint4 meta = __ldg(mn + 1);
  rk = (((oct & 4u) ? meta.z : meta.y) >> ((oct & 3u) * 8u)) & 0xffu;
}

// A traversal stack whose first SS entries per thread live in shared memory
// (entry-major, so the 32 lanes of a warp always touch 32 different banks)
// and the rest in local memory; SS = 0 keeps the whole stack local.
template <int SS>
struct SplitStack {
  int* sn;     // shared node ids: entry k of this thread at sn[k * stride]
  float* st;   // shared T values
  int stride;  // threads per block
  int2 loc[kStackCapacity - SS];
  __device__ __forceinline__ void set(int i, int node, float T) {
    if (SS > 0 && i < SS) {
      sn[i * stride] = node;
      st[i * stride] = T;
    } else {
      loc[i - SS] = make_int2(node, __float_as_int(T));
    }
  }
  __device__ __forceinline__ int2 get(int i) const {
    if (SS > 0 && i < SS) return make_int2(sn[i * stride], __float_as_int(st[i * stride]));
    return loc[i - SS];
  }
};

// push_ranked for a SplitStack.
template <class S>
__device__ __forceinline__ bool push_ranked_s(S& stk, int& sp, unsigned mask, const int4& ch, const float (&tn)[4],
                                              unsigned rk, int& next, float& nextT, int& status) {
  if (mask == 0) return false;
  const unsigned r0 = rk & 3u, r1 = (rk >> 2) & 3u, r2 = (rk >> 4) & 3u, r3 = (rk >> 6) & 3u;
  const unsigned rmask = ((mask & 1u) << r0) | (((mask >> 1) & 1u) << r1) | (((mask >> 2) & 1u) << r2) |
                         (((mask >> 3) & 1u) << r3);
  const unsigned rtop = 31u - __clz(rmask);
  const int npush = __popc(rmask) - 1;
  if (sp + npush > kStackCapacity) {
    status = kStatusStackOverflow;
    return false;
  }
  const unsigned rr[4] = {r0, r1, r2, r3};
  const int cv[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    if (mask & (1u << c)) {
      if (rr[c] == rtop) {
        next = cv[c];
        nextT = tn[c];
      } else {
        stk.set(sp + __popc(rmask & ((1u << rr[c]) - 1u)), cv[c], tn[c]);
      }
    }
  }
  sp += npush;
  return true;
}

// Push the hit children in rank order (rank r_c = bits 2c..2c+1 of rk);
// the highest-ranked child is returned as the next entry instead.
__device__ __forceinline__ bool push_ranked(int2* stk, int& sp, unsigned mask, const int4& ch, const float (&tn)[4],
                                            unsigned rk, int& next, float& nextT, int& status) {
  if (mask == 0) return false;
  const unsigned r0 = rk & 3u, r1 = (rk >> 2) & 3u, r2 = (rk >> 4) & 3u, r3 = (rk >> 6) & 3u;
  const unsigned rmask = ((mask & 1u) << r0) | (((mask >> 1) & 1u) << r1) | (((mask >> 2) & 1u) << r2) |
                         (((mask >> 3) & 1u) << r3);
  const unsigned rtop = 31u - __clz(rmask);
  const int npush = __popc(rmask) - 1;
  if (sp + npush > kStackCapacity) {
    status = kStatusStackOverflow;
    return false;
  }
  const unsigned rr[4] = {r0, r1, r2, r3};
  const int cv[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    if (mask & (1u << c)) {
      if (rr[c] == rtop) {
        next = cv[c];
        nextT = tn[c];
      } else {
        stk[sp + __popc(rmask & ((1u << rr[c]) - 1u))] = make_int2(cv[c], __float_as_int(tn[c]));
      }
    }
  }
  sp += npush;
  return true;
}

// One leaf of TraceElems / TraceMotionElems: triangles [first, first+count)
// in order; returns the position of the last accepted triangle or -1.
template <bool MOTION, int C>
__device__ __forceinline__ int32_t leaf_scan(const DMesh& m, TRay& r, uint32_t first, uint32_t count,
                                             const float4* tr0, const float4* tr1, float tm, float omt, float& U,
                                             float& V, float& W) {
  int32_t idx = -1;
  for (uint32_t i = first; i < first + count; ++i) {
    if (MOTION) {
      float4 a[3], c[3], v[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        a[j] = __ldg(tr0 + 3 * (size_t)i + j);
        c[j] = __ldg(tr1 + 3 * (size_t)i + j);
      }
#pragma unroll
      for (int j = 0; j < 3; ++j)  // Vec3Lerp (math/vec3.go:52-58)
        v[j] = make_float4(__fadd_rn(__fmul_rn(omt, a[j].x), __fmul_rn(tm, c[j].x)),
                           __fadd_rn(__fmul_rn(omt, a[j].y), __fmul_rn(tm, c[j].y)),
                           __fadd_rn(__fmul_rn(omt, a[j].z), __fmul_rn(tm, c[j].z)), 0.f);
      if (tri_test<false, C>(r, v[0], v[1], v[2], m.ray_bias, U, V, W)) idx = (int32_t)i;
    } else {
      const float4 v0 = __ldg(tr0 + 3 * (size_t)i);
      const float4 v1 = __ldg(tr0 + 3 * (size_t)i + 1);
      const float4 v2 = __ldg(tr0 + 3 * (size_t)i + 2);
      if (tri_test<true, C>(r, v0, v1, v2, m.lower_static, U, V, W)) idx = (int32_t)i;
    }
  }
  return idx;
}

// Warp-uniform permutation class -> the compile-time instance; mixed warps
// take the run-time-select instance.  Both compute the same bits.
template <bool MOTION>
__device__ __forceinline__ int32_t leaf_scan_dispatch(const DMesh& m, TRay& r, uint32_t first, uint32_t count,
                                                      const float4* tr0, const float4* tr1, float tm, float omt,
                                                      float& U, float& V, float& W) {
  const unsigned act = __activemask();
  const int c0 = __shfl_sync(act, r.cls, __ffs(act) - 1);
  if (__all_sync(act, r.cls == c0)) {
    switch (c0) {
      case 0: return leaf_scan<MOTION, 0>(m, r, first, count, tr0, tr1, tm, omt, U, V, W);
      case 1: return leaf_scan<MOTION, 1>(m, r, first, count, tr0, tr1, tm, omt, U, V, W);
      case 2: return leaf_scan<MOTION, 2>(m, r, first, count, tr0, tr1, tm, omt, U, V, W);
      case 3: return leaf_scan<MOTION, 3>(m, r, first, count, tr0, tr1, tm, omt, U, V, W);
      case 4: return leaf_scan<MOTION, 4>(m, r, first, count, tr0, tr1, tm, omt, U, V, W);
      default: return leaf_scan<MOTION, 5>(m, r, first, count, tr0, tr1, tm, omt, U, V, W);
    }
  }
  return leaf_scan<MOTION, -1>(m, r, first, count, tr0, tr1, tm, omt, U, V, W);
}

// Warp-cooperative leaf scan of a static mesh.  The leaves the lanes hold
// are laid end to end as one list of (ray, triangle) pairs and tested 32 per
// round, one pair per lane: consecutive lanes read consecutive triangles of
// a leaf (a leaf is one contiguous run) and no lane idles while another
// still has triangles.  tri_prepare does not depend on Tclosest, so it can
// run in any order; the Tclosest-dependent acceptance then runs on the
// owning lane, over its candidates in the reference's triangle order (a
// round's candidates in lane order, rounds in order), exactly as the
// sequential scan.  Called by all 32 lanes; has: the lane holds a leaf.
// tris, lower: the lane's mesh (its triangles and lower bound); the tester
// uses its owner's (one mesh per launch in the mesh kernel, one per lane in
// the scene kernel).
template <int C>
__device__ __forceinline__ int32_t coop_leaf(const float4* tris, float lower, TRay& r, bool has, uint32_t first,
                                             uint32_t count, float& U, float& V, float& W) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t cnt = has ? count : 0u;
  uint32_t incl = cnt;  // inclusive prefix of the leaf sizes
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(kFull, incl, o);
    if (lane >= (unsigned)o) incl += v;
  }
  const uint32_t total = __shfl_sync(kFull, incl, 31);
  const uint32_t excl = incl - cnt;
  int32_t idx = -1;
  for (uint32_t base = 0; base < total; base += 32) {
    const uint32_t g = base + lane;
    // owner: the lowest lane whose inclusive prefix exceeds g
    int lo = 0, hi = 31;
#pragma unroll
    for (int st = 0; st < 5; ++st) {
      const int mid = (lo + hi) >> 1;
      if (__shfl_sync(kFull, incl, mid) > g) hi = mid;
      else lo = mid + 1;
    }
    const int o = lo;
    const uint32_t i = __shfl_sync(kFull, first, o) + (g - __shfl_sync(kFull, excl, o));
    TRay q;  // the owner's ray: the fields tri_prepare reads
    q.pkx = __shfl_sync(kFull, r.pkx, o);
    q.pky = __shfl_sync(kFull, r.pky, o);
    q.pkz = __shfl_sync(kFull, r.pkz, o);
    q.s0 = __shfl_sync(kFull, r.s0, o);
    q.s1 = __shfl_sync(kFull, r.s1, o);
    q.s2 = __shfl_sync(kFull, r.s2, o);
    if (C < 0) {
      q.kx = __shfl_sync(kFull, r.kx, o);
      q.ky = __shfl_sync(kFull, r.ky, o);
      q.kz = __shfl_sync(kFull, r.kz, o);
    }
    const float4* ot = reinterpret_cast<const float4*>(
        __shfl_sync(kFull, (unsigned long long)reinterpret_cast<uintptr_t>(tris), o));
    const float olower = __shfl_sync(kFull, lower, o);
    float fU = 0.f, fV = 0.f, fW = 0.f, det = 0.f, T = 0.f;
    bool cand = false;
    if (g < total) {
      const float4 v0 = __ldg(ot + 3 * (size_t)i);
      const float4 v1 = __ldg(ot + 3 * (size_t)i + 1);
      const float4 v2 = __ldg(ot + 3 * (size_t)i + 2);
      cand = tri_prepare<true, C>(q, v0, v1, v2, olower, fU, fV, fW, det, T);
    }
    unsigned cm = __ballot_sync(kFull, cand);
    while (cm != 0u) {  // candidates in lane order, i.e. in each owner's triangle order
      const int c = __ffs(cm) - 1;
      cm &= cm - 1u;
      const int oc = __shfl_sync(kFull, o, c);
      const float cU = __shfl_sync(kFull, fU, c), cV = __shfl_sync(kFull, fV, c), cW = __shfl_sync(kFull, fW, c);
      const float cdet = __shfl_sync(kFull, det, c), cT = __shfl_sync(kFull, T, c);
      const uint32_t ci = __shfl_sync(kFull, i, c);
      if ((int)lane == oc && tri_accept(r, cU, cV, cW, cdet, cT, U, V, W)) idx = (int32_t)ci;
    }
  }
  return idx;
}

// The cooperative scan over leaves of static and motion meshes (the scene
// kernel's motion instantiation).  A tester takes its owner's mesh mode with
// the ray: a static pair is TraceElems' test (trace.go:123-193) on the
// stored vertices above EpsilonFloat32 + RayBias; a motion pair is
// TraceMotionElems' (trace.go:563-612) on the vertices of the two keys
// lerped at the owner's time, Vec3Lerp (math/vec3.go:52-58), above RayBias.
// Acceptance on the owner in triangle order, as in coop_leaf.  t1, tm, omt
// are unused by static owners.
template <int C>
__device__ __forceinline__ int32_t coop_leaf_mix(const float4* t0, const float4* t1, float tm, float omt, bool mot,
                                                 float lower, TRay& r, bool has, uint32_t first, uint32_t count,
                                                 float& U, float& V, float& W) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t cnt = has ? count : 0u;
  uint32_t incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(kFull, incl, o);
    if (lane >= (unsigned)o) incl += v;
  }
  const uint32_t total = __shfl_sync(kFull, incl, 31);
  const uint32_t excl = incl - cnt;
  int32_t idx = -1;
  for (uint32_t base = 0; base < total; base += 32) {
    const uint32_t g = base + lane;
    int lo = 0, hi = 31;
#pragma unroll
    for (int st = 0; st < 5; ++st) {
      const int mid = (lo + hi) >> 1;
      if (__shfl_sync(kFull, incl, mid) > g) hi = mid;
      else lo = mid + 1;
    }
    const int o = lo;
    const uint32_t i = __shfl_sync(kFull, first, o) + (g - __shfl_sync(kFull, excl, o));
    TRay q;
    q.pkx = __shfl_sync(kFull, r.pkx, o);
    q.pky = __shfl_sync(kFull, r.pky, o);
    q.pkz = __shfl_sync(kFull, r.pkz, o);
    q.s0 = __shfl_sync(kFull, r.s0, o);
    q.s1 = __shfl_sync(kFull, r.s1, o);
    q.s2 = __shfl_sync(kFull, r.s2, o);
    if (C < 0) {
      q.kx = __shfl_sync(kFull, r.kx, o);
      q.ky = __shfl_sync(kFull, r.ky, o);
      q.kz = __shfl_sync(kFull, r.kz, o);
    }
    const float4* a0 = reinterpret_cast<const float4*>(
        __shfl_sync(kFull, (unsigned long long)reinterpret_cast<uintptr_t>(t0), o));
    const float4* a1 = reinterpret_cast<const float4*>(
        __shfl_sync(kFull, (unsigned long long)reinterpret_cast<uintptr_t>(t1), o));
    const float otm = __shfl_sync(kFull, tm, o), oomt = __shfl_sync(kFull, omt, o);
    const bool omot = __shfl_sync(kFull, mot ? 1 : 0, o) != 0;
    const float olower = __shfl_sync(kFull, lower, o);
    float fU = 0.f, fV = 0.f, fW = 0.f, det = 0.f, T = 0.f;
    bool cand = false;
    if (g < total) {
      if (omot) {
        float4 v[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float4 a = __ldg(a0 + 3 * (size_t)i + j), c = __ldg(a1 + 3 * (size_t)i + j);
          v[j] = make_float4(__fadd_rn(__fmul_rn(oomt, a.x), __fmul_rn(otm, c.x)),
                             __fadd_rn(__fmul_rn(oomt, a.y), __fmul_rn(otm, c.y)),
                             __fadd_rn(__fmul_rn(oomt, a.z), __fmul_rn(otm, c.z)), 0.f);
        }
        cand = tri_prepare<false, C>(q, v[0], v[1], v[2], olower, fU, fV, fW, det, T);
      } else {
        const float4 v0 = __ldg(a0 + 3 * (size_t)i);
        const float4 v1 = __ldg(a0 + 3 * (size_t)i + 1);
        const float4 v2 = __ldg(a0 + 3 * (size_t)i + 2);
        cand = tri_prepare<true, C>(q, v0, v1, v2, olower, fU, fV, fW, det, T);
      }
    }
    unsigned cm = __ballot_sync(kFull, cand);
    while (cm != 0u) {
      const int c = __ffs(cm) - 1;
      cm &= cm - 1u;
      const int oc = __shfl_sync(kFull, o, c);
      const float cU = __shfl_sync(kFull, fU, c), cV = __shfl_sync(kFull, fV, c), cW = __shfl_sync(kFull, fW, c);
      const float cdet = __shfl_sync(kFull, det, c), cT = __shfl_sync(kFull, T, c);
      const uint32_t ci = __shfl_sync(kFull, i, c);
      if ((int)lane == oc && tri_accept(r, cU, cV, cW, cdet, cT, U, V, W)) idx = (int32_t)ci;
    }
  }
  return idx;
}

__device__ __forceinline__ int32_t coop_leaf_mix_dispatch(const float4* t0, const float4* t1, float tm, float omt,
                                                          bool mot, float lower, TRay& r, bool has, uint32_t first,
                                                          uint32_t count, float& U, float& V, float& W) {
  const unsigned hm = __ballot_sync(kFull, has);
  if (hm == 0u) return -1;
  const int c0 = __shfl_sync(kFull, r.cls, __ffs(hm) - 1);
  if (__all_sync(kFull, !has || r.cls == c0)) {
    switch (c0) {
      case 0: return coop_leaf_mix<0>(t0, t1, tm, omt, mot, lower, r, has, first, count, U, V, W);
      case 1: return coop_leaf_mix<1>(t0, t1, tm, omt, mot, lower, r, has, first, count, U, V, W);
      case 2: return coop_leaf_mix<2>(t0, t1, tm, omt, mot, lower, r, has, first, count, U, V, W);
      case 3: return coop_leaf_mix<3>(t0, t1, tm, omt, mot, lower, r, has, first, count, U, V, W);
      case 4: return coop_leaf_mix<4>(t0, t1, tm, omt, mot, lower, r, has, first, count, U, V, W);
      default: return coop_leaf_mix<5>(t0, t1, tm, omt, mot, lower, r, has, first, count, U, V, W);
    }
  }
  return coop_leaf_mix<-1>(t0, t1, tm, omt, mot, lower, r, has, first, count, U, V, W);
}

// The class the lanes holding a leaf share picks the compile-time instance;
// mixed classes take the run-time-select one.  All 32 lanes call this.
__device__ __forceinline__ int32_t coop_leaf_dispatch(const float4* tris, float lower, TRay& r, bool has,
                                                      uint32_t first, uint32_t count, float& U, float& V, float& W) {
  const unsigned hm = __ballot_sync(kFull, has);
  if (hm == 0u) return -1;
  const int c0 = __shfl_sync(kFull, r.cls, __ffs(hm) - 1);
  if (__all_sync(kFull, !has || r.cls == c0)) {
    switch (c0) {
      case 0: return coop_leaf<0>(tris, lower, r, has, first, count, U, V, W);
      case 1: return coop_leaf<1>(tris, lower, r, has, first, count, U, V, W);
      case 2: return coop_leaf<2>(tris, lower, r, has, first, count, U, V, W);
      case 3: return coop_leaf<3>(tris, lower, r, has, first, count, U, V, W);
      case 4: return coop_leaf<4>(tris, lower, r, has, first, count, U, V, W);
      default: return coop_leaf<5>(tris, lower, r, has, first, count, U, V, W);
    }
  }
  return coop_leaf<-1>(tris, lower, r, has, first, count, U, V, W);
}

template <bool MOTION, bool ANY, bool COUNT, bool PF, int MINB, int SS, bool COOP = false>
__global__ void __launch_bounds__(MINB > 0 ? 128 : 256, MINB > 0 ? MINB : 1)
    k_trace_mesh_ww(const DMesh m, RaySoA rays, HitSoA hits, uint64_t n, DScratch* scratch, const uint32_t* order,
                    int walk_tail, const unsigned long long* n_dev) {
  if (n_dev) n = *n_dev < n ? *n_dev : n;  // a wavefront queue's length
  extern __shared__ int stack_smem[];
  SplitStack<SS> stk;
  if (SS > 0) {
    stk.stride = blockDim.x;
    stk.sn = stack_smem + threadIdx.x;
    stk.st = reinterpret_cast<float*>(stack_smem + SS * blockDim.x) + threadIdx.x;
  }
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lanes_below = (1u << lane) - 1u;
  TRay r;
  HitRec h{-1, -1, 0.f, 0.f, 0.f};
  // Current entry (as if just popped); -1 = no entry left.
  int node = -1, sp = 0;
  float nodeT = 0.f;
  uint64_t rid = 0;
  uint32_t iter = 0;
  bool alive = false, hit = false;
  bool more = true;  // warp-uniform: the pool may still hold rays
  int status = kStatusOk;
  Counters cnt{0, 0, 0};
  float tm = 0.f, omt = 1.f;
  const float4* bx0 = nullptr;
  const float4* bx1 = nullptr;
  const float4* tr0 = reinterpret_cast<const float4*>(MOTION ? m.mtris : m.tris);
  const float4* tr1 = tr0;
  for (;;) {
    const unsigned need = __ballot_sync(kFull, !alive);
    if (need != 0u && more) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) {
        base = atomicAdd(&scratch->next_ray, (unsigned long long)__popc(need));
        // A ray that hit a bound stops the whole launch at the next fetch.
        if (*reinterpret_cast<volatile int*>(&scratch->status) != kStatusOk) base = n;
      }
      base = __shfl_sync(kFull, base, leader);
      if (base + __popc(need) >= n) more = false;
      if (!alive) {
        const uint64_t i = base + __popc(need & lanes_below);
        if (i < n) {
          if (!MOTION && rays.rec) {  // the key-ordered copy as records (RaySoA::rec)
            const float4* A = static_cast<const float4*>(rays.rec);
            const float4 a = __ldg(A + 2 * i), b = __ldg(A + 2 * i + 1);
            r.ox = a.x; r.oy = a.y; r.oz = a.z;
            r.dx = a.w; r.dy = b.x; r.dz = b.y;
            r.tclosest = b.z;
            r.time = 0.0f;
            ray_setup(r);
            rid = __float_as_uint(b.w);
          } else {
            rid = order ? (uint64_t)__ldg(order + i) : i;
            load_ray(rays, i, r);
          }
          h = HitRec{-1, -1, 0.f, 0.f, 0.f};
          hit = false;
          node = 0;  // the root, pushed with T = Tclosest (intersect.go:93-95)
          nodeT = r.tclosest;
          sp = 0;
          iter = 0;
          alive = true;
          if (MOTION) {
            // k = Time*float32(keys-1); time = k-Floor(k); key = Floor(k),
            // key2 = Ceil(k) (builtin/geom/polymesh/trace.go:79-84)
            const float k = __fmul_rn(r.time, (float)(m.keys - 1));
            const float fk = floorf(k);
            tm = __fsub_rn(k, fk);
            omt = __fsub_rn(1.0f, tm);
            const int key = (int)fk, key2 = (int)ceilf(k);
            if (key < 0 || key2 >= (int)m.keys) {
              // out of the key range: the reference indexes out of bounds; miss
              store_hit(hits, rid, r, false, h);
              alive = false;
            } else {
              bx0 = reinterpret_cast<const float4*>(m.mboxes) + (size_t)key * m.n_mnodes * 6;
              bx1 = reinterpret_cast<const float4*>(m.mboxes) + (size_t)key2 * m.n_mnodes * 6;
              tr0 = reinterpret_cast<const float4*>(m.mtris) + (size_t)key * m.n_tris * 3;
              tr1 = reinterpret_cast<const float4*>(m.mtris) + (size_t)key2 * m.n_tris * 3;
            }
          }
        }
      }
    }
    const unsigned alive_mask = __ballot_sync(kFull, alive);
    if (alive_mask == 0u) {
      if (!more) break;
      continue;
    }
    constexpr bool kCoop = COOP;
    bool done = false, walking = false;
    if (alive) {
      // ---- node phase: one entry per step (a cull-pop, a leaf found, or an
      // inner-node visit) for every lane still walking.  The warp steps in
      // lock-step; it stops when no lane walks, or when at most walk_tail
      // lanes walk and some lane holds a leaf (the stragglers resume in the
      // next node phase).
      walking = node != -1;
      for (;;) {
        const unsigned wmask = __ballot_sync(alive_mask, walking);
        if (wmask == 0u) break;
        if (walk_tail > 0 && __popc(wmask) <= walk_tail) {
          const unsigned leafy = __ballot_sync(alive_mask, !walking && node < -1);
          if (leafy != 0u) break;
        }
        if (!walking) continue;
        if (++iter > m.iter_cap) {
          status = kStatusIterationCap;
          done = true;
          walking = false;
          continue;
        }
        if (r.tclosest < nodeT) {  // pop-time cull (intersect.go:106)
          if (sp == 0) {
            node = -1;
            walking = false;
          } else {
            const int2 e = stk.get(--sp);
            node = e.x;
            nodeT = __int_as_float(e.y);
          }
          continue;
        }
        if (node < 0) {  // a leaf: the leaf phase scans it
          walking = false;
          continue;
        }
        if (COUNT) cnt.nodes++;
        float4 b[6];
        int4 ch;
        unsigned rk;
        if (MOTION) fetch_mnode(m.mnodes, node, r.oct, bx0, bx1, tm, omt, b, ch, rk);
        else fetch_node(m, node, r.oct, b, ch, rk);
        float tn[4];
        unsigned mask = r.exact ? box4<true>(r, b, tn) : box4<false>(r, b, tn);
        if (ch.x == kEmptyChild || r.tclosest < tn[0]) mask &= ~1u;
        if (ch.y == kEmptyChild || r.tclosest < tn[1]) mask &= ~2u;
        if (ch.z == kEmptyChild || r.tclosest < tn[2]) mask &= ~4u;
        if (ch.w == kEmptyChild || r.tclosest < tn[3]) mask &= ~8u;
        int next = 0;
        float nextT = 0.f;
        if (push_ranked_s(stk, sp, mask, ch, tn, rk, next, nextT, status)) {
          node = next;
          nodeT = nextT;
        } else if (status != kStatusOk) {
          done = true;
          walking = false;
        } else if (sp == 0) {
          node = -1;
          walking = false;
        } else {
          const int2 e = stk.get(--sp);
          node = e.x;
          nodeT = __int_as_float(e.y);
        }
      }
      // ---- leaf phase: lanes whose current entry is a leaf scan it, in the
      // order the reference pops it, then pop the next entry.
      if (!kCoop && !done && !walking && node < -1) {
        uint32_t first, count;
        leaf_decode(node, first, count);
        if (COUNT) { cnt.leafs++; cnt.tris += count; }
        float U = 0.f, V = 0.f, W = 0.f;
        const int32_t idx = leaf_scan_dispatch<MOTION>(m, r, first, count, tr0, tr1, tm, omt, U, V, W);
        if (idx != -1) {
          h.elem = MOTION ? __ldg(m.elem + idx) : idx;
          h.u = U;
          h.v = V;
          h.w = W;
          hit = true;
        }
        if ((ANY && idx != -1) || sp == 0) {  // shadow rays stop at the first hit leaf (intersect.go:231-236)
          done = true;
        } else {
          const int2 e = stk.get(--sp);
          node = e.x;
          nodeT = __int_as_float(e.y);
          if (PF && !MOTION && node >= 0) prefetch_l1(m.nodes + node);
        }
      }
    }
    if (kCoop) {  // the leaf phase as one warp-wide list of triangle tests
      const bool has = alive && !done && !walking && node < -1;
      uint32_t first = 0, count = 0;
      if (has) {
        leaf_decode(node, first, count);
        if (COUNT) { cnt.leafs++; cnt.tris += count; }
      }
      float U = 0.f, V = 0.f, W = 0.f;
      // motion: every tester lerps its owner's two keys at the owner's time
      const int32_t idx =
          MOTION ? coop_leaf_mix_dispatch(tr0, tr1, tm, omt, true, m.ray_bias, r, has, first, count, U, V, W)
                 : coop_leaf_dispatch(reinterpret_cast<const float4*>(m.tris), m.lower_static, r, has, first, count,
                                      U, V, W);
      if (has) {
        if (idx != -1) {
          h.elem = MOTION ? __ldg(m.elem + idx) : idx;
          h.u = U;
          h.v = V;
          h.w = W;
          hit = true;
        }
        if ((ANY && idx != -1) || sp == 0) {
          done = true;
        } else {
          const int2 e = stk.get(--sp);
          node = e.x;
          nodeT = __int_as_float(e.y);
        }
      }
    }
    if (alive) {
      if (!walking && node == -1) done = true;
      if (done) {
        store_hit(hits, rid, r, hit, h);
        alive = false;
        if (status != kStatusOk) {
          atomicMax(&scratch->status, status);
          status = kStatusOk;
        }
      }
    }
  }
  flush_counters<COUNT>(scratch, cnt);
}

// ------------------------------------------------------------------------
// While-while persistent kernel for a static two-level scene.
//
// As k_trace_mesh_ww, with the lane's current entry in either the top level
// (geom < 0) or the mesh it entered at a top-level leaf.  A top-level leaf
// enters its geoms one after the other (Scene.TraceElems, scene.go:61-97):
// the mesh traversal starts one slot above the top-level entries on the
// same stack with its root at T = Tclosest (Traversal.StackTop = stackTop+1,
// intersect.go:226) and ends when its part of the stack is empty, after
// which the next geom of the leaf, or the top level, continues.  Node
// visits, pops, culls and triangle tests per ray are the reference's.
// The key pair and lerp weight of a motion mesh at the ray's time
// (builtin/geom/polymesh/trace.go:79-84); false outside the key range (the
// reference would index out of bounds: a miss, as the mesh kernels treat it).
__device__ __forceinline__ bool motion_keys(uint32_t keys, float time, float& tm, float& omt, int& key, int& key2) {
  const float k = __fmul_rn(time, (float)(keys - 1));
  const float fk = floorf(k);
  tm = __fsub_rn(k, fk);
  omt = __fsub_rn(1.0f, tm);
  key = (int)fk;
  key2 = (int)ceilf(k);
  return !(key < 0 || key2 >= (int)keys);
}

// Capped for 7 resident blocks per SM (72 registers; the two-level sphere
// grid 1% faster than at 8).  MOT (motion meshes and top levels) holds more
// state: capped for 5 (96 registers) instead, as at 8 it spilled 1 KB per
// thread and measured 27% slower on the batched jobs.
template <bool ANY, bool COOP = false, bool MOT = false>
__global__ void __launch_bounds__(128, MOT ? 5 : 7)
    k_trace_scene_ww(const DTop top, RaySoA rays, HitSoA hits, uint64_t n, DScratch* scratch,
                     const unsigned long long* n_dev, const uint32_t* order, int walk_tail,
                     const uint32_t* ray_path, const uint32_t* path_geom) {
  if (n_dev) {
    const uint64_t nd = *n_dev;
    n = nd < n ? nd : n;
  }
  int2 stk[kStackCapacity];
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lanes_below = (1u << lane) - 1u;
  TRay r;
  HitRec h{-1, -1, 0.f, 0.f, 0.f};
  int node = -1, sp = 0;
  float nodeT = 0.f;
  uint64_t rid = 0;
  uint32_t iter = 0, miter = 0;
  bool alive = false, hit = false, more = true;
  int status = kStatusOk;
  // current mesh (geom >= 0) and the top-level leaf's remaining geoms
  int geom = -1, base = 0;
  uint32_t leaf_next = 0, leaf_left = 0;
  const GNode* mnodes = nullptr;
  const float4* mtris = nullptr;
  float lower = 0.f;
  uint32_t mcap = 0;
  bool mmot = false;  // the current mesh has motion keys (its key data is re-read from top.meshes)
  bool mxf = false;   // the current mesh has a transform: r is its object-space ray
  uint64_t li = 0;    // the ray's position in rays (the world ray is reloaded from it)
  float tm_unused = 0.f, omt_unused = 1.f;
  int key_unused = 0, key2_unused = 0;
  for (;;) {
    const unsigned need = __ballot_sync(kFull, !alive);
    if (need != 0u && more) {
      const int leader = __ffs(need) - 1;
      unsigned long long b0 = 0;
      if ((int)lane == leader) {
        b0 = atomicAdd(&scratch->next_ray, (unsigned long long)__popc(need));
        if (*reinterpret_cast<volatile int*>(&scratch->status) != kStatusOk) b0 = n;
      }
      b0 = __shfl_sync(kFull, b0, leader);
      if (b0 + __popc(need) >= n) more = false;
      if (!alive) {
        const uint64_t i = b0 + __popc(need & lanes_below);
        if (i < n) {
          rid = order ? (uint64_t)__ldg(order + i) : i;
          li = i;
          load_ray(rays, i, r);
          h = HitRec{-1, -1, 0.f, 0.f, 0.f};
          hit = false;
          node = 0;  // the top-level root, pushed with T = Tclosest
          nodeT = r.tclosest;
          sp = 0;
          iter = 0;
          geom = -1;
          leaf_left = 0;
          alive = true;
          if (ray_path) {  // job mode: enter the ray's own mesh, as a top-level leaf would
            const uint32_t g = __ldg(path_geom + __ldg(ray_path + rid));
            const DMesh& M = top.meshes[g];
            if (M.kind == 1) {  // an analytic sphere: tested here
              if (sphere_hit(M, r, h)) {
                h.geom = (int)g;
                hit = true;
              }
              node = -1;
            } else if (M.n_tris == 0) {
              node = -1;
            } else if (MOT && M.keys > 1 && !motion_keys(M.keys, r.time, tm_unused, omt_unused, key_unused, key2_unused)) {
              node = -1;
            } else {
              base = 1;
              geom = (int)g;
              mmot = MOT && M.keys > 1;
              if (MOT && M.has_xf) ray_to_object(r, M.xf_inv);  // the mesh is the ray's whole walk
              mnodes = M.nodes;
              mtris = reinterpret_cast<const float4*>(M.tris);
              lower = M.lower_static;
              mcap = M.iter_cap;
              miter = 0;
              sp = base;
            }
          } else if (MOT && top.keys > 1 && !motion_keys(top.keys, r.time, tm_unused, omt_unused, key_unused,
                                                         key2_unused)) {
            node = -1;  // outside the top level's key range: a miss
          }
        }
      }
    }
    const unsigned alive_mask = __ballot_sync(kFull, alive);
    if (alive_mask == 0u) {
      if (!more) break;
      continue;
    }
    bool done = false, walking = false;
    if (alive) {
      walking = node != -1;
      for (;;) {
        const unsigned wmask = __ballot_sync(alive_mask, walking);
        if (wmask == 0u) break;
        if (walk_tail > 0 && __popc(wmask) <= walk_tail) {
          // a leaf for the cooperative scan ends the walk early; without it
          // (COOP off) a motion leaf is scanned by its own lane, and a walk
          // cut short for it idles the warp
          const unsigned leafy = __ballot_sync(alive_mask, !walking && node < -1 && geom >= 0 && !(MOT && mmot && !COOP));
          if (leafy != 0u) break;
        }
        if (!walking) continue;
        if (geom < 0 ? ++iter > top.iter_cap : ++miter > mcap) {
          status = kStatusIterationCap;
          done = true;
          walking = false;
          continue;
        }
        // next entry: a pop, the next geom of the leaf, or the end
        bool need_pop = false;
        if (r.tclosest < nodeT) {  // pop-time cull (intersect.go:106)
          need_pop = true;
        } else if (node >= 0) {
          float4 b[6];
          int4 ch;
          unsigned rk;
          if (MOT && geom >= 0 && mmot) {  // a motion mesh: boxes lerped at the ray's time
            const DMesh& M = top.meshes[geom];
            float tm, omt;
            int key, key2;
            motion_keys(M.keys, r.time, tm, omt, key, key2);
            const float4* bx = reinterpret_cast<const float4*>(M.mboxes);
            fetch_mnode(M.mnodes, node, r.oct, bx + (size_t)key * M.n_mnodes * 6, bx + (size_t)key2 * M.n_mnodes * 6, tm,
                        omt, b, ch, rk);
          } else if (MOT && geom < 0 && top.keys > 1) {  // a motion top level
            float tm, omt;
            int key, key2;
            motion_keys(top.keys, r.time, tm, omt, key, key2);
            const float4* bx = reinterpret_cast<const float4*>(top.mboxes);
            fetch_mnode(top.mnodes, node, r.oct, bx + (size_t)key * top.n_mnodes * 6,
                        bx + (size_t)key2 * top.n_mnodes * 6, tm, omt, b, ch, rk);
          } else {
            const GNode* nb = geom < 0 ? top.nodes : mnodes;
            uint4 meta;
            ld_node(nb + node, b, ch, meta);
            rk = (((r.oct & 4u) ? meta.z : meta.y) >> ((r.oct & 3u) * 8u)) & 0xffu;
          }
          float tn[4];
          unsigned mask = r.exact ? box4<true>(r, b, tn) : box4<false>(r, b, tn);
          if (ch.x == kEmptyChild || r.tclosest < tn[0]) mask &= ~1u;
          if (ch.y == kEmptyChild || r.tclosest < tn[1]) mask &= ~2u;
          if (ch.z == kEmptyChild || r.tclosest < tn[2]) mask &= ~4u;
          if (ch.w == kEmptyChild || r.tclosest < tn[3]) mask &= ~8u;
          int next = 0;
          float nextT = 0.f;
          if (push_ranked(stk, sp, mask, ch, tn, rk, next, nextT, status)) {
            node = next;
            nodeT = nextT;
            continue;
          }
          if (status != kStatusOk) {
            done = true;
            walking = false;
            continue;
          }
          need_pop = true;
        } else if (node == kEmptyChild) {
          need_pop = true;
        } else if (geom >= 0) {  // a mesh leaf: the leaf phase scans it
          walking = false;
          continue;
        } else {  // a top-level leaf: its geoms, in order
          uint32_t first, count;
          leaf_decode(node, first, count);
          leaf_next = first;
          leaf_left = count;
          need_pop = true;  // handled below: enter the first geom
        }
        // pop / enter the next geom / leave a finished mesh
        for (;;) {
          if (geom >= 0 && sp > base) {  // the mesh's own entries
            const int2 e = stk[--sp];
            node = e.x;
            nodeT = __int_as_float(e.y);
            break;
          }
          if (geom >= 0) {  // the mesh traversal is done
            geom = -1;
            sp = base - 1;
            if (MOT && mxf) {  // back to the world ray (Tclosest kept)
              load_ray_pd(rays, li, r);
              mxf = false;
            }
          }
          if (leaf_left > 0) {  // enter the next geom of the top-level leaf
            const uint32_t g = __ldg(top.geom_order + leaf_next);
            ++leaf_next;
            --leaf_left;
            const DMesh& M = top.meshes[g];
            if (M.kind == 1) {  // an analytic sphere: tested here, no stack
              if (sphere_hit(M, r, h)) {
                h.geom = (int)g;
                hit = true;
                if (ANY) {
                  node = -1;
                  break;
                }
              }
              continue;
            }
            if (M.n_tris == 0) continue;
            if (MOT && M.keys > 1 && !motion_keys(M.keys, r.time, tm_unused, omt_unused, key_unused, key2_unused)) continue;
            base = sp + 1;
            if (base >= kStackCapacity) {
              status = kStatusStackOverflow;
              break;
            }
            geom = (int)g;
            mmot = MOT && M.keys > 1;
            mxf = MOT && M.has_xf;
            if (mxf) ray_to_object(r, M.xf_inv);
            mnodes = M.nodes;
            mtris = reinterpret_cast<const float4*>(M.tris);
            lower = M.lower_static;
            mcap = M.iter_cap;
            miter = 0;
            sp = base;
            node = 0;
            nodeT = r.tclosest;
            break;
          }
          if (hit && ANY) {  // shadow rays stop after the leaf that hit (intersect.go:231-236)
            node = -1;
            break;
          }
          if (sp == 0) {
            node = -1;
            break;
          }
          const int2 e = stk[--sp];
          node = e.x;
          nodeT = __int_as_float(e.y);
          break;
        }
        if (status != kStatusOk) {
          done = true;
          walking = false;
          continue;
        }
        (void)need_pop;
        if (node == -1) walking = false;
      }
    }
    // ---- leaf phase: a mesh leaf, scanned in the reference's order (COOP:
    // the warp's leaves as one list of triangle tests, all lanes)
    const bool any_leaf = alive && !done && !walking && node < -1 && geom >= 0;
    int32_t cidx = -1;
    float cU = 0.f, cV = 0.f, cW = 0.f;
    if (COOP && MOT) {  // static and motion leaves in one cooperative list
      uint32_t first = 0, count = 0;
      const float4* t0 = mtris;
      const float4* t1 = mtris;
      float tm = 0.f, omt = 1.f, lo = lower;
      if (any_leaf) {
        leaf_decode(node, first, count);
        if (mmot) {
          const DMesh& M = top.meshes[geom];
          int key, key2;
          motion_keys(M.keys, r.time, tm, omt, key, key2);
          const float4* tr = reinterpret_cast<const float4*>(M.mtris);
          t0 = tr + (size_t)key * M.n_tris * 3;
          t1 = tr + (size_t)key2 * M.n_tris * 3;
          lo = M.ray_bias;
        }
      }
      cidx = coop_leaf_mix_dispatch(t0, t1, tm, omt, any_leaf && mmot, lo, r, any_leaf, first, count, cU, cV, cW);
    } else if (COOP) {
      uint32_t first = 0, count = 0;
      if (any_leaf) leaf_decode(node, first, count);
      cidx = coop_leaf_dispatch(mtris, lower, r, any_leaf, first, count, cU, cV, cW);
    }
    if (alive) {
      if (any_leaf) {
        uint32_t first, count;
        leaf_decode(node, first, count);
        float U = cU, V = cV, W = cW;
        int32_t idx = cidx;
        int32_t elem = idx;
        if (COOP && MOT && mmot) {  // scanned cooperatively: the leaf position to ElemID
          elem = idx != -1 ? __ldg(top.meshes[geom].elem + idx) : -1;
        } else if (MOT && mmot) {  // a motion leaf: vertices lerped at the ray's time, scanned by its lane
          const DMesh& M = top.meshes[geom];
          float tm, omt;
          int key, key2;
          motion_keys(M.keys, r.time, tm, omt, key, key2);
          const float4* tr = reinterpret_cast<const float4*>(M.mtris);
          idx = leaf_scan_dispatch<true>(M, r, first, count, tr + (size_t)key * M.n_tris * 3,
                                         tr + (size_t)key2 * M.n_tris * 3, tm, omt, U, V, W);
          elem = idx != -1 ? __ldg(M.elem + idx) : -1;
        } else if (!COOP) {
          DMesh M;
          M.lower_static = lower;
          idx = leaf_scan_dispatch<false>(M, r, first, count, mtris, mtris, 0.f, 1.f, U, V, W);
          elem = idx;
        }
        if (idx != -1) {
          h.elem = elem;
          h.geom = geom;
          h.u = U;
          h.v = V;
          h.w = W;
          hit = true;
        }
        if (ANY && idx != -1) {
          done = true;
        } else {
          // the rest of the mesh, then the leaf's next geom or the top level
          for (;;) {
            if (sp > base) {
              const int2 e = stk[--sp];
              node = e.x;
              nodeT = __int_as_float(e.y);
              break;
            }
            geom = -1;
            sp = base - 1;
            if (MOT && mxf) {  // back to the world ray (Tclosest kept)
              load_ray_pd(rays, li, r);
              mxf = false;
            }
            if (leaf_left > 0) {
              const uint32_t g = __ldg(top.geom_order + leaf_next);
              ++leaf_next;
              --leaf_left;
              const DMesh& MM = top.meshes[g];
              if (MM.kind == 1) {
                if (sphere_hit(MM, r, h)) {
                  h.geom = (int)g;
                  hit = true;
                  if (ANY) {
                    node = -1;
                    break;
                  }
                }
                continue;
              }
              if (MM.n_tris == 0) continue;
              if (MOT && MM.keys > 1 && !motion_keys(MM.keys, r.time, tm_unused, omt_unused, key_unused, key2_unused)) continue;
              base = sp + 1;
              geom = (int)g;
              mmot = MOT && MM.keys > 1;
              mxf = MOT && MM.has_xf;
              if (mxf) ray_to_object(r, MM.xf_inv);
              mnodes = MM.nodes;
              mtris = reinterpret_cast<const float4*>(MM.tris);
              lower = MM.lower_static;
              mcap = MM.iter_cap;
              miter = 0;
              sp = base;
              node = 0;
              nodeT = r.tclosest;
              break;
            }
            if (hit && ANY) {
              node = -1;
              break;
            }
            if (sp == 0) {
              node = -1;
              break;
            }
            const int2 e = stk[--sp];
            node = e.x;
            nodeT = __int_as_float(e.y);
            break;
          }
        }
      }
      if (!walking && node == -1) done = true;
      if (done) {
        store_hit(hits, rid, r, hit, h);
        alive = false;
        if (status != kStatusOk) {
          atomicMax(&scratch->status, status);
          status = kStatusOk;
        }
      }
    }
  }
}

// ------------------------------------------------------------------------
// Step-scheduled persistent kernel.  Each lane is IDLE, at an inner-node
// entry (NODE) or inside a leaf (LEAF, next triangle ti of [ti, tend)).  A
// step runs ONE node visit for the NODE lanes or ONE triangle test for the
// LEAF lanes, whichever group holds more lanes (one ballot per step), so a
// lane never waits for another lane's whole node walk or whole leaf.  Idle
// lanes are refilled once at least `refill_min` of them are idle.  Per ray
// the sequence of pops, visits, culls and triangle tests is the
// reference's.
enum LaneState : int { kIdle = 0, kNode = 1, kLeaf = 2 };

template <bool MOTION>
__device__ __forceinline__ bool test_tri(const DMesh& m, TRay& r, uint32_t i, const float4* tr0, const float4* tr1,
                                         float tm, float omt, float& U, float& V, float& W) {
  if (MOTION) {
    float4 a[3], c[3], v[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      a[j] = __ldg(tr0 + 3 * (size_t)i + j);
      c[j] = __ldg(tr1 + 3 * (size_t)i + j);
    }
#pragma unroll
    for (int j = 0; j < 3; ++j)  // Vec3Lerp (math/vec3.go:52-58)
      v[j] = make_float4(__fadd_rn(__fmul_rn(omt, a[j].x), __fmul_rn(tm, c[j].x)),
                         __fadd_rn(__fmul_rn(omt, a[j].y), __fmul_rn(tm, c[j].y)),
                         __fadd_rn(__fmul_rn(omt, a[j].z), __fmul_rn(tm, c[j].z)), 0.f);
    return tri_test<false>(r, v[0], v[1], v[2], m.ray_bias, U, V, W);
  }
  const float4 v0 = __ldg(tr0 + 3 * (size_t)i);
  const float4 v1 = __ldg(tr0 + 3 * (size_t)i + 1);
  const float4 v2 = __ldg(tr0 + 3 * (size_t)i + 2);
  return tri_test<true>(r, v0, v1, v2, m.lower_static, U, V, W);
}

template <bool MOTION, bool ANY, bool COUNT, bool PF>
__global__ void __launch_bounds__(256) k_trace_mesh_sched(const DMesh m, RaySoA rays, HitSoA hits, uint64_t n,
                                                          DScratch* scratch, int refill_min, const uint32_t* order) {
  int2 stk[kStackCapacity];
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lanes_below = (1u << lane) - 1u;
  TRay r;
  HitRec h{-1, -1, 0.f, 0.f, 0.f};
  int state = kIdle;
  int node = 0, sp = 0;
  float nodeT = 0.f;
  uint32_t ti = 0, tend = 0;
  uint64_t rid = 0;
  uint32_t iter = 0;
  bool hit = false, leafhit = false;
  bool more = true;
  int status = kStatusOk;
  Counters cnt{0, 0, 0};
  float tm = 0.f, omt = 1.f;
  const float4* bx0 = nullptr;
  const float4* bx1 = nullptr;
  const float4* tr0 = reinterpret_cast<const float4*>(MOTION ? m.mtris : m.tris);
  const float4* tr1 = tr0;
  for (;;) {
    const unsigned idle = __ballot_sync(kFull, state == kIdle);
    if (more && idle != 0u && (__popc(idle) >= refill_min || idle == kFull)) {
      const int leader = __ffs(idle) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) {
        base = atomicAdd(&scratch->next_ray, (unsigned long long)__popc(idle));
        if (*reinterpret_cast<volatile int*>(&scratch->status) != kStatusOk) base = n;
      }
      base = __shfl_sync(kFull, base, leader);
      if (base + __popc(idle) >= n) more = false;
      if (state == kIdle) {
        const uint64_t i = base + __popc(idle & lanes_below);
        if (i < n) {
          rid = order ? (uint64_t)__ldg(order + i) : i;
          load_ray(rays, i, r);
          h = HitRec{-1, -1, 0.f, 0.f, 0.f};
          hit = false;
          node = 0;
          nodeT = r.tclosest;
          sp = 0;
          iter = 0;
          state = kNode;
          if (MOTION) {
            const float k = __fmul_rn(r.time, (float)(m.keys - 1));
            const float fk = floorf(k);
            tm = __fsub_rn(k, fk);
            omt = __fsub_rn(1.0f, tm);
            const int key = (int)fk, key2 = (int)ceilf(k);
            if (key < 0 || key2 >= (int)m.keys) {
              store_hit(hits, rid, r, false, h);
              state = kIdle;
            } else {
              bx0 = reinterpret_cast<const float4*>(m.mboxes) + (size_t)key * m.n_mnodes * 6;
              bx1 = reinterpret_cast<const float4*>(m.mboxes) + (size_t)key2 * m.n_mnodes * 6;
              tr0 = reinterpret_cast<const float4*>(m.mtris) + (size_t)key * m.n_tris * 3;
              tr1 = reinterpret_cast<const float4*>(m.mtris) + (size_t)key2 * m.n_tris * 3;
            }
          }
        }
      }
    }
    const unsigned leafm = __ballot_sync(kFull, state == kLeaf);
    const unsigned nodem = __ballot_sync(kFull, state == kNode);
    if ((leafm | nodem) == 0u) {
      if (!more) break;
      continue;
    }
    bool finish = false;
    if (__popc(leafm) >= __popc(nodem)) {
      if (state == kLeaf) {
        float U, V, W;
        if (test_tri<MOTION>(m, r, ti, tr0, tr1, tm, omt, U, V, W)) {
          h.elem = MOTION ? __ldg(m.elem + ti) : (int32_t)ti;
          h.u = U;
          h.v = V;
          h.w = W;
          hit = true;
          leafhit = true;
        }
        if (++ti == tend) {
          if ((ANY && leafhit) || sp == 0) {
            finish = true;
          } else {
            const int2 e = stk[--sp];
            node = e.x;
            nodeT = __int_as_float(e.y);
            state = kNode;
            if (PF && !MOTION && node >= 0) prefetch_l1(m.nodes + node);
          }
        }
      }
    } else if (state == kNode) {
      if (++iter > m.iter_cap) {
        status = kStatusIterationCap;
        finish = true;
      } else if (r.tclosest < nodeT) {  // pop-time cull (intersect.go:106)
        if (sp == 0) {
          finish = true;
        } else {
          const int2 e = stk[--sp];
          node = e.x;
          nodeT = __int_as_float(e.y);
        }
      } else if (node < 0) {
        leaf_decode(node, ti, tend);
        if (PF && !MOTION) prefetch_leaf(tr0, ti, tend);
        tend += ti;
        leafhit = false;
        state = kLeaf;
        if (COUNT) { cnt.leafs++; cnt.tris += tend - ti; }
      } else {
        if (COUNT) cnt.nodes++;
        float4 b[6];
        int4 ch;
        unsigned rk;
        if (MOTION) fetch_mnode(m.mnodes, node, r.oct, bx0, bx1, tm, omt, b, ch, rk);
        else fetch_node(m, node, r.oct, b, ch, rk);
        float tn[4];
        unsigned mask = r.exact ? box4<true>(r, b, tn) : box4<false>(r, b, tn);
        if (ch.x == kEmptyChild || r.tclosest < tn[0]) mask &= ~1u;
        if (ch.y == kEmptyChild || r.tclosest < tn[1]) mask &= ~2u;
        if (ch.z == kEmptyChild || r.tclosest < tn[2]) mask &= ~4u;
        if (ch.w == kEmptyChild || r.tclosest < tn[3]) mask &= ~8u;
        int next = 0;
        float nextT = 0.f;
        if (push_ranked(stk, sp, mask, ch, tn, rk, next, nextT, status)) {
          node = next;
          nodeT = nextT;
        } else if (status != kStatusOk || sp == 0) {
          finish = true;
        } else {
          const int2 e = stk[--sp];
          node = e.x;
          nodeT = __int_as_float(e.y);
        }
      }
    }
    if (finish) {
      store_hit(hits, rid, r, hit, h);
      state = kIdle;
      if (status != kStatusOk) {
        atomicMax(&scratch->status, status);
        status = kStatusOk;
      }
    }
  }
  flush_counters<COUNT>(scratch, cnt);
}

template <class K>
int persistent_grid(K kernel, int block, int want_per_sm = 0) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
  if (per_sm < 1) per_sm = 1;
  if (want_per_sm > 0 && want_per_sm < per_sm) per_sm = want_per_sm;
  return sms * per_sm;
}

template <class K, class... A>
int launch_persistent(K k, const TraceLaunch& l, int block, A... args) {
  const int grid = persistent_grid(k, block, l.grid);
  k<<<grid, block, 0, (cudaStream_t)l.stream>>>(args...);
  return (int)cudaGetLastError();
}

// tuning.kernel: bit 0 = while-while (else step-scheduled), bit 1 = L1
// prefetch of the next node, bit 2 = 64-register cap (while-while, 128
// threads, 8 resident blocks), bit 3 = ray reordering (host side).
template <class K, class... A>
int launch_persistent_smem(K k, const TraceLaunch& l, int block, size_t smem, A... args) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessorWithFlags(&per_sm, k, block, smem, cudaOccupancyDefault);
  if (per_sm < 1) per_sm = 1;
  if (l.grid > 0 && l.grid < per_sm) per_sm = l.grid;
  k<<<sms * per_sm, block, smem, (cudaStream_t)l.stream>>>(args...);
  return (int)cudaGetLastError();
}

template <bool MOTION, bool ANY, bool COUNT, int MINB>
int launch_ww(const DMesh& mesh, const TraceLaunch& l, int block) {
  const int tail = l.walk_tail;
  if ((l.kernel & kKernelCoopLeaf) && !(l.kernel & (kKernelSharedStack | kKernelPrefetch)))
    return launch_persistent(k_trace_mesh_ww<MOTION, ANY, COUNT, false, MINB, 0, true>, l, block, mesh, l.rays, l.hits,
                             l.n, l.scratch, l.order, tail, l.n_dev);
  if (l.kernel & kKernelSharedStack) {
    constexpr int SS = kSharedStackEntries;
    return launch_persistent_smem(k_trace_mesh_ww<MOTION, ANY, COUNT, false, MINB, SS>, l, block,
                                  (size_t)SS * block * 8, mesh, l.rays, l.hits, l.n, l.scratch, l.order, tail, l.n_dev);
  }
  if (l.kernel & kKernelPrefetch)
    return launch_persistent(k_trace_mesh_ww<MOTION, ANY, COUNT, true, MINB, 0>, l, block, mesh, l.rays, l.hits, l.n,
                             l.scratch, l.order, tail, l.n_dev);
  return launch_persistent(k_trace_mesh_ww<MOTION, ANY, COUNT, false, MINB, 0>, l, block, mesh, l.rays, l.hits, l.n,
                           l.scratch, l.order, tail, l.n_dev);
}

template <bool MOTION, bool ANY, bool COUNT>
int launch_mesh_t(const DMesh& mesh, const TraceLaunch& l) {
  const int block = l.block > 0 ? l.block : 128;
  const int v = l.kernel;
  if (v & kKernelWhileWhile) {
    // the register cap: 7 resident blocks per SM (72 registers) for static
    // meshes (with the record fetch, 8 blocks at 64 registers spilled 108 B
    // and ran 5% slower); motion meshes hold both keys' boxes and vertices
    // and run fastest at 5 blocks (96 registers: 130 against 100 Mrays/s
    // at 8)
    if (v & kKernelRegCap) return launch_ww<MOTION, ANY, COUNT, MOTION ? 5 : 7>(mesh, l, 128);
    return launch_ww<MOTION, ANY, COUNT, 0>(mesh, l, block);
  }
  const int refill = l.refill_min > 0 ? l.refill_min : 4;
  if (v & kKernelPrefetch)
    return launch_persistent(k_trace_mesh_sched<MOTION, ANY, COUNT, true>, l, block, mesh, l.rays, l.hits, l.n, l.scratch, refill, l.order);
  return launch_persistent(k_trace_mesh_sched<MOTION, ANY, COUNT, false>, l, block, mesh, l.rays, l.hits, l.n, l.scratch, refill, l.order);
}

template <bool MOTION>
int launch_mesh_m(const DMesh& mesh, const TraceLaunch& l) {
  if (l.any_hit) return l.count ? launch_mesh_t<MOTION, true, true>(mesh, l) : launch_mesh_t<MOTION, true, false>(mesh, l);
  return l.count ? launch_mesh_t<MOTION, false, true>(mesh, l) : launch_mesh_t<MOTION, false, false>(mesh, l);
}

template <bool ANY, bool COUNT>
int launch_scene_t(const DTop& top, const TraceLaunch& l) {
  // Instances, Procs and keyed transforms are traced by the single-loop kernel.
  if (!COUNT && (l.kernel & kKernelWhileWhile) && !top.simple_only) {
    // Motion meshes and motion top levels take the MOT instantiation (lerped
    // node boxes, motion leaves in the cooperative phase with both keys'
    // vertices lerped); only-static scenes keep the leaner kernel.
    const bool coop = (l.kernel & kKernelCoopLeaf) != 0;
    auto k = top.all_static ? (coop ? k_trace_scene_ww<ANY, true, false> : k_trace_scene_ww<ANY, false, false>)
                            : (coop ? k_trace_scene_ww<ANY, true, true> : k_trace_scene_ww<ANY, false, true>);
    const int grid = persistent_grid(k, 128, l.grid);
    k<<<grid, 128, 0, (cudaStream_t)l.stream>>>(top, l.rays, l.hits, l.n, l.scratch, l.n_dev, l.order, l.walk_tail,
                                                l.ray_path, l.path_geom);
    return (int)cudaGetLastError();
  }
  auto k = k_trace_scene<ANY, COUNT>;
  const int block = 128;
  const int grid = persistent_grid(k, block, l.grid);  // l.grid: resident blocks per SM
  k<<<grid, block, 0, (cudaStream_t)l.stream>>>(top, l.rays, l.hits, l.n, l.scratch, l.n_dev, l.order,
                                                l.ray_path, l.path_geom);
  return (int)cudaGetLastError();
}

}  // namespace

int launch_trace_mesh(const DMesh& mesh, const TraceLaunch& l) {
  return mesh.keys > 1 ? launch_mesh_m<true>(mesh, l) : launch_mesh_m<false>(mesh, l);
}

int launch_trace_scene(const DTop& top, const TraceLaunch& l) {
  if (l.any_hit) return l.count ? launch_scene_t<true, true>(top, l) : launch_scene_t<true, false>(top, l);
  return l.count ? launch_scene_t<false, true>(top, l) : launch_scene_t<false, false>(top, l);
}

int launch_trace_jobs(const JobDesc* jobs, uint32_t n_jobs, uint64_t n_rays, const DTop& top, const JobWork& w,
                      TraceLaunch l) {
  if (n_jobs == 0 || n_rays == 0) return 0;
  cudaStream_t st = (cudaStream_t)l.stream;
  const int block = 256;
  const uint64_t want = (n_rays + block - 1) / block, cap = (uint64_t)device_sm_count() * 16;
  const int grid = (int)(want < cap ? want : cap);
  k_jobs_gather<<<grid, block, 0, st>>>(jobs, n_jobs, n_rays, w.rays, w.ray_job);
  int e = (int)cudaGetLastError();
  if (e != 0) return e;
  l.rays = w.rays;
  l.hits = w.hits;
  l.n = n_rays;
  l.ray_path = w.ray_job;
  l.path_geom = w.job_geom;
  e = launch_trace_scene(top, l);
  if (e != 0) return e;
  k_jobs_scatter<<<grid, block, 0, st>>>(jobs, n_jobs, n_rays, w.hits);
  return (int)cudaGetLastError();
}

int device_sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

}  // namespace vmr
