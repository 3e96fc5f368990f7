// orc_core.cpp - CPU oracle: QBVH build + traversal, watertight triangle test,
// motion traversal and the two-level scene.
//
// TEST INFRASTRUCTURE ONLY (see orc.h).  A scalar restatement of Vermeer's
// algorithms, written for readability and compiled with -ffp-contract=off.
// Every function names the reference file:line it restates.
#include "orc.h"
#include "orc_internal.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_err;

// ---------------------------------------------------------------- math ----
inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
const float kInf = bitsf(0x7f800000u);

// math.Min / math.Max (math/dim_amd64.s:8-21): MINSS/MAXSS with x in X0,
// y in X1, so Min(x,y) = x<y ? x : y and Max(x,y) = x>y ? x : y.  The
// operand order decides which argument a NaN or a signed-zero tie returns.
inline float gmin(float x, float y) { return x < y ? x : y; }
inline float gmax(float x, float y) { return x > y ? x : y; }
// math.Abs (math/abs.go:13-15): clear the sign bit.
inline float gabs(float x) { return bitsf(fbits(x) & 0x7fffffffu); }
// math.SignMask / Xorf (math/unsafe.go:15-37).
inline uint32_t signmask(float x) { return fbits(x) & 0x80000000u; }
inline float xorf(float x, uint32_t m) { return bitsf(fbits(x) ^ m); }

// math.EpsilonFloat32 (math/ferror.go:16): 1.19209290e-7 as float32 = 2^-23.
const float kEpsilonFloat32 = 1.19209290e-07f;

struct Vec3 { float v[3]; };

// math.BoundingBox (math/boundingbox.go:8-127).
struct Box { float b[2][3]; };
inline void box_reset(Box& b) {
  for (int i = 0; i < 3; ++i) { b.b[0][i] = kInf; b.b[1][i] = -kInf; }
}
// Grow (boundingbox.go:107-116): Min(X, box) operand order.
inline void box_grow(Box& b, const float* p) {
  b.b[0][0] = gmin(p[0], b.b[0][0]); b.b[1][0] = gmax(p[0], b.b[1][0]);
  b.b[0][1] = gmin(p[1], b.b[0][1]); b.b[1][1] = gmax(p[1], b.b[1][1]);
  b.b[0][2] = gmin(p[2], b.b[0][2]); b.b[1][2] = gmax(p[2], b.b[1][2]);
}
// GrowBox (boundingbox.go:99-104): Min(box, other) operand order.
inline void box_grow_box(Box& b, const Box& p) {
  for (int k = 0; k < 3; ++k) {
    b.b[0][k] = gmin(b.b[0][k], p.b[0][k]);
    b.b[1][k] = gmax(b.b[1][k], p.b[1][k]);
  }
}
inline float box_dim(const Box& b, int a) { return b.b[1][a] - b.b[0][a]; }
// SurfaceArea (boundingbox.go:17-19), evaluated left to right.
inline float box_area(const Box& b) {
  return box_dim(b, 0) * box_dim(b, 1) * 2.0f + box_dim(b, 1) * box_dim(b, 2) * 2.0f +
         box_dim(b, 0) * box_dim(b, 2) * 2.0f;
}
// LongestAxis (boundingbox.go:54-70).
inline int box_max_dim(const Box& b) {
  if (box_dim(b, 0) < box_dim(b, 1)) return box_dim(b, 1) < box_dim(b, 2) ? 2 : 1;
  return box_dim(b, 0) < box_dim(b, 2) ? 2 : 0;
}
// Centroid (boundingbox.go:27-32).
inline Vec3 box_centroid(const Box& b) {
  Vec3 o;
  for (int k = 0; k < 3; ++k) o.v[k] = (b.b[1][k] + b.b[0][k]) * 0.5f;
  return o;
}
// BoundingBoxLerp (boundingbox.go:119-127).
inline Box box_lerp(const Box& a, const Box& c, float t) {
  Box o;
  for (int i = 0; i < 2; ++i)
    for (int k = 0; k < 3; ++k) o.b[i][k] = (1 - t) * a.b[i][k] + t * c.b[i][k];
  return o;
}
// Vec3Lerp (math/vec3.go:52-58).
inline Vec3 vlerp(const float* a, const float* b, float t) {
  Vec3 o;
  for (int k = 0; k < 3; ++k) o.v[k] = (1.0f - t) * a[k] + t * b[k];
  return o;
}
const Box kInfBox = {{{kInf, kInf, kInf}, {kInf, kInf, kInf}}};  // boundingbox.go:14

// --------------------------------------------------------- QBVH build ----
// Node accessors (qbvh/qbvh.go:39-113).
inline void node_set_bounds(float* boxes, int idx, const Box& b) {
  for (int i = 0; i < 2; ++i)
    for (int k = 0; k < 3; ++k) boxes[idx + i * 12 + k * 4] = b.b[i][k];
}
inline Box node_bounds(const float* boxes, int idx) {
  Box b;
  for (int i = 0; i < 2; ++i)
    for (int k = 0; k < 3; ++k) b.b[i][k] = boxes[idx + i * 12 + k * 4];
  return b;
}
inline int32_t leaf_code(uint32_t first, uint32_t count) {  // SetLeaf qbvh.go:82-93
  uint32_t v = (1u << 31) | ((first << 4) & 0xfffffff0u) | ((count - 1) & 0xfu);
  return (int32_t)v;
}
inline int leaf_count(int32_t l) { return (int)((l & 0xf) + 1); }       // qbvh.go:61
inline int leaf_base(int32_t l) { return (int)((l & 0x7ffffff) >> 4); }  // qbvh.go:64

struct BuildErr {};

// calcMinCost (qbvh/build.go:28-136).  8 bins along the longest axis of
// the centroid bounds; partitions boxes/centroids/indxs in lock-step.
int calc_min_cost(const Box& bounds, Vec3* cent, Box* boxes, int32_t* indxs, int n,
                  int* pivot) {
  const int nbins = 8;
  Box bin_bounds[nbins];
  int32_t bin_n[nbins] = {0};
  int axis = box_max_dim(bounds);
  if (bounds.b[1][axis] == bounds.b[0][axis]) {  // flat centroid bounds (build.go:34-43)
    *pivot = n / 2 + 1;
    return axis;
  }
  // float32(nbins)*(1.0-0.00006) is a float32 constant: 8 * float32(0.99994).
  const float knum = 8.0f * 0.99994f;
  float k1 = knum / (bounds.b[1][axis] - bounds.b[0][axis]);
  float k0 = bounds.b[0][axis];
  for (int i = 0; i < nbins; ++i) box_reset(bin_bounds[i]);
  for (int i = 0; i < n; ++i) {
    float c = cent[i].v[axis];
    int bin = (int)(k1 * (c - k0));
    if (bin < 0 || bin > nbins - 1) {  // the reference panics here (build.go:57-66)
      g_err = "calcMinCost: bin out of range";
      throw BuildErr();
    }
    bin_n[bin]++;
    box_grow_box(bin_bounds[bin], boxes[i]);
  }
  Box lbox[nbins], rbox[nbins];
  int32_t ln[nbins], rn[nbins];
  Box box;
  box_reset(box);
  int32_t cnt = 0;
  for (int i = 0; i < nbins; ++i) {
    box_grow_box(box, bin_bounds[i]);
    cnt += bin_n[i];
    lbox[i] = box;
    ln[i] = cnt;
  }
  box_reset(box);
  cnt = 0;
  for (int i = 0; i < nbins; ++i) {
    box_grow_box(box, bin_bounds[nbins - 1 - i]);
    cnt += bin_n[nbins - 1 - i];
    rbox[nbins - 1 - i] = box;
    rn[nbins - 1 - i] = cnt;
  }
  int best = -1;
  float min_cost = kInf;
  for (int i = 1; i < nbins; ++i) {
    float cost = box_area(lbox[i - 1]) * (float)ln[i - 1] + box_area(rbox[i]) * (float)rn[i];
    if (cost < min_cost) { best = i; min_cost = cost; }
  }
  int left = 0, right = n - 1;
  while (left <= right) {
    float c = cent[left].v[axis];
    int bin = (int)(k1 * (c - k0));
    if (bin < best) {
      left++;
    } else {
      std::swap(indxs[left], indxs[right]);
      std::swap(cent[left], cent[right]);
      std::swap(boxes[left], boxes[right]);
      right--;
    }
  }
  *pivot = left;
  return axis;
}

Box calc_box(const Box* boxes, int n) {  // build.go:138-149
  Box b;
  box_reset(b);
  for (int i = 0; i < n; ++i) box_grow_box(b, boxes[i]);
  return b;
}

// binarySplit (build.go:151-178).
void binary_split(Box* boxes, Vec3* cent, int leaf_max, int32_t* indxs, int n, int* axis,
                  int* pivot) {
  Box bounds;
  box_reset(bounds);
  for (int i = 0; i < n; ++i) box_grow(bounds, cent[i].v);
  if (n <= leaf_max) { *axis = 0; *pivot = n; return; }
  *axis = calc_min_cost(bounds, cent, boxes, indxs, n, pivot);
}

// buildAccelRec (build.go:180-287) and buildAccelMotionRec
// (motionbuild.go:12-73) share the split logic; `motion` selects the node
// kind.  Nodes are appended in pre-order: a node gets its index after its
// three binary splits and before its children recurse.
struct TreeBuilder {
  std::vector<orc_node>* nodes = nullptr;
  std::vector<orc_mnode>* mnodes = nullptr;
  int leaf_max = 16;
  int depth = 0;

  int32_t rec(Box* boxes, Vec3* cent, int32_t* indxs, int n, int baseidx, Box* nodebox) {
    if (++depth > 4096) { g_err = "QBVH build recursion does not terminate"; throw BuildErr(); }
    int axis0, pivot0, axis1, pivot1, axis2, pivot2;
    binary_split(boxes, cent, leaf_max, indxs, n, &axis0, &pivot0);
    binary_split(boxes, cent, leaf_max, indxs, pivot0, &axis1, &pivot1);
    binary_split(boxes + pivot0, cent + pivot0, leaf_max, indxs + pivot0, n - pivot0, &axis2,
                 &pivot2);
    int32_t nodei;
    if (mnodes) {
      nodei = (int32_t)mnodes->size();
      orc_mnode mn;
      std::memset(&mn, 0, sizeof(mn));
      mn.axis0 = axis0; mn.axis1 = axis1; mn.axis2 = axis2;
      mnodes->push_back(mn);
    } else {
      nodei = (int32_t)nodes->size();
      orc_node nd;
      std::memset(&nd, 0, sizeof(nd));
      nd.axis0 = (uint32_t)axis0; nd.axis1 = (uint32_t)axis1; nd.axis2 = (uint32_t)axis2;
      nodes->push_back(nd);
    }
    const int starts[4] = {0, pivot1, pivot0, pivot0 + pivot2};
    const int ends[4] = {pivot1, pivot0, pivot0 + pivot2, n};
    for (int c = 0; c < 4; ++c) {
      int s = starts[c], len = ends[c] - starts[c];
      if (len <= leaf_max) {
        if (mnodes) {
          (*mnodes)[nodei].children[c] = len == 0 ? -1 : leaf_code((uint32_t)(baseidx + s), (uint32_t)len);
        } else {
          orc_node& nd = (*nodes)[nodei];
          node_set_bounds(nd.boxes, c, calc_box(boxes + s, len));
          if (len == 0) {  // SetEmptyLeaf (qbvh.go:67-79) overwrites the bounds
            nd.children[c] = -1;
            node_set_bounds(nd.boxes, c, kInfBox);
          } else {
            nd.children[c] = leaf_code((uint32_t)(baseidx + s), (uint32_t)len);
          }
        }
      } else {
        Box cb;
        int32_t child = rec(boxes + s, cent + s, indxs + s, len, baseidx + s, &cb);
        if (mnodes) {
          (*mnodes)[nodei].children[c] = child;
        } else {
          node_set_bounds((*nodes)[nodei].boxes, c, cb);
          (*nodes)[nodei].children[c] = child;
        }
      }
    }
    if (nodebox && !mnodes) {  // build.go:276-283: union of the non-empty children
      box_reset(*nodebox);
      for (int i = 0; i < 4; ++i)
        if ((*nodes)[nodei].children[i] != -1) box_grow_box(*nodebox, node_bounds((*nodes)[nodei].boxes, i));
    }
    --depth;
    return nodei;
  }
};

// --------------------------------------------------------------- rays ----
// core.Ray (core/ray.go:27-51), only the fields the traversal reads.
struct Ray {
  float P[3], D[3], Dinv[3];
  float Tclosest;
  float S[3];
  int Kx, Ky, Kz;
  float Time;
  bool shadow;
};

// Ray.Setup (core/ray.go:103-148).  float32(float64(a)/float64(b)) is the
// correctly rounded float32 quotient, so the double division is kept.
void ray_setup(Ray& r) {
  r.Kz = 0;
  if (gabs(r.D[1]) > gabs(r.D[2])) {
    if (gabs(r.D[1]) > gabs(r.D[0])) r.Kz = 1;
  } else {
    if (gabs(r.D[2]) > gabs(r.D[0])) r.Kz = 2;
  }
  r.Kx = r.Kz + 1;
  if (r.Kx == 3) r.Kx = 0;
  r.Ky = r.Kx + 1;
  if (r.Ky == 3) r.Ky = 0;
  if (r.D[r.Kz] < 0.0f) std::swap(r.Kx, r.Ky);
  double z = (double)r.D[r.Kz];
  r.S[2] = (float)(1.0 / z);
  r.S[0] = (float)((double)r.D[r.Kx] / z);
  r.S[1] = (float)((double)r.D[r.Ky] / z);
  for (int k = 0; k < 3; ++k) r.Dinv[k] = (float)(1.0 / (double)r.D[k]);
}

Ray make_ray(const float* in, bool shadow) {
  Ray r;
  for (int k = 0; k < 3; ++k) { r.P[k] = in[k]; r.D[k] = in[3 + k]; }
  r.Tclosest = in[6];
  r.Time = in[7];
  r.shadow = shadow;
  ray_setup(r);
  return r;
}

// Per-ray traversal state: RenderTask.Traversal (core/ray.go:152-166).
const int kStackSize = 90;
struct Task {
  struct { float T; int32_t Node; } stack[kStackSize];
  int stack_top = 0;  // Traversal.StackTop
  bool overflow = false;
  uint32_t nodes_t = 0, leafs_t = 0, tris_t = 0;
  // ShaderContext fields the trace fills.
  int32_t elem = -1;
  int32_t geom = -1;
  float bu = 0, bv = 0, bw = 0;
};

// intersectBoxes (qbvh/intersect_amd64.s:13-100), SSE operand order:
// lo = MINPS(t2,t1) = t2<t1?t2:t1, hi = MAXPS(t2,t1) = t2>t1?t2:t1; the y and
// z slabs fold in with MAXPS(lo,ylo) and MINPS(hi,yhi); tNear = MAXPS(0,lo);
// hit = CMPPS LE (tNear <= hi), an ordered compare (NaN = miss).
void intersect_boxes(const Ray& r, const float* bx, int32_t hits[4], float t[4]) {
  for (int i = 0; i < 4; ++i) {
    float x1 = (bx[i + 0] - r.P[0]) * r.Dinv[0];
    float x2 = (bx[i + 12] - r.P[0]) * r.Dinv[0];
    float lo = x2 < x1 ? x2 : x1;
    float hi = x2 > x1 ? x2 : x1;
    float y1 = (bx[i + 4] - r.P[1]) * r.Dinv[1];
    float y2 = (bx[i + 16] - r.P[1]) * r.Dinv[1];
    float ylo = y2 < y1 ? y2 : y1;
    float yhi = y2 > y1 ? y2 : y1;
    lo = lo > ylo ? lo : ylo;
    hi = hi < yhi ? hi : yhi;
    float z1 = (bx[i + 8] - r.P[2]) * r.Dinv[2];
    float z2 = (bx[i + 20] - r.P[2]) * r.Dinv[2];
    float zlo = z2 < z1 ? z2 : z1;
    float zhi = z2 > z1 ? z2 : z1;
    lo = lo > zlo ? lo : zlo;
    hi = hi < zhi ? hi : zhi;
    float tn = 0.0f > lo ? 0.0f : lo;
    t[i] = tn;
    hits[i] = (tn <= hi) ? -1 : 0;
  }
}

// ---------------------------------------------------------------- mesh ----
struct Mesh {
  uint32_t nverts = 0, keys = 1, ntris = 0;
  std::vector<float> verts;     // keys * nverts * 3
  std::vector<uint32_t> idxp;   // leaf order (static) / original order (motion)
  std::vector<int32_t> accel_idx;
  float ray_bias = 0.0f;
  bool motion_fixed = false;
  std::vector<orc_node> nodes;  // static
  std::vector<orc_mnode> mnodes;                // motion topology
  std::vector<std::vector<float>> mboxes;       // [key][node*24]
  std::vector<Box> motion_bounds;
  Box bounds;
  std::vector<uint8_t> shaderidx;  // leaf order (static) / face order (motion)
  std::vector<float> normals;      // per vertex, key 0
  // PolyMesh.Normals with as many keys as the vertices (motion meshes):
  // [key][mnormals_per_key][3], read at ElemID*3 + corner
  std::vector<float> mnormals;
  uint32_t mnormals_per_key = 0;
  // An analytic sphere geom (builtin/geom/sphere) instead of triangles.
  bool sphere = false;
  float sc[3] = {0, 0, 0}, sr = 0;
  // PolyMesh.Transform (one matrix, column-major) and Matrix4Inverse of it
  bool has_xf = false;
  float xf[16] = {}, xinv[16] = {};
  // PolyMesh.Transform of two or more keys, decomposed (init.go:14-16)
  std::vector<orc_internal::Decomp> xkeys;
  // A GeomInstance (group 1, builtin/geom/instance) or Proc (group 2,
  // builtin/geom/proc): its transform keys (always decomposed), its given
  // bounds (BMin/BMax of key 0), the geoms it traces and, for a Proc, the id
  // each child's hits report.
  int group = 0;
  std::vector<orc_internal::Decomp> gkeys;
  std::vector<const Mesh*> children;
  std::vector<int32_t> child_ids;
  Box user_bounds;
  // Set on a Proc's children: the Proc's transform keys (used in shading).
  const std::vector<orc_internal::Decomp>* outer = nullptr;

  const float* vert(uint32_t i, int key) const { return &verts[((size_t)key * nverts + i) * 3]; }
  int motion_keys() const {  // polymesh.go:103-112; a sphere has one key (sphere.go:58-60)
    if (group == 1) return children[0]->motion_keys();  // Instance.MotionKeys (instance.go:144-148)
    if (group == 2) return (int)gkeys.size();           // Proc.MotionKeys (proc.go:181-185)
    if (sphere) return 1;
    return nodes.empty() ? (int)mboxes.size() : 1;
  }
  // PolyMesh.Bounds (builtin/geom/polymesh/bounds.go:25-53); an instance or
  // a Proc returns its key-0 bounds at every time (instance.go:64-68).
  Box bounds_at(float time) const {
    if (group) return user_bounds;
    if (!nodes.empty() || mboxes.empty()) return bounds;
    float k = time * (float)(motion_bounds.size() - 1);
    float t = k - std::floor(k);
    int key = (int)std::floor(k), key2 = (int)std::ceil(k);
    return box_lerp(motion_bounds[key], motion_bounds[key2], t);
  }
};

// initMotionBoxesRec (buildqbvh.go:159-212).
Box mesh_motion_boxes_rec(Mesh& m, int key, int32_t node) {
  Box nodebox;
  box_reset(nodebox);
  for (int k = 0; k < 4; ++k) {
    int32_t ch = m.mnodes[node].children[k];
    if (ch < 0) {
      if (ch == -1) continue;
      Box box;
      box_reset(box);
      int base = leaf_base(ch), cnt = leaf_count(ch);
      for (int i = base; i < base + cnt; ++i) {
        int faceidx = m.accel_idx[i];
        for (int j = 0; j < 3; ++j) box_grow(box, m.vert(m.idxp[faceidx * 3 + j], key));
      }
      node_set_bounds(&m.mboxes[key][(size_t)node * 24], k, box);
      box_grow_box(nodebox, box);
    } else {
      Box box = mesh_motion_boxes_rec(m, key, ch);
      node_set_bounds(&m.mboxes[key][(size_t)node * 24], k, box);
      box_grow_box(nodebox, box);
    }
  }
  return nodebox;
}

// PolyMesh.initAccel (builtin/geom/polymesh/buildqbvh.go:14-144).
void mesh_init_accel(Mesh& m) {
  uint32_t n = m.ntris;
  std::vector<Box> boxes(n);
  std::vector<Vec3> cent(n);
  std::vector<int32_t> idxs(n);
  if (m.keys > 1) {
    float k = 0.5f * (float)(m.keys - 1);
    float time = k - std::floor(k);
    int key = (int)std::floor(k), key2 = (int)std::ceil(k);
    for (uint32_t i = 0; i < n; ++i) {
      Vec3 V[3];
      for (int j = 0; j < 3; ++j) V[j] = vlerp(m.vert(m.idxp[i * 3 + j], key), m.vert(m.idxp[i * 3 + j], key2), time);
      box_reset(boxes[i]);
      for (int j = 0; j < 3; ++j) box_grow(boxes[i], V[j].v);
      for (int c = 0; c < 3; ++c) cent[i].v[c] = (V[0].v[c] + V[1].v[c] + V[2].v[c]) / 3.0f;
      idxs[i] = (int32_t)i;
    }
    TreeBuilder tb;
    tb.mnodes = &m.mnodes;
    tb.leaf_max = 16;
    if (n > 0) tb.rec(boxes.data(), cent.data(), idxs.data(), (int)n, 0, nullptr);
    m.accel_idx = idxs;
    // initMotionBoxes (buildqbvh.go:148-169)
    m.mboxes.assign(m.keys, std::vector<float>(m.mnodes.size() * 24, 0.0f));
    Box full;
    box_reset(full);
    for (uint32_t kk = 0; kk < m.keys; ++kk) {
      Box b = mesh_motion_boxes_rec(m, (int)kk, 0);
      m.motion_bounds.push_back(b);
      box_grow_box(full, b);
    }
    m.bounds = full;
    return;
  }
  for (uint32_t i = 0; i < n; ++i) {
    const float* V0 = m.vert(m.idxp[i * 3 + 0], 0);
    const float* V1 = m.vert(m.idxp[i * 3 + 1], 0);
    const float* V2 = m.vert(m.idxp[i * 3 + 2], 0);
    box_reset(boxes[i]);
    box_grow(boxes[i], V0);
    box_grow(boxes[i], V1);
    box_grow(boxes[i], V2);
    for (int c = 0; c < 3; ++c) cent[i].v[c] = (V0[c] + V1[c] + V2[c]) / 3.0f;
    idxs[i] = (int32_t)i;
  }
  TreeBuilder tb;
  tb.nodes = &m.nodes;
  tb.leaf_max = 16;
  Box bounds;
  box_reset(bounds);
  if (n > 0) tb.rec(boxes.data(), cent.data(), idxs.data(), (int)n, 0, &bounds);
  m.bounds = bounds;
  m.accel_idx = idxs;
  std::vector<uint32_t> idxp(m.idxp.size());
  for (uint32_t i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) idxp[i * 3 + j] = m.idxp[(size_t)idxs[i] * 3 + j];
  m.idxp.swap(idxp);
}

// The watertight test shared by all three TraceElems variants
// (builtin/geom/polymesh/trace.go:123-193, :202-269, :556-623).  `strict`
// selects the lower bound: true = the static idxp path
// (xT < (EpsilonFloat32+RayBias)*xdet, trace.go:182), false = the motion
// path (xT <= RayBias*xdet, trace.go:612).  Returns true and updates the ray
// when the triangle is accepted.
inline bool tri_test(Ray& r, const float* V0, const float* V1, const float* V2, float lower,
                     bool strict, float* U, float* V, float* W) {
  const int Kx = r.Kx, Ky = r.Ky, Kz = r.Kz;
  float AKz = V0[Kz] - r.P[Kz];
  float BKz = V1[Kz] - r.P[Kz];
  float CKz = V2[Kz] - r.P[Kz];
  float Cx = (V2[Kx] - r.P[Kx]) - r.S[0] * CKz;
  float By = (V1[Ky] - r.P[Ky]) - r.S[1] * BKz;
  float Cy = (V2[Ky] - r.P[Ky]) - r.S[1] * CKz;
  float Bx = (V1[Kx] - r.P[Kx]) - r.S[0] * BKz;
  float Ax = (V0[Kx] - r.P[Kx]) - r.S[0] * AKz;
  float Ay = (V0[Ky] - r.P[Ky]) - r.S[1] * AKz;
  float fU = Cx * By - Cy * Bx;
  float fV = Ax * Cy - Ay * Cx;
  float fW = Bx * Ay - By * Ax;
  if (fU == 0.0f || fV == 0.0f || fW == 0.0f) {  // FP64 edge fallback (trace.go:142-155)
    double CxBy = (double)Cx * (double)By;
    double CyBx = (double)Cy * (double)Bx;
    fU = (float)(CxBy - CyBx);
    double AxCy = (double)Ax * (double)Cy;
    double AyCx = (double)Ay * (double)Cx;
    fV = (float)(AxCy - AyCx);
    double BxAy = (double)Bx * (double)Ay;
    double ByAx = (double)By * (double)Ax;
    fW = (float)(BxAy - ByAx);
  }
  if ((fU < 0.0f || fV < 0.0f || fW < 0.0f) && (fU > 0.0f || fV > 0.0f || fW > 0.0f)) return false;
  float det = fU + fV + fW;
  if (det == 0.0f) return false;
  float T = r.S[2] * (fU * AKz + fV * BKz + fW * CKz);
  uint32_t ds = signmask(det);
  float xT = xorf(T, ds), xdet = xorf(det, ds);
  bool below = strict ? (xT < lower * xdet) : (xT <= lower * xdet);
  if (below || xT > r.Tclosest * xdet) return false;
  float rcp = 1.0f / det;
  *U = fU * rcp;
  *V = fV * rcp;
  *W = fW * rcp;
  r.Tclosest = T * rcp;
  return true;
}

// PolyMesh.TraceElems, idxp path (trace.go:108-194).  Every mesh holds idxp
// after init (init.go:12-134), so the non-idxp branch is never taken.
bool mesh_trace_elems(const Mesh& m, Ray& r, Task& tk, int base, int count) {
  int32_t idx = -1;
  float U = 0, V = 0, W = 0;
  const float lower = kEpsilonFloat32 + m.ray_bias;
  tk.tris_t += (uint32_t)count;
  for (int i = base; i < base + count; ++i) {
    const float* V0 = m.vert(m.idxp[i * 3 + 0], 0);
    const float* V1 = m.vert(m.idxp[i * 3 + 1], 0);
    const float* V2 = m.vert(m.idxp[i * 3 + 2], 0);
    if (tri_test(r, V0, V1, V2, lower, true, &U, &V, &W)) idx = i;
  }
  if (idx == -1) return false;
  tk.elem = idx;
  tk.bu = U; tk.bv = V; tk.bw = W;
  return true;
}

// PolyMesh.TraceMotionElems (trace.go:520-719).  Faithful mode reads idxp at
// the leaf position (the reference; idxp is not reordered for motion
// meshes, trace.go:532-537); fixed mode maps the position through accel
// idx first, which is the face the leaf boxes were built from
// (buildqbvh.go:190-195).
bool mesh_trace_motion_elems(const Mesh& m, float time, int key, int key2, Ray& r, Task& tk,
                             int base, int count) {
  int32_t idx = -1;
  float U = 0, V = 0, W = 0;
  tk.tris_t += (uint32_t)count;
  for (int i = base; i < base + count; ++i) {
    int32_t face = m.motion_fixed ? m.accel_idx[i] : (int32_t)i;
    uint32_t i0 = m.idxp[(size_t)face * 3 + 0], i1 = m.idxp[(size_t)face * 3 + 1], i2 = m.idxp[(size_t)face * 3 + 2];
    Vec3 V0 = vlerp(m.vert(i0, key), m.vert(i0, key2), time);
    Vec3 V1 = vlerp(m.vert(i1, key), m.vert(i1, key2), time);
    Vec3 V2 = vlerp(m.vert(i2, key), m.vert(i2, key2), time);
    if (tri_test(r, V0.v, V1.v, V2.v, m.ray_bias, false, &U, &V, &W)) idx = face;
  }
  if (idx == -1) return false;
  tk.elem = idx;
  tk.bu = U; tk.bv = V; tk.bw = W;
  return true;
}

// qbvh.Trace (qbvh/intersect.go:91-246).  `leaf` is the Primitive callback.
// The stack is written exactly as the reference does: all four child slots
// are written at stackTop and stackTop advances only for hit children.
template <class Leaf>
bool qbvh_trace(const orc_node* q, Ray& r, Task& tk, Leaf&& leaf) {
  int stackTop = tk.stack_top;
  if (stackTop >= kStackSize) { tk.overflow = true; return false; }
  tk.stack[stackTop].Node = 0;
  tk.stack[stackTop].T = r.Tclosest;
  bool hit = false;
  stackTop++;
  int32_t hits[4];
  float tt[4];
  while (stackTop > tk.stack_top) {
    stackTop--;
    int32_t node = tk.stack[stackTop].Node;
    if (r.Tclosest < tk.stack[stackTop].T || node == -1) continue;
    if (node >= 0) {
      tk.nodes_t++;
      const orc_node& nd = q[node];
      intersect_boxes(r, nd.boxes, hits, tt);
      int order[4];
      // intersect.go:137-216: pairs (0,1) and (2,3), each ordered by the sign
      // of D along the pair's split axis; the pair order by D[Axis0].
      int p01a = r.D[nd.axis1] < 0 ? 0 : 1, p01b = 1 - p01a;
      int p23a = r.D[nd.axis2] < 0 ? 2 : 3, p23b = 5 - p23a;
      if (r.D[nd.axis0] < 0) {
        order[0] = p01a; order[1] = p01b; order[2] = p23a; order[3] = p23b;
      } else {
        order[0] = p23a; order[1] = p23b; order[2] = p01a; order[3] = p01b;
      }
      for (int j = 0; j < 4; ++j) {
        int c = order[j];
        if (stackTop >= kStackSize) { tk.overflow = true; return hit; }
        tk.stack[stackTop].Node = nd.children[c];
        tk.stack[stackTop].T = tt[c];
        stackTop -= hits[c];
      }
    } else {
      tk.leafs_t++;
      int tmp = tk.stack_top;
      tk.stack_top = stackTop + 1;
      bool h = leaf(r, tk, leaf_base(node), leaf_count(node));
      tk.stack_top = tmp;
      if (tk.overflow) return hit;
      if (h) {
        hit = true;
        if (r.shadow) return true;
      }
    }
  }
  return hit;
}

// qbvh.TraceMotion (qbvh/motionintersect.go:22-127).  The node boxes are
// lerped per float between the two keys before the slab test.
template <class Leaf>
bool qbvh_trace_motion(const orc_mnode* nodes, const std::vector<std::vector<float>>& boxes,
                       float time, int key, int key2, Ray& r, Task& tk, Leaf&& leaf) {
  int stackTop = tk.stack_top;
  if (stackTop >= kStackSize) { tk.overflow = true; return false; }
  tk.stack[stackTop].Node = 0;
  tk.stack[stackTop].T = r.Tclosest;
  bool hit = false;
  int32_t hits[4];
  float tt[4];
  float bx[24];
  while (stackTop >= tk.stack_top) {
    int32_t node = tk.stack[stackTop].Node;
    float T = tk.stack[stackTop].T;
    stackTop--;
    if (r.Tclosest < T) node = -1;
    if (node >= 0) {
      tk.nodes_t++;
      const orc_mnode& nd = nodes[node];
      const float* b0 = &boxes[key][(size_t)node * 24];
      const float* b1 = &boxes[key2][(size_t)node * 24];
      for (int i = 0; i < 24; ++i) bx[i] = (1.0f - time) * b0[i] + time * b1[i];
      intersect_boxes(r, bx, hits, tt);
      int order[4] = {0, 1, 2, 3};
      if (r.D[nd.axis0] < 0) {
        if (r.D[nd.axis2] < 0) { order[3] = 3; order[2] = 2; } else { order[3] = 2; order[2] = 3; }
        if (r.D[nd.axis1] < 0) { order[1] = 1; order[0] = 0; } else { order[1] = 0; order[0] = 1; }
      } else {
        if (r.D[nd.axis2] < 0) { order[1] = 3; order[0] = 2; } else { order[1] = 2; order[0] = 3; }
        if (r.D[nd.axis1] < 0) { order[3] = 1; order[2] = 0; } else { order[3] = 0; order[2] = 1; }
      }
      for (int j = 0; j < 4; ++j) {
        int c = order[j];
        if (hits[c] != 0) {
          stackTop++;
          if (stackTop >= kStackSize) { tk.overflow = true; return hit; }
          tk.stack[stackTop].Node = nd.children[c];
          tk.stack[stackTop].T = tt[c];
        }
      }
    } else if (node < -1) {
      tk.leafs_t++;
      int tmp = tk.stack_top;
      tk.stack_top = stackTop + 1;
      bool h = leaf(r, tk, leaf_base(node), leaf_count(node));
      tk.stack_top = tmp;
      if (tk.overflow) return hit;
      if (h) {
        hit = true;
        if (r.shadow) return true;
      }
    }
  }
  return hit;
}

// PolyMesh.Trace without a transform (trace.go:57-101).
// solveQuadratic and raySphereIntersect (builtin/geom/sphere/trace.go).
bool ray_sphere(const float Ro[3], const float Rd[3], const float P[3], float radius, float& t) {
  const float L[3] = {Ro[0] - P[0], Ro[1] - P[1], Ro[2] - P[2]};
  const float a = Rd[0] * Rd[0] + Rd[1] * Rd[1] + Rd[2] * Rd[2];
  const float b = 2 * (Rd[0] * L[0] + Rd[1] * L[1] + Rd[2] * L[2]);
  const float c = (L[0] * L[0] + L[1] * L[1] + L[2] * L[2]) - radius * radius;
  float x0, x1;
  const float discr = b * b - 4 * a * c;
  if (discr < 0) return false;
  if (discr == 0) {
    x1 = -0.5f * b / a;
    x0 = x1;
  } else {
    const float q = b > 0 ? -0.5f * (b + std::sqrt(discr)) : -0.5f * (b - std::sqrt(discr));
    x0 = q / a;
    x1 = c / q;
  }
  if (x0 > x1) std::swap(x0, x1);
  if (x0 > x1) std::swap(x0, x1);  // raySphereIntersect orders them again
  if (x0 < 0) {
    x0 = x1;
    if (x0 < 0) return false;
  }
  t = x0;
  return true;
}

// Sphere.Trace (sphere/trace.go): the closest root if below Tclosest.
bool sphere_trace(const Mesh& m, Ray& r, Task& tk) {
  float t;
  if (!ray_sphere(r.P, r.D, m.sc, m.sr, t)) return false;
  if (!(t < r.Tclosest)) return false;
  r.Tclosest = t;
  tk.elem = 0;
  tk.bu = tk.bv = tk.bw = 0.0f;
  return true;
}

bool mesh_trace(const Mesh& m, Ray& r, Task& tk) {
  if (m.sphere) return sphere_trace(m, r, tk);
  if (!m.nodes.empty()) {
    return qbvh_trace(m.nodes.data(), r, tk, [&](Ray& rr, Task& t, int b, int c) {
      return mesh_trace_elems(m, rr, t, b, c);
    });
  }
  if (m.mnodes.empty()) return false;
  float k = r.Time * (float)(m.keys - 1);
  float time = k - std::floor(k);
  int key = (int)std::floor(k), key2 = (int)std::ceil(k);
  if (key < 0 || key2 >= (int)m.keys) return false;  // the reference would index out of range
  return qbvh_trace_motion(m.mnodes.data(), m.mboxes, time, key, key2, r, tk,
                           [&](Ray& rr, Task& t, int b, int c) {
                             return mesh_trace_motion_elems(m, time, key, key2, rr, t, b, c);
                           });
}

// ---------------------------------------------------------------- scene ---
struct Scene {
  std::vector<Mesh*> geoms;          // leaf order
  std::vector<int32_t> geom_order;   // leaf position -> index passed at creation
  std::vector<orc_node> nodes;
  std::vector<orc_mnode> mnodes;
  std::vector<std::vector<float>> mboxes;
  int keys = 1;
};

// Scene.initMotionBoxesRec (builtin/scene/scene.go:228-268).
Box scene_motion_boxes_rec(Scene& s, int key, int32_t node) {
  Box nodebox;
  box_reset(nodebox);
  for (int k = 0; k < 4; ++k) {
    int32_t ch = s.mnodes[node].children[k];
    if (ch < 0) {
      if (ch == -1) continue;
      Box box;
      box_reset(box);
      int base = leaf_base(ch), cnt = leaf_count(ch);
      for (int i = base; i < base + cnt; ++i) {
        float time = (float)key / (float)(s.mboxes.size() - 1);
        box_grow_box(box, s.geoms[i]->bounds_at(time));
      }
      node_set_bounds(&s.mboxes[key][(size_t)node * 24], k, box);
      box_grow_box(nodebox, box);
    } else {
      Box box = scene_motion_boxes_rec(s, key, ch);
      node_set_bounds(&s.mboxes[key][(size_t)node * 24], k, box);
      box_grow_box(nodebox, box);
    }
  }
  return nodebox;
}

// Scene.initAccel (builtin/scene/scene.go:135-203), leafMax 1.
void scene_init(Scene& s, Mesh* const* meshes, uint32_t n) {
  int max_keys = 0;
  for (uint32_t i = 0; i < n; ++i) max_keys = std::max(max_keys, meshes[i]->motion_keys());
  std::vector<Box> boxes(n);
  std::vector<Vec3> cent(n);
  std::vector<int32_t> idx(n);
  float t0 = max_keys == 1 ? 0.0f : 0.5f;
  for (uint32_t i = 0; i < n; ++i) {
    boxes[i] = meshes[i]->bounds_at(t0);
    cent[i] = box_centroid(boxes[i]);
    idx[i] = (int32_t)i;
  }
  TreeBuilder tb;
  tb.leaf_max = 1;
  if (max_keys == 1) {
    tb.nodes = &s.nodes;
    Box b;
    if (n > 0) tb.rec(boxes.data(), cent.data(), idx.data(), (int)n, 0, &b);
  } else {
    tb.mnodes = &s.mnodes;
    if (n > 0) tb.rec(boxes.data(), cent.data(), idx.data(), (int)n, 0, nullptr);
  }
  s.geom_order = idx;
  for (uint32_t i = 0; i < n; ++i) s.geoms.push_back(meshes[idx[i]]);
  s.keys = max_keys;
  if (max_keys > 1) {
    s.mboxes.assign(max_keys, std::vector<float>(s.mnodes.size() * 24, 0.0f));
    for (int k = 0; k < max_keys; ++k) scene_motion_boxes_rec(s, k, 0);
  }
}

// math.Matrix4Inverse (math/matrix4.go:116-160).  Each adjugate element is
// six signed triple products in the order listed (one string per element:
// sign and three matrix indices per term); each product rounds as
// (m[a]*m[b])*m[c] and the terms add left to right, in float32.
void matrix4_inverse(const float m[16], float c[16]) {
  static const char* kTerms[16] = {
      "+5,10,15 -5,11,14 -9,6,15 +9,7,14 +13,6,11 -13,7,10",   // 0
      "-1,10,15 +1,11,14 +9,2,15 -9,3,14 -13,2,11 +13,3,10",   // 1
      "+1,6,15 -1,7,14 -5,2,15 +5,3,14 +13,2,7 -13,3,6",       // 2
      "-1,6,11 +1,7,10 +5,2,11 -5,3,10 -9,2,7 +9,3,6",         // 3
      "-4,10,15 +4,11,14 +8,6,15 -8,7,14 -12,6,11 +12,7,10",   // 4
      "+0,10,15 -0,11,14 -8,2,15 +8,3,14 +12,2,11 -12,3,10",   // 5
      "-0,6,15 +0,7,14 +4,2,15 -4,3,14 -12,2,7 +12,3,6",       // 6
      "+0,6,11 -0,7,10 -4,2,11 +4,3,10 +8,2,7 -8,3,6",         // 7
      "+4,9,15 -4,11,13 -8,5,15 +8,7,13 +12,5,11 -12,7,9",     // 8
      "-0,9,15 +0,11,13 +8,1,15 -8,3,13 -12,1,11 +12,3,9",     // 9
      "+0,5,15 -0,7,13 -4,1,15 +4,3,13 +12,1,7 -12,3,5",       // 10
      "-0,5,11 +0,7,9 +4,1,11 -4,3,9 -8,1,7 +8,3,5",           // 11
      "-4,9,14 +4,10,13 +8,5,14 -8,6,13 -12,5,10 +12,6,9",     // 12
      "+0,9,14 -0,10,13 -8,1,14 +8,2,13 +12,1,10 -12,2,9",     // 13
      "-0,5,14 +0,6,13 +4,1,14 -4,2,13 -12,1,6 +12,2,5",       // 14
      "+0,5,10 -0,6,9 -4,1,10 +4,2,9 +8,1,6 -8,2,5",           // 15
  };
  float inv[16];
  for (int e = 0; e < 16; ++e) {
    const char* p = kTerms[e];
    float acc = 0.0f;
    for (int k = 0; k < 6; ++k) {
      while (*p == ' ') ++p;
      const bool neg = *p++ == '-';
      int idx[3];
      for (int q = 0; q < 3; ++q) {
        idx[q] = 0;
        while (*p >= '0' && *p <= '9') idx[q] = idx[q] * 10 + (*p++ - '0');
        if (*p == ',') ++p;
      }
      const float v = (m[idx[0]] * m[idx[1]]) * m[idx[2]];
      acc = k == 0 ? (neg ? -v : v) : (neg ? acc - v : acc + v);
    }
    inv[e] = acc;
  }
  float det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  for (int i = 0; i < 16; ++i) c[i] = 0.0f;  // Matrix4Inverse's c when det == 0
  if (det == 0.0f) return;
  det = 1.0f / det;
  for (int i = 0; i < 16; ++i) c[i] = inv[i] * det;
}

// The ray mapped by Matrix4MulPoint/Matrix4MulVec of an inverse
// (math/matrix4.go:177-218), then Ray.Setup.
void ray_to_space(Ray& ro, const Ray& r, const float* a) {
  for (int i = 0; i < 3; ++i) {
    ro.P[i] = a[i] * r.P[0] + a[4 + i] * r.P[1] + a[8 + i] * r.P[2] + a[12 + i];
    ro.D[i] = a[i] * r.D[0] + a[4 + i] * r.D[1] + a[8 + i] * r.D[2];
  }
  ray_setup(ro);
}

// PolyMesh.Trace's transform (builtin/geom/polymesh/trace.go:22-55, 64-69):
// one key used as it is, two or more blended (TransformDecompLerp of the
// keys around the ray's time, rebuilt), Matrix4Inverse, the ray mapped into
// object space, the walk, then the world ray again with the walk's Tclosest.
bool mesh_trace_xf(const Mesh& m, Ray& r, Task& tk) {
  if (!m.has_xf && m.xkeys.empty()) return mesh_trace(m, r, tk);
  float inv[16];
  if (!m.xkeys.empty()) {
    float M[16];
    if (!orc_internal::decomp_at(m.xkeys, r.Time, false, M)) return false;  // the reference panics
    orc_internal::matrix_inverse(M, inv);
  } else {
    for (int i = 0; i < 16; ++i) inv[i] = m.xinv[i];
  }
  Ray ro = r;
  ray_to_space(ro, r, inv);
  const bool hit = mesh_trace(m, ro, tk);
  r.Tclosest = ro.Tclosest;
  return hit;
}

// Instance.Trace (builtin/geom/instance/instance.go:72-115) and Proc.Trace
// (builtin/geom/proc/proc.go:88-140): the transform at the ray's time
// (TransformSRTArray.TimeKey, rebuilt), Matrix4Inverse, the ray mapped and
// Ray.Setup, then the children in order, each through its own
// PolyMesh.Trace; a Proc stops at the first child that hits unless the ray
// is a shadow ray (proc.go:117-124).  hit_id: the id the hit reports.
bool group_trace(const Mesh& m, Ray& r, Task& tk, int32_t& hit_id) {
  float M[16], inv[16];
  if (!orc_internal::decomp_at(m.gkeys, r.Time, false, M)) return false;
  orc_internal::matrix_inverse(M, inv);
  Ray rg = r;
  ray_to_space(rg, r, inv);
  bool hit = false;
  for (size_t c = 0; c < m.children.size(); ++c) {
    if (mesh_trace_xf(*m.children[c], rg, tk)) {
      hit = true;
      hit_id = m.group == 2 ? m.child_ids[c] : -1;
      if (!r.shadow) break;
    }
    if (tk.overflow) break;
  }
  r.Tclosest = rg.Tclosest;
  return hit;
}

// Scene.TraceElems / TraceMotionElems (scene.go:61-97).
bool scene_trace_elems(const Scene& s, Ray& r, Task& tk, int base, int count) {
  bool hit = false;
  for (int i = base; i < base + count; ++i) {
    const Mesh& g = *s.geoms[i];
    int32_t hid = -1;
    const bool gh = g.group ? group_trace(g, r, tk, hid) : mesh_trace_xf(g, r, tk);
    if (gh) {
      tk.geom = hid >= 0 ? hid : s.geom_order[i];
      hit = true;
      if (r.shadow) return true;
    }
    if (tk.overflow) return hit;
  }
  return hit;
}

// Scene.Trace (scene.go:30-58).
bool scene_trace(const Scene& s, Ray& r, Task& tk) {
  if (!s.nodes.empty()) {
    return qbvh_trace(s.nodes.data(), r, tk, [&](Ray& rr, Task& t, int b, int c) {
      return scene_trace_elems(s, rr, t, b, c);
    });
  }
  if (s.mnodes.empty()) return false;
  float k = r.Time * (float)(s.mboxes.size() - 1);
  float time = k - std::floor(k);
  int key = (int)std::floor(k), key2 = (int)std::ceil(k);
  if (key < 0 || key2 >= (int)s.mboxes.size()) return false;
  return qbvh_trace_motion(s.mnodes.data(), s.mboxes, time, key, key2, r, tk,
                           [&](Ray& rr, Task& t, int b, int c) {
                             return scene_trace_elems(s, rr, t, b, c);
                           });
}

template <class F>
void parallel_for(size_t n, int nthreads, F&& f) {
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  if ((size_t)nthreads > n) nthreads = (int)std::max<size_t>(n, 1);
  if (nthreads == 1) { for (size_t i = 0; i < n; ++i) f(i); return; }
  std::atomic<size_t> next(0);
  const size_t chunk = 1024;
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([&]() {
      for (;;) {
        size_t s = next.fetch_add(chunk);
        if (s >= n) break;
        size_t e = std::min(n, s + chunk);
        for (size_t i = s; i < e; ++i) f(i);
      }
    });
  for (auto& x : th) x.join();
}

}  // namespace

struct orc_mesh { Mesh m; };
struct orc_scene { Scene s; };

#include "orc_internal.h"

namespace orc_internal {

Hit trace(const orc_scene* s, const float P[3], const float D[3], float tmax, float time, bool shadow) {
  float in[8] = {P[0], P[1], P[2], D[0], D[1], D[2], tmax, time};
  Ray r = make_ray(in, shadow);
  Task tk;
  Hit h;
  h.hit = scene_trace(s->s, r, tk);
  h.elem = tk.elem;
  h.geom = tk.geom;
  h.t = r.Tclosest;
  h.u = tk.bu;
  h.v = tk.bv;
  h.w = tk.bw;
  h.overflow = tk.overflow;
  return h;
}

MeshView mesh_view(const orc_mesh* om) {
  // An instance shades as the geom it traces, through its own transform.
  const Mesh& m = om->m.group == 1 ? *om->m.children[0] : om->m;
  MeshView v;
  v.verts = m.verts.data();
  v.nverts = m.nverts;
  v.keys = m.keys;
  v.idxp = m.idxp.data();
  v.shaderidx = m.shaderidx.empty() ? nullptr : m.shaderidx.data();
  v.normals = m.normals.empty() ? nullptr : m.normals.data();
  v.mnormals = m.mnormals.empty() ? nullptr : m.mnormals.data();
  v.mnormals_per_key = m.mnormals_per_key;
  v.motion = m.keys > 1;
  v.sphere = m.sphere;
  for (int k = 0; k < 3; ++k) v.sc[k] = m.sc[k];
  v.sr = m.sr;
  v.has_xf = m.has_xf;
  for (int k = 0; k < 16; ++k) {
    v.xf[k] = m.xf[k];
    v.xinv[k] = m.xinv[k];
  }
  v.xkeys = m.xkeys.empty() ? nullptr : &m.xkeys;
  v.outer = om->m.group == 1 ? &om->m.gkeys : m.outer;
  return v;
}

}  // namespace orc_internal

extern "C" {

const char* orc_last_error(void) { return g_err.c_str(); }

orc_mesh* orc_mesh_create(const float* verts, uint32_t nverts, uint32_t keys, const uint32_t* idxp,
                          uint32_t ntris, float ray_bias, int motion_fixed) {
  if (keys < 1 || (ntris > 0 && (!verts || !idxp))) { g_err = "invalid mesh arguments"; return nullptr; }
  for (size_t i = 0; i < (size_t)ntris * 3; ++i)
    if (idxp[i] >= nverts) { g_err = "vertex index out of range"; return nullptr; }
  if (ntris >= (1u << 23)) { g_err = "more than 2^23-1 triangles: leaf base field overflows"; return nullptr; }
  orc_mesh* om = new orc_mesh();
  Mesh& m = om->m;
  m.nverts = nverts; m.keys = keys; m.ntris = ntris;
  m.verts.assign(verts, verts + (size_t)keys * nverts * 3);
  m.idxp.assign(idxp, idxp + (size_t)ntris * 3);
  m.ray_bias = ray_bias;
  m.motion_fixed = motion_fixed != 0;
  try {
    mesh_init_accel(m);
  } catch (const BuildErr&) {
    delete om;
    return nullptr;
  }
  return om;
}

void orc_mesh_destroy(orc_mesh* m) { delete m; }

void orc_mesh_set_transform_keys(orc_mesh* om, const float* keys16, uint32_t n) {
  Mesh& me = om->m;
  me.xkeys.clear();
  if (n <= 1) {
    orc_mesh_set_transform(om, n == 1 ? keys16 : nullptr);
    return;
  }
  me.has_xf = false;
  me.xkeys.resize(n);
  for (uint32_t i = 0; i < n; ++i) orc_internal::decomp_matrix(keys16 + 16 * i, me.xkeys[i]);
}

static orc_mesh* make_group(int kind, const float* keys16, uint32_t n_keys, const float bmin[3], const float bmax[3]) {
  orc_mesh* om = new orc_mesh();
  Mesh& g = om->m;
  g.group = kind;
  g.gkeys.resize(n_keys);
  for (uint32_t i = 0; i < n_keys; ++i) orc_internal::decomp_matrix(keys16 + 16 * i, g.gkeys[i]);
  box_reset(g.user_bounds);  // BoundingBox.GrowVec3 of BMin and BMax (instance.go:123-128)
  box_grow(g.user_bounds, bmin);
  box_grow(g.user_bounds, bmax);
  return om;
}

orc_mesh* orc_instance_create(const orc_mesh* of, const float* keys16, uint32_t n_keys, const float bmin[3],
                              const float bmax[3]) {
  if (!of || of->m.group || n_keys < 1 || !keys16) { g_err = "bad instance arguments"; return nullptr; }
  orc_mesh* om = make_group(1, keys16, n_keys, bmin, bmax);
  om->m.children.push_back(&of->m);
  return om;
}

orc_mesh* orc_proc_create(orc_mesh* const* children, const int32_t* child_ids, uint32_t n, const float* keys16,
                          uint32_t n_keys, const float bmin[3], const float bmax[3]) {
  if (n == 0 || !children || !child_ids) { g_err = "a Proc needs geoms"; return nullptr; }
  for (uint32_t i = 0; i < n; ++i)
    if (!children[i] || children[i]->m.group) { g_err = "a Proc's children are meshes or spheres"; return nullptr; }
  static const float kIdentity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  // Proc.PreRender: no Transform means one identity key (proc.go:157-160)
  orc_mesh* om = n_keys ? make_group(2, keys16, n_keys, bmin, bmax) : make_group(2, kIdentity, 1, bmin, bmax);
  for (uint32_t i = 0; i < n; ++i) {
    om->m.children.push_back(&children[i]->m);
    om->m.child_ids.push_back(child_ids[i]);
    children[i]->m.outer = &om->m.gkeys;
  }
  return om;
}

void orc_mesh_set_transform(orc_mesh* om, const float* m) {
  Mesh& me = om->m;
  me.has_xf = m != nullptr;
  for (int k = 0; k < 16; ++k) me.xf[k] = m ? m[k] : 0.0f;
  if (m) matrix4_inverse(me.xf, me.xinv);
}

// Shading data as PolyMesh holds it after initAccel (buildqbvh.go:98-104):
// shader indices permuted to leaf order for a static mesh, face order for a
// motion mesh; normals indexed by vertex (NormalIdx = FaceIdx).
orc_mesh* orc_sphere_create(const float center[3], float radius) {
  orc_mesh* om = new orc_mesh();
  Mesh& m = om->m;
  m.sphere = true;
  for (int k = 0; k < 3; ++k) {
    m.sc[k] = center[k];
    m.bounds.b[0][k] = center[k] - radius;  // Sphere.Bounds (sphere.go:62-72)
    m.bounds.b[1][k] = center[k] + radius;
  }
  m.sr = radius;
  return om;
}

int orc_mesh_set_shading(orc_mesh* om, const uint8_t* face_shader, const float* normals) {
  Mesh& m = om->m;
  m.shaderidx.clear();
  if (face_shader) {
    m.shaderidx.resize(m.ntris);
    for (uint32_t i = 0; i < m.ntris; ++i)
      m.shaderidx[i] = m.nodes.empty() ? face_shader[i] : face_shader[m.accel_idx[i]];
  }
  m.normals.clear();
  if (normals) m.normals.assign(normals, normals + (size_t)m.nverts * 3);
  return 0;
}

// PolyMesh.Normals of a motion mesh with as many keys as its vertices: the
// motion hit reads Normals.Elems[idx*3 + j + ElemsPerKey*key] directly, idx
// being the element the hit reports (trace.go:694-712), not through
// NormalIdx.
int orc_mesh_set_motion_normals(orc_mesh* om, const float* normals, uint32_t n_per_key, uint32_t keys) {
  Mesh& m = om->m;
  m.mnormals.clear();
  m.mnormals_per_key = 0;
  if (!normals) return 0;
  if (m.keys < 2 || keys != m.keys || (uint64_t)n_per_key < 3ull * m.ntris) return -1;
  m.mnormals.assign(normals, normals + (size_t)keys * n_per_key * 3);
  m.mnormals_per_key = n_per_key;
  return 0;
}

void orc_mesh_info(const orc_mesh* om, uint32_t* n_nodes, uint32_t* n_mnodes, float* bounds6) {
  const Mesh& m = om->m;
  if (n_nodes) *n_nodes = (uint32_t)m.nodes.size();
  if (n_mnodes) *n_mnodes = (uint32_t)m.mnodes.size();
  if (bounds6) {
    for (int k = 0; k < 3; ++k) { bounds6[k] = m.bounds.b[0][k]; bounds6[3 + k] = m.bounds.b[1][k]; }
  }
}

void orc_mesh_export(const orc_mesh* om, orc_node* nodes, int32_t* accel_idx, uint32_t* idxp_out,
                     orc_mnode* mnodes, float* mboxes) {
  const Mesh& m = om->m;
  if (nodes && !m.nodes.empty()) std::memcpy(nodes, m.nodes.data(), m.nodes.size() * sizeof(orc_node));
  if (accel_idx && !m.accel_idx.empty()) std::memcpy(accel_idx, m.accel_idx.data(), m.accel_idx.size() * 4);
  if (idxp_out && !m.idxp.empty()) std::memcpy(idxp_out, m.idxp.data(), m.idxp.size() * 4);
  if (mnodes && !m.mnodes.empty()) std::memcpy(mnodes, m.mnodes.data(), m.mnodes.size() * sizeof(orc_mnode));
  if (mboxes)
    for (size_t k = 0; k < m.mboxes.size(); ++k)
      std::memcpy(mboxes + k * m.mnodes.size() * 24, m.mboxes[k].data(), m.mboxes[k].size() * 4);
}

static void write_out(size_t i, const Task& tk, const Ray& r, bool hit, int32_t* prim, int32_t* geom,
                      float* t, float* u, float* v, float* w, uint32_t* counters) {
  if (prim) prim[i] = hit ? tk.elem : -1;
  if (geom) geom[i] = hit ? tk.geom : -1;
  if (t) t[i] = r.Tclosest;
  if (u) u[i] = hit ? tk.bu : 0.0f;
  if (v) v[i] = hit ? tk.bv : 0.0f;
  if (w) w[i] = hit ? tk.bw : 0.0f;
  if (counters) {
    counters[i * 3 + 0] = tk.nodes_t;
    counters[i * 3 + 1] = tk.leafs_t;
    counters[i * 3 + 2] = tk.tris_t;
  }
}

int orc_trace_mesh(const orc_mesh* om, const float* rays, size_t n, int shadow, int nthreads,
                   int32_t* prim, float* t, float* u, float* v, float* w, uint32_t* counters) {
  std::atomic<int> status(0);
  parallel_for(n, nthreads, [&](size_t i) {
    Ray r = make_ray(rays + i * ORC_RAY_STRIDE, shadow != 0);
    Task tk;
    bool hit = mesh_trace(om->m, r, tk);
    if (tk.overflow) status = -5;
    write_out(i, tk, r, hit, prim, nullptr, t, u, v, w, counters);
  });
  return status.load();
}

orc_scene* orc_scene_create(orc_mesh* const* meshes, uint32_t n) { return orc_scene_create_ids(meshes, nullptr, n); }

orc_scene* orc_scene_create_ids(orc_mesh* const* meshes, const int32_t* ids, uint32_t n) {
  std::vector<Mesh*> ms(n);
  for (uint32_t i = 0; i < n; ++i) {
    if (!meshes[i]) { g_err = "null mesh"; return nullptr; }
    ms[i] = &meshes[i]->m;
  }
  orc_scene* os = new orc_scene();
  try {
    scene_init(os->s, ms.data(), n);
  } catch (const BuildErr&) {
    delete os;
    return nullptr;
  }
  if (ids)
    for (auto& g : os->s.geom_order) g = ids[g];
  return os;
}

void orc_scene_destroy(orc_scene* s) { delete s; }

void orc_scene_info(const orc_scene* os, uint32_t* n_nodes, uint32_t* n_mnodes, uint32_t* keys) {
  if (n_nodes) *n_nodes = (uint32_t)os->s.nodes.size();
  if (n_mnodes) *n_mnodes = (uint32_t)os->s.mnodes.size();
  if (keys) *keys = (uint32_t)os->s.keys;
}

void orc_scene_export(const orc_scene* os, orc_node* nodes, int32_t* geom_order, orc_mnode* mnodes,
                      float* mboxes) {
  const Scene& s = os->s;
  if (nodes && !s.nodes.empty()) std::memcpy(nodes, s.nodes.data(), s.nodes.size() * sizeof(orc_node));
  if (geom_order && !s.geom_order.empty()) std::memcpy(geom_order, s.geom_order.data(), s.geom_order.size() * 4);
  if (mnodes && !s.mnodes.empty()) std::memcpy(mnodes, s.mnodes.data(), s.mnodes.size() * sizeof(orc_mnode));
  if (mboxes)
    for (size_t k = 0; k < s.mboxes.size(); ++k)
      std::memcpy(mboxes + k * s.mnodes.size() * 24, s.mboxes[k].data(), s.mboxes[k].size() * 4);
}

int orc_trace_scene(const orc_scene* os, const float* rays, size_t n, int shadow, int nthreads,
                    int32_t* prim, int32_t* geom, float* t, float* u, float* v, float* w,
                    uint32_t* counters) {
  std::atomic<int> status(0);
  parallel_for(n, nthreads, [&](size_t i) {
    Ray r = make_ray(rays + i * ORC_RAY_STRIDE, shadow != 0);
    Task tk;
    bool hit = scene_trace(os->s, r, tk);
    if (tk.overflow) status = -5;
    write_out(i, tk, r, hit, prim, geom, t, u, v, w, counters);
  });
  return status.load();
}

}  // extern "C"
