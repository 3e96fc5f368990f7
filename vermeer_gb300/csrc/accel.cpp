// accel.cpp - host QBVH construction, bit-identical to the reference builder.
//
// Compiled with -ffp-contract=off: every float expression below is evaluated
// as separately rounded operations in source order, as Go does on amd64.
#include "accel.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <future>
#include <numeric>
#include <thread>

namespace vmr {
namespace {

constexpr float kInf = __builtin_huge_valf();

// math.Min/Max (math/dim_amd64.s:8-21): first operand wins unless the
// second compares strictly smaller/larger.
inline float go_min(float x, float y) { return x < y ? x : y; }
inline float go_max(float x, float y) { return x > y ? x : y; }

inline Bounds empty_bounds() {
  return Bounds{{kInf, kInf, kInf}, {-kInf, -kInf, -kInf}};
}
// BoundingBox.Grow (math/boundingbox.go:107-116): Min(point, box).
inline void add_point(Bounds& b, const float* p) {
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = go_min(p[k], b.lo[k]);
    b.hi[k] = go_max(p[k], b.hi[k]);
  }
}
// BoundingBox.GrowBox (boundingbox.go:99-104): Min(box, other).
inline void add_bounds(Bounds& b, const Bounds& o) {
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = go_min(b.lo[k], o.lo[k]);
    b.hi[k] = go_max(b.hi[k], o.hi[k]);
  }
}
inline float extent(const Bounds& b, int a) { return b.hi[a] - b.lo[a]; }
// SurfaceArea (boundingbox.go:17-19).
inline float half_sum_area(const Bounds& b) {
  float e0 = extent(b, 0), e1 = extent(b, 1), e2 = extent(b, 2);
  return e0 * e1 * 2.0f + e1 * e2 * 2.0f + e0 * e2 * 2.0f;
}
// LongestAxis (boundingbox.go:54-70).
inline int widest_axis(const Bounds& b) {
  float e0 = extent(b, 0), e1 = extent(b, 1), e2 = extent(b, 2);
  if (e0 < e1) return e1 < e2 ? 2 : 1;
  return e0 < e2 ? 2 : 0;
}
// BoundingBoxLerp (boundingbox.go:119-127).
inline Bounds lerp_bounds(const Bounds& a, const Bounds& b, float t) {
  Bounds o;
  for (int k = 0; k < 3; ++k) {
    o.lo[k] = (1 - t) * a.lo[k] + t * b.lo[k];
    o.hi[k] = (1 - t) * a.hi[k] + t * b.hi[k];
  }
  return o;
}

inline void store_child_box(float* boxes, int c, const Bounds& b) {  // Node.SetBounds
  for (int k = 0; k < 3; ++k) {
    boxes[c + 4 * k] = b.lo[k];
    boxes[c + 12 + 4 * k] = b.hi[k];
  }
}
inline Bounds load_child_box(const float* boxes, int c) {
  Bounds b;
  for (int k = 0; k < 3; ++k) { b.lo[k] = boxes[c + 4 * k]; b.hi[k] = boxes[c + 12 + 4 * k]; }
  return b;
}
// Node.SetLeaf (qbvh/qbvh.go:82-93).
inline int32_t encode_leaf(uint32_t first, uint32_t count) {
  return (int32_t)((1u << 31) | ((first << 4) & 0xfffffff0u) | ((count - 1) & 0xfu));
}
inline uint32_t leaf_first(int32_t c) { return (uint32_t)((c & 0x7ffffff) >> 4); }
inline uint32_t leaf_size(int32_t c) { return (uint32_t)((c & 0xf) + 1); }

// Working set of one build: primitive boxes, centroids and ids, permuted in
// lock-step by the partition.
struct Prims {
  std::vector<Bounds> box;
  std::vector<float> cen;  // 3 per primitive
  std::vector<int32_t> id;
};

struct Split {
  int axis;
  int pivot;
};

// binarySplit + calcMinCost (qbvh/build.go:28-178) over [first, first+n).
Split split_range(Prims& p, int first, int n, int leaf_max) {
  Bounds cb = empty_bounds();
  const float* cen = p.cen.data();
  for (int i = first; i < first + n; ++i) add_point(cb, cen + 3 * (size_t)i);
  if (n <= leaf_max) return {0, n};
  int axis = widest_axis(cb);
  if (cb.hi[axis] == cb.lo[axis]) return {axis, n / 2 + 1};  // build.go:34-43
  const float scale = (8.0f * 0.99994f) / (cb.hi[axis] - cb.lo[axis]);
  const float origin = cb.lo[axis];
  Bounds bin_box[8];
  int32_t bin_cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (auto& b : bin_box) b = empty_bounds();
  for (int i = first; i < first + n; ++i) {
    int bin = (int)(scale * (cen[3 * (size_t)i + axis] - origin));
    if (bin < 0 || bin > 7) throw std::runtime_error("QBVH build: centroid bin out of range");
    bin_cnt[bin]++;
    add_bounds(bin_box[bin], p.box[i]);
  }
  // Prefix unions from the left and from the right.
  Bounds left[8], right[8];
  int32_t nleft[8], nright[8];
  Bounds acc = empty_bounds();
  int32_t cnt = 0;
  for (int i = 0; i < 8; ++i) {
    add_bounds(acc, bin_box[i]);
    cnt += bin_cnt[i];
    left[i] = acc;
    nleft[i] = cnt;
  }
  acc = empty_bounds();
  cnt = 0;
  for (int i = 7; i >= 0; --i) {
    add_bounds(acc, bin_box[i]);
    cnt += bin_cnt[i];
    right[i] = acc;
    nright[i] = cnt;
  }
  int plane = -1;
  float best = kInf;
  for (int i = 1; i < 8; ++i) {
    float cost = half_sum_area(left[i - 1]) * (float)nleft[i - 1] + half_sum_area(right[i]) * (float)nright[i];
    if (cost < best) { best = cost; plane = i; }
  }
  // Two-ended in-place partition, swapping from the back (build.go:114-130).
  int lo = first, hi = first + n - 1;
  while (lo <= hi) {
    int bin = (int)(scale * (p.cen[3 * (size_t)lo + axis] - origin));
    if (bin < plane) {
      ++lo;
    } else {
      std::swap(p.id[lo], p.id[hi]);
      for (int k = 0; k < 3; ++k) std::swap(p.cen[3 * (size_t)lo + k], p.cen[3 * (size_t)hi + k]);
      std::swap(p.box[lo], p.box[hi]);
      --hi;
    }
  }
  return {axis, lo - first};
}

Bounds union_range(const Prims& p, int first, int n) {
  Bounds b = empty_bounds();
  for (int i = first; i < first + n; ++i) add_bounds(b, p.box[i]);
  return b;
}

// A subtree with local pre-order numbering (root = 0).  The upper levels of
// a build produce their four child subtrees concurrently and splice them in
// child order, which reproduces the reference's single-threaded numbering.
template <class Node>
struct Subtree {
  std::vector<Node> nodes;
  Bounds box;
};

template <class Node>
struct TreeBuild {
  Prims& p;
  int leaf_max;
  bool motion;
  size_t parallel_min;  // ranges at least this large build children concurrently

  void set_axes(Node& nd, int a0, int a1, int a2);

  // Serial recursion appending to `out`; returns the node index.
  int32_t serial(std::vector<Node>& out, int first, int n, Bounds* box, int depth) {
    if (depth > 4096) throw std::runtime_error("QBVH build recursion does not terminate");
    Split s0 = split_range(p, first, n, leaf_max);
    Split s1 = split_range(p, first, s0.pivot, leaf_max);
    Split s2 = split_range(p, first + s0.pivot, n - s0.pivot, leaf_max);
    int32_t me = (int32_t)out.size();
    out.emplace_back();
    std::memset(&out[me], 0, sizeof(Node));
    set_axes(out[me], s0.axis, s1.axis, s2.axis);
    const int beg[4] = {0, s1.pivot, s0.pivot, s0.pivot + s2.pivot};
    const int end[4] = {s1.pivot, s0.pivot, s0.pivot + s2.pivot, n};
    Bounds cbox[4];
    for (int c = 0; c < 4; ++c) {
      int len = end[c] - beg[c];
      if (len <= leaf_max) {
        set_leaf(out[me], c, first + beg[c], len);
      } else {
        int32_t ch = serial(out, first + beg[c], len, &cbox[c], depth + 1);
        set_inner(out[me], c, ch, cbox[c]);
      }
    }
    if (box) *box = node_union(out[me]);
    return me;
  }

  Subtree<Node> parallel(int first, int n, int depth) {
    Subtree<Node> st;
    if ((size_t)n < parallel_min) {
      serial(st.nodes, first, n, &st.box, depth);
      return st;
    }
    Split s0 = split_range(p, first, n, leaf_max);
    Split s1 = split_range(p, first, s0.pivot, leaf_max);
    Split s2 = split_range(p, first + s0.pivot, n - s0.pivot, leaf_max);
    st.nodes.emplace_back();
    std::memset(&st.nodes[0], 0, sizeof(Node));
    set_axes(st.nodes[0], s0.axis, s1.axis, s2.axis);
    const int beg[4] = {0, s1.pivot, s0.pivot, s0.pivot + s2.pivot};
    const int end[4] = {s1.pivot, s0.pivot, s0.pivot + s2.pivot, n};
    std::future<Subtree<Node>> kids[4];
    for (int c = 0; c < 4; ++c) {
      int len = end[c] - beg[c];
      if (len > leaf_max)
        kids[c] = std::async(std::launch::async, [this, first, b = beg[c], len, depth] {
          return parallel(first + b, len, depth + 1);
        });
    }
    for (int c = 0; c < 4; ++c) {
      int len = end[c] - beg[c];
      if (len <= leaf_max) {
        set_leaf(st.nodes[0], c, first + beg[c], len);
        continue;
      }
      Subtree<Node> kid = kids[c].get();
      int32_t off = (int32_t)st.nodes.size();
      for (auto& nd : kid.nodes) {
        for (int k = 0; k < 4; ++k)
          if (nd.children[k] >= 0) nd.children[k] += off;
        st.nodes.push_back(nd);
      }
      set_inner(st.nodes[0], c, off, kid.box);
    }
    st.box = node_union(st.nodes[0]);
    return st;
  }

  void set_leaf(Node& nd, int c, int first, int len);
  void set_inner(Node& nd, int c, int32_t child, const Bounds& b);
  Bounds node_union(const Node& nd);
};

template <>
void TreeBuild<vmr_qbvh_node>::set_axes(vmr_qbvh_node& nd, int a0, int a1, int a2) {
  nd.axis0 = (uint32_t)a0; nd.axis1 = (uint32_t)a1; nd.axis2 = (uint32_t)a2;
}
template <>
void TreeBuild<vmr_mqbvh_node>::set_axes(vmr_mqbvh_node& nd, int a0, int a1, int a2) {
  nd.axis0 = a0; nd.axis1 = a1; nd.axis2 = a2;
}
template <>
void TreeBuild<vmr_qbvh_node>::set_leaf(vmr_qbvh_node& nd, int c, int first, int len) {
  if (len == 0) {  // SetEmptyLeaf (qbvh.go:67-79): -1 with the +inf box
    nd.children[c] = -1;
    Bounds inf{{kInf, kInf, kInf}, {kInf, kInf, kInf}};
    store_child_box(nd.boxes, c, inf);
  } else {
    store_child_box(nd.boxes, c, union_range(p, first, len));
    nd.children[c] = encode_leaf((uint32_t)first, (uint32_t)len);
  }
}
template <>
void TreeBuild<vmr_mqbvh_node>::set_leaf(vmr_mqbvh_node& nd, int c, int first, int len) {
  nd.children[c] = len == 0 ? -1 : encode_leaf((uint32_t)first, (uint32_t)len);
}
template <>
void TreeBuild<vmr_qbvh_node>::set_inner(vmr_qbvh_node& nd, int c, int32_t child, const Bounds& b) {
  store_child_box(nd.boxes, c, b);
  nd.children[c] = child;
}
template <>
void TreeBuild<vmr_mqbvh_node>::set_inner(vmr_mqbvh_node& nd, int c, int32_t child, const Bounds&) {
  nd.children[c] = child;
}
template <>
Bounds TreeBuild<vmr_qbvh_node>::node_union(const vmr_qbvh_node& nd) {  // build.go:276-283
  Bounds b = empty_bounds();
  for (int c = 0; c < 4; ++c)
    if (nd.children[c] != -1) add_bounds(b, load_child_box(nd.boxes, c));
  return b;
}
template <>
Bounds TreeBuild<vmr_mqbvh_node>::node_union(const vmr_mqbvh_node&) {
  return empty_bounds();
}

template <class Node>
std::vector<Node> build_tree(Prims& p, int leaf_max, Bounds* box) {
  std::vector<Node> out;
  if (p.id.empty()) {
    if (box) *box = empty_bounds();
    return out;
  }
  TreeBuild<Node> tb{p, leaf_max, false, (size_t)1 << 17};
  Subtree<Node> st = tb.parallel(0, (int)p.id.size(), 0);
  if (box) *box = st.box;
  return std::move(st.nodes);
}

template <class F>
void parallel_rows(size_t n, F&& f) {
  unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (n < 65536 || nt == 1) { f(0, n); return; }
  std::vector<std::thread> th;
  size_t chunk = (n + nt - 1) / nt;
  for (unsigned t = 0; t < nt; ++t) {
    size_t s = t * chunk, e = std::min(n, s + chunk);
    if (s < e) th.emplace_back([&f, s, e] { f(s, e); });
  }
  for (auto& x : th) x.join();
}

// Per-key leaf boxes of a motion tree (buildqbvh.go:159-212 and
// scene.go:228-268): leaf_box(key, first, count) gives a leaf's box.
template <class LeafBox>
Bounds fill_motion_boxes(const std::vector<vmr_mqbvh_node>& nodes, float* boxes, int32_t node,
                         LeafBox&& leaf_box) {
  Bounds acc = empty_bounds();
  for (int c = 0; c < 4; ++c) {
    int32_t ch = nodes[node].children[c];
    if (ch == -1) continue;  // empty children keep a zero box
    Bounds b = ch < 0 ? leaf_box(leaf_first(ch), leaf_size(ch))
                      : fill_motion_boxes(nodes, boxes, ch, leaf_box);
    store_child_box(boxes + (size_t)node * 24, c, b);
    add_bounds(acc, b);
  }
  return acc;
}

}  // namespace

Bounds HostMesh::bounds_at(float time) const {
  if (!motion()) return bounds;
  float k = time * (float)(key_bounds.size() - 1);
  float t = k - std::floor(k);
  int key = (int)std::floor(k), key2 = (int)std::ceil(k);
  return lerp_bounds(key_bounds[key], key_bounds[key2], t);
}

bool build_mesh_accel(HostMesh& m, std::string& err) {
  try {
    const uint32_t n = m.n_tris;
    Prims p;
    p.box.resize(n);
    p.cen.resize((size_t)n * 3);
    p.id.resize(n);
    // Build-time geometry: the mesh at key 0, or lerped to time 0.5 for a
    // motion mesh (buildqbvh.go:19-50, 62-83).
    float kf = 0.5f * (float)(m.keys - 1);
    float tt = kf - std::floor(kf);
    uint32_t ka = (uint32_t)std::floor(kf), kb = (uint32_t)std::ceil(kf);
    parallel_rows(n, [&](size_t s, size_t e) {
      for (size_t i = s; i < e; ++i) {
        float v[3][3];
        for (int j = 0; j < 3; ++j) {
          const float* a = &m.verts[((size_t)ka * m.n_verts + m.idxp[i * 3 + j]) * 3];
          if (m.keys > 1) {
            const float* b = &m.verts[((size_t)kb * m.n_verts + m.idxp[i * 3 + j]) * 3];
            for (int k = 0; k < 3; ++k) v[j][k] = (1.0f - tt) * a[k] + tt * b[k];  // Vec3Lerp
          } else {
            for (int k = 0; k < 3; ++k) v[j][k] = a[k];
          }
        }
        Bounds b = empty_bounds();
        for (int j = 0; j < 3; ++j) add_point(b, v[j]);
        p.box[i] = b;
        for (int k = 0; k < 3; ++k) p.cen[i * 3 + k] = (v[0][k] + v[1][k] + v[2][k]) / 3.0f;
        p.id[i] = (int32_t)i;
      }
    });
    if (m.keys > 1) {
      m.mnodes = build_tree<vmr_mqbvh_node>(p, 16, nullptr);
      m.accel_idx = p.id;
      m.mboxes.assign((size_t)m.keys * m.mnodes.size() * 24, 0.0f);
      m.key_bounds.clear();
      Bounds full = empty_bounds();
      for (uint32_t key = 0; key < m.keys; ++key) {
        Bounds kb2 = empty_bounds();
        if (!m.mnodes.empty())
          kb2 = fill_motion_boxes(m.mnodes, m.mboxes.data() + (size_t)key * m.mnodes.size() * 24, 0,
                                  [&](uint32_t first, uint32_t cnt) {
                                    Bounds b = empty_bounds();
                                    for (uint32_t i = first; i < first + cnt; ++i) {
                                      int32_t f = m.accel_idx[i];
                                      for (int j = 0; j < 3; ++j)
                                        add_point(b, &m.verts[((size_t)key * m.n_verts + m.idxp[(size_t)f * 3 + j]) * 3]);
                                    }
                                    return b;
                                  });
        m.key_bounds.push_back(kb2);
        add_bounds(full, kb2);
      }
      m.bounds = full;
      return true;
    }
    m.nodes = build_tree<vmr_qbvh_node>(p, 16, &m.bounds);
    m.accel_idx = p.id;
    std::vector<uint32_t> leaf_idxp((size_t)n * 3);
    for (uint32_t i = 0; i < n; ++i)
      for (int j = 0; j < 3; ++j) leaf_idxp[(size_t)i * 3 + j] = m.idxp[(size_t)p.id[i] * 3 + j];
    m.idxp.swap(leaf_idxp);
    if (!m.shader_idx.empty()) {
      std::vector<uint8_t> s(n);
      for (uint32_t i = 0; i < n; ++i) s[i] = m.shader_idx[p.id[i]];
      m.shader_idx.swap(s);
    }
    return true;
  } catch (const std::exception& e) {
    err = e.what();
    return false;
  }
}

bool build_top_level(const std::vector<const HostMesh*>& meshes, const std::vector<uint32_t>& ids,
                     HostTop& top, std::string& err) {
  try {
    const size_t n = meshes.size();
    int max_keys = 0;
    for (auto* m : meshes) max_keys = std::max(max_keys, m->motion_keys());
    Prims p;
    p.box.resize(n);
    p.cen.resize(n * 3);
    p.id.resize(n);
    const float t0 = max_keys == 1 ? 0.0f : 0.5f;  // Bounds(0) or Bounds(0.5)
    for (size_t i = 0; i < n; ++i) {
      p.box[i] = meshes[i]->bounds_at(t0);
      for (int k = 0; k < 3; ++k) p.cen[i * 3 + k] = (p.box[i].hi[k] + p.box[i].lo[k]) * 0.5f;  // Centroid
      p.id[i] = (int32_t)i;
    }
    top = HostTop();
    if (max_keys <= 1) {
      top.nodes = build_tree<vmr_qbvh_node>(p, 1, nullptr);
      top.keys = 1;
    } else {
      top.mnodes = build_tree<vmr_mqbvh_node>(p, 1, nullptr);
      top.keys = (uint32_t)max_keys;
    }
    top.geom_order.resize(n);
    for (size_t i = 0; i < n; ++i) top.geom_order[i] = ids[p.id[i]];
    if (max_keys > 1 && !top.mnodes.empty()) {
      top.mboxes.assign((size_t)top.keys * top.mnodes.size() * 24, 0.0f);
      for (uint32_t key = 0; key < top.keys; ++key) {
        float time = (float)key / (float)(top.keys - 1);
        fill_motion_boxes(top.mnodes, top.mboxes.data() + (size_t)key * top.mnodes.size() * 24, 0,
                          [&](uint32_t first, uint32_t cnt) {
                            Bounds b = empty_bounds();
                            for (uint32_t i = first; i < first + cnt; ++i)
                              add_bounds(b, meshes[p.id[i]]->bounds_at(time));
                            return b;
                          });
      }
    }
    return true;
  } catch (const std::exception& e) {
    err = e.what();
    return false;
  }
}

}  // namespace vmr
