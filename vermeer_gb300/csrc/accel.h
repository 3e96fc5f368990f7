// accel.h - host-side accelerator construction for libvmr.
//
// The reference builds every QBVH on the CPU at PreRender (qbvh/build.go,
// builtin/geom/polymesh/buildqbvh.go, builtin/scene/scene.go).  A Go host
// passes those reference-built nodes to vmr_mesh_upload; every other caller
// uses this builder, which produces the identical node arrays (same binned
// SAH, same split order, same pre-order node numbering) and runs the
// independent subtrees of the upper levels on separate host threads.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "vmr.h"

namespace vmr {

struct Bounds {
  float lo[3], hi[3];
};

struct HostMesh {
  uint32_t n_verts = 0, keys = 1, n_tris = 0;
  std::vector<float> verts;          // keys * n_verts * 3 (key-major)
  std::vector<uint32_t> idxp;        // leaf order (static) / face order (motion)
  std::vector<int32_t> accel_idx;    // leaf position -> face
  float ray_bias = 0.0f;
  int motion_mode = VMR_MOTION_FAITHFUL;
  std::vector<vmr_qbvh_node> nodes;  // static accelerator
  std::vector<vmr_mqbvh_node> mnodes;  // motion topology
  std::vector<float> mboxes;         // keys * n_mnodes * 24
  std::vector<Bounds> key_bounds;    // PolyMesh.motionBounds (motion only)
  Bounds bounds{};                   // PolyMesh.bounds
  std::vector<uint8_t> shader_idx;   // leaf order (static) / face order (motion)
  bool sphere = false;               // an analytic sphere geom (centre, radius)
  float sphere_c[3] = {0, 0, 0}, sphere_r = 0;
  // A GeomInstance (group 1) or Proc (group 2): no triangles of its own; its
  // bounds are the given BMin/BMax of key 0 at every time
  // (builtin/geom/instance/instance.go:64-68) and its motion keys those of
  // the geom it instances or the number of its transform keys
  // (instance.go:144-148, proc.go:181-185).
  int group = 0;
  int group_keys = 1;

  bool motion() const { return keys > 1; }
  int motion_keys() const { return group ? group_keys : (motion() ? (int)keys : 1); }
  // PolyMesh.Bounds (builtin/geom/polymesh/bounds.go:25-53).
  Bounds bounds_at(float time) const;
};

// PolyMesh.initAccel: fills nodes/mnodes/mboxes/accel_idx/bounds and
// permutes idxp (and shader_idx) to leaf order for a static mesh.
bool build_mesh_accel(HostMesh& m, std::string& err);

struct HostTop {
  std::vector<vmr_qbvh_node> nodes;
  std::vector<vmr_mqbvh_node> mnodes;
  std::vector<float> mboxes;         // keys * n_mnodes * 24
  uint32_t keys = 1;
  std::vector<uint32_t> geom_order;  // leaf position -> geom id
};

// Scene.initAccel (builtin/scene/scene.go:135-268) over the given meshes,
// which are identified by ids[i].
bool build_top_level(const std::vector<const HostMesh*>& meshes, const std::vector<uint32_t>& ids,
                     HostTop& top, std::string& err);

}  // namespace vmr
