// orc_internal.h - what the oracle's renderer needs from its traversal code.
// TEST INFRASTRUCTURE ONLY (see orc.h).
#pragma once
#include <cstdint>

#include "orc.h"

namespace orc_internal {

struct Hit {
  bool hit;
  bool overflow;
  int32_t elem;  // ShaderContext.ElemID
  int32_t geom;  // index of the hit mesh among those given to orc_scene_create
  float t, u, v, w;
};

// Scene.Trace of one ray (builtin/scene/scene.go:30-58); shadow = RayTypeShadow.
Hit trace(const orc_scene* s, const float P[3], const float D[3], float tmax, float time, bool shadow);

struct MeshView {
  const float* verts;       // keys * nverts * 3
  uint32_t nverts, keys;
  const uint32_t* idxp;     // leaf order (static) / face order (motion)
  const uint8_t* shaderidx; // indexed by ElemID, or null
  const float* normals;     // per vertex, or null
  bool motion;
};
MeshView mesh_view(const orc_mesh* m);

}  // namespace orc_internal
