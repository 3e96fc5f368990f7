// orc_internal.h - what the oracle's renderer needs from its traversal code.
// TEST INFRASTRUCTURE ONLY (see orc.h).
#pragma once
#include <cstdint>
#include <vector>

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

// A decomposed transform (math/animdecomp.go:14-18): translation, rotation
// quaternion (x, y, z, w), stretch matrix (column-major); orc_anim.cpp.
struct Decomp {
  float T[3];
  float R[4];
  float S[16];
};
void decomp_matrix(const float* m, Decomp& d);                       // TransformDecompMatrix4
void decomp_to_matrix(const Decomp& d, float* m);                    // TransformDecompToMatrix4
void decomp_lerp(const Decomp& a, const Decomp& b, float t, Decomp& o);  // TransformDecompLerp
// The keyed matrix at a time: one key as it is (TimeKey) unless blend_one
// (the camera blends it with itself), else the two keys around time blended.
bool decomp_at(const std::vector<Decomp>& keys, float time, bool blend_one, float* m);
bool matrix_inverse(const float* m, float* c);                       // Matrix4Inverse

struct MeshView {
  const float* verts;       // keys * nverts * 3
  uint32_t nverts, keys;
  const uint32_t* idxp;     // leaf order (static) / face order (motion)
  const uint8_t* shaderidx; // indexed by ElemID, or null
  const float* normals;     // per vertex, or null
  const float* mnormals;    // motion meshes: [key][mnormals_per_key][3], or null
  uint32_t mnormals_per_key;
  bool motion;
  bool sphere;              // analytic sphere geom: centre sc, radius sr
  float sc[3], sr;
  bool has_xf;              // PolyMesh.Transform and its inverse (column-major)
  float xf[16], xinv[16];
  const std::vector<Decomp>* xkeys;   // PolyMesh.Transform of >= 2 keys (else null)
  // The GeomInstance / Proc that reaches this mesh (its hits report this
  // view's id): ApplyTransform then uses that geom's transform at the ray's
  // time instead of the mesh's own (core/trace.go:69, instance.go:105-110).
  const std::vector<Decomp>* outer;   // null: none
};
MeshView mesh_view(const orc_mesh* m);

// A pixel filter's sampling tables (filter.go Sampler): n = 0 is no filter.
struct FilterTable {
  int n = 0;
  double w = 0.0;
  std::vector<double> cdfV, cdfVU;  // cdfVU row-major, row j = cdfVU[j]
};
FilterTable make_filter(const orc_pixel_filter& f);
void warp_sample(const FilterTable& t, double r0, double r1, double& u, double& v);

// What orc_render_create was given, for the extended path tracer (orc_pt.cpp).
struct RenderScene {
  const orc_scene* scene;
  std::vector<MeshView> meshes;
  std::vector<std::vector<uint32_t>> mesh_shaders;  // PolyMesh.Shader per mesh
  std::vector<orc_shader> shaders;
  std::vector<orc_trilight> lights;
  orc_camera cam;
  std::vector<Decomp> cam_keys;  // Camera.LocalToWorld keys, decomposed (camera.go:207-236)
  FilterTable filter;
};
RenderScene render_scene(const orc_render* r);

// core.Render's per-sample setup and the pinhole Camera.ComputeRay
// (core/render.go:89-120, builtin/camera/camera.go:244-284) for iteration j
// (render(iter+1)) of pixel pix: ray origin, direction and time; filt (may
// be null or empty) warps the sample inside its pixel first.
// M = TransformDecompToMatrix4(TransformDecompLerp(...)) of the camera keys at
// the sample's time (camera.go:223-236).
void camera_primary(const orc_camera& c, const std::vector<Decomp>& keys, uint32_t w, uint32_t h, uint32_t j,
                    uint64_t pix, uint64_t seed, float P[3], float D[3], float* time,
                    const FilterTable* filt = nullptr);

}  // namespace orc_internal
