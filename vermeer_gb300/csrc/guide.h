// guide.h - launch interface of the path-guiding network (guide.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace vmr {
namespace guide {

constexpr int kGuideWeights = 20032;  // W0 64x80, W1..W3 64x64, W4 41x64
constexpr int kGuideOut = 41;        // 8 lobes x 5, then the selection logit
constexpr int kGuideOutStride = 44;  // floats per row of an inference output
constexpr uint32_t kSaveRows = 640;   // values saved per training record (chunk-blocked)

// Path vertices (SoA, device pointers): hit point, shading normal, direction
// toward the previous vertex; n rows, or *n_dev rows when n_dev is set.  The
// training kernel reads row r at element r * rstride of every array
// (inference reads rows contiguously).
struct GuideRows {
  const float *px, *py, *pz, *nx, *ny, *nz, *wx, *wy, *wz;
  uint64_t n;
  const unsigned long long* n_dev;
  float lo[3], inv_ext[3];  // scene bounds: q = (p - lo) * inv_ext
  uint32_t rstride = 1;
};

// Training records: the rows plus the sampled direction and its weight
// (incident radiance over the density it was sampled with), and optionally
// the BSDF's density of that direction: with it the loss is that of the
// vertex's full sampling density alpha p_guide + (1 - alpha) p_bsdf, alpha =
// amax * sigmoid(selection logit), which also trains the selection.
struct GuideTrain {
  GuideRows rows;
  const float *ox, *oy, *oz, *weight;
  const float* pb;  // nullptr: the guide's own density
  float amax;
  uint32_t stride;  // records the save buffer holds (a multiple of 128)
};

struct GuideAdam {
  float lr, beta1, beta2, eps;
  int step;  // 0: only refresh the bf16 copies
};

size_t wf_elems();
// Shared-memory limits of the guide kernels (outside any stream capture).
void prepare_kernels();
// Random initial weights (seed 0) unless the context's guide already has some.
int ensure_ready(struct ::vmr_ctx* ctx);
size_t wb_elems();
// out: kGuideOutStride floats per row; sms: the device's SM count.
int launch_infer(const GuideRows& rows, const void* wf, float* out, int* err, int sms, cudaStream_t st);
// sms: the device's SM count (the kernel runs at most one CTA per SM).
int launch_train(const GuideTrain& tr, const void* wf, const void* wb, void* save, float* sums, int* err, int sms,
                 cudaStream_t st);
// save: the training kernel's chunk-blocked activations (record stride B,
// a multiple of 128); sms: the device's SM count.
int launch_wgrad(const void* save, uint32_t B, uint64_t n, const unsigned long long* n_dev, float* grad, int* err,
                 int sms, cudaStream_t st);
int launch_adam(float* W, float* m, float* v, float* grad, const float* sums, const GuideAdam& a, void* wf, void* wb,
                cudaStream_t st);

}  // namespace guide
}  // namespace vmr
