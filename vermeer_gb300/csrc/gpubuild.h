// gpubuild.h - the device QBVH builder (gpubuild.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "accel.h"

namespace vmr {

struct DevBuf;

enum { kBuildOk = 0, kBuildDeclined = 1, kBuildError = -1 };

// Builds m's accelerator on the device with the same result as
// build_mesh_accel (nodes or motion nodes and boxes, accel_idx, bounds, idxp
// and shader_idx in leaf order for a static mesh).  For a static mesh the
// device triangle table is left in tris_out.  Returns kBuildDeclined for an
// empty mesh, build geometry that is not finite, or a task table overflow
// (the host builder takes those), kBuildError with err set on the
// reference's own build failures.
int device_build_mesh(HostMesh& m, DevBuf& tris_out, cudaStream_t s, std::string& err);

}  // namespace vmr
