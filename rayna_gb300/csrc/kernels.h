// kernels.h — host-side launchers of the device kernels.
#pragma once

#include <cuda_runtime.h>

#include "gpu_scene.h"

namespace rg {

// `block`: threads per block (a multiple of 32, at most 256; 0 = 256, the launch bound). The
// launch takes sc.shared_stack x block x 8 bytes of dynamic shared memory.
cudaError_t launch_megakernel(const GpuScene& sc, const FrameParams& fp, bool counters, cudaStream_t stream,
                              uint32_t block = 0);
cudaError_t launch_query(const GpuScene& sc, uint32_t n, const float* o, const float* d, const float* tmin,
                         const float* tmax, const float* vol_u, rg_hit* out, uint32_t* err, cudaStream_t stream);

}  // namespace rg
