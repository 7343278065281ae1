// wavefront.cu — the wavefront kernel form (generate / extend / shade /
// accumulate over structure-of-arrays path queues).
#include <cuda_runtime.h>

#include "kernels.h"
#include "renderer_state.h"
#include "trace.cuh"

namespace rg {

cudaError_t launch_wavefront(rg_renderer* h, const FrameParams& fp) {
  (void)h;
  (void)fp;
  return cudaErrorNotSupported;
}

void free_extra(rg_renderer* h) {
  if (h->wf.arena) cudaFree(h->wf.arena);
  h->wf = WavefrontState{};
}

void on_scene_changed(rg_renderer* h) { (void)h; }

}  // namespace rg
