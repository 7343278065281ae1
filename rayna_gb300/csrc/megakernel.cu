// megakernel.cu — the plain kernel form: one thread per pixel-sample, each
// warp one round of whole pixels (mega.cuh). There is no block-wide barrier:
// a warp finishes as soon as its own paths do. Also the ray-query kernel.
#include <cuda_runtime.h>

#include "kernels.h"
#include "mega.cuh"

namespace rg {

// Threads per block: rg_tuning.block (64, 128 or 256; 256 by default). The
// launch bounds admit the largest.
constexpr int kMegaBlock = 256;

// The top sc.shared_stack entries of each thread's traversal stack live in
// the block's dynamic shared memory (shared_stack x blockDim x 8 bytes), the
// deeper ones in local memory; the current node and the postponed leaf stay
// in registers.
template <uint32_t F, bool COUNT, uint32_t KIND = kSamplePbr>
__global__ void __launch_bounds__(kMegaBlock) k_megakernel(GpuScene sc, FrameParams fp, uint32_t n_pix) {
  extern __shared__ uint2 mega_stack_sh[];
  const uint32_t warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  uint2 stack_loc[kTravStack];
  DynStack stack{mega_stack_sh + threadIdx.x, stack_loc, (int)sc.shared_stack, (int)blockDim.x};
  Counters cnt;
  uint32_t segments = 0;
  mega_round<F, COUNT, KIND>(sc, fp, warp * pixels_per_round(fp.spp), n_pix, cnt, segments, stack);
  flush_counters<COUNT>(fp, cnt, segments);
}

template <uint32_t F>
static void launch_mega(const GpuScene& sc, const FrameParams& fp, bool counters, uint32_t blocks, uint32_t block,
                        size_t smem, uint32_t n_pix, cudaStream_t stream) {
  if (counters) k_megakernel<F, true><<<blocks, block, smem, stream>>>(sc, fp, n_pix);
  else k_megakernel<F, false><<<blocks, block, smem, stream>>>(sc, fp, n_pix);
}

cudaError_t launch_megakernel(const GpuScene& sc, const FrameParams& fp, bool counters, cudaStream_t stream,
                              uint32_t block) {
  if (block == 0) block = kMegaBlock;
  if (block % 32 || block > (uint32_t)kMegaBlock) return cudaErrorInvalidValue;
  const uint32_t warps_per_block = block / 32;
  const size_t smem = (size_t)sc.shared_stack * block * sizeof(uint2);
  const uint32_t n_pix = fp.width * fp.height;
  const uint32_t ppw = pixels_per_round(fp.spp);
  const uint32_t warps = (n_pix + ppw - 1) / ppw;
  const uint32_t blocks = (warps + warps_per_block - 1) / warps_per_block;
  if (fp.mode != RG_MODE_PBR || fp.branching > 1) {
    // Debug render modes and ray_branching > 1: one variant over every
    // primitive kind (these are not throughput paths); work counters off.
    const uint32_t kind = fp.mode != RG_MODE_PBR ? kSampleMode : kSampleBranch;
    const bool wide = (sc.features & F_WIDE) != 0;
    if (kind == kSampleMode) {
      if (wide) k_megakernel<F_ANY | F_WIDE, false, kSampleMode><<<blocks, block, smem, stream>>>(sc, fp, n_pix);
      else k_megakernel<F_ANY, false, kSampleMode><<<blocks, block, smem, stream>>>(sc, fp, n_pix);
    } else {
      if (wide) k_megakernel<F_ANY | F_WIDE, false, kSampleBranch><<<blocks, block, smem, stream>>>(sc, fp, n_pix);
      else k_megakernel<F_ANY, false, kSampleBranch><<<blocks, block, smem, stream>>>(sc, fp, n_pix);
    }
    return cudaGetLastError();
  }
  dispatch_features(sc.features, [&](auto f) {
    launch_mega<decltype(f)::value>(sc, fp, counters, blocks, block, smem, n_pix, stream);
    return 0;
  });
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Ray queries: one thread per ray, closest hit with the full hit record.
// ---------------------------------------------------------------------------
template <uint32_t F>
__global__ void k_query(GpuScene sc, uint32_t n, const float* o, const float* d, const float* tmin, const float* tmax,
                        const float* vol_u, rg_hit* out, uint32_t* err) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Ray r = make_ray(v3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), v3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
  RngCtx ctx{0, 0, i, 0, 0, vol_u ? vol_u + (size_t)i * sc.n_volumes : nullptr};
  HitRec h;
  Counters cnt;
  rg_hit res;
  res.hit = 0; res.prim = 0; res.t = 0.0f;
  res.normal[0] = res.normal[1] = res.normal[2] = 0.0f;
  res.ray_normal[0] = res.ray_normal[1] = res.ray_normal[2] = 0.0f;
  res.front_face = 0; res.material = 0; res.side = 0;
  if (closest_hit<F, false>(sc, r, tmin[i], tmax[i], ctx, h, cnt, err)) {
    Surface s;
    finalize_hit<F>(sc, r, h, ctx, s, tmin[i]);
    res.hit = 1;
    res.prim = s.prim_id;
    res.t = h.t;
    res.normal[0] = s.normal.x; res.normal[1] = s.normal.y; res.normal[2] = s.normal.z;
    res.ray_normal[0] = s.ray_normal.x; res.ray_normal[1] = s.ray_normal.y; res.ray_normal[2] = s.ray_normal.z;
    res.front_face = s.front ? 1u : 0u;
    res.material = s.material;
    res.side = s.side;
  }
  out[i] = res;
}

cudaError_t launch_query(const GpuScene& sc, uint32_t n, const float* o, const float* d, const float* tmin, const float* tmax,
                         const float* vol_u, rg_hit* out, uint32_t* err, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  // The query traverses the tree the handle renders with, over every primitive kind.
  if (sc.features & F_WIDE) k_query<F_ANY | F_WIDE><<<(n + 127) / 128, 128, 0, stream>>>(sc, n, o, d, tmin, tmax, vol_u, out, err);
  else k_query<F_ANY><<<(n + 127) / 128, 128, 0, stream>>>(sc, n, o, d, tmin, tmax, vol_u, out, err);
  return cudaGetLastError();
}

}  // namespace rg
