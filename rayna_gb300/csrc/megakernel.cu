// megakernel.cu — the plain kernel form: one thread per pixel-sample, each
// warp one round of whole pixels (mega.cuh). There is no block-wide barrier:
// a warp finishes as soon as its own paths do. Also the ray-query kernel.
#include <cuda_runtime.h>

#include "kernels.h"
#include "mega.cuh"

namespace rg {

constexpr int kMegaBlock = 256;
constexpr int kWarpsPerBlock = kMegaBlock / 32;

template <uint32_t F, bool COUNT, uint32_t KIND = kSamplePbr>
__global__ void __launch_bounds__(kMegaBlock) k_megakernel(GpuScene sc, FrameParams fp, uint32_t n_pix) {
  const uint32_t warp = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  Counters cnt;
  uint32_t segments = 0;
  mega_round<F, COUNT, KIND>(sc, fp, warp * pixels_per_round(fp.spp), n_pix, cnt, segments);
  flush_counters<COUNT>(fp, cnt, segments);
}

template <uint32_t F>
static void launch_mega(const GpuScene& sc, const FrameParams& fp, bool counters, uint32_t blocks, uint32_t n_pix,
                        cudaStream_t stream) {
  if (counters) k_megakernel<F, true><<<blocks, kMegaBlock, 0, stream>>>(sc, fp, n_pix);
  else k_megakernel<F, false><<<blocks, kMegaBlock, 0, stream>>>(sc, fp, n_pix);
}

cudaError_t launch_megakernel(const GpuScene& sc, const FrameParams& fp, bool counters, cudaStream_t stream) {
  const uint32_t n_pix = fp.width * fp.height;
  const uint32_t ppw = pixels_per_round(fp.spp);
  const uint32_t warps = (n_pix + ppw - 1) / ppw;
  const uint32_t blocks = (warps + kWarpsPerBlock - 1) / kWarpsPerBlock;
  if (fp.mode != RG_MODE_PBR || fp.branching > 1) {
    // Debug render modes and ray_branching > 1: one variant over every
    // primitive kind (these are not throughput paths); work counters off.
    const uint32_t kind = fp.mode != RG_MODE_PBR ? kSampleMode : kSampleBranch;
    const bool wide = (sc.features & F_WIDE) != 0;
    if (kind == kSampleMode) {
      if (wide) k_megakernel<F_ANY | F_WIDE, false, kSampleMode><<<blocks, kMegaBlock, 0, stream>>>(sc, fp, n_pix);
      else k_megakernel<F_ANY, false, kSampleMode><<<blocks, kMegaBlock, 0, stream>>>(sc, fp, n_pix);
    } else {
      if (wide) k_megakernel<F_ANY | F_WIDE, false, kSampleBranch><<<blocks, kMegaBlock, 0, stream>>>(sc, fp, n_pix);
      else k_megakernel<F_ANY, false, kSampleBranch><<<blocks, kMegaBlock, 0, stream>>>(sc, fp, n_pix);
    }
    return cudaGetLastError();
  }
  dispatch_features(sc.features, [&](auto f) {
    launch_mega<decltype(f)::value>(sc, fp, counters, blocks, n_pix, stream);
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
