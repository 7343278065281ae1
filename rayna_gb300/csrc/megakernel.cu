// megakernel.cu — the plain kernel form: one thread per pixel-sample.
//
// Each warp owns whole pixels: 32/spp pixels when spp <= 32 (lane l traces
// sample l % spp of pixel l / spp), or one pixel when spp > 32 (lane l traces
// samples l, l+32, ... one after another). Each thread traces full paths
// (trace.cuh); the warp then sums every pixel's samples with shuffles, divides
// by spp, and updates the accumulation buffer in place
// (AccumulationValue::insert_sample, accum_buffer.rs:37-42). There is no
// block-wide barrier: a warp finishes as soon as its own paths do.
//
// Sample sums follow one canonical order, shared with the wavefront form:
// for spp <= 32 samples 0..spp-1 in turn (the order of render_px_msaa's fold,
// renderer.rs:396-401); for spp > 32 lane partials (samples l, l+32, ... in
// turn) added for l = 0..31 in turn.
#include <cuda_runtime.h>

#include "kernels.h"
#include "trace.cuh"

namespace rg {

constexpr int kMegaBlock = 256;
constexpr int kWarpsPerBlock = kMegaBlock / 32;

__device__ __forceinline__ void write_pixel(const FrameParams& fp, uint32_t pix, int c, float sum, double sumd, double sqd,
                                            uint32_t n) {
  uint32_t x = pix % fp.width, y = pix / fp.width;
  size_t idx = ((size_t)x * fp.height + y) * 3 + c;
  float mean = sum / (float)n;
  float acc = fp.accum[idx] + mean;
  fp.accum[idx] = acc;
  if (fp.out) fp.out[idx] = (float)((double)acc / (double)fp.accum_count);
  if (fp.frame_mean) fp.frame_mean[idx] = mean;
  if (fp.frame_var) {
    double m = sumd / n;
    fp.frame_var[idx] = n > 1 ? (float)fmax(0.0, (sqd - n * m * m) / (n - 1)) : 0.0f;
  }
}

template <uint32_t F, bool COUNT>
__global__ void __launch_bounds__(kMegaBlock) k_megakernel(GpuScene sc, FrameParams fp, uint32_t n_pix) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  const uint32_t spp = fp.spp;
  Counters cnt;
  uint32_t segments = 0;
  if (spp <= 32) {
    const uint32_t ppw = 32 / spp;
    const uint32_t lp = lane / spp, s = lane % spp;
    const uint32_t pix = warp * ppw + lp;
    const bool active = lp < ppw && pix < n_pix;
    C3f col{0.0f, 0.0f, 0.0f};
    if (active) col = trace_path<F, COUNT>(sc, fp, pix % fp.width, pix / fp.width, s, cnt, segments);
    // Lane holding sample 0 of a pixel adds samples 1..spp-1 in order.
    const uint32_t base = lp * spp;
    float v[3] = {col.r, col.g, col.b};
    float sum[3] = {v[0], v[1], v[2]};
    double sumd[3] = {v[0], v[1], v[2]};
    double sqd[3] = {(double)v[0] * v[0], (double)v[1] * v[1], (double)v[2] * v[2]};
    for (uint32_t k = 1; k < spp; ++k) {
      uint32_t src = (base + k) & 31;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float o = __shfl_sync(0xffffffffu, v[c], src);
        sum[c] = sum[c] + o;
        sumd[c] += o;
        sqd[c] += (double)o * o;
      }
    }
    if (active && s == 0)
      for (int c = 0; c < 3; ++c) write_pixel(fp, pix, c, sum[c], sumd[c], sqd[c], spp);
  } else {
    const uint32_t pix = warp;
    const bool active = pix < n_pix;
    float part[3] = {0.0f, 0.0f, 0.0f};
    double psq[3] = {0.0, 0.0, 0.0};
    if (active) {
      for (uint32_t s = lane; s < spp; s += 32) {
        C3f col = trace_path<F, COUNT>(sc, fp, pix % fp.width, pix / fp.width, s, cnt, segments);
        part[0] = part[0] + col.r; part[1] = part[1] + col.g; part[2] = part[2] + col.b;
        psq[0] += (double)col.r * col.r; psq[1] += (double)col.g * col.g; psq[2] += (double)col.b * col.b;
      }
    }
    float sum[3] = {part[0], part[1], part[2]};
    double sumd[3] = {part[0], part[1], part[2]};
    double sqd[3] = {psq[0], psq[1], psq[2]};
    for (uint32_t k = 1; k < 32; ++k) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float o = __shfl_sync(0xffffffffu, part[c], k);
        double oq = __shfl_sync(0xffffffffu, psq[c], k);
        sum[c] = sum[c] + o;
        sumd[c] += o;
        sqd[c] += oq;
      }
    }
    if (active && lane == 0)
      for (int c = 0; c < 3; ++c) write_pixel(fp, pix, c, sum[c], sumd[c], sqd[c], spp);
  }
  // Work counters: one atomic per warp.
  unsigned long long seg = segments;
  for (int o = 16; o > 0; o >>= 1) seg += __shfl_down_sync(0xffffffffu, seg, o);
  if (lane == 0 && seg) atomicAdd(fp.counters + CNT_RAYS, seg);
  if (COUNT) {
    unsigned long long a = cnt.nodes, b = cnt.prims, c = cnt.sdf_steps;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if (lane == 0) {
      atomicAdd(fp.counters + CNT_NODES, a);
      atomicAdd(fp.counters + CNT_PRIMS, b);
      atomicAdd(fp.counters + CNT_SDF, c);
    }
  }
}

template <uint32_t F>
static void launch_mega(const GpuScene& sc, const FrameParams& fp, bool counters, uint32_t blocks, uint32_t n_pix,
                        cudaStream_t stream) {
  if (counters) k_megakernel<F, true><<<blocks, kMegaBlock, 0, stream>>>(sc, fp, n_pix);
  else k_megakernel<F, false><<<blocks, kMegaBlock, 0, stream>>>(sc, fp, n_pix);
}

cudaError_t launch_megakernel(const GpuScene& sc, const FrameParams& fp, bool counters, cudaStream_t stream) {
  const uint32_t n_pix = fp.width * fp.height;
  const uint32_t ppw = fp.spp <= 32 ? 32 / fp.spp : 1u;
  const uint32_t warps = (n_pix + ppw - 1) / ppw;
  const uint32_t blocks = (warps + kWarpsPerBlock - 1) / kWarpsPerBlock;
  if (sc.features == F_TRI) launch_mega<F_TRI>(sc, fp, counters, blocks, n_pix, stream);
  else if (sc.features == F_SPHERE) launch_mega<F_SPHERE>(sc, fp, counters, blocks, n_pix, stream);
  else launch_mega<F_ALL>(sc, fp, counters, blocks, n_pix, stream);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Ray queries: one thread per ray, closest hit with the full hit record.
// ---------------------------------------------------------------------------
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
  if (closest_hit<F_ALL, false>(sc, r, tmin[i], tmax[i], ctx, h, cnt, err)) {
    Surface s;
    finalize_hit<F_ALL>(sc, r, h, ctx, s);
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
  k_query<<<(n + 127) / 128, 128, 0, stream>>>(sc, n, o, d, tmin, tmax, vol_u, out, err);
  return cudaGetLastError();
}

}  // namespace rg
