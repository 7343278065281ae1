// megakernel.cu — the plain kernel form: one thread per pixel-sample.
//
// A block of 256 threads takes 256/spp consecutive pixels (row-major) and all
// of their samples, so the primary rays of a warp are coherent. Each thread
// traces one full path (trace.cuh); the block then sums every pixel's samples
// in sample order (the order of render_px_msaa's fold, renderer.rs:396-401),
// divides by spp, and updates the accumulation buffer in place
// (AccumulationValue::insert_sample, accum_buffer.rs:37-42). For spp > 256
// each thread loops over samples s = tid, tid + 256, ... and the block sums
// the per-thread partials in thread order.
#include <cuda_runtime.h>

#include "kernels.h"
#include "trace.cuh"

namespace rg {

constexpr int kMegaBlock = 256;

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

template <bool COUNT>
__global__ void __launch_bounds__(kMegaBlock) k_megakernel(GpuScene sc, FrameParams fp, uint32_t ppb, uint32_t n_pix) {
  __shared__ float sh[kMegaBlock][3];
  __shared__ unsigned long long sh_seg;
  const uint32_t tid = threadIdx.x;
  const uint32_t spp = fp.spp;
  if (tid == 0) sh_seg = 0;
  Counters cnt;
  uint32_t segments = 0;
  if (spp <= kMegaBlock) {
    uint32_t lp = tid / spp, s = tid % spp;
    uint32_t pix = blockIdx.x * ppb + lp;
    C3f col{0.0f, 0.0f, 0.0f};
    if (lp < ppb && pix < n_pix) col = trace_path<COUNT>(sc, fp, pix % fp.width, pix / fp.width, s, cnt, segments);
    sh[tid][0] = col.r; sh[tid][1] = col.g; sh[tid][2] = col.b;
    __syncthreads();
    if (tid < ppb * 3) {
      uint32_t p = tid / 3, c = tid % 3;
      uint32_t px = blockIdx.x * ppb + p;
      if (px < n_pix) {
        float sum = 0.0f;
        double sumd = 0.0, sqd = 0.0;
        for (uint32_t k = 0; k < spp; ++k) {
          float v = sh[p * spp + k][c];
          sum = sum + v;
          sumd += v;
          sqd += (double)v * v;
        }
        write_pixel(fp, px, (int)c, sum, sumd, sqd, spp);
      }
    }
  } else {
    __shared__ double shd[kMegaBlock][3];
    uint32_t pix = blockIdx.x;
    float sum[3] = {0.0f, 0.0f, 0.0f};
    double sq[3] = {0.0, 0.0, 0.0};
    for (uint32_t s = tid; s < spp; s += kMegaBlock) {
      C3f col = trace_path<COUNT>(sc, fp, pix % fp.width, pix / fp.width, s, cnt, segments);
      sum[0] = sum[0] + col.r; sum[1] = sum[1] + col.g; sum[2] = sum[2] + col.b;
      sq[0] += (double)col.r * col.r; sq[1] += (double)col.g * col.g; sq[2] += (double)col.b * col.b;
    }
    for (int c = 0; c < 3; ++c) { sh[tid][c] = sum[c]; shd[tid][c] = sq[c]; }
    __syncthreads();
    if (tid < 3) {
      float total = 0.0f;
      double td = 0.0, tq = 0.0;
      for (int k = 0; k < kMegaBlock; ++k) { total = total + sh[k][tid]; td += sh[k][tid]; tq += shd[k][tid]; }
      write_pixel(fp, pix, (int)tid, total, td, tq, spp);
    }
  }
  // Work counters: one atomic per warp.
  unsigned long long seg = segments;
  for (int o = 16; o > 0; o >>= 1) seg += __shfl_down_sync(0xffffffffu, seg, o);
  if ((tid & 31) == 0) atomicAdd(&sh_seg, seg);
  if (COUNT) {
    unsigned long long a = cnt.nodes, b = cnt.prims, c = cnt.sdf_steps;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if ((tid & 31) == 0) {
      atomicAdd(fp.counters + CNT_NODES, a);
      atomicAdd(fp.counters + CNT_PRIMS, b);
      atomicAdd(fp.counters + CNT_SDF, c);
    }
  }
  __syncthreads();
  if (tid == 0) atomicAdd(fp.counters + CNT_RAYS, sh_seg);
}

cudaError_t launch_megakernel(const GpuScene& sc, const FrameParams& fp, bool counters, cudaStream_t stream) {
  const uint32_t n_pix = fp.width * fp.height;
  uint32_t ppb = fp.spp <= (uint32_t)kMegaBlock ? kMegaBlock / fp.spp : 1u;
  uint32_t blocks = (n_pix + ppb - 1) / ppb;
  if (counters) k_megakernel<true><<<blocks, kMegaBlock, 0, stream>>>(sc, fp, ppb, n_pix);
  else k_megakernel<false><<<blocks, kMegaBlock, 0, stream>>>(sc, fp, ppb, n_pix);
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
  if (closest_hit<false>(sc, r, tmin[i], tmax[i], ctx, h, cnt, err)) {
    Surface s;
    finalize_hit(sc, r, h, ctx, s);
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
