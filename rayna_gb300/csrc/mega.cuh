// mega.cuh — the per-warp body of the megakernel, shared by the one-frame
// megakernel and the persistent batch kernel.
//
// A warp round covers whole pixels: 32/spp pixels when spp <= 32 (lane l
// traces sample l % spp of pixel l / spp), or one pixel when spp > 32 (lane l
// traces samples l, l+32, ... one after another). The warp then sums every
// pixel's samples with shuffles in the canonical order (samples 0..spp-1 in
// turn for spp <= 32, the order of render_px_msaa's fold, renderer.rs:396-401;
// for spp > 32 lane partials added for l = 0..31 in turn), divides by spp and
// updates the accumulation buffer (AccumulationValue::insert_sample,
// accum_buffer.rs:37-42).
#pragma once

#include "trace.cuh"

namespace rg {

__device__ __forceinline__ void write_pixel(const FrameParams& fp, uint32_t pix, int c, float sum, double sumd, double sqd,
                                            uint32_t n) {
  uint32_t x = pix % fp.width, y = pix / fp.width;
  size_t idx = ((size_t)x * fp.height + y) * 3 + c;
  float mean = sum / (float)n;
  // the accumulation adds sum / spp_total: the mean itself for a whole frame,
  // this range's share of it for one sample range of the frame
  float acc = fp.accum[idx] + (n == fp.spp_total ? mean : sum / (float)fp.spp_total);
  fp.accum[idx] = acc;
  if (fp.out) fp.out[idx] = (float)((double)acc / (double)fp.accum_count);
  if (fp.frame_mean) fp.frame_mean[idx] = mean;
  if (fp.frame_var) {
    double m = sumd / n;
    fp.frame_var[idx] = n > 1 ? (float)fmax(0.0, (sqd - n * m * m) / (n - 1)) : 0.0f;
  }
}

// Pixels covered by one warp round.
__host__ __device__ __forceinline__ uint32_t pixels_per_round(uint32_t spp) { return spp <= 32 ? 32 / spp : 1u; }

// One warp round starting at pixel `first` (all 32 lanes must call it).
template <uint32_t F, bool COUNT, uint32_t KIND, class Stack>
__device__ __forceinline__ void mega_round(const GpuScene& sc, const FrameParams& fp, uint32_t first, uint32_t n_pix,
                                           Counters& cnt, uint32_t& segments, Stack& stack) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t spp = fp.spp;
  if (spp <= 32) {
    const uint32_t ppw = 32 / spp;
    const uint32_t lp = lane / spp, s = lane % spp;
    const uint32_t pix = first + lp;
    const bool active = lp < ppw && pix < n_pix;
    C3f col{0.0f, 0.0f, 0.0f};
    if (active)
      col = trace_path<F, COUNT, KIND>(sc, fp, pix % fp.width, pix / fp.width, fp.sample_base + s, cnt, segments, stack);
    // The lane holding sample 0 of a pixel adds samples 1..spp-1 in order.
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
    const uint32_t pix = first;
    const bool active = pix < n_pix;
    float part[3] = {0.0f, 0.0f, 0.0f};
    double psq[3] = {0.0, 0.0, 0.0};
    if (active) {
      for (uint32_t s = lane; s < spp; s += 32) {
        C3f col = trace_path<F, COUNT, KIND>(sc, fp, pix % fp.width, pix / fp.width, fp.sample_base + s, cnt, segments,
                                             stack);
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
}

// Warp-summed work counters: one atomic per warp.
template <bool COUNT>
__device__ __forceinline__ void flush_counters(const FrameParams& fp, const Counters& cnt, uint32_t segments) {
  const uint32_t lane = threadIdx.x & 31;
  unsigned long long seg = segments;
  for (int o = 16; o > 0; o >>= 1) seg += __shfl_down_sync(0xffffffffu, seg, o);
  if (lane == 0 && seg) atomicAdd(fp.counters + CNT_RAYS, seg);
  if (COUNT) {
    unsigned long long a = cnt.nodes, b = cnt.prims, c = cnt.sdf_steps, d = cnt.sdf_iters, e = cnt.hits;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      c += __shfl_down_sync(0xffffffffu, c, o);
      d += __shfl_down_sync(0xffffffffu, d, o);
      e += __shfl_down_sync(0xffffffffu, e, o);
    }
    if (lane == 0) {
      atomicAdd(fp.counters + CNT_NODES, a);
      atomicAdd(fp.counters + CNT_PRIMS, b);
      atomicAdd(fp.counters + CNT_SDF, c);
      atomicAdd(fp.counters + CNT_SDF_ITERS, d);
      atomicAdd(fp.counters + CNT_HITS, e);
    }
  }
}

}  // namespace rg
