// wavefront.cuh — path state and per-path device functions shared by the
// wavefront form (wavefront.cu) and the batched wavefront (batch.cu).
//
// Path state is one 48-byte record per slot (origin + depth, direction + hit
// distance, throughput + hit primitive), read and written as three float4. A
// path's radiance is zero until it ends (emission is only met at a light,
// which ends the path, or at the sky), so it is written once, at the end, to
// the per-slot sample buffer.
#pragma once

#include <cuda_runtime.h>

#include "renderer_state.h"
#include "trace.cuh"

namespace rg {

constexpr int kWfBlock = 256;
// Traversal stack entries per thread kept in shared memory by the persistent
// batched kernel (16 KB per block of 256); deeper entries live in local
// memory. The split measured 1.07x on the 1.3M-triangle mesh (8 and 16
// entries alike), 0.98x on scenes of spheres only (shallow trees) and 1.00x
// on the SDF scene; it is used where it was measured to pay, the
// triangle-only variants. (Single renders take the count from the handle's
// tuning, rg_tuning.shared_stack, with the same default.)
constexpr int kSharedStack = 8;
template <uint32_t F> constexpr int kSharedStackOf = kinds_of(F) == F_TRI ? kSharedStack : 0;
constexpr int kKinds = 6;  // miss, lambertian, metal, dielectric, isotropic, light
enum : uint32_t { KQ_MISS = 0 };
constexpr int kPrimMiss = -1;  // rec[2].w: >= 0 BVH primitive, -1 miss, -2 - k SDF k

struct PathState {
  float4* rec;          // 3 x float4 per slot: (origin, depth) (direction, t) (throughput, prim)
  float4* aux;          // per slot: SDF hit normal + (front bit 31 | side); transformed hit: mesh-space distance in x
  float *sr, *sg, *sb;  // per-slot sample radiance
  uint32_t* active[2];
  uint32_t* kindq;      // kKinds x capacity
  uint32_t* marchq;     // per-SDF march queues (n_march x capacity, counts at kMarchQueueCount0 + k), or null: one
                        // march queue (the next bounce's active array) for every stage
  uint32_t* counts;     // [0], [1]: active counts; [2 .. 2+kKinds): kind counts; [kFetchCounter]: the traversal kernels'
                        // fetch counter; [kMarchCounter]: the march queue's count
};
constexpr int kFetchCounter = 2 + kKinds;
constexpr int kMarchCounter = kFetchCounter + 1;
constexpr int kMarchQueueCount0 = 16;  // counts[16 + k]: SDF k's march queue
constexpr int kMaxRoutedSdfs = 48;     // SDFs that get queues of their own (the counts array holds 64 words)

struct WaveParams {
  uint32_t first_pixel, n_pixels, n_paths, capacity;
};

__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
  unsigned mask = __activemask();
  unsigned ballot = __ballot_sync(mask, pred);
  int lane = threadIdx.x & 31;
  int leader = __ffs(mask) - 1;
  uint32_t base = 0;
  if (lane == leader && ballot) base = atomicAdd(counter, (uint32_t)__popc(ballot));
  base = __shfl_sync(mask, base, leader);
  return base + __popc(ballot & ((1u << lane) - 1u));
}

__device__ __forceinline__ void store_path(const PathState& s, uint32_t p, V3 o, uint32_t depth, V3 d, C3f beta) {
  s.rec[3 * (size_t)p] = make_float4(o.x, o.y, o.z, __uint_as_float(depth));
  s.rec[3 * (size_t)p + 1] = make_float4(d.x, d.y, d.z, 0.0f);
  s.rec[3 * (size_t)p + 2] = make_float4(beta.r, beta.g, beta.b, __int_as_float(kPrimMiss));
}

__device__ __forceinline__ void finish_path(const PathState& s, uint32_t p, C3f L) {
  s.sr[p] = L.r; s.sg[p] = L.g; s.sb[p] = L.b;
}

// Whether this warp of a persistent kernel has nothing to do: only the first
// ceil(n / 32) warps of the grid take paths from a queue of n, so that a
// short queue (the tail bounces) is not fetched from by every resident warp
// (thousands of atomics on one counter) just to find it empty.
__device__ __forceinline__ bool warp_unneeded(uint32_t n) {
  const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  return (uint64_t)gwarp * 32u >= n;
}

__device__ __forceinline__ uint32_t clamp_count(uint32_t n, const WaveParams& wp, uint32_t* err) {
  if (n > wp.n_paths) {  // never expected: record and clamp instead of reading past the queue
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, ERR_QUEUE_OVERFLOW);
    return wp.n_paths;
  }
  return n;
}

// Shading of one path at its closest hit (or miss). Returns true when the path
// continues; then its record holds the scattered ray. Ended paths write their
// radiance.
// CHECK (the counting variants): RG_FLAG_VALIDATE's checks of the hit and of
// the path's colour.
template <uint32_t F, bool CHECK = false>
__device__ __forceinline__ bool shade_path(const GpuScene& sc, const FrameParams& fp, const PathState& s, uint32_t p,
                                           uint32_t pix, uint32_t smp, uint32_t depth, const Ray& r, C3f beta,
                                           bool hit, const HitRec& h) {
  if (!hit) {
    C3f sk = sky_of<F>(sc, r.d);
    const C3f L{0.0f + beta.r * sk.r, 0.0f + beta.g * sk.g, 0.0f + beta.b * sk.b};
    if (CHECK && fp.validate) validate_colour(fp, L);
    finish_path(s, p, L);
    return false;
  }
  RngCtx ctx{fp.seed_lo, fp.seed_hi, pix, smp, depth, nullptr};
  Surface surf;
  finalize_hit<F>(sc, r, h, ctx, surf, 1e-3f);
  if (CHECK && fp.validate) validate_hit(fp, r, h.t, surf, 1e-3f, 3.402823466e38f);
  const rg_material m = sc.materials[surf.material];
  if (m.kind == RG_MAT_LIGHT) {
    const C3f e = material_colour<F>(sc, m, surf);
    const C3f L{0.0f + beta.r * e.r, 0.0f + beta.g * e.g, 0.0f + beta.b * e.b};
    if (CHECK && fp.validate) validate_colour(fp, L);
    finish_path(s, p, L);
    return false;
  }
  if (depth < fp.ray_depth) {
    V3 dir;
    if (scatter(m, r, surf, ctx, dir)) {
      C3f a = attenuation<F>(sc, m, r, surf);
      beta = C3f{beta.r * a.r, beta.g * a.g, beta.b * a.b};
      Ray nr = make_ray(surf.pos, dir);
      store_path(s, p, nr.o, depth + 1, nr.d, beta);
      return true;
    }
  }
  finish_path(s, p, C3f{0.0f, 0.0f, 0.0f});
  return false;
}

template <bool COUNT>
__device__ __forceinline__ void flush_wave_counters(const FrameParams& fp, const Counters& cnt, uint32_t queries) {
  unsigned long long q = queries;
  for (int o = 16; o > 0; o >>= 1) q += __shfl_down_sync(0xffffffffu, q, o);
  if ((threadIdx.x & 31) == 0 && q) atomicAdd(fp.counters + CNT_RAYS, q);
  if (COUNT) {
    unsigned long long a = cnt.nodes, b = cnt.prims, c = cnt.sdf_steps, d = cnt.sdf_iters, e = cnt.hits;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      c += __shfl_down_sync(0xffffffffu, c, o);
      d += __shfl_down_sync(0xffffffffu, d, o);
      e += __shfl_down_sync(0xffffffffu, e, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(fp.counters + CNT_NODES, a);
      atomicAdd(fp.counters + CNT_PRIMS, b);
      atomicAdd(fp.counters + CNT_SDF, c);
      atomicAdd(fp.counters + CNT_SDF_ITERS, d);
      atomicAdd(fp.counters + CNT_HITS, e);
    }
  }
}

// Per-pixel sums in the megakernel's canonical order: samples 0..spp-1 in
// turn for spp <= 32; for larger spp, lane partials (samples l, l+32, ...)
// added for l = 0..31 in turn. `base` is the pixel's first slot; `pix` its
// index in the frame (x-major output order [x][y][rgb]).
__device__ __forceinline__ void accumulate_pixel(const FrameParams& fp, const PathState& s, size_t base, uint32_t pix,
                                                 uint32_t c) {
  const uint32_t spp = fp.spp;
  const float* src = (c == 0 ? s.sr : (c == 1 ? s.sg : s.sb)) + base;
  float sum = 0.0f;
  double sumd = 0.0, sqd = 0.0;
  if (spp <= 32) {
    for (uint32_t k = 0; k < spp; ++k) {
      float v = src[k];
      sum = sum + v;
      sumd += v;
      sqd += (double)v * v;
    }
  } else {
    for (uint32_t l = 0; l < 32; ++l) {
      float part = 0.0f;
      double psq = 0.0;
      for (uint32_t k = l; k < spp; k += 32) {
        float v = src[k];
        part = part + v;
        psq += (double)v * v;
      }
      sum = sum + part;
      sumd += part;
      sqd += psq;
    }
  }
  uint32_t x = pix % fp.width, y = pix / fp.width;
  size_t idx = ((size_t)x * fp.height + y) * 3 + c;
  float mean = sum / (float)spp;
  // the accumulation adds sum / spp_total: the mean itself for a whole frame,
  // this range's share of it for one sample range of the frame
  float acc = fp.accum[idx] + (spp == fp.spp_total ? mean : sum / (float)fp.spp_total);
  fp.accum[idx] = acc;
  if (fp.out) fp.out[idx] = (float)((double)acc / (double)fp.accum_count);
  if (fp.frame_mean) fp.frame_mean[idx] = mean;
  if (fp.frame_var) {
    double m = sumd / spp;
    fp.frame_var[idx] = spp > 1 ? (float)fmax(0.0, (sqd - spp * m * m) / (spp - 1)) : 0.0f;
  }
}

// Bytes per path slot of each path array, in the order carve lays them out:
// the records, the side record, the sample radiance r, g, b, the two active
// queues and the material-kind queues; then the counts.
constexpr size_t kSlotArrayBytes[] = {48, 16, 4, 4, 4, 4, 4, 4 * kKinds};
constexpr size_t kCountsBytes = 64 * 4;
constexpr size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

// Bytes carve uses for `cap` slots (108 per slot, each array 256-byte aligned, plus the counts).
constexpr size_t arena_bytes(size_t cap) {
  size_t used = 0;
  for (size_t b : kSlotArrayBytes) used += round256(cap * b);
  return used + round256(kCountsBytes);
}

// Lays the path arrays out from `arena` (256-byte aligned each) and returns
// the number of bytes used, arena_bytes(cap).
inline size_t carve(char* arena, size_t cap, PathState& s) {
  size_t used = 0;
  int k = 0;
  auto take = [&](size_t bytes) {
    char* r = arena + used;
    used += round256(bytes);
    return r;
  };
  s.rec = (float4*)take(cap * kSlotArrayBytes[k++]);
  s.aux = (float4*)take(cap * kSlotArrayBytes[k++]);
  s.sr = (float*)take(cap * kSlotArrayBytes[k++]);
  s.sg = (float*)take(cap * kSlotArrayBytes[k++]);
  s.sb = (float*)take(cap * kSlotArrayBytes[k++]);
  s.active[0] = (uint32_t*)take(cap * kSlotArrayBytes[k++]);
  s.active[1] = (uint32_t*)take(cap * kSlotArrayBytes[k++]);
  s.kindq = (uint32_t*)take(cap * kSlotArrayBytes[k++]);
  s.marchq = nullptr;
  s.counts = (uint32_t*)take(kCountsBytes);
  return used;
}

inline int sm_count(int device) {
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
  return n > 0 ? n : 1;
}

}  // namespace rg
