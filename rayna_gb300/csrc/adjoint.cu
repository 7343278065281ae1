// adjoint.cu — gradients of an image loss by path-replay backpropagation
// (Vicini, Speierer, Jakob, "Path Replay Backpropagation", SIGGRAPH 2021).
//
// The frame's image I (mean of spp path samples per pixel) is a function of
// the material albedos and emissions and of the media densities. Given the
// adjoint image dLoss/dI, each path is traced again from its counter-based
// random stream (nothing of the forward pass is stored: memory stays
// O(pixels)); the replay records the path's vertices in thread-local memory
// and a backward loop over them accumulates
//   dL/d albedo_m   += delta * beta_j * g_j * c_{j+1}   (vertex j of material m)
//   dL/d emission_m += delta * beta_j                    (light vertex j)
//   dL/d density_v  += sum_c delta_c * s_{j,v} * beta_j,c * c_j,c
// where beta_j is the throughput before vertex j, g_j the attenuation factor
// other than the albedo (Beer term), c_j = e_j + a_j * c_{j+1} the radiance
// leaving vertex j (sky or 0 at the end), and s_{j,v} the score of the
// free-flight decision of medium v on segment j: 1/density - (t - enter) for
// the medium that scattered, -(min(exit, t) - enter) for one passed through.
// Scattered directions do not depend on albedos, so the albedo and emission
// gradients of a sample are exact; density gradients are the score-function
// estimator of the derivative of the expectation. Geometric edges are out of
// scope. Gradients are summed with warp-aggregated atomics
// (__match_any_sync on the material or medium index), per block in shared
// memory when the scene's gradients fit there.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <vector>

#include "kernels.h"
#include "renderer_state.h"
#include "trace.cuh"

namespace rg {

namespace {

constexpr int kAdjBlock = 256;
constexpr int kAdjMaxVertices = 17;  // ray_depth + 1
constexpr int kAdjMaxVolumes = 4;

struct AdjParams {
  const float* adjoint;  // [x][y][rgb] dLoss/dI
  float* g_albedo;       // n_mat x 3
  float* g_emission;     // n_mat x 3
  float* g_density;      // n_vol
  uint32_t n_vol;
  uint32_t n_mat;
  int block_sums;        // accumulate per block in shared memory, flush to g_* at the end
};

// Gradient entries a block can sum in shared memory (48 KB less the 16 KB
// of traversal stacks): scenes with up to 1365 materials. RG_ADJ_BLOCK_SUMS=0
// at build time sends every gradient atomic to global memory instead.
constexpr uint32_t kAdjSharedGrads = 8192;
#ifndef RG_ADJ_BLOCK_SUMS
#define RG_ADJ_BLOCK_SUMS 1
#endif

// Adds (v0, v1, v2) to base[3*key .. 3*key+2], one atomic per distinct key in the warp.
__device__ __forceinline__ void warp_add3(float* base, int key, float v0, float v1, float v2) {
  unsigned act = __activemask();
  unsigned peers = __match_any_sync(act, key);
  float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
  for (unsigned m = peers; m; m &= m - 1) {
    int src = __ffs(m) - 1;
    s0 += __shfl_sync(peers, v0, src);
    s1 += __shfl_sync(peers, v1, src);
    s2 += __shfl_sync(peers, v2, src);
  }
  if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) {
    atomicAdd(base + 3 * key, s0);
    atomicAdd(base + 3 * key + 1, s1);
    atomicAdd(base + 3 * key + 2, s2);
  }
}

__device__ __forceinline__ void warp_add1(float* base, int key, float v) {
  unsigned act = __activemask();
  unsigned peers = __match_any_sync(act, key);
  float s = 0.0f;
  for (unsigned m = peers; m; m &= m - 1) s += __shfl_sync(peers, v, __ffs(m) - 1);
  if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(base + key, s);
}

// Free-flight scores of every medium for one ray segment that ended at
// `t_final` (+inf when it escaped); `winner` is the medium that scattered, or -1.
__device__ __forceinline__ void medium_scores(const GpuScene& sc, const Ray& r, float start, float t_final, int winner,
                                              uint32_t n_vol, float* score) {
  for (uint32_t v = 0; v < n_vol; ++v) {
    score[v] = 0.0f;
    const GpuPrim p = sc.prims[sc.vol_prim[v]];
    uint32_t kind = prim_kind(p);
    float d_enter, d_exit;
    if (!boundary_t(p, kind, r, -CUDART_INF_F, CUDART_INF_F, d_enter)) continue;
    float enter = fmaxf(d_enter, start);
    if (!boundary_t(p, kind, r, enter + 0.001f, CUDART_INF_F, d_exit)) continue;
    if ((int)v == winner) {
      score[v] = __frcp_rn(sc.vol_density[v]) - (t_final - enter);
    } else {
      float l = fminf(d_exit, t_final) - enter;
      score[v] = l > 0.0f ? -l : 0.0f;
    }
  }
}

// Traversal stack entries per thread in shared memory (the rest local), as
// in the persistent wavefront kernels.
constexpr int kAdjSharedStack = 8;
using AdjStack = SplitStack<kAdjSharedStack, kAdjBlock>;

// One replayed path's vertices (thread-local): material, light and
// albedo-dependence flags, the non-albedo factor g_j (Beer term), the
// throughput before each vertex and the media's free-flight scores of each
// segment.
struct ReplayPath {
  int mat[kAdjMaxVertices];
  uint32_t light, albdep;  // bit j: vertex j
  float g[kAdjMaxVertices];
  float beta[kAdjMaxVertices + 1][3];
  float score[kAdjMaxVertices + 1][kAdjMaxVolumes];
  float b0, b1, b2;
  int K;
  bool escaped;
  C3f sky;
};

// Where a path's gradients go: the block's shared-memory sums, or global memory.
struct GradSink {
  float* albedo;
  float* emission;
  float* density;
};

__device__ __forceinline__ void replay_begin(ReplayPath& P) {
  P.b0 = P.b1 = P.b2 = 1.0f;
  P.K = 0;
  P.light = P.albdep = 0u;
  P.escaped = false;
  P.sky = C3f{0.0f, 0.0f, 0.0f};
}

// The segment of the path that just ended at its closest hit (or escaped):
// records the vertex and, when the path goes on, replaces `ray` with the
// scattered ray and returns true (the forward path's decisions, trace.cuh's
// trace_path, with the same random streams).
template <uint32_t F>
__device__ __forceinline__ bool replay_segment(const GpuScene& sc, const FrameParams& fp, const AdjParams& ap,
                                               ReplayPath& P, Ray& ray, const RngCtx& ctx, uint32_t depth, bool hit,
                                               const HitRec& h) {
  const int K = P.K;
  int winner = -1;
  if (hit && h.sdf < 0 && (F & F_VOL)) {
    uint32_t kind = prim_kind(sc.prims[h.prim]);
    if (kind == PK_VOL_SPHERE || kind == PK_VOL_BOX) winner = (int)(prim_id(sc.prims[h.prim]) - sc.vol_base);
  }
  P.beta[K][0] = P.b0; P.beta[K][1] = P.b1; P.beta[K][2] = P.b2;
  if (F & F_VOL) medium_scores(sc, ray, 1e-3f, hit ? h.t : CUDART_INF_F, winner, ap.n_vol, P.score[K]);
  if (!hit) {
    P.escaped = true;
    P.sky = sky_colour(sc.sky, ray.d);
    return false;
  }
  Surface surf;
  finalize_hit<F>(sc, ray, h, ctx, surf, 1e-3f);
  const rg_material m = sc.materials[surf.material];
  P.mat[K] = (int)surf.material;
  if (m.kind == RG_MAT_LIGHT) P.light |= 1u << K;
  P.g[K] = 1.0f;
  P.K = K + 1;
  if (m.kind == RG_MAT_LIGHT || depth == fp.ray_depth) return false;
  V3 dir;
  if (!scatter(m, ray, surf, ctx, dir)) return false;
  const C3f a = attenuation<F>(sc, m, ray, surf);
  if (m.kind == RG_MAT_LAMBERTIAN || m.kind == RG_MAT_METAL) {
    P.albdep |= 1u << K;
  } else if (!(m.kind == RG_MAT_DIELECTRIC && surf.front)) {
    P.albdep |= 1u << K;
    P.g[K] = expf(-m.density * length3(surf.pos - ray.o));
  }
  P.b0 = P.b0 * a.r; P.b1 = P.b1 * a.g; P.b2 = P.b2 * a.b;
  ray = make_ray(surf.pos, dir);
  return true;
}

// Backward over a finished path's vertices, gradients to global memory with
// warp-aggregated atomics among the lanes finishing together. (d0, d1, d2)
// is the pixel's dLoss/dI divided by its samples.
template <uint32_t F>
__device__ __forceinline__ void replay_backward(const GpuScene& sc, const AdjParams& ap, const GradSink& gs,
                                                const ReplayPath& P, float d0, float d1, float d2) {
  const int K = P.K;
  const uint32_t n_vol = ap.n_vol;
  float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
  if (P.escaped) {
    c0 = P.sky.r; c1 = P.sky.g; c2 = P.sky.b;
    if (F & F_VOL)
      for (uint32_t v = 0; v < n_vol; ++v) {
        float sv = P.score[K][v];
        float gv = sv * (d0 * P.beta[K][0] * c0 + d1 * P.beta[K][1] * c1 + d2 * P.beta[K][2] * c2);
        if (gv != 0.0f) warp_add1(gs.density, (int)v, gv);
      }
  }
  for (int j = K - 1; j >= 0; --j) {
    const int m = P.mat[j];
    const rg_material mm = sc.materials[m];
    if ((P.light >> j) & 1u) {
      warp_add3(gs.emission, m, d0 * P.beta[j][0], d1 * P.beta[j][1], d2 * P.beta[j][2]);
      c0 = mm.albedo[0]; c1 = mm.albedo[1]; c2 = mm.albedo[2];
    } else if ((P.albdep >> j) & 1u) {
      const float gj = P.g[j];
      warp_add3(gs.albedo, m, d0 * P.beta[j][0] * gj * c0, d1 * P.beta[j][1] * gj * c1, d2 * P.beta[j][2] * gj * c2);
      c0 = c0 * (mm.albedo[0] * gj);
      c1 = c1 * (mm.albedo[1] * gj);
      c2 = c2 * (mm.albedo[2] * gj);
    }
    // a vertex that does not depend on the albedo (dielectric entry) passes c on unchanged
    if (F & F_VOL)
      for (uint32_t v = 0; v < n_vol; ++v) {
        float sv = P.score[j][v];
        float gv = sv * (d0 * P.beta[j][0] * c0 + d1 * P.beta[j][1] * c1 + d2 * P.beta[j][2] * c2);
        if (gv != 0.0f) warp_add1(gs.density, (int)v, gv);
      }
  }
}

// The block's gradient sink: shared-memory sums (zeroed here; the whole
// block calls this) when `block_sums`, else global memory.
__device__ __forceinline__ GradSink block_sink(const AdjParams& ap, float* grad_sh) {
  GradSink gs{ap.g_albedo, ap.g_emission, ap.g_density};
  if (ap.block_sums) {
    const uint32_t n_grad = 6 * ap.n_mat + ap.n_vol;
    for (uint32_t i = threadIdx.x; i < n_grad; i += blockDim.x) grad_sh[i] = 0.0f;
    gs = GradSink{grad_sh, grad_sh + 3 * ap.n_mat, grad_sh + 6 * ap.n_mat};
    __syncthreads();
  }
  return gs;
}

// Adds the block's shared-memory sums to global memory (the whole block calls this).
__device__ __forceinline__ void flush_block_sums(const AdjParams& ap, const float* grad_sh) {
  if (!ap.block_sums) return;
  __syncthreads();
  const uint32_t n_grad = 6 * ap.n_mat + ap.n_vol;
  for (uint32_t i = threadIdx.x; i < n_grad; i += blockDim.x) {
    const float v = grad_sh[i];
    if (v != 0.0f) {
      float* dst = i < 3 * ap.n_mat ? ap.g_albedo + i
                 : (i < 6 * ap.n_mat ? ap.g_emission + (i - 3 * ap.n_mat) : ap.g_density + (i - 6 * ap.n_mat));
      atomicAdd(dst, v);
    }
  }
}

// One path of pixel (x, y), sample s: traced again with its random streams,
// then differentiated; (d0, d1, d2) is the pixel's dLoss/dI over its samples.
template <uint32_t F>
__device__ __forceinline__ void replay_path(AdjStack& stack, const GpuScene& sc, const FrameParams& fp,
                                            const AdjParams& ap, const GradSink& gs, uint32_t x, uint32_t y, uint32_t s,
                                            float d0, float d1, float d2) {
  const uint32_t pix = y * fp.width + x;
  Ray ray = camera_ray(fp, x, y, s, RngCtx{fp.seed_lo, fp.seed_hi, pix, s, 0, nullptr});
  ReplayPath P;
  replay_begin(P);
  Counters cnt;
  for (uint32_t depth = 0;; ++depth) {
    const RngCtx ctx{fp.seed_lo, fp.seed_hi, pix, s, depth, nullptr};
    HitRec h;
    const bool hit = closest_hit_with<F, false>(stack, sc, ray, 1e-3f, 3.402823466e38f, ctx, h, cnt, fp.err);
    if (!replay_segment<F>(sc, fp, ap, P, ray, ctx, depth, hit, h)) break;
  }
  replay_backward<F>(sc, ap, gs, P, d0, d1, d2);
}

// The replay's grid form (RG_ADJ_PERSISTENT=0): one thread per pixel-sample,
// a warp taking whole pixels as the megakernel does (its lanes then end their
// backward passes together, so the warp-aggregated atomics group every lane
// with the same material). With `block_sums` the gradients go to the block's
// shared memory and each block adds its sums to global memory once, at the
// end. It measured 4.54 ms per iteration of the adjoint workload against the
// persistent form's 3.60.
template <uint32_t F>
__global__ void __launch_bounds__(kAdjBlock) k_replay(GpuScene sc, FrameParams fp, AdjParams ap, uint32_t n_pix) {
  extern __shared__ float grad_sh[];  // albedo, emission (n_mat x 3 each), density (n_vol), with block_sums
  const GradSink gs = block_sink(ap, grad_sh);
  __shared__ uint2 stack_sh[kAdjSharedStack * kAdjBlock];
  uint2 stack_loc[kTravStack - kAdjSharedStack];
  AdjStack stack{stack_sh + threadIdx.x, stack_loc};
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = blockIdx.x * (kAdjBlock / 32) + (threadIdx.x >> 5);
  const uint32_t spp = fp.spp;
  const float inv = 1.0f / (float)spp;
  if (spp <= 32) {
    const uint32_t ppw = 32 / spp;
    const uint32_t lp = lane / spp, s = lane % spp;
    const uint32_t pix = warp * ppw + lp;
    if (lp < ppw && pix < n_pix) {
      const uint32_t x = pix % fp.width, y = pix / fp.width;
      const size_t idx = ((size_t)x * fp.height + y) * 3;
      replay_path<F>(stack, sc, fp, ap, gs, x, y, s, ap.adjoint[idx] * inv, ap.adjoint[idx + 1] * inv,
                     ap.adjoint[idx + 2] * inv);
    }
  } else {
    const uint32_t pix = warp;
    if (pix < n_pix) {
      const uint32_t x = pix % fp.width, y = pix / fp.width;
      const size_t idx = ((size_t)x * fp.height + y) * 3;
      const float d0 = ap.adjoint[idx] * inv, d1 = ap.adjoint[idx + 1] * inv, d2 = ap.adjoint[idx + 2] * inv;
      for (uint32_t s = lane; s < spp; s += 32) replay_path<F>(stack, sc, fp, ap, gs, x, y, s, d0, d1, d2);
    }
  }
  flush_block_sums(ap, grad_sh);
}

// The replay (default form) as a persistent kernel with dynamic fetch, as the forward's
// wavefront traversal kernels run: each lane holds one path (samples taken
// in pixel order from one counter, one atomic per warp and refill), traverses
// `budget` node visits at a time, and the lanes whose segment has ended are
// finished together once `shade_lanes` of them (or all of the warp's live
// lanes) are ready: the vertex is recorded and the path scattered, or, at
// its end, differentiated, so the backward passes and their warp-aggregated
// atomics run on many lanes at once. Gradients are summed per block in
// shared memory when they fit.
template <uint32_t F>
__global__ void __launch_bounds__(kAdjBlock) k_replay_persistent(GpuScene sc, FrameParams fp, AdjParams ap,
                                                                 uint32_t n_items, uint32_t* counter, int budget,
                                                                 int shade_lanes) {
  extern __shared__ float grad_sh[];
  const GradSink gs = block_sink(ap, grad_sh);
  __shared__ uint2 stack_sh[kAdjSharedStack * kAdjBlock];
  uint2 stack_loc[kTravStack - kAdjSharedStack];
  AdjStack stack{stack_sh + threadIdx.x, stack_loc};
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t spp = fp.spp;
  const float inv = 1.0f / (float)spp;
  bool has = false, done = false, drained = false;
  uint32_t pix = 0, smp = 0, depth = 0;
  float d0 = 0.0f, d1 = 0.0f, d2 = 0.0f;
  Ray ray;
  Traversal t;
  ReplayPath P;
  Counters cnt;
  for (;;) {
    const unsigned idle = __ballot_sync(0xffffffffu, !has);
    if (idle && !drained) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(counter, (uint32_t)__popc(idle));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + (uint32_t)__popc(idle) >= n_items) drained = true;
      if (!has) {
        const uint32_t i = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
        if (i < n_items) {
          pix = i / spp;
          smp = i % spp;
          const uint32_t x = pix % fp.width, y = pix / fp.width;
          const size_t idx = ((size_t)x * fp.height + y) * 3;
          d0 = ap.adjoint[idx] * inv;
          d1 = ap.adjoint[idx + 1] * inv;
          d2 = ap.adjoint[idx + 2] * inv;
          ray = camera_ray(fp, x, y, smp, RngCtx{fp.seed_lo, fp.seed_hi, pix, smp, 0, nullptr});
          replay_begin(P);
          depth = 0;
          trav_init<F>(t, sc, ray, 3.402823466e38f);
          has = true;
        }
      }
    }
    const unsigned live = __ballot_sync(0xffffffffu, has);
    if (!live) break;
    const RngCtx ctx{fp.seed_lo, fp.seed_hi, pix, smp, depth, nullptr};
    if (has && !done) done = trav_run<F, false, true>(t, stack, sc, ray, 1e-3f, ctx, cnt, fp.err, budget);
    if (finish_now(done, live, shade_lanes)) {
      HitRec h;
      const bool hit = finish_hit<F, false>(sc, ray, 1e-3f, 3.402823466e38f, t, h, cnt);
      if (replay_segment<F>(sc, fp, ap, P, ray, ctx, depth, hit, h)) {
        ++depth;
        trav_init<F>(t, sc, ray, 3.402823466e38f);
      } else {
        replay_backward<F>(sc, ap, gs, P, d0, d1, d2);
        has = false;
      }
      done = false;
    }
  }
  flush_block_sums(ap, grad_sh);
}

// L2 loss against a target: adjoint = 2 (I - T), loss = sum (I - T)^2.
__global__ void k_l2_adjoint(const float* image, const float* target, float* adjoint, size_t n, double* loss) {
  double acc = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float d = image[i] - target[i];
    adjoint[i] = 2.0f * d;
    acc += (double)d * d;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// RG_ADJ_KIND_VARIANTS=0 at build time replays spheres with media in the
// general kernel variant.
#ifndef RG_ADJ_KIND_VARIANTS
#define RG_ADJ_KIND_VARIANTS 1
#endif

// RG_ADJ_PERSISTENT=0 at build time selects the one-thread-per-sample grid
// form of the replay instead of the persistent one.
#ifndef RG_ADJ_PERSISTENT
#define RG_ADJ_PERSISTENT 1
#endif

// `counter`: a zeroed device word (the persistent form's fetch counter).
template <uint32_t F>
cudaError_t launch_replay(const GpuScene& sc, const FrameParams& fp, const AdjParams& ap, uint32_t* counter,
                          int budget, int shade_lanes, int device, cudaStream_t st) {
  const uint32_t n_pix = fp.width * fp.height;
  const size_t smem = ap.block_sums ? (6 * (size_t)ap.n_mat + ap.n_vol) * sizeof(float) : 0;
  if (RG_ADJ_PERSISTENT) {
    int per_sm = 0, sms = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_replay_persistent<F>, kAdjBlock, smem);
    if (e != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) return e;
    const uint32_t blocks = (uint32_t)std::max(sms, 1) * (uint32_t)std::max(per_sm, 1);
    k_replay_persistent<F><<<blocks, kAdjBlock, smem, st>>>(sc, fp, ap, n_pix * fp.spp, counter, budget, shade_lanes);
  } else {
    const uint32_t ppw = fp.spp <= 32 ? 32 / fp.spp : 1u;
    const uint32_t warps = (n_pix + ppw - 1) / ppw;
    const uint32_t blocks = (warps + kAdjBlock / 32 - 1) / (kAdjBlock / 32);
    k_replay<F><<<blocks, kAdjBlock, smem, st>>>(sc, fp, ap, n_pix);
  }
  return cudaGetLastError();
}

}  // namespace

rg_status backward_device(rg_renderer* h, uint64_t seed, const float* adjoint, const float* target, rg_gradients* out,
                          bool last_frame) {
  const uint32_t w = h->opts.width, hh = h->opts.height;
  const size_t npx3 = (size_t)w * hh * 3;
  const uint32_t n_mat = (uint32_t)h->host.materials.size(), n_vol = h->host.nv;
  if (h->opts.mode != RG_MODE_PBR || h->opts.ray_branching != 1)
    return set_error(h, RG_UNSUPPORTED_VARIANT, "rg_backward differentiates RenderMode::PBR with ray_branching 1");
  if (h->opts.ray_depth + 1 > (uint32_t)kAdjMaxVertices)
    return set_error(h, RG_UNSUPPORTED_VARIANT, "rg_backward supports ray_depth <= 16");
  if (n_vol > (uint32_t)kAdjMaxVolumes) return set_error(h, RG_UNSUPPORTED_VARIANT, "rg_backward supports at most 4 media");
  if (h->host.textured)
    return set_error(h, RG_UNSUPPORTED_VARIANT, "rg_backward differentiates solid albedos: no textures or image sky");
  if (h->host.vol_transformed)
    return set_error(h, RG_UNSUPPORTED_VARIANT, "rg_backward's density scores need untransformed media");
  if (h->range_count)
    return set_error(h, RG_NOT_READY, "rg_backward differentiates whole frames: reset the sample range first");
  cudaStream_t st = h->stream;
  // Device scratch of the adjoint: image, target/adjoint image, gradients, loss.
  size_t need = (2 * npx3 + 2 * (size_t)n_mat * 3 + n_vol + 4) * sizeof(float) + sizeof(double) + 512 + 64;
  if (h->adj_bytes < need) {
    if (h->d_adj) cudaFree(h->d_adj);
    h->d_adj = nullptr;
    h->adj_bytes = 0;
    cudaError_t e = cudaMalloc(&h->d_adj, need);
    if (e != cudaSuccess) { cudaGetLastError(); return set_error(h, RG_OOM, "rg_backward: device scratch"); }
    h->adj_bytes = need;
  }
  char* p = (char*)h->d_adj;
  double* d_loss = (double*)p; p += 256;
  float* d_image = (float*)p; p += npx3 * sizeof(float);
  float* d_adjoint = (float*)p; p += npx3 * sizeof(float);
  float* d_galb = (float*)p; p += (size_t)n_mat * 3 * sizeof(float);
  float* d_gem = (float*)p; p += (size_t)n_mat * 3 * sizeof(float);
  float* d_gden = (float*)p;
  cudaError_t e;
  auto cuda_err = [&](cudaError_t err) { cudaGetLastError(); return set_error(h, RG_CUDA_ERROR, cudaGetErrorString(err)); };
  if ((e = cudaMemsetAsync(h->d_adj, 0, need, st)) != cudaSuccess) return cuda_err(e);
  if ((e = cudaMemsetAsync(h->d_err, 0, sizeof(uint32_t), st)) != cudaSuccess) return cuda_err(e);
  FrameParams fp;
  fill_frame_params(h, seed, fp);
  if (target && last_frame) {
    // I: the frame mean of the handle's last render (same scene and parameters)
    d_image = h->d_fmean;
    if ((e = cudaMemcpyAsync(d_adjoint, target, npx3 * sizeof(float), cudaMemcpyHostToDevice, st)) != cudaSuccess)
      return cuda_err(e);
    k_l2_adjoint<<<1024, 256, 0, st>>>(d_image, d_adjoint, d_adjoint, npx3, d_loss);
  } else if (target) {
    // Forward frame into a scratch image (the accumulation buffer is untouched).
    FrameParams ff = fp;
    ff.accum = d_adjoint;  // used as a zeroed running-sum scratch, overwritten below
    ff.out = nullptr;
    ff.frame_mean = d_image;
    ff.frame_var = nullptr;
    ff.accum_count = 1;
    // the handle's kernel form renders it (both forms give the same image)
    e = h->form == RG_FORM_WAVEFRONT ? launch_wavefront(h, ff) : launch_megakernel(h->gs, ff, false, st, h->mega_block ? h->mega_block : kDefaultMegaBlock);
    if (e != cudaSuccess) return cuda_err(e);
    if ((e = cudaMemcpyAsync(d_adjoint, target, npx3 * sizeof(float), cudaMemcpyHostToDevice, st)) != cudaSuccess)
      return cuda_err(e);
    k_l2_adjoint<<<1024, 256, 0, st>>>(d_image, d_adjoint, d_adjoint, npx3, d_loss);
  } else {
    if ((e = cudaMemcpyAsync(d_adjoint, adjoint, npx3 * sizeof(float), cudaMemcpyHostToDevice, st)) != cudaSuccess)
      return cuda_err(e);
  }
  AdjParams ap{d_adjoint, d_galb, d_gem, d_gden, n_vol, n_mat,
               RG_ADJ_BLOCK_SUMS && 6 * n_mat + n_vol <= kAdjSharedGrads ? 1 : 0};
  uint32_t* d_counter = (uint32_t*)((char*)d_loss + 64);  // zeroed with the scratch above
  const int budget = (int)effective_budget(h);
  const int shade_lanes = (int)(h->shade_lanes ? h->shade_lanes : kShadeLanesDefault);
  // Spheres with media (the differentiable workloads' scenes) have a replay
  // of their own: the general variant's code for every other kind made the
  // persistent kernel stall on instruction fetch.
  if (RG_ADJ_KIND_VARIANTS && h->have == (F_SPHERE | F_VOL) && !(h->gs.features & F_WIDE))
    e = launch_replay<F_SPHERE | F_VOL>(h->gs, fp, ap, d_counter, budget, shade_lanes, h->device, st);
  else
    e = dispatch_features(h->gs.features, [&](auto f) {
      return launch_replay<decltype(f)::value>(h->gs, fp, ap, d_counter, budget, shade_lanes, h->device, st);
    });
  if (e != cudaSuccess) return cuda_err(e);
  double loss = 0.0;
  if (out->albedo && (e = cudaMemcpyAsync(out->albedo, d_galb, (size_t)n_mat * 3 * sizeof(float), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return cuda_err(e);
  if (out->emission && (e = cudaMemcpyAsync(out->emission, d_gem, (size_t)n_mat * 3 * sizeof(float), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return cuda_err(e);
  if (out->density && n_vol && (e = cudaMemcpyAsync(out->density, d_gden, n_vol * sizeof(float), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return cuda_err(e);
  if ((e = cudaMemcpyAsync(&loss, d_loss, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return cuda_err(e);
  uint32_t err = 0;
  if ((e = cudaMemcpyAsync(&err, h->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return cuda_err(e);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_err(e);
  out->loss = loss;
  const rg_status dst = device_status(err);
  if (dst != RG_OK) return set_error(h, dst, "rg_backward: device error bits set (traversal stack, queue or tree index)");
  return RG_OK;
}

}  // namespace rg
