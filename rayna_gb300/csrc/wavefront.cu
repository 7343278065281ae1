// wavefront.cu — the wavefront kernel form.
//
// A frame is split into waves of whole pixels (all samples of a pixel are in
// one wave). For every wave:
//   generate    one camera ray per path slot (slot p = pixel-in-wave * spp + sample)
//   bounce      (default) one kernel per bounce over the compacted queue of
//               live paths: closest hit, emission/sky, scatter, attenuation;
//               survivors are compacted into the next queue with warp ballots
//               (one atomic per warp)
//   extend +    (material-sorted variant) the closest hit of every live path,
//   shade       each path appended to the queue of its hit's material kind,
//               then shading over the kind queues laid end to end, so warps
//               shade one material kind at a time
//   accumulate  per-pixel sums in the megakernel's order, then the
//               accumulation buffer
// Paths run the same per-path functions as the megakernel (trace.cuh) with the
// same counter-based random streams, and per-pixel sums are taken in the same
// order, so every form produces the same image bit for bit.
//
// Path state and the per-path functions are in wavefront.cuh. Counts live in
// device memory, so a wave is a fixed launch sequence with no host round trip.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "kernels.h"
#include "renderer_state.h"
#include "wavefront.cuh"

namespace rg {

namespace {

__global__ void __launch_bounds__(kWfBlock) k_generate(FrameParams fp, PathState s, WaveParams wp) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    s.counts[0] = wp.n_paths;
    s.counts[1] = 0;
  }
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < wp.n_paths; p += gridDim.x * blockDim.x) {
    uint32_t pix = wp.first_pixel + p / fp.spp, smp = fp.sample_base + p % fp.spp;
    uint32_t x = pix % fp.width, y = pix / fp.width;
    RngCtx ctx{fp.seed_lo, fp.seed_hi, pix, smp, 0, nullptr};
    Ray r = camera_ray(fp, x, y, smp, ctx);
    store_path(s, p, r.o, 0, r.d, C3f{1.0f, 1.0f, 1.0f});
    s.active[0][p] = p;
  }
}

// One bounce of every live path: closest hit and shading in one kernel,
// persistent with dynamic ray fetch (Aila & Laine 2009, "replacing terminated
// rays"): a warp keeps 32 paths in flight, traverses for `budget` node visits
// at a time, and lanes whose traversal has finished shade their paths and
// then take the next ones from the queue (one atomic per warp and refill), so
// lanes do not idle while the warp's longest ray finishes. Finished lanes wait
// until `shade_lanes` of them (or every live lane) are ready and then shade
// together: shading is long code, and run for the one or two lanes that finish
// in a given step it cost more than the wait.
// A bounce whose queue holds at most `tail_paths` paths (the long tail of deep
// scenes, where a few paths keep bouncing) runs each of them to its end in
// this launch instead of queueing it for the next: every bounce launch costs
// the latency of a path's whole dependent chain through L2, while within one
// launch the later bounces find the tree in L1. The later launches then find
// their queues empty.
template <uint32_t F, bool COUNT>
__global__ void __launch_bounds__(kWfBlock) k_bounce(GpuScene sc, FrameParams fp, PathState s, WaveParams wp, int cur,
                                                     int budget, int shade_lanes, uint32_t tail_paths) {
  const uint32_t n = clamp_count(s.counts[cur], wp, fp.err);
  if (warp_unneeded(n)) return;
  const bool tail = n <= tail_paths;
  const int nxt = cur ^ 1;
  uint32_t* next = s.counts + kFetchCounter;
  const uint32_t lane = threadIdx.x & 31u;
  Counters cnt;
  uint32_t queries = 0;
  bool has = false, done = false, drained = false;
  uint32_t p = 0, pix = 0, smp = 0, depth = 0;
  Ray r;
  C3f beta;
  Traversal t;
  extern __shared__ uint2 wf_stack_sh[];  // sc.shared_stack entries per thread
  uint2 stack_loc[kTravStack];
  DynStack stack{wf_stack_sh + threadIdx.x, stack_loc, (int)sc.shared_stack, kWfBlock};
  for (;;) {
    const unsigned idle = __ballot_sync(0xffffffffu, !has);
    if (idle && !drained) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(next, (uint32_t)__popc(idle));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + (uint32_t)__popc(idle) >= n) drained = true;
      if (!has) {
        const uint32_t i = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
        if (i < n) {
          p = s.active[cur][i];
          pix = wp.first_pixel + p / fp.spp;
          smp = fp.sample_base + p % fp.spp;
          const float4 r0 = s.rec[3 * (size_t)p], r1 = s.rec[3 * (size_t)p + 1], r2 = s.rec[3 * (size_t)p + 2];
          depth = __float_as_uint(r0.w);
          r.o = v3(r0.x, r0.y, r0.z);
          r.d = v3(r1.x, r1.y, r1.z);
          r.inv = v3(__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z));
          beta = C3f{r2.x, r2.y, r2.z};
          trav_init<F>(t, sc, r, 3.402823466e38f);
          has = true;
          ++queries;
        }
      }
    }
    const unsigned live = __ballot_sync(0xffffffffu, has);
    if (!live) break;
    if (has && !done) {
      const RngCtx ctx{fp.seed_lo, fp.seed_hi, pix, smp, depth, nullptr};
      done = trav_run<F, COUNT, true>(t, stack, sc, r, 1e-3f, ctx, cnt, fp.err, budget);
    }
    if (finish_now(done, live, shade_lanes)) {
      HitRec h;
      const bool hit = finish_hit<F, COUNT>(sc, r, 1e-3f, 3.402823466e38f, t, h, cnt);
      bool go_on = false;
      if (shade_path<F, COUNT>(sc, fp, s, p, pix, smp, depth, r, beta, hit, h)) {
        if (tail) {
          go_on = true;
        } else {
          uint32_t slot = warp_append(s.counts + nxt, true);
          if (slot < wp.n_paths) s.active[nxt][slot] = p;
          else atomicOr(fp.err, ERR_QUEUE_OVERFLOW);
        }
      }
      if (go_on) {  // the path's next segment, from the record shade_path just wrote
        const float4 r0 = s.rec[3 * (size_t)p], r1 = s.rec[3 * (size_t)p + 1], r2 = s.rec[3 * (size_t)p + 2];
        depth = __float_as_uint(r0.w);
        r.o = v3(r0.x, r0.y, r0.z);
        r.d = v3(r1.x, r1.y, r1.z);
        r.inv = v3(__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z));
        beta = C3f{r2.x, r2.y, r2.z};
        trav_init<F>(t, sc, r, 3.402823466e38f);
        ++queries;
      } else {
        has = false;
      }
      done = false;
    }
  }
  flush_wave_counters<COUNT>(fp, cnt, queries);
}

// Material-sorted variant, stage 1: closest hit; each path goes to the queue
// of its hit's material kind. The kernel is persistent with dynamic ray fetch
// (Aila & Laine 2009, "replacing terminated rays"): a warp keeps 32 rays in
// flight, traverses for `budget` node visits at a time, and lanes whose ray
// has finished take the next rays from the queue (one atomic per warp), so
// lanes do not idle while the warp's longest ray finishes. Finished lanes
// record their hits together (finish_now), as the fused kernel shades.

template <uint32_t F, bool COUNT>
__device__ __forceinline__ void record_hit(const GpuScene& sc, const FrameParams& fp, const PathState& s,
                                           const WaveParams& wp, uint32_t p, bool hit, const HitRec& h) {
  uint32_t kind = KQ_MISS;
  if (hit) {
    uint32_t mat;
    int code = h.prim;
    if ((F & (F_SDF | F_PLANE)) && h.sdf >= 0) {
      mat = sc.sdfs[h.sdf].material;
      code = -2 - h.sdf;
      s.aux[p] = make_float4(h.sh.n.x, h.sh.n.y, h.sh.n.z,
                             __uint_as_float((h.sh.front ? 0x80000000u : 0u) | (h.sh.flip ? 0x40000000u : 0u) |
                                             (h.sh.side & 0x3FFFFFFFu)));
    } else {
      mat = prim_material(sc.prims[h.prim]);
      if ((F & F_EXT) && sc.prim_xform) s.aux[p].x = h.tl;  // mesh-space distance of a transformed hit
    }
    kind = 1u + sc.materials[mat].kind;
    s.rec[3 * (size_t)p + 1].w = h.t;
    s.rec[3 * (size_t)p + 2].w = __int_as_float(code);
  }
#pragma unroll
  for (uint32_t k = 0; k < kKinds; ++k) {
    bool mine = kind == k;
    if (__any_sync(__activemask(), mine)) {
      uint32_t slot = warp_append(s.counts + 2 + k, mine);
      if (mine) {
        if (slot < wp.capacity) s.kindq[(size_t)k * wp.capacity + slot] = p;
        else atomicOr(fp.err, ERR_QUEUE_OVERFLOW);
      }
    }
  }
}

// After the last SDF's march: the infinite planes (tested after the SDFs, in
// list order, replacing the hit only when strictly closer) and the path's
// material-kind queue.
template <uint32_t F, bool COUNT>
__device__ __forceinline__ void finish_march(const GpuScene& sc, const FrameParams& fp, const PathState& s,
                                             const WaveParams& wp, uint32_t p, const Ray& r, Counters& cnt) {
  HitRec h;
  const float4 r1 = s.rec[3 * (size_t)p + 1];
  const int code = __float_as_int(s.rec[3 * (size_t)p + 2].w);
  bool any = code != kPrimMiss;
  h.t = r1.w;
  h.prim = code >= 0 ? code : -1;
  h.sdf = code <= -2 ? -2 - code : -1;
  h.tl = 0.0f;
  if (h.sdf >= 0) {
    const float4 a = s.aux[p];
    const uint32_t fl = __float_as_uint(a.w);
    h.sh = SdfHit{h.t, v3(a.x, a.y, a.z), (fl >> 31) != 0, fl & 0x3FFFFFFFu, false};
  } else if ((F & F_EXT) && sc.prim_xform && h.prim >= 0) {
    h.tl = s.aux[p].x;
  }
  if (F & F_PLANE) {
    for (uint32_t k = 0; k < sc.n_sdfs; ++k) {
      const GpuSdf& f = sc.sdfs[k];
      if (f.kind != kUnboundedPlane) continue;
      // InfinitePlaneMesh::intersect (mesh/planar/infinite_plane.rs:87-92)
      float pt, denom;
      if (!plane_t(v3(f.cx, f.cy, f.cz), f.p0, r, 1e-3f, 3.402823466e38f, pt, denom) || (any && !(pt < h.t))) continue;
      h.t = pt;
      h.sdf = (int)k;
      h.prim = -1;
      h.sh = SdfHit{pt, v3(f.cx, f.cy, f.cz), (bool)signbit(denom), 0u, !signbit(denom)};
      any = true;
    }
  }
  if (COUNT && any) ++cnt.hits;
  record_hit<F, COUNT>(sc, fp, s, wp, p, any, h);
}

// Appends path p to the march queue of SDF `k` (per-SDF queues) or to the
// one march queue (k >= 0 then only says "some SDF"); k < 0 appends nothing.
// Called by the lanes that are finishing together; every lane passes its k.
__device__ __forceinline__ void march_append(const FrameParams& fp, const PathState& s, const WaveParams& wp, int cur,
                                             int n_march, uint32_t p, int k) {
  if (!s.marchq) {
    const bool mine = k >= 0;
    if (__any_sync(__activemask(), mine)) {
      const uint32_t slot = warp_append(s.counts + kMarchCounter, mine);
      if (mine) {
        if (slot < wp.n_paths) s.active[cur ^ 1][slot] = p;
        else atomicOr(fp.err, ERR_QUEUE_OVERFLOW);
      }
    }
    return;
  }
  for (int j = 0; j < n_march; ++j) {
    const bool mine = k == j;
    if (__any_sync(__activemask(), mine)) {
      const uint32_t slot = warp_append(s.counts + kMarchQueueCount0 + j, mine);
      if (mine) {
        if (slot < wp.n_paths) s.marchq[(size_t)j * wp.capacity + slot] = p;
        else atomicOr(fp.err, ERR_QUEUE_OVERFLOW);
      }
    }
  }
}

// The first SDF from `k0` on whose bound sphere the segment [start, lim] can
// reach, or -1.
__device__ __forceinline__ int next_reachable(const GpuScene& sc, int k0, int n_march, const Ray& r, float start,
                                              float lim) {
  for (int k = k0; k < n_march; ++k)
    if (sdf_bound_reachable(sc.sdfs[k], r, start, lim)) return k;
  return -1;
}

// With `n_march` > 0 the scene's first n_march unbounded objects are
// raymarched SDFs, left to the k_march stages: this kernel stores the tree's
// closest hit in the path record (distance, primitive, mesh-space distance of
// a transformed hit); a path whose segment up to that hit can reach one of
// the SDFs' bound spheres goes to the march queue of the first such SDF (or
// to the one march queue), and any other path is finished here as the last
// march stage would finish it (finish_march): no SDF can replace its hit.
template <uint32_t F, bool COUNT>
__global__ void __launch_bounds__(kWfBlock) k_extend(GpuScene sc, FrameParams fp, PathState s, WaveParams wp, int cur,
                                                     int budget, int n_march, int shade_lanes) {
  const uint32_t n = clamp_count(s.counts[cur], wp, fp.err);
  if (warp_unneeded(n)) return;
  uint32_t* next = s.counts + kFetchCounter;
  const uint32_t lane = threadIdx.x & 31u;
  Counters cnt;
  uint32_t queries = 0;
  bool has = false, done = false, drained = false;
  uint32_t p = 0, pix = 0, smp = 0, depth = 0;
  Ray r;
  Traversal t;
  extern __shared__ uint2 wf_stack_sh[];  // sc.shared_stack entries per thread
  uint2 stack_loc[kTravStack];
  DynStack stack{wf_stack_sh + threadIdx.x, stack_loc, (int)sc.shared_stack, kWfBlock};
  for (;;) {
    const unsigned idle = __ballot_sync(0xffffffffu, !has);
    if (idle && !drained) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(next, (uint32_t)__popc(idle));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + (uint32_t)__popc(idle) >= n) drained = true;
      if (!has) {
        const uint32_t i = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
        if (i < n) {
          p = s.active[cur][i];
          pix = wp.first_pixel + p / fp.spp;
          smp = fp.sample_base + p % fp.spp;
          const float4 r0 = s.rec[3 * (size_t)p], r1 = s.rec[3 * (size_t)p + 1];
          depth = __float_as_uint(r0.w);
          r.o = v3(r0.x, r0.y, r0.z);
          r.d = v3(r1.x, r1.y, r1.z);
          r.inv = v3(__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z));
          trav_init<F>(t, sc, r, 3.402823466e38f);
          has = true;
          ++queries;
        }
      }
    }
    const unsigned live = __ballot_sync(0xffffffffu, has);
    if (!live) break;
    if (has && !done) {
      const RngCtx ctx{fp.seed_lo, fp.seed_hi, pix, smp, depth, nullptr};
      done = trav_run<F, COUNT, true>(t, stack, sc, r, 1e-3f, ctx, cnt, fp.err, budget);
    }
    if (finish_now(done, live, shade_lanes)) {
      HitRec h;
      if ((F & F_SDF) && n_march > 0) {
        const bool tree_hit = finish_hit<F & ~(F_SDF | F_PLANE), false>(sc, r, 1e-3f, 3.402823466e38f, t, h, cnt);
        if (tree_hit) {
          s.rec[3 * (size_t)p + 1].w = h.t;
          s.rec[3 * (size_t)p + 2].w = __int_as_float(h.prim);
          if ((F & F_EXT) && sc.prim_xform) s.aux[p].x = h.tl;
        }
        // The march stages only shorten the segment, so one that cannot reach
        // an SDF's bound sphere now never can.
        const int first = next_reachable(sc, 0, n_march, r, 1e-3f, tree_hit ? h.t : 3.402823466e38f);
        march_append(fp, s, wp, cur, n_march, p, first);
        if (first < 0) finish_march<F, COUNT>(sc, fp, s, wp, p, r, cnt);
      } else {
        const bool hit = finish_hit<F, COUNT>(sc, r, 1e-3f, 3.402823466e38f, t, h, cnt);
        record_hit<F, COUNT>(sc, fp, s, wp, p, hit, h);
      }
      has = false;
      done = false;
    }
  }
  flush_wave_counters<COUNT>(fp, cnt, queries);
}

// After path p's march of SDF k (or its rejection at fetch): with per-SDF
// queues, on to the queue of the next SDF its segment [start, lim] can reach,
// or finished when there is none; with one march queue, finished by the last
// stage. `lim`: the distance the remaining SDFs must beat.
template <uint32_t F, bool COUNT>
__device__ __forceinline__ void pass_on(const GpuScene& sc, const FrameParams& fp, const PathState& s,
                                        const WaveParams& wp, int cur, int k, int n_march, uint32_t p, const Ray& r,
                                        float lim, Counters& cnt) {
  if (!s.marchq) {
    if (k + 1 == n_march) finish_march<F, COUNT>(sc, fp, s, wp, p, r, cnt);
    return;
  }
  const int nk = next_reachable(sc, k + 1, n_march, r, 1e-3f, lim);
  march_append(fp, s, wp, cur, n_march, p, nk);
  if (nk < 0) finish_march<F, COUNT>(sc, fp, s, wp, p, r, cnt);
}

// Material-sorted variant with raymarched SDFs, stage 1b: the march of SDF k
// (the unbounded list's k-th object) for every path of its march queue: the
// paths whose segment, after the tree and the SDFs before k, can reach its
// bound sphere (with one march queue for every stage: all paths that can
// reach some SDF). A hit replaces the path's hit when strictly closer (or
// when nothing was hit), as ObjectList's loop over unbounded objects does
// (object/list.rs:112-129); then the path goes on to the queue of the next SDF
// it can reach, or is finished (infinite planes, material-kind queue).
// Persistent with dynamic fetch: every lane marches the same function,
// `budget` evaluations at a time, and lanes whose march has ended take the
// next path (one atomic per warp), so a long march does not hold idle lanes.
// A warp finishes its ended marches together (the hit normal, six distance
// evaluations; passing the path on) once `shade_lanes` of them, or all of its
// live lanes, have ended.
template <uint32_t F, bool COUNT>
__global__ void __launch_bounds__(kWfBlock) k_march(GpuScene sc, FrameParams fp, PathState s, WaveParams wp, int cur,
                                                    uint32_t k, int n_march, int budget, int shade_lanes) {
  const uint32_t n = clamp_count(s.counts[s.marchq ? kMarchQueueCount0 + k : kMarchCounter], wp, fp.err);
  if (warp_unneeded(n)) return;
  const uint32_t* queue = s.marchq ? s.marchq + (size_t)k * wp.capacity : s.active[cur ^ 1];
  uint32_t* next = s.counts + kFetchCounter;
  const uint32_t lane = threadIdx.x & 31u;
  const GpuSdf f = sc.sdfs[k];
  const float start = 1e-3f, end = 3.402823466e38f;
  Counters cnt;
  bool has = false, done = false, drained = false;
  uint32_t p = 0;
  Ray r;
  float best = 0.0f;
  bool any = false;
  int st = kMarchOn;  // a finished march's outcome, kept until the warp finishes it
  SdfMarch m;
  for (;;) {
    // Refill idle lanes until every lane has a march or the queue is drained:
    // a path whose segment no longer reaches the bound sphere (an earlier
    // SDF's hit shortened it) ends at fetch, and its lane must not wait out
    // the marching lanes' budget before its next fetch.
    while (!drained) {
      const unsigned idle = __ballot_sync(0xffffffffu, !has);
      if (!idle) break;
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(next, (uint32_t)__popc(idle));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + (uint32_t)__popc(idle) >= n) drained = true;
      if (!has) {
        const uint32_t i = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
        if (i < n) {
          p = queue[i];
          const float4 r0 = s.rec[3 * (size_t)p], r1 = s.rec[3 * (size_t)p + 1];
          r.o = v3(r0.x, r0.y, r0.z);
          r.d = v3(r1.x, r1.y, r1.z);
          any = __float_as_int(s.rec[3 * (size_t)p + 2].w) != kPrimMiss;
          best = r1.w;
          has = true;
          sdf_march_begin(r, start, m);
          if (!sdf_bound_reachable(f, r, start, any ? best : end)) {
            has = false;
            pass_on<F, COUNT>(sc, fp, s, wp, cur, (int)k, n_march, p, r, any ? best : end, cnt);
          }
        }
      }
    }
    const unsigned live = __ballot_sync(0xffffffffu, has);
    if (!live) break;  // drained, and nothing left to march
    if (has && !done) {
      st = kMarchOn;
      for (int e = 0; e < budget && st == kMarchOn; ++e)
        st = sdf_march_step<COUNT>(f, r, start, end, any ? best : end, !any, m, cnt.sdf_steps, cnt.sdf_iters);
      done = st != kMarchOn;
    }
    if (finish_now(done, live, shade_lanes)) {
      if (st == kMarchHit) {
        SdfHit sh;
        sdf_march_hit<COUNT>(f, m, sh, cnt.sdf_steps);
        s.rec[3 * (size_t)p + 1].w = sh.t;
        s.rec[3 * (size_t)p + 2].w = __int_as_float(-2 - (int)k);
        s.aux[p] = make_float4(sh.n.x, sh.n.y, sh.n.z,
                               __uint_as_float((sh.front ? 0x80000000u : 0u) | (sh.side & 0x3FFFFFFFu)));
      }
      pass_on<F, COUNT>(sc, fp, s, wp, cur, (int)k, n_march, p, r, st == kMarchHit ? m.total : (any ? best : end), cnt);
      has = false;
      done = false;
    }
  }
  flush_wave_counters<COUNT>(fp, cnt, 0);
}

// Material-sorted variant, stage 2: shading over the kind queues end to end.
template <uint32_t F>
__global__ void __launch_bounds__(kWfBlock) k_shade(GpuScene sc, FrameParams fp, PathState s, WaveParams wp, int cur) {
  __shared__ uint32_t off[kKinds + 1];
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (int k = 0; k < kKinds; ++k) {
      uint32_t c = s.counts[2 + k];
      if (c > wp.n_paths) { atomicOr(fp.err, ERR_QUEUE_OVERFLOW); c = 0; }
      off[k] = acc;
      acc += c;
    }
    off[kKinds] = acc;
  }
  __syncthreads();
  const uint32_t total = off[kKinds];
  const int nxt = cur ^ 1;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    uint32_t k = 0;
#pragma unroll
    for (int j = 1; j < kKinds; ++j) k += i >= off[j] ? 1u : 0u;
    const uint32_t p = s.kindq[(size_t)k * wp.capacity + (i - off[k])];
    const uint32_t pix = wp.first_pixel + p / fp.spp, smp = fp.sample_base + p % fp.spp;
    const float4 r0 = s.rec[3 * (size_t)p], r1 = s.rec[3 * (size_t)p + 1], r2 = s.rec[3 * (size_t)p + 2];
    Ray r;
    r.o = v3(r0.x, r0.y, r0.z);
    r.d = v3(r1.x, r1.y, r1.z);
    r.inv = v3(__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z));
    HitRec h;
    h.t = r1.w;
    const int code = __float_as_int(r2.w);
    h.prim = code >= 0 ? code : -1;
    h.sdf = code <= -2 ? -2 - code : -1;
    if (h.sdf >= 0) {
      float4 a = s.aux[p];
      uint32_t f = __float_as_uint(a.w);
      h.sh.n = v3(a.x, a.y, a.z);
      h.sh.front = (f >> 31) != 0;
      h.sh.flip = ((f >> 30) & 1u) != 0;
      h.sh.side = f & 0x3FFFFFFFu;
      h.sh.t = h.t;
    } else if ((F & F_EXT) && sc.prim_xform && h.prim >= 0) {
      h.tl = s.aux[p].x;
    }
    const bool alive = shade_path<F>(sc, fp, s, p, pix, smp, __float_as_uint(r0.w), r, C3f{r2.x, r2.y, r2.z},
                                     k != KQ_MISS, h);
    if (alive) {
      uint32_t slot = warp_append(s.counts + nxt, true);
      if (slot < wp.n_paths) s.active[nxt][slot] = p;
      else atomicOr(fp.err, ERR_QUEUE_OVERFLOW);
    }
  }
}

__global__ void __launch_bounds__(kWfBlock) k_accumulate(FrameParams fp, PathState s, WaveParams wp) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < wp.n_pixels * 3; q += gridDim.x * blockDim.x) {
    const uint32_t lp = q / 3, c = q % 3;
    accumulate_pixel(fp, s, (size_t)lp * fp.spp, wp.first_pixel + lp, c);
  }
}

// Runs every wave of one frame on the path arrays `s` (capacity `cap` slots).
// `timed`: bracket the traversal launches with the handle's stage events.
template <uint32_t F>
cudaError_t run_waves(rg_renderer* h, const FrameParams& fp, const PathState& s, size_t cap, size_t pix_per_wave,
                      bool timed) {
  const size_t spp = fp.spp;
  const size_t n_pix = (size_t)fp.width * fp.height;
  const bool counters = (h->flags & RG_FLAG_COUNTERS) != 0;
  const bool sorted = effective_sort(h);
  const int budget = (int)effective_budget(h);
  const int shade_lanes = (int)(h->shade_lanes ? h->shade_lanes : kShadeLanesDefault);
  const uint32_t tail_paths = h->tail_paths ? h->tail_paths : kTailPathsDefault;
  const int grid = sm_count(h->device) * 8;
  // The persistent traversal kernels run as many blocks as are resident at
  // once, each with its threads' shared stack entries.
  const size_t smem = (size_t)h->gs.shared_stack * kWfBlock * sizeof(uint2);
  int ext_per_sm = 0;
  if (counters) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ext_per_sm, k_extend<F, true>, kWfBlock, smem);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ext_per_sm, k_extend<F, false>, kWfBlock, smem);
  const int ext_grid = sm_count(h->device) * std::max(ext_per_sm, 1);
  int bounce_per_sm = 0;
  if (counters) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bounce_per_sm, k_bounce<F, true>, kWfBlock, smem);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bounce_per_sm, k_bounce<F, false>, kWfBlock, smem);
  const int bounce_grid = sm_count(h->device) * std::max(bounce_per_sm, 1);
  // Raymarched SDFs in the material-sorted form: one k_march stage per SDF
  // after the tree (h->host.nsdf SDFs lead the unbounded list).
  const uint32_t n_march = (F & F_SDF) && sorted ? h->host.nsdf : 0u;
  const int march_budget = (int)(h->march_budget ? h->march_budget : kMarchBudgetDefault);
  int march_per_sm = 0;
  if (n_march) {
    if (counters) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&march_per_sm, k_march<F, true>, kWfBlock, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&march_per_sm, k_march<F, false>, kWfBlock, 0);
  }
  const int march_grid = sm_count(h->device) * std::max(march_per_sm, 1);
  cudaStream_t st = h->stream;
  cudaError_t e;
  uint32_t launches = 0;
  for (size_t first = 0; first < n_pix; first += pix_per_wave) {
    WaveParams wp;
    wp.first_pixel = (uint32_t)first;
    wp.n_pixels = (uint32_t)std::min(pix_per_wave, n_pix - first);
    wp.n_paths = (uint32_t)(wp.n_pixels * spp);
    wp.capacity = (uint32_t)cap;
    uint32_t gen_blocks = (uint32_t)std::min<size_t>((wp.n_paths + kWfBlock - 1) / kWfBlock, (size_t)grid * 4);
    k_generate<<<gen_blocks, kWfBlock, 0, st>>>(fp, s, wp);
    // A fused wave whose first queue is within the tail threshold runs every
    // path to its end in the first bounce launch: the later ones would find
    // empty queues, so they are not launched.
    const uint32_t last_bounce = !sorted && wp.n_paths <= tail_paths ? 0u : fp.ray_depth;
    // generate, accumulate, and per bounce the bounce kernel or extend + march stages + shade
    launches += 2 + (last_bounce + 1) * (sorted ? 2 + n_march : 1);
    int cur = 0;
    for (uint32_t d = 0; d <= last_bounce; ++d) {
      if ((e = cudaMemsetAsync(s.counts + (cur ^ 1), 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
      if ((e = cudaMemsetAsync(s.counts + kFetchCounter, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
      if (sorted) {
        // the kind counts, the fetch counter and the march queue's count
        if ((e = cudaMemsetAsync(s.counts + 2, 0, (kKinds + 2) * sizeof(uint32_t), st)) != cudaSuccess) return e;
        if (s.marchq && (e = cudaMemsetAsync(s.counts + kMarchQueueCount0, 0, n_march * sizeof(uint32_t), st)) != cudaSuccess)
          return e;
        if (timed && (e = stage_mark(h)) != cudaSuccess) return e;
        if (counters) k_extend<F, true><<<ext_grid, kWfBlock, smem, st>>>(h->gs, fp, s, wp, cur, budget, (int)n_march,
                                                               shade_lanes);
        else k_extend<F, false><<<ext_grid, kWfBlock, smem, st>>>(h->gs, fp, s, wp, cur, budget, (int)n_march,
                                                                shade_lanes);
        // the SDFs in list order, each over its march queue
        for (uint32_t k = 0; k < n_march; ++k) {
          if ((e = cudaMemsetAsync(s.counts + kFetchCounter, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
          if (counters) k_march<F, true><<<march_grid, kWfBlock, 0, st>>>(h->gs, fp, s, wp, cur, k, (int)n_march,
                                                                        march_budget, shade_lanes);
          else k_march<F, false><<<march_grid, kWfBlock, 0, st>>>(h->gs, fp, s, wp, cur, k, (int)n_march,
                                                                 march_budget, shade_lanes);
        }
        if (timed && (e = stage_mark(h)) != cudaSuccess) return e;
        k_shade<F><<<grid, kWfBlock, 0, st>>>(h->gs, fp, s, wp, cur);
      } else {
        if (timed && (e = stage_mark(h)) != cudaSuccess) return e;
        if (counters) k_bounce<F, true><<<bounce_grid, kWfBlock, smem, st>>>(h->gs, fp, s, wp, cur, budget, shade_lanes,
                                                                         tail_paths);
        else k_bounce<F, false><<<bounce_grid, kWfBlock, smem, st>>>(h->gs, fp, s, wp, cur, budget, shade_lanes,
                                                                     tail_paths);
        if (timed && (e = stage_mark(h)) != cudaSuccess) return e;
      }
      cur ^= 1;
    }
    uint32_t acc_blocks = (uint32_t)std::min<size_t>((wp.n_pixels * 3 + kWfBlock - 1) / kWfBlock, (size_t)grid * 4);
    k_accumulate<<<acc_blocks, kWfBlock, 0, st>>>(fp, s, wp);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  h->last_launches = launches;
  return cudaSuccess;
}

cudaError_t run_frame(rg_renderer* h, const FrameParams& fp, const PathState& s, size_t cap, size_t pix_per_wave,
                      bool timed) {
  return dispatch_features(h->gs.features,
                           [&](auto f) { return run_waves<decltype(f)::value>(h, fp, s, cap, pix_per_wave, timed); });
}

}  // namespace


cudaError_t launch_wavefront(rg_renderer* h, const FrameParams& fp) {
  const size_t spp = fp.spp;
  const size_t n_pix = (size_t)fp.width * fp.height;
  size_t budget = h->wf_paths ? h->wf_paths : kDefaultWavePaths;
  size_t pix_per_wave = std::max<size_t>(1, budget / spp);
  pix_per_wave = std::min(pix_per_wave, n_pix);
  size_t cap = pix_per_wave * spp;
  if (cap > 0xFFFFFFFFull) return cudaErrorInvalidValue;
  if (h->wf.capacity < cap) {
    free_extra(h);
    cudaError_t e = cudaMalloc(&h->wf.arena, arena_bytes(cap));
    if (e != cudaSuccess) return e;
    h->wf.capacity = cap;
    h->wf.arena_bytes = arena_bytes(cap);
  }
  PathState s;
  carve((char*)h->wf.arena, h->wf.capacity, s);
  // Per-SDF march queues for the material-sorted form of scenes with
  // raymarched SDFs (without them every stage reads one march queue).
  const uint32_t n_march = effective_sort(h) ? h->host.nsdf : 0u;
  if (n_march > 0 && n_march <= (uint32_t)kMaxRoutedSdfs) {
    const size_t need = (size_t)n_march * h->wf.capacity * sizeof(uint32_t);
    if (h->wf.marchq_bytes < need) {
      if (h->wf.marchq) cudaFree(h->wf.marchq);
      h->wf.marchq = nullptr;
      h->wf.marchq_bytes = 0;
      cudaError_t e = cudaMalloc(&h->wf.marchq, need);
      if (e != cudaSuccess) return e;
      h->wf.marchq_bytes = need;
    }
    s.marchq = (uint32_t*)h->wf.marchq;
  }
  return run_frame(h, fp, s, h->wf.capacity, pix_per_wave, (h->flags & RG_FLAG_STAGE_TIMES) != 0);
}

// ---------------------------------------------------------------------------
// Allocation-free variant: the path state of one wave lives in a fixed
// file-scope device array instead of a cudaMalloc'ed arena.
// ---------------------------------------------------------------------------
constexpr size_t kStaticArenaBytes = arena_bytes(RG_STATIC_WAVE_PATHS);
static_assert(kStaticArenaBytes <= 108ull * RG_STATIC_WAVE_PATHS + 256ull, "static scratch larger than documented");
static __device__ __align__(256) unsigned char g_wave_scratch[kStaticArenaBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};
}  // namespace

// Device address of g_wave_scratch on `device` (which must be current),
// looked up once per device. In host code the array's name is only a
// host-side stand-in, so kernels get this address instead.
static cudaError_t static_scratch(int device, void** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_wave_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = p;
  }
  *out = g_scratch_ptr[device];
  return cudaSuccess;
}

cudaError_t launch_wavefront_static(rg_renderer* h, const FrameParams& fp) {
  const size_t spp = fp.spp;
  const size_t n_pix = (size_t)fp.width * fp.height;
  const size_t cap = RG_STATIC_WAVE_PATHS;
  if (arena_bytes(cap) > kStaticArenaBytes || spp > cap) return cudaErrorInvalidValue;
  void* arena = nullptr;
  cudaError_t e = static_scratch(h->device, &arena);
  if (e != cudaSuccess) return e;
  PathState s;
  carve((char*)arena, cap, s);
  // No stage timing here: its events are created on demand, and this entry allocates nothing.
  return run_frame(h, fp, s, cap, std::min(cap / spp, n_pix), false);
}

}  // namespace rg

// The allocation-free entry point (see rayna_gpu.h).
extern "C" rg_status rg_render_static_scratch(rg_handle h, uint64_t seed, float* d_accum, uint32_t accum_count,
                                              float* d_out) {
  using namespace rg;
  if (!h) return RG_INVALID_ARG;
  h->frame_current = false;  // this entry does not write the handle's frame mean
  if (!d_accum || accum_count == 0)
    return set_error(h, RG_INVALID_ARG, "rg_render_static_scratch: d_accum must be a device buffer and accum_count >= 1");
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return set_error(h, RG_CUDA_ERROR, cudaGetErrorString(e));
  if (!h->cam_ok) return set_error(h, RG_INVALID_CAMERA, "camera viewport could not be calculated");
  if (h->opts.mode != RG_MODE_PBR || h->opts.ray_branching != 1)
    return set_error(h, RG_UNSUPPORTED_VARIANT,
                     "rg_render_static_scratch renders RenderMode::PBR with ray_branching 1 only");
  if (h->opts.samples > RG_STATIC_WAVE_PATHS)
    return set_error(h, RG_INVALID_ARG,
                     "rg_render_static_scratch: samples per pixel exceed the 65536 path slots of the static scratch");
  FrameParams fp;
  fill_frame_params(h, seed, fp);
  fp.accum = d_accum;
  fp.out = d_out;
  fp.frame_mean = nullptr;
  fp.frame_var = nullptr;
  fp.accum_count = accum_count;
  // The frame's bookkeeping, as rg_render keeps it, so rg_sync_stats reports
  // this frame: counters and error bits cleared, events around the launches.
  h->stage_used = 0;
  h->last_launches = 0;
  h->last_samples = (uint64_t)fp.width * fp.height * fp.spp;
  if ((e = cudaMemsetAsync(h->d_counters, 0, CNT_N * sizeof(unsigned long long), h->stream)) != cudaSuccess ||
      (e = cudaMemsetAsync(h->d_err, 0, sizeof(uint32_t), h->stream)) != cudaSuccess ||
      (e = cudaEventRecord(h->ev0, h->stream)) != cudaSuccess)
    return set_error(h, RG_CUDA_ERROR, cudaGetErrorString(e));
  if ((e = launch_wavefront_static(h, fp)) != cudaSuccess || (e = cudaEventRecord(h->ev1, h->stream)) != cudaSuccess) {
    cudaGetLastError();
    return set_error(h, RG_CUDA_ERROR, cudaGetErrorString(e));
  }
  return RG_OK;
}

namespace rg {

void free_extra(rg_renderer* h) {
  if (h->wf.arena) cudaFree(h->wf.arena);
  if (h->wf.marchq) cudaFree(h->wf.marchq);
  h->wf = WavefrontState{};
}

void on_scene_changed(rg_renderer* h) { (void)h; }

}  // namespace rg
