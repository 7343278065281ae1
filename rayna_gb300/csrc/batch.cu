// batch.cu — many renders in one graph-replayed frame.
//
// Every render of a batch is an ordinary handle (its own scene buffers,
// camera, options and accumulation). Two batched forms:
//
// RG_BATCH_WAVEFRONT (default). The paths of all renders fill shared waves of
// path slots: a wave is a list of chunks (render, run of whole pixels), laid
// out one after another, and each slot remembers its chunk. Per wave:
// k_bgenerate (camera rays of every chunk), one persistent dynamic-fetch
// k_bbounce per bounce over the live paths of all renders (each lane reads
// its render's scene and frame parameters through its chunk), and
// k_baccumulate (per-pixel sums in the canonical order into each render's
// accumulation buffer). Renders of uneven size share every launch, so no
// render's tail leaves SMs idle and small renders cost no launch of their own.
//
// RG_BATCH_TILES. One launch of k_batch: as many blocks as fit on the SMs,
// whose warps take work items from one global queue (an atomic counter) until
// it is empty. A work item is `rounds_per_item` consecutive warp rounds
// (mega.cuh) of one render; items of all renders are numbered one after
// another, so a warp finds its render by a binary search over the prefix sums
// of item counts.
//
// The frame's launch sequence (parameter table upload, counter resets,
// kernels) is captured once as a CUDA graph and replayed; the host only
// rewrites the pinned parameter table (frame keys, accumulation counts)
// before each replay.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "kernels.h"
#include "mega.cuh"
#include "renderer_state.h"
#include "wavefront.cuh"

namespace rg {

struct BatchItemDev {
  GpuScene sc;
  FrameParams fp;
};

// A run of whole pixels of one render inside a wave.
struct BatchChunk {
  uint32_t item;         // render index
  uint32_t first_pixel;  // first pixel (row-major index) of the run in its render
  uint32_t n_pixels;
  uint32_t spp;
  uint32_t slot0;        // first path slot of the run in the wave
  uint32_t pix0;         // position of the run's first pixel among the wave's pixels
  uint32_t pad[2];
};

namespace {

template <uint32_t F>
__global__ void k_batch(const BatchItemDev* __restrict__ items, const uint32_t* __restrict__ prefix, uint32_t n_items,
                        uint32_t total, uint32_t rounds_per_item, uint32_t* counter, unsigned long long* counters) {
  const uint32_t lane = threadIdx.x & 31;
  Counters cnt;
  uint32_t segments = 0;
  uint2 stack_entries[kTravStack];
  LocalStack stack{stack_entries};
  for (;;) {
    uint32_t w = 0;
    if (lane == 0) w = atomicAdd(counter, 1u);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= total) break;
    uint32_t lo = 0, hi = n_items;  // largest lo with prefix[lo] <= w
    while (hi - lo > 1) {
      uint32_t mid = (lo + hi) >> 1;
      if (prefix[mid] <= w) lo = mid;
      else hi = mid;
    }
    const GpuScene sc = items[lo].sc;
    const FrameParams fp = items[lo].fp;
    const uint32_t n_pix = fp.width * fp.height;
    const uint32_t ppr = pixels_per_round(fp.spp);
    const uint32_t round0 = (w - prefix[lo]) * rounds_per_item;
    for (uint32_t r = 0; r < rounds_per_item; ++r) {
      uint32_t first = (round0 + r) * ppr;
      if (first >= n_pix) break;
      mega_round<F, false, kSamplePbr>(sc, fp, first, n_pix, cnt, segments, stack);
    }
  }
  FrameParams f0;
  f0.counters = counters;
  flush_counters<false>(f0, cnt, segments);
}

// ---------------------------------------------------------------------------
// Batched wavefront
// ---------------------------------------------------------------------------
// Largest c in [first, first + n) with key(c) <= v (chunks are in ascending key order).
template <class Key>
__device__ __forceinline__ uint32_t find_chunk(uint32_t first, uint32_t n, uint32_t v, Key key) {
  uint32_t lo = first, hi = first + n;
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (key(mid) <= v) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(kWfBlock) k_bgenerate(const BatchItemDev* __restrict__ items,
                                                        const BatchChunk* __restrict__ chunks, uint32_t first_chunk,
                                                        uint32_t n_chunks, uint32_t n_paths, PathState s,
                                                        uint32_t* __restrict__ chunk_of) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    s.counts[0] = n_paths;
    s.counts[1] = 0;
  }
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n_paths; p += gridDim.x * blockDim.x) {
    const uint32_t c = find_chunk(first_chunk, n_chunks, p, [&](uint32_t i) { return chunks[i].slot0; });
    const BatchChunk ch = chunks[c];
    const FrameParams& fp = items[ch.item].fp;
    const uint32_t rel = p - ch.slot0;
    const uint32_t pix = ch.first_pixel + rel / ch.spp, smp = rel % ch.spp;
    const uint32_t x = pix % fp.width, y = pix / fp.width;
    RngCtx ctx{fp.seed_lo, fp.seed_hi, pix, smp, 0, nullptr};
    Ray r = camera_ray(fp, x, y, smp, ctx);
    store_path(s, p, r.o, 0, r.d, C3f{1.0f, 1.0f, 1.0f});
    s.active[0][p] = p;
    chunk_of[p] = c;
  }
}

// One bounce of the live paths of every render of the wave: closest hit and
// shading, persistent with dynamic ray fetch as in the single-render form
// (finished lanes shade together, finish_now); a lane reads its render's
// scene and frame parameters through its chunk.
template <uint32_t F>
__global__ void __launch_bounds__(kWfBlock) k_bbounce(const BatchItemDev* __restrict__ items,
                                                      const BatchChunk* __restrict__ chunks, WaveParams wp, PathState s,
                                                      const uint32_t* __restrict__ chunk_of, int cur, int budget,
                                                      int shade_lanes, uint32_t* err, unsigned long long* counters) {
  const uint32_t n = clamp_count(s.counts[cur], wp, err);
  if (warp_unneeded(n)) return;
  const int nxt = cur ^ 1;
  uint32_t* next = s.counts + kFetchCounter;
  const uint32_t lane = threadIdx.x & 31u;
  Counters cnt;
  uint32_t queries = 0;
  bool has = false, done = false, drained = false;
  uint32_t p = 0, pix = 0, smp = 0, depth = 0, item = 0;
  Ray r;
  C3f beta;
  Traversal t;
  __shared__ uint2 stack_sh[kSharedStackOf<F> > 0 ? kSharedStackOf<F> * kWfBlock : 1];
  uint2 stack_loc[kTravStack - kSharedStackOf<F>];
  SplitStack<kSharedStackOf<F>, kWfBlock> stack{stack_sh + threadIdx.x, stack_loc};
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
          const BatchChunk ch = chunks[chunk_of[p]];
          item = ch.item;
          const uint32_t rel = p - ch.slot0;
          pix = ch.first_pixel + rel / ch.spp;
          smp = rel % ch.spp;
          const float4 r0 = s.rec[3 * (size_t)p], r1 = s.rec[3 * (size_t)p + 1], r2 = s.rec[3 * (size_t)p + 2];
          depth = __float_as_uint(r0.w);
          r.o = v3(r0.x, r0.y, r0.z);
          r.d = v3(r1.x, r1.y, r1.z);
          r.inv = v3(__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z));
          beta = C3f{r2.x, r2.y, r2.z};
          trav_init<F>(t, items[item].sc, r, 3.402823466e38f);
          has = true;
          ++queries;
        }
      }
    }
    const unsigned live = __ballot_sync(0xffffffffu, has);
    if (!live) break;
    if (has && !done) {
      const GpuScene& sc = items[item].sc;
      const FrameParams& fp = items[item].fp;
      const RngCtx ctx{fp.seed_lo, fp.seed_hi, pix, smp, depth, nullptr};
      done = trav_run<F, false, true>(t, stack, sc, r, 1e-3f, ctx, cnt, fp.err, budget);
    }
    if (finish_now(done, live, shade_lanes)) {
      const GpuScene& sc = items[item].sc;
      const FrameParams& fp = items[item].fp;
      HitRec h;
      const bool hit = finish_hit<F, false>(sc, r, 1e-3f, 3.402823466e38f, t, h, cnt);
      if (shade_path<F>(sc, fp, s, p, pix, smp, depth, r, beta, hit, h)) {
        uint32_t slot = warp_append(s.counts + nxt, true);
        if (slot < wp.n_paths) s.active[nxt][slot] = p;
        else atomicOr(err, ERR_QUEUE_OVERFLOW);
      }
      has = false;
      done = false;
    }
  }
  FrameParams f0;
  f0.counters = counters;
  flush_wave_counters<false>(f0, cnt, queries);
}

// Per-pixel sums of every render of the wave, in the canonical order.
__global__ void __launch_bounds__(kWfBlock) k_baccumulate(const BatchItemDev* __restrict__ items,
                                                          const BatchChunk* __restrict__ chunks, uint32_t first_chunk,
                                                          uint32_t n_chunks, uint32_t n_pixels, PathState s) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n_pixels * 3; q += gridDim.x * blockDim.x) {
    const uint32_t lp = q / 3, c = q % 3;
    const uint32_t k = find_chunk(first_chunk, n_chunks, lp, [&](uint32_t i) { return chunks[i].pix0; });
    const BatchChunk ch = chunks[k];
    const uint32_t rel = lp - ch.pix0;
    accumulate_pixel(items[ch.item].fp, s, (size_t)ch.slot0 + (size_t)rel * ch.spp, ch.first_pixel + rel, c);
  }
}

uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

}  // namespace rg

using namespace rg;

struct rg_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<rg_renderer*> items;
  std::string err;
  BatchItemDev* d_items = nullptr;
  BatchItemDev* h_items = nullptr;  // pinned
  uint32_t* d_prefix = nullptr;
  uint32_t* d_counter = nullptr;
  unsigned long long* d_counters = nullptr;
  uint32_t total_work = 0;
  uint32_t features = 0;
  rg_batch_tuning tuning{};
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  uint32_t launches = 0;            // kernels of one frame
  // RG_BATCH_WAVEFRONT
  struct Wave {
    uint32_t first_chunk, n_chunks, n_paths, n_pixels, max_depth;
  };
  std::vector<Wave> waves;
  BatchChunk* d_chunks = nullptr;
  void* wf_arena = nullptr;         // path state of one wave + per-slot chunk index
  size_t wf_cap = 0;
  uint32_t* d_err = nullptr;        // queue overflows of the batched kernels
};

namespace {

rg_status bfail(rg_batch* b, rg_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return st;
}

rg_status bcuda(rg_batch* b, cudaError_t e, const char* what) {
  cudaGetLastError();
  return bfail(b, e == cudaErrorMemoryAllocation ? RG_OOM : RG_CUDA_ERROR, "%s: %s", what, cudaGetErrorString(e));
}

#define BCUDA(b, call, what)                                  \
  do {                                                        \
    cudaError_t e__ = (call);                                 \
    if (e__ != cudaSuccess) return bcuda(b, e__, what);       \
  } while (0)

void drop_graph(rg_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
}

// Waves of the batched wavefront: renders in order, each cut into runs of
// whole pixels that fill waves of `cap` path slots.
rg_status plan_waves(rg_batch* b) {
  uint64_t total = 0;
  for (rg_renderer* h : b->items) total += (uint64_t)h->opts.width * h->opts.height * h->opts.samples;
  uint64_t cap = b->tuning.wave_paths ? b->tuning.wave_paths : std::min<uint64_t>(kDefaultWavePaths, total);
  for (rg_renderer* h : b->items) cap = std::max<uint64_t>(cap, h->opts.samples);  // a wave holds whole pixels
  if (cap > 0x7FFFFFFFull) return bfail(b, RG_INVALID_ARG, "wave_paths too large");
  std::vector<BatchChunk> chunks;
  b->waves.clear();
  rg_batch::Wave cur{0, 0, 0, 0, 0};
  auto close = [&]() {
    if (cur.n_chunks) b->waves.push_back(cur);
    cur = rg_batch::Wave{(uint32_t)chunks.size(), 0, 0, 0, 0};
  };
  for (size_t i = 0; i < b->items.size(); ++i) {
    const rg_render_opts& o = b->items[i]->opts;
    const uint64_t npix = (uint64_t)o.width * o.height;
    uint64_t done = 0;
    while (done < npix) {
      uint64_t fit = (cap - cur.n_paths) / o.samples;
      if (fit == 0) { close(); continue; }
      const uint64_t take = std::min(fit, npix - done);
      BatchChunk c{};
      c.item = (uint32_t)i;
      c.first_pixel = (uint32_t)done;
      c.n_pixels = (uint32_t)take;
      c.spp = o.samples;
      c.slot0 = cur.n_paths;
      c.pix0 = cur.n_pixels;
      chunks.push_back(c);
      cur.n_chunks += 1;
      cur.n_paths += (uint32_t)(take * o.samples);
      cur.n_pixels += (uint32_t)take;
      cur.max_depth = std::max(cur.max_depth, o.ray_depth);
      done += take;
    }
  }
  close();
  if (b->d_chunks) cudaFree(b->d_chunks);
  b->d_chunks = nullptr;
  BCUDA(b, cudaMalloc((void**)&b->d_chunks, std::max<size_t>(1, chunks.size()) * sizeof(BatchChunk)), "batch waves");
  if (!chunks.empty())
    BCUDA(b, cudaMemcpy(b->d_chunks, chunks.data(), chunks.size() * sizeof(BatchChunk), cudaMemcpyHostToDevice), "batch waves");
  if (b->wf_cap != cap) {
    if (b->wf_arena) cudaFree(b->wf_arena);
    b->wf_arena = nullptr;
    b->wf_cap = 0;
    BCUDA(b, cudaMalloc(&b->wf_arena, arena_bytes(cap) + cap * sizeof(uint32_t)), "batch path state");
    b->wf_cap = cap;
  }
  return RG_OK;
}

template <uint32_t F>
cudaError_t launch_batch_wavefront(rg_batch* b) {
  PathState s;
  const size_t used = carve((char*)b->wf_arena, b->wf_cap, s);
  uint32_t* chunk_of = (uint32_t*)((char*)b->wf_arena + used);
  const int sms = sm_count(b->device);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bbounce<F>, kWfBlock, 0);
  const int bounce_grid = sms * std::max(per_sm, 1);
  const int grid = sms * 8;
  const int budget = (int)kDefaultFetchBudget;
  const int shade_lanes = (int)(b->tuning.shade_lanes ? b->tuning.shade_lanes : kBatchShadeLanesDefault);
  cudaStream_t st = b->stream;
  cudaError_t e;
  b->launches = 0;
  for (const rg_batch::Wave& w : b->waves) {
    WaveParams wp;
    wp.first_pixel = 0;
    wp.n_pixels = w.n_pixels;
    wp.n_paths = w.n_paths;
    wp.capacity = (uint32_t)b->wf_cap;
    const uint32_t gen_blocks = (uint32_t)std::min<size_t>((w.n_paths + kWfBlock - 1) / kWfBlock, (size_t)grid * 4);
    k_bgenerate<<<gen_blocks, kWfBlock, 0, st>>>(b->d_items, b->d_chunks, w.first_chunk, w.n_chunks, w.n_paths, s,
                                                 chunk_of);
    int cur = 0;
    for (uint32_t d = 0; d <= w.max_depth; ++d) {
      if ((e = cudaMemsetAsync(s.counts + (cur ^ 1), 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
      if ((e = cudaMemsetAsync(s.counts + kFetchCounter, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
      k_bbounce<F><<<bounce_grid, kWfBlock, 0, st>>>(b->d_items, b->d_chunks, wp, s, chunk_of, cur, budget,
                                                     shade_lanes, b->d_err, b->d_counters);
      cur ^= 1;
    }
    const uint32_t acc_blocks = (uint32_t)std::min<size_t>((w.n_pixels * 3 + kWfBlock - 1) / kWfBlock, (size_t)grid * 4);
    k_baccumulate<<<acc_blocks, kWfBlock, 0, st>>>(b->d_items, b->d_chunks, w.first_chunk, w.n_chunks, w.n_pixels, s);
    b->launches += w.max_depth + 3;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Work-item prefix sums for the current tuning.
rg_status layout(rg_batch* b) {
  const uint32_t rpi = b->tuning.rounds_per_item ? b->tuning.rounds_per_item : 4u;
  std::vector<uint32_t> prefix(b->items.size() + 1, 0);
  uint64_t acc = 0;
  for (size_t i = 0; i < b->items.size(); ++i) {
    const rg_render_opts& o = b->items[i]->opts;
    uint64_t npix = (uint64_t)o.width * o.height;
    uint64_t ppr = pixels_per_round(o.samples);
    uint64_t rounds = (npix + ppr - 1) / ppr;
    prefix[i] = (uint32_t)acc;
    acc += (rounds + rpi - 1) / rpi;
  }
  if (acc >= 0xFFFFFFFFull) return bfail(b, RG_INVALID_ARG, "batch too large");
  prefix[b->items.size()] = (uint32_t)acc;
  b->total_work = (uint32_t)acc;
  BCUDA(b, cudaMemcpy(b->d_prefix, prefix.data(), prefix.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "batch layout");
  if (b->tuning.form == RG_BATCH_WAVEFRONT) return plan_waves(b);
  return RG_OK;
}

template <uint32_t F>
cudaError_t launch_batch_kernel(rg_batch* b) {
  const int block = b->tuning.block ? (int)b->tuning.block : 256;
  int sms = 1, fit = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k_batch<F>, block, 0);
  int per_sm = b->tuning.blocks_per_sm ? std::min<int>((int)b->tuning.blocks_per_sm, std::max(fit, 1)) : std::max(fit, 1);
  const uint32_t rpi = b->tuning.rounds_per_item ? b->tuning.rounds_per_item : 4u;
  k_batch<F><<<sms * per_sm, block, 0, b->stream>>>(b->d_items, b->d_prefix, (uint32_t)b->items.size(), b->total_work, rpi,
                                                    b->d_counter, b->d_counters);
  return cudaGetLastError();
}

// Kernel variant of the batch: the union of the renders' primitive kinds,
// traversing the 8-wide trees when the tuning asks for them and every render
// has one.
uint32_t batch_features(const rg_batch* b) {
  bool wide = !b->items.empty();
  for (const rg_renderer* h : b->items)
    wide = wide && effective_bvh_width(b->tuning.bvh_width, h->gs, RG_FORM_MEGAKERNEL) == 8;
  return b->features | (wide ? F_WIDE : 0u);
}

// Clears the error bits of the batch and of every render: each frame reports its own.
cudaError_t clear_errors(rg_batch* b) {
  cudaError_t e = cudaMemsetAsync(b->d_err, 0, sizeof(uint32_t), b->stream);
  for (size_t i = 0; e == cudaSuccess && i < b->items.size(); ++i)
    e = cudaMemsetAsync(b->items[i]->d_err, 0, sizeof(uint32_t), b->stream);
  return e;
}

cudaError_t enqueue_frame(rg_batch* b) {
  cudaError_t e;
  if ((e = cudaMemcpyAsync(b->d_items, b->h_items, b->items.size() * sizeof(BatchItemDev), cudaMemcpyHostToDevice,
                           b->stream)) != cudaSuccess)
    return e;
  if ((e = cudaMemsetAsync(b->d_counter, 0, sizeof(uint32_t), b->stream)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(b->d_counters, 0, CNT_N * sizeof(unsigned long long), b->stream)) != cudaSuccess) return e;
  if ((e = clear_errors(b)) != cudaSuccess) return e;
  if (b->tuning.form == RG_BATCH_WAVEFRONT)
    return dispatch_features(batch_features(b), [&](auto f) { return launch_batch_wavefront<decltype(f)::value>(b); });
  b->launches = 1;
  return dispatch_features(batch_features(b), [&](auto f) { return launch_batch_kernel<decltype(f)::value>(b); });
}

// Fills the pinned parameter table for frame `seed` (one frame per render).
rg_status prepare_frame(rg_batch* b, uint64_t seed) {
  for (size_t i = 0; i < b->items.size(); ++i) {
    rg_renderer* h = b->items[i];
    rg_status st = ensure_frame_buffers(h);
    if (st != RG_OK) return bfail(b, st, "render %zu: %s", i, h->err.c_str());
    h->frame_count += 1;
    h->pixel_accum += 1;
    FrameParams fp;
    fill_frame_params(h, rg_batch_item_seed(seed, (uint32_t)i), fp);
    fp.accum_count = h->pixel_accum;
    fp.counters = b->d_counters;
    b->h_items[i].sc = h->gs;
    b->h_items[i].fp = fp;
  }
  return RG_OK;
}

rg_status finish_stats(rg_batch* b, rg_render_stats* stats, std::chrono::steady_clock::time_point t0) {
  BCUDA(b, cudaStreamSynchronize(b->stream), "batch frame");
  if (!stats) return RG_OK;
  std::memset(stats, 0, sizeof(*stats));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  unsigned long long c[CNT_N];
  BCUDA(b, cudaMemcpy(c, b->d_counters, sizeof(c), cudaMemcpyDeviceToHost), "batch counters");
  uint32_t err = 0;
  BCUDA(b, cudaMemcpy(&err, b->d_err, sizeof(err), cudaMemcpyDeviceToHost), "batch error flags");
  for (rg_renderer* h : b->items) {
    stats->samples += (uint64_t)h->opts.width * h->opts.height * h->opts.samples;
    uint32_t e1 = 0;
    cudaMemcpy(&e1, h->d_err, sizeof(e1), cudaMemcpyDeviceToHost);
    err |= e1;
  }
  stats->kernel_ms = ms;
  stats->rays = c[CNT_RAYS];
  stats->accum_frames = b->items.empty() ? 0 : b->items[0]->frame_count;
  stats->error_flags = err;
  stats->kernel_launches = b->launches;
  stats->duration_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  const rg_status dst = device_status(err);
  if (dst != RG_OK) return bfail(b, dst, "device error bits 0x%x this frame", err);
  return RG_OK;
}

}  // namespace

uint64_t rg_batch_item_seed(uint64_t seed, uint32_t index) { return splitmix64(seed + index); }

rg_status rg_batch_create(const rg_device_opts* opts, uint32_t n, const rg_scene_desc* const* scenes, const rg_camera* cameras,
                          const rg_render_opts* options, rg_batch_handle* out) {
  if (!out || (n && (!scenes || !cameras || !options))) return RG_INVALID_ARG;
  *out = nullptr;
  rg_batch* b = new (std::nothrow) rg_batch();
  if (!b) return RG_OOM;
  rg_device_opts o{};
  if (opts) o = *opts;
  b->device = o.device;
  cudaError_t e = cudaSetDevice(o.device);
  if (e != cudaSuccess) { delete b; cudaGetLastError(); return RG_NO_DEVICE; }
  if (o.stream) {
    b->stream = (cudaStream_t)o.stream;
  } else {
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) { delete b; return RG_CUDA_ERROR; }
    b->own_stream = true;
  }
  rg_status st = RG_OK;
  rg_device_opts io = o;
  io.stream = b->stream;
  io.form = RG_FORM_MEGAKERNEL;
  for (uint32_t i = 0; i < n && st == RG_OK; ++i) {
    rg_renderer* h = nullptr;
    st = rg_create(&io, &h);
    if (st != RG_OK) break;
    b->items.push_back(h);
    if ((st = rg_set_scene(h, scenes[i])) != RG_OK) { b->err = h->err; break; }
    if ((st = rg_set_camera(h, &cameras[i])) != RG_OK) { b->err = h->err; break; }
    if ((st = rg_set_options(h, &options[i])) != RG_OK) { b->err = h->err; break; }
    if (!h->cam_ok) { st = bfail(b, RG_INVALID_CAMERA, "render %u: invalid camera", i); break; }
    if (h->opts.mode != RG_MODE_PBR || h->opts.ray_branching != 1) {
      st = bfail(b, RG_UNSUPPORTED_VARIANT, "render %u: batches render RenderMode::PBR with ray_branching 1", i);
      break;
    }
    if ((st = ensure_frame_buffers(h)) != RG_OK) { b->err = h->err; break; }
    b->features |= kinds_of(h->gs.features);
  }
  if (st == RG_OK) {
    b->features = b->features == F_TRI ? F_TRI
                : (b->features == F_SPHERE ? F_SPHERE : ((b->features & F_EXT) ? F_ANY : F_ALL));
    size_t nb = std::max<size_t>(1, n);
    if ((e = cudaMalloc((void**)&b->d_items, nb * sizeof(BatchItemDev))) != cudaSuccess ||
        (e = cudaMallocHost((void**)&b->h_items, nb * sizeof(BatchItemDev))) != cudaSuccess ||
        (e = cudaMalloc((void**)&b->d_prefix, (nb + 1) * sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMalloc((void**)&b->d_counter, sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMalloc((void**)&b->d_counters, CNT_N * sizeof(unsigned long long))) != cudaSuccess ||
        (e = cudaMalloc((void**)&b->d_err, sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMemset(b->d_err, 0, sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaEventCreate(&b->ev0)) != cudaSuccess || (e = cudaEventCreate(&b->ev1)) != cudaSuccess) {
      st = bcuda(b, e, "rg_batch_create");
    } else {
      st = layout(b);
    }
  }
  if (st != RG_OK) {
    std::string msg = b->err;
    rg_batch_destroy(b);
    return st;
  }
  *out = b;
  return RG_OK;
}

rg_status rg_batch_destroy(rg_batch_handle b) {
  if (!b) return RG_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  for (rg_renderer* h : b->items) rg_destroy(h);
  if (b->d_items) cudaFree(b->d_items);
  if (b->h_items) cudaFreeHost(b->h_items);
  if (b->d_prefix) cudaFree(b->d_prefix);
  if (b->d_counter) cudaFree(b->d_counter);
  if (b->d_counters) cudaFree(b->d_counters);
  if (b->d_err) cudaFree(b->d_err);
  if (b->d_chunks) cudaFree(b->d_chunks);
  if (b->wf_arena) cudaFree(b->wf_arena);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return RG_OK;
}

rg_status rg_batch_last_error(rg_batch_handle b, char* buf, size_t len) {
  if (!b || !buf || len == 0) return RG_INVALID_ARG;
  size_t n = std::min(len - 1, b->err.size());
  std::memcpy(buf, b->err.data(), n);
  buf[n] = '\0';
  return RG_OK;
}

rg_status rg_batch_set_tuning(rg_batch_handle b, const rg_batch_tuning* t) {
  if (!b || !t) return RG_INVALID_ARG;
  if (t->reserved) return bfail(b, RG_INVALID_ARG, "rg_batch_tuning: reserved field must be 0");
  if (t->shade_lanes > 32) return bfail(b, RG_INVALID_ARG, "rg_batch_tuning: shade_lanes must be at most 32");
  if (t->block && (t->block % 32 || t->block < 64 || t->block > 512))
    return bfail(b, RG_INVALID_ARG, "block must be a multiple of 32 in [64, 512]");
  if (t->rounds_per_item > 4096) return bfail(b, RG_INVALID_ARG, "rounds_per_item too large");
  if (t->bvh_width != 0 && t->bvh_width != 2 && t->bvh_width != 8)
    return bfail(b, RG_INVALID_ARG, "rg_batch_tuning: bvh_width must be 0, 2 or 8");
  if (t->form > RG_BATCH_TILES) return bfail(b, RG_INVALID_ARG, "rg_batch_tuning: unknown form %u", t->form);
  if (t->wave_paths > 0x7FFFFFFFu) return bfail(b, RG_INVALID_ARG, "rg_batch_tuning: wave_paths too large");
  cudaSetDevice(b->device);
  if (t->block) {
    cudaFuncAttributes fa{};
    rg_batch_tuning prev = b->tuning;
    b->tuning.bvh_width = t->bvh_width;
    const uint32_t feats = batch_features(b);
    b->tuning = prev;
    cudaError_t e = dispatch_features(feats, [&](auto f) { return cudaFuncGetAttributes(&fa, k_batch<decltype(f)::value>); });
    if (e != cudaSuccess) return bcuda(b, e, "rg_batch_set_tuning");
    if ((int)t->block > fa.maxThreadsPerBlock)
      return bfail(b, RG_INVALID_ARG, "block %u exceeds the kernel's %d threads per block (registers)", t->block,
                   fa.maxThreadsPerBlock);
  }
  b->tuning = *t;
  drop_graph(b);
  return layout(b);
}

rg_status rg_batch_render(rg_batch_handle b, uint64_t seed, rg_render_stats* stats) {
  if (!b) return RG_INVALID_ARG;
  auto t0 = std::chrono::steady_clock::now();
  cudaSetDevice(b->device);
  if (b->items.empty()) return RG_OK;
  BCUDA(b, cudaStreamSynchronize(b->stream), "batch");  // the pinned table is rewritten below
  rg_status st = prepare_frame(b, seed);
  if (st != RG_OK) return st;
  if (!b->graph) {
    cudaGraph_t g = nullptr;
    BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
    cudaError_t e = enqueue_frame(b);
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return bcuda(b, e, "graph capture"); }
    if (e2 != cudaSuccess) return bcuda(b, e2, "graph capture");
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { b->graph = nullptr; return bcuda(b, e, "graph instantiate"); }
  }
  BCUDA(b, cudaEventRecord(b->ev0, b->stream), "event");
  BCUDA(b, cudaGraphLaunch(b->graph, b->stream), "graph launch");
  BCUDA(b, cudaEventRecord(b->ev1, b->stream), "event");
  return finish_stats(b, stats, t0);
}

rg_status rg_batch_render_sequential(rg_batch_handle b, uint64_t seed, rg_render_stats* stats) {
  if (!b) return RG_INVALID_ARG;
  auto t0 = std::chrono::steady_clock::now();
  cudaSetDevice(b->device);
  BCUDA(b, cudaStreamSynchronize(b->stream), "batch");
  rg_status st = prepare_frame(b, seed);
  if (st != RG_OK) return st;
  BCUDA(b, cudaMemsetAsync(b->d_counters, 0, CNT_N * sizeof(unsigned long long), b->stream), "batch counters");
  BCUDA(b, clear_errors(b), "batch error bits");
  BCUDA(b, cudaEventRecord(b->ev0, b->stream), "event");
  for (size_t i = 0; i < b->items.size(); ++i) {
    cudaError_t e = launch_megakernel(b->h_items[i].sc, b->h_items[i].fp, false, b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "sequential launch");
  }
  BCUDA(b, cudaEventRecord(b->ev1, b->stream), "event");
  return finish_stats(b, stats, t0);
}

rg_status rg_batch_image(rg_batch_handle b, uint32_t index, float* out_rgb) {
  if (!b || !out_rgb || index >= b->items.size()) return RG_INVALID_ARG;
  cudaSetDevice(b->device);
  rg_renderer* h = b->items[index];
  size_t n = (size_t)h->opts.width * h->opts.height * 3;
  BCUDA(b, cudaMemcpyAsync(out_rgb, h->d_out, n * sizeof(float), cudaMemcpyDeviceToHost, b->stream), "batch image");
  BCUDA(b, cudaStreamSynchronize(b->stream), "batch image");
  return RG_OK;
}
