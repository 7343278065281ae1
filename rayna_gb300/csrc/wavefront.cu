// wavefront.cu — the wavefront kernel form.
//
// A frame is split into waves of whole pixels (all samples of a pixel are in
// one wave). For every wave:
//   generate    one camera ray per path slot (slot p = pixel-in-wave * spp + sample)
//   extend      closest hit of every active path (BVH + unbounded list); each
//               path is appended to the queue of its hit's material kind
//               (warp-ballot compaction: one atomic per warp and kind), which
//               sorts the shade work by material key
//   shade       over the kind queues laid end to end: emission, sky, scatter,
//               attenuation; survivors are compacted into the next active queue
//   accumulate  per-pixel sums in sample order, then the accumulation buffer
// Paths run the same per-path functions as the megakernel (trace.cuh) with the
// same counter-based random streams, and the per-pixel sums are taken in the
// same order, so both forms produce the same image bit for bit.
//
// Path state is structure-of-arrays in one device arena (80 bytes per slot);
// counts live in device memory, so a wave is a fixed launch sequence with no
// host round trip.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "kernels.h"
#include "renderer_state.h"
#include "trace.cuh"

namespace rg {

namespace {

constexpr int kWfBlock = 256;
constexpr int kKinds = 6;  // miss, lambertian, metal, dielectric, isotropic, light
enum : uint32_t { KQ_MISS = 0 };

struct PathSoA {
  float *ox, *oy, *oz, *dx, *dy, *dz;
  float *br, *bg, *bb, *lr, *lg, *lb;
  float* t;
  int* prim;
  int* sdf;
  float *snx, *sny, *snz;
  uint32_t* sflags;  // front bit 31 | side
  uint32_t* depth;
  uint32_t* active[2];
  uint32_t* kindq;     // kKinds x capacity
  uint32_t* counts;    // [0], [1]: active counts; [2 .. 2+kKinds): kind counts
  float *sr, *sg, *sb; // per-slot sample radiance
};

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

__global__ void __launch_bounds__(kWfBlock) k_generate(FrameParams fp, PathSoA s, WaveParams wp) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    s.counts[0] = wp.n_paths;
    s.counts[1] = 0;
  }
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < wp.n_paths; p += gridDim.x * blockDim.x) {
    uint32_t pix = wp.first_pixel + p / fp.spp, smp = p % fp.spp;
    uint32_t x = pix % fp.width, y = pix / fp.width;
    RngCtx ctx{fp.seed_lo, fp.seed_hi, pix, smp, 0, nullptr};
    Ray r = camera_ray(fp, x, y, smp, ctx);
    s.ox[p] = r.o.x; s.oy[p] = r.o.y; s.oz[p] = r.o.z;
    s.dx[p] = r.d.x; s.dy[p] = r.d.y; s.dz[p] = r.d.z;
    s.br[p] = 1.0f; s.bg[p] = 1.0f; s.bb[p] = 1.0f;
    s.lr[p] = 0.0f; s.lg[p] = 0.0f; s.lb[p] = 0.0f;
    s.depth[p] = 0;
    s.active[0][p] = p;
  }
}

template <uint32_t F, bool COUNT>
__global__ void __launch_bounds__(kWfBlock) k_extend(GpuScene sc, FrameParams fp, PathSoA s, WaveParams wp, int cur) {
  uint32_t n = s.counts[cur];
  if (n > wp.n_paths) {  // never expected: record and clamp instead of reading past the queue
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(fp.err, ERR_QUEUE_OVERFLOW);
    n = wp.n_paths;
  }
  Counters cnt;
  uint32_t queries = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint32_t p = s.active[cur][i];
    uint32_t pix = wp.first_pixel + p / fp.spp, smp = p % fp.spp;
    Ray r;
    r.o = v3(s.ox[p], s.oy[p], s.oz[p]);
    r.d = v3(s.dx[p], s.dy[p], s.dz[p]);
    r.inv = v3(__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z));
    RngCtx ctx{fp.seed_lo, fp.seed_hi, pix, smp, s.depth[p], nullptr};
    HitRec h;
    ++queries;
    bool hit = closest_hit<F, COUNT>(sc, r, 1e-3f, 3.402823466e38f, ctx, h, cnt, fp.err);
    uint32_t kind = KQ_MISS;
    if (hit) {
      uint32_t mat;
      if (h.sdf >= 0) {
        mat = sc.sdfs[h.sdf].material;
        s.snx[p] = h.sh.n.x; s.sny[p] = h.sh.n.y; s.snz[p] = h.sh.n.z;
        s.sflags[p] = (h.sh.front ? 0x80000000u : 0u) | (h.sh.side & 0x7FFFFFFFu);
      } else {
        mat = prim_material(sc.prims[h.prim]);
      }
      kind = 1u + sc.materials[mat].kind;
      s.t[p] = h.t;
      s.prim[p] = h.prim;
      s.sdf[p] = h.sdf;
    }
    // Append to the queue of this kind: one atomic per warp and kind present.
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
  unsigned long long q = queries;
  for (int o = 16; o > 0; o >>= 1) q += __shfl_down_sync(0xffffffffu, q, o);
  if ((threadIdx.x & 31) == 0 && q) atomicAdd(fp.counters + CNT_RAYS, q);
  if (COUNT) {
    unsigned long long a = cnt.nodes, b = cnt.prims, c = cnt.sdf_steps;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(fp.counters + CNT_NODES, a);
      atomicAdd(fp.counters + CNT_PRIMS, b);
      atomicAdd(fp.counters + CNT_SDF, c);
    }
  }
}

template <uint32_t F>
__global__ void __launch_bounds__(kWfBlock) k_shade(GpuScene sc, FrameParams fp, PathSoA s, WaveParams wp, int cur) {
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
    uint32_t p = s.kindq[(size_t)k * wp.capacity + (i - off[k])];
    uint32_t pix = wp.first_pixel + p / fp.spp, smp = p % fp.spp;
    uint32_t depth = s.depth[p];
    Ray r;
    r.o = v3(s.ox[p], s.oy[p], s.oz[p]);
    r.d = v3(s.dx[p], s.dy[p], s.dz[p]);
    r.inv = v3(__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z));
    C3f L{s.lr[p], s.lg[p], s.lb[p]};
    C3f beta{s.br[p], s.bg[p], s.bb[p]};
    bool alive = false;
    if (k == KQ_MISS) {
      C3f sk = sky_colour(sc.sky, r.d);
      L = C3f{L.r + beta.r * sk.r, L.g + beta.g * sk.g, L.b + beta.b * sk.b};
    } else {
      RngCtx ctx{fp.seed_lo, fp.seed_hi, pix, smp, depth, nullptr};
      HitRec h;
      h.t = s.t[p];
      h.prim = s.prim[p];
      h.sdf = s.sdf[p];
      if (h.sdf >= 0) {
        h.sh.n = v3(s.snx[p], s.sny[p], s.snz[p]);
        uint32_t f = s.sflags[p];
        h.sh.front = (f >> 31) != 0;
        h.sh.side = f & 0x7FFFFFFFu;
        h.sh.t = h.t;
      }
      Surface surf;
      finalize_hit<F>(sc, r, h, ctx, surf);
      const rg_material m = sc.materials[surf.material];
      if (m.kind == RG_MAT_LIGHT) {
        L = C3f{L.r + beta.r * m.albedo[0], L.g + beta.g * m.albedo[1], L.b + beta.b * m.albedo[2]};
      } else if (depth < fp.ray_depth) {
        V3 dir;
        if (scatter(m, r, surf, ctx, dir)) {
          C3f a = attenuation(m, r, surf);
          beta = C3f{beta.r * a.r, beta.g * a.g, beta.b * a.b};
          Ray nr = make_ray(surf.pos, dir);
          s.ox[p] = nr.o.x; s.oy[p] = nr.o.y; s.oz[p] = nr.o.z;
          s.dx[p] = nr.d.x; s.dy[p] = nr.d.y; s.dz[p] = nr.d.z;
          s.br[p] = beta.r; s.bg[p] = beta.g; s.bb[p] = beta.b;
          s.depth[p] = depth + 1;
          alive = true;
        }
      }
    }
    if (alive) {
      uint32_t slot = warp_append(s.counts + nxt, true);
      if (slot < wp.n_paths) s.active[nxt][slot] = p;
      else atomicOr(fp.err, ERR_QUEUE_OVERFLOW);
    } else {
      s.sr[p] = L.r; s.sg[p] = L.g; s.sb[p] = L.b;
    }
  }
}

// Per-pixel sums in the megakernel's canonical order: samples 0..spp-1 in
// turn for spp <= 32; for larger spp, lane partials (samples l, l+32, ...)
// added for l = 0..31 in turn.
__global__ void __launch_bounds__(kWfBlock) k_accumulate(FrameParams fp, PathSoA s, WaveParams wp) {
  const uint32_t spp = fp.spp;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < wp.n_pixels * 3; q += gridDim.x * blockDim.x) {
    uint32_t lp = q / 3, c = q % 3;
    const float* src = c == 0 ? s.sr : (c == 1 ? s.sg : s.sb);
    const float* base = src + (size_t)lp * spp;
    float sum = 0.0f;
    double sumd = 0.0, sqd = 0.0;
    if (spp <= 32) {
      for (uint32_t k = 0; k < spp; ++k) {
        float v = base[k];
        sum = sum + v;
        sumd += v;
        sqd += (double)v * v;
      }
    } else {
      for (uint32_t l = 0; l < 32; ++l) {
        float part = 0.0f;
        double psq = 0.0;
        for (uint32_t k = l; k < spp; k += 32) {
          float v = base[k];
          part = part + v;
          psq += (double)v * v;
        }
        sum = sum + part;
        sumd += part;
        sqd += psq;
      }
    }
    uint32_t pix = wp.first_pixel + lp;
    uint32_t x = pix % fp.width, y = pix / fp.width;
    size_t idx = ((size_t)x * fp.height + y) * 3 + c;
    float mean = sum / (float)spp;
    float acc = fp.accum[idx] + mean;
    fp.accum[idx] = acc;
    if (fp.out) fp.out[idx] = (float)((double)acc / (double)fp.accum_count);
    if (fp.frame_mean) fp.frame_mean[idx] = mean;
    if (fp.frame_var) {
      double m = sumd / spp;
      fp.frame_var[idx] = spp > 1 ? (float)fmax(0.0, (sqd - spp * m * m) / (spp - 1)) : 0.0f;
    }
  }
}

// Lays the path arrays out from `arena` (256-byte aligned each) and returns
// the number of bytes used; with a null arena it only measures.
size_t carve(char* arena, size_t cap, PathSoA& s) {
  size_t used = 0;
  auto take = [&](size_t bytes) {
    char* r = arena ? arena + used : nullptr;
    used += (bytes + 255) & ~size_t(255);
    return r;
  };
  float** fl[] = {&s.ox, &s.oy, &s.oz, &s.dx, &s.dy, &s.dz, &s.br, &s.bg, &s.bb, &s.lr, &s.lg, &s.lb, &s.t,
                  &s.snx, &s.sny, &s.snz, &s.sr, &s.sg, &s.sb};
  for (float** f : fl) *f = (float*)take(cap * 4);
  s.prim = (int*)take(cap * 4);
  s.sdf = (int*)take(cap * 4);
  s.sflags = (uint32_t*)take(cap * 4);
  s.depth = (uint32_t*)take(cap * 4);
  s.active[0] = (uint32_t*)take(cap * 4);
  s.active[1] = (uint32_t*)take(cap * 4);
  s.kindq = (uint32_t*)take(cap * 4 * kKinds);
  s.counts = (uint32_t*)take(64 * 4);
  return used;
}

size_t arena_bytes(size_t cap) {
  PathSoA s;
  return carve(nullptr, cap, s);
}

int sm_count(int device) {
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
  return n > 0 ? n : 1;
}

// Runs every wave of one frame on the path arrays `s` (capacity `cap` slots).
template <uint32_t F>
cudaError_t run_waves(rg_renderer* h, const FrameParams& fp, const PathSoA& s, size_t cap, size_t pix_per_wave) {
  const size_t spp = fp.spp;
  const size_t n_pix = (size_t)fp.width * fp.height;
  const bool counters = (h->flags & RG_FLAG_COUNTERS) != 0;
  const int grid = sm_count(h->device) * 8;
  cudaStream_t st = h->stream;
  cudaError_t e;
  for (size_t first = 0; first < n_pix; first += pix_per_wave) {
    WaveParams wp;
    wp.first_pixel = (uint32_t)first;
    wp.n_pixels = (uint32_t)std::min(pix_per_wave, n_pix - first);
    wp.n_paths = (uint32_t)(wp.n_pixels * spp);
    wp.capacity = (uint32_t)cap;
    uint32_t gen_blocks = (uint32_t)std::min<size_t>((wp.n_paths + kWfBlock - 1) / kWfBlock, (size_t)grid * 4);
    k_generate<<<gen_blocks, kWfBlock, 0, st>>>(fp, s, wp);
    int cur = 0;
    for (uint32_t d = 0; d <= fp.ray_depth; ++d) {
      if ((e = cudaMemsetAsync(s.counts + 2, 0, kKinds * sizeof(uint32_t), st)) != cudaSuccess) return e;
      if ((e = cudaMemsetAsync(s.counts + (cur ^ 1), 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
      if (counters) k_extend<F, true><<<grid, kWfBlock, 0, st>>>(h->gs, fp, s, wp, cur);
      else k_extend<F, false><<<grid, kWfBlock, 0, st>>>(h->gs, fp, s, wp, cur);
      k_shade<F><<<grid, kWfBlock, 0, st>>>(h->gs, fp, s, wp, cur);
      cur ^= 1;
    }
    uint32_t acc_blocks = (uint32_t)std::min<size_t>((wp.n_pixels * 3 + kWfBlock - 1) / kWfBlock, (size_t)grid * 4);
    k_accumulate<<<acc_blocks, kWfBlock, 0, st>>>(fp, s, wp);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t run_frame(rg_renderer* h, const FrameParams& fp, const PathSoA& s, size_t cap, size_t pix_per_wave) {
  if (h->gs.features == F_TRI) return run_waves<F_TRI>(h, fp, s, cap, pix_per_wave);
  if (h->gs.features == F_SPHERE) return run_waves<F_SPHERE>(h, fp, s, cap, pix_per_wave);
  return run_waves<F_ALL>(h, fp, s, cap, pix_per_wave);
}

}  // namespace

// Default path budget per wave: 2^23 slots (about 700 MB of path state).
constexpr size_t kDefaultWavePaths = size_t(1) << 23;

cudaError_t launch_wavefront(rg_renderer* h, const FrameParams& fp) {
  const size_t spp = fp.spp;
  const size_t n_pix = (size_t)fp.width * fp.height;
  size_t budget = h->wf_paths ? h->wf_paths : kDefaultWavePaths;
  size_t pix_per_wave = std::max<size_t>(1, budget / spp);
  pix_per_wave = std::min(pix_per_wave, n_pix);
  size_t cap = pix_per_wave * spp;
  if (cap > 0xFFFFFFFFull) return cudaErrorInvalidValue;
  if (h->wf.capacity < cap) {
    if (h->wf.arena) cudaFree(h->wf.arena);
    h->wf = WavefrontState{};
    cudaError_t e = cudaMalloc(&h->wf.arena, arena_bytes(cap));
    if (e != cudaSuccess) return e;
    h->wf.capacity = cap;
    h->wf.arena_bytes = arena_bytes(cap);
  }
  PathSoA s;
  carve((char*)h->wf.arena, h->wf.capacity, s);
  return run_frame(h, fp, s, h->wf.capacity, pix_per_wave);
}

// ---------------------------------------------------------------------------
// Allocation-free variant: the path state of one wave lives in a fixed
// file-scope device array instead of a cudaMalloc'ed arena.
// ---------------------------------------------------------------------------
constexpr size_t kStaticArenaBytes = 31ull * 4ull * RG_STATIC_WAVE_PATHS + 256ull;
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
  PathSoA s;
  carve((char*)arena, cap, s);
  return run_frame(h, fp, s, cap, std::min(cap / spp, n_pix));
}

}  // namespace rg

// The allocation-free entry point (see rayna_gpu.h).
extern "C" rg_status rg_render_static_scratch(rg_handle h, uint64_t seed, float* d_accum, uint32_t accum_count,
                                              float* d_out) {
  using namespace rg;
  if (!h) return RG_INVALID_ARG;
  if (!d_accum || accum_count == 0)
    return set_error(h, RG_INVALID_ARG, "rg_render_static_scratch: d_accum must be a device buffer and accum_count >= 1");
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return set_error(h, RG_CUDA_ERROR, cudaGetErrorString(e));
  if (!h->cam_ok) return set_error(h, RG_INVALID_CAMERA, "camera viewport could not be calculated");
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
  if ((e = cudaMemsetAsync(h->d_counters, 0, CNT_N * sizeof(unsigned long long), h->stream)) != cudaSuccess)
    return set_error(h, RG_CUDA_ERROR, cudaGetErrorString(e));
  if ((e = launch_wavefront_static(h, fp)) != cudaSuccess) {
    cudaGetLastError();
    return set_error(h, RG_CUDA_ERROR, cudaGetErrorString(e));
  }
  return RG_OK;
}

namespace rg {

void free_extra(rg_renderer* h) {
  if (h->wf.arena) cudaFree(h->wf.arena);
  h->wf = WavefrontState{};
}

void on_scene_changed(rg_renderer* h) { (void)h; }

}  // namespace rg
