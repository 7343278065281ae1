// oracle_capi.cpp — TEST INFRASTRUCTURE ONLY: C entry points of the CPU
// oracle (rayna_oracle.hpp) for the parity tests and the CPU baseline.
#include <chrono>
#include <cstdio>

#include "rayna_oracle.hpp"

using namespace orc;

namespace {

template <class P>
void fill_hit(const Hit<typename P::T>& h, bool hit, rg_hit* o, double* t64, double* n64) {
  std::memset(o, 0, sizeof(*o));
  o->hit = hit ? 1u : 0u;
  if (!hit) return;
  o->prim = h.prim;
  o->t = (float)h.dist;
  o->normal[0] = (float)h.normal.x; o->normal[1] = (float)h.normal.y; o->normal[2] = (float)h.normal.z;
  o->ray_normal[0] = (float)h.ray_normal.x; o->ray_normal[1] = (float)h.ray_normal.y; o->ray_normal[2] = (float)h.ray_normal.z;
  o->front_face = h.front_face ? 1u : 0u;
  o->material = h.material;
  o->side = h.side;
  if (t64) *t64 = (double)h.dist;
  if (n64) { n64[0] = (double)h.normal.x; n64[1] = (double)h.normal.y; n64[2] = (double)h.normal.z; }
}

template <class P>
int query_impl(const rg_scene_desc* d, int pretest, uint32_t n, const float* o, const float* dir, const float* tmin,
               const float* tmax, const float* vol_u, rg_hit* out, double* t64, double* n64) {
  using T = typename P::T;
  Scene<P> sc;
  Options opt;
  opt.prim_pretest = pretest == 1;
  opt.brute_force = pretest == 2;
  sc.load(*d, opt);
  for (uint32_t i = 0; i < n; ++i) {
    Ray<P> r = Ray<P>::make({(T)o[3 * i], (T)o[3 * i + 1], (T)o[3 * i + 2]}, {(T)dir[3 * i], (T)dir[3 * i + 1], (T)dir[3 * i + 2]});
    Interval<T> iv = Interval<T>::range((T)tmin[i], (T)tmax[i]);
    PathRng rng(true, 0, i, 0);
    rng.injected_volume_u = vol_u ? vol_u + (size_t)i * d->n_volumes : nullptr;
    Hit<T> h;
    bool hit = sc.intersect(r, iv, rng, 0, h);
    fill_hit<P>(h, hit, out + i, t64 ? t64 + i : nullptr, n64 ? n64 + 3 * i : nullptr);
  }
  return 0;
}

// Renders the window [x0, x0 + ww) x [y0, y0 + wh) of the W x H frame (the
// same pixels, samples and random streams as in the whole frame), samples
// [s0, s0 + ns) of each pixel's opts->samples (ns 0: all), `frames` frames.
// out_mean / out_var are ww x wh x 3, [x][y][rgb] within the window.
template <class P>
int render_impl(const rg_scene_desc* d, const rg_camera* cam, const rg_render_opts* opts, uint64_t seed, uint32_t frames,
                int gpu_sampling, int threads, uint32_t x0, uint32_t y0, uint32_t ww, uint32_t wh, uint32_t s0,
                uint32_t ns, double* out_mean, double* out_var, double* out_seconds) {
  Viewport vp;
  if (!calculate_viewport(*cam, vp)) return RG_INVALID_CAMERA;
  if (opts->width == 0 || opts->height == 0 || opts->samples == 0 || opts->ray_branching == 0) return RG_INVALID_ARG;
  if (opts->mode > RG_MODE_SIDE) return RG_UNSUPPORTED_VARIANT;
  const uint32_t W = opts->width, H = opts->height;
  if (ww == 0 || wh == 0 || (uint64_t)x0 + ww > W || (uint64_t)y0 + wh > H) return RG_INVALID_ARG;
  if (ns == 0) { s0 = 0; ns = opts->samples; }
  if ((uint64_t)s0 + ns > opts->samples) return RG_INVALID_ARG;
  Scene<P> sc;
  sc.load(*d, Options{});
  std::vector<double> sum((size_t)ww * wh * 3, 0.0), sq((size_t)ww * wh * 3, 0.0);
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  auto t0 = std::chrono::steady_clock::now();
  for (uint32_t f = 0; f < frames; ++f) {
    uint64_t fseed = seed + (uint64_t)f * 0x9E3779B97F4A7C15ull;
    RenderParams rp{W, H, opts->samples, opts->ray_depth, fseed};
    rp.mode = opts->mode;
    rp.branching = opts->ray_branching;
    Renderer<P> R(sc, vp, rp);
    std::atomic<uint32_t> next_row{0};
    auto work = [&]() {
      for (;;) {
        uint32_t yy = next_row.fetch_add(1);
        if (yy >= wh) break;
        const uint32_t y = y0 + yy;
        for (uint32_t xx = 0; xx < ww; ++xx) {
          const uint32_t x = x0 + xx;
          SeqRng msaa(fseed, y * W + x, 0xFFFFFFFFu, 0x4d5341u);
          size_t o = ((size_t)xx * wh + yy) * 3;
          for (uint32_t s = s0; s < s0 + ns; ++s) {
            C3 c = R.sample(x, y, s, gpu_sampling != 0, &msaa);
            double v[3] = {c.r, c.g, c.b};
            for (int k = 0; k < 3; ++k) { sum[o + k] += v[k]; sq[o + k] += v[k] * v[k]; }
          }
        }
      }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
  }
  auto t1 = std::chrono::steady_clock::now();
  if (out_seconds) *out_seconds = std::chrono::duration<double>(t1 - t0).count();
  const double N = (double)frames * ns;
  for (size_t i = 0; i < sum.size(); ++i) {
    double m = sum[i] / N;
    if (out_mean) out_mean[i] = m;
    if (out_var) out_var[i] = N > 1 ? std::max(0.0, (sq[i] - N * m * m) / (N - 1)) : 0.0;
  }
  return RG_OK;
}

template <class P>
int backward_impl(const rg_scene_desc* d, const rg_camera* cam, const rg_render_opts* opts, uint64_t seed, int threads,
                  const float* target, const float* adjoint, double* g_alb, double* g_em, double* g_den, double* loss) {
  Viewport vp;
  if (!calculate_viewport(*cam, vp)) return RG_INVALID_CAMERA;
  const uint32_t W = opts->width, H = opts->height;
  const size_t n3 = (size_t)W * H * 3;
  std::vector<double> delta(n3, 0.0);
  double l = 0.0;
  if (target) {
    std::vector<double> img(n3);
    int st = render_impl<P>(d, cam, opts, seed, 1, 1, threads, 0, 0, W, H, 0, 0, img.data(), nullptr, nullptr);
    if (st != RG_OK) return st;
    for (size_t i = 0; i < n3; ++i) {
      double e = img[i] - (double)target[i];
      delta[i] = 2.0 * e;
      l += e * e;
    }
  } else {
    for (size_t i = 0; i < n3; ++i) delta[i] = adjoint[i];
  }
  Scene<P> sc;
  sc.load(*d, Options{});
  RenderParams rp{W, H, opts->samples, opts->ray_depth, seed};
  Renderer<P> R(sc, vp, rp);
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  const size_t nm = sc.materials.size();
  std::vector<typename Renderer<P>::Grad> grads(threads);
  for (auto& g : grads) { g.alb.assign(nm * 3, 0.0); g.em.assign(nm * 3, 0.0); g.den.assign(sc.nv, 0.0); }
  std::atomic<uint32_t> next_row{0};
  auto work = [&](int t) {
    for (;;) {
      uint32_t y = next_row.fetch_add(1);
      if (y >= H) break;
      for (uint32_t x = 0; x < W; ++x) {
        const double* dl = delta.data() + ((size_t)x * H + y) * 3;
        for (uint32_t s = 0; s < opts->samples; ++s) R.adjoint_sample(x, y, s, dl, grads[t]);
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& t : pool) t.join();
  for (size_t i = 0; i < nm * 3; ++i) {
    g_alb[i] = 0.0;
    g_em[i] = 0.0;
    for (auto& g : grads) { g_alb[i] += g.alb[i]; g_em[i] += g.em[i]; }
  }
  for (uint32_t v = 0; v < sc.nv; ++v) {
    g_den[v] = 0.0;
    for (auto& g : grads) g_den[v] += g.den[v];
  }
  if (loss) *loss = l;
  return RG_OK;
}

}  // namespace

// The colour each ray sees at its closest hit: the hit material's texture
// value (or solid albedo; a light's emission), or the sky on a miss. For
// known-answer tests of textures and skies.
template <class P>
int query_colour_impl(const rg_scene_desc* d, uint32_t n, const float* o, const float* dir, float* rgb) {
  using T = typename P::T;
  Scene<P> sc;
  sc.load(*d, Options{});
  for (uint32_t i = 0; i < n; ++i) {
    Ray<P> r = Ray<P>::make({(T)o[3 * i], (T)o[3 * i + 1], (T)o[3 * i + 2]}, {(T)dir[3 * i], (T)dir[3 * i + 1], (T)dir[3 * i + 2]});
    Interval<T> iv = Interval<T>::range(T(1e-3), std::numeric_limits<T>::max());
    PathRng rng(true, 0, i, 0);
    Hit<T> h;
    const C3 c = sc.intersect(r, iv, rng, 0, h) ? sc.colour(sc.materials[h.material], h) : sky_of<P>(sc, r);
    rgb[3 * i] = c.r;
    rgb[3 * i + 1] = c.g;
    rgb[3 * i + 2] = c.b;
  }
  return 0;
}

extern "C" {

// Path-replay adjoint on the CPU (device sampler assignment). policy 0 = f64,
// 1 = f32. With `target` the loss is sum (I - target)^2 for the frame `seed`;
// otherwise `adjoint` is dLoss/dI. Gradients in double.
int orc_backward(const rg_scene_desc* d, const rg_camera* cam, const rg_render_opts* opts, uint64_t seed, int policy,
                 int threads, const float* target, const float* adjoint, double* g_alb, double* g_em, double* g_den,
                 double* loss) {
  if (policy == 0) return backward_impl<RefF64>(d, cam, opts, seed, threads, target, adjoint, g_alb, g_em, g_den, loss);
  return backward_impl<GpuF32>(d, cam, opts, seed, threads, target, adjoint, g_alb, g_em, g_den, loss);
}

// Philox4x32-10 known-answer access.
void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  U4 r = philox4x32_10(U4{{ctr[0], ctr[1], ctr[2], ctr[3]}}, key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}

// Camera::calculate_viewport in f64; out = pos, pixel_center, viewport_u,
// viewport_v, defocus_u, defocus_v (18 doubles). Returns RG_INVALID_CAMERA on Err.
int orc_viewport(const rg_camera* cam, double* out) {
  Viewport vp;
  if (!calculate_viewport(*cam, vp)) return RG_INVALID_CAMERA;
  std::memcpy(out, &vp, sizeof(vp));
  return RG_OK;
}

// Closest-hit queries. policy 0 = RefF64, 1 = GpuF32. `structure` 1 follows
// the reference's BVH with its per-object Aabb test before each leaf object,
// 0 the same BVH without that test, 2 no bounding volumes at all.
int orc_query(const rg_scene_desc* d, int policy, int pretest, uint32_t n, const float* o, const float* dir,
              const float* tmin, const float* tmax, const float* vol_u, rg_hit* out, double* t64, double* n64) {
  if (policy == 0) return query_impl<RefF64>(d, pretest, n, o, dir, tmin, tmax, vol_u, out, t64, n64);
  return query_impl<GpuF32>(d, pretest, n, o, dir, tmin, tmax, vol_u, out, t64, n64);
}

// Renders `frames` frames of opts->samples samples per pixel and returns the
// per-pixel mean and unbiased sample variance over all samples ([x][y][rgb]).
// policy 0 = RefF64 with the reference samplers; 1 = GpuF32 with the device
// samplers and counter assignment (gpu_sampling is then forced on).
int orc_render(const rg_scene_desc* d, const rg_camera* cam, const rg_render_opts* opts, uint64_t seed, uint32_t frames,
               int policy, int gpu_sampling, int threads, double* out_mean, double* out_var, double* out_seconds) {
  const uint32_t W = opts->width, H = opts->height;
  if (policy == 0)
    return render_impl<RefF64>(d, cam, opts, seed, frames, gpu_sampling, threads, 0, 0, W, H, 0, 0, out_mean, out_var,
                               out_seconds);
  return render_impl<GpuF32>(d, cam, opts, seed, frames, 1, threads, 0, 0, W, H, 0, 0, out_mean, out_var, out_seconds);
}

// orc_render over the window [x0, x0 + ww) x [y0, y0 + wh) of the frame and
// the samples [s0, s0 + ns) of each pixel (ns 0: all); the outputs are
// ww x wh x 3, the mean and variance over the window's traced samples.
int orc_render_window(const rg_scene_desc* d, const rg_camera* cam, const rg_render_opts* opts, uint64_t seed,
                      uint32_t frames, int policy, int gpu_sampling, int threads, uint32_t x0, uint32_t y0, uint32_t ww,
                      uint32_t wh, uint32_t s0, uint32_t ns, double* out_mean, double* out_var, double* out_seconds) {
  if (policy == 0)
    return render_impl<RefF64>(d, cam, opts, seed, frames, gpu_sampling, threads, x0, y0, ww, wh, s0, ns, out_mean, out_var,
                               out_seconds);
  return render_impl<GpuF32>(d, cam, opts, seed, frames, 1, threads, x0, y0, ww, wh, s0, ns, out_mean, out_var,
                             out_seconds);
}

int orc_query_colour(const rg_scene_desc* d, int policy, uint32_t n, const float* o, const float* dir, float* rgb) {
  if (policy == 0) return query_colour_impl<RefF64>(d, n, o, dir, rgb);
  return query_colour_impl<GpuF32>(d, n, o, dir, rgb);
}

int orc_hardware_threads(void) { return (int)std::thread::hardware_concurrency(); }

// The f32 policy's (and the device's) natural logarithm over an array.
void orc_ln_f32(const float* x, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) out[i] = ln_f32(x[i]);
}

}  // extern "C"
