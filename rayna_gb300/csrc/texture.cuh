// Non-solid textures and the image sky (the extended kernel variant only).
//
// Texture::value (texture/mod.rs:21-24) for the checker, image and noise
// textures, Image::get_bilinear (core/image.rs:87-109) and HdrImageSkybox
// (skybox/hdri.rs:17-26). All arithmetic in f32 with the operation order
// written here (the oracle's GpuF32 policy follows it).
#pragma once

namespace rg {

// Image::bilinear_coords (core/image.rs:89-95): floor and ceil clamped to the
// image, the fraction taken against the clamped floor.
__device__ __forceinline__ void bilinear_coords(float val, uint32_t max, uint32_t& lo, uint32_t& hi, float& frac) {
  const float top = (float)(max - 1u);
  // fmaxf first: a NaN coordinate maps to texel 0, as Rust's `NaN as usize` does.
  const float fl = fminf(fmaxf(floorf(val), 0.0f), top);
  const float ce = fminf(fmaxf(ceilf(val), 0.0f), top);
  lo = (uint32_t)fl;
  hi = (uint32_t)ce;
  frac = val - fl;
}

__device__ __forceinline__ C3f lerp3(C3f a, C3f b, float t) {
  return C3f{a.r + (b.r - a.r) * t, a.g + (b.g - a.g) * t, a.b + (b.b - a.b) * t};
}

__device__ __forceinline__ C3f texel(const GpuScene& sc, const GpuImage& im, uint32_t x, uint32_t y) {
  const float4 t = __ldg(sc.texels + im.first + (size_t)x * im.height + y);
  return C3f{t.x, t.y, t.z};
}

// Image::get_bilinear (core/image.rs:97-109): interpolate along x at both
// rows, then along y.
__device__ __forceinline__ C3f image_bilinear(const GpuScene& sc, uint32_t image, float px, float py) {
  const GpuImage im = sc.images[image];
  uint32_t x1, x2, y1, y2;
  float xl, yl;
  bilinear_coords(px, im.width, x1, x2, xl);
  bilinear_coords(py, im.height, y1, y2, yl);
  const C3f c11 = texel(sc, im, x1, y1), c12 = texel(sc, im, x1, y2);
  const C3f c21 = texel(sc, im, x2, y1), c22 = texel(sc, im, x2, y2);
  return lerp3(lerp3(c11, c21, xl), lerp3(c12, c22, xl), yl);
}

// Improved Perlin noise (K. Perlin, "Improving Noise", SIGGRAPH 2002): the
// quintic fade, the twelve edge gradients (four repeated) picked by the low
// four hash bits, trilinear blending. `perm` holds 512 entries (a
// permutation of 0..255, repeated).
__device__ __forceinline__ float perlin_fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
__device__ __forceinline__ float perlin_lerp(float t, float a, float b) { return a + t * (b - a); }
__device__ __forceinline__ float perlin_grad(uint32_t h, float x, float y, float z) {
  h &= 15u;
  const float u = h < 8u ? x : y;
  const float v = h < 4u ? y : (h == 12u || h == 14u ? x : z);
  return ((h & 1u) ? -u : u) + ((h & 2u) ? -v : v);
}
__device__ __forceinline__ float perlin3(const uint8_t* perm, float x, float y, float z) {
  const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
  // __float2int_rz saturates (and maps NaN to 0): defined for any coordinate
  const uint32_t X = (uint32_t)__float2int_rz(fx) & 255u, Y = (uint32_t)__float2int_rz(fy) & 255u,
                 Z = (uint32_t)__float2int_rz(fz) & 255u;
  x = x - fx;
  y = y - fy;
  z = z - fz;
  const float u = perlin_fade(x), v = perlin_fade(y), w = perlin_fade(z);
  auto P = [&](uint32_t i) { return (uint32_t)__ldg(perm + i); };
  const uint32_t A = P(X) + Y, AA = P(A) + Z, AB = P(A + 1u) + Z;
  const uint32_t B = P(X + 1u) + Y, BA = P(B) + Z, BB = P(B + 1u) + Z;
  return perlin_lerp(w,
                     perlin_lerp(v, perlin_lerp(u, perlin_grad(P(AA), x, y, z), perlin_grad(P(BA), x - 1.0f, y, z)),
                                 perlin_lerp(u, perlin_grad(P(AB), x, y - 1.0f, z),
                                             perlin_grad(P(BB), x - 1.0f, y - 1.0f, z))),
                     perlin_lerp(v,
                                 perlin_lerp(u, perlin_grad(P(AA + 1u), x, y, z - 1.0f),
                                             perlin_grad(P(BA + 1u), x - 1.0f, y, z - 1.0f)),
                                 perlin_lerp(u, perlin_grad(P(AB + 1u), x, y - 1.0f, z - 1.0f),
                                             perlin_grad(P(BB + 1u), x - 1.0f, y - 1.0f, z - 1.0f))));
}

// rem_euclid(sum, 2) < 1 (num_traits::Euclid for floats), as do_checker
// (texture/checker.rs:46-63) decides the even cells.
__device__ __forceinline__ bool checker_even(float sum) {
  float r = fmodf(sum, 2.0f);
  if (r < 0.0f) r = r + 2.0f;
  return r < 1.0f;
}

// Texture::value of texture `t` at a hit (world point, mesh-local point,
// uv). Checkers descend into their cells' textures (an acyclic table, at most
// RG_MAX_TEXTURE_DEPTH deep, as the host checks).
static __device__ __noinline__ C3f texture_value(const GpuScene& sc, uint32_t t, V3 pos, V3 pos_l, float u, float v) {
  for (uint32_t level = 0; level <= RG_MAX_TEXTURE_DEPTH; ++level) {
    const rg_texture& tx = sc.textures[t];
    switch (tx.kind) {
      case RG_TEX_WORLD_CHECKER: {
        const float sc0 = tx.scale[0];
        const float sum = ((0.0f + floorf(pos.x / sc0 + tx.offset[0])) + floorf(pos.y / sc0 + tx.offset[1])) +
                          floorf(pos.z / sc0 + tx.offset[2]);
        t = checker_even(sum) ? tx.even : tx.odd;
        continue;
      }
      case RG_TEX_UV_CHECKER: {
        const float sc0 = tx.scale[0];
        const float sum = (0.0f + floorf(u / sc0 + tx.offset[0])) + floorf(v / sc0 + tx.offset[1]);
        t = checker_even(sum) ? tx.even : tx.odd;
        continue;
      }
      case RG_TEX_IMAGE: {
        // ImageTexture::value (texture/image.rs:29-39)
        const float tu = tx.offset[0] + u * tx.scale[0];
        const float tv = tx.offset[1] + v * tx.scale[1];
        const GpuImage im = sc.images[tx.image];
        return image_bilinear(sc, tx.image, tu * (float)im.width, (1.0f - tv) * (float)im.height);
      }
      case RG_TEX_NOISE: {
        // ColourSource::get (texture/noise.rs): value / 2 + 0.5 per channel,
        // the point scaled first (ScalePoint)
        V3 q = tx.noise_place == RG_NOISE_WORLD ? pos : (tx.noise_place == RG_NOISE_LOCAL ? pos_l : v3(u, v, 0.0f));
        const float k = tx.scale[0];
        q = v3(q.x * k, q.y * k, q.z * k);
        const uint8_t* perm = sc.perm + 512ull * tx.image;
        const float g = perlin3(perm, q.x, q.y, q.z);
        if (tx.noise_channels == 1u) {
          const float c = g / 2.0f + 0.5f;
          return C3f{c, c, c};
        }
        const float gg = perlin3(perm + 512, q.x, q.y, q.z), gb = perlin3(perm + 1024, q.x, q.y, q.z);
        return C3f{g / 2.0f + 0.5f, gg / 2.0f + 0.5f, gb / 2.0f + 0.5f};
      }
      default:  // RG_TEX_SOLID
        return C3f{tx.colour[0], tx.colour[1], tx.colour[2]};
    }
  }
  return C3f{0.0f, 0.0f, 0.0f};  // unreachable for a validated table
}

// The material's colour at the hit: its texture, or the solid albedo.
template <uint32_t F>
__device__ __forceinline__ C3f material_colour(const GpuScene& sc, const rg_material& m, const Surface& s) {
  if ((F & F_EXT) && m.texture != 0u) return texture_value(sc, m.texture - 1u, s.pos, s.pos_l, s.u, s.v);
  return C3f{m.albedo[0], m.albedo[1], m.albedo[2]};
}

}  // namespace rg
