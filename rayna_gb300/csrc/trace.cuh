// trace.cuh — per-ray device code shared by every kernel form: camera rays,
// closest-hit traversal of the binary BVH, the primitive tests, media,
// sphere-traced SDFs, materials and the sky.
//
// Arithmetic contract: the library is compiled with -fmad=false, so every
// fused multiply-add below is written out (__fmaf_rn) and every other
// operation is a separately rounded IEEE op. With the same contract on the
// host (-ffp-contract=off + explicit fma) the CPU oracle reproduces the
// closed-form intersections bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "gpu_scene.h"

namespace rg {

// ---------------------------------------------------------------------------
// Vector arithmetic
// ---------------------------------------------------------------------------
struct V3 { float x, y, z; };
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 xyz(float4 f) { return v3(f.x, f.y, f.z); }

// dot = fma(x, x', fma(y, y', z*z'))
__device__ __forceinline__ float dot3(V3 a, V3 b) { return __fmaf_rn(a.x, b.x, __fmaf_rn(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
  return v3(__fmaf_rn(a.y, b.z, -(a.z * b.y)), __fmaf_rn(a.z, b.x, -(a.x * b.z)), __fmaf_rn(a.x, b.y, -(a.y * b.x)));
}
// Ray::at: pos + dir * t
__device__ __forceinline__ V3 at3(V3 o, V3 d, float t) { return v3(__fmaf_rn(d.x, t, o.x), __fmaf_rn(d.y, t, o.y), __fmaf_rn(d.z, t, o.z)); }
__device__ __forceinline__ float length3(V3 v) { return __fsqrt_rn(dot3(v, v)); }
// glam normalize / try_normalize: v * (1 / |v|)
__device__ __forceinline__ V3 normalize3(V3 v) { return v * __frcp_rn(length3(v)); }
__device__ __forceinline__ bool try_normalize3(V3 v, V3& out) {
  float r = __frcp_rn(length3(v));
  if (isfinite(r) && r > 0.0f) { out = v * r; return true; }
  return false;
}
__device__ __forceinline__ float signumf(float x) { return isnan(x) ? x : copysignf(1.0f, x); }

// Natural logarithm, written out so that the oracle's f32 policy evaluates
// the same operations (its own ln_f32) and the free-flight distances and the
// Mandelbulb's distance bit for bit alike: x = m 2^e with m in [sqrt(1/2),
// sqrt(2)), ln m = 2 atanh(s) = 2 (s + s^3/3 + ... + s^9/9) with s = (m - 1) /
// (m + 1), |s| < 0.172 (the series of Abramowitz & Stegun 4.1.27; the
// truncation is below 1e-9), and e ln 2 in two parts. Error within 3 ulp of
// the exact logarithm over the normal and subnormal range (the roundings of s
// and of the series); 0 gives -inf,
// negative values NaN, +inf itself.
__device__ __forceinline__ float ln_f32(float x) {
  if (!(x > 0.0f)) return x == 0.0f ? -CUDART_INF_F : CUDART_NAN_F;
  if (isinf(x)) return x;
  int e = 0;
  if (x < 1.17549435e-38f) { x = __fmul_rn(x, 8388608.0f); e = -23; }  // subnormal: scale by 2^23
  const uint32_t bits = __float_as_uint(x);
  e += (int)((bits >> 23) & 0xFFu) - 127;
  float m = __uint_as_float((bits & 0x7FFFFFu) | 0x3F800000u);
  if (m > 1.41421356f) { m = __fmul_rn(m, 0.5f); e += 1; }
  const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float s2 = __fmul_rn(s, s);
  float p = __fmaf_rn(s2, 0.111111111f, 0.142857143f);
  p = __fmaf_rn(s2, p, 0.2f);
  p = __fmaf_rn(s2, p, 0.333333333f);
  p = __fmaf_rn(s2, p, 1.0f);
  const float lm = __fmul_rn(__fmul_rn(2.0f, s), p);
  const float fe = (float)e;
  return __fmaf_rn(fe, 0.693145751953125f, __fmaf_rn(fe, 1.42860676533018e-06f, lm));
}

// ---------------------------------------------------------------------------
// Philox4x32-10 counter-based random numbers (Salmon et al., SC'11).
// Block (pixel, sample, depth, purpose) keyed by the frame seed.
// ---------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };
__device__ __forceinline__ U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return U4{c0, c1, c2, c3};
}
__device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }
__device__ __forceinline__ float u01_open0(uint32_t x) { return ((float)(x >> 8) + 1.0f) * (1.0f / 16777216.0f); }

enum : uint32_t { kPurposeCamera = 0, kPurposeScatter = 1, kPurposeVolume0 = 2 };
constexpr uint32_t kCameraDepth = 0xFFFFFFFFu;

struct RngCtx {
  uint32_t k0, k1, pix, smp, depth;
  const float* vol_u;  // injected free-flight uniforms (ray queries) or null
  __device__ __forceinline__ U4 block(uint32_t purpose) const { return philox(pix, smp, depth, purpose, k0, k1); }
};

// normal_on_unit_sphere (rayna_engine/src/shared/rng.rs:75-87)
__device__ __forceinline__ V3 unit_sphere_from(float r1, float r2) {
  const float two_pi = (float)(2.0 * 3.14159265358979323846);
  float s = 2.0f * __fsqrt_rn(r2 * (1.0f - r2));
  return v3(cosf(two_pi * r1) * s, sinf(two_pi * r1) * s, 1.0f - 2.0f * r2);
}

// ---------------------------------------------------------------------------
// Rays
// ---------------------------------------------------------------------------
struct Ray {
  V3 o, d, inv;
};
// Ray::new (rayna_engine/src/shared/ray.rs:15-23)
__device__ __forceinline__ Ray make_ray(V3 o, V3 dir) {
  Ray r;
  r.o = o;
  r.d = normalize3(dir);
  r.inv = v3(__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z));
  return r;
}

// Relative slack that makes the slab test conservative: the computed entry
// and exit distances (b - o) * inv carry at most a few units of roundoff, so
// widening the exit side by 2^-20 relative never rejects a box the ray
// meets inside [start, end] (Ize, "Robust BVH Ray Traversal", JCGT 2013).
// Bounding boxes therefore never change which primitive is closest: the
// result equals the closest hit of the primitive tests alone.
constexpr float kSlabSlack = 9.5367431640625e-7f;  // 2^-20

// Aabb::hit (rayna_engine/src/shared/aabb.rs:117-153) against [start, end];
// returns the entry distance in `tnear`.
__device__ __forceinline__ bool slab(float lx, float hx, float ly, float hy, float lz, float hz, const Ray& r, float start,
                                     float end, float& tnear) {
  float t1x = (lx - r.o.x) * r.inv.x, t2x = (hx - r.o.x) * r.inv.x;
  float t1y = (ly - r.o.y) * r.inv.y, t2y = (hy - r.o.y) * r.inv.y;
  float t1z = (lz - r.o.z) * r.inv.z, t2z = (hz - r.o.z) * r.inv.z;
  float tmin = fmaxf(fmaxf(fminf(t1x, t2x), fminf(t1y, t2y)), fminf(t1z, t2z));
  float tmax = fminf(fminf(fmaxf(t1x, t2x), fmaxf(t1y, t2y)), fmaxf(t1z, t2z));
  float low = fmaxf(tmin, start), high = fminf(tmax, end);
  tnear = low;
  return low <= __fmaf_rn(fabsf(high), kSlabSlack, high);
}

// ---------------------------------------------------------------------------
// Primitive tests. Each returns the hit distance through `t` when it hits
// inside [start, end]. Full hit records are built once, for the closest hit.
// ---------------------------------------------------------------------------
// SphereMesh::intersect (mesh/primitive/sphere.rs:44-99): the roots
// -half_b -/+ sqrt(disc) of |oc + t d|^2 = r^2, the near one first, each
// tested against [start, end]. In f32 the reference's disc = half_b^2 - c
// cancels catastrophically for a small, distant sphere (both terms near
// |oc|^2); for a unit d it equals r^2 - |l|^2 with l = oc - half_b d, the
// centre-to-line vector, which does not. The roots are q = -(half_b +
// sign(half_b) sqrt(disc)) and c / q (Vieta), so neither subtracts nearly
// equal terms (Haines, Guenther, Akenine-Moller, "Precision Improvements for
// Ray/Sphere Intersection", Ray Tracing Gems, 2019).
__device__ __forceinline__ bool sphere_t(V3 c, float r2, const Ray& r, float start, float end, float& t) {
  const V3 oc = r.o - c;
  const float half_b = dot3(oc, r.d);
  const V3 l = v3(__fmaf_rn(-half_b, r.d.x, oc.x), __fmaf_rn(-half_b, r.d.y, oc.y), __fmaf_rn(-half_b, r.d.z, oc.z));
  const float disc = r2 - dot3(l, l);
  if (disc < 0.0f) return false;
  const float cc = __fmaf_rn(oc.x, oc.x, __fmaf_rn(oc.y, oc.y, __fmaf_rn(oc.z, oc.z, -r2)));
  const float sq = __fsqrt_rn(disc);
  const float q = half_b > 0.0f ? -half_b - sq : -half_b + sq;
  const float other = q != 0.0f ? __fdiv_rn(cc, q) : q;
  float root = fminf(q, other);
  if (!(start <= root && root <= end)) {
    root = fmaxf(q, other);
    if (!(start <= root && root <= end)) return false;
  }
  t = root;
  return true;
}

// Triangle::intersect (mesh/primitive/triangle.rs:53-109), Moller-Trumbore
// with precomputed edges e1 = v1 - v0, e2 = v2 - v0. Outputs u, v, det.
__device__ __forceinline__ bool triangle_t(V3 v0, V3 e1, V3 e2, const Ray& r, float start, float end, float& t, float& u,
                                           float& v, float& det) {
  V3 pvec = cross3(r.d, e2);
  det = dot3(e1, pvec);
  if (det == 0.0f) return false;
  float inv_det = __frcp_rn(det);
  V3 tvec = r.o - v0;
  u = dot3(tvec, pvec) * inv_det;
  if (u < 0.0f || u > 1.0f) return false;
  V3 qvec = cross3(tvec, e1);
  v = dot3(r.d, qvec) * inv_det;
  if (v < 0.0f || u + v > 1.0f) return false;
  t = dot3(e2, qvec) * inv_det;
  return start <= t && t <= end;
}

// Triangle::interpolate_normals (triangle.rs:114-119): fold from zero.
__device__ __forceinline__ bool tri_normal(const float* n9, float u, float v, V3& out) {
  float b0 = (1.0f - u) - v;
  V3 n0 = v3(__ldg(n9 + 0), __ldg(n9 + 1), __ldg(n9 + 2));
  V3 n1 = v3(__ldg(n9 + 3), __ldg(n9 + 4), __ldg(n9 + 5));
  V3 n2 = v3(__ldg(n9 + 6), __ldg(n9 + 7), __ldg(n9 + 8));
  V3 n = v3(__fmaf_rn(n2.x, v, __fmaf_rn(n1.x, u, n0.x * b0)), __fmaf_rn(n2.y, v, __fmaf_rn(n1.y, u, n0.y * b0)),
            __fmaf_rn(n2.z, v, __fmaf_rn(n1.z, u, n0.z * b0)));
  return try_normalize3(n, out);
}

struct BoxHit { float t; int axis; float u0, u1; float winding; float sgn; };

// AxisBoxMesh::intersect (mesh/primitive/axis_box.rs:64-145), Majercik et al. 2018.
__device__ __forceinline__ bool box_t(V3 centre, V3 radius, V3 inv_radius, const Ray& r, float start, float end, BoxHit& bh) {
  V3 ro = r.o - centre;
  V3 rd = r.d;
  float qx = fabsf(ro.x) * inv_radius.x, qy = fabsf(ro.y) * inv_radius.y, qz = fabsf(ro.z) * inv_radius.z;
  float winding = signumf(fmaxf(qx, fmaxf(qy, qz)) - 1.0f);
  V3 sgn = v3(-signumf(rd.x), -signumf(rd.y), -signumf(rd.z));
  float pd[3] = {((radius.x * winding) * sgn.x - ro.x) * r.inv.x, ((radius.y * winding) * sgn.y - ro.y) * r.inv.y,
                 ((radius.z * winding) * sgn.z - ro.z) * r.inv.z};
  float rov[3] = {ro.x, ro.y, ro.z}, rdv[3] = {rd.x, rd.y, rd.z}, rad[3] = {radius.x, radius.y, radius.z};
  float sg[3] = {sgn.x, sgn.y, sgn.z};
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    float dist = pd[ax];
    if (!(start <= dist && dist <= end)) continue;
    int a1 = ax == 0 ? 1 : (ax == 1 ? 2 : 0);
    int a2 = ax == 0 ? 2 : (ax == 1 ? 0 : 1);
    float u0 = __fmaf_rn(rdv[a1], dist, rov[a1]);
    float u1 = __fmaf_rn(rdv[a2], dist, rov[a2]);
    if (fabsf(u0) < rad[a1] && fabsf(u1) < rad[a2]) {
      bh.t = dist; bh.axis = ax; bh.u0 = u0 / rad[a1]; bh.u1 = u1 / rad[a2]; bh.winding = winding; bh.sgn = sg[ax];
      return true;
    }
  }
  return false;
}

__device__ __forceinline__ uint32_t prim_kind(const GpuPrim& p) { return __float_as_uint(p.a.w) >> kKindShift; }
__device__ __forceinline__ uint32_t prim_material(const GpuPrim& p) { return __float_as_uint(p.a.w) & kMaterialMask; }
__device__ __forceinline__ uint32_t prim_id(const GpuPrim& p) { return __float_as_uint(p.b.w); }

// Boundary intersection of a medium with an interval given by [start, end]
// (+-infinity stand for absent bounds).
__device__ __forceinline__ bool boundary_t(const GpuPrim& p, uint32_t kind, const Ray& r, float start, float end, float& t) {
  if (kind == PK_VOL_SPHERE) return sphere_t(xyz(p.a), p.b.y, r, start, end, t);
  BoxHit bh;
  if (!box_t(xyz(p.a), xyz(p.b), xyz(p.c), r, start, end, bh)) return false;
  t = bh.t;
  return true;
}

// VolumetricObject::full_intersect (object/volumetric.rs:86-160).
__device__ __forceinline__ bool volume_t(const GpuPrim& p, uint32_t kind, uint32_t vol_index, const Ray& r, float start,
                                         float end, const RngCtx& ctx, float& t) {
  float d_enter, d_exit;
  if (!boundary_t(p, kind, r, -CUDART_INF_F, CUDART_INF_F, d_enter)) return false;
  float enter = fmaxf(d_enter, start);
  if (!boundary_t(p, kind, r, enter + 0.001f, CUDART_INF_F, d_exit)) return false;
  float exitd = fminf(d_exit, end);
  float inside = exitd - enter;
  float u = ctx.vol_u ? ctx.vol_u[vol_index] : u01_open0(ctx.block(kPurposeVolume0 + vol_index).x);
  float neg_inv_density = kind == PK_VOL_SPHERE ? p.b.z : p.c.w;
  float hit_dist = __fmul_rn(neg_inv_density, ln_f32(u));
  if (hit_dist > inside) return false;
  t = enter + hit_dist;
  return true;
}

// ---------------------------------------------------------------------------
// Signed distance functions (world space) and the sphere tracer.
// ---------------------------------------------------------------------------
constexpr float kBulbInner = 1.2f, kBulbOuter = 1.5f;

// `iter_count`, when given, counts the Mandelbulb's escape-loop iterations
// (work counters). Every multiply-add here is written out (explicit fma, and
// __fmul_rn where a product must not fuse into the caller's subtraction, as in
// the normal's central differences), so the performance build evaluates the
// function exactly as the arithmetic-contract build does, whichever kernel
// inlines it.
__device__ __forceinline__ float sdf_eval(const GpuSdf& s, V3 x, unsigned long long* iter_count = nullptr) {
  V3 q = x - v3(s.cx, s.cy, s.cz);
  if (s.kind == RG_SDF_SPHERE) return length3(q) - s.p0;
  if (s.kind == RG_SDF_TORUS) {
    float a = __fsqrt_rn(__fmaf_rn(q.x, q.x, __fmul_rn(q.z, q.z))) - s.p0;
    return __fsqrt_rn(__fmaf_rn(a, a, __fmul_rn(q.y, q.y))) - s.p1;
  }
  // Mandelbulb distance estimator: z -> z^power + c in spherical coordinates
  // with the running derivative dr; outside kBulbOuter the distance to the
  // enclosing sphere of radius kBulbInner is used (a lower bound).
  unsigned long long* counted = iter_count;
  float sc = s.p2;
  // q / scale; for a power-of-two scale the product with its reciprocal is
  // the same correctly rounded quotient, without three divisions
  V3 z0 = s.inv_scale != 0.0f ? v3(__fmul_rn(q.x, s.inv_scale), __fmul_rn(q.y, s.inv_scale), __fmul_rn(q.z, s.inv_scale))
                              : v3(q.x / sc, q.y / sc, q.z / sc);
  float rq = length3(z0);
  if (rq > kBulbOuter) return __fmul_rn(rq - kBulbInner, sc);
  float power = s.p0;
  int iters = (int)s.p1;
  V3 z = z0;
  float dr = 1.0f, rr = 0.0f;
  if (power == 8.0f) {
    // z^8 without transcendentals or per-iteration normalisation of the polar
    // angle: with w = z + i rho (|w| = r, arg w = t) three complex squarings
    // give w^8 = r^8 (cos 8t + i sin 8t); the azimuth's unit complex number
    // (x + i y) / rho, squared three times, gives cos 8p + i sin 8p. One
    // division and two square roots per iteration.
    for (int i = 0; i < iters; ++i) {
      if (counted) ++*counted;
      float rho2 = __fmaf_rn(z.x, z.x, __fmul_rn(z.y, z.y));
      float r2 = __fmaf_rn(z.z, z.z, rho2);
      rr = __fsqrt_rn(r2);
      if (rr > 2.0f) break;
      float rho = __fsqrt_rn(rho2);
      float wa = z.z, wb = rho, cp = 1.0f, sp = 0.0f;
      if (rho > 0.0f) {
        const float inv = __fdiv_rn(1.0f, rho);
        cp = __fmul_rn(z.x, inv);
        sp = __fmul_rn(z.y, inv);
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        float a2 = __fmaf_rn(wa, wa, -__fmul_rn(wb, wb));
        wb = __fmul_rn(2.0f * wa, wb);
        wa = a2;
        float d2 = __fmaf_rn(cp, cp, -__fmul_rn(sp, sp));
        sp = __fmul_rn(2.0f * cp, sp);
        cp = d2;
      }
      float r4 = __fmul_rn(r2, r2);
      dr = __fmaf_rn(__fmul_rn(__fmul_rn(__fmul_rn(r4, r2), rr), 8.0f), dr, 1.0f);
      z = v3(__fmaf_rn(wb, cp, z0.x), __fmaf_rn(wb, sp, z0.y), __fadd_rn(wa, z0.z));
    }
  } else {
    for (int i = 0; i < iters; ++i) {
      rr = length3(z);
      if (rr > 2.0f) break;
      float theta = acosf(z.z / rr);
      float phi = atan2f(z.y, z.x);
      dr = __fmaf_rn(__fmul_rn(powf(rr, power - 1.0f), power), dr, 1.0f);
      float zr = powf(rr, power);
      theta = theta * power;
      phi = phi * power;
      float st = sinf(theta);
      z = v3(__fmaf_rn(zr, __fmul_rn(st, cosf(phi)), z0.x), __fmaf_rn(zr, __fmul_rn(sinf(phi), st), z0.y),
             __fmaf_rn(zr, cosf(theta), z0.z));
    }
  }
  return __fmul_rn(__fdiv_rn(__fmul_rn(__fmul_rn(0.5f, ln_f32(rr)), rr), dr), sc);
}

// Planar::intersect_bounded (mesh/planar/mod.rs:161-194): the distance to
// the plane n.x + d = 0 if it lies in [start, end]; `denom` = dot(n, dir).
__device__ __forceinline__ bool plane_t(V3 n, float dc, const Ray& r, float start, float end, float& t, float& denom) {
  denom = dot3(n, r.d);
  if (denom == 0.0f) return false;
  t = __fdiv_rn(-(dot3(n, r.o) + dc), denom);
  return start <= t && t <= end;
}

// The hit's planar coordinates (mesh/planar/mod.rs:181-185): alpha along u,
// beta along v, from w = cross(u, v) / |cross(u, v)|^2. `ext` = u, v, w.
__device__ __forceinline__ void planar_uv(const float* ext, V3 p, V3 pos, float& alpha, float& beta) {
  const V3 u = v3(__ldg(ext), __ldg(ext + 1), __ldg(ext + 2));
  const V3 v = v3(__ldg(ext + 3), __ldg(ext + 4), __ldg(ext + 5));
  const V3 w = v3(__ldg(ext + 6), __ldg(ext + 7), __ldg(ext + 8));
  const V3 pl = v3(pos.x - p.x, pos.y - p.y, pos.z - p.z);
  alpha = dot3(w, cross3(pl, v));
  beta = dot3(w, cross3(u, pl));
}

// ParallelogramMesh::intersect (mesh/planar/parallelogram.rs:49-57): the
// plane hit with both planar coordinates in [0, 1].
__device__ __forceinline__ bool quad_t(const GpuPrim& p, const float* quad_ext, const Ray& r, float start, float end,
                                       float& t) {
  float denom;
  if (!plane_t(xyz(p.a), p.b.x, r, start, end, t, denom)) return false;
  float al, be;
  planar_uv(quad_ext + 9ull * __float_as_uint(p.c.w), xyz(p.c), at3(r.o, r.d, t), al, be);
  return al >= 0.0f && al <= 1.0f && be >= 0.0f && be <= 1.0f;
}

// CylinderMesh::intersect (mesh/primitive/cylinder.rs:64-183): distance and
// face (0 body, 1 the p1 cap, 2 the p2 cap), including the reference's cap
// choice (its far-cap distance is max(min(near, far), far)) and its miss of
// rays parallel to the axis (a = 0). The reference's test is not monotone in
// the interval's end (a cap nearer than the body roots is dropped when both
// body roots lie beyond the end), so its closest hit can depend on the order
// objects are tested in; callers evaluate it against [start, inf) and clip
// the result to their end, which is order-independent and equals the
// reference's answer for the first object tested.
//
// The body quadratic a t^2 + 2 b t + c (a = L^2 - (ba.d)^2, b = L^2 oc.d -
// (ba.oc)(ba.d), c = L^2 |oc|^2 - (ba.oc)^2 - r^2 L^2 with ba = p2 - p1 of
// length L) is the reference's; in f32 its discriminant b^2 - a c cancels
// for grazing rays (normals off by up to 2e-3). It is evaluated here without
// that cancellation, as the sphere's is: with dp = L^2 d - (ba.d) ba and
// op = L^2 oc - (ba.oc) ba (the components normal to the axis, scaled),
// b = op.d, c = |op|^2 / L^2 - r^2 L^2 and b^2 - a c = a (r^2 L^2 -
// |op - (b/a) dp|^2 / L^2), the vector being the ray's closest approach to
// the axis; the roots are q / a and c / q with q = -(b + sign(b) sqrt(disc)).
// A ray parallel to the axis (a = 0) misses, as in the reference (its body
// roots are infinite and its cap test |a t + b| < |b| fails).
struct CylHit { float t, dan; uint32_t face; };
__device__ __forceinline__ bool cylinder_t(const GpuPrim& p, const Ray& r, float start, float end, CylHit& ch) {
  const V3 o1 = xyz(p.a), along = xyz(p.b);
  const float lsq = p.c.x, rad = p.c.y;
  const V3 oc = v3(r.o.x - o1.x, r.o.y - o1.y, r.o.z - o1.z);
  const float bard = dot3(along, r.d), baoc = dot3(along, oc);
  const float a = __fmaf_rn(-bard, bard, lsq);
  if (a == 0.0f) return false;
  const V3 dp = v3(__fmaf_rn(lsq, r.d.x, -(bard * along.x)), __fmaf_rn(lsq, r.d.y, -(bard * along.y)),
                   __fmaf_rn(lsq, r.d.z, -(bard * along.z)));
  const V3 op = v3(__fmaf_rn(lsq, oc.x, -(baoc * along.x)), __fmaf_rn(lsq, oc.y, -(baoc * along.y)),
                   __fmaf_rn(lsq, oc.z, -(baoc * along.z)));
  const float b = dot3(op, r.d);
  const float c = __fmaf_rn(-(rad * rad), lsq, __fdiv_rn(dot3(op, op), lsq));
  const float k = __fdiv_rn(b, a);
  const V3 w = v3(__fmaf_rn(-k, dp.x, op.x), __fmaf_rn(-k, dp.y, op.y), __fmaf_rn(-k, dp.z, op.z));
  const float disc = a * __fmaf_rn(rad * rad, lsq, -__fdiv_rn(dot3(w, w), lsq));
  if (disc < 0.0f) return false;
  const float sq = __fsqrt_rn(disc);
  const float q = b > 0.0f ? -b - sq : -b + sq;
  const float r1 = __fdiv_rn(q, a), r2 = q != 0.0f ? __fdiv_rn(c, q) : q;
  float dist = fminf(r1, r2);
  if (!(start <= dist && dist <= end)) dist = fmaxf(r1, r2);
  if (!(start <= dist && dist <= end)) return false;
  const float dan = __fdiv_rn(__fmaf_rn(dist, bard, baoc), lsq);
  ch.dan = dan;
  if (dan > 0.0f && dan < 1.0f) {
    ch.t = dist;
    ch.face = 0;
    return true;
  }
  float dn, df;
  if (signbit(baoc) == signbit(bard)) {
    dn = __fdiv_rn(0.0f - baoc, bard);
    df = __fdiv_rn(lsq - baoc, bard);
  } else {
    dn = __fdiv_rn(lsq - baoc, bard);
    df = __fdiv_rn(0.0f - baoc, bard);
  }
  dn = fminf(dn, df);
  df = fmaxf(dn, df);
  if (start <= dn && dn <= end && fabsf(__fmaf_rn(a, dn, b)) < sq) dist = dn;
  else if (start <= df && df <= end && fabsf(__fmaf_rn(a, df, b)) < sq) dist = df;
  else return false;
  ch.t = dist;
  ch.face = signbit(dan) ? 1u : 2u;
  return true;
}

// Hit on an unbounded object. `flip`: the ray normal is -n (infinite planes
// face the ray; raymarched surfaces keep their normal).
struct SdfHit { float t; V3 n; bool front; uint32_t side; bool flip; };

// RaymarchedIsosurfaceMesh::intersect (mesh/isosurface/raymarched.rs:73-122)
// as a resumable march: sdf_march_begin, then sdf_march_step until it returns
// a hit or a miss, then sdf_march_hit for the hit record. Two exact early
// exits cannot change the result:
//  - total distance is non-decreasing, so once it passes the distance that
//    must be beaten (`beat`, inclusive when nothing has been hit yet) no later
//    step can produce the closest hit;
//  - outside the function's bound radius and moving away, every later step
//    evaluates to more than epsilon, so no later step can hit.
struct SdfMarch {
  float total;  // distance marched from the ray's origin
  V3 point;     // ray.at(total)
  uint32_t i;   // steps taken (the hit's Intersection::side)
  float d;      // the last evaluation (its sign is the hit's front face)
};
enum : int { kMarchOn = 0, kMarchHit = 1, kMarchMiss = 2 };

__device__ __forceinline__ void sdf_march_begin(const Ray& r, float start, SdfMarch& m) {
  m.total = start;
  m.point = at3(r.o, r.d, start);
  m.i = 0;
  m.d = 0.0f;
}

template <bool COUNT>
__device__ __forceinline__ int sdf_march_step(const GpuSdf& s, const Ray& r, float start, float end, float beat,
                                              bool beat_inclusive, SdfMarch& m, unsigned long long& steps,
                                              unsigned long long& iters) {
  const float d = sdf_eval(s, m.point, COUNT ? &iters : nullptr);
  if (COUNT) ++steps;
  m.total = m.total + fabsf(d);
  m.point = at3(r.o, r.d, m.total);
  m.d = d;
  const bool beaten = beat_inclusive ? m.total <= beat : m.total < beat;
  if (fabsf(d) < s.eps && start <= m.total && m.total <= end) return beaten ? kMarchHit : kMarchMiss;
  if (m.i > s.max_iter) return kMarchMiss;
  if (!beaten) return kMarchMiss;
  const V3 q = m.point - v3(s.cx, s.cy, s.cz);
  if (dot3(q, q) > s.bound_radius * s.bound_radius && dot3(q, r.d) > 0.0f) return kMarchMiss;
  ++m.i;
  return kMarchOn;
}

// The hit record at a step that returned kMarchHit: the normal by central
// differences with step epsilon (raymarched.rs:107-111), not flipped.
template <bool COUNT>
__device__ __forceinline__ void sdf_march_hit(const GpuSdf& s, const SdfMarch& m, SdfHit& h, unsigned long long& steps) {
  const float eps = s.eps;
  const V3 pp = m.point;
  if (COUNT) steps += 6;
  V3 g = v3(sdf_eval(s, v3(pp.x + eps, pp.y, pp.z)) - sdf_eval(s, v3(pp.x - eps, pp.y, pp.z)),
            sdf_eval(s, v3(pp.x, pp.y + eps, pp.z)) - sdf_eval(s, v3(pp.x, pp.y - eps, pp.z)),
            sdf_eval(s, v3(pp.x, pp.y, pp.z + eps)) - sdf_eval(s, v3(pp.x, pp.y, pp.z - eps)));
  h.t = m.total;
  h.n = normalize3(g);
  h.front = !signbit(m.d);
  h.side = m.i;
  h.flip = false;
}

// The whole march in one call.
template <bool COUNT>
__device__ bool sdf_march(const GpuSdf& s, const Ray& r, float start, float end, float beat, bool beat_inclusive, SdfHit& h,
                          unsigned long long& steps, unsigned long long& iters) {
  SdfMarch m;
  sdf_march_begin(r, start, m);
  for (;;) {
    const int st = sdf_march_step<COUNT>(s, r, start, end, beat, beat_inclusive, m, steps, iters);
    if (st == kMarchMiss) return false;
    if (st == kMarchHit) {
      sdf_march_hit<COUNT>(s, m, h, steps);
      return true;
    }
  }
}

// Whether the segment [start, lim] of the ray can reach the SDF's bound
// sphere (radius widened by 1e-3 relative for the test's own rounding): when
// it cannot, the march above returns no hit, since a hit needs a point within
// epsilon of the surface and every such point lies inside the bound.
__device__ __forceinline__ bool sdf_bound_reachable(const GpuSdf& s, const Ray& r, float start, float lim) {
  const V3 oc = r.o - v3(s.cx, s.cy, s.cz);
  const float R = s.bound_radius * 1.001f;
  const float b = dot3(oc, r.d);
  // r^2 - |l|^2 with l the centre-to-line vector: no cancellation for distant origins
  const V3 l = v3(__fmaf_rn(-b, r.d.x, oc.x), __fmaf_rn(-b, r.d.y, oc.y), __fmaf_rn(-b, r.d.z, oc.z));
  const float disc = R * R - dot3(l, l);
  if (disc < 0.0f) return false;
  const float sq = __fsqrt_rn(disc);
  const float slack = 1e-3f * (fabsf(b) + R);
  return -b + sq + slack >= start && -b - sq - slack <= lim;
}

// ---------------------------------------------------------------------------
// Closest hit over the BVH and the unbounded list.
// ---------------------------------------------------------------------------
struct HitRec {
  float t;
  float tl;      // transformed primitive: the distance along the mesh-space ray
  int prim;      // index into the reordered prim array, or -1
  int sdf;       // SDF index when an unbounded object won, else -1
  SdfHit sh;
};

struct Counters {
  unsigned long long nodes = 0, prims = 0, sdf_steps = 0, sdf_iters = 0, hits = 0;
};


// A transformed object's matrices: inverse (world to mesh space) at m,
// forward (mesh to world space) at m + 12, both 3 x 4 row-major.
__device__ __forceinline__ const float* prim_xform_of(const GpuScene& sc, int i) {
  return sc.xforms + 24ull * __ldg(sc.prim_xform + i);
}
__device__ __forceinline__ V3 xf_point(const float* m, V3 p) {
  return v3(__fmaf_rn(__ldg(m + 0), p.x, __fmaf_rn(__ldg(m + 1), p.y, __fmaf_rn(__ldg(m + 2), p.z, __ldg(m + 3)))),
            __fmaf_rn(__ldg(m + 4), p.x, __fmaf_rn(__ldg(m + 5), p.y, __fmaf_rn(__ldg(m + 6), p.z, __ldg(m + 7)))),
            __fmaf_rn(__ldg(m + 8), p.x, __fmaf_rn(__ldg(m + 9), p.y, __fmaf_rn(__ldg(m + 10), p.z, __ldg(m + 11)))));
}
__device__ __forceinline__ V3 xf_vector(const float* m, V3 v) {
  return v3(__fmaf_rn(__ldg(m + 0), v.x, __fmaf_rn(__ldg(m + 1), v.y, __ldg(m + 2) * v.z)),
            __fmaf_rn(__ldg(m + 4), v.x, __fmaf_rn(__ldg(m + 5), v.y, __ldg(m + 6) * v.z)),
            __fmaf_rn(__ldg(m + 8), v.x, __fmaf_rn(__ldg(m + 9), v.y, __ldg(m + 10) * v.z)));
}
// ObjectTransform::incoming_ray (object/transform.rs:90-97): origin and
// direction mapped by the inverse, the direction normalised again (Ray::new).
__device__ __forceinline__ Ray xf_incoming(const float* m, const Ray& r) { return make_ray(xf_point(m, r.o), xf_vector(m, r.d)); }

// Test the primitives of one leaf, shrinking `end` to each accepted hit
// (object/bvh.rs:82-96: a later hit at equal distance replaces the earlier).
// A primitive of a transformed object (SimpleObject::full_intersect,
// object/simple.rs:107-116) is tested against the mesh-space ray from the
// same start; its distance is the world-space length from the ray's origin
// to the mapped hit point (transform.rs:101-130), and that distance must lie
// within `end`. (The reference bounds the mesh-space distance by the world
// bound instead; the two agree for rigid transforms, and under scaling the
// reference's result depends on its traversal order, while this one is the
// closest world-space hit.) `best_tl` keeps the mesh-space distance of the
// closest hit.
template <uint32_t F, bool COUNT>
__device__ __forceinline__ void test_leaf(const GpuScene& sc, int first, int count, const Ray& rw, float start, float& end,
                                          int& best, float& best_tl, const RngCtx& ctx, Counters& cnt) {
  for (int i = first; i < first + count; ++i) {
    const GpuPrim* pp = sc.prims + i;
    float4 a = __ldg(&pp->a);
    uint32_t kind = kinds_of(F) == F_TRI ? (uint32_t)PK_TRIANGLE
                  : (kinds_of(F) == F_SPHERE ? (uint32_t)PK_SPHERE : (__float_as_uint(a.w) >> kKindShift));
    if (COUNT) ++cnt.prims;
    const float* xf = nullptr;
    Ray r = rw;
    float tend = end;  // a transformed primitive is tested on [start, inf), then bounded in world space
    if ((F & F_EXT) && (__float_as_uint(a.w) & kXformBit)) {
      xf = prim_xform_of(sc, i);
      r = xf_incoming(xf, rw);
      tend = CUDART_INF_F;
    }
    float t;
    if ((F & F_TRI) && kind == PK_TRIANGLE) {
      float4 b = __ldg(&pp->b), c = __ldg(&pp->c);
      float u, v, det;
      if (!triangle_t(xyz(a), xyz(b), xyz(c), r, start, tend, t, u, v, det)) continue;
      if (__float_as_uint(c.w) & kTriCheckNormals) {
        V3 n;
        if (!tri_normal(sc.tri_normals + 9ull * (__float_as_uint(b.w) - sc.tri_base), u, v, n)) continue;
      }
    } else if ((F & F_SPHERE) && kind == PK_SPHERE) {
      float4 b = __ldg(&pp->b);
      if (!sphere_t(xyz(a), b.y, r, start, tend, t)) continue;
    } else if ((F & F_BOX) && kind == PK_BOX) {
      float4 b = __ldg(&pp->b), c = __ldg(&pp->c);
      BoxHit bh;
      if (!box_t(xyz(a), xyz(b), xyz(c), r, start, tend, bh)) continue;
      t = bh.t;
    } else if ((F & F_QUAD) && kind == PK_QUAD) {
      GpuPrim p;
      p.a = a; p.b = __ldg(&pp->b); p.c = __ldg(&pp->c);
      if (!quad_t(p, sc.quad_ext, r, start, tend, t)) continue;
    } else if ((F & F_CYLINDER) && kind == PK_CYLINDER) {
      GpuPrim p;
      p.a = a; p.b = __ldg(&pp->b); p.c = __ldg(&pp->c);
      CylHit ch;
      if (!cylinder_t(p, r, start, CUDART_INF_F, ch) || !(ch.t <= tend)) continue;
      t = ch.t;
    } else if ((F & F_VOL) && (kind == PK_VOL_SPHERE || kind == PK_VOL_BOX)) {
      GpuPrim p;
      p.a = a; p.b = __ldg(&pp->b); p.c = __ldg(&pp->c);
      if (!volume_t(p, kind, __float_as_uint(p.b.w) - sc.vol_base, r, start, end, ctx, t)) continue;
    } else {
      continue;
    }
    if ((F & F_EXT) && xf) {
      const float tl = t;
      t = length3(xf_point(xf + 12, at3(r.o, r.d, tl)) - rw.o);
      if (!(t <= end)) continue;
      best_tl = tl;
    }
    end = t;
    best = i;
  }
}

// Child reference: an internal node pair index (>= 0), or a leaf encoded as
// ~(first << 3 | count) (< 0). kDone ends the traversal.
constexpr int kDone = 0x7FFFFFFF;
__device__ __forceinline__ int child_ref(int index, int count) { return count > 0 ? ~((index << 3) | count) : index; }

// 2^23 + byte `sel` (0..3) of w, as a float (bit pattern 0x4B0000bb): one
// byte permute instead of an integer-to-float conversion.
__device__ __forceinline__ float byte_plus_2p23(uint32_t w, uint32_t sel) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | sel));
}

constexpr int kTravStack = 64;
static_assert(kTravStack >= kStackSize && kTravStack >= kWideMaxDepth + 1, "traversal stack too small");

// Traversal stacks. LocalStack: every entry in local memory. SplitStack: the
// first SH entries of each thread in shared memory (entry i of thread x at
// i * STRIDE + x, so a warp's 8-byte accesses are contiguous and no node data
// evicts them from L1), the deeper ones in local memory.
struct LocalStack {
  uint2* s;
  __device__ __forceinline__ uint2 get(int i) const { return s[i]; }
  __device__ __forceinline__ void set(int i, uint2 v) { s[i] = v; }
};
// DynStack: the same split with the shared entries per thread and the
// stride chosen at launch (rg_tuning.shared_stack, the block size); `loc`
// has kTravStack entries, of which the first n_sh stay unused.
struct DynStack {
  uint2* sh;   // this thread's column of the block's dynamic shared array
  uint2* loc;
  int n_sh, stride;
  __device__ __forceinline__ uint2 get(int i) const { return i < n_sh ? sh[i * stride] : loc[i]; }
  __device__ __forceinline__ void set(int i, uint2 v) {
    if (i < n_sh) sh[i * stride] = v;
    else loc[i] = v;
  }
};
template <int SH, int STRIDE>
struct SplitStack {
  uint2* sh;   // this thread's column of the block's shared array (unused when SH is 0)
  uint2* loc;  // kTravStack - SH entries in local memory
  __device__ __forceinline__ uint2 get(int i) const {
    if constexpr (SH > 0) return i < SH ? sh[i * STRIDE] : loc[i - SH];
    else return loc[i];
  }
  __device__ __forceinline__ void set(int i, uint2 v) {
    if constexpr (SH > 0) {
      if (i < SH) sh[i * STRIDE] = v;
      else loc[i - SH] = v;
    } else {
      loc[i] = v;
    }
  }
};

// Resumable traversal of one ray over the binary or the 8-wide tree. A run
// goes on to completion, or (BOUNDED) for at most `budget` node visits, and
// returns true once the traversal is complete (the closest hit so far is in
// best / tmax), so a persistent kernel can hand idle lanes new rays between
// runs. The stack is a separate array (local memory) so that these scalars
// stay in registers.
struct Traversal {
  int sp;
  float tmax;
  int best;
  float best_tl;          // transformed primitive: mesh-space distance of the closest hit
  bool wide;
  int ref, leaf;          // binary: next node (or leaf code, or kDone), postponed leaf
  uint2 ng;               // wide: current node group
  uint32_t visits, oct;   // wide: node visits so far, ray octant
};

template <uint32_t F>
__device__ __forceinline__ void trav_init(Traversal& t, const GpuScene& sc, const Ray& r, float end) {
  t.sp = 0;
  t.tmax = end;
  t.best = -1;
  t.best_tl = 0.0f;
  t.wide = false;
  if (F & F_WIDE) {
    // A zero (or underflowing) direction component makes that axis's inverse
    // infinite: the 8-wide box test cannot cull on such an axis, while the
    // binary slab test handles the infinities exactly, so those rays (which
    // the samplers do produce, e.g. a ball sample of exactly (0, 0, r) off an
    // axis-aligned wall) take the binary tree. Both trees index the same
    // primitives, so the closest hit is the same.
    const float kInf = __int_as_float(0x7f800000);
    t.wide = sc.n_wnodes > 0 && fabsf(r.inv.x) < kInf && fabsf(r.inv.y) < kInf && fabsf(r.inv.z) < kInf;
  }
  if (t.wide) {
    t.oct = (__float_as_uint(r.inv.x) >> 31) | ((__float_as_uint(r.inv.y) >> 31) << 1) |
            ((__float_as_uint(r.inv.z) >> 31) << 2);
    t.ng = make_uint2(0u, (1u << (24 + t.oct)) | 1u);  // the root, as slot 0 of a one-child group
    t.visits = 0;
  } else {
    t.ref = sc.n_nodes > 0 ? 0 : kDone;
    t.leaf = 0;
  }
}

// Binary traversal, after Aila & Laine ("Understanding the efficiency of ray
// traversal on GPUs", HPG 2009): an inner-node loop that postpones the first
// leaf it meets and keeps going until every lane of the warp holds a leaf,
// then a leaf loop, so that lanes step through nodes together and through
// primitives together. Near children go first; far children wait on the
// stack as (node, entry distance) and are dropped on pop once they lie beyond
// the closest hit (the same conservative comparison as the slab test, so the
// result does not change).
template <uint32_t F, bool COUNT, bool BOUNDED, class Stack>
__device__ __forceinline__ bool run_binary(Traversal& t, Stack& stack, const GpuScene& sc, const Ray& r, float start,
                                           const RngCtx& ctx, Counters& cnt, uint32_t* err, int budget) {
  auto pop = [&]() -> int {
    const float lim = __fmaf_rn(fabsf(t.tmax), kSlabSlack, t.tmax);
    while (t.sp > 0) {
      --t.sp;
      const uint2 e = stack.get(t.sp);
      if (__uint_as_float(e.y) <= lim) return (int)e.x;
    }
    return kDone;
  };
  int it = 0;
  for (;;) {
    while (t.ref >= 0 && t.ref != kDone) {
      const BvhNode2* np = sc.nodes + t.ref;
      float4 xs = __ldg(&np->xs), ys = __ldg(&np->ys), zs = __ldg(&np->zs);
      int4 m = __ldg(&np->meta);
      if (COUNT) ++cnt.nodes;
      if (BOUNDED) ++it;
      float tn0, tn1;
      bool h0 = slab(xs.x, xs.y, ys.x, ys.y, zs.x, zs.y, r, start, t.tmax, tn0);
      bool h1 = slab(xs.z, xs.w, ys.z, ys.w, zs.z, zs.w, r, start, t.tmax, tn1) && m.y >= 0;
      int r0 = child_ref(m.x, m.z), r1 = child_ref(m.y, m.w);
      if (h0 && h1) {
        bool swap = tn1 < tn0;
        t.ref = swap ? r1 : r0;
        if (t.sp < (int)sc.stack_limit) {
          stack.set(t.sp, make_uint2((uint32_t)(swap ? r0 : r1), __float_as_uint(swap ? tn0 : tn1)));
          ++t.sp;
        } else {
          atomicOr(err, ERR_STACK_OVERFLOW);
        }
      } else if (h0) {
        t.ref = r0;
      } else if (h1) {
        t.ref = r1;
      } else {
        t.ref = pop();
      }
      if (t.ref < 0 && t.leaf == 0) {  // postpone the first leaf and keep traversing
        t.leaf = t.ref;
        t.ref = pop();
      }
      if (!__any_sync(__activemask(), t.leaf == 0) || (BOUNDED && it >= budget)) break;
    }
    while (t.leaf < 0) {
      int code = ~t.leaf;
      test_leaf<F, COUNT>(sc, code >> 3, code & 7, r, start, t.tmax, t.best, t.best_tl, ctx, cnt);
      t.leaf = 0;
      if (t.ref < 0) {
        t.leaf = t.ref;
        t.ref = pop();
      }
    }
    if (t.ref == kDone) return true;
    if (BOUNDED && it >= budget) return false;
  }
}

// Traversal of the compressed 8-wide tree (layout in gpu_scene.h), after
// Ylitie, Karras and Laine (HPG 2017). A group is (base, bits): a node group
// holds the not yet visited hit internal children of one node in bits 24..31
// (in visit order: bit 24 + (slot ^ octant)) and the node's imask in bits
// 0..7; a primitive group holds hit primitives prim_base + b in bits 0..23.
// The stack holds node groups, at most one per tree level. Primitive tests
// run as soon as their leaf is hit: postponing them while few lanes want
// them (as Ylitie et al. do) keeps tmax at its initial value for longer, and
// where lanes are not converged (the persistent extend kernel) it defers
// every test and culls nothing.
//
// Child boxes. A plane at grid step q is t* = (p + q s - o) / d. With
//   A = s / d (exact: s is a power of two),  B = fl((p - o) / d),
//   C = fl(B - 2^23 A),  e = 1.0005 |A| + 2^-19 |B|,
// near planes are evaluated as fma(2^23 + q, A, fl(C - e)) and far planes as
// fma(2^23 + q, A, fl(C + e)) (2^23 + q comes from one byte permute). The
// roundings of 1/d, p - o, B, C, C -+ e and the fma move a plane by at most
// |A| (1 + 512u) + 6u |B| + O(u^2) (u = 2^-24; the |A| from C, whose
// magnitude is about 2^23 |A|), which e exceeds, so every near plane comes out
// at or before its exact value and every far plane at or after it. A child is
// entered when max(near planes, start) <= min(far planes, tmax): no box is
// rejected that its exact grid box (which contains the child's box) would
// accept, so the closest hit is the one the primitive tests alone give. The
// widening is per axis and amounts to one grid step in that axis's own
// coordinate, whatever the direction. Rays with a zero direction component
// do not come here (closest_hit sends them to the binary tree); an axis whose
// A or C still overflows (a huge node, a tiny component) yields NaN planes,
// which fminf/fmaxf skip: that axis then does not cull.
template <uint32_t F, bool COUNT, bool BOUNDED, class Stack>
__device__ __forceinline__ bool run_wide(Traversal& t, Stack& stack, const GpuScene& sc, const Ray& r, float start,
                                         const RngCtx& ctx, Counters& cnt, uint32_t* err, int budget) {
  const float kNaN = __int_as_float(0x7fffffff), kInf = __int_as_float(0x7f800000);
  const uint32_t oct = t.oct;
  int it = 0;
  for (;;) {
    uint2 pg = make_uint2(0u, 0u);
    if (t.ng.y > 0x00FFFFFFu) {
      const uint32_t k = __ffs(t.ng.y >> 24) - 1;
      t.ng.y &= ~(1u << (24 + k));
      const uint32_t slot = k ^ oct;
      const uint32_t idx = t.ng.x + __popc(t.ng.y & ((1u << slot) - 1u) & 0xFFu);
      if (t.ng.y > 0x00FFFFFFu) {
        if (t.sp < (int)sc.stack_limit) {
          stack.set(t.sp, t.ng);
          ++t.sp;
        } else {
          atomicOr(err, ERR_STACK_OVERFLOW);
        }
      }
      // A tree visits each node at most once per ray; the host checks the
      // tree's structure, and this guard keeps a damaged one bounded (the
      // traversal then ends through the loop's normal exit).
      const bool bad = idx >= sc.n_wnodes || ++t.visits > sc.n_wnodes;
      if (bad) {
        atomicOr(err, ERR_BAD_INDEX);
        t.sp = 0;
      }
      const WideNode* np = sc.wnodes + (bad ? 0u : idx);
      const float4 w0 = __ldg(&np->w0);
      const uint4 w1 = __ldg(&np->w1), qx = __ldg(&np->qx), qy = __ldg(&np->qy), qz = __ldg(&np->qz);
      if (COUNT) ++cnt.nodes;
      if (BOUNDED) ++it;
      const uint32_t hdr = __float_as_uint(w0.w);
      const float ax = __uint_as_float((hdr & 0xFFu) << 23) * r.inv.x;
      const float ay = __uint_as_float(((hdr >> 8) & 0xFFu) << 23) * r.inv.y;
      const float az = __uint_as_float(((hdr >> 16) & 0xFFu) << 23) * r.inv.z;
      const float bx = (w0.x - r.o.x) * r.inv.x, by = (w0.y - r.o.y) * r.inv.y, bz = (w0.z - r.o.z) * r.inv.z;
      const float cx = __fmaf_rn(-8388608.0f, ax, bx), cy = __fmaf_rn(-8388608.0f, ay, by),
                  cz = __fmaf_rn(-8388608.0f, az, bz);
      const float ex = __fmaf_rn(fabsf(ax), 1.0005f, 1.9073486328125e-6f * fabsf(bx));
      const float ey = __fmaf_rn(fabsf(ay), 1.0005f, 1.9073486328125e-6f * fabsf(by));
      const float ez = __fmaf_rn(fabsf(az), 1.0005f, 1.9073486328125e-6f * fabsf(bz));
      float cnx = cx - ex, cfx = cx + ex, cny = cy - ey, cfy = cy + ey, cnz = cz - ez, cfz = cz + ez;
      if (!(fabsf(ax) < kInf && fabsf(cx) < kInf)) cnx = cfx = kNaN;
      if (!(fabsf(ay) < kInf && fabsf(cy) < kInf)) cny = cfy = kNaN;
      if (!(fabsf(az) < kInf && fabsf(cz) < kInf)) cnz = cfz = kNaN;
      // near planes: lo for a positive direction component, hi for a negative one
      const bool sx = oct & 1u, sy = oct & 2u, sz = oct & 4u;
      const uint32_t nx0 = sx ? qx.z : qx.x, nx1 = sx ? qx.w : qx.y, fx0 = sx ? qx.x : qx.z, fx1 = sx ? qx.y : qx.w;
      const uint32_t ny0 = sy ? qy.z : qy.x, ny1 = sy ? qy.w : qy.y, fy0 = sy ? qy.x : qy.z, fy1 = sy ? qy.y : qy.w;
      const uint32_t nz0 = sz ? qz.z : qz.x, nz1 = sz ? qz.w : qz.y, fz0 = sz ? qz.x : qz.z, fz1 = sz ? qz.y : qz.w;
      // internal children's meta bytes (0x38..0x3F) get the octant folded into their slot bits
      uint32_t m0 = w1.z, m1 = w1.w;
      m0 ^= ((m0 >> 3) & (m0 >> 4) & 0x01010101u) * oct;
      m1 ^= ((m1 >> 3) & (m1 >> 4) & 0x01010101u) * oct;
      uint32_t hits = 0;
#pragma unroll
      for (uint32_t c = 0; c < 8; ++c) {
        const uint32_t b = c & 3u;
        const float tnx = __fmaf_rn(byte_plus_2p23(c < 4 ? nx0 : nx1, b), ax, cnx);
        const float tny = __fmaf_rn(byte_plus_2p23(c < 4 ? ny0 : ny1, b), ay, cny);
        const float tnz = __fmaf_rn(byte_plus_2p23(c < 4 ? nz0 : nz1, b), az, cnz);
        const float tfx = __fmaf_rn(byte_plus_2p23(c < 4 ? fx0 : fx1, b), ax, cfx);
        const float tfy = __fmaf_rn(byte_plus_2p23(c < 4 ? fy0 : fy1, b), ay, cfy);
        const float tfz = __fmaf_rn(byte_plus_2p23(c < 4 ? fz0 : fz1, b), az, cfz);
        const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, start));
        const float tf = fminf(fminf(tfx, tfy), fminf(tfz, t.tmax));
        const uint32_t meta = ((c < 4 ? m0 : m1) >> (8 * b)) & 0xFFu;
        if (tn <= tf) hits |= (meta >> 5) << (meta & 31u);
      }
      if (bad) hits = 0;
      t.ng = make_uint2(w1.x, (hits & 0xFF000000u) | (hdr >> 24));
      pg = make_uint2(w1.y, hits & 0x00FFFFFFu);
    }
    while (pg.y) {
      const uint32_t pi = pg.x + (uint32_t)(__ffs(pg.y) - 1);
      pg.y &= pg.y - 1u;
      if (pi < sc.n_prims) test_leaf<F, COUNT>(sc, (int)pi, 1, r, start, t.tmax, t.best, t.best_tl, ctx, cnt);
      else atomicOr(err, ERR_BAD_INDEX);
    }
    if (t.ng.y <= 0x00FFFFFFu) {
      if (t.sp == 0) return true;
      --t.sp;
      t.ng = stack.get(t.sp);
    }
    if (BOUNDED && it >= budget) return false;
  }
}

// Whether this lane finishes its ready path now: a warp of a persistent
// kernel finishes its ready lanes together once at least `min_ready` of them
// are ready or all of its live lanes (`live`, a subset of which is ready)
// are, so the finishing code runs on many lanes at once. Called by the whole
// warp.
__device__ __forceinline__ bool finish_now(bool ready, unsigned live, int min_ready) {
  const unsigned r = __ballot_sync(0xffffffffu, ready);
  return ready && ((int)__popc(r) >= min_ready || r == live);
}

// Runs a traversal to completion (BOUNDED false) or for at most `budget`
// node visits (BOUNDED true); returns true once it is complete.
template <uint32_t F, bool COUNT, bool BOUNDED, class Stack>
__device__ __forceinline__ bool trav_run(Traversal& t, Stack& stack, const GpuScene& sc, const Ray& r, float start,
                                         const RngCtx& ctx, Counters& cnt, uint32_t* err, int budget) {
  if ((F & F_WIDE) && t.wide) return run_wide<F, COUNT, BOUNDED>(t, stack, sc, r, start, ctx, cnt, err, budget);
  return run_binary<F, COUNT, BOUNDED>(t, stack, sc, r, start, ctx, cnt, err, budget);
}

// ObjectList::full_intersect (object/list.rs:112-129) after the tree: every
// unbounded object with the original interval [start, end]; it replaces the
// result only if strictly closer.
template <uint32_t F, bool COUNT>
__device__ __forceinline__ bool finish_hit(const GpuScene& sc, const Ray& r, float start, float end, const Traversal& t,
                                           HitRec& h, Counters& cnt) {
  h.prim = t.best;
  h.sdf = -1;
  h.t = t.tmax;
  h.tl = t.best_tl;
  bool any = t.best >= 0;
  if (F & (F_SDF | F_PLANE)) {
    for (uint32_t k = 0; k < sc.n_sdfs; ++k) {
      const GpuSdf& f = sc.sdfs[k];
      SdfHit sh;
      if ((F & F_PLANE) && f.kind == kUnboundedPlane) {
        // InfinitePlaneMesh::intersect (mesh/planar/infinite_plane.rs:87-92)
        float pt, denom;
        if (!plane_t(v3(f.cx, f.cy, f.cz), f.p0, r, start, end, pt, denom) || (any && !(pt < h.t))) continue;
        sh = SdfHit{pt, v3(f.cx, f.cy, f.cz), (bool)signbit(denom), 0u, !signbit(denom)};
      } else if (F & F_SDF) {
        if (!sdf_march<COUNT>(f, r, start, end, any ? h.t : end, !any, sh, cnt.sdf_steps, cnt.sdf_iters)) continue;
      } else {
        continue;
      }
      h.t = sh.t;
      h.sdf = (int)k;
      h.sh = sh;
      any = true;
    }
  }
  if (COUNT && any) ++cnt.hits;
  return any;
}

// Closest hit over the BVH (binary or 8-wide, by F_WIDE), then the unbounded
// list, with the caller's traversal stack.
template <uint32_t F, bool COUNT, class Stack>
__device__ bool closest_hit_with(Stack& stack, const GpuScene& sc, const Ray& r, float start, float end,
                                 const RngCtx& ctx, HitRec& h, Counters& cnt, uint32_t* err) {
  Traversal t;
  trav_init<F>(t, sc, r, end);
  trav_run<F, COUNT, false>(t, stack, sc, r, start, ctx, cnt, err, 0);
  return finish_hit<F, COUNT>(sc, r, start, end, t, h, cnt);
}

// The same with the whole stack in local memory.
template <uint32_t F, bool COUNT>
__device__ bool closest_hit(const GpuScene& sc, const Ray& r, float start, float end, const RngCtx& ctx, HitRec& h,
                            Counters& cnt, uint32_t* err) {
  uint2 entries[kTravStack];
  LocalStack stack{entries};
  return closest_hit_with<F, COUNT>(stack, sc, r, start, end, ctx, h, cnt, err);
}

// Full hit record of the closest hit.
struct Surface {
  V3 pos, normal, ray_normal;
  V3 pos_l;  // the mesh-local point (Intersection::pos_l), set by the extended variant only
  bool front;
  uint32_t material, prim_id, side;
  float u, v;
};

// sphere_uv (mesh/primitive/sphere.rs:114-121)
__device__ __forceinline__ void sphere_uv(V3 local, float& u, float& v) {
  const float kPi = 3.14159265358979323846f;
  const float theta = acosf(-local.y);
  const float phi = atan2f(-local.z, local.x) + kPi;
  u = phi / (2.0f * kPi);
  v = theta / kPi;
}

// Vector3::any_orthonormal_pair of a unit vector (cylinder.rs:41): Duff et
// al., "Building an Orthonormal Basis, Revisited" (JCGT 2017).
__device__ __forceinline__ void orthonormal_pair(V3 n, V3& b1, V3& b2) {
  const float sign = copysignf(1.0f, n.z);
  const float a = __fdiv_rn(-1.0f, sign + n.z);
  const float b = n.x * n.y * a;
  b1 = v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  b2 = v3(b, sign + n.y * n.y * a, -n.y);
}

// UvWrappingMode::apply (mesh/planar/infinite_plane.rs:26-41)
__device__ __forceinline__ void wrap_uv(uint32_t mode, float& u, float& v) {
  if (mode == RG_UV_WRAP) {
    u = fmodf(u, 1.0f); if (u < 0.0f) u = u + 1.0f;  // rem_euclid(1.0)
    v = fmodf(v, 1.0f); if (v < 0.0f) v = v + 1.0f;
  } else if (mode == RG_UV_MIRROR) {
    u = fabsf(fmodf(u, 2.0f) - 1.0f);
    v = fabsf(fmodf(v, 2.0f) - 1.0f);
  } else if (!(0.0f <= u && u <= 1.0f && 0.0f <= v && v <= 1.0f)) {
    u = v = 0.0f;
  }
}

// The bounded primitive part of finalize_hit: the hit of `p` at distance `ht`
// along `r` (world space, or mesh space for a transformed object).
template <uint32_t F, bool UV>
__device__ __forceinline__ void finalize_prim(const GpuScene& sc, const GpuPrim& p, uint32_t kind, const Ray& r, float ht,
                                              const RngCtx& ctx, Surface& s, float start) {
  s.pos = at3(r.o, r.d, ht);
  s.side = 0;
  if (kinds_of(F) == F_TRI) kind = PK_TRIANGLE;
  if (kinds_of(F) == F_SPHERE) kind = PK_SPHERE;
  if ((F & F_SPHERE) && kind == PK_SPHERE) {
    V3 c = xyz(p.a);
    float rad = p.b.x;
    V3 local = v3((s.pos.x - c.x) / rad, (s.pos.y - c.y) / rad, (s.pos.z - c.z) / rad);
    bool inside = dot3(r.d, local) > 0.0f;
    s.normal = local;
    s.ray_normal = inside ? -local : local;
    s.front = !inside;
    s.u = s.v = 0.0f;
    if (UV) sphere_uv(local, s.u, s.v);
    if (F & F_EXT) s.pos_l = local;  // sphere.rs:77-91
  } else if ((F & F_TRI) && kind == PK_TRIANGLE) {
    float t, u, v, det;
    triangle_t(xyz(p.a), xyz(p.b), xyz(p.c), r, -CUDART_INF_F, CUDART_INF_F, t, u, v, det);
    V3 n;
    tri_normal(sc.tri_normals + 9ull * (s.prim_id - sc.tri_base), u, v, n);
    s.normal = n;
    s.ray_normal = n * (-signumf(det));
    s.front = signbit(det);
    s.u = u; s.v = v;
    if (F & F_EXT) s.pos_l = v3(1.0f - u - v, u, v);  // barycentric (triangle.rs:92-101)
  } else if ((F & F_BOX) && kind == PK_BOX) {
    BoxHit bh;
    box_t(xyz(p.a), xyz(p.b), xyz(p.c), r, -CUDART_INF_F, ht, bh);
    V3 rn = v3(bh.axis == 0 ? bh.sgn : 0.0f, bh.axis == 1 ? bh.sgn : 0.0f, bh.axis == 2 ? bh.sgn : 0.0f);
    s.ray_normal = rn;
    s.normal = rn * bh.winding;
    s.front = !signbit(bh.winding);
    s.side = (uint32_t)bh.axis * 2u + (bh.sgn > 0.0f ? 1u : 0u);
    s.u = (bh.u0 + 1.0f) / 2.0f;
    s.v = (bh.u1 + 1.0f) / 2.0f;
    if (F & F_EXT) s.pos_l = s.pos - xyz(p.a);  // less the centre (axis_box.rs:122)
  } else if ((F & F_QUAD) && kind == PK_QUAD) {
    const V3 n = xyz(p.a);
    const float denom = dot3(n, r.d);
    s.normal = n;
    s.ray_normal = (-n) * signumf(denom);
    s.front = signbit(denom);
    planar_uv(sc.quad_ext + 9ull * __float_as_uint(p.c.w), xyz(p.c), s.pos, s.u, s.v);
    if (F & F_EXT) s.pos_l = s.pos - xyz(p.c);  // less the corner (planar/mod.rs:176)
  } else if ((F & F_CYLINDER) && kind == PK_CYLINDER) {
    // cylinder.rs:118-172: the same root, then its normal
    CylHit ch;
    cylinder_t(p, r, start, CUDART_INF_F, ch);
    const V3 o1 = xyz(p.a), along = xyz(p.b);
    const float rad = p.c.y, len = p.c.z;
    V3 n;
    if (ch.face == 0) {
      const V3 oc = v3(r.o.x - o1.x, r.o.y - o1.y, r.o.z - o1.z);
      const V3 rel = at3(oc, r.d, ch.t);
      const V3 out = v3(rel.x - along.x * ch.dan, rel.y - along.y * ch.dan, rel.z - along.z * ch.dan);
      n = v3(__fdiv_rn(out.x, rad), __fdiv_rn(out.y, rad), __fdiv_rn(out.z, rad));
    } else {
      n = v3(__fdiv_rn(along.x, len), __fdiv_rn(along.y, len), __fdiv_rn(along.z, len)) * signumf(ch.dan);
    }
    const float inside = -signumf(dot3(r.d, n));
    s.normal = n;
    s.ray_normal = n * inside;
    s.front = signbit(inside);
    s.side = ch.face;
    s.u = s.v = 0.0f;
    if (F & F_EXT) {  // less the centre (cylinder.rs:171)
      const V3 c = v3(o1.x + along.x / 2.0f, o1.y + along.y / 2.0f, o1.z + along.z / 2.0f);
      s.pos_l = s.pos - c;
    }
    if (UV) {  // cylinder.rs:130-172
      const V3 ax = v3(__fdiv_rn(along.x, len), __fdiv_rn(along.y, len), __fdiv_rn(along.z, len));
      V3 o0, o1v;
      orthonormal_pair(ax, o0, o1v);
      const V3 oc = v3(r.o.x - o1.x, r.o.y - o1.y, r.o.z - o1.z);
      if (ch.face == 0) {
        const float kPi = 3.14159265358979323846f;
        const float theta = acosf(dot3(n, o1v)) * signumf(dot3(n, o0));
        s.u = theta / kPi / 2.0f + 0.5f;
        s.v = ch.dan;
      } else {
        const V3 rel = at3(oc, r.d, ch.t);
        const V3 q = v3(__fdiv_rn(rel.x, rad), __fdiv_rn(rel.y, rad), __fdiv_rn(rel.z, rad));
        s.u = dot3(q, o0) / 2.0f + 0.5f;
        s.v = dot3(q, o1v) / 2.0f + 0.5f;
      }
    }
  } else {
    // Media: arbitrary normals drawn from the free-flight block (volumetric.rs:147-153)
    uint32_t vi = s.prim_id - sc.vol_base;
    U4 b = ctx.vol_u ? U4{0, 0, 0, 0} : ctx.block(kPurposeVolume0 + vi);
    s.normal = unit_sphere_from(u01(b.y), u01(b.z));
    s.ray_normal = s.normal;
    s.front = true;
    s.u = s.v = u01(b.w);
    if (F & F_EXT) s.pos_l = s.pos;  // volumetric.rs:143
  }
}

// A transformed object's hit, rebuilt in mesh space (the same ray and
// distance as its test) and mapped out (ObjectTransform::
// outgoing_intersection, transform.rs:101-130): the point by the transform,
// both normals by its linear part and normalised (the reference maps normals
// with the transform itself, not its inverse transpose). Not inlined: the
// untransformed path keeps its registers.
template <uint32_t F, bool UV>
__device__ __forceinline__ void finalize_xformed(const GpuScene& sc, const GpuPrim& p, uint32_t kind, const Ray& rw,
                                              const HitRec& h, const RngCtx& ctx, Surface& s, float start) {
  const float* xf = prim_xform_of(sc, h.prim);
  finalize_prim<F, UV>(sc, p, kind, xf_incoming(xf, rw), h.tl, ctx, s, start);
  s.pos = xf_point(xf + 12, s.pos);
  s.pos_l = xf_point(xf + 12, s.pos_l);  // the reference maps pos_l as a point too (transform.rs:123)
  s.normal = normalize3(xf_vector(xf + 12, s.normal));
  s.ray_normal = normalize3(xf_vector(xf + 12, s.ray_normal));
}

// Full hit record of the closest hit. UV: also the texture coordinates that
// only the Uv render mode reads (sphere, cylinder and infinite-plane uv cost
// transcendentals or extra fetches; the other kinds compute them anyway).
template <uint32_t F, bool UV = (F & F_EXT) != 0>
__device__ __forceinline__ void finalize_hit(const GpuScene& sc, const Ray& rw, const HitRec& h, const RngCtx& ctx, Surface& s,
                                             float start) {
  if ((F & (F_SDF | F_PLANE)) && h.sdf >= 0) {
    const GpuSdf& f = sc.sdfs[h.sdf];
    s.pos = at3(rw.o, rw.d, h.t);
    // pos_l: the raymarched point itself (raymarched.rs:104-105), a plane's
    // point less its corner (planar/mod.rs:176)
    if (F & F_EXT) s.pos_l = ((F & F_PLANE) && f.kind == kUnboundedPlane) ? s.pos - v3(f.p1, f.p2, f.p3) : s.pos;
    s.normal = h.sh.n;
    // raymarched.rs:113-114: not flipped; planar/mod.rs:190: -n * signum(denom)
    s.ray_normal = h.sh.flip ? -h.sh.n : h.sh.n;
    if (UV && (F & F_PLANE) && f.kind == kUnboundedPlane) {
      float u, v;
      planar_uv(sc.quad_ext + 9ull * f.max_iter, v3(f.p1, f.p2, f.p3), s.pos, u, v);
      wrap_uv(__float_as_uint(f.pad[0]), u, v);
      s.front = h.sh.front;
      s.material = f.material;
      s.prim_id = f.prim_id;
      s.side = 0;
      s.u = u; s.v = v;
      return;
    }
    s.front = h.sh.front;
    s.material = f.material;
    s.prim_id = f.prim_id;
    s.side = h.sh.side;
    s.u = s.v = 0.0f;
    return;
  }
  const GpuPrim p = sc.prims[h.prim];
  const uint32_t kind = prim_kind(p);
  s.material = prim_material(p);
  s.prim_id = prim_id(p);
  if ((F & F_EXT) && (__float_as_uint(p.a.w) & kXformBit)) finalize_xformed<F, UV>(sc, p, kind, rw, h, ctx, s, start);
  else finalize_prim<F, UV>(sc, p, kind, rw, h.t, ctx, s, start);
}

// ---------------------------------------------------------------------------
// Materials, sky
// ---------------------------------------------------------------------------
struct C3f { float r, g, b; };

// Skybox::sky_colour (skybox/simple.rs:12-30, skybox/none.rs:8-13)
__device__ __forceinline__ C3f sky_colour(uint32_t sky, V3 dir) {
  if (sky == RG_SKY_WHITE) return C3f{1.0f, 1.0f, 1.0f};
  if (sky == RG_SKY_NONE) return C3f{0.0f, 0.0f, 0.0f};
  float a = 0.5f * dir.y + 0.5f;
  return C3f{1.0f + (0.5f - 1.0f) * a, 1.0f + (0.7f - 1.0f) * a, 1.0f + (1.0f - 1.0f) * a};
}

}  // namespace rg
#include "texture.cuh"
namespace rg {

// The sky of a missed ray: an HdrImageSkybox samples its image at
// sphere_uv(dir), v flipped (skybox/hdri.rs:17-26).
template <uint32_t F>
__device__ __forceinline__ C3f sky_of(const GpuScene& sc, V3 dir) {
  if ((F & F_EXT) && sc.sky == RG_SKY_IMAGE) {
    float u, v;
    sphere_uv(dir, u, v);
    const GpuImage im = sc.images[sc.sky_image];
    return image_bilinear(sc, sc.sky_image, u * (float)im.width, (1.0f - v) * (float)im.height);
  }
  return sky_colour(sc.sky, dir);
}

// Material::scatter (material/*.rs) with inverse-CDF samplers of the same
// distributions as the reference's rejection samplers.
__device__ __forceinline__ bool scatter(const rg_material& m, const Ray& ray, const Surface& s, const RngCtx& ctx, V3& out) {
  U4 b = ctx.block(kPurposeScatter);
  switch (m.kind) {
    case RG_MAT_LAMBERTIAN: {
      // uniform in the unit ball: uniform direction times cbrt(U) radius
      const float two_pi = (float)(2.0 * 3.14159265358979323846);
      float z = 1.0f - 2.0f * u01(b.x);
      float phi = two_pi * u01(b.y);
      float sn = __fsqrt_rn(fmaxf(0.0f, 1.0f - z * z));
      float rad = cbrtf(u01(b.z));
      V3 rnd = v3(sn * cosf(phi) * rad, sn * sinf(phi) * rad, z * rad);
      V3 vec = s.ray_normal + rnd;
      if (!try_normalize3(vec, out)) out = s.ray_normal;
      return true;
    }
    case RG_MAT_METAL: {
      V3 d = ray.d;
      V3 refl = d - s.ray_normal * (2.0f * dot3(d, s.ray_normal));
      V3 rnd = unit_sphere_from(u01(b.x), u01(b.y));
      V3 vec = refl + rnd * m.fuzz;
      if (!(dot3(vec, s.ray_normal) > 0.0f)) return false;
      out = normalize3(vec);
      return true;
    }
    case RG_MAT_DIELECTRIC: {
      float ior = m.refractive_index;
      float ratio = s.front ? __frcp_rn(ior) : ior;
      V3 d = ray.d;
      float cos_t = fminf(dot3(-d, s.ray_normal), 1.0f);
      float sin_t = __fsqrt_rn(1.0f - cos_t * cos_t);
      bool tir = ratio * sin_t > 1.0f;
      float r0 = (1.0f - ratio) / (1.0f + ratio);
      float r02 = r0 * r0;
      float x = 1.0f - cos_t;
      float x2 = x * x;
      float x5 = (x2 * x2) * x;
      float refl_p = r02 + (1.0f - r02) * x5;
      bool schlick = refl_p > u01(b.x);
      if (tir || schlick) {
        out = d - s.ray_normal * (2.0f * dot3(d, s.ray_normal));
      } else {  // math::refract (shared/math.rs:20-25)
        float c2 = fminf(dot3(-d, s.ray_normal), 1.0f);
        V3 perp = (d + s.ray_normal * c2) * ratio;
        V3 par = s.ray_normal * (-__fsqrt_rn(fabsf(1.0f - dot3(perp, perp))));
        out = perp + par;
      }
      return true;
    }
    case RG_MAT_ISOTROPIC:
      out = unit_sphere_from(u01(b.x), u01(b.y));
      return true;
    default:
      return false;
  }
}

// Material::reflected_light as the factor multiplying future_col.
template <uint32_t F>
__device__ __forceinline__ C3f attenuation(const GpuScene& sc, const rg_material& m, const Ray& ray, const Surface& s) {
  if (m.kind == RG_MAT_DIELECTRIC && s.front) return C3f{1.0f, 1.0f, 1.0f};
  const C3f alb = material_colour<F>(sc, m, s);
  if (m.kind == RG_MAT_LAMBERTIAN || m.kind == RG_MAT_METAL) return alb;
  float dist = length3(s.pos - ray.o);
  float e = expf(-m.density * dist);
  return C3f{alb.r * e, alb.g * e, alb.b * e};
}

// ---------------------------------------------------------------------------
// RG_FLAG_VALIDATE: the invariants of shared/validate.rs:21-197 (number,
// normal3, uv, colour, intersection), counted instead of asserted.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool finite3(V3 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }
// approx::relative_eq with epsilon 1e-6 and max_relative 1e-3 (validate.rs:14-16)
__device__ __forceinline__ bool rel_eq(float a, float b) {
  const float d = fabsf(a - b);
  return d <= 1e-6f || d <= 1e-3f * fmaxf(fabsf(a), fabsf(b));
}
static __device__ __noinline__ void validate_hit(const FrameParams& fp, const Ray& r, float t, const Surface& s, float start,
                                          float end) {
  uint32_t bad = 0;
  if (!isfinite(t) || !finite3(s.pos) || !finite3(s.normal) || !finite3(s.ray_normal)) bad |= RG_INVALID_NONFINITE;
  // unit length within the reference's relative tolerance 1e-3 (its f64
  // normals pass glam's tighter is_normalized; an f32 sphere normal (p - c) / r
  // carries the root's rounding divided by r, up to a few 1e-4 for small,
  // distant spheres)
  if (!(fabsf(dot3(s.normal, s.normal) - 1.0f) <= 2e-3f) || !(fabsf(dot3(s.ray_normal, s.ray_normal) - 1.0f) <= 2e-3f))
    bad |= RG_INVALID_NOT_NORMALISED;
  if (!(start <= t && t <= end)) bad |= RG_INVALID_INTERVAL;
  const V3 at = at3(r.o, r.d, t);
  if (!rel_eq(length3(s.pos - r.o), t) || !rel_eq(s.pos.x, at.x) || !rel_eq(s.pos.y, at.y) || !rel_eq(s.pos.z, at.z))
    bad |= RG_INVALID_POSITION;
  if (!(s.u >= 0.0f && s.u <= 1.0f && s.v >= 0.0f && s.v <= 1.0f)) bad |= RG_INVALID_UV;
  if (bad) {
    atomicAdd(fp.counters + CNT_INVALID, 1ull);
    atomicOr(fp.counters + CNT_INVALID_MASK, (unsigned long long)bad);
  }
}
__device__ __forceinline__ void validate_colour(const FrameParams& fp, C3f c) {
  if (!(isfinite(c.r) && isfinite(c.g) && isfinite(c.b) && c.r >= 0.0f && c.g >= 0.0f && c.b >= 0.0f)) {
    atomicAdd(fp.counters + CNT_INVALID, 1ull);
    atomicOr(fp.counters + CNT_INVALID_MASK, (unsigned long long)RG_INVALID_COLOUR);
  }
}

// ---------------------------------------------------------------------------
// Camera: render_px_msaa stratification (render/renderer.rs:350-389) and
// Viewport::calc_ray (scene/camera.rs:191-213).
// ---------------------------------------------------------------------------
__device__ __forceinline__ Ray camera_ray(const FrameParams& fp, uint32_t x, uint32_t y, uint32_t s, const RngCtx& ctx) {
  const float two_pi = (float)(2.0 * 3.14159265358979323846);
  U4 b = philox(ctx.pix, ctx.smp, kCameraDepth, kPurposeCamera, ctx.k0, ctx.k1);
  float jx = u01(b.x) - 0.5f, jy = u01(b.y) - 0.5f;
  float lr = __fsqrt_rn(u01(b.z));
  float ph = two_pi * u01(b.w);
  float lx = lr * cosf(ph), ly = lr * sinf(ph);
  float fx, fy;
  uint32_t d = fp.strat_d;
  if (s < d * d) {
    float dinv = fp.strat_inv;
    uint32_t i = s % d, j = s / d;
    fx = ((float)x + jx * dinv) + (float)i * dinv;
    fy = ((float)y + jy * dinv) + (float)j * dinv;
  } else {
    fx = (float)x + jx;
    fy = (float)y + jy;
  }
  float w = (float)fp.width, h = (float)fp.height;
  float u = (fx - (w / 2.0f)) / h;
  float v = (fy - (h / 2.0f)) / h;
  V3 pc = v3(fp.pixel_center[0], fp.pixel_center[1], fp.pixel_center[2]);
  V3 vu = v3(fp.viewport_u[0], fp.viewport_u[1], fp.viewport_u[2]);
  V3 vv = v3(fp.viewport_v[0], fp.viewport_v[1], fp.viewport_v[2]);
  V3 pos = v3(fp.pos[0], fp.pos[1], fp.pos[2]);
  V3 du = v3(fp.defocus_u[0], fp.defocus_u[1], fp.defocus_u[2]);
  V3 dv = v3(fp.defocus_v[0], fp.defocus_v[1], fp.defocus_v[2]);
  V3 ps = (pc + vu * u) + vv * v;
  V3 rpos = (pos + du * lx) + dv * ly;
  return make_ray(rpos, ps - rpos);
}

// What a megakernel sample computes (k_megakernel's KIND): the PBR path with
// one scattered ray per bounce, a debug render mode, or ray_branching > 1.
enum : uint32_t { kSamplePbr = 0, kSampleMode = 1, kSampleBranch = 2 };

// Render::render_px_once for the debug modes (renderer.rs:427-490): one
// intersection of the camera ray, coloured by mode; the sky on a miss.
template <uint32_t F, bool COUNT, class Stack>
__device__ C3f mode_sample(const GpuScene& sc, const FrameParams& fp, const Ray& ray, RngCtx& ctx, Counters& cnt,
                           uint32_t& segments, Stack& stack) {
  ctx.depth = 0;
  HitRec h;
  ++segments;
  if (!closest_hit_with<F, COUNT>(stack, sc, ray, 1e-3f, 3.402823466e38f, ctx, h, cnt, fp.err)) return sky_of<F>(sc, ray.d);
  Surface s;
  finalize_hit<F, true>(sc, ray, h, ctx, s, 1e-3f);
  // The reference's visualisation colours (renderer.rs:439-453)
  const float kCol[13][3] = {{1, 1, 1}, {1, 0, 0},     {1, 0.5f, 0}, {1, 1, 0}, {0.5f, 1, 0},  {0, 1, 0}, {0, 1, 0.5f},
                             {0, 1, 1}, {0, 0.5f, 1}, {0, 0, 1},    {0.5f, 0, 1}, {1, 0, 1}, {0, 0, 0}};
  auto half = [](V3 v) { return C3f{v.x / 2.0f + 0.5f, v.y / 2.0f + 0.5f, v.z / 2.0f + 0.5f}; };
  switch (fp.mode) {
    case RG_MODE_OUTWARD_NORMAL:
      return half(s.normal);
    case RG_MODE_RAY_NORMAL:
      return half(s.ray_normal);
    case RG_MODE_SCATTER: {
      V3 dir = v3(0.0f, 0.0f, 0.0f);  // unwrap_or_default
      if (!scatter(sc.materials[s.material], ray, s, ctx, dir)) dir = v3(0.0f, 0.0f, 0.0f);
      return half(dir);
    }
    case RG_MODE_UV:
      return C3f{fminf(fmaxf(s.u, 0.0f), 1.0f), fminf(fmaxf(s.v, 0.0f), 1.0f), 0.0f};
    case RG_MODE_FRONT_FACE: {
      const float* c = kCol[s.front ? 1 : 0];
      return C3f{c[0], c[1], c[2]};
    }
    case RG_MODE_SIDE: {
      const float* c = kCol[s.side % 12u + 1u];
      return C3f{c[0], c[1], c[2]};
    }
    default: {  // RG_MODE_DISTANCE
      const float val = 2.0f * cbrtf(h.t);
      const float fl = fminf(fmaxf(floorf(val), 0.0f), 12.0f), ce = fminf(fmaxf(ceilf(val), 0.0f), 12.0f);
      const float frac = val - fl;
      const float* a = kCol[(int)fl];
      const float* b = kCol[(int)ce];
      return C3f{a[0] + (b[0] - a[0]) * frac, a[1] + (b[1] - a[1]) * frac, a[2] + (b[2] - a[2]) * frac};
    }
  }
}

// ray_colour_recursive with ray_branching b > 1 (renderer.rs:508-572): every
// surface hit below ray_depth spawns b scattered rays and averages their
// colours. Walked depth-first with an explicit stack; each tree node keeps its
// weight (the product of attenuation / b down to it), so a node adds weight x
// (emission or sky). Random streams are keyed by node: node n's children are
// n b + 1 + i, its free-flight draws use key n and the scatter of branch i key
// n b + i (for b = 1 these reduce to the depth keys of the PBR path).
template <uint32_t F, bool COUNT, class Stack>
__device__ C3f branch_sample(const GpuScene& sc, const FrameParams& fp, Ray ray, RngCtx& ctx, Counters& cnt,
                             uint32_t& segments, Stack& stack) {
  struct Level {
    Surface surf;
    Ray in;
    C3f w;
    uint32_t node, next;
  };
  Level st[kBranchStack];
  int top = -1;
  const uint32_t b = fp.branching;
  const float inv_b = 1.0f / (float)b;
  C3f L{0.0f, 0.0f, 0.0f}, w{1.0f, 1.0f, 1.0f};
  uint32_t node = 0, depth = 0;
  for (;;) {
    ctx.depth = node;
    HitRec h;
    ++segments;
    if (!closest_hit_with<F, COUNT>(stack, sc, ray, 1e-3f, 3.402823466e38f, ctx, h, cnt, fp.err)) {
      const C3f sk = sky_of<F>(sc, ray.d);
      L = C3f{L.r + w.r * sk.r, L.g + w.g * sk.g, L.b + w.b * sk.b};
    } else {
      Surface surf;
      finalize_hit<F>(sc, ray, h, ctx, surf, 1e-3f);
      const rg_material m = sc.materials[surf.material];
      if (m.kind == RG_MAT_LIGHT) {
        const C3f e = material_colour<F>(sc, m, surf);
        L = C3f{L.r + w.r * e.r, L.g + w.g * e.g, L.b + w.b * e.b};
      } else if (depth < fp.ray_depth && top + 1 < kBranchStack) {
        ++top;
        st[top] = Level{surf, ray, w, node, 0u};
      }
    }
    // next child: the deepest level with branches left
    bool found = false;
    while (top >= 0) {
      Level& lv = st[top];
      if (lv.next >= b) {
        --top;
        continue;
      }
      const uint32_t i = lv.next++;
      const rg_material m = sc.materials[lv.surf.material];
      ctx.depth = lv.node * b + i;
      V3 dir;
      if (!scatter(m, lv.in, lv.surf, ctx, dir)) continue;  // a black branch
      const C3f a = attenuation<F>(sc, m, lv.in, lv.surf);
      w = C3f{lv.w.r * a.r * inv_b, lv.w.g * a.g * inv_b, lv.w.b * a.b * inv_b};
      ray = make_ray(lv.surf.pos, dir);
      node = lv.node * b + 1u + i;
      depth = (uint32_t)top + 1u;
      found = true;
      break;
    }
    if (!found) break;
  }
  return L;
}

// One sample of pixel (x, y); `s` is the sample's index among the pixel's
// spp_total samples. PBR: ray_colour_recursive (renderer.rs:508-572)
// evaluated front to back, L = sum_k beta_k * emitted_k + beta_K * sky.
template <uint32_t F, bool COUNT, uint32_t KIND, class Stack>
__device__ C3f trace_path(const GpuScene& sc, const FrameParams& fp, uint32_t x, uint32_t y, uint32_t s, Counters& cnt,
                          uint32_t& segments, Stack& stack) {
  RngCtx ctx{fp.seed_lo, fp.seed_hi, y * fp.width + x, s, 0, nullptr};
  Ray ray = camera_ray(fp, x, y, s, ctx);
  if (KIND == kSampleMode) return mode_sample<F, COUNT>(sc, fp, ray, ctx, cnt, segments, stack);
  if (KIND == kSampleBranch) return branch_sample<F, COUNT>(sc, fp, ray, ctx, cnt, segments, stack);
  C3f L{0.0f, 0.0f, 0.0f}, beta{1.0f, 1.0f, 1.0f};
  for (uint32_t depth = 0; depth <= fp.ray_depth; ++depth) {
    ctx.depth = depth;
    HitRec h;
    ++segments;
    if (!closest_hit_with<F, COUNT>(stack, sc, ray, 1e-3f, 3.402823466e38f, ctx, h, cnt, fp.err)) {
      C3f sk = sky_of<F>(sc, ray.d);
      L = C3f{L.r + beta.r * sk.r, L.g + beta.g * sk.g, L.b + beta.b * sk.b};
      break;
    }
    Surface surf;
    finalize_hit<F>(sc, ray, h, ctx, surf, 1e-3f);
    if (COUNT && fp.validate) validate_hit(fp, ray, h.t, surf, 1e-3f, 3.402823466e38f);
    const rg_material m = sc.materials[surf.material];
    if (m.kind == RG_MAT_LIGHT) {
      const C3f e = material_colour<F>(sc, m, surf);
      L = C3f{L.r + beta.r * e.r, L.g + beta.g * e.g, L.b + beta.b * e.b};
      break;
    }
    V3 dir;
    if (!scatter(m, ray, surf, ctx, dir)) break;
    C3f a = attenuation<F>(sc, m, ray, surf);
    beta = C3f{beta.r * a.r, beta.g * a.g, beta.b * a.b};
    ray = make_ray(surf.pos, dir);
  }
  if (COUNT && fp.validate) validate_colour(fp, L);
  return L;
}

}  // namespace rg
