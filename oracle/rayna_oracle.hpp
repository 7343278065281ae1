// rayna_oracle.hpp — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of rayna_engine's per-sample path-tracing path (the
// reference is the Rust crate rayna_engine of v0x0g/rayna). Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg use this code, as
// the checker; the GPU library never links it.
//
// Parity status: PARTIALLY PINNED. The reference cannot be compiled in this
// environment (no Rust toolchain, no crate registry, git-over-ssh patched
// dependencies), so no reference output can be generated. The only known
// answers the reference's own tests hold for this path are the four pixel
// class checks of rayna_engine/tests/simple_renders.rs:22-142; tests/
// pins this oracle against them and against closed-form cases (furnace
// identities, analytic sphere/triangle hits). Everything else — including
// the glam vector arithmetic (dot, cross, normalize/try_normalize) and the
// `rand` streams, which are entropy-seeded in the reference — is unpinned:
// the restatement follows the documented behaviour of those crates.
//
// Two arithmetic policies:
//   RefF64 — f64 with the reference's operation order (glam scalar
//            formulas, no fused multiply-add). Faithful to the reference.
//   GpuF32 — f32 with the operation order and explicit fused multiply-adds
//            of the CUDA kernels, so closed-form intersections (sphere,
//            triangle, box, slab) are bit-identical to the device.
// Two sampler modes:
//   kRefSampling — the reference's rejection samplers on a sequential
//                  per-path stream (rng.rs:64-142).
//   kGpuSampling — the device's inverse-CDF samplers and its counter
//                  assignment, so paths can be compared one by one.
// Compile with -ffp-contract=off: every fused multiply-add is explicit.
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <thread>
#include <type_traits>
#include <vector>

#include "../include/rayna_gpu.h"

namespace orc {

// ---------------------------------------------------------------------------
// Counter-based random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11).
// ---------------------------------------------------------------------------
struct U4 { uint32_t v[4]; };

inline U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)M0 * c.v[0];
    uint64_t p1 = (uint64_t)M1 * c.v[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    U4 n;
    n.v[0] = hi1 ^ c.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ c.v[3] ^ k1;
    n.v[3] = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// [0,1) and (0,1] floats from the top 24 bits (the device uses the same maps).
inline float u01f(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }
inline float u01f_open0(uint32_t x) { return ((float)(x >> 8) + 1.0f) * (1.0f / 16777216.0f); }
inline double u01d(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// Counter purposes of the device's random-number assignment.
enum : uint32_t { kPurposeCamera = 0, kPurposeScatter = 1, kPurposeVolume0 = 2 };

// Sequential stream used in the reference-sampling mode: one Philox block of
// four words per refill, counter (a, b, c, k++).
struct SeqRng {
  uint32_t k0, k1, a, b, c, k = 0;
  U4 buf{};
  int left = 0;
  SeqRng(uint64_t seed, uint32_t a_, uint32_t b_, uint32_t c_)
      : k0((uint32_t)seed), k1((uint32_t)(seed >> 32)), a(a_), b(b_), c(c_) {}
  uint32_t next_u32() {
    if (left == 0) {
      buf = philox4x32_10(U4{{a, b, c, k++}}, k0, k1);
      left = 4;
    }
    return buf.v[4 - (left--)];
  }
  double gen() { uint32_t x = next_u32(); uint32_t y = next_u32(); return u01d(x, y); }  // rng.gen::<f64>() in [0,1)
  double range_incl(double lo, double hi) { return lo + (hi - lo) * gen(); }           // gen_range(lo..=hi)
};

// ---------------------------------------------------------------------------
// Arithmetic policies.
// ---------------------------------------------------------------------------
struct RefF64 { using T = double; static constexpr bool gpu = false; };
struct GpuF32 { using T = float; static constexpr bool gpu = true; };

template <class T> struct V3 { T x, y, z; };
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline T comp(V3<T> v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// The device's natural logarithm (trace.cuh, ln_f32), operation for
// operation: x = m 2^e with m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh(s) by
// the series of Abramowitz & Stegun 4.1.27 to s^9, e ln 2 in two parts. The
// f32 policy uses it for the free-flight distance and the Mandelbulb; the f64
// policy uses std::log.
inline float ln_f32(float x) {
  if (!(x > 0.0f)) return x == 0.0f ? -std::numeric_limits<float>::infinity() : std::numeric_limits<float>::quiet_NaN();
  if (std::isinf(x)) return x;
  int e = 0;
  if (x < 1.17549435e-38f) { x = x * 8388608.0f; e = -23; }
  uint32_t bits;
  std::memcpy(&bits, &x, 4);
  e += (int)((bits >> 23) & 0xFFu) - 127;
  const uint32_t mb = (bits & 0x7FFFFFu) | 0x3F800000u;
  float m;
  std::memcpy(&m, &mb, 4);
  if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = std::fma(s2, 0.111111111f, 0.142857143f);
  p = std::fma(s2, p, 0.2f);
  p = std::fma(s2, p, 0.333333333f);
  p = std::fma(s2, p, 1.0f);
  const float lm = (2.0f * s) * p;
  const float fe = (float)e;
  return std::fma(fe, 0.693145751953125f, std::fma(fe, 1.42860676533018e-06f, lm));
}
template <class T> inline T policy_log(T x) {
  if constexpr (std::is_same_v<T, float>) return ln_f32(x);
  else return std::log(x);
}

template <class P> struct Math {
  using T = typename P::T;
  using V = V3<T>;
  // glam: (x*x') + (y*y') + (z*z'); device: fma(x,x', fma(y,y', z*z')).
  static T dot(V a, V b) {
    if constexpr (P::gpu) return std::fma(a.x, b.x, std::fma(a.y, b.y, a.z * b.z));
    else return a.x * b.x + a.y * b.y + a.z * b.z;
  }
  static V cross(V a, V b) {
    if constexpr (P::gpu)
      return {std::fma(a.y, b.z, -(a.z * b.y)), std::fma(a.z, b.x, -(a.x * b.z)), std::fma(a.x, b.y, -(a.y * b.x))};
    else
      return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
  }
  // Ray::at: pos + dir * t
  static V at(V o, V d, T t) {
    if constexpr (P::gpu) return {std::fma(d.x, t, o.x), std::fma(d.y, t, o.y), std::fma(d.z, t, o.z)};
    else return o + d * t;
  }
  static T length(V v) { return std::sqrt(dot(v, v)); }
  // glam normalize: self * (1 / length)
  static V normalize(V v) { T r = T(1) / length(v); return v * r; }
  // glam try_normalize: Some(self * rcp) if rcp is finite and > 0
  static bool try_normalize(V v, V& out) {
    T r = T(1) / length(v);
    if (std::isfinite(r) && r > T(0)) { out = v * r; return true; }
    return false;
  }
  static T signum(T x) { return std::isnan(x) ? x : std::copysign(T(1), x); }
};

// ---------------------------------------------------------------------------
// Ray, Interval, Aabb (shared/ray.rs, shared/interval.rs, shared/aabb.rs)
// ---------------------------------------------------------------------------
template <class P> struct Ray {
  using T = typename P::T;
  V3<T> pos, dir, inv;
  // Ray::new (ray.rs:15-23): normalise the direction and store its reciprocal.
  static Ray make(V3<T> p, V3<T> d) {
    Ray r;
    r.pos = p;
    r.dir = Math<P>::normalize(d);
    r.inv = {T(1) / r.dir.x, T(1) / r.dir.y, T(1) / r.dir.z};
    return r;
  }
};

template <class T> struct Interval {
  bool has_start = false, has_end = false;
  T start = 0, end = 0;
  static Interval full() { return Interval{}; }
  static Interval range(T s, T e) { Interval i; i.has_start = i.has_end = true; i.start = s; i.end = e; return i; }
  static Interval from(T s) { Interval i; i.has_start = true; i.start = s; return i; }
  // interval.rs:108-124
  bool contains(T x) const {
    if (has_start && has_end) return start <= x && x <= end;
    if (has_start) return start <= x;
    if (has_end) return x <= end;
    return true;
  }
  // interval.rs:67-93
  bool range_overlaps(T mn, T mx) const {
    if (!has_start && !has_end) return true;
    if (has_start && has_end) {
      T low = mn > start ? mn : start;
      T high = mx < end ? mx : end;
      return low <= high;
    }
    if (has_end) { T high = mx < end ? mx : end; return mn <= high; }
    T low = mn > start ? mn : start;
    return low <= mx;
  }
  Interval with_end(T e) const { Interval i = *this; i.has_end = true; i.end = e; return i; }
};

template <class T> struct Aabb {
  V3<T> mn{0, 0, 0}, mx{0, 0, 0};  // Default: a zero box at the origin (aabb.rs:16, derive(Default))
  static Aabb make(V3<T> a, V3<T> b) {
    Aabb r;
    r.mn = {std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)};
    r.mx = {std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)};
    return r;
  }
  static Aabb encompass(const Aabb& a, const Aabb& b) { return make(V3<T>{std::fmin(a.mn.x, b.mn.x), std::fmin(a.mn.y, b.mn.y), std::fmin(a.mn.z, b.mn.z)}, V3<T>{std::fmax(a.mx.x, b.mx.x), std::fmax(a.mx.y, b.mx.y), std::fmax(a.mx.z, b.mx.z)}); }
  // aabb.rs:37-38: ((sx*sy) + (sy*sz) + (sz*sx)) * 2
  double area() const {
    double sx = (double)mx.x - (double)mn.x, sy = (double)mx.y - (double)mn.y, sz = (double)mx.z - (double)mn.z;
    return ((sx * sy) + (sy * sz) + (sz * sx)) * 2.0;
  }
};

// Aabb::hit (aabb.rs:117-153). The GpuF32 policy follows the device, which
// widens the exit side by 2^-20 relative so that roundoff never rejects a box
// the ray meets (Ize, "Robust BVH Ray Traversal", JCGT 2013); the RefF64
// policy is the reference's exact test.
template <class P> inline bool aabb_hit(const Aabb<typename P::T>& b, const Ray<P>& r, const Interval<typename P::T>& iv) {
  using T = typename P::T;
  T t1[3], t2[3];
  for (int a = 0; a < 3; ++a) {
    T lo = comp(b.mn, a), hi = comp(b.mx, a), o = comp(r.pos, a), inv = comp(r.inv, a);
    t1[a] = (lo - o) * inv;
    t2[a] = (hi - o) * inv;
  }
  T tmin = std::fmin(t1[0], t2[0]);
  T tmax = std::fmax(t1[0], t2[0]);
  tmin = std::fmax(tmin, std::fmin(t1[1], t2[1]));
  tmax = std::fmin(tmax, std::fmax(t1[1], t2[1]));
  tmin = std::fmax(tmin, std::fmin(t1[2], t2[2]));
  tmax = std::fmin(tmax, std::fmax(t1[2], t2[2]));
  if constexpr (P::gpu) {
    T low = tmin > iv.start ? tmin : iv.start;
    T high = tmax < iv.end ? tmax : iv.end;
    return low <= std::fma(std::fabs(high), T(9.5367431640625e-7), high);
  } else {
    return iv.range_overlaps(tmin, tmax);
  }
}

// Intersection (shared/intersect.rs:8-43) plus the material and primitive.
template <class T> struct Hit {
  T dist = 0;
  V3<T> pos_w{0, 0, 0}, normal{0, 0, 0}, ray_normal{0, 0, 0};
  V3<T> pos_l{0, 0, 0};  // the mesh-local point (noise textures)
  bool front_face = false;
  T u = 0, v = 0;
  uint32_t side = 0;
  uint32_t prim = 0;
  uint32_t material = 0;
};

// ---------------------------------------------------------------------------
// Meshes
// ---------------------------------------------------------------------------
template <class P> struct Sphere {
  using T = typename P::T;
  V3<T> c; T r, r2;
  Aabb<T> aabb() const { V3<T> s{r, r, r}; return Aabb<T>::make(c - s, c + s); }  // sphere.rs:34
  // SphereMesh::intersect (sphere.rs:44-99)
  bool intersect(const Ray<P>& ray, const Interval<T>& iv, Hit<T>& h) const {
    V3<T> oc = ray.pos - c;
    T root, far_root;
    if constexpr (P::gpu) {
      // the device's form: disc = r^2 - |oc - half_b d|^2, roots q and c / q
      // (trace.cuh sphere_t; Ray Tracing Gems 2019, "Precision Improvements
      // for Ray/Sphere Intersection")
      const T half_b = Math<P>::dot(oc, ray.dir);
      const V3<T> l{std::fma(-half_b, ray.dir.x, oc.x), std::fma(-half_b, ray.dir.y, oc.y),
                    std::fma(-half_b, ray.dir.z, oc.z)};
      const T disc = r2 - Math<P>::dot(l, l);
      if (disc < T(0)) return false;
      const T cc = std::fma(oc.x, oc.x, std::fma(oc.y, oc.y, std::fma(oc.z, oc.z, -r2)));
      const T sq = std::sqrt(disc);
      const T q = half_b > T(0) ? -half_b - sq : -half_b + sq;
      const T other = q != T(0) ? cc / q : q;
      root = std::fmin(q, other);
      far_root = std::fmax(q, other);
    } else {
      const T half_b = Math<P>::dot(oc, ray.dir);
      const T cc = Math<P>::dot(oc, oc) - r2;
      const T disc = (half_b * half_b) - cc;
      if (disc < T(0)) return false;
      const T sq = std::sqrt(disc);
      root = -half_b - sq;
      far_root = -half_b + sq;
    }
    if (!iv.contains(root)) {
      root = far_root;
      if (!iv.contains(root)) return false;
    }
    h.dist = root;
    h.pos_w = Math<P>::at(ray.pos, ray.dir, root);
    V3<T> local = (h.pos_w - c) / r;
    h.normal = local;
    bool inside = Math<P>::dot(ray.dir, local) > T(0);
    h.ray_normal = inside ? -local : local;
    h.front_face = !inside;
    // sphere_uv (sphere.rs:114-121)
    T theta = std::acos(-local.y);
    T phi = std::atan2(-local.z, local.x) + T(M_PI);
    h.u = phi / T(2 * M_PI);
    h.pos_l = local;
    h.v = theta / T(M_PI);
    h.side = 0;
    return true;
  }
};

template <class P> struct Triangle {
  using T = typename P::T;
  V3<T> v0, v1, v2, n0, n1, n2;
  Aabb<T> aabb() const {  // Aabb::encompass_points (aabb.rs:70-80)
    V3<T> mn{std::fmin(std::fmin(v0.x, v1.x), v2.x), std::fmin(std::fmin(v0.y, v1.y), v2.y), std::fmin(std::fmin(v0.z, v1.z), v2.z)};
    V3<T> mx{std::fmax(std::fmax(v0.x, v1.x), v2.x), std::fmax(std::fmax(v0.y, v1.y), v2.y), std::fmax(std::fmax(v0.z, v1.z), v2.z)};
    return Aabb<T>::make(mn, mx);
  }
  V3<T> centre() const { return (v0 + v1 + v2) / T(3); }
  // Triangle::intersect (triangle.rs:53-109), Moller-Trumbore.
  bool intersect(const Ray<P>& ray, const Interval<T>& iv, Hit<T>& h) const {
    using M = Math<P>;
    V3<T> e1 = v1 - v0, e2 = v2 - v0;
    V3<T> pvec = M::cross(ray.dir, e2);
    T det = M::dot(e1, pvec);
    if (det == T(0)) return false;
    T inv_det = T(1) / det;
    V3<T> tvec = ray.pos - v0;
    T u = M::dot(tvec, pvec) * inv_det;
    if (u < T(0) || u > T(1)) return false;
    V3<T> qvec = M::cross(tvec, e1);
    T v = M::dot(ray.dir, qvec) * inv_det;
    if (v < T(0) || u + v > T(1)) return false;
    T t = M::dot(e2, qvec) * inv_det;
    if (!iv.contains(t)) return false;
    T b0 = (T(1) - u) - v;
    // interpolate_normals (triangle.rs:114-119): fold from zero, then try_normalize
    V3<T> n;
    if constexpr (P::gpu) {
      n = {std::fma(n2.x, v, std::fma(n1.x, u, n0.x * b0)), std::fma(n2.y, v, std::fma(n1.y, u, n0.y * b0)),
           std::fma(n2.z, v, std::fma(n1.z, u, n0.z * b0))};
    } else {
      n = (n0 * b0 + n1 * u) + n2 * v;
    }
    V3<T> nn;
    if (!M::try_normalize(n, nn)) return false;  // opposing vertex normals: a miss
    h.dist = t;
    h.pos_w = M::at(ray.pos, ray.dir, t);
    h.front_face = std::signbit(det);
    h.u = u;
    h.v = v;
    h.pos_l = {T(1) - u - v, u, v};  // barycentric (triangle.rs:92-101)
    h.side = 0;
    h.normal = nn;
    h.ray_normal = nn * (-M::signum(det));
    return true;
  }
};

template <class P> struct AxisBox {
  using T = typename P::T;
  V3<T> centre, radius, inv_radius;
  Aabb<T> box;
  static AxisBox make(V3<T> a, V3<T> b) {  // axis_box.rs:29-37
    AxisBox r;
    r.box = Aabb<T>::make(a, b);
    r.centre = (r.box.mn + r.box.mx) / T(2);
    V3<T> size = r.box.mx - r.box.mn;
    r.radius = size / T(2);
    r.inv_radius = {T(1) / r.radius.x, T(1) / r.radius.y, T(1) / r.radius.z};
    return r;
  }
  Aabb<T> aabb() const { return box; }
  // AxisBoxMesh::intersect (axis_box.rs:64-145), Majercik et al. 2018.
  bool intersect(const Ray<P>& ray, const Interval<T>& iv, Hit<T>& h) const {
    using M = Math<P>;
    V3<T> ro = ray.pos - centre;
    V3<T> rd = ray.dir;
    V3<T> q = {std::fabs(ro.x) * inv_radius.x, std::fabs(ro.y) * inv_radius.y, std::fabs(ro.z) * inv_radius.z};
    T winding = M::signum(std::fmax(q.x, std::fmax(q.y, q.z)) - T(1));
    V3<T> sgn = {-M::signum(rd.x), -M::signum(rd.y), -M::signum(rd.z)};
    V3<T> pd = {((radius.x * winding) * sgn.x - ro.x) * ray.inv.x, ((radius.y * winding) * sgn.y - ro.y) * ray.inv.y,
                ((radius.z * winding) * sgn.z - ro.z) * ray.inv.z};
    for (int ax = 0; ax < 3; ++ax) {
      T dist = comp(pd, ax);
      if (!iv.contains(dist)) continue;
      int a1 = ax == 0 ? 1 : (ax == 1 ? 2 : 0);  // x: yz, y: zx, z: xy
      int a2 = ax == 0 ? 2 : (ax == 1 ? 0 : 1);
      T u0, u1;
      if constexpr (P::gpu) {
        u0 = std::fma(comp(rd, a1), dist, comp(ro, a1));
        u1 = std::fma(comp(rd, a2), dist, comp(ro, a2));
      } else {
        u0 = comp(ro, a1) + comp(rd, a1) * dist;
        u1 = comp(ro, a2) + comp(rd, a2) * dist;
      }
      T r1 = comp(radius, a1), r2 = comp(radius, a2);
      if (std::fabs(u0) < r1 && std::fabs(u1) < r2) {
        T s = comp(sgn, ax);
        V3<T> rn{0, 0, 0};
        if (ax == 0) rn.x = s; else if (ax == 1) rn.y = s; else rn.z = s;
        h.dist = dist;
        h.pos_w = M::at(ray.pos, ray.dir, dist);
        h.ray_normal = rn;
        h.normal = rn * winding;
        h.front_face = !std::signbit(winding);
        h.u = (u0 / r1 + T(1)) / T(2);
        h.pos_l = h.pos_w - centre;
        h.v = (u1 / r2 + T(1)) / T(2);
        h.side = (uint32_t)ax * 2u + (s > T(0) ? 1u : 0u);
        return true;
      }
    }
    return false;
  }
};

// Planar (mesh/planar/mod.rs:33-194). n, d and w are derived in f64 exactly
// as Planar::new does; the f32 policy takes them rounded to f32, as the device
// does.
template <class P> struct Planar {
  using T = typename P::T;
  V3<T> p, u, v, n, w;
  T d;
  static bool make(const float* q, Planar& out) {
    double pp[3], uu[3], vv[3];
    for (int k = 0; k < 3; ++k) { pp[k] = q[k]; uu[k] = q[3 + k]; vv[k] = q[6 + k]; }
    const double nr[3] = {uu[1] * vv[2] - vv[1] * uu[2], uu[2] * vv[0] - vv[2] * uu[0], uu[0] * vv[1] - vv[0] * uu[1]};
    const double l2 = nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2];
    const double rl = 1.0 / std::sqrt(l2);
    if (!std::isfinite(rl) || !(rl > 0.0)) return false;
    const double nn[3] = {nr[0] * rl, nr[1] * rl, nr[2] * rl};
    out.p = {(T)pp[0], (T)pp[1], (T)pp[2]};
    out.u = {(T)uu[0], (T)uu[1], (T)uu[2]};
    out.v = {(T)vv[0], (T)vv[1], (T)vv[2]};
    out.n = {(T)nn[0], (T)nn[1], (T)nn[2]};
    out.d = (T)(-(nn[0] * pp[0] + nn[1] * pp[1] + nn[2] * pp[2]));
    out.w = {(T)(nr[0] / l2), (T)(nr[1] / l2), (T)(nr[2] / l2)};
    return true;
  }
  // Planar::intersect_bounded (mod.rs:161-194)
  bool intersect(const Ray<P>& ray, const Interval<T>& iv, Hit<T>& h) const {
    using M = Math<P>;
    T denom = M::dot(n, ray.dir);
    if (denom == T(0)) return false;
    T t = -(M::dot(n, ray.pos) + d) / denom;
    if (!iv.contains(t)) return false;
    h.dist = t;
    h.pos_w = M::at(ray.pos, ray.dir, t);
    V3<T> pl = h.pos_w - p;
    h.pos_l = pl;
    h.u = M::dot(w, M::cross(pl, v));
    h.v = M::dot(w, M::cross(u, pl));
    h.normal = n;
    h.front_face = std::signbit(denom);
    h.ray_normal = (-n) * M::signum(denom);
    h.side = 0;
    return true;
  }
};

// ParallelogramMesh (mesh/planar/parallelogram.rs): the plane hit with uv in [0, 1]^2.
template <class P> struct Parallelogram {
  using T = typename P::T;
  Planar<P> pl;
  Aabb<T> aabb() const {  // encompass the corners, min_padded(AABB_PADDING = 1e-6) (parallelogram.rs:24-34)
    V3<T> c[4] = {pl.p, pl.p + pl.u, pl.p + pl.v, pl.p + pl.u + pl.v};
    V3<T> mn = c[0], mx = c[0];
    for (int k = 1; k < 4; ++k) {
      mn = {std::fmin(mn.x, c[k].x), std::fmin(mn.y, c[k].y), std::fmin(mn.z, c[k].z)};
      mx = {std::fmax(mx.x, c[k].x), std::fmax(mx.y, c[k].y), std::fmax(mx.z, c[k].z)};
    }
    V3<T> size = mx - mn, centre = mn + size / T(2);
    size = {std::fmax(size.x, T(1e-6)), std::fmax(size.y, T(1e-6)), std::fmax(size.z, T(1e-6))};
    return Aabb<T>::make(centre - size / T(2), centre + size / T(2));
  }
  bool intersect(const Ray<P>& ray, const Interval<T>& iv, Hit<T>& h) const {
    if (!pl.intersect(ray, iv, h)) return false;
    return h.u >= T(0) && h.u <= T(1) && h.v >= T(0) && h.v <= T(1);
  }
};

// CylinderMesh (mesh/primitive/cylinder.rs:24-183). The f32 policy follows the
// device's operation order (explicit fused multiply-adds; the body roots
// evaluated without the discriminant's cancellation) and, like the
// device, evaluates the test against [start, inf) before clipping to the
// interval's end: the reference's test is not monotone in the end (a cap
// nearer than the body roots is dropped when both roots lie beyond it), so
// only the open-ended evaluation is independent of the traversal order. The
// f64 policy keeps the reference's exact semantics. uv is left at 0.
template <class P> struct Cylinder {
  using T = typename P::T;
  V3<T> origin, along;
  T lsq, length, radius;
  static Cylinder make(const float* c) {
    const double al[3] = {(double)c[3] - c[0], (double)c[4] - c[1], (double)c[5] - c[2]};
    const double l2 = al[0] * al[0] + al[1] * al[1] + al[2] * al[2];
    Cylinder y;
    y.origin = {(T)c[0], (T)c[1], (T)c[2]};
    y.along = {(T)al[0], (T)al[1], (T)al[2]};
    y.lsq = (T)l2;
    y.length = (T)std::sqrt(l2);
    y.radius = (T)c[6];
    return y;
  }
  Aabb<T> aabb() const {
    V3<T> p2 = origin + along, r{radius, radius, radius};
    V3<T> mn{std::fmin(origin.x, p2.x), std::fmin(origin.y, p2.y), std::fmin(origin.z, p2.z)};
    V3<T> mx{std::fmax(origin.x, p2.x), std::fmax(origin.y, p2.y), std::fmax(origin.z, p2.z)};
    return Aabb<T>::make(mn - r, mx + r);
  }
  bool intersect(const Ray<P>& ray, const Interval<T>& iv_in, Hit<T>& h) const {
    if constexpr (P::gpu) {
      Interval<T> open = iv_in;
      open.has_end = false;
      return test(ray, open, h) && iv_in.contains(h.dist);
    } else {
      return test(ray, iv_in, h);
    }
  }
  bool test(const Ray<P>& ray, const Interval<T>& iv, Hit<T>& h) const {
    using M = Math<P>;
    V3<T> rd = ray.dir, oc = ray.pos - origin;
    T bard = M::dot(along, rd), baoc = M::dot(along, oc);
    T a, b, c, disc, sq, dist;
    if constexpr (P::gpu) {
      // the device's evaluation of the same roots without the discriminant's
      // cancellation (trace.cuh, cylinder_t): components normal to the axis,
      // the closest approach to the axis, roots q / a and c / q
      a = std::fma(-bard, bard, lsq);
      if (a == T(0)) return false;
      V3<T> dp{std::fma(lsq, rd.x, -(bard * along.x)), std::fma(lsq, rd.y, -(bard * along.y)),
               std::fma(lsq, rd.z, -(bard * along.z))};
      V3<T> op{std::fma(lsq, oc.x, -(baoc * along.x)), std::fma(lsq, oc.y, -(baoc * along.y)),
               std::fma(lsq, oc.z, -(baoc * along.z))};
      b = M::dot(op, rd);
      c = std::fma(-(radius * radius), lsq, M::dot(op, op) / lsq);
      T k = b / a;
      V3<T> w{std::fma(-k, dp.x, op.x), std::fma(-k, dp.y, op.y), std::fma(-k, dp.z, op.z)};
      disc = a * std::fma(radius * radius, lsq, -(M::dot(w, w) / lsq));
      if (disc < T(0)) return false;
      sq = std::sqrt(disc);
      T q = b > T(0) ? -b - sq : -b + sq;
      T r1 = q / a, r2 = q != T(0) ? c / q : q;
      dist = std::fmin(r1, r2);
      if (!iv.contains(dist)) dist = std::fmax(r1, r2);
      if (!iv.contains(dist)) return false;
    } else {
      a = lsq - bard * bard;
      b = lsq * M::dot(oc, rd) - baoc * bard;
      c = lsq * M::dot(oc, oc) - baoc * baoc - radius * radius * lsq;
      disc = b * b - c * a;
      if (disc < T(0)) return false;
      sq = std::sqrt(disc);
      dist = (-b - sq) / a;
      if (!iv.contains(dist)) dist = (-b + sq) / a;
      if (!iv.contains(dist)) return false;
    }
    T dan;
    if constexpr (P::gpu) dan = std::fma(dist, bard, baoc) / lsq;
    else dan = (baoc + dist * bard) / lsq;
    V3<T> normal;
    uint32_t face;
    if (dan > T(0) && dan < T(1)) {
      V3<T> rel = M::at(oc, rd, dist);
      V3<T> out = rel - along * dan;
      normal = out / radius;
      face = 0;
    } else {
      T dn, df;
      if (std::signbit(baoc) == std::signbit(bard)) { dn = (T(0) - baoc) / bard; df = (lsq - baoc) / bard; }
      else { dn = (lsq - baoc) / bard; df = (T(0) - baoc) / bard; }
      dn = std::fmin(dn, df);
      df = std::fmax(dn, df);  // as the reference: max of the new near and the far
      auto radial = [&](T x) { if constexpr (P::gpu) return std::fabs(std::fma(a, x, b)); else return std::fabs(b + a * x); };
      if (iv.contains(dn) && radial(dn) < sq) dist = dn;
      else if (iv.contains(df) && radial(df) < sq) dist = df;
      else return false;
      normal = (along / length) * M::signum(dan);
      face = std::signbit(dan) ? 1u : 2u;
    }
    T inside = -M::signum(M::dot(rd, normal));
    h.dist = dist;
    h.pos_w = M::at(ray.pos, ray.dir, dist);
    h.normal = normal;
    h.ray_normal = normal * inside;
    h.front_face = std::signbit(inside);
    h.side = face;
    h.pos_l = h.pos_w - (origin + along / T(2));  // less the centre (cylinder.rs:171)
    // uv (cylinder.rs:130-172) in the frame of Vector3::any_orthonormal_pair of the axis
    V3<T> o0, o1;
    orthonormal_pair(along / length, o0, o1);
    if (face == 0) {
      T theta = std::acos(M::dot(normal, o1)) * M::signum(M::dot(normal, o0));
      h.u = theta / T(M_PI) / T(2) + T(0.5);
      h.v = dan;
    } else {
      V3<T> q = M::at(oc, rd, dist) / radius;
      h.u = M::dot(q, o0) / T(2) + T(0.5);
      h.v = M::dot(q, o1) / T(2) + T(0.5);
    }
    return true;
  }
  // Duff et al., "Building an Orthonormal Basis, Revisited" (JCGT 2017), the
  // method of glam's any_orthonormal_pair.
  static void orthonormal_pair(V3<T> n, V3<T>& b1, V3<T>& b2) {
    T sign = std::copysign(T(1), n.z);
    T a = T(-1) / (sign + n.z);
    T b = n.x * n.y * a;
    b1 = {T(1) + sign * n.x * n.x * a, sign * b, -sign * n.x};
    b2 = {b, sign + n.y * n.y * a, -n.y};
  }
};

// UvWrappingMode::apply (mesh/planar/infinite_plane.rs:26-41)
template <class T> inline void wrap_uv(uint32_t mode, T& u, T& v) {
  if (mode == RG_UV_WRAP) {
    u = std::fmod(u, T(1)); if (u < T(0)) u = u + T(1);
    v = std::fmod(v, T(1)); if (v < T(0)) v = v + T(1);
  } else if (mode == RG_UV_MIRROR) {
    u = std::fabs(std::fmod(u, T(2)) - T(1));
    v = std::fabs(std::fmod(v, T(2)) - T(1));
  } else if (!(T(0) <= u && u <= T(1) && T(0) <= v && v <= T(1))) {
    u = v = T(0);
  }
}

// Signed distance functions evaluated in world space.
template <class P> struct Sdf {
  using T = typename P::T;
  uint32_t kind;
  V3<T> c;
  T p[4];
  uint32_t max_iter;
  T eps;
  // Bounding radius outside of which the function is replaced by the
  // distance to an enclosing sphere (a valid lower bound of the distance).
  static constexpr double kBulbInner = 1.2, kBulbOuter = 1.5;
  T eval(V3<T> x) const {
    V3<T> q = x - c;
    if (kind == RG_SDF_SPHERE) return Math<P>::length(q) - p[0];
    if (kind == RG_SDF_TORUS) {
      if constexpr (P::gpu) {  // the device's explicit fused multiply-adds
        T a = std::sqrt(std::fma(q.x, q.x, q.z * q.z)) - p[0];
        return std::sqrt(std::fma(a, a, q.y * q.y)) - p[1];
      }
      T a = std::sqrt(q.x * q.x + q.z * q.z) - p[0];
      return std::sqrt(a * a + q.y * q.y) - p[1];
    }
    // Mandelbulb distance estimator (spherical-coordinate power map with the
    // running derivative; Hart et al. 1989 / the standard escape-time DE).
    T s = p[2];
    V3<T> z0 = q / s;
    T rq = Math<P>::length(z0);
    if (rq > T(kBulbOuter)) return (rq - T(kBulbInner)) * s;
    T power = p[0];
    int iters = (int)p[1];
    V3<T> z = z0;
    T dr = T(1), r = T(0);
    if (power == T(8)) {
      // z^8 without transcendentals: w = z + i rho (|w| = r, arg w = t) squared
      // three times is r^8 (cos 8t + i sin 8t); the azimuth's unit complex
      // number (x + i y) / rho squared three times is cos 8p + i sin 8p.
      for (int i = 0; i < iters; ++i) {
        T rho2, r2;
        if constexpr (P::gpu) {  // the device's explicit fused multiply-adds
          rho2 = std::fma(z.x, z.x, z.y * z.y);
          r2 = std::fma(z.z, z.z, rho2);
        } else {
          rho2 = z.x * z.x + z.y * z.y;
          r2 = rho2 + z.z * z.z;
        }
        r = std::sqrt(r2);
        if (r > T(2)) break;
        T rho = std::sqrt(rho2);
        T wa = z.z, wb = rho, cp = T(1), sp = T(0);
        if (rho > T(0)) {
          T inv = T(1) / rho;
          cp = z.x * inv;
          sp = z.y * inv;
        }
        for (int k = 0; k < 3; ++k) {
          T a2, d2;
          if constexpr (P::gpu) a2 = std::fma(wa, wa, -(wb * wb));
          else a2 = wa * wa - wb * wb;
          wb = T(2) * wa * wb;
          wa = a2;
          if constexpr (P::gpu) d2 = std::fma(cp, cp, -(sp * sp));
          else d2 = cp * cp - sp * sp;
          sp = T(2) * cp * sp;
          cp = d2;
        }
        T r4 = r2 * r2;
        if constexpr (P::gpu) {
          dr = std::fma((r4 * r2 * r) * T(8), dr, T(1));
          z = V3<T>{std::fma(wb, cp, z0.x), std::fma(wb, sp, z0.y), wa + z0.z};
        } else {
          dr = (r4 * r2 * r) * T(8) * dr + T(1);
          z = V3<T>{wb * cp + z0.x, wb * sp + z0.y, wa + z0.z};
        }
      }
      return (T(0.5) * policy_log(r) * r / dr) * s;
    }
    for (int i = 0; i < iters; ++i) {
      r = Math<P>::length(z);
      if (r > T(2)) break;
      T theta = std::acos(z.z / r);
      T phi = std::atan2(z.y, z.x);
      T zr = std::pow(r, power);
      T st;
      if constexpr (P::gpu) {
        dr = std::fma(std::pow(r, power - T(1)) * power, dr, T(1));
        theta = theta * power;
        phi = phi * power;
        st = std::sin(theta);
        z = V3<T>{std::fma(zr, st * std::cos(phi), z0.x), std::fma(zr, std::sin(phi) * st, z0.y),
                  std::fma(zr, std::cos(theta), z0.z)};
      } else {
        dr = std::pow(r, power - T(1)) * power * dr + T(1);
        theta = theta * power;
        phi = phi * power;
        st = std::sin(theta);
        z = V3<T>{zr * (st * std::cos(phi)), zr * (std::sin(phi) * st), zr * std::cos(theta)} + z0;
      }
    }
    return (T(0.5) * policy_log(r) * r / dr) * s;
  }
  // RaymarchedIsosurfaceMesh::intersect (raymarched.rs:73-122)
  bool intersect(const Ray<P>& ray, const Interval<T>& iv, Hit<T>& h) const {
    T total = iv.has_start ? iv.start : T(0);
    V3<T> point = Math<P>::at(ray.pos, ray.dir, total);
    uint32_t i = 0;
    for (;;) {
      T d = eval(point);
      total = total + std::fabs(d);
      point = Math<P>::at(ray.pos, ray.dir, total);
      if (std::fabs(d) < eps && iv.contains(total)) {
        V3<T> pp = point;
        V3<T> g{eval(V3<T>{pp.x + eps, pp.y, pp.z}) - eval(V3<T>{pp.x - eps, pp.y, pp.z}),
                eval(V3<T>{pp.x, pp.y + eps, pp.z}) - eval(V3<T>{pp.x, pp.y - eps, pp.z}),
                eval(V3<T>{pp.x, pp.y, pp.z + eps}) - eval(V3<T>{pp.x, pp.y, pp.z - eps})};
        V3<T> n = Math<P>::normalize(g);
        h.dist = total;
        h.pos_w = pp;
        h.pos_l = pp;
        h.normal = n;
        h.ray_normal = n;
        h.front_face = !std::signbit(d);
        h.u = h.v = 0;
        h.side = i;
        return true;
      }
      if (i > max_iter) return false;
      ++i;
    }
  }
};

// ---------------------------------------------------------------------------
// Sampling
// ---------------------------------------------------------------------------
// Per-path random source. In kGpuSampling mode it reproduces the device's
// counter assignment: block (pixel, sample, depth, purpose).
struct PathRng {
  bool gpu;
  uint64_t seed;
  uint32_t pixel, sample;
  SeqRng seq;
  const float* injected_volume_u = nullptr;  // query mode: per-volume uniforms
  PathRng(bool g, uint64_t s, uint32_t px, uint32_t smp)
      : gpu(g), seed(s), pixel(px), sample(smp), seq(s, px, smp, 0x52u) {}
  U4 block(uint32_t depth, uint32_t purpose) const {
    return philox4x32_10(U4{{pixel, sample, depth, purpose}}, (uint32_t)seed, (uint32_t)(seed >> 32));
  }
};

template <class T> inline V3<T> unit_sphere_from(T r1, T r2) {
  // normal_on_unit_sphere (rng.rs:75-87)
  T two_pi = T(2 * M_PI);
  T s = T(2) * std::sqrt(r2 * (T(1) - r2));
  return {std::cos(two_pi * r1) * s, std::sin(two_pi * r1) * s, T(1) - T(2) * r2};
}

// ---------------------------------------------------------------------------
// Scene
// ---------------------------------------------------------------------------
enum ObjKind : uint32_t { OBJ_SPHERE, OBJ_TRIANGLE, OBJ_MESH, OBJ_BOX, OBJ_VOLUME, OBJ_SDF, OBJ_QUAD, OBJ_CYLINDER };

// ---------------------------------------------------------------------------
// ObjectTransform (object/transform.rs): 3 x 4 affine matrices, row-major.
// ---------------------------------------------------------------------------
// [A | t]^-1 = [A^-1 | -A^-1 t] in double, A^-1 from cofactors; false if A is
// singular. The device's host build computes the same, then rounds to f32.
inline bool affine_inverse(const double* m, double* inv) {
  const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], hh = m[9], i = m[10];
  const double c00 = e * i - f * hh, c01 = f * g - d * i, c02 = d * hh - e * g;
  const double det = a * c00 + b * c01 + c * c02;
  if (!std::isfinite(det) || det == 0.0) return false;
  const double r = 1.0 / det;
  const double A[9] = {c00 * r, (c * hh - b * i) * r, (b * f - c * e) * r,
                       c01 * r, (a * i - c * g) * r, (c * d - a * f) * r,
                       c02 * r, (b * g - a * hh) * r, (a * e - b * d) * r};
  for (int row = 0; row < 3; ++row) {
    for (int k = 0; k < 3; ++k) inv[4 * row + k] = A[3 * row + k];
    inv[4 * row + 3] = -(A[3 * row] * m[3] + A[3 * row + 1] * m[7] + A[3 * row + 2] * m[11]);
  }
  for (int k = 0; k < 12; ++k)
    if (!std::isfinite(inv[k])) return false;
  return true;
}

// Transform3::map_point / map_vector. RefF64: glam's column order
// ((c0 x + c1 y) + c2 z) + t; GpuF32: the device's fma chain.
template <class P> inline V3<typename P::T> xf_point(const typename P::T* m, V3<typename P::T> p) {
  if constexpr (P::gpu)
    return {std::fma(m[0], p.x, std::fma(m[1], p.y, std::fma(m[2], p.z, m[3]))),
            std::fma(m[4], p.x, std::fma(m[5], p.y, std::fma(m[6], p.z, m[7]))),
            std::fma(m[8], p.x, std::fma(m[9], p.y, std::fma(m[10], p.z, m[11])))};
  else
    return {((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3], ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
            ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]};
}
template <class P> inline V3<typename P::T> xf_vector(const typename P::T* m, V3<typename P::T> v) {
  if constexpr (P::gpu)
    return {std::fma(m[0], v.x, std::fma(m[1], v.y, m[2] * v.z)), std::fma(m[4], v.x, std::fma(m[5], v.y, m[6] * v.z)),
            std::fma(m[8], v.x, std::fma(m[9], v.y, m[10] * v.z))};
  else
    return {(m[0] * v.x + m[1] * v.y) + m[2] * v.z, (m[4] * v.x + m[5] * v.y) + m[6] * v.z,
            (m[8] * v.x + m[9] * v.y) + m[10] * v.z};
}

template <class P> struct Xform {
  using T = typename P::T;
  T inv[12], fwd[12];
  double fwd64[12];
  // ObjectTransform::incoming_ray (transform.rs:90-97)
  Ray<P> incoming(const Ray<P>& r) const { return Ray<P>::make(xf_point<P>(inv, r.pos), xf_vector<P>(inv, r.dir)); }
  // ObjectTransform::outgoing_intersection (transform.rs:101-130): the point
  // at the mesh-space distance mapped out, both normals by the transform's
  // linear part and normalised, the distance recomputed in world space.
  void outgoing(const Ray<P>& world, const Ray<P>& local, Hit<T>& h) const {
    h.pos_w = xf_point<P>(fwd, Math<P>::at(local.pos, local.dir, h.dist));
    h.pos_l = xf_point<P>(fwd, h.pos_l);
    h.normal = Math<P>::normalize(xf_vector<P>(fwd, h.normal));
    h.ray_normal = Math<P>::normalize(xf_vector<P>(fwd, h.ray_normal));
    h.dist = Math<P>::length(h.pos_w - world.pos);
  }
  // ObjectTransform::calculate_aabb (transform.rs:133-144): the mapped
  // corners, encompassed. In f64, rounded outward for the f32 policy.
  Aabb<T> map_box(const Aabb<T>& b) const {
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
      const double q[3] = {(double)((c & 1) ? b.mx.x : b.mn.x), (double)((c & 2) ? b.mx.y : b.mn.y),
                           (double)((c & 4) ? b.mx.z : b.mn.z)};
      for (int a = 0; a < 3; ++a) {
        const double v = ((fwd64[4 * a] * q[0] + fwd64[4 * a + 1] * q[1]) + fwd64[4 * a + 2] * q[2]) + fwd64[4 * a + 3];
        mn[a] = std::min(mn[a], v);
        mx[a] = std::max(mx[a], v);
      }
    }
    Aabb<T> r;
    auto dn = [](double v) { return P::gpu ? (T)std::nextafter((float)v, -INFINITY) : (T)v; };
    auto up = [](double v) { return P::gpu ? (T)std::nextafter((float)v, INFINITY) : (T)v; };
    r.mn = {dn(mn[0]), dn(mn[1]), dn(mn[2])};
    r.mx = {up(mx[0]), up(mx[1]), up(mx[2])};
    return r;
  }
};

template <class P> struct Scene;

// GenericBvh node (shared/generic_bvh.rs:30-36): Nested(aabb) with children,
// or Object(item).
template <class T> struct BvhNode {
  bool is_item = false;
  uint32_t item = 0;
  Aabb<T> box;
  std::vector<uint32_t> children;
};

template <class T> struct Bvh {
  std::vector<BvhNode<T>> nodes;
  int root = -1;
};

// Exhaustive SAH builder of GenericBvh::generate_nodes_sah (generic_bvh.rs:
// 97-290): two binary splits per node (up to four children), leaves of at most
// 8 items, costs from boxes folded from the origin-anchored default box. The
// per-split box folds are computed by prefix/suffix sweeps (the same boxes as
// the reference's per-split Aabb::encompass_iter, in O(n) per axis).
template <class T> struct RefBvhBuilder {
  const std::vector<Aabb<T>>& boxes;
  Bvh<T>& out;
  explicit RefBvhBuilder(const std::vector<Aabb<T>>& b, Bvh<T>& o) : boxes(b), out(o) {}

  Aabb<T> fold(const uint32_t* it, size_t n) const {
    Aabb<T> a;  // default: zero box at the origin
    for (size_t i = 0; i < n; ++i) a = Aabb<T>::encompass(a, boxes[it[i]]);
    return a;
  }
  void sort_axis(std::vector<uint32_t>& v, int ax) const {
    std::stable_sort(v.begin(), v.end(), [&](uint32_t a, uint32_t b) { return comp(boxes[a].mn, ax) < comp(boxes[b].mn, ax); });
  }
  // calculate_optimal_split::<1, 2> (generic_bvh.rs:173-290)
  bool split(std::vector<uint32_t>& v, int& best_axis, size_t& best_left) const {
    size_t n = v.size();
    if (n <= 2) return false;
    bool have = false;
    double best = 0;
    std::vector<Aabb<T>> pre(n + 1), suf(n + 1);
    for (int ax = 0; ax < 3; ++ax) {
      sort_axis(v, ax);
      pre[0] = Aabb<T>();
      for (size_t i = 0; i < n; ++i) pre[i + 1] = Aabb<T>::encompass(pre[i], boxes[v[i]]);
      suf[n] = Aabb<T>();
      for (size_t i = n; i-- > 0;) suf[i] = Aabb<T>::encompass(suf[i + 1], boxes[v[i]]);
      for (size_t p = 1; p + 2 <= n; ++p) {  // split positions 1 ..= n-2
        double cost = (double)p * pre[p].area() + (double)(n - p) * suf[p].area();
        if (!have || cost < best) { have = true; best = cost; best_axis = ax; best_left = p; }
      }
    }
    return have;
  }
  uint32_t leaf(uint32_t item) {
    BvhNode<T> nd; nd.is_item = true; nd.item = item; nd.box = boxes[item];
    out.nodes.push_back(nd);
    return (uint32_t)out.nodes.size() - 1;
  }
  uint32_t build(std::vector<uint32_t> v) {
    if (v.size() == 1) return leaf(v[0]);
    uint32_t me = (uint32_t)out.nodes.size();
    out.nodes.push_back(BvhNode<T>{});
    out.nodes[me].box = fold(v.data(), v.size());
    if (v.size() <= 8) {
      for (uint32_t it : v) { uint32_t c = leaf(it); out.nodes[me].children.push_back(c); }
      return me;
    }
    int ax; size_t p;
    split(v, ax, p);
    sort_axis(v, ax);
    std::vector<uint32_t> parts[2] = {std::vector<uint32_t>(v.begin(), v.begin() + p), std::vector<uint32_t>(v.begin() + p, v.end())};
    for (auto& part : parts) {
      int ax2; size_t p2;
      if (split(part, ax2, p2)) {
        sort_axis(part, ax2);
        std::vector<uint32_t> a(part.begin(), part.begin() + p2), b(part.begin() + p2, part.end());
        uint32_t ca = build(std::move(a)); out.nodes[me].children.push_back(ca);
        uint32_t cb = build(std::move(b)); out.nodes[me].children.push_back(cb);
      } else {
        uint32_t c = build(std::move(part)); out.nodes[me].children.push_back(c);
      }
    }
    return me;
  }
};

// Binned SAH builder (16 bins, leaves of at most 4 items) for inputs too large
// for the reference's exhaustive builder. Deviation from the reference, used
// only for the tree shape: traversal results are independent of it except for
// exact-distance ties.
template <class T> struct BinnedBvhBuilder {
  const std::vector<Aabb<T>>& boxes;
  std::vector<V3<double>> cent;
  Bvh<T>& out;
  BinnedBvhBuilder(const std::vector<Aabb<T>>& b, Bvh<T>& o) : boxes(b), out(o) {
    cent.resize(b.size());
    for (size_t i = 0; i < b.size(); ++i)
      cent[i] = {0.5 * ((double)b[i].mn.x + b[i].mx.x), 0.5 * ((double)b[i].mn.y + b[i].mx.y), 0.5 * ((double)b[i].mn.z + b[i].mx.z)};
  }
  uint32_t build(uint32_t* it, size_t n) {
    uint32_t me = (uint32_t)out.nodes.size();
    out.nodes.push_back(BvhNode<T>{});
    Aabb<T> bb = boxes[it[0]];
    for (size_t i = 1; i < n; ++i) bb = Aabb<T>::encompass(bb, boxes[it[i]]);
    out.nodes[me].box = bb;
    auto make_leaf = [&]() {
      for (size_t i = 0; i < n; ++i) {
        BvhNode<T> nd; nd.is_item = true; nd.item = it[i]; nd.box = boxes[it[i]];
        out.nodes.push_back(nd);
        out.nodes[me].children.push_back((uint32_t)out.nodes.size() - 1);
      }
      return me;
    };
    if (n <= 4) return make_leaf();
    double cmin[3] = {1e300, 1e300, 1e300}, cmax[3] = {-1e300, -1e300, -1e300};
    for (size_t i = 0; i < n; ++i) for (int a = 0; a < 3; ++a) { double c = comp(cent[it[i]], a); cmin[a] = std::min(cmin[a], c); cmax[a] = std::max(cmax[a], c); }
    const int B = 16;
    double best = 1e300; int bax = -1, bsplit = -1;
    for (int a = 0; a < 3; ++a) {
      double ext = cmax[a] - cmin[a];
      if (!(ext > 0)) continue;
      Aabb<T> bin[B]; int cnt[B] = {0}; bool init[B] = {false};
      for (size_t i = 0; i < n; ++i) {
        int k = std::min(B - 1, (int)((comp(cent[it[i]], a) - cmin[a]) / ext * B));
        bin[k] = init[k] ? Aabb<T>::encompass(bin[k], boxes[it[i]]) : boxes[it[i]]; init[k] = true; cnt[k]++;
      }
      double la[B], ra[B]; int lc[B], rc[B];
      Aabb<T> acc; bool ai = false; int c = 0;
      for (int k = 0; k < B; ++k) { if (init[k]) { acc = ai ? Aabb<T>::encompass(acc, bin[k]) : bin[k]; ai = true; } c += cnt[k]; la[k] = ai ? acc.area() : 0; lc[k] = c; }
      ai = false; c = 0;
      for (int k = B - 1; k >= 0; --k) { if (init[k]) { acc = ai ? Aabb<T>::encompass(acc, bin[k]) : bin[k]; ai = true; } c += cnt[k]; ra[k] = ai ? acc.area() : 0; rc[k] = c; }
      for (int k = 0; k + 1 < B; ++k) {
        if (lc[k] == 0 || rc[k + 1] == 0) continue;
        double cost = lc[k] * la[k] + rc[k + 1] * ra[k + 1];
        if (cost < best) { best = cost; bax = a; bsplit = k; }
      }
    }
    size_t mid;
    if (bax < 0) {
      mid = n / 2;  // all centroids coincide: median split
    } else {
      double ext = cmax[bax] - cmin[bax];
      uint32_t* m = std::partition(it, it + n, [&](uint32_t i) { return std::min(B - 1, (int)((comp(cent[i], bax) - cmin[bax]) / ext * B)) <= bsplit; });
      mid = (size_t)(m - it);
      if (mid == 0 || mid == n) mid = n / 2;
    }
    uint32_t l = build(it, mid);
    out.nodes[me].children.push_back(l);
    uint32_t r = build(it + mid, n - mid);
    out.nodes[me].children.push_back(r);
    return me;
  }
};

template <class T> inline void build_bvh(const std::vector<Aabb<T>>& boxes, Bvh<T>& out, size_t exact_limit) {
  out.nodes.clear();
  out.root = -1;
  if (boxes.empty()) return;
  std::vector<uint32_t> idx(boxes.size());
  for (size_t i = 0; i < idx.size(); ++i) idx[i] = (uint32_t)i;
  if (boxes.size() <= exact_limit) {
    RefBvhBuilder<T> b(boxes, out);
    out.root = (int)b.build(std::move(idx));
  } else {
    BinnedBvhBuilder<T> b(boxes, out);
    out.root = (int)b.build(idx.data(), idx.size());
  }
}

struct Options {
  bool prim_pretest = true;    // test each leaf object's own Aabb first (object/bvh.rs:100-106)
  bool brute_force = false;    // no bounding volumes: every primitive, in object order
  size_t exact_bvh_limit = 200000;
};

// ---------------------------------------------------------------------------
// Colour arithmetic is f32 (Channel), as in the reference.
// ---------------------------------------------------------------------------
struct C3 { float r, g, b; };
inline C3 operator+(C3 a, C3 b) { return {a.r + b.r, a.g + b.g, a.b + b.b}; }
inline C3 operator*(C3 a, C3 b) { return {a.r * b.r, a.g * b.g, a.b * b.b}; }
inline C3 operator*(C3 a, float s) { return {a.r * s, a.g * s, a.b * s}; }

// ---------------------------------------------------------------------------
// Textures (texture/*.rs), images (core/image.rs), the image sky (skybox/hdri.rs)
// ---------------------------------------------------------------------------
// A noise source's permutation: Fisher-Yates over 0..255 driven by SplitMix64
// (Steele, Lea and Flood, OOPSLA 2014) seeded with `seed`, repeated to 512.
inline void noise_permutation(uint32_t seed, uint8_t* out) {
  uint64_t state = seed;
  auto next = [&]() {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  uint8_t p[256];
  for (int i = 0; i < 256; ++i) p[i] = (uint8_t)i;
  for (int i = 255; i > 0; --i) std::swap(p[i], p[next() % (uint64_t)(i + 1)]);
  for (int i = 0; i < 512; ++i) out[i] = p[i & 255];
}

// Perlin's improved noise (SIGGRAPH 2002) in T, the operation order of the
// device's perlin3.
template <class T> inline T perlin_fade(T t) { return t * t * t * (t * (t * T(6) - T(15)) + T(10)); }
template <class T> inline T perlin_lerp(T t, T a, T b) { return a + t * (b - a); }
template <class T> inline T perlin_grad(uint32_t h, T x, T y, T z) {
  h &= 15u;
  const T u = h < 8u ? x : y;
  const T v = h < 4u ? y : (h == 12u || h == 14u ? x : z);
  return ((h & 1u) ? -u : u) + ((h & 2u) ? -v : v);
}
// Saturating float-to-int conversion (NaN to 0), as the device's cvt.rzi.
template <class T> inline uint32_t perlin_cell(T f) {
  if (std::isnan(f)) return 0u;
  if (f <= T(-2147483648.0)) return 0x80000000u & 255u;
  if (f >= T(2147483647.0)) return 0x7FFFFFFFu & 255u;
  return (uint32_t)(int64_t)f & 255u;
}
template <class T> inline T perlin3(const uint8_t* perm, T x, T y, T z) {
  const T fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
  const uint32_t X = perlin_cell(fx), Y = perlin_cell(fy), Z = perlin_cell(fz);
  x = x - fx;
  y = y - fy;
  z = z - fz;
  const T u = perlin_fade(x), v = perlin_fade(y), w = perlin_fade(z);
  auto Pm = [&](uint32_t i) { return (uint32_t)perm[i]; };
  const uint32_t A = Pm(X) + Y, AA = Pm(A) + Z, AB = Pm(A + 1u) + Z;
  const uint32_t B = Pm(X + 1u) + Y, BA = Pm(B) + Z, BB = Pm(B + 1u) + Z;
  return perlin_lerp(w,
                     perlin_lerp(v, perlin_lerp(u, perlin_grad(Pm(AA), x, y, z), perlin_grad(Pm(BA), x - T(1), y, z)),
                                 perlin_lerp(u, perlin_grad(Pm(AB), x, y - T(1), z), perlin_grad(Pm(BB), x - T(1), y - T(1), z))),
                     perlin_lerp(v,
                                 perlin_lerp(u, perlin_grad(Pm(AA + 1u), x, y, z - T(1)),
                                             perlin_grad(Pm(BA + 1u), x - T(1), y, z - T(1))),
                                 perlin_lerp(u, perlin_grad(Pm(AB + 1u), x, y - T(1), z - T(1)),
                                             perlin_grad(Pm(BB + 1u), x - T(1), y - T(1), z - T(1)))));
}

struct OImage { uint32_t w = 0, h = 0; std::vector<float> rgb; };  // [x][y][rgb]

// Image::get_bilinear (core/image.rs:87-109). GpuF32: f32 as the device;
// RefF64: coordinates and weights in f64, colours in f32.
template <class P> inline C3 image_bilinear(const OImage& im, typename P::T px, typename P::T py) {
  using T = typename P::T;
  auto coords = [](T val, uint32_t max, uint32_t& lo, uint32_t& hi, T& frac) {
    const T top = (T)(max - 1u);
    T fl = std::floor(val), ce = std::ceil(val);
    fl = std::isnan(fl) ? T(0) : std::fmin(std::fmax(fl, T(0)), top);
    ce = std::isnan(ce) ? T(0) : std::fmin(std::fmax(ce, T(0)), top);
    lo = (uint32_t)fl;
    hi = (uint32_t)ce;
    frac = val - fl;
  };
  uint32_t x1, x2, y1, y2;
  T xl, yl;
  coords(px, im.w, x1, x2, xl);
  coords(py, im.h, y1, y2, yl);
  auto at = [&](uint32_t x, uint32_t y) {
    const float* c = im.rgb.data() + 3 * ((size_t)x * im.h + y);
    return C3{c[0], c[1], c[2]};
  };
  auto lerp = [](C3 a, C3 b, T t) {
    if constexpr (P::gpu) return C3{a.r + (b.r - a.r) * t, a.g + (b.g - a.g) * t, a.b + (b.b - a.b) * t};
    else return C3{(float)(a.r + (double)(b.r - a.r) * t), (float)(a.g + (double)(b.g - a.g) * t),
                   (float)(a.b + (double)(b.b - a.b) * t)};
  };
  return lerp(lerp(at(x1, y1), at(x2, y1), xl), lerp(at(x1, y2), at(x2, y2), xl), yl);
}

// rem_euclid(sum, 2) < 1: the even cells of do_checker (texture/checker.rs:46-63)
template <class T> inline bool checker_even(T sum) {
  T r = std::fmod(sum, T(2));
  if (r < T(0)) r = r + T(2);
  return r < T(1);
}

template <class P> struct Scene {
  using T = typename P::T;
  std::vector<Sphere<P>> spheres;
  std::vector<Triangle<P>> tris;
  std::vector<AxisBox<P>> boxes;
  struct Volume { uint32_t boundary; Sphere<P> s; AxisBox<P> b; T density, neg_inv_density; uint32_t material; };
  std::vector<Volume> volumes;
  std::vector<Sdf<P>> sdfs;
  std::vector<Parallelogram<P>> quads;
  std::vector<Cylinder<P>> cylinders;
  std::vector<Planar<P>> planes;
  std::vector<uint32_t> sphere_mat, tri_mat, box_mat, quad_mat, cyl_mat, plane_mat, plane_wrap;
  std::vector<rg_material> materials;
  uint32_t skybox = RG_SKY_SIMPLE;
  uint32_t ns = 0, nt = 0, nb = 0, nv = 0, nsdf = 0, nq = 0, nc = 0, npl = 0;

  struct Mesh { std::vector<uint32_t> tris; Bvh<T> bvh; uint32_t material; Aabb<T> box; int32_t xf = -1; };
  std::vector<Mesh> meshes;
  std::vector<Xform<P>> xforms;
  std::vector<rg_texture> textures;
  std::vector<uint32_t> tex_perm;  // per texture: first permutation slot (noise)
  std::vector<uint8_t> perm;       // 512 entries per slot
  std::vector<OImage> images;
  uint32_t sky_image = 0;
  std::vector<int32_t> sphere_xf, tri_xf, box_xf, quad_xf, cyl_xf, vol_xf;  // transform index, or -1
  struct Object { uint32_t kind, index; Aabb<T> box; int32_t xf = -1; };
  std::vector<Object> bounded;    // ObjectList::bvh items, in list order
  struct Unbounded { bool plane; uint32_t index; };
  std::vector<Unbounded> unbounded; // SDFs, then infinite planes, in list order
  Bvh<T> top;
  Options opt;

  uint32_t prim_sphere(uint32_t i) const { return i; }
  uint32_t prim_tri(uint32_t i) const { return ns + i; }
  uint32_t prim_box(uint32_t i) const { return ns + nt + i; }
  uint32_t prim_vol(uint32_t i) const { return ns + nt + nb + i; }
  uint32_t prim_sdf(uint32_t i) const { return ns + nt + nb + nv + i; }
  uint32_t prim_quad(uint32_t i) const { return ns + nt + nb + nv + nsdf + i; }
  uint32_t prim_cyl(uint32_t i) const { return ns + nt + nb + nv + nsdf + nq + i; }
  uint32_t prim_plane(uint32_t i) const { return ns + nt + nb + nv + nsdf + nq + nc + i; }

  void load(const rg_scene_desc& d, const Options& o) {
    opt = o;
    ns = d.n_spheres; nt = d.n_triangles; nb = d.n_boxes; nv = d.n_volumes; nsdf = d.n_sdfs;
    nq = d.n_quads; nc = d.n_cylinders; npl = d.n_planes;
    skybox = d.skybox;
    for (uint32_t i = 0; i < nq; ++i) {
      Parallelogram<P> q;
      Planar<P>::make(d.quads + 9 * i, q.pl);
      quads.push_back(q);
      quad_mat.push_back(d.quad_material[i]);
    }
    for (uint32_t i = 0; i < nc; ++i) {
      cylinders.push_back(Cylinder<P>::make(d.cylinders + 7 * i));
      cyl_mat.push_back(d.cylinder_material[i]);
    }
    for (uint32_t i = 0; i < npl; ++i) {
      Planar<P> q;
      Planar<P>::make(d.planes + 9 * i, q);
      planes.push_back(q);
      plane_mat.push_back(d.plane_material[i]);
      plane_wrap.push_back(d.plane_uv_wrap ? d.plane_uv_wrap[i] : (uint32_t)RG_UV_WRAP);
    }
    materials.assign(d.materials, d.materials + d.n_materials);
    textures.assign(d.textures, d.textures + d.n_textures);
    tex_perm.assign(d.n_textures, 0);
    for (uint32_t i = 0; i < d.n_textures; ++i) {
      if (textures[i].kind != RG_TEX_NOISE) continue;
      tex_perm[i] = (uint32_t)(perm.size() / 512);
      for (uint32_t c = 0; c < textures[i].noise_channels; ++c) {
        perm.resize(perm.size() + 512);
        noise_permutation(textures[i].noise_seed + c, perm.data() + perm.size() - 512);
      }
    }
    for (uint32_t i = 0; i < d.n_images; ++i) {
      OImage im;
      im.w = d.images[i].width;
      im.h = d.images[i].height;
      im.rgb.assign(d.images[i].rgb, d.images[i].rgb + 3ull * im.w * im.h);
      images.push_back(std::move(im));
    }
    sky_image = d.sky_image;
    for (uint32_t k = 0; k < d.n_transforms; ++k) {
      Xform<P> x;
      double inv[12];
      affine_inverse(d.transforms + 12 * k, inv);
      for (int j = 0; j < 12; ++j) {
        x.fwd64[j] = d.transforms[12 * k + j];
        x.inv[j] = P::gpu ? (T)(float)inv[j] : (T)inv[j];
        x.fwd[j] = P::gpu ? (T)(float)d.transforms[12 * k + j] : (T)d.transforms[12 * k + j];
      }
      xforms.push_back(x);
    }
    auto xf_list = [](const uint32_t* idx, uint32_t n, std::vector<int32_t>& out) {
      out.assign(n, -1);
      if (idx)
        for (uint32_t i = 0; i < n; ++i) out[i] = idx[i] == RG_NO_TRANSFORM ? -1 : (int32_t)idx[i];
    };
    xf_list(d.sphere_transform, ns, sphere_xf);
    xf_list(d.tri_transform, nt, tri_xf);
    xf_list(d.box_transform, nb, box_xf);
    xf_list(d.quad_transform, nq, quad_xf);
    xf_list(d.cylinder_transform, nc, cyl_xf);
    xf_list(d.volume_transform, nv, vol_xf);
    for (uint32_t i = 0; i < ns; ++i) {
      Sphere<P> s;
      s.c = {(T)d.spheres[4 * i], (T)d.spheres[4 * i + 1], (T)d.spheres[4 * i + 2]};
      s.r = (T)d.spheres[4 * i + 3];
      s.r2 = s.r * s.r;
      spheres.push_back(s);
      sphere_mat.push_back(d.sphere_material[i]);
    }
    for (uint32_t i = 0; i < nt; ++i) {
      const float* v = d.tri_vertices + 9 * i;
      const float* n = d.tri_normals + 9 * i;
      Triangle<P> t;
      t.v0 = {(T)v[0], (T)v[1], (T)v[2]}; t.v1 = {(T)v[3], (T)v[4], (T)v[5]}; t.v2 = {(T)v[6], (T)v[7], (T)v[8]};
      t.n0 = {(T)n[0], (T)n[1], (T)n[2]}; t.n1 = {(T)n[3], (T)n[4], (T)n[5]}; t.n2 = {(T)n[6], (T)n[7], (T)n[8]};
      tris.push_back(t);
      tri_mat.push_back(d.tri_material[i]);
    }
    for (uint32_t i = 0; i < nb; ++i) {
      const float* b = d.boxes + 6 * i;
      boxes.push_back(AxisBox<P>::make({(T)b[0], (T)b[1], (T)b[2]}, {(T)b[3], (T)b[4], (T)b[5]}));
      box_mat.push_back(d.box_material[i]);
    }
    for (uint32_t i = 0; i < nv; ++i) {
      const rg_volume& v = d.volumes[i];
      Volume vol{};
      vol.boundary = v.boundary;
      if (v.boundary == RG_BOUNDARY_SPHERE) {
        vol.s.c = {(T)v.a[0], (T)v.a[1], (T)v.a[2]}; vol.s.r = (T)v.b[0]; vol.s.r2 = vol.s.r * vol.s.r;
      } else {
        vol.b = AxisBox<P>::make({(T)v.a[0], (T)v.a[1], (T)v.a[2]}, {(T)v.b[0], (T)v.b[1], (T)v.b[2]});
      }
      vol.density = (T)v.density;
      vol.neg_inv_density = T(-1) / vol.density;
      vol.material = v.material;
      volumes.push_back(vol);
    }
    for (uint32_t i = 0; i < nsdf; ++i) {
      const rg_sdf& s = d.sdfs[i];
      sdf_material.push_back(s.material);
      Sdf<P> f;
      f.kind = s.kind; f.c = {(T)s.centre[0], (T)s.centre[1], (T)s.centre[2]};
      for (int k = 0; k < 4; ++k) f.p[k] = (T)s.params[k];
      f.max_iter = s.max_iterations; f.eps = (T)s.epsilon;
      sdfs.push_back(f);
    }
    // Objects in list order: spheres, standalone triangles, meshes, boxes, volumes, parallelograms,
    // cylinders; SDFs and infinite planes unbounded.
    // SimpleObject::new (object/simple.rs:67-91): a transformed object's box
    // is its mesh's box mapped by the transform.
    auto obj = [&](uint32_t kind, uint32_t i, const Aabb<T>& box, int32_t xf) {
      bounded.push_back({kind, i, xf >= 0 ? xforms[xf].map_box(box) : box, xf});
    };
    for (uint32_t i = 0; i < ns; ++i) obj(OBJ_SPHERE, i, spheres[i].aabb(), sphere_xf[i]);
    std::vector<int32_t> mesh_ids;
    for (uint32_t i = 0; i < nt; ++i) {
      int32_t g = d.tri_mesh ? d.tri_mesh[i] : -1;
      if (g < 0) { obj(OBJ_TRIANGLE, i, tris[i].aabb(), tri_xf[i]); continue; }
      size_t k = std::find(mesh_ids.begin(), mesh_ids.end(), g) - mesh_ids.begin();
      if (k == mesh_ids.size()) {
        mesh_ids.push_back(g);
        meshes.push_back(Mesh{});
        meshes.back().material = tri_mat[i];
        meshes.back().xf = tri_xf[i];
      }
      meshes[k].tris.push_back(i);
    }
    std::vector<size_t> order(meshes.size());
    for (size_t k = 0; k < order.size(); ++k) order[k] = k;
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return mesh_ids[a] < mesh_ids[b]; });
    for (size_t k : order) {
      Mesh& m = meshes[k];
      std::vector<Aabb<T>> bx;
      for (uint32_t t : m.tris) bx.push_back(tris[t].aabb());
      build_bvh(bx, m.bvh, opt.exact_bvh_limit);
      m.box = m.bvh.nodes[m.bvh.root].box;  // BvhMesh::aabb: the root's box (mesh/advanced/bvh.rs:117-131)
      obj(OBJ_MESH, (uint32_t)k, m.box, m.xf);
    }
    for (uint32_t i = 0; i < nb; ++i) obj(OBJ_BOX, i, boxes[i].aabb(), box_xf[i]);
    for (uint32_t i = 0; i < nv; ++i)
      obj(OBJ_VOLUME, i, volumes[i].boundary == RG_BOUNDARY_SPHERE ? volumes[i].s.aabb() : volumes[i].b.aabb(), vol_xf[i]);
    for (uint32_t i = 0; i < nq; ++i) obj(OBJ_QUAD, i, quads[i].aabb(), quad_xf[i]);
    for (uint32_t i = 0; i < nc; ++i) obj(OBJ_CYLINDER, i, cylinders[i].aabb(), cyl_xf[i]);
    for (uint32_t i = 0; i < nsdf; ++i) unbounded.push_back({false, i});
    for (uint32_t i = 0; i < npl; ++i) unbounded.push_back({true, i});
    std::vector<Aabb<T>> bx;
    for (auto& o : bounded) bx.push_back(o.box);
    build_bvh(bx, top, opt.exact_bvh_limit);
  }

  // Texture::value (texture/*.rs) of texture `t` at hit `h`.
  C3 texture_value(uint32_t t, const Hit<T>& h) const {
    for (uint32_t level = 0; level <= RG_MAX_TEXTURE_DEPTH; ++level) {
      const rg_texture& tx = textures[t];
      switch (tx.kind) {
        case RG_TEX_WORLD_CHECKER: {  // WorldCheckerTexture (checker.rs:20-27)
          const T k = (T)tx.scale[0];
          const T sum = ((T(0) + std::floor(h.pos_w.x / k + (T)tx.offset[0])) + std::floor(h.pos_w.y / k + (T)tx.offset[1])) +
                        std::floor(h.pos_w.z / k + (T)tx.offset[2]);
          t = checker_even(sum) ? tx.even : tx.odd;
          continue;
        }
        case RG_TEX_UV_CHECKER: {  // UvCheckerTexture (checker.rs:37-44)
          const T k = (T)tx.scale[0];
          const T sum = (T(0) + std::floor(h.u / k + (T)tx.offset[0])) + std::floor(h.v / k + (T)tx.offset[1]);
          t = checker_even(sum) ? tx.even : tx.odd;
          continue;
        }
        case RG_TEX_IMAGE: {  // ImageTexture::value (image.rs:29-39)
          const T tu = (T)tx.offset[0] + h.u * (T)tx.scale[0];
          const T tv = (T)tx.offset[1] + h.v * (T)tx.scale[1];
          const OImage& im = images[tx.image];
          return image_bilinear<P>(im, tu * (T)im.w, (T(1) - tv) * (T)im.h);
        }
        case RG_TEX_NOISE: {  // ColourSource::get (noise.rs): ScalePoint, then value / 2 + 0.5
          V3<T> q = tx.noise_place == RG_NOISE_WORLD ? h.pos_w
                  : (tx.noise_place == RG_NOISE_LOCAL ? h.pos_l : V3<T>{h.u, h.v, T(0)});
          const T k = (T)tx.scale[0];
          q = V3<T>{q.x * k, q.y * k, q.z * k};
          const uint8_t* pm = perm.data() + 512ull * tex_perm[t];
          const T g = perlin3<T>(pm, q.x, q.y, q.z);
          if (tx.noise_channels == 1u) {
            const float c = (float)(g / T(2) + T(0.5));
            return C3{c, c, c};
          }
          const T gg = perlin3<T>(pm + 512, q.x, q.y, q.z), gb = perlin3<T>(pm + 1024, q.x, q.y, q.z);
          return C3{(float)(g / T(2) + T(0.5)), (float)(gg / T(2) + T(0.5)), (float)(gb / T(2) + T(0.5))};
        }
        default:
          return C3{tx.colour[0], tx.colour[1], tx.colour[2]};
      }
    }
    return C3{0, 0, 0};
  }
  // The material's colour at a hit: its texture, or the solid albedo.
  C3 colour(const rg_material& m, const Hit<T>& h) const {
    if (m.texture != 0u) return texture_value(m.texture - 1u, h);
    return C3{m.albedo[0], m.albedo[1], m.albedo[2]};
  }

  bool boundary_hit(const Volume& v, const Ray<P>& r, const Interval<T>& iv, Hit<T>& h) const {
    return v.boundary == RG_BOUNDARY_SPHERE ? v.s.intersect(r, iv, h) : v.b.intersect(r, iv, h);
  }

  // VolumetricObject::full_intersect (object/volumetric.rs:86-160). `u` is the
  // uniform of the free-flight draw; the arbitrary normals are drawn after a hit.
  bool volume_intersect(uint32_t vi, const Ray<P>& ray, const Interval<T>& iv, PathRng& rng, uint32_t depth, Hit<T>& h) const {
    const Volume& v = volumes[vi];
    Hit<T> tmp;
    if (!boundary_hit(v, ray, Interval<T>::full(), tmp)) return false;
    T enter = tmp.dist;
    if (iv.has_start) enter = std::fmax(enter, iv.start);
    if (!boundary_hit(v, ray, Interval<T>::from(enter + T(0.001)), tmp)) return false;
    T exitd = tmp.dist;
    if (iv.has_end) exitd = std::fmin(exitd, iv.end);
    T inside = exitd - enter;
    T u;
    U4 blk{};
    if (rng.injected_volume_u) u = (T)rng.injected_volume_u[vi];
    else if (rng.gpu) { blk = rng.block(depth, kPurposeVolume0 + vi); u = (T)u01f_open0(blk.v[0]); }
    else u = (T)rng.seq.gen();
    T hit_dist = v.neg_inv_density * policy_log(u);
    T dist = enter + hit_dist;
    if (hit_dist > inside) return false;
    h.dist = dist;
    h.pos_w = Math<P>::at(ray.pos, ray.dir, dist);
    h.pos_l = h.pos_w;
    if (rng.gpu || rng.injected_volume_u) {
      if (!rng.injected_volume_u) blk = rng.block(depth, kPurposeVolume0 + vi);
      h.normal = unit_sphere_from<T>((T)u01f(blk.v[1]), (T)u01f(blk.v[2]));
      h.ray_normal = h.normal;
      h.u = (T)u01f(blk.v[3]); h.v = h.u;
    } else {
      h.normal = unit_sphere_from<T>((T)rng.seq.gen(), (T)rng.seq.gen());
      h.ray_normal = unit_sphere_from<T>((T)rng.seq.gen(), (T)rng.seq.gen());
      h.u = (T)rng.seq.gen(); h.v = (T)rng.seq.gen();
    }
    h.front_face = true;
    h.side = 0;
    h.material = v.material;
    h.prim = prim_vol(vi);
    return true;
  }

  // SimpleObject::full_intersect (object/simple.rs:107-116): a transformed
  // object tests its mesh against the mapped ray with the caller's interval
  // (RefF64). The device (GpuF32) tests from the same start without an end
  // and bounds the world-space distance instead; both agree for rigid
  // transforms, and under scaling the reference's result depends on the
  // order in which objects are tested.
  bool object_intersect(const Object& o, const Ray<P>& ray, const Interval<T>& iv, PathRng& rng, uint32_t depth, Hit<T>& h) const {
    if (o.xf < 0) return mesh_intersect(o, ray, iv, rng, depth, h);
    const Xform<P>& x = xforms[o.xf];
    const Ray<P> local = x.incoming(ray);
    if constexpr (P::gpu) {
      Interval<T> open = iv;
      open.has_end = false;
      if (!mesh_intersect(o, local, open, rng, depth, h)) return false;
      x.outgoing(ray, local, h);
      return !iv.has_end || h.dist <= iv.end;
    } else {
      if (!mesh_intersect(o, local, iv, rng, depth, h)) return false;
      x.outgoing(ray, local, h);
      return true;
    }
  }

  bool mesh_intersect(const Object& o, const Ray<P>& ray, const Interval<T>& iv, PathRng& rng, uint32_t depth, Hit<T>& h) const {
    switch (o.kind) {
      case OBJ_SPHERE:
        if (!spheres[o.index].intersect(ray, iv, h)) return false;
        h.material = sphere_mat[o.index]; h.prim = prim_sphere(o.index); return true;
      case OBJ_TRIANGLE:
        if (!tris[o.index].intersect(ray, iv, h)) return false;
        h.material = tri_mat[o.index]; h.prim = prim_tri(o.index); return true;
      case OBJ_MESH: {
        const Mesh& m = meshes[o.index];
        if (!mesh_node(m, m.bvh.root, ray, iv, h)) return false;
        h.material = m.material; return true;
      }
      case OBJ_BOX:
        if (!boxes[o.index].intersect(ray, iv, h)) return false;
        h.material = box_mat[o.index]; h.prim = prim_box(o.index); return true;
      case OBJ_VOLUME:
        return volume_intersect(o.index, ray, iv, rng, depth, h);
      case OBJ_QUAD:
        if (!quads[o.index].intersect(ray, iv, h)) return false;
        h.material = quad_mat[o.index]; h.prim = prim_quad(o.index); return true;
      case OBJ_CYLINDER:
        if (!cylinders[o.index].intersect(ray, iv, h)) return false;
        h.material = cyl_mat[o.index]; h.prim = prim_cyl(o.index); return true;
    }
    return false;
  }

  // BvhMesh::bvh_node_intersect (mesh/advanced/bvh.rs:63-103)
  bool mesh_node(const Mesh& m, int node, const Ray<P>& ray, const Interval<T>& iv, Hit<T>& h) const {
    const BvhNode<T>& n = m.bvh.nodes[node];
    if (n.is_item) {
      const Triangle<P>& t = tris[m.tris[n.item]];
      if (opt.prim_pretest && !aabb_hit<P>(n.box, ray, iv)) return false;
      if (!t.intersect(ray, iv, h)) return false;
      h.prim = prim_tri(m.tris[n.item]);
      return true;
    }
    if (!aabb_hit<P>(n.box, ray, iv)) return false;
    Interval<T> sh = iv;
    bool any = false;
    for (uint32_t c : n.children) {
      Hit<T> hc;
      if (!mesh_node(m, (int)c, ray, sh, hc)) continue;
      sh = sh.with_end(hc.dist);
      h = hc;
      any = true;
    }
    return any;
  }

  // BvhObject::bvh_node_intersect (object/bvh.rs:70-108)
  bool top_node(int node, const Ray<P>& ray, const Interval<T>& iv, PathRng& rng, uint32_t depth, Hit<T>& h) const {
    const BvhNode<T>& n = top.nodes[node];
    if (n.is_item) {
      if (opt.prim_pretest && !aabb_hit<P>(n.box, ray, iv)) return false;
      return object_intersect(bounded[n.item], ray, iv, rng, depth, h);
    }
    if (!aabb_hit<P>(n.box, ray, iv)) return false;
    Interval<T> sh = iv;
    bool any = false;
    for (uint32_t c : n.children) {
      Hit<T> hc;
      if (!top_node((int)c, ray, sh, rng, depth, hc)) continue;
      sh = sh.with_end(hc.dist);
      h = hc;
      any = true;
    }
    return any;
  }

  // ObjectList::full_intersect (object/list.rs:112-129): the BVH result, then
  // every unbounded object with the original interval; the first minimum wins.
  // Closest hit of the primitive tests alone, in object order, with the same
  // shrinking interval (a later hit at equal distance replaces the earlier).
  bool brute_force(const Ray<P>& ray, const Interval<T>& iv, PathRng& rng, uint32_t depth, Hit<T>& h) const {
    Interval<T> sh = iv;
    bool any = false;
    for (const Object& o : bounded) {
      if (o.kind == OBJ_MESH) {
        const Mesh& m = meshes[o.index];
        const Ray<P> local = m.xf >= 0 ? xforms[m.xf].incoming(ray) : ray;
        for (uint32_t t : m.tris) {
          Hit<T> hc;
          if (m.xf >= 0) {  // as object_intersect, one triangle at a time
            Interval<T> ti = sh;
            if (P::gpu) ti.has_end = false;
            if (!tris[t].intersect(local, ti, hc)) continue;
            xforms[m.xf].outgoing(ray, local, hc);
            if (P::gpu && sh.has_end && !(hc.dist <= sh.end)) continue;
          } else if (!tris[t].intersect(local, sh, hc)) {
            continue;
          }
          hc.prim = prim_tri(t);
          hc.material = m.material;
          sh = sh.with_end(hc.dist);
          h = hc;
          any = true;
        }
        continue;
      }
      Hit<T> hc;
      if (!object_intersect(o, ray, sh, rng, depth, hc)) continue;
      sh = sh.with_end(hc.dist);
      h = hc;
      any = true;
    }
    return any;
  }

  bool intersect(const Ray<P>& ray, const Interval<T>& iv, PathRng& rng, uint32_t depth, Hit<T>& h) const {
    bool any = false;
    if (opt.brute_force) any = brute_force(ray, iv, rng, depth, h);
    else if (top.root >= 0) any = top_node(top.root, ray, iv, rng, depth, h);
    for (const Unbounded& u : unbounded) {
      Hit<T> hs;
      if (u.plane) {
        if (!planes[u.index].intersect(ray, iv, hs)) continue;  // InfinitePlaneMesh::intersect (infinite_plane.rs:87-92)
        wrap_uv(plane_wrap[u.index], hs.u, hs.v);
      } else if (!sdfs[u.index].intersect(ray, iv, hs)) {
        continue;
      }
      if (!any || hs.dist < h.dist) {
        h = hs;
        h.prim = u.plane ? prim_plane(u.index) : prim_sdf(u.index);
        h.material = u.plane ? plane_mat[u.index] : sdf_material[u.index];
        any = true;
      }
    }
    return any;
  }
  std::vector<uint32_t> sdf_material;
};

// ---------------------------------------------------------------------------
// Camera (scene/camera.rs:114-213), in f64 on the host.
// ---------------------------------------------------------------------------
struct Viewport {
  double pos[3], pixel_center[3], viewport_u[3], viewport_v[3], defocus_u[3], defocus_v[3];
};

// Camera::calculate_viewport. Returns false for the Err cases.
inline bool calculate_viewport(const rg_camera& c, Viewport& vp) {
  using M = Math<RefF64>;
  using V = V3<double>;
  double focal = c.focus_dist;
  if (c.v_fov == 0.0) return false;
  if (focal == 0.0) return false;
  V fwd{c.fwd[0], c.fwd[1], c.fwd[2]};
  V wn;
  if (!M::try_normalize(fwd, wn)) return false;
  V w = -wn;
  V uu;
  if (!M::try_normalize(M::cross(V{0, 1, 0}, w), uu)) return false;
  V v = M::cross(w, uu);
  V pos{c.pos[0], c.pos[1], c.pos[2]};
  V pc = pos - (w * focal);
  double rad = focal * std::tan(c.defocus_angle / 2.0);
  V du = uu * rad, dv = v * rad;
  double h = std::tan(c.v_fov / 2.0);
  double size = 2.0 * h * focal;
  V vu = uu * size;
  V vv = (-v) * size;
  auto put = [](double* o, V x) { o[0] = x.x; o[1] = x.y; o[2] = x.z; };
  put(vp.pos, pos); put(vp.pixel_center, pc); put(vp.viewport_u, vu); put(vp.viewport_v, vv);
  put(vp.defocus_u, du); put(vp.defocus_v, dv);
  return true;
}

template <class P> inline C3 sky_colour(uint32_t sky, const Ray<P>& r) {
  if (sky == RG_SKY_WHITE) return {1, 1, 1};
  if (sky == RG_SKY_NONE) return {0, 0, 0};
  // SimpleSkybox (skybox/simple.rs:13-21): white + (blue - white) * a
  float a;
  if constexpr (P::gpu) a = 0.5f * r.dir.y + 0.5f;
  else a = (float)((0.5 * r.dir.y) + 0.5);
  return {1.0f + (0.5f - 1.0f) * a, 1.0f + (0.7f - 1.0f) * a, 1.0f + (1.0f - 1.0f) * a};
}

// The sky of a missed ray; HdrImageSkybox (skybox/hdri.rs:17-26) samples its
// image at sphere_uv(dir), v flipped.
template <class P> inline C3 sky_of(const Scene<P>& sc, const Ray<P>& r) {
  using T = typename P::T;
  if (sc.skybox == RG_SKY_IMAGE) {
    const T theta = std::acos(-r.dir.y);
    const T phi = std::atan2(-r.dir.z, r.dir.x) + T(M_PI);
    const T u = phi / T(2 * M_PI), v = theta / T(M_PI);
    const OImage& im = sc.images[sc.sky_image];
    return image_bilinear<P>(im, u * (T)im.w, (T(1) - v) * (T)im.h);
  }
  return sky_colour<P>(sc.skybox, r);
}

// Material::scatter for each variant. Returns false for None.
template <class P>
inline bool scatter(const rg_material& m, const Ray<P>& ray, const Hit<typename P::T>& h, PathRng& rng, uint32_t depth,
                    V3<typename P::T>& out) {
  using T = typename P::T;
  using M = Math<P>;
  using V = V3<T>;
  U4 blk{};
  if (rng.gpu) blk = rng.block(depth, kPurposeScatter);
  switch (m.kind) {
    case RG_MAT_LAMBERTIAN: {  // lambertian.rs:29-37
      V rnd;
      if (rng.gpu) {
        T z = T(1) - T(2) * (T)u01f(blk.v[0]);
        T phi = T(2 * M_PI) * (T)u01f(blk.v[1]);
        T s = std::sqrt(std::fmax(T(0), T(1) - z * z));
        T rad = std::cbrt((T)u01f(blk.v[2]));
        rnd = {s * std::cos(phi) * rad, s * std::sin(phi) * rad, z * rad};
      } else {
        for (;;) {  // vector_in_unit_sphere (rng.rs:64-72)
          rnd = {(T)rng.seq.range_incl(-1, 1), (T)rng.seq.range_incl(-1, 1), (T)rng.seq.range_incl(-1, 1)};
          if (M::dot(rnd, rnd) <= T(1)) break;
        }
      }
      V vec = h.ray_normal + rnd;
      if (!M::try_normalize(vec, out)) out = h.ray_normal;
      return true;
    }
    case RG_MAT_METAL: {  // metal.rs:17-34
      V d = ray.dir;
      V refl = d - h.ray_normal * (T(2) * M::dot(d, h.ray_normal));
      V rnd;
      if (rng.gpu) rnd = unit_sphere_from<T>((T)u01f(blk.v[0]), (T)u01f(blk.v[1]));
      else { T r1 = (T)rng.seq.range_incl(0, 1); T r2 = (T)rng.seq.range_incl(0, 1); rnd = unit_sphere_from<T>(r1, r2); }
      V vec = refl + rnd * (T)m.fuzz;
      if (!(M::dot(vec, h.ray_normal) > T(0))) return false;
      out = M::normalize(vec);
      return true;
    }
    case RG_MAT_DIELECTRIC: {  // dielectric.rs:19-37
      T ior = (T)m.refractive_index;
      T ratio = h.front_face ? T(1) / ior : ior;
      V d = ray.dir;
      T cos_t = std::fmin(M::dot(-d, h.ray_normal), T(1));
      T sin_t = std::sqrt(T(1) - cos_t * cos_t);
      bool tir = ratio * sin_t > T(1);
      T r0 = (T(1) - ratio) / (T(1) + ratio);
      T r02 = r0 * r0;
      T x = T(1) - cos_t;
      T x2 = x * x;
      T x5 = (x2 * x2) * x;
      T refl_p = r02 + (T(1) - r02) * x5;
      T u = rng.gpu ? (T)u01f(blk.v[0]) : (T)rng.seq.gen();
      bool schlick = refl_p > u;
      if (tir || schlick) {
        out = d - h.ray_normal * (T(2) * M::dot(d, h.ray_normal));
      } else {  // math::refract (shared/math.rs:20-25)
        T c2 = std::fmin(M::dot(-d, h.ray_normal), T(1));
        V perp = (d + h.ray_normal * c2) * ratio;
        V par = h.ray_normal * (-std::sqrt(std::fabs(T(1) - M::dot(perp, perp))));
        out = perp + par;
      }
      return true;
    }
    case RG_MAT_ISOTROPIC: {  // isotropic.rs:29-31
      if (rng.gpu) out = unit_sphere_from<T>((T)u01f(blk.v[0]), (T)u01f(blk.v[1]));
      else { T r1 = (T)rng.seq.range_incl(0, 1); T r2 = (T)rng.seq.range_incl(0, 1); out = unit_sphere_from<T>(r1, r2); }
      return true;
    }
    default:  // LightMaterial: no scatter (light.rs:17)
      return false;
  }
}

// Material::reflected_light factor: the colour multiplying future_col.
template <class P>
inline C3 attenuation(const Scene<P>& sc, const rg_material& m, const Ray<P>& ray, const Hit<typename P::T>& h) {
  if (m.kind == RG_MAT_DIELECTRIC && h.front_face) return {1, 1, 1};  // entering: future_col unchanged (dielectric.rs:63-65)
  if (m.kind > RG_MAT_ISOTROPIC) return {0, 0, 0};
  const C3 alb = sc.colour(m, h);
  if (m.kind == RG_MAT_LAMBERTIAN || m.kind == RG_MAT_METAL) return alb;
  double dist = (double)Math<P>::length(h.pos_w - ray.pos);
  float tr = (float)(-(double)m.density * dist);
  if constexpr (P::gpu) tr = -m.density * (float)dist;
  float e = std::exp(tr);
  return alb * e;
}

// ---------------------------------------------------------------------------
// Integrator
// ---------------------------------------------------------------------------
struct RenderParams {
  uint32_t width, height, spp, ray_depth;
  uint64_t seed;
  uint32_t mode = RG_MODE_PBR;  // RenderOpts::mode
  uint32_t branching = 1;       // RenderOpts::ray_branching
};

template <class P> struct Renderer {
  using T = typename P::T;
  using V = V3<T>;
  const Scene<P>& sc;
  Viewport vp;
  RenderParams rp;
  Renderer(const Scene<P>& s, const Viewport& v, const RenderParams& r) : sc(s), vp(v), rp(r) {}

  // ray_colour_recursive (renderer.rs:508-572): `branching` scattered rays per
  // bounce, a failed scatter counting as a black sample, their mean added to
  // the emission.
  C3 colour_recursive(const Ray<P>& ray, uint32_t depth, PathRng& rng) const {
    if (depth > rp.ray_depth) return {0, 0, 0};
    Hit<T> h;
    Interval<T> iv = Interval<T>::range(T(1e-3), std::numeric_limits<T>::max());
    if (!sc.intersect(ray, iv, rng, depth, h)) return sky_of<P>(sc, ray);
    const rg_material& m = sc.materials[h.material];
    C3 emitted = m.kind == RG_MAT_LIGHT ? sc.colour(m, h) : C3{0, 0, 0};
    C3 sum{0, 0, 0};
    for (uint32_t i = 0; i < rp.branching; ++i) {
      V dir;
      if (!scatter<P>(m, ray, h, rng, depth, dir)) continue;  // Colour::BLACK
      Ray<P> next = Ray<P>::make(h.pos_w, dir);
      C3 fut = colour_recursive(next, depth + 1, rng);
      C3 scattered = m.kind == RG_MAT_LIGHT ? C3{0, 0, 0} : fut * attenuation<P>(sc, m, ray, h);
      sum = sum + scattered;
    }
    return emitted + sum * (1.0f / (float)rp.branching);
  }

  // The device's walk of the branching tree (trace.cuh, branch_sample): node
  // weights pushed down, streams keyed by node (children n b + 1 + i, scatter
  // of branch i keyed n b + i).
  C3 colour_branch_gpu(Ray<P> ray, PathRng& rng) const {
    struct Level { Hit<T> h; Ray<P> in; C3 w; uint32_t node, next; };
    std::vector<Level> st;
    const uint32_t b = rp.branching;
    const float inv_b = 1.0f / (float)b;
    C3 L{0, 0, 0}, w{1, 1, 1};
    uint32_t node = 0, depth = 0;
    for (;;) {
      Hit<T> h;
      Interval<T> iv = Interval<T>::range(T(1e-3), std::numeric_limits<T>::max());
      if (!sc.intersect(ray, iv, rng, node, h)) {
        L = L + w * sky_of<P>(sc, ray);
      } else {
        const rg_material& m = sc.materials[h.material];
        if (m.kind == RG_MAT_LIGHT) L = L + w * sc.colour(m, h);
        else if (depth < rp.ray_depth && st.size() < 32) st.push_back(Level{h, ray, w, node, 0});
      }
      bool found = false;
      while (!st.empty()) {
        Level& lv = st.back();
        if (lv.next >= b) { st.pop_back(); continue; }
        uint32_t i = lv.next++;
        const rg_material& m = sc.materials[lv.h.material];
        V dir;
        if (!scatter<P>(m, lv.in, lv.h, rng, lv.node * b + i, dir)) continue;
        C3 a = attenuation<P>(sc, m, lv.in, lv.h);
        w = lv.w * a * inv_b;
        ray = Ray<P>::make(lv.h.pos_w, dir);
        node = lv.node * b + 1 + i;
        depth = (uint32_t)st.size();
        found = true;
        break;
      }
      if (!found) break;
    }
    return L;
  }

  // Render::render_px_once for the debug modes (renderer.rs:427-490).
  C3 mode_colour(const Ray<P>& ray, PathRng& rng) const {
    Hit<T> h;
    Interval<T> iv = Interval<T>::range(T(1e-3), std::numeric_limits<T>::max());
    if (!sc.intersect(ray, iv, rng, 0, h)) return sky_of<P>(sc, ray);
    static const float kCol[13][3] = {{1, 1, 1}, {1, 0, 0}, {1, 0.5f, 0}, {1, 1, 0}, {0.5f, 1, 0}, {0, 1, 0}, {0, 1, 0.5f},
                                      {0, 1, 1}, {0, 0.5f, 1}, {0, 0, 1}, {0.5f, 0, 1}, {1, 0, 1}, {0, 0, 0}};
    auto half = [](V v) { return C3{(float)(v.x / T(2)) + 0.5f, (float)(v.y / T(2)) + 0.5f, (float)(v.z / T(2)) + 0.5f}; };
    auto col = [&](int k) { return C3{kCol[k][0], kCol[k][1], kCol[k][2]}; };
    switch (rp.mode) {
      case RG_MODE_OUTWARD_NORMAL: return half(h.normal);
      case RG_MODE_RAY_NORMAL: return half(h.ray_normal);
      case RG_MODE_SCATTER: {
        V dir{0, 0, 0};
        if (!scatter<P>(sc.materials[h.material], ray, h, rng, 0, dir)) dir = V{0, 0, 0};
        return half(dir);
      }
      case RG_MODE_UV:
        return C3{std::fmin(std::fmax((float)h.u, 0.0f), 1.0f), std::fmin(std::fmax((float)h.v, 0.0f), 1.0f), 0.0f};
      case RG_MODE_FRONT_FACE: return col(h.front_face ? 1 : 0);
      case RG_MODE_SIDE: return col((int)(h.side % 12u + 1u));
      default: {  // distance
        T val = T(2) * std::cbrt(h.dist);
        T fl = std::fmin(std::fmax(std::floor(val), T(0)), T(12)), ce = std::fmin(std::fmax(std::ceil(val), T(0)), T(12));
        float frac = (float)(val - fl);
        C3 a = col((int)fl), bcol = col((int)ce);
        return C3{a.r + (bcol.r - a.r) * frac, a.g + (bcol.g - a.g) * frac, a.b + (bcol.b - a.b) * frac};
      }
    }
  }

  // The device integrator: the same recursion evaluated front to back.
  C3 colour_iterative(Ray<P> ray, PathRng& rng) const {
    C3 L{0, 0, 0}, beta{1, 1, 1};
    for (uint32_t depth = 0; depth <= rp.ray_depth; ++depth) {
      Hit<T> h;
      Interval<T> iv = Interval<T>::range(T(1e-3), std::numeric_limits<T>::max());
      if (!sc.intersect(ray, iv, rng, depth, h)) {
        C3 s = sky_of<P>(sc, ray);
        L = L + beta * s;
        break;
      }
      const rg_material& m = sc.materials[h.material];
      if (m.kind == RG_MAT_LIGHT) {
        L = L + beta * sc.colour(m, h);
        break;
      }
      V dir;
      if (!scatter<P>(m, ray, h, rng, depth, dir)) break;
      beta = beta * attenuation<P>(sc, m, ray, h);
      ray = Ray<P>::make(h.pos_w, dir);
    }
    return L;
  }

  // Viewport::calc_ray (camera.rs:191-213) for sub-pixel coordinates (fx, fy).
  Ray<P> camera_ray(T fx, T fy, T lx, T ly) const {
    T w = (T)rp.width, hh = (T)rp.height;
    T u = (fx - (w / T(2))) / hh;
    T v = (fy - (hh / T(2))) / hh;
    V pc{(T)vp.pixel_center[0], (T)vp.pixel_center[1], (T)vp.pixel_center[2]};
    V vu{(T)vp.viewport_u[0], (T)vp.viewport_u[1], (T)vp.viewport_u[2]};
    V vv{(T)vp.viewport_v[0], (T)vp.viewport_v[1], (T)vp.viewport_v[2]};
    V pos{(T)vp.pos[0], (T)vp.pos[1], (T)vp.pos[2]};
    V du{(T)vp.defocus_u[0], (T)vp.defocus_u[1], (T)vp.defocus_u[2]};
    V dv{(T)vp.defocus_v[0], (T)vp.defocus_v[1], (T)vp.defocus_v[2]};
    V ps = (pc + vu * u) + vv * v;
    V rpos = (pos + du * lx) + dv * ly;
    return Ray<P>::make(rpos, ps - rpos);
  }

  // Gradient accumulators of the adjoint (double).
  struct Grad {
    std::vector<double> alb, em, den;
  };

  // Free-flight scores of every medium on one segment ending at t_final.
  void medium_scores(const Ray<P>& ray, T t_final, int winner, std::vector<double>& score) const {
    score.assign(sc.nv, 0.0);
    for (uint32_t v = 0; v < sc.nv; ++v) {
      Hit<T> tmp;
      if (!sc.boundary_hit(sc.volumes[v], ray, Interval<T>::full(), tmp)) continue;
      T enter = std::fmax(tmp.dist, T(1e-3));
      if (!sc.boundary_hit(sc.volumes[v], ray, Interval<T>::from(enter + T(0.001)), tmp)) continue;
      if ((int)v == winner) {
        score[v] = 1.0 / (double)sc.volumes[v].density - ((double)t_final - (double)enter);
      } else {
        double l = (double)std::fmin(tmp.dist, t_final) - (double)enter;
        score[v] = l > 0.0 ? -l : 0.0;
      }
    }
  }

  // Path-replay adjoint of one sample (device sampler assignment): the same
  // estimator as the device's replay kernel, accumulated in double.
  void adjoint_sample(uint32_t x, uint32_t y, uint32_t s, const double* delta, Grad& g) const {
    const double inv = 1.0 / (double)rp.spp;
    const double d[3] = {delta[0] * inv, delta[1] * inv, delta[2] * inv};
    uint32_t dd = (uint32_t)std::sqrt((double)rp.spp);
    while ((dd + 1) * (dd + 1) <= rp.spp) ++dd;
    while (dd * dd > rp.spp) --dd;
    PathRng rng(true, rp.seed, y * rp.width + x, s);
    U4 b = rng.block(0xFFFFFFFFu, kPurposeCamera);
    T jx = (T)u01f(b.v[0]) - T(0.5), jy = (T)u01f(b.v[1]) - T(0.5);
    T lr = std::sqrt((T)u01f(b.v[2])), ph = T(2 * M_PI) * (T)u01f(b.v[3]);
    T fx, fy;
    if (s < dd * dd) {
      T dinv = T(1) / (T)dd;
      fx = ((T)x + jx * dinv) + (T)(s % dd) * dinv;
      fy = ((T)y + jy * dinv) + (T)(s / dd) * dinv;
    } else {
      fx = (T)x + jx;
      fy = (T)y + jy;
    }
    Ray<P> ray = camera_ray(fx, fy, lr * std::cos(ph), lr * std::sin(ph));
    struct Vtx { uint32_t mat; bool light, albdep; double g, beta[3]; std::vector<double> score; };
    std::vector<Vtx> vs;
    double bt[3] = {1, 1, 1};
    bool escaped = false;
    C3 sky{0, 0, 0};
    std::vector<double> esc_score;
    for (uint32_t depth = 0; depth <= rp.ray_depth; ++depth) {
      Hit<T> h;
      Interval<T> iv = Interval<T>::range(T(1e-3), std::numeric_limits<T>::max());
      bool hit = sc.intersect(ray, iv, rng, depth, h);
      int winner = -1;
      if (hit && h.prim >= sc.prim_vol(0) && h.prim < sc.prim_vol(sc.nv)) winner = (int)(h.prim - sc.prim_vol(0));
      std::vector<double> score;
      medium_scores(ray, hit ? h.dist : std::numeric_limits<T>::infinity(), winner, score);
      if (!hit) {
        escaped = true;
        sky = sky_of<P>(sc, ray);
        esc_score = score;
        break;
      }
      const rg_material& m = sc.materials[h.material];
      Vtx vx{h.material, m.kind == RG_MAT_LIGHT, false, 1.0, {bt[0], bt[1], bt[2]}, score};
      vs.push_back(vx);
      if (m.kind == RG_MAT_LIGHT || depth == rp.ray_depth) break;
      V dir;
      if (!scatter<P>(m, ray, h, rng, depth, dir)) break;
      C3 a = attenuation<P>(sc, m, ray, h);
      if (m.kind == RG_MAT_LAMBERTIAN || m.kind == RG_MAT_METAL) {
        vs.back().albdep = true;
      } else if (!(m.kind == RG_MAT_DIELECTRIC && h.front_face)) {
        vs.back().albdep = true;
        vs.back().g = std::exp(-(double)m.density * (double)Math<P>::length(h.pos_w - ray.pos));
      }
      bt[0] *= a.r; bt[1] *= a.g; bt[2] *= a.b;
      ray = Ray<P>::make(h.pos_w, dir);
    }
    double c[3] = {0, 0, 0};
    if (escaped) {
      c[0] = sky.r; c[1] = sky.g; c[2] = sky.b;
      for (uint32_t v = 0; v < sc.nv; ++v)
        g.den[v] += esc_score[v] * (d[0] * bt[0] * c[0] + d[1] * bt[1] * c[1] + d[2] * bt[2] * c[2]);
    }
    for (int j = (int)vs.size() - 1; j >= 0; --j) {
      const Vtx& vx = vs[j];
      const rg_material& m = sc.materials[vx.mat];
      if (vx.light) {
        for (int k = 0; k < 3; ++k) g.em[3 * vx.mat + k] += d[k] * vx.beta[k];
        for (int k = 0; k < 3; ++k) c[k] = m.albedo[k];
      } else if (vx.albdep) {
        for (int k = 0; k < 3; ++k) {
          g.alb[3 * vx.mat + k] += d[k] * vx.beta[k] * vx.g * c[k];
          c[k] *= (double)m.albedo[k] * vx.g;
        }
      }
      for (uint32_t v = 0; v < sc.nv; ++v)
        g.den[v] += vx.score[v] * (d[0] * vx.beta[0] * c[0] + d[1] * vx.beta[1] * c[1] + d[2] * vx.beta[2] * c[2]);
    }
  }

  // One sample of pixel (x, y); sample index s of spp.
  C3 sample(uint32_t x, uint32_t y, uint32_t s, bool gpu_sampling, SeqRng* msaa) const {
    uint32_t d = (uint32_t)std::sqrt((double)rp.spp);
    while ((d + 1) * (d + 1) <= rp.spp) ++d;
    while (d * d > rp.spp) --d;
    uint32_t pix = y * rp.width + x;
    PathRng rng(gpu_sampling, rp.seed, pix, s);
    T jx, jy, lx = 0, ly = 0;
    if (gpu_sampling) {
      U4 b = rng.block(0xFFFFFFFFu, kPurposeCamera);
      jx = (T)u01f(b.v[0]) - T(0.5);
      jy = (T)u01f(b.v[1]) - T(0.5);
      T r = std::sqrt((T)u01f(b.v[2]));
      T ph = T(2 * M_PI) * (T)u01f(b.v[3]);
      lx = r * std::cos(ph);
      ly = r * std::sin(ph);
    } else {
      jx = (T)msaa->range_incl(-0.5, 0.5);
      jy = (T)msaa->range_incl(-0.5, 0.5);
      for (;;) {  // vector_in_unit_circle (rng.rs:134-142)
        lx = (T)rng.seq.range_incl(-1, 1);
        ly = (T)rng.seq.range_incl(-1, 1);
        if (lx * lx + ly * ly <= T(1)) break;
      }
    }
    T fx, fy;
    if (s < d * d) {  // render_px_msaa (renderer.rs:370-384): index i + d*j
      T dinv = T(1) / (T)d;
      uint32_t i = s % d, j = s / d;
      fx = ((T)x + jx * dinv) + (T)i * dinv;
      fy = ((T)y + jy * dinv) + (T)j * dinv;
    } else {
      fx = (T)x + jx;
      fy = (T)y + jy;
    }
    Ray<P> ray = camera_ray(fx, fy, lx, ly);
    if (rp.mode != RG_MODE_PBR) return mode_colour(ray, rng);
    if (rp.branching > 1) return gpu_sampling ? colour_branch_gpu(ray, rng) : colour_recursive(ray, 0, rng);
    return gpu_sampling ? colour_iterative(ray, rng) : colour_recursive(ray, 0, rng);
  }
};

}  // namespace orc
