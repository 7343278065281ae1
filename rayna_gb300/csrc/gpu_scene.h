// gpu_scene.h — device-side layout of a flattened scene, shared by the host
// builder (bvh_build.cpp, renderer.cpp) and the kernels.
//
// HBM layout (structure of arrays, every array 256-byte aligned by cudaMalloc):
//   nodes       BvhNode2[n_nodes]      64 B each: the two child boxes of one
//                                      binary node plus their child words
//   prims       float4[3 * n_prims]    48 B each, reordered so that every
//                                      leaf is a contiguous range
//   tri_normals float[9 * n_tris]      vertex normals, by triangle id,
//                                      fetched only for the closest hit
//   materials   rg_material[n_mat]     32 B each
//   sdfs        GpuSdf[n_sdf]          unbounded objects, marched after the BVH
#pragma once

#include <stdint.h>

#include "../../include/rayna_gpu.h"

#include <vector_types.h>

namespace rg {

// Primitive kinds, stored in the top 3 bits of prim.a.w.
enum : uint32_t {
  PK_SPHERE = 0,
  PK_TRIANGLE = 1,
  PK_BOX = 2,
  PK_VOL_SPHERE = 3,
  PK_VOL_BOX = 4,
};
constexpr uint32_t kKindShift = 29;
constexpr uint32_t kMaterialMask = (1u << kKindShift) - 1u;

// Triangle flag (prim.c.w bits): the three vertex normals can sum to zero
// inside the triangle, so the interpolated normal must be checked while
// traversing (Triangle::intersect treats an unnormalisable normal as a miss).
constexpr uint32_t kTriCheckNormals = 1u;

// One primitive, 48 bytes:
//   sphere      a = (centre, bits kind|mat)  b = (r, r*r, 0, id)          c = unused
//   triangle    a = (v0, bits)               b = (v1-v0, id)              c = (v2-v0, flags)
//   box         a = (centre, bits)           b = (radius, id)             c = (1/radius, 0)
//   vol sphere  a = (centre, bits)           b = (r, r*r, -1/density, id) c = unused
//   vol box     a = (centre, bits)           b = (radius, id)             c = (1/radius, -1/density)
// `id` is the global primitive id (see rg_scene_desc).
struct alignas(16) GpuPrim {
  float4 a, b, c;
};

// Binary BVH node holding both children (Aila & Laine 2009 layout):
//   xs = (c0.lo.x, c0.hi.x, c1.lo.x, c1.hi.x), ys, zs likewise,
//   meta = (c0, c1, n0, n1): n == 0 means child c is the internal node
//   nodes[c]; n > 0 means a leaf over prims [c, c + n). An absent child
//   (only next to a root that is a single leaf) has c = -1, n = 0.
struct alignas(64) BvhNode2 {
  float4 xs, ys, zs;
  int4 meta;
};
static_assert(sizeof(BvhNode2) == 64, "node pair must be 64 bytes");
static_assert(sizeof(GpuPrim) == 48, "primitive must be 48 bytes");

// Traversal stack depth; the builder keeps the tree shallower than this.
constexpr int kStackSize = 64;
constexpr int kMaxBuildDepth = 60;

struct GpuSdf {
  uint32_t kind;
  float cx, cy, cz;
  float p0, p1, p2, p3;
  uint32_t max_iter;
  float eps;
  uint32_t material;
  uint32_t prim_id;
  float bound_radius;  // outside this radius (and moving away) no hit is possible
  float pad[3];
};

struct GpuScene {
  const BvhNode2* nodes;
  const GpuPrim* prims;
  const float* tri_normals;
  const rg_material* materials;
  const GpuSdf* sdfs;
  uint32_t n_nodes;
  uint32_t n_prims;
  uint32_t n_sdfs;
  uint32_t n_volumes;
  uint32_t sky;
  uint32_t tri_base;   // global id of triangle 0
  uint32_t vol_base;   // global id of volume 0
  uint32_t n_tris;
  uint32_t features;   // F_* bits of the kernel variant to launch (primitive kinds present)
  const float* vol_density;   // per medium: VolumetricObject::density
  const uint32_t* vol_prim;   // per medium: its position in `prims`
};

// Device error bits (rg_render_stats::error_flags).
enum : uint32_t {
  ERR_STACK_OVERFLOW = 1u,
  ERR_BAD_INDEX = 2u,
  ERR_QUEUE_OVERFLOW = 4u,
};

// Counters (RG_FLAG_COUNTERS): indices into the u64 counter array.
enum : uint32_t { CNT_RAYS = 0, CNT_NODES = 1, CNT_PRIMS = 2, CNT_SDF = 3, CNT_SAMPLES = 4, CNT_N = 8 };

// Per-frame launch parameters (all f32 values rounded from the f64 host viewport).
struct FrameParams {
  uint32_t width, height, spp, ray_depth;
  uint32_t strat_d;
  float strat_inv;
  uint32_t seed_lo, seed_hi;
  float pos[3], pixel_center[3], viewport_u[3], viewport_v[3], defocus_u[3], defocus_v[3];
  uint32_t accum_count;   // per-pixel accumulation count after this frame
  float* accum;           // [x][y][rgb] running sum
  float* out;             // [x][y][rgb] running mean (may be null)
  float* frame_mean;      // [x][y][rgb] this frame's sample mean (may be null)
  float* frame_var;       // [x][y][rgb] this frame's sample variance (may be null)
  unsigned long long* counters;
  uint32_t* err;
};

}  // namespace rg
