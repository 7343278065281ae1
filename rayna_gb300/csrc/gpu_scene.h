// gpu_scene.h — device-side layout of a flattened scene, shared by the host
// builder (bvh_build.cpp, renderer.cpp) and the kernels.
//
// HBM layout (structure of arrays, every array 256-byte aligned by cudaMalloc):
//   nodes       BvhNode2[n_nodes]      64 B each: the two child boxes of one
//                                      binary node plus their child words
//   wnodes      WideNode[n_wnodes]     80 B each: the same tree collapsed to
//                                      eight children per node
//   prims       float4[3 * n_prims]    48 B each, reordered so that every
//                                      leaf is a contiguous range
//   tri_normals float[9 * n_tris]      vertex normals, by triangle id,
//                                      fetched only for the closest hit
//   materials   rg_material[n_mat]     32 B each
//   sdfs        GpuSdf[n_sdf]          unbounded objects, marched after the BVH
#pragma once

#include <stdint.h>

#include <type_traits>

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
  PK_QUAD = 5,
  PK_CYLINDER = 6,
};
constexpr uint32_t kKindShift = 29;
// Bit 28 of prim.a.w: the primitive belongs to a transformed object; its
// transform index is prim_xform[position in prims].
constexpr uint32_t kXformBit = 1u << 28;
constexpr uint32_t kMaterialMask = kXformBit - 1u;

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
//   quad        a = (n, bits)                b = (d, 0, 0, id)            c = (p, quad index)
//               (plane n.x + d = 0; u, v, w of the Planar in quad_ext, read after a plane hit)
//   cylinder    a = (p1, bits)               b = (p2 - p1, id)            c = (|p2-p1|^2, radius, |p2-p1|, 0)
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

// Compressed 8-wide node, 80 bytes (five float4), after Ylitie, Karras and
// Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide
// BVHs" (HPG 2017). Up to eight children; each child box is quantised to 8
// bits per plane on a per-node grid:
//   plane = p[a] + q * 2^(e[a] - 127),  q in 0..255,
// rounded outward, so the real (unrounded) grid box contains the child's box.
//   w0 = (p.x, p.y, p.z, bits e.x | e.y << 8 | e.z << 16 | imask << 24)
//   w1 = (child_base, prim_base, meta[0..3], meta[4..7])   (u32 bits)
//   w2 = (qlo.x[0..3], qlo.x[4..7], qhi.x[0..3], qhi.x[4..7]), w3 / w4 for y / z
// Child slot s is internal when imask bit s is set; internal children are
// stored contiguously from child_base in slot order, so slot s is node
// child_base + popc(imask & ((1 << s) - 1)). meta[s] is
//   0                                   empty slot
//   0x20 | (24 + s)                     internal child
//   ((1 << count) - 1) << 5 | offset    leaf over prims [prim_base + offset,
//                                       + count), count <= 3, offset <= 21
// so a hit child contributes the bits (meta >> 5) << (meta & 31) to one
// 32-bit hit mask: bits 24..31 internal children, bits 0..23 primitives.
// Slots are assigned per node so that visiting the internal hits in the
// order of slot ^ (ray octant) is roughly front to back.
struct alignas(16) WideNode {
  float4 w0;
  uint4 w1;
  uint4 qx, qy, qz;
};
static_assert(sizeof(WideNode) == 80, "wide node must be 80 bytes");
constexpr int kWideMaxLeaf = 3;
// ray_branching > 1: largest branching factor, and depth of the per-sample
// tree walk's stack (b^(ray_depth + 1) < 2^32 keeps ray_depth + 1 <= 32).
constexpr uint32_t kMaxBranching = 64;
constexpr int kBranchStack = 32;
// The wide traversal's stack holds at most one node group per tree level, so
// trees deeper than this traverse the binary layout instead.
constexpr int kWideMaxDepth = 60;

// Traversal stack depth; the builder keeps the tree shallower than this.
constexpr int kStackSize = 64;
constexpr int kMaxBuildDepth = 60;

// Unbounded objects, tested after the tree in list order: the SDF kinds of
// rg_sdf, and infinite planes (kind kUnboundedPlane: normal in (cx, cy, cz),
// plane offset d in p0, corner p in (p1, p2, p3), its u, v, w at quad_ext
// entry max_iter, uv wrap mode in the bits of pad[0]).
constexpr uint32_t kUnboundedPlane = 16;
struct GpuSdf {
  uint32_t kind;
  float cx, cy, cz;
  float p0, p1, p2, p3;
  uint32_t max_iter;
  float eps;
  uint32_t material;
  uint32_t prim_id;
  float bound_radius;  // outside this radius (and moving away) no hit is possible
  float inv_scale;     // Mandelbulb: 1 / scale when the scale is a power of two (the division is then an exact
                       // product), else 0
  float pad[2];
};

// Kernel variant bits (GpuScene::features): the primitive kinds a kernel is
// specialised for, and F_WIDE when it traverses the 8-wide tree.
enum : uint32_t {
  F_SPHERE = 1u,
  F_TRI = 2u,
  F_BOX = 4u,
  F_VOL = 8u,
  F_SDF = 16u,
  F_QUAD = 32u,
  F_CYLINDER = 64u,
  F_PLANE = 128u,  // unbounded infinite planes
  F_ALL = 255u,    // every primitive kind
  // Transformed objects, non-solid textures or an image sky: a separate
  // variant, so that scenes without them keep their registers.
  F_EXT = 256u,
  F_ANY = F_ALL | F_EXT,
  F_WIDE = 512u,
};
constexpr uint32_t kinds_of(uint32_t f) { return f & F_ANY; }

// Host-side dispatch: calls fn(std::integral_constant<uint32_t, F>{}) with
// the compiled kernel variant F for `features` (triangles only, spheres only,
// every kind, or every kind with transformed objects; binary or 8-wide
// traversal).
template <class Fn>
auto dispatch_features(uint32_t features, Fn&& fn) {
  const bool wide = (features & F_WIDE) != 0;
  switch (kinds_of(features)) {
    case F_TRI:
      return wide ? fn(std::integral_constant<uint32_t, F_TRI | F_WIDE>{}) : fn(std::integral_constant<uint32_t, F_TRI>{});
    case F_SPHERE:
      return wide ? fn(std::integral_constant<uint32_t, F_SPHERE | F_WIDE>{})
                  : fn(std::integral_constant<uint32_t, F_SPHERE>{});
    case F_ALL:
      return wide ? fn(std::integral_constant<uint32_t, F_ALL | F_WIDE>{}) : fn(std::integral_constant<uint32_t, F_ALL>{});
    default:
      return wide ? fn(std::integral_constant<uint32_t, F_ANY | F_WIDE>{}) : fn(std::integral_constant<uint32_t, F_ANY>{});
  }
}

// An image in HBM: `width` x `height` texels at texels[first + x * height + y].
struct GpuImage {
  uint32_t width, height, first, pad;
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
  uint32_t features;   // F_* bits of the kernel variant to launch (primitive kinds present, F_WIDE)
  const float* vol_density;   // per medium: VolumetricObject::density
  const uint32_t* vol_prim;   // per medium: its position in `prims`
  const WideNode* wnodes;     // the same primitives under the 8-wide tree (node 0 is the root)
  uint32_t n_wnodes;
  const float* quad_ext;      // per parallelogram: Planar u, v, w (9 floats)
  const float* xforms;        // per transform: inverse then forward 3 x 4 matrix, row-major (24 floats)
  const uint32_t* prim_xform; // per primitive position: its transform index (read only for flagged primitives)
  const rg_texture* textures; // non-solid textures (rg_material::texture - 1)
  const GpuImage* images;     // image headers; texels in `texels`
  const float4* texels;       // every image's texels, RGB + pad, [x][y]
  const uint8_t* perm;        // noise: per Perlin source, 512 permutation entries
  uint32_t sky_image;         // RG_SKY_IMAGE: index into images
  uint32_t stack_limit;       // traversal stack entries a ray may use (rg_tuning.stack_limit; kStackSize by default)
  uint32_t shared_stack;      // traversal stack entries per thread in shared memory (0: all in local memory)
};

// Device error bits (rg_render_stats::error_flags, RG_DEVICE_* in the C ABI).
enum : uint32_t {
  ERR_STACK_OVERFLOW = RG_DEVICE_STACK_OVERFLOW,
  ERR_BAD_INDEX = RG_DEVICE_BAD_INDEX,
  ERR_QUEUE_OVERFLOW = RG_DEVICE_QUEUE_OVERFLOW,
};

// Counters (RG_FLAG_COUNTERS): indices into the u64 counter array.
enum : uint32_t {
  CNT_RAYS = 0, CNT_NODES = 1, CNT_PRIMS = 2, CNT_SDF = 3, CNT_SAMPLES = 4,
  CNT_INVALID = 5, CNT_INVALID_MASK = 6,  // RG_FLAG_VALIDATE: broken invariants, and which (RG_INVALID_*)
  CNT_SDF_ITERS = 7,  // Mandelbulb escape-loop iterations inside the SDF evaluations
  CNT_HITS = 8,       // closest-hit queries that found a surface
  CNT_N = 16
};

// Per-frame launch parameters (all f32 values rounded from the f64 host viewport).
// `spp` is the number of samples per pixel traced by this frame: samples
// sample_base .. sample_base + spp - 1 of the pixel's spp_total (the whole
// frame unless rg_set_sample_range split it). The stratification and the
// divisor of the per-pixel sum follow spp_total.
struct FrameParams {
  uint32_t width, height, spp, ray_depth;
  uint32_t sample_base, spp_total;
  uint32_t mode;          // RG_MODE_*: PBR, or a single-intersection visualisation
  uint32_t branching;     // RenderOpts::ray_branching: scattered rays per bounce
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
  uint32_t validate;      // RG_FLAG_VALIDATE: the counting kernel variants check hits and colours
};

}  // namespace rg
