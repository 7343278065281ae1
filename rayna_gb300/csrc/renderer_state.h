// renderer_state.h — the state behind an rg_handle, shared by the
// translation units of the library.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/rayna_gpu.h"
#include "gpu_scene.h"

namespace rg {

struct HostViewport {
  double pos[3], pixel_center[3], viewport_u[3], viewport_v[3], defocus_u[3], defocus_v[3];
};

// Host copy of a flattened scene (kept for the adjoint and for rebuilding).
struct HostScene {
  uint32_t ns = 0, nt = 0, nb = 0, nv = 0, nsdf = 0, nq = 0, nc = 0, npl = 0;
  uint32_t sky = RG_SKY_SIMPLE;
  uint32_t vol_base = 0;
  int max_depth = 0;
  std::vector<BvhNode2> nodes;
  std::vector<WideNode> wnodes;        // empty when the 8-wide tree is not usable
  int wide_depth = 0;
  std::vector<GpuPrim> prims;
  std::vector<float> tri_normals;
  std::vector<rg_material> materials;
  std::vector<rg_volume> volumes;
  std::vector<GpuSdf> sdfs;            // unbounded list: SDFs, then infinite planes
  std::vector<float> quad_ext;         // per parallelogram: u, v, w
  std::vector<float> xforms;           // per transform: inverse, forward (3 x 4 each)
  std::vector<uint32_t> prim_xform;    // per primitive position: transform index (empty: no transforms)
  std::vector<rg_texture> textures;    // noise textures: `image` holds their first permutation slot
  std::vector<GpuImage> images;
  std::vector<float4> texels;
  std::vector<uint8_t> perm;           // 512 entries per noise source
  uint32_t sky_image = 0;
  bool textured = false;               // non-solid textures or an image sky
  bool vol_transformed = false;        // a medium has an object transform
  std::vector<float> vol_density;      // per medium
  std::vector<uint32_t> vol_prim;      // per medium: position in `prims`
};

struct DeviceScene {
  BvhNode2* nodes = nullptr;
  WideNode* wnodes = nullptr;
  GpuPrim* prims = nullptr;
  float* tri_normals = nullptr;
  rg_material* materials = nullptr;
  GpuSdf* sdfs = nullptr;
  float* quad_ext = nullptr;
  float* xforms = nullptr;
  uint32_t* prim_xform = nullptr;
  rg_texture* textures = nullptr;
  GpuImage* images = nullptr;
  float4* texels = nullptr;
  uint8_t* perm = nullptr;
  float* vol_density = nullptr;
  uint32_t* vol_prim = nullptr;
};

// Wavefront queues (allocated on first use, sized by the path budget).
struct WavefrontState {
  size_t capacity = 0;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  void* marchq = nullptr;  // per-SDF march queues (SDFs x capacity u32)
  size_t marchq_bytes = 0;
};

}  // namespace rg

struct rg_renderer {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  uint32_t form = RG_FORM_MEGAKERNEL;
  uint32_t flags = 0;
  std::string err;

  bool have_scene = false;
  rg::HostScene host;
  rg::DeviceScene dev;
  rg::GpuScene gs{};

  rg_camera cam{};
  bool cam_ok = false;
  rg::HostViewport vp{};
  rg_render_opts opts{};

  uint32_t acc_w = 0, acc_h = 0;
  float* d_accum = nullptr;
  float* d_out = nullptr;
  float* d_fmean = nullptr;
  float* d_fvar = nullptr;
  uint32_t frame_count = 0;   // AccumulationBuffer::counter
  bool frame_current = false; // d_fmean holds a PBR frame of the current scene, camera, options and parameters
  uint32_t pixel_accum = 0;   // AccumulationValue::accum (per pixel; equal for all pixels)
  uint64_t last_samples = 0;
  uint32_t last_launches = 0; // kernels launched by the last frame
  std::vector<cudaEvent_t> stage_ev;  // RG_FLAG_STAGE_TIMES: (start, end) pairs of traversal launches
  uint32_t stage_used = 0;            // events of stage_ev recorded by the last frame

  unsigned long long* d_counters = nullptr;
  uint32_t* d_err = nullptr;
  // Page-locked host copy of the frame's counters and error word, read back
  // with one asynchronous copy each and a single stream synchronisation.
  unsigned long long* h_counters = nullptr;  // CNT_N counters, then the error word
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  rg::WavefrontState wf;
  size_t wf_paths = 0;        // wavefront path slots per wave (0: library default)
  uint32_t wf_sort = 0;       // wavefront: 1 sorted extend/shade stages, 2 fused bounce kernel, 0 by scene
  uint32_t wf_budget = 0;     // wavefront: node visits between refills (0: library default)
  uint32_t bvh_width = 0;     // requested traversal: 2, 8, or 0 for the library default
  uint32_t shared_stack = 0;  // requested shared traversal-stack entries: 0 default, RG_SHARED_STACK_NONE, 4, 8, 16
  uint32_t mega_block = 0;    // megakernel threads per block (0: 256)
  uint32_t stack_limit = 0;   // traversal stack entries a ray may use (0: kStackSize)
  uint32_t march_budget = 0;  // SDF evaluations per lane between refills in the march stages (0: kMarchBudgetDefault)
  uint32_t shade_lanes = 0;   // ready lanes before a persistent wavefront warp finishes them (0: kShadeLanesDefault)
  uint32_t tail_paths = 0;    // fused bounce: queues of at most this many paths run to their ends (0: kTailPathsDefault)
  uint32_t range_first = 0;   // rg_set_sample_range: the frame's first sample
  uint32_t range_count = 0;   //   and its number of samples (0: whole frames)
  uint32_t kinds = 0;         // F_* primitive-kind bits of the scene's kernel variant
  uint32_t have = 255u;       // F_* bits of the kinds the scene holds (F_EXT with transforms or textures); F_ALL

  void* d_adj = nullptr;      // adjoint scratch (image, adjoint image, gradients)
  size_t adj_bytes = 0;
};

namespace rg {

// Traversal width used when the tuning leaves it at 0. The 8-wide tree
// visits about a third of the nodes, but each visit tests eight boxes, and
// every form measured faster on the binary tree.
constexpr uint32_t kDefaultBvhWidthWavefront = 2;
constexpr uint32_t kDefaultBvhWidthMegakernel = 2;
// Node visits between refills of the persistent traversal kernels: 6
// (measured on the fused mesh workload 614 Msamples/s at 6 against 598 at 8
// and 565 at 12; on the random-spheres workload 1195 at 6, 1100 at 8, 1096 at
// 4).
constexpr uint32_t kDefaultFetchBudget = 6;
// Megakernel threads per block when the tuning leaves it at 0: 128 (the three
// workloads measured within 1 % of their best at 128: mesh 350 Msamples/s
// against 353 at 64 and 345 at 256, random spheres 820 / 823 / 798, SDF 177
// against 173 at 256).
constexpr uint32_t kDefaultMegaBlock = 128;
// Distance evaluations per lane between refills in the SDF march stages when
// the tuning leaves it at 0. With per-SDF march queues (few paths rejected at
// fetch, so refills are cheap) the SDF workload measured 1005, 1010, 1009,
// 1009 and 994 Msamples/s at 8, 12, 16, 24 and 32; with one queue for every
// stage it had peaked at 32 (819, against 778 at 16 and 779 at 64).
constexpr uint32_t kMarchBudgetDefault = 16;
// A warp of a persistent wavefront kernel finishes its ready paths (shading,
// hit records, SDF hit normals: long code that would otherwise run for one or
// two lanes at a time) together once this many lanes are ready, or all of its
// live lanes are. The fused mesh workload measured 610 Msamples/s at 1 (each
// path finished when ready), 676 at 8, 695 at 16, 653 at 24 and 503 at 32;
// random spheres 1237 at 1, 1305 at 16, 1313 at 24; the SDF workload (extend
// and march stages) 822 at 1, 835 at 16, 817 at 24.
constexpr uint32_t kShadeLanesDefault = 16;
// The same for the batched wavefront's bounce kernel: the 64-scene batch
// measured 1917 Msamples/s at 1, 2282 at 16 and 2331 at 24.
constexpr uint32_t kBatchShadeLanesDefault = 24;
// A fused bounce whose queue holds at most this many paths runs them to their
// ends in that launch (rg_tuning.tail_paths). Random spheres (2.88 M paths,
// depth 50) measured 1329 Msamples/s with no continuation, 1735 at 2^16, 1808
// at 2^20 and 1888 with the whole frame continued from the first launch; the
// mesh (67 M paths, depth 8) 708 with none or up to 2^24, 696 with all.
constexpr uint32_t kTailPathsDefault = 1u << 22;
// Default path slots per wave (at most about 14.5 GB of path state at 108
// bytes per slot; clamped to the frame). Every wave pays each bounce's tail,
// the few longest paths (a long march, a deep traversal) that hold the stage
// while most of the GPU idles, so frames run best as few waves as memory
// allows: the SDF workload (118 M paths) measured 814, 891 and 937
// Msamples/s at 2^25, 2^26 and 2^27 slots, the mesh (67 M) 699 and 710 at
// 2^25 and 2^26, the 64-scene batch 2354, 2410 and 2432.
constexpr size_t kDefaultWavePaths = size_t(1) << 27;

// Defined in renderer.cpp
// RG_FLAG_STAGE_TIMES: records the next event of the frame's traversal timing
// (start before a traversal launch, end after it) on the handle's stream.
cudaError_t stage_mark(rg_renderer* h);
// Traversal width in effect for a request (0 = default) on a scene.
uint32_t effective_bvh_width(uint32_t requested, const GpuScene& g, uint32_t form);
// Whether the wavefront shades in material-kind order: as requested, else
// sorted for scenes with SDFs or media (whose marching and free-flight work
// diverges inside one fused kernel) and fused otherwise (measured: SDF
// workload 318 sorted vs 134 fused Msamples/s; mesh 543 vs 569; spheres 878
// vs 1143).
bool effective_sort(const rg_renderer* h);
// Node visits between refills of the persistent kernels: as requested, else
// the default for the scene's kinds.
uint32_t effective_budget(const rg_renderer* h);
// Shared traversal-stack entries per thread when the tuning leaves them at 0:
// 8 for scenes of triangles only (the 1.3M-triangle mesh measured 1.07x with
// the split in the persistent kernels), none elsewhere (0.98x on spheres,
// 1.00x on the SDF scene).
constexpr uint32_t kDefaultSharedStackTriangles = 8;
// Kernel variant bits (the scene's primitive kinds, plus F_WIDE when the
// handle traverses the 8-wide tree) and the stack knobs of the handle's scene.
void apply_features(rg_renderer* h);
// Status of a frame's device error bits (RG_DEVICE_*): RG_OK when none.
rg_status device_status(uint32_t err);
// RAYNA_GPU_FAIL_ALLOC=n: the n-th allocation the library counts (host scene
// build or device buffer, from 1) fails as if memory ran out. A test hook for
// the RG_OOM paths; every allocation site asks before allocating.
bool alloc_fault();
rg_status build_scene_host(rg_renderer* h, const rg_scene_desc& d, HostScene& hs);
void fill_frame_params(rg_renderer* h, uint64_t seed, FrameParams& fp);
rg_status ensure_frame_buffers(rg_renderer* h);
rg_status set_error(rg_renderer* h, rg_status st, const char* msg);

// Defined in adjoint.cu
// `last_frame`: with a target, I is the handle's last rendered frame (d_fmean)
// instead of a frame rendered here.
rg_status backward_device(rg_renderer* h, uint64_t seed, const float* adjoint, const float* target, rg_gradients* out,
                          bool last_frame = false);

// Defined in wavefront.cu
cudaError_t launch_wavefront(rg_renderer* h, const FrameParams& fp);
cudaError_t launch_wavefront_static(rg_renderer* h, const FrameParams& fp);
void free_extra(rg_renderer* h);
void on_scene_changed(rg_renderer* h);

}  // namespace rg
