/*
 * rayna_gpu.h — C ABI of the GB300 (sm_103a) path-tracing library.
 *
 * This is the drop-in boundary for rayna_engine's CPU render call. Every entry
 * point below replaces one method of `Renderer<Obj, Sky, Rng>`
 * (rayna_engine/src/render/renderer.rs) or a piece of state it owns; the
 * comment on each names the reference interface it stands in for.
 *
 * Conventions
 *   - Every function returns rg_status; nothing unwinds across the boundary.
 *     rg_last_error() gives a human-readable message for the last failure on
 *     a handle (or the last handle-less failure when h == NULL).
 *   - A handle is not thread-safe: calls on one handle must be serialised by
 *     the caller, exactly as `&mut self` serialises them in the reference.
 *     Separate handles may be used from separate threads.
 *   - All scene arrays are host pointers owned by the caller; the library
 *     copies what it needs during the call.
 *   - Geometry and radiance are FP32 on the device. The camera is given in
 *     f64 (the reference's `Number`) and its viewport is computed on the host
 *     in f64 exactly like Camera::calculate_viewport, then rounded to f32.
 *   - Images are laid out [x][y][rgb] (x-major), which is the memory order of
 *     the reference's `Image` (an ndarray of shape (width, height),
 *     rayna_engine/src/core/image.rs:24-25): pixel (x, y) starts at float
 *     offset 3 * (x * height + y).
 */
#ifndef RAYNA_GPU_H
#define RAYNA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RG_ABI_VERSION 8u

/* Status codes. 0 is success. */
typedef enum rg_status {
    RG_OK = 0,
    RG_INVALID_ARG = 1,          /* malformed descriptor, NaN/Inf parameter, bad size */
    RG_UNSUPPORTED_VARIANT = 2,  /* a reference variant this library does not run (e.g. a non-identity transform) */
    RG_INVALID_CAMERA = 3,       /* Camera::calculate_viewport returned Err (scene/camera.rs:114-167) */
    RG_OOM = 4,                  /* device or host allocation failed */
    RG_CUDA_ERROR = 5,           /* a CUDA runtime call failed; see rg_last_error */
    RG_QUEUE_OVERFLOW = 6,       /* a device queue or traversal stack ran out of space */
    RG_STEP_LIMIT = 7,           /* a device loop hit its iteration budget */
    RG_TIMEOUT = 8,              /* a bounded wait ran out */
    RG_NO_DEVICE = 9,            /* no CUDA device is visible */
    RG_NOT_READY = 10            /* call order violated (e.g. render before set_scene) */
} rg_status;

typedef struct rg_renderer* rg_handle;

/* ------------------------------------------------------------------------ */
/* Scene description (flattened StandardScene)                               */
/* ------------------------------------------------------------------------ */

/* Material kinds: MaterialInstance variants (rayna_engine/src/material/mod.rs:168-175).
 * Their colour is `albedo` (a SolidTexture, texture/solid.rs:28-30) unless
 * `texture` names an entry of rg_scene_desc.textures. */
enum {
    RG_MAT_LAMBERTIAN = 0,  /* LambertianMaterial { albedo }                      material/lambertian.rs */
    RG_MAT_METAL = 1,       /* MetalMaterial { albedo, fuzz }                      material/metal.rs */
    RG_MAT_DIELECTRIC = 2,  /* DielectricMaterial { albedo, refractive_index, density } material/dielectric.rs */
    RG_MAT_ISOTROPIC = 3,   /* IsotropicMaterial { albedo, density }               material/isotropic.rs */
    RG_MAT_LIGHT = 4        /* LightMaterial { emissive } (colour in `albedo`)     material/light.rs */
};

/* 32 bytes; the device material table holds these verbatim. */
typedef struct rg_material {
    uint32_t kind;
    float albedo[3];          /* albedo, or emissive radiance for RG_MAT_LIGHT */
    float fuzz;               /* metal */
    float refractive_index;   /* dielectric */
    float density;            /* dielectric / isotropic Beer term (material density) */
    uint32_t texture;         /* 0: the solid `albedo`; k > 0: texture k - 1 of rg_scene_desc.textures */
} rg_material;

/* Texture kinds (texture/mod.rs:27-37). */
enum {
    RG_TEX_SOLID = 0,          /* SolidTexture: `colour` (texture/solid.rs:28-30) */
    RG_TEX_WORLD_CHECKER = 1,  /* WorldCheckerTexture (texture/checker.rs:20-27): pos_w / scale[0] + offset */
    RG_TEX_UV_CHECKER = 2,     /* UvCheckerTexture (checker.rs:37-44): uv / scale[0] + offset.xy */
    RG_TEX_IMAGE = 3,          /* ImageTexture (texture/image.rs:29-39): bilinear in image `image` at
                                  offset.xy + uv * scale.xy, v flipped */
    RG_TEX_NOISE = 4           /* World/Local/UvNoiseTexture over a Perlin source (texture/noise.rs) */
};

/* Where a noise texture samples its Perlin source (texture/noise.rs). */
enum {
    RG_NOISE_WORLD = 0,        /* WorldNoiseTexture: at pos_w */
    RG_NOISE_LOCAL = 1,        /* LocalNoiseTexture: at the mesh-local point pos_l */
    RG_NOISE_UV = 2            /* UvNoiseTexture: at uv (2-D) */
};

/* 64 bytes. A checker's `odd` / `even` are indices into the same table; the
 * table must be acyclic, at most RG_MAX_TEXTURE_DEPTH checkers deep. */
typedef struct rg_texture {
    uint32_t kind;             /* RG_TEX_* */
    uint32_t odd, even;        /* checker: the textures of odd / even cells */
    uint32_t image;            /* image: index into rg_scene_desc.images */
    float scale[2];            /* checker: scale[0]; image: Size2 scale; noise: the ScalePoint factor in scale[0] */
    float offset[3];           /* world checker: xyz; uv checker and image: xy */
    float colour[3];           /* solid: the colour */
    uint32_t noise_seed;       /* noise: Perlin::new(seed) */
    uint32_t noise_place;      /* noise: RG_NOISE_* */
    uint32_t noise_channels;   /* noise: 1 = ColourSource::Greyscale; 3 = Rgb of sources seeded seed, seed+1, seed+2 */
    uint32_t reserved;         /* must be 0 */
} rg_texture;

#define RG_MAX_TEXTURE_DEPTH 16u

/* An RGB f32 image, [x][y][rgb] (core/image.rs: ndarray of shape (width, height)). */
typedef struct rg_image {
    uint32_t width, height;    /* both > 0 */
    const float* rgb;          /* width x height x 3 */
} rg_image;

/* Skybox variants (rayna_engine/src/skybox/mod.rs:28-43). */
enum {
    RG_SKY_SIMPLE = 0,  /* SimpleSkybox: lerp(white, (0.5,0.7,1), 0.5*dir.y+0.5) */
    RG_SKY_WHITE = 1,   /* WhiteSkybox */
    RG_SKY_NONE = 2,    /* NoSkybox (black) */
    RG_SKY_IMAGE = 3    /* HdrImageSkybox (skybox/hdri.rs:17-26): bilinear in image `sky_image` at sphere_uv(dir) */
};

/* Constant-density medium: VolumetricObject (rayna_engine/src/object/volumetric.rs). */
enum { RG_BOUNDARY_SPHERE = 0, RG_BOUNDARY_BOX = 1 };
typedef struct rg_volume {
    uint32_t boundary;  /* RG_BOUNDARY_SPHERE: a = centre, b[0] = radius; RG_BOUNDARY_BOX: a, b = two corners */
    float a[3];
    float b[3];
    float density;      /* medium density (VolumetricObject::density) */
    uint32_t material;  /* index into the material table */
} rg_volume;

/* Signed-distance functions that can cross the C ABI. The reference takes an
 * arbitrary closure (mesh/isosurface/mod.rs:7-9); closures cannot cross an FFI,
 * so RaymarchedIsosurfaceMesh is described by one of these kinds. */
enum {
    RG_SDF_SPHERE = 0,      /* params[0] = radius */
    RG_SDF_TORUS = 1,       /* params[0] = major radius R, params[1] = minor radius r; axis = +y */
    RG_SDF_MANDELBULB = 2   /* params[0] = power, params[1] = iterations, params[2] = scale (world units per unit bulb) */
};
typedef struct rg_sdf {
    uint32_t kind;
    float centre[3];
    float params[4];
    uint32_t max_iterations;  /* RaymarchedIsosurfaceMesh::max_iterations */
    float epsilon;            /* RaymarchedIsosurfaceMesh::epsilon */
    uint32_t material;
} rg_sdf;

/* A flattened scene. Object order (which decides exact-distance ties and the
 * order of unbounded objects) is: spheres, standalone triangles, triangle
 * meshes (by mesh id), boxes, volumes, parallelograms, cylinders; then the
 * unbounded objects: SDFs, infinite planes. Global primitive ids, as reported
 * by rg_query_rays, number the arrays in this order: spheres [0, ns),
 * triangles [ns, ns+nt), boxes, volumes, SDFs, parallelograms, cylinders,
 * infinite planes. */
typedef struct rg_scene_desc {
    uint32_t n_spheres;
    const float* spheres;            /* n x 4: centre xyz, radius */
    const uint32_t* sphere_material; /* n */

    uint32_t n_triangles;
    const float* tri_vertices;       /* n x 3 x 3 */
    const float* tri_normals;        /* n x 3 x 3, unit length (Triangle::new asserts it) */
    const uint32_t* tri_material;    /* n */
    const int32_t* tri_mesh;         /* n: BvhMesh id, or -1 for a standalone Triangle object; NULL = all standalone */

    uint32_t n_boxes;
    const float* boxes;              /* n x 6: corner a xyz, corner b xyz (AxisBoxMesh::new) */
    const uint32_t* box_material;    /* n */

    uint32_t n_volumes;
    const rg_volume* volumes;

    uint32_t n_sdfs;
    const rg_sdf* sdfs;

    uint32_t n_materials;
    const rg_material* materials;

    uint32_t skybox;                 /* RG_SKY_* */

    uint32_t n_quads;                /* ParallelogramMesh (mesh/planar/parallelogram.rs) */
    const float* quads;              /* n x 9: Planar p, u, v (corner and two sides; uv in [0,1]^2 is inside) */
    const uint32_t* quad_material;   /* n */

    uint32_t n_cylinders;            /* CylinderMesh (mesh/primitive/cylinder.rs) */
    const float* cylinders;          /* n x 7: p1 xyz, p2 xyz, radius (> 0, p1 != p2) */
    const uint32_t* cylinder_material;

    uint32_t n_planes;               /* InfinitePlaneMesh (mesh/planar/infinite_plane.rs): unbounded */
    const float* planes;             /* n x 9: Planar p, u, v */
    const uint32_t* plane_material;
    const uint32_t* plane_uv_wrap;   /* n: RG_UV_WRAP_* (UvWrappingMode, infinite_plane.rs:18-45); NULL = all WRAP */

    /* ObjectTransform of SimpleObjects (object/transform.rs): a ray is mapped
     * into mesh space by the inverse, tested against the mesh from the caller's
     * start, and the hit mapped back (point and normals by the transform,
     * distance recomputed in world space and bounded by the caller's end). */
    uint32_t n_transforms;
    const double* transforms;            /* n x 12: 3 x 4 affine matrix, mesh space to world space, row-major, with
                                            SimpleObject::new's correction about the mesh centre already applied */
    const uint32_t* sphere_transform;    /* n_spheres: index into transforms or RG_NO_TRANSFORM; NULL = none */
    const uint32_t* tri_transform;       /* n_triangles */
    const uint32_t* box_transform;       /* n_boxes */
    const uint32_t* quad_transform;      /* n_quads */
    const uint32_t* cylinder_transform;  /* n_cylinders */

    /* Non-solid textures (rg_material.texture) and images (ImageTexture, HdrImageSkybox). */
    uint32_t n_textures;
    const rg_texture* textures;
    uint32_t n_images;
    const rg_image* images;
    uint32_t sky_image;              /* RG_SKY_IMAGE: index into images */
    const uint32_t* volume_transform;/* n_volumes: ObjectTransform of VolumetricObjects (object/volumetric.rs:21-45),
                                        index into transforms or RG_NO_TRANSFORM; NULL = none */
} rg_scene_desc;

#define RG_NO_TRANSFORM 0xFFFFFFFFu

/* UvWrappingMode of an infinite plane's texture coordinates. */
enum { RG_UV_WRAP = 0, RG_UV_MIRROR = 1, RG_UV_CLAMP_ZERO = 2 };

/* Camera (rayna_engine/src/scene/camera.rs:10-25), angles in radians. */
typedef struct rg_camera {
    double pos[3];
    double fwd[3];
    double v_fov;
    double focus_dist;
    double defocus_angle;
} rg_camera;

/* RenderMode (rayna_engine/src/render/render_opts.rs:34-52). */
enum {
    RG_MODE_PBR = 0,
    RG_MODE_RAY_NORMAL = 1,
    RG_MODE_OUTWARD_NORMAL = 2,
    RG_MODE_SCATTER = 3,
    RG_MODE_FRONT_FACE = 4,
    RG_MODE_DISTANCE = 5,
    RG_MODE_UV = 6,
    RG_MODE_SIDE = 7
};

/* RenderOpts (render_opts.rs:8-29). Every RenderMode renders (the debug modes
 * and ray_branching > 1 by the megakernel, whatever the handle's form);
 * ray_branching^(ray_depth + 1) must stay below 2^32. width/height/samples/ray_branching are
 * NonZeroUsize in the reference: 0 is rejected with RG_INVALID_ARG. */
typedef struct rg_render_opts {
    uint32_t width;
    uint32_t height;
    uint32_t samples;
    uint32_t mode;
    uint32_t ray_depth;
    uint32_t ray_branching;
} rg_render_opts;

/* Which kernel form renders a frame. Both forms run the same estimator and
 * produce the same image for the same seed. The wavefront is the fast form
 * (the Python binding's default); the megakernel is the plain form that a
 * zero-initialised rg_device_opts selects. */
enum { RG_FORM_MEGAKERNEL = 0, RG_FORM_WAVEFRONT = 1 };

typedef struct rg_device_opts {
    int32_t device;        /* CUDA ordinal */
    void* stream;          /* cudaStream_t to run on, or NULL for a library-owned stream */
    uint32_t form;         /* RG_FORM_* */
    uint32_t flags;        /* RG_FLAG_* */
} rg_device_opts;

enum {
    RG_FLAG_COUNTERS = 1u,     /* maintain device work counters (node visits, tests) for the roofline */
    RG_FLAG_STAGE_TIMES = 2u,  /* time the traversal kernels of each frame with CUDA events (traverse_ms) */
    RG_FLAG_VALIDATE = 4u      /* check every closest hit and path colour against shared/validate.rs's invariants
                                  (counted in invalid_hits / invalid_mask; implies RG_FLAG_COUNTERS; the wavefront
                                  then shades fused) */
};

/* RenderStats (render/render.rs:4-15) plus device figures. */
typedef struct rg_render_stats {
    double duration_ms;       /* wall time of the call */
    double kernel_ms;         /* device time of this frame's kernels (CUDA events on the handle's stream) */
    uint64_t samples;         /* path samples traced this frame */
    uint64_t rays;            /* extend queries (ray segments) this frame */
    uint64_t node_visits;     /* BVH node pairs fetched (RG_FLAG_COUNTERS only, else 0) */
    uint64_t prim_tests;      /* primitive tests (RG_FLAG_COUNTERS only, else 0) */
    uint64_t sdf_steps;       /* SDF evaluations, the normals' central differences included (RG_FLAG_COUNTERS only) */
    uint32_t accum_frames;    /* AccumulationBuffer::frame_count */
    uint32_t img_width;       /* dimensions of the image written to out_rgb */
    uint32_t img_height;
    uint32_t num_threads;     /* 0: the device renders */
    uint32_t error_flags;     /* device-side error bits seen this frame (0 = none): RG_DEVICE_* */
    uint32_t kernel_launches; /* kernels the library launched for this frame */
    double traverse_ms;       /* device time of the frame's traversal kernels (RG_FLAG_STAGE_TIMES only, else 0):
                                 the megakernel, or the wavefront's extend / bounce launches */
    uint64_t invalid_hits;    /* RG_FLAG_VALIDATE: hits or path colours that broke an invariant this frame */
    uint32_t invalid_mask;    /* RG_FLAG_VALIDATE: RG_INVALID_* bits of the invariants broken */
    uint32_t reserved0;
    uint64_t hits;            /* closest-hit queries that found a surface (RG_FLAG_COUNTERS only, else 0) */
    uint64_t sdf_iterations;  /* Mandelbulb escape-loop iterations in the SDF evaluations (RG_FLAG_COUNTERS only) */
} rg_render_stats;

/* Device error bits (rg_render_stats.error_flags). They are cleared at the start
 * of every frame (and every query or backward call); a frame that sets any of
 * them returns a status other than RG_OK from rg_render, rg_sync_stats,
 * rg_batch_render and rg_query_rays, while the image is still written:
 *   RG_DEVICE_STACK_OVERFLOW, RG_DEVICE_QUEUE_OVERFLOW -> RG_QUEUE_OVERFLOW
 *   RG_DEVICE_BAD_INDEX (a damaged tree: the traversal's visit guard ran out) -> RG_STEP_LIMIT */
enum {
    RG_DEVICE_STACK_OVERFLOW = 1u,  /* a ray needed more traversal stack than it may use; its far subtree was dropped */
    RG_DEVICE_BAD_INDEX = 2u,       /* a node or primitive index out of range, or a node visited twice */
    RG_DEVICE_QUEUE_OVERFLOW = 4u   /* a path queue ran out of slots; the path was dropped */
};

/* Invariants of RG_FLAG_VALIDATE (shared/validate.rs:21-197). */
enum {
    RG_INVALID_NONFINITE = 1u,       /* hit distance, point or a normal not finite */
    RG_INVALID_NOT_NORMALISED = 2u,  /* |normal|^2 or |ray_normal|^2 off 1 by more than 2e-3 (length 1e-3 relative) */
    RG_INVALID_INTERVAL = 4u,        /* hit distance outside the query interval */
    RG_INVALID_POSITION = 8u,        /* the point is not at the distance along the ray (1e-6 abs or 1e-3 rel) */
    RG_INVALID_UV = 16u,             /* uv outside [0, 1]^2 or NaN */
    RG_INVALID_COLOUR = 32u          /* a path's colour channel negative or not finite */
};

/* Hit record of rg_query_rays. */
typedef struct rg_hit {
    uint32_t hit;        /* 0 or 1 */
    uint32_t prim;       /* global primitive id (see rg_scene_desc) */
    float t;             /* Intersection::dist */
    float normal[3];     /* Intersection::normal (outward) */
    float ray_normal[3]; /* Intersection::ray_normal (against the ray) */
    uint32_t front_face;
    uint32_t material;
    uint32_t side;       /* Intersection::side */
} rg_hit;  /* 48 bytes */

/* Host-side summary of a scene as the library would build it. */
typedef struct rg_scene_info {
    uint32_t n_prims;        /* bounded primitives in the BVH */
    uint32_t n_unbounded;    /* SDFs and infinite planes */
    uint32_t n_nodes;        /* 64-byte node pairs */
    uint32_t max_depth;      /* deepest node pair (traversal stack bound) */
    uint32_t n_leaves;
    uint32_t max_leaf_size;
    double sah_cost;         /* sum over node pairs of child area x prims / root area */
    uint64_t device_bytes;   /* bytes the scene occupies in device memory (both trees) */
    uint32_t n_wide_nodes;   /* 80-byte nodes of the 8-wide tree (0: the scene traverses the binary tree only) */
    uint32_t wide_depth;     /* deepest 8-wide node */
} rg_scene_info;

/* ------------------------------------------------------------------------ */
/* Renderer lifecycle                                                         */
/* ------------------------------------------------------------------------ */

/* ABI version of the loaded library (RG_ABI_VERSION). */
uint32_t rg_abi_version(void);

/* Replaces Renderer::new_from / new_default (renderer.rs:66-107). Creates the
 * handle and its stream; scene, camera and options are set separately. */
rg_status rg_create(const rg_device_opts* opts, rg_handle* out);

/* Drop for Renderer. Frees every device buffer of the handle. */
rg_status rg_destroy(rg_handle h);

/* Last error message for `h` (or the thread's last handle-less error when h is NULL). */
rg_status rg_last_error(rg_handle h, char* buf, size_t len);

/* Validates a scene and builds its BVH on the host only, without a device
 * (no reference counterpart: the preflight half of Renderer::set_scene,
 * renderer.rs:165-168, so callers can reject a scene before creating a
 * handle). Fails exactly where rg_set_scene would fail validation. */
rg_status rg_inspect_scene(const rg_scene_desc* scene, rg_scene_info* out);

/* Renderer::set_scene (renderer.rs:165-168): copies the scene to the device,
 * builds the BVH and clears the accumulation buffer. A scene rejected by
 * validation leaves the previous one in place; a failed device upload
 * (RG_OOM, RG_CUDA_ERROR) leaves the empty scene. */
rg_status rg_set_scene(rg_handle h, const rg_scene_desc* scene);

/* Launch-shape knobs of the kernel forms (no reference counterpart: the
 * reference has no device; these are what the autotuner sets). Zero fields
 * select the library defaults. Changing them does not change the image. */
typedef struct rg_tuning {
    uint32_t wave_paths;      /* wavefront: path slots per wave (whole pixels per wave; 108 bytes of device memory
                                 each); 0 = 2^27, clamped to the frame */
    uint32_t sort_materials;  /* wavefront: 1 = separate extend and shade stages, shading in material-kind order;
                                 2 = one fused bounce kernel; 0 = library default (fused for scenes of spheres
                                 only, sorted otherwise) */
    uint32_t bvh_width;       /* 2 = binary node pairs, 8 = compressed 8-wide nodes; 0 = library default (2).
                                 Either tree gives the same closest hits. */
    uint32_t fetch_budget;    /* wavefront: node visits a lane traverses between refills of idle lanes; 0 = 6 */
    uint32_t shared_stack;    /* entries of each thread's traversal stack kept in shared memory (the deeper ones
                                 live in local memory): 0 = library default (8 for scenes of triangles only, else
                                 none), RG_SHARED_STACK_NONE = all in local memory, else 4, 8 or 16 */
    uint32_t block;           /* megakernel: threads per block, 64, 128 or 256; 0 = 128 */
    uint32_t stack_limit;     /* test knob: traversal stack entries a ray may use (1-64); a ray that needs more
                                 drops the far subtree and the frame reports RG_QUEUE_OVERFLOW; 0 = all 64 */
    uint32_t march_budget;    /* material-sorted wavefront with raymarched SDFs: distance evaluations a lane of a
                                 march stage performs between refills of idle lanes (1-4096); 0 = 16 */
    uint32_t shade_lanes;     /* wavefront: a warp of a persistent kernel finishes its ready paths (shading in the
                                 fused bounce kernel, the hit record in the extend stage, the hit normal in a march
                                 stage) together, once at least this many of its lanes are ready or all of its live
                                 lanes are (1-32; 1 = each path as soon as it is ready); 0 = 16 */
    uint32_t tail_paths;      /* fused wavefront: a bounce whose queue holds at most this many paths runs each of them
                                 to its end in that launch (the tail of deep scenes); 0 = 2^22, 1 = never in effect */
    uint32_t reserved;        /* must be 0 */
} rg_tuning;

#define RG_SHARED_STACK_NONE 0xFFFFFFFFu

rg_status rg_set_tuning(rg_handle h, const rg_tuning* t);
/* The knobs in effect: library defaults appear resolved (never 0). */
rg_status rg_get_tuning(rg_handle h, rg_tuning* out);

/* Renderer::set_camera (renderer.rs:158-161): also clears accumulation. An
 * invalid camera is accepted here, as in the reference; render reports it. */
rg_status rg_set_camera(rg_handle h, const rg_camera* camera);

/* Renderer::set_options (renderer.rs:173-176): also clears accumulation. */
rg_status rg_set_options(rg_handle h, const rg_render_opts* opts);

/* Renderer::clear_accumulation (renderer.rs:153). */
rg_status rg_clear_accumulation(rg_handle h);

/* Renderer::render (renderer.rs:224-264). Adds one frame of `samples`
 * samples per pixel to the accumulation buffer and writes the running mean to
 * `out_rgb` (host memory, width*height*3 floats, [x][y][rgb]) when it is not
 * NULL. `seed` keys the counter-based random streams of this frame.
 * With an invalid camera the call returns RG_INVALID_CAMERA and writes the
 * reference's fallback checker image (renderer.rs:269-292), whose dimensions
 * are ilog2(width) x ilog2(height), reported in out_stats. */
rg_status rg_render(rg_handle h, uint64_t seed, float* out_rgb, rg_render_stats* out_stats);

/* Same frame as rg_render, but the running mean is written to device memory
 * `d_out_rgb` (or not written when NULL) and the call does not wait for the
 * device: it returns once the frame's kernels are queued on the stream.
 * Stats other than `samples` are filled by rg_sync_stats. */
rg_status rg_render_async(rg_handle h, uint64_t seed, float* d_out_rgb, rg_render_stats* out_stats);

/* Waits for the handle's stream and fills device timings and counters of the
 * last queued frame. */
rg_status rg_sync_stats(rg_handle h, rg_render_stats* out_stats);

/* Splits one frame across devices by sample range (no reference counterpart:
 * the reference folds every sample of a pixel on one machine,
 * render/renderer.rs:313-336 and accum_buffer.rs:37-42). After this call each
 * frame of the handle traces only samples [first, first + count) of every
 * pixel's `samples`, with the random streams those samples have in a whole
 * frame, and adds their sum divided by `samples` to the accumulation buffer.
 * Handles that cover disjoint ranges of [0, samples) with the same frame keys
 * therefore hold accumulation sums whose element-wise sum is the whole
 * frames' sum (up to float summation order), with the same frame count: the
 * exchange is one sum-reduce of rg_get_accumulation's sums. count 0 restores
 * whole frames. Clears the accumulation; rg_set_options restores whole
 * frames. rg_frame_moments then describes the range's samples, and
 * rg_backward_frame refuses a sharded frame (RG_NOT_READY). first + count
 * above `samples` is RG_INVALID_ARG. */
rg_status rg_set_sample_range(rg_handle h, uint32_t first, uint32_t count);

/* Checkpoint/resume of the AccumulationBuffer (accum_buffer.rs:9-78):
 * `sum` is width*height*3 floats in [x][y][rgb] order, `frames` the count. */
rg_status rg_get_accumulation(rg_handle h, float* sum, uint32_t* frames);
rg_status rg_set_accumulation(rg_handle h, const float* sum, uint32_t frames);

/* Per-pixel sample statistics of the last frame: mean and unbiased sample
 * variance over the frame's `samples` samples, [x][y][rgb] each. Used to state
 * Monte Carlo standard errors. */
rg_status rg_frame_moments(rg_handle h, float* mean, float* variance);

/* Ray-query entry (no reference counterpart as a public call: it exposes
 * ObjectInstance::full_intersect, object/mod.rs:59-71, for parity tests).
 * Rays are traced against the current scene with interval [tmin[i], tmax[i]].
 * `volume_u`, if not NULL, is n x n_volumes uniforms in (0,1] used for the
 * free-flight draw of each medium instead of the counter-based stream. */
rg_status rg_query_rays(rg_handle h, uint32_t n, const float* origins, const float* dirs,
                        const float* tmin, const float* tmax, const float* volume_u, rg_hit* out);

/* ------------------------------------------------------------------------ */
/* Batched rendering (no reference counterpart: many Renderers at once)       */
/* ------------------------------------------------------------------------ */

typedef struct rg_batch* rg_batch_handle;

/* Launch shape of the persistent batch kernel (what the autotuner sets). */
/* Batched forms (rg_batch_tuning.form). */
enum {
    RG_BATCH_WAVEFRONT = 0,  /* default: the paths of every render in shared waves of path slots; one persistent
                                dynamic-fetch bounce launch per bounce serves all renders */
    RG_BATCH_TILES = 1       /* one persistent launch whose warps take (render, tile) items, megakernel style */
};

typedef struct rg_batch_tuning {
    uint32_t block;            /* RG_BATCH_TILES: threads per block, multiple of 32 in [64, 512]; 0 = 256 */
    uint32_t blocks_per_sm;    /* RG_BATCH_TILES: blocks launched per SM; 0 = as many as fit */
    uint32_t rounds_per_item;  /* RG_BATCH_TILES: warp rounds of pixels per work item; 0 = 4 */
    uint32_t bvh_width;        /* 2 or 8 as in rg_tuning; 0 = library default (2) */
    uint32_t form;             /* RG_BATCH_WAVEFRONT or RG_BATCH_TILES */
    uint32_t wave_paths;       /* RG_BATCH_WAVEFRONT: path slots per wave; 0 = min(2^27, all paths of a frame) */
    uint32_t shade_lanes;      /* RG_BATCH_WAVEFRONT: as rg_tuning.shade_lanes (1-32); 0 = 24 */
    uint32_t reserved;         /* must be 0 */
} rg_batch_tuning;

/* Creates a batch of `n` independent renders (scene, camera, options each,
 * as rg_set_scene/rg_set_camera/rg_set_options take them). */
rg_status rg_batch_create(const rg_device_opts* opts, uint32_t n, const rg_scene_desc* const* scenes,
                          const rg_camera* cameras, const rg_render_opts* options, rg_batch_handle* out);
rg_status rg_batch_destroy(rg_batch_handle b);
rg_status rg_batch_last_error(rg_batch_handle b, char* buf, size_t len);
rg_status rg_batch_set_tuning(rg_batch_handle b, const rg_batch_tuning* t);

/* Adds one frame to every render of the batch. RG_BATCH_WAVEFRONT (default):
 * the paths of all renders fill shared waves of path slots and each bounce is
 * one persistent launch over every render's live paths, warps refilling idle
 * lanes from one queue (work stealing by atomic counter). RG_BATCH_TILES: one
 * persistent launch whose warps take (scene, tile) work items from one global
 * queue. Either way the frame's launch sequence is captured once as a CUDA
 * graph and replayed. Render i uses the frame key splitmix64(seed + i). Waits
 * for the device; stats cover the whole batch. */
rg_status rg_batch_render(rg_batch_handle b, uint64_t seed, rg_render_stats* stats);

/* The same frame as one megakernel launch per render, in sequence (the
 * comparison form). Produces the same images as rg_batch_render. */
rg_status rg_batch_render_sequential(rg_batch_handle b, uint64_t seed, rg_render_stats* stats);

/* Running mean of render `index`, [x][y][rgb], host memory. */
rg_status rg_batch_image(rg_batch_handle b, uint32_t index, float* out_rgb);

/* Frame key rg_batch_render gives render `index` for `seed`. */
uint64_t rg_batch_item_seed(uint64_t seed, uint32_t index);

/* ------------------------------------------------------------------------ */
/* Differentiation (no reference counterpart: the adjoint of render())        */
/* ------------------------------------------------------------------------ */

/* Gradient outputs of rg_backward (host arrays; NULL entries are skipped). */
typedef struct rg_gradients {
    float* albedo;     /* n_materials x 3: d loss / d material albedo (isotropic media included) */
    float* emission;   /* n_materials x 3: d loss / d emissive radiance of light materials */
    float* density;    /* n_volumes: d loss / d VolumetricObject::density (score-function estimator) */
    double loss;       /* with a target: sum over pixels and channels of (I - target)^2; else 0 */
} rg_gradients;

/* Replaces material albedos (emissive radiance for lights), n_materials x 3,
 * and media densities, n_volumes, without rebuilding the BVH. NULL leaves a
 * group unchanged. Clears the accumulation, as set_scene does. */
rg_status rg_set_parameters(rg_handle h, const float* albedo, const float* density);

/* Adjoint of one frame by path-replay backpropagation: the frame `seed`
 * renders image I (mean of `samples` paths per pixel, [x][y][rgb]). With
 * `target_rgb` (host, width*height*3) the loss is sum (I - target)^2, I is
 * rendered on the device and the loss returned; otherwise `adjoint_rgb` (host)
 * is dLoss/dI. Every path is re-traced from its random stream (memory stays
 * O(pixels)); gradients are returned for albedos, emissions and media
 * densities. Supports ray_depth <= 16 and at most 4 media. The accumulation
 * buffer is not touched. */
rg_status rg_backward(rg_handle h, uint64_t seed, const float* adjoint_rgb, const float* target_rgb, rg_gradients* out);

/* rg_backward with a target whose I is the handle's last rendered frame (its
 * per-pixel mean), so the forward frame an optimisation loop renders anyway is
 * not rendered again: the loss is sum (I - target)^2 and frame `seed`'s paths
 * are replayed. With `seed` other than the rendered frame's, the image and
 * the replayed paths are independent samples. RG_NOT_READY unless a PBR frame
 * was rendered since the scene, camera, options, parameters or accumulation
 * last changed. */
rg_status rg_backward_frame(rg_handle h, uint64_t seed, const float* target_rgb, rg_gradients* out);

/* Path slots of the fixed device array used by rg_render_static_scratch
 * (108 bytes each: about 7 MB, held by every device that loads the library). */
#define RG_STATIC_WAVE_PATHS 65536u

/* No counterpart in the reference: the reference renders on the CPU and never
 * allocates device memory.
 *
 * Renders one frame of the handle's current scene, camera and options with the
 * wavefront kernels, without allocating anything. It is for callers that cannot
 * call cudaMalloc: a host that hands out all device memory from its own pool or
 * arena, or a render loop in which allocation is not allowed. The path queues of
 * the frame live in one fixed, library-owned device array of RG_STATIC_WAVE_PATHS
 * path slots instead of cudaMalloc'ed scratch; the frame runs in waves of whole
 * pixels that fit in it.
 *
 * The caller passes the outputs: `d_accum` is a device buffer of width*height*3
 * floats ([x][y][rgb]) holding the running sum, updated in place, and
 * `accum_count` the number of frames in it after this one (>= 1); `d_out`, if not
 * NULL, is a device buffer of the same size that receives the running mean. The
 * scene must already be on the device (rg_set_scene). The image is the same as
 * rg_render's for the same seed.
 *
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture. Every
 * call shares the one array and finds it as the last call left it: calls whose
 * kernels overlap on the GPU (other streams, other handles) race. Samples per
 * pixel above RG_STATIC_WAVE_PATHS are rejected with RG_INVALID_ARG. Returns
 * once the kernels are queued on the handle's stream; rg_sync_stats then
 * reports this frame (device time, samples, launches, counters, error bits and
 * their status). RG_FLAG_STAGE_TIMES is not honoured here (its events are
 * created on demand): traverse_ms reads 0. */
rg_status rg_render_static_scratch(rg_handle h, uint64_t seed, float* d_accum, uint32_t accum_count, float* d_out);

#ifdef __cplusplus
}
#endif

#endif /* RAYNA_GPU_H */
