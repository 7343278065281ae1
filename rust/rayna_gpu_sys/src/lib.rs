//! Raw bindings of `include/rayna_gpu.h` (C ABI version 8). Not compiled here:
//! this image has no Rust toolchain. Layouts follow the header field for
//! field; every function returns an `rg_status` (0 = `RG_OK`).
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_void};

pub const RG_ABI_VERSION: u32 = 8;

pub type rg_status = i32;
pub const RG_OK: rg_status = 0;
pub const RG_INVALID_ARG: rg_status = 1;
pub const RG_UNSUPPORTED_VARIANT: rg_status = 2;
pub const RG_INVALID_CAMERA: rg_status = 3;
pub const RG_OOM: rg_status = 4;
pub const RG_CUDA_ERROR: rg_status = 5;
pub const RG_QUEUE_OVERFLOW: rg_status = 6;
pub const RG_STEP_LIMIT: rg_status = 7;
pub const RG_TIMEOUT: rg_status = 8;
pub const RG_NO_DEVICE: rg_status = 9;
pub const RG_NOT_READY: rg_status = 10;

pub const RG_MAT_LAMBERTIAN: u32 = 0;
pub const RG_MAT_METAL: u32 = 1;
pub const RG_MAT_DIELECTRIC: u32 = 2;
pub const RG_MAT_ISOTROPIC: u32 = 3;
pub const RG_MAT_LIGHT: u32 = 4;

pub const RG_TEX_SOLID: u32 = 0;
pub const RG_TEX_WORLD_CHECKER: u32 = 1;
pub const RG_TEX_UV_CHECKER: u32 = 2;
pub const RG_TEX_IMAGE: u32 = 3;
pub const RG_TEX_NOISE: u32 = 4;
pub const RG_NOISE_WORLD: u32 = 0;
pub const RG_NOISE_LOCAL: u32 = 1;
pub const RG_NOISE_UV: u32 = 2;
pub const RG_MAX_TEXTURE_DEPTH: u32 = 16;

pub const RG_SKY_SIMPLE: u32 = 0;
pub const RG_SKY_WHITE: u32 = 1;
pub const RG_SKY_NONE: u32 = 2;
pub const RG_SKY_IMAGE: u32 = 3;

pub const RG_BOUNDARY_SPHERE: u32 = 0;
pub const RG_BOUNDARY_BOX: u32 = 1;
pub const RG_SDF_SPHERE: u32 = 0;
pub const RG_SDF_TORUS: u32 = 1;
pub const RG_SDF_MANDELBULB: u32 = 2;
pub const RG_NO_TRANSFORM: u32 = 0xFFFF_FFFF;
pub const RG_UV_WRAP: u32 = 0;
pub const RG_UV_MIRROR: u32 = 1;
pub const RG_UV_CLAMP_ZERO: u32 = 2;

pub const RG_MODE_PBR: u32 = 0;
pub const RG_MODE_RAY_NORMAL: u32 = 1;
pub const RG_MODE_OUTWARD_NORMAL: u32 = 2;
pub const RG_MODE_SCATTER: u32 = 3;
pub const RG_MODE_FRONT_FACE: u32 = 4;
pub const RG_MODE_DISTANCE: u32 = 5;
pub const RG_MODE_UV: u32 = 6;
pub const RG_MODE_SIDE: u32 = 7;

pub const RG_FORM_MEGAKERNEL: u32 = 0;
pub const RG_FORM_WAVEFRONT: u32 = 1;
pub const RG_FLAG_COUNTERS: u32 = 1;
pub const RG_FLAG_STAGE_TIMES: u32 = 2;
pub const RG_FLAG_VALIDATE: u32 = 4;

pub const RG_DEVICE_STACK_OVERFLOW: u32 = 1;
pub const RG_DEVICE_BAD_INDEX: u32 = 2;
pub const RG_DEVICE_QUEUE_OVERFLOW: u32 = 4;
pub const RG_INVALID_NONFINITE: u32 = 1;
pub const RG_INVALID_NOT_NORMALISED: u32 = 2;
pub const RG_INVALID_INTERVAL: u32 = 4;
pub const RG_INVALID_POSITION: u32 = 8;
pub const RG_INVALID_UV: u32 = 16;
pub const RG_INVALID_COLOUR: u32 = 32;

pub const RG_SHARED_STACK_NONE: u32 = 0xFFFF_FFFF;
pub const RG_BATCH_WAVEFRONT: u32 = 0;
pub const RG_BATCH_TILES: u32 = 1;
pub const RG_STATIC_WAVE_PATHS: u32 = 65536;

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rg_material {
    pub kind: u32,
    pub albedo: [f32; 3],
    pub fuzz: f32,
    pub refractive_index: f32,
    pub density: f32,
    pub texture: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rg_texture {
    pub kind: u32,
    pub odd: u32,
    pub even: u32,
    pub image: u32,
    pub scale: [f32; 2],
    pub offset: [f32; 3],
    pub colour: [f32; 3],
    pub noise_seed: u32,
    pub noise_place: u32,
    pub noise_channels: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct rg_image {
    pub width: u32,
    pub height: u32,
    pub rgb: *const f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rg_volume {
    pub boundary: u32,
    pub a: [f32; 3],
    pub b: [f32; 3],
    pub density: f32,
    pub material: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rg_sdf {
    pub kind: u32,
    pub centre: [f32; 3],
    pub params: [f32; 4],
    pub max_iterations: u32,
    pub epsilon: f32,
    pub material: u32,
}

/// A flattened scene; arrays are borrowed for the duration of `rg_set_scene`.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct rg_scene_desc {
    pub n_spheres: u32,
    pub spheres: *const f32,
    pub sphere_material: *const u32,
    pub n_triangles: u32,
    pub tri_vertices: *const f32,
    pub tri_normals: *const f32,
    pub tri_material: *const u32,
    pub tri_mesh: *const i32,
    pub n_boxes: u32,
    pub boxes: *const f32,
    pub box_material: *const u32,
    pub n_volumes: u32,
    pub volumes: *const rg_volume,
    pub n_sdfs: u32,
    pub sdfs: *const rg_sdf,
    pub n_materials: u32,
    pub materials: *const rg_material,
    pub skybox: u32,
    pub n_quads: u32,
    pub quads: *const f32,
    pub quad_material: *const u32,
    pub n_cylinders: u32,
    pub cylinders: *const f32,
    pub cylinder_material: *const u32,
    pub n_planes: u32,
    pub planes: *const f32,
    pub plane_material: *const u32,
    pub plane_uv_wrap: *const u32,
    pub n_transforms: u32,
    pub transforms: *const f64,
    pub sphere_transform: *const u32,
    pub tri_transform: *const u32,
    pub box_transform: *const u32,
    pub quad_transform: *const u32,
    pub cylinder_transform: *const u32,
    pub n_textures: u32,
    pub textures: *const rg_texture,
    pub n_images: u32,
    pub images: *const rg_image,
    pub sky_image: u32,
    pub volume_transform: *const u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rg_camera {
    pub pos: [f64; 3],
    pub fwd: [f64; 3],
    pub v_fov: f64,
    pub focus_dist: f64,
    pub defocus_angle: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rg_render_opts {
    pub width: u32,
    pub height: u32,
    pub samples: u32,
    pub mode: u32,
    pub ray_depth: u32,
    pub ray_branching: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct rg_device_opts {
    pub device: i32,
    pub stream: *mut c_void,
    pub form: u32,
    pub flags: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rg_render_stats {
    pub duration_ms: f64,
    pub kernel_ms: f64,
    pub samples: u64,
    pub rays: u64,
    pub node_visits: u64,
    pub prim_tests: u64,
    pub sdf_steps: u64,
    pub accum_frames: u32,
    pub img_width: u32,
    pub img_height: u32,
    pub num_threads: u32,
    pub error_flags: u32,
    pub kernel_launches: u32,
    pub traverse_ms: f64,
    pub invalid_hits: u64,
    pub invalid_mask: u32,
    pub reserved0: u32,
    pub hits: u64,
    pub sdf_iterations: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rg_hit {
    pub hit: u32,
    pub prim: u32,
    pub t: f32,
    pub normal: [f32; 3],
    pub ray_normal: [f32; 3],
    pub front_face: u32,
    pub material: u32,
    pub side: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rg_scene_info {
    pub n_prims: u32,
    pub n_unbounded: u32,
    pub n_nodes: u32,
    pub max_depth: u32,
    pub n_leaves: u32,
    pub max_leaf_size: u32,
    pub sah_cost: f64,
    pub device_bytes: u64,
    pub n_wide_nodes: u32,
    pub wide_depth: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rg_tuning {
    pub wave_paths: u32,
    pub sort_materials: u32,
    pub bvh_width: u32,
    pub fetch_budget: u32,
    pub shared_stack: u32,
    pub block: u32,
    pub stack_limit: u32,
    pub march_budget: u32,
    pub shade_lanes: u32,
    pub tail_paths: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rg_batch_tuning {
    pub block: u32,
    pub blocks_per_sm: u32,
    pub rounds_per_item: u32,
    pub bvh_width: u32,
    pub form: u32,
    pub wave_paths: u32,
    pub shade_lanes: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct rg_gradients {
    pub albedo: *mut f32,
    pub emission: *mut f32,
    pub density: *mut f32,
    pub loss: f64,
}

pub enum rg_renderer {}
pub type rg_handle = *mut rg_renderer;
pub enum rg_batch {}
pub type rg_batch_handle = *mut rg_batch;

extern "C" {
    pub fn rg_abi_version() -> u32;
    pub fn rg_create(opts: *const rg_device_opts, out: *mut rg_handle) -> rg_status;
    pub fn rg_destroy(h: rg_handle) -> rg_status;
    pub fn rg_last_error(h: rg_handle, buf: *mut c_char, len: usize) -> rg_status;
    pub fn rg_inspect_scene(scene: *const rg_scene_desc, out: *mut rg_scene_info) -> rg_status;
    pub fn rg_set_scene(h: rg_handle, scene: *const rg_scene_desc) -> rg_status;
    pub fn rg_set_tuning(h: rg_handle, t: *const rg_tuning) -> rg_status;
    pub fn rg_get_tuning(h: rg_handle, out: *mut rg_tuning) -> rg_status;
    pub fn rg_set_camera(h: rg_handle, camera: *const rg_camera) -> rg_status;
    pub fn rg_set_options(h: rg_handle, opts: *const rg_render_opts) -> rg_status;
    pub fn rg_clear_accumulation(h: rg_handle) -> rg_status;
    pub fn rg_render(h: rg_handle, seed: u64, out_rgb: *mut f32, stats: *mut rg_render_stats) -> rg_status;
    pub fn rg_render_async(h: rg_handle, seed: u64, d_out_rgb: *mut f32, stats: *mut rg_render_stats) -> rg_status;
    pub fn rg_sync_stats(h: rg_handle, stats: *mut rg_render_stats) -> rg_status;
    pub fn rg_set_sample_range(h: rg_handle, first: u32, count: u32) -> rg_status;
    pub fn rg_get_accumulation(h: rg_handle, sum: *mut f32, frames: *mut u32) -> rg_status;
    pub fn rg_set_accumulation(h: rg_handle, sum: *const f32, frames: u32) -> rg_status;
    pub fn rg_frame_moments(h: rg_handle, mean: *mut f32, variance: *mut f32) -> rg_status;
    pub fn rg_query_rays(h: rg_handle, n: u32, origins: *const f32, dirs: *const f32, tmin: *const f32,
                         tmax: *const f32, volume_u: *const f32, out: *mut rg_hit) -> rg_status;
    pub fn rg_batch_create(opts: *const rg_device_opts, n: u32, scenes: *const *const rg_scene_desc,
                           cameras: *const rg_camera, options: *const rg_render_opts, out: *mut rg_batch_handle)
                           -> rg_status;
    pub fn rg_batch_destroy(b: rg_batch_handle) -> rg_status;
    pub fn rg_batch_last_error(b: rg_batch_handle, buf: *mut c_char, len: usize) -> rg_status;
    pub fn rg_batch_set_tuning(b: rg_batch_handle, t: *const rg_batch_tuning) -> rg_status;
    pub fn rg_batch_render(b: rg_batch_handle, seed: u64, stats: *mut rg_render_stats) -> rg_status;
    pub fn rg_batch_render_sequential(b: rg_batch_handle, seed: u64, stats: *mut rg_render_stats) -> rg_status;
    pub fn rg_batch_image(b: rg_batch_handle, index: u32, out_rgb: *mut f32) -> rg_status;
    pub fn rg_batch_item_seed(seed: u64, index: u32) -> u64;
    pub fn rg_set_parameters(h: rg_handle, albedo: *const f32, density: *const f32) -> rg_status;
    pub fn rg_backward(h: rg_handle, seed: u64, adjoint_rgb: *const f32, target_rgb: *const f32,
                       out: *mut rg_gradients) -> rg_status;
    pub fn rg_backward_frame(h: rg_handle, seed: u64, target_rgb: *const f32, out: *mut rg_gradients) -> rg_status;
    pub fn rg_render_static_scratch(h: rg_handle, seed: u64, d_accum: *mut f32, accum_count: u32, d_out: *mut f32)
                                    -> rg_status;
}
