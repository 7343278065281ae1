//! `GpuRenderer`: the methods of rayna_engine's `Renderer<Obj, Sky, Rng>`
//! (render/renderer.rs:38-183) over the C ABI of `rayna_gpu_sys`. Not
//! compiled here: this image has no Rust toolchain.
//!
//! The scene crosses the ABI flattened (`SceneDesc`, owned arrays); building
//! one from a `StandardScene` follows the mapping of INTEGRATION.md (the one
//! `rayna_gb300/scene.py:flatten` implements): spheres, triangles of meshes,
//! boxes, media, SDF descriptors, parallelograms, cylinders, infinite planes,
//! the material and texture tables, the sky, and per-object transforms.
use rayna_gpu_sys as sys;
use std::ffi::CStr;
use std::fmt;

/// A non-zero `rg_status` with the library's message.
#[derive(Debug, Clone)]
pub struct GpuError {
    pub status: i32,
    pub message: String,
}

impl fmt::Display for GpuError {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "rg_status {}: {}", self.status, self.message)
    }
}

impl std::error::Error for GpuError {}

fn last_error(h: sys::rg_handle) -> String {
    let mut buf = [0 as std::os::raw::c_char; 1024];
    unsafe {
        sys::rg_last_error(h, buf.as_mut_ptr(), buf.len());
        CStr::from_ptr(buf.as_ptr()).to_string_lossy().into_owned()
    }
}

fn check(h: sys::rg_handle, status: i32) -> Result<(), GpuError> {
    if status == sys::RG_OK {
        Ok(())
    } else {
        Err(GpuError { status, message: last_error(h) })
    }
}

/// A flattened scene with owned arrays (rg_scene_desc's layout, one Vec per array).
#[derive(Default, Clone, Debug)]
pub struct SceneDesc {
    pub spheres: Vec<[f32; 4]>,
    pub sphere_material: Vec<u32>,
    pub tri_vertices: Vec<[[f32; 3]; 3]>,
    pub tri_normals: Vec<[[f32; 3]; 3]>,
    pub tri_material: Vec<u32>,
    pub tri_mesh: Vec<i32>,
    pub boxes: Vec<[f32; 6]>,
    pub box_material: Vec<u32>,
    pub volumes: Vec<sys::rg_volume>,
    pub sdfs: Vec<sys::rg_sdf>,
    pub materials: Vec<sys::rg_material>,
    pub skybox: u32,
    pub quads: Vec<[f32; 9]>,
    pub quad_material: Vec<u32>,
    pub cylinders: Vec<[f32; 7]>,
    pub cylinder_material: Vec<u32>,
    pub planes: Vec<[f32; 9]>,
    pub plane_material: Vec<u32>,
    pub plane_uv_wrap: Vec<u32>,
    pub transforms: Vec<[f64; 12]>,
    pub sphere_transform: Vec<u32>,
    pub tri_transform: Vec<u32>,
    pub box_transform: Vec<u32>,
    pub quad_transform: Vec<u32>,
    pub cylinder_transform: Vec<u32>,
    pub volume_transform: Vec<u32>,
    pub textures: Vec<sys::rg_texture>,
    /// (width, height, [x][y][rgb] texels)
    pub images: Vec<(u32, u32, Vec<f32>)>,
    pub sky_image: u32,
}

fn ptr_or_null<T>(v: &[T]) -> *const T {
    if v.is_empty() { std::ptr::null() } else { v.as_ptr() }
}

impl SceneDesc {
    /// The C descriptor borrowing this scene's arrays (valid while `self` and `images` live).
    fn desc(&self, images: &[sys::rg_image]) -> sys::rg_scene_desc {
        sys::rg_scene_desc {
            n_spheres: self.spheres.len() as u32,
            spheres: ptr_or_null(&self.spheres) as *const f32,
            sphere_material: ptr_or_null(&self.sphere_material),
            n_triangles: self.tri_vertices.len() as u32,
            tri_vertices: ptr_or_null(&self.tri_vertices) as *const f32,
            tri_normals: ptr_or_null(&self.tri_normals) as *const f32,
            tri_material: ptr_or_null(&self.tri_material),
            tri_mesh: ptr_or_null(&self.tri_mesh),
            n_boxes: self.boxes.len() as u32,
            boxes: ptr_or_null(&self.boxes) as *const f32,
            box_material: ptr_or_null(&self.box_material),
            n_volumes: self.volumes.len() as u32,
            volumes: ptr_or_null(&self.volumes),
            n_sdfs: self.sdfs.len() as u32,
            sdfs: ptr_or_null(&self.sdfs),
            n_materials: self.materials.len() as u32,
            materials: ptr_or_null(&self.materials),
            skybox: self.skybox,
            n_quads: self.quads.len() as u32,
            quads: ptr_or_null(&self.quads) as *const f32,
            quad_material: ptr_or_null(&self.quad_material),
            n_cylinders: self.cylinders.len() as u32,
            cylinders: ptr_or_null(&self.cylinders) as *const f32,
            cylinder_material: ptr_or_null(&self.cylinder_material),
            n_planes: self.planes.len() as u32,
            planes: ptr_or_null(&self.planes) as *const f32,
            plane_material: ptr_or_null(&self.plane_material),
            plane_uv_wrap: ptr_or_null(&self.plane_uv_wrap),
            n_transforms: self.transforms.len() as u32,
            transforms: ptr_or_null(&self.transforms) as *const f64,
            sphere_transform: ptr_or_null(&self.sphere_transform),
            tri_transform: ptr_or_null(&self.tri_transform),
            box_transform: ptr_or_null(&self.box_transform),
            quad_transform: ptr_or_null(&self.quad_transform),
            cylinder_transform: ptr_or_null(&self.cylinder_transform),
            n_textures: self.textures.len() as u32,
            textures: ptr_or_null(&self.textures),
            n_images: images.len() as u32,
            images: ptr_or_null(images),
            sky_image: self.sky_image,
            volume_transform: ptr_or_null(&self.volume_transform),
        }
    }
}

/// RenderOpts (render/render_opts.rs:8-29).
#[derive(Clone, Copy, Debug)]
pub struct RenderOpts {
    pub width: u32,
    pub height: u32,
    pub samples: u32,
    pub mode: u32,
    pub ray_depth: u32,
    pub ray_branching: u32,
}

impl Default for RenderOpts {
    fn default() -> Self {
        RenderOpts { width: 740, height: 480, samples: 1, mode: sys::RG_MODE_PBR, ray_depth: 5, ray_branching: 1 }
    }
}

/// An image of (width, height) RGB pixels stored [x][y][rgb], the memory
/// order of rayna_engine's `Image` (core/image.rs:24-25).
pub struct Image {
    pub width: u32,
    pub height: u32,
    pub rgb: Vec<f32>,
}

/// Render (render/render.rs): the image and its statistics.
pub struct Render {
    pub img: Image,
    pub stats: sys::rg_render_stats,
    /// RG_INVALID_CAMERA: `img` is the reference's ilog2-sized checker (renderer.rs:269-292)
    pub camera_invalid: bool,
}

fn splitmix64(mut z: u64) -> u64 {
    z = z.wrapping_add(0x9E37_79B9_7F4A_7C15);
    z = (z ^ (z >> 30)).wrapping_mul(0xBF58_476D_1CE4_E5B9);
    z = (z ^ (z >> 27)).wrapping_mul(0x94D0_49BB_1331_11EB);
    z ^ (z >> 31)
}

/// The GPU stand-in for `Renderer`: owns one handle (a CUDA stream and the
/// scene's device buffers). `&mut self` serialises calls, as in the reference.
pub struct GpuRenderer {
    h: sys::rg_handle,
    opts: RenderOpts,
    seed: u64,
    frame: u64,
}

unsafe impl Send for GpuRenderer {}

impl GpuRenderer {
    /// Renderer::new_from (renderer.rs:86-107). `wavefront`: the persistent
    /// wavefront kernels (the fast form) instead of the plain megakernel.
    pub fn new_from(scene: &SceneDesc, camera: sys::rg_camera, options: RenderOpts, device: i32, wavefront: bool)
                    -> Result<Self, GpuError> {
        let opts = sys::rg_device_opts {
            device,
            stream: std::ptr::null_mut(),
            form: if wavefront { sys::RG_FORM_WAVEFRONT } else { sys::RG_FORM_MEGAKERNEL },
            flags: if cfg!(debug_assertions) { sys::RG_FLAG_VALIDATE } else { 0 },
        };
        let mut h: sys::rg_handle = std::ptr::null_mut();
        check(std::ptr::null_mut(), unsafe { sys::rg_create(&opts, &mut h) })?;
        let mut r = GpuRenderer { h, opts: options, seed: 0, frame: 0 };
        r.set_scene(scene)?;
        r.set_camera(camera)?;
        r.set_options(options)?;
        Ok(r)
    }

    /// Renderer::set_scene (renderer.rs:165-168): clears the accumulation.
    pub fn set_scene(&mut self, scene: &SceneDesc) -> Result<(), GpuError> {
        let images: Vec<sys::rg_image> =
            scene.images.iter().map(|(w, h, px)| sys::rg_image { width: *w, height: *h, rgb: px.as_ptr() }).collect();
        let desc = scene.desc(&images);
        check(self.h, unsafe { sys::rg_set_scene(self.h, &desc) })
    }

    /// Renderer::set_camera (renderer.rs:158-161): clears the accumulation.
    pub fn set_camera(&mut self, camera: sys::rg_camera) -> Result<(), GpuError> {
        check(self.h, unsafe { sys::rg_set_camera(self.h, &camera) })
    }

    /// Renderer::set_options (renderer.rs:173-176): clears the accumulation.
    pub fn set_options(&mut self, options: RenderOpts) -> Result<(), GpuError> {
        let o = sys::rg_render_opts {
            width: options.width,
            height: options.height,
            samples: options.samples,
            mode: options.mode,
            ray_depth: options.ray_depth,
            ray_branching: options.ray_branching,
        };
        check(self.h, unsafe { sys::rg_set_options(self.h, &o) })?;
        self.opts = options;
        Ok(())
    }

    /// Renderer::clear_accumulation (renderer.rs:153).
    pub fn clear_accumulation(&mut self) -> Result<(), GpuError> {
        check(self.h, unsafe { sys::rg_clear_accumulation(self.h) })
    }

    /// Renderer::set_thread_count (renderer.rs:179-182): the device decides its own parallelism.
    pub fn set_thread_count(&mut self, _num_threads: usize) {}

    pub fn options(&self) -> RenderOpts {
        self.opts
    }

    /// Renderer::render (renderer.rs:224-264): one progressive frame, the
    /// running mean of every frame so far. An invalid camera gives the
    /// reference's checker image, as the reference does.
    pub fn render(&mut self) -> Result<Render, GpuError> {
        let (w, h) = (self.opts.width, self.opts.height);
        let mut rgb = vec![0f32; w as usize * h as usize * 3];
        let mut stats = sys::rg_render_stats::default();
        let key = splitmix64(self.seed.wrapping_add(0x9E37_79B9_7F4A_7C15u64.wrapping_mul(self.frame + 1)));
        self.frame += 1;
        let st = unsafe { sys::rg_render(self.h, key, rgb.as_mut_ptr(), &mut stats) };
        if st == sys::RG_INVALID_CAMERA {
            let (cw, ch) = (stats.img_width, stats.img_height);
            rgb.truncate(cw as usize * ch as usize * 3);
            return Ok(Render { img: Image { width: cw, height: ch, rgb }, stats, camera_invalid: true });
        }
        check(self.h, st)?;
        if cfg!(debug_assertions) {
            // the reference's debug invariants (shared/validate.rs), counted on the device
            debug_assert_eq!(stats.invalid_hits, 0, "broken invariants: mask {:#x}", stats.invalid_mask);
        }
        Ok(Render { img: Image { width: w, height: h, rgb }, stats, camera_invalid: false })
    }

    /// Shares one frame across devices: this renderer traces samples
    /// [first, first + count) of every pixel (rg_set_sample_range); the
    /// element-wise sum of the shards' accumulation sums is the whole frames'.
    pub fn set_sample_range(&mut self, first: u32, count: u32) -> Result<(), GpuError> {
        check(self.h, unsafe { sys::rg_set_sample_range(self.h, first, count) })
    }

    /// The accumulation buffer's sums ([x][y][rgb]) and frame count.
    pub fn accumulation(&self) -> Result<(Vec<f32>, u32), GpuError> {
        let mut sum = vec![0f32; self.opts.width as usize * self.opts.height as usize * 3];
        let mut frames = 0u32;
        check(self.h, unsafe { sys::rg_get_accumulation(self.h, sum.as_mut_ptr(), &mut frames) })?;
        Ok((sum, frames))
    }
}

impl Drop for GpuRenderer {
    fn drop(&mut self) {
        unsafe {
            sys::rg_destroy(self.h);
        }
    }
}
