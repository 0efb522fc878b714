//! omg-scene's late-field seam (crates/omg-scene/src/late.rs:28-101) over
//! libomg_cuda, the GB300 tracer (include/omg_cuda.h).
//!
//! `CudaLateBackend` implements `LateBackend` (late.rs:28-49) with
//! `omg_trace_box`; `CudaWorldLateBackend` implements `WorldLateBackend`
//! (late.rs:81-91) with `omg_trace_world` over the world mesh, uploaded once
//! when the backend is built (the backend owns it, late.rs:75-80). Both are
//! synchronous, as the reference's wgpu backends are (omg-gpu/src/lib.rs:876-880),
//! so `poll_into` keeps its default. A failed call returns `false`: no fresh
//! echogram this tick, the Sim's average holds.
//!
//! Registration, beside crates/omg-app/src/main.rs:207-253:
//!
//! ```ignore
//! if std::env::var("OMG_GPU").as_deref() == Ok("cuda") {
//!     if let Some(b) = omg_cuda::CudaLateBackend::new() {
//!         omg_scene::late::set_late_backend(Box::new(b));
//!         omg_scene::quality::set_gpu_backend(true);
//!     }
//! }
//! ```
//!
//! Source only: there is no Rust toolchain where libomg_cuda is built, so this
//! crate has not been compiled. The same C ABI is exercised from Python
//! (ctypes) by the library's tests and benchmark.

use omg_core::material::Material;
use omg_core::rng::Rng;
use omg_core::scene::Shoebox;
use omg_core::tracer::Echogram;
use omg_core::vec3::Vec3;
use omg_core::NBANDS;
use omg_scene::late::{LateBackend, WorldLateBackend};

const MAXB: usize = 8; // OMG_MAX_BANDS

/// omg_material: per-band absorption, scattering, AMPLITUDE transmission.
#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct OmgMaterial {
    absorption: [f32; MAXB],
    scattering: f32,
    transmission: [f32; MAXB],
}

/// omg_params, field for field.
#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct OmgParams {
    pub n_bands: u32,
    pub n_bins: u32,
    pub bin_dt: f32,
    pub max_time: f32,
    pub max_bounces: u32,
    pub energy_floor: f32,
    pub receiver_radius: f32,
    pub wall_eps: f32,
    pub speed_of_sound: f32,
    pub dir_band: u32,
    pub device: i32,
    pub timeout_ms: u32,
    pub tie_mode: u32,
    pub walk_budget: u32,
    pub loop_guard: u32,
    pub tri_test: u32,
}

#[repr(C)]
struct OmgBoxJob {
    size: [f32; 3],
    walls: [OmgMaterial; 6],
    src: [f32; 3],
    lis: [f32; 3],
    n_rays: u32,
    energy: [f32; MAXB],
    seed: u32,
}

#[repr(C)]
struct OmgWorldJob {
    src: [f32; 3],
    lis: [f32; 3],
    n_rays: u32,
    energy: [f32; MAXB],
    seed: u32,
}

#[repr(C)]
struct OmgPanel {
    mn: [f32; 3],
    mx: [f32; 3],
    material: OmgMaterial,
}

#[repr(C)]
#[derive(Default)]
struct OmgReverb {
    rt60: [f32; MAXB],
    level: [f32; MAXB],
    rt60_fit: [f32; MAXB],
    segments: u64,
}

enum OmgCtx {}
enum OmgMeshBuilder {}

const OMG_BVH_SAH: u32 = 0;

#[link(name = "omg_cuda")]
extern "C" {
    fn omg_abi_version() -> i32;
    fn omg_params_default(p: *mut OmgParams);
    fn omg_create(p: *const OmgParams) -> *mut OmgCtx;
    fn omg_destroy(ctx: *mut OmgCtx);
    fn omg_set_limits(ctx: *mut OmgCtx, walk_budget: u32, loop_guard: u32) -> i32;
    fn omg_trace_box(ctx: *mut OmgCtx, job: *const OmgBoxJob, bins: *mut f32, dirs: *mut f32,
                     reverb: *mut OmgReverb) -> i32;
    fn omg_trace_world(ctx: *mut OmgCtx, scene: u32, job: *const OmgWorldJob, panels: *const OmgPanel,
                       n_panels: u32, bins: *mut f32, dirs: *mut f32, reverb: *mut OmgReverb) -> i32;
    fn omg_mb_create() -> *mut OmgMeshBuilder;
    fn omg_mb_material(mb: *mut OmgMeshBuilder, m: *const OmgMaterial) -> u32;
    fn omg_mb_tri(mb: *mut OmgMeshBuilder, a: *const f32, b: *const f32, c: *const f32, m: u32);
    fn omg_mb_destroy(mb: *mut OmgMeshBuilder);
    fn omg_scene_from_builder(ctx: *mut OmgCtx, mb: *const OmgMeshBuilder, n_bands: u32, bvh: u32,
                              scene: *mut u32) -> i32;
}

/// The ABI version this binding was written against (OMG_ABI_VERSION).
pub const ABI_VERSION: i32 = 3;

fn mat(m: &Material) -> OmgMaterial {
    let mut o = OmgMaterial::default();
    o.absorption[..NBANDS].copy_from_slice(&m.absorption);
    o.scattering = m.scattering;
    o.transmission[..NBANDS].copy_from_slice(&m.transmission);
    o
}

/// The reference's constants (tracer.rs:12-16): Echogram::new()'s bins.
fn params() -> OmgParams {
    let mut p = OmgParams::default();
    unsafe { omg_params_default(&mut p) };
    p
}

/// A context on the default device, or None (no usable device, or a library
/// of another ABI): the caller keeps the CPU tracer (omg-gpu/src/lib.rs:33-37).
fn context() -> Option<*mut OmgCtx> {
    if unsafe { omg_abi_version() } != ABI_VERSION {
        return None;
    }
    let p = params();
    let ctx = unsafe { omg_create(&p) };
    if ctx.is_null() { None } else { Some(ctx) }
}

/// bins[n][NBANDS] then dirs[n][3] (f32, the library's layout) into the
/// caller's Echogram, overwritten whole (tracer.rs:35-42 clears first).
fn fill(out: &mut Echogram, bins: &[f32], dirs: &[f32]) {
    for (i, b) in out.bins.iter_mut().enumerate() {
        b.copy_from_slice(&bins[NBANDS * i..NBANDS * i + NBANDS]);
    }
    for (i, d) in out.dirs.iter_mut().enumerate() {
        d.copy_from_slice(&dirs[3 * i..3 * i + 3]);
    }
}

/// The per-ray stream seed of the next trace: a PCG LCG step, as
/// GpuLateBackend advances its own (omg-gpu/src/lib.rs:1064).
fn next_seed(s: &mut u32) -> u32 {
    *s = s.wrapping_mul(747_796_405).wrapping_add(2_891_336_453);
    *s
}

/// `LateBackend` on the GPU: the analytic shoebox traced by omg_trace_box.
pub struct CudaLateBackend {
    ctx: *mut OmgCtx,
    seed: u32,
    bins: Vec<f32>,
    dirs: Vec<f32>,
}

// The context is used by one thread at a time: the seam's global Mutex
// serializes every call (late.rs:51).
unsafe impl Send for CudaLateBackend {}

impl CudaLateBackend {
    pub fn new() -> Option<Self> {
        let ctx = context()?;
        let n = params().n_bins as usize;
        Some(Self { ctx, seed: 0x0D15_EA5E, bins: vec![0.0; n * NBANDS], dirs: vec![0.0; n * 3] })
    }

    /// Device-side limits (omg_set_limits; 0 = the library's defaults).
    pub fn set_limits(&mut self, walk_budget: u32, loop_guard: u32) -> bool {
        unsafe { omg_set_limits(self.ctx, walk_budget, loop_guard) == 0 }
    }
}

impl Drop for CudaLateBackend {
    fn drop(&mut self) {
        unsafe { omg_destroy(self.ctx) }
    }
}

impl LateBackend for CudaLateBackend {
    fn trace(&mut self, _id: u32, room: &Shoebox, src: Vec3, lis: Vec3, n_rays: u32, energy: [f32; NBANDS],
             _rng: &mut Rng, out: &mut Echogram) -> bool {
        // the GPU draws its own per-ray stream (the reference's GPU backend
        // ignores `rng` the same way)
        let mut e = [0.0f32; MAXB];
        e[..NBANDS].copy_from_slice(&energy);
        let job = OmgBoxJob {
            size: [room.size.x, room.size.y, room.size.z],
            walls: core::array::from_fn(|w| mat(&room.walls[w])),
            src: [src.x, src.y, src.z],
            lis: [lis.x, lis.y, lis.z],
            n_rays,
            energy: e,
            seed: next_seed(&mut self.seed),
        };
        let rc = unsafe {
            omg_trace_box(self.ctx, &job, self.bins.as_mut_ptr(), self.dirs.as_mut_ptr(), core::ptr::null_mut())
        };
        if rc != 0 {
            return false;
        }
        fill(out, &self.bins, &self.dirs);
        true
    }
}

/// `WorldLateBackend` on the GPU: the world mesh, uploaded once with the
/// reference's own tree (OMG_BVH_SAH: with tie_mode 0 every exact tie
/// resolves as Mesh::raycast does), traced with the call's panel overlays.
pub struct CudaWorldLateBackend {
    ctx: *mut OmgCtx,
    scene: u32,
    seed: u32,
    bins: Vec<f32>,
    dirs: Vec<f32>,
}

unsafe impl Send for CudaWorldLateBackend {}

impl CudaWorldLateBackend {
    pub fn new(mesh: &omg_core::mesh::Mesh) -> Option<Self> {
        let ctx = context()?;
        let mb = unsafe { omg_mb_create() };
        for m in &mesh.materials {
            unsafe { omg_mb_material(mb, &mat(m)) };
        }
        for (t, idx) in mesh.indices.iter().enumerate() {
            let v = |i: u32| {
                let p = mesh.positions[i as usize];
                [p.x, p.y, p.z]
            };
            let (a, b, c) = (v(idx[0]), v(idx[1]), v(idx[2]));
            unsafe { omg_mb_tri(mb, a.as_ptr(), b.as_ptr(), c.as_ptr(), mesh.tri_material[t] as u32) };
        }
        let mut scene = 0u32;
        let rc = unsafe { omg_scene_from_builder(ctx, mb, NBANDS as u32, OMG_BVH_SAH, &mut scene) };
        unsafe { omg_mb_destroy(mb) };
        if rc != 0 {
            unsafe { omg_destroy(ctx) };
            return None;
        }
        let n = params().n_bins as usize;
        Some(Self { ctx, scene, seed: 0x5EED_C6D1, bins: vec![0.0; n * NBANDS], dirs: vec![0.0; n * 3] })
    }
}

impl Drop for CudaWorldLateBackend {
    fn drop(&mut self) {
        unsafe { omg_destroy(self.ctx) }
    }
}

impl WorldLateBackend for CudaWorldLateBackend {
    fn trace_world(&mut self, _id: u32, src: Vec3, lis: Vec3, rays: u32, panels: &[(Vec3, Vec3, Material)],
                   out: &mut Echogram) -> bool {
        // `rays` is the CPU budget; a GPU backend may multiply it (late.rs:76-80):
        // x8, capped at 8192, as the reference's GpuWorldLateBackend does
        let n_rays = rays.saturating_mul(8).min(8192);
        let pan: Vec<OmgPanel> = panels
            .iter()
            .map(|(mn, mx, m)| OmgPanel { mn: [mn.x, mn.y, mn.z], mx: [mx.x, mx.y, mx.z], material: mat(m) })
            .collect();
        let mut e = [0.0f32; MAXB];
        e[..NBANDS].copy_from_slice(&[1.0; NBANDS]);
        let job = OmgWorldJob {
            src: [src.x, src.y, src.z],
            lis: [lis.x, lis.y, lis.z],
            n_rays,
            energy: e,
            seed: next_seed(&mut self.seed),
        };
        let rc = unsafe {
            omg_trace_world(self.ctx, self.scene, &job, pan.as_ptr(), pan.len() as u32, self.bins.as_mut_ptr(),
                            self.dirs.as_mut_ptr(), core::ptr::null_mut())
        };
        if rc != 0 {
            return false;
        }
        fill(out, &self.bins, &self.dirs);
        true
    }
}
