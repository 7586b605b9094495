//! Rust side of the woxel_gb300 C ABI (include/woxel_gb300.h).
//!
//! NOT COMPILED IN THIS ENVIRONMENT: there is no Rust toolchain here. This is
//! the module a woxel maintainer would add (e.g. as `src/render/gb300.rs`) to
//! replace the wgpu compute pass (src/render/wgpu_context.rs:243-282) and the
//! atlas/mask upload (src/render/wgpu_context.rs:101-159) with calls into
//! libwoxel_gb300.so. Link with `cargo:rustc-link-lib=dylib=woxel_gb300`.

#![allow(non_camel_case_types)]

use std::ffi::{c_void, CStr};
use std::os::raw::{c_char, c_int};

use crate::render::gpu_types::ComputeState;
use crate::vdb::VDB345;

pub const WX_OK: c_int = 0;
pub const WX_ERR_INVALID: c_int = 1;
pub const WX_ERR_CUDA: c_int = 2;
pub const WX_ERR_OOM: c_int = 3;
pub const WX_ERR_UNSUPPORTED: c_int = 4;
pub const WX_ERR_BUDGET: c_int = 5;
pub const WX_ERR_TIMEOUT: c_int = 6;
pub const WX_ERR_CANCELLED: c_int = 7;
pub const WX_SERVE_FIFO: u32 = 1;

#[repr(C)]
pub struct wx_ctx {
    _private: [u8; 0],
}
#[repr(C)]
pub struct wx_grid {
    _private: [u8; 0],
}
#[repr(C)]
pub struct wx_batch {
    _private: [u8; 0],
}
#[repr(C)]
pub struct wx_topology {
    _private: [u8; 0],
}
#[repr(C)]
pub struct wx_server {
    _private: [u8; 0],
}

/// Same bytes as `ComputeState` (src/render/gpu_types/compute_state.rs:9-29).
pub type wx_state_uniform = ComputeState;

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct wx_hit {
    pub p: [f32; 3],
    pub t: f32,
    pub node: u32,
    pub info: u32,
    pub shadow: u32,
    pub reserved: u32,
}

#[repr(C)]
pub struct wx_vdb345_view {
    pub kids5: *const u32,
    pub vals5: *const u32,
    pub kids4: *const u32,
    pub vals4: *const u32,
    pub vals3: *const u32,
    pub origins: *const i32,
    pub n5: u64,
    pub n4: u64,
    pub n3: u64,
    pub origin_stride: u32,
    pub atlas: [*const u32; 3],
    pub dims: [[u32; 3]; 3],
}

#[repr(C)]
pub struct wx_frame {
    pub grid: *const wx_grid,
    pub state: wx_state_uniform,
    pub width: u32,
    pub height: u32,
    pub rgba8: *mut u8,
    pub hits: *mut wx_hit,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct wx_grid_info {
    pub n5: u64,
    pub n4: u64,
    pub n3: u64,
    pub device_bytes: u64,
    pub active_voxels: u64,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct wx_tuning {
    pub kernel: i32,
    pub warps_per_block: i32,
    pub blocks_per_sm: i32,
    pub tile_width: i32,
    pub tile_order: i32,
    pub rays_per_lane: i32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct wx_server_config {
    pub budget_bytes: u64,
    pub max_inflight: u32,
    pub slice_tiles: u32,
    pub max_frames: u32,
    pub flags: u32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct wx_request {
    pub grid_id: u32,
    pub want_hits: u32,
    pub width: u32,
    pub height: u32,
    pub state: wx_state_uniform,
    pub user: u64,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct wx_result {
    pub ticket: u64,
    pub user: u64,
    pub status: i32,
    pub width: u32,
    pub height: u32,
    pub rgba8: *const u8,
    pub hits: *const wx_hit,
    pub t_submit: f64,
    pub t_admit: f64,
    pub t_done: f64,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct wx_server_stats {
    pub submitted: u64,
    pub completed: u64,
    pub cancelled: u64,
    pub launches: u64,
    pub rays_done: u64,
    pub arena_bytes: u64,
    pub arena_in_use: u64,
    pub arena_peak: u64,
    pub pending: u64,
    pub active: u64,
    pub tiles_cancelled_queued: u64,
    pub tiles_cancelled_launched: u64,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct wx_vdb_info {
    pub file_version: u32,
    pub compression: u32,
    pub half_float: u32,
    pub reserved: u32,
    pub file_voxel_count: i64,
    pub grid_name: [c_char; 64],
}

// Every entry point of include/woxel_gb300.h, in its order there.
extern "C" {
    pub fn wx_status_string(status: c_int) -> *const c_char;
    pub fn wx_thread_last_error() -> *const c_char;
    pub fn wx_version() -> *const c_char;
    pub fn wx_ctx_create(device: c_int, out: *mut *mut wx_ctx) -> c_int;
    pub fn wx_ctx_destroy(ctx: *mut wx_ctx) -> c_int;
    pub fn wx_last_error(ctx: *const wx_ctx) -> *const c_char;
    pub fn wx_grid_upload(ctx: *mut wx_ctx, view: *const wx_vdb345_view, out: *mut *mut wx_grid) -> c_int;
    pub fn wx_grid_build(ctx: *mut wx_ctx, topo: *mut wx_topology, out: *mut *mut wx_grid) -> c_int;
    pub fn wx_grid_build_gpu(ctx: *mut wx_ctx, topo: *const wx_topology, out: *mut *mut wx_grid) -> c_int;
    pub fn wx_ctx_set_sdf_wait_limit(ctx: *mut wx_ctx, polls: u32) -> c_int;
    pub fn wx_inject_alloc_failures(count: u32) -> c_int;
    pub fn wx_grid_release(ctx: *mut wx_ctx, grid: *mut wx_grid) -> c_int;
    pub fn wx_grid_set_values(ctx: *mut wx_ctx, grid: *mut wx_grid, values: *const f32, band: f32) -> c_int;
    pub fn wx_grid_get_info(grid: *const wx_grid, out: *mut wx_grid_info) -> c_int;
    pub fn wx_grid_read_pools(ctx: *mut wx_ctx, grid: *const wx_grid, slot5: *mut u32, slot4: *mut u32, leaf: *mut u8, ovf: *mut u32, n_ovf: *mut u64) -> c_int;
    pub fn wx_render(ctx: *mut wx_ctx, grid: *const wx_grid, state: *const wx_state_uniform, width: u32, height: u32, rgba8: *mut u8, hits: *mut wx_hit, stream: *mut c_void) -> c_int;
    pub fn wx_ctx_set_tuning(ctx: *mut wx_ctx, tuning: *const wx_tuning) -> c_int;
    pub fn wx_ctx_get_tuning(ctx: *const wx_ctx, tuning: *mut wx_tuning) -> c_int;
    pub fn wx_autotune(ctx: *mut wx_ctx, frames: *const wx_frame, n: u32, candidates: *const wx_tuning, ncand: u32, reps: u32, best: *mut wx_tuning, times_ms: *mut f64) -> c_int;
    pub fn wx_render_batch(ctx: *mut wx_ctx, frames: *const wx_frame, n: u32, stream: *mut c_void) -> c_int;
    pub fn wx_batch_create(ctx: *mut wx_ctx, frames: *const wx_frame, n: u32, out: *mut *mut wx_batch) -> c_int;
    pub fn wx_batch_launch(batch: *mut wx_batch, stream: *mut c_void) -> c_int;
    pub fn wx_batch_info(batch: *const wx_batch, frames: *mut u32, tiles: *mut u32, rays: *mut u64) -> c_int;
    pub fn wx_batch_destroy(batch: *mut wx_batch) -> c_int;
    pub fn wx_render_batch_noalloc(frames: *const wx_frame, n: u32, stream: *mut c_void) -> c_int;
    pub fn wx_server_create(ctx: *mut wx_ctx, cfg: *const wx_server_config, out: *mut *mut wx_server) -> c_int;
    pub fn wx_server_add_grid(srv: *mut wx_server, grid: *const wx_grid, grid_id: *mut u32) -> c_int;
    pub fn wx_server_submit(srv: *mut wx_server, req: *const wx_request, ticket: *mut u64) -> c_int;
    pub fn wx_server_cancel(srv: *mut wx_server, ticket: u64) -> c_int;
    pub fn wx_server_poll(srv: *mut wx_server, out: *mut wx_result, max: u32, n: *mut u32, wait_ms: c_int) -> c_int;
    pub fn wx_server_copy_result(srv: *mut wx_server, ticket: u64, rgba8_host: *mut u8, hits_host: *mut wx_hit) -> c_int;
    pub fn wx_server_release(srv: *mut wx_server, ticket: u64) -> c_int;
    pub fn wx_server_get_stats(srv: *mut wx_server, out: *mut wx_server_stats) -> c_int;
    pub fn wx_server_replay(srv: *mut wx_server, reqs: *const wx_request, arrival_s: *const f64, n: u32, results: *mut wx_result, release: c_int, timeout_s: f64) -> c_int;
    pub fn wx_server_destroy(srv: *mut wx_server) -> c_int;
    pub fn wx_check_division(ctx: *mut wx_ctx, max_m: u32, out: *mut u64) -> c_int;
    pub fn wx_bounds_violations(ctx: *mut wx_ctx, count: *mut u64) -> c_int;
    pub fn wx_state_build(eye: *const f32, target: *const f32, up: *const f32, aspect: f32, fovy_deg: f32, resolution_width: f32, render_mode: u32, show_345: *const u32, sun_dir: *const f32, sun_color: *const f32, sun_intensity: f32, out: *mut wx_state_uniform) -> c_int;
    pub fn wx_sun_default(dir: *mut f32, color: *mut f32, intensity: *mut f32);
    pub fn wx_topology_from_masks(kids5: *const u32, vals5: *const u32, n5: u64, kids4: *const u32, vals4: *const u32, n4: u64, vals3: *const u32, n3: u64, origins: *const i32, origin_stride: u32, out: *mut *mut wx_topology) -> c_int;
    pub fn wx_topology_from_voxels(ijk: *const i32, n: u64, out: *mut *mut wx_topology) -> c_int;
    pub fn wx_topology_from_leaves(origins: *const i32, masks: *const u64, n: u64, out: *mut *mut wx_topology) -> c_int;
    pub fn wx_topology_free(topo: *mut wx_topology);
    pub fn wx_topology_counts(topo: *const wx_topology, counts: *mut u64) -> c_int;
    pub fn wx_topology_active_voxels(topo: *const wx_topology) -> u64;
    pub fn wx_topology_masks(topo: *const wx_topology, kids5: *mut u32, vals5: *mut u32, kids4: *mut u32, vals4: *mut u32, vals3: *mut u32, origins: *mut i32) -> c_int;
    pub fn wx_topology_sdf(topo: *mut wx_topology, nthreads: c_int) -> c_int;
    pub fn wx_topology_atlas(topo: *const wx_topology, side: *mut u32, a5: *mut u32, a4: *mut u32, a3: *mut u32, value_texel: u32) -> c_int;
    pub fn wx_vdb_read_topology(path: *const c_char, grid_name: *const c_char, out: *mut *mut wx_topology, info: *mut wx_vdb_info) -> c_int;
    pub fn wx_vdb_read_leaf_values(path: *const c_char, grid_name: *const c_char, values: *mut f32, capacity: u64, count: *mut u64, background: *mut f32) -> c_int;
    pub fn wx_gen_sphere(cx: f32, cy: f32, cz: f32, radius: f32, band: f32, out: *mut *mut wx_topology) -> c_int;
    pub fn wx_gen_spheres(count: u32, rmin: f32, rmax: f32, lo: f32, hi: f32, band: f32, seed: u64, out: *mut *mut wx_topology) -> c_int;
    pub fn wx_gen_sphere_values(topo: *const wx_topology, cx: f32, cy: f32, cz: f32, radius: f32, band: f32, values: *mut f32) -> c_int;
    pub fn wx_gen_spheres_values(topo: *const wx_topology, count: u32, rmin: f32, rmax: f32, lo: f32, hi: f32, band: f32, seed: u64, values: *mut f32) -> c_int;
    pub fn wx_gen_noise_leaves(lo: i32, extent: u32, occupancy: f64, p_voxel: f64, seed: u64, nthreads: c_int, out: *mut *mut wx_topology) -> c_int;
    pub fn wx_orbit_eyes(count: u32, radius: f32, seed: u64, eyes_xyz: *mut f32) -> c_int;
}

/// Owns a device context; one per render thread (the reference renders on the
/// winit thread, src/runtime.rs:97-109).
pub struct Gb300 {
    ctx: *mut wx_ctx,
}

pub struct Grid<'a> {
    owner: &'a Gb300,
    grid: *mut wx_grid,
}

#[derive(Debug)]
pub struct Gb300Error(pub c_int, pub String);

impl Gb300 {
    pub fn new(device: i32) -> Result<Self, Gb300Error> {
        let mut ctx = std::ptr::null_mut();
        let rc = unsafe { wx_ctx_create(device, &mut ctx) };
        if rc != WX_OK {
            return Err(Gb300Error(rc, "wx_ctx_create failed".into()));
        }
        Ok(Self { ctx })
    }

    fn err(&self, rc: c_int) -> Gb300Error {
        let msg = unsafe { CStr::from_ptr(wx_last_error(self.ctx)) }.to_string_lossy().into_owned();
        Gb300Error(rc, msg)
    }

    /// Replaces wgpu_context.rs:101-159: the same masks()/origins()/atlas()
    /// the wgpu path uploads, handed over once per model.
    pub fn upload(&self, vdb: &VDB345<u32>) -> Result<Grid<'_>, Gb300Error> {
        let (kids5, vals5, kids4, vals4, vals3) = vdb.masks();
        let origins: Vec<[i32; 4]> = vdb.origins().iter().map(|&[x, y, z]| [x, y, z, 0]).collect();
        let atlas = vdb.atlas();
        // Flatten exactly as wgpu_context.rs:119-134 does for write_texture:
        // texel (x, y, z) at (z * H + y) * W + x holds cube[x][y][z].
        let flat: Vec<Vec<u32>> = atlas
            .iter()
            .map(|cube| {
                let n = cube.len();
                let mut f = vec![0u32; n * n * n];
                for x in 0..n {
                    for y in 0..n {
                        for z in 0..n {
                            f[(z * n + y) * n + x] = cube[x][y][z];
                        }
                    }
                }
                f
            })
            .collect();
        let side = |i: usize| atlas[i].len() as u32;
        let view = wx_vdb345_view {
            kids5: kids5.as_ptr() as *const u32,
            vals5: vals5.as_ptr() as *const u32,
            kids4: kids4.as_ptr() as *const u32,
            vals4: vals4.as_ptr() as *const u32,
            vals3: vals3.as_ptr() as *const u32,
            origins: origins.as_ptr() as *const i32,
            n5: kids5.len() as u64,
            n4: kids4.len() as u64,
            n3: vals3.len() as u64,
            origin_stride: 4,
            atlas: [flat[0].as_ptr(), flat[1].as_ptr(), flat[2].as_ptr()],
            dims: [[side(0); 3], [side(1); 3], [side(2); 3]],
        };
        let mut grid = std::ptr::null_mut();
        let rc = unsafe { wx_grid_upload(self.ctx, &view, &mut grid) };
        if rc != WX_OK {
            return Err(self.err(rc));
        }
        Ok(Grid { owner: self, grid })
    }

    /// Replaces the compute pass of wgpu_context.rs:270-282. `rgba8` receives
    /// width*height*4 bytes (host memory here; a device pointer also works).
    pub fn render(
        &self,
        grid: &Grid,
        state: &ComputeState,
        width: u32,
        height: u32,
        rgba8: &mut [u8],
    ) -> Result<(), Gb300Error> {
        assert!(rgba8.len() >= (width * height * 4) as usize);
        let rc = unsafe {
            wx_render(
                self.ctx,
                grid.grid,
                state,
                width,
                height,
                rgba8.as_mut_ptr(),
                std::ptr::null_mut(),
                std::ptr::null_mut(),
            )
        };
        if rc != WX_OK {
            return Err(self.err(rc));
        }
        Ok(())
    }
}

impl Drop for Grid<'_> {
    fn drop(&mut self) {
        unsafe { wx_grid_release(self.owner.ctx, self.grid) };
    }
}

impl Drop for Gb300 {
    fn drop(&mut self) {
        unsafe { wx_ctx_destroy(self.ctx) };
    }
}
