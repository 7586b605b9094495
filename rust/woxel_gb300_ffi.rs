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

extern "C" {
    pub fn wx_ctx_create(device: c_int, out: *mut *mut wx_ctx) -> c_int;
    pub fn wx_ctx_destroy(ctx: *mut wx_ctx) -> c_int;
    pub fn wx_last_error(ctx: *const wx_ctx) -> *const c_char;
    pub fn wx_grid_upload(ctx: *mut wx_ctx, view: *const wx_vdb345_view, out: *mut *mut wx_grid) -> c_int;
    pub fn wx_grid_release(ctx: *mut wx_ctx, grid: *mut wx_grid) -> c_int;
    pub fn wx_render(
        ctx: *mut wx_ctx,
        grid: *const wx_grid,
        state: *const wx_state_uniform,
        width: u32,
        height: u32,
        rgba8: *mut u8,
        hits: *mut wx_hit,
        stream: *mut c_void,
    ) -> c_int;
    pub fn wx_render_batch(ctx: *mut wx_ctx, frames: *const wx_frame, n: u32, stream: *mut c_void) -> c_int;
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
