//! Raw declarations of the C ABI of libmantaray_gpu.so (include/mantaray_gpu.h)
//! used by this crate.

use std::os::raw::{c_char, c_int, c_void};

#[repr(C)]
pub struct MrBathymetry {
    _private: [u8; 0],
}

#[repr(C)]
pub struct MrCurrent {
    _private: [u8; 0],
}

pub const MR_OK: c_int = 0;
pub const MR_ERR_INVALID_ARGUMENT: c_int = -1;
pub const MR_ERR_CUDA: c_int = -2;
pub const MR_ERR_IO: c_int = -3;
pub const MR_ERR_READ: c_int = -4;
pub const MR_ERR_CAPACITY: c_int = -5;
pub const MR_ERR_OUT_OF_MEMORY: c_int = -6;

pub const MR_RAY_COMPLETE: u8 = 0;
pub const MR_RAY_STOPPED: u8 = 1;

pub const MR_STOP_STAGE1: c_int = 0x0;
pub const MR_STOP_FRESH: c_int = 0x1;
pub const MR_MATH_IDENTITY: c_int = 0x0;
pub const MR_MATH_LIBM: c_int = 0x10;

extern "C" {
    pub fn mr_bathymetry_grid(nx: usize, ny: usize, x: *const f32, y: *const f32,
                              depth: *const f64, depth_len: usize,
                              out: *mut *mut MrBathymetry) -> c_int;
    pub fn mr_bathymetry_open(path: *const c_char, x_name: *const c_char,
                              y_name: *const c_char, depth_name: *const c_char,
                              out: *mut *mut MrBathymetry) -> c_int;
    pub fn mr_bathymetry_constant(h: f32, out: *mut *mut MrBathymetry) -> c_int;
    pub fn mr_bathymetry_slope(h0: f32, x0: f32, y0: f32, dhdx: f32, dhdy: f32,
                               out: *mut *mut MrBathymetry) -> c_int;
    pub fn mr_bathymetry_destroy(b: *mut MrBathymetry);

    pub fn mr_current_grid(nx: usize, ny: usize, x: *const f64, y: *const f64, u: *const f64,
                           u_len: usize, v: *const f64, v_len: usize,
                           out: *mut *mut MrCurrent) -> c_int;
    pub fn mr_current_open(path: *const c_char, x_name: *const c_char, y_name: *const c_char,
                           u_name: *const c_char, v_name: *const c_char,
                           out: *mut *mut MrCurrent) -> c_int;
    pub fn mr_current_constant(u: f64, v: f64, out: *mut *mut MrCurrent) -> c_int;
    pub fn mr_current_destroy(c: *mut MrCurrent);

    pub fn mr_num_steps(t0: f64, t_end: f64, dt: f64) -> u64;
    pub fn mr_trace(b: *const MrBathymetry, c: *const MrCurrent, n: usize, x0: *const f64,
                    y0: *const f64, kx0: *const f64, ky0: *const f64, t0: f64, t_end: f64,
                    dt: f64, options: c_int, rows_cap: usize, traj: *mut f64,
                    n_rows: *mut i32, status: *mut u8) -> c_int;
    pub fn mr_trace_device(b: *const MrBathymetry, c: *const MrCurrent, n: usize,
                           x0: *const f64, y0: *const f64, kx0: *const f64, ky0: *const f64,
                           t0: f64, t_end: f64, dt: f64, options: c_int, rows_cap: usize,
                           traj: *mut f64, n_rows: *mut i32, status: *mut u8,
                           stream: *mut c_void) -> c_int;

    pub fn mr_last_error() -> *const c_char;
    pub fn mr_version() -> c_int;
}
