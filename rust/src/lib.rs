//! mantaray's Rust entry points over the GB300 library.
//!
//! The reference crate traces each ray with `ode_solvers::Rk4` on CPU threads
//! (`ManyRays::trace_many`, src/ray.rs:98-127; `SingleRay::trace_individual`,
//! src/ray.rs:198-213) behind the PyO3 module `_mantaray` (src/ffi.rs:18-85).
//! Here the same calls run the plain FP64 CUDA kernel of libmantaray_gpu.so
//! (one ray per GPU thread, the reference's stepper, equations and lookups,
//! within 1e-9 of the reference at every step).  Fields are opened once into
//! device memory and may be shared by any number of calls.
//!
//! Differences from the reference, all on failure paths: a file that cannot
//! be opened is an `Err` instead of a panic (src/ffi.rs:36-38), and rays are
//! never dropped from `ray_tracing` (the reference's filter at src/ffi.rs:75
//! only removes rays whose integration returned `Err`, which the stepper
//! never does: every field error becomes a NaN derivative and ends the ray).

mod sys;

use std::ffi::{CStr, CString};
use std::fmt;
use std::path::Path;
use std::ptr;

pub use sys::{MR_MATH_IDENTITY, MR_MATH_LIBM, MR_STOP_FRESH, MR_STOP_STAGE1};

/// A failed library call: its MR_ERR_* code and message.
#[derive(Debug, Clone)]
pub struct Error {
    pub code: i32,
    pub message: String,
}

impl fmt::Display for Error {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "mantaray_gpu error {}: {}", self.code, self.message)
    }
}

impl std::error::Error for Error {}

pub type Result<T> = std::result::Result<T, Error>;

fn check(rc: i32) -> Result<()> {
    if rc == sys::MR_OK {
        return Ok(());
    }
    // SAFETY: mr_last_error returns a thread-local NUL-terminated string.
    let message = unsafe { CStr::from_ptr(sys::mr_last_error()) }
        .to_string_lossy()
        .into_owned();
    Err(Error { code: rc, message })
}

fn c_string(s: &str) -> Result<CString> {
    CString::new(s).map_err(|_| Error {
        code: sys::MR_ERR_INVALID_ARGUMENT,
        message: format!("{s:?} holds a NUL byte"),
    })
}

fn path_string(p: &Path) -> Result<CString> {
    c_string(&p.to_string_lossy())
}

/// Bathymetry staged in device memory (CartesianNetcdf3, ConstantDepth,
/// ConstantSlope of the reference).
pub struct Bathymetry {
    raw: *mut sys::MrBathymetry,
}

// The handle is immutable after creation: calls on several threads may share it.
unsafe impl Send for Bathymetry {}
unsafe impl Sync for Bathymetry {}

impl Bathymetry {
    /// CartesianNetcdf3::open(path, x_name, y_name, depth_name)
    /// (src/bathymetry/cartesian_netcdf3.rs:167-256).
    pub fn open(path: &Path, x_name: &str, y_name: &str, depth_name: &str) -> Result<Self> {
        let (p, x, y, d) = (path_string(path)?, c_string(x_name)?, c_string(y_name)?,
                            c_string(depth_name)?);
        let mut raw = ptr::null_mut();
        check(unsafe { sys::mr_bathymetry_open(p.as_ptr(), x.as_ptr(), y.as_ptr(), d.as_ptr(),
                                               &mut raw) })?;
        Ok(Self { raw })
    }

    /// A grid: f32 axes, f64 depth read with flat index nx * j + i.
    pub fn grid(x: &[f32], y: &[f32], depth: &[f64]) -> Result<Self> {
        let mut raw = ptr::null_mut();
        check(unsafe { sys::mr_bathymetry_grid(x.len(), y.len(), x.as_ptr(), y.as_ptr(),
                                               depth.as_ptr(), depth.len(), &mut raw) })?;
        Ok(Self { raw })
    }

    /// ConstantDepth (src/bathymetry/constant_depth.rs).
    pub fn constant(h: f32) -> Result<Self> {
        let mut raw = ptr::null_mut();
        check(unsafe { sys::mr_bathymetry_constant(h, &mut raw) })?;
        Ok(Self { raw })
    }

    /// ConstantSlope (src/bathymetry/constant_slope.rs).
    pub fn slope(h0: f32, x0: f32, y0: f32, dhdx: f32, dhdy: f32) -> Result<Self> {
        let mut raw = ptr::null_mut();
        check(unsafe { sys::mr_bathymetry_slope(h0, x0, y0, dhdx, dhdy, &mut raw) })?;
        Ok(Self { raw })
    }
}

impl Drop for Bathymetry {
    fn drop(&mut self) {
        unsafe { sys::mr_bathymetry_destroy(self.raw) }
    }
}

/// Current staged in device memory (CartesianCurrent, ConstantCurrent).
pub struct Current {
    raw: *mut sys::MrCurrent,
}

unsafe impl Send for Current {}
unsafe impl Sync for Current {}

impl Current {
    /// CartesianCurrent::open(path, x_name, y_name, u_name, v_name)
    /// (src/current/cartesian_current.rs:58-213).
    pub fn open(path: &Path, x_name: &str, y_name: &str, u_name: &str, v_name: &str)
                -> Result<Self> {
        let (p, x, y, u, v) = (path_string(path)?, c_string(x_name)?, c_string(y_name)?,
                               c_string(u_name)?, c_string(v_name)?);
        let mut raw = ptr::null_mut();
        check(unsafe { sys::mr_current_open(p.as_ptr(), x.as_ptr(), y.as_ptr(), u.as_ptr(),
                                            v.as_ptr(), &mut raw) })?;
        Ok(Self { raw })
    }

    /// A grid: f64 axes, f64 u and v read with flat index nx * j + i.
    pub fn grid(x: &[f64], y: &[f64], u: &[f64], v: &[f64]) -> Result<Self> {
        let mut raw = ptr::null_mut();
        check(unsafe { sys::mr_current_grid(x.len(), y.len(), x.as_ptr(), y.as_ptr(), u.as_ptr(),
                                            u.len(), v.as_ptr(), v.len(), &mut raw) })?;
        Ok(Self { raw })
    }

    /// ConstantCurrent (src/current/constant_current.rs).
    pub fn constant(u: f64, v: f64) -> Result<Self> {
        let mut raw = ptr::null_mut();
        check(unsafe { sys::mr_current_constant(u, v, &mut raw) })?;
        Ok(Self { raw })
    }
}

impl Drop for Current {
    fn drop(&mut self) {
        unsafe { sys::mr_current_destroy(self.raw) }
    }
}

/// Initial state of a ray (RayState, src/datatype.rs:117-150).
#[derive(Debug, Clone, Copy)]
pub struct RayState {
    pub x: f64,
    pub y: f64,
    pub kx: f64,
    pub ky: f64,
}

/// One ray's result: the times and states the stepper recorded, the initial
/// state first (`SolverResult::get()` of ode_solvers as the reference reads it).
#[derive(Debug, Clone, Default)]
pub struct Trajectory {
    pub t: Vec<f64>,
    pub state: Vec<[f64; 4]>,
}

impl Trajectory {
    /// The reference's (t, x, y, kx, ky) tuples (src/ffi.rs:42-47).
    pub fn tuples(&self) -> Vec<(f64, f64, f64, f64, f64)> {
        self.t.iter().zip(&self.state).map(|(t, s)| (*t, s[0], s[1], s[2], s[3])).collect()
    }
}

/// Traces rays from t0 to t_end with step dt on the GPU (one launch).
/// `options`: MR_STOP_* | MR_MATH_* (MR_MATH_IDENTITY, 0, is the default).
pub fn trace(bathymetry: &Bathymetry, current: &Current, rays: &[RayState], t0: f64,
             t_end: f64, dt: f64, options: i32) -> Result<Vec<Trajectory>> {
    let n = rays.len();
    let rows = unsafe { sys::mr_num_steps(t0, t_end, dt) } as usize + 1;
    let (x0, y0): (Vec<f64>, Vec<f64>) = rays.iter().map(|r| (r.x, r.y)).unzip();
    let (kx0, ky0): (Vec<f64>, Vec<f64>) = rays.iter().map(|r| (r.kx, r.ky)).unzip();
    let mut traj = vec![0f64; 5 * rows * n];
    let mut n_rows = vec![0i32; n];
    let mut status = vec![0u8; n];
    check(unsafe {
        sys::mr_trace(bathymetry.raw, current.raw, n, x0.as_ptr(), y0.as_ptr(), kx0.as_ptr(),
                      ky0.as_ptr(), t0, t_end, dt, options, rows, traj.as_mut_ptr(),
                      n_rows.as_mut_ptr(), status.as_mut_ptr())
    })?;
    // traj is [5][rows][n]: variable v of ray i at row r is traj[(v * rows + r) * n + i]
    Ok((0..n)
        .map(|i| {
            let at = |v: usize, r: usize| traj[(v * rows + r) * n + i];
            let len = n_rows[i] as usize;
            Trajectory {
                t: (0..len).map(|r| at(0, r)).collect(),
                state: (0..len).map(|r| [at(1, r), at(2, r), at(3, r), at(4, r)]).collect(),
            }
        })
        .collect())
}

/// SingleRay (src/ray.rs:130-213): one ray over borrowed fields.
pub struct SingleRay<'a> {
    bathymetry: &'a Bathymetry,
    current: &'a Current,
    initial: RayState,
}

impl<'a> SingleRay<'a> {
    pub fn new(bathymetry: &'a Bathymetry, current: &'a Current, initial: &RayState) -> Self {
        Self { bathymetry, current, initial: *initial }
    }

    /// trace_individual(t0, t_end, step_size) (src/ray.rs:198-213).
    pub fn trace_individual(&self, t0: f64, t_end: f64, step_size: f64) -> Result<Trajectory> {
        let mut v = trace(self.bathymetry, self.current, &[self.initial], t0, t_end, step_size,
                          MR_STOP_STAGE1 | MR_MATH_IDENTITY)?;
        Ok(v.pop().unwrap_or_default())
    }
}

/// ManyRays (src/ray.rs:22-127): many rays over borrowed fields.
pub struct ManyRays<'a> {
    bathymetry: &'a Bathymetry,
    current: &'a Current,
    initial: &'a [RayState],
}

impl<'a> ManyRays<'a> {
    pub fn new(bathymetry: &'a Bathymetry, current: &'a Current, initial: &'a [RayState]) -> Self {
        Self { bathymetry, current, initial }
    }

    /// trace_many(t0, t_end, step_size) (src/ray.rs:98-127): one result per
    /// ray, `None` where the reference would give `None` (never, see the
    /// crate notes), all rays `None` when the call itself fails.
    pub fn trace_many(&self, t0: f64, t_end: f64, step_size: f64) -> Vec<Option<Trajectory>> {
        match trace(self.bathymetry, self.current, self.initial, t0, t_end, step_size,
                    MR_STOP_STAGE1 | MR_MATH_IDENTITY) {
            Ok(v) => v.into_iter().map(Some).collect(),
            Err(e) => {
                eprintln!("{e}");
                vec![None; self.initial.len()]
            }
        }
    }
}

/// The extension module of the reference (src/ffi.rs:18-85), same names and
/// signatures: `mantaray.core` imports it unchanged.
#[cfg(feature = "python")]
mod python {
    use super::*;
    use pyo3::exceptions::{PyIOError, PyRuntimeError, PyValueError};
    use pyo3::prelude::*;

    fn to_py(e: Error) -> PyErr {
        match e.code {
            sys::MR_ERR_IO | sys::MR_ERR_READ => PyIOError::new_err(e.to_string()),
            sys::MR_ERR_INVALID_ARGUMENT | sys::MR_ERR_CAPACITY => {
                PyValueError::new_err(e.to_string())
            }
            _ => PyRuntimeError::new_err(e.to_string()),
        }
    }

    fn fields(bathymetry_filename: &str, current_filename: &str)
              -> PyResult<(Bathymetry, Current)> {
        let b = Bathymetry::open(Path::new(bathymetry_filename), "x", "y", "depth")
            .map_err(to_py)?;
        let c = Current::open(Path::new(current_filename), "x", "y", "u", "v").map_err(to_py)?;
        Ok((b, c))
    }

    /// _mantaray.single_ray (src/ffi.rs:25-49).
    #[pyfunction]
    #[allow(clippy::too_many_arguments)]
    fn single_ray(py: Python<'_>, x0: f64, y0: f64, kx0: f64, ky0: f64, duration: f64,
                  step_size: f64, bathymetry_filename: String, current_filename: String)
                  -> PyResult<Vec<(f64, f64, f64, f64, f64)>> {
        let (b, c) = fields(&bathymetry_filename, &current_filename)?;
        let initial = RayState { x: x0, y: y0, kx: kx0, ky: ky0 };
        py.allow_threads(|| SingleRay::new(&b, &c, &initial).trace_individual(0.0, duration,
                                                                               step_size))
            .map(|t| t.tuples())
            .map_err(to_py)
    }

    /// _mantaray.ray_tracing (src/ffi.rs:51-85).
    #[pyfunction]
    #[allow(clippy::too_many_arguments)]
    fn ray_tracing(py: Python<'_>, x0: Vec<f64>, y0: Vec<f64>, kx0: Vec<f64>, ky0: Vec<f64>,
                   duration: f64, step_size: f64, bathymetry_filename: String,
                   current_filename: String) -> PyResult<Vec<Vec<(f64, f64, f64, f64, f64)>>> {
        if y0.len() != x0.len() || kx0.len() != x0.len() || ky0.len() != x0.len() {
            return Err(PyValueError::new_err("x0, y0, kx0 and ky0 must have the same length"));
        }
        let (b, c) = fields(&bathymetry_filename, &current_filename)?;
        let rays: Vec<RayState> = (0..x0.len())
            .map(|i| RayState { x: x0[i], y: y0[i], kx: kx0[i], ky: ky0[i] })
            .collect();
        let res = py.allow_threads(|| trace(&b, &c, &rays, 0.0, duration, step_size,
                                            MR_STOP_STAGE1 | MR_MATH_IDENTITY));
        Ok(res.map_err(to_py)?.iter().map(Trajectory::tuples).collect())
    }

    #[pymodule]
    fn _mantaray(m: &Bound<'_, PyModule>) -> PyResult<()> {
        m.add_function(wrap_pyfunction!(single_ray, m)?)?;
        m.add_function(wrap_pyfunction!(ray_tracing, m)?)?;
        Ok(())
    }
}
