//! GPU backend of prestige: particle systems resident on one GB300, stepped by the CUDA library
//! through its C ABI (include/prestige_gpu.h, bound in `ffi`).
//!
//! The reference runs fused pairwise equations as a CPU loop `for i in 0..n { for j in 0..n {
//! body } }` (prestige/src/codegen/simple_cpu.rs:3-22), over slices addressed by the names that
//! `#[equation]` records (prestige_macros/src/lib.rs:64-133, EquationIR.reads / .writes in
//! prestige/src/equations/ir.rs:3-14).  Here a `System` owns those slices on the device, by the
//! same names, and runs:
//!   * `run_equations` / `run_gpu`: the fused bodies as a gather over the cell-list neighbour set
//!     (the GPU counterpart of generate_simple_cpu);
//!   * `step`: the SPH step (continuity, Tait pressure, artificial viscosity, symplectic Euler)
//!     or the DEM step (spring-dashpot contacts with tangential history);
//!   * `forward_checkpointed` / `backward`: the adjoint of the SPH run, returning dL/dalpha,
//!     dL/dB and dL/dv0;
//!   * `System::batch`: many independent SPH systems in one handle.
//!
//! There is no CPU fallback: every call runs on the GPU or returns an error.
#![allow(clippy::missing_safety_doc)]

pub mod ffi;

use std::ffi::{CStr, CString};
use std::fmt;
use std::os::raw::{c_char, c_int, c_void};
use std::ptr;

/// A failed call: the library's status code and the message of `pg_last_error()`.
#[derive(Clone, Debug, PartialEq, Eq)]
pub struct Error {
    pub status: i32,
    pub message: String,
}

impl fmt::Display for Error {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "prestige_gpu status {}: {}", self.status, self.message)
    }
}

impl std::error::Error for Error {}

pub type Result<T> = std::result::Result<T, Error>;

fn check(status: c_int) -> Result<()> {
    if status == ffi::PG_OK {
        return Ok(());
    }
    let message = unsafe {
        let p = ffi::pg_last_error();
        if p.is_null() { String::new() } else { CStr::from_ptr(p).to_string_lossy().into_owned() }
    };
    Err(Error { status, message })
}

fn cname(name: &str) -> Result<CString> {
    CString::new(name).map_err(|_| Error { status: ffi::PG_EINVAL, message: format!("field name {name:?} has a NUL") })
}

/// Particle model of a handle.
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Model {
    Sph,
    Dem,
}

/// Configuration of a system (`pg_config`), starting from the library's defaults.
#[derive(Clone, Copy, Debug)]
pub struct Config(pub ffi::pg_config);

impl Default for Config {
    fn default() -> Self {
        let mut c = ffi::pg_config::default();
        unsafe { ffi::pg_config_default(&mut c) };
        Config(c)
    }
}

impl Config {
    pub fn sph(dim: i32, h: f64, dt: f64) -> Self {
        let mut c = Config::default();
        c.0.model = ffi::PG_MODEL_SPH;
        c.0.dim = dim;
        c.0.h = h;
        c.0.dt = dt;
        c
    }
    pub fn dem(r_max: f64, dt: f64) -> Self {
        let mut c = Config::default();
        c.0.model = ffi::PG_MODEL_DEM;
        c.0.dim = 3;
        c.0.r_max = r_max;
        c.0.dt = dt;
        c
    }
    pub fn domain(mut self, lo: [f64; 3], hi: [f64; 3]) -> Self {
        self.0.domain_lo = lo;
        self.0.domain_hi = hi;
        self
    }
    /// PG_F64_NATIVE (IEEE, bit-exact with the oracle) or PG_F64_FAST (double-word pair terms).
    pub fn f64_mode(mut self, mode: i32) -> Self {
        self.0.f64_mode = mode;
        self
    }
    pub fn single_precision(mut self) -> Self {
        self.0.precision = ffi::PG_F32;
        self
    }
}

/// Gradients returned by `System::backward`.
#[derive(Clone, Debug)]
pub struct Gradients {
    pub d_alpha: f64,
    pub d_tait_b: f64,
    /// dL/dv0, n * dim, particle-id order.
    pub d_v0: Vec<f64>,
}

/// One GPU-resident particle system (or a batch of independent SPH systems).  Dropping it
/// frees its device memory.  Calls on one `System` take `&mut self`: the library requires
/// them to be serialised.
pub struct System {
    raw: *mut ffi::pg_system,
    n: usize,
    dim: usize,
    double: bool,
    model: Model,
}

// The handle is used by one thread at a time (&mut self); moving it between threads is fine.
unsafe impl Send for System {}

impl Drop for System {
    fn drop(&mut self) {
        if !self.raw.is_null() {
            unsafe { ffi::pg_destroy(self.raw) };
            self.raw = ptr::null_mut();
        }
    }
}

impl System {
    pub fn new(cfg: &Config, n: usize) -> Result<System> {
        let mut raw = ptr::null_mut();
        check(unsafe { ffi::pg_create(&cfg.0, n, &mut raw) })?;
        Ok(Self::wrap(raw, n, &cfg.0))
    }

    /// `counts[s]` particles of system s, concatenated in id order (shared dim, precision,
    /// arithmetic mode and cell multiplier).
    pub fn batch(cfgs: &[Config], counts: &[usize]) -> Result<System> {
        if cfgs.len() != counts.len() || cfgs.is_empty() {
            return Err(Error { status: ffi::PG_EINVAL, message: "one count per configuration".into() });
        }
        let raw_cfgs: Vec<ffi::pg_config> = cfgs.iter().map(|c| c.0).collect();
        let mut raw = ptr::null_mut();
        check(unsafe { ffi::pg_batch_create(raw_cfgs.as_ptr(), counts.as_ptr(), cfgs.len() as c_int, &mut raw) })?;
        Ok(Self::wrap(raw, counts.iter().sum(), &cfgs[0].0))
    }

    fn wrap(raw: *mut ffi::pg_system, n: usize, c: &ffi::pg_config) -> System {
        let model = if c.model == ffi::PG_MODEL_DEM { Model::Dem } else { Model::Sph };
        System { raw, n, dim: if model == Model::Dem { 3 } else { c.dim as usize }, double: c.precision != ffi::PG_F32, model }
    }

    pub fn len(&self) -> usize {
        self.n
    }
    pub fn is_empty(&self) -> bool {
        self.n == 0
    }
    pub fn dim(&self) -> usize {
        self.dim
    }
    pub fn model(&self) -> Model {
        self.model
    }
    /// True if the SPH state is stored in double precision (DEM state always is).
    pub fn is_double(&self) -> bool {
        self.double
    }

    /// Copy a named slice from the host (id order, vectors interleaved), in double precision;
    /// the library converts to the stored precision.
    pub fn set(&mut self, name: &str, values: &[f64]) -> Result<()> {
        let n = cname(name)?;
        check(unsafe {
            ffi::pg_set_field(self.raw, n.as_ptr(), values.as_ptr() as *const c_void, values.len(), ffi::PG_F64)
        })
    }

    pub fn set_f32(&mut self, name: &str, values: &[f32]) -> Result<()> {
        let n = cname(name)?;
        check(unsafe {
            ffi::pg_set_field(self.raw, n.as_ptr(), values.as_ptr() as *const c_void, values.len(), ffi::PG_F32)
        })
    }

    /// Number of values of a named slice: n * dim for pos, vel, acc (DEM: and omega), else n.
    pub fn field_len(&self, name: &str) -> usize {
        match name {
            "pos" | "vel" | "acc" => self.n * self.dim,
            "omega" => self.n * 3,
            _ => self.n,
        }
    }

    pub fn get(&mut self, name: &str) -> Result<Vec<f64>> {
        let n = cname(name)?;
        let mut out = vec![0.0f64; self.field_len(name)];
        check(unsafe {
            ffi::pg_get_field(self.raw, n.as_ptr(), out.as_mut_ptr() as *mut c_void, out.len(), ffi::PG_F64)
        })?;
        Ok(out)
    }

    /// Stage an upload of a named slice (f64 values) on the input copy stream; it takes effect
    /// before the next call on the handle.
    ///
    /// # Safety
    /// `values` must stay valid and unchanged until `wait_io` returns; page-locked memory lets the
    /// copy overlap the steps.
    pub unsafe fn set_async(&mut self, name: &str, values: *const f64, count: usize) -> Result<()> {
        let n = cname(name)?;
        check(ffi::pg_set_field_async(self.raw, n.as_ptr(), values as *const c_void, count, ffi::PG_F64))
    }

    /// Snapshot a named slice now and download it on the output copy stream.
    ///
    /// # Safety
    /// `out` must stay valid for `count` values until `wait_io` returns.
    pub unsafe fn get_async(&mut self, name: &str, out: *mut f64, count: usize) -> Result<()> {
        let n = cname(name)?;
        check(ffi::pg_get_field_async(self.raw, n.as_ptr(), out as *mut c_void, count, ffi::PG_F64))
    }

    /// Wait for every staged copy and step of the handle; reports device-side errors.
    pub fn wait_io(&mut self) -> Result<()> {
        check(unsafe { ffi::pg_wait_io(self.raw) })
    }

    /// Neighbour search (cell hash, stable sort, cell table): per sorted slot its cell and
    /// particle id, and the cell-start table.
    pub fn neighbors(&mut self) -> Result<(Vec<u32>, Vec<u32>, Vec<u32>)> {
        check(unsafe { ffi::pg_build_neighbors(self.raw) })?;
        let mut nc = 0usize;
        check(unsafe { ffi::pg_num_cells(self.raw, &mut nc) })?;
        let mut cell = vec![0u32; self.n];
        let mut ids = vec![0u32; self.n];
        let mut start = vec![0u32; nc + 1];
        check(unsafe {
            ffi::pg_get_neighbors(self.raw, cell.as_mut_ptr(), ids.as_mut_ptr(), start.as_mut_ptr(), nc + 1)
        })?;
        Ok((cell, ids, start))
    }

    /// Neighbour count of every particle (itself included), id order.
    pub fn neighbor_counts(&mut self) -> Result<Vec<u32>> {
        let mut out = vec![0u32; self.n];
        check(unsafe { ffi::pg_count_neighbors(self.raw, out.as_mut_ptr()) })?;
        Ok(out)
    }

    /// The reference's eq1 over the neighbour set: dst[i] += sum_j src[j] (prestige/src/lib.rs:7-12).
    pub fn gather_sum(&mut self, dst: &str, src: &str) -> Result<()> {
        let (d, s) = (cname(dst)?, cname(src)?);
        check(unsafe { ffi::pg_gather_sum(self.raw, d.as_ptr(), s.as_ptr()) })
    }

    /// Fused pairwise bodies given as source text (the `body` strings of FusedEquations), run
    /// for every i over its neighbours j on the GPU.
    pub fn run_equations<S: AsRef<str>>(&mut self, bodies: &[S]) -> Result<()> {
        let owned: Vec<CString> = bodies.iter().map(|b| cname(b.as_ref())).collect::<Result<_>>()?;
        let ptrs: Vec<*const c_char> = owned.iter().map(|c| c.as_ptr()).collect();
        check(unsafe { ffi::pg_run_equations(self.raw, ptrs.as_ptr(), ptrs.len() as c_int) })
    }

    /// SPH rates of the current state without integrating: (acc without gravity, drho/dt).
    pub fn compute_rates(&mut self) -> Result<(Vec<f64>, Vec<f64>)> {
        check(unsafe { ffi::pg_compute_rates(self.raw) })?;
        Ok((self.get("acc")?, self.get("drho")?))
    }

    pub fn step(&mut self, nsteps: i32) -> Result<()> {
        check(unsafe { ffi::pg_step(self.raw, nsteps) })
    }

    /// Half a step: 0 = continuity (rho' into "rho"), 1 = momentum with the densities in "rho".
    pub fn step_stage(&mut self, stage: i32) -> Result<()> {
        check(unsafe { ffi::pg_step_stage(self.raw, stage) })
    }

    pub fn step_async(&mut self, nsteps: i32) -> Result<()> {
        check(unsafe { ffi::pg_step_async(self.raw, nsteps) })
    }

    pub fn sync(&mut self) -> Result<()> {
        check(unsafe { ffi::pg_sync(self.raw) })
    }

    /// Replay a captured CUDA graph of the step from now on.
    pub fn enable_graph(&mut self, enable: bool) -> Result<()> {
        check(unsafe { ffi::pg_enable_graph(self.raw, enable as c_int) })
    }

    /// DEM: particle-particle contacts of the last step (both sides counted).
    pub fn dem_contacts(&mut self) -> Result<i64> {
        let mut c = 0;
        check(unsafe { ffi::pg_dem_contacts(self.raw, &mut c) })?;
        Ok(c)
    }

    /// DEM: the tangential history, id order: partner ids (n * capacity; 0xFFFFFFF0 + face for
    /// a wall, u32::MAX for an empty slot) and springs (n * capacity * 3).  `capacity` is the
    /// configuration's contact capacity (the library refuses any other).
    pub fn dem_history(&mut self, capacity: usize) -> Result<(Vec<u32>, Vec<f64>)> {
        let mut partner = vec![0u32; self.n * capacity];
        let mut xi = vec![0.0f64; self.n * capacity * 3];
        check(unsafe { ffi::pg_dem_get_history(self.raw, partner.as_mut_ptr(), xi.as_mut_ptr(), capacity) })?;
        Ok((partner, xi))
    }

    /// DEM: replace the tangential history (the layout of `dem_history`).
    pub fn set_dem_history(&mut self, partner: &[u32], xi: &[f64], capacity: usize) -> Result<()> {
        if partner.len() != self.n * capacity || xi.len() != self.n * capacity * 3 {
            return Err(Error { status: ffi::PG_EINVAL, message: "history of n * capacity partners and springs".into() });
        }
        check(unsafe { ffi::pg_dem_set_history(self.raw, partner.as_ptr(), xi.as_ptr(), capacity) })
    }

    /// Differentiable run: nsteps from the current state, checkpoints every `every` steps.
    pub fn forward_checkpointed(&mut self, nsteps: i32, every: i32) -> Result<()> {
        check(unsafe { ffi::pg_forward_checkpointed(self.raw, nsteps, every) })
    }

    /// Adjoint of the last forward_checkpointed run for dL/dx of the final positions (n * dim,
    /// id order).
    pub fn backward(&mut self, dl_dx: &[f64]) -> Result<Gradients> {
        if dl_dx.len() != self.n * self.dim {
            return Err(Error { status: ffi::PG_EINVAL, message: format!("dL/dx needs {} values", self.n * self.dim) });
        }
        let mut g = Gradients { d_alpha: 0.0, d_tait_b: 0.0, d_v0: vec![0.0; self.n * self.dim] };
        check(unsafe {
            ffi::pg_backward(self.raw, dl_dx.as_ptr(), &mut g.d_alpha, &mut g.d_tait_b, g.d_v0.as_mut_ptr())
        })?;
        Ok(g)
    }

    /// Autotune block size, cell multiplier and arithmetic mode on the current state (restored
    /// afterwards); returns (block, multiplier, f64 mode, ms per step).
    pub fn autotune(&mut self, trial_steps: i32) -> Result<(i32, f64, i32, f64)> {
        let (mut b, mut m, mut f, mut ms) = (0, 0.0, 0, 0.0);
        check(unsafe { ffi::pg_autotune(self.raw, trial_steps, &mut b, &mut m, &mut f, &mut ms) })?;
        Ok((b, m, f, ms))
    }

    pub fn set_tuning(&mut self, block: i32, cell_multiplier: f64, f64_mode: i32) -> Result<()> {
        check(unsafe { ffi::pg_set_tuning(self.raw, block, cell_multiplier, f64_mode) })
    }

    /// Particles per warp of the continuity and momentum passes (32, 16 or 8).
    pub fn set_particles_per_warp(&mut self, ppw: i32) -> Result<()> {
        check(unsafe { ffi::pg_set_particles_per_warp(self.raw, ppw) })
    }

    pub fn info(&mut self) -> Result<ffi::pg_info> {
        let mut i = ffi::pg_info::default();
        check(unsafe { ffi::pg_get_info(self.raw, &mut i) })?;
        Ok(i)
    }

    pub fn raw(&mut self) -> *mut ffi::pg_system {
        self.raw
    }
}

/// The GPU form of `generate_simple_cpu(&fused)` (prestige/src/codegen/simple_cpu.rs:3-22):
/// instead of returning the loop's text, run the fused bodies on the system's slices.  The
/// slices a body reads or writes must exist on the handle (set them with `System::set`).
#[cfg(feature = "prestige")]
pub fn run_gpu(fused: &prestige::equations::fuse::FusedEquations, sys: &mut System) -> Result<()> {
    sys.run_equations(&fused.bodies)
}
