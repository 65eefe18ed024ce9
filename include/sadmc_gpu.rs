// Rust binding of the C ABI in include/sadmc_gpu.h for the reference crate (sadmc):
// a maintainer copies this file to src/gpu.rs and links libsadmc_gb300 from build.rs
// (`println!("cargo:rustc-link-lib=sadmc_gb300")`).  GpuBatch replaces the
// `loop { mc.move_once() }` of src/bin/histogram.rs:8-10 for a batch of walkers.
// The struct layouts mirror the header field for field (#[repr(C)]).
#![allow(non_camel_case_types)]
use std::os::raw::{c_char, c_void};

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct sadmc_config {
    pub system: i32, pub method: i32, pub n_walkers: i32, pub max_atoms: i32,
    pub min_T: f64, pub t0: f64, pub has_min_gamma: i32, pub pad0: i32, pub min_gamma: f64,
    pub T: f64, pub has_energy_bin: i32, pub pad1: i32, pub energy_bin: f64,
    pub has_min_allowed: i32, pub has_max_allowed: i32, pub min_allowed: f64, pub max_allowed: f64,
    pub e_lo: f64, pub e_hi: f64, pub acceptance_rate_mode: i32, pub pad2: i32,
    pub target_rate: f64, pub translation_scale: f64, pub well_width: f64, pub seed: u64,
    pub descent_limit: u64, pub lanes_per_walker: i32, pub resum_interval: i32, pub drift_tol: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct sadmc_geometry { pub n: i32, pub pad: i32, pub radius: f64, pub box_: [f64; 3] }

#[repr(C)]
pub struct sadmc_proposal { pub which: i32, pub j: i32, pub g: [f64; 3], pub scale: f64 }

pub enum sadmc_handle {}

#[link(name = "sadmc_gb300")]
extern "C" {
    pub fn sadmc_last_error() -> *const c_char;
    pub fn sadmc_create(cfg: *const sadmc_config, geom: *const sadmc_geometry,
                        out: *mut *mut sadmc_handle) -> i32;
    pub fn sadmc_destroy(h: *mut sadmc_handle) -> i32;
    pub fn sadmc_upload_state(h: *mut sadmc_handle, begin: i32, count: i32, state: *const f64) -> i32;
    pub fn sadmc_initialize(h: *mut sadmc_handle) -> i32;
    pub fn sadmc_run(h: *mut sadmc_handle, moves: u64) -> i32;
    pub fn sadmc_energy(h: *mut sadmc_handle, e: *mut f64) -> i32;
    pub fn sadmc_compute_energy(h: *mut sadmc_handle, e: *mut f64) -> i32;
    pub fn sadmc_plan_move_injected(h: *mut sadmc_handle, walker: i32, p: *const sadmc_proposal,
                                    e: *mut f64, possible: *mut i32) -> i32;
    pub fn sadmc_confirm(h: *mut sadmc_handle, walker: i32) -> i32;
    pub fn sadmc_nbins(h: *mut sadmc_handle, walker: i32, n: *mut i64, min: *mut f64, w: *mut f64) -> i32;
    pub fn sadmc_read_bins(h: *mut sadmc_handle, walker: i32, lnw: *mut f64, hist: *mut u64,
                           t_found: *mut u64, e_tot: *mut f64, e2_tot: *mut f64,
                           round_trips: *mut u64, visited: *mut u8) -> i32;
    pub fn sadmc_counters(h: *mut sadmc_handle, moves: *mut u64, accepted: *mut u64) -> i32;
    pub fn sadmc_status(h: *mut sadmc_handle, flags: *mut u32) -> i32;
}

/// A GPU batch of EnergyMC walkers; replaces `loop { mc.move_once() }`.
pub struct GpuBatch { h: *mut sadmc_handle, pub n_walkers: usize }

impl GpuBatch {
    pub fn new(cfg: &sadmc_config, geom: &[sadmc_geometry], state: &[f64]) -> Result<Self, String> {
        let mut h = std::ptr::null_mut();
        unsafe {
            check(sadmc_create(cfg, geom.as_ptr(), &mut h))?;
            let b = GpuBatch { h, n_walkers: geom.len() };
            check(sadmc_upload_state(h, 0, geom.len() as i32, state.as_ptr()))?;
            check(sadmc_initialize(h))?;
            Ok(b)
        }
    }
    pub fn run(&mut self, moves: u64) -> Result<(), String> { unsafe { check(sadmc_run(self.h, moves)) } }
    pub fn energies(&self) -> Result<Vec<f64>, String> {
        let mut e = vec![0.0; self.n_walkers];
        unsafe { check(sadmc_energy(self.h, e.as_mut_ptr()))?; }
        Ok(e)
    }
}
impl Drop for GpuBatch { fn drop(&mut self) { unsafe { sadmc_destroy(self.h); } } }

fn check(rc: i32) -> Result<(), String> {
    if rc == 0 { return Ok(()); }
    let msg = unsafe { std::ffi::CStr::from_ptr(sadmc_last_error()) };
    Err(format!("sadmc error {}: {}", rc, msg.to_string_lossy()))
}

// ---- the rest of the surface ------------------------------------------------------

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct sadmc_grand_config {
    pub method: i32, pub n_walkers: i32, pub max_N: i32, pub acceptance_rate_mode: i32,
    pub t0: f64, pub energy_bin: f64, pub radius: f64,
    pub has_min_allowed: i32, pub has_max_allowed: i32, pub min_allowed: f64, pub max_allowed: f64,
    pub target_rate: f64, pub translation_scale: f64, pub addremove_probability: f64,
    pub e_lo: f64, pub e_hi: f64, pub seed: u64, pub resum_interval: i32, pub system: i32,
    pub drift_tol: f64, pub box_: [f64; 3], pub lanes_per_walker: i32,
}
pub enum sadmc_grand {}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct sadmc_online {
    pub collect_interval: u64, pub retrain_interval: u64, pub train_steps: i32, pub batch: i32,
    pub lr: f32, pub pad: i32, pub seed: u64,
}

#[link(name = "sadmc_gb300")]
extern "C" {
    pub fn sadmc_version() -> i32;
    pub fn sadmc_read_state(h: *mut sadmc_handle, begin: i32, count: i32, state: *mut f64) -> i32;
    pub fn sadmc_run_async(h: *mut sadmc_handle, moves: u64, cuda_stream: *mut c_void) -> i32;
    pub fn sadmc_synchronize(h: *mut sadmc_handle) -> i32;
    pub fn sadmc_plane_bins(h: *mut sadmc_handle, plane_bins: *mut i64) -> i32;
    pub fn sadmc_read_planes(h: *mut sadmc_handle, lnw: *mut f64, hist: *mut u64, range: *mut i32,
                             bins_min: *mut f64) -> i32;
    pub fn sadmc_read_wl_hist(h: *mut sadmc_handle, walker: i32, hist: *mut u64, n: *mut i64,
                              min_energy: *mut f64) -> i32;
    pub fn sadmc_read_extra(h: *mut sadmc_handle, walker: i32, count: *mut u64, total: *mut f64) -> i32;
    pub fn sadmc_read_scalars(h: *mut sadmc_handle, walker: i32, out: *mut f64) -> i32;
    pub fn sadmc_set_trace(h: *mut sadmc_handle, capacity: u64) -> i32;
    pub fn sadmc_read_trace(h: *mut sadmc_handle, walker: i32, e1: *mut f64, e2: *mut f64,
                            count: *mut u64) -> i32;
    pub fn sadmc_read_trace_ds(h: *mut sadmc_handle, walker: i32, ds: *mut f32, count: *mut u64) -> i32;
    pub fn sadmc_lanes_per_walker(h: *mut sadmc_handle) -> i32;
    pub fn sadmc_autotune(h: *mut sadmc_handle, moves: u64, best_lpw: *mut i32, best_ms: *mut f64) -> i32;
    pub fn sadmc_checkpoint(h: *mut sadmc_handle, path: *const c_char) -> i32;
    pub fn sadmc_resume(path: *const c_char, out: *mut *mut sadmc_handle) -> i32;
    pub fn sadmc_get_config(h: *mut sadmc_handle, cfg: *mut sadmc_config, geom: *mut sadmc_geometry) -> i32;
    pub fn sadmc_surrogate_init(h: *mut sadmc_handle, seed: u64, ring_capacity: i32) -> i32;
    pub fn sadmc_surrogate_get_params(h: *mut sadmc_handle, params: *mut f32) -> i32;
    pub fn sadmc_surrogate_set_params(h: *mut sadmc_handle, params: *const f32) -> i32;
    pub fn sadmc_surrogate_collect(h: *mut sadmc_handle, ring_count: *mut i32) -> i32;
    pub fn sadmc_surrogate_train(h: *mut sadmc_handle, steps: i32, batch: i32, lr: f32, seed: u64,
                                 loss: *mut f64) -> i32;
    pub fn sadmc_surrogate_loss_grads(h: *mut sadmc_handle, pos: *const f32, target: *const f32,
                                      configs: i32, loss: *mut f64, grads: *mut f32) -> i32;
    pub fn sadmc_surrogate_loss_grads_noalloc(h: *mut sadmc_handle, pos: *const f32, target: *const f32,
                                              configs: i32, loss: *mut f64, grads: *mut f32,
                                              stream: *mut c_void) -> i32;
    pub fn sadmc_run_da(h: *mut sadmc_handle, moves: u64, refresh_interval: i32, stats: *mut u64) -> i32;
    pub fn sadmc_run_online(h: *mut sadmc_handle, moves: u64, delayed: i32, refresh_interval: i32,
                            o: *const sadmc_online, stats: *mut u64) -> i32;
    pub fn sadmc_surrogate_predict(h: *mut sadmc_handle, pos: *const f32, configs: i32,
                                   energies: *mut f32) -> i32;
    pub fn sadmc_check_numerics(n: u64, seed: u64, mismatches: *mut u64, first: *mut f64) -> i32;
    pub fn sadmc_draws(system: i32, n: u32, seed: u64, walker: u32, t0: u64, count: i32,
                       stream_pair: u32, idx2: *mut u32, g3: *mut f32, u: *mut f64) -> i32;
    pub fn sadmc_heat_capacity(t: *const f64, n_t: i32, e: *const f64, s: *const f64, n: i32,
                               c: *mut f64) -> i32;
    pub fn sadmc_walker_heat_capacity(h: *mut sadmc_handle, t: *const f64, n_t: i32, c: *mut f64) -> i32;
    pub fn sadmc_grand_create(cfg: *const sadmc_grand_config, out: *mut *mut sadmc_grand) -> i32;
    pub fn sadmc_grand_destroy(h: *mut sadmc_grand) -> i32;
    pub fn sadmc_grand_run(h: *mut sadmc_grand, moves: u64) -> i32;
    pub fn sadmc_grand_set_trace(h: *mut sadmc_grand, capacity: u64) -> i32;
    pub fn sadmc_grand_read_trace(h: *mut sadmc_grand, walker: i32, e1: *mut f64, e2: *mut f64,
                                  n: *mut u64) -> i32;
    pub fn sadmc_grand_read_state(h: *mut sadmc_grand, walker: i32, pos: *mut f64, n: *mut i32) -> i32;
    pub fn sadmc_grand_read_scalars(h: *mut sadmc_grand, walker: i32, out: *mut f64) -> i32;
    pub fn sadmc_grand_read_bins(h: *mut sadmc_grand, walker: i32, lnw: *mut f64, hist: *mut u64,
                                 wl_hist: *mut u64, visited: *mut u8, round_trips: *mut u64,
                                 n_e: *mut i64, n_n: *mut i64) -> i32;
    pub fn sadmc_grand_translation_counts(h: *mut sadmc_grand, walker: i32, attempts: *mut u64,
                                          accepted: *mut u64) -> i32;
}
