//! Raw bindings of include/degpu.h.  Every pointer in `BatchIn`/`BatchOut` is a device pointer for
//! `degpu_solve_ensemble` and a host pointer for `degpu_solve_ensemble_host`.
#![allow(non_camel_case_types)]
use std::os::raw::{c_char, c_int, c_void};

pub type degpu_status = c_int;
pub const DEGPU_OK: degpu_status = 0;
pub const DEGPU_BAD_INPUT: degpu_status = 1;

pub const DEGPU_RK4: i32 = 0;
pub const DEGPU_DOPRI5: i32 = 1;
pub const DEGPU_DOP853: i32 = 2;
pub const DEGPU_FP64_PARITY: i32 = 0;
pub const DEGPU_FP64_FAST: i32 = 1;
pub const DEGPU_MIXED: i32 = 2;

pub const DEGPU_COMPLETE: i32 = 0;
pub const DEGPU_ERR_BAD_INPUT: i32 = 1;
pub const DEGPU_ERR_MAX_STEPS: i32 = 2;
pub const DEGPU_ERR_STEP_SIZE: i32 = 3;
pub const DEGPU_ERR_STIFFNESS: i32 = 4;

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct degpu_method_cfg {
    pub method: i32,
    pub precision: i32,
    pub kernel: i32,
    pub dense_mode: i32,
    pub h0: f64,
    pub h_min: f64,
    pub h_max: f64,
    pub max_steps: i64,
    pub safety_factor: f64,
    pub min_scale: f64,
    pub max_scale: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct degpu_problem {
    pub rhs_id: i32,
    pub dim: i32,
    pub n_params: i32,
    pub reserved: i32,
}

#[repr(C)]
pub struct degpu_batch_in {
    pub n: i64,
    pub t0: *const f64,
    pub tf: *const f64,
    pub y0: *const f64,
    pub params: *const f64,
    pub rtol: *const f64,
    pub atol: *const f64,
    pub dims: *const i32,
    pub family: *const i32,
    pub t_eval: *const f64,
    pub n_eval: i32,
    pub reserved: i32,
}

#[repr(C)]
pub struct degpu_batch_out {
    pub y_final: *mut f64,
    pub t_final: *mut f64,
    pub dense: *mut f64,
    pub accepted: *mut i64,
    pub rejected: *mut i64,
    pub fevals: *mut i64,
    pub status: *mut i32,
}

extern "C" {
    pub fn degpu_default_cfg(cfg: *mut degpu_method_cfg, method: i32);
    pub fn degpu_rhs_info(rhs_id: i32, dim: *mut i32, n_params: *mut i32) -> degpu_status;
    pub fn degpu_solve_ensemble(pb: *const degpu_problem, cfg: *const degpu_method_cfg, inp: *const degpu_batch_in,
                                out: *mut degpu_batch_out, stream: *mut c_void) -> degpu_status;
    pub fn degpu_solve_ensemble_host(pb: *const degpu_problem, cfg: *const degpu_method_cfg,
                                     inp: *const degpu_batch_in, out: *mut degpu_batch_out) -> degpu_status;
    pub fn degpu_register_rhs_nvrtc(source: *const c_char, name: *const c_char, dim: i32, n_params: i32,
                                    rhs_id: *mut i32, log: *mut c_char, log_size: usize) -> degpu_status;
    pub fn degpu_status_string(s: degpu_status) -> *const c_char;
}
