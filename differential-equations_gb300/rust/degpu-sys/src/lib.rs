//! Raw bindings of include/degpu.h.  Every array pointer in `degpu_batch_in` / `degpu_batch_out`
//! (and the crossing, event and BVP outputs) is a device pointer for the stream-ordered entry
//! points and a host pointer for the `_host` ones.
#![allow(non_camel_case_types)]
use std::os::raw::{c_char, c_int, c_void};

pub type degpu_status = c_int;
pub const DEGPU_OK: degpu_status = 0;
pub const DEGPU_BAD_INPUT: degpu_status = 1;
pub const DEGPU_OOM: degpu_status = 2;
pub const DEGPU_TIMEOUT: degpu_status = 3;
pub const DEGPU_CUDA_ERROR: degpu_status = 4;
pub const DEGPU_UNSUPPORTED: degpu_status = 5;

// degpu_method
pub const DEGPU_RK4: i32 = 0;
pub const DEGPU_DOPRI5: i32 = 1;
pub const DEGPU_DOP853: i32 = 2;
pub const DEGPU_RKF45: i32 = 3;
pub const DEGPU_CASH_KARP: i32 = 4;
pub const DEGPU_RKV655E: i32 = 5;
pub const DEGPU_RKV656E: i32 = 6;
pub const DEGPU_RKV766E: i32 = 7;
pub const DEGPU_RKV767E: i32 = 8;
pub const DEGPU_RKV877E: i32 = 9;
pub const DEGPU_RKV878E: i32 = 10;
pub const DEGPU_RKV988E: i32 = 11;
pub const DEGPU_RKV989E: i32 = 12;

// degpu_precision, degpu_kernel, degpu_dense_mode
pub const DEGPU_FP64_PARITY: i32 = 0;
pub const DEGPU_FP64_FAST: i32 = 1;
pub const DEGPU_MIXED: i32 = 2;
pub const DEGPU_FP64_PLAIN: i32 = 3;
pub const DEGPU_MIXED_FP64_CTRL: i32 = 4;
pub const DEGPU_KERNEL_AUTO: i32 = 0;
pub const DEGPU_KERNEL_THREAD: i32 = 1;
pub const DEGPU_KERNEL_WARP: i32 = 2;
pub const DEGPU_KERNEL_PERSISTENT: i32 = 3;
pub const DEGPU_DENSE_REFERENCE: i32 = 0;
pub const DEGPU_DENSE_HAIRER: i32 = 1;

// degpu_instance_status
pub const DEGPU_COMPLETE: i32 = 0;
pub const DEGPU_ERR_BAD_INPUT: i32 = 1;
pub const DEGPU_ERR_MAX_STEPS: i32 = 2;
pub const DEGPU_ERR_STEP_SIZE: i32 = 3;
pub const DEGPU_ERR_STIFFNESS: i32 = 4;
pub const DEGPU_INTERRUPTED: i32 = 5;
pub const DEGPU_ERR_LINEAR_ALGEBRA: i32 = 6;

// degpu_crossing_direction, degpu_event_kind, degpu_bvp_method
pub const DEGPU_CROSS_BOTH: i32 = 0;
pub const DEGPU_CROSS_POSITIVE: i32 = 1;
pub const DEGPU_CROSS_NEGATIVE: i32 = -1;
pub const DEGPU_HYPERPLANE_MAX_DIM: usize = 8;
pub const DEGPU_EVENT_MAX_TERMS: usize = 8;
pub const DEGPU_EVENT_LINEAR: i32 = 0;
pub const DEGPU_EVENT_MAX_ABS: i32 = 1;
pub const DEGPU_BVP_SINGLE: i32 = 0;
pub const DEGPU_BVP_MULTIPLE: i32 = 1;
pub const DEGPU_BVP_MAX_UNKNOWNS: usize = 64;
pub const DEGPU_NOALLOC_MAX_INSTANCES: i64 = 262144;

// degpu_pde_id, degpu_bc_kind
pub const DEGPU_MOL_MAX_FIELDS: usize = 4;
pub const DEGPU_MOL_MAX_PARAMS: usize = 8;
pub const DEGPU_PDE_DIFFUSION: i32 = 1;
pub const DEGPU_PDE_COUPLED_DIFFUSION: i32 = 2;
pub const DEGPU_PDE_GRAY_SCOTT: i32 = 3;
pub const DEGPU_BC_DIRICHLET: i32 = 0;
pub const DEGPU_BC_NEUMANN: i32 = 1;
pub const DEGPU_BC_PERIODIC: i32 = 2;

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
    pub rtol_vec: *const f64,
    pub atol_vec: *const f64,
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

/// `.crossing(component, threshold, direction)`
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct degpu_crossing {
    pub component: i32,
    pub direction: i32,
    pub max_points: i32,
    pub reserved: i32,
    pub threshold: f64,
}

/// Crossing, hyperplane and event points: t [max_points][n], y [max_points][dim][n], count [n].
#[repr(C)]
pub struct degpu_crossing_out {
    pub t: *mut f64,
    pub y: *mut f64,
    pub count: *mut i32,
}

/// `.hyperplane_crossing(point, normal, extractor, direction)`, the extractor as components.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct degpu_hyperplane {
    pub dim: i32,
    pub direction: i32,
    pub max_points: i32,
    pub reserved: i32,
    pub components: [i32; DEGPU_HYPERPLANE_MAX_DIM],
    pub point: [f64; DEGPU_HYPERPLANE_MAX_DIM],
    pub normal: [f64; DEGPU_HYPERPLANE_MAX_DIM],
}

/// `.event(&event)`: `Event::event` as a linear or max-of-absolute-values form.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct degpu_event {
    pub kind: i32,
    pub direction: i32,
    pub terminate: i32,
    pub max_points: i32,
    pub n_terms: i32,
    pub reserved: i32,
    pub components: [i32; DEGPU_EVENT_MAX_TERMS],
    pub weights: [f64; DEGPU_EVENT_MAX_TERMS],
    pub t_weight: f64,
    pub offset: f64,
}

/// `BVP::ode(..).method(Shooting::single | Shooting::multiple)`: rows r_i = y_side[component] - value.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct degpu_bvp {
    pub method: i32,
    pub segments: i32,
    pub max_iterations: i32,
    pub reserved: i32,
    pub tolerance: f64,
    pub side: [i32; DEGPU_HYPERPLANE_MAX_DIM],
    pub component: [i32; DEGPU_HYPERPLANE_MAX_DIM],
    pub value: [f64; DEGPU_HYPERPLANE_MAX_DIM],
}

#[repr(C)]
pub struct degpu_bvp_out {
    pub y_a: *mut f64,
    pub iterations: *mut i32,
    pub jacobian: *mut i64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct degpu_gray_scott {
    pub nx: i32,
    pub ny: i32,
    pub dx: f64,
    pub du: f64,
    pub dv: f64,
    pub f: f64,
    pub k: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct degpu_mol {
    pub pde_id: i32,
    pub dims: i32,
    pub fields: i32,
    pub reserved: i32,
    pub nodes: [i32; 2],
    pub lower: [f64; 2],
    pub dx: [f64; 2],
    pub bc_kind: [[i32; 2]; 2],
    pub bc_value: [[[f64; DEGPU_MOL_MAX_FIELDS]; 2]; 2],
    pub params: [f64; DEGPU_MOL_MAX_PARAMS],
}

#[repr(C)]
pub struct degpu_server {
    _private: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct degpu_server_cfg {
    pub memory_budget_bytes: u64,
    pub max_active: i32,
    pub round_budget: i32,
}

extern "C" {
    pub fn degpu_default_cfg(cfg: *mut degpu_method_cfg, method: i32);
    pub fn degpu_set_mixed_min_rtol(method: i32, min_rtol: f64) -> degpu_status;
    pub fn degpu_mixed_min_rtol(method: i32) -> f64;
    pub fn degpu_rhs_info(rhs_id: i32, dim: *mut i32, n_params: *mut i32) -> degpu_status;
    pub fn degpu_solve_ensemble(pb: *const degpu_problem, cfg: *const degpu_method_cfg, inp: *const degpu_batch_in,
                                out: *mut degpu_batch_out, stream: *mut c_void) -> degpu_status;
    pub fn degpu_solve_ensemble_noalloc(pb: *const degpu_problem, cfg: *const degpu_method_cfg,
                                        inp: *const degpu_batch_in, out: *mut degpu_batch_out,
                                        stream: *mut c_void) -> degpu_status;
    pub fn degpu_solve_ensemble_host(pb: *const degpu_problem, cfg: *const degpu_method_cfg,
                                     inp: *const degpu_batch_in, out: *mut degpu_batch_out) -> degpu_status;
    pub fn degpu_solve_ensemble_crossing(pb: *const degpu_problem, cfg: *const degpu_method_cfg,
                                         inp: *const degpu_batch_in, crossing: *const degpu_crossing,
                                         out: *mut degpu_batch_out, crossing_out: *mut degpu_crossing_out,
                                         stream: *mut c_void) -> degpu_status;
    pub fn degpu_solve_ensemble_crossing_host(pb: *const degpu_problem, cfg: *const degpu_method_cfg,
                                              inp: *const degpu_batch_in, crossing: *const degpu_crossing,
                                              out: *mut degpu_batch_out,
                                              crossing_out: *mut degpu_crossing_out) -> degpu_status;
    pub fn degpu_solve_ensemble_hyperplane(pb: *const degpu_problem, cfg: *const degpu_method_cfg,
                                           inp: *const degpu_batch_in, plane: *const degpu_hyperplane,
                                           out: *mut degpu_batch_out, crossing_out: *mut degpu_crossing_out,
                                           stream: *mut c_void) -> degpu_status;
    pub fn degpu_solve_ensemble_hyperplane_host(pb: *const degpu_problem, cfg: *const degpu_method_cfg,
                                                inp: *const degpu_batch_in, plane: *const degpu_hyperplane,
                                                out: *mut degpu_batch_out,
                                                crossing_out: *mut degpu_crossing_out) -> degpu_status;
    pub fn degpu_solve_ensemble_event(pb: *const degpu_problem, cfg: *const degpu_method_cfg,
                                      inp: *const degpu_batch_in, event: *const degpu_event,
                                      out: *mut degpu_batch_out, event_out: *mut degpu_crossing_out,
                                      stream: *mut c_void) -> degpu_status;
    pub fn degpu_solve_ensemble_event_host(pb: *const degpu_problem, cfg: *const degpu_method_cfg,
                                           inp: *const degpu_batch_in, event: *const degpu_event,
                                           out: *mut degpu_batch_out,
                                           event_out: *mut degpu_crossing_out) -> degpu_status;
    pub fn degpu_solve_bvp_host(pb: *const degpu_problem, cfg: *const degpu_method_cfg, inp: *const degpu_batch_in,
                                bvp: *const degpu_bvp, out: *mut degpu_batch_out,
                                bvp_out: *mut degpu_bvp_out) -> degpu_status;
    pub fn degpu_eval_rhs(rhs_id: i32, precision: i32, n: i64, dim: i32, n_params: i32, t: *const f64,
                          y: *const f64, params: *const f64, dydt: *mut f64, stream: *mut c_void) -> degpu_status;
    pub fn degpu_register_rhs_nvrtc(source: *const c_char, name: *const c_char, dim: i32, n_params: i32,
                                    rhs_id: *mut i32, log: *mut c_char, log_size: usize) -> degpu_status;
    pub fn degpu_gray_scott_rk4(gs: *const degpu_gray_scott, precision: i32, t0: f64, dt: f64, steps: i64,
                                u: *mut c_void, v: *mut c_void, stream: *mut c_void) -> degpu_status;
    pub fn degpu_gray_scott_rhs(gs: *const degpu_gray_scott, u: *const f64, v: *const f64, du: *mut f64,
                                dv: *mut f64, stream: *mut c_void) -> degpu_status;
    pub fn degpu_mol_rhs(mol: *const degpu_mol, precision: i32, t: f64, y: *const c_void, dydt: *mut c_void,
                         stream: *mut c_void) -> degpu_status;
    pub fn degpu_mol_rk4(mol: *const degpu_mol, precision: i32, t0: f64, tf: f64, h: f64, y: *mut c_void,
                         steps: *mut i64, stream: *mut c_void) -> degpu_status;
    pub fn degpu_server_create(cfg: *const degpu_server_cfg, server: *mut *mut degpu_server) -> degpu_status;
    pub fn degpu_server_submit(server: *mut degpu_server, pb: *const degpu_problem, cfg: *const degpu_method_cfg,
                               inp: *const degpu_batch_in, out: *mut degpu_batch_out,
                               request_id: *mut u64) -> degpu_status;
    pub fn degpu_server_poll(server: *mut degpu_server, request_id: u64, done: *mut i32,
                             latency_ms: *mut f64) -> degpu_status;
    pub fn degpu_server_wait(server: *mut degpu_server, request_id: u64, latency_ms: *mut f64) -> degpu_status;
    pub fn degpu_server_destroy(server: *mut degpu_server) -> degpu_status;
    pub fn degpu_status_string(s: degpu_status) -> *const c_char;
    pub fn degpu_version() -> *const c_char;
}
