//! `solve_ensemble`: many `IVP::ode(&sys, t0, tf, y0).method(m).solve()` calls in one GPU call.
//!
//! A system opts in by naming its CUDA twin (`DeviceOde::RHS_ID`, a built-in family of libdegpu or
//! an id returned by `register_nvrtc`) and exporting its fields as parameters.  Results come back
//! as the crate's own `Result<Solution, Error>` per instance.
use degpu_sys as sys;
use differential_equations::prelude::*;

/// An `ODE` whose right-hand side exists on the device.
pub trait DeviceOde<const N: usize>: ODE<f64, [f64; N]> {
    const RHS_ID: i32;
    const N_PARAMS: usize;
    fn params(&self) -> Vec<f64>;
}

/// Method settings, mirroring `ExplicitRungeKutta`'s constructors and setters.
#[derive(Clone, Copy)]
pub struct Method {
    pub cfg: sys::degpu_method_cfg,
    pub rtol: f64,
    pub atol: f64,
}

impl Method {
    fn new(m: i32) -> Self {
        let mut cfg = unsafe { std::mem::zeroed::<sys::degpu_method_cfg>() };
        unsafe { sys::degpu_default_cfg(&mut cfg, m) };
        Method { cfg, rtol: 1e-6, atol: 1e-6 }
    }
    pub fn rk4(h0: f64) -> Self { let mut m = Self::new(sys::DEGPU_RK4); m.cfg.h0 = h0; m }
    pub fn dopri5() -> Self { Self::new(sys::DEGPU_DOPRI5) }
    pub fn dop853() -> Self { Self::new(sys::DEGPU_DOP853) }
    pub fn rkf45() -> Self { Self::new(sys::DEGPU_RKF45) }
    pub fn cash_karp() -> Self { Self::new(sys::DEGPU_CASH_KARP) }
    pub fn rkv655e() -> Self { Self::new(sys::DEGPU_RKV655E) }
    pub fn rkv656e() -> Self { Self::new(sys::DEGPU_RKV656E) }
    pub fn rkv766e() -> Self { Self::new(sys::DEGPU_RKV766E) }
    pub fn rkv767e() -> Self { Self::new(sys::DEGPU_RKV767E) }
    pub fn rkv877e() -> Self { Self::new(sys::DEGPU_RKV877E) }
    pub fn rkv878e() -> Self { Self::new(sys::DEGPU_RKV878E) }
    pub fn rkv988e() -> Self { Self::new(sys::DEGPU_RKV988E) }
    pub fn rkv989e() -> Self { Self::new(sys::DEGPU_RKV989E) }
    pub fn rtol(mut self, v: f64) -> Self { self.rtol = v; self }
    pub fn atol(mut self, v: f64) -> Self { self.atol = v; self }
    pub fn max_steps(mut self, v: i64) -> Self { self.cfg.max_steps = v; self }
    pub fn precision(mut self, p: i32) -> Self { self.cfg.precision = p; self }
}

/// One solve per (system, t0, tf, y0), all on the GPU.
pub fn solve_ensemble<S: DeviceOde<N>, const N: usize>(
    problems: &[(&S, f64, f64, [f64; N])],
    method: Method,
) -> Vec<Result<Solution<f64, [f64; N]>, Error<f64, [f64; N]>>> {
    let n = problems.len();
    let np = S::N_PARAMS;
    let mut t0 = vec![0.0; n];
    let mut tf = vec![0.0; n];
    let mut y0 = vec![0.0; N * n];
    let mut params = vec![0.0; np.max(1) * n];
    for (i, (s, a, b, y)) in problems.iter().enumerate() {
        t0[i] = *a;
        tf[i] = *b;
        for c in 0..N { y0[c * n + i] = y[c]; }
        for (q, v) in s.params().iter().enumerate() { params[q * n + i] = *v; }
    }
    let rtol = vec![method.rtol; n];
    let atol = vec![method.atol; n];
    let (mut yf, mut tfin) = (vec![0.0; N * n], vec![0.0; n]);
    let (mut acc, mut rej, mut fev, mut st) = (vec![0i64; n], vec![0i64; n], vec![0i64; n], vec![0i32; n]);
    let pb = sys::degpu_problem { rhs_id: S::RHS_ID, dim: N as i32, n_params: np as i32, reserved: 0 };
    let inp = sys::degpu_batch_in {
        n: n as i64, t0: t0.as_ptr(), tf: tf.as_ptr(), y0: y0.as_ptr(), params: params.as_ptr(),
        rtol: rtol.as_ptr(), atol: atol.as_ptr(), dims: std::ptr::null(), family: std::ptr::null(),
        t_eval: std::ptr::null(), n_eval: 0, reserved: 0,
    };
    let mut out = sys::degpu_batch_out {
        y_final: yf.as_mut_ptr(), t_final: tfin.as_mut_ptr(), dense: std::ptr::null_mut(),
        accepted: acc.as_mut_ptr(), rejected: rej.as_mut_ptr(), fevals: fev.as_mut_ptr(), status: st.as_mut_ptr(),
    };
    let rc = unsafe { sys::degpu_solve_ensemble_host(&pb, &method.cfg, &inp, &mut out) };
    assert_eq!(rc, sys::DEGPU_OK, "degpu_solve_ensemble_host failed");
    (0..n).map(|i| {
        let mut y = [0.0; N];
        for c in 0..N { y[c] = yf[c * n + i]; }
        match st[i] {
            sys::DEGPU_COMPLETE => {
                let mut s = Solution::new();
                s.push(tfin[i], y);
                s.evals.function = fev[i] as usize;
                s.steps.accepted = acc[i] as usize;
                s.steps.rejected = rej[i] as usize;
                s.status = Status::Complete;
                Ok(s)
            }
            sys::DEGPU_ERR_MAX_STEPS => Err(Error::MaxSteps { t: tfin[i], y }),
            sys::DEGPU_ERR_STEP_SIZE => Err(Error::StepSize { t: tfin[i], y }),
            sys::DEGPU_ERR_STIFFNESS => Err(Error::Stiffness { t: tfin[i], y }),
            _ => Err(Error::BadInput { msg: "Invalid input: step size or integration interval".to_string() }),
        }
    }).collect()
}
