// group_erk.cuh — G-lanes-per-system explicit Runge–Kutta solve for systems of up to a few
// hundred components whose size varies per instance (the FPU-beta chain family).
//
// Layout: a group of G lanes (G = 8, 16 or 32; 32/G systems per warp) owns one instance;
// component c lives in lane c % G, slot c / G (CPL slots per lane, d <= G*CPL).  The stage
// vectors k[0..I), the stage state handed to the right-hand side and the dense coefficients are
// in shared memory, [vector][component] per system, so lane-strided accesses are conflict free.
// The state y (and its Kahan compensation) stays in registers.  The groups are persistent: a
// group whose instance finishes takes the next one from a device work queue.
//
// Arithmetic mirrors erk_core.cuh (and through it the crate, src/methods/erk/dormandprince/
// ordinary.rs:63-337, src/ode/solve_ivp.rs:138-277) component by component.  The two
// reductions over components — the error norm (src/traits.rs:394-410) and the stiffness
// numerators — are summed by the group leader in component order on the parity path, so results
// are bitwise those of the crate's sequential loop; the FP64_FAST and MIXED paths use a
// shuffle-tree reduction.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <tuple>
#include <vector>

#include "registry.cuh"
#include "side_paths.cuh"

namespace degpu {

struct GroupArgs {
    EnsArgs a;
    const int32_t* dims;  // per-instance dimension
};

// FPU-beta right-hand side for the components this lane owns; `sy` is the stage state.
template <class P, int G, int CPL>
__device__ __forceinline__ void fpu_rhs(const typename P::S* sy, typename P::S* out, int d, int lane,
                                        typename P::S b) {
    using S = typename P::S;
    const int m = d / 2;
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        int c = lane + G * j;
        if (c >= d) break;
        if (c < m) {
            out[j] = sy[m + c];
        } else {
            int i = c - m;
            S xi = sy[i];
            S xprev = i > 0 ? sy[i - 1] : (S)0;
            S xnext = i + 1 < m ? sy[i + 1] : (S)0;
            S dprev = xi - xprev;
            S dcur = xnext - xi;
            out[j] = (dcur - dprev) + b * (dcur * dcur * dcur - dprev * dprev * dprev);
        }
    }
}

// Scalars of a group-per-system solve parked between serving rounds; the slot continues with the
// lane-distributed vectors (GroupLane::park).
struct GroupPark {
    int32_t phase;  // 0 not started, 1 in progress, 2 finished
    int32_t d, stiff, nonstiff, next_eval, status, last_rejected, pad;
    int64_t inst, steps, acc, rej, fev;
    double t, tf, h, h_prev, t_prev, dir, rtol, atol, beta;
};

template <class Tab, class P, int G, int CPL, bool DENSE>
struct GroupLane {
    static constexpr int DG = G * CPL;
    static constexpr int I = Tab::I;
    static constexpr int NS = Tab::S;
    static constexpr int O = Tab::ORDER;
    static constexpr int NC = DENSE ? O : 1;
    using S = typename P::S;
    using AccT = typename AccOf<S>::type;  // stage sums: S itself, or a lazily normalised pair

    // shared memory of this system
    S* k;     // [I][DG]
    S* sy;    // [DG]   stage state / scratch vector
    S* cont;  // [NC][DG]
    double* red;  // [DG] per-component terms for the ordered reduction

    int lane;          // 0..G-1
    unsigned gmask;    // lanes of this group
    int d;
    int64_t inst;
    double t, tf, h, h_prev, t_prev, dir, rtol, atol, beta;
    // pair stages: h as a pair, formed once per step attempt, and FP32 copies of the tolerances
    // (their error terms, norm terms and stiffness terms are FP32, widened for the FP64 sums)
    S hc;
    float rtolf, atolf;
    S betas;  // beta in the stage arithmetic, converted once per instance
    S y[CPL], yc[CPL];
    int64_t steps, acc, rej, fev;
    int stiff, nonstiff, next_eval, status;
    bool last_rejected, done;

    __device__ __forceinline__ void sync() const { __syncwarp(gmask); }

    // Tolerances of component c (src/tolerance.rs:33-40): per component when the batch has them.
    __device__ __forceinline__ double rtol_c(int c, const EnsArgs& a) const {
        return a.rtol_vec ? a.rtol_vec[(int64_t)c * a.n + inst] : rtol;
    }
    __device__ __forceinline__ double atol_c(int c, const EnsArgs& a) const {
        return a.atol_vec ? a.atol_vec[(int64_t)c * a.n + inst] : atol;
    }

    // sum of red[0..d) — in component order on the parity path
    __device__ double reduce_terms(const double* terms) {
        if constexpr (P::ID == PrecParity::ID) {
#pragma unroll
            for (int j = 0; j < CPL; ++j) {
                int c = lane + G * j;
                if (c < d) red[c] = terms[j];
            }
            sync();
            double s = 0.0;
            if (lane == 0)
                for (int c = 0; c < d; ++c) s = s + red[c];
            s = __shfl_sync(gmask, s, 0, G);
            sync();
            return s;
        } else {
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < CPL; ++j)
                if (lane + G * j < d) s += terms[j];
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(gmask, s, o, G);
            return s;
        }
    }

    // dydt of the lane's components at state sy (all lanes of the group call it together)
    // the per-instance values derived from rtol, atol and beta
    __device__ __forceinline__ void set_derived() {
        betas = (S)beta;
        if constexpr (P::PAIR) {
            rtolf = narrow_rz(rtol);
            atolf = narrow_rz(atol);
        }
    }

    __device__ __forceinline__ void rhs(S* out) { fpu_rhs<P, G, CPL>(sy, out, d, lane, betas); }

    __device__ __forceinline__ S stage_coef(double aij) const {
        if constexpr (P::PAIR)
            return df(aij) * hc;  // the pairs nearest to a_ij and h
        else if constexpr (P::KAHAN)
            return (float)aij * (float)h;
        else
            return aij * h;
    }

    __device__ void initial_step(double t0, const EnsArgs& a, S* f0) {
        double posneg = rs_signum(tf - t0);
        // f0 = f(t0, y0)
#pragma unroll
        for (int j = 0; j < CPL; ++j)
            if (lane + G * j < d) sy[lane + G * j] = y[j];
        sync();
        rhs(f0);
        sync();
        fev += 1;
        double tf_[CPL], ty_[CPL], sk[CPL];
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            const int c = lane + G * j < d ? lane + G * j : 0;
            sk[j] = atol_c(c, a) + rtol_c(c, a) * fabs(to_f64(y[j]));
            double q = to_f64(f0[j]) / sk[j];
            tf_[j] = q * q;
            double r = to_f64(y[j]) / sk[j];
            ty_[j] = r * r;
        }
        double dnf = reduce_terms(tf_);
        double dny = reduce_terms(ty_);
        double hh;
        if (dnf <= 1.0e-10 || dny <= 1.0e-10)
            hh = 1.0e-6;
        else
            hh = sqrt(dny / dnf) * 0.01;
        hh = fmin(hh, a.h_max);
        hh = hh * posneg;
        S hs = P::from(hh);
#pragma unroll
        for (int j = 0; j < CPL; ++j)
            if (lane + G * j < d) sy[lane + G * j] = y[j] + hs * f0[j];
        sync();
        S f1[CPL];
        rhs(f1);
        sync();
        fev += 1;
        double q2[CPL];
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            double q = (to_f64(f1[j]) - to_f64(f0[j])) / sk[j];
            q2[j] = q * q;
        }
        double der2 = reduce_terms(q2);
        der2 = sqrt(der2) / fabs(hh);
        double der12 = fmax(sqrt(dnf), der2);
        double h1;
        if (der12 <= 1.0e-15)
            h1 = fabs(hh) * fmax(1.0e-3, 1.0e-6);
        else
            h1 = P::pow(0.01 / der12, 1.0 / (double)O);
        double interval = fabs(tf - t0);
        hh = fmin(fmax(fmin(fmin(fabs(hh) * 100.0, h1), a.h_max), a.h_min), interval);
        h = hh * posneg;
    }

    __device__ __forceinline__ double eval_time(int idx, const EnsArgs& a) const {
        return dir > 0.0 ? a.t_eval[idx] : a.t_eval[a.n_eval - 1 - idx];
    }
    __device__ __forceinline__ int eval_slot(int idx, const EnsArgs& a) const {
        return dir > 0.0 ? a.eval_perm[idx] : a.eval_perm[a.n_eval - 1 - idx];
    }
    __device__ void write_dense(int idx, const S* v, const EnsArgs& a) const {
        int slot = eval_slot(idx, a);
        double* out = a.dense + ((int64_t)slot * a.dmax) * a.n + inst;
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            int c = lane + G * j;
            if (c < d) out[(int64_t)c * a.n] = to_f64(v[j]);
        }
    }
    __device__ void interpolate(double te, S* out, const EnsArgs& a) const {
        if constexpr (DENSE) {
            double s = (te - t_prev) / h_prev;
            double s1 = 1.0 - s;
            S ss = P::from(s), ss1 = P::from(s1);
            const bool hairer = a.dense_mode == DEGPU_DENSE_HAIRER;
#pragma unroll
            for (int j = 0; j < CPL; ++j) {
                int c = lane + G * j;
                if (c >= d) break;
                S accv = cont[(O - 1) * DG + c];
#pragma unroll
                for (int i = O - 2; i >= 1; --i) {
                    S f;
                    if (i >= 4) {
                        bool odd = ((O - 1 - i) % 2) == 1;
                        if (hairer) odd = !odd;
                        f = odd ? ss1 : ss;
                    } else {
                        f = (i % 2 == 1) ? ss1 : ss;
                    }
                    accv = accv * f;
                    accv = accv + cont[i * DG + c];
                }
                out[j] = cont[c] + ss * accv;
            }
        }
    }
    __device__ void solout(const EnsArgs& a) {
        if constexpr (DENSE) {
            int idx = next_eval;
            while (idx < a.n_eval) {
                double te = eval_time(idx, a);
                bool in_range = dir > 0.0 ? ((te == t_prev && idx == 0) || (te > t_prev && te <= t))
                                          : ((te == t_prev && idx == 0) || (te < t_prev && te >= t));
                if (in_range) {
                    if (te == t) {
                        write_dense(idx, y, a);
                    } else {
                        S v[CPL];
                        interpolate(te, v, a);
                        write_dense(idx, v, a);
                    }
                    idx += 1;
                } else {
                    if ((dir > 0.0 && te > t) || (dir < 0.0 && te < t)) break;
                    idx += 1;
                }
            }
            next_eval = idx;
        }
    }

    __device__ void begin(int64_t instance, const GroupArgs& ga) {
        const EnsArgs& a = ga.a;
        inst = instance;
        const int64_t n = a.n;
        d = ga.dims[inst];
        double t0 = a.t0[inst];
        tf = a.tf[inst];
        rtol = a.rtol[inst];
        atol = a.atol[inst];
        beta = a.params[inst];
        set_derived();
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            int c = lane + G * j;
            y[j] = c < d ? P::from(a.y0[(int64_t)c * n + inst]) : (S)0;
            yc[j] = (S)0;
        }
        t = t0;
        t_prev = t0;
        h_prev = 0.0;
        steps = acc = rej = fev = 0;
        stiff = nonstiff = 0;
        next_eval = 0;
        last_rejected = false;
        done = false;
        status = DEGPU_COMPLETE;
        double sg = rs_signum(tf - t0);
        if (!(sg == 1.0 || sg == -1.0) || d <= 0 || d > DG || (d & 1)) {
            status = DEGPU_ERR_BAD_INPUT;
            done = true;
            return;
        }
        dir = sg;
        S f0[CPL];
        double h0 = a.h0;
        if constexpr (Tab::ADAPTIVE) {
            if (h0 == 0.0) {
                initial_step(t0, a, f0);
                h0 = h;
            }
        } else {
            if (h0 == 0.0) h0 = fabs(tf - t0) / 100.0;
        }
        // validate_step_size_parameters (src/utils.rs:60-157)
        bool ok = !(tf == t0) && rs_signum(h0) == rs_signum(tf - t0) && !(a.h_min < 0.0 || a.h_max < 0.0 ||
                  a.h_min > a.h_max) && !(fabs(h0) < a.h_min || fabs(h0) > a.h_max) &&
                  !(fabs(h0) > fabs(tf - t0)) && h0 != 0.0;
        if (!ok) {
            status = DEGPU_ERR_BAD_INPUT;
            done = true;
            return;
        }
        h = h0;
        // k0 = f(t0, y0)
#pragma unroll
        for (int j = 0; j < CPL; ++j)
            if (lane + G * j < d) sy[lane + G * j] = y[j];
        sync();
        S kk[CPL];
        rhs(kk);
        sync();
#pragma unroll
        for (int j = 0; j < CPL; ++j)
            if (lane + G * j < d) k[lane + G * j] = kk[j];
        fev += 1;
        sync();
        solout(a);
    }

    // combination y + sum_j (a_ij h) k_j of stage i into sy; then f -> k[i]
    template <int Ii>
    __device__ __forceinline__ void stage(S* kout) {
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            int c = lane + G * j;
            if (c >= d) break;
            AccT ys = acc_begin(y[j]);
            static_for<0, Ii>([&](auto jj) {
                constexpr double aij = Tab::a(Ii, jj);
                if constexpr (aij != 0.0) acc_fma(ys, stage_coef(aij), k[jj * DG + c]);
            });
            sy[c] = acc_end(ys);
        }
        sync();
        S o[CPL];
        rhs(o);
        sync();
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            int c = lane + G * j;
            if (c < d) kout[c] = o[j];
        }
        sync();
    }

    __device__ int step_dp(const EnsArgs& a) {
        if (fabs(h) < fabs(h_prev) * 1e-14) {
            status = DEGPU_ERR_STEP_SIZE;
            return 3;
        }
        if (steps >= a.max_steps) {
            status = DEGPU_ERR_MAX_STEPS;
            return 3;
        }
        steps += 1;
        if constexpr (P::PAIR) hc = P::from(h);
        static_for<1, NS>([&](auto i) { stage<i>(k + i * DG); });
        // sy holds the last stage state (ysti)
        S ysti[CPL], yseg[CPL], ynew[CPL], ycn[CPL];
        double e1[CPL], e2[CPL];
        S hs = P::from(h);
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            int c = lane + G * j;
            bool live = c < d;
            int cc = live ? c : 0;
            ysti[j] = sy[cc];
            AccT sa = acc_begin((S)0);
            static_for<0, NS>([&](auto i) {
                constexpr double bv = Tab::b(i);
                if constexpr (bv != 0.0) acc_fma(sa, (S)bv, k[i * DG + cc]);
            });
            const S s = acc_end(sa);
            yseg[j] = s;
            if constexpr (P::KAHAN && !P::PAIR) {  // pairs carry 48 bits: no compensation
                S inc = hs * s;
                S yk = inc - yc[j];
                S ts = y[j] + yk;
                ycn[j] = (ts - y[j]) - yk;
                ynew[j] = ts;
            } else {
                ynew[j] = y[j] + hs * s;
                ycn[j] = (S)0;
            }
            AccT ea = acc_begin((S)0);
            static_for<0, NS>([&](auto jj) {
                constexpr double ev = Tab::er(jj);
                if constexpr (ev != 0.0) acc_fma(ea, (S)ev, k[jj * DG + cc]);
            });
            const S es = acc_end(ea);
            double sk = 0.0;
            if constexpr (P::PAIR) {
                // FP32 norm terms: the estimate's leading part against an FP32 scale
                const float skf = (a.atol_vec ? narrow_rz(atol_c(cc, a)) : atolf) +
                                  (a.rtol_vec ? narrow_rz(rtol_c(cc, a)) : rtolf) *
                                      fmaxf(fabsf(lead(y[j])), fabsf(lead(ynew[j])));
                const float qf = __fdividef(lead(es), skf);
                e1[j] = live ? widen_f32(qf * qf) : 0.0;
            } else {
                sk = atol_c(cc, a) + rtol_c(cc, a) * fmax(fabs(to_f64(y[j])), fabs(to_f64(ynew[j])));
                double q = to_f64(es) / sk;
                e1[j] = live ? q * q : 0.0;
            }
            if constexpr (Tab::HAS_BH) {
                AccT e2a = acc_begin(s);
                static_for<0, NS>([&](auto jj) {
                    constexpr double bhv = Tab::bh(jj);
                    if constexpr (bhv != 0.0) acc_fma(e2a, (S)(-bhv), k[jj * DG + cc]);
                });
                const S es2 = acc_end(e2a);
                if constexpr (P::PAIR) {
                    const float skf = (a.atol_vec ? narrow_rz(atol_c(cc, a)) : atolf) +
                                      (a.rtol_vec ? narrow_rz(rtol_c(cc, a)) : rtolf) *
                                          fmaxf(fabsf(lead(y[j])), fabsf(lead(ynew[j])));
                    const float q2 = __fdividef(lead(es2), skf);
                    e2[j] = live ? widen_f32(q2 * q2) : 0.0;
                } else {
                    double q2 = to_f64(es2) / sk;
                    e2[j] = live ? q2 * q2 : 0.0;
                }
            }
        }
        double t_new = t + h;
        fev += NS - 1;
        double err = reduce_terms(e1);
        double err2 = 0.0;
        if constexpr (Tab::HAS_BH) err2 = reduce_terms(e2);
        double deno = Tab::HAS_BH ? err + 0.01 * err2 : err;
        if (deno <= 0.0) deno = 1.0;
        err = fabs(h) * err * sqrt(1.0 / (deno * (double)d));
        double scale = a.safety * P::pow(err, -(1.0 / (double)O));
        scale = fmin(fmax(scale, a.min_scale), a.max_scale);
        int result;
        if (err <= 1.0) {
            // dydt = f(t_new, y_new)
#pragma unroll
            for (int j = 0; j < CPL; ++j)
                if (lane + G * j < d) sy[lane + G * j] = ynew[j];
            sync();
            S dydt[CPL];
            rhs(dydt);
            sync();
            fev += 1;
            if (steps % 100 == 0) {
                double n1[CPL], n2[CPL];
#pragma unroll
                for (int j = 0; j < CPL; ++j) {
                    int c = lane + G * j;
                    int cc = c < d ? c : 0;
                    if constexpr (P::PAIR) {
                        const float a1 = lead(yseg[j] - k[(NS - 1) * DG + cc]);
                        const float a2 = lead(dydt[j] - ysti[j]);
                        n1[j] = c < d ? widen_f32(a1 * a1) : 0.0;
                        n2[j] = c < d ? widen_f32(a2 * a2) : 0.0;
                    } else {
                        double a1 = to_f64(yseg[j]) - to_f64(k[(NS - 1) * DG + cc]);
                        double a2 = to_f64(dydt[j]) - to_f64(ysti[j]);
                        n1[j] = c < d ? a1 * a1 : 0.0;
                        n2[j] = c < d ? a2 * a2 : 0.0;
                    }
                }
                double stdnum = reduce_terms(n1);
                double stden = reduce_terms(n2);
                if (stden > 0.0) {
                    double h_lamb = h * sqrt(stdnum / stden);
                    if (h_lamb > 6.1) {
                        nonstiff = 0;
                        stiff += 1;
                        if (stiff == 15) {
                            status = DEGPU_ERR_STIFFNESS;
                            return 3;
                        }
                    }
                } else {
                    nonstiff += 1;
                    if (nonstiff == 6) stiff = 0;
                }
            }
            if constexpr (DENSE) {
#pragma unroll
                for (int j = 0; j < CPL; ++j) {
                    int c = lane + G * j;
                    if (c >= d) break;
                    cont[0 * DG + c] = y[j];
                    S ydiff = ynew[j] - y[j];
                    cont[1 * DG + c] = ydiff;
                    S bspl = hs * k[c];
                    bspl = bspl - ydiff;
                    cont[2 * DG + c] = bspl;
                    S c3 = ydiff - hs * dydt[j];
                    c3 = c3 - bspl;
                    cont[3 * DG + c] = c3;
                    if constexpr (I > NS) k[NS * DG + c] = dydt[j];
                }
                sync();
                if constexpr (I > NS) static_for<NS + 1, I>([&](auto i) {
                    stage<i>(k + i * DG);
                    fev += 1;
                });
                static_for<4, O>([&](auto i) {
#pragma unroll
                    for (int j = 0; j < CPL; ++j) {
                        int c = lane + G * j;
                        if (c >= d) break;
                        S s = (S)0;
                        static_for<0, I>([&](auto jj) {
                            constexpr double v = Tab::bi(i, jj);
                            if constexpr (v != 0.0) s = s + (S)v * k[jj * DG + c];
                        });
                        cont[i * DG + c] = s * hs;
                    }
                });
            } else {
                fev += I - NS - (I > NS ? 1 : 0);
            }
            t_prev = t;
            h_prev = h;
            t = t_new;
#pragma unroll
            for (int j = 0; j < CPL; ++j) {
                y[j] = ynew[j];
                yc[j] = ycn[j];
                int c = lane + G * j;
                if (c < d) k[c] = dydt[j];
            }
            sync();
            if (last_rejected) {
                last_rejected = false;
                scale = fmin(scale, 1.0);
            }
            result = 1;
        } else {
            last_rejected = true;
            result = 2;
        }
        h = h * scale;
        if (fabs(h) < a.h_min)
            h = rs_signum(h) * a.h_min;
        else if (fabs(h) > a.h_max)
            h = rs_signum(h) * a.h_max;
        return result;
    }

    __device__ void iterate(const EnsArgs& a) {
        const double eps10 = 2.220446049250313e-16 * 10.0;
        if ((t + h - tf) * dir > 0.0) {
            double h_new = tf - t;
            if (fabs(h_new) < eps10) {
                done = true;
                return;
            }
            h = h_new;
        }
        int r = step_dp(a);
        if (r == 3) {
            done = true;
            return;
        }
        if (r == 2) {
            rej += 1;
            return;
        }
        acc += 1;
        solout(a);
        if (fabs(tf - t) <= eps10) done = true;
    }

    // Serving rounds: the state that lives across driver iterations — the scalars (written by
    // lane 0) and, per component, y, its compensation and the derivative k0 at t (k[0] in shared
    // memory).  Everything else a step reads is rebuilt inside the step.
    __device__ void park(GroupPark& pk, S* vec) const {
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            const int c = lane + G * j;
            if (c < d) {
                vec[c] = y[j];
                vec[DG + c] = yc[j];
                vec[2 * DG + c] = k[c];
            }
        }
        if (lane == 0) {
            pk.d = d;
            pk.stiff = stiff;
            pk.nonstiff = nonstiff;
            pk.next_eval = next_eval;
            pk.status = status;
            pk.last_rejected = last_rejected ? 1 : 0;
            pk.inst = inst;
            pk.steps = steps;
            pk.acc = acc;
            pk.rej = rej;
            pk.fev = fev;
            pk.t = t;
            pk.tf = tf;
            pk.h = h;
            pk.h_prev = h_prev;
            pk.t_prev = t_prev;
            pk.dir = dir;
            pk.rtol = rtol;
            pk.atol = atol;
            pk.beta = beta;
        }
    }
    __device__ void resume(const GroupPark& pk, const S* vec) {
        d = pk.d;
        stiff = pk.stiff;
        nonstiff = pk.nonstiff;
        next_eval = pk.next_eval;
        status = pk.status;
        last_rejected = pk.last_rejected != 0;
        done = false;
        inst = pk.inst;
        steps = pk.steps;
        acc = pk.acc;
        rej = pk.rej;
        fev = pk.fev;
        t = pk.t;
        tf = pk.tf;
        h = pk.h;
        h_prev = pk.h_prev;
        t_prev = pk.t_prev;
        dir = pk.dir;
        rtol = pk.rtol;
        atol = pk.atol;
        beta = pk.beta;
        set_derived();
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            const int c = lane + G * j;
            y[j] = c < d ? vec[c] : (S)0;
            yc[j] = c < d ? vec[DG + c] : (S)0;
            if (c < d) k[c] = vec[2 * DG + c];
        }
        sync();
    }

    __device__ void finish(const EnsArgs& a) const {
        const int64_t n = a.n;
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            int c = lane + G * j;
            if (c < d) a.y_final[(int64_t)c * n + inst] = to_f64(y[j]) - to_f64(yc[j]);
        }
        for (int c = d + lane; c < a.dmax; c += G) a.y_final[(int64_t)c * n + inst] = 0.0;
        if (lane == 0) {
            if (a.t_final) a.t_final[inst] = t;
            if (a.accepted) a.accepted[inst] = acc;
            if (a.rejected) a.rejected[inst] = rej;
            if (a.fevals) a.fevals[inst] = fev;
            if (a.status) a.status[inst] = status;
        }
    }
};

template <class Tab, class P, int G, int CPL, bool DENSE>
__host__ __device__ constexpr size_t group_smem_per_system() {
    using S = typename P::S;
    constexpr int DG = G * CPL;
    return (size_t)(Tab::I + 1 + (DENSE ? Tab::ORDER : 0)) * DG * sizeof(S) + (size_t)DG * sizeof(double);
}

template <class Tab, class P, int G, int CPL, bool DENSE>
__global__ void __launch_bounds__(128) erk_group_kernel(GroupArgs ga) {
    using GL = GroupLane<Tab, P, G, CPL, DENSE>;
    using S = typename P::S;
    constexpr int DG = G * CPL;
    extern __shared__ __align__(16) unsigned char smem[];
    const int gid = threadIdx.x / G;  // group within the block
    constexpr size_t per = group_smem_per_system<Tab, P, G, CPL, DENSE>();
    unsigned char* base = smem + per * gid;
    GL L;
    L.k = (S*)base;
    L.sy = L.k + Tab::I * DG;
    L.cont = L.sy + DG;
    L.red = (double*)(base + (size_t)(Tab::I + 1 + (DENSE ? Tab::ORDER : 0)) * DG * sizeof(S));
    L.lane = threadIdx.x % G;
    const int wlane = threadIdx.x % 32;
    L.gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (wlane / G * G));
    const EnsArgs& a = ga.a;
    for (;;) {
        unsigned long long w = 0;
        if (L.lane == 0) w = atomicAdd(a.ticket, 1ULL);
        w = __shfl_sync(L.gmask, w, 0, G);
        if (w >= (unsigned long long)a.count) break;
        L.begin(a.index ? a.index[w] : (int64_t)w, ga);
        while (!L.done) L.iterate(a);
        L.finish(a);
        __syncwarp(L.gmask);
    }
}

// Bytes of one parked system: the scalars, then y, its compensation and k0 over DG components.
template <class Tab, class P, int G, int CPL>
__host__ __device__ constexpr size_t group_park_bytes() {
    return ((sizeof(GroupPark) + 15) / 16) * 16 + (size_t)3 * G * CPL * sizeof(typename P::S);
}

// Resumable form of erk_group_kernel for the server: every work item is visited once per round;
// a visit starts the system (phase 0) or resumes its parked state, runs at most `budget` driver
// iterations, then parks it again or finishes it.  `done_count` counts finished systems across
// rounds.  Slot w of `park` holds work item w (instance a.index[w] when an index list is given).
template <class Tab, class P, int G, int CPL, bool DENSE>
__global__ void __launch_bounds__(128) erk_group_round_kernel(GroupArgs ga, unsigned char* park, int budget,
                                                              unsigned long long* done_count) {
    using GL = GroupLane<Tab, P, G, CPL, DENSE>;
    using S = typename P::S;
    constexpr int DG = G * CPL;
    constexpr size_t slot_bytes = group_park_bytes<Tab, P, G, CPL>();
    constexpr size_t scal_bytes = ((sizeof(GroupPark) + 15) / 16) * 16;
    extern __shared__ __align__(16) unsigned char smem[];
    const int gid = threadIdx.x / G;
    constexpr size_t per = group_smem_per_system<Tab, P, G, CPL, DENSE>();
    unsigned char* base = smem + per * gid;
    GL L;
    L.k = (S*)base;
    L.sy = L.k + Tab::I * DG;
    L.cont = L.sy + DG;
    L.red = (double*)(base + (size_t)(Tab::I + 1 + (DENSE ? Tab::ORDER : 0)) * DG * sizeof(S));
    L.lane = threadIdx.x % G;
    const int wlane = threadIdx.x % 32;
    L.gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (wlane / G * G));
    const EnsArgs& a = ga.a;
    for (;;) {
        unsigned long long w = 0;
        if (L.lane == 0) w = atomicAdd(a.ticket, 1ULL);
        w = __shfl_sync(L.gmask, w, 0, G);
        if (w >= (unsigned long long)a.count) break;
        GroupPark& pk = *reinterpret_cast<GroupPark*>(park + w * slot_bytes);
        S* vec = reinterpret_cast<S*>(park + w * slot_bytes + scal_bytes);
        const int phase = pk.phase;
        __syncwarp(L.gmask);  // every lane has read the phase before lane 0 may rewrite it
        if (phase == 2) continue;
        if (phase == 0)
            L.begin(a.index ? a.index[w] : (int64_t)w, ga);
        else
            L.resume(pk, vec);
        for (int it = 0; it < budget && !L.done; ++it) L.iterate(a);
        if (L.done) {
            L.finish(a);
            if (L.lane == 0) {
                pk.phase = 2;
                atomicAdd(done_count, 1ULL);
            }
        } else {
            L.park(pk, vec);
            if (L.lane == 0) pk.phase = 1;
        }
        __syncwarp(L.gmask);
    }
}

template <class Tab, class P, int G, int CPL, bool DENSE>
cudaError_t launch_group_round(const EnsArgs& a, void* park, int budget, unsigned long long* done, int max_blocks,
                               cudaStream_t s) {
    auto kern = erk_group_round_kernel<Tab, P, G, CPL, DENSE>;
    constexpr size_t per = group_smem_per_system<Tab, P, G, CPL, DENSE>();
    const int threads = 128;
    const size_t smem = per * (threads / G);
    if (a.count <= 0) return cudaSuccess;
    static int blocks_per_sm = -1;
    if (blocks_per_sm < 0) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, threads, smem);
        if (e != cudaSuccess) return e;
        if (blocks_per_sm < 1) return cudaErrorInvalidConfiguration;
    }
    long long grid = (long long)blocks_per_sm * device_sm_count();
    long long need = (a.count * G + threads - 1) / threads;
    if (grid > need) grid = need;
    if (max_blocks > 0 && grid > max_blocks) grid = max_blocks;
    if (grid < 1) grid = 1;
    GroupArgs ga;
    ga.a = a;
    ga.dims = a.dims;
    kern<<<(unsigned)grid, threads, smem, s>>>(ga, (unsigned char*)park, budget, done);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// dispatch
// ---------------------------------------------------------------------------------------------
using GroupLaunch = cudaError_t (*)(const GroupArgs&, cudaStream_t);

template <class Tab, class P, int G, int CPL, bool DENSE>
cudaError_t launch_group(const GroupArgs& ga, cudaStream_t s) {
    auto kern = erk_group_kernel<Tab, P, G, CPL, DENSE>;
    constexpr size_t per = group_smem_per_system<Tab, P, G, CPL, DENSE>();
    const int threads = 128;
    const size_t smem = per * (threads / G);
    static int blocks_per_sm = -1;
    if (blocks_per_sm < 0) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, threads, smem);
        if (e != cudaSuccess) return e;
        if (blocks_per_sm < 1) return cudaErrorInvalidConfiguration;
    }
    long long grid = (long long)blocks_per_sm * device_sm_count();
    long long need = (ga.a.count * G + threads - 1) / threads;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, threads, smem, s>>>(ga);
    return cudaGetLastError();
}

struct GroupKey {
    int method, prec, dense, g, cpl;
    bool operator<(const GroupKey& o) const {
        return std::tie(method, prec, dense, g, cpl) < std::tie(o.method, o.prec, o.dense, o.g, o.cpl);
    }
};

std::map<GroupKey, GroupLaunch>& group_registry();

template <class Tab, class P, int G, int CPL>
void reg_group() {
    group_registry()[GroupKey{method_id<Tab>(), P::ID, 0, G, CPL}] = &launch_group<Tab, P, G, CPL, false>;
    group_registry()[GroupKey{method_id<Tab>(), P::ID, 1, G, CPL}] = &launch_group<Tab, P, G, CPL, true>;
}

// Only the kernel without output times: the layouts where the pair form with output times holds
// too many registers to beat FP64 (measured on FPU-beta chains of 66..128 components).
template <class Tab, class P, int G, int CPL>
void reg_group_final() {
    group_registry()[GroupKey{method_id<Tab>(), P::ID, 0, G, CPL}] = &launch_group<Tab, P, G, CPL, false>;
}

// Resumable group kernels of the server, keyed like group_registry: bytes per parked system and
// the round launcher (the signature of the other round kernels, dims in EnsArgs).
struct GroupRoundOps {
    size_t park_bytes;
    cudaError_t (*launch)(const EnsArgs& a, void* park, int budget, unsigned long long* done, int max_blocks,
                          cudaStream_t s);
};
std::map<GroupKey, GroupRoundOps>& group_round_registry();

template <class Tab, class P, int G, int CPL>
void reg_group_round() {
    group_round_registry()[GroupKey{method_id<Tab>(), P::ID, 0, G, CPL}] =
        GroupRoundOps{group_park_bytes<Tab, P, G, CPL>(), &launch_group_round<Tab, P, G, CPL, false>};
    group_round_registry()[GroupKey{method_id<Tab>(), P::ID, 1, G, CPL}] =
        GroupRoundOps{group_park_bytes<Tab, P, G, CPL>(), &launch_group_round<Tab, P, G, CPL, true>};
}
template <class Tab, class P, int G, int CPL>
void reg_group_round_final() {
    group_round_registry()[GroupKey{method_id<Tab>(), P::ID, 0, G, CPL}] =
        GroupRoundOps{group_park_bytes<Tab, P, G, CPL>(), &launch_group_round<Tab, P, G, CPL, false>};
}

// The work of a ragged request split for the resumable group kernels: one part per (precision,
// G, CPL) bucket, with its instances (the host copies of dims and rtol are read).  DEGPU_OK when
// every bucket has a round kernel.
struct GroupRoundPart {
    GroupRoundOps ops;
    std::vector<int64_t> idx;
};
degpu_status group_round_parts(const degpu_problem* pb, const degpu_method_cfg* cfg, const int32_t* dims_host,
                               const double* rtol_host, int64_t n, int dense, std::vector<GroupRoundPart>& parts);

void register_group_parity();
void register_group_fast();
void register_group_rounds();
void register_group_pair853();
void register_group_pair853_rounds();
void register_group_pair5();
// every group kernel (run to completion and resumable), once
void register_groups();

}  // namespace degpu
