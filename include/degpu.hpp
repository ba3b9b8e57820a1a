// degpu.hpp — C++17 host API over the C ABI (degpu.h), with the crate's builder shape.
//
//   auto m   = degpu::ExplicitRungeKutta::dopri5().rtol(1e-8).atol(1e-10);   // src/methods/erk/mod.rs:165-174
//   auto sol = degpu::IVP::ode(degpu::System::lorenz(10, 28, 8.0 / 3), 0.0, 20.0, {1, 1, 1})  // src/ivp.rs:279
//                  .method(m)                                                 // src/ivp.rs:632
//                  .t_eval({0.5, 1.0})                                        // src/ivp.rs:656-660
//                  .solve();                                                  // src/ivp.rs:781-791
//   if (sol.ok()) ... sol.value().y.back() ... else sol.error().kind == degpu::ErrorKind::MaxSteps
//
// and solve_ensemble() for n instances in one call.  Errors are values, as in the crate
// (`Result<Solution, Error>`, src/error.rs:13-40): BadInput carries a message starting with
// "Invalid input"; MaxSteps / StepSize / Stiffness carry the (t, y) where the solve stopped.
#pragma once

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <filesystem>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "degpu.h"

namespace degpu {

enum class ErrorKind { BadInput, MaxSteps, StepSize, Stiffness, Device };

struct Error {
    ErrorKind kind;
    std::string msg;
    double t = 0.0;
    std::vector<double> y;
};

// Rust's `format!("{:?}", x)` for an f64: the shortest digits that round-trip, in decimal
// notation for 1e-4 <= |x| < 1e16 (always with a fractional part) and in exponential notation
// otherwise ("1e-5", "1.5e16"); "NaN", "inf", "-inf".
inline std::string rust_debug_f64(double x) {
    if (std::isnan(x)) return "NaN";
    if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
    if (x == 0.0) return std::signbit(x) ? "-0.0" : "0.0";
    char buf[64];
    auto r = std::to_chars(buf, buf + sizeof(buf), x, std::chars_format::scientific);  // shortest digits
    std::string sci(buf, r.ptr);
    const bool neg = sci[0] == '-';
    if (neg) sci.erase(0, 1);
    const std::size_t epos = sci.find('e');
    std::string digits = sci.substr(0, epos);
    digits.erase(std::remove(digits.begin(), digits.end(), '.'), digits.end());
    const int e10 = std::stoi(sci.substr(epos + 1));
    const double ax = std::fabs(x);
    std::string out;
    if (ax >= 1e-4 && ax < 1e16) {
        const int point = e10 + 1;  // digits before the decimal point
        if (point <= 0)
            out = "0." + std::string((std::size_t)(-point), '0') + digits;
        else if (point >= (int)digits.size())
            out = digits + std::string((std::size_t)point - digits.size(), '0') + ".0";
        else
            out = digits.substr(0, (std::size_t)point) + "." + digits.substr((std::size_t)point);
    } else {
        out = digits.substr(0, 1);
        if (digits.size() > 1) out += "." + digits.substr(1);
        out += "e" + std::to_string(e10);
    }
    return neg ? "-" + out : out;
}

// Solution fields the GPU produces (src/solution.rs:30-52, src/stats.rs).
struct Solution {
    std::vector<double> t;
    std::vector<std::vector<double>> y;
    std::size_t evals = 0;      // Evals.function
    std::size_t accepted = 0;   // Steps.accepted
    std::size_t rejected = 0;   // Steps.rejected
    bool interrupted = false;   // Status::Interrupted (a terminal event ended the solve)

    // Solution::to_csv (src/solution.rs:190-226): header t,y0,..,yN-1 and one row per point, numbers
    // in Rust's Debug format; the parent directory is created when missing.  False on an I/O error.
    bool to_csv(const std::string& filename) const {
        const std::filesystem::path path(filename);
        std::error_code ec;
        if (path.has_parent_path() && !std::filesystem::exists(path.parent_path()))
            std::filesystem::create_directories(path.parent_path(), ec);
        std::FILE* f = std::fopen(filename.c_str(), "w");
        if (!f) return false;
        const std::size_t n = y.empty() ? 0 : y[0].size();
        std::string line = "t";
        for (std::size_t i = 0; i < n; ++i) line += ",y" + std::to_string(i);
        std::fprintf(f, "%s\n", line.c_str());
        for (std::size_t k = 0; k < t.size(); ++k) {
            line = rust_debug_f64(t[k]);
            for (std::size_t i = 0; i < n; ++i) line += "," + rust_debug_f64(y[k][i]);
            std::fprintf(f, "%s\n", line.c_str());
        }
        return std::fclose(f) == 0;
    }
};

template <class T>
class Result {
   public:
    static Result ok_value(T v) { Result r; r.ok_ = true; r.v_ = std::move(v); return r; }
    static Result err(Error e) { Result r; r.ok_ = false; r.e_ = std::move(e); return r; }
    bool ok() const { return ok_; }
    const T& value() const { if (!ok_) throw std::runtime_error(e_.msg); return v_; }
    const Error& error() const { return e_; }
   private:
    bool ok_ = false;
    T v_{};
    Error e_{};
};

class ExplicitRungeKutta {
   public:
    static ExplicitRungeKutta rk4(double h0) { ExplicitRungeKutta m(DEGPU_RK4); m.cfg_.h0 = h0; return m; }
    static ExplicitRungeKutta dopri5() { return ExplicitRungeKutta(DEGPU_DOPRI5); }
    static ExplicitRungeKutta dop853() { return ExplicitRungeKutta(DEGPU_DOP853); }
    static ExplicitRungeKutta rkf45() { return ExplicitRungeKutta(DEGPU_RKF45); }        // adaptive/mod.rs:43-50
    static ExplicitRungeKutta cash_karp() { return ExplicitRungeKutta(DEGPU_CASH_KARP); }  // adaptive/mod.rs:51-58
    // Verner's pairs, adaptive/mod.rs:59-122 (tableaus src/tableau/verner.rs)
    static ExplicitRungeKutta rkv655e() { return ExplicitRungeKutta(DEGPU_RKV655E); }
    static ExplicitRungeKutta rkv656e() { return ExplicitRungeKutta(DEGPU_RKV656E); }
    static ExplicitRungeKutta rkv766e() { return ExplicitRungeKutta(DEGPU_RKV766E); }
    static ExplicitRungeKutta rkv767e() { return ExplicitRungeKutta(DEGPU_RKV767E); }
    static ExplicitRungeKutta rkv877e() { return ExplicitRungeKutta(DEGPU_RKV877E); }
    static ExplicitRungeKutta rkv878e() { return ExplicitRungeKutta(DEGPU_RKV878E); }
    static ExplicitRungeKutta rkv988e() { return ExplicitRungeKutta(DEGPU_RKV988E); }
    static ExplicitRungeKutta rkv989e() { return ExplicitRungeKutta(DEGPU_RKV989E); }
    ExplicitRungeKutta& rtol(double v) { rtol_ = v; return *this; }
    ExplicitRungeKutta& atol(double v) { atol_ = v; return *this; }
    ExplicitRungeKutta& h0(double v) { cfg_.h0 = v; return *this; }
    ExplicitRungeKutta& h_min(double v) { cfg_.h_min = v; return *this; }
    ExplicitRungeKutta& h_max(double v) { cfg_.h_max = v; return *this; }
    ExplicitRungeKutta& max_steps(int64_t v) { cfg_.max_steps = v; return *this; }
    ExplicitRungeKutta& safety_factor(double v) { cfg_.safety_factor = v; return *this; }
    ExplicitRungeKutta& min_scale(double v) { cfg_.min_scale = v; return *this; }
    ExplicitRungeKutta& max_scale(double v) { cfg_.max_scale = v; return *this; }
    // GPU knobs
    ExplicitRungeKutta& precision(degpu_precision p) { cfg_.precision = p; return *this; }
    ExplicitRungeKutta& kernel(degpu_kernel k) { cfg_.kernel = k; return *this; }
    ExplicitRungeKutta& dense_mode(degpu_dense_mode d) { cfg_.dense_mode = d; return *this; }
    const degpu_method_cfg& cfg() const { return cfg_; }
    double rtol() const { return rtol_; }
    double atol() const { return atol_; }

   private:
    explicit ExplicitRungeKutta(int method) { degpu_default_cfg(&cfg_, method); }
    degpu_method_cfg cfg_{};
    double rtol_ = 1e-6, atol_ = 1e-6;  // src/methods/erk/mod.rs:135-136
};

// A right-hand side with a device twin: a built-in family or an id from degpu_register_rhs_nvrtc.
struct System {
    int32_t rhs_id;
    std::vector<double> params;
    static System lorenz(double sigma, double rho, double beta) { return {DEGPU_RHS_LORENZ, {sigma, rho, beta}}; }
    static System van_der_pol(double mu) { return {DEGPU_RHS_VAN_DER_POL, {mu}}; }
    static System pendulum(double gamma, double a, double omega) { return {DEGPU_RHS_PENDULUM, {gamma, a, omega}}; }
    static System exponential_growth(double k) { return {DEGPU_RHS_EXP_GROWTH, {k}}; }
    static System harmonic(double k) { return {DEGPU_RHS_HARMONIC, {k}}; }
    static System fpu_beta(double beta) { return {DEGPU_RHS_FPU_BETA, {beta}}; }
    static System brusselator(double a, double b) { return {DEGPU_RHS_BRUSSELATOR, {a, b}}; }
    static System cr3bp(double mu) { return {DEGPU_RHS_CR3BP, {mu}}; }
};

// src/solout/crossing.rs:17-26
enum class CrossingDirection { Both = DEGPU_CROSS_BOTH, Positive = DEGPU_CROSS_POSITIVE, Negative = DEGPU_CROSS_NEGATIVE };

// Results of an ensemble solve, structure of arrays (layout of degpu.h).
struct EnsembleResult {
    int64_t n = 0;
    int32_t dim = 0;
    std::vector<double> y_final, t_final, dense;
    std::vector<int64_t> accepted, rejected, fevals;
    std::vector<int32_t> status;
};

inline EnsembleResult solve_ensemble(int32_t rhs_id, int32_t dim, int32_t n_params, const std::vector<double>& t0,
                                     const std::vector<double>& tf, const std::vector<double>& y0,
                                     const std::vector<double>& params, const std::vector<double>& rtol,
                                     const std::vector<double>& atol, const ExplicitRungeKutta& m,
                                     const std::vector<double>& t_eval = {},
                                     const std::vector<int32_t>& dims = {}) {
    EnsembleResult r;
    r.n = (int64_t)t0.size();
    r.dim = dim;
    const size_t n = (size_t)r.n;
    r.y_final.resize((size_t)dim * n);
    r.t_final.resize(n);
    r.dense.resize(t_eval.size() * (size_t)dim * n);
    r.accepted.resize(n);
    r.rejected.resize(n);
    r.fevals.resize(n);
    r.status.resize(n);
    degpu_problem pb{rhs_id, dim, n_params, 0};
    degpu_batch_in in{};
    in.n = r.n;
    in.t0 = t0.data();
    in.tf = tf.data();
    in.y0 = y0.data();
    in.params = params.empty() ? nullptr : params.data();
    in.rtol = rtol.data();
    in.atol = atol.data();
    in.dims = dims.empty() ? nullptr : dims.data();
    in.t_eval = t_eval.empty() ? nullptr : t_eval.data();
    in.n_eval = (int32_t)t_eval.size();
    degpu_batch_out out{r.y_final.data(), r.t_final.data(), t_eval.empty() ? nullptr : r.dense.data(),
                        r.accepted.data(), r.rejected.data(), r.fevals.data(), r.status.data()};
    degpu_status st = degpu_solve_ensemble_host(&pb, &m.cfg(), &in, &out);
    if (st != DEGPU_OK) throw std::runtime_error(std::string("degpu_solve_ensemble_host: ") + degpu_status_string(st));
    return r;
}

class IVP {
   public:
    static IVP ode(System sys, double t0, double tf, std::vector<double> y0) {
        IVP p;
        p.sys_ = std::move(sys);
        p.t0_ = t0;
        p.tf_ = tf;
        p.y0_ = std::move(y0);
        return p;
    }
    IVP& method(const ExplicitRungeKutta& m) { m_ = m; return *this; }
    IVP& t_eval(std::vector<double> pts) {
        te_ = std::move(pts);
        if (cross_ != 3) cross_ = 0;
        return *this;
    }
    // src/ivp.rs:661-679: wraps the current output (t_eval, else the final point) with event
    // detection; the solution holds the output points and the recorded events in time order, and a
    // terminal event ends it with Status::Interrupted (Solution::interrupted)
    IVP& event(const degpu_event& ev) {
        cross_ = 3;
        ev_ = ev;
        return *this;
    }
    // src/ivp.rs:682-693: the solution holds the points where y[component] crosses threshold
    IVP& crossing(int32_t component, double threshold, CrossingDirection dir = CrossingDirection::Both,
                  int32_t max_points = 1024) {
        cross_ = 1;
        cr_ = degpu_crossing{component, (int32_t)dir, max_points, 0, threshold};
        te_.clear();
        return *this;
    }
    // src/ivp.rs:695-706: the points where pos = y[components] crosses the plane through point
    // with normal; the crate's extractor function is given as the components it picks
    IVP& hyperplane_crossing(const std::vector<double>& point, const std::vector<double>& normal,
                             const std::vector<int32_t>& components, CrossingDirection dir = CrossingDirection::Both,
                             int32_t max_points = 1024) {
        cross_ = 2;
        hp_ = degpu_hyperplane{};
        hp_.dim = (int32_t)components.size();
        hp_.direction = (int32_t)dir;
        hp_.max_points = max_points;
        for (size_t j = 0; j < components.size() && j < DEGPU_HYPERPLANE_MAX_DIM; ++j) {
            hp_.components[j] = components[j];
            hp_.point[j] = j < point.size() ? point[j] : NAN;
            hp_.normal[j] = j < normal.size() ? normal[j] : NAN;
        }
        if (components.size() > DEGPU_HYPERPLANE_MAX_DIM || point.size() != components.size() ||
            normal.size() != components.size())
            hp_.dim = 0;  // rejected as bad input by the library
        te_.clear();
        return *this;
    }

    Result<Solution> solve() const {
        if (cross_) return solve_crossing();
        const int32_t d = (int32_t)y0_.size();
        EnsembleResult r;
        try {
            r = solve_ensemble(sys_.rhs_id, d, (int32_t)sys_.params.size(), {t0_}, {tf_}, y0_, sys_.params,
                               {m_.rtol()}, {m_.atol()}, m_, te_,
                               sys_.rhs_id == DEGPU_RHS_FPU_BETA ? std::vector<int32_t>{d} : std::vector<int32_t>{});
        } catch (const std::exception& ex) {
            return Result<Solution>::err(Error{ErrorKind::Device, ex.what()});
        }
        std::vector<double> yf(r.y_final.begin(), r.y_final.begin() + d);
        switch (r.status[0]) {
            case DEGPU_ERR_BAD_INPUT:
                return Result<Solution>::err(Error{ErrorKind::BadInput, "Invalid input: step size or interval"});
            case DEGPU_ERR_MAX_STEPS: return Result<Solution>::err(Error{ErrorKind::MaxSteps, "MaxSteps", r.t_final[0], yf});
            case DEGPU_ERR_STEP_SIZE: return Result<Solution>::err(Error{ErrorKind::StepSize, "StepSize", r.t_final[0], yf});
            case DEGPU_ERR_STIFFNESS: return Result<Solution>::err(Error{ErrorKind::Stiffness, "Stiffness", r.t_final[0], yf});
            default: break;
        }
        Solution s;
        s.evals = (size_t)r.fevals[0];
        s.accepted = (size_t)r.accepted[0];
        s.rejected = (size_t)r.rejected[0];
        if (te_.empty()) {
            s.t.push_back(r.t_final[0]);
            s.y.push_back(yf);
        } else {
            // requested points in integration order (TEvalSolout sorts by direction)
            std::vector<size_t> idx(te_.size());
            for (size_t i = 0; i < idx.size(); ++i) idx[i] = i;
            const bool fwd = tf_ >= t0_;
            std::stable_sort(idx.begin(), idx.end(),
                             [&](size_t a, size_t b) { return fwd ? te_[a] < te_[b] : te_[a] > te_[b]; });
            for (size_t e : idx) {
                if (std::isnan(r.dense[e * (size_t)d])) continue;
                s.t.push_back(te_[e]);
                s.y.emplace_back(r.dense.begin() + e * d, r.dense.begin() + (e + 1) * d);
            }
        }
        return Result<Solution>::ok_value(std::move(s));
    }

   private:
    static Result<Solution> status_error(int32_t status, double t, const std::vector<double>& y) {
        switch (status) {
            case DEGPU_ERR_BAD_INPUT:
                return Result<Solution>::err(Error{ErrorKind::BadInput, "Invalid input: step size or interval"});
            case DEGPU_ERR_MAX_STEPS: return Result<Solution>::err(Error{ErrorKind::MaxSteps, "MaxSteps", t, y});
            case DEGPU_ERR_STEP_SIZE: return Result<Solution>::err(Error{ErrorKind::StepSize, "StepSize", t, y});
            default: return Result<Solution>::err(Error{ErrorKind::Stiffness, "Stiffness", t, y});
        }
    }

    // One instance through degpu_solve_ensemble_crossing_host / _hyperplane_host / _event_host.
    Result<Solution> solve_crossing() const {
        const int32_t d = (int32_t)y0_.size();
        const int32_t cap = cross_ == 1 ? cr_.max_points : cross_ == 2 ? hp_.max_points : ev_.max_points;
        const size_t m = cap > 0 ? (size_t)cap : 0;
        std::vector<double> yf(d), tf(1), ct(m), cy(m * d);
        std::vector<int64_t> acc(1), rej(1), fev(1);
        std::vector<int32_t> st(1), cc(1);
        double t0 = t0_, t1 = tf_, rtol = m_.rtol(), atol = m_.atol();
        degpu_problem pb{sys_.rhs_id, d, (int32_t)sys_.params.size(), 0};
        degpu_batch_in in{};
        in.n = 1;
        in.t0 = &t0;
        in.tf = &t1;
        in.y0 = y0_.data();
        in.params = sys_.params.empty() ? nullptr : sys_.params.data();
        in.rtol = &rtol;
        in.atol = &atol;
        const bool with_te = cross_ == 3 && !te_.empty();
        std::vector<double> dense(with_te ? te_.size() * (size_t)d : 0);
        if (with_te) {
            in.t_eval = te_.data();
            in.n_eval = (int32_t)te_.size();
        }
        degpu_batch_out out{yf.data(), tf.data(), with_te ? dense.data() : nullptr, acc.data(), rej.data(), fev.data(),
                            st.data()};
        degpu_crossing_out co{m ? ct.data() : nullptr, m ? cy.data() : nullptr, cc.data()};
        degpu_status rc;
        if (cross_ == 1)
            rc = degpu_solve_ensemble_crossing_host(&pb, &m_.cfg(), &in, &cr_, &out, &co);
        else if (cross_ == 2)
            rc = degpu_solve_ensemble_hyperplane_host(&pb, &m_.cfg(), &in, &hp_, &out, &co);
        else
            rc = degpu_solve_ensemble_event_host(&pb, &m_.cfg(), &in, &ev_, &out, &co);
        if (rc == DEGPU_BAD_INPUT) return Result<Solution>::err(Error{ErrorKind::BadInput, "Invalid input: crossing"});
        if (rc != DEGPU_OK)
            return Result<Solution>::err(Error{ErrorKind::Device, std::string("crossing solve: ") + degpu_status_string(rc)});
        if (st[0] != DEGPU_COMPLETE && st[0] != DEGPU_INTERRUPTED) return status_error(st[0], tf[0], yf);
        Solution s;
        s.evals = (size_t)fev[0];
        s.accepted = (size_t)acc[0];
        s.rejected = (size_t)rej[0];
        s.interrupted = st[0] == DEGPU_INTERRUPTED;
        std::vector<std::pair<double, std::vector<double>>> pts;
        const size_t k = std::min(m, (size_t)cc[0]);
        for (size_t j = 0; j < k; ++j) {
            std::vector<double> yj(d);
            for (int32_t c = 0; c < d; ++c) yj[c] = cy[j * d + c];
            pts.emplace_back(ct[j], std::move(yj));
        }
        if (cross_ == 3) {  // the base output: output times reached, else the final point
            if (with_te) {
                for (size_t e = 0; e < te_.size(); ++e)
                    if (!std::isnan(dense[e * d])) pts.emplace_back(te_[e], std::vector<double>(dense.begin() + e * d, dense.begin() + (e + 1) * d));
            } else {
                pts.emplace_back(tf[0], yf);
            }
            const bool fwd = tf_ >= t0_;
            std::stable_sort(pts.begin(), pts.end(),
                             [&](const auto& x, const auto& y) { return fwd ? x.first < y.first : x.first > y.first; });
        }
        for (auto& p : pts) {
            s.t.push_back(p.first);
            s.y.push_back(std::move(p.second));
        }
        return Result<Solution>::ok_value(std::move(s));
    }

    System sys_{};
    double t0_ = 0, tf_ = 0;
    std::vector<double> y0_, te_;
    ExplicitRungeKutta m_ = ExplicitRungeKutta::dopri5();
    int cross_ = 0;  // 0 none, 1 component crossing, 2 hyperplane crossing, 3 event
    degpu_crossing cr_{};
    degpu_hyperplane hp_{};
    degpu_event ev_{};
};

}  // namespace degpu
