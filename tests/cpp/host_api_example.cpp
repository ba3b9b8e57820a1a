// C++ host API (include/degpu.hpp) used the way the crate's tests use the crate:
// exp growth to t=10 with DOP853 rtol=atol=1e-12 (tests/ode/accuracy.rs:70-79) and a t_eval
// interpolation (tests/ode/interpolation.rs:14-87), plus an ensemble call.  Prints "ok" or fails.
#include <cmath>
#include <cstdio>

#include "degpu.hpp"

int main() {
    using namespace degpu;
    auto sol = IVP::ode(System::exponential_growth(1.0), 0.0, 10.0, {1.0})
                   .method(ExplicitRungeKutta::dop853().rtol(1e-12).atol(1e-12))
                   .solve();
    if (!sol.ok()) { std::printf("solve failed: %s\n", sol.error().msg.c_str()); return 1; }
    double y = sol.value().y.back()[0];
    if (std::fabs(y - 22026.46579479) >= 1e-3) { std::printf("accuracy %f\n", y); return 2; }
    auto s2 = IVP::ode(System::exponential_growth(1.0), 0.0, 2.0, {1.0})
                  .method(ExplicitRungeKutta::dopri5())
                  .t_eval({1.69, 0.5, 1.0})
                  .solve();
    if (!s2.ok() || s2.value().t.size() != 3 || s2.value().t[0] != 0.5) { std::printf("t_eval\n"); return 3; }
    if (std::fabs(s2.value().y[0][0] - std::exp(0.5)) >= 1e-3) { std::printf("interp\n"); return 4; }
    auto bad = IVP::ode(System::exponential_growth(1.0), 0.0, 1.0, {1.0})
                   .method(ExplicitRungeKutta::dopri5().h0(10.0))
                   .solve();
    if (bad.ok() || bad.error().kind != ErrorKind::BadInput || bad.error().msg.rfind("Invalid input", 0) != 0) {
        std::printf("bad input\n");
        return 5;
    }
    auto er = solve_ensemble(DEGPU_RHS_HARMONIC, 2, 1, {0.0, 0.0}, {10.0, 5.0}, {1.0, 1.0, 0.0, 0.0}, {1.0, 1.0},
                             {1e-10, 1e-10}, {1e-12, 1e-12}, ExplicitRungeKutta::dop853());
    if (er.status[0] != DEGPU_COMPLETE || std::fabs(er.y_final[0] - std::cos(10.0)) > 1e-8) { std::printf("ens\n"); return 6; }
    // crossings of the harmonic oscillator x = cos t: x = 0 at pi/2 + j pi, x + v = 0 at pi/4 + j pi
    const double pi = 3.141592653589793;
    auto hm = ExplicitRungeKutta::dop853().rtol(1e-11).atol(1e-11).dense_mode(DEGPU_DENSE_HAIRER);
    auto cx = IVP::ode(System::harmonic(1.0), 0.0, 10.0, {1.0, 0.0}).method(hm).crossing(0, 0.0).solve();
    if (!cx.ok() || cx.value().t.size() != 3 || std::fabs(cx.value().t[1] - 1.5 * pi) > 1e-9) {
        std::printf("crossing\n");
        return 7;
    }
    auto hx = IVP::ode(System::harmonic(1.0), 0.0, 10.0, {1.0, 0.0})
                  .method(hm)
                  .hyperplane_crossing({0.0, 0.0}, {2.0, 2.0}, {0, 1}, CrossingDirection::Negative)
                  .solve();
    // the signed distance (x + v)/sqrt(2) falls through zero at pi/4 + 2 j pi
    if (!hx.ok() || hx.value().t.size() != 2 || std::fabs(hx.value().t[1] - 2.25 * pi) > 1e-9) {
        std::printf("hyperplane\n");
        return 8;
    }
    auto hb = IVP::ode(System::harmonic(1.0), 0.0, 1.0, {1.0, 0.0}).hyperplane_crossing({0.0}, {1.0, 0.0}, {0}).solve();
    if (hb.ok() || hb.error().kind != ErrorKind::BadInput) {
        std::printf("hyperplane bad input\n");
        return 9;
    }
    // the crate's logistic example (examples/ode/03_logistic_growth): terminal event y - 0.9 m at ln 81
    degpu_event ev{};
    ev.kind = DEGPU_EVENT_LINEAR;
    ev.terminate = 1;
    ev.max_points = 4;
    ev.n_terms = 1;
    ev.components[0] = 0;
    ev.weights[0] = 1.0;
    ev.offset = -(0.9 * 10.0);
    auto lg = IVP::ode(System{DEGPU_RHS_LOGISTIC, {1.0, 10.0}}, 0.0, 10.0, {1.0})
                  .method(ExplicitRungeKutta::dop853().rtol(1e-12).atol(1e-12))
                  .t_eval({0.0, 2.0, 4.0, 6.0})
                  .event(ev)
                  .solve();
    if (!lg.ok() || !lg.value().interrupted || lg.value().t.size() != 4 ||
        std::fabs(lg.value().t[3] - std::log(81.0)) > 1e-7 || std::fabs(lg.value().y[3][0] - 9.0) > 1e-7) {
        std::printf("event\n");
        return 10;
    }
    // tests/ode/accuracy.rs:395-422 with Verner's RKV989e at its defaults
    auto vr = IVP::ode(System::harmonic(1.0), 0.0, 10.0, {1.0, 0.0}).method(ExplicitRungeKutta::rkv989e()).solve();
    if (!vr.ok() || std::fabs(vr.value().y.back()[0] - (-0.83907153)) >= 1e-3) {
        std::printf("verner\n");
        return 11;
    }
    std::printf("ok\n");
    return 0;
}
