// oracle.hpp — TEST INFRASTRUCTURE ONLY.  Never linked into, imported by or called from the
// product path.  This is the CPU restatement of the explicit Runge–Kutta path of the Rust crate
// `differential-equations` v0.6.1, written to follow the crate's algorithm operation by
// operation so that it can serve as the parity oracle of the GPU integrator:
//
//   solve_ode driver ................ src/ode/solve_ivp.rs:116-277
//   DormandPrince init/step/interp .. src/methods/erk/dormandprince/ordinary.rs:16-337
//   Fixed (RK4) init/step/interp .... src/methods/erk/fixed/ordinary.rs:16-221
//   InitialStepSize<Ordinary> ....... src/methods/h_init.rs:45-136
//   defaults ........................ src/methods/erk/mod.rs:112-159
//   constrain / validate ............ src/utils.rs:22-157
//   State algebra ................... src/traits.rs:316-410
//   cubic Hermite ................... src/interpolate.rs:40-60
//   Adaptive ERK (RKF45, Cash-Karp,  src/methods/erk/adaptive/ordinary.rs:16-290,
//   Verner RKV655e..RKV989e) ........ src/tableau/verner.rs
//   TEvalSolout ..................... src/solout/t_eval.rs:82-171
//   CrossingSolout .................. src/solout/crossing.rs:200-330, src/solout/hyperplane.rs
//   EventSolout ..................... src/solout/event.rs:67-521
//   tableaus ........................ src/tableau/runge_kutta.rs:39-70, src/tableau/dorman_prince.rs:37-381
//
// Compile with -ffp-contract=off: Rust never contracts a*b+c into an FMA, so neither may this.
//
// The crate calls the platform libm for `powf` (simba -> f64::powf -> pow) and for the
// `sin`/`cos` of user right-hand sides.  Two math modes are offered:
//   MathMode::Libm             — the host libm, what the crate itself calls on this machine;
//   MathMode::CorrectlyRounded — results rounded once from binary128 evaluations (libquadmath on
//                                x86-64, long double on aarch64), i.e. the correctly rounded
//                                value, which is what the GPU product computes.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../include/degpu.h"

namespace oracle {

// ---------------------------------------------------------------------------------------------
// Math policy
// ---------------------------------------------------------------------------------------------
enum class MathMode : int { Libm = 0, CorrectlyRounded = 1 };

double cr_pow(double x, double y);  // correctly rounded pow (binary128 evaluation)
double cr_sin(double x);
double cr_cos(double x);

struct Math {
    MathMode mode = MathMode::CorrectlyRounded;
    double pow(double x, double y) const { return mode == MathMode::Libm ? std::pow(x, y) : cr_pow(x, y); }
    double sin(double x) const { return mode == MathMode::Libm ? std::sin(x) : cr_sin(x); }
    double cos(double x) const { return mode == MathMode::Libm ? std::cos(x) : cr_cos(x); }
};

// ---------------------------------------------------------------------------------------------
// Butcher tableaus (transcribed from the crate; entries not set there are zero)
// ---------------------------------------------------------------------------------------------
struct Tableau {
    int S = 0;       // stages
    int I = 0;       // stages incl. dense-output stages
    int order = 0;   // O
    double c[32] = {};
    double a[32][32] = {};
    double b[32] = {};
    double bh[32] = {};
    bool has_bh = false;
    double er[32] = {};
    bool has_er = false;
    double bi[32][32] = {};
    bool has_bi = false;
    bool fsal = false;  // adaptive family: the last stage is the next step's first (ordinary.rs:174-177)
};

// src/tableau/runge_kutta.rs:39-70; constructor src/methods/erk/fixed/mod.rs:69-75 (O=4, S=I=4).
inline Tableau tableau_rk4() {
    Tableau t;
    t.S = 4; t.I = 4; t.order = 4;
    t.c[0] = 0.0; t.c[1] = 0.5; t.c[2] = 0.5; t.c[3] = 1.0;
    t.a[1][0] = 0.5;
    t.a[2][1] = 0.5;
    t.a[3][2] = 1.0;
    t.b[0] = 1.0 / 6.0; t.b[1] = 1.0 / 3.0; t.b[2] = 1.0 / 3.0; t.b[3] = 1.0 / 6.0;
    return t;
}

// src/tableau/runge_kutta.rs:335-406; constructor adaptive/mod.rs:43-50 (O=5, S=I=6).
inline Tableau tableau_rkf45() {
    Tableau t;
    t.S = 6; t.I = 6; t.order = 5;
    t.c[0] = 0.0; t.c[1] = 1.0 / 4.0; t.c[2] = 3.0 / 8.0; t.c[3] = 12.0 / 13.0; t.c[4] = 1.0; t.c[5] = 1.0 / 2.0;
    t.a[1][0] = 1.0 / 4.0;
    t.a[2][0] = 3.0 / 32.0; t.a[2][1] = 9.0 / 32.0;
    t.a[3][0] = 1932.0 / 2197.0; t.a[3][1] = -7200.0 / 2197.0; t.a[3][2] = 7296.0 / 2197.0;
    t.a[4][0] = 439.0 / 216.0; t.a[4][1] = -8.0; t.a[4][2] = 3680.0 / 513.0; t.a[4][3] = -845.0 / 4104.0;
    t.a[5][0] = -8.0 / 27.0; t.a[5][1] = 2.0; t.a[5][2] = -3544.0 / 2565.0; t.a[5][3] = 1859.0 / 4104.0;
    t.a[5][4] = -11.0 / 40.0;
    t.b[0] = 16.0 / 135.0; t.b[1] = 0.0; t.b[2] = 6656.0 / 12825.0; t.b[3] = 28561.0 / 56430.0;
    t.b[4] = -9.0 / 50.0; t.b[5] = 2.0 / 55.0;
    t.bh[0] = 25.0 / 216.0; t.bh[1] = 0.0; t.bh[2] = 1408.0 / 2565.0; t.bh[3] = 2197.0 / 4104.0;
    t.bh[4] = -1.0 / 5.0; t.bh[5] = 0.0;
    t.has_bh = true;
    return t;
}

// src/tableau/runge_kutta.rs:420-480; constructor adaptive/mod.rs:51-58 (O=5, S=I=6).
inline Tableau tableau_cash_karp() {
    Tableau t;
    t.S = 6; t.I = 6; t.order = 5;
    t.c[0] = 0.0; t.c[1] = 1.0 / 5.0; t.c[2] = 3.0 / 10.0; t.c[3] = 3.0 / 5.0; t.c[4] = 1.0; t.c[5] = 7.0 / 8.0;
    t.a[1][0] = 1.0 / 5.0;
    t.a[2][0] = 3.0 / 40.0; t.a[2][1] = 9.0 / 40.0;
    t.a[3][0] = 3.0 / 10.0; t.a[3][1] = -9.0 / 10.0; t.a[3][2] = 6.0 / 5.0;
    t.a[4][0] = -11.0 / 54.0; t.a[4][1] = 5.0 / 2.0; t.a[4][2] = -70.0 / 27.0; t.a[4][3] = 35.0 / 27.0;
    t.a[5][0] = 1631.0 / 55296.0; t.a[5][1] = 175.0 / 512.0; t.a[5][2] = 575.0 / 13824.0;
    t.a[5][3] = 44275.0 / 110592.0; t.a[5][4] = 253.0 / 4096.0;
    t.b[0] = 37.0 / 378.0; t.b[1] = 0.0; t.b[2] = 250.0 / 621.0; t.b[3] = 125.0 / 594.0; t.b[4] = 0.0;
    t.b[5] = 512.0 / 1771.0;
    t.bh[0] = 2825.0 / 27648.0; t.bh[1] = 0.0; t.bh[2] = 18575.0 / 48384.0; t.bh[3] = 13525.0 / 55296.0;
    t.bh[4] = 277.0 / 14336.0; t.bh[5] = 1.0 / 4.0;
    t.has_bh = true;
    return t;
}

// Verner's pairs (src/tableau/verner.rs; S, I, O and FSAL from src/methods/erk/adaptive/mod.rs:59-122).
// The coefficient tables are the crate's literals, generated into verner_tables.inc by
// differential-equations_gb300/csrc/gen_verner_tables.py.
namespace verner {
#include "verner_tables.inc"
}
template <class V>
inline Tableau tableau_verner() {
    Tableau t;
    t.S = V::S;
    t.I = V::I;
    t.order = V::ORDER;
    t.fsal = V::FSAL;
    for (int i = 0; i < V::I; ++i) {
        t.c[i] = V::C[i];
        for (int j = 0; j < V::I; ++j) {
            t.a[i][j] = V::A[i][j];
            t.bi[i][j] = V::BI[i][j];
        }
    }
    for (int i = 0; i < V::S; ++i) {
        t.b[i] = V::B[i];
        t.bh[i] = V::BH[i];
    }
    t.has_bh = true;
    t.has_bi = true;
    return t;
}
inline Tableau tableau_for_method(int method) {
    switch (method) {
        case DEGPU_RKF45: return tableau_rkf45();
        case DEGPU_CASH_KARP: return tableau_cash_karp();
        case DEGPU_RKV655E: return tableau_verner<verner::rkv655e>();
        case DEGPU_RKV656E: return tableau_verner<verner::rkv656e>();
        case DEGPU_RKV766E: return tableau_verner<verner::rkv766e>();
        case DEGPU_RKV767E: return tableau_verner<verner::rkv767e>();
        case DEGPU_RKV877E: return tableau_verner<verner::rkv877e>();
        case DEGPU_RKV878E: return tableau_verner<verner::rkv878e>();
        case DEGPU_RKV988E: return tableau_verner<verner::rkv988e>();
        default: return tableau_verner<verner::rkv989e>();
    }
}

// src/tableau/dorman_prince.rs:37-118; constructor dormandprince/mod.rs:52-58 (O=5, S=I=7).
inline Tableau tableau_dopri5() {
    Tableau t;
    t.S = 7; t.I = 7; t.order = 5;
    t.c[0] = 0.0; t.c[1] = 0.2; t.c[2] = 0.3; t.c[3] = 0.8; t.c[4] = 8.0 / 9.0; t.c[5] = 1.0; t.c[6] = 1.0;
    t.a[1][0] = 0.2;
    t.a[2][0] = 3.0 / 40.0; t.a[2][1] = 9.0 / 40.0;
    t.a[3][0] = 44.0 / 45.0; t.a[3][1] = -56.0 / 15.0; t.a[3][2] = 32.0 / 9.0;
    t.a[4][0] = 19372.0 / 6561.0; t.a[4][1] = -25360.0 / 2187.0; t.a[4][2] = 64448.0 / 6561.0;
    t.a[4][3] = -212.0 / 729.0;
    t.a[5][0] = 9017.0 / 3168.0; t.a[5][1] = -355.0 / 33.0; t.a[5][2] = 46732.0 / 5247.0;
    t.a[5][3] = 49.0 / 176.0; t.a[5][4] = -5103.0 / 18656.0;
    t.a[6][0] = 35.0 / 384.0; t.a[6][1] = 0.0; t.a[6][2] = 500.0 / 1113.0; t.a[6][3] = 125.0 / 192.0;
    t.a[6][4] = -2187.0 / 6784.0; t.a[6][5] = 11.0 / 84.0;
    t.b[0] = 35.0 / 384.0; t.b[1] = 0.0; t.b[2] = 500.0 / 1113.0; t.b[3] = 125.0 / 192.0;
    t.b[4] = -2187.0 / 6784.0; t.b[5] = 11.0 / 84.0; t.b[6] = 0.0;
    t.has_er = true;
    t.er[0] = 71.0 / 57600.0; t.er[1] = 0.0; t.er[2] = -71.0 / 16695.0; t.er[3] = 71.0 / 1920.0;
    t.er[4] = -17253.0 / 339200.0; t.er[5] = 22.0 / 525.0; t.er[6] = -1.0 / 40.0;
    // Only row 0 of `bi` is filled by the crate (dorman_prince.rs:95-101); the step reads row 4.
    t.has_bi = true;
    t.bi[0][0] = -12715105075.0 / 11282082432.0; t.bi[0][1] = 0.0;
    t.bi[0][2] = 87487479700.0 / 32700410799.0; t.bi[0][3] = -10690763975.0 / 1880347072.0;
    t.bi[0][4] = 701980252875.0 / 199316789632.0; t.bi[0][5] = -1453857185.0 / 822651844.0;
    t.bi[0][6] = 69997945.0 / 29380423.0;
    return t;
}

// src/tableau/dorman_prince.rs:155-381; constructor dormandprince/mod.rs:45-51 (O=8, S=12, I=16).
inline Tableau tableau_dop853() {
    Tableau t;
    t.S = 12; t.I = 16; t.order = 8;
    double* c = t.c;
    auto& a = t.a;
    c[0] = 0.0;
    c[1] = 5.260015195876773E-2;
    c[2] = 7.89002279381516E-2;
    c[3] = 1.183503419072274E-1;
    c[4] = 2.816496580927726E-1;
    c[5] = 3.333333333333333E-1;
    c[6] = 0.25E+00;
    c[7] = 3.076923076923077E-1;
    c[8] = 6.512820512820513E-1;
    c[9] = 0.6E+00;
    c[10] = 8.571428571428571E-1;
    c[11] = 1.0;

    a[1][0] = 5.260015195876773E-2;
    a[2][0] = 1.97250569845379E-2;
    a[2][1] = 5.91751709536137E-2;
    a[3][0] = 2.958758547680685E-2;
    a[3][2] = 8.876275643042054E-2;
    a[4][0] = 2.413651341592667E-1;
    a[4][2] = -8.845494793282861E-1;
    a[4][3] = 9.24834003261792E-1;
    a[5][0] = 3.7037037037037035E-2;
    a[5][3] = 1.7082860872947386E-1;
    a[5][4] = 1.2546768756682242E-1;
    a[6][0] = 3.7109375E-2;
    a[6][3] = 1.7025221101954405E-1;
    a[6][4] = 6.021653898045596E-2;
    a[6][5] = -1.7578125E-2;
    a[7][0] = 3.709200011850479E-2;
    a[7][3] = 1.7038392571223998E-1;
    a[7][4] = 1.0726203044637328E-1;
    a[7][5] = -1.5319437748624402E-2;
    a[7][6] = 8.273789163814023E-3;
    a[8][0] = 6.241109587160757E-1;
    a[8][3] = -3.3608926294469414;
    a[8][4] = -8.68219346841726E-1;
    a[8][5] = 2.759209969944671E1;
    a[8][6] = 2.0154067550477894E1;
    a[8][7] = -4.348988418106996E1;
    a[9][0] = 4.7766253643826434E-1;
    a[9][3] = -2.4881146199716677;
    a[9][4] = -5.90290826836843E-1;
    a[9][5] = 2.1230051448181193E1;
    a[9][6] = 1.5279233632882423E1;
    a[9][7] = -3.328821096898486E1;
    a[9][8] = -2.0331201708508627E-2;
    a[10][0] = -9.371424300859873E-1;
    a[10][3] = 5.186372428844064;
    a[10][4] = 1.0914373489967295;
    a[10][5] = -8.149787010746927;
    a[10][6] = -1.852006565999696E1;
    a[10][7] = 2.2739487099350505E1;
    a[10][8] = 2.4936055526796523;
    a[10][9] = -3.0467644718982196;
    a[11][0] = 2.273310147516538;
    a[11][3] = -1.053449546673725E1;
    a[11][4] = -2.0008720582248625;
    a[11][5] = -1.79589318631188E1;
    a[11][6] = 2.794888452941996E1;
    a[11][7] = -2.8589982771350235;
    a[11][8] = -8.87285693353063;
    a[11][9] = 1.2360567175794303E1;
    a[11][10] = 6.433927460157636E-1;

    double* b = t.b;
    b[0] = 5.4293734116568765E-2;
    b[5] = 4.450312892752409;
    b[6] = 1.8915178993145003;
    b[7] = -5.801203960010585;
    b[8] = 3.111643669578199E-1;
    b[9] = -1.521609496625161E-1;
    b[10] = 2.0136540080403034E-1;
    b[11] = 4.471061572777259E-2;

    t.has_bh = true;
    t.bh[0] = 2.440944881889764E-1;
    t.bh[8] = 7.338466882816118E-1;
    t.bh[11] = 2.2058823529411766E-2;

    t.has_er = true;
    t.er[0] = 1.312004499419488E-2;
    t.er[5] = -1.2251564463762044;
    t.er[6] = -4.957589496572502E-1;
    t.er[7] = 1.6643771824549864;
    t.er[8] = -3.5032884874997366E-1;
    t.er[9] = 3.341791187130175E-1;
    t.er[10] = 8.192320648511571E-2;
    t.er[11] = -2.2355307863886294E-2;

    c[13] = 0.1E+00;
    a[13][0] = 5.6167502283047954E-2;
    a[13][6] = 2.5350021021662483E-1;
    a[13][7] = -2.462390374708025E-1;
    a[13][8] = -1.2419142326381637E-1;
    a[13][9] = 1.5329179827876568E-1;
    a[13][10] = 8.20105229563469E-3;
    a[13][11] = 7.567897660545699E-3;
    a[13][12] = -8.298E-3;
    c[14] = 0.2E+00;
    a[14][0] = 3.183464816350214E-2;
    a[14][5] = 2.8300909672366776E-2;
    a[14][6] = 5.3541988307438566E-2;
    a[14][7] = -5.492374857139099E-2;
    a[14][10] = -1.0834732869724932E-4;
    a[14][11] = 3.825710908356584E-4;
    a[14][12] = -3.4046500868740456E-4;
    a[14][13] = 1.413124436746325E-1;
    c[15] = 7.777777777777778E-1;
    a[15][0] = -4.2889630158379194E-1;
    a[15][5] = -4.697621415361164;
    a[15][6] = 7.683421196062599;
    a[15][7] = 4.06898981839711;
    a[15][8] = 3.567271874552811E-1;
    a[15][12] = -1.3990241651590145E-3;
    a[15][13] = 2.9475147891527724;
    a[15][14] = -9.15095847217987;

    t.has_bi = true;
    auto& bi = t.bi;
    bi[4][0] = -8.428938276109013;
    bi[4][5] = 5.667149535193777E-1;
    bi[4][6] = -3.0689499459498917;
    bi[4][7] = 2.38466765651207;
    bi[4][8] = 2.117034582445028;
    bi[4][9] = -8.71391583777973E-1;
    bi[4][10] = 2.2404374302607883;
    bi[4][11] = 6.315787787694688E-1;
    bi[4][12] = -8.899033645133331E-2;
    bi[4][13] = 1.8148505520854727E1;
    bi[4][14] = -9.194632392478356;
    bi[4][15] = -4.436036387594894;
    bi[5][0] = 1.0427508642579134E1;
    bi[5][5] = 2.4228349177525817E2;
    bi[5][6] = 1.6520045171727028E2;
    bi[5][7] = -3.745467547226902E2;
    bi[5][8] = -2.2113666853125306E1;
    bi[5][9] = 7.733432668472264;
    bi[5][10] = -3.0674084731089398E1;
    bi[5][11] = -9.332130526430229;
    bi[5][12] = 1.5697238121770845E1;
    bi[5][13] = -3.1139403219565178E1;
    bi[5][14] = -9.35292435884448;
    bi[5][15] = 3.581684148639408E1;
    bi[6][0] = 1.9985053242002433E1;
    bi[6][5] = -3.870373087493518E2;
    bi[6][6] = -1.8917813819516758E2;
    bi[6][7] = 5.278081592054236E2;
    bi[6][8] = -1.157390253995963E1;
    bi[6][9] = 6.8812326946963;
    bi[6][10] = -1.0006050966910838;
    bi[6][11] = 7.777137798053443E-1;
    bi[6][12] = -2.778205752353508;
    bi[6][13] = -6.019669523126412E1;
    bi[6][14] = 8.432040550667716E1;
    bi[6][15] = 1.199229113618279E1;
    bi[7][0] = -2.569393346270375E1;
    bi[7][5] = -1.5418974869023643E2;
    bi[7][6] = -2.315293791760455E2;
    bi[7][7] = 3.576391179106141E2;
    bi[7][8] = 9.340532418362432E1;
    bi[7][9] = -3.745832313645163E1;
    bi[7][10] = 1.040996495089623E2;
    bi[7][11] = 2.98402934266605E1;
    bi[7][12] = -4.353345659001114E1;
    bi[7][13] = 9.632455395918828E1;
    bi[7][14] = -3.917726167561544E1;
    bi[7][15] = -1.4972683625798564E2;
    return t;
}

// ---------------------------------------------------------------------------------------------
// State algebra — src/traits.rs:316-410 (generic) and :587-595 ([T; N]).  Each `+=` is one IEEE
// multiply followed by one IEEE add.
// ---------------------------------------------------------------------------------------------
using State = std::vector<double>;

inline void add_scaled(State& self, double alpha, const State& other) {  // traits.rs:316-320
    for (size_t i = 0; i < self.size(); ++i) self[i] += alpha * other[i];
}
inline State plus_scaled(const State& self, double alpha, const State& other) {  // traits.rs:336-340
    State out = self;
    add_scaled(out, alpha, other);
    return out;
}
inline State minus(const State& self, const State& other) {  // traits.rs:352-354
    return plus_scaled(self, -1.0, other);
}
inline void scale_by(State& self, double alpha) {  // traits.rs:323-326
    for (auto& v : self) v *= alpha;
}
inline void fill(State& self, double v) {
    for (auto& x : self) x = v;
}
inline double diff_norm_squared(const State& self, const State& other) {  // traits.rs:383-391
    double sum = 0.0;
    for (size_t i = 0; i < self.size(); ++i) {
        double diff = self[i] - other[i];
        sum += diff * diff;
    }
    return sum;
}
// src/tolerance.rs:11-40: a scalar tolerance (which every index reads) or one per component.
struct Tolerance {
    double scalar = 0.0;
    std::vector<double> vec;
    Tolerance() = default;
    Tolerance(double v) : scalar(v) {}  // From<T> (tolerance.rs:52-56)
    double operator[](size_t i) const { return vec.empty() ? scalar : vec[i]; }  // Index (tolerance.rs:33-40)
};

// traits.rs:394-410.
inline double error_norm(const State& self, const State& y_new, const State& err, const Tolerance& atol,
                         const Tolerance& rtol) {
    double sum = 0.0;
    for (size_t i = 0; i < self.size(); ++i) {
        double sk = atol[i] + rtol[i] * std::fmax(std::fabs(self[i]), std::fabs(y_new[i]));
        double e = err[i] / sk;
        sum += e * e;
    }
    return sum;
}

// ---------------------------------------------------------------------------------------------
// ODE right-hand sides (`ODE::diff`, src/ode/ode.rs:20-44)
// ---------------------------------------------------------------------------------------------
struct Ode {
    virtual ~Ode() = default;
    virtual void diff(double t, const State& y, State& dydt) const = 0;
};

// Built-in families; parameters p[] in the order documented in include/degpu.h.
struct BuiltinOde : Ode {
    int rhs_id;
    int dim;
    std::vector<double> p;
    Math math;
    BuiltinOde(int id, int d, std::vector<double> params, Math m) : rhs_id(id), dim(d), p(std::move(params)), math(m) {}
    void diff(double t, const State& y, State& dydt) const override;
};

// Returns (dim, n_params); dim = -1 for variable-size families; rhs_id unknown -> n_params = -1.
inline void builtin_info(int rhs_id, int& dim, int& np) {
    switch (rhs_id) {
        case DEGPU_RHS_LORENZ: dim = 3; np = 3; return;
        case DEGPU_RHS_VAN_DER_POL: dim = 2; np = 1; return;
        case DEGPU_RHS_PENDULUM: dim = 2; np = 3; return;
        case DEGPU_RHS_FPU_BETA: dim = -1; np = 1; return;
        case DEGPU_RHS_EXP_GROWTH: dim = 1; np = 1; return;
        case DEGPU_RHS_LINEAR: dim = 1; np = 2; return;
        case DEGPU_RHS_HARMONIC: dim = 2; np = 1; return;
        case DEGPU_RHS_LOGISTIC: dim = 1; np = 2; return;
        case DEGPU_RHS_ROBERTSON: dim = 3; np = 0; return;
        case DEGPU_RHS_HIRES: dim = 8; np = 0; return;
        case DEGPU_RHS_BRUSSELATOR: dim = 2; np = 2; return;
        case DEGPU_RHS_CR3BP: dim = 6; np = 1; return;
        case DEGPU_RHS_PIPE_HEAT: dim = 2; np = 2; return;
        case DEGPU_RHS_DAMPED_QUADRATURE: dim = 3; np = 3; return;
        default: dim = 0; np = -1; return;
    }
}

inline void BuiltinOde::diff(double t, const State& y, State& dydt) const {
    switch (rhs_id) {
        case DEGPU_RHS_LORENZ: {  // tests/ode/systems.rs:91-100
            double sigma = p[0], rho = p[1], beta = p[2];
            double x = y[0], yv = y[1], z = y[2];
            dydt[0] = sigma * (yv - x);
            dydt[1] = x * (rho - z) - yv;
            dydt[2] = x * yv - beta * z;
            return;
        }
        case DEGPU_RHS_VAN_DER_POL: {  // tests/ode/systems.rs:70-77
            double mu = p[0];
            double y1 = y[0], y2 = y[1];
            dydt[0] = y2;
            dydt[1] = mu * (1.0 - y1 * y1) * y2 - y1;
            return;
        }
        case DEGPU_RHS_PENDULUM: {
            // Damped driven pendulum with g/l = 1: the model of
            // examples/ode/05_damped_pendulum/main.rs:34-40 plus a drive A cos(Omega t).
            double gamma = p[0], A = p[1], Omega = p[2];
            double theta = y[0], omega = y[1];
            dydt[0] = omega;
            dydt[1] = -gamma * omega - math.sin(theta) + A * math.cos(Omega * t);
            return;
        }
        case DEGPU_RHS_FPU_BETA: {
            // FPU-beta chain, m = d/2 masses, fixed ends x_0 = x_{m+1} = 0, Hamiltonian layout
            // y = [x_1..x_m, p_1..p_m] (src/ivp.rs:329).  Delta_i = x_{i+1} - x_i.
            double beta = p[0];
            int m = (int)y.size() / 2;
            double dprev = y[0] - 0.0;  // Delta_0 = x_1 - x_0
            for (int i = 0; i < m; ++i) {
                double xnext = (i + 1 < m) ? y[i + 1] : 0.0;
                double dcur = xnext - y[i];  // Delta_{i+1} in 1-based masses
                dydt[i] = y[m + i];
                dydt[m + i] = (dcur - dprev) + beta * (dcur * dcur * dcur - dprev * dprev * dprev);
                dprev = dcur;
            }
            return;
        }
        case DEGPU_RHS_EXP_GROWTH: dydt[0] = p[0] * y[0]; return;       // systems.rs:14-16
        case DEGPU_RHS_LINEAR: dydt[0] = p[0] + p[1] * y[0]; return;    // systems.rs:28-30
        case DEGPU_RHS_HARMONIC:                                         // systems.rs:42-45
            dydt[0] = y[1];
            dydt[1] = -p[0] * y[0];
            return;
        case DEGPU_RHS_LOGISTIC:                                         // systems.rs:57-59
            dydt[0] = p[0] * y[0] * (1.0 - y[0] / p[1]);
            return;
        case DEGPU_RHS_ROBERTSON: {                                      // systems.rs:164-172
            double y1 = y[0], y2 = y[1], y3 = y[2];
            dydt[0] = -0.04 * y1 + 1.0e4 * y2 * y3;
            dydt[1] = 0.04 * y1 - 1.0e4 * y2 * y3 - 3.0e7 * y2 * y2;
            dydt[2] = 3.0e7 * y2 * y2;
            return;
        }
        case DEGPU_RHS_HIRES:                                            // systems.rs:180-189
            dydt[0] = -1.71 * y[0] + 0.43 * y[1] + 8.32 * y[2] + 0.0007;
            dydt[1] = 1.71 * y[0] - 8.75 * y[1];
            dydt[2] = -10.03 * y[2] + 0.43 * y[3] + 0.035 * y[4];
            dydt[3] = 8.32 * y[1] + 1.71 * y[2] - 1.12 * y[3];
            dydt[4] = -1.745 * y[4] + 0.43 * y[5] + 0.43 * y[6];
            dydt[5] = -280.0 * y[5] * y[7] + 0.69 * y[3] + 1.71 * y[4] - 0.43 * y[5] + 0.69 * y[6];
            dydt[6] = 280.0 * y[5] * y[7] - 1.81 * y[6];
            dydt[7] = -280.0 * y[5] * y[7] + 1.81 * y[6];
            return;
        case DEGPU_RHS_BRUSSELATOR: {                                    // systems.rs:113-119
            double a = p[0], b = p[1], y1 = y[0], y2 = y[1];
            dydt[0] = a + y1 * y1 * y2 - (b + 1.0) * y1;
            dydt[1] = b * y1 - y1 * y1 * y2;
            return;
        }
        case DEGPU_RHS_PIPE_HEAT: {  // tests/bvp/systems.rs:45-50; powi(2) -> b*b
            const double b = p[0], amb = p[1];
            dydt[0] = y[1];
            dydt[1] = (b * b) * (y[0] - amb);
            return;
        }
        case DEGPU_RHS_DAMPED_QUADRATURE: {  // examples/ode/17_quadrature/main.rs:47-55
            const double k = p[0], m = p[1], c = p[2], x = y[0], v = y[1];
            dydt[0] = v;
            dydt[1] = -(k / m) * x - (c / m) * v;
            dydt[2] = c * v * v;
            return;
        }
        case DEGPU_RHS_CR3BP: {                                          // systems.rs:131-152
            // powi(2) and powi(3) lower to x*x and x*(x*x) (LLVM's multiply expansion).
            double mu = p[0];
            double rx = y[0], ry = y[1], rz = y[2], vx = y[3], vy = y[4], vz = y[5];
            auto sq = [](double v) { return v * v; };
            auto cube = [](double v) { return v * (v * v); };
            double r13 = std::sqrt(sq(rx + mu) + sq(ry) + sq(rz));
            double r23 = std::sqrt(sq(rx - 1.0 + mu) + sq(ry) + sq(rz));
            dydt[0] = vx;
            dydt[1] = vy;
            dydt[2] = vz;
            dydt[3] = rx + 2.0 * vy - (1.0 - mu) * (rx + mu) / cube(r13) - mu * (rx - 1.0 + mu) / cube(r23);
            dydt[4] = ry - 2.0 * vx - (1.0 - mu) * ry / cube(r13) - mu * ry / cube(r23);
            dydt[5] = -(1.0 - mu) * rz / cube(r13) - mu * rz / cube(r23);
            return;
        }
        default: return;
    }
}

// ---------------------------------------------------------------------------------------------
// Errors / status (src/error.rs:13-40, src/status.rs:26-45)
// ---------------------------------------------------------------------------------------------
struct Outcome {
    int status = DEGPU_COMPLETE;  // degpu_instance_status
    std::string msg;              // BadInput message, starts with "Invalid input" where the crate's does
    double t = 0.0;               // Error{t, y}
    State y;
};

// src/utils.rs:22-33
inline double constrain_step_size(double h, double h_min, double h_max) {
    double sign = std::copysign(1.0, h);  // f64::signum: +-1 (also for +-0), NaN for NaN
    if (std::isnan(h)) sign = h;
    if (std::fabs(h) < h_min) return sign * h_min;
    if (std::fabs(h) > h_max) return sign * h_max;
    return h;
}

// f64::signum (std): 1.0 for +0.0 and positive, -1.0 for -0.0 and negative, NaN for NaN.
inline double rust_signum(double x) {
    if (std::isnan(x)) return x;
    return std::copysign(1.0, x);
}

// src/utils.rs:60-157.  Returns true and sets h_out on success, false and fills `o` otherwise.
inline bool validate_step_size_parameters(double h0, double h_min, double h_max, double t0, double tf, double& h_out,
                                          Outcome& o) {
    auto bad = [&](const char* m) {
        o.status = DEGPU_ERR_BAD_INPUT;
        o.msg = m;
        return false;
    };
    if (tf == t0) return bad("Invalid input: tf cannot be equal to t0");
    double sign = rust_signum(tf - t0);
    if (rust_signum(h0) != sign)
        return bad("Invalid input: Initial step size must have the same sign as the integration direction");
    if (h_min < 0.0) return bad("Invalid input: Minimum step size must be non-negative");
    if (h_max < 0.0) return bad("Invalid input: Maximum step size must be non-negative");
    if (h_min > h_max) return bad("Invalid input: Minimum step size must be less than or equal to maximum step size");
    if (std::fabs(h0) < h_min)
        return bad("Invalid input: Absolute value of initial step size must be greater than or equal to minimum step size");
    if (std::fabs(h0) > h_max)
        return bad("Invalid input: Absolute value of initial step size must be less than or equal to maximum step size");
    if (std::fabs(h0) > std::fabs(tf - t0))
        return bad("Invalid input: Absolute value of initial step size must be less than or equal to the absolute value of the integration interval");
    if (h0 == 0.0) return bad("Invalid input: Initial step size cannot be zero");
    h_out = h0;
    return true;
}

struct Settings {  // src/methods/erk/mod.rs:112-159 defaults
    Tolerance rtol = 1.0e-6;
    Tolerance atol = 1.0e-6;
    double h0 = 0.0;
    double h_min = 0.0;
    double h_max = std::numeric_limits<double>::infinity();
    int64_t max_steps = 10000;
    double safety_factor = 0.9;
    double min_scale = 0.2;
    double max_scale = 10.0;
};

// src/methods/h_init.rs:45-136 (InitialStepSize<Ordinary>::compute).
inline double h_init(const Ode& ode, double t0, double tf, const State& y0, int order, const Tolerance& rtol,
                     const Tolerance& atol, double h_min, double h_max, int64_t& fevals, const Math& math) {
    double posneg = rust_signum(tf - t0);
    size_t n_dim = y0.size();
    State f0(n_dim, 0.0), f1(n_dim, 0.0);
    ode.diff(t0, y0, f0);
    fevals += 1;
    double dnf = 0.0, dny = 0.0;
    std::vector<double> sk_vec(n_dim);
    for (size_t n = 0; n < n_dim; ++n) {
        double sk = atol[n] + rtol[n] * std::fabs(y0[n]);
        sk_vec[n] = sk;
        double a = f0[n] / sk;
        dnf += a * a;  // powi(2) -> x*x
        double b = y0[n] / sk;
        dny += b * b;
    }
    double h;
    if (dnf <= 1.0e-10 || dny <= 1.0e-10) {
        h = 1.0e-6;
    } else {
        h = std::sqrt(dny / dnf) * 0.01;
    }
    h = std::fmin(h, h_max);
    h *= posneg;
    State y1 = plus_scaled(y0, h, f0);
    ode.diff(t0 + h, y1, f1);
    fevals += 1;
    double der2 = 0.0;
    for (size_t n = 0; n < n_dim; ++n) {
        double q = (f1[n] - f0[n]) / sk_vec[n];
        der2 += q * q;
    }
    der2 = std::sqrt(der2) / std::fabs(h);
    double der12 = std::fmax(std::sqrt(dnf), der2);
    double h1;
    if (der12 <= 1.0e-15) {
        h1 = std::fabs(h) * std::fmax(1.0e-3, 1.0e-6);
    } else {
        double order_t = (double)order;
        h1 = math.pow(0.01 / der12, 1.0 / order_t);
    }
    // (h.abs() * 100).min(h1).min(h_max).max(h_min).min(interval)
    double interval = std::fabs(tf - t0);
    h = std::fmin(std::fmax(std::fmin(std::fmin(std::fabs(h) * 100.0, h1), h_max), h_min), interval);
    return h * posneg;
}

// ---------------------------------------------------------------------------------------------
// Dense-output requests: TEvalSolout (src/solout/t_eval.rs:82-171)
// ---------------------------------------------------------------------------------------------
struct Interpolator {
    virtual ~Interpolator() = default;
    virtual State interpolate(double t_interp) = 0;
};

// The time of the last point pushed to the solution by any solout (`solution.t.last()`), which
// EventWrappedSolout compares with a new event time before it pushes it.
struct PushLog {
    bool any = false;
    double last = 0.0;
    void push(double t) {
        any = true;
        last = t;
    }
};

struct TEvalSolout {
    PushLog* log = nullptr;         // optional: records the pushed times
    std::vector<double> t_evals;    // sorted by direction
    std::vector<int> order;         // t_evals[k] came from caller index order[k]
    size_t next_eval_idx = 0;
    double integration_direction = 1.0;
    // outputs, indexed by the caller's point index; unset points stay NaN
    std::vector<State>* out = nullptr;

    TEvalSolout(const std::vector<double>& pts, double t0, double tf, std::vector<State>* dense_out) {
        integration_direction = rust_signum(tf - t0);
        std::vector<int> idx(pts.size());
        for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int)i;
        // stable sort by direction (sort_by is stable; NaN compare as Equal)
        auto less = [&](int a, int b) {
            double x = pts[a], y = pts[b];
            if (integration_direction > 0.0) return x < y;
            return x > y;
        };
        for (size_t i = 1; i < idx.size(); ++i) {  // insertion sort: stable
            int v = idx[i];
            size_t j = i;
            while (j > 0 && less(v, idx[j - 1])) {
                idx[j] = idx[j - 1];
                --j;
            }
            idx[j] = v;
        }
        order = idx;
        t_evals.resize(pts.size());
        for (size_t i = 0; i < idx.size(); ++i) t_evals[i] = pts[idx[i]];
        out = dense_out;
    }

    void solout(double t_curr, double t_prev, const State& y_curr, Interpolator& interp) {
        size_t idx = next_eval_idx;
        while (idx < t_evals.size()) {
            double t_eval = t_evals[idx];
            bool in_range;
            if (integration_direction > 0.0)
                in_range = (t_eval == t_prev && idx == 0) || (t_eval > t_prev && t_eval <= t_curr);
            else
                in_range = (t_eval == t_prev && idx == 0) || (t_eval < t_prev && t_eval >= t_curr);
            if (in_range) {
                if (t_eval == t_curr)
                    (*out)[order[idx]] = y_curr;
                else
                    (*out)[order[idx]] = interp.interpolate(t_eval);
                if (log) log->push(t_eval);
                idx += 1;
            } else {
                if ((integration_direction > 0.0 && t_eval > t_curr) ||
                    (integration_direction < 0.0 && t_eval < t_curr))
                    break;
                idx += 1;
            }
        }
        next_eval_idx = idx;
    }
};

// ---------------------------------------------------------------------------------------------
// Crossing detection: CrossingSolout (src/solout/crossing.rs:200-330) and
// HyperplaneCrossingSolout (src/solout/hyperplane.rs). After each call (at t0 and after every
// accepted step) the monitored offset is compared in sign with the previous one:
//   * component form: y[comp] - threshold;
//   * hyperplane form: the signed distance (pos - point) . normal, pos[j] = y[plane_comp[j]],
//     with the normal scaled to unit length at construction; leaving or reaching the plane
//     exactly also counts as a crossing.
// A crossing in the requested direction is located by find_crossing_newton on the step's
// interpolant, or by the linear estimate when that does not converge.
// ---------------------------------------------------------------------------------------------
struct CrossingSolout {
    int comp = 0;
    double threshold = 0.0;
    int direction = 0;  // 0 both, 1 positive (from below), -1 negative
    bool plane = false;
    std::vector<int> plane_comp;
    std::vector<double> plane_point, plane_normal;
    bool have_last = false;
    double last_offset = 0.0;
    std::vector<double> t;  // crossings in the order found
    std::vector<State> y;

    // HyperplaneCrossingSolout::new: normal *= 1/|normal| when |normal| > eps; the squared norm
    // folds from zero in component order (src/traits.rs:574-576), scale_by multiplies each
    // component (src/traits.rs:323-326).
    void set_plane(const std::vector<int>& comps, const std::vector<double>& point, const std::vector<double>& normal) {
        plane = true;
        plane_comp = comps;
        plane_point = point;
        plane_normal = normal;
        double nn = 0.0;
        for (double v : plane_normal) nn = nn + v * v;
        const double norm = std::sqrt(nn);
        if (norm > std::numeric_limits<double>::epsilon()) {
            const double inv = 1.0 / norm;
            for (double& v : plane_normal) v = v * inv;
        }
    }

    // crossing.rs:207 / hyperplane.rs signed_distance: (extract(y) - point).dot(normal), the dot
    // folded from zero in component order (src/traits.rs:551-555)
    double offset(const State& v) const {
        if (!plane) return v[comp] - threshold;
        double sum = 0.0;
        for (size_t j = 0; j < plane_comp.size(); ++j) {
            const double d = v[plane_comp[j]] - plane_point[j];
            sum = sum + d * plane_normal[j];
        }
        return sum;
    }

    void solout(double t_curr, double t_prev, const State& y_curr, Interpolator& interp) {
        const double off = offset(y_curr);
        if (have_last) {
            bool is_crossing = rust_signum(last_offset) != rust_signum(off);  // crossing.rs:210
            if (plane)  // hyperplane.rs: the zero cases
                is_crossing = is_crossing || (last_offset == 0.0 && off != 0.0) || (last_offset != 0.0 && off == 0.0);
            if (is_crossing) {
                bool record;  // crossing.rs:214-218
                if (direction > 0)
                    record = last_offset < 0.0 && off >= 0.0;
                else if (direction < 0)
                    record = last_offset > 0.0 && off <= 0.0;
                else
                    record = true;
                if (record) {
                    double tc;
                    if (!find_crossing_newton(interp, t_prev, t_curr, last_offset, off, tc)) {
                        // crossing.rs:234-238: linear estimate
                        const double frac = -last_offset / (off - last_offset);
                        tc = t_prev + frac * (t_curr - t_prev);
                    }
                    t.push_back(tc);
                    y.push_back(interp.interpolate(tc));
                }
            }
        }
        last_offset = off;
        have_last = true;
    }

    // crossing.rs:254-328; the hyperplane form breaks on a derivative below eps (not 10 eps)
    // and has no step-change test
    bool find_crossing_newton(Interpolator& interp, double t_lower, double t_upper, double offset_lower,
                              double offset_upper, double& t_out) const {
        const double eps = std::numeric_limits<double>::epsilon();
        double t = t_lower - offset_lower * (t_upper - t_lower) / (offset_upper - offset_lower);
        const double tolerance = eps * 100.0;
        double off;
        for (int it = 0; it < 10; ++it) {
            off = offset(interp.interpolate(t));
            if (std::fabs(off) < tolerance) {
                t_out = t;
                return true;
            }
            const double delta_t = (t_upper - t_lower) * 1e-6;
            const double t_plus = t + delta_t;
            const double offset_plus = offset(interp.interpolate(t_plus));
            const double derivative = (offset_plus - off) / delta_t;
            if (std::fabs(derivative) < (plane ? eps : eps * 10.0)) break;
            const double t_new = t - off / derivative;
            if (t_new < t_lower || t_new > t_upper) {
                t = (t_lower + t_upper) / 2.0;
            } else {
                const double change = std::fabs(t_new - t);
                if (!plane && change < tolerance * 0.1) {
                    t = t_new;
                    break;
                }
                t = t_new;
            }
        }
        off = offset(interp.interpolate(t));
        if (std::fabs(off) < tolerance * 10.0) {
            t_out = t;
            return true;
        }
        return false;
    }
};

// ---------------------------------------------------------------------------------------------
// Event detection: EventWrappedSolout (src/solout/event.rs:299-521; EventSolout, event.rs:67-297,
// is the same detector without a base). After the base output of each call, the event function
// g(t, y) at the step's end is compared in sign with its value at the previous call (the first
// call, at t0, only records it). A change of sign in the requested direction is located by the
// crate's Brent–Dekker search on the step's interpolant; a located event is pushed unless it lies
// within abs_tol of the last point already in the solution, is counted either way, and ends the
// solve (Status::Interrupted) once `terminate` events were counted. The event functions are the
// two forms of the crate's examples:
//   LINEAR  g = ((sum_j w_j y[c_j]) + w_t t) + offset, folded from zero in term order
//           (`y[0] - 0.9 * m`, `t - 10.0`, `y.infected - 1.0`);
//   MAX_ABS g = max_j |y[c_j]| + offset, f64::max folded from the first term
//           (`theta.abs().max(omega.abs()) - 0.01`).
// ---------------------------------------------------------------------------------------------
struct EventSolout {
    int kind = DEGPU_EVENT_LINEAR;
    std::vector<int> comp;
    std::vector<double> w;
    double t_weight = 0.0, offset = 0.0;
    int direction = 0;   // CrossingDirection
    int terminate = 0;   // EventConfig::terminate; 0 = None
    double integration_direction = 1.0;
    double rel_tol = 1e-12, abs_tol = 1e-14;  // event.rs:329-330
    bool have_last = false;
    double last_g = 0.0;
    int64_t event_count = 0;
    PushLog* log = nullptr;
    std::vector<double> t;  // pushed event points
    std::vector<State> y;

    double g(double te, const State& v) const {
        if (kind == DEGPU_EVENT_MAX_ABS) {
            double m = std::fabs(v[comp[0]]);
            for (size_t j = 1; j < comp.size(); ++j) m = std::fmax(m, std::fabs(v[comp[j]]));  // f64::max
            return m + offset;
        }
        double sum = 0.0;
        for (size_t j = 0; j < comp.size(); ++j) {
            const double term = w[j] * v[comp[j]];
            sum = sum + term;
        }
        const double tt = t_weight * te;
        sum = sum + tt;
        return sum + offset;
    }

    // Returns true when the solve is to stop (ControlFlag::Terminate).
    bool solout(double t_curr, double t_prev, const State& y_curr, Interpolator& interp) {
        const double g_curr = g(t_curr, y_curr);
        if (!have_last) {  // event.rs:335-350: the first call only records g
            have_last = true;
            last_g = g_curr;
            return false;
        }
        const double g_prev = last_g;
        const bool sign_change = rust_signum(g_prev) != rust_signum(g_curr);
        bool direction_ok;
        if (direction > 0)
            direction_ok = sign_change && g_prev < 0.0 && g_curr >= 0.0;
        else if (direction < 0)
            direction_ok = sign_change && g_prev > 0.0 && g_curr <= 0.0;
        else
            direction_ok = sign_change;
        if (direction_ok) {
            double a = t_prev, b = t_curr, fa = g_prev, fb = g_curr;
            if ((integration_direction > 0.0 && a > b) || (integration_direction < 0.0 && a < b)) {
                std::swap(a, b);
                std::swap(fa, fb);
            }
            double t_event;
            if (fa * fb <= 0.0 && brent_dekker(a, b, fa, fb, t_prev, t_curr, interp, t_event)) {
                const State y_event = interp.interpolate(t_event);
                const bool push_point = !log->any || std::fabs(t_event - log->last) > abs_tol;
                if (push_point) {
                    t.push_back(t_event);
                    y.push_back(y_event);
                    log->push(t_event);
                }
                event_count += 1;
                if (terminate > 0 && event_count >= terminate) {
                    last_g = g_curr;
                    return true;
                }
            }
        }
        last_g = g_curr;
        return false;
    }

    // event.rs:395-490. The crate's interpolator refuses times outside [t_prev, t_curr]
    // (OutOfBounds), which ends the search without a root.
    bool brent_dekker(double a, double b, double fa, double fb, double t_lo, double t_hi, Interpolator& interp,
                      double& root) const {
        if (std::fabs(fa) < std::fabs(fb)) {
            std::swap(a, b);
            std::swap(fa, fb);
        }
        double c = a, fc = fa, d = b - a, e = d;
        const double one = 1.0, two = 2.0, half = one / two, three = 3.0;
        for (int it = 0; it < 50; ++it) {
            if (fb == 0.0) {
                root = b;
                return true;
            }
            if (rust_signum(fa) == rust_signum(fb)) {
                a = c;
                fa = fc;
                c = b;
                fc = fb;
                d = b - a;
                e = d;
            }
            if (std::fabs(fa) < std::fabs(fb)) {
                c = b;
                b = a;
                a = c;
                fc = fb;
                fb = fa;
                fa = fc;
            }
            const double tol = std::fmax(abs_tol, rel_tol * std::fabs(b));
            const double m = half * (a - b);
            if (std::fabs(m) <= tol || fb == 0.0) {
                root = b;
                return true;
            }
            bool use_bis = true;
            if (std::fabs(e) > tol && std::fabs(fa) > std::fabs(fb)) {
                const double s = fb / fa;
                double p, q;
                if (a == c) {
                    p = two * m * s;
                    q = one - s;
                } else {
                    const double q1 = fa / fc;
                    const double r = fb / fc;
                    p = s * (two * m * q1 * (q1 - r) - (b - a) * (r - one));
                    q = (q1 - one) * (r - one) * (s - one);
                }
                if (q > 0.0)
                    p = -p;
                else
                    q = -q;
                if (std::fabs(two * p) < (three * m * q - std::fabs(tol * q)) && p < std::fabs(e * half * q)) {
                    e = d;
                    d = p / q;
                    use_bis = false;
                }
            }
            if (use_bis) {
                d = m;
                e = m;
            }
            a = b;
            fa = fb;
            if (std::fabs(d) > tol)
                b = b + d;
            else
                b = b + (m > 0.0 ? tol : -tol);
            if (b < t_lo || b > t_hi) return false;  // interpolate(b).ok()?
            fb = g(b, interp.interpolate(b));
            c = a;
            fc = fa;
        }
        return false;
    }
};

// ---------------------------------------------------------------------------------------------
// Numerical methods
// ---------------------------------------------------------------------------------------------
enum class Status { Uninitialized, Initialized, Solving, RejectedStep, Complete, Error };

// DormandPrince family: src/methods/erk/dormandprince/ordinary.rs.
struct DormandPrince : Interpolator {
    Tableau tab;
    Settings set;
    Math math;
    bool hairer_dense = false;  // opt-in: published DOP853 continuous extension fold

    double h = 0.0, t = 0.0, h_prev = 0.0, t_prev = 0.0;
    State y, dydt, y_prev, dydt_prev;
    std::vector<State> k;     // [I]
    std::vector<State> cont;  // [O]
    int64_t stiffness_counter = 0, non_stiffness_counter = 0, steps = 0;
    Status status = Status::Uninitialized;

    // ordinary.rs:16-61
    bool init(const Ode& ode, double t0, double tf, const State& y0, int64_t& fevals, Outcome& o) {
        if (set.h0 == 0.0)
            set.h0 = h_init(ode, t0, tf, y0, tab.order, set.rtol, set.atol, set.h_min, set.h_max, fevals, math);
        double h0v;
        if (!validate_step_size_parameters(set.h0, set.h_min, set.h_max, t0, tf, h0v, o)) return false;
        h = h0v;
        stiffness_counter = 0;
        t = t0;
        y = y0;
        size_t n = y0.size();
        dydt.assign(n, 0.0);
        y_prev = y0;
        dydt_prev.assign(n, 0.0);
        k.assign(tab.I, State(n, 0.0));
        cont.assign(tab.order, State(n, 0.0));
        ode.diff(t, y, k[0]);
        dydt = k[0];
        fevals += 1;
        t_prev = t;
        y_prev = y;
        dydt_prev = dydt;
        status = Status::Initialized;
        return true;
    }

    // ordinary.rs:63-268.  Returns false with `o` filled on an error.
    bool step(const Ode& ode, int64_t& fevals, Outcome& o) {
        if (std::fabs(h) < std::fabs(h_prev) * 1e-14) {
            status = Status::Error;
            o.status = DEGPU_ERR_STEP_SIZE;
            o.t = t;
            o.y = y;
            return false;
        }
        if (steps >= set.max_steps) {
            status = Status::Error;
            o.status = DEGPU_ERR_MAX_STEPS;
            o.t = t;
            o.y = y;
            return false;
        }
        steps += 1;

        const int S = tab.S, I = tab.I;
        size_t n = y.size();
        State y_stage(n, 0.0);
        for (int i = 1; i < S; ++i) {
            y_stage = y;
            for (int j = 0; j < i; ++j) add_scaled(y_stage, tab.a[i][j] * h, k[j]);
            ode.diff(t + tab.c[i] * h, y_stage, k[i]);
        }
        State ysti = y_stage;

        State yseg(n, 0.0);
        for (int i = 0; i < S; ++i) add_scaled(yseg, tab.b[i], k[i]);
        State y_new = plus_scaled(y, h, yseg);
        double t_new = t + h;
        fevals += S - 1;

        double err2 = 0.0;
        State err_state(n, 0.0);
        for (int j = 0; j < S; ++j) add_scaled(err_state, tab.er[j], k[j]);
        double err = error_norm(y, y_new, err_state, set.atol, set.rtol);
        if (tab.has_bh) {
            State err2_state = yseg;
            for (int j = 0; j < S; ++j) add_scaled(err2_state, -tab.bh[j], k[j]);
            err2 = error_norm(y, y_new, err2_state, set.atol, set.rtol);
        }
        double deno = err + 0.01 * err2;
        if (deno <= 0.0) deno = 1.0;
        err = std::fabs(h) * err * std::sqrt(1.0 / (deno * (double)n));

        double order = (double)tab.order;
        double error_exponent = 1.0 / order;
        double scale = set.safety_factor * math.pow(err, -error_exponent);
        scale = std::fmin(std::fmax(scale, set.min_scale), set.max_scale);

        if (err <= 1.0) {
            ode.diff(t_new, y_new, dydt);
            fevals += 1;

            // stiffness detection, ordinary.rs:165-194
            if (steps % 100 == 0) {
                double stdnum = diff_norm_squared(yseg, k[S - 1]);
                double stden = diff_norm_squared(dydt, ysti);
                if (stden > 0.0) {
                    double h_lamb = h * std::sqrt(stdnum / stden);
                    if (h_lamb > 6.1) {
                        non_stiffness_counter = 0;
                        stiffness_counter += 1;
                        if (stiffness_counter == 15) {
                            status = Status::Error;
                            o.status = DEGPU_ERR_STIFFNESS;
                            o.t = t;
                            o.y = y;
                            return false;
                        }
                    }
                } else {
                    non_stiffness_counter += 1;
                    if (non_stiffness_counter == 6) stiffness_counter = 0;
                }
            }

            // dense output preparation, ordinary.rs:196-235
            cont[0] = y;
            State ydiff = minus(y_new, y);
            cont[1] = ydiff;
            State bspl(n, 0.0);
            add_scaled(bspl, h, k[0]);
            add_scaled(bspl, -1.0, ydiff);
            cont[2] = bspl;
            State cont3 = ydiff;
            add_scaled(cont3, -h, dydt);
            add_scaled(cont3, -1.0, bspl);
            cont[3] = cont3;
            if (tab.has_bi) {
                if (I > S) {
                    k[S] = dydt;
                    for (int i = S + 1; i < I; ++i) {
                        State ys = y;
                        for (int j = 0; j < i; ++j) add_scaled(ys, tab.a[i][j] * h, k[j]);
                        ode.diff(t + tab.c[i] * h, ys, k[i]);
                        fevals += 1;
                    }
                }
                for (int i = 4; i < tab.order; ++i) {
                    fill(cont[i], 0.0);
                    for (int j = 0; j < I; ++j) add_scaled(cont[i], tab.bi[i][j], k[j]);
                    scale_by(cont[i], h);
                }
            }

            t_prev = t;
            y_prev = y;
            dydt_prev = k[0];
            h_prev = h;
            t = t_new;
            y = y_new;
            k[0] = dydt;
            if (status == Status::RejectedStep) {
                status = Status::Solving;
                scale = std::fmin(scale, 1.0);
            }
        } else {
            status = Status::RejectedStep;
        }

        h *= scale;
        h = constrain_step_size(h, set.h_min, set.h_max);
        return true;
    }

    // ordinary.rs:301-336
    State interpolate(double t_interp) override {
        double s = (t_interp - t_prev) / h_prev;
        double s1 = 1.0 - s;
        int ilast = (int)cont.size() - 1;
        State acc = cont[ilast];
        for (int i = ilast - 1; i >= 1; --i) {
            double factor;
            if (i >= 4) {
                bool odd = ((ilast - i) % 2) == 1;
                if (hairer_dense) odd = !odd;  // published form: c4 + s(c5 + s1(c6 + s c7))
                factor = odd ? s1 : s;
            } else {
                factor = (i % 2 == 1) ? s1 : s;
            }
            scale_by(acc, factor);
            add_scaled(acc, 1.0, cont[i]);
        }
        return plus_scaled(cont[0], s, acc);
    }

    void set_h(double hn) { h = hn; }
};

// Adaptive family (RKF45, Cash-Karp): src/methods/erk/adaptive/ordinary.rs.  FSAL is false for
// both (adaptive/mod.rs:43-58); no `bi`, so dense output is cubic Hermite.
struct AdaptiveRK : Interpolator {
    Tableau tab;
    Settings set;
    Math math;
    int64_t max_rejects = 100;  // src/methods/erk/mod.rs:140

    double h = 0.0, t = 0.0, h_prev = 0.0, t_prev = 0.0;
    State y, dydt, y_prev, dydt_prev;
    std::vector<State> k;
    int64_t stiffness_counter = 0, steps = 0;
    Status status = Status::Uninitialized;

    // adaptive/ordinary.rs:16-58
    bool init(const Ode& ode, double t0, double tf, const State& y0, int64_t& fevals, Outcome& o) {
        if (set.h0 == 0.0) {
            set.h0 = h_init(ode, t0, tf, y0, tab.order, set.rtol, set.atol, set.h_min, set.h_max, fevals, math);
            fevals += 2;  // ordinary.rs:28: counted again on top of the two inside compute
        }
        double h0v;
        if (!validate_step_size_parameters(set.h0, set.h_min, set.h_max, t0, tf, h0v, o)) return false;
        h = h0v;
        stiffness_counter = 0;
        t = t0;
        y = y0;
        size_t n = y0.size();
        dydt.assign(n, 0.0);
        y_prev = y0;
        dydt_prev.assign(n, 0.0);
        k.assign(tab.I, State(n, 0.0));
        ode.diff(t, y, dydt);
        fevals += 1;
        t_prev = t;
        y_prev = y;
        dydt_prev = dydt;
        status = Status::Initialized;
        return true;
    }

    // adaptive/ordinary.rs:63-212.  Returns false with `o` filled on an error.
    bool step(const Ode& ode, int64_t& fevals, Outcome& o) {
        if (std::fabs(h) < std::fabs(h_prev) * 1e-14) {
            status = Status::Error;
            o.status = DEGPU_ERR_STEP_SIZE;
            o.t = t;
            o.y = y;
            return false;
        }
        if (steps >= set.max_steps) {
            status = Status::Error;
            o.status = DEGPU_ERR_MAX_STEPS;
            o.t = t;
            o.y = y;
            return false;
        }
        steps += 1;
        k[0] = dydt;
        const int S = tab.S;
        for (int i = 1; i < S; ++i) {
            State ys = y;
            for (int j = 0; j < i; ++j) add_scaled(ys, tab.a[i][j] * h, k[j]);
            ode.diff(t + tab.c[i] * h, ys, k[i]);
        }
        fevals += S - 1;
        State y_high = y;
        for (int i = 0; i < S; ++i) add_scaled(y_high, tab.b[i] * h, k[i]);
        State y_low = y;
        for (int i = 0; i < S; ++i) add_scaled(y_low, tab.bh[i] * h, k[i]);
        State err = minus(y_high, y_low);
        // error_norm_inf, traits.rs:413-433 (f64::max keeps the non-NaN operand)
        double err_norm = 0.0;
        for (size_t i = 0; i < y.size(); ++i) {
            double sk = set.atol[i] + set.rtol[i] * std::fmax(std::fabs(y[i]), std::fabs(y_high[i]));
            err_norm = std::fmax(err_norm, std::fabs(err[i] / sk));
        }
        double error_exponent = 1.0 / (double)tab.order;
        double scale = set.safety_factor * math.pow(err_norm, -error_exponent);
        scale = std::fmin(std::fmax(scale, set.min_scale), set.max_scale);
        if (err_norm <= 1.0) {
            t_prev = t;
            y_prev = y;
            dydt_prev = k[0];
            h_prev = h;
            if (status == Status::RejectedStep) {
                stiffness_counter = 0;
                status = Status::Solving;
                scale = std::fmin(scale, 1.0);
            }
            if (tab.has_bi) {  // ordinary.rs:146-163: the dense-output stages, from the step's start
                for (int i = 0; i < tab.I - S; ++i) {
                    State ys = y;
                    for (int j = 0; j < S + i; ++j) add_scaled(ys, tab.a[S + i][j] * h, k[j]);
                    ode.diff(t + tab.c[S + i] * h, ys, k[S + i]);
                }
                fevals += tab.I - S;
            }
            t += h;
            y = y_high;
            if (tab.fsal) {  // ordinary.rs:171-180
                dydt = k[S - 1];
            } else {
                ode.diff(t, y, dydt);
                fevals += 1;
            }
        } else {
            status = Status::RejectedStep;
            stiffness_counter += 1;
            if (stiffness_counter >= max_rejects) {
                status = Status::Error;
                o.status = DEGPU_ERR_STIFFNESS;
                o.t = t;
                o.y = y;
                return false;
            }
        }
        h *= scale;
        h = constrain_step_size(h, set.h_min, set.h_max);
        return true;
    }

    // adaptive/ordinary.rs:236-290: with `bi`, Horner in s per stage and y_prev + sum (cont_i
    // h_prev) k_i; without, cubic Hermite (src/interpolate.rs:40-60)
    State interpolate(double t_interp) override {
        if (tab.has_bi) {
            const double s = (t_interp - t_prev) / h_prev;
            State out = y_prev;
            for (int i = 0; i < tab.I; ++i) {
                double ci = tab.bi[i][tab.order - 1];
                for (int j = tab.order - 2; j >= 0; --j) ci = ci * s + tab.bi[i][j];
                ci *= s;
                add_scaled(out, ci * h_prev, k[i]);
            }
            return out;
        }
        double t0 = t_prev, t1 = t;
        double hh = t1 - t0;
        double s = (t_interp - t0) / hh;
        double s2 = s * s;
        double s3 = s2 * s;
        double h00 = 2.0 * s3 - 3.0 * s2 + 1.0;
        double h10 = s3 - 2.0 * s2 + s;
        double h01 = -2.0 * s3 + 3.0 * s2;
        double h11 = s3 - s2;
        State out(y.size(), 0.0);
        add_scaled(out, h00, y_prev);
        add_scaled(out, h10 * hh, dydt_prev);
        add_scaled(out, h01, y);
        add_scaled(out, h11 * hh, dydt);
        return out;
    }

    void set_h(double hn) { h = hn; }
};

// Fixed family (RK4): src/methods/erk/fixed/ordinary.rs.
struct FixedRK : Interpolator {
    Tableau tab;
    Settings set;
    bool fsal = false;  // rk4 constructor passes false (fixed/mod.rs:69-75)

    double h = 0.0, t = 0.0, h_prev = 0.0, t_prev = 0.0;
    State y, dydt, y_prev, dydt_prev;
    std::vector<State> k;
    int64_t steps = 0;
    Status status = Status::Uninitialized;

    bool init(const Ode& ode, double t0, double tf, const State& y0, int64_t& fevals, Outcome& o) {
        if (set.h0 == 0.0) {
            double duration = std::fabs(tf - t0);
            set.h0 = duration / 100.0;
        }
        double h0v;
        if (!validate_step_size_parameters(set.h0, set.h_min, set.h_max, t0, tf, h0v, o)) return false;
        h = h0v;
        t = t0;
        y = y0;
        size_t n = y0.size();
        dydt.assign(n, 0.0);
        y_prev = y0;
        dydt_prev.assign(n, 0.0);
        k.assign(tab.I, State(n, 0.0));
        ode.diff(t, y, dydt);
        fevals += 1;
        t_prev = t;
        y_prev = y;
        dydt_prev = dydt;
        status = Status::Initialized;
        return true;
    }

    bool step(const Ode& ode, int64_t& fevals, Outcome& o) {
        if (steps >= set.max_steps) {
            status = Status::Error;
            o.status = DEGPU_ERR_MAX_STEPS;
            o.t = t;
            o.y = y;
            return false;
        }
        steps += 1;
        k[0] = dydt;
        const int S = tab.S;
        for (int i = 1; i < S; ++i) {
            State ys = y;
            for (int j = 0; j < i; ++j) add_scaled(ys, tab.a[i][j] * h, k[j]);
            ode.diff(t + tab.c[i] * h, ys, k[i]);
        }
        fevals += S - 1;
        t_prev = t;
        y_prev = y;
        dydt_prev = k[0];
        h_prev = h;
        State y_next = y;
        for (int i = 0; i < S; ++i) add_scaled(y_next, tab.b[i] * h, k[i]);
        t += h;
        y = y_next;
        if (fsal) {
            dydt = k[S - 1];
        } else {
            ode.diff(t, y, dydt);
            fevals += 1;
        }
        status = Status::Solving;
        return true;
    }

    // fixed/ordinary.rs:169-221 without `bi` -> cubic Hermite (src/interpolate.rs:40-60)
    State interpolate(double t_interp) override {
        double t0 = t_prev, t1 = t;
        double hh = t1 - t0;
        double s = (t_interp - t0) / hh;
        double s2 = s * s;
        double s3 = s2 * s;
        double h00 = 2.0 * s3 - 3.0 * s2 + 1.0;
        double h10 = s3 - 2.0 * s2 + s;
        double h01 = -2.0 * s3 + 3.0 * s2;
        double h11 = s3 - s2;
        // linear_combination: zeros, then add_scaled term by term (traits.rs:357-375)
        State out(y.size(), 0.0);
        add_scaled(out, h00, y_prev);
        add_scaled(out, h10 * hh, dydt_prev);
        add_scaled(out, h01, y);
        add_scaled(out, h11 * hh, dydt);
        return out;
    }

    void set_h(double hn) { h = hn; }
};

// ---------------------------------------------------------------------------------------------
// Driver: solve_ode, src/ode/solve_ivp.rs:116-277, with DefaultSolout (final state kept) or
// TEvalSolout.
// ---------------------------------------------------------------------------------------------
struct Result {
    Outcome outcome;
    double t_final = 0.0;
    State y_final;
    int64_t accepted = 0, rejected = 0, fevals = 0;
    std::vector<State> dense;  // per requested point (caller order); NaN if never reached
};

template <class Solver>
Result solve_ode(Solver& solver, const Ode& ode, double t0, double tf, const State& y0,
                 const std::vector<double>* t_eval, CrossingSolout* cross = nullptr, EventSolout* event = nullptr) {
    Result r;
    double integration_direction;
    {
        double sg = rust_signum(tf - t0);
        if (sg == 1.0)
            integration_direction = 1.0;
        else if (sg == -1.0)
            integration_direction = -1.0;
        else {
            r.outcome.status = DEGPU_ERR_BAD_INPUT;
            r.outcome.msg = "Final time tf must be different from initial time t0.";
            r.t_final = t0;
            r.y_final = y0;
            return r;
        }
    }
    if (t_eval) r.dense.assign(t_eval->size(), State(y0.size(), std::numeric_limits<double>::quiet_NaN()));
    if (!solver.init(ode, t0, tf, y0, r.fevals, r.outcome)) {
        r.t_final = t0;
        r.y_final = y0;
        return r;
    }
    TEvalSolout* te = nullptr;
    TEvalSolout te_obj(t_eval ? *t_eval : std::vector<double>{}, t0, tf, &r.dense);
    if (t_eval) te = &te_obj;
    // EventWrappedSolout's base: TEvalSolout, or DefaultSolout (every step's end is pushed)
    PushLog log;
    te_obj.log = &log;
    if (event) {
        event->log = &log;
        event->integration_direction = integration_direction;
    }
    if (te) te->solout(solver.t, solver.t_prev, solver.y, solver);
    if (!te) log.push(solver.t);
    if (cross) cross->solout(solver.t, solver.t_prev, solver.y, solver);
    if (event) event->solout(solver.t, solver.t_prev, solver.y, solver);  // records g(t0, y0) only
    solver.status = Status::Solving;

    const double eps10 = std::numeric_limits<double>::epsilon() * 10.0;
    for (;;) {
        if ((solver.t + solver.h - tf) * integration_direction > 0.0) {
            double h_new = tf - solver.t;
            if (std::fabs(h_new) < eps10) {
                solver.status = Status::Complete;
                break;
            }
            solver.set_h(h_new);
        }
        if (!solver.step(ode, r.fevals, r.outcome)) {
            r.t_final = r.outcome.t;
            r.y_final = r.outcome.y;
            return r;
        }
        if (solver.status == Status::RejectedStep) {
            r.rejected += 1;
            continue;
        }
        r.accepted += 1;
        if (te) te->solout(solver.t, solver.t_prev, solver.y, solver);
        if (!te) log.push(solver.t);
        if (cross) cross->solout(solver.t, solver.t_prev, solver.y, solver);
        if (event && event->solout(solver.t, solver.t_prev, solver.y, solver)) {
            // ControlFlag::Terminate (solve_ivp.rs:254-259)
            r.outcome.status = DEGPU_INTERRUPTED;
            r.t_final = solver.t;
            r.y_final = solver.y;
            return r;
        }
        if (std::fabs(tf - solver.t) <= eps10) break;
    }
    r.outcome.status = DEGPU_COMPLETE;
    r.t_final = solver.t;
    r.y_final = solver.y;
    return r;
}

// One IVP solve with one of the three methods.
inline Result solve_one(int method, const Ode& ode, double t0, double tf, const State& y0, const Settings& set,
                        const Math& math, const std::vector<double>* t_eval, bool hairer_dense = false,
                        CrossingSolout* cross = nullptr, EventSolout* event = nullptr) {
    if (method == DEGPU_RK4) {
        FixedRK s;
        s.tab = tableau_rk4();
        s.set = set;
        return solve_ode(s, ode, t0, tf, y0, t_eval, cross, event);
    }
    if (method >= DEGPU_RKF45) {
        AdaptiveRK s;
        s.tab = tableau_for_method(method);
        s.set = set;
        s.math = math;
        return solve_ode(s, ode, t0, tf, y0, t_eval, cross, event);
    }
    DormandPrince s;
    s.tab = method == DEGPU_DOP853 ? tableau_dop853() : tableau_dopri5();
    s.set = set;
    s.math = math;
    s.hairer_dense = hairer_dense;
    return solve_ode(s, ode, t0, tf, y0, t_eval, cross, event);
}

}  // namespace oracle
