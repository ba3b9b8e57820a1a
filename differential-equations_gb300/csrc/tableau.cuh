// tableau.cuh — Butcher tableaus of the methods, as compile-time constants.
//
// Values are the crate's (src/tableau/runge_kutta.rs:39-70 and :335-480,
// src/tableau/dorman_prince.rs:37-118 and :155-381, src/tableau/verner.rs); every coefficient is a binary64 constant evaluated exactly as the crate's
// `T::from_f64(x)` of the same literal or quotient.  Being constexpr, each coefficient is an
// immediate operand after unrolling, and terms whose coefficient is zero are removed at compile
// time (`if constexpr`).  Removing a term `acc + 0*k` leaves every finite result unchanged bit for
// bit: the accumulations start from +0 or from a state value and the only possible difference is
// the sign of an exact zero, which no right-hand side here can turn into a different non-zero value.
#pragma once

#include "../../include/degpu.h"

namespace degpu {

struct TabRK4 {
    static constexpr int S = 4, I = 4, ORDER = 4, METHOD = DEGPU_RK4;
    static constexpr bool ADAPTIVE = false, DP = false, HAS_BH = false, FSAL = false, HAS_BI = false;
    static constexpr double C[4] = {0.0, 0.5, 0.5, 1.0};
    static constexpr double A[4][4] = {{0, 0, 0, 0}, {0.5, 0, 0, 0}, {0, 0.5, 0, 0}, {0, 0, 1.0, 0}};
    static constexpr double B[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    static constexpr double BH[4] = {0, 0, 0, 0};
    static constexpr double ER[4] = {0, 0, 0, 0};
    static constexpr double BI[4][4] = {};
    __host__ __device__ static constexpr double c(int i) { return C[i]; }
    __host__ __device__ static constexpr double a(int i, int j) { return A[i][j]; }
    __host__ __device__ static constexpr double b(int i) { return B[i]; }
    __host__ __device__ static constexpr double bh(int i) { return BH[i]; }
    __host__ __device__ static constexpr double er(int i) { return ER[i]; }
    __host__ __device__ static constexpr double bi(int i, int j) { return BI[i][j]; }
};

struct TabDopri5 {
    static constexpr int S = 7, I = 7, ORDER = 5, METHOD = DEGPU_DOPRI5;
    // FSAL: the last row of A equals b and c = 1, so the last stage's state is y_new
    static constexpr bool ADAPTIVE = true, DP = true, HAS_BH = false, FSAL = true, HAS_BI = false;
    static constexpr double C[7] = {0.0, 0.2, 0.3, 0.8, 8.0 / 9.0, 1.0, 1.0};
    static constexpr double A[7][7] = {
        {0, 0, 0, 0, 0, 0, 0},
        {0.2, 0, 0, 0, 0, 0, 0},
        {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0, 0, 0},
        {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0, 0, 0},
        {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0, 0, 0},
        {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0, 0, 0},
        {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0, 0}};
    static constexpr double B[7] = {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0,
                                    11.0 / 84.0, 0.0};
    static constexpr double BH[7] = {0, 0, 0, 0, 0, 0, 0};
    static constexpr double ER[7] = {71.0 / 57600.0, 0.0, -71.0 / 16695.0, 71.0 / 1920.0, -17253.0 / 339200.0,
                                     22.0 / 525.0, -1.0 / 40.0};
    // The crate fills only row 0 of its 7x7 `bi` (dorman_prince.rs:95-101) while the step reads
    // row 4 (dormandprince/ordinary.rs:228-234): the fifth dense coefficient is identically zero.
    static constexpr double BI[7][7] = {};
    __host__ __device__ static constexpr double c(int i) { return C[i]; }
    __host__ __device__ static constexpr double a(int i, int j) { return A[i][j]; }
    __host__ __device__ static constexpr double b(int i) { return B[i]; }
    __host__ __device__ static constexpr double bh(int i) { return BH[i]; }
    __host__ __device__ static constexpr double er(int i) { return ER[i]; }
    __host__ __device__ static constexpr double bi(int i, int j) { return BI[i][j]; }
};

// The FSAL flag is a property of the coefficients: check it.
template <class Tab>
__host__ __device__ constexpr bool fsal_holds() {
    if (Tab::C[Tab::S - 1] != 1.0) return false;
    for (int j = 0; j < Tab::S; ++j)
        if (Tab::A[Tab::S - 1][j] != Tab::B[j]) return false;
    return true;
}
static_assert(fsal_holds<TabDopri5>(), "DOPRI5: last row of A must equal b with c = 1");

struct TabDop853 {
    static constexpr int S = 12, I = 16, ORDER = 8, METHOD = DEGPU_DOP853;
    static constexpr bool ADAPTIVE = true, DP = true, HAS_BH = true, FSAL = false, HAS_BI = false;
    static constexpr double C[16] = {0.0,
                                     5.260015195876773E-2,
                                     7.89002279381516E-2,
                                     1.183503419072274E-1,
                                     2.816496580927726E-1,
                                     3.333333333333333E-1,
                                     0.25,
                                     3.076923076923077E-1,
                                     6.512820512820513E-1,
                                     0.6,
                                     8.571428571428571E-1,
                                     1.0,
                                     0.0,
                                     0.1,
                                     0.2,
                                     7.777777777777778E-1};
    static constexpr double A[16][16] = {
        {},
        {5.260015195876773E-2},
        {1.97250569845379E-2, 5.91751709536137E-2},
        {2.958758547680685E-2, 0.0, 8.876275643042054E-2},
        {2.413651341592667E-1, 0.0, -8.845494793282861E-1, 9.24834003261792E-1},
        {3.7037037037037035E-2, 0.0, 0.0, 1.7082860872947386E-1, 1.2546768756682242E-1},
        {3.7109375E-2, 0.0, 0.0, 1.7025221101954405E-1, 6.021653898045596E-2, -1.7578125E-2},
        {3.709200011850479E-2, 0.0, 0.0, 1.7038392571223998E-1, 1.0726203044637328E-1, -1.5319437748624402E-2,
         8.273789163814023E-3},
        {6.241109587160757E-1, 0.0, 0.0, -3.3608926294469414, -8.68219346841726E-1, 2.759209969944671E1,
         2.0154067550477894E1, -4.348988418106996E1},
        {4.7766253643826434E-1, 0.0, 0.0, -2.4881146199716677, -5.90290826836843E-1, 2.1230051448181193E1,
         1.5279233632882423E1, -3.328821096898486E1, -2.0331201708508627E-2},
        {-9.371424300859873E-1, 0.0, 0.0, 5.186372428844064, 1.0914373489967295, -8.149787010746927,
         -1.852006565999696E1, 2.2739487099350505E1, 2.4936055526796523, -3.0467644718982196},
        {2.273310147516538, 0.0, 0.0, -1.053449546673725E1, -2.0008720582248625, -1.79589318631188E1,
         2.794888452941996E1, -2.8589982771350235, -8.87285693353063, 1.2360567175794303E1, 6.433927460157636E-1},
        {},
        {5.6167502283047954E-2, 0, 0, 0, 0, 0, 2.5350021021662483E-1, -2.462390374708025E-1, -1.2419142326381637E-1,
         1.5329179827876568E-1, 8.20105229563469E-3, 7.567897660545699E-3, -8.298E-3},
        {3.183464816350214E-2, 0, 0, 0, 0, 2.8300909672366776E-2, 5.3541988307438566E-2, -5.492374857139099E-2, 0,
         0, -1.0834732869724932E-4, 3.825710908356584E-4, -3.4046500868740456E-4, 1.413124436746325E-1},
        {-4.2889630158379194E-1, 0, 0, 0, 0, -4.697621415361164, 7.683421196062599, 4.06898981839711,
         3.567271874552811E-1, 0, 0, 0, -1.3990241651590145E-3, 2.9475147891527724, -9.15095847217987}};
    static constexpr double B[12] = {5.4293734116568765E-2, 0, 0, 0, 0, 4.450312892752409, 1.8915178993145003,
                                     -5.801203960010585, 3.111643669578199E-1, -1.521609496625161E-1,
                                     2.0136540080403034E-1, 4.471061572777259E-2};
    static constexpr double BH[12] = {2.440944881889764E-1, 0, 0, 0, 0, 0, 0, 0, 7.338466882816118E-1, 0, 0,
                                      2.2058823529411766E-2};
    static constexpr double ER[12] = {1.312004499419488E-2, 0, 0, 0, 0, -1.2251564463762044,
                                      -4.957589496572502E-1, 1.6643771824549864, -3.5032884874997366E-1,
                                      3.341791187130175E-1, 8.192320648511571E-2, -2.2355307863886294E-2};
    static constexpr double BI[16][16] = {
        {}, {}, {}, {},
        {-8.428938276109013, 0, 0, 0, 0, 5.667149535193777E-1, -3.0689499459498917, 2.38466765651207,
         2.117034582445028, -8.71391583777973E-1, 2.2404374302607883, 6.315787787694688E-1, -8.899033645133331E-2,
         1.8148505520854727E1, -9.194632392478356, -4.436036387594894},
        {1.0427508642579134E1, 0, 0, 0, 0, 2.4228349177525817E2, 1.6520045171727028E2, -3.745467547226902E2,
         -2.2113666853125306E1, 7.733432668472264, -3.0674084731089398E1, -9.332130526430229, 1.5697238121770845E1,
         -3.1139403219565178E1, -9.35292435884448, 3.581684148639408E1},
        {1.9985053242002433E1, 0, 0, 0, 0, -3.870373087493518E2, -1.8917813819516758E2, 5.278081592054236E2,
         -1.157390253995963E1, 6.8812326946963, -1.0006050966910838, 7.777137798053443E-1, -2.778205752353508,
         -6.019669523126412E1, 8.432040550667716E1, 1.199229113618279E1},
        {-2.569393346270375E1, 0, 0, 0, 0, -1.5418974869023643E2, -2.315293791760455E2, 3.576391179106141E2,
         9.340532418362432E1, -3.745832313645163E1, 1.040996495089623E2, 2.98402934266605E1, -4.353345659001114E1,
         9.632455395918828E1, -3.917726167561544E1, -1.4972683625798564E2},
        {}, {}, {}, {}, {}, {}, {}, {}};
    __host__ __device__ static constexpr double c(int i) { return C[i]; }
    __host__ __device__ static constexpr double a(int i, int j) { return A[i][j]; }
    __host__ __device__ static constexpr double b(int i) { return i < 12 ? B[i] : 0.0; }
    __host__ __device__ static constexpr double bh(int i) { return i < 12 ? BH[i] : 0.0; }
    __host__ __device__ static constexpr double er(int i) { return i < 12 ? ER[i] : 0.0; }
    __host__ __device__ static constexpr double bi(int i, int j) { return BI[i][j]; }
};

// Type selection (std::conditional without <type_traits>, which run-time compilation lacks).
template <bool B, class T, class F>
struct Select {
    using type = T;
};
template <class T, class F>
struct Select<false, T, F> {
    using type = F;
};

// Compile-time loop: f(std::integral_constant<int, k>) for k in [Begin, End).
template <int V>
struct IC {
    static constexpr int value = V;
    __host__ __device__ constexpr operator int() const { return V; }
};
template <int Begin, int End, class F>
__host__ __device__ __forceinline__ void static_for(F&& f) {
    if constexpr (Begin < End) {
        f(IC<Begin>{});
        static_for<Begin + 1, End>(f);
    }
}

// Embedded pairs of the crate's Adaptive ERK family (src/methods/erk/adaptive/mod.rs:43-58,
// ordinary.rs:63-212): y_high from b, y_low from BL (the crate's `bh`), an infinity norm of their
// difference, cubic Hermite dense output; order 5 in the controller for both.
struct TabRKF45 {  // src/tableau/runge_kutta.rs:335-406 (Fehlberg 1969)
    static constexpr int S = 6, I = 6, ORDER = 5, METHOD = DEGPU_RKF45;
    static constexpr bool ADAPTIVE = true, DP = false, HAS_BH = false, FSAL = false, HAS_BI = false;
    static constexpr double C[6] = {0.0, 1.0 / 4.0, 3.0 / 8.0, 12.0 / 13.0, 1.0, 1.0 / 2.0};
    static constexpr double A[6][6] = {{0, 0, 0, 0, 0, 0},
                                       {1.0 / 4.0, 0, 0, 0, 0, 0},
                                       {3.0 / 32.0, 9.0 / 32.0, 0, 0, 0, 0},
                                       {1932.0 / 2197.0, -7200.0 / 2197.0, 7296.0 / 2197.0, 0, 0, 0},
                                       {439.0 / 216.0, -8.0, 3680.0 / 513.0, -845.0 / 4104.0, 0, 0},
                                       {-8.0 / 27.0, 2.0, -3544.0 / 2565.0, 1859.0 / 4104.0, -11.0 / 40.0, 0}};
    static constexpr double B[6] = {16.0 / 135.0, 0.0, 6656.0 / 12825.0, 28561.0 / 56430.0, -9.0 / 50.0, 2.0 / 55.0};
    static constexpr double BL[6] = {25.0 / 216.0, 0.0, 1408.0 / 2565.0, 2197.0 / 4104.0, -1.0 / 5.0, 0.0};
    static constexpr double BH[6] = {0, 0, 0, 0, 0, 0};
    static constexpr double ER[6] = {0, 0, 0, 0, 0, 0};
    static constexpr double BI[6][6] = {};
    __host__ __device__ static constexpr double c(int i) { return C[i]; }
    __host__ __device__ static constexpr double a(int i, int j) { return A[i][j]; }
    __host__ __device__ static constexpr double b(int i) { return B[i]; }
    __host__ __device__ static constexpr double bl(int i) { return BL[i]; }
    __host__ __device__ static constexpr double bh(int i) { return BH[i]; }
    __host__ __device__ static constexpr double er(int i) { return ER[i]; }
    __host__ __device__ static constexpr double bi(int i, int j) { return BI[i][j]; }
};

struct TabCashKarp {  // src/tableau/runge_kutta.rs:420-480 (Cash and Karp 1990)
    static constexpr int S = 6, I = 6, ORDER = 5, METHOD = DEGPU_CASH_KARP;
    static constexpr bool ADAPTIVE = true, DP = false, HAS_BH = false, FSAL = false, HAS_BI = false;
    static constexpr double C[6] = {0.0, 1.0 / 5.0, 3.0 / 10.0, 3.0 / 5.0, 1.0, 7.0 / 8.0};
    static constexpr double A[6][6] = {
        {0, 0, 0, 0, 0, 0},
        {1.0 / 5.0, 0, 0, 0, 0, 0},
        {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0, 0},
        {3.0 / 10.0, -9.0 / 10.0, 6.0 / 5.0, 0, 0, 0},
        {-11.0 / 54.0, 5.0 / 2.0, -70.0 / 27.0, 35.0 / 27.0, 0, 0},
        {1631.0 / 55296.0, 175.0 / 512.0, 575.0 / 13824.0, 44275.0 / 110592.0, 253.0 / 4096.0, 0}};
    static constexpr double B[6] = {37.0 / 378.0, 0.0, 250.0 / 621.0, 125.0 / 594.0, 0.0, 512.0 / 1771.0};
    static constexpr double BL[6] = {2825.0 / 27648.0, 0.0, 18575.0 / 48384.0, 13525.0 / 55296.0, 277.0 / 14336.0,
                                     1.0 / 4.0};
    static constexpr double BH[6] = {0, 0, 0, 0, 0, 0};
    static constexpr double ER[6] = {0, 0, 0, 0, 0, 0};
    static constexpr double BI[6][6] = {};
    __host__ __device__ static constexpr double c(int i) { return C[i]; }
    __host__ __device__ static constexpr double a(int i, int j) { return A[i][j]; }
    __host__ __device__ static constexpr double b(int i) { return B[i]; }
    __host__ __device__ static constexpr double bl(int i) { return BL[i]; }
    __host__ __device__ static constexpr double bh(int i) { return BH[i]; }
    __host__ __device__ static constexpr double er(int i) { return ER[i]; }
    __host__ __device__ static constexpr double bi(int i, int j) { return BI[i][j]; }
};

// Verner's pairs of the crate's Adaptive family (src/tableau/verner.rs; constructors
// src/methods/erk/adaptive/mod.rs:59-122): the embedded pair of TabRKF45 with more stages, plus
// I - S dense-output stages evaluated on every accepted step and interpolation weights BI
// (adaptive/ordinary.rs:146-163, 251-275). The coefficient tables are generated from the crate's
// literals by gen_verner_tables.py.
namespace verner {
#include "verner_tables.inc"
}

template <class V, int M>
struct TabVerner {
    static constexpr int S = V::S, I = V::I, ORDER = V::ORDER, METHOD = M;
    static constexpr bool ADAPTIVE = true, DP = false, HAS_BH = false, FSAL = V::FSAL, HAS_BI = true;
    __host__ __device__ static constexpr double c(int i) { return V::C[i]; }
    __host__ __device__ static constexpr double a(int i, int j) { return V::A[i][j]; }
    __host__ __device__ static constexpr double b(int i) { return V::B[i]; }
    __host__ __device__ static constexpr double bl(int i) { return V::BH[i]; }
    __host__ __device__ static constexpr double bh(int i) { return 0.0; }
    __host__ __device__ static constexpr double er(int i) { return 0.0; }
    __host__ __device__ static constexpr double bi(int i, int j) { return V::BI[i][j]; }
};
using TabRKV655E = TabVerner<verner::rkv655e, DEGPU_RKV655E>;
using TabRKV656E = TabVerner<verner::rkv656e, DEGPU_RKV656E>;
using TabRKV766E = TabVerner<verner::rkv766e, DEGPU_RKV766E>;
using TabRKV767E = TabVerner<verner::rkv767e, DEGPU_RKV767E>;
using TabRKV877E = TabVerner<verner::rkv877e, DEGPU_RKV877E>;
using TabRKV878E = TabVerner<verner::rkv878e, DEGPU_RKV878E>;
using TabRKV988E = TabVerner<verner::rkv988e, DEGPU_RKV988E>;
using TabRKV989E = TabVerner<verner::rkv989e, DEGPU_RKV989E>;

}  // namespace degpu
