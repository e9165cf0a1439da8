// tableaus.h -- method coefficients (host + device constexpr).
//
// Every table is restated from the method's published source and is checked
// by the order-condition tests (rooted-tree elementary weights) in
// tests/test_tableaus.py, which parses this file.  Entries are written one
// per line as `constexpr double NAME = value;` so that they can be parsed.
//
//  * Tsit5: Ch. Tsitouras, "Runge-Kutta pairs of order 5(4) satisfying only
//    the first column simplifying assumption", Comput. Math. Appl. 62 (2011)
//    770-775: tableau, embedded weights (as btilde = b - bhat) and the
//    4th-order continuous extension b_i(theta).
//  * Vern7: J.H. Verner, "Numerically optimal Runge-Kutta pairs with
//    interpolants", Numer. Algorithms 53 (2010) 383-396, "most efficient"
//    7(6) pair.  Its dense output is 7th order: a 5th-order continuous
//    extension over the 10 stages plus f(t+h, y1), bootstrapped to order 7 by
//    seven lazy stages on steps that save (Enright, Jackson, Norsett and
//    Thomsen, ACM TOMS 12 (1986); derived by derive_dense_output.py beside
//    this file).  Verner's own lazy interpolant (six extra stages) is not
//    restated: its coefficients are not in a source this build can cite.
//  * Rosenbrock23: L.F. Shampine, M.W. Reichelt, "The MATLAB ODE suite",
//    SIAM J. Sci. Comput. 18 (1997) 1-22, the ode23s W-method and its
//    continuous extension.
//  * Rodas5: G. Di Marzo, RODAS5(4) (1993), in the transformed form of
//    E. Hairer, G. Wanner, Solving ODEs II, Sec. IV.7 (7.4'):
//       (I/(h*gamma) - J) u_i = f(y0 + sum_j a_ij u_j) + sum_j (C_ij/h) u_j,
//       y1 = y0 + sum_j m_j u_j,
//    stiffly accurate (m = row 8 of a, plus u_8; the error estimate is u_8).
//  * Rodas5P: G. Steinebach, "Construction of Rosenbrock-Wanner method
//    Rodas5P and numerical benchmarks within the Julia Differential
//    Equations package", BIT 63 (2023), same transformed form.
//  * Rodas dense output: this library's own 4th-order continuous extension
//       y(theta) = (1-theta) y0 + theta y1
//                  + theta (1-theta) (K2 + theta K3 + theta^2 K4),
//       K_q = sum_{j<=7} Hq_j u_j,
//    whose H2/H3/H4 satisfy the continuous order conditions up to order 4
//    and give R_theta(inf) = (1-theta)^4 on y' = lambda y (derived by
//    derive_dense_output.py).
#pragma once

namespace gbde {
namespace tab {

// ---------------------------------------------------------------- Tsit5
namespace tsit5 {
constexpr double c2 = 0.161;
constexpr double c3 = 0.327;
constexpr double c4 = 0.9;
constexpr double c5 = 0.9800255409045097;
constexpr double a21 = 0.161;
constexpr double a31 = -0.008480655492356989;
constexpr double a32 = 0.335480655492357;
constexpr double a41 = 2.897153057105493;
constexpr double a42 = -6.359448489975075;
constexpr double a43 = 4.3622954328695815;
constexpr double a51 = 5.325864828439257;
constexpr double a52 = -11.748883564062828;
constexpr double a53 = 7.4955393428898365;
constexpr double a54 = -0.09249506636175525;
constexpr double a61 = 5.86145544294642;
constexpr double a62 = -12.92096931784711;
constexpr double a63 = 8.159367898576159;
constexpr double a64 = -0.071584973281401;
constexpr double a65 = -0.028269050394068383;
constexpr double a71 = 0.09646076681806523;
constexpr double a72 = 0.01;
constexpr double a73 = 0.4798896504144996;
constexpr double a74 = 1.379008574103742;
constexpr double a75 = -3.290069515436081;
constexpr double a76 = 2.324710524099774;
// btilde = b - bhat (b = row 7 of a: first-same-as-last)
constexpr double bt1 = -0.00178001105222577714;
constexpr double bt2 = -0.0008164344596567469;
constexpr double bt3 = 0.007880878010261995;
constexpr double bt4 = -0.1447110071732629;
constexpr double bt5 = 0.5823571654525552;
constexpr double bt6 = -0.45808210592918697;
constexpr double bt7 = 0.015151515151515152;
// continuous extension, factored as in the paper
constexpr double r11 = -1.0530884977290216;
constexpr double r12 = 1.3299890189751412;
constexpr double r13 = 1.4364028541716351;
constexpr double r14 = 0.7139816917074209;
constexpr double r21 = 0.1017;
constexpr double r22 = 2.1966568338249754;
constexpr double r23 = 1.2949852507374631;
constexpr double r31 = 2.490627285651252793;
constexpr double r32 = 2.38535645472061657;
constexpr double r33 = 1.57803468208092486;
constexpr double r41 = -16.54810288924490272;
constexpr double r42 = 1.21712927295533244;
constexpr double r43 = 0.61620406037800089;
constexpr double r51 = 47.37952196281928122;
constexpr double r52 = 1.203071208372362603;
constexpr double r53 = 0.658047292653547382;
constexpr double r61 = -34.87065786149660974;
constexpr double r62 = 1.2;
constexpr double r63 = 0.666666666666666667;
constexpr double r71 = 2.5;
constexpr double r72 = 1.0;
constexpr double r73 = 0.6;
}  // namespace tsit5

// ---------------------------------------------------------------- Vern7
namespace vern7 {
constexpr double c2 = 0.005;
constexpr double c3 = 0.10888888888888888;
constexpr double c4 = 0.16333333333333333;
constexpr double c5 = 0.4555;
constexpr double c6 = 0.6095094489978381;
constexpr double c7 = 0.884;
constexpr double c8 = 0.925;
constexpr double a21 = 0.005;
constexpr double a31 = -1.07679012345679;
constexpr double a32 = 1.185679012345679;
constexpr double a41 = 0.04083333333333333;
constexpr double a43 = 0.1225;
constexpr double a51 = 0.6389139236255726;
constexpr double a53 = -2.455672638223657;
constexpr double a54 = 2.272258714598084;
constexpr double a61 = -2.6615773750187572;
constexpr double a63 = 10.804513886456137;
constexpr double a64 = -8.3539146573962;
constexpr double a65 = 0.820487594956657;
constexpr double a71 = 6.067741434696772;
constexpr double a73 = -24.711273635911088;
constexpr double a74 = 20.427517930788895;
constexpr double a75 = -1.9061579788166472;
constexpr double a76 = 1.006172249242068;
constexpr double a81 = 12.054670076253203;
constexpr double a83 = -49.75478495046899;
constexpr double a84 = 41.142888638604674;
constexpr double a85 = -4.461760149974004;
constexpr double a86 = 2.042334822239175;
constexpr double a87 = -0.09834843665406107;
constexpr double a91 = 10.138146522881808;
constexpr double a93 = -42.6411360317175;
constexpr double a94 = 35.76384003992257;
constexpr double a95 = -4.3480228403929075;
constexpr double a96 = 2.0098622683770357;
constexpr double a97 = 0.3487490460338272;
constexpr double a98 = -0.27143900510483127;
constexpr double a101 = -45.030072034298676;
constexpr double a103 = 187.3272437654589;
constexpr double a104 = -154.02882369350186;
constexpr double a105 = 18.56465306347536;
constexpr double a106 = -7.141809679295079;
constexpr double a107 = 1.3088085781613787;
constexpr double b1 = 0.04715561848627222;
constexpr double b4 = 0.25750564298434153;
constexpr double b5 = 0.2621665397741262;
constexpr double b6 = 0.15216092656738558;
constexpr double b7 = 0.4939969170032485;
constexpr double b8 = -0.29430311714032503;
constexpr double b9 = 0.08131747232495111;
constexpr double bh1 = 0.044608606606341174;
constexpr double bh4 = 0.26716403785713727;
constexpr double bh5 = 0.22010183001772932;
constexpr double bh6 = 0.2188431703143157;
constexpr double bh7 = 0.22898717054112028;
constexpr double bh10 = 0.02029518466335628;
}  // namespace vern7

// --------------------------------------------------------- Rosenbrock23
namespace ros23 {
// d = 1/(2 + sqrt(2)), e32 = 6 + sqrt(2)
constexpr double d = 0.29289321881345247560;
constexpr double e32 = 7.41421356237309504880;
}  // namespace ros23

// --------------------------------------------------------------- Rodas5
namespace rodas5 {
constexpr double gamma = 0.19;
constexpr double a21 = 2.0;
constexpr double a31 = 3.040894194418781;
constexpr double a32 = 1.041747909077569;
constexpr double a41 = 2.576417536461461;
constexpr double a42 = 1.622083060776640;
constexpr double a43 = -0.9089668560264532;
constexpr double a51 = 2.760842080225597;
constexpr double a52 = 1.446624659844071;
constexpr double a53 = -0.3036980084553738;
constexpr double a54 = 0.2877498600325443;
constexpr double a61 = -14.09640773051259;
constexpr double a62 = 6.925207756232704;
constexpr double a63 = -41.47510893210728;
constexpr double a64 = 2.343771018586405;
constexpr double a65 = 24.13215229196062;
constexpr double C21 = -10.31323885133993;
constexpr double C31 = -21.04823117650003;
constexpr double C32 = -7.234992135176716;
constexpr double C41 = 32.22751541853323;
constexpr double C42 = -4.943732386540191;
constexpr double C43 = 19.44922031041879;
constexpr double C51 = -20.69865579590063;
constexpr double C52 = -8.816374604402768;
constexpr double C53 = 1.260436877740897;
constexpr double C54 = -0.7495647613787146;
constexpr double C61 = -46.22004352711257;
constexpr double C62 = -17.49534862857472;
constexpr double C63 = -289.6389582892057;
constexpr double C64 = 93.60855400400906;
constexpr double C65 = 318.3822534212147;
constexpr double C71 = 34.20013733472935;
constexpr double C72 = -14.15535402717690;
constexpr double C73 = 57.82335640988400;
constexpr double C74 = 25.83362985412365;
constexpr double C75 = 1.408950972071624;
constexpr double C76 = -6.551835421242162;
constexpr double C81 = 42.57076742291101;
constexpr double C82 = -13.80770672017997;
constexpr double C83 = 93.98938432427124;
constexpr double C84 = 18.77919633714503;
constexpr double C85 = -31.58359187223370;
constexpr double C86 = -6.685968952921985;
constexpr double C87 = -5.810979938412932;
}  // namespace rodas5

// -------------------------------------------------------------- Rodas5P
namespace rodas5p {
constexpr double gamma = 0.21193756319429014;
constexpr double a21 = 3.0;
constexpr double a31 = 2.849394379747939;
constexpr double a32 = 0.45842242204463923;
constexpr double a41 = -6.954028509809101;
constexpr double a42 = 2.489845061869568;
constexpr double a43 = -10.358996098473584;
constexpr double a51 = 2.8029986275628964;
constexpr double a52 = 0.5072464736228206;
constexpr double a53 = -0.3988312541770524;
constexpr double a54 = -0.04721187230404641;
constexpr double a61 = -7.502846399306121;
constexpr double a62 = 2.561846144803919;
constexpr double a63 = -11.627539656261098;
constexpr double a64 = -0.18268767659942256;
constexpr double a65 = 0.030198172008377946;
constexpr double C21 = -14.155112264123755;
constexpr double C31 = -17.97296035885952;
constexpr double C32 = -2.859693295451294;
constexpr double C41 = 147.12150275711716;
constexpr double C42 = -1.41221402718213;
constexpr double C43 = 71.68940251302358;
constexpr double C51 = 165.43517024871676;
constexpr double C52 = -0.4592823456491126;
constexpr double C53 = 42.90938336958603;
constexpr double C54 = -5.961986721573306;
constexpr double C61 = 24.854864614690072;
constexpr double C62 = -3.0009227002832186;
constexpr double C63 = 47.4931110020768;
constexpr double C64 = 5.5814197821558125;
constexpr double C65 = -0.6610691825249471;
constexpr double C71 = 30.91273214028599;
constexpr double C72 = -3.1208243349937974;
constexpr double C73 = 77.79954646070892;
constexpr double C74 = 34.28646028294783;
constexpr double C75 = -19.097331116725623;
constexpr double C76 = -28.087943162872662;
constexpr double C81 = 37.80277123390563;
constexpr double C82 = -3.2571969029072276;
constexpr double C83 = 112.26918849496327;
constexpr double C84 = 66.9347231244047;
constexpr double C85 = -40.06618937091002;
constexpr double C86 = -54.66780262877968;
constexpr double C87 = -9.48861652309627;
}  // namespace rodas5p

// ---------------------------------------------------------------- SRIW1
// A. Roessler, SIAM J. Numer. Anal. 48 (2010) 922-952: 4-stage SRI, strong
// order 1.5 for diagonal noise (entries not listed are zero).
namespace sriw1 {
constexpr double A0_21 = 0.75;
constexpr double B0_21 = 1.5;
constexpr double A1_21 = 0.25;
constexpr double A1_31 = 1.0;
constexpr double A1_43 = 0.25;
constexpr double B1_21 = 0.5;
constexpr double B1_31 = -1.0;
constexpr double B1_41 = -5.0;
constexpr double B1_42 = 3.0;
constexpr double B1_43 = 0.5;
constexpr double al1 = 0.3333333333333333;
constexpr double al2 = 0.6666666666666666;
constexpr double b1_1 = -1.0;
constexpr double b1_2 = 1.3333333333333333;
constexpr double b1_3 = 0.6666666666666666;
constexpr double b1_4 = 0.0;
constexpr double b2_1 = -1.0;
constexpr double b2_2 = 1.3333333333333333;
constexpr double b2_3 = -0.3333333333333333;
constexpr double b2_4 = 0.0;
constexpr double b3_1 = 2.0;
constexpr double b3_2 = -1.3333333333333333;
constexpr double b3_3 = -0.6666666666666666;
constexpr double b3_4 = 0.0;
constexpr double b4_1 = -2.0;
constexpr double b4_2 = 1.6666666666666667;
constexpr double b4_3 = -0.6666666666666666;
constexpr double b4_4 = 1.0;
}  // namespace sriw1

// ---------------------------------------------------------------- SOSRI
// C. Rackauckas, Q. Nie, "Stability-optimized high order methods and
// stiffness detection for pathwise stiff stochastic differential equations",
// arXiv:1804.04344 (2018): the 4-stage SRI of strong order 1.5 for diagonal
// noise whose free coefficients were chosen to enlarge the stability region
// (SOSRI).  Same stage structure as SRIW1 (Roessler's SRI):
//   H0_i = X + sum_j A0_ij f(H0_j) h + sum_j B0_ij g(H1_j) I10/h
//   H1_i = X + sum_j A1_ij f(H0_j) h + sum_j B1_ij g(H1_j) sqrt(h)
// with every strictly lower entry in use.  The values are the published ones;
// they satisfy the strong-order-1.5 conditions to ~1e-16 except
// al . B0 e = 1 and al . (B0 e)^2 = 3/2, which they meet to ~7e-11.
namespace sosri {
constexpr double A0_21 = -0.04199224421316468;
constexpr double A0_31 = 2.842612915017106;
constexpr double A0_32 = -2.0527723684000727;
constexpr double A0_41 = 4.338237071435815;
constexpr double A0_42 = -2.8895936137439793;
constexpr double A0_43 = 2.3017575594644466;
constexpr double A1_21 = 0.26204282091330466;
constexpr double A1_31 = 0.20903646383505375;
constexpr double A1_32 = -0.1502377115150361;
constexpr double A1_41 = 0.05836595312746999;
constexpr double A1_42 = 0.6149440396332373;
constexpr double A1_43 = 0.08535117634046772;
constexpr double B0_21 = -0.21641093549612528;
constexpr double B0_31 = 1.5336352863679572;
constexpr double B0_32 = 0.26066223492647056;
constexpr double B0_41 = -1.0536037558179159;
constexpr double B0_42 = 1.7015284721089472;
constexpr double B0_43 = -0.20725685514492662;
constexpr double B1_21 = -0.5119011827621657;
constexpr double B1_31 = 2.67767339866713;
constexpr double B1_32 = -4.9395031322250995;
constexpr double B1_41 = 0.15580956238299215;
constexpr double B1_42 = 3.2361551006624674;
constexpr double B1_43 = -1.4223118283355949;
constexpr double al1 = 1.140099274172029;
constexpr double al2 = -0.6401334255743456;
constexpr double al3 = 0.4736296532772559;
constexpr double al4 = 0.026404498125060714;
constexpr double b1_1 = -1.8453464565104432;
constexpr double b1_2 = 2.688764531100726;
constexpr double b1_3 = -0.2523866501071323;
constexpr double b1_4 = 0.40896857551684956;
constexpr double b2_1 = 0.4969658141589478;
constexpr double b2_2 = -0.5771202869753592;
constexpr double b2_3 = -0.12919702470322217;
constexpr double b2_4 = 0.2093514975196336;
constexpr double b3_1 = 2.8453464565104425;
constexpr double b3_2 = -2.688764531100725;
constexpr double b3_3 = 0.2523866501071322;
constexpr double b3_4 = -0.40896857551684945;
constexpr double b4_1 = 0.11522663875443433;
constexpr double b4_2 = -0.57877086147738;
constexpr double b4_3 = 0.2857851028163886;
constexpr double b4_4 = 0.17775911990655704;
}  // namespace sosri

// Both SRI tables as full 4 x 4 arrays (entries not listed are zero), for the
// stage loops of the kernels and of the oracle; b[q] holds beta^(q+1).
#define GBDE_SRI_ARRAYS(NS, A0_3, A0_4, A1_3, A1_4, B0_3, B0_4, B1_3, B1_4, AL)               \
  static constexpr double A0[4][4] = {{0, 0, 0, 0}, {NS::A0_21, 0, 0, 0}, A0_3, A0_4};        \
  static constexpr double B0[4][4] = {{0, 0, 0, 0}, {NS::B0_21, 0, 0, 0}, B0_3, B0_4};        \
  static constexpr double A1[4][4] = {{0, 0, 0, 0}, {NS::A1_21, 0, 0, 0}, A1_3, A1_4};        \
  static constexpr double B1[4][4] = {{0, 0, 0, 0}, {NS::B1_21, 0, 0, 0}, B1_3, B1_4};        \
  static constexpr double al[4] = AL;                                                       \
  static constexpr double b[4][4] = {{NS::b1_1, NS::b1_2, NS::b1_3, NS::b1_4},               \
                                     {NS::b2_1, NS::b2_2, NS::b2_3, NS::b2_4},               \
                                     {NS::b3_1, NS::b3_2, NS::b3_3, NS::b3_4},               \
                                     {NS::b4_1, NS::b4_2, NS::b4_3, NS::b4_4}};
#define GBDE_ROW(...) {__VA_ARGS__}
struct SosriTab {
  GBDE_SRI_ARRAYS(sosri, GBDE_ROW(sosri::A0_31, sosri::A0_32, 0, 0),
                  GBDE_ROW(sosri::A0_41, sosri::A0_42, sosri::A0_43, 0),
                  GBDE_ROW(sosri::A1_31, sosri::A1_32, 0, 0),
                  GBDE_ROW(sosri::A1_41, sosri::A1_42, sosri::A1_43, 0),
                  GBDE_ROW(sosri::B0_31, sosri::B0_32, 0, 0),
                  GBDE_ROW(sosri::B0_41, sosri::B0_42, sosri::B0_43, 0),
                  GBDE_ROW(sosri::B1_31, sosri::B1_32, 0, 0),
                  GBDE_ROW(sosri::B1_41, sosri::B1_42, sosri::B1_43, 0),
                  GBDE_ROW(sosri::al1, sosri::al2, sosri::al3, sosri::al4))
};
struct Sriw1Tab {
  GBDE_SRI_ARRAYS(sriw1, GBDE_ROW(0, 0, 0, 0), GBDE_ROW(0, 0, 0, 0),
                  GBDE_ROW(sriw1::A1_31, 0, 0, 0), GBDE_ROW(0, 0, sriw1::A1_43, 0),
                  GBDE_ROW(0, 0, 0, 0), GBDE_ROW(0, 0, 0, 0),
                  GBDE_ROW(sriw1::B1_31, 0, 0, 0),
                  GBDE_ROW(sriw1::B1_41, sriw1::B1_42, sriw1::B1_43, 0),
                  GBDE_ROW(sriw1::al1, sriw1::al2, 0, 0))
};
#undef GBDE_ROW
#undef GBDE_SRI_ARRAYS

}  // namespace tab
}  // namespace gbde

// Generated dense-output coefficients (Vern7 5th-order extension, Rodas
// 4th-order extension).
#include "dense_coeffs.h"
