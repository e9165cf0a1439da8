// dense_coeffs.h -- GENERATED by derive_dense_output.py; do not edit.
#pragma once
namespace gbde {
namespace tab {
// Vern7 5th-order continuous extension: b_j(theta) = sum_k B_j_k theta^k,
// j = 1..10 the Vern7 stages, j = 11 the stage f(t+h, y1).
// max residual of the defining equations: 7.638e-14
namespace vern7d {
constexpr double B1_1 = 0.994446149414611;
constexpr double B1_2 = -4.958812965305387;
constexpr double B1_3 = 9.768339951719183;
constexpr double B1_4 = -8.40453712333771;
constexpr double B1_5 = 2.6477196059955572;
constexpr double B2_1 = 0.0;
constexpr double B2_2 = 0.0;
constexpr double B2_3 = 0.0;
constexpr double B2_4 = 0.0;
constexpr double B2_5 = 0.0;
constexpr double B3_1 = 0.0;
constexpr double B3_2 = 0.0;
constexpr double B3_3 = 0.0;
constexpr double B3_4 = 0.0;
constexpr double B3_5 = 0.0;
constexpr double B4_1 = 0.01679459293952862;
constexpr double B4_2 = 6.174538408281388;
constexpr double B4_3 = -17.10197143292259;
constexpr double B4_4 = 16.91467803895081;
constexpr double B4_5 = -5.746533964264811;
constexpr double B5_1 = -0.03991100150954518;
constexpr double B5_2 = -0.18419256214375304;
constexpr double B5_3 = 4.866149698899478;
constexpr double B5_4 = -7.8116529662944965;
constexpr double B5_5 = 3.431773370822425;
constexpr double B6_1 = 0.035497427879333084;
constexpr double B6_2 = -2.189070330278462;
constexpr double B6_3 = 7.979571935843278;
constexpr double B6_4 = -8.576156303385819;
constexpr double B6_5 = 2.902318196509069;
constexpr double B7_1 = 0.055631850833719104;
constexpr double B7_2 = 1.341707510781685;
constexpr double B7_3 = -6.519695285393735;
constexpr double B7_4 = 10.233724673373933;
constexpr double B7_5 = -4.617371832592358;
constexpr double B8_1 = -0.09441053405181421;
constexpr double B8_2 = 1.2299807377706762;
constexpr double B8_3 = -6.2529575925490875;
constexpr double B8_4 = 8.904410788994564;
constexpr double B8_5 = -4.0813265173046585;
constexpr double B9_1 = 0.04257815456015379;
constexpr double B9_2 = -0.030657935112560555;
constexpr double B9_3 = 0.13577533522053176;
constexpr double B9_4 = -0.2905413104599823;
constexpr double B9_5 = 0.22416322811680445;
constexpr double B10_1 = -0.010626640065008991;
constexpr double B10_2 = 0.6165071360051799;
constexpr double B10_3 = -2.8752126108066713;
constexpr double B10_4 = 4.030074202140125;
constexpr double B10_5 = -1.7607420872736324;
constexpr double B11_1 = -9.876544027065393e-13;
constexpr double B11_2 = -1.999999999998785;
constexpr double B11_3 = 9.999999999989614;
constexpr double B11_4 = -14.999999999981425;
constexpr double B11_5 = 6.999999999991588;
}  // namespace vern7d
// rodas5 4th-order continuous extension (transformed stages u_1..u_7), max residual 5.684e-14
namespace rodas5d {
constexpr double H2_1 = 46.33506133332498;
constexpr double H2_2 = -6.136914790750268;
constexpr double H2_3 = 108.4071261859024;
constexpr double H2_4 = -15.432459674308959;
constexpr double H2_5 = -79.50999799548705;
constexpr double H2_6 = -1.905016570565929;
constexpr double H2_7 = -2.7727981784326463;
constexpr double H3_1 = -39.141063581018344;
constexpr double H3_2 = -3.460898857776812;
constexpr double H3_3 = -157.10746284885568;
constexpr double H3_4 = 34.66137042566592;
constexpr double H3_5 = 146.53644774504696;
constexpr double H3_6 = 4.746961424329122;
constexpr double H3_7 = 8.033032645033895;
constexpr double H4_1 = 35.36683737690469;
constexpr double H4_2 = 3.300351318510028;
constexpr double H4_3 = 162.0764418691674;
constexpr double H4_4 = -9.977463628954938;
constexpr double H4_5 = -129.99923473376202;
constexpr double H4_6 = -8.753639789002799;
constexpr double H4_7 = -10.993114152190547;
}  // namespace rodas5d
// rodas5p 4th-order continuous extension (transformed stages u_1..u_7), max residual 7.105e-14
namespace rodas5pd {
constexpr double H2_1 = 18.16834780540308;
constexpr double H2_2 = -2.403976485650891;
constexpr double H2_3 = -28.490339497899754;
constexpr double H2_4 = -39.23532392483474;
constexpr double H2_5 = 24.203612973330184;
constexpr double H2_6 = 31.138884328778953;
constexpr double H2_7 = 5.813992390806126;
constexpr double H3_1 = 20.20463917943479;
constexpr double H3_2 = -1.565157467658963;
constexpr double H3_3 = 153.7304542929287;
constexpr double H3_4 = 118.22912892648053;
constexpr double H3_5 = -71.49081351328452;
constexpr double H3_6 = -100.21520495678132;
constexpr double H3_7 = -27.642530934778755;
constexpr double H4_1 = -15.086356891229629;
constexpr double H4_2 = 3.4125953268018083;
constexpr double H4_3 = -59.68473410629569;
constexpr double H4_4 = -45.47407592789013;
constexpr double H4_5 = 28.595178703252632;
constexpr double H4_6 = 42.46386356047385;
constexpr double H4_7 = 18.195502534434848;
}  // namespace rodas5pd
}  // namespace tab
}  // namespace gbde
