/* Runge-Kutta coefficient tables of SimpleDiffEq.jl, extracted verbatim.
 *
 * Generated by gen_tableaus.py from the reference's coefficient files; do
 * not edit by hand.  Each group is a namespace of constexpr doubles named
 * as in the reference, an enum of positions (<group>_<name>) and an
 * initializer list (GBTAB_<GROUP>_INIT) holding the values in that order,
 * so device code can place a group in __constant__ memory and index it
 * with compile-time positions.
 */
#pragma once

/* tsit5: src/tsit5/atsit5_cache.jl:1-105 (56 values) */
namespace gbtab { namespace tsit5 {
constexpr double c1 = 0.161;
constexpr double c2 = 0.327;
constexpr double c3 = 0.9;
constexpr double c4 = 0.9800255409045097;
constexpr double c5 = 1.0;
constexpr double c6 = 1.0;
constexpr double a21 = 0.161;
constexpr double a31 = -0.008480655492356989;
constexpr double a32 = 0.335480655492357;
constexpr double a41 = 2.8971530571054935;
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
constexpr double btilde1 = -0.001780011052225777;
constexpr double btilde2 = -0.0008164344596567469;
constexpr double btilde3 = 0.007880878010261995;
constexpr double btilde4 = -0.1447110071732629;
constexpr double btilde5 = 0.5823571654525552;
constexpr double btilde6 = -0.45808210592918697;
constexpr double btilde7 = 0.015151515151515152;
constexpr double r11 = 1.0;
constexpr double r12 = -2.763706197274826;
constexpr double r13 = 2.9132554618219126;
constexpr double r14 = -1.0530884977290216;
constexpr double r22 = 0.13169999999999998;
constexpr double r23 = -0.2234;
constexpr double r24 = 0.1017;
constexpr double r32 = 3.9302962368947516;
constexpr double r33 = -5.941033872131505;
constexpr double r34 = 2.490627285651253;
constexpr double r42 = -12.411077166933676;
constexpr double r43 = 30.33818863028232;
constexpr double r44 = -16.548102889244902;
constexpr double r52 = 37.50931341651104;
constexpr double r53 = -88.1789048947664;
constexpr double r54 = 47.37952196281928;
constexpr double r62 = -27.896526289197286;
constexpr double r63 = 65.09189467479366;
constexpr double r64 = -34.87065786149661;
constexpr double r72 = 1.5;
constexpr double r73 = -4.0;
constexpr double r74 = 2.5;
} }
enum gbtab_tsit5_pos {
  tsit5_c1 = 0,
  tsit5_c2 = 1,
  tsit5_c3 = 2,
  tsit5_c4 = 3,
  tsit5_c5 = 4,
  tsit5_c6 = 5,
  tsit5_a21 = 6,
  tsit5_a31 = 7,
  tsit5_a32 = 8,
  tsit5_a41 = 9,
  tsit5_a42 = 10,
  tsit5_a43 = 11,
  tsit5_a51 = 12,
  tsit5_a52 = 13,
  tsit5_a53 = 14,
  tsit5_a54 = 15,
  tsit5_a61 = 16,
  tsit5_a62 = 17,
  tsit5_a63 = 18,
  tsit5_a64 = 19,
  tsit5_a65 = 20,
  tsit5_a71 = 21,
  tsit5_a72 = 22,
  tsit5_a73 = 23,
  tsit5_a74 = 24,
  tsit5_a75 = 25,
  tsit5_a76 = 26,
  tsit5_btilde1 = 27,
  tsit5_btilde2 = 28,
  tsit5_btilde3 = 29,
  tsit5_btilde4 = 30,
  tsit5_btilde5 = 31,
  tsit5_btilde6 = 32,
  tsit5_btilde7 = 33,
  tsit5_r11 = 34,
  tsit5_r12 = 35,
  tsit5_r13 = 36,
  tsit5_r14 = 37,
  tsit5_r22 = 38,
  tsit5_r23 = 39,
  tsit5_r24 = 40,
  tsit5_r32 = 41,
  tsit5_r33 = 42,
  tsit5_r34 = 43,
  tsit5_r42 = 44,
  tsit5_r43 = 45,
  tsit5_r44 = 46,
  tsit5_r52 = 47,
  tsit5_r53 = 48,
  tsit5_r54 = 49,
  tsit5_r62 = 50,
  tsit5_r63 = 51,
  tsit5_r64 = 52,
  tsit5_r72 = 53,
  tsit5_r73 = 54,
  tsit5_r74 = 55,
  tsit5_COUNT = 56
};
#define GBTAB_TSIT5_INIT { \
  0.161, \
  0.327, \
  0.9, \
  0.9800255409045097, \
  1.0, \
  1.0, \
  0.161, \
  -0.008480655492356989, \
  0.335480655492357, \
  2.8971530571054935, \
  -6.359448489975075, \
  4.3622954328695815, \
  5.325864828439257, \
  -11.748883564062828, \
  7.4955393428898365, \
  -0.09249506636175525, \
  5.86145544294642, \
  -12.92096931784711, \
  8.159367898576159, \
  -0.071584973281401, \
  -0.028269050394068383, \
  0.09646076681806523, \
  0.01, \
  0.4798896504144996, \
  1.379008574103742, \
  -3.290069515436081, \
  2.324710524099774, \
  -0.001780011052225777, \
  -0.0008164344596567469, \
  0.007880878010261995, \
  -0.1447110071732629, \
  0.5823571654525552, \
  -0.45808210592918697, \
  0.015151515151515152, \
  1.0, \
  -2.763706197274826, \
  2.9132554618219126, \
  -1.0530884977290216, \
  0.13169999999999998, \
  -0.2234, \
  0.1017, \
  3.9302962368947516, \
  -5.941033872131505, \
  2.490627285651253, \
  -12.411077166933676, \
  30.33818863028232, \
  -16.548102889244902, \
  37.50931341651104, \
  -88.1789048947664, \
  47.37952196281928, \
  -27.896526289197286, \
  65.09189467479366, \
  -34.87065786149661, \
  1.5, \
  -4.0, \
  2.5 \
}

/* vern7: src/verner/verner_tableaus.jl:376-452 (58 values) */
namespace gbtab { namespace vern7 {
constexpr double c2 = 0.005;
constexpr double c3 = 0.10888888888888888;
constexpr double c4 = 0.16333333333333333;
constexpr double c5 = 0.4555;
constexpr double c6 = 0.6095094489978381;
constexpr double c7 = 0.884;
constexpr double c8 = 0.925;
constexpr double a021 = 0.005;
constexpr double a031 = -1.07679012345679;
constexpr double a032 = 1.185679012345679;
constexpr double a041 = 0.04083333333333333;
constexpr double a043 = 0.1225;
constexpr double a051 = 0.6389139236255726;
constexpr double a053 = -2.455672638223657;
constexpr double a054 = 2.272258714598084;
constexpr double a061 = -2.6615773750187572;
constexpr double a063 = 10.804513886456137;
constexpr double a064 = -8.3539146573962;
constexpr double a065 = 0.820487594956657;
constexpr double a071 = 6.067741434696772;
constexpr double a073 = -24.711273635911088;
constexpr double a074 = 20.427517930788895;
constexpr double a075 = -1.9061579788166472;
constexpr double a076 = 1.006172249242068;
constexpr double a081 = 12.054670076253203;
constexpr double a083 = -49.75478495046899;
constexpr double a084 = 41.142888638604674;
constexpr double a085 = -4.461760149974004;
constexpr double a086 = 2.042334822239175;
constexpr double a087 = -0.09834843665406107;
constexpr double a091 = 10.138146522881808;
constexpr double a093 = -42.6411360317175;
constexpr double a094 = 35.76384003992257;
constexpr double a095 = -4.3480228403929075;
constexpr double a096 = 2.0098622683770357;
constexpr double a097 = 0.3487490460338272;
constexpr double a098 = -0.27143900510483127;
constexpr double a101 = -45.030072034298676;
constexpr double a103 = 187.3272437654589;
constexpr double a104 = -154.02882369350186;
constexpr double a105 = 18.56465306347536;
constexpr double a106 = -7.141809679295079;
constexpr double a107 = 1.3088085781613787;
constexpr double b1 = 0.04715561848627222;
constexpr double b4 = 0.25750564298434153;
constexpr double b5 = 0.26216653977412624;
constexpr double b6 = 0.15216092656738558;
constexpr double b7 = 0.4939969170032485;
constexpr double b8 = -0.29430311714032503;
constexpr double b9 = 0.08131747232495111;
constexpr double btilde1 = 0.002547011879931045;
constexpr double btilde4 = -0.00965839487279575;
constexpr double btilde5 = 0.04206470975639691;
constexpr double btilde6 = -0.0666822437469301;
constexpr double btilde7 = 0.2650097464621281;
constexpr double btilde8 = -0.29430311714032503;
constexpr double btilde9 = 0.08131747232495111;
constexpr double btilde10 = -0.02029518466335628;
} }
enum gbtab_vern7_pos {
  vern7_c2 = 0,
  vern7_c3 = 1,
  vern7_c4 = 2,
  vern7_c5 = 3,
  vern7_c6 = 4,
  vern7_c7 = 5,
  vern7_c8 = 6,
  vern7_a021 = 7,
  vern7_a031 = 8,
  vern7_a032 = 9,
  vern7_a041 = 10,
  vern7_a043 = 11,
  vern7_a051 = 12,
  vern7_a053 = 13,
  vern7_a054 = 14,
  vern7_a061 = 15,
  vern7_a063 = 16,
  vern7_a064 = 17,
  vern7_a065 = 18,
  vern7_a071 = 19,
  vern7_a073 = 20,
  vern7_a074 = 21,
  vern7_a075 = 22,
  vern7_a076 = 23,
  vern7_a081 = 24,
  vern7_a083 = 25,
  vern7_a084 = 26,
  vern7_a085 = 27,
  vern7_a086 = 28,
  vern7_a087 = 29,
  vern7_a091 = 30,
  vern7_a093 = 31,
  vern7_a094 = 32,
  vern7_a095 = 33,
  vern7_a096 = 34,
  vern7_a097 = 35,
  vern7_a098 = 36,
  vern7_a101 = 37,
  vern7_a103 = 38,
  vern7_a104 = 39,
  vern7_a105 = 40,
  vern7_a106 = 41,
  vern7_a107 = 42,
  vern7_b1 = 43,
  vern7_b4 = 44,
  vern7_b5 = 45,
  vern7_b6 = 46,
  vern7_b7 = 47,
  vern7_b8 = 48,
  vern7_b9 = 49,
  vern7_btilde1 = 50,
  vern7_btilde4 = 51,
  vern7_btilde5 = 52,
  vern7_btilde6 = 53,
  vern7_btilde7 = 54,
  vern7_btilde8 = 55,
  vern7_btilde9 = 56,
  vern7_btilde10 = 57,
  vern7_COUNT = 58
};
#define GBTAB_VERN7_INIT { \
  0.005, \
  0.10888888888888888, \
  0.16333333333333333, \
  0.4555, \
  0.6095094489978381, \
  0.884, \
  0.925, \
  0.005, \
  -1.07679012345679, \
  1.185679012345679, \
  0.04083333333333333, \
  0.1225, \
  0.6389139236255726, \
  -2.455672638223657, \
  2.272258714598084, \
  -2.6615773750187572, \
  10.804513886456137, \
  -8.3539146573962, \
  0.820487594956657, \
  6.067741434696772, \
  -24.711273635911088, \
  20.427517930788895, \
  -1.9061579788166472, \
  1.006172249242068, \
  12.054670076253203, \
  -49.75478495046899, \
  41.142888638604674, \
  -4.461760149974004, \
  2.042334822239175, \
  -0.09834843665406107, \
  10.138146522881808, \
  -42.6411360317175, \
  35.76384003992257, \
  -4.3480228403929075, \
  2.0098622683770357, \
  0.3487490460338272, \
  -0.27143900510483127, \
  -45.030072034298676, \
  187.3272437654589, \
  -154.02882369350186, \
  18.56465306347536, \
  -7.141809679295079, \
  1.3088085781613787, \
  0.04715561848627222, \
  0.25750564298434153, \
  0.26216653977412624, \
  0.15216092656738558, \
  0.4939969170032485, \
  -0.29430311714032503, \
  0.08131747232495111, \
  0.002547011879931045, \
  -0.00965839487279575, \
  0.04206470975639691, \
  -0.0666822437469301, \
  0.2650097464621281, \
  -0.29430311714032503, \
  0.08131747232495111, \
  -0.02029518466335628 \
}

/* vern7x: src/verner/verner_tableaus.jl:65-135 (60 values) */
namespace gbtab { namespace vern7x {
constexpr double c11 = 1.0;
constexpr double a1101 = 0.04715561848627222;
constexpr double a1104 = 0.25750564298434153;
constexpr double a1105 = 0.2621665397741262;
constexpr double a1106 = 0.15216092656738558;
constexpr double a1107 = 0.49399691700324844;
constexpr double a1108 = -0.29430311714032503;
constexpr double a1109 = 0.0813174723249511;
constexpr double c12 = 0.29;
constexpr double a1201 = 0.0523222769159969;
constexpr double a1204 = 0.22495861826705715;
constexpr double a1205 = 0.017443709248776376;
constexpr double a1206 = -0.007669379876829393;
constexpr double a1207 = 0.03435896044073285;
constexpr double a1208 = -0.0410209723009395;
constexpr double a1209 = 0.025651133005205617;
constexpr double a1211 = -0.0160443457;
constexpr double c13 = 0.125;
constexpr double a1301 = 0.053053341257859085;
constexpr double a1304 = 0.12195301011401886;
constexpr double a1305 = 0.017746840737602496;
constexpr double a1306 = -0.0005928372667681495;
constexpr double a1307 = 0.008381833970853752;
constexpr double a1308 = -0.01293369259698612;
constexpr double a1309 = 0.009412056815253861;
constexpr double a1311 = -0.005353253107275676;
constexpr double a1312 = -0.06666729992455811;
constexpr double c14 = 0.25;
constexpr double a1401 = 0.03887903257436304;
constexpr double a1404 = -0.0024403203308301317;
constexpr double a1405 = -0.0013928917214672623;
constexpr double a1406 = -0.00047446291558680135;
constexpr double a1407 = 0.00039207932413159514;
constexpr double a1408 = -0.00040554733285128004;
constexpr double a1409 = 0.00019897093147716726;
constexpr double a1411 = -0.00010278198793179169;
constexpr double a1412 = 0.03385661513870267;
constexpr double a1413 = 0.1814893063199928;
constexpr double c15 = 0.53;
constexpr double a1501 = 0.05723681204690013;
constexpr double a1504 = 0.22265948066761182;
constexpr double a1505 = 0.12344864200186899;
constexpr double a1506 = 0.04006332526666491;
constexpr double a1507 = -0.05269894848581452;
constexpr double a1508 = 0.04765971214244523;
constexpr double a1509 = -0.02138895885042213;
constexpr double a1511 = 0.015193891064036402;
constexpr double a1512 = 0.12060546716289655;
constexpr double a1513 = -0.022779423016187374;
constexpr double c16 = 0.79;
constexpr double a1601 = 0.051372038802756814;
constexpr double a1604 = 0.5414214473439406;
constexpr double a1605 = 0.350399806692184;
constexpr double a1606 = 0.14193112269692182;
constexpr double a1607 = 0.10527377478429423;
constexpr double a1608 = -0.031081847805874016;
constexpr double a1609 = -0.007401883149519145;
constexpr double a1611 = -0.006377932504865363;
constexpr double a1612 = -0.17325495908361865;
constexpr double a1613 = -0.18228156777622026;
} }
enum gbtab_vern7x_pos {
  vern7x_c11 = 0,
  vern7x_a1101 = 1,
  vern7x_a1104 = 2,
  vern7x_a1105 = 3,
  vern7x_a1106 = 4,
  vern7x_a1107 = 5,
  vern7x_a1108 = 6,
  vern7x_a1109 = 7,
  vern7x_c12 = 8,
  vern7x_a1201 = 9,
  vern7x_a1204 = 10,
  vern7x_a1205 = 11,
  vern7x_a1206 = 12,
  vern7x_a1207 = 13,
  vern7x_a1208 = 14,
  vern7x_a1209 = 15,
  vern7x_a1211 = 16,
  vern7x_c13 = 17,
  vern7x_a1301 = 18,
  vern7x_a1304 = 19,
  vern7x_a1305 = 20,
  vern7x_a1306 = 21,
  vern7x_a1307 = 22,
  vern7x_a1308 = 23,
  vern7x_a1309 = 24,
  vern7x_a1311 = 25,
  vern7x_a1312 = 26,
  vern7x_c14 = 27,
  vern7x_a1401 = 28,
  vern7x_a1404 = 29,
  vern7x_a1405 = 30,
  vern7x_a1406 = 31,
  vern7x_a1407 = 32,
  vern7x_a1408 = 33,
  vern7x_a1409 = 34,
  vern7x_a1411 = 35,
  vern7x_a1412 = 36,
  vern7x_a1413 = 37,
  vern7x_c15 = 38,
  vern7x_a1501 = 39,
  vern7x_a1504 = 40,
  vern7x_a1505 = 41,
  vern7x_a1506 = 42,
  vern7x_a1507 = 43,
  vern7x_a1508 = 44,
  vern7x_a1509 = 45,
  vern7x_a1511 = 46,
  vern7x_a1512 = 47,
  vern7x_a1513 = 48,
  vern7x_c16 = 49,
  vern7x_a1601 = 50,
  vern7x_a1604 = 51,
  vern7x_a1605 = 52,
  vern7x_a1606 = 53,
  vern7x_a1607 = 54,
  vern7x_a1608 = 55,
  vern7x_a1609 = 56,
  vern7x_a1611 = 57,
  vern7x_a1612 = 58,
  vern7x_a1613 = 59,
  vern7x_COUNT = 60
};
#define GBTAB_VERN7X_INIT { \
  1.0, \
  0.04715561848627222, \
  0.25750564298434153, \
  0.2621665397741262, \
  0.15216092656738558, \
  0.49399691700324844, \
  -0.29430311714032503, \
  0.0813174723249511, \
  0.29, \
  0.0523222769159969, \
  0.22495861826705715, \
  0.017443709248776376, \
  -0.007669379876829393, \
  0.03435896044073285, \
  -0.0410209723009395, \
  0.025651133005205617, \
  -0.0160443457, \
  0.125, \
  0.053053341257859085, \
  0.12195301011401886, \
  0.017746840737602496, \
  -0.0005928372667681495, \
  0.008381833970853752, \
  -0.01293369259698612, \
  0.009412056815253861, \
  -0.005353253107275676, \
  -0.06666729992455811, \
  0.25, \
  0.03887903257436304, \
  -0.0024403203308301317, \
  -0.0013928917214672623, \
  -0.00047446291558680135, \
  0.00039207932413159514, \
  -0.00040554733285128004, \
  0.00019897093147716726, \
  -0.00010278198793179169, \
  0.03385661513870267, \
  0.1814893063199928, \
  0.53, \
  0.05723681204690013, \
  0.22265948066761182, \
  0.12344864200186899, \
  0.04006332526666491, \
  -0.05269894848581452, \
  0.04765971214244523, \
  -0.02138895885042213, \
  0.015193891064036402, \
  0.12060546716289655, \
  -0.022779423016187374, \
  0.79, \
  0.051372038802756814, \
  0.5414214473439406, \
  0.350399806692184, \
  0.14193112269692182, \
  0.10527377478429423, \
  -0.031081847805874016, \
  -0.007401883149519145, \
  -0.006377932504865363, \
  -0.17325495908361865, \
  -0.18228156777622026 \
}

/* vern7r: src/verner/verner_tableaus.jl:219-311 (79 values) */
namespace gbtab { namespace vern7r {
constexpr double r011 = 1.0;
constexpr double r012 = -8.413387198332767;
constexpr double r013 = 33.675508884490895;
constexpr double r014 = -70.80159089484886;
constexpr double r015 = 80.64695108301298;
constexpr double r016 = -47.19413969837522;
constexpr double r017 = 11.133813442539243;
constexpr double r042 = 8.754921980674396;
constexpr double r043 = -88.4596828699771;
constexpr double r044 = 346.9017638429916;
constexpr double r045 = -629.2580030059837;
constexpr double r046 = 529.6773755604193;
constexpr double r047 = -167.35886986514018;
constexpr double r052 = 8.913387586637922;
constexpr double r053 = -90.06081846893218;
constexpr double r054 = 353.1807459217058;
constexpr double r055 = -640.6476819744374;
constexpr double r056 = 539.2646279047156;
constexpr double r057 = -170.38809442991547;
constexpr double r062 = 5.1733120298478;
constexpr double r063 = -52.271115900055385;
constexpr double r064 = 204.9853867374073;
constexpr double r065 = -371.8306118563603;
constexpr double r066 = 312.9880934374529;
constexpr double r067 = -98.89290352172495;
constexpr double r072 = 16.79537744079696;
constexpr double r073 = -169.70040000059728;
constexpr double r074 = 665.4937727009246;
constexpr double r075 = -1207.1638892336007;
constexpr double r076 = 1016.1291515818546;
constexpr double r077 = -321.06001557237494;
constexpr double r082 = -10.005997536098665;
constexpr double r083 = 101.1005433052275;
constexpr double r084 = -396.47391512378437;
constexpr double r085 = 719.1787707014183;
constexpr double r086 = -605.3681033918824;
constexpr double r087 = 191.27439892797935;
constexpr double r092 = 2.764708833638599;
constexpr double r093 = -27.934602637390462;
constexpr double r094 = 109.54779186137893;
constexpr double r095 = -198.7128113064482;
constexpr double r096 = 167.26633571640318;
constexpr double r097 = -52.85010499525706;
constexpr double r112 = -2.1696320280163506;
constexpr double r113 = 22.016696037569876;
constexpr double r114 = -86.90152427798948;
constexpr double r115 = 159.22388973861476;
constexpr double r116 = -135.9618306534588;
constexpr double r117 = 43.792401183280006;
constexpr double r122 = -4.890070188793804;
constexpr double r123 = 22.75407737425176;
constexpr double r124 = -30.78034218537731;
constexpr double r125 = -2.797194317207249;
constexpr double r126 = 31.369456637508403;
constexpr double r127 = -15.655927320381801;
constexpr double r132 = 10.862170929551967;
constexpr double r133 = -50.542971417827104;
constexpr double r134 = 68.37148040407511;
constexpr double r135 = 6.213326521632409;
constexpr double r136 = -69.68006323194157;
constexpr double r137 = 34.776056794509195;
constexpr double r142 = -11.37286691922923;
constexpr double r143 = 130.79058078246717;
constexpr double r144 = -488.65113677785604;
constexpr double r145 = 832.2148793276441;
constexpr double r146 = -664.7743368554426;
constexpr double r147 = 201.79288044241662;
constexpr double r152 = -5.919778732715007;
constexpr double r153 = 63.27679965889219;
constexpr double r154 = -265.432682088738;
constexpr double r155 = 520.1009254140611;
constexpr double r156 = -467.412109533902;
constexpr double r157 = 155.3868452824017;
constexpr double r162 = -10.492146197961823;
constexpr double r163 = 105.35538525188011;
constexpr double r164 = -409.43975011988937;
constexpr double r165 = 732.831448907654;
constexpr double r166 = -606.3044574733512;
constexpr double r167 = 188.0495196316683;
} }
enum gbtab_vern7r_pos {
  vern7r_r011 = 0,
  vern7r_r012 = 1,
  vern7r_r013 = 2,
  vern7r_r014 = 3,
  vern7r_r015 = 4,
  vern7r_r016 = 5,
  vern7r_r017 = 6,
  vern7r_r042 = 7,
  vern7r_r043 = 8,
  vern7r_r044 = 9,
  vern7r_r045 = 10,
  vern7r_r046 = 11,
  vern7r_r047 = 12,
  vern7r_r052 = 13,
  vern7r_r053 = 14,
  vern7r_r054 = 15,
  vern7r_r055 = 16,
  vern7r_r056 = 17,
  vern7r_r057 = 18,
  vern7r_r062 = 19,
  vern7r_r063 = 20,
  vern7r_r064 = 21,
  vern7r_r065 = 22,
  vern7r_r066 = 23,
  vern7r_r067 = 24,
  vern7r_r072 = 25,
  vern7r_r073 = 26,
  vern7r_r074 = 27,
  vern7r_r075 = 28,
  vern7r_r076 = 29,
  vern7r_r077 = 30,
  vern7r_r082 = 31,
  vern7r_r083 = 32,
  vern7r_r084 = 33,
  vern7r_r085 = 34,
  vern7r_r086 = 35,
  vern7r_r087 = 36,
  vern7r_r092 = 37,
  vern7r_r093 = 38,
  vern7r_r094 = 39,
  vern7r_r095 = 40,
  vern7r_r096 = 41,
  vern7r_r097 = 42,
  vern7r_r112 = 43,
  vern7r_r113 = 44,
  vern7r_r114 = 45,
  vern7r_r115 = 46,
  vern7r_r116 = 47,
  vern7r_r117 = 48,
  vern7r_r122 = 49,
  vern7r_r123 = 50,
  vern7r_r124 = 51,
  vern7r_r125 = 52,
  vern7r_r126 = 53,
  vern7r_r127 = 54,
  vern7r_r132 = 55,
  vern7r_r133 = 56,
  vern7r_r134 = 57,
  vern7r_r135 = 58,
  vern7r_r136 = 59,
  vern7r_r137 = 60,
  vern7r_r142 = 61,
  vern7r_r143 = 62,
  vern7r_r144 = 63,
  vern7r_r145 = 64,
  vern7r_r146 = 65,
  vern7r_r147 = 66,
  vern7r_r152 = 67,
  vern7r_r153 = 68,
  vern7r_r154 = 69,
  vern7r_r155 = 70,
  vern7r_r156 = 71,
  vern7r_r157 = 72,
  vern7r_r162 = 73,
  vern7r_r163 = 74,
  vern7r_r164 = 75,
  vern7r_r165 = 76,
  vern7r_r166 = 77,
  vern7r_r167 = 78,
  vern7r_COUNT = 79
};
#define GBTAB_VERN7R_INIT { \
  1.0, \
  -8.413387198332767, \
  33.675508884490895, \
  -70.80159089484886, \
  80.64695108301298, \
  -47.19413969837522, \
  11.133813442539243, \
  8.754921980674396, \
  -88.4596828699771, \
  346.9017638429916, \
  -629.2580030059837, \
  529.6773755604193, \
  -167.35886986514018, \
  8.913387586637922, \
  -90.06081846893218, \
  353.1807459217058, \
  -640.6476819744374, \
  539.2646279047156, \
  -170.38809442991547, \
  5.1733120298478, \
  -52.271115900055385, \
  204.9853867374073, \
  -371.8306118563603, \
  312.9880934374529, \
  -98.89290352172495, \
  16.79537744079696, \
  -169.70040000059728, \
  665.4937727009246, \
  -1207.1638892336007, \
  1016.1291515818546, \
  -321.06001557237494, \
  -10.005997536098665, \
  101.1005433052275, \
  -396.47391512378437, \
  719.1787707014183, \
  -605.3681033918824, \
  191.27439892797935, \
  2.764708833638599, \
  -27.934602637390462, \
  109.54779186137893, \
  -198.7128113064482, \
  167.26633571640318, \
  -52.85010499525706, \
  -2.1696320280163506, \
  22.016696037569876, \
  -86.90152427798948, \
  159.22388973861476, \
  -135.9618306534588, \
  43.792401183280006, \
  -4.890070188793804, \
  22.75407737425176, \
  -30.78034218537731, \
  -2.797194317207249, \
  31.369456637508403, \
  -15.655927320381801, \
  10.862170929551967, \
  -50.542971417827104, \
  68.37148040407511, \
  6.213326521632409, \
  -69.68006323194157, \
  34.776056794509195, \
  -11.37286691922923, \
  130.79058078246717, \
  -488.65113677785604, \
  832.2148793276441, \
  -664.7743368554426, \
  201.79288044241662, \
  -5.919778732715007, \
  63.27679965889219, \
  -265.432682088738, \
  520.1009254140611, \
  -467.412109533902, \
  155.3868452824017, \
  -10.492146197961823, \
  105.35538525188011, \
  -409.43975011988937, \
  732.831448907654, \
  -606.3044574733512, \
  188.0495196316683 \
}

/* vern9: src/verner/verner_tableaus.jl:1201-1335 (108 values) */
namespace gbtab { namespace vern9 {
constexpr double c1 = 0.03462;
constexpr double c2 = 0.09702435063878045;
constexpr double c3 = 0.14553652595817068;
constexpr double c4 = 0.561;
constexpr double c5 = 0.22900791159048503;
constexpr double c6 = 0.544992088409515;
constexpr double c7 = 0.645;
constexpr double c8 = 0.48375;
constexpr double c9 = 0.06757;
constexpr double c10 = 0.25;
constexpr double c11 = 0.6590650618730999;
constexpr double c12 = 0.8206;
constexpr double c13 = 0.9012;
constexpr double a0201 = 0.03462;
constexpr double a0301 = -0.03893354388572875;
constexpr double a0302 = 0.13595789452450918;
constexpr double a0401 = 0.03638413148954267;
constexpr double a0403 = 0.10915239446862801;
constexpr double a0501 = 2.0257639143939694;
constexpr double a0503 = -7.638023836496291;
constexpr double a0504 = 6.173259922102322;
constexpr double a0601 = 0.05112275589406061;
constexpr double a0604 = 0.17708237945550218;
constexpr double a0605 = 0.0008027762409222536;
constexpr double a0701 = 0.13160063579752163;
constexpr double a0704 = -0.2957276252669636;
constexpr double a0705 = 0.08781378035642955;
constexpr double a0706 = 0.6213052975225274;
constexpr double a0801 = 0.07166666666666667;
constexpr double a0806 = 0.33055335789153195;
constexpr double a0807 = 0.2427799754418014;
constexpr double a0901 = 0.071806640625;
constexpr double a0906 = 0.3294380283228177;
constexpr double a0907 = 0.1165190029271823;
constexpr double a0908 = -0.034013671875;
constexpr double a1001 = 0.04836757646340646;
constexpr double a1006 = 0.03928989925676164;
constexpr double a1007 = 0.10547409458903446;
constexpr double a1008 = -0.021438652846483126;
constexpr double a1009 = -0.10412291746271944;
constexpr double a1101 = -0.026645614872014785;
constexpr double a1106 = 0.03333333333333333;
constexpr double a1107 = -0.1631072244872467;
constexpr double a1108 = 0.03396081684127761;
constexpr double a1109 = 0.1572319413814626;
constexpr double a1110 = 0.21522674780318796;
constexpr double a1201 = 0.03689009248708622;
constexpr double a1206 = -0.1465181576725543;
constexpr double a1207 = 0.2242577768172024;
constexpr double a1208 = 0.02294405717066073;
constexpr double a1209 = -0.0035850052905728597;
constexpr double a1210 = 0.08669223316444385;
constexpr double a1211 = 0.43838406519683376;
constexpr double a1301 = -0.4866012215113341;
constexpr double a1306 = -6.304602650282853;
constexpr double a1307 = -0.2812456182894729;
constexpr double a1308 = -2.679019236219849;
constexpr double a1309 = 0.5188156639241577;
constexpr double a1310 = 1.3653531876033418;
constexpr double a1311 = 5.8850910885039465;
constexpr double a1312 = 2.8028087862720628;
constexpr double a1401 = 0.4185367457753472;
constexpr double a1406 = 6.724547581906459;
constexpr double a1407 = -0.42544428016461133;
constexpr double a1408 = 3.3432791530012653;
constexpr double a1409 = 0.6170816631175374;
constexpr double a1410 = -0.9299661239399329;
constexpr double a1411 = -6.099948804751011;
constexpr double a1412 = -3.002206187889399;
constexpr double a1413 = 0.2553202529443446;
constexpr double a1501 = -0.7793740861228848;
constexpr double a1506 = -13.937342538107776;
constexpr double a1507 = 1.2520488533793563;
constexpr double a1508 = -14.691500408016868;
constexpr double a1509 = -0.494705058533141;
constexpr double a1510 = 2.2429749091462368;
constexpr double a1511 = 13.367893803828643;
constexpr double a1512 = 14.396650486650687;
constexpr double a1513 = -0.79758133317768;
constexpr double a1514 = 0.4409353709534278;
constexpr double a1601 = 2.0580513374668867;
constexpr double a1606 = 22.357937727968032;
constexpr double a1607 = 0.9094981099755646;
constexpr double a1608 = 35.89110098240264;
constexpr double a1609 = -3.442515027624454;
constexpr double a1610 = -4.865481358036369;
constexpr double a1611 = -18.909803813543427;
constexpr double a1612 = -34.26354448030452;
constexpr double a1613 = 1.2647565216956427;
constexpr double b1 = 0.014611976858423152;
constexpr double b8 = -0.3915211862331339;
constexpr double b9 = 0.23109325002895065;
constexpr double b10 = 0.12747667699928525;
constexpr double b11 = 0.2246434176204158;
constexpr double b12 = 0.5684352689748513;
constexpr double b13 = 0.058258715572158275;
constexpr double b14 = 0.13643174034822156;
constexpr double b15 = 0.030570139830827976;
constexpr double btilde1 = -0.005357988290444578;
constexpr double btilde8 = -2.583020491182464;
constexpr double btilde9 = 0.14252253154686625;
constexpr double btilde10 = 0.013420653512688676;
constexpr double btilde11 = -0.02867296291409493;
constexpr double btilde12 = 2.624999655215792;
constexpr double btilde13 = -0.2825509643291537;
constexpr double btilde14 = 0.13643174034822156;
constexpr double btilde15 = 0.030570139830827976;
constexpr double btilde16 = -0.04834231373823958;
} }
enum gbtab_vern9_pos {
  vern9_c1 = 0,
  vern9_c2 = 1,
  vern9_c3 = 2,
  vern9_c4 = 3,
  vern9_c5 = 4,
  vern9_c6 = 5,
  vern9_c7 = 6,
  vern9_c8 = 7,
  vern9_c9 = 8,
  vern9_c10 = 9,
  vern9_c11 = 10,
  vern9_c12 = 11,
  vern9_c13 = 12,
  vern9_a0201 = 13,
  vern9_a0301 = 14,
  vern9_a0302 = 15,
  vern9_a0401 = 16,
  vern9_a0403 = 17,
  vern9_a0501 = 18,
  vern9_a0503 = 19,
  vern9_a0504 = 20,
  vern9_a0601 = 21,
  vern9_a0604 = 22,
  vern9_a0605 = 23,
  vern9_a0701 = 24,
  vern9_a0704 = 25,
  vern9_a0705 = 26,
  vern9_a0706 = 27,
  vern9_a0801 = 28,
  vern9_a0806 = 29,
  vern9_a0807 = 30,
  vern9_a0901 = 31,
  vern9_a0906 = 32,
  vern9_a0907 = 33,
  vern9_a0908 = 34,
  vern9_a1001 = 35,
  vern9_a1006 = 36,
  vern9_a1007 = 37,
  vern9_a1008 = 38,
  vern9_a1009 = 39,
  vern9_a1101 = 40,
  vern9_a1106 = 41,
  vern9_a1107 = 42,
  vern9_a1108 = 43,
  vern9_a1109 = 44,
  vern9_a1110 = 45,
  vern9_a1201 = 46,
  vern9_a1206 = 47,
  vern9_a1207 = 48,
  vern9_a1208 = 49,
  vern9_a1209 = 50,
  vern9_a1210 = 51,
  vern9_a1211 = 52,
  vern9_a1301 = 53,
  vern9_a1306 = 54,
  vern9_a1307 = 55,
  vern9_a1308 = 56,
  vern9_a1309 = 57,
  vern9_a1310 = 58,
  vern9_a1311 = 59,
  vern9_a1312 = 60,
  vern9_a1401 = 61,
  vern9_a1406 = 62,
  vern9_a1407 = 63,
  vern9_a1408 = 64,
  vern9_a1409 = 65,
  vern9_a1410 = 66,
  vern9_a1411 = 67,
  vern9_a1412 = 68,
  vern9_a1413 = 69,
  vern9_a1501 = 70,
  vern9_a1506 = 71,
  vern9_a1507 = 72,
  vern9_a1508 = 73,
  vern9_a1509 = 74,
  vern9_a1510 = 75,
  vern9_a1511 = 76,
  vern9_a1512 = 77,
  vern9_a1513 = 78,
  vern9_a1514 = 79,
  vern9_a1601 = 80,
  vern9_a1606 = 81,
  vern9_a1607 = 82,
  vern9_a1608 = 83,
  vern9_a1609 = 84,
  vern9_a1610 = 85,
  vern9_a1611 = 86,
  vern9_a1612 = 87,
  vern9_a1613 = 88,
  vern9_b1 = 89,
  vern9_b8 = 90,
  vern9_b9 = 91,
  vern9_b10 = 92,
  vern9_b11 = 93,
  vern9_b12 = 94,
  vern9_b13 = 95,
  vern9_b14 = 96,
  vern9_b15 = 97,
  vern9_btilde1 = 98,
  vern9_btilde8 = 99,
  vern9_btilde9 = 100,
  vern9_btilde10 = 101,
  vern9_btilde11 = 102,
  vern9_btilde12 = 103,
  vern9_btilde13 = 104,
  vern9_btilde14 = 105,
  vern9_btilde15 = 106,
  vern9_btilde16 = 107,
  vern9_COUNT = 108
};
#define GBTAB_VERN9_INIT { \
  0.03462, \
  0.09702435063878045, \
  0.14553652595817068, \
  0.561, \
  0.22900791159048503, \
  0.544992088409515, \
  0.645, \
  0.48375, \
  0.06757, \
  0.25, \
  0.6590650618730999, \
  0.8206, \
  0.9012, \
  0.03462, \
  -0.03893354388572875, \
  0.13595789452450918, \
  0.03638413148954267, \
  0.10915239446862801, \
  2.0257639143939694, \
  -7.638023836496291, \
  6.173259922102322, \
  0.05112275589406061, \
  0.17708237945550218, \
  0.0008027762409222536, \
  0.13160063579752163, \
  -0.2957276252669636, \
  0.08781378035642955, \
  0.6213052975225274, \
  0.07166666666666667, \
  0.33055335789153195, \
  0.2427799754418014, \
  0.071806640625, \
  0.3294380283228177, \
  0.1165190029271823, \
  -0.034013671875, \
  0.04836757646340646, \
  0.03928989925676164, \
  0.10547409458903446, \
  -0.021438652846483126, \
  -0.10412291746271944, \
  -0.026645614872014785, \
  0.03333333333333333, \
  -0.1631072244872467, \
  0.03396081684127761, \
  0.1572319413814626, \
  0.21522674780318796, \
  0.03689009248708622, \
  -0.1465181576725543, \
  0.2242577768172024, \
  0.02294405717066073, \
  -0.0035850052905728597, \
  0.08669223316444385, \
  0.43838406519683376, \
  -0.4866012215113341, \
  -6.304602650282853, \
  -0.2812456182894729, \
  -2.679019236219849, \
  0.5188156639241577, \
  1.3653531876033418, \
  5.8850910885039465, \
  2.8028087862720628, \
  0.4185367457753472, \
  6.724547581906459, \
  -0.42544428016461133, \
  3.3432791530012653, \
  0.6170816631175374, \
  -0.9299661239399329, \
  -6.099948804751011, \
  -3.002206187889399, \
  0.2553202529443446, \
  -0.7793740861228848, \
  -13.937342538107776, \
  1.2520488533793563, \
  -14.691500408016868, \
  -0.494705058533141, \
  2.2429749091462368, \
  13.367893803828643, \
  14.396650486650687, \
  -0.79758133317768, \
  0.4409353709534278, \
  2.0580513374668867, \
  22.357937727968032, \
  0.9094981099755646, \
  35.89110098240264, \
  -3.442515027624454, \
  -4.865481358036369, \
  -18.909803813543427, \
  -34.26354448030452, \
  1.2647565216956427, \
  0.014611976858423152, \
  -0.3915211862331339, \
  0.23109325002895065, \
  0.12747667699928525, \
  0.2246434176204158, \
  0.5684352689748513, \
  0.058258715572158275, \
  0.13643174034822156, \
  0.030570139830827976, \
  -0.005357988290444578, \
  -2.583020491182464, \
  0.14252253154686625, \
  0.013420653512688676, \
  -0.02867296291409493, \
  2.624999655215792, \
  -0.2825509643291537, \
  0.13643174034822156, \
  0.030570139830827976, \
  -0.04834231373823958 \
}

/* vern9x: src/verner/verner_tableaus.jl:595-751 (135 values) */
namespace gbtab { namespace vern9x {
constexpr double c17 = 1.0;
constexpr double a1701 = 0.014611976858423152;
constexpr double a1708 = -0.3915211862331339;
constexpr double a1709 = 0.23109325002895065;
constexpr double a1710 = 0.12747667699928525;
constexpr double a1711 = 0.2246434176204158;
constexpr double a1712 = 0.5684352689748513;
constexpr double a1713 = 0.058258715572158275;
constexpr double a1714 = 0.13643174034822156;
constexpr double a1715 = 0.030570139830827976;
constexpr double c18 = 0.7404185470631561;
constexpr double a1801 = 0.015499736681895594;
constexpr double a1808 = 0.3355153219059635;
constexpr double a1809 = 0.20036139441918607;
constexpr double a1810 = 0.12520606592835493;
constexpr double a1811 = 0.22986763931842066;
constexpr double a1812 = -0.20202506534761813;
constexpr double a1813 = 0.05917103230665457;
constexpr double a1814 = -0.026518347830476387;
constexpr double a1815 = -0.023840946021309713;
constexpr double a1817 = 0.027181715702085017;
constexpr double c19 = 0.888;
constexpr double a1901 = 0.013024539431143383;
constexpr double a1908 = -0.7452850902413112;
constexpr double a1909 = 0.2643867896429301;
constexpr double a1910 = 0.1313961758372754;
constexpr double a1911 = 0.21672538151229273;
constexpr double a1912 = 0.8734117564076053;
constexpr double a1913 = 0.011859056439357767;
constexpr double a1914 = 0.05876002941689551;
constexpr double a1915 = 0.003266518630202088;
constexpr double a1917 = -0.00895930864841793;
constexpr double a1918 = 0.06941415157202692;
constexpr double c20 = 0.696;
constexpr double a2001 = 0.013970899969259426;
constexpr double a2008 = -0.46657653359576745;
constexpr double a2009 = 0.24163727872162571;
constexpr double a2010 = 0.12903633413456747;
constexpr double a2011 = 0.22167006717351054;
constexpr double a2012 = 0.6257275123364645;
constexpr double a2013 = 0.04355312415679284;
constexpr double a2014 = 0.10119624916672908;
constexpr double a2015 = 0.01808582254679721;
constexpr double a2017 = -0.020798755876891697;
constexpr double a2018 = -0.09022232517086219;
constexpr double a2019 = -0.12127967356222542;
constexpr double c21 = 0.487;
constexpr double a2101 = 0.016046388883181127;
constexpr double a2108 = 0.09517712399458336;
constexpr double a2109 = 0.13591872646553177;
constexpr double a2110 = 0.1237765280959854;
constexpr double a2111 = 0.2335656264102966;
constexpr double a2112 = -0.09051508172625873;
constexpr double a2113 = -0.02537574270006131;
constexpr double a2114 = -0.13596316968871622;
constexpr double a2115 = -0.04679214284145113;
constexpr double a2117 = 0.05177958859391748;
constexpr double a2118 = 0.09672595677476774;
constexpr double a2119 = 0.14773126903407427;
constexpr double a2120 = -0.11507507129585039;
constexpr double c22 = 0.025;
constexpr double a2201 = 0.018029186238936207;
constexpr double a2208 = 0.06983601042028874;
constexpr double a2209 = -0.025412476607916634;
constexpr double a2210 = 0.008487827035463275;
constexpr double a2211 = -0.002427525516089802;
constexpr double a2212 = -0.10478397528938199;
constexpr double a2213 = -0.014731477952480419;
constexpr double a2214 = -0.03916338390816177;
constexpr double a2215 = -0.010056573432939595;
constexpr double a2217 = 0.011025103922048344;
constexpr double a2218 = 0.005092830749095398;
constexpr double a2219 = 0.04759715599420645;
constexpr double a2220 = 0.03386307003288383;
constexpr double a2221 = 0.02764422831404798;
constexpr double c23 = 0.15;
constexpr double a2301 = 0.01677431640522778;
constexpr double a2308 = 0.6220437408820475;
constexpr double a2309 = -0.2060859809768842;
constexpr double a2310 = 0.11563949897660589;
constexpr double a2311 = 0.026641017933783588;
constexpr double a2312 = -0.937681079341877;
constexpr double a2313 = -0.13678064667021603;
constexpr double a2314 = -0.3678480995268297;
constexpr double a2315 = -0.09547871314402478;
constexpr double a2317 = 0.10134920184223697;
constexpr double a2318 = -0.08911323084568594;
constexpr double a2319 = 0.46641409889747604;
constexpr double a2320 = 0.450273629235458;
constexpr double a2321 = 0.18385224633268188;
constexpr double c24 = 0.32;
constexpr double a2401 = 0.010711497314914442;
constexpr double a2408 = -0.07094336118221108;
constexpr double a2409 = 0.10021649003400916;
constexpr double a2410 = 0.13834539804680251;
constexpr double a2411 = 0.17963306335781634;
constexpr double a2412 = 0.09048246545576182;
constexpr double a2413 = -0.005460662294523339;
constexpr double a2414 = -0.030004579051196197;
constexpr double a2415 = -0.011451920269627991;
constexpr double a2417 = 0.010033946861093851;
constexpr double a2418 = -0.09506485282809046;
constexpr double a2419 = 0.04853358804093592;
constexpr double a2420 = 0.08013325919783924;
constexpr double a2421 = -0.1251643326835242;
constexpr double c25 = 0.78;
constexpr double a2501 = 0.014101720888692213;
constexpr double a2508 = -0.3713379753704491;
constexpr double a2509 = 0.22312655481171803;
constexpr double a2510 = 0.12870053459181202;
constexpr double a2511 = 0.22246006596754947;
constexpr double a2512 = 0.5382853042550702;
constexpr double a2513 = 0.05417202616988763;
constexpr double a2514 = 0.1256968791308744;
constexpr double a2515 = 0.027844927890020542;
constexpr double a2517 = -0.0307740924620506;
constexpr double a2518 = 0.008569805293689777;
constexpr double a2519 = -0.15351746905870445;
constexpr double a2520 = -0.021799570305481963;
constexpr double a2521 = 0.014471288197371868;
constexpr double c26 = 0.96;
constexpr double a2601 = 0.014246004117356466;
constexpr double a2608 = -0.3767107393295407;
constexpr double a2609 = 0.22523997807304214;
constexpr double a2610 = 0.128360307629253;
constexpr double a2611 = 0.22302387052616926;
constexpr double a2612 = 0.5463127827750747;
constexpr double a2613 = 0.0552619079137578;
constexpr double a2614 = 0.12856135087499826;
constexpr double a2615 = 0.028572506812964065;
constexpr double a2617 = -0.02398761886357109;
constexpr double a2618 = 0.055562244589105095;
constexpr double a2619 = -0.017406756507628386;
constexpr double a2620 = -0.03815462365996979;
constexpr double a2621 = 0.011118785048989178;
} }
enum gbtab_vern9x_pos {
  vern9x_c17 = 0,
  vern9x_a1701 = 1,
  vern9x_a1708 = 2,
  vern9x_a1709 = 3,
  vern9x_a1710 = 4,
  vern9x_a1711 = 5,
  vern9x_a1712 = 6,
  vern9x_a1713 = 7,
  vern9x_a1714 = 8,
  vern9x_a1715 = 9,
  vern9x_c18 = 10,
  vern9x_a1801 = 11,
  vern9x_a1808 = 12,
  vern9x_a1809 = 13,
  vern9x_a1810 = 14,
  vern9x_a1811 = 15,
  vern9x_a1812 = 16,
  vern9x_a1813 = 17,
  vern9x_a1814 = 18,
  vern9x_a1815 = 19,
  vern9x_a1817 = 20,
  vern9x_c19 = 21,
  vern9x_a1901 = 22,
  vern9x_a1908 = 23,
  vern9x_a1909 = 24,
  vern9x_a1910 = 25,
  vern9x_a1911 = 26,
  vern9x_a1912 = 27,
  vern9x_a1913 = 28,
  vern9x_a1914 = 29,
  vern9x_a1915 = 30,
  vern9x_a1917 = 31,
  vern9x_a1918 = 32,
  vern9x_c20 = 33,
  vern9x_a2001 = 34,
  vern9x_a2008 = 35,
  vern9x_a2009 = 36,
  vern9x_a2010 = 37,
  vern9x_a2011 = 38,
  vern9x_a2012 = 39,
  vern9x_a2013 = 40,
  vern9x_a2014 = 41,
  vern9x_a2015 = 42,
  vern9x_a2017 = 43,
  vern9x_a2018 = 44,
  vern9x_a2019 = 45,
  vern9x_c21 = 46,
  vern9x_a2101 = 47,
  vern9x_a2108 = 48,
  vern9x_a2109 = 49,
  vern9x_a2110 = 50,
  vern9x_a2111 = 51,
  vern9x_a2112 = 52,
  vern9x_a2113 = 53,
  vern9x_a2114 = 54,
  vern9x_a2115 = 55,
  vern9x_a2117 = 56,
  vern9x_a2118 = 57,
  vern9x_a2119 = 58,
  vern9x_a2120 = 59,
  vern9x_c22 = 60,
  vern9x_a2201 = 61,
  vern9x_a2208 = 62,
  vern9x_a2209 = 63,
  vern9x_a2210 = 64,
  vern9x_a2211 = 65,
  vern9x_a2212 = 66,
  vern9x_a2213 = 67,
  vern9x_a2214 = 68,
  vern9x_a2215 = 69,
  vern9x_a2217 = 70,
  vern9x_a2218 = 71,
  vern9x_a2219 = 72,
  vern9x_a2220 = 73,
  vern9x_a2221 = 74,
  vern9x_c23 = 75,
  vern9x_a2301 = 76,
  vern9x_a2308 = 77,
  vern9x_a2309 = 78,
  vern9x_a2310 = 79,
  vern9x_a2311 = 80,
  vern9x_a2312 = 81,
  vern9x_a2313 = 82,
  vern9x_a2314 = 83,
  vern9x_a2315 = 84,
  vern9x_a2317 = 85,
  vern9x_a2318 = 86,
  vern9x_a2319 = 87,
  vern9x_a2320 = 88,
  vern9x_a2321 = 89,
  vern9x_c24 = 90,
  vern9x_a2401 = 91,
  vern9x_a2408 = 92,
  vern9x_a2409 = 93,
  vern9x_a2410 = 94,
  vern9x_a2411 = 95,
  vern9x_a2412 = 96,
  vern9x_a2413 = 97,
  vern9x_a2414 = 98,
  vern9x_a2415 = 99,
  vern9x_a2417 = 100,
  vern9x_a2418 = 101,
  vern9x_a2419 = 102,
  vern9x_a2420 = 103,
  vern9x_a2421 = 104,
  vern9x_c25 = 105,
  vern9x_a2501 = 106,
  vern9x_a2508 = 107,
  vern9x_a2509 = 108,
  vern9x_a2510 = 109,
  vern9x_a2511 = 110,
  vern9x_a2512 = 111,
  vern9x_a2513 = 112,
  vern9x_a2514 = 113,
  vern9x_a2515 = 114,
  vern9x_a2517 = 115,
  vern9x_a2518 = 116,
  vern9x_a2519 = 117,
  vern9x_a2520 = 118,
  vern9x_a2521 = 119,
  vern9x_c26 = 120,
  vern9x_a2601 = 121,
  vern9x_a2608 = 122,
  vern9x_a2609 = 123,
  vern9x_a2610 = 124,
  vern9x_a2611 = 125,
  vern9x_a2612 = 126,
  vern9x_a2613 = 127,
  vern9x_a2614 = 128,
  vern9x_a2615 = 129,
  vern9x_a2617 = 130,
  vern9x_a2618 = 131,
  vern9x_a2619 = 132,
  vern9x_a2620 = 133,
  vern9x_a2621 = 134,
  vern9x_COUNT = 135
};
#define GBTAB_VERN9X_INIT { \
  1.0, \
  0.014611976858423152, \
  -0.3915211862331339, \
  0.23109325002895065, \
  0.12747667699928525, \
  0.2246434176204158, \
  0.5684352689748513, \
  0.058258715572158275, \
  0.13643174034822156, \
  0.030570139830827976, \
  0.7404185470631561, \
  0.015499736681895594, \
  0.3355153219059635, \
  0.20036139441918607, \
  0.12520606592835493, \
  0.22986763931842066, \
  -0.20202506534761813, \
  0.05917103230665457, \
  -0.026518347830476387, \
  -0.023840946021309713, \
  0.027181715702085017, \
  0.888, \
  0.013024539431143383, \
  -0.7452850902413112, \
  0.2643867896429301, \
  0.1313961758372754, \
  0.21672538151229273, \
  0.8734117564076053, \
  0.011859056439357767, \
  0.05876002941689551, \
  0.003266518630202088, \
  -0.00895930864841793, \
  0.06941415157202692, \
  0.696, \
  0.013970899969259426, \
  -0.46657653359576745, \
  0.24163727872162571, \
  0.12903633413456747, \
  0.22167006717351054, \
  0.6257275123364645, \
  0.04355312415679284, \
  0.10119624916672908, \
  0.01808582254679721, \
  -0.020798755876891697, \
  -0.09022232517086219, \
  -0.12127967356222542, \
  0.487, \
  0.016046388883181127, \
  0.09517712399458336, \
  0.13591872646553177, \
  0.1237765280959854, \
  0.2335656264102966, \
  -0.09051508172625873, \
  -0.02537574270006131, \
  -0.13596316968871622, \
  -0.04679214284145113, \
  0.05177958859391748, \
  0.09672595677476774, \
  0.14773126903407427, \
  -0.11507507129585039, \
  0.025, \
  0.018029186238936207, \
  0.06983601042028874, \
  -0.025412476607916634, \
  0.008487827035463275, \
  -0.002427525516089802, \
  -0.10478397528938199, \
  -0.014731477952480419, \
  -0.03916338390816177, \
  -0.010056573432939595, \
  0.011025103922048344, \
  0.005092830749095398, \
  0.04759715599420645, \
  0.03386307003288383, \
  0.02764422831404798, \
  0.15, \
  0.01677431640522778, \
  0.6220437408820475, \
  -0.2060859809768842, \
  0.11563949897660589, \
  0.026641017933783588, \
  -0.937681079341877, \
  -0.13678064667021603, \
  -0.3678480995268297, \
  -0.09547871314402478, \
  0.10134920184223697, \
  -0.08911323084568594, \
  0.46641409889747604, \
  0.450273629235458, \
  0.18385224633268188, \
  0.32, \
  0.010711497314914442, \
  -0.07094336118221108, \
  0.10021649003400916, \
  0.13834539804680251, \
  0.17963306335781634, \
  0.09048246545576182, \
  -0.005460662294523339, \
  -0.030004579051196197, \
  -0.011451920269627991, \
  0.010033946861093851, \
  -0.09506485282809046, \
  0.04853358804093592, \
  0.08013325919783924, \
  -0.1251643326835242, \
  0.78, \
  0.014101720888692213, \
  -0.3713379753704491, \
  0.22312655481171803, \
  0.12870053459181202, \
  0.22246006596754947, \
  0.5382853042550702, \
  0.05417202616988763, \
  0.1256968791308744, \
  0.027844927890020542, \
  -0.0307740924620506, \
  0.008569805293689777, \
  -0.15351746905870445, \
  -0.021799570305481963, \
  0.014471288197371868, \
  0.96, \
  0.014246004117356466, \
  -0.3767107393295407, \
  0.22523997807304214, \
  0.128360307629253, \
  0.22302387052616926, \
  0.5463127827750747, \
  0.0552619079137578, \
  0.12856135087499826, \
  0.028572506812964065, \
  -0.02398761886357109, \
  0.055562244589105095, \
  -0.017406756507628386, \
  -0.03815462365996979, \
  0.011118785048989178 \
}

/* vern9r: src/verner/verner_tableaus.jl:909-1083 (153 values) */
namespace gbtab { namespace vern9r {
constexpr double r011 = 1.0;
constexpr double r012 = -28.330488700617398;
constexpr double r013 = 257.6535452078578;
constexpr double r014 = -1152.1544557434572;
constexpr double r015 = 2909.390878345409;
constexpr double r016 = -4355.005172868188;
constexpr double r017 = 3834.083497036262;
constexpr double r018 = -1835.419052683407;
constexpr double r019 = 368.7958613829998;
constexpr double r082 = 2.649656243770091;
constexpr double r083 = -96.30312807816006;
constexpr double r084 = 869.3095462492796;
constexpr double r085 = -3395.688567551074;
constexpr double r086 = 6796.933987158715;
constexpr double r087 = -7340.848417712072;
constexpr double r088 = 4082.8488969923656;
constexpr double r089 = -919.2934944890586;
constexpr double r092 = -1.5639451819287329;
constexpr double r093 = 56.8423973927286;
constexpr double r094 = -513.1052300304285;
constexpr double r095 = 2004.2867021103232;
constexpr double r096 = -4011.8533059139295;
constexpr double r097 = 4332.895839278586;
constexpr double r098 = -2409.8793479371448;
constexpr double r099 = 542.6079835318221;
constexpr double r102 = -0.8627103334967224;
constexpr double r103 = 31.355653751851733;
constexpr double r104 = -283.0413682227354;
constexpr double r105 = 1105.613463426007;
constexpr double r106 = -2213.0362006784526;
constexpr double r107 = 2390.1310977541207;
constexpr double r108 = -1329.3482661468738;
constexpr double r109 = 299.31580712657853;
constexpr double r112 = -1.5202953379012147;
constexpr double r113 = 55.25592121120227;
constexpr double r114 = -498.7844190970741;
constexpr double r115 = 1948.346888525776;
constexpr double r116 = -3899.8821364075516;
constexpr double r117 = 4211.964345158858;
constexpr double r118 = -2342.619408856117;
constexpr double r119 = 527.4637482204279;
constexpr double r122 = -3.8469388441255234;
constexpr double r123 = 139.81898409868404;
constexpr double r124 = -1262.1186876216004;
constexpr double r125 = 4930.075848057311;
constexpr double r126 = -9868.21948606954;
constexpr double r127 = 10657.908924348867;
constexpr double r128 = -5927.738759872814;
constexpr double r129 = 1334.688551172191;
constexpr double r132 = -0.39427130612001415;
constexpr double r133 = 14.329994760676497;
constexpr double r134 = -129.35406659945582;
constexpr double r135 = 505.28160770025175;
constexpr double r136 = -1011.3900801394333;
constexpr double r137 = 1092.3250517818917;
constexpr double r138 = -607.531701930281;
constexpr double r139 = 136.79172444804232;
constexpr double r142 = -0.9233145622082102;
constexpr double r143 = 33.55834582309799;
constexpr double r144 = -302.9246397549736;
constexpr double r145 = 1183.2813069678675;
constexpr double r146 = -2368.4989867901113;
constexpr double r147 = 2558.034559755808;
constexpr double r148 = -1422.7331755778803;
constexpr double r149 = 320.3423358787482;
constexpr double r152 = -0.20688628029300538;
constexpr double r153 = 7.519388975651663;
constexpr double r154 = -67.87605708082904;
constexpr double r155 = 265.136799698415;
constexpr double r156 = -530.7074807559026;
constexpr double r157 = 573.176549564149;
constexpr double r158 = -318.7905688834869;
constexpr double r159 = 71.77882490212657;
constexpr double r172 = -0.44724419067440996;
constexpr double r173 = 16.44684676010504;
constexpr double r174 = -154.40861059212955;
constexpr double r175 = 641.8986298540249;
constexpr double r176 = -1391.9392256879823;
constexpr double r177 = 1643.890568302952;
constexpr double r178 = -1004.0652972233179;
constexpr double r179 = 248.6243327770223;
constexpr double r182 = -0.1507876007899798;
constexpr double r183 = 5.527328824824632;
constexpr double r184 = -51.33833743084619;
constexpr double r185 = 209.60220027032804;
constexpr double r186 = -442.7692650421826;
constexpr double r187 = 505.0579312588053;
constexpr double r188 = -295.63364106156195;
constexpr double r189 = 69.70457078142275;
constexpr double r192 = -0.6413652207435296;
constexpr double r193 = 23.510132486246846;
constexpr double r194 = -218.36426832469724;
constexpr double r195 = 891.5292818535365;
constexpr double r196 = -1883.290177206008;
constexpr double r197 = 2148.2309544883997;
constexpr double r198 = -1257.4584015217124;
constexpr double r199 = 296.4838434449778;
constexpr double r202 = 1.8107293134448457;
constexpr double r203 = -66.37479657295337;
constexpr double r204 = 616.4952025401107;
constexpr double r205 = -2517.0030307773227;
constexpr double r206 = 5316.984175781034;
constexpr double r207 = -6064.976140789574;
constexpr double r208 = 3550.1095388883914;
constexpr double r209 = -837.0456783831302;
constexpr double r212 = 0.05176008760353718;
constexpr double r213 = -1.8973378625803488;
constexpr double r214 = 17.622648207936294;
constexpr double r215 = -71.94907400242467;
constexpr double r216 = 151.9871383765666;
constexpr double r217 = -173.36864987478606;
constexpr double r218 = 101.4806461521468;
constexpr double r219 = -23.927131084462175;
constexpr double r222 = 31.321782556688;
constexpr double r223 = -355.6570858339106;
constexpr double r224 = 1752.6852824895159;
constexpr double r225 = -4708.092293138363;
constexpr double r226 = 7370.900776193489;
constexpr double r227 = -6716.504964764566;
constexpr double r228 = 3303.940398161186;
constexpr double r229 = -678.5938956640391;
constexpr double r232 = -2.7196073341859246;
constexpr double r233 = 86.64045615858264;
constexpr double r234 = -454.1926030939031;
constexpr double r235 = 1014.7492211005434;
constexpr double r236 = -1133.583456714544;
constexpr double r237 = 610.4671827718666;
constexpr double r238 = -109.02334994495438;
constexpr double r239 = -12.337842943405471;
constexpr double r242 = 3.1772148014329233;
constexpr double r243 = -113.8098697715143;
constexpr double r244 = 978.0935981825675;
constexpr double r245 = -3575.1293776236703;
constexpr double r246 = 6764.3615198384505;
constexpr double r247 = -6987.161043852012;
constexpr double r248 = 3751.9057627895713;
constexpr double r249 = -821.4378043648254;
constexpr double r252 = 0.877284308346553;
constexpr double r253 = -31.51810423988375;
constexpr double r254 = 273.1229151353221;
constexpr double r255 = -993.2198643101782;
constexpr double r256 = 1787.888078312664;
constexpr double r257 = -1677.394835799641;
constexpr double r258 = 781.3579535062688;
constexpr double r259 = -141.11342691289855;
constexpr double r262 = 1.7194275817987157;
constexpr double r263 = -62.89867309250732;
constexpr double r264 = 580.333550787398;
constexpr double r265 = -2348.110620506761;
constexpr double r266 = 4921.119298612906;
constexpr double r267 = -5597.912448707917;
constexpr double r268 = 3288.5977751496216;
constexpr double r269 = -782.8483098245397;
} }
enum gbtab_vern9r_pos {
  vern9r_r011 = 0,
  vern9r_r012 = 1,
  vern9r_r013 = 2,
  vern9r_r014 = 3,
  vern9r_r015 = 4,
  vern9r_r016 = 5,
  vern9r_r017 = 6,
  vern9r_r018 = 7,
  vern9r_r019 = 8,
  vern9r_r082 = 9,
  vern9r_r083 = 10,
  vern9r_r084 = 11,
  vern9r_r085 = 12,
  vern9r_r086 = 13,
  vern9r_r087 = 14,
  vern9r_r088 = 15,
  vern9r_r089 = 16,
  vern9r_r092 = 17,
  vern9r_r093 = 18,
  vern9r_r094 = 19,
  vern9r_r095 = 20,
  vern9r_r096 = 21,
  vern9r_r097 = 22,
  vern9r_r098 = 23,
  vern9r_r099 = 24,
  vern9r_r102 = 25,
  vern9r_r103 = 26,
  vern9r_r104 = 27,
  vern9r_r105 = 28,
  vern9r_r106 = 29,
  vern9r_r107 = 30,
  vern9r_r108 = 31,
  vern9r_r109 = 32,
  vern9r_r112 = 33,
  vern9r_r113 = 34,
  vern9r_r114 = 35,
  vern9r_r115 = 36,
  vern9r_r116 = 37,
  vern9r_r117 = 38,
  vern9r_r118 = 39,
  vern9r_r119 = 40,
  vern9r_r122 = 41,
  vern9r_r123 = 42,
  vern9r_r124 = 43,
  vern9r_r125 = 44,
  vern9r_r126 = 45,
  vern9r_r127 = 46,
  vern9r_r128 = 47,
  vern9r_r129 = 48,
  vern9r_r132 = 49,
  vern9r_r133 = 50,
  vern9r_r134 = 51,
  vern9r_r135 = 52,
  vern9r_r136 = 53,
  vern9r_r137 = 54,
  vern9r_r138 = 55,
  vern9r_r139 = 56,
  vern9r_r142 = 57,
  vern9r_r143 = 58,
  vern9r_r144 = 59,
  vern9r_r145 = 60,
  vern9r_r146 = 61,
  vern9r_r147 = 62,
  vern9r_r148 = 63,
  vern9r_r149 = 64,
  vern9r_r152 = 65,
  vern9r_r153 = 66,
  vern9r_r154 = 67,
  vern9r_r155 = 68,
  vern9r_r156 = 69,
  vern9r_r157 = 70,
  vern9r_r158 = 71,
  vern9r_r159 = 72,
  vern9r_r172 = 73,
  vern9r_r173 = 74,
  vern9r_r174 = 75,
  vern9r_r175 = 76,
  vern9r_r176 = 77,
  vern9r_r177 = 78,
  vern9r_r178 = 79,
  vern9r_r179 = 80,
  vern9r_r182 = 81,
  vern9r_r183 = 82,
  vern9r_r184 = 83,
  vern9r_r185 = 84,
  vern9r_r186 = 85,
  vern9r_r187 = 86,
  vern9r_r188 = 87,
  vern9r_r189 = 88,
  vern9r_r192 = 89,
  vern9r_r193 = 90,
  vern9r_r194 = 91,
  vern9r_r195 = 92,
  vern9r_r196 = 93,
  vern9r_r197 = 94,
  vern9r_r198 = 95,
  vern9r_r199 = 96,
  vern9r_r202 = 97,
  vern9r_r203 = 98,
  vern9r_r204 = 99,
  vern9r_r205 = 100,
  vern9r_r206 = 101,
  vern9r_r207 = 102,
  vern9r_r208 = 103,
  vern9r_r209 = 104,
  vern9r_r212 = 105,
  vern9r_r213 = 106,
  vern9r_r214 = 107,
  vern9r_r215 = 108,
  vern9r_r216 = 109,
  vern9r_r217 = 110,
  vern9r_r218 = 111,
  vern9r_r219 = 112,
  vern9r_r222 = 113,
  vern9r_r223 = 114,
  vern9r_r224 = 115,
  vern9r_r225 = 116,
  vern9r_r226 = 117,
  vern9r_r227 = 118,
  vern9r_r228 = 119,
  vern9r_r229 = 120,
  vern9r_r232 = 121,
  vern9r_r233 = 122,
  vern9r_r234 = 123,
  vern9r_r235 = 124,
  vern9r_r236 = 125,
  vern9r_r237 = 126,
  vern9r_r238 = 127,
  vern9r_r239 = 128,
  vern9r_r242 = 129,
  vern9r_r243 = 130,
  vern9r_r244 = 131,
  vern9r_r245 = 132,
  vern9r_r246 = 133,
  vern9r_r247 = 134,
  vern9r_r248 = 135,
  vern9r_r249 = 136,
  vern9r_r252 = 137,
  vern9r_r253 = 138,
  vern9r_r254 = 139,
  vern9r_r255 = 140,
  vern9r_r256 = 141,
  vern9r_r257 = 142,
  vern9r_r258 = 143,
  vern9r_r259 = 144,
  vern9r_r262 = 145,
  vern9r_r263 = 146,
  vern9r_r264 = 147,
  vern9r_r265 = 148,
  vern9r_r266 = 149,
  vern9r_r267 = 150,
  vern9r_r268 = 151,
  vern9r_r269 = 152,
  vern9r_COUNT = 153
};
#define GBTAB_VERN9R_INIT { \
  1.0, \
  -28.330488700617398, \
  257.6535452078578, \
  -1152.1544557434572, \
  2909.390878345409, \
  -4355.005172868188, \
  3834.083497036262, \
  -1835.419052683407, \
  368.7958613829998, \
  2.649656243770091, \
  -96.30312807816006, \
  869.3095462492796, \
  -3395.688567551074, \
  6796.933987158715, \
  -7340.848417712072, \
  4082.8488969923656, \
  -919.2934944890586, \
  -1.5639451819287329, \
  56.8423973927286, \
  -513.1052300304285, \
  2004.2867021103232, \
  -4011.8533059139295, \
  4332.895839278586, \
  -2409.8793479371448, \
  542.6079835318221, \
  -0.8627103334967224, \
  31.355653751851733, \
  -283.0413682227354, \
  1105.613463426007, \
  -2213.0362006784526, \
  2390.1310977541207, \
  -1329.3482661468738, \
  299.31580712657853, \
  -1.5202953379012147, \
  55.25592121120227, \
  -498.7844190970741, \
  1948.346888525776, \
  -3899.8821364075516, \
  4211.964345158858, \
  -2342.619408856117, \
  527.4637482204279, \
  -3.8469388441255234, \
  139.81898409868404, \
  -1262.1186876216004, \
  4930.075848057311, \
  -9868.21948606954, \
  10657.908924348867, \
  -5927.738759872814, \
  1334.688551172191, \
  -0.39427130612001415, \
  14.329994760676497, \
  -129.35406659945582, \
  505.28160770025175, \
  -1011.3900801394333, \
  1092.3250517818917, \
  -607.531701930281, \
  136.79172444804232, \
  -0.9233145622082102, \
  33.55834582309799, \
  -302.9246397549736, \
  1183.2813069678675, \
  -2368.4989867901113, \
  2558.034559755808, \
  -1422.7331755778803, \
  320.3423358787482, \
  -0.20688628029300538, \
  7.519388975651663, \
  -67.87605708082904, \
  265.136799698415, \
  -530.7074807559026, \
  573.176549564149, \
  -318.7905688834869, \
  71.77882490212657, \
  -0.44724419067440996, \
  16.44684676010504, \
  -154.40861059212955, \
  641.8986298540249, \
  -1391.9392256879823, \
  1643.890568302952, \
  -1004.0652972233179, \
  248.6243327770223, \
  -0.1507876007899798, \
  5.527328824824632, \
  -51.33833743084619, \
  209.60220027032804, \
  -442.7692650421826, \
  505.0579312588053, \
  -295.63364106156195, \
  69.70457078142275, \
  -0.6413652207435296, \
  23.510132486246846, \
  -218.36426832469724, \
  891.5292818535365, \
  -1883.290177206008, \
  2148.2309544883997, \
  -1257.4584015217124, \
  296.4838434449778, \
  1.8107293134448457, \
  -66.37479657295337, \
  616.4952025401107, \
  -2517.0030307773227, \
  5316.984175781034, \
  -6064.976140789574, \
  3550.1095388883914, \
  -837.0456783831302, \
  0.05176008760353718, \
  -1.8973378625803488, \
  17.622648207936294, \
  -71.94907400242467, \
  151.9871383765666, \
  -173.36864987478606, \
  101.4806461521468, \
  -23.927131084462175, \
  31.321782556688, \
  -355.6570858339106, \
  1752.6852824895159, \
  -4708.092293138363, \
  7370.900776193489, \
  -6716.504964764566, \
  3303.940398161186, \
  -678.5938956640391, \
  -2.7196073341859246, \
  86.64045615858264, \
  -454.1926030939031, \
  1014.7492211005434, \
  -1133.583456714544, \
  610.4671827718666, \
  -109.02334994495438, \
  -12.337842943405471, \
  3.1772148014329233, \
  -113.8098697715143, \
  978.0935981825675, \
  -3575.1293776236703, \
  6764.3615198384505, \
  -6987.161043852012, \
  3751.9057627895713, \
  -821.4378043648254, \
  0.877284308346553, \
  -31.51810423988375, \
  273.1229151353221, \
  -993.2198643101782, \
  1787.888078312664, \
  -1677.394835799641, \
  781.3579535062688, \
  -141.11342691289855, \
  1.7194275817987157, \
  -62.89867309250732, \
  580.333550787398, \
  -2348.110620506761, \
  4921.119298612906, \
  -5597.912448707917, \
  3288.5977751496216, \
  -782.8483098245397 \
}

