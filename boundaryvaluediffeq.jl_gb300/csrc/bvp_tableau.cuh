// MIRK tableaus and continuous-extension weights for the device code, folded at compile
// time for the order BVP_ORDER.
//
// The coefficients are the published MIRK schemes as the reference tabulates them:
//   discrete tableaus   lib/BoundaryValueDiffEqMIRK/src/mirk_tableaus.jl:13-152
//   stage counts        lib/BoundaryValueDiffEqMIRK/src/alg_utils.jl:1-13 (s = order - 1)
//   interpolant weights lib/BoundaryValueDiffEqMIRK/src/interpolation.jl:459-580
// x_star is indexed [extra stage r][stage j] (the reference's column-major layout,
// interpolation.jl:308-309).
#pragma once

namespace bvp {

constexpr int ORD = BVP_ORDER;
constexpr int S = ORD - 1;
constexpr int SS = (ORD == 2 || ORD == 3) ? 3 : (ORD == 4 ? 4 : (ORD == 5 ? 6 : 9));
constexpr int NSX = SS - S;           // extra interpolant stages
constexpr int NSXA = NSX > 0 ? NSX : 1;

BVP_DEV constexpr double tab_c(int r) {
    if (ORD == 2) return 0.5;
    if (ORD == 3) return r == 0 ? 0.0 : 2.0 / 3.0;
    if (ORD == 4) return r == 0 ? 0.0 : (r == 1 ? 1.0 : 0.5);
    if (ORD == 5) return r == 0 ? 0.0 : (r == 1 ? 1.0 : (r == 2 ? 0.75 : 0.3));
    return r == 0 ? 0.0 : (r == 1 ? 1.0 : (r == 2 ? 0.25 : (r == 3 ? 0.75 : 0.5)));
}
BVP_DEV constexpr double tab_v(int r) {
    if (ORD == 2) return 0.5;
    if (ORD == 3) return r == 0 ? 0.0 : 4.0 / 9.0;
    if (ORD == 4) return r == 0 ? 0.0 : (r == 1 ? 1.0 : 0.5);
    if (ORD == 5) return r == 0 ? 0.0 : (r == 1 ? 1.0 : (r == 2 ? 27.0 / 32.0 : 837.0 / 1250.0));
    return r == 0 ? 0.0 : (r == 1 ? 1.0 : (r == 2 ? 5.0 / 32.0 : (r == 3 ? 27.0 / 32.0 : 0.5)));
}
BVP_DEV constexpr double tab_b(int r) {
    if (ORD == 2) return 1.0;
    if (ORD == 3) return r == 0 ? 0.25 : 0.75;
    if (ORD == 4) return r == 2 ? 2.0 / 3.0 : 1.0 / 6.0;
    if (ORD == 5) return r == 0 ? 5.0 / 54.0 : (r == 1 ? 1.0 / 14.0 : (r == 2 ? 32.0 / 81.0 : 250.0 / 567.0));
    return r <= 1 ? 7.0 / 90.0 : (r <= 3 ? 16.0 / 45.0 : 2.0 / 15.0);
}
BVP_DEV constexpr double tab_x(int r, int j) {
    if (ORD == 3) return (r == 1 && j == 0) ? 2.0 / 9.0 : 0.0;
    if (ORD == 4) return r == 2 ? (j == 0 ? 0.125 : (j == 1 ? -0.125 : 0.0)) : 0.0;
    if (ORD == 5) {
        if (r == 2) return j == 0 ? 3.0 / 64.0 : (j == 1 ? -9.0 / 64.0 : 0.0);
        if (r == 3) return j == 0 ? 21.0 / 1000.0 : (j == 1 ? 63.0 / 5000.0 : (j == 2 ? -252.0 / 625.0 : 0.0));
        return 0.0;
    }
    if (ORD == 6) {
        if (r == 2) return j == 0 ? 9.0 / 64.0 : (j == 1 ? -3.0 / 64.0 : 0.0);
        if (r == 3) return j == 0 ? 3.0 / 64.0 : (j == 1 ? -9.0 / 64.0 : 0.0);
        if (r == 4) return j == 0 ? -5.0 / 24.0 : (j == 1 ? 5.0 / 24.0 : (j == 2 ? 2.0 / 3.0 : (j == 3 ? -2.0 / 3.0 : 0.0)));
        return 0.0;
    }
    return 0.0;
}
BVP_DEV constexpr double tab_cs(int r) {
    if (ORD == 2) return r == 0 ? 0.0 : 1.0;
    if (ORD == 3) return 1.0;
    if (ORD == 4) return 0.75;
    if (ORD == 5) return r == 0 ? 0.8 : 13.0 / 23.0;
    return r == 0 ? 7.0 / 16.0 : (r == 1 ? 3.0 / 8.0 : (r == 2 ? 9.0 / 16.0 : 1.0 / 8.0));
}
BVP_DEV constexpr double tab_vs(int r) {
    if (ORD == 4) return 27.0 / 32.0;
    return tab_cs(r);
}
BVP_DEV constexpr double tab_xs(int r, int j) {
    if (ORD == 4) return j == 0 ? 3.0 / 64.0 : (j == 1 ? -9.0 / 64.0 : 0.0);
    if (ORD == 5) {
        if (r == 0) return j == 0 ? 14.0 / 1125.0 : (j == 1 ? -74.0 / 875.0 : (j == 2 ? -128.0 / 3375.0 : (j == 3 ? 104.0 / 945.0 : 0.0)));
        return j == 0 ? 0.5 : (j == 1 ? 4508233.0 / 1958887.0 : (j == 2 ? 48720832.0 / 2518569.0 :
               (j == 3 ? -27646420.0 / 17629983.0 : (j == 4 ? -11517095.0 / 559682.0 : 0.0))));
    }
    if (ORD == 6) {
        if (r == 0) return j == 0 ? 1547.0 / 32768.0 : (j == 1 ? -1225.0 / 32768.0 : (j == 2 ? 749.0 / 4096.0 : (j == 3 ? -287.0 / 2048.0 : (j == 4 ? -861.0 / 16384.0 : 0.0))));
        if (r == 1) return j == 0 ? 83.0 / 1536.0 : (j == 1 ? -13.0 / 384.0 : (j == 2 ? 283.0 / 1536.0 : (j == 3 ? -167.0 / 1536.0 : (j == 4 ? -49.0 / 512.0 : 0.0))));
        if (r == 2) return j == 0 ? 1225.0 / 32768.0 : (j == 1 ? -1547.0 / 32768.0 : (j == 2 ? 287.0 / 2048.0 : (j == 3 ? -749.0 / 4096.0 : (j == 4 ? 861.0 / 16384.0 : 0.0))));
        return j == 0 ? 233.0 / 3456.0 : (j == 1 ? -19.0 / 1152.0 : (j == 5 ? -5.0 / 72.0 : (j == 6 ? 7.0 / 72.0 : (j == 7 ? -17.0 / 216.0 : 0.0))));
    }
    return 0.0;
}
BVP_DEV constexpr double tau_star() {
    return ORD == 2 ? 0.25 : (ORD == 3 ? 0.25 : (ORD == 4 ? 0.226 : (ORD == 5 ? 0.3 : 0.7156)));
}

// w(τ) and w'(τ), SS entries each, evaluated in the precision R
template <class R>
BVP_DEV void interp_weights(R t, R* w, R* wp) {
#define WC(x) R(x)
    const R t2 = t * t, t3 = t2 * t, t4 = t3 * t, t5 = t4 * t, t6 = t5 * t;
    if (ORD == 2) {
        w[0] = WC(0); w[1] = t * (WC(1) - t / WC(2)); w[2] = t2 / WC(2);
        wp[0] = WC(0); wp[1] = WC(1) - t; wp[2] = t;
    } else if (ORD == 3) {
        w[0] = t / WC(4.0) * (WC(2.0) * t2 - WC(5.0) * t + WC(4.0));
        w[1] = WC(-3.0 / 4.0) * t2 * (WC(2.0) * t - WC(3.0));
        w[2] = t2 * (t - WC(1.0));
        wp[0] = WC(3.0 / 2.0) * (t - WC(2.0 / 3.0)) * (t - WC(1.0));
        wp[1] = WC(-9.0 / 2.0) * t * (t - WC(1.0));
        wp[2] = WC(3.0) * t * (t - WC(2.0 / 3.0));
    } else if (ORD == 4) {
        const R tm1 = t - WC(1.0), t4m3 = t * WC(4.0) - WC(3.0), t2m1 = t * WC(2.0) - WC(1.0);
        w[0] = -t * (WC(2.0) * t - WC(3.0)) * (WC(2.0) * t2 - WC(3.0) * t + WC(2.0)) / WC(6.0);
        w[1] = t2 * (WC(12.0) * t2 - WC(20.0) * t + WC(9.0)) / WC(6.0);
        w[2] = WC(2.0) * t2 * (WC(6.0) * t2 - WC(14.0) * t + WC(9.0)) / WC(3.0);
        w[3] = WC(-16.0) * t2 * tm1 * tm1 / WC(3.0);
        wp[0] = -tm1 * t4m3 * t2m1 / WC(3.0);
        wp[1] = t * t2m1 * t4m3;
        wp[2] = WC(4.0) * t * t4m3 * tm1;
        wp[3] = WC(-32.0) * t * t2m1 * tm1 / WC(3.0);
    } else if (ORD == 5) {
        w[0] = t * (WC(22464.0) - WC(83910.0) * t + WC(143041.0) * t2 - WC(113808.0) * t3 + WC(33256.0) * t4) / WC(22464.0);
        w[1] = t2 * (WC(-2418.0) + WC(12303.0) * t - WC(19512.0) * t2 + WC(10904.0) * t3) / WC(3360.0);
        w[2] = WC(-8.0 / 81.0) * t2 * (WC(-78.0) + WC(209.0) * t - WC(204.0) * t2 + WC(8.0) * t3);
        w[3] = WC(-25.0 / 1134.0) * t2 * (WC(-390.0) + WC(1045.0) * t - WC(1020.0) * t2 + WC(328.0) * t3);
        w[4] = WC(-25.0 / 5184.0) * t2 * (WC(390.0) + WC(255.0) * t - WC(1680.0) * t2 + WC(2072.0) * t3);
        w[5] = WC(279841.0 / 168480.0) * t2 * (WC(-6.0) + WC(21.0) * t - WC(24.0) * t2 + WC(8.0) * t3);
        wp[0] = WC(1.0) - WC(13985.0 / 1872.0) * t + WC(143041.0 / 7488.0) * t2 - WC(2371.0 / 117.0) * t3 + WC(20785.0 / 2808.0) * t4;
        wp[1] = WC(-403.0 / 280.0) * t + WC(12303.0 / 1120.0) * t2 - WC(813.0 / 35.0) * t3 + WC(1363.0 / 84.0) * t4;
        wp[2] = WC(416.0 / 27.0) * t - WC(1672.0 / 27.0) * t2 + WC(2176.0 / 27.0) * t3 - WC(320.0 / 81.0) * t4;
        wp[3] = WC(3250.0 / 189.0) * t - WC(26125.0 / 378.0) * t2 + WC(17000.0 / 189.0) * t3 - WC(20500.0 / 567.0) * t4;
        wp[4] = WC(-1625.0 / 432.0) * t - WC(2125.0 / 576.0) * t2 + WC(875.0 / 27.0) * t3 - WC(32375.0 / 648.0) * t4;
        wp[5] = WC(-279841.0 / 14040.0) * t + WC(1958887.0 / 18720.0) * t2 - WC(279841.0 / 1755.0) * t3 + WC(279841.0 / 4212.0) * t4;
    } else {
        w[0] = t - WC(28607.0 / 7434.0) * t2 - WC(166210.0 / 33453.0) * t3 + WC(334780.0 / 11151.0) * t4 -
               WC(1911296.0 / 55755.0) * t5 + WC(406528.0 / 33453.0) * t6;
        w[1] = WC(777.0 / 590.0) * t2 - WC(2534158.0 / 234171.0) * t3 + WC(2088580.0 / 78057.0) * t4 -
               WC(10479104.0 / 390285.0) * t5 + WC(11328512.0 / 1170855.0) * t6;
        w[2] = WC(-1008.0 / 59.0) * t2 + WC(222176.0 / 1593.0) * t3 - WC(180032.0 / 531.0) * t4 +
               WC(876544.0 / 2655.0) * t5 - WC(180224.0 / 1593.0) * t6;
        w[3] = w[2];
        w[4] = WC(-378.0 / 59.0) * t2 + WC(27772.0 / 531.0) * t3 - WC(22504.0 / 177.0) * t4 +
               WC(109568.0 / 885.0) * t5 - WC(22528.0 / 531.0) * t6;
        w[5] = WC(-95232.0 / 413.0) * t2 + WC(62384128.0 / 33453.0) * t3 - WC(49429504.0 / 11151.0) * t4 +
               WC(46759936.0 / 11151.0) * t5 - WC(46661632.0 / 33453.0) * t6;
        w[6] = WC(896.0 / 5.0) * t2 - WC(4352.0 / 3.0) * t3 + WC(3456.0) * t4 - WC(16384.0 / 5.0) * t5 +
               WC(16384.0 / 15.0) * t6;
        w[7] = WC(50176.0 / 531.0) * t2 - WC(179554304.0 / 234171.0) * t3 + WC(143363072.0 / 78057.0) * t4 -
               WC(136675328.0 / 78057.0) * t5 + WC(137363456.0 / 234171.0) * t6;
        w[8] = WC(16384.0 / 441.0) * t3 - WC(16384.0 / 147.0) * t4 + WC(16384.0 / 147.0) * t5 - WC(16384.0 / 441.0) * t6;
        wp[0] = WC(1) - WC(28607.0 / 3717.0) * t - WC(166210.0 / 11151.0) * t2 + WC(1339120.0 / 11151.0) * t3 -
                WC(1911296.0 / 11151.0) * t4 + WC(813056.0 / 11151.0) * t5;
        wp[1] = WC(777.0 / 295.0) * t - WC(2534158.0 / 78057.0) * t2 + WC(8354320.0 / 78057.0) * t3 -
                WC(10479104.0 / 78057.0) * t4 + WC(22657024.0 / 390285.0) * t5;
        wp[2] = WC(-2016.0 / 59.0) * t + WC(222176.0 / 531.0) * t2 - WC(720128.0 / 531.0) * t3 +
                WC(876544.0 / 531.0) * t4 - WC(360448.0 / 531.0) * t5;
        wp[3] = wp[2];
        wp[4] = WC(-756.0 / 59.0) * t + WC(27772.0 / 177.0) * t2 - WC(90016.0 / 177.0) * t3 +
                WC(109568.0 / 177.0) * t4 - WC(45056.0 / 177.0) * t5;
        wp[5] = WC(-190464.0 / 413.0) * t + WC(62384128.0 / 11151.0) * t2 - WC(197718016.0 / 11151.0) * t3 +
                WC(233799680.0 / 11151.0) * t4 - WC(93323264.0 / 11151.0) * t5;
        wp[6] = WC(1792.0 / 5.0) * t - WC(4352.0) * t2 + WC(13824.0) * t3 - WC(16384.0) * t4 + WC(32768.0 / 5.0) * t5;
        wp[7] = WC(100352.0 / 531.0) * t - WC(179554304.0 / 78057.0) * t2 + WC(573452288.0 / 78057.0) * t3 -
                WC(683376640.0 / 78057.0) * t4 + WC(274726912.0 / 78057.0) * t5;
        wp[8] = WC(16384.0 / 147.0) * t2 - WC(65536.0 / 147.0) * t3 + WC(81920.0 / 147.0) * t4 - WC(32768.0 / 147.0) * t5;
    }
#undef WC
}

}  // namespace bvp
