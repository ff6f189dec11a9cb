// Wigner 3j symbol for the reference's basis-set setup (test infrastructure only).
//
// gsl_sf_coupling_3j takes doubled angular momenta (two_ja, ...), as GSL does.
// The value is computed from the Racah closed form
//   (j1 j2 j3; m1 m2 m3) = (-1)^(j1-j2-m3) sqrt(Delta(j1 j2 j3))
//     sqrt((j1+m1)!(j1-m1)!(j2+m2)!(j2-m2)!(j3+m3)!(j3-m3)!)
//     sum_k (-1)^k / [k!(j3-j2+k+m1)!(j3-j1+k-m2)!(j1+j2-j3-k)!(j1-k-m1)!(j2-k+m2)!]
// with Delta = (j1+j2-j3)!(j1-j2+j3)!(-j1+j2+j3)!/(j1+j2+j3+1)!.
#pragma once

#include <cmath>

inline double chiml_shim_fact(int n) {
    double r = 1.0;
    for (int i = 2; i <= n; ++i) r *= i;
    return r;
}

inline double gsl_sf_coupling_3j(int two_ja, int two_jb, int two_jc, int two_ma, int two_mb, int two_mc) {
    if ((two_ja + two_jb + two_jc) % 2 != 0) return 0.0;
    if (two_ma + two_mb + two_mc != 0) return 0.0;
    if (std::abs(two_ma) > two_ja || std::abs(two_mb) > two_jb || std::abs(two_mc) > two_jc) return 0.0;
    if ((two_ja + two_ma) % 2 || (two_jb + two_mb) % 2 || (two_jc + two_mc) % 2) return 0.0;
    if (two_jc > two_ja + two_jb || two_jc < std::abs(two_ja - two_jb)) return 0.0;
    const int j1 = two_ja, j2 = two_jb, j3 = two_jc, m1 = two_ma, m2 = two_mb, m3 = two_mc;
    // all quantities below are (doubled value)/2, exact integers by the checks above
    auto h = [](int twice) { return twice / 2; };
    const double tri = chiml_shim_fact(h(j1 + j2 - j3)) * chiml_shim_fact(h(j1 - j2 + j3)) *
                       chiml_shim_fact(h(-j1 + j2 + j3)) / chiml_shim_fact(h(j1 + j2 + j3) + 1);
    const double pre = std::sqrt(tri * chiml_shim_fact(h(j1 + m1)) * chiml_shim_fact(h(j1 - m1)) *
                                 chiml_shim_fact(h(j2 + m2)) * chiml_shim_fact(h(j2 - m2)) *
                                 chiml_shim_fact(h(j3 + m3)) * chiml_shim_fact(h(j3 - m3)));
    double sum = 0.0;
    for (int k = 0; k <= h(j1 + j2 + j3); ++k) {
        const int a = h(j3 - j2 + m1) + k, b = h(j3 - j1 - m2) + k, c = h(j1 + j2 - j3) - k;
        const int d = h(j1 - m1) - k, e = h(j2 + m2) - k;
        if (a < 0 || b < 0 || c < 0 || d < 0 || e < 0) continue;
        const double den = chiml_shim_fact(k) * chiml_shim_fact(a) * chiml_shim_fact(b) * chiml_shim_fact(c) *
                           chiml_shim_fact(d) * chiml_shim_fact(e);
        sum += ((k % 2) ? -1.0 : 1.0) / den;
    }
    const int phase = h(j1 - j2 - m3);
    return ((phase % 2) ? -1.0 : 1.0) * pre * sum;
}
