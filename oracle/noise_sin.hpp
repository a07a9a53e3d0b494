// noise_sin.hpp — TEST INFRASTRUCTURE ONLY.
//
// The FP32 sine of the force planes' noise edge offset (compute_delta.cl:158:
// sin(noisePos.x) + ...).  The reference builds with -cl-fast-relaxed-math,
// where sin's accuracy is implementation-defined, so the contract fixes one
// definition that host and device evaluate identically:
//   - Cody-Waite reduction x - k pi/2 with k = rint(x 2/pi), pi/2 split into
//     three parts (pi/2 cut to 8, then 12 significant bits, then the rest,
//     so k * part is exact for |k| < 2^12): W. J. Cody and W. Waite,
//     "Software Manual for the Elementary Functions", 1980;
//   - the Taylor polynomials of sin (to r^11) and cos (to r^10) on
//     [-pi/4, pi/4], Horner form, coefficients 1/n! rounded to float;
//   - |x| > 1e6 gives +-0, NaN stays NaN.
// Every step is one separately rounded IEEE FP32 operation (this file is
// compiled with -ffp-contract=off).  Used by the oracle and by the shimmed
// reference kernels.
#pragma once

#include <cmath>

inline float noise_sinf_ref(float x) {
    if (!(std::fabs(x) <= 1.0e6f)) return x * 0.0f;
    const float k = std::rint(x * 0x1.45f306p-1f);
    const float r = ((x - k * 0x1.92p+0f) - k * 0x1.fb4p-12f) - k * 0x1.4442d2p-24f;
    const float r2 = r * r;
    const float s = r + (r * r2) * (-0x1.555556p-3f + r2 * (0x1.111112p-7f + r2 * (-0x1.a01a02p-13f +
                    r2 * (0x1.71de3ap-19f + r2 * -0x1.ae6456p-26f))));
    const float c = 1.0f + r2 * (-0.5f + r2 * (0x1.555556p-5f + r2 * (-0x1.6c16c2p-10f +
                    r2 * (0x1.a01a02p-16f + r2 * -0x1.27e4fcp-22f))));
    const int q = (int)k & 3;
    const float v = (q & 1) ? c : s;
    return (q & 2) ? -v : v;
}
