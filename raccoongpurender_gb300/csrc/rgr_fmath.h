// rgr_fmath.h — deterministic single-precision math shared by host and device.
//
// The reference kernels call OpenCL built-ins (sin, cos, log, exp, atan, atan2,
// pow, normalize, dot, cross, mix, min, max) whose last-bit behaviour is
// implementation-defined.  This header fixes one definition of each so that the
// CUDA kernels (sm_103a) and the CPU oracle produce bit-identical per-path
// results.  Every function is built only from IEEE-754 single-precision
// +, -, *, /, sqrt, floor and rint (all correctly rounded on both sides) and
// must be compiled WITHOUT floating-point contraction:
//   nvcc --fmad=false          g++ -ffp-contract=off
//
// Methods (all published, coefficients derived here from the Taylor series):
//  * sin/cos: Cody & Waite argument reduction by pi/2 with a three-part split
//    constant (each part carries 12 significant bits so q*C1, q*C2 are exact
//    for |q| < 4096), then Taylor polynomials on [-pi/4, pi/4] (sin to r^9,
//    cos to r^10; truncation error < 0.03 ulp).
//  * log: x = 2^e * m, m in [sqrt(1/2), sqrt(2)), f = m - 1, s = f/(2+f),
//    log(1+f) = f - (hf - s*(hf + R(s^2))) with hf = f^2/2 and R the atanh
//    series 2/3 z + 2/5 z^2 + ... (Tang / fdlibm formulation); ln2 split in a
//    16-bit head and a tail.
//  * exp: k = rint(x/ln2), r = x - k*ln2 (two-part), Taylor to r^8, scaling by
//    2^k with an explicit two-step multiply for sub-normal results.
//  * atan: four-interval reduction atan(x) = atan(c) + atan((x-c)/(1+c*x)) for
//    c in {0, 1/2, 1, 3/2, inf}, Taylor series in u^2 on |u| <= 7/16.
//  * atan2: C99 Annex F special cases, quadrant fix-up with pi split hi+lo.
//  * pow: exp(y*log(x)) for x > 0, C99 special cases otherwise.  Error grows
//    like (1 + |y ln x|) ulp (OpenCL allows 16 ulp for pow).
// Accuracy against libm in double is checked by tests/test_fmath.py.
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define RGR_HD __host__ __device__ __forceinline__
#else
#define RGR_HD static inline
#endif

namespace rgr {
namespace fm {

RGR_HD uint32_t as_uint(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
RGR_HD float as_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
RGR_HD bool is_nan(float x) { return (as_uint(x) & 0x7fffffffu) > 0x7f800000u; }
RGR_HD bool is_inf(float x) { return (as_uint(x) & 0x7fffffffu) == 0x7f800000u; }
RGR_HD bool is_finite(float x) { return (as_uint(x) & 0x7f800000u) != 0x7f800000u; }
RGR_HD float fabs_(float x) { return as_float(as_uint(x) & 0x7fffffffu); }
RGR_HD float copysign_(float x, float s) {
    return as_float((as_uint(x) & 0x7fffffffu) | (as_uint(s) & 0x80000000u));
}
RGR_HD float rint_(float x) {
#if defined(__CUDA_ARCH__)
    return rintf(x);
#else
    // round half to even without depending on the host rounding mode
    float ax = fabs_(x);
    if (!(ax < 8388608.0f)) return x;  // already integral (or NaN/inf)
    float t = (ax + 8388608.0f) - 8388608.0f;
    return copysign_(t, x);
#endif
}
RGR_HD float floor_(float x) { return floorf(x); }
RGR_HD float sqrt_(float x) { return sqrtf(x); }

// OpenCL fmin/fmax semantics with a fixed rule for equal operands (returns x)
// so that the sign of a zero result is the same on host and device.
RGR_HD float fmin_(float x, float y) {
    if (is_nan(x)) return y;
    if (is_nan(y)) return x;
    return (y < x) ? y : x;
}
RGR_HD float fmax_(float x, float y) {
    if (is_nan(x)) return y;
    if (is_nan(y)) return x;
    return (x < y) ? y : x;
}
RGR_HD float clamp_(float x, float lo, float hi) { return fmin_(fmax_(x, lo), hi); }
// OpenCL mix(a, b, t) = a + (b - a) * t
RGR_HD float mix_(float a, float b, float t) { return a + (b - a) * t; }

// 2^k as a float for k in [-126, 127]
RGR_HD float pow2i(int k) { return as_float((uint32_t)(k + 127) << 23); }

// ---------------------------------------------------------------- sin / cos
RGR_HD void sincos_(float x, float* s_out, float* c_out) {
    if (!is_finite(x)) {
        float n = as_float(0x7fc00000u);
        *s_out = n;
        *c_out = n;
        return;
    }
    if (x == 0.0f) {  // keeps the sign of zero: sin(-0) = -0
        *s_out = x;
        *c_out = 1.0f;
        return;
    }
    const float kTwoOverPi = 0.636619747f;
    const float C1 = 1.57080078125f;            // 12 significant bits
    const float C2 = -4.45358455181121826e-06f; // 12 significant bits
    const float C3 = -8.70551575271605e-10f;
    float q, r;
    if (fabs_(x) < 6000.0f) {
        q = rint_(x * kTwoOverPi);
        r = ((x - q * C1) - q * C2) - q * C3;
    } else {
        // large arguments: reduce in double (IEEE on both sides), then round
        double xd = (double)x;
        double qd = rint(xd * 0.63661977236758134);
        double rd = (xd - qd * 1.5707963267948966) - qd * 6.123233995736766e-17;
        double q4 = qd - 4.0 * floor(qd * 0.25);  // qd mod 4, exact
        q = (float)q4;
        r = (float)rd;
    }
    float z = r * r;
    // sin(r) = r + r^3 * (-1/6 + z*(1/120 + z*(-1/5040 + z/362880)))
    float ps = -1.98412698e-04f + z * 2.75573192e-06f;
    ps = 8.33333377e-03f + z * ps;
    ps = -1.66666672e-01f + z * ps;
    float sr = r + (r * z) * ps;
    // cos(r) = 1 + z * (-1/2 + z*(1/24 + z*(-1/720 + z*(1/40320 - z/3628800))))
    float pc = 2.48015876e-05f + z * -2.75573188e-07f;
    pc = -1.38888892e-03f + z * pc;
    pc = 4.16666679e-02f + z * pc;
    float cr = (1.0f - 0.5f * z) + (z * z) * pc;
    int qi = (int)q & 3;
    float sv, cv;
    if (qi == 0) {
        sv = sr; cv = cr;
    } else if (qi == 1) {
        sv = cr; cv = -sr;
    } else if (qi == 2) {
        sv = -sr; cv = -cr;
    } else {
        sv = -cr; cv = sr;
    }
    *s_out = sv;
    *c_out = cv;
}
RGR_HD float sin_(float x) {
    float s, c;
    sincos_(x, &s, &c);
    return s;
}
RGR_HD float cos_(float x) {
    float s, c;
    sincos_(x, &s, &c);
    return c;
}

// ---------------------------------------------------------------- log
RGR_HD float log_(float x) {
    uint32_t ux = as_uint(x);
    if (is_nan(x)) return x;
    if ((ux & 0x7fffffffu) == 0) return as_float(0xff800000u);  // -inf
    if (ux & 0x80000000u) return as_float(0x7fc00000u);          // NaN
    if (ux == 0x7f800000u) return x;                              // +inf
    int e = 0;
    if (ux < 0x00800000u) {  // sub-normal: scale by 2^25
        x = x * 33554432.0f;
        ux = as_uint(x);
        e = -25;
    }
    e += (int)((ux >> 23) & 0xffu) - 127;
    uint32_t mb = (ux & 0x007fffffu) | 0x3f800000u;  // m in [1, 2)
    if (mb > 0x3fb504f3u) {                           // m > sqrt(2)
        mb -= 0x00800000u;                            // m *= 0.5
        e += 1;
    }
    float m = as_float(mb);
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float z = s * s;
    // R(z) = z*(2/3 + z*(2/5 + z*(2/7 + z*(2/9 + z*2/11))))
    float R = 0.222222224f + z * 0.181818187f;
    R = 0.285714298f + z * R;
    R = 0.400000006f + z * R;
    R = 0.666666687f + z * R;
    R = z * R;
    float hf = 0.5f * (f * f);
    float fe = (float)e;
    const float kLn2Hi = 0.693145751953125f;     // 16 significant bits
    const float kLn2Lo = 1.42860676533018e-06f;
    return fe * kLn2Hi - ((hf - (s * (hf + R) + fe * kLn2Lo)) - f);
}

// ---------------------------------------------------------------- exp
RGR_HD float exp_(float x) {
    if (is_nan(x)) return x;
    if (x > 88.7228394f) return as_float(0x7f800000u);
    if (x < -103.972084f) return 0.0f;
    const float kLog2e = 1.44269502f;
    const float kLn2Hi = 0.693145751953125f;
    const float kLn2Lo = 1.42860676533018e-06f;
    float k = rint_(x * kLog2e);
    float r = (x - k * kLn2Hi) - k * kLn2Lo;
    // Taylor to r^8
    float p = 2.48015876e-05f;                 // 1/40320
    p = 1.98412701e-04f + r * p;               // 1/5040
    p = 1.38888892e-03f + r * p;               // 1/720
    p = 8.33333377e-03f + r * p;               // 1/120
    p = 4.16666679e-02f + r * p;               // 1/24
    p = 1.66666672e-01f + r * p;               // 1/6
    p = 0.5f + r * p;
    p = 1.0f + r * p;
    p = 1.0f + r * p;
    int ki = (int)k;
    if (ki > 127) return (p * pow2i(127)) * pow2i(ki - 127);
    if (ki < -126) return (p * pow2i(ki + 64)) * pow2i(-64);
    return p * pow2i(ki);
}

// ---------------------------------------------------------------- atan
// Taylor series of atan on |u| <= 7/16 (terms to u^23)
RGR_HD float atan_poly(float u) {
    float w = u * u;
    float p = -4.34782617e-02f;        // -1/23
    p = 4.76190485e-02f + w * p;       //  1/21
    p = -5.26315793e-02f + w * p;      // -1/19
    p = 5.88235296e-02f + w * p;       //  1/17
    p = -6.66666701e-02f + w * p;      // -1/15
    p = 7.69230798e-02f + w * p;       //  1/13
    p = -9.09090936e-02f + w * p;      // -1/11
    p = 0.111111112f + w * p;          //  1/9
    p = -0.142857149f + w * p;         // -1/7
    p = 0.200000003f + w * p;          //  1/5
    p = -0.333333343f + w * p;         // -1/3
    return u + (u * w) * p;
}
RGR_HD float atan_(float x) {
    if (is_nan(x)) return x;
    float a = fabs_(x);
    float r;
    if (a <= 0.4375f) {
        r = atan_poly(a);
    } else if (a <= 0.6875f) {
        float u = (2.0f * a - 1.0f) / (2.0f + a);
        r = 0.463647604f + (5.01215869e-09f + atan_poly(u));
    } else if (a <= 1.1875f) {
        float u = (a - 1.0f) / (a + 1.0f);
        r = 0.785398185f + (-2.18556941e-08f + atan_poly(u));
    } else if (a <= 2.4375f) {
        float u = (a - 1.5f) / (1.0f + 1.5f * a);
        r = 0.982793748f + (-2.51314241e-08f + atan_poly(u));
    } else {
        float u = -1.0f / a;
        r = 1.57079637f + (-4.37113883e-08f + atan_poly(u));
    }
    return copysign_(r, x);
}

// ---------------------------------------------------------------- atan2
RGR_HD float atan2_(float y, float x) {
    const float kPi = 3.14159274f;
    const float kPiLo = -8.74227766e-08f;
    const float kPio2 = 1.57079637f;
    const float kPio4 = 0.785398185f;
    if (is_nan(x) || is_nan(y)) return x + y;
    bool xneg = (as_uint(x) & 0x80000000u) != 0;
    float ay = fabs_(y), ax = fabs_(x);
    float r;
    if (ay == 0.0f) {
        r = xneg ? kPi : 0.0f;
    } else if (ax == 0.0f) {
        r = kPio2;
    } else if (is_inf(ax) && is_inf(ay)) {
        r = xneg ? 2.35619450f : kPio4;
    } else if (is_inf(ax)) {
        r = xneg ? kPi : 0.0f;
    } else if (is_inf(ay)) {
        r = kPio2;
    } else {
        float t = ay / ax;
        float a = atan_(t);
        r = xneg ? (kPi - (a - kPiLo)) : a;
    }
    return copysign_(r, y);
}

// ---------------------------------------------------------------- pow
RGR_HD bool is_odd_integer(float y) {
    float ay = fabs_(y);
    if (!(ay < 16777216.0f)) return false;
    if (floor_(ay) != ay) return false;
    float h = ay * 0.5f;
    return floor_(h) != h;
}
RGR_HD float pow_(float x, float y) {
    if (y == 0.0f) return 1.0f;
    if (x == 1.0f) return 1.0f;
    if (is_nan(x) || is_nan(y)) return x + y;
    float ax = fabs_(x);
    bool yodd = is_odd_integer(y);
    if (ax == 0.0f) {
        if (y > 0.0f) return yodd ? x : 0.0f;
        return yodd ? copysign_(as_float(0x7f800000u), x) : as_float(0x7f800000u);
    }
    if (is_inf(y)) {
        if (ax == 1.0f) return 1.0f;
        bool big = ax > 1.0f;
        return (big == (y > 0.0f)) ? as_float(0x7f800000u) : 0.0f;
    }
    if (is_inf(x)) {
        float m = (y > 0.0f) ? as_float(0x7f800000u) : 0.0f;
        return (x < 0.0f && yodd) ? -m : m;
    }
    float sign = 1.0f;
    if (x < 0.0f) {
        if (floor_(y) != y) return as_float(0x7fc00000u);
        if (yodd) sign = -1.0f;
    }
    return sign * exp_(y * log_(ax));
}

}  // namespace fm
}  // namespace rgr
