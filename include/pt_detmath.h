/*
 * pt_detmath.h -- deterministic power function for the integrator's step-size
 * control, shared by the CUDA kernels and the CPU oracle.
 *
 * odeint's step adjuster scales the step by 0.9 * err^(-1/3) on rejection and
 * 0.9 * max(err, 5^-5)^(-1/5) on growth.  Library pow() differs between the
 * host libm and the device by up to an ulp, and the reference algorithm
 * amplifies one-ulp step-size differences (cancellation in the embedded error
 * estimate, then 1e-8 m bisection brackets that shift with the step grid) to
 * ~1e-7 m end-state differences.  This file therefore defines x^p from IEEE
 * basic operations only (add, sub, mul, div, exact power-of-two scaling), so
 * host and device produce identical bits:
 *   ln(x):  x = 2^k m with m in [1/sqrt(2), sqrt(2)), s = (m-1)/(m+1),
 *           ln m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...)   (|s| < 0.172)
 *   exp(y): y = j ln2 + r, |r| <= ln2/2, exp(r) by its Taylor series
 *           in Horner form, times 2^j.
 * Relative error against the library pow (tests/test_detmath.py): below
 * 1e-15 where the step adjuster uses the result (err in [5^-5, 91]: above
 * (0.9/0.2)^3 the shrink factor is clamped at 0.2), below 1e-13 on
 * [1e-300, 1e300], where the rounding of ln 2 times the binary exponent
 * dominates.
 */
#ifndef PT_DETMATH_H
#define PT_DETMATH_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define PTDM_FN __host__ __device__ __forceinline__
#else
#define PTDM_FN static inline
#endif

PTDM_FN double ptdm_mul(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
PTDM_FN double ptdm_add(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
PTDM_FN double ptdm_sub(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
PTDM_FN double ptdm_div(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}
PTDM_FN uint64_t ptdm_bits(double x) {
    uint64_t u;
    memcpy(&u, &x, sizeof(u));
    return u;
}
PTDM_FN double ptdm_from_bits(uint64_t u) {
    double x;
    memcpy(&x, &u, sizeof(x));
    return x;
}

/* natural log of a positive, finite, normal x */
PTDM_FN double ptdm_log(double x) {
    const double LN2_HI = 0.6931471805599453094; /* rounded ln 2 */
    uint64_t u = ptdm_bits(x);
    int k = (int)((u >> 52) & 0x7ff) - 1023;
    double m = ptdm_from_bits((u & 0x000fffffffffffffull) | 0x3ff0000000000000ull); /* [1, 2) */
    if (m > 1.4142135623730951) {
        m = ptdm_mul(m, 0.5);
        k += 1;
    }
    double s = ptdm_div(ptdm_sub(m, 1.0), ptdm_add(m, 1.0));
    double s2 = ptdm_mul(s, s);
    /* 2 * (s + s^3/3 + ... + s^23/23), Horner in s^2 */
    double p = 1.0 / 23;
    p = ptdm_add(ptdm_mul(p, s2), 1.0 / 21);
    p = ptdm_add(ptdm_mul(p, s2), 1.0 / 19);
    p = ptdm_add(ptdm_mul(p, s2), 1.0 / 17);
    p = ptdm_add(ptdm_mul(p, s2), 1.0 / 15);
    p = ptdm_add(ptdm_mul(p, s2), 1.0 / 13);
    p = ptdm_add(ptdm_mul(p, s2), 1.0 / 11);
    p = ptdm_add(ptdm_mul(p, s2), 1.0 / 9);
    p = ptdm_add(ptdm_mul(p, s2), 1.0 / 7);
    p = ptdm_add(ptdm_mul(p, s2), 1.0 / 5);
    p = ptdm_add(ptdm_mul(p, s2), 1.0 / 3);
    p = ptdm_add(ptdm_mul(p, s2), 1.0);
    double lnm = ptdm_mul(2.0, ptdm_mul(s, p));
    return ptdm_add(ptdm_mul((double)k, LN2_HI), lnm);
}

/* exp(y) for |y| < 700 */
PTDM_FN double ptdm_exp(double y) {
    const double LN2 = 0.6931471805599453094, INV_LN2 = 1.4426950408889634074;
    double jf = ptdm_mul(y, INV_LN2);
    int j = (int)(jf >= 0 ? jf + 0.5 : jf - 0.5);
    double r = ptdm_sub(y, ptdm_mul((double)j, LN2));
    /* Taylor series of exp(r), |r| <= 0.35: terms to r^18/18! */
    double q = 1.0 / 6402373705728000.0; /* 1/18! */
    const double inv[18] = {1.0 / 355687428096000.0, 1.0 / 20922789888000.0, 1.0 / 1307674368000.0, 1.0 / 87178291200.0,
                            1.0 / 6227020800.0, 1.0 / 479001600.0, 1.0 / 39916800.0, 1.0 / 3628800.0, 1.0 / 362880.0,
                            1.0 / 40320.0, 1.0 / 5040.0, 1.0 / 720.0, 1.0 / 120.0, 1.0 / 24.0, 1.0 / 6.0, 0.5, 1.0, 1.0};
    for (int i = 0; i < 18; ++i) q = ptdm_add(ptdm_mul(q, r), inv[i]);
    /* scale by 2^j exactly (j in the normal range for |y| < 700) */
    uint64_t e = (uint64_t)(j + 1023) << 52;
    return ptdm_mul(q, ptdm_from_bits(e));
}

/* x^p for x > 0 normal, |p ln x| < 700 */
PTDM_FN double ptdm_pow(double x, double p) { return ptdm_exp(ptdm_mul(p, ptdm_log(x))); }

#endif /* PT_DETMATH_H */
