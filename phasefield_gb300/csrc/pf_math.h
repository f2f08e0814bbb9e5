/* pf_math.h -- exp and log that round identically on the host and the GPU.
 *
 * The solute-drag velocity of the Fortran model is found by a bisection whose
 * stopping point depends on every bit of exp and log; the host oracle and the
 * GPU kernel must therefore evaluate the same functions.  These are written
 * from the mathematics with +, -, *, / and the exact frexp/ldexp only, so a
 * build without multiply-add contraction (-fmad=false on the device,
 * -ffp-contract=off on the host) gives the same bits on both:
 *   exp: x = k ln2 + r with |r| <= ln2/2 (ln2 split into a 33-bit head and a
 *        tail, so k*head is exact -- the Cody-Waite reduction), e^r by its
 *        Taylor series to degree 13 (truncation below 1e-17), times 2^k.
 *   log: x = m 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s) with
 *        s = (m-1)/(m+1), |s| <= 0.172, by its series to s^23.
 * Both are within a few ulp of the correctly rounded values (checked against
 * the C library in the tests).  C and C++ (host and device) alike. */
#ifndef PF_MATH_H
#define PF_MATH_H
#include <math.h>

#if defined(__CUDACC__)
#define PF_MATH_FN static __host__ __device__ __forceinline__
#else
#define PF_MATH_FN static inline
#endif

#define PF_LN2_HI 0.6931471806019545        /* ln 2 rounded to a multiple of 2^-32 */
#define PF_LN2_LO (-4.2009150726810846e-11) /* ln 2 - PF_LN2_HI */
#define PF_INV_LN2 1.4426950408889634

PF_MATH_FN double pf_exp(double x) {
    if (x != x) return x;
    if (x > 709.78) return HUGE_VAL;
    if (x < -745.2) return 0.0;
    const double kd = floor(x * PF_INV_LN2 + 0.5);
    const int k = (int)kd;
    const double r = (x - kd * PF_LN2_HI) - kd * PF_LN2_LO;
    double p = 1.6059043836821613e-10;  /* 1/13! */
    p = p * r + 2.08767569878681e-09;   /* 1/12! */
    p = p * r + 2.505210838544172e-08;
    p = p * r + 2.755731922398589e-07;
    p = p * r + 2.7557319223985893e-06;
    p = p * r + 2.48015873015873e-05;
    p = p * r + 0.0001984126984126984;
    p = p * r + 0.001388888888888889;
    p = p * r + 0.008333333333333333;
    p = p * r + 0.041666666666666664;
    p = p * r + 0.16666666666666666;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    return ldexp(p, k);
}

PF_MATH_FN double pf_log(double x) {
    if (x != x || x < 0.0) return NAN;
    if (x == 0.0) return -HUGE_VAL;
    if (x == HUGE_VAL) return x;
    int e;
    double m = frexp(x, &e); /* m in [0.5, 1) */
    if (m < 0.7071067811865476) {
        m = m * 2.0;
        e = e - 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double q = 1.0 / 23.0;
    q = q * s2 + 1.0 / 21.0;
    q = q * s2 + 1.0 / 19.0;
    q = q * s2 + 1.0 / 17.0;
    q = q * s2 + 1.0 / 15.0;
    q = q * s2 + 1.0 / 13.0;
    q = q * s2 + 1.0 / 11.0;
    q = q * s2 + 1.0 / 9.0;
    q = q * s2 + 1.0 / 7.0;
    q = q * s2 + 1.0 / 5.0;
    q = q * s2 + 1.0 / 3.0;
    q = q * s2 + 1.0;
    const double lm = 2.0 * s * q;
    const double ed = (double)e;
    return ed * PF_LN2_HI + (ed * PF_LN2_LO + lm);
}

#endif
