/*
 * cg_math32.h -- deterministic single-precision sin, cos and acos.
 *
 * Used by the FP32-storage path for the rotation axes and angles of MC moves.
 * Every operation is an IEEE-754 binary32 add, multiply, divide, square root
 * or fused multiply-add, so the same source gives bit-identical results
 * compiled by nvcc for the GPU and by a C compiler for the host (with FMA
 * contraction off and no flush-to-zero).
 *
 * Method (textbook series, not any library's implementation):
 *   sin / cos: reduce x = k (pi/2) + r, |r| <= pi/4, with a three-part
 *     (Cody-Waite) split of pi/2 applied by fmaf; then the Taylor series
 *     sin r = sum (-1)^n r^(2n+1) / (2n+1)!  to r^11 and
 *     cos r = sum (-1)^n r^(2n) / (2n)!      to r^12
 *     (truncation below 2e-9 for |r| <= pi/4), and the quadrant k mod 4.
 *     Valid for |x| < 2^15.
 *   acos: for |x| <= 1/2, acos x = pi/2 - asin x with the Taylor series
 *     asin t = sum (2n)! / (4^n (n!)^2 (2n+1)) t^(2n+1) to t^23 (truncation
 *     below 3e-10); for |x| > 1/2 the half-angle identity
 *     acos x = 2 asin(sqrt((1 - x) / 2)), and acos(-x) = pi - acos(x).
 * Accuracy: a few ulp from the correctly rounded value (checked against libm
 * in the test suite).
 */
#ifndef CG_MATH32_H
#define CG_MATH32_H

#ifdef __CUDACC__
#define CGM_FN __host__ __device__ static inline
#else
#include <math.h>
#define CGM_FN static inline
#endif

/* pi/2 = C1 + C2 + C3; C1 has 8 significant bits, so k * C1 is exact */
#define CGM_PIO2_1 1.5703125f
#define CGM_PIO2_2 4.837512969970703125e-4f
#define CGM_PIO2_3 7.5497899548918821e-8f
#define CGM_2OPI 0.636619772367581343f
#define CGM_PIO2 1.57079632679489662f
#define CGM_PI 3.14159265358979324f

CGM_FN void cgm_sincosf(float x, float *s_out, float *c_out)
{
    float k = rintf(x * CGM_2OPI);
    float r = fmaf(-k, CGM_PIO2_1, x);
    r = fmaf(-k, CGM_PIO2_2, r);
    r = fmaf(-k, CGM_PIO2_3, r);
    float r2 = r * r;
    float ps = -2.5052107943679403e-08f;           /* -1/11! */
    ps = fmaf(ps, r2, 2.7557318844628753e-06f);    /*  1/9!  */
    ps = fmaf(ps, r2, -0.00019841270113829523f);   /* -1/7!  */
    ps = fmaf(ps, r2, 0.008333333767950535f);      /*  1/5!  */
    ps = fmaf(ps, r2, -0.1666666716337204f);       /* -1/3!  */
    float s = fmaf(r * r2, ps, r);
    float pc = 2.0876755879584152e-09f;            /*  1/12! */
    pc = fmaf(pc, r2, -2.755731998149713e-07f);    /* -1/10! */
    pc = fmaf(pc, r2, 2.4801587642286904e-05f);    /*  1/8!  */
    pc = fmaf(pc, r2, -0.0013888889225199819f);    /* -1/6!  */
    pc = fmaf(pc, r2, 0.0416666679084301f);        /*  1/4!  */
    pc = fmaf(pc, r2, -0.5f);                      /* -1/2!  */
    float c = fmaf(r2, pc, 1.0f);
    int q = ((int)k) & 3;
    if (q == 0) { *s_out = s; *c_out = c; }
    else if (q == 1) { *s_out = c; *c_out = -s; }
    else if (q == 2) { *s_out = -s; *c_out = -c; }
    else { *s_out = -c; *c_out = s; }
}

/* asin t for |t| <= 1/2 */
CGM_FN float cgm_asin_small(float t)
{
    float t2 = t * t;
    float p = 0.007312525995075703f;            /* n = 11 */
    p = fmaf(p, t2, 0.008390335366129875f);     /* n = 10 */
    p = fmaf(p, t2, 0.009761609137058258f);     /* n = 9  */
    p = fmaf(p, t2, 0.01155180111527443f);      /* n = 8  */
    p = fmaf(p, t2, 0.013964843936264515f);     /* n = 7  */
    p = fmaf(p, t2, 0.017352763563394547f);     /* n = 6  */
    p = fmaf(p, t2, 0.022372158244252205f);     /* n = 5  */
    p = fmaf(p, t2, 0.0303819440305233f);       /* n = 4  */
    p = fmaf(p, t2, 0.0446428582072258f);       /* n = 3  */
    p = fmaf(p, t2, 0.07500000298023224f);      /* n = 2  */
    p = fmaf(p, t2, 0.1666666716337204f);       /* n = 1  */
    return fmaf(t * t2, p, t);
}

CGM_FN float cgm_acosf(float x)
{
    if (x > 1.0f) x = 1.0f;
    if (x < -1.0f) x = -1.0f;
    float ax = fabsf(x);
    if (ax <= 0.5f) return CGM_PIO2 - cgm_asin_small(x);
    float h = 2.0f * cgm_asin_small(sqrtf((1.0f - ax) * 0.5f));
    return x > 0.0f ? h : CGM_PI - h;
}

/* 24-bit uniform in [0, 1) from a 31-bit draw (exact in binary32) */
CGM_FN float cgm_unif24(unsigned x) { return (float)(x >> 7) * 5.9604644775390625e-08f; }

/*
 * round(w * 2^40), ties to even, for 0 <= w <= 1: the fixed-point value of a
 * trilinear weight, with 32-bit conversions only (a conversion of a float to
 * a 64-bit integer runs at the FP64 rate on GB300).  a = w * 2^30 is exact;
 * w * 2^40 = floor(a) * 2^10 + f * 2^10 with f = a - floor(a) exact (Sterbenz
 * for a >= 1, f = a below), and floor(a) * 2^10 is even, so rounding f * 2^10
 * (exact: a power-of-two scaling of a number below 1) to nearest-even rounds
 * the whole.  Equals llrint((double)w * 2^40) for every binary32 w in [0, 1]
 * (checked exhaustively in the test suite).
 */
CGM_FN long long cgm_q40f(float w)
{
    float a = w * 1073741824.0f;
    float fl = floorf(a);
    float fr = (a - fl) * 1024.0f;
    return (long long)(int)fl * 1024LL + (long long)(int)rintf(fr);
}

#endif /* CG_MATH32_H */
