/*
 * yapt_fmath.h -- deterministic single-precision elementary functions.
 *
 * The spectral path tracer must give the same per-sample radiance on the GPU and
 * in any host code that reproduces it. IEEE-754 add/sub/mul/div/sqrt/fma are
 * correctly rounded on both sides (device code is compiled with -fmad=false
 * -prec-div=true -prec-sqrt=true -ftz=false, host code with -ffp-contract=off),
 * but vendor sin/cos/exp/log/pow are not specified bit-for-bit. These functions
 * are built only from correctly rounded operations, so they return identical
 * bits wherever they are compiled.
 *
 * Methods (published, restated here from the mathematics):
 *  - argument reduction: Cody & Waite, "Software Manual for the Elementary
 *    Functions" (1980): x = k*C + r with C split into exactly representable parts;
 *  - sin/cos/exp kernels: truncated Taylor series with exact rational coefficients
 *    1/n!, evaluated by Horner's rule with fused multiply-add;
 *  - log kernel: log(m) = 2*atanh(s), s = (m-1)/(m+1), truncated odd series.
 * Accuracy (measured against float64 references, tests/test_fmath_cpu.py): sin and cos within
 * 1e-7 absolute for |x| < 2^10 (2 ulp on [-pi, pi]); exp within 1 ulp on [-87, 88]; log within
 * 2 ulp on [1e-30, 1e30] (1e-9 absolute where |log x| < 1e-3); pow, computed as exp(y log x) in
 * single precision, within 2 + 2 |y ln x| ulp. They are not correctly rounded and are not meant to replace libm
 * elsewhere.
 */
#ifndef YAPT_FMATH_H
#define YAPT_FMATH_H

#if defined(__CUDACC__)
#define YGM_FN static __host__ __device__ __forceinline__
#include <cuda_runtime.h>
#else
#define YGM_FN static inline
#include <math.h>
#endif

/* 2/pi, and pi/2 split into three floats (12 + 12 significant bits, then the rest):
 * k*PIO2_1 and k*PIO2_2 are exact for |k| < 2^12 */
#define YGM_TWO_OVER_PI 0.636619772367581343f
#define YGM_PIO2_1 1.5703125f
#define YGM_PIO2_2 4.837512969970703125e-04f
#define YGM_PIO2_3 7.549790126404332e-08f
/* log2(e) and ln(2) split: hi has 16 significant bits so k*hi is exact */
#define YGM_LOG2E 1.44269504088896341f
#define YGM_LN2_HI 0.693145751953125f
#define YGM_LN2_LO 1.428606765330187e-06f

YGM_FN float ygm_rint(float x)
{
    /* round half away from zero on a float that fits an int */
    return (x >= 0.0f) ? floorf(x + 0.5f) : -floorf(-x + 0.5f);
}

/* sin(r), cos(r) on |r| <= pi/4 (Taylor to r^11 / r^12) */
YGM_FN float ygm_sin_kernel(float r)
{
    float r2 = r * r;
    float p = -2.50521083854417188e-08f;       /* -1/11! */
    p = fmaf(p, r2, 2.75573192239858907e-06f);  /*  1/9!  */
    p = fmaf(p, r2, -1.98412698412698413e-04f); /* -1/7!  */
    p = fmaf(p, r2, 8.33333333333333333e-03f);  /*  1/5!  */
    p = fmaf(p, r2, -1.66666666666666667e-01f); /* -1/3!  */
    return fmaf(p * r2, r, r);
}

YGM_FN float ygm_cos_kernel(float r)
{
    float r2 = r * r;
    float p = 2.08767569878680990e-09f;         /*  1/12! */
    p = fmaf(p, r2, -2.75573192239858907e-07f); /* -1/10! */
    p = fmaf(p, r2, 2.48015873015873016e-05f);  /*  1/8!  */
    p = fmaf(p, r2, -1.38888888888888889e-03f); /* -1/6!  */
    p = fmaf(p, r2, 4.16666666666666667e-02f);  /*  1/4!  */
    p = fmaf(p, r2, -0.5f);
    return fmaf(p, r2, 1.0f);
}

YGM_FN void ygm_sincosf(float x, float* s, float* c)
{
    float k = ygm_rint(x * YGM_TWO_OVER_PI);
    float r = fmaf(-k, YGM_PIO2_1, x);
    r = fmaf(-k, YGM_PIO2_2, r);
    r = fmaf(-k, YGM_PIO2_3, r);
    float sr = ygm_sin_kernel(r);
    float cr = ygm_cos_kernel(r);
    int q = ((int)k) & 3;
    switch (q)
    {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
    }
}

YGM_FN float ygm_sinf(float x) { float s, c; ygm_sincosf(x, &s, &c); return s; }
YGM_FN float ygm_cosf(float x) { float s, c; ygm_sincosf(x, &s, &c); return c; }

/* exp(x): x = k ln2 + r, |r| <= ln2/2, Taylor to r^8 */
YGM_FN float ygm_expf(float x)
{
    if (x != x) return x;
    if (x > 88.72283905206835f) return 1.0f / 0.0f;
    if (x < -103.972077083991796f) return 0.0f;
    float k = ygm_rint(x * YGM_LOG2E);
    float r = fmaf(-k, YGM_LN2_HI, x);
    r = fmaf(-k, YGM_LN2_LO, r);
    float p = 2.48015873015873016e-05f;         /* 1/8! */
    p = fmaf(p, r, 1.98412698412698413e-04f);   /* 1/7! */
    p = fmaf(p, r, 1.38888888888888889e-03f);   /* 1/6! */
    p = fmaf(p, r, 8.33333333333333333e-03f);   /* 1/5! */
    p = fmaf(p, r, 4.16666666666666667e-02f);   /* 1/4! */
    p = fmaf(p, r, 1.66666666666666667e-01f);   /* 1/3! */
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    /* scale by 2^k in two exact steps so that subnormal results are handled */
    int ki = (int)k;
    int k1 = ki / 2;
    return ldexpf(ldexpf(p, k1), ki - k1);
}

/* log(x) for x > 0: x = m 2^e, m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s) */
YGM_FN float ygm_logf(float x)
{
    if (x != x || x < 0.0f) return 0.0f / 0.0f;
    if (x == 0.0f) return -1.0f / 0.0f;
    if (x == 1.0f / 0.0f) return x;
    int e;
    float m = frexpf(x, &e); /* m in [0.5, 1) */
    if (m < 0.70710678118654752f)
    {
        m = m * 2.0f;
        e -= 1;
    }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = 7.69230769230769231e-02f;        /* 1/13 */
    p = fmaf(p, s2, 9.09090909090909091e-02f); /* 1/11 */
    p = fmaf(p, s2, 1.11111111111111111e-01f); /* 1/9  */
    p = fmaf(p, s2, 1.42857142857142857e-01f); /* 1/7  */
    p = fmaf(p, s2, 2.0e-01f);                 /* 1/5  */
    p = fmaf(p, s2, 3.33333333333333333e-01f); /* 1/3  */
    float logm = 2.0f * fmaf(p * s2, s, s);
    float fe = (float)e;
    return fmaf(fe, YGM_LN2_HI, fmaf(fe, YGM_LN2_LO, logm));
}

/* pow(x, y) for x >= 0 as exp(y log x); the tracer never raises negative bases */
YGM_FN float ygm_powf(float x, float y)
{
    if (y == 0.0f) return 1.0f;
    if (x == 1.0f) return 1.0f;
    if (x == 0.0f) return (y > 0.0f) ? 0.0f : 1.0f / 0.0f;
    if (x < 0.0f) return 0.0f / 0.0f;
    return ygm_expf(y * ygm_logf(x));
}

#endif /* YAPT_FMATH_H */
