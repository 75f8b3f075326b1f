/*
 * Deterministic FP64 helpers shared by the CUDA kernels and the CPU oracle.
 *
 * Library pow() and cos() differ between CUDA and host libm in the last bit,
 * and on trajectories that graze the clamped edge of a spline grid such a
 * last-bit difference in the DOP853 step-size factor is enough to flip an
 * accept/reject decision.  Everything here is built only from + - * / and
 * sqrt (all correctly rounded in IEEE arithmetic), so with FMA contraction
 * disabled it gives the same bits on the GPU and on the host.
 *
 *   nbcs_root8(x)     = x^(1/8) as sqrt(sqrt(sqrt(x)))        (<= ~1 ulp)
 *   nbcs_cos_deg(d)   = cos(d * pi / 180), d in degrees: exact reduction of
 *                       d to [0, 45] degrees, then the Taylor series of cos
 *                       or sin to degree 20 / 21 (truncation < 1e-23)
 */
#ifndef NBCS_DETMATH_H
#define NBCS_DETMATH_H

#include <math.h>

#ifdef __CUDACC__
#define NBCS_HD __host__ __device__ __forceinline__
#else
#define NBCS_HD static inline
#endif

NBCS_HD double nbcs_root8(double x) { return sqrt(sqrt(sqrt(x))); }

NBCS_HD float nbcs_root8f(float x) { return sqrtf(sqrtf(sqrtf(x))); }

/* Taylor series in x^2, Horner form, |x| <= pi/4 */
NBCS_HD double nbcs_cos_poly(double x)
{
    double z = x * x;
    double p = 1.0 / 2432902008176640000.0;        /* 1/20! */
    p = -1.0 / 6402373705728000.0 + z * p;         /* 1/18! */
    p = 1.0 / 20922789888000.0 + z * p;            /* 1/16! */
    p = -1.0 / 87178291200.0 + z * p;              /* 1/14! */
    p = 1.0 / 479001600.0 + z * p;                 /* 1/12! */
    p = -1.0 / 3628800.0 + z * p;                  /* 1/10! */
    p = 1.0 / 40320.0 + z * p;                     /* 1/8!  */
    p = -1.0 / 720.0 + z * p;                      /* 1/6!  */
    p = 1.0 / 24.0 + z * p;                        /* 1/4!  */
    p = -0.5 + z * p;                              /* 1/2!  */
    return 1.0 + z * p;
}

NBCS_HD double nbcs_sin_poly(double x)
{
    double z = x * x;
    double p = 1.0 / 51090942171709440000.0;       /* 1/21! */
    p = -1.0 / 121645100408832000.0 + z * p;       /* 1/19! */
    p = 1.0 / 355687428096000.0 + z * p;           /* 1/17! */
    p = -1.0 / 1307674368000.0 + z * p;            /* 1/15! */
    p = 1.0 / 6227020800.0 + z * p;                /* 1/13! */
    p = -1.0 / 39916800.0 + z * p;                 /* 1/11! */
    p = 1.0 / 362880.0 + z * p;                    /* 1/9!  */
    p = -1.0 / 5040.0 + z * p;                     /* 1/7!  */
    p = 1.0 / 120.0 + z * p;                       /* 1/5!  */
    p = -1.0 / 6.0 + z * p;                        /* 1/3!  */
    return x + x * (z * p);
}

NBCS_HD double nbcs_cos_deg(double d)
{
    const double rad = 3.141592653589793 / 180.0;
    double a = fabs(d);
    if (!(a <= 1.0e15)) return a == a ? 1.0 : a; /* huge: give up gracefully; NaN -> NaN */
    a = fmod(a, 360.0);                 /* exact */
    if (a > 180.0) a = 360.0 - a;       /* exact (Sterbenz) */
    double sgn = 1.0;
    if (a > 90.0) {
        a = 180.0 - a;                  /* exact */
        sgn = -1.0;
    }
    double r = (a <= 45.0) ? nbcs_cos_poly(a * rad) : nbcs_sin_poly((90.0 - a) * rad);
    return sgn * r;
}

#endif /* NBCS_DETMATH_H */
