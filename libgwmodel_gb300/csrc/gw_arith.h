/*
 * gw_arith.h -- portable FP64 arithmetic shared by the CUDA kernels and by
 * the CPU oracle, so that both evaluate distances and kernel weights with
 * the SAME sequence of correctly rounded operations (+ - * / sqrt fma).
 *
 * Why: the reference computes great-circle distances with the platform
 * libm (CRSDistance.cpp:15-69).  CUDA's device sin/cos/atan and glibc's
 * differ in the last ulp, so a GPU distance computed with CUDA's libm can
 * never be bit-identical to a CPU one.  Adaptive bandwidths pick the b-th
 * smallest distance, and a one-ulp difference can change the neighbour set
 * at a tie.  The sin/cos/atan below are written from their Taylor series
 * (coefficients are the exact rationals (-1)^k/(2k+1)! etc. rounded to
 * double) with Cody-Waite reduction by pi/2, so host and device agree to
 * the bit.  They agree with glibc to a few ulp (tested on the CPU).
 *
 * Planar distance (CRSDistance.h:95-99) and the five kernel functions
 * (BandwidthWeight.h:68-121) are written with the reference's operation
 * order and no fused multiply-add, so they reproduce the reference's
 * doubles exactly.
 *
 * Compile host users with -ffp-contract=off.  Device code uses the _rn
 * intrinsics, which nvcc never contracts.
 */
#ifndef GW_ARITH_H
#define GW_ARITH_H

#include <math.h>

#if defined(__CUDACC__)
#define GW_HD __host__ __device__ __forceinline__
#else
#define GW_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define GW_MUL(a, b) __dmul_rn((a), (b))
#define GW_ADD(a, b) __dadd_rn((a), (b))
#define GW_SUB(a, b) __dsub_rn((a), (b))
#define GW_DIV(a, b) __ddiv_rn((a), (b))
#define GW_SQRT(a) __dsqrt_rn(a)
#define GW_FMA(a, b, c) __fma_rn((a), (b), (c))
#define GW_RINT(a) rint(a)
#else
#define GW_MUL(a, b) ((a) * (b))
#define GW_ADD(a, b) ((a) + (b))
#define GW_SUB(a, b) ((a) - (b))
#define GW_DIV(a, b) ((a) / (b))
#define GW_SQRT(a) sqrt(a)
#define GW_FMA(a, b, c) fma((a), (b), (c))
#define GW_RINT(a) nearbyint(a)
#endif

/* Kernel function ids: BandwidthWeight::KernelFunctionType (BandwidthWeight.h:46-53). */
#define GW_KERNEL_GAUSSIAN 0
#define GW_KERNEL_EXPONENTIAL 1
#define GW_KERNEL_BISQUARE 2
#define GW_KERNEL_TRICUBE 3
#define GW_KERNEL_BOXCAR 4

/* DOUBLE_EPS compile definition of the reference (src/CMakeLists.txt:33-36). */
#define GW_DOUBLE_EPS 1e-8

/* pi/2 split for Cody-Waite reduction: P1 and P2 carry 33 significant bits,
 * so k*P1 and k*P2 are exact for |k| < 2^20. */
#define GW_PIO2_1 0x1.921fb54400000p+0
#define GW_PIO2_2 0x1.0b4611a600000p-34
#define GW_PIO2_3 0x1.3198a2e037073p-69
#define GW_PIO2_HI 0x1.921fb54442d18p+0
#define GW_PIO2_LO 0x1.1a62633145c07p-54
#define GW_TWO_OVER_PI 0x1.45f306dc9c883p-1

/* sin and cos of r, |r| <= pi/4, by Taylor series to r^19 / r^20. */
GW_HD void gw_sincos_reduced(double r, double* s, double* c)
{
    double z = GW_MUL(r, r);
    double ps = -0x1.2f49b46814157p-57;            /* -1/19! */
    ps = GW_FMA(ps, z, 0x1.952c77030ad4ap-49);     /*  1/17! */
    ps = GW_FMA(ps, z, -0x1.ae7f3e733b81fp-41);    /* -1/15! */
    ps = GW_FMA(ps, z, 0x1.6124613a86d09p-33);     /*  1/13! */
    ps = GW_FMA(ps, z, -0x1.ae64567f544e4p-26);    /* -1/11! */
    ps = GW_FMA(ps, z, 0x1.71de3a556c734p-19);     /*  1/9!  */
    ps = GW_FMA(ps, z, -0x1.a01a01a01a01ap-13);    /* -1/7!  */
    ps = GW_FMA(ps, z, 0x1.1111111111111p-7);      /*  1/5!  */
    ps = GW_FMA(ps, z, -0x1.5555555555555p-3);     /* -1/3!  */
    *s = GW_FMA(GW_MUL(r, z), ps, r);
    double pc = 0x1.e542ba4020225p-62;             /*  1/20! */
    pc = GW_FMA(pc, z, -0x1.6827863b97d97p-53);    /* -1/18! */
    pc = GW_FMA(pc, z, 0x1.ae7f3e733b81fp-45);     /*  1/16! */
    pc = GW_FMA(pc, z, -0x1.93974a8c07c9dp-37);    /* -1/14! */
    pc = GW_FMA(pc, z, 0x1.1eed8eff8d898p-29);     /*  1/12! */
    pc = GW_FMA(pc, z, -0x1.27e4fb7789f5cp-22);    /* -1/10! */
    pc = GW_FMA(pc, z, 0x1.a01a01a01a01ap-16);     /*  1/8!  */
    pc = GW_FMA(pc, z, -0x1.6c16c16c16c17p-10);    /* -1/6!  */
    pc = GW_FMA(pc, z, 0x1.5555555555555p-5);      /*  1/4!  */
    pc = GW_FMA(pc, z, -0.5);                      /* -1/2!  */
    *c = GW_FMA(z, pc, 1.0);
}

/* sin and cos of x for |x| < 2^19 * pi/2: Cody-Waite reduction, quadrant select. */
GW_HD void gw_sincos(double x, double* s, double* c)
{
    double k = GW_RINT(GW_MUL(x, GW_TWO_OVER_PI));
    double r = GW_FMA(-k, GW_PIO2_1, x);
    r = GW_FMA(-k, GW_PIO2_2, r);
    r = GW_FMA(-k, GW_PIO2_3, r);
    double sr, cr;
    gw_sincos_reduced(r, &sr, &cr);
    long long q = (long long)k & 3;
    if (q == 0) { *s = sr; *c = cr; }
    else if (q == 1) { *s = cr; *c = -sr; }
    else if (q == 2) { *s = -sr; *c = -cr; }
    else { *s = -cr; *c = sr; }
}

/* atan(x) for x >= 0 (NaN propagates, +inf gives pi/2).  Two half-angle
 * reductions atan(t) = 2 atan(t / (1 + sqrt(1 + t^2))) bring t below
 * tan(pi/16) ~ 0.199, where the alternating series to t^25 is below 1e-18. */
GW_HD double gw_atan_nonneg(double x)
{
    int inv = x > 1.0;
    double t = inv ? GW_DIV(1.0, x) : x;
    t = GW_DIV(t, GW_ADD(1.0, GW_SQRT(GW_FMA(t, t, 1.0))));
    t = GW_DIV(t, GW_ADD(1.0, GW_SQRT(GW_FMA(t, t, 1.0))));
    double z = GW_MUL(t, t);
    double p = 0x1.47ae147ae147bp-5;             /*  1/25 */
    p = GW_FMA(p, z, -0x1.642c8590b2164p-5);     /* -1/23 */
    p = GW_FMA(p, z, 0x1.8618618618618p-5);      /*  1/21 */
    p = GW_FMA(p, z, -0x1.af286bca1af28p-5);     /* -1/19 */
    p = GW_FMA(p, z, 0x1.e1e1e1e1e1e1ep-5);      /*  1/17 */
    p = GW_FMA(p, z, -0x1.1111111111111p-4);     /* -1/15 */
    p = GW_FMA(p, z, 0x1.3b13b13b13b14p-4);      /*  1/13 */
    p = GW_FMA(p, z, -0x1.745d1745d1746p-4);     /* -1/11 */
    p = GW_FMA(p, z, 0x1.c71c71c71c71cp-4);      /*  1/9  */
    p = GW_FMA(p, z, -0x1.2492492492492p-3);     /* -1/7  */
    p = GW_FMA(p, z, 0x1.999999999999ap-3);      /*  1/5  */
    p = GW_FMA(p, z, -0x1.5555555555555p-2);     /* -1/3  */
    double a = GW_MUL(4.0, GW_FMA(GW_MUL(t, z), p, t));
    if (inv) a = GW_ADD(GW_SUB(GW_PIO2_HI, a), GW_PIO2_LO);
    return a;
}

/* Planar distance, CRSDistance::EuclideanDistance (CRSDistance.h:95-99):
 * diff = data - focus, sqrt(dx*dx + dy*dy), no contraction. */
GW_HD double gw_planar_dist(double ud, double vd, double uf, double vf)
{
    double dx = GW_SUB(ud, uf), dy = GW_SUB(vd, vf);
    return GW_SQRT(GW_ADD(GW_MUL(dx, dx), GW_MUL(dy, dy)));
}

/* Great-circle (ellipsoidal, WGS-84) distance in km, CRSDistance::SpGcdist
 * (CRSDistance.cpp:15-69), with argument order (lon1, lon2, lat1, lat2) and
 * the reference's operation order.  lonR/latR are lon*(M_PI/180) and
 * lat*(M_PI/180) precomputed per point exactly as the reference rounds them
 * (DE2RA = M_PI / 180; lat1R = lat1 * DE2RA). */
GW_HD double gw_gc_dist(double lon1, double lon2, double lat1, double lat2,
                        double lon1R, double lon2R, double lat1R, double lat2R)
{
    const double a = 6378.137;
    const double f = 1.0 / 298.257223563;
    if (fabs(GW_SUB(lat1, lat2)) < GW_DOUBLE_EPS)
    {
        if (fabs(GW_SUB(lon1, lon2)) < GW_DOUBLE_EPS)
            return 0.0;
        else if (fabs(GW_SUB(GW_ADD(fabs(lon1), fabs(lon2)), 360.0)) < GW_DOUBLE_EPS)
            return 0.0;
    }
    double F = GW_DIV(GW_ADD(lat1R, lat2R), 2.0);
    double G = GW_DIV(GW_SUB(lat1R, lat2R), 2.0);
    double L = GW_DIV(GW_SUB(lon1R, lon2R), 2.0);
    double sF, cF, sG, cG, sL, cL;
    gw_sincos(F, &sF, &cF);
    gw_sincos(G, &sG, &cG);
    gw_sincos(L, &sL, &cL);
    double sinG2 = GW_MUL(sG, sG), cosG2 = GW_MUL(cG, cG);
    double sinF2 = GW_MUL(sF, sF), cosF2 = GW_MUL(cF, cF);
    double sinL2 = GW_MUL(sL, sL), cosL2 = GW_MUL(cL, cL);
    double S = GW_ADD(GW_MUL(sinG2, cosL2), GW_MUL(cosF2, sinL2));
    double C = GW_ADD(GW_MUL(cosG2, cosL2), GW_MUL(sinF2, sinL2));
    double w = gw_atan_nonneg(GW_SQRT(GW_DIV(S, C)));
    double R = GW_DIV(GW_SQRT(GW_MUL(S, C)), w);
    double D = GW_MUL(GW_MUL(2.0, w), a);
    double H1 = GW_DIV(GW_SUB(GW_MUL(3.0, R), 1.0), GW_MUL(2.0, C));
    double H2 = GW_DIV(GW_ADD(GW_MUL(3.0, R), 1.0), GW_MUL(2.0, S));
    double t1 = GW_MUL(GW_MUL(GW_MUL(f, H1), sinF2), cosG2);
    double t2 = GW_MUL(GW_MUL(GW_MUL(f, H2), cosF2), sinG2);
    return GW_MUL(D, GW_SUB(GW_ADD(1.0, t1), t2));
}

/* Kernel functions, BandwidthWeight.h:68-121, element by element with the
 * reference's operation order.  The indicator (d < bw) multiplies the
 * polynomial as a double 0/1, as Armadillo's mixed-type product does, so a
 * zero bandwidth yields NaN exactly where the reference does.  The reference evaluates exp with libm; the
 * device uses CUDA's exp (within 1 ulp), so gaussian/exponential weights are
 * parity-tested to a tolerance while the compactly supported kernels are
 * bit-exact. */
GW_HD double gw_kernel_weight(int kernel, double d, double bw)
{
    switch (kernel)
    {
    case GW_KERNEL_GAUSSIAN:
        return exp(GW_DIV(GW_MUL(d, d), GW_MUL(-2.0, GW_MUL(bw, bw))));
    case GW_KERNEL_EXPONENTIAL:
        return exp(GW_DIV(-d, bw));
    case GW_KERNEL_BISQUARE:
    {
        double t = GW_SUB(1.0, GW_DIV(GW_MUL(d, d), GW_MUL(bw, bw)));
        return GW_MUL(d < bw ? 1.0 : 0.0, GW_MUL(t, t));
    }
    case GW_KERNEL_TRICUBE:
    {
        double t = GW_SUB(1.0, GW_DIV(GW_MUL(GW_MUL(d, d), d), GW_MUL(GW_MUL(bw, bw), bw)));
        return GW_MUL(d < bw ? 1.0 : 0.0, GW_MUL(GW_MUL(t, t), t));
    }
    default: /* GW_KERNEL_BOXCAR */
        return d < bw ? 1.0 : 0.0;
    }
}

#endif /* GW_ARITH_H */
