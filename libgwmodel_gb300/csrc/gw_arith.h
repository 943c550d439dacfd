/*
 * gw_arith.h -- FP64 arithmetic of the distance and kernel-weight formulas,
 * compiled for the device by nvcc and for the host by gcc, with the same
 * sequence of correctly rounded operations (+ - * / sqrt fma) on both.
 *
 * Great-circle distance.  The reference evaluates CRSDistance::SpGcdist
 * (CRSDistance.cpp:15-69) with the platform libm.  glibc's sin, cos and atan
 * return the correctly rounded result for all but a tiny fraction of
 * arguments, and every other operation of the formula is an IEEE operation,
 * so a distance evaluated with CORRECTLY ROUNDED sin, cos and atan is the
 * reference's double.  gw_sincos_cr and gw_atan_cr compute those results in
 * double-double arithmetic (Dekker/Knuth error-free transforms, ~104-bit
 * accuracy) and round once, so they are correctly rounded except when the
 * exact value lies within ~2^-100 relative of a rounding midpoint:
 *   - sin/cos: reduction by pi/2 split into three doubles, then the Taylor
 *     series of sin and cos to r^29 / r^28 (|r| <= pi/4), the small terms in
 *     double and the leading ones in double-double;
 *   - atan: atan(x) = pi/2 - atan(1/x) for x > 1, then
 *     atan(t) = atan(k/16) + atan((t - k/16) / (1 + t k/16)) with k = rint(16 t)
 *     and the alternating series to u^23 (|u| <= 1/32).
 * The constants (1/n!, atan(k/16), pi/2) are those exact values split into
 * double pairs (computed at 300 bits).  gw_gc_dist uses them: the exact
 * select stage and every other place whose result must be the reference's
 * double.  gw_gc_dist_fast evaluates the same formula with single-double
 * Taylor series (a few ulp), for kernel weights, where an ulp of distance
 * moves a weight by ~1e-16 relative.
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
/* out of line: a rarely taken call keeps the callers' register budget */
#define GW_HD_CALL static __host__ __device__ __noinline__
#else
#define GW_HD static inline
#define GW_HD_CALL static
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

/* ------------------------------------------------ double-double arithmetic */
/* A value hi + lo with |lo| <= ulp(hi) / 2.  Error-free transforms: TwoSum
 * (Knuth), FastTwoSum (Dekker, |a| >= |b|) and TwoProd through one fma. */
typedef struct
{
    double hi, lo;
} gw_dd;

GW_HD gw_dd gw_dd_make(double hi, double lo)
{
    gw_dd r;
    r.hi = hi;
    r.lo = lo;
    return r;
}

GW_HD gw_dd gw_two_sum(double a, double b)
{
    double s = GW_ADD(a, b);
    double bb = GW_SUB(s, a);
    double e = GW_ADD(GW_SUB(a, GW_SUB(s, bb)), GW_SUB(b, bb));
    return gw_dd_make(s, e);
}

GW_HD gw_dd gw_fast_two_sum(double a, double b)
{
    double s = GW_ADD(a, b);
    return gw_dd_make(s, GW_SUB(b, GW_SUB(s, a)));
}

GW_HD gw_dd gw_two_prod(double a, double b)
{
    double p = GW_MUL(a, b);
    return gw_dd_make(p, GW_FMA(a, b, -p));
}

GW_HD gw_dd gw_dd_add(gw_dd x, gw_dd y)
{
    gw_dd s = gw_two_sum(x.hi, y.hi);
    gw_dd t = gw_two_sum(x.lo, y.lo);
    s = gw_fast_two_sum(s.hi, GW_ADD(s.lo, t.hi));
    return gw_fast_two_sum(s.hi, GW_ADD(s.lo, t.lo));
}

GW_HD gw_dd gw_dd_add_d(gw_dd x, double y)
{
    gw_dd s = gw_two_sum(x.hi, y);
    return gw_fast_two_sum(s.hi, GW_ADD(s.lo, x.lo));
}

GW_HD gw_dd gw_dd_mul(gw_dd x, gw_dd y)
{
    gw_dd p = gw_two_prod(x.hi, y.hi);
    double c = GW_FMA(x.hi, y.lo, GW_MUL(x.lo, y.hi));
    return gw_fast_two_sum(p.hi, GW_ADD(p.lo, c));
}

GW_HD gw_dd gw_dd_mul_d(gw_dd x, double y)
{
    gw_dd p = gw_two_prod(x.hi, y);
    return gw_fast_two_sum(p.hi, GW_FMA(x.lo, y, p.lo));
}

/* x / y by two correction steps of the double quotient. */
GW_HD gw_dd gw_dd_div(gw_dd x, gw_dd y)
{
    double q1 = GW_DIV(x.hi, y.hi);
    gw_dd r = gw_dd_add(x, gw_dd_mul_d(y, -q1));
    double q2 = GW_DIV(r.hi, y.hi);
    r = gw_dd_add(r, gw_dd_mul_d(y, -q2));
    double q3 = GW_DIV(r.hi, y.hi);
    gw_dd q = gw_fast_two_sum(q1, q2);
    return gw_dd_add_d(q, q3);
}

/* 1/n! as double pairs, n = 0..29 (exact values split at 300 bits). */
GW_HD double gw_inv_fact_hi(int n)
{
    switch (n)
    {
    case 0: case 1: return 1.0;
    case 2: return 0x1.0000000000000p-1;
    case 3: return 0x1.5555555555555p-3;
    case 4: return 0x1.5555555555555p-5;
    case 5: return 0x1.1111111111111p-7;
    case 6: return 0x1.6c16c16c16c17p-10;
    case 7: return 0x1.a01a01a01a01ap-13;
    case 8: return 0x1.a01a01a01a01ap-16;
    case 9: return 0x1.71de3a556c734p-19;
    case 10: return 0x1.27e4fb7789f5cp-22;
    case 11: return 0x1.ae64567f544e4p-26;
    case 12: return 0x1.1eed8eff8d898p-29;
    case 13: return 0x1.6124613a86d09p-33;
    case 14: return 0x1.93974a8c07c9dp-37;
    case 15: return 0x1.ae7f3e733b81fp-41;
    case 16: return 0x1.ae7f3e733b81fp-45;
    case 17: return 0x1.952c77030ad4ap-49;
    case 18: return 0x1.6827863b97d97p-53;
    case 19: return 0x1.2f49b46814157p-57;
    case 20: return 0x1.e542ba4020225p-62;
    case 21: return 0x1.71b8ef6dcf572p-66;
    case 22: return 0x1.0ce396db7f853p-70;
    case 23: return 0x1.761b41316381ap-75;
    case 24: return 0x1.f2cf01972f578p-80;
    case 25: return 0x1.3f3ccdd165fa9p-84;
    case 26: return 0x1.88e85fc6a4e5ap-89;
    case 27: return 0x1.d1ab1c2dccea3p-94;
    case 28: return 0x1.0a18a2635085dp-98;
    default: return 0x1.259f98b4358adp-103; /* 29 */
    }
}
GW_HD double gw_inv_fact_lo(int n)
{
    switch (n)
    {
    case 3: return 0x1.5555555555555p-57;
    case 4: return 0x1.5555555555555p-59;
    case 5: return 0x1.1111111111111p-63;
    case 6: return -0x1.f49f49f49f49fp-65;
    case 7: return 0x1.a01a01a01a01ap-73;
    case 8: return 0x1.a01a01a01a01ap-76;
    case 9: return -0x1.c154f8ddc6c00p-73;
    case 10: return 0x1.cbbc05b4fa99ap-76;
    case 11: return -0x1.c062e06d1f209p-80;
    case 12: return -0x1.2aec959e14c06p-83;
    case 13: return 0x1.f28e0cc748ebep-87;
    case 14: return 0x1.05d6f8a2efd1fp-92;
    case 15: return 0x1.1d8656b0ee8cbp-97;
    case 16: return 0x1.1d8656b0ee8cbp-101;
    default: return 0.0; /* 0, 1, 2 exact; beyond 16 the tail is summed in double */
    }
}

/* sin and cos of r = rh + rl, |r| <= pi/4 (+ a hair), in double-double.
 * sin r = r S(z), cos r = C(z), z = r^2, S and C the Taylor series in z;
 * the terms from z^8 on (< 6e-17 relative) are summed in double. */
GW_HD void gw_sincos_dd(gw_dd r, gw_dd* s, gw_dd* c)
{
    const gw_dd z = gw_dd_mul(r, r);
    const double zh = z.hi;
    /* S tail: sum_{k=8..14} (-1)^k z^(k-8) / (2k+1)! */
    double ts = gw_inv_fact_hi(29);
    ts = GW_FMA(ts, zh, -gw_inv_fact_hi(27));
    ts = GW_FMA(ts, zh, gw_inv_fact_hi(25));
    ts = GW_FMA(ts, zh, -gw_inv_fact_hi(23));
    ts = GW_FMA(ts, zh, gw_inv_fact_hi(21));
    ts = GW_FMA(ts, zh, -gw_inv_fact_hi(19));
    ts = GW_FMA(ts, zh, gw_inv_fact_hi(17));
    /* C tail: sum_{k=8..14} (-1)^k z^(k-8) / (2k)! */
    double tc = gw_inv_fact_hi(28);
    tc = GW_FMA(tc, zh, -gw_inv_fact_hi(26));
    tc = GW_FMA(tc, zh, gw_inv_fact_hi(24));
    tc = GW_FMA(tc, zh, -gw_inv_fact_hi(22));
    tc = GW_FMA(tc, zh, gw_inv_fact_hi(20));
    tc = GW_FMA(tc, zh, -gw_inv_fact_hi(18));
    tc = GW_FMA(tc, zh, gw_inv_fact_hi(16));
    gw_dd ps = gw_dd_make(ts, 0.0), pc = gw_dd_make(tc, 0.0);
    for (int k = 7; k >= 0; k--)
    {
        const double sg = (k & 1) ? -1.0 : 1.0;
        ps = gw_dd_add(gw_dd_mul(ps, z), gw_dd_make(sg * gw_inv_fact_hi(2 * k + 1), sg * gw_inv_fact_lo(2 * k + 1)));
        pc = gw_dd_add(gw_dd_mul(pc, z), gw_dd_make(sg * gw_inv_fact_hi(2 * k), sg * gw_inv_fact_lo(2 * k)));
    }
    *s = gw_dd_mul(r, ps);
    *c = pc;
}

/* Correctly rounded sin(x) and cos(x) for |x| <= 2^20 (the great-circle
 * formula takes half-differences and half-sums of radians, |x| <= 2 pi for
 * longitudes in [-360, 360]).  r = x - k pi/2 with pi/2 = P1 + P2 + P3
 * (~160 bits) and the products k P1, k P2 kept exact as double pairs. */
GW_HD void gw_sincos_cr(double x, double* s, double* c)
{
    const double P1 = 0x1.921fb54442d18p+0, P2 = 0x1.1a62633145c07p-54, P3 = -0x1.f1976b7ed8fbcp-110;
    const double k = GW_RINT(GW_MUL(x, GW_TWO_OVER_PI));
    const gw_dd k1 = gw_two_prod(-k, P1);
    gw_dd r = gw_two_sum(x, k1.hi);
    r = gw_dd_add_d(r, k1.lo);
    r = gw_dd_add(r, gw_two_prod(-k, P2));
    r = gw_dd_add_d(r, GW_MUL(-k, P3));
    gw_dd sr, cr;
    gw_sincos_dd(r, &sr, &cr);
    const double sv = GW_ADD(sr.hi, sr.lo), cv = GW_ADD(cr.hi, cr.lo);
    const long long q = (long long)k & 3;
    if (q == 0) { *s = sv; *c = cv; }
    else if (q == 1) { *s = cv; *c = -sv; }
    else if (q == 2) { *s = -sv; *c = -cv; }
    else { *s = -cv; *c = sv; }
}

/* atan(k/16), k = 0..16, as double pairs. */
GW_HD gw_dd gw_atan_k16(int k)
{
    switch (k)
    {
    case 1: return gw_dd_make(0x1.ff55bb72cfdeap-5, -0x1.c934d86d23f1dp-60);
    case 2: return gw_dd_make(0x1.fd5ba9aac2f6ep-4, -0x1.cd37686760c17p-59);
    case 3: return gw_dd_make(0x1.7b97b4bce5b02p-3, 0x1.347b0b4f881cap-58);
    case 4: return gw_dd_make(0x1.f5b75f92c80ddp-3, 0x1.8ab6e3cf7afbdp-57);
    case 5: return gw_dd_make(0x1.362773707ebccp-2, -0x1.963a544b672d8p-57);
    case 6: return gw_dd_make(0x1.6f61941e4def1p-2, -0x1.c63aae6f6e918p-56);
    case 7: return gw_dd_make(0x1.a64eec3cc23fdp-2, -0x1.24dec1b50b7ffp-56);
    case 8: return gw_dd_make(0x1.dac670561bb4fp-2, 0x1.a2b7f222f65e2p-56);
    case 9: return gw_dd_make(0x1.0657e94db30d0p-1, -0x1.d5b495f6349e6p-56);
    case 10: return gw_dd_make(0x1.1e00babdefeb4p-1, -0x1.928df287a668fp-58);
    case 11: return gw_dd_make(0x1.345f01cce37bbp-1, 0x1.1021137c71102p-55);
    case 12: return gw_dd_make(0x1.4978fa3269ee1p-1, 0x1.2419a87f2a458p-56);
    case 13: return gw_dd_make(0x1.5d58987169b18p-1, 0x1.0028e4bc5e7cap-57);
    case 14: return gw_dd_make(0x1.700a7c5784634p-1, -0x1.8c34d25aadef6p-56);
    case 15: return gw_dd_make(0x1.819d0b7158a4dp-1, -0x1.bf76229d3b917p-56);
    case 16: return gw_dd_make(0x1.921fb54442d18p-1, 0x1.1a62633145c07p-55);
    default: return gw_dd_make(0.0, 0.0);
    }
}

/* Correctly rounded atan(x) for x >= 0 (NaN propagates, +inf gives pi/2). */
GW_HD double gw_atan_cr(double x)
{
    if (!(x == x)) return x;
    if (x > 0x1p60) return GW_PIO2_HI;
    const int inv = x > 1.0;
    gw_dd t = inv ? gw_dd_div(gw_dd_make(1.0, 0.0), gw_dd_make(x, 0.0)) : gw_dd_make(x, 0.0);
    const int k = (int)GW_RINT(GW_MUL(t.hi, 16.0));
    const double ck = GW_MUL((double)k, 0.0625);
    /* u = (t - c) / (1 + t c): numerator exact to double-double, denominator too */
    const gw_dd num = gw_dd_add_d(t, -ck);
    const gw_dd den = gw_dd_add_d(gw_dd_mul_d(t, ck), 1.0);
    const gw_dd u = k ? gw_dd_div(num, den) : t;
    const gw_dd z = gw_dd_mul(u, u);
    /* alternating series sum_{j=0..11} (-1)^j z^j / (2j + 1); the terms from z^6 on in double */
    const double zh = z.hi;
    double tail = -0x1.642c8590b2164p-5;           /* -1/23 */
    tail = GW_FMA(tail, zh, 0x1.8618618618618p-5); /*  1/21 */
    tail = GW_FMA(tail, zh, -0x1.af286bca1af28p-5); /* -1/19 */
    tail = GW_FMA(tail, zh, 0x1.e1e1e1e1e1e1ep-5); /*  1/17 */
    tail = GW_FMA(tail, zh, -0x1.1111111111111p-4); /* -1/15 */
    tail = GW_FMA(tail, zh, 0x1.3b13b13b13b14p-4); /*  1/13 */
    gw_dd p = gw_dd_make(tail, 0.0);
    p = gw_dd_add(gw_dd_mul(p, z), gw_dd_make(-0x1.745d1745d1746p-4, 0x1.745d1745d1746p-59)); /* -1/11 */
    p = gw_dd_add(gw_dd_mul(p, z), gw_dd_make(0x1.c71c71c71c71cp-4, 0x1.c71c71c71c71cp-58));  /*  1/9 */
    p = gw_dd_add(gw_dd_mul(p, z), gw_dd_make(-0x1.2492492492492p-3, -0x1.2492492492492p-57)); /* -1/7 */
    p = gw_dd_add(gw_dd_mul(p, z), gw_dd_make(0x1.999999999999ap-3, -0x1.999999999999ap-57)); /*  1/5 */
    p = gw_dd_add(gw_dd_mul(p, z), gw_dd_make(-0x1.5555555555555p-2, -0x1.5555555555555p-56)); /* -1/3 */
    p = gw_dd_add_d(gw_dd_mul(p, z), 1.0);
    gw_dd a = gw_dd_add(gw_atan_k16(k), gw_dd_mul(u, p));
    if (inv) a = gw_dd_add(gw_dd_make(GW_PIO2_HI, GW_PIO2_LO), gw_dd_make(-a.hi, -a.lo));
    return GW_ADD(a.hi, a.lo);
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
 * (DE2RA = M_PI / 180; lat1R = lat1 * DE2RA).  CR selects the correctly
 * rounded sin/cos/atan (the reference's doubles) or the single-double ones. */
GW_HD double gw_gc_dist_impl(double lon1, double lon2, double lat1, double lat2, double lon1R, double lon2R,
                             double lat1R, double lat2R, int cr)
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
    if (cr)
    {
        gw_sincos_cr(F, &sF, &cF);
        gw_sincos_cr(G, &sG, &cG);
        gw_sincos_cr(L, &sL, &cL);
    }
    else
    {
        gw_sincos(F, &sF, &cF);
        gw_sincos(G, &sG, &cG);
        gw_sincos(L, &sL, &cL);
    }
    double sinG2 = GW_MUL(sG, sG), cosG2 = GW_MUL(cG, cG);
    double sinF2 = GW_MUL(sF, sF), cosF2 = GW_MUL(cF, cF);
    double sinL2 = GW_MUL(sL, sL), cosL2 = GW_MUL(cL, cL);
    double S = GW_ADD(GW_MUL(sinG2, cosL2), GW_MUL(cosF2, sinL2));
    double C = GW_ADD(GW_MUL(cosG2, cosL2), GW_MUL(sinF2, sinL2));
    double q = GW_SQRT(GW_DIV(S, C));
    double w = cr ? gw_atan_cr(q) : gw_atan_nonneg(q);
    double R = GW_DIV(GW_SQRT(GW_MUL(S, C)), w);
    double D = GW_MUL(GW_MUL(2.0, w), a);
    double H1 = GW_DIV(GW_SUB(GW_MUL(3.0, R), 1.0), GW_MUL(2.0, C));
    double H2 = GW_DIV(GW_ADD(GW_MUL(3.0, R), 1.0), GW_MUL(2.0, S));
    double t1 = GW_MUL(GW_MUL(GW_MUL(f, H1), sinF2), cosG2);
    double t2 = GW_MUL(GW_MUL(GW_MUL(f, H2), cosF2), sinG2);
    return GW_MUL(D, GW_SUB(GW_ADD(1.0, t1), t2));
}

/* The reference's double (correctly rounded sin/cos/atan). */
GW_HD_CALL double gw_gc_dist(double lon1, double lon2, double lat1, double lat2, double lon1R, double lon2R,
                        double lat1R, double lat2R)
{
    return gw_gc_dist_impl(lon1, lon2, lat1, lat2, lon1R, lon2R, lat1R, lat2R, 1);
}

/* Within a few ulp of the reference's double (single-double sin/cos/atan). */
GW_HD double gw_gc_dist_fast(double lon1, double lon2, double lat1, double lat2, double lon1R, double lon2R,
                             double lat1R, double lat2R)
{
    return gw_gc_dist_impl(lon1, lon2, lat1, lat2, lon1R, lon2R, lat1R, lat2R, 0);
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
