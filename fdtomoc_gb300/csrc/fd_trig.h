/* Double-precision sin, cos and atan2 evaluated in double-double arithmetic and rounded once, so that
 * the result is the correctly rounded value except when the exact value lies within about 2^-100
 * (relative) of a rounding boundary.  The same source is compiled for the host and the device, with
 * no fused multiply-add contraction, and gives the same bits on both; it is what the ray tracer uses
 * wherever sphrayderv calls the C library's sin, cos and atan2 (src/sphrayderv.c:1794-1990).
 *
 * Method (textbook double-double arithmetic, Dekker 1971 / Knuth TAOCP vol. 2 4.2.2):
 *  - exact sum (two-sum) and exact product (the rounding error of a*b recovered with one fma);
 *  - sin, cos: Cody-Waite reduction x = k*pi/2 + r with pi/2 split into three doubles, |r| <= ~pi/4,
 *    then the Taylor series of sin r and cos r to r^29 / r^28 in double-double (the first omitted
 *    term is below 1e-33 for |r| <= 0.8);
 *  - atan2: the platform atan2 gives a first value a0; one Newton correction in double-double,
 *    a = a0 + (y cos a0 - x sin a0) / (x cos a0 + y sin a0), removes its error (|a - a0| ~ 1e-16, so
 *    the neglected cubic term is ~1e-48).  Different first values (host and device) lead to the same
 *    rounded result unless the exact value is within ~1e-32 of a rounding boundary.
 * The series coefficients 1/n! are double-double constants (hi = nearest double, lo = nearest double
 * to the remainder), computed with 60-digit arithmetic. */
#ifndef FD_TRIG_H
#define FD_TRIG_H

#include <math.h>

#ifdef __CUDACC__
#define FDT_FN static __device__ __forceinline__
#define FDT_FMA(a, b, c) fma((a), (b), (c))
#else
#define FDT_FN static inline
#define FDT_FMA(a, b, c) fma((a), (b), (c))
#endif

typedef struct {
    double hi, lo;
} fdt_dd;

FDT_FN fdt_dd fdt_two_sum(double a, double b)
{
    fdt_dd r;
    r.hi = a + b;
    const double bb = r.hi - a;
    r.lo = (a - (r.hi - bb)) + (b - bb);
    return r;
}

FDT_FN fdt_dd fdt_fast_two_sum(double a, double b)   /* |a| >= |b| */
{
    fdt_dd r;
    r.hi = a + b;
    r.lo = b - (r.hi - a);
    return r;
}

FDT_FN fdt_dd fdt_two_prod(double a, double b)
{
    fdt_dd r;
    r.hi = a * b;
    r.lo = FDT_FMA(a, b, -r.hi);
    return r;
}

FDT_FN fdt_dd fdt_add(fdt_dd a, fdt_dd b)
{
    fdt_dd s = fdt_two_sum(a.hi, b.hi);
    const fdt_dd t = fdt_two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fdt_fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fdt_fast_two_sum(s.hi, s.lo);
}

FDT_FN fdt_dd fdt_mul(fdt_dd a, fdt_dd b)
{
    fdt_dd p = fdt_two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo + a.lo * b.hi;
    return fdt_fast_two_sum(p.hi, p.lo);
}

FDT_FN fdt_dd fdt_mul_d(fdt_dd a, double b)
{
    fdt_dd p = fdt_two_prod(a.hi, b);
    p.lo += a.lo * b;
    return fdt_fast_two_sum(p.hi, p.lo);
}

/* pi/2 as three doubles: hi + mid + lo to ~160 bits */
#define FDT_PIO2_1 1.5707963267948966e+00
#define FDT_PIO2_2 6.123233995736766e-17
#define FDT_PIO2_3 -1.4973849048591698e-33
#define FDT_2OPI 0.6366197723675814

/* 1/n! for n = 2 .. 29 as double-double (index n) */
#define FDT_NFACT 30
#ifdef __CUDACC__
__constant__
#endif
static const double fdt_inv_fact[FDT_NFACT][2] = {
    {1.0, 0.0},
    {1.0, 0.0},
    {0.5, 0.0},
    {0.16666666666666666, 9.25185853854297e-18},
    {0.041666666666666664, 2.3129646346357427e-18},
    {0.008333333333333333, 1.1564823173178714e-19},
    {0.001388888888888889, -5.300543954373577e-20},
    {0.0001984126984126984, 1.7209558293420705e-22},
    {2.48015873015873e-05, 2.1511947866775882e-23},
    {2.7557319223985893e-06, -1.858393274046472e-22},
    {2.755731922398589e-07, 2.3767714622250297e-23},
    {2.505210838544172e-08, -1.448814070935912e-24},
    {2.08767569878681e-09, -1.20734505911326e-25},
    {1.6059043836821613e-10, 1.2585294588752098e-26},
    {1.1470745597729725e-11, 2.0655512752830745e-28},
    {7.647163731819816e-13, 7.03872877733453e-30},
    {4.779477332387385e-14, 4.399205485834081e-31},
    {2.8114572543455206e-15, 1.6508842730861433e-31},
    {1.5619206968586225e-16, 1.1910679660273754e-32},
    {8.22063524662433e-18, 2.2141894119604265e-34},
    {4.110317623312165e-19, 1.4412973378659527e-36},
    {1.9572941063391263e-20, -1.3643503830087908e-36},
    {8.896791392450574e-22, -7.911402614872376e-38},
    {3.868170170630684e-23, -8.843177655482344e-40},
    {1.6117375710961184e-24, -3.6846573564509766e-41},
    {6.446950284384474e-26, -1.9330404233703465e-42},
    {2.4795962632247976e-27, -1.2953730964765229e-43},
    {9.183689863795546e-29, 1.4303150396787322e-45},
    {3.279889237069838e-30, 1.5117542744029879e-46},
    {1.1309962886447716e-31, 1.0498015412959506e-47},
};

#ifdef __CUDACC__
#define FDT_FACT(n) fdt_dd{fdt_inv_fact[(n)][0], fdt_inv_fact[(n)][1]}
#else
#define FDT_FACT(n) ((fdt_dd){fdt_inv_fact[(n)][0], fdt_inv_fact[(n)][1]})
#endif

/* r = x - k pi/2 in double-double, k = nearest integer to x * 2/pi */
FDT_FN fdt_dd fdt_reduce(double x, int *quadrant)
{
    const double k = rint(x * FDT_2OPI);
    fdt_dd t = fdt_two_prod(k, FDT_PIO2_1);
    fdt_dd r = fdt_two_sum(x, -t.hi);
    r.lo -= t.lo;
    r = fdt_fast_two_sum(r.hi, r.lo);
    t = fdt_two_prod(k, FDT_PIO2_2);
    t.lo += k * FDT_PIO2_3;
    t.hi = -t.hi;
    t.lo = -t.lo;
    r = fdt_add(r, t);
    *quadrant = ((int)k) & 3;
    return r;
}

/* sin r and cos r, |r| <= ~0.8, as double-double */
FDT_FN void fdt_sincos_dd(fdt_dd r, fdt_dd *s, fdt_dd *c)
{
    const fdt_dd r2 = fdt_mul(r, r);
    fdt_dd ps = FDT_FACT(29), pc = FDT_FACT(28);
    for (int n = 27; n >= 3; n -= 2) {            /* sin: sum (-1)^m r^(2m+1)/(2m+1)! */
        ps = fdt_mul(ps, r2);
        ps.hi = -ps.hi;
        ps.lo = -ps.lo;
        ps = fdt_add(ps, FDT_FACT(n));
    }
    for (int n = 26; n >= 2; n -= 2) {            /* cos */
        pc = fdt_mul(pc, r2);
        pc.hi = -pc.hi;
        pc.lo = -pc.lo;
        pc = fdt_add(pc, FDT_FACT(n));
    }
    /* sin r = r (1 - r^2 ps'), written as r - r^3 ps with ps the series from 1/3! */
    fdt_dd t = fdt_mul(fdt_mul(r2, r), ps);
    t.hi = -t.hi;
    t.lo = -t.lo;
    *s = fdt_add(r, t);
    fdt_dd u = fdt_mul(r2, pc);
    u.hi = -u.hi;
    u.lo = -u.lo;
    fdt_dd one;
    one.hi = 1.0;
    one.lo = 0.0;
    *c = fdt_add(one, u);
}

FDT_FN void fdt_sincos_full(double x, fdt_dd *s, fdt_dd *c)
{
    int q = 0;
    const fdt_dd r = fdt_reduce(x, &q);
    fdt_dd sr, cr;
    fdt_sincos_dd(r, &sr, &cr);
    fdt_dd ns = sr, nc = cr;
    ns.hi = -sr.hi;
    ns.lo = -sr.lo;
    nc.hi = -cr.hi;
    nc.lo = -cr.lo;
    switch (q) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = ns; break;
    case 2: *s = ns; *c = nc; break;
    default: *s = nc; *c = sr; break;
    }
}

FDT_FN double fdt_sin(double x)
{
    fdt_dd s, c;
    fdt_sincos_full(x, &s, &c);
    return s.hi + s.lo;
}

FDT_FN double fdt_cos(double x)
{
    fdt_dd s, c;
    fdt_sincos_full(x, &s, &c);
    return c.hi + c.lo;
}

/* atan2(y, x) for finite y, x not both zero */
FDT_FN double fdt_atan2(double y, double x)
{
    const double a0 = atan2(y, x);
    fdt_dd s, c;
    fdt_sincos_full(a0, &s, &c);
    /* num = y cos a0 - x sin a0 (double-double), den = x cos a0 + y sin a0 (double) */
    fdt_dd num = fdt_add(fdt_mul_d(c, y), fdt_mul_d(s, -x));
    const double den = x * c.hi + y * s.hi;
    const double delta = (num.hi + num.lo) / den;
    const fdt_dd a = fdt_two_sum(a0, delta);
    return a.hi + a.lo;
}

#endif
