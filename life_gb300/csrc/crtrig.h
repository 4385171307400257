/*
 * Correctly rounded sin, cos and atan2 for the corotational FEM (the element
 * angle, FEMBodyClass::updateFEMValues, reference src/FEMBody.cpp:217, and
 * the element rotation, FEMElementClass::setElementTransform,
 * src/FEMElement.cpp:255-262), written once for the device and the host.
 *
 * The flexible-body coupling amplifies a one-unit change in the last place of
 * an element angle's sine or cosine into ~1e-11 relative changes of the
 * marker forces, so the result must not depend on which math library
 * evaluated it. These routines return the correctly rounded value (the
 * double nearest the exact result) on the ranges below, with the same
 * sequence of IEEE operations on the GPU and on the host, so the device and a
 * host checker that calls them agree bit for bit.
 *
 * Method (double-double arithmetic, Dekker 1971 / Knuth TAOCP 4.2.2, with the
 * exact product of a fused multiply-add; table-driven reduction as in Tang's
 * table methods, ACM TOMS 1990-1992):
 *   sin/cos: Cody-Waite reduction x = k pi/2 + r with pi/2 split into three
 *     33-bit pieces and a 53-bit tail (k*piece exact for |k| < 2^20); then
 *     r = a + s with a = j/128 the nearest table point (|s| <= 1/256), the
 *     Taylor series of sin s and cos s (three double-double Horner steps and
 *     a double tail), and sin r = sin a cos s + cos a sin s, cos r = cos a
 *     cos s - sin a sin s with sin a, cos a from a 102-entry double-double
 *     table.
 *   atan2: with n = min(|x|,|y|), m = max(|x|,|y|) and c = k/256 the table
 *     point nearest n/m (k from the quotient in single precision, which only
 *     selects the point), atan(n/m) = atan(c) + atan(d),
 *     d = (n - c m) / (m + c n) formed in double-double (one division), the
 *     Taylor series of atan d (|d| <= 1/512 + 2^-20) and atan(k/256) from a
 *     257-entry double-double table; then the octant: pi/2 - a, pi - a, and
 *     the sign of y. Special operands follow C99 Annex F.9.1.4.
 *   Every result is a double-double (hi, lo) normalised so that
 *   hi = RN(hi + lo), with a relative error below about 2^-100; hi is
 *   returned, the correctly rounded value unless the exact result lies within
 *   that distance of a rounding midpoint.
 * The tables and coefficients (crtrig_tables.h) are computed in 400-bit
 * arithmetic (mpmath) from their definitions by crtrig_tables.py.
 *
 * Ranges with the exact path: sin/cos for |x| <= 2^19; atan2 for finite
 * operands whose quotient min/max is 0 or at least 2^-900. Other operands go
 * to the C library's (host) or CUDA's (device) function, whose results then
 * may differ between the two.
 */
#ifndef LIFE_CRTRIG_H
#define LIFE_CRTRIG_H

#include <math.h>

#include "crtrig_tables.h"

#ifdef __CUDACC__
#define LIFE_CR_FN static __host__ __device__ __forceinline__
#else
#define LIFE_CR_FN static inline
#endif

typedef struct {
    double h, l;
} life_dd;

/* The tables, once for the device (global memory) and once for the host. */
#ifdef __CUDACC__
static __device__ const double life_cr_atan256_dev[514] = {LIFE_CR_ATAN256};
static __device__ const double life_cr_sincos128_dev[408] = {LIFE_CR_SINCOS128};
#endif
static const double life_cr_atan256_host[514] = {LIFE_CR_ATAN256};
static const double life_cr_sincos128_host[408] = {LIFE_CR_SINCOS128};

LIFE_CR_FN const double* life_cr_atan_tab(void) {
#ifdef __CUDA_ARCH__
    return life_cr_atan256_dev;
#else
    return life_cr_atan256_host;
#endif
}
LIFE_CR_FN const double* life_cr_sincos_tab(void) {
#ifdef __CUDA_ARCH__
    return life_cr_sincos128_dev;
#else
    return life_cr_sincos128_host;
#endif
}

LIFE_CR_FN life_dd life_dd_make(double h, double l) {
    life_dd r;
    r.h = h;
    r.l = l;
    return r;
}
/* a + b exactly as h + l (Knuth's two-sum) */
LIFE_CR_FN life_dd life_dd_two_sum(double a, double b) {
    const double s = a + b;
    const double bb = s - a;
    return life_dd_make(s, (a - (s - bb)) + (b - bb));
}
/* a + b exactly as h + l when |a| >= |b| or a == 0 (Dekker's fast two-sum) */
LIFE_CR_FN life_dd life_dd_fast(double a, double b) {
    const double s = a + b;
    return life_dd_make(s, b - (s - a));
}
LIFE_CR_FN life_dd life_dd_neg(life_dd a) { return life_dd_make(-a.h, -a.l); }
/* a + b, both double-doubles, accurate also under cancellation */
LIFE_CR_FN life_dd life_dd_add(life_dd a, life_dd b) {
    life_dd s = life_dd_two_sum(a.h, b.h);
    const life_dd t = life_dd_two_sum(a.l, b.l);
    s.l += t.h;
    s = life_dd_fast(s.h, s.l);
    s.l += t.l;
    return life_dd_fast(s.h, s.l);
}
/* a + b when |b| is well below |a| (the Horner steps: no cancellation) */
LIFE_CR_FN life_dd life_dd_add_nc(life_dd a, life_dd b) {
    life_dd s = life_dd_two_sum(a.h, b.h);
    s.l += a.l + b.l;
    return life_dd_fast(s.h, s.l);
}
LIFE_CR_FN life_dd life_dd_add_d(life_dd a, double b) {
    life_dd s = life_dd_two_sum(a.h, b);
    s.l += a.l;
    return life_dd_fast(s.h, s.l);
}
LIFE_CR_FN life_dd life_dd_mul(life_dd a, life_dd b) {
    const double p = a.h * b.h;
    double e = fma(a.h, b.h, -p);
    e += a.h * b.l + a.l * b.h;
    return life_dd_fast(p, e);
}
LIFE_CR_FN life_dd life_dd_mul_d(life_dd a, double b) {
    const double p = a.h * b;
    double e = fma(a.h, b, -p);
    e += a.l * b;
    return life_dd_fast(p, e);
}

/* ------------------------------------------------------------ sin / cos -- */

/* sin and cos of x, each correctly rounded (|x| <= 2^19). */
LIFE_CR_FN void life_cr_sincos(double x, double* s, double* c) {
    if (!(fabs(x) <= 0x1p+19)) {
        *s = sin(x);
        *c = cos(x);
        return;
    }
    if (x == 0.0) { /* keeps the sign of a zero */
        *s = x;
        *c = 1.0;
        return;
    }
    /* x = k pi/2 + r */
    const double kd = rint(x * LIFE_CR_TWO_OVER_PI);
    const double t = x - kd * LIFE_CR_PIO2_1; /* exact (Sterbenz; k * piece exact) */
    life_dd r = life_dd_two_sum(t, -(kd * LIFE_CR_PIO2_2));
    r = life_dd_add_d(r, -(kd * LIFE_CR_PIO2_3));
    {
        const double ph = kd * LIFE_CR_PIO2_4;
        const double pl = fma(kd, LIFE_CR_PIO2_4, -ph);
        r = life_dd_add(r, life_dd_make(-ph, -pl));
    }
    /* r = a + s, a = j/128 (r.h - a is exact: Sterbenz for j != 0) */
    const double jd = rint(r.h * 128.0);
    const life_dd sr = life_dd_two_sum(r.h - jd * 0x1p-7, r.l);
    const int ja = (int)fabs(jd);
    const double* tab = life_cr_sincos_tab() + 4 * ja;
    const double sg = jd < 0.0 ? -1.0 : 1.0;
    const life_dd sa = life_dd_make(sg * tab[0], sg * tab[1]), ca = life_dd_make(tab[2], tab[3]);
    const life_dd z = life_dd_mul(sr, sr);
    /* sin s = s (1 + z (S1 + z (S2 + z (S3 + z (S4 + z S5))))) */
    const double ts = LIFE_CR_S3H + z.h * (LIFE_CR_S4H + z.h * LIFE_CR_S5H);
    /* cos s = 1 + z (C1 + z (C2 + z (C3 + z (C4 + z C5)))) */
    const double tc = LIFE_CR_C3H + z.h * (LIFE_CR_C4H + z.h * LIFE_CR_C5H);
    life_dd ps = life_dd_add_nc(life_dd_make(LIFE_CR_S2H, LIFE_CR_S2L), life_dd_mul_d(z, ts));
    life_dd pc = life_dd_add_nc(life_dd_make(LIFE_CR_C2H, LIFE_CR_C2L), life_dd_mul_d(z, tc));
    ps = life_dd_add_nc(life_dd_make(LIFE_CR_S1H, LIFE_CR_S1L), life_dd_mul(z, ps));
    pc = life_dd_add_nc(life_dd_make(LIFE_CR_C1H, LIFE_CR_C1L), life_dd_mul(z, pc));
    ps = life_dd_add_nc(life_dd_make(1.0, 0.0), life_dd_mul(z, ps));
    pc = life_dd_add_nc(life_dd_make(1.0, 0.0), life_dd_mul(z, pc));
    const life_dd sin_s = life_dd_mul(sr, ps);
    const life_dd sin_r = life_dd_add(life_dd_mul(sa, pc), life_dd_mul(ca, sin_s));
    const life_dd cos_r = life_dd_add(life_dd_mul(ca, pc), life_dd_neg(life_dd_mul(sa, sin_s)));
    const int q = ((int)kd) & 3;
    const double sv = sin_r.h, cv = cos_r.h;
    *s = q == 0 ? sv : q == 1 ? cv : q == 2 ? -sv : -cv;
    *c = q == 0 ? cv : q == 1 ? -sv : q == 2 ? -cv : sv;
}

LIFE_CR_FN double life_cr_sin(double x) {
    double s, c;
    life_cr_sincos(x, &s, &c);
    return s;
}
LIFE_CR_FN double life_cr_cos(double x) {
    double s, c;
    life_cr_sincos(x, &s, &c);
    return c;
}

/* ---------------------------------------------------------------- atan2 -- */

/* atan(num/den) for 0 < num <= den (finite, quotient at least 2^-900). */
LIFE_CR_FN life_dd life_cr_atan_ratio(double num, double den) {
    /* the table point: any k near 256 num/den will do (|d| stays below
     * 1/512 + 2^-20); single precision when the operands allow it */
    int k;
    if (den <= 0x1p+100 && num >= 0x1p-100 && num >= den * 0x1p-60) k = (int)rintf(((float)num / (float)den) * 256.0f);
    else k = (int)rint((num / den) * 256.0);
    const double c = (double)k * 0x1p-8;
    /* d = (num - c den) / (den + c num), numerator and denominator exact
     * products (fma) summed in double-double */
    const double p = c * den, pe = fma(c, den, -p);
    const life_dd N = life_dd_add_d(life_dd_two_sum(num, -p), -pe);
    const double q = c * num, qe = fma(c, num, -q);
    const life_dd D = life_dd_add_d(life_dd_two_sum(den, q), qe);
    const double inv = 1.0 / D.h;
    const double q1 = N.h * inv;
    const double t1 = q1 * D.h, t1e = fma(q1, D.h, -t1);
    life_dd rr = life_dd_two_sum(N.h, -t1);
    rr.l += ((N.l - t1e) - q1 * D.l);
    const double q2 = (rr.h + rr.l) * inv;
    const life_dd d = life_dd_fast(q1, q2);
    const life_dd z = life_dd_mul(d, d);
    /* atan d = d (1 + z (A1 + z (A2 + z (A3 + z (A4 + z A5))))) */
    const double ta = LIFE_CR_A3H + z.h * (LIFE_CR_A4H + z.h * LIFE_CR_A5H);
    life_dd pa = life_dd_add_nc(life_dd_make(LIFE_CR_A2H, LIFE_CR_A2L), life_dd_mul_d(z, ta));
    pa = life_dd_add_nc(life_dd_make(LIFE_CR_A1H, LIFE_CR_A1L), life_dd_mul(z, pa));
    pa = life_dd_add_nc(life_dd_make(1.0, 0.0), life_dd_mul(z, pa));
    const double* tab = life_cr_atan_tab() + 2 * k;
    return life_dd_add(life_dd_make(tab[0], tab[1]), life_dd_mul(d, pa));
}

/* atan2(y, x), correctly rounded. */
LIFE_CR_FN double life_cr_atan2(double y, double x) {
    if (isnan(x) || isnan(y)) return x + y;
    const double ax = fabs(x), ay = fabs(y);
    const double sy = signbit(y) ? -1.0 : 1.0;
    /* C99 Annex F.9.1.4 */
    if (ay == 0.0) return (signbit(x) ? LIFE_CR_PI_H : 0.0) * sy;
    if (isinf(ay)) return (isinf(ax) ? (signbit(x) ? LIFE_CR_TPIO4_H : LIFE_CR_PIO4_H) : LIFE_CR_PIO2_H) * sy;
    if (ax == 0.0) return LIFE_CR_PIO2_H * sy;
    if (isinf(ax)) return (signbit(x) ? LIFE_CR_PI_H : 0.0) * sy;
    const int swap = ay > ax;
    const double num = swap ? ax : ay, den = swap ? ay : ax;
    /* quotient at least 2^-900, tested with exact scalings */
    if (!(den >= 0x1p-100 ? num >= den * 0x1p-900 : num * 0x1p+900 >= den)) return atan2(y, x);
    life_dd a = life_cr_atan_ratio(num, den);
    if (swap) a = life_dd_add(life_dd_make(LIFE_CR_PIO2_H, LIFE_CR_PIO2_L), life_dd_neg(a));
    if (signbit(x)) a = life_dd_add(life_dd_make(LIFE_CR_PI_H, LIFE_CR_PI_L), life_dd_neg(a));
    return a.h * sy;
}

#endif /* LIFE_CRTRIG_H */
