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
 * exact product of a fused multiply-add):
 *   sin/cos: Cody-Waite reduction x = k pi/2 + r with pi/2 split into three
 *     33-bit pieces and a 53-bit tail (k*piece exact for |k| < 2^20), then
 *     the Taylor series of sin r and cos r (|r| <= pi/4 + tiny) evaluated by
 *     Horner's rule, in double-double for the leading terms and in double
 *     for the tail; total relative error below 2^-99.
 *   atan2: t = min(|x|,|y|) / max(|x|,|y|) in double-double; atan t =
 *     atan(c) + atan((t - c) / (1 + t c)) with c = k/32 the nearest table
 *     point (a 33-entry table of atan(k/32) in double-double) and the Taylor
 *     series of the small remainder; then the octant: pi/2 - a, pi - a, and
 *     the sign of y. Special operands follow C99 Annex F.9.1.4.
 *   The double-double result (hi, lo) is normalised so that hi = RN(hi + lo),
 *   and hi is returned: it is the correctly rounded value unless the exact
 *   result lies within 2^-99 relative of a rounding midpoint.
 * The constants were computed in 400-bit arithmetic (mpmath) from their
 * definitions: the pieces of pi/2, pi/2 and pi as double-doubles, the Taylor
 * coefficients (-1)^j / n!, (-1)^j / (2j + 1), and atan(k/32).
 *
 * Ranges with the exact path: sin/cos for |x| <= 2^19; atan2 for finite
 * operands whose quotient min/max is 0 or at least 2^-900. Other operands go
 * to the C library's (host) or CUDA's (device) function, whose results then
 * may differ between the two.
 */
#ifndef LIFE_CRTRIG_H
#define LIFE_CRTRIG_H

#include <math.h>

#ifdef __CUDACC__
#define LIFE_CR_FN static __host__ __device__ __forceinline__
#else
#define LIFE_CR_FN static inline
#endif

typedef struct {
    double h, l;
} life_dd;

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
LIFE_CR_FN life_dd life_dd_add(life_dd a, life_dd b) {
    life_dd s = life_dd_two_sum(a.h, b.h);
    const life_dd t = life_dd_two_sum(a.l, b.l);
    s.l += t.h;
    s = life_dd_fast(s.h, s.l);
    s.l += t.l;
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
LIFE_CR_FN life_dd life_dd_div(life_dd a, life_dd b) {
    const double q1 = a.h / b.h;
    life_dd r = life_dd_add(a, life_dd_neg(life_dd_mul_d(b, q1)));
    const double q2 = r.h / b.h;
    r = life_dd_add(r, life_dd_neg(life_dd_mul_d(b, q2)));
    const double q3 = r.h / b.h;
    return life_dd_add_d(life_dd_fast(q1, q2), q3);
}

/* ------------------------------------------------------------ sin / cos -- */

/* (-1)^j / (2j+1)!, j = 0..14: double-double for j <= 7, double above */
#define LIFE_CR_SIN_DD(j)                                                                   \
    ((j) == 0 ? life_dd_make(0x1p+0, 0.0)                                                   \
     : (j) == 1 ? life_dd_make(-0x1.5555555555555p-3, -0x1.5555555555555p-57)               \
     : (j) == 2 ? life_dd_make(0x1.1111111111111p-7, 0x1.1111111111111p-63)                 \
     : (j) == 3 ? life_dd_make(-0x1.a01a01a01a01ap-13, -0x1.a01a01a01a01ap-73)              \
     : (j) == 4 ? life_dd_make(0x1.71de3a556c734p-19, -0x1.c154f8ddc6c00p-73)               \
     : (j) == 5 ? life_dd_make(-0x1.ae64567f544e4p-26, 0x1.c062e06d1f209p-80)               \
     : (j) == 6 ? life_dd_make(0x1.6124613a86d09p-33, 0x1.f28e0cc748ebep-87)                \
                : life_dd_make(-0x1.ae7f3e733b81fp-41, -0x1.1d8656b0ee8cbp-97))
/* (-1)^j / (2j)!, j = 0..15: double-double for j <= 8, double above */
#define LIFE_CR_COS_DD(j)                                                                   \
    ((j) == 0 ? life_dd_make(0x1p+0, 0.0)                                                   \
     : (j) == 1 ? life_dd_make(-0x1p-1, 0.0)                                                \
     : (j) == 2 ? life_dd_make(0x1.5555555555555p-5, 0x1.5555555555555p-59)                 \
     : (j) == 3 ? life_dd_make(-0x1.6c16c16c16c17p-10, 0x1.f49f49f49f49fp-65)               \
     : (j) == 4 ? life_dd_make(0x1.a01a01a01a01ap-16, 0x1.a01a01a01a01ap-76)                \
     : (j) == 5 ? life_dd_make(-0x1.27e4fb7789f5cp-22, -0x1.cbbc05b4fa99ap-76)              \
     : (j) == 6 ? life_dd_make(0x1.1eed8eff8d898p-29, -0x1.2aec959e14c06p-83)               \
     : (j) == 7 ? life_dd_make(-0x1.93974a8c07c9dp-37, -0x1.05d6f8a2efd1fp-92)              \
                : life_dd_make(0x1.ae7f3e733b81fp-45, 0x1.1d8656b0ee8cbp-101))

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
    const double kd = rint(x * 0x1.45f306dc9c883p-1);
    const double t = x - kd * 0x1.921fb54400000p+0; /* exact (Sterbenz; k * piece exact) */
    life_dd r = life_dd_two_sum(t, -(kd * 0x1.0b4611a600000p-34));
    r = life_dd_add_d(r, -(kd * 0x1.3198a2e000000p-69));
    {
        const double ph = kd * 0x1.b839a252049c1p-104;
        const double pl = fma(kd, 0x1.b839a252049c1p-104, -ph);
        r = life_dd_add(r, life_dd_make(-ph, -pl));
    }
    const life_dd z = life_dd_mul(r, r);
    /* sin r = r * sum_j (-1)^j z^j / (2j+1)! */
    double sd = 0x1.259f98b4358adp-103;
    sd = sd * z.h + -0x1.d1ab1c2dccea3p-94;
    sd = sd * z.h + 0x1.3f3ccdd165fa9p-84;
    sd = sd * z.h + -0x1.761b41316381ap-75;
    sd = sd * z.h + 0x1.71b8ef6dcf572p-66;
    sd = sd * z.h + -0x1.2f49b46814157p-57;
    sd = sd * z.h + 0x1.952c77030ad4ap-49;
    life_dd S = life_dd_make(sd, 0.0);
    /* cos r = sum_j (-1)^j z^j / (2j)! */
    double cd = -0x1.3932c5047d60ep-108;
    cd = cd * z.h + 0x1.0a18a2635085dp-98;
    cd = cd * z.h + -0x1.88e85fc6a4e5ap-89;
    cd = cd * z.h + 0x1.f2cf01972f578p-80;
    cd = cd * z.h + -0x1.0ce396db7f853p-70;
    cd = cd * z.h + 0x1.e542ba4020225p-62;
    cd = cd * z.h + -0x1.6827863b97d97p-53;
    life_dd Cp = life_dd_make(cd, 0.0);
    Cp = life_dd_add(life_dd_mul(Cp, z), LIFE_CR_COS_DD(8));
    for (int j = 7; j >= 0; j--) {
        S = life_dd_add(life_dd_mul(S, z), LIFE_CR_SIN_DD(j));
        Cp = life_dd_add(life_dd_mul(Cp, z), LIFE_CR_COS_DD(j));
    }
    const life_dd sn = life_dd_mul(r, S);
    const int q = ((int)kd) & 3;
    const double sr = sn.h, cr = Cp.h;
    *s = q == 0 ? sr : q == 1 ? cr : q == 2 ? -sr : -cr;
    *c = q == 0 ? cr : q == 1 ? -sr : q == 2 ? -cr : sr;
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

/* atan(k/32), k = 0..32, double-double */
LIFE_CR_FN life_dd life_cr_atan_table(int k) {
    switch (k) {
        case 0: return life_dd_make(0.0, 0.0);
        case 1: return life_dd_make(0x1.ffd55bba97625p-6, -0x1.5ec431444912cp-60);
        case 2: return life_dd_make(0x1.ff55bb72cfdeap-5, -0x1.c934d86d23f1dp-60);
        case 3: return life_dd_make(0x1.7ee182602f10fp-4, -0x1.cfb654c0c3d98p-58);
        case 4: return life_dd_make(0x1.fd5ba9aac2f6ep-4, -0x1.cd37686760c17p-59);
        case 5: return life_dd_make(0x1.3d6eee8c6626cp-3, 0x1.61a3b0ce9281bp-57);
        case 6: return life_dd_make(0x1.7b97b4bce5b02p-3, 0x1.347b0b4f881cap-58);
        case 7: return life_dd_make(0x1.b90d7529260a2p-3, 0x1.17b10d2e0e5abp-61);
        case 8: return life_dd_make(0x1.f5b75f92c80ddp-3, 0x1.8ab6e3cf7afbdp-57);
        case 9: return life_dd_make(0x1.18bf5a30bf178p-2, 0x1.30ca4748b1bf9p-57);
        case 10: return life_dd_make(0x1.362773707ebccp-2, -0x1.963a544b672d8p-57);
        case 11: return life_dd_make(0x1.530ad9951cd4ap-2, -0x1.2566480884082p-57);
        case 12: return life_dd_make(0x1.6f61941e4def1p-2, -0x1.c63aae6f6e918p-56);
        case 13: return life_dd_make(0x1.8b24d394a1b25p-2, 0x1.b6d0ba3748fa8p-56);
        case 14: return life_dd_make(0x1.a64eec3cc23fdp-2, -0x1.24dec1b50b7ffp-56);
        case 15: return life_dd_make(0x1.c0db4c94ec9f0p-2, -0x1.cc1ce70934c34p-56);
        case 16: return life_dd_make(0x1.dac670561bb4fp-2, 0x1.a2b7f222f65e2p-56);
        case 17: return life_dd_make(0x1.f40dd0b541418p-2, -0x1.a3992dc382a23p-57);
        case 18: return life_dd_make(0x1.0657e94db30d0p-1, -0x1.d5b495f6349e6p-56);
        case 19: return life_dd_make(0x1.1255d9bfbd2a9p-1, -0x1.2bdaee1c0ee35p-58);
        case 20: return life_dd_make(0x1.1e00babdefeb4p-1, -0x1.928df287a668fp-58);
        case 21: return life_dd_make(0x1.2958e59308e31p-1, -0x1.09e73b0c6c087p-56);
        case 22: return life_dd_make(0x1.345f01cce37bbp-1, 0x1.1021137c71102p-55);
        case 23: return life_dd_make(0x1.3f13fb89e96f4p-1, 0x1.ecf8b492644f0p-56);
        case 24: return life_dd_make(0x1.4978fa3269ee1p-1, 0x1.2419a87f2a458p-56);
        case 25: return life_dd_make(0x1.538f57b89061fp-1, -0x1.1bb74abda520cp-55);
        case 26: return life_dd_make(0x1.5d58987169b18p-1, 0x1.0028e4bc5e7cap-57);
        case 27: return life_dd_make(0x1.66d663923e087p-1, -0x1.6ea6febe8bbbap-56);
        case 28: return life_dd_make(0x1.700a7c5784634p-1, -0x1.8c34d25aadef6p-56);
        case 29: return life_dd_make(0x1.78f6bbd5d315ep-1, 0x1.406a089803740p-55);
        case 30: return life_dd_make(0x1.819d0b7158a4dp-1, -0x1.bf76229d3b917p-56);
        case 31: return life_dd_make(0x1.89ff5ff57f1f8p-1, -0x1.55b9a5e177a1bp-55);
        default: return life_dd_make(0x1.921fb54442d18p-1, 0x1.1a62633145c07p-55);
    }
}

/* (-1)^j / (2j+1), j = 0..10: double-double for j <= 4, double above */
#define LIFE_CR_ATAN_DD(j)                                                      \
    ((j) == 0 ? life_dd_make(0x1p+0, 0.0)                                       \
     : (j) == 1 ? life_dd_make(-0x1.5555555555555p-2, -0x1.5555555555555p-56)   \
     : (j) == 2 ? life_dd_make(0x1.999999999999ap-3, -0x1.999999999999ap-57)    \
     : (j) == 3 ? life_dd_make(-0x1.2492492492492p-3, -0x1.2492492492492p-57)   \
                : life_dd_make(0x1.c71c71c71c71cp-4, 0x1.c71c71c71c71cp-58))

/* atan t for a double-double t in [0, 1] */
LIFE_CR_FN life_dd life_cr_atan01(life_dd t) {
    const int k = (int)rint(t.h * 32.0);
    const double c = (double)k * 0x1p-5;
    const life_dd num = life_dd_add_d(t, -c);
    const life_dd den = life_dd_add_d(life_dd_mul_d(t, c), 1.0);
    const life_dd d = life_dd_div(num, den);
    const life_dd d2 = life_dd_mul(d, d);
    double pd = 0x1.8618618618618p-5;
    pd = pd * d2.h + -0x1.af286bca1af28p-5;
    pd = pd * d2.h + 0x1.e1e1e1e1e1e1ep-5;
    pd = pd * d2.h + -0x1.1111111111111p-4;
    pd = pd * d2.h + 0x1.3b13b13b13b14p-4;
    pd = pd * d2.h + -0x1.745d1745d1746p-4;
    life_dd P = life_dd_make(pd, 0.0);
    for (int j = 4; j >= 0; j--) P = life_dd_add(life_dd_mul(P, d2), LIFE_CR_ATAN_DD(j));
    return life_dd_add(life_cr_atan_table(k), life_dd_mul(d, P));
}

/* atan2(y, x), correctly rounded. */
LIFE_CR_FN double life_cr_atan2(double y, double x) {
    const double PI_H = 0x1.921fb54442d18p+1, PIO2_H = 0x1.921fb54442d18p+0;
    const double PIO4_H = 0x1.921fb54442d18p-1, TPIO4_H = 0x1.2d97c7f3321d2p+1;
    if (isnan(x) || isnan(y)) return x + y;
    const double ax = fabs(x), ay = fabs(y);
    const double sy = signbit(y) ? -1.0 : 1.0;
    /* C99 Annex F.9.1.4 */
    if (ay == 0.0) return (signbit(x) ? PI_H : 0.0) * sy;
    if (isinf(ay)) return (isinf(ax) ? (signbit(x) ? TPIO4_H : PIO4_H) : PIO2_H) * sy;
    if (ax == 0.0) return PIO2_H * sy;
    if (isinf(ax)) return (signbit(x) ? PI_H : 0.0) * sy;
    const int swap = ay > ax;
    const double num = swap ? ax : ay, den = swap ? ay : ax;
    const double qh = num / den;
    if (!(qh >= 0x1p-900)) return atan2(y, x);
    const life_dd t = life_dd_make(qh, fma(-qh, den, num) / den);
    life_dd a = life_cr_atan01(life_dd_fast(t.h, t.l));
    if (swap) a = life_dd_add(life_dd_make(PIO2_H, 0x1.1a62633145c07p-54), life_dd_neg(a));
    if (signbit(x)) a = life_dd_add(life_dd_make(PI_H, 0x1.1a62633145c07p-53), life_dd_neg(a));
    return a.h * sy;
}

#endif /* LIFE_CRTRIG_H */
