/*
 * gpugo_oracle.c -- CPU oracle for the interval branch-and-bound path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker: the tests, the
 * smoke check and the CPU-baseline leg of bench.py load it; the product
 * (gpugo_gb300/) never links, calls or falls back to it.
 *
 * It restates, in plain C, the algorithm of the GPUGO reference scripts
 * (paths relative to the reference project):
 *   - interval library        "Updated Interval Arithmetic Operations/IA.py"
 *   - box decoder             GPUGO_1.1/1-Ackley/ackley50.py:482-594 (device),
 *                             :820-948 (host completeRegion)
 *   - value / sample / derivative code lists
 *                             GPUGO_1.1/7-Rastrigin/rastrigin50.py:111-372   (family F1)
 *                             GPUGO_1.1/11-Rosenbrock/rosenbrock50.py:116-451 (family F2)
 *                             GPUGO_1.1/1-Ackley/ackley50.py:116-479        (family F3)
 *                             GPUGO_1.1/5-Griewank/griewank50.py:111-433    (family F4)
 *                             any objective as a code list (family 5): the value,
 *                             sample and derivative code lists of e.g.
 *                             GPUGO_1.1/6-Levy/levy50.py:103-563 run by an
 *                             interpreter of the compiled form that
 *                             gpugo_gb300/codelist.py writes
 *   - kernels                 ackley50.py:602-684 (sampling), :686-766 (ruleOutGPU),
 *                             :768-810 (constructFlagArr)
 *   - host B&B loop           ackley50.py:950-1396 (rastrigin50.py:844-1289)
 *   - result-box merging      GPUGO_1.1/11-Rosenbrock/rosenbrock50.py:926-1049
 *                             (combine, connectivity)
 *
 * The reference calls libdevice's dadd_rd/dmul_ru/... (emulated here exactly with
 * error-free transformations and an exact 128-bit slow path) and libdevice's
 * sin/cos/exp/pow (closed source, CUDA 12.8).  In their place this file uses its
 * own functions (Cody-Waite reduction in double-double + Taylor series); their
 * error is below 1.2 ulp, inside the 5-ulp (sin, cos, pow) and 2-ulp (exp)
 * widening the reference applies, so the enclosures stay rigorous.  The CUDA
 * product implements the same functions with the same operation sequence, which
 * makes every bound bit-comparable between this oracle and the GPU.
 *
 * Reference quirks that are NOT reproduced (each is a rigour bug):
 *   IA.py:195,198   divide by a [c,0] interval divides by its zero endpoint
 *   IA.py:188       divide of a non-positive numerator by [0,d] uses the wrong endpoint
 *   IA.py:312       times() assumes a non-negative scalar (scripts pass -0.02, -20)
 *   IA.py:396-404   sine/cosine of -0.0 turn into NaN through the bit-pattern bump
 *   IA.py:562       exp lower bound 5e-324 when exp underflows (0 is the rigorous bound)
 *   ackley50.py:432-469  Ackley gradient overwrites its chain-rule factor and drops 1/n
 * Derived constants that are not exactly representable (1/n, e, 1/sqrt(i), ...)
 * are carried as two-sided enclosures instead of round-to-nearest doubles.
 *
 * Build: see oracle/Makefile (gcc -O2 -ffp-contract=off -fopenmp -shared).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OC_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------------- */
/* bit helpers                                                               */
/* ------------------------------------------------------------------------- */
static inline uint64_t d2u(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double u2d(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
static const uint64_t ABS_MASK = 0x7fffffffffffffffULL;
static const uint64_t INF_BITS = 0x7ff0000000000000ULL;

static inline double next_up(double x) { return nextafter(x, INFINITY); }
static inline double next_dn(double x) { return nextafter(x, -INFINITY); }

/* ------------------------------------------------------------------------- */
/* exact directed rounding (stand-in for libdevice dadd_rd/ru, dmul_rd/ru,   */
/* ddiv_rd/ru, drcp_rd/ru, dsqrt_rd/ru)                                      */
/* ------------------------------------------------------------------------- */
enum { RD = 0, RU = 1 };

/* Round m * 2^q (+ sticky fraction below the last bit of m) to a double. */
static double round_scaled(unsigned __int128 m, int q, int sticky, int neg, int dir)
{
    if (m == 0 && !sticky) return neg ? -0.0 : 0.0;
    int nb = 0;
    { unsigned __int128 t = m; while (t) { nb++; t >>= 1; } }
    int lsb = (nb - 1 + q) - 52;          /* exponent of the last kept bit */
    if (lsb < -1074) lsb = -1074;
    int shift = lsb - q;
    unsigned __int128 kept;
    int inexact = sticky;
    if (shift > 0) {
        if (shift >= 128) { kept = 0; inexact |= (m != 0); }
        else {
            unsigned __int128 mask = (((unsigned __int128)1) << shift) - 1;
            inexact |= ((m & mask) != 0);
            kept = m >> shift;
        }
    } else {
        kept = m << (-shift);              /* exact: value = kept * 2^lsb, kept < 2^53 */
    }
    /* away from zero when the direction asks for it */
    int away = inexact && ((dir == RU && !neg) || (dir == RD && neg));
    if (away) kept += 1;
    if (kept >> 53) { kept >>= 1; lsb += 1; }   /* carry out (exact: low bit was 0) */
    double r;
    if (lsb > 971) r = INFINITY;                 /* beyond DBL_MAX */
    else r = ldexp((double)(uint64_t)kept, lsb);
    if (isinf(r)) {
        /* overflow: directed rounding toward zero stops at DBL_MAX */
        if ((dir == RD && !neg) || (dir == RU && neg)) r = DBL_MAX;
    }
    return neg ? -r : r;
}

static inline void decompose(double x, uint64_t* mant, int* e2)
{
    uint64_t b = d2u(x) & ABS_MASK;
    int be = (int)(b >> 52);
    uint64_t f = b & 0x000fffffffffffffULL;
    if (be == 0) { *mant = f; *e2 = -1074; }
    else { *mant = f | 0x0010000000000000ULL; *e2 = be - 1075; }
}

static inline double add_dir(double a, double b, int dir)
{
    double s = a + b;
    if (!isfinite(s)) {
        if (isnan(s)) return s;
        if (isfinite(a) && isfinite(b)) {           /* finite overflow */
            if (s > 0) return dir == RD ? DBL_MAX : INFINITY;
            return dir == RU ? -DBL_MAX : -INFINITY;
        }
        return s;
    }
    if (s == 0.0) {
        /* exact zero: IEEE sign rules under directed rounding */
        if (a == 0.0 && b == 0.0) {
            int na = signbit(a) != 0, nb = signbit(b) != 0;
            if (dir == RD) return (na || nb) ? -0.0 : 0.0;
            return (na && nb) ? -0.0 : 0.0;
        }
        /* TwoSum error is zero when the sum is exactly zero from opposite operands */
        double bb = s - a;
        double e = (a - (s - bb)) + (b - bb);
        if (e == 0.0) return dir == RD ? -0.0 : 0.0;
        if (e > 0) return dir == RU ? next_up(s) : s;
        return dir == RD ? next_dn(s) : s;
    }
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    if (e > 0 && dir == RU) return next_up(s);
    if (e < 0 && dir == RD) return next_dn(s);
    return s;
}

static double mul_dir(double a, double b, int dir)
{
    double p = a * b;
    if (isnan(p)) return p;
    if (a == 0.0 || b == 0.0 || isinf(a) || isinf(b)) return p;
    if (isinf(p)) {
        if (p > 0) return dir == RD ? DBL_MAX : INFINITY;
        return dir == RU ? -DBL_MAX : -INFINITY;
    }
    if (fabs(p) >= 0x1p-966) {
        double e = fma(a, b, -p);               /* exact product error */
        if (e > 0 && dir == RU) return next_up(p);
        if (e < 0 && dir == RD) return next_dn(p);
        return p;
    }
    uint64_t ma, mb; int ea, eb;
    decompose(a, &ma, &ea); decompose(b, &mb, &eb);
    int neg = (signbit(a) != 0) ^ (signbit(b) != 0);
    return round_scaled((unsigned __int128)ma * mb, ea + eb, 0, neg, dir);
}

static double div_dir(double a, double b, int dir)
{
    double q = a / b;
    if (isnan(q)) return q;
    if (a == 0.0 || isinf(a) || isinf(b) || b == 0.0) return q;
    if (isinf(q)) {
        if (q > 0) return dir == RD ? DBL_MAX : INFINITY;
        return dir == RU ? -DBL_MAX : -INFINITY;
    }
    double aq = fabs(q), aa = fabs(a), ab = fabs(b);
    if (aq >= 0x1p-960 && aq <= 0x1p960 && aa >= 0x1p-960 && ab >= 0x1p-960 && ab <= 0x1p960) {
        double r = fma(-q, b, a);               /* exact remainder a - q*b */
        if (r == 0.0) return q;
        /* sign of (a/b - q) = sign(r) * sign(b) */
        int above = ((r > 0) == (b > 0));       /* true quotient above q */
        if (above && dir == RU) return next_up(q);
        if (!above && dir == RD) return next_dn(q);
        return q;
    }
    uint64_t ma, mb; int ea, eb;
    decompose(a, &ma, &ea); decompose(b, &mb, &eb);
    while (!(ma & 0x0010000000000000ULL)) { ma <<= 1; ea--; }
    while (!(mb & 0x0010000000000000ULL)) { mb <<= 1; eb--; }
    unsigned __int128 num = ((unsigned __int128)ma) << 64;
    unsigned __int128 quo = num / mb, rem = num % mb;
    int neg = (signbit(a) != 0) ^ (signbit(b) != 0);
    return round_scaled(quo, ea - 64 - eb, rem != 0, neg, dir);
}

static inline double sqrt_dir(double x, int dir)
{
    double s = sqrt(x);
    if (!(x > 0) || isinf(x)) return s;
    if (x >= 0x1p-900) {
        double e = fma(s, s, -x);               /* exact: s*s - x */
        if (e > 0 && dir == RD) return next_dn(s);
        if (e < 0 && dir == RU) return next_up(s);
        return s;
    }
    /* tiny x: scale by an even power of two (exact) */
    double t = sqrt_dir(x * 0x1p1000, dir);
    return t * 0x1p-500;
}

#define add_rd(a, b) add_dir((a), (b), RD)
#define add_ru(a, b) add_dir((a), (b), RU)
#define mul_rd(a, b) mul_dir((a), (b), RD)
#define mul_ru(a, b) mul_dir((a), (b), RU)
#define div_rd(a, b) div_dir((a), (b), RD)
#define div_ru(a, b) div_dir((a), (b), RU)
#define rcp_rd(b) div_dir(1.0, (b), RD)
#define rcp_ru(b) div_dir(1.0, (b), RU)

/* ------------------------------------------------------------------------- */
/* own transcendentals (round-to-nearest quality, error < 1.2 ulp)           */
/* ------------------------------------------------------------------------- */
/* Error-free transformations. */
static inline void two_sum(double a, double b, double* s, double* e)
{
    double ss = a + b, bb = ss - a;
    *s = ss; *e = (a - (ss - bb)) + (b - bb);
}

static const double INV_LN2 = 0x1.71547652b82fep+0;
static const double LN2_HI  = 0x1.62e42fee00000p-1;   /* 32 significant bits */
static const double LN2_LO  = 0x1.a39ef35793c76p-33;

/* 1/k! for k = 2..13 (round to nearest) */
static const double EXP_C[12] = {
    0x1.0000000000000p-1,  0x1.5555555555555p-3,  0x1.5555555555555p-5,
    0x1.1111111111111p-7,  0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13,
    0x1.a01a01a01a01ap-16, 0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22,
    0x1.ae64567f544e4p-26, 0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33 };

double oc_exp(double x)
{
    if (isnan(x)) return x;
    if (x > 709.79) return INFINITY;
    if (x < -745.2) return 0.0;
    double k = rint(x * INV_LN2);
    double rh = fma(-k, LN2_HI, x);             /* exact (Sterbenz) */
    double th = k * LN2_LO;
    double tl = fma(k, LN2_LO, -th);
    double s, e1;
    two_sum(rh, -th, &s, &e1);
    double e = e1 - tl;                         /* r = s + e */
    /* p = s^2 * (1/2 + s/6 + ... + s^11/13!) */
    double p = EXP_C[11];
    for (int i = 10; i >= 0; --i) p = fma(p, s, EXP_C[i]);
    double s2 = s * s;
    double tail = fma(s2, p, e);                /* s^2 P(s) + e */
    double hi = 1.0 + s;                        /* exact split of 1 + s */
    double lo = (1.0 - hi) + s;
    double y = hi + (lo + tail);
    int ki = (int)k;
    if (ki > 1023) return (y * 0x1p1023) * 2.0;
    if (ki >= -1022) return y * u2d((uint64_t)(ki + 1023) << 52);
    return (y * u2d((uint64_t)(ki + 600 + 1023) << 52)) * 0x1p-600;
}

/* pi/2 = C1 + C2 + C3 (+5.6e-50) */
static const double PIO2_C1 = 0x1.921fb54442d18p+0;
static const double PIO2_C2 = 0x1.1a62633145c07p-54;
static const double PIO2_C3 = -0x1.f1976b7ed8fbcp-110;
static const double TWO_OVER_PI = 0x1.45f306dc9c883p-1;
static const double TRIG_MAX_ARG = 0x1p22;

/* (-1)^(k+1) / k! for odd k = 3..23 (sine) */
static const double SIN_C[11] = {
    -0x1.5555555555555p-3,  0x1.1111111111111p-7, -0x1.a01a01a01a01ap-13,
     0x1.71de3a556c734p-19, -0x1.ae64567f544e4p-26, 0x1.6124613a86d09p-33,
    -0x1.ae7f3e733b81fp-41, 0x1.952c77030ad4ap-49, -0x1.2f49b46814157p-57,
     0x1.71b8ef6dcf572p-66, -0x1.761b41316381ap-75 };
/* (-1)^(k/2) / k! for even k = 4..24 (cosine tail) */
static const double COS_C[11] = {
     0x1.5555555555555p-5, -0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-16,
    -0x1.27e4fb7789f5cp-22, 0x1.1eed8eff8d898p-29, -0x1.93974a8c07c9dp-37,
     0x1.ae7f3e733b81fp-45, -0x1.6827863b97d97p-53, 0x1.e542ba4020225p-62,
    -0x1.0ce396db7f853p-70, 0x1.f2cf01972f578p-80 };

/* Reduce x to r = rh + rl = x - k*pi/2, returns k mod 4; -1 if out of range. */
static int trig_reduce(double x, double* prh, double* prl)
{
    if (!(fabs(x) <= TRIG_MAX_ARG)) return -1;
    double k = rint(x * TWO_OVER_PI);
    double p1h = k * PIO2_C1, p1l = fma(k, PIO2_C1, -p1h);
    double p2h = k * PIO2_C2, p2l = fma(k, PIO2_C2, -p2h);
    double s0 = x - p1h;                        /* exact (Sterbenz) */
    double a, ae, b, be;
    two_sum(s0, -p1l, &a, &ae);
    two_sum(a, -p2h, &b, &be);
    double t = fma(-k, PIO2_C3, (ae + be) - p2l);
    two_sum(b, t, prh, prl);
    long long ki = (long long)k;
    return (int)(((ki % 4) + 4) % 4);
}

static double sin_core(double rh, double rl)
{
    double z = rh * rh;
    double p = SIN_C[10];
    for (int i = 9; i >= 0; --i) p = fma(p, z, SIN_C[i]);
    double t = rh * z;
    double corr = fma(t, p, fma(-0.5 * z, rl, rl));
    return rh + corr;
}

static double cos_core(double rh, double rl)
{
    double z = rh * rh;
    double ze = fma(rh, rh, -z);
    double h = 0.5 * z;
    double w = 1.0 - h;
    double we = (1.0 - w) - h;
    double p = COS_C[10];
    for (int i = 9; i >= 0; --i) p = fma(p, z, COS_C[i]);
    double q = z * z;
    double tail = fma(q, p, fma(-rl, rh, we - 0.5 * ze));
    return w + tail;
}

/* returns 0 and the value, or -1 when the argument is out of range */
int oc_sin(double x, double* out)
{
    double rh, rl;
    int q = trig_reduce(x, &rh, &rl);
    if (q < 0) return -1;
    double v;
    switch (q) {
        case 0: v = sin_core(rh, rl); break;
        case 1: v = cos_core(rh, rl); break;
        case 2: v = -sin_core(rh, rl); break;
        default: v = -cos_core(rh, rl); break;
    }
    *out = v;
    return 0;
}

int oc_cos(double x, double* out)
{
    double rh, rl;
    int q = trig_reduce(x, &rh, &rl);
    if (q < 0) return -1;
    double v;
    switch (q) {
        case 0: v = cos_core(rh, rl); break;
        case 1: v = -sin_core(rh, rl); break;
        case 2: v = -cos_core(rh, rl); break;
        default: v = sin_core(rh, rl); break;
    }
    *out = v;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* interval library (IA.py)                                                  */
/* ------------------------------------------------------------------------- */
typedef struct { double lo, hi; } iv;

static inline iv mk(double lo, double hi) { iv r = { lo, hi }; return r; }

/* Python's min(a, b) / max(a, b): keep the first unless the second is strictly better. */
static inline double pmin(double a, double b) { return (b < a) ? b : a; }
static inline double pmax(double a, double b) { return (b > a) ? b : a; }

/* Move a lower bound down by k ulps through its bit pattern (IA.py:263-281). */
static double bump_lo(double v, int k)
{
    if (isnan(v)) return v;
    uint64_t m = d2u(v) & ABS_MASK;
    if (v < 0) {
        if (m + (uint64_t)k >= INF_BITS) return -INFINITY;
        return -u2d(m + (uint64_t)k);
    }
    if (m < (uint64_t)k) return -u2d((uint64_t)k);   /* crossed zero: -k * 2^-1074 */
    return u2d(m - (uint64_t)k);
}

/* Move an upper bound up by k ulps (IA.py:283-302). */
static double bump_hi(double v, int k)
{
    if (isnan(v)) return v;
    uint64_t m = d2u(v) & ABS_MASK;
    if (v < 0) {
        if (m < (uint64_t)k) return u2d((uint64_t)k);  /* crossed zero */
        return -u2d(m - (uint64_t)k);
    }
    if (m + (uint64_t)k >= INF_BITS) return INFINITY;
    return u2d(m + (uint64_t)k);
}

/* IA.py:57-85 */
static inline iv ia_add(iv a, iv b) { return mk(add_rd(a.lo, b.lo), add_ru(a.hi, b.hi)); }
/* IA.py:87-115 */
static inline iv ia_minus(iv a, iv b) { return mk(add_rd(a.lo, -b.hi), add_ru(a.hi, -b.lo)); }
/* IA.py:117-152 */
static iv ia_mul(iv a, iv b)
{
    double l = mul_rd(a.lo, b.lo);
    l = pmin(l, mul_rd(a.lo, b.hi));
    l = pmin(l, mul_rd(a.hi, b.lo));
    l = pmin(l, mul_rd(a.hi, b.hi));
    double h = mul_ru(a.lo, b.lo);
    h = pmax(h, mul_ru(a.lo, b.hi));
    h = pmax(h, mul_ru(a.hi, b.lo));
    h = pmax(h, mul_ru(a.hi, b.hi));
    return mk(l, h);
}
/* IA.py:154-207, zero-endpoint branches corrected */
static iv ia_div(iv a, iv b)
{
    if (b.lo < 0 && b.hi > 0) return mk(-INFINITY, INFINITY);
    if (b.lo == 0) {
        if (b.hi == 0) return mk(-INFINITY, INFINITY);
        if (a.lo >= 0) return mk(div_rd(a.lo, b.hi), INFINITY);
        if (a.hi <= 0) return mk(-INFINITY, div_ru(a.hi, b.hi));
        return mk(-INFINITY, INFINITY);
    }
    if (b.hi == 0) {
        if (a.lo >= 0) return mk(-INFINITY, div_ru(a.lo, b.lo));
        if (a.hi <= 0) return mk(div_rd(a.hi, b.lo), INFINITY);
        return mk(-INFINITY, INFINITY);
    }
    return ia_mul(a, mk(rcp_rd(b.hi), rcp_ru(b.lo)));
}
/* IA.py:209-304 with pow = 2; x*x (round to nearest) stands in for pow(x, 2) */
static iv ia_sqr(iv a)
{
    double pl = a.lo * a.lo, ph = a.hi * a.hi;
    if (a.lo < 0 && a.hi > 0) return mk(0.0, bump_hi(pmax(pl, ph), 5));
    return mk(bump_lo(pmin(pl, ph), 5), bump_hi(pmax(pl, ph), 5));
}
/* IA.py:209-304 with pow = 1/2; correctly rounded sqrt stands in for pow(x, 0.5).
 * A lower endpoint below zero (only from the widening of sums of squares) is
 * clamped to zero before the root. */
static iv ia_sqrt(iv a)
{
    double l = a.lo < 0 ? 0.0 : a.lo;
    double h = a.hi < 0 ? 0.0 : a.hi;
    double pl = sqrt(l), ph = sqrt(h);
    return mk(bump_lo(pmin(pl, ph), 5), bump_hi(pmax(pl, ph), 5));
}
/* IA.py:306-333, sign of the scalar handled */
static inline iv ia_times(iv a, double v)
{
    if (v < 0) return mk(mul_rd(a.hi, v), mul_ru(a.lo, v));
    return mk(mul_rd(a.lo, v), mul_ru(a.hi, v));
}
/* IA.py:335-361 */
static inline iv ia_plus(iv a, double v) { return mk(add_rd(a.lo, v), add_ru(a.hi, v)); }

static const double P_UP = 0x1.921fb54442d1ap+0;   /* 1.570796326794897, above pi/2 */
static const double P_DN = 0x1.921fb54442d16p+0;   /* 1.5707963267948961, below pi/2 */

static inline long long floordiv4(long long t) { return (t >= 0) ? t / 4 : -((-t + 3) / 4); }

/* quarter-period indices of the endpoints, widened outward (IA.py:429-436) */
static inline void quarter_idx(iv a, long long* t1, long long* t2)
{
    *t1 = (long long)floor(div_rd(a.lo, a.lo >= 0 ? P_UP : P_DN));
    *t2 = (long long)floor(div_rd(a.hi, a.hi >= 0 ? P_DN : P_UP));
}

/* IA.py:363-446 */
static iv ia_sin(iv a)
{
    double s1, s2;
    if (oc_sin(a.lo, &s1) || oc_sin(a.hi, &s2)) return mk(-1.0, 1.0);
    double lo = bump_lo(pmin(s1, s2), 5);
    double hi = bump_hi(pmax(s1, s2), 5);
    if (lo < -1) lo = -1;
    if (hi > 1) hi = 1;
    long long t1, t2;
    quarter_idx(a, &t1, &t2);
    if (floordiv4(t1 + 1) != floordiv4(t2 + 1)) lo = -1;
    if (floordiv4(t1 - 1) != floordiv4(t2 - 1)) hi = 1;
    return mk(lo, hi);
}
/* IA.py:448-530 */
static iv ia_cos(iv a)
{
    double c1, c2;
    if (oc_cos(a.lo, &c1) || oc_cos(a.hi, &c2)) return mk(-1.0, 1.0);
    double lo = bump_lo(pmin(c1, c2), 5);
    double hi = bump_hi(pmax(c1, c2), 5);
    if (lo < -1) lo = -1;
    if (hi > 1) hi = 1;
    long long t1, t2;
    quarter_idx(a, &t1, &t2);
    if (floordiv4(t1 + 2) != floordiv4(t2 + 2)) lo = -1;
    if (floordiv4(t1) != floordiv4(t2)) hi = 1;
    return mk(lo, hi);
}
/* IA.py:532-570 (lower bound 0 on underflow) */
static iv ia_exp(iv a)
{
    double l = oc_exp(a.lo), h = oc_exp(a.hi);
    double lo, hi;
    if (isnan(l)) lo = l;
    else { uint64_t m = d2u(l); lo = (m < 2) ? 0.0 : u2d(m - 2); }
    if (isnan(h)) hi = h;
    else { uint64_t m = d2u(h); hi = (m + 2 >= INF_BITS) ? INFINITY : u2d(m + 2); }
    return mk(lo, hi);
}

/* ------------------------------------------------------------------------- */
/* problem description                                                       */
/* ------------------------------------------------------------------------- */
enum { FAM_COSQUAD = 1, FAM_CHAINED = 2, FAM_EXPSQRT = 3, FAM_PRODCOS = 4, FAM_CODELIST = 5 };
enum { STOP_WIDTH = 0, STOP_GAP = 1 };

/* Same field layout as gpugo_spec in include/gpugo.h. */
typedef struct {
    int32_t family, n, wid, group, samples, stop_mode;
    double width_tol, gap_tol, ub_init;
    const double* domain;      /* [2n] lo_1, hi_1, ..., lo_n, hi_n */
    const double* coef;
    int64_t ncoef;
    int64_t max_iter;
    int64_t pool_cap;
    int64_t parent_cap;
} oc_spec;

static const double TWO_PI = 0x1.921fb54442d18p+2;     /* 2*math.pi */
static const double E_LO = 0x1.5bf0a8b145769p+1;       /* RN(e) < e */

/* derived constants; every entry is an enclosure of the exact expression */
typedef struct {
    int n;
    /* F1 */
    double *k, *a2, *b, *a;  iv *bk;  iv bsum;
    /* F2 */
    double *p, *q, *p4, *p2, *q2, *m2q; iv *c202;
    /* F3 */
    double A, B; iv inv_n, ape, abn; iv *kn;
    /* F4 */
    iv *rsq, inv_d, inv_d2;
    /* code list: words of the header, sections and instructions; constants */
    const double* clc;
    uint32_t* clw;
    double* store;
    iv* istore;
} consts;

static int cl_parse(const oc_spec* sp, consts* c);

static int consts_init(const oc_spec* sp, consts* c)
{
    int n = sp->n;
    memset(c, 0, sizeof(*c));
    c->n = n;
    c->store = (double*)calloc((size_t)n * 12 + 8, sizeof(double));
    c->istore = (iv*)calloc((size_t)n * 4 + 8, sizeof(iv));
    if (!c->store || !c->istore) return -1;
    double* s = c->store; iv* is = c->istore;
    const double* cf = sp->coef;
    switch (sp->family) {
    case FAM_COSQUAD: {                     /* coef = a[n], b[n], c[n] */
        if (sp->ncoef < 3 * (int64_t)n) return -2;
        c->a = s; c->b = s + n; c->k = s + 2 * n; c->a2 = s + 3 * n; c->bk = is;
        double bl = 0.0, bh = 0.0;
        for (int i = 0; i < n; ++i) {
            c->a[i] = cf[i];
            c->b[i] = cf[n + i];
            c->k[i] = TWO_PI * cf[2 * n + i];
            c->a2[i] = 2.0 * cf[i];
            c->bk[i] = mk(mul_rd(c->b[i], c->k[i]), mul_ru(c->b[i], c->k[i]));
            bl = add_rd(bl, c->b[i]); bh = add_ru(bh, c->b[i]);
        }
        c->bsum = mk(bl, bh);
        break; }
    case FAM_CHAINED: {                     /* coef = p[n-1], q[n-1] */
        if (n < 2 || sp->ncoef < 2 * (int64_t)(n - 1)) return -2;
        c->p = s; c->q = s + n; c->p4 = s + 2 * n; c->p2 = s + 3 * n; c->q2 = s + 4 * n; c->m2q = s + 5 * n;
        c->c202 = is;
        for (int i = 0; i < n - 1; ++i) {
            c->p[i] = cf[i]; c->q[i] = cf[n - 1 + i];
            c->p4[i] = 4.0 * c->p[i]; c->p2[i] = 2.0 * c->p[i];
            c->q2[i] = 2.0 * c->q[i]; c->m2q[i] = -2.0 * c->q[i];
        }
        for (int j = 1; j < n - 1; ++j)
            c->c202[j] = mk(add_rd(c->q2[j], c->p2[j - 1]), add_ru(c->q2[j], c->p2[j - 1]));
        break; }
    case FAM_EXPSQRT: {                     /* coef = A, B, w[n] */
        if (sp->ncoef < 2 + (int64_t)n) return -2;
        c->A = cf[0]; c->B = cf[1];
        if (!(c->A > 0 && c->B > 0)) return -2;
        c->k = s; c->kn = is;
        c->inv_n = mk(div_rd(1.0, (double)n), div_ru(1.0, (double)n));
        c->ape = mk(add_rd(c->A, E_LO), add_ru(c->A, next_up(E_LO)));
        c->abn = mk(div_rd(mul_rd(c->A, c->B), (double)n), div_ru(mul_ru(c->A, c->B), (double)n));
        for (int i = 0; i < n; ++i) {
            c->k[i] = TWO_PI * cf[2 + i];
            c->kn[i] = mk(div_rd(c->k[i], (double)n), div_ru(c->k[i], (double)n));
        }
        break; }
    case FAM_CODELIST:
        return cl_parse(sp, c);
    case FAM_PRODCOS: {                     /* coef = d */
        if (sp->ncoef < 1 || !(cf[0] > 0)) return -2;
        c->rsq = is;
        for (int i = 0; i < n; ++i) {
            double ii = (double)(i + 1);
            c->rsq[i] = mk(rcp_rd(sqrt_dir(ii, RU)), rcp_ru(sqrt_dir(ii, RD)));
        }
        c->inv_d = mk(rcp_rd(cf[0]), rcp_ru(cf[0]));
        c->inv_d2 = mk(2.0 * c->inv_d.lo, 2.0 * c->inv_d.hi);
        break; }
    default:
        return -2;
    }
    return 0;
}

static void consts_free(consts* c) { free(c->store); free(c->istore); free(c->clw); }

/* ------------------------------------------------------------------------- */
/* box decoder (ackley50.py:482-594, :820-948)                               */
/* ------------------------------------------------------------------------- */
typedef struct {
    const double* pbox;   /* parent box [2n] */
    int n, wid, cyc, gsz; /* cyc is 1-based; split coordinates cyc..cyc+gsz-1 */
    uint64_t code;
} child_t;

static inline int group_size(int n, int group, int cyc) { int g = n - cyc + 1; return g < group ? g : group; }

static inline iv child_iv(const child_t* c, int i /* 0-based */)
{
    double lo = c->pbox[2 * i], hi = c->pbox[2 * i + 1];
    int k = i - (c->cyc - 1);
    if (k >= 0 && k < c->gsz) {
        uint64_t d = c->code;
        for (int t = 0; t < k; ++t) d /= (uint64_t)c->wid;
        d %= (uint64_t)c->wid;
        double w = (hi - lo) / (double)c->wid;
        double l2 = w * (double)d + lo;
        double h2 = w * (double)(d + 1) + lo;
        return mk(l2, h2);
    }
    return mk(lo, hi);
}

/* sample point j of a child interval (ackley50.py:288-290) */
static inline double sample_pt(iv x, int S, int j)
{
    double inc = (x.hi - x.lo) / (double)(S + 1);
    return x.lo + inc * (double)(j + 1);
}

/* ------------------------------------------------------------------------- */
/* family 5: compiled code lists (format in gpugo_gb300/codelist.py)           */
/* ------------------------------------------------------------------------- */
enum {
    CL_LDX = 1, CL_LDC, CL_LDI, CL_LDK, CL_LDKI, CL_ADD, CL_MINUS, CL_MUL, CL_DIV, CL_TIMES, CL_PLUS,
    CL_TIMESK, CL_PLUSK, CL_SQR, CL_SQRT, CL_EXP, CL_SIN, CL_COS, CL_MOV, CL_LOOP, CL_ENDLOOP, CL_TRED
};
enum { CL_MAGIC = 0x314C4347u, CL_HEADER = 16, CL_SEC = 12, CL_TAB = 12, CL_INS = 4, CL_MAXREG = 16, CL_MAXTAB = 8 };
#define CL_NONE 0xFFFFFFFFu

/* header words */
enum { H_MAGIC, H_N, H_NREG, H_NINS, H_NCST, H_VS, H_VL, H_PS, H_PL, H_NSEC, H_SKIP, H_RES, H_NTAB };
/* term-table words: a reduction whose body is evaluated per coordinate (TRED) */
enum { T_LO_, T_HI_, T_KIND, T_NOFF, T_OFF0, T_OFF1, T_PAD, T_START, T_LEN, T_REG };

static inline uint32_t cl_u32(double d) { uint64_t u = d2u(d); return (uint32_t)u; }
static inline int cl_hi_zero(double d) { return (d2u(d) >> 32) == 0; }

/* index of base + off; base 0 absolute, 1 loop index i, 2 gradient coordinate j */
static inline long cl_idx(int base, int32_t off, long i, long j)
{
    return (base == 0 ? 0 : base == 1 ? i : j) + (long)off;
}

/* Checks every instruction once, over the ranges its indexes can take, so that
 * the interpreter never reads outside the coordinates, constants or registers.
 * tb (a table body, or NULL): X is read only as X[i + o] for the table's
 * offsets o, i in [lo, hi); no loops and no nested reductions. */
static int cl_check_range(const uint32_t* ins, int nins, int start, int len, int n, int ncst, int nreg,
                          int jlo, int jhi, int allow_j, uint32_t* written, const uint32_t* tb, int ntab,
                          const uint32_t* sec)
{
    /* sec (a tabled gradient section's words, or NULL): X read only as X[j + o]
     * for the section's offsets o; no loops, no reductions */
    long lo = 0, hi = 0;
    int in_loop = 0;
    if (tb) { in_loop = 1; lo = tb[T_LO_]; hi = tb[T_HI_]; }
    if (start < 0 || len < 0 || (long)start + len > nins) return -2;
    for (int p = start; p < start + len; ++p) {
        const uint32_t* w = ins + (size_t)CL_INS * p;
        int op = (int)(w[0] & 255u), d = (int)((w[0] >> 8) & 255u), a = (int)((w[0] >> 16) & 255u),
            b = (int)(w[0] >> 24);
        int32_t i1 = (int32_t)w[1], i2 = (int32_t)w[2];
        int base = -1, size = n;
        long kbase = 0;
        uint32_t reads = 0;
        switch (op) {
        case CL_LDX: base = a; break;
        case CL_LDC: if (i2 < 0 || i2 >= ncst) return -2; break;
        case CL_LDI: if (i2 < 0 || i2 + 1 >= ncst) return -2; break;
        case CL_LDK: case CL_LDKI: base = a; kbase = i2; size = -1; break;
        case CL_TIMESK: case CL_PLUSK:
            base = b; kbase = i2; size = -1;
            if (a >= nreg) return -2;
            reads = 1u << a;
            break;
        case CL_ADD: case CL_MINUS: case CL_MUL: case CL_DIV:
            if (a >= nreg || b >= nreg) return -2;
            reads = (1u << a) | (1u << b);
            break;
        case CL_TIMES: case CL_PLUS: if (i2 < 0 || i2 >= ncst) return -2; /* fall through */
        case CL_SQR: case CL_SQRT: case CL_EXP: case CL_SIN: case CL_COS: case CL_MOV:
            if (a >= nreg) return -2;
            reads = 1u << a;
            break;
        case CL_LOOP:
            if (sec || tb || in_loop || i1 < 0 || i1 >= i2 || i2 > n) return -2;
            in_loop = 1; lo = i1; hi = i2;
            continue;
        case CL_ENDLOOP:
            if (tb || !in_loop) return -2;
            in_loop = 0;
            continue;
        case CL_TRED:
            if (sec || tb || i1 < 0 || i1 >= ntab || a >= nreg) return -2;
            reads = 1u << a;
            break;
        default:
            return -2;
        }
        if (tb && op == CL_LDX) {   /* only X[i + o], o one of the table's offsets */
            uint32_t no = tb[T_NOFF];
            if (a != 1 || !((no > 0 && i1 == (int32_t)tb[T_OFF0]) || (no > 1 && i1 == (int32_t)tb[T_OFF1]))) return -2;
        }
        if (sec && op == CL_LDX) {  /* only X[j + o], o one of the section's offsets */
            int hit = 0;
            for (uint32_t q = 0; q < sec[8]; ++q) hit |= i1 == (int32_t)sec[9 + q];
            if (a != 2 || !hit) return -2;
        }
        if (d >= nreg || (reads & ~*written)) return -2;   /* a register is written before it is read */
        if (base >= 0) {
            long mn, mx;
            if (base == 0) { mn = mx = i1; }
            else if (base == 1) { if (!in_loop) return -2; mn = lo + i1; mx = hi - 1 + i1; }
            else if (base == 2) { if (!allow_j) return -2; mn = jlo + i1; mx = jhi - 1 + i1; }
            else return -2;
            if (mn < 0) return -2;
            if (size > 0) {
                if (mx >= size) return -2;
            } else {
                long per = (op == CL_LDKI) ? 2 : 1;
                if (kbase < 0 || kbase + per * mx + per - 1 >= ncst) return -2;
            }
        }
        *written |= 1u << d;
    }
    return (in_loop && !tb) ? -2 : 0;
}

static int cl_parse(const oc_spec* sp, consts* c)
{
    const double* cf = sp->coef;
    int64_t nc = sp->ncoef;
    if (!cf || nc < CL_HEADER) return -2;
    for (int k = 0; k < CL_HEADER; ++k) if (!cl_hi_zero(cf[k])) return -2;
    uint32_t h[CL_HEADER];
    for (int k = 0; k < CL_HEADER; ++k) h[k] = cl_u32(cf[k]);
    if (h[H_MAGIC] != CL_MAGIC || (int)h[H_N] != sp->n) return -2;
    if (h[H_NREG] < 1 || h[H_NREG] > CL_MAXREG || h[H_NINS] > (1u << 20) || h[H_NCST] > (1u << 26)) return -2;
    if (h[H_NSEC] > (uint32_t)sp->n || h[H_NTAB] > CL_MAXTAB) return -2;
    int64_t nw = CL_HEADER + (int64_t)CL_SEC * h[H_NSEC] + (int64_t)CL_TAB * h[H_NTAB] + (int64_t)CL_INS * h[H_NINS];
    if (nc < nw + (int64_t)h[H_NCST]) return -2;
    uint32_t* w = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)nw);
    if (!w) return -1;
    for (int64_t k = 0; k < nw; ++k) {
        if (!cl_hi_zero(cf[k])) { free(w); return -2; }
        w[k] = cl_u32(cf[k]);
    }
    c->clw = w;
    c->clc = cf + nw;
    const int n = sp->n, nreg = (int)h[H_NREG], nins = (int)h[H_NINS], ncst = (int)h[H_NCST], ntab = (int)h[H_NTAB];
    const uint32_t* tabs = w + CL_HEADER + (size_t)CL_SEC * h[H_NSEC];
    const uint32_t* ins = tabs + (size_t)CL_TAB * ntab;
    for (int t = 0; t < ntab; ++t) {
        const uint32_t* tb = tabs + (size_t)CL_TAB * t;
        const uint32_t no = tb[T_NOFF];
        if (tb[T_LO_] >= tb[T_HI_] || tb[T_HI_] > (uint32_t)n || tb[T_KIND] > 1 || no > 2) return -2;
        for (uint32_t k = 0; k < no; ++k) {
            const long o = (int32_t)tb[T_OFF0 + k];
            if ((long)tb[T_LO_] + o < 0 || (long)tb[T_HI_] - 1 + o >= n) return -2;
        }
        if (no == 2 && tb[T_OFF0] == tb[T_OFF1]) return -2;
        uint32_t wt = 0;
        if (tb[T_REG] >= (uint32_t)nreg) return -2;
        if (cl_check_range(ins, nins, (int)tb[T_START], (int)tb[T_LEN], n, ncst, nreg, 0, 0, 0, &wt, tb, ntab, NULL)) return -2;
        if (!(wt & (1u << tb[T_REG]))) return -2;
    }
    uint32_t wv = 0, wp = 0;
    if (h[H_VL] < 1 || h[H_RES] >= (uint32_t)nreg) return -2;
    if (cl_check_range(ins, nins, (int)h[H_VS], (int)h[H_VL], n, ncst, nreg, 0, 0, 0, &wv, NULL, ntab, NULL)) return -2;
    if (!(wv & (1u << h[H_RES]))) return -2;
    if (cl_check_range(ins, nins, (int)h[H_PS], (int)h[H_PL], n, ncst, nreg, 0, 0, 0, &wp, NULL, ntab, NULL)) return -2;
    if (h[H_SKIP] != CL_NONE && h[H_SKIP] >= (uint32_t)ncst) return -2;
    int prev_hi = 0;
    for (uint32_t s = 0; s < h[H_NSEC]; ++s) {
        const uint32_t* q = w + CL_HEADER + (size_t)CL_SEC * s;
        int lo = (int)q[0], hi = (int)q[1], st = (int)q[2], ln = (int)q[3];
        int32_t chk = (int32_t)q[5];
        uint32_t r = q[4], rs = q[6];
        if (lo < prev_hi || lo >= hi || hi > n) return -2;   /* sections ascend and do not overlap */
        prev_hi = hi;
        if (r >= (uint32_t)nreg || (rs != CL_NONE && rs >= (uint32_t)nreg)) return -2;
        if ((long)lo + chk < 0 || (long)hi - 1 + chk >= n) return -2;
        /* a tabled section: its flag per (j, digits of X[j + o]) is what its code gives */
        if (q[7] > 1) return -2;
        if (q[7]) {
            if (s >= 8 || q[8] < 1 || q[8] > 3) return -2;
            int has_chk = 0;
            for (uint32_t a = 0; a < q[8]; ++a) {
                const long o = (int32_t)q[9 + a];
                if ((long)lo + o < 0 || (long)hi - 1 + o >= n) return -2;
                for (uint32_t b = 0; b < a; ++b) if (q[9 + b] == q[9 + a]) return -2;
                has_chk |= o == chk;
            }
            if (!has_chk || pow((double)sp->wid, (double)q[8]) > 4096.0) return -2;
        }
        uint32_t ws = q[7] ? 0u : wp;   /* tabled sections read nothing from the prologue */
        if (cl_check_range(ins, nins, st, ln, n, ncst, nreg, lo, hi, 1, &ws, NULL, ntab, q[7] ? q : NULL)) return -2;
        if (!(ws & (1u << r)) || (rs != CL_NONE && !(ws & (1u << rs)))) return -2;
    }
    return 0;
}

/* Runs instructions start .. start+len-1; j is the gradient coordinate, i0 the
 * loop index of a table body. */
static void cl_exec(const consts* c, int start, int len, const iv* X, iv* R, long j, long i0)
{
    const uint32_t* h = c->clw;
    const uint32_t* tabs = h + CL_HEADER + (size_t)CL_SEC * h[H_NSEC];
    const uint32_t* ins = tabs + (size_t)CL_TAB * h[H_NTAB];
    const double* K = c->clc;
    long i = i0, hi = 0;
    int body = 0;
    for (int p = start; p < start + len; ++p) {
        const uint32_t* w = ins + (size_t)CL_INS * p;
        const int op = (int)(w[0] & 255u), d = (int)((w[0] >> 8) & 255u), a = (int)((w[0] >> 16) & 255u),
                  b = (int)(w[0] >> 24);
        const int32_t i1 = (int32_t)w[1], i2 = (int32_t)w[2];
        switch (op) {
        case CL_LDX: R[d] = X[cl_idx(a, i1, i, j)]; break;
        case CL_LDC: R[d] = mk(K[i2], K[i2]); break;
        case CL_LDI: R[d] = mk(K[i2], K[i2 + 1]); break;
        case CL_LDK: { double v = K[i2 + cl_idx(a, i1, i, j)]; R[d] = mk(v, v); break; }
        case CL_LDKI: { long k = i2 + 2 * cl_idx(a, i1, i, j); R[d] = mk(K[k], K[k + 1]); break; }
        case CL_ADD: R[d] = ia_add(R[a], R[b]); break;
        case CL_MINUS: R[d] = ia_minus(R[a], R[b]); break;
        case CL_MUL: R[d] = ia_mul(R[a], R[b]); break;
        case CL_DIV: R[d] = ia_div(R[a], R[b]); break;
        case CL_TIMES: R[d] = ia_times(R[a], K[i2]); break;
        case CL_PLUS: R[d] = ia_plus(R[a], K[i2]); break;
        case CL_TIMESK: R[d] = ia_times(R[a], K[i2 + cl_idx(b, i1, i, j)]); break;
        case CL_PLUSK: R[d] = ia_plus(R[a], K[i2 + cl_idx(b, i1, i, j)]); break;
        case CL_SQR: R[d] = ia_sqr(R[a]); break;
        case CL_SQRT: R[d] = ia_sqrt(R[a]); break;
        case CL_EXP: R[d] = ia_exp(R[a]); break;
        case CL_SIN: R[d] = ia_sin(R[a]); break;
        case CL_COS: R[d] = ia_cos(R[a]); break;
        case CL_MOV: R[d] = R[a]; break;
        case CL_LOOP: i = i1; hi = i2; body = p + 1; break;
        case CL_ENDLOOP: if (++i < hi) p = body - 1; break;
        case CL_TRED: {
            /* the loop the table stands for: acc op= body(k) for k in [lo, hi) */
            const uint32_t* tb = tabs + (size_t)CL_TAB * i1;
            iv acc = R[a];
            for (long k = tb[T_LO_]; k < (long)tb[T_HI_]; ++k) {
                iv R2[CL_MAXREG];
                for (int q = 0; q < CL_MAXREG; ++q) R2[q] = mk(0.0, 0.0);
                cl_exec(c, (int)tb[T_START], (int)tb[T_LEN], X, R2, j, k);
                acc = tb[T_KIND] ? ia_mul(acc, R2[tb[T_REG]]) : ia_add(acc, R2[tb[T_REG]]);
            }
            R[d] = acc;
            break;
        }
        }
    }
}

static iv cl_value(const consts* c, const iv* X)
{
    const uint32_t* h = c->clw;
    iv R[CL_MAXREG];
    for (int k = 0; k < CL_MAXREG; ++k) R[k] = mk(0.0, 0.0);
    cl_exec(c, (int)h[H_VS], (int)h[H_VL], X, R, 0, 0);
    return R[h[H_RES]];
}

/* generalized KKT test over every coordinate; 1 = rule out */
static int cl_deriv(const oc_spec* sp, const consts* c, const iv* X)
{
    const uint32_t* h = c->clw;
    const double* dom = sp->domain;
    const int n = sp->n;
    if (h[H_NSEC] == 0) return 0;
    if (h[H_SKIP] != CL_NONE) {
        const double v = c->clc[h[H_SKIP]];
        int all = 1;
        for (int k = 0; k < n; ++k) if (X[k].lo > v || X[k].hi < v) { all = 0; break; }
        if (all) return 0;
    }
    iv R[CL_MAXREG];
    for (int k = 0; k < CL_MAXREG; ++k) R[k] = mk(0.0, 0.0);
    cl_exec(c, (int)h[H_PS], (int)h[H_PL], X, R, 0, 0);
    for (uint32_t s = 0; s < h[H_NSEC]; ++s) {
        const uint32_t* q = h + CL_HEADER + (size_t)CL_SEC * s;
        for (long j = q[0]; j < (long)q[1]; ++j) {
            cl_exec(c, (int)q[2], (int)q[3], X, R, j, 0);
            if (q[6] != CL_NONE) {
                const iv t = R[q[6]];
                if (t.lo == -INFINITY || t.hi == INFINITY) continue;
            }
            const long k = j + (int32_t)q[5];
            const iv d = R[q[4]];
            if (d.lo > 0 && X[k].lo != dom[2 * k]) return 1;
            if (d.hi < 0 && X[k].hi != dom[2 * k + 1]) return 1;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* code lists                                                                */
/* ------------------------------------------------------------------------- */
/* X[i] holds the child's coordinate intervals (degenerate for sample points). */
static iv f_value(const oc_spec* sp, const consts* c, const iv* X)
{
    int n = sp->n;
    switch (sp->family) {
    case FAM_COSQUAD: {                 /* rastrigin50.py:161-188 */
        iv s = mk(0.0, 0.0);
        for (int i = 0; i < n; ++i) {
            iv t1 = ia_times(ia_sqr(X[i]), c->a[i]);
            iv t2 = ia_times(ia_cos(ia_times(X[i], c->k[i])), c->b[i]);
            s = ia_add(s, ia_minus(t1, t2));
        }
        return ia_add(s, c->bsum);
    }
    case FAM_CHAINED: {                 /* rosenbrock50.py:168-198 */
        iv f = mk(0.0, 0.0);
        for (int i = 0; i < n - 1; ++i) {
            iv u = ia_times(ia_sqr(ia_plus(X[i], -1.0)), c->q[i]);
            iv v = ia_times(ia_sqr(ia_minus(ia_sqr(X[i]), X[i + 1])), c->p[i]);
            f = ia_add(f, ia_add(v, u));
        }
        return f;
    }
    case FAM_EXPSQRT: {                 /* ackley50.py:166-212 */
        iv s = mk(0.0, 0.0);
        for (int i = 0; i < n; ++i) s = ia_add(s, ia_sqr(X[i]));
        iv t = ia_sqrt(ia_mul(s, c->inv_n));
        t = ia_times(ia_exp(ia_times(t, -c->B)), -c->A);
        iv cs = mk(0.0, 0.0);
        for (int i = 0; i < n; ++i) cs = ia_add(cs, ia_cos(ia_times(X[i], c->k[i])));
        iv u = ia_exp(ia_mul(cs, c->inv_n));
        return ia_add(ia_minus(t, u), c->ape);
    }
    case FAM_PRODCOS: {                 /* griewank50.py:161-198 */
        iv pr = mk(-1.0, -1.0);
        for (int i = 0; i < n; ++i) pr = ia_mul(pr, ia_cos(ia_mul(X[i], c->rsq[i])));
        iv s = mk(0.0, 0.0);
        for (int i = 0; i < n; ++i) s = ia_add(s, ia_sqr(X[i]));
        s = ia_plus(ia_mul(s, c->inv_d), 1.0);
        return ia_add(s, pr);
    }
    case FAM_CODELIST:
        return cl_value(c, X);
    }
    return mk(NAN, NAN);
}

/* generalized KKT test of one coordinate (rastrigin50.py:365-370) */
static inline int kkt_prune(iv d, iv x, double dlo, double dhi)
{
    if (d.lo > 0 && x.lo != dlo) return 1;
    if (d.hi < 0 && x.hi != dhi) return 1;
    return 0;
}

static int f_deriv(const oc_spec* sp, const consts* c, const iv* X)
{
    int n = sp->n;
    const double* dom = sp->domain;
    switch (sp->family) {
    case FAM_CODELIST:
        return cl_deriv(sp, c, X);
    case FAM_COSQUAD:                   /* rastrigin50.py:340-372 */
        for (int j = 0; j < n; ++j) {
            iv d = ia_times(X[j], c->a2[j]);
            iv h = ia_mul(ia_sin(ia_times(X[j], c->k[j])), c->bk[j]);
            d = ia_add(d, h);
            if (kkt_prune(d, X[j], dom[2 * j], dom[2 * j + 1])) return 1;
        }
        return 0;
    case FAM_CHAINED:                   /* rosenbrock50.py:367-451 */
        for (int j = 0; j < n; ++j) {
            iv d;
            if (j == 0) {
                d = ia_times(ia_plus(X[0], -1.0), c->q2[0]);
                iv t = ia_times(ia_mul(ia_minus(ia_sqr(X[0]), X[1]), X[0]), c->p4[0]);
                d = ia_add(d, t);
            } else if (j == n - 1) {
                d = ia_times(ia_minus(X[n - 1], ia_sqr(X[n - 2])), c->p2[n - 2]);
            } else {
                d = ia_times(ia_minus(ia_sqr(X[j]), X[j + 1]), c->p4[j]);
                d = ia_add(d, c->c202[j]);
                d = ia_plus(ia_mul(d, X[j]), c->m2q[j]);
                iv t = ia_times(ia_sqr(X[j - 1]), c->p2[j - 1]);
                d = ia_minus(d, t);
            }
            if (kkt_prune(d, X[j], dom[2 * j], dom[2 * j + 1])) return 1;
        }
        return 0;
    case FAM_EXPSQRT: {                 /* ackley50.py:393-479 (gradient corrected) */
        int origin = 1;
        for (int i = 0; i < n; ++i) if (X[i].lo > 0 || X[i].hi < 0) { origin = 0; break; }
        if (origin) return 0;
        iv s = mk(0.0, 0.0);
        for (int i = 0; i < n; ++i) s = ia_add(s, ia_sqr(X[i]));
        iv r = ia_sqrt(ia_mul(s, c->inv_n));
        iv g = ia_exp(ia_times(r, -c->B));
        g = ia_mul(ia_div(g, r), c->abn);
        iv cs = mk(0.0, 0.0);
        for (int i = 0; i < n; ++i) cs = ia_add(cs, ia_cos(ia_times(X[i], c->k[i])));
        iv u = ia_exp(ia_mul(cs, c->inv_n));
        for (int j = 0; j < n; ++j) {
            iv d = ia_mul(g, X[j]);
            iv h = ia_mul(ia_mul(ia_sin(ia_times(X[j], c->k[j])), u), c->kn[j]);
            d = ia_add(d, h);
            if (kkt_prune(d, X[j], dom[2 * j], dom[2 * j + 1])) return 1;
        }
        return 0;
    }
    case FAM_PRODCOS: {                 /* griewank50.py:372-433 */
        iv P = mk(1.0, 1.0);
        for (int i = 0; i < n; ++i) P = ia_mul(P, ia_cos(ia_mul(X[i], c->rsq[i])));
        for (int j = 0; j < n; ++j) {
            iv a = ia_mul(X[j], c->rsq[j]);
            iv q = ia_div(P, ia_cos(a));
            q = ia_mul(ia_mul(q, ia_sin(a)), c->rsq[j]);
            q = ia_add(q, ia_mul(X[j], c->inv_d2));
            if (kkt_prune(q, X[j], dom[2 * j], dom[2 * j + 1])) return 1;
        }
        return 0;
    }
    }
    return 0;
}

/* per-child evaluation: LB (value code list), smallest sampled upper bound
 * (sample code list, ackley50.py:222-352) and the derivative flag */
typedef struct { double lb, samp; int deriv; } child_eval;

static void eval_child(const oc_spec* sp, const consts* c, const child_t* ch, iv* X, iv* Xs,
                       int want_samp, int want_deriv, child_eval* out)
{
    int n = sp->n;
    for (int i = 0; i < n; ++i) X[i] = child_iv(ch, i);
    out->lb = f_value(sp, c, X).lo;
    out->samp = INFINITY;
    if (want_samp) {
        double best = 0.0;
        for (int j = 0; j < sp->samples; ++j) {
            for (int i = 0; i < n; ++i) { double x = sample_pt(X[i], sp->samples, j); Xs[i] = mk(x, x); }
            double fh = f_value(sp, c, Xs).hi;
            if (j == 0 || best > fh) best = fh;
        }
        out->samp = best;
    }
    out->deriv = want_deriv ? f_deriv(sp, c, X) : 0;
}

static int validate(const oc_spec* sp)
{
    if (sp->n < 1 || sp->n > 16384) return -2;
    if (sp->wid < 2 || sp->group < 1 || sp->samples < 1 || sp->samples > 255) return -2;  /* 8-bit sample index */
    if (sp->stop_mode != STOP_WIDTH && sp->stop_mode != STOP_GAP) return -2;
    if (!sp->domain) return -2;
    int g = sp->group < sp->n ? sp->group : sp->n;
    double m = pow((double)sp->wid, (double)g);
    if (m > 4294967296.0) return -2;
    for (int i = 0; i < sp->n; ++i) if (!(sp->domain[2 * i] < sp->domain[2 * i + 1])) return -2;
    return 0;
}

static inline uint64_t n_children(const oc_spec* sp, int cyc)
{
    int g = group_size(sp->n, sp->group, cyc);
    uint64_t m = 1;
    for (int i = 0; i < g; ++i) m *= (uint64_t)sp->wid;
    return m;
}

/* ------------------------------------------------------------------------- */
/* exported single-op entry points (for the interval-library tests)          */
/* ------------------------------------------------------------------------- */
enum { OP_ADD = 0, OP_MINUS, OP_MUL, OP_DIV, OP_SQR, OP_SQRT, OP_TIMES, OP_PLUS, OP_SIN, OP_COS, OP_EXP };

OC_API void oc_ia_op(int op, long m, const double* a, const double* b, double* out)
{
    for (long t = 0; t < m; ++t) {
        iv x = mk(a[2 * t], a[2 * t + 1]);
        iv y = b ? mk(b[2 * t], b[2 * t + 1]) : mk(0, 0);
        iv r;
        switch (op) {
            case OP_ADD: r = ia_add(x, y); break;
            case OP_MINUS: r = ia_minus(x, y); break;
            case OP_MUL: r = ia_mul(x, y); break;
            case OP_DIV: r = ia_div(x, y); break;
            case OP_SQR: r = ia_sqr(x); break;
            case OP_SQRT: r = ia_sqrt(x); break;
            case OP_TIMES: r = ia_times(x, y.lo); break;
            case OP_PLUS: r = ia_plus(x, y.lo); break;
            case OP_SIN: r = ia_sin(x); break;
            case OP_COS: r = ia_cos(x); break;
            case OP_EXP: r = ia_exp(x); break;
            default: r = mk(NAN, NAN);
        }
        out[2 * t] = r.lo; out[2 * t + 1] = r.hi;
    }
}

/* directed scalar ops: op 0 add, 1 mul, 2 div, 3 sqrt; dir 0 down, 1 up */
OC_API void oc_round_op(int op, int dir, long m, const double* a, const double* b, double* out)
{
    for (long t = 0; t < m; ++t) {
        switch (op) {
            case 0: out[t] = add_dir(a[t], b[t], dir); break;
            case 1: out[t] = mul_dir(a[t], b[t], dir); break;
            case 2: out[t] = div_dir(a[t], b[t], dir); break;
            case 3: out[t] = sqrt_dir(a[t], dir); break;
            default: out[t] = NAN;
        }
    }
}

/* point functions: 0 exp, 1 sin, 2 cos (NaN when out of range) */
OC_API void oc_point_fn(int fn, long m, const double* x, double* out)
{
    for (long t = 0; t < m; ++t) {
        double v = NAN;
        if (fn == 0) v = oc_exp(x[t]);
        else if (fn == 1) { if (oc_sin(x[t], &v)) v = NAN; }
        else if (fn == 2) { if (oc_cos(x[t], &v)) v = NAN; }
        out[t] = v;
    }
}

/* child interval of coordinate i (0-based), completeRegion semantics */
OC_API int oc_child_box(const oc_spec* sp, const double* pbox, int cyc, uint64_t code, double* out)
{
    int rc = validate(sp);
    if (rc) return rc;
    child_t ch = { pbox, sp->n, sp->wid, cyc, group_size(sp->n, sp->group, cyc), code };
    for (int i = 0; i < sp->n; ++i) { iv x = child_iv(&ch, i); out[2 * i] = x.lo; out[2 * i + 1] = x.hi; }
    return 0;
}

/* Evaluate m children of one parent: lb, smallest sampled upper bound, and the
 * ruleOutGPU flag (value test against ub, then derivative test). */
OC_API int oc_eval_children(const oc_spec* sp, const double* pbox, int cyc, const uint64_t* codes, long m,
                            double ub, double* lb, double* samp, int32_t* flag, int32_t* dflag)
{
    int rc = validate(sp);
    if (rc) return rc;
    consts c;
    if ((rc = consts_init(sp, &c))) { consts_free(&c); return rc; }
    int n = sp->n;
    int gsz = group_size(n, sp->group, cyc);
    #pragma omp parallel
    {
        iv* X = (iv*)malloc(sizeof(iv) * (size_t)n * 2);
        iv* Xs = X + n;
        #pragma omp for schedule(static)
        for (long t = 0; t < m; ++t) {
            child_t ch = { pbox, n, sp->wid, cyc, gsz, codes[t] };
            child_eval e;
            eval_child(sp, &c, &ch, X, Xs, 1, 1, &e);
            lb[t] = e.lb; samp[t] = e.samp;
            int f = (e.lb > ub);
            if (dflag) dflag[t] = e.deriv;
            flag[t] = f ? 1 : e.deriv;
        }
        free(X);
    }
    consts_free(&c);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* the branch-and-bound driver (ackley50.py:950-1396)                        */
/* ------------------------------------------------------------------------- */
typedef struct {
    double lb, ub;
    int64_t n_boxes;         /* output boxes (width rule) + remaining pool (gap mode) */
    int64_t iterations;      /* expansions (the reference's `iter`) */
    int64_t boxes_bounded;   /* children bounded */
    int64_t pool_size;       /* live list entries at exit */
    int32_t status;          /* 0 certified/finished, 1 iteration limit, <0 error */
    int32_t n_out;           /* boxes written to boxes_out */
    int64_t samples_evaluated;
} oc_result;

typedef struct {
    int64_t cap;             /* entries available in each array */
    double* ub;              /* UB after the sampling step */
    int64_t* n_surv;         /* survivors appended */
    int64_t* pool;           /* live list length after the update */
    int64_t* sel;            /* (parent << 32 | code) of the next parent, -1 at exit */
} oc_trace;

typedef struct { double lb; uint32_t parent; uint32_t code; } entry;

static inline int entry_less(const entry* a, const entry* b)
{
    if (a->lb != b->lb) return a->lb < b->lb;
    if (a->parent != b->parent) return a->parent < b->parent;
    return a->code < b->code;
}

static int cmp_entry(const void* x, const void* y)
{
    const entry* a = (const entry*)x; const entry* b = (const entry*)y;
    if (entry_less(a, b)) return -1;
    if (entry_less(b, a)) return 1;
    return 0;
}

/* mode bit 0: skip sampling children whose LB already exceeds the running UB
 * (their samples cannot lower it; the result is identical). */
OC_API int oc_solve(const oc_spec* sp, int mode, oc_result* res, double* boxes_out, double* lbs_out,
                    int64_t cap, oc_trace* tr)
{
    memset(res, 0, sizeof(*res));
    int rc = validate(sp);
    if (rc) { res->status = rc; return rc; }
    consts c;
    if ((rc = consts_init(sp, &c))) { consts_free(&c); res->status = rc; return rc; }
    const int n = sp->n, g = sp->group;
    const int max_cyc = 1 + g * ((n - 1) / g);
    int64_t max_iter = sp->max_iter > 0 ? sp->max_iter : INT64_MAX;
    int skip = mode & 1;

    /* parent table: region_list (ackley50.py:971) */
    int64_t pcap = 64;
    double* parents = (double*)malloc(sizeof(double) * 2 * n * pcap);
    int32_t* pcyc = (int32_t*)malloc(sizeof(int32_t) * pcap);
    memcpy(parents, sp->domain, sizeof(double) * 2 * n);
    pcyc[0] = 1;

    int64_t lcap = 1024, L = 0;
    entry* list = (entry*)malloc(sizeof(entry) * lcap);
    uint64_t mmax = n_children(sp, 1);
    for (int cy = 1; cy <= max_cyc; cy += g) { uint64_t mm = n_children(sp, cy); if (mm > mmax) mmax = mm; }
    double* clb = (double*)malloc(sizeof(double) * mmax);
    int8_t* ckeep = (int8_t*)malloc(mmax);

    int64_t n_out = 0, out_cap = cap;
    double out_lb_min = INFINITY;
    double UB = sp->ub_init;
    if (UB == 0.0) UB = 0.0;  /* normalise -0 */
    int64_t iter = 0, cur = 0;  /* cur: index of the selected region in the parent table */
    int status = 0;

    for (;;) {
        if (iter >= max_iter) { status = 1; break; }
        const double* pbox = parents + 2 * n * cur;
        int cyc = pcyc[cur];
        int gsz = group_size(n, g, cyc);
        uint64_t M = n_children(sp, cyc);
        double ub_prev = UB;

        /* Step 1: sampling kernel (ackley50.py:602-684): UB <- min(UB, min samples) */
        /* Step 2: ruleOutGPU (ackley50.py:686-766) needs the final UB, so the
         * children are bounded first and pruned in a second sweep. */
        double ub_run = UB;
        int64_t nsamp = 0;
        #pragma omp parallel reduction(+:nsamp)
        {
            iv* X = (iv*)malloc(sizeof(iv) * (size_t)n * 2);
            iv* Xs = X + n;
            double local = INFINITY;
            #pragma omp for schedule(dynamic, 256)
            for (uint64_t code = 0; code < M; ++code) {
                child_t ch = { pbox, n, sp->wid, cyc, gsz, code };
                child_eval e;
                for (int i = 0; i < n; ++i) X[i] = child_iv(&ch, i);
                e.lb = f_value(sp, &c, X).lo;
                clb[code] = e.lb;
                int want = 1;
                if (skip) {
                    double cur_ub;
                    #pragma omp atomic read
                    cur_ub = ub_run;
                    want = (e.lb <= cur_ub) && (e.lb <= local);
                }
                if (want) {
                    double best = 0.0;
                    for (int j = 0; j < sp->samples; ++j) {
                        for (int i = 0; i < n; ++i) { double x = sample_pt(X[i], sp->samples, j); Xs[i] = mk(x, x); }
                        double fh = f_value(sp, &c, Xs).hi;
                        if (j == 0 || best > fh) best = fh;
                    }
                    nsamp++;
                    if (best < local) {
                        local = best;
                        if (skip) {
                            #pragma omp critical
                            { if (local < ub_run) ub_run = local; }
                        }
                    }
                }
            }
            #pragma omp critical
            { if (local < ub_run) ub_run = local; }
            free(X);
        }
        if (ub_run < UB) UB = ub_run;
        if (UB == 0.0) UB = 0.0;
        res->samples_evaluated += nsamp;

        /* value test + derivative test, survivors in ascending child code */
        #pragma omp parallel
        {
            iv* X = (iv*)malloc(sizeof(iv) * (size_t)n);
            #pragma omp for schedule(dynamic, 256)
            for (uint64_t code = 0; code < M; ++code) {
                int keep = 0;
                if (!(clb[code] > UB)) {
                    child_t ch = { pbox, n, sp->wid, cyc, gsz, code };
                    for (int i = 0; i < n; ++i) X[i] = child_iv(&ch, i);
                    keep = !f_deriv(sp, &c, X);
                }
                ckeep[code] = (int8_t)keep;
            }
            free(X);
        }
        res->boxes_bounded += (int64_t)M;

        /* Step 3: list rule-out when UB changed (ackley50.py:1154-1166, :1193-1220) */
        if (iter > 0 && UB != ub_prev && L > 0) {
            int64_t w = 0;
            for (int64_t i = 0; i < L; ++i) if (!(list[i].lb > UB)) list[w++] = list[i];
            L = w;
        }
        /* append survivors (ackley50.py:1234-1242) */
        int64_t ns = 0;
        for (uint64_t code = 0; code < M; ++code) {
            if (!ckeep[code]) continue;
            if (L == lcap) { lcap *= 2; list = (entry*)realloc(list, sizeof(entry) * lcap); }
            entry e = { clb[code] == 0.0 ? 0.0 : clb[code], (uint32_t)cur, (uint32_t)code };
            list[L++] = e;
            ns++;
        }
        if (tr && iter < tr->cap) { tr->ub[iter] = UB; tr->n_surv[iter] = ns; tr->pool[iter] = L; tr->sel[iter] = -1; }
        int64_t it_done = iter;
        iter++;

        /* Step 4: selection (ackley50.py:1269-1370).  The parent table grows
         * first: the child box below points into it. */
        if (iter >= pcap) {
            pcap *= 2;
            parents = (double*)realloc(parents, sizeof(double) * 2 * n * pcap);
            pcyc = (int32_t*)realloc(pcyc, sizeof(int32_t) * pcap);
        }
        int found = 0, terminate = 0;
        while (!found) {
            if (L == 0) { terminate = 1; break; }
            int64_t k = 0;
            for (int64_t i = 1; i < L; ++i) if (entry_less(&list[i], &list[k])) k = i;
            if (sp->stop_mode == STOP_GAP) {
                double lbstar = list[k].lb < out_lb_min ? list[k].lb : out_lb_min;
                if (UB - lbstar <= sp->gap_tol) { terminate = 1; break; }
            }
            entry e = list[k];
            memmove(list + k, list + k + 1, sizeof(entry) * (size_t)(L - k - 1));
            L--;
            int ccyc = pcyc[e.parent];
            child_t ch = { parents + 2 * n * e.parent, n, sp->wid, ccyc, group_size(n, g, ccyc), e.code };
            iv x0 = child_iv(&ch, 0);
            double width = x0.hi - x0.lo;
            if (width < sp->width_tol && ccyc == max_cyc) {
                if (n_out < out_cap) {
                    for (int i = 0; i < n; ++i) { iv x = child_iv(&ch, i); boxes_out[2 * n * n_out + 2 * i] = x.lo; boxes_out[2 * n * n_out + 2 * i + 1] = x.hi; }
                    if (lbs_out) lbs_out[n_out] = e.lb;
                }
                n_out++;
                if (e.lb < out_lb_min) out_lb_min = e.lb;
                continue;
            }
            found = 1;
            for (int i = 0; i < n; ++i) { iv x = child_iv(&ch, i); parents[2 * n * iter + 2 * i] = x.lo; parents[2 * n * iter + 2 * i + 1] = x.hi; }
            pcyc[iter] = (ccyc == max_cyc) ? 1 : ccyc + g;
            cur = iter;
            if (tr && it_done < tr->cap) tr->sel[it_done] = ((int64_t)e.parent << 32) | e.code;
        }
        if (terminate) break;
        if (sp->parent_cap > 0 && iter >= sp->parent_cap) { status = -5; break; }
        if (sp->pool_cap > 0 && L > sp->pool_cap) { status = -4; break; }
    }

    /* enclosure: [min(outputValLower), UB] (ackley50.py:1387); gap mode adds the list */
    double lbstar = out_lb_min;
    for (int64_t i = 0; i < L; ++i) if (list[i].lb < lbstar) lbstar = list[i].lb;
    res->lb = lbstar;
    res->ub = UB;
    res->iterations = iter;
    res->pool_size = L;
    res->status = status;
    int64_t total = n_out;
    if (sp->stop_mode == STOP_GAP && L > 0) {
        qsort(list, (size_t)L, sizeof(entry), cmp_entry);
        for (int64_t i = 0; i < L; ++i, ++total) {
            if (total >= out_cap) continue;
            const entry* e = &list[i];
            int ccyc = pcyc[e->parent];
            child_t ch = { parents + 2 * n * e->parent, n, sp->wid, ccyc, group_size(n, g, ccyc), e->code };
            for (int j = 0; j < n; ++j) { iv x = child_iv(&ch, j); boxes_out[2 * n * total + 2 * j] = x.lo; boxes_out[2 * n * total + 2 * j + 1] = x.hi; }
            if (lbs_out) lbs_out[total] = e->lb;
        }
    }
    res->n_boxes = total;
    res->n_out = (int32_t)(total < out_cap ? total : out_cap);
    free(parents); free(pcyc); free(list); free(clb); free(ckeep);
    consts_free(&c);
    return 0;
}

/* Result-box merging, in order (rosenbrock50.py:926-985 combine, :987-1049
 * connectivity).  A new box joins the first root it is connected to: in every
 * coordinate it lies inside the root, or |new.lo - root.hi| < tol and
 * |new.hi - new.lo| < tol (the reference's second difference is the new box's own
 * width); the root becomes the coordinate-wise hull.  Otherwise the box becomes a
 * new root.  Returns the number of roots (roots_out holds the first cap). */
static int connected(const double* root, const double* nb, int n, double tol)
{
    for (int i = 0; i < n; ++i) {
        double rl = root[2 * i], rh = root[2 * i + 1], nl = nb[2 * i], nh = nb[2 * i + 1];
        if (rl <= nl && nl <= rh && rl <= nh && nh <= rh) continue;
        if (!(fabs(nl - rh) < tol)) return 0;
        if (!(fabs(nh - nl) < tol)) return 0;
    }
    return 1;
}

OC_API int64_t oc_combine(const double* boxes, int64_t nbox, int n, double tol, double* roots_out, int64_t cap)
{
    double* roots = (double*)malloc(sizeof(double) * 2 * (size_t)n * (size_t)(nbox > 0 ? nbox : 1));
    int64_t nr = 0;
    for (int64_t b = 0; b < nbox; ++b) {
        const double* nb = boxes + 2 * (int64_t)n * b;
        int64_t hit = -1;
        for (int64_t r = 0; r < nr && hit < 0; ++r)
            if (connected(roots + 2 * (int64_t)n * r, nb, n, tol)) hit = r;
        double* dst = roots + 2 * (int64_t)n * (hit < 0 ? nr : hit);
        if (hit < 0) {
            memcpy(dst, nb, sizeof(double) * 2 * (size_t)n);
            ++nr;
        } else {
            /* np.minimum(root, new) / np.maximum(root, new): the root's value
               only when it is strictly better (no NaN here) */
            for (int i = 0; i < n; ++i) {
                if (!(dst[2 * i] < nb[2 * i])) dst[2 * i] = nb[2 * i];
                if (!(dst[2 * i + 1] > nb[2 * i + 1])) dst[2 * i + 1] = nb[2 * i + 1];
            }
        }
    }
    int64_t k = nr < cap ? nr : cap;
    if (k > 0) memcpy(roots_out, roots, sizeof(double) * 2 * (size_t)n * (size_t)k);
    free(roots);
    return nr;
}

OC_API int oc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
