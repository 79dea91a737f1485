// ia.cuh -- FP64 interval arithmetic on sm_103a with directed-rounding intrinsics.
//
// Semantics follow the reference's updated interval library
// ("Updated Interval Arithmetic Operations/IA.py" in the GPUGO project):
//   add  IA.py:57-85      minus IA.py:87-115     multiply IA.py:117-152
//   divide IA.py:154-207  power IA.py:209-304    times IA.py:306-333
//   plus IA.py:335-361    sine IA.py:363-446     cosine IA.py:448-530
//   exp  IA.py:532-570
// The reference widens libdevice's sin/cos/pow results by 5 ulp and exp by 2
// ulp through their bit patterns.  The endpoint functions here are this
// project's own (Cody-Waite reduction in double-double, Taylor series; largest
// error measured against mpmath 0.66 ulp for sin/cos and 0.59 ulp for exp, the
// tests bounding it by 1.2 and 1.0 ulp), so the same widening keeps every bound
// rigorous.  Every
// round-to-nearest operation is written as an explicit __d*_rn / __fma_rn call
// so that no contraction changes a rounding: the same sequence, compiled for the
// host in the CPU oracle, yields identical bits.
//
// Deviations from IA.py (all rigour fixes): divide's zero-endpoint branches use
// the correct endpoint, times() handles a negative scalar, the bit-pattern bump
// treats -0.0 as +0.0, exp's lower bound is 0 (not 5e-324) on underflow, and an
// overflowing bump saturates at infinity instead of turning into NaN.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gg {

struct iv { double lo, hi; };

__device__ __forceinline__ iv mk(double lo, double hi) { iv r; r.lo = lo; r.hi = hi; return r; }

__device__ __forceinline__ uint64_t d2u(double x) { return (uint64_t)__double_as_longlong(x); }
__device__ __forceinline__ double u2d(uint64_t u) { return __longlong_as_double((long long)u); }

constexpr uint64_t ABS_MASK = 0x7fffffffffffffffULL;
constexpr uint64_t INF_BITS = 0x7ff0000000000000ULL;
constexpr double INF_D = __builtin_huge_val();

// Comparisons run on the integer bit patterns (an FP64 compare costs as much as
// an FP64 add on this part); each one returns exactly what the IEEE comparison
// returns, NaN and signed-zero cases included.
__device__ __forceinline__ bool isnan_(double x) { return (d2u(x) & ABS_MASK) > INF_BITS; }
__device__ __forceinline__ uint64_t cmpkey(double x) {
  uint64_t u = d2u(x);
  if ((u & ABS_MASK) == 0) u = 0;  // -0 == +0
  return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}
// IEEE a < b
__device__ __forceinline__ bool flt(double a, double b) {
  if (isnan_(a) || isnan_(b)) return false;
  return cmpkey(a) < cmpkey(b);
}
// IEEE a == b
__device__ __forceinline__ bool feq(double a, double b) {
  if (isnan_(a) || isnan_(b)) return false;
  return cmpkey(a) == cmpkey(b);
}
// IEEE a < 0 and a > 0
__device__ __forceinline__ bool fneg(double a) { uint64_t u = d2u(a); return (u >> 63) && (u & ABS_MASK) && !isnan_(a); }
__device__ __forceinline__ bool fpos(double a) { uint64_t u = d2u(a); return !(u >> 63) && (u & ABS_MASK) && !isnan_(a); }

// Python min(a, b) / max(a, b): keep the first unless the second is strictly better.
__device__ __forceinline__ double pmin(double a, double b) { return flt(b, a) ? b : a; }
__device__ __forceinline__ double pmax(double a, double b) { return flt(a, b) ? b : a; }

// Lower bound moved down by k ulps (IA.py:263-281).
__device__ __forceinline__ double bump_lo(double v, int k) {
  if (isnan_(v)) return v;
  uint64_t m = d2u(v) & ABS_MASK;
  if (fneg(v)) {
    if (m + (uint64_t)k >= INF_BITS) return -__longlong_as_double(0x7ff0000000000000LL);
    return -u2d(m + (uint64_t)k);
  }
  if (m < (uint64_t)k) return -u2d((uint64_t)k);
  return u2d(m - (uint64_t)k);
}

// Upper bound moved up by k ulps (IA.py:283-302).
__device__ __forceinline__ double bump_hi(double v, int k) {
  if (isnan_(v)) return v;
  uint64_t m = d2u(v) & ABS_MASK;
  if (fneg(v)) {
    if (m < (uint64_t)k) return u2d((uint64_t)k);
    return -u2d(m - (uint64_t)k);
  }
  if (m + (uint64_t)k >= INF_BITS) return u2d(INF_BITS);
  return u2d(m + (uint64_t)k);
}

// ---------------------------------------------------------------------------
// endpoint functions (round-to-nearest quality)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  double ss = __dadd_rn(a, b);
  double bb = __dsub_rn(ss, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(ss, bb)), __dsub_rn(b, bb));
  s = ss;
}

__constant__ static const double EXP_C[12] = {
    0x1.0000000000000p-1,  0x1.5555555555555p-3,  0x1.5555555555555p-5,
    0x1.1111111111111p-7,  0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13,
    0x1.a01a01a01a01ap-16, 0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22,
    0x1.ae64567f544e4p-26, 0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33};

__device__ __forceinline__ double gg_exp(double x) {
  const double INV_LN2 = 0x1.71547652b82fep+0;
  const double LN2_HI = 0x1.62e42fee00000p-1;
  const double LN2_LO = 0x1.a39ef35793c76p-33;
  if (isnan_(x)) return x;
  if (flt(709.79, x)) return u2d(INF_BITS);
  if (flt(x, -745.2)) return 0.0;
  double k = rint(__dmul_rn(x, INV_LN2));
  double rh = __fma_rn(-k, LN2_HI, x);
  double th = __dmul_rn(k, LN2_LO);
  double tl = __fma_rn(k, LN2_LO, -th);
  double s, e1;
  two_sum(rh, -th, s, e1);
  double e = __dsub_rn(e1, tl);
  double p = EXP_C[11];
#pragma unroll
  for (int i = 10; i >= 0; --i) p = __fma_rn(p, s, EXP_C[i]);
  double s2 = __dmul_rn(s, s);
  double tail = __fma_rn(s2, p, e);
  double hi = __dadd_rn(1.0, s);
  double lo = __dadd_rn(__dsub_rn(1.0, hi), s);
  double y = __dadd_rn(hi, __dadd_rn(lo, tail));
  int ki = (int)k;
  if (ki > 1023) return __dmul_rn(__dmul_rn(y, 0x1p1023), 2.0);
  if (ki >= -1022) return __dmul_rn(y, u2d((uint64_t)(ki + 1023) << 52));
  return __dmul_rn(__dmul_rn(y, u2d((uint64_t)(ki + 600 + 1023) << 52)), 0x1p-600);
}

__constant__ static const double SIN_C[11] = {
    -0x1.5555555555555p-3,  0x1.1111111111111p-7, -0x1.a01a01a01a01ap-13,
     0x1.71de3a556c734p-19, -0x1.ae64567f544e4p-26, 0x1.6124613a86d09p-33,
    -0x1.ae7f3e733b81fp-41, 0x1.952c77030ad4ap-49, -0x1.2f49b46814157p-57,
     0x1.71b8ef6dcf572p-66, -0x1.761b41316381ap-75};
__constant__ static const double COS_C[11] = {
     0x1.5555555555555p-5, -0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-16,
    -0x1.27e4fb7789f5cp-22, 0x1.1eed8eff8d898p-29, -0x1.93974a8c07c9dp-37,
     0x1.ae7f3e733b81fp-45, -0x1.6827863b97d97p-53, 0x1.e542ba4020225p-62,
    -0x1.0ce396db7f853p-70, 0x1.f2cf01972f578p-80};

// x - k*pi/2 as rh + rl; returns k mod 4, or -1 when |x| > 2^22 (or not finite).
__device__ __forceinline__ int trig_reduce(double x, double& rh, double& rl) {
  const double C1 = 0x1.921fb54442d18p+0;
  const double C2 = 0x1.1a62633145c07p-54;
  const double C3 = -0x1.f1976b7ed8fbcp-110;
  const double TWO_OVER_PI = 0x1.45f306dc9c883p-1;
  if (isnan_(x) || (d2u(x) & ABS_MASK) > d2u(0x1p22)) return -1;
  double k = rint(__dmul_rn(x, TWO_OVER_PI));
  double p1h = __dmul_rn(k, C1), p1l = __fma_rn(k, C1, -p1h);
  double p2h = __dmul_rn(k, C2), p2l = __fma_rn(k, C2, -p2h);
  double s0 = __dsub_rn(x, p1h);
  double a, ae, b, be;
  two_sum(s0, -p1l, a, ae);
  two_sum(a, -p2h, b, be);
  double t = __fma_rn(-k, C3, __dsub_rn(__dadd_rn(ae, be), p2l));
  two_sum(b, t, rh, rl);
  long long ki = (long long)k;
  return (int)(((ki % 4) + 4) % 4);
}

__device__ __forceinline__ double sin_core(double rh, double rl) {
  double z = __dmul_rn(rh, rh);
  double p = SIN_C[10];
#pragma unroll
  for (int i = 9; i >= 0; --i) p = __fma_rn(p, z, SIN_C[i]);
  double t = __dmul_rn(rh, z);
  double corr = __fma_rn(t, p, __fma_rn(__dmul_rn(-0.5, z), rl, rl));
  return __dadd_rn(rh, corr);
}

__device__ __forceinline__ double cos_core(double rh, double rl) {
  double z = __dmul_rn(rh, rh);
  double ze = __fma_rn(rh, rh, -z);
  double h = __dmul_rn(0.5, z);
  double w = __dsub_rn(1.0, h);
  double we = __dsub_rn(__dsub_rn(1.0, w), h);
  double p = COS_C[10];
#pragma unroll
  for (int i = 9; i >= 0; --i) p = __fma_rn(p, z, COS_C[i]);
  double q = __dmul_rn(z, z);
  double tail = __fma_rn(q, p, __fma_rn(-rl, rh, __dsub_rn(we, __dmul_rn(0.5, ze))));
  return __dadd_rn(w, tail);
}

__device__ __forceinline__ int gg_sin(double x, double& out) {
  double rh, rl;
  int q = trig_reduce(x, rh, rl);
  if (q < 0) return -1;
  if (q == 0) out = sin_core(rh, rl);
  else if (q == 1) out = cos_core(rh, rl);
  else if (q == 2) out = -sin_core(rh, rl);
  else out = -cos_core(rh, rl);
  return 0;
}

__device__ __forceinline__ int gg_cos(double x, double& out) {
  double rh, rl;
  int q = trig_reduce(x, rh, rl);
  if (q < 0) return -1;
  if (q == 0) out = cos_core(rh, rl);
  else if (q == 1) out = -sin_core(rh, rl);
  else if (q == 2) out = -cos_core(rh, rl);
  else out = sin_core(rh, rl);
  return 0;
}

// ---------------------------------------------------------------------------
// interval operations
// ---------------------------------------------------------------------------
__device__ __forceinline__ iv add(iv a, iv b) { return mk(__dadd_rd(a.lo, b.lo), __dadd_ru(a.hi, b.hi)); }
__device__ __forceinline__ iv minus(iv a, iv b) { return mk(__dadd_rd(a.lo, -b.hi), __dadd_ru(a.hi, -b.lo)); }

__device__ __forceinline__ bool finite_(double x) { return (d2u(x) & ABS_MASK) < INF_BITS; }

// Full form: minimum of the four rounded-down products and maximum of the four
// rounded-up products, in the order IA.py:143-150 lists them.
__device__ __forceinline__ iv mul4(iv a, iv b) {
  double l = __dmul_rd(a.lo, b.lo);
  l = pmin(l, __dmul_rd(a.lo, b.hi));
  l = pmin(l, __dmul_rd(a.hi, b.lo));
  l = pmin(l, __dmul_rd(a.hi, b.hi));
  double h = __dmul_ru(a.lo, b.lo);
  h = pmax(h, __dmul_ru(a.lo, b.hi));
  h = pmax(h, __dmul_ru(a.hi, b.lo));
  h = pmax(h, __dmul_ru(a.hi, b.hi));
  return mk(l, h);
}

// Same result from the signs of the operands: with four finite endpoints the
// extreme products are fixed by the signs, so only those are formed.  With
// a >= 0 or a <= 0 (and the same for b) the order of the four cases below is the
// order of the sign tests; an operand that contains zero in its interior takes
// the other operand's larger-magnitude endpoint for both bounds, and two such
// operands compare the two candidate products of each bound.  Directed rounding
// is monotone, so the rounded extreme product is the extreme rounded product:
// the value returned equals mul4's; only the sign of a zero result can differ,
// which no comparison here distinguishes.  Operands are selected without
// branches so that lanes with different sign cases stay converged.
__device__ __forceinline__ iv mul(iv a, iv b) {
  if (!(finite_(a.lo) && finite_(a.hi) && finite_(b.lo) && finite_(b.hi))) return mul4(a, b);
  const bool a_nn = !fneg(a.lo), a_np = !fpos(a.hi);   // a >= 0, a <= 0
  const bool b_nn = !fneg(b.lo), b_np = !fpos(b.hi);
  const bool a_s = !a_nn && !a_np, b_s = !b_nn && !b_np; // zero in the interior
  if (a_s && b_s) {
    // lo = min(a.lo b.hi, a.hi b.lo), hi = max(a.lo b.lo, a.hi b.hi)
    const double l1 = __dmul_rd(a.lo, b.hi), l2 = __dmul_rd(a.hi, b.lo);
    const double h1 = __dmul_ru(a.lo, b.lo), h2 = __dmul_ru(a.hi, b.hi);
    return mk(pmin(l1, l2), pmax(h1, h2));
  }
  double x1, y1, x2, y2;   // lo = x1 * y1 (down), hi = x2 * y2 (up)
  if (!a_s && !b_s) {
    const bool c1 = a_nn && b_nn, c2 = a_np && b_np, c3 = a_nn && b_np;
    const bool lo_a = c1 || (!c2 && !c3);         // a.lo for (a>=0, b>=0) and (a<=0, b>=0)
    const bool lo_b = c1 || (!c2 && c3);          // b.lo for (a>=0, b>=0) and (a>=0, b<=0)
    x1 = lo_a ? a.lo : a.hi; x2 = lo_a ? a.hi : a.lo;
    y1 = lo_b ? b.lo : b.hi; y2 = lo_b ? b.hi : b.lo;
  } else if (a_s) {
    // b >= 0: [a.lo b.hi, a.hi b.hi]; b <= 0: [a.hi b.lo, a.lo b.lo]
    const double m = b_nn ? b.hi : b.lo;
    x1 = b_nn ? a.lo : a.hi; x2 = b_nn ? a.hi : a.lo;
    y1 = m; y2 = m;
  } else {
    // a >= 0: [a.hi b.lo, a.hi b.hi]; a <= 0: [a.lo b.hi, a.lo b.lo]
    const double m = a_nn ? a.hi : a.lo;
    x1 = m; x2 = m;
    y1 = a_nn ? b.lo : b.hi; y2 = a_nn ? b.hi : b.lo;
  }
  return mk(__dmul_rd(x1, y1), __dmul_ru(x2, y2));
}

__device__ __forceinline__ iv entire() { return mk(-u2d(INF_BITS), u2d(INF_BITS)); }

__device__ __forceinline__ iv div(iv a, iv b) {
  const double INF = u2d(INF_BITS);
  const bool blz = feq(b.lo, 0.0), bhz = feq(b.hi, 0.0);
  const bool alo_ge0 = !isnan_(a.lo) && !fneg(a.lo), ahi_le0 = !isnan_(a.hi) && !fpos(a.hi);
  if (fneg(b.lo) && fpos(b.hi)) return entire();
  if (blz) {
    if (bhz) return entire();
    if (alo_ge0) return mk(__ddiv_rd(a.lo, b.hi), INF);
    if (ahi_le0) return mk(-INF, __ddiv_ru(a.hi, b.hi));
    return entire();
  }
  if (bhz) {
    if (alo_ge0) return mk(-INF, __ddiv_ru(a.lo, b.lo));
    if (ahi_le0) return mk(__ddiv_rd(a.hi, b.lo), INF);
    return entire();
  }
  return mul(a, mk(__drcp_rd(b.hi), __drcp_ru(b.lo)));
}

// The reciprocal interval div(a, b) multiplies by when b does not touch zero
// (div(a, b) == mul(a, div_recip(b)) then); NaN endpoints otherwise.  Tables of
// divisors store it so that the reciprocals are formed once per table entry.
__device__ __forceinline__ iv div_recip(iv b) {
  if ((fneg(b.lo) && fpos(b.hi)) || feq(b.lo, 0.0) || feq(b.hi, 0.0)) return mk(u2d(~0ULL), u2d(~0ULL));
  return mk(__drcp_rd(b.hi), __drcp_ru(b.lo));
}

// power(., 2): x*x rounded to nearest, widened by 5 ulp
__device__ __forceinline__ iv sqr(iv a) {
  double pl = __dmul_rn(a.lo, a.lo), ph = __dmul_rn(a.hi, a.hi);
  if (fneg(a.lo) && fpos(a.hi)) return mk(0.0, bump_hi(pmax(pl, ph), 5));
  return mk(bump_lo(pmin(pl, ph), 5), bump_hi(pmax(pl, ph), 5));
}

// power(., 1/2): correctly rounded sqrt, widened by 5 ulp; negative endpoints clamp to 0
__device__ __forceinline__ iv sqrt_iv(iv a) {
  double l = fneg(a.lo) ? 0.0 : a.lo;
  double h = fneg(a.hi) ? 0.0 : a.hi;
  double pl = __dsqrt_rn(l), ph = __dsqrt_rn(h);
  return mk(bump_lo(pmin(pl, ph), 5), bump_hi(pmax(pl, ph), 5));
}

__device__ __forceinline__ iv times(iv a, double v) {
  if (fneg(v)) return mk(__dmul_rd(a.hi, v), __dmul_ru(a.lo, v));
  return mk(__dmul_rd(a.lo, v), __dmul_ru(a.hi, v));
}

__device__ __forceinline__ iv plus(iv a, double v) { return mk(__dadd_rd(a.lo, v), __dadd_ru(a.hi, v)); }

__device__ __forceinline__ long long floordiv4(long long t) { return (t >= 0) ? t / 4 : -((-t + 3) / 4); }

// floor(x / P) exactly for P > 0 and |x| <= 2^22 (IA.py:430-436 use Python's floor
// division): the product with 1/P is within 2^-30 of x/P, so its floor is off by
// at most one, and the sign of the exact remainder x - t P (one rounding of an
// fma never changes a sign) settles it.
__device__ __forceinline__ long long floor_div(double x, double P, double invP) {
  double t = floor(__dmul_rn(x, invP));
  double r0 = __fma_rn(-t, P, x);
  if (fneg(r0)) {
    t = __dsub_rn(t, 1.0);
  } else {
    double t1 = __dadd_rn(t, 1.0);
    double r1 = __fma_rn(-t1, P, x);
    if (!fneg(r1)) t = t1;
  }
  return (long long)t;
}

__device__ __forceinline__ void quarter_idx(iv a, long long& t1, long long& t2) {
  const double P_UP = 0x1.921fb54442d1ap+0;   // 1.570796326794897 (above pi/2)
  const double P_DN = 0x1.921fb54442d16p+0;   // 1.5707963267948961 (below pi/2)
  const double I_UP = 0x1.45f306dc9c881p-1;   // RN(1/P_UP)
  const double I_DN = 0x1.45f306dc9c884p-1;   // RN(1/P_DN)
  const bool l0 = !fneg(a.lo), h0 = !fneg(a.hi);
  t1 = floor_div(a.lo, l0 ? P_UP : P_DN, l0 ? I_UP : I_DN);
  t2 = floor_div(a.hi, h0 ? P_DN : P_UP, h0 ? I_DN : I_UP);
}

__device__ __forceinline__ iv sin_iv(iv a) {
  double s1, s2;
  if (gg_sin(a.lo, s1) || gg_sin(a.hi, s2)) return mk(-1.0, 1.0);
  double lo = bump_lo(pmin(s1, s2), 5);
  double hi = bump_hi(pmax(s1, s2), 5);
  if (flt(lo, -1.0)) lo = -1;
  if (flt(1.0, hi)) hi = 1;
  long long t1, t2;
  quarter_idx(a, t1, t2);
  if (floordiv4(t1 + 1) != floordiv4(t2 + 1)) lo = -1;
  if (floordiv4(t1 - 1) != floordiv4(t2 - 1)) hi = 1;
  return mk(lo, hi);
}

__device__ __forceinline__ iv cos_iv(iv a) {
  double c1, c2;
  if (gg_cos(a.lo, c1) || gg_cos(a.hi, c2)) return mk(-1.0, 1.0);
  double lo = bump_lo(pmin(c1, c2), 5);
  double hi = bump_hi(pmax(c1, c2), 5);
  if (flt(lo, -1.0)) lo = -1;
  if (flt(1.0, hi)) hi = 1;
  long long t1, t2;
  quarter_idx(a, t1, t2);
  if (floordiv4(t1 + 2) != floordiv4(t2 + 2)) lo = -1;
  if (floordiv4(t1) != floordiv4(t2)) hi = 1;
  return mk(lo, hi);
}

__device__ __forceinline__ iv exp_iv(iv a) {
  double l = gg_exp(a.lo), h = gg_exp(a.hi);
  double lo, hi;
  if (isnan_(l)) lo = l;
  else { uint64_t m = d2u(l); lo = (m < 2) ? 0.0 : u2d(m - 2); }
  if (isnan_(h)) hi = h;
  else { uint64_t m = d2u(h); hi = (m + 2 >= INF_BITS) ? u2d(INF_BITS) : u2d(m + 2); }
  return mk(lo, hi);
}

// Order-preserving map of a double to an unsigned key (atomicMin / argmin).
__device__ __forceinline__ uint64_t ord_key(double x) {
  uint64_t u = d2u(x);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}
__device__ __forceinline__ double ord_val(uint64_t k) {
  return (k >> 63) ? u2d(k & 0x7fffffffffffffffULL) : u2d(~k);
}

}  // namespace gg
