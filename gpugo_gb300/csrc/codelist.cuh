// codelist.cuh -- device interpreter of compiled objective code lists (family 5).
//
// The reference writes each objective as hand-made code lists of interval
// operations: value (e.g. GPUGO_1.1/6-Levy/levy50.py:141-226), sample (the same
// list on the diagonal points, :235-379) and derivative (:382-563).  A compiled
// code list (format written by gpugo_gb300/codelist.py, checked by the host
// before admission) holds the same operations as instructions over a small
// file of interval registers; this file runs them for one child box.
//
// Coordinates come from a per-iteration table, like the term tables of the
// built-in families: entry (i, digit) holds the child interval of coordinate i
// (T_LO, two doubles) and its S sample points (T_SHI).  Reductions whose terms
// read only X[i + o] (instruction TRED) have their own tables: every term for
// every coordinate, digit combination and sample pass is evaluated once per
// iteration, and a child adds (multiplies) its entries in the loop's order.
//
// Every instruction is one operation of ia.cuh applied in the order written,
// so every bound is the one the oracle's interpreter computes, bit for bit.
#pragma once

namespace gg {

enum {
  CL_LDX = 1, CL_LDC, CL_LDI, CL_LDK, CL_LDKI, CL_ADD, CL_MINUS, CL_MUL, CL_DIV, CL_TIMES, CL_PLUS,
  CL_TIMESK, CL_PLUSK, CL_SQR, CL_SQRT, CL_EXP, CL_SIN, CL_COS, CL_MOV, CL_LOOP, CL_ENDLOOP, CL_TRED
};
enum { CL_HEADER = 16, CL_SEC = 12, CL_TAB = 12, CL_INS = 4, CL_MAXREG = 16, CL_MAXTAB = 8 };
enum { CLH_MAGIC, CLH_N, CLH_NREG, CLH_NINS, CLH_NCST, CLH_VS, CLH_VL, CLH_PS, CLH_PL, CLH_NSEC, CLH_SKIP, CLH_RES,
       CLH_NTAB };
// term-table words
enum { CLT_LO, CLT_HI, CLT_KIND, CLT_NOFF, CLT_OFF0, CLT_OFF1, CLT_PAD, CLT_START, CLT_LEN, CLT_REG };
// gradient-section words
enum { CLS_LO, CLS_HI, CLS_START, CLS_LEN, CLS_REG, CLS_CHK, CLS_SKIP, CLS_TABLED, CLS_NOFF, CLS_OFF0 };
constexpr int CL_FLAG_TABLES = 8;   // Desc::cl_toff[8 + s]: KKT flags of tabled section s
constexpr unsigned CL_NONE = 0xFFFFFFFFu;
constexpr unsigned CL_MAGIC = 0x314C4347u;

// word k of a compiled code list: the low 32 bits of coef[k]
__device__ __forceinline__ unsigned cl_word(const double* c, long long k) {
  return (unsigned)(unsigned long long)__double_as_longlong(c[k]);
}
__device__ __forceinline__ long long cl_tabs(const double* c) {
  return CL_HEADER + (long long)CL_SEC * cl_word(c, CLH_NSEC);
}
__device__ __forceinline__ long long cl_ins(const double* c) {
  return cl_tabs(c) + (long long)CL_TAB * cl_word(c, CLH_NTAB);
}
__device__ __forceinline__ int ipow(int w, int e) {
  int r = 1;
  for (int k = 0; k < e; ++k) r *= w;
  return r;
}

// coordinate k of the child: its interval (js < 0) or sample point js
__device__ __forceinline__ iv cl_x(const Desc& D, const double* T, ChildCtx C, unsigned long long pc, int js,
                                   int k) {
  const long long e = (long long)k * D.wid + digit(D, C.c0, C.gsz, pc, k);
  if (js < 0) return ldiv(T + D.t_off[T_LO] + 2 * e);
  const double p = T[D.t_off[T_SHI] + e * D.S + js];
  return mk(p, p);
}

// Coordinates of one child (from the iteration's table).
struct ClChildX {
  const Desc* D;
  const double* T;
  ChildCtx C;
  unsigned long long pc;
  int js;
  __device__ __forceinline__ iv operator()(int k) const { return cl_x(*D, T, C, pc, js, k); }
};

// Coordinates i + off0 and i + off1 at digits d0 and d1, straight from the
// parent box (a term-table entry; the coordinate table is built alongside).
struct ClTermX {
  const Desc* D;
  const double* pbox;
  const double* pw;
  int c0, gsz, i, js, off0, d0, d1;
  __device__ __forceinline__ iv operator()(int k) const {
    const iv x = child_iv(*D, pbox, pw, c0, gsz, k, (k - i == off0) ? d0 : d1);
    if (js < 0) return x;
    const double p = sample_pt(x, D->S, js);
    return mk(p, p);
  }
};

// Runs instructions start .. start+len-1 on the register file R.  j is the
// gradient coordinate (index base 2); i0 the loop index of a table body.
// TRED (child code only) reads the child's entries of a term table.
template <class XF>
__device__ __noinline__ void cl_exec(const Desc& D, const double* T, const XF& xf, int start, int len, int j, int i0,
                                     iv* R, ChildCtx C, unsigned long long pc, int js) {
  const double* cf = D.coef;
  const long long U = cl_tabs(cf), I = cl_ins(cf);
  const double* K = cf + I + (long long)CL_INS * cl_word(cf, CLH_NINS);
  const double2* ins = (const double2*)(cf + I);   // I is even: 16-byte aligned
  int i = i0, hi = 0, body = 0;
  for (int p = start; p < start + len; ++p) {
    const double2 w01 = ins[2 * p];
    const unsigned w0 = (unsigned)(unsigned long long)__double_as_longlong(w01.x);
    const int i1 = (int)(unsigned)(unsigned long long)__double_as_longlong(w01.y);
    const int i2 = (int)cl_word(cf, I + (long long)CL_INS * p + 2);
    const int op = (int)(w0 & 255u), d = (int)((w0 >> 8) & 255u), a = (int)((w0 >> 16) & 255u),
              b = (int)(w0 >> 24);
    switch (op) {
      case CL_LDX: R[d] = xf((a == 0 ? 0 : a == 1 ? i : j) + i1); break;
      case CL_LDC: R[d] = mk(K[i2], K[i2]); break;
      case CL_LDI: R[d] = mk(K[i2], K[i2 + 1]); break;
      case CL_LDK: {
        const double v = K[i2 + (a == 0 ? 0 : a == 1 ? i : j) + i1];
        R[d] = mk(v, v);
        break;
      }
      case CL_LDKI: R[d] = ldiv(K + i2 + 2 * ((a == 0 ? 0 : a == 1 ? i : j) + i1)); break;
      case CL_ADD: R[d] = add(R[a], R[b]); break;
      case CL_MINUS: R[d] = minus(R[a], R[b]); break;
      case CL_MUL: R[d] = mul(R[a], R[b]); break;
      case CL_DIV: R[d] = div(R[a], R[b]); break;
      case CL_TIMES: R[d] = times(R[a], K[i2]); break;
      case CL_PLUS: R[d] = plus(R[a], K[i2]); break;
      case CL_TIMESK: R[d] = times(R[a], K[i2 + (b == 0 ? 0 : b == 1 ? i : j) + i1]); break;
      case CL_PLUSK: R[d] = plus(R[a], K[i2 + (b == 0 ? 0 : b == 1 ? i : j) + i1]); break;
      case CL_SQR: R[d] = sqr(R[a]); break;
      case CL_SQRT: R[d] = sqrt_iv(R[a]); break;
      case CL_EXP: R[d] = exp_iv(R[a]); break;
      case CL_SIN: R[d] = sin_iv(R[a]); break;
      case CL_COS: R[d] = cos_iv(R[a]); break;
      case CL_MOV: R[d] = R[a]; break;
      case CL_LOOP: i = i1; hi = i2; body = p + 1; break;
      case CL_ENDLOOP:
        if (++i < hi) p = body - 1;
        break;
      case CL_TRED: {
        const long long q = U + (long long)CL_TAB * i1;
        const int lo = (int)cl_word(cf, q + CLT_LO), thi = (int)cl_word(cf, q + CLT_HI);
        const int noff = (int)cl_word(cf, q + CLT_NOFF);
        const int o0 = (int)cl_word(cf, q + CLT_OFF0), o1 = (int)cl_word(cf, q + CLT_OFF1);
        const bool prod = cl_word(cf, q + CLT_KIND) != 0;
        const int W = ipow(D.wid, noff);
        const double* tb = T + D.cl_toff[i1] + 2LL * (js + 1) * (thi - lo) * W;
        iv acc = R[a];
        for (int k = lo; k < thi; ++k) {
          int combo = 0;
          if (noff > 0) combo = digit(D, C.c0, C.gsz, pc, k + o0);
          if (noff > 1) combo = combo * D.wid + digit(D, C.c0, C.gsz, pc, k + o1);
          const iv t = ldiv(tb + 2LL * ((long long)(k - lo) * W + combo));
          acc = prod ? mul(acc, t) : add(acc, t);
        }
        R[d] = acc;
        break;
      }
      default: break;
    }
  }
}

// Coordinates j + o (o one of a tabled section's offsets) at the digits of one
// flag-table entry, straight from the parent box.
struct ClSecX {
  const Desc* D;
  const double* pbox;
  const double* pw;
  int c0, gsz, j, noff;
  int off[3], dig[3];
  __device__ __forceinline__ iv operator()(int k) const {
    int d = dig[0];
    for (int q = 1; q < noff; ++q)
      if (k - j == off[q]) d = dig[q];
    return child_iv(*D, pbox, pw, c0, gsz, k, d);
  }
};

// Entry u of the iteration's KKT flag tables (tabled sections one after the
// other): 1.0 when the section's test rules the box out, else 0.0.
__device__ __noinline__ void cl_build_flag(const Desc& D, const double* pbox, const double* pw, int c0, int gsz,
                                           long long u) {
  const int w = D.wid;
  const double* cf = D.coef;
  const int nsec = (int)cl_word(cf, CLH_NSEC);
  for (int s = 0; s < nsec && s < CL_FLAG_TABLES; ++s) {
    const long long q = CL_HEADER + (long long)CL_SEC * s;
    if (!cl_word(cf, q + CLS_TABLED)) continue;
    const int lo = (int)cl_word(cf, q + CLS_LO), hi = (int)cl_word(cf, q + CLS_HI);
    const int noff = (int)cl_word(cf, q + CLS_NOFF);
    const int W = ipow(w, noff);
    const long long cnt = (long long)(hi - lo) * W;
    if (u >= cnt) { u -= cnt; continue; }
    ClSecX xf;
    xf.D = &D; xf.pbox = pbox; xf.pw = pw; xf.c0 = c0; xf.gsz = gsz; xf.noff = noff;
    xf.j = lo + (int)(u / W);
    int combo = (int)(u % W);
    for (int k = noff - 1; k >= 0; --k) {
      xf.off[k] = (int)cl_word(cf, q + CLS_OFF0 + k);
      xf.dig[k] = combo % w;
      combo /= w;
      if (xf.dig[k] >= ndig(D, c0, gsz, xf.j + xf.off[k])) return;   // a digit this coordinate does not have
    }
    iv R[CL_MAXREG];
    ChildCtx C0;
    C0.c0 = c0;
    C0.gsz = gsz;
    cl_exec(D, D.tab, xf, (int)cl_word(cf, q + CLS_START), (int)cl_word(cf, q + CLS_LEN), xf.j, 0, R, C0, 0ULL, -1);
    const unsigned rs = cl_word(cf, q + CLS_SKIP);
    bool prune = true;
    if (rs != CL_NONE) {
      const iv t = R[rs];
      if (feq(t.lo, -INF_D) || feq(t.hi, INF_D)) prune = false;   // corrupted50.py:418-421
    }
    const int k = xf.j + (int)cl_word(cf, q + CLS_CHK);
    prune = prune && kkt_prune(R[cl_word(cf, q + CLS_REG)], xf(k), D.dom[2 * k], D.dom[2 * k + 1]);
    D.tab[D.cl_toff[CL_FLAG_TABLES + s] + u] = prune ? 1.0 : 0.0;
    return;
  }
}

// Entry u of the iteration's term tables (all tables one after the other).
__device__ __noinline__ void cl_build_term(const Desc& D, const double* pbox, const double* pw, int c0, int gsz,
                                           long long u, long long* rest) {
  const int S = D.S, w = D.wid;
  const double* cf = D.coef;
  const int ntab = (int)cl_word(cf, CLH_NTAB);
  const long long U = cl_tabs(cf);
  for (int tt = 0; tt < ntab; ++tt) {
    const long long q = U + (long long)CL_TAB * tt;
    const int lo = (int)cl_word(cf, q + CLT_LO), thi = (int)cl_word(cf, q + CLT_HI);
    const int noff = (int)cl_word(cf, q + CLT_NOFF);
    const int W = ipow(w, noff);
    const long long cnt = (long long)(S + 1) * (thi - lo) * W;
    if (u >= cnt) { u -= cnt; continue; }
    const int combo = (int)(u % W);
    const long long r = u / W;
    const int i = lo + (int)(r % (thi - lo));
    const int js = (int)(r / (thi - lo)) - 1;
    const int o0 = (int)cl_word(cf, q + CLT_OFF0), o1 = (int)cl_word(cf, q + CLT_OFF1);
    const int d0 = (noff == 2) ? combo / w : combo, d1 = combo % w;
    if (noff > 0 && d0 >= ndig(D, c0, gsz, i + o0)) return;
    if (noff > 1 && d1 >= ndig(D, c0, gsz, i + o1)) return;
    ClTermX xf{&D, pbox, pw, c0, gsz, i, js, o0, d0, noff > 1 ? d1 : d0};
    iv R[CL_MAXREG];
    ChildCtx C0;
    C0.c0 = c0;
    C0.gsz = gsz;
    cl_exec(D, D.tab, xf, (int)cl_word(cf, q + CLT_START), (int)cl_word(cf, q + CLT_LEN), 0, i, R, C0, 0ULL, js);
    stiv(D.tab + D.cl_toff[tt] + 2 * u, R[cl_word(cf, q + CLT_REG)]);
    *rest = -1;
    return;
  }
  *rest = u;   // past the term tables: an entry of the flag tables
}

// Table entries of one iteration: items [0, n w) are coordinate intervals,
// items [n w, n w (S + 1)) sample points (coordinate-major, then digit, then j),
// then every term table: [S + 1 passes][hi - lo coordinates][w^offsets digit
// combinations] intervals (pass 0 the interval pass, pass 1 + j sample j).
__device__ __forceinline__ void cl_build_item(const Desc& D, const double* pbox, const double* pw, int cyc,
                                              long long t) {
  const int n = D.n, S = D.S, w = D.wid;
  const int c0 = cyc - 1, gsz = group_size(n, D.group, cyc);
  const long long NW = (long long)n * w;
  double* T = D.tab;
  if (t < NW) {
    const int i = (int)(t / w), d = (int)(t - (long long)i * w);
    if (d >= ndig(D, c0, gsz, i)) return;
    stiv(T + D.t_off[T_LO] + 2 * t, child_iv(D, pbox, pw, c0, gsz, i, d));
    return;
  }
  if (t < NW * (S + 1)) {
    const long long u = t - NW;
    const long long e = u / S;
    const int js = (int)(u - e * S);
    const int i = (int)(e / w), d = (int)(e - (long long)i * w);
    if (d >= ndig(D, c0, gsz, i)) return;
    T[D.t_off[T_SHI] + u] = sample_pt(child_iv(D, pbox, pw, c0, gsz, i, d), S, js);
    return;
  }
  long long rest;
  cl_build_term(D, pbox, pw, c0, gsz, t - NW * (S + 1), &rest);
  if (rest >= 0) cl_build_flag(D, pbox, pw, c0, gsz, rest);
}

// interval of f over the child (js < 0) or at its sample point js
__device__ __noinline__ iv cl_value(const Desc& D, const double* T, ChildCtx C, unsigned long long pc, int js) {
  iv R[CL_MAXREG];
  ClChildX xf{&D, T, C, pc, js};
  cl_exec(D, T, xf, (int)cl_word(D.coef, CLH_VS), (int)cl_word(D.coef, CLH_VL), 0, 0, R, C, pc, js);
  return R[cl_word(D.coef, CLH_RES)];
}

// Generalized KKT test of coordinates j0, j0 + jstep, ... (1 = rule out).
// Every caller runs the once-per-box prologue itself: an FP64 instruction costs
// the same for one lane or for 32, so lanes that split the coordinates share it.
__device__ __noinline__ int cl_deriv(const Desc& D, const double* T, ChildCtx C, unsigned long long pc, int j0,
                                     int jstep) {
  const double* cf = D.coef;
  const int nsec = (int)cl_word(cf, CLH_NSEC);
  if (nsec == 0) return 0;
  const unsigned skc = cl_word(cf, CLH_SKIP);
  if (skc != CL_NONE) {
    // the box contains the given point in every coordinate (salomon50.py:374-381)
    const double v = cf[cl_ins(cf) + (long long)CL_INS * cl_word(cf, CLH_NINS) + skc];
    bool all = true;
    for (int k = 0; k < D.n && all; ++k) {
      const iv x = cl_x(D, T, C, pc, -1, k);
      if (flt(v, x.lo) || flt(x.hi, v)) all = false;
    }
    if (all) return 0;
  }
  iv R[CL_MAXREG];
  ClChildX xf{&D, T, C, pc, -1};
  cl_exec(D, T, xf, (int)cl_word(cf, CLH_PS), (int)cl_word(cf, CLH_PL), 0, 0, R, C, pc, -1);
  for (int s = 0; s < nsec; ++s) {
    const long long q = CL_HEADER + (long long)CL_SEC * s;
    const int lo = (int)cl_word(cf, q + CLS_LO), hi = (int)cl_word(cf, q + CLS_HI);
    const int st = (int)cl_word(cf, q + CLS_START), ln = (int)cl_word(cf, q + CLS_LEN);
    const int rg = (int)cl_word(cf, q + CLS_REG), chk = (int)cl_word(cf, q + CLS_CHK);
    const unsigned rs = cl_word(cf, q + CLS_SKIP);
    // first coordinate of this caller's stride in [lo, hi)
    int j = j0;
    if (j < lo) j += ((lo - j + jstep - 1) / jstep) * jstep;
    if (cl_word(cf, q + CLS_TABLED)) {
      // the flags of this section were computed for every digit combination
      const int noff = (int)cl_word(cf, q + CLS_NOFF);
      const int W = ipow(D.wid, noff);
      const double* fl = T + D.cl_toff[CL_FLAG_TABLES + s];
      for (; j < hi; j += jstep) {
        int combo = 0;
        for (int k = 0; k < noff; ++k) combo = combo * D.wid + digit(D, C.c0, C.gsz, pc, j + (int)cl_word(cf, q + CLS_OFF0 + k));
        if (__double_as_longlong(fl[(long long)(j - lo) * W + combo]) != 0) return 1;   // 1.0, not 0.0
      }
      continue;
    }
    for (; j < hi; j += jstep) {
      cl_exec(D, T, xf, st, ln, j, 0, R, C, pc, -1);
      if (rs != CL_NONE) {
        const iv t = R[rs];
        if (feq(t.lo, -INF_D) || feq(t.hi, INF_D)) continue;   // corrupted50.py:418-421
      }
      const int k = j + chk;
      if (kkt_prune(R[rg], cl_x(D, T, C, pc, -1, k), D.dom[2 * k], D.dom[2 * k + 1])) return 1;
    }
  }
  return 0;
}

}  // namespace gg
