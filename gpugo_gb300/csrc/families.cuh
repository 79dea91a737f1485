// families.cuh -- objective code lists split into per-coordinate term tables
// (built once per iteration for the selected parent) and per-child reductions.
//
// The reference evaluates, for every child box, its value code list (e.g.
// GPUGO_1.1/7-Rastrigin/rastrigin50.py:161-196), its sample code list at numSamples
// diagonal points (:245-299) and its derivative code list (:340-372), all from
// scratch (ackley50.py:602-766).  Every per-coordinate sub-expression of these code
// lists depends on one child digit only (two for the chained family's terms,
// three for its gradient), so it is computed once per parent and digit value
// and stored in a table; a child then only runs the reductions that combine the
// terms.  Reductions run in the reference's order (left to right from [0,0]),
// so every bound is bit-identical to evaluating the code list per child.
// Where the lower (upper) bound of a sum depends only on the lower (upper)
// bounds of its terms, only that side is reduced.
#pragma once
#include "ia.cuh"

namespace gg {

enum { FAM_COSQUAD = 1, FAM_CHAINED = 2, FAM_EXPSQRT = 3, FAM_PRODCOS = 4, FAM_CODELIST = 5 };
enum { STOP_WIDTH = 0, STOP_GAP = 1 };

constexpr double TWO_PI = 0x1.921fb54442d18p+2;   // 2*math.pi in the reference
constexpr double E_LO = 0x1.5bf0a8b145769p+1;     // RN(e), below e
constexpr double E_HI = 0x1.5bf0a8b14576ap+1;     // next double, above e

// Table offsets (doubles) within an instance's table region.
enum {
  T_LO = 0, T_SHI, T_PRB,                               // cosquad / chained / codelist
  T_SQ = 0, T_CS, T_XI, T_SN, T_ZB, T_SQS, T_CSS,       // expsqrt
  T_CR = 0, T_SQ4, T_SNA, T_XD2, T_XI4, T_CRS, T_SQS4, T_RCP4,  // prodcos
  T_PFX = 8,                                            // shared sample prefixes (all families)
  T_NOFF = 9
};

// Derived-constant offsets (doubles) within an instance's constant region.
struct CstLayout {
  // cosquad: K[n] A2[n] A[n] B[n] BK[2n] BSUM[2]
  // chained: P[n] Q[n] P4[n] P2[n] Q2[n] M2Q[n] C202[2n]
  // expsqrt: A B INV_N[2] APE[2] ABN[2] K[n] KN[2n]
  // prodcos: INV_D[2] INV_D2[2] RSQ[2n]
};

struct Desc {
  int family, n, wid, group, S, stop_mode, max_cyc, wlog;
  int dbits;                         // bits of one digit field of a packed child code
  unsigned long long wmag;           // floor(2^64 / wid) + 1 (wid not a power of two)
  double width_tol, gap_tol;
  long long max_iter;
  long long pool_cap, parent_cap, out_cap, trace_cap, tiles_cap, ubc_cap;
  long long a_items;                 // table-build items with every coordinate split (table_items: per iteration)
  long long tab_doubles;             // table region size (doubles)
  long long t_off[T_NOFF];           // table offsets (doubles)
  const double* dom;                 // [2n]
  const double* coef;
  double* cst;                       // derived constants
  double* tab;                       // tables
  double* parents;                   // [parent_cap][2n]
  double* pwid;                      // [parent_cap][n] (hi - lo) / wid of each parent coordinate
  int* pcyc;                         // [parent_cap]
  double* pool_lb[2];
  unsigned long long* pool_key[2];
  unsigned long long* tile_best;     // [tiles_cap][3]
  double* ubc_val;                   // [ubc_cap] sample minima below the iteration's starting UB
  unsigned long long* ubc_id;        // [ubc_cap] code << 8 | sample index
  unsigned long long* out_key;       // [out_cap] emitted boxes (width rule)
  double* out_lb;
  double* tr_ub;                     // trace rows [trace_cap]
  long long* tr_surv;
  long long* tr_pool;
  long long* tr_sel;
  // code lists: offsets of the term tables (doubles); last, so that the fields
  // every iteration reads keep their cache lines
  long long cl_toff[16];   // [0, 8) term tables, [8, 16) KKT flags of tabled sections
};

// ---------------------------------------------------------------------------
// child geometry
// ---------------------------------------------------------------------------
__device__ __forceinline__ int group_size(int n, int group, int cyc) {
  int g = n - cyc + 1;
  return g < group ? g : group;
}

// A child code is a mixed-radix number: the digit of coordinate c0 + k is digit k
// in base wid, least significant first (ackley50.py:544-577).  Kernels repack a
// code once into fixed dbits-wide fields, after which every digit lookup is a
// shift and a mask.  Division by wid is a multiply-high (Granlund and Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994): with
// M = floor(2^64 / wid) + 1 = (2^64 + e) / wid, 0 < e < wid, the product
// r M / 2^64 exceeds r / wid by less than r / 2^64 < 2^-32 < 1 / wid for every
// r < 2^32, so its integer part is floor(r / wid).  Codes of a power-of-two wid
// are packed already.
__device__ __forceinline__ unsigned long long pack_code(const Desc& D, int gsz, unsigned long long code) {
  if (D.wlog >= 0) return code;
  unsigned long long p = 0, r = code;
  for (int k = 0; k < gsz; ++k) {
    unsigned long long q = __umul64hi(r, D.wmag);
    p |= (r - q * (unsigned long long)D.wid) << (k * D.dbits);
    r = q;
  }
  return p;
}

// digit of coordinate i (0-based) in a packed child code; 0 outside the split group
__device__ __forceinline__ int digit(const Desc& D, int c0, int gsz, unsigned long long pc, int i) {
  int k = i - c0;
  if (k < 0 || k >= gsz) return 0;
  return (int)((pc >> (k * D.dbits)) & ((1ULL << D.dbits) - 1ULL));
}

// number of digit values of coordinate i this iteration
__device__ __forceinline__ int ndig(const Desc& D, int c0, int gsz, int i) {
  if (i < 0 || i >= D.n) return 0;
  int k = i - c0;
  return (k >= 0 && k < gsz) ? D.wid : 1;
}

// (double)v built from the bits (exact for every 32-bit v); an integer-to-FP64
// conversion instruction costs as much as an FP64 add.
__device__ __forceinline__ double u32_to_double(unsigned v) {
  if (v == 0) return 0.0;
  const int e = 31 - __clz(v);
  const unsigned long long m = ((unsigned long long)v << (52 - e)) & ((1ULL << 52) - 1);
  return u2d(((unsigned long long)(1023 + e) << 52) | m);
}

// child interval of coordinate i for digit d (ackley50.py:583-586, :903-906);
// pw holds the parent's (hi - lo) / wid per coordinate
__device__ __forceinline__ iv child_iv(const Desc& D, const double* pbox, const double* pw, int c0, int gsz, int i,
                                       int d) {
  double lo = pbox[2 * i], hi = pbox[2 * i + 1];
  int k = i - c0;
  if (k >= 0 && k < gsz) {
    double w = pw[i];
    return mk(__dadd_rn(__dmul_rn(w, u32_to_double(d)), lo), __dadd_rn(__dmul_rn(w, u32_to_double(d + 1)), lo));
  }
  return mk(lo, hi);
}

__device__ __forceinline__ double part_width(const Desc& D, double lo, double hi) {
  return __ddiv_rn(__dsub_rn(hi, lo), (double)D.wid);
}

// sample point j of an interval (ackley50.py:288-290)
__device__ __forceinline__ double sample_pt(iv x, int S, int j) {
  double inc = __ddiv_rn(__dsub_rn(x.hi, x.lo), u32_to_double(S + 1));
  return __dadd_rn(x.lo, __dmul_rn(inc, u32_to_double(j + 1)));
}

__device__ __forceinline__ int kkt_prune(iv d, iv x, double dlo, double dhi) {
  if (fpos(d.lo) && !feq(x.lo, dlo)) return 1;
  if (fneg(d.hi) && !feq(x.hi, dhi)) return 1;
  return 0;
}

__device__ __forceinline__ iv ldiv(const double* p) { return mk(p[0], p[1]); }
__device__ __forceinline__ void stiv(double* p, iv v) { p[0] = v.lo; p[1] = v.hi; }

struct ChildCtx {
  int c0, gsz;
};

}  // namespace gg

#include "codelist.cuh"

namespace gg {

// ---------------------------------------------------------------------------
// derived constants (one thread per instance)
// ---------------------------------------------------------------------------
__device__ void init_consts(const Desc& D) {
  const int n = D.n;
  for (int i = 0; i < n; ++i) D.pwid[i] = part_width(D, D.parents[2 * i], D.parents[2 * i + 1]);
  const double* c = D.coef;
  double* k = D.cst;
  switch (D.family) {
    case FAM_COSQUAD: {
      double bl = 0.0, bh = 0.0;
      for (int i = 0; i < n; ++i) {
        double a = c[i], b = c[n + i];
        double K = __dmul_rn(TWO_PI, c[2 * n + i]);
        k[i] = K;
        k[n + i] = __dmul_rn(2.0, a);
        k[2 * n + i] = a;
        k[3 * n + i] = b;
        k[4 * n + 2 * i] = __dmul_rd(b, K);
        k[4 * n + 2 * i + 1] = __dmul_ru(b, K);
        bl = __dadd_rd(bl, b);
        bh = __dadd_ru(bh, b);
      }
      k[6 * n] = bl;
      k[6 * n + 1] = bh;
      break;
    }
    case FAM_CHAINED: {
      for (int i = 0; i < n - 1; ++i) {
        double p = c[i], q = c[n - 1 + i];
        k[i] = p; k[n + i] = q;
        k[2 * n + i] = __dmul_rn(4.0, p);
        k[3 * n + i] = __dmul_rn(2.0, p);
        k[4 * n + i] = __dmul_rn(2.0, q);
        k[5 * n + i] = __dmul_rn(-2.0, q);
      }
      for (int j = 1; j < n - 1; ++j) {
        k[6 * n + 2 * j] = __dadd_rd(k[4 * n + j], k[3 * n + j - 1]);
        k[6 * n + 2 * j + 1] = __dadd_ru(k[4 * n + j], k[3 * n + j - 1]);
      }
      break;
    }
    case FAM_EXPSQRT: {
      double A = c[0], B = c[1], dn = (double)n;
      k[0] = A; k[1] = B;
      k[2] = __ddiv_rd(1.0, dn); k[3] = __ddiv_ru(1.0, dn);
      k[4] = __dadd_rd(A, E_LO); k[5] = __dadd_ru(A, E_HI);
      k[6] = __ddiv_rd(__dmul_rd(A, B), dn); k[7] = __ddiv_ru(__dmul_ru(A, B), dn);
      for (int i = 0; i < n; ++i) {
        double K = __dmul_rn(TWO_PI, c[2 + i]);
        k[8 + i] = K;
        k[8 + n + 2 * i] = __ddiv_rd(K, dn);
        k[8 + n + 2 * i + 1] = __ddiv_ru(K, dn);
      }
      break;
    }
    case FAM_PRODCOS: {
      double d = c[0];
      k[0] = __drcp_rd(d); k[1] = __drcp_ru(d);
      k[2] = __dmul_rn(2.0, k[0]); k[3] = __dmul_rn(2.0, k[1]);
      for (int i = 0; i < n; ++i) {
        double ii = (double)(i + 1);
        k[4 + 2 * i] = __drcp_rd(__dsqrt_ru(ii));
        k[4 + 2 * i + 1] = __drcp_ru(__dsqrt_rd(ii));
      }
      break;
    }
  }
}

// ---------------------------------------------------------------------------
// table build: one work item -> one table entry
// ---------------------------------------------------------------------------
// Table entries of one iteration.  Coordinate i has ndig(i) digit values: wid in
// the split group [c0, c0 + gsz), one outside it, so a pass over the coordinates
// holds n + gsz (wid - 1) entries (a chained pair or gradient triple touching the
// group runs all wid^2 or wid^3 digit combinations, the invalid ones returning at
// once).  Items are numbered densely over these entries: the lanes of a warp do
// not idle on digit values a coordinate does not have this iteration.  a_items
// is the count with every coordinate split (the largest over the cycle).
struct ChainZones {
  int pl, pr;   // pair positions [0, pl) and [pr, n - 1): one item each; [pl, pr): wid^2 each
  int gl, gr;   // gradient positions [0, gl) and [gr, n): one item each; [gl, gr): wid^3 each
};
__device__ __forceinline__ ChainZones chain_zones(int n, int c0, int gsz) {
  ChainZones z;
  z.pl = c0 > 0 ? c0 - 1 : 0;
  z.pr = c0 + gsz < n - 1 ? c0 + gsz : n - 1;
  z.gl = z.pl;
  z.gr = c0 + gsz + 1 < n ? c0 + gsz + 1 : n;
  return z;
}

// Each kind of item (sample points, intervals, sines or gradient tests) starts
// on a multiple of 32, so that no warp runs two kinds' code one after the other:
// the numbers in between are padding (the item returns at once).
template <typename U>
__device__ __forceinline__ U pad32(U x) { return (x + 31) & ~(U)31; }

// all_kkt: KKT flags for every coordinate (per-child evaluation of any parent);
// inside a solve only the coordinates kkt_span names are built.
__device__ __forceinline__ long long table_items(const Desc& D, int cyc, bool all_kkt) {
  if (D.family == FAM_CODELIST) return D.a_items;
  const long long n = D.n, w = D.wid, S = D.S;
  const int c0 = cyc - 1, gsz = group_size(D.n, D.group, cyc);
  if (D.family == FAM_CHAINED) {
    const ChainZones z = chain_zones(D.n, c0, gsz);
    const long long pairs = z.pl + (long long)(z.pr - z.pl) * w * w + (n - 1 - z.pr);
    const long long grads = (long long)(z.gr - z.gl) * w * w * w + (all_kkt ? z.gl + (n - z.gr) : 0);
    return pad32(pairs * (S + 1)) + grads;
  }
  const long long ne = n + (long long)gsz * (w - 1);
  const long long last = (D.family == FAM_COSQUAD && !all_kkt) ? (long long)gsz * w : ne;
  return pad32(ne * S) + pad32(ne) + last;
}

// Coordinates whose KKT flag a child of a solve's parent can have set.  For the
// two separable one-sum families the flag of coordinate j depends on its own
// interval (cos-quadratic) or on those of j - 1 .. j + 1 (chained gradient).
// Outside the split group a child keeps its parent's intervals, and the parent
// -- a child kept by the same test, or the whole domain, where no flag is set
// (every interval touches both domain bounds) -- has those flags clear.  The
// other families test every coordinate: their derivative scalars change with
// any coordinate.
__device__ __forceinline__ void kkt_span(const Desc& D, ChildCtx C, int* lo, int* hi) {
  if (D.family == FAM_COSQUAD) {
    *lo = C.c0;
    *hi = C.c0 + C.gsz;
  } else if (D.family == FAM_CHAINED) {
    *lo = C.c0 > 0 ? C.c0 - 1 : 0;
    *hi = C.c0 + C.gsz + 1 < D.n ? C.c0 + C.gsz + 1 : D.n;
  } else {
    *lo = 0;
    *hi = D.n;
  }
}

// dense entry q of a pass -> (coordinate, digit)
template <typename U>
__device__ __forceinline__ void dense_entry(U q, int c0, int gsz, U w, int* i, int* d) {
  if (q < (U)c0) { *i = (int)q; *d = 0; return; }
  const U r = q - (U)c0, gw = (U)gsz * w;
  if (r < gw) { *i = c0 + (int)(r / w); *d = (int)(r % w); return; }
  *i = c0 + gsz + (int)(r - gw);
  *d = 0;
}

// dense position q of a chained zone list (one item per position outside [lo, hi),
// per items per position inside) -> (position, combination number within it)
template <typename U>
__device__ __forceinline__ void zone_entry(U q, int lo, int hi, U per, int* i, U* e) {
  if (q < (U)lo) { *i = (int)q; *e = 0; return; }
  const U r = q - (U)lo, span = (U)(hi - lo) * per;
  if (r < span) { *i = lo + (int)(r / per); *e = r % per; return; }
  *i = hi + (int)(r - span);
  *e = 0;
}

// chained family: gradient of coordinate j given its (up to) three child intervals
__device__ __forceinline__ iv chained_grad(const Desc& D, int j, iv Xm, iv X, iv Xp) {
  const int n = D.n;
  const double* k = D.cst;
  iv d;
  if (j == 0) {
    d = times(plus(X, -1.0), k[4 * n + 0]);
    iv t = times(mul(minus(sqr(X), Xp), X), k[2 * n + 0]);
    d = add(d, t);
  } else if (j == n - 1) {
    d = times(minus(X, sqr(Xm)), k[3 * n + n - 2]);
  } else {
    d = times(minus(sqr(X), Xp), k[2 * n + j]);
    d = add(d, mk(k[6 * n + 2 * j], k[6 * n + 2 * j + 1]));
    d = plus(mul(d, X), k[5 * n + j]);
    iv t = times(sqr(Xm), k[3 * n + j - 1]);
    d = minus(d, t);
  }
  return d;
}

// Work items are numbered kind by kind (all sample-point items, ordered by
// sample index, then the interval items), so that the 32 lanes of a warp mostly
// run the same code path; index arithmetic is 32-bit (U = unsigned) unless an
// instance has 2^31 items or more.
template <typename U>
__device__ __forceinline__ void build_item_t(const Desc& D, const double* pbox, const double* pw, int cyc, U t,
                                             bool all_kkt) {
  const int n = D.n, S = D.S;
  const U w = (U)D.wid;
  const int c0 = cyc - 1, gsz = group_size(n, D.group, cyc);
  const double* k = D.cst;
  double* T = D.tab;
  const long long* off = D.t_off;
  const U NE = (U)n + (U)gsz * (w - 1);   // entries of one pass (dense_entry)
  // per-coordinate families: S sample passes, then two kinds of NE items, each
  // kind from a multiple of 32 (pad32)
  const U SNE = (U)S * NE, K1 = pad32(SNE), K2 = K1 + pad32(NE);
  switch (D.family) {
    case FAM_COSQUAD: {
      // [S sample passes][LB terms] over the NE entries, then the gradient tests:
      // over the NE entries (all_kkt) or over the split group's entries only
      int j, i, d;
      if (t < SNE) {
        j = (int)(t / NE);
        dense_entry<U>(t - (U)j * NE, c0, gsz, w, &i, &d);
      } else if (t < K1) {
        return;
      } else if (t < K1 + NE) {
        j = S;
        dense_entry<U>(t - K1, c0, gsz, w, &i, &d);
      } else if (t < K2) {
        return;
      } else if (all_kkt) {
        j = S + 1;
        dense_entry<U>(t - K2, c0, gsz, w, &i, &d);
      } else {
        const U r = t - K2;
        j = S + 1;
        i = c0 + (int)(r / w);
        d = (int)(r % w);
      }
      const U e = (U)i * w + (U)d;
      iv X = child_iv(D, pbox, pw, c0, gsz, i, d);
      double K = k[i], a = k[2 * n + i], b = k[3 * n + i];
      if (j == S) {
        iv term = minus(times(sqr(X), a), times(cos_iv(times(X, K)), b));
        T[off[T_LO] + e] = term.lo;
      } else if (j == S + 1) {
        iv g = add(times(X, k[n + i]), mul(sin_iv(times(X, K)), mk(k[4 * n + 2 * i], k[4 * n + 2 * i + 1])));
        ((unsigned char*)(T + off[T_PRB]))[e] = (unsigned char)kkt_prune(g, X, D.dom[2 * i], D.dom[2 * i + 1]);
      } else {
        double x = sample_pt(X, S, j);
        iv P = mk(x, x);
        iv term = minus(times(sqr(P), a), times(cos_iv(times(P, K)), b));
        T[off[T_SHI] + (long long)e * S + j] = term.hi;
      }
      return;
    }
    case FAM_CHAINED: {
      const U w2 = w * w;
      const ChainZones z = chain_zones(n, c0, gsz);
      const U P1 = (U)z.pl + (U)(z.pr - z.pl) * w2 + (U)(n - 1 - z.pr);   // pairs of one pass
      const U part1 = P1 * (U)(S + 1);
      if (t >= part1 && t < pad32(part1)) return;
      if (t < part1) {
        // [S + 1 passes (samples, then LB) x the pairs (i, i + 1)]
        const int j = (int)(t / P1);
        int i;
        U r;
        zone_entry<U>(t - (U)j * P1, z.pl, z.pr, w2, &i, &r);
        const int d1 = (int)(r % w), d0 = (int)(r / w);
        if (d0 >= ndig(D, c0, gsz, i) || d1 >= ndig(D, c0, gsz, i + 1)) return;
        const double kq = k[n + i], kp = k[i];   // loaded with the parent box, not after the chain
        iv X = child_iv(D, pbox, pw, c0, gsz, i, d0);
        iv Y = child_iv(D, pbox, pw, c0, gsz, i + 1, d1);
        if (j < S) {
          double x = sample_pt(X, S, j), y = sample_pt(Y, S, j);
          X = mk(x, x); Y = mk(y, y);
        }
        iv u = times(sqr(plus(X, -1.0)), kq);
        iv v = times(sqr(minus(sqr(X), Y)), kp);
        iv term = add(v, u);
        const long long e = (long long)i * w2 + (long long)d0 * w + d1;
        if (j == S) T[off[T_LO] + e] = term.lo;
        else T[off[T_SHI] + e * S + j] = term.hi;
      } else {
        // the gradient triples: positions [gl, gr) only, unless all_kkt
        const U w3 = w2 * w;
        int j;
        U e;
        if (all_kkt) {
          zone_entry<U>(t - pad32(part1), z.gl, z.gr, w3, &j, &e);
        } else {
          const U r = t - pad32(part1);
          j = z.gl + (int)(r / w3);
          e = r % w3;
        }
        const int dm = (int)(e / w2), d = (int)((e / w) % w), dp = (int)(e % w);
        int nm = (j > 0) ? ndig(D, c0, gsz, j - 1) : 1;
        int np = (j + 1 < n) ? ndig(D, c0, gsz, j + 1) : 1;
        if (dm >= nm || d >= ndig(D, c0, gsz, j) || dp >= np) return;
        iv X = child_iv(D, pbox, pw, c0, gsz, j, d);
        iv Xm = (j > 0) ? child_iv(D, pbox, pw, c0, gsz, j - 1, dm) : X;
        iv Xp = (j + 1 < n) ? child_iv(D, pbox, pw, c0, gsz, j + 1, dp) : X;
        iv g = chained_grad(D, j, Xm, X, Xp);
        ((unsigned char*)(T + off[T_PRB]))[(long long)j * w3 + e] =
            (unsigned char)kkt_prune(g, X, D.dom[2 * j], D.dom[2 * j + 1]);
      }
      return;
    }
    case FAM_EXPSQRT: {
      // [S sample passes][interval items][sine items], each over the NE entries
      int j, i, d;
      if (t < SNE) {
        j = (int)(t / NE);
        dense_entry<U>(t - (U)j * NE, c0, gsz, w, &i, &d);
      } else if (t < K1 || (t >= K1 + NE && t < K2)) {
        return;
      } else {
        j = (t < K2) ? S : S + 1;
        dense_entry<U>(t - ((t < K2) ? K1 : K2), c0, gsz, w, &i, &d);
      }
      const U e = (U)i * w + (U)d;
      iv X = child_iv(D, pbox, pw, c0, gsz, i, d);
      double K = k[8 + i];
      if (j == S) {
        stiv(T + off[T_SQ] + 2 * (long long)e, sqr(X));
        stiv(T + off[T_CS] + 2 * (long long)e, cos_iv(times(X, K)));
        stiv(T + off[T_XI] + 2 * (long long)e, X);
        ((unsigned char*)(T + off[T_ZB]))[e] = (unsigned char)((fpos(X.lo) || fneg(X.hi)) ? 0 : 1);
      } else if (j == S + 1) {
        stiv(T + off[T_SN] + 2 * (long long)e, sin_iv(times(X, K)));
      } else {
        double x = sample_pt(X, S, j);
        iv P = mk(x, x);
        const long long q = 2 * ((long long)e * S + j);
        stiv(T + off[T_SQS] + q, sqr(P));
        stiv(T + off[T_CSS] + q, cos_iv(times(P, K)));
      }
      return;
    }
    case FAM_PRODCOS: {
      // [S sample passes][interval items][sine items], each over the NE entries
      int j, i, d;
      if (t < SNE) {
        j = (int)(t / NE);
        dense_entry<U>(t - (U)j * NE, c0, gsz, w, &i, &d);
      } else if (t < K1 || (t >= K1 + NE && t < K2)) {
        return;
      } else {
        j = (t < K2) ? S : S + 1;
        dense_entry<U>(t - ((t < K2) ? K1 : K2), c0, gsz, w, &i, &d);
      }
      const U e = (U)i * w + (U)d;
      iv X = child_iv(D, pbox, pw, c0, gsz, i, d);
      iv RSQ = mk(k[4 + 2 * i], k[4 + 2 * i + 1]);
      if (j == S) {
        iv cr = cos_iv(mul(X, RSQ));
        stiv(T + off[T_CR] + 2 * (long long)e, cr);
        stiv(T + off[T_RCP4] + 2 * (long long)e, div_recip(cr));
        stiv(T + off[T_SQ4] + 2 * (long long)e, sqr(X));
        stiv(T + off[T_XD2] + 2 * (long long)e, mul(X, mk(k[2], k[3])));
        stiv(T + off[T_XI4] + 2 * (long long)e, X);
      } else if (j == S + 1) {
        stiv(T + off[T_SNA] + 2 * (long long)e, sin_iv(mul(X, RSQ)));
      } else {
        double x = sample_pt(X, S, j);
        iv P = mk(x, x);
        const long long q = 2 * ((long long)e * S + j);
        stiv(T + off[T_CRS] + q, cos_iv(mul(P, RSQ)));
        stiv(T + off[T_SQS4] + q, sqr(P));
      }
      return;
    }
  }
}

template <bool CL = true>
__device__ __forceinline__ void build_item(const Desc& D, const double* pbox, const double* pw, int cyc, long long t,
                                           bool all_kkt) {
  if constexpr (CL) {
    if (D.family == FAM_CODELIST) { cl_build_item(D, pbox, pw, cyc, t); return; }
  }
  if (D.a_items < (1LL << 31)) build_item_t<unsigned>(D, pbox, pw, cyc, (unsigned)t, all_kkt);
  else build_item_t<unsigned long long>(D, pbox, pw, cyc, (unsigned long long)t, all_kkt);
}

// ---------------------------------------------------------------------------
// per-child reductions
// ---------------------------------------------------------------------------

// One side of the interval operations with a positive interval constant [kl, kh]
// (IA.py:117-152 with the sign of the constant known): the lower bound of a*k
// depends on a's lower bound only, the upper bound on a's upper bound only.
__device__ __forceinline__ double mulk_lo(double al, double kl, double kh) {
  return fneg(al) ? __dmul_rd(al, kh) : __dmul_rd(al, kl);
}
__device__ __forceinline__ double mulk_hi(double ah, double kl, double kh) {
  return fneg(ah) ? __dmul_ru(ah, kl) : __dmul_ru(ah, kh);
}
// one side of power(., 1/2) and exp (IA.py:209-304, :532-570)
__device__ __forceinline__ double sqrt_lo(double l) { return bump_lo(__dsqrt_rn(fneg(l) ? 0.0 : l), 5); }
__device__ __forceinline__ double sqrt_hi(double h) { return bump_hi(__dsqrt_rn(fneg(h) ? 0.0 : h), 5); }
// our exp moved down / up by two units in the last place (exp_iv's endpoints)
__device__ __forceinline__ double exp_lo_of(double l) {
  if (isnan_(l)) return l;
  uint64_t m = d2u(l);
  return (m < 2) ? 0.0 : u2d(m - 2);
}
__device__ __forceinline__ double exp_hi_of(double h) {
  if (isnan_(h)) return h;
  uint64_t m = d2u(h);
  return (m + 2 >= INF_BITS) ? u2d(INF_BITS) : u2d(m + 2);
}
__device__ __forceinline__ double exp_lo(double x) { return exp_lo_of(gg_exp(x)); }
__device__ __forceinline__ double exp_hi(double x) { return exp_hi_of(gg_exp(x)); }
__device__ __forceinline__ double neg_(double x) { return u2d(d2u(x) ^ 0x8000000000000000ULL); }

// expsqrt f = -A exp(-B sqrt(mean x^2)) - exp(mean cos) + A + e (ackley50.py:166-212):
// f's lower bound from the lower bound of the sum of squares and the upper bound of
// the cosine sum; its upper bound from the opposite sides.
__device__ __forceinline__ double expsqrt_lo(const double* k, double s_lo, double c_hi) {
  double r_lo = sqrt_lo(mulk_lo(s_lo, k[2], k[3]));
  double E_hi = exp_hi(__dmul_ru(r_lo, -k[1]));        // times(r, -B).hi
  double t_lo = __dmul_rd(E_hi, -k[0]);                // times(E, -A).lo
  double u_hi = exp_hi(mulk_hi(c_hi, k[2], k[3]));
  return __dadd_rd(__dadd_rd(t_lo, -u_hi), k[4]);
}
__device__ __forceinline__ double expsqrt_hi(const double* k, double s_hi, double c_lo) {
  double r_hi = sqrt_hi(mulk_hi(s_hi, k[2], k[3]));
  double E_lo = exp_lo(__dmul_rd(r_hi, -k[1]));        // times(r, -B).lo
  double t_hi = __dmul_ru(E_lo, -k[0]);                // times(E, -A).hi
  double u_lo = exp_lo(mulk_lo(c_lo, k[2], k[3]));
  return __dadd_ru(__dadd_ru(t_hi, -u_lo), k[5]);
}

// Screening bounds.  exp_upper(x) is an upper bound of exp(x) widened by 2^-13:
// y = RN32(x log2 e) is within 2^-18 of x log2 e for |x| < 80, ex2.approx.f32 is
// within 2^-21 of 2^y, so e = 2^y >= exp(x) (1 - 2^-18) and RU(e (1 + 2^-12)) >=
// exp(x) (1 + 2^-13).  Our exp is within two units in the last place, so exp_hi and
// exp_lo (our exp moved outward by two units) never exceed it.  Replacing the
// exponentials of expsqrt_lo / expsqrt_hi by exp_upper, with every other operation
// unchanged and directed the same way (A > 0, and every step is monotone in the
// replaced value), gives a value that is never above the exact bound.  Such a value
// already above the UB settles a comparison without the exact exponentials.
__device__ __forceinline__ bool exp_upper(double x, double* out) {
  if (!(flt(-80.0, x) && flt(x, 80.0))) return false;   // also NaN
  const float y = __double2float_rn(__dmul_rn(x, 0x1.71547652b82fep+0));
  float e;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(y));
  *out = __dmul_ru((double)e, 1.0 + 0x1p-12);
  return true;
}
// lower bound of expsqrt_lo(k, s_lo, c_hi); false when it cannot bound
__device__ __forceinline__ bool expsqrt_lo_bound(const double* k, double s_lo, double c_hi, double* out) {
  double r_lo = sqrt_lo(mulk_lo(s_lo, k[2], k[3]));
  double E, U;
  if (!exp_upper(__dmul_ru(r_lo, -k[1]), &E) || !exp_upper(mulk_hi(c_hi, k[2], k[3]), &U)) return false;
  *out = __dadd_rd(__dadd_rd(__dmul_rd(E, -k[0]), -U), k[4]);
  return true;
}
// lower bound of expsqrt_hi(k, s_hi, c_lo); false when it cannot bound
__device__ __forceinline__ bool expsqrt_hi_bound(const double* k, double s_hi, double c_lo, double* out) {
  double r_hi = sqrt_hi(mulk_hi(s_hi, k[2], k[3]));
  double E, U;
  if (!exp_upper(__dmul_rd(r_hi, -k[1]), &E) || !exp_upper(mulk_lo(c_lo, k[2], k[3]), &U)) return false;
  *out = __dadd_ru(__dadd_ru(__dmul_ru(E, -k[0]), -U), k[5]);
  return true;
}

// Per-child functions take packed child codes (pack_code).
__device__ __forceinline__ long long eidx(const Desc& D, ChildCtx C, unsigned long long pc, int i) {
  return (long long)i * D.wid + digit(D, C.c0, C.gsz, pc, i);
}

// aux (may be null) receives the product-cosine value product (two doubles),
// which the derivative test reuses.  With a finite cut the function may return,
// instead of the LB, a lower bound of it that is already above cut (the caller
// only compares it with cut).
// Two independent reductions over the coordinates share one loop; each keeps
// the reference's left-to-right order.
// CL = false leaves the code-list case out (the persistent kernel is built
// twice, and the copy without code lists runs whenever none is resident).
template <bool CL = true>
__device__ __noinline__ double child_lb(const Desc& D, const double* T, ChildCtx C, unsigned long long pc,
                                        double* aux = nullptr, double cut = INF_D) {
  const int n = D.n, w = D.wid;
  const double* k = D.cst;
  const long long* off = D.t_off;
  switch (D.family) {
    case FAM_COSQUAD: {
      double s = 0.0;
      const double* tl = T + off[T_LO];
      for (int i = 0; i < n; ++i) s = __dadd_rd(s, tl[eidx(D, C, pc, i)]);
      return __dadd_rd(s, k[6 * n]);
    }
    case FAM_CHAINED: {
      double f = 0.0;
      const double* tl = T + off[T_LO];
      int dcur = digit(D, C.c0, C.gsz, pc, 0);
      for (int i = 0; i < n - 1; ++i) {
        int dn = digit(D, C.c0, C.gsz, pc, i + 1);
        f = __dadd_rd(f, tl[(long long)i * w * w + dcur * w + dn]);
        dcur = dn;
      }
      return f;
    }
    case FAM_EXPSQRT: {
      double s_lo = 0.0, c_hi = 0.0;
      for (int i = 0; i < n; ++i) {
        const long long e = eidx(D, C, pc, i);
        s_lo = __dadd_rd(s_lo, T[off[T_SQ] + 2 * e]);
        c_hi = __dadd_ru(c_hi, T[off[T_CS] + 2 * e + 1]);
      }
      double b;
      if (expsqrt_lo_bound(k, s_lo, c_hi, &b) && flt(cut, b)) return b;
      return expsqrt_lo(k, s_lo, c_hi);
    }
    case FAM_PRODCOS: {
      iv pr = mk(-1.0, -1.0);
      double s_lo = 0.0;
      for (int i = 0; i < n; ++i) {
        const long long e = eidx(D, C, pc, i);
        pr = mul(pr, ldiv(T + off[T_CR] + 2 * e));
        s_lo = __dadd_rd(s_lo, T[off[T_SQ4] + 2 * e]);
      }
      if (aux) { aux[0] = pr.lo; aux[1] = pr.hi; }
      return __dadd_rd(__dadd_rd(mulk_lo(s_lo, k[0], k[1]), 1.0), pr.lo);
    }
    case FAM_CODELIST:
      if constexpr (CL) return cl_value(D, T, C, pc, -1).lo;
      break;
  }
  return 0.0;
}

// Running values of one pass of the sample code list: cosquad / chained the sum
// (a); expsqrt the sum of squares (a, upper side) and of cosines (b, lower side);
// prodcos the cosine product [a, b] and the sum of squares (c, upper side).
struct SAcc {
  double a, b, c;
};

__device__ __forceinline__ SAcc sacc_init(const Desc& D) {
  SAcc r;
  r.a = r.b = (D.family == FAM_PRODCOS) ? -1.0 : 0.0;
  r.c = 0.0;
  return r;
}

// number of terms of the sample reduction, and how many of them (those of
// coordinates before the split group, whose digit is 0 in every child) are the
// same for all children of the parent
__device__ __forceinline__ int samp_terms(const Desc& D) { return D.family == FAM_CHAINED ? D.n - 1 : D.n; }
// (built-in families only: code lists have no seed pass and no sample prefixes)
__device__ __forceinline__ int samp_shared(const Desc& D, ChildCtx C) {
  return D.family == FAM_CHAINED ? (C.c0 > 0 ? C.c0 - 1 : 0) : C.c0;
}

// Terms ib .. ie-1 of the sample passes j0 .. j0+M-1, added to acc in the
// reference's order (M passes side by side in one loop over the coordinates).
template <int M>
__device__ __forceinline__ void samp_run(const Desc& D, const double* T, ChildCtx C, unsigned long long pc, int j0,
                                         int ib, int ie, SAcc* acc) {
  const int w = D.wid, S = D.S;
  const long long* off = D.t_off;
  switch (D.family) {
    case FAM_COSQUAD: {
      const double* th = T + off[T_SHI] + j0;
      for (int i = ib; i < ie; ++i) {
        const double* t = th + eidx(D, C, pc, i) * S;
#pragma unroll
        for (int q = 0; q < M; ++q) acc[q].a = __dadd_ru(acc[q].a, t[q]);
      }
      return;
    }
    case FAM_CHAINED: {
      const double* th = T + off[T_SHI] + j0;
      int dcur = digit(D, C.c0, C.gsz, pc, ib);
      for (int i = ib; i < ie; ++i) {
        int dn = digit(D, C.c0, C.gsz, pc, i + 1);
        const double* t = th + ((long long)i * w * w + dcur * w + dn) * S;
#pragma unroll
        for (int q = 0; q < M; ++q) acc[q].a = __dadd_ru(acc[q].a, t[q]);
        dcur = dn;
      }
      return;
    }
    case FAM_EXPSQRT: {
      const double* ts = T + off[T_SQS] + 2 * j0 + 1;
      const double* tc = T + off[T_CSS] + 2 * j0;
      for (int i = ib; i < ie; ++i) {
        const long long e2 = 2 * eidx(D, C, pc, i) * S;
#pragma unroll
        for (int q = 0; q < M; ++q) {
          acc[q].a = __dadd_ru(acc[q].a, ts[e2 + 2 * q]);
          acc[q].b = __dadd_rd(acc[q].b, tc[e2 + 2 * q]);
        }
      }
      return;
    }
    default: {  // FAM_PRODCOS
      const double* tr = T + off[T_CRS] + 2 * j0;
      const double* ts = T + off[T_SQS4] + 2 * j0 + 1;
      for (int i = ib; i < ie; ++i) {
        const long long e2 = 2 * eidx(D, C, pc, i) * S;
#pragma unroll
        for (int q = 0; q < M; ++q) {
          iv pr = mul(mk(acc[q].a, acc[q].b), ldiv(tr + e2 + 2 * q));
          acc[q].a = pr.lo;
          acc[q].b = pr.hi;
          acc[q].c = __dadd_ru(acc[q].c, ts[e2 + 2 * q]);
        }
      }
      return;
    }
  }
}

// The value of a finished sample pass.  With a finite cut the value may be
// replaced by a lower bound of it that is not below cut (callers only look for
// values below cut).
__device__ __forceinline__ double samp_value(const Desc& D, const SAcc& r, double cut) {
  const double* k = D.cst;
  switch (D.family) {
    case FAM_COSQUAD: return __dadd_ru(r.a, k[6 * D.n + 1]);
    case FAM_CHAINED: return r.a;
    case FAM_EXPSQRT: {
      double b;
      if (expsqrt_hi_bound(k, r.a, r.b, &b) && !flt(b, cut)) return b;
      return expsqrt_hi(k, r.a, r.b);
    }
    default: return __dadd_ru(__dadd_ru(mulk_hi(r.c, k[0], k[1]), 1.0), r.b);
  }
}

// Upper bounds of f at sample points j0 .. j0+M-1 of the child.  pfx (may be
// null) holds the running values after the shared terms (samp_shared) for every
// sample index: pfx[j], pfx[S + j], pfx[2S + j] = a, b, c.
template <int M>
__device__ __forceinline__ void samp_multi(const Desc& D, const double* T, ChildCtx C, unsigned long long pc, int j0,
                                           double* v, double cut = INF_D, const double* pfx = nullptr) {
  SAcc acc[M];
  int ib = 0;
  const int sh = samp_shared(D, C);
  if (pfx && sh > 0) {
    ib = sh;
#pragma unroll
    for (int q = 0; q < M; ++q) {
      acc[q].a = pfx[j0 + q];
      acc[q].b = pfx[D.S + j0 + q];
      acc[q].c = pfx[2 * D.S + j0 + q];
    }
  } else {
#pragma unroll
    for (int q = 0; q < M; ++q) acc[q] = sacc_init(D);
  }
  samp_run<M>(D, T, C, pc, j0, ib, samp_terms(D), acc);
  if (D.family != FAM_EXPSQRT || M == 1) {
#pragma unroll
    for (int q = 0; q < M; ++q) v[q] = samp_value(D, acc[q], cut);
    return;
  }
  // exp-sqrt: screen all M values first; the exact tails that remain run one per
  // lane per round (a lane takes its next pending value), so the warp pays for
  // max-over-lanes of them instead of one round per sample index any lane needs
  const double* k = D.cst;
  unsigned pend = 0;
#pragma unroll
  for (int q = 0; q < M; ++q) {
    double b;
    if (expsqrt_hi_bound(k, acc[q].a, acc[q].b, &b) && !flt(b, cut)) v[q] = b;
    else pend |= 1u << q;
  }
  const unsigned am = __activemask();
  while (__any_sync(am, pend != 0)) {
    if (pend) {
      const int q = __ffs(pend) - 1;
      pend &= pend - 1;
      double sa = acc[0].a, sb = acc[0].b;
#pragma unroll
      for (int t = 1; t < M; ++t)
        if (t == q) { sa = acc[t].a; sb = acc[t].b; }
      const double e = expsqrt_hi(k, sa, sb);
#pragma unroll
      for (int t = 0; t < M; ++t)
        if (t == q) v[t] = e;
    }
  }
}

// Running values of sample pass j after the shared terms, stored in pfx
// (samp_multi's layout); returns them.
__device__ __forceinline__ SAcc samp_prefix(const Desc& D, const double* T, ChildCtx C, int j, double* pfx) {
  SAcc r = sacc_init(D);
  samp_run<1>(D, T, C, 0ULL, j, 0, samp_shared(D, C), &r);
  pfx[j] = r.a;
  pfx[D.S + j] = r.b;
  pfx[2 * D.S + j] = r.c;
  return r;
}

// upper bound of f at sample point j of the child (one pass of the sample code list)
template <bool CL = true>
__device__ __noinline__ double samp_one(const Desc& D, const double* T, ChildCtx C, unsigned long long pc, int j,
                                        double cut = INF_D, const double* pfx = nullptr) {
  if constexpr (CL) {
    if (D.family == FAM_CODELIST) return cl_value(D, T, C, pc, j).hi;
  }
  double v;
  samp_multi<1>(D, T, C, pc, j, &v, cut, pfx);
  return v;
}

// The sample code list keeps the first sample with the smallest upper bound
// (rastrigin50.py:289-297): minimum over (value, sample index).
__device__ __forceinline__ bool samp_better(double v, int j, double bv, int bj) {
  // NaN at j = 0 sticks (best > x is false for every x); later NaNs never win
  if (bj == 0 && isnan_(bv)) return false;
  if (j == 0 && isnan_(v)) return true;
  if (isnan_(v)) return false;
  if (isnan_(bv)) return true;
  return flt(v, bv) || (feq(v, bv) && j < bj);
}

// smallest sampled upper bound; *jbest receives its sample index
__device__ __noinline__ double child_samp(const Desc& D, const double* T, ChildCtx C, unsigned long long pc,
                                          int* jbest) {
  double best = 0.0;
  int jb = 0;
  for (int j = 0; j < D.S; ++j) {
    double fh = samp_one(D, T, C, pc, j);
    if (j == 0 || flt(fh, best)) { best = fh; jb = j; }
  }
  *jbest = jb;
  return best;
}

// Per-child scalars of the derivative code lists that do not depend on the
// coordinate: expsqrt g = A B exp(-B r) / (n r) and u = exp(mean cos) (ackley50.py:413-455),
// prodcos P = prod cos(x_i / sqrt(i)) (griewank50.py:383-396).  Returns 1 when the
// test is skipped (expsqrt box containing the origin, ackley50.py:402-409).
struct DerivPre {
  iv g, u;
};

__device__ __noinline__ int deriv_pre(const Desc& D, const double* T, ChildCtx C, unsigned long long pc,
                                      DerivPre* P) {
  const int n = D.n;
  const double* k = D.cst;
  const long long* off = D.t_off;
  if (D.family == FAM_EXPSQRT) {
    const unsigned char* zb = (const unsigned char*)(T + off[T_ZB]);
    int origin = 1;
    for (int i = 0; i < n; ++i)
      if (!zb[eidx(D, C, pc, i)]) { origin = 0; break; }
    if (origin) return 1;
    iv s = mk(0.0, 0.0), c = mk(0.0, 0.0);
    for (int i = 0; i < n; ++i) {
      const long long e = eidx(D, C, pc, i);
      s = add(s, ldiv(T + off[T_SQ] + 2 * e));
      c = add(c, ldiv(T + off[T_CS] + 2 * e));
    }
    iv inv_n = mk(k[2], k[3]);
    iv r = sqrt_iv(mul(s, inv_n));
    iv g = exp_iv(times(r, -k[1]));
    P->g = mul(div(g, r), mk(k[6], k[7]));
    P->u = exp_iv(mul(c, inv_n));
  } else if (D.family == FAM_PRODCOS) {
    iv pr = mk(1.0, 1.0);
    for (int i = 0; i < n; ++i) pr = mul(pr, ldiv(T + off[T_CR] + 2 * eidx(D, C, pc, i)));
    P->g = pr;
  }
  return 0;
}

// The product-cosine derivative scalar from the value pass: the value product
// starts from [-1,-1] and the derivative product from [1,1]; interval
// multiplication commutes with negation bit for bit, so P is the negated value
// product (griewank50.py:383-396).
__device__ __forceinline__ void deriv_pre_aux(const double* aux, DerivPre* P) { P->g = mk(-aux[1], -aux[0]); }

// One expsqrt candidate with the whole warp.  An FP64 instruction costs the same
// however many lanes it serves, so the work is laid out across lanes:
//   lanes j < S       sum of squares of sample pass j (upper side)
//   lanes S + j       sum of cosines of sample pass j (lower side)
//   lanes 2S .. 2S+3  the four endpoint sums of the derivative scalars
// all run as one loop of upward additions (a downward sum is the negated upward
// sum of the negated terms, RD(a + b) = -RU(-a - b), signed zeros included, so
// the negated chains start from -0).  The square roots and exponentials of the
// sample bounds (expsqrt_hi) and of the derivative scalars (deriv_pre) then share
// instructions across lanes.  Every value is the one the per-pass code computes.
// Lane j < S returns the value of sample pass j in *v (or, with a finite cut, a
// lower bound of it not below cut, as samp_value); every lane returns P and the
// skip flag of deriv_pre.  Requires 2S + 4 <= 32.
__device__ __noinline__ void expsqrt_warp(const Desc& D, const double* T, ChildCtx C, unsigned long long pc,
                                          double cut, double* v, DerivPre* P, int* skip) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, n = D.n, S = D.S;
  const double* k = D.cst;
  const long long* off = D.t_off;
  // deriv_pre's origin test: every coordinate's child interval contains 0
  const unsigned char* zb = (const unsigned char*)(T + off[T_ZB]);
  int notzero = 0;
  for (int i = lane; i < n; i += 32) notzero |= !zb[eidx(D, C, pc, i)];
  *skip = !__any_sync(FULL, notzero);
  const double* src;
  long long stride, add;
  bool dn;
  if (lane < S) { src = T + off[T_SQS]; stride = 2 * S; add = 2 * lane + 1; dn = false; }
  else if (lane < 2 * S) { src = T + off[T_CSS]; stride = 2 * S; add = 2 * (lane - S); dn = true; }
  else if (lane < 2 * S + 4) {
    const int q = lane - 2 * S;   // s.lo, s.hi, c.lo, c.hi
    src = T + off[q < 2 ? T_SQ : T_CS]; stride = 2; add = q & 1; dn = !(q & 1);
  } else { src = T + off[T_SQ]; stride = 2; add = 0; dn = false; }
  double acc = dn ? -0.0 : 0.0;
  // terms are loaded eight at a time ahead of the additions
  int i = 0;
  for (; i + 8 <= n; i += 8) {
    double t[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) t[q] = src[eidx(D, C, pc, i + q) * stride + add];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc = __dadd_ru(acc, dn ? neg_(t[q]) : t[q]);
  }
  for (; i < n; ++i) {
    const double t = src[eidx(D, C, pc, i) * stride + add];
    acc = __dadd_ru(acc, dn ? neg_(t) : t);
  }
  const double val = dn ? neg_(acc) : acc;
  const iv inv_n = mk(k[2], k[3]);
  const iv m = mul(mk(__shfl_sync(FULL, val, 2 * S), __shfl_sync(FULL, val, 2 * S + 1)), inv_n);
  const iv mc = mul(mk(__shfl_sync(FULL, val, 2 * S + 2), __shfl_sync(FULL, val, 2 * S + 3)), inv_n);
  const double my_c = __shfl_sync(FULL, val, lane < S ? lane + S : lane);
  // square roots: sample lanes sqrt_hi of their pass, lanes S and S+1 sqrt_iv(m)
  const double sa = (lane < S) ? mulk_hi(val, k[2], k[3]) : (lane == S ? m.lo : m.hi);
  const double sy = __dsqrt_rn(fneg(sa) ? 0.0 : sa);
  const double pl = __shfl_sync(FULL, sy, S), ph = __shfl_sync(FULL, sy, S + 1);
  const iv r = mk(bump_lo(pmin(pl, ph), 5), bump_hi(pmax(pl, ph), 5));
  // sample bounds, screened first (samp_value)
  double a1 = 0.0, a2 = 0.0, vb = 0.0;
  bool need = false;
  if (lane < S) {
    a1 = __dmul_rd(bump_hi(sy, 5), -k[1]);
    a2 = mulk_lo(my_c, k[2], k[3]);
    double E, U;
    if (exp_upper(a1, &E) && exp_upper(a2, &U)) {
      vb = __dadd_ru(__dadd_ru(__dmul_ru(E, -k[0]), -U), k[5]);
      need = flt(vb, cut);
    } else {
      need = true;
    }
  }
  // exponentials: the derivative endpoints and the first one of unscreened
  // samples in one round, the second one of unscreened samples in another
  double x1 = 0.0;
  if (lane < S) x1 = need ? a1 : 0.0;
  else if (lane == S) x1 = __dmul_rd(r.hi, -k[1]);       // times(r, -B).lo
  else if (lane == S + 1) x1 = __dmul_ru(r.lo, -k[1]);   // times(r, -B).hi
  else if (lane == S + 2) x1 = mc.lo;
  else if (lane == S + 3) x1 = mc.hi;
  const double y1 = gg_exp(x1);
  double y2 = 0.0;
  if (__any_sync(FULL, need)) y2 = gg_exp(need ? a2 : 0.0);
  if (lane < S) {
    *v = need ? __dadd_ru(__dadd_ru(__dmul_ru(exp_lo_of(y1), -k[0]), -exp_lo_of(y2)), k[5]) : vb;
  }
  const iv E = mk(exp_lo_of(__shfl_sync(FULL, y1, S)), exp_hi_of(__shfl_sync(FULL, y1, S + 1)));
  P->u = mk(exp_lo_of(__shfl_sync(FULL, y1, S + 2)), exp_hi_of(__shfl_sync(FULL, y1, S + 3)));
  P->g = mul(div(E, r), mk(k[6], k[7]));
}

// generalized KKT test of coordinate j (rastrigin50.py:365-370); 1 = rule out
__device__ __forceinline__ int deriv_coord(const Desc& D, const double* T, ChildCtx C, unsigned long long pc,
                                           int j, const DerivPre& P) {
  const int n = D.n, w = D.wid;
  const double* k = D.cst;
  const long long* off = D.t_off;
  switch (D.family) {
    case FAM_COSQUAD:
      return ((const unsigned char*)(T + off[T_PRB]))[eidx(D, C, pc, j)];
    case FAM_CHAINED: {
      const long long w2 = (long long)w * w, w3 = w2 * w;
      int dm = (j > 0) ? digit(D, C.c0, C.gsz, pc, j - 1) : 0;
      int d = digit(D, C.c0, C.gsz, pc, j);
      int dp = (j + 1 < n) ? digit(D, C.c0, C.gsz, pc, j + 1) : 0;
      return ((const unsigned char*)(T + off[T_PRB]))[(long long)j * w3 + (long long)dm * w2 + (long long)d * w + dp];
    }
    case FAM_EXPSQRT: {
      long long e = eidx(D, C, pc, j);
      iv X = ldiv(T + off[T_XI] + 2 * e);
      iv dd = mul(P.g, X);
      iv h = mul(mul(ldiv(T + off[T_SN] + 2 * e), P.u), mk(k[8 + n + 2 * j], k[8 + n + 2 * j + 1]));
      dd = add(dd, h);
      return kkt_prune(dd, X, D.dom[2 * j], D.dom[2 * j + 1]);
    }
    default: {  // FAM_PRODCOS
      long long e = eidx(D, C, pc, j);
      iv R = ldiv(T + off[T_RCP4] + 2 * e);
      iv q = isnan_(R.lo) ? div(P.g, ldiv(T + off[T_CR] + 2 * e)) : mul(P.g, R);
      q = mul(mul(q, ldiv(T + off[T_SNA] + 2 * e)), mk(k[4 + 2 * j], k[4 + 2 * j + 1]));
      q = add(q, ldiv(T + off[T_XD2] + 2 * e));
      iv X = ldiv(T + off[T_XI4] + 2 * e);
      return kkt_prune(q, X, D.dom[2 * j], D.dom[2 * j + 1]);
    }
  }
}

// 1 when the generalized KKT test rules the child out
__device__ __noinline__ int child_deriv(const Desc& D, const double* T, ChildCtx C, unsigned long long pc) {
  if (D.family == FAM_CODELIST) return cl_deriv(D, T, C, pc, 0, 1);
  DerivPre P;
  if (deriv_pre(D, T, C, pc, &P)) return 0;
  for (int j = 0; j < D.n; ++j)
    if (deriv_coord(D, T, C, pc, j, P)) return 1;
  return 0;
}

}  // namespace gg
