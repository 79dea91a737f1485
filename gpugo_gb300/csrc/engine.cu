// engine.cu -- persistent interval branch-and-bound engine for GB300 (sm_103a).
//
// One cooperative kernel runs the reference's iteration loop
// (GPUGO_1.1/1-Ackley/ackley50.py:950-1396) for every resident instance at once.
// Each iteration has four phases separated by grid barriers:
//
//   A  term tables for each instance's selected parent        (families.cuh)
//   B  children: lower bound, sample upper bounds -> atomicMin(UB), KKT test,
//      survivors appended to the instance's box pool          (sampling + ruleOutGPU,
//      in passes of at most the candidate queue's capacity     ackley50.py:602-766)
//   D  pool: drop entries with LB > UB when UB moved and an    (ackley50.py:1154-1166,
//      entry may lie above it, argmin; large lists per 2048-   :768-810, :1273)
//      entry tile streamed through shared memory by bulk copies
//   E  one warp per instance: pop the best entry, width/gap rule, decode the
//      next parent into the parent table                       (ackley50.py:1269-1370)
//
// Work in A, B and D is a flat list over (instance, item) built by the block that
// arrives last at the preceding barrier, so one instance or thousands share the
// same launch.  Samples of a child are evaluated only when its LB is not above the
// running UB: a skipped child's smallest sampled upper bound is at least its LB,
// which exceeds the UB, so the final UB of the iteration is unchanged.
// Every device-side wait is bounded by a %globaltimer budget.
#include <cuda_runtime.h>
#include <cooperative_groups.h>
#include <nvtx3/nvToolsExt.h>   // header-only: ranges are free unless a profiler is attached

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "ia.cuh"
#include "families.cuh"
#include "../../include/gpugo.h"

// Named ranges around the host entry points (admission, runs, result collection,
// whole solves) for nsys / ncu --nvtx.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

namespace gg {

constexpr int TD = 2048;           // pool entries per phase-D tile
constexpr int MAX_THREADS = 512;  // block size is 256 or 512

// instance life cycle
enum { ST_FREE = 0, ST_EXPAND = 1, ST_REPOP = 2, ST_DONE = 3 };

// Pools up to this many entries are compacted and searched by one block right
// after the instance's children are done; larger pools take the grid-wide path.
constexpr long long POOL_BLOCK_MAX = 1LL << 12;

// Candidate queue entry: slot << 32 | child code, LB bits, six intermediates of the
// value code list reused by the derivative test.
constexpr int CAND_WORDS = 4;   // key, LB, two words of value-pass intermediates

// Shared memory per block holding one instance's term tables during phase B.
constexpr int SMEM_TAB_BYTES = 96 * 1024;

struct State {
  int status;                 // ST_*
  int outcome;                // GPUGO_CERTIFIED / FINISHED / ITER_LIMIT or GPUGO_ERR_*
  int cur;                    // live pool buffer
  int cyc;                    // 1-based first split coordinate of the current parent
  long long iter;             // expansions so far == parent-table row of the current parent
  unsigned long long ub;      // ord_key of the UB (atomicMin target)
  unsigned long long ub_start;
  unsigned long long ub_who;  // row << 40 | code << 8 | sample index of the point that set the UB
  long long count;            // entries in the live buffer
  long long count_new;        // entries written to the other buffer by a grid-wide compaction
  long long count_before;     // live entries before this iteration's appends
  long long removed_new;      // this iteration's appends dropped by a grid-wide compaction
  long long out_count;        // boxes emitted by the width rule
  double out_lb_min;
  long long bounded;          // children bounded
  long long samples;          // children whose samples were evaluated
  long long ubc_count;        // UB candidates recorded this iteration
  long long m_children;       // children of the current parent
  long long b_done;           // (unused)
  unsigned long long seed_key;  // high half of the smallest candidate LB key << 32 | its child code
  long long cand_total;       // candidates queued this iteration
  long long cand_done;        // candidates processed this iteration
  int has_who;
  int pad;
  unsigned long long lb_max;  // ord_key at or above every list entry's LB (0: no entry yet)
};

struct Ctl {
  unsigned int bar_count;
  unsigned int bar_gen;
  int error;
  int nA;                     // instances expanding this iteration
  int nE;                     // instances active this iteration
  int nBig;                   // instances whose pool takes the grid-wide path
  long long totA, totB, totD; // flat work sizes
  long long iters;            // iterations run by the last launch
  int q_tail;                 // ready queue: slots reserved
  int q_head;                 // ready queue: slots claimed
  int n_big_q;                // big list length (appended during the children phase)
  unsigned int epoch;         // iteration tag of the ready-queue entries
  unsigned long long chunk_next;  // children phase: next chunk to hand out
  unsigned long long cand_tail;   // candidates of the pass (numbered across the instances' runs)
  unsigned long long cand_head;   // candidate queue: entries claimed in pass 2
  long long cand_claim;           // entries claimed per atomic in pass 2
  int seed_on;                    // run the seed pass this iteration
  int b_last;                     // the children pass [b_lo, b_hi) is the iteration's last
  long long b_lo, b_hi;           // flat children range of the current pass
};

struct KArgs {
  Desc* desc;
  State* st;
  Ctl* ctl;
  int* idsA;                  // [max_slots] expanding instances
  long long* prefA;           // [max_slots + 1] table items prefix
  long long* prefB;           // [max_slots + 1] children prefix
  int* idsE;                  // [max_slots] big-pool instances (grid-wide path)
  long long* prefD;           // [max_slots + 1] pool tiles prefix of big instances
  unsigned long long* queue;  // [max_slots] ready queue entries: epoch << 32 | slot
  unsigned long long* cands;  // [cand_cap][CAND_WORDS] candidate queue: slot << 32 | code, lb bits, aux
  long long* prefC;           // [max_slots + 1] candidates of the pass before each work-list position
  unsigned long long* cpass;  // [max_slots] candidates of the pass per work-list position (zero between passes)
  long long cand_cap;
  long long chunk;            // children bounded per pass (at most cand_cap)
  int cand_mode;              // GPUGO_CAND_AUTO / _WARP / _LANE
  int max_slots;
  int fam_hi;                 // highest family number resident (work lists are grouped up to it)
  long long max_iters;        // iterations in this launch (<= 0: until idle)
  unsigned long long timeout_ns;
  unsigned long long* stamps; // optional: %globaltimer at each barrier release
  long long stamp_cap;
  unsigned long long* bstamps; // optional: per block, per iteration: BSTAMP_W values inside phases A and B
  long long bstamp_iters;
  long long cur_it;            // iteration index for bstamps (set by the kernel loop)
};

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// per block and iteration: 0/1 table phase start/end, 2/3 pass 1 start/end,
// 4 pass 2 claims end, 5 list updates end, 6 pass 2 claims start, 7 candidates claimed
constexpr int BSTAMP_W = 8;
__device__ __forceinline__ void bstamp_val(const KArgs& a, int k, unsigned long long v) {
  if (a.bstamps && threadIdx.x == 0 && a.cur_it < a.bstamp_iters)
    a.bstamps[(a.cur_it * gridDim.x + blockIdx.x) * BSTAMP_W + k] = v;
}
__device__ __forceinline__ void bstamp(const KArgs& a, int k) { bstamp_val(a, k, gtimer()); }

__device__ __forceinline__ double atomic_ub_read(const unsigned long long* p) {
  return ord_val(*(volatile const unsigned long long*)p);
}

// Reads of values other blocks wrote during the current phase bypass L1.
template <typename T>
__device__ __forceinline__ T vload(const T& x) { return *(volatile const T*)&x; }

// ---------------------------------------------------------------------------
// block-wide helpers
// ---------------------------------------------------------------------------
template <typename T>
__device__ T block_exclusive_scan(T v, T* total) {
  __shared__ T s_warp[MAX_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    T w = (lane < nw) ? s_warp[lane] : (T)0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) s_warp[lane] = w;
  }
  __syncthreads();
  T base = (wid > 0) ? s_warp[wid - 1] : (T)0;
  T tot = s_warp[nw - 1];
  __syncthreads();
  *total = tot;
  return base + x - v;
}

struct Best {
  unsigned long long lbk, key, idx;
};

__device__ __forceinline__ bool best_less(const Best& x, const Best& y) {
  if (x.lbk != y.lbk) return x.lbk < y.lbk;
  return x.key < y.key;
}

__device__ __forceinline__ Best best_none() { Best b; b.lbk = ~0ULL; b.key = ~0ULL; b.idx = ~0ULL; return b; }

__device__ __forceinline__ Best warp_min(Best b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Best c;
    c.lbk = __shfl_xor_sync(0xffffffffu, b.lbk, o);
    c.key = __shfl_xor_sync(0xffffffffu, b.key, o);
    c.idx = __shfl_xor_sync(0xffffffffu, b.idx, o);
    if (best_less(c, b)) b = c;
  }
  return b;
}

// every thread of the block returns the block minimum
__device__ Best block_min(Best b) {
  __shared__ Best s_b[MAX_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  b = warp_min(b);
  if (lane == 0) s_b[wid] = b;
  __syncthreads();
  Best c = (lane < nw) ? s_b[lane] : best_none();
  c = warp_min(c);
  __syncthreads();
  return c;
}

// ---------------------------------------------------------------------------
// work lists (run by the last block at a barrier)
// ---------------------------------------------------------------------------
__device__ long long children_of(const Desc& D, int cyc) {
  int g = group_size(D.n, D.group, cyc);
  long long m = 1;
  for (int i = 0; i < g; ++i) m *= D.wid;
  return m;
}

// An iteration's children are bounded in passes of at most a.chunk children (the
// candidate queue's capacity unless the engine sets fewer), so that every
// candidate of a pass has a place in the queue however many children the
// iteration has (up to 2^32 for one instance).  Instances are updated after
// the last pass.
__device__ __forceinline__ void set_first_pass(const KArgs& a, long long totB) {
  a.ctl->b_lo = 0;
  a.ctl->b_hi = totB < a.chunk ? totB : a.chunk;
  a.ctl->b_last = totB <= a.chunk;
}

// Lists for the next iteration: expanding instances (tables, children) and the
// ready queue pre-filled with instances that only pop (width-rule emissions).
// Large batches list the expanding instances family by family: warps walk the
// work lists in order, so the SMs then run one family's code at a time instead
// of all four side by side (instruction-cache pressure).  Results do not depend
// on the order.
// At most 32 slots (single solves, small engines): warp 0 builds the lists with
// shuffles, no block barriers.
__device__ void build_lists_warp(const KArgs& a) {
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  const int s = lane;
  const bool have = s < a.max_slots;
  const int stt = have ? a.st[s].status : ST_DONE;
  const bool ex = stt == ST_EXPAND, rp = stt == ST_REPOP;
  const long long items = ex ? table_items(a.desc[s], a.st[s].cyc, false) : 0, kids = ex ? a.st[s].m_children : 0;
  const unsigned mA = __ballot_sync(0xffffffffu, ex), mR = __ballot_sync(0xffffffffu, rp);
  const unsigned mE = __ballot_sync(0xffffffffu, ex || rp);
  const unsigned below = (1u << lane) - 1u;
  long long pA = items, pB = kids;   // inclusive scans
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long ya = __shfl_up_sync(0xffffffffu, pA, o), yb = __shfl_up_sync(0xffffffffu, pB, o);
    if (lane >= o) { pA += ya; pB += yb; }
  }
  if (ex) {
    const int o = __popc(mA & below);
    a.idsA[o] = s;
    a.prefA[o] = pA - items;
    a.prefB[o] = pB - kids;
  }
  if (rp) a.queue[__popc(mR & below)] = ((unsigned long long)(a.ctl->epoch + 1) << 32) | (unsigned)s;
  const long long totA = __shfl_sync(0xffffffffu, pA, 31), totB = __shfl_sync(0xffffffffu, pB, 31);
  __syncwarp();
  if (lane == 0) {
    const int nA = __popc(mA);
    a.prefA[nA] = totA;
    a.prefB[nA] = totB;
    a.ctl->nA = nA;
    a.ctl->nE = __popc(mE);
    a.ctl->totA = totA;
    a.ctl->totB = totB;
    a.ctl->q_tail = __popc(mR);
    a.ctl->q_head = 0;
    a.ctl->n_big_q = 0;
    a.ctl->nBig = 0;
    a.ctl->epoch = a.ctl->epoch + 1;
    a.ctl->chunk_next = 0;
    a.ctl->cand_tail = 0;
    a.ctl->cand_head = 0;
    set_first_pass(a, totB);
  }
}

__device__ void build_lists(const KArgs& a) {
  const int S = a.max_slots;
  if (S <= 32) {
    build_lists_warp(a);
    return;
  }
  const int per = (S + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per, hi = min(S, lo + per);
  const int prev = a.ctl->nA;   // 0 before the first iteration of an engine
  const bool grouped = prev >= 128 || (prev == 0 && S >= 128);
  long long cE = 0, cR = 0;
  for (int s = lo; s < hi; ++s) {
    int stt = a.st[s].status;
    if (stt == ST_REPOP) cR++;
    if (stt == ST_EXPAND || stt == ST_REPOP) cE++;
  }
  long long tE, tR;
  block_exclusive_scan(cE, &tE);
  long long oR = block_exclusive_scan(cR, &tR);
  long long baseA = 0, baseSA = 0, baseSB = 0;
  for (int f = grouped ? 1 : 0; f <= (grouped ? a.fam_hi : 0); ++f) {
    long long cA = 0, sA = 0, sB = 0;
    for (int s = lo; s < hi; ++s) {
      if (a.st[s].status == ST_EXPAND && (f == 0 || a.desc[s].family == f)) {
        cA++; sA += table_items(a.desc[s], a.st[s].cyc, false); sB += a.st[s].m_children;
      }
    }
    long long tA, tSA, tSB;
    long long oA = baseA + block_exclusive_scan(cA, &tA);
    long long oSA = baseSA + block_exclusive_scan(sA, &tSA);
    long long oSB = baseSB + block_exclusive_scan(sB, &tSB);
    for (int s = lo; s < hi; ++s) {
      if (a.st[s].status == ST_EXPAND && (f == 0 || a.desc[s].family == f)) {
        a.idsA[oA] = s;
        a.prefA[oA] = oSA;
        a.prefB[oA] = oSB;
        oA++;
        oSA += table_items(a.desc[s], a.st[s].cyc, false);
        oSB += a.st[s].m_children;
      }
    }
    baseA += tA; baseSA += tSA; baseSB += tSB;
  }
  for (int s = lo; s < hi; ++s)
    if (a.st[s].status == ST_REPOP) a.queue[oR++] = ((unsigned long long)(a.ctl->epoch + 1) << 32) | (unsigned)s;
  __syncthreads();
  if (threadIdx.x == 0) {
    a.prefA[baseA] = baseSA;
    a.prefB[baseA] = baseSB;
    a.ctl->nA = (int)baseA;
    a.ctl->nE = (int)tE;
    a.ctl->totA = baseSA;
    a.ctl->totB = baseSB;
    a.ctl->q_tail = (int)tR;
    a.ctl->q_head = 0;
    a.ctl->n_big_q = 0;
    a.ctl->nBig = 0;
    a.ctl->epoch = a.ctl->epoch + 1;
    a.ctl->chunk_next = 0;
    a.ctl->cand_tail = 0;
    a.ctl->cand_head = 0;
    set_first_pass(a, baseSB);
  }
}

__device__ __forceinline__ long long pool_tiles(const Desc& D, const State& st) {
  long long c = st.count < D.pool_cap ? st.count : D.pool_cap;
  return (c + TD - 1) / TD;
}

// pool tiles of the big-pool instances (grid-wide path)
__device__ void build_list_big(const KArgs& a) {
  const int nB = a.ctl->n_big_q;
  const int per = (nB + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per, hi = min(nB, lo + per);
  long long t = 0;
  for (int k = lo; k < hi; ++k) t += pool_tiles(a.desc[a.idsE[k]], a.st[a.idsE[k]]);
  long long tot;
  long long o = block_exclusive_scan(t, &tot);
  for (int k = lo; k < hi; ++k) {
    a.prefD[k] = o;
    o += pool_tiles(a.desc[a.idsE[k]], a.st[a.idsE[k]]);
  }
  if (threadIdx.x == 0) {
    a.prefD[nB] = tot;
    a.ctl->totD = tot;
    a.ctl->nBig = nB;
  }
}

// Grid barrier; the last block to arrive runs `tail` before releasing the others.
// Returns false when an error is pending (a wait expired somewhere).
template <typename Tail>
__device__ bool grid_barrier(const KArgs& a, Tail tail) {
  __shared__ int s_last, s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int gen = *(volatile unsigned int*)&a.ctl->bar_gen;
    __threadfence();
    unsigned int arrived = atomicAdd(&a.ctl->bar_count, 1u);
    s_last = (arrived == gridDim.x - 1);
    s_ok = 1;
    if (!s_last) {
      unsigned long long t0 = gtimer();
      while (*(volatile unsigned int*)&a.ctl->bar_gen == gen) {
        if (*(volatile int*)&a.ctl->error) { s_ok = 0; break; }
        if (gtimer() - t0 > a.timeout_ns) {
          atomicCAS(&a.ctl->error, 0, GPUGO_ERR_TIMEOUT);
          s_ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  if (s_last) {
    tail();
    __syncthreads();
    if (threadIdx.x == 0) {
      a.ctl->bar_count = 0;
      __threadfence();
      atomicAdd(&a.ctl->bar_gen, 1u);
    }
  }
  __syncthreads();
  bool ok = s_ok && (*(volatile int*)&a.ctl->error == 0);
  __syncthreads();
  return ok;
}

struct NoTail { __device__ void operator()() const {} };

// list position k with pref[k] <= item < pref[k+1]; walks forward from a hint
__device__ __forceinline__ int find_seg(const long long* pref, int n, long long item, int hint) {
  int k = hint;
  if (k < 0 || k >= n || pref[k] > item) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (pref[mid] <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
  }
  while (k + 1 < n && pref[k + 1] <= item) k++;
  return k;
}

// ---------------------------------------------------------------------------
// phase A: term tables; items are dealt round-robin over the blocks so that the
// FP64 work of a single instance spreads over every SM
// ---------------------------------------------------------------------------
template <bool CL>
__device__ void phase_tables(const KArgs& a) {
  bstamp(a, 0);
  const long long tot = a.ctl->totA;
  const int nA = a.ctl->nA;
  const int lane = threadIdx.x & 31;
  // 32 consecutive items per warp (same instance, mostly the same coordinate and
  // digit), warps dealt round-robin over the blocks
  const long long W = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long w = ((long long)(threadIdx.x >> 5)) * gridDim.x + blockIdx.x;
  int hint = -1;
  for (long long base = w * 32; base < tot; base += W * 32) {
    long long it = base + lane;
    if (it >= tot) continue;
    int k = find_seg(a.prefA, nA, it, hint);
    hint = k;
    int s = a.idsA[k];
    const Desc& D = a.desc[s];
    const State& st = a.st[s];
    build_item<CL>(D, D.parents + 2LL * D.n * st.iter, D.pwid + (long long)D.n * st.iter, st.cyc, it - a.prefA[k],
                   false);
  }
  __syncthreads();
  bstamp(a, 1);
}

// ---------------------------------------------------------------------------
// selection: one warp finishes an instance's iteration
// ---------------------------------------------------------------------------
// The point that set the UB: the smallest recorded (code, sample) whose sampled
// upper bound equals the new UB.
__device__ void locate_who(const Desc& D, State& st) {
  const int lane = threadIdx.x & 31;
  const long long ubc = vload(st.ubc_count);
  long long nc = ubc < D.ubc_cap ? ubc : D.ubc_cap;
  const double ubv = ord_val(vload(st.ub));
  unsigned long long who = ~0ULL;
  for (long long c = lane; c < nc; c += 32) {
    double v = __ldcg(D.ubc_val + c);
    unsigned long long id = __ldcg(D.ubc_id + c);
    if (feq(v, ubv) && id < who) who = id;
  }
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long y = __shfl_xor_sync(0xffffffffu, who, o);
    who = y < who ? y : who;
  }
  if (lane == 0) {
    if (who != ~0ULL) { st.ub_who = ((unsigned long long)st.iter << 40) | who; st.has_who = 1; }
    else if (ubc > D.ubc_cap) st.has_who = 0;
  }
  __syncwarp();
}

// Pop the best list entry and apply the width / gap rules (ackley50.py:1269-1370).
// `cnt` live entries in buffer st.cur, `b` their minimum, `n_surv` survivors appended.
__device__ void finish_iteration(const Desc& D, State& st, Best b, long long cnt, long long n_surv,
                                 bool expanded) {
  const int lane = threadIdx.x & 31;
  const int n = D.n;
  // Every field read below is loaded up front, in one round of independent
  // loads, instead of one L2 round trip after another along the decisions.
  const int outcome0 = vload(st.outcome);
  const unsigned long long ubk = vload(st.ub);
  const long long iter = st.iter;
  const int cur = st.cur;
  const long long out_count = st.out_count;
  const double out_lb_min = st.out_lb_min;
  const long long bounded = st.bounded, m_children = st.m_children;
  const int stop_mode = D.stop_mode, max_cyc = D.max_cyc, group = D.group;
  const long long trace_cap = D.trace_cap, parent_cap = D.parent_cap, out_cap = D.out_cap, max_iter = D.max_iter;
  const double gap_tol = D.gap_tol, width_tol = D.width_tol;
  const bool have_best = !(cnt == 0 || b.idx == ~0ULL);
  const long long prow = (long long)(b.key >> 32);
  const unsigned long long code = b.key & 0xffffffffULL;
  // the selected entry's parent cycle and box, and the list's last entry (moved
  // into the selected slot), fetched together
  int pcyc = 1;
  double plo = 0.0, phi = 0.0, pwd = 0.0, last_lb = 0.0;
  unsigned long long last_key = 0;
  if (lane == 0 && have_best && outcome0 >= 0) {
    pcyc = D.pcyc[prow];
    plo = D.parents[2LL * n * prow];
    phi = D.parents[2LL * n * prow + 1];
    pwd = D.pwid[(long long)n * prow];
    last_lb = __ldcg(D.pool_lb[cur] + cnt - 1);
    last_key = __ldcg(D.pool_key[cur] + cnt - 1);
  }
  int decision = 0;  // 0 stop, 1 emit (pop again next iteration), 2 expand
  unsigned long long key = 0;
  int ccyc = 1;
  if (lane == 0) {
    st.count = cnt;
    if (expanded) {
      st.bounded = bounded + m_children;
      if (iter < trace_cap) {
        D.tr_ub[iter] = ord_val(ubk);
        D.tr_surv[iter] = n_surv;
        D.tr_pool[iter] = cnt;
        D.tr_sel[iter] = -1;
      }
    }
    if (outcome0 < 0) {
      decision = 0;
    } else if (!have_best) {
      st.outcome = GPUGO_FINISHED;
    } else {
      const double lbbest = ord_val(b.lbk);
      const double lbstar = flt(lbbest, out_lb_min) ? lbbest : out_lb_min;
      if (stop_mode == STOP_GAP && ord_val(ubk) - lbstar <= gap_tol) {
        st.outcome = GPUGO_CERTIFIED;
      } else {
        D.pool_lb[cur][b.idx] = last_lb;
        D.pool_key[cur][b.idx] = last_key;
        st.count = cnt - 1;
        key = b.key;
        ccyc = pcyc;
        const int gsz = group_size(n, group, ccyc);
        // child interval of coordinate 0 (child_iv on the prefetched parent values)
        iv x0 = mk(plo, phi);
        if (ccyc - 1 <= 0 && 0 < ccyc - 1 + gsz) {
          const int dg = digit(D, ccyc - 1, gsz, pack_code(D, gsz, code), 0);
          x0 = mk(__dadd_rn(__dmul_rn(pwd, u32_to_double(dg)), plo),
                  __dadd_rn(__dmul_rn(pwd, u32_to_double(dg + 1)), plo));
        }
        double width = __dsub_rn(x0.hi, x0.lo);
        if (width < width_tol && ccyc == max_cyc) {
          decision = 1;
          if (out_count < out_cap) { D.out_key[out_count] = key; D.out_lb[out_count] = lbbest; }
          st.out_count = out_count + 1;
          if (flt(lbbest, out_lb_min)) st.out_lb_min = lbbest;
        } else if (iter + 1 >= parent_cap) {
          st.outcome = GPUGO_ERR_PARENT_OVERFLOW;
        } else {
          decision = 2;
          if (iter < trace_cap) D.tr_sel[iter] = (long long)key;
        }
      }
    }
  }
  decision = __shfl_sync(0xffffffffu, decision, 0);
  key = __shfl_sync(0xffffffffu, key, 0);
  ccyc = __shfl_sync(0xffffffffu, ccyc, 0);
  if (decision == 2) {
    const long long row = (long long)(key >> 32);
    const double* pb = D.parents + 2LL * n * row;
    const double* pw = D.pwid + (long long)n * row;
    double* nb = D.parents + 2LL * n * (iter + 1);
    double* nw = D.pwid + (long long)n * (iter + 1);
    const int gsz = group_size(n, group, ccyc);
    const unsigned long long pc = pack_code(D, gsz, key & 0xffffffffULL);
    for (int i = lane; i < n; i += 32) {
      iv x = child_iv(D, pb, pw, ccyc - 1, gsz, i, digit(D, ccyc - 1, gsz, pc, i));
      nb[2 * i] = x.lo;
      nb[2 * i + 1] = x.hi;
      // a coordinate outside the split group keeps the parent's interval, so its
      // part width is the parent's (same operation on the same operands)
      const int k = i - (ccyc - 1);
      nw[i] = (k >= 0 && k < gsz) ? part_width(D, x.lo, x.hi) : pw[i];
    }
  }
  __syncwarp();
  if (lane == 0) {
    if (decision == 0) {
      st.status = ST_DONE;
      if (vload(st.outcome) == 0) st.outcome = GPUGO_FINISHED;
    } else if (decision == 1) {
      st.status = ST_REPOP;
    } else {
      const long long row = iter + 1;
      const int ncyc = (ccyc == max_cyc) ? 1 : ccyc + group;
      D.pcyc[row] = ncyc;
      st.iter = row;
      st.cyc = ncyc;
      st.m_children = children_of(D, ncyc);
      if (max_iter > 0 && row >= max_iter) {
        st.status = ST_DONE;
        st.outcome = GPUGO_ITER_LIMIT;
      } else {
        st.status = ST_EXPAND;
      }
    }
    st.ub_start = ubk;
    st.count_before = vload(st.count);
    st.ubc_count = 0;
    st.b_done = 0;
    st.cand_total = 0;
    st.cand_done = 0;
    st.seed_key = ~0ULL;
    st.removed_new = 0;
  }
  __syncwarp();
}

// ord_key of a UB with both zeros taken as +0 (list entries store -0 as +0)
__device__ __forceinline__ unsigned long long zkey(unsigned long long k) {
  return (k == ord_key(-0.0)) ? ord_key(0.0) : k;
}

// Whether the list update has entries to rule out: the UB moved this iteration
// and some entry's LB may lie above it (lb_max bounds them all from above).
// When no entry can be ruled out the list is left as it is: the compaction
// would keep every entry, and selection does not depend on their order.
__device__ __forceinline__ bool must_compact(unsigned long long ubk, unsigned long long ub_start,
                                             unsigned long long lb_max) {
  return ubk != ub_start && lb_max > zkey(ubk);
}

// Block-level list update of one instance whose children are all done:
// in-place compaction when the UB moved (list rule-out, ackley50.py:1154-1166),
// argmin (ackley50.py:1273), then the selection.
__device__ void block_instance(const KArgs& a, int s) {
  const Desc& D = a.desc[s];
  State& st = a.st[s];
  const bool expanded = (vload(st.status) == ST_EXPAND);
  const long long count = vload(st.count);
  long long cnt = count < D.pool_cap ? count : D.pool_cap;
  if (vload(st.outcome) < 0) cnt = 0;
  const unsigned long long ubk = vload(st.ub);
  const bool moved = ubk != vload(st.ub_start);
  const bool compact = must_compact(ubk, vload(st.ub_start), vload(st.lb_max));
  const double ub = ord_val(ubk);
  const long long before = vload(st.count_before);
  const int c = vload(st.cur);
  if (expanded && moved && threadIdx.x < 32) locate_who(D, st);
  Best b = best_none();
  long long kept = 0, removed_new = 0;
  for (long long base = 0; base < cnt; base += blockDim.x) {
    long long e = base + threadIdx.x;
    bool in = e < cnt;
    double lbv = in ? __ldcg(D.pool_lb[c] + e) : 0.0;
    unsigned long long key = in ? __ldcg(D.pool_key[c] + e) : 0ULL;
    bool keep = in && !(compact && flt(ub, lbv));
    if (in && !keep && e >= before) removed_new++;
    long long pos = e;
    if (compact) {
      long long tot;
      long long off = block_exclusive_scan((long long)keep, &tot);  // synchronises: all reads done
      pos = kept + off;
      if (keep) {
        D.pool_lb[c][pos] = lbv;
        D.pool_key[c][pos] = key;
      }
      kept += tot;
    }
    if (keep) {
      Best cb; cb.lbk = ord_key(lbv); cb.key = key; cb.idx = (unsigned long long)pos;
      if (best_less(cb, b)) b = cb;
    }
  }
  if (!compact) kept = cnt;
  long long rn;
  block_exclusive_scan(removed_new, &rn);
  b = block_min(b);
  if (compact && threadIdx.x == 0) st.lb_max = zkey(ubk);   // every kept LB is at most the UB
  if (threadIdx.x < 32) {
    long long n_surv = (cnt - before) - rn;
    finish_iteration(D, st, b, kept, n_surv, expanded);
  }
  __syncthreads();
}

// The same list update done by one warp, for small lists: the warp that finishes
// an instance's last candidate runs it at once (no ready-queue round trip, no
// block barriers).  Compaction positions come from ballots; every lane has read
// its entry before any lane of the chunk writes (positions never pass the entry
// being read).
constexpr long long POOL_WARP_MAX = 256;
__device__ void warp_instance(const KArgs& a, int s) {
  const int lane = threadIdx.x & 31;
  const Desc& D = a.desc[s];
  State& st = a.st[s];
  const bool expanded = (vload(st.status) == ST_EXPAND);
  const long long count = vload(st.count);
  long long cnt = count < D.pool_cap ? count : D.pool_cap;
  if (vload(st.outcome) < 0) cnt = 0;
  const unsigned long long ubk = vload(st.ub);
  const bool moved = ubk != vload(st.ub_start);
  const bool compact = must_compact(ubk, vload(st.ub_start), vload(st.lb_max));
  const double ub = ord_val(ubk);
  const long long before = vload(st.count_before);
  const int c = vload(st.cur);
  if (expanded && moved) locate_who(D, st);
  Best b = best_none();
  long long kept = 0, removed_new = 0;
  for (long long base = 0; base < cnt; base += 32) {
    const long long e = base + lane;
    const bool in = e < cnt;
    const double lbv = in ? __ldcg(D.pool_lb[c] + e) : 0.0;
    const unsigned long long key = in ? __ldcg(D.pool_key[c] + e) : 0ULL;
    const bool keep = in && !(compact && flt(ub, lbv));
    if (in && !keep && e >= base && e >= before) removed_new++;
    long long pos = e;
    if (compact) {
      const unsigned int km = __ballot_sync(0xffffffffu, keep);
      pos = kept + __popc(km & ((1u << lane) - 1u));
      if (keep) {
        D.pool_lb[c][pos] = lbv;
        D.pool_key[c][pos] = key;
      }
      kept += __popc(km);
    }
    if (keep) {
      Best cb; cb.lbk = ord_key(lbv); cb.key = key; cb.idx = (unsigned long long)pos;
      if (best_less(cb, b)) b = cb;
    }
  }
  if (!compact) kept = cnt;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) removed_new += __shfl_xor_sync(0xffffffffu, removed_new, o);
  b = warp_min(b);
  if (compact && lane == 0) st.lb_max = zkey(ubk);   // every kept LB is at most the UB
  finish_iteration(D, st, b, kept, (cnt - before) - removed_new, expanded);
}

// ---------------------------------------------------------------------------
// phase B: children; each block takes a contiguous range of the flat list
// ---------------------------------------------------------------------------
__device__ void drain_queue(const KArgs& a) {
  __shared__ int s_s;
  for (;;) {
    if (threadIdx.x == 0) {
      s_s = -1;
      for (;;) {
        int h = *(volatile int*)&a.ctl->q_head;
        int t = *(volatile int*)&a.ctl->q_tail;
        if (h >= t) break;
        if (atomicCAS(&a.ctl->q_head, h, h + 1) == h) {
          // the slot was reserved before q_tail moved; its entry lands right after
          const unsigned int ep = a.ctl->epoch;
          unsigned long long t0 = gtimer();
          unsigned long long v;
          while (((v = *(volatile unsigned long long*)&a.queue[h]) >> 32) != ep) {
            if (gtimer() - t0 > a.timeout_ns) { atomicCAS(&a.ctl->error, 0, GPUGO_ERR_TIMEOUT); break; }
          }
          s_s = ((v >> 32) == ep) ? (int)(v & 0xffffffffu) : -1;
          __threadfence();
          break;
        }
      }
    }
    __syncthreads();
    int s = s_s;
    __syncthreads();
    if (s < 0) return;
    const Desc& D = a.desc[s];
    const State& st = a.st[s];
    const long long cnt_now = vload(st.count);
    if ((cnt_now < D.pool_cap ? cnt_now : D.pool_cap) > POOL_BLOCK_MAX) {
      if (threadIdx.x == 0) {
        int k = atomicAdd(&a.ctl->n_big_q, 1);
        a.idsE[k] = s;
      }
      __syncthreads();
    } else {
      block_instance(a, s);
    }
    if (threadIdx.x == 0) __threadfence();
  }
}

__device__ __forceinline__ void queue_push(const KArgs& a, int s) {
  __threadfence();
  int slot = atomicAdd(&a.ctl->q_tail, 1);
  *(volatile unsigned long long*)&a.queue[slot] = ((unsigned long long)a.ctl->epoch << 32) | (unsigned)s;
  __threadfence();
}

// order used to pick a child's smallest sampled upper bound (see samp_better)
constexpr int J_NONE = 0x7fffffff;
__device__ __forceinline__ bool samp_less(double v, int j, double bv, int bj) {
  if (j == J_NONE) return false;
  if (bj == J_NONE) return true;
  return samp_better(v, j, bv, bj);
}

__device__ __forceinline__ double shfl_d(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// One candidate child (its LB is not above the running UB) processed by the whole
// warp: its sample points spread over the lanes, then its KKT coordinates.
// Returns true when the child survives.  Every lane returns the same value.
// pfx (may be null): the instance's shared sample prefixes.
template <bool CL>
__device__ bool warp_candidate(const KArgs& a, int s, const double* T, unsigned long long code, double lb,
                               const double* aux, const double* pfx) {
  const int lane = threadIdx.x & 31;
  const Desc& D = a.desc[s];
  State& st = a.st[s];
  ChildCtx C;
  C.c0 = st.cyc - 1;
  C.gsz = group_size(D.n, D.group, st.cyc);
  double ub = atomic_ub_read(&st.ub);
  if (flt(ub, lb)) return false;
  const unsigned long long pc = pack_code(D, C.gsz, code);
  double bv = 0.0;
  int bj = J_NONE;
  DerivPre P;
  P.g = mk(0.0, 0.0);
  P.u = P.g;
  int skip = 0;
  bool have_pre = false;
  if (D.family == FAM_EXPSQRT && 2 * D.S + 4 <= 32) {
    double v = 0.0;
    expsqrt_warp(D, T, C, pc, ub, &v, &P, &skip);
    if (lane < D.S) { bv = v; bj = lane; }
    have_pre = true;
  } else {
    for (int j = lane; j < D.S; j += 32) {
      double v = samp_one<CL>(D, T, C, pc, j, ub, pfx);
      if (samp_less(v, j, bv, bj)) { bv = v; bj = j; }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_xor_sync(0xffffffffu, bv, o);
    int oj = __shfl_xor_sync(0xffffffffu, bj, o);
    if (samp_less(ov, oj, bv, bj)) { bv = ov; bj = oj; }
  }
  double sm = bv;
  if (feq(sm, 0.0)) sm = 0.0;  // -0 -> +0
  if (lane == 0) {
    atomicAdd((unsigned long long*)&st.samples, 1ULL);
    if (flt(sm, ub)) {
      long long slot = atomicAdd((unsigned long long*)&st.ubc_count, 1ULL);
      if (slot < D.ubc_cap) {
        D.ubc_val[slot] = sm;
        D.ubc_id[slot] = (code << 8) | (unsigned long long)bj;
      }
      atomicMin(&st.ub, ord_key(sm));
    }
  }
  __syncwarp();
  ub = atomic_ub_read(&st.ub);
  ub = shfl_d(ub, 0);
  if (flt(ub, lb)) return false;
  if (!have_pre && (D.family == FAM_EXPSQRT || D.family == FAM_PRODCOS)) {
    if (lane == 0) {
      if (aux && D.family == FAM_PRODCOS) deriv_pre_aux(aux, &P);
      else skip = deriv_pre(D, T, C, pc, &P);
    }
    skip = __shfl_sync(0xffffffffu, skip, 0);
    P.g.lo = shfl_d(P.g.lo, 0); P.g.hi = shfl_d(P.g.hi, 0);
    P.u.lo = shfl_d(P.u.lo, 0); P.u.hi = shfl_d(P.u.hi, 0);
  }
  int pruned = 0;
  bool done = false;
  if constexpr (CL) {
    if (D.family == FAM_CODELIST) {
      pruned = cl_deriv(D, T, C, pc, lane, 32);
      done = true;
    }
  }
  {
    int klo, khi;
    kkt_span(D, C, &klo, &khi);
    if (!done && !skip)
      for (int j = klo + lane; j < khi && !pruned; j += 32) pruned = deriv_coord(D, T, C, pc, j, P);
  }
  return !__any_sync(0xffffffffu, pruned);
}

// Lanes per candidate in group_candidate for instance D (0: a warp per candidate).
__device__ __forceinline__ int group_lanes(const Desc& D) {
  return (D.S <= 16 && D.family != FAM_EXPSQRT) ? D.S : 0;
}

// Candidates of instances with S <= 16 samples (exp-sqrt excepted: it spreads
// its sums over 2S + 4 lanes) taken 32 / G at a time, G = S: group g (lanes
// g G .. g G + G - 1) processes candidate g, lane j of the group computing
// sample j, and its lanes then split the KKT coordinates.  An FP64 instruction
// costs the same for 10 active lanes as for 30, so three candidates of S = 10
// share what a warp per candidate pays for one.  has: the group holds a
// candidate (the other lanes only take part in the warp's shuffles).  Returns,
// on every lane of a group, whether its candidate survives.
template <bool CL>
__device__ __noinline__ bool group_candidate(const KArgs& a, int G, bool has, int s, const double* T,
                                             unsigned long long code, double lb, const double* aux, const double* pfx) {
  const int lane = threadIdx.x & 31;
  const int base = (lane / G) * G, lig = lane - base;
  const Desc& D = a.desc[has ? s : 0];
  State& st = a.st[has ? s : 0];
  ChildCtx C;
  C.c0 = has ? st.cyc - 1 : 0;
  C.gsz = has ? group_size(D.n, D.group, st.cyc) : 1;
  double ub = has ? atomic_ub_read(&st.ub) : 0.0;
  ub = __shfl_sync(0xffffffffu, ub, base);   // one view of the UB per group
  bool live = has && !flt(ub, lb);
  const unsigned long long pc = live ? pack_code(D, C.gsz, code) : 0ULL;
  double bv = 0.0;
  int bj = J_NONE;
  if (live && lig < D.S) {
    bv = samp_one<CL>(D, T, C, pc, lig, ub, pfx);
    bj = lig;
  }
  // minimum over the group's samples (segments of G lanes, G <= 16)
#pragma unroll
  for (int o = 1; o < 16; o <<= 1) {
    const double ov = __shfl_down_sync(0xffffffffu, bv, o);
    const int oj = __shfl_down_sync(0xffffffffu, bj, o);
    if (lig + o < G && samp_less(ov, oj, bv, bj)) { bv = ov; bj = oj; }
  }
  if (live && lig == 0) {
    double sm = bv;
    if (feq(sm, 0.0)) sm = 0.0;  // -0 -> +0
    atomicAdd((unsigned long long*)&st.samples, 1ULL);
    if (flt(sm, ub)) {
      long long slot = atomicAdd((unsigned long long*)&st.ubc_count, 1ULL);
      if (slot < D.ubc_cap) {
        D.ubc_val[slot] = sm;
        D.ubc_id[slot] = (code << 8) | (unsigned long long)bj;
      }
      atomicMin(&st.ub, ord_key(sm));
    }
  }
  __syncwarp();
  // the leader's view of the UB decides for the whole group
  ub = live ? atomic_ub_read(&st.ub) : 0.0;
  ub = __shfl_sync(0xffffffffu, ub, base);
  live = live && !flt(ub, lb);
  DerivPre P;
  P.g = mk(0.0, 0.0);
  P.u = P.g;
  if (live && D.family == FAM_PRODCOS) deriv_pre_aux(aux, &P);
  int pruned = 0;
  if (live) {
    bool done = false;
    if constexpr (CL) {
      if (D.family == FAM_CODELIST) {
        pruned = cl_deriv(D, T, C, pc, lig, G);
        done = true;
      }
    }
    if (!done) {
      int klo, khi;
      kkt_span(D, C, &klo, &khi);
      for (int j = klo + lig; j < khi && !pruned; j += G) pruned = deriv_coord(D, T, C, pc, j, P);
    }
  }
  const unsigned int pm = __ballot_sync(0xffffffffu, pruned != 0);
  const unsigned int gm = ((1u << G) - 1u) << base;
  return live && (pm & gm) == 0;
}

// thread_candidate for a code-list instance (one interpreter run per sample)
__device__ __noinline__ int thread_candidate_cl(const KArgs& a, int s, const double* T, unsigned long long code,
                                                double lb) {
  const Desc& D = a.desc[s];
  State& st = a.st[s];
  ChildCtx C;
  C.c0 = st.cyc - 1;
  C.gsz = group_size(D.n, D.group, st.cyc);
  double ub = atomic_ub_read(&st.ub);
  if (flt(ub, lb)) return 0;
  const unsigned long long pc = pack_code(D, C.gsz, code);
  for (int j = 0; j < D.S; ++j) {
    double v = cl_value(D, T, C, pc, j).hi;
    if (feq(v, 0.0)) v = 0.0;
    if (flt(v, ub)) {
      long long slot = atomicAdd((unsigned long long*)&st.ubc_count, 1ULL);
      if (slot < D.ubc_cap) {
        D.ubc_val[slot] = v;
        D.ubc_id[slot] = (code << 8) | (unsigned long long)j;
      }
      atomicMin(&st.ub, ord_key(v));
      ub = v;
    }
  }
  ub = atomic_ub_read(&st.ub);
  if (flt(ub, lb)) return 2;
  return cl_deriv(D, T, C, pc, 0, 1) ? 2 : 3;
}

// One candidate processed by one thread (long queues): the samples run one after
// the other and every sample value below the running UB lowers it (the minimum
// over all of them is the same value the per-child minimum would give).
// returns bit 0: the child survives, bit 1: its samples were evaluated
template <bool CL>
__device__ int thread_candidate(const KArgs& a, int s, const double* T, unsigned long long code, double lb,
                                const double* aux, const double* pfx) {
  if constexpr (CL) {
    if (a.desc[s].family == FAM_CODELIST) return thread_candidate_cl(a, s, T, code, lb);
  }
  const Desc& D = a.desc[s];
  State& st = a.st[s];
  ChildCtx C;
  C.c0 = st.cyc - 1;
  C.gsz = group_size(D.n, D.group, st.cyc);
  double ub = atomic_ub_read(&st.ub);
  if (flt(ub, lb)) return 0;
  const unsigned long long pc = pack_code(D, C.gsz, code);
  // Samples are evaluated four (then two, then one) at a time and considered in
  // index order.  A sample is recorded (for the minimiser point) only when it
  // lowers this lane's view of the UB: the first sample to reach the final UB
  // always does.
  auto consider = [&](double v, int j) {
    if (feq(v, 0.0)) v = 0.0;
    if (flt(v, ub)) {
      long long slot = atomicAdd((unsigned long long*)&st.ubc_count, 1ULL);
      if (slot < D.ubc_cap) {
        D.ubc_val[slot] = v;
        D.ubc_id[slot] = (code << 8) | (unsigned long long)j;
      }
      atomicMin(&st.ub, ord_key(v));
      ub = v;
    }
  };
  int j = 0;
  for (; j + 4 <= D.S; j += 4) {
    double v[4];
    samp_multi<4>(D, T, C, pc, j, v, ub, pfx);
#pragma unroll
    for (int q = 0; q < 4; ++q) consider(v[q], j + q);
  }
  if (j + 2 <= D.S) {
    double v[2];
    samp_multi<2>(D, T, C, pc, j, v, ub, pfx);
    consider(v[0], j);
    consider(v[1], j + 1);
    j += 2;
  }
  if (j < D.S) {
    double v[1];
    samp_multi<1>(D, T, C, pc, j, v, ub, pfx);
    consider(v[0], j);
  }
  ub = atomic_ub_read(&st.ub);
  if (flt(ub, lb)) return 2;
  DerivPre P;
  if (D.family == FAM_EXPSQRT) {
    if (deriv_pre(D, T, C, pc, &P)) return 3;
  } else if (D.family == FAM_PRODCOS) {
    deriv_pre_aux(aux, &P);
  }
  int klo, khi;
  kkt_span(D, C, &klo, &khi);
  for (int jj = klo; jj < khi; ++jj)
    if (deriv_coord(D, T, C, pc, jj, P)) return 2;
  return 3;
}

// Term tables of a single-instance iteration go to shared memory (when the block
// has enough work to pay for the copy): the blocks copy them in parallel, and
// every later access avoids an L2 round trip.
__device__ int stage_tables(const KArgs& a, bool worth = true) {
  extern __shared__ __align__(16) double s_tab[];
  if (a.ctl->nA != 1 || !worth) return -1;
  const int si = a.idsA[0];
  const Desc& D = a.desc[si];
  if (D.tab_doubles * 8 > SMEM_TAB_BYTES) return -1;
  const double2* src = (const double2*)D.tab;
  double2* dst = (double2*)s_tab;
  const long long n2 = (D.tab_doubles + 1) / 2;
  for (long long t = threadIdx.x; t < n2; t += blockDim.x) dst[t] = src[t];
  __syncthreads();
  return si;
}

// Survivors of one warp (lanes with keep set; lane i's child `code` of instance
// `s` with lower bound `lb`) appended to their instances' lists with one
// atomicAdd per instance present in the warp: lanes are grouped by instance with
// ballots and each takes its place from its rank in the group.  Every lane of
// the warp calls it.  Positions inside the list carry no meaning (selection ties
// are broken by the key), so any order of the appends gives the same solve.
__device__ __noinline__ void warp_append_survivors(const KArgs& a, bool keep, int s, unsigned long long code,
                                                      double lb) {
  const int lane = threadIdx.x & 31;
  unsigned int act = __ballot_sync(0xffffffffu, keep);
  while (act) {
    const int leader = __ffs(act) - 1;
    const int ls = __shfl_sync(0xffffffffu, s, leader);
    const unsigned int m = __ballot_sync(0xffffffffu, keep && s == ls);
    // the group's largest LB raises the instance's bound on its list's LBs
    unsigned long long mk = (keep && s == ls) ? ord_key(feq(lb, 0.0) ? 0.0 : lb) : 0ULL;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long y = __shfl_xor_sync(0xffffffffu, mk, o);
      mk = y > mk ? y : mk;
    }
    unsigned long long base = 0;
    if (lane == leader) {
      base = atomicAdd((unsigned long long*)&a.st[ls].count, (unsigned long long)__popc(m));
      atomicMax(&a.st[ls].lb_max, mk);
    }
    base = __shfl_sync(0xffffffffu, base, leader);
    if (keep && s == ls) {
      const Desc& D = a.desc[ls];
      State& st = a.st[ls];
      const long long pos = (long long)base + __popc(m & ((1u << lane) - 1u));
      if (pos < D.pool_cap) {
        D.pool_lb[st.cur][pos] = feq(lb, 0.0) ? 0.0 : lb;  // list keys order -0 before +0; LB comparisons do not
        D.pool_key[st.cur][pos] = ((unsigned long long)st.iter << 32) | code;
      } else {
        atomicCAS(&st.outcome, 0, GPUGO_ERR_POOL_OVERFLOW);
      }
    }
    act &= ~m;
  }
}

// Pass 1: every child's lower bound (uniform cost, static interleave over warps);
// children whose LB is not above the UB go to the candidate queue.
template <bool CL>
__device__ void phase_bound(const KArgs& a) {
  bstamp(a, 2);
  extern __shared__ __align__(16) double s_tab[];
  const int si = stage_tables(a);
  const long long lo = vload(a.ctl->b_lo), tot = vload(a.ctl->b_hi);   // this pass's children
  const int nA = a.ctl->nA;
  const int lane = threadIdx.x & 31;
  const long long W = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long w = ((long long)(threadIdx.x >> 5)) * gridDim.x + blockIdx.x;
  int hint = -1;
  for (long long base = lo + w * 32; base < tot; base += W * 32) {
    long long it = base + lane;
    bool valid = it < tot;
    int k = valid ? find_seg(a.prefB, nA, it, hint) : -1;
    if (valid) hint = k;
    int s = valid ? a.idsA[k] : -1;
    double lb = 0.0;
    double aux[2] = {0, 0};
    unsigned long long code = 0;
    bool cand = false;
    if (valid) {
      const Desc& D = a.desc[s];
      const State& st = a.st[s];
      const double* T = (s == si) ? s_tab : D.tab;
      code = (unsigned long long)(it - a.prefB[k]);
      ChildCtx C;
      C.c0 = st.cyc - 1;
      C.gsz = group_size(D.n, D.group, st.cyc);
      const unsigned long long pc = pack_code(D, C.gsz, code);
      lb = child_lb<CL>(D, T, C, pc, aux, ord_val(st.ub_start));
      cand = !flt(ord_val(st.ub_start), lb);
    }
    unsigned int cm = __ballot_sync(0xffffffffu, cand);
    if (!cm) continue;
    {
      // the lowest-LB candidate of each instance seeds the UB before pass 2
      unsigned long long sk = cand ? (((ord_key(lb) >> 32) << 32) | code) : ~0ULL;
      unsigned int act = cm;
      while (act) {
        int leader = __ffs(act) - 1;
        int ls = __shfl_sync(0xffffffffu, s, leader);
        unsigned long long v = (cand && s == ls) ? sk : ~0ULL;
        for (int o = 16; o > 0; o >>= 1) {
          unsigned long long y = __shfl_xor_sync(0xffffffffu, v, o);
          v = y < v ? y : v;
        }
        if (lane == leader) atomicMin(&a.st[ls].seed_key, v);
        act &= ~__ballot_sync(0xffffffffu, cand && s == ls);
      }
    }
    // Candidates are stored in runs, one per instance: instance k's run starts
    // where its children of this pass start in the pass's flat range (so it
    // cannot overflow into the next run, and the pass has at most cand_cap
    // children).  Pass 2 then takes claims of one instance's candidates.
    unsigned long long pos = 0;
    unsigned int act = cm;
    while (act) {
      const int leader = __ffs(act) - 1;
      const int lk = __shfl_sync(0xffffffffu, k, leader);
      const unsigned int m = __ballot_sync(0xffffffffu, cand && k == lk);
      unsigned long long base = 0;
      if (lane == leader) {
        base = atomicAdd(&a.cpass[lk], (unsigned long long)__popc(m));
        atomicAdd((unsigned long long*)&a.st[s].cand_total, (unsigned long long)__popc(m));
      }
      base = __shfl_sync(0xffffffffu, base, leader);
      if (cand && k == lk) {
        const long long start = (a.prefB[k] > lo ? a.prefB[k] : lo) - lo;
        pos = (unsigned long long)start + base + __popc(m & ((1u << lane) - 1u));
      }
      act &= ~m;
    }
    if (cand) {
      unsigned long long* e = a.cands + CAND_WORDS * pos;
      e[0] = ((unsigned long long)s << 32) | code;
      e[1] = (unsigned long long)__double_as_longlong(lb);
#pragma unroll
      for (int q = 0; q < 2; ++q) e[2 + q] = (unsigned long long)__double_as_longlong(aux[q]);
    }
  }
  __syncthreads();
  bstamp(a, 3);
}

// Candidates per warp from which each lane takes its own candidate instead of a
// group of S lanes (or a whole warp) taking one.  A group spreads the S sample
// passes over S lanes (short latency); a lane per candidate keeps all 32 lanes
// busy but runs the S passes one after the other, in claims of 32 or 64 that
// leave warps idle when the queue is short.  Measured on the GB300 with the
// 1024-instance mixed batch (S = 10): 108.4 ms to certified at 24 per warp, 107.8
// at 32, 110.4 at 48, 124.2 at 96 and with no lane per candidate at all; with the
// later tail hand-out and seed threshold 102.3 at 16, 99.5 at 20, 99.6 at 24, 101.4
// at 32, 102.9 at 40.
constexpr long long LANE_FROM = 24;
// Candidates left per warp below which a lane-per-candidate pass hands its last
// candidates out TAIL_CLAIM at a time (three groups of ten lanes for S = 10).
// Measured with LANE_FROM 32: tails from 4, 8, 16, 32 per warp 105.6, 105.0,
// 102.1 (on the later per-instance queue runs; 102.9 at 8 there), 107.7 ms;
// claims of 1 107.8, of 6 102.6 (at 16 per warp).
constexpr unsigned long long TAIL_FROM = 16;
constexpr unsigned long long TAIL_CLAIM = 3;

// instances without queued candidates are ready for their list update at once
__device__ void prefill_ready(const KArgs& a) {
  const int nA = a.ctl->nA;
  // after the last children pass: instances whose candidates are all done (or
  // that had none) go to their list update at once
  if (vload(a.ctl->b_last)) {
    for (int k = threadIdx.x; k < nA; k += blockDim.x) {
      int s = a.idsA[k];
      if (vload(a.st[s].cand_total) == vload(a.st[s].cand_done)) queue_push(a, s);
    }
  }
  {
    // number the pass's candidates across the per-instance runs (prefC) and
    // clear the run counters for the next pass
    const int per = (nA + blockDim.x - 1) / blockDim.x;
    const int lo = threadIdx.x * per, hi = min(nA, lo + per);
    long long c = 0;
    for (int k = lo; k < hi; ++k) c += (long long)__ldcg(a.cpass + k);
    long long total;
    long long o = block_exclusive_scan(c, &total);
    for (int k = lo; k < hi; ++k) {
      a.prefC[k] = o;
      o += (long long)__ldcg(a.cpass + k);
      a.cpass[k] = 0ULL;
    }
    if (threadIdx.x == 0) {
      a.prefC[nA] = total;
      a.ctl->cand_tail = (unsigned long long)total;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    long long tot = (long long)vload(a.ctl->cand_tail);
    if (tot > a.cand_cap) tot = a.cand_cap;
    long long W = ((long long)gridDim.x * blockDim.x) >> 5;
    long long c = tot / (2 * W);
    // lane groups (or a warp) per candidate while there are fewer than LANE_FROM
    // candidates per warp; beyond that each lane takes its own, 32 per claim (claims
    // of 64 when the queue allowed: 99.9 ms on the 1024 batch against 99.6)
    long long k = (tot >= LANE_FROM * W) ? 32 : (c < 1 ? 1 : (c > 31 ? 31 : c));
    if (a.cand_mode == GPUGO_CAND_WARP && k >= 32) k = 31;
    if (a.cand_mode == GPUGO_CAND_LANE && k < 32) k = 32;
    a.ctl->cand_claim = k;
    a.ctl->cand_head = (k < 32) ? (unsigned long long)(W * k) : 0ULL;   // short queues: static first claims
    // the seed pass costs a sample chain per instance; it pays from 4 candidates
    // per warp with a single instance, from 16 in batches (measured: config 3
    // 3.86 ms seeding from 1 per warp, 3.88 from 4, 4.06 from 16; the 1024
    // batch 102.5, 102.2, 101.2 ms)
    a.ctl->seed_on = (tot > (nA <= 4 ? 4 : 16) * W) ? 1 : 0;
    a.ctl->cand_tail = (unsigned long long)tot;
  }
}

// Seed pass (long candidate queues): one warp per instance evaluates the samples
// of its lowest-LB candidate and lowers the UB with them.  The child is processed
// again in pass 2; the UB stays the minimum over the same set of sample values.
// The same warp stores the instance's shared sample prefixes (samp_prefix), which
// pass 2 then starts every candidate's sample passes from.
template <bool CL>
__device__ void phase_seed(const KArgs& a) {
  extern __shared__ __align__(16) double s_tab[];
  const int si = stage_tables(a);
  const int nA = a.ctl->nA;
  const int lane = threadIdx.x & 31;
  const int gw = ((threadIdx.x >> 5) * gridDim.x) + blockIdx.x;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int k = gw; k < nA; k += nwarps) {
    const int s = a.idsA[k];
    const Desc& D = a.desc[s];
    State& st = a.st[s];
    const unsigned long long sk = st.seed_key;
    if (sk == ~0ULL) continue;
    const unsigned long long code = sk & 0xffffffffULL;
    const double* T = (s == si) ? s_tab : D.tab;
    ChildCtx C;
    C.c0 = st.cyc - 1;
    C.gsz = group_size(D.n, D.group, st.cyc);
    const unsigned long long pc = pack_code(D, C.gsz, code);
    const double cut = atomic_ub_read(&st.ub);
    const int sh = samp_shared(D, C);
    double bv = 0.0;
    int bj = J_NONE;
    bool cl = false;
    if constexpr (CL) cl = D.family == FAM_CODELIST;
    for (int j = lane; j < D.S; j += 32) {
      double v;
      if (cl) {
        v = samp_one<CL>(D, T, C, pc, j);   // code lists: the value list at the sample point, no prefixes
      } else {
        SAcc r = (sh > 0) ? samp_prefix(D, T, C, j, D.tab + D.t_off[T_PFX]) : sacc_init(D);
        samp_run<1>(D, T, C, pc, j, sh, samp_terms(D), &r);
        v = samp_value(D, r, cut);
      }
      if (samp_less(v, j, bv, bj)) { bv = v; bj = j; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_xor_sync(0xffffffffu, bv, o);
      int oj = __shfl_xor_sync(0xffffffffu, bj, o);
      if (samp_less(ov, oj, bv, bj)) { bv = ov; bj = oj; }
    }
    if (lane == 0 && bj != J_NONE) {
      double sm = feq(bv, 0.0) ? 0.0 : bv;
      if (flt(sm, atomic_ub_read(&st.ub))) {
        long long slot = atomicAdd((unsigned long long*)&st.ubc_count, 1ULL);
        if (slot < D.ubc_cap) { D.ubc_val[slot] = sm; D.ubc_id[slot] = (code << 8) | (unsigned long long)bj; }
        atomicMin(&st.ub, ord_key(sm));
      }
    }
  }
}

// Pass 2: candidates claimed dynamically by warps; the warp finishing an
// instance's last candidate queues it for its list update.  Short queues give a
// group of S lanes (or a whole warp) to each candidate (samples and KKT
// coordinates across the lanes); long queues give each lane its own candidate.
// Called by one lane; returns true when these were the instance's last candidates.
__device__ __forceinline__ bool count_done(const KArgs& a, int s, long long n) {
  __threadfence();
  State& st = a.st[s];
  unsigned long long old = atomicAdd((unsigned long long*)&st.cand_done, (unsigned long long)n);
  return (long long)old + n == st.cand_total;
}

// Every lane of the warp: an instance whose candidates are all done gets its list
// update from this warp when the list is small, from a block (ready queue) otherwise.
__device__ __forceinline__ void instance_ready(const KArgs& a, int s) {
  const State& st = a.st[s];
  const long long count = vload(st.count);
  const long long cnt = count < a.desc[s].pool_cap ? count : a.desc[s].pool_cap;
  if (cnt <= POOL_WARP_MAX) {
    warp_instance(a, s);
  } else if ((threadIdx.x & 31) == 0) {
    queue_push(a, s);
  }
  __syncwarp();
}

// Queue position of candidate number q of the pass: instance k's candidates
// (numbers prefC[k] .. prefC[k + 1] - 1) lie in its run, which starts where its
// children of the pass start.  hint: the lane's last instance.
__device__ __forceinline__ unsigned long long cand_pos(const KArgs& a, unsigned long long q, long long b_lo, int nA,
                                                       int& hint) {
  const int k = find_seg(a.prefC, nA, (long long)q, hint);
  hint = k;
  const long long pb = a.prefB[k];
  return (unsigned long long)((pb > b_lo ? pb : b_lo) - b_lo + ((long long)q - a.prefC[k]));
}

template <bool CL>
__device__ void phase_candidates(const KArgs& a) {
  extern __shared__ __align__(16) double s_tab[];
  __shared__ unsigned int s_surv[MAX_THREADS / 32][64];
  __shared__ unsigned long long s_claimed;
  // a few candidates per block do not pay for copying the tables
  const int si = stage_tables(a, vload(a.ctl->cand_tail) >= 16ULL * gridDim.x);
  if (threadIdx.x == 0) s_claimed = 0;
  __syncthreads();
  bstamp(a, 6);
  const int lane = threadIdx.x & 31;
  const unsigned long long tot = vload(a.ctl->cand_tail);
  const unsigned long long K = (unsigned long long)vload(a.ctl->cand_claim);
  const bool pfx_on = vload(a.ctl->seed_on) != 0;   // the seed pass stored the shared sample prefixes
  // instances are updated only after the iteration's last children pass
  const bool last = vload(a.ctl->b_last) != 0;
  const long long b_lo = vload(a.ctl->b_lo);
  const int nA = a.ctl->nA;
  int chint = -1;
  // With a short queue (lane groups or a warp per candidate) the first claim of
  // warp g (numbered across the blocks first) is the range g*K: the candidates
  // land on warps of different SMs, which do not share an FP64 unit.  Later
  // claims, and every claim of a long queue, come from the shared counter.
  const unsigned long long g = (unsigned long long)(threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
  bool first = K < 32;
  for (;;) {
    unsigned long long h = g * K, Kc = K;
    if (!first) {
      if (lane == 0) {
        // The tail of a long queue goes to lane groups, a few candidates per
        // claim: a lane-per-candidate claim runs each lane's sample passes one
        // after the other, so the last such claims would keep a few warps busy
        // while all others wait.
        if (K >= 32) {
          const unsigned long long hd = vload(a.ctl->cand_head);
          const unsigned long long rem = hd < tot ? tot - hd : 0ULL;
          if (rem < TAIL_FROM * nwarps) Kc = TAIL_CLAIM;
        }
        h = atomicAdd(&a.ctl->cand_head, Kc);
      }
      h = __shfl_sync(0xffffffffu, h, 0);
      Kc = __shfl_sync(0xffffffffu, Kc, 0);
    }
    first = false;
    if (h >= tot) break;   // a static range past the end: the shared counter starts later still
    const unsigned long long e = min(tot, h + Kc);
    if (a.bstamps && lane == 0) atomicAdd(&s_claimed, e - h);
    if (Kc >= 32) {
      // One candidate per lane.  The claim is filtered first (LB against the
      // current UB) and the survivors are packed densely, so that no lane idles
      // through another lane's sample chains.
      unsigned int* surv = s_surv[threadIdx.x >> 5];
      int nsurv = 0;
      for (unsigned long long q0 = h; q0 < e; q0 += 32) {
        unsigned long long q = q0 + lane;
        bool valid = q < e;
        bool live = false;
        int s = -1;
        unsigned long long p = 0;
        if (valid) {
          p = cand_pos(a, q, b_lo, nA, chint);
          const unsigned long long* en = a.cands + CAND_WORDS * p;
          s = (int)(en[0] >> 32);
          double lb = __longlong_as_double((long long)en[1]);
          live = !flt(atomic_ub_read(&a.st[s].ub), lb);
        }
        unsigned int lm = __ballot_sync(0xffffffffu, live);
        // queue positions of the survivors (below cand_cap <= 2^24)
        if (live) surv[nsurv + __popc(lm & ((1u << lane) - 1u))] = (unsigned int)p;
        nsurv += __popc(lm);
        // candidates ruled out here are done
        unsigned int act = __ballot_sync(0xffffffffu, valid && !live);
        while (act) {
          int leader = __ffs(act) - 1;
          int ls = __shfl_sync(0xffffffffu, s, leader);
          unsigned int m = __ballot_sync(0xffffffffu, valid && !live && s == ls);
          {
            int fin = 0;
            if (lane == leader) fin = count_done(a, ls, __popc(m));
            if (__shfl_sync(0xffffffffu, fin, leader) && last) instance_ready(a, ls);
          }
          act &= ~m;
        }
      }
      __syncwarp();
      for (int r0 = 0; r0 < nsurv; r0 += 32) {
        int idx = r0 + lane;
        bool valid = idx < nsurv;
        int s = -1;
        bool keep = false, sampled = false;
        if (valid) {
          const unsigned long long q = surv[idx];
          const unsigned long long* en = a.cands + CAND_WORDS * q;
          s = (int)(en[0] >> 32);
          unsigned long long code = en[0] & 0xffffffffULL;
          double lb = __longlong_as_double((long long)en[1]);
          double aux[2];
#pragma unroll
          for (int t = 0; t < 2; ++t) aux[t] = __longlong_as_double((long long)en[2 + t]);
          const double* T = (s == si) ? s_tab : a.desc[s].tab;
          int rr = thread_candidate<CL>(a, s, T, code, lb, aux, pfx_on ? T + a.desc[s].t_off[T_PFX] : nullptr);
          keep = rr & 1;
          sampled = rr & 2;
        }
        {
          const unsigned long long q = valid ? surv[idx] : 0ULL;
          const unsigned long long code = valid ? (a.cands[CAND_WORDS * q] & 0xffffffffULL) : 0ULL;
          const double lb = valid ? __longlong_as_double((long long)a.cands[CAND_WORDS * q + 1]) : 0.0;
          warp_append_survivors(a, keep, s, code, lb);
        }
        unsigned int act = __ballot_sync(0xffffffffu, valid);
        while (act) {
          int leader = __ffs(act) - 1;
          int ls = __shfl_sync(0xffffffffu, s, leader);
          unsigned int m = __ballot_sync(0xffffffffu, valid && s == ls);
          unsigned int sm = __ballot_sync(0xffffffffu, valid && s == ls && sampled);
          int fin = 0;
          if (lane == leader) {
            if (sm) atomicAdd((unsigned long long*)&a.st[ls].samples, (unsigned long long)__popc(sm));
            fin = count_done(a, ls, __popc(m));
          }
          if (__shfl_sync(0xffffffffu, fin, leader) && last) instance_ready(a, ls);
          act &= ~m;
        }
      }
      __syncwarp();
      continue;
    }
    // Lane groups or a warp per candidate.  The claim (at most 32 entries) is
    // loaded by the lanes at once and filtered against the current UB; the
    // survivors of the filter are then processed a group size at a time
    // (group_candidate) or one after the other by the whole warp.
    {
      const unsigned long long q = h + lane;
      const bool valid = q < e;
      int s = -1;
      unsigned long long code = 0;
      double lb = 0.0, aux[2] = {0.0, 0.0};
      bool live = false;
      if (valid) {
        const unsigned long long* en = a.cands + CAND_WORDS * cand_pos(a, q, b_lo, nA, chint);
        const unsigned long long w0 = en[0];
        s = (int)(w0 >> 32);
        code = w0 & 0xffffffffULL;
        lb = __longlong_as_double((long long)en[1]);
        aux[0] = __longlong_as_double((long long)en[2]);
        aux[1] = __longlong_as_double((long long)en[3]);
        live = !flt(atomic_ub_read(&a.st[s].ub), lb);
      }
      unsigned int lm = __ballot_sync(0xffffffffu, live);
      bool kept = false;   // this lane's own entry survived
      // entries whose instance takes groups of S lanes (group_candidate)
      const int my_g = live ? group_lanes(a.desc[s]) : 0;
      while (lm) {
        const int b = __ffs(lm) - 1;
        const int G = __shfl_sync(0xffffffffu, my_g, b);
        if (G > 0) {
          // the next 32 / G live entries of the same group size, one per group
          unsigned int same = __ballot_sync(0xffffffffu, ((lm >> lane) & 1u) && my_g == G);
          unsigned int take = 0;
          for (int k = 32 / G; k > 0 && same; --k) {
            take |= same & (~same + 1u);
            same &= same - 1u;
          }
          lm &= ~take;
          // group g takes the g-th entry of `take`
          const int g = lane / G;
          unsigned int t = take;
          for (int k = 0; k < g && t; ++k) t &= t - 1u;
          const bool has = g < 32 / G && t != 0;
          const int src = has ? __ffs(t) - 1 : 0;
          const int gs = __shfl_sync(0xffffffffu, s, src);
          const unsigned long long gc = __shfl_sync(0xffffffffu, code, src);
          const double gl = shfl_d(lb, src);
          double ga[2];
          ga[0] = shfl_d(aux[0], src);
          ga[1] = shfl_d(aux[1], src);
          const double* T = !has ? nullptr : (gs == si) ? s_tab : a.desc[gs].tab;
          const bool keep = group_candidate<CL>(a, G, has, gs, T, gc, gl, ga,
                                                (has && pfx_on) ? T + a.desc[gs].t_off[T_PFX] : nullptr);
          // each entry of `take` reads its group's result from the group's first lane
          const bool mine = (take >> lane) & 1u;
          const int from = mine ? __popc(take & ((1u << lane) - 1u)) * G : 0;
          const bool k2 = __shfl_sync(0xffffffffu, keep, from);
          if (mine) kept = k2;
          continue;
        }
        lm &= lm - 1;
        const int cs = __shfl_sync(0xffffffffu, s, b);
        const unsigned long long cc = __shfl_sync(0xffffffffu, code, b);
        const double cl = shfl_d(lb, b);
        double ca[2];
        ca[0] = shfl_d(aux[0], b);
        ca[1] = shfl_d(aux[1], b);
        const double* T = (cs == si) ? s_tab : a.desc[cs].tab;
        const bool keep = warp_candidate<CL>(a, cs, T, cc, cl, ca, pfx_on ? T + a.desc[cs].t_off[T_PFX] : nullptr);
        if (lane == b) kept = keep;
      }
      warp_append_survivors(a, kept, s, code, lb);
      __syncwarp();
      // every entry of the claim is done: count them per instance
      unsigned int act = __ballot_sync(0xffffffffu, valid);
      while (act) {
        const int leader = __ffs(act) - 1;
        const int ls = __shfl_sync(0xffffffffu, s, leader);
        const unsigned int m = __ballot_sync(0xffffffffu, valid && s == ls);
        {
            int fin = 0;
            if (lane == leader) fin = count_done(a, ls, __popc(m));
            if (__shfl_sync(0xffffffffu, fin, leader) && last) instance_ready(a, ls);
          }
        act &= ~m;
      }
    }
    __syncwarp();
  }
  __syncthreads();
  bstamp(a, 4);
  bstamp_val(a, 7, s_claimed);
  drain_queue(a);
  __syncthreads();
  bstamp(a, 5);
}

// ---------------------------------------------------------------------------
// grid-wide path for large pools: compaction + per-tile argmin, then selection
// ---------------------------------------------------------------------------
// The list pass streams each tile's LB and key slices (2048 entries, 32 KB)
// from global memory into shared memory with bulk asynchronous copies
// (cp.async.bulk, completion counted in bytes on an mbarrier), three tiles in
// flight per block in the dynamic shared memory the tables use in the other
// phases.  While a tile is filtered and its survivors written, the copies of
// the next two are under way, so the block never waits for a whole round trip
// to memory per tile.
constexpr int POOL_STAGES = 3;
constexpr int POOL_STAGE_BYTES = TD * 16;   // LB slice, then key slice
static_assert(POOL_STAGES * POOL_STAGE_BYTES <= SMEM_TAB_BYTES, "pool stages exceed the dynamic shared memory");

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(unsigned long long* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for phase `parity` of an mbarrier: false when the budget ran out.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, unsigned long long budget_ns) {
  const unsigned long long t0 = gtimer();
  while (!mbar_try_wait(bar, parity))
    if (gtimer() - t0 > budget_ns) return false;
  return true;
}
// Global -> shared bulk copy whose completion is counted on `bar` (16-byte
// aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

struct PoolTile {
  long long lo, hi, count_before;
  double ub;
  int s, cur, compact, tile;
};

// Each warp filters its own contiguous quarter/eighth of a tile, reserves the
// places of its survivors with one atomicAdd and writes them in order (its
// stores are contiguous); the block meets once per tile, to combine the warps'
// minima and to hand the stage to the next copy.
__device__ void phase_pool(const KArgs& a) {
  extern __shared__ __align__(16) double s_tab[];
  __shared__ __align__(8) unsigned long long s_bar[POOL_STAGES];
  __shared__ PoolTile s_meta[POOL_STAGES];
  __shared__ Best s_wbest[2][MAX_THREADS / 32];   // per warp, double-buffered by tile parity
  __shared__ int s_fail;
  const long long tot = a.ctl->totD;
  const int nB = a.ctl->nBig;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int span = TD / nw;        // entries per warp and tile: 256 (8 warps) or 128 (16 warps)
  const int rounds = span >> 5;    // 8 or 4
  const long long mine = (long long)blockIdx.x < tot ? (tot - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  if (mine == 0) return;   // the same for every thread of the block
  char* smem = (char*)s_tab;
  // the current instance's fields (stable during this phase), kept by thread 0
  // in shared memory: consecutive tiles of a block mostly belong to one instance
  struct InstCache {
    PoolTile m;
    long long start, end, cnt;
    const double* lb;
    const unsigned long long* key;
    int k;
  };
  __shared__ InstCache s_inst;
  // thread 0: tile j of this block into stage j % POOL_STAGES.  Every thread has
  // finished with the stage's earlier contents (block barrier before the call);
  // the proxy fence orders those reads before the copy's writes.
  auto issue = [&](long long j) {
    const int k = (int)(j % POOL_STAGES);
    const long long t = blockIdx.x + j * gridDim.x;
    InstCache& c = s_inst;
    if (t >= c.end) {
      c.k = find_seg(a.prefD, nB, t, c.k);
      c.start = a.prefD[c.k];
      c.end = a.prefD[c.k + 1];
      c.m.s = a.idsE[c.k];
      const Desc& D = a.desc[c.m.s];
      const State& st = a.st[c.m.s];
      const long long count = vload(st.count);
      c.cnt = count < D.pool_cap ? count : D.pool_cap;
      const unsigned long long ubk = vload(st.ub);
      c.m.cur = vload(st.cur);
      c.m.compact = must_compact(ubk, vload(st.ub_start), vload(st.lb_max));
      c.m.ub = ord_val(ubk);
      c.m.count_before = vload(st.count_before);
      c.lb = D.pool_lb[c.m.cur];
      c.key = D.pool_key[c.m.cur];
    }
    PoolTile m = c.m;
    m.tile = (int)(t - c.start);
    m.lo = (long long)m.tile * TD;
    m.hi = min(c.cnt, m.lo + TD);
    s_meta[k] = m;
    // an even number of entries: 16-byte multiples from a 16 KB-aligned tile start
    const unsigned pair = (unsigned)((m.hi - m.lo) & ~1LL);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_arrive_expect_tx(&s_bar[k], pair * 16u);
    if (pair) {
      bulk_load(smem + k * POOL_STAGE_BYTES, c.lb + m.lo, pair * 8u, &s_bar[k]);
      bulk_load(smem + k * POOL_STAGE_BYTES + TD * 8, c.key + m.lo, pair * 8u, &s_bar[k]);
    }
  };
  if (threadIdx.x == 0) {
    s_inst.k = -1;
    s_inst.end = -1;
    for (int k = 0; k < POOL_STAGES; ++k) mbar_init(&s_bar[k], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_fail = 0;
    for (long long j = 0; j < mine && j < POOL_STAGES; ++j) issue(j);
  }
  __syncthreads();
  long long waited = 0;   // tiles whose copies this block has seen complete
  for (long long j = 0; j < mine; ++j) {
    const int k = (int)(j % POOL_STAGES);
    const unsigned parity = (unsigned)((j / POOL_STAGES) & 1);
    const bool ok = __all_sync(0xffffffffu, mbar_wait(&s_bar[k], parity, a.timeout_ns));
    Best b = best_none();
    if (ok) {
      const PoolTile m = s_meta[k];
      const Desc& D = a.desc[m.s];
      State& st = a.st[m.s];
      const double* slb = (const double*)(smem + k * POOL_STAGE_BYTES);
      const unsigned long long* skey = (const unsigned long long*)(smem + k * POOL_STAGE_BYTES + TD * 8);
      const long long n = m.hi - m.lo, pair = n & ~1LL;
      // entry i of the tile: from the stage, or (the odd last entry of a list, not
      // in the bulk copy) from global memory
      auto entry_lb = [&](long long i) { return i < pair ? slb[i] : __ldcg(D.pool_lb[m.cur] + m.lo + i); };
      auto entry_key = [&](long long i) { return i < pair ? skey[i] : __ldcg(D.pool_key[m.cur] + m.lo + i); };
      const long long w0 = (long long)wid * span;
      unsigned bal[TD / 256];   // survivors of each round of 32 (warp-uniform)
      unsigned tk = 0;
      long long removed_new = 0;
#pragma unroll
      for (int r = 0; r < TD / 256; ++r) {
        bal[r] = 0;
        if (r < rounds) {
          const long long i = w0 + r * 32 + lane;
          const bool in = i < n;
          const bool keep = in && (!m.compact || !flt(m.ub, entry_lb(i)));
          if (m.compact && in && !keep && m.lo + i >= m.count_before) removed_new++;
          bal[r] = __ballot_sync(0xffffffffu, keep);
          tk += __popc(bal[r]);
        }
      }
      unsigned long long base = 0;
      if (m.compact) {
        if (lane == 0 && tk) base = atomicAdd((unsigned long long*)&st.count_new, (unsigned long long)tk);
        base = __shfl_sync(0xffffffffu, base, 0);
      }
      unsigned pre = 0;
#pragma unroll
      for (int r = 0; r < TD / 256; ++r) {
        if (r < rounds) {
          const long long i = w0 + r * 32 + lane;
          if ((bal[r] >> lane) & 1u) {
            const double lv = entry_lb(i);
            const unsigned long long kv = entry_key(i);
            unsigned long long pos = (unsigned long long)(m.lo + i);
            if (m.compact) {
              pos = base + pre + __popc(bal[r] & ((1u << lane) - 1u));
              D.pool_lb[m.cur ^ 1][pos] = lv;
              D.pool_key[m.cur ^ 1][pos] = kv;
            }
            Best c; c.lbk = ord_key(lv); c.key = kv; c.idx = pos;
            if (best_less(c, b)) b = c;
          }
          pre += __popc(bal[r]);
        }
      }
      if (m.compact) {
        for (int o = 16; o > 0; o >>= 1) removed_new += __shfl_xor_sync(0xffffffffu, removed_new, o);
        if (lane == 0 && removed_new) atomicAdd((unsigned long long*)&st.removed_new, (unsigned long long)removed_new);
      }
    } else if (lane == 0) {
      atomicCAS(&a.ctl->error, 0, GPUGO_ERR_TIMEOUT);
      s_fail = 1;
    }
    b = warp_min(b);
    if (lane == 0) s_wbest[j & 1][wid] = b;
    __syncthreads();   // every warp is done with the stage and has posted its minimum
    if (s_fail) break;
    waited = j + 1;
    if (wid == 0) {
      Best c = lane < nw ? s_wbest[j & 1][lane] : best_none();
      c = warp_min(c);
      if (lane == 0) {
        const PoolTile& m = s_meta[k];
        unsigned long long* tb = a.desc[m.s].tile_best + 3 * m.tile;
        tb[0] = c.lbk; tb[1] = c.key; tb[2] = c.idx;
        if (j + POOL_STAGES < mine) issue(j + POOL_STAGES);
      }
    }
  }
  // after an expired wait: wait (bounded again) for the copies still in flight
  // before the shared memory is used for anything else
  if (s_fail && threadIdx.x == 0) {
    // at least two seconds, however short the engine's budget: a bulk copy
    // normally lands within microseconds
    const unsigned long long budget = a.timeout_ns > 2000000000ULL ? a.timeout_ns : 2000000000ULL;
    const long long issued = mine < waited + POOL_STAGES ? mine : waited + POOL_STAGES;
    for (long long j = waited; j < issued; ++j)
      mbar_wait(&s_bar[j % POOL_STAGES], (unsigned)((j / POOL_STAGES) & 1), budget);
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < POOL_STAGES; ++k) mbar_inval(&s_bar[k]);
  __syncthreads();
}

__device__ void phase_select_big(const KArgs& a) {
  const int nB = a.ctl->nBig;
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int k = gw; k < nB; k += nwarps) {
    int s = a.idsE[k];
    const Desc& D = a.desc[s];
    State& st = a.st[s];
    const bool expanded = (st.status == ST_EXPAND);
    const bool moved = st.ub != st.ub_start;
    const bool compact = must_compact(st.ub, st.ub_start, st.lb_max);
    long long cnt = st.count < D.pool_cap ? st.count : D.pool_cap;
    if (expanded && moved) locate_who(D, st);
    long long n_surv = (cnt - st.count_before) - (compact ? st.removed_new : 0);
    Best b = best_none();
    const long long tiles = pool_tiles(D, st);
    for (long long t = lane; t < tiles; t += 32) {
      const unsigned long long* tb = D.tile_best + 3 * t;
      Best c; c.lbk = tb[0]; c.key = tb[1]; c.idx = tb[2];
      if (best_less(c, b)) b = c;
    }
    b = warp_min(b);
    if (compact) {
      cnt = st.count_new;
      __syncwarp();
      if (lane == 0) { st.cur ^= 1; st.count_new = 0; st.lb_max = zkey(st.ub); }
      __syncwarp();
    }
    finish_iteration(D, st, b, cnt, n_surv, expanded);
  }
}

struct TailLists {
  const KArgs* a;
  __device__ void operator()() const { build_lists(*a); }
};
struct TailPrefill {
  const KArgs* a;
  __device__ void operator()() const { prefill_ready(*a); }
};
// the next children pass of the iteration
struct TailNextPass {
  const KArgs* a;
  __device__ void operator()() const {
    if (threadIdx.x == 0) {
      Ctl* c = a->ctl;
      const long long lo = c->b_hi, tot = c->totB;
      c->b_lo = lo;
      c->b_hi = (tot - lo < a->chunk) ? tot : lo + a->chunk;
      c->b_last = c->b_hi >= tot;
      c->cand_tail = 0;
      c->cand_head = 0;
    }
  }
};
struct TailAfterChildren {
  const KArgs* a;
  __device__ void operator()() const {
    const bool big = *(volatile int*)&a->ctl->n_big_q > 0;
    if (big) build_list_big(*a);
    else build_lists(*a);
  }
};

__device__ __forceinline__ void stamp(const KArgs& a, long long it, int k) {
  if (a.stamps && blockIdx.x == 0 && threadIdx.x == 0 && (it * 8 + k) < a.stamp_cap) {
    a.stamps[it * 8 + k] = gtimer();
    if (k == 2) {
      a.stamps[it * 8 + 5] = a.ctl->cand_tail;
      a.stamps[it * 8 + 6] = (unsigned long long)a.ctl->nA;
      a.stamps[it * 8 + 7] = (unsigned long long)a.ctl->totB;
    }
  }
}

// CL: the build that runs code-list instances (used while one is resident)
template <bool CL>
__global__ void __launch_bounds__(MAX_THREADS, 1) solve_kernel(KArgs a) {
  TailLists tl{&a};
  TailAfterChildren tc{&a};
  TailPrefill tp{&a};
  TailNextPass tn{&a};
  // queue entries of earlier launches carry stale epochs
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.max_slots; i += gridDim.x * blockDim.x) {
    a.queue[i] = 0ULL;
    a.cpass[i] = 0ULL;
  }
  if (!grid_barrier(a, tl)) return;
  long long it = 0;
  while (a.ctl->nE > 0 && (a.max_iters <= 0 || it < a.max_iters)) {
    a.cur_it = it;
    stamp(a, it, 0);
    phase_tables<CL>(a);
    if (!grid_barrier(a, NoTail{})) return;
    stamp(a, it, 1);
    for (;;) {   // the iteration's children, one pass of at most a.chunk after the other
      phase_bound<CL>(a);
      if (!grid_barrier(a, tp)) return;
      if (vload(a.ctl->seed_on)) {
        phase_seed<CL>(a);
        if (!grid_barrier(a, NoTail{})) return;
      }
      phase_candidates<CL>(a);
      if (vload(a.ctl->b_last)) break;
      if (!grid_barrier(a, tn)) return;
    }
    if (!grid_barrier(a, tc)) return;
    stamp(a, it, 2);
    if (a.ctl->nBig > 0) {
      phase_pool(a);
      if (!grid_barrier(a, NoTail{})) return;
      stamp(a, it, 3);
      phase_select_big(a);
      if (!grid_barrier(a, tl)) return;
    }
    stamp(a, it, 4);
    ++it;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl->iters = it;
}

// Results of finished instances, one block each, written as one record per
// instance into a buffer the host copies back at once (instead of copying each
// instance's list and parent table).  Record (doubles): [0] LB, [1] boxes k,
// [2, 2+k) their LBs, then k boxes of 2n endpoints, then the sample point that
// set the UB (n) and [end] 1 when it exists.  The k boxes are the emitted
// (width-rule) boxes first, then, in gap mode, the k - emitted smallest list
// entries in (LB, key) order -- the order the host path sorts into.
struct FinRec {
  long long slot, k, emitted, off;
};

__device__ void decode_box(const Desc& D, unsigned long long key, double* out) {
  const int n = D.n;
  const long long prow = (long long)(key >> 32);
  const int cyc = D.pcyc[prow];
  const int gsz = group_size(n, D.group, cyc);
  const unsigned long long pc = pack_code(D, gsz, key & 0xffffffffULL);
  const double* pb = D.parents + 2LL * n * prow;
  const double* pw = D.pwid + (long long)n * prow;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const iv x = child_iv(D, pb, pw, cyc - 1, gsz, i, digit(D, cyc - 1, gsz, pc, i));
    out[2 * i] = x.lo;
    out[2 * i + 1] = x.hi;
  }
}

__global__ void __launch_bounds__(256) finalize_kernel(const Desc* desc, const State* st, const FinRec* recs,
                                                       double* outbuf) {
  __shared__ double s_v[8];
  __shared__ unsigned long long s_k[8];
  const FinRec fr = recs[blockIdx.x];
  const Desc& D = desc[fr.slot];
  const State& S = st[fr.slot];
  const int n = D.n;
  double* o = outbuf + fr.off;
  double* lbs = o + 2;
  double* boxes = lbs + fr.k;
  double* xh = boxes + 2LL * n * fr.k;
  const long long cnt = S.count < D.pool_cap ? S.count : D.pool_cap;
  const double* plb = D.pool_lb[S.cur];
  const unsigned long long* pkey = D.pool_key[S.cur];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // LB: the smallest of the emitted boxes' LBs and the list's
  double m = S.out_lb_min;
  for (long long i = threadIdx.x; i < cnt; i += blockDim.x) m = flt(plb[i], m) ? plb[i] : m;
  for (int off = 16; off > 0; off >>= 1) {
    const double y = __shfl_xor_sync(0xffffffffu, m, off);
    m = flt(y, m) ? y : m;
  }
  if (lane == 0) s_v[wid] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = s_v[0];
    for (int w = 1; w < nw; ++w) b = flt(s_v[w], b) ? s_v[w] : b;
    o[0] = b;
    o[1] = (double)fr.k;
  }
  __syncthreads();
  for (long long i = 0; i < fr.emitted; ++i) {
    if (threadIdx.x == 0) lbs[i] = D.out_lb[i];
    decode_box(D, D.out_key[i], boxes + 2LL * n * i);
  }
  // the smallest list entries, one selection pass each, in (LB, key) order
  unsigned long long prev_lbk = 0, prev_key = 0;
  bool first = true;
  for (long long r = fr.emitted; r < fr.k; ++r) {
    unsigned long long bl = ~0ULL, bk = ~0ULL;
    for (long long i = threadIdx.x; i < cnt; i += blockDim.x) {
      const unsigned long long l = ord_key(plb[i]), k = pkey[i];
      const bool after = first || l > prev_lbk || (l == prev_lbk && k > prev_key);
      if (after && (l < bl || (l == bl && k < bk))) { bl = l; bk = k; }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const unsigned long long yl = __shfl_xor_sync(0xffffffffu, bl, off);
      const unsigned long long yk = __shfl_xor_sync(0xffffffffu, bk, off);
      if (yl < bl || (yl == bl && yk < bk)) { bl = yl; bk = yk; }
    }
    if (lane == 0) { s_k[wid] = bl; s_v[wid] = __longlong_as_double((long long)bk); }
    __syncthreads();
    bl = s_k[0]; bk = (unsigned long long)__double_as_longlong(s_v[0]);
    for (int w = 1; w < nw; ++w) {
      const unsigned long long yl = s_k[w], yk = (unsigned long long)__double_as_longlong(s_v[w]);
      if (yl < bl || (yl == bl && yk < bk)) { bl = yl; bk = yk; }
    }
    __syncthreads();
    if (threadIdx.x == 0) lbs[r] = ord_val(bl);
    decode_box(D, bk, boxes + 2LL * n * r);
    prev_lbk = bl; prev_key = bk; first = false;
  }
  // the sample point that set the UB
  const long long rows = (S.iter + 1 < D.parent_cap) ? S.iter + 1 : D.parent_cap;
  const long long prow = (long long)(S.ub_who >> 40);
  const bool has = S.has_who && prow < rows;
  if (has) {
    const unsigned long long key = ((unsigned long long)prow << 32) | ((S.ub_who >> 8) & 0xffffffffULL);
    const int j = (int)(S.ub_who & 0xff);
    const int cyc = D.pcyc[prow];
    const int gsz = group_size(n, D.group, cyc);
    const unsigned long long pc = pack_code(D, gsz, key & 0xffffffffULL);
    const double* pb = D.parents + 2LL * n * prow;
    const double* pw = D.pwid + (long long)n * prow;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const iv x = child_iv(D, pb, pw, cyc - 1, gsz, i, digit(D, cyc - 1, gsz, pc, i));
      xh[i] = sample_pt(x, D.S, j);
    }
  }
  if (threadIdx.x == 0) xh[n] = has ? 1.0 : 0.0;
}

// Admission of the problems submitted since the last run: one block per record
// (word offsets in offs): slot, 2n, ncoef, the Desc, the initial State, domain,
// coefficients, then segments (device address, bytes, payload in words) that a
// restored checkpoint carries (parent table, list, emitted boxes, trace).  The
// block writes them into place (the domain also as parent row 0) and derives
// the constants.
constexpr int DESC_WORDS = (int)((sizeof(Desc) + 7) / 8);
constexpr int STATE_WORDS = (int)((sizeof(State) + 7) / 8);
__global__ void admit_kernel(Desc* desc, State* st, const unsigned long long* stage, const long long* offs) {
  const unsigned long long* r = stage + offs[blockIdx.x];
  const int s = (int)r[0];
  const long long ndom = (long long)r[1], ncoef = (long long)r[2];
  const unsigned long long* dw = r + 3;
  const unsigned long long* sw = dw + DESC_WORDS;
  const double* dom = (const double*)(sw + STATE_WORDS);
  const double* coef = dom + ndom;
  unsigned long long* ddst = (unsigned long long*)(desc + s);
  unsigned long long* sdst = (unsigned long long*)(st + s);
  for (int i = threadIdx.x; i < DESC_WORDS; i += blockDim.x) ddst[i] = dw[i];
  for (int i = threadIdx.x; i < STATE_WORDS; i += blockDim.x) sdst[i] = sw[i];
  const Desc* hd = (const Desc*)dw;  // the record's copy (its pointers are device addresses)
  double* ddom = (double*)hd->dom;
  double* dcoef = (double*)hd->coef;
  for (long long i = threadIdx.x; i < ndom; i += blockDim.x) {
    ddom[i] = dom[i];
    hd->parents[i] = dom[i];
  }
  for (long long i = threadIdx.x; i < ncoef; i += blockDim.x) dcoef[i] = coef[i];
  if (threadIdx.x == 0) hd->pcyc[0] = 1;
  __syncthreads();
  const unsigned long long* sg = (const unsigned long long*)(coef + ncoef);
  const long long nseg = (long long)sg[0];
  sg += 1;
  for (long long q = 0; q < nseg; ++q) {
    unsigned char* dst = (unsigned char*)sg[0];
    const long long nbytes = (long long)sg[1];
    const unsigned char* src = (const unsigned char*)(sg + 2);
    for (long long i = threadIdx.x; i < nbytes; i += blockDim.x) dst[i] = src[i];
    sg += 2 + (nbytes + 7) / 8;
  }
  __syncthreads();
  if (threadIdx.x == 0) init_consts(desc[s]);
}

// standalone table build and per-child evaluation (gpugo_eval_children)
__global__ void eval_init_kernel(Desc* desc) {
  if (blockIdx.x == 0 && threadIdx.x == 0) init_consts(desc[0]);
}

__global__ void eval_tables_kernel(Desc* desc, int cyc) {
  const Desc& D = desc[0];
  const long long items = table_items(D, cyc, true);   // any parent box: every KKT flag
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < items; t += (long long)gridDim.x * blockDim.x)
    build_item(D, D.parents, D.pwid, cyc, t, true);
}

__global__ void eval_children_kernel(Desc* desc, int cyc, const unsigned long long* codes, long long m, double ub,
                                     double* lb_out, double* samp_out, int* flag_out) {
  const Desc& D = desc[0];
  ChildCtx C;
  C.c0 = cyc - 1;
  C.gsz = group_size(D.n, D.group, cyc);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (long long)gridDim.x * blockDim.x) {
    const unsigned long long pc = pack_code(D, C.gsz, codes[t]);
    double lb = child_lb(D, D.tab, C, pc);
    int jb;
    double sm = child_samp(D, D.tab, C, pc, &jb);
    lb_out[t] = lb;
    samp_out[t] = sm;
    flag_out[t] = flt(ub, lb) ? 1 : child_deriv(D, D.tab, C, pc);
  }
}

// ---------------------------------------------------------------------------
// result-box merging (rosenbrock50.py:926-1049, combine / connectivity)
// ---------------------------------------------------------------------------
// A new box joins the first root it is connected to: in every coordinate it lies
// inside the root, or |new.lo - root.hi| < tol and |new.hi - new.lo| < tol (the
// reference's second difference is the new box's own width); the root becomes
// the coordinate-wise hull.  Otherwise the box is a new root.  The boxes are
// taken in order (the result depends on it); one block tests the roots in
// parallel for each box.
__device__ __forceinline__ bool box_connected(const double* root, const double* nb, int n, double tol) {
  for (int i = 0; i < n; ++i) {
    const double rl = root[2 * i], rh = root[2 * i + 1], nl = nb[2 * i], nh = nb[2 * i + 1];
    if (rl <= nl && nl <= rh && rl <= nh && nh <= rh) continue;
    if (!(fabs(__dsub_rn(nl, rh)) < tol)) return false;
    if (!(fabs(__dsub_rn(nh, nl)) < tol)) return false;
  }
  return true;
}

__global__ void __launch_bounds__(256) combine_kernel(const double* boxes, long long nbox, int n, double tol,
                                                      double* roots, long long* nroots) {
  __shared__ long long s_nr, s_hit[8];
  if (threadIdx.x == 0) s_nr = 0;
  __syncthreads();
  for (long long b = 0; b < nbox; ++b) {
    const double* nb = boxes + 2LL * n * b;
    const long long nr = s_nr;
    long long mine = LLONG_MAX;
    for (long long r = threadIdx.x; r < nr; r += blockDim.x)
      if (box_connected(roots + 2LL * n * r, nb, n, tol)) { mine = r; break; }
    for (int o = 16; o > 0; o >>= 1) {
      long long y = __shfl_xor_sync(0xffffffffu, mine, o);
      mine = y < mine ? y : mine;
    }
    if ((threadIdx.x & 31) == 0) s_hit[threadIdx.x >> 5] = mine;
    __syncthreads();
    long long hit = LLONG_MAX;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) hit = s_hit[w] < hit ? s_hit[w] : hit;
    double* dst = roots + 2LL * n * (hit == LLONG_MAX ? nr : hit);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      if (hit == LLONG_MAX) {
        dst[2 * i] = nb[2 * i];
        dst[2 * i + 1] = nb[2 * i + 1];
      } else {
        // np.minimum(root, new) / np.maximum(root, new)
        if (!(dst[2 * i] < nb[2 * i])) dst[2 * i] = nb[2 * i];
        if (!(dst[2 * i + 1] > nb[2 * i + 1])) dst[2 * i + 1] = nb[2 * i + 1];
      }
    }
    __syncthreads();
    if (threadIdx.x == 0 && hit == LLONG_MAX) s_nr = nr + 1;
    __syncthreads();
  }
  if (threadIdx.x == 0) *nroots = s_nr;
}

// FP64 peak probe: 8 independent DFMA chains per thread, 4096 steps each
__global__ void __launch_bounds__(256) fp64_probe_kernel(double* out, double seed, int steps) {
  double a0 = seed + threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
  double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
  const double m = 0.999999999, c = 1e-9;
  for (int i = 0; i < steps; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = __fma_rn(a0, m, c); a1 = __fma_rn(a1, m, c); a2 = __fma_rn(a2, m, c); a3 = __fma_rn(a3, m, c);
      a4 = __fma_rn(a4, m, c); a5 = __fma_rn(a5, m, c); a6 = __fma_rn(a6, m, c); a7 = __fma_rn(a7, m, c);
    }
  }
  double r = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (r == 12345.0) out[blockIdx.x] = r;  // keeps the chains live
}

}  // namespace gg

// ===========================================================================
// host side
// ===========================================================================
using namespace gg;

namespace {

struct HostSlot {
  bool used = false;
  int64_t ticket = -1;
  gpugo_spec spec{};
  std::vector<double> dom, coef;
  size_t arena_off = 0, arena_bytes = 0;
  Desc desc{};
  double* boxes_out = nullptr;
  double* box_lb_out = nullptr;
  int64_t cap = 0;
  double* xhat_out = nullptr;
  gpugo_trace trace{};
  bool has_trace = false;
};

struct Arena {
  char* base = nullptr;
  size_t size = 0;
  std::map<size_t, size_t> free_;  // offset -> size
  void init(char* b, size_t s) { base = b; size = s; free_.clear(); free_[0] = s; }
  bool alloc(size_t bytes, size_t* off) {
    bytes = (bytes + 255) & ~size_t(255);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        size_t rem = it->second - bytes, noff = it->first + bytes;
        free_.erase(it);
        if (rem) free_[noff] = rem;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
    }
  }
  size_t free_bytes() const { size_t s = 0; for (auto& kv : free_) s += kv.second; return s; }
};

}  // namespace

struct gpugo_engine {
  int dev = 0, nsm = 0, threads = 256, blocks = 0;
  int max_slots = 0;
  int cand_mode = 0;
  double timeout_s = 60.0;
  cudaStream_t stream = nullptr;
  Desc* d_desc = nullptr;
  State* d_state = nullptr;
  Ctl* d_ctl = nullptr;
  int* d_ids = nullptr;          // idsA | idsE | init list
  unsigned long long* d_queue = nullptr;
  unsigned long long* d_cands = nullptr;
  long long cand_cap = 0;
  long long chunk = 0;           // children per pass (<= cand_cap)
  long long* d_pref = nullptr;   // prefA | prefB | prefD | prefC | cpass
  char* d_arena = nullptr;
  Arena arena;
  std::vector<HostSlot> slots;
  int free_from = 0;             // every slot below this index is in use
  std::vector<int> pending_init;
  // admissions since the last run, packed as records (admit_kernel's layout)
  std::vector<unsigned long long> stage;
  std::vector<long long> stage_offs;
  char* d_stage = nullptr;
  size_t d_stage_cap = 0;
  // results of finished instances (finalize_kernel records)
  char* d_fin = nullptr;
  size_t d_fin_cap = 0;
  int64_t next_ticket = 1;
  std::vector<State> h_state;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_run_ms = 0.0, total_run_ms = 0.0;
  int64_t launches = 0, iterations = 0, h2d = 0, d2h = 0;
  // phase timestamps (debug aid, enabled by GPUGO_PHASE_STAMPS=<file>)
  unsigned long long* d_stamps = nullptr;
  long long stamp_cap = 0;
  unsigned long long* d_bstamps = nullptr;
  long long bstamp_iters = 0;
  const char* stamp_path = nullptr;
};

namespace {

int cuda_err(cudaError_t e) {
  if (e == cudaSuccess) return GPUGO_OK;
  fprintf(stderr, "gpugo: CUDA error %s\n", cudaGetErrorString(e));
  return GPUGO_ERR_CUDA;
}
#define CK(x) do { int _r = cuda_err(x); if (_r) return _r; } while (0)

int ilog2_exact(int w) {
  if (w <= 0 || (w & (w - 1))) return -1;
  int l = 0;
  while ((1 << l) < w) ++l;
  return l;
}

// A compiled code list (GPUGO_CODELIST): the header, every index an instruction
// can form over the range of its loop or gradient section (coordinates,
// constants, registers), and that every register is written before it is read.
// The device interpreter relies on this and checks nothing itself.
// tb: the words of a term table when the code is its body (X read only as
// X[i + o] for the table's offsets o; no loops, no reductions); sec: the words
// of a tabled gradient section (X read only as X[j + o] for its offsets).
static int cl_check_code(const double* cf, int64_t I, int nins, int start, int len, int n, int64_t ncst, int nreg,
                         int jlo, int jhi, bool allow_j, uint32_t* written, const uint32_t* tb, int ntab,
                         const uint32_t* sec = nullptr) {
  if (start < 0 || len < 0 || (int64_t)start + len > nins) return GPUGO_ERR_INVALID;
  auto word = [&](int64_t k) { uint64_t u; memcpy(&u, cf + k, 8); return (uint32_t)u; };
  bool in_loop = tb != nullptr;
  int64_t lo = tb ? tb[CLT_LO] : 0, hi = tb ? tb[CLT_HI] : 0;
  for (int p = start; p < start + len; ++p) {
    const int64_t q = I + (int64_t)CL_INS * p;
    const uint32_t w0 = word(q);
    const int32_t i1 = (int32_t)word(q + 1), i2 = (int32_t)word(q + 2);
    const int op = (int)(w0 & 255u), d = (int)((w0 >> 8) & 255u), a = (int)((w0 >> 16) & 255u), b = (int)(w0 >> 24);
    int base = -1, per = 0;  // per > 0: index into the constants with this stride
    int64_t kbase = 0;
    uint32_t reads = 0;
    switch (op) {
      case CL_LDX: base = a; break;
      case CL_LDC: if (i2 < 0 || i2 >= ncst) return GPUGO_ERR_INVALID; break;
      case CL_LDI: if (i2 < 0 || (int64_t)i2 + 1 >= ncst) return GPUGO_ERR_INVALID; break;
      case CL_LDK: base = a; kbase = i2; per = 1; break;
      case CL_LDKI: base = a; kbase = i2; per = 2; break;
      case CL_TIMESK: case CL_PLUSK: base = b; kbase = i2; per = 1; reads = 1u << (a & 31); if (a >= nreg) return GPUGO_ERR_INVALID; break;
      case CL_ADD: case CL_MINUS: case CL_MUL: case CL_DIV:
        if (a >= nreg || b >= nreg) return GPUGO_ERR_INVALID;
        reads = (1u << a) | (1u << b);
        break;
      case CL_TIMES: case CL_PLUS:
        if (i2 < 0 || i2 >= ncst) return GPUGO_ERR_INVALID;
        // fall through
      case CL_SQR: case CL_SQRT: case CL_EXP: case CL_SIN: case CL_COS: case CL_MOV:
        if (a >= nreg) return GPUGO_ERR_INVALID;
        reads = 1u << a;
        break;
      case CL_LOOP:
        if (sec || tb || in_loop || i1 < 0 || i1 >= i2 || i2 > n) return GPUGO_ERR_INVALID;
        in_loop = true; lo = i1; hi = i2;
        continue;
      case CL_ENDLOOP:
        if (tb || !in_loop) return GPUGO_ERR_INVALID;
        in_loop = false;
        continue;
      case CL_TRED:
        if (sec || tb || i1 < 0 || i1 >= ntab || a >= nreg) return GPUGO_ERR_INVALID;
        reads = 1u << a;
        break;
      default:
        return GPUGO_ERR_INVALID;
    }
    if (tb && op == CL_LDX) {   // only X[i + o], o one of the table's offsets
      const uint32_t no = tb[CLT_NOFF];
      if (a != 1 || !((no > 0 && i1 == (int32_t)tb[CLT_OFF0]) || (no > 1 && i1 == (int32_t)tb[CLT_OFF1])))
        return GPUGO_ERR_INVALID;
    }
    if (sec && op == CL_LDX) {  // only X[j + o], o one of the section's offsets
      bool hit = false;
      for (uint32_t q = 0; q < sec[CLS_NOFF]; ++q) hit |= i1 == (int32_t)sec[CLS_OFF0 + q];
      if (a != 2 || !hit) return GPUGO_ERR_INVALID;
    }
    if (d >= nreg || (reads & ~*written)) return GPUGO_ERR_INVALID;
    if (base >= 0) {
      int64_t mn, mx;
      if (base == 0) { mn = mx = i1; }
      else if (base == 1) { if (!in_loop) return GPUGO_ERR_INVALID; mn = lo + i1; mx = hi - 1 + i1; }
      else if (base == 2) { if (!allow_j) return GPUGO_ERR_INVALID; mn = (int64_t)jlo + i1; mx = (int64_t)jhi - 1 + i1; }
      else return GPUGO_ERR_INVALID;
      if (mn < 0) return GPUGO_ERR_INVALID;
      if (per == 0) {
        if (mx >= n) return GPUGO_ERR_INVALID;
      } else if (kbase < 0 || kbase + per * mx + per - 1 >= ncst) {
        return GPUGO_ERR_INVALID;
      }
    }
    *written |= 1u << d;
  }
  return (in_loop && !tb) ? GPUGO_ERR_INVALID : GPUGO_OK;
}

int validate_codelist(const gpugo_spec* s) {
  const double* cf = s->coef;
  if (s->ncoef < CL_HEADER) return GPUGO_ERR_INVALID;
  auto word = [&](int64_t k, uint32_t* out) {
    uint64_t u; memcpy(&u, cf + k, 8);
    *out = (uint32_t)u;
    return (u >> 32) == 0;
  };
  uint32_t h[CL_HEADER];
  for (int k = 0; k < CL_HEADER; ++k) if (!word(k, &h[k])) return GPUGO_ERR_INVALID;
  if (h[CLH_MAGIC] != CL_MAGIC || (int)h[CLH_N] != s->n) return GPUGO_ERR_INVALID;
  if (h[CLH_NREG] < 1 || h[CLH_NREG] > CL_MAXREG || h[CLH_NINS] > (1u << 20) || h[CLH_NCST] > (1u << 26))
    return GPUGO_ERR_INVALID;
  if (h[CLH_NSEC] > (uint32_t)s->n || h[CLH_NTAB] > CL_MAXTAB) return GPUGO_ERR_INVALID;
  const int64_t U = CL_HEADER + (int64_t)CL_SEC * h[CLH_NSEC];
  const int64_t I = U + (int64_t)CL_TAB * h[CLH_NTAB];
  const int64_t C = I + (int64_t)CL_INS * h[CLH_NINS];
  if (s->ncoef < C + (int64_t)h[CLH_NCST]) return GPUGO_ERR_INVALID;
  for (int64_t k = CL_HEADER; k < C; ++k) { uint32_t t; if (!word(k, &t)) return GPUGO_ERR_INVALID; }
  const int n = s->n, nreg = (int)h[CLH_NREG], nins = (int)h[CLH_NINS], ntab = (int)h[CLH_NTAB];
  const int64_t ncst = h[CLH_NCST];
  for (int t = 0; t < ntab; ++t) {
    uint32_t tb[CL_TAB];
    for (int k = 0; k < CL_TAB; ++k) word(U + (int64_t)CL_TAB * t + k, &tb[k]);
    const uint32_t no = tb[CLT_NOFF];
    if (tb[CLT_LO] >= tb[CLT_HI] || tb[CLT_HI] > (uint32_t)n || tb[CLT_KIND] > 1 || no > 2) return GPUGO_ERR_INVALID;
    for (uint32_t k = 0; k < no; ++k) {
      const int64_t o = (int32_t)tb[CLT_OFF0 + k];
      if ((int64_t)tb[CLT_LO] + o < 0 || (int64_t)tb[CLT_HI] - 1 + o >= n) return GPUGO_ERR_INVALID;
    }
    if (no == 2 && tb[CLT_OFF0] == tb[CLT_OFF1]) return GPUGO_ERR_INVALID;
    double cells = 1.0;
    for (uint32_t k = 0; k < no; ++k) cells *= s->wid;
    if (cells > 4096.0 || tb[CLT_REG] >= (uint32_t)nreg) return GPUGO_ERR_INVALID;
    uint32_t wt = 0;
    if (cl_check_code(cf, I, nins, (int)tb[CLT_START], (int)tb[CLT_LEN], n, ncst, nreg, 0, 0, false, &wt, tb, ntab))
      return GPUGO_ERR_INVALID;
    if (!(wt & (1u << tb[CLT_REG]))) return GPUGO_ERR_INVALID;
  }
  uint32_t wv = 0;
  if (h[CLH_VL] < 1 || h[CLH_RES] >= (uint32_t)nreg) return GPUGO_ERR_INVALID;
  if (cl_check_code(cf, I, nins, (int)h[CLH_VS], (int)h[CLH_VL], n, ncst, nreg, 0, 0, false, &wv, nullptr, ntab))
    return GPUGO_ERR_INVALID;
  if (!(wv & (1u << h[CLH_RES]))) return GPUGO_ERR_INVALID;
  uint32_t wp = 0;
  if (cl_check_code(cf, I, nins, (int)h[CLH_PS], (int)h[CLH_PL], n, ncst, nreg, 0, 0, false, &wp, nullptr, ntab))
    return GPUGO_ERR_INVALID;
  if (h[CLH_SKIP] != CL_NONE && h[CLH_SKIP] >= (uint32_t)ncst) return GPUGO_ERR_INVALID;
  int prev_hi = 0;
  for (uint32_t q = 0; q < h[CLH_NSEC]; ++q) {
    uint32_t w[CL_SEC];
    for (int t = 0; t < CL_SEC; ++t) word(CL_HEADER + (int64_t)CL_SEC * q + t, &w[t]);
    const int lo = (int)w[0], hi = (int)w[1];
    const int32_t chk = (int32_t)w[5];
    if (lo < prev_hi || lo >= hi || hi > n) return GPUGO_ERR_INVALID;  // ascending, disjoint
    prev_hi = hi;
    if (w[4] >= (uint32_t)nreg || (w[6] != CL_NONE && w[6] >= (uint32_t)nreg)) return GPUGO_ERR_INVALID;
    if ((int64_t)lo + chk < 0 || (int64_t)hi - 1 + chk >= n) return GPUGO_ERR_INVALID;
    // a tabled section: its KKT flag per (j, digits of the coordinates j + o)
    if (w[CLS_TABLED] > 1) return GPUGO_ERR_INVALID;
    if (w[CLS_TABLED]) {
      const uint32_t no = w[CLS_NOFF];
      if (q >= (uint32_t)CL_FLAG_TABLES || no < 1 || no > 3) return GPUGO_ERR_INVALID;
      bool has_chk = false;
      double cells = 1.0;
      for (uint32_t a = 0; a < no; ++a) {
        const int64_t o = (int32_t)w[CLS_OFF0 + a];
        if ((int64_t)lo + o < 0 || (int64_t)hi - 1 + o >= n) return GPUGO_ERR_INVALID;
        for (uint32_t b = 0; b < a; ++b) if (w[CLS_OFF0 + b] == w[CLS_OFF0 + a]) return GPUGO_ERR_INVALID;
        has_chk |= o == chk;
        cells *= s->wid;
      }
      if (!has_chk || cells > 4096.0) return GPUGO_ERR_INVALID;
    }
    uint32_t ws = w[CLS_TABLED] ? 0u : wp;   // tabled sections read nothing from the prologue
    if (cl_check_code(cf, I, nins, (int)w[2], (int)w[3], n, ncst, nreg, lo, hi, true, &ws, nullptr, ntab,
                      w[CLS_TABLED] ? w : nullptr))
      return GPUGO_ERR_INVALID;
    if (!(ws & (1u << w[4])) || (w[6] != CL_NONE && !(ws & (1u << w[6])))) return GPUGO_ERR_INVALID;
  }
  return GPUGO_OK;
}

int validate(const gpugo_spec* s) {
  if (!s || !s->domain || !s->coef) return GPUGO_ERR_INVALID;
  if (s->family < 1 || s->family > 5) return GPUGO_ERR_INVALID;
  if (s->n < 1 || s->n > 16384) return GPUGO_ERR_INVALID;   // the reference goes up to 10 000 (levy10000.py)
  if (s->family == GPUGO_CHAINED && s->n < 2) return GPUGO_ERR_INVALID;
  if (s->wid < 2 || s->group < 1 || s->samples < 1 || s->samples > 255) return GPUGO_ERR_INVALID;
  if (s->stop_mode != GPUGO_STOP_WIDTH && s->stop_mode != GPUGO_STOP_GAP) return GPUGO_ERR_INVALID;
  int g = std::min(s->group, s->n);
  double m = std::pow((double)s->wid, (double)g);
  if (m > 4294967296.0) return GPUGO_ERR_INVALID;
  int dbits = 0;
  while ((1LL << dbits) < s->wid) ++dbits;
  if ((int64_t)dbits * g > 64) return GPUGO_ERR_INVALID;  // packed child codes (never with m <= 2^32)
  for (int i = 0; i < s->n; ++i)
    if (!(s->domain[2 * i] < s->domain[2 * i + 1])) return GPUGO_ERR_INVALID;
  int64_t need = 0;
  switch (s->family) {
    case GPUGO_COSQUAD: need = 3LL * s->n; break;
    case GPUGO_CHAINED: need = 2LL * (s->n - 1); break;
    case GPUGO_EXPSQRT: need = 2LL + s->n; break;
    case GPUGO_PRODCOS: need = 1; break;
    case GPUGO_CODELIST: return validate_codelist(s);
  }
  if (s->ncoef < need) return GPUGO_ERR_INVALID;
  if (s->family == GPUGO_EXPSQRT && !(s->coef[0] > 0 && s->coef[1] > 0)) return GPUGO_ERR_INVALID;
  if (s->family == GPUGO_PRODCOS && !(s->coef[0] > 0)) return GPUGO_ERR_INVALID;
  if (s->wid > 64 && s->family == GPUGO_CHAINED) return GPUGO_ERR_INVALID;  // w^3 gradient table
  return GPUGO_OK;
}

struct Layout {
  int64_t cst, tab, t_off[T_NOFF], a_items;
  int64_t cl_toff[2 * CL_FLAG_TABLES];
  int64_t pool_cap, parent_cap, tiles_cap, ubc_cap, out_cap, trace_cap;
  int64_t bytes;
  // byte offsets
  int64_t o_dom, o_coef, o_cst, o_tab, o_par, o_pw, o_pcyc, o_plb0, o_plb1, o_pk0, o_pk1, o_tile, o_ubcv, o_ubci,
      o_outk, o_outl, o_trub, o_trs, o_trp, o_trsel;
};

int64_t max_children(const gpugo_spec* s) {
  int g = std::min(s->group, s->n);
  int64_t m = 1;
  for (int i = 0; i < g; ++i) m *= s->wid;
  return m;
}

void layout(const gpugo_spec* s, int64_t out_cap, int64_t trace_cap, Layout* L) {
  const int64_t n = s->n, w = s->wid, S = s->samples;
  memset(L, 0, sizeof(*L));
  switch (s->family) {
    case GPUGO_COSQUAD: L->cst = 6 * n + 2; break;
    case GPUGO_CHAINED: L->cst = 8 * n; break;
    case GPUGO_EXPSQRT: L->cst = 8 + 3 * n; break;
    case GPUGO_CODELIST: L->cst = 0; break;
    default: L->cst = 4 + 2 * n; break;
  }
  int64_t o = 0;
  auto put = [&](int idx, int64_t doubles) { L->t_off[idx] = o; o += (doubles + 1) & ~int64_t(1); };
  switch (s->family) {
    case GPUGO_COSQUAD:
      put(T_LO, n * w); put(T_SHI, n * w * S); put(T_PRB, (n * w + 7) / 8);
      L->a_items = n * w * (S + 2) + 64;   // + the padding that aligns item kinds to warps
      break;
    case GPUGO_CHAINED:
      put(T_LO, (n - 1) * w * w); put(T_SHI, (n - 1) * w * w * S); put(T_PRB, (n * w * w * w + 7) / 8);
      L->a_items = (n - 1) * w * w * (S + 1) + n * w * w * w + 32;
      break;
    case GPUGO_CODELIST: {
      put(T_LO, 2 * n * w); put(T_SHI, n * w * S);
      L->a_items = n * w * (S + 1);
      // term tables: [S + 1 passes][hi - lo][w^offsets] intervals each
      auto word = [&](int64_t k) { uint64_t u; memcpy(&u, s->coef + k, 8); return (uint32_t)u; };
      const int64_t U = CL_HEADER + (int64_t)CL_SEC * word(CLH_NSEC);
      const int ntab = (int)word(CLH_NTAB);
      for (int t = 0; t < ntab; ++t) {
        const int64_t q = U + (int64_t)CL_TAB * t;
        int64_t cells = 1;
        for (uint32_t k = 0; k < word(q + CLT_NOFF); ++k) cells *= w;
        const int64_t items = (S + 1) * (int64_t)(word(q + CLT_HI) - word(q + CLT_LO)) * cells;
        L->cl_toff[t] = o;
        o += 2 * items;
        L->a_items += items;
      }
      // KKT flag tables of tabled sections: [hi - lo][w^offsets] doubles each
      for (uint32_t q = 0; q < word(CLH_NSEC) && q < (uint32_t)CL_FLAG_TABLES; ++q) {
        const int64_t b = CL_HEADER + (int64_t)CL_SEC * q;
        if (!word(b + CLS_TABLED)) continue;
        int64_t cells = 1;
        for (uint32_t k = 0; k < word(b + CLS_NOFF); ++k) cells *= w;
        const int64_t items = (int64_t)(word(b + CLS_HI) - word(b + CLS_LO)) * cells;
        L->cl_toff[CL_FLAG_TABLES + q] = o;
        o += items + (items & 1);
        L->a_items += items;
      }
      break;
    }
    case GPUGO_EXPSQRT:
      put(T_SQ, 2 * n * w); put(T_CS, 2 * n * w); put(T_XI, 2 * n * w); put(T_SN, 2 * n * w);
      put(T_ZB, (n * w + 7) / 8); put(T_SQS, 2 * n * w * S); put(T_CSS, 2 * n * w * S);
      L->a_items = n * w * (S + 2) + 64;
      break;
    default:
      put(T_CR, 2 * n * w); put(T_SQ4, 2 * n * w); put(T_SNA, 2 * n * w); put(T_XD2, 2 * n * w);
      put(T_XI4, 2 * n * w); put(T_CRS, 2 * n * w * S); put(T_SQS4, 2 * n * w * S); put(T_RCP4, 2 * n * w);
      L->a_items = n * w * (S + 2) + 64;
      break;
  }
  put(T_PFX, 3 * S);
  L->tab = o;
  const int64_t M = max_children(s);
  L->pool_cap = s->pool_cap > 0 ? s->pool_cap : std::max<int64_t>(1 << 19, std::min<int64_t>(16 * M, 1 << 26));
  L->parent_cap = s->parent_cap > 0 ? s->parent_cap : 2048;
  if (s->max_iter > 0) L->parent_cap = std::min<int64_t>(L->parent_cap, s->max_iter + 1);
  L->tiles_cap = (L->pool_cap + TD - 1) / TD;
  L->ubc_cap = 4096;
  L->out_cap = std::max<int64_t>(out_cap, 1);
  L->trace_cap = trace_cap;
  int64_t b = 0;
  auto take = [&](int64_t bytes) { int64_t r = b; b += (bytes + 255) & ~int64_t(255); return r; };
  L->o_dom = take(8 * 2 * n);
  L->o_coef = take(8 * std::max<int64_t>(s->ncoef, 1));
  L->o_cst = take(8 * L->cst);
  L->o_tab = take(8 * L->tab);
  L->o_par = take(8 * 2 * n * L->parent_cap);
  L->o_pw = take(8 * n * L->parent_cap);
  L->o_pcyc = take(4 * L->parent_cap);
  L->o_plb0 = take(8 * L->pool_cap);
  L->o_plb1 = take(8 * L->pool_cap);
  L->o_pk0 = take(8 * L->pool_cap);
  L->o_pk1 = take(8 * L->pool_cap);
  L->o_tile = take(24 * L->tiles_cap);
  L->o_ubcv = take(8 * L->ubc_cap);
  L->o_ubci = take(8 * L->ubc_cap);
  L->o_outk = take(8 * L->out_cap);
  L->o_outl = take(8 * L->out_cap);
  L->o_trub = take(8 * std::max<int64_t>(trace_cap, 1));
  L->o_trs = take(8 * std::max<int64_t>(trace_cap, 1));
  L->o_trp = take(8 * std::max<int64_t>(trace_cap, 1));
  L->o_trsel = take(8 * std::max<int64_t>(trace_cap, 1));
  L->bytes = b;
}

void fill_desc(const gpugo_spec* s, const Layout& L, char* base, Desc* D) {
  memset(D, 0, sizeof(*D));
  D->family = s->family; D->n = s->n; D->wid = s->wid; D->group = s->group; D->S = s->samples;
  D->stop_mode = s->stop_mode;
  D->max_cyc = 1 + s->group * ((s->n - 1) / s->group);
  D->wlog = ilog2_exact(s->wid);
  if (D->wlog >= 0) {
    D->dbits = D->wlog;
    D->wmag = 0;
  } else {
    int b = 0;
    while ((1LL << b) < s->wid) ++b;
    D->dbits = b;
    D->wmag = (~0ULL) / (unsigned long long)s->wid + 1ULL;
  }
  D->width_tol = s->width_tol; D->gap_tol = s->gap_tol;
  D->max_iter = s->max_iter;
  D->pool_cap = L.pool_cap; D->parent_cap = L.parent_cap; D->out_cap = L.out_cap; D->trace_cap = L.trace_cap;
  D->tiles_cap = L.tiles_cap; D->ubc_cap = L.ubc_cap; D->a_items = L.a_items;
  D->tab_doubles = L.tab;
  for (int i = 0; i < T_NOFF; ++i) D->t_off[i] = L.t_off[i];
  for (int i = 0; i < 2 * CL_FLAG_TABLES; ++i) D->cl_toff[i] = L.cl_toff[i];
  D->dom = (const double*)(base + L.o_dom);
  D->coef = (const double*)(base + L.o_coef);
  D->cst = (double*)(base + L.o_cst);
  D->tab = (double*)(base + L.o_tab);
  D->parents = (double*)(base + L.o_par);
  D->pwid = (double*)(base + L.o_pw);
  D->pcyc = (int*)(base + L.o_pcyc);
  D->pool_lb[0] = (double*)(base + L.o_plb0);
  D->pool_lb[1] = (double*)(base + L.o_plb1);
  D->pool_key[0] = (unsigned long long*)(base + L.o_pk0);
  D->pool_key[1] = (unsigned long long*)(base + L.o_pk1);
  D->tile_best = (unsigned long long*)(base + L.o_tile);
  D->ubc_val = (double*)(base + L.o_ubcv);
  D->ubc_id = (unsigned long long*)(base + L.o_ubci);
  D->out_key = (unsigned long long*)(base + L.o_outk);
  D->out_lb = (double*)(base + L.o_outl);
  D->tr_ub = (double*)(base + L.o_trub);
  D->tr_surv = (long long*)(base + L.o_trs);
  D->tr_pool = (long long*)(base + L.o_trp);
  D->tr_sel = (long long*)(base + L.o_trsel);
}

inline int64_t children_host(const gpugo_spec* s, int cyc) {
  int g = std::min(s->group, s->n - cyc + 1);
  int64_t m = 1;
  for (int i = 0; i < g; ++i) m *= s->wid;
  return m;
}

inline int digit_host(const gpugo_spec* s, int c0, int gsz, uint64_t code, int i) {
  int k = i - c0;
  if (k < 0 || k >= gsz) return 0;
  for (int t = 0; t < k; ++t) code /= (uint64_t)s->wid;
  return (int)(code % (uint64_t)s->wid);
}

// child box on the host; round-to-nearest arithmetic identical to child_iv
void child_box_host(const gpugo_spec* s, const double* pb, int cyc, uint64_t code, double* out) {
  const int n = s->n, c0 = cyc - 1, gsz = std::min(s->group, n - cyc + 1);
  for (int i = 0; i < n; ++i) {
    double lo = pb[2 * i], hi = pb[2 * i + 1];
    int k = i - c0;
    if (k >= 0 && k < gsz) {
      int d = digit_host(s, c0, gsz, code, i);
      volatile double w = (hi - lo) / (double)s->wid;
      volatile double a = w * (double)d;
      volatile double b = w * (double)(d + 1);
      out[2 * i] = a + lo;
      out[2 * i + 1] = b + lo;
    } else {
      out[2 * i] = lo;
      out[2 * i + 1] = hi;
    }
  }
}

inline double ord_val_host(uint64_t k) {
  uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
  double x;
  memcpy(&x, &u, 8);
  return x;
}
inline uint64_t ord_key_host(double x) {
  uint64_t u;
  memcpy(&u, &x, 8);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}

int collect(gpugo_engine* E, int slot, gpugo_result* res) {
  int64_t d2h0 = E->d2h;
  auto D2H = [&](void* dst, const void* src, size_t bytes) {
    E->d2h += (int64_t)bytes;
    return cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost);
  };
  HostSlot& h = E->slots[slot];
  const State& st = E->h_state[slot];
  const gpugo_spec* s = &h.spec;
  const Desc& D = h.desc;
  const int n = s->n;
  memset(res, 0, sizeof(*res));
  res->ub = ord_val_host(st.ub);
  res->boxes_bounded = st.bounded;
  res->samples_evaluated = st.samples;
  res->status = st.outcome;
  // rows 0..iter of the parent table were expanded, except a parent selected
  // right before the iteration limit
  res->iterations = (st.outcome == GPUGO_ITER_LIMIT) ? st.iter : st.iter + 1;
  const int64_t cnt = std::min<int64_t>(st.count, D.pool_cap);
  res->pool_size = cnt;
  std::vector<double> plb(cnt);
  std::vector<unsigned long long> pkey(cnt);
  if (cnt) {
    CK(D2H(plb.data(), D.pool_lb[st.cur], 8 * cnt));
    CK(D2H(pkey.data(), D.pool_key[st.cur], 8 * cnt));
  }
  const int64_t rows = std::min<int64_t>(st.iter + 1, D.parent_cap);
  std::vector<double> par(2 * n * rows);
  std::vector<int> pcyc(rows);
  CK(D2H(par.data(), D.parents, 8 * 2 * n * rows));
  CK(D2H(pcyc.data(), D.pcyc, 4 * rows));
  const int64_t nout = std::min<int64_t>(st.out_count, D.out_cap);
  std::vector<unsigned long long> okey(nout);
  std::vector<double> olb(nout);
  if (nout) {
    CK(D2H(okey.data(), D.out_key, 8 * nout));
    CK(D2H(olb.data(), D.out_lb, 8 * nout));
  }
  double lbstar = st.out_lb_min;
  for (int64_t i = 0; i < cnt; ++i) if (plb[i] < lbstar) lbstar = plb[i];
  res->lb = lbstar;
  int64_t written = 0;
  auto emit = [&](unsigned long long key, double lb) {
    if (written < h.cap && h.boxes_out) {
      int64_t prow = (int64_t)(key >> 32);
      child_box_host(s, &par[2 * n * prow], pcyc[prow], key & 0xffffffffULL, h.boxes_out + 2 * n * written);
      if (h.box_lb_out) h.box_lb_out[written] = lb;
      written++;
    }
  };
  for (int64_t i = 0; i < nout; ++i) emit(okey[i], olb[i]);
  int64_t total = st.out_count;
  if (s->stop_mode == GPUGO_STOP_GAP && cnt) {
    std::vector<int64_t> idx(cnt);
    for (int64_t i = 0; i < cnt; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int64_t x, int64_t y) {
      if (plb[x] != plb[y]) return plb[x] < plb[y];
      return pkey[x] < pkey[y];
    });
    for (int64_t i = 0; i < cnt && written < h.cap; ++i) emit(pkey[idx[i]], plb[idx[i]]);
    total += cnt;
  }
  res->n_boxes = total;
  res->n_out = (int32_t)written;
  res->has_xhat = 0;
  if (st.has_who && h.xhat_out) {
    int64_t prow = (int64_t)(st.ub_who >> 40);
    uint64_t code = (st.ub_who >> 8) & 0xffffffffULL;
    int j = (int)(st.ub_who & 0xff);
    if (prow < rows) {
      std::vector<double> box(2 * n);
      child_box_host(s, &par[2 * n * prow], pcyc[prow], code, box.data());
      for (int i = 0; i < n; ++i) {
        volatile double inc = (box[2 * i + 1] - box[2 * i]) / (double)(s->samples + 1);
        volatile double step = inc * (double)(j + 1);
        h.xhat_out[i] = box[2 * i] + step;
      }
      res->has_xhat = 1;
    }
  }
  if (h.has_trace && h.trace.cap > 0) {
    int64_t k = std::min<int64_t>(std::min<int64_t>(h.trace.cap, D.trace_cap), res->iterations);
    if (k > 0) {
      CK(D2H(h.trace.ub, D.tr_ub, 8 * k));
      CK(D2H(h.trace.n_surv, D.tr_surv, 8 * k));
      CK(D2H(h.trace.pool, D.tr_pool, 8 * k));
      CK(D2H(h.trace.sel, D.tr_sel, 8 * k));
    }
  }
  res->d2h_bytes = E->d2h - d2h0;
  return GPUGO_OK;
}

}  // namespace

extern "C" {

const char* gpugo_strerror(int code) {
  switch (code) {
    case GPUGO_OK: return "ok";
    case GPUGO_ERR_INVALID: return "invalid problem or argument";
    case GPUGO_ERR_CUDA: return "CUDA runtime error";
    case GPUGO_ERR_NOMEM: return "out of device or host memory";
    case GPUGO_ERR_POOL_OVERFLOW: return "box pool capacity exceeded";
    case GPUGO_ERR_PARENT_OVERFLOW: return "parent table capacity exceeded";
    case GPUGO_ERR_TIMEOUT: return "a bounded device wait expired";
    case GPUGO_ERR_BUSY: return "no free slot or pool memory";
    case GPUGO_ERR_NOT_FOUND: return "unknown ticket";
    case GPUGO_ERR_NO_DEVICE: return "no CUDA device";
    case GPUGO_ERR_SCRATCH_LIMIT: return "request exceeds the fixed scratch of gpugo_eval_children_static";
    case GPUGO_CERTIFIED: return "certified";
    case GPUGO_FINISHED: return "finished";
    case GPUGO_ITER_LIMIT: return "iteration limit";
  }
  return "unknown";
}

int gpugo_device_info(int32_t* sm_out, int32_t* num_sms_out) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return GPUGO_ERR_NO_DEVICE;
  int dev;
  CK(cudaGetDevice(&dev));
  cudaDeviceProp p;
  CK(cudaGetDeviceProperties(&p, dev));
  if (sm_out) *sm_out = p.major * 10 + p.minor;
  if (num_sms_out) *num_sms_out = p.multiProcessorCount;
  return GPUGO_OK;
}

int gpugo_combine(const double* boxes, int64_t nbox, int32_t n, double tol, double* roots_out, int64_t cap,
                  int64_t* nroots_out) {
  NvtxRange nvtx_range("gpugo_combine");
  if (nbox < 0 || n < 1 || cap < 0 || !nroots_out || (nbox > 0 && !boxes) || (cap > 0 && !roots_out) ||
      !(tol >= 0.0))
    return GPUGO_ERR_INVALID;
  *nroots_out = 0;
  if (nbox == 0) return GPUGO_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPUGO_ERR_NO_DEVICE;
  const size_t bytes = sizeof(double) * 2 * (size_t)n * (size_t)nbox;
  double *d_boxes = nullptr, *d_roots = nullptr;
  long long* d_nr = nullptr;
  int rc = GPUGO_OK;
  do {
    if ((rc = cuda_err(cudaMalloc(&d_boxes, bytes)))) break;
    if ((rc = cuda_err(cudaMalloc(&d_roots, bytes)))) break;
    if ((rc = cuda_err(cudaMalloc(&d_nr, sizeof(long long))))) break;
    if ((rc = cuda_err(cudaMemcpy(d_boxes, boxes, bytes, cudaMemcpyHostToDevice)))) break;
    combine_kernel<<<1, 256>>>(d_boxes, nbox, n, tol, d_roots, d_nr);
    if ((rc = cuda_err(cudaGetLastError()))) break;
    long long nr = 0;
    if ((rc = cuda_err(cudaMemcpy(&nr, d_nr, sizeof(long long), cudaMemcpyDeviceToHost)))) break;
    const int64_t k = std::min<int64_t>(nr, cap);
    if (k > 0 && (rc = cuda_err(cudaMemcpy(roots_out, d_roots, sizeof(double) * 2 * (size_t)n * (size_t)k,
                                           cudaMemcpyDeviceToHost))))
      break;
    *nroots_out = nr;
  } while (0);
  cudaFree(d_boxes);
  cudaFree(d_roots);
  cudaFree(d_nr);
  return rc;
}

int gpugo_fp64_peak(int32_t repeats, double* tflops_out, double* ms_out) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPUGO_ERR_NO_DEVICE;
  int dev;
  CK(cudaGetDevice(&dev));
  cudaDeviceProp p;
  CK(cudaGetDeviceProperties(&p, dev));
  int occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fp64_probe_kernel, 256, 0));
  const int blocks = p.multiProcessorCount * std::max(occ, 1);
  const int steps = 4096;
  double* d_out = nullptr;
  CK(cudaMalloc(&d_out, 8 * blocks));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int r = 0; r < std::max(repeats, 1) + 1; ++r) {
    cudaEventRecord(e0);
    fp64_probe_kernel<<<blocks, 256>>>(d_out, 1.0, steps);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && ms < best) best = ms;  // first launch is warm-up
  }
  int rc = cuda_err(cudaGetLastError());
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d_out);
  if (rc) return rc;
  const double flops = 2.0 * 8 * 16 * (double)steps * 256.0 * blocks;
  if (tflops_out) *tflops_out = flops / (best * 1e-3) / 1e12;
  if (ms_out) *ms_out = best;
  return GPUGO_OK;
}

int gpugo_instance_bytes(const gpugo_spec* spec, int64_t* bytes_out) {
  if (!bytes_out) return GPUGO_ERR_INVALID;
  int rc = validate(spec);
  if (rc) return rc;
  Layout L;
  layout(spec, 1, 0, &L);
  *bytes_out = L.bytes;
  return GPUGO_OK;
}

int gpugo_engine_create(const gpugo_engine_cfg* cfg, gpugo_engine** out) {
  if (!cfg || !out || cfg->max_slots < 1 || cfg->max_slots > 8192 || cfg->arena_bytes <= 0) return GPUGO_ERR_INVALID;
  if (cfg->cand_mode < GPUGO_CAND_AUTO || cfg->cand_mode > GPUGO_CAND_LANE) return GPUGO_ERR_INVALID;
  if (cfg->chunk_children < 0) return GPUGO_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPUGO_ERR_NO_DEVICE;
  gpugo_engine* E = new (std::nothrow) gpugo_engine();
  if (!E) return GPUGO_ERR_NOMEM;
  E->max_slots = cfg->max_slots;
  E->threads = cfg->threads > 0 ? cfg->threads : 256;
  if (E->threads != 256 && E->threads != 512) { delete E; return GPUGO_ERR_INVALID; }
  E->timeout_s = cfg->wait_timeout_s > 0 ? cfg->wait_timeout_s : 60.0;
  E->cand_mode = cfg->cand_mode;
  int rc = GPUGO_OK;
  do {
    if ((rc = cuda_err(cudaGetDevice(&E->dev)))) break;
    cudaDeviceProp p;
    if ((rc = cuda_err(cudaGetDeviceProperties(&p, E->dev)))) break;
    E->nsm = p.multiProcessorCount;
    if (!p.cooperativeLaunch) { rc = GPUGO_ERR_CUDA; break; }
    int occ = 0;
    // both builds of the persistent kernel must fit the same cooperative grid
    int occ_cl = 0;
    if ((rc = cuda_err(cudaFuncSetAttribute(solve_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_TAB_BYTES)))) break;
    if ((rc = cuda_err(cudaFuncSetAttribute(solve_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_TAB_BYTES)))) break;
    if ((rc = cuda_err(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, solve_kernel<false>, E->threads, SMEM_TAB_BYTES)))) break;
    if ((rc = cuda_err(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_cl, solve_kernel<true>, E->threads, SMEM_TAB_BYTES)))) break;
    occ = std::min(occ, occ_cl);
    if (occ < 1) { rc = GPUGO_ERR_CUDA; break; }
    if (cfg->blocks_per_sm > 0) occ = std::min(occ, cfg->blocks_per_sm);
    // an engine for a handful of solves is latency-bound: one block per SM halves
    // the arrivals at every grid barrier (measured faster on single solves)
    else if (cfg->max_slots <= 4) occ = std::min(occ, 1);
    E->blocks = occ * E->nsm;
    if ((rc = cuda_err(cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking)))) break;
    if ((rc = cuda_err(cudaMalloc(&E->d_desc, sizeof(Desc) * E->max_slots)))) break;
    if ((rc = cuda_err(cudaMalloc(&E->d_state, sizeof(State) * E->max_slots)))) break;
    if ((rc = cuda_err(cudaMemset(E->d_state, 0, sizeof(State) * E->max_slots)))) break;
    if ((rc = cuda_err(cudaMalloc(&E->d_ctl, sizeof(Ctl))))) break;
    if ((rc = cuda_err(cudaMemset(E->d_ctl, 0, sizeof(Ctl))))) break;
    if ((rc = cuda_err(cudaMalloc(&E->d_ids, sizeof(int) * 3 * E->max_slots)))) break;
    if ((rc = cuda_err(cudaMalloc(&E->d_queue, sizeof(unsigned long long) * E->max_slots)))) break;
    E->cand_cap = std::min<long long>(1LL << 24, std::max<long long>(1LL << 20, 8192LL * E->max_slots));
    if ((rc = cuda_err(cudaMalloc(&E->d_cands, 8 * CAND_WORDS * (size_t)E->cand_cap)))) break;
    E->chunk = cfg->chunk_children > 0 ? std::min<long long>(cfg->chunk_children, E->cand_cap) : E->cand_cap;
    if ((rc = cuda_err(cudaMalloc(&E->d_pref, sizeof(long long) * 5 * (E->max_slots + 1))))) break;
    if (cudaMalloc(&E->d_arena, (size_t)cfg->arena_bytes) != cudaSuccess) { cudaGetLastError(); rc = GPUGO_ERR_NOMEM; break; }
    E->arena.init(E->d_arena, (size_t)cfg->arena_bytes);
    if (const char* sp = getenv("GPUGO_PHASE_STAMPS")) {
      E->stamp_path = sp;
      E->stamp_cap = 8 * 65536;
      if ((rc = cuda_err(cudaMalloc(&E->d_stamps, 8 * E->stamp_cap)))) break;
      E->bstamp_iters = 64;
      if ((rc = cuda_err(cudaMalloc(&E->d_bstamps, 8 * BSTAMP_W * (size_t)E->bstamp_iters * E->blocks)))) break;
    }
    if ((rc = cuda_err(cudaEventCreate(&E->ev0)))) break;
    if ((rc = cuda_err(cudaEventCreate(&E->ev1)))) break;
  } while (0);
  if (rc) { gpugo_engine_destroy(E); return rc; }
  E->slots.resize(E->max_slots);
  E->h_state.resize(E->max_slots);
  *out = E;
  return GPUGO_OK;
}

int gpugo_engine_destroy(gpugo_engine* E) {
  if (!E) return GPUGO_OK;
  if (E->stream) cudaStreamSynchronize(E->stream);
  cudaFree(E->d_desc); cudaFree(E->d_state); cudaFree(E->d_ctl);
  cudaFree(E->d_ids); cudaFree(E->d_queue); cudaFree(E->d_cands); cudaFree(E->d_pref); cudaFree(E->d_arena); cudaFree(E->d_stamps); cudaFree(E->d_bstamps);
  cudaFree(E->d_stage);
  cudaFree(E->d_fin);
  if (E->ev0) cudaEventDestroy(E->ev0);
  if (E->ev1) cudaEventDestroy(E->ev1);
  if (E->stream) cudaStreamDestroy(E->stream);
  delete E;
  return GPUGO_OK;
}

int gpugo_engine_stats(gpugo_engine* E, gpugo_stats* out) {
  if (!E || !out) return GPUGO_ERR_INVALID;
  out->last_run_ms = E->last_run_ms;
  out->total_run_ms = E->total_run_ms;
  out->kernel_launches = E->launches;
  out->iterations = E->iterations;
  out->h2d_bytes = E->h2d;
  out->d2h_bytes = E->d2h;
  return GPUGO_OK;
}

int gpugo_engine_free_bytes(gpugo_engine* E, int64_t* free_out) {
  if (!E || !free_out) return GPUGO_ERR_INVALID;
  *free_out = (int64_t)E->arena.free_bytes();
  return GPUGO_OK;
}

}  // extern "C"

namespace {
// A payload piece of an admission record: bytes copied into the instance's region.
struct Piece {
  size_t arena_rel;     // destination: byte offset inside the instance's arena region
  const void* src;      // host bytes
  size_t bytes;
};

// Admission of one problem: a slot, an arena region, the record admit_kernel
// applies at the next run.  `saved` (may be null) replaces the initial state and
// `pieces` are copied into the region (a restored checkpoint).
int admit(gpugo_engine* E, const gpugo_spec* spec, double* boxes_out, double* box_lb_out, int64_t cap,
          double* xhat_out, gpugo_trace* trace, const State* saved, const std::vector<Piece>& pieces,
          int64_t* ticket_out) {
  if (!E) return GPUGO_ERR_INVALID;
  int rc = validate(spec);
  if (rc) return rc;
  // output sizes become device allocations: bounded before they are multiplied out
  if (cap > (1LL << 40) || (trace && trace->cap > (1LL << 40))) return GPUGO_ERR_INVALID;
  if (trace && trace->cap > 0 && (!trace->ub || !trace->n_surv || !trace->pool || !trace->sel))
    return GPUGO_ERR_INVALID;
  int slot = -1;
  for (int s = E->free_from; s < E->max_slots; ++s) if (!E->slots[s].used) { slot = s; break; }
  if (slot < 0) return GPUGO_ERR_BUSY;
  Layout L;
  layout(spec, cap, trace ? trace->cap : 0, &L);
  size_t off;
  if (!E->arena.alloc((size_t)L.bytes, &off)) return GPUGO_ERR_BUSY;
  HostSlot& h = E->slots[slot];
  h = HostSlot();
  h.used = true;
  E->free_from = slot + 1;
  h.ticket = E->next_ticket++;
  h.spec = *spec;
  h.dom.assign(spec->domain, spec->domain + 2 * spec->n);
  h.coef.assign(spec->coef, spec->coef + spec->ncoef);
  h.spec.domain = h.dom.data();
  h.spec.coef = h.coef.data();
  h.arena_off = off;
  h.arena_bytes = (size_t)L.bytes;
  h.boxes_out = boxes_out; h.box_lb_out = box_lb_out; h.cap = cap; h.xhat_out = xhat_out;
  if (trace) { h.trace = *trace; h.has_trace = true; }
  char* base = E->d_arena + off;
  fill_desc(&h.spec, L, base, &h.desc);
  State s0;
  memset(&s0, 0, sizeof(s0));
  s0.status = ST_EXPAND;
  s0.cyc = 1;
  double ub0 = spec->ub_init;
  if (ub0 == 0.0) ub0 = 0.0;
  s0.ub = ord_key_host(ub0);
  s0.ub_start = s0.ub;
  s0.seed_key = ~0ULL;
  s0.out_lb_min = INFINITY;
  s0.m_children = children_host(spec, 1);
  if (saved) s0 = *saved;
  // one record for admit_kernel; copied with the others when the engine next runs
  const size_t at = E->stage.size();
  size_t seg_words = 1;
  for (const Piece& pc : pieces) seg_words += 2 + (pc.bytes + 7) / 8;
  const size_t words = 3 + DESC_WORDS + STATE_WORDS + h.dom.size() + h.coef.size() + seg_words;
  E->stage.resize(at + words, 0ULL);
  unsigned long long* rec = E->stage.data() + at;
  rec[0] = (unsigned long long)slot;
  rec[1] = (unsigned long long)h.dom.size();
  rec[2] = (unsigned long long)h.coef.size();
  memcpy(rec + 3, &h.desc, sizeof(Desc));
  memcpy(rec + 3 + DESC_WORDS, &s0, sizeof(State));
  memcpy(rec + 3 + DESC_WORDS + STATE_WORDS, h.dom.data(), 8 * h.dom.size());
  memcpy(rec + 3 + DESC_WORDS + STATE_WORDS + h.dom.size(), h.coef.data(), 8 * h.coef.size());
  unsigned long long* sg = rec + 3 + DESC_WORDS + STATE_WORDS + h.dom.size() + h.coef.size();
  *sg++ = (unsigned long long)pieces.size();
  for (const Piece& pc : pieces) {
    sg[0] = (unsigned long long)(uintptr_t)(base + pc.arena_rel);
    sg[1] = (unsigned long long)pc.bytes;
    memcpy(sg + 2, pc.src, pc.bytes);
    sg += 2 + (pc.bytes + 7) / 8;
  }
  E->stage_offs.push_back((long long)at);
  E->pending_init.push_back(slot);
  if (ticket_out) *ticket_out = h.ticket;
  return GPUGO_OK;
}
}  // namespace

extern "C" {

int gpugo_submit(gpugo_engine* E, const gpugo_spec* spec, double* boxes_out, double* box_lb_out, int64_t cap,
                 double* xhat_out, gpugo_trace* trace, int64_t* ticket_out) {
  NvtxRange nvtx_range("gpugo_submit");
  return admit(E, spec, boxes_out, box_lb_out, cap, xhat_out, trace, nullptr, {}, ticket_out);
}

int gpugo_submit_batch(gpugo_engine* E, const gpugo_spec* specs, int64_t count, double* boxes_out,
                       double* box_lb_out, int64_t cap, double* xhat_out, int64_t* tickets_out,
                       int64_t* admitted_out) {
  NvtxRange nvtx_range("gpugo_submit_batch");
  if (!E || !admitted_out || count < 0 || (count > 0 && (!specs || !tickets_out))) return GPUGO_ERR_INVALID;
  *admitted_out = 0;
  if (cap < 0 || cap > (1LL << 40)) return GPUGO_ERR_INVALID;
  int64_t coords = 0;   // n_0 + ... + n_{i-1}
  for (int64_t i = 0; i < count; ++i) {
    // the byte offset of problem i's boxes, 16 * cap * coords, must be representable
    if (cap > 0 && coords > (INT64_MAX / 16) / cap) return GPUGO_ERR_INVALID;
    double* bx = boxes_out ? boxes_out + 2 * cap * coords : nullptr;
    double* bl = box_lb_out ? box_lb_out + cap * i : nullptr;
    double* xh = xhat_out ? xhat_out + coords : nullptr;
    const int rc = admit(E, &specs[i], bx, bl, cap, xh, nullptr, nullptr, {}, &tickets_out[i]);
    if (rc) return rc;
    coords += specs[i].n;   // validated by admit: 1..16384
    *admitted_out = i + 1;
  }
  return GPUGO_OK;
}

// ---------------------------------------------------------------------------
// checkpoint / resume of one instance (between runs)
// ---------------------------------------------------------------------------
}  // extern "C"
namespace {
struct CkptHeader {
  char magic[8];                      // "GPUGOCK2"
  int32_t family, n, wid, group, samples, stop_mode;
  double width_tol, gap_tol, ub_init;
  int64_t ncoef, max_iter, pool_cap, parent_cap;
  State st;
  int64_t rows, cnt, nout, ntrace;
};
const char CKPT_MAGIC[8] = {'G', 'P', 'U', 'G', 'O', 'C', 'K', '2'};
size_t pad8(size_t b) { return (b + 7) & ~size_t(7); }

// The kernels trust a restored solve as they trust one they built: every index
// its state and lists can form is checked here, so that a damaged or foreign
// buffer is refused instead of read out of bounds.  `o` points at the parent
// rows; the state is the one every iteration ends with (the checkpoint is taken
// between runs).
int check_restored(const gpugo_spec& sp, const CkptHeader& hd, const char* o) {
  const State& st = hd.st;
  const int n = sp.n;
  if (st.status != ST_EXPAND && st.status != ST_REPOP && st.status != ST_DONE) return GPUGO_ERR_INVALID;
  if (st.cyc < 1 || st.cyc > n || st.iter < 0 || st.iter + 1 != hd.rows) return GPUGO_ERR_INVALID;
  if (st.m_children != children_host(&sp, st.cyc)) return GPUGO_ERR_INVALID;
  if (st.out_count < hd.nout || st.count_before < 0 || st.count_before > hd.cnt || st.ubc_count < 0 ||
      st.cand_total < 0 || st.cand_done < 0 || st.removed_new < 0 || st.bounded < 0 || st.samples < 0)
    return GPUGO_ERR_INVALID;
  if (st.has_who && (int)(st.ub_who & 0xff) >= sp.samples) return GPUGO_ERR_INVALID;
  const char* q = o + 24 * (size_t)n * hd.rows;               // past the parent boxes and part widths
  std::vector<int64_t> nchild((size_t)hd.rows);
  for (int64_t r = 0; r < hd.rows; ++r) {
    int32_t c;
    memcpy(&c, q + 4 * r, 4);
    if (c < 1 || c > n) return GPUGO_ERR_INVALID;
    nchild[(size_t)r] = children_host(&sp, c);
  }
  q += pad8(4 * (size_t)hd.rows) + 8 * (size_t)hd.cnt;       // to the list keys
  auto keys_ok = [&](const char* k, int64_t m) {
    for (int64_t e = 0; e < m; ++e) {
      uint64_t key;
      memcpy(&key, k + 8 * e, 8);
      const uint64_t row = key >> 32;
      if (row >= (uint64_t)hd.rows || (int64_t)(key & 0xffffffffULL) >= nchild[(size_t)row]) return false;
    }
    return true;
  };
  if (!keys_ok(q, hd.cnt)) return GPUGO_ERR_INVALID;
  q += 8 * (size_t)hd.cnt;                                     // emitted boxes
  if (!keys_ok(q, hd.nout)) return GPUGO_ERR_INVALID;
  return GPUGO_OK;
}

// Header, problem and state of a checkpoint buffer, all checked; *rows_at is
// where the parent rows start.  The spec points into the buffer.
int parse_checkpoint(const void* buf, int64_t bytes, CkptHeader* hdp, gpugo_spec* sp, const char** rows_at) {
  if (!buf || bytes < (int64_t)sizeof(CkptHeader)) return GPUGO_ERR_INVALID;
  CkptHeader& hd = *hdp;
  memcpy(&hd, buf, sizeof(hd));
  // every count is bounded by the buffer before the sizes are multiplied out
  if (memcmp(hd.magic, CKPT_MAGIC, 8) != 0 || hd.n < 1 || hd.n > 16384 || hd.rows < 1 || hd.cnt < 0 ||
      hd.nout < 0 || hd.ntrace < 0 || hd.ncoef < 0 || hd.rows > bytes / 4 || hd.cnt > bytes / 16 ||
      hd.nout > bytes / 16 || hd.ntrace > bytes / 32 || hd.ncoef > bytes / 8)
    return GPUGO_ERR_INVALID;
  const int n = hd.n;
  const size_t total = pad8(sizeof(hd)) + 8 * (2 * (size_t)n + (size_t)hd.ncoef) + 8 * 3 * (size_t)n * hd.rows +
                       pad8(4 * (size_t)hd.rows) + 16 * (size_t)hd.cnt + 16 * (size_t)hd.nout +
                       32 * (size_t)hd.ntrace;
  if ((size_t)bytes < total) return GPUGO_ERR_INVALID;
  const char* o = (const char*)buf + pad8(sizeof(hd));
  const double* dom = (const double*)o; o += 16 * (size_t)n;
  const double* coef = (const double*)o; o += 8 * (size_t)hd.ncoef;
  memset(sp, 0, sizeof(*sp));
  sp->family = hd.family; sp->n = n; sp->wid = hd.wid; sp->group = hd.group; sp->samples = hd.samples;
  sp->stop_mode = hd.stop_mode; sp->width_tol = hd.width_tol; sp->gap_tol = hd.gap_tol; sp->ub_init = hd.ub_init;
  sp->domain = dom; sp->coef = coef; sp->ncoef = hd.ncoef; sp->max_iter = hd.max_iter;
  sp->pool_cap = hd.pool_cap; sp->parent_cap = hd.parent_cap;
  int rc = validate(sp);
  if (rc) return rc;
  Layout L;
  layout(sp, 1, 0, &L);   // list and parent capacities do not depend on the output sizes
  if (hd.rows > L.parent_cap || hd.cnt > L.pool_cap) return GPUGO_ERR_INVALID;
  if ((rc = check_restored(*sp, hd, o))) return rc;
  *rows_at = o;
  return GPUGO_OK;
}
}  // namespace
extern "C" {

int gpugo_checkpoint(gpugo_engine* E, int64_t ticket, void* buf, int64_t cap, int64_t* bytes_out) {
  NvtxRange nvtx_range("gpugo_checkpoint");
  if (!E || !bytes_out) return GPUGO_ERR_INVALID;
  int slot = -1;
  for (int s = 0; s < E->max_slots; ++s)
    if (E->slots[s].used && E->slots[s].ticket == ticket) { slot = s; break; }
  if (slot < 0) return GPUGO_ERR_NOT_FOUND;
  for (int p : E->pending_init)
    if (p == slot) return GPUGO_ERR_BUSY;   // not admitted to the device yet: run first
  const HostSlot& h = E->slots[slot];
  const State& st = E->h_state[slot];
  const Desc& D = h.desc;
  const int n = h.spec.n;
  CkptHeader hd;
  memset(&hd, 0, sizeof(hd));
  memcpy(hd.magic, CKPT_MAGIC, 8);
  hd.family = h.spec.family; hd.n = n; hd.wid = h.spec.wid; hd.group = h.spec.group;
  hd.samples = h.spec.samples; hd.stop_mode = h.spec.stop_mode;
  hd.width_tol = h.spec.width_tol; hd.gap_tol = h.spec.gap_tol; hd.ub_init = h.spec.ub_init;
  hd.ncoef = h.spec.ncoef; hd.max_iter = h.spec.max_iter; hd.pool_cap = h.spec.pool_cap;
  hd.parent_cap = h.spec.parent_cap;
  hd.st = st;
  hd.rows = std::min<int64_t>(st.iter + 1, D.parent_cap);
  hd.cnt = std::min<int64_t>(st.count, D.pool_cap);
  hd.nout = std::min<int64_t>(st.out_count, D.out_cap);
  hd.ntrace = std::min<int64_t>(st.iter + 1, D.trace_cap);
  const size_t total = pad8(sizeof(hd)) + 8 * (2 * (size_t)n + (size_t)hd.ncoef) + 8 * 3 * (size_t)n * hd.rows +
                       pad8(4 * (size_t)hd.rows) + 16 * (size_t)hd.cnt + 16 * (size_t)hd.nout +
                       32 * (size_t)hd.ntrace;
  *bytes_out = (int64_t)total;
  if (!buf) return GPUGO_OK;
  if (cap < (int64_t)total) return GPUGO_ERR_INVALID;
  char* o = (char*)buf;
  memset(o, 0, total);
  memcpy(o, &hd, sizeof(hd));
  o += pad8(sizeof(hd));
  memcpy(o, h.dom.data(), 16 * (size_t)n); o += 16 * (size_t)n;
  memcpy(o, h.coef.data(), 8 * (size_t)hd.ncoef); o += 8 * (size_t)hd.ncoef;
  auto D2H = [&](const void* src, size_t bytes, size_t advance) -> int {
    if (bytes) {
      int rc = cuda_err(cudaMemcpy(o, src, bytes, cudaMemcpyDeviceToHost));
      if (rc) return rc;
      E->d2h += (int64_t)bytes;
    }
    o += advance;
    return GPUGO_OK;
  };
  int rc;
  if ((rc = D2H(D.parents, 16 * (size_t)n * hd.rows, 16 * (size_t)n * hd.rows))) return rc;
  if ((rc = D2H(D.pwid, 8 * (size_t)n * hd.rows, 8 * (size_t)n * hd.rows))) return rc;
  if ((rc = D2H(D.pcyc, 4 * (size_t)hd.rows, pad8(4 * (size_t)hd.rows)))) return rc;
  if ((rc = D2H(D.pool_lb[st.cur], 8 * (size_t)hd.cnt, 8 * (size_t)hd.cnt))) return rc;
  if ((rc = D2H(D.pool_key[st.cur], 8 * (size_t)hd.cnt, 8 * (size_t)hd.cnt))) return rc;
  if ((rc = D2H(D.out_key, 8 * (size_t)hd.nout, 8 * (size_t)hd.nout))) return rc;
  if ((rc = D2H(D.out_lb, 8 * (size_t)hd.nout, 8 * (size_t)hd.nout))) return rc;
  if ((rc = D2H(D.tr_ub, 8 * (size_t)hd.ntrace, 8 * (size_t)hd.ntrace))) return rc;
  if ((rc = D2H(D.tr_surv, 8 * (size_t)hd.ntrace, 8 * (size_t)hd.ntrace))) return rc;
  if ((rc = D2H(D.tr_pool, 8 * (size_t)hd.ntrace, 8 * (size_t)hd.ntrace))) return rc;
  if ((rc = D2H(D.tr_sel, 8 * (size_t)hd.ntrace, 8 * (size_t)hd.ntrace))) return rc;
  return GPUGO_OK;
}

int gpugo_checkpoint_check(const void* buf, int64_t bytes) {
  CkptHeader hd;
  gpugo_spec sp;
  const char* o;
  return parse_checkpoint(buf, bytes, &hd, &sp, &o);
}

int gpugo_restore(gpugo_engine* E, const void* buf, int64_t bytes, double* boxes_out, double* box_lb_out,
                  int64_t cap, double* xhat_out, gpugo_trace* trace, int64_t* ticket_out) {
  NvtxRange nvtx_range("gpugo_restore");
  if (!E) return GPUGO_ERR_INVALID;
  CkptHeader hd;
  gpugo_spec sp;
  const char* o;
  int rc = parse_checkpoint(buf, bytes, &hd, &sp, &o);
  if (rc) return rc;
  const int n = hd.n;
  Layout L;
  layout(&sp, cap, trace ? trace->cap : 0, &L);
  std::vector<Piece> pcs;
  auto take = [&](int64_t rel, size_t b, size_t advance) {
    if (b) pcs.push_back(Piece{(size_t)rel, o, b});
    o += advance;
  };
  take(L.o_par, 16 * (size_t)n * hd.rows, 16 * (size_t)n * hd.rows);
  take(L.o_pw, 8 * (size_t)n * hd.rows, 8 * (size_t)n * hd.rows);
  take(L.o_pcyc, 4 * (size_t)hd.rows, pad8(4 * (size_t)hd.rows));
  take(L.o_plb0, 8 * (size_t)hd.cnt, 8 * (size_t)hd.cnt);
  take(L.o_pk0, 8 * (size_t)hd.cnt, 8 * (size_t)hd.cnt);
  const int64_t nout = std::min<int64_t>(hd.nout, L.out_cap);
  take(L.o_outk, 8 * (size_t)nout, 8 * (size_t)hd.nout);
  take(L.o_outl, 8 * (size_t)nout, 8 * (size_t)hd.nout);
  const int64_t ntr = std::min<int64_t>(hd.ntrace, L.trace_cap);
  take(L.o_trub, 8 * (size_t)ntr, 8 * (size_t)hd.ntrace);
  take(L.o_trs, 8 * (size_t)ntr, 8 * (size_t)hd.ntrace);
  take(L.o_trp, 8 * (size_t)ntr, 8 * (size_t)hd.ntrace);
  take(L.o_trsel, 8 * (size_t)ntr, 8 * (size_t)hd.ntrace);
  State st = hd.st;
  st.cur = 0;               // the list was packed into buffer 0
  st.count = hd.cnt;
  st.count_new = 0;
  st.lb_max = ~0ULL;        // no bound taken from the buffer: the next UB move compacts
  return admit(E, &sp, boxes_out, box_lb_out, cap, xhat_out, trace, &st, pcs, ticket_out);
}

int gpugo_run(gpugo_engine* E, int64_t max_iters, int32_t* active_out) {
  NvtxRange nvtx_range("gpugo_run");
  if (!E) return GPUGO_ERR_INVALID;
  cudaStream_t st = E->stream;
  if (!E->pending_init.empty()) {
    // every admission since the last run: one copy, one kernel
    const int m = (int)E->stage_offs.size();
    const size_t rec_bytes = 8 * E->stage.size(), off_bytes = 8 * (size_t)m;
    const size_t need = ((off_bytes + 255) & ~size_t(255)) + rec_bytes;
    if (need > E->d_stage_cap) {
      const size_t cap = std::max<size_t>(need, 2 * E->d_stage_cap);
      CK(cudaStreamSynchronize(st));
      cudaFree(E->d_stage);
      E->d_stage = nullptr;
      E->d_stage_cap = 0;
      CK(cudaMalloc(&E->d_stage, cap));
      E->d_stage_cap = cap;
    }
    long long* d_offs = (long long*)E->d_stage;
    unsigned long long* d_rec = (unsigned long long*)(E->d_stage + ((off_bytes + 255) & ~size_t(255)));
    // pageable sources: the copies are staged by the runtime before the calls return
    CK(cudaMemcpyAsync(d_offs, E->stage_offs.data(), off_bytes, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_rec, E->stage.data(), rec_bytes, cudaMemcpyHostToDevice, st));
    admit_kernel<<<m, 128, 0, st>>>(E->d_desc, E->d_state, d_rec, d_offs);
    CK(cudaGetLastError());
    E->h2d += (int64_t)(rec_bytes + off_bytes);
    E->launches++;
    E->pending_init.clear();
    E->stage.clear();
    E->stage_offs.clear();
  }
  CK(cudaMemsetAsync(E->d_ctl, 0, sizeof(Ctl), st));
  KArgs a;
  a.desc = E->d_desc;
  a.st = E->d_state;
  a.ctl = E->d_ctl;
  a.idsA = E->d_ids;
  a.idsE = E->d_ids + E->max_slots;
  a.prefA = E->d_pref;
  a.prefB = E->d_pref + (E->max_slots + 1);
  a.prefD = E->d_pref + 2 * (E->max_slots + 1);
  a.prefC = E->d_pref + 3 * (E->max_slots + 1);
  a.cpass = (unsigned long long*)(E->d_pref + 4 * (E->max_slots + 1));
  a.queue = E->d_queue;
  a.cands = E->d_cands;
  a.cand_cap = E->cand_cap;
  a.chunk = E->chunk;
  a.cand_mode = E->cand_mode;
  a.max_slots = E->max_slots;
  a.max_iters = max_iters;
  a.fam_hi = FAM_PRODCOS;
  a.timeout_ns = (unsigned long long)(E->timeout_s * 1e9);
  a.stamps = E->d_stamps;
  a.stamp_cap = E->stamp_cap;
  a.bstamps = E->d_bstamps;
  a.bstamp_iters = E->bstamp_iters;
  a.cur_it = 0;
  void* args[] = {&a};
  bool any_cl = false;   // the build with the code-list interpreter only while one is resident
  for (int s = 0; s < E->max_slots && !any_cl; ++s) any_cl = E->slots[s].used && E->slots[s].spec.family == GPUGO_CODELIST;
  const void* kern = any_cl ? (const void*)solve_kernel<true> : (const void*)solve_kernel<false>;
  if (any_cl) a.fam_hi = FAM_CODELIST;
  CK(cudaEventRecord(E->ev0, st));
  CK(cudaLaunchCooperativeKernel(kern, dim3(E->blocks), dim3(E->threads), args, SMEM_TAB_BYTES, st));
  CK(cudaEventRecord(E->ev1, st));
  CK(cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, E->ev0, E->ev1);
  E->last_run_ms = ms;
  E->total_run_ms += ms;
  E->launches++;
  Ctl c;
  CK(cudaMemcpy(&c, E->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(E->h_state.data(), E->d_state, sizeof(State) * E->max_slots, cudaMemcpyDeviceToHost));
  E->iterations += c.iters;
  E->d2h += (int64_t)(sizeof(Ctl) + sizeof(State) * E->max_slots);
  if (E->d_stamps && c.iters > 0) {
    long long k = std::min<long long>(8 * c.iters, E->stamp_cap);
    std::vector<unsigned long long> ts(k);
    CK(cudaMemcpy(ts.data(), E->d_stamps, 8 * k, cudaMemcpyDeviceToHost));
    if (FILE* f = fopen(E->stamp_path, "a")) {
      fprintf(f, "run blocks=%d threads=%d iters=%lld\n", E->blocks, E->threads, (long long)c.iters);
      for (long long i = 0; i < k; ++i) fprintf(f, "%llu%c", ts[i], (i % 8 == 7) ? '\n' : ' ');
      fclose(f);
    }
    long long ki = std::min<long long>(c.iters, E->bstamp_iters);
    std::vector<unsigned long long> bs(BSTAMP_W * ki * E->blocks);
    CK(cudaMemcpy(bs.data(), E->d_bstamps, 8 * bs.size(), cudaMemcpyDeviceToHost));
    std::string bp = std::string(E->stamp_path) + ".blocks";
    if (FILE* f = fopen(bp.c_str(), "a")) {
      fprintf(f, "run blocks=%d iters=%lld width=%d\n", E->blocks, ki, BSTAMP_W);
      for (size_t i = 0; i < bs.size(); ++i) fprintf(f, "%llu%c", bs[i], (i % BSTAMP_W == BSTAMP_W - 1) ? '\n' : ' ');
      fclose(f);
    }
  }
  int active = 0;
  for (int s = 0; s < E->max_slots; ++s)
    if (E->slots[s].used && (E->h_state[s].status == ST_EXPAND || E->h_state[s].status == ST_REPOP)) active++;
  if (active_out) *active_out = active;
  if (c.error) return c.error;
  return GPUGO_OK;
}

int gpugo_poll(gpugo_engine* E, gpugo_done* done, int32_t max_done, int32_t* n_done_out) {
  NvtxRange nvtx_range("gpugo_poll");
  if (!E || max_done < 0 || (max_done > 0 && !done)) return GPUGO_ERR_INVALID;
  std::vector<int> fin;
  for (int s = 0; s < E->max_slots && (int)fin.size() < max_done; ++s)
    if (E->slots[s].used && E->h_state[s].status == ST_DONE) fin.push_back(s);
  // Small outputs (no trace, at most 64 boxes) come from finalize_kernel records,
  // all finished instances in one launch and one copy; the others are collected
  // from their lists and parent tables.
  std::vector<FinRec> recs;
  std::vector<int> rec_of(fin.size(), -1);
  long long total = 0;
  for (size_t f = 0; f < fin.size(); ++f) {
    const int s = fin[f];
    const HostSlot& h = E->slots[s];
    const State& st = E->h_state[s];
    if (h.has_trace || h.cap > 64) continue;
    const long long cnt = std::min<long long>(st.count, h.desc.pool_cap);
    const long long nout = std::min<long long>(st.out_count, h.desc.out_cap);
    const long long emitted = std::min<long long>(nout, h.cap);
    const long long pool_boxes = (h.spec.stop_mode == GPUGO_STOP_GAP) ? cnt : 0;
    const long long k = std::min<long long>(h.cap, nout + pool_boxes);
    FinRec r;
    r.slot = s; r.k = k; r.emitted = emitted; r.off = total;
    total += 2 + k + 2LL * h.spec.n * k + h.spec.n + 1;
    rec_of[f] = (int)recs.size();
    recs.push_back(r);
  }
  std::vector<double> out;
  if (!recs.empty()) {
    cudaStream_t st = E->stream;
    const size_t rb = (sizeof(FinRec) * recs.size() + 255) & ~size_t(255);
    const size_t need = rb + 8 * (size_t)total;
    if (need > E->d_fin_cap) {
      const size_t cap = std::max<size_t>(need, 2 * E->d_fin_cap);
      CK(cudaStreamSynchronize(st));
      cudaFree(E->d_fin);
      E->d_fin = nullptr;
      E->d_fin_cap = 0;
      CK(cudaMalloc(&E->d_fin, cap));
      E->d_fin_cap = cap;
    }
    FinRec* d_recs = (FinRec*)E->d_fin;
    double* d_out = (double*)(E->d_fin + rb);
    CK(cudaMemcpyAsync(d_recs, recs.data(), sizeof(FinRec) * recs.size(), cudaMemcpyHostToDevice, st));
    finalize_kernel<<<(unsigned)recs.size(), 256, 0, st>>>(E->d_desc, E->d_state, d_recs, d_out);
    CK(cudaGetLastError());
    out.resize((size_t)total);
    CK(cudaMemcpyAsync(out.data(), d_out, 8 * (size_t)total, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    E->launches++;
    E->h2d += (int64_t)(sizeof(FinRec) * recs.size());
    E->d2h += (int64_t)(8 * total);
  }
  int k = 0;
  for (size_t f = 0; f < fin.size(); ++f) {
    const int s = fin[f];
    HostSlot& h = E->slots[s];
    gpugo_result r;
    if (rec_of[f] < 0) {
      int rc = collect(E, s, &r);
      if (rc) return rc;
    } else {
      const FinRec& fr = recs[rec_of[f]];
      const State& st = E->h_state[s];
      const int n = h.spec.n;
      const double* o = out.data() + fr.off;
      memset(&r, 0, sizeof(r));
      r.lb = o[0];
      r.ub = ord_val_host(st.ub);
      r.boxes_bounded = st.bounded;
      r.samples_evaluated = st.samples;
      r.status = st.outcome;
      r.iterations = (st.outcome == GPUGO_ITER_LIMIT) ? st.iter : st.iter + 1;
      const long long cnt = std::min<long long>(st.count, h.desc.pool_cap);
      r.pool_size = cnt;
      r.n_boxes = st.out_count + ((h.spec.stop_mode == GPUGO_STOP_GAP) ? cnt : 0);
      r.n_out = (int32_t)fr.k;
      const double* lbs = o + 2;
      const double* boxes = lbs + fr.k;
      const double* xh = boxes + 2LL * n * fr.k;
      if (h.boxes_out && fr.k) memcpy(h.boxes_out, boxes, sizeof(double) * 2 * n * (size_t)fr.k);
      if (h.box_lb_out && fr.k) memcpy(h.box_lb_out, lbs, sizeof(double) * (size_t)fr.k);
      r.has_xhat = 0;
      if (xh[n] != 0.0 && h.xhat_out) {
        memcpy(h.xhat_out, xh, sizeof(double) * n);
        r.has_xhat = 1;
      }
      r.d2h_bytes = (int64_t)(8 * (2 + fr.k + 2LL * n * fr.k + n + 1));
    }
    done[k].ticket = h.ticket;
    done[k].result = r;
    k++;
    E->arena.release(h.arena_off, h.arena_bytes);
    // the device state keeps ST_DONE (out of every work list) until the slot's
    // next admission overwrites it
    State z;
    memset(&z, 0, sizeof(z));
    E->h_state[s] = z;
    h = HostSlot();
    if (s < E->free_from) E->free_from = s;
  }
  if (n_done_out) *n_done_out = k;
  return GPUGO_OK;
}

// ---------------------------------------------------------------------------
// no-allocation variant of gpugo_eval_children
// ---------------------------------------------------------------------------
}  // extern "C"

// The only working memory of gpugo_eval_children_static.  In host code this name
// is a stand-in, not a device address: each call looks the address up.
static __device__ __align__(256) unsigned char g_static_scratch[GPUGO_STATIC_SCRATCH_BYTES];

namespace {
std::mutex g_static_mu;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Checks both eval_children entry points make on the host, before any device
// call: the problem, the pointers, the cycle, the code count, and every child
// code against the children of the cycle (compared unsigned: a code is an index
// in [0, wid^g); a packed code of a larger value would yield digits >= wid).
int check_eval_args(const gpugo_spec* spec, const double* parent_box, int32_t cyc, const uint64_t* codes, int64_t m,
                    const double* lb_out, const double* samp_out, const int32_t* flag_out) {
  int rc = validate(spec);
  if (rc) return rc;
  if (!parent_box || m < 0 || m > (1LL << 40) || (m > 0 && (!codes || !lb_out || !samp_out || !flag_out)) ||
      cyc < 1 || cyc > spec->n)
    return GPUGO_ERR_INVALID;
  const uint64_t M = (uint64_t)children_host(spec, cyc);
  for (int64_t t = 0; t < m; ++t)
    if (codes[t] >= M) return GPUGO_ERR_INVALID;
  return GPUGO_OK;
}

// Byte offsets of gpugo_eval_children_static's scratch:
// descriptor | instance region | codes | lb | samp | flag
struct StaticLayout {
  Layout L;
  size_t o_desc, o_inst, o_codes, o_lb, o_samp, o_flag, total;
};

void static_layout(const gpugo_spec* spec, int64_t m, StaticLayout* S) {
  gpugo_spec s2 = *spec;
  s2.pool_cap = 1;
  s2.parent_cap = 1;
  layout(&s2, 1, 0, &S->L);
  S->o_desc = 0;
  S->o_inst = align256(sizeof(Desc));
  S->o_codes = S->o_inst + align256((size_t)S->L.bytes);
  S->o_lb = S->o_codes + align256(8 * (size_t)m);
  S->o_samp = S->o_lb + align256(8 * (size_t)m);
  S->o_flag = S->o_samp + align256(8 * (size_t)m);
  S->total = S->o_flag + align256(4 * (size_t)m);
}
}  // namespace

extern "C" {

int gpugo_eval_children_static(const gpugo_spec* spec, const double* parent_box, int32_t cyc, const uint64_t* codes,
                               int64_t m, double ub, double* lb_out, double* samp_out, int32_t* flag_out) {
  // every check is made on the host before the device is touched; an oversize
  // request is refused before its codes are scanned
  int rc = validate(spec);
  if (rc) return rc;
  if (m < 0 || m > (1LL << 40)) return GPUGO_ERR_INVALID;
  StaticLayout S;
  static_layout(spec, m, &S);
  if (S.total > GPUGO_STATIC_SCRATCH_BYTES) return GPUGO_ERR_SCRATCH_LIMIT;
  if ((rc = check_eval_args(spec, parent_box, cyc, codes, m, lb_out, samp_out, flag_out))) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPUGO_ERR_NO_DEVICE;

  std::lock_guard<std::mutex> lock(g_static_mu);
  // the array's device address in the context current now (looked up on every
  // call: a cudaDeviceReset or another context since the last call moves it)
  void* sp = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&sp, g_static_scratch);
  if (e != cudaSuccess || !sp) return cuda_err(e != cudaSuccess ? e : cudaErrorInvalidSymbol);
  char* base = (char*)sp;
  Desc* d_desc = (Desc*)(base + S.o_desc);
  unsigned long long* d_codes = (unsigned long long*)(base + S.o_codes);
  double* d_lb = (double*)(base + S.o_lb);
  double* d_samp = (double*)(base + S.o_samp);
  int* d_flag = (int*)(base + S.o_flag);
  gpugo_spec s2 = *spec;
  s2.pool_cap = 1;
  s2.parent_cap = 1;
  Desc D;
  fill_desc(&s2, S.L, base + S.o_inst, &D);
  CK(cudaMemcpy((void*)D.dom, spec->domain, 8 * 2 * spec->n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy((void*)D.coef, spec->coef, 8 * spec->ncoef, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(D.parents, parent_box, 8 * 2 * spec->n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_desc, &D, sizeof(Desc), cudaMemcpyHostToDevice));
  if (m > 0) CK(cudaMemcpy(d_codes, codes, 8 * m, cudaMemcpyHostToDevice));
  eval_init_kernel<<<1, 32>>>(d_desc);
  CK(cudaGetLastError());
  const int blocks = (int)std::min<int64_t>((S.L.a_items + 255) / 256, 4096);
  eval_tables_kernel<<<std::max(blocks, 1), 256>>>(d_desc, cyc);
  CK(cudaGetLastError());
  if (m > 0) {
    const int b2 = (int)std::min<int64_t>((m + 255) / 256, 4096);
    eval_children_kernel<<<b2, 256>>>(d_desc, cyc, d_codes, m, ub, d_lb, d_samp, d_flag);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(0));
  if (m > 0) {
    CK(cudaMemcpy(lb_out, d_lb, 8 * m, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(samp_out, d_samp, 8 * m, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(flag_out, d_flag, 4 * m, cudaMemcpyDeviceToHost));
  }
  return GPUGO_OK;
}

// ---------------------------------------------------------------------------
// single solve: a cached one-slot engine
// ---------------------------------------------------------------------------
static std::mutex g_mu;
static gpugo_engine* g_single = nullptr;
static int64_t g_single_bytes = 0;

int gpugo_solve(const gpugo_spec* spec, gpugo_result* res, double* boxes_out, double* box_lb_out, int64_t cap,
                double* xhat_out, gpugo_trace* trace) {
  NvtxRange nvtx_range("gpugo_solve");
  if (!res) return GPUGO_ERR_INVALID;
  int rc = validate(spec);
  if (rc) return rc;
  if (cap > (1LL << 40) || (trace && trace->cap > (1LL << 40))) return GPUGO_ERR_INVALID;
  if (trace && trace->cap > 0 && (!trace->ub || !trace->n_surv || !trace->pool || !trace->sel))
    return GPUGO_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_mu);
  Layout L;
  layout(spec, cap, trace ? trace->cap : 0, &L);
  if (!g_single || g_single_bytes < L.bytes) {
    if (g_single) { gpugo_engine_destroy(g_single); g_single = nullptr; }
    gpugo_engine_cfg cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.max_slots = 1;
    cfg.threads = 256;
    cfg.arena_bytes = std::max<int64_t>(L.bytes, 64LL << 20);
    cfg.wait_timeout_s = 60.0;
    if ((rc = gpugo_engine_create(&cfg, &g_single))) return rc;
    g_single_bytes = cfg.arena_bytes;
  }
  int64_t ticket;
  const int64_t h2d0 = g_single->h2d, d2h0 = g_single->d2h;
  if ((rc = gpugo_submit(g_single, spec, boxes_out, box_lb_out, cap, xhat_out, trace, &ticket))) return rc;
  int32_t active = 1;
  double total_ms = 0.0;
  while (active > 0) {
    rc = gpugo_run(g_single, 0, &active);
    total_ms += g_single->last_run_ms;
    if (rc) {
      // drop the slot so the engine stays usable
      gpugo_done d;
      int32_t nd = 0;
      g_single->h_state[0].status = ST_DONE;
      if (g_single->h_state[0].outcome == 0) g_single->h_state[0].outcome = rc;
      gpugo_poll(g_single, &d, 1, &nd);
      if (nd) *res = d.result;
      res->status = rc;
      return rc;
    }
  }
  gpugo_done d;
  int32_t nd = 0;
  if ((rc = gpugo_poll(g_single, &d, 1, &nd))) return rc;
  if (nd != 1) return GPUGO_ERR_CUDA;
  *res = d.result;
  res->device_ms = total_ms;
  res->h2d_bytes = g_single->h2d - h2d0;
  res->d2h_bytes = g_single->d2h - d2h0;
  return res->status < 0 ? res->status : GPUGO_OK;
}

int gpugo_eval_children(const gpugo_spec* spec, const double* parent_box, int32_t cyc, const uint64_t* codes,
                        int64_t m, double ub, double* lb_out, double* samp_out, int32_t* flag_out) {
  NvtxRange nvtx_range("gpugo_eval_children");
  int rc = check_eval_args(spec, parent_box, cyc, codes, m, lb_out, samp_out, flag_out);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPUGO_ERR_NO_DEVICE;
  gpugo_spec s2 = *spec;
  s2.pool_cap = 1;
  s2.parent_cap = 1;
  Layout L;
  layout(&s2, 1, 0, &L);
  char* base = nullptr;
  Desc* d_desc = nullptr;
  unsigned long long* d_codes = nullptr;
  double *d_lb = nullptr, *d_samp = nullptr;
  int* d_flag = nullptr;
  rc = GPUGO_OK;
  do {
    if ((rc = cuda_err(cudaMalloc(&base, (size_t)L.bytes)))) break;
    if ((rc = cuda_err(cudaMalloc(&d_desc, sizeof(Desc))))) break;
    size_t mm = (size_t)std::max<int64_t>(m, 1);
    if ((rc = cuda_err(cudaMalloc(&d_codes, 8 * mm)))) break;
    if ((rc = cuda_err(cudaMalloc(&d_lb, 8 * mm)))) break;
    if ((rc = cuda_err(cudaMalloc(&d_samp, 8 * mm)))) break;
    if ((rc = cuda_err(cudaMalloc(&d_flag, 4 * mm)))) break;
    Desc D;
    fill_desc(&s2, L, base, &D);
    if ((rc = cuda_err(cudaMemcpy((void*)D.dom, spec->domain, 8 * 2 * spec->n, cudaMemcpyHostToDevice)))) break;
    if ((rc = cuda_err(cudaMemcpy((void*)D.coef, spec->coef, 8 * spec->ncoef, cudaMemcpyHostToDevice)))) break;
    if ((rc = cuda_err(cudaMemcpy(D.parents, parent_box, 8 * 2 * spec->n, cudaMemcpyHostToDevice)))) break;
    if ((rc = cuda_err(cudaMemcpy(d_desc, &D, sizeof(Desc), cudaMemcpyHostToDevice)))) break;
    if (m > 0 && (rc = cuda_err(cudaMemcpy(d_codes, codes, 8 * m, cudaMemcpyHostToDevice)))) break;
    eval_init_kernel<<<1, 32>>>(d_desc);
    if ((rc = cuda_err(cudaGetLastError()))) break;
    int blocks = (int)std::min<int64_t>((L.a_items + 255) / 256, 4096);
    eval_tables_kernel<<<std::max(blocks, 1), 256>>>(d_desc, cyc);
    if ((rc = cuda_err(cudaGetLastError()))) break;
    if (m > 0) {
      int b2 = (int)std::min<int64_t>((m + 255) / 256, 4096);
      eval_children_kernel<<<b2, 256>>>(d_desc, cyc, d_codes, m, ub, d_lb, d_samp, d_flag);
      if ((rc = cuda_err(cudaGetLastError()))) break;
    }
    if ((rc = cuda_err(cudaDeviceSynchronize()))) break;
    if (m > 0) {
      if ((rc = cuda_err(cudaMemcpy(lb_out, d_lb, 8 * m, cudaMemcpyDeviceToHost)))) break;
      if ((rc = cuda_err(cudaMemcpy(samp_out, d_samp, 8 * m, cudaMemcpyDeviceToHost)))) break;
      if ((rc = cuda_err(cudaMemcpy(flag_out, d_flag, 4 * m, cudaMemcpyDeviceToHost)))) break;
    }
  } while (0);
  cudaFree(base); cudaFree(d_desc); cudaFree(d_codes); cudaFree(d_lb); cudaFree(d_samp); cudaFree(d_flag);
  return rc;
}

}  // extern "C"
