/*
 * gpugo.h -- C ABI of the GB300 interval branch-and-bound solver (libgpugo.so).
 *
 * The reference (CMU GPUGO, Python + Numba CUDA) has no function-call API: each
 * script is the per-problem call.  Its constants go in (objective code lists,
 * domain, split rule, sample count, width tolerance, initial UB) and the
 * enclosure plus the surviving boxes are printed.  Citations below name the
 * reference lines each entry point replaces (paths within the GPUGO project).
 *
 * Conventions
 *   - Every function returns GPUGO_OK (0) or a negative GPUGO_ERR_* code.
 *   - All pointers in these signatures are HOST pointers.  Device memory is
 *     owned by the library (one arena per engine, allocated at creation).
 *   - An engine is single-producer: one host thread submits, runs and polls.
 *   - Device-side waits are bounded; an expired wait returns GPUGO_ERR_TIMEOUT
 *     and leaves the CUDA context usable.
 */
#ifndef GPUGO_H
#define GPUGO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status / error codes */
#define GPUGO_OK                   0
#define GPUGO_ERR_INVALID         -1   /* bad spec or argument */
#define GPUGO_ERR_CUDA            -2   /* CUDA runtime error */
#define GPUGO_ERR_NOMEM           -3   /* arena or host allocation failed */
#define GPUGO_ERR_POOL_OVERFLOW   -4   /* box pool capacity exceeded */
#define GPUGO_ERR_PARENT_OVERFLOW -5   /* parent table capacity exceeded */
#define GPUGO_ERR_TIMEOUT         -6   /* a bounded device wait expired */
#define GPUGO_ERR_BUSY            -7   /* no free slot or pool memory: retry after a run */
#define GPUGO_ERR_NOT_FOUND       -8   /* unknown ticket */
#define GPUGO_ERR_NO_DEVICE       -9   /* no CUDA device */
#define GPUGO_ERR_SCRATCH_LIMIT  -10   /* request larger than the fixed scratch of gpugo_eval_children_static */

/* per-instance outcome (gpugo_result.status) */
#define GPUGO_CERTIFIED   1   /* UB - LB <= gap_tol (gap mode) */
#define GPUGO_FINISHED    2   /* list exhausted (width mode: every remaining box met the width rule) */
#define GPUGO_ITER_LIMIT  3   /* max_iter expansions reached */

/* objective families (coefficient layout in gpugo_spec.coef) */
#define GPUGO_COSQUAD 1   /* sum a_i x_i^2 - b_i cos(K_i x_i) + sum b_i,  K_i = fl(fl(2pi) c_i); coef a[n] b[n] c[n]  (rastrigin50.py:161-188) */
#define GPUGO_CHAINED 2   /* sum_{i<n} p_i (x_{i+1} - x_i^2)^2 + q_i (1 - x_i)^2; coef p[n-1] q[n-1]       (rosenbrock50.py:168-198) */
#define GPUGO_EXPSQRT 3   /* -A exp(-B sqrt(mean x^2)) - exp(mean cos(K_i x_i)) + A + e; coef A B w[n]     (ackley50.py:166-212) */
#define GPUGO_PRODCOS 4   /* 1 + sum x_i^2 / d - prod cos(x_i / sqrt(i)); coef d                          (griewank50.py:161-198) */
/* Any objective as a compiled code list (value, sample and derivative code lists
 * as in levy50.py:103-563): coef is the array gpugo_gb300/codelist.py writes.
 * Word k of its header and code is the low 32 bits of coef[k]:
 *   [0] 0x314C4347 [1] n [2] registers (<= 16) [3] instructions [4] constants
 *   [5] value start [6] value length [7] gradient prologue start [8] length
 *   [9] sections [10] skip constant (0xFFFFFFFF none) [11] value result register
 *   [12] term tables (<= 8) [13..15] 0
 *   [16 + 12s] section: lo, hi, start, length, gradient register, check offset,
 *              skip register, tabled, offsets, offset 0..2
 *   [U + 12t]  term table: lo, hi, kind, offsets, offset 0, offset 1, 0, body start,
 *              body length, body result register, 0, 0            (U = 16 + 12 sections)
 *   [I + 4t]   instruction: op | dst << 8 | a << 16 | b << 24, imm1, imm2, 0
 *                                                                  (I = U + 12 tables)
 *   [I + 4 instructions ...] constants (doubles)
 * The library checks every index an instruction can form against n, the
 * constants and the registers, and that registers are written before they are
 * read, before it accepts the problem (GPUGO_ERR_INVALID). */
#define GPUGO_CODELIST 5

#define GPUGO_STOP_WIDTH 0   /* reference rule: emit a box when width(x_1) < width_tol at the last cycle (ackley50.py:1306-1343) */
#define GPUGO_STOP_GAP   1   /* certify when UB - LB <= gap_tol */

/* One problem: the constants of a reference script made explicit. */
typedef struct gpugo_spec {
    int32_t family;        /* GPUGO_COSQUAD .. GPUGO_CODELIST */
    int32_t n;             /* variables, 1..16384 (reference: 50..10000, hard-coded per script) */
    int32_t wid;           /* parts per split coordinate (reference wid = 4, ackley50.py:527) */
    int32_t group;         /* coordinates split per iteration (reference cycleSize = 10, :530) */
    int32_t samples;       /* sample points per child (reference numSamples = 10, :1015) */
    int32_t stop_mode;     /* GPUGO_STOP_WIDTH or GPUGO_STOP_GAP */
    double  width_tol;     /* reference widthTolerance = 1e-4 (:1010) */
    double  gap_tol;       /* UB - LB tolerance in gap mode */
    double  ub_init;       /* initial UB (reference lowestUpperVal, :994); +inf allowed */
    const double* domain;  /* [2n] lo_1, hi_1, ..., lo_n, hi_n (reference initialRegion, :958) */
    const double* coef;    /* family coefficients, see above */
    int64_t ncoef;
    int64_t max_iter;      /* 0: unlimited expansions */
    int64_t pool_cap;      /* 0: default list capacity (entries) */
    int64_t parent_cap;    /* 0: default parent-table rows */
} gpugo_spec;

typedef struct gpugo_result {
    double  lb;                 /* guaranteed lower bound of the global minimum */
    double  ub;                 /* guaranteed upper bound (smallest sampled upper bound) */
    int64_t n_boxes;            /* minimiser boxes available (may exceed the caller's cap) */
    int64_t iterations;         /* expansions (the reference's `iter`) */
    int64_t boxes_bounded;      /* child boxes bounded */
    int64_t pool_size;          /* live list entries at exit */
    int32_t status;             /* GPUGO_CERTIFIED / FINISHED / ITER_LIMIT, or a GPUGO_ERR_* code */
    int32_t n_out;              /* boxes written to the caller's buffers */
    int64_t samples_evaluated;  /* children whose sample points were evaluated */
    int32_t has_xhat;           /* 1 when xhat_out holds the point that achieved ub */
    int32_t reserved;
    double  device_ms;          /* device time of the solve (persistent-kernel launches) */
    int64_t h2d_bytes;          /* host -> device bytes copied for this solve */
    int64_t d2h_bytes;          /* device -> host bytes copied for this solve */
} gpugo_result;

/* Trace of one solve, one row per expansion (optional). */
typedef struct gpugo_trace {
    int64_t  cap;        /* rows available */
    double*  ub;         /* UB after the sampling step */
    int64_t* n_surv;     /* survivors appended (the reference's atomic_index) */
    int64_t* pool;       /* live list length after the update */
    int64_t* sel;        /* (parent << 32 | child code) selected as next parent, -1 at exit */
} gpugo_trace;

/*
 * Solve one problem to completion on the current CUDA device.
 * Replaces one run of a reference script: the host loop ackley50.py:950-1396 with
 * its kernels sampling (:602-684), ruleOutGPU (:686-766), constructFlagArr (:768-810)
 * and the selection step (:1269-1370); the printed enclosure (:1384-1387) is
 * res->lb / res->ub and the printed output regions are boxes_out.
 *   boxes_out  [cap][2n] minimiser boxes (width mode: emitted boxes in emission
 *              order; gap mode: emitted boxes, then the remaining list by LB)
 *   box_lb_out [cap] their lower bounds (may be NULL)
 *   xhat_out   [n] the sample point that achieved res->ub (may be NULL)
 *   trace      per-expansion record (may be NULL)
 */
int gpugo_solve(const gpugo_spec* spec, gpugo_result* res, double* boxes_out, double* box_lb_out,
                int64_t cap, double* xhat_out, gpugo_trace* trace);

/*
 * One bound/prune pass over given children of one parent box: for each child
 * code, the lower bound (value code list, e.g. rastrigin50.py:111-196), the
 * smallest sampled upper bound (sample code list, :199-299) and the ruleOutGPU
 * flag (value test against `ub`, then the derivative code list, :302-372).
 * Replaces one launch of sampling + ruleOutGPU (ackley50.py:602-766) restricted
 * to the listed threads.  cyc is the 1-based first split coordinate.
 */
int gpugo_eval_children(const gpugo_spec* spec, const double* parent_box, int32_t cyc,
                        const uint64_t* codes, int64_t m, double ub,
                        double* lb_out, double* samp_out, int32_t* flag_out);

/*
 * gpugo_eval_children_static: the same pass as gpugo_eval_children, for callers
 * that must not allocate device memory.  No counterpart in the reference.
 *
 * Some hosts own all of the GPU's memory themselves: an application that reserves
 * the device heap at start-up and hands out pieces of it, a plugin running inside
 * such a process, or a real-time loop that cannot afford cudaMalloc/cudaFree
 * (both may synchronise the whole device and may fail late under memory
 * pressure).  This entry point calls no allocator: its working memory (problem
 * descriptor, derived constants, term tables, child codes and result staging) is
 * one fixed array of GPUGO_STATIC_SCRATCH_BYTES in the library's own device
 * memory, loaded with the library on every GPU that uses it and kept until the
 * process exits.  Inputs and outputs are host buffers, as for gpugo_eval_children.
 *
 * Limit: a request whose term tables plus 28 bytes per child code exceed the
 * scratch returns GPUGO_ERR_SCRATCH_LIMIT, checked on the host before anything
 * else is done (the 8-variable chained instance with wid = 4 fits 296 672 child
 * codes per call).  Every call looks up the array's device address
 * (cudaGetSymbolAddress) in the context current at the call, so the address
 * stays right after a cudaDeviceReset or under another context.  The first call
 * on a device also loads the library's device code there; make it before any
 * stream capture.  The array is shared by every call through one loaded copy
 * of the library on that device and keeps the last call's contents; nothing in
 * it has to start at zero because every value a call reads is written earlier
 * in the same call.  Calls that overlapped on the GPU would race on the array:
 * the library prevents that with a lock that each call holds until its results
 * are back in the caller's host buffers.
 */
#define GPUGO_STATIC_SCRATCH_BYTES (8u << 20)
int gpugo_eval_children_static(const gpugo_spec* spec, const double* parent_box, int32_t cyc,
                               const uint64_t* codes, int64_t m, double ub,
                               double* lb_out, double* samp_out, int32_t* flag_out);

/* ---------------------------------------------------------------------------
 * Engines: many solves share one persistent kernel (batching and serving).  The
 * reference runs one solve per script (GPUGO_1.1/1-Ackley/ackley50.py:950-1396);
 * these calls have no counterpart there: each admitted problem is that script's
 * solve, with the same inputs (gpugo_spec) and results (gpugo_result).
 * ------------------------------------------------------------------------- */
typedef struct gpugo_engine gpugo_engine;

typedef struct gpugo_engine_cfg {
    int32_t max_slots;          /* instances resident at once (<= 8192) */
    int32_t threads;            /* threads per block (0: 256) */
    int64_t arena_bytes;        /* device memory for pools, tables and parent tables */
    double  wait_timeout_s;     /* bound of every device-side wait (0: 60 s) */
    int32_t blocks_per_sm;      /* 0: occupancy maximum (one per SM for engines of at most 4 slots) */
    int32_t cand_mode;          /* candidate scheduling, GPUGO_CAND_* (results are the same in every mode) */
    int64_t chunk_children;     /* children bounded per pass (0: the candidate queue's capacity, 2^20 to 2^24).
                                   An iteration with more children (up to 2^32 for one instance, against the
                                   reference's 4^10, ackley50.py:1053-1054) streams them through the queue in
                                   passes of this size; results do not depend on it */
} gpugo_engine_cfg;

/* Candidate children (LB not above the UB) are sampled and KKT-tested either by
   a group of lanes each (S lanes for S <= 16 sample points, else a whole warp:
   sample points and coordinates across the lanes; short queues, GPUGO_CAND_WARP)
   or by one lane each (long queues, GPUGO_CAND_LANE).  AUTO picks by queue
   length. */
#define GPUGO_CAND_AUTO 0
#define GPUGO_CAND_WARP 1
#define GPUGO_CAND_LANE 2

typedef struct gpugo_done {
    int64_t ticket;
    gpugo_result result;
} gpugo_done;

int gpugo_engine_create(const gpugo_engine_cfg* cfg, gpugo_engine** out);
int gpugo_engine_destroy(gpugo_engine* eng);

/* Admit one problem if a slot and pool memory are free (GPUGO_ERR_BUSY otherwise).
 * Output buffers are host memory owned by the caller and filled by gpugo_poll. */
int gpugo_submit(gpugo_engine* eng, const gpugo_spec* spec, double* boxes_out, double* box_lb_out,
                 int64_t cap, double* xhat_out, gpugo_trace* trace, int64_t* ticket_out);

/* Admit specs[0..count) in order, as that many gpugo_submit calls without a
 * trace would, in one call (a batch of a thousand problems crosses the boundary
 * once).  The output buffers are packed: with N_i = n_0 + ... + n_{i-1},
 * problem i's boxes start at boxes_out + 2 * cap * N_i, its box LBs at
 * box_lb_out + cap * i and its sample point at xhat_out + N_i (buffers of
 * 2 * cap * N_count, cap * count and N_count doubles).  Stops at the first
 * problem that is not admitted: *admitted_out = the number admitted, their
 * tickets in tickets_out[0 .. *admitted_out).  Returns GPUGO_OK when all were
 * admitted, GPUGO_ERR_BUSY when problem *admitted_out found no free slot or
 * memory, and that problem's error when its spec is invalid; the problems
 * before it stay admitted in every case. */
int gpugo_submit_batch(gpugo_engine* eng, const gpugo_spec* specs, int64_t count, double* boxes_out,
                       double* box_lb_out, int64_t cap, double* xhat_out, int64_t* tickets_out,
                       int64_t* admitted_out);

/* Run the persistent kernel for at most max_iters iterations (0: until every
 * admitted instance has finished).  Returns the number of instances still active
 * through *active_out. */
int gpugo_run(gpugo_engine* eng, int64_t max_iters, int32_t* active_out);

/* Collect finished instances (results and boxes), freeing their slots. */
int gpugo_poll(gpugo_engine* eng, gpugo_done* done, int32_t max_done, int32_t* n_done_out);

/* Counters of an engine since its creation. */
typedef struct gpugo_stats {
    double  last_run_ms;        /* device time of the last gpugo_run (CUDA events on the engine stream) */
    double  total_run_ms;
    int64_t kernel_launches;    /* kernels this engine launched */
    int64_t iterations;         /* persistent-kernel iterations run */
    int64_t h2d_bytes, d2h_bytes;
} gpugo_stats;

int gpugo_engine_stats(gpugo_engine* eng, gpugo_stats* out);

/* Checkpoint / resume of one resident solve (between runs), for long solves that
   must survive a process or a device: the reference has no counterpart (its
   list lives in host NumPy arrays for the length of one script run,
   ackley50.py:1269-1370).  gpugo_checkpoint serialises the instance's problem,
   state, parent table, list, emitted boxes and trace into buf (pass buf = NULL
   to get the size in *bytes_out; GPUGO_ERR_BUSY if the instance has not run
   yet).  gpugo_restore admits a serialised instance into an engine (any engine
   on any device); it continues exactly where the checkpoint was taken: the
   restored solve's remaining iterations and result are bit-identical to the
   uninterrupted solve's. */
int gpugo_checkpoint(gpugo_engine* eng, int64_t ticket, void* buf, int64_t cap, int64_t* bytes_out);
int gpugo_restore(gpugo_engine* eng, const void* buf, int64_t bytes, double* boxes_out, double* box_lb_out,
                  int64_t cap, double* xhat_out, gpugo_trace* trace, int64_t* ticket_out);

/* The checks gpugo_restore makes before it admits anything, on the host and
   without a device: the problem, the state (status, cycle, iteration and row
   count, counters) and every parent row and child code the lists hold.
   GPUGO_OK or GPUGO_ERR_INVALID.  For checkpoints kept in files or sent
   between processes; no counterpart in the reference. */
int gpugo_checkpoint_check(const void* buf, int64_t bytes);

/* Free bytes of the engine's arena (admission control). */
int gpugo_engine_free_bytes(gpugo_engine* eng, int64_t* free_out);

/* Arena bytes one problem needs when admitted. */
int gpugo_instance_bytes(const gpugo_spec* spec, int64_t* bytes_out);

const char* gpugo_strerror(int code);

/* Library version and the device it runs on (sm number, e.g. 103). */
int gpugo_device_info(int32_t* sm_out, int32_t* num_sms_out);

/* FP64 throughput probe: independent DFMA chains on every SM, timed with CUDA
 * events (best of `repeats`); FMA counts 2 flops.  No reference counterpart: the
 * roofline denominator for the FP64-bound bound kernels. */
int gpugo_fp64_peak(int32_t repeats, double* tflops_out, double* ms_out);

/* Result-box merging: replaces the reference's host functions combine /
   connectivity (GPUGO_1.1/11-Rosenbrock/rosenbrock50.py:926-1049, called at
   :1439 on every emitted output region with combineTolerance = 1e-3, :1115).
   boxes: nbox boxes of n coordinates, lo/hi interleaved, in emission order.
   A box joins the first earlier root it is connected to (in every coordinate it
   lies inside the root, or |lo - root.hi| < tol and its own width < tol) and the
   root becomes the hull; otherwise it becomes a new root.  Runs on the device
   (one block tests the roots of each box in parallel).  *nroots_out receives the
   number of roots; roots_out the first cap of them. */
int gpugo_combine(const double* boxes, int64_t nbox, int32_t n, double tol, double* roots_out, int64_t cap,
                  int64_t* nroots_out);

#ifdef __cplusplus
}
#endif
#endif /* GPUGO_H */
