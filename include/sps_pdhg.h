/*
 * sps_pdhg.h — C ABI of the GB300 restarted-PDHG LP engine (libsps_gb300.so).
 *
 * The reference has no native boundary: its hot path is the Python call
 *   solve_lp_pdhg(problem, max_iters, tol)          solver/lp/pdhg.py:152-156
 *   solve_lp_pdhg_gpu(problem, device, max_iters, tol)  solver/lp/pdhg_gpu.py:315-320
 * reached from Solver.solve(method='pdhg' | 'pdhg_gpu')   solver/solver.py:113-119.
 * These entry points are what a binding for that call binds (ctypes in
 * sovereign-solver_gb300/_native.py).  The problem descriptor carries the
 * reference Problem fields (solver/problem.py:57-64) as plain arrays.
 *
 * Conventions
 *  - Every function returns 0 (SPS_OK) or a negative SPS_ERR_* code and never
 *    aborts or traps; sps_last_error() gives the message.
 *  - Host arrays are read during the call only (copied to the device).
 *  - One handle per thread; calls on one handle are serialised by the caller.
 *  - No CPU fallback: without a usable sm_103a device sps_create fails with
 *    SPS_ERR_CUDA.
 */
#ifndef SPS_PDHG_H
#define SPS_PDHG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* return codes */
#define SPS_OK               0
#define SPS_ERR_INVALID     -1   /* malformed input (shapes, indices, NaN, lb > ub) */
#define SPS_ERR_CUDA        -2   /* CUDA runtime error or no usable device */
#define SPS_ERR_OOM         -3   /* device allocation failed */
#define SPS_ERR_STATE       -4   /* call out of order (e.g. get_solution before solve) */
#define SPS_ERR_TIMEOUT     -5   /* host watchdog expired and the device did not stop */

/* solve status (sps_result.status) — solver/lp/simplex_dense.py:49 names */
#define SPS_STATUS_OPTIMAL          0   /* relative KKT error < tol */
#define SPS_STATUS_ITERATION_LIMIT  1
#define SPS_STATUS_TIME_LIMIT       2
#define SPS_STATUS_NUMERIC_ERROR    3   /* NaN/Inf appeared in the iterates */
#define SPS_STATUS_STALLED          4   /* FP32 iterates stopped making progress (returned
                                           only with sps_options.escalate = 2) */
#define SPS_STATUS_INFEASIBLE       5   /* adaptive mode: the change of y since the last restart is
                                           a Farkas certificate (primal infeasible) */
#define SPS_STATUS_UNBOUNDED        6   /* adaptive mode: the change of x since the last restart is
                                           an improving ray (dual infeasible) */

/* algorithm */
#define SPS_MODE_REFERENCE  0  /* the reference's rules: standard form with bound rows and
                                  slacks, fixed diagonal steps, theta = 1, ergodic average,
                                  KKT of the average every 50 iterations, restart on halving
                                  (solver/lp/pdhg.py:62-259) */
#define SPS_MODE_ADAPTIVE   1  /* box form, Ruiz + Pock-Chambolle scaling, adaptive steps,
                                  primal weight, KKT-based restarts to average or current */

#define SPS_FP32  0  /* FP32 iterates and SpMV, FP64 checks */
#define SPS_FP64  1  /* FP64 everywhere */

/* relative KKT error measure of the adaptive single-LP engine (sps_options.kkt_form) */
#define SPS_KKT_LAGRANGIAN  0  /* dual objective = Lagrangian bound b^T y + sum_j min over
                                  [lb_j, ub_j] of r_j x_j, r = c - K^T y: every finite bound
                                  enters the gap (default) */
#define SPS_KKT_PDLP        1  /* a finite bound farther from x_j than |x_j| does not enter the
                                  dual objective; the part of r_j it would absorb counts as dual
                                  residual instead (PDLP's default handling, OR-tools
                                  handle_some_primal_gradients_on_finite_bounds_as_residuals) */

typedef struct {
    int32_t n;                      /* variables */
    int32_t m_ub;                   /* rows of A_ub x <= b_ub */
    int32_t m_eq;                   /* rows of A_eq x == b_eq */
    const int32_t *ub_indptr;       /* CSR of A_ub: m_ub+1 offsets */
    const int32_t *ub_indices;      /*   column of each nonzero */
    const double  *ub_values;       /*   value of each nonzero */
    const int32_t *eq_indptr;       /* CSR of A_eq */
    const int32_t *eq_indices;
    const double  *eq_values;
    const double  *c;               /* n, objective of the minimisation */
    const double  *b_ub;            /* m_ub */
    const double  *b_eq;            /* m_eq */
    const double  *lb;              /* n, -INFINITY allowed */
    const double  *ub;              /* n, +INFINITY allowed */
} sps_problem_desc;

typedef struct {
    int32_t mode;             /* SPS_MODE_* (default ADAPTIVE) */
    int32_t precision;        /* SPS_FP32 / SPS_FP64 (default FP32) */
    int64_t max_iters;        /* default 100000 (solver/config.py:37) */
    double  tol;              /* relative KKT tolerance, default 1e-6 (solver/config.py:12) */
    int32_t check_interval;   /* iterations between KKT checks; 0 = 50 (reference) / 64 (adaptive) */
    int32_t ruiz_iters;       /* adaptive mode: Ruiz passes before Pock-Chambolle, default 10 */
    double  time_limit_s;     /* 0 = none; enforced on the device clock and by the host watchdog */
    int32_t graph_mode;       /* 0 = plain launches, 1 = replayed window graph,
                                 2 = one graph with a device-driven while loop (default) */
    int32_t device;           /* CUDA device ordinal */
    int32_t max_blocks;       /* schedule tuning: blocks per matrix-pass launch, 0 = one resident wave */
    int32_t batch_group;      /* batched solver: lanes per column (1, 2, 4, 8, 16, 32), 0 = autotune */
    int32_t escalate;         /* adaptive FP32 stall handling.  A solve stalls when its best
                                 relative KKT error has not halved for max(2048, k/2) attempts
                                 (k = attempt of the last halving); a single LP only once that
                                 error is at most 1e-3 (counting from when it got there), a
                                 batch instance at any error.  1 (default): continue in
                                 FP64 from the best point seen, with the primal weight it had;
                                 2: stop with SPS_STATUS_STALLED; 0: no stall test (FP32 only) */
    int32_t warm_fallback;    /* 1 (default): a warm start whose relative KKT error is larger than
                                 the cold start's (x = clip(0, lb, ub), y = 0) is dropped and the
                                 solve starts cold; 0: always start from the warm point */
    int32_t batch_team;       /* batched solver: blocks (one thread-block cluster) per large
                                 instance, 1..8; 1 = one block per instance; 0 = 4, or in a
                                 batch of fewer instances than half the resident blocks the
                                 largest of 2, 4, 8 that keeps every instance resident */
    int32_t batch_team_nnz;   /* batched solver: instances with at least this many nonzeros are
                                 large; 0 = 65536 in such a small batch, else the larger of
                                 65536 and twice the median instance */
    int32_t batch_handoff_nnz;/* batched solver: > 0: once the instance queue is empty and 7/8
                                 of the blocks have left, an instance with at least this many
                                 nonzeros and 512 attempts still running stops at its next check
                                 and is finished by the single-LP engine (FP32, the whole GPU)
                                 from its current point.  Which instances leave depends on
                                 timing, so results are no longer bit-identical from run to run;
                                 0 (default) = never */
    int32_t kkt_form;         /* SPS_KKT_LAGRANGIAN (default) or SPS_KKT_PDLP; adaptive mode of
                                 the single-LP engine only (sps_batch_create rejects PDLP) */
} sps_options;

typedef struct {
    int32_t status;           /* SPS_STATUS_* */
    int32_t restarts;
    int64_t iterations;       /* PDHG iterations run (adaptive: step attempts) */
    int64_t accepted_steps;   /* adaptive mode: accepted attempts */
    double  objective;        /* c^T x of the returned x (minimisation c), FP64 */
    double  rel_kkt;          /* max(rel_primal, rel_dual, rel_gap) of the returned point */
    double  rel_primal;
    double  rel_dual;
    double  rel_gap;
    double  primal_weight;    /* adaptive mode: final omega */
    double  step_size;        /* adaptive mode: final eta */
    double  setup_ms;         /* sps_create device work (upload, layout, scaling) */
    double  solve_ms;         /* device time of sps_solve */
    int64_t kernel_launches;  /* kernels launched by sps_solve (graph nodes executed count once per run) */
    int32_t returned_average; /* 1 if the returned point is the ergodic average */
    int32_t escalated;        /* 1 if the solve stalled in FP32 and was finished in FP64; the
                                 iteration, restart and time fields then cover both parts */
    int32_t warm_start_used;  /* 1 if the solve started from the caller's warm start (0 when none
                                 was given or the cold-start fallback rejected it) */
    int32_t reserved;
    double  rel_kkt_lagrangian; /* the returned point's relative KKT error in the Lagrangian form
                                   (SPS_KKT_LAGRANGIAN); equals rel_kkt unless kkt_form is PDLP */
} sps_result;

typedef struct sps_handle sps_handle;

/* Fill *opt with defaults. */
int sps_options_init(sps_options *opt);

/* Upload a problem, build the device layout (row/column-binned CSR and CSC),
 * scale it, and allocate iterate storage.  Replaces the reference's
 * _to_standard_form_pdhg + _compute_step_sizes + DeviceEngine.prepare_data
 * (solver/lp/pdhg.py:62-147, solver/lp/pdhg_gpu.py:123-194). */
int sps_create(const sps_problem_desc *prob, const sps_options *opt, sps_handle **out);

/* Start the next solve from (x0, y0) in the original space (either may be
 * NULL = zero) with primal weight omega0 (<= 0 = default).  Adaptive mode only.
 * With sps_options.warm_fallback the solve compares the start point's relative
 * KKT error with the cold start's and keeps the better (sps_result.warm_start_used).
 * New API surface: the reference always starts from zero (solver/lp/pdhg.py:175-176). */
int sps_set_warm_start(sps_handle *h, const double *x0, const double *y0, double omega0);

/* Run restarted PDHG to tolerance or limit; blocking.  Replaces the iteration
 * loop of solve_lp_pdhg / solve_lp_pdhg_gpu (solver/lp/pdhg.py:209-244,
 * solver/lp/pdhg_gpu.py:378-427). */
int sps_solve(sps_handle *h, sps_result *res);

/* Copy the solution of the last solve into caller buffers (either may be NULL):
 * x (n) in the original space, clipped to [lb, ub] as solver/lp/pdhg.py:247-253;
 * y (m_ub + m_eq) duals of the A_ub rows then the A_eq rows. */
int sps_get_solution(sps_handle *h, double *x, double *y);

/* Benchmark support (no reference counterpart): after a sps_solve, launch
 * `reps` iterations' kernels one by one on the handle's stream and time each
 * launch with CUDA events.  out[0] = mean ms of the row-pass kernel (CSR SpMV
 * fused with the dual update), out[1] = mean ms of the column-pass kernel (CSC
 * SpMV fused with the primal update), out[2] = fraction of step attempts whose
 * column pass ran the SpMV (accepted steps; 1 in the reference mode).  The
 * solution returned by sps_get_solution is not affected. */
int sps_time_iteration_kernels(sps_handle *h, int32_t reps, double *out);

/* The same kernels and outputs as sps_time_iteration_kernels, timed as the
 * solve's own graph runs them (back to back from the device, no host launch
 * gaps): one CUDA graph of `reps` x [row pass, column pass] and one of `reps`
 * x [row pass] are captured on the handle's stream and replayed (after one
 * warm-up replay each) between two events; out[0] = the second's time / reps,
 * out[1] = (the first's - the second's) / reps, so out[0] + out[1] is the
 * in-graph time of one step attempt. */
int sps_time_iteration_kernels_graph(sps_handle *h, int32_t reps, double *out);

/* Benchmark support (no reference counterpart): the floor of a sparse pass over
 * nnz nonzeros whose column indices are uniform random over a vector of
 * vec_len FP32 entries — each thread reads four consecutive int32 indices and
 * FP32 values as 16-byte loads and gathers x at them, nothing else — timed with
 * CUDA events on device `device`, `reps` passes after one warm-up, one
 * resident wave of blocks.  out[0] = mean ms with random indices, out[1] = mean
 * ms with indices walking x in order (the same bytes streamed).  Allocates and
 * frees its own device memory.  Errors: sps_last_error(NULL). */
int sps_time_gather_floor(int64_t nnz, int32_t vec_len, int32_t reps, int32_t device, double *out);

/* Message of the last error on this handle (or of the last failed sps_create when h is NULL). */
const char *sps_last_error(const sps_handle *h);

/* Release the handle (the reference's DeviceEngine, solver/lp/pdhg_gpu.py:72,
 * is released by garbage collection).  Its device memory returns to the library's
 * memory pool of the CUDA context, which keeps up to 8 GiB of freed memory
 * mapped for later sps_create calls; memory beyond that goes back to the
 * system at the next synchronisation. */
void sps_destroy(sps_handle *h);

/* Page-lock / release caller host memory so uploads run at full link speed. */
int sps_pin_host(void *ptr, uint64_t bytes);
int sps_unpin_host(void *ptr);

/* Library build string (arch, precision support). */
const char *sps_version(void);

/* ---- batched solver: thousands of independent LPs in one persistent launch.
 * New API surface (the reference solves one LP per call; its MILP strong
 * branching, solver/milp/branching.py:132-210, is the natural batch caller).
 * Adaptive mode, FP32 iterates, FP64 checks; every instance keeps its own step
 * size, primal weight, restarts and termination. */
typedef struct sps_batch sps_batch;

typedef struct {
    double  setup_ms;           /* sps_batch_create device work (upload excluded) */
    double  solve_ms;           /* the persistent launch plus the continuations after it */
    int64_t total_iterations;   /* sum over instances */
    int32_t optimal;            /* instances that reached tol */
    int32_t lanes_per_column;   /* schedule used: given, autotuned at create, or taken from an
                                   earlier batch of the same shape in this process */
    int32_t blocks;             /* persistent blocks */
    int32_t escalated;          /* instances that stalled in FP32 and were finished in FP64 by the
                                   single-LP engine after the persistent launch (in solve_ms) */
    int32_t lanes_per_row;      /* row-pass schedule (4, 8, 16, 32 lanes per row; timed) */
    int32_t team;               /* blocks per large instance in the launch (1 = no clusters) */
    int32_t handed_off;         /* instances finished by the single-LP engine after leaving the
                                   launch's tail (batch_handoff_nnz; in solve_ms) */
    int32_t reserved[1];
} sps_batch_stats;

/* Pack `count` problems, upload and scale them (one block per instance) and pick
 * the schedule: lanes per column (opt->batch_group, or timed on a sample when 0),
 * then lanes per row (timed). */
int sps_batch_create(int32_t count, const sps_problem_desc *probs, const sps_options *opt, sps_batch **out);
/* Solve every instance: one persistent launch, captured in a CUDA graph on the
 * first call and replayed afterwards; blocking. */
int sps_batch_solve(sps_batch *b, sps_batch_stats *stats);
/* Warm starts for the following solves, packed in instance order: x0 (sum of n),
 * y0 (sum of m_ub + m_eq), omega0 (count; <= 0 = the instance's default), all in
 * the original space; x0 = y0 = NULL clears them.  With sps_options.warm_fallback
 * (default) an instance whose warm point has a larger relative KKT error than its
 * cold start starts cold (sps_result.warm_start_used = 0). */
int sps_batch_set_warm_starts(sps_batch *b, const double *x0, const double *y0, const double *omega0);
/* Instance k of the last solve: x (n, clipped to bounds), y (m_ub + m_eq), result.
 * res->solve_ms is the instance's own device time inside the persistent launch
 * (plus its FP64 continuation, if any); setup_ms is the batch's. */
int sps_batch_get(sps_batch *b, int32_t k, double *x, double *y, sps_result *res);
const char *sps_batch_last_error(const sps_batch *b);
void sps_batch_destroy(sps_batch *b);

/* An LP whose arrays already live in device memory (all pointers are device
 * pointers): K = [A_ub; A_eq] in CSR with the m_ub '<=' rows first. */
typedef struct {
    int32_t n, m_ub, m_eq;
    const int32_t *indptr;          /* m_ub + m_eq + 1 */
    const int32_t *indices;
    const double  *values;
    const double  *c;               /* n */
    const double  *rhs;             /* m_ub + m_eq: b_ub then b_eq */
    const double  *lb, *ub;         /* n, +-INFINITY allowed */
} sps_device_lp;

/* Relative KKT error of a point (x, y) of a device-resident LP, computed in
 * FP64 without allocating any device memory.  No counterpart in the
 * reference.  For callers that cannot call cudaMalloc at that point: code
 * inside another framework's memory pool or a fixed device-memory budget, or a
 * latency-critical loop where an allocation would synchronise the device.
 * x (n), y (m_ub + m_eq) and out are device pointers; out receives 6 doubles:
 * rel_kkt, rel_primal, rel_dual, rel_gap, primal objective, dual objective —
 * the same measure sps_solve reports (sps_result.rel_*).  Work is queued on
 * `stream` (a cudaStream_t, NULL = default stream); the call does not wait.
 * Preconditions the call cannot check without reading device memory: every
 * column index lies in [0, n), indptr is non-decreasing from 0.  Every array
 * the LP needs must be non-NULL, also for rows without nonzeros (indptr,
 * indices, values and rhs when m_ub + m_eq > 0; c, lb, ub when n > 0), else
 * SPS_ERR_INVALID.  K^T y is summed with integer digits, so the result is
 * bitwise reproducible from call to call.
 * Scratch is a fixed ~6.3 MB device array inside the library (held by every
 * GPU that loads it until exit), so n is limited to 262144 columns (larger n
 * returns SPS_ERR_INVALID); rows are unlimited.  All calls share that array:
 * calls that overlap on the GPU race — order them on one stream.  The first
 * call in each CUDA context looks up the array's device address; make that
 * first call before any stream capture.  Errors: sps_last_error(NULL). */
int sps_kkt_noalloc(const sps_device_lp *lp, const double *x, const double *y, double *out, void *stream);

/* Number of visible CUDA devices (0 when none or the driver is unusable).
 * Backs get_available_device (solver/lp/pdhg_gpu.py:42-67), without its
 * CuPy/MPS/CPU probing. */
int sps_device_count(void);

#ifdef __cplusplus
}
#endif
#endif /* SPS_PDHG_H */
