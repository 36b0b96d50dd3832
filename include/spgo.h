/*
 * spgo.h - C ABI of the GB300-native stereo pose-graph / bundle-adjustment
 * Levenberg-Marquardt solver (drop-in for S-PGO's CUDA solver).
 *
 * Plain C: pointers, sizes and an int status on every call; no C++ or torch
 * types.  All device memory is caller-owned (for example torch tensors): the
 * library sizes it, the caller allocates it, the library only reads and
 * writes it.  Every call that touches the GPU takes an explicit cudaStream_t
 * (passed as void*) and only enqueues work on it unless stated otherwise.
 *
 * Reference interface each entry point replaces (paths inside S-PGO):
 *   spgo_plan_create          Solver::Solver + loadCalibration + writeObservations
 *                             (include/Solver.hpp:20-57, src/Optimization/Solver.cpp:29-56):
 *                             one bulk, landmark-major upload instead of one
 *                             index_put_ per scalar
 *   spgo_solver_create        LMvariables::allocateMemory (src/Optimization/LMutils.cu:5-130),
 *                             done once instead of on every step()
 *   spgo_gn_step              Solver::step / updateState (Solver.cpp:5-27,
 *                             src/Optimization/Solver_cuda.cu:557-795)
 *   spgo_lm_reset/iterate/status   new: Nielsen-damped LM with FP64 gain ratio
 *                             (no counterpart in the reference)
 *   spgo_export_system        LMvariables::*_to_txt debug dumps (LMutils.cu:188-536)
 *                             and Optimizer.getHessians (PythonUtils/Optimizer.py:376-383)
 * Pose and inverse-depth read/write (Solver.cpp:59-128) are plain copies of the
 * caller-owned state buffers and need no entry point.
 */
#ifndef SPGO_H
#define SPGO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define SPGO_OK                   0
#define SPGO_ERR_INVALID_ARG     -1
#define SPGO_ERR_UNSUPPORTED     -2   /* e.g. a landmark window wider than SPGO_MAX_WINDOW */
#define SPGO_ERR_BUFFER_SMALL    -3
#define SPGO_ERR_CUDA            -4
#define SPGO_ERR_NOT_SPD         -5   /* reduced camera system not positive definite */

#define SPGO_MAX_WINDOW          96   /* max pose blocks one landmark's Jacobian spans */

/* precision of the linearisation, Schur complement and factorisation */
#define SPGO_PREC_MIXED           0   /* FP32 J/H/Schur, FP32 Cholesky + FP64 refinement, FP64 cost */
#define SPGO_PREC_FP64            1   /* plain FP64 everywhere */

/* robust loss */
#define SPGO_LOSS_L2              0
#define SPGO_LOSS_CAUCHY          1
#define SPGO_LOSS_HUBER           2

/* per-problem LM status */
#define SPGO_STATUS_RUNNING       0
#define SPGO_STATUS_CONVERGED     1   /* relative cost decrease below tol on an accepted step */
#define SPGO_STATUS_MAX_ITERS     2
#define SPGO_STATUS_STALLED       3   /* lambda exceeded lambda_max */

/* ---- host-side problem description (one problem, host memory) ---------
 * Landmark-major CSR: landmark l has its host (anchor) frame host[l], the
 * left pixel it was observed at in the host, and observations
 * [obs_ptr[l], obs_ptr[l+1]) with strictly ascending frames.  Frame 0 is
 * fixed; frames run 0..n_poses.  The host frame's own observation is part of
 * the list (it carries the stereo depth constraint).  Mirrors the arguments of
 * Solver::loadCalibration and Solver::writeObservations (Solver.cpp:29-56). */
typedef struct spgo_host_problem {
    int32_t        n_poses;      /* N incremental poses, N + 1 frames        */
    int32_t        n_landmarks;  /* L                                         */
    int64_t        n_obs;        /* O stereo observations                     */
    const float   *intrinsics;   /* [8] fx_l, fy_l, cx_l, cy_l, fx_r, fy_r, cx_r, cy_r */
    const double  *T_r_to_l;     /* [16] row-major pose of the right camera in the left frame */
    const int32_t *host;         /* [L]                                       */
    const float   *anchor_uv;    /* [L*2]                                     */
    const int64_t *obs_ptr;      /* [L+1]                                     */
    const int32_t *obs_frame;    /* [O]                                       */
    const float   *obs_uv;       /* [O*4] uL, vL, uR, vR                      */
    /* Optional FP64 pixels: when non-null they are read instead of anchor_uv /
     * obs_uv (which may then be null) and rounded to float as the plan is built,
     * so a caller holding double pixels needs no conversion pass of its own. */
    const double  *anchor_uv_f64; /* [L*2] or NULL */
    const double  *obs_uv_f64;    /* [O*4] or NULL */
} spgo_host_problem;

/* sizes a plan needs (bytes unless noted) */
typedef struct spgo_plan_sizes {
    int32_t n_problems;
    int32_t total_poses;         /* length of the pose state in 12-double records */
    int32_t total_landmarks;     /* length of the inverse-depth state            */
    int64_t total_obs;
    int32_t n_chunks;
    int32_t n_schur_items;
    int32_t max_params;          /* max 6N over problems */
    int32_t schur_chunk_tiles;   /* (chunk, 48x48 output tile) products per Schur pass */
    size_t  static_bytes;        /* device buffer for the uploaded problem data   */
    size_t  workspace_bytes;     /* device buffer for per-iteration scratch       */
    int64_t slab_elems;          /* elements of the landmark-chunk slabs (W blocks) */
    int64_t pair_records;        /* (lo, hi) pose-pair accumulators               */
    int64_t schur_flops;         /* algorithmic FLOPs of one landmark Schur pass:
                                    sum over chunks of 2 (6 nb)^2 x 32 (W D^-1 W^T blocks) */
    int32_t n_tc_items;          /* tensor-core Schur work items (128x128 tiles x chunk lists) */
    int32_t tc_chunk_tiles;      /* (chunk, 128x128 tile) products per tensor-core pass */
    int64_t schur_flops_landmark; /* algorithmic FLOPs of the landmark Schur complement:
                                    sum over landmarks of 2 (6 k)^2, k = pose blocks its
                                    Jacobian spans (no chunk padding, no split products) */
    int32_t tc_split;            /* the plan's Schur work shapes (spgo_plan_options) */
    int32_t simt_split;
} spgo_plan_sizes;

/* Plan-time shapes of the Schur complement's work lists (spgo_plan_create_opts; a
 * zero field takes its default).  tc_split: landmark chunks per tensor-core work item
 * (one 128x128 output tile), 1..64, default 64; simt_split: chunks per SIMT work item
 * (one 48x48 tile), 1..64, default 16.  Fewer chunks per item: more CTAs, more partial
 * tiles added into S_L.  BatchSolver.autotune_plan times them on the caller's batch. */
typedef struct spgo_plan_options {
    int32_t tc_split;
    int32_t simt_split;
    int32_t reserved[6];         /* zero */
} spgo_plan_options;

/* solver parameters */
typedef struct spgo_params {
    int32_t loss;                /* SPGO_LOSS_*                                  */
    int32_t near_boost;          /* 1: x4 weight when |target-anchor| < 2 (Solver_cuda.cu:226-228) */
    float   loss_scale;          /* Cauchy c (reference c^2 = 9) or Huber delta  */
    float   eps;                 /* inverse-depth diagonal guard (LMutils.h:50: 1e-4) */
    float   alpha_min;           /* inverse-depth clamp (LMutils.h:54-55)        */
    float   alpha_max;
    double  lambda0;             /* Nielsen initial damping (Marquardt scaling)  */
    double  lambda_max;
    double  tol;                 /* relative cost decrease that counts as converged */
    int32_t max_iters;           /* per-problem LM iteration cap                 */
    int32_t refine_steps;        /* mixed path with outer_steps = 0: refinement steps of the
                                    reduced solve against the exactly assembled S (default 1);
                                    with outer_steps > 0 the refinement of the whole step
                                    replaces them */
    int32_t use_graph;           /* 1: spgo_lm_iterate replays a captured CUDA graph
                                    (not on the legacy default stream, not while profiling) */
    int32_t use_tc;              /* 1 (default): mixed path forms the landmark Schur complement
                                    on the tensor cores (tcgen05, split TF32, FP32 accumulate);
                                    0: FP32 SIMT */
    int32_t cost_block;          /* threads per CTA of the cost pass (0: 64; else 32..256, x32) */
    int32_t lin_block;           /* threads per CTA of the Jacobian pass (0: 256; else 32..256, x32) */
    int32_t outer_steps;         /* mixed path: steps of iterative refinement of the whole damped
                                    normal equations (poses and inverse depths) against a
                                    residual J^T (r - J x) - Lambda x formed from the FP32
                                    Jacobian with exact products and FP64-grade sums; the FP32
                                    system (pose Hessian, tensor-core Schur complement, FP32
                                    Cholesky) only preconditions.  Default 2 (the second only
                                    where outer_tol asks for it); 0: the FP32 step as solved */
    int32_t wait_us;             /* limit of every bounded device-side wait, microseconds
                                    (0: 2 s).  Shortening it only makes waits give up sooner:
                                    the problem is flagged and its step rejected */
    float   ctl_min_log10;       /* learned damping: the largest decrease of lambda one proposal
                                    may make, as log10 of the factor, in [-6, 0] (default -6:
                                    the network's own range) */
    float   outer_tol;           /* mixed path, outer_steps > 1: a problem takes the next
                                    refinement step only while its last correction exceeds
                                    outer_tol times its step (largest entries); default 1e-3;
                                    0: every step */
    float   stop_rho;            /* an accepted step whose relative decrease is below tol ends
                                    the solve only if its gain ratio (actual / predicted
                                    decrease) is at least stop_rho, or its predicted decrease
                                    is itself below tol, or the accepted step before it was
                                    also below tol; a single poorly modelled step that
                                    predicted more marks a plateau, not a converged problem,
                                    and the solve goes on.  In [0, 1); default 0: every such
                                    step ends it */
} spgo_params;

typedef struct spgo_problem_status {
    double  cost0;               /* cost at the first linearisation */
    double  cost;                /* current (accepted) cost          */
    double  lambda;
    int32_t iterations;          /* LM solves (accepted + rejected)  */
    int32_t accepted;
    int32_t status;              /* SPGO_STATUS_*                    */
    int32_t factor_failures;     /* steps rejected for a non-positive pivot  */
    int32_t wait_timeouts;       /* steps rejected because a bounded device wait ran out
                                    (spgo_params.wait_us)               */
    int32_t pad;
} spgo_problem_status;

typedef struct spgo_plan   spgo_plan;
typedef struct spgo_solver spgo_solver;

int         spgo_version(void);
const char *spgo_last_error(void);
void        spgo_default_params(spgo_params *p);

/* Host-side planning: validates the problems, orders landmarks by Jacobian
 * window, groups them into 32-landmark chunks and builds the Schur tile work
 * list, on up to 16 host threads (two cores are left to other threads).  No
 * device work: the static tables are written into page-locked host staging
 * (ordinary heap memory without a CUDA device) taken from a small process-wide
 * cache, so it may run on any thread, e.g. for the next batch while the
 * current one solves.  Thread-safe. */
int spgo_plan_create(const spgo_host_problem *problems, int32_t n_problems,
                     int32_t precision, spgo_plan **out);
/* The same with the work shapes of `opts` (NULL: the defaults). */
int spgo_plan_create_opts(const spgo_host_problem *problems, int32_t n_problems,
                          int32_t precision, const spgo_plan_options *opts, spgo_plan **out);
int spgo_plan_sizes_get(const spgo_plan *plan, spgo_plan_sizes *out);
int spgo_plan_destroy(spgo_plan *plan);
/* Landmark permutation: internal slot -> (problem-local) landmark order is
 * handled inside; this returns the global landmark offset of each problem
 * ([n_problems]) and the pose offset ([n_problems]) into the state buffers. */
int spgo_plan_offsets(const spgo_plan *plan, int32_t *lm_off, int32_t *pose_off);

/* Binds caller-owned device memory and uploads the plan: two asynchronous DMA
 * copies on `stream` from the plan's page-locked staging (spgo_plan_destroy
 * waits for them before the staging is reused).  The solver keeps reading the
 * plan's host tables, so the plan must outlive the solver.  State buffers:
 * poses [total_poses*12] (3x4 row-major incremental T_curr_to_next, FP64) and
 * alpha [total_landmarks] (FP64), both in the caller's problem/landmark order. */
int spgo_solver_create(const spgo_plan *plan, void *d_static, size_t static_bytes,
                       void *d_workspace, size_t workspace_bytes,
                       double *d_poses, double *d_alpha, void *stream, spgo_solver **out);
int spgo_solver_destroy(spgo_solver *s);
int spgo_set_params(spgo_solver *s, const spgo_params *p);

/* The reference's step(iterations): undamped Gauss-Newton with C + eps, pose
 * step scaled by step_size, unscaled clamped inverse-depth update
 * (Solver_cuda.cu:594-782).  Enqueue only. */
int spgo_gn_step(spgo_solver *s, int32_t iterations, float step_size, void *stream);

/* Nielsen LM.  reset: lambda = lambda0, nu = 2, counters cleared, first
 * linearisation pending.  iterate: enqueue n_iters LM iterations for every
 * problem still running (no host synchronisation; capturable in a CUDA
 * graph).  status: synchronises `stream` and copies per-problem status to
 * host memory out[n_problems]. */
int spgo_lm_reset(spgo_solver *s, void *stream);
int spgo_lm_iterate(spgo_solver *s, int32_t n_iters, void *stream);
int spgo_lm_status(spgo_solver *s, spgo_problem_status *out, void *stream);
/* Per-iteration trace of every problem since the last reset (the cost trace the
 * reference's callers build by reading poses back after each step()): for
 * iteration k < min(iterations, SPGO_TRACE_MAX) of problem b, host arrays indexed
 * [b * capacity + k] receive the cost after the iteration (the candidate's when it
 * was accepted, else unchanged), the lambda the step was solved with, and 1 / 0
 * for accepted / rejected.  n_iters[b] = iterations recorded.  Synchronises the
 * stream.  Any output pointer may be NULL. */
#define SPGO_TRACE_MAX 128
int spgo_lm_trace(spgo_solver *s, int32_t capacity, double *cost, double *lambda, int32_t *accepted,
                  int32_t *n_iters, void *stream);
/* Convenience: reset, iterate until every problem stops or max_iters, with a
 * status check every `check_every` iterations.  Returns the iteration count
 * in *iters_done (max over problems). */
int spgo_lm_solve(spgo_solver *s, int32_t check_every, int32_t *iters_done, void *stream);

/* Autotuner (no reference counterpart): times the launch shapes that can change
 * without re-planning on this solver's own batch -- cost-pass CTA size {64, 128,
 * 256}, Jacobian-pass CTA size {128, 256}, and (mixed precision) the Schur path
 * {tensor cores, SIMT} -- over a reset plus two LM iterations each (CUDA graphs
 * off, events on), keeps the fastest of each, and applies them.  The poses and
 * inverse depths are restored afterwards; the LM state is reset; profiling is
 * switched off.  `chosen` (optional) receives the resulting parameters. */
int spgo_autotune(spgo_solver *s, spgo_params *chosen, void *stream);

/* Linearise at the current state and export one problem's dense system into
 * caller-owned DEVICE buffers (any pointer may be NULL):
 * A [P*P] and g [P] (FP64, incremental parameterisation), B [P*L] (FP64,
 * row-major, the problem's landmark order), C [L], g_a [L] (FP64), cost [1].
 * For parity checks on small problems. */
int spgo_export_system(spgo_solver *s, int32_t problem, double *A, double *g, double *B,
                       double *C, double *g_a, double *cost, void *stream);

/* Linearise every problem at its current state and export one problem's damped
 * reduced camera system S = A + lambda diag(A) - B D^-1 B^T, D = C (1 + lambda) + eps,
 * and g_S = g - B D^-1 g_a, as FP64 into caller-owned DEVICE buffers S [P*P],
 * gS [P].  For parity checks of the Schur complement. */
int spgo_export_reduced(spgo_solver *s, int32_t problem, double lambda, double *S, double *gS, void *stream);

/* ---- learned damping controller (no counterpart in the reference) ---------
 * A 16 -> 64 -> 64 -> 2 MLP (exact GELU) proposes the next LM damping from the
 * cost, gain-ratio history, lambda, gradient and Hessian-diagonal statistics.
 * Parameters: one flat FP32 vector of SPGO_MLP_PARAMS floats, W1 [64x16] (out x
 * in), b1 [64], W2 [64x64], b2 [64], W3 [2x64], b3 [2].  Outputs: change of
 * log10(lambda) and the logit that the current damping yields an accepted step. */
#define SPGO_MLP_PARAMS 5378
#define SPGO_MLP_INPUTS 16
#define SPGO_MLP_CACHE_PER_SAMPLE 386   /* floats of spgo_mlp_grad scratch per sample */

/* FP32 forward of n feature rows d_X [n*16] -> d_out [n*2]; d_cache [n*128]
 * (or NULL) keeps the pre-activations for spgo_mlp_grad. */
int spgo_mlp_forward(const float *d_params, const float *d_X, int32_t n, float *d_out, float *d_cache,
                     void *stream);
/* Mean loss (out0 - t0)^2 + BCE(out1, t1) over n samples with targets d_T [n*2]
 * and its gradient d_grad [SPGO_MLP_PARAMS]; d_loss [1]; scratch d_out [n*2],
 * d_cache [n*SPGO_MLP_CACHE_PER_SAMPLE]. */
int spgo_mlp_grad(const float *d_params, const float *d_X, const float *d_T, int32_t n, float *d_grad,
                  float *d_loss, float *d_out, float *d_cache, void *stream);
/* One Adam step (beta 0.9 / 0.999) on the parameters; step counts from 1. */
int spgo_mlp_adam(float *d_params, const float *d_grad, float *d_m, float *d_v, int32_t step, float lr,
                  void *stream);
/* Use the controller (BF16 weights, converted from d_params) in spgo_lm_iterate:
 * after an accepted step its proposal replaces the Nielsen update when its
 * accept logit is positive; a rejected step always falls back to Nielsen.
 * d_params = NULL switches it off. */
int spgo_lm_set_controller(spgo_solver *s, const float *d_params, void *stream);
/* The controller's 16 inputs for every problem at its current state, d_feat [B*16]. */
int spgo_lm_features(spgo_solver *s, float *d_feat, void *stream);
/* Linearise where needed, then for each of n_factors (<= 32) damping factors f
 * evaluate the cost of the step taken with lambda * f for every running problem,
 * leaving the state and the LM bookkeeping unchanged; host costs [n_factors*B]
 * (synchronises the stream). */
int spgo_lm_probe(spgo_solver *s, int32_t n_factors, const double *factors, double *costs, void *stream);

/* Count of kernel launches enqueued since the solver was created, graph replays
 * included, by the calling thread (drive a solver from one thread at a time;
 * solvers on other threads do not count here). */
int64_t spgo_launch_count(const spgo_solver *s);

/* Optional per-kernel timing with CUDA events on the launching stream.
 * enable: create `capacity` event pairs (0 disables); each profiled launch
 * uses one pair until they run out.  read: synchronise `stream`, return the
 * summed milliseconds and launch counts per kind, and recycle the events.
 * Kinds (n_kinds >= 12): 0 pose chain, 1 linearisation, 2 cost pass,
 * 3 pair reduction, 4 Schur complement, 5 assembly, 6 factor + solve,
 * 7 inverse-depth back-substitution, 8 pose update, 9 LM bookkeeping,
 * 10 step refinement: its reduced solves and pair twists (mixed path),
 * 11 step refinement: one residual pass over the observations (mixed path). */
#define SPGO_PROFILE_KINDS 12
int spgo_profile_enable(spgo_solver *s, int32_t capacity);
int spgo_profile_read(spgo_solver *s, double *ms, int64_t *count, int32_t n_kinds, void *stream);

/* ---- allocation-free cost evaluation ------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory: code running inside a CUDA graph capture it does not own, plugins
 * whose host framework owns the device memory pool and forbids cudaMalloc,
 * and real-time threads where an allocation (and the synchronisation it can
 * imply) is not allowed.  It evaluates the same robust cost as the cost pass
 * of the solver (0.5 * sum of the weighted robust loss over both cameras of
 * every observation, FP64) for ONE problem whose arrays the caller already
 * holds in device memory, at the state d_poses [n_poses*12] (3x4 row-major
 * incremental poses) and d_alpha [n_landmarks], and writes it to d_cost[0].
 * Only params->loss, loss_scale and near_boost are read.
 *
 * Preconditions the host cannot check (the arrays are in device memory):
 * d_poses holds n_poses * 12 doubles and d_alpha n_landmarks doubles; host[l]
 * and obs_frame[o] lie in [0, n_poses]; obs_ptr is non-decreasing with
 * obs_ptr[0] >= 0 and obs_ptr[n_landmarks] <= n_obs.  The kernel checks the
 * indices it dereferences: a landmark or observation that breaks them is skipped
 * and the returned cost is NaN.
 *
 * It calls no cudaMalloc/cudaFree or allocating library routine: its scratch
 * is a file-scope device array of about 0.9 MB that every GPU loading this
 * library keeps until the process exits, so problems are limited to
 * n_poses + 1 <= SPGO_NOALLOC_MAX_FRAMES and n_landmarks <=
 * SPGO_NOALLOC_MAX_LANDMARKS (larger ones return SPGO_ERR_UNSUPPORTED).
 * The first call on a device looks up that array's device address (no
 * allocation); make that first call before any stream capture.  The address is
 * kept for the process: a device reset (cudaDeviceReset) after the first call
 * is not supported (a failed launch makes the next call look it up again).  All calls
 * share the array: calls whose kernels overlap on the GPU race, so order them
 * (one stream, or events).  Enqueue only; d_cost is valid once `stream`
 * reaches the end of the call. */
#define SPGO_NOALLOC_MAX_FRAMES     2048
#define SPGO_NOALLOC_MAX_LANDMARKS  (1 << 21)

typedef struct spgo_device_problem {   /* same fields as spgo_host_problem, DEVICE pointers */
    int32_t        n_poses;
    int32_t        n_landmarks;
    int64_t        n_obs;
    const float   *intrinsics;   /* [8]   */
    const double  *T_r_to_l;     /* [16]  */
    const int32_t *host;         /* [L]   */
    const float   *anchor_uv;    /* [L*2] */
    const int64_t *obs_ptr;      /* [L+1] */
    const int32_t *obs_frame;    /* [O]   */
    const float   *obs_uv;       /* [O*4] */
} spgo_device_problem;

int spgo_cost_noalloc(const spgo_device_problem *prob, const double *d_poses, const double *d_alpha,
                      const spgo_params *params, double *d_cost, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SPGO_H */
