// Internal definitions shared by the planner (host C++) and the CUDA kernels.
//
// Data layout in HBM (all offsets are element offsets into per-kind arrays):
//   frames      f = frame_off[b] + k, k = 0..N_b           (N_b + 1 frames per problem)
//   poses       p = pose_off[b] + k,  k = 0..N_b - 1       (12 doubles: 3x4 row-major)
//   params      param_off[b] + 6k + {psi0..2, rho0..2}     (P_b = 6 N_b)
//   dense PxP   S_off[b] + r * P_b + c                     (A, S_L, S, factor)
//   landmarks   internal order = problem-major, sorted by Jacobian window;
//               lm_user[li] maps to the caller's (problem-major) order
//   obs         grouped by internal landmark, frames ascending
//   pairs       pair_off[b] + lo * D_b + (d - 1), d = hi - lo in [1, D_b]: the
//               (lo, hi) accumulators of the incremental-chain Hessian
//   chunks      <= 32 landmarks of one problem with windows inside
//               [f0, f0 + nb); slab = (6 nb) x 32 row-major (landmark-contiguous)
#pragma once
#include <stdint.h>
#include <stddef.h>
#include "spgo.h"

#define SPGO_CHUNK 32          // landmarks per chunk (slab columns)
#define SPGO_TILE_BLOCKS 8     // pose blocks per Schur output tile (48 rows)
#define SPGO_KSPLIT 16         // chunks per Schur work item
#define SPGO_TC_SPLIT 64       // chunks per tensor-core Schur work item
#define SPGO_FACTOR_SMEM (200 * 1024)  // shared-memory budget of the batched factorisation

namespace spgo {

// which problems a kernel works on: all, those needing a relinearisation, those still
// running, those about to be linearised for the first time since the reset, those
// still running whose last step was rejected (after the decision)
enum Gate { GATE_ALL = 0, GATE_RELIN = 1, GATE_RUNNING = 2, GATE_FIRST = 3, GATE_REJECTED = 4 };

struct PlanView {                 // device pointers into the static buffer
  int32_t B, F, NP, L;
  int64_t O;
  int32_t n_chunks, n_items, max_P, max_D, max_nb, n_work_chunks;
  int64_t total_S, total_pairs;
  int32_t total_params;
  // per problem
  const int32_t *p_npose, *p_frame_off, *p_pose_off, *p_lm_off, *p_lm_cnt, *p_pair_D,
      *p_param_off, *p_chunk_off, *p_chunk_cnt;
  const int64_t *p_S_off, *p_pair_off;
  const int64_t *p_nres;   // residual rows (4 per stereo observation)
  const float *p_intr;    // [B][8]
  const double *p_Trl;    // [B][12]
  // per landmark (internal order)
  const int32_t *lm_prob, *lm_host, *lm_lo, *lm_hi, *lm_user, *lm_chunk, *lm_slot;
  const float *lm_uv;     // [L][2]
  const int64_t *lm_obs;  // [L+1]
  // per observation
  const uint8_t *obs_slot;   // landmark slot inside its chunk
  const int32_t *obs_frame;
  const float *obs_uv;    // [O][4]
  // chunks
  const int32_t *ch_prob, *ch_f0, *ch_nb, *ch_lm0, *ch_cnt;
  const int64_t *ch_slab;
  // Schur work items
  const int32_t *wk_prob, *wk_ti, *wk_tj, *wk_cbeg, *wk_cend, *wk_chunks;
  // frame -> problem
  const int32_t *fr_prob;
  const int32_t *pose_prob;
  // tensor-core Schur work items
  const int32_t *tc_prob, *tc_row0, *tc_col0, *tc_ncols, *tc_cbeg, *tc_cend, *tc_chunks;
  // batched factorisation order: CTA k factors problem fs_prob[k] (widest first)
  const int32_t *fs_prob;
  int32_t n_tc_items;
  int32_t max_P_small;    // widest problem the batched (shared-memory) factorisation takes
};

struct LMState {
  double lam, nu, cost, cost_cand, pred, cost0, cost_lin;
  int32_t iters, accepted, status, relin;
  int32_t fail;  // this iteration's step failed: bit 0 a non-positive pivot, bit 1 a bounded wait ran out
  int32_t flag, factor_failures;
  int32_t res_sel;  // which half of WorkView::res holds the residuals of the state (the other: the candidate's)
  // history and statistics the learned damping controller reads
  double rho1, rho2, rho3, last_rel, last_predrel;
  double gnorm, dmean, dmax, dmin, cmean;
  int32_t last_acc, rej_streak;
  int32_t wait_timeouts;  // steps rejected because a bounded device wait ran out
  int32_t ref_done;       // this step's refinement has converged (outer_tol): skip its further steps
  int32_t small_prev;     // the last accepted step lowered the cost by less than tol (relative)
  int32_t pad_;
};

constexpr int32_t FAIL_PIVOT = 1, FAIL_TIMEOUT = 2;

// per-iteration scratch (precision-dependent arrays typed at the kernel)
struct WorkView {
  // frame tables: [F][2 cams] rotation (cam->world) and centre
  float *fr_Rf;     // [F][2][9]
  float *fr_Rl;     // [F][2][9] float(R - float(R))
  double *fr_Rd;    // [F][2][9]
  double *fr_c;     // [F][2][3]
  float *fr_ch;     // [F][2][3] float(c)
  float *fr_cl;     // [F][2][3] float(c - float(c))
  double *poses_cand;   // [NP][12]
  double *alpha_cand;   // [L] (caller order)
  float *res;           // [2][O][4] residuals of the cost passes (FP32 path): u_l, v_l, u_r, v_r; half
                        // LMState::res_sel holds the state's, the other the last candidate's
  float *tcam;          // [2][O][6] the camera-frame points of the same cost passes (left, right),
                        // the double-float value rounded once; halves as res (mixed path)
  float *xanc;          // [2][L][8] per landmark (internal order), from the same cost passes: the
                        // anchor point's double-float value rounded to its high part (x, y, z),
                        // then d/d alpha of that rounded point (x, y, z), 2 pad; halves as res
                        // (mixed path)
  void *pair_acc;       // [total_pairs][27] T  (accumulated by the linearisation)
  void *pairF;          // [total_pairs][27] T  (prefix / suffix sums)
  void *A;              // [total_S] T      pose-pose blocks
  void *g;              // [total_params] T pose gradient
  void *SL;             // [total_S] T      landmark Schur term (lower tiles)
  void *gL;             // [total_params] T
  void *fac;            // [total_S] T   (global-memory factor for large problems)
  double *delta;        // [total_params]
  void *C;              // [L] T
  void *ga;             // [L] T
  void *slab;           // [sum slab] T
  LMState *lm;          // [B]
  LMState *lm_backup;   // [B] (lambda probes)
  double *probe_costs;  // [32][B]
  double *trace;        // [B][SPGO_TRACE_MAX][3]: cost after the iteration, lambda used, accepted
  void *ctrl;           // deployed controller weights (BF16-rounded, inference layout)
  // large reduced systems (k_chol_large.cu), allocated when the batch has any
  void *Sx;             // [total_S] exact S: (hi, lo) float pairs on the FP32 path, doubles on FP64
  double *lg_g0, *lg_x; // [total_params] g - g_L; the solution so far
  float *lg_xs;         // [2 total_params] its double-float split
  void *lg_y, *lg_dinv; // [total_params] T: right-hand side / residual; 1 / L_kk
  int *lg_flag;         // [2 total_params]: block-done flags of the multi-CTA substitutions
  double *lg_red;       // [NP + B][12] mixed path, wide problems: per pose the refinement's row and
                        // column sums of the pair duals ([N + 1][6] each), then the rows' prefix
  double *cost_acc;     // [B]
  double *pred_acc;     // [B]
  // iterative refinement of the mixed path's step (k_refine.cu); null on the FP64 path
  float *facs;          // [total_S] per problem: packed FP32 Cholesky factor, then 1 / L_kk
  float *twist;         // [total_pairs][6] sum over the pair's poses of Ad_i delta_i (about c_lo)
  double *pdual;        // [total_pairs][6] J^T W e per pose pair, about c_lo
  double *dal;          // [L] internal order: the inverse-depth step so far
  float *tl;            // [L] internal order: D^-1 r_a of the last residual pass
  double *gaacc;        // [L] internal order: exactly summed inverse-depth gradient (linearisation)
  double *gacc;         // [total_params] exactly summed pose gradient (linearisation)
  float *rhsB;          // [total_params] B D^-1 r_a of the last residual pass
  double *ddelta;       // [total_params] the last pose correction
};

struct Params {
  int32_t loss, near_boost;
  float loss_scale, eps, alpha_min, alpha_max;
  double lambda0, lambda_max, tol;
  int32_t max_iters, refine_steps;
  int32_t use_graph, use_tc;
  int32_t cost_block, lin_block;
  int32_t outer_steps, wait_us;
  float ctl_min_log10;
  float outer_tol;
  float stop_rho;
};

// bounded device-side waits: the limit in nanoseconds (wait_us = 0: 2 s)
__host__ __device__ inline unsigned long long wait_limit_ns(const Params &p) {
  return p.wait_us > 0 ? 1000ull * (unsigned long long)p.wait_us : 2000000000ull;
}

// launch wrappers (defined in the .cu files); all return cudaError_t as int
int launch_chain(const PlanView &pv, const WorkView &wv, const double *poses, int gate, int f64, void *stream);
template <typename T>
int launch_linearize(const PlanView &pv, const WorkView &wv, const Params &prm, const double *alpha,
                     int cost_only, int gate, void *stream);
template <typename T>
int launch_system(const PlanView &pv, const WorkView &wv, int gate, void *stream);
template <typename T>
int launch_schur(const PlanView &pv, const WorkView &wv, const Params &prm, void *stream);
size_t factor_packed_bytes(int P, size_t ts);  // shared memory of the batched factorisation
template <typename T>
int launch_factor_large(const PlanView &pv, const WorkView &wv, const Params &prm, int b, int P, int param_off,
                        int refine, void *stream, void *side = nullptr, void *ev_a = nullptr, void *ev_b = nullptr);
template <typename T>
int launch_factor_solve(const PlanView &pv, const WorkView &wv, const Params &prm, int mixed,
                        void *stream);
// iterative refinement of the mixed path's step (k_refine.cu)
int launch_pair_twists(const PlanView &pv, const WorkView &wv, void *stream);
int launch_resid_pass(const PlanView &pv, const WorkView &wv, const Params &prm, const double *alpha, int first,
                      void *stream);
int launch_resid_solve(const PlanView &pv, const WorkView &wv, const Params &prm, int first, void *stream);
int launch_resid_reduce_large(const PlanView &pv, const WorkView &wv, int b, int N, void *stream);
int launch_refine_large(const PlanView &pv, const WorkView &wv, const Params &prm, int b, int P, int param_off,
                        void *stream);
int launch_backsub_refined(const PlanView &pv, const WorkView &wv, const Params &prm, const double *alpha,
                           double *alpha_out, void *stream);
size_t resid_solve_smem(int max_P_small, int max_N);
template <typename T>
int launch_backsub(const PlanView &pv, const WorkView &wv, const Params &prm, const double *alpha,
                   double *alpha_out, int direct, void *stream);
template <typename T>
int launch_update_poses(const PlanView &pv, const WorkView &wv, const double *poses, double *poses_out,
                        double scale, int direct, void *stream, const double *gacc = nullptr);
int launch_decide(const PlanView &pv, const WorkView &wv, const Params &prm, void *stream);
int launch_commit(const PlanView &pv, const WorkView &wv, double *poses, double *alpha, void *stream);
int launch_post_linearize(const PlanView &pv, const WorkView &wv, void *stream);
int launch_reset(const PlanView &pv, const WorkView &wv, const Params &prm, double lam, void *stream);
template <typename T>
int launch_export_B_n(const PlanView &pv, const WorkView &wv, int problem, int n_chunks, double *B,
                      double *C, double *ga, void *stream);

int launch_lm_stats(const PlanView &pv, const WorkView &wv, int f64, void *stream);
int launch_controller(const PlanView &pv, const WorkView &wv, const Params &prm, const void *Wb, void *stream);
int launch_features(const PlanView &pv, const WorkView &wv, float *feat, void *stream);
int launch_mlp_deploy(const float *theta, void *dst, void *stream);
size_t mlp_deployed_bytes();
int launch_scale_lambda(const PlanView &pv, const WorkView &wv, double factor, void *stream);
int launch_take_probe(const PlanView &pv, const WorkView &wv, int j, void *stream);
int launch_schur_tc(const PlanView &pv, const WorkView &wv, const Params &prm, void *stream);
template <typename T>
int launch_export_S(const PlanView &pv, const WorkView &wv, int problem, double *S, double *gS, void *stream);
int launch_to_double(const void *src, int f64, double *dst, int64_t n, void *stream);

// count of kernel launches made by this library on the calling thread (a solver is
// driven by one thread at a time; several solvers may run on several threads)
extern thread_local int64_t g_launches;
// sets the message spgo_last_error returns (thread-local)
void set_last_error(const char *msg);

}  // namespace spgo
