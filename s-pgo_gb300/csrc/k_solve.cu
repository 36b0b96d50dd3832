// Reduced-camera-system factorisation and solve, inverse-depth back-substitution,
// the SE(3) update, and the per-problem LM bookkeeping.
//
// Replaces solve_torch_torch (src/Optimization/linear_solvers.cu:195-218: libtorch
// Cholesky, FP32, failure ignored), the B^T delta GEMV + compute_delta_a
// (src/Optimization/Solver_cuda.cu:739-753, :361-374) and updateEstimation
// (Solver_cuda.cu:497-553).
#include "kernels.cuh"

namespace spgo {

// storage of the factor: packed lower triangle, column-major (column j holds rows j..P-1)
struct PackedCol {
  int P;
  __device__ __forceinline__ size_t operator()(int i, int j) const {
    return (size_t)j * P - ((size_t)j * (j - 1)) / 2 + (size_t)(i - j);
  }
};
struct FullCol {
  int P;
  __device__ __forceinline__ size_t operator()(int i, int j) const { return (size_t)j * P + i; }
};

// Right-looking Cholesky S = L L^T of one problem by one CTA, then L L^T x = g_S,
// then `refine` FP64 iterative-refinement steps r = g_S - S x, x += solve(r)
// (used when T = float).  Matrix in shared memory (packed) when it fits, else
// in the global scratch `fac` (full, column-major).
template <typename T, typename Idx>
__device__ void factor_solve_body(T *Lm, Idx ix, T *y, double *x, const double *S, const double *gS, int P,
                                  int refine, int *fail_s) {
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
  for (int j = tid; j < P; j += nt)
    for (int i = j; i < P; ++i) Lm[ix(i, j)] = (T)S[(size_t)i * P + j];
  if (tid == 0) *fail_s = 0;
  __syncthreads();
  for (int k = 0; k < P; ++k) {
    if (tid == 0) {
      const T d = Lm[ix(k, k)];
      if (!(d > T(0)) || !isfinite((double)d)) *fail_s = 1;
      else Lm[ix(k, k)] = sqrt(d);
    }
    __syncthreads();
    if (*fail_s) return;
    const T inv = T(1) / Lm[ix(k, k)];
    for (int i = k + 1 + tid; i < P; i += nt) Lm[ix(i, k)] *= inv;
    __syncthreads();
    for (int j = k + 1 + warp; j < P; j += nw) {
      const T ljk = Lm[ix(j, k)];
      for (int i = j + lane; i < P; i += 32) Lm[ix(i, j)] -= Lm[ix(i, k)] * ljk;
    }
    __syncthreads();
  }
  for (int i = tid; i < P; i += nt) {
    y[i] = (T)gS[i];
    x[i] = 0.0;
  }
  __syncthreads();
  for (int it = 0; it <= refine; ++it) {
    // forward L z = y
    for (int k = 0; k < P; ++k) {
      if (tid == 0) y[k] = y[k] / Lm[ix(k, k)];
      __syncthreads();
      const T yk = y[k];
      for (int i = k + 1 + tid; i < P; i += nt) y[i] -= Lm[ix(i, k)] * yk;
      __syncthreads();
    }
    // backward L^T w = z
    for (int k = P - 1; k >= 0; --k) {
      if (tid == 0) y[k] = y[k] / Lm[ix(k, k)];
      __syncthreads();
      const T yk = y[k];
      for (int i = tid; i < k; i += nt) y[i] -= Lm[ix(k, i)] * yk;
      __syncthreads();
    }
    for (int i = tid; i < P; i += nt) x[i] += (double)y[i];
    __syncthreads();
    if (it == refine) break;
    // FP64 residual r = g_S - S x
    for (int i = warp; i < P; i += nw) {
      double acc = 0.0;
      for (int j = lane; j < P; j += 32) acc += S[(size_t)i * P + j] * x[j];
      acc = warp_sum(acc);
      if (lane == 0) y[i] = (T)(gS[i] - acc);
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(512) k_factor_solve(PlanView pv, WorkView wv, int refine, int use_smem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int fail_s;
  const int b = blockIdx.x;
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  const int N = pv.p_npose[b], P = 6 * N;
  const size_t off = pv.p_S_off[b];
  const int po = pv.p_param_off[b];
  const double *S = wv.S + off;
  const double *gS = wv.gS + po;
  double *x;
  T *y;
  if (use_smem) {
    const size_t npk = (size_t)P * (P + 1) / 2;
    T *Lm = reinterpret_cast<T *>(smem_raw);
    x = reinterpret_cast<double *>(smem_raw + ((npk * sizeof(T) + 15) & ~(size_t)15));
    y = reinterpret_cast<T *>(x + P);
    factor_solve_body<T, PackedCol>(Lm, PackedCol{P}, y, x, S, gS, P, refine, &fail_s);
  } else {
    x = reinterpret_cast<double *>(smem_raw);
    y = reinterpret_cast<T *>(x + P);
    T *Lm = reinterpret_cast<T *>(wv.fac) + off;
    factor_solve_body<T, FullCol>(Lm, FullCol{P}, y, x, S, gS, P, refine, &fail_s);
  }
  __syncthreads();
  const bool failed = fail_s != 0;
  for (int i = threadIdx.x; i < P; i += blockDim.x) wv.delta[po + i] = failed ? 0.0 : x[i];
  if (threadIdx.x == 0 && failed) wv.lm[b].fail = 1;
}

static const size_t kSmemBudget = 200 * 1024;

template <typename T>
int launch_factor_solve(const PlanView &pv, const WorkView &wv, const Params &prm, int mixed, void *stream) {
  const int P = pv.max_P;
  const size_t vec = (size_t)P * (sizeof(double) + sizeof(T)) + 16;
  const size_t packed = (((size_t)P * (P + 1) / 2) * sizeof(T) + 15) / 16 * 16 + vec;
  const int use_smem = packed <= kSmemBudget;
  const size_t sm = use_smem ? packed : vec;
  const int refine = mixed ? prm.refine_steps : 0;
  cudaFuncSetAttribute(k_factor_solve<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_factor_solve<T><<<pv.B, 512, sm, (cudaStream_t)stream>>>(pv, wv, refine, use_smem);
  ++g_launches;
  return (int)cudaGetLastError();
}

// ---- inverse-depth back-substitution: da = (g_a - B^T delta) / (C (1 + lam) + eps) ----
// one warp per chunk, lane = landmark slot; reads the slab column and delta.
template <typename T>
__global__ void k_backsub(PlanView pv, WorkView wv, Params prm, const double *alpha, double *alpha_out,
                          int gate) {
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int slot = threadIdx.x & 31;
  if (c >= pv.n_chunks) return;
  const int b = pv.ch_prob[c];
  if (!problem_active(wv.lm, b, gate)) return;
  const int f0 = pv.ch_f0[c], nb = pv.ch_nb[c], lm0 = pv.ch_lm0[c], cnt = pv.ch_cnt[c];
  const int po = pv.p_param_off[b];
  const T *slab = reinterpret_cast<const T *>(wv.slab) + pv.ch_slab[c];
  double pred = 0.0;
  if (slot < cnt) {
    const int li = lm0 + slot;
    const double *dl = wv.delta + po + 6 * f0;
    double s = 0.0;
    for (int r = 0; r < 6 * nb; ++r) s += (double)slab[(size_t)r * SPGO_CHUNK + slot] * dl[r];
    const double C = (double)reinterpret_cast<const T *>(wv.C)[li];
    const double ga = (double)reinterpret_cast<const T *>(wv.ga)[li];
    const double lam = wv.lm[b].lam;
    const double Dd = C * (1.0 + lam) + (double)prm.eps;
    const double da = (ga - s) / Dd;
    pred = da * (ga + (Dd - C) * da);
    const int u = pv.lm_user[li];
    const double an = alpha[u] + da;
    alpha_out[u] = fmin(fmax(an, (double)prm.alpha_min), (double)prm.alpha_max);
  }
  pred = warp_sum(pred);
  if (slot == 0 && pred != 0.0) atomicAdd(wv.pred_acc + b, pred);
}

template <typename T>
int launch_backsub(const PlanView &pv, const WorkView &wv, const Params &prm, const double *alpha,
                   double *alpha_out, int direct, void *stream) {
  if (pv.n_chunks == 0) return 0;
  const int gate = direct ? GATE_ALL : GATE_RUNNING;
  k_backsub<T><<<grid_for(pv.n_chunks, 4), 128, 0, (cudaStream_t)stream>>>(pv, wv, prm, alpha, alpha_out, gate);
  ++g_launches;
  return (int)cudaGetLastError();
}

// ---- T_k <- T_k Exp(scale * delta_k) in FP64; pred += delta^T (g + lam diag(A) delta) ----
__global__ void k_update_poses(PlanView pv, WorkView wv, const double *poses, double *out, double scale,
                               int gate) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= pv.NP) return;
  const int b = pv.pose_prob[p];
  if (!problem_active(wv.lm, b, gate)) return;
  const int k = p - pv.p_pose_off[b];
  const int P = 6 * pv.p_npose[b];
  const int po = pv.p_param_off[b] + 6 * k;
  double xi[6];
#pragma unroll
  for (int q = 0; q < 6; ++q) xi[q] = scale * wv.delta[po + q];
  double E[12], Tn[12];
  exp_se3(xi, E);
  compose34(poses + 12 * (size_t)p, E, Tn);
#pragma unroll
  for (int q = 0; q < 12; ++q) out[12 * (size_t)p + q] = Tn[q];
  const double lam = wv.lm[b].lam;
  const double *A = wv.A + pv.p_S_off[b];
  double pred = 0.0;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const double d = wv.delta[po + q];
    const double akk = A[(size_t)(6 * k + q) * P + 6 * k + q];
    pred += d * (wv.g[po + q] + lam * akk * d);
  }
  atomicAdd(wv.pred_acc + b, pred);
}

int launch_update_poses(const PlanView &pv, const WorkView &wv, const double *poses, double *poses_out,
                        double scale, int direct, void *stream) {
  k_update_poses<<<grid_for(pv.NP, 128), 128, 0, (cudaStream_t)stream>>>(pv, wv, poses, poses_out, scale,
                                                                       direct ? GATE_ALL : GATE_RUNNING);
  ++g_launches;
  return (int)cudaGetLastError();
}

// ---- per-problem LM bookkeeping (thread per problem) ---------------------------
__global__ void k_reset(PlanView pv, WorkView wv, double lam) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= pv.B) return;
  LMState s;
  s.lam = lam;
  s.nu = 2.0;
  s.cost = s.cost_cand = s.pred = s.cost0 = s.cost_lin = 0.0;
  s.iters = s.accepted = s.status = 0;
  s.relin = 1;
  s.fail = s.flag = s.factor_failures = s.pad = 0;
  wv.lm[b] = s;
  wv.cost_acc[b] = 0.0;
  wv.pred_acc[b] = 0.0;
}

int launch_reset(const PlanView &pv, const WorkView &wv, const Params &prm, double lam, void *stream) {
  (void)prm;
  k_reset<<<grid_for(pv.B, 128), 128, 0, (cudaStream_t)stream>>>(pv, wv, lam);
  ++g_launches;
  return (int)cudaGetLastError();
}

// after a linearisation: the cost at the linearisation point becomes the current cost
__global__ void k_post_linearize(PlanView pv, WorkView wv) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= pv.B) return;
  LMState &s = wv.lm[b];
  if (s.status != 0 || !s.relin) return;
  const double c = wv.cost_acc[b];
  s.cost_lin = c;
  s.cost = c;
  if (s.iters == 0) s.cost0 = c;
  s.relin = 0;
  wv.cost_acc[b] = 0.0;
}

int launch_post_linearize(const PlanView &pv, const WorkView &wv, void *stream) {
  k_post_linearize<<<grid_for(pv.B, 128), 128, 0, (cudaStream_t)stream>>>(pv, wv);
  ++g_launches;
  return (int)cudaGetLastError();
}

// Nielsen schedule: rho = (F - F') / pred, pred = 0.5 d^T (g + Lambda d).
// accept (rho > 0): lam *= max(1/3, 1 - (2 rho - 1)^3), nu = 2; else lam *= nu, nu *= 2.
__global__ void k_decide(PlanView pv, WorkView wv, Params prm) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= pv.B) return;
  LMState &s = wv.lm[b];
  if (s.status != 0) {
    s.flag = 0;
    return;
  }
  const double F = s.cost;
  const double Fn = wv.cost_acc[b];
  const double pred = 0.5 * wv.pred_acc[b];
  wv.cost_acc[b] = 0.0;
  wv.pred_acc[b] = 0.0;
  s.cost_cand = Fn;
  s.pred = pred;
  s.iters += 1;
  const bool ok = !s.fail && isfinite(Fn) && pred > 0.0 && Fn < F;
  if (ok) {
    const double rho = (F - Fn) / pred;
    const double rel = (F - Fn) / fmax(F, 1e-300);
    s.accepted += 1;
    s.flag = 1;
    s.cost = Fn;
    const double t = 2.0 * rho - 1.0;
    s.lam *= fmax(1.0 / 3.0, 1.0 - t * t * t);
    s.nu = 2.0;
    s.relin = 1;
    if (rel < prm.tol) s.status = SPGO_STATUS_CONVERGED;
  } else {
    if (s.fail) s.factor_failures += 1;
    s.flag = 0;
    s.relin = 0;
    s.lam *= s.nu;
    s.nu *= 2.0;
    if (s.lam > prm.lambda_max) s.status = SPGO_STATUS_STALLED;
  }
  s.fail = 0;
  if (s.status == 0 && s.iters >= prm.max_iters) s.status = SPGO_STATUS_MAX_ITERS;
}

int launch_decide(const PlanView &pv, const WorkView &wv, const Params &prm, void *stream) {
  k_decide<<<grid_for(pv.B, 128), 128, 0, (cudaStream_t)stream>>>(pv, wv, prm);
  ++g_launches;
  return (int)cudaGetLastError();
}

// accepted candidates become the state
__global__ void k_commit(PlanView pv, WorkView wv, double *poses, double *alpha) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < pv.NP) {
    const int b = pv.pose_prob[t];
    if (wv.lm[b].flag) {
#pragma unroll
      for (int q = 0; q < 12; ++q) poses[12 * t + q] = wv.poses_cand[12 * t + q];
    }
  }
  if (t < pv.L) {
    const int b = pv.lm_prob[t];
    if (wv.lm[b].flag) {
      const int u = pv.lm_user[t];
      alpha[u] = wv.alpha_cand[u];
    }
  }
}

int launch_commit(const PlanView &pv, const WorkView &wv, double *poses, double *alpha, void *stream) {
  const long long n = pv.NP > pv.L ? pv.NP : pv.L;
  k_commit<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(pv, wv, poses, alpha);
  ++g_launches;
  return (int)cudaGetLastError();
}

// dense B (P x L, row-major, problem-local landmark order), C and g_a of one problem
template <typename T>
__global__ void k_export_B(PlanView pv, WorkView wv, int b, double *B, double *C, double *ga) {
  const int c = pv.p_chunk_off[b] + blockIdx.x;
  const int N = pv.p_npose[b];
  const int Lb = pv.p_lm_cnt[b], lo = pv.p_lm_off[b];
  const int f0 = pv.ch_f0[c], nb = pv.ch_nb[c], lm0 = pv.ch_lm0[c], cnt = pv.ch_cnt[c];
  const T *slab = reinterpret_cast<const T *>(wv.slab) + pv.ch_slab[c];
  (void)N;
  for (int idx = threadIdx.x; idx < 6 * nb * SPGO_CHUNK; idx += blockDim.x) {
    const int r = idx / SPGO_CHUNK, slot = idx % SPGO_CHUNK;
    if (slot >= cnt) continue;
    const int ul = pv.lm_user[lm0 + slot] - lo;
    if (B) B[(size_t)(6 * f0 + r) * Lb + ul] = (double)slab[idx];
  }
  for (int slot = threadIdx.x; slot < cnt; slot += blockDim.x) {
    const int ul = pv.lm_user[lm0 + slot] - lo;
    if (C) C[ul] = (double)reinterpret_cast<const T *>(wv.C)[lm0 + slot];
    if (ga) ga[ul] = (double)reinterpret_cast<const T *>(wv.ga)[lm0 + slot];
  }
}

template <typename T>
int launch_export_B_n(const PlanView &pv, const WorkView &wv, int problem, int n_chunks, double *B, double *C,
                      double *ga, void *stream) {
  if (n_chunks == 0) return 0;
  k_export_B<T><<<n_chunks, 256, 0, (cudaStream_t)stream>>>(pv, wv, problem, B, C, ga);
  ++g_launches;
  return (int)cudaGetLastError();
}

template int launch_factor_solve<float>(const PlanView &, const WorkView &, const Params &, int, void *);
template int launch_factor_solve<double>(const PlanView &, const WorkView &, const Params &, int, void *);
template int launch_backsub<float>(const PlanView &, const WorkView &, const Params &, const double *, double *, int, void *);
template int launch_backsub<double>(const PlanView &, const WorkView &, const Params &, const double *, double *, int, void *);
template int launch_export_B_n<float>(const PlanView &, const WorkView &, int, int, double *, double *, double *, void *);
template int launch_export_B_n<double>(const PlanView &, const WorkView &, int, int, double *, double *, double *, void *);

}  // namespace spgo
