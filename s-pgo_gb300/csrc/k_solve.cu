// Reduced-camera-system factorisation and solve, inverse-depth back-substitution,
// the SE(3) update, and the per-problem LM bookkeeping.
//
// Replaces solve_torch_torch (src/Optimization/linear_solvers.cu:195-218: libtorch
// Cholesky, FP32, failure ignored), the B^T delta GEMV + compute_delta_a
// (src/Optimization/Solver_cuda.cu:739-753, :361-374) and updateEstimation
// (Solver_cuda.cu:497-553).
#include "kernels.cuh"
#include "dfloat.cuh"
#include "chol_subst.cuh"

#include <type_traits>

namespace spgo {

// Storage of the factor: element (i, j), i >= j, at Lm[cb[j] + i] with per-column
// base offsets cb in shared memory: packed lower triangle, column-major (column j
// holds rows j..P-1; cb[j] = j P - j (j + 1) / 2).  The block width kPanel and the
// substitutions are in chol_subst.cuh.
constexpr int kRowRegs = 8; // row entries per lane held in registers by the assembly and residual (P <= 256)

// S(r, c) of the damped reduced system for r >= c, from A (pose blocks), S_L
// (landmark Schur term, lower tiles) and lambda:  S = A + lam diag(A) - S_L
// (in T: the FP32 difference A - S_L is the correctly rounded exact difference,
// the same value an FP64 evaluation rounded to FP32 would give off the diagonal)
template <typename T>
__device__ __forceinline__ T s_entry(const T *A, const T *SL, int P, int r, int c, T lam) {
  const size_t k = (size_t)r * P + c;
  T v = A[k] - SL[k];
  if (r == c) v += lam * A[k];
  return v;
}

// One CTA per problem: assemble S (lower) into the factor storage, then a
// right-looking blocked Cholesky S = L L^T with 16-column blocks: warp 0
// factorises the 16x16 diagonal block, all threads solve the rows below it
// (independent per row) and apply the rank-16 trailing update, the next block's
// columns first, so that warp 0 factorises the next diagonal block while the other
// warps update the rest (one block of look-ahead); three barriers per block.  The substitutions are blocked the same way (two barriers per
// block).  `refine` iterative-refinement steps form the residual g_S - S x
// (double-float on the FP32 path, FP64 otherwise) from A and S_L in one
// coalesced pass over the lower triangle.  Clears the S_L / g_L tiles it consumed.
template <typename T>
__device__ void factor_solve_body(T *Lm, const int *cb, T *y, double *x, float *xs, T *dinv, T *tmp, T *colacc,
                                  const T *A, T *SL, const T *g, T *gL, double lam, int P, int refine,
                                  int *fail_s) {
#define ix(i, j) (cb[(j)] + (i))
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
  const T lam_t = (T)lam;
  // assembly: rows over warps, columns over lanes (coalesced reads of A and S_L);
  // each warp loads kAsmRows rows (up to kRowRegs columns per lane) before it stores
  // any, so a warp waits for one memory round trip per kAsmRows rows
  if (P <= 32 * kRowRegs) {
    constexpr int kAsmRows = sizeof(T) == 4 ? 4 : 2;
    for (int r0 = warp; r0 < P; r0 += kAsmRows * nw) {
      T av[kAsmRows][kRowRegs], sv[kAsmRows][kRowRegs];
#pragma unroll
      for (int q = 0; q < kAsmRows; ++q) {
        const int r = r0 + q * nw;
        const T *Ar = A + (size_t)r * P, *Sr = SL + (size_t)r * P;
#pragma unroll
        for (int m = 0; m < kRowRegs; ++m) {
          const int c = lane + 32 * m;
          const bool ok = r < P && c <= r;
          av[q][m] = ok ? Ar[c] : T(0);
          sv[q][m] = ok ? Sr[c] : T(0);
        }
      }
#pragma unroll
      for (int q = 0; q < kAsmRows; ++q) {
        const int r = r0 + q * nw;
#pragma unroll
        for (int m = 0; m < kRowRegs; ++m) {
          const int c = lane + 32 * m;
          if (r < P && c <= r) Lm[ix(r, c)] = av[q][m] - sv[q][m] + (c == r ? lam_t * av[q][m] : T(0));
        }
      }
    }
  } else {
    for (int r = warp; r < P; r += nw)
      for (int c = lane; c <= r; c += 32) Lm[ix(r, c)] = s_entry(A, SL, P, r, c, lam_t);
  }
  for (int i = tid; i < P; i += nt) {
    y[i] = g[i] - gL[i];
    x[i] = 0.0;
  }
  if (tid == 0) *fail_s = 0;
  __syncthreads();
  // warp 0: the diagonal block [kb, kb + kPanel) in registers; lane i < w holds row i
  // (a[j] = L(kb+i, kb+j), j <= i); column k is finished with one shuffle of the pivot
  // and one per later row
  auto factor_diag = [&](int kb) {
    const int w = min(kb + kPanel, P) - kb;
    T a[kPanel];
#pragma unroll
    for (int j = 0; j < kPanel; ++j) a[j] = (lane < w && j <= lane) ? Lm[ix(kb + lane, kb + j)] : T(0);
    bool bad = false;
    // (columns k >= w of a narrow last block run on a unit pivot and are discarded)
#pragma unroll
    for (int k = 0; k < kPanel; ++k) {
      const T dk = __shfl_sync(0xffffffffu, a[k], k);
      const T d = k < w ? dk : T(1);
      bad = bad || !(d > T(0)) || !(d < T(INFINITY));  // (no FP64 conversion on the pivot chain)
      const T lkk = sqrt(d), rinv = T(1) / lkk;  // correctly rounded: the refinement step relies on it
      const T lik = lane > k ? a[k] * rinv : (lane == k ? lkk : a[k]);
      a[k] = lik;
#pragma unroll
      for (int j = 0; j < kPanel; ++j) {
        const T ljk = __shfl_sync(0xffffffffu, lik, j);
        if (j > k && lane >= j) a[j] -= lik * ljk;
      }
      if (lane == 0 && k < w) dinv[kb + k] = rinv;
    }
#pragma unroll
    for (int j = 0; j < kPanel; ++j)
      if (lane < w && j <= lane) Lm[ix(kb + lane, kb + j)] = a[j];
    if (bad && lane == 0) *fail_s = 1;
  };
  // the update of columns [c0, c1) (rows i >= j) with the finished block kb: warp wi of
  // nwu, KC columns per warp pass (each loaded panel row serves KC columns)
  auto update_cols = [&](auto kc_tag, const int (&cbk)[kPanel], int w, int c0, int c1, int wi, int nwu) {
    constexpr int KC = decltype(kc_tag)::value;
    for (int j0 = c0 + KC * wi; j0 < c1; j0 += KC * nwu) {
      T ljk[KC][kPanel];
#pragma unroll
      for (int c = 0; c < KC; ++c)
#pragma unroll
        for (int k = 0; k < kPanel; ++k) ljk[c][k] = (k < w && j0 + c < c1) ? Lm[cbk[k] + j0 + c] : T(0);
      for (int i = j0 + lane; i < P; i += 32) {
        T li[kPanel];
#pragma unroll
        for (int k = 0; k < kPanel; ++k) li[k] = Lm[cbk[k] + i];
#pragma unroll
        for (int c = 0; c < KC; ++c) {
          if (j0 + c < c1 && i >= j0 + c) {
            T a0 = T(0), a1 = T(0);  // two half-length FMA chains per output
#pragma unroll
            for (int k = 0; k < kPanel; k += 2) {
              a0 += li[k] * ljk[c][k];
              a1 += li[k + 1] * ljk[c][k + 1];
            }
            Lm[cb[j0 + c] + i] -= a0 + a1;
          }
        }
      }
    }
  };
  // right-looking with one block of look-ahead: once block kb's rows are solved, the
  // next block's columns take its update first; then warp 0 factors the next diagonal
  // block while the other warps update the remaining columns.  Every element takes
  // the same updates in the same order as without the look-ahead.
  if (warp == 0) factor_diag(0);
  __syncthreads();
  if (*fail_s) return;
  for (int kb = 0; kb < P; kb += kPanel) {
    const int ke = min(kb + kPanel, P), w = ke - kb;
    // rows below the block: L(i, kb:ke) = S(i, kb:ke) L_D^-T
    int cbk[kPanel];
#pragma unroll
    for (int c = 0; c < kPanel; ++c) cbk[c] = c < w ? cb[kb + c] : 0;
    for (int i = ke + tid; i < P; i += nt) {
      T r[kPanel];
#pragma unroll
      for (int c = 0; c < kPanel; ++c) r[c] = c < w ? Lm[cbk[c] + i] : T(0);
#pragma unroll
      for (int c = 0; c < kPanel; ++c) {
        if (c < w) {
          T v = r[c];
#pragma unroll
          for (int m = 0; m < c; ++m) v -= r[m] * Lm[ix(kb + c, kb + m)];
          r[c] = v * dinv[kb + c];
        }
      }
#pragma unroll
      for (int c = 0; c < kPanel; ++c)
        if (c < w) Lm[cbk[c] + i] = r[c];
    }
    __syncthreads();
    if (ke >= P) break;
    const int ke2 = min(ke + kPanel, P);
    update_cols(std::integral_constant<int, 2>{}, cbk, w, ke, ke2, warp, nw);  // the next block's columns
    __syncthreads();
    // (4 columns per pass in FP32, 2 in FP64 to bound registers)
    if (warp == 0)
      factor_diag(ke);
    else
      update_cols(std::integral_constant<int, sizeof(T) == 8 ? 2 : 4>{}, cbk, w, ke2, P, warp - 1, nw - 1);
    __syncthreads();
    if (*fail_s) return;
  }
  for (int it = 0; it <= refine; ++it) {
    chol_substitute<T>(Lm, cb, y, dinv, tmp, P);
    for (int i = tid; i < P; i += nt) x[i] += (double)y[i];
    __syncthreads();
    if (it == refine) break;
    // residual r = g_S - S x with ~48-bit accuracy: FP64 when T = double, else
    // double-float sums on the FP32 pipes (S entries are exact in float)
    if constexpr (std::is_same<T, float>::value) {
      for (int j = tid; j < P; j += nt) {
        const df xj = df_from_double(x[j]);
        xs[2 * j] = xj.h;
        xs[2 * j + 1] = xj.l;
      }
      __syncthreads();
    }
    // one coalesced pass over the lower triangle, row i per warp, column j per
    // lane: S_ij x_j feeds row i's sum (warp reduction) and S_ij x_i feeds
    // column j's sum, kept per warp in shared memory and added up at the end.
    // Layout: colacc[w][2 P] (float path: h, l pairs; FP64 path: P doubles),
    // then the row sums [2 P].
    T *rowp = colacc + (size_t)nw * 2 * P;
    for (int k = tid; k < (nw + 1) * 2 * P; k += nt) colacc[k] = T(0);
    __syncthreads();
    T *mine = colacc + (size_t)warp * 2 * P;
    // (the FP32 path takes two rows per warp pass: both rows' entries are loaded
    // before either is used, so a warp waits for one round trip per two rows)
    constexpr int kResRows = std::is_same<T, float>::value ? 2 : 1;
    for (int i0 = warp; i0 < P; i0 += kResRows * nw) {
      if constexpr (std::is_same<T, float>::value) {
        float av[kResRows][kRowRegs], sv[kResRows][kRowRegs];
        const bool regs = P <= 32 * kRowRegs;
        if (regs) {
#pragma unroll
          for (int q = 0; q < kResRows; ++q) {
            const int i = i0 + q * nw;
            const float *Ai = A + (size_t)i * P, *Si = SL + (size_t)i * P;
#pragma unroll
            for (int m = 0; m < kRowRegs; ++m) {
              const int j = lane + 32 * m;
              const bool ok = i < P && j <= i;
              av[q][m] = ok ? Ai[j] : 0.f;
              sv[q][m] = ok ? Si[j] : 0.f;
            }
          }
        }
#pragma unroll
        for (int q = 0; q < kResRows; ++q) {
          const int i = i0 + q * nw;
          if (i >= P) break;
          const float *Ai = A + (size_t)i * P, *Si = SL + (size_t)i * P;
          const df xi{xs[2 * i], xs[2 * i + 1]};
          df acc = df_make(0.f);
          auto term = [&](int j, float a, float sl) {
            df sij = df_sub(a, sl);
            if (j == i) sij = sij + df_from_double(lam * (double)a);
            acc = acc + sij * df{xs[2 * j], xs[2 * j + 1]};
            if (j < i) {
              const df c = df{mine[2 * j], mine[2 * j + 1]} + sij * xi;
              mine[2 * j] = c.h;
              mine[2 * j + 1] = c.l;
            }
          };
          if (regs) {
#pragma unroll
            for (int m = 0; m < kRowRegs; ++m)
              if (lane + 32 * m <= i) term(lane + 32 * m, av[q][m], sv[q][m]);
          } else {
            for (int j = lane; j <= i; j += 32) term(j, Ai[j], Si[j]);
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            const df other{__shfl_xor_sync(0xffffffffu, acc.h, o), __shfl_xor_sync(0xffffffffu, acc.l, o)};
            acc = acc + other;
          }
          if (lane == 0) {
            rowp[2 * i] = acc.h;
            rowp[2 * i + 1] = acc.l;
          }
        }
      } else {
        const int i = i0;
        const T *Ai = A + (size_t)i * P, *Si = SL + (size_t)i * P;
        const double xi = x[i];
        double acc = 0.0;
        for (int j = lane; j <= i; j += 32) {
          double sij = (double)Ai[j] - (double)Si[j];
          if (j == i) sij += lam * (double)Ai[j];
          acc += sij * x[j];
          if (j < i) mine[j] += sij * xi;
        }
        acc = warp_sum(acc);
        if (lane == 0) rowp[i] = acc;
      }
    }
    __syncthreads();
    for (int i = tid; i < P; i += nt) {
      double sx;
      if constexpr (std::is_same<T, float>::value) {
        df t{rowp[2 * i], rowp[2 * i + 1]};
        for (int w = 0; w < nw; ++w) t = t + df{colacc[(size_t)w * 2 * P + 2 * i], colacc[(size_t)w * 2 * P + 2 * i + 1]};
        sx = (double)t.h + (double)t.l;
      } else {
        sx = rowp[i];
        for (int w = 0; w < nw; ++w) sx += colacc[(size_t)w * 2 * P + i];
      }
      y[i] = (T)((double)g[i] - (double)gL[i] - sx);
    }
    __syncthreads();
  }
}

#undef ix

// store: keep the packed factor and the pivots in wv.facs for the refinement solves
template <typename T>
__global__ void __launch_bounds__(256) k_factor_solve(PlanView pv, WorkView wv, int refine, int store) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int fail_s;
  __shared__ T tmp_s[kPanel];
  const int b = pv.fs_prob[blockIdx.x];
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  const int N = pv.p_npose[b], P = 6 * N;
  if (P > pv.max_P_small) return;  // a large system: k_chol_large.cu
  const size_t off = pv.p_S_off[b];
  const int po = pv.p_param_off[b];
  const T *A = reinterpret_cast<const T *>(wv.A) + off;
  T *SL = reinterpret_cast<T *>(wv.SL) + off;
  const T *g = reinterpret_cast<const T *>(wv.g) + po;
  T *gL = reinterpret_cast<T *>(wv.gL) + po;
  const double lam = wv.lm[b].lam;
  double *x;
  T *y;
  const size_t npk = (size_t)P * (P + 1) / 2;
  T *Lm = reinterpret_cast<T *>(smem_raw);
  x = reinterpret_cast<double *>(smem_raw + ((npk * sizeof(T) + 15) & ~(size_t)15));
  y = reinterpret_cast<T *>(x + P);
  float *xs = reinterpret_cast<float *>(y + P);
  int *cb = reinterpret_cast<int *>(xs + 2 * P);
  T *dinv = reinterpret_cast<T *>(smem_raw + ((npk * sizeof(T) + 15) & ~(size_t)15) +
                                  (((size_t)P * (sizeof(double) + sizeof(T) + 2 * sizeof(float) + sizeof(int)) + 15) &
                                   ~(size_t)15));
  T *colacc = reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(dinv) + (((size_t)P * sizeof(T) + 15) & ~(size_t)15));
  for (int j = threadIdx.x; j < P; j += blockDim.x) cb[j] = j * P - (j * (j + 1)) / 2;
  __syncthreads();
  factor_solve_body<T>(Lm, cb, y, x, xs, dinv, tmp_s, colacc, A, SL, g, gL, lam, P, refine, &fail_s);
  __syncthreads();
  const bool failed = fail_s != 0;
  for (int i = threadIdx.x; i < P; i += blockDim.x) wv.delta[po + i] = failed ? 0.0 : x[i];
  if (threadIdx.x == 0) wv.lm[b].ref_done = 0;  // this step's refinement starts afresh
  if (threadIdx.x == 0 && failed) atomicOr(&wv.lm[b].fail, FAIL_PIVOT);
  if constexpr (std::is_same<T, float>::value) {
    if (store && !failed) {  // packed factor, then the pivots' reciprocals
      float *dst = wv.facs + off;
      for (size_t k = threadIdx.x; k < npk; k += blockDim.x) dst[k] = Lm[k];
      for (int k = threadIdx.x; k < P; k += blockDim.x) dst[npk + k] = dinv[k];
    }
  }
  // clear the consumed S_L tiles (every element whose row tile >= column tile) and g_L
  constexpr int TR = 6 * SPGO_TILE_BLOCKS;
  for (int r = threadIdx.x >> 5; r < P; r += blockDim.x >> 5) {
    const int cmax = min(P, (r / TR + 1) * TR);
    for (int c = threadIdx.x & 31; c < cmax; c += 32) SL[(size_t)r * P + c] = T(0);
  }
  for (int i = threadIdx.x; i < P; i += blockDim.x) gL[i] = T(0);
}

// dynamic shared memory of k_factor_solve for a P-wide problem: the packed factor,
// the vectors, the pivots and the residual's column sums
size_t factor_packed_bytes(int P, size_t ts) {
  const size_t vec = (size_t)P * (sizeof(double) + ts + 2 * sizeof(float) + sizeof(int)) + 16 + (size_t)P * ts + 16;
  const size_t colacc = (size_t)(256 / 32 + 1) * 2 * P * ts;
  return (((size_t)P * (P + 1) / 2) * ts + 15) / 16 * 16 + vec + colacc + 16;
}

template <typename T>
int launch_factor_solve(const PlanView &pv, const WorkView &wv, const Params &prm, int mixed, void *stream) {
  if (pv.max_P_small <= 0) return 0;
  const size_t sm = factor_packed_bytes(pv.max_P_small, sizeof(T));
  const int store = (mixed && prm.outer_steps > 0 && wv.facs) ? 1 : 0;
  // the reduced solve's own refinement only without the refinement of the whole step,
  // which supersedes it (its residual is exact, not that of the assembled S)
  const int refine = (mixed && !store) ? prm.refine_steps : 0;
  cudaFuncSetAttribute(k_factor_solve<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_factor_solve<T><<<pv.B, 256, sm, (cudaStream_t)stream>>>(pv, wv, refine, store);
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
  // B_l^T delta over the chunk's rows: delta comes in 32 rows at a time (one
  // coalesced load, then shuffles), four independent accumulators
  const double *dl = wv.delta + po + 6 * f0;
  const int rows = 6 * nb;
  T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
  for (int rb = 0; rb < rows; rb += 32) {
    const T dv = rb + slot < rows ? (T)dl[rb + slot] : T(0);
    const T *sr = slab + (size_t)rb * SPGO_CHUNK + slot;
    const int nr = min(32, rows - rb);
    T v[32];  // the block's 32 slab rows loaded before any is used
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = k < nr ? sr[(size_t)k * SPGO_CHUNK] : T(0);
#pragma unroll
    for (int k = 0; k < 32; k += 4) {
      s0 += v[k] * __shfl_sync(0xffffffffu, dv, k);
      s1 += v[k + 1] * __shfl_sync(0xffffffffu, dv, k + 1);
      s2 += v[k + 2] * __shfl_sync(0xffffffffu, dv, k + 2);
      s3 += v[k + 3] * __shfl_sync(0xffffffffu, dv, k + 3);
    }
  }
  if (slot < cnt) {
    const int li = lm0 + slot;
    const T s = (s0 + s1) + (s2 + s3);
    const T C = reinterpret_cast<const T *>(wv.C)[li];
    const T ga = reinterpret_cast<const T *>(wv.ga)[li];
    const double lam = wv.lm[b].lam;
    // the per-landmark update in T (its inputs are T already); the state update in FP64
    const T Dd = C * (T)(1.0 + lam) + (T)prm.eps;
    const T da = (ga - s) / Dd;
    pred = (double)(da * (ga + (Dd - C) * da));
    const int u = pv.lm_user[li];
    const double an = alpha[u] + (double)da;
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
// gacc: the accurate pose gradient of the refined step (else g of the linearisation)
template <typename T>
__global__ void k_update_poses(PlanView pv, WorkView wv, const double *poses, double *out, double scale,
                               int gate, const double *gacc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= pv.NP) return;
  const int b = pv.pose_prob[p];
  if (!problem_active(wv.lm, b, gate)) return;
  const int k = p - pv.p_pose_off[b];
  const int P = 6 * pv.p_npose[b];
  const int po = pv.p_param_off[b] + 6 * k;
  double xi[6], T0[12];
#pragma unroll
  for (int q = 0; q < 6; ++q) xi[q] = scale * wv.delta[po + q];
#pragma unroll
  for (int q = 0; q < 12; ++q) T0[q] = poses[12 * (size_t)p + q];
  double Tn[12];
  if constexpr (std::is_same<T, float>::value) {
    // FP32 path: T_new = T + T (Exp(xi) - I), the increment Exp(xi) - I formed in FP32
    // (relative precision of the increment itself) and the sum in double-float, so
    // FP64 (a small fraction of the FP32 rate here) is left with the conversions
    const float px = (float)xi[0], py = (float)xi[1], pz = (float)xi[2];
    const float t2 = px * px + py * py + pz * pz, th = sqrtf(t2);
    float a, b, c;
    if (th < 0.5f) {  // series, truncation below 1e-10 relative at 0.5
      const float t4 = t2 * t2, t6 = t4 * t2, t8 = t4 * t4;
      a = 1.f - t2 / 6.f + t4 / 120.f - t6 / 5040.f + t8 / 362880.f;
      b = 0.5f - t2 / 24.f + t4 / 720.f - t6 / 40320.f + t8 / 3628800.f;
      c = 1.f / 6.f - t2 / 120.f + t4 / 5040.f - t6 / 362880.f + t8 / 39916800.f;
    } else {
      float sn, cs;
      sincosf(th, &sn, &cs);
      const float sh = sinf(0.5f * th);
      a = sn / th;
      b = 2.f * sh * sh / t2;
      c = (th - sn) / (t2 * th);
    }
    const float S[9] = {0.f, -pz, py, pz, 0.f, -px, -py, px, 0.f};
    float S2[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        S2[3 * i + j] = S[3 * i] * S[j] + S[3 * i + 1] * S[3 + j] + S[3 * i + 2] * S[6 + j];
    float D[12];  // Exp(xi) - I, 3x4
    const float rx = (float)xi[3], ry = (float)xi[4], rz = (float)xi[5];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int j = 0; j < 3; ++j) D[4 * i + j] = a * S[3 * i + j] + b * S2[3 * i + j];
      const float jx = (i == 0 ? 1.f : 0.f) + b * S[3 * i] + c * S2[3 * i];
      const float jy = (i == 1 ? 1.f : 0.f) + b * S[3 * i + 1] + c * S2[3 * i + 1];
      const float jz = (i == 2 ? 1.f : 0.f) + b * S[3 * i + 2] + c * S2[3 * i + 2];
      D[4 * i + 3] = jx * rx + jy * ry + jz * rz;
    }
    df Rd[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Rd[3 * i + j] = df_from_double(T0[4 * i + j]);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        // (T D)(i, j) = sum_k R(i, k) D(k, j)  (D's last row is zero)
        const df td = Rd[3 * i] * D[j] + Rd[3 * i + 1] * D[4 + j] + Rd[3 * i + 2] * D[8 + j];
        const df v = df_from_double(T0[4 * i + j]) + td;
        Tn[4 * i + j] = (double)v.h + (double)v.l;
      }
    }
  } else {
    double E[12];
    exp_se3(xi, E);
    compose34(T0, E, Tn);
  }
#pragma unroll
  for (int q = 0; q < 12; ++q) out[12 * (size_t)p + q] = Tn[q];
  const double lam = wv.lm[b].lam;
  const T *A = reinterpret_cast<const T *>(wv.A) + pv.p_S_off[b];
  const T *g = reinterpret_cast<const T *>(wv.g);
  double pred = 0.0;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const double d = wv.delta[po + q];
    const double akk = (double)A[(size_t)(6 * k + q) * P + 6 * k + q];
    pred += d * ((gacc ? gacc[po + q] : (double)g[po + q]) + lam * akk * d);
  }
  atomicAdd(wv.pred_acc + b, pred);
}

template <typename T>
int launch_update_poses(const PlanView &pv, const WorkView &wv, const double *poses, double *poses_out,
                        double scale, int direct, void *stream, const double *gacc) {
  k_update_poses<T><<<grid_for(pv.NP, 128), 128, 0, (cudaStream_t)stream>>>(pv, wv, poses, poses_out, scale,
                                                                       direct ? GATE_ALL : GATE_RUNNING, gacc);
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
  s.fail = s.flag = s.factor_failures = s.res_sel = 0;
  s.rho1 = s.rho2 = s.rho3 = s.last_rel = s.last_predrel = 0.0;
  s.gnorm = s.dmean = s.dmax = s.dmin = s.cmean = 0.0;
  s.last_acc = s.rej_streak = 0;
  s.wait_timeouts = s.ref_done = 0;
  s.small_prev = s.pad_ = 0;
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

// after a linearisation: at the first one, the cost pass's value becomes the
// current (and initial) cost; later linearisation points are accepted candidates
// whose cost the candidate's cost pass already set
__global__ void k_post_linearize(PlanView pv, WorkView wv) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= pv.B) return;
  LMState &s = wv.lm[b];
  if (s.status != 0 || !s.relin) return;
  if (s.iters == 0) {
    s.cost = wv.cost_acc[b];
    s.cost0 = s.cost;
  }
  s.cost_lin = s.cost;
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
  if (wv.lm[b].status != 0) {
    wv.lm[b].flag = 0;
    return;
  }
  LMState s = wv.lm[b];  // one read of the record, one write at the end
  const double F = s.cost;
  const double Fn = wv.cost_acc[b];
  const double pred = 0.5 * wv.pred_acc[b];
  const int it = s.iters;
  const double lam_used = s.lam;
  wv.cost_acc[b] = 0.0;
  wv.pred_acc[b] = 0.0;
  s.cost_cand = Fn;
  s.pred = pred;
  s.iters += 1;
  const bool ok = !s.fail && isfinite(Fn) && pred > 0.0 && Fn < F;
  s.rho3 = s.rho2;
  s.rho2 = s.rho1;
  s.rho1 = s.fail ? -2.0 : (pred > 0.0 && isfinite(Fn) ? (F - Fn) / pred : -2.0);
  s.last_acc = ok ? 1 : 0;
  s.last_predrel = pred / fmax(F, 1e-300);
  s.rej_streak = ok ? 0 : s.rej_streak + 1;
  if (ok) {
    const double rho = (F - Fn) / pred;
    const double rel = (F - Fn) / fmax(F, 1e-300);
    s.last_rel = rel;
    s.accepted += 1;
    s.flag = 1;
    s.cost = Fn;
    const double t = 2.0 * rho - 1.0;
    s.lam *= fmax(1.0 / 3.0, 1.0 - t * t * t);
    s.nu = 2.0;
    s.relin = 1;
    s.res_sel ^= 1;  // the candidate's residuals are now the state's
    // a small decrease ends the solve when the model predicted it (rho >= stop_rho), when
    // the model itself predicts no more than tol, or when the last accepted step was
    // small too
    const bool small = rel < prm.tol;
    if (small && (rho >= (double)prm.stop_rho || pred < prm.tol * F || s.small_prev))
      s.status = SPGO_STATUS_CONVERGED;
    s.small_prev = small ? 1 : 0;
  } else {
    if (s.fail & FAIL_TIMEOUT)
      s.wait_timeouts += 1;
    else if (s.fail)
      s.factor_failures += 1;
    s.flag = 0;
    s.relin = 0;
    s.lam *= s.nu;
    s.nu *= 2.0;
    if (s.lam > prm.lambda_max) s.status = SPGO_STATUS_STALLED;
  }
  s.fail = 0;
  if (s.status == 0 && s.iters >= prm.max_iters) s.status = SPGO_STATUS_MAX_ITERS;
  wv.lm[b] = s;
  if (it < SPGO_TRACE_MAX) {
    double *t = wv.trace + ((size_t)b * SPGO_TRACE_MAX + it) * 3;
    t[0] = s.cost;
    t[1] = lam_used;
    t[2] = ok ? 1.0 : 0.0;
  }
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
      double v[12];  // all loads before the stores (the two buffers may alias as far as the compiler knows)
#pragma unroll
      for (int q = 0; q < 12; ++q) v[q] = wv.poses_cand[12 * t + q];
#pragma unroll
      for (int q = 0; q < 12; ++q) poses[12 * t + q] = v[q];
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

// dense damped reduced system of one problem, FP64 (both triangles), from A, S_L, g, g_L
template <typename T>
__global__ void k_export_S(PlanView pv, WorkView wv, int b, double *S, double *gS) {
  const int P = 6 * pv.p_npose[b];
  const size_t off = pv.p_S_off[b];
  const int po = pv.p_param_off[b];
  const T *A = reinterpret_cast<const T *>(wv.A) + off;
  T *SL = reinterpret_cast<T *>(wv.SL) + off;
  const double lam = wv.lm[b].lam;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)P * P) return;
  const int r = (int)(t / P), c = (int)(t % P);
  if (c > r) return;
  const size_t k = (size_t)r * P + c;
  const double v = (double)A[k] - (double)SL[k] + (r == c ? lam * (double)A[k] : 0.0);
  S[(size_t)r * P + c] = v;
  S[(size_t)c * P + r] = v;
  if (c == 0) {
    T *gL = reinterpret_cast<T *>(wv.gL) + po;
    gS[r] = (double)reinterpret_cast<const T *>(wv.g)[po + r] - (double)gL[r];
  }
}

template <typename T>
int launch_export_S(const PlanView &pv, const WorkView &wv, int problem, double *S, double *gS, void *stream) {
  const long long n = (long long)pv.max_P * pv.max_P;
  k_export_S<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(pv, wv, problem, S, gS);
  ++g_launches;
  // the Schur pass ran for every problem: clear all of S_L / g_L for the next one
  cudaMemsetAsync(wv.SL, 0, (size_t)pv.total_S * sizeof(T), (cudaStream_t)stream);
  cudaMemsetAsync(wv.gL, 0, (size_t)pv.total_params * sizeof(T), (cudaStream_t)stream);
  return (int)cudaGetLastError();
}
template int launch_export_S<float>(const PlanView &, const WorkView &, int, double *, double *, void *);
template int launch_export_S<double>(const PlanView &, const WorkView &, int, double *, double *, void *);

__global__ void k_scale_lambda(PlanView pv, WorkView wv, double factor) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < pv.B) wv.lm[b].lam = wv.lm_backup[b].lam * factor;
}

__global__ void k_take_probe(PlanView pv, WorkView wv, int j) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= pv.B) return;
  wv.probe_costs[(size_t)j * pv.B + b] = wv.lm[b].status == 0 ? wv.cost_acc[b] : 0.0;
  wv.cost_acc[b] = 0.0;
  wv.pred_acc[b] = 0.0;
}

int launch_scale_lambda(const PlanView &pv, const WorkView &wv, double factor, void *stream) {
  k_scale_lambda<<<grid_for(pv.B, 128), 128, 0, (cudaStream_t)stream>>>(pv, wv, factor);
  ++g_launches;
  return (int)cudaGetLastError();
}

int launch_take_probe(const PlanView &pv, const WorkView &wv, int j, void *stream) {
  k_take_probe<<<grid_for(pv.B, 128), 128, 0, (cudaStream_t)stream>>>(pv, wv, j);
  ++g_launches;
  return (int)cudaGetLastError();
}

__global__ void k_to_double(const void *src, int f64, double *dst, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dst[i] = f64 ? reinterpret_cast<const double *>(src)[i] : (double)reinterpret_cast<const float *>(src)[i];
}

int launch_to_double(const void *src, int f64, double *dst, int64_t n, void *stream) {
  if (n <= 0) return 0;
  k_to_double<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(src, f64, dst, n);
  ++g_launches;
  return (int)cudaGetLastError();
}

template int launch_factor_solve<float>(const PlanView &, const WorkView &, const Params &, int, void *);
template int launch_factor_solve<double>(const PlanView &, const WorkView &, const Params &, int, void *);
template int launch_update_poses<float>(const PlanView &, const WorkView &, const double *, double *, double, int, void *,
                                        const double *);
template int launch_update_poses<double>(const PlanView &, const WorkView &, const double *, double *, double, int, void *,
                                         const double *);
template int launch_backsub<float>(const PlanView &, const WorkView &, const Params &, const double *, double *, int, void *);
template int launch_backsub<double>(const PlanView &, const WorkView &, const Params &, const double *, double *, int, void *);
template int launch_export_B_n<float>(const PlanView &, const WorkView &, int, int, double *, double *, double *, void *);
template int launch_export_B_n<double>(const PlanView &, const WorkView &, int, int, double *, double *, double *, void *);

}  // namespace spgo
