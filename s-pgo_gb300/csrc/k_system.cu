// Reduced camera system: pose-pose Hessian from the (lo, hi) pair accumulators,
// the landmark Schur complement W D^-1 W^T, and S = A + damping - W D^-1 W^T.
//
// Replaces the reference's dense cuBLAS products A = J_T^T J_T, g_T = J_T^T r,
// B C^-1 B^T, B C^-1 g_a and the element-wise subtraction
// (src/Optimization/Solver_cuda.cu:626-730, kernel :35-45).
//
// Pose-pose blocks (incremental chain, S-PGO's parameterisation): for i <= j,
//   A(i, j) = Ad_i^T F(i, j) Ad_j,  F(i, j) = sum_{lo <= i, hi > j} M_{lo,hi},
// with every M shifted to the world origin in FP64 first (E_x^T M E_x), then a
// prefix sum over lo (fixed hi) and a suffix sum over hi (fixed i), in place.
// g(i) = Ad_i^T sum_{lo <= i < hi} m_{lo,hi} is the e = 0 diagonal of the same sums.
#include "kernels.cuh"

namespace spgo {

__device__ __forceinline__ constexpr int t6(int i, int j) {  // symmetric 6x6 upper index, any order
  return i <= j ? i * 6 - (i * (i - 1)) / 2 + (j - i) : j * 6 - (j * (j - 1)) / 2 + (i - j);
}

// shift one pair record from origin x = left centre of frame lo to the world
// origin (FP64) and clear the accumulator for the next linearisation
template <typename T>
__global__ void k_pair_shift(PlanView pv, WorkView wv) {
  const int b = blockIdx.y;
  if (!problem_active(wv.lm, b, GATE_RELIN)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * D) return;
  const int lo = t / D, d = t % D + 1;
  if (lo + d > N) return;
  const size_t rec = (size_t)(pv.p_pair_off[b] + t);
  T *src = reinterpret_cast<T *>(wv.pair_acc) + rec * 27;
  double M[21], m[6];
#pragma unroll
  for (int k = 0; k < 21; ++k) { M[k] = (double)src[k]; src[k] = T(0); }
#pragma unroll
  for (int k = 0; k < 6; ++k) { m[k] = (double)src[21 + k]; src[21 + k] = T(0); }
  const double *x = wv.fr_c + (size_t)(pv.p_frame_off[b] + lo) * 6;
  const double X[9] = {0, -x[2], x[1], x[2], 0, -x[0], -x[1], x[0], 0};
  // blocks: P = M[w w], Q = M[w v], R = M[v v]
  double P[9], Q[9], R[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      P[3 * i + j] = M[t6(i, j)];
      Q[3 * i + j] = M[t6(i, 3 + j)];
      R[3 * i + j] = M[t6(3 + i, 3 + j)];
    }
  // P' = P - Q X + X Q^T - X R X ;  Q' = Q + X R ;  R' = R
  double QX[9], XQt[9], XR[9], XRX[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double a = 0, bq = 0, c = 0;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        a += Q[3 * i + k] * X[3 * k + j];
        bq += X[3 * i + k] * Q[3 * j + k];
        c += X[3 * i + k] * R[3 * k + j];
      }
      QX[3 * i + j] = a;
      XQt[3 * i + j] = bq;
      XR[3 * i + j] = c;
    }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double a = 0;
#pragma unroll
      for (int k = 0; k < 3; ++k) a += XR[3 * i + k] * X[3 * k + j];
      XRX[3 * i + j] = a;
    }
  double *dst = wv.pair64 + rec * 27;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j)
      dst[t6(i, j)] = P[3 * i + j] - QX[3 * i + j] + XQt[3 * i + j] - XRX[3 * i + j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) dst[t6(i, 3 + j)] = Q[3 * i + j] + XR[3 * i + j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) dst[t6(3 + i, 3 + j)] = R[3 * i + j];
  // m' = [m_w + X m_v ; m_v]
#pragma unroll
  for (int i = 0; i < 3; ++i)
    dst[21 + i] = m[i] + X[3 * i] * m[3] + X[3 * i + 1] * m[4] + X[3 * i + 2] * m[5];
#pragma unroll
  for (int i = 0; i < 3; ++i) dst[24 + i] = m[3 + i];
}

// prefix over lo for fixed hi:  P(i, hi) = sum_{lo <= i} M(lo, hi), in place
__global__ void k_pair_prefix_lo(PlanView pv, WorkView wv) {
  const int b = blockIdx.y;
  if (!problem_active(wv.lm, b, GATE_RELIN)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * 27) return;
  const int hi = 1 + t / 27, comp = t % 27;
  double *base = wv.pair64 + (size_t)pv.p_pair_off[b] * 27 + comp;
  double acc = 0.0;
  for (int lo = max(0, hi - D); lo < hi; ++lo) {
    double *p = base + ((size_t)lo * D + (hi - lo - 1)) * 27;
    acc += *p;
    *p = acc;
  }
}

// suffix over hi for fixed i:  F(i, i + e) = sum_{d' > e} P(i, i + d'), in place
__global__ void k_pair_suffix_hi(PlanView pv, WorkView wv) {
  const int b = blockIdx.y;
  if (!problem_active(wv.lm, b, GATE_RELIN)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * 27) return;
  const int i = t / 27, comp = t % 27;
  double *base = wv.pair64 + ((size_t)pv.p_pair_off[b] + (size_t)i * D) * 27 + comp;
  double acc = 0.0;
  for (int dp = min(D, N - i); dp >= 1; --dp) {
    double *p = base + (size_t)(dp - 1) * 27;
    acc += *p;
    *p = acc;
  }
}

// A(i, j) = Ad_i^T F(i, j) Ad_j and g(i) = Ad_i^T f(i); Ad = [[R, 0], [[c]x R, R]]
__global__ void k_pairs_to_A(PlanView pv, WorkView wv) {
  const int b = blockIdx.y;
  if (!problem_active(wv.lm, b, GATE_RELIN)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * D) return;
  const int i = t / D, e = t % D;
  if (e >= min(D, N - i)) return;
  const int j = i + e;
  const int P = 6 * N;
  const int fo = pv.p_frame_off[b];
  const double *F = wv.pair64 + ((size_t)pv.p_pair_off[b] + (size_t)i * D + e) * 27;
  const double *Ri = wv.fr_Rd + (size_t)(fo + i) * 18, *ci = wv.fr_c + (size_t)(fo + i) * 6;
  const double *Rj = wv.fr_Rd + (size_t)(fo + j) * 18, *cj = wv.fr_c + (size_t)(fo + j) * 6;
  // C R = [c]x R for both frames
  double CRi[9], CRj[9];
  {
    const double Xi[9] = {0, -ci[2], ci[1], ci[2], 0, -ci[0], -ci[1], ci[0], 0};
    const double Xj[9] = {0, -cj[2], cj[1], cj[2], 0, -cj[0], -cj[1], cj[0], 0};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        double a = 0, bb = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          a += Xi[3 * r + k] * Ri[3 * k + c];
          bb += Xj[3 * r + k] * Rj[3 * k + c];
        }
        CRi[3 * r + c] = a;
        CRj[3 * r + c] = bb;
      }
  }
  double *A = wv.A + pv.p_S_off[b];
  for (int col = 0; col < 6; ++col) {
    // column `col` of Ad_j
    double adj[6];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      adj[r] = col < 3 ? Rj[3 * r + col] : 0.0;
      adj[3 + r] = col < 3 ? CRj[3 * r + col] : Rj[3 * r + col - 3];
    }
    double w[6];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      double a = 0;
#pragma unroll
      for (int k = 0; k < 6; ++k) a += F[t6(r, k)] * adj[k];
      w[r] = a;
    }
    // out = Ad_i^T w : rows 0-2 = R_i^T w_w + (C_i R_i)^T w_v ; rows 3-5 = R_i^T w_v
    double out[6];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      out[r] = Ri[r] * w[0] + Ri[3 + r] * w[1] + Ri[6 + r] * w[2] + CRi[r] * w[3] + CRi[3 + r] * w[4] +
               CRi[6 + r] * w[5];
      out[3 + r] = Ri[r] * w[3] + Ri[3 + r] * w[4] + Ri[6 + r] * w[5];
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      A[(size_t)(6 * i + r) * P + 6 * j + col] = out[r];
      if (i != j) A[(size_t)(6 * j + col) * P + 6 * i + r] = out[r];
    }
  }
  if (e == 0) {
    const double *f = F + 21;
    double *g = wv.g + pv.p_param_off[b] + 6 * i;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      g[r] = Ri[r] * f[0] + Ri[3 + r] * f[1] + Ri[6 + r] * f[2] + CRi[r] * f[3] + CRi[3 + r] * f[4] +
             CRi[6 + r] * f[5];
      g[3 + r] = Ri[r] * f[3] + Ri[3 + r] * f[4] + Ri[6 + r] * f[5];
    }
  }
}

template <typename T>
int launch_system(const PlanView &pv, const WorkView &wv, int gate, void *stream) {
  (void)gate;
  cudaStream_t st = (cudaStream_t)stream;
  const int nd = pv.max_D > 0 ? pv.max_D : 1;
  dim3 g1(grid_for((long long)(pv.max_P / 6) * nd, 128), pv.B);
  k_pair_shift<T><<<g1, 128, 0, st>>>(pv, wv);
  dim3 g2(grid_for((long long)(pv.max_P / 6) * 27, 128), pv.B);
  k_pair_prefix_lo<<<g2, 128, 0, st>>>(pv, wv);
  k_pair_suffix_hi<<<g2, 128, 0, st>>>(pv, wv);
  k_pairs_to_A<<<g1, 128, 0, st>>>(pv, wv);
  g_launches += 4;
  return (int)cudaGetLastError();
}

// ---- landmark Schur complement ------------------------------------------------
// S_L(I, J) = sum over chunks of W_I diag(d) W_J^T with d_l = 1 / (C_l (1 + lam) + eps),
// g_L = sum W d g_a.  One CTA per work item = (problem, 48x48 output tile, <= 16 chunks);
// partial tiles are added atomically (S_L is cleared by the assembly that reads it).
template <typename T>
__global__ void __launch_bounds__(256) k_schur(PlanView pv, WorkView wv, Params prm, int gate) {
  const int w = blockIdx.x;
  const int b = pv.wk_prob[w];
  if (!problem_active(wv.lm, b, gate)) return;
  const int ti = pv.wk_ti[w], tj = pv.wk_tj[w];
  const int N = pv.p_npose[b], P = 6 * N;
  const double lam = wv.lm[b].lam;
  const T eps = (T)prm.eps;
  constexpr int TR = 6 * SPGO_TILE_BLOCKS;  // 48
  __shared__ T WI[TR][SPGO_CHUNK + 1];
  __shared__ T WJ[TR][SPGO_CHUNK + 1];
  __shared__ T dg[SPGO_CHUNK];
  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;
  T acc[3][3];
#pragma unroll
  for (int x = 0; x < 3; ++x)
#pragma unroll
    for (int y = 0; y < 3; ++y) acc[x][y] = T(0);
  T accg = T(0);
  const bool diag = (ti == tj);
  const T *Cv = reinterpret_cast<const T *>(wv.C);
  const T *gav = reinterpret_cast<const T *>(wv.ga);
  const T *slab_all = reinterpret_cast<const T *>(wv.slab);
  for (int k = pv.wk_cbeg[w]; k < pv.wk_cend[w]; ++k) {
    const int c = pv.wk_chunks[k];
    const int f0 = pv.ch_f0[c], nb = pv.ch_nb[c], lm0 = pv.ch_lm0[c], cnt = pv.ch_cnt[c];
    const T *slab = slab_all + pv.ch_slab[c];
    for (int idx = tid; idx < TR * SPGO_CHUNK; idx += blockDim.x) {
      const int r = idx / SPGO_CHUNK, col = idx % SPGO_CHUNK;
      const int bi = SPGO_TILE_BLOCKS * ti + r / 6;
      const int bj = SPGO_TILE_BLOCKS * tj + r / 6;
      T dv = T(0);
      if (col < cnt) dv = T(1) / (Cv[lm0 + col] * (T)(1.0 + lam) + eps);
      T vi = T(0), vj = T(0);
      if (bi >= f0 && bi < f0 + nb && bi < N) vi = slab[(size_t)(6 * (bi - f0) + r % 6) * SPGO_CHUNK + col];
      if (bj >= f0 && bj < f0 + nb && bj < N) vj = slab[(size_t)(6 * (bj - f0) + r % 6) * SPGO_CHUNK + col];
      WI[r][col] = vi;
      WJ[r][col] = vj * dv;
      if (r == 0) dg[col] = (col < cnt) ? dv * gav[lm0 + col] : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < SPGO_CHUNK; ++kk) {
      const T a0 = WI[3 * tr][kk], a1 = WI[3 * tr + 1][kk], a2 = WI[3 * tr + 2][kk];
      const T b0 = WJ[3 * tc][kk], b1 = WJ[3 * tc + 1][kk], b2 = WJ[3 * tc + 2][kk];
      acc[0][0] += a0 * b0; acc[0][1] += a0 * b1; acc[0][2] += a0 * b2;
      acc[1][0] += a1 * b0; acc[1][1] += a1 * b1; acc[1][2] += a1 * b2;
      acc[2][0] += a2 * b0; acc[2][1] += a2 * b1; acc[2][2] += a2 * b2;
    }
    if (diag && tid < TR) {
#pragma unroll 8
      for (int kk = 0; kk < SPGO_CHUNK; ++kk) accg += WI[tid][kk] * dg[kk];
    }
    __syncthreads();
  }
  T *SL = reinterpret_cast<T *>(wv.SL) + pv.p_S_off[b];
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    const int row = TR * ti + 3 * tr + x;
    if (row >= P) continue;
#pragma unroll
    for (int y = 0; y < 3; ++y) {
      const int col = TR * tj + 3 * tc + y;
      if (col < P && acc[x][y] != T(0)) red_add(SL + (size_t)row * P + col, acc[x][y]);
    }
  }
  if (diag && tid < TR) {
    const int row = TR * ti + tid;
    if (row < P && accg != T(0)) red_add(reinterpret_cast<T *>(wv.gL) + pv.p_param_off[b] + row, accg);
  }
}

template <typename T>
int launch_schur(const PlanView &pv, const WorkView &wv, const Params &prm, void *stream) {
  if (pv.n_items == 0) return 0;
  k_schur<T><<<pv.n_items, 256, 0, (cudaStream_t)stream>>>(pv, wv, prm, GATE_RUNNING);
  ++g_launches;
  return (int)cudaGetLastError();
}

// ---- S = A + lam diag(A) - S_L (both triangles), g_S = g - g_L; clears S_L / g_L ----
template <typename T>
__global__ void k_assemble(PlanView pv, WorkView wv) {
  const int b = blockIdx.y;
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  const int N = pv.p_npose[b], P = 6 * N;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)P * P) return;
  const int r = (int)(t / P), c = (int)(t % P);
  constexpr int TR = 6 * SPGO_TILE_BLOCKS;
  if (r / TR < c / TR) return;  // handled by the mirrored element
  const double lam = wv.lm[b].lam;
  const size_t off = pv.p_S_off[b];
  T *SL = reinterpret_cast<T *>(wv.SL) + off;
  const double sl = (double)SL[(size_t)r * P + c];
  SL[(size_t)r * P + c] = T(0);
  const double *A = wv.A + off;
  double *S = wv.S + off;
  double v = A[(size_t)r * P + c] - sl;
  if (r == c) v += lam * A[(size_t)r * P + c];
  S[(size_t)r * P + c] = v;
  // diagonal tiles hold both halves; an off-diagonal tile also fills its mirror
  if (r / TR != c / TR) S[(size_t)c * P + r] = v;
  if (c == 0) {
    const int po = pv.p_param_off[b];
    T *gL = reinterpret_cast<T *>(wv.gL) + po;
    wv.gS[po + r] = wv.g[po + r] - (double)gL[r];
    gL[r] = T(0);
  }
}

template <typename T>
int launch_assemble(const PlanView &pv, const WorkView &wv, void *stream) {
  dim3 g(grid_for((long long)pv.max_P * pv.max_P, 256), pv.B);
  k_assemble<T><<<g, 256, 0, (cudaStream_t)stream>>>(pv, wv);
  ++g_launches;
  return (int)cudaGetLastError();
}

template int launch_system<float>(const PlanView &, const WorkView &, int, void *);
template int launch_system<double>(const PlanView &, const WorkView &, int, void *);
template int launch_schur<float>(const PlanView &, const WorkView &, const Params &, void *);
template int launch_schur<double>(const PlanView &, const WorkView &, const Params &, void *);
template int launch_assemble<float>(const PlanView &, const WorkView &, void *);
template int launch_assemble<double>(const PlanView &, const WorkView &, void *);

}  // namespace spgo
