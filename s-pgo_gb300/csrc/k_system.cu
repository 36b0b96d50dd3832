// Reduced camera system: pose-pose Hessian from the (lo, hi) pair accumulators,
// the landmark Schur complement W D^-1 W^T, and S = A + damping - W D^-1 W^T.
//
// Replaces the reference's dense cuBLAS products A = J_T^T J_T, g_T = J_T^T r,
// B C^-1 B^T, B C^-1 g_a and the element-wise subtraction
// (src/Optimization/Solver_cuda.cu:626-730, kernel :35-45).
//
// Pose-pose blocks (incremental chain, S-PGO's parameterisation): for i <= j,
//   A(i, j) = Ad_i^T F(i, j) Ad_j,  F(i, j) = sum_{lo <= i, hi > j} M_{lo,hi},
// computed by a prefix sum over lo (fixed hi, re-centring the running sum on
// each row's camera centre) and a suffix sum over hi (fixed i).  Every sum is
// kept about a nearby camera centre, so the working precision (FP32 in the
// mixed path) never sees world-sized lever arms.
// g(i) = Ad_i^T sum_{lo <= i < hi} m_{lo,hi} is the e = 0 diagonal of the same sums.
#include <type_traits>
#include "kernels.cuh"
#include "frames.cuh"
#include "dfloat.cuh"

namespace spgo {

__device__ __forceinline__ constexpr int t6(int i, int j) {  // symmetric 6x6 upper index, any order
  return i <= j ? i * 6 - (i * (i - 1)) / 2 + (j - i) : j * 6 - (j * (j - 1)) / 2 + (i - j);
}

// pass A, one thread per (problem, hi):
// P(i, hi) = sum_{lo <= i} M(lo, hi), each term about its own origin c_lo; the
// running sum is re-centred from c_{lo-1} to c_lo before adding M(lo, hi), so
// every partial sum sits at the origin of its row i and only relative centres
// enter the arithmetic.  Re-centring a record: E_z^T M E_z and E_z^T m for
// E_z = [[I, 0], [-[z]x, I]] move a record from origin x to origin y = x - z
// (K^y = K^x E_{x - y}).  With the 6x6 block M = [[P, Q], [Q^T, R]] (upper triangle,
// 21 values), m = [m_w; m_v] and Z = [z]x:  P' = P - Q Z + Z Q^T - Z R Z,
// Q' = Q + Z R,  R' = R,  m' = [m_w + Z m_v ; m_v].  Reads and clears the records.
// The thread holds the whole 27-value running sum, so the shift's shared products
// are formed once per step (about a sixth of the arithmetic of one lane per
// component, which matters in FP64):
//   (Z R)[:, j] = z x R[:, j],  (Q Z)[i, :] = -(z x Q[i, :]),  ((Z R) Z)[i, :] = -(z x (Z R)[i, :]),
//   P' = P - Q Z - (Q Z)^T - (Z R) Z,  Q' = Q + Z R,  m_w' = m_w + z x m_v.
template <typename V>
__device__ __forceinline__ void cross3(const V *a, const V *b, V *o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

// V = double, or df (the mixed path's reduction, on the FP32 pipes)
template <typename V>
__device__ __forceinline__ void shift_record(V *v, const V *z) {
  V P[3][3], Q[3][3], R[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      P[a][c] = v[t6(a, c)];
      Q[a][c] = v[t6(a, 3 + c)];
      R[a][c] = v[t6(3 + a, 3 + c)];
    }
  V ZR[3][3], QZ[3][3], ZRZ[3][3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {  // columns of Z R
    const V rc[3] = {R[0][j], R[1][j], R[2][j]};
    V o[3];
    cross3(z, rc, o);
    ZR[0][j] = o[0];
    ZR[1][j] = o[1];
    ZR[2][j] = o[2];
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {  // rows of Q Z and (Z R) Z
    V o[3];
    cross3(z, Q[i], o);
    QZ[i][0] = -o[0];
    QZ[i][1] = -o[1];
    QZ[i][2] = -o[2];
    cross3(z, ZR[i], o);
    ZRZ[i][0] = -o[0];
    ZRZ[i][1] = -o[1];
    ZRZ[i][2] = -o[2];
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int c = a; c < 3; ++c) v[t6(a, c)] = P[a][c] - QZ[a][c] - QZ[c][a] - ZRZ[a][c];
#pragma unroll
    for (int c = 0; c < 3; ++c) v[t6(a, 3 + c)] = Q[a][c] + ZR[a][c];
  }
  const V mv[3] = {v[24], v[25], v[26]};
  V o[3];
  cross3(z, mv, o);
  v[21] += o[0];
  v[22] += o[1];
  v[23] += o[2];
}

__global__ void __launch_bounds__(64) k_pair_prefix_rec(PlanView pv, WorkView wv) {
  const int b = blockIdx.y;
  if (!problem_active(wv.lm, b, GATE_RELIN)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b];
  const int hi = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (hi > N) return;
  const int fo = pv.p_frame_off[b];
  double *acc_base = reinterpret_cast<double *>(wv.pair_acc) + (size_t)pv.p_pair_off[b] * 27;
  double *out_base = reinterpret_cast<double *>(wv.pairF) + (size_t)pv.p_pair_off[b] * 27;
  const int lo0 = max(0, hi - D);
  double v[27];
#pragma unroll
  for (int k = 0; k < 27; ++k) v[k] = 0.0;
  for (int lo = lo0; lo < hi; ++lo) {
    if (lo > lo0) {
      const Vec3<double> zz = FramesT<double>::rel(wv, fo + lo - 1, 0, fo + lo, 0);
      const double z[3] = {zz.x, zz.y, zz.z};
      shift_record(v, z);
    }
    double *rec = acc_base + ((size_t)lo * D + (hi - lo - 1)) * 27;
    double *out = out_base + ((size_t)lo * D + (hi - lo - 1)) * 27;
    double r[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) r[k] = rec[k];
#pragma unroll
    for (int k = 0; k < 27; ++k) {
      rec[k] = 0.0;  // cleared for the next linearisation
      v[k] += r[k];
      out[k] = v[k];
    }
  }
}

// pass B, one thread per (problem, i, component): F(i, i + e) = sum_{d' > e} P(i, i + d')
// (all about origin c_i), in place
template <typename T>
__global__ void k_pair_suffix(PlanView pv, WorkView wv) {
  const int b = blockIdx.y;
  if (!problem_active(wv.lm, b, GATE_RELIN)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * 27) return;
  const int i = t / 27, comp = t % 27;
  T *base = reinterpret_cast<T *>(wv.pairF) + ((size_t)pv.p_pair_off[b] + (size_t)i * D) * 27 + comp;
  T acc = T(0);
  int dp = min(D, N - i);
  for (; dp >= 8; dp -= 8) {  // eight records loaded before any is summed
    T v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = base[(size_t)(dp - 1 - q) * 27];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      acc += v[q];
      base[(size_t)(dp - 1 - q) * 27] = acc;
    }
  }
  for (; dp >= 1; --dp) {
    T *p = base + (size_t)(dp - 1) * 27;
    acc += *p;
    *p = acc;
  }
}

template <typename T> struct Pair2;
template <> struct Pair2<float> {
  using type = float2;
  __device__ static float2 make(float a, float b) { return make_float2(a, b); }
};
template <> struct Pair2<double> {
  using type = double2;
  __device__ static double2 make(double a, double b) { return make_double2(a, b); }
};

// A(i, j) = Ad_i^T F(i, j) Ad_j about origin c_i: Ad_i = diag(R_i, R_i),
// Ad_j = [[R_j, 0], [[c_j - c_i]x R_j, R_j]];  g(i) = [R_i^T f_w ; R_i^T f_v].
// Computed in T, stored as TO (the mixed path reduces in FP64 and stores FP32: one
// rounding of the exact sums)
template <typename T, typename TO = T>
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
  // the record and both rotations in registers first (the A stores below could
  // otherwise alias them and force reloads)
  const T *Fg = reinterpret_cast<const T *>(wv.pairF) + ((size_t)pv.p_pair_off[b] + (size_t)i * D + e) * 27;
  const T *Rig = FramesT<T>::R(wv, fo + i, 0);
  const T *Rjg = FramesT<T>::R(wv, fo + j, 0);
  T F[27], Ri[9], Rj[9];
#pragma unroll
  for (int k = 0; k < 27; ++k) F[k] = Fg[k];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    Ri[k] = Rig[k];
    Rj[k] = Rjg[k];
  }
  const Vec3<T> cji = FramesT<T>::rel(wv, fo + j, 0, fo + i, 0);
  // C R_j with C = [c_j - c_i]x
  T CRj[9];
  {
    const T X[9] = {T(0), -cji.z, cji.y, cji.z, T(0), -cji.x, -cji.y, cji.x, T(0)};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        CRj[3 * r + c] = X[3 * r] * Rj[c] + X[3 * r + 1] * Rj[3 + c] + X[3 * r + 2] * Rj[6 + c];
  }
  // the whole 6x6 block first: out[r][c] = A(6i + r, 6j + c)
  T out[6][6];
#pragma unroll
  for (int col = 0; col < 6; ++col) {
    T adj[6];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      adj[r] = col < 3 ? Rj[3 * r + col] : T(0);
      adj[3 + r] = col < 3 ? CRj[3 * r + col] : Rj[3 * r + col - 3];
    }
    T w[6];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      T a = T(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) a += F[t6(r, k)] * adj[k];
      w[r] = a;
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      out[r][col] = Ri[r] * w[0] + Ri[3 + r] * w[1] + Ri[6 + r] * w[2];
      out[3 + r][col] = Ri[r] * w[3] + Ri[3 + r] * w[4] + Ri[6 + r] * w[5];
    }
  }
  // both copies as pairs of adjacent elements (every offset below is even and the
  // workspace segment 256-byte aligned): the block (i, j) row by row, and for
  // i != j its transpose (j, i), whose rows are 6 elements at 6i of rows 6j + c
  using V2 = typename Pair2<TO>::type;
  TO *A = reinterpret_cast<TO *>(wv.A) + pv.p_S_off[b];
#pragma unroll
  for (int r = 0; r < 6; ++r)
#pragma unroll
    for (int c = 0; c < 6; c += 2)
      *reinterpret_cast<V2 *>(A + (size_t)(6 * i + r) * P + 6 * j + c) =
          Pair2<TO>::make((TO)out[r][c], (TO)out[r][c + 1]);
  if (i != j) {
#pragma unroll
    for (int c = 0; c < 6; ++c)
#pragma unroll
      for (int r = 0; r < 6; r += 2)
        *reinterpret_cast<V2 *>(A + (size_t)(6 * j + c) * P + 6 * i + r) =
            Pair2<TO>::make((TO)out[r][c], (TO)out[r + 1][c]);
  }
  if (e == 0) {
    const T *f = F + 21;
    TO *g = reinterpret_cast<TO *>(wv.g) + pv.p_param_off[b] + 6 * i;
    T gi[6];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      gi[r] = Ri[r] * f[0] + Ri[3 + r] * f[1] + Ri[6 + r] * f[2];
      gi[3 + r] = Ri[r] * f[3] + Ri[3 + r] * f[4] + Ri[6 + r] * f[5];
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) g[r] = (TO)gi[r];
    if (wv.gacc) {  // the mixed path's refined step: the gradient unrounded, for its predicted decrease
      double *ga = wv.gacc + pv.p_param_off[b] + 6 * i;
#pragma unroll
      for (int r = 0; r < 6; ++r) ga[r] = (double)gi[r];
    }
  }
}

// ---- the mixed path's pair reduction, in double-float ----------------------------
// The records arrive as FP64 sums (the linearisation's atomics).  FP64 arithmetic runs at
// a small fraction of the FP32 rate on this GPU, so the reduction runs in double-float
// (~48 bits on the FP32 pipes, far more than the FP32 blocks it produces keep).  Instead
// of re-centring a running sum along each chain (a serial chain of shifts), every record
// is moved once to the problem's own origin o = c_0 (its lever arms are at most the
// window's extent, tens of metres, which costs a few of the 48 bits), the prefix and
// suffix sums run about o, and each block moves its sum from o to c_i on the way to A.
__device__ __forceinline__ void df_rel_c(const WorkView &wv, int fx, int fy, df *z) {  // c_x - c_y, left cameras
#pragma unroll
  for (int k = 0; k < 3; ++k)
    z[k] = df_sub(wv.fr_ch[(size_t)fx * 6 + k], wv.fr_ch[(size_t)fy * 6 + k]) +
           df_make(wv.fr_cl[(size_t)fx * 6 + k] - wv.fr_cl[(size_t)fy * 6 + k]);
}

constexpr int kPrThreads = 512;

// 0. every record (lo, hi): read (FP64) and cleared, split into double-float, moved from
// c_lo to o; one thread per record
__global__ void __launch_bounds__(128) k_pair_shift_df(PlanView pv, WorkView wv) {
  const int b = blockIdx.y;
  if (!problem_active(wv.lm, b, GATE_RELIN)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= N * D) return;
  const int lo = r / D, hi = lo + r % D + 1;
  if (hi > N) return;
  const int fo = pv.p_frame_off[b];
  double *rec = reinterpret_cast<double *>(wv.pair_acc) + ((size_t)pv.p_pair_off[b] + r) * 27;
  df v[27];
#pragma unroll
  for (int k = 0; k < 27; ++k) v[k] = df_split_double(rec[k]);
#pragma unroll
  for (int k = 0; k < 27; ++k) rec[k] = 0.0;  // cleared for the next linearisation
  if (lo > 0) {
    df z[3];
    df_rel_c(wv, fo + lo, fo, z);  // from c_lo to o = c_0
    shift_record(v, z);
  }
  df *out = reinterpret_cast<df *>(wv.pairF) + ((size_t)pv.p_pair_off[b] + r) * 27;
#pragma unroll
  for (int k = 0; k < 27; ++k) out[k] = v[k];
}

// one CTA per problem: 1. thread per (hi, component): prefix over lo,
// P(i, hi) = sum_{lo <= i} M(lo, hi);  2. thread per (i, component): suffix over hi,
// F(i, i + e) = sum_{d > e} P(i, i + d)
__global__ void __launch_bounds__(kPrThreads) k_pair_scan_df(PlanView pv, WorkView wv) {
  const int b = blockIdx.x;
  if (!problem_active(wv.lm, b, GATE_RELIN)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b];
  const int tid = threadIdx.x, nt = blockDim.x;
  df *F = reinterpret_cast<df *>(wv.pairF) + (size_t)pv.p_pair_off[b] * 27;
  // the running sums: eight records loaded before any is summed and stored back (the
  // stores could alias later loads, so without that each step is a round trip)
  for (int t = tid; t < N * 27; t += nt) {
    const int hi = t / 27 + 1, comp = t % 27;
    df s = df_make(0.f);
    for (int lo0 = max(0, hi - D); lo0 < hi; lo0 += 8) {
      df v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (lo0 + q < hi) v[q] = F[((size_t)(lo0 + q) * D + (hi - lo0 - q - 1)) * 27 + comp];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (lo0 + q < hi) {
          s = s + v[q];
          F[((size_t)(lo0 + q) * D + (hi - lo0 - q - 1)) * 27 + comp] = s;
        }
    }
  }
  __syncthreads();
  for (int t = tid; t < N * 27; t += nt) {
    const int i = t / 27, comp = t % 27;
    df *base = F + (size_t)i * D * 27 + comp;
    df s = df_make(0.f);
    for (int dp0 = min(D, N - i); dp0 >= 1; dp0 -= 8) {
      df v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (dp0 - q >= 1) v[q] = base[(size_t)(dp0 - q - 1) * 27];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (dp0 - q >= 1) {
          s = s + v[q];
          base[(size_t)(dp0 - q - 1) * 27] = s;
        }
    }
  }
}

// A(i, j) = Ad_i^T F(i, j) Ad_j about c_i (F moved there from o first) and g(i), in
// double-float, rounded once to FP32; the unrounded g also to gacc (the refined step's
// predicted decrease)
__global__ void __launch_bounds__(128) k_pairs_to_A_df(PlanView pv, WorkView wv) {
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
  const df *Fg = reinterpret_cast<const df *>(wv.pairF) + ((size_t)pv.p_pair_off[b] + (size_t)i * D + e) * 27;
  df F[27], Ri[9], Rj[9];
#pragma unroll
  for (int k = 0; k < 27; ++k) F[k] = Fg[k];
  {
    const float *h = wv.fr_Rf + (size_t)(fo + i) * 18, *l = wv.fr_Rl + (size_t)(fo + i) * 18;
    const float *hj = wv.fr_Rf + (size_t)(fo + j) * 18, *lj = wv.fr_Rl + (size_t)(fo + j) * 18;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      Ri[k] = df{h[k], l[k]};
      Rj[k] = df{hj[k], lj[k]};
    }
  }
  if (i > 0) {
    df z[3];
    df_rel_c(wv, fo, fo + i, z);  // from o = c_0 to c_i
    shift_record(F, z);
  }
  df cji[3];
  df_rel_c(wv, fo + j, fo + i, cji);
  // C R_j with C = [c_j - c_i]x
  df CRj[9];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    CRj[c] = cji[1] * Rj[6 + c] - cji[2] * Rj[3 + c];
    CRj[3 + c] = cji[2] * Rj[c] - cji[0] * Rj[6 + c];
    CRj[6 + c] = cji[0] * Rj[3 + c] - cji[1] * Rj[c];
  }
  float out[6][6];
#pragma unroll
  for (int col = 0; col < 6; ++col) {
    // column col of Ad_j: [R_j e_col ; C R_j e_col] (col < 3), [0 ; R_j e_(col-3)]
    df w[6];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      df a = col < 3 ? F[t6(r, 0)] * Rj[col] + F[t6(r, 1)] * Rj[3 + col] + F[t6(r, 2)] * Rj[6 + col]
                     : df_make(0.f);
      const int cc = col < 3 ? col : col - 3;
      const df *ad = col < 3 ? CRj : Rj;
      a = a + F[t6(r, 3)] * ad[cc] + F[t6(r, 4)] * ad[3 + cc] + F[t6(r, 5)] * ad[6 + cc];
      w[r] = a;
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      out[r][col] = df_to_float(Ri[r] * w[0] + Ri[3 + r] * w[1] + Ri[6 + r] * w[2]);
      out[3 + r][col] = df_to_float(Ri[r] * w[3] + Ri[3 + r] * w[4] + Ri[6 + r] * w[5]);
    }
  }
  float *A = reinterpret_cast<float *>(wv.A) + pv.p_S_off[b];
#pragma unroll
  for (int r = 0; r < 6; ++r)
#pragma unroll
    for (int c = 0; c < 6; c += 2)
      *reinterpret_cast<float2 *>(A + (size_t)(6 * i + r) * P + 6 * j + c) = make_float2(out[r][c], out[r][c + 1]);
  if (i != j) {
#pragma unroll
    for (int c = 0; c < 6; ++c)
#pragma unroll
      for (int r = 0; r < 6; r += 2)
        *reinterpret_cast<float2 *>(A + (size_t)(6 * j + c) * P + 6 * i + r) = make_float2(out[r][c], out[r + 1][c]);
  }
  if (e == 0) {
    const df *f = F + 21;
    float *g = reinterpret_cast<float *>(wv.g) + pv.p_param_off[b] + 6 * i;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const df gw = Ri[r] * f[0] + Ri[3 + r] * f[1] + Ri[6 + r] * f[2];
      const df gv = Ri[r] * f[3] + Ri[3 + r] * f[4] + Ri[6 + r] * f[5];
      g[r] = df_to_float(gw);
      g[3 + r] = df_to_float(gv);
      if (wv.gacc) {
        wv.gacc[pv.p_param_off[b] + 6 * i + r] = df_to_double(gw);
        wv.gacc[pv.p_param_off[b] + 6 * i + 3 + r] = df_to_double(gv);
      }
    }
  }
}

// The pose-pair records are FP64 sums on both paths.  The FP64 path reduces them in
// FP64 along each chain; the mixed path (T = float) in double-float about one origin
// per problem, storing A and g as FP32.
template <typename T>
int launch_system(const PlanView &pv, const WorkView &wv, int gate, void *stream) {
  (void)gate;
  cudaStream_t st = (cudaStream_t)stream;
  const int nmax = pv.max_P / 6;
  const int nd = pv.max_D > 0 ? pv.max_D : 1;
  if constexpr (std::is_same<T, float>::value) {
    k_pair_shift_df<<<dim3(grid_for((long long)nmax * nd, 128), pv.B), 128, 0, st>>>(pv, wv);
    k_pair_scan_df<<<pv.B, kPrThreads, 0, st>>>(pv, wv);
    k_pairs_to_A_df<<<dim3(grid_for((long long)nmax * nd, 128), pv.B), 128, 0, st>>>(pv, wv);
    g_launches += 3;
  } else {
    k_pair_prefix_rec<<<dim3(grid_for(nmax, 64), pv.B), 64, 0, st>>>(pv, wv);
    k_pair_suffix<double><<<dim3(grid_for((long long)nmax * 27, 128), pv.B), 128, 0, st>>>(pv, wv);
    k_pairs_to_A<double, T><<<dim3(grid_for((long long)nmax * nd, 128), pv.B), 128, 0, st>>>(pv, wv);
    g_launches += 3;
  }
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

template int launch_system<float>(const PlanView &, const WorkView &, int, void *);
template int launch_system<double>(const PlanView &, const WorkView &, int, void *);
template int launch_schur<float>(const PlanView &, const WorkView &, const Params &, void *);
template int launch_schur<double>(const PlanView &, const WorkView &, const Params &, void *);

}  // namespace spgo
