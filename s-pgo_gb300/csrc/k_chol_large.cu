// Large reduced camera systems: problems whose packed factor does not fit in one
// CTA's shared memory (P beyond ~300 in FP32; config 1's 600 and config 2's 3000).
//
// Same mathematics as k_factor_solve (S = A + lam diag(A) - S_L, Cholesky, one
// refinement step with an exact residual), spread over the GPU instead of one CTA:
//   k_lg_assemble  row per CTA: the FP32/T copy of S into the factor storage
//                  (column-major, lower), the exact S (double-float / FP64,
//                  full, row-major) for the residual, g0 = g - g_L; clears S_L, g_L
//   per 64-column panel kb:
//     k_lg_potrf   one CTA factors the 64x64 diagonal block in shared memory,
//                  16 columns at a time (register-resident 16x16 blocks); on the
//                  FP32 path k_lg_potrf_rows, one thread per row of the block
//     k_lg_trsm    thread per row below it: L(i, kb:) = S(i, kb:) L_kk^-T
//     k_lg_syrk    one CTA per 64x64 tile of the trailing lower triangle,
//                  C -= L_i L_j^T from shared-memory tiles, 4x4 outputs per thread;
//                  the next panel's tile column first, then (with the solver's second
//                  stream) the next k_lg_potrf beside the rest of the update
//   k_lg_fwd/bwd   forward / backward substitution with one CTA per 64-row block,
//                  chained by per-block flags (32-unknown shuffle chains inside each
//                  diagonal block, staged in shared memory while the CTA waits its
//                  turn), x += solution
//   k_lg_resid     warp per row: g0 - S x from the exact S (between two solves)
// Replaces, for such problems, the reference's libtorch Cholesky of the dense
// reduced system (src/Optimization/linear_solvers.cu:195-218).
#include "kernels.cuh"
#include "dfloat.cuh"

#include <type_traits>

namespace spgo {

constexpr int kLgNB = 64;

template <typename T> struct ExactS;
template <> struct ExactS<float> { using type = float2; };  // (hi, lo) double-float
template <> struct ExactS<double> { using type = double; };

template <typename T>
__global__ void __launch_bounds__(256) k_lg_assemble(PlanView pv, WorkView wv, int b) {
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  const int P = 6 * pv.p_npose[b], r = blockIdx.x;
  if (r >= P) return;
  const size_t off = pv.p_S_off[b];
  const T *A = reinterpret_cast<const T *>(wv.A) + off;
  T *SL = reinterpret_cast<T *>(wv.SL) + off;
  T *fac = reinterpret_cast<T *>(wv.fac) + off;
  auto *Sx = reinterpret_cast<typename ExactS<T>::type *>(wv.Sx) + off;
  const double lam = wv.lm[b].lam;
  // S_L may hold entries up to the end of the row's 48-wide SIMT tile (both Schur paths clear here)
  constexpr int TR = 6 * SPGO_TILE_BLOCKS;
  const int cmax = min(P, (r / TR + 1) * TR);
  for (int c = threadIdx.x; c < cmax; c += blockDim.x) {
    if (c <= r) {
      const T a = A[(size_t)r * P + c], sl = SL[(size_t)r * P + c];
      T v = a - sl;
      if (c == r) v += (T)lam * a;
      fac[(size_t)c * P + r] = v;
      if constexpr (std::is_same<T, float>::value) {
        df e = df_sub(a, sl);
        if (c == r) e = e + df_from_double(lam * (double)a);
        Sx[(size_t)r * P + c] = make_float2(e.h, e.l);
        if (c < r) Sx[(size_t)c * P + r] = make_float2(e.h, e.l);
      } else {
        const double e = (double)a - (double)sl + (c == r ? lam * (double)a : 0.0);
        Sx[(size_t)r * P + c] = e;
        if (c < r) Sx[(size_t)c * P + r] = e;
      }
    }
    SL[(size_t)r * P + c] = T(0);
  }
  if (threadIdx.x == 0) {
    const int po = pv.p_param_off[b];
    T *gL = reinterpret_cast<T *>(wv.gL) + po;
    wv.lg_g0[po + r] = (double)reinterpret_cast<const T *>(wv.g)[po + r] - (double)gL[r];
    gL[r] = T(0);
  }
}

// One CTA factors the 64x64 diagonal block in shared memory, 16 columns at a time:
// warp 0 factors each 16x16 diagonal sub-block in registers (lane = row; column k
// takes one shuffle of the pivot and one per later row), then all threads solve
// the panel rows below it and update the rest of the panel's lower triangle:
// three barriers per 16 columns.
template <typename T>
__global__ void __launch_bounds__(256) k_lg_potrf(PlanView pv, WorkView wv, int b, int kb) {
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  constexpr int kSub = 16;
  __shared__ T D[kLgNB][kLgNB + 1];
  __shared__ T di[kLgNB];
  __shared__ int bad;
  const int P = 6 * pv.p_npose[b], nb = min(kLgNB, P - kb), tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  T *fac = reinterpret_cast<T *>(wv.fac) + pv.p_S_off[b];
  T *dinv = reinterpret_cast<T *>(wv.lg_dinv) + pv.p_param_off[b];
  for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
    const int i = idx % nb, j = idx / nb;
    if (i >= j) D[i][j] = fac[(size_t)(kb + j) * P + kb + i];
  }
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int s0 = 0; s0 < nb; s0 += kSub) {
    const int w = min(kSub, nb - s0), se = s0 + w;
    if (warp == 0) {
      T a[kSub];
#pragma unroll
      for (int j = 0; j < kSub; ++j) a[j] = (lane < w && j <= lane) ? D[s0 + lane][s0 + j] : T(0);
      bool badl = false;
      // (columns k >= w of a narrow last sub-block run on a unit pivot and are discarded)
#pragma unroll
      for (int k = 0; k < kSub; ++k) {
        const T dk = __shfl_sync(0xffffffffu, a[k], k);
        const T d = k < w ? dk : T(1);
        badl = badl || !(d > T(0)) || !(d < T(INFINITY));
        const T lkk = sqrt(d), rinv = T(1) / lkk;
        const T lik = lane > k ? a[k] * rinv : (lane == k ? lkk : a[k]);
        a[k] = lik;
#pragma unroll
        for (int j = 0; j < kSub; ++j) {
          const T ljk = __shfl_sync(0xffffffffu, lik, j);
          if (j > k && lane >= j) a[j] -= lik * ljk;
        }
        if (lane == 0 && k < w) di[s0 + k] = rinv;
      }
#pragma unroll
      for (int j = 0; j < kSub; ++j)
        if (lane < w && j <= lane) D[s0 + lane][s0 + j] = a[j];
      if (badl && lane == 0) bad = 1;
    }
    __syncthreads();
    // panel rows below the sub-block: L(i, s0:se) = D(i, s0:se) L_sub^-T (right-looking)
    for (int i = se + tid; i < nb; i += blockDim.x) {
      T x[kSub];
#pragma unroll
      for (int c = 0; c < kSub; ++c) x[c] = c < w ? D[i][s0 + c] : T(0);
#pragma unroll
      for (int c = 0; c < kSub; ++c) {
        x[c] = c < w ? x[c] * di[s0 + c] : T(0);
#pragma unroll
        for (int m = c + 1; m < kSub; ++m)
          if (m < w) x[m] -= x[c] * D[s0 + m][s0 + c];
      }
#pragma unroll
      for (int c = 0; c < kSub; ++c)
        if (c < w) D[i][s0 + c] = x[c];
    }
    __syncthreads();
    // the rest of the panel: D(i, j) -= sum_c L(i, c) L(j, c) for se <= j <= i < nb
    const int m = nb - se;
    for (int idx = tid; idx < m * m; idx += blockDim.x) {
      const int ii = se + idx % m, jj = se + idx / m;
      if (ii >= jj) {
        T acc = T(0);
#pragma unroll
        for (int c = 0; c < kSub; ++c)
          if (c < w) acc += D[ii][s0 + c] * D[jj][s0 + c];
        D[ii][jj] -= acc;
      }
    }
    __syncthreads();
  }
  if (tid == 0 && bad) atomicOr(&wv.lm[b].fail, FAIL_PIVOT);
  for (int k = tid; k < nb; k += blockDim.x) dinv[kb + k] = di[k];
  for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
    const int i = idx % nb, j = idx / nb;
    if (i >= j) fac[(size_t)(kb + j) * P + kb + i] = D[i][j];
  }
}

// FP32 path: one CTA of 64 threads factors the 64x64 diagonal block, thread i holding row i of
// the block in registers.  Column k: the threads of rows i >= k put their entry of
// column k into a shared column (double-buffered: one barrier per column), then each
// reads the pivot, and row i > k forms L(i, k) = a(i, k) / L(k, k) and updates its own
// entries j in (k, i]: a(i, j) -= L(i, k) L(j, k), with L(j, k) taken as a(j, k) from
// the shared column times 1 / L(k, k).  The serial part per column is one barrier,
// one square root and one reciprocal; the update is spread over the rows.  (The FP64
// path keeps k_lg_potrf: FP64 issues at 1/64 of the FP32 rate, and 64 threads carrying
// the update alone made it slower.)
__global__ void __launch_bounds__(kLgNB) k_lg_potrf_rows(PlanView pv, WorkView wv, int b, int kb) {
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  __shared__ float col[2][kLgNB];
  const int P = 6 * pv.p_npose[b], nb = min(kLgNB, P - kb), i = threadIdx.x;
  float *fac = reinterpret_cast<float *>(wv.fac) + pv.p_S_off[b];
  float *dinv = reinterpret_cast<float *>(wv.lg_dinv) + pv.p_param_off[b];
  float a[kLgNB];
#pragma unroll
  for (int j = 0; j < kLgNB; ++j) a[j] = (i < nb && j <= i) ? fac[(size_t)(kb + j) * P + kb + i] : 0.f;
  bool bad = false;
  float rdiag = 0.f;  // 1 / L(i, i)
#pragma unroll
  for (int k = 0; k < kLgNB; ++k) {
    if (k >= nb) break;  // (uniform: a narrow last panel)
    float *c = col[k & 1];
    if (i >= k) c[i] = a[k];
    __syncthreads();
    const float d = c[k];
    bad = bad || !(d > 0.f) || !(d < INFINITY);
    const float lkk = sqrtf(d), rinv = 1.f / lkk;  // correctly rounded, as in the batched factorisation
    if (i == k) {
      a[k] = lkk;
      rdiag = rinv;
    } else if (i > k) {
      const float lik = a[k] * rinv;
      a[k] = lik;
      const float s = lik * rinv;  // L(i, k) / L(k, k): times a(j, k) gives L(i, k) L(j, k)
#pragma unroll
      for (int j = k + 1; j < kLgNB; ++j)
        if (j <= i) a[j] -= s * c[j];
    }
  }
  if (i < nb) {
#pragma unroll
    for (int j = 0; j < kLgNB; ++j)
      if (j <= i) fac[(size_t)(kb + j) * P + kb + i] = a[j];
    dinv[kb + i] = rdiag;
  }
  if (bad && i == 0) atomicOr(&wv.lm[b].fail, FAIL_PIVOT);
}

// thread per row below the panel: L(i, kb:ke) = S(i, kb:ke) L_kk^-T, right-looking
// (once x_j is final it is removed from every later column: independent updates
// instead of one dependent chain per column)
template <typename T>
__global__ void __launch_bounds__(128) k_lg_trsm(PlanView pv, WorkView wv, int b, int kb) {
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  __shared__ T D[kLgNB][kLgNB + 1];
  __shared__ T di[kLgNB];
  const int P = 6 * pv.p_npose[b], nb = min(kLgNB, P - kb), ke = kb + nb, tid = threadIdx.x;
  const T *fac_c = reinterpret_cast<const T *>(wv.fac) + pv.p_S_off[b];
  T *fac = reinterpret_cast<T *>(wv.fac) + pv.p_S_off[b];
  const T *dinv = reinterpret_cast<const T *>(wv.lg_dinv) + pv.p_param_off[b];
  for (int idx0 = tid; idx0 < kLgNB * kLgNB; idx0 += 8 * blockDim.x) {
    T v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {  // loads first
      const int idx = idx0 + q * blockDim.x, i = idx % kLgNB, j = idx / kLgNB;
      v[q] = (idx < kLgNB * kLgNB && i > j && i < nb) ? fac_c[(size_t)(kb + j) * P + kb + i] : T(0);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int idx = idx0 + q * blockDim.x;
      if (idx < kLgNB * kLgNB) D[idx % kLgNB][idx / kLgNB] = v[q];
    }
  }
  for (int j = tid; j < kLgNB; j += blockDim.x) di[j] = j < nb ? dinv[kb + j] : T(0);
  __syncthreads();
  const int i = ke + blockIdx.x * blockDim.x + tid;
  if (i >= P) return;
  T x[kLgNB];
#pragma unroll
  for (int j = 0; j < kLgNB; ++j) x[j] = j < nb ? fac_c[(size_t)(kb + j) * P + i] : T(0);
#pragma unroll
  for (int j = 0; j < kLgNB; ++j) {
    x[j] *= di[j];
#pragma unroll
    for (int m = j + 1; m < kLgNB; ++m) x[m] -= x[j] * D[m][j];
  }
#pragma unroll
  for (int j = 0; j < kLgNB; ++j)
    if (j < nb) fac[(size_t)(kb + j) * P + i] = x[j];
}

// tiles of the trailing lower triangle: mode 0 all of them, mode 1 the first tile column
// (the next panel's columns), mode 2 the others
template <typename T>
__global__ void __launch_bounds__(256) k_lg_syrk(PlanView pv, WorkView wv, int b, int kb, int mode) {
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  __shared__ T LR[kLgNB][kLgNB + 1];
  __shared__ T LC[kLgNB][kLgNB + 1];
  const int P = 6 * pv.p_npose[b], nb = min(kLgNB, P - kb), ke = kb + nb, tid = threadIdx.x;
  // tile t -> (ti >= tj) of the trailing lower triangle (mode 2: of the triangle without
  // its first tile column, shifted by one)
  const int t = blockIdx.x;
  int ti, tj;
  if (mode == 1) {
    ti = t;
    tj = 0;
  } else {
    ti = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
    while (ti * (ti + 1) / 2 > t) --ti;
    tj = t - ti * (ti + 1) / 2;
    if (mode == 2) {
      ++ti;
      ++tj;
    }
  }
  const int R0 = ke + kLgNB * ti, C0 = ke + kLgNB * tj;
  T *fac = reinterpret_cast<T *>(wv.fac) + pv.p_S_off[b];
  for (int idx = tid; idx < nb * kLgNB; idx += blockDim.x) {
    const int r = idx % kLgNB, k = idx / kLgNB;
    LR[k][r] = R0 + r < P ? fac[(size_t)(kb + k) * P + R0 + r] : T(0);
    LC[k][r] = C0 + r < P ? fac[(size_t)(kb + k) * P + C0 + r] : T(0);
  }
  __syncthreads();
  const int tx = tid % 16, ty = tid / 16;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
  for (int k = 0; k < nb; ++k) {
    T a[4], c[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      a[i] = LR[k][tx + 16 * i];
      c[i] = LC[k][ty + 16 * i];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * c[j];
  }
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = R0 + tx + 16 * i, c = C0 + ty + 16 * j;
      if (r < P && c < P && r >= c) fac[(size_t)c * P + r] -= acc[i][j];
    }
}

// ---- substitutions spread over the GPU: one CTA per 64-row block ----
// Forward L z = r: the CTA of block k adds up L(k, j) z_j for every earlier block j
// as soon as that block's flag is up, then solves its diagonal block and raises its
// own flag; backward L^T x = z the same from the bottom (the CTA of block k waits
// only for blocks finished by lower-numbered CTAs, so the chain never waits on a CTA
// that has not started).  Thread (r, q) handles unknown r of the block and a 16-wide
// quarter q of each other block.  Every wait is bounded (the parameter's limit,
// 2 s by default); a timeout marks the problem failed (the step is rejected and
// counted as a timeout, not as a factorisation failure) and the CTA carries on.

__device__ __forceinline__ uint64_t lg_clock_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool lg_wait_flag(const int *flag, uint64_t deadline) {
  for (int it = 0;; ++it) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(flag) : "memory");
    if (v) return true;
    if ((it & 7) == 7 && lg_clock_ns() > deadline) return false;  // (~1 us between looks at the clock)
    __nanosleep(100);
  }
}

__device__ __forceinline__ void lg_set_flag(int *flag) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(flag), "r"(1) : "memory");
}

template <typename T>
__global__ void __launch_bounds__(256) k_lg_fwd(PlanView pv, WorkView wv, int b, int first, uint64_t wait_ns) {
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  __shared__ T part[4][kLgNB];
  __shared__ T zs[kLgNB];
  __shared__ T Ld[kLgNB][kLgNB + 1];  // the diagonal block (lower, zero elsewhere) and its pivots,
  __shared__ T ds[kLgNB];             // staged while the earlier blocks are still being solved
  __shared__ int timed_out;
  const int P = 6 * pv.p_npose[b], po = pv.p_param_off[b];
  const int k = blockIdx.x, kb = k * kLgNB, nb = min(kLgNB, P - kb);
  const int tid = threadIdx.x, r = tid & 63, q = tid >> 6, warp = tid >> 5, lane = tid & 31;
  const T *L = reinterpret_cast<const T *>(wv.fac) + pv.p_S_off[b];
  auto Lat = [&](int i, int j) { return L[(size_t)j * P + i]; };  // L(i, j), i >= j
  const T *dinv = reinterpret_cast<const T *>(wv.lg_dinv) + po;
  T *z = reinterpret_cast<T *>(wv.lg_y) + po;  // in place: this block's right-hand side in, z out
  int *flag = wv.lg_flag + po;
  const uint64_t deadline = lg_clock_ns() + wait_ns;
  if (tid == 0) timed_out = 0;
  for (int idx = tid; idx < kLgNB * kLgNB; idx += blockDim.x) {
    const int i = idx % kLgNB, j = idx / kLgNB;
    Ld[i][j] = (i < nb && j <= i) ? Lat(kb + i, kb + j) : T(0);
  }
  if (tid < kLgNB) ds[tid] = tid < nb ? dinv[kb + tid] : T(0);
  __syncthreads();
  T acc = T(0);
  for (int j = 0; j < k; ++j) {  // earlier blocks are full 64-wide
    // this block's part of L is loaded before the wait for block j's solution
    const int c0 = j * kLgNB + 16 * q;
    T lv[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) lv[c] = r < nb ? Lat(kb + r, c0 + c) : T(0);
    if (tid == 0 && !timed_out && !lg_wait_flag(flag + j, deadline)) timed_out = 1;
    __syncthreads();
    if (r < nb) {
      T zv[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) zv[c] = __ldcg(z + c0 + c);
#pragma unroll
      for (int c = 0; c < 16; ++c) acc += lv[c] * zv[c];
    }
  }
  part[q][r] = acc;
  __syncthreads();
  if (tid < nb) {
    const T rhs = first ? (T)wv.lg_g0[po + kb + tid] : z[kb + tid];
    zs[tid] = rhs - ((part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]));
  }
  __syncthreads();
  if (warp == 0) {  // L_kk z_k = zs: two 32-unknown halves, lane = unknown
    for (int h = 0; h < nb; h += 32) {
      const int w = min(32, nb - h);
      T v = lane < w ? zs[h + lane] : T(0);
      if (h > 0) {  // the first half is final: loads first, four chains
        T lq[32];
#pragma unroll
        for (int c = 0; c < 32; ++c) lq[c] = lane < w ? Ld[h + lane][c] : T(0);
        T v1 = T(0), v2 = T(0), v3 = T(0);
#pragma unroll
        for (int c = 0; c < 32; c += 4) {
          v -= lq[c] * zs[c];
          v1 -= lq[c + 1] * zs[c + 1];
          v2 -= lq[c + 2] * zs[c + 2];
          v3 -= lq[c + 3] * zs[c + 3];
        }
        v += (v1 + v2) + v3;
      }
      T lr[32], di[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        lr[c] = (lane < w && c < lane) ? Ld[h + lane][h + c] : T(0);
        di[c] = c < w ? ds[h + c] : T(0);
      }
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        T yc = v * di[c];
        yc = __shfl_sync(0xffffffffu, yc, c);
        if (lane == c) v = yc;
        v -= lr[c] * yc;
      }
      if (lane < w) zs[h + lane] = v;
      __syncwarp();
    }
  }
  __syncthreads();
  if (tid < nb) z[kb + tid] = zs[tid];
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    lg_set_flag(flag + k);
    if (timed_out) atomicOr(&wv.lm[b].fail, FAIL_TIMEOUT);
  }
}

// backward L^T x = z (z in place in lg_y); then x is added to the solution so far
// (first: x itself) and written to delta (last) or to lg_x and its split; accum
// (a refinement correction of the mixed path): delta += x and ddelta = x
template <typename T>
__global__ void __launch_bounds__(256) k_lg_bwd(PlanView pv, WorkView wv, int b, int first, int last, int accum,
                                                 uint64_t wait_ns) {
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  __shared__ T part[4][kLgNB];
  __shared__ T zs[kLgNB];
  __shared__ T Ld[kLgNB][kLgNB + 1];  // the diagonal block (lower, zero elsewhere) and its pivots,
  __shared__ T ds[kLgNB];             // staged while the later blocks are still being solved
  __shared__ int timed_out;
  const int P = 6 * pv.p_npose[b], po = pv.p_param_off[b];
  const int nblk = (P + kLgNB - 1) / kLgNB, k = nblk - 1 - (int)blockIdx.x;
  const int kb = k * kLgNB, nb = min(kLgNB, P - kb);
  const int tid = threadIdx.x, r = tid & 63, q = tid >> 6, warp = tid >> 5, lane = tid & 31;
  const T *L = reinterpret_cast<const T *>(wv.fac) + pv.p_S_off[b];
  auto Lat = [&](int i, int j) { return L[(size_t)j * P + i]; };
  const T *dinv = reinterpret_cast<const T *>(wv.lg_dinv) + po;
  T *x = reinterpret_cast<T *>(wv.lg_y) + po;
  int *flag = wv.lg_flag + pv.total_params + po;
  const uint64_t deadline = lg_clock_ns() + wait_ns;
  if (tid == 0) timed_out = 0;
  for (int idx = tid; idx < kLgNB * kLgNB; idx += blockDim.x) {
    const int i = idx % kLgNB, j = idx / kLgNB;
    Ld[i][j] = (i < nb && j <= i) ? Lat(kb + i, kb + j) : T(0);
  }
  if (tid < kLgNB) ds[tid] = tid < nb ? dinv[kb + tid] : T(0);
  __syncthreads();
  T acc = T(0);
  for (int j = nblk - 1; j > k; --j) {  // later blocks, finished by lower-numbered CTAs
    // this block's part of L is loaded before the wait for block j's solution
    const int jb = j * kLgNB, nbj = min(kLgNB, P - jb);
    T lv[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const int i = 16 * q + c;
      lv[c] = (r < nb && i < nbj) ? Lat(jb + i, kb + r) : T(0);  // column kb + r: contiguous per thread
    }
    if (tid == 0 && !timed_out && !lg_wait_flag(flag + j, deadline)) timed_out = 1;
    __syncthreads();
    if (r < nb) {
      T xv[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int i = 16 * q + c;
        xv[c] = i < nbj ? __ldcg(x + jb + i) : T(0);
      }
#pragma unroll
      for (int c = 0; c < 16; ++c) acc += lv[c] * xv[c];
    }
  }
  part[q][r] = acc;
  __syncthreads();
  if (tid < nb) zs[tid] = x[kb + tid] - ((part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]));
  __syncthreads();
  if (warp == 0) {  // L_kk^T x_k = zs, halves from the bottom
    for (int h = ((nb - 1) / 32) * 32; h >= 0; h -= 32) {
      const int w = min(32, nb - h);
      T v = lane < w ? zs[h + lane] : T(0);
      if (h + w < nb) {  // the later half is final (h = 0): loads first
        T lq[32];
#pragma unroll
        for (int c = 0; c < 32; ++c) lq[c] = (lane < w && 32 + c < nb) ? Ld[32 + c][h + lane] : T(0);
        T v1 = T(0), v2 = T(0), v3 = T(0);
#pragma unroll
        for (int c = 0; c < 32; c += 4) {
          v -= lq[c] * (32 + c < nb ? zs[32 + c] : T(0));
          v1 -= lq[c + 1] * (33 + c < nb ? zs[33 + c] : T(0));
          v2 -= lq[c + 2] * (34 + c < nb ? zs[34 + c] : T(0));
          v3 -= lq[c + 3] * (35 + c < nb ? zs[35 + c] : T(0));
        }
        v += (v1 + v2) + v3;
      }
      T lc[32], di[32];  // column `lane` of the diagonal block, pivots
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        lc[c] = (c < w && lane < c) ? Ld[h + c][h + lane] : T(0);
        di[c] = c < w ? ds[h + c] : T(0);
      }
#pragma unroll
      for (int c = 31; c >= 0; --c) {
        T xc = v * di[c];
        xc = __shfl_sync(0xffffffffu, xc, c);
        if (lane == c) v = xc;
        v -= lc[c] * xc;
      }
      if (lane < w) zs[h + lane] = v;
      __syncwarp();
    }
  }
  __syncthreads();
  if (tid < nb) x[kb + tid] = zs[tid];
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    lg_set_flag(flag + k);
    if (timed_out) atomicOr(&wv.lm[b].fail, FAIL_TIMEOUT);
  }
  if (tid < nb && accum) {
    const int i = kb + tid;
    wv.delta[po + i] += (double)zs[tid];
    wv.ddelta[po + i] = (double)zs[tid];
  } else if (tid < nb) {
    const int i = kb + tid;
    const double xi = (first ? 0.0 : wv.lg_x[po + i]) + (double)zs[tid];
    if (last) {
      wv.delta[po + i] = xi;  // (a failed factorisation zeroes delta after the solve)
    } else {
      wv.lg_x[po + i] = xi;
      const df sp = df_from_double(xi);
      wv.lg_xs[2 * (po + i)] = sp.h;
      wv.lg_xs[2 * (po + i) + 1] = sp.l;
    }
  }
}

// a failed factorisation (or a timed-out substitution) leaves no step
__global__ void k_lg_zero_failed(PlanView pv, WorkView wv, int b) {
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  if (!wv.lm[b].fail) return;
  const int P = 6 * pv.p_npose[b], po = pv.p_param_off[b];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) wv.delta[po + i] = 0.0;
}

// residual y = g0 - S x from the exact S, warp per row
template <typename T>
__global__ void __launch_bounds__(256) k_lg_resid(PlanView pv, WorkView wv, int b) {
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  const int P = 6 * pv.p_npose[b], po = pv.p_param_off[b];
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i >= P) return;
  const auto *Sx = reinterpret_cast<const typename ExactS<T>::type *>(wv.Sx) + pv.p_S_off[b] + (size_t)i * P;
  double r;
  if constexpr (std::is_same<T, float>::value) {
    const float *xs = wv.lg_xs + 2 * (size_t)po;
    df acc = df_make(0.f);
    for (int j = lane; j < P; j += 32) {
      const float2 s = Sx[j];
      acc = acc + df{s.x, s.y} * df{xs[2 * j], xs[2 * j + 1]};
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const df other{__shfl_xor_sync(0xffffffffu, acc.h, o), __shfl_xor_sync(0xffffffffu, acc.l, o)};
      acc = acc + other;
    }
    r = (double)acc.h + (double)acc.l;
  } else {
    double acc = 0.0;
    for (int j = lane; j < P; j += 32) acc += Sx[j] * wv.lg_x[po + j];
    r = warp_sum(acc);
  }
  if (lane == 0) reinterpret_cast<T *>(wv.lg_y)[po + i] = (T)(wv.lg_g0[po + i] - r);
}

template <typename T>
int launch_factor_large(const PlanView &pv, const WorkView &wv, const Params &prm, int b, int P, int param_off,
                        int refine, void *stream, void *side, void *ev_a, void *ev_b) {
  cudaStream_t st = (cudaStream_t)stream;
  const uint64_t wait_ns = wait_limit_ns(prm);
  k_lg_assemble<T><<<P, 256, 0, st>>>(pv, wv, b);
  int n = 1;
  auto potrf = [&](int kb, cudaStream_t on) {
    if constexpr (std::is_same<T, float>::value)
      k_lg_potrf_rows<<<1, kLgNB, 0, on>>>(pv, wv, b, kb);
    else
      k_lg_potrf<T><<<1, 256, 0, on>>>(pv, wv, b, kb);
    ++n;
  };
  // one panel of look-ahead: once panel kb's rows are solved, the next panel's columns take
  // its update first and the next diagonal block is factored on the side stream while the
  // rest of the trailing matrix is updated; every element takes the same updates in the
  // same order as without it
  cudaStream_t sd = (cudaStream_t)side;
  cudaEvent_t ea = (cudaEvent_t)ev_a, eb = (cudaEvent_t)ev_b;
  const bool ahead = sd && ea && eb;
  potrf(0, st);
  for (int kb = 0; kb < P; kb += kLgNB) {
    const int ke = min(P, kb + kLgNB);
    if (ke >= P) break;  // (the last diagonal block is factored: nothing below it)
    const int M = P - ke, nt = (M + kLgNB - 1) / kLgNB;
    k_lg_trsm<T><<<(M + 127) / 128, 128, 0, st>>>(pv, wv, b, kb);
    n += 1;
    if (!ahead) {
      k_lg_syrk<T><<<nt * (nt + 1) / 2, 256, 0, st>>>(pv, wv, b, kb, 0);
      ++n;
      potrf(ke, st);
      continue;
    }
    k_lg_syrk<T><<<nt, 256, 0, st>>>(pv, wv, b, kb, 1);
    ++n;
    cudaError_t e = cudaEventRecord(ea, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(sd, ea, 0);
    if (e != cudaSuccess) return (int)e;
    potrf(ke, sd);
    if ((e = cudaEventRecord(eb, sd)) != cudaSuccess) return (int)e;
    if (nt > 1) {
      k_lg_syrk<T><<<(nt - 1) * nt / 2, 256, 0, st>>>(pv, wv, b, kb, 2);
      ++n;
    }
    if ((e = cudaStreamWaitEvent(st, eb, 0)) != cudaSuccess) return (int)e;
  }
  const int nblk = (P + kLgNB - 1) / kLgNB;
  int *ff = wv.lg_flag + param_off, *fb = wv.lg_flag + pv.total_params + param_off;
  for (int it = 0; it <= refine; ++it) {
    if (it > 0) {
      k_lg_resid<T><<<(P + 7) / 8, 256, 0, st>>>(pv, wv, b);
      ++n;
    }
    cudaError_t e = cudaMemsetAsync(ff, 0, sizeof(int) * (size_t)nblk, st);
    if (e != cudaSuccess) return (int)e;
    k_lg_fwd<T><<<nblk, 256, 0, st>>>(pv, wv, b, it == 0, wait_ns);
    e = cudaMemsetAsync(fb, 0, sizeof(int) * (size_t)nblk, st);
    if (e != cudaSuccess) return (int)e;
    k_lg_bwd<T><<<nblk, 256, 0, st>>>(pv, wv, b, it == 0, it == refine, 0, wait_ns);
    n += 2;
  }
  k_lg_zero_failed<<<grid_for(P, 256), 256, 0, st>>>(pv, wv, b);
  ++n;
  g_launches += n;
  return (int)cudaGetLastError();
}

// one refinement correction of the mixed path: the right-hand side is in lg_y
// (k_resid_solve); delta += S^-1 lg_y with the factor of this iteration
int launch_refine_large(const PlanView &pv, const WorkView &wv, const Params &prm, int b, int P, int param_off,
                        void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  const uint64_t wait_ns = wait_limit_ns(prm);
  const int nblk = (P + kLgNB - 1) / kLgNB;
  int *ff = wv.lg_flag + param_off, *fb = wv.lg_flag + pv.total_params + param_off;
  cudaError_t e = cudaMemsetAsync(ff, 0, sizeof(int) * (size_t)nblk, st);
  if (e != cudaSuccess) return (int)e;
  k_lg_fwd<float><<<nblk, 256, 0, st>>>(pv, wv, b, 0, wait_ns);
  e = cudaMemsetAsync(fb, 0, sizeof(int) * (size_t)nblk, st);
  if (e != cudaSuccess) return (int)e;
  k_lg_bwd<float><<<nblk, 256, 0, st>>>(pv, wv, b, 0, 0, 1, wait_ns);
  g_launches += 2;
  return (int)cudaGetLastError();
}

template int launch_factor_large<float>(const PlanView &, const WorkView &, const Params &, int, int, int, int,
                                        void *, void *, void *, void *);
template int launch_factor_large<double>(const PlanView &, const WorkView &, const Params &, int, int, int, int,
                                         void *, void *, void *, void *);

}  // namespace spgo
