// Landmark Schur complement on the 5th-generation tensor cores (mixed path).
//
//   S_L = sum_l B_l B_l^T / (C_l (1 + lam) + eps)       (W D^-1 W^T)
//
// replaces the reference's B C^-1 B^T cuBLAS SGEMM over a dense P x L matrix
// (src/Optimization/Solver_cuda.cu:690-699).  The landmark-chunk slabs written by
// the linearisation are already K-major operands: rows = pose parameters,
// K = the chunk's 32 landmarks.  One CTA (4 warps) per work item = (problem,
// 128-row tile, column range <= 256, list of chunks): for every chunk the warps
// stage A = W[rows] and B = W[cols] D^-1 into shared memory (core-matrix layout,
// double buffered), one thread issues four kind::tf32 MMAs (K = 8 each) into a
// TMEM accumulator of 128 lanes x N columns, and commits them to the buffer's
// mbarrier; the epilogue reads TMEM with tcgen05.ld and adds the lower triangle
// into S_L.  TF32 operands (10-bit mantissa), FP32 accumulation.
//
// The g-side term g_L = sum_l B_l g_a,l / D_l is a matrix-vector product and
// runs on the SIMT cores (k_schur_g).
#include "kernels.cuh"
#include "tc.cuh"

namespace spgo {

constexpr int kTcM = 128;
constexpr int kTcNmax = 256;
constexpr int kTcK = SPGO_CHUNK;  // 32 landmarks per chunk
constexpr uint32_t kWaitLimit = 1u << 24;

struct TcSmem {
  float A[2][kTcM * kTcK];       // 16 KB per buffer
  float B[2][kTcNmax * kTcK];    // 32 KB per buffer
  float dk[2][kTcK];
  uint64_t mbar[2];
  uint32_t tmem_slot;
};

__global__ void __launch_bounds__(128) k_schur_tc(PlanView pv, WorkView wv, Params prm, int gate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // 1024-byte aligned base for the operand tiles
  unsigned char *base = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  TcSmem &sm = *reinterpret_cast<TcSmem *>(base);
  const int w = blockIdx.x;
  const int b = pv.tc_prob[w];
  if (!problem_active(wv.lm, b, gate)) return;
  const int row0 = pv.tc_row0[w], col0 = pv.tc_col0[w], ncols = pv.tc_ncols[w];
  const int P = 6 * pv.p_npose[b];
  const float lam1 = (float)(1.0 + wv.lm[b].lam);
  const float eps = prm.eps;
  const float *Cv = reinterpret_cast<const float *>(wv.C);
  const float *slab_all = reinterpret_cast<const float *>(wv.slab);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t ncols_alloc = ncols <= 32 ? 32u : ncols <= 64 ? 64u : ncols <= 128 ? 128u : 256u;
  if (tid == 0) {
    tc::mbar_init(&sm.mbar[0], 1);
    tc::mbar_init(&sm.mbar[1], 1);
    tc::mbar_init_fence();
  }
  if (warp == 0) tc::tmem_alloc(&sm.tmem_slot, ncols_alloc);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = sm.tmem_slot;
  const uint32_t idesc = tc::idesc_tf32(kTcM, ncols);
  const int cb = pv.tc_cbeg[w], ce = pv.tc_cend[w];
  int ok = 1;
  for (int kc = cb; kc < ce && ok; ++kc) {
    const int it = kc - cb, buf = it & 1;
    if (it >= 2) ok = tc::mbar_wait(&sm.mbar[buf], ((it >> 1) - 1) & 1, kWaitLimit) ? 1 : 0;
    ok = __syncthreads_and(ok);
    if (!ok) break;
    const int c = pv.tc_chunks[kc];
    const int f0 = pv.ch_f0[c], nb = pv.ch_nb[c], lm0 = pv.ch_lm0[c], cnt = pv.ch_cnt[c];
    const float *slab = slab_all + pv.ch_slab[c];
    const int s0 = 6 * f0, s1 = 6 * (f0 + nb);  // parameter rows the slab covers
    if (tid < kTcK) sm.dk[buf][tid] = tid < cnt ? 1.f / (Cv[lm0 + tid] * lam1 + eps) : 0.f;
    __syncthreads();
    unsigned char *Ab = reinterpret_cast<unsigned char *>(sm.A[buf]);
    unsigned char *Bb = reinterpret_cast<unsigned char *>(sm.B[buf]);
    for (int idx = tid; idx < kTcM * 8; idx += blockDim.x) {
      const int r = idx >> 3, kq = idx & 7;
      const int gr = row0 + r;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gr < P && gr >= s0 && gr < s1) v = reinterpret_cast<const float4 *>(slab + (size_t)(gr - s0) * kTcK)[kq];
      *reinterpret_cast<float4 *>(Ab + tc::kmajor_offset(r, 4 * kq)) = v;
    }
    for (int idx = tid; idx < ncols * 8; idx += blockDim.x) {
      const int r = idx >> 3, kq = idx & 7;
      const int gc = col0 + r;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gc < P && gc >= s0 && gc < s1) {
        v = reinterpret_cast<const float4 *>(slab + (size_t)(gc - s0) * kTcK)[kq];
        const float *d = sm.dk[buf] + 4 * kq;
        v.x *= d[0];
        v.y *= d[1];
        v.z *= d[2];
        v.w *= d[3];
      }
      *reinterpret_cast<float4 *>(Bb + tc::kmajor_offset(r, 4 * kq)) = v;
    }
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(Ab), b0 = tc::smem_u32(Bb);
#pragma unroll
      for (int ks = 0; ks < kTcK / 8; ++ks) {
        const uint64_t ad = tc::smem_desc(a0 + ks * 256, 128, 1024);
        const uint64_t bd = tc::smem_desc(b0 + ks * 256, 128, 1024);
        tc::mma_tf32(tmem, ad, bd, idesc, (it > 0 || ks > 0) ? 1u : 0u);
      }
      tc::commit(&sm.mbar[buf]);
    }
  }
  const int n = ce - cb;
  if (ok && n > 0) ok = tc::mbar_wait(&sm.mbar[(n - 1) & 1], ((n - 1) >> 1) & 1, kWaitLimit) ? 1 : 0;
  ok = __syncthreads_and(ok);
  tc::fence_after_sync();
  if (ok && n > 0) {
    float *SL = reinterpret_cast<float *>(wv.SL) + pv.p_S_off[b];
    const int row = row0 + 32 * warp + lane;
    for (int cc = 0; cc < ncols; cc += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)cc, v);
      if (row < P) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int col = col0 + cc + i;
          if (col < P && col <= row && v[i] != 0.f) red_add(SL + (size_t)row * P + col, v[i]);
        }
      }
    }
  } else if (!ok) {
    // a wait ran out: flag the problem, give the in-flight MMAs a last bounded wait
    if (tid == 0) wv.lm[b].fail = 1;
    for (int q = 0; q < 2; ++q) (void)tc::mbar_wait(&sm.mbar[q], 0, kWaitLimit);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols_alloc);
}

// g_L(rows of the chunk) += sum_k slab[row][k] g_a,k / D_k   (one CTA per chunk)
template <typename T>
__global__ void k_schur_g(PlanView pv, WorkView wv, Params prm, int gate) {
  __shared__ T dg[SPGO_CHUNK];
  const int c = blockIdx.x;
  const int b = pv.ch_prob[c];
  if (!problem_active(wv.lm, b, gate)) return;
  const int f0 = pv.ch_f0[c], nb = pv.ch_nb[c], lm0 = pv.ch_lm0[c], cnt = pv.ch_cnt[c];
  const double lam1 = 1.0 + wv.lm[b].lam;
  if (threadIdx.x < SPGO_CHUNK) {
    const int k = threadIdx.x;
    dg[k] = k < cnt ? (T)((double)reinterpret_cast<const T *>(wv.ga)[lm0 + k] /
                          ((double)reinterpret_cast<const T *>(wv.C)[lm0 + k] * lam1 + (double)prm.eps))
                    : T(0);
  }
  __syncthreads();
  const T *slab = reinterpret_cast<const T *>(wv.slab) + pv.ch_slab[c];
  T *gL = reinterpret_cast<T *>(wv.gL) + pv.p_param_off[b] + 6 * f0;
  for (int row = threadIdx.x; row < 6 * nb; row += blockDim.x) {
    T s = T(0);
#pragma unroll 8
    for (int k = 0; k < SPGO_CHUNK; ++k) s += slab[(size_t)row * SPGO_CHUNK + k] * dg[k];
    if (s != T(0)) red_add(gL + row, s);
  }
}

size_t tc_smem_bytes() { return sizeof(TcSmem) + 1024; }

int launch_schur_tc(const PlanView &pv, const WorkView &wv, const Params &prm, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (pv.n_tc_items > 0) {
    const size_t sm = tc_smem_bytes();
    cudaFuncSetAttribute(k_schur_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_schur_tc<<<pv.n_tc_items, 128, sm, st>>>(pv, wv, prm, GATE_RUNNING);
    ++g_launches;
  }
  if (pv.n_chunks > 0) {
    k_schur_g<float><<<pv.n_chunks, 128, 0, st>>>(pv, wv, prm, GATE_RUNNING);
    ++g_launches;
  }
  return (int)cudaGetLastError();
}

}  // namespace spgo
