// Landmark Schur complement on the 5th-generation tensor cores (mixed path).
//
//   S_L = sum_l B_l B_l^T / (C_l (1 + lam) + eps)       (W D^-1 W^T)
//
// replaces the reference's B C^-1 B^T cuBLAS SGEMM over a dense P x L matrix
// (src/Optimization/Solver_cuda.cu:690-699).  The landmark-chunk slabs written by
// the linearisation are already K-major operands: rows = pose parameters,
// K = the chunk's 32 landmarks.  With s_k = D_k^-1/2 both operands are the same
// scaled slab rows, X = W diag(s), and S_L = X X^T.
//
// One CTA per work item = (problem, 128 x 128 output tile of the lower triangle,
// <= 64 chunks whose rows meet the tile), warp-specialised, all hand-offs on
// mbarriers:
//   warp 9     copy: 1-D bulk copies (cp.async.bulk) of the chunk's slab rows that
//              fall in the tile's row range (and column range, off the diagonal)
//              plus a 16-byte aligned superset of its C values, into a 3-slot ring;
//   warps 0-3  transform: scale by s_k and split each value into TF32 parts,
//              x = hi + lo (hi rounded to 10 mantissa bits, lo = x - hi rounded
//              again), written in the no-swizzle K-major core-matrix layout into
//              a double-buffered operand stage (zero rows outside the chunk);
//              on diagonal tiles they also accumulate the g-side term
//              g_L(row) += sum_k x_k (g_a,k s_k) = sum_k W_k g_a,k / D_k;
//   warp 8     one thread issues 3 x 4 kind::tf32 MMAs per chunk (hi.hi + hi.lo +
//              lo.hi, K = 8 each) into one of two 128-lane x 128-column FP32 TMEM
//              accumulators, trimming N to the chunk's last column;
//   warps 4-7  every 4 chunks read the finished accumulator with tcgen05.ld and
//              add it into FP32 registers (one tile row per thread), then stage
//              the tile in shared memory and add its lower triangle into S_L with
//              coalesced reductions.
// The split product carries ~21 mantissa bits.  Reading the accumulator back
// every 4 chunks keeps the tensor core's own accumulation short: accumulating a
// whole chunk list in TMEM loses ~25x more than FP32 SIMT on wide problems,
// which the reduced system S = A - S_L, cancelling most of A, would expose.
// Every wait is bounded by the global timer; a timeout sets the problem's
// failure flag, lets the copies and MMAs in flight finish, frees TMEM and returns.
//
// (The SIMT Schur path in k_system.cu forms g_L the same way inside its tiles.)
#include "kernels.cuh"
#include "tc.cuh"

namespace spgo {

constexpr int kTcTile = 128;
constexpr int kTcK = SPGO_CHUNK;  // 32 landmarks per chunk
constexpr int kRawSlots = 3;
constexpr int kOpStages = 2;
constexpr int kGroup = 4;           // chunks accumulated in TMEM between readbacks
constexpr int kTcThreads = 320;     // 10 warps, roles above
constexpr int kTcMaxChunks = SPGO_TC_SPLIT;  // the planner's split
constexpr uint64_t kTimeoutNs = 2000000000ull;

struct OpStage {                    // 64 KB, 1024-byte aligned
  float xh[kTcTile * kTcK];
  float xl[kTcTile * kTcK];
  float yh[kTcTile * kTcK];
  float yl[kTcTile * kTcK];
};

struct RawSlot {                    // 33,024 bytes (16-byte multiple)
  float x[kTcTile * kTcK];          // tile-row slab rows [xr0, xr1), row-major
  float y[kTcTile * kTcK];          // tile-column slab rows [yr0, yr1)
  float c[36];                      // C[cstart .. cstart + 36), cstart = lm0 & ~3
  float ga[36];                     // g_a over the same range
  int32_t s1, cnt, coff, xr0, xr1, yr0, yr1, pad[9];
};

struct TcSmem {
  OpStage op[kOpStages];
  RawSlot raw[kRawSlots];
  float sk[2][kTcK];
  float gs[2][kTcK];                // g_a,k s_k of the chunk being split (diagonal tiles)
  int32_t op_ncols[kOpStages];
  uint64_t raw_full[kRawSlots], raw_empty[kRawSlots], op_full[kOpStages], op_empty[kOpStages];
  uint64_t acc_full[2], acc_empty[2], fin;
  uint32_t tmem_slot;
  int err;
  int zero;  // never set: waits that must not be cut short by an error
};
static_assert(sizeof(OpStage) % 1024 == 0, "operand stage alignment");
static_assert(sizeof(RawSlot) % 16 == 0, "raw slot alignment");
static_assert(sizeof(TcSmem) + 1024 <= 232448, "fits the 227 KB opt-in shared memory");

// scale one slab row (or zeros) by s and write its hi/lo parts as row r of an
// operand in core-matrix layout; piece order rotated by r (bank-conflict free).
// With gs != nullptr also returns sum_k x_k gs_k.
__device__ __forceinline__ float split_row(const float *src, bool valid, const float *s, const float *gs, int r,
                                           float *h, float *l) {
  float gacc = 0.f;
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const int kq = (m + r) & 7;
    float4 v = valid ? *reinterpret_cast<const float4 *>(src + 4 * kq) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float x[4] = {v.x * s[4 * kq], v.y * s[4 * kq + 1], v.z * s[4 * kq + 2], v.w * s[4 * kq + 3]};
    if (gs) gacc += x[0] * gs[4 * kq] + x[1] * gs[4 * kq + 1] + x[2] * gs[4 * kq + 2] + x[3] * gs[4 * kq + 3];
    float hi[4], lo[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      hi[i] = tc::tf32_round(x[i]);
      lo[i] = tc::tf32_round(x[i] - hi[i]);
    }
    const uint32_t off = tc::kmajor_offset(r, 4 * kq);
    *reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(h) + off) = make_float4(hi[0], hi[1], hi[2], hi[3]);
    *reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(l) + off) = make_float4(lo[0], lo[1], lo[2], lo[3]);
  }
  return gacc;
}


__global__ void __launch_bounds__(kTcThreads, 1) k_schur_tc(PlanView pv, WorkView wv, Params prm, int gate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char *base = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  TcSmem &sm = *reinterpret_cast<TcSmem *>(base);
  const int w = blockIdx.x;
  const int b = pv.tc_prob[w];
  if (!problem_active(wv.lm, b, gate)) return;
  const int row0 = pv.tc_row0[w], col0 = pv.tc_col0[w], ncols = pv.tc_ncols[w];
  const bool diag = row0 == col0;
  const int P = 6 * pv.p_npose[b];
  const int cb = pv.tc_cbeg[w], n = min(pv.tc_cend[w] - cb, kTcMaxChunks);
  const int ngroups = (n + kGroup - 1) / kGroup;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  volatile int *err = &sm.err;
  if (tid == 0) {
    for (int i = 0; i < kRawSlots; ++i) {
      tc::mbar_init(&sm.raw_full[i], 1);
      tc::mbar_init(&sm.raw_empty[i], 128);
    }
    for (int i = 0; i < kOpStages; ++i) {
      tc::mbar_init(&sm.op_full[i], 128);
      tc::mbar_init(&sm.op_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&sm.acc_full[i], 1);
      tc::mbar_init(&sm.acc_empty[i], 128);
    }
    tc::mbar_init(&sm.fin, 1);
    sm.err = 0;
    sm.zero = 0;
    tc::mbar_init_fence();
  }
  if (warp == 8) tc::tmem_alloc(&sm.tmem_slot, 256);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = sm.tmem_slot;
  // the waits of the pipeline give up at `deadline` (the parameter's limit); the drains
  // of copies and MMAs already issued keep their own 2 s beyond it, so a CTA that gave
  // up never exits with asynchronous work in flight
  const uint64_t deadline = tc::globaltimer_ns() + wait_limit_ns(prm);
  float acc[kTcTile];  // warps 4-7: one tile row per thread

  if (warp == 9) {
    // ---- copy warp ----
    if (lane == 0) {
      const float *slab_all = reinterpret_cast<const float *>(wv.slab);
      const float *Cv = reinterpret_cast<const float *>(wv.C);
      const float *Gv = reinterpret_cast<const float *>(wv.ga);
      int issued = 0;
      for (int i = 0; i < n; ++i) {
        const int r = i % kRawSlots, u = i / kRawSlots;
        if (u >= 1 && !tc::mbar_wait_until(&sm.raw_empty[r], (u - 1) & 1, deadline, err)) {
          *err = 1;
          break;
        }
        const int c = pv.tc_chunks[cb + i];
        const int s0 = 6 * pv.ch_f0[c], s1 = 6 * (pv.ch_f0[c] + pv.ch_nb[c]);
        const int lm0 = pv.ch_lm0[c];
        const float *slab = slab_all + pv.ch_slab[c];
        RawSlot &R = sm.raw[r];
        const int xr0 = max(s0, row0), xr1 = min(s1, row0 + kTcTile);
        const int yr0 = max(s0, col0), yr1 = min(s1, col0 + ncols);
        const int cstart = lm0 & ~3;
        R.s1 = s1;
        R.cnt = pv.ch_cnt[c];
        R.coff = lm0 - cstart;
        R.xr0 = xr0;
        R.xr1 = xr1;
        R.yr0 = yr0;
        R.yr1 = yr1;
        const uint32_t bx = xr1 > xr0 ? (uint32_t)(xr1 - xr0) * kTcK * 4 : 0u;
        const uint32_t by = (!diag && yr1 > yr0) ? (uint32_t)(yr1 - yr0) * kTcK * 4 : 0u;
        tc::mbar_arrive_expect_tx(&sm.raw_full[r], bx + by + (diag ? 288u : 144u));
        if (bx) tc::bulk_g2s(R.x, slab + (size_t)(xr0 - s0) * kTcK, bx, &sm.raw_full[r]);
        if (by) tc::bulk_g2s(R.y, slab + (size_t)(yr0 - s0) * kTcK, by, &sm.raw_full[r]);
        tc::bulk_g2s(R.c, Cv + cstart, 144u, &sm.raw_full[r]);
        if (diag) tc::bulk_g2s(R.ga, Gv + cstart, 144u, &sm.raw_full[r]);
        issued = i + 1;
      }
      // let every copy in flight land before the CTA can exit
      for (int i = max(0, issued - kRawSlots); i < issued; ++i)
        (void)tc::mbar_wait_until(&sm.raw_full[i % kRawSlots], (i / kRawSlots) & 1, deadline + kTimeoutNs,
                                  &sm.zero);
    }
  } else if (warp < 4) {
    // ---- transform warps ----
    const float lam1 = (float)(1.0 + wv.lm[b].lam);
    const float eps = prm.eps;
    float gl = 0.f;  // g_L of tile row tid (diagonal tiles)
    bool done = true;
    for (int i = 0; i < n; ++i) {
      const int r = i % kRawSlots, u = i / kRawSlots, o = i % kOpStages, uo = i / kOpStages;
      bool ok = tc::mbar_wait_until(&sm.raw_full[r], u & 1, deadline, err);
      if (ok && uo >= 1) ok = tc::mbar_wait_until(&sm.op_empty[o], (uo - 1) & 1, deadline, err);
      if (!ok) *err = 1;
      const RawSlot &R = sm.raw[r];
      float *sk = sm.sk[i & 1];
      float *gs = sm.gs[i & 1];
      if (warp == 0) {
        const float sv = lane < R.cnt ? rsqrtf(R.c[R.coff + lane] * lam1 + eps) : 0.f;
        sk[lane] = sv;
        if (diag) gs[lane] = lane < R.cnt ? R.ga[R.coff + lane] * sv : 0.f;
      }
      named_sync(1, 128);
      if (*err) {
        done = false;
        break;
      }
      const int n_eff = (i % kGroup == 0) ? ncols : min(ncols, ((R.s1 - col0 + 15) / 16) * 16);
      if (tid == 0) sm.op_ncols[o] = n_eff;
      OpStage &S = sm.op[o];
      const int t = tid;  // tile row (and column row) of this thread
      {
        const int gr = row0 + t;
        const bool v = gr >= R.xr0 && gr < R.xr1;
        gl += split_row(R.x + (size_t)(v ? gr - R.xr0 : 0) * kTcK, v, sk, diag ? gs : nullptr, t, S.xh, S.xl);
      }
      if (!diag && t < n_eff) {
        const int gc = col0 + t;
        const bool v = gc >= R.yr0 && gc < R.yr1;
        (void)split_row(R.y + (size_t)(v ? gc - R.yr0 : 0) * kTcK, v, sk, nullptr, t, S.yh, S.yl);
      }
      tc::fence_proxy_async();
      tc::mbar_arrive(&sm.op_full[o]);
      tc::mbar_arrive(&sm.raw_empty[r]);
    }
    if (diag && done && row0 + tid < P && gl != 0.f)
      red_add(reinterpret_cast<float *>(wv.gL) + pv.p_param_off[b] + row0 + tid, gl);
  } else if (warp == 8) {
    // ---- MMA issue ----
    if (lane == 0) {
      for (int i = 0; i < n; ++i) {
        const int o = i % kOpStages, uo = i / kOpStages;
        const int j = i / kGroup, a = j & 1;
        const bool first = i % kGroup == 0;
        if (first && j >= 2 && !tc::mbar_wait_until(&sm.acc_empty[a], ((j >> 1) - 1) & 1, deadline, err)) {
          *err = 1;
          break;
        }
        if (!tc::mbar_wait_until(&sm.op_full[o], uo & 1, deadline, err)) {
          *err = 1;
          break;
        }
        tc::fence_after_sync();
        const uint32_t idesc = tc::idesc_tf32(kTcTile, sm.op_ncols[o]);
        const OpStage &S = sm.op[o];
        const uint32_t xh = tc::smem_u32(S.xh), xl = tc::smem_u32(S.xl);
        const uint32_t yh = diag ? xh : tc::smem_u32(S.yh), yl = diag ? xl : tc::smem_u32(S.yl);
        const uint32_t d = tmem + (uint32_t)(a * kTcTile);
#pragma unroll
        for (int ks = 0; ks < kTcK / 8; ++ks) {
          const uint32_t off = ks * 256;
          tc::mma_tf32(d, tc::smem_desc(xh + off, 128, 1024), tc::smem_desc(yh + off, 128, 1024), idesc,
                       (first && ks == 0) ? 0u : 1u);
          tc::mma_tf32(d, tc::smem_desc(xh + off, 128, 1024), tc::smem_desc(yl + off, 128, 1024), idesc, 1u);
          tc::mma_tf32(d, tc::smem_desc(xl + off, 128, 1024), tc::smem_desc(yh + off, 128, 1024), idesc, 1u);
        }
        tc::commit(&sm.op_empty[o]);
        if (i % kGroup == kGroup - 1 || i == n - 1) tc::commit(&sm.acc_full[a]);
      }
      // every MMA issued has completed once this commit arrives
      tc::commit(&sm.fin);
      (void)tc::mbar_wait_until(&sm.fin, 0, deadline + kTimeoutNs, &sm.zero);
    }
  } else {
    // ---- accumulator warps 4-7 ----
    const int q = warp - 4;
#pragma unroll
    for (int c = 0; c < kTcTile; ++c) acc[c] = 0.f;
    for (int j = 0; j < ngroups; ++j) {
      const int a = j & 1;
      if (!tc::mbar_wait_until(&sm.acc_full[a], (j >> 1) & 1, deadline, err)) {
        *err = 1;
        break;
      }
      tc::fence_after_sync();
#pragma unroll
      for (int cc = 0; cc < kTcTile / 32; ++cc) {
        if (32 * cc < ncols) {
          uint32_t v[32];
          tc::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(a * kTcTile + 32 * cc), v);
          tc::tmem_wait_ld();
#pragma unroll
          for (int k = 0; k < 32; ++k) acc[32 * cc + k] += __uint_as_float(v[k]);
        }
      }
      tc::fence_before_sync();
      tc::mbar_arrive(&sm.acc_empty[a]);
    }
  }

  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const bool failed = sm.err != 0;
  if (!failed && warp >= 4 && warp < 8 && n > 0) {
    // stage the tile (row stride 129 floats: conflict-free) in the free operand
    // buffers, then add its lower triangle into S_L with coalesced reductions
    float *st = reinterpret_cast<float *>(sm.op);
    const int q = warp - 4, row = 32 * q + lane;
#pragma unroll
    for (int c = 0; c < kTcTile; ++c)
      if (c < ncols) st[row * (kTcTile + 1) + c] = acc[c];
    named_sync(2, 128);
    float *SL = reinterpret_cast<float *>(wv.SL) + pv.p_S_off[b];
    for (int rr = 32 * q; rr < 32 * q + 32; ++rr) {
      const int grow = row0 + rr;
      if (grow >= P) break;
      for (int c = lane; c < ncols; c += 32) {
        const int gcol = col0 + c;
        const float v = st[rr * (kTcTile + 1) + c];
        if (gcol < P && gcol <= grow && v != 0.f) red_add(SL + (size_t)grow * P + gcol, v);
      }
    }
  }
  if (failed && tid == 0) atomicOr(&wv.lm[b].fail, FAIL_TIMEOUT);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 8) tc::tmem_dealloc(tmem, 256);
}

size_t tc_smem_bytes() { return sizeof(TcSmem) + 1024; }

int launch_schur_tc(const PlanView &pv, const WorkView &wv, const Params &prm, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (pv.n_tc_items > 0) {
    const size_t sm = tc_smem_bytes();
    cudaFuncSetAttribute(k_schur_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_schur_tc<<<pv.n_tc_items, kTcThreads, sm, st>>>(pv, wv, prm, GATE_RUNNING);
    ++g_launches;
  }
  return (int)cudaGetLastError();
}

}  // namespace spgo
