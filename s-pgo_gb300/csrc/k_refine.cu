// Iterative refinement of the mixed path's LM step.
//
// The FP32 reduced system (pose Hessian from FP32 pair sums, tensor-core Schur
// complement, FP32 Cholesky) gives a step whose error, on the ill-conditioned
// systems of the circle scenes, reaches 1e-3 relative.  Such steps do not change
// where LM converges, but they change where it is after a fixed iteration budget,
// and the accepted cost then differs from the FP64 solver's by far more than the
// 1e-6 the solvers are compared at.  The cause is the accumulation of the normal
// equations (the sums over observations and landmarks, which cancel in S = A -
// W D^-1 W^T and in the gradient), not the FP32 Jacobian itself.
//
// So the FP32 system only preconditions.  Each refinement step forms the
// residual of the whole damped system
//   r_p = J_p^T W (r - J x) - lam diag(A) x_p,   r_a = J_a^T W (r - J x) - (lam C + eps) x_a
// from the FP32 Jacobian, recomputed per observation, with every product J e
// exact (two-product) and every sum in double-float / FP64, then applies the FP32
// system's inverse: x_p += S^-1 (r_p - W D^-1 r_a), x_a += D^-1 (r_a - W^T dx_p).
// The first residual pass also sums the accurate gradient J^T W r, which the
// predicted decrease of the gain ratio uses.
//
//   k_pair_twists     per problem: the world twist of every pose pair's poses,
//                     W(lo, hi) = sum_{i in [lo, hi)} Ad_i x_i about c_lo (FP64 sums,
//                     stored FP32), so J_o x_p = s_o K_o W(lo, hi) per observation
//   k_resid_pass      per landmark chunk: the inverse-depth step of the chunk's
//                     landmarks, then one thread per observation: e = r - J x and its
//                     dual s K^T W e (pair records, FP64 atomics per run of equal
//                     target frame) and j_a^T W e (per landmark, FP64); then
//                     t = D^-1 r_a and W t into the pose right-hand side
//   k_resid_solve     per problem: the pair records reduced to per-pose vectors
//                     (FP64), the right-hand side, and the solve with the stored FP32
//                     factor; systems too wide for one CTA take the same reduction
//                     from k_rs_sums_large, k_rs_scan_large and k_rs_rhs_large (spread
//                     over the GPU) and the multi-CTA substitutions of k_chol_large.cu
//   k_backsub_refined per chunk: the last inverse-depth correction, the candidate
//                     inverse depths and their share of the predicted decrease
//
// Replaces nothing in the reference, whose GPU step is an FP32 Gauss-Newton step
// solved once (src/Optimization/Solver_cuda.cu:594-782, linear_solvers.cu:195-218).
#include "kernels.cuh"
#include "frames.cuh"
#include "dfloat.cuh"
#include "chol_subst.cuh"

namespace spgo {

// a b + c d exactly rounded to a double-float
__device__ __forceinline__ df prod2(float a, float b, float c, float d) {
  const df p = two_prod(a, b), q = two_prod(c, d);
  df s = two_sum(p.h, q.h);
  s.l += p.l + q.l;
  return fast_two_sum(s.h, s.l);
}

// left camera of frame f: rotation (cam -> world) and centre, FP64 from the
// double-float frame tables of the mixed path
__device__ __forceinline__ void frame_Rc(const WorkView &wv, int f, double *R, double *c) {
  const float *Rh = wv.fr_Rf + (size_t)f * 18, *Rl = wv.fr_Rl + (size_t)f * 18;
#pragma unroll
  for (int k = 0; k < 9; ++k) R[k] = (double)Rh[k] + (double)Rl[k];
#pragma unroll
  for (int k = 0; k < 3; ++k) c[k] = (double)wv.fr_ch[(size_t)f * 6 + k] + (double)wv.fr_cl[(size_t)f * 6 + k];
}

// a problem takes (the next step of) the refinement: running, its step not failed, and
// its refinement not yet converged (outer_tol)
__device__ __forceinline__ bool refine_active(const WorkView &wv, int b) {
  return problem_active(wv.lm, b, GATE_RUNNING) && !wv.lm[b].fail && !wv.lm[b].ref_done;
}

// ---- pose-pair twists -------------------------------------------------------
// Ad_i x_i = [R_i psi_i ; (c_i - o) x R_i psi_i + R_i rho_i] about origin o (the
// convention of the pose blocks, k_system.cu).  With the prefix sums
// Om(k) = sum_{i<k} R_i psi_i and V(k) = sum_{i<k} c_i x R_i psi_i + R_i rho_i,
// W(lo, hi) = [Om(hi) - Om(lo) ; V(hi) - V(lo) - c_lo x (Om(hi) - Om(lo))].
constexpr int kTwThreads = 128;

__global__ void __launch_bounds__(kTwThreads) k_pair_twists(PlanView pv, WorkView wv) {
  extern __shared__ double tw_s[];  // [(N + 1) * 6]
  const int b = blockIdx.x;
  if (!refine_active(wv, b)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b], fo = pv.p_frame_off[b], po = pv.p_param_off[b];
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double R[9], c[3];
    frame_Rc(wv, fo + i, R, c);
    const double *x = wv.delta + po + 6 * i;
    double w[3], v[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      w[r] = R[3 * r] * x[0] + R[3 * r + 1] * x[1] + R[3 * r + 2] * x[2];
      v[r] = R[3 * r] * x[3] + R[3 * r + 1] * x[4] + R[3 * r + 2] * x[5];
    }
    double *o = tw_s + (size_t)(i + 1) * 6;
    o[0] = w[0];
    o[1] = w[1];
    o[2] = w[2];
    o[3] = v[0] + (c[1] * w[2] - c[2] * w[1]);
    o[4] = v[1] + (c[2] * w[0] - c[0] * w[2]);
    o[5] = v[2] + (c[0] * w[1] - c[1] * w[0]);
  }
  if (threadIdx.x < 6) tw_s[threadIdx.x] = 0.0;
  __syncthreads();
  if (threadIdx.x < 6) {
    double acc = 0.0;
    for (int i = 1; i <= N; ++i) {
      acc += tw_s[i * 6 + threadIdx.x];
      tw_s[i * 6 + threadIdx.x] = acc;
    }
  }
  __syncthreads();
  float *out = wv.twist + (size_t)pv.p_pair_off[b] * 6;
  for (int t = threadIdx.x; t < N * D; t += blockDim.x) {
    const int lo = t / D, hi = lo + t % D + 1;
    if (hi > N) continue;
    double R[9], c[3];
    frame_Rc(wv, fo + lo, R, c);
    double dw[3], dv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      dw[k] = tw_s[hi * 6 + k] - tw_s[lo * 6 + k];
      dv[k] = tw_s[hi * 6 + 3 + k] - tw_s[lo * 6 + 3 + k];
    }
    float *o = out + (size_t)t * 6;
    o[0] = (float)dw[0];
    o[1] = (float)dw[1];
    o[2] = (float)dw[2];
    o[3] = (float)(dv[0] - (c[1] * dw[2] - c[2] * dw[1]));
    o[4] = (float)(dv[1] - (c[2] * dw[0] - c[0] * dw[2]));
    o[5] = (float)(dv[2] - (c[0] * dw[1] - c[1] * dw[0]));
  }
}

int launch_pair_twists(const PlanView &pv, const WorkView &wv, void *stream) {
  const size_t sm = (size_t)(pv.max_P / 6 + 1) * 6 * sizeof(double);
  k_pair_twists<<<pv.B, kTwThreads, sm, (cudaStream_t)stream>>>(pv, wv);
  ++g_launches;
  return (int)cudaGetLastError();
}

// ---- residual pass ------------------------------------------------------------
constexpr int kRpThreads = 128;
constexpr int kRpWarps = kRpThreads / 32;
constexpr int kRpPitch = 33;

struct RefSmem {
  float X[SPGO_CHUNK][3];   // anchor point, world axes, relative to the anchor centre
  float dX[SPGO_CHUNK][3];  // dX / d alpha
  float da[SPGO_CHUNK];     // inverse-depth step (FP32 copy for the residuals)
  __align__(16) float t[SPGO_CHUNK];  // D^-1 r_a
  int a[SPGO_CHUNK];
  float dlh[kRpWarps][SPGO_CHUNK];  // j_a^T W e, per warp, double-float (h, l)
  float dll[kRpWarps][SPGO_CHUNK];
  int key[kRpWarps][32];
  float bt[2][SPGO_CHUNK];  // warps 0 and 1: partial W^T x_p over their slab row blocks
};

// dynamic shared memory (W = window frames): the window's rotations [W][18] (both
// cameras) | the pair origins' offsets [W][4] | the pair twists [W][6] | the per-warp
// staging [warps][2 x 6][33] float of the pair duals
struct RpLayout {
  size_t rw, xpo, tws, stage, total;
  __host__ __device__ explicit RpLayout(int max_nb) {
    const size_t W = (size_t)max_nb + 1;
    auto up = [](size_t x) { return (x + 15) & ~(size_t)15; };
    rw = 0;
    xpo = rw + up(W * 18 * sizeof(float));
    tws = xpo + up(W * 4 * sizeof(float));
    stage = tws + up(W * 6 * sizeof(float));
    total = stage + (size_t)kRpWarps * 2 * 6 * kRpPitch * sizeof(float);
  }
};

// The accurate gradient itself (J^T W r, pose and inverse-depth parts) comes from the
// linearisation, which sums it exactly (k_linearize.cu, k_system.cu); each pass here
// forms only the duals of e.
template <bool FIRST>
__global__ void __launch_bounds__(kRpThreads, 8) k_resid_pass(PlanView pv, WorkView wv, Params prm,
                                                           const double *__restrict__ alpha_state) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ RefSmem sm;
  const int c = blockIdx.x;
  const int b = pv.ch_prob[c];
  if (!refine_active(wv, b)) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int f0 = pv.ch_f0[c], nb = pv.ch_nb[c], lm0 = pv.ch_lm0[c], cnt = pv.ch_cnt[c];
  const int fo = pv.p_frame_off[b], po = pv.p_param_off[b];
  const float *intr = pv.p_intr + 8 * b;
  const float fxs[2] = {intr[0], intr[4]}, fys[2] = {intr[1], intr[5]};
  const double lam = wv.lm[b].lam;
  const float eps = prm.eps;
  {
    // the chunk's observation records (slot, frame, residuals) towards L2 while the
    // prologue runs: one prefetch per 128-byte line
    const int64_t ob0 = pv.lm_obs[lm0], oe0 = pv.lm_obs[lm0 + cnt];
    const float *res0 = wv.res + (size_t)wv.lm[b].res_sel * (size_t)pv.O * 4;
    const int nres = (int)(((oe0 - ob0) * 16 + 127) / 128), nfr = (int)(((oe0 - ob0) * 4 + 127) / 128);
    for (int k = tid; k < nres + nfr; k += blockDim.x) {
      const void *a = k < nres ? (const void *)(reinterpret_cast<const char *>(res0 + 4 * ob0) + 128 * k)
                               : (const void *)(reinterpret_cast<const char *>(pv.obs_frame + ob0) + 128 * (k - nres));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
    }
  }
  const RpLayout lay(pv.max_nb);
  float *Rw = reinterpret_cast<float *>(smem_raw + lay.rw);
  float *xpo = reinterpret_cast<float *>(smem_raw + lay.xpo);
  float *tws = reinterpret_cast<float *>(smem_raw + lay.tws);
  float *stage = reinterpret_cast<float *>(smem_raw + lay.stage);
  const int D = pv.p_pair_D[b];
  const float *slab = reinterpret_cast<const float *>(wv.slab) + pv.ch_slab[c];
  const float *Cv = reinterpret_cast<const float *>(wv.C);
  const int rows = 6 * nb;

  if (warp < 2) {
    // inverse-depth step: first pass x_a = D^-1 (g_a - W^T x_p) from the FP32 system,
    // later x_a += t - D^-1 W^T dx_p (the previous pass's t and pose correction); warps
    // 0 and 1 take alternate 32-row blocks of the slab for W^T x_p
    const double *v = (FIRST ? wv.delta : wv.ddelta) + po + 6 * f0;
    float s0 = 0.f, s1 = 0.f;
    for (int rb = 32 * warp; rb < rows; rb += 64) {
      const float dv = rb + lane < rows ? (float)v[rb + lane] : 0.f;
      const float *sr = slab + (size_t)rb * SPGO_CHUNK + lane;
      const int nr = min(32, rows - rb);
      float q[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) q[k] = k < nr ? sr[(size_t)k * SPGO_CHUNK] : 0.f;
#pragma unroll
      for (int k = 0; k < 32; k += 2) {
        s0 += q[k] * __shfl_sync(0xffffffffu, dv, k);
        s1 += q[k + 1] * __shfl_sync(0xffffffffu, dv, k + 1);
      }
    }
    sm.bt[warp][lane] = s0 + s1;
  }
  if (warp == 0) {
    // the chunk's anchor points, as the cost pass at this state formed them (the same
    // points the linearisation used)
    if (lane < cnt) {
      const int li = lm0 + lane;
      const float4 *xa = reinterpret_cast<const float4 *>(wv.xanc + ((size_t)wv.lm[b].res_sel * pv.L + li) * 8);
      const float4 x0 = xa[0], x1 = xa[1];
      sm.X[lane][0] = x0.x;
      sm.X[lane][1] = x0.y;
      sm.X[lane][2] = x0.z;
      sm.dX[lane][0] = x0.w;
      sm.dX[lane][1] = x1.x;
      sm.dX[lane][2] = x1.y;
      sm.a[lane] = pv.lm_host[li];
    }
#pragma unroll
    for (int w = 0; w < kRpWarps; ++w) sm.dlh[w][lane] = sm.dll[w][lane] = 0.f;
  }
  if (warp < 2) named_sync(1, 64);  // both partial sums written
  if (warp == 1) {
    if (lane < cnt) {
      const int li = lm0 + lane;
      const float C = Cv[li];
      const float Dd = C * (float)(1.0 + lam) + eps;
      const float s = sm.bt[0][lane] + sm.bt[1][lane];
      double da;
      if (FIRST)
        da = (double)((reinterpret_cast<const float *>(wv.ga)[li] - s) / Dd);
      else
        da = wv.dal[li] + (double)(wv.tl[li] - s / Dd);
      wv.dal[li] = da;
      sm.da[lane] = (float)da;
    }
  } else if (warp >= 2) {
    // the window's rotations, and per window frame n the offset c_a - c_n of the pair
    // origin (n < a) and the twist of the pair (a, n)
    const int ah = pv.lm_host[lm0], fh = fo + ah;
    for (int idx = tid - 64; idx < (nb + 1) * 18; idx += blockDim.x - 64)
      Rw[idx] = wv.fr_Rf[(size_t)(fo + f0) * 18 + idx];
    for (int f = tid - 64; f < nb + 1; f += blockDim.x - 64) {
      const int n = f0 + f;
      Vec3<float> d = v3<float>(0.f, 0.f, 0.f);
      if (n < ah) d = FramesT<float>::rel(wv, fh, 0, fo + n, 0);
      xpo[4 * f] = d.x;
      xpo[4 * f + 1] = d.y;
      xpo[4 * f + 2] = d.z;
      const int lo = min(ah, n), hi = max(ah, n);
      float t6v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (hi > lo && hi - lo <= D) {  // a pair that observations of this chunk can form
        const float *tw = wv.twist + ((size_t)pv.p_pair_off[b] + (size_t)lo * D + (hi - lo - 1)) * 6;
#pragma unroll
        for (int k = 0; k < 6; ++k) t6v[k] = tw[k];
      }
#pragma unroll
      for (int k = 0; k < 6; ++k) tws[6 * f + k] = t6v[k];
    }
  }
  __syncthreads();

  const int64_t ob = pv.lm_obs[lm0], oe = pv.lm_obs[lm0 + cnt];
  const float lscale = prm.loss_scale;
  // residuals at the linearisation point: the state's half of the residual store
  const float *res_buf = wv.res + (size_t)wv.lm[b].res_sel * (size_t)pv.O * 4;
  const float *tcam_buf = wv.tcam + (size_t)wv.lm[b].res_sel * (size_t)pv.O * 6;
  for (int64_t base = ob + (tid & ~31); base < oe; base += blockDim.x) {
    const int64_t o = base + lane;
    // this observation's pose rows s K of both cameras (zero without a pose term), its
    // inverse-depth rows, and the weighted linearised residuals w^2 e; each dual is
    // then formed once as the exact sum of its four products
    float K[2][2][6], JA[2][2], EW[2][2];
#pragma unroll
    for (int c2 = 0; c2 < 2; ++c2)
#pragma unroll
      for (int r2 = 0; r2 < 2; ++r2) {
        JA[c2][r2] = EW[c2][r2] = 0.f;
#pragma unroll
        for (int k = 0; k < 6; ++k) K[c2][r2][k] = 0.f;
      }
    int key = -1, slot = -1;
    if (o < oe) {
      slot = pv.obs_slot[o];
      const int n = pv.obs_frame[o];
      const float4 rl = reinterpret_cast<const float4 *>(res_buf)[o];
      const int a = sm.a[slot];
      const int fw = n - f0;
      const bool has_pose = n != a;
      const float sgn = n > a ? 1.f : -1.f;
      const float boost = (prm.near_boost && abs(n - a) < 2) ? 16.f : 1.f;
      const float da = sm.da[slot];
      const Vec3<float> X = v3<float>(sm.X[slot][0], sm.X[slot][1], sm.X[slot][2]);
      const Vec3<float> dXda = v3<float>(sm.dX[slot][0], sm.dX[slot][1], sm.dX[slot][2]);
      // point relative to the pair origin (the left centre of frame min(a, n)), the
      // pair's twist (zero without a pose term)
      const Vec3<float> Xp = v3<float>(X.x + xpo[4 * fw], X.y + xpo[4 * fw + 1], X.z + xpo[4 * fw + 2]);
      float W[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) W[k] = tws[6 * fw + k];
      const float2 *tp = reinterpret_cast<const float2 *>(tcam_buf + (size_t)o * 6);
      const float2 t01 = tp[0], t23 = tp[1], t45 = tp[2];
#pragma unroll
      for (int cam = 0; cam < 2; ++cam) {
        // the camera-frame point as the cost pass at the state formed it (double-float,
        // rounded once): the same Jacobian the linearisation used
        const float *Rn = Rw + fw * 18 + cam * 9;
        const Vec3<float> t = cam ? v3<float>(t23.y, t45.x, t45.y) : v3<float>(t01.x, t01.y, t23.x);
        const float r0 = cam ? rl.z : rl.x, r1 = cam ? rl.w : rl.y;
        float rho;
        const float w2 = boost * robust<float>(prm.loss, lscale, r0 * r0 + r1 * r1, rho);
        const float fx = fxs[cam], fy = fys[cam], iz = 1.f / t.z;
        const float j00 = fx * iz, j02 = -fx * t.x * iz * iz, j11 = fy * iz, j12 = -fy * t.y * iz * iz;
        const Vec3<float> u0 = v3<float>(j00 * Rn[0] + j02 * Rn[2], j00 * Rn[3] + j02 * Rn[5], j00 * Rn[6] + j02 * Rn[8]);
        const Vec3<float> u1 = v3<float>(j11 * Rn[1] + j12 * Rn[2], j11 * Rn[4] + j12 * Rn[5], j11 * Rn[7] + j12 * Rn[8]);
        const float ja0 = dot(u0, dXda), ja1 = dot(u1, dXda);
        float e0 = r0 - ja0 * da, e1 = r1 - ja1 * da;
        if (has_pose) {
          const Vec3<float> k0 = cross(Xp, u0), k1 = cross(Xp, u1);
          K[cam][0][0] = sgn * k0.x; K[cam][0][1] = sgn * k0.y; K[cam][0][2] = sgn * k0.z;
          K[cam][0][3] = sgn * u0.x; K[cam][0][4] = sgn * u0.y; K[cam][0][5] = sgn * u0.z;
          K[cam][1][0] = sgn * k1.x; K[cam][1][1] = sgn * k1.y; K[cam][1][2] = sgn * k1.z;
          K[cam][1][3] = sgn * u1.x; K[cam][1][4] = sgn * u1.y; K[cam][1][5] = sgn * u1.z;
          float jw0 = 0.f, jw1 = 0.f;
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            jw0 += K[cam][0][k] * W[k];
            jw1 += K[cam][1][k] * W[k];
          }
          e0 -= jw0;
          e1 -= jw1;
        }
        JA[cam][0] = ja0;
        JA[cam][1] = ja1;
        EW[cam][0] = w2 * e0;
        EW[cam][1] = w2 * e1;
      }
      if (has_pose) key = n;
    }
    const df vle =  // this observation's landmark dual
        slot >= 0 ? sum4_prod(JA[0][0], EW[0][0], JA[0][1], EW[0][1], JA[1][0], EW[1][0], JA[1][1], EW[1][1])
                  : df_make(0.f);
    {
      // the warp's own landmark accumulators: lanes sharing a landmark (different
      // frames) add in rounds of their rank among those peers, no atomics
      const unsigned peers = __match_any_sync(0xffffffffu, slot);
      const int rank = __popc(peers & ((1u << lane) - 1u));
      for (int r = 0; __any_sync(0xffffffffu, slot >= 0 && rank >= r); ++r) {
        if (slot >= 0 && rank == r) {
          df_acc a;
          a.h = sm.dlh[warp][slot];
          a.l = sm.dll[warp][slot];
          a.add(vle.h, vle.l);
          sm.dlh[warp][slot] = a.h;
          sm.dll[warp][slot] = a.l;
        }
        __syncwarp();
      }
    }
    // stage the six pair duals; then 24 lanes, one per (dual, 8-observation segment),
    // each sum their segment's runs of equal target frame and add every run to its
    // pair record (FP64; a run crossing a segment boundary arrives in two parts)
    float *st = stage + (size_t)warp * 2 * 6 * kRpPitch;
    int *keys = sm.key[warp];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const df v = sum4_prod(K[0][0][k], EW[0][0], K[0][1][k], EW[0][1], K[1][0][k], EW[1][0], K[1][1][k], EW[1][1]);
      st[(2 * k) * kRpPitch + lane] = v.h;
      st[(2 * k + 1) * kRpPitch + lane] = v.l;
    }
    keys[lane] = key;
    __syncwarp();
    if (__any_sync(0xffffffffu, key >= 0) && lane < 24) {
      const int host_a = sm.a[0];
      const int v = lane % 6, i0 = (lane / 6) * 8;
      const float *ch = st + (2 * v) * kRpPitch, *cl = st + (2 * v + 1) * kRpPitch;
      double *rec0 = wv.pdual + (size_t)pv.p_pair_off[b] * 6 + v;
      auto emit = [&](int n, const df_acc &a) {
        const int lo = min(host_a, n), hi = max(host_a, n);
        atomicAdd(rec0 + ((size_t)lo * D + (hi - lo - 1)) * 6, df_acc_value(a));
      };
      df_acc acc;
      int cur = keys[i0];
#pragma unroll
      for (int i = i0; i < i0 + 8; ++i) {
        const int k = keys[i];
        if (k != cur) {
          if (cur >= 0) emit(cur, acc);
          acc = df_acc();
          cur = k;
        }
        acc.add(ch[i], cl[i]);
      }
      if (cur >= 0) emit(cur, acc);
    }
    __syncwarp();
  }
  __syncthreads();
  // landmark residuals r_a = j_a^T W e - (lam C + eps) x_a, t = D^-1 r_a
  if (tid < cnt) {
    const int li = lm0 + tid;
    const float C = Cv[li];
    const float Dd = C * (float)(1.0 + lam) + eps;
    df_acc acc;
#pragma unroll
    for (int w = 0; w < kRpWarps; ++w) acc.add(sm.dlh[w][tid], sm.dll[w][tid]);
    const double dsum = df_acc_value(acc);
    const double ra = dsum - (lam * (double)C + (double)eps) * wv.dal[li];  // summed in FP64
    const float t = (float)ra / Dd;  // (t is an FP32 preconditioner term: no FP64 division)
    sm.t[tid] = t;
    wv.tl[li] = t;
  } else if (tid < SPGO_CHUNK) {
    sm.t[tid] = 0.f;
  }
  __syncthreads();
  // W t into the pose right-hand side: thread per slab row, its 32 landmark entries read
  // as eight 16-byte loads (the chunk's slab starts 16-byte aligned, rows are 128 bytes)
  const float4 *t4 = reinterpret_cast<const float4 *>(sm.t);
  for (int r = tid; r < rows; r += blockDim.x) {
    const float4 *sr = reinterpret_cast<const float4 *>(slab + (size_t)r * SPGO_CHUNK);
    float4 x[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = sr[q];
    float v0 = 0.f, v1 = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 t = t4[q];
      v0 += x[q].x * t.x + x[q].y * t.y;
      v1 += x[q].z * t.z + x[q].w * t.w;
    }
    const float v = v0 + v1;
    if (v != 0.f) atomicAdd(wv.rhsB + po + 6 * f0 + r, v);
  }
}

int launch_resid_pass(const PlanView &pv, const WorkView &wv, const Params &prm, const double *alpha, int first,
                      void *stream) {
  if (pv.n_chunks == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t sm = RpLayout(pv.max_nb).total;
  if (first)
    k_resid_pass<true><<<pv.n_chunks, kRpThreads, sm, st>>>(pv, wv, prm, alpha);
  else
    k_resid_pass<false><<<pv.n_chunks, kRpThreads, sm, st>>>(pv, wv, prm, alpha);
  ++g_launches;
  return (int)cudaGetLastError();
}

// ---- pair records -> per-pose right-hand side, and the solve ---------------------
// A record (lo, hi) holds m = [m_w ; m_v] about c_lo; about the world origin it is
// n = [m_w + c_lo x m_v ; m_v].  Pose i collects every record with lo <= i < hi,
// moved to c_i: sum n_w - c_i x sum m_v.  With diff(k) = sum_{lo = k} n - sum_{hi = k} n
// that sum is the prefix sum of diff up to i.  Then r(i) = [R_i^T (.)_w ; R_i^T (.)_v].
// The row sums (fixed lo) re-centre linearly: sum_hi n = sum_hi m_w + c_lo x sum_hi m_v;
// the column sums (fixed hi) take c_lo x m_v per record.  One thread per (row or column,
// component), no atomics.
constexpr int kRsThreads = 256;

// shared memory: centres, row and column sums | cb | y | tmp | the packed factor
// followed by its pivots' reciprocals (as stored by the factorisation)
__host__ __device__ inline size_t rs_layout(int max_Ps, int max_N, size_t *off_cb, size_t *off_y, size_t *off_tmp,
                                            size_t *off_L) {
  auto up = [](size_t x) { return (x + 15) & ~(size_t)15; };
  size_t o = up((size_t)(max_N + 1) * 15 * sizeof(double));  // centres [N+1][3], rows, columns [N+1][6]
  *off_cb = o;
  o = up(o + (size_t)max_Ps * sizeof(int));
  *off_y = o;
  o = up(o + (size_t)max_Ps * sizeof(float));
  *off_tmp = o;
  o = up(o + (size_t)kPanel * sizeof(float));
  *off_L = o;
  o = up(o + ((size_t)max_Ps * (max_Ps + 1) / 2 + max_Ps) * sizeof(float));
  return o;
}

size_t resid_solve_smem(int max_P_small, int max_N) {
  size_t a, b, c, d;
  return rs_layout(max_P_small, max_N, &a, &b, &c, &d);
}

// 16-byte asynchronous global -> shared copies (no registers held while in flight)
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

__global__ void __launch_bounds__(kRsThreads) k_resid_solve(PlanView pv, WorkView wv, float outer_tol) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int b = pv.fs_prob[blockIdx.x];
  if (!refine_active(wv, b)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b], P = 6 * N;
  const int fo = pv.p_frame_off[b], po = pv.p_param_off[b];
  const int tid = threadIdx.x, nt = blockDim.x;
  size_t o_cb, o_y, o_tmp, o_L;
  rs_layout(pv.max_P_small, pv.max_P / 6, &o_cb, &o_y, &o_tmp, &o_L);
  const bool small = P <= pv.max_P_small;
  if (!small && wv.lg_red) return;  // wide problems: the grid-wide kernels below
  const size_t npk = (size_t)P * (P + 1) / 2;
  float *Lm = reinterpret_cast<float *>(smem_raw + o_L);
  if (small) {
    // the stored factor and pivots (contiguous, 16-byte aligned: S offsets are multiples
    // of 36 floats) start copying now and land while the pair duals are reduced
    const float *fac = wv.facs + pv.p_S_off[b];
    const size_t n = npk + P, n4 = n / 4;
    for (size_t k = tid; k < n4; k += nt) cp_async16(Lm + 4 * k, fac + 4 * k);
    for (size_t k = 4 * n4 + tid; k < n; k += nt) Lm[k] = fac[k];
  }
  double *cs = reinterpret_cast<double *>(smem_raw);  // [N + 1][3] left camera centres
  double *rowm = cs + (size_t)(N + 1) * 3;            // [N + 1][6]: sum over hi of m(lo, hi)
  double *colm = rowm + (size_t)(N + 1) * 6;          // [N + 1][6]: sum over lo of n(lo, hi)
  for (int k = tid; k < N * 3; k += nt)
    cs[k] = (double)wv.fr_ch[(size_t)(fo + k / 3) * 6 + k % 3] + (double)wv.fr_cl[(size_t)(fo + k / 3) * 6 + k % 3];
  __syncthreads();
  double *recs = wv.pdual + (size_t)pv.p_pair_off[b] * 6;
  for (int t = tid; t < 12 * N; t += nt) {
    const int k = t % 6;
    if (t < 6 * N) {  // row lo = t / 6
      const int lo = t / 6;
      const double *r = recs + (size_t)lo * D * 6 + k;
      const int nd = min(D, N - lo);
      double acc = 0.0;
#pragma unroll 4
      for (int d = 0; d < nd; ++d) acc += r[(size_t)d * 6];
      rowm[lo * 6 + k] = acc;
    } else {  // column hi = (t - 6 N) / 6 + 1
      const int hi = (t - 6 * N) / 6 + 1;
      double acc = 0.0;
      if (k < 3) {
        const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
#pragma unroll 4
        for (int lo = max(0, hi - D); lo < hi; ++lo) {
          const double *r = recs + ((size_t)lo * D + (hi - lo - 1)) * 6;
          acc += r[k] + (cs[lo * 3 + k1] * r[3 + k2] - cs[lo * 3 + k2] * r[3 + k1]);
        }
      } else {
#pragma unroll 4
        for (int lo = max(0, hi - D); lo < hi; ++lo) acc += recs[((size_t)lo * D + (hi - lo - 1)) * 6 + k];
      }
      colm[hi * 6 + k] = acc;
    }
  }
  if (tid < 6) colm[tid] = 0.0;  // no record ends at pose 0
  __syncthreads();
  for (size_t k = tid; k < (size_t)N * D * 6; k += nt) recs[k] = 0.0;  // cleared for the next pass
  if (tid < 6) {  // prefix sums over the poses; rowm(i) becomes the sum of the records covering pose i
    const int k = tid, k1 = (k + 1) % 3, k2 = (k + 2) % 3;
    double acc = 0.0;
    for (int i = 0; i < N; ++i) {
      const double *c = cs + i * 3;
      const double *m = rowm + i * 6;
      const double nrow = k < 3 ? m[k] + (c[k1] * m[3 + k2] - c[k2] * m[3 + k1]) : m[k];
      acc += nrow - colm[i * 6 + k];
      __syncwarp(0x3fu);
      rowm[i * 6 + k] = acc;  // every lane has read row i's m_v above
    }
  }
  __syncthreads();
  float *y = reinterpret_cast<float *>(smem_raw + o_y);
  const double lam = wv.lm[b].lam;
  const float *A = reinterpret_cast<const float *>(wv.A) + pv.p_S_off[b];
  for (int i = tid; i < N; i += nt) {
    double R[9], ci[3];
    frame_Rc(wv, fo + i, R, ci);
    const double *S = rowm + i * 6;
    const double w[3] = {S[0] - (ci[1] * S[5] - ci[2] * S[4]), S[1] - (ci[2] * S[3] - ci[0] * S[5]),
                         S[2] - (ci[0] * S[4] - ci[1] * S[3])};
    double out[6];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      out[r] = R[r] * w[0] + R[3 + r] * w[1] + R[6 + r] * w[2];
      out[3 + r] = R[r] * S[3] + R[3 + r] * S[4] + R[6 + r] * S[5];
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const int p = 6 * i + k;
      const double x = wv.delta[po + p];
      const double rhs = out[k] - lam * (double)A[(size_t)p * P + p] * x - (double)wv.rhsB[po + p];
      wv.rhsB[po + p] = 0.f;
      if (small)
        y[p] = (float)rhs;
      else
        reinterpret_cast<float *>(wv.lg_y)[po + p] = (float)rhs;
    }
  }
  if (!small) return;  // the multi-CTA substitutions (k_chol_large.cu) follow
  int *cb = reinterpret_cast<int *>(smem_raw + o_cb);
  float *tmp = reinterpret_cast<float *>(smem_raw + o_tmp);
  const float *dinv = Lm + npk;
  for (int k = tid; k < P; k += nt) cb[k] = k * P - (k * (k + 1)) / 2;
  cp_async_wait_all();
  __syncthreads();
  chol_substitute<float>(Lm, cb, y, dinv, tmp, P);
  __shared__ unsigned mx_dx, mx_x;  // largest |correction|, |step| (float bits: non-negative floats order as ints)
  if (tid == 0) mx_dx = mx_x = 0u;
  __syncthreads();
  for (int k = tid; k < P; k += nt) {
    const double dx = (double)y[k];
    const double x = wv.delta[po + k] + dx;
    wv.delta[po + k] = x;
    wv.ddelta[po + k] = dx;
    if (outer_tol > 0.f) {
      atomicMax(&mx_dx, __float_as_uint(fabsf((float)dx)));
      atomicMax(&mx_x, __float_as_uint(fabsf((float)x)));
    }
  }
  __syncthreads();
  // converged: the correction is a small fraction of the step, further steps are skipped
  if (tid == 0 && outer_tol > 0.f && __uint_as_float(mx_dx) <= outer_tol * __uint_as_float(mx_x))
    wv.lm[b].ref_done = 1;
}

// ---- the same reduction for wide problems, spread over the GPU ----------------------
// One CTA per problem puts a wide problem's FP64 pair sums on one SM (GB300 issues FP64
// at 1/64 of its FP32 rate): for P = 3000 that was 267 us per refinement step.  Here
//   k_rs_sums_large   thread per (pose, component): the row sums (over hi) and the
//                     column sums (over lo, moved to c_lo) of the pair duals, into lg_red
//   k_rs_scan_large   one CTA: the rows' prefix over the poses, as segment sums, an
//                     exclusive scan of the segments and a second walk of each segment
//   k_rs_rhs_large    thread per pose: the world-to-pose transform, the right-hand side
//                     into lg_y for the multi-CTA substitutions; clears the pair duals
// The per-pose values are those of k_resid_solve; only the prefix is summed in another
// order (FP64, segments of ~N / 42 poses).
__global__ void __launch_bounds__(256) k_rs_sums_large(PlanView pv, WorkView wv, int b) {
  if (!refine_active(wv, b)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b], fo = pv.p_frame_off[b];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 12 * N) return;
  double *rowm = wv.lg_red + ((size_t)pv.p_pose_off[b] + b) * 12, *colm = rowm + (size_t)(N + 1) * 6;
  const double *recs = wv.pdual + (size_t)pv.p_pair_off[b] * 6;
  auto cen = [&](int f, int k) {
    return (double)wv.fr_ch[(size_t)(fo + f) * 6 + k] + (double)wv.fr_cl[(size_t)(fo + f) * 6 + k];
  };
  const int k = t % 6;
  if (t < 6 * N) {  // row lo = t / 6
    const int lo = t / 6;
    const double *r = recs + (size_t)lo * D * 6 + k;
    const int nd = min(D, N - lo);
    double acc = 0.0;
#pragma unroll 4
    for (int d = 0; d < nd; ++d) acc += r[(size_t)d * 6];
    rowm[lo * 6 + k] = acc;
    if (lo == 0) colm[k] = 0.0;  // no record ends at pose 0
  } else {  // column hi = (t - 6 N) / 6 + 1
    const int hi = (t - 6 * N) / 6 + 1;
    double acc = 0.0;
    if (k < 3) {
      const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
#pragma unroll 4
      for (int lo = max(0, hi - D); lo < hi; ++lo) {
        const double *r = recs + ((size_t)lo * D + (hi - lo - 1)) * 6;
        acc += r[k] + (cen(lo, k1) * r[3 + k2] - cen(lo, k2) * r[3 + k1]);
      }
    } else {
#pragma unroll 4
      for (int lo = max(0, hi - D); lo < hi; ++lo) acc += recs[((size_t)lo * D + (hi - lo - 1)) * 6 + k];
    }
    colm[hi * 6 + k] = acc;
  }
}

constexpr int kScanSegs = 42;  // segments per component: 6 x 42 = 252 of the 256 threads

// dynamic shared memory: the per-pose terms [N][6] (FP64)
__global__ void __launch_bounds__(256) k_rs_scan_large(PlanView pv, WorkView wv, int b) {
  if (!refine_active(wv, b)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *val = reinterpret_cast<double *>(smem_raw);
  __shared__ double seg[6][kScanSegs];
  const int N = pv.p_npose[b], fo = pv.p_frame_off[b], tid = threadIdx.x;
  double *rowm = wv.lg_red + ((size_t)pv.p_pose_off[b] + b) * 12;
  const double *colm = rowm + (size_t)(N + 1) * 6;
  // pose i's term: its row sums moved from c_i (the origin of the records starting there)
  // less the column sums of the records ending there
  for (int t = tid; t < 6 * N; t += blockDim.x) {
    const int i = t / 6, k = t % 6, k1 = (k + 1) % 3, k2 = (k + 2) % 3;
    const double *m = rowm + i * 6;
    double nrow = m[k];
    if (k < 3) {
      const double c1 = (double)wv.fr_ch[(size_t)(fo + i) * 6 + k1] + (double)wv.fr_cl[(size_t)(fo + i) * 6 + k1];
      const double c2 = (double)wv.fr_ch[(size_t)(fo + i) * 6 + k2] + (double)wv.fr_cl[(size_t)(fo + i) * 6 + k2];
      nrow += c1 * m[3 + k2] - c2 * m[3 + k1];
    }
    val[t] = nrow - colm[t];
  }
  __syncthreads();
  const int len = (N + kScanSegs - 1) / kScanSegs;
  const int k = tid / kScanSegs, s = tid % kScanSegs, i0 = s * len, i1 = min(N, i0 + len);
  if (tid < 6 * kScanSegs) {
    double acc = 0.0;
    for (int i = i0; i < i1; ++i) acc += val[i * 6 + k];
    seg[k][s] = acc;
  }
  __syncthreads();
  if (tid < 6) {  // exclusive scan of the segment sums
    double acc = 0.0;
    for (int q = 0; q < kScanSegs; ++q) {
      const double v = seg[tid][q];
      seg[tid][q] = acc;
      acc += v;
    }
  }
  __syncthreads();
  if (tid < 6 * kScanSegs) {
    double acc = seg[k][s];
    for (int i = i0; i < i1; ++i) {
      acc += val[i * 6 + k];
      rowm[i * 6 + k] = acc;  // the sum of the records covering pose i
    }
  }
}

__global__ void __launch_bounds__(128) k_rs_rhs_large(PlanView pv, WorkView wv, int b) {
  if (!refine_active(wv, b)) return;
  const int N = pv.p_npose[b], D = pv.p_pair_D[b], P = 6 * N;
  const int fo = pv.p_frame_off[b], po = pv.p_param_off[b];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const double *rowm = wv.lg_red + ((size_t)pv.p_pose_off[b] + b) * 12;
  // the pair duals are summed: cleared for the next pass
  double *recs = wv.pdual + (size_t)pv.p_pair_off[b] * 6;
  for (size_t q = t; q < (size_t)N * D * 6; q += (size_t)gridDim.x * blockDim.x) recs[q] = 0.0;
  if (t >= N) return;
  const int i = t;
  const double lam = wv.lm[b].lam;
  const float *A = reinterpret_cast<const float *>(wv.A) + pv.p_S_off[b];
  double R[9], ci[3];
  frame_Rc(wv, fo + i, R, ci);
  const double *S = rowm + i * 6;
  const double w[3] = {S[0] - (ci[1] * S[5] - ci[2] * S[4]), S[1] - (ci[2] * S[3] - ci[0] * S[5]),
                       S[2] - (ci[0] * S[4] - ci[1] * S[3])};
  double out[6];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    out[r] = R[r] * w[0] + R[3 + r] * w[1] + R[6 + r] * w[2];
    out[3 + r] = R[r] * S[3] + R[3 + r] * S[4] + R[6 + r] * S[5];
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const int p = 6 * i + k;
    const double x = wv.delta[po + p];
    const double rhs = out[k] - lam * (double)A[(size_t)p * P + p] * x - (double)wv.rhsB[po + p];
    wv.rhsB[po + p] = 0.f;
    reinterpret_cast<float *>(wv.lg_y)[po + p] = (float)rhs;
  }
}

int launch_resid_reduce_large(const PlanView &pv, const WorkView &wv, int b, int N, void *stream) {
  if (!wv.lg_red) return 0;  // (the FP64 path has no refinement)
  cudaStream_t st = (cudaStream_t)stream;
  k_rs_sums_large<<<(12 * N + 255) / 256, 256, 0, st>>>(pv, wv, b);
  const size_t sm = (size_t)N * 6 * sizeof(double);
  cudaFuncSetAttribute(k_rs_scan_large, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_rs_scan_large<<<1, 256, sm, st>>>(pv, wv, b);
  k_rs_rhs_large<<<(N + 127) / 128, 128, 0, st>>>(pv, wv, b);
  g_launches += 3;
  return (int)cudaGetLastError();
}

int launch_resid_solve(const PlanView &pv, const WorkView &wv, const Params &prm, int first, void *stream) {
  (void)first;  // every pass reduces the same duals of e
  const size_t sm = resid_solve_smem(pv.max_P_small, pv.max_P / 6);
  cudaStream_t st = (cudaStream_t)stream;
  cudaFuncSetAttribute(k_resid_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_resid_solve<<<pv.B, kRsThreads, sm, st>>>(pv, wv, prm.outer_steps > 1 ? prm.outer_tol : 0.f);
  ++g_launches;
  return (int)cudaGetLastError();
}

// ---- the last inverse-depth correction, candidate and predicted decrease -------------
// one warp per chunk, lane = landmark slot: x_a += t - D^-1 W^T dx_p, alpha' =
// clamp(alpha + x_a), pred += x_a (g_a + (lam C + eps) x_a) with the accurate g_a
__global__ void k_backsub_refined(PlanView pv, WorkView wv, Params prm, const double *alpha, double *alpha_out) {
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int slot = threadIdx.x & 31;
  if (c >= pv.n_chunks) return;
  const int b = pv.ch_prob[c];
  if (!problem_active(wv.lm, b, GATE_RUNNING)) return;
  const bool failed = wv.lm[b].fail != 0;
  const int f0 = pv.ch_f0[c], nb = pv.ch_nb[c], lm0 = pv.ch_lm0[c], cnt = pv.ch_cnt[c];
  const int po = pv.p_param_off[b];
  const float *slab = reinterpret_cast<const float *>(wv.slab) + pv.ch_slab[c];
  const double *dl = wv.ddelta + po + 6 * f0;
  const int rows = 6 * nb;
  float s0 = 0.f, s1 = 0.f;
  if (!failed) {
    for (int rb = 0; rb < rows; rb += 32) {
      const float dv = rb + slot < rows ? (float)dl[rb + slot] : 0.f;
      const float *sr = slab + (size_t)rb * SPGO_CHUNK + slot;
      const int nr = min(32, rows - rb);
      float v[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) v[k] = k < nr ? sr[(size_t)k * SPGO_CHUNK] : 0.f;
#pragma unroll
      for (int k = 0; k < 32; k += 2) {
        s0 += v[k] * __shfl_sync(0xffffffffu, dv, k);
        s1 += v[k + 1] * __shfl_sync(0xffffffffu, dv, k + 1);
      }
    }
  }
  double pred = 0.0;
  if (slot < cnt && !failed) {
    const int li = lm0 + slot;
    const double lam = wv.lm[b].lam;
    const float C = reinterpret_cast<const float *>(wv.C)[li];
    const float Dd = C * (float)(1.0 + lam) + prm.eps;
    const double da = wv.dal[li] + (double)(wv.tl[li] - (s0 + s1) / Dd);
    pred = da * (wv.gaacc[li] + (lam * (double)C + (double)prm.eps) * da);
    const int u = pv.lm_user[li];
    alpha_out[u] = fmin(fmax(alpha[u] + da, (double)prm.alpha_min), (double)prm.alpha_max);
  }
  pred = warp_sum(pred);
  if (slot == 0 && pred != 0.0) atomicAdd(wv.pred_acc + b, pred);
}

int launch_backsub_refined(const PlanView &pv, const WorkView &wv, const Params &prm, const double *alpha,
                           double *alpha_out, void *stream) {
  if (pv.n_chunks == 0) return 0;
  k_backsub_refined<<<grid_for(pv.n_chunks, 4), 128, 0, (cudaStream_t)stream>>>(pv, wv, prm, alpha, alpha_out);
  ++g_launches;
  return (int)cudaGetLastError();
}

}  // namespace spgo
