// Pose chain, fused residual + Jacobian + accumulation kernel, and the cost pass.
//
// Replaces S-PGO's computeGlobalPoses (src/Optimization/Solver_cuda.cu:440-493),
// LevenbergMarquardt (Solver_cuda.cu:49-310, helpers src/Optimization/LMutils.cu:538-628)
// and compute_B_C_inv (Solver_cuda.cu:322-345).
//
// Factorisation used instead of the reference's dense J_T (4O x 6N) rows: the
// Jacobian of observation o (landmark anchored in frame a, seen in frame n)
// with respect to incremental pose i in [lo, hi) = [min(a,n), max(a,n)) is
//     J_{o,i} = s_o * K_o * Ad_i,   s_o = +1 (n > a) or -1 (n < a),
// where K_o = [ (X - x) x u_k , u_k ] (2x6, u = dpi/dt R_n^T) is the derivative
// with respect to a world-frame twist about an origin x, and Ad_i maps frame i's
// perturbation (psi, rho) to that world twist.  So one observation costs O(1)
// instead of O(window), and
//   * the pose-pose blocks come from per-(lo, hi) accumulators
//     M_{lo,hi} = sum K^T K, m_{lo,hi} = sum s K^T r  (pairs, 27 values),
//     combined later by 2-D prefix sums (k_system.cu);
//   * the pose-depth column of landmark l is B_l(i) = Ad_i^T b_l(i),
//     b_l(i) = sum over its observations covering i of s K^T j_alpha, written into
//     the chunk's landmark-contiguous slab for the Schur GEMM.
// Pair accumulators use the left centre of frame lo as origin and the slab
// uses the landmark's anchor centre, so no large world coordinates enter FP32.
#include "kernels.cuh"
#include "frames.cuh"
#include "dfloat.cuh"

#include <type_traits>

namespace spgo {

// ---- global poses: G[0] = I, G[k+1] = G[k] inv(T_k); right camera G T_r_to_l ----
// One warp per problem: an inclusive shuffle scan of the 3x4 products (FP64),
// 32 frames per pass with the running prefix carried between passes
// (the reference walks the chain with one thread, Solver_cuda.cu:472-491).
__device__ __forceinline__ void write_frame(const WorkView &wv, size_t f, const double *G, const double *Trl) {
  double Gr[12];
  compose34(G, Trl, Gr);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      wv.fr_Rd[f * 18 + 3 * i + j] = G[4 * i + j];
      wv.fr_Rd[f * 18 + 9 + 3 * i + j] = Gr[4 * i + j];
      const float gl = (float)G[4 * i + j], gr = (float)Gr[4 * i + j];
      wv.fr_Rf[f * 18 + 3 * i + j] = gl;
      wv.fr_Rf[f * 18 + 9 + 3 * i + j] = gr;
      wv.fr_Rl[f * 18 + 3 * i + j] = (float)(G[4 * i + j] - (double)gl);
      wv.fr_Rl[f * 18 + 9 + 3 * i + j] = (float)(Gr[4 * i + j] - (double)gr);
    }
    const double cl = G[4 * i + 3], cr = Gr[4 * i + 3];
    wv.fr_c[f * 6 + i] = cl;
    wv.fr_c[f * 6 + 3 + i] = cr;
    const float hl = (float)cl, hr = (float)cr;
    wv.fr_ch[f * 6 + i] = hl;
    wv.fr_ch[f * 6 + 3 + i] = hr;
    wv.fr_cl[f * 6 + i] = (float)(cl - (double)hl);
    wv.fr_cl[f * 6 + 3 + i] = (float)(cr - (double)hr);
  }
}

__global__ void k_chain(PlanView pv, WorkView wv, const double *__restrict__ poses, int gate) {
  const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= pv.B) return;
  if (!problem_active(wv.lm, b, gate)) return;
  const int N = pv.p_npose[b], fo = pv.p_frame_off[b], po = pv.p_pose_off[b];
  const double *Trl = pv.p_Trl + 12 * b;
  double carry[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  if (lane == 0) write_frame(wv, (size_t)fo, carry, Trl);
  for (int s = 0; s < N; s += 32) {
    const int k = s + lane;
    double M[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    if (k < N) invert34(poses + 12 * (size_t)(po + k), M);
    // inclusive scan: M_k <- M_0 M_1 ... M_k (earlier factors on the left)
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      double P[12];
#pragma unroll
      for (int q = 0; q < 12; ++q) P[q] = __shfl_up_sync(0xffffffffu, M[q], d);
      if (lane >= d) {
        double C[12];
        compose34(P, M, C);
#pragma unroll
        for (int q = 0; q < 12; ++q) M[q] = C[q];
      }
    }
    double G[12];
    compose34(carry, M, G);
    if (k < N) write_frame(wv, (size_t)(fo + k + 1), G, Trl);
#pragma unroll
    for (int q = 0; q < 12; ++q) carry[q] = __shfl_sync(0xffffffffu, G[q], 31);
  }
}

// upper-triangle index of a symmetric 6x6 (row i <= col j)
__device__ __forceinline__ constexpr int tri6(int i, int j) { return i * 6 - (i * (i - 1)) / 2 + (j - i); }

template <typename T>
struct LinSmem {
  T X[SPGO_CHUNK][3];      // anchor point, world axes, relative to the anchor centre
  float Xl[SPGO_CHUNK][3]; // FP32 path: low words of X as a double-float
  T dX[SPGO_CHUNK][3];     // dX / d alpha
  T C[SPGO_CHUNK], ga[SPGO_CHUNK];
  int a[SPGO_CHUNK], lo[SPGO_CHUNK], hi[SPGO_CHUNK];
  double cost[8];
  int key[8][32];                   // per warp: target frame of each lane's observation (-1: none)
};
constexpr int kStagePitch = 33;     // per-warp staging of the 27 pair values, [27][33]

// Dynamic shared memory after LinSmem, sized by the batch's widest chunk window
// (W = max_nb + 1 frames) and the CTA's warps:
//   dc    [W][6] float x 2   FP32 path: c_host - c_(f0 + f, cam), hi and lo
//   stage [warps][27][33] T  per-warp staging of the pair terms
//   slab  [6 (W - 1)][32] T  the chunk's slab
// (the cost pass uses dc only).
template <typename T>
struct LinLayout {
  size_t dc, stage, slab, total;
  __host__ __device__ LinLayout(int max_nb, int warps, bool cost) {
    const size_t W = (size_t)max_nb + 1;
    auto up = [](size_t x) { return (x + 15) & ~(size_t)15; };
    dc = up(sizeof(LinSmem<T>));
    stage = dc + up(W * 12 * sizeof(float));
    slab = stage + up((size_t)warps * 27 * kStagePitch * sizeof(T));
    total = cost ? stage : slab + (size_t)6 * (W - 1) * SPGO_CHUNK * sizeof(T);
  }
};

// ---- fused linearisation / cost -----------------------------------------------
// One CTA per chunk of <= 32 landmarks.  Phase A: per-landmark anchor point.
// Phase B: one thread per observation (both cameras): residual, robust weight,
// inverse-depth Jacobian (C, g_a by shared atomics), pair accumulators, and the
// observation's s K^T j_alpha written into the slab row of its frame.  The pair
// terms of a warp are staged in shared memory and summed over runs of equal
// target frame (observations are sorted by frame, and every landmark of the
// chunk has the same host) by 27 lanes, one value each, and each run's sum is
// added to the global pair accumulator.  Phase C: per landmark,
// the suffix (frames after the anchor) and prefix (frames before it) sums that
// turn those rows into b_l(i), then B_l(i) = Ad_i^T b_l(i).
// COST = true is the cost pass: residuals only, in double-float on the FP32 path
// (FP64-accurate cost for the gain ratio), which it also stores as FP32 per
// observation.  The linearisation always follows a cost pass at the same state
// (the first one after a reset, or the accepted candidate's) and takes the cost
// from it.  COST = false here is the FP64 path's Jacobian pass; the FP32 path's is
// k_jacobian_acc below, which reads those stored residuals instead of forming them
// from pixel-sized FP32 quantities (whose ~3e-5 px rounding would move the optimum
// by ~1e-5 m).
// Register cap (FP32 cost pass): 64, a latency-bound stream over the observations
// that runs in small CTAs and gains from the extra resident warps (16 instead of
// 12 64-thread CTAs per SM).
template <typename T, bool COST>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 1) k_linearize(PlanView pv, WorkView wv, Params prm,
                                                   const double *__restrict__ alpha_state, int gate) {
  // (the FP32 path's Jacobian pass is k_jacobian_acc)
  static_assert(COST || std::is_same<T, double>::value, "FP32 linearisation: k_jacobian_acc");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int c = blockIdx.x;
  const int b = pv.ch_prob[c];
  if (!problem_active(wv.lm, b, gate)) return;
  const int tid = threadIdx.x;
  const int f0 = pv.ch_f0[c], nb = pv.ch_nb[c], lm0 = pv.ch_lm0[c], cnt = pv.ch_cnt[c];
  const int fo = pv.p_frame_off[b];
  const float *intr = pv.p_intr + 8 * b;
  const T fxs[2] = {(T)intr[0], (T)intr[4]}, fys[2] = {(T)intr[1], (T)intr[5]};
  const T cxs[2] = {(T)intr[2], (T)intr[6]}, cys[2] = {(T)intr[3], (T)intr[7]};
  LinSmem<T> &sm = *reinterpret_cast<LinSmem<T> *>(smem_raw);
  const LinLayout<T> lay(pv.max_nb, blockDim.x >> 5, COST);
  float *dch = reinterpret_cast<float *>(smem_raw + lay.dc);  // [W][6] hi, then [W][6] lo
  float *dcl = dch + (size_t)(pv.max_nb + 1) * 6;
  T *stage = reinterpret_cast<T *>(smem_raw + lay.stage);
  T *slab_s = reinterpret_cast<T *>(smem_raw + lay.slab);
  const int rows = 6 * nb;
  const int64_t ob = pv.lm_obs[lm0], oe = pv.lm_obs[lm0 + cnt];
  // residual store: the Jacobian pass reads the state's half; the cost pass of the
  // state after a reset writes the state's half, a candidate's the other half
  const int sel = wv.lm[b].res_sel;
  const size_t half = (size_t)(COST && gate != GATE_FIRST ? 1 - sel : sel);
  float *res_buf = wv.res + half * (size_t)pv.O * 4;
  float *tcam_buf = wv.tcam ? wv.tcam + half * (size_t)pv.O * 6 : nullptr;  // mixed path: camera-frame points
  float *xanc_buf = wv.xanc ? wv.xanc + half * (size_t)pv.L * 8 : nullptr;   // and anchor points
  // cost pass: each thread's observation record is loaded one loop pass ahead (the
  // first one here, so its DRAM latency overlaps phase A), so a pass does not open
  // with a round trip to DRAM; the Jacobian pass has no registers to spare for it
  int nx_slot = 0, nx_n = 0;
  float4 nx_z = make_float4(0.f, 0.f, 0.f, 0.f);
  auto load_obs = [&](int64_t o) {
    if (o < oe) {
      nx_slot = pv.obs_slot[o];
      nx_n = pv.obs_frame[o];
      nx_z = reinterpret_cast<const float4 *>(pv.obs_uv)[o];
    }
  };
  if (COST) load_obs(ob + tid);

  // phase A
  if (tid < cnt) {
    const int li = lm0 + tid;
    const int a = pv.lm_host[li];
    const T alpha = (T)alpha_state[pv.lm_user[li]];
    const T ua = (T)pv.lm_uv[2 * li], va = (T)pv.lm_uv[2 * li + 1];
    const T *Ra = FramesT<T>::R(wv, fo + a, 0);
    const Vec3<T> ta = v3<T>((ua - cxs[0]) / fxs[0] / alpha, (va - cys[0]) / fys[0] / alpha, T(1) / alpha);
    Vec3<T> X = mul(Ra, ta);
    if constexpr (std::is_same<T, float>::value) {
      // the same point as a double-float, for the residuals
      const df al = df_from_double(alpha_state[pv.lm_user[li]]);
      const df t3[3] = {df_sub(pv.lm_uv[2 * li], intr[2]) / df_make(intr[0]) / al,
                        df_sub(pv.lm_uv[2 * li + 1], intr[3]) / df_make(intr[1]) / al, df_make(1.f) / al};
      const float *Rh = wv.fr_Rf + (size_t)(fo + a) * 18, *Rl = wv.fr_Rl + (size_t)(fo + a) * 18;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const df v = df{Rh[3 * k], Rl[3 * k]} * t3[0] + df{Rh[3 * k + 1], Rl[3 * k + 1]} * t3[1] +
                     df{Rh[3 * k + 2], Rl[3 * k + 2]} * t3[2];
        sm.Xl[tid][k] = v.l;
        if (k == 0) X.x = v.h;
        if (k == 1) X.y = v.h;
        if (k == 2) X.z = v.h;
      }
    }
    sm.X[tid][0] = X.x; sm.X[tid][1] = X.y; sm.X[tid][2] = X.z;
    sm.dX[tid][0] = -X.x / alpha; sm.dX[tid][1] = -X.y / alpha; sm.dX[tid][2] = -X.z / alpha;
    if (COST && xanc_buf) {  // kept for the Jacobian and residual passes at this state
      float4 *xa = reinterpret_cast<float4 *>(xanc_buf + (size_t)li * 8);
      xa[0] = make_float4((float)X.x, (float)X.y, (float)X.z, (float)sm.dX[tid][0]);
      xa[1] = make_float4((float)sm.dX[tid][1], (float)sm.dX[tid][2], 0.f, 0.f);
    }
    sm.C[tid] = T(0);
    sm.ga[tid] = T(0);
    sm.a[tid] = a;
    sm.lo[tid] = pv.lm_lo[li];
    sm.hi[tid] = pv.lm_hi[li];
  }
  if constexpr (std::is_same<T, float>::value) {
    // the host's left centre minus every window frame's camera centres, as double-floats
    const int fh = fo + pv.lm_host[lm0];
    for (int idx = tid; idx < (nb + 1) * 6; idx += blockDim.x) {
      const int f = idx / 6, cam = (idx / 3) & 1, k = idx % 3;
      const size_t fn = (size_t)(fo + f0 + f);
      df d = df_sub(wv.fr_ch[(size_t)fh * 6 + k], wv.fr_ch[fn * 6 + cam * 3 + k]);
      d = d + df_make(wv.fr_cl[(size_t)fh * 6 + k] - wv.fr_cl[fn * 6 + cam * 3 + k]);
      dch[idx] = d.h;
      dcl[idx] = d.l;
    }
  }
  if (!COST)
    for (int i = tid; i < rows * SPGO_CHUNK; i += blockDim.x) slab_s[i] = T(0);
  __syncthreads();

  // phase B: observations are sorted by target frame inside the chunk and every
  // landmark of the chunk has the same host, so a warp's pair terms (host, target)
  // form contiguous runs: each run's sum goes straight into the global pair
  // accumulator (lo, hi) = (min, max)(host, target), one reduction per value and run
  // (about as many as a per-chunk shared copy would flush, without its shared
  // memory, its zeroing and its flush pass)
  const int D = pv.p_pair_D[b];
  auto pair_add = [&](int n, int comp, T v) {  // (operands re-read here: few registers stay live)
    const int host_a = sm.a[0];
    const int lo = min(host_a, n), hi = max(host_a, n);
    red_add(reinterpret_cast<T *>(wv.pair_acc) + ((size_t)pv.p_pair_off[b] + (size_t)lo * D + (hi - lo - 1)) * 27 + comp,
            v);
  };
  const int lane = tid & 31;
  const T lscale = (T)prm.loss_scale;
  T cost_t = T(0);  // a thread sums a handful of terms; the FP64 reduction starts at the warp
  for (int64_t base = ob + (tid & ~31); base < oe; base += blockDim.x) {
    const int64_t o = base + lane;
    T M[21], m[6];
    int key = -1;
    if (!COST) {
#pragma unroll
      for (int k = 0; k < 21; ++k) M[k] = T(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) m[k] = T(0);
    }
    int cur_slot = nx_slot, cur_n = nx_n;
    float4 cur_z = nx_z;
    if (COST) {
      load_obs(o + blockDim.x);  // the next pass's record, in flight during this one
    } else if (o < oe) {
      cur_slot = pv.obs_slot[o];
      cur_n = pv.obs_frame[o];
      cur_z = reinterpret_cast<const float4 *>(pv.obs_uv)[o];
    }
    if (o < oe) {
      const int slot = cur_slot;
      const int n = cur_n;
      const float4 z = cur_z;
      float4 rstore = make_float4(0.f, 0.f, 0.f, 0.f);  // cost pass: residuals to keep
      float tstore[6];                                    // and the camera-frame points
      const int a = sm.a[slot];
      const Vec3<T> X = v3<T>(sm.X[slot][0], sm.X[slot][1], sm.X[slot][2]);
      const int fa = fo + a, fn = fo + n;
      const bool has_pose = (n != a);
      const int lo = min(a, n);
      const T sgn = n > a ? T(1) : T(-1);
      const T boost = (prm.near_boost && abs(n - a) < 2) ? T(16) : T(1);
      T q[6], accC = T(0), accG = T(0);
      Vec3<T> Xp = X, dXda = X;
      if (!COST) {
#pragma unroll
        for (int k = 0; k < 6; ++k) q[k] = T(0);
        dXda = v3<T>(sm.dX[slot][0], sm.dX[slot][1], sm.dX[slot][2]);
        if (has_pose && lo != a) {  // point relative to the pair origin: left centre of frame lo
          const Vec3<T> d = FramesT<T>::rel(wv, fa, 0, fo + lo, 0);
          Xp = v3<T>(X.x + d.x, X.y + d.y, X.z + d.z);
        }
      }
#pragma unroll
      for (int cam = 0; cam < 2; ++cam) {
        const T *Rn = FramesT<T>::R(wv, fn, cam);
        const T fx = fxs[cam], fy = fys[cam];
        Vec3<T> t;
        T r0, r1;
        if constexpr (COST && std::is_same<T, float>::value) {
          // residual in double-float: X + (c_a - c_n), rotated, then projected as
          // r = ((z - c) t_z - f t_x) / t_z (the small numerator carries the
          // precision, the division is plain FP32)
          const float *Rl = wv.fr_Rl + (size_t)fn * 18 + cam * 9;
          const int fw = n - f0;
          df Xc[3];
#pragma unroll
          for (int k = 0; k < 3; ++k)
            Xc[k] = df{sm.X[slot][k], sm.Xl[slot][k]} + df{dch[fw * 6 + cam * 3 + k], dcl[fw * 6 + cam * 3 + k]};
          df tt[3];
#pragma unroll
          for (int k = 0; k < 3; ++k)
            tt[k] = df_dot3(Rn[k], Rl[k], Rn[3 + k], Rl[3 + k], Rn[6 + k], Rl[6 + k], Xc[0], Xc[1], Xc[2]);
          const df nu = df_sub(cam ? z.z : z.x, cxs[cam]) * tt[2] - tt[0] * fx;
          const df nv = df_sub(cam ? z.w : z.y, cys[cam]) * tt[2] - tt[1] * fy;
          const float itz = 1.f / tt[2].h;
          r0 = (nu.h + nu.l) * itz;
          r1 = (nv.h + nv.l) * itz;
          t = v3<T>(tt[0].h, tt[1].h, tt[2].h);
          tstore[3 * cam] = tt[0].h;
          tstore[3 * cam + 1] = tt[1].h;
          tstore[3 * cam + 2] = tt[2].h;
          if (cam) {
            rstore.z = r0;
            rstore.w = r1;
          } else {
            rstore.x = r0;
            rstore.y = r1;
          }
        } else {
          const Vec3<T> d = FramesT<T>::rel(wv, fa, 0, fn, cam);
          t = mulT(Rn, v3<T>(X.x + d.x, X.y + d.y, X.z + d.z));
          {
            const T izr = T(1) / t.z;
            r0 = (T)(cam ? z.z : z.x) - (fx * t.x * izr + cxs[cam]);
            r1 = (T)(cam ? z.w : z.y) - (fy * t.y * izr + cys[cam]);
          }
        }
        const T iz = T(1) / t.z;
        T rho;
        const T w2 = boost * robust<T>(prm.loss, lscale, r0 * r0 + r1 * r1, rho);
        if (COST) {
          cost_t += T(0.5) * boost * rho;
          continue;
        }
        // dpi/dt (2x3) then u = dpi/dt R_n^T (rows u0, u1)
        const T j00 = fx * iz, j02 = -fx * t.x * iz * iz, j11 = fy * iz, j12 = -fy * t.y * iz * iz;
        const Vec3<T> u0 = v3<T>(j00 * Rn[0] + j02 * Rn[2], j00 * Rn[3] + j02 * Rn[5], j00 * Rn[6] + j02 * Rn[8]);
        const Vec3<T> u1 = v3<T>(j11 * Rn[1] + j12 * Rn[2], j11 * Rn[4] + j12 * Rn[5], j11 * Rn[7] + j12 * Rn[8]);
        const T ja0 = dot(u0, dXda), ja1 = dot(u1, dXda);
        accC += w2 * (ja0 * ja0 + ja1 * ja1);
        accG += w2 * (ja0 * r0 + ja1 * r1);
        if (has_pose) {
          const Vec3<T> k0 = cross(Xp, u0), k1 = cross(Xp, u1);
          const T K0[6] = {k0.x, k0.y, k0.z, u0.x, u0.y, u0.z};
          const T K1[6] = {k1.x, k1.y, k1.z, u1.x, u1.y, u1.z};
#pragma unroll
          for (int i = 0; i < 6; ++i) {
#pragma unroll
            for (int j = i; j < 6; ++j) M[tri6(i, j)] += w2 * (K0[i] * K0[j] + K1[i] * K1[j]);
            m[i] += sgn * w2 * (K0[i] * r0 + K1[i] * r1);
          }
          const Vec3<T> h0 = cross(X, u0), h1 = cross(X, u1);
          const T sj0 = sgn * w2 * ja0, sj1 = sgn * w2 * ja1;
          q[0] += h0.x * sj0 + h1.x * sj1;
          q[1] += h0.y * sj0 + h1.y * sj1;
          q[2] += h0.z * sj0 + h1.z * sj1;
          q[3] += u0.x * sj0 + u1.x * sj1;
          q[4] += u0.y * sj0 + u1.y * sj1;
          q[5] += u0.z * sj0 + u1.z * sj1;
        }
      }
      if constexpr (COST && std::is_same<T, float>::value) {
        reinterpret_cast<float4 *>(res_buf)[o] = rstore;
        if (tcam_buf) {  // 24 bytes at 8-byte alignment
          float2 *tp = reinterpret_cast<float2 *>(tcam_buf + (size_t)o * 6);
          tp[0] = make_float2(tstore[0], tstore[1]);
          tp[1] = make_float2(tstore[2], tstore[3]);
          tp[2] = make_float2(tstore[4], tstore[5]);
        }
      }
      if (!COST) {
        atomicAdd(&sm.C[slot], accC);
        atomicAdd(&sm.ga[slot], accG);
        if (has_pose) {
          key = n;
          // frames after the anchor cover blocks [a, n): row n - 1 feeds a suffix sum;
          // frames before it cover [n, a): row n feeds a prefix sum.  Rows are distinct.
          const int row = (n > a ? n - 1 : n) - f0;
          T *dstq = slab_s + (size_t)(6 * row) * SPGO_CHUNK + slot;
#pragma unroll
          for (int k = 0; k < 6; ++k) dstq[k * SPGO_CHUNK] = q[k];
        }
      }
    }
    if (!COST) {
      // stage the 27 pair values, then lanes 0..26 each sum one value over the
      // runs of equal target frame and add each run to its global pair accumulator
      T *st = stage + (size_t)(tid >> 5) * 27 * kStagePitch;
      int *keys = sm.key[tid >> 5];
#pragma unroll
      for (int k = 0; k < 21; ++k) st[k * kStagePitch + lane] = M[k];
#pragma unroll
      for (int k = 0; k < 6; ++k) st[(21 + k) * kStagePitch + lane] = m[k];
      keys[lane] = key;
      __syncwarp();
      if (__any_sync(0xffffffffu, key >= 0) && lane < 27) {
        const T *col = st + lane * kStagePitch;
        T acc = T(0);
        int cur = keys[0];
        for (int i = 0; i < 32; ++i) {
          const int k = keys[i];
          if (k != cur) {
            if (cur >= 0 && acc != T(0)) pair_add(cur, lane, acc);
            acc = T(0);
            cur = k;
          }
          acc += col[i];
        }
        if (cur >= 0 && acc != T(0)) pair_add(cur, lane, acc);
      }
      __syncwarp();
    }
  }
  if (COST) {
    // cost: warp sums, then one FP64 atomic per CTA
    const double cost = warp_sum((double)cost_t);
    if ((tid & 31) == 0) sm.cost[tid >> 5] = cost;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm.cost[w];
      if (t != 0.0) atomicAdd(wv.cost_acc + b, t);
    }
    return;
  }
  __syncthreads();

  // phase C.1: per (landmark, component) suffix / prefix sums along the window
  for (int idx = tid; idx < cnt * 6; idx += blockDim.x) {
    const int slot = idx % cnt, k = idx / cnt;  // consecutive threads: consecutive slots (banks)
    const int a = sm.a[slot], lo_l = sm.lo[slot], hi_l = sm.hi[slot];
    T acc = T(0);
    for (int i = hi_l - 1; i >= a; --i) {
      T *p = slab_s + (size_t)(6 * (i - f0) + k) * SPGO_CHUNK + slot;
      acc += *p;
      *p = acc;
    }
    acc = T(0);
    for (int i = lo_l; i < a; ++i) {
      T *p = slab_s + (size_t)(6 * (i - f0) + k) * SPGO_CHUNK + slot;
      acc += *p;
      *p = acc;
    }
  }
  __syncthreads();
  // phase C.2: B_l(i) = Ad_i^T b_l(i) about the anchor centre:
  //   [R_i^T (b_w - (c_i - c_a) x b_v) ; R_i^T b_v]
  for (int idx = tid; idx < cnt * nb; idx += blockDim.x) {
    const int slot = idx % cnt, i = f0 + idx / cnt;
    if (i < sm.lo[slot] || i >= sm.hi[slot]) continue;
    const int fi = fo + i;
    const T *Ri = FramesT<T>::R(wv, fi, 0);
    const Vec3<T> d = FramesT<T>::rel(wv, fi, 0, fo + sm.a[slot], 0);
    T *dst = slab_s + (size_t)(6 * (i - f0)) * SPGO_CHUNK + slot;
    const Vec3<T> bw = v3<T>(dst[0], dst[SPGO_CHUNK], dst[2 * SPGO_CHUNK]);
    const Vec3<T> bv = v3<T>(dst[3 * SPGO_CHUNK], dst[4 * SPGO_CHUNK], dst[5 * SPGO_CHUNK]);
    const Vec3<T> dxb = cross(d, bv);
    const Vec3<T> Bw = mulT(Ri, v3<T>(bw.x - dxb.x, bw.y - dxb.y, bw.z - dxb.z));
    const Vec3<T> Bv = mulT(Ri, bv);
    dst[0] = Bw.x;
    dst[SPGO_CHUNK] = Bw.y;
    dst[2 * SPGO_CHUNK] = Bw.z;
    dst[3 * SPGO_CHUNK] = Bv.x;
    dst[4 * SPGO_CHUNK] = Bv.y;
    dst[5 * SPGO_CHUNK] = Bv.z;
  }
  __syncthreads();
  // phase D: slab, C and g_a to global
  T *gslab = reinterpret_cast<T *>(wv.slab) + pv.ch_slab[c];
  for (int i = tid; i < rows * SPGO_CHUNK; i += blockDim.x) gslab[i] = slab_s[i];
  if (tid < cnt) {
    reinterpret_cast<T *>(wv.C)[lm0 + tid] = sm.C[tid];
    reinterpret_cast<T *>(wv.ga)[lm0 + tid] = sm.ga[tid];
  }
}

// ---- the mixed path's Jacobian pass: exactly summed normal equations --------------
// The same FP32 Jacobian as k_linearize (the camera-frame point formed in
// double-float from the frame tables and rounded once; the residuals of the cost
// pass at the same state), but the sums that build the normal equations are not
// left to FP32: the reduced camera system S = A + damping - W D^-1 W^T cancels most
// of A, and FP32 sums over thousands of observations put errors into A and W that,
// measured against S, reach its smallest eigenvalues (an FP32-assembled S of a
// badly initialised circle problem came out indefinite where the FP64 one has
// scaled smallest eigenvalue 4e-4).  So, with the weighted rows w K (w^2 the robust
// weight) and the weighted residuals w r rounded once:
//   * every product of the pair records (21 Hessian and 6 gradient values per
//     observation) is formed exactly (two-product) and summed in double-float;
//     each run of equal target frame goes to the FP64 pair record by an FP64 atomic
//     (the pair reduction then runs in double-float about one origin, k_system.cu);
//   * the slab terms s (w h)(w j_alpha) likewise, from the same rounded rows (moved
//     from the pair origin to the anchor centre in double-float), and the
//     per-landmark suffix / prefix sums along the window and the move to each pose
//     frame run in double-float; the slab is rounded to FP32 once, at the end.  The
//     slab only enters the preconditioner of the refined step, but a slab accumulated
//     in FP32, and also one whose double-float moments were rounded before an FP32
//     rotation to the pose axes, left single ill-conditioned problems of the config-3
//     batch with an unusable preconditioner: they stalled 7 % to 70x above the plain
//     FP64 cost (the assembled S cancels A against W D^-1 W^T, and W must match A's
//     rounding-once accuracy).
// C and g_a (positive sums and the preconditioner's own right-hand side) stay FP32;
// g_a is also summed exactly (per observation an exact four-product sum, per landmark
// double-float) for the refined step's predicted decrease, which near the optimum is a
// small difference of large terms.
struct JacSmem {
  float X[SPGO_CHUNK][3];   // anchor point, world axes, relative to the anchor centre
  float dX[SPGO_CHUNK][3];  // dX / d alpha
  float C[SPGO_CHUNK], ga[SPGO_CHUNK];
  int a[SPGO_CHUNK], lo[SPGO_CHUNK], hi[SPGO_CHUNK];
  unsigned rmask[SPGO_MAX_WINDOW];  // per window row: the landmarks whose window holds its frame
  int rsp[SPGO_MAX_WINDOW + 1];     // exclusive prefix of the rows' landmark counts
  int key[8][32];           // per warp: target frame of each lane's observation (-1: none)
  float glh[8][SPGO_CHUNK];  // per warp: exactly summed g_a, double-float (h, l)
  float gll[8][SPGO_CHUNK];
};
constexpr int kJacVals = 27;          // 21 Hessian + 6 gradient values per pair record
constexpr int kJacRound = 9;          // pair values staged per round (three rounds of 9)
constexpr int kJacSegs = 3;           // observation segments per staged value in the run sums
constexpr int kJacSegLen = 11;        // ceil(32 / 3)
constexpr int kJacPitch = 33;

// dynamic shared memory: dc [W][6] float x 2 (hi, lo) | stage [warps][2 * 9][33]
// float (double-float pair terms, one round) | slab hi and lo [6 (W - 1)][32] float
// each.  For 32-frame windows 74.6 KB: three 8-warp CTAs per SM.
struct JacLayout {
  size_t dc, stage, slab_h, slab_l, total;
  __host__ __device__ JacLayout(int max_nb, int warps) {
    const size_t W = (size_t)max_nb + 1;
    auto up = [](size_t x) { return (x + 15) & ~(size_t)15; };
    dc = up(sizeof(JacSmem));
    stage = dc + up(W * 12 * sizeof(float));
    slab_h = stage + up((size_t)warps * 2 * kJacRound * kJacPitch * sizeof(float));
    slab_l = slab_h + up((size_t)6 * (W - 1) * SPGO_CHUNK * sizeof(float));
    total = slab_l + (size_t)6 * (W - 1) * SPGO_CHUNK * sizeof(float);
  }
};

// Stages pair values [V0, V1) (the packed upper 6 x 6 block 0..20, then the gradient
// 21..26) of the lane's observation, each the exact four-product sum, as (h, l) rows
template <int V0, int V1>
__device__ __forceinline__ void jac_stage(const float (&K)[2][2][6], const float (&RW)[2][2], float *st, int lane) {
#pragma unroll
  for (int i = 0; i < 6; ++i) {
#pragma unroll
    for (int j = i; j < 6; ++j) {
      const int v = tri6(i, j);
      if (v >= V0 && v < V1) {
        const df x = sum4_prod(K[0][0][i], K[0][0][j], K[0][1][i], K[0][1][j], K[1][0][i], K[1][0][j], K[1][1][i],
                               K[1][1][j]);
        st[(2 * (v - V0)) * kJacPitch + lane] = x.h;
        st[(2 * (v - V0) + 1) * kJacPitch + lane] = x.l;
      }
    }
    const int v = 21 + i;
    if (v >= V0 && v < V1) {
      const df x = sum4_prod(K[0][0][i], RW[0][0], K[0][1][i], RW[0][1], K[1][0][i], RW[1][0], K[1][1][i], RW[1][1]);
      st[(2 * (v - V0)) * kJacPitch + lane] = x.h;
      st[(2 * (v - V0) + 1) * kJacPitch + lane] = x.l;
    }
  }
}

// Sums the staged values [V0, V1) over the runs of equal target frame: lane = (value,
// 11-observation segment); every run goes to its FP64 pair record (a run crossing a
// segment boundary arrives in parts)
template <int V0, int V1>
__device__ __forceinline__ void jac_runs(const float *st, const int *keys, int lane, int host_a, int D,
                                         double *pair_base) {
  constexpr int NV = V1 - V0;
  if (lane >= kJacSegs * NV) return;
  const int v = lane % NV, i0 = (lane / NV) * kJacSegLen, i1 = min(32, i0 + kJacSegLen);
  const float *ch = st + (2 * v) * kJacPitch, *cl = st + (2 * v + 1) * kJacPitch;
  auto emit = [&](int n, const df_acc &a) {
    const int lo = min(host_a, n), hi = max(host_a, n);
    atomicAdd(pair_base + ((size_t)lo * D + (hi - lo - 1)) * kJacVals + V0 + v, df_acc_value(a));
  };
  df_acc acc;
  int cur = keys[i0];
#pragma unroll 4
  for (int i = i0; i < i1; ++i) {
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

__global__ void __launch_bounds__(256, 3) k_jacobian_acc(PlanView pv, WorkView wv, Params prm,
                                                         const double *__restrict__ alpha_state, int gate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int c = blockIdx.x;
  const int b = pv.ch_prob[c];
  if (!problem_active(wv.lm, b, gate)) return;
  const int tid = threadIdx.x, lane = tid & 31;
  const int f0 = pv.ch_f0[c], nb = pv.ch_nb[c], lm0 = pv.ch_lm0[c], cnt = pv.ch_cnt[c];
  const int fo = pv.p_frame_off[b];
  const float *intr = pv.p_intr + 8 * b;
  const float fxs[2] = {intr[0], intr[4]}, fys[2] = {intr[1], intr[5]};
  JacSmem &sm = *reinterpret_cast<JacSmem *>(smem_raw);
  const JacLayout lay(pv.max_nb, blockDim.x >> 5);
  float *dch = reinterpret_cast<float *>(smem_raw + lay.dc);
  float *dcl = dch + (size_t)(pv.max_nb + 1) * 6;
  float *stage = reinterpret_cast<float *>(smem_raw + lay.stage);
  float *slab_h = reinterpret_cast<float *>(smem_raw + lay.slab_h);
  float *slab_l = reinterpret_cast<float *>(smem_raw + lay.slab_l);
  const int rows = 6 * nb;
  const int64_t ob = pv.lm_obs[lm0], oe = pv.lm_obs[lm0 + cnt];
  const float *res_buf = wv.res + (size_t)wv.lm[b].res_sel * (size_t)pv.O * 4;  // the state's residuals
  const float *tcam_buf = wv.tcam + (size_t)wv.lm[b].res_sel * (size_t)pv.O * 6;  // and camera-frame points

  // phase A: the chunk's anchor points, as the cost pass at this state formed them
  // (double-float, rounded to the high part)
  if (tid < cnt) {
    const int li = lm0 + tid;
    const int a = pv.lm_host[li];
    const float4 *xa = reinterpret_cast<const float4 *>(wv.xanc + ((size_t)wv.lm[b].res_sel * pv.L + li) * 8);
    const float4 x0 = xa[0], x1 = xa[1];
    sm.X[tid][0] = x0.x;
    sm.X[tid][1] = x0.y;
    sm.X[tid][2] = x0.z;
    sm.dX[tid][0] = x0.w;
    sm.dX[tid][1] = x1.x;
    sm.dX[tid][2] = x1.y;
    sm.C[tid] = 0.f;
    sm.ga[tid] = 0.f;
    sm.a[tid] = a;
    sm.lo[tid] = pv.lm_lo[li];
    sm.hi[tid] = pv.lm_hi[li];
  }
  if (tid < 32) {  // per window row, the landmarks whose window [lo, hi) holds its frame
    const int lo = tid < cnt ? pv.lm_lo[lm0 + tid] : 0, hi = tid < cnt ? pv.lm_hi[lm0 + tid] : 0;
    int run = 0;
    for (int i = 0; i < nb; ++i) {
      const unsigned m = __ballot_sync(0xffffffffu, lo <= f0 + i && f0 + i < hi);
      if (tid == 0) {
        sm.rmask[i] = m;
        sm.rsp[i] = run;
      }
      run += __popc(m);
    }
    if (tid == 0) sm.rsp[nb] = run;
  }
  {  // the host's left centre minus every window frame's camera centres (double-float)
    const int fh = fo + pv.lm_host[lm0];
    for (int idx = tid; idx < (nb + 1) * 6; idx += blockDim.x) {
      const int f = idx / 6, cam = (idx / 3) & 1, k = idx % 3;
      const size_t fn = (size_t)(fo + f0 + f);
      df d = df_sub(wv.fr_ch[(size_t)fh * 6 + k], wv.fr_ch[fn * 6 + cam * 3 + k]);
      d = d + df_make(wv.fr_cl[(size_t)fh * 6 + k] - wv.fr_cl[fn * 6 + cam * 3 + k]);
      dch[idx] = d.h;
      dcl[idx] = d.l;
    }
  }
  for (int i = tid; i < rows * SPGO_CHUNK; i += blockDim.x) slab_h[i] = slab_l[i] = 0.f;
  for (int i = tid; i < 8 * SPGO_CHUNK; i += blockDim.x) (&sm.glh[0][0])[i] = (&sm.gll[0][0])[i] = 0.f;
  __syncthreads();

  // phase B: thread per observation; runs of equal target frame inside a warp go to
  // the FP64 pair record (host, target).  A lane keeps its observation's weighted
  // pose rows of both cameras (zero without a pose term) and forms each of the 27
  // pair values once, as the exact sum of its four products, straight into the staging.
  const int D = pv.p_pair_D[b];
  double *pair_base = reinterpret_cast<double *>(wv.pair_acc) + (size_t)pv.p_pair_off[b] * kJacVals;
  const float lscale = prm.loss_scale;
  for (int64_t base = ob + (tid & ~31); base < oe; base += blockDim.x) {
    const int64_t o = base + lane;
    float K[2][2][6];  // [camera][row][parameter]: w K, about the pair origin
    float RW[2][2];    // s w r
    float JW[2][2];    // s w j_alpha
#pragma unroll
    for (int c2 = 0; c2 < 2; ++c2)
#pragma unroll
      for (int r2 = 0; r2 < 2; ++r2) {
        RW[c2][r2] = JW[c2][r2] = 0.f;
#pragma unroll
        for (int k = 0; k < 6; ++k) K[c2][r2][k] = 0.f;
      }
    int key = -1, slot = -1;
    if (o < oe) {
      slot = pv.obs_slot[o];
      const int n = pv.obs_frame[o];
      const float4 rl = reinterpret_cast<const float4 *>(res_buf)[o];
      const int a = sm.a[slot];
      const Vec3<float> X = v3<float>(sm.X[slot][0], sm.X[slot][1], sm.X[slot][2]);
      const Vec3<float> dXda = v3<float>(sm.dX[slot][0], sm.dX[slot][1], sm.dX[slot][2]);
      const int fn = fo + n;
      const bool has_pose = (n != a);
      const int lo = min(a, n);
      const float sgn = n > a ? 1.f : -1.f;
      const float boost = (prm.near_boost && abs(n - a) < 2) ? 16.f : 1.f;
      // point relative to the pair origin (the left centre of frame lo): X + d
      Vec3<float> d = v3<float>(0.f, 0.f, 0.f);
      if (has_pose && lo != a) d = FramesT<float>::rel(wv, fo + a, 0, fo + lo, 0);
      const Vec3<float> Xp = v3<float>(X.x + d.x, X.y + d.y, X.z + d.z);
      float accC = 0.f, accG = 0.f;
      // the camera-frame points of both cameras, as the cost pass at this state formed
      // them (double-float, rounded once)
      const float2 *tp = reinterpret_cast<const float2 *>(tcam_buf + (size_t)o * 6);
      const float2 t01 = tp[0], t23 = tp[1], t45 = tp[2];
#pragma unroll
      for (int cam = 0; cam < 2; ++cam) {
        const float *Rn = FramesT<float>::R(wv, fn, cam);
        const Vec3<float> t = cam ? v3<float>(t23.y, t45.x, t45.y) : v3<float>(t01.x, t01.y, t23.x);
        const float r0 = cam ? rl.z : rl.x, r1 = cam ? rl.w : rl.y;
        float rho;
        const float w2 = boost * robust<float>(prm.loss, lscale, r0 * r0 + r1 * r1, rho);
        const float w = sqrtf(w2);
        const float fx = fxs[cam], fy = fys[cam], iz = 1.f / t.z;
        const float j00 = fx * iz, j02 = -fx * t.x * iz * iz, j11 = fy * iz, j12 = -fy * t.y * iz * iz;
        const Vec3<float> u0 = v3<float>(j00 * Rn[0] + j02 * Rn[2], j00 * Rn[3] + j02 * Rn[5], j00 * Rn[6] + j02 * Rn[8]);
        const Vec3<float> u1 = v3<float>(j11 * Rn[1] + j12 * Rn[2], j11 * Rn[4] + j12 * Rn[5], j11 * Rn[7] + j12 * Rn[8]);
        const float ja0 = dot(u0, dXda), ja1 = dot(u1, dXda);
        accC += w2 * (ja0 * ja0 + ja1 * ja1);
        accG += w2 * (ja0 * r0 + ja1 * r1);
        RW[cam][0] = sgn * (w * r0);
        RW[cam][1] = sgn * (w * r1);
        const float jw0 = sgn * (w * ja0), jw1 = sgn * (w * ja1);
        JW[cam][0] = jw0;
        JW[cam][1] = jw1;
        if (has_pose) {
          const Vec3<float> k0 = cross(Xp, u0), k1 = cross(Xp, u1);
          K[cam][0][0] = w * k0.x; K[cam][0][1] = w * k0.y; K[cam][0][2] = w * k0.z;
          K[cam][0][3] = w * u0.x; K[cam][0][4] = w * u0.y; K[cam][0][5] = w * u0.z;
          K[cam][1][0] = w * k1.x; K[cam][1][1] = w * k1.y; K[cam][1][2] = w * k1.z;
          K[cam][1][3] = w * u1.x; K[cam][1][4] = w * u1.y; K[cam][1][5] = w * u1.z;
        }
      }
      atomicAdd(&sm.C[slot], accC);
      atomicAdd(&sm.ga[slot], accG);
      if (has_pose) {
        key = n;
        // the observation's slab term q = sum over its rows of (w h)(s w j_alpha), h the
        // pose row about the anchor centre: from the same rounded rows w K (about the
        // pair origin, X + d) as the pair records, each value an exact four-product sum,
        // then moved to the anchor centre in double-float: q_w -= d x q_v
        df q[6];
#pragma unroll
        for (int k = 0; k < 6; ++k)
          q[k] = sum4_prod(K[0][0][k], JW[0][0], K[0][1][k], JW[0][1], K[1][0][k], JW[1][0], K[1][1][k], JW[1][1]);
        if (lo != a) {
          const df c0 = q[5] * d.y - q[4] * d.z, c1 = q[3] * d.z - q[5] * d.x, c2 = q[4] * d.x - q[3] * d.y;  // d x q_v
          q[0] = q[0] - c0;
          q[1] = q[1] - c1;
          q[2] = q[2] - c2;
        }
        // frames after the anchor cover blocks [a, n): row n - 1 feeds a suffix sum;
        // frames before it cover [n, a): row n feeds a prefix sum.  Rows are distinct.
        const int row = (n > a ? n - 1 : n) - f0;
        const size_t at = (size_t)(6 * row) * SPGO_CHUNK + slot;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          slab_h[at + k * SPGO_CHUNK] = q[k].h;
          slab_l[at + k * SPGO_CHUNK] = q[k].l;
        }
      }
    }
    {
      // exactly summed g_a: the observation's j_a^T W r (the signs of JW and RW cancel),
      // added by the lanes sharing a landmark in rounds of their rank among those peers
      const df vg = slot >= 0 ? sum4_prod(JW[0][0], RW[0][0], JW[0][1], RW[0][1], JW[1][0], RW[1][0], JW[1][1],
                                          RW[1][1])
                              : df_make(0.f);
      const unsigned peers = __match_any_sync(0xffffffffu, slot);
      const int rank = __popc(peers & ((1u << lane) - 1u));
      for (int r = 0; __any_sync(0xffffffffu, slot >= 0 && rank >= r); ++r) {
        if (slot >= 0 && rank == r) {
          df_acc a;
          a.h = sm.glh[tid >> 5][slot];
          a.l = sm.gll[tid >> 5][slot];
          a.add(vg.h, vg.l);
          sm.glh[tid >> 5][slot] = a.h;
          sm.gll[tid >> 5][slot] = a.l;
        }
        __syncwarp();
      }
    }
    // the 27 pair values in three rounds of 9: each staged as double-float rows, then
    // summed over the runs of equal target frame into the FP64 pair records
    float *st = stage + (size_t)(tid >> 5) * 2 * kJacRound * kJacPitch;
    int *keys = sm.key[tid >> 5];
    keys[lane] = key;
    const bool any_pose = __any_sync(0xffffffffu, key >= 0);
    if (any_pose) {
      const int host_a = sm.a[0];
      jac_stage<0, kJacRound>(K, RW, st, lane);
      __syncwarp();
      jac_runs<0, kJacRound>(st, keys, lane, host_a, D, pair_base);
      __syncwarp();
      jac_stage<kJacRound, 2 * kJacRound>(K, RW, st, lane);
      __syncwarp();
      jac_runs<kJacRound, 2 * kJacRound>(st, keys, lane, host_a, D, pair_base);
      __syncwarp();
      jac_stage<2 * kJacRound, kJacVals>(K, RW, st, lane);
      __syncwarp();
      jac_runs<2 * kJacRound, kJacVals>(st, keys, lane, host_a, D, pair_base);
    }
    __syncwarp();
  }
  __syncthreads();

  // phase C.1: per (landmark, component) suffix / prefix sums along the window (double-float)
  for (int idx = tid; idx < cnt * 6; idx += blockDim.x) {
    const int slot = idx % cnt, k = idx / cnt;
    const int a = sm.a[slot], lo_l = sm.lo[slot], hi_l = sm.hi[slot];
    df acc = df_make(0.f);
    for (int i = hi_l - 1; i >= a; --i) {
      const size_t at = (size_t)(6 * (i - f0) + k) * SPGO_CHUNK + slot;
      acc = acc + df{slab_h[at], slab_l[at]};
      slab_h[at] = acc.h;
      slab_l[at] = acc.l;
    }
    acc = df_make(0.f);
    for (int i = lo_l; i < a; ++i) {
      const size_t at = (size_t)(6 * (i - f0) + k) * SPGO_CHUNK + slot;
      acc = acc + df{slab_h[at], slab_l[at]};
      slab_h[at] = acc.h;
      slab_l[at] = acc.l;
    }
  }
  __syncthreads();
  // phase C.2: B_l(i) = Ad_i^T b_l(i) about the anchor centre,
  //   [R_i^T (b_w - (c_i - c_a) x b_v) ; R_i^T b_v], in double-float, rounded once,
  // for the (landmark, frame) pairs inside the landmark's window [lo, hi) only (about
  // 60 % of the chunk window's pairs), enumerated row by row so that a warp's lanes
  // take different landmarks (slab columns, distinct banks); each result replaces its
  // own b_l(i) in slab_h, whose other entries (outside the windows, empty columns) are
  // still zero
  const int n_in = sm.rsp[nb];
  for (int j = tid; j < n_in; j += blockDim.x) {
    int row = 0;  // the last window row whose pairs start at or before pair j
#pragma unroll
    for (int step = 64; step >= 1; step >>= 1)
      if (row + step < nb && sm.rsp[row + step] <= j) row += step;
    // the landmark: the (j - rsp[row])-th set bit of the row's mask
    unsigned m = sm.rmask[row];
    int r = j - sm.rsp[row], slot = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
      const int c = __popc(m & ((1u << w) - 1u));
      if (r >= c) {
        r -= c;
        m >>= w;
        slot += w;
      }
    }
    const int i = f0 + row;
    const size_t at = (size_t)(6 * (i - f0)) * SPGO_CHUNK + slot;
    const float *Rh = wv.fr_Rf + (size_t)(fo + i) * 18, *Rl = wv.fr_Rl + (size_t)(fo + i) * 18;
    df d[3], bw[3], bv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      // c_i - c_a: the negated host-to-frame offset of the window table (one host per chunk)
      d[k] = df{-dch[(i - f0) * 6 + k], -dcl[(i - f0) * 6 + k]};
      bw[k] = df{slab_h[at + k * SPGO_CHUNK], slab_l[at + k * SPGO_CHUNK]};
      bv[k] = df{slab_h[at + (3 + k) * SPGO_CHUNK], slab_l[at + (3 + k) * SPGO_CHUNK]};
    }
    const df tw[3] = {bw[0] - (d[1] * bv[2] - d[2] * bv[1]), bw[1] - (d[2] * bv[0] - d[0] * bv[2]),
                      bw[2] - (d[0] * bv[1] - d[1] * bv[0])};
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      // (R^T v)_r = sum_k R(k, r) v_k
      const df Bw = df_dot3(Rh[r], Rl[r], Rh[3 + r], Rl[3 + r], Rh[6 + r], Rl[6 + r], tw[0], tw[1], tw[2]);
      const df Bv = df_dot3(Rh[r], Rl[r], Rh[3 + r], Rl[3 + r], Rh[6 + r], Rl[6 + r], bv[0], bv[1], bv[2]);
      slab_h[at + r * SPGO_CHUNK] = Bw.h + Bw.l;
      slab_h[at + (3 + r) * SPGO_CHUNK] = Bv.h + Bv.l;
    }
  }
  __syncthreads();
  {  // the chunk's slab, every row and all 32 columns (the Schur pass reads them all)
    float4 *g4 = reinterpret_cast<float4 *>(reinterpret_cast<float *>(wv.slab) + pv.ch_slab[c]);
    const float4 *s4 = reinterpret_cast<const float4 *>(slab_h);
    for (int idx = tid; idx < rows * (SPGO_CHUNK / 4); idx += blockDim.x) g4[idx] = s4[idx];
  }
  if (tid < cnt) {
    reinterpret_cast<float *>(wv.C)[lm0 + tid] = sm.C[tid];
    reinterpret_cast<float *>(wv.ga)[lm0 + tid] = sm.ga[tid];
    if (wv.gaacc) {
      df_acc g;
#pragma unroll
      for (int w = 0; w < 8; ++w) g.add(sm.glh[w][tid], sm.gll[w][tid]);
      wv.gaacc[lm0 + tid] = df_acc_value(g);
    }
  }
}

// ---- the FP32 path's pose chain in double-float ----
// The same scan with 3x4 products in double-float (~48 significant bits, the
// precision of the FP32 path's frame tables: fr_Rf + fr_Rl, fr_ch + fr_cl), on the
// FP32 pipes instead of FP64 (which runs at a small fraction of their rate on
// this GPU).  Writes only the tables the FP32 kernels read.
__device__ __forceinline__ void compose34_df(const df *A, const df *B, df *C) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      df v = df_dot3(A[4 * i].h, A[4 * i].l, A[4 * i + 1].h, A[4 * i + 1].l, A[4 * i + 2].h, A[4 * i + 2].l,
                     B[j], B[4 + j], B[8 + j]);
      if (j == 3) v = v + A[4 * i + 3];
      C[4 * i + j] = v;
    }
  }
}

// (also the FP64 copies, h + l, which the FP64 reduction of the pose-pair records reads)
__device__ __forceinline__ void write_frame_df(const WorkView &wv, size_t f, const df *G, const df *Trl) {
  df Gr[12];
  compose34_df(G, Trl, Gr);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      wv.fr_Rf[f * 18 + 3 * i + j] = G[4 * i + j].h;
      wv.fr_Rf[f * 18 + 9 + 3 * i + j] = Gr[4 * i + j].h;
      wv.fr_Rl[f * 18 + 3 * i + j] = G[4 * i + j].l;
      wv.fr_Rl[f * 18 + 9 + 3 * i + j] = Gr[4 * i + j].l;
      wv.fr_Rd[f * 18 + 3 * i + j] = (double)G[4 * i + j].h + (double)G[4 * i + j].l;
      wv.fr_Rd[f * 18 + 9 + 3 * i + j] = (double)Gr[4 * i + j].h + (double)Gr[4 * i + j].l;
    }
    wv.fr_ch[f * 6 + i] = G[4 * i + 3].h;
    wv.fr_ch[f * 6 + 3 + i] = Gr[4 * i + 3].h;
    wv.fr_cl[f * 6 + i] = G[4 * i + 3].l;
    wv.fr_cl[f * 6 + 3 + i] = Gr[4 * i + 3].l;
    wv.fr_c[f * 6 + i] = (double)G[4 * i + 3].h + (double)G[4 * i + 3].l;
    wv.fr_c[f * 6 + 3 + i] = (double)Gr[4 * i + 3].h + (double)Gr[4 * i + 3].l;
  }
}

__global__ void k_chain_df(PlanView pv, WorkView wv, const double *__restrict__ poses, int gate) {
  const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= pv.B) return;
  if (!problem_active(wv.lm, b, gate)) return;
  const int N = pv.p_npose[b], fo = pv.p_frame_off[b], po = pv.p_pose_off[b];
  df Trl[12], carry[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) {
    Trl[q] = df_from_double(pv.p_Trl[12 * b + q]);
    carry[q] = df_make((q == 0 || q == 5 || q == 10) ? 1.f : 0.f);
  }
  if (lane == 0) write_frame_df(wv, (size_t)fo, carry, Trl);
  for (int s = 0; s < N; s += 32) {
    const int k = s + lane;
    df M[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) M[q] = df_make((q == 0 || q == 5 || q == 10) ? 1.f : 0.f);
    if (k < N) {  // inverse of the incremental pose: [R^T, -R^T t]
      const double *T = poses + 12 * (size_t)(po + k);
      df Td[12];
#pragma unroll
      for (int q = 0; q < 12; ++q) Td[q] = df_from_double(T[q]);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) M[4 * i + j] = Td[4 * j + i];
        M[4 * i + 3] = -df_dot3(Td[i].h, Td[i].l, Td[4 + i].h, Td[4 + i].l, Td[8 + i].h, Td[8 + i].l, Td[3], Td[7],
                                Td[11]);
      }
    }
    // inclusive scan: M_k <- M_0 M_1 ... M_k (earlier factors on the left)
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      df P[12];
#pragma unroll
      for (int q = 0; q < 12; ++q)
        P[q] = df{__shfl_up_sync(0xffffffffu, M[q].h, d), __shfl_up_sync(0xffffffffu, M[q].l, d)};
      if (lane >= d) {
        df C[12];
        compose34_df(P, M, C);
#pragma unroll
        for (int q = 0; q < 12; ++q) M[q] = C[q];
      }
    }
    df G[12];
    compose34_df(carry, M, G);
    if (k < N) write_frame_df(wv, (size_t)(fo + k + 1), G, Trl);
#pragma unroll
    for (int q = 0; q < 12; ++q) carry[q] = df{__shfl_sync(0xffffffffu, G[q].h, 31), __shfl_sync(0xffffffffu, G[q].l, 31)};
  }
}

int launch_chain(const PlanView &pv, const WorkView &wv, const double *poses, int gate, int f64, void *stream) {
  if (f64)
    k_chain<<<pv.B, 32, 0, (cudaStream_t)stream>>>(pv, wv, poses, gate);  // one warp (and SM slot) per problem
  else
    k_chain_df<<<pv.B, 32, 0, (cudaStream_t)stream>>>(pv, wv, poses, gate);
  ++g_launches;
  return (int)cudaGetLastError();
}

constexpr int kCostThreads = 64;   // cost pass: short CTAs, many per SM (latency-bound)
constexpr int kLinThreads = 256;

template <typename T>
int launch_linearize(const PlanView &pv, const WorkView &wv, const Params &prm, const double *alpha,
                     int cost_only, int gate, void *stream) {
  if (pv.n_chunks == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  if (cost_only) {
    const int nt = prm.cost_block > 0 ? prm.cost_block : kCostThreads;
    const size_t sm = LinLayout<T>(pv.max_nb, nt / 32, true).total;
    k_linearize<T, true><<<pv.n_chunks, nt, sm, st>>>(pv, wv, prm, alpha, gate);
  } else if constexpr (std::is_same<T, float>::value) {
    const int nt = prm.lin_block > 0 ? prm.lin_block : kLinThreads;
    const size_t sm = JacLayout(pv.max_nb, nt / 32).total;
    cudaFuncSetAttribute(k_jacobian_acc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    // all of the unified L1 / shared memory as shared: three CTAs of 74.6 KB per SM
    cudaFuncSetAttribute(k_jacobian_acc, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxShared);
    k_jacobian_acc<<<pv.n_chunks, nt, sm, st>>>(pv, wv, prm, alpha, gate);
  } else {
    const int nt = prm.lin_block > 0 ? prm.lin_block : kLinThreads;
    const size_t sm = LinLayout<T>(pv.max_nb, nt / 32, false).total;
    cudaFuncSetAttribute(k_linearize<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_linearize<T, false><<<pv.n_chunks, nt, sm, st>>>(pv, wv, prm, alpha, gate);
  }
  ++g_launches;
  return (int)cudaGetLastError();
}

template int launch_linearize<float>(const PlanView &, const WorkView &, const Params &, const double *, int, int, void *);
template int launch_linearize<double>(const PlanView &, const WorkView &, const Params &, const double *, int, int, void *);

}  // namespace spgo
