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

namespace spgo {

template <typename T> __device__ __forceinline__ const T *frame_R(const WorkView &wv, int f, int cam);
template <> __device__ __forceinline__ const float *frame_R<float>(const WorkView &wv, int f, int cam) {
  return wv.fr_Rf + (size_t)f * 18 + cam * 9;
}
template <> __device__ __forceinline__ const double *frame_R<double>(const WorkView &wv, int f, int cam) {
  return wv.fr_Rd + (size_t)f * 18 + cam * 9;
}

// ---- global poses: G[0] = I, G[k+1] = G[k] inv(T_k); right camera G T_r_to_l ----
// One thread per problem, FP64 (Solver_cuda.cu:472-491).
__global__ void k_chain(PlanView pv, WorkView wv, const double *__restrict__ poses, int gate) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= pv.B) return;
  if (!problem_active(wv.lm, b, gate)) return;
  const int N = pv.p_npose[b], fo = pv.p_frame_off[b], po = pv.p_pose_off[b];
  const double *Trl = pv.p_Trl + 12 * b;
  double G[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  for (int k = 0; k <= N; ++k) {
    if (k > 0) {
      double Ti[12], Gn[12];
      invert34(poses + 12 * (size_t)(po + k - 1), Ti);
      compose34(G, Ti, Gn);
#pragma unroll
      for (int q = 0; q < 12; ++q) G[q] = Gn[q];
    }
    double Gr[12];
    compose34(G, Trl, Gr);
    const size_t f = (size_t)(fo + k);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        wv.fr_Rd[f * 18 + 3 * i + j] = G[4 * i + j];
        wv.fr_Rd[f * 18 + 9 + 3 * i + j] = Gr[4 * i + j];
        wv.fr_Rf[f * 18 + 3 * i + j] = (float)G[4 * i + j];
        wv.fr_Rf[f * 18 + 9 + 3 * i + j] = (float)Gr[4 * i + j];
      }
      wv.fr_c[f * 6 + i] = G[4 * i + 3];
      wv.fr_c[f * 6 + 3 + i] = Gr[4 * i + 3];
    }
  }
}

// upper-triangle index of a symmetric 6x6 (row i <= col j)
__device__ __forceinline__ constexpr int tri6(int i, int j) { return i * 6 - (i * (i - 1)) / 2 + (j - i); }

// ---- fused linearisation / cost -----------------------------------------------
// Grid: one CTA (8 warps) per chunk of <= 32 landmarks; one warp per landmark,
// lanes over its observations.  COST = true evaluates the cost only.
template <typename T, bool COST>
__global__ void __launch_bounds__(256) k_linearize(PlanView pv, WorkView wv, Params prm,
                                                   const double *__restrict__ alpha_state, int gate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int c = blockIdx.x;
  const int b = pv.ch_prob[c];
  if (!problem_active(wv.lm, b, gate)) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int f0 = pv.ch_f0[c], nb = pv.ch_nb[c], lm0 = pv.ch_lm0[c], cnt = pv.ch_cnt[c];
  const int fo = pv.p_frame_off[b];
  const int D = pv.p_pair_D[b];
  const int64_t pair_base = pv.p_pair_off[b];
  const float *intr = pv.p_intr + 8 * b;
  const T fxs[2] = {(T)intr[0], (T)intr[4]}, fys[2] = {(T)intr[1], (T)intr[5]};
  const T cxs[2] = {(T)intr[2], (T)intr[6]}, cys[2] = {(T)intr[3], (T)intr[7]};
  const T lscale = (T)prm.loss_scale;

  const int rows = 6 * nb;
  T *slab_s = reinterpret_cast<T *>(smem_raw);                 // [rows][32]
  T *q_s = slab_s + (COST ? 0 : rows * SPGO_CHUNK);            // [8][32][6]
  int *qr_s = reinterpret_cast<int *>(q_s + (COST ? 0 : 8 * 32 * 6));  // [8][32][2]
  if (!COST) {
    for (int i = tid; i < rows * SPGO_CHUNK; i += blockDim.x) slab_s[i] = T(0);
    __syncthreads();
  }
  T *pair_acc = reinterpret_cast<T *>(wv.pair_acc);

  double cost_lane = 0.0;
  for (int s = warp; s < cnt; s += 8) {
    const int li = lm0 + s;
    const int a = pv.lm_host[li];
    const int lo_l = pv.lm_lo[li], hi_l = pv.lm_hi[li];
    const T alpha = (T)alpha_state[pv.lm_user[li]];
    const T ua = (T)pv.lm_uv[2 * li], va = (T)pv.lm_uv[2 * li + 1];
    const int fa = fo + a;
    const T *Ra = frame_R<T>(wv, fa, 0);
    const double *ca = wv.fr_c + (size_t)fa * 6;
    // anchor ray t_a = K_l^-1 p_a / alpha, rotated to world axes (origin: anchor centre)
    const Vec3<T> ta = v3<T>((ua - cxs[0]) / fxs[0] / alpha, (va - cys[0]) / fys[0] / alpha, T(1) / alpha);
    const Vec3<T> X = mul(Ra, ta);
    const Vec3<T> dXda = v3<T>(-X.x / alpha, -X.y / alpha, -X.z / alpha);
    T accC = T(0), accG = T(0);
    const int64_t ob = pv.lm_obs[li], oe = pv.lm_obs[li + 1];
    for (int64_t base = ob; base < oe; base += 32) {
      const int64_t o = base + lane;
      T q[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
      int qlo = 0, qhi = 0;
      if (o < oe) {
        const int n = pv.obs_frame[o];
        const float4 z = reinterpret_cast<const float4 *>(pv.obs_uv)[o];
        const int fn = fo + n;
        const bool has_pose = (n != a);
        const int lo = min(a, n), hi = max(a, n);
        const T sgn = n > a ? T(1) : T(-1);
        Vec3<T> Xp = X;  // point relative to the pair origin (left centre of frame lo)
        if (!COST && has_pose && lo != a) {
          const double *cl = wv.fr_c + (size_t)(fo + lo) * 6;
          Xp = v3<T>(X.x + (T)(ca[0] - cl[0]), X.y + (T)(ca[1] - cl[1]), X.z + (T)(ca[2] - cl[2]));
        }
        T M[21], m[6];
        if (!COST) {
#pragma unroll
          for (int k = 0; k < 21; ++k) M[k] = T(0);
#pragma unroll
          for (int k = 0; k < 6; ++k) m[k] = T(0);
        }
        const T boost = (prm.near_boost && abs(n - a) < 2) ? T(16) : T(1);
#pragma unroll
        for (int cam = 0; cam < 2; ++cam) {
          const T *Rn = frame_R<T>(wv, fn, cam);
          const double *cn = wv.fr_c + (size_t)fn * 6 + cam * 3;
          const Vec3<T> Xc = v3<T>(X.x + (T)(ca[0] - cn[0]), X.y + (T)(ca[1] - cn[1]), X.z + (T)(ca[2] - cn[2]));
          const Vec3<T> t = mulT(Rn, Xc);
          const T iz = T(1) / t.z;
          const T fx = fxs[cam], fy = fys[cam];
          const T r0 = (T)(cam ? z.z : z.x) - (fx * t.x * iz + cxs[cam]);
          const T r1 = (T)(cam ? z.w : z.y) - (fy * t.y * iz + cys[cam]);
          T rho;
          const T w2 = boost * robust<T>(prm.loss, lscale, r0 * r0 + r1 * r1, rho);
          cost_lane += 0.5 * (double)(boost * rho);
          if (COST) continue;
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
        if (!COST && has_pose) {
          T *dst = pair_acc + (size_t)(pair_base + (int64_t)lo * D + (hi - lo - 1)) * 27;
#pragma unroll
          for (int k = 0; k < 21; ++k) red_add(dst + k, M[k]);
#pragma unroll
          for (int k = 0; k < 6; ++k) red_add(dst + 21 + k, m[k]);
          qlo = lo;
          qhi = hi;
        }
      }
      if (!COST) {
        // b_l(i) += sum of q over this batch's observations whose range covers i
        T *qw = q_s + (size_t)(warp * 32 + lane) * 6;
#pragma unroll
        for (int k = 0; k < 6; ++k) qw[k] = q[k];
        qr_s[(warp * 32 + lane) * 2] = qlo;
        qr_s[(warp * 32 + lane) * 2 + 1] = qhi;
        __syncwarp();
        const int nq = (int)min((int64_t)32, oe - base);
        for (int bi = lane; bi < hi_l - lo_l; bi += 32) {
          const int i = lo_l + bi;
          T acc[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
          for (int j = 0; j < nq; ++j) {
            const int jlo = qr_s[(warp * 32 + j) * 2], jhi = qr_s[(warp * 32 + j) * 2 + 1];
            if (jlo <= i && i < jhi) {
              const T *qj = q_s + (size_t)(warp * 32 + j) * 6;
#pragma unroll
              for (int k = 0; k < 6; ++k) acc[k] += qj[k];
            }
          }
          T *dst = slab_s + (size_t)(6 * (i - f0)) * SPGO_CHUNK + s;
#pragma unroll
          for (int k = 0; k < 6; ++k) dst[k * SPGO_CHUNK] += acc[k];
        }
        __syncwarp();
      }
    }
    if (!COST) {
      accC = warp_sum(accC);
      accG = warp_sum(accG);
      if (lane == 0) {
        reinterpret_cast<T *>(wv.C)[li] = accC;
        reinterpret_cast<T *>(wv.ga)[li] = accG;
      }
      // B_l(i) = Ad_i^T b_l(i) about the anchor centre:
      //   [R_i^T (b_w - (c_i - c_a) x b_v) ; R_i^T b_v]
      for (int bi = lane; bi < hi_l - lo_l; bi += 32) {
        const int i = lo_l + bi;
        const int fi = fo + i;
        const T *Ri = frame_R<T>(wv, fi, 0);
        const double *ci = wv.fr_c + (size_t)fi * 6;
        const Vec3<T> d = v3<T>((T)(ci[0] - ca[0]), (T)(ci[1] - ca[1]), (T)(ci[2] - ca[2]));
        T *dst = slab_s + (size_t)(6 * (i - f0)) * SPGO_CHUNK + s;
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
    }
  }
  const double cw = warp_sum(cost_lane);
  if (lane == 0 && cw != 0.0) atomicAdd(wv.cost_acc + b, cw);
  if (!COST) {
    __syncthreads();
    T *gslab = reinterpret_cast<T *>(wv.slab) + pv.ch_slab[c];
    for (int i = tid; i < rows * SPGO_CHUNK; i += blockDim.x) gslab[i] = slab_s[i];
  }
}

int launch_chain(const PlanView &pv, const WorkView &wv, const double *poses, int gate, void *stream) {
  k_chain<<<grid_for(pv.B, 128), 128, 0, (cudaStream_t)stream>>>(pv, wv, poses, gate);
  ++g_launches;
  return (int)cudaGetLastError();
}

template <typename T>
static size_t lin_smem(int max_nb, bool cost) {
  if (cost) return 16;
  return (size_t)6 * max_nb * SPGO_CHUNK * sizeof(T) + (size_t)8 * 32 * 6 * sizeof(T) + (size_t)8 * 32 * 2 * sizeof(int);
}

template <typename T>
int launch_linearize(const PlanView &pv, const WorkView &wv, const Params &prm, const double *alpha,
                     int cost_only, int gate, void *stream) {
  if (pv.n_chunks == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  if (cost_only) {
    k_linearize<T, true><<<pv.n_chunks, 256, lin_smem<T>(pv.max_nb, true), st>>>(pv, wv, prm, alpha, gate);
  } else {
    const size_t sm = lin_smem<T>(pv.max_nb, false);
    cudaFuncSetAttribute(k_linearize<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_linearize<T, false><<<pv.n_chunks, 256, sm, st>>>(pv, wv, prm, alpha, gate);
  }
  ++g_launches;
  return (int)cudaGetLastError();
}

template int launch_linearize<float>(const PlanView &, const WorkView &, const Params &, const double *, int, int, void *);
template int launch_linearize<double>(const PlanView &, const WorkView &, const Params &, const double *, int, int, void *);

}  // namespace spgo
