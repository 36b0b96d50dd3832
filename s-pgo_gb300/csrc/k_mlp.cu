// Learned LM damping controller: a 16 -> 64 -> 64 -> 2 MLP with exact GELU.
//
// No counterpart in the reference (S-PGO has no damping schedule at all).
// Parameters are one flat FP32 vector: W1 [64x16] (out x in), b1 [64],
// W2 [64x64], b2 [64], W3 [2x64], b3 [2]  (5378 floats).  Outputs: out0 =
// proposed change of log10(lambda), out1 = logit that the current damping gives
// an accepted step.  Training loss per sample: (out0 - t0)^2 + BCE(out1, t1),
// averaged over the batch.
//
// Kernels: FP32 forward (thread per sample, weights in shared memory), fused
// loss + per-sample deltas (thread per sample), the parameter gradient as batch
// sums (thread per parameter, no atomics), Adam, and the BF16 inference the LM
// loop runs (warp per problem, FP32 accumulation).
#include <cuda_bf16.h>

#include "kernels.cuh"
#include "dfloat.cuh"

#include <type_traits>

namespace spgo {

constexpr int kIn = 16, kH = 64, kOut = 2;
constexpr int kW1 = 0, kB1 = kW1 + kH * kIn, kW2 = kB1 + kH, kB2 = kW2 + kH * kH, kW3 = kB2 + kH,
              kB3 = kW3 + kOut * kH, kParams = kB3 + kOut;
static_assert(kParams == SPGO_MLP_PARAMS, "parameter count");

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * expf(-0.5f * x * x) * 0.39894228040143268f;
}

// forward; cache (optional) holds z1 [n x 64] then z2 [n x 64]
__global__ void __launch_bounds__(128) k_mlp_fwd(const float *__restrict__ theta, const float *__restrict__ X, int n,
                                                 float *__restrict__ out, float *__restrict__ cache) {
  __shared__ float W[kParams];
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) W[i] = theta[i];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float x[kIn];
#pragma unroll
  for (int k = 0; k < kIn; ++k) x[k] = X[(size_t)s * kIn + k];
  float h1[kH];
#pragma unroll 4
  for (int j = 0; j < kH; ++j) {
    float z = W[kB1 + j];
#pragma unroll
    for (int k = 0; k < kIn; ++k) z += W[kW1 + j * kIn + k] * x[k];
    if (cache) cache[(size_t)s * kH + j] = z;
    h1[j] = gelu(z);
  }
  float o0 = W[kB3], o1 = W[kB3 + 1];
  for (int j = 0; j < kH; ++j) {
    float z = W[kB2 + j];
#pragma unroll 8
    for (int k = 0; k < kH; ++k) z += W[kW2 + j * kH + k] * h1[k];
    if (cache) cache[(size_t)n * kH + (size_t)s * kH + j] = z;
    const float h2 = gelu(z);
    o0 += W[kW3 + j] * h2;
    o1 += W[kW3 + kH + j] * h2;
  }
  out[2 * s] = o0;
  out[2 * s + 1] = o1;
}

// Backward in two passes, no atomics on the parameters:
//   k_mlp_delta  (thread per sample): loss, and the per-sample activations and
//                deltas h1, h2, dz1, dz2, dout into the cache;
//   k_mlp_param  (thread per parameter): the batch sum of delta x activation,
//                written straight into grad.
// Cache layout (floats): [z1 | z2 | h1 | h2 | dz1 | dz2] each n x 64, then dout n x 2.
constexpr int kCachePerSample = 6 * kH + 2;
static_assert(kCachePerSample == SPGO_MLP_CACHE_PER_SAMPLE, "cache size");

__global__ void __launch_bounds__(128) k_mlp_delta(const float *__restrict__ theta, const float *__restrict__ T, int n,
                                                   const float *__restrict__ out, float *__restrict__ cache,
                                                   float *__restrict__ loss) {
  __shared__ float W[kParams];
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) W[i] = theta[i];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  float lsum = 0.f;
  if (s < n) {
    const size_t nh = (size_t)n * kH;
    const float *z1 = cache + (size_t)s * kH;
    const float *z2 = cache + nh + (size_t)s * kH;
    float *h1 = cache + 2 * nh + (size_t)s * kH;
    float *h2 = cache + 3 * nh + (size_t)s * kH;
    float *dz1 = cache + 4 * nh + (size_t)s * kH;
    float *dz2 = cache + 5 * nh + (size_t)s * kH;
    float *dout = cache + 6 * nh + 2 * (size_t)s;
    const float inv_n = 1.f / (float)n;
    const float o0 = out[2 * s], o1 = out[2 * s + 1];
    const float t0 = T[2 * s], t1 = T[2 * s + 1];
    const float sig = 1.f / (1.f + expf(-o1));
    lsum = (o0 - t0) * (o0 - t0) + (fmaxf(o1, 0.f) + log1pf(expf(-fabsf(o1)))) - t1 * o1;
    const float d0 = 2.f * (o0 - t0) * inv_n, d1 = (sig - t1) * inv_n;
    dout[0] = d0;
    dout[1] = d1;
    float g2[kH];
    for (int j = 0; j < kH; ++j) {
      const float zj = z2[j];
      h2[j] = gelu(zj);
      g2[j] = (d0 * W[kW3 + j] + d1 * W[kW3 + kH + j]) * gelu_grad(zj);
      dz2[j] = g2[j];
    }
    for (int k = 0; k < kH; ++k) {
      const float zk = z1[k];
      h1[k] = gelu(zk);
      float acc = 0.f;
#pragma unroll 8
      for (int j = 0; j < kH; ++j) acc += g2[j] * W[kW2 + j * kH + k];
      dz1[k] = acc * gelu_grad(zk);
    }
  }
  lsum = warp_sum(lsum);
  if ((threadIdx.x & 31) == 0 && lsum != 0.f) atomicAdd(loss, lsum / (float)n);
}

__global__ void __launch_bounds__(128) k_mlp_param(const float *__restrict__ X, int n, const float *__restrict__ cache,
                                                   float *__restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  const size_t nh = (size_t)n * kH;
  const float *h1 = cache + 2 * nh, *h2 = cache + 3 * nh, *dz1 = cache + 4 * nh, *dz2 = cache + 5 * nh;
  const float *dout = cache + 6 * nh;
  float acc = 0.f;
  if (p < kB1) {
    const int j = p / kIn, k = p % kIn;
    for (int s = 0; s < n; ++s) acc += dz1[(size_t)s * kH + j] * X[(size_t)s * kIn + k];
  } else if (p < kW2) {
    const int j = p - kB1;
    for (int s = 0; s < n; ++s) acc += dz1[(size_t)s * kH + j];
  } else if (p < kB2) {
    const int j = (p - kW2) / kH, k = (p - kW2) % kH;
    for (int s = 0; s < n; ++s) acc += dz2[(size_t)s * kH + j] * h1[(size_t)s * kH + k];
  } else if (p < kW3) {
    const int j = p - kB2;
    for (int s = 0; s < n; ++s) acc += dz2[(size_t)s * kH + j];
  } else if (p < kB3) {
    const int o = (p - kW3) / kH, j = (p - kW3) % kH;
    for (int s = 0; s < n; ++s) acc += dout[2 * (size_t)s + o] * h2[(size_t)s * kH + j];
  } else {
    const int o = p - kB3;
    for (int s = 0; s < n; ++s) acc += dout[2 * (size_t)s + o];
  }
  grad[p] = acc;
}

__global__ void k_mlp_adam(float *theta, const float *grad, float *m, float *v, int step, float lr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float b1 = 0.9f, b2 = 0.999f, e = 1e-8f;
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * g;
  const float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.f - powf(b1, (float)step)), vh = vi / (1.f - powf(b2, (float)step));
  theta[i] -= lr * mh / (sqrtf(vh) + e);
}

// the controller's inference weights: each parameter rounded to BF16, stored as
// FP32 in the shared-memory layout below (weight matrices transposed)
__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16(v)); }

// BF16-weight inference, one feature vector per warp: lanes split the hidden
// units, FP32 accumulation.  The weights live in shared memory as FP32 copies of
// the BF16-rounded parameters, both matrices transposed so that lanes read
// consecutive hidden units; spgo_lm_set_controller writes that layout once into
// the workspace and every controller launch copies it in with 16-byte loads.
struct MlpSmem {
  float w1t[kIn][kH], b1[kH], w2t[kH][kH], b2[kH], w3[kOut][kH], b3[kOut];
  float pad[2];  // 16-byte multiple
};
static_assert(sizeof(MlpSmem) % 16 == 0, "float4 staging");

__global__ void k_mlp_deploy(const float *__restrict__ theta, MlpSmem *__restrict__ m) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kH * kIn) m->w1t[i % kIn][i / kIn] = bf16r(theta[kW1 + i]);
  if (i < kH * kH) m->w2t[i % kH][i / kH] = bf16r(theta[kW2 + i]);
  if (i < kH) {
    m->b1[i] = bf16r(theta[kB1 + i]);
    m->b2[i] = bf16r(theta[kB2 + i]);
    m->w3[0][i] = bf16r(theta[kW3 + i]);
    m->w3[1][i] = bf16r(theta[kW3 + kH + i]);
  }
  if (i < kOut) m->b3[i] = bf16r(theta[kB3 + i]);
  if (i < 2) m->pad[i] = 0.f;
}

__device__ void stage_mlp(const MlpSmem *__restrict__ src, MlpSmem &m) {
  const float4 *s4 = reinterpret_cast<const float4 *>(src);
  float4 *d4 = reinterpret_cast<float4 *>(&m);
  constexpr int n = (int)(sizeof(MlpSmem) / 16);
  for (int i0 = threadIdx.x; i0 < n; i0 += 8 * blockDim.x) {  // eight 16-byte loads in flight
    float4 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int i = i0 + q * blockDim.x;
      if (i < n) v[q] = s4[i];
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int i = i0 + q * blockDim.x;
      if (i < n) d4[i] = v[q];
    }
  }
}

__device__ void mlp_infer_warp(const MlpSmem &m, const float *x, float &o0, float &o1) {
  const int lane = threadIdx.x & 31;
  float h1[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int j = lane + 32 * q;
    float z = m.b1[j];
#pragma unroll
    for (int k = 0; k < kIn; ++k) z += m.w1t[k][j] * x[k];
    h1[q] = gelu(z);
  }
  float p0 = 0.f, p1 = 0.f;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int j = lane + 32 * q;
    float z = m.b2[j];
#pragma unroll 8
    for (int k = 0; k < kH; ++k) {
      const float hk = __shfl_sync(0xffffffffu, h1[k >> 5], k & 31);
      z += m.w2t[k][j] * hk;
    }
    const float h2 = gelu(z);
    p0 += m.w3[0][j] * h2;
    p1 += m.w3[1][j] * h2;
  }
  o0 = warp_sum(p0) + m.b3[0];
  o1 = warp_sum(p1) + m.b3[1];
}

__device__ __forceinline__ float feat_clip(double v) {
  return v == v ? (float)fmin(40.0, fmax(-40.0, v)) : 0.f;
}
__device__ __forceinline__ double lg(double v) { return log10(fmax(v, 1e-300)); }

// The controller's 16 inputs for problem b (see spgo_lm_features), each finite and
// clipped to [-40, 40], computed by one warp: the twelve logarithms they take
// (FP64, which this GPU runs at a small fraction of its FP32 rate) are spread over
// the lanes, one per lane, and broadcast; every lane then holds all 16 features.
// log2(nu) comes out as log10(nu) / log10(2) rounded: nu is a power of two.
__device__ void lm_features_warp(const PlanView &pv, const LMState &s, int b, float *f) {
  const int lane = threadIdx.x & 31;
  const double nres = fmax(1.0, (double)pv.p_nres[b]);
  double arg = 1.0;
  switch (lane) {
    case 0: arg = fmax(s.cost, 1e-300); break;
    case 1: arg = nres; break;
    case 2: arg = fmax(s.cost0, 1e-300); break;
    case 3: arg = fmax(s.lam, 1e-300); break;
    case 4: arg = fmax(s.gnorm, 1e-300); break;
    case 5: arg = fmax(s.dmean, 1e-300); break;
    case 6: arg = fmax(s.dmax, 1e-300); break;
    case 7: arg = fmax(s.dmin, 1e-300); break;
    case 8: arg = fmax(s.cmean, 1e-300); break;
    case 9: arg = fmax(s.last_rel, 1e-12); break;
    case 10: arg = fmax(s.last_predrel, 1e-16); break;
    case 11: arg = fmax(s.nu, 1.0); break;
    default: break;
  }
  const double mine = log10(arg);
  double Lg[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) Lg[k] = __shfl_sync(0xffffffffu, mine, k);
  f[0] = feat_clip(Lg[0] - Lg[1]);
  f[1] = feat_clip(Lg[0] - Lg[2]);
  f[2] = feat_clip(fmin(2.0, fmax(-2.0, s.rho1)));
  f[3] = feat_clip(fmin(2.0, fmax(-2.0, s.rho2)));
  f[4] = feat_clip(fmin(2.0, fmax(-2.0, s.rho3)));
  f[5] = feat_clip(Lg[3]);
  f[6] = feat_clip(Lg[4] - 0.5 * Lg[5]);
  f[7] = feat_clip(Lg[5] - Lg[1]);
  f[8] = feat_clip(Lg[6] - Lg[7]);
  f[9] = feat_clip(Lg[8]);
  f[10] = feat_clip((double)s.iters / 30.0);
  f[11] = feat_clip((double)s.last_acc);
  f[12] = feat_clip(Lg[9]);
  f[13] = feat_clip(Lg[10]);
  f[14] = feat_clip(rint(Lg[11] / 0.30102999566398120));  // log2 of a power of two
  f[15] = feat_clip((double)s.rej_streak / 5.0);
}

// Runs once per LM iteration after the linearisation pass, before the step is
// solved: at the first iteration and after every accepted step (the state was
// just relinearised and the cost is current), the controller's
// proposal lambda * 10^out0 replaces the schedule's lambda when its logit out1 > 0
// (it predicts that deviating from the schedule gives the lower cost).  After a
// rejected step no relinearisation happens and the Nielsen increase stands: the
// fallback whenever a step fails the gain-ratio test.  A proposal lowers lambda by at
// most a factor 10^-min_dl (prm.ctl_min_log10, default -6: the network's own range).
// Tightening the bound does not make the network's choices safer: its proposals were
// learned with the full range, and cutting them short leaves lambda neither where the
// schedule nor where the network would put it.
__global__ void k_controller(PlanView pv, WorkView wv, const MlpSmem *Wd, float min_dl) {
  __shared__ MlpSmem m;
  stage_mlp(Wd, m);
  __syncthreads();
  const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (b >= pv.B) return;
  LMState &s = wv.lm[b];
  if (s.status != 0 || !(s.iters == 0 || s.last_acc)) return;
  float x[kIn];
  lm_features_warp(pv, s, b, x);
  float o0, o1;
  mlp_infer_warp(m, x, o0, o1);
  if ((threadIdx.x & 31) == 0 && o1 > 0.f) {
    const double dl = fmin(3.0, fmax((double)min_dl, (double)o0));
    s.lam = fmin(1e12, fmax(1e-14, s.lam * exp10(dl)));
  }
}

__global__ void k_features(PlanView pv, WorkView wv, float *feat) {
  const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);  // warp per problem
  if (b >= pv.B) return;
  float x[kIn];
  lm_features_warp(pv, wv.lm[b], b, x);
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < kIn; ++k) feat[(size_t)b * kIn + k] = x[k];
}

// FP32 path of k_lm_stats: the maxima and minimum are exact in float and the sums
// run in double-float, on the FP32 pipes (FP64 runs at a small fraction of their
// rate on this GPU).  One CTA, blockDim a multiple of 32.
__device__ void lm_stats_f32(const PlanView &pv, const WorkView &wv, LMState &s, int b, int P, const float *A,
                             const float *g) {
  float gmx = 0.f, dmx = 0.f, dmn = INFINITY;
  df ds = df_make(0.f), cs = df_make(0.f);
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    gmx = fmaxf(gmx, fabsf(g[i]));
    const float d = A[(size_t)i * P + i];
    ds = ds + df_make(d);
    dmx = fmaxf(dmx, d);
    dmn = fminf(dmn, d);
  }
  const int l0 = pv.p_lm_off[b], lc = pv.p_lm_cnt[b];
  const float *C = reinterpret_cast<const float *>(wv.C) + l0;
  for (int i0 = threadIdx.x; i0 < lc; i0 += 8 * blockDim.x) {  // eight loads in flight
    float v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int i = i0 + q * blockDim.x;
      v[q] = i < lc ? C[i] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) cs = cs + df_make(v[q]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    gmx = fmaxf(gmx, __shfl_xor_sync(0xffffffffu, gmx, o));
    dmx = fmaxf(dmx, __shfl_xor_sync(0xffffffffu, dmx, o));
    dmn = fminf(dmn, __shfl_xor_sync(0xffffffffu, dmn, o));
    ds = ds + df{__shfl_xor_sync(0xffffffffu, ds.h, o), __shfl_xor_sync(0xffffffffu, ds.l, o)};
    cs = cs + df{__shfl_xor_sync(0xffffffffu, cs.h, o), __shfl_xor_sync(0xffffffffu, cs.l, o)};
  }
  __shared__ float r7[32][7];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    r7[w][0] = gmx; r7[w][1] = ds.h; r7[w][2] = ds.l; r7[w][3] = dmx; r7[w][4] = dmn;
    r7[w][5] = cs.h; r7[w][6] = cs.l;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
      gmx = fmaxf(gmx, r7[k][0]);
      ds = ds + df{r7[k][1], r7[k][2]};
      dmx = fmaxf(dmx, r7[k][3]);
      dmn = fminf(dmn, r7[k][4]);
      cs = cs + df{r7[k][5], r7[k][6]};
    }
    s.gnorm = (double)gmx;
    s.dmean = P ? ((double)ds.h + (double)ds.l) / P : 0.0;
    s.dmax = (double)dmx;
    s.dmin = P ? (double)dmn : 0.0;
    s.cmean = lc ? ((double)cs.h + (double)cs.l) / lc : 0.0;
  }
}

// per-problem statistics of the fresh linearisation: max |g|, diag(A) mean/max/min, mean C
template <typename T>
__global__ void k_lm_stats(PlanView pv, WorkView wv) {
  __shared__ double red[4][32];
  const int b = blockIdx.x;
  LMState &s = wv.lm[b];
  if (s.status != 0 || !s.relin) return;
  const int P = 6 * pv.p_npose[b];
  const T *A = reinterpret_cast<const T *>(wv.A) + pv.p_S_off[b];
  const T *g = reinterpret_cast<const T *>(wv.g) + pv.p_param_off[b];
  if constexpr (std::is_same<T, float>::value) {
    lm_stats_f32(pv, wv, s, b, P, A, g);
    return;
  }
  double gmax = 0.0, dsum = 0.0, dmax = 0.0, dmin = 1e300, csum = 0.0;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    gmax = fmax(gmax, fabs((double)g[i]));
    const double d = (double)A[(size_t)i * P + i];
    dsum += d;
    dmax = fmax(dmax, d);
    dmin = fmin(dmin, d);
  }
  const int l0 = pv.p_lm_off[b], lc = pv.p_lm_cnt[b];
  for (int i = threadIdx.x; i < lc; i += blockDim.x) csum += (double)reinterpret_cast<const T *>(wv.C)[l0 + i];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    gmax = fmax(gmax, __shfl_xor_sync(0xffffffffu, gmax, o));
    dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
    dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    dmin = fmin(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
    csum += __shfl_xor_sync(0xffffffffu, csum, o);
  }
  __shared__ double r5[32][5];
  if (lane == 0) {
    r5[w][0] = gmax; r5[w][1] = dsum; r5[w][2] = dmax; r5[w][3] = dmin; r5[w][4] = csum;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
      r5[0][0] = fmax(r5[0][0], r5[k][0]);
      r5[0][1] += r5[k][1];
      r5[0][2] = fmax(r5[0][2], r5[k][2]);
      r5[0][3] = fmin(r5[0][3], r5[k][3]);
      r5[0][4] += r5[k][4];
    }
    s.gnorm = r5[0][0];
    s.dmean = P ? r5[0][1] / P : 0.0;
    s.dmax = r5[0][2];
    s.dmin = P ? r5[0][3] : 0.0;
    s.cmean = lc ? r5[0][4] / lc : 0.0;
  }
  (void)red;
}

int launch_lm_stats(const PlanView &pv, const WorkView &wv, int f64, void *stream) {
  if (f64)
    k_lm_stats<double><<<pv.B, 128, 0, (cudaStream_t)stream>>>(pv, wv);
  else
    k_lm_stats<float><<<pv.B, 128, 0, (cudaStream_t)stream>>>(pv, wv);
  ++g_launches;
  return (int)cudaGetLastError();
}

int launch_controller(const PlanView &pv, const WorkView &wv, const Params &prm, const void *Wd, void *stream) {
  k_controller<<<grid_for(pv.B, 8), 256, 0, (cudaStream_t)stream>>>(pv, wv, reinterpret_cast<const MlpSmem *>(Wd),
                                                                    prm.ctl_min_log10);
  ++g_launches;
  return (int)cudaGetLastError();
}

int launch_features(const PlanView &pv, const WorkView &wv, float *feat, void *stream) {
  k_features<<<grid_for(pv.B, 4), 128, 0, (cudaStream_t)stream>>>(pv, wv, feat);
  ++g_launches;
  return (int)cudaGetLastError();
}

int launch_mlp_deploy(const float *theta, void *dst, void *stream) {
  k_mlp_deploy<<<grid_for(kH * kH, 256), 256, 0, (cudaStream_t)stream>>>(theta, reinterpret_cast<MlpSmem *>(dst));
  ++g_launches;
  return (int)cudaGetLastError();
}
size_t mlp_deployed_bytes() { return sizeof(MlpSmem); }

}  // namespace spgo

using namespace spgo;

extern "C" int spgo_mlp_forward(const float *d_params, const float *d_X, int32_t n, float *d_out, float *d_cache,
                                void *stream) {
  if (!d_params || !d_X || !d_out || n < 0) return SPGO_ERR_INVALID_ARG;
  if (n == 0) return SPGO_OK;
  k_mlp_fwd<<<grid_for(n, 128), 128, 0, (cudaStream_t)stream>>>(d_params, d_X, n, d_out, d_cache);
  ++g_launches;
  return cudaGetLastError() == cudaSuccess ? SPGO_OK : SPGO_ERR_CUDA;
}

extern "C" int spgo_mlp_grad(const float *d_params, const float *d_X, const float *d_T, int32_t n, float *d_grad,
                             float *d_loss, float *d_out, float *d_cache, void *stream) {
  if (!d_params || !d_X || !d_T || !d_grad || !d_loss || !d_out || !d_cache || n <= 0) return SPGO_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  cudaMemsetAsync(d_loss, 0, sizeof(float), st);
  k_mlp_fwd<<<grid_for(n, 128), 128, 0, st>>>(d_params, d_X, n, d_out, d_cache);
  k_mlp_delta<<<grid_for(n, 128), 128, 0, st>>>(d_params, d_T, n, d_out, d_cache, d_loss);
  k_mlp_param<<<grid_for(kParams, 128), 128, 0, st>>>(d_X, n, d_cache, d_grad);
  g_launches += 3;
  return cudaGetLastError() == cudaSuccess ? SPGO_OK : SPGO_ERR_CUDA;
}

extern "C" int spgo_mlp_adam(float *d_params, const float *d_grad, float *d_m, float *d_v, int32_t step, float lr,
                             void *stream) {
  if (!d_params || !d_grad || !d_m || !d_v || step < 1) return SPGO_ERR_INVALID_ARG;
  k_mlp_adam<<<grid_for(kParams, 256), 256, 0, (cudaStream_t)stream>>>(d_params, d_grad, d_m, d_v, step, lr);
  ++g_launches;
  return cudaGetLastError() == cudaSuccess ? SPGO_OK : SPGO_ERR_CUDA;
}
