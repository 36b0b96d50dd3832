// Allocation-free variant of the cost pass: spgo_cost_noalloc.
//
// For callers that cannot allocate device memory: code running inside a CUDA
// graph capture it does not own, plugins whose host framework owns the device
// memory pool and forbids cudaMalloc, and real-time threads where an
// allocation (with the implicit synchronisation cudaMalloc/cudaFree can bring)
// is not allowed.  The caller passes the problem, the state and the output in
// its own device memory; the only scratch (the per-frame pose table and the
// per-block partial sums) lives in the file-scope array below, which every GPU
// that loads this library holds until the process exits.
//
// Every call shares that array and it keeps the last call's contents; each
// call overwrites everything it reads before reading it, so nothing needs
// clearing between calls.  Calls whose kernels overlap on the GPU (different
// streams, or different host threads, without ordering between them) race on
// the array: the caller must order them.
//
// The problem's arrays are in the caller's device memory, so the host cannot
// check them: the cost kernel checks every index it dereferences (host and
// observation frames in [0, n_poses], obs_ptr non-decreasing inside [0, n_obs]),
// skips an access that would leave the arrays and marks its block's partial sum
// NaN, so the returned cost is NaN instead of a value read from a previous call's
// frames or from outside the scratch array.
#include <cuda_runtime.h>

#include <mutex>

#include "kernels.cuh"

namespace {

constexpr int kFrameRec = 2 * 12;                       // doubles per frame: 2 cams x (R 9 + c 3)
constexpr int kLmPerBlock = 32;
constexpr size_t kFrameBytes = (size_t)SPGO_NOALLOC_MAX_FRAMES * kFrameRec * sizeof(double);
constexpr size_t kPartialBytes =
    (size_t)((SPGO_NOALLOC_MAX_LANDMARKS + kLmPerBlock - 1) / kLmPerBlock) * sizeof(double);
constexpr size_t kScratchBytes = kFrameBytes + kPartialBytes;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Host-side device address of g_scratch per device (the symbol's name in host
// code is only a host stand-in, never a device address).
std::mutex g_mu;
void *g_addr[128] = {nullptr};

// G[0] = I, G[k+1] = G[k] inv(T_k); right camera G T_r_to_l (one thread, FP64)
__global__ void k_noalloc_chain(int N, const double *__restrict__ poses, const double *__restrict__ Trl16,
                                double *__restrict__ frames) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double Trl[12];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) Trl[4 * r + c] = Trl16[4 * r + c];
  double G[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  for (int k = 0; k <= N; ++k) {
    if (k > 0) {
      double Ti[12], Gn[12];
      spgo::invert34(poses + 12 * (size_t)(k - 1), Ti);
      spgo::compose34(G, Ti, Gn);
      for (int q = 0; q < 12; ++q) G[q] = Gn[q];
    }
    double Gr[12];
    spgo::compose34(G, Trl, Gr);
    double *f = frames + (size_t)k * kFrameRec;
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) {
        f[3 * i + j] = G[4 * i + j];
        f[12 + 3 * i + j] = Gr[4 * i + j];
      }
      f[9 + i] = G[4 * i + 3];
      f[21 + i] = Gr[4 * i + 3];
    }
  }
}

// cost of 32 landmarks per block (warp per landmark, lanes over observations),
// FP64 throughout; one partial sum per block (NaN when an index was out of range)
__global__ void __launch_bounds__(256) k_noalloc_cost(spgo_device_problem pr, const double *__restrict__ alpha,
                                                      spgo_params prm, const double *__restrict__ frames,
                                                      double *__restrict__ partial) {
  __shared__ double warp_sum_s[8];
  __shared__ int bad_s;
  if (threadIdx.x == 0) bad_s = 0;
  __syncthreads();
  const int N = pr.n_poses;
  bool bad = false;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double fx[2] = {pr.intrinsics[0], pr.intrinsics[4]}, fy[2] = {pr.intrinsics[1], pr.intrinsics[5]};
  const double cx[2] = {pr.intrinsics[2], pr.intrinsics[6]}, cy[2] = {pr.intrinsics[3], pr.intrinsics[7]};
  double acc = 0.0;
  for (int s = warp; s < kLmPerBlock; s += 8) {
    const int l = blockIdx.x * kLmPerBlock + s;
    if (l >= pr.n_landmarks) break;
    const int a = pr.host[l];
    const int64_t ob = pr.obs_ptr[l], oe = pr.obs_ptr[l + 1];
    if (a < 0 || a > N || ob < 0 || oe < ob || oe > pr.n_obs) {
      bad = true;
      continue;
    }
    const double al = alpha[l];
    const double *fa = frames + (size_t)a * kFrameRec;
    const double tx = ((double)pr.anchor_uv[2 * l] - cx[0]) / fx[0] / al;
    const double ty = ((double)pr.anchor_uv[2 * l + 1] - cy[0]) / fy[0] / al;
    const double tz = 1.0 / al;
    const double X[3] = {fa[0] * tx + fa[1] * ty + fa[2] * tz, fa[3] * tx + fa[4] * ty + fa[5] * tz,
                         fa[6] * tx + fa[7] * ty + fa[8] * tz};
    for (int64_t o = ob + lane; o < oe; o += 32) {
      const int n = pr.obs_frame[o];
      if (n < 0 || n > N) {
        bad = true;
        continue;
      }
      const double *fn = frames + (size_t)n * kFrameRec;
      const double boost = (prm.near_boost && abs(n - a) < 2) ? 16.0 : 1.0;
      for (int cam = 0; cam < 2; ++cam) {
        const double *R = fn + 12 * cam;
        const double *cn = R + 9;
        const double Xc[3] = {X[0] + (fa[9] - cn[0]), X[1] + (fa[10] - cn[1]), X[2] + (fa[11] - cn[2])};
        const double t0 = R[0] * Xc[0] + R[3] * Xc[1] + R[6] * Xc[2];
        const double t1 = R[1] * Xc[0] + R[4] * Xc[1] + R[7] * Xc[2];
        const double t2 = R[2] * Xc[0] + R[5] * Xc[1] + R[8] * Xc[2];
        const double r0 = (double)pr.obs_uv[4 * o + 2 * cam] - (fx[cam] * t0 / t2 + cx[cam]);
        const double r1 = (double)pr.obs_uv[4 * o + 2 * cam + 1] - (fy[cam] * t1 / t2 + cy[cam]);
        double rho;
        (void)spgo::robust<double>(prm.loss, (double)prm.loss_scale, r0 * r0 + r1 * r1, rho);
        acc += 0.5 * boost * rho;
      }
    }
  }
  acc = spgo::warp_sum(acc);
  if (lane == 0) warp_sum_s[warp] = acc;
  if (bad) bad_s = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += warp_sum_s[w];
    partial[blockIdx.x] = bad_s ? __longlong_as_double(0x7ff8000000000000LL) : t;
  }
}

// fixed-order sum of the partials (deterministic) into the caller's output
__global__ void k_noalloc_reduce(int nparts, const double *__restrict__ partial, double *__restrict__ out) {
  __shared__ double s[256];
  double t = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) t += partial[i];
  s[threadIdx.x] = t;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

int fail_na(int code, const char *msg) {
  spgo::set_last_error(msg);
  return code;
}

}  // namespace

extern "C" int spgo_cost_noalloc(const spgo_device_problem *prob, const double *d_poses, const double *d_alpha,
                                 const spgo_params *params, double *d_cost, void *stream) {
  if (!prob || !d_poses || !d_alpha || !params || !d_cost || !prob->intrinsics || !prob->T_r_to_l)
    return fail_na(SPGO_ERR_INVALID_ARG, "spgo_cost_noalloc: null argument");
  const int N = prob->n_poses, L = prob->n_landmarks;
  if (N < 1 || L < 0 || prob->n_obs < 0) return fail_na(SPGO_ERR_INVALID_ARG, "spgo_cost_noalloc: bad problem size");
  if (N + 1 > SPGO_NOALLOC_MAX_FRAMES || L > SPGO_NOALLOC_MAX_LANDMARKS)
    return fail_na(SPGO_ERR_UNSUPPORTED,
                   "spgo_cost_noalloc: problem exceeds the allocation-free limits "
                   "(n_poses + 1 <= SPGO_NOALLOC_MAX_FRAMES, n_landmarks <= SPGO_NOALLOC_MAX_LANDMARKS)");
  if (L > 0 && (!prob->host || !prob->anchor_uv || !prob->obs_ptr ||
                (prob->n_obs > 0 && (!prob->obs_frame || !prob->obs_uv))))
    return fail_na(SPGO_ERR_INVALID_ARG, "spgo_cost_noalloc: null problem array");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 128)
    return fail_na(SPGO_ERR_CUDA, "spgo_cost_noalloc: cudaGetDevice failed");
  void *base = nullptr;
  {
    // first call on a device: resolve the scratch array's device address (no allocation)
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
      e = cudaGetSymbolAddress(&g_addr[dev], g_scratch);
      if (e != cudaSuccess) {
        g_addr[dev] = nullptr;
        return fail_na(SPGO_ERR_CUDA, "spgo_cost_noalloc: cudaGetSymbolAddress failed");
      }
    }
    base = g_addr[dev];
  }
  double *frames = reinterpret_cast<double *>(base);
  double *partial = reinterpret_cast<double *>(static_cast<unsigned char *>(base) + kFrameBytes);
  cudaStream_t st = (cudaStream_t)stream;
  const int nblk = (L + kLmPerBlock - 1) / kLmPerBlock;
  k_noalloc_chain<<<1, 1, 0, st>>>(N, d_poses, prob->T_r_to_l, frames);
  if (nblk > 0) k_noalloc_cost<<<nblk, 256, 0, st>>>(*prob, d_alpha, *params, frames, partial);
  k_noalloc_reduce<<<1, 256, 0, st>>>(nblk, partial, d_cost);
  if (cudaGetLastError() != cudaSuccess) {
    // (e.g. the context was reset after the address was resolved: resolve it again next time)
    std::lock_guard<std::mutex> lk(g_mu);
    g_addr[dev] = nullptr;
    return fail_na(SPGO_ERR_CUDA, "spgo_cost_noalloc: kernel launch failed");
  }
  return SPGO_OK;
}
