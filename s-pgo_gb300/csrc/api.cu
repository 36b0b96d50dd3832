// C ABI: planner (host), solver binding and the LM / Gauss-Newton orchestration.
//
// The reference allocates every workspace with cudaMalloc and frees it on each
// step() (src/Optimization/LMutils.cu:5-185, Solver_cuda.cu:576-580, :793-794),
// creates a cuBLAS handle per iteration (Solver_cuda.cu:627-628) and
// synchronises about ten times per iteration.  Here the caller owns two device
// buffers (static problem data and scratch) sized once by the plan; an LM
// iteration is a fixed, host-synchronisation-free sequence of kernels whose
// per-problem work is gated on device-side status, so any number of iterations
// can be enqueued (or captured in a CUDA graph) and the host only reads status.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <cstdlib>
#include <numeric>
#include <thread>
#include <atomic>
#include <type_traits>
#include <stdexcept>
#include <string>
#include <vector>

#include "spgo_internal.h"

static thread_local std::string g_err;

namespace spgo {
thread_local int64_t g_launches = 0;
void set_last_error(const char *msg) { g_err = msg; }
}  // namespace spgo

using namespace spgo;

static int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

#define CUDA_TRY(expr)                                                                     \
  do {                                                                                     \
    int _e = (int)(expr);                                                                  \
    if (_e != 0) return fail(SPGO_ERR_CUDA, std::string(#expr) + ": " +                    \
                                                cudaGetErrorString((cudaError_t)_e));      \
  } while (0)

// ---------------------------------------------------------------------------
// plan
// ---------------------------------------------------------------------------
struct Seg {
  size_t off;
  size_t bytes;
};

// ---- page-locked host staging, reused across plans ----------------------------
// A plan's static data (every array the kernels read) is written straight into
// host blocks laid out like the device buffer, so the upload is two DMA copies
// from page-locked memory.  Blocks come from a small process-wide cache: a caller
// that plans batch after batch reuses the same locked pages (no page faults, no
// re-locking).  Without a CUDA device the blocks are ordinary heap memory.
struct HostBlock {
  unsigned char *ptr = nullptr;
  size_t cap = 0;
  bool pinned = false;
};

static std::mutex g_arena_mu;
static std::vector<HostBlock> g_arena_free;
constexpr size_t kArenaKeep = 16;             // cached blocks at most
constexpr size_t kArenaKeepBytes = 2ull << 30;  // and bytes at most

static void block_free(HostBlock &b) {
  if (!b.ptr) return;
  if (b.pinned)
    cudaFreeHost(b.ptr);
  else
    std::free(b.ptr);
  b = HostBlock();
}

static size_t arena_cap(size_t bytes) {  // blocks come in whole MiB
  return (std::max<size_t>(bytes, 256) + (1u << 20) - 1) & ~(size_t)((1u << 20) - 1);
}

static HostBlock arena_get(size_t bytes) {
  bytes = std::max<size_t>(bytes, 256);
  {
    std::lock_guard<std::mutex> lk(g_arena_mu);
    size_t best = g_arena_free.size();
    for (size_t i = 0; i < g_arena_free.size(); ++i) {  // smallest cached block that fits, at most 2x
      const size_t c = g_arena_free[i].cap;
      if (c >= bytes && c <= 2 * arena_cap(bytes) && (best == g_arena_free.size() || c < g_arena_free[best].cap))
        best = i;
    }
    if (best < g_arena_free.size()) {
      HostBlock b = g_arena_free[best];
      g_arena_free.erase(g_arena_free.begin() + (std::ptrdiff_t)best);
      return b;
    }
  }
  HostBlock b;
  b.cap = arena_cap(bytes);
  void *q = nullptr;
  if (cudaHostAlloc(&q, b.cap, cudaHostAllocPortable) == cudaSuccess) {  // locked for every context
    b.ptr = (unsigned char *)q;
    b.pinned = true;
  } else {
    cudaGetLastError();  // no device (planning on a CPU-only host): not an error of this library
    b.ptr = (unsigned char *)std::malloc(b.cap);
    if (!b.ptr) throw std::runtime_error("host allocation of " + std::to_string(b.cap) + " bytes failed");
  }
  return b;
}

static void arena_put(HostBlock &b) {
  if (!b.ptr) return;
  std::lock_guard<std::mutex> lk(g_arena_mu);
  g_arena_free.push_back(b);
  b = HostBlock();
  size_t total = 0;
  for (const HostBlock &x : g_arena_free) total += x.cap;
  while (g_arena_free.size() > kArenaKeep || (total > kArenaKeepBytes && g_arena_free.size() > 1)) {
    total -= g_arena_free.front().cap;  // the oldest goes
    block_free(g_arena_free.front());
    g_arena_free.erase(g_arena_free.begin());
  }
}

struct spgo_plan {
  int32_t precision = SPGO_PREC_MIXED;
  int32_t tc_split = SPGO_TC_SPLIT, simt_split = SPGO_KSPLIT;  // Schur work shapes (spgo_plan_options)
  int32_t B = 0, F = 0, NP = 0, L = 0;
  int64_t O = 0;
  int32_t max_P = 0, max_D = 1, max_nb = 1, total_params = 0;
  int32_t max_P_small = 0;                 // widest problem of the batched factorisation
  std::vector<int32_t> large;              // problems factored by k_chol_large.cu
  int64_t total_S = 0, total_pairs = 0, total_slab = 0;
  std::vector<int32_t> p_npose, p_frame_off, p_pose_off, p_lm_off, p_lm_cnt, p_pair_D, p_param_off, p_chunk_off,
      p_chunk_cnt, fr_prob, pose_prob;
  std::vector<int64_t> p_S_off, p_pair_off, p_nres;
  std::vector<float> p_intr;
  std::vector<double> p_Trl;
  // per-landmark and per-observation arrays: written by the planner directly into
  // the big block, at their offsets in the device buffer
  int32_t *lm_prob = nullptr, *lm_host = nullptr, *lm_lo = nullptr, *lm_hi = nullptr, *lm_user = nullptr,
          *lm_chunk = nullptr, *lm_slot = nullptr;
  float *lm_uv = nullptr;
  int64_t *lm_obs = nullptr;
  int32_t *obs_frame = nullptr;
  float *obs_uv = nullptr;
  uint8_t *obs_slot = nullptr;
  size_t off_lm[7] = {}, off_lm_uv = 0, off_lm_obs = 0, off_obs_frame = 0, off_obs_uv = 0, off_obs_slot = 0;
  size_t big_bytes = 0;
  std::vector<int32_t> ch_prob, ch_f0, ch_nb, ch_lm0, ch_cnt;
  std::vector<int64_t> ch_slab;
  std::vector<int32_t> wk_prob, wk_ti, wk_tj, wk_cbeg, wk_cend, wk_chunks;
  // tensor-core Schur work: (problem, 128-row tile, column range <= 256, chunks)
  std::vector<int32_t> tc_prob, tc_row0, tc_col0, tc_ncols, tc_cbeg, tc_cend, tc_chunks;
  // batched factorisation: CTA k factors problem fs_prob[k], widest first
  std::vector<int32_t> fs_prob;
  std::vector<Seg> segs;
  size_t static_bytes = 0, ws_bytes = 0;
  // host staging: [0, big_bytes) of the device buffer, then the small arrays
  HostBlock big, small;
  mutable std::vector<cudaEvent_t> uploads;  // one per upload from the blocks
  mutable std::mutex upload_mu;              // solvers bound from several threads
  // workspace segment offsets
  size_t w_Sx = 0, w_lg = 0, w_lgflag = 0, w_lgred = 0;
  size_t w_frRf, w_frRl, w_frRd, w_frc, w_frch, w_frcl, w_pcand, w_acand, w_res, w_pacc, w_pF, w_A, w_g, w_SL, w_gL, w_fac,
      w_delta, w_C, w_ga, w_slab, w_lm, w_cost, w_pred, w_lmb, w_probe, w_ctrl, w_trace;
  // refinement of the mixed path's step (k_refine.cu)
  size_t w_tcam = 0, w_xanc = 0, w_facs = 0, w_twist = 0, w_pdual = 0, w_dal = 0, w_tl = 0, w_gaacc = 0, w_gacc = 0, w_rhsB = 0, w_ddelta = 0;

  ~spgo_plan() {
    for (cudaEvent_t e : uploads) {  // the blocks go back to the cache only once no copy reads them
      cudaEventSynchronize(e);
      cudaEventDestroy(e);
    }
    arena_put(big);
    arena_put(small);
  }
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// a small array: packed after the big block (copied into the small block later)
template <typename V>
static void add_seg(spgo_plan *p, const V &v) {
  Seg s;
  s.off = p->static_bytes;
  s.bytes = v.size() * sizeof(typename V::value_type);
  p->segs.push_back(s);
  p->static_bytes = align256(p->static_bytes + s.bytes);
}

// a big array at its fixed offset in the big block
static void add_big(spgo_plan *p, size_t off, size_t bytes) {
  Seg s;
  s.off = off;
  s.bytes = bytes;
  p->segs.push_back(s);
}

// offsets of the per-landmark and per-observation arrays, then the big block
static void layout_big(spgo_plan *p, int64_t Lt, int64_t Ot) {
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t r = o;
    o = align256(o + bytes);
    return r;
  };
  for (int k = 0; k < 7; ++k) p->off_lm[k] = take((size_t)Lt * 4);
  p->off_lm_uv = take((size_t)Lt * 8);
  p->off_lm_obs = take((size_t)(Lt + 1) * 8);
  p->off_obs_frame = take((size_t)Ot * 4);
  p->off_obs_uv = take((size_t)Ot * 16);
  p->off_obs_slot = take((size_t)Ot);
  p->big_bytes = o;
  p->big = arena_get(o);
  unsigned char *b = p->big.ptr;
  int32_t **lm[7] = {&p->lm_prob, &p->lm_host, &p->lm_lo, &p->lm_hi, &p->lm_user, &p->lm_chunk, &p->lm_slot};
  for (int k = 0; k < 7; ++k) *lm[k] = reinterpret_cast<int32_t *>(b + p->off_lm[k]);
  p->lm_uv = reinterpret_cast<float *>(b + p->off_lm_uv);
  p->lm_obs = reinterpret_cast<int64_t *>(b + p->off_lm_obs);
  p->obs_frame = reinterpret_cast<int32_t *>(b + p->off_obs_frame);
  p->obs_uv = reinterpret_cast<float *>(b + p->off_obs_uv);
  p->obs_slot = reinterpret_cast<uint8_t *>(b + p->off_obs_slot);
}

static void build_layout(spgo_plan *p) {
  // static segments, in PlanView order (see make_views)
  // static segments, in PlanView order (see make_views): the big arrays sit at their
  // offsets in the big block, the small ones are packed after it
  p->segs.clear();
  p->static_bytes = p->big_bytes;
  const int64_t Lt = p->L, Ot = p->O;
  std::vector<const void *> small_src;
  auto small = [&](const auto &v) {
    add_seg(p, v);
    small_src.push_back(v.data());
  };
  auto big = [&](size_t off, size_t bytes) {
    add_big(p, off, bytes);
    small_src.push_back(nullptr);
  };
  small(p->p_npose); small(p->p_frame_off); small(p->p_pose_off); small(p->p_lm_off);
  small(p->p_lm_cnt); small(p->p_pair_D); small(p->p_param_off); small(p->p_chunk_off);
  small(p->p_chunk_cnt); small(p->p_S_off); small(p->p_pair_off); small(p->p_nres);
  small(p->p_intr);
  small(p->p_Trl);
  for (int k = 0; k < 7; ++k) big(p->off_lm[k], (size_t)Lt * 4);  // lm_prob .. lm_slot
  big(p->off_lm_uv, (size_t)Lt * 8);
  big(p->off_lm_obs, (size_t)(Lt + 1) * 8); big(p->off_obs_frame, (size_t)Ot * 4); big(p->off_obs_uv, (size_t)Ot * 16);
  small(p->ch_prob);
  small(p->ch_f0); small(p->ch_nb); small(p->ch_lm0); small(p->ch_cnt); small(p->ch_slab);
  small(p->wk_prob); small(p->wk_ti); small(p->wk_tj); small(p->wk_cbeg);
  small(p->wk_cend); small(p->wk_chunks); small(p->fr_prob); small(p->pose_prob);
  big(p->off_obs_slot, (size_t)Ot);
  small(p->tc_prob); small(p->tc_row0); small(p->tc_col0); small(p->tc_ncols);
  small(p->tc_cbeg); small(p->tc_cend); small(p->tc_chunks);
  small(p->fs_prob);
  p->small = arena_get(p->static_bytes - p->big_bytes);
  for (size_t i = 0; i < p->segs.size(); ++i)
    if (small_src[i] && p->segs[i].bytes)
      std::memcpy(p->small.ptr + (p->segs[i].off - p->big_bytes), small_src[i], p->segs[i].bytes);
  // workspace
  const size_t ts = p->precision == SPGO_PREC_FP64 ? 8 : 4;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t r = o;
    o = align256(o + bytes);
    return r;
  };
  p->w_frRf = take((size_t)p->F * 18 * 4);
  p->w_frRl = take((size_t)p->F * 18 * 4);
  p->w_frRd = take((size_t)p->F * 18 * 8);
  p->w_frc = take((size_t)p->F * 6 * 8);
  p->w_frch = take((size_t)p->F * 6 * 4);
  p->w_frcl = take((size_t)p->F * 6 * 4);
  p->w_pcand = take((size_t)p->NP * 12 * 8);
  p->w_acand = take((size_t)p->L * 8);
  p->w_res = take((size_t)p->O * 16 * 2);  // the state's and the candidate's residuals
  // pose-pair records and their prefix / suffix sums: FP64 on both paths (the mixed
  // path's Jacobian pass sums them exactly, its pair reduction runs in FP64)
  p->w_pacc = take((size_t)p->total_pairs * 27 * 8);
  p->w_pF = take((size_t)p->total_pairs * 27 * 8);
  p->w_A = take((size_t)p->total_S * ts);
  p->w_g = take((size_t)p->total_params * ts);
  p->w_SL = take((size_t)p->total_S * ts);
  p->w_gL = take((size_t)p->total_params * ts);
  // factor storage, exact S and vectors of the multi-CTA factorisation, when any problem needs it
  const bool any_large = !p->large.empty();
  p->w_fac = take(any_large ? (size_t)p->total_S * ts : 0);
  p->w_Sx = take(any_large ? (size_t)p->total_S * 8 : 0);
  p->w_lg = take(any_large ? (size_t)p->total_params * 8 * 6 : 0);
  p->w_lgflag = take(any_large ? (size_t)p->total_params * 2 * sizeof(int) : 0);
  p->w_lgred = take(any_large && p->precision == SPGO_PREC_MIXED ? (size_t)(p->NP + p->B) * 12 * 8 : 0);
  p->w_delta = take((size_t)p->total_params * 8);
  p->w_C = take((size_t)(p->L + 64) * ts);  // + 64: the tensor-core Schur copies 16-byte aligned supersets
  p->w_ga = take((size_t)(p->L + 64) * ts);  // + 64: as C
  p->w_slab = take((size_t)p->total_slab * ts);
  p->w_lm = take((size_t)p->B * sizeof(LMState));
  p->w_cost = take((size_t)p->B * 8);
  p->w_pred = take((size_t)p->B * 8);
  p->w_lmb = take((size_t)p->B * sizeof(LMState));
  p->w_probe = take((size_t)p->B * 32 * 8);
  p->w_ctrl = take(mlp_deployed_bytes());
  p->w_trace = take((size_t)p->B * SPGO_TRACE_MAX * 3 * 8);
  if (p->precision == SPGO_PREC_MIXED) {
    p->w_tcam = take((size_t)p->O * 24 * 2);  // camera-frame points, halves as the residuals
    p->w_xanc = take((size_t)p->L * 32 * 2);  // anchor points, halves as the residuals
    p->w_facs = take((size_t)p->total_S * 4);
    p->w_twist = take((size_t)p->total_pairs * 6 * 4);
    p->w_pdual = take((size_t)p->total_pairs * 6 * 8);
    p->w_dal = take((size_t)p->L * 8);
    p->w_tl = take((size_t)p->L * 4);
    p->w_gaacc = take((size_t)p->L * 8);
    p->w_gacc = take((size_t)p->total_params * 8);
    p->w_rhsB = take((size_t)p->total_params * 4);
    p->w_ddelta = take((size_t)p->total_params * 8);
  }
  p->ws_bytes = o;
}

// One problem's share of the plan.  Landmark and observation records go straight
// into the plan's pre-sized arrays at the problem's offsets (lm_chunk holds the
// problem-local chunk index until the merge); chunk and work lists are local.
struct ProbPlan {
  int code = SPGO_OK;
  std::string err;
  int32_t maxw = 1, max_nb = 1;
  int64_t slab = 0;  // slab elements of the problem
  std::vector<int32_t> ch_f0, ch_nb, ch_lm0, ch_cnt;
  std::vector<int64_t> ch_slab;  // problem-local slab offsets
  std::vector<int32_t> wk_ti, wk_tj, wk_cbeg, wk_cend, wk_chunks;
  std::vector<int32_t> tc_row0, tc_col0, tc_ncols, tc_cbeg, tc_cend, tc_chunks;
};

static void plan_problem(const spgo_host_problem &q, int b, int64_t lm_base, int64_t obs_base, spgo_plan *p,
                         ProbPlan &o) {
  auto bad = [&](const std::string &m) {
    o.code = SPGO_ERR_INVALID_ARG;
    o.err = m;
  };
  const int N = q.n_poses, L = q.n_landmarks;
  // per-landmark window [lo, hi) of pose blocks
  std::vector<int32_t> lo(L), hi(L);
  for (int l = 0; l < L; ++l) {
    const int a = q.host[l];
    if (a < 0 || a > N) return bad("landmark " + std::to_string(l) + ": host out of range");
    if (q.obs_ptr[l + 1] < q.obs_ptr[l]) return bad("obs_ptr decreasing");
    int32_t mn = a, mx = a, prev = -1;
    for (int64_t ob = q.obs_ptr[l]; ob < q.obs_ptr[l + 1]; ++ob) {
      const int n = q.obs_frame[ob];
      if (n < 0 || n > N) return bad("observation frame out of range");
      if (n <= prev) return bad("frames must ascend strictly inside a landmark");
      prev = n;
      mn = std::min(mn, n);
      mx = std::max(mx, n);
    }
    lo[l] = mn;
    hi[l] = mx;
    if (mx - mn > SPGO_MAX_WINDOW) {
      o.code = SPGO_ERR_UNSUPPORTED;
      o.err = "landmark " + std::to_string(l) + " spans more than SPGO_MAX_WINDOW poses";
      return;
    }
    o.maxw = std::max(o.maxw, mx - mn);
  }
  // order landmarks by host frame, then window; a chunk holds <= 32 landmarks of ONE
  // host, so all its pose-pair contributions (host, target) are indexed by the target
  std::vector<int32_t> order(L);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    if (q.host[x] != q.host[y]) return q.host[x] < q.host[y];
    return lo[x] != lo[y] ? lo[x] < lo[y] : hi[x] < hi[y];
  });
  std::vector<int32_t> fcount;  // counting sort of a chunk's observations by frame
  int32_t cur = -1;
  int k_open = 0;          // first landmark (position in `order`) of the open chunk
  int64_t obs_local = 0;   // observations emitted so far
  // emit the open chunk's observations sorted by frame (stable: landmark order
  // inside a frame) with a counting sort over its frame window
  auto close_chunk = [&](int k_end) {
    if (cur < 0) return;
    o.slab += (int64_t)6 * o.ch_nb[cur] * SPGO_CHUNK;
    const int f0 = o.ch_f0[cur], nf = o.ch_nb[cur] + 1;
    fcount.assign((size_t)nf + 1, 0);
    int64_t n_chunk = 0;
    for (int k = k_open; k < k_end; ++k) {
      const int l = order[k];
      for (int64_t ob = q.obs_ptr[l]; ob < q.obs_ptr[l + 1]; ++ob) ++fcount[(size_t)(q.obs_frame[ob] - f0) + 1];
      n_chunk += q.obs_ptr[l + 1] - q.obs_ptr[l];
    }
    for (int f = 0; f < nf; ++f) fcount[(size_t)f + 1] += fcount[(size_t)f];
    for (int k = k_open; k < k_end; ++k) {
      const int l = order[k];
      const uint8_t slot = (uint8_t)(k - k_open);
      for (int64_t ob = q.obs_ptr[l]; ob < q.obs_ptr[l + 1]; ++ob) {
        const int n = q.obs_frame[ob];
        const size_t dst = (size_t)(obs_base + obs_local + fcount[(size_t)(n - f0)]++);
        p->obs_frame[dst] = n;
        p->obs_slot[dst] = slot;
        if (q.obs_uv_f64)
          for (int j = 0; j < 4; ++j) p->obs_uv[4 * dst + j] = (float)q.obs_uv_f64[4 * ob + j];
        else
          std::memcpy(&p->obs_uv[4 * dst], q.obs_uv + 4 * ob, 4 * sizeof(float));
      }
    }
    obs_local += n_chunk;
  };
  int32_t host_prev = -1;
  for (int k = 0; k < L; ++k) {
    const int l = order[k];
    bool fresh = cur < 0 || o.ch_cnt[cur] == SPGO_CHUNK || host_prev != q.host[l];
    if (!fresh) {
      const int f0 = o.ch_f0[cur];
      const int nb_new = std::max(o.ch_f0[cur] + o.ch_nb[cur], hi[l]) - f0;
      if (nb_new > SPGO_MAX_WINDOW) fresh = true;
    }
    if (fresh) {
      close_chunk(k);
      k_open = k;
      cur = (int32_t)o.ch_f0.size();
      o.ch_f0.push_back(std::min(lo[l], N - 1));
      o.ch_nb.push_back(1);
      o.ch_lm0.push_back((int32_t)(lm_base + k));
      o.ch_cnt.push_back(0);
      o.ch_slab.push_back(o.slab);
    }
    host_prev = q.host[l];
    const int f0 = o.ch_f0[cur];
    o.ch_nb[cur] = std::max(o.ch_nb[cur], hi[l] - f0);
    o.ch_cnt[cur] += 1;
    // internal landmark lm_base + k; lm_obs holds the start of its CHUNK's observations
    const size_t li = (size_t)(lm_base + k);
    p->lm_prob[li] = b;
    p->lm_host[li] = q.host[l];
    p->lm_lo[li] = lo[l];
    p->lm_hi[li] = hi[l];
    p->lm_user[li] = (int32_t)(lm_base + l);
    p->lm_chunk[li] = cur;  // problem-local until the merge
    p->lm_slot[li] = o.ch_cnt[cur] - 1;
    p->lm_uv[2 * li] = q.anchor_uv_f64 ? (float)q.anchor_uv_f64[2 * l] : q.anchor_uv[2 * l];
    p->lm_uv[2 * li + 1] = q.anchor_uv_f64 ? (float)q.anchor_uv_f64[2 * l + 1] : q.anchor_uv[2 * l + 1];
    p->lm_obs[li] = obs_base + obs_local;
  }
  close_chunk(L);
  const int nch = (int)o.ch_f0.size();
  for (int c = 0; c < nch; ++c) {
    if (o.ch_f0[c] < 0 || o.ch_f0[c] + o.ch_nb[c] > N) return bad("internal: chunk window outside the problem");
    o.max_nb = std::max(o.max_nb, o.ch_nb[c]);
  }
  // Schur work list: every (ti >= tj) tile pair a chunk's window touches
  const int ntile = (N + SPGO_TILE_BLOCKS - 1) / SPGO_TILE_BLOCKS;
  std::vector<std::vector<int32_t>> lists((size_t)ntile * ntile);
  for (int c = 0; c < nch; ++c) {
    const int t0 = o.ch_f0[c] / SPGO_TILE_BLOCKS;
    const int t1 = std::min(ntile - 1, (o.ch_f0[c] + o.ch_nb[c] - 1) / SPGO_TILE_BLOCKS);
    for (int ti = t0; ti <= t1; ++ti)
      for (int tj = t0; tj <= ti; ++tj) lists[(size_t)ti * ntile + tj].push_back(c);
  }
  for (int ti = 0; ti < ntile; ++ti)
    for (int tj = 0; tj <= ti; ++tj) {
      const auto &lst = lists[(size_t)ti * ntile + tj];
      const size_t ks = (size_t)p->simt_split;
      for (size_t s0 = 0; s0 < lst.size(); s0 += ks) {
        o.wk_ti.push_back(ti);
        o.wk_tj.push_back(tj);
        o.wk_cbeg.push_back((int32_t)o.wk_chunks.size());
        for (size_t k = s0; k < std::min(lst.size(), s0 + ks); ++k) o.wk_chunks.push_back(lst[k]);
        o.wk_cend.push_back((int32_t)o.wk_chunks.size());
      }
    }
  // tensor-core Schur work list: 128 x 128 tiles of the lower triangle, <= tc_split chunks each
  const int P = 6 * N;
  for (int row0 = 0; row0 < P; row0 += 128) {
    for (int col0 = 0; col0 <= row0; col0 += 128) {
      const int ncols = ((std::min(128, P - col0) + 15) / 16) * 16;
      std::vector<int32_t> lst;
      for (int c = 0; c < nch; ++c) {
        const int s0 = 6 * o.ch_f0[c], s1 = 6 * (o.ch_f0[c] + o.ch_nb[c]);
        if (s1 > row0 && s0 < row0 + 128 && s1 > col0 && s0 < col0 + ncols) lst.push_back(c);
      }
      const size_t ts = (size_t)p->tc_split;
      for (size_t st = 0; st < lst.size(); st += ts) {
        o.tc_row0.push_back(row0);
        o.tc_col0.push_back(col0);
        o.tc_ncols.push_back(ncols);
        o.tc_cbeg.push_back((int32_t)o.tc_chunks.size());
        for (size_t k = st; k < std::min(lst.size(), st + ts); ++k) o.tc_chunks.push_back(lst[k]);
        o.tc_cend.push_back((int32_t)o.tc_chunks.size());
      }
    }
  }
}

static int plan_build(const spgo_host_problem *probs, int nprob, int precision, spgo_plan *p) {
  if (nprob <= 0 || !probs) return fail(SPGO_ERR_INVALID_ARG, "no problems");
  if (precision != SPGO_PREC_MIXED && precision != SPGO_PREC_FP64)
    return fail(SPGO_ERR_INVALID_ARG, "unknown precision");
  p->precision = precision;
  p->B = nprob;
  // sizes, pointers and CSR shape first; the per-problem work then runs in parallel
  std::vector<int64_t> lm_base(nprob + 1, 0), obs_base(nprob + 1, 0);
  for (int b = 0; b < nprob; ++b) {
    const spgo_host_problem &q = probs[b];
    const int N = q.n_poses, L = q.n_landmarks;
    if (N < 1) return fail(SPGO_ERR_INVALID_ARG, "problem " + std::to_string(b) + ": n_poses < 1");
    if (L < 0 || q.n_obs < 0) return fail(SPGO_ERR_INVALID_ARG, "negative size");
    if (!q.intrinsics || !q.T_r_to_l || (L > 0 && (!q.host || (!q.anchor_uv && !q.anchor_uv_f64) || !q.obs_ptr)) ||
        (q.n_obs > 0 && (!q.obs_frame || (!q.obs_uv && !q.obs_uv_f64))))
      return fail(SPGO_ERR_INVALID_ARG, "problem " + std::to_string(b) + ": null array");
    if (L > 0 && (q.obs_ptr[0] != 0 || q.obs_ptr[L] != q.n_obs))
      return fail(SPGO_ERR_INVALID_ARG, "problem " + std::to_string(b) + ": obs_ptr is not a CSR over n_obs");
    if (L == 0 && q.n_obs != 0)
      return fail(SPGO_ERR_INVALID_ARG, "problem " + std::to_string(b) + ": observations without landmarks");
    lm_base[b + 1] = lm_base[b] + L;
    obs_base[b + 1] = obs_base[b] + q.n_obs;
  }
  const int64_t Lt = lm_base[nprob], Ot = obs_base[nprob];
  p->L = (int32_t)Lt;
  p->O = Ot;
  layout_big(p, Lt, Ot);
  std::vector<ProbPlan> pp((size_t)nprob);
  {
    // up to 16 threads, leaving two cores to the threads that drive the GPU (a caller
    // plans the next batch while the current one solves)
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned use = std::max(1u, std::min(hw, 16u) - std::min(hw - 1, 2u));
    const int nthr = (int)std::min<unsigned>(use, (unsigned)nprob);
    std::atomic<int> next(0);
    auto work = [&]() {
      for (int b; (b = next.fetch_add(1)) < nprob;) plan_problem(probs[b], b, lm_base[b], obs_base[b], p, pp[b]);
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthr; ++t) th.emplace_back(work);
    work();
    for (auto &t : th) t.join();
  }
  // merge in problem order: global chunk indices, slab offsets, work lists, records
  int32_t frame_off = 0, pose_off = 0, lm_off = 0, param_off = 0;
  int64_t S_off = 0, pair_off = 0, slab_off = 0;
  for (int b = 0; b < nprob; ++b) {
    const spgo_host_problem &q = probs[b];
    const ProbPlan &o = pp[b];
    if (o.code != SPGO_OK) return fail(o.code, "problem " + std::to_string(b) + ": " + o.err);
    const int N = q.n_poses, L = q.n_landmarks, P = 6 * N;
    const int32_t ch_begin = (int32_t)p->ch_prob.size();
    const int nch = (int)o.ch_f0.size();
    for (int c = 0; c < nch; ++c) {
      p->ch_prob.push_back(b);
      p->ch_f0.push_back(o.ch_f0[c]);
      p->ch_nb.push_back(o.ch_nb[c]);
      p->ch_lm0.push_back(o.ch_lm0[c]);
      p->ch_cnt.push_back(o.ch_cnt[c]);
      p->ch_slab.push_back(slab_off + o.ch_slab[c]);
    }
    p->max_nb = std::max(p->max_nb, o.max_nb);
    for (int64_t k = lm_base[b]; k < lm_base[b + 1]; ++k) p->lm_chunk[(size_t)k] += ch_begin;
    {
      const int32_t base = (int32_t)p->wk_chunks.size();
      for (size_t i = 0; i < o.wk_ti.size(); ++i) {
        p->wk_prob.push_back(b);
        p->wk_ti.push_back(o.wk_ti[i]);
        p->wk_tj.push_back(o.wk_tj[i]);
        p->wk_cbeg.push_back(base + o.wk_cbeg[i]);
        p->wk_cend.push_back(base + o.wk_cend[i]);
      }
      for (const int32_t c : o.wk_chunks) p->wk_chunks.push_back(ch_begin + c);
    }
    {
      const int32_t base = (int32_t)p->tc_chunks.size();
      for (size_t i = 0; i < o.tc_row0.size(); ++i) {
        p->tc_prob.push_back(b);
        p->tc_row0.push_back(o.tc_row0[i]);
        p->tc_col0.push_back(o.tc_col0[i]);
        p->tc_ncols.push_back(o.tc_ncols[i]);
        p->tc_cbeg.push_back(base + o.tc_cbeg[i]);
        p->tc_cend.push_back(base + o.tc_cend[i]);
      }
      for (const int32_t c : o.tc_chunks) p->tc_chunks.push_back(ch_begin + c);
    }
    const int32_t maxw = o.maxw;
    p->p_npose.push_back(N);
    p->p_frame_off.push_back(frame_off);
    p->p_pose_off.push_back(pose_off);
    p->p_lm_off.push_back(lm_off);
    p->p_lm_cnt.push_back(L);
    p->p_pair_D.push_back(maxw);
    p->p_param_off.push_back(param_off);
    p->p_chunk_off.push_back(ch_begin);
    p->p_chunk_cnt.push_back(nch);
    p->p_S_off.push_back(S_off);
    p->p_pair_off.push_back(pair_off);
    p->p_nres.push_back(4 * q.n_obs);
    for (int k = 0; k < 8; ++k) p->p_intr.push_back(q.intrinsics[k]);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 4; ++c) p->p_Trl.push_back(q.T_r_to_l[4 * r + c]);
    for (int k = 0; k <= N; ++k) p->fr_prob.push_back(b);
    for (int k = 0; k < N; ++k) p->pose_prob.push_back(b);
    p->max_P = std::max(p->max_P, P);
    p->max_D = std::max(p->max_D, maxw);
    frame_off += N + 1;
    pose_off += N;
    lm_off += L;
    param_off += P;
    S_off += (int64_t)P * P;
    pair_off += (int64_t)N * maxw;
    slab_off += o.slab;
  }
  const int64_t obs_total = Ot;
  p->lm_obs[(size_t)Lt] = obs_total;
  {  // tensor-core Schur items longest first (one CTA per SM: the last wave stays short)
    const size_t n = p->tc_prob.size();
    std::vector<size_t> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](size_t x, size_t y) {
      return p->tc_cend[x] - p->tc_cbeg[x] > p->tc_cend[y] - p->tc_cbeg[y];
    });
    auto perm = [&](std::vector<int32_t> &v) {
      std::vector<int32_t> t(n);
      for (size_t i = 0; i < n; ++i) t[i] = v[ord[i]];
      v.swap(t);
    };
    perm(p->tc_prob); perm(p->tc_row0); perm(p->tc_col0); perm(p->tc_ncols); perm(p->tc_cbeg); perm(p->tc_cend);
  }
  p->F = frame_off;
  p->NP = pose_off;
  p->L = lm_off;
  p->O = obs_total;
  p->total_params = param_off;
  p->total_S = S_off;
  p->total_pairs = pair_off;
  p->total_slab = slab_off;
  {  // factorisation route per problem: batched in shared memory, or the multi-CTA path
    const size_t ts = precision == SPGO_PREC_FP64 ? 8 : 4;
    for (int b = 0; b < nprob; ++b) {
      const int P = 6 * p->p_npose[b];
      if (factor_packed_bytes(P, ts) <= SPGO_FACTOR_SMEM)
        p->max_P_small = std::max(p->max_P_small, P);
      else
        p->large.push_back(b);
    }
    // widest first: the CTAs of the widest systems (the longest) start first and
    // the narrow ones fill in beside and behind them
    p->fs_prob.resize(nprob);
    std::iota(p->fs_prob.begin(), p->fs_prob.end(), 0);
    std::stable_sort(p->fs_prob.begin(), p->fs_prob.end(),
                     [&](int32_t x, int32_t y) { return p->p_npose[x] > p->p_npose[y]; });
  }
  build_layout(p);
  return SPGO_OK;
}

// ---------------------------------------------------------------------------
// solver
// ---------------------------------------------------------------------------
struct spgo_solver {
  const spgo_plan *plan;
  PlanView pv;
  WorkView wv;
  Params prm;
  double *poses, *alpha;
  unsigned char *d_static, *d_ws;
  int64_t launches0;
  bool controller = false;  // learned damping active
  // optional per-kernel timing: event pairs recorded around each launch
  bool prof = false;
  std::vector<cudaEvent_t> ev;
  std::vector<int> ev_kind;
  size_t ev_used = 0;
  // captured LM iterations: one graph per iteration count, rebuilt when parameters change
  struct Graph {
    int n_iters;
    cudaGraphExec_t exec;
    int64_t kernels;  // kernel nodes, for the launch count
  };
  std::vector<Graph> graphs;
  // page-locked copy of the per-problem LM states for status reads: a copy into
  // pageable memory would hold the driver until the stream drains, stalling the
  // API calls of threads that drive other solvers
  HostBlock h_lm;  // from the staging cache (freeing page-locked memory synchronises the device)
  // status reads poll this event and yield the core between polls: several solver
  // threads and the planner's share the host cores, and a spinning wait would take
  // one from them, while a sleeping wait would wake up late and leave the GPU idle
  cudaEvent_t status_ev = nullptr;
  // a second stream for the LM iteration's fork: the pose-pair reduction runs beside
  // the landmark Schur complement (both read only the linearisation's output)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

static void drop_graphs(spgo_solver *s) {
  for (auto &g : s->graphs) cudaGraphExecDestroy(g.exec);
  s->graphs.clear();
}

// profiled kernel kinds (spgo_profile_read order)
enum { K_CHAIN, K_LINEARIZE, K_COST, K_SYSTEM, K_SCHUR, K_ASSEMBLE, K_FACTOR, K_BACKSUB, K_UPDATE,
       K_BOOKKEEP, K_REFINE, K_RESID, K_NKINDS };
static_assert(K_NKINDS == SPGO_PROFILE_KINDS, "profile kinds");

struct ProfScope {
  spgo_solver *s;
  cudaStream_t st;
  int kind;
  size_t slot;
  ProfScope(spgo_solver *s_, cudaStream_t st_, int kind_) : s(s_), st(st_), kind(kind_), slot((size_t)-1) {
    if (s->prof && s->ev_used + 2 <= s->ev.size()) {
      slot = s->ev_used;
      s->ev_used += 2;
      s->ev_kind[slot / 2] = kind;
      cudaEventRecord(s->ev[slot], st);
    }
  }
  ~ProfScope() {
    if (slot != (size_t)-1) cudaEventRecord(s->ev[slot + 1], st);
  }
};
#define PROF(kind) ProfScope _prof_scope(s, st, kind)

template <typename T>
static const T *seg_ptr(const spgo_plan *p, unsigned char *base, int idx) {
  return reinterpret_cast<const T *>(base + p->segs[idx].off);
}

static void make_views(spgo_solver *s) {
  const spgo_plan *p = s->plan;
  unsigned char *st = s->d_static;
  PlanView &v = s->pv;
  std::memset(&v, 0, sizeof(v));
  v.B = p->B; v.F = p->F; v.NP = p->NP; v.L = p->L; v.O = p->O;
  v.n_chunks = (int32_t)p->ch_prob.size();
  v.n_items = (int32_t)p->wk_prob.size();
  v.max_P = p->max_P; v.max_D = p->max_D; v.max_nb = p->max_nb;
  v.n_work_chunks = (int32_t)p->wk_chunks.size();
  v.total_S = p->total_S; v.total_pairs = p->total_pairs; v.total_params = p->total_params;
  int i = 0;
  v.p_npose = seg_ptr<int32_t>(p, st, i++); v.p_frame_off = seg_ptr<int32_t>(p, st, i++);
  v.p_pose_off = seg_ptr<int32_t>(p, st, i++); v.p_lm_off = seg_ptr<int32_t>(p, st, i++);
  v.p_lm_cnt = seg_ptr<int32_t>(p, st, i++); v.p_pair_D = seg_ptr<int32_t>(p, st, i++);
  v.p_param_off = seg_ptr<int32_t>(p, st, i++); v.p_chunk_off = seg_ptr<int32_t>(p, st, i++);
  v.p_chunk_cnt = seg_ptr<int32_t>(p, st, i++); v.p_S_off = seg_ptr<int64_t>(p, st, i++);
  v.p_pair_off = seg_ptr<int64_t>(p, st, i++); v.p_nres = seg_ptr<int64_t>(p, st, i++);
  v.p_intr = seg_ptr<float>(p, st, i++);
  v.p_Trl = seg_ptr<double>(p, st, i++); v.lm_prob = seg_ptr<int32_t>(p, st, i++);
  v.lm_host = seg_ptr<int32_t>(p, st, i++); v.lm_lo = seg_ptr<int32_t>(p, st, i++);
  v.lm_hi = seg_ptr<int32_t>(p, st, i++); v.lm_user = seg_ptr<int32_t>(p, st, i++);
  v.lm_chunk = seg_ptr<int32_t>(p, st, i++); v.lm_slot = seg_ptr<int32_t>(p, st, i++);
  v.lm_uv = seg_ptr<float>(p, st, i++); v.lm_obs = seg_ptr<int64_t>(p, st, i++);
  v.obs_frame = seg_ptr<int32_t>(p, st, i++); v.obs_uv = seg_ptr<float>(p, st, i++);
  v.ch_prob = seg_ptr<int32_t>(p, st, i++); v.ch_f0 = seg_ptr<int32_t>(p, st, i++);
  v.ch_nb = seg_ptr<int32_t>(p, st, i++); v.ch_lm0 = seg_ptr<int32_t>(p, st, i++);
  v.ch_cnt = seg_ptr<int32_t>(p, st, i++); v.ch_slab = seg_ptr<int64_t>(p, st, i++);
  v.wk_prob = seg_ptr<int32_t>(p, st, i++); v.wk_ti = seg_ptr<int32_t>(p, st, i++);
  v.wk_tj = seg_ptr<int32_t>(p, st, i++); v.wk_cbeg = seg_ptr<int32_t>(p, st, i++);
  v.wk_cend = seg_ptr<int32_t>(p, st, i++); v.wk_chunks = seg_ptr<int32_t>(p, st, i++);
  v.fr_prob = seg_ptr<int32_t>(p, st, i++); v.pose_prob = seg_ptr<int32_t>(p, st, i++);
  v.obs_slot = seg_ptr<uint8_t>(p, st, i++);
  v.tc_prob = seg_ptr<int32_t>(p, st, i++); v.tc_row0 = seg_ptr<int32_t>(p, st, i++);
  v.tc_col0 = seg_ptr<int32_t>(p, st, i++); v.tc_ncols = seg_ptr<int32_t>(p, st, i++);
  v.tc_cbeg = seg_ptr<int32_t>(p, st, i++); v.tc_cend = seg_ptr<int32_t>(p, st, i++);
  v.tc_chunks = seg_ptr<int32_t>(p, st, i++);
  v.fs_prob = seg_ptr<int32_t>(p, st, i++);
  v.n_tc_items = (int32_t)p->tc_prob.size();
  v.max_P_small = p->max_P_small;
  unsigned char *w = s->d_ws;
  WorkView &x = s->wv;
  x.fr_Rf = reinterpret_cast<float *>(w + p->w_frRf);
  x.fr_Rl = reinterpret_cast<float *>(w + p->w_frRl);
  x.fr_Rd = reinterpret_cast<double *>(w + p->w_frRd);
  x.fr_c = reinterpret_cast<double *>(w + p->w_frc);
  x.fr_ch = reinterpret_cast<float *>(w + p->w_frch);
  x.fr_cl = reinterpret_cast<float *>(w + p->w_frcl);
  x.poses_cand = reinterpret_cast<double *>(w + p->w_pcand);
  x.alpha_cand = reinterpret_cast<double *>(w + p->w_acand);
  x.res = reinterpret_cast<float *>(w + p->w_res);
  x.pair_acc = w + p->w_pacc;
  x.pairF = w + p->w_pF;
  x.A = w + p->w_A;
  x.g = w + p->w_g;
  x.SL = w + p->w_SL;
  x.gL = w + p->w_gL;
  x.fac = w + p->w_fac;
  if (!p->large.empty()) {
    x.Sx = w + p->w_Sx;
    double *lg = reinterpret_cast<double *>(w + p->w_lg);
    const size_t tp = (size_t)p->total_params;
    x.lg_g0 = lg;
    x.lg_x = lg + tp;
    x.lg_xs = reinterpret_cast<float *>(lg + 2 * tp);  // 2 tp floats
    x.lg_y = lg + 3 * tp;
    x.lg_dinv = lg + 4 * tp;
    x.lg_flag = reinterpret_cast<int *>(w + p->w_lgflag);
    x.lg_red = p->w_lgred ? reinterpret_cast<double *>(w + p->w_lgred) : nullptr;
  }
  x.delta = reinterpret_cast<double *>(w + p->w_delta);
  x.C = w + p->w_C;
  x.ga = w + p->w_ga;
  x.slab = w + p->w_slab;
  x.lm = reinterpret_cast<LMState *>(w + p->w_lm);
  x.cost_acc = reinterpret_cast<double *>(w + p->w_cost);
  x.pred_acc = reinterpret_cast<double *>(w + p->w_pred);
  x.lm_backup = reinterpret_cast<LMState *>(w + p->w_lmb);
  x.probe_costs = reinterpret_cast<double *>(w + p->w_probe);
  x.trace = reinterpret_cast<double *>(w + p->w_trace);
  x.ctrl = w + p->w_ctrl;
  if (p->precision == SPGO_PREC_MIXED) {
    x.tcam = reinterpret_cast<float *>(w + p->w_tcam);
    x.xanc = reinterpret_cast<float *>(w + p->w_xanc);
    x.facs = reinterpret_cast<float *>(w + p->w_facs);
    x.twist = reinterpret_cast<float *>(w + p->w_twist);
    x.pdual = reinterpret_cast<double *>(w + p->w_pdual);
    x.dal = reinterpret_cast<double *>(w + p->w_dal);
    x.tl = reinterpret_cast<float *>(w + p->w_tl);
    x.gaacc = reinterpret_cast<double *>(w + p->w_gaacc);
    x.gacc = reinterpret_cast<double *>(w + p->w_gacc);
    x.rhsB = reinterpret_cast<float *>(w + p->w_rhsB);
    x.ddelta = reinterpret_cast<double *>(w + p->w_ddelta);
  }
}

// one linearisation + reduced system (+ damping from the device-side lambda)
// `stats`: refresh the controller's per-problem statistics; `ctrl`: let the learned
// controller set lambda for the step about to be taken from the fresh linearisation
template <typename T>
constexpr int kF64 = std::is_same<T, double>::value ? 1 : 0;

template <typename T>
static int enqueue_linearize(spgo_solver *s, cudaStream_t st, bool stats, bool ctrl) {
  // (the frame tables and the cost of the state come from enqueue_reset for the first
  // linearisation, and from the accepted candidate's chain and cost pass after that)
  { PROF(K_LINEARIZE); CUDA_TRY(launch_linearize<T>(s->pv, s->wv, s->prm, s->alpha, 0, GATE_RELIN, st)); }
  { PROF(K_SYSTEM); CUDA_TRY(launch_system<T>(s->pv, s->wv, GATE_RELIN, st)); }
  {
    PROF(K_BOOKKEEP);
    if (stats || ctrl) CUDA_TRY(launch_lm_stats(s->pv, s->wv, std::is_same<T, double>::value, st));
    CUDA_TRY(launch_post_linearize(s->pv, s->wv, st));
    if (ctrl) CUDA_TRY(launch_controller(s->pv, s->wv, s->prm, s->wv.ctrl, st));
  }
  return SPGO_OK;
}

// reset every problem's LM state, then the frame tables and the cost of the state for
// the first linearisation (outside the per-iteration sequence, so the iterations a
// CUDA graph replays carry no launches that only the first one needs)
template <typename T>
static int enqueue_reset_t(spgo_solver *s, cudaStream_t st, double lam) {
  { PROF(K_BOOKKEEP); CUDA_TRY(launch_reset(s->pv, s->wv, s->prm, lam, st)); }
  { PROF(K_CHAIN); CUDA_TRY(launch_chain(s->pv, s->wv, s->poses, GATE_FIRST, kF64<T>, st)); }
  { PROF(K_COST); CUDA_TRY(launch_linearize<T>(s->pv, s->wv, s->prm, s->alpha, 1, GATE_FIRST, st)); }
  return SPGO_OK;
}
static int enqueue_reset(spgo_solver *s, cudaStream_t st, double lam) {
  return s->plan->precision == SPGO_PREC_FP64 ? enqueue_reset_t<double>(s, st, lam)
                                               : enqueue_reset_t<float>(s, st, lam);
}

template <typename T>
static int enqueue_schur(spgo_solver *s, cudaStream_t st) {
  PROF(K_SCHUR);
  if (s->plan->precision == SPGO_PREC_MIXED && s->prm.use_tc)
    CUDA_TRY(launch_schur_tc(s->pv, s->wv, s->prm, st));
  else
    CUDA_TRY(launch_schur<T>(s->pv, s->wv, s->prm, st));
  return SPGO_OK;
}

template <typename T>
static int enqueue_factor(spgo_solver *s, cudaStream_t st) {
  const int mixed = s->plan->precision == SPGO_PREC_MIXED;
  {
    PROF(K_FACTOR);
    CUDA_TRY(launch_factor_solve<T>(s->pv, s->wv, s->prm, mixed, st));
    for (const int b : s->plan->large)
      CUDA_TRY(launch_factor_large<T>(s->pv, s->wv, s->prm, b, 6 * s->plan->p_npose[b], s->plan->p_param_off[b],
                                      (mixed && !(s->prm.outer_steps > 0 && s->wv.facs)) ? s->prm.refine_steps : 0,
                                      st, s->side, s->ev_fork, s->ev_join));
  }
  return SPGO_OK;
}

template <typename T>
static int enqueue_solve_step(spgo_solver *s, cudaStream_t st) {
  int rc;
  if ((rc = enqueue_schur<T>(s, st)) != SPGO_OK) return rc;
  return enqueue_factor<T>(s, st);
}

// the candidate state of the damped step: solve, then (mixed path, outer_steps > 0)
// iterative refinement against the accurately summed residual of the whole system,
// then the inverse-depth back-substitution and the pose update (each adding its share
// of the predicted decrease)
template <typename T>
static int enqueue_candidate(spgo_solver *s, cudaStream_t st, bool solved = false) {
  int rc;
  if (!solved && (rc = enqueue_solve_step<T>(s, st)) != SPGO_OK) return rc;
  const int outer = std::is_same<T, float>::value && s->wv.facs ? s->prm.outer_steps : 0;
  if (outer <= 0) {
    { PROF(K_BACKSUB); CUDA_TRY(launch_backsub<T>(s->pv, s->wv, s->prm, s->alpha, s->wv.alpha_cand, 0, st)); }
    { PROF(K_UPDATE); CUDA_TRY(launch_update_poses<T>(s->pv, s->wv, s->poses, s->wv.poses_cand, 1.0, 0, st)); }
    return SPGO_OK;
  }
  { PROF(K_REFINE); CUDA_TRY(launch_pair_twists(s->pv, s->wv, st)); }
  for (int k = 0; k < outer; ++k) {
    { PROF(K_RESID); CUDA_TRY(launch_resid_pass(s->pv, s->wv, s->prm, s->alpha, k == 0, st)); }
    PROF(K_REFINE);
    CUDA_TRY(launch_resid_solve(s->pv, s->wv, s->prm, k == 0, st));
    for (const int b : s->plan->large) {
      CUDA_TRY(launch_resid_reduce_large(s->pv, s->wv, b, s->plan->p_npose[b], st));
      CUDA_TRY(launch_refine_large(s->pv, s->wv, s->prm, b, 6 * s->plan->p_npose[b], s->plan->p_param_off[b], st));
    }
    if (k + 1 < outer) CUDA_TRY(launch_pair_twists(s->pv, s->wv, st));
  }
  { PROF(K_BACKSUB); CUDA_TRY(launch_backsub_refined(s->pv, s->wv, s->prm, s->alpha, s->wv.alpha_cand, st)); }
  {
    PROF(K_UPDATE);
    CUDA_TRY(launch_update_poses<T>(s->pv, s->wv, s->poses, s->wv.poses_cand, 1.0, 0, st, s->wv.gacc));
  }
  return SPGO_OK;
}

// Without the learned controller (whose statistics read A and g, and whose lambda the
// Schur complement uses) the iteration forks after the Jacobian pass: the pose-pair
// reduction (A, g) on the solver's second stream beside the landmark Schur complement
// (S_L, g_L) on the caller's; both read only the linearisation's output, the
// factorisation joins them.  Under stream capture the fork becomes two graph branches.
template <typename T>
static int enqueue_lm_iteration(spgo_solver *s, cudaStream_t st) {
  int rc;
  if (!s->controller && s->side) {
    { PROF(K_LINEARIZE); CUDA_TRY(launch_linearize<T>(s->pv, s->wv, s->prm, s->alpha, 0, GATE_RELIN, st)); }
    CUDA_TRY(cudaEventRecord(s->ev_fork, st));
    CUDA_TRY(cudaStreamWaitEvent(s->side, s->ev_fork, 0));
    {
      ProfScope side_scope(s, s->side, K_SYSTEM);
      CUDA_TRY(launch_system<T>(s->pv, s->wv, GATE_RELIN, s->side));
    }
    CUDA_TRY(cudaEventRecord(s->ev_join, s->side));
    if ((rc = enqueue_schur<T>(s, st)) != SPGO_OK) return rc;
    CUDA_TRY(cudaStreamWaitEvent(st, s->ev_join, 0));
    // (the pair reduction gates on the relinearisation flag this clears)
    { PROF(K_BOOKKEEP); CUDA_TRY(launch_post_linearize(s->pv, s->wv, st)); }
    if ((rc = enqueue_factor<T>(s, st)) != SPGO_OK) return rc;
    if ((rc = enqueue_candidate<T>(s, st, true)) != SPGO_OK) return rc;
  } else {
    if ((rc = enqueue_linearize<T>(s, st, s->controller, s->controller)) != SPGO_OK) return rc;
    if ((rc = enqueue_candidate<T>(s, st)) != SPGO_OK) return rc;
  }
  { PROF(K_CHAIN); CUDA_TRY(launch_chain(s->pv, s->wv, s->wv.poses_cand, GATE_RUNNING, kF64<T>, st)); }
  { PROF(K_COST); CUDA_TRY(launch_linearize<T>(s->pv, s->wv, s->prm, s->wv.alpha_cand, 1, GATE_RUNNING, st)); }
  {
    PROF(K_BOOKKEEP);
    CUDA_TRY(launch_decide(s->pv, s->wv, s->prm, st));
  }
  { PROF(K_BOOKKEEP); CUDA_TRY(launch_commit(s->pv, s->wv, s->poses, s->alpha, st)); }
  if (std::is_same<T, float>::value && s->wv.facs && s->prm.outer_steps > 0) {
    // the refinement recomputes the Jacobian at the state from the frame tables, which
    // a rejected candidate's chain has overwritten: back to the state's
    PROF(K_CHAIN);
    CUDA_TRY(launch_chain(s->pv, s->wv, s->poses, GATE_REJECTED, kF64<T>, st));
  }
  return SPGO_OK;
}

template <typename T>
static int enqueue_gn(spgo_solver *s, int iters, float step_size, cudaStream_t st) {
  for (int it = 0; it < iters; ++it) {
    int rc;
    if ((rc = enqueue_reset_t<T>(s, st, 0.0)) != SPGO_OK) return rc;
    if ((rc = enqueue_linearize<T>(s, st, false, false)) != SPGO_OK) return rc;
    if ((rc = enqueue_solve_step<T>(s, st)) != SPGO_OK) return rc;
    { PROF(K_BACKSUB); CUDA_TRY(launch_backsub<T>(s->pv, s->wv, s->prm, s->alpha, s->alpha, 1, st)); }
    { PROF(K_UPDATE); CUDA_TRY(launch_update_poses<T>(s->pv, s->wv, s->poses, s->poses, (double)step_size, 1, st)); }
  }
  return SPGO_OK;
}

template <typename T>
static int enqueue_probe(spgo_solver *s, int nf, const double *factors, cudaStream_t st) {
  int rc;
  // the statistics feed the features of the probed states; the controller does not act
  if ((rc = enqueue_linearize<T>(s, st, true, false)) != SPGO_OK) return rc;
  CUDA_TRY(cudaMemcpyAsync(s->wv.lm_backup, s->wv.lm, sizeof(LMState) * s->plan->B, cudaMemcpyDeviceToDevice, st));
  for (int j = 0; j < nf; ++j) {
    CUDA_TRY(launch_scale_lambda(s->pv, s->wv, factors[j], st));
    if ((rc = enqueue_candidate<T>(s, st)) != SPGO_OK) return rc;
    CUDA_TRY(launch_chain(s->pv, s->wv, s->wv.poses_cand, GATE_RUNNING, kF64<T>, st));
    CUDA_TRY(launch_linearize<T>(s->pv, s->wv, s->prm, s->wv.alpha_cand, 1, GATE_RUNNING, st));
    CUDA_TRY(launch_take_probe(s->pv, s->wv, j, st));
    // (the next probe's refinement reads the state's frame tables)
    if (std::is_same<T, float>::value && s->wv.facs && s->prm.outer_steps > 0 && j + 1 < nf)
      CUDA_TRY(launch_chain(s->pv, s->wv, s->poses, GATE_RUNNING, kF64<T>, st));
  }
  CUDA_TRY(cudaMemcpyAsync(s->wv.lm, s->wv.lm_backup, sizeof(LMState) * s->plan->B, cudaMemcpyDeviceToDevice, st));
  // the probes overwrote the frame tables: back to the state's
  CUDA_TRY(launch_chain(s->pv, s->wv, s->poses, GATE_RUNNING, kF64<T>, st));
  return SPGO_OK;
}

extern "C" {

int spgo_version(void) { return 1; }

const char *spgo_last_error(void) { return g_err.c_str(); }

void spgo_default_params(spgo_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->loss = SPGO_LOSS_L2;
  p->near_boost = 0;
  p->loss_scale = 3.0f;
  p->eps = 1e-4f;
  p->alpha_min = 1.0f / 30.0f;
  p->alpha_max = 1.0f / 0.2f;
  p->lambda0 = 1e-4;
  p->lambda_max = 1e16;
  p->tol = 1e-6;
  p->max_iters = 30;
  p->refine_steps = 1;
  p->use_graph = 1;
  p->use_tc = 1;
  p->outer_steps = 2;
  p->wait_us = 0;
  p->ctl_min_log10 = -6.0f;
  p->outer_tol = 1e-3f;
  p->stop_rho = 0.f;
}

int spgo_plan_create(const spgo_host_problem *problems, int32_t n_problems, int32_t precision, spgo_plan **out) {
  return spgo_plan_create_opts(problems, n_problems, precision, nullptr, out);
}

int spgo_plan_create_opts(const spgo_host_problem *problems, int32_t n_problems, int32_t precision,
                          const spgo_plan_options *opts, spgo_plan **out) {
  if (!out) return fail(SPGO_ERR_INVALID_ARG, "out is null");
  *out = nullptr;
  if (opts) {
    if (opts->tc_split < 0 || opts->tc_split > SPGO_TC_SPLIT || opts->simt_split < 0 || opts->simt_split > 64)
      return fail(SPGO_ERR_INVALID_ARG, "plan options out of range (tc_split 1..64, simt_split 1..64, 0: default)");
    for (int k = 0; k < 6; ++k)
      if (opts->reserved[k] != 0) return fail(SPGO_ERR_INVALID_ARG, "plan options: reserved fields must be zero");
  }
  spgo_plan *p = new (std::nothrow) spgo_plan();
  if (!p) return fail(SPGO_ERR_INVALID_ARG, "host allocation failed");
  if (opts && opts->tc_split > 0) p->tc_split = opts->tc_split;
  if (opts && opts->simt_split > 0) p->simt_split = opts->simt_split;
  int rc;
  try {
    rc = plan_build(problems, n_problems, precision, p);
  } catch (const std::exception &e) {
    rc = fail(SPGO_ERR_INVALID_ARG, e.what());
  }
  if (rc != SPGO_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return SPGO_OK;
}

int spgo_plan_sizes_get(const spgo_plan *p, spgo_plan_sizes *o) {
  if (!p || !o) return fail(SPGO_ERR_INVALID_ARG, "null argument");
  std::memset(o, 0, sizeof(*o));
  o->n_problems = p->B;
  o->total_poses = p->NP;
  o->total_landmarks = p->L;
  o->total_obs = p->O;
  o->n_chunks = (int32_t)p->ch_prob.size();
  o->n_schur_items = (int32_t)p->wk_prob.size();
  o->max_params = p->max_P;
  o->schur_chunk_tiles = (int32_t)p->wk_chunks.size();
  o->schur_flops = 0;
  for (size_t c = 0; c < p->ch_nb.size(); ++c) o->schur_flops += 2LL * (6LL * p->ch_nb[c]) * (6LL * p->ch_nb[c]) * 32;
  o->schur_flops_landmark = 0;
  for (int32_t l = 0; l < p->L; ++l) {
    const int64_t k = p->lm_hi[l] - p->lm_lo[l];
    o->schur_flops_landmark += 2 * (6 * k) * (6 * k);
  }
  o->n_tc_items = (int32_t)p->tc_prob.size();
  o->tc_chunk_tiles = (int32_t)p->tc_chunks.size();
  o->tc_split = p->tc_split;
  o->simt_split = p->simt_split;
  o->static_bytes = p->static_bytes;
  o->workspace_bytes = p->ws_bytes;
  o->slab_elems = p->total_slab;
  o->pair_records = p->total_pairs;
  return SPGO_OK;
}

int spgo_plan_offsets(const spgo_plan *p, int32_t *lm_off, int32_t *pose_off) {
  if (!p) return fail(SPGO_ERR_INVALID_ARG, "null plan");
  for (int b = 0; b < p->B; ++b) {
    if (lm_off) lm_off[b] = p->p_lm_off[b];
    if (pose_off) pose_off[b] = p->p_pose_off[b];
  }
  return SPGO_OK;
}

int spgo_plan_destroy(spgo_plan *p) {
  delete p;
  return SPGO_OK;
}

int spgo_solver_create(const spgo_plan *plan, void *d_static, size_t static_bytes, void *d_workspace,
                       size_t workspace_bytes, double *d_poses, double *d_alpha, void *stream, spgo_solver **out) {
  if (!out || !plan || !d_poses || !d_alpha) return fail(SPGO_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (static_bytes < plan->static_bytes || workspace_bytes < plan->ws_bytes)
    return fail(SPGO_ERR_BUFFER_SMALL, "device buffers smaller than spgo_plan_sizes_get reports");
  if ((plan->static_bytes && !d_static) || (plan->ws_bytes && !d_workspace))
    return fail(SPGO_ERR_INVALID_ARG, "null device buffer");
  if (((uintptr_t)d_static & 255) || ((uintptr_t)d_workspace & 255))
    return fail(SPGO_ERR_INVALID_ARG, "device buffers must be 256-byte aligned");
  spgo_solver *s = new (std::nothrow) spgo_solver();
  if (!s) return fail(SPGO_ERR_INVALID_ARG, "host allocation failed");
  s->plan = plan;
  s->d_static = (unsigned char *)d_static;
  s->d_ws = (unsigned char *)d_workspace;
  s->poses = d_poses;
  s->alpha = d_alpha;
  spgo_params dp;
  spgo_default_params(&dp);
  std::memcpy(&s->prm, &dp, sizeof(Params));
  cudaStream_t st = (cudaStream_t)stream;
  {  // two copies from the page-locked staging blocks; the event keeps the blocks
     // out of the cache until the copies have read them
    std::lock_guard<std::mutex> lk(plan->upload_mu);
    cudaError_t e = cudaSuccess;
    if (plan->big_bytes)
      e = cudaMemcpyAsync(s->d_static, plan->big.ptr, plan->big_bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && plan->static_bytes > plan->big_bytes)
      e = cudaMemcpyAsync(s->d_static + plan->big_bytes, plan->small.ptr, plan->static_bytes - plan->big_bytes,
                          cudaMemcpyHostToDevice, st);
    cudaEvent_t ev = nullptr;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) {
      plan->uploads.push_back(ev);
      e = cudaEventRecord(ev, st);
    }
    if (e != cudaSuccess) {
      delete s;
      return fail(SPGO_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
    }
  }
  cudaError_t e = cudaMemsetAsync(s->d_ws, 0, plan->ws_bytes, st);
  if (e != cudaSuccess) {
    delete s;
    return fail(SPGO_ERR_CUDA, std::string("workspace clear: ") + cudaGetErrorString(e));
  }
  make_views(s);
  try {
    s->h_lm = arena_get(sizeof(LMState) * (size_t)std::max(1, plan->B));
  } catch (const std::exception &ex) {
    delete s;
    return fail(SPGO_ERR_INVALID_ARG, ex.what());
  }
  {
    cudaError_t e = cudaEventCreateWithFlags(&s->status_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      if (s->ev_fork) cudaEventDestroy(s->ev_fork);
      if (s->side) cudaStreamDestroy(s->side);
      if (s->status_ev) cudaEventDestroy(s->status_ev);
      arena_put(s->h_lm);
      delete s;
      return fail(SPGO_ERR_CUDA, std::string("solver events / stream: ") + cudaGetErrorString(e));
    }
  }
  s->launches0 = g_launches;
  *out = s;
  return SPGO_OK;
}

int spgo_solver_destroy(spgo_solver *s) {
  if (s) {
    for (cudaEvent_t e : s->ev) cudaEventDestroy(e);
    drop_graphs(s);
    arena_put(s->h_lm);
    if (s->status_ev) cudaEventDestroy(s->status_ev);
    if (s->side) {
      cudaStreamSynchronize(s->side);  // its work always joins the caller's stream; this is belt and braces
      cudaStreamDestroy(s->side);
    }
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
  }
  delete s;
  return SPGO_OK;
}

int spgo_profile_enable(spgo_solver *s, int32_t capacity) {
  if (!s || capacity < 0) return fail(SPGO_ERR_INVALID_ARG, "bad argument");
  for (cudaEvent_t e : s->ev) cudaEventDestroy(e);
  s->ev.assign((size_t)capacity * 2, nullptr);
  s->ev_kind.assign((size_t)capacity, 0);
  for (auto &e : s->ev) CUDA_TRY(cudaEventCreate(&e));
  s->ev_used = 0;
  s->prof = capacity > 0;
  return SPGO_OK;
}

int spgo_profile_read(spgo_solver *s, double *ms, int64_t *count, int32_t n_kinds, void *stream) {
  if (!s || !ms || !count || n_kinds < K_NKINDS) return fail(SPGO_ERR_INVALID_ARG, "bad argument");
  CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  for (int k = 0; k < n_kinds; ++k) {
    ms[k] = 0.0;
    count[k] = 0;
  }
  for (size_t i = 0; i + 1 < s->ev_used; i += 2) {
    float t = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&t, s->ev[i], s->ev[i + 1]));
    ms[s->ev_kind[i / 2]] += t;
    count[s->ev_kind[i / 2]] += 1;
  }
  s->ev_used = 0;
  return SPGO_OK;
}

int spgo_set_params(spgo_solver *s, const spgo_params *p) {
  if (!s || !p) return fail(SPGO_ERR_INVALID_ARG, "null argument");
  if (p->loss < 0 || p->loss > 2) return fail(SPGO_ERR_INVALID_ARG, "unknown loss");
  if (!(p->loss_scale > 0) || !(p->eps >= 0) || !(p->alpha_min < p->alpha_max) || p->max_iters < 0 ||
      p->refine_steps < 0 || !(p->lambda0 >= 0) || p->outer_steps < 0 || p->outer_steps > 8 || p->wait_us < 0 ||
      !(p->ctl_min_log10 <= 0.f && p->ctl_min_log10 >= -6.f) || !(p->outer_tol >= 0.f && p->outer_tol < 1.f) ||
      !(p->stop_rho >= 0.f && p->stop_rho < 1.f))
    return fail(SPGO_ERR_INVALID_ARG, "parameter out of range");
  for (const int32_t blk : {p->cost_block, p->lin_block})
    if (blk != 0 && (blk < 32 || blk > 256 || blk % 32 != 0))
      return fail(SPGO_ERR_INVALID_ARG, "CTA size must be 0 or a multiple of 32 in [32, 256]");
  static_assert(sizeof(Params) == sizeof(spgo_params), "params layout");
  std::memcpy(&s->prm, p, sizeof(Params));
  drop_graphs(s);  // captured launches carry the old parameters
  return SPGO_OK;
}

int spgo_gn_step(spgo_solver *s, int32_t iterations, float step_size, void *stream) {
  if (!s || iterations < 0) return fail(SPGO_ERR_INVALID_ARG, "bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  return s->plan->precision == SPGO_PREC_FP64 ? enqueue_gn<double>(s, iterations, step_size, st)
                                              : enqueue_gn<float>(s, iterations, step_size, st);
}

int spgo_lm_reset(spgo_solver *s, void *stream) {
  if (!s) return fail(SPGO_ERR_INVALID_ARG, "null solver");
  return enqueue_reset(s, (cudaStream_t)stream, s->prm.lambda0);
}

static int enqueue_iterations(spgo_solver *s, int32_t n_iters, cudaStream_t st) {
  for (int it = 0; it < n_iters; ++it) {
    int rc = s->plan->precision == SPGO_PREC_FP64 ? enqueue_lm_iteration<double>(s, st)
                                                  : enqueue_lm_iteration<float>(s, st);
    if (rc != SPGO_OK) return rc;
  }
  return SPGO_OK;
}

int spgo_lm_iterate(spgo_solver *s, int32_t n_iters, void *stream) {
  if (!s || n_iters < 0) return fail(SPGO_ERR_INVALID_ARG, "bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  const bool graphable = s->prm.use_graph && !s->prof && st != nullptr && st != cudaStreamLegacy &&
                         st != cudaStreamPerThread;
  if (!graphable || n_iters == 0) return enqueue_iterations(s, n_iters, st);
  for (auto &g : s->graphs)
    if (g.n_iters == n_iters) {
      CUDA_TRY(cudaGraphLaunch(g.exec, st));
      g_launches += g.kernels;
      return SPGO_OK;
    }
  // capture n_iters iterations once; device-side gating keeps replays exact
  cudaStreamCaptureStatus cs;
  CUDA_TRY(cudaStreamIsCapturing(st, &cs));
  if (cs != cudaStreamCaptureStatusNone) return enqueue_iterations(s, n_iters, st);  // caller is capturing
  CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const int64_t l0 = g_launches;
  int rc = enqueue_iterations(s, n_iters, st);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(st, &graph);
  if (rc != SPGO_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return fail(SPGO_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(SPGO_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  const int64_t kernels = g_launches - l0;
  g_launches = l0;  // the capture itself ran nothing; replays are counted
  s->graphs.push_back(spgo_solver::Graph{n_iters, exec, kernels});
  CUDA_TRY(cudaGraphLaunch(exec, st));
  g_launches += kernels;
  return SPGO_OK;
}

int spgo_lm_status(spgo_solver *s, spgo_problem_status *out, void *stream) {
  if (!s) return fail(SPGO_ERR_INVALID_ARG, "null argument");
  LMState *h = reinterpret_cast<LMState *>(s->h_lm.ptr);
  CUDA_TRY(cudaMemcpyAsync(h, s->wv.lm, sizeof(LMState) * (size_t)s->plan->B, cudaMemcpyDeviceToHost,
                           (cudaStream_t)stream));
  CUDA_TRY(cudaEventRecord(s->status_ev, (cudaStream_t)stream));
  {
    cudaError_t e;
    while ((e = cudaEventQuery(s->status_ev)) == cudaErrorNotReady) std::this_thread::yield();
    if (e != cudaSuccess) return fail(SPGO_ERR_CUDA, std::string("status wait: ") + cudaGetErrorString(e));
  }
  for (int b = 0; out && b < s->plan->B; ++b) {
    out[b].cost0 = h[b].cost0;
    out[b].cost = h[b].cost;
    out[b].lambda = h[b].lam;
    out[b].iterations = h[b].iters;
    out[b].accepted = h[b].accepted;
    out[b].status = h[b].status;
    out[b].factor_failures = h[b].factor_failures;
    out[b].wait_timeouts = h[b].wait_timeouts;
  }
  return SPGO_OK;
}

int spgo_lm_trace(spgo_solver *s, int32_t capacity, double *cost, double *lambda, int32_t *accepted,
                  int32_t *n_iters, void *stream) {
  if (!s || capacity < 0) return fail(SPGO_ERR_INVALID_ARG, "bad argument");
  const int B = s->plan->B;
  std::vector<double> h((size_t)B * SPGO_TRACE_MAX * 3);
  CUDA_TRY(cudaMemcpyAsync(h.data(), s->wv.trace, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                           (cudaStream_t)stream));
  int rc = spgo_lm_status(s, nullptr, stream);  // (synchronises; fills the status cache)
  if (rc != SPGO_OK) return rc;
  const LMState *st = reinterpret_cast<const LMState *>(s->h_lm.ptr);
  for (int b = 0; b < B; ++b) {
    const int n = std::min(std::min((int)st[b].iters, (int)SPGO_TRACE_MAX), capacity);
    if (n_iters) n_iters[b] = n;
    for (int k = 0; k < n; ++k) {
      const double *t = &h[((size_t)b * SPGO_TRACE_MAX + k) * 3];
      if (cost) cost[(size_t)b * capacity + k] = t[0];
      if (lambda) lambda[(size_t)b * capacity + k] = t[1];
      if (accepted) accepted[(size_t)b * capacity + k] = t[2] != 0.0 ? 1 : 0;
    }
  }
  return SPGO_OK;
}

int spgo_lm_solve(spgo_solver *s, int32_t check_every, int32_t *iters_done, void *stream) {
  if (!s) return fail(SPGO_ERR_INVALID_ARG, "null solver");
  if (check_every < 1) check_every = 1;
  int rc = spgo_lm_reset(s, stream);
  if (rc != SPGO_OK) return rc;
  std::vector<spgo_problem_status> stv(s->plan->B);
  int done = 0;
  while (done < s->prm.max_iters) {
    const int n = std::min(check_every, s->prm.max_iters - done);
    if ((rc = spgo_lm_iterate(s, n, stream)) != SPGO_OK) return rc;
    done += n;
    if ((rc = spgo_lm_status(s, stv.data(), stream)) != SPGO_OK) return rc;
    bool running = false;
    for (const auto &x : stv) running |= (x.status == SPGO_STATUS_RUNNING);
    if (!running) break;
  }
  if (iters_done) {
    int mx = 0;
    for (const auto &x : stv) mx = std::max(mx, (int)x.iterations);
    *iters_done = mx;
  }
  return SPGO_OK;
}

int spgo_autotune(spgo_solver *s, spgo_params *chosen, void *stream) {
  if (!s) return fail(SPGO_ERR_INVALID_ARG, "null solver");
  cudaStream_t st = (cudaStream_t)stream;
  const spgo_plan *p = s->plan;
  const bool f64 = p->precision == SPGO_PREC_FP64;
  const size_t np = (size_t)p->NP * 12, nl = (size_t)p->L;
  double *save = nullptr;
  CUDA_TRY(cudaMalloc(&save, sizeof(double) * (np + nl + 1)));
  cudaError_t ce = cudaMemcpyAsync(save, s->poses, sizeof(double) * np, cudaMemcpyDeviceToDevice, st);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(save + np, s->alpha, sizeof(double) * nl, cudaMemcpyDeviceToDevice, st);
  if (ce != cudaSuccess) {
    cudaFree(save);
    return fail(SPGO_ERR_CUDA, std::string("autotune: state copy: ") + cudaGetErrorString(ce));
  }
  const Params base = s->prm;
  struct Cand {
    int cost_block, lin_block, use_tc;
  };
  // every value of each dimension appears at least once; the dimensions time different kernels
  const Cand cands[] = {{64, 256, 1}, {64, 256, 1}, {128, 128, 0}, {256, 256, 1}};
  double t_cost[257] = {}, t_lin[257] = {}, t_schur[2] = {1e30, 1e30};
  for (int k = 0; k < 257; ++k) t_cost[k] = t_lin[k] = 1e30;
  int rc = SPGO_OK;
  rc = spgo_profile_enable(s, 4096);
  for (size_t ci = 0; rc == SPGO_OK && ci < sizeof(cands) / sizeof(cands[0]); ++ci) {
    s->prm = base;
    s->prm.use_graph = 0;
    s->prm.cost_block = cands[ci].cost_block;
    s->prm.lin_block = cands[ci].lin_block;
    s->prm.use_tc = cands[ci].use_tc;
    rc = enqueue_reset(s, st, s->prm.lambda0);
    for (int it = 0; rc == SPGO_OK && it < 2; ++it)
      rc = f64 ? enqueue_lm_iteration<double>(s, st) : enqueue_lm_iteration<float>(s, st);
    double ms[K_NKINDS];
    int64_t cnt[K_NKINDS];
    if (rc == SPGO_OK) rc = spgo_profile_read(s, ms, cnt, K_NKINDS, stream);
    if (rc == SPGO_OK && ci > 0) {  // the first run warms up
      t_cost[cands[ci].cost_block] = std::min(t_cost[cands[ci].cost_block], ms[K_COST]);
      t_lin[cands[ci].lin_block] = std::min(t_lin[cands[ci].lin_block], ms[K_LINEARIZE]);
      t_schur[cands[ci].use_tc] = std::min(t_schur[cands[ci].use_tc], ms[K_SCHUR]);
    }
    cudaMemcpyAsync(s->poses, save, sizeof(double) * np, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(s->alpha, save + np, sizeof(double) * nl, cudaMemcpyDeviceToDevice, st);
  }
  s->prm = base;
  if (rc == SPGO_OK) {
    int best_c = 64, best_l = 256;
    for (const int c : {64, 128, 256})
      if (t_cost[c] < t_cost[best_c]) best_c = c;
    for (const int l : {128, 256})
      if (t_lin[l] < t_lin[best_l]) best_l = l;
    s->prm.cost_block = best_c;
    s->prm.lin_block = best_l;
    if (!f64) s->prm.use_tc = t_schur[1] <= t_schur[0] ? 1 : 0;
  }
  spgo_profile_enable(s, 0);
  drop_graphs(s);
  cudaStreamSynchronize(st);
  cudaFree(save);
  if (rc == SPGO_OK) rc = enqueue_reset(s, st, s->prm.lambda0);
  if (rc == SPGO_OK && chosen) std::memcpy(chosen, &s->prm, sizeof(Params));
  return rc;
}

int spgo_export_system(spgo_solver *s, int32_t problem, double *A, double *g, double *B, double *C, double *g_a,
                       double *cost, void *stream) {
  if (!s || problem < 0 || problem >= s->plan->B) return fail(SPGO_ERR_INVALID_ARG, "bad problem index");
  cudaStream_t st = (cudaStream_t)stream;
  const spgo_plan *p = s->plan;
  // linearise every problem at its current state (lambda untouched: reset sets lambda0)
  int rc = enqueue_reset(s, st, s->prm.lambda0);
  if (rc != SPGO_OK) return rc;
  rc = p->precision == SPGO_PREC_FP64 ? enqueue_linearize<double>(s, st, false, false) : enqueue_linearize<float>(s, st, false, false);
  if (rc != SPGO_OK) return rc;
  const int N = p->p_npose[problem], P = 6 * N, L = p->p_lm_cnt[problem];
  const bool f64 = p->precision == SPGO_PREC_FP64;
  const size_t ts = f64 ? 8 : 4;
  if (A)
    CUDA_TRY(launch_to_double(static_cast<unsigned char *>(s->wv.A) + p->p_S_off[problem] * ts, f64, A,
                              (int64_t)P * P, st));
  if (g)
    CUDA_TRY(launch_to_double(static_cast<unsigned char *>(s->wv.g) + (size_t)p->p_param_off[problem] * ts, f64, g,
                              P, st));
  if (B) CUDA_TRY(cudaMemsetAsync(B, 0, (size_t)P * L * 8, st));
  rc = f64 ? launch_export_B_n<double>(s->pv, s->wv, problem, p->p_chunk_cnt[problem], B, C, g_a, st)
           : launch_export_B_n<float>(s->pv, s->wv, problem, p->p_chunk_cnt[problem], B, C, g_a, st);
  CUDA_TRY(rc);
  if (cost)
    CUDA_TRY(cudaMemcpyAsync(cost, &s->wv.lm[problem].cost, sizeof(double), cudaMemcpyDeviceToDevice, st));
  return SPGO_OK;
}

int spgo_export_reduced(spgo_solver *s, int32_t problem, double lambda, double *S, double *gS, void *stream) {
  if (!s || problem < 0 || problem >= s->plan->B || !S || !gS) return fail(SPGO_ERR_INVALID_ARG, "bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  const spgo_plan *p = s->plan;
  const bool f64 = p->precision == SPGO_PREC_FP64;
  int rc = enqueue_reset(s, st, lambda);
  if (rc != SPGO_OK) return rc;
  rc = f64 ? enqueue_linearize<double>(s, st, false, false) : enqueue_linearize<float>(s, st, false, false);
  if (rc != SPGO_OK) return rc;
  if (!f64 && s->prm.use_tc) {
    CUDA_TRY(launch_schur_tc(s->pv, s->wv, s->prm, st));
  } else {
    CUDA_TRY(f64 ? launch_schur<double>(s->pv, s->wv, s->prm, st) : launch_schur<float>(s->pv, s->wv, s->prm, st));
  }
  CUDA_TRY(f64 ? launch_export_S<double>(s->pv, s->wv, problem, S, gS, st)
               : launch_export_S<float>(s->pv, s->wv, problem, S, gS, st));
  return SPGO_OK;
}

int spgo_lm_set_controller(spgo_solver *s, const float *d_params, void *stream) {
  if (!s) return fail(SPGO_ERR_INVALID_ARG, "null solver");
  if (!d_params) {
    s->controller = false;
  } else {
    CUDA_TRY(launch_mlp_deploy(d_params, s->wv.ctrl, stream));
    s->controller = true;
  }
  drop_graphs(s);
  return SPGO_OK;
}

int spgo_lm_features(spgo_solver *s, float *d_feat, void *stream) {
  if (!s || !d_feat) return fail(SPGO_ERR_INVALID_ARG, "null argument");
  CUDA_TRY(launch_features(s->pv, s->wv, d_feat, stream));
  return SPGO_OK;
}

int spgo_lm_probe(spgo_solver *s, int32_t n_factors, const double *factors, double *costs, void *stream) {
  if (!s || !factors || !costs || n_factors < 1 || n_factors > 32) return fail(SPGO_ERR_INVALID_ARG, "bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = s->plan->precision == SPGO_PREC_FP64 ? enqueue_probe<double>(s, n_factors, factors, st)
                                                : enqueue_probe<float>(s, n_factors, factors, st);
  if (rc != SPGO_OK) return rc;
  CUDA_TRY(cudaMemcpyAsync(costs, s->wv.probe_costs, sizeof(double) * n_factors * s->plan->B, cudaMemcpyDeviceToHost,
                           st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return SPGO_OK;
}

int64_t spgo_launch_count(const spgo_solver *s) { return s ? g_launches - s->launches0 : 0; }

}  // extern "C"
