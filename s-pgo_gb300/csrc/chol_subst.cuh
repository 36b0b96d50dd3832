// Blocked forward / backward substitution with a packed Cholesky factor held in
// shared memory, shared by the batched factorisation (k_solve.cu) and the
// refinement solves of the mixed path (k_refine.cu).
//
// Storage: element (i, j), i >= j, of L at Lm[cb[j] + i] (packed lower triangle,
// column-major: cb[j] = j P - j (j + 1) / 2); dinv[k] = 1 / L(k, k).
#pragma once
#include "kernels.cuh"

namespace spgo {

constexpr int kPanel = 16;  // block width of the factorisation and the substitutions

// Solves L L^T w = y in place (y in shared memory), 16-unknown blocks: warp 0
// runs each diagonal block's chain (lane = unknown, one shuffle per unknown),
// all threads apply the block to the rows below (forward) or gather the rows
// below into the block (backward); two barriers per block.  tmp: kPanel
// elements of shared scratch.  Every thread of the CTA must call it.
template <typename T>
__device__ void chol_substitute(const T *Lm, const int *cb, T *y, const T *dinv, T *tmp, int P) {
#define ix(i, j) (cb[(j)] + (i))
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
  // forward L z = y, block by block; warp 0 solves the 16x16 diagonal block with
  // lane c owning unknown c (one shuffle per unknown)
  for (int kb = 0; kb < P; kb += kPanel) {
    const int ke = min(kb + kPanel, P), w = ke - kb;
    if (warp == 0) {
      // lane = unknown; its row of the diagonal block and the pivots are loaded
      // first, so the serial chain is multiply, shuffle, FMA per unknown
      T lr[kPanel], di[kPanel];
#pragma unroll
      for (int c = 0; c < kPanel; ++c) {
        lr[c] = (lane < w && c < lane) ? Lm[ix(kb + lane, kb + c)] : T(0);
        di[c] = c < w ? dinv[kb + c] : T(0);
      }
      T v = lane < w ? y[kb + lane] : T(0);
#pragma unroll
      for (int c = 0; c < kPanel; ++c) {
        T yc = v * di[c];
        yc = __shfl_sync(0xffffffffu, yc, c);
        if (lane == c) v = yc;
        v -= lr[c] * yc;
      }
      if (lane < w) y[kb + lane] = v;
    }
    __syncthreads();
    for (int i = ke + tid; i < P; i += nt) {
      T v = y[i];
      for (int c = 0; c < w; ++c) v -= Lm[ix(i, kb + c)] * y[kb + c];
      y[i] = v;
    }
    __syncthreads();
  }
  // backward L^T w = z, blocks from the bottom
  for (int kb = ((P - 1) / kPanel) * kPanel; kb >= 0; kb -= kPanel) {
    const int ke = min(kb + kPanel, P), w = ke - kb;
    for (int c = warp; c < w; c += nw) {
      T acc = T(0);
      for (int i = ke + lane; i < P; i += 32) acc += Lm[ix(i, kb + c)] * y[i];
      acc = warp_sum(acc);
      if (lane == 0) tmp[c] = acc;
    }
    __syncthreads();
    if (warp == 0) {
      T lc[kPanel], di[kPanel];  // column `lane` of the diagonal block, pivots
#pragma unroll
      for (int c = 0; c < kPanel; ++c) {
        lc[c] = (c < w && lane < c) ? Lm[ix(kb + c, kb + lane)] : T(0);
        di[c] = c < w ? dinv[kb + c] : T(0);
      }
      T v = lane < w ? y[kb + lane] - tmp[lane] : T(0);
#pragma unroll
      for (int c = kPanel - 1; c >= 0; --c) {
        T xc = v * di[c];
        xc = __shfl_sync(0xffffffffu, xc, c);
        if (lane == c) v = xc;
        v -= lc[c] * xc;
      }
      if (lane < w) y[kb + lane] = v;
    }
    __syncthreads();
  }
#undef ix
}

}  // namespace spgo
