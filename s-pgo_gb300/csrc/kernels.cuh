// Device helpers shared by the solver kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include "spgo_internal.h"

namespace spgo {

__device__ __forceinline__ bool problem_active(const LMState *lm, int b, int gate) {
  if (gate == GATE_ALL) return true;
  const LMState &s = lm[b];
  if (s.status != 0) return false;
  if (gate == GATE_RELIN) return s.relin != 0;
  if (gate == GATE_FIRST) return s.relin != 0 && s.iters == 0;
  if (gate == GATE_REJECTED) return s.relin == 0;
  return true;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// fire-and-forget accumulation (compiles to RED for an unused return value)
__device__ __forceinline__ void red_add(float *p, float v) { atomicAdd(p, v); }
// barrier `id` (1..15) for the first n threads of the CTA (n a multiple of 32)
__device__ __forceinline__ void named_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void red_add(double *p, double v) { atomicAdd(p, v); }

template <typename T> struct Vec3 { T x, y, z; };

template <typename T>
__device__ __forceinline__ Vec3<T> v3(T x, T y, T z) { return Vec3<T>{x, y, z}; }

template <typename T>
__device__ __forceinline__ Vec3<T> cross(const Vec3<T> &a, const Vec3<T> &b) {
  return v3<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

template <typename T>
__device__ __forceinline__ T dot(const Vec3<T> &a, const Vec3<T> &b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}

// R (row-major 3x3, cam->world) applied transposed: R^T v
template <typename T>
__device__ __forceinline__ Vec3<T> mulT(const T *R, const Vec3<T> &v) {
  return v3<T>(R[0] * v.x + R[3] * v.y + R[6] * v.z, R[1] * v.x + R[4] * v.y + R[7] * v.z,
               R[2] * v.x + R[5] * v.y + R[8] * v.z);
}

template <typename T>
__device__ __forceinline__ Vec3<T> mul(const T *R, const Vec3<T> &v) {
  return v3<T>(R[0] * v.x + R[1] * v.y + R[2] * v.z, R[3] * v.x + R[4] * v.y + R[5] * v.z,
               R[6] * v.x + R[7] * v.y + R[8] * v.z);
}

// robust loss: returns w^2 = beta * rho'(s) and sets rho = beta * rho(s); s = |r|^2
template <typename T>
__device__ __forceinline__ T robust(int kind, T scale, T s, T &rho) {
  if (kind == 1) {  // Cauchy, c = scale
    T c2 = scale * scale;
    T q = s / c2;
    rho = c2 * log1p(q);
    return T(1) / (T(1) + q);
  } else if (kind == 2) {  // Huber, delta = scale
    T rs = sqrt(s);
    if (rs <= scale) {
      rho = s;
      return T(1);
    }
    rho = T(2) * scale * rs - scale * scale;
    return scale / rs;
  }
  rho = s;
  return T(1);
}

// FP64 SO(3) exponential and left Jacobian (S-PGO src/LieUtils/SO3.cu:5-32, :82-107;
// closed-form Rodrigues with Taylor branches near zero)
__device__ __forceinline__ void so3_coeffs(double th, double &a, double &b, double &c) {
  double t2 = th * th;
  if (th < 1e-4) {
    a = 1.0 - t2 / 6.0 + t2 * t2 / 120.0;
    b = 0.5 - t2 / 24.0 + t2 * t2 / 720.0;
    c = 1.0 / 6.0 - t2 / 120.0 + t2 * t2 / 5040.0;
  } else {
    double s, co;
    sincos(th, &s, &co);
    a = s / th;
    b = (1.0 - co) / t2;
    c = (th - s) / (t2 * th);
  }
}

// Exp_SE3(xi) as a 3x4 row-major matrix, xi = (psi, rho) (S-PGO src/LieUtils/SE3.cu:3-38)
__device__ __forceinline__ void exp_se3(const double *xi, double *T) {
  double px = xi[0], py = xi[1], pz = xi[2];
  double th = sqrt(px * px + py * py + pz * pz);
  double a, b, c;
  so3_coeffs(th, a, b, c);
  // S = skew(psi), S2 = S*S
  double S[9] = {0, -pz, py, pz, 0, -px, -py, px, 0};
  double S2[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      S2[3 * i + j] = S[3 * i] * S[j] + S[3 * i + 1] * S[3 + j] + S[3 * i + 2] * S[6 + j];
  double R[9], J[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    double id = (k == 0 || k == 4 || k == 8) ? 1.0 : 0.0;
    R[k] = id + a * S[k] + b * S2[k];
    J[k] = id + b * S[k] + c * S2[k];
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    T[4 * i + 0] = R[3 * i + 0];
    T[4 * i + 1] = R[3 * i + 1];
    T[4 * i + 2] = R[3 * i + 2];
    T[4 * i + 3] = J[3 * i] * xi[3] + J[3 * i + 1] * xi[4] + J[3 * i + 2] * xi[5];
  }
}

// C = A * B for 3x4 rigid transforms (implicit last row 0 0 0 1)
__device__ __forceinline__ void compose34(const double *A, const double *B, double *C) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      double v = A[4 * i] * B[j] + A[4 * i + 1] * B[4 + j] + A[4 * i + 2] * B[8 + j];
      if (j == 3) v += A[4 * i + 3];
      C[4 * i + j] = v;
    }
  }
}

__device__ __forceinline__ void invert34(const double *T, double *Ti) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Ti[4 * i + j] = T[4 * j + i];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    Ti[4 * i + 3] = -(Ti[4 * i] * T[3] + Ti[4 * i + 1] * T[7] + Ti[4 * i + 2] * T[11]);
}

inline int grid_for(long long n, int block) { return (int)((n + block - 1) / block); }

}  // namespace spgo
