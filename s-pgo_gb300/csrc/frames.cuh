// Frame-table access shared by the linearisation and the pair reduction.
//
// Per frame f and camera (0 left, 1 right) the pose chain writes the
// camera-to-world rotation (FP32 and FP64 copies) and the camera centre (FP64,
// plus a (hi, lo) float pair).  The FP32 path forms relative centres
// c_x - c_y as (hi_x - hi_y) + (lo_x - lo_y), which keeps the FP32 precision
// of the (small) difference without FP64 arithmetic per observation.
#pragma once
#include "kernels.cuh"

namespace spgo {

template <typename T> struct FramesT;
template <> struct FramesT<float> {
  __device__ static const float *R(const WorkView &wv, int f, int cam) { return wv.fr_Rf + (size_t)f * 18 + cam * 9; }
  // c(fx, camx) - c(fy, camy)
  __device__ static Vec3<float> rel(const WorkView &wv, int fx, int camx, int fy, int camy) {
    const float *xh = wv.fr_ch + (size_t)fx * 6 + camx * 3, *xl = wv.fr_cl + (size_t)fx * 6 + camx * 3;
    const float *yh = wv.fr_ch + (size_t)fy * 6 + camy * 3, *yl = wv.fr_cl + (size_t)fy * 6 + camy * 3;
    return v3<float>((xh[0] - yh[0]) + (xl[0] - yl[0]), (xh[1] - yh[1]) + (xl[1] - yl[1]),
                     (xh[2] - yh[2]) + (xl[2] - yl[2]));
  }
};
template <> struct FramesT<double> {
  __device__ static const double *R(const WorkView &wv, int f, int cam) { return wv.fr_Rd + (size_t)f * 18 + cam * 9; }
  __device__ static Vec3<double> rel(const WorkView &wv, int fx, int camx, int fy, int camy) {
    const double *x = wv.fr_c + (size_t)fx * 6 + camx * 3, *y = wv.fr_c + (size_t)fy * 6 + camy * 3;
    return v3<double>(x[0] - y[0], x[1] - y[1], x[2] - y[2]);
  }
};

}  // namespace spgo
