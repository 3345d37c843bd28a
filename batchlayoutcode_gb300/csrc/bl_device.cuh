// bl_device.cuh -- device helpers shared by the layout kernels.
#pragma once

#include "bl_internal.cuh"

namespace bl {

// Repulsion of source s on target i (algorithms.cpp:764-768):
// f -= d / |d|^2 with d = x_s - x_i, zero for coincident points.
__device__ __forceinline__ void rep_pair(float xs, float ys, float xi, float yi, float &fx, float &fy) {
  const float dx = xs - xi, dy = ys - yi;
  const float d2 = fmaf(dx, dx, fmaf(dy, dy, kTinyD2));
  const float r = rcp_approx(d2);
  fx = fmaf(-dx, r, fx);
  fy = fmaf(-dy, r, fy);
}

// Unit-vector repulsion of source s on target i, the second phase of algo 5
// (algorithms.cpp:1117-1122): f -= d / |d|, zero for coincident points.
__device__ __forceinline__ void rep_unit_pair(float xs, float ys, float xi, float yi, float &fx, float &fy) {
  const float dx = xs - xi, dy = ys - yi;
  const float d2 = fmaf(dx, dx, fmaf(dy, dy, kTinyD2));
  const float r = rsqrt_approx(d2);
  fx = fmaf(-dx, r, fx);
  fy = fmaf(-dy, r, fy);
}

// Repulsion law of the minibatch sweep: REP_INV -d/|d|^2 (algo 2/3/7/8),
// REP_UNIT -d/|d| (algo 5, second phase).
enum RepLaw { REP_INV = 0, REP_UNIT = 1 };

template <int kRep>
__device__ __forceinline__ void rep_law_pair(float xs, float ys, float xi, float yi, float &fx, float &fy) {
  if (kRep == REP_UNIT) rep_unit_pair(xs, ys, xi, yi, fx, fy);
  else rep_pair(xs, ys, xi, yi, fx, fy);
}

// Attraction of a matched neighbour, FP32 (algorithms.cpp:759 FR, :912 LinLog, :985 FA).
__device__ __forceinline__ void attract_pair(int model, float W, float xs, float ys, float xi, float yi,
                                             float &fx, float &fy) {
  const float dx = xs - xi, dy = ys - yi;
  float sc;
  if (model == MODEL_FR) sc = W * sqrtf(fmaf(dx, dx, dy * dy));
  else if (model == MODEL_LINLOG) sc = log2f(1.0f + W * sqrtf(fmaf(dx, dx, dy * dy)));
  else sc = W;
  fx = fmaf(dx, sc, fx);
  fy = fmaf(dy, sc, fy);
}

// Compensated float-float accumulation (Knuth's TwoSum): hi + lo carries a
// sum of FP32 terms to about 48 bits without the FP64 pipe.
__device__ __forceinline__ void ff_add(float &hi, float &lo, float t) {
  const float sum = hi + t;
  const float bb = sum - hi;
  const float err = (hi - (sum - bb)) + (t - bb);
  hi = sum;
  lo += err;
}

// Unit-step update x += STEP * f/|f| (algorithms.cpp:777) in FP32; |f| = 0
// leaves x unchanged (the reference would write NaN).
__device__ __forceinline__ float2 unit_step(float2 p, double fx, double fy, float step) {
  const float fxf = (float)fx, fyf = (float)fy;
  const float m2 = fmaf(fxf, fxf, fyf * fyf);
  if (m2 >= 1.17549435e-38f && m2 <= 3.0e38f) {
    const float rm = rsqrt_approx(m2);
    p.x = fmaf(step, fxf * rm, p.x);
    p.y = fmaf(step, fyf * rm, p.y);
  } else if (fx != 0.0 || fy != 0.0) {  // |f|^2 outside the FP32 range
    const double mag = sqrt(fx * fx + fy * fy);
    p.x = (float)((double)p.x + (fx / mag) * (double)step);
    p.y = (float)((double)p.y + (fy / mag) * (double)step);
  }
  return p;
}

}  // namespace bl
