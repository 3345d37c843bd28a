// bh_device.cuh -- Barnes-Hut arithmetic shared by the whole-device pipeline
// (barnes_hut.cu) and the one-block-per-graph path (batched.cu), so that both
// produce the same bits for the same graph.
//
// Reference: sample/MortonCode.h:42-97 (frame, quantisation, order),
// sample/BarnesHut.h:69-86 (opening test, unit-vector repulsion),
// :197-217 (centroids), sample/algorithms.cpp:1050-1066 (attraction, update).
#pragma once

#include <climits>

#include "bl_device.cuh"

namespace bl {

typedef unsigned long long u64;

// order-preserving map of a float onto uint32 (for integer min/max)
__device__ __forceinline__ unsigned int f2ord(float f) {
  const unsigned int u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned int u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ u64 spread32(unsigned int v) {
  u64 x = v;
  x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
  x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
  x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  return x;
}

// float -> double without the conversion instruction (exact; the bits are
// rebiased and shifted): normal floats and +-0; subnormal, infinite and NaN
// floats take the conversion.
__device__ __forceinline__ double f2d_int(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  if (e == 0u) {
    if (u & 0x7fffffu) return (double)f;
    return __longlong_as_double((long long)sign);
  }
  if (e == 0xffu) return (double)f;
  return __longlong_as_double(
      (long long)(sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// double -> float rounded to nearest even, with integer operations for the
// normal range of float (the conversion instruction runs on the FP64 pipe);
// anything else takes the conversion.
__device__ __forceinline__ float d2f_int(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ffu) - 1023 + 127;  // float exponent field
  if (e < 1 || e > 253) return __double2float_rn(x);    // zero, subnormal, near overflow, inf, NaN
  const unsigned int sign = (unsigned int)(b >> 63) << 31;
  const unsigned long long man = b & ((1ull << 52) - 1ull);
  unsigned int m = (unsigned int)(man >> 29);             // 23 bits
  const unsigned long long rest = man & ((1ull << 29) - 1ull);
  const unsigned long long half = 1ull << 28;
  unsigned int bits = sign | ((unsigned int)e << 23) | m;
  if (rest > half || (rest == half && (m & 1u))) bits += 1u;  // a carry moves into the exponent correctly
  return __uint_as_float(bits);
}

// 0.0 + x exactly: x, except that -0 becomes +0.
__device__ __forceinline__ double zero_plus(double x) {
  return (__double_as_longlong(x) == (long long)0x8000000000000000ll) ? 0.0 : x;
}

// Frame (MortonCode.h:42-52) from the ordered-uint bbox {min x, max x, min y,
// max y}; FP64 like the reference.
__device__ __forceinline__ void frame_from_bbox(const unsigned int *bbox, double &minX, double &minY,
                                                double &maxmin) {
  minX = (double)ord2f(bbox[0]);
  const double maxX = (double)ord2f(bbox[1]);
  minY = (double)ord2f(bbox[2]);
  const double maxY = (double)ord2f(bbox[3]);
  const double ry = __dsub_rn(maxY, minY), rx = __dsub_rn(maxX, minX);
  maxmin = (ry < rx) ? rx : ry;  // std::max(y-range, x-range)
}

// (uint32)(4294967295.0 * (v - mn) / maxmin), MortonCode.h:62-67, no contraction.
// The quotient is formed with the reciprocal (one multiply); its error is a
// couple of ulp, so unless it lies within 8 ulp of an integer its truncation
// equals the truncation of the correctly rounded quotient.  Otherwise the
// exact division decides.  The truncation and the distance to the nearest
// integers are read from the bits of the quotient with integer operations:
// the FP64 pipe (a small fraction of the FP32 rate on this part) only sees
// the subtraction and the two products.
__device__ __forceinline__ unsigned int quantise(float v, double mn, double maxmin, double inv) {
  if (!(maxmin > 0.0)) return 0u;
  const double a = __dmul_rn(4294967295.0, __dsub_rn(f2d_int(v), mn));
  const double qf = __dmul_rn(a, inv);
  const unsigned long long b = (unsigned long long)__double_as_longlong(qf);
  const int e = (int)((b >> 52) & 0x7ffu) - 1023;  // qf in [2^e, 2^(e+1)) when positive
  if ((b >> 63) == 0ull && e >= 0 && e < 32) {
    const unsigned long long m = (b & ((1ull << 52) - 1ull)) | (1ull << 52);
    const int sh = 52 - e;  // fraction bits, 21..52
    const unsigned long long frac = m & ((1ull << sh) - 1ull);
    if (frac > 8ull && (1ull << sh) - frac > 8ull) return (unsigned int)(m >> sh);
  }
  return __double2uint_rz(__ddiv_rn(a, maxmin));  // near an integer, below 1 or out of range
}

// 64-bit Morton key, y bit above x bit of every digit (MortonCode.h:83-97).
__device__ __forceinline__ u64 morton_key(float2 p, double minX, double minY, double maxmin, double inv) {
  return (spread32(quantise(p.y, minY, maxmin, inv)) << 1) | spread32(quantise(p.x, minX, maxmin, inv));
}

// x / c for the child count c of a quad node, correctly rounded like the
// reference's `c_x /= count` (BarnesHut.h:214-216) but without a division:
// c = 2 and 4 scale exactly; for c = 3 the product with RN(1/3) is corrected
// once with its exact FMA residual (Markstein, "IA-64 and Elementary
// Functions", 2000), which is correctly rounded because x/3 is never a tie.
__device__ __forceinline__ double div_count(double x, int c) {
  if (c == 1) return x;
  if (c == 2) return __dmul_rn(x, 0.5);
  if (c == 4) return __dmul_rn(x, 0.25);
  if (c == 3) {
    const double r3 = 0.33333333333333331;  // RN(1/3)
    const double q0 = __dmul_rn(x, r3);
    const double r = __fma_rn(-3.0, q0, x);
    return __fma_rn(r, r3, q0);
  }
  return __ddiv_rn(x, (double)c);
}

// The same quotient with integer operations where they are exact, so that the
// FP64 pipe (a small fraction of the FP32 rate on this part) only sees the
// division by 3 and the run lengths: x/2 and x/4 lower the exponent of a
// normal x (and leave +-0 alone); anything else takes div_count.
__device__ __forceinline__ double div_count_int(double x, int c) {
  if (c == 2 || c == 4) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned int e = (unsigned int)(b >> 52) & 0x7ffu;
    const unsigned int k = c == 2 ? 1u : 2u;
    if ((b << 1) == 0ull) return x;  // +-0
    if (e > k && e < 0x7ffu) return __longlong_as_double((long long)(b - ((unsigned long long)k << 52)));
  }
  return div_count(x, c);
}

// Loads of the tree records and positions: through the read-only data cache
// (kRO) when the launch does not write them, plain loads otherwise (the
// one-block path rewrites them every iteration, ordered by block barriers).
template <bool kRO, typename T>
__device__ __forceinline__ T ldx(const T *p) {
  if constexpr (kRO) return __ldg(p);
  else return *p;
}

// FP64 opening test exactly as BarnesHut.h:71-72: diameter / distance < theta.
template <bool kRO>
static __device__ __noinline__ bool open_test_fp64(const double2 *c64, const unsigned char *lvl, double maxmin,
                                                   double theta, int idx, float qx, float qy) {
  const double2 c = ldx<kRO>(&c64[idx]);
  const double D = ldexp(maxmin, -(int)ldx<kRO>(&lvl[idx]));
  const double dx = __dsub_rn(c.x, (double)qx), dy = __dsub_rn(c.y, (double)qy);
  const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
  return __ddiv_rn(D, dist) < theta;
}

// Pre-order record {x, y, z, skip} of the walk: a quad node's FP32 centroid,
// z = D^2 / theta^2 rounded to FP32 (D its diameter, BarnesHut.h:128,157, the
// threshold of the opening test folded in), and the record after its
// subtree; a leaf point's coordinates, z = -inf (always added) and the next
// record.
constexpr float kLeafZ = -__builtin_huge_valf();

__device__ __forceinline__ float bh_record_z(double D, double inv_theta2) {
  return d2f_int(__dmul_rn(__dmul_rn(D, D), inv_theta2));
}

// Error bound of the FP32 opening test m = d^2 - z > 0 (the reference's
// D / dist < theta is dist^2 > D^2 / theta^2): 2^-18 d^2 for the roundings of
// the centroid, of z and of the products (a wide margin over a few ulp; when
// z > 3 d^2 the margin |m| > 2 d^2 is never in doubt), plus
// 2^-21 s (2 (|qx| + |qy|) + s), s = |dx| + |dy|, for the rounding of the
// coordinates and of their differences (with 0.2 % to spare).
constexpr float kTolRel = 3.8146973e-06f;        // 2^-18
constexpr float kTolA = 4.7683716e-07f * 1.002f;  // 2^-21
__device__ __forceinline__ float bh_tol_q(float2 q) { return kTolA * 2.f * (fabsf(q.x) + fabsf(q.y)); }

// One record of the walk: the opening test on record i, the accepted
// record's unit vector added to (fx, fy), and the next record.  The FP32 test
// decides unless its margin is within the error bound; then the FP64 test
// (the reference's own arithmetic) decides.
template <bool kRO, bool kStats>
__device__ __forceinline__ void bh_walk_step(const float4 *nodes, const double2 *c64, const unsigned char *lvl,
                                             double maxmin, double theta, float tq, float2 q, int &i, float &fx,
                                             float &fy, unsigned int &visits, unsigned int &exact) {
  const float4 nd = ldx<kRO>(&nodes[i]);
  const float dx = nd.x - q.x, dy = nd.y - q.y;
  const float d2 = fmaf(dx, dx, fmaf(dy, dy, kTinyD2));
  const float m = d2 - nd.z;  // +inf for a leaf
  bool accept = m > 0.f;
  const float sd = fabsf(dx) + fabsf(dy);
  const float tol = fmaf(sd, fmaf(kTolA, sd, tq), kTolRel * d2);
  if (fabsf(m) <= tol) {
    accept = open_test_fp64<kRO>(c64, lvl, maxmin, theta, i, q.x, q.y);
    if (kStats) exact++;
  }
  if (kStats) visits++;
  const float r = rsqrt_approx(d2);
  if (accept) {
    fx = fmaf(dx, r, fx);
    fy = fmaf(dy, r, fy);
  }
  i = accept ? max(__float_as_int(nd.w), i + 1) : i + 1;
}

// Stackless walk of the pre-order records (record 0 is the root, its skip
// link is the number of records): repulsion on q (BarnesHut.h:69-86).  Every
// decision equals the reference's FP64 decision (see bh_walk_step).  A leaf
// at q itself adds nothing (its vector is zero).  The step to the next
// record is max(skip, i + 1) on acceptance, so the walk ends after at most
// `total` records whatever the records hold (the layout checks every skip
// link).  kStats counts record visits and FP64 decisions.
template <bool kRO, bool kStats = false>
__device__ __forceinline__ float2 bh_repulsion(const float4 *nodes, const double2 *c64, const unsigned char *lvl,
                                               double maxmin, double theta, int total, float2 q,
                                               unsigned int &visits, unsigned int &exact) {
  const float tq = bh_tol_q(q);
  float fx = 0.f, fy = 0.f;
  int i = 0;
  while (i < total) bh_walk_step<kRO, kStats>(nodes, c64, lvl, maxmin, theta, tq, q, i, fx, fy, visits, exact);
  return make_float2(fx, fy);
}

// FR attraction of one neighbour (algorithms.cpp:1056-1058) added to the
// float-float sum (hx, lx), (hy, ly).
__device__ __forceinline__ void bh_attract(float2 pj, float2 pv, float W, float &hx, float &lx, float &hy,
                                           float &ly) {
  const float dx = pj.x - pv.x, dy = pj.y - pv.y;
  const float sc = W * sqrtf(fmaf(dx, dx, dy * dy));
  ff_add(hx, lx, dx * sc);
  ff_add(hy, ly, dy * sc);
}

// The attraction of the neighbours j of v that are not moved before v in
// this iteration (j at or after v's batch start), read at their
// iteration-start positions; CSR order, float-float {hx, hy, lx, ly}.
__device__ __forceinline__ float4 bh_unmoved_attraction(int v, const int *__restrict__ rowptr,
                                                        const int *__restrict__ colids, const float2 *pold, int batch,
                                                        float W) {
  const float2 pv = pold[v];
  const int batch_lo = (v / batch) * batch;
  float hx = 0.f, lx = 0.f, hy = 0.f, ly = 0.f;
  const int e1 = rowptr[v + 1];
  constexpr int kU = 4;  // index loads first, then position loads, then the ordered sum
  for (int e = rowptr[v]; e < e1; e += kU) {
    int j[kU];
    float2 pj[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) j[u] = (e + u < e1) ? colids[e + u] : -1;
#pragma unroll
    for (int u = 0; u < kU; u++)
      if (j[u] >= batch_lo) pj[u] = pold[j[u]];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      if (j[u] < batch_lo) continue;  // moved earlier in this iteration, or past the row end
      bh_attract(pj[u], pv, W, hx, lx, hy, ly);
    }
  }
  return make_float4(hx, hy, lx, ly);
}

// f (float-float {hx, hy, lx, ly}) minus the repulsion: the sum the level
// sweep starts from.
__device__ __forceinline__ float4 bh_minus_repulsion(float4 f, float2 rep) {
  ff_add(f.x, f.z, -rep.x);
  ff_add(f.y, f.w, -rep.y);
  return f;
}

// Unit-step update (algorithms.cpp:1062-1066) from the float-float force:
// FP32 unit vector, FP64 only when |f|^2 leaves the FP32 range; |f| = 0
// leaves the point where it is.
__device__ __forceinline__ float2 bh_step(float2 pi, float hx, float lx, float hy, float ly, float step) {
  const float fxf = hx + lx, fyf = hy + ly;
  float2 np = pi;
  const float m2 = fmaf(fxf, fxf, fyf * fyf);
  if (m2 >= 1.17549435e-38f && m2 <= 3.0e38f) {
    const float rm = rsqrt_approx(m2);
    np.x = fmaf(step, fxf * rm, pi.x);
    np.y = fmaf(step, fyf * rm, pi.y);
  } else if (fxf != 0.f || fyf != 0.f) {
    const double fx = (double)hx + (double)lx, fy = (double)hy + (double)ly;
    const double mag = sqrt(fx * fx + fy * fy);
    np.x = (float)((double)pi.x + (fx / mag) * (double)step);
    np.y = (float)((double)pi.y + (fy / mag) * (double)step);
  }
  return np;
}

}  // namespace bl
