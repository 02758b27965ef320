// Device helpers shared by the 4-state (kernels.cu) and 20-state
// (kernels20.cu) sweeps: vector loads, scaling rules, lane reductions.
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

namespace netlk {
namespace {

constexpr unsigned kFull = 0xffffffffu;

template <typename real>
struct Vec;

template <>
struct Vec<float> {
  static __device__ __forceinline__ void load(const float *p, float (&v)[4]) {
    float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  }
  static __device__ __forceinline__ void store(float *p, const float (&v)[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
  static __device__ __forceinline__ void ldg(const float *p, float (&v)[4]) {
    float4 t = __ldg(reinterpret_cast<const float4 *>(p));
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  }
};

template <>
struct Vec<double> {
  static __device__ __forceinline__ void load(const double *p, double (&v)[4]) {
    double2 a = reinterpret_cast<const double2 *>(p)[0];
    double2 b = reinterpret_cast<const double2 *>(p)[1];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
  static __device__ __forceinline__ void store(double *p, const double (&v)[4]) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
  }
  static __device__ __forceinline__ void ldg(const double *p, double (&v)[4]) {
    double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
};

// Scaling rules. FP64 restates libpll's per-site rule: when every entry of a
// site is below 2^-256 multiply the site by 2^256 and add one to its counter.
// FP32 uses its own power-of-two unit: when the site maximum falls below
// 2^-32, shift the site by 2^-e (max becomes [0.5, 1)) and add -e.
template <typename real>
struct Scale;

template <>
struct Scale<float> {
  static constexpr double kLogUnit = -0.69314718055994530942;  // log(2^-1)
  static __device__ __forceinline__ int rescale(float m, float (&v)[4]) {
    if (m < 0x1p-32f && m > 0.0f) {
      int e;
      frexpf(m, &e);
      const int k = -e;
#pragma unroll
      for (int i = 0; i < 4; ++i) v[i] = ldexpf(v[i], k);
      return k;
    }
    return 0;
  }
  // x * 2^k for the local shift k >= 0 of a site (applied to adjoint products)
  static __device__ __forceinline__ float shift(float x, int k) { return ldexpf(x, k); }
};

template <>
struct Scale<double> {
  static constexpr double kLogUnit = -177.44567822334599921;  // log(2^-256)
  static __device__ __forceinline__ int rescale(double m, double (&v)[4]) {
    if (m < 0x1p-256) {
#pragma unroll
      for (int i = 0; i < 4; ++i) v[i] *= 0x1p256;
      return 1;
    }
    return 0;
  }
  static __device__ __forceinline__ double shift(double x, int k) { return ldexp(x, 256 * k); }
};

__device__ __forceinline__ FwdOp load_fwd_op(const FwdOp *ops, int i) {
  const int4 *q = reinterpret_cast<const int4 *>(ops + i);
  const int4 a = __ldg(q), b = __ldg(q + 1);
  FwdOp o;
  o.out = a.x; o.a = a.y; o.b = a.z; o.ea = a.w;
  o.eb = b.x; o.slot = b.y; o.pad0 = b.z; o.pad1 = b.w;
  return o;
}

__device__ __forceinline__ BwdOp load_bwd_op(const BwdOp *ops, int i) {
  const int4 *q = reinterpret_cast<const int4 *>(ops + i);
  const int4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
  BwdOp o;
  o.x = a.x; o.a = a.y; o.b = a.z; o.ea = a.w;
  o.eb = b.x; o.seed = b.y; o.out_a = b.z; o.out_b = b.w;
  o.msg_begin = c.x; o.msg_count = c.y; o.pad0 = o.pad1 = o.pad2 = o.pad3 = o.pad4 = o.pad5 = 0;
  return o;
}

template <int R, typename T>
__device__ __forceinline__ T rate_sum(T v) {
#pragma unroll
  for (int o = 1; o < R; o <<= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

template <int R, typename T>
__device__ __forceinline__ T rate_max(T v) {
#pragma unroll
  for (int o = 1; o < R; o <<= 1) v = max(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

}  // namespace
}  // namespace netlk
