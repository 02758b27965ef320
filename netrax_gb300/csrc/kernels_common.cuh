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

// FULL: also the inline message slots msg1, msg2 and pad4 (the walk
// schedule's fields); otherwise they read as -1 / 0.
template <bool FULL = false>
__device__ __forceinline__ BwdOp load_bwd_op(const BwdOp *ops, int i) {
  const int4 *q = reinterpret_cast<const int4 *>(ops + i);
  const int4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
  const int4 d = FULL ? __ldg(q + 3) : make_int4(-1, -1, 0, 0);
  BwdOp o;
  o.x = a.x; o.a = a.y; o.b = a.z; o.ea = a.w;
  o.eb = b.x; o.seed = b.y; o.out_a = b.z; o.out_b = b.w;
  o.msg_begin = c.x; o.msg_count = c.y; o.pad0 = c.z; o.msg0 = c.w; o.msg1 = d.x; o.msg2 = d.y;
  o.pad4 = d.z; o.pad5 = d.w;
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

// ------------------------------------------------- float-float arithmetic
// A value is the unevaluated sum hi + lo of two floats (about 48 significant
// bits). Error-free transforms: TwoSum (Knuth, TAOCP vol. 2, 4.2.2) and the
// FMA product error (a*b - fl(a*b) is exact in one fma). The FP32 sweeps use
// it for their per-site log-likelihood sums, so they issue no FP64
// instruction: GB300 runs FP64 at a small fraction of its FP32 rate.
struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return FF{s, (a - (s - bb)) + (b - bb)};
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ FF quick_two_sum(float a, float b) {
  const float s = a + b;
  return FF{s, b - (s - a)};
}

__device__ __forceinline__ FF ff_add(FF x, FF y) {
  const FF s = two_sum(x.hi, y.hi);
  return quick_two_sum(s.hi, s.lo + (x.lo + y.lo));
}

__device__ __forceinline__ FF ff_mul(FF x, FF y) {
  const float p = x.hi * y.hi;
  const float e = __fmaf_rn(x.hi, y.hi, -p);
  return quick_two_sum(p, e + (x.hi * y.lo + x.lo * y.hi));
}

__device__ __forceinline__ FF warp_sum_ff(FF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const FF t{__shfl_xor_sync(kFull, v.hi, o), __shfl_xor_sync(kFull, v.lo, o)};
    v = ff_add(v, t);
  }
  return v;
}

// The double a float pair stands for (hi + lo rounded once).
__host__ __device__ __forceinline__ double ff_to_double(float2 v) { return (double)v.x + (double)v.y; }

// Sum over a warp's sites of w_s (log t_s + k_s log unit): the root
// log-likelihood of pll_compute_root_loglikelihood for the sites a warp
// covers. add() is called by the lane that owns a site; store() by the whole
// warp, lane 0 writing the 8-byte result: a double in FP64 sweeps, a float
// pair in FP32 ones. A zero-weight site (padding) adds nothing; a site whose
// likelihood is 0 makes the sum -inf, as in double arithmetic.
template <typename real>
struct SiteSum;

template <>
struct SiteSum<double> {
  double ll = 0.0;
  __device__ __forceinline__ void add(const SweepParams &p, size_t g, double t, int k) {
    const double w = p.weights[g];
    if (w != 0.0) ll += w * (log(t) + (double)k * Scale<double>::kLogUnit);
  }
  // with invariant sites: w log(gf (t 2^(-256 k) + iq))
  __device__ __forceinline__ void add_inv(const SweepParams &p, int part, size_t g, double t, int k) {
    const double w = p.weights[g];
    if (w == 0.0) return;
    double a = log(t) + (double)k * Scale<double>::kLogUnit;
    const double iq = p.inv_term[g];
    if (iq > 0.0) {
      const double b = log(iq);
      a = a > b ? a + log1p(exp(b - a)) : b + log1p(exp(a - b));
    }
    ll += w * (a + log(p.gamma_frac[part]));
  }
  __device__ __forceinline__ void store(double *dst, int lane) {
    ll = warp_sum(ll);
    if (lane == 0) *dst = ll;
  }
};

template <>
struct SiteSum<float> {
  static constexpr float kUnitHi = (float)Scale<float>::kLogUnit;
  static constexpr float kUnitLo = (float)(Scale<float>::kLogUnit - (double)kUnitHi);
  FF ll{0.f, 0.f};
  float bad = 0.f;  // sum of the non-finite terms (-inf or NaN), kept apart
  __device__ __forceinline__ void add(const SweepParams &p, size_t g, float t, int k) { add_w(p.weights32[g], t, k); }
  __device__ __forceinline__ void add_w(float2 w, float t, int k) {
    if (w.x == 0.f) return;
    const float lt = logf(t);
    if (!isfinite(lt)) {
      bad += w.x * lt;
      return;
    }
    const float kf = (float)k;  // exact: |k| < 2^24
    const float ph = kf * kUnitHi;
    const FF ku = quick_two_sum(ph, __fmaf_rn(kf, kUnitHi, -ph) + kf * kUnitLo);
    const FF y = ff_add(ku, FF{lt, 0.f});
    ll = ff_add(ll, ff_mul(FF{w.x, w.y}, y));
  }
  // with invariant sites: w log(gf (t 2^(-k) + iq)), gf and iq given
  __device__ __forceinline__ void add_inv_w(float2 w, float t, int k, float gf, float iq) {
    if (w.x == 0.f) return;
    const float lt = logf(t);
    const float lg = logf(gf);
    FF y;
    if (!(iq > 0.f)) {
      add_w(w, t, k);
      if (isfinite(lt)) ll = ff_add(ll, ff_mul(FF{w.x, w.y}, FF{lg, 0.f}));
      return;
    }
    const float b = logf(iq);
    if (!isfinite(lt)) {
      y = FF{b, 0.f};
    } else {
      const float kf = (float)k;
      const float ph = kf * kUnitHi;
      const FF a = ff_add(quick_two_sum(ph, __fmaf_rn(kf, kUnitHi, -ph) + kf * kUnitLo), FF{lt, 0.f});
      const float d = b - a.hi;
      y = d > 0.f ? ff_add(FF{b, 0.f}, FF{log1pf(expf(-d)), 0.f}) : ff_add(a, FF{log1pf(expf(d)), 0.f});
    }
    ll = ff_add(ll, ff_mul(FF{w.x, w.y}, ff_add(y, FF{lg, 0.f})));
  }
  __device__ __forceinline__ void add_inv(const SweepParams &p, int part, size_t g, float t, int k) {
    add_inv_w(p.weights32[g], t, k, p.gamma_frac32[part], p.inv_term32[g]);
  }
  __device__ __forceinline__ void store(double *dst, int lane) {
    ll = warp_sum_ff(ll);
    bad = warp_sum(bad);
    if (lane == 0) *reinterpret_cast<float2 *>(dst) = bad != 0.f ? make_float2(bad, 0.f) : make_float2(ll.hi, ll.lo);
  }
};

// A model value as the sweep's arithmetic type: the float copy in FP32
// sweeps, the double itself in FP64 ones.
template <typename real>
__device__ __forceinline__ real model_val(const double *d, const float *f, size_t i) {
  if constexpr (sizeof(real) == 4) return f[i];
  else return d[i];
}

// With invariant sites, the invariant term of site g in the scaled units of
// a root CLV with scale counter k (0 without +I): the adjoint seed of a
// displayed-tree root is w rw pi / (t + root_inv_term), t its rate mixture.
template <typename real>
__device__ __forceinline__ real root_inv_term(const SweepParams &p, size_t g, int k) {
  real iq;
  if constexpr (sizeof(real) == 4) iq = p.inv_term32[g];
  else iq = p.inv_term[g];
  return iq > (real)0 ? Scale<real>::shift(iq, k) : (real)0;
}

// A pattern's weight as the sweep's arithmetic type.
template <typename real>
__device__ __forceinline__ real pattern_weight(const SweepParams &p, size_t g) {
  if constexpr (sizeof(real) == 4) return p.weights32[g].x;
  else return p.weights[g];
}

// Writes one (a, b) pair of edge terms: two doubles, or two float pairs
// (value, 0) in FP32 sweeps.
template <typename real>
__device__ __forceinline__ void store_edge_terms(double *dst, real a, real b) {
  if constexpr (sizeof(real) == 4) {
    *reinterpret_cast<float4 *>(dst) = make_float4(a, 0.f, b, 0.f);
  } else {
    dst[0] = a;
    dst[1] = b;
  }
}

}  // namespace
}  // namespace netlk
