// 20-state (protein) sweeps.
//
// Same schedule, layout and arithmetic as the 4-state sweeps of kernels.cu
// with S = 20: CLV of a variant is clv[v][pattern][rate][20], tips are 20-bit
// state masks (uint32), P-matrices are 20x20 per rate. A lane owns one
// (pattern, rate) pair and keeps its 20-vectors in registers; a warp covers
// 32/R patterns per pass and walks its unit in passes. The op's two
// P-matrices (all rates; and Q, frequencies, rates for the adjoint) are staged
// once per block in shared memory - every warp of a block shares the op and
// the partition - with a padded rate stride so the R rate rows of one warp
// instruction fall in different banks.
#include "kernels.cuh"
#include "kernels_common.cuh"

namespace netlk {
namespace {

constexpr int S20 = 20;
constexpr int kWarps20 = 4;  // warps per block
// rate stride of a staged 20x20 matrix: 400 values + padding
template <typename real>
struct P20 {
  static constexpr int kStride = (sizeof(real) == 4) ? 404 : 402;
};

// c = child operand of the lane's (pattern, rate): CLV values and scale
// counter, 0/1 expansion of a tip's state mask, or the fake all-ones child.
template <typename real, int R>
__device__ __forceinline__ void load20(const SweepParams &p, int32_t ref, size_t g, int r, real (&c)[S20], int &s) {
  if (ref >= 0) {
    const real *src = static_cast<const real *>(p.clv) + (((size_t)ref * p.n_patterns + g) * R + r) * S20;
    if (sizeof(real) == 4) {
#pragma unroll
      for (int q = 0; q < 5; ++q) {
        const float4 t = reinterpret_cast<const float4 *>(src)[q];
        c[4 * q] = t.x; c[4 * q + 1] = t.y; c[4 * q + 2] = t.z; c[4 * q + 3] = t.w;
      }
    } else {
#pragma unroll
      for (int q = 0; q < 10; ++q) {
        const double2 t = reinterpret_cast<const double2 *>(src)[q];
        c[2 * q] = t.x; c[2 * q + 1] = t.y;
      }
    }
    s = p.scaler[(size_t)ref * p.n_patterns + g];
  } else if (ref != INT32_MIN) {
    const unsigned code = p.tips32[(size_t)(-1 - ref) * p.n_patterns + g];
#pragma unroll
    for (int i = 0; i < S20; ++i) c[i] = (real)((code >> i) & 1u);
    s = 0;
  } else {
#pragma unroll
    for (int i = 0; i < S20; ++i) c[i] = (real)1;
    s = 0;
  }
}

template <typename real, int R>
__device__ __forceinline__ void store20(real *dst, const real (&v)[S20]) {
  if (sizeof(real) == 4) {
#pragma unroll
    for (int q = 0; q < 5; ++q)
      reinterpret_cast<float4 *>(dst)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  } else {
#pragma unroll
    for (int q = 0; q < 10; ++q) reinterpret_cast<double2 *>(dst)[q] = make_double2(v[2 * q], v[2 * q + 1]);
  }
}

// 16-byte shared-memory vectors of a 20-wide row: 5 float4 / 10 double2.
template <typename real>
struct Row16;
template <>
struct Row16<float> {
  using V = float4;
  static constexpr int kPer = 4;
  __device__ static void get(const V &v, float (&o)[4]) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }
};
template <>
struct Row16<double> {
  using V = double2;
  static constexpr int kPer = 2;
  __device__ static void get(const V &v, double (&o)[2]) { o[0] = v.x; o[1] = v.y; }
};

// out = P . c with P row-major 20x20 in shared memory (16-byte aligned rows),
// read as 16-byte vectors; the sum over j runs in index order.
template <typename real>
__device__ __forceinline__ void mv20(const real *P, const real (&c)[S20], real (&out)[S20]) {
  using RV = Row16<real>;
  constexpr int K = RV::kPer;
  const typename RV::V *P4 = reinterpret_cast<const typename RV::V *>(P);
#pragma unroll
  for (int i = 0; i < S20; ++i) {
    real acc = 0;
#pragma unroll
    for (int q = 0; q < S20 / K; ++q) {
      real e[K];
      RV::get(P4[i * (S20 / K) + q], e);
#pragma unroll
      for (int t = 0; t < K; ++t) acc += e[t] * c[q * K + t];
    }
    out[i] = acc;
  }
}

// out = P^T . u
template <typename real>
__device__ __forceinline__ void mv20_t(const real *P, const real (&u)[S20], real (&out)[S20]) {
  using RV = Row16<real>;
  constexpr int K = RV::kPer;
  const typename RV::V *P4 = reinterpret_cast<const typename RV::V *>(P);
#pragma unroll
  for (int j = 0; j < S20; ++j) out[j] = 0;
#pragma unroll
  for (int i = 0; i < S20; ++i) {
#pragma unroll
    for (int q = 0; q < S20 / K; ++q) {
      real e[K];
      RV::get(P4[i * (S20 / K) + q], e);
#pragma unroll
      for (int t = 0; t < K; ++t) out[q * K + t] += e[t] * u[i];
    }
  }
}

// Stages the op's two P-matrices (all rates) of `part` in shared memory:
// sP[(m*R + r)*stride + 20*i + j], m = 0 for ea, 1 for eb (zero for the fake child).
template <typename real, int R>
__device__ __forceinline__ void stage_p20(const SweepParams &p, real *sP, int part, int ea, int eb) {
  constexpr int ST = P20<real>::kStride;
  const real *pm = static_cast<const real *>(p.pmat) + (size_t)part * p.n_edges * (R * 400);
  for (int i = threadIdx.x; i < 2 * R * 400; i += blockDim.x) {
    const int m = i / (R * 400), rem = i - m * (R * 400), rr = rem / 400, k = rem - rr * 400;
    const int e = m ? eb : ea;
    sP[(m * R + rr) * ST + k] = (e >= 0) ? __ldg(pm + (size_t)e * (R * 400) + rem) : (real)0;
  }
}

template <typename real>
__device__ __forceinline__ int rescale20(real m, real (&v)[S20]);

template <>
__device__ __forceinline__ int rescale20<float>(float m, float (&v)[S20]) {
  if (m < 0x1p-32f && m > 0.0f) {
    int e;
    frexpf(m, &e);
#pragma unroll
    for (int i = 0; i < S20; ++i) v[i] = ldexpf(v[i], -e);
    return -e;
  }
  return 0;
}

template <>
__device__ __forceinline__ int rescale20<double>(double m, double (&v)[S20]) {
  if (m < 0x1p-256) {
#pragma unroll
    for (int i = 0; i < S20; ++i) v[i] *= 0x1p256;
    return 1;
  }
  return 0;
}

// ------------------------------------------------------------------ forward
template <typename real, int R>
__global__ void __launch_bounds__(kWarps20 * 32) forward20_kernel(const SweepParams p, int op_begin) {
  constexpr int PPW = 32 / R, UNIT = PPW * kPPLForward, ST = P20<real>::kStride;
  __shared__ __align__(16) real sP[2 * R * ST];
  const FwdOp op = load_fwd_op(p.fwd_ops, op_begin + blockIdx.y);
  const int unit0 = blockIdx.x * kWarps20;
  // partitions are padded to whole 8-unit blocks: one block = one partition
  const int part = p.unit_part[unit0 * (kPPLForward / kPPLBase)];
  stage_p20<real, R>(p, sP, part, op.ea, op.b == INT32_MIN ? -1 : op.eb);
  __syncthreads();
  const int lane = threadIdx.x & 31, r = lane % R, pl = lane / R;
  const int unit = unit0 + (threadIdx.x >> 5);
  if (unit >= p.n_units_fwd) return;  // whole warp, after the only barrier
  const size_t N = (size_t)p.n_patterns;
  const real *Pa = sP + r * ST, *Pb = sP + (R + r) * ST;
  const real rw = model_val<real>(p.rate_weights, p.rate_weights32, part * R + r);
  SiteSum<real> ll;
  for (int pass = 0; pass < kPPLForward; ++pass) {
    const size_t g = (size_t)unit * UNIT + pass * PPW + pl;
    real ca[S20], v[S20];
    int sa, sb;
    load20<real, R>(p, op.a, g, r, ca, sa);
    mv20<real>(Pa, ca, v);
    if (op.b != INT32_MIN) {
      real cb[S20], pb[S20];
      load20<real, R>(p, op.b, g, r, cb, sb);
      mv20<real>(Pb, cb, pb);
#pragma unroll
      for (int i = 0; i < S20; ++i) v[i] *= pb[i];
    } else {
      sb = 0;
    }
    real m = v[0];
#pragma unroll
    for (int i = 1; i < S20; ++i) m = max(m, v[i]);
    m = rate_max<R>(m);
    const int s = sa + sb + rescale20<real>(m, v);
    store20<real, R>(static_cast<real *>(p.clv) + (((size_t)op.out * N + g) * R + r) * S20, v);
    if (r == 0) p.scaler[(size_t)op.out * N + g] = s;
    if (op.slot >= 0) {
      real t = 0;
#pragma unroll
      for (int i = 0; i < S20; ++i) t += model_val<real>(p.freqs, p.freqs32, part * S20 + i) * v[i];
      t = rate_sum<R>(rw * t);
      if (r == 0) {
        if (p.inv_term)
          ll.add_inv(p, part, g, t, s);
        else
          ll.add(p, g, t, s);
      }
    }
  }
  if (op.slot >= 0) ll.store(p.site_partial + (size_t)op.slot * p.n_units_fwd + unit, lane);
}

// One side of an adjoint op: u = 2^sh adj_x * other (the sibling's projected
// vector), returns u . (Q own) (times the rate by the caller: d/dt of
// P(t r) c = r Q P(t r) c), and writes the message P^T u to slot `out`.
template <typename real, int R>
__device__ __noinline__ real side20(const real (&ax)[S20], const real (&other)[S20], const real (&own)[S20],
                                    const real *P, const real *sQ, int sh, int out, real *msg, size_t N, size_t row) {
  real u[S20];
#pragma unroll
  for (int i = 0; i < S20; ++i) u[i] = ax[i] * other[i];
  if (sh != 0) {
#pragma unroll
    for (int i = 0; i < S20; ++i) u[i] = Scale<real>::shift(u[i], sh);
  }
  real g = 0;
  {
    real q[S20];
    mv20<real>(sQ, own, q);
#pragma unroll
    for (int i = 0; i < S20; ++i) g += u[i] * q[i];
  }
  if (out >= 0) {
    real n[S20];
    mv20_t<real>(P, u, n);
    store20<real, R>(msg + (size_t)out * N * (R * S20) + row, n);
  }
  return g;
}

// ------------------------------------------------------------------ adjoint
template <typename real, int R>
__global__ void __launch_bounds__(kWarps20 * 32) backward20_kernel(const SweepParams p, int op_begin) {
  constexpr int PPW = 32 / R, UNIT = PPW * kPPLBase, ST = P20<real>::kStride;
  __shared__ __align__(16) real sP[2 * R * ST];
  __shared__ __align__(16) real sQ[400];
  __shared__ real sF[S20];
  const int opi = op_begin + blockIdx.y;
  const BwdOp op = load_bwd_op(p.bwd_ops, opi);
  const bool fake = op.b == INT32_MIN;
  const int unit0 = blockIdx.x * kWarps20;
  const int part = p.unit_part[unit0];
  stage_p20<real, R>(p, sP, part, op.ea, fake ? -1 : op.eb);
  for (int i = threadIdx.x; i < 400; i += blockDim.x) sQ[i] = model_val<real>(p.Q, p.Q32, part * 400 + i);
  if (threadIdx.x < S20) sF[threadIdx.x] = model_val<real>(p.freqs, p.freqs32, part * S20 + threadIdx.x);
  __syncthreads();
  const int lane = threadIdx.x & 31, r = lane % R, pl = lane / R;
  const int unit = unit0 + (threadIdx.x >> 5);
  if (unit >= p.n_units) return;  // whole warp, after the only barrier
  const size_t N = (size_t)p.n_patterns;
  const real *Pa = sP + r * ST, *Pb = sP + (R + r) * ST;
  const real rw = model_val<real>(p.rate_weights, p.rate_weights32, part * R + r);
  const real rate = model_val<real>(p.rates, p.rates32, part * R + r);
  real *msg = static_cast<real *>(p.msg);
  real ga = 0, gb = 0;
  for (int pass = 0; pass < kPPLBase; ++pass) {
    const size_t g = (size_t)unit * UNIT + pass * PPW + pl;
    const size_t row = ((size_t)g * R + r) * S20;
    real ax[S20];
#pragma unroll
    for (int i = 0; i < S20; ++i) ax[i] = 0;
    for (int mi = 0; mi < op.msg_count; ++mi) {
      const real *src = msg + (size_t)__ldg(p.msg_slots + op.msg_begin + mi) * N * (R * S20) + row;
#pragma unroll
      for (int i = 0; i < S20; ++i) ax[i] += src[i];
    }
    if (op.seed >= 0) {
      // d(w_s log L_s)/d clv_x = w_s rw_r pi_i / L_s, times the tree weight
      const real *cx = static_cast<const real *>(p.clv) + (size_t)op.x * N * (R * S20) + row;
      real t = 0;
#pragma unroll
      for (int i = 0; i < S20; ++i) t += sF[i] * cx[i];
      t = rate_sum<R>(rw * t);
      const real sw = model_val<real>(p.seeds, p.seeds32, (size_t)op.seed * p.n_parts + part) *
                      pattern_weight<real>(p, g);
      if (t > (real)0 && sw != (real)0) {
        const real e = p.inv_term ? root_inv_term<real>(p, g, p.scaler[(size_t)op.x * N + g]) : (real)0;
        const real f = sw * rw / (t + e);
#pragma unroll
        for (int i = 0; i < S20; ++i) ax[i] += f * sF[i];
      }
    }
    real pa[S20], pb[S20];
    int sa, sb;
    {
      real c[S20];
      load20<real, R>(p, op.a, g, r, c, sa);
      mv20<real>(Pa, c, pa);
    }
    if (!fake) {
      real c[S20];
      load20<real, R>(p, op.b, g, r, c, sb);
      mv20<real>(Pb, c, pb);
    } else {
      sb = 0;
#pragma unroll
      for (int i = 0; i < S20; ++i) pb[i] = 1;
    }
    const int sh = p.scaler[(size_t)op.x * N + g] - sa - sb;
    ga += side20<real, R>(ax, pb, pa, Pa, sQ, sh, op.out_a, msg, N, row);
    if (!fake) gb += side20<real, R>(ax, pa, pb, Pb, sQ, sh, op.out_b, msg, N, row);
  }
  ga = warp_sum(ga * rate);
  gb = warp_sum(gb * rate);
  // row op.pad0: the op's index in the full schedule, also when a subset of
  // the ops is launched (edge derivatives)
  if (lane == 0) store_edge_terms<real>(p.grad_partial + ((size_t)op.pad0 * p.n_units + unit) * 2, ga, gb);
}

template <typename real, int R>
void run20(cudaStream_t s, const SweepParams &p, const int32_t *level_begin, int n_levels, bool backward) {
  const int units = backward ? p.n_units : p.n_units_fwd;
  const int bx = (units + kWarps20 - 1) / kWarps20;
  for (int L = 0; L < n_levels; ++L) {
    const int n = level_begin[L + 1] - level_begin[L];
    if (n <= 0) continue;
    if (backward)
      backward20_kernel<real, R><<<dim3(bx, n), kWarps20 * 32, 0, s>>>(p, level_begin[L]);
    else
      forward20_kernel<real, R><<<dim3(bx, n), kWarps20 * 32, 0, s>>>(p, level_begin[L]);
  }
}

}  // namespace

void launch_sweep20(cudaStream_t s, int precision, int R, bool backward, const SweepParams &p,
                    const int32_t *level_begin, int n_levels) {
  if (precision == 1) {
    switch (R) {
      case 1: run20<float, 1>(s, p, level_begin, n_levels, backward); break;
      case 2: run20<float, 2>(s, p, level_begin, n_levels, backward); break;
      case 4: run20<float, 4>(s, p, level_begin, n_levels, backward); break;
      default: run20<float, 8>(s, p, level_begin, n_levels, backward); break;
    }
  } else {
    switch (R) {
      case 1: run20<double, 1>(s, p, level_begin, n_levels, backward); break;
      case 2: run20<double, 2>(s, p, level_begin, n_levels, backward); break;
      case 4: run20<double, 4>(s, p, level_begin, n_levels, backward); break;
      default: run20<double, 8>(s, p, level_begin, n_levels, backward); break;
    }
  }
  int launched = 0;
  for (int L = 0; L < n_levels; ++L) launched += level_begin[L + 1] > level_begin[L];
  add_launches(launched);
}

}  // namespace netlk
