// Analytic first and second derivatives of the network log-likelihood along
// one branch, by forward-mode differentiation of the pruning above it.
//
// For the branch e and every variant x whose subtree contains e, with
// X = f (M_d d) * (M_o o) (d the child on e's side, o the other child, f the
// op's power-of-two rescaling), the tangents are
//   X'  = f (M'_e d) * (M_o o),  X'' = f (M''_e d) * (M_o o)   where d hangs from e,
//   X'  = f (M_d d') * (M_o o),  X'' = f (M_d d'') * (M_o o)   where d contains e,
// (a branch occurs at most once in a displayed tree, so never on both sides).
// At a displayed tree's root, L'/L and L''/L per site follow from the same
// root sums as L; per tree, l' = sum_s w_s L'/L and l'' = sum_s w_s (L''/L -
// (L'/L)^2). The host mixes the trees (AVERAGE: posterior-weighted; BEST: the
// chosen tree). The reference evaluates the same per-tree derivatives through
// sumtables at the virtually rerooted branch
// (src/likelihood/LikelihoodDerivatives.cpp:249-344, pll_compute_loglikelihood_derivatives
// at :95-104) and combines them at :13-188.
//
// Edge sumtables (DNA): the same forward-mode sweep with the S unit
// directions of e's message m = P_e I in place of the two tangents gives, at
// every displayed-tree root, its outside vector O = dL/dm per (pattern,
// rate); a Newton-Raphson iterate at length t is then one pass over those
// tables, L = sum_r O_r . (P_r(t) I_r) and L', L'' with P', P''
// (sumtable_walk_kernel builds them, sumtable_eval_kernel evaluates them).
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.cuh"
#include "kernels_common.cuh"
#include "tc.cuh"

namespace netlk {

namespace {

// dP/dt and d2P/dt2 of P(rho_r t) = U diag(exp(lambda rho_r t)) U^-1 for one
// edge, every partition (its length brlen[part * len_stride + edge]) and
// rate: out [part][2][R][S][S].
__global__ void pderiv_kernel(int n_parts, int R, int S, const double *__restrict__ lambda,
                              const double *__restrict__ U, const double *__restrict__ Uinv,
                              const double *__restrict__ rates, const double *__restrict__ brlen, int len_stride,
                              int edge, double *__restrict__ out64, float *__restrict__ out32) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int SS = S * S;
  const int64_t total = (int64_t)n_parts * 2 * R * SS;
  if (idx >= total) return;
  const int ij = (int)(idx % SS);
  const int i = ij / S, j = ij - i * S;
  const int64_t q = idx / SS;  // (part, order, rate)
  const int rr = (int)(q % R);
  const int order = (int)(q / R % 2);
  const int part = (int)(q / R / 2);
  const double rho = rates[part * R + rr];
  const double t = brlen[(size_t)part * len_stride + edge];
  double v = 0.0;
  for (int k = 0; k < S; ++k) {
    const double lr = lambda[part * S + k] * rho;
    const double f = order ? lr * lr : lr;
    v += U[(size_t)part * SS + i * S + k] * f * exp(lr * t) * Uinv[(size_t)part * SS + k * S + j];
  }
  out64[idx] = v;
  if (out32) out32[idx] = (float)v;
}

// x times the op's rescaling factor for a counter increase of k: FP32
// counters count single powers of two, FP64 counters factors of 2^256.
template <typename real>
struct ScaleShift;
template <>
struct ScaleShift<float> {
  static constexpr double kLogUnit = -0.69314718055994530942;  // log(2^-1)
  static __device__ __forceinline__ float apply(float x, int k) { return ldexpf(x, k); }
  static __device__ __forceinline__ float log(float x) { return logf(x); }
};
template <>
struct ScaleShift<double> {
  static constexpr double kLogUnit = -177.44567822334599921;  // log(2^-256)
  static __device__ __forceinline__ double apply(double x, int k) { return ldexp(x, 256 * k); }
  static __device__ __forceinline__ double log(double x) { return ::log(x); }
};

// S consecutive reals through the read-only path, 16 bytes at a time (S is a
// multiple of 4; rows start on 16-byte boundaries).
template <typename real, int S>
__device__ __forceinline__ void ldg_row(const real *src, real (&c)[S]) {
  if constexpr (sizeof(real) == 4) {
#pragma unroll
    for (int i = 0; i < S; i += 4) {
      const float4 v = __ldg(reinterpret_cast<const float4 *>(src + i));
      c[i] = v.x;
      c[i + 1] = v.y;
      c[i + 2] = v.z;
      c[i + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < S; i += 2) {
      const double2 v = __ldg(reinterpret_cast<const double2 *>(src + i));
      c[i] = v.x;
      c[i + 1] = v.y;
    }
  }
}

template <typename real, int S>
__device__ __forceinline__ void st_row(real *dst, const real (&c)[S]) {
  if constexpr (sizeof(real) == 4) {
#pragma unroll
    for (int i = 0; i < S; i += 4) *reinterpret_cast<float4 *>(dst + i) = make_float4(c[i], c[i + 1], c[i + 2], c[i + 3]);
  } else {
#pragma unroll
    for (int i = 0; i < S; i += 2) *reinterpret_cast<double2 *>(dst + i) = make_double2(c[i], c[i + 1]);
  }
}

// One child's row for the thread's (pattern, rate): a CLV row, a tip's 0/1
// state mask, or the fake child's ones; returns its scale counter.
template <typename real, int R, int S>
__device__ __forceinline__ int load_row(const TanParams &p, int32_t ref, int64_t s, int r, real (&c)[S]) {
  if (ref >= 0) {
    ldg_row<real, S>(static_cast<const real *>(p.clv) + (((size_t)ref * p.n_patterns + s) * R + r) * S, c);
    return __ldg(p.scaler + (size_t)ref * p.n_patterns + s);
  }
  if (ref == INT32_MIN) {
#pragma unroll
    for (int i = 0; i < S; ++i) c[i] = (real)1;
    return 0;
  }
  uint32_t code;
  if constexpr (S == 4)
    code = __ldg(p.tips + (size_t)(-1 - ref) * p.n_patterns + s);
  else
    code = __ldg(p.tips32 + (size_t)(-1 - ref) * p.n_patterns + s);
#pragma unroll
  for (int i = 0; i < S; ++i) c[i] = (real)((code >> i) & 1u);
  return 0;
}

template <typename real, int S>
__device__ __forceinline__ void matvec(const real *M, const real (&x)[S], real (&y)[S]) {
#pragma unroll
  for (int i = 0; i < S; ++i) {
    real acc = M[i * S] * x[0];
#pragma unroll
    for (int j = 1; j < S; ++j) acc = fma(M[i * S + j], x[j], acc);
    y[i] = acc;
  }
}

// Patterns per thread: a block covers kTanPPT * 256 / R patterns, which is
// the padding unit of every partition, so a block never spans two.
constexpr int kTanPPT = 4;

// One launch per DAG level (blockIdx.y = op of the level); a thread owns one
// rate of kTanPPT patterns (strided by 256 / R), a block 1024 / R patterns of
// one partition. Shared memory: the other side's P, then the two matrices
// applied to the e side (P'_e and P''_e, or P_d twice), then the partition's
// frequencies and rate weights. Every read goes through the read-only path:
// nothing a launch reads is written in it (a tangent slot is reused only
// after the level that read it). At displayed-tree roots the site sums run
// in the context's precision; only the per-site accumulation is FP64.
template <typename real, int R, int S>
__global__ void __launch_bounds__(256) tangent_kernel(const TanParams p, int op_begin) {
  constexpr int RSS = R * S * S;
  constexpr int ROWS = 256 / R;  // patterns per pass of the block
  extern __shared__ __align__(16) unsigned char smem_raw[];
  real *sM = reinterpret_cast<real *>(smem_raw);
  real *sPi = sM + 3 * RSS, *sRw = sPi + S;
  const TanOp op = p.ops[op_begin + blockIdx.y];
  const int part = p.block_part[blockIdx.x];
  const real *pm = static_cast<const real *>(p.pmat) + (size_t)part * p.n_edges * RSS;
  const real *pd = static_cast<const real *>(p.pderiv) + (size_t)part * 2 * RSS;
  for (int i = threadIdx.x; i < RSS; i += blockDim.x) {
    sM[i] = op.eo >= 0 ? __ldg(pm + (size_t)op.eo * RSS + i) : (real)0;
    if (op.mode == 1) {
      sM[RSS + i] = __ldg(pd + i);
      sM[2 * RSS + i] = __ldg(pd + RSS + i);
    } else {
      const real v = __ldg(pm + (size_t)op.ed * RSS + i);
      sM[RSS + i] = v;
      sM[2 * RSS + i] = v;
    }
  }
  if (threadIdx.x < S) sPi[threadIdx.x] = (real)p.freqs[part * S + threadIdx.x];
  if (threadIdx.x < R) sRw[threadIdx.x] = (real)p.rate_weights[part * R + threadIdx.x];
  __syncthreads();
  const int r = threadIdx.x % R;
  const size_t plane = (size_t)p.n_patterns * R * S;
  const real *Mo = sM + r * S * S, *M1 = sM + RSS + r * S * S, *M2 = sM + 2 * RSS + r * S * S;
  const real *tsrc = static_cast<const real *>(p.tan) + (size_t)op.td * 2 * plane;
  real *tdst = static_cast<real *>(p.tan) + (size_t)op.tx * 2 * plane;
  double a1 = 0.0, a2 = 0.0;  // root slots: this thread's site sums
#pragma unroll
  for (int q = 0; q < kTanPPT; ++q) {
    const int64_t s = ((int64_t)blockIdx.x * kTanPPT + q) * ROWS + threadIdx.x / R;
    const size_t row = ((size_t)s * R + r) * S;
    real c[S], vo[S], t1[S], t2[S];
    const int so = load_row<real, R, S>(p, op.o, s, r, c);
    if (op.o == INT32_MIN) {
#pragma unroll
      for (int i = 0; i < S; ++i) vo[i] = (real)1;
    } else {
      matvec<real, S>(Mo, c, vo);
    }
    int sd;
    if (op.mode == 1) {
      sd = load_row<real, R, S>(p, op.d, s, r, c);
      matvec<real, S>(M1, c, t1);
      matvec<real, S>(M2, c, t2);
    } else {
      sd = __ldg(p.scaler + (size_t)op.d * p.n_patterns + s);
      ldg_row<real, S>(tsrc + row, c);
      matvec<real, S>(M1, c, t1);
      ldg_row<real, S>(tsrc + plane + row, c);
      matvec<real, S>(M2, c, t2);
    }
    const int k = __ldg(p.scaler + (size_t)op.x * p.n_patterns + s) - sd - so;
#pragma unroll
    for (int i = 0; i < S; ++i) {
      t1[i] = ScaleShift<real>::apply(t1[i] * vo[i], k);
      t2[i] = ScaleShift<real>::apply(t2[i] * vo[i], k);
    }
    if (op.tx >= 0) {
      st_row<real, S>(tdst + row, t1);
      st_row<real, S>(tdst + plane + row, t2);
    }
    if (op.slot < 0) continue;  // uniform over the block
    // displayed-tree root: L, L', L'' of the site (sums over the R rate lanes)
    real xr[S];
    ldg_row<real, S>(static_cast<const real *>(p.clv) + (size_t)op.x * plane + row, xr);
    real L = 0, L1 = 0, L2 = 0;
#pragma unroll
    for (int i = 0; i < S; ++i) {
      L = fma(sPi[i], xr[i], L);
      L1 = fma(sPi[i], t1[i], L1);
      L2 = fma(sPi[i], t2[i], L2);
    }
    L *= sRw[r];
    L1 *= sRw[r];
    L2 *= sRw[r];
#pragma unroll
    for (int o = 1; o < R; o <<= 1) {
      L += __shfl_xor_sync(0xffffffffu, L, o);
      L1 += __shfl_xor_sync(0xffffffffu, L1, o);
      L2 += __shfl_xor_sync(0xffffffffu, L2, o);
    }
    if (r == 0) {
      const double w = __ldg(p.weights + s);
      if (w != 0.0) {
        if (p.inv_term) {  // invariant sites: L = gf (L_mix + iq), gf cancels in the ratios
          const real iq = (real)p.inv_term[s];
          if (iq > (real)0) L += ScaleShift<real>::apply(iq, __ldg(p.scaler + (size_t)op.x * p.n_patterns + s));
        }
        const real q1 = L1 / L, q2 = L2 / L;
        a1 += w * (double)q1;
        a2 += w * ((double)q2 - (double)q1 * (double)q1);
      }
    }
  }
  if (op.slot < 0) return;  // uniform over the block
  // fixed-order block sum: warp shuffles, then thread 0 over the warp sums
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a1 += __shfl_down_sync(0xffffffffu, a1, o);
    a2 += __shfl_down_sync(0xffffffffu, a2, o);
  }
  __shared__ double red[2][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][warp] = a1;
    red[1][warp] = a2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double b1 = 0.0, b2 = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      b1 += red[0][k];
      b2 += red[1][k];
    }
    p.partial[((size_t)op.slot * 2 + 0) * p.n_blocks + blockIdx.x] = b1;
    p.partial[((size_t)op.slot * 2 + 1) * p.n_blocks + blockIdx.x] = b2;
  }
}

// out[(slot * n_parts + part) * 2 + q] = compensated sum of the slot's block
// partials over the partition's blocks, for the slots listed in `slots`.
__global__ void tangent_reduce_kernel(const TanParams p, const int32_t *__restrict__ slots,
                                      const int32_t *__restrict__ part_block_begin, int n_parts,
                                      double *__restrict__ out) {
  const int slot = slots[blockIdx.x], part = blockIdx.y, q = blockIdx.z;
  const int b0 = part_block_begin[part], b1 = part_block_begin[part + 1];
  const double *src = p.partial + ((size_t)slot * 2 + q) * p.n_blocks;
  const float2 *src32 = reinterpret_cast<const float2 *>(src);
  double s = 0.0, c = 0.0;
  for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
    const double y = (p.ff ? (double)src32[b].x + (double)src32[b].y : src[b]) - c;
    const double t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __shared__ double red[128];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[((size_t)slot * n_parts + part) * 2 + q] = red[0];
}

// The tangent sweep as a walk (DNA): one warp per PPL * 32 / R patterns
// (lane = (rate, PPL patterns)) runs every op of the schedule in depth-first
// order (walk_order: each op right before the ops that read its tangents),
// so tangent rows come back from L2. Per op the arithmetic of
// tangent_kernel: where x takes e's message, X' and X'' are P'_e d and
// P''_e d times vo; above, P_d times the child's X' and X''; both times the
// op's rescaling. At a displayed-tree root the site sums L, L', L'' (over
// the R rate lanes), then per pattern w L'/L and w (L''/L - (L'/L)^2),
// summed over the warp into partial[slot][q][unit] (FP64 contexts: FP64;
// FP32 contexts: FP32 terms, float-float warp sums). Tangent rows are
// read with plain (coherent) loads: this kernel writes them.
template <typename real, int R, int PPL>
__global__ void __launch_bounds__(256) tangent_walk_kernel(const TanParams p, int n_ops, int64_t n_units) {
  constexpr int S = 4, PPW = 32 / R, RSS = R * S * S;
  const int lane = threadIdx.x & 31, r = lane % R;
  const int64_t unit = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  if (unit >= n_units) return;  // whole warp
  const int64_t s0 = unit * PPL * PPW + lane / R;
  const int part = p.block_part[s0 / (kTanPPT * 256 / R)];
  const real *pm = static_cast<const real *>(p.pmat) + ((size_t)part * p.n_edges * R + r) * S * S;
  const real *pd = static_cast<const real *>(p.pderiv) + ((size_t)part * 2 * R + r) * S * S;
  real pi[S];
#pragma unroll
  for (int i = 0; i < S; ++i) pi[i] = (real)p.freqs[part * S + i];
  const real rw = (real)p.rate_weights[part * R + r];
  const size_t plane = (size_t)p.n_patterns * R * S;
  real *tan = static_cast<real *>(p.tan);
  auto load_m = [&](const real *src, real (&M)[S * S]) {
#pragma unroll
    for (int i = 0; i < S; ++i) ldg_row<real, S>(src + i * S, *reinterpret_cast<real(*)[S]>(M + i * S));
  };
  for (int j = 0; j < n_ops; ++j) {
    const TanOp op = p.ops[j];
    if (j + 1 < n_ops) {  // ask L2 for the next op's other child (a CLV written long before)
      const int32_t on = __ldg(&p.ops[j + 1].o);
      if (on >= 0)
#pragma unroll
        for (int q = 0; q < PPL; ++q)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(static_cast<const real *>(p.clv) +
                                                        (((size_t)on * p.n_patterns + s0 + q * PPW) * R + r) * S));
    }
    real M[S * S], vo[PPL][S], t1[PPL][S], t2[PPL][S];
    int k[PPL];
#pragma unroll
    for (int q = 0; q < PPL; ++q) {
      const int64_t s = s0 + q * PPW;
      real c[S];
      const int so = load_row<real, R, S>(p, op.o, s, r, c);
      const int sd = op.d >= 0 ? __ldg(p.scaler + (size_t)op.d * p.n_patterns + s) : 0;
      k[q] = __ldg(p.scaler + (size_t)op.x * p.n_patterns + s) - sd - so;
#pragma unroll
      for (int i = 0; i < S; ++i) vo[q][i] = c[i];
    }
    if (op.o == INT32_MIN) {
#pragma unroll
      for (int q = 0; q < PPL; ++q)
#pragma unroll
        for (int i = 0; i < S; ++i) vo[q][i] = (real)1;
    } else {
      load_m(pm + (size_t)op.eo * RSS, M);
#pragma unroll
      for (int q = 0; q < PPL; ++q) {
        real c[S];
#pragma unroll
        for (int i = 0; i < S; ++i) c[i] = vo[q][i];
        matvec<real, S>(M, c, vo[q]);
      }
    }
    if (op.mode == 1) {
      real cd[PPL][S];
#pragma unroll
      for (int q = 0; q < PPL; ++q) load_row<real, R, S>(p, op.d, s0 + q * PPW, r, cd[q]);
      load_m(pd, M);
#pragma unroll
      for (int q = 0; q < PPL; ++q) matvec<real, S>(M, cd[q], t1[q]);
      load_m(pd + (size_t)R * S * S, M);
#pragma unroll
      for (int q = 0; q < PPL; ++q) matvec<real, S>(M, cd[q], t2[q]);
    } else {
      load_m(pm + (size_t)op.ed * RSS, M);
#pragma unroll
      for (int q = 0; q < PPL; ++q) {
        const size_t row = ((size_t)(s0 + q * PPW) * R + r) * S;
        real a[S], b[S];
#pragma unroll
        for (int i = 0; i < S; ++i) {
          a[i] = tan[((size_t)op.td * 2) * plane + row + i];
          b[i] = tan[((size_t)op.td * 2 + 1) * plane + row + i];
        }
        matvec<real, S>(M, a, t1[q]);
        matvec<real, S>(M, b, t2[q]);
      }
    }
    // root site terms: FP64 sums in FP64 contexts; in FP32 ones FP32 terms
    // whose warp sums are float-float pairs (no FP64 instruction per root)
    double a1 = 0.0, a2 = 0.0;
    float f1 = 0.f, f2 = 0.f;
#pragma unroll
    for (int q = 0; q < PPL; ++q) {
      const int64_t s = s0 + q * PPW;
      const size_t row = ((size_t)s * R + r) * S;
#pragma unroll
      for (int i = 0; i < S; ++i) {
        t1[q][i] = ScaleShift<real>::apply(t1[q][i] * vo[q][i], k[q]);
        t2[q][i] = ScaleShift<real>::apply(t2[q][i] * vo[q][i], k[q]);
      }
      if (op.tx >= 0) {
        st_row<real, S>(tan + ((size_t)op.tx * 2) * plane + row, t1[q]);
        st_row<real, S>(tan + ((size_t)op.tx * 2 + 1) * plane + row, t2[q]);
      }
      if (op.slot < 0) continue;  // uniform over the warp
      real xr[S];
      ldg_row<real, S>(static_cast<const real *>(p.clv) + (size_t)op.x * plane + row, xr);
      real L = 0, L1 = 0, L2 = 0;
#pragma unroll
      for (int i = 0; i < S; ++i) {
        L = fma(pi[i], xr[i], L);
        L1 = fma(pi[i], t1[q][i], L1);
        L2 = fma(pi[i], t2[q][i], L2);
      }
      L *= rw;
      L1 *= rw;
      L2 *= rw;
#pragma unroll
      for (int o = 1; o < R; o <<= 1) {
        L += __shfl_xor_sync(0xffffffffu, L, o);
        L1 += __shfl_xor_sync(0xffffffffu, L1, o);
        L2 += __shfl_xor_sync(0xffffffffu, L2, o);
      }
      if (r == 0) {
        if constexpr (sizeof(real) == 4) {
          const float w = __ldg(p.weights32 + s).x;
          if (w != 0.f) {
            if (p.inv_term32) {  // invariant sites: L = gf (L_mix + iq), gf cancels in the ratios
              const float iq = p.inv_term32[s];
              if (iq > 0.f) L += ldexpf(iq, __ldg(p.scaler + (size_t)op.x * p.n_patterns + s));
            }
            const float inv = 1.0f / L, q1 = L1 * inv, q2 = L2 * inv;
            f1 += w * q1;
            f2 += w * (q2 - q1 * q1);
          }
        } else {
          const double w = __ldg(p.weights + s);
          if (w != 0.0) {
            if (p.inv_term) {  // invariant sites: L = gf (L_mix + iq), gf cancels in the ratios
              const real iq = (real)p.inv_term[s];
              if (iq > (real)0) L += ScaleShift<real>::apply(iq, __ldg(p.scaler + (size_t)op.x * p.n_patterns + s));
            }
            const real q1 = L1 / L, q2 = L2 / L;
            a1 += w * (double)q1;
            a2 += w * ((double)q2 - (double)q1 * (double)q1);
          }
        }
      }
    }
    if (op.slot < 0) continue;  // uniform over the warp
    if constexpr (sizeof(real) == 4) {
      const FF g1 = warp_sum_ff(FF{f1, 0.f}), g2 = warp_sum_ff(FF{f2, 0.f});
      if (lane == 0) {
        float2 *dst = reinterpret_cast<float2 *>(p.partial);
        dst[((size_t)op.slot * 2 + 0) * n_units + unit] = make_float2(g1.hi, g1.lo);
        dst[((size_t)op.slot * 2 + 1) * n_units + unit] = make_float2(g2.hi, g2.lo);
      }
    } else {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        a1 += __shfl_down_sync(0xffffffffu, a1, o);
        a2 += __shfl_down_sync(0xffffffffu, a2, o);
      }
      if (lane == 0) {
        p.partial[((size_t)op.slot * 2 + 0) * n_units + unit] = a1;
        p.partial[((size_t)op.slot * 2 + 1) * n_units + unit] = a2;
      }
    }
  }
}

// ------------------------------------------------------------ sumtables
// One table's site terms for the thread's pattern s (site likelihood L and
// its derivatives L1, L2 in the table's scaled units), summed over the warp
// into partial[table][q][warp].
template <typename real>
__device__ __forceinline__ void sumtable_site_terms(const StabParams &sp, int tb, int64_t gw, int64_t n_warps,
                                                    double w, real iq, int k, real L, real L1, real L2) {
  const bool lead = (threadIdx.x & 31) == 0;
  if constexpr (sizeof(real) == 4) {
    // FP32 sweeps: per-site terms and the warp sums in FP32 (the log term as
    // a float-float pair), stored as float pairs in the partial's 8 bytes:
    // no FP64 instruction per table
    float v0 = 0.f, v1 = 0.f, v2 = 0.f;
    const float wf = (float)w;
    if (wf != 0.f) {
      if (iq > 0.f) L += ldexpf(iq, k);
      const float inv = 1.0f / L, q1 = L1 * inv, q2 = L2 * inv;
      v0 = wf * (logf(L) + (float)k * (float)ScaleShift<float>::kLogUnit);
      v1 = wf * q1;
      v2 = wf * (q2 - q1 * q1);
    }
    const FF f0 = warp_sum_ff(FF{v0, 0.f});
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v1 += __shfl_xor_sync(0xffffffffu, v1, o);
      v2 += __shfl_xor_sync(0xffffffffu, v2, o);
    }
    if (lead) {
      float2 *dst = reinterpret_cast<float2 *>(sp.partial);
      dst[((size_t)tb * 3 + 0) * n_warps + gw] = make_float2(f0.hi, f0.lo);
      dst[((size_t)tb * 3 + 1) * n_warps + gw] = make_float2(v1, 0.f);
      dst[((size_t)tb * 3 + 2) * n_warps + gw] = make_float2(v2, 0.f);
    }
  } else {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    if (w != 0.0) {
      if (iq > (real)0) L += ScaleShift<real>::apply(iq, k);
      const real q1 = L1 / L, q2 = L2 / L;
      a0 = w * ((double)ScaleShift<real>::log(L) + (double)k * ScaleShift<real>::kLogUnit);
      a1 = w * (double)q1;
      a2 = w * ((double)q2 - (double)q1 * (double)q1);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_down_sync(0xffffffffu, a0, o);
      a1 += __shfl_down_sync(0xffffffffu, a1, o);
      a2 += __shfl_down_sync(0xffffffffu, a2, o);
    }
    if (lead) {
      sp.partial[((size_t)tb * 3 + 0) * n_warps + gw] = a0;
      sp.partial[((size_t)tb * 3 + 1) * n_warps + gw] = a1;
      sp.partial[((size_t)tb * 3 + 2) * n_warps + gw] = a2;
    }
  }
}

// Table build as a walk: one warp per unit of PPL * 32 / R patterns (lane =
// (rate, PPL patterns)) runs every op of the tangent schedule in level order, so
// the direction rows an op writes are read back by the same lanes soon
// after, mostly from L2 (the level form, one launch per DAG level, wrote and
// re-read them through DRAM). Per op: where x takes e's message (mode 1)
// direction i is vo_i at state i and 0 elsewhere; where x's child d contains
// e (mode 2) it is (P_d times d's direction i) * vo, vo = P_o o the other
// child's message; both times the op's rescaling (its scale counter minus
// the children's). At a displayed-tree root the lane writes its (pattern,
// rate) row of the outside vector, O_i = w_r sum_j pi_j X_i[j], and lane
// r = 0 the root's scale counter. Direction rows are read with plain
// (coherent) loads: this kernel writes them.
template <typename real, int R, int PPL>
__global__ void __launch_bounds__(256) sumtable_walk_kernel(const StabParams sp, int n_ops) {
  constexpr int S = 4, PPW = 32 / R;
  const TanParams &p = sp.t;
  const int lane = threadIdx.x & 31, r = lane % R;
  // the warp's PPL * PPW patterns; lane: rate r of patterns s0 + q PPW
  const int64_t s0 = ((int64_t)blockIdx.x * 8 + (threadIdx.x >> 5)) * PPL * PPW + lane / R;
  if (s0 >= p.n_patterns) return;  // whole warps: n_patterns is a multiple of PPL * 32 / R
  const int part = p.block_part[s0 / (kTanPPT * 256 / R)];
  const real *pm = static_cast<const real *>(p.pmat) + ((size_t)part * p.n_edges * R + r) * S * S;
  real pi[S];
#pragma unroll
  for (int i = 0; i < S; ++i) pi[i] = (real)p.freqs[part * S + i];
  const real rw = (real)p.rate_weights[part * R + r];
  const size_t plane = (size_t)p.n_patterns * R * S;
  real *dir = static_cast<real *>(p.tan);
  for (int j = 0; j < n_ops; ++j) {
    const TanOp op = p.ops[j];
    if (j + 1 < n_ops) {  // ask L2 for the next op's other child (a CLV written long before)
      const int32_t on = __ldg(&p.ops[j + 1].o);
      if (on >= 0) {
#pragma unroll
        for (int q = 0; q < PPL; ++q) {
          const int64_t s = s0 + q * PPW;
          asm volatile("prefetch.global.L2 [%0];" ::"l"(static_cast<const real *>(p.clv) +
                                                        (((size_t)on * p.n_patterns + s) * R + r) * S));
        }
      }
    }
    real M[S * S], c[PPL][S], vo[PPL][S];
    int k[PPL], sx[PPL];
#pragma unroll
    for (int q = 0; q < PPL; ++q) {
      const int64_t s = s0 + q * PPW;
      const int so = load_row<real, R, S>(p, op.o, s, r, c[q]);
      const int sd = op.d >= 0 ? __ldg(p.scaler + (size_t)op.d * p.n_patterns + s) : 0;
      sx[q] = __ldg(p.scaler + (size_t)op.x * p.n_patterns + s);
      k[q] = sx[q] - sd - so;
    }
    if (op.o == INT32_MIN) {
#pragma unroll
      for (int q = 0; q < PPL; ++q)
#pragma unroll
        for (int i = 0; i < S; ++i) vo[q][i] = (real)1;
    } else {
#pragma unroll
      for (int i = 0; i < S; ++i)
        ldg_row<real, S>(pm + (size_t)op.eo * R * S * S + i * S, *reinterpret_cast<real(*)[S]>(M + i * S));
#pragma unroll
      for (int q = 0; q < PPL; ++q) matvec<real, S>(M, c[q], vo[q]);
    }
    if (op.mode == 2)
#pragma unroll
      for (int i = 0; i < S; ++i)
        ldg_row<real, S>(pm + (size_t)op.ed * R * S * S + i * S, *reinterpret_cast<real(*)[S]>(M + i * S));
#pragma unroll
    for (int q = 0; q < PPL; ++q) {
      const int64_t s = s0 + q * PPW;
      const size_t row = ((size_t)s * R + r) * S;
      real o[S];
#pragma unroll
      for (int i = 0; i < S; ++i) {
        real t[S];
        if (op.mode == 1) {
#pragma unroll
          for (int jj = 0; jj < S; ++jj) t[jj] = jj == i ? ScaleShift<real>::apply(vo[q][jj], k[q]) : (real)0;
        } else {
          const real *src = dir + ((size_t)op.td * S + i) * plane + row;
          real d[S];
#pragma unroll
          for (int jj = 0; jj < S; ++jj) d[jj] = src[jj];
          matvec<real, S>(M, d, t);
#pragma unroll
          for (int jj = 0; jj < S; ++jj) t[jj] = ScaleShift<real>::apply(t[jj] * vo[q][jj], k[q]);
        }
        if (op.tx >= 0) st_row<real, S>(dir + ((size_t)op.tx * S + i) * plane + row, t);
        real a = (real)0;
#pragma unroll
        for (int jj = 0; jj < S; ++jj) a = fma(pi[jj], t[jj], a);
        o[i] = a * rw;
      }
      if (op.slot < 0) continue;  // uniform over the warp
      st_row<real, S>(static_cast<real *>(sp.table) + ((size_t)op.slot * p.n_patterns + (s & ~(int64_t)127)) * R * S +
                          ((size_t)r * 128 + (s & 127)) * S,
                      o);
      if (r == 0) sp.table_scaler[(size_t)op.slot * p.n_patterns + s] = sx[q];
    }
  }
}

// Table evaluation: one thread per pattern, 128 per block (a partition's
// padding unit, 1024 / R patterns, is a multiple of 128, so a block never
// spans two), blockIdx.y = a run of tables_per_block tables (enough blocks
// to fill the GPU whatever the pattern count). A table's rows for the
// block's 128 patterns are one contiguous 128 R S-real chunk, its scale
// counters one 512-byte chunk: thread 0 streams both into a ring of
// kEvalStages shared-memory stages with cp.async.bulk (completion on the
// stage's mbarrier), so several tables per block are in flight while the
// threads reduce an earlier one. Per child group the threads form
// m = P I, m' = P' I and m'' = P'' I for their R rates once, then per table
// L, L', L'' (dot products with the table's rows), the site's w log L (with
// the table's scale counter and the +I term) and w L'/L, w (L''/L -
// (L'/L)^2); the warp's sums go to partial[table][q][warp] (fixed order;
// FP32 tables: float pairs whose sum is the value). Every mbarrier wait is
// bounded: past about a second the block sets *fault, waits (bounded) for
// its copies in flight and returns.
template <typename real, int R>
__host__ __device__ constexpr int eval_stages() {
  return 128 * R * 4 * (int)sizeof(real) <= 8192 ? 4 : 2;
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

__device__ __forceinline__ void mbar_expect(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

template <typename real, int R, int S>
__global__ void __launch_bounds__(128) sumtable_eval_kernel(const StabParams sp) {
  const TanParams &p = sp.t;
  constexpr int RSS = R * S * S;
  constexpr int K = eval_stages<real, R>();
  constexpr uint32_t kRows = 128 * R * S * sizeof(real), kSc = 128 * 4;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  real *stage_rows = reinterpret_cast<real *>(smem_raw);                          // [K][128][R][S]
  int32_t *stage_sc = reinterpret_cast<int32_t *>(smem_raw + K * kRows);          // [K][128]
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw + K * (kRows + kSc));    // [K]
  real *sM = reinterpret_cast<real *>(smem_raw + K * (kRows + kSc) + 8 * K);      // [3][R][S][S]
  const int64_t x0 = (int64_t)blockIdx.x * 128, s = x0 + threadIdx.x;
  const int part = p.block_part[x0 / (kTanPPT * 256 / R)];
  const real *src = static_cast<const real *>(sp.pm3) + (size_t)part * 3 * RSS;
  for (int i = threadIdx.x; i < 3 * RSS; i += blockDim.x) sM[i] = src[i];
  const int tb_lo = blockIdx.y * sp.tables_per_block;
  const int tb_end = min(tb_lo + sp.tables_per_block, sp.n_tables);
  const int n = tb_end - tb_lo;  // tables of this block, streamed in order
  const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(bars);
  const uint32_t rows0 = (uint32_t)__cvta_generic_to_shared(stage_rows);
  const uint32_t sc0 = (uint32_t)__cvta_generic_to_shared(stage_sc);
  auto issue = [&](int j) {  // thread 0: table tb_lo + j into stage j % K
    const int st = j % K;
    const size_t tb = (size_t)(tb_lo + j);
    mbar_expect(bar0 + 8 * st, kRows + kSc);
    bulk_load(rows0 + st * kRows, static_cast<const real *>(sp.table) + (tb * p.n_patterns + x0) * R * S, kRows,
              bar0 + 8 * st);
    bulk_load(sc0 + st * kSc, sp.table_scaler + tb * p.n_patterns + x0, kSc, bar0 + 8 * st);
  };
  if (threadIdx.x == 0) {
    for (int st = 0; st < K; ++st) tc::mbar_init(bar0 + 8 * st, 1);
    for (int j = 0; j < min(K, n); ++j) issue(j);
  }
  __syncthreads();
  const double w = __ldg(p.weights + s);
  const real iq = p.inv_term ? (real)p.inv_term[s] : (real)0;
  int g = 0;
  while (g < sp.n_groups && sp.group_begin[g + 1] <= tb_lo) ++g;
  real m0[R][S], m1[R][S], m2[R][S];
  int g_end = -1;  // first table past the group m0..m2 belong to
  for (int j = 0; j < n; ++j) {
    const int tb = tb_lo + j;
    if (tb >= g_end) {  // uniform over the block
      while (sp.group_begin[g + 1] <= tb) ++g;
      g_end = sp.group_begin[g + 1];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        real c[S];
        load_row<real, R, S>(p, sp.group_ref[g], s, r, c);
        matvec<real, S>(sM + r * S * S, c, m0[r]);
        matvec<real, S>(sM + RSS + r * S * S, c, m1[r]);
        matvec<real, S>(sM + 2 * RSS + r * S * S, c, m2[r]);
      }
    }
    const int st = j % K;
    const bool ok = tc::mbar_wait(bar0 + 8 * st, (uint32_t)((j / K) & 1));
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        *sp.fault = 1;
        for (int q = j; q < min(j + K, n); ++q) (void)tc::mbar_wait(bar0 + 8 * (q % K), (uint32_t)((q / K) & 1));
      }
      return;  // uniform over the block
    }
    // the thread's rows: rate r of the chunk's 128 patterns are contiguous,
    // so a warp's reads of one rate cover consecutive 16-byte pieces
    const real *chunk = stage_rows + (size_t)st * 128 * R * S;
    real L = 0, L1 = 0, L2 = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      real o[S];
#pragma unroll
      for (int i = 0; i < S; ++i) o[i] = chunk[((size_t)r * 128 + threadIdx.x) * S + i];
#pragma unroll
      for (int i = 0; i < S; ++i) {
        L = fma(o[i], m0[r][i], L);
        L1 = fma(o[i], m1[r][i], L1);
        L2 = fma(o[i], m2[r][i], L2);
      }
    }
    const int k = stage_sc[st * 128 + threadIdx.x];
    __syncthreads();  // every thread is done with stage st
    if (threadIdx.x == 0 && j + K < n) {
      tc::fence_proxy_async();
      issue(j + K);
    }
    sumtable_site_terms<real>(sp, tb, s / 32, p.n_patterns / 32, w, iq, k, L, L1, L2);
  }
}

// Tables for 20-state partitions, by reverse walks (the forward-mode build
// would carry 20 directions): per displayed tree containing e, from its
// root down the path to e (the tangent schedule's chain of children that
// hold e), O starts as w_r pi at the root; at a variant v with the path
// child d and the other child o, u = O * (P_o o) * 2^k (k: v's scale counter
// minus its children's), then O <- P_d^T u; at the variant that takes e's
// message, u is the table row (the same O = dL/dm as the DNA build).
// Block: 256 threads = 256 / R patterns x R rates of one partition,
// blockIdx.y = table; each op's two P matrices staged in shared memory.
template <typename real, int R>
__global__ void __launch_bounds__(256) sumtable_path20_kernel(const StabParams sp) {
  constexpr int S = 20, SS = S * S, ROWS = 256 / R;
  const TanParams &p = sp.t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  real *sPo = reinterpret_cast<real *>(smem_raw);  // [R][S][S]
  real *sPd = sPo + R * SS;                         // [R][S][S]
  const int tb = blockIdx.y, r = threadIdx.x % R;
  const int64_t s = (int64_t)blockIdx.x * ROWS + threadIdx.x / R;
  const int part = p.block_part[(blockIdx.x * ROWS) / (kTanPPT * 256 / R)];
  const real *pm = static_cast<const real *>(p.pmat) + (size_t)part * p.n_edges * R * SS;
  const real rw = (real)p.rate_weights[part * R + r];
  real O[S], u[S];
#pragma unroll
  for (int i = 0; i < S; ++i) O[i] = rw * (real)p.freqs[part * S + i];
  int sx_root = 0;
  const int kb = sp.path_begin[tb], ke = sp.path_begin[tb + 1];
  for (int q = kb; q < ke; ++q) {
    const int32_t *po = sp.path_ops + 6 * (size_t)q;  // x, d, o, ed, eo, mode
    const int32_t x = po[0], d = po[1], o = po[2], ed = po[3], eo = po[4], mode = po[5];
    __syncthreads();  // every thread is done with the previous op's matrices
    for (int i = threadIdx.x; i < R * SS; i += blockDim.x) {
      sPo[i] = eo >= 0 ? __ldg(pm + (size_t)eo * R * SS + i) : (real)0;
      sPd[i] = mode == 2 ? __ldg(pm + (size_t)ed * R * SS + i) : (real)0;
    }
    __syncthreads();
    real c[S], vo[S];
    const int so = load_row<real, R, S>(p, o, s, r, c);
    if (o == INT32_MIN) {
#pragma unroll
      for (int i = 0; i < S; ++i) vo[i] = (real)1;
    } else {
      matvec<real, S>(sPo + r * SS, c, vo);
    }
    const int sd = d >= 0 ? __ldg(p.scaler + (size_t)d * p.n_patterns + s) : 0;
    const int sx = __ldg(p.scaler + (size_t)x * p.n_patterns + s);
    if (q == kb) sx_root = sx;
#pragma unroll
    for (int i = 0; i < S; ++i) u[i] = ScaleShift<real>::apply(O[i] * vo[i], sx - sd - so);
    if (mode == 2) {  // O = P_d^T u
      const real *Md = sPd + r * SS;
#pragma unroll
      for (int j = 0; j < S; ++j) {
        real a = (real)0;
#pragma unroll
        for (int i = 0; i < S; ++i) a = fma(Md[i * S + j], u[i], a);
        O[j] = a;
      }
    }
  }
  // the path ends at the op that takes e's message: u is the table row
  real *dst = static_cast<real *>(sp.table) + (((size_t)tb * p.n_patterns + s) * R + r) * S;
#pragma unroll
  for (int i = 0; i < S; i += 4) {
    if constexpr (sizeof(real) == 4)
      *reinterpret_cast<float4 *>(dst + i) = make_float4(u[i], u[i + 1], u[i + 2], u[i + 3]);
    else
      for (int j = 0; j < 4; ++j) dst[i + j] = u[i + j];
  }
  if (r == 0) sp.table_scaler[(size_t)tb * p.n_patterns + s] = sx_root;
}

// Evaluation of 20-state tables: thread = (pattern, rate), 256 per block;
// per child group P I, P' I, P'' I for the thread's rate, then per table the
// dot products with its row, summed over the R rate lanes, and the site
// terms (as the DNA evaluation) summed over the warp into
// partial[table][q][warp], warps of 32 / R patterns.
template <typename real, int R>
__global__ void __launch_bounds__(256) sumtable_eval20_kernel(const StabParams sp) {
  constexpr int S = 20, SS = S * S, ROWS = 256 / R;
  const TanParams &p = sp.t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  real *sM = reinterpret_cast<real *>(smem_raw);  // [3][R][S][S]
  const int r = threadIdx.x % R;
  const int64_t s = (int64_t)blockIdx.x * ROWS + threadIdx.x / R;
  const int part = p.block_part[(blockIdx.x * ROWS) / (kTanPPT * 256 / R)];
  const real *src = static_cast<const real *>(sp.pm3) + (size_t)part * 3 * R * SS;
  for (int i = threadIdx.x; i < 3 * R * SS; i += blockDim.x) sM[i] = src[i];
  __syncthreads();
  const double w = r == 0 ? __ldg(p.weights + s) : 0.0;
  const real iq = p.inv_term ? (real)p.inv_term[s] : (real)0;
  const int64_t n_warps = p.n_patterns * R / 32, gw = ((int64_t)blockIdx.x * 256 + threadIdx.x) / 32;
  const int tb_lo = blockIdx.y * sp.tables_per_block;
  const int tb_end = min(tb_lo + sp.tables_per_block, sp.n_tables);
  for (int g = 0; g < sp.n_groups; ++g) {
    const int g_lo = max(sp.group_begin[g], tb_lo), g_hi = min(sp.group_begin[g + 1], tb_end);
    if (g_lo >= g_hi) continue;  // uniform over the block
    real c[S], m0[S], m1[S], m2[S];
    load_row<real, R, S>(p, sp.group_ref[g], s, r, c);
    matvec<real, S>(sM + r * SS, c, m0);
    matvec<real, S>(sM + (R + r) * SS, c, m1);
    matvec<real, S>(sM + (2 * R + r) * SS, c, m2);
    for (int tb = g_lo; tb < g_hi; ++tb) {
      real o[S];
      ldg_row<real, S>(static_cast<const real *>(sp.table) + (((size_t)tb * p.n_patterns + s) * R + r) * S, o);
      real L = 0, L1 = 0, L2 = 0;
#pragma unroll
      for (int i = 0; i < S; ++i) {
        L = fma(o[i], m0[i], L);
        L1 = fma(o[i], m1[i], L1);
        L2 = fma(o[i], m2[i], L2);
      }
#pragma unroll
      for (int x = 1; x < R; x <<= 1) {
        L += __shfl_xor_sync(0xffffffffu, L, x);
        L1 += __shfl_xor_sync(0xffffffffu, L1, x);
        L2 += __shfl_xor_sync(0xffffffffu, L2, x);
      }
      const int k = __ldg(sp.table_scaler + (size_t)tb * p.n_patterns + s);
      sumtable_site_terms<real>(sp, tb, gw, n_warps, w, iq, k, L, L1, L2);
    }
  }
}

// out[(table * n_parts + part) * 3 + q] = compensated sum of the table's warp
// partials over the partition's warps: block (table, partition), warp q.
__global__ void __launch_bounds__(96) sumtable_reduce_kernel(const double *__restrict__ partial, int64_t n_warps,
                                                             const int32_t *__restrict__ part_warp_begin,
                                                             int n_parts, double *__restrict__ out, int ff) {
  const int tb = blockIdx.x, part = blockIdx.y, q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b0 = part_warp_begin[part], b1 = part_warp_begin[part + 1];
  const double *src = partial + ((size_t)tb * 3 + q) * n_warps;
  const float2 *src32 = reinterpret_cast<const float2 *>(src);
  double s = 0.0, c = 0.0;
  // eight loads in flight per lane before they are added (in a fixed order)
  for (int b = b0 + lane; b < b1; b += 32 * 8) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int i = b + 32 * u;
      v[u] = i < b1 ? (ff ? (double)src32[i].x + (double)src32[i].y : src[i]) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const double y = v[u] - c;
      const double t = s + y;
      c = (t - s) - y;
      s = t;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) out[((size_t)tb * n_parts + part) * 3 + q] = s;
}

template <typename real, int R, int S>
void run_sumtable(cudaStream_t st, const StabParams &p, const int32_t *level_begin, int n_levels) {
  // patterns per lane: two (two rows' loads in flight per op) once one per
  // lane gives more than about two waves of warps, else one (more warps)
  const int64_t warps1 = p.t.n_patterns * R / 32;
  if (warps1 > 2 * 152 * 24) {
    sumtable_walk_kernel<real, R, 2><<<(unsigned)((warps1 / 2 + 7) / 8), 256, 0, st>>>(p, level_begin[n_levels]);
  } else {
    sumtable_walk_kernel<real, R, 1><<<(unsigned)((warps1 + 7) / 8), 256, 0, st>>>(p, level_begin[n_levels]);
  }
}

template <typename real, int R, int S>
constexpr size_t eval_smem() {
  return eval_stages<real, R>() * (128 * R * S * sizeof(real) + 128 * 4) + 8 * eval_stages<real, R>() +
         3 * R * S * S * sizeof(real);
}

template <typename real, int R, int S>
void run_sumtable_eval(cudaStream_t st, const StabParams &p) {
  const size_t smem = eval_smem<real, R, S>();
  const unsigned ny = (unsigned)((p.n_tables + p.tables_per_block - 1) / p.tables_per_block);
  sumtable_eval_kernel<real, R, S><<<dim3((unsigned)(p.t.n_patterns / 128), ny), 128, smem, st>>>(p);
}

template <typename real>
bool dispatch_sumtable(cudaStream_t st, int R, int S, const StabParams &p, const int32_t *level_begin, int n_levels,
                       bool eval) {
  if (S != 4) return false;
  switch (R) {
    case 1: eval ? run_sumtable_eval<real, 1, 4>(st, p) : run_sumtable<real, 1, 4>(st, p, level_begin, n_levels); return true;
    case 2: eval ? run_sumtable_eval<real, 2, 4>(st, p) : run_sumtable<real, 2, 4>(st, p, level_begin, n_levels); return true;
    case 4: eval ? run_sumtable_eval<real, 4, 4>(st, p) : run_sumtable<real, 4, 4>(st, p, level_begin, n_levels); return true;
    case 8: eval ? run_sumtable_eval<real, 8, 4>(st, p) : run_sumtable<real, 8, 4>(st, p, level_begin, n_levels); return true;
    default: return false;
  }
}

template <typename real, int R, int S>
void run_levels(cudaStream_t st, const TanParams &p, const int32_t *level_begin, int n_levels) {
  const size_t smem = (3 * (size_t)R * S * S + S + R) * sizeof(real);
  for (int L = 0; L < n_levels; ++L) {
    const int n = level_begin[L + 1] - level_begin[L];
    if (n > 0) tangent_kernel<real, R, S><<<dim3(p.n_blocks, n), 256, smem, st>>>(p, level_begin[L]);
  }
}

template <typename real>
bool dispatch_levels(cudaStream_t st, int R, int S, const TanParams &p, const int32_t *level_begin, int n_levels) {
  // DNA runs the walk (tangent_walk_kernel); the level launches serve 20 states
  if (S == 20) {
    switch (R) {
      case 1: run_levels<real, 1, 20>(st, p, level_begin, n_levels); return true;
      case 2: run_levels<real, 2, 20>(st, p, level_begin, n_levels); return true;
      case 4: run_levels<real, 4, 20>(st, p, level_begin, n_levels); return true;
      default: return false;
    }
  }
  return false;
}

}  // namespace

int tangent_patterns_per_block(int R) { return kTanPPT * 256 / R; }

void launch_pderiv(cudaStream_t s, int n_parts, int R, int S, const double *lambda, const double *U,
                   const double *Uinv, const double *rates, const double *brlen, int len_stride, int edge,
                   double *out64, float *out32) {
  const int64_t total = (int64_t)n_parts * 2 * R * S * S;
  pderiv_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n_parts, R, S, lambda, U, Uinv, rates, brlen,
                                                                len_stride, edge, out64, out32);
  add_launches(1);
}

int tangent_walk_patterns_per_unit(int R) { return 32 / R; }

bool launch_tangent_walk(cudaStream_t s, int precision, int R, int S, const TanParams &p, int n_ops) {
  if (S != 4) return false;
  const int64_t n_units = p.n_patterns * R / 32;
  const unsigned grid = (unsigned)((n_units + 7) / 8);
  auto go = [&](auto kernel) { kernel<<<grid, 256, 0, s>>>(p, n_ops, n_units); };
  const bool f32 = precision == 1;
  switch (R) {
    case 1: f32 ? go(tangent_walk_kernel<float, 1, 1>) : go(tangent_walk_kernel<double, 1, 1>); break;
    case 2: f32 ? go(tangent_walk_kernel<float, 2, 1>) : go(tangent_walk_kernel<double, 2, 1>); break;
    case 4: f32 ? go(tangent_walk_kernel<float, 4, 1>) : go(tangent_walk_kernel<double, 4, 1>); break;
    case 8: f32 ? go(tangent_walk_kernel<float, 8, 1>) : go(tangent_walk_kernel<double, 8, 1>); break;
    default: return false;
  }
  add_launches(1);
  return true;
}

bool launch_tangent(cudaStream_t s, int precision, int R, int S, const TanParams &p, const int32_t *level_begin,
                    int n_levels) {
  const bool ok = precision == 1 ? dispatch_levels<float>(s, R, S, p, level_begin, n_levels)
                                 : dispatch_levels<double>(s, R, S, p, level_begin, n_levels);
  if (ok)
    for (int L = 0; L < n_levels; ++L) add_launches(level_begin[L + 1] > level_begin[L]);
  return ok;
}

void launch_tangent_reduce(cudaStream_t s, const TanParams &p, const int32_t *slots, int n_slots,
                           const int32_t *part_block_begin, int n_parts, double *out) {
  if (n_slots <= 0) return;
  tangent_reduce_kernel<<<dim3(n_slots, n_parts, 2), 128, 0, s>>>(p, slots, part_block_begin, n_parts, out);
  add_launches(1);
}

bool launch_sumtable_path20(cudaStream_t s, int precision, int R, const StabParams &p, int n_tab) {
  if (n_tab <= 0) return true;
  const dim3 grid((unsigned)(p.t.n_patterns * R / 256), (unsigned)n_tab);
  const size_t smem = (size_t)2 * R * 400 * (precision == 1 ? 4 : 8);
  if (precision == 1 && R == 4) sumtable_path20_kernel<float, 4><<<grid, 256, smem, s>>>(p);
  else if (precision == 1 && R == 2) sumtable_path20_kernel<float, 2><<<grid, 256, smem, s>>>(p);
  else if (precision == 1 && R == 1) sumtable_path20_kernel<float, 1><<<grid, 256, smem, s>>>(p);
  else if (precision != 1 && R == 4) sumtable_path20_kernel<double, 4><<<grid, 256, smem, s>>>(p);
  else if (precision != 1 && R == 2) sumtable_path20_kernel<double, 2><<<grid, 256, smem, s>>>(p);
  else if (precision != 1 && R == 1) sumtable_path20_kernel<double, 1><<<grid, 256, smem, s>>>(p);
  else return false;
  add_launches(1);
  return true;
}

bool launch_sumtable_build(cudaStream_t s, int precision, int R, int S, const StabParams &p,
                           const int32_t *level_begin, int n_levels) {
  const bool ok = precision == 1 ? dispatch_sumtable<float>(s, R, S, p, level_begin, n_levels, false)
                                 : dispatch_sumtable<double>(s, R, S, p, level_begin, n_levels, false);
  if (ok) add_launches(1);
  return ok;
}

bool sumtable_eval_setup(int precision, int R, int S) {
  if (S == 20) return R == 1 || R == 2 || R == 4;  // shared memory below 48 KB
  if (S != 4) return false;
  auto set = [](auto kernel, size_t smem) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
  };
  switch (R * 2 + (precision == 1)) {
    case 2: return set(sumtable_eval_kernel<double, 1, 4>, eval_smem<double, 1, 4>());
    case 3: return set(sumtable_eval_kernel<float, 1, 4>, eval_smem<float, 1, 4>());
    case 4: return set(sumtable_eval_kernel<double, 2, 4>, eval_smem<double, 2, 4>());
    case 5: return set(sumtable_eval_kernel<float, 2, 4>, eval_smem<float, 2, 4>());
    case 8: return set(sumtable_eval_kernel<double, 4, 4>, eval_smem<double, 4, 4>());
    case 9: return set(sumtable_eval_kernel<float, 4, 4>, eval_smem<float, 4, 4>());
    case 16: return set(sumtable_eval_kernel<double, 8, 4>, eval_smem<double, 8, 4>());
    case 17: return set(sumtable_eval_kernel<float, 8, 4>, eval_smem<float, 8, 4>());
    default: return false;
  }
}

bool launch_sumtable_eval(cudaStream_t s, int precision, int R, int S, const StabParams &p, int n_tab,
                          const int32_t *part_warp_begin, int n_parts, double *out) {
  if (n_tab <= 0) return true;
  bool ok;
  if (S == 20) {
    const unsigned ny = (unsigned)((p.n_tables + p.tables_per_block - 1) / p.tables_per_block);
    const dim3 grid((unsigned)(p.t.n_patterns * R / 256), ny);
    const size_t smem = (size_t)3 * R * 400 * (precision == 1 ? 4 : 8);
    ok = true;
    if (precision == 1 && R == 4) sumtable_eval20_kernel<float, 4><<<grid, 256, smem, s>>>(p);
    else if (precision == 1 && R == 2) sumtable_eval20_kernel<float, 2><<<grid, 256, smem, s>>>(p);
    else if (precision == 1 && R == 1) sumtable_eval20_kernel<float, 1><<<grid, 256, smem, s>>>(p);
    else if (precision != 1 && R == 4) sumtable_eval20_kernel<double, 4><<<grid, 256, smem, s>>>(p);
    else if (precision != 1 && R == 2) sumtable_eval20_kernel<double, 2><<<grid, 256, smem, s>>>(p);
    else if (precision != 1 && R == 1) sumtable_eval20_kernel<double, 1><<<grid, 256, smem, s>>>(p);
    else ok = false;
  } else {
    ok = precision == 1 ? dispatch_sumtable<float>(s, R, S, p, nullptr, 0, true)
                        : dispatch_sumtable<double>(s, R, S, p, nullptr, 0, true);
  }
  if (!ok) return false;
  const int64_t n_warps = S == 20 ? p.t.n_patterns * R / 32 : p.t.n_patterns / 32;
  sumtable_reduce_kernel<<<dim3(n_tab, n_parts), 96, 0, s>>>(p.partial, n_warps, part_warp_begin, n_parts, out,
                                                              precision == 1);
  add_launches(2);
  return true;
}

}  // namespace netlk
