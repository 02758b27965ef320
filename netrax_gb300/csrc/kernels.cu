// netlk device kernels (sm_103a).
//
// Layout in HBM (N = padded patterns over all partitions, R rate categories):
//   CLV of variant v:      clv[v][N][R][4]   (float or double, 16/32 B per (pattern, rate))
//   scale counter:         scaler[v][N]      (int32, cumulative over the subtree)
//   adjoint slot a:        adj[a][N][R][4]
//   tips:                  tips[tip][N]      (uint8 4-bit state masks)
//   P-matrices:            pmat[part][edge][R][4][4]
// A warp owns 32/R consecutive patterns (lane = pattern*R + rate) and walks
// the whole variant DAG for them: every (pattern, rate) value a lane reads in
// the forward and adjoint sweeps was written by that same lane, so the sweeps
// need no block- or grid-level synchronisation. Scaling decisions reduce over
// the R lanes of a pattern with shuffles; per-site log-likelihood and edge
// gradient sums reduce over the warp.
//
// Reference arithmetic restated (libpll is not vendored by NetRAX):
//   pll_update_partials_single   (called at src/likelihood/ImprovedLoglikelihood.cpp:145,185)
//   pll_compute_root_loglikelihood (src/likelihood/ImprovedLoglikelihood.cpp:450)
//   pllmod_treeinfo_update_prob_matrices (src/likelihood/ImprovedLoglikelihood.cpp:661)
//   AVERAGE / BEST mixing        (src/likelihood/ImprovedLoglikelihood.cpp:521-644)
#include <algorithm>
#include <cstdio>

#include "kernels.cuh"
#include "kernels_common.cuh"

namespace netlk {

static int64_t g_launches = 0;
int64_t launches_issued() { return g_launches; }
void add_launches(int64_t n) { g_launches += n; }

namespace {

// Loads one child operand for the lane's kPPL patterns: a variant CLV (with
// its scale counters), a tip (state mask expanded to 0/1) or the fake all-ones
// child. g0: the lane's first pattern, r: its rate; `stride` patterns
// separate the lane's patterns.
template <typename real, int R, int PPL>
__device__ __forceinline__ void load_child(const SweepParams &p, int32_t ref, size_t g0, int r, int stride,
                                           real (&c)[PPL][4], int (&s)[PPL]) {
  if (ref >= 0) {
    const real *clv = static_cast<const real *>(p.clv) + ((size_t)ref * p.n_patterns + g0) * (R * 4) + r * 4;
    const int32_t *sc = p.scaler + (size_t)ref * p.n_patterns + g0;
#pragma unroll
    for (int k = 0; k < PPL; ++k) {
      Vec<real>::load(clv + (size_t)k * stride * (R * 4), c[k]);
      s[k] = sc[(size_t)k * stride];
    }
  } else if (ref != INT32_MIN) {
    const uint8_t *t = p.tips + (size_t)(-1 - ref) * p.n_patterns + g0;
#pragma unroll
    for (int k = 0; k < PPL; ++k) {
      const unsigned code = t[(size_t)k * stride];
#pragma unroll
      for (int i = 0; i < 4; ++i) c[k][i] = (real)((code >> i) & 1u);
      s[k] = 0;
    }
  } else {
#pragma unroll
    for (int k = 0; k < PPL; ++k) {
#pragma unroll
      for (int i = 0; i < 4; ++i) c[k][i] = (real)1;
      s[k] = 0;
    }
  }
}

// Asks L2 for the lane's part of child `ref`'s CLV and scale counters (a
// variant only: tips are small and stay cached), ahead of their use by a
// later op of a walk.
template <typename real, int R, int PPL>
__device__ __forceinline__ void prefetch_child(const SweepParams &p, int32_t ref, size_t g0, int r, int stride) {
  if (ref < 0) return;
  const real *clv = static_cast<const real *>(p.clv) + ((size_t)ref * p.n_patterns + g0) * (R * 4) + r * 4;
#pragma unroll
  for (int k = 0; k < PPL; ++k) asm volatile("prefetch.global.L2 [%0];" ::"l"(clv + (size_t)k * stride * (R * 4)));
  if (r == 0) {
    const int32_t *sc = p.scaler + (size_t)ref * p.n_patterns + g0;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(sc));
  }
}

// FP32 mat-vecs on pairs of output states with paired FP32 instructions
// (FMUL2 / FFMA2; the input entry is broadcast to both halves of the pair),
// half the instructions of the scalar form and the same operation order:
// out_i = fma(M_i3, c_3, fma(M_i2, c_2, fma(M_i1, c_1, M_i0 c_0))).
// out[k] = M . c[k] with MT = M transposed (row j of MT = column j of M).
template <int PPL>
__device__ __forceinline__ void mv_pairs_cols(const float *MT, const float (&c)[PPL][4], float (&out)[PPL][4]) {
  float2 m01[4], m23[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float4 q = *reinterpret_cast<const float4 *>(MT + 4 * j);
    m01[j] = make_float2(q.x, q.y);
    m23[j] = make_float2(q.z, q.w);
  }
#pragma unroll
  for (int k = 0; k < PPL; ++k) {
    float2 a = __fmul2_rn(m01[0], make_float2(c[k][0], c[k][0]));
    float2 b = __fmul2_rn(m23[0], make_float2(c[k][0], c[k][0]));
#pragma unroll
    for (int j = 1; j < 4; ++j) {
      a = __ffma2_rn(m01[j], make_float2(c[k][j], c[k][j]), a);
      b = __ffma2_rn(m23[j], make_float2(c[k][j], c[k][j]), b);
    }
    out[k][0] = a.x;
    out[k][1] = a.y;
    out[k][2] = b.x;
    out[k][3] = b.y;
  }
}

// out[k] = M^T . u[k] with M row-major.
template <int PPL>
__device__ __forceinline__ void mv_pairs_rows_t(const float *M, const float (&u)[PPL][4], float (&out)[PPL][4]) {
  float2 m01[4], m23[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 q = *reinterpret_cast<const float4 *>(M + 4 * i);
    m01[i] = make_float2(q.x, q.y);
    m23[i] = make_float2(q.z, q.w);
  }
#pragma unroll
  for (int k = 0; k < PPL; ++k) {
    float2 a = __fmul2_rn(m01[0], make_float2(u[k][0], u[k][0]));
    float2 b = __fmul2_rn(m23[0], make_float2(u[k][0], u[k][0]));
#pragma unroll
    for (int i = 1; i < 4; ++i) {
      a = __ffma2_rn(m01[i], make_float2(u[k][i], u[k][i]), a);
      b = __ffma2_rn(m23[i], make_float2(u[k][i], u[k][i]), b);
    }
    out[k][0] = a.x;
    out[k][1] = a.y;
    out[k][2] = b.x;
    out[k][3] = b.y;
  }
}

// Staged P-matrix slices in shared memory. One slice per (child, rate),
// kRow values apart so the four rate groups of a warp's 16-byte loads hit
// distinct banks: FP64 holds P row-major (16 values + 2 padding); FP32 holds
// P row-major in [0, 16) and P transposed in [16, 32) (+ 4 padding), the two
// layouts the paired mat-vecs read.
template <typename real>
struct PLayout {
  static constexpr int kRow = (sizeof(real) == 4) ? 36 : 18;
  static constexpr int kT = (sizeof(real) == 4) ? 16 : 0;  // transposed copy (FP32)
};

// out[k] = P . c[k] for the lane's patterns; P: the lane's (child, rate)
// slice in shared memory.
template <typename real, int PPL>
__device__ __forceinline__ void matvec2_s(const real *P, const real (&c)[PPL][4], real (&out)[PPL][4]) {
  if constexpr (sizeof(real) == 4) {
    mv_pairs_cols<PPL>(P + PLayout<float>::kT, c, out);
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      real row[4];
      Vec<real>::load(P + 4 * i, row);
#pragma unroll
      for (int k = 0; k < PPL; ++k)
        out[k][i] = row[0] * c[k][0] + row[1] * c[k][1] + row[2] * c[k][2] + row[3] * c[k][3];
    }
  }
}

// out[k] = P^T . u[k], P: the lane's slice in shared memory.
template <typename real, int PPL>
__device__ __forceinline__ void matvec2_ts(const real *P, const real (&u)[PPL][4], real (&out)[PPL][4]) {
  if constexpr (sizeof(real) == 4) {
    mv_pairs_rows_t<PPL>(P, u, out);
  } else {
#pragma unroll
    for (int k = 0; k < PPL; ++k)
#pragma unroll
      for (int j = 0; j < 4; ++j) out[k][j] = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      real row[4];
      Vec<real>::load(P + 4 * i, row);
#pragma unroll
      for (int k = 0; k < PPL; ++k)
#pragma unroll
        for (int j = 0; j < 4; ++j) out[k][j] += row[j] * u[k][i];
    }
  }
}

// Stages the op's two P-matrices (all R rates) of one partition in the
// warp's own shared-memory slice: sP[(m*R + r)*kRow + 0..15], m = 0 for edge
// ea, 1 for edge eb (zero for the fake child). 2*R*16 values = one 16-byte
// load per lane at R = 4 in FP32; a __syncwarp (no block barrier) publishes them.
template <typename real, int R>
__device__ __forceinline__ void stage_pmats_warp(real *sP, const real *pm_part, int ea, int eb, int lane) {
  constexpr int V = 16 / sizeof(real);  // values per 16-byte vector
  constexpr int NV = 2 * R * 16 / V;
  constexpr int ROW = PLayout<real>::kRow;
  for (int i = lane; i < NV; i += 32) {
    const int m = (i * V) / (R * 16), j = i * V - m * (R * 16);
    const int rr = j / 16, c = j - rr * 16;
    real *dst = sP + (m * R + rr) * ROW + c;
    const int e = m ? eb : ea;
    if constexpr (sizeof(real) == 4) {
      // one row of P: row-major, and as a column of the transposed copy
      const float4 v = e >= 0 ? __ldg(reinterpret_cast<const float4 *>(pm_part + (size_t)e * (R * 16) + j))
                              : make_float4(0.f, 0.f, 0.f, 0.f);
      *reinterpret_cast<float4 *>(dst) = v;
      real *t = sP + (m * R + rr) * ROW + PLayout<real>::kT + c / 4;
      t[0] = v.x;
      t[4] = v.y;
      t[8] = v.z;
      t[12] = v.w;
    } else if (e >= 0) {
      *reinterpret_cast<double2 *>(dst) = __ldg(reinterpret_cast<const double2 *>(pm_part + (size_t)e * (R * 16) + j));
    } else {
#pragma unroll
      for (int q = 0; q < V; ++q) dst[q] = (real)0;
    }
  }
  __syncwarp();
}



// ------------------------------------------------------------------ forward
// The CLV (and scale counters) a walk's previous op left in registers, for a
// next op that has it as a child.
template <typename real, int PPL>
struct FwdCarry {
  real v[PPL][4];
  int s[PPL];
  int32_t var = INT32_MAX;  // variant held, INT32_MAX: none
};

// One op for one warp's unit of patterns: CLV_out = (P[ea] . a) * (P[eb] . b),
// rescaled per site; site log-likelihoods of displayed-tree root variants are
// summed over the warp's patterns into site_partial[slot][unit]. sP: the
// warp's shared-memory P staging slice. With CARRY, a child held in `carry`
// is taken from there instead of memory, and the result is left in it.
template <typename real, int R, int PPL, bool CARRY = false>
__device__ __forceinline__ void forward_op(const SweepParams &p, const FwdOp &op, int unit, real *sP, int lane,
                                           FwdCarry<real, PPL> *carry = nullptr) {
  constexpr int PPW = 32 / R;          // patterns per pass of the lane rows
  constexpr int UNIT = PPW * PPL;      // patterns per forward unit
  const int r = lane % R;
  const int pl = lane / R;
  // a warp covers UFW forward units (kPPLForward patterns per lane each)
  constexpr int UFW = PPL / kPPLForward;
  const int part = p.unit_part[unit * (PPL / kPPLBase)];
  const size_t N = (size_t)p.n_patterns;
  const size_t g0 = (size_t)unit * UNIT + pl;  // the lane's first pattern; the second is g0 + PPW
  real ca[PPL][4], cb[PPL][4];
  int sa[PPL], sb[PPL];
  if constexpr (CARRY) {
    auto take = [&](int32_t ref, real(&c)[PPL][4], int(&sc)[PPL]) {
      if (ref == carry->var) {
#pragma unroll
        for (int k = 0; k < PPL; ++k) {
#pragma unroll
          for (int i = 0; i < 4; ++i) c[k][i] = carry->v[k][i];
          sc[k] = carry->s[k];
        }
      } else {
        load_child<real, R, PPL>(p, ref, g0, r, PPW, c, sc);
      }
    };
    take(op.a, ca, sa);
    take(op.b, cb, sb);
  } else {
    load_child<real, R, PPL>(p, op.a, g0, r, PPW, ca, sa);
    load_child<real, R, PPL>(p, op.b, g0, r, PPW, cb, sb);
  }
  stage_pmats_warp<real, R>(sP, static_cast<const real *>(p.pmat) + (size_t)part * p.n_edges * (R * 16), op.ea,
                            op.b == INT32_MIN ? -1 : op.eb, lane);

  constexpr int ROW = PLayout<real>::kRow;
  real v[PPL][4];
  matvec2_s<real, PPL>(sP + r * ROW, ca, v);
  if (op.b != INT32_MIN) {
    real pb[PPL][4];
    matvec2_s<real, PPL>(sP + (R + r) * ROW, cb, pb);
#pragma unroll
    for (int k = 0; k < PPL; ++k)
#pragma unroll
      for (int i = 0; i < 4; ++i) v[k][i] *= pb[k][i];
  }
  real *dst = static_cast<real *>(p.clv) + ((size_t)op.out * N + g0) * (R * 4) + r * 4;
  int32_t *sdst = p.scaler + (size_t)op.out * N + g0;
  int s[PPL];
#pragma unroll
  for (int k = 0; k < PPL; ++k) {
    real m = max(max(v[k][0], v[k][1]), max(v[k][2], v[k][3]));
    m = rate_max<R>(m);
    s[k] = sa[k] + sb[k] + Scale<real>::rescale(m, v[k]);
    Vec<real>::store(dst + (size_t)k * PPW * (R * 4), v[k]);
    if (r == 0) sdst[(size_t)k * PPW] = s[k];
  }
  if constexpr (CARRY) {
#pragma unroll
    for (int k = 0; k < PPL; ++k) {
#pragma unroll
      for (int i = 0; i < 4; ++i) carry->v[k][i] = v[k][i];
      carry->s[k] = s[k];
    }
    carry->var = op.out;
  }
  if (op.slot >= 0) {
    // pll_compute_root_loglikelihood for the lane's sites, summed over the warp
    const real rw = model_val<real>(p.rate_weights, p.rate_weights32, part * R + r);
    real freq[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) freq[i] = model_val<real>(p.freqs, p.freqs32, part * 4 + i);
    SiteSum<real> ll;
#pragma unroll
    for (int k = 0; k < PPL; ++k) {
      real t = rw * (freq[0] * v[k][0] + freq[1] * v[k][1] + freq[2] * v[k][2] + freq[3] * v[k][3]);
      t = rate_sum<R>(t);
      if (r == 0) {
        if (p.inv_term)
          ll.add_inv(p, part, g0 + (size_t)k * PPW, t, s[k]);
        else
          ll.add(p, g0 + (size_t)k * PPW, t, s[k]);
      }
    }
    // the warp's first forward unit carries its sum, the others zero
    double *sp = p.site_partial + (size_t)op.slot * p.n_units_fwd + (size_t)unit * UFW;
    ll.store(sp, lane);
    if (lane == 0) {
#pragma unroll
      for (int k = 1; k < UFW; ++k) sp[k] = 0.0;
    }
  }
}

// One launch per DAG level: blockIdx.y picks the op of the level, each warp
// one unit of patterns.
template <typename real, int R, int THREADS, int MINB, int PPL>
__global__ void __launch_bounds__(THREADS, MINB) forward_kernel(const SweepParams p, int op_begin) {
  constexpr int WPB = THREADS / 32;
  __shared__ __align__(16) real sPw[WPB][2 * R * PLayout<real>::kRow];
  const int unit = blockIdx.x * WPB + (threadIdx.x >> 5);
  if (unit >= p.n_units_fwd / (PPL / kPPLForward)) return;  // whole warp
  forward_op<real, R, PPL>(p, load_fwd_op(p.fwd_ops, op_begin + blockIdx.y), unit, sPw[threadIdx.x >> 5],
                           threadIdx.x & 31);
}

// The whole sweep in one launch: each warp walks every op of walk_fwd_ops
// (a topological order chosen for cache locality) for its own unit. A lane
// only reads values it wrote itself, so no warp waits for another; a child
// CLV is read back soon after it was written, mostly from L2.
template <typename real, int R, int PPL>
__device__ __forceinline__ void forward_walk_unit(const SweepParams &p, int unit, real *sP, int lane) {
  constexpr int PPW = 32 / R;
  const size_t g0 = (size_t)unit * PPW * PPL + lane / R;
  const int n = p.n_walk_fwd;
  FwdCarry<real, PPL> carry;  // a parent right after its child reads it from here
  for (int i = 0; i < n; ++i) {
    int4 h = make_int4(-1, -1, -1, -1);
    if (i + 1 < n) h = __ldg(reinterpret_cast<const int4 *>(p.walk_fwd_ops + i + 1));  // out, a, b, ea
    __syncwarp();  // every lane is done with the previous op's P
    forward_op<real, R, PPL, true>(p, load_fwd_op(p.walk_fwd_ops, i), unit, sP, lane, &carry);
    // the next op's children are asked for in L2 as this op ends (a child
    // written long before, not the one just computed, may be in DRAM)
    prefetch_child<real, R, PPL>(p, h.y, g0, lane % R, PPW);
    prefetch_child<real, R, PPL>(p, h.z, g0, lane % R, PPW);
  }
}

template <typename real, int R, int THREADS, int MINB, int PPL>
__global__ void __launch_bounds__(THREADS, MINB) forward_walk_kernel(const SweepParams p, int unit_begin, int unit_end) {
  constexpr int WPB = THREADS / 32;
  __shared__ __align__(16) real sPw[WPB][2 * R * PLayout<real>::kRow];
  const int unit = unit_begin + blockIdx.x * WPB + (threadIdx.x >> 5);
  if (unit >= unit_end) return;  // whole warp
  forward_walk_unit<real, R, PPL>(p, unit, sPw[threadIdx.x >> 5], threadIdx.x & 31);
}

// ------------------------------------------------------------------ adjoint
// The partition's rate matrix, frequencies, rate weights and rates into a
// warp's shared-memory slice sQ: [0,16) Q (transposed in FP32), [16,20) pi,
// then R rate weights and R rates. Published by the next __syncwarp.
template <typename real, int R>
__device__ __forceinline__ void stage_model(const SweepParams &p, int part, real *sQ, int lane) {
  // FP32 keeps Q transposed (sQ[4j + i] = Q[i][j]) for the paired mat-vec
  if (lane < 16)
    sQ[lane] = model_val<real>(p.Q, p.Q32, part * 16 + (sizeof(real) == 4 ? (lane % 4) * 4 + lane / 4 : lane));
  if (lane < 4) sQ[16 + lane] = model_val<real>(p.freqs, p.freqs32, part * 4 + lane);
  if (lane < R) {
    sQ[20 + lane] = model_val<real>(p.rate_weights, p.rate_weights32, part * R + lane);
    sQ[20 + R + lane] = model_val<real>(p.rates, p.rates32, part * R + lane);
  }
}

// Values per warp in the model slice: Q, pi, R rate weights, R rates,
// rounded up to whole 16-byte vectors (the paired mat-vec reads Q's rows as
// float4 in every warp's slice).
template <int R>
struct ModelSlice {
  static constexpr int kSize = (16 + 4 + 2 * R + 3) / 4 * 4;
};

// q[k] = Q . x[k] with sQ as stage_model leaves it.
template <typename real, int PPL>
__device__ __forceinline__ void matvec_q(const real *sQ, const real (&x)[PPL][4], real (&q)[PPL][4]) {
  if constexpr (sizeof(real) == 4) {
    mv_pairs_cols<PPL>(sQ, x, q);
  } else {
#pragma unroll
    for (int k = 0; k < PPL; ++k)
#pragma unroll
      for (int i = 0; i < 4; ++i)
        q[k][i] = sQ[4 * i] * x[k][0] + sQ[4 * i + 1] * x[k][1] + sQ[4 * i + 2] * x[k][2] + sQ[4 * i + 3] * x[k][3];
  }
}

// Reverse sweep as message passing, one launch per level (deepest first).
// For op x with CLV_x = 2^k (Pa a) * (Pb b):
//   adj_x   = sum of incoming messages (+ seed: tree weight * w_s rw_r pi_i / L_s)
//   u_a     = 2^k adj_x * (Pb b),  u_b = 2^k adj_x * (Pa a)
//   dlogL/dt_ea += sum u_a . (r Q Pa a),  dlogL/dt_eb += sum u_b . (r Q Pb b)
//   message to a = Pa^T u_a, message to b = Pb^T u_b
// The two edge terms are summed over the block and written to
// grad_partial[op][blockIdx.x][2] for a deterministic reduction per edge.
// One adjoint op for one warp's unit. opi: the op's index in the level
// schedule (its grad_partial row); msg_slots: the schedule's message slot list.
// sP, sQ: the warp's shared-memory staging slices.
// Patterns per register group in the adjoint op: 4 where the launch shape
// leaves 128 or more registers per thread, else one base unit.
template <int THREADS, int MINB, int PPL>
struct AdjGroup {
  static constexpr int G = (65536 / (THREADS * MINB) >= 128 && PPL >= 4) ? 4 : kPPLBase;
};

// WALK: the walk schedule's op: model values already staged in sQ, and a
// message marked for the next op (out = -2) passed in `carry` (pad4 = 1:
// the op's adjoint starts from it).
template <typename real, int R, int PPL, int G, bool WALK = false>
__device__ __forceinline__ void backward_op(const SweepParams &p, const BwdOp &op, int opi,
                                            const int32_t *__restrict__ msg_slots, int unit, real *sP, real *sQ,
                                            int lane, real (&carry)[PPL][4]) {
  constexpr int PPW = 32 / R;
  constexpr int UNIT = PPW * PPL;      // patterns per adjoint unit
  // the lane's patterns are processed in groups of G (whole base units): the
  // op's decode and staging serve them all, registers hold one group
  static_assert(PPL % G == 0 && G % kPPLBase == 0, "whole groups of whole units");
  const int r = lane % R;
  const int pl = lane / R;
  // a warp covers UPU base units (kPPLBase patterns per lane each)
  constexpr int UPU = PPL / kPPLBase;
  real *sF = sQ + 16, *sRW = sQ + 20, *sRate = sQ + 20 + R;
  const bool fake = op.b == INT32_MIN;
  const int part = p.unit_part[unit * UPU];
  const size_t N = (size_t)p.n_patterns;
  const size_t g0 = (size_t)unit * UNIT + pl;
  const size_t lane_off = g0 * (R * 4) + r * 4;
  const real *clv = static_cast<const real *>(p.clv);
  real *msg = static_cast<real *>(p.msg);

  real ca[G][4], cb[G][4], ax[G][4], cx[G][4];
  int sa[G], sb[G], sx[G];
  // the group's children, counters, incoming messages (+ the message kept in
  // registers by the previous op) and, at a displayed-tree root, its own CLV
  auto load_group = [&](int grp) {
    const size_t gg = g0 + (size_t)grp * G * PPW;
    const size_t off = lane_off + (size_t)grp * G * PPW * (R * 4);
#pragma unroll
    for (int k = 0; k < G; ++k)
#pragma unroll
      for (int i = 0; i < 4; ++i) ax[k][i] = 0;
    if constexpr (WALK) {
      if (op.pad4) {
#pragma unroll
        for (int k = 0; k < G; ++k)
#pragma unroll
          for (int i = 0; i < 4; ++i) ax[k][i] += carry[grp * G + k][i];
      }
    }
    load_child<real, R, G>(p, op.a, gg, r, PPW, ca, sa);
    load_child<real, R, G>(p, op.b, gg, r, PPW, cb, sb);
    const int32_t *sxp = p.scaler + (size_t)op.x * N + gg;
#pragma unroll
    for (int k = 0; k < G; ++k) sx[k] = sxp[(size_t)k * PPW];
    for (int m = 0; m < op.msg_count; ++m) {
      int slot;
      if constexpr (WALK) slot = m == 0 ? op.msg0 : m == 1 ? op.msg1 : m == 2 ? op.msg2 : __ldg(msg_slots + op.msg_begin + m);
      else slot = __ldg(msg_slots + op.msg_begin + m);
      const real *src = msg + (size_t)slot * N * (R * 4) + off;
#pragma unroll
      for (int k = 0; k < G; ++k) {
        real t[4];
        Vec<real>::load(src + (size_t)k * PPW * (R * 4), t);
#pragma unroll
        for (int i = 0; i < 4; ++i) ax[k][i] += t[i];
      }
    }
    if (op.seed >= 0) {
      const real *cxp = clv + (size_t)op.x * N * (R * 4) + off;
#pragma unroll
      for (int k = 0; k < G; ++k) Vec<real>::load(cxp + (size_t)k * PPW * (R * 4), cx[k]);
    }
  };
  load_group(0);
  if (!WALK) stage_model<real, R>(p, part, sQ, lane);
  stage_pmats_warp<real, R>(sP, static_cast<const real *>(p.pmat) + (size_t)part * p.n_edges * (R * 16), op.ea,
                            fake ? -1 : op.eb, lane);  // its __syncwarp also publishes sQ

  const real rw = sRW[r];
  const real sd = op.seed >= 0 ? model_val<real>(p.seeds, p.seeds32, (size_t)op.seed * p.n_parts + part) : (real)0;
  const real *Pa = sP + r * PLayout<real>::kRow;
  const real *Pb = sP + (R + r) * PLayout<real>::kRow;
  // edge terms per base unit (patterns k < kPPLBase of the lane in unit 0,
  // the next kPPLBase in unit 1, ...): every launch shape sums them in the
  // same order, so the gradient does not depend on the shape
  real ga[UPU], gb[UPU];
#pragma unroll
  for (int u = 0; u < UPU; ++u) ga[u] = gb[u] = 0;
#pragma unroll
  for (int grp = 0; grp < PPL / G; ++grp) {
    if (grp > 0) load_group(grp);
    const size_t gg = g0 + (size_t)grp * G * PPW;
    const size_t off = lane_off + (size_t)grp * G * PPW * (R * 4);
    if (op.seed >= 0) {
      // d(w_s log L_s)/d clv_x = w_s rw_r pi_i / L_s, times the tree weight
#pragma unroll
      for (int k = 0; k < G; ++k) {
        real t = rw * (sF[0] * cx[k][0] + sF[1] * cx[k][1] + sF[2] * cx[k][2] + sF[3] * cx[k][3]);
        t = rate_sum<R>(t);
        const real sw = sd * pattern_weight<real>(p, gg + (size_t)k * PPW);
        if (t > (real)0 && sw != (real)0) {
          const real e = p.inv_term ? root_inv_term<real>(p, gg + (size_t)k * PPW, sx[k]) : (real)0;
          const real f = sw * rw / (t + e);
#pragma unroll
          for (int i = 0; i < 4; ++i) ax[k][i] += f * sF[i];
        }
      }
    }
    real pa[G][4], pb[G][4];
    matvec2_s<real, G>(Pa, ca, pa);
    if (!fake) {
      matvec2_s<real, G>(Pb, cb, pb);
    } else {
#pragma unroll
      for (int k = 0; k < G; ++k)
#pragma unroll
        for (int i = 0; i < 4; ++i) pb[k][i] = 1;
    }
    real ua[G][4], ub[G][4];
#pragma unroll
    for (int k = 0; k < G; ++k) {
      const int sh = sx[k] - sa[k] - sb[k];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        ua[k][i] = ax[k][i] * pb[k][i];
        ub[k][i] = ax[k][i] * pa[k][i];
      }
      if (sh != 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          ua[k][i] = Scale<real>::shift(ua[k][i], sh);
          ub[k][i] = Scale<real>::shift(ub[k][i], sh);
        }
      }
    }
    // d/dt of P(t r) c = r Q P(t r) c
    {
      real qa[G][4];
      matvec_q<real, G>(sQ, pa, qa);
#pragma unroll
      for (int k = 0; k < G; ++k)
#pragma unroll
        for (int i = 0; i < 4; ++i) ga[(grp * G + k) / kPPLBase] += ua[k][i] * qa[k][i];
      if (!fake) {
        real qb[G][4];
        matvec_q<real, G>(sQ, pb, qb);
#pragma unroll
        for (int k = 0; k < G; ++k)
#pragma unroll
          for (int i = 0; i < 4; ++i) gb[(grp * G + k) / kPPLBase] += ub[k][i] * qb[k][i];
      }
    }
    if (op.out_a >= 0) {
      real na[G][4];
      matvec2_ts<real, G>(Pa, ua, na);
      real *d = msg + (size_t)op.out_a * N * (R * 4) + off;
#pragma unroll
      for (int k = 0; k < G; ++k) Vec<real>::store(d + (size_t)k * PPW * (R * 4), na[k]);
    } else if constexpr (WALK) {
      if (op.out_a == -2) {
        real na[G][4];
        matvec2_ts<real, G>(Pa, ua, na);
#pragma unroll
        for (int k = 0; k < G; ++k)
#pragma unroll
          for (int i = 0; i < 4; ++i) carry[grp * G + k][i] = na[k][i];
      }
    }
    if (op.out_b >= 0) {
      real nb[G][4];
      matvec2_ts<real, G>(Pb, ub, nb);
      real *d = msg + (size_t)op.out_b * N * (R * 4) + off;
#pragma unroll
      for (int k = 0; k < G; ++k) Vec<real>::store(d + (size_t)k * PPW * (R * 4), nb[k]);
    } else if constexpr (WALK) {
      if (op.out_b == -2) {
        real nb[G][4];
        matvec2_ts<real, G>(Pb, ub, nb);
#pragma unroll
        for (int k = 0; k < G; ++k)
#pragma unroll
          for (int i = 0; i < 4; ++i) carry[grp * G + k][i] = nb[k][i];
      }
    }
  }
  // Every message slot is read by exactly one op, and the slot's next message
  // rewrites the warp's whole range of it, so once all lanes have read them
  // the incoming messages are dead: drop the warp's lines from L2 without
  // writing them back to DRAM. The range is UNIT * R * 4 reals at a multiple
  // of itself inside a slot of N * R * 4 reals (N is a multiple of 1024 / R
  // patterns), all multiples of 128 bytes.
  if (op.msg_count > 0) {
    constexpr int kBytes = UNIT * R * 4 * (int)sizeof(real);
    static_assert(kBytes % 128 == 0, "whole L2 lines per warp range");
    __syncwarp();
    for (int m = 0; m < op.msg_count; ++m) {
      int slot;
      if constexpr (WALK) slot = m == 0 ? op.msg0 : m == 1 ? op.msg1 : m == 2 ? op.msg2 : __ldg(msg_slots + op.msg_begin + m);
      else slot = __ldg(msg_slots + op.msg_begin + m);
      const char *base = reinterpret_cast<const char *>(msg + (size_t)slot * N * (R * 4)) + (size_t)unit * kBytes;
      for (int l = lane; l < kBytes / 128; l += 32)
        asm volatile("discard.global.L2 [%0], 128;" ::"l"(base + (size_t)l * 128) : "memory");
    }
  }
  // per-unit edge terms, reduced in a fixed order by op_reduce_kernel
  if constexpr (UPU == 1) {
    const real sa_ = warp_sum(ga[0] * sRate[r]);
    const real sb_ = warp_sum(gb[0] * sRate[r]);
    if (lane == 0) store_edge_terms<real>(p.grad_partial + ((size_t)opi * p.n_units + unit) * 2, sa_, sb_);
  } else {
    double *gp = p.grad_partial + ((size_t)opi * p.n_units + (size_t)unit * UPU) * 2;
#pragma unroll
    for (int u = 0; u < UPU; ++u) {
      const real sa_ = warp_sum(ga[u] * sRate[r]);
      const real sb_ = warp_sum(gb[u] * sRate[r]);
      if (lane == 0) store_edge_terms<real>(gp + 2 * u, sa_, sb_);
    }
  }
}

// One launch per level (deepest first): blockIdx.y picks the op.
template <typename real, int R, int THREADS, int MINB, int PPL>
__global__ void __launch_bounds__(THREADS, MINB) backward_kernel(const SweepParams p, int op_begin) {
  constexpr int WPB = THREADS / 32;
  __shared__ __align__(16) real sPw[WPB][2 * R * PLayout<real>::kRow];
  __shared__ __align__(16) real sQw[WPB][ModelSlice<R>::kSize];
  const int unit = blockIdx.x * WPB + (threadIdx.x >> 5);
  if (unit >= p.n_units / (PPL / kPPLBase)) return;  // whole warp
  const BwdOp op = load_bwd_op(p.bwd_ops, op_begin + blockIdx.y);
  real unused[PPL][4];  // the level schedule passes no message in registers
  // op.pad0: the op's grad_partial row (its index in the full schedule, also
  // when a subset of the ops is launched)
  backward_op<real, R, PPL, AdjGroup<THREADS, MINB, PPL>::G>(p, op, op.pad0, p.msg_slots, unit,
                                                             sPw[threadIdx.x >> 5], sQw[threadIdx.x >> 5],
                                                             threadIdx.x & 31, unused);
}

// The whole adjoint sweep in one launch: each warp walks walk_bwd_ops (the
// reverse of the forward walk, with its own message slots) for its unit. An
// op's level-schedule index (its grad_partial row) travels in pad0.
template <typename real, int R, int PPL, int G>
__device__ __forceinline__ void backward_walk_unit(const SweepParams &p, int unit, real *sP, real *sQ, int lane) {
  // a warp's patterns belong to one partition for the whole walk
  stage_model<real, R>(p, p.unit_part[unit * (PPL / kPPLBase)], sQ, lane);
  constexpr int PPW = 32 / R;
  const size_t g0 = (size_t)unit * PPW * PPL + lane / R;
  const int n = p.n_walk_bwd;
  real carry[PPL][4];  // a message passed to the next op in registers
  // the next op's children are asked for in L2 as each op ends (the first
  // op's before the loop)
  if (n > 0) {
    const int4 h = __ldg(reinterpret_cast<const int4 *>(p.walk_bwd_ops));  // x, a, b, ea
    prefetch_child<real, R, PPL>(p, h.y, g0, lane % R, PPW);
    prefetch_child<real, R, PPL>(p, h.z, g0, lane % R, PPW);
  }
  for (int i = 0; i < n; ++i) {
    int4 h = make_int4(-1, -1, -1, -1);
    if (i + 1 < n) h = __ldg(reinterpret_cast<const int4 *>(p.walk_bwd_ops + i + 1));
    __syncwarp();  // every lane is done with the previous op's staged values
    const BwdOp op = load_bwd_op<true>(p.walk_bwd_ops, i);
    backward_op<real, R, PPL, G, true>(p, op, op.pad0, p.walk_msg_slots, unit, sP, sQ, lane, carry);
    prefetch_child<real, R, PPL>(p, h.y, g0, lane % R, PPW);
    prefetch_child<real, R, PPL>(p, h.z, g0, lane % R, PPW);
  }
}

template <typename real, int R, int THREADS, int MINB, int PPL>
__global__ void __launch_bounds__(THREADS, MINB) backward_walk_kernel(const SweepParams p, int unit_begin,
                                                                       int unit_end) {
  constexpr int WPB = THREADS / 32;
  __shared__ __align__(16) real sPw[WPB][2 * R * PLayout<real>::kRow];
  __shared__ __align__(16) real sQw[WPB][ModelSlice<R>::kSize];
  const int unit = unit_begin + blockIdx.x * WPB + (threadIdx.x >> 5);
  if (unit >= unit_end) return;  // whole warp
  backward_walk_unit<real, R, PPL, AdjGroup<THREADS, MINB, PPL>::G>(p, unit, sPw[threadIdx.x >> 5],
                                                                    sQw[threadIdx.x >> 5], threadIdx.x & 31);
}

// ------------------------------------------------------------- P-matrices
// P(t r) = U diag(exp(lambda r t)) U^-1 in FP64; a zero length gives the
// identity. One thread per entry of pmat[part][edge][rate][S][S].
// len_stride: 0 when every partition shares the lengths brlen[e] (linked),
// n_edges when partition p has its own, brlen[p * n_edges + e].
__device__ __forceinline__ void pmatrix_entry(int64_t idx, int n_parts, int n_edges, int R, int S,
                                              const double *__restrict__ lambda, const double *__restrict__ U,
                                              const double *__restrict__ Uinv, const double *__restrict__ rates,
                                              const double *__restrict__ brlen, double *__restrict__ pmat64,
                                              float *__restrict__ pmat32, int len_stride = 0) {
  const int SS = S * S;
  const int64_t total = (int64_t)n_parts * n_edges * R * SS;
  if (idx >= total) return;
  const int ij = (int)(idx % SS);
  const int i = ij / S, j = ij - i * S;
  const int64_t q = idx / SS;  // (part, edge, rate)
  const int rr = (int)(q % R);
  const int e = (int)(q / R % n_edges);
  const int part = (int)(q / R / n_edges);
  const double len = brlen[(size_t)part * len_stride + e];
  const double t = len * rates[part * R + rr];
  double v;
  if (len == 0.0) {
    v = (i == j) ? 1.0 : 0.0;
  } else {
    v = 0.0;
    for (int k = 0; k < S; ++k)
      v += U[(size_t)part * SS + i * S + k] * exp(lambda[part * S + k] * t) * Uinv[(size_t)part * SS + k * S + j];
  }
  pmat64[idx] = v;
  if (pmat32) pmat32[idx] = (float)v;
}

__global__ void pmatrix_kernel(int n_parts, int n_edges, int R, int S, const double *__restrict__ lambda,
                               const double *__restrict__ U, const double *__restrict__ Uinv,
                               const double *__restrict__ rates, const double *__restrict__ brlen,
                               double *__restrict__ pmat64, float *__restrict__ pmat32, int len_stride) {
  pmatrix_entry((int64_t)blockIdx.x * blockDim.x + threadIdx.x, n_parts, n_edges, R, S, lambda, U, Uinv, rates,
                brlen, pmat64, pmat32, len_stride);
}

// ------------------------------------------ per-(tree, partition) site sums
// Deterministic compensated (Kahan) FP64 sum of the per-unit partials.
__device__ __forceinline__ void tree_reduce_block(const MixParams &m, int slot, int part) {
  const int ub = m.parts[part].unit_begin, ue = m.parts[part].unit_end;
  const double *src = m.site_partial + (size_t)slot * m.n_units;
  const float2 *src32 = reinterpret_cast<const float2 *>(src);
  double s = 0.0, c = 0.0;
  for (int u = ub + threadIdx.x; u < ue; u += blockDim.x) {
    const double y = (m.ff ? ff_to_double(src32[u]) : src[u]) - c;
    const double t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) m.tree_logl[(size_t)slot * m.n_parts + part] = red[0];
}

__global__ void tree_reduce_kernel(const MixParams m) { tree_reduce_block(m, blockIdx.x, blockIdx.y); }

// --------------------------------------------------------------- mixture
// AVERAGE: logL_p = log sum_T P(T) L_{T,p} (max-shifted); BEST: max_T.
// Posterior tree weights become the adjoint seeds; the reticulation gradient
// is sum_p sum_T w_{T,p} d log P(T) / d p_k.
// Mixture, one warp per partition (partitions p = warp, warp + 8, ...):
// per partition the best root (ties to the lower index), AVERAGE = max-shifted
// log-sum-exp over the roots with log P(T) >= min_logprob, BEST = the max;
// posterior weights w[p][root], the adjoint seeds per slot, and the partition's
// d logL / d p_k partials; then thread 0 adds the partitions in index order.
// All sums use fixed shuffle trees, so results do not depend on scheduling.
__device__ __forceinline__ void mix_block(const MixParams &m) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
  for (int part = warp; part < m.n_parts; part += n_warps) {
    double *wts = m.weights + (size_t)part * m.n_roots;
    double best = -INFINITY;
    int arg = 0x7fffffff;
    for (int i = lane; i < m.n_roots; i += 32) {
      if (m.root_logprob[i] < m.min_logprob) continue;
      const double v = m.root_logprob[i] + m.tree_logl[(size_t)m.root_slot[i] * m.n_parts + part];
      if (v > best || (v == best && i < arg)) {
        best = v;
        arg = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double b = __shfl_xor_sync(0xffffffffu, best, o);
      const int ib = __shfl_xor_sync(0xffffffffu, arg, o);
      if (b > best || (b == best && ib < arg)) {
        best = b;
        arg = ib;
      }
    }
    double lp;
    if (m.variant == 0) {  // AVERAGE
      double acc = 0.0;
      for (int i = lane; i < m.n_roots; i += 32) {
        if (m.root_logprob[i] < m.min_logprob) continue;
        acc += exp(m.root_logprob[i] + m.tree_logl[(size_t)m.root_slot[i] * m.n_parts + part] - best);
      }
      acc = warp_sum(acc);
      lp = best + log(acc);
      for (int i = lane; i < m.n_roots; i += 32)
        wts[i] = (m.root_logprob[i] < m.min_logprob)
                     ? 0.0
                     : exp(m.root_logprob[i] + m.tree_logl[(size_t)m.root_slot[i] * m.n_parts + part] - lp);
    } else {  // BEST
      lp = best;
      for (int i = lane; i < m.n_roots; i += 32) wts[i] = (i == arg) ? 1.0 : 0.0;
    }
    __syncwarp();
    if (lane == 0) m.out[2 + part] = lp;
    for (int sl = lane; sl < m.n_slots; sl += 32) {
      double sum = 0.0;
      for (int q = m.slot_begin[sl]; q < m.slot_begin[sl + 1]; ++q) sum += wts[m.slot_roots[q]];
      m.seeds[(size_t)sl * m.n_parts + part] = sum;
      if (m.seeds32) m.seeds32[(size_t)sl * m.n_parts + part] = (float)sum;
    }
    // d logL_p / d p_k = sum_T w_T d log P(T) / d p_k, 8 reticulations per pass
    for (int k0 = 0; k0 < m.n_ret; k0 += 8) {
      double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int i = lane; i < m.n_roots; i += 32) {
        const double w = wts[i];
        if (w == 0.0) continue;
        const double *d = m.root_dlogprob + (size_t)i * m.n_ret;
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (k0 + j < m.n_ret) acc[j] += w * d[k0 + j];
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const double v = warp_sum(acc[j]);
        if (lane == 0 && k0 + j < m.n_ret) m.dret_part[(size_t)part * m.n_ret + k0 + j] = v;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double total = 0.0;
    for (int p = 0; p < m.n_parts; ++p) total += m.out[2 + p];
    for (int k = 0; k < m.n_ret; ++k) {
      double sum = 0.0;
      for (int p = 0; p < m.n_parts; ++p) sum += m.dret_part[(size_t)p * m.n_ret + k];
      m.out[2 + m.n_parts + k] = sum;
    }
    m.out[0] = total;
    m.out[1] = (isfinite(total) ? 0.0 : 1.0);
  }
}

__global__ void mix_kernel(const MixParams m) { mix_block(m); }

// Gradient reduction in two fixed-order stages: per adjoint op, the block
// partials of its launch (grid_partial[op][b][side]) -> op_sum[op][side];
// then per edge e, the op sides that use it (CSR edge_entries[edge_begin[e] ..
// edge_begin[e+1]) = op * 2 + side) -> d logL / d t_e.
// ff: each partial is a pair of float pairs (FP32 sweeps), else two doubles.
__device__ __forceinline__ void op_reduce_block(int op, int n_bx, const double *__restrict__ partial,
                                                double *__restrict__ op_sum, int ff) {
  __shared__ double ra[128], rb[128];
  const double2 *src = reinterpret_cast<const double2 *>(partial) + (size_t)op * n_bx;
  const float4 *src32 = reinterpret_cast<const float4 *>(src);
  double a = 0.0, b = 0.0;
  if (ff) {
    // float-float sums (about 48 bits; no FP64 instruction per element: GB300
    // runs FP64 at a small fraction of its FP32 rate), one double per thread
    FF fa{0.f, 0.f}, fb{0.f, 0.f};
    for (int i = threadIdx.x; i < n_bx; i += blockDim.x) {
      const float4 v = src32[i];
      fa = ff_add(fa, FF{v.x, v.y});
      fb = ff_add(fb, FF{v.z, v.w});
    }
    a = ff_to_double(make_float2(fa.hi, fa.lo));
    b = ff_to_double(make_float2(fb.hi, fb.lo));
  } else {
    for (int i = threadIdx.x; i < n_bx; i += blockDim.x) {
      const double2 v = src[i];
      a += v.x;
      b += v.y;
    }
  }
  ra[threadIdx.x] = a;
  rb[threadIdx.x] = b;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      ra[threadIdx.x] += ra[threadIdx.x + o];
      rb[threadIdx.x] += rb[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    op_sum[2 * op] = ra[0];
    op_sum[2 * op + 1] = rb[0];
  }
}

__global__ void op_reduce_kernel(int n_bx, const double *__restrict__ partial, double *__restrict__ op_sum,
                                 int ff) {
  op_reduce_block(blockIdx.x, n_bx, partial, op_sum, ff);
}

__global__ void edge_reduce_kernel(int n_edges, const int32_t *__restrict__ edge_begin,
                                   const int32_t *__restrict__ edge_entries, const double *__restrict__ op_sum,
                                   double *__restrict__ grad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_edges) return;
  double s = 0.0;
  for (int q = edge_begin[e]; q < edge_begin[e + 1]; ++q) s += op_sum[edge_entries[q]];
  grad[e] = s;
}

// Launch shapes (threads per block, minimum resident blocks per SM) the
// autotuner chooses from. Shape 0 is the default and exists for every
// precision and rate count; the FP32 4-rate path (DNA GTR+G4) carries all.
// Shapes 5-7 and 10-11 give the adjoint four patterns per lane (two base
// units per warp) and shapes 8-9 eight (the forward sweep keeps four: eight
// measured slower on the DNA workloads), which amortises an op's decode and P staging
// over more patterns at the cost of registers (occupancy); their edge terms
// are still summed per 16-pattern unit, so every shape gives the same bits.
struct Shape {
  int threads, minb, forward_ppl, adjoint_ppl;
};
constexpr Shape kShapes[] = {{256, 4, 4, 2}, {128, 8, 4, 2}, {256, 3, 4, 2}, {128, 6, 4, 2}, {64, 12, 4, 2},
                             {256, 2, 4, 4}, {128, 4, 4, 4}, {64, 8, 4, 4},  {128, 2, 4, 8}, {64, 4, 4, 8},
                             {32, 16, 4, 4}, {64, 6, 4, 4}};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

template <typename real, int R, int T, int M, int FPPL, int BPPL>
struct FwdRun {
  static int run(cudaStream_t s, const SweepParams &p, const int32_t *level_begin, int n_levels) {
    const int warps = p.n_units_fwd / (FPPL / kPPLForward);
    const int bx = (warps + T / 32 - 1) / (T / 32);
    for (int L = 0; L < n_levels; ++L) {
      const int n = level_begin[L + 1] - level_begin[L];
      if (n > 0) forward_kernel<real, R, T, M, FPPL><<<dim3(bx, n), T, 0, s>>>(p, level_begin[L]);
    }
    return 0;
  }
};
template <typename real, int R, int T, int M, int FPPL, int BPPL>
struct BwdRun {
  static int run(cudaStream_t s, const SweepParams &p, const int32_t *level_begin, int n_levels) {
    const int warps = p.n_units / (BPPL / kPPLBase);
    const int bx = (warps + T / 32 - 1) / (T / 32);
    for (int L = 0; L < n_levels; ++L) {
      const int n = level_begin[L + 1] - level_begin[L];
      if (n > 0) backward_kernel<real, R, T, M, BPPL><<<dim3(bx, n), T, 0, s>>>(p, level_begin[L]);
    }
    return 0;
  }
};
// Walk sweeps run every op in one launch per warp, so a warp that starts in a
// later wave than the others would run a whole sweep alone: the units are cut
// into chunks of at most one wave (every warp resident) of nearly equal size,
// one launch each.
template <class K>
int walk_chunks(K kernel, int threads, int warps) {
  int dev = 0, sms = 1, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
  const int wave = std::max(1, per_sm * sms * (threads / 32));
  return std::max(1, (warps + wave - 1) / wave);
}
template <class K>
int launch_walk_chunks(K kernel, int threads, int warps, cudaStream_t s, const SweepParams &p, bool count_only) {
  const int wpb = threads / 32;
  const int n_chunks = walk_chunks(kernel, threads, warps);
  if (count_only) return n_chunks;
  const int per = (warps + n_chunks - 1) / n_chunks;
  for (int c = 0; c < n_chunks; ++c) {
    const int b = c * per, e = std::min(warps, b + per);
    kernel<<<(e - b + wpb - 1) / wpb, threads, 0, s>>>(p, b, e);
  }
  return n_chunks;
}
template <typename real, int R, int T, int M, int FPPL, int BPPL>
struct FwdWalkRun {
  static int run(cudaStream_t s, const SweepParams &p, bool count_only) {
    return launch_walk_chunks(forward_walk_kernel<real, R, T, M, FPPL>, T, p.n_units_fwd / (FPPL / kPPLForward), s, p,
                              count_only);
  }
};
template <typename real, int R, int T, int M, int FPPL, int BPPL>
struct BwdWalkRun {
  static int run(cudaStream_t s, const SweepParams &p, bool count_only) {
    return launch_walk_chunks(backward_walk_kernel<real, R, T, M, BPPL>, T, p.n_units / (BPPL / kPPLBase), s, p,
                              count_only);
  }
};
template <typename real, int R, int T, int M, int FPPL, int BPPL>
struct ThreadsRun {
  static int run() { return T; }
};

// Calls F<real, R, threads, minb>::run for a runtime (precision, R, shape).
template <template <typename, int, int, int, int, int> class F, class... A>
int dispatch(int precision, int R, int shape, A &&...a) {
  if (precision == 1 && R == 4) {
    switch (shape) {
      case 1: return F<float, 4, 128, 8, 4, 2>::run(a...);
      case 2: return F<float, 4, 256, 3, 4, 2>::run(a...);
      case 3: return F<float, 4, 128, 6, 4, 2>::run(a...);
      case 4: return F<float, 4, 64, 12, 4, 2>::run(a...);
      case 5: return F<float, 4, 256, 2, 4, 4>::run(a...);
      case 6: return F<float, 4, 128, 4, 4, 4>::run(a...);
      case 7: return F<float, 4, 64, 8, 4, 4>::run(a...);
      case 8: return F<float, 4, 128, 2, 4, 8>::run(a...);
      case 9: return F<float, 4, 64, 4, 4, 8>::run(a...);
      case 10: return F<float, 4, 32, 16, 4, 4>::run(a...);
      case 11: return F<float, 4, 64, 6, 4, 4>::run(a...);
      default: return F<float, 4, 256, 4, 4, 2>::run(a...);
    }
  }
  if (precision == 1) {
    switch (R) {
      case 1: return F<float, 1, 256, 4, 4, 2>::run(a...);
      case 2: return F<float, 2, 256, 4, 4, 2>::run(a...);
      default: return F<float, 8, 256, 4, 4, 2>::run(a...);
    }
  }
  switch (R) {
    case 1: return F<double, 1, 256, 2, 4, 2>::run(a...);
    case 2: return F<double, 2, 256, 2, 4, 2>::run(a...);
    case 4: return F<double, 4, 256, 2, 4, 2>::run(a...);
    default: return F<double, 8, 256, 2, 4, 2>::run(a...);
  }
}

// Walk shapes (one warp per block, so a chunk spreads evenly over the SMs):
// {threads, minimum blocks per SM, forward and adjoint patterns per lane}.
constexpr Shape kWalkShapes[] = {{32, 32, 4, 2}, {32, 24, 4, 2}, {32, 16, 4, 4}, {32, 19, 4, 4}, {32, 20, 4, 4}};
constexpr int kNumWalkShapes = sizeof(kWalkShapes) / sizeof(kWalkShapes[0]);

template <template <typename, int, int, int, int, int> class F, class... A>
int dispatch_walk(int w, A &&...a) {
  switch (w) {
    case 1: return F<float, 4, 32, 24, 4, 2>::run(a...);
    case 2: return F<float, 4, 32, 16, 4, 4>::run(a...);
    case 3: return F<float, 4, 32, 19, 4, 4>::run(a...);
    case 4: return F<float, 4, 32, 20, 4, 4>::run(a...);
    default: return F<float, 4, 32, 32, 4, 2>::run(a...);
  }
}

// ---------------------------------------------------- persistent batches
// The candidates of a search move in a handful of launches: every warp of a
// persistent grid takes (candidate, unit) items from a counter, LPT order
// (the candidates with the longest walks first), and walks that candidate's
// whole DAG for its unit - the single-context walk, with the candidate's
// parameters copied into shared memory. No warp waits for another.
__device__ __forceinline__ void load_params(const SweepParams *src, SweepParams *dst, int lane) {
  static_assert(sizeof(SweepParams) % 16 == 0 && alignof(SweepParams) <= 16, "copied as int4 words");
  const int4 *a = reinterpret_cast<const int4 *>(src);
  int4 *d = reinterpret_cast<int4 *>(dst);
  for (int i = lane; i < (int)(sizeof(SweepParams) / 16); i += 32) d[i] = a[i];
  __syncwarp();
}

__device__ __forceinline__ int next_item(const BatchParams &b, int lane) {
  int it = 0;
  if (lane == 0) it = atomicAdd(b.counter, 1);
  return __shfl_sync(kFull, it, 0);
}

template <typename real, int R, int THREADS, int MINB, int PPL>
__global__ void __launch_bounds__(THREADS, MINB) forward_walk_batch_kernel(const BatchParams b) {
  constexpr int WPB = THREADS / 32;
  __shared__ __align__(16) real sPw[WPB][2 * R * PLayout<real>::kRow];
  __shared__ __align__(16) SweepParams sp[WPB];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int item = next_item(b, lane); item < b.n_items; item = next_item(b, lane)) {
    const int2 it = b.items[item];
    __syncwarp();  // the previous item is done with sp and sP
    load_params(&b.cands[it.x].sweep, &sp[w], lane);
    forward_walk_unit<real, R, PPL>(sp[w], it.y, sPw[w], lane);
  }
}

template <typename real, int R, int THREADS, int MINB, int PPL>
__global__ void __launch_bounds__(THREADS, MINB) backward_walk_batch_kernel(const BatchParams b) {
  constexpr int WPB = THREADS / 32;
  __shared__ __align__(16) real sPw[WPB][2 * R * PLayout<real>::kRow];
  __shared__ __align__(16) real sQw[WPB][ModelSlice<R>::kSize];
  __shared__ __align__(16) SweepParams sp[WPB];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int item = next_item(b, lane); item < b.n_items; item = next_item(b, lane)) {
    const int2 it = b.items[item];
    __syncwarp();
    load_params(&b.cands[it.x].sweep, &sp[w], lane);
    backward_walk_unit<real, R, PPL, AdjGroup<THREADS, MINB, PPL>::G>(sp[w], it.y, sPw[w], sQw[w], lane);
  }
}

__global__ void pmatrix_batch_kernel(const BatchParams b) {
  const BatchCand &c = b.cands[blockIdx.y];
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= c.n_pmat) return;
  pmatrix_entry(idx, c.n_parts, c.n_edges, 4, 4, c.lambda, c.U, c.Uinv, c.rates, c.brlen, c.pmat64, c.pmat32);
}

__global__ void tree_reduce_batch_kernel(const BatchParams b) {
  const MixParams &m = b.cands[blockIdx.z].mix;
  if ((int)blockIdx.x >= m.n_slots || (int)blockIdx.y >= m.n_parts) return;  // whole block
  tree_reduce_block(m, blockIdx.x, blockIdx.y);
}

__global__ void mix_batch_kernel(const BatchParams b) { mix_block(b.cands[blockIdx.x].mix); }

__global__ void op_reduce_batch_kernel(const BatchParams b) {
  const BatchCand &c = b.cands[blockIdx.y];
  if ((int)blockIdx.x >= c.n_ops) return;  // whole block
  op_reduce_block(blockIdx.x, c.n_bx, c.grad_partial, c.op_sum, 1);
}

__global__ void edge_reduce_batch_kernel(const BatchParams b) {
  const BatchCand &c = b.cands[blockIdx.y];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= c.n_edges) return;
  double s = 0.0;
  for (int q = c.edge_begin[e]; q < c.edge_begin[e + 1]; ++q) s += c.op_sum[c.edge_entries[q]];
  c.grad[e] = s;
  b.results[c.result_offset + c.n_out + e] = s;
}

__global__ void gather_out_batch_kernel(const BatchParams b) {
  const BatchCand &c = b.cands[blockIdx.x];
  for (int i = threadIdx.x; i < c.n_out; i += blockDim.x) b.results[c.result_offset + i] = c.out[i];
}

template <typename real, int R, int T, int M, int FPPL, int BPPL>
struct FwdBatchRun {
  static int run(cudaStream_t s, const BatchParams &b) {
    auto k = forward_walk_batch_kernel<real, R, T, M, FPPL>;
    int dev = 0, sms = 1, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, T, 0);
    const int grid = std::max(1, std::min(per_sm * sms, (b.n_items + T / 32 - 1) / (T / 32)));
    k<<<grid, T, 0, s>>>(b);
    return 1;
  }
};
template <typename real, int R, int T, int M, int FPPL, int BPPL>
struct BwdBatchRun {
  static int run(cudaStream_t s, const BatchParams &b) {
    auto k = backward_walk_batch_kernel<real, R, T, M, BPPL>;
    int dev = 0, sms = 1, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, T, 0);
    const int grid = std::max(1, std::min(per_sm * sms, (b.n_items + T / 32 - 1) / (T / 32)));
    k<<<grid, T, 0, s>>>(b);
    return 1;
  }
};
template <typename real, int R, int T, int M, int FPPL, int BPPL>
struct BwdPplRun {
  static int run() { return BPPL; }
};

}  // namespace

int num_batch_shapes() { return kNumWalkShapes; }
int batch_shape_bwd_ppl(int shape) { return dispatch_walk<BwdPplRun>(shape); }

void launch_batch_forward(cudaStream_t s, const BatchParams &b, int shape) {
  pmatrix_batch_kernel<<<dim3((unsigned)((b.max_pmat + 255) / 256), b.n_cands), 256, 0, s>>>(b);
  cudaMemsetAsync(b.counter, 0, 4, s);
  g_launches += 1 + dispatch_walk<FwdBatchRun>(shape, s, b);
  tree_reduce_batch_kernel<<<dim3(b.max_slots, b.max_parts, b.n_cands), 256, 0, s>>>(b);
  mix_batch_kernel<<<b.n_cands, 256, 0, s>>>(b);
  g_launches += 2;
}

void launch_batch_backward(cudaStream_t s, const BatchParams &b, int shape) {
  cudaMemsetAsync(b.counter, 0, 4, s);
  g_launches += dispatch_walk<BwdBatchRun>(shape, s, b);
  op_reduce_batch_kernel<<<dim3(std::max(1, b.max_ops), b.n_cands), 128, 0, s>>>(b);
  edge_reduce_batch_kernel<<<dim3((b.max_edges + 127) / 128, b.n_cands), 128, 0, s>>>(b);
  gather_out_batch_kernel<<<b.n_cands, 64, 0, s>>>(b);
  g_launches += 3;
}

int num_level_shapes(int precision, int R) { return (precision == 1 && R == 4) ? kNumShapes : 1; }
int num_shapes(int precision, int R) { return (precision == 1 && R == 4) ? kNumShapes + kNumWalkShapes : 1; }

int sweep_launches(int precision, int R, int shape, const SweepParams &p, bool backward, const int32_t *level_begin,
                   int n_levels) {
  const int nl = num_level_shapes(precision, R);
  if (shape >= nl)
    return backward ? dispatch_walk<BwdWalkRun>(shape - nl, cudaStream_t(nullptr), p, true)
                    : dispatch_walk<FwdWalkRun>(shape - nl, cudaStream_t(nullptr), p, true);
  int n = 0;
  for (int L = 0; L < n_levels; ++L) n += level_begin[L + 1] > level_begin[L];
  return n;
}

int shape_threads(int precision, int R, int shape) {
  const int nl = num_level_shapes(precision, R);
  return shape >= nl ? kWalkShapes[shape - nl].threads : dispatch<ThreadsRun>(precision, R, shape);
}

void launch_forward(cudaStream_t s, int precision, int R, int shape, const SweepParams &p,
                    const int32_t *level_begin, int n_levels) {
  const int nl = num_level_shapes(precision, R);
  if (shape >= nl) {
    g_launches += dispatch_walk<FwdWalkRun>(shape - nl, s, p, false);
    return;
  }
  dispatch<FwdRun>(precision, R, shape, s, p, level_begin, n_levels);
  for (int L = 0; L < n_levels; ++L) g_launches += level_begin[L + 1] > level_begin[L];
}

void launch_backward(cudaStream_t s, int precision, int R, int shape, const SweepParams &p,
                     const int32_t *level_begin, int n_levels) {
  const int nl = num_level_shapes(precision, R);
  if (shape >= nl) {
    g_launches += dispatch_walk<BwdWalkRun>(shape - nl, s, p, false);
    return;
  }
  dispatch<BwdRun>(precision, R, shape, s, p, level_begin, n_levels);
  for (int L = 0; L < n_levels; ++L) g_launches += level_begin[L + 1] > level_begin[L];
}

void launch_pmatrix(cudaStream_t s, int n_parts, int n_edges, int R, int S, const double *lambda, const double *U,
                    const double *Uinv, const double *rates, const double *brlen, double *pmat64,
                    float *pmat32, int len_stride) {
  const int64_t total = (int64_t)n_parts * n_edges * R * S * S;
  pmatrix_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n_parts, n_edges, R, S, lambda, U, Uinv, rates,
                                                                 brlen, pmat64, pmat32, len_stride);
  g_launches++;
}

// Per-partition gradient (for branch lengths that differ between partitions):
// per adjoint op and partition, the edge terms of the partition's units
// (base units [unit_begin, unit_end)) in a fixed order -> op_sum[op][part][2];
// per edge and partition, the op sides that use the edge -> grad[part][edge].
__global__ void op_reduce_part_kernel(int n_units, const double *__restrict__ partial,
                                      const int32_t *__restrict__ part_unit_begin, int n_parts,
                                      double *__restrict__ op_sum, int ff) {
  const int op = blockIdx.x, part = blockIdx.y;
  const int ub = part_unit_begin[part], ue = part_unit_begin[part + 1];
  __shared__ double ra[128], rb[128];
  const double2 *src = reinterpret_cast<const double2 *>(partial) + (size_t)op * n_units;
  const float4 *src32 = reinterpret_cast<const float4 *>(src);
  double a = 0.0, b = 0.0;
  if (ff) {
    FF fa{0.f, 0.f}, fb{0.f, 0.f};
    for (int i = ub + threadIdx.x; i < ue; i += blockDim.x) {
      const float4 v = src32[i];
      fa = ff_add(fa, FF{v.x, v.y});
      fb = ff_add(fb, FF{v.z, v.w});
    }
    a = ff_to_double(make_float2(fa.hi, fa.lo));
    b = ff_to_double(make_float2(fb.hi, fb.lo));
  } else {
    for (int i = ub + threadIdx.x; i < ue; i += blockDim.x) {
      const double2 v = src[i];
      a += v.x;
      b += v.y;
    }
  }
  ra[threadIdx.x] = a;
  rb[threadIdx.x] = b;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      ra[threadIdx.x] += ra[threadIdx.x + o];
      rb[threadIdx.x] += rb[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    op_sum[((size_t)op * n_parts + part) * 2] = ra[0];
    op_sum[((size_t)op * n_parts + part) * 2 + 1] = rb[0];
  }
}

__global__ void edge_reduce_part_kernel(int n_edges, int n_parts, const int32_t *__restrict__ edge_begin,
                                        const int32_t *__restrict__ edge_entries, const double *__restrict__ op_sum,
                                        double *__restrict__ grad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x, part = blockIdx.y;
  if (e >= n_edges) return;
  double s = 0.0;
  for (int q = edge_begin[e]; q < edge_begin[e + 1]; ++q) {
    const int entry = edge_entries[q];  // op * 2 + side
    s += op_sum[((size_t)(entry >> 1) * n_parts + part) * 2 + (entry & 1)];
  }
  grad[(size_t)part * n_edges + e] = s;
}

void launch_grad_reduce_partitions(cudaStream_t s, int n_ops, int n_edges, int n_units, int n_parts,
                                   const int32_t *part_unit_begin, const int32_t *edge_begin,
                                   const int32_t *edge_entries, const double *partial, double *op_sum,
                                   double *grad, bool ff) {
  if (n_ops > 0) op_reduce_part_kernel<<<dim3(n_ops, n_parts), 128, 0, s>>>(n_units, partial, part_unit_begin,
                                                                              n_parts, op_sum, ff ? 1 : 0);
  edge_reduce_part_kernel<<<dim3((n_edges + 127) / 128, n_parts), 128, 0, s>>>(n_edges, n_parts, edge_begin,
                                                                              edge_entries, op_sum, grad);
  g_launches += 2;
}

void launch_tree_reduce(cudaStream_t s, const MixParams &m) {
  dim3 grid(m.n_slots, m.n_parts);
  tree_reduce_kernel<<<grid, 256, 0, s>>>(m);
  g_launches++;
}

void launch_mix(cudaStream_t s, const MixParams &m) {
  mix_kernel<<<1, 256, 0, s>>>(m);
  g_launches++;
}

void launch_grad_reduce(cudaStream_t s, int n_ops, int n_edges, int n_bx, const int32_t *edge_begin,
                        const int32_t *edge_entries, const double *partial, double *op_sum, double *grad,
                        bool ff) {
  op_reduce_kernel<<<n_ops, 128, 0, s>>>(n_bx, partial, op_sum, ff ? 1 : 0);
  edge_reduce_kernel<<<(n_edges + 127) / 128, 128, 0, s>>>(n_edges, edge_begin, edge_entries, op_sum, grad);
  g_launches += 2;
}

}  // namespace netlk
