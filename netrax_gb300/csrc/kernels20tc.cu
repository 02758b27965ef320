// Tensor-core forward sweep for 20-state partitions with 4 rate categories,
// FP32 CLVs (tcgen05, kind::tf32, accumulators in TMEM).
//
// Per op and tile of 128 patterns (the MMA's M), child c's contribution for
// rate r is the GEMM D[128 x 20] = A[128 x 20] . P_r^T with A the child's CLV
// rows. The CLV tile [128 patterns][4 rates x 20 states] is already K-major:
// rate r's operand is columns 20r..20r+19 of it. K runs in steps of 8, so
// rate r reads columns 20r..20r+23 and B's columns 20..23 are zero (the four
// extra A columns are the next rate's first states, or a zero pad chunk).
//
// FP32 accuracy from TF32 inputs (3xTF32): every operand x = hi + lo with hi
// = x rounded to TF32 and lo = x - hi rounded to TF32. One N=64 MMA computes
// A_hi . [B_hi | B_lo] into columns [0, 64) and one N=32 MMA adds A_lo . B_hi
// into columns [0, 32); the epilogue adds column i and 32 + i. Tip children
// are exact 0/1 rows and need no lo part.
//
// A CTA (one per SM) walks a contiguous range of (op, tile) items; 256
// threads split the child tiles into shared memory, one thread issues the
// MMAs while all threads fetch the next item's tiles, and 8 warps
// read TMEM (warp w: patterns 32(w%4)..+31, rates 2(w/4) and 2(w/4)+1),
// multiply the children, rescale and store. TMEM: 512 columns, child c rate r
// at column 256c + 64r, so the kernel runs one CTA per SM (its shared memory
// allows no more).
#include "kernels.cuh"
#include "kernels_common.cuh"
#include "tc.cuh"

namespace netlk {
namespace {

constexpr int kTM = 128;                       // patterns per tile
constexpr int kTThreads = 256;
constexpr int kAChunk = kTM * 16 + 16;         // one 4-column slab of a tile (+16 B: bank spread)
constexpr int kAChunks = 21;                   // 80 columns + one zero slab
constexpr int kABytes = kAChunks * kAChunk;    // 43344
constexpr int kBChunk = 64 * 16;               // 64 B rows (hi 0-31, lo 32-63) x 4 columns
constexpr int kBBytes = 6 * kBChunk;           // K = 24
constexpr int kSmemA = 4 * kABytes;            // [child][hi, lo]
constexpr int kOutRow = 336;                   // staged output row: 320 B + 16 B bank spread
static_assert(kTM * kOutRow <= kABytes, "output staging fits one A tile");
constexpr int kSmemB = 8 * kBBytes;            // [child][rate]
constexpr int kSmemMisc = 16 + 4 * kTM * 4;    // mbarrier, TMEM address, two exchange arrays
constexpr int kSmemBytes = kSmemA + kSmemB + kSmemMisc;
static_assert(kSmemBytes <= 232448, "shared memory of one CTA");

constexpr uint32_t kIdN64 = tc::idesc_tf32(128, 64);
constexpr uint32_t kIdN32 = tc::idesc_tf32(128, 32);

// Child kinds: absent (the fake all-ones child), tip (0/1 rows), inner (CLV).
enum { kAbsent = 0, kTip = 1, kInner = 2 };

__device__ __forceinline__ int child_kind(int32_t ref) {
  return ref >= 0 ? kInner : (ref == INT32_MIN ? kAbsent : kTip);
}

// TF32 split with round-to-nearest parts: x = hi + lo, |lo| <= 2^-12 |x|, and
// lo itself rounded to TF32 (so the tensor core reads both exactly).
__device__ __forceinline__ void split4(const float4 &x, float4 &hi, float4 &lo) {
  hi = make_float4(tc::tf32_rna(x.x), tc::tf32_rna(x.y), tc::tf32_rna(x.z), tc::tf32_rna(x.w));
  lo = make_float4(tc::tf32_rna(x.x - hi.x), tc::tf32_rna(x.y - hi.y), tc::tf32_rna(x.z - hi.z), tc::tf32_rna(x.w - hi.w));
}

// Stages P_r (20x20, row = output state) of both children as B tiles: row
// n < 20 holds hi(P[n][k]), row 32 + n holds lo(P[n][k]). Rows 20-31, 52-63
// and columns 20-23 stay zero from the kernel's start.
__device__ __forceinline__ void stage_b(const SweepParams &p, unsigned char *sB, int part, int ea, int eb) {
  const float4 *pm = reinterpret_cast<const float4 *>(static_cast<const float *>(p.pmat) +
                                                      (size_t)part * p.n_edges * 1600);
  float4 v[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int f = threadIdx.x + u * kTThreads, c = f / 400, e = c ? eb : ea;
    if (f < 800 && e >= 0) v[u] = __ldg(pm + (size_t)e * 400 + (f - c * 400));
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int f = threadIdx.x + u * kTThreads, c = f / 400, e = c ? eb : ea;
    if (f >= 800 || e < 0) continue;
    const int rem = f - c * 400, r = rem / 100, e2 = rem - r * 100, i = e2 / 5, j4 = e2 - i * 5;
    unsigned char *base = sB + (c * 4 + r) * kBBytes + j4 * kBChunk + (i & 7) * 16;
    float4 hi, lo;
    split4(v[u], hi, lo);
    *reinterpret_cast<float4 *>(base + (i >> 3) * 128) = hi;
    *reinterpret_cast<float4 *>(base + (4 + (i >> 3)) * 128) = lo;
  }
}

// Issues the global loads of child `ref` of tile g0 into registers: CLV
// float4s for an inner child, the tip's state masks (in .x) for a tip.
__device__ __forceinline__ void fetch(const SweepParams &p, int kind, int32_t ref, size_t g0, float4 (&x)[10]) {
  const size_t N = (size_t)p.n_patterns;
  if (kind == kInner) {
    const float4 *src = reinterpret_cast<const float4 *>(static_cast<const float *>(p.clv) + ((size_t)ref * N + g0) * 80);
#pragma unroll
    for (int i = 0; i < 10; ++i) x[i] = __ldg(src + threadIdx.x + i * kTThreads);
  } else if (kind == kTip) {
    const uint32_t *code = p.tips32 + (size_t)(-1 - ref) * N + g0;
#pragma unroll
    for (int i = 0; i < 10; ++i) x[i].x = __uint_as_float(__ldg(code + (threadIdx.x + i * kTThreads) / 20));
  }
}

// Writes fetched registers into the A tiles: split hi/lo for an inner child,
// 0/1 expansion of the mask (columns 4kc.. = rate kc/5, states 4(kc%5)..) for a tip.
__device__ __forceinline__ void put(int kind, const float4 (&x)[10], unsigned char *sAh, unsigned char *sAl) {
  if (kind == kInner) {
#pragma unroll
    for (int i = 0; i < 10; ++i) {
      const int f = threadIdx.x + i * kTThreads, m = f / 20, kc = f - m * 20, off = kc * kAChunk + m * 16;
      float4 hi, lo;
      split4(x[i], hi, lo);
      *reinterpret_cast<float4 *>(sAh + off) = hi;
      *reinterpret_cast<float4 *>(sAl + off) = lo;
    }
  } else if (kind == kTip) {
#pragma unroll
    for (int i = 0; i < 10; ++i) {
      const int f = threadIdx.x + i * kTThreads, m = f / 20, kc = f - m * 20;
      const uint32_t b = __float_as_uint(x[i].x) >> (4 * (kc % 5));
      *reinterpret_cast<float4 *>(sAh + kc * kAChunk + m * 16) =
          make_float4((float)(b & 1u), (float)((b >> 1) & 1u), (float)((b >> 2) & 1u), (float)((b >> 3) & 1u));
    }
  }
}

// Reads the 20 states of one (child, rate) accumulator for this lane's
// pattern: columns i (hi . B_hi + lo . B_hi) plus 32 + i (hi . B_lo).
__device__ __forceinline__ void read_d(uint32_t t, float (&v)[20]) {
  uint32_t a[16], b[4], c[16], d[4];
  tc::ld16(t, a);
  tc::ld4(t + 16, b);
  tc::ld16(t + 32, c);
  tc::ld4(t + 48, d);
  tc::ld_wait();
  tc::ld_fence(a);
  tc::ld_fence(b);
  tc::ld_fence(c);
  tc::ld_fence(d);
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(a[i]) + __uint_as_float(c[i]);
#pragma unroll
  for (int i = 0; i < 4; ++i) v[16 + i] = __uint_as_float(b[i]) + __uint_as_float(d[i]);
}

// Persistent over the level: CTA b takes work items [b W / G, (b+1) W / G)
// of the W = ops x tiles items (item = op * n_tiles + tile), so consecutive
// items share the op and its staged B tiles. The next item's child tiles are
// fetched into registers while the current item's MMAs and epilogue run.
__global__ void __launch_bounds__(kTThreads, 1)
    forward20_tc_kernel(const SweepParams p, int op_begin, int n_ops, int n_tiles) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *sA = smem;
  unsigned char *sB = smem + kSmemA;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sB + kSmemB);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sB + kSmemB + 8);
  float *s_max = reinterpret_cast<float *>(sB + kSmemB + 16);  // [2][128]
  float *s_t = s_max + 2 * kTM;                                 // [2][128]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t N = (size_t)p.n_patterns;
  const long long W = (long long)n_ops * n_tiles;
  const int item_begin = (int)(W * blockIdx.x / gridDim.x), item_end = (int)(W * (blockIdx.x + 1) / gridDim.x);

  if (warp == 0) tc::tmem_alloc(tc::smem_u32(tmem_slot), 512);
  if (threadIdx.x == 0) tc::mbar_init(tc::smem_u32(mbar), 2);
  // zero slab 20 of every A tile (rate 3's last K step reads it) and all of B
  for (int i = threadIdx.x; i < 4 * kTM; i += kTThreads)
    *reinterpret_cast<float4 *>(sA + (i / kTM) * kABytes + 20 * kAChunk + (i % kTM) * 16) = make_float4(0, 0, 0, 0);
  for (int i = threadIdx.x; i < kSmemB / 16; i += kTThreads)
    reinterpret_cast<float4 *>(sB)[i] = make_float4(0, 0, 0, 0);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  const int q = warp & 3, h = warp >> 2;
  const int m = 32 * q + lane;
  const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
  int staged_op = -1, staged_part = -1;
  uint32_t phase = 0;
  bool failed = false;

  int oi = item_begin / n_tiles;
  FwdOp op = load_fwd_op(p.fwd_ops, op_begin + oi);
  int ka = child_kind(op.a), kb = child_kind(op.b);
  float4 xa[10], xb[10];
  // partitions are padded to whole 256-pattern blocks: a tile has one partition
  int part_next = 0;
  if (item_begin < item_end) {
    const size_t g0 = (size_t)(item_begin - oi * n_tiles) * kTM;
    fetch(p, ka, op.a, g0, xa);
    fetch(p, kb, op.b, g0, xb);
    part_next = p.unit_part[g0 / 16];
  }
  for (int item = item_begin; item < item_end; ++item) {
    const int tile = item - oi * n_tiles;
    const size_t g0 = (size_t)tile * kTM;
    const int part = part_next;
    if (oi != staged_op || part != staged_part) {
      stage_b(p, sB, part, op.ea, kb == kAbsent ? -1 : op.eb);
      staged_op = oi;
      staged_part = part;
    }
    put(ka, xa, sA, sA + kABytes);
    put(kb, xb, sA + 2 * kABytes, sA + 3 * kABytes);
    tc::fence_proxy_async();
    __syncthreads();
    // child c's MMAs are issued by thread 32c (one per warp of warps 0-1):
    // their accumulators are disjoint, and each issuer commits its own
    // MMAs to the mbarrier (two arrivals per item)
    if ((threadIdx.x & 31) == 0 && threadIdx.x < 64) {
      const int c = threadIdx.x >> 5;
      const int kind = c ? kb : ka;
      tc::fence_after_sync();
      if (kind != kAbsent) {
        // descriptors of the tiles' first slabs; a K step adds its byte offset / 16
        const uint64_t dah = tc::smem_desc(tc::smem_u32(sA + (2 * c) * kABytes), kAChunk, 128);
        const uint64_t dal = dah + (kABytes >> 4);
        const uint64_t db = tc::smem_desc(tc::smem_u32(sB + (c * 4) * kBBytes), kBChunk, 128);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const uint32_t d = tmem + 256 * c + 64 * r;
#pragma unroll
          for (int s = 0; s < 3; ++s) {
            const uint32_t ko = ((5 * r + 2 * s) * kAChunk) >> 4;
            const uint64_t bd = db + ((r * kBBytes + 2 * s * kBChunk) >> 4);
            tc::mma_tf32(d, dah + ko, bd, kIdN64, s > 0);
            if (kind == kInner) tc::mma_tf32(d, dal + ko, bd, kIdN32, 1);
          }
        }
      }
      tc::commit(tc::smem_u32(mbar));  // arrives at once when this thread issued nothing
    }
    // the current item's op, for the epilogue; then prefetch the next item
    const FwdOp cur = op;
    const int cka = ka, ckb = kb;
    const size_t g = g0 + m;
    const int sab = (cka == kInner ? p.scaler[(size_t)cur.a * N + g] : 0) +
                    (ckb == kInner ? p.scaler[(size_t)cur.b * N + g] : 0);
    const float2 wg = p.weights32[g];
    if (item + 1 < item_end) {
      const int noi = (item + 1) / n_tiles;
      if (noi != oi) {
        oi = noi;
        op = load_fwd_op(p.fwd_ops, op_begin + oi);
        ka = child_kind(op.a);
        kb = child_kind(op.b);
      }
      const size_t gn = (size_t)(item + 1 - oi * n_tiles) * kTM;
      fetch(p, ka, op.a, gn, xa);
      fetch(p, kb, op.b, gn, xb);
      part_next = p.unit_part[gn / 16];
    }
    const bool ok = tc::mbar_wait(tc::smem_u32(mbar), phase);
    phase ^= 1;
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    tc::fence_after_sync();

    // ------------------------------------------------------------ epilogue
    float v[2][20];
    float mx = 0.f;
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
      const int r = 2 * h + rr;
      read_d(lane_base + 64 * r, v[rr]);
      if (ckb != kAbsent) {
        float w[20];
        read_d(lane_base + 256 + 64 * r, w);
#pragma unroll
        for (int i = 0; i < 20; ++i) v[rr][i] *= w[i];
      }
#pragma unroll
      for (int i = 0; i < 20; ++i) mx = fmaxf(mx, v[rr][i]);
    }
    s_max[h * kTM + m] = mx;
    __syncthreads();
    mx = fmaxf(s_max[m], s_max[kTM + m]);
    int sc = sab;
    if (mx < 0x1p-32f && mx > 0.0f) {
      int e;
      frexpf(mx, &e);
#pragma unroll
      for (int rr = 0; rr < 2; ++rr)
#pragma unroll
        for (int i = 0; i < 20; ++i) v[rr][i] = ldexpf(v[rr][i], -e);
      sc -= e;
    }
    // output tile through shared memory (child a's hi tile is free now): rows
    // of kOutRow bytes, so the 8 lanes of a 16-byte store phase hit distinct banks
    {
      unsigned char *row = sA + m * kOutRow + 160 * h;
#pragma unroll
      for (int j = 0; j < 10; ++j) {
        const int rr = j / 5, i = 4 * (j % 5);
        *reinterpret_cast<float4 *>(row + 16 * j) = make_float4(v[rr][i], v[rr][i + 1], v[rr][i + 2], v[rr][i + 3]);
      }
    }
    if (h == 0) p.scaler[(size_t)cur.out * N + g] = sc;
    if (cur.slot >= 0) {
      float t = 0.f;
#pragma unroll
      for (int rr = 0; rr < 2; ++rr) {
        float u = 0.f;
#pragma unroll
        for (int i = 0; i < 20; ++i) u += p.freqs32[part * 20 + i] * v[rr][i];
        t += p.rate_weights32[part * 4 + 2 * h + rr] * u;
      }
      s_t[h * kTM + m] = t;
      __syncthreads();
      if (h == 0) {
        SiteSum<float> ll;
        if (p.inv_term32)
          ll.add_inv_w(wg, s_t[m] + s_t[kTM + m], sc, p.gamma_frac32[part], p.inv_term32[g]);
        else
          ll.add_w(wg, s_t[m] + s_t[kTM + m], sc);
        ll.store(p.site_partial + (size_t)cur.slot * p.n_units_fwd + g0 / 32 + q, lane);
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    {  // coalesced copy of the staged tile: 128 rows x 320 contiguous bytes in the CLV
      float4 *dst = reinterpret_cast<float4 *>(static_cast<float *>(p.clv) + ((size_t)cur.out * N + g0) * 80);
#pragma unroll
      for (int i = 0; i < 10; ++i) {
        const int f = threadIdx.x + i * kTThreads, r = f / 20;
        dst[f] = *reinterpret_cast<const float4 *>(sA + r * kOutRow + (f - r * 20) * 16);
      }
    }
    __syncthreads();
    // the staging rows overlap the tile's zero slab: clear it again
    if (threadIdx.x < (kTM * kOutRow - 20 * kAChunk) / 16)
      *reinterpret_cast<float4 *>(sA + 20 * kAChunk + 16 * threadIdx.x) = make_float4(0, 0, 0, 0);
  }
  if (failed) {
    if (threadIdx.x == 0) atomicExch(p.fault, 1);
    // the MMAs may still run: give them one more bounded wait before TMEM is released
    tc::mbar_wait(tc::smem_u32(mbar), phase ^ 1);
    __syncthreads();
  }
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_free(tmem, 512);
}

// ------------------------------------------------------------------ adjoint
// Per op and tile of 128 patterns, for each half of the rates (2 rates):
//   round 1: D = c . [P_r | Q] for both children (c = child CLV rows; Q is
//            the rate matrix, the same for every edge and rate), giving
//            p = P_r c and Q c in TMEM;
//   epilogue 1: u_a = 2^sh adj_x (*) p_b, u_b = 2^sh adj_x (*) p_a (adj_x =
//            the sum of x's incoming messages + the displayed-tree seed);
//   round 2: D = u . P_r (the messages P_r^T u);
//   epilogue 2: edge terms rate_r (P_r^T u) . (Q c) = rate_r u . (Q P_r c)
//            (P_r = exp(Q t r) commutes with Q), and the messages go to the
//            children's slots.
// TMEM: child c, local rate l at column 256c + 128l: [0,64) p (or the message
// in round 2), [64,128) Q c. A tiles hold one rate half (40 columns + a zero
// slab); B tiles hold P_r (rows = output state), Q, and P_r^T for all rates.
constexpr int kHChunks = 11;
constexpr int kHBytes = kHChunks * kAChunk;            // 22704
constexpr int kBwdA = 4 * kHBytes;                     // [child][hi, lo]
constexpr int kBwdB1 = 8 * kBBytes;                    // [child][rate] P_r
constexpr int kBwdB2 = 8 * kBBytes;                    // [child][rate] P_r^T
constexpr int kStageRow = 176;                         // staged message row: 160 B + 16 B bank spread
constexpr int kBwdMisc = 16 + 4 * 2 * kTM * 4;         // mbarrier, TMEM address, 4 exchange arrays [2][128]
constexpr int kBwdSmem = kBwdA + kBwdB1 + kBBytes + kBwdB2 + kBwdMisc;
static_assert(2 * kTM * kStageRow <= kBwdA, "message staging fits the A tiles");
static_assert(kBwdSmem <= 232448, "shared memory of one CTA");

// B tiles of the adjoint: P_r (as the forward) and P_r^T (row n = j, column
// k = i holds P_r[i][j]) of both children, and Q when `with_q`.
__device__ __forceinline__ void stage_b_adj(const SweepParams &p, unsigned char *sB1, unsigned char *sBQ,
                                            unsigned char *sB2, int part, int ea, int eb, bool with_q) {
  const float4 *pm = reinterpret_cast<const float4 *>(static_cast<const float *>(p.pmat) +
                                                      (size_t)part * p.n_edges * 1600);
  float4 v[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int f = threadIdx.x + u * kTThreads, c = f / 400, e = c ? eb : ea;
    if (f < 800 && e >= 0) v[u] = __ldg(pm + (size_t)e * 400 + (f - c * 400));
  }
  if (with_q && threadIdx.x < 100) {  // Q[i][4 j4 .. 4 j4 + 3]
    const int i = threadIdx.x / 5, j4 = threadIdx.x - i * 5;
    const float4 x = __ldg(reinterpret_cast<const float4 *>(p.Q32 + (size_t)part * 400 + i * 20 + 4 * j4));
    float4 hi, lo;
    split4(x, hi, lo);
    unsigned char *base = sBQ + j4 * kBChunk + (i & 7) * 16;
    *reinterpret_cast<float4 *>(base + (i >> 3) * 128) = hi;
    *reinterpret_cast<float4 *>(base + (4 + (i >> 3)) * 128) = lo;
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int f = threadIdx.x + u * kTThreads, c = f / 400, e = c ? eb : ea;
    if (f >= 800 || e < 0) continue;
    const int rem = f - c * 400, r = rem / 100, e2 = rem - r * 100, i = e2 / 5, j4 = e2 - i * 5;
    float4 hi, lo;
    split4(v[u], hi, lo);
    unsigned char *base = sB1 + (c * 4 + r) * kBBytes + j4 * kBChunk + (i & 7) * 16;
    *reinterpret_cast<float4 *>(base + (i >> 3) * 128) = hi;
    *reinterpret_cast<float4 *>(base + (4 + (i >> 3)) * 128) = lo;
    // transposed: rows n = 4 j4 + t, column k = i
    unsigned char *tb = sB2 + (c * 4 + r) * kBBytes + (i >> 2) * kBChunk + (i & 3) * 4;
    const float h4[4] = {hi.x, hi.y, hi.z, hi.w}, l4[4] = {lo.x, lo.y, lo.z, lo.w};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int n = 4 * j4 + t;
      *reinterpret_cast<float *>(tb + (n >> 3) * 128 + (n & 7) * 16) = h4[t];
      *reinterpret_cast<float *>(tb + ((32 + n) >> 3) * 128 + (n & 7) * 16) = l4[t];
    }
  }
}

// Child rows of one rate half (columns 40h .. 40h+39) into registers: CLV
// float4s of an inner child, the state masks (in .x) of a tip. Both
// children are fetched before either is stored, so their loads overlap.
__device__ __forceinline__ void fetch_half(const SweepParams &p, int kind, int32_t ref, size_t g0, int h,
                                           float4 (&x)[5]) {
  const size_t N = (size_t)p.n_patterns;
  if (kind == kInner) {
    const float *src = static_cast<const float *>(p.clv) + ((size_t)ref * N + g0) * 80 + 40 * h;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const int f = threadIdx.x + i * kTThreads, m = f / 10, kc = f - m * 10;
      x[i] = __ldg(reinterpret_cast<const float4 *>(src + (size_t)m * 80) + kc);
    }
  } else if (kind == kTip) {
    const uint32_t *code = p.tips32 + (size_t)(-1 - ref) * N + g0;
#pragma unroll
    for (int i = 0; i < 5; ++i) x[i].x = __uint_as_float(__ldg(code + (threadIdx.x + i * kTThreads) / 10));
  }
}

// The fetched half rows into an A tile pair: split hi / lo for an inner
// child, 0/1 expansion of the mask (local columns 4kc.. = states 4(kc%5)..)
// for a tip.
__device__ __forceinline__ void put_half(int kind, const float4 (&x)[5], unsigned char *sAh, unsigned char *sAl) {
  if (kind == kInner) {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const int f = threadIdx.x + i * kTThreads, m = f / 10, kc = f - m * 10, off = kc * kAChunk + m * 16;
      float4 hi, lo;
      split4(x[i], hi, lo);
      *reinterpret_cast<float4 *>(sAh + off) = hi;
      *reinterpret_cast<float4 *>(sAl + off) = lo;
    }
  } else if (kind == kTip) {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const int f = threadIdx.x + i * kTThreads, m = f / 10, kc = f - m * 10;
      const uint32_t b = __float_as_uint(x[i].x) >> (4 * (kc % 5));
      *reinterpret_cast<float4 *>(sAh + kc * kAChunk + m * 16) =
          make_float4((float)(b & 1u), (float)((b >> 1) & 1u), (float)((b >> 2) & 1u), (float)((b >> 3) & 1u));
    }
  }
}

// 20 values of one thread's row into an A tile pair: local columns
// 20l .. 20l + 19 (slabs 5l .. 5l + 4), split hi / lo.
__device__ __forceinline__ void put_row(const float (&v)[20], int m, int l, unsigned char *sAh, unsigned char *sAl) {
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    const int off = (5 * l + q) * kAChunk + m * 16;
    float4 hi, lo;
    split4(make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]), hi, lo);
    *reinterpret_cast<float4 *>(sAh + off) = hi;
    *reinterpret_cast<float4 *>(sAl + off) = lo;
  }
}

// Asks L2 for the DRAM data of adjoint item (op, tile g0): its children's
// CLV rows (or tip state masks), its own CLV at a displayed-tree root, the
// scale counters and the incoming messages. All CTAs of a level move through
// their items in step, so without this each item's loads arrive as one burst
// the whole GPU waits for; issued an item ahead they stream in while the
// current item's MMAs and epilogues run.
__device__ __forceinline__ void prefetch_item20(const SweepParams &p, const BwdOp &op, size_t g0) {
  const size_t N = (size_t)p.n_patterns;
  const int t = threadIdx.x;
  auto pf = [](const void *a) { asm volatile("prefetch.global.L2 [%0];" ::"l"(a)); };
  auto rows = [&](const float *base) {  // 128 rows x 320 B = 320 lines of 128 B
    const char *b = reinterpret_cast<const char *>(base + g0 * 80);
    pf(b + 128 * t);
    if (t < 320 - kTThreads) pf(b + 128 * (t + kTThreads));
  };
  const float *clv = static_cast<const float *>(p.clv);
  const int32_t refs[2] = {op.a, op.b};
  for (int c = 0; c < 2; ++c) {
    const int32_t ref = refs[c];
    if (ref >= 0) {
      rows(clv + (size_t)ref * N * 80);
      if (t < 4) pf(p.scaler + (size_t)ref * N + g0 + 32 * t);
    } else if (ref != INT32_MIN && t < 4) {
      pf(p.tips32 + (size_t)(-1 - ref) * N + g0 + 32 * t);
    }
  }
  if (t >= 4 && t < 8) pf(p.scaler + (size_t)op.x * N + g0 + 32 * (t - 4));
  if (op.seed >= 0) rows(clv + (size_t)op.x * N * 80);
  const float *msg = static_cast<const float *>(p.msg);
  for (int mi = 0; mi < op.msg_count; ++mi) rows(msg + (size_t)__ldg(p.msg_slots + op.msg_begin + mi) * N * 80);
}

__global__ void __launch_bounds__(kTThreads, 1)
    backward20_tc_kernel(const SweepParams p, int op_begin, int n_ops, int n_tiles) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *sA = smem;
  unsigned char *sB1 = smem + kBwdA;
  unsigned char *sBQ = sB1 + kBwdB1;
  unsigned char *sB2 = sBQ + kBBytes;
  unsigned char *misc = sB2 + kBwdB2;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(misc);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(misc + 8);
  float *s_t = reinterpret_cast<float *>(misc + 16);  // [2][128] seed denominators
  float *s_ga = s_t + 2 * kTM;                         // [2][128] edge terms, side a
  float *s_gb = s_ga + 2 * kTM;                        // [2][128] edge terms, side b

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t N = (size_t)p.n_patterns;
  const long long W = (long long)n_ops * n_tiles;
  const int item_begin = (int)(W * blockIdx.x / gridDim.x), item_end = (int)(W * (blockIdx.x + 1) / gridDim.x);

  if (warp == 0) tc::tmem_alloc(tc::smem_u32(tmem_slot), 512);
  if (threadIdx.x == 0) tc::mbar_init(tc::smem_u32(mbar), 2);  // one commit per child's issuing thread
  for (int i = threadIdx.x; i < 4 * kTM; i += kTThreads)
    *reinterpret_cast<float4 *>(sA + (i / kTM) * kHBytes + 10 * kAChunk + (i % kTM) * 16) = make_float4(0, 0, 0, 0);
  for (int i = threadIdx.x; i < (kBwdB1 + kBBytes + kBwdB2) / 16; i += kTThreads)
    reinterpret_cast<float4 *>(sB1)[i] = make_float4(0, 0, 0, 0);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  const int q = warp & 3, hh = warp >> 2;  // pattern quarter, local rate
  const int m = 32 * q + lane;
  const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
  const float *clv = static_cast<const float *>(p.clv);
  float *msg = static_cast<float *>(p.msg);
  int staged_op = -1, staged_part = -1;
  uint32_t phase = 0;
  bool failed = false;

  for (int item = item_begin; item < item_end && !failed; ++item) {
    const int oi = item / n_tiles, tile = item - oi * n_tiles, opi = op_begin + oi;
    const size_t g0 = (size_t)tile * kTM, g = g0 + m;
    const BwdOp op = load_bwd_op(p.bwd_ops, opi);
    const int ka = child_kind(op.a), kb = child_kind(op.b);
    if (item + 1 < item_end) {
      const int noi = (item + 1) / n_tiles;
      prefetch_item20(p, noi == oi ? op : load_bwd_op(p.bwd_ops, op_begin + noi),
                      (size_t)(item + 1 - noi * n_tiles) * kTM);
    }
    const int part = p.unit_part[g0 / 16];  // partitions are padded to whole 256-pattern blocks
    if (oi != staged_op || part != staged_part) {
      stage_b_adj(p, sB1, sBQ, sB2, part, op.ea, kb == kAbsent ? -1 : op.eb, part != staged_part);
      staged_op = oi;
      staged_part = part;
    }
    const int sh = p.scaler[(size_t)op.x * N + g] - (ka == kInner ? p.scaler[(size_t)op.a * N + g] : 0) -
                   (kb == kInner ? p.scaler[(size_t)op.b * N + g] : 0);
    // displayed-tree seed: w_s rw_r pi_i / L_s with L_s summed over all rates
    float tseed = 0.f, sw = 0.f;
    if (op.seed >= 0) {
      // the thread's 2 rates x 20 states: 160 contiguous bytes as 10 vector loads
      const float4 *cx4 = reinterpret_cast<const float4 *>(clv + ((size_t)op.x * N + g) * 80 + 40 * hh);
      float cx[40];
#pragma unroll
      for (int j = 0; j < 10; ++j) {
        const float4 v = cx4[j];
        cx[4 * j] = v.x;
        cx[4 * j + 1] = v.y;
        cx[4 * j + 2] = v.z;
        cx[4 * j + 3] = v.w;
      }
      float part_t = 0.f;
#pragma unroll
      for (int l = 0; l < 2; ++l) {
        float u = 0.f;
#pragma unroll
        for (int i = 0; i < 20; ++i) u += p.freqs32[part * 20 + i] * cx[20 * l + i];
        part_t += p.rate_weights32[part * 4 + 2 * hh + l] * u;
      }
      s_t[hh * kTM + m] = part_t;
      __syncthreads();
      tseed = s_t[m] + s_t[kTM + m];
      sw = p.seeds32[(size_t)op.seed * p.n_parts + part] * p.weights32[g].x;
    }
    float ga = 0.f, gb = 0.f;
    for (int h = 0; h < 2; ++h) {
      const int r = 2 * h + hh;  // this thread's rate in this half
      // ---------------------------------------------------- round 1: p and Q c
      {
        float4 xa[5], xb[5];
        fetch_half(p, ka, op.a, g0, h, xa);
        fetch_half(p, kb, op.b, g0, h, xb);
        put_half(ka, xa, sA, sA + kHBytes);
        put_half(kb, xb, sA + 2 * kHBytes, sA + 3 * kHBytes);
      }
      tc::fence_proxy_async();
      __syncthreads();
      // child c's MMAs are issued by thread 32c: the two children's
      // accumulators are disjoint, and each issuer commits its own MMAs to
      // the mbarrier (two arrivals per round)
      if ((threadIdx.x & 31) == 0 && threadIdx.x < 64) {
        tc::fence_after_sync();
        const int c = threadIdx.x >> 5;
        const int kind = c ? kb : ka;
        if (kind != kAbsent) {
          const uint64_t dah = tc::smem_desc(tc::smem_u32(sA + (2 * c) * kHBytes), kAChunk, 128);
          const uint64_t dal = dah + (kHBytes >> 4);
          const uint64_t dq = tc::smem_desc(tc::smem_u32(sBQ), kBChunk, 128);
#pragma unroll
          for (int l = 0; l < 2; ++l) {
            const uint64_t db = tc::smem_desc(tc::smem_u32(sB1 + (c * 4 + 2 * h + l) * kBBytes), kBChunk, 128);
            const uint32_t d = tmem + 256 * c + 128 * l;
#pragma unroll
            for (int st = 0; st < 3; ++st) {
              const uint32_t ko = ((5 * l + 2 * st) * kAChunk) >> 4, bo = (2 * st * kBChunk) >> 4;
              tc::mma_tf32(d, dah + ko, db + bo, kIdN64, st > 0);
              tc::mma_tf32(d + 64, dah + ko, dq + bo, kIdN64, st > 0);
              if (kind == kInner) {
                tc::mma_tf32(d, dal + ko, db + bo, kIdN32, 1);
                tc::mma_tf32(d + 64, dal + ko, dq + bo, kIdN32, 1);
              }
            }
          }
        }
        tc::commit(tc::smem_u32(mbar));  // arrives at once when this thread issued nothing
      }
      // adjoint of x for (pattern g, rate r): incoming messages + seed
      float ax[20];
#pragma unroll
      for (int i = 0; i < 20; ++i) ax[i] = 0.f;
      for (int mi = 0; mi < op.msg_count; ++mi) {
        const float4 *src = reinterpret_cast<const float4 *>(
            msg + ((size_t)__ldg(p.msg_slots + op.msg_begin + mi) * N + g) * 80 + 20 * r);
#pragma unroll
        for (int j = 0; j < 5; ++j) {
          const float4 v = src[j];
          ax[4 * j] += v.x;
          ax[4 * j + 1] += v.y;
          ax[4 * j + 2] += v.z;
          ax[4 * j + 3] += v.w;
        }
      }
      if (op.seed >= 0 && tseed > 0.f && sw != 0.f) {
        const float e = p.inv_term32 ? root_inv_term<float>(p, g, p.scaler[(size_t)op.x * N + g]) : 0.f;
        const float f = sw * p.rate_weights32[part * 4 + r] / (tseed + e);
#pragma unroll
        for (int i = 0; i < 20; ++i) ax[i] += f * p.freqs32[part * 20 + i];
      }
      bool ok = tc::mbar_wait(tc::smem_u32(mbar), phase);
      phase ^= 1;
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      tc::fence_after_sync();
      // ----------------------------------------------------------- epilogue 1
      {
        float pa[20], pb[20];
        read_d(lane_base + 128 * hh, pa);
        if (kb != kAbsent) {
          read_d(lane_base + 256 + 128 * hh, pb);
        } else {
#pragma unroll
          for (int i = 0; i < 20; ++i) pb[i] = 1.f;
        }
        float u[20];
#pragma unroll
        for (int i = 0; i < 20; ++i) u[i] = Scale<float>::shift(ax[i] * pb[i], sh);
        put_row(u, m, hh, sA, sA + kHBytes);
        if (kb != kAbsent) {
#pragma unroll
          for (int i = 0; i < 20; ++i) u[i] = Scale<float>::shift(ax[i] * pa[i], sh);
          put_row(u, m, hh, sA + 2 * kHBytes, sA + 3 * kHBytes);
        }
      }
      tc::fence_proxy_async();
      tc::fence_before_sync();
      __syncthreads();
      // ------------------------------------------------- round 2: P_r^T u
      if ((threadIdx.x & 31) == 0 && threadIdx.x < 64) {
        tc::fence_after_sync();
        const int c = threadIdx.x >> 5;
        if ((c ? kb : ka) != kAbsent) {
          const uint64_t dah = tc::smem_desc(tc::smem_u32(sA + (2 * c) * kHBytes), kAChunk, 128);
          const uint64_t dal = dah + (kHBytes >> 4);
#pragma unroll
          for (int l = 0; l < 2; ++l) {
            const uint64_t db = tc::smem_desc(tc::smem_u32(sB2 + (c * 4 + 2 * h + l) * kBBytes), kBChunk, 128);
            const uint32_t d = tmem + 256 * c + 128 * l;
#pragma unroll
            for (int st = 0; st < 3; ++st) {
              const uint32_t ko = ((5 * l + 2 * st) * kAChunk) >> 4, bo = (2 * st * kBChunk) >> 4;
              tc::mma_tf32(d, dah + ko, db + bo, kIdN64, st > 0);
              tc::mma_tf32(d, dal + ko, db + bo, kIdN32, 1);
            }
          }
        }
        tc::commit(tc::smem_u32(mbar));  // arrives at once when this thread issued nothing
      }
      ok = tc::mbar_wait(tc::smem_u32(mbar), phase);
      phase ^= 1;
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      tc::fence_after_sync();
      // ----------------------------------------------------------- epilogue 2
      const float rate = p.rates32[part * 4 + r];
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        if ((c ? kb : ka) == kAbsent) continue;
        float mv[20], qc[20];
        read_d(lane_base + 256 * c + 128 * hh, mv);
        read_d(lane_base + 256 * c + 128 * hh + 64, qc);
        float dot = 0.f;
#pragma unroll
        for (int i = 0; i < 20; ++i) dot += mv[i] * qc[i];
        if (c) gb += rate * dot; else ga += rate * dot;
        // message row (this rate's 20 states) staged for a coalesced copy
        float4 *row = reinterpret_cast<float4 *>(sA + (c * kTM + m) * kStageRow + 80 * hh);
#pragma unroll
        for (int j = 0; j < 5; ++j) row[j] = make_float4(mv[4 * j], mv[4 * j + 1], mv[4 * j + 2], mv[4 * j + 3]);
      }
      tc::fence_before_sync();
      __syncthreads();
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int out = c ? op.out_b : op.out_a;
        if (out < 0 || (c ? kb : ka) == kAbsent) continue;
        float4 *dst = reinterpret_cast<float4 *>(msg + ((size_t)out * N + g0) * 80 + 40 * h);
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          const int f = threadIdx.x + i * kTThreads, rr = f / 10, c4 = f - rr * 10;
          dst[(size_t)rr * 20 + c4] = *reinterpret_cast<const float4 *>(sA + (c * kTM + rr) * kStageRow + 16 * c4);
        }
      }
      __syncthreads();
      // the staging rows overlap the zero slabs of the child-a tiles: clear them again
      if (threadIdx.x < 2 * kTM) {
        const int t = threadIdx.x >> 7, rr = threadIdx.x & (kTM - 1);
        *reinterpret_cast<float4 *>(sA + t * kHBytes + 10 * kAChunk + rr * 16) = make_float4(0, 0, 0, 0);
      }
    }
    if (failed) break;
    // edge terms per 16-pattern unit, summed in a fixed order
    s_ga[hh * kTM + m] = ga;
    s_gb[hh * kTM + m] = gb;
    __syncthreads();
    if (hh == 0) {
      // float-float sums over the unit's 16 lanes (no FP64 instruction)
      FF va = two_sum(s_ga[m], s_ga[kTM + m]);
      FF vb = two_sum(s_gb[m], s_gb[kTM + m]);
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) {
        va = ff_add(va, FF{__shfl_xor_sync(0xffffffffu, va.hi, o), __shfl_xor_sync(0xffffffffu, va.lo, o)});
        vb = ff_add(vb, FF{__shfl_xor_sync(0xffffffffu, vb.hi, o), __shfl_xor_sync(0xffffffffu, vb.lo, o)});
      }
      if ((lane & 15) == 0) {
        const size_t unit = g0 / 16 + (size_t)(m >> 4);
        // row op.pad0: the op's index in the full schedule, also when a
        // subset of the ops is launched (edge derivatives)
        *reinterpret_cast<float4 *>(p.grad_partial + ((size_t)op.pad0 * p.n_units + unit) * 2) =
            make_float4(va.hi, va.lo, vb.hi, vb.lo);
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  if (failed) {
    if (threadIdx.x == 0) atomicExch(p.fault, 1);
    tc::mbar_wait(tc::smem_u32(mbar), phase ^ 1);
    __syncthreads();
  }
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_free(tmem, 512);
}

}  // namespace

bool sweep20_tc_supported(int precision, int R) { return precision == 1 && R == 4; }

void launch_forward20_tc(cudaStream_t s, const SweepParams &p, const int32_t *level_begin, int n_levels,
                         int n_sms) {
  int dev = 0;
  cudaGetDevice(&dev);
  static bool attr_set[64] = {};
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    cudaFuncSetAttribute(forward20_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    attr_set[dev] = true;
  }
  const int n_tiles = (int)(p.n_patterns / kTM);
  int launched = 0;
  for (int L = 0; L < n_levels; ++L) {
    const int n = level_begin[L + 1] - level_begin[L];
    if (n <= 0) continue;
    const long long items = (long long)n * n_tiles;
    const int grid = (int)(items < n_sms ? items : n_sms);  // one CTA per SM
    forward20_tc_kernel<<<grid, kTThreads, kSmemBytes, s>>>(p, level_begin[L], n, n_tiles);
    ++launched;
  }
  add_launches(launched);
}

}  // namespace netlk

namespace netlk {

void launch_backward20_tc(cudaStream_t s, const SweepParams &p, const int32_t *level_begin, int n_levels,
                          int n_sms) {
  int dev = 0;
  cudaGetDevice(&dev);
  static bool attr_set[64] = {};
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    cudaFuncSetAttribute(backward20_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kBwdSmem);
    attr_set[dev] = true;
  }
  const int n_tiles = (int)(p.n_patterns / kTM);
  int launched = 0;
  for (int L = 0; L < n_levels; ++L) {
    const int n = level_begin[L + 1] - level_begin[L];
    if (n <= 0) continue;
    const long long items = (long long)n * n_tiles;
    const int grid = (int)(items < n_sms ? items : n_sms);
    backward20_tc_kernel<<<grid, kTThreads, kBwdSmem, s>>>(p, level_begin[L], n, n_tiles);
    ++launched;
  }
  add_launches(launched);
}

}  // namespace netlk
