// Device-side data layout and kernel launchers of netlk (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace netlk {

// Patterns per lane: a lane handles rate r of patterns s, s + 32/R, ... of
// its unit, so one P-row load and one op decode serve several patterns. The
// adjoint sweep (more live values per pattern) uses kPPLBase, the forward
// sweep kPPLForward; units, the unit -> partition map and the adjoint's
// per-unit gradient partials are counted in kPPLBase units.
constexpr int kPPLBase = 2;
constexpr int kPPLForward = 4;
static_assert(kPPLForward % kPPLBase == 0, "forward units must be whole adjoint units");
// Blocks have at most 8 warps (one unit each); partitions are padded to a
// whole number of 8-unit blocks so that a block never spans two partitions.
constexpr int kMaxWarpsPerBlock = 8;
constexpr int kThreads = 256;

// Forward op: CLV of variant `out` = (P[ea] . child a) (*) (P[eb] . child b).
// Child refs: >= 0 variant, -1-tip for a tip, INT32_MIN for the fake all-ones
// child (eb == -1). slot >= 0: the variant holds a displayed tree's root CLV;
// its per-site log-likelihoods are summed into site_partial[slot].
struct alignas(32) FwdOp {
  int32_t out, a, b, ea, eb, slot, pad0, pad1;
};

// Adjoint op for variant x (reverse level order), as message passing: the
// adjoint of x is the sum of the messages its parents wrote for it
// (msg_slots[msg_begin .. msg_begin + msg_count)); x then writes one message
// per inner child (out_a / out_b: message slot, or -1) and adds its two edge
// gradient terms. seed: displayed-tree root slot whose tree weight seeds x,
// or -1. A message buffer is reused only by levels launched after the level
// that read it. msg0..msg2 repeat the first three message slots, so a sweep
// reads them with the op instead of through the slot list. In the walk
// schedule out_a / out_b = -2 keeps that message in registers for the next
// op, whose pad4 = 1 (its only message).
struct alignas(64) BwdOp {
  int32_t x, a, b, ea, eb, seed, out_a, out_b;
  int32_t msg_begin, msg_count, pad0, msg0, msg1, msg2, pad4, pad5;
};

struct DevPartition {
  int32_t unit_begin, unit_end;  // forward units of this partition
};

// Everything the sweeps read, in device memory.
struct SweepParams {
  int32_t n_units;      // adjoint units: kPPLBase*32/R patterns (one per warp and op)
  int32_t n_units_fwd;  // forward units: kPPLForward*32/R patterns
  int64_t n_patterns;   // padded total (N)
  int32_t n_edges;
  int32_t n_fwd_ops;
  int32_t n_bwd_ops;
  int32_t n_parts;
  const FwdOp *fwd_ops;
  const BwdOp *bwd_ops;
  const int32_t *unit_part;     // [n_units]
  const uint8_t *tips;          // [n_tips][N] 4-bit state masks (4-state partitions)
  const uint32_t *tips32;       // [n_tips][N] 20-bit state masks (20-state partitions)
  const double *weights;        // [N] pattern weights (0 for padding)
  const void *pmat;             // [n_parts][n_edges][R][S][S] real
  const double *freqs;          // [n_parts][S]
  const double *rate_weights;   // [n_parts][R]
  const double *rates;          // [n_parts][R]
  const double *Q;              // [n_parts][S*S]
  // FP32 sweeps read float copies instead (GB300's FP64 pipe is a small
  // fraction of its FP32 one, so the FP32 kernels issue no FP64 instruction):
  const float2 *weights32;      // [N] (hi, lo): hi + lo == the double weight to ~2^-48
  const float *freqs32;         // [n_parts][S]
  const float *rate_weights32;  // [n_parts][R]
  const float *rates32;         // [n_parts][R]
  const float *Q32;             // [n_parts][S*S]
  const float *seeds32;         // [n_slots][n_parts]
  // invariant sites (+I): null when no partition has any; else the site
  // likelihood at a displayed-tree root is
  // gamma_frac[part] * (rate mixture + inv_term[pattern]), inv_term =
  // pinv * pi(invariant state) / (1 - pinv), 0 for a pattern without one
  const double *gamma_frac;     // [n_parts] 1 - pinv
  const float *gamma_frac32;
  const double *inv_term;       // [N]
  const float *inv_term32;
  void *clv;                    // [V][N][R][S] real
  int32_t *scaler;              // [V][N]
  void *msg;                    // [M][N][R][4] real adjoint messages
  const int32_t *msg_slots;     // message slots read by the adjoint ops
  // site_partial and grad_partial hold doubles in FP64 contexts and, in FP32
  // contexts, float pairs (hi, lo) in the same 8 bytes whose exact sum is the
  // value (see ff_to_double)
  double *site_partial;         // [n_slots][n_units_fwd]
  const double *seeds;          // [n_slots][n_parts]
  double *grad_partial;         // [n_bwd_ops][n_units][2] per-warp edge terms (a, b)
  int32_t *fault;               // set to 1 by a sweep whose bounded wait gave up
  // single-launch (walk) sweeps: every op in one cache-friendly topological
  // order; the adjoint ops carry their level-schedule index in pad0
  const FwdOp *walk_fwd_ops;
  int32_t n_walk_fwd;
  const BwdOp *walk_bwd_ops;
  int32_t n_walk_bwd;
  const int32_t *walk_msg_slots;
};

struct MixParams {
  int32_t n_slots, n_parts, n_roots, n_ret, variant, n_units;  // n_units: forward units
  int32_t ff;                     // 1: site_partial holds float pairs (FP32 sweeps)
  double min_logprob;
  const DevPartition *parts;      // [n_parts]
  const double *site_partial;     // [n_slots][n_units] (forward units)
  double *tree_logl;              // [n_slots][n_parts]
  const int32_t *root_slot;       // [n_roots]
  const double *root_logprob;     // [n_roots]
  const double *root_dlogprob;    // [n_roots][n_ret]
  double *seeds;                  // [n_slots][n_parts]
  float *seeds32;                 // [n_slots][n_parts] float copy for the FP32 sweeps (or null)
  double *weights;                // [n_parts][n_roots] scratch: tree posterior weights
  double *dret_part;              // [n_parts][n_ret] scratch: per-partition d logL / d p_k
  const int32_t *slot_begin;      // [n_slots+1] CSR: roots whose tree root is a slot
  const int32_t *slot_roots;      // [n_roots]
  double *out;                    // [2 + n_parts + n_ret]: total, status, part logl, dret
};

// len_stride 0: brlen[e] for every partition; n_edges: brlen[part * n_edges + e].
void launch_pmatrix(cudaStream_t s, int n_parts, int n_edges, int R, int S, const double *lambda,
                    const double *U, const double *Uinv, const double *rates, const double *brlen,
                    double *pmat64, float *pmat32, int len_stride = 0);
// The gradient per partition, grad [n_parts][n_edges], from the adjoint's
// per-unit edge terms (part_unit_begin: [n_parts + 1] base units); op_sum
// scratch [n_ops][n_parts][2].
void launch_grad_reduce_partitions(cudaStream_t s, int n_ops, int n_edges, int n_units, int n_parts,
                                   const int32_t *part_unit_begin, const int32_t *edge_begin,
                                   const int32_t *edge_entries, const double *partial, double *op_sum,
                                   double *grad, bool ff);
// Sweep launch shapes (threads per block, minimum blocks per SM): shape 0 is
// the default; num_shapes() > 1 where the autotuner has alternatives. Shapes
// from num_level_shapes() on are walk shapes: the whole sweep in one launch
// over the walk schedule (level_begin / n_levels are then unused).
int num_shapes(int precision, int R);
int num_level_shapes(int precision, int R);
// Kernel launches one sweep issues with this shape.
int sweep_launches(int precision, int R, int shape, const SweepParams &p, bool backward, const int32_t *level_begin,
                   int n_levels);
int shape_threads(int precision, int R, int shape);
// One launch per level: ops [level_begin[L], level_begin[L+1]) of the schedule.
void launch_forward(cudaStream_t s, int precision, int R, int shape, const SweepParams &p,
                    const int32_t *level_begin, int n_levels);
void launch_backward(cudaStream_t s, int precision, int R, int shape, const SweepParams &p,
                     const int32_t *level_begin, int n_levels);
void launch_tree_reduce(cudaStream_t s, const MixParams &m);
void launch_mix(cudaStream_t s, const MixParams &m);
// ff: the partials are float pairs (FP32 sweeps) rather than doubles.
void launch_grad_reduce(cudaStream_t s, int n_ops, int n_edges, int n_bx, const int32_t *edge_begin,
                        const int32_t *edge_entries, const double *partial, double *op_sum, double *grad,
                        bool ff);
// 20-state forward (backward = false) or adjoint sweep, one launch per level.
void launch_sweep20(cudaStream_t s, int precision, int R, bool backward, const SweepParams &p,
                    const int32_t *level_begin, int n_levels);
// Tensor-core (tcgen05) forward and adjoint sweeps for 20-state FP32
// contexts with 4 rate categories; one launch per level.
bool sweep20_tc_supported(int precision, int R);
void launch_forward20_tc(cudaStream_t s, const SweepParams &p, const int32_t *level_begin, int n_levels, int n_sms);
void launch_backward20_tc(cudaStream_t s, const SweepParams &p, const int32_t *level_begin, int n_levels, int n_sms);
// Candidate batch in persistent launches (DNA, FP32, 4 rates, walk
// schedules): everything one logL + gradient evaluation of candidate c reads
// and writes, in a device table the batch kernels index by candidate.
struct BatchCand {
  SweepParams sweep;            // walk ops, CLVs, messages, site / gradient partials
  MixParams mix;                // site sums and mixture
  // P-matrices: n_pmat = n_parts * n_edges * R * 16 entries from brlen
  const double *lambda, *U, *Uinv, *rates, *brlen;
  double *pmat64;
  float *pmat32;
  int64_t n_pmat;
  int32_t n_parts, n_edges;
  // gradient reduction (as launch_grad_reduce)
  int32_t n_ops, n_bx;
  const int32_t *edge_begin, *edge_entries;
  const double *grad_partial;
  double *op_sum, *grad;
  // results: out [n_out] then grad [n_edges] go to results + result_offset
  const double *out;
  int32_t n_out;
  int64_t result_offset;
};

struct BatchParams {
  const BatchCand *cands;
  int32_t n_cands;
  const int2 *items;            // (candidate, unit) in the order warps take them
  int32_t n_items;
  int32_t *counter;             // next item (reset before every walk launch)
  double *results;
  // grid extents: the largest candidate's
  int64_t max_pmat;
  int32_t max_slots, max_parts, max_ops, max_edges;
};

// Walk shapes the persistent batch kernels run (0 .. num_batch_shapes() - 1),
// and the adjoint patterns per lane of each (the items differ: a unit is
// 32 * ppl / 4 patterns).
int num_batch_shapes();
int batch_shape_bwd_ppl(int shape);
// Forward half: P-matrices, counter reset, persistent forward walk over every
// (candidate, unit) item, site sums, mixture. b.items: forward items.
void launch_batch_forward(cudaStream_t s, const BatchParams &b, int shape);
// Adjoint half: counter reset, persistent adjoint walk, gradient reduction,
// results gathered into b.results. b.items: adjoint items for the shape.
void launch_batch_backward(cudaStream_t s, const BatchParams &b, int shape);

// Forward-mode (tangent) sweep for the derivatives along one branch e
// (tangent.cu). Op for a variant x whose subtree contains e: d = child on e's
// side (mode 1: d hangs from e itself; mode 2: d contains e and its tangents
// are in tangent slot td), o = the other child (ref as in FwdOp), ed / eo their
// edges (eo = -1 for the fake child); tx: tangent slot x writes (-1: none
// reads it); slot: displayed-tree root slot whose site sums x feeds, or -1.
struct alignas(16) TanOp {
  int32_t x, d, o, ed, eo, mode, td, tx, slot, pad0, pad1, pad2;
};

struct TanParams {
  int64_t n_patterns;
  int32_t n_edges;
  int32_t n_blocks;             // blocks of tangent_patterns_per_block(R) patterns
  const void *clv;              // [V][N][R][S] real
  const int32_t *scaler;        // [V][N]
  const uint8_t *tips;          // 4-state tip masks [n_tips][N]
  const uint32_t *tips32;       // 20-state tip masks [n_tips][N]
  const void *pmat;             // [n_parts][n_edges][R][S][S] real
  const void *pderiv;           // [n_parts][2][R][S][S] real: d/dt and d2/dt2 of P_e
  void *tan;                    // [n_tan][2][N][R][S] real: X', X''
  const TanOp *ops;
  const int32_t *block_part;    // [n_blocks] partition of each block
  const double *weights;        // [N]
  const double *freqs;          // [n_parts][S]
  const double *rate_weights;   // [n_parts][R]
  const double *inv_term;       // invariant sites (+I), as in SweepParams; null without
  const float *inv_term32;      // FP32 contexts: its float copy (the tangent walk reads it)
  const float2 *weights32;      // FP32 contexts: pattern weights as (hi, lo) float pairs
  int32_t ff;                   // 1: partials are float pairs (hi, lo) in each double's 8 bytes
  double *partial;              // [n_slots][2][n_blocks] sums of w L'/L and w (L''/L - (L'/L)^2)
};

int tangent_patterns_per_block(int R);
// at length brlen[part * len_stride + edge] for each partition
void launch_pderiv(cudaStream_t s, int n_parts, int R, int S, const double *lambda, const double *U,
                   const double *Uinv, const double *rates, const double *brlen, int len_stride, int edge,
                   double *out64, float *out32);
// One launch per level of ops [level_begin[L], level_begin[L+1]) (20
// states; DNA takes launch_tangent_walk); false for an unsupported (R, S).
bool launch_tangent(cudaStream_t s, int precision, int R, int S, const TanParams &p, const int32_t *level_begin,
                    int n_levels);
// DNA: the same sweep as one walk launch over ops in walk order
// (netlk_ctx::walk_order), partials per unit of tangent_walk_patterns_per_unit(R)
// patterns: p.partial [n_slots][2][n_patterns / that]; false for S != 4.
int tangent_walk_patterns_per_unit(int R);
bool launch_tangent_walk(cudaStream_t s, int precision, int R, int S, const TanParams &p, int n_ops);
// out [n_slots_total][n_parts][2] for the root slots listed in `slots`.
void launch_tangent_reduce(cudaStream_t s, const TanParams &p, const int32_t *slots, int n_slots,
                           const int32_t *part_block_begin, int n_parts, double *out);

// Edge sumtables (tangent.cu): for branch e, each displayed tree's outside
// vector at e, O[i] = d L_site / d m_i with m = P_e I the message e carries
// up from its child CLV I (the tree's root site likelihood in the scaled
// units of the forward sweep), per (tree, pattern, rate). Built by a
// forward-mode sweep of the S unit directions of m over the variants above
// e (the tangent schedule); then L(t) = sum_r O_r . (P_r(t) I_r) for any
// length t, and L', L'' with P', P'': one pass over the tables per
// Newton-Raphson iterate. Every term is non-negative, so L keeps full
// relative precision at short lengths (a sum over eigencomponents would
// cancel there).
struct StabParams {
  TanParams t;                  // t.tan: [n_work][S][N][R][S] unit-direction planes; t.ops' slot = table index
  void *table;                  // [n_tab][N / 128][R][128][S] real: O per (table, pattern, rate)
  int32_t *table_scaler;        // [n_tab][N]: the root's scale counter when the table was built
  const void *pm3;              // [n_parts][3][R][S][S] real: P, P', P'' at the evaluated lengths (host-made)
  const int32_t *group_ref;     // [n_groups] child ref (as FwdOp) whose CLV is I for the group's tables
  const int32_t *group_begin;   // [n_groups + 1] tables of each group (tables sorted by child)
  int32_t n_groups;
  int32_t n_tables, tables_per_block;  // evaluation: tables, and tables per block (blockIdx.y)
  int32_t *fault;                      // set to 1 by an evaluation whose bounded wait gave up
  double *partial;              // [n_tab][3][N / 32] per-warp sums of w log L, w L'/L, w (L''/L - (L'/L)^2); FP32: float pairs
                                // (20 states: [n_tab][3][N R / 32], warps of 32 / R patterns)
  // 20 states: tables [n_tab][N][R][S], built by reverse walks along each
  // tree's path: path_ops [6 per op] = (x, d, o, ed, eo, mode) from the
  // root down, path_begin [n_tab + 1]
  const int32_t *path_ops;
  const int32_t *path_begin;
};

// Builds the tables (one walk launch over the tangent schedule's ops in
// depth-first order); false for an unsupported (R, S): DNA.
// 20 states: the reverse path walks (grid.y = table); false for R > 4.
bool launch_sumtable_path20(cudaStream_t s, int precision, int R, const StabParams &p, int n_tab);
bool launch_sumtable_build(cudaStream_t s, int precision, int R, int S, const StabParams &p,
                           const int32_t *level_begin, int n_levels);
// Once per context before the first evaluation (outside any graph capture):
// the evaluation's shared-memory size; false for an unsupported (R, S).
bool sumtable_eval_setup(int precision, int R, int S);
// Evaluates every table at p.pm3 and reduces per (table, partition):
// out [n_tab][n_parts][3] (w log L with the scale counters applied, l', l'').
bool launch_sumtable_eval(cudaStream_t s, int precision, int R, int S, const StabParams &p, int n_tab,
                          const int32_t *part_warp_begin, int n_parts, double *out);

// Number of kernel launches issued by the launchers above (host counter).
int64_t launches_issued();
void add_launches(int64_t n);

}  // namespace netlk
