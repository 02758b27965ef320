// netlk context and C ABI.
//
// A context mirrors what the reference keeps in AnnotatedNetwork +
// fake_treeinfo for the likelihood path (src/graph/AnnotatedNetwork.hpp:42-89):
// topology, per-partition model and tips, branch lengths and reticulation
// probabilities, and one CLV per displayed-tree variant of every inner node
// (DisplayedTreeData, src/graph/DisplayedTreeData.hpp:18-42) - here in device
// memory, computed by one forward sweep and differentiated by one adjoint
// sweep.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/netlk.h"
#include "internal.hpp"
#include "kernels.cuh"

using namespace netlk;

namespace {

thread_local std::string g_create_error;

// Copies an adjoint op's first three message slots (already appended to
// `slots` from op.msg_begin on) into the op itself.
void set_inline_msgs(BwdOp &op, const std::vector<int32_t> &slots) {
  int32_t *inl[3] = {&op.msg0, &op.msg1, &op.msg2};
  for (int m = 0; m < 3; ++m) *inl[m] = m < op.msg_count ? slots[op.msg_begin + m] : -1;
}

#define CUDA_OK(expr)                                                                     \
  do {                                                                                    \
    cudaError_t _e = (expr);                                                              \
    if (_e != cudaSuccess) {                                                              \
      if (_e == cudaErrorMemoryAllocation)                                                \
        throw Error(NETLK_ERR_OUT_OF_MEMORY, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
      throw Error(NETLK_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));   \
    }                                                                                     \
  } while (0)

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  void alloc(size_t b, int64_t &total) {
    free();
    if (b == 0) b = 16;
    CUDA_OK(cudaMalloc(&p, b));
    bytes = b;
    total += (int64_t)b;
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T *as() const { return static_cast<T *>(p); }
};

struct PinnedBuf {
  void *p = nullptr;
  void alloc(size_t b) {
    if (p) cudaFreeHost(p);
    CUDA_OK(cudaHostAlloc(&p, std::max<size_t>(b, 16), cudaHostAllocDefault));
  }
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  template <class T>
  T *as() const { return static_cast<T *>(p); }
};

struct PartInfo {
  int n = 0;             // patterns
  int n_pad = 0;         // padded to a whole number of 32-pattern blocks
  int64_t offset = 0;    // first global pattern
  int unit_begin = 0, unit_end = 0;
  std::vector<double> freqs, exch, rates, rate_weights;
  double alpha = 1.0;
  double pinv = 0.0;  // proportion of invariant sites (+I)
  double wsum = 0.0;  // sum of the pattern weights
  bool explicit_rates = false;
  Eigen eig;
};

}  // namespace

struct netlk_ctx {
  netlk_options opts{};
  int S = 4, R = 4, P = 0;
  Topology topo;
  Dag dag;
  std::vector<double> brlen, ret_probs;
  // branch-length linkage: unlinked and scaled contexts keep per-partition
  // lengths plen [P][E] (what the device uses); linked ones use brlen for
  // every partition
  int linkage = NETLK_BRLEN_LINKED;
  std::vector<double> plen, scalers;
  int len_stride() const { return linkage == NETLK_BRLEN_LINKED ? 0 : topo.n_edges; }
  const std::vector<double> &dev_len() const { return linkage == NETLK_BRLEN_LINKED ? brlen : plen; }
  void refresh_scaled() {
    const int E = topo.n_edges;
    for (int p = 0; p < P; ++p)
      for (int e = 0; e < E; ++e) plen[(size_t)p * E + e] = scalers[p] * brlen[e];
  }
  std::vector<PartInfo> parts;
  int64_t N = 0;
  int n_units = 0, n_units_fwd = 0, ppw = 8;
  // schedules
  std::vector<FwdOp> fwd;
  std::vector<BwdOp> bwd;
  int n_slots = 0, n_adj = 0, n_bwd_real = 0;
  std::vector<int32_t> root_slot, slot_begin, slot_roots, msg_slots;
  std::vector<int32_t> fwd_level_begin, bwd_level_begin;  // op ranges per launch
  std::vector<int32_t> edge_begin, edge_entries;         // edge -> adjoint op sides
  int fwd_launches = 0, bwd_launches = 0;
  // CLV checkpointing: levels cut into segments; a variant read by an op of a
  // later segment keeps a permanent CLV slot, the others share one segment's
  // worth of slots and are recomputed before their segment's adjoint levels
  int n_segments = 1, n_clv_slots = 0;
  std::vector<int32_t> var_slot;           // CLV / scale-counter slot per variant
  std::vector<char> var_ckpt;              // permanent slot
  std::vector<int> seg_lo, seg_hi;         // level range (1-based) per segment
  std::vector<FwdOp> rfwd;                 // recompute ops (no site sums)
  std::vector<int32_t> rfwd_level_begin;   // per level, like fwd_level_begin
  int rfwd_launches = 0;
  int64_t recompute_updates = 0;
  // incremental evaluation: the lengths the stored CLVs were computed with
  bool clv_valid = false;
  std::vector<double> clv_brlen;
  std::vector<FwdOp> ifwd;                 // ops of the variants to recompute
  std::vector<int32_t> ifwd_level_begin;
  // walk schedules: each sweep as one op list per warp, in a depth-first
  // order kept segment by segment (so checkpointing works with them); wbwd
  // carries its level-schedule index in pad0. With k segments the forward is
  // one walk over all segments, the adjoint one walk per segment from the
  // top, each but the top one after a walk recomputing that segment's
  // non-permanent CLVs (wrfwd).
  std::vector<FwdOp> wfwd, wrfwd;
  std::vector<BwdOp> wbwd;
  std::vector<int32_t> wmsg_slots;
  std::vector<int32_t> wfwd_var, wrfwd_var, wbwd_var;    // variant of each walk op
  std::vector<std::pair<int32_t, int32_t>> wrfwd_range;  // per segment: [begin, end) in wrfwd
  std::vector<std::pair<int32_t, int32_t>> wbwd_range;   // per segment: [begin, end) in wbwd
  int n_wadj = 0;
  bool walk_ok = false;
  int fwd_wshape = 0;  // forward walk shape the checkpoint recompute walks use
  int rfwd_level_launches = 0;
  // best level-schedule shapes (the walk shapes only run the full sweeps)
  int fwd_lshape = 0, bwd_lshape = 0;
  int64_t last_updates = 0;
  int32_t inject_status = 0;  // netlk_inject_failure: fail the next result check
  int fwd_shape = 0, bwd_shape = 0, sms = 0;
  bool tuned = false;
  bool use_tc = false;  // 20-state FP32 forward on the tensor cores
  std::vector<double> tune_fwd_ms, tune_bwd_ms;
  int64_t site_updates = 0, tip_uses = 0, fake_uses = 0;
  // device
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t dev_bytes = 0;
  DevBuf d_clv, d_scaler, d_adj, d_msg_slots, d_tips, d_weights, d_unit_part, d_fwd, d_bwd, d_rfwd, d_ifwd;
  DevBuf d_wfwd, d_wrfwd, d_wbwd, d_wmsg_slots;
  // analytic edge derivatives: tangent buffers and per-call schedule
  DevBuf d_tan, d_tan_ops, d_tan_partial, d_tan_out, d_pderiv64, d_pderiv32, d_block_part, d_part_block_begin,
      d_tan_slots, d_part_tunit_begin;
  PinnedBuf h_tan_ops, h_tan_out, h_tan_slots;
  int n_tan_cap = -1;  // tangent slot pairs allocated (-1: not set up yet)
  int tan_blocks = 0;
  // edge sumtables: unit-direction work planes, per-tree outside vectors at
  // the edge (tables), their scale counters, and the evaluation buffers
  DevBuf d_stab_work, d_stab, d_stab_scaler, d_stab_partial, d_stab_out, d_stab_pm3_64, d_stab_pm3_32,
      d_stab_groups, d_stab_ops, d_part_warp_begin, d_stab_paths;
  PinnedBuf h_stab_pm3, h_stab_out, h_stab_ops, h_stab_paths;
  int64_t stab_cap_path = 0;  // 20 states: path ops allocated
  cudaGraphExec_t graph_stab = nullptr;  // one evaluation of the current tables
  int stab_cap_work = -1, stab_cap_tab = 0;  // work slots / tables allocated (-1: not set up yet)
  int stab_edge = -1;                        // edge whose tables are current (-1: none)
  int stab_n_tab = 0, stab_n_groups = 0;
  std::vector<int32_t> stab_root_tab;                  // per root: its table, or -1 (edge not in the tree)
  std::vector<double> stab_lens, stab_probs, stab_tree;  // parameters at the build; per-(slot, part) tree logL
  uint64_t model_gen = 0, stab_gen = 0;
  DevBuf d_pmat64, d_pmat32, d_lambda, d_U, d_Uinv, d_rates, d_rw, d_freqs, d_Q, d_brlen;
  DevBuf d_grad_part, d_op_sum_part, d_part_unit_begin;  // per-partition gradient (on request)
  // FP32 contexts: float copies the sweeps read (weights as hi/lo pairs)
  DevBuf d_weights32, d_model32, d_seeds32;
  // invariant sites (+I): per partition 1 - pinv, per pattern pinv * pi of its
  // invariant state / (1 - pinv) (0 if it has none); used only while has_pinv
  DevBuf d_gfrac, d_gfrac32, d_invt, d_invt32;
  std::vector<int8_t> inv_state;  // [N] the one state every tip admits, or -1
  bool has_pinv = false;
  size_t m32_freqs = 0, m32_rw = 0, m32_rates = 0;  // offsets (floats) in d_model32; Q at 0
  DevBuf d_site_partial, d_tree_logl, d_root_slot, d_root_lp, d_root_dlp, d_seeds, d_wts, d_dret;
  DevBuf d_slot_begin, d_slot_roots, d_parts, d_out, d_grad_partial, d_grad, d_edge_begin, d_edge_entries, d_op_sum;
  PinnedBuf h_brlen, h_root_lp, h_root_dlp, h_out, h_grad, h_tree, h_ifwd;
  cudaGraphExec_t graph_logl = nullptr, graph_grad = nullptr, graph_partials = nullptr,
                  graph_mixbwd = nullptr;
  bool probs_dirty = true, model_dirty = true;
  bool device_brlen = false;  // last branch lengths came from device memory
  int64_t launches = 0;
  int64_t fwd_bytes = 0, bwd_bytes = 0, rfwd_bytes = 0;
  // per-kernel event timing (profiling mode launches without graphs)
  bool profiling = false;
  std::vector<cudaEvent_t> prof_ev;
  std::vector<int> prof_kernel;
  int prof_n = 0;
  double prof_ms[6] = {0, 0, 0, 0, 0, 0};
  int64_t prof_cnt[6] = {0, 0, 0, 0, 0, 0};
  void prof_mark(int kernel) {
    if (!profiling) return;
    if (prof_n >= (int)prof_ev.size()) {
      cudaEvent_t e;
      CUDA_OK(cudaEventCreate(&e));
      prof_ev.push_back(e);
      prof_kernel.push_back(-1);
    }
    prof_kernel[prof_n] = kernel;
    CUDA_OK(cudaEventRecord(prof_ev[prof_n], stream));
    prof_n++;
  }
  void prof_collect() {
    if (!profiling || prof_n == 0) return;
    CUDA_OK(cudaEventSynchronize(prof_ev[prof_n - 1]));
    for (int i = 1; i < prof_n; ++i) {
      float ms = 0.f;
      CUDA_OK(cudaEventElapsedTime(&ms, prof_ev[i - 1], prof_ev[i]));
      const int k = prof_kernel[i];
      if (k >= 0 && k < 6) {
        prof_ms[k] += ms;
        prof_cnt[k]++;
      }
    }
    prof_n = 0;
  }
  std::string err;

  ~netlk_ctx() {
    if (device >= 0) cudaSetDevice(device);
    for (auto e : prof_ev) cudaEventDestroy(e);
    for (auto g : {graph_logl, graph_grad, graph_partials, graph_mixbwd, graph_stab})
      if (g) cudaGraphExecDestroy(g);
    for (DevBuf *b : {&d_clv, &d_scaler, &d_adj, &d_msg_slots, &d_tips, &d_weights, &d_unit_part, &d_fwd, &d_bwd, &d_rfwd, &d_ifwd,
                      &d_pmat64, &d_pmat32, &d_lambda, &d_U, &d_Uinv, &d_rates, &d_rw, &d_freqs, &d_Q,
                      &d_brlen, &d_site_partial, &d_tree_logl, &d_root_slot, &d_root_lp, &d_root_dlp,
                      &d_seeds, &d_wts, &d_dret, &d_slot_begin, &d_slot_roots, &d_parts, &d_out, &d_grad_partial, &d_grad,
                      &d_edge_begin, &d_edge_entries, &d_op_sum, &d_weights32, &d_model32, &d_seeds32,
                      &d_wfwd, &d_wrfwd, &d_wbwd, &d_wmsg_slots, &d_tan, &d_tan_ops, &d_tan_partial, &d_tan_out,
                      &d_pderiv64, &d_pderiv32, &d_block_part, &d_part_block_begin, &d_tan_slots, &d_gfrac,
                      &d_gfrac32, &d_invt, &d_invt32, &d_grad_part, &d_op_sum_part, &d_part_unit_begin, &d_stab_work,
                      &d_stab, &d_stab_scaler, &d_stab_partial, &d_stab_out, &d_stab_pm3_64, &d_stab_pm3_32,
                      &d_stab_groups, &d_stab_ops, &d_part_warp_begin, &d_part_tunit_begin, &d_stab_paths})
      b->free();
    if (stream) cudaStreamDestroy(stream);
  }

  SweepParams sweep() const {
    SweepParams p{};
    p.n_units = n_units;
    p.n_units_fwd = n_units_fwd;
    p.n_patterns = N;
    p.n_edges = topo.n_edges;
    p.n_fwd_ops = (int)fwd.size();
    p.n_bwd_ops = (int)bwd.size();
    p.n_parts = P;
    p.fwd_ops = d_fwd.as<FwdOp>();
    p.bwd_ops = d_bwd.as<BwdOp>();
    p.unit_part = d_unit_part.as<int32_t>();
    p.tips = S == 4 ? d_tips.as<uint8_t>() : nullptr;
    p.tips32 = S == 20 ? d_tips.as<uint32_t>() : nullptr;
    p.weights = d_weights.as<double>();
    p.pmat = opts.precision == NETLK_FP32 ? d_pmat32.p : d_pmat64.p;
    p.freqs = d_freqs.as<double>();
    p.rate_weights = d_rw.as<double>();
    p.rates = d_rates.as<double>();
    p.Q = d_Q.as<double>();
    if (opts.precision == NETLK_FP32) {
      const float *m32 = d_model32.as<float>();
      p.weights32 = d_weights32.as<float2>();
      p.Q32 = m32;
      p.freqs32 = m32 + m32_freqs;
      p.rate_weights32 = m32 + m32_rw;
      p.rates32 = m32 + m32_rates;
      p.seeds32 = d_seeds32.as<float>();
    }
    p.clv = d_clv.p;
    p.scaler = d_scaler.as<int32_t>();
    p.msg = d_adj.p;
    p.msg_slots = d_msg_slots.as<int32_t>();
    p.site_partial = d_site_partial.as<double>();
    p.seeds = d_seeds.as<double>();
    p.grad_partial = d_grad_partial.as<double>();
    p.fault = reinterpret_cast<int32_t *>(d_out.as<double>() + 2 + P + topo.n_ret);
    if (has_pinv) {
      p.gamma_frac = d_gfrac.as<double>();
      p.gamma_frac32 = d_gfrac32.as<float>();
      p.inv_term = d_invt.as<double>();
      p.inv_term32 = d_invt32.as<float>();
    }
    if (walk_ok) {
      p.walk_fwd_ops = d_wfwd.as<FwdOp>();
      p.n_walk_fwd = (int32_t)wfwd.size();
      p.walk_bwd_ops = d_wbwd.as<BwdOp>();
      p.n_walk_bwd = (int32_t)wbwd.size();
      p.walk_msg_slots = d_wmsg_slots.as<int32_t>();
    }
    return p;
  }

  MixParams mix() const {
    MixParams m{};
    m.n_slots = n_slots;
    m.n_parts = P;
    m.n_roots = (int)dag.roots.size();
    m.n_ret = topo.n_ret;
    m.variant = opts.variant;
    m.n_units = n_units_fwd;
    m.min_logprob = opts.min_interesting_tree_logprob;
    m.parts = d_parts.as<DevPartition>();
    m.site_partial = d_site_partial.as<double>();
    m.tree_logl = d_tree_logl.as<double>();
    m.root_slot = d_root_slot.as<int32_t>();
    m.root_logprob = d_root_lp.as<double>();
    m.root_dlogprob = d_root_dlp.as<double>();
    m.seeds = d_seeds.as<double>();
    m.ff = opts.precision == NETLK_FP32 ? 1 : 0;
    m.seeds32 = opts.precision == NETLK_FP32 ? d_seeds32.as<float>() : nullptr;
    m.weights = d_wts.as<double>();
    m.dret_part = d_dret.as<double>();
    m.slot_begin = d_slot_begin.as<int32_t>();
    m.slot_roots = d_slot_roots.as<int32_t>();
    m.out = d_out.as<double>();
    return m;
  }

  void autotune();
  void count_launches();
  void build_schedules(int segments);
  void build_walk(const std::vector<char> &inb, const std::vector<int> &slot_of,
                  const std::vector<std::vector<int>> &by_level, const std::vector<int> &bwd_var);
  int choose_segments(size_t free_bytes) const;
  void allocate_and_upload(const netlk_partition *in_parts);
  void upload_model();
  void upload_probs();
  void enqueue(bool pm, bool fwd_on, bool reduce, bool mixk, bool bwd_on);
  void enqueue_adjoint(const SweepParams &sp, int bshape);
  bool adjoint_walks(int bshape) const;
  void run(cudaGraphExec_t *cache, bool pm, bool fwd_on, bool reduce, bool mixk, bool bwd_on);
  // logL recomputing only the CLVs above changed branch lengths; false when a
  // full evaluation is needed instead
  bool run_incremental();
  // d logL / d t_e from an incremental forward and the adjoint ops edge e's
  // terms depend on, bit-identical to the full gradient's entry; false where
  // the full evaluation is needed instead
  // analytic d1 and d2 along edge e from a tangent sweep over the variants
  // above it; false where that path does not apply (several checkpoint
  // segments, device-resident lengths)
  // part >= 0: that partition's share only
  bool edge_derivs_analytic(int e, int mode, double *d1, double *d2, int part = -1);
  void setup_tangent_blocks();
  // mode 1 reproduces the reference's derivative formula, which refuses
  // scaled branch lengths (LikelihoodDerivatives.cpp:42-46)
  void check_reference_mode(int mode) const {
    if (mode == 1 && linkage == NETLK_BRLEN_SCALED)
      throw Error(NETLK_ERR_UNSUPPORTED,
                  "the reference's derivative formula (mode 1) does not take scaled branch lengths; mode 0 does");
  }
  TanParams tan_params() const {  // the fields shared by the tangent and sumtable sweeps
    TanParams tp{};
    tp.n_patterns = N;
    tp.n_edges = topo.n_edges;
    tp.n_blocks = tan_blocks;
    tp.clv = d_clv.p;
    tp.scaler = d_scaler.as<int32_t>();
    tp.tips = S == 4 ? d_tips.as<uint8_t>() : nullptr;
    tp.tips32 = S == 20 ? d_tips.as<uint32_t>() : nullptr;
    tp.pmat = opts.precision == NETLK_FP32 ? d_pmat32.p : d_pmat64.p;
    tp.block_part = d_block_part.as<int32_t>();
    tp.weights = d_weights.as<double>();
    tp.freqs = d_freqs.as<double>();
    tp.rate_weights = d_rw.as<double>();
    tp.inv_term = has_pinv ? d_invt.as<double>() : nullptr;
    if (opts.precision == NETLK_FP32) {
      tp.inv_term32 = has_pinv ? d_invt32.as<float>() : nullptr;
      tp.weights32 = d_weights32.as<float2>();
    }
    return tp;
  }
  StabParams stab_params() const {
    StabParams sp{};
    sp.t = tan_params();
    sp.t.tan = d_stab_work.p;
    sp.t.ops = d_stab_ops.as<TanOp>();
    sp.table = d_stab.p;
    sp.table_scaler = d_stab_scaler.as<int32_t>();
    sp.pm3 = opts.precision == NETLK_FP32 ? d_stab_pm3_32.p : d_stab_pm3_64.p;
    sp.group_ref = d_stab_groups.as<int32_t>();
    sp.group_begin = d_stab_groups.as<int32_t>() + stab_n_groups;
    sp.n_groups = stab_n_groups;
    sp.n_tables = stab_n_tab;
    // about four blocks of each pattern range per SM at the largest counts,
    // at least 4 tables per block (the child's P I is formed once per block)
    sp.tables_per_block = std::max(4, (int)((int64_t)stab_n_tab * (N / 128) / (152 * 16) + 1));
    sp.partial = d_stab_partial.as<double>();
    sp.fault = reinterpret_cast<int32_t *>(d_stab_out.as<double>() + (size_t)std::max(1, stab_cap_tab) * P * 3);
    return sp;
  }
  // Per-partition mixture of per-tree (l, l', l'') along edge e: logL of the
  // partition (over every tree) and its first / second derivative (mode 0:
  // of the mixture; mode 1: the reference's formula over the trees active at
  // e). false when mode 1 finds no tree.
  template <class LL, class A1, class A2>
  bool mix_edge(int e_mode, const std::vector<char> &act, LL ll, A1 a1, A2 a2, double *logl, double *D1,
                double *D2) const;
  // edge sumtables (Newton-Raphson along one edge): build at the current
  // parameters (false where the path does not apply: 20 states, several
  // checkpoint segments, device-resident lengths, too little memory);
  // current while only edge e's lengths and nothing else changed since
  bool sumtable_build(int e);
  // The walk of edge e's table build: ops in depth-first order with work
  // slots (walk_order), their slot fields renumbered to table indices, the
  // tables grouped by the child whose CLV the edge's message starts from
  // (gref: that child per group, gbegin: [n_groups + 1] table ranges),
  // slot_tab: table of each displayed-tree root slot (-1: edge not in it).
  // Returns the work slots used, or -1.
  int sumtable_schedule(int e, std::vector<TanOp> &ops, std::vector<int32_t> &gref, std::vector<int32_t> &gbegin,
                        std::vector<int32_t> &slot_tab) const;
  // Reorders a tangent schedule depth-first for one walk (each op right
  // before the ops that read its directions) and reassigns the work slots
  // by live range in that order; returns the slots used, or -1.
  static int walk_order(std::vector<TanOp> &ops);
  // 20 states: per table (ops' slot fields numbered as tables), the ops from
  // its root down to the op that takes the edge's message, 6 ints each
  // (x, d, o, ed, eo, mode); path_begin [n_tab + 1]
  void sumtable_paths(const std::vector<TanOp> &ops, int n_tab, std::vector<int32_t> &path_ops,
                      std::vector<int32_t> &path_begin) const;
  bool sumtable_current(int e) const;
  // per_part: len, logl, d1, d2 hold one entry per partition (each at its
  // own length); else len[0] is the edge's (linked or scaled) length and the
  // outputs are totals w.r.t. it
  void sumtable_eval(int e, const double *len, bool per_part, int mode, double *logl, double *d1, double *d2);
  int tangent_schedule(int e, std::vector<TanOp> &ops, std::vector<int32_t> &level_begin,
                       std::vector<int32_t> &slots) const;
  // d logL / d (partition p's length of edge e) [P][E] from the last adjoint
  // sweep's per-unit edge terms (two extra reductions)
  void partition_gradient(double *out);
  // roots (displayed trees) on which edge e counts as active for the
  // reference's derivative formula
  std::vector<char> active_roots_of(int e) const;
  void prepare_state();  // model / probabilities uploads and launch-shape tuning
  void prepare();        // prepare_state + branch-length upload
  void finish(double *total, double *part_logl, double *d_brlen, double *d_ret);
  // a failure planted by netlk_inject_failure, thrown once
  void check_injected() {
    if (inject_status) {
      const int st = inject_status;
      inject_status = 0;
      throw Error(st, "injected failure (netlk_inject_failure)");
    }
  }
  // results from the pinned host copies of the last evaluation
  void read_results(double *total, double *part_logl, double *d_brlen, double *d_ret);
};

// ------------------------------------------------------------------ schedules
// Segments: contiguous level ranges with about V / k variants each.
void netlk_ctx::build_schedules(int segments) {
  const int V = (int)dag.vars.size();
  n_segments = std::max(1, std::min(segments, std::max(1, dag.n_levels)));
  std::vector<int> seg_of_level(dag.n_levels + 2, 0);
  seg_lo.assign(n_segments, 1);
  seg_hi.assign(n_segments, dag.n_levels);
  {
    std::vector<int64_t> cnt(dag.n_levels + 2, 0);
    for (const Variant &v : dag.vars) cnt[v.level]++;
    int s = 0;
    int64_t acc = 0;
    for (int L = 1; L <= dag.n_levels; ++L) {
      // open the next segment once this one holds its share (levels left >= segments left)
      if (s + 1 < n_segments && acc >= (int64_t)(s + 1) * V / n_segments && dag.n_levels - L + 1 >= n_segments - s - 1) {
        seg_hi[s] = L - 1;
        ++s;
        seg_lo[s] = L;
      }
      seg_of_level[L] = s;
      acc += cnt[L];
    }
    n_segments = s + 1;
    seg_lo.resize(n_segments);
    seg_hi.resize(n_segments);
    seg_hi[n_segments - 1] = dag.n_levels;
  }
  // permanent slots: variants read by an op of a later segment
  var_ckpt.assign(V, 0);
  var_slot.assign(V, 0);
  if (n_segments == 1) {
    for (int v = 0; v < V; ++v) var_slot[v] = v;
    n_clv_slots = V;
  } else {
    for (int v = 0; v < V; ++v)
      for (int i = 0; i < 2; ++i) {
        const int32_t c = dag.vars[v].ref[i];
        if (c >= 0 && seg_of_level[dag.vars[v].level] > seg_of_level[dag.vars[c].level]) var_ckpt[c] = 1;
      }
    int n_ckpt = 0;
    for (int v = 0; v < V; ++v)
      if (var_ckpt[v]) var_slot[v] = n_ckpt++;
    std::vector<int> used(n_segments, 0);
    int region = 0;
    for (int v = 0; v < V; ++v)
      if (!var_ckpt[v]) {
        const int sg = seg_of_level[dag.vars[v].level];
        var_slot[v] = n_ckpt + used[sg]++;
        region = std::max(region, used[sg]);
      }
    n_clv_slots = n_ckpt + region;
  }
  auto map_ref = [&](int32_t r) { return r >= 0 ? var_slot[r] : r; };
  // displayed-tree root slots
  std::vector<int> slot_of(V, -1);
  n_slots = 0;
  root_slot.clear();
  for (auto &rv : dag.roots) {
    if (slot_of[rv.dtroot_variant] < 0) slot_of[rv.dtroot_variant] = n_slots++;
    root_slot.push_back(slot_of[rv.dtroot_variant]);
  }
  slot_begin.assign(n_slots + 1, 0);
  for (int s : root_slot) slot_begin[s + 1]++;
  for (int s = 0; s < n_slots; ++s) slot_begin[s + 1] += slot_begin[s];
  slot_roots.assign(dag.roots.size(), 0);
  {
    std::vector<int> fill(slot_begin.begin(), slot_begin.end() - 1);
    for (int i = 0; i < (int)dag.roots.size(); ++i) slot_roots[fill[root_slot[i]]++] = i;
  }
  // forward: level order, each level padded to whole groups
  std::vector<std::vector<int>> by_level(dag.n_levels + 1);
  for (int v = 0; v < V; ++v) by_level[dag.vars[v].level].push_back(v);
  fwd.clear();
  fwd_level_begin.assign(1, 0);
  tip_uses = fake_uses = 0;
  for (int L = 1; L <= dag.n_levels; ++L) {
    for (int v : by_level[L]) {
      const Variant &var = dag.vars[v];
      FwdOp op{var_slot[v], map_ref(var.ref[0]), map_ref(var.ref[1]), var.edge[0], var.edge[1], slot_of[v], 0, 0};
      fwd.push_back(op);
      tip_uses += is_tip_ref(var.ref[0]) + is_tip_ref(var.ref[1]);
      fake_uses += var.ref[1] == kFake;
    }
    fwd_level_begin.push_back((int32_t)fwd.size());
  }
  fwd_launches = 0;
  for (int L = 0; L < dag.n_levels; ++L) fwd_launches += fwd_level_begin[L + 1] > fwd_level_begin[L];
  // recompute ops: the non-permanent variants of every segment but the last
  // (whose CLVs are still in place when the adjoint starts)
  rfwd.clear();
  rfwd_level_begin.assign(1, 0);
  rfwd_launches = 0;
  recompute_updates = 0;
  for (int L = 1; L <= dag.n_levels; ++L) {
    if (n_segments > 1 && seg_of_level[L] < n_segments - 1)
      for (int v : by_level[L]) {
        if (var_ckpt[v]) continue;
        const Variant &var = dag.vars[v];
        rfwd.push_back(FwdOp{var_slot[v], map_ref(var.ref[0]), map_ref(var.ref[1]), var.edge[0], var.edge[1], -1, 0, 0});
      }
    rfwd_level_begin.push_back((int32_t)rfwd.size());
    rfwd_launches += rfwd_level_begin[L] > rfwd_level_begin[L - 1];
  }
  rfwd_level_launches = rfwd_launches;
  recompute_updates = (int64_t)rfwd.size() * N;
  site_updates = (int64_t)V * N;
  const int64_t clv_b = (int64_t)R * S * (opts.precision == NETLK_FP32 ? 4 : 8);
  auto child_bytes = [&](int32_t ref) -> int64_t {
    if (ref >= 0) return clv_b + 4;
    if (ref == kFake) return 0;
    return S == 4 ? 1 : 4;  // tip state mask
  };
  fwd_bytes = 0;
  for (const FwdOp &op : fwd) {
    fwd_bytes += N * (clv_b + 4 + child_bytes(op.a) + child_bytes(op.b));
    if (op.slot >= 0) fwd_bytes += (int64_t)n_units_fwd * 8;
  }
  rfwd_bytes = 0;
  for (const FwdOp &op : rfwd) rfwd_bytes += N * (clv_b + 4 + child_bytes(op.a) + child_bytes(op.b));
  // adjoint: variants reachable backwards from the displayed-tree roots
  std::vector<char> inb(V, 0);
  for (auto &rv : dag.roots) inb[rv.dtroot_variant] = 1;
  for (int L = dag.n_levels; L >= 1; --L)
    for (int v : by_level[L])
      if (inb[v])
        for (int i = 0; i < 2; ++i)
          if (dag.vars[v].ref[i] >= 0) inb[dag.vars[v].ref[i]] = 1;
  bwd.clear();
  msg_slots.clear();
  bwd_level_begin.assign(1, 0);
  n_bwd_real = 0;
  bwd_bytes = 0;
  n_adj = 0;  // message buffers after liveness reuse
  // messages waiting for each variant: (sending variant, slot); an op sums
  // its messages in sender order, in every schedule, so the walk and the
  // level sweeps add them in the same order
  std::vector<std::vector<std::pair<int32_t, int32_t>>> pending(V);
  std::vector<int> free_slots;
  std::vector<int> bwd_var;  // variant id of each adjoint op
  for (int L = dag.n_levels; L >= 1; --L) {
    const size_t base = bwd.size();
    std::vector<int32_t> read_here;
    for (int x : by_level[L]) {
      if (!inb[x]) continue;
      BwdOp op{};
      op.x = var_slot[x];
      op.a = dag.vars[x].ref[0];  // variant ids until the message slots are placed
      op.b = dag.vars[x].ref[1];
      op.ea = dag.vars[x].edge[0];
      op.eb = dag.vars[x].edge[1];
      op.seed = slot_of[x];
      op.out_a = op.out_b = -1;
      op.msg_begin = (int32_t)msg_slots.size();
      op.msg_count = (int32_t)pending[x].size();
      std::sort(pending[x].begin(), pending[x].end());
      for (const auto &m : pending[x]) {
        msg_slots.push_back(m.second);
        read_here.push_back(m.second);
      }
      set_inline_msgs(op, msg_slots);
      pending[x].clear();
      bwd.push_back(op);
      bwd_var.push_back(x);
      n_bwd_real++;
    }
    // outputs of this level take buffers freed by earlier levels only: the
    // ops of one launch run concurrently
    auto alloc_slot = [&]() {
      if (!free_slots.empty()) {
        int s = free_slots.back();
        free_slots.pop_back();
        return s;
      }
      return n_adj++;
    };
    for (size_t j = base; j < bwd.size(); ++j) {
      BwdOp &op = bwd[j];
      if (op.a >= 0) {
        op.out_a = alloc_slot();
        pending[op.a].push_back({bwd_var[j], op.out_a});
      }
      if (op.b >= 0) {
        op.out_b = alloc_slot();
        pending[op.b].push_back({bwd_var[j], op.out_b});
      }
      int64_t b = 4 + child_bytes(op.a) + child_bytes(op.b) + (int64_t)op.msg_count * clv_b;
      if (op.seed >= 0) b += clv_b;
      if (op.out_a >= 0) b += clv_b;
      if (op.out_b >= 0) b += clv_b;
      bwd_bytes += N * b;
    }
    for (int32_t m : read_here) free_slots.push_back(m);
    bwd_level_begin.push_back((int32_t)bwd.size());
  }
  build_walk(inb, slot_of, by_level, bwd_var);
  for (size_t j = 0; j < bwd.size(); ++j) {  // variant ids -> CLV slots
    BwdOp &op = bwd[j];
    op.a = map_ref(op.a);
    op.b = map_ref(op.b);
    op.pad0 = (int32_t)j;  // the op's grad_partial row, wherever it is launched from
  }
  bwd_launches = 0;
  for (int L = 0; L < dag.n_levels; ++L) bwd_launches += bwd_level_begin[L + 1] > bwd_level_begin[L];
  // edge -> (adjoint op, side) entries for the gradient reduction
  edge_begin.assign(topo.n_edges + 1, 0);
  for (const BwdOp &op : bwd) {
    edge_begin[op.ea + 1]++;
    if (op.b != kFake) edge_begin[op.eb + 1]++;
  }
  for (int e = 0; e < topo.n_edges; ++e) edge_begin[e + 1] += edge_begin[e];
  edge_entries.assign(edge_begin.back(), 0);
  {
    std::vector<int32_t> fill(edge_begin.begin(), edge_begin.end() - 1);
    for (size_t j = 0; j < bwd.size(); ++j) {
      edge_entries[fill[bwd[j].ea]++] = (int32_t)(2 * j);
      if (bwd[j].b != kFake) edge_entries[fill[bwd[j].eb]++] = (int32_t)(2 * j + 1);
    }
  }
}

// Walk schedules: a lane only reads values it wrote itself, so every op can
// run in any topological order, one warp carrying its patterns through all
// of them. The forward order is a depth-first post-order from the top levels
// down, the child with the larger subtree first, so a child CLV is read soon
// after it was written (while it is still in L2), kept segment by segment:
// a segment's non-permanent CLV slots are reused by the next segment, and
// nothing outside a segment reads them. The adjoint runs the reverse order
// (top segment first), one launch per segment, each but the top one after a
// walk that recomputes the segment's non-permanent CLVs in forward walk
// order. Message slots are reused as soon as their reader has run; a message
// is handed over in registers only to the next op of the same launch.
// Called while the level schedule's adjoint ops still hold variant ids.
void netlk_ctx::build_walk(const std::vector<char> &inb, const std::vector<int> &slot_of,
                           const std::vector<std::vector<int>> &by_level, const std::vector<int> &bwd_var) {
  wfwd.clear();
  wrfwd.clear();
  wbwd.clear();
  wmsg_slots.clear();
  wfwd_var.clear();
  wrfwd_var.clear();
  wbwd_var.clear();
  wrfwd_range.assign(n_segments, {0, 0});
  wbwd_range.assign(n_segments, {0, 0});
  n_wadj = 0;
  walk_ok = false;
  if (S != 4) return;
  const int V = (int)dag.vars.size();
  auto map_ref = [&](int32_t r) { return r >= 0 ? var_slot[r] : r; };
  std::vector<int> seg_of_var(V, 0);
  for (int v = 0; v < V; ++v)
    for (int sg = 0; sg < n_segments; ++sg)
      if (dag.vars[v].level >= seg_lo[sg] && dag.vars[v].level <= seg_hi[sg]) seg_of_var[v] = sg;
  std::vector<double> size(V, 1.0);  // ordering heuristic: shared descendants counted per path
  for (int L = 1; L <= dag.n_levels; ++L)
    for (int v : by_level[L])
      for (int i = 0; i < 2; ++i)
        if (dag.vars[v].ref[i] >= 0) size[v] += size[dag.vars[v].ref[i]];
  std::vector<int> order;
  order.reserve(V);
  std::vector<char> seen(V, 0);
  std::vector<std::pair<int, int>> st;  // (variant, children visited)
  for (int L = dag.n_levels; L >= 1; --L)
    for (int v0 : by_level[L]) {
      if (seen[v0]) continue;
      seen[v0] = 1;
      st.assign(1, {v0, 0});
      while (!st.empty()) {
        const int v = st.back().first, k = st.back().second;
        int c[2] = {dag.vars[v].ref[0], dag.vars[v].ref[1]};
        if (c[1] >= 0 && (c[0] < 0 || size[c[1]] > size[c[0]])) std::swap(c[0], c[1]);
        if (k < 2) {
          st.back().second++;
          if (c[k] >= 0 && !seen[c[k]]) {
            seen[c[k]] = 1;
            st.push_back({c[k], 0});
          }
        } else {
          order.push_back(v);
          st.pop_back();
        }
      }
    }
  // segment by segment (a stable partition keeps the order topological)
  std::stable_sort(order.begin(), order.end(), [&](int u, int v) { return seg_of_var[u] < seg_of_var[v]; });
  for (int v : order) {
    const Variant &var = dag.vars[v];
    wfwd.push_back(FwdOp{var_slot[v], map_ref(var.ref[0]), map_ref(var.ref[1]), var.edge[0], var.edge[1],
                         slot_of[v], 0, 0});
    wfwd_var.push_back(v);
  }
  for (int sg = n_segments - 2; sg >= 0; --sg) {
    wrfwd_range[sg].first = (int32_t)wrfwd.size();
    for (int v : order)
      if (seg_of_var[v] == sg && !var_ckpt[v]) {
        const Variant &var = dag.vars[v];
        wrfwd.push_back(FwdOp{var_slot[v], map_ref(var.ref[0]), map_ref(var.ref[1]), var.edge[0], var.edge[1], -1,
                              0, 0});
        wrfwd_var.push_back(v);
      }
    wrfwd_range[sg].second = (int32_t)wrfwd.size();
  }
  std::vector<int> level_index(V, -1);
  for (size_t j = 0; j < bwd.size(); ++j) level_index[bwd_var[j]] = (int)j;
  std::vector<std::vector<std::pair<int32_t, int32_t>>> pending(V);
  std::vector<int> free_slots;
  // adjoint walk order, and how many adjoint ops send a message to each variant
  std::vector<int> radj;
  for (auto it = order.rbegin(); it != order.rend(); ++it)
    if (inb[*it]) radj.push_back(*it);
  std::vector<int> n_senders(V, 0);
  for (int x : radj)
    for (int i = 0; i < 2; ++i)
      if (dag.vars[x].ref[i] >= 0) n_senders[dag.vars[x].ref[i]]++;
  for (auto &r : wbwd_range) r = {-1, -1};
  int carried_to = -1;  // variant whose only message the previous op kept in registers
  for (size_t j = 0; j < radj.size(); ++j) {
    const int x = radj[j];
    // the next op of the same launch (segment), if any
    const int y = j + 1 < radj.size() && seg_of_var[radj[j + 1]] == seg_of_var[x] ? radj[j + 1] : -1;
    BwdOp op = bwd[level_index[x]];  // a, b still variant ids
    op.pad0 = level_index[x];
    op.pad4 = x == carried_to;  // the adjoint starts from the message in registers
    carried_to = -1;
    op.msg_begin = (int32_t)wmsg_slots.size();
    op.msg_count = (int32_t)pending[x].size();
    std::sort(pending[x].begin(), pending[x].end());
    for (const auto &m : pending[x]) wmsg_slots.push_back(m.second);
    set_inline_msgs(op, wmsg_slots);
    auto alloc_slot = [&]() {
      if (!free_slots.empty()) {
        const int sl = free_slots.back();
        free_slots.pop_back();
        return sl;
      }
      return n_wadj++;
    };
    op.out_a = op.out_b = -1;
    // a child that is the next op and hears from no other op gets its
    // message in registers (out = -2)
    auto keep = [&](int32_t c) { return c >= 0 && c == y && n_senders[c] == 1 && op.a != op.b; };
    if (keep(op.a)) {
      op.out_a = -2;
      carried_to = op.a;
    } else if (op.a >= 0) {
      op.out_a = alloc_slot();
      pending[op.a].push_back({x, op.out_a});
    }
    if (keep(op.b)) {
      op.out_b = -2;
      carried_to = op.b;
    } else if (op.b >= 0) {
      op.out_b = alloc_slot();
      pending[op.b].push_back({x, op.out_b});
    }
    for (const auto &m : pending[x]) free_slots.push_back(m.second);
    pending[x].clear();
    op.a = map_ref(op.a);
    op.b = map_ref(op.b);
    auto &rg = wbwd_range[seg_of_var[x]];
    if (rg.first < 0) rg.first = (int32_t)wbwd.size();
    wbwd.push_back(op);
    wbwd_var.push_back(x);
    rg.second = (int32_t)wbwd.size();
  }
  for (auto &r : wbwd_range)
    if (r.first < 0) r = {0, 0};
  // the walk shares the message buffers sized for the level schedule
  walk_ok = n_wadj <= std::max(1, n_adj) && (int)wbwd.size() == n_bwd_real;
}

// ------------------------------------------------------------ device setup
void netlk_ctx::allocate_and_upload(const netlk_partition *in) {
  const int V = (int)dag.vars.size();
  ppw = (32 / R) * kPPLBase;                 // patterns per adjoint unit
  const int ppw_f = (32 / R) * kPPLForward;  // patterns per forward unit
  // patterns: every partition padded to whole blocks of the largest launch
  // shape (8 warps x one forward unit each), so a block never spans two partitions
  const int align = 8 * ppw_f;
  N = 0;
  n_units = 0;
  for (auto &pi : parts) {
    pi.n_pad = (pi.n + align - 1) / align * align;
    pi.offset = N;
    pi.unit_begin = (int)(N / ppw_f);
    N += pi.n_pad;
    pi.unit_end = (int)(N / ppw_f);
  }
  n_units = (int)(N / ppw);
  n_units_fwd = (int)(N / ppw_f);
  int segments = opts.checkpoint_segments;
  if (segments <= 0) {
    size_t free_b = 0, total_b = 0;
    if (!opts.host_only && cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
    segments = opts.host_only ? 1 : choose_segments(free_b);
  }
  build_schedules(segments);
  if (opts.host_only) return;
  // host staging of tips / weights / unit map
  const uint32_t all_states = S == 4 ? 0xfu : 0xfffffu;
  std::vector<uint8_t> tips(S == 4 ? (size_t)topo.n_tips * N : 0, 0x0f);
  std::vector<uint32_t> tips32(S == 20 ? (size_t)topo.n_tips * N : 0, all_states);
  std::vector<double> weights(N, 0.0);
  std::vector<int32_t> unit_part(n_units);
  for (int p = 0; p < P; ++p) {
    const PartInfo &pi = parts[p];
    for (int t = 0; t < topo.n_tips; ++t)
      for (int s = 0; s < pi.n; ++s) {
        uint32_t code = in[p].tip_states[(size_t)t * pi.n + s] & all_states;
        if (!code) throw Error(NETLK_ERR_INVALID_ARGUMENT, "tip state mask 0");
        if (S == 4)
          tips[(size_t)t * N + pi.offset + s] = (uint8_t)code;
        else
          tips32[(size_t)t * N + pi.offset + s] = code;
      }
    for (int s = 0; s < pi.n; ++s) {
      double w = in[p].pattern_weights ? in[p].pattern_weights[s] : 1.0;
      if (!(w >= 0.0) || !std::isfinite(w)) throw Error(NETLK_ERR_INVALID_ARGUMENT, "pattern weight");
      weights[pi.offset + s] = w;
      parts[p].wsum += w;
    }
    for (int u = (int)(pi.offset / ppw); u < (int)((pi.offset + pi.n_pad) / ppw); ++u) unit_part[u] = p;
  }
  // invariant states: the AND of every tip's mask at a pattern, when it is one state
  inv_state.assign(N, -1);
  for (int p = 0; p < P; ++p) {
    const PartInfo &pi = parts[p];
    for (int s = 0; s < pi.n; ++s) {
      uint32_t common = all_states;
      for (int t = 0; t < topo.n_tips; ++t) common &= in[p].tip_states[(size_t)t * pi.n + s];
      if (common && !(common & (common - 1))) {
        int k = 0;
        while (!((common >> k) & 1u)) ++k;
        inv_state[pi.offset + s] = (int8_t)k;
      }
    }
  }
  const size_t real_sz = opts.precision == NETLK_FP32 ? 4 : 8;
  const size_t clv_per_var = (size_t)N * R * S * real_sz;
  (void)V;
  d_clv.alloc(clv_per_var * n_clv_slots, dev_bytes);
  d_scaler.alloc((size_t)N * n_clv_slots * 4, dev_bytes);
  d_adj.alloc(clv_per_var * std::max(1, n_adj), dev_bytes);
  d_msg_slots.alloc(std::max<size_t>(1, msg_slots.size()) * 4, dev_bytes);
  d_tips.alloc(S == 4 ? tips.size() : tips32.size() * 4, dev_bytes);
  d_weights.alloc(N * 8, dev_bytes);
  d_unit_part.alloc(n_units * 4, dev_bytes);
  d_fwd.alloc(fwd.size() * sizeof(FwdOp), dev_bytes);
  d_bwd.alloc(bwd.size() * sizeof(BwdOp), dev_bytes);
  d_rfwd.alloc(std::max<size_t>(1, rfwd.size()) * sizeof(FwdOp), dev_bytes);
  if (walk_ok) {
    d_wfwd.alloc(wfwd.size() * sizeof(FwdOp), dev_bytes);
    d_wrfwd.alloc(std::max<size_t>(1, wrfwd.size()) * sizeof(FwdOp), dev_bytes);
    d_wbwd.alloc(std::max<size_t>(1, wbwd.size()) * sizeof(BwdOp), dev_bytes);
    d_wmsg_slots.alloc(std::max<size_t>(1, wmsg_slots.size()) * 4, dev_bytes);
  }
  d_ifwd.alloc(fwd.size() * sizeof(FwdOp), dev_bytes);
  const size_t nm = (size_t)P * topo.n_edges * R * S * S;
  d_pmat64.alloc(nm * 8, dev_bytes);
  if (opts.precision == NETLK_FP32) d_pmat32.alloc(nm * 4, dev_bytes);
  d_lambda.alloc(P * S * 8, dev_bytes);
  d_U.alloc(P * S * S * 8, dev_bytes);
  d_Uinv.alloc(P * S * S * 8, dev_bytes);
  d_rates.alloc(P * R * 8, dev_bytes);
  d_gfrac.alloc(P * 8, dev_bytes);
  d_gfrac32.alloc(P * 4, dev_bytes);
  d_invt.alloc(N * 8, dev_bytes);
  d_invt32.alloc(N * 4, dev_bytes);
  d_rw.alloc(P * R * 8, dev_bytes);
  d_freqs.alloc(P * S * 8, dev_bytes);
  d_Q.alloc(P * S * S * 8, dev_bytes);
  d_brlen.alloc((size_t)topo.n_edges * (linkage == NETLK_BRLEN_LINKED ? 1 : P) * 8, dev_bytes);
  d_site_partial.alloc((size_t)n_slots * n_units_fwd * 8, dev_bytes);
  d_tree_logl.alloc((size_t)n_slots * P * 8, dev_bytes);
  d_root_slot.alloc(root_slot.size() * 4, dev_bytes);
  d_root_lp.alloc(dag.roots.size() * 8, dev_bytes);
  d_root_dlp.alloc(dag.roots.size() * std::max(1, topo.n_ret) * 8, dev_bytes);
  d_seeds.alloc((size_t)n_slots * P * 8, dev_bytes);
  if (opts.precision == NETLK_FP32) {
    auto up4 = [](size_t n) { return (n + 3) & ~(size_t)3; };  // 16-byte aligned sub-arrays
    m32_freqs = up4((size_t)P * S * S);
    m32_rw = m32_freqs + up4((size_t)P * S);
    m32_rates = m32_rw + up4((size_t)P * R);
    d_model32.alloc((m32_rates + up4((size_t)P * R)) * 4, dev_bytes);
    d_weights32.alloc(N * 8, dev_bytes);
    d_seeds32.alloc((size_t)n_slots * P * 4, dev_bytes);
  }
  d_wts.alloc((size_t)P * dag.roots.size() * 8, dev_bytes);
  d_dret.alloc((size_t)P * std::max(1, topo.n_ret) * 8, dev_bytes);
  d_slot_begin.alloc(slot_begin.size() * 4, dev_bytes);
  d_slot_roots.alloc(slot_roots.size() * 4, dev_bytes);
  d_parts.alloc(P * sizeof(DevPartition), dev_bytes);
  d_out.alloc((3 + P + topo.n_ret) * 8, dev_bytes);  // + the sweeps' fault word
  d_grad.alloc(topo.n_edges * 8, dev_bytes);

  CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  fwd_shape = bwd_shape = 0;
  d_grad_partial.alloc(std::max<size_t>(1, bwd.size()) * n_units * 2 * 8, dev_bytes);
  d_op_sum.alloc(std::max<size_t>(1, bwd.size()) * 2 * 8, dev_bytes);
  d_edge_begin.alloc(edge_begin.size() * 4, dev_bytes);
  d_edge_entries.alloc(std::max<size_t>(1, edge_entries.size()) * 4, dev_bytes);
  CUDA_OK(cudaMemcpyAsync(d_edge_begin.p, edge_begin.data(), edge_begin.size() * 4, cudaMemcpyHostToDevice, stream));
  if (!edge_entries.empty())
    CUDA_OK(cudaMemcpyAsync(d_edge_entries.p, edge_entries.data(), edge_entries.size() * 4,
                            cudaMemcpyHostToDevice, stream));

  std::vector<DevPartition> dparts(P);
  for (int p = 0; p < P; ++p) dparts[p] = DevPartition{parts[p].unit_begin, parts[p].unit_end};
  if (S == 4)
    CUDA_OK(cudaMemcpyAsync(d_tips.p, tips.data(), tips.size(), cudaMemcpyHostToDevice, stream));
  else
    CUDA_OK(cudaMemcpyAsync(d_tips.p, tips32.data(), tips32.size() * 4, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_weights.p, weights.data(), N * 8, cudaMemcpyHostToDevice, stream));
  std::vector<float> w32;
  if (opts.precision == NETLK_FP32) {
    w32.resize(2 * (size_t)N);
    for (int64_t g = 0; g < N; ++g) {
      const float hi = (float)weights[g];
      w32[2 * g] = hi;
      w32[2 * g + 1] = (float)(weights[g] - (double)hi);
    }
    CUDA_OK(cudaMemcpyAsync(d_weights32.p, w32.data(), N * 8, cudaMemcpyHostToDevice, stream));
  }
  CUDA_OK(cudaMemcpyAsync(d_unit_part.p, unit_part.data(), n_units * 4, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_fwd.p, fwd.data(), fwd.size() * sizeof(FwdOp), cudaMemcpyHostToDevice, stream));
  if (!rfwd.empty())
    CUDA_OK(cudaMemcpyAsync(d_rfwd.p, rfwd.data(), rfwd.size() * sizeof(FwdOp), cudaMemcpyHostToDevice, stream));
  if (walk_ok) {
    CUDA_OK(cudaMemcpyAsync(d_wfwd.p, wfwd.data(), wfwd.size() * sizeof(FwdOp), cudaMemcpyHostToDevice, stream));
    if (!wrfwd.empty())
      CUDA_OK(cudaMemcpyAsync(d_wrfwd.p, wrfwd.data(), wrfwd.size() * sizeof(FwdOp), cudaMemcpyHostToDevice, stream));
    if (!wbwd.empty())
      CUDA_OK(cudaMemcpyAsync(d_wbwd.p, wbwd.data(), wbwd.size() * sizeof(BwdOp), cudaMemcpyHostToDevice, stream));
    if (!wmsg_slots.empty())
      CUDA_OK(cudaMemcpyAsync(d_wmsg_slots.p, wmsg_slots.data(), wmsg_slots.size() * 4, cudaMemcpyHostToDevice,
                              stream));
  }
  if (!bwd.empty())
    CUDA_OK(cudaMemcpyAsync(d_bwd.p, bwd.data(), bwd.size() * sizeof(BwdOp), cudaMemcpyHostToDevice, stream));
  if (!msg_slots.empty())
    CUDA_OK(cudaMemcpyAsync(d_msg_slots.p, msg_slots.data(), msg_slots.size() * 4, cudaMemcpyHostToDevice,
                            stream));
  CUDA_OK(cudaMemcpyAsync(d_root_slot.p, root_slot.data(), root_slot.size() * 4, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_slot_begin.p, slot_begin.data(), slot_begin.size() * 4, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_slot_roots.p, slot_roots.data(), slot_roots.size() * 4, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_parts.p, dparts.data(), P * sizeof(DevPartition), cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaStreamSynchronize(stream));  // host staging vectors go out of scope

  h_brlen.alloc((size_t)topo.n_edges * (linkage == NETLK_BRLEN_LINKED ? 1 : P) * 8);
  h_root_lp.alloc(dag.roots.size() * 8);
  h_root_dlp.alloc(dag.roots.size() * std::max(1, topo.n_ret) * 8);
  h_out.alloc((3 + P + topo.n_ret) * 8);
  h_grad.alloc(topo.n_edges * 8);
  h_tree.alloc((size_t)n_slots * P * 8);
  h_ifwd.alloc(fwd.size() * sizeof(FwdOp));
}

void netlk_ctx::upload_model() {
  std::vector<double> lam(P * S), U(P * S * S), Ui(P * S * S), rates(P * R), rw(P * R), fr(P * S), Q(P * S * S);
  for (int p = 0; p < P; ++p) {
    PartInfo &pi = parts[p];
    pi.eig = gtr_eigen(S, pi.freqs.data(), pi.exch.data());
    if (!pi.explicit_rates) pi.rates = gamma_mean_rates(pi.alpha, R);
    std::copy(pi.eig.lambda.begin(), pi.eig.lambda.end(), lam.begin() + p * S);
    std::copy(pi.eig.U.begin(), pi.eig.U.end(), U.begin() + p * S * S);
    std::copy(pi.eig.Uinv.begin(), pi.eig.Uinv.end(), Ui.begin() + p * S * S);
    std::copy(pi.eig.Q.begin(), pi.eig.Q.end(), Q.begin() + p * S * S);
    // with invariant sites the rate categories carry 1 - pinv of the sites:
    // rates / (1 - pinv) keep the mean substitution rate at 1
    for (int k = 0; k < R; ++k) rates[p * R + k] = pi.rates[k] / (1.0 - pi.pinv);
    std::copy(pi.rate_weights.begin(), pi.rate_weights.end(), rw.begin() + p * R);
    std::copy(pi.freqs.begin(), pi.freqs.end(), fr.begin() + p * S);
  }
  CUDA_OK(cudaMemcpyAsync(d_lambda.p, lam.data(), lam.size() * 8, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_U.p, U.data(), U.size() * 8, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_Uinv.p, Ui.data(), Ui.size() * 8, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_rates.p, rates.data(), rates.size() * 8, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_rw.p, rw.data(), rw.size() * 8, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_freqs.p, fr.data(), fr.size() * 8, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_Q.p, Q.data(), Q.size() * 8, cudaMemcpyHostToDevice, stream));
  has_pinv = false;
  for (const PartInfo &pi : parts) has_pinv = has_pinv || pi.pinv > 0.0;
  if (has_pinv) {
    std::vector<double> gf(P), it(N, 0.0);
    std::vector<float> gf32(P), it32(N, 0.f);
    for (int p = 0; p < P; ++p) {
      const PartInfo &pi = parts[p];
      gf[p] = 1.0 - pi.pinv;
      gf32[p] = (float)gf[p];
      for (int s = 0; s < pi.n; ++s) {
        const int k = inv_state[pi.offset + s];
        if (k >= 0 && pi.pinv > 0.0) {  // relative to the rate mixture's weight 1 - pinv
          it[pi.offset + s] = pi.pinv * pi.freqs[k] / (1.0 - pi.pinv);
          it32[pi.offset + s] = (float)it[pi.offset + s];
        }
      }
    }
    CUDA_OK(cudaMemcpyAsync(d_gfrac.p, gf.data(), P * 8, cudaMemcpyHostToDevice, stream));
    CUDA_OK(cudaMemcpyAsync(d_gfrac32.p, gf32.data(), P * 4, cudaMemcpyHostToDevice, stream));
    CUDA_OK(cudaMemcpyAsync(d_invt.p, it.data(), N * 8, cudaMemcpyHostToDevice, stream));
    CUDA_OK(cudaMemcpyAsync(d_invt32.p, it32.data(), N * 4, cudaMemcpyHostToDevice, stream));
    CUDA_OK(cudaStreamSynchronize(stream));  // the host vectors go out of scope
  }
  std::vector<float> m32;
  if (opts.precision == NETLK_FP32) {
    m32.assign(d_model32.bytes / 4, 0.f);
    for (size_t i = 0; i < Q.size(); ++i) m32[i] = (float)Q[i];
    for (size_t i = 0; i < fr.size(); ++i) m32[m32_freqs + i] = (float)fr[i];
    for (size_t i = 0; i < rw.size(); ++i) m32[m32_rw + i] = (float)rw[i];
    for (size_t i = 0; i < rates.size(); ++i) m32[m32_rates + i] = (float)rates[i];
    CUDA_OK(cudaMemcpyAsync(d_model32.p, m32.data(), m32.size() * 4, cudaMemcpyHostToDevice, stream));
  }
  CUDA_OK(cudaStreamSynchronize(stream));
  model_dirty = false;
  clv_valid = false;
}

void netlk_ctx::upload_probs() {
  root_probabilities(topo, dag, ret_probs);
  const int nr = std::max(1, topo.n_ret);
  double *lp = h_root_lp.as<double>(), *dlp = h_root_dlp.as<double>();
  for (size_t i = 0; i < dag.roots.size(); ++i) {
    lp[i] = dag.roots[i].logprob;
    for (int k = 0; k < topo.n_ret; ++k) dlp[i * nr + k] = dag.roots[i].dlogprob[k];
  }
  CUDA_OK(cudaMemcpyAsync(d_root_lp.p, lp, dag.roots.size() * 8, cudaMemcpyHostToDevice, stream));
  if (topo.n_ret)
    CUDA_OK(cudaMemcpyAsync(d_root_dlp.p, dlp, dag.roots.size() * nr * 8, cudaMemcpyHostToDevice, stream));
  probs_dirty = false;
}

// Automatic checkpointing: every CLV is stored while all of them take at most
// 70 % of the free device memory; otherwise ceil(sqrt(levels)) segments, or
// more until the permanent + one segment's CLVs fit.
int netlk_ctx::choose_segments(size_t free_bytes) const {
  const size_t per = (size_t)N * R * S * (opts.precision == NETLK_FP32 ? 4 : 8) + (size_t)N * 4;
  const double budget = 0.7 * (double)free_bytes;
  if ((double)per * dag.vars.size() <= budget || dag.n_levels <= 1) return 1;
  const int n_levels = dag.n_levels;
  int k = (int)std::ceil(std::sqrt((double)n_levels));
  for (; k <= n_levels; ++k) {
    netlk_ctx probe;  // slot count of a k-segment split, host side only
    probe.dag = dag;
    probe.N = N;
    probe.R = R;
    probe.S = S;
    probe.opts = opts;
    probe.topo = topo;
    probe.device = -1;
    probe.build_schedules(k);
    if ((double)per * probe.n_clv_slots <= budget) return k;
  }
  return n_levels;
}

void netlk_ctx::enqueue(bool pm, bool fwd_on, bool reduce, bool mixk, bool bwd_on) {
  prof_mark(-1);
  if (pm) {
    launch_pmatrix(stream, P, topo.n_edges, R, S, d_lambda.as<double>(), d_U.as<double>(), d_Uinv.as<double>(),
                   d_rates.as<double>(), d_brlen.as<double>(), d_pmat64.as<double>(),
                   opts.precision == NETLK_FP32 ? d_pmat32.as<float>() : nullptr, len_stride());
    prof_mark(0);
  }
  const SweepParams sp = sweep();
  const MixParams mp = mix();
  if (use_tc && (fwd_on || bwd_on)) CUDA_OK(cudaMemsetAsync(sp.fault, 0, 8, stream));
  if (fwd_on) {
    if (use_tc)
      launch_forward20_tc(stream, sp, fwd_level_begin.data(), dag.n_levels, sms);
    else if (S == 20)
      launch_sweep20(stream, opts.precision, R, false, sp, fwd_level_begin.data(), dag.n_levels);
    else
      launch_forward(stream, opts.precision, R, fwd_shape, sp, fwd_level_begin.data(), dag.n_levels);
    prof_mark(1);
  }
  if (reduce) {
    launch_tree_reduce(stream, mp);
    prof_mark(2);
  }
  if (mixk) {
    launch_mix(stream, mp);
    prof_mark(3);
  }
  if (bwd_on && !bwd.empty()) {
    enqueue_adjoint(sp, bwd_shape);
    prof_mark(4);
    launch_grad_reduce(stream, (int)bwd.size(), topo.n_edges, n_units, d_edge_begin.as<int32_t>(),
                       d_edge_entries.as<int32_t>(), d_grad_partial.as<double>(), d_op_sum.as<double>(),
                       d_grad.as<double>(), opts.precision == NETLK_FP32);
    prof_mark(5);
  }
}

// The adjoint sweep with launch shape `bshape`: segments from the top, each
// but the top one after recomputing its non-permanent CLVs. Walk shapes run
// one walk launch per segment (and one recompute walk before it), level
// shapes one launch per level.
bool netlk_ctx::adjoint_walks(int bshape) const {
  return S == 4 && walk_ok && bshape >= num_level_shapes(opts.precision, R);
}

void netlk_ctx::enqueue_adjoint(const SweepParams &sp, int bshape) {
  const bool walk = adjoint_walks(bshape);
  SweepParams rp = sp;
  rp.fwd_ops = d_rfwd.as<FwdOp>();
  for (int sg = n_segments - 1; sg >= 0; --sg) {
    const int lo = seg_lo[sg], nl = seg_hi[sg] - seg_lo[sg] + 1;
    if (sg < n_segments - 1) {
      if (walk) {
        const auto rg = wrfwd_range[sg];
        if (rg.second > rg.first) {
          SweepParams wp = sp;
          wp.walk_fwd_ops = d_wrfwd.as<FwdOp>() + rg.first;
          wp.n_walk_fwd = rg.second - rg.first;
          launch_forward(stream, opts.precision, R, fwd_wshape, wp, nullptr, 0);
        }
      } else {
        const int32_t *rb = rfwd_level_begin.data() + (lo - 1);
        if (use_tc)
          launch_forward20_tc(stream, rp, rb, nl, sms);
        else if (S == 20)
          launch_sweep20(stream, opts.precision, R, false, rp, rb, nl);
        else
          launch_forward(stream, opts.precision, R, fwd_lshape, rp, rb, nl);
      }
    }
    if (walk) {
      const auto rg = wbwd_range[sg];
      if (rg.second > rg.first) {
        SweepParams wp = sp;
        wp.walk_bwd_ops = d_wbwd.as<BwdOp>() + rg.first;
        wp.n_walk_bwd = rg.second - rg.first;
        launch_backward(stream, opts.precision, R, bshape, wp, nullptr, 0);
      }
      continue;
    }
    const int32_t *bb = bwd_level_begin.data() + (dag.n_levels - seg_hi[sg]);
    if (use_tc)
      launch_backward20_tc(stream, sp, bb, nl, sms);
    else if (S == 20)
      launch_sweep20(stream, opts.precision, R, true, sp, bb, nl);
    else
      launch_backward(stream, opts.precision, R, bshape, sp, bb, nl);
  }
}

void netlk_ctx::run(cudaGraphExec_t *cache, bool pm, bool fwd_on, bool reduce, bool mixk, bool bwd_on) {
  const int n = (int)pm + (fwd_on ? fwd_launches : 0) + (int)reduce + (int)mixk +
                (bwd_on && !bwd.empty() ? bwd_launches + rfwd_launches + 2 : 0);
  if (fwd_on && pm) {  // every CLV recomputed from the current lengths
    clv_valid = !device_brlen;
    clv_brlen = dev_len();
    last_updates = site_updates;
  }
  if (!opts.use_cuda_graph || profiling) {
    enqueue(pm, fwd_on, reduce, mixk, bwd_on);
    launches += n;
    return;
  }
  if (!*cache) {
    cudaGraph_t graph;
    CUDA_OK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    enqueue(pm, fwd_on, reduce, mixk, bwd_on);
    CUDA_OK(cudaStreamEndCapture(stream, &graph));
    cudaError_t e = cudaGraphInstantiate(cache, graph, 0);
    cudaGraphDestroy(graph);
    CUDA_OK(e);
  }
  CUDA_OK(cudaGraphLaunch(*cache, stream));
  launches += n;
}

bool netlk_ctx::run_incremental() {
  if (!opts.incremental || !clv_valid || n_segments != 1 || device_brlen || profiling) return false;
  const int E = topo.n_edges;
  std::vector<char> dirty_edge(E, 0);
  {  // an edge is dirty when any partition's length of it changed
    const std::vector<double> &L = dev_len();
    const int np = linkage == NETLK_BRLEN_LINKED ? 1 : P;
    for (int p = 0; p < np; ++p)
      for (int e = 0; e < E; ++e) dirty_edge[e] |= L[(size_t)p * E + e] != clv_brlen[(size_t)p * E + e];
  }
  // with one segment the CLV slots are the variant ids; fwd is in level order
  std::vector<char> dirty(dag.vars.size(), 0);
  ifwd.clear();
  ifwd_level_begin.assign(1, 0);
  int n_launch = 0;
  for (int L = 0; L < dag.n_levels; ++L) {
    for (int i = fwd_level_begin[L]; i < fwd_level_begin[L + 1]; ++i) {
      const FwdOp &op = fwd[i];
      const bool d = dirty_edge[op.ea] || (op.eb >= 0 && dirty_edge[op.eb]) || (op.a >= 0 && dirty[op.a]) ||
                     (op.b >= 0 && dirty[op.b]);
      if (d) {
        dirty[op.out] = 1;
        ifwd.push_back(op);
      }
    }
    ifwd_level_begin.push_back((int32_t)ifwd.size());
    n_launch += ifwd_level_begin[L + 1] > ifwd_level_begin[L];
  }
  const SweepParams sp = sweep();
  const MixParams mp = mix();
  if (use_tc) CUDA_OK(cudaMemsetAsync(sp.fault, 0, 8, stream));
  launch_pmatrix(stream, P, topo.n_edges, R, S, d_lambda.as<double>(), d_U.as<double>(), d_Uinv.as<double>(),
                 d_rates.as<double>(), d_brlen.as<double>(), d_pmat64.as<double>(),
                 opts.precision == NETLK_FP32 ? d_pmat32.as<float>() : nullptr, len_stride());
  if (!ifwd.empty()) {
    std::memcpy(h_ifwd.p, ifwd.data(), ifwd.size() * sizeof(FwdOp));
    CUDA_OK(cudaMemcpyAsync(d_ifwd.p, h_ifwd.p, ifwd.size() * sizeof(FwdOp), cudaMemcpyHostToDevice, stream));
    SweepParams ip = sp;
    ip.fwd_ops = d_ifwd.as<FwdOp>();
    if (use_tc)
      launch_forward20_tc(stream, ip, ifwd_level_begin.data(), dag.n_levels, sms);
    else if (S == 20)
      launch_sweep20(stream, opts.precision, R, false, ip, ifwd_level_begin.data(), dag.n_levels);
    else
      launch_forward(stream, opts.precision, R, fwd_lshape, ip, ifwd_level_begin.data(), dag.n_levels);
  }
  launch_tree_reduce(stream, mp);
  launch_mix(stream, mp);
  launches += 3 + n_launch;
  clv_brlen = dev_len();
  last_updates = (int64_t)ifwd.size() * N;
  return true;
}

// isActiveBranch (src/helper/EdgeHelper.cpp:84-95): a displayed tree's
// configuration set is compatible with taking this edge's parent; always true
// for an edge that does not enter a reticulation.
std::vector<char> netlk_ctx::active_roots_of(int edge) const {
  const Topology &T = topo;
  const int child = T.edge_child[edge], k = T.node_ret[child];
  std::vector<char> act(dag.roots.size(), 1);
  if (k < 0) return act;
  const int want = edge == T.ret_second_edge[k] ? 1 : 0;
  const size_t n_cfg = (size_t)1 << T.n_ret;
  for (size_t i = 0; i < dag.roots.size(); ++i) {
    const Bits &set = dag.vars[dag.roots[i].variant].set;
    bool any = false;
    for (size_t t = 0; t < n_cfg && !any; ++t)
      if (set.test(t) && (int)((t >> k) & 1) == want) any = true;
    act[i] = any;
  }
  return act;
}

void netlk_ctx::partition_gradient(double *out) {
  prepare_state();
  const int E = topo.n_edges;
  if (bwd.empty()) {
    std::fill(out, out + (size_t)P * E, 0.0);
    return;
  }
  if (!d_part_unit_begin.p) {
    std::vector<int32_t> pub(P + 1);
    for (int p = 0; p < P; ++p) pub[p] = (int32_t)(parts[p].offset / ppw);
    pub[P] = n_units;
    int64_t scratch = 0;
    d_part_unit_begin.alloc(pub.size() * 4, scratch);
    d_op_sum_part.alloc(bwd.size() * P * 2 * 8, scratch);
    d_grad_part.alloc((size_t)P * E * 8, scratch);
    dev_bytes += scratch;
    CUDA_OK(cudaMemcpy(d_part_unit_begin.p, pub.data(), pub.size() * 4, cudaMemcpyHostToDevice));
  }
  launch_grad_reduce_partitions(stream, (int)bwd.size(), E, n_units, P, d_part_unit_begin.as<int32_t>(),
                                d_edge_begin.as<int32_t>(), d_edge_entries.as<int32_t>(),
                                d_grad_partial.as<double>(), d_op_sum_part.as<double>(), d_grad_part.as<double>(),
                                opts.precision == NETLK_FP32);
  launches += 2;
  CUDA_OK(cudaMemcpyAsync(out, d_grad_part.p, (size_t)P * E * 8, cudaMemcpyDeviceToHost, stream));
  CUDA_OK(cudaStreamSynchronize(stream));
  CUDA_OK(cudaGetLastError());
}

// Tangent schedule for edge e, level by level over the forward schedule (one
// checkpoint segment: CLV slots are variant ids): every variant whose
// subtree contains e, with its e-side child (mode 1: the child hangs from e;
// mode 2: the child contains e), tangent slots reused once their last reader's
// level has run, and the displayed-tree root slots it feeds. Returns the
// tangent slots needed, or -1 where a variant would contain e on both sides
// (impossible in a displayed tree; the caller then takes another path).
int netlk_ctx::tangent_schedule(int e, std::vector<TanOp> &ops, std::vector<int32_t> &level_begin,
                                std::vector<int32_t> &slots) const {
  const int V = (int)dag.vars.size();
  std::vector<int32_t> dirty_op(V, -1);  // variant -> its tangent op
  std::vector<int> last_read(V, -1);     // variant -> level of its last tangent reader
  ops.clear();
  slots.clear();
  level_begin.assign(1, 0);
  std::vector<int> lvl;
  for (int L = 0; L < dag.n_levels; ++L) {
    for (int i = fwd_level_begin[L]; i < fwd_level_begin[L + 1]; ++i) {
      const FwdOp &f = fwd[i];
      const bool fake = f.b == kFake;
      const bool da = f.a >= 0 && dirty_op[f.a] >= 0, db = f.b >= 0 && dirty_op[f.b] >= 0;
      const bool ua = f.ea == e, ub = !fake && f.eb == e;
      const int n_dirty = (int)da + (int)db + (int)ua + (int)ub;
      if (n_dirty == 0) continue;
      if (n_dirty > 1) return -1;
      TanOp t{};
      const bool side_a = da || ua;
      t.x = f.out;
      t.d = side_a ? f.a : f.b;
      t.o = side_a ? f.b : f.a;
      t.ed = side_a ? f.ea : f.eb;
      t.eo = side_a ? (fake ? -1 : f.eb) : f.ea;
      t.mode = (ua || ub) ? 1 : 2;
      t.td = -1;
      t.tx = -1;
      t.slot = f.slot;
      if (t.mode == 2) last_read[t.d] = L;
      dirty_op[f.out] = (int32_t)ops.size();
      ops.push_back(t);
      lvl.push_back(L);
      if (f.slot >= 0) slots.push_back(f.slot);
    }
    level_begin.push_back((int32_t)ops.size());
  }
  // tangent slots: an op's output is kept only if a later level reads it;
  // a slot read at level L is free again from level L + 1 on
  std::vector<int> free_slots;
  std::vector<std::vector<int>> release(dag.n_levels + 1);
  int n_slots_used = 0;
  for (int L = 0; L < dag.n_levels; ++L) {
    for (int j = level_begin[L]; j < level_begin[L + 1]; ++j) {
      TanOp &t = ops[j];
      if (t.mode == 2) t.td = ops[dirty_op[t.d]].tx;
      if (last_read[t.x] >= 0) {
        if (!free_slots.empty()) {
          t.tx = free_slots.back();
          free_slots.pop_back();
        } else {
          t.tx = n_slots_used++;
        }
        release[last_read[t.x]].push_back(t.tx);
      }
    }
    for (int sl : release[L]) free_slots.push_back(sl);
  }
  return n_slots_used;
}

bool netlk_ctx::edge_derivs_analytic(int e, int mode, double *d1, double *d2, int part) {
  if (n_segments != 1 || device_brlen) return false;
  prepare();
  const size_t real_b = opts.precision == NETLK_FP32 ? 4 : 8;
  const size_t plane = (size_t)N * R * S * real_b;  // one tangent plane (X' or X'')
  // DNA: one walk launch over the ops in walk order; 20 states: one launch
  // per level
  const bool walk = S == 4;
  const int64_t n_units = walk ? N / tangent_walk_patterns_per_unit(R) : 0;
  if (n_tan_cap < 0) {
    // set up once: the most tangent slots any edge needs, and the block maps
    int need = 0;
    std::vector<TanOp> ops;
    std::vector<int32_t> lb, sl;
    for (int k = 0; k < topo.n_edges; ++k) {
      const int nk = tangent_schedule(k, ops, lb, sl);
      need = std::max(need, walk && nk >= 0 ? walk_order(ops) : nk);
    }
    setup_tangent_blocks();
    size_t free_b = 0, total_b = 0;
    CUDA_OK(cudaMemGetInfo(&free_b, &total_b));
    if ((double)need * 2 * plane > 0.5 * (double)free_b) {  // too big: keep the full-gradient path
      n_tan_cap = 0;
      return false;
    }
    int64_t scratch = 0;
    d_tan.alloc(std::max<size_t>(1, (size_t)need) * 2 * plane, scratch);
    d_tan_ops.alloc(dag.vars.size() * sizeof(TanOp), scratch);
    d_tan_partial.alloc((size_t)std::max(1, n_slots) * 2 * (walk ? n_units : tan_blocks) * 8, scratch);
    if (walk) {
      std::vector<int32_t> pub(P + 1);
      for (int p = 0; p < P; ++p) pub[p] = (int32_t)(parts[p].offset / tangent_walk_patterns_per_unit(R));
      pub[P] = (int32_t)n_units;
      d_part_tunit_begin.alloc(pub.size() * 4, scratch);
      CUDA_OK(cudaMemcpy(d_part_tunit_begin.p, pub.data(), pub.size() * 4, cudaMemcpyHostToDevice));
    }
    d_tan_out.alloc((size_t)std::max(1, n_slots) * P * 2 * 8, scratch);
    d_tan_slots.alloc((size_t)std::max(1, n_slots) * 4, scratch);
    d_pderiv64.alloc((size_t)P * 2 * R * S * S * 8, scratch);
    d_pderiv32.alloc((size_t)P * 2 * R * S * S * 4, scratch);
    dev_bytes += scratch;
    h_tan_ops.alloc(dag.vars.size() * sizeof(TanOp));
    h_tan_out.alloc((size_t)std::max(1, n_slots) * P * 2 * 8);
    h_tan_slots.alloc((size_t)std::max(1, n_slots) * 4);
    n_tan_cap = need;
  }
  std::vector<TanOp> ops;
  std::vector<int32_t> lb, dslots;
  int need = tangent_schedule(e, ops, lb, dslots);
  if (walk && need >= 0) need = walk_order(ops);
  if (need < 0 || need > n_tan_cap || n_tan_cap == 0) return false;
  // CLVs and per-tree logL at the current lengths
  if (!run_incremental()) run(&graph_logl, true, true, true, true, false);
  CUDA_OK(cudaMemcpyAsync(h_tree.p, d_tree_logl.p, (size_t)n_slots * P * 8, cudaMemcpyDeviceToHost, stream));
  if (!ops.empty()) {
    std::memcpy(h_tan_ops.p, ops.data(), ops.size() * sizeof(TanOp));
    CUDA_OK(cudaMemcpyAsync(d_tan_ops.p, h_tan_ops.p, ops.size() * sizeof(TanOp), cudaMemcpyHostToDevice, stream));
    std::memcpy(h_tan_slots.p, dslots.data(), dslots.size() * 4);
    if (!dslots.empty())
      CUDA_OK(cudaMemcpyAsync(d_tan_slots.p, h_tan_slots.p, dslots.size() * 4, cudaMemcpyHostToDevice, stream));
    launch_pderiv(stream, P, R, S, d_lambda.as<double>(), d_U.as<double>(), d_Uinv.as<double>(), d_rates.as<double>(),
                  d_brlen.as<double>(), len_stride(), e, d_pderiv64.as<double>(),
                  opts.precision == NETLK_FP32 ? d_pderiv32.as<float>() : nullptr);
    TanParams tp = tan_params();
    tp.pderiv = opts.precision == NETLK_FP32 ? d_pderiv32.p : d_pderiv64.p;
    tp.tan = d_tan.p;
    tp.ops = d_tan_ops.as<TanOp>();
    tp.partial = d_tan_partial.as<double>();
    if (walk) {
      if (!launch_tangent_walk(stream, opts.precision, R, S, tp, (int)ops.size())) return false;
      tp.n_blocks = (int32_t)n_units;  // the reduction's partials are per walk unit
      tp.ff = opts.precision == NETLK_FP32;  // and float pairs in FP32 contexts
      launch_tangent_reduce(stream, tp, d_tan_slots.as<int32_t>(), (int)dslots.size(),
                            d_part_tunit_begin.as<int32_t>(), P, d_tan_out.as<double>());
    } else {
      if (!launch_tangent(stream, opts.precision, R, S, tp, lb.data(), dag.n_levels)) return false;
      launch_tangent_reduce(stream, tp, d_tan_slots.as<int32_t>(), (int)dslots.size(),
                            d_part_block_begin.as<int32_t>(), P, d_tan_out.as<double>());
    }
    if (!dslots.empty())
      CUDA_OK(cudaMemcpyAsync(h_tan_out.p, d_tan_out.p, (size_t)n_slots * P * 2 * 8, cudaMemcpyDeviceToHost, stream));
  }
  const int nout = 3 + P + topo.n_ret;
  CUDA_OK(cudaMemcpyAsync(h_out.p, d_out.p, nout * 8, cudaMemcpyDeviceToHost, stream));
  CUDA_OK(cudaStreamSynchronize(stream));
  CUDA_OK(cudaGetLastError());
  check_injected();
  const double *o = h_out.as<double>();
  if (use_tc && *reinterpret_cast<const int32_t *>(o + nout - 1) != 0)
    throw Error(NETLK_ERR_TIMEOUT, "tensor-core sweep: an MMA completion wait timed out");
  if (o[1] != 0.0 || !std::isfinite(o[0]))
    throw Error(NETLK_ERR_NUMERIC, "Invalid network likelihood: negative infinity or NaN");
  // per-tree l' and l'' (0 for trees without e), mixed per partition
  std::vector<char> has(n_slots, 0);
  for (int32_t sl : dslots) has[sl] = 1;
  const double *tl = h_tree.as<double>(), *tan = h_tan_out.as<double>();
  const std::vector<char> act = mode == 1 ? active_roots_of(e) : std::vector<char>(dag.roots.size(), 1);
  std::vector<double> D1(P, 0.0), D2(P, 0.0);  // per partition, w.r.t. its own length
  for (int p = 0; p < P; ++p) {
    auto a1 = [&](size_t i) { return has[root_slot[i]] ? tan[((size_t)root_slot[i] * P + p) * 2] : 0.0; };
    auto a2 = [&](size_t i) { return has[root_slot[i]] ? tan[((size_t)root_slot[i] * P + p) * 2 + 1] : 0.0; };
    auto ll = [&](size_t i) { return tl[(size_t)root_slot[i] * P + p]; };
    if (!mix_edge(mode, act, ll, a1, a2, nullptr, &D1[p], &D2[p]))
      throw Error(NETLK_ERR_NUMERIC, "no displayed tree contains the edge");
  }
  // the derivative of the total w.r.t. the length the caller moves: one
  // partition's own, all partitions' together, or the linked length of a
  // scaled context (partition p's length is s_p t)
  double T1 = 0.0, T2 = 0.0;
  for (int p = 0; p < P; ++p) {
    if (part >= 0 && p != part) continue;
    const double f = part < 0 && linkage == NETLK_BRLEN_SCALED ? scalers[p] : 1.0;
    T1 += f * D1[p];
    T2 += f * f * D2[p];
  }
  if (d1) *d1 = T1;
  if (d2) *d2 = T2;
  return true;
}

void netlk_ctx::setup_tangent_blocks() {
  if (tan_blocks > 0) return;
  const int ppb = tangent_patterns_per_block(R);
  if (N % ppb) throw Error(NETLK_ERR_INVALID_ARGUMENT, "tangent sweep: patterns not a whole number of blocks");
  const int nb = (int)(N / ppb);
  std::vector<int32_t> block_part(nb), pbb(P + 1);
  for (int p = 0; p < P; ++p) {
    pbb[p] = (int32_t)(parts[p].offset / ppb);
    for (int64_t b = parts[p].offset / ppb; b < (parts[p].offset + parts[p].n_pad) / ppb; ++b) block_part[b] = p;
  }
  pbb[P] = nb;
  int64_t scratch = 0;
  d_block_part.alloc(block_part.size() * 4, scratch);
  d_part_block_begin.alloc(pbb.size() * 4, scratch);
  dev_bytes += scratch;
  CUDA_OK(cudaMemcpy(d_block_part.p, block_part.data(), block_part.size() * 4, cudaMemcpyHostToDevice));
  CUDA_OK(cudaMemcpy(d_part_block_begin.p, pbb.data(), pbb.size() * 4, cudaMemcpyHostToDevice));
  tan_blocks = nb;
}

template <class LL, class A1, class A2>
bool netlk_ctx::mix_edge(int mode, const std::vector<char> &act, LL ll, A1 a1, A2 a2, double *logl, double *D1,
                         double *D2) const {
  const double min_lp = opts.min_interesting_tree_logprob;
  const size_t nr = dag.roots.size();
  if (logl) {  // the partition's logL over every tree, as the mixture kernel forms it
    double best = -INFINITY;
    for (size_t i = 0; i < nr; ++i)
      if (dag.roots[i].logprob >= min_lp) best = std::max(best, dag.roots[i].logprob + ll(i));
    if (opts.variant == NETLK_AVERAGE && best > -INFINITY) {
      double acc = 0.0;
      for (size_t i = 0; i < nr; ++i)
        if (dag.roots[i].logprob >= min_lp) acc += std::exp(dag.roots[i].logprob + ll(i) - best);
      best += std::log(acc);
    }
    *logl = best;
  }
  *D1 = *D2 = 0.0;
  if (opts.variant == NETLK_AVERAGE) {
    double m = -INFINITY;
    for (size_t i = 0; i < nr; ++i)
      if (act[i] && dag.roots[i].logprob >= min_lp) m = std::max(m, dag.roots[i].logprob + ll(i));
    if (!(m > -INFINITY)) return mode != 1;
    double z = 0.0, s1 = 0.0, s2 = 0.0;
    for (size_t i = 0; i < nr; ++i) {
      if (!act[i] || dag.roots[i].logprob < min_lp) continue;
      const double w = std::exp(dag.roots[i].logprob + ll(i) - m);
      const double g1 = a1(i);
      z += w;
      s1 += w * g1;
      s2 += w * (a2(i) + g1 * g1);
    }
    const double g = s1 / z;
    *D1 = g;
    *D2 = s2 / z - g * g;
    return true;
  }
  int best = -1;
  double score = -INFINITY;
  for (size_t i = 0; i < nr; ++i) {
    const double lpi = dag.roots[i].logprob;
    if (!act[i] || lpi < min_lp) continue;
    // mode 0: the tree the BEST mixture takes (ties to the lower index);
    // mode 1: the reference's choice by tree_logl * tree_prob
    const double v = mode == 1 ? ll(i) * std::exp(lpi) : lpi + ll(i);
    if (best < 0 || v > score) {
      score = v;
      best = (int)i;
    }
  }
  if (best < 0) return mode != 1;
  *D1 = a1(best);
  *D2 = a2(best);
  return true;
}

int netlk_ctx::walk_order(std::vector<TanOp> &ops) {
  const int n = (int)ops.size();
  std::unordered_map<int32_t, int> op_of;  // variant -> its op
  for (int j = 0; j < n; ++j) op_of[ops[j].x] = j;
  std::vector<std::vector<int>> readers(n);
  std::vector<int> roots;  // ops that take e's message itself
  for (int j = 0; j < n; ++j) {
    if (ops[j].mode == 1) {
      roots.push_back(j);
    } else {
      auto it = op_of.find(ops[j].d);
      if (it == op_of.end() || it->second >= j) return -1;
      readers[it->second].push_back(j);
    }
  }
  std::vector<int> order;
  order.reserve(n);
  std::vector<int> stack(roots.rbegin(), roots.rend());
  while (!stack.empty()) {
    const int j = stack.back();
    stack.pop_back();
    order.push_back(j);
    for (auto it = readers[j].rbegin(); it != readers[j].rend(); ++it) stack.push_back(*it);
  }
  if ((int)order.size() != n) return -1;
  std::vector<int> pos(n), last(n, -1);
  for (int q = 0; q < n; ++q) pos[order[q]] = q;
  for (int j = 0; j < n; ++j)
    for (int rd : readers[j]) last[j] = std::max(last[j], pos[rd]);
  std::vector<TanOp> out(n);
  std::vector<int32_t> slot_of(n, -1), free_slots;
  std::vector<std::vector<int32_t>> release(n);
  int used = 0;
  for (int q = 0; q < n; ++q) {
    const int j = order[q];
    TanOp t = ops[j];
    t.td = t.mode == 2 ? slot_of[op_of[t.d]] : -1;
    t.tx = -1;
    if (last[j] >= 0) {
      if (!free_slots.empty()) {
        t.tx = free_slots.back();
        free_slots.pop_back();
      } else {
        t.tx = used++;
      }
      slot_of[j] = t.tx;
      release[last[j]].push_back(t.tx);
    }
    for (int32_t sl : release[q]) free_slots.push_back(sl);  // read for the last time here
    out[q] = t;
  }
  ops.swap(out);
  return used;
}

int netlk_ctx::sumtable_schedule(int e, std::vector<TanOp> &ops, std::vector<int32_t> &gref,
                                 std::vector<int32_t> &gbegin, std::vector<int32_t> &slot_tab) const {
  std::vector<int32_t> lb, dslots;
  gref.clear();
  gbegin.clear();
  slot_tab.assign(n_slots, -1);
  if (tangent_schedule(e, ops, lb, dslots) < 0) return -1;
  const int need = walk_order(ops);
  if (need < 0) return -1;
  // the child whose CLV each root's path starts from (the message e carries);
  // tables sorted by it so the evaluation forms P I once per child
  std::vector<int32_t> origin(ops.size()), op_of(dag.vars.size(), -1);
  std::vector<std::pair<int32_t, int32_t>> roots_by_child;  // (child ref, op)
  for (size_t j = 0; j < ops.size(); ++j) {
    op_of[ops[j].x] = (int32_t)j;
    origin[j] = ops[j].mode == 1 ? ops[j].d : origin[op_of[ops[j].d]];
    if (ops[j].slot >= 0) roots_by_child.push_back({origin[j], (int32_t)j});
  }
  std::stable_sort(roots_by_child.begin(), roots_by_child.end(),
                   [](const std::pair<int32_t, int32_t> &a, const std::pair<int32_t, int32_t> &b) {
                     return a.first < b.first;
                   });
  for (size_t t = 0; t < roots_by_child.size(); ++t) {
    TanOp &op = ops[roots_by_child[t].second];
    slot_tab[op.slot] = (int32_t)t;
    op.slot = (int32_t)t;
    if (gref.empty() || gref.back() != roots_by_child[t].first) {
      gref.push_back(roots_by_child[t].first);
      gbegin.push_back((int32_t)t);
    }
  }
  gbegin.push_back((int32_t)roots_by_child.size());
  return need;
}

void netlk_ctx::sumtable_paths(const std::vector<TanOp> &ops, int n_tab, std::vector<int32_t> &path_ops,
                               std::vector<int32_t> &path_begin) const {
  std::unordered_map<int32_t, int> op_of;  // variant -> its op
  std::vector<int> op_of_tab(n_tab, -1);
  for (size_t j = 0; j < ops.size(); ++j) {
    op_of[ops[j].x] = (int)j;
    if (ops[j].slot >= 0) op_of_tab[ops[j].slot] = (int)j;
  }
  path_ops.clear();
  path_begin.assign(1, 0);
  for (int t = 0; t < n_tab; ++t) {
    for (int j = op_of_tab[t]; j >= 0;) {
      const TanOp &o = ops[j];
      const int32_t row[6] = {o.x, o.d, o.o, o.ed, o.eo, o.mode};
      path_ops.insert(path_ops.end(), row, row + 6);
      if (o.mode == 1) break;
      auto it = op_of.find(o.d);
      j = it == op_of.end() ? -1 : it->second;
    }
    path_begin.push_back((int32_t)(path_ops.size() / 6));
  }
}

bool netlk_ctx::sumtable_current(int e) const {
  if (stab_edge != e || stab_gen != model_gen || device_brlen || stab_probs != ret_probs) return false;
  const std::vector<double> &L = dev_len();
  const int E = topo.n_edges;
  for (size_t i = 0; i < L.size(); ++i)
    if ((int)(i % E) != e && L[i] != stab_lens[i]) return false;
  return true;
}

bool netlk_ctx::sumtable_build(int e) {
  stab_edge = -1;
  if (graph_stab) {  // captured for the previous tables
    cudaGraphExecDestroy(graph_stab);
    graph_stab = nullptr;
  }
  const bool prot = S == 20;  // 20 states: tables by reverse path walks
  if (n_segments != 1 || device_brlen || !(S == 4 || (prot && R <= 4)) || opts.host_only || !opts.sumtables)
    return false;
  prepare();
  const size_t real_b = opts.precision == NETLK_FP32 ? 4 : 8;
  const size_t plane = (size_t)N * R * S * real_b;  // one (pattern, rate, state) plane
  const int64_t n_warps = prot ? N * R / 32 : N / 32;  // evaluation partials per table
  if (stab_cap_work < 0) {
    // set up once: the most work slots, tables and path ops any edge needs
    int need = 0, tabs = 0;
    int64_t paths = 0;
    std::vector<TanOp> ops;
    std::vector<int32_t> gref, gbegin, slot_tab, pops, pbeg;
    for (int k = 0; k < topo.n_edges; ++k) {
      const int nk = sumtable_schedule(k, ops, gref, gbegin, slot_tab);
      if (nk < 0) continue;
      need = std::max(need, prot ? 0 : nk);
      tabs = std::max(tabs, gbegin.back());
      if (prot) {
        sumtable_paths(ops, gbegin.back(), pops, pbeg);
        paths = std::max<int64_t>(paths, (int64_t)pops.size() / 6);
      }
    }
    setup_tangent_blocks();
    size_t free_b = 0, total_b = 0;
    CUDA_OK(cudaMemGetInfo(&free_b, &total_b));
    const double bytes = ((double)need * S + tabs) * plane + (double)tabs * (N * 4 + n_warps * 3 * 8);
    if (bytes > 0.5 * (double)free_b) {  // too big: keep the tangent path
      stab_cap_work = 0;
      return false;
    }
    int64_t scratch = 0;
    d_stab_work.alloc(prot ? 16 : std::max<size_t>(1, (size_t)need * S) * plane, scratch);
    d_stab.alloc(std::max<size_t>(1, (size_t)tabs) * plane, scratch);
    d_stab_scaler.alloc(std::max<size_t>(1, (size_t)tabs) * N * 4, scratch);
    d_stab_partial.alloc(std::max<size_t>(1, (size_t)tabs) * 3 * n_warps * 8, scratch);
    if (prot) {
      d_stab_paths.alloc(((size_t)std::max<int64_t>(1, paths) * 6 + tabs + 1) * 4, scratch);
      h_stab_paths.alloc(((size_t)std::max<int64_t>(1, paths) * 6 + tabs + 1) * 4);
      stab_cap_path = paths;
    }
    d_stab_out.alloc((std::max<size_t>(1, (size_t)tabs) * P * 3 + 1) * 8, scratch);  // + the fault word
    d_stab_pm3_64.alloc((size_t)P * 3 * R * S * S * 8, scratch);
    d_stab_pm3_32.alloc((size_t)P * 3 * R * S * S * 4, scratch);
    d_stab_groups.alloc((size_t)(2 * tabs + 2) * 4, scratch);
    d_stab_ops.alloc(dag.vars.size() * sizeof(TanOp), scratch);
    d_part_warp_begin.alloc((size_t)(P + 1) * 4, scratch);
    dev_bytes += scratch;
    h_stab_pm3.alloc((size_t)P * 3 * R * S * S * 8);
    if (!sumtable_eval_setup(opts.precision, R, S)) {
      stab_cap_work = 0;
      return false;
    }
    h_stab_out.alloc((std::max<size_t>(1, (size_t)tabs) * P * 3 + 1) * 8);
    h_stab_ops.alloc(dag.vars.size() * sizeof(TanOp) + (size_t)(2 * tabs + 2) * 4);
    std::vector<int32_t> pwb(P + 1);  // each partition's evaluation warps
    for (int p = 0; p < P; ++p) pwb[p] = (int32_t)(prot ? parts[p].offset * R / 32 : parts[p].offset / 32);
    pwb[P] = (int32_t)n_warps;
    CUDA_OK(cudaMemcpy(d_part_warp_begin.p, pwb.data(), pwb.size() * 4, cudaMemcpyHostToDevice));
    stab_cap_work = std::max(1, need);  // 0 is kept for "not available"
    stab_cap_tab = tabs;
  }
  std::vector<TanOp> ops;
  std::vector<int32_t> gref, gbegin, slot_tab;
  const int need = sumtable_schedule(e, ops, gref, gbegin, slot_tab);
  const int n_tab = gbegin.empty() ? 0 : gbegin.back();
  if (need < 0 || (!prot && need > stab_cap_work) || stab_cap_work == 0 || n_tab > stab_cap_tab) return false;
  const int32_t lb[2] = {0, (int32_t)ops.size()};  // one walk over every op
  stab_n_tab = n_tab;
  stab_n_groups = (int)gref.size();
  stab_root_tab.assign(dag.roots.size(), -1);
  for (size_t i = 0; i < dag.roots.size(); ++i) stab_root_tab[i] = slot_tab[root_slot[i]];
  // CLVs and per-tree logL at the current parameters
  if (!run_incremental()) run(&graph_logl, true, true, true, true, false);
  CUDA_OK(cudaMemcpyAsync(h_tree.p, d_tree_logl.p, (size_t)n_slots * P * 8, cudaMemcpyDeviceToHost, stream));
  if (!ops.empty()) {
    unsigned char *hp = static_cast<unsigned char *>(h_stab_ops.p);
    std::memcpy(hp, ops.data(), ops.size() * sizeof(TanOp));
    CUDA_OK(cudaMemcpyAsync(d_stab_ops.p, hp, ops.size() * sizeof(TanOp), cudaMemcpyHostToDevice, stream));
    int32_t *hg = reinterpret_cast<int32_t *>(hp + dag.vars.size() * sizeof(TanOp));
    std::memcpy(hg, gref.data(), gref.size() * 4);
    std::memcpy(hg + gref.size(), gbegin.data(), gbegin.size() * 4);
    CUDA_OK(cudaMemcpyAsync(d_stab_groups.p, hg, (gref.size() + gbegin.size()) * 4, cudaMemcpyHostToDevice, stream));
    StabParams sp = stab_params();
    if (prot) {
      std::vector<int32_t> pops, pbeg;
      sumtable_paths(ops, n_tab, pops, pbeg);
      if ((int64_t)pops.size() / 6 > stab_cap_path) return false;
      // one reverse walk per tree costs about a quarter of a tangent-sweep op
      // per path op (measured on 40 taxa / 3 reticulations): past 16 path ops
      // per tangent op the build would cost over four tangent sweeps, more
      // than a Newton-Raphson search saves, so keep the tangent path
      if (pops.size() / 6 > 16 * ops.size()) return false;
      int32_t *hpth = h_stab_paths.as<int32_t>();
      std::memcpy(hpth, pops.data(), pops.size() * 4);
      std::memcpy(hpth + pops.size(), pbeg.data(), pbeg.size() * 4);
      CUDA_OK(cudaMemcpyAsync(d_stab_paths.p, hpth, (pops.size() + pbeg.size()) * 4, cudaMemcpyHostToDevice,
                              stream));
      sp.path_ops = d_stab_paths.as<int32_t>();
      sp.path_begin = d_stab_paths.as<int32_t>() + pops.size();
      if (!launch_sumtable_path20(stream, opts.precision, R, sp, n_tab)) return false;
    } else if (!launch_sumtable_build(stream, opts.precision, R, S, sp, lb, 1)) {
      return false;
    }
  }
  const int nout = 3 + P + topo.n_ret;
  CUDA_OK(cudaMemcpyAsync(h_out.p, d_out.p, nout * 8, cudaMemcpyDeviceToHost, stream));
  CUDA_OK(cudaStreamSynchronize(stream));
  CUDA_OK(cudaGetLastError());
  check_injected();
  const double *o = h_out.as<double>();
  if (o[1] != 0.0 || !std::isfinite(o[0]))
    throw Error(NETLK_ERR_NUMERIC, "Invalid network likelihood: negative infinity or NaN");
  stab_tree.assign(h_tree.as<double>(), h_tree.as<double>() + (size_t)n_slots * P);
  stab_lens = dev_len();
  stab_probs = ret_probs;
  stab_gen = model_gen;
  stab_edge = e;
  return true;
}

void netlk_ctx::sumtable_eval(int e, const double *len, bool per_part, int mode, double *logl, double *d1,
                             double *d2) {
  std::vector<double> lp(P);  // each partition's length of e
  for (int p = 0; p < P; ++p) {
    const double t = std::min(std::max(per_part ? len[p] : len[0], 1e-6), 100.0);
    lp[p] = !per_part && linkage == NETLK_BRLEN_SCALED ? scalers[p] * t : t;
  }
  if (stab_n_tab > 0) {
    // P, P', P'' of each partition's length, as pmatrix_kernel and
    // pderiv_kernel form them (rates scaled for +I as the device's)
    const int SS = S * S;
    const bool f32 = opts.precision == NETLK_FP32;
    double *h64 = h_stab_pm3.as<double>();
    float *h32 = h_stab_pm3.as<float>();
    std::vector<double> f(3 * S);  // per eigenvalue: the factor of order 0, 1, 2
    for (int p = 0; p < P; ++p) {
      const Eigen &eg = parts[p].eig;
      for (int r = 0; r < R; ++r) {
        const double rho = parts[p].rates[r] / (1.0 - parts[p].pinv), t = lp[p];
        for (int k = 0; k < S; ++k) {
          const double lr = eg.lambda[k] * rho, ed = std::exp(lr * t);
          f[k] = std::exp(eg.lambda[k] * (t * rho));
          f[S + k] = lr * ed;
          f[2 * S + k] = lr * lr * ed;
        }
        for (int o = 0; o < 3; ++o)
          for (int i = 0; i < S; ++i)
            for (int j = 0; j < S; ++j) {
              double v = 0.0;
              if (o == 0 && t == 0.0)
                v = i == j ? 1.0 : 0.0;
              else
                for (int k = 0; k < S; ++k) v += eg.U[i * S + k] * f[o * S + k] * eg.Uinv[k * S + j];
              const size_t idx = (((size_t)p * 3 + o) * R + r) * SS + i * S + j;
              if (f32) h32[idx] = (float)v;
              else h64[idx] = v;
            }
      }
    }
    const size_t tail = (size_t)std::max(1, stab_cap_tab) * P * 3;  // fault word, after the largest output
    auto enqueue_eval = [&]() {
      StabParams sp = stab_params();
      const size_t pm_b = (size_t)P * 3 * R * SS * (f32 ? 4 : 8);
      CUDA_OK(cudaMemcpyAsync(f32 ? d_stab_pm3_32.p : d_stab_pm3_64.p, h_stab_pm3.p, pm_b, cudaMemcpyHostToDevice,
                              stream));
      CUDA_OK(cudaMemsetAsync(sp.fault, 0, 8, stream));
      if (!launch_sumtable_eval(stream, opts.precision, R, S, sp, stab_n_tab, d_part_warp_begin.as<int32_t>(), P,
                                d_stab_out.as<double>()))
        throw Error(NETLK_ERR_UNSUPPORTED, "edge sumtables: unsupported state or rate count");
      CUDA_OK(cudaMemcpyAsync(h_stab_out.p, d_stab_out.p, (size_t)stab_n_tab * P * 3 * 8, cudaMemcpyDeviceToHost,
                              stream));
      CUDA_OK(cudaMemcpyAsync(h_stab_out.as<double>() + tail, sp.fault, 8, cudaMemcpyDeviceToHost, stream));
    };
    if (!opts.use_cuda_graph || profiling) {
      enqueue_eval();
    } else {
      if (!graph_stab) {
        cudaGraph_t graph;
        CUDA_OK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        try {
          enqueue_eval();
        } catch (...) {
          cudaStreamEndCapture(stream, &graph);
          if (graph) cudaGraphDestroy(graph);
          throw;
        }
        CUDA_OK(cudaStreamEndCapture(stream, &graph));
        cudaError_t err = cudaGraphInstantiate(&graph_stab, graph, 0);
        cudaGraphDestroy(graph);
        CUDA_OK(err);
      }
      CUDA_OK(cudaGraphLaunch(graph_stab, stream));
    }
    CUDA_OK(cudaStreamSynchronize(stream));
    CUDA_OK(cudaGetLastError());
    if (*reinterpret_cast<const int32_t *>(h_stab_out.as<double>() + tail))
      throw Error(NETLK_ERR_TIMEOUT, "edge sumtable evaluation: a bulk-copy wait timed out");
  }
  check_injected();
  const double *out = h_stab_out.as<double>();
  const std::vector<char> act = mode == 1 ? active_roots_of(e) : std::vector<char>(dag.roots.size(), 1);
  double T0 = 0.0, T1 = 0.0, T2 = 0.0;
  for (int p = 0; p < P; ++p) {
    const double lg = parts[p].pinv > 0.0 ? parts[p].wsum * std::log(1.0 - parts[p].pinv) : 0.0;
    auto q = [&](size_t i, int k) { return out[((size_t)stab_root_tab[i] * P + p) * 3 + k]; };
    auto ll = [&](size_t i) {
      return stab_root_tab[i] >= 0 ? q(i, 0) + lg : stab_tree[(size_t)root_slot[i] * P + p];
    };
    auto a1 = [&](size_t i) { return stab_root_tab[i] >= 0 ? q(i, 1) : 0.0; };
    auto a2 = [&](size_t i) { return stab_root_tab[i] >= 0 ? q(i, 2) : 0.0; };
    double L0, D1, D2;
    if (!mix_edge(mode, act, ll, a1, a2, &L0, &D1, &D2))
      throw Error(NETLK_ERR_NUMERIC, "no displayed tree contains the edge");
    if (!std::isfinite(L0) || !std::isfinite(D1) || !std::isfinite(D2))
      throw Error(NETLK_ERR_NUMERIC, "Invalid network likelihood: negative infinity or NaN");
    if (per_part) {
      if (logl) logl[p] = L0;
      if (d1) d1[p] = D1;
      if (d2) d2[p] = D2;
    } else {
      const double f = linkage == NETLK_BRLEN_SCALED ? scalers[p] : 1.0;
      T0 += L0;
      T1 += f * D1;
      T2 += f * f * D2;
    }
  }
  if (!per_part) {
    if (logl) *logl = T0;
    if (d1) *d1 = T1;
    if (d2) *d2 = T2;
  }
}

// Times every launch shape of the two sweeps once on this context's own
// workload (after one full evaluation with the default shapes, so the
// adjoint sweep sees real seeds) and keeps the fastest for the CUDA graphs.
// Launch counts of the chosen shapes (a walk shape issues one launch per chunk).
void netlk_ctx::count_launches() {
  if (S != 4) return;
  const SweepParams sp = sweep();
  fwd_launches = sweep_launches(opts.precision, R, fwd_shape, sp, false, fwd_level_begin.data(), dag.n_levels);
  if (bwd.empty()) return;
  if (!adjoint_walks(bwd_shape)) {
    bwd_launches = sweep_launches(opts.precision, R, bwd_shape, sp, true, bwd_level_begin.data(), dag.n_levels);
    rfwd_launches = rfwd_level_launches;
    return;
  }
  // one walk (in chunks of at most one wave) per segment, plus the recompute walks
  const int bw = sweep_launches(opts.precision, R, bwd_shape, sp, true, nullptr, 0);
  const int fw = sweep_launches(opts.precision, R, fwd_wshape, sp, false, nullptr, 0);
  bwd_launches = rfwd_launches = 0;
  for (int sg = 0; sg < n_segments; ++sg) {
    bwd_launches += wbwd_range[sg].second > wbwd_range[sg].first ? bw : 0;
    rfwd_launches += wrfwd_range[sg].second > wrfwd_range[sg].first ? fw : 0;
  }
}

void netlk_ctx::autotune() {
  tuned = true;
  // walk shapes only where the walk schedule exists (DNA)
  const int nls = S == 4 ? num_level_shapes(opts.precision, R) : 1;
  const int ns = S == 4 && walk_ok ? num_shapes(opts.precision, R) : nls;
  tune_fwd_ms.assign(ns, 0.0);
  tune_bwd_ms.assign(ns, 0.0);
  fwd_wshape = nls < ns ? nls : 0;
  if (const char *forced = std::getenv("NETLK_SHAPES")) {  // "fwd,bwd": fixed shapes, no timing
    int f = 0, b = 0;
    if (std::sscanf(forced, "%d,%d", &f, &b) == 2 && f >= 0 && f < ns && b >= 0 && b < ns) {
      fwd_shape = f;
      bwd_shape = b;
      fwd_lshape = f < nls ? f : 0;
      bwd_lshape = b < nls ? b : 0;
      if (f >= nls) fwd_wshape = f;
      count_launches();
      return;
    }
  }
  if (ns <= 1 || !opts.autotune) {
    count_launches();
    return;
  }
  std::memcpy(h_brlen.p, dev_len().data(), dev_len().size() * 8);
  CUDA_OK(cudaMemcpyAsync(d_brlen.p, h_brlen.p, dev_len().size() * 8, cudaMemcpyHostToDevice, stream));
  enqueue(true, true, true, true, true);
  cudaEvent_t e0, e1;
  CUDA_OK(cudaEventCreate(&e0));
  CUDA_OK(cudaEventCreate(&e1));
  const SweepParams sp = sweep();
  auto time_one = [&](bool backward, int sh) {
    float best = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
      // the adjoint (with its checkpoint recomputes) starts from a fresh forward
      if (backward) launch_forward(stream, opts.precision, R, fwd_shape, sp, fwd_level_begin.data(), dag.n_levels);
      CUDA_OK(cudaEventRecord(e0, stream));
      if (backward)
        enqueue_adjoint(sp, sh);
      else
        launch_forward(stream, opts.precision, R, sh, sp, fwd_level_begin.data(), dag.n_levels);
      CUDA_OK(cudaEventRecord(e1, stream));
      CUDA_OK(cudaEventSynchronize(e1));
      float ms = 0.f;
      CUDA_OK(cudaEventElapsedTime(&ms, e0, e1));
      if (rep) best = std::min(best, ms);
    }
    return (double)best;
  };
  for (int sh = 0; sh < ns; ++sh) tune_fwd_ms[sh] = time_one(false, sh);
  fwd_shape = (int)(std::min_element(tune_fwd_ms.begin(), tune_fwd_ms.end()) - tune_fwd_ms.begin());
  if (nls < ns)
    fwd_wshape = (int)(std::min_element(tune_fwd_ms.begin() + nls, tune_fwd_ms.end()) - tune_fwd_ms.begin());
  for (int sh = 0; sh < ns; ++sh) tune_bwd_ms[sh] = time_one(true, sh);
  CUDA_OK(cudaGetLastError());
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  fwd_shape = (int)(std::min_element(tune_fwd_ms.begin(), tune_fwd_ms.end()) - tune_fwd_ms.begin());
  bwd_shape = (int)(std::min_element(tune_bwd_ms.begin(), tune_bwd_ms.end()) - tune_bwd_ms.begin());
  fwd_lshape = (int)(std::min_element(tune_fwd_ms.begin(), tune_fwd_ms.begin() + nls) - tune_fwd_ms.begin());
  bwd_lshape = (int)(std::min_element(tune_bwd_ms.begin(), tune_bwd_ms.begin() + nls) - tune_bwd_ms.begin());
  count_launches();
}

void netlk_ctx::prepare_state() {
  if (opts.host_only) throw Error(NETLK_ERR_NO_DEVICE, "context was created host_only");
  CUDA_OK(cudaSetDevice(device));
  if (model_dirty) upload_model();
  if (probs_dirty) upload_probs();
  if (!tuned) autotune();
}

void netlk_ctx::prepare() {
  prepare_state();
  if (!device_brlen) {  // lengths set from device memory stay where they are
    std::memcpy(h_brlen.p, dev_len().data(), dev_len().size() * 8);
    CUDA_OK(cudaMemcpyAsync(d_brlen.p, h_brlen.p, dev_len().size() * 8, cudaMemcpyHostToDevice, stream));
  }
}

void netlk_ctx::finish(double *total, double *part_logl, double *d_brlen, double *d_ret) {
  const int nout = 3 + P + topo.n_ret;
  CUDA_OK(cudaMemcpyAsync(h_out.p, d_out.p, nout * 8, cudaMemcpyDeviceToHost, stream));
  if (d_brlen)
    CUDA_OK(cudaMemcpyAsync(h_grad.p, d_grad.p, topo.n_edges * 8, cudaMemcpyDeviceToHost, stream));
  CUDA_OK(cudaStreamSynchronize(stream));
  CUDA_OK(cudaGetLastError());
  prof_collect();
  read_results(total, part_logl, d_brlen, d_ret);
}

void netlk_ctx::read_results(double *total, double *part_logl, double *d_brlen, double *d_ret) {
  const int nout = 3 + P + topo.n_ret;
  const double *o = h_out.as<double>();
  check_injected();
  if (use_tc && *reinterpret_cast<const int32_t *>(o + nout - 1) != 0)
    throw Error(NETLK_ERR_TIMEOUT, "tensor-core sweep: an MMA completion wait timed out");
  if (o[1] != 0.0 || !std::isfinite(o[0]))
    throw Error(NETLK_ERR_NUMERIC, "Invalid network likelihood: negative infinity or NaN");
  if (total) *total = o[0];
  if (part_logl) std::memcpy(part_logl, o + 2, P * 8);
  if (d_ret && topo.n_ret) std::memcpy(d_ret, o + 2 + P, topo.n_ret * 8);
  if (d_brlen) std::memcpy(d_brlen, h_grad.p, topo.n_edges * 8);
}

// ------------------------------------------------------------------ C ABI
namespace netlk {
// Error text for context-free entry points (netlk_last_error(NULL)).
void set_global_error(const std::string &msg) { g_create_error = msg; }
}  // namespace netlk

namespace {

// Every failed call forgets the stored CLVs: an error thrown after a launch
// (a timed-out MMA wait, a CUDA error, a -inf logL) may leave them partial,
// so the next evaluation runs a full forward sweep instead of an
// incremental one over buffers it cannot trust.
template <class F>
int guarded(netlk_ctx *ctx, F &&f) {
  try {
    f();
    if (ctx) ctx->err.clear();
    return NETLK_OK;
  } catch (const Error &e) {
    if (ctx) {
      ctx->err = e.what();
      ctx->clv_valid = false;
      ctx->stab_edge = -1;  // the tables read the edge's child CLV at every evaluation
    } else {
      g_create_error = e.what();
    }
    return e.status;
  } catch (const std::bad_alloc &) {
    if (ctx) {
      ctx->err = "host allocation failed";
      ctx->clv_valid = false;
      ctx->stab_edge = -1;  // the tables read the edge's child CLV at every evaluation
    } else {
      g_create_error = "host allocation failed";
    }
    return NETLK_ERR_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    if (ctx) {
      ctx->err = e.what();
      ctx->clv_valid = false;
      ctx->stab_edge = -1;  // the tables read the edge's child CLV at every evaluation
    } else {
      g_create_error = e.what();
    }
    return NETLK_ERR_INVALID_ARGUMENT;
  }
}

void check_finite(const double *v, int n, const char *what, double lo, double hi) {
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(v[i]) || v[i] < lo || v[i] > hi)
      throw Error(NETLK_ERR_INVALID_ARGUMENT, std::string(what) + " out of range or not finite");
}

void set_brlen(netlk_ctx *c, const double *b) {
  check_finite(b, c->topo.n_edges, "branch length", 0.0, 1e300);
  c->brlen.assign(b, b + c->topo.n_edges);
  for (double &x : c->brlen) x = std::min(std::max(x, 1e-6), 100.0);  // brlen_min / brlen_max
  c->device_brlen = false;
  if (c->linkage == NETLK_BRLEN_UNLINKED)  // every partition the same lengths
    for (int p = 0; p < c->P; ++p) std::copy(c->brlen.begin(), c->brlen.end(), c->plen.begin() + (size_t)p * c->topo.n_edges);
  else if (c->linkage == NETLK_BRLEN_SCALED)
    c->refresh_scaled();
}

void set_probs(netlk_ctx *c, const double *p) {
  check_finite(p, c->topo.n_ret, "reticulation probability", 0.0, 1.0);
  c->ret_probs.assign(p, p + c->topo.n_ret);
  for (double &x : c->ret_probs) x = std::min(std::max(x, 1e-6), 1.0 - 1e-6);  // brprob_min / max
  c->probs_dirty = true;
}

}  // namespace

extern "C" {

int netlk_options_default(netlk_options *o) {
  if (!o) return NETLK_ERR_INVALID_ARGUMENT;
  o->variant = NETLK_AVERAGE;
  o->precision = NETLK_FP32;
  o->min_interesting_tree_logprob = std::log(1e-6);
  o->device = 0;
  o->use_cuda_graph = 1;
  o->host_only = 0;
  o->autotune = 1;
  o->tensor_cores = 1;
  o->checkpoint_segments = 0;
  o->incremental = 1;
  o->brlen_linkage = NETLK_BRLEN_LINKED;
  o->sumtables = 1;
  return NETLK_OK;
}

int netlk_create(const netlk_topology *topo, const netlk_partition *in_parts, int32_t n_parts,
                 const double *branch_lengths, const double *ret_first_probs, const netlk_options *opts,
                 netlk_ctx **out) {
  if (!out) return NETLK_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::unique_ptr<netlk_ctx> c(new netlk_ctx());
  g_create_error.clear();
  int st = guarded(nullptr, [&] {
    if (!topo || !in_parts || n_parts < 1 || !branch_lengths)
      throw Error(NETLK_ERR_INVALID_ARGUMENT, "null argument");
    if (opts) c->opts = *opts; else netlk_options_default(&c->opts);
    if (c->opts.variant != NETLK_AVERAGE && c->opts.variant != NETLK_BEST)
      throw Error(NETLK_ERR_INVALID_ARGUMENT, "variant");
    if (c->opts.precision != NETLK_FP32 && c->opts.precision != NETLK_FP64)
      throw Error(NETLK_ERR_INVALID_ARGUMENT, "precision");
    Topology &t = c->topo;
    t.n_nodes = topo->n_nodes;
    t.n_tips = topo->n_tips;
    t.n_edges = topo->n_edges;
    t.n_ret = topo->n_reticulations;
    t.root = topo->root;
    if (t.n_nodes <= 0 || t.n_edges <= 0 || t.n_ret < 0 || !topo->edge_parent || !topo->edge_child ||
        !topo->node_child_edges || (t.n_ret && (!topo->ret_node || !topo->ret_first_edge || !topo->ret_second_edge)))
      throw Error(NETLK_ERR_INVALID_ARGUMENT, "topology arrays");
    if (t.n_ret > NETLK_MAX_RETICULATIONS)
      throw Error(NETLK_ERR_UNSUPPORTED, "at most 16 reticulations are supported");
    t.edge_parent.assign(topo->edge_parent, topo->edge_parent + t.n_edges);
    t.edge_child.assign(topo->edge_child, topo->edge_child + t.n_edges);
    t.child_edge.assign(topo->node_child_edges, topo->node_child_edges + 2 * t.n_nodes);
    t.ret_node.assign(topo->ret_node, topo->ret_node + t.n_ret);
    t.ret_first_edge.assign(topo->ret_first_edge, topo->ret_first_edge + t.n_ret);
    t.ret_second_edge.assign(topo->ret_second_edge, topo->ret_second_edge + t.n_ret);
    t.validate_and_derive();
    c->P = n_parts;
    c->S = in_parts[0].states;
    c->R = in_parts[0].rate_cats;
    if (c->S != 4 && c->S != 20)
      throw Error(NETLK_ERR_UNSUPPORTED, "states must be 4 (DNA) or 20 (protein)");
    if (c->R != 1 && c->R != 2 && c->R != 4 && (c->R != 8 || c->S != 4))
      throw Error(NETLK_ERR_UNSUPPORTED, "rate_cats must be 1, 2, 4 or 8 (at most 4 with 20 states)");
    c->use_tc = c->opts.tensor_cores && c->S == 20 && sweep20_tc_supported(c->opts.precision, c->R);
    c->parts.resize(n_parts);
    for (int p = 0; p < n_parts; ++p) {
      const netlk_partition &ip = in_parts[p];
      if (ip.states != c->S || ip.rate_cats != c->R)
        throw Error(NETLK_ERR_UNSUPPORTED, "all partitions of a context share states and rate_cats");
      if (ip.n_patterns <= 0 || !ip.tip_states || !ip.freqs || !ip.exchangeabilities)
        throw Error(NETLK_ERR_INVALID_ARGUMENT, "partition arrays");
      PartInfo &pi = c->parts[p];
      pi.n = ip.n_patterns;
      pi.freqs.assign(ip.freqs, ip.freqs + c->S);
      pi.exch.assign(ip.exchangeabilities, ip.exchangeabilities + c->S * (c->S - 1) / 2);
      pi.alpha = ip.alpha;
      if (!(ip.prop_invar >= 0.0 && ip.prop_invar <= 0.99))
        throw Error(NETLK_ERR_INVALID_ARGUMENT, "prop_invar must lie in [0, 0.99]");
      pi.pinv = ip.prop_invar;
      pi.explicit_rates = ip.rates != nullptr;
      if (ip.rates) {
        pi.rates.assign(ip.rates, ip.rates + c->R);
        check_finite(pi.rates.data(), c->R, "rate", 0.0, 1e300);
      }
      if (ip.rate_weights) pi.rate_weights.assign(ip.rate_weights, ip.rate_weights + c->R);
      else pi.rate_weights.assign(c->R, 1.0 / c->R);
      (void)gtr_eigen(c->S, pi.freqs.data(), pi.exch.data());  // validate now
      if (!pi.explicit_rates) (void)gamma_mean_rates(pi.alpha, c->R);
    }
    if (c->opts.brlen_linkage < NETLK_BRLEN_LINKED || c->opts.brlen_linkage > NETLK_BRLEN_SCALED)
      throw Error(NETLK_ERR_INVALID_ARGUMENT, "brlen_linkage");
    c->linkage = c->opts.brlen_linkage;
    c->scalers.assign(c->P, 1.0);
    if (c->linkage != NETLK_BRLEN_LINKED) c->plen.assign((size_t)c->P * t.n_edges, 0.0);
    set_brlen(c.get(), branch_lengths);
    if (t.n_ret) {
      if (!ret_first_probs) throw Error(NETLK_ERR_INVALID_ARGUMENT, "reticulation probabilities");
      set_probs(c.get(), ret_first_probs);
    }
    c->dag = compile_dag(t);
    if (c->opts.host_only) {
      c->device = -1;
      c->allocate_and_upload(in_parts);
      return;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
      throw Error(NETLK_ERR_NO_DEVICE, "no CUDA device");
    c->device = c->opts.device;
    if (c->device < 0 || c->device >= ndev) throw Error(NETLK_ERR_NO_DEVICE, "device ordinal");
    CUDA_OK(cudaSetDevice(c->device));
    CUDA_OK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->allocate_and_upload(in_parts);
    c->upload_model();
  });
  if (st != NETLK_OK) return st;
  *out = c.release();
  return NETLK_OK;
}

int netlk_destroy(netlk_ctx *ctx) {
  delete ctx;
  return NETLK_OK;
}

const char *netlk_last_error(const netlk_ctx *ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

const char *netlk_status_string(int s) {
  switch (s) {
    case NETLK_OK: return "ok";
    case NETLK_ERR_INVALID_ARGUMENT: return "invalid argument";
    case NETLK_ERR_TOPOLOGY: return "invalid topology";
    case NETLK_ERR_ENUMERATION: return "displayed-tree enumeration failed";
    case NETLK_ERR_CUDA: return "CUDA error";
    case NETLK_ERR_OUT_OF_MEMORY: return "out of memory";
    case NETLK_ERR_NUMERIC: return "non-finite log-likelihood";
    case NETLK_ERR_UNSUPPORTED: return "unsupported";
    case NETLK_ERR_NO_DEVICE: return "no CUDA device";
    case NETLK_ERR_TIMEOUT: return "timeout";
  }
  return "unknown status";
}

int netlk_get_dag_stats(const netlk_ctx *ctx, netlk_dag_stats *o) {
  if (!ctx || !o) return NETLK_ERR_INVALID_ARGUMENT;
  o->n_variants = (int32_t)ctx->dag.vars.size();
  o->n_root_variants = (int32_t)ctx->dag.roots.size();
  o->n_dtroot_slots = ctx->n_slots;
  o->n_levels = ctx->dag.n_levels;
  o->n_backward_ops = ctx->n_bwd_real;
  o->n_adjoint_slots = ctx->n_adj;
  o->max_variants_per_node = ctx->dag.max_per_node;
  o->n_degenerate = ctx->dag.n_degenerate;
  o->n_patterns_total = ctx->N;
  o->site_clv_updates = ctx->site_updates;
  o->tip_child_uses = ctx->tip_uses;
  o->fake_child_uses = ctx->fake_uses;
  o->device_bytes = ctx->dev_bytes;
  o->launches_per_gradient_eval =
      3 + ctx->fwd_launches + (ctx->bwd.empty() ? 0 : ctx->bwd_launches + ctx->rfwd_launches + 2);
  o->forward_bytes = ctx->fwd_bytes;
  o->backward_bytes = ctx->bwd_bytes;
  o->checkpoint_segments = ctx->n_segments;
  o->clv_slots = ctx->n_clv_slots;
  o->recompute_site_updates = ctx->recompute_updates;
  o->recompute_bytes = ctx->rfwd_bytes;
  return NETLK_OK;
}

int netlk_dag_export(const netlk_ctx *ctx, int32_t *node_of_variant, int32_t *children, int32_t *edges,
                     uint64_t *covered, int32_t words) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  const auto &d = ctx->dag;
  if (covered && words < (int32_t)d.words) return NETLK_ERR_INVALID_ARGUMENT;
  for (size_t v = 0; v < d.vars.size(); ++v) {
    if (node_of_variant) node_of_variant[v] = d.vars[v].node;
    if (children) {
      children[2 * v] = d.vars[v].ref[0];
      children[2 * v + 1] = d.vars[v].ref[1];
    }
    if (edges) {
      edges[2 * v] = d.vars[v].edge[0];
      edges[2 * v + 1] = d.vars[v].edge[1];
    }
    if (covered)
      for (int w = 0; w < words; ++w) covered[v * words + w] = w < (int)d.words ? d.vars[v].set.w[w] : 0;
  }
  return NETLK_OK;
}

int netlk_walk_export(const netlk_ctx *ctx, int32_t *n_fwd, int32_t *n_bwd, int32_t *n_slot_reads,
                      int32_t *fwd_variant, int32_t *bwd_ops, int32_t *slot_reads) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  const bool w = ctx->walk_ok;
  if (n_fwd) *n_fwd = w ? (int32_t)ctx->wfwd.size() : 0;
  if (n_bwd) *n_bwd = w ? (int32_t)ctx->wbwd.size() : 0;
  if (n_slot_reads) *n_slot_reads = w ? (int32_t)ctx->wmsg_slots.size() : 0;
  if (!w) return NETLK_OK;
  if (fwd_variant)
    for (size_t i = 0; i < ctx->wfwd.size(); ++i) fwd_variant[i] = ctx->wfwd_var[i];
  if (bwd_ops)
    for (size_t i = 0; i < ctx->wbwd.size(); ++i) {
      const BwdOp &o = ctx->wbwd[i];
      const int32_t row[6] = {ctx->wbwd_var[i], o.out_a, o.out_b, o.pad4, o.msg_begin, o.msg_count};
      for (int k = 0; k < 6; ++k) bwd_ops[6 * i + k] = row[k];
    }
  if (slot_reads)
    for (size_t i = 0; i < ctx->wmsg_slots.size(); ++i) slot_reads[i] = ctx->wmsg_slots[i];
  return NETLK_OK;
}

int netlk_walk_segments(const netlk_ctx *ctx, int32_t *n_segments, int32_t *n_recompute, int32_t *bwd_range,
                        int32_t *recompute_variant, int32_t *recompute_range) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  const bool w = ctx->walk_ok;
  if (n_segments) *n_segments = w ? ctx->n_segments : 0;
  if (n_recompute) *n_recompute = w ? (int32_t)ctx->wrfwd_var.size() : 0;
  if (!w) return NETLK_OK;
  for (int sg = 0; sg < ctx->n_segments; ++sg) {
    if (bwd_range) {
      bwd_range[2 * sg] = ctx->wbwd_range[sg].first;
      bwd_range[2 * sg + 1] = ctx->wbwd_range[sg].second;
    }
    if (recompute_range) {
      recompute_range[2 * sg] = ctx->wrfwd_range[sg].first;
      recompute_range[2 * sg + 1] = ctx->wrfwd_range[sg].second;
    }
  }
  if (recompute_variant)
    for (size_t i = 0; i < ctx->wrfwd_var.size(); ++i) recompute_variant[i] = ctx->wrfwd_var[i];
  return NETLK_OK;
}

int netlk_checkpoint_export(const netlk_ctx *ctx, int32_t *n_segments, int32_t *n_clv_slots, int32_t *var_slot,
                            int32_t *permanent, int32_t *seg_levels) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  if (n_segments) *n_segments = ctx->n_segments;
  if (n_clv_slots) *n_clv_slots = ctx->n_clv_slots;
  for (size_t v = 0; v < ctx->var_slot.size(); ++v) {
    if (var_slot) var_slot[v] = ctx->var_slot[v];
    if (permanent) permanent[v] = ctx->n_segments > 1 ? ctx->var_ckpt[v] : 1;
  }
  if (seg_levels)
    for (int s = 0; s < ctx->n_segments; ++s) {
      seg_levels[2 * s] = ctx->seg_lo[s];
      seg_levels[2 * s + 1] = ctx->seg_hi[s];
    }
  return NETLK_OK;
}

int netlk_adjoint_export(const netlk_ctx *ctx, int32_t *n_ops, int32_t *n_slot_reads, int32_t *n_levels,
                         int32_t *ops, int32_t *slot_reads, int32_t *level_begin) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  if (n_ops) *n_ops = (int32_t)ctx->bwd.size();
  if (n_slot_reads) *n_slot_reads = (int32_t)ctx->msg_slots.size();
  if (n_levels) *n_levels = (int32_t)ctx->bwd_level_begin.size() - 1;
  if (ops)
    for (size_t i = 0; i < ctx->bwd.size(); ++i) {
      const BwdOp &o = ctx->bwd[i];
      const int32_t row[7] = {o.x, o.a, o.b, o.out_a, o.out_b, o.msg_begin, o.msg_count};
      for (int k = 0; k < 7; ++k) ops[7 * i + k] = row[k];
    }
  if (slot_reads)
    for (size_t i = 0; i < ctx->msg_slots.size(); ++i) slot_reads[i] = ctx->msg_slots[i];
  if (level_begin)
    for (size_t i = 0; i < ctx->bwd_level_begin.size(); ++i) level_begin[i] = ctx->bwd_level_begin[i];
  return NETLK_OK;
}

int netlk_root_export(const netlk_ctx *ctx, int32_t *root_variant, int32_t *dtroot_variant, double *logprob) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  netlk_ctx *c = const_cast<netlk_ctx *>(ctx);
  return guarded(c, [&] {
    if (c->probs_dirty || logprob) root_probabilities(c->topo, c->dag, c->ret_probs);
    for (size_t i = 0; i < c->dag.roots.size(); ++i) {
      if (root_variant) root_variant[i] = c->dag.roots[i].variant;
      if (dtroot_variant) dtroot_variant[i] = c->dag.roots[i].dtroot_variant;
      if (logprob) logprob[i] = c->dag.roots[i].logprob;
    }
  });
}

int netlk_set_branch_lengths(netlk_ctx *ctx, const double *b, int32_t n) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (!b || n != ctx->topo.n_edges) throw Error(NETLK_ERR_INVALID_ARGUMENT, "branch length count");
    set_brlen(ctx, b);
  });
}

int netlk_set_reticulation_probs(netlk_ctx *ctx, const double *p, int32_t n) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (n != ctx->topo.n_ret || (n && !p)) throw Error(NETLK_ERR_INVALID_ARGUMENT, "reticulation count");
    set_probs(ctx, p);
  });
}

int netlk_set_model(netlk_ctx *ctx, int32_t part, const double *freqs, const double *exch, double alpha,
                    const double *rates) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (part < 0 || part >= ctx->P || !freqs || !exch) throw Error(NETLK_ERR_INVALID_ARGUMENT, "partition");
    PartInfo &pi = ctx->parts[part];
    std::vector<double> f(freqs, freqs + ctx->S), x(exch, exch + ctx->S * (ctx->S - 1) / 2);
    (void)gtr_eigen(ctx->S, f.data(), x.data());
    if (!rates) (void)gamma_mean_rates(alpha, ctx->R);
    pi.freqs = f;
    pi.exch = x;
    pi.alpha = alpha;
    pi.explicit_rates = rates != nullptr;
    if (rates) pi.rates.assign(rates, rates + ctx->R);
    ctx->model_dirty = true;
    ++ctx->model_gen;
  });
}

int netlk_set_prop_invar(netlk_ctx *ctx, int32_t part, double prop_invar) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (part < 0 || part >= ctx->P) throw Error(NETLK_ERR_INVALID_ARGUMENT, "partition");
    if (!(prop_invar >= 0.0 && prop_invar <= 0.99))
      throw Error(NETLK_ERR_INVALID_ARGUMENT, "prop_invar must lie in [0, 0.99]");
    ctx->parts[part].pinv = prop_invar;
    ctx->model_dirty = true;
    ++ctx->model_gen;
  });
}

int netlk_loglikelihood(netlk_ctx *ctx, double *total, double *part_logl, double *tree_partition_logl) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    ctx->prepare();
    if (!ctx->run_incremental()) ctx->run(&ctx->graph_logl, true, true, true, true, false);
    if (tree_partition_logl)
      CUDA_OK(cudaMemcpyAsync(ctx->h_tree.p, ctx->d_tree_logl.p, (size_t)ctx->n_slots * ctx->P * 8,
                              cudaMemcpyDeviceToHost, ctx->stream));
    ctx->finish(total, part_logl, nullptr, nullptr);
    if (tree_partition_logl) {
      const double *t = ctx->h_tree.as<double>();
      for (size_t i = 0; i < ctx->dag.roots.size(); ++i)
        for (int p = 0; p < ctx->P; ++p)
          tree_partition_logl[i * ctx->P + p] = ctx->dag.roots[i].logprob < ctx->opts.min_interesting_tree_logprob
                                                    ? NAN
                                                    : t[(size_t)ctx->root_slot[i] * ctx->P + p];
    }
  });
}

int netlk_loglikelihood_gradient(netlk_ctx *ctx, double *total, double *part_logl, double *d_brlen,
                                 double *d_retprob) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    ctx->prepare();
    ctx->run(&ctx->graph_grad, true, true, true, true, true);
    std::vector<double> g(ctx->topo.n_edges);
    ctx->finish(total, part_logl, g.data(), d_retprob);
    if (ctx->bwd.empty()) std::fill(g.begin(), g.end(), 0.0);
    if (d_brlen && ctx->linkage == NETLK_BRLEN_SCALED && !ctx->bwd.empty()) {
      // w.r.t. the linked length t_e: sum_p s_p d logL / d (s_p t_e)
      const int E = ctx->topo.n_edges;
      std::vector<double> gp((size_t)ctx->P * E);
      ctx->partition_gradient(gp.data());
      std::fill(g.begin(), g.end(), 0.0);
      for (int p = 0; p < ctx->P; ++p)
        for (int e = 0; e < E; ++e) g[e] += ctx->scalers[p] * gp[(size_t)p * E + e];
    }
    if (d_brlen) {
      // the gradient is taken w.r.t. the clamped length; zero where the clamp binds
      for (int e = 0; e < ctx->topo.n_edges; ++e) d_brlen[e] = g[e];
    }
  });
}

namespace {

// Roots on which an edge is active for the reference's derivative formula.
std::vector<char> active_roots(const netlk_ctx *c, int edge) { return c->active_roots_of(edge); }

// d logL / d t_edge as the reference's computeLoglikelihoodDerivatives
// computes it (src/likelihood/LikelihoodDerivatives.cpp:30-183), per
// partition: AVERAGE mixes only the trees on which the edge is active
// (numerator and denominator), BEST takes the derivative of the active tree
// with the largest tree_logl * tree_prob.
double reference_edge_d1(netlk_ctx *c, int edge) {
  const std::vector<char> act = active_roots(c, edge);
  const size_t nr = c->dag.roots.size();
  std::vector<double> g(c->topo.n_edges, 0.0);
  double tot = 0.0;
  c->prepare();
  if (c->opts.variant == NETLK_AVERAGE) {
    double *lp = c->h_root_lp.as<double>();
    for (size_t i = 0; i < nr; ++i)
      if (!act[i]) lp[i] = -INFINITY;
    CUDA_OK(cudaMemcpyAsync(c->d_root_lp.p, lp, nr * 8, cudaMemcpyHostToDevice, c->stream));
    c->probs_dirty = true;  // the next evaluation uploads the real log-probabilities again
    c->run(&c->graph_grad, true, true, true, true, true);
    c->finish(&tot, nullptr, g.data(), nullptr);
    return g[edge];
  }
  c->run(&c->graph_partials, true, true, true, false, false);
  CUDA_OK(cudaMemcpyAsync(c->h_tree.p, c->d_tree_logl.p, (size_t)c->n_slots * c->P * 8, cudaMemcpyDeviceToHost,
                          c->stream));
  CUDA_OK(cudaStreamSynchronize(c->stream));
  double *t = c->h_tree.as<double>();
  std::vector<double> keep((size_t)c->n_slots * c->P, -INFINITY);
  for (int p = 0; p < c->P; ++p) {
    int best = -1;
    double score = -INFINITY;
    for (size_t i = 0; i < nr; ++i) {
      const double lpi = c->dag.roots[i].logprob;
      if (!act[i] || lpi < c->opts.min_interesting_tree_logprob) continue;
      const double v = t[(size_t)c->root_slot[i] * c->P + p] * std::exp(lpi);
      if (v > score || best < 0) {
        score = v;
        best = (int)i;
      }
    }
    if (best < 0) throw Error(NETLK_ERR_NUMERIC, "no displayed tree contains the edge");
    const size_t sl = (size_t)c->root_slot[best] * c->P + p;
    keep[sl] = t[sl];
  }
  std::memcpy(t, keep.data(), keep.size() * 8);
  CUDA_OK(cudaMemcpyAsync(c->d_tree_logl.p, t, keep.size() * 8, cudaMemcpyHostToDevice, c->stream));
  c->run(&c->graph_mixbwd, false, false, false, true, true);
  c->finish(&tot, nullptr, g.data(), nullptr);
  return g[edge];
}

}  // namespace

int netlk_edge_derivatives(netlk_ctx *ctx, int32_t edge, int32_t mode, double *d1, double *d2) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (edge < 0 || edge >= ctx->topo.n_edges) throw Error(NETLK_ERR_INVALID_ARGUMENT, "edge");
    if (mode != 0 && mode != 1) throw Error(NETLK_ERR_INVALID_ARGUMENT, "mode must be 0 or 1");
    ctx->check_reference_mode(mode);
    // DNA: the edge's sumtables evaluated at the current lengths (built on
    // the first call for the edge and kept while only its lengths change,
    // so a Newton-Raphson loop that sets each proposal and asks for the
    // derivatives pays for one build per edge); else analytic d1 and d2
    // from one tangent sweep over the variants above the edge
    if (!ctx->device_brlen && (ctx->sumtable_current(edge) || ctx->sumtable_build(edge))) {
      const int E = ctx->topo.n_edges, P = ctx->P;
      if (ctx->linkage != NETLK_BRLEN_UNLINKED || P == 1) {
        const double t = ctx->linkage == NETLK_BRLEN_UNLINKED ? ctx->plen[edge] : ctx->brlen[edge];
        ctx->sumtable_eval(edge, &t, false, mode, nullptr, d1, d2);
      } else {  // each partition at its own length: the sum of the shares
        std::vector<double> t(P), a(P), b(P);
        for (int p = 0; p < P; ++p) t[p] = ctx->plen[(size_t)p * E + edge];
        ctx->sumtable_eval(edge, t.data(), true, mode, nullptr, a.data(), b.data());
        if (d1) *d1 = std::accumulate(a.begin(), a.end(), 0.0);
        if (d2) *d2 = std::accumulate(b.begin(), b.end(), 0.0);
      }
      return;
    }
    if (ctx->edge_derivs_analytic(edge, mode, d1, d2)) return;
    if (ctx->linkage != NETLK_BRLEN_LINKED)
      throw Error(NETLK_ERR_UNSUPPORTED,
                  "edge derivatives of per-partition lengths need one checkpoint segment and host lengths");
    // checkpointed contexts and device-resident lengths: d1 from full adjoint
    // sweeps, d2 as a central difference of d1 (below)
    auto first = [&]() -> double {
      if (mode == 1) return reference_edge_d1(ctx, edge);
      std::vector<double> g(ctx->topo.n_edges);
      double tot;
      ctx->prepare();
      ctx->run(&ctx->graph_grad, true, true, true, true, true);
      ctx->finish(&tot, nullptr, g.data(), nullptr);
      return ctx->bwd.empty() ? 0.0 : g[edge];
    };
    const double g0 = first();
    if (d1) *d1 = g0;
    if (d2) {  // central difference of the first derivative
      // FP64: a step of 1e-6 (second derivatives within ~1e-8 of the analytic
      // value), t/200 below t = 2e-4: near the 1e-6 length clamp a site that
      // needs a change on the branch has L ~ t, so d2 ~ -1/t^2 and only a step
      // well below t resolves it (30 % median error at the clamp with 1e-6,
      // 0.2 % with t/200). FP32: the first derivative carries rounding noise of
      // ~1e-5 relative, which a 1e-6 step amplifies to errors of tens of
      // percent, so the step grows with the length: t/200, but at least 1e-4
      // where that keeps t - h above a third of t (worst error ~2e-3 of the
      // analytic value on the golden cases, measured against t/100, t/50, 1e-4
      // and 1e-6).
      const double b0 = ctx->brlen[edge];
      const double h = ctx->opts.precision == NETLK_FP32
                           ? std::max(b0 / 200.0, std::min(1e-4, (b0 - 1e-6) / 3.0))
                           : std::min(1e-6, b0 / 200.0);
      // the edge gets its length back however this block is left
      struct Restore {
        double &len;
        double value;
        ~Restore() { len = value; }
      } restore{ctx->brlen[edge], b0};
      ctx->brlen[edge] = std::min(b0 + h, 100.0);
      const double hp = ctx->brlen[edge] - b0;
      const double gp = first();
      ctx->brlen[edge] = std::max(b0 - h, 1e-6);
      const double hm = b0 - ctx->brlen[edge];
      const double gm = first();
      ctx->brlen[edge] = b0;
      *d2 = (gp - gm) / (hp + hm);
    }
  });
}

int netlk_edge_loglikelihood(netlk_ctx *ctx, int32_t edge, double length, double *total) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (edge < 0 || edge >= ctx->topo.n_edges) throw Error(NETLK_ERR_INVALID_ARGUMENT, "edge");
    if (!std::isfinite(length) || length < 0.0) throw Error(NETLK_ERR_INVALID_ARGUMENT, "branch length");
    if (ctx->device_brlen)
      throw Error(NETLK_ERR_INVALID_ARGUMENT, "branch lengths are device-resident: set them on the host first");
    ctx->brlen[edge] = std::min(std::max(length, 1e-6), 100.0);
    const int E = ctx->topo.n_edges;
    if (ctx->linkage == NETLK_BRLEN_UNLINKED)  // every partition's length of the edge
      for (int p = 0; p < ctx->P; ++p) ctx->plen[(size_t)p * E + edge] = ctx->brlen[edge];
    else if (ctx->linkage == NETLK_BRLEN_SCALED)
      ctx->refresh_scaled();
    ctx->prepare();
    if (!ctx->run_incremental()) ctx->run(&ctx->graph_logl, true, true, true, true, false);
    ctx->finish(total, nullptr, nullptr, nullptr);
  });
}

int netlk_edge_loglikelihood_partition(netlk_ctx *ctx, int32_t edge, int32_t part, double length,
                                       double *total) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (ctx->linkage != NETLK_BRLEN_UNLINKED)
      throw Error(NETLK_ERR_UNSUPPORTED, "per-partition lengths need a NETLK_BRLEN_UNLINKED context");
    if (edge < 0 || edge >= ctx->topo.n_edges) throw Error(NETLK_ERR_INVALID_ARGUMENT, "edge");
    if (part < 0 || part >= ctx->P) throw Error(NETLK_ERR_INVALID_ARGUMENT, "partition");
    if (!std::isfinite(length) || length < 0.0) throw Error(NETLK_ERR_INVALID_ARGUMENT, "branch length");
    ctx->plen[(size_t)part * ctx->topo.n_edges + edge] = std::min(std::max(length, 1e-6), 100.0);
    ctx->prepare();
    if (!ctx->run_incremental()) ctx->run(&ctx->graph_logl, true, true, true, true, false);
    ctx->finish(total, nullptr, nullptr, nullptr);
  });
}

int netlk_edge_derivatives_partition(netlk_ctx *ctx, int32_t edge, int32_t part, int32_t mode, double *d1,
                                     double *d2) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (edge < 0 || edge >= ctx->topo.n_edges) throw Error(NETLK_ERR_INVALID_ARGUMENT, "edge");
    if (part < 0 || part >= ctx->P) throw Error(NETLK_ERR_INVALID_ARGUMENT, "partition");
    if (mode != 0 && mode != 1) throw Error(NETLK_ERR_INVALID_ARGUMENT, "mode must be 0 or 1");
    ctx->check_reference_mode(mode);
    // DNA: the edge's sumtables, every partition at its own current length
    if (!ctx->device_brlen && (ctx->sumtable_current(edge) || ctx->sumtable_build(edge))) {
      const int E = ctx->topo.n_edges, P = ctx->P;
      const std::vector<double> &L = ctx->dev_len();
      std::vector<double> t(P), a(P), b(P);
      for (int p = 0; p < P; ++p) t[p] = L[(size_t)p * (ctx->linkage == NETLK_BRLEN_LINKED ? 0 : E) + edge];
      ctx->sumtable_eval(edge, t.data(), true, mode, nullptr, a.data(), b.data());
      if (d1) *d1 = a[part];
      if (d2) *d2 = b[part];
      return;
    }
    if (!ctx->edge_derivs_analytic(edge, mode, d1, d2, part))
      throw Error(NETLK_ERR_UNSUPPORTED, "per-partition edge derivatives need one checkpoint segment and host lengths");
  });
}

int netlk_edge_sumtable(netlk_ctx *ctx, int32_t edge, int32_t *built, int32_t *n_tables) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (edge < 0 || edge >= ctx->topo.n_edges) throw Error(NETLK_ERR_INVALID_ARGUMENT, "edge");
    const bool ok = ctx->sumtable_build(edge);
    if (built) *built = ok ? 1 : 0;
    if (n_tables) *n_tables = ok ? ctx->stab_n_tab : 0;
  });
}

int netlk_edge_sumtable_derivatives(netlk_ctx *ctx, int32_t edge, const double *lengths, int32_t n_lengths,
                                    int32_t mode, double *logl, double *d1, double *d2) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    const int E = ctx->topo.n_edges, P = ctx->P;
    if (edge < 0 || edge >= E) throw Error(NETLK_ERR_INVALID_ARGUMENT, "edge");
    if (mode != 0 && mode != 1) throw Error(NETLK_ERR_INVALID_ARGUMENT, "mode must be 0 or 1");
    ctx->check_reference_mode(mode);
    if (!lengths || !(n_lengths == 1 || (n_lengths == P && ctx->linkage == NETLK_BRLEN_UNLINKED)))
      throw Error(NETLK_ERR_INVALID_ARGUMENT, "one length, or one per partition on an unlinked context");
    check_finite(lengths, n_lengths, "branch length", 0.0, 1e300);
    if (ctx->device_brlen)
      throw Error(NETLK_ERR_UNSUPPORTED, "branch lengths are device-resident: set them on the host first");
    if (ctx->sumtable_current(edge) || ctx->sumtable_build(edge)) {
      ctx->sumtable_eval(edge, lengths, n_lengths > 1, mode, logl, d1, d2);
      return;
    }
    // the tangent path at the proposed length; the lengths are put back
    // however this block is left
    struct Restore {
      netlk_ctx *c;
      std::vector<double> b, pl;
      ~Restore() {
        c->brlen = b;
        c->plen = pl;
      }
    } restore{ctx, ctx->brlen, ctx->plen};
    auto clamp = [](double t) { return std::min(std::max(t, 1e-6), 100.0); };
    if (n_lengths == 1) {
      ctx->brlen[edge] = clamp(lengths[0]);
      if (ctx->linkage == NETLK_BRLEN_UNLINKED)
        for (int p = 0; p < P; ++p) ctx->plen[(size_t)p * E + edge] = ctx->brlen[edge];
      else if (ctx->linkage == NETLK_BRLEN_SCALED)
        ctx->refresh_scaled();
    } else {
      for (int p = 0; p < P; ++p) ctx->plen[(size_t)p * E + edge] = clamp(lengths[p]);
    }
    ctx->prepare();
    if (!ctx->run_incremental()) ctx->run(&ctx->graph_logl, true, true, true, true, false);
    double total;
    std::vector<double> pl(P);
    ctx->finish(&total, pl.data(), nullptr, nullptr);
    const char *why = "edge derivatives need one checkpoint segment and host lengths";
    if (n_lengths == 1) {
      if (!ctx->edge_derivs_analytic(edge, mode, d1, d2)) throw Error(NETLK_ERR_UNSUPPORTED, why);
      if (logl) *logl = total;
    } else {
      for (int p = 0; p < P; ++p) {
        double a = 0.0, b = 0.0;
        if (!ctx->edge_derivs_analytic(edge, mode, &a, &b, p)) throw Error(NETLK_ERR_UNSUPPORTED, why);
        if (logl) logl[p] = pl[p];
        if (d1) d1[p] = a;
        if (d2) d2[p] = b;
      }
    }
  });
}

int netlk_sumtable_export(const netlk_ctx *ctx, int32_t edge, int32_t *n_ops, int32_t *n_work, int32_t *n_tables,
                          int32_t *n_groups, int32_t *ops, int32_t *group_ref, int32_t *group_begin) {
  if (!ctx || edge < 0 || edge >= ctx->topo.n_edges) return NETLK_ERR_INVALID_ARGUMENT;
  try {  // introspection: a failure leaves the context as it was
    std::vector<TanOp> o;
    std::vector<int32_t> gref, gbegin, slot_tab;
    const int need = ctx->sumtable_schedule(edge, o, gref, gbegin, slot_tab);
    if (need < 0) return NETLK_ERR_UNSUPPORTED;
    if (n_ops) *n_ops = (int32_t)o.size();
    if (n_work) *n_work = need;
    if (n_tables) *n_tables = gbegin.back();
    if (n_groups) *n_groups = (int32_t)gref.size();
    if (ops)
      for (size_t i = 0; i < o.size(); ++i) {
        const int32_t row[7] = {o[i].x, o[i].d, o[i].o, o[i].mode, o[i].td, o[i].tx, o[i].slot};
        for (int k = 0; k < 7; ++k) ops[7 * i + k] = row[k];
      }
    if (group_ref) std::copy(gref.begin(), gref.end(), group_ref);
    if (group_begin) std::copy(gbegin.begin(), gbegin.end(), group_begin);
  } catch (const std::bad_alloc &) {
    return NETLK_ERR_OUT_OF_MEMORY;
  }
  return NETLK_OK;
}

int netlk_set_partition_branch_lengths(netlk_ctx *ctx, int32_t part, const double *b, int32_t n) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (ctx->linkage != NETLK_BRLEN_UNLINKED)
      throw Error(NETLK_ERR_UNSUPPORTED, "per-partition lengths need a NETLK_BRLEN_UNLINKED context");
    if (part < 0 || part >= ctx->P) throw Error(NETLK_ERR_INVALID_ARGUMENT, "partition");
    if (!b || n != ctx->topo.n_edges) throw Error(NETLK_ERR_INVALID_ARGUMENT, "branch length count");
    check_finite(b, n, "branch length", 0.0, 1e300);
    for (int e = 0; e < n; ++e)
      ctx->plen[(size_t)part * n + e] = std::min(std::max(b[e], 1e-6), 100.0);
    ctx->device_brlen = false;
  });
}

int netlk_set_branch_length_scalers(netlk_ctx *ctx, const double *sc, int32_t n) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (ctx->linkage != NETLK_BRLEN_SCALED)
      throw Error(NETLK_ERR_UNSUPPORTED, "length scalers need a NETLK_BRLEN_SCALED context");
    if (!sc || n != ctx->P) throw Error(NETLK_ERR_INVALID_ARGUMENT, "scaler count");
    check_finite(sc, n, "branch length scaler", 1e-300, 1e300);
    ctx->scalers.assign(sc, sc + n);
    ctx->refresh_scaled();
  });
}

int netlk_partition_gradient(netlk_ctx *ctx, double *out) {
  if (!ctx || !out) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] { ctx->partition_gradient(out); });
}

int netlk_last_site_updates(const netlk_ctx *ctx, int64_t *site_updates) {
  if (!ctx || !site_updates) return NETLK_ERR_INVALID_ARGUMENT;
  *site_updates = ctx->last_updates;
  return NETLK_OK;
}

int netlk_tree_partials(netlk_ctx *ctx, double *out) {
  if (!ctx || !out) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    ctx->prepare();
    ctx->run(&ctx->graph_partials, true, true, true, false, false);
    CUDA_OK(cudaMemcpyAsync(ctx->h_tree.p, ctx->d_tree_logl.p, (size_t)ctx->n_slots * ctx->P * 8,
                            cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_OK(cudaStreamSynchronize(ctx->stream));
    const double *t = ctx->h_tree.as<double>();
    for (size_t i = 0; i < ctx->dag.roots.size(); ++i)
      for (int p = 0; p < ctx->P; ++p) out[i * ctx->P + p] = t[(size_t)ctx->root_slot[i] * ctx->P + p];
  });
}

int netlk_mix_and_backward(netlk_ctx *ctx, const double *global, double *total, double *part_logl,
                           double *d_brlen_partial, double *d_retprob) {
  if (!ctx || !global) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    ctx->prepare();
    // scatter the global (root variant, partition) sums back onto slots
    double *t = ctx->h_tree.as<double>();
    for (size_t i = 0; i < ctx->dag.roots.size(); ++i)
      for (int p = 0; p < ctx->P; ++p) t[(size_t)ctx->root_slot[i] * ctx->P + p] = global[i * ctx->P + p];
    CUDA_OK(cudaMemcpyAsync(ctx->d_tree_logl.p, t, (size_t)ctx->n_slots * ctx->P * 8, cudaMemcpyHostToDevice,
                            ctx->stream));
    ctx->run(&ctx->graph_mixbwd, false, false, false, true, true);
    std::vector<double> g(ctx->topo.n_edges, 0.0);
    ctx->finish(total, part_logl, g.data(), d_retprob);
    if (ctx->bwd.empty()) std::fill(g.begin(), g.end(), 0.0);
    if (d_brlen_partial) std::memcpy(d_brlen_partial, g.data(), g.size() * 8);
  });
}

int netlk_set_branch_lengths_device(netlk_ctx *ctx, const double *d_b, int32_t n) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (ctx->linkage != NETLK_BRLEN_LINKED)
      throw Error(NETLK_ERR_UNSUPPORTED, "device-resident lengths need linked branch lengths");
    if (ctx->opts.host_only) throw Error(NETLK_ERR_NO_DEVICE, "context was created host_only");
    if (!d_b || n != ctx->topo.n_edges) throw Error(NETLK_ERR_INVALID_ARGUMENT, "branch length count");
    CUDA_OK(cudaSetDevice(ctx->device));
    CUDA_OK(cudaMemcpyAsync(ctx->d_brlen.p, d_b, (size_t)n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->device_brlen = true;
  });
}

int netlk_enqueue(netlk_ctx *ctx, int32_t with_gradient) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (ctx->opts.host_only) throw Error(NETLK_ERR_NO_DEVICE, "context was created host_only");
    CUDA_OK(cudaSetDevice(ctx->device));
    if (ctx->model_dirty) ctx->upload_model();
    if (ctx->probs_dirty) ctx->upload_probs();
    if (!ctx->tuned) ctx->autotune();
    if (!ctx->device_brlen) {
      std::memcpy(ctx->h_brlen.p, ctx->brlen.data(), ctx->brlen.size() * 8);
      CUDA_OK(cudaMemcpyAsync(ctx->d_brlen.p, ctx->h_brlen.p, ctx->brlen.size() * 8, cudaMemcpyHostToDevice,
                              ctx->stream));
    }
    if (with_gradient)
      ctx->run(&ctx->graph_grad, true, true, true, true, true);
    else
      ctx->run(&ctx->graph_logl, true, true, true, true, false);
    if (ctx->profiling) ctx->prof_collect();
  });
}

int netlk_result_pointers(netlk_ctx *ctx, const double **d_out, const double **d_brlen) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (ctx->opts.host_only) throw Error(NETLK_ERR_NO_DEVICE, "context was created host_only");
    if (d_out) *d_out = ctx->d_out.as<double>();
    if (d_brlen) *d_brlen = ctx->d_grad.as<double>();
  });
}

int netlk_set_profiling(netlk_ctx *ctx, int32_t enable) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    ctx->profiling = enable != 0;
    ctx->prof_n = 0;
    for (int k = 0; k < 6; ++k) {
      ctx->prof_ms[k] = 0.0;
      ctx->prof_cnt[k] = 0;
    }
  });
}

int netlk_kernel_times(netlk_ctx *ctx, double *ms, int64_t *launches, int32_t n) {
  if (!ctx || n < 6) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (ctx->stream) CUDA_OK(cudaStreamSynchronize(ctx->stream));
    ctx->prof_collect();
    for (int k = 0; k < 6; ++k) {
      if (ms) ms[k] = ctx->prof_ms[k];
      if (launches) launches[k] = ctx->prof_cnt[k];
    }
  });
}

int netlk_get_clv(netlk_ctx *ctx, int32_t variant, int32_t part, double *clv, int32_t *scaler) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (variant < 0 || variant >= (int)ctx->dag.vars.size() || part < 0 || part >= ctx->P)
      throw Error(NETLK_ERR_INVALID_ARGUMENT, "variant / partition");
    if (ctx->opts.host_only) throw Error(NETLK_ERR_NO_DEVICE, "context was created host_only");
    if (!ctx->var_ckpt.empty() && ctx->n_segments > 1 && !ctx->var_ckpt[variant])
      throw Error(NETLK_ERR_UNSUPPORTED, "with checkpointing only the CLVs kept across segments are resident");
    CUDA_OK(cudaSetDevice(ctx->device));
    const PartInfo &pi = ctx->parts[part];
    variant = ctx->var_slot[variant];
    const size_t per = (size_t)ctx->R * ctx->S;
    const size_t n = (size_t)pi.n * per;
    if (clv) {
      if (ctx->opts.precision == NETLK_FP32) {
        std::vector<float> tmp(n);
        CUDA_OK(cudaMemcpy(tmp.data(), ctx->d_clv.as<float>() + ((size_t)variant * ctx->N + pi.offset) * per,
                           n * 4, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; ++i) clv[i] = tmp[i];
      } else {
        CUDA_OK(cudaMemcpy(clv, ctx->d_clv.as<double>() + ((size_t)variant * ctx->N + pi.offset) * per, n * 8,
                           cudaMemcpyDeviceToHost));
      }
    }
    if (scaler)
      CUDA_OK(cudaMemcpy(scaler, ctx->d_scaler.as<int32_t>() + (size_t)variant * ctx->N + pi.offset,
                         (size_t)pi.n * 4, cudaMemcpyDeviceToHost));
  });
}

int netlk_tuning(const netlk_ctx *ctx, int32_t *fwd_shape, int32_t *bwd_shape, double *fwd_ms, double *bwd_ms,
                 int32_t n) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  if (fwd_shape) *fwd_shape = ctx->fwd_shape;
  if (bwd_shape) *bwd_shape = ctx->bwd_shape;
  for (int i = 0; i < n; ++i) {
    if (fwd_ms) fwd_ms[i] = i < (int)ctx->tune_fwd_ms.size() ? ctx->tune_fwd_ms[i] : 0.0;
    if (bwd_ms) bwd_ms[i] = i < (int)ctx->tune_bwd_ms.size() ? ctx->tune_bwd_ms[i] : 0.0;
  }
  return NETLK_OK;
}

int netlk_walk_shape_begin(const netlk_ctx *ctx, int32_t *first_walk_shape) {
  if (!ctx || !first_walk_shape) return NETLK_ERR_INVALID_ARGUMENT;
  const int nls = ctx->S == 4 ? num_level_shapes(ctx->opts.precision, ctx->R) : 1;
  *first_walk_shape = ctx->S == 4 && ctx->walk_ok ? nls : (int32_t)ctx->tune_fwd_ms.size();
  return NETLK_OK;
}

int netlk_inject_failure(netlk_ctx *ctx, int32_t status) {
  if (!ctx || status < 0 || status > NETLK_ERR_TIMEOUT) return NETLK_ERR_INVALID_ARGUMENT;
  ctx->inject_status = status;
  return NETLK_OK;
}

int netlk_get_stream(netlk_ctx *ctx, void **stream) {
  if (!ctx || !stream) return NETLK_ERR_INVALID_ARGUMENT;
  *stream = (void *)ctx->stream;
  return NETLK_OK;
}

int netlk_launch_count(const netlk_ctx *ctx, int64_t *launches) {
  if (!ctx || !launches) return NETLK_ERR_INVALID_ARGUMENT;
  *launches = ctx->launches;
  return NETLK_OK;
}

}  // extern "C"

// ------------------------------------------------------- batched candidates
struct netlk_batch {
  std::vector<netlk_ctx *> ctxs;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t exec = nullptr;
  // persistent path: every context DNA, FP32, 4 rate categories, one
  // checkpoint segment, with walk schedules. A call is one graph of nine
  // launches: batched P-matrices, one persistent forward walk over every
  // (candidate, unit) item, batched site sums and mixtures, one persistent
  // adjoint walk, batched gradient reductions and a result gather, plus one
  // upload of all lengths and one download of all results.
  bool persistent = false, ready = false;
  int fshape = 0, bshape = 0;
  int64_t launches_per_call = 0;
  DevBuf d_cands, d_items_f, d_items_b2, d_items_b4, d_counter, d_results, d_lengths;
  PinnedBuf h_results, h_lengths;
  int n_items_f = 0, n_items_b2 = 0, n_items_b4 = 0;
  std::vector<int64_t> res_off, len_off;
  int64_t n_results = 0, n_lengths = 0, dev_bytes = 0;
  BatchParams base{};
  std::vector<double> tune_fwd_ms, tune_bwd_ms;

  BatchParams fwd_params() const {
    BatchParams p = base;
    p.items = d_items_f.as<int2>();
    p.n_items = n_items_f;
    return p;
  }
  BatchParams bwd_params(int shape) const {
    BatchParams p = base;
    const bool two = batch_shape_bwd_ppl(shape) == 2;
    p.items = two ? d_items_b2.as<int2>() : d_items_b4.as<int2>();
    p.n_items = two ? n_items_b2 : n_items_b4;
    return p;
  }

  static bool eligible(const netlk_ctx *c) {
    return c->S == 4 && c->R == 4 && c->opts.precision == NETLK_FP32 && c->n_segments == 1 && c->walk_ok;
  }

  // Device tables of every candidate, the work items (longest walks first),
  // and the walk shapes, timed on this batch.
  void setup_persistent() {
    const int n = (int)ctxs.size();
    std::vector<BatchCand> cands(n);
    res_off.assign(n, 0);
    len_off.assign(n, 0);
    n_results = n_lengths = 0;
    for (int i = 0; i < n; ++i) {
      const netlk_ctx *c = ctxs[i];
      res_off[i] = n_results;
      len_off[i] = n_lengths;
      n_results += 3 + c->P + c->topo.n_ret + c->topo.n_edges;
      n_lengths += c->topo.n_edges;
    }
    d_lengths.alloc(n_lengths * 8, dev_bytes);
    d_results.alloc(n_results * 8, dev_bytes);
    d_counter.alloc(16, dev_bytes);
    h_lengths.alloc(n_lengths * 8);
    h_results.alloc(n_results * 8);
    stage_lengths();
    BatchParams b{};
    for (int i = 0; i < n; ++i) {
      const netlk_ctx *c = ctxs[i];
      BatchCand &k = cands[i];
      k.sweep = c->sweep();
      k.mix = c->mix();
      k.lambda = c->d_lambda.as<double>();
      k.U = c->d_U.as<double>();
      k.Uinv = c->d_Uinv.as<double>();
      k.rates = c->d_rates.as<double>();
      k.brlen = d_lengths.as<double>() + len_off[i];
      k.pmat64 = c->d_pmat64.as<double>();
      k.pmat32 = c->d_pmat32.as<float>();
      k.n_pmat = (int64_t)c->P * c->topo.n_edges * 16 * 4;
      k.n_parts = c->P;
      k.n_edges = c->topo.n_edges;
      k.n_ops = (int32_t)c->bwd.size();
      k.n_bx = c->n_units;
      k.edge_begin = c->d_edge_begin.as<int32_t>();
      k.edge_entries = c->d_edge_entries.as<int32_t>();
      k.grad_partial = c->d_grad_partial.as<double>();
      k.op_sum = c->d_op_sum.as<double>();
      k.grad = c->d_grad.as<double>();
      k.out = c->d_out.as<double>();
      k.n_out = 3 + c->P + c->topo.n_ret;
      k.result_offset = res_off[i];
      b.max_pmat = std::max(b.max_pmat, k.n_pmat);
      b.max_slots = std::max(b.max_slots, c->n_slots);
      b.max_parts = std::max(b.max_parts, c->P);
      b.max_ops = std::max(b.max_ops, k.n_ops);
      b.max_edges = std::max(b.max_edges, k.n_edges);
    }
    d_cands.alloc(cands.size() * sizeof(BatchCand), dev_bytes);
    CUDA_OK(cudaMemcpy(d_cands.p, cands.data(), cands.size() * sizeof(BatchCand), cudaMemcpyHostToDevice));
    // items: candidates with the longest walks first, units in order
    auto items = [&](bool backward, int per_warp_units) {
      std::vector<int> order(n);
      for (int i = 0; i < n; ++i) order[i] = i;
      std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        const size_t la = backward ? ctxs[a]->wbwd.size() : ctxs[a]->wfwd.size();
        const size_t lc = backward ? ctxs[c]->wbwd.size() : ctxs[c]->wfwd.size();
        return la > lc;
      });
      std::vector<int2> out;
      for (int i : order) {
        const int units = (backward ? ctxs[i]->n_units : ctxs[i]->n_units_fwd) / per_warp_units;
        if (backward && ctxs[i]->bwd.empty()) continue;
        for (int u = 0; u < units; ++u) out.push_back(make_int2(i, u));
      }
      return out;
    };
    const std::vector<int2> f = items(false, 1), b2 = items(true, 1), b4 = items(true, 2);
    n_items_f = (int)f.size();
    n_items_b2 = (int)b2.size();
    n_items_b4 = (int)b4.size();
    d_items_f.alloc(std::max<size_t>(1, f.size()) * sizeof(int2), dev_bytes);
    d_items_b2.alloc(std::max<size_t>(1, b2.size()) * sizeof(int2), dev_bytes);
    d_items_b4.alloc(std::max<size_t>(1, b4.size()) * sizeof(int2), dev_bytes);
    if (!f.empty()) CUDA_OK(cudaMemcpy(d_items_f.p, f.data(), f.size() * sizeof(int2), cudaMemcpyHostToDevice));
    if (!b2.empty()) CUDA_OK(cudaMemcpy(d_items_b2.p, b2.data(), b2.size() * sizeof(int2), cudaMemcpyHostToDevice));
    if (!b4.empty()) CUDA_OK(cudaMemcpy(d_items_b4.p, b4.data(), b4.size() * sizeof(int2), cudaMemcpyHostToDevice));
    b.cands = d_cands.as<BatchCand>();
    b.n_cands = n;
    b.counter = d_counter.as<int32_t>();
    b.results = d_results.as<double>();
    base = b;
    // time every walk shape on this batch, forward and adjoint
    CUDA_OK(cudaMemcpyAsync(d_lengths.p, h_lengths.p, n_lengths * 8, cudaMemcpyHostToDevice, stream));
    const int ns = num_batch_shapes();
    tune_fwd_ms.assign(ns, 0.0);
    tune_bwd_ms.assign(ns, 0.0);
    cudaEvent_t e0, e1;
    CUDA_OK(cudaEventCreate(&e0));
    CUDA_OK(cudaEventCreate(&e1));
    auto time = [&](bool backward, int sh) {
      float best = 1e30f;
      for (int rep = 0; rep < 2; ++rep) {
        if (backward) launch_batch_forward(stream, fwd_params(), fshape);
        CUDA_OK(cudaEventRecord(e0, stream));
        if (backward)
          launch_batch_backward(stream, bwd_params(sh), sh);
        else
          launch_batch_forward(stream, fwd_params(), sh);
        CUDA_OK(cudaEventRecord(e1, stream));
        CUDA_OK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CUDA_OK(cudaEventElapsedTime(&ms, e0, e1));
        if (rep) best = std::min(best, ms);
      }
      return (double)best;
    };
    for (int sh = 0; sh < ns; ++sh) tune_fwd_ms[sh] = time(false, sh);
    fshape = (int)(std::min_element(tune_fwd_ms.begin(), tune_fwd_ms.end()) - tune_fwd_ms.begin());
    for (int sh = 0; sh < ns; ++sh) tune_bwd_ms[sh] = time(true, sh);
    bshape = (int)(std::min_element(tune_bwd_ms.begin(), tune_bwd_ms.end()) - tune_bwd_ms.begin());
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CUDA_OK(cudaGetLastError());
    ready = true;
  }

  // every context's host lengths into the pinned upload buffer
  void stage_lengths() {
    for (size_t i = 0; i < ctxs.size(); ++i)
      std::memcpy(h_lengths.as<double>() + len_off[i], ctxs[i]->brlen.data(), ctxs[i]->brlen.size() * 8);
  }

  void capture_persistent() {
    CUDA_OK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    CUDA_OK(cudaMemcpyAsync(d_lengths.p, h_lengths.p, n_lengths * 8, cudaMemcpyHostToDevice, stream));
    launch_batch_forward(stream, fwd_params(), fshape);
    launch_batch_backward(stream, bwd_params(bshape), bshape);
    CUDA_OK(cudaMemcpyAsync(h_results.p, d_results.p, n_results * 8, cudaMemcpyDeviceToHost, stream));
    cudaGraph_t graph;
    CUDA_OK(cudaStreamEndCapture(stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    CUDA_OK(e);
  }

  ~netlk_batch() {
    cudaSetDevice(device);
    for (DevBuf *b : {&d_cands, &d_items_f, &d_items_b2, &d_items_b4, &d_counter, &d_results, &d_lengths}) b->free();
    if (exec) cudaGraphExecDestroy(exec);
    for (cudaEvent_t e : join) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (stream) cudaStreamDestroy(stream);
  }

  // One graph: fork from the batch stream into every context's stream, per
  // context the branch-length upload, the logL + gradient launch sequence and
  // the result downloads, then join back.
  void capture() {
    CUDA_OK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    CUDA_OK(cudaEventRecord(fork, stream));
    for (size_t i = 0; i < ctxs.size(); ++i) {
      netlk_ctx *c = ctxs[i];
      const bool prof = c->profiling;
      c->profiling = false;
      CUDA_OK(cudaStreamWaitEvent(c->stream, fork, 0));
      CUDA_OK(cudaMemcpyAsync(c->d_brlen.p, c->h_brlen.p, c->brlen.size() * 8, cudaMemcpyHostToDevice,
                              c->stream));
      c->enqueue(true, true, true, true, true);
      CUDA_OK(cudaMemcpyAsync(c->h_out.p, c->d_out.p, (3 + c->P + c->topo.n_ret) * 8, cudaMemcpyDeviceToHost,
                              c->stream));
      CUDA_OK(cudaMemcpyAsync(c->h_grad.p, c->d_grad.p, c->topo.n_edges * 8, cudaMemcpyDeviceToHost, c->stream));
      CUDA_OK(cudaEventRecord(join[i], c->stream));
      CUDA_OK(cudaStreamWaitEvent(stream, join[i], 0));
      c->profiling = prof;
    }
    cudaGraph_t graph;
    CUDA_OK(cudaStreamEndCapture(stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    CUDA_OK(e);
  }
};


int netlk_batch_create(netlk_ctx *const *ctxs, int32_t n, netlk_batch **out) {
  return netlk_batch_create_ex(ctxs, n, NETLK_BATCH_AUTO, out);
}

int netlk_batch_create_ex(netlk_ctx *const *ctxs, int32_t n, int32_t mode, netlk_batch **out) {
  if (mode != NETLK_BATCH_AUTO && mode != NETLK_BATCH_PER_CONTEXT) {
    netlk::set_global_error("batch: mode must be NETLK_BATCH_AUTO or NETLK_BATCH_PER_CONTEXT");
    return NETLK_ERR_INVALID_ARGUMENT;
  }
  if (!ctxs || n <= 0 || !out) {
    netlk::set_global_error("batch: contexts and output pointer required, n > 0");
    return NETLK_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  return guarded(nullptr, [&] {
    auto b = std::make_unique<netlk_batch>();
    for (int i = 0; i < n; ++i) {
      if (!ctxs[i]) throw Error(NETLK_ERR_INVALID_ARGUMENT, "batch: context " + std::to_string(i) + " is NULL");
      if (ctxs[i]->opts.host_only)
        throw Error(NETLK_ERR_NO_DEVICE, "batch: context " + std::to_string(i) + " was created host_only");
      if (ctxs[i]->linkage != NETLK_BRLEN_LINKED)
        throw Error(NETLK_ERR_UNSUPPORTED, "batch: context " + std::to_string(i) + " has per-partition lengths");
      if (i && ctxs[i]->device != ctxs[0]->device)
        throw Error(NETLK_ERR_INVALID_ARGUMENT, "batch: all contexts must be on one device");
      for (int j = 0; j < i; ++j)
        if (ctxs[j] == ctxs[i]) throw Error(NETLK_ERR_INVALID_ARGUMENT, "batch: a context appears twice");
    }
    b->ctxs.assign(ctxs, ctxs + n);
    b->device = ctxs[0]->device;
    b->persistent = mode == NETLK_BATCH_AUTO;
    for (int i = 0; i < n; ++i) b->persistent = b->persistent && netlk_batch::eligible(ctxs[i]);
    if (b->persistent) b->launches_per_call = 9;
    CUDA_OK(cudaSetDevice(b->device));
    CUDA_OK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CUDA_OK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    b->join.resize(n);
    for (auto &e : b->join) CUDA_OK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    *out = b.release();
  });
}

int netlk_batch_loglikelihood_gradient(netlk_batch *b, double *totals, double *const *d_brlen,
                                       double *const *d_retprob) {
  if (!b) {
    netlk::set_global_error("batch: NULL batch");
    return NETLK_ERR_INVALID_ARGUMENT;
  }
  return guarded(nullptr, [&] {
    for (size_t i = 0; i < b->ctxs.size(); ++i) {
      netlk_ctx *c = b->ctxs[i];
      if (c->device_brlen)
        throw Error(NETLK_ERR_INVALID_ARGUMENT,
                    "batch: context " + std::to_string(i) + " has device-resident branch lengths");
      c->prepare_state();  // uploads and tuning happen outside the graph
      CUDA_OK(cudaStreamSynchronize(c->stream));
      c->clv_valid = false;  // the graph rewrites its CLVs; valid again once its results check out
      std::memcpy(c->h_brlen.p, c->brlen.data(), c->brlen.size() * 8);
    }
    CUDA_OK(cudaSetDevice(b->device));
    if (b->persistent) {
      if (!b->ready) b->setup_persistent();
      b->stage_lengths();
      if (!b->exec) b->capture_persistent();
      CUDA_OK(cudaGraphLaunch(b->exec, b->stream));
      CUDA_OK(cudaStreamSynchronize(b->stream));
      CUDA_OK(cudaGetLastError());
      const double *res = b->h_results.as<double>();
      for (size_t i = 0; i < b->ctxs.size(); ++i) {
        netlk_ctx *c = b->ctxs[i];
        const double *o = res + b->res_off[i];
        const int nout = 3 + c->P + c->topo.n_ret;
        if (o[1] != 0.0 || !std::isfinite(o[0]))
          throw Error(NETLK_ERR_NUMERIC, "batch: candidate " + std::to_string(i) +
                                             ": Invalid network likelihood: negative infinity or NaN");
        if (totals) totals[i] = o[0];
        if (d_retprob && d_retprob[i] && c->topo.n_ret) std::memcpy(d_retprob[i], o + 2 + c->P, c->topo.n_ret * 8);
        if (d_brlen && d_brlen[i]) {
          if (c->bwd.empty())
            std::fill(d_brlen[i], d_brlen[i] + c->topo.n_edges, 0.0);
          else
            std::memcpy(d_brlen[i], o + nout, c->topo.n_edges * 8);
        }
        c->clv_valid = true;  // every CLV now matches the context's host lengths
        c->clv_brlen = c->dev_len();
        c->last_updates = c->site_updates;
      }
      return;
    }
    if (!b->exec) b->capture();
    CUDA_OK(cudaGraphLaunch(b->exec, b->stream));
    CUDA_OK(cudaStreamSynchronize(b->stream));
    CUDA_OK(cudaGetLastError());
    for (size_t i = 0; i < b->ctxs.size(); ++i) {
      netlk_ctx *c = b->ctxs[i];
      c->launches += 1 + c->fwd_launches + 2 + (c->bwd.empty() ? 0 : c->bwd_launches + c->rfwd_launches + 2);
      std::vector<double> g(c->topo.n_edges, 0.0);
      double tot = 0.0;
      try {
        c->read_results(&tot, nullptr, g.data(), d_retprob ? d_retprob[i] : nullptr);
      } catch (const Error &e) {
        throw Error(e.status, "batch: candidate " + std::to_string(i) + ": " + e.what());
      }
      if (c->bwd.empty()) std::fill(g.begin(), g.end(), 0.0);
      c->clv_valid = true;  // every CLV now matches the context's host lengths
      c->clv_brlen = c->dev_len();
      c->last_updates = c->site_updates;
      if (totals) totals[i] = tot;
      if (d_brlen && d_brlen[i]) std::memcpy(d_brlen[i], g.data(), g.size() * 8);
    }
  });
}

int netlk_batch_info(const netlk_batch *b, int32_t *persistent, int64_t *launches_per_call, int32_t *fwd_shape,
                     int32_t *bwd_shape) {
  if (!b) return NETLK_ERR_INVALID_ARGUMENT;
  if (persistent) *persistent = b->persistent ? 1 : 0;
  if (launches_per_call) {
    int64_t n = b->launches_per_call;
    if (!b->persistent)
      for (const netlk_ctx *c : b->ctxs)
        n += 1 + c->fwd_launches + 2 + (c->bwd.empty() ? 0 : c->bwd_launches + c->rfwd_launches + 2);
    *launches_per_call = n;
  }
  if (fwd_shape) *fwd_shape = b->fshape;
  if (bwd_shape) *bwd_shape = b->bshape;
  return NETLK_OK;
}

int netlk_batch_destroy(netlk_batch *b) {
  delete b;
  return NETLK_OK;
}
