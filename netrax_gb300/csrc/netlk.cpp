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
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/netlk.h"
#include "internal.hpp"
#include "kernels.cuh"

using namespace netlk;

namespace {

thread_local std::string g_create_error;

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
  std::vector<PartInfo> parts;
  int64_t N = 0;
  int n_units = 0, ppw = 8;
  // schedules
  std::vector<FwdOp> fwd;
  std::vector<BwdOp> bwd;
  int n_slots = 0, n_adj = 0, n_bwd_real = 0;
  std::vector<int32_t> root_slot, slot_begin, slot_roots;
  int grid_fwd = 0, grid_bwd = 0;
  int64_t site_updates = 0, tip_uses = 0, fake_uses = 0;
  // device
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t dev_bytes = 0;
  DevBuf d_clv, d_scaler, d_adj, d_tips, d_weights, d_unit_part, d_fwd, d_bwd;
  DevBuf d_pmat64, d_pmat32, d_lambda, d_U, d_Uinv, d_rates, d_rw, d_freqs, d_Q, d_brlen;
  DevBuf d_site_partial, d_tree_logl, d_root_slot, d_root_lp, d_root_dlp, d_seeds, d_wts;
  DevBuf d_slot_begin, d_slot_roots, d_parts, d_out, d_grad_partial, d_grad;
  PinnedBuf h_brlen, h_root_lp, h_root_dlp, h_out, h_grad, h_tree;
  cudaGraphExec_t graph_logl = nullptr, graph_grad = nullptr, graph_partials = nullptr,
                  graph_mixbwd = nullptr;
  bool probs_dirty = true, model_dirty = true;
  int64_t launches = 0;
  std::string err;

  ~netlk_ctx() {
    if (device >= 0) cudaSetDevice(device);
    for (auto g : {graph_logl, graph_grad, graph_partials, graph_mixbwd})
      if (g) cudaGraphExecDestroy(g);
    for (DevBuf *b : {&d_clv, &d_scaler, &d_adj, &d_tips, &d_weights, &d_unit_part, &d_fwd, &d_bwd,
                      &d_pmat64, &d_pmat32, &d_lambda, &d_U, &d_Uinv, &d_rates, &d_rw, &d_freqs, &d_Q,
                      &d_brlen, &d_site_partial, &d_tree_logl, &d_root_slot, &d_root_lp, &d_root_dlp,
                      &d_seeds, &d_wts, &d_slot_begin, &d_slot_roots, &d_parts, &d_out, &d_grad_partial, &d_grad})
      b->free();
    if (stream) cudaStreamDestroy(stream);
  }

  SweepParams sweep() const {
    SweepParams p{};
    p.n_units = n_units;
    p.n_patterns = N;
    p.n_edges = topo.n_edges;
    p.n_fwd_ops = (int)fwd.size();
    p.n_bwd_ops = (int)bwd.size();
    p.n_parts = P;
    p.fwd_ops = d_fwd.as<FwdOp>();
    p.bwd_ops = d_bwd.as<BwdOp>();
    p.unit_part = d_unit_part.as<int32_t>();
    p.tips = d_tips.as<uint8_t>();
    p.weights = d_weights.as<double>();
    p.pmat = opts.precision == NETLK_FP32 ? d_pmat32.p : d_pmat64.p;
    p.freqs = d_freqs.as<double>();
    p.rate_weights = d_rw.as<double>();
    p.rates = d_rates.as<double>();
    p.Q = d_Q.as<double>();
    p.clv = d_clv.p;
    p.scaler = d_scaler.as<int32_t>();
    p.adj = d_adj.p;
    p.site_partial = d_site_partial.as<double>();
    p.seeds = d_seeds.as<double>();
    p.grad_partial = d_grad_partial.as<double>();
    return p;
  }

  MixParams mix() const {
    MixParams m{};
    m.n_slots = n_slots;
    m.n_parts = P;
    m.n_roots = (int)dag.roots.size();
    m.n_ret = topo.n_ret;
    m.variant = opts.variant;
    m.n_units = n_units;
    m.min_logprob = opts.min_interesting_tree_logprob;
    m.parts = d_parts.as<DevPartition>();
    m.site_partial = d_site_partial.as<double>();
    m.tree_logl = d_tree_logl.as<double>();
    m.root_slot = d_root_slot.as<int32_t>();
    m.root_logprob = d_root_lp.as<double>();
    m.root_dlogprob = d_root_dlp.as<double>();
    m.seeds = d_seeds.as<double>();
    m.weights = d_wts.as<double>();
    m.slot_begin = d_slot_begin.as<int32_t>();
    m.slot_roots = d_slot_roots.as<int32_t>();
    m.out = d_out.as<double>();
    return m;
  }

  void build_schedules();
  void allocate_and_upload(const netlk_partition *in_parts);
  void upload_model();
  void upload_probs();
  void enqueue(bool pm, bool fwd_on, bool reduce, bool mixk, bool bwd_on);
  void run(cudaGraphExec_t *cache, bool pm, bool fwd_on, bool reduce, bool mixk, bool bwd_on);
  void prepare();
  void finish(double *total, double *part_logl, double *d_brlen, double *d_ret);
};

// ------------------------------------------------------------------ schedules
void netlk_ctx::build_schedules() {
  const int V = (int)dag.vars.size();
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
  tip_uses = fake_uses = 0;
  for (int L = 1; L <= dag.n_levels; ++L) {
    for (int v : by_level[L]) {
      const Variant &var = dag.vars[v];
      FwdOp op{v, var.ref[0], var.ref[1], var.edge[0], var.edge[1], slot_of[v], 0, 0};
      fwd.push_back(op);
      tip_uses += is_tip_ref(var.ref[0]) + is_tip_ref(var.ref[1]);
      fake_uses += var.ref[1] == kFake;
    }
    while (fwd.size() % kGroup) fwd.push_back(FwdOp{-1, 0, 0, 0, 0, -1, 0, 0});
  }
  site_updates = (int64_t)V * N;
  // adjoint: variants reachable backwards from the displayed-tree roots
  std::vector<char> inb(V, 0);
  for (auto &rv : dag.roots) inb[rv.dtroot_variant] = 1;
  for (int L = dag.n_levels; L >= 1; --L)
    for (int v : by_level[L])
      if (inb[v])
        for (int i = 0; i < 2; ++i)
          if (dag.vars[v].ref[i] >= 0) inb[dag.vars[v].ref[i]] = 1;
  bwd.clear();
  n_bwd_real = 0;
  std::vector<int> adj_of(V, -1);
  std::vector<int> free_slots;
  n_adj = 0;
  auto alloc_slot = [&]() {
    if (!free_slots.empty()) {
      int s = free_slots.back();
      free_slots.pop_back();
      return s;
    }
    return n_adj++;
  };
  for (int L = dag.n_levels; L >= 1; --L) {
    std::vector<int> ops;
    for (int v : by_level[L])
      if (inb[v]) ops.push_back(v);
    for (size_t g0 = 0; g0 < ops.size(); g0 += kGroup) {
      const size_t g1 = std::min(ops.size(), g0 + kGroup);
      const size_t base = bwd.size();
      // phase 1 of the kernel: every op of the group reads its own adjoint
      for (size_t j = g0; j < g1; ++j) {
        const int x = ops[j];
        BwdOp op{};
        op.x = x;
        op.a = dag.vars[x].ref[0];
        op.b = dag.vars[x].ref[1];
        op.ea = dag.vars[x].edge[0];
        op.eb = dag.vars[x].edge[1];
        op.adj_x = adj_of[x];
        op.seed = slot_of[x];
        op.adj_a = op.adj_b = -1;
        bwd.push_back(op);
        n_bwd_real++;
      }
      for (size_t j = g0; j < g1; ++j)
        if (adj_of[ops[j]] >= 0) free_slots.push_back(adj_of[ops[j]]);
      // phase 2: children adjoints are stored (first writer) or accumulated
      for (size_t j = g0; j < g1; ++j) {
        BwdOp &op = bwd[base + (j - g0)];
        int modes[2] = {0, 0};
        int32_t refs[2] = {op.a, op.b};
        int32_t *dst[2] = {&op.adj_a, &op.adj_b};
        for (int i = 0; i < 2; ++i) {
          if (refs[i] < 0) continue;
          if (adj_of[refs[i]] < 0) {
            adj_of[refs[i]] = alloc_slot();
            modes[i] = 1;
          } else {
            modes[i] = 2;
          }
          *dst[i] = adj_of[refs[i]];
        }
        op.modes = modes[0] | (modes[1] << 8);
      }
      while (bwd.size() % kGroup) {
        BwdOp nop{};
        nop.x = -1;
        nop.adj_x = nop.seed = nop.adj_a = nop.adj_b = -1;
        bwd.push_back(nop);
      }
    }
  }
}

// ------------------------------------------------------------ device setup
void netlk_ctx::allocate_and_upload(const netlk_partition *in) {
  const int V = (int)dag.vars.size();
  ppw = 32 / R;
  // patterns: every partition padded to whole 32-pattern blocks
  N = 0;
  n_units = 0;
  for (auto &pi : parts) {
    pi.n_pad = (pi.n + 31) / 32 * 32;
    pi.offset = N;
    pi.unit_begin = (int)(N / ppw);
    N += pi.n_pad;
    pi.unit_end = (int)(N / ppw);
  }
  n_units = (int)(N / ppw);
  build_schedules();
  if (opts.host_only) return;
  // host staging of tips / weights / unit map
  std::vector<uint8_t> tips((size_t)topo.n_tips * N, 0x0f);
  std::vector<double> weights(N, 0.0);
  std::vector<int32_t> unit_part(n_units);
  for (int p = 0; p < P; ++p) {
    const PartInfo &pi = parts[p];
    for (int t = 0; t < topo.n_tips; ++t)
      for (int s = 0; s < pi.n; ++s) {
        uint32_t code = in[p].tip_states[(size_t)t * pi.n + s] & 0xfu;
        if (!code) throw Error(NETLK_ERR_INVALID_ARGUMENT, "tip state mask 0");
        tips[(size_t)t * N + pi.offset + s] = (uint8_t)code;
      }
    for (int s = 0; s < pi.n; ++s) {
      double w = in[p].pattern_weights ? in[p].pattern_weights[s] : 1.0;
      if (!(w >= 0.0) || !std::isfinite(w)) throw Error(NETLK_ERR_INVALID_ARGUMENT, "pattern weight");
      weights[pi.offset + s] = w;
    }
    for (int u = pi.unit_begin; u < pi.unit_end; ++u) unit_part[u] = p;
  }
  const size_t real_sz = opts.precision == NETLK_FP32 ? 4 : 8;
  const size_t clv_per_var = (size_t)N * R * S * real_sz;
  d_clv.alloc(clv_per_var * V, dev_bytes);
  d_scaler.alloc((size_t)N * V * 4, dev_bytes);
  d_adj.alloc(clv_per_var * std::max(1, n_adj), dev_bytes);
  d_tips.alloc(tips.size(), dev_bytes);
  d_weights.alloc(N * 8, dev_bytes);
  d_unit_part.alloc(n_units * 4, dev_bytes);
  d_fwd.alloc(fwd.size() * sizeof(FwdOp), dev_bytes);
  d_bwd.alloc(bwd.size() * sizeof(BwdOp), dev_bytes);
  const size_t nm = (size_t)P * topo.n_edges * R * S * S;
  d_pmat64.alloc(nm * 8, dev_bytes);
  if (opts.precision == NETLK_FP32) d_pmat32.alloc(nm * 4, dev_bytes);
  d_lambda.alloc(P * S * 8, dev_bytes);
  d_U.alloc(P * S * S * 8, dev_bytes);
  d_Uinv.alloc(P * S * S * 8, dev_bytes);
  d_rates.alloc(P * R * 8, dev_bytes);
  d_rw.alloc(P * R * 8, dev_bytes);
  d_freqs.alloc(P * S * 8, dev_bytes);
  d_Q.alloc(P * S * S * 8, dev_bytes);
  d_brlen.alloc(topo.n_edges * 8, dev_bytes);
  d_site_partial.alloc((size_t)n_slots * n_units * 8, dev_bytes);
  d_tree_logl.alloc((size_t)n_slots * P * 8, dev_bytes);
  d_root_slot.alloc(root_slot.size() * 4, dev_bytes);
  d_root_lp.alloc(dag.roots.size() * 8, dev_bytes);
  d_root_dlp.alloc(dag.roots.size() * std::max(1, topo.n_ret) * 8, dev_bytes);
  d_seeds.alloc((size_t)n_slots * P * 8, dev_bytes);
  d_wts.alloc(dag.roots.size() * 8, dev_bytes);
  d_slot_begin.alloc(slot_begin.size() * 4, dev_bytes);
  d_slot_roots.alloc(slot_roots.size() * 4, dev_bytes);
  d_parts.alloc(P * sizeof(DevPartition), dev_bytes);
  d_out.alloc((2 + P + topo.n_ret) * 8, dev_bytes);
  d_grad.alloc(topo.n_edges * 8, dev_bytes);

  int sms = 0;
  CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  auto grid_for = [&](bool backward) {
    const int per_sm = max_resident_blocks(opts.precision, R, backward, topo.n_edges);
    const int64_t resident_warps = (int64_t)per_sm * sms * (kThreads / 32);
    const int64_t rounds = (n_units + resident_warps - 1) / resident_warps;
    const int64_t warps = (n_units + rounds - 1) / rounds;
    return (int)std::max<int64_t>(1, (warps + kThreads / 32 - 1) / (kThreads / 32));
  };
  grid_fwd = grid_for(false);
  grid_bwd = grid_for(true);
  d_grad_partial.alloc((size_t)grid_bwd * topo.n_edges * 8, dev_bytes);

  std::vector<DevPartition> dparts(P);
  for (int p = 0; p < P; ++p) dparts[p] = DevPartition{parts[p].unit_begin, parts[p].unit_end};
  CUDA_OK(cudaMemcpyAsync(d_tips.p, tips.data(), tips.size(), cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_weights.p, weights.data(), N * 8, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_unit_part.p, unit_part.data(), n_units * 4, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_fwd.p, fwd.data(), fwd.size() * sizeof(FwdOp), cudaMemcpyHostToDevice, stream));
  if (!bwd.empty())
    CUDA_OK(cudaMemcpyAsync(d_bwd.p, bwd.data(), bwd.size() * sizeof(BwdOp), cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_root_slot.p, root_slot.data(), root_slot.size() * 4, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_slot_begin.p, slot_begin.data(), slot_begin.size() * 4, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_slot_roots.p, slot_roots.data(), slot_roots.size() * 4, cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaMemcpyAsync(d_parts.p, dparts.data(), P * sizeof(DevPartition), cudaMemcpyHostToDevice, stream));
  CUDA_OK(cudaStreamSynchronize(stream));  // host staging vectors go out of scope

  h_brlen.alloc(topo.n_edges * 8);
  h_root_lp.alloc(dag.roots.size() * 8);
  h_root_dlp.alloc(dag.roots.size() * std::max(1, topo.n_ret) * 8);
  h_out.alloc((2 + P + topo.n_ret) * 8);
  h_grad.alloc(topo.n_edges * 8);
  h_tree.alloc((size_t)n_slots * P * 8);
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
    std::copy(pi.rates.begin(), pi.rates.end(), rates.begin() + p * R);
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
  CUDA_OK(cudaStreamSynchronize(stream));
  model_dirty = false;
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

void netlk_ctx::enqueue(bool pm, bool fwd_on, bool reduce, bool mixk, bool bwd_on) {
  if (pm)
    launch_pmatrix(stream, P, topo.n_edges, R, d_lambda.as<double>(), d_U.as<double>(), d_Uinv.as<double>(),
                   d_rates.as<double>(), d_brlen.as<double>(), d_pmat64.as<double>(),
                   opts.precision == NETLK_FP32 ? d_pmat32.as<float>() : nullptr);
  const SweepParams sp = sweep();
  const MixParams mp = mix();
  if (fwd_on) launch_forward(stream, opts.precision, R, grid_fwd, sp);
  if (reduce) launch_tree_reduce(stream, mp);
  if (mixk) launch_mix(stream, mp);
  if (bwd_on && !bwd.empty()) {
    launch_backward(stream, opts.precision, R, grid_bwd, sp);
    launch_grad_reduce(stream, grid_bwd, topo.n_edges, d_grad_partial.as<double>(), d_grad.as<double>());
  }
}

void netlk_ctx::run(cudaGraphExec_t *cache, bool pm, bool fwd_on, bool reduce, bool mixk, bool bwd_on) {
  const int n = (int)pm + (int)fwd_on + (int)reduce + (int)mixk + (bwd_on && !bwd.empty() ? 2 : 0);
  if (!opts.use_cuda_graph) {
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

void netlk_ctx::prepare() {
  if (opts.host_only) throw Error(NETLK_ERR_NO_DEVICE, "context was created host_only");
  CUDA_OK(cudaSetDevice(device));
  if (model_dirty) upload_model();
  if (probs_dirty) upload_probs();
  std::memcpy(h_brlen.p, brlen.data(), brlen.size() * 8);
  CUDA_OK(cudaMemcpyAsync(d_brlen.p, h_brlen.p, brlen.size() * 8, cudaMemcpyHostToDevice, stream));
}

void netlk_ctx::finish(double *total, double *part_logl, double *d_brlen, double *d_ret) {
  const int nout = 2 + P + topo.n_ret;
  CUDA_OK(cudaMemcpyAsync(h_out.p, d_out.p, nout * 8, cudaMemcpyDeviceToHost, stream));
  if (d_brlen)
    CUDA_OK(cudaMemcpyAsync(h_grad.p, d_grad.p, topo.n_edges * 8, cudaMemcpyDeviceToHost, stream));
  CUDA_OK(cudaStreamSynchronize(stream));
  CUDA_OK(cudaGetLastError());
  const double *o = h_out.as<double>();
  if (o[1] != 0.0 || !std::isfinite(o[0]))
    throw Error(NETLK_ERR_NUMERIC, "Invalid network likelihood: negative infinity or NaN");
  if (total) *total = o[0];
  if (part_logl) std::memcpy(part_logl, o + 2, P * 8);
  if (d_ret && topo.n_ret) std::memcpy(d_ret, o + 2 + P, topo.n_ret * 8);
  if (d_brlen) std::memcpy(d_brlen, h_grad.p, topo.n_edges * 8);
}

// ------------------------------------------------------------------ C ABI
namespace {

template <class F>
int guarded(netlk_ctx *ctx, F &&f) {
  try {
    f();
    if (ctx) ctx->err.clear();
    return NETLK_OK;
  } catch (const Error &e) {
    if (ctx) ctx->err = e.what(); else g_create_error = e.what();
    return e.status;
  } catch (const std::bad_alloc &) {
    if (ctx) ctx->err = "host allocation failed"; else g_create_error = "host allocation failed";
    return NETLK_ERR_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    if (ctx) ctx->err = e.what(); else g_create_error = e.what();
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
    if (c->S != 4) throw Error(NETLK_ERR_UNSUPPORTED, "this build evaluates 4-state (DNA) partitions");
    if (c->R != 1 && c->R != 2 && c->R != 4 && c->R != 8)
      throw Error(NETLK_ERR_UNSUPPORTED, "rate_cats must be 1, 2, 4 or 8");
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
  });
}

int netlk_loglikelihood(netlk_ctx *ctx, double *total, double *part_logl, double *tree_partition_logl) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    ctx->prepare();
    ctx->run(&ctx->graph_logl, true, true, true, true, false);
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
    if (d_brlen) {
      // the gradient is taken w.r.t. the clamped length; zero where the clamp binds
      for (int e = 0; e < ctx->topo.n_edges; ++e) d_brlen[e] = g[e];
    }
  });
}

int netlk_edge_derivatives(netlk_ctx *ctx, int32_t edge, int32_t mode, double *d1, double *d2) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (edge < 0 || edge >= ctx->topo.n_edges) throw Error(NETLK_ERR_INVALID_ARGUMENT, "edge");
    if (mode != 0) throw Error(NETLK_ERR_UNSUPPORTED, "only mode 0 (true derivative) is built");
    std::vector<double> g(ctx->topo.n_edges);
    double tot;
    ctx->prepare();
    ctx->run(&ctx->graph_grad, true, true, true, true, true);
    ctx->finish(&tot, nullptr, g.data(), nullptr);
    if (d1) *d1 = g[edge];
    if (d2) {
      const double h = 1e-6, b0 = ctx->brlen[edge];
      double gp, gm;
      ctx->brlen[edge] = b0 + h;
      ctx->prepare();
      ctx->run(&ctx->graph_grad, true, true, true, true, true);
      ctx->finish(&tot, nullptr, g.data(), nullptr);
      gp = g[edge];
      ctx->brlen[edge] = std::max(b0 - h, 1e-6);
      const double hm = b0 - ctx->brlen[edge];
      ctx->prepare();
      ctx->run(&ctx->graph_grad, true, true, true, true, true);
      ctx->finish(&tot, nullptr, g.data(), nullptr);
      gm = g[edge];
      ctx->brlen[edge] = b0;
      *d2 = (gp - gm) / (h + hm);
    }
  });
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

int netlk_get_clv(netlk_ctx *ctx, int32_t variant, int32_t part, double *clv, int32_t *scaler) {
  if (!ctx) return NETLK_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    if (variant < 0 || variant >= (int)ctx->dag.vars.size() || part < 0 || part >= ctx->P)
      throw Error(NETLK_ERR_INVALID_ARGUMENT, "variant / partition");
    if (ctx->opts.host_only) throw Error(NETLK_ERR_NO_DEVICE, "context was created host_only");
    CUDA_OK(cudaSetDevice(ctx->device));
    const PartInfo &pi = ctx->parts[part];
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
