// Displayed-tree DAG compiler.
//
// Restates the schedule of the reference's improved log-likelihood on bitsets
// over the 2^r full reticulation configurations:
//  - processNodeImprovedSingleChild  src/likelihood/ImprovedLoglikelihood.cpp:194-223
//  - processNodeImprovedTwoChildren  src/likelihood/ImprovedLoglikelihood.cpp:225-345
//  - getRestrictionsToTake/DismissNeighbor, getReticulationChoicesThisOnly,
//    deadNodeSettings               src/helper/ReticulationConfigHelper.cpp:26-186
//  - tree_already_present_and_fine  src/likelihood/ImprovedLoglikelihood.cpp:30-57
//    (an equal set at the same node is computed once)
//  - displayed-tree root search     src/helper/NetworkFunctions.cpp:228-279 and
//    findMatchingDisplayedTree      src/helper/ReticulationConfigHelper.cpp:205-249
// A reference config set is an OR of {-,0,1} vectors; its meaning is the set
// of full configurations it covers, and every operation the schedule uses
// (combine = intersection, compatible = non-empty intersection, union) is a
// set operation, so the variants produced here cover the same configuration
// sets as the reference's, node by node and in the same order.
#include <algorithm>
#include <cmath>
#include <deque>
#include <unordered_map>

#include "../../include/netlk.h"
#include "internal.hpp"

namespace netlk {

void Topology::validate_and_derive() {
  auto bad = [](const std::string &m) { throw Error(NETLK_ERR_TOPOLOGY, m); };
  if (n_nodes < 3 || n_tips < 2 || n_tips >= n_nodes) bad("need >= 2 tips and inner nodes");
  if (root < n_tips || root >= n_nodes) bad("root must be an inner node");
  if (n_ret < 0 || n_ret > NETLK_MAX_RETICULATIONS)
    throw Error(NETLK_ERR_UNSUPPORTED, "at most 16 reticulations are supported");
  if ((int)edge_parent.size() != n_edges || (int)edge_child.size() != n_edges) bad("edge arrays");
  node_ret.assign(n_nodes, -1);
  ret_first_parent.assign(n_ret, -1);
  ret_second_parent.assign(n_ret, -1);
  tree_parent.assign(n_nodes, -1);
  for (int k = 0; k < n_ret; ++k) {
    int v = ret_node[k];
    if (v < n_tips || v >= n_nodes || node_ret[v] >= 0) bad("bad reticulation node");
    node_ret[v] = k;
    int e1 = ret_first_edge[k], e2 = ret_second_edge[k];
    if (e1 < 0 || e1 >= n_edges || e2 < 0 || e2 >= n_edges || e1 == e2) bad("bad reticulation edges");
    if (edge_child[e1] != v || edge_child[e2] != v) bad("reticulation edges must end at the reticulation");
    ret_first_parent[k] = edge_parent[e1];
    ret_second_parent[k] = edge_parent[e2];
    if (ret_first_parent[k] == ret_second_parent[k])
      bad("both parents of a reticulation are the same node");
  }
  std::vector<int> indeg(n_nodes, 0);
  for (int e = 0; e < n_edges; ++e) {
    int p = edge_parent[e], c = edge_child[e];
    if (p < 0 || p >= n_nodes || c < 0 || c >= n_nodes || p == c) bad("edge endpoint out of range");
    if (p < n_tips) bad("a tip has a child");
    indeg[c]++;
    if (node_ret[c] < 0) tree_parent[c] = p;
  }
  for (int v = 0; v < n_nodes; ++v) {
    int want = v == root ? 0 : (node_ret[v] >= 0 ? 2 : 1);
    if (indeg[v] != want) bad("node " + std::to_string(v) + " has a wrong number of parents");
  }
  if ((int)child_edge.size() != 2 * n_nodes) bad("node_child_edges size");
  std::vector<int> seen(n_edges, 0);
  for (int v = 0; v < n_nodes; ++v) {
    for (int i = 0; i < 2; ++i) {
      int e = child_edge[2 * v + i];
      if (e < 0) continue;
      if (e >= n_edges || edge_parent[e] != v) bad("node_child_edges inconsistent");
      if (seen[e]++) bad("edge listed twice");
    }
    if (child_edge[2 * v] < 0 && child_edge[2 * v + 1] >= 0) bad("node_child_edges: -1 before an edge");
    int nc = n_children(v);
    if (v < n_tips && nc != 0) bad("tip with children");
    if (v >= n_tips) {
      if (node_ret[v] >= 0 && nc != 1) bad("reticulation nodes need exactly one child");
      if (node_ret[v] < 0 && nc != 2) bad("inner tree nodes need exactly two children");
    }
  }
  for (int e = 0; e < n_edges; ++e)
    if (!seen[e]) bad("edge missing from node_child_edges");
  // post order (Kahn from the tips; reversed_topological_sort, NetworkFunctions.cpp:542-598)
  std::vector<int> outdeg(n_nodes);
  std::deque<int> q;
  for (int v = 0; v < n_nodes; ++v) {
    outdeg[v] = n_children(v);
    if (!outdeg[v]) q.push_back(v);
  }
  post_order.clear();
  while (!q.empty()) {
    int v = q.front();
    q.pop_front();
    post_order.push_back(v);
    for (int e = 0; e < n_edges; ++e) {
      if (edge_child[e] != v) continue;
      int p = edge_parent[e];
      if (--outdeg[p] == 0) q.push_back(p);
    }
  }
  if ((int)post_order.size() != n_nodes) bad("cycle in network detected");
}

namespace {

struct Compiler {
  const Topology &T;
  Dag &D;
  size_t n_trees;
  Bits ALL, EMPTY;
  std::vector<Bits> first_mask, second_mask;

  // Per node, owner[c] = index (in node_vars) of the variant whose set holds
  // configuration c, or -1. The variant sets of a node are pairwise disjoint
  // (every configuration displays at most one tree below a node), which turns
  // the pairwise set intersections of the two-child step and of the root
  // matching into one pass over the configurations; a node whose sets do
  // overlap (owner_state 2) keeps the pairwise path. 0: not built yet.
  std::vector<std::vector<int32_t>> owner;
  std::vector<signed char> owner_state;
  // the node being processed: hash of each variant set -> variant, for the
  // equal-set check of add()
  std::unordered_multimap<uint64_t, int32_t> node_sets;

  Compiler(const Topology &t, Dag &d) : T(t), D(d) {
    D.r = T.n_ret;
    n_trees = (size_t)1 << D.r;
    D.words = std::max<size_t>(1, (n_trees + 63) / 64);
    ALL = Bits(D.words, false);
    for (size_t t2 = 0; t2 < n_trees; ++t2) ALL.set(t2);
    EMPTY = Bits(D.words, false);
    first_mask.assign(D.r, EMPTY);
    second_mask.assign(D.r, EMPTY);
    for (size_t t2 = 0; t2 < n_trees; ++t2)
      for (int k = 0; k < D.r; ++k) ((t2 >> k) & 1 ? second_mask : first_mask)[k].set(t2);
  }

  // getRestrictionsToTakeNeighbor(parent, child) for a child edge.
  Bits take(int parent, int child) const {
    int k = T.node_ret[child];
    if (k >= 0) {
      if (parent == T.ret_first_parent[k]) return first_mask[k];
      if (parent == T.ret_second_parent[k]) return second_mask[k];
    }
    return ALL;
  }
  // getRestrictionsToDismissNeighbor(parent, child); empty when nothing restricts.
  Bits dismiss(int parent, int child) const {
    int k = T.node_ret[child];
    if (k >= 0) {
      if (parent == T.ret_first_parent[k]) return second_mask[k];
      if (parent == T.ret_second_parent[k]) return first_mask[k];
    }
    return EMPTY;
  }
  const Bits &set_of(int32_t ref) const { return is_tip_ref(ref) ? ALL : D.vars[ref].set; }
  int level_of(int32_t ref) const { return (ref >= 0) ? D.vars[ref].level : 0; }

  const std::vector<int32_t> *owners(int node) {
    if (owner_state[node] == 0) {
      std::vector<int32_t> &o = owner[node];
      o.assign(n_trees, -1);
      owner_state[node] = 1;
      const std::vector<int32_t> &vars = D.node_vars[node];
      for (int32_t i = 0; i < (int32_t)vars.size(); ++i)
        set_of(vars[i]).for_each([&](size_t c) {
          if (o[c] >= 0) owner_state[node] = 2;
          o[c] = i;
        });
    }
    return owner_state[node] == 1 ? &owner[node] : nullptr;
  }

  void add(int node, const Bits &set, int32_t r0, int e0, int32_t r1, int e1) {
    if (!set.any()) {
      D.n_degenerate++;
      return;
    }
    // tree_already_present_and_fine: an equal set at this node is kept once
    const uint64_t h = set.hash();
    for (auto it = node_sets.equal_range(h); it.first != it.second; ++it.first)
      if (D.vars[it.first->second].set == set) return;
    node_sets.emplace(h, (int32_t)D.vars.size());
    Variant var;
    var.node = node;
    var.ref[0] = r0;
    var.ref[1] = r1;
    var.edge[0] = e0;
    var.edge[1] = e1;
    var.level = 1 + std::max(level_of(r0), r1 == kFake ? 0 : level_of(r1));
    var.set = set;
    D.node_vars[node].push_back((int32_t)D.vars.size());
    D.vars.push_back(std::move(var));
  }

  void single(int v) {
    int c = T.child(v, 0), e = T.cedge(v, 0);
    Bits restr = take(v, c);
    for (int32_t ref : D.node_vars[c]) {
      const Bits &s = set_of(ref);
      if (s.intersects(restr)) add(v, s & restr, ref, e, kFake, -1);
    }
  }

  // deadNodeSettings: dismissed, or taken with no displayed tree of the child.
  Bits dead_settings(int parent, int child) const {
    Bits covered = EMPTY;
    for (int32_t ref : D.node_vars[child]) covered = covered | set_of(ref);
    return dismiss(parent, child) | take(parent, child).andnot(covered);
  }

  // getReticulationChoicesThisOnly
  Bits this_only(const Bits &cfg, const Bits &other_dead, int parent, int this_c, int other_c) const {
    Bits restricted = cfg & take(parent, this_c);
    if (!restricted.any()) return EMPTY;
    Bits part1 = restricted & dismiss(parent, other_c);
    Bits part2 = restricted & take(parent, other_c) & other_dead;
    return part1 | part2;
  }

  void two(int v) {
    int lc = T.child(v, 0), le = T.cedge(v, 0);
    int rc = T.child(v, 1), re = T.cedge(v, 1);
    Bits both = take(v, lc) & take(v, rc);
    const std::vector<int32_t> lv = D.node_vars[lc], rv = D.node_vars[rc];
    const std::vector<int32_t> *ol = owners(lc), *orr = owners(rc);
    if (ol && orr) {
      // the pairs (l, r) whose sets share a configuration, with l and r both
      // meeting `both`, in the order of the nested loop below; each gets the
      // configurations of `both` it holds (none: a degenerate pair, counted
      // by add() like the nested loop's)
      std::vector<char> lb(lv.size(), 0), rb(rv.size(), 0);
      both.for_each([&](size_t c) {
        if ((*ol)[c] >= 0) lb[(*ol)[c]] = 1;
        if ((*orr)[c] >= 0) rb[(*orr)[c]] = 1;
      });
      std::unordered_map<int64_t, size_t> at;
      std::vector<std::pair<int64_t, std::vector<uint32_t>>> pairs;
      for (size_t c = 0; c < n_trees; ++c) {
        const int32_t li = (*ol)[c], ri = (*orr)[c];
        if (li < 0 || ri < 0 || !lb[li] || !rb[ri]) continue;
        const int64_t key = (int64_t)li * (int64_t)rv.size() + ri;
        auto ins = at.emplace(key, pairs.size());
        if (ins.second) pairs.emplace_back(key, std::vector<uint32_t>());
        if (both.test(c)) pairs[ins.first->second].second.push_back((uint32_t)c);
      }
      std::sort(pairs.begin(), pairs.end(),
                [](const auto &a, const auto &b) { return a.first < b.first; });
      for (const auto &pr : pairs) {
        Bits s = EMPTY;
        for (uint32_t c : pr.second) s.set(c);
        const int64_t li = pr.first / (int64_t)rv.size(), ri = pr.first % (int64_t)rv.size();
        add(v, s, lv[li], le, rv[ri], re);
      }
    } else {
      for (int32_t l : lv) {
        // a copy: add() below may grow D.vars and move the set a reference points to
        const Bits ls = set_of(l);
        if (!ls.intersects(both)) continue;
        for (int32_t r : rv) {
          const Bits &rs = set_of(r);
          if (!rs.intersects(both)) continue;
          if (ls.intersects(rs)) add(v, ls & rs & both, l, le, r, re);
        }
      }
    }
    Bits rdead = dead_settings(v, rc);
    for (int32_t l : lv) {
      Bits only = this_only(set_of(l), rdead, v, lc, rc);
      if (only.any()) add(v, only, l, le, kFake, -1);
    }
    Bits ldead = dead_settings(v, lc);
    for (int32_t r : rv) {
      Bits only = this_only(set_of(r), ldead, v, rc, lc);
      if (only.any()) add(v, only, r, re, kFake, -1);
    }
  }

  // collect_dead_nodes for one full configuration; returns the displayed-tree root.
  int displayed_tree_root(size_t t) const {
    std::vector<char> dead(T.n_nodes, 0);
    auto active_alive = [&](int u, int *only) {
      int cnt = 0;
      for (int i = 0; i < 2; ++i) {
        int e = T.child_edge[2 * u + i];
        if (e < 0) continue;
        int c = T.edge_child[e];
        if (dead[c]) continue;
        int k = T.node_ret[c];
        if (k >= 0) {
          int active_edge = ((t >> k) & 1) ? T.ret_second_edge[k] : T.ret_first_edge[k];
          if (active_edge != e) continue;
        }
        if (only) *only = c;
        cnt++;
      }
      return cnt;
    };
    for (int u : T.post_order) {
      if (u < T.n_tips) continue;
      dead[u] = active_alive(u, nullptr) == 0;
    }
    int u = T.root, nxt = -1;
    while (active_alive(u, &nxt) == 1) u = nxt;
    return u;
  }

  void run() {
    D.vars.clear();
    D.node_vars.assign(T.n_nodes, {});
    owner.assign(T.n_nodes, {});
    owner_state.assign(T.n_nodes, 0);
    for (int t = 0; t < T.n_tips; ++t) D.node_vars[t].push_back(tip_ref(t));
    for (int v : T.post_order) {
      if (v < T.n_tips) continue;
      node_sets.clear();
      if (T.n_children(v) == 1)
        single(v);
      else
        two(v);
      if (D.node_vars[v].empty())
        throw Error(NETLK_ERR_ENUMERATION, "node " + std::to_string(v) + " has no displayed tree");
      D.max_per_node = std::max<int>(D.max_per_node, (int)D.node_vars[v].size());
    }
    D.n_levels = 0;
    for (auto &var : D.vars) D.n_levels = std::max(D.n_levels, var.level);
    D.roots.clear();
    for (int32_t v : D.node_vars[T.root]) {
      RootVariant rv;
      rv.variant = v;
      size_t t0 = (size_t)D.vars[v].set.first();
      int dt = displayed_tree_root(t0);
      int found = -1, n_found = 0;
      if (const std::vector<int32_t> *od = owners(dt)) {
        // the variants of dt meeting the root variant's set
        std::vector<int32_t> hit;
        D.vars[v].set.for_each([&](size_t c) {
          const int32_t i = (*od)[c];
          if (i >= 0 && std::find(hit.begin(), hit.end(), i) == hit.end()) hit.push_back(i);
        });
        n_found = (int)hit.size();
        if (n_found) found = D.node_vars[dt][*std::max_element(hit.begin(), hit.end())];
      } else {
        for (int32_t cand : D.node_vars[dt]) {
          if (set_of(cand).intersects(D.vars[v].set)) {
            found = cand;
            n_found++;
          }
        }
      }
      if (n_found != 1 || found < 0)
        throw Error(NETLK_ERR_ENUMERATION,
                    n_found > 1 ? "Found multiple suitable trees" : "Found no suitable displayed tree");
      rv.dtroot_variant = found;
      rv.dtroot_node = dt;
      D.roots.push_back(rv);
    }
  }
};

}  // namespace

Dag compile_dag(const Topology &topo) {
  Dag dag;
  Compiler c(topo, dag);
  c.run();
  return dag;
}

void root_probabilities(const Topology &topo, Dag &dag, const std::vector<double> &p) {
  const int r = dag.r;
  const size_t n = (size_t)1 << r;
  std::vector<double> lp(n, 0.0);
  for (size_t t = 0; t < n; ++t) {
    double s = 0.0;
    for (int k = 0; k < r; ++k) s += ((t >> k) & 1) ? std::log1p(-p[k]) : std::log(p[k]);
    lp[t] = s;
  }
  (void)topo;
  for (auto &rv : dag.roots) {
    const Bits &set = dag.vars[rv.variant].set;
    double m = -INFINITY;
    set.for_each([&](size_t t) { m = std::max(m, lp[t]); });
    double acc = 0.0;
    std::vector<double> dacc(r, 0.0);
    set.for_each([&](size_t t) {
      double w = std::exp(lp[t] - m);
      acc += w;
      for (int k = 0; k < r; ++k) dacc[k] += w * (((t >> k) & 1) ? -1.0 / (1.0 - p[k]) : 1.0 / p[k]);
    });
    rv.logprob = m + std::log(acc);
    rv.dlogprob.assign(r, 0.0);
    for (int k = 0; k < r; ++k) rv.dlogprob[k] = dacc[k] / acc;
  }
}

}  // namespace netlk
