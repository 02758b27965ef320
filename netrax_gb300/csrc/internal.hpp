// Host-side internals of netlk: topology, displayed-tree DAG, model math.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace netlk {

// Error carrying a netlk status code; converted to the status at the C ABI.
struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

// Set of full reticulation configurations (tree indices 0..2^r-1) as a bitset.
// The reference keeps these sets as OR-lists of {-,0,1} vectors
// (src/graph/ReticulationConfigSet.hpp:17-82); combine == intersection,
// compatible == non-empty intersection, addOr == union, so a bitset over the
// 2^r configurations is an exact, representation-free encoding.
struct Bits {
  std::vector<uint64_t> w;
  Bits() = default;
  explicit Bits(size_t words, bool all = false) : w(words, all ? ~0ull : 0ull) {}
  bool any() const {
    for (uint64_t x : w)
      if (x) return true;
    return false;
  }
  bool intersects(const Bits &o) const {
    for (size_t i = 0; i < w.size(); ++i)
      if (w[i] & o.w[i]) return true;
    return false;
  }
  Bits operator&(const Bits &o) const {
    Bits r(*this);
    for (size_t i = 0; i < w.size(); ++i) r.w[i] &= o.w[i];
    return r;
  }
  Bits operator|(const Bits &o) const {
    Bits r(*this);
    for (size_t i = 0; i < w.size(); ++i) r.w[i] |= o.w[i];
    return r;
  }
  Bits andnot(const Bits &o) const {
    Bits r(*this);
    for (size_t i = 0; i < w.size(); ++i) r.w[i] &= ~o.w[i];
    return r;
  }
  bool operator==(const Bits &o) const { return w == o.w; }
  bool test(size_t t) const { return (w[t >> 6] >> (t & 63)) & 1ull; }
  void set(size_t t) { w[t >> 6] |= 1ull << (t & 63); }
  int64_t first() const {
    for (size_t i = 0; i < w.size(); ++i)
      if (w[i]) return (int64_t)(i * 64 + __builtin_ctzll(w[i]));
    return -1;
  }
  // f(t) for every member t, in increasing order
  template <class F>
  void for_each(F &&f) const {
    for (size_t i = 0; i < w.size(); ++i)
      for (uint64_t x = w[i]; x; x &= x - 1) f(i * 64 + (size_t)__builtin_ctzll(x));
  }
  uint64_t hash() const {
    uint64_t h = 1469598103934665603ull;
    for (uint64_t x : w) h = (h ^ x) * 1099511628211ull;
    return h;
  }
};

constexpr int32_t kFake = INT32_MIN;  // fake all-ones child (Operation.cpp:19-33)
inline int32_t tip_ref(int tip) { return -1 - tip; }
inline bool is_tip_ref(int32_t r) { return r < 0 && r != kFake; }
inline int tip_of_ref(int32_t r) { return -1 - r; }

struct Topology {
  int n_nodes = 0, n_tips = 0, n_edges = 0, n_ret = 0, root = -1;
  std::vector<int> edge_parent, edge_child;
  std::vector<int> child_edge;  // [2*n_nodes], -1 absent
  std::vector<int> ret_node, ret_first_edge, ret_second_edge;
  // derived
  std::vector<int> node_ret;          // reticulation index of a node or -1
  std::vector<int> ret_first_parent, ret_second_parent;
  std::vector<int> tree_parent;       // parent of a non-reticulation node or -1
  std::vector<int> post_order;        // children before parents

  int n_children(int v) const {
    return (child_edge[2 * v] >= 0) + (child_edge[2 * v + 1] >= 0);
  }
  int child(int v, int i) const { return edge_child[child_edge[2 * v + i]]; }
  int cedge(int v, int i) const { return child_edge[2 * v + i]; }
  void validate_and_derive();
};

struct Variant {
  int node = -1;
  int32_t ref[2] = {kFake, kFake};  // child variant id, tip ref, or kFake
  int edge[2] = {-1, -1};
  int level = 0;
  Bits set;
};

struct RootVariant {
  int variant = -1;       // variant id at the network root
  int dtroot_variant = -1;// variant whose CLV gives the tree log-likelihood
  int dtroot_node = -1;
  double logprob = 0.0;   // log P(covered configurations)
  std::vector<double> dlogprob;  // d logprob / d p_k (first-parent probs)
};

struct Dag {
  int r = 0;
  size_t words = 1;
  std::vector<Variant> vars;
  std::vector<std::vector<int32_t>> node_vars;  // per node: variant refs
  std::vector<RootVariant> roots;
  int n_levels = 0;
  int n_degenerate = 0;
  int max_per_node = 0;
};

// Builds the displayed-tree DAG and the displayed-tree roots.
Dag compile_dag(const Topology &topo);
// Fills logprob / dlogprob of the root variants for first-parent probs p.
void root_probabilities(const Topology &topo, Dag &dag, const std::vector<double> &p);

// ---------------------------------------------------------------- model math
struct Eigen {
  int S = 0;
  std::vector<double> lambda;  // [S]
  std::vector<double> U;       // [S*S] row-major, columns = right eigenvectors
  std::vector<double> Uinv;    // [S*S]
  std::vector<double> Q;       // [S*S] normalised rate matrix
};
Eigen gtr_eigen(int S, const double *freqs, const double *exch);
std::vector<double> gamma_mean_rates(double alpha, int ncat);

}  // namespace netlk
