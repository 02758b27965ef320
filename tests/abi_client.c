/* A plain C99 caller of the netlk C ABI, without a GPU (host-only context).
 *
 * Built and run by tests/test_c_client.py: it shows that include/netlk.h is
 * usable from C as a reference-side binding would use it (no C++ types, no
 * Python). It reads a 3-taxon, 1-reticulation network in the reference's own
 * numbering, encodes and compresses a small alignment with the library's front
 * end, builds a host-only context and prints its DAG statistics as key=value
 * lines; it also checks the error surface (a NaN branch length, an evaluation
 * without a device). Exit status 0 when every call behaved as documented. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "netlk.h"

#define CHECK(cond, what)                                     \
  do {                                                        \
    if (!(cond)) {                                            \
      fprintf(stderr, "abi_client: %s failed\n", what);       \
      return 1;                                               \
    }                                                         \
  } while (0)

int main(void) {
  /* ((A:0.1,(B:0.2)#H1:0.05::0.6):0.1,(C:0.3,#H1:0.1::0.4):0.2); */
  const int32_t edge_parent[7] = {4, 6, 3, 5, 5, 4, 3};
  const int32_t edge_child[7] = {0, 1, 2, 3, 4, 6, 6};
  const int32_t child_edges[14] = {-1, -1, -1, -1, -1, -1, 6, 2, 5, 0, 3, 4, 1, -1};
  const int32_t ret_node[1] = {6}, ret_first[1] = {5}, ret_second[1] = {6};
  const double lengths[7] = {0.1, 0.2, 0.3, 0.2, 0.1, 0.05, 0.1};
  const double first_prob[1] = {0.6};
  netlk_topology topo = {7, 3, 7, 1, 5, edge_parent, edge_child, child_edges, ret_node, ret_first, ret_second};

  /* alignment: tips A, B, C (in tip-id order), 8 sites with repeats */
  const char *rows[3] = {"ACGTACGA", "ACGTTCGA", "AYGTACNA"};
  uint32_t masks[3 * 8], patterns[3 * 8];
  double weights[8];
  int64_t bad = -1, n_patterns = 0;
  for (int t = 0; t < 3; ++t)
    CHECK(netlk_encode_states(rows[t], 8, 4, masks + 8 * t, &bad) == NETLK_OK, "netlk_encode_states");
  CHECK(netlk_encode_states("AC!T", 4, 4, masks, &bad) == NETLK_ERR_INVALID_ARGUMENT && bad == 2,
        "netlk_encode_states rejects an unknown character");
  for (int t = 0; t < 3; ++t)  /* restore row 0 */
    CHECK(netlk_encode_states(rows[t], 8, 4, masks + 8 * t, &bad) == NETLK_OK, "netlk_encode_states");
  CHECK(netlk_compress_patterns(masks, 3, 8, patterns, weights, &n_patterns) == NETLK_OK,
        "netlk_compress_patterns");
  printf("n_site_patterns=%lld\n", (long long)n_patterns);

  const double freqs[4] = {0.2, 0.3, 0.3, 0.2};
  const double exch[6] = {1.0, 2.5, 0.8, 1.2, 3.0, 1.0};
  netlk_partition part;
  memset(&part, 0, sizeof part);
  part.states = 4;
  part.rate_cats = 4;
  part.n_patterns = (int32_t)n_patterns;
  part.tip_states = patterns;
  part.pattern_weights = weights;
  part.freqs = freqs;
  part.exchangeabilities = exch;
  part.alpha = 0.8;

  netlk_options opts;
  CHECK(netlk_options_default(&opts) == NETLK_OK, "netlk_options_default");
  opts.host_only = 1;
  netlk_ctx *ctx = NULL;
  CHECK(netlk_create(&topo, &part, 1, lengths, first_prob, &opts, &ctx) == NETLK_OK && ctx, "netlk_create");

  netlk_dag_stats st;
  CHECK(netlk_get_dag_stats(ctx, &st) == NETLK_OK, "netlk_get_dag_stats");
  printf("n_variants=%d\nn_root_variants=%d\nn_levels=%d\nn_backward_ops=%d\nsite_clv_updates=%lld\n",
         st.n_variants, st.n_root_variants, st.n_levels, st.n_backward_ops, (long long)st.site_clv_updates);

  /* the edge-sumtable schedule of edge 2 (host work only) and the table
     build, which a host-only context declines */
  int32_t n_ops = 0, n_work = 0, n_tables = 0, n_groups = 0, built = -1, n_built = -1;
  CHECK(netlk_sumtable_export(ctx, 2, &n_ops, &n_work, &n_tables, &n_groups, NULL, NULL, NULL) == NETLK_OK,
        "netlk_sumtable_export");
  CHECK(netlk_edge_sumtable(ctx, 2, &built, &n_built) == NETLK_OK && built == 0 && n_built == 0,
        "netlk_edge_sumtable declines on a host-only context");
  printf("sumtable_ops=%d\nsumtable_tables=%d\nsumtable_groups=%d\n", n_ops, n_tables, n_groups);

  double total = 0.0;
  const int s = netlk_loglikelihood(ctx, &total, NULL, NULL);
  CHECK(s == NETLK_ERR_NO_DEVICE, "a host-only context refuses evaluation");
  printf("evaluate_status=%s\n", netlk_status_string(s));
  CHECK(netlk_destroy(ctx) == NETLK_OK, "netlk_destroy");

  double bad_lengths[7];
  memcpy(bad_lengths, lengths, sizeof bad_lengths);
  bad_lengths[3] = NAN;
  ctx = NULL;
  CHECK(netlk_create(&topo, &part, 1, bad_lengths, first_prob, &opts, &ctx) == NETLK_ERR_INVALID_ARGUMENT && !ctx,
        "netlk_create rejects a NaN branch length");
  printf("nan_length_error=%s\n", netlk_last_error(NULL));
  return 0;
}
