/*
 * netlk - GB300 (sm_103a) phylogenetic-network likelihood, C ABI.
 *
 * Drop-in for the network log-likelihood hot path of NetRAX (the reference):
 * Felsenstein pruning over every displayed tree of a rooted phylogenetic
 * network, with subtrees shared across reticulation configurations, combined
 * per partition under the AVERAGE (mixture) or BEST (maximum) model, plus the
 * gradient with respect to every branch length and every reticulation
 * probability from one adjoint sweep.
 *
 * Conventions
 *  - Every entry point returns an int status (NETLK_OK == 0). No C++
 *    exception crosses this boundary. netlk_last_error(ctx) gives a message.
 *  - Plain pointers and sizes only. Host pointers unless a name says device.
 *  - A context owns one CUDA stream and its device buffers; it is not
 *    re-entrant (one host thread at a time per context).
 *  - Node numbering follows the reference's Network: tips 0..n_tips-1, then
 *    inner tree nodes, then reticulation nodes; edge ids are the reference's
 *    pmatrix indices (src/io/NetworkIO.cpp:114-185).
 */
#ifndef NETLK_H
#define NETLK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status codes */
#define NETLK_OK 0
#define NETLK_ERR_INVALID_ARGUMENT 1 /* bad sizes, indices, NaN parameters   */
#define NETLK_ERR_TOPOLOGY 2         /* not a rooted binary network, cycle   */
#define NETLK_ERR_ENUMERATION 3      /* displayed-tree matching failed        */
#define NETLK_ERR_CUDA 4             /* CUDA runtime error                    */
#define NETLK_ERR_OUT_OF_MEMORY 5    /* device or host allocation failed      */
#define NETLK_ERR_NUMERIC 6          /* -inf / NaN network log-likelihood     */
#define NETLK_ERR_UNSUPPORTED 7      /* e.g. too many reticulations           */
#define NETLK_ERR_NO_DEVICE 8        /* no CUDA device / wrong architecture   */
#define NETLK_ERR_TIMEOUT 9          /* a bounded device wait ran out         */

/* ------------------------------------------------------------ enumerations */
#define NETLK_AVERAGE 0 /* LikelihoodVariant::AVERAGE_DISPLAYED_TREES */
#define NETLK_BEST 1    /* LikelihoodVariant::BEST_DISPLAYED_TREE     */

#define NETLK_FP64 0 /* plain FP64 CLVs, libpll scaling (2^-256 / 2^256)     */
#define NETLK_FP32 1 /* FP32 CLVs, per-site power-of-two rescaling          */

#define NETLK_MAX_RETICULATIONS 16

/* ------------------------------------------------------------- descriptors */

/* Rooted phylogenetic network.
 * Replaces the reference's Network / AnnotatedNetwork topology
 * (src/graph/Network.hpp:20-76, src/graph/AnnotatedNetwork.hpp:42-89). */
typedef struct {
  int32_t n_nodes;
  int32_t n_tips;
  int32_t n_edges;
  int32_t n_reticulations;
  int32_t root;                    /* node id of the root                    */
  const int32_t *edge_parent;      /* [n_edges]                              */
  const int32_t *edge_child;       /* [n_edges]                              */
  const int32_t *node_child_edges; /* [2*n_nodes] outgoing edges of each node
                                      in the reference's child order
                                      (getChildren, src/helper/ChildrenHelper.cpp:6-21);
                                      -1 where absent                        */
  const int32_t *ret_node;         /* [n_reticulations] node of reticulation k */
  const int32_t *ret_first_edge;   /* [n_reticulations] edge from first parent */
  const int32_t *ret_second_edge;  /* [n_reticulations] edge from second parent */
} netlk_topology;

/* One alignment partition (pattern-compressed) with a GTR+Gamma model.
 * Replaces the pll_partition_t + model parameters held by the reference's
 * fake_treeinfo (src/RaxmlWrapper.cpp:671-766). */
typedef struct {
  int32_t states;                 /* 4 (DNA) or 20 (protein)                  */
  int32_t rate_cats;              /* 1..8                                     */
  int32_t n_patterns;
  const uint32_t *tip_states;     /* [n_tips*n_patterns] state bitmask per tip
                                     (row = tip); DNA A=1 C=2 G=4 T=8          */
  const double *pattern_weights;  /* [n_patterns]                             */
  const double *freqs;            /* [states]                                 */
  const double *exchangeabilities;/* [states*(states-1)/2], row-major upper
                                     triangle (AC AG AT CG CT GT for DNA)      */
  double alpha;                   /* Gamma shape; used when rates == NULL     */
  const double *rates;            /* optional [rate_cats] category rates      */
  const double *rate_weights;     /* optional [rate_cats]; default 1/rate_cats */
  double prop_invar;              /* proportion of invariant sites (+I), in
                                     [0, 0.99]; 0 = none. With p > 0 a site's
                                     likelihood is (1 - p) x the rate mixture
                                     (category rates divided by 1 - p) + p x
                                     the frequency of the one state every tip
                                     admits, if any (libpll's prop_invar)     */
} netlk_partition;

typedef struct {
  int32_t variant;                   /* NETLK_AVERAGE / NETLK_BEST           */
  int32_t precision;                 /* NETLK_FP64 / NETLK_FP32              */
  double min_interesting_tree_logprob; /* NetraxOptions, default log(1e-6)   */
  int32_t device;                    /* CUDA device ordinal                  */
  int32_t use_cuda_graph;            /* 1: replay captured launch sequences  */
  int32_t host_only;                 /* 1: build the DAG and schedules only,
                                        touch no device (evaluation calls then
                                        return NETLK_ERR_NO_DEVICE)          */
  int32_t autotune;                  /* 1: time the launch shapes of the two
                                        sweeps on the first evaluation and keep
                                        the fastest (default); 0: default shape.
                                        The environment variable NETLK_SHAPES=
                                        "f,b" fixes both shapes instead.      */
  int32_t tensor_cores;              /* 1 (default): 20-state FP32 contexts
                                        with 4 rate categories run the P x CLV
                                        products of the forward and adjoint
                                        sweeps on the tensor cores (3xTF32
                                        split, FP32 accumulation); 0: CUDA
                                        cores only. No effect on other
                                        contexts.                            */
  int32_t checkpoint_segments;       /* CLV checkpointing for DAGs whose CLVs
                                        do not fit in device memory:
                                        0 (default) = automatic - all CLVs are
                                        stored while they fit in 70 % of the
                                        free device memory, otherwise the
                                        levels are cut into ceil(sqrt(levels))
                                        segments (more if needed); 1 = store
                                        every CLV; k >= 2 = k segments. With
                                        k segments only the CLVs read across a
                                        segment boundary are kept, the adjoint
                                        recomputes the other CLVs of each
                                        segment before its levels (one extra
                                        forward over them).                   */
  int32_t incremental;               /* 1 (default): netlk_loglikelihood and
                                        netlk_edge_loglikelihood recompute
                                        only the CLVs that depend on branch
                                        lengths changed since the last full
                                        forward sweep (the reference's
                                        clv_valid flags, InvalidationHelper.cpp
                                        :52-237); 0: every call recomputes
                                        every CLV. Results are identical.     */
  int32_t brlen_linkage;             /* NETLK_BRLEN_LINKED (default): one
                                        length per edge for every partition;
                                        NETLK_BRLEN_UNLINKED: each partition
                                        has its own lengths
                                        (netlk_set_partition_branch_lengths);
                                        NETLK_BRLEN_SCALED: partition p uses
                                        scaler[p] x the linked length
                                        (netlk_set_branch_length_scalers). The
                                        reference's --brlen linked / unlinked /
                                        scaled (src/main.cpp:101,226-230).    */
  int32_t sumtables;                 /* 1 (default): edge derivatives from
                                        the edge's sumtables
                                        (netlk_edge_sumtable); 0: one tangent
                                        sweep per call                        */
} netlk_options;

#define NETLK_BRLEN_LINKED 0
#define NETLK_BRLEN_UNLINKED 1
#define NETLK_BRLEN_SCALED 2

typedef struct {
  int32_t n_variants;        /* inner displayed-tree variants (DAG nodes)    */
  int32_t n_root_variants;   /* displayed trees at the network root          */
  int32_t n_dtroot_slots;    /* distinct variants holding a tree's root CLV  */
  int32_t n_levels;          /* dependency levels of the variant DAG         */
  int32_t n_backward_ops;    /* variants visited by the adjoint sweep        */
  int32_t n_adjoint_slots;   /* adjoint buffers after liveness reuse         */
  int32_t max_variants_per_node;
  int32_t n_degenerate;      /* child pairs whose combined set is empty (the
                                reference stores a CLV for them; never used) */
  int64_t n_patterns_total;  /* padded patterns over all partitions          */
  int64_t site_clv_updates;  /* per forward pass: sum_variants patterns      */
  int64_t tip_child_uses;    /* child operands that are tips                 */
  int64_t fake_child_uses;   /* unary variants (fake all-ones right child)   */
  int64_t device_bytes;      /* device memory held by the context            */
  int64_t forward_bytes;     /* algorithmic HBM bytes of one forward sweep:
                                parent CLV + scaler writes, inner-child CLV +
                                scaler reads, tip-code reads                  */
  int64_t backward_bytes;    /* algorithmic HBM bytes of one adjoint sweep   */
  int64_t launches_per_gradient_eval; /* kernels of one logL + gradient call:
                                P-matrices, one forward launch per level,
                                site sums, mixture, one adjoint launch per
                                level, the recompute launches of checkpointed
                                segments, two gradient reduction stages       */
  int32_t checkpoint_segments; /* segments in use (1 = every CLV stored)     */
  int32_t clv_slots;           /* CLV buffers held (= n_variants when 1)     */
  int64_t recompute_site_updates; /* extra forward updates per gradient eval */
  int64_t recompute_bytes;     /* algorithmic HBM bytes of those recomputes
                                  (counted like forward_bytes)              */
} netlk_dag_stats;

/* --------------------------------------------------------------- lifecycle */
typedef struct netlk_ctx netlk_ctx;

int netlk_options_default(netlk_options *opts);

/* Builds the displayed-tree DAG (the reference's processNodeImproved schedule,
 * src/likelihood/ImprovedLoglikelihood.cpp:194-408, on bitsets over the 2^r
 * reticulation configurations), uploads tips and parameters.
 * Replaces init_annotated_network (src/graph/AnnotatedNetwork.cpp:80-185) and
 * createNetworkPllTreeinfo (src/RaxmlWrapper.cpp:671-766).
 * branch_lengths: [n_edges] (clamped to [1e-6, 100] like the reference,
 * src/RaxmlWrapper.cpp:754-763); ret_first_probs: [n_reticulations]. */
int netlk_create(const netlk_topology *topo, const netlk_partition *parts,
                 int32_t n_parts, const double *branch_lengths,
                 const double *ret_first_probs, const netlk_options *opts,
                 netlk_ctx **out);
int netlk_destroy(netlk_ctx *ctx);

/* Message of the last failing call on ctx (or, with ctx NULL, of the last
 * failed netlk_create / context-free call on this thread). Valid until the
 * next call on the same context. */
const char *netlk_last_error(const netlk_ctx *ctx);
const char *netlk_status_string(int status);

int netlk_get_dag_stats(const netlk_ctx *ctx, netlk_dag_stats *out);

/* Displayed-tree DAG export, for enumeration parity checks.
 * node_of_variant [n_variants]; children [2*n_variants] (variant id >= 0,
 * -1-tip for a tip, INT32_MIN for the fake all-ones child); edges
 * [2*n_variants] (-1 for the fake child); covered [n_variants*words] bitset of
 * the full reticulation configurations (bit t = tree index t of
 * getTreeConfig, src/helper/ReticulationConfigHelper.cpp:188-203) the variant
 * stands for; words = max(1, 2^r/64). Any output pointer may be NULL. */
int netlk_dag_export(const netlk_ctx *ctx, int32_t *node_of_variant,
                     int32_t *children, int32_t *edges, uint64_t *covered,
                     int32_t words);

/* Root-variant export: variant id [n_root_variants], the variant whose CLV
 * gives its tree log-likelihood (findFirstNodeWithTwoActiveChildren +
 * findMatchingDisplayedTree, src/likelihood/ImprovedLoglikelihood.cpp:428-432)
 * [n_root_variants], and its log-probability [n_root_variants]. */
int netlk_root_export(const netlk_ctx *ctx, int32_t *root_variant,
                      int32_t *dtroot_variant, double *logprob);

/* CLV checkpointing plan, no counterpart in the reference (introspection of
 * this library's O(sqrt n) memory plan). n_segments: level segments (1 = every
 * CLV stored); n_clv_slots: CLV buffers held. Arrays (NULL: counts only):
 *   var_slot [n_variants]    CLV buffer of each variant (dag_export order)
 *   permanent [n_variants]   1 if the variant is read by an op of a later
 *                            segment and keeps its buffer for the whole
 *                            evaluation; the others share their segment's
 *                            buffers and are recomputed before the segment's
 *                            adjoint (all but the last segment)
 *   seg_levels [2 * n_segments]  first and last DAG level of each segment
 *                            (levels count from 1 = variants above tips only) */
int netlk_checkpoint_export(const netlk_ctx *ctx, int32_t *n_segments, int32_t *n_clv_slots, int32_t *var_slot,
                            int32_t *permanent, int32_t *seg_levels);
/* Level schedule of the adjoint sweep (one launch per DAG level, deepest
 * first), no counterpart in the reference (introspection of its message
 * buffers). Counts: n_ops adjoint ops, n_slot_reads message-buffer reads,
 * n_levels levels. Arrays (NULL: counts only):
 *   ops [7 * n_ops]      per op in launch order: CLV buffer of its variant,
 *                        of child a and of child b (-1-tip for a tip,
 *                        INT32_MIN for the fake child), message buffer
 *                        written for a and for b (-1 none), first index into
 *                        slot_reads, count
 *   slot_reads [n_slot_reads]  message buffers the ops read
 *   level_begin [n_levels + 1] first op of each launch */
int netlk_adjoint_export(const netlk_ctx *ctx, int32_t *n_ops, int32_t *n_slot_reads, int32_t *n_levels,
                         int32_t *ops, int32_t *slot_reads, int32_t *level_begin);
/* Walk schedule export, for checks of the host schedule. No counterpart in
 * the reference (introspection of this library's single-launch sweeps).
 * Counts: n_fwd forward ops, n_bwd adjoint ops, n_slot_reads message-slot
 * reads; all 0 when the context has no walk schedule (20 states; FP64
 * contexts have one but run the level sweeps). With checkpoint segments the
 * forward walk lists the segments one after the other and the adjoint walk
 * runs one launch per segment (netlk_walk_segments). Arrays (NULL: counts
 * only):
 *   fwd_variant [n_fwd]   variant computed by each forward op, in walk order
 *   bwd_ops [6 * n_bwd]   per adjoint op in walk order: variant x, message
 *                         slot written for child a and for child b (-1 none,
 *                         -2 kept in registers for the next op), 1 if its
 *                         only message comes from the previous op's
 *                         registers, first index into slot_reads, count
 *   slot_reads [n_slot_reads]  message slots the adjoint ops read */
int netlk_walk_export(const netlk_ctx *ctx, int32_t *n_fwd, int32_t *n_bwd, int32_t *n_slot_reads,
                      int32_t *fwd_variant, int32_t *bwd_ops, int32_t *slot_reads);
/* The walk schedule per checkpoint segment, no counterpart in the reference
 * (introspection of the checkpointed single-launch sweeps). n_segments (0
 * without a walk schedule), n_recompute: variants the recompute walks
 * compute. Arrays (NULL: not written), segment s:
 *   bwd_range [2 * n_segments]       adjoint walk ops [begin, end) of s in
 *                                    netlk_walk_export's bwd_ops; segments
 *                                    launch from the top (highest s) down
 *   recompute_variant [n_recompute]  variants recomputed, in walk order
 *   recompute_range [2 * n_segments] [begin, end) of s in recompute_variant:
 *                                    its non-permanent variants, recomputed
 *                                    right before its adjoint launch (empty
 *                                    for the top segment) */
int netlk_walk_segments(const netlk_ctx *ctx, int32_t *n_segments, int32_t *n_recompute, int32_t *bwd_range,
                        int32_t *recompute_variant, int32_t *recompute_range);

/* ----------------------------------------------------- parameter updates */
/* Replace linked_branch_lengths (src/optimization/NetworkState.cpp:93-306). */
int netlk_set_branch_lengths(netlk_ctx *ctx, const double *branch_lengths,
                             int32_t n_edges);
/* Replace setReticulationProb for all reticulations
 * (src/optimization/ReticulationOptimization.cpp:25-38). */
int netlk_set_reticulation_probs(netlk_ctx *ctx, const double *first_probs,
                                 int32_t n_reticulations);
/* Replace the substitution model of one partition (freqs, exchangeabilities,
 * Gamma shape; rates NULL = mean discrete Gamma). */
int netlk_set_model(netlk_ctx *ctx, int32_t partition, const double *freqs,
                    const double *exchangeabilities, double alpha,
                    const double *rates);

/* Per-partition branch lengths (NETLK_BRLEN_UNLINKED contexts): partition
 * `partition`'s lengths [n_edges], clamped like every length. Replaces
 * fake_treeinfo->branch_lengths[partition] (the reference's unlinked
 * linkage, src/optimization/BranchLengthOptimization.cpp:174-185). On an
 * unlinked context netlk_set_branch_lengths gives every partition the same
 * lengths. */
int netlk_set_partition_branch_lengths(netlk_ctx *ctx, int32_t partition, const double *branch_lengths,
                                       int32_t n_edges);
/* Per-partition length scalers (NETLK_BRLEN_SCALED contexts) [n_parts], each
 * > 0: partition p's length of edge e is scalers[p] x the linked length
 * (pllmod_treeinfo's brlen_scalers). */
int netlk_set_branch_length_scalers(netlk_ctx *ctx, const double *scalers, int32_t n_parts);
/* d logL / d (partition p's length of edge e) [n_parts * n_edges] of the last
 * logL + gradient evaluation (any linkage; on a linked context the rows add
 * up to the gradient). On a scaled context d logL / d scaler[p] =
 * sum_e linked_length[e] * row p [e]. */
int netlk_partition_gradient(netlk_ctx *ctx, double *d_brlen_partition);

/* Replace the proportion of invariant sites of one partition (libpll's
 * pll_update_invariant_sites_proportion, which raxml-ng's model code calls
 * for NetRAX's partitions, src/RaxmlWrapper.cpp:621-640; the model
 * optimizer's PINV step, src/optimization/ModelOptimization.cpp:68-76).
 * prop_invar in [0, 0.99]. */
int netlk_set_prop_invar(netlk_ctx *ctx, int32_t partition, double prop_invar);

/* -------------------------------------------------------------- evaluation */
/* Network log-likelihood. Replaces computeLoglikelihood(ann_network, 0, 1)
 * (src/likelihood/LikelihoodComputation.hpp:17-18 ->
 * src/likelihood/ImprovedLoglikelihood.cpp:646-671). partition_logl
 * [n_parts] mirrors fake_treeinfo->partition_loglh; tree_partition_logl
 * [n_root_variants*n_parts] mirrors TreeLoglData::tree_partition_logl
 * (NaN for trees below min_interesting_tree_logprob). Outputs may be NULL. */
int netlk_loglikelihood(netlk_ctx *ctx, double *total, double *partition_logl,
                        double *tree_partition_logl);

/* Log-likelihood plus d logL / d branch length [n_edges] and
 * d logL / d first-parent probability [n_reticulations] from one forward and
 * one adjoint sweep. Replaces the per-edge sumtable / derivative recomputation
 * of src/likelihood/LikelihoodDerivatives.cpp:190-344 and the Brent probes of
 * src/optimization/ReticulationOptimization.cpp:25-118. */
int netlk_loglikelihood_gradient(netlk_ctx *ctx, double *total,
                                 double *partition_logl, double *d_brlen,
                                 double *d_retprob);

/* Log-likelihood with branch `edge` set to `length` (clamped like every
 * length; the other lengths, the model and the probabilities unchanged);
 * the context keeps the new length. Replaces computeLoglikelihoodBrlenOpt
 * (src/likelihood/VirtualRerooting.cpp:348-585), the per-edge evaluation of
 * the branch-length optimizer's Newton-Raphson accept / revert and Brent
 * probes: with incremental evaluation on, only the variants above the edge
 * are recomputed. */
int netlk_edge_loglikelihood(netlk_ctx *ctx, int32_t edge, double length, double *total);
/* The same for one partition's length of the edge (NETLK_BRLEN_UNLINKED
 * contexts): the reference's computeLoglikelihoodBrlenOpt with
 * fake_treeinfo->branch_lengths[partition] changed. */
int netlk_edge_loglikelihood_partition(netlk_ctx *ctx, int32_t edge, int32_t partition, double length,
                                       double *total);
/* Site-CLV updates the last evaluation computed in its forward sweep
 * (fewer than n_variants * patterns after an incremental evaluation). */
int netlk_last_site_updates(const netlk_ctx *ctx, int64_t *site_updates);

/* First and second derivative of the log-likelihood w.r.t. one branch
 * length, for the Newton-Raphson callback (network_derivative_func_multi,
 * src/optimization/BranchLengthOptimization.cpp:171-200) that calls
 * computeLoglikelihoodDerivatives (src/likelihood/LikelihoodDerivatives.cpp:190-232).
 * mode 0: the true derivative of the network logL (adjoint sweep).
 * mode 1: the reference's own formula, per partition: AVERAGE mixes only the
 *   displayed trees on which the edge is active (isActiveBranch: a
 *   reticulation edge counts where the tree's configurations may take it) in
 *   numerator and denominator; BEST differentiates the active tree with the
 *   largest tree_logl * tree_prob. Trees are grouped by displayed tree at the
 *   network root (the reference groups by the virtually rerooted tree pairs
 *   at the edge).
 * With unlinked lengths d1 / d2 are w.r.t. moving every partition's length
 * of the edge together (the sum of the partition shares); with scaled
 * lengths w.r.t. the linked length (sum of s_p x and s_p^2 x the shares),
 * mode 0 only: mode 1 returns NETLK_ERR_UNSUPPORTED there, as the
 * reference's formula throws for scaled lengths (LikelihoodDerivatives.cpp:42-46).
 * Both derivatives are analytic. Contexts evaluate the edge's sumtables
 * (netlk_edge_sumtable below) at the current lengths: built on the first
 * call for the edge and kept while only that edge's lengths change, so a
 * Newton-Raphson loop that sets each proposal (netlk_edge_loglikelihood)
 * and asks for the derivatives pays for one build per edge. Where the
 * tables do not apply (the `sumtables` option 0, more than 4 rate
 * categories with 20 states, tables too large) one forward-mode (tangent)
 * sweep over the variants above the edge runs per call (the log-likelihood
 * at the current lengths recomputed incrementally on the way). Either way
 * every displayed tree's first and
 * second derivative is mixed like the reference's sumtable derivatives
 * (LikelihoodDerivatives.cpp:13-188). Contexts with several
 * checkpoint segments or device-resident lengths take d1 from full adjoint
 * sweeps and d2, when not NULL, as the central difference of d1 over +-h (kept
 * inside [1e-6, 100]): h = min(1e-6, t/200) for FP64 contexts; for FP32
 * contexts h = max(t/200, min(1e-4, (t - 1e-6)/3)). */
int netlk_edge_derivatives(netlk_ctx *ctx, int32_t edge, int32_t mode,
                           double *d1, double *d2);
/* Partition `partition`'s share: the derivatives of that partition's logL
 * w.r.t. its own length of the edge - the df[p] / ddf[p] the reference's
 * Newton-Raphson callback returns for unlinked lengths
 * (BranchLengthOptimization.cpp:189-195). On linked and scaled contexts the
 * same per-partition terms (w.r.t. the partition's effective length), from
 * the edge's sumtables with each partition at its current length where they
 * apply, else the tangent sweep. Needs one checkpoint segment and host
 * lengths. */
int netlk_edge_derivatives_partition(netlk_ctx *ctx, int32_t edge, int32_t partition, int32_t mode, double *d1,
                                     double *d2);

/* Edge sumtables for the Newton-Raphson iterations along one edge: the
 * reference computes the sumtables of an edge once per optimize_branch
 * (computePartitionSumtables, src/likelihood/LikelihoodDerivatives.cpp:249-344,
 * at the virtual reroot of computeLoglikelihoodBrlenOpt) and every NR
 * callback (network_derivative_func_multi,
 * src/optimization/BranchLengthOptimization.cpp:171-200) evaluates them at
 * the proposed length (pll_compute_loglikelihood_derivatives,
 * LikelihoodDerivatives.cpp:95-104). Here the tables are, per displayed tree
 * containing the edge, its outside vector at the edge per (pattern, rate):
 * one forward-mode sweep of the message's S unit directions over the
 * variants above the edge. An evaluation at length t is one pass over them:
 * L = sum_r O_r . (P_r(t) I_r) with I the edge's child CLV (every term
 * non-negative), and L', L'' with P', P''.
 *
 * netlk_edge_sumtable builds the tables at the current parameters (the
 * evaluation builds them itself when they are missing or stale; this entry
 * lets a caller pay for the build where it chooses). *built = 1 when the
 * sumtable path applies, 0 when it does not (20 states with more than 4
 * rate categories, several checkpoint segments, device-resident lengths,
 * the context's `sumtables` option 0, or tables that would take more than
 * half the free device memory); evaluations then take the tangent path.
 * DNA tables come from one forward-mode sweep of the message's 4 unit
 * directions; 20-state tables from one reverse walk per displayed tree
 * down its path to the edge. *n_tables (may be NULL): the tables built, one per displayed tree
 * that contains the edge. */
int netlk_edge_sumtable(netlk_ctx *ctx, int32_t edge, int32_t *built, int32_t *n_tables);
/* logL and its first / second derivative with the edge at the given
 * length(s), without changing the context's parameters. n_lengths = 1: one
 * length t for the edge (scaled contexts: partition p at s_p t); logl[0],
 * d1[0], d2[0] are the totals w.r.t. t, mode as in netlk_edge_derivatives.
 * n_lengths = n_parts (unlinked contexts): partition p's length is
 * lengths[p], and logl[p], d1[p], d2[p] are partition p's logL and its
 * derivatives w.r.t. its own length - the reference's df[p], ddf[p].
 * Lengths are clamped to [1e-6, 100]. The tables stay current while only
 * this edge's lengths (or nothing) change; any other length, model,
 * +I or reticulation probability change rebuilds them on the next call.
 * Where the sumtable path does not apply, the edge is set to the length,
 * evaluated incrementally with the tangent sweep, and set back (its CLVs
 * are recomputed by the next evaluation); contexts with several checkpoint
 * segments or device-resident lengths get NETLK_ERR_UNSUPPORTED there. */
int netlk_edge_sumtable_derivatives(netlk_ctx *ctx, int32_t edge, const double *lengths, int32_t n_lengths,
                                    int32_t mode, double *logl, double *d1, double *d2);
/* The walk of an edge's table build, for checks of the host schedule (works
 * on host-only contexts). No counterpart in the reference (introspection of
 * netlk_edge_sumtable). Counts: n_ops ops (the variants whose subtree holds
 * the edge), n_work work slots, n_tables tables (displayed-tree roots among
 * them), n_groups child groups. Arrays (NULL: counts only):
 *   ops [7 * n_ops]   per op in walk order: variant x, its child on the
 *                     edge's side d and the other child o (refs as in
 *                     netlk_dag_export), mode (1: d hangs from the edge,
 *                     2: d's subtree holds it), work slot read (-1 for
 *                     mode 1), work slot written (-1: no later op reads
 *                     it), table written (-1: x is no displayed-tree root)
 *   group_ref [n_groups]        child whose CLV the edge's message starts
 *                               from, for the group's tables
 *   group_begin [n_groups + 1]  each group's table range */
int netlk_sumtable_export(const netlk_ctx *ctx, int32_t edge, int32_t *n_ops, int32_t *n_work, int32_t *n_tables,
                          int32_t *n_groups, int32_t *ops, int32_t *group_ref, int32_t *group_begin);

/* ------------------------------------------------- sharded (multi-rank) use */
/* Per-(root variant, partition) log-likelihood partial sums over the patterns
 * this context holds [n_root_variants*n_parts]; ranks that hold disjoint
 * pattern slices all-reduce (SUM) these, which is what parallel_reduce_cb does
 * at src/likelihood/ImprovedLoglikelihood.cpp:473-483. */
int netlk_tree_partials(netlk_ctx *ctx, double *tree_partition_logl);
/* Mixes global partials (AVERAGE / BEST, ImprovedLoglikelihood.cpp:521-644)
 * and runs the adjoint sweep over the local patterns: d_brlen_partial
 * [n_edges] must then be all-reduced (SUM); d_retprob [n_reticulations] and
 * total are already global. */
int netlk_mix_and_backward(netlk_ctx *ctx, const double *global_partials,
                           double *total, double *partition_logl,
                           double *d_brlen_partial, double *d_retprob);

/* ------------------------------------------------ device-resident stepping */
/* Enqueue an async copy of n_edges branch lengths from DEVICE memory into the
 * context (no clamping; values must already lie in [1e-6, 100]). */
int netlk_set_branch_lengths_device(netlk_ctx *ctx, const double *d_branch_lengths,
                                    int32_t n_edges);
/* Enqueue one evaluation on the context stream without waiting for it:
 * with_gradient 0 = logL, 1 = logL + gradient. Results stay on the device
 * (netlk_result_pointers); synchronise the stream before reading them. */
int netlk_enqueue(netlk_ctx *ctx, int32_t with_gradient);
/* Device pointers of the results: out [2 + n_parts + n_reticulations]
 * (total, status flag, partition logL, d logL / d reticulation probability)
 * and d_brlen [n_edges]. */
int netlk_result_pointers(netlk_ctx *ctx, const double **d_out, const double **d_brlen);

/* ----------------------------------------------------------- measurement */
/* 1: launch without CUDA graphs and time every kernel with CUDA events on the
 * context stream; 0: off (default). Switching resets the accumulators. */
int netlk_set_profiling(netlk_ctx *ctx, int32_t enable);
/* Per-kernel device time (ms, summed) and launch counts since profiling was
 * enabled, for kernels 0 P-matrices, 1 forward sweep, 2 per-tree site sums,
 * 3 mixture, 4 adjoint sweep, 5 gradient reduction. n >= 6. */
int netlk_kernel_times(netlk_ctx *ctx, double *ms, int64_t *launches, int32_t n);

/* Launch shapes the autotuner chose (index into its shape table) and the
 * time (ms) it measured for each of the first n shapes (0 where untimed). */
int netlk_tuning(const netlk_ctx *ctx, int32_t *fwd_shape, int32_t *bwd_shape, double *fwd_ms,
                 double *bwd_ms, int32_t n);
/* Index of the first walk shape in the autotuner's table: shapes from it on
 * run a sweep as one op walk per warp (the whole DAG, or with checkpointing
 * one segment, per launch) instead of one launch per DAG level. Equals the
 * table size where the context has no walk shapes (20 states, FP64). No
 * counterpart in the reference (measurement). */
int netlk_walk_shape_begin(const netlk_ctx *ctx, int32_t *first_walk_shape);

/* ---------------------------------------------------- allocation-free mixing */
/* No counterpart in the reference: an extra entry point for callers that
 * cannot allocate device memory: programs whose device memory belongs to
 * another allocator or a fixed budget, and latency-bound loops that must not
 * pay for cudaMalloc / cudaFree, which synchronise the device.
 *
 * Mixes displayed-tree site log-likelihoods into the network log-likelihood
 * exactly as netlk_loglikelihood mixes its own: per partition, AVERAGE =
 * log sum_T exp(logprob_T + sum of the tree's site values) or BEST = max_T,
 * skipping trees with logprob_T < min_interesting_tree_logprob; the total is
 * the sum over partitions.
 *   d_site_logl       device [n_trees * n_sites], row = displayed tree: weighted
 *                     per-site (or per-site-block) log-likelihood contributions
 *   d_part_site_begin device [n_parts + 1]: site range of each partition,
 *                     0 <= begin[0] <= ... <= begin[n_parts] <= n_sites (a range
 *                     outside [0, n_sites] is clipped to it, so a bad range
 *                     gives a wrong sum but reads nothing out of bounds)
 *   d_tree_logprob    device [n_trees]: log P(tree)
 *   d_out             device [1 + n_parts]: total, then per-partition logL
 *   stream            cudaStream_t to launch on (NULL = default stream)
 * Works in a fixed device array of NETLK_NOALLOC_MAX_TREE_PARTITIONS doubles
 * (n_trees * n_parts above that is rejected with NETLK_ERR_INVALID_ARGUMENT;
 * the message is in netlk_last_error(NULL)). Asynchronous: results are ready
 * when the stream is. The first call on a device looks up that array's
 * device address (and looks it up again after the device's context was
 * recreated, e.g. by cudaDeviceReset), so make it before any stream capture.
 * All calls on a device share the array: calls whose work overlaps on the
 * GPU race. */
#define NETLK_NOALLOC_MAX_TREE_PARTITIONS 65536
int netlk_mix_site_loglikelihoods_noalloc(const double *d_site_logl, int32_t n_trees, int64_t n_sites,
                                          const int64_t *d_part_site_begin, int32_t n_parts,
                                          const double *d_tree_logprob, int32_t variant,
                                          double min_interesting_tree_logprob, double *d_out,
                                          void *stream);

/* ------------------------------------------------------- batched candidates */
/* The candidate networks of one search move, scored together. Replaces the
 * sequential perform / computeLoglikelihood / undo loop over candidates in
 * filterCandidates (src/search/Filtering.cpp:239-249). A batch holds n
 * contexts (any topologies and partitions, one device) and captures one
 * logL + gradient evaluation of each - branch-length upload, the launches,
 * result download - into ONE CUDA graph (below: persistent launches over all
 * candidates, or each context's launch sequence on its own stream); every
 * call is one graph launch and one synchronisation. The contexts stay owned
 * by the caller, must outlive
 * the batch, and must not be evaluated concurrently with it. Each context
 * uses the branch lengths of its last netlk_set_branch_lengths
 * (netlk_set_branch_lengths_device lengths are rejected). Errors return a
 * status; netlk_last_error(NULL) names the failing candidate. */
typedef struct netlk_batch netlk_batch;
/* Same as netlk_batch_create_ex(..., NETLK_BATCH_AUTO, ...). */
int netlk_batch_create(netlk_ctx *const *ctxs, int32_t n, netlk_batch **out);
/* mode NETLK_BATCH_AUTO: when every context is DNA, FP32, 4 rate categories,
 * with one checkpoint segment, a call runs all candidates in persistent
 * launches - P-matrices of every candidate in one launch, one forward walk
 * whose warps take (candidate, pattern unit) items from a device counter,
 * longest candidate first, site sums and mixtures in one launch each, one
 * adjoint walk the same way, batched gradient reductions and one result
 * gather (nine kernels, one upload of every length, one download of every
 * result, captured once as a CUDA graph); the walk shape of the two
 * persistent launches is timed on the batch at its first call. Otherwise,
 * and with mode NETLK_BATCH_PER_CONTEXT, the graph holds each context's own
 * launch sequence on its own stream. */
#define NETLK_BATCH_AUTO 0
#define NETLK_BATCH_PER_CONTEXT 1
int netlk_batch_create_ex(netlk_ctx *const *ctxs, int32_t n, int32_t mode, netlk_batch **out);
/* Introspection, no counterpart in the reference: whether the batch runs
 * the persistent launches, kernels per call, and the walk shapes chosen. */
int netlk_batch_info(const netlk_batch *b, int32_t *persistent, int64_t *launches_per_call, int32_t *fwd_shape,
                     int32_t *bwd_shape);
/* totals [n]; d_brlen[i] [n_edges of context i] and d_retprob[i]
 * [n_reticulations of context i] may be NULL (either array or entry). */
int netlk_batch_loglikelihood_gradient(netlk_batch *batch, double *totals, double *const *d_brlen,
                                       double *const *d_retprob);
int netlk_batch_destroy(netlk_batch *batch);

/* ----------------------------------------------------- alignment front end */
/* The steps between an alignment file and netlk_partition, done in the
 * reference by raxml-ng / libpll before NetRAX builds its partitions
 * (pattern compression: opts.use_pattern_compression, src/RaxmlWrapper.cpp:329-330).
 * netlk_encode_states: characters -> state masks. states 4: bit i = A C G T
 * (U = T; IUPAC codes R Y S W K M B D H V = their unions; N ? - . O X = all);
 * states 20: bit i = A R N D C Q E G H I L K M F P S T W Y V (B = N|D,
 * Z = Q|E, J = I|L; X ? - . * = all). Case-insensitive. An unknown character
 * returns NETLK_ERR_INVALID_ARGUMENT with its index in bad_index. */
int netlk_encode_states(const char *chars, int64_t n, int32_t states, uint32_t *out_masks, int64_t *bad_index);
/* Distinct alignment columns and their multiplicities. tip_states
 * [n_tips][n_sites] (row = tip); out_patterns receives [n_tips][*n_patterns]
 * (capacity n_tips * n_sites), out_weights [*n_patterns] (capacity n_sites);
 * columns keep the order of their first occurrence. */
int netlk_compress_patterns(const uint32_t *tip_states, int32_t n_tips, int64_t n_sites, uint32_t *out_patterns,
                            double *out_weights, int64_t *n_patterns);

/* ------------------------------------------------------------------- debug */
/* Copies the CLV (converted to double) and scale counters of one variant:
 * clv [n_patterns*rate_cats*states] and scaler [n_patterns] of partition
 * `partition`, after the last evaluation. */
int netlk_get_clv(netlk_ctx *ctx, int32_t variant, int32_t partition,
                  double *clv, int32_t *scaler);
/* The context's CUDA stream (cudaStream_t) for external event timing. */
int netlk_get_stream(netlk_ctx *ctx, void **stream);
/* Kernels launched by this context since creation. */
int netlk_launch_count(const netlk_ctx *ctx, int64_t *launches);
/* Host-side failure injection for tests, no counterpart in the reference:
 * the next evaluation call on ctx fails with `status` (a NETLK_ERR_* code)
 * after its kernels have run, where a timed-out device wait or a CUDA error
 * would be reported. Nothing is done on the device. 0 clears it. */
int netlk_inject_failure(netlk_ctx *ctx, int32_t status);

#ifdef __cplusplus
}
#endif
#endif
