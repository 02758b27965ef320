"""CPU oracle for the phylogenetic-network likelihood path.

TEST INFRASTRUCTURE ONLY. Nothing in the product (``netrax_gb300``) imports,
links or runs anything under this folder; only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm use
it, and only as the checker or as the timed CPU restatement.

What it restates (file:line cites the NetRAX sources, path within the project):

* ``newick.py``   - Extended Newick grammar and the node / edge / reticulation
  index assignment of ``src/io/RootedNetworkParser.cpp:85-381`` and
  ``src/io/NetworkIO.cpp:39-299``.
* ``configsets.py`` - the ReticulationConfigSet algebra of
  ``src/graph/ReticulationConfigSet.cpp:9-242`` and the restriction helpers of
  ``src/helper/ReticulationConfigHelper.cpp:26-203``, on the reference's own
  representation (lists of {DONT_CARE, FIRST, SECOND, INVALID} vectors), with
  the same greedy simplification order.
* ``improved.py`` - the displayed-tree DAG schedule of
  ``src/likelihood/ImprovedLoglikelihood.cpp:115-519`` (single/two-child
  processing, dead-node settings, fake all-ones child), the displayed-tree root
  search of ``src/helper/NetworkFunctions.cpp:228-279``, root log-likelihoods
  (``:410-486``) and AVERAGE / BEST mixing (``:521-644``).
* ``pllmath.py`` / ``clv.c`` - the libpll arithmetic the reference calls but does
  not vendor (the ``libs/raxml-ng`` submodule is empty): GTR eigensystem,
  P = U diag(exp(lambda r t)) U^-1, Yang (1994) mean discrete-Gamma rates,
  Felsenstein pruning with per-site 2^256 scaling, root log-likelihood.
* ``derivatives.py`` - the per-edge branch-length derivatives of
  ``src/likelihood/LikelihoodDerivatives.cpp:13-344`` (per-tree sumtable
  derivatives at the edge, AVERAGE / BEST combination, the ``isActiveBranch``
  restriction of ``src/helper/EdgeHelper.cpp:84-95``) and the exact gradient of
  the network log-likelihood, analytic in both cases.
* ``naive.py``    - the naive per-displayed-tree evaluator of
  ``src/likelihood/NaiveLoglikelihood.cpp:35-115`` (branch lengths merged across
  unary nodes as in ``src/helper/NetworkFunctions.cpp:132-226``), an
  independent cross-check of ``improved.py``.

Parity pinning: the reference cannot be built here (libpll / pll-modules /
raxml-ng sources are absent, MPFR headers are absent), and its own tests hold no
absolute log-likelihood values. The oracle is pinned against the reference's
test invariants on its own fixture networks (improved == naive, repeated ==
repeated, incremental == full) and against an mpmath high-precision evaluation
on small cases; the absolute libpll arithmetic is therefore "parity unpinned".
"""
