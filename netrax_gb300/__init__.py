"""netrax_gb300 - GB300-native network likelihood (NetRAX hot path).

The compute lives in ``libnetlk.so`` (host C++ + sm_103a CUDA, C ABI in
``include/netlk.h``); this package builds and binds it and holds the host-side
helpers (Extended Newick reader, synthetic workloads, autograd wrapper).
"""
from .network import NetworkDesc, parse_extended_newick  # noqa: F401


def build_library(force=False):
    """Compile libnetlk.so in-tree and return its path."""
    import importlib
    return importlib.import_module(__name__ + ".build").build(force=force)
