"""ctypes binding of the netlk C ABI (``include/netlk.h``).

The product path has no CPU fallback: if ``libnetlk.so`` cannot be built or
loaded, importing the likelihood API raises.
"""
import ctypes
import os

import importlib

_build = importlib.import_module(__package__ + ".build")

c_int32_p = ctypes.POINTER(ctypes.c_int32)
c_uint32_p = ctypes.POINTER(ctypes.c_uint32)
c_uint64_p = ctypes.POINTER(ctypes.c_uint64)
c_double_p = ctypes.POINTER(ctypes.c_double)

NETLK_OK = 0
NETLK_AVERAGE, NETLK_BEST = 0, 1
NETLK_FP64, NETLK_FP32 = 0, 1
NETLK_ERR_INVALID_ARGUMENT = 1
NETLK_ERR_NO_DEVICE = 8
NETLK_ERR_TIMEOUT = 9

STATUS_NAMES = {
    1: "INVALID_ARGUMENT", 2: "TOPOLOGY", 3: "ENUMERATION", 4: "CUDA",
    5: "OUT_OF_MEMORY", 6: "NUMERIC", 7: "UNSUPPORTED", 8: "NO_DEVICE", 9: "TIMEOUT",
}

EXPORTED = [
    "netlk_options_default", "netlk_create", "netlk_destroy", "netlk_last_error",
    "netlk_status_string", "netlk_get_dag_stats", "netlk_dag_export", "netlk_root_export", "netlk_walk_export",
    "netlk_checkpoint_export", "netlk_adjoint_export",
    "netlk_set_branch_lengths", "netlk_set_reticulation_probs", "netlk_set_model",
    "netlk_loglikelihood", "netlk_loglikelihood_gradient", "netlk_edge_derivatives",
    "netlk_tree_partials", "netlk_mix_and_backward", "netlk_get_clv", "netlk_get_stream",
    "netlk_launch_count", "netlk_set_branch_lengths_device", "netlk_enqueue",
    "netlk_result_pointers", "netlk_set_profiling", "netlk_kernel_times", "netlk_tuning", "netlk_walk_shape_begin",
    "netlk_mix_site_loglikelihoods_noalloc", "netlk_batch_create",
    "netlk_batch_loglikelihood_gradient", "netlk_batch_destroy", "netlk_edge_loglikelihood",
    "netlk_last_site_updates", "netlk_encode_states", "netlk_compress_patterns", "netlk_inject_failure",
    "netlk_walk_segments", "netlk_batch_create_ex", "netlk_batch_info",
    "netlk_set_prop_invar", "netlk_set_partition_branch_lengths", "netlk_set_branch_length_scalers",
    "netlk_partition_gradient", "netlk_edge_loglikelihood_partition", "netlk_edge_derivatives_partition",
    "netlk_edge_sumtable", "netlk_edge_sumtable_derivatives", "netlk_sumtable_export",
]
NETLK_BRLEN_LINKED, NETLK_BRLEN_UNLINKED, NETLK_BRLEN_SCALED = 0, 1, 2


class Topology(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int32), ("n_tips", ctypes.c_int32),
                ("n_edges", ctypes.c_int32), ("n_reticulations", ctypes.c_int32),
                ("root", ctypes.c_int32), ("edge_parent", c_int32_p),
                ("edge_child", c_int32_p), ("node_child_edges", c_int32_p),
                ("ret_node", c_int32_p), ("ret_first_edge", c_int32_p),
                ("ret_second_edge", c_int32_p)]


class Partition(ctypes.Structure):
    _fields_ = [("states", ctypes.c_int32), ("rate_cats", ctypes.c_int32),
                ("n_patterns", ctypes.c_int32), ("tip_states", c_uint32_p),
                ("pattern_weights", c_double_p), ("freqs", c_double_p),
                ("exchangeabilities", c_double_p), ("alpha", ctypes.c_double),
                ("rates", c_double_p), ("rate_weights", c_double_p), ("prop_invar", ctypes.c_double)]


class Options(ctypes.Structure):
    _fields_ = [("variant", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("min_interesting_tree_logprob", ctypes.c_double),
                ("device", ctypes.c_int32), ("use_cuda_graph", ctypes.c_int32),
                ("host_only", ctypes.c_int32), ("autotune", ctypes.c_int32),
                ("tensor_cores", ctypes.c_int32), ("checkpoint_segments", ctypes.c_int32),
                ("incremental", ctypes.c_int32), ("brlen_linkage", ctypes.c_int32),
                ("sumtables", ctypes.c_int32)]


class DagStats(ctypes.Structure):
    _fields_ = [("n_variants", ctypes.c_int32), ("n_root_variants", ctypes.c_int32),
                ("n_dtroot_slots", ctypes.c_int32), ("n_levels", ctypes.c_int32),
                ("n_backward_ops", ctypes.c_int32), ("n_adjoint_slots", ctypes.c_int32),
                ("max_variants_per_node", ctypes.c_int32), ("n_degenerate", ctypes.c_int32),
                ("n_patterns_total", ctypes.c_int64), ("site_clv_updates", ctypes.c_int64),
                ("tip_child_uses", ctypes.c_int64), ("fake_child_uses", ctypes.c_int64),
                ("device_bytes", ctypes.c_int64), ("forward_bytes", ctypes.c_int64),
                ("backward_bytes", ctypes.c_int64), ("launches_per_gradient_eval", ctypes.c_int64),
                ("checkpoint_segments", ctypes.c_int32), ("clv_slots", ctypes.c_int32),
                ("recompute_site_updates", ctypes.c_int64), ("recompute_bytes", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class NetlkError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("netlk %s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


_lib = None


def lib():
    """Load (building if needed) libnetlk.so."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("NETLK_LIB") or _build.LIB  # NETLK_LIB: an alternative build
    if not os.environ.get("NETLK_LIB") and (not os.path.exists(path) or os.environ.get("NETLK_REBUILD")):
        path = _build.build()
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    L.netlk_options_default.argtypes = [ctypes.POINTER(Options)]
    L.netlk_create.argtypes = [ctypes.POINTER(Topology), ctypes.POINTER(Partition), ctypes.c_int32,
                               c_double_p, c_double_p, ctypes.POINTER(Options), ctypes.POINTER(vp)]
    L.netlk_destroy.argtypes = [vp]
    L.netlk_last_error.argtypes = [vp]
    L.netlk_last_error.restype = ctypes.c_char_p
    L.netlk_status_string.argtypes = [ctypes.c_int]
    L.netlk_status_string.restype = ctypes.c_char_p
    L.netlk_get_dag_stats.argtypes = [vp, ctypes.POINTER(DagStats)]
    L.netlk_dag_export.argtypes = [vp, c_int32_p, c_int32_p, c_int32_p, c_uint64_p, ctypes.c_int32]
    L.netlk_root_export.argtypes = [vp, c_int32_p, c_int32_p, c_double_p]
    L.netlk_walk_export.argtypes = [vp, c_int32_p, c_int32_p, c_int32_p, c_int32_p, c_int32_p, c_int32_p]
    L.netlk_checkpoint_export.argtypes = [vp, c_int32_p, c_int32_p, c_int32_p, c_int32_p, c_int32_p]
    L.netlk_adjoint_export.argtypes = [vp, c_int32_p, c_int32_p, c_int32_p, c_int32_p, c_int32_p, c_int32_p]
    L.netlk_set_branch_lengths.argtypes = [vp, c_double_p, ctypes.c_int32]
    L.netlk_set_reticulation_probs.argtypes = [vp, c_double_p, ctypes.c_int32]
    L.netlk_set_model.argtypes = [vp, ctypes.c_int32, c_double_p, c_double_p, ctypes.c_double, c_double_p]
    L.netlk_set_prop_invar.argtypes = [vp, ctypes.c_int32, ctypes.c_double]
    L.netlk_set_partition_branch_lengths.argtypes = [vp, ctypes.c_int32, c_double_p, ctypes.c_int32]
    L.netlk_set_branch_length_scalers.argtypes = [vp, c_double_p, ctypes.c_int32]
    L.netlk_partition_gradient.argtypes = [vp, c_double_p]
    L.netlk_edge_loglikelihood_partition.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                                     c_double_p]
    L.netlk_edge_derivatives_partition.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                   c_double_p, c_double_p]
    L.netlk_edge_sumtable.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                      ctypes.POINTER(ctypes.c_int32)]
    L.netlk_edge_sumtable_derivatives.argtypes = [vp, ctypes.c_int32, c_double_p, ctypes.c_int32, ctypes.c_int32,
                                                  c_double_p, c_double_p, c_double_p]
    i32p = ctypes.POINTER(ctypes.c_int32)
    L.netlk_sumtable_export.argtypes = [vp, ctypes.c_int32, i32p, i32p, i32p, i32p, i32p, i32p, i32p]
    L.netlk_loglikelihood.argtypes = [vp, c_double_p, c_double_p, c_double_p]
    L.netlk_loglikelihood_gradient.argtypes = [vp, c_double_p, c_double_p, c_double_p, c_double_p]
    L.netlk_edge_derivatives.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, c_double_p, c_double_p]
    L.netlk_tree_partials.argtypes = [vp, c_double_p]
    L.netlk_mix_and_backward.argtypes = [vp, c_double_p, c_double_p, c_double_p, c_double_p, c_double_p]
    L.netlk_get_clv.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, c_double_p, c_int32_p]
    L.netlk_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
    L.netlk_launch_count.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
    L.netlk_inject_failure.argtypes = [vp, ctypes.c_int32]
    L.netlk_walk_segments.argtypes = [vp, c_int32_p, c_int32_p, c_int32_p, c_int32_p, c_int32_p]
    L.netlk_set_branch_lengths_device.argtypes = [vp, ctypes.c_void_p, ctypes.c_int32]
    L.netlk_enqueue.argtypes = [vp, ctypes.c_int32]
    L.netlk_result_pointers.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.netlk_set_profiling.argtypes = [vp, ctypes.c_int32]
    L.netlk_mix_site_loglikelihoods_noalloc.argtypes = [
        vp, ctypes.c_int32, ctypes.c_int64, vp, ctypes.c_int32, vp, ctypes.c_int32, ctypes.c_double, vp, vp]
    L.netlk_tuning.argtypes = [vp, c_int32_p, c_int32_p, c_double_p, c_double_p, ctypes.c_int32]
    L.netlk_walk_shape_begin.argtypes = [vp, c_int32_p]
    L.netlk_kernel_times.argtypes = [vp, c_double_p, ctypes.POINTER(ctypes.c_int64), ctypes.c_int32]
    L.netlk_batch_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int32, ctypes.POINTER(vp)]
    L.netlk_batch_create_ex.argtypes = [ctypes.POINTER(vp), ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(vp)]
    L.netlk_batch_info.argtypes = [vp, c_int32_p, ctypes.POINTER(ctypes.c_int64), c_int32_p, c_int32_p]
    L.netlk_batch_loglikelihood_gradient.argtypes = [vp, c_double_p, ctypes.POINTER(c_double_p),
                                                     ctypes.POINTER(c_double_p)]
    L.netlk_batch_destroy.argtypes = [vp]
    L.netlk_edge_loglikelihood.argtypes = [vp, ctypes.c_int32, ctypes.c_double, c_double_p]
    L.netlk_last_site_updates.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
    L.netlk_encode_states.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.c_int32, c_uint32_p,
                                      ctypes.POINTER(ctypes.c_int64)]
    L.netlk_compress_patterns.argtypes = [c_uint32_p, ctypes.c_int32, ctypes.c_int64, c_uint32_p, c_double_p,
                                          ctypes.POINTER(ctypes.c_int64)]
    for name in EXPORTED:
        f = getattr(L, name)
        if f.restype is ctypes.c_int or f.restype is None:
            if name not in ("netlk_last_error", "netlk_status_string"):
                f.restype = ctypes.c_int
    _lib = L
    return L


def check(status, ctx=None):
    if status != NETLK_OK:
        msg = lib().netlk_last_error(ctx)
        raise NetlkError(status, msg.decode() if msg else "")
