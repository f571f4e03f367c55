"""ctypes binding of libargweaver_gb300.so (include/argweaver_gb300.h).

The reference-compatible prototypes mirror the reference's own ctypes declarations
(argweaver/argweaverc.py:133-167) so Python callers of the reference keep their calls;
the awg_* prototypes expose the flat batch API. Loading fails loudly when the library is
missing: there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

from . import build

_lock = threading.Lock()
_lib = None

c_int_p = C.POINTER(C.c_int)
c_int_pp = C.POINTER(c_int_p)
c_double_p = C.POINTER(C.c_double)
c_double_pp = C.POINTER(c_double_p)
c_char_pp = C.POINTER(C.c_char_p)


class AwgProblem(C.Structure):
    _fields_ = [("ntrees", C.c_int), ("nnodes", C.c_int), ("ntimes", C.c_int),
                ("nseqs", C.c_int), ("seqlen", C.c_int), ("internal", C.c_int),
                ("start_coord", C.c_int), ("minage", C.c_int),
                ("ptrees", C.c_void_p), ("ages", C.c_void_p), ("sprs", C.c_void_p),
                ("blocklens", C.c_void_p), ("mapping", C.c_void_p),
                ("root_child0", C.c_void_p), ("times", C.c_void_p),
                ("popsizes", C.c_void_p), ("rho", C.c_double), ("mu", C.c_double),
                ("seqs", C.c_void_p), ("infsites_penalty", C.c_double)]


class AwgOutputs(C.Structure):
    _fields_ = [("forward", C.c_void_p), ("forward32", C.c_void_p),
                ("posterior", C.c_void_p), ("path", C.c_void_p), ("loglik", C.c_void_p),
                ("uniforms", C.c_void_p)]


AWG_FP64 = 0
AWG_FP32 = 1

# (name, restype, argtypes) of every export declared in include/argweaver_gb300.h
PROTOTYPES = [
    ("arghmm_new_trees", C.c_void_p,
     [c_int_pp, c_int_pp, c_int_pp, c_int_p, C.c_int, C.c_int, C.c_int]),
    ("delete_local_trees", None, [C.c_void_p]),
    ("get_local_trees_ntrees", C.c_int, [C.c_void_p]),
    ("get_local_trees_nnodes", C.c_int, [C.c_void_p]),
    ("get_state_spaces", C.c_void_p, [C.c_void_p, C.c_int, C.c_bool]),
    ("delete_state_spaces", None, [C.c_void_p, C.c_int]),
    ("read_local_trees", C.c_void_p, [C.c_char_p, c_double_p, C.c_int]),
    ("arghmm_copy_trees", C.c_void_p, [C.c_void_p]),
    ("get_local_trees_blocks", None, [C.c_void_p, c_int_p, c_int_p]),
    ("get_treelens", None, [C.c_void_p, c_double_p, C.c_int, c_double_p]),
    ("arghmm_get_nstates", None, [C.c_void_p, C.c_int, C.c_bool, c_int_p]),
    ("arghmm_forward_alg", c_double_pp,
     [C.c_void_p, c_double_p, C.c_int, c_double_p, C.c_double, C.c_double, c_char_pp,
      C.c_int, C.c_int, C.c_bool, c_double_p, C.c_bool, C.c_bool]),
    ("arghmm_backward_alg", c_double_pp,
     [C.c_void_p, c_double_p, C.c_int, c_double_p, C.c_double, C.c_double, c_char_pp,
      C.c_int, C.c_int, C.c_bool]),
    ("arghmm_posterior_marginals", c_double_pp,
     [C.c_void_p, c_double_p, C.c_int, c_double_p, C.c_double, C.c_double, c_char_pp,
      C.c_int, C.c_int, C.c_bool]),
    ("arghmm_sample_posterior", c_int_p,
     [c_int_pp, c_int_pp, c_int_pp, c_int_p, C.c_int, C.c_int, c_double_p, C.c_int,
      c_double_p, C.c_double, C.c_double, c_char_pp, C.c_int, C.c_int, C.c_void_p]),
    ("arghmm_sample_arg_thread_internal", None,
     [C.c_void_p, c_double_p, C.c_int, c_double_p, C.c_double, C.c_double, c_char_pp,
      C.c_int, C.c_int, c_int_p]),
    ("delete_path", None, [c_int_p]),
    ("delete_double_matrix", None, [c_double_pp, C.c_int]),
    ("delete_forward_matrix", None, [c_double_pp, C.c_int]),
    ("new_transition_probs", c_double_pp,
     [C.c_int, c_int_p, c_int_p, C.c_double, c_int_p, C.c_int, C.c_int, c_double_p, c_double_p,
      c_int_p, c_int_p, c_int_p, c_double_p, C.c_double]),
    ("new_transition_probs_switch", c_double_pp,
     [c_int_p, c_int_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, c_int_p, c_int_p,
      C.c_double, C.c_double, c_int_p, C.c_int, c_int_p, C.c_int, C.c_int, c_double_p,
      c_double_p, c_int_p, c_int_p, c_int_p, c_double_p, C.c_double]),
    ("delete_transition_probs", None, [c_double_pp, C.c_int]),
    ("new_emissions", c_double_pp,
     [c_int_p, C.c_int, c_int_p, C.c_int, c_int_p, C.POINTER(C.c_char_p), C.c_int, C.c_int,
      c_double_p, C.c_int, C.c_double]),
    ("delete_emissions", None, [c_double_pp, C.c_int]),
    ("arghmm_likelihood", C.c_double, [C.c_void_p, c_double_p, C.c_int, C.c_double,
                                        c_char_pp, C.c_int, C.c_int]),
    ("arghmm_prior_prob", C.c_double, [C.c_void_p, c_double_p, C.c_int, c_double_p,
                                        C.c_double]),
    ("arghmm_tree_prior_prob", C.c_double, [C.c_void_p, c_double_p, C.c_int, c_double_p]),
    ("arghmm_joint_prob", C.c_double, [C.c_void_p, c_double_p, C.c_int, c_double_p,
                                        C.c_double, C.c_double, c_char_pp, C.c_int, C.c_int]),
    ("awg_sample_recombinations", C.c_int, [C.POINTER(AwgProblem), c_int_p, c_double_p,
                                            C.c_int, c_int_p, c_int_p, c_int_p, C.c_int,
                                            c_int_p]),
    ("get_local_trees_ptrees", None, [C.c_void_p, c_int_pp, c_int_pp, c_int_pp, c_int_p]),
    ("awg_local_trees_seqids", C.c_int, [C.c_void_p, c_int_p]),
    ("awg_local_trees_mapping", C.c_int, [C.c_void_p, c_int_p]),
    ("awg_local_trees_children", C.c_int, [C.c_void_p, c_int_p, c_int_p]),
    ("awg_local_trees_set_structure", C.c_int, [C.c_void_p, c_int_p, c_int_p]),
    ("arghmm_sample_thread", C.c_void_p, [C.c_void_p, c_double_p, C.c_int, c_double_p,
                                          C.c_double, C.c_double, c_char_pp, C.c_int, C.c_int]),
    ("awg_add_arg_thread", C.c_int, [C.c_void_p, C.c_int, c_int_p, C.c_int, c_int_p, c_int_p,
                                     c_int_p, C.c_int]),
    ("awg_remove_arg_thread", C.c_int, [C.c_void_p, C.c_int]),
    ("arghmm_sample_arg_removal_path", None, [C.c_void_p, C.c_int, c_int_p]),
    ("arghmm_sample_arg_removal_path2", None, [C.c_void_p, C.c_int, C.c_int, c_int_p]),
    ("arghmm_sample_arg_removal_leaf_path", None, [C.c_void_p, C.c_int, c_int_p]),
    ("arghmm_sample_arg_removal_path_recomb", None, [C.c_void_p, C.c_double, c_int_p]),
    ("awg_sample_arg_removal_path_uniform", C.c_double, [C.c_void_p, c_int_p]),
    ("arghmm_remove_arg_thread_path", None, [C.c_void_p, c_int_p, C.c_int]),
    ("arghmm_remove_arg_thread_path2", None, [C.c_void_p, c_int_p, C.c_int, c_int_p]),
    ("arghmm_get_thread_times", None, [C.c_void_p, C.c_int, c_int_p, c_int_p]),
    ("awg_add_arg_thread_path", C.c_int, [C.c_void_p, C.c_int, C.c_int, c_int_p, C.c_int,
                                          c_int_p, c_int_p, c_int_p, C.c_int]),
    ("awg_sample_arg_thread", C.c_int, [C.c_void_p, c_double_p, C.c_int, c_double_p, C.c_double,
                                        C.c_double, c_char_pp, C.c_int, C.c_int, C.c_int]),
    ("awg_sample_arg_thread_internal", C.c_int, [C.c_void_p, c_double_p, C.c_int, c_double_p,
                                                 C.c_double, C.c_double, c_char_pp, C.c_int,
                                                 C.c_int, C.c_int, c_int_p]),
    ("awg_read_arg_input", C.c_void_p, [C.c_char_p, C.c_char_p, C.c_int, c_double_p, C.c_int]),
    ("awg_arg_input_dims", C.c_int, [C.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p]),
    ("awg_arg_input_name", C.c_char_p, [C.c_void_p, C.c_int]),
    ("awg_arg_input_copy", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p]),
    ("awg_free_arg_input", None, [C.c_void_p]),
    ("awg_write_sites", C.c_int, [C.c_char_p, c_char_pp, C.c_int, C.c_char_p, C.c_int, C.c_int,
                                  C.c_void_p]),
    ("awg_write_smc", C.c_int, [C.c_char_p, c_char_pp, C.c_char_p, C.c_int, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                c_double_p, C.c_int]),
    ("awg_formats_last_error", C.c_char_p, []),
    ("forward_alg", None, [C.c_int, C.c_int, c_double_pp, c_double_pp, c_double_pp]),
    ("backward_alg", None, [C.c_int, C.c_int, c_double_pp, c_double_pp, c_double_pp]),
    ("sample_hmm_posterior", None, [C.c_int, C.c_int, c_double_pp, c_double_pp, c_int_p]),
    ("awg_problem_cells", C.c_longlong, [C.POINTER(AwgProblem)]),
    ("awg_problems_cells", C.c_int, [C.POINTER(AwgProblem), C.c_int, C.c_void_p]),
    ("awg_run_batch", C.c_int, [C.POINTER(AwgProblem), C.POINTER(AwgOutputs), C.c_int,
                                C.c_int]),
    ("awg_forward_static", C.c_int, [C.POINTER(AwgProblem), C.POINTER(AwgOutputs), C.c_int,
                                     C.c_void_p]),
    ("awg_last_error", C.c_char_p, []),
    ("awg_device_name", C.c_int, [C.c_char_p, C.c_int]),
    ("awg_kernel_launches", C.c_longlong, []),
]

# helpers exported beside the header's API (timing of the last batch)
EXTRA = [
    ("awg_debug_tables", C.c_int, [C.POINTER(AwgProblem), C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p]),
    ("awg_set_timing", None, [C.c_int]),
    ("awg_last_timings", None, [c_double_p]),
]
class AwgServerOptions(C.Structure):
    _fields_ = [("device_bytes", C.c_size_t), ("max_inflight", C.c_int), ("max_batch", C.c_int),
                ("length_ratio", C.c_double)]


class AwgServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("failed", C.c_longlong),
                ("cells", C.c_longlong), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double), ("span_s", C.c_double),
                ("busy_s", C.c_double), ("launch_s", C.c_double), ("inflight_max", C.c_int),
                ("queue_p50_ms", C.c_double), ("queue_p99_ms", C.c_double),
                ("service_p50_ms", C.c_double), ("service_p99_ms", C.c_double)]


# exports of the batch API beyond the reference's (declared in include/argweaver_gb300.h)
PROTOTYPES += [
    ("awg_server_create", C.c_void_p, [C.POINTER(AwgServerOptions)]),
    ("awg_server_destroy", None, [C.c_void_p]),
    ("awg_server_submit", C.c_longlong, [C.c_void_p, C.POINTER(AwgProblem),
                                         C.POINTER(AwgOutputs), C.c_int, C.c_int]),
    ("awg_server_wait", C.c_int, [C.c_void_p, C.c_longlong, C.c_int]),
    ("awg_server_request_times", C.c_int, [C.c_void_p, C.c_longlong, c_double_p]),
    ("awg_server_forget", C.c_int, [C.c_void_p, C.c_longlong]),
    ("awg_server_stats_get", C.c_int, [C.c_void_p, C.POINTER(AwgServerStats)]),
    ("awg_server_resample", C.c_int, [C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]),
    ("awg_server_release", C.c_int, [C.c_void_p, C.c_longlong]),
    ("awg_server_last_error", C.c_char_p, []),
    ("awg_autotune", C.c_int, [C.POINTER(AwgProblem), C.POINTER(AwgOutputs), C.c_int, C.c_int,
                               C.c_int, C.c_char_p, C.c_int]),
    ("awg_batch_device_bytes", C.c_longlong, [C.POINTER(AwgProblem), C.c_int, C.c_int, C.c_int,
                                              C.c_int]),
    ("awg_batch_ctx_create", C.c_void_p, []),
    ("awg_batch_launch", C.c_int, [C.c_void_p, C.POINTER(AwgProblem), C.POINTER(AwgOutputs),
                                   C.c_int, C.c_int]),
    ("awg_batch_finish", C.c_int, [C.c_void_p]),
    ("awg_batch_ctx_destroy", None, [C.c_void_p]),
    ("awg_release_memory", C.c_int, []),
    ("awg_sample_path_conditioned", C.c_int,
     [C.POINTER(AwgProblem), c_double_p, C.c_int, c_double_p, c_int_p, c_double_p]),
    ("awg_set_graphs", None, [C.c_int]),
    ("awg_set_schedule", None, [C.c_int, C.c_int, C.c_int, C.c_int]),
    ("awg_graph_replays", C.c_longlong, []),
    ("awg_graph_captures", C.c_longlong, []),
]


def library_path() -> str:
    return build.CUDA_LIB


def load(build_if_missing: bool = True):
    """Load the library (building it in-tree when missing)."""
    global _lib
    with _lock:
        if _lib is None:
            path = library_path()
            if not os.path.exists(path):
                if not build_if_missing:
                    raise RuntimeError(f"{path} is missing: run argweaver_gb300.build first")
                build.build_cuda()
            lib = C.CDLL(path)
            for name, res, args in PROTOTYPES + EXTRA:
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def last_error() -> str:
    msg = load().awg_last_error()
    return msg.decode() if msg else ""
