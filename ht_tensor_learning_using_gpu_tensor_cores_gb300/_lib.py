"""ctypes binding of the C ABI declared in include/htgb.h.

Loading fails loudly when libhtgb.so is missing: there is no fallback path.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, Structure, c_char_p, c_double, c_float, c_int, c_long, c_longlong, c_ulonglong, c_void_p

MAX_NODES = 7
MAX_ORDER = 4

HT_OK = 0
STATUS = {0: "HT_OK", 1: "HT_ERR_INVALID_ARG", 2: "HT_ERR_CUDA", 3: "HT_ERR_OUT_OF_MEMORY",
          4: "HT_ERR_NOT_CONVERGED", 5: "HT_ERR_TIMEOUT", 6: "HT_ERR_UNSUPPORTED", 7: "HT_ERR_NO_DEVICE",
          8: "HT_ERR_NUMERICAL"}
PREC_FP32, PREC_BF16 = 0, 1
LEAF_GRAM, LEAF_SKETCH = 0, 1
FLAG_COMPUTE_ERROR, FLAG_SYNC_TIMING = 1, 2

#: every extern "C" function declared in include/htgb.h
EXPORTED = ["ht_config_default", "ht_tree_reference_3d", "ht_tree_balanced_4d", "ht_tree_validate",
            "ht_decompose", "ht_reconstruct_error", "ht_workspace_size", "ht_release_workspace",
            "ht_status_string", "ht_last_error", "ht_kernel_launch_count", "htd", "htd4",
            "ht_mode_gram", "ht_mode_product", "ht_corange_product", "ht_tsqr", "ht_selftest_wait_timeout", "ht_mode_gram_noalloc",
            "ht_decompose_batched", "ht_release_batch", "ht_batch_set_tuning", "ht_sketch_loss_grad", "ht_sketch_adam",
            "ht_reconstruct", "ht_evaluate", "ht_layer_weight", "ht_layer_forward", "ht_layer_backward",
            "ht_layer_check", "ht_layer_release", "ht_decompose_streaming"]


class HtTree(Structure):
    _fields_ = [("order", c_int), ("n_nodes", c_int), ("parent", c_int * MAX_NODES), ("left", c_int * MAX_NODES),
                ("right", c_int * MAX_NODES), ("mode_mask", c_int * MAX_NODES), ("rank", c_int * MAX_NODES)]


class HtConfig(Structure):
    _fields_ = [("precision", c_int), ("leaf_method", c_int), ("oversample", c_int), ("eig_iters", c_int),
                ("power_steps", c_int), ("seed", c_ulonglong), ("sketch", c_void_p * MAX_ORDER), ("flags", c_int),
                ("eig_tol", c_double)]


class HtReport(Structure):
    _fields_ = [("rel_err", c_double), ("norm_x", c_double), ("ms_total", c_float), ("ms_stage", c_float * 8),
                ("eig_residual", c_double * MAX_NODES), ("gpu_launches", c_int), ("path_flags", c_int)]


class HtBatchReport(Structure):
    _fields_ = [("rel_err_p50", c_double), ("rel_err_p99", c_double), ("rel_err_max", c_double),
                ("ms_total", c_float), ("gpu_launches", c_int), ("graph_replayed", c_int), ("lanes", c_int),
                ("grouped", c_int), ("ms_phase", c_float * 6)]


class HtLayerShape(Structure):
    _fields_ = [("n", c_int * 3), ("m", c_int * 3), ("r", c_int * 4)]


class HTError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libhtgb.so")
_lib = None


def lib():
    """Load libhtgb.so (build it first with __graft_entry__.build() or
    python -m ht_tensor_learning_using_gpu_tensor_cores_gb300._build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA extension first "
                           "(python -m ht_tensor_learning_using_gpu_tensor_cores_gb300._build)")
    L = ctypes.CDLL(LIB_PATH)
    L.ht_config_default.argtypes = [POINTER(HtConfig)]
    L.ht_tree_reference_3d.argtypes = [POINTER(HtTree), POINTER(c_int)]
    L.ht_tree_balanced_4d.argtypes = [POINTER(HtTree), POINTER(c_int)]
    L.ht_tree_validate.argtypes = [POINTER(HtTree), POINTER(c_long), c_int]
    L.ht_decompose.argtypes = [c_void_p, POINTER(c_long), c_int, POINTER(HtTree), POINTER(HtConfig),
                               POINTER(c_void_p), POINTER(c_void_p), POINTER(HtReport), c_void_p]
    L.ht_reconstruct_error.argtypes = [c_void_p, POINTER(c_long), c_int, POINTER(HtTree), POINTER(c_void_p),
                                       POINTER(c_void_p), POINTER(c_double), c_void_p]
    L.ht_reconstruct.argtypes = [POINTER(c_long), c_int, POINTER(HtTree), POINTER(c_void_p), POINTER(c_void_p),
                                 c_void_p, c_void_p]
    L.ht_evaluate.argtypes = [POINTER(c_long), c_int, POINTER(HtTree), POINTER(c_void_p), POINTER(c_void_p),
                              c_void_p, c_longlong, c_void_p, c_void_p]
    L.ht_decompose_streaming.argtypes = [c_void_p, POINTER(c_long), c_int, POINTER(HtTree), POINTER(HtConfig),
                                         POINTER(c_void_p), POINTER(c_void_p), c_ulonglong, POINTER(HtReport),
                                         c_void_p]
    L.ht_layer_weight.argtypes = [POINTER(HtLayerShape)] + [c_void_p] * 7
    L.ht_layer_forward.argtypes = [POINTER(HtLayerShape)] + [c_void_p] * 6 + [c_int, c_int, c_void_p, c_longlong,
                                                                              c_void_p, c_void_p]
    L.ht_layer_backward.argtypes = [POINTER(HtLayerShape)] + [c_void_p] * 5 + [c_int, c_void_p, c_void_p, c_longlong] \
        + [c_void_p] * 8
    L.ht_layer_check.argtypes = []
    L.ht_layer_release.argtypes = []
    L.ht_workspace_size.argtypes = [POINTER(c_long), c_int, POINTER(HtTree), POINTER(HtConfig), POINTER(c_ulonglong)]
    L.ht_release_workspace.argtypes = []
    L.ht_status_string.argtypes = [c_int]
    L.ht_status_string.restype = c_char_p
    L.ht_last_error.argtypes = []
    L.ht_last_error.restype = c_char_p
    L.ht_kernel_launch_count.argtypes = []
    L.ht_kernel_launch_count.restype = c_ulonglong
    L.htd.argtypes = [c_void_p, c_long, c_long, c_long, POINTER(c_int)]
    L.htd.restype = c_float
    L.htd4.argtypes = [c_void_p, c_long, c_long, c_long, c_long, POINTER(c_int), c_void_p, c_void_p]
    L.htd4.restype = None
    L.ht_mode_gram.argtypes = [c_void_p, POINTER(c_long), c_int, c_int, c_int, c_int, c_void_p, c_void_p]
    L.ht_mode_product.argtypes = [c_void_p, POINTER(c_long), c_int, c_int, c_int, c_void_p, c_int, c_int, c_void_p,
                                  c_void_p]
    L.ht_mode_gram_noalloc.argtypes = [c_void_p, POINTER(c_long), c_int, c_int, c_int, c_void_p, c_void_p]
    L.ht_decompose_batched.argtypes = [c_int, POINTER(c_void_p), POINTER(c_long), c_int, POINTER(HtTree),
                                       POINTER(HtConfig), POINTER(c_void_p), POINTER(c_void_p), POINTER(c_double),
                                       POINTER(HtBatchReport), c_void_p]
    L.ht_release_batch.argtypes = []
    L.ht_sketch_loss_grad.argtypes = [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, POINTER(c_double),
                                      c_void_p]
    L.ht_sketch_adam.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_longlong, c_float, c_int, c_void_p]
    L.ht_corange_product.argtypes = [c_void_p, POINTER(c_long), c_int, c_int, c_int, c_void_p, c_int, c_int,
                                     c_void_p, c_void_p]
    L.ht_tsqr.argtypes = [c_void_p, c_longlong, c_int, c_longlong, c_void_p, c_void_p]
    L.ht_selftest_wait_timeout.argtypes = [c_int, c_double, c_void_p]
    L.ht_batch_set_tuning.argtypes = [c_int, c_int]
    for name in ("ht_decompose_streaming", "ht_layer_weight", "ht_layer_forward", "ht_layer_backward", "ht_layer_check", "ht_layer_release",
                 "ht_reconstruct", "ht_evaluate", "ht_sketch_loss_grad", "ht_sketch_adam", "ht_decompose_batched", "ht_release_batch", "ht_mode_gram", "ht_mode_gram_noalloc", "ht_mode_product", "ht_corange_product", "ht_tsqr", "ht_selftest_wait_timeout", "ht_batch_set_tuning", "ht_config_default", "ht_tree_reference_3d", "ht_tree_balanced_4d", "ht_tree_validate",
                 "ht_decompose", "ht_reconstruct_error", "ht_workspace_size", "ht_release_workspace"):
        getattr(L, name).restype = c_int
    _lib = L
    return L


def check(status: int):
    if status != HT_OK:
        raise HTError(status, lib().ht_last_error().decode(errors="replace"))
