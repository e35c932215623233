"""ctypes binding of libdeeds_gpu.so (the C ABI declared in include/deeds_gpu.h).

There is no fallback: if the library is missing or cannot be loaded the import
of the functions that need it raises.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libdeeds_gpu.so")
MAX_LEVELS = 10

DEEDS_OK = 0
ERR_NAMES = {1: "DEEDS_ERR_INVALID", 2: "DEEDS_ERR_CUDA", 3: "DEEDS_ERR_NOMEM", 4: "DEEDS_ERR_TIMEOUT",
             5: "DEEDS_ERR_INTERNAL"}

# every symbol include/deeds_gpu.h declares
EXPORTS = [
    "deeds_default_params", "deeds_create", "deeds_destroy", "deeds_last_error", "deeds_version",
    "deeds_register", "deeds_register_dev", "deeds_warp_segmentation", "deeds_apply_flow",
    "deeds_mind_ssc_dev", "deeds_data_cost_dev", "deeds_mst_edges_dev", "deeds_image_stats", "deeds_image_stats_dev", "deeds_mst_path_counts",
    "deeds_prims_from_sad", "deeds_tree_bp_dev", "deeds_upsample_dev", "deeds_warp_affine_dev",
    "deeds_warp_image_dev", "deeds_warp_seg_dev", "deeds_consistent_dev", "deeds_jacobian_dev",
    "deeds_set_profiling", "deeds_stage_times", "deeds_reset_stage_times", "deeds_kernel_launches",
    "deeds_measure_popc_rate", "deeds_register_batch", "deeds_consistent_noalloc_dev",
    "deeds_soft_default_params", "deeds_soft_descriptor_dev", "deeds_soft_cost_dev", "deeds_soft_forward_dev",
    "deeds_soft_backward_dev", "deeds_soft_upsample_dev", "deeds_soft_upsample_backward_dev", "deeds_soft_warp_dev",
    "deeds_soft_warp_backward_dev", "deeds_soft_forward_keep_dev", "deeds_soft_backward_kept_dev",
    "deeds_soft_release", "deeds_soft_trim", "deeds_soft_forward_batch_dev", "deeds_soft_backward_batch_dev",
    "deeds_soft_release_batch",
    "deeds_linear_default_params", "deeds_linear_register", "deeds_linear_register_dev", "deeds_lin_warp_dev",
    "deeds_lin_smooth_dev", "deeds_estimate_affine_dev", "deeds_affine_robust", "deeds_affine_warp_segmentation",
    "deeds_fuse_labels_dev", "deeds_multi_atlas",
    "deeds_gz_write", "deeds_gz_read", "deeds_gz_last_error", "deeds_selftest_bounded_waits",
]
NOALLOC_MAX_NODES = 131072
STAGES = ["mind", "datacost", "mst_edges", "bp_up", "bp_down", "transform", "consistent", "tree_wait", "bp_argmin"]


class DeedsParams(C.Structure):
    _fields_ = [
        ("levels", C.c_int),
        ("grid", C.c_int * MAX_LEVELS),
        ("radius", C.c_int * MAX_LEVELS),
        ("quant", C.c_int * MAX_LEVELS),
        ("alpha", C.c_float),
        ("intensity_shift", C.c_float),
        ("verbose", C.c_int),
    ]


class DeedsLinearParams(C.Structure):
    _fields_ = [
        ("levels", C.c_int),
        ("grid", C.c_int * MAX_LEVELS),
        ("radius", C.c_int * MAX_LEVELS),
        ("quant", C.c_int * MAX_LEVELS),
        ("rigid", C.c_int),
        ("intensity_shift", C.c_float),
        ("verbose", C.c_int),
    ]


class DeedsPair(C.Structure):
    _fields_ = [
        ("fixed", C.c_void_p),
        ("moving", C.c_void_p),
        ("m", C.c_int),
        ("n", C.c_int),
        ("o", C.c_int),
        ("X", C.c_void_p),
        ("flow_out", C.c_void_p),
        ("warped_out", C.c_void_p),
    ]


class DeedsSoftParams(C.Structure):
    _fields_ = [
        ("grid", C.c_int),
        ("radius", C.c_int),
        ("quant", C.c_int),
        ("mind_radius", C.c_int),
        ("alpha", C.c_float),
        ("tau", C.c_float),
        ("eps", C.c_float),
    ]


class DeedsError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{ERR_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None


def load():
    """Load the library (build it first with deedsbcv_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libdeeds_gpu.so not built ({LIB_PATH}); run python -m deedsbcv_gb300.build")
    L = C.CDLL(LIB_PATH)
    P, I, F, S = C.c_void_p, C.c_int, C.c_float, C.c_size_t
    L.deeds_default_params.argtypes = [C.POINTER(DeedsParams)]
    L.deeds_default_params.restype = None
    L.deeds_create.argtypes = [C.POINTER(P), I]
    L.deeds_destroy.argtypes = [P]
    L.deeds_destroy.restype = None
    L.deeds_last_error.argtypes = [P]
    L.deeds_last_error.restype = C.c_char_p
    L.deeds_version.restype = C.c_char_p
    L.deeds_register.argtypes = [P, P, P, I, I, I, P, C.POINTER(DeedsParams), P, P]
    L.deeds_register_dev.argtypes = [P, P, P, I, I, I, P, C.POINTER(DeedsParams), P, P, P]
    L.deeds_warp_segmentation.argtypes = [P, P, P]
    L.deeds_apply_flow.argtypes = [P, P, S, I, P, P, I, I, I, I, P]
    L.deeds_mind_ssc_dev.argtypes = [P, P, I, I, I, I, P, P]
    L.deeds_data_cost_dev.argtypes = [P, P, P, I, I, I, I, I, I, F, P, P]
    L.deeds_mst_edges_dev.argtypes = [P, P, I, I, I, I, P, P]
    L.deeds_image_stats.argtypes = [P, S, P, P]
    L.deeds_image_stats_dev.argtypes = [P, P, S, P, P]
    L.deeds_mst_path_counts.argtypes = [P]
    L.deeds_fuse_labels_dev.argtypes = [P, P, P, P, I, I, I, I, I, F, I, P, P]
    L.deeds_multi_atlas.argtypes = [P, P, P, P, I, I, I, I, C.POINTER(DeedsParams), I, I, F, I, P, P, P]
    L.deeds_mst_path_counts.restype = None
    L.deeds_prims_from_sad.argtypes = [P, F, I, I, I, I, P, P, P]
    L.deeds_tree_bp_dev.argtypes = [P, P, P, P, P, I, I, I, I, I, P, P, P, P, P, P, P, P]
    L.deeds_upsample_dev.argtypes = [P, P, P, I, I, I, P, P, P, I, I, I, P]
    L.deeds_warp_affine_dev.argtypes = [P, P, P, P, P, I, I, I, P, P]
    L.deeds_warp_image_dev.argtypes = [P, P, P, P, I, I, I, P, P]
    L.deeds_warp_seg_dev.argtypes = [P, P, P, P, P, I, I, I, P, P]
    L.deeds_consistent_dev.argtypes = [P, P, P, P, P, P, P, I, I, I, I, P]
    L.deeds_jacobian_dev.argtypes = [P, P, P, P, I, I, I, I, P, P, P]
    L.deeds_set_profiling.argtypes = [P, I]
    L.deeds_stage_times.argtypes = [P, P, P]
    L.deeds_reset_stage_times.argtypes = [P]
    L.deeds_kernel_launches.argtypes = []
    L.deeds_measure_popc_rate.argtypes = [P, P]
    L.deeds_register_batch.argtypes = [P, P, I, C.POINTER(DeedsParams), I]
    L.deeds_consistent_noalloc_dev.argtypes = [P, P, P, P, P, P, I, I, I, I, P]
    SP = C.POINTER(DeedsSoftParams)
    L.deeds_soft_default_params.argtypes = [SP]
    L.deeds_soft_default_params.restype = None
    L.deeds_soft_descriptor_dev.argtypes = [P, P, I, I, I, I, P, P]
    L.deeds_soft_cost_dev.argtypes = [P, P, P, I, I, I, SP, P, P]
    L.deeds_soft_forward_dev.argtypes = [P, P, P, I, I, I, SP, P, P, P, P, P, P]
    L.deeds_soft_backward_dev.argtypes = [P, P, P, I, I, I, SP, P, P, P, P, P, P, P, P, P, P]
    L.deeds_soft_forward_keep_dev.argtypes = [P, P, P, I, I, I, SP, P, P, P, P, P, C.POINTER(C.c_int), P]
    L.deeds_soft_backward_kept_dev.argtypes = [P, I, P, P, I, I, I, SP, P, P, P, P, P, P, P]
    L.deeds_soft_release.argtypes = [P, I]
    L.deeds_soft_trim.argtypes = [P]
    IP = C.POINTER(C.c_int)
    L.deeds_soft_forward_batch_dev.argtypes = [P, I, P, P, I, I, I, SP, P, P, P, P, P, IP, P]
    L.deeds_soft_backward_batch_dev.argtypes = [P, I, IP, P, P, I, I, I, SP, P, P, P, P, P, P, P, P, P, P]
    L.deeds_soft_release_batch.argtypes = [P, I, IP]
    L.deeds_soft_upsample_dev.argtypes = [P, P, I, I, I, P, I, I, I, P]
    L.deeds_soft_upsample_backward_dev.argtypes = [P, P, I, I, I, P, I, I, I, P]
    L.deeds_soft_warp_dev.argtypes = [P, P, I, I, I, P, I, I, I, P, P]
    L.deeds_soft_warp_backward_dev.argtypes = [P, P, I, I, I, P, I, I, I, P, P, P, P]
    LP = C.POINTER(DeedsLinearParams)
    L.deeds_linear_default_params.argtypes = [LP]
    L.deeds_linear_default_params.restype = None
    L.deeds_linear_register.argtypes = [P, P, P, I, I, I, LP, P]
    L.deeds_linear_register_dev.argtypes = [P, P, P, I, I, I, LP, P, P]
    L.deeds_lin_warp_dev.argtypes = [P, P, I, I, I, P, P]
    L.deeds_lin_smooth_dev.argtypes = [P, I, I, I, I, P]
    L.deeds_estimate_affine_dev.argtypes = [P, P, P, P, P, I, I, I, I, I, I, I, P, P, P, P]
    L.deeds_affine_robust.argtypes = [P, P, I, I, P]
    L.deeds_affine_warp_segmentation.argtypes = [P, P, I, I, I, P, P]
    L.deeds_gz_write.argtypes = [C.c_char_p, P, S, P, S, I, I]
    L.deeds_gz_read.argtypes = [C.c_char_p, P, S, C.POINTER(S), I]
    L.deeds_gz_last_error.argtypes = []
    L.deeds_gz_last_error.restype = C.c_char_p
    L.deeds_selftest_bounded_waits.argtypes = [P, P, P, P]
    for name in EXPORTS:
        fn = getattr(L, name)
        if name not in ("deeds_default_params", "deeds_destroy", "deeds_last_error", "deeds_version",
                        "deeds_soft_default_params", "deeds_linear_default_params", "deeds_gz_last_error"):
            fn.restype = I
    L.deeds_kernel_launches.restype = C.c_longlong
    _lib = L
    return L


def check(status, ctx=None):
    if status != DEEDS_OK:
        msg = load().deeds_last_error(ctx)
        raise DeedsError(status, msg.decode() if msg else "")
