"""ctypes binding of the C ABI in ``include/cvo_gb300.h``.

The native library is required: importing this module raises if
``_lib/libcvo_gb300.so`` is missing (build it with ``rkhs_ba_gb300._build.build()``).
There is no Python or CPU fallback for the GPU entry points.
"""
from __future__ import annotations

import ctypes as C
import os

from ._build import LIB_PATH

_f = C.c_float
_i = C.c_int
_d = C.c_double

PARAM_FIELDS = [
    ("ell_init_first_frame", _f), ("ell_init", _f), ("ell_min", _f), ("min_ell_iter_limit", _i),
    ("ell_max", _f), ("dl", _d), ("dl_step", _d), ("sigma", _f), ("sp_thres", _f), ("c", _f), ("d", _f),
    ("c_ell", _f), ("c_sigma", _f), ("s_ell", _f), ("s_sigma", _f), ("MAX_ITER", _i), ("eps", _f),
    ("eps_2", _f), ("min_step", _f), ("max_step", _f), ("step", _f), ("nearest_neighbors_max", _i),
    ("ell_decay_rate", _f), ("ell_decay_rate_first_frame", _f), ("ell_decay_start", _i),
    ("ell_decay_start_first_frame", _i), ("indicator_window_size", _i), ("indicator_stable_threshold", _f),
    ("is_pcl_visualization_on", _i), ("is_using_least_square", _i), ("is_ell_adaptive", _i),
    ("is_full_ip_matrix", _i), ("is_using_geometry", _i), ("is_using_intensity", _i),
    ("is_using_semantics", _i), ("is_using_range_ell", _i), ("is_using_kdtree", _i),
    ("is_exporting_association", _i), ("is_using_geometric_type", _i), ("is_global_angle_registration", _i),
    ("multiframe_using_cpu", _i), ("multiframe_max_iters", _i), ("multiframe_ell_init", _f),
    ("multiframe_ell_min", _f), ("multiframe_ell_max", _f), ("multiframe_iter_per_ell", _i),
    ("multiframe_ell_decay_rate", _f), ("multiframe_iterations_per_ell", _i),
    ("multiframe_iterations_per_solve", _i), ("multiframe_expected_points", _i),
    ("multiframe_downsample_voxel_size", _f), ("multiframe_num_neighbors", _i),
    ("multiframe_least_squares_num_threads", _i), ("multiframe_min_nonzeros", _i),
    ("multiframe_is_optimizing_ell", _i), ("multiframe_is_sorting_inner_product", _i),
    ("multiframe_is_free_memory_each_iter", _i),
]


class CvoParamsC(C.Structure):
    _fields_ = PARAM_FIELDS


class CvoCloudC(C.Structure):
    _fields_ = [("n", _i), ("F", _i), ("C", _i), ("xyz_stride", _i),
                ("xyz", C.POINTER(_f)), ("features", C.POINTER(_f)),
                ("labels", C.POINTER(_f)), ("geom_type", C.POINTER(_f))]


# status codes (include/cvo_gb300.h)
CVO_OK = 0
CVO_ZERO_GRADIENT = -1
CVO_ERR_INVALID_ARG = -2
CVO_ERR_EMPTY_CLOUD = -3
CVO_ERR_BAD_YAML = -4
CVO_ERR_CUDA = -5
CVO_ERR_OUT_OF_MEMORY = -6
CVO_ERR_TIMEOUT = -7
CVO_ERR_UNSUPPORTED = -8
CVO_ERR_IO = -9
CVO_ERR_CAPACITY = -10

# every symbol declared in include/cvo_gb300.h with (restype, argtypes)
_P = C.c_void_p
_FP = C.POINTER(_f)
_DP = C.POINTER(_d)
_IP = C.POINTER(_i)
SIGNATURES = {
    "cvo_params_default": (None, [C.POINTER(CvoParamsC)]),
    "cvo_params_read_yaml": (_i, [C.c_char_p, C.POINTER(CvoParamsC)]),
    "cvo_create": (_i, [C.c_char_p, C.POINTER(_P)]),
    "cvo_create_with_params": (_i, [C.POINTER(CvoParamsC), C.POINTER(_P)]),
    "cvo_destroy": (_i, [_P]),
    "cvo_get_params": (_i, [_P, C.POINTER(CvoParamsC)]),
    "cvo_write_params": (_i, [_P, C.POINTER(CvoParamsC)]),
    "cvo_cloud_upload": (_i, [_P, C.POINTER(CvoCloudC), C.POINTER(_P)]),
    "cvo_cloud_free": (_i, [_P, _P]),
    "cvo_cloud_size": (_i, [_P]),
    "cvo_align": (_i, [_P, C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _FP, _FP, _P, _DP, _IP]),
    "cvo_align_dev": (_i, [_P, _P, _P, _FP, _FP, _P, _DP, _IP]),
    "cvo_align_s2t": (_i, [_P, C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _FP, _i, _FP, _P, _DP, _IP, _IP]),
    "cvo_align_batch_dev": (_i, [_P, _i, C.POINTER(_P), C.POINTER(_P), _FP, _FP, _IP, _IP, _DP]),
    "cvo_inner_product": (_i, [_P, C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _FP, _f, _FP]),
    "cvo_inner_product_dev": (_i, [_P, _P, _P, _FP, _f, _FP]),
    "cvo_inner_product_cpu": (_i, [_P, C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _FP, _f, _FP]),
    "cvo_function_angle": (_i, [_P, C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _FP, _f, _i, _i, _FP]),
    "cvo_inner_product_batch_dev": (_i, [_P, _P, _P, _i, _FP, _f, _FP]),
    "cvo_compute_association": (_i, [_P, C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _FP, _f, _P]),
    "cvo_cloud_dims": (_i, [_P, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)]),
    "cvo_cloud_download": (_i, [_P, _P, _FP, _FP, _FP, _FP]),
    "cvo_cloud_from_rgbd": (_i, [_P, _P, _i, _i, _i, _FP, _FP, _f, C.POINTER(_i), _i, _FP, _i, _FP, C.POINTER(_P),
                                 C.POINTER(_i)]),
    "cvo_compute_association_aniso": (_i, [_P, C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _FP, _FP, _P]),
    "cvo_compute_association_aniso_dev": (_i, [_P, _P, _P, _FP, _FP, _P]),
    "cvo_assoc_create": (_i, [C.POINTER(_P)]),
    "cvo_assoc_destroy": (_i, [_P]),
    "cvo_assoc_info": (_i, [_P, _IP, _IP, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "cvo_assoc_copy": (_i, [_P, C.POINTER(C.c_int64), _IP, _FP, _IP, _IP]),
    "cvo_get_nearest_init_pose": (_i, [_P, C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _f, _i, _i, _FP, _DP]),
    "cvo_get_nearest_init_pose_dev": (_i, [_P, _P, _P, _f, _i, _i, _FP, _DP]),
    "cvo_rotation_grid": (_i, [_i, _i, _FP, _i]),
    "cvo_register_hypotheses_dev": (_i, [_P, _P, _P, _i, _FP, _f, _FP, _IP, _FP, _DP]),
    "cvo_autotune_dev": (_i, [_P, _P, _P, _FP, _f, _i, _i, _IP, _FP, _FP, _FP, _IP]),
    "cvo_tune_set": (_i, [_P, _i, _i, C.c_int64, _f, _f]),
    "cvo_autotune_launch_dev": (_i, [_P, _P, _P, _FP, _f, _i, _i, _IP, _FP, _FP, _IP, _FP, _IP]),
    "cvo_tune_set_launch": (_i, [_P, _i, _i, C.c_int64, _f, _f, _i]),
    "cvo_tune_get_launch": (_i, [_P, _i, _i, C.c_int64, _FP, _FP, _IP]),
    "cvo_tune_get": (_i, [_P, _i, _i, C.c_int64, _FP, _FP]),
    "cvo_align_adaptive": (_i, [_P, C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _FP, _FP, _DP, _IP]),
    "cvo_align_adaptive_dev": (_i, [_P, _P, _P, _FP, _FP, _DP, _IP, _DP, _i]),
    "cvo_compute_association_adaptive": (_i, [_P, C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _FP, _f, _P]),
    "cvo_pose_graph_create": (_i, [C.POINTER(_P)]),
    "cvo_pose_graph_destroy": (_i, [_P]),
    "cvo_pose_graph_insert": (_i, [_P, C.c_int64, _DP]),
    "cvo_pose_graph_add_prior": (_i, [_P, C.c_int64, _DP, _DP]),
    "cvo_pose_graph_add_between": (_i, [_P, C.c_int64, C.c_int64, _DP, _DP]),
    "cvo_pose_graph_optimize": (_i, [_P, _i, _DP, _DP, _IP]),
    "cvo_pose_graph_get": (_i, [_P, C.c_int64, _DP]),
    "cvo_pose_graph_size": (_i, [_P, _IP, _IP]),
    "cvo_pose_graph_cost": (_i, [_P, _DP]),
    "cvo_proposal_create": (_i, [_P, _i, C.c_uint32, C.POINTER(_P)]),
    "cvo_proposal_destroy": (_i, [_P]),
    "cvo_proposal_dims": (_i, [_P, _IP, _IP, _IP]),
    "cvo_proposal_get": (_i, [_P, _P, _i, _FP]),
    "cvo_proposal_set": (_i, [_P, _P, _FP]),
    "cvo_proposal_set_gemm": (_i, [_P, _i]),
    "cvo_proposal_train_pool_dev": (_i, [_P, _P, _i, _i, _P, _P, _i, _IP, _FP, _f, C.c_uint32, _FP]),
    "cvo_proposal_forward_pool_dev": (_i, [_P, _P, _i, _i, _P, _P, _i, _IP, _FP, C.c_uint32, _FP, _FP]),
    "cvo_proposal_hypotheses_dev": (_i, [_P, _P, _i, C.POINTER(_P), C.POINTER(_P), C.c_uint32, _FP]),
    "cvo_register_learned_batch_dev": (_i, [_P, _P, _i, C.POINTER(_P), C.POINTER(_P), _i, _f, _f, _f, _f,
                                            C.c_uint32, _FP, _FP, _IP, _IP, _DP]),
    "cvo_global_register": (_i, [_P, _i, C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _i, _P, _FP, _IP, _DP]),
    "cvo_align_multi": (_i, [_P, _i, C.POINTER(CvoCloudC), _DP, C.POINTER(C.c_uint8), _i, _IP, _DP, _IP]),
    "cvo_align_multi_dev": (_i, [_P, _i, C.POINTER(_P), _DP, C.POINTER(C.c_uint8), _i, _IP, _DP, _IP]),
    "cvo_status_string": (C.c_char_p, [_i]),
    "cvo_kernel_launch_count": (C.c_int64, [_P]),
    "cvo_last_error": (C.c_char_p, [_P]),
    "cvo_set_stream": (_i, [_P, _P]),
    "cvo_get_stream": (_P, [_P]),
    "cvo_profile_enable": (_i, [_P, _i]),
    "cvo_profile_read": (_i, [_P, _DP, C.POINTER(C.c_int64), _DP, C.POINTER(C.c_int64)]),
    "cvo_profile_reset": (_i, [_P]),
    "cvo_profile_kernels": (_i, [_P, _DP]),
    "cvo_profile_assoc_split": (_i, [_P, _DP]),
    "cvo_inner_product_noalloc": (_i, [C.POINTER(CvoParamsC), C.POINTER(CvoCloudC), C.POINTER(CvoCloudC), _FP, _f,
                                       _P, _P]),
}

_LIB = None


def lib() -> C.CDLL:
    """Loads the native library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("rkhs_ba_gb300 native library missing at %s; run rkhs_ba_gb300._build.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


class CvoError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        msg = lib().cvo_status_string(code).decode()
        super().__init__("%s failed: %s (%d)%s" % (what, msg, code, ""))
        self.code = code


def check(code: int, what: str, handle=None) -> int:
    if code < 0 and code != CVO_ZERO_GRADIENT:
        err = CvoError(code, what)
        if handle is not None:
            detail = lib().cvo_last_error(handle)
            if detail:
                err.args = (err.args[0] + " [" + detail.decode() + "]",)
        raise err
    return code
