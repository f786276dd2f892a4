"""ctypes binding of libctgb.so.

The library is the only compute path of this package: there is no CPU
fallback.  ``lib()`` builds it (nvcc, sm_103a) when it is missing or older
than its sources and raises if it cannot be built or loaded.
"""
from __future__ import annotations

import ctypes as C
import threading

from . import _build

_LOCK = threading.Lock()
_LIB = None

_vp, _i, _d, _f, _ll = C.c_void_p, C.c_int, C.c_double, C.c_float, C.c_longlong
_fp, _dp = C.POINTER(C.c_float), C.POINTER(C.c_double)

# name -> (restype, argtypes); every symbol declared in include/ctgb.h
SIGNATURES = {
    "ct_last_error": (C.c_char_p, []),
    "ct_version": (C.c_char_p, []),
    "ct_dropin_release": (_i, []),
    "ct_ProjectionCone_3D": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _d, _d, _i, _i, _i, _d, _vp]),
    "ct_BackPro": (_i, [_vp, _vp, _vp, _vp, _vp, _d, _i, _i, _i, _vp, _i, _i, _i]),
    "ct_FDKpro": (_i, [_vp, _vp, _vp, _vp, _vp, _d, _i, _i, _i, _vp, _i, _i, _i]),
    "ct_ProjectionFan_2D": (_i, [_vp, _vp, _vp, _vp, _i, _i, _d, _d, _i, _i, _d, _vp]),
    "ct_ProjectionParallel_2D": (_i, [_vp, _vp, _vp, _vp, _i, _i, _d, _d, _i, _i, _vp]),
    "ct_BackprojectionFan2D": (_i, [_vp, _vp, _vp, _vp, _i, _i, _vp, _i, _i, _d]),
    "ct_FBPfan": (_i, [_vp, _vp, _vp, _vp, _i, _i, _vp, _i, _i, _d]),
    "ct_FBPpara": (_i, [_vp, _vp, _vp, _vp, _i, _i, _vp, _i, _i]),
    "ct_FBPfan_noalloc": (_i, [_vp, _vp, _vp, _vp, _i, _i, _vp, _i, _i, _d, _vp]),
    "ct_cone_plan_create": (_i, [C.POINTER(_vp), _i, _i, _i, _vp, _vp, _i, _vp, _i, _vp, _i, _d]),
    "ct_cone_plan_destroy": (_i, [_vp]),
    "ct_cone_plan_set_fdk_mode": (_i, [_vp, _i, _i]),
    "ct_cone_plan_set_filter": (_i, [_vp, _i, _i]),
    "ct_cone_plan_set_short_scan": (_i, [_vp, _i]),
    "ct_cone_plan_workspace_bytes": (C.c_size_t, [_vp]),
    "ct_cone_plan_set_bp_chunk": (_i, [_vp, _i]),
    "ct_cone_plan_get_bp_chunk": (_i, [_vp, _vp]),
    "ct_cone_fp": (_i, [_vp, _vp, _vp, _vp]),
    "ct_cone_fp_residual": (_i, [_vp, _vp, _vp, _vp, _f, _vp, _vp, _vp]),
    "ct_cone_bp": (_i, [_vp, _vp, _vp, _vp]),
    "ct_cone_bp_update": (_i, [_vp, _vp, _vp, _f, _f, _f, _f, _vp, _vp]),
    "ct_cone_fdk": (_i, [_vp, _vp, _vp, _vp]),
    "ct_cone_fdk_filter": (_i, [_vp, _vp, _vp, _vp]),
    "ct_cone_fdk_bp": (_i, [_vp, _vp, _vp, _vp]),
    "ct_cone_count_segments": (_i, [_vp, C.POINTER(_ll), _vp]),
    "ct_cone_plan_grazing_rays": (_i, [_vp, C.POINTER(_ll), _vp]),
    "ct_fan_plan_grazing_rays": (_i, [_vp, C.POINTER(_ll), _vp]),
    "ct_fan_batch_grazing_rays": (_i, [_vp, C.POINTER(_ll), _vp]),
    "ct_set_graze_list_capacity": (_i, [_i]),
    "ct_cone_sysmat": (_i, [_vp, _i, _i, _vp, _vp, _vp, _ll, C.POINTER(_ll), _vp]),
    "ct_par_plan_create": (_i, [C.POINTER(_vp), _i, _i, _vp, _vp, _i, _vp, _i]),
    "ct_fan_sysmat": (_i, [_vp, _vp, _vp, _vp, _ll, C.POINTER(_ll), _vp]),
    "ct_fan_plan_create": (_i, [C.POINTER(_vp), _i, _i, _vp, _vp, _i, _vp, _i, _d]),
    "ct_fan_plan_destroy": (_i, [_vp]),
    "ct_fan_plan_set_filter": (_i, [_vp, _i, _i]),
    "ct_fan_plan_set_short_scan": (_i, [_vp, _i]),
    "ct_fan_fp": (_i, [_vp, _vp, _vp, _vp]),
    "ct_fan_fp_residual": (_i, [_vp, _vp, _vp, _vp, _f, _vp, _vp, _vp]),
    "ct_fan_bp": (_i, [_vp, _vp, _vp, _vp]),
    "ct_fan_bp_update": (_i, [_vp, _vp, _vp, _f, _f, _f, _f, _vp, _vp]),
    "ct_fan_fbp": (_i, [_vp, _vp, _vp, _i, _vp]),
    "ct_fan_batch_create": (_i, [C.POINTER(_vp), _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ct_fan_batch_destroy": (_i, [_vp]),
    "ct_fan_batch_layout": (_i, [_vp, _vp, _vp]),
    "ct_fan_batch_set_blocks": (_i, [_vp, _i, _i]),
    "ct_fan_batch_fp": (_i, [_vp, _vp, _vp, _vp]),
    "ct_fan_batch_fp_residual": (_i, [_vp, _vp, _vp, _vp, _f, _vp, _vp, _vp]),
    "ct_fan_batch_bp": (_i, [_vp, _vp, _vp, _vp]),
    "ct_fan_batch_bp_update": (_i, [_vp, _vp, _vp, _f, _f, _f, _f, _vp, _vp]),
    "ct_fan_batch_fbp": (_i, [_vp, _vp, _vp, _i, _vp]),
    "ct_fan_batch_set_filter": (_i, [_vp, _i, _i, _i]),
    "ct_IterativeFDKerrCompute": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _d, _d, _i, _i, _i, _i, _d,
                                       _vp, _i, _f, _f, _d]),
    "ct_iterfdk_err": (_i, [_vp, _vp, _vp, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i, _i, _i, _d, _i, _vp]),
    "ct_FDKUI": (_i, [_vp, _vp, _vp, _vp, _vp, _d, _d, _d, _d, _i, _i, _i, _vp, _i]),
    "ct_fdkui_filter": (_i, [_vp, _vp, _vp, _vp, _vp, _d, _d, _d, _d, _i, _i, _i, _vp]),
    "ct_fdkui_bp": (_i, [_vp, _vp, _vp, _vp, _vp, _d, _d, _i, _i, _i, _vp, _i, _vp]),
    "ct_csr_kaczmarz": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _i, _f, _vp]),
    "ct_tv_flow": (_i, [_vp, _vp, _vp, _i, _i, _i, _i, _f, _f, _f, _vp]),
    "ct_sq_diff_sum": (_i, [_vp, _vp, _ll, _vp, _vp]),
    "ct_tv_flow_asd": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _i, _i, _i, _f, _f, _f, _f, _vp]),
    "ct_unet_conv3d": (_i, [_vp, _i, _vp, _i, _i, _i, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _vp, _vp]),
    "ct_unet_conv3d_wgrad": (_i, [_vp, _vp, _vp, _i, _vp, _i, _i, _i, _i, _i, _i, _i, _vp, _vp]),
    "ct_unet_status": (_i, [C.POINTER(_i)]),
    "ct_unet_wait_selftest": (_i, [_ll, _vp]),
    "ct_unet_im2col27": (_i, [_vp, _i, _i, _i, _i, _vp, _vp]),
    "ct_unet_pool2": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp]),
    "ct_unet_pool2_bwd": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _i, _i, _vp]),
    "ct_unet_up2": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp]),
    "ct_unet_up2_bwd": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp]),
    "ct_unet_shift_t": (_i, [_vp, _i, _i, _i, _i, _i, _vp, _vp, _vp, _i, _i, _vp]),
    "ct_unet_head": (_i, [_vp, _vp, _vp, _vp, _vp, _ll, _vp]),
    "ct_unet_head_bwd": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _ll, _vp]),
    "ct_unet_colsum": (_i, [_vp, _i, _ll, _vp, _vp]),
}

STATUS = {0: "CT_OK", 1: "CT_ERR_ARG", 2: "CT_ERR_OOM", 3: "CT_ERR_LAUNCH", 4: "CT_ERR_CUDA", 5: "CT_ERR_TIMEOUT"}


class CTError(RuntimeError):
    """A libctgb entry point returned a non-zero ct_status."""

    def __init__(self, status: int, func: str, msg: str):
        super().__init__(f"{func} failed with {STATUS.get(status, status)}: {msg}")
        self.status = status


def load(path=None):
    """Load (building if needed) and return the ctypes library."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        p = path or _build.build()
        lib = C.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _LIB = lib
        return lib


def lib():
    return _LIB if _LIB is not None else load()


def check(status: int, func: str):
    if status != 0:
        msg = lib().ct_last_error().decode(errors="replace")
        raise CTError(status, func, msg)


def call(name: str, *args):
    f = getattr(lib(), name)
    check(f(*args), name)
