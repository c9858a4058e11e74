"""ctypes binding of the C ABI declared in ``include/pvd.h``.

This is the only bridge between the Python host code and the CUDA library;
the Python layer passes raw device pointers (from torch tensors) and a
``cudaStream_t`` handle.  Loading fails loudly: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import _build

PVD_OK = 0
STATUS_NAMES = {
    0: "PVD_OK", 1: "PVD_ERR_ARG", 2: "PVD_ERR_CUDA", 3: "PVD_ERR_OOM", 4: "PVD_ERR_TIMEOUT",
    5: "PVD_ERR_NUMERIC", 6: "PVD_ERR_UNSUPPORTED", 7: "PVD_ERR_STATE",
}
PVD_MODE_LINEAR = 0
PVD_MODE_CIRCULAR = 1
PVD_KERNEL_NORMALIZE = 1
PVD_PLAN_TMA = 1
(PVD_FIT_MONO_LAMBDA, PVD_FIT_F2, PVD_FIT_F3, PVD_FIT_F3A, PVD_FIT_F4A, PVD_FIT_F4B, PVD_FIT_F4C,
 PVD_FIT_LM_MONO, PVD_FIT_LM_BI, PVD_FIT_LM_TRI) = range(10)
PVD_FIT_FORCE_ZERO_AT_T0 = 1
PVD_FIT_P0_GIVEN = 2
PVD_FIT_P0_FROM_DATA = 4
PVD_FIT_AUC_INF = 8
PVD_FIT_MIXED = 16
PVD_FIT_VARPRO = 32
PVD_DTYPE_U8, PVD_DTYPE_F32, PVD_DTYPE_F64 = 0, 1, 2
PVD_MAX_KERNELS = 8
PVD_MAX_TIMEPOINTS = 16

# Every symbol include/pvd.h declares, in declaration order.
EXPORTED_SYMBOLS = [
    "pvd_plan_create", "pvd_plan_get_info", "pvd_plan_set_kernel", "pvd_conv_execute",
    "pvd_conv_execute_host", "pvd_conv_execute_weighted", "pvd_plan_destroy", "pvd_plan_status",
    "pvd_conv_execute_static",
    "pvd_fast_lengths", "pvd_plan_profile", "pvd_plan_pass_times",
    "pvd_weighted_sum", "pvd_tac_fit",
    "pvd_mc_plan_create", "pvd_mc_run", "pvd_mc_plan_destroy",
    "pvd_batch_execute", "pvd_batch_create", "pvd_batch_run", "pvd_batch_destroy",
    "pvd_roi_stats", "pvd_histogram", "pvd_dvh",
    "pvd_bspline_prefilter", "pvd_resample", "pvd_resample_separable",
    "pvd_hu_composition",
    "pvd_radial_kernel",
    "pvd_unet_geometry", "pvd_unet_conv3d", "pvd_unet_wgrad_workspace", "pvd_unet_conv3d_wgrad",
    "pvd_unet_pack_weights", "pvd_unet_pack_input", "pvd_unet_pack_input_sym", "pvd_unet_symmetry_accumulate",
    "pvd_unet_pool", "pvd_unet_pool_backward",
    "pvd_unet_upsample", "pvd_unet_upsample_backward", "pvd_unet_head", "pvd_unet_head_loss_workspace",
    "pvd_unet_head_loss", "pvd_unet_head_loss_sym", "pvd_unet_apply_correction", "pvd_unet_input_maxima", "pvd_unet_bias_grad_workspace", "pvd_unet_bias_grad", "pvd_adam_step", "pvd_grad_clip",
    "pvd_unet_status",
    "pvd_wait_check", "pvd_set_plan_alloc_cap",
    "pvd_last_error", "pvd_version", "pvd_launch_count",
]
PVD_WAITCHECK_PLAN, PVD_WAITCHECK_UNET = 0, 1
PVD_HU_ARTIFACTS = 1
PVD_UNET_SYMMETRIES = 48


class PvdError(RuntimeError):
    """A C-ABI call returned a non-OK status."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class ConvDesc(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("kmax", C.c_int * 3), ("mode", C.c_int), ("n_kernels", C.c_int),
                ("pad", C.c_int * 3), ("flags", C.c_int)]


class McDesc(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("voxel_mm", C.c_double * 3),
                ("beta_icdf", C.c_void_p), ("n_beta", C.c_int),
                ("range", C.c_void_p), ("n_range", C.c_int), ("range_de", C.c_float),
                ("mu_rho", C.c_void_p), ("compton_frac", C.c_void_p), ("n_photon", C.c_int), ("photon_de", C.c_float),
                ("n_gamma", C.c_int), ("gamma_e", C.c_float * 8), ("gamma_yield", C.c_float * 8),
                ("beta_yield", C.c_float), ("e_cut", C.c_float)]


class McStats(C.Structure):
    _fields_ = [("total_weight", C.c_ulonglong), ("emitted", C.c_ulonglong), ("escaped", C.c_ulonglong),
                ("steps", C.c_ulonglong), ("activity_bq", C.c_double)]


class BatchItem(C.Structure):
    _fields_ = [("plan", C.c_void_p), ("activity_d", C.c_void_p), ("times", C.c_void_p), ("n_times", C.c_int),
                ("density_d", C.c_void_p), ("params_d", C.c_void_p), ("auc_d", C.c_void_p), ("ok_d", C.c_void_p),
                ("cum_d", C.c_void_p), ("dose_d", C.c_void_p)]


class RoiStats(C.Structure):
    _fields_ = [("min", C.c_double), ("max", C.c_double), ("count", C.c_longlong), ("nonfinite", C.c_longlong)]


class RadialTerm(C.Structure):
    _fields_ = [("type", C.c_int), ("center", C.c_int), ("weight", C.c_double), ("p1", C.c_double),
                ("p2", C.c_double), ("p3", C.c_double)]


PVD_TERM_COLE, PVD_TERM_PHOTON, PVD_TERM_ALPHA, PVD_TERM_EXP_R2 = 0, 1, 2, 3
PVD_CENTER_R0, PVD_CENTER_ZERO, PVD_CENTER_NAN = 0, 1, 2
PVD_MAX_RADIAL_TERMS = 16


class UnetGeom(C.Structure):
    _fields_ = [("dims", C.c_int * 3), ("padded", C.c_int64), ("padded_tiles", C.c_int64),
                ("margin", C.c_int64), ("rows", C.c_int64)]


PVD_UNET_ACT_LEAKY, PVD_UNET_ACCUMULATE = 1, 2


class PlanInfo(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("p", C.c_int * 3), ("h", C.c_int), ("hs", C.c_int),
                ("n_kernels", C.c_int), ("workspace_bytes", C.c_size_t)]


_lib = None
_lock = threading.Lock()


def lib_path() -> Path:
    return _build.LIB_PATH


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load ``libpvd_gb300.so`` (building it first if it is missing or stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_missing and _build.needs_build():
            _build.build()
        path = _build.LIB_PATH
        if not path.exists():
            raise RuntimeError(f"{path} is missing; run pyvoxeldosimetry_gb300._build.build()")
        lib = C.CDLL(str(path))
        _declare(lib)
        _lib = lib
        return lib


def _declare(lib: C.CDLL) -> None:
    vp, i, f, d, st = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_int
    sig = {
        "pvd_plan_create": (st, [C.POINTER(ConvDesc), C.POINTER(vp)]),
        "pvd_plan_get_info": (st, [vp, C.POINTER(PlanInfo)]),
        "pvd_plan_set_kernel": (st, [vp, i, vp, i, i, i, d, i]),
        "pvd_conv_execute": (st, [vp, vp, vp, vp, f, vp]),
        "pvd_conv_execute_host": (st, [vp, vp, vp, vp, f, vp]),
        "pvd_conv_execute_weighted": (st, [vp, vp, vp, i, vp, vp, f, vp]),
        "pvd_plan_destroy": (st, [vp]),
        "pvd_plan_profile": (st, [vp, i]),
        "pvd_plan_status": (st, [vp]),
        "pvd_conv_execute_static": (st, [vp, vp, vp, i, i, i, vp, i, i, i, d, i, f, vp]),
        "pvd_fast_lengths": (i, [C.POINTER(C.c_int), i]),
        "pvd_plan_pass_times": (st, [vp, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
        "pvd_weighted_sum": (st, [vp, vp, i, C.c_longlong, vp, vp]),
        "pvd_tac_fit": (st, [i, vp, vp, i, vp, d, d, i, i, vp, C.c_longlong, vp, vp, vp, vp, d, vp]),
        "pvd_mc_plan_create": (st, [C.POINTER(McDesc), C.POINTER(vp)]),
        "pvd_mc_run": (st, [vp, vp, vp, C.c_ulonglong, C.c_ulonglong, vp, vp, C.POINTER(McStats), vp]),
        "pvd_mc_plan_destroy": (st, [vp]),
        "pvd_batch_execute": (st, [C.POINTER(BatchItem), i, i, i, d, vp]),
        "pvd_batch_create": (st, [C.POINTER(BatchItem), i, i, i, d, C.POINTER(vp)]),
        "pvd_batch_run": (st, [vp, vp]),
        "pvd_batch_destroy": (st, [vp]),
        "pvd_roi_stats": (st, [vp, i, vp, i, C.c_longlong, C.POINTER(RoiStats), vp]),
        "pvd_histogram": (st, [vp, i, vp, i, C.c_longlong, vp, i, vp, vp]),
        "pvd_dvh": (st, [vp, i, vp, i, C.c_longlong, i, vp, vp, vp]),
        "pvd_bspline_prefilter": (st, [vp, vp, vp, i, i, i, vp]),
        "pvd_hu_composition": (st, [vp, i, i, i, i, C.POINTER(f), C.POINTER(f), i, vp, vp, vp, vp]),
        "pvd_radial_kernel": (st, [C.POINTER(RadialTerm), i, d, i, i, i, C.POINTER(C.c_double), vp, vp]),
        "pvd_resample": (st, [vp, i, i, i, vp, i, i, i, C.POINTER(C.c_double), C.POINTER(C.c_double), i, f, vp]),
        "pvd_resample_separable": (st, [vp, i, i, i, vp, i, i, i, C.POINTER(C.c_double), C.POINTER(C.c_double), i, f,
                                        vp, C.c_longlong, vp]),
        "pvd_unet_geometry": (st, [i, i, i, C.POINTER(UnetGeom)]),
        "pvd_unet_conv3d": (st, [C.POINTER(UnetGeom), vp, i, vp, vp, vp, i, vp, i, f, vp]),
        "pvd_unet_wgrad_workspace": (st, [C.POINTER(UnetGeom), i, i, C.POINTER(C.c_size_t)]),
        "pvd_unet_conv3d_wgrad": (st, [C.POINTER(UnetGeom), vp, i, vp, i, vp, i, vp, C.c_size_t, vp]),
        "pvd_unet_pack_weights": (st, [vp, i, i, vp, vp, vp]),
        "pvd_unet_pack_input": (st, [C.POINTER(UnetGeom), C.POINTER(vp), C.POINTER(f), vp, C.POINTER(i), i,
                                     C.POINTER(i), C.POINTER(i), vp, vp]),
        "pvd_unet_pack_input_sym": (st, [C.POINTER(UnetGeom), C.POINTER(vp), C.POINTER(f), vp, C.POINTER(i), i,
                                         C.POINTER(i), C.POINTER(i), i, vp, vp]),
        "pvd_unet_symmetry_accumulate": (st, [C.POINTER(UnetGeom), vp, C.POINTER(UnetGeom), C.POINTER(i), i, f, i,
                                              vp, vp]),
        "pvd_unet_pool": (st, [C.POINTER(UnetGeom), vp, C.POINTER(UnetGeom), vp, i, vp]),
        "pvd_unet_pool_backward": (st, [C.POINTER(UnetGeom), vp, C.POINTER(UnetGeom), vp, vp, i, i, f, vp]),
        "pvd_unet_upsample": (st, [C.POINTER(UnetGeom), vp, C.POINTER(UnetGeom), vp, i, vp]),
        "pvd_unet_upsample_backward": (st, [C.POINTER(UnetGeom), vp, C.POINTER(UnetGeom), vp, vp, i, f, vp]),
        "pvd_unet_head": (st, [C.POINTER(UnetGeom), vp, vp, vp, vp]),
        "pvd_unet_head_loss_workspace": (st, [C.POINTER(UnetGeom), C.POINTER(C.c_size_t)]),
        "pvd_unet_head_loss": (st, [C.POINTER(UnetGeom), vp, vp, vp, vp, vp, C.POINTER(i), C.POINTER(i), f, f, vp,
                                    vp, vp, C.c_size_t, vp]),
        "pvd_unet_head_loss_sym": (st, [C.POINTER(UnetGeom), vp, vp, vp, vp, vp, C.POINTER(i), C.POINTER(i), i, f,
                                        f, vp, vp, vp, C.c_size_t, vp]),
        "pvd_unet_apply_correction": (st, [C.POINTER(UnetGeom), vp, vp, C.POINTER(i), C.POINTER(i), f, f, vp, vp,
                                           vp]),
        "pvd_unet_input_maxima": (st, [vp, vp, vp, C.c_int64, f, vp, vp]),
        "pvd_unet_bias_grad_workspace": (st, [C.POINTER(UnetGeom), i, C.POINTER(C.c_size_t)]),
        "pvd_unet_bias_grad": (st, [C.POINTER(UnetGeom), vp, i, vp, vp, C.c_size_t, vp]),
        "pvd_adam_step": (st, [vp, vp, vp, vp, C.c_int64, f, f, f, f, f, i, vp]),
        "pvd_grad_clip": (st, [vp, C.c_int64, f, f, vp, vp]),
        "pvd_unet_status": (st, [C.POINTER(i), i]),
        "pvd_wait_check": (st, [i, vp, C.c_ulonglong, vp]),
        "pvd_set_plan_alloc_cap": (st, [C.c_size_t]),
        "pvd_last_error": (st, [C.c_char_p, C.c_size_t]),
        "pvd_version": (i, []),
        "pvd_launch_count": (C.c_uint64, [i]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def fast_lengths() -> list:
    """FFT lengths with register four-step pass kernels."""
    lib = load()
    n = lib.pvd_fast_lengths(None, 0)
    buf = (C.c_int * n)()
    lib.pvd_fast_lengths(buf, n)
    return list(buf)


def last_error() -> str:
    lib = load()
    buf = C.create_string_buffer(1024)
    lib.pvd_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    if status != PVD_OK:
        raise PvdError(status, last_error())
