"""ctypes binding of libses3d_gpu.so (include/ses3d_gpu.h).

The product path has no fallback: if the native library is missing or no CUDA
device is present, the calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libses3d_gpu.so")

c_int, c_float, c_double, c_long, c_char_p, c_void_p = (ctypes.c_int, ctypes.c_float, ctypes.c_double,
                                                         ctypes.c_long, ctypes.c_char_p, ctypes.c_void_p)
P_f = ctypes.POINTER(ctypes.c_float)
P_d = ctypes.POINTER(ctypes.c_double)
P_i = ctypes.POINTER(ctypes.c_int)

SES3D_OK = 0
ERRORS = {-1: "SES3D_E_CONFIG", -2: "SES3D_E_OOM", -3: "SES3D_E_CUDA", -4: "SES3D_E_STATE",
          -5: "SES3D_E_NAN", -6: "SES3D_E_NOTFOUND", -7: "SES3D_E_NODEV"}

FIELDS = ["vx", "vy", "vz", "vx_global", "vy_global", "vz_global",
          "sxx_pml", "syy_pml", "szz_pml", "sxy_pml", "syx_pml", "sxz_pml", "szx_pml", "syz_pml", "szy_pml",
          "dxux", "dyuy", "dzuz", "dxuy", "dyux", "dxuz", "dzux", "dyuz", "dzuy",
          "Mxx", "Myy", "Mzz", "Mxy", "Mxz", "Myz", "MM_global"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
KERNELS = ["rho", "cp", "csh", "csv", "Q_mu", "alpha_mu", "Q_kappa", "alpha_kappa"]
KERNEL_ID = {n: i for i, n in enumerate(KERNELS)}


class Config(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("lpd", ctypes.c_int32), ("pml", ctypes.c_int32), ("is_diss", ctypes.c_int32),
                ("adjoint_flag", ctypes.c_int32), ("samp_ad", ctypes.c_int32), ("nt", ctypes.c_int32),
                ("n_events", ctypes.c_int32), ("grad_variant", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("dt", c_float), ("xmin", c_float), ("xmax", c_float), ("ymin", c_float), ("ymax", c_float),
                ("zmin", c_float), ("zmax", c_float), ("zmax_global", c_float),
                ("tau_p", c_float * 3), ("D_p", c_float * 3)]


class Ses3dError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, msg))
        self.code = code


_lib = None

SIGNATURES = {
    "ses3d_gpu_version": (c_char_p, []),
    "ses3d_gpu_select_device": (c_int, [c_int]),
    "ses3d_gpu_create": (c_int, [ctypes.POINTER(Config), ctypes.POINTER(c_void_p)]),
    "ses3d_gpu_destroy": (c_int, [c_void_p]),
    "ses3d_gpu_last_error": (c_char_p, [c_void_p]),
    "ses3d_gpu_set_model": (c_int, [c_void_p] + [P_f] * 7),
    "ses3d_gpu_set_model_device": (c_int, [c_void_p] + [c_void_p] * 7),
    "ses3d_gpu_set_source": (c_int, [c_void_p, c_int, c_float, c_float, c_float, c_int, P_f, P_f, P_i]),
    "ses3d_gpu_set_receivers": (c_int, [c_void_p, c_int, c_int, P_f, P_i, P_i]),
    "ses3d_gpu_set_adjoint_sources": (c_int, [c_void_p, c_int, c_int, P_f, P_f, P_i]),
    "ses3d_gpu_step": (c_int, [c_void_p, c_int]),
    "ses3d_gpu_current_step": (c_int, [c_void_p]),
    "ses3d_gpu_get_seismograms": (c_int, [c_void_p, c_int, P_f, P_f, P_f]),
    "ses3d_gpu_get_field": (c_int, [c_void_p, c_int, c_int, P_f]),
    "ses3d_gpu_set_field": (c_int, [c_void_p, c_int, c_int, P_f]),
    "ses3d_gpu_get_kernel": (c_int, [c_void_p, c_int, c_int, P_d]),
    "ses3d_gpu_get_kernel_sum": (c_int, [c_void_p, c_int, P_d]),
    "ses3d_gpu_get_kernel_sum_device": (c_int, [c_void_p, c_int, c_void_p]),
    "ses3d_gpu_add_kernel_sum_device": (c_int, [c_void_p, c_int, c_void_p]),
    "ses3d_gpu_misfit_gradient_device": (c_int, [ctypes.POINTER(Config), c_void_p, ctypes.c_double, c_void_p,
                                                 c_void_p, c_int]),
    "ses3d_gpu_selftest_wait": (c_int, [c_void_p, c_int]),
    "ses3d_gpu_record_count": (c_int, [c_void_p, c_int]),
    "ses3d_gpu_get_record": (c_int, [c_void_p, c_int, c_int, P_f]),
    "ses3d_gpu_put_record": (c_int, [c_void_p, c_int, c_int, P_f]),
    "ses3d_gpu_get_saving_vector": (c_int, [c_void_p, P_i]),
    "ses3d_gpu_set_saving_vector": (c_int, [c_void_p, P_i]),
    "ses3d_gpu_begin_adjoint": (c_int, [c_void_p]),
    "ses3d_gpu_set_checkpointing": (c_int, [c_void_p, c_int]),
    "ses3d_gpu_set_checkpoint_levels": (c_int, [c_void_p, c_int, c_int]),
    "ses3d_gpu_set_kernel_shape": (c_int, [c_void_p, c_int, c_int]),
    "ses3d_gpu_kernel_shape_count": (c_int, []),
    "ses3d_gpu_exact_adjoint": (c_int, [c_void_p, c_int, c_int]),
    "ses3d_gpu_exact_set_seismogram_adjoint": (c_int, [c_void_p, c_int, P_f, P_f, P_f]),
    "ses3d_gpu_exact_backward": (c_int, [c_void_p]),
    "ses3d_gpu_exact_gradient": (c_int, [c_void_p, c_int, c_void_p, c_int]),
    "ses3d_gpu_exact_get_field": (c_int, [c_void_p, c_int, c_int, P_f]),
    "ses3d_gpu_exact_set_field": (c_int, [c_void_p, c_int, c_int, P_f]),
    "ses3d_gpu_memory_bytes": (ctypes.c_int64, [c_void_p]),
    "ses3d_gpu_get_setup_int": (c_long, [c_void_p, c_int, c_char_p, P_i]),
    "ses3d_gpu_get_setup_real": (c_long, [c_void_p, c_int, c_char_p, P_f]),
    "ses3d_gpu_vmax": (c_int, [c_void_p, P_f]),
    "ses3d_gpu_stream": (c_void_p, [c_void_p]),
    "ses3d_gpu_launch_count": (ctypes.c_int64, [c_void_p]),
    "ses3d_gpu_use_graph": (c_int, [c_void_p, c_int, c_int]),
    "ses3d_gpu_set_block_elements": (c_int, [c_void_p, c_int]),
    "ses3d_gpu_set_lean": (c_int, [c_void_p, c_int]),
    "ses3d_gpu_step_external": (c_int, [c_void_p, c_void_p, c_void_p, c_int]),
    "ses3d_gpu_profile": (c_int, [c_void_p, c_int]),
    "ses3d_gpu_kernel_time": (c_int, [c_void_p, c_int, P_d, ctypes.POINTER(ctypes.c_int64)]),
}


def load(path: str = LIB_PATH):
    """Loads the native library (built by ses3d_gb300.build.build()); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libses3d_gpu.so not found at %s: build it with ses3d_gb300.build.build()" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def fptr(a: np.ndarray):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(P_f)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(P_d)


def iptr(a: np.ndarray):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(P_i)


def check(rc, h=None):
    if rc < 0:
        msg = load().ses3d_gpu_last_error(h)
        raise Ses3dError(int(rc), msg.decode() if msg else "")
    return rc
