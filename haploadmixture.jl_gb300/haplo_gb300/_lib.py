"""ctypes binding of libhaplo_gb300.so (include/haplo_gb300.h).

The shared library is built in-tree by build_ext.py.  Loading fails loudly
when it is missing: there is no CPU fallback for any entry point.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhaplo_gb300.so")

HX_OK, HX_EINVAL, HX_ECUDA, HX_ENAN, HX_ETIMEOUT, HX_ENOMEM, HX_ESTATE, HX_EUNSUPPORTED = range(8)
HX_KMAX = 12
HX_QMAX = 6
HX_PREC_FP64 = 0
HX_PREC_MIXED = 1
HX_PATH_AUTO = 0
HX_PATH_CUDA_CORES = 1


class HxOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("device", C.c_int32), ("Qsec", C.c_int32), ("verbose", C.c_int32),
                ("rho", C.c_double), ("pseudocount", C.c_double), ("path", C.c_int32), ("reserved", C.c_int32)]


class HxLoopOpts(C.Structure):
    _fields_ = [("fix_q", C.c_int32), ("fix_p", C.c_int32), ("guarantee_increase", C.c_int32),
                ("penalty", C.c_int32),
                ("mode", C.c_int32)]


class HxIterInfo(C.Structure):
    _fields_ = [("iter", C.c_int32), ("accepted_qn", C.c_int32), ("ll_prev", C.c_double),
                ("ll_basic", C.c_double), ("ll_qn", C.c_double), ("ll_new", C.c_double),
                ("reldiff", C.c_double), ("seconds", C.c_double)]


class HxFitInfo(C.Structure):
    _fields_ = [("iters", C.c_int32), ("converged", C.c_int32), ("em_iters", C.c_int32), ("pad_", C.c_int32),
                ("ll", C.c_double), ("seconds", C.c_double)]


P = C.c_void_p
D = C.POINTER(C.c_double)
I64 = C.c_int64
I32 = C.c_int32

# name -> (restype, argtypes); every entry point of include/haplo_gb300.h
SIGNATURES = {
    "hx_opts_default": (I32, [C.POINTER(HxOpts)]),
    "hx_loop_opts_default": (I32, [C.POINTER(HxLoopOpts)]),
    "hx_create_shared": (I32, [P, I32, C.POINTER(HxOpts), C.POINTER(P)]),
    "hx_lws_features": (I32, [P, P]),
    "hx_lws_forward": (I32, [P, C.c_int64, I32, P, P, P]),
    "hx_lws_grad": (I32, [P, P, C.c_int64, I32, P, P, P, P]),
    "hx_lws_train": (I32, [P, P, C.c_int64, I32, P, P, P, I32, C.c_int64, C.c_float, C.c_uint64, I32, P, P]),
    "hx_lws_warm_start": (I32, [P, P, I32, C.POINTER(I32)]),
    "hx_fit_many": (I32, [C.POINTER(P), I32, I32, C.c_double, I32, I32, C.POINTER(HxFitInfo), C.POINTER(I32)]),
    "hx_set_loop_opts": (I32, [P, C.POINTER(HxLoopOpts)]),
    "hx_status_string": (C.c_char_p, [I32]),
    "hx_last_error": (C.c_char_p, [P]),
    "hx_create": (I32, [P, I64, I64, I64, I64, I32, C.POINTER(HxOpts), C.POINTER(P)]),
    "hx_create_device": (I32, [P, I64, I64, I64, I64, I32, C.POINTER(HxOpts), C.POINTER(P)]),
    "hx_destroy": (I32, [P]),
    "hx_dims": (I32, [P, C.POINTER(I64), C.POINTER(I64), C.POINTER(I32)]),
    "hx_set_qp": (I32, [P, P, P]),
    "hx_set_qp_device": (I32, [P, P, P]),
    "hx_get_qp": (I32, [P, I32, P, P]),
    "hx_get_ll": (I32, [P, D]),
    "hx_census": (I32, [P, P]),
    "hx_double_missing": (I32, [P, P]),
    "hx_loglikelihood": (I32, [P, P, P, D]),
    "hx_em_accum": (I32, [P, P, P, P, P]),
    "hx_update_q_accum": (I32, [P, P, P, P, P]),
    "hx_update_p_accum": (I32, [P, P, P, P, P]),
    "hx_em_p_accum": (I32, [P, P, P, P]),
    "hx_set_wait_budget": (I32, [P, I64]),
    "hx_autotune": (I32, [P, P]),
    "hx_skfr": (I32, [P, I64, I64, I64, I32, I64, I32, C.c_uint64, I32, P, P, C.POINTER(I32), D]),
    "hx_qp_q": (I32, [P, I64, P, P, P, P]),
    "hx_qp_p": (I32, [P, I64, P, P, P, P]),
    "hx_project_q": (I32, [P, I64, P]),
    "hx_project_p": (I32, [P, I64, P]),
    "hx_zal": (I32, [P, P, P, P, P, P, I32, P]),
    "hx_em_step": (I32, [P]),
    "hx_init_em": (I32, [P, I32]),
    "hx_update_q": (I32, [P, I32]),
    "hx_update_p": (I32, [P, I32]),
    "hx_qn_iteration": (I32, [P, C.POINTER(HxIterInfo)]),
    "hx_admixture_qn": (I32, [P, I32, C.c_double, I32, C.POINTER(HxFitInfo)]),
    "hx_fit": (I32, [P, I32, C.c_double, I32, C.POINTER(HxFitInfo)]),
    "hx_set_profiling": (I32, [P, I32]),
    "hx_kernel_stats": (I32, [P, I32, C.POINTER(I64), D]),
    "hx_reset_stats": (I32, [P]),
    "hx_synth_bed_device": (I32, [C.c_uint64, I64, I64, I32, P, P, C.c_double, P, I32]),
    "hx_loglikelihood_noalloc": (I32, [P, I64, I64, I64, I32, P, P, I32, P, P]),
}

_lib = None


def load(path=LIB_PATH):
    """Loads the library once; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libhaplo_gb300.so not built (%s); run haploadmixture.jl_gb300/build_ext.py" % path)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class HxError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d): %s" % (load().hx_status_string(status).decode(), status, msg))
        self.status = status


def check(status, ctx=None):
    if status != HX_OK:
        msg = load().hx_last_error(ctx).decode() if ctx else ""
        raise HxError(status, msg)


def ptr(a):
    """Pointer to a C-contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)
