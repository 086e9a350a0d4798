"""ctypes binding of libgigalens_cuda.so (the C ABI in include/gigalens_cuda.h).

The library is the only compute path: importing this module never falls back
to anything else.  ``lib()`` loads it (building it first when it is missing
or older than its sources) and raises if that fails.
"""
import ctypes
import os
import threading

from . import _build

GL_ABI_VERSION = 4   # include/gigalens_cuda.h

GL_OK = 0
GL_ERR_INVALID = -1
GL_ERR_UNSUPPORTED = -2
GL_ERR_CUDA = -3
GL_ERR_NOMEM = -4
GL_ERR_INTERNAL = -5

GL_PROF_NONE = 0
GL_PROF_EPL = 1
GL_PROF_SHEAR = 2
GL_PROF_SIS = 3
GL_PROF_SIE = 4
GL_PROF_TNFW = 5
GL_PROF_SERSIC = 10
GL_PROF_SERSIC_ELLIPSE = 11
GL_PROF_SHAPELETS = 12
GL_PROF_CORE_SERSIC = 13

GL_GROUP_LENS = 0
GL_GROUP_LENS_LIGHT = 1
GL_GROUP_SOURCE = 2

GL_MAX_PROFILES = 8
GL_MAX_PROFILE_PARAMS = 12
GL_MAX_IMAGES = 8
GL_MAX_PARAMS = 64

GL_DIST_NORMAL = 1
GL_DIST_LOGNORMAL = 2
GL_DIST_UNIFORM = 3
GL_DIST_TRUNCNORMAL = 4

PROFILE_TYPES = {
    "EPL": GL_PROF_EPL,
    "SHEAR": GL_PROF_SHEAR,
    "SIS": GL_PROF_SIS,
    "SIE": GL_PROF_SIE,
    "TNFW": GL_PROF_TNFW,
    "SERSIC": GL_PROF_SERSIC,
    "SERSIC_ELLIPSE": GL_PROF_SERSIC_ELLIPSE,
    "SHAPELETS": GL_PROF_SHAPELETS,
    "CORE_SERSIC": GL_PROF_CORE_SERSIC,
}

# canonical parameter order of each type (the header's table)
CANONICAL_PARAMS = {
    "EPL": ["theta_E", "gamma", "e1", "e2", "center_x", "center_y"],
    "SHEAR": ["gamma1", "gamma2"],
    "SIS": ["theta_E", "center_x", "center_y"],
    "SIE": ["theta_E", "e1", "e2", "center_x", "center_y"],
    "SERSIC": ["R_sersic", "n_sersic", "center_x", "center_y", "Ie"],
    "TNFW": ["Rs", "alpha_Rs", "r_trunc", "center_x", "center_y"],
    "SERSIC_ELLIPSE": ["R_sersic", "n_sersic", "e1", "e2", "center_x", "center_y", "Ie"],
    "CORE_SERSIC": ["R_sersic", "n_sersic", "Rb", "alpha", "gamma", "e1", "e2", "center_x", "center_y", "Ie"],
    "SHAPELETS": ["beta", "center_x", "center_y"],   # + amp0: first amplitude column (see _plan)
}


class gl_profile_desc(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int),
        ("group", ctypes.c_int),
        ("niter", ctypes.c_int),
        ("use_lstsq", ctypes.c_int),
        ("col", ctypes.c_int * GL_MAX_PROFILE_PARAMS),
        ("interpolate", ctypes.c_int),
    ]


class gl_model_desc(ctypes.Structure):
    _fields_ = [
        ("n_profiles", ctypes.c_int),
        ("n_params", ctypes.c_int),
        ("prof", gl_profile_desc * GL_MAX_PROFILES),
    ]


class gl_tune_result(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("threads_per_block", "blocks", "samples_per_cta", "smem_bytes",
                                            "family", "global_planes", "subkernel_side", "col_block")]


class gl_tuning(ctypes.Structure):
    _fields_ = [("lsq_ctas_per_sm", ctypes.c_int), ("lsq_col_block", ctypes.c_int),
                ("fused_corr", ctypes.c_int), ("lsq_gram", ctypes.c_int),
                ("reserved", ctypes.c_int * 4)]


class gl_image_desc(ctypes.Structure):
    _fields_ = [
        ("num_pix", ctypes.c_int),
        ("supersample", ctypes.c_int),
        ("transform_pix2angle", ctypes.c_float * 4),
        ("kernel_size", ctypes.c_int),
        ("kernel", ctypes.POINTER(ctypes.c_float)),
        ("observed", ctypes.POINTER(ctypes.c_float)),
        ("background_rms", ctypes.c_float),
        ("exp_time", ctypes.c_float),
        ("err_map", ctypes.POINTER(ctypes.c_float)),
    ]


class gl_prior_leaf(ctypes.Structure):
    _fields_ = [
        ("dist", ctypes.c_int),
        ("a", ctypes.c_float),
        ("b", ctypes.c_float),
        ("c", ctypes.c_float),
        ("d", ctypes.c_float),
    ]


GL_LR_CONSTANT = 0
GL_LR_POLYNOMIAL = 1


class gl_adam_cfg(ctypes.Structure):
    _fields_ = [
        ("schedule", ctypes.c_int),
        ("lr0", ctypes.c_float),
        ("lr_end", ctypes.c_float),
        ("decay_steps", ctypes.c_float),
        ("power", ctypes.c_float),
        ("beta1", ctypes.c_float),
        ("beta2", ctypes.c_float),
        ("eps", ctypes.c_float),
    ]


_vp = ctypes.c_void_p
_i = ctypes.c_int
_i64 = ctypes.c_int64

# (name, restype, argtypes) for every function the header declares
SIGNATURES = [
    ("gl_abi_version", _i, []),
    ("gl_struct_size", _i, [_i]),
    ("gl_last_error", ctypes.c_char_p, []),
    ("gl_device_info", _i, [ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    ("gl_plan_create", _i, [ctypes.POINTER(gl_model_desc), ctypes.POINTER(gl_image_desc), _i,
                            ctypes.POINTER(_vp)]),
    ("gl_plan_set_prior", _i, [_vp, ctypes.POINTER(gl_prior_leaf), _i]),
    ("gl_plan_destroy", _i, [_vp]),
    ("gl_plan_query", _i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    ("gl_forward", _i, [_vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp]),
    ("gl_forward_grad", _i, [_vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp]),
    ("gl_adjoint", _i, [_vp, _vp, _vp, _i, _vp, _vp, _vp, _vp]),
    ("gl_log_prob", _i, [_vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp]),
    ("gl_bijector_forward", _i, [_vp, _vp, _i, _vp, _vp]),
    ("gl_profile_eval", _i, [_i, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp]),
    ("gl_epl_term_count", _i, [_vp, _vp, _i64, _i, _vp, _vp]),
    ("gl_adam_step", _i, [_vp, _vp, _vp, _vp, _i64, ctypes.c_float, ctypes.POINTER(gl_adam_cfg), _vp, _vp]),
    ("gl_probe_fp32_fma", _i, [_vp, _i, _i, ctypes.POINTER(ctypes.c_double), _vp]),
    ("gl_shapelets_eval", _i, [_i, _i, _vp, _vp, _i64, _vp, _vp, _vp, _vp]),
    ("gl_lstsq_workspace", _i, [_vp, _i, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(_i)]),
    ("gl_lstsq", _i, [_vp, _vp, _vp, _i, _vp, ctypes.c_size_t, _vp, _vp, _vp, _vp, _vp]),
    ("gl_lstsq_noalloc", _i, [_vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp]),
    ("gl_lstsq_grad", _i, [_vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp]),
    ("gl_lstsq_status", _i, [_vp, _i, _vp, _vp, _vp]),
    ("gl_test_set_wait_polls", _i, [_i]),
    ("gl_autotune", _i, [_vp, _i, _vp]),
    ("gl_plan_set_tuning", _i, [_vp, ctypes.POINTER(gl_tuning)]),
    ("gl_plan_get_tuning", _i, [_vp, ctypes.POINTER(gl_tuning)]),
    ("gl_nn_gemm", _i, [_i, _i, _i, _i, _i, _i, ctypes.c_float, _vp, _i, ctypes.c_longlong, _vp, _i,
                        ctypes.c_longlong, ctypes.c_float, _vp, _i, ctypes.c_longlong, _i, _i, _vp]),
    ("gl_nn_im2col3x3", _i, [_vp, _i, _i, _i, _i, _i, _vp, _vp]),
    ("gl_nn_col2im3x3", _i, [_vp, _i, _i, _i, _i, _i, _vp, _vp]),
    ("gl_nn_permute01", _i, [_vp, _i, _i, _i, _vp, _vp]),
    ("gl_nn_bias_act", _i, [_vp, _vp, _i, _i, _i, _i, _vp]),
    ("gl_nn_bias_act_backward", _i, [_vp, _vp, _i, _i, _i, _i, _vp, _vp]),
    ("gl_nn_gauss_nll", _i, [_vp, _vp, _i, _i, _vp, _vp, _vp]),
    ("gl_nn_transpose", _i, [_vp, _i, _i, _vp, _vp]),
    ("gl_nn_cast_bf16", _i, [_vp, _vp, ctypes.c_longlong, _vp]),
]

_lock = threading.Lock()
_lib = None


class GigaLensCudaError(RuntimeError):
    """A C-ABI call returned an error code."""

    def __init__(self, fn, code, msg):
        super().__init__("%s failed (%d): %s" % (fn, code, msg))
        self.code = code


def lib_path():
    return _build.LIB


def lib():
    """The loaded library (built on first use if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not _build.up_to_date():
                _build.build()
            handle = ctypes.CDLL(_build.LIB, mode=ctypes.RTLD_GLOBAL)
            for name, res, args in SIGNATURES:
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            if handle.gl_abi_version() != GL_ABI_VERSION:
                raise RuntimeError("%s has ABI version %d, this binding expects %d: rebuild it"
                                   % (_build.LIB, handle.gl_abi_version(), GL_ABI_VERSION))
            _lib = handle
    return _lib


def check(fn_name, rc):
    if rc != GL_OK:
        msg = lib().gl_last_error()
        raise GigaLensCudaError(fn_name, rc, msg.decode() if msg else "")
    return rc


def call(fn_name, *args):
    return check(fn_name, getattr(lib(), fn_name)(*args))


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)
