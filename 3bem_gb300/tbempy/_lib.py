"""ctypes binding of lib/libtbem_gpu.so (the C ABI in include/tbem_gpu.h).

The library is the only compute path: importing an operator without it
raises, there is no CPU fallback.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libtbem_gpu.so")

TBEM_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA failure", -3: "allocation failure",
          -4: "invalid state", -5: "device wait timed out"}

PRECISION = {"fp64": 0, "mixed": 1, "fp64_compressed": 2}


class TbemFmmConfig(C.Structure):
    _fields_ = [("mac", C.c_double), ("order", C.c_long), ("min_pts_per_cell", C.c_long),
                ("d", C.c_double), ("account_for_small_cells", C.c_int)]


class TbemGpuOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("device", C.c_int), ("svd_threshold", C.c_double),
                ("m2l_path", C.c_int), ("p2p_block", C.c_int), ("host_only", C.c_int),
                ("m2l_rank_tol", C.c_double), ("p2m_block", C.c_int), ("tc_shape", C.c_int)]


class TbemIntegrator(C.Structure):
    _fields_ = [("strategy", C.c_int), ("near_tol", C.c_double),
                ("sinh_order", C.c_long), ("obs_near_order", C.c_long),
                ("obs_far_order", C.c_long), ("src_far_order", C.c_long),
                ("n_singular_steps", C.c_long), ("far_threshold", C.c_double)]


class TbemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, msg))
        self.code = code


_P, _L, _I, _D = C.c_void_p, C.c_long, C.c_int, C.c_double

# name -> (restype, argtypes); every symbol include/tbem_gpu.h declares
SIGNATURES = {
    "tbem_default_options": (None, [_P]),
    "tbem_fmm_create": (_I, [_I, _P, _P, _P, _L, _P, _P, _P, _L, _P, _P, _P]),
    "tbem_fmm_batch_create": (_I, [_I, _P, _I, _P, _P, _P, _P, _P, _P, _P]),
    "tbem_fmm_n_meshes": (_L, [_P]),
    "tbem_fmm_apply": (_I, [_P, _P, _P, _I, _P]),
    "tbem_fmm_apply_adjoint": (_I, [_P, _P, _P, _I, _P]),
    "tbem_fmm_source_gradients": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "tbem_fmm_observation_gradients": (_I, [_P, _P, _P, _P, _P, _P]),
    "tbem_fmm_n_rows": (_L, [_P]),
    "tbem_fmm_n_cols": (_L, [_P]),
    "tbem_fmm_clone": (_I, [_P, _P]),
    "tbem_fmm_destroy": (None, [_P]),
    "tbem_fmm_tree_cells": (_L, [_P, _I, _P, _P, _P, _P, _P, _P]),
    "tbem_fmm_tree_indices": (_L, [_P, _I, _P]),
    "tbem_fmm_list": (_L, [_P, _I, _P, _P]),
    "tbem_fmm_n_surface": (_L, [_P]),
    "tbem_fmm_n_c2e_levels": (_L, [_P, _I]),
    "tbem_fmm_get_c2e": (_I, [_P, _I, _L, _P]),
    "tbem_fmm_set_c2e": (_I, [_P, _I, _L, _P]),
    "tbem_fmm_set_timing": (_I, [_P, _I]),
    "tbem_fmm_phase_times": (_I, [_P, _P, _P, _I]),
    "tbem_fmm_setup_times": (_I, [_P, _P, _P, _I]),
    "tbem_fma_peak": (_I, [_I, _I, _P]),
    "tbem_setup_cache_clear": (_I, []),
    "tbem_fmm_last_launches": (_L, [_P]),
    "tbem_fmm_sync": (_I, [_P, _P]),
    "tbem_fmm_set_wait_cycles": (_I, [_P, C.c_longlong]),
    "tbem_fmm_p2p_block": (_L, [_P]),
    "tbem_fmm_tc_tile": (_L, [_P]),
    "tbem_fmm_m2l_ranks": (_I, [_P, _P, _P]),
    "tbem_fmm_graph_create": (_I, [_P, _I, _P, _P, _I, _I, _P]),
    "tbem_fmm_graph_launch": (_I, [_P, _P]),
    "tbem_fmm_graph_destroy": (None, [_P]),
    "tbem_direct_apply": (_I, [_I, _P, _P, _P, _L, _P, _P, _P, _L, _P, _P, _I, _P]),
    "tbem_direct_gradients": (_I, [_I, _P, _P, _P, _L, _P, _P, _P, _L, _P, _P, _P, _P, _P, _P,
                                   _P, _P, _P]),
    "tbem_direct_apply_noalloc": (_I, [_I, _P, _P, _P, _L, _P, _P, _P, _L, _P, _P, _I, _P]),
    "tbem_csr_create": (_I, [_L, _L, _P, _P, _P, _P]),
    "tbem_csr_apply": (_I, [_P, _P, _P, _I, _P]),
    "tbem_csr_nnz": (_L, [_P]),
    "tbem_csr_shape": (_I, [_P, _P, _P]),
    "tbem_csr_download": (_I, [_P, _P, _P, _P]),
    "tbem_nearfield_create": (_I, [_I, _P, _P, _L, _P, _L, _P, _L, _P, _L, _P, _I, _P]),
    "tbem_gauss_facet": (_L, [_I, _L, _P, _P]),
    "tbem_galerkin_obs_points": (_L, [_I, _P, _L, _P, _L, _P, _L, _L, _P, _P, _P]),
    "tbem_nearfield_points_create": (_I, [_I, _P, _P, _P, _L, _P, _L, _P, _L, _P, _L, _P, _I, _P]),
    "tbem_interior_obs_points": (_L, [_I, _P, _L, _P, _L, _P, _L, _P]),
    "tbem_csr_destroy": (None, [_P]),
    "tbem_integral_create": (_I, [_P, _P, _P, _P, _P, _P]),
    "tbem_integral_apply": (_I, [_P, _P, _P, _I, _P]),
    "tbem_integral_n_rows": (_L, [_P]),
    "tbem_integral_n_cols": (_L, [_P]),
    "tbem_integral_destroy": (None, [_P]),
    "tbem_last_error": (C.c_char_p, []),
}

_lib = None


def lib():
    """Load the library (raises if it was not built: no fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libtbem_gpu.so not built (run __graft_entry__.build() or "
                              "python 3bem_gb300/build.py): " + LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc < 0:
        msg = lib().tbem_last_error()
        raise TbemError(rc, msg.decode() if msg else "")
    return rc
