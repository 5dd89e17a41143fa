"""ctypes binding of libbfgb300.so (the C ABI in include/boostfractor_gb300.h).

The library is built in-tree by ``boostfractor.jl_gb300/build.py``.  Loading
fails loudly when it is missing: there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "lib", "libbfgb300.so")

BF_OK = 0
BF_ERR_INVALID = 1
BF_ERR_NOMEM = 2
BF_ERR_CUDA = 3
BF_ERR_TIMEOUT = 4
BF_ERR_UNSUPPORTED = 5
BF_ERR_SINGULAR = 6

BF_PROP_3D = 0
BF_PROP_NOTILTS = 1
BF_PROP_MOMENTUM = 2
BF_PROP_1D = 3
BF_NOALLOC_MAX_N = 256

BF_PREC_FP64 = 0
BF_PREC_MIXED = 1
BF_PREC_TF32 = 2
BF_PREC_MIXED_SIMT = 3

BF_OUT_DEVICE = 1
BF_IN_DEVICE = 2

_c_int = ctypes.c_int
_c_dbl = ctypes.c_double
_p_dbl = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p
_ull = ctypes.c_ulonglong

BF_SOLVER_CHEERLEADER = 0
BF_SOLVER_DANCER = 1
BF_SOLVER_TRANSFORMER = 2
BF_SOLVER_PGRID = 3
BF_PENDING = -1
BF_SERVER_DRYRUN = 1
BF_SERVER_RESERVE_HBM = 2


class BFRequest(ctypes.Structure):
    """struct bf_request of include/boostfractor_gb300.h."""
    _fields_ = [("solver", _c_int), ("stack", _vp), ("modes", _vp), ("nf", _c_int), ("freqs", _p_dbl),
                ("distance", _p_dbl), ("nmax", _c_int), ("prop_kind", _c_int), ("precision", _c_int),
                ("beta2_scale", _c_dbl), ("out_beta2", _p_dbl), ("out_boost", _p_dbl),
                ("footprint_bytes", _ull), ("pgrid", _vp), ("lane", _c_int)]


# name -> (restype, argtypes); every symbol declared in include/boostfractor_gb300.h
_SIGS = {
    "bf_version": (_c_int, []),
    "bf_create": (_c_int, [_c_int, _ull, ctypes.POINTER(_vp)]),
    "bf_destroy": (_c_int, [_vp]),
    "bf_last_error": (ctypes.c_char_p, [_vp]),
    "bf_device_bytes": (_ull, [_vp]),
    "bf_set_stream": (_c_int, [_vp, _vp]),
    "bf_set_profiling": (_c_int, [_vp, _c_int]),
    "bf_last_profile": (_c_int, [_vp, _p_dbl]),
    "bf_get_kspace_coords": (_c_int, [_c_int, _p_dbl, _p_dbl]),
    "bf_fresnel_reflectivities": (_c_int, [_c_int, _p_dbl, _p_dbl]),
    "bf_propagate": (_c_int, [_vp, _c_int, _c_int, _p_dbl, _c_int, _c_int, _p_dbl, _p_dbl, _p_dbl,
                              _p_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _p_dbl, _c_dbl]),
    "bf_propagate_noalloc": (_c_int, [_vp, _c_int, _vp, _c_int, _c_int, _p_dbl, _p_dbl, _p_dbl, _p_dbl,
                                      _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _p_dbl, _c_dbl]),
    "bf_gauss_profile": (_c_int, [_c_int, _c_int, _p_dbl, _p_dbl, _c_dbl, _c_dbl, _c_dbl, _p_dbl]),
    "bf_unnormalized_match": (_c_int, [_vp, _c_int, _c_int, _vp, _p_dbl, _c_dbl, _c_dbl, _c_int, _p_dbl]),
    "bf_transformer_coupled": (_c_int, [_vp, _vp, _vp, _c_int, _p_dbl, _c_int, _c_int, _p_dbl, _p_dbl, _p_dbl,
                                        _c_int, _p_dbl, _p_dbl]),
    "bf_transformer_1d_batch": (_c_int, [_vp, _c_int, _c_int, _p_dbl, _p_dbl, _c_int, _p_dbl, _p_dbl, _p_dbl,
                                         _p_dbl]),
    "bf_pgrid_create": (_c_int, [_vp, _vp, _vp, _c_int, _p_dbl, _c_int, _c_dbl, _c_dbl, _c_int, _c_int,
                                 ctypes.POINTER(_vp)]),
    "bf_pgrid_destroy": (_c_int, [_vp, _vp]),
    "bf_pgrid_matrices": (_c_int, [_vp, _vp, _p_dbl, _p_dbl]),
    "bf_pgrid_transformer": (_c_int, [_vp, _vp, _p_dbl, _p_dbl, _p_dbl, _p_dbl]),
    "bf_pgrid_cost": (_c_int, [_vp, _vp, _p_dbl, _p_dbl, ctypes.c_double, _p_dbl, _p_dbl]),
    "bf_stack_graph_stats": (_c_int, [_vp, ctypes.POINTER(_ull), ctypes.POINTER(_ull)]),
    "bf_transformer_trace_back": (_c_int, [_vp, _vp, _vp, _c_int, _p_dbl, _c_int, _c_int, _p_dbl, _p_dbl, _c_int,
                                           _c_int, _p_dbl, _p_dbl, _c_int, _p_dbl]),
    "bf_server_create": (_c_int, [_c_int, _ull, _c_int, _c_int, ctypes.POINTER(_vp)]),
    "bf_server_destroy": (_c_int, [_vp]),
    "bf_submit": (_c_int, [_vp, ctypes.POINTER(BFRequest), ctypes.POINTER(_ull)]),
    "bf_poll": (_c_int, [_vp, _ull, ctypes.POINTER(_c_int), _p_dbl]),
    "bf_wait": (_c_int, [_vp, _ull, _c_int, ctypes.POINTER(_c_int), _p_dbl]),
    "bf_server_stats": (_c_int, [_vp, _c_int, _p_dbl]),
    "bf_server_reset_stats": (_c_int, [_vp]),
    "bf_server_set_latency_lane": (_c_int, [_vp, _c_int]),
    "bf_server_last_error": (ctypes.c_char_p, [_vp]),
    "bf_stack_create": (_c_int, [_vp, _c_int, _p_dbl, _p_dbl, _p_dbl, _p_dbl, _p_dbl, _p_dbl, _c_int,
                                 _c_int, _p_dbl, _p_dbl, _p_dbl, _p_dbl, _c_dbl, ctypes.POINTER(_vp)]),
    "bf_stack_destroy": (_c_int, [_vp, _vp]),
    "bf_stack_set_distance": (_c_int, [_vp, _vp, _p_dbl]),
    "bf_stack_cheerleader": (_c_int, [_vp, _vp, _c_int, _p_dbl, _c_dbl, _c_int, _c_int, _c_int, _p_dbl,
                                      _p_dbl, _c_int, _c_dbl, _c_int, _p_dbl, _p_dbl, _p_dbl]),
    "bf_stack_dancer": (_c_int, [_vp, _vp, _c_int, _p_dbl, _c_dbl, _c_int, _c_int, _c_int, _p_dbl,
                                 _p_dbl, _c_int, _c_int, _c_dbl, _c_int, _p_dbl, _p_dbl]),
    "bf_cheerleader": (_c_int, [_vp, _c_int, _p_dbl, _p_dbl, _p_dbl, _p_dbl, _p_dbl, _p_dbl, _c_int,
                                _c_int, _p_dbl, _p_dbl, _p_dbl, _p_dbl, _c_dbl, _c_int, _p_dbl, _c_dbl,
                                _c_int, _c_int, _c_int, _p_dbl, _p_dbl, _c_int, _c_dbl, _p_dbl, _p_dbl,
                                _p_dbl]),
    "bf_dancer": (_c_int, [_vp, _c_int, _p_dbl, _p_dbl, _p_dbl, _p_dbl, _p_dbl, _p_dbl, _c_int, _c_int,
                           _p_dbl, _p_dbl, _p_dbl, _p_dbl, _c_dbl, _c_int, _p_dbl, _c_dbl, _c_int,
                           _c_int, _c_int, _p_dbl, _p_dbl, _c_int, _c_int, _c_dbl, _p_dbl, _p_dbl]),
    "bf_modes_create": (_c_int, [_vp, _c_int, _c_int, _p_dbl, _p_dbl, _c_int, _c_int, _c_int, _c_dbl, _p_dbl,
                                 _p_dbl, ctypes.POINTER(_vp)]),
    "bf_modes_destroy": (_c_int, [_vp, _vp]),
    "bf_modes_get": (_c_int, [_vp, _vp, ctypes.POINTER(_c_int), _p_dbl, _p_dbl]),
    "bf_axion_induced_modes": (_c_int, [_vp, _vp, _p_dbl, _c_dbl, _c_dbl, _c_dbl, _p_dbl]),
    "bf_modes2field": (_c_int, [_vp, _vp, _p_dbl, _p_dbl]),
    "bf_calc_propagation_matrices": (_c_int, [_vp, _vp, _vp, _c_int, _p_dbl, _c_int, _c_int, _p_dbl]),
    "bf_transformer": (_c_int, [_vp, _vp, _vp, _c_int, _p_dbl, _c_int, _c_int, _p_dbl, _p_dbl, _p_dbl, _c_int,
                                _p_dbl, _p_dbl, _p_dbl]),
    "bf_test_tc_withhold_loads": (_c_int, [_c_int]),
    "bf_test_force_fused_variant": (_c_int, [_c_int]),
    "bf_autotune": (_c_int, [_c_int]),
    "bf_autotune_report": (_c_int, [ctypes.c_char_p, _c_int]),
    "bf_transformer_group": (_c_int, [_vp, _c_int, ctypes.POINTER(_vp), _vp, _c_int, _p_dbl, _c_int, _c_int, _p_dbl,
                                      _p_dbl]),
}

_lib = None


def lib():
    """The loaded library (loads on first use; raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python boostfractor.jl_gb300/build.py` "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def symbols():
    return list(_SIGS)


class BFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"bf error {code}: {msg}")
        self.code = code


class SingularError(BFError):
    """An exactly singular propagation matrix or boundary system: where the
    reference's inv / \\ raise SingularException
    (src/boost_fractor_transformer.jl:247,346,356)."""


def ptr(a):
    """double* of a contiguous numpy array (None -> NULL)."""
    if a is None:
        return None
    return a.ctypes.data_as(_p_dbl)
