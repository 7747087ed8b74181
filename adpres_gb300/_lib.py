"""ctypes binding of the C ABI declared in include/adpres_gb300.h.

The library is loaded from the package directory.  There is no fallback: if
the library is missing or cannot be loaded, import of the solver fails with
the reason, because the CUDA path is the product.
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
# ADPRES_LIB selects another build of the library (the variants of
# adpres_gb300/build.py); by default the in-tree one.
LIB_PATH = os.environ.get("ADPRES_LIB") or os.path.join(PKG, "libadpres_gb300.so")

ADP_OK = 0
ADP_ERR_INPUT = 1
ADP_ERR_BADXS = 2
ADP_ERR_PIVOT = 3
ADP_ERR_DIVERGED = 4
ADP_ERR_MAXOUTER = 5
ADP_ERR_ZEROPOWER = 6
ADP_ERR_UNSUPPORTED = 7
ADP_ERR_CUDA = 8
ADP_ERR_NAN = 9
ADP_ERR_BREAKDOWN = 10
ADP_ERR_TIMEOUT = 11
ADP_ERR_STATE = 12
ADP_ERR_BOUNDS = 13

STATUS_NAMES = {
    0: "ADP_OK", 1: "ADP_ERR_INPUT", 2: "ADP_ERR_BADXS", 3: "ADP_ERR_PIVOT", 4: "ADP_ERR_DIVERGED",
    5: "ADP_ERR_MAXOUTER", 6: "ADP_ERR_ZEROPOWER", 7: "ADP_ERR_UNSUPPORTED", 8: "ADP_ERR_CUDA",
    9: "ADP_ERR_NAN", 10: "ADP_ERR_BREAKDOWN", 11: "ADP_ERR_TIMEOUT", 12: "ADP_ERR_STATE", 13: "ADP_ERR_BOUNDS",
}

ADP_FORWARD, ADP_ADJOINT, ADP_FROZEN_DN = 0, 1, 4
ADP_KERN_FDM, ADP_KERN_PNM, ADP_KERN_SANM = 0, 1, 2
ADP_FP64, ADP_MIXED = 0, 1

_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)


class AdpGeom(ctypes.Structure):
    _fields_ = [("nxx", ctypes.c_int), ("nyy", ctypes.c_int), ("nzz", ctypes.c_int), ("nnod", ctypes.c_int),
                ("ix", _ip), ("iy", _ip), ("iz", _ip), ("xdel", _dp), ("ydel", _dp), ("zdel", _dp),
                ("east", ctypes.c_int), ("west", ctypes.c_int), ("north", ctypes.c_int),
                ("south", ctypes.c_int), ("bottom", ctypes.c_int), ("top", ctypes.c_int)]


class AdpOpts(ctypes.Structure):
    _fields_ = [("ng", ctypes.c_int), ("nin", ctypes.c_int), ("nout", ctypes.c_int), ("nac", ctypes.c_int),
                ("nupd", ctypes.c_int), ("serc", ctypes.c_double), ("ferc", ctypes.c_double),
                ("kern", ctypes.c_int), ("precision", ctypes.c_int)]


class AdpReport(ctypes.Structure):
    _fields_ = [("outers", ctypes.c_int), ("converged", ctypes.c_int), ("nodal_updates", ctypes.c_int),
                ("keff", ctypes.c_double), ("ser", ctypes.c_double), ("fer", ctypes.c_double),
                ("ndmax", ctypes.c_double), ("im", ctypes.c_int), ("jm", ctypes.c_int), ("km", ctypes.c_int),
                ("trace_cap", ctypes.c_int), ("trace_k", _dp), ("trace_ser", _dp), ("trace_fer", _dp),
                ("trace_flags", _ip), ("trace_ndmax", _dp), ("device_ms", ctypes.c_double)]


class AdpTimers(ctypes.Structure):
    _fields_ = [("outer_kernel_ms", ctypes.c_double), ("outer_kernel_launches", ctypes.c_long),
                ("nodal_ms", ctypes.c_double), ("nodal_updates", ctypes.c_long), ("other_ms", ctypes.c_double),
                ("outers", ctypes.c_long), ("bicg_rows", ctypes.c_long), ("grid_blocks", ctypes.c_int),
                ("block_threads", ctypes.c_int), ("adjoint_ms", ctypes.c_double), ("adjoint_outers", ctypes.c_long)]


class AdpTransOpts(ctypes.Structure):
    _fields_ = [("nf", ctypes.c_int), ("beta", ctypes.POINTER(ctypes.c_double)),
                ("lambda_", ctypes.POINTER(ctypes.c_double)), ("velo", ctypes.POINTER(ctypes.c_double)),
                ("theta", ctypes.c_double), ("extr", ctypes.c_int)]


class AdpTransResult(ctypes.Structure):
    _fields_ = [("rho", ctypes.c_double), ("rho_dollar", ctypes.c_double), ("relpow", ctypes.c_double),
                ("power", ctypes.c_double), ("maxi", ctypes.c_int), ("outers", ctypes.c_int),
                ("device_ms", ctypes.c_double)]


ADP_FB_BORON, ADP_FB_FUEL_TEMP, ADP_FB_MOD_TEMP, ADP_FB_COOL_DENS = 0, 1, 2, 3


class AdpFbTables(ctypes.Structure):
    _fields_ = [("nmat", ctypes.c_int), ("xsigtr", _dp), ("xsiga", _dp), ("xnuf", _dp), ("xsigf", _dp),
                ("xsigs", _dp), ("chi", _dp), ("mat", _ip), ("dc", _dp), ("nstate", ctypes.c_int),
                ("kind", _ip), ("ref", _dp), ("dsig", ctypes.POINTER(_dp)), ("nbank", ctypes.c_int),
                ("rsig", ctypes.POINTER(_dp)), ("bank", _ip), ("coreh", ctypes.c_double),
                ("pos0", ctypes.c_double), ("ssize", ctypes.c_double)]


class AdpBatchConfig(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int), ("max_team", ctypes.c_int), ("grain", ctypes.c_double),
                ("blocks_per_sm", ctypes.c_int), ("use_graph", ctypes.c_int)]


class AdpBatchResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("converged", ctypes.c_int), ("outers", ctypes.c_int),
                ("nodal_updates", ctypes.c_int), ("keff", ctypes.c_double), ("ser", ctypes.c_double),
                ("fer", ctypes.c_double), ("ndmax", ctypes.c_double), ("device_ms", ctypes.c_double),
                ("team", ctypes.c_int)]


# Every entry point declared in include/adpres_gb300.h, with its ctypes signature.
SIGNATURES = {
    "adp_create": (ctypes.c_int, [ctypes.POINTER(AdpGeom), ctypes.POINTER(AdpOpts), ctypes.POINTER(ctypes.c_void_p)]),
    "adp_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "adp_last_error": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    "adp_set_xs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp]),
    "adp_xs_updt": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp]),
    "adp_xs_updt_nodes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp]),
    "adp_fb_set": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AdpFbTables)]),
    "adp_fb_updt": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    "adp_fb_rod_tips": (ctypes.c_int, [ctypes.c_int, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int, _dp, _ip, _dp]),
    "adp_outer": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(AdpReport)]),
    "adp_get_state": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, _dp]),
    "adp_set_state": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, _dp]),
    "adp_power": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "adp_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "adp_power_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "adp_adjoint_sens": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, _dp, _dp, ctypes.POINTER(AdpReport)]),
    "adp_adjoint_sens_frozen": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, _dp, _dp, ctypes.POINTER(AdpReport)]),
    "adp_nodal_vjp": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]),
    "adp_set_wait_limit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "adp_get_matrix": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "adp_nodal_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AdpReport)]),
    "adp_get_nodal_sources": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "adp_test_missing_block": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "adp_get_timers": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AdpTimers)]),
    "adp_reactivity": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, ctypes.POINTER(ctypes.c_double)]),
    "adp_core_beta": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int, _dp, _ip,
                                     ctypes.POINTER(ctypes.c_double)]),
    "adp_edit_asmpow": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _ip, _ip, _dp, _ip, _ip]),
    "adp_edit_axipow": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _ip, _dp, _ip]),
    "adp_edit_asmflux": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _ip, _ip, ctypes.c_double, _dp,
                                        _ip]),
    "adp_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(AdpGeom), ctypes.POINTER(AdpOpts),
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "adp_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "adp_batch_last_error": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    "adp_batch_set_xs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _ip,
                                        _dp, _dp]),
    "adp_batch_set_config": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AdpBatchConfig)]),
    "adp_batch_get_config": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AdpBatchConfig)]),
    "adp_batch_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AdpBatchResult),
                                       ctypes.POINTER(ctypes.c_double)]),
    "adp_batch_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AdpBatchConfig),
                                          ctypes.POINTER(ctypes.c_double)]),
    "adp_batch_core": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "adp_batch_plan_preview": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, ctypes.POINTER(AdpBatchConfig),
                                              ctypes.c_int, _ip, _ip, _ip, _ip, _dp]),
    "adp_batch_power": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp]),
    "adp_batch_trace": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _ip, _dp]),
    "adp_set_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "adp_trans_init": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AdpTransOpts), _dp,
                                      ctypes.POINTER(AdpTransResult)]),
    "adp_trans_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                      ctypes.POINTER(AdpTransResult)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the in-tree CUDA library (raises if absent: there is no CPU path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the solver has no CPU fallback)")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def last_error(h=None) -> str:
    L = load()
    buf = ctypes.create_string_buffer(1024)
    L.adp_last_error(h, buf, 1024)
    return buf.value.decode(errors="replace")


class AdpError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def dptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


def iptr(a):
    return None if a is None else a.ctypes.data_as(_ip)
