"""ctypes binding of libsoapgb (include/soapgb.h).

The library is the product's only compute path: importing this module fails loudly
when ``soap_gpu_gb300/lib/libsoapgb.so`` is missing or does not load (build it with
``python -m soap_gpu_gb300.build`` or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libsoapgb.so")
BIN_DIR = os.path.join(_HERE, "bin")

OK, ERR_ARG, ERR_CUDA, ERR_ALLOC, ERR_NUMERIC, ERR_DEVICE = 0, 1, 2, 3, 4, 5
HOST, DEVICE = 0, 1
PLAIN64, FAST64, FAST32 = 0, 1, 2
FORMS = {"plain64": PLAIN64, "fast64": FAST64, "fast32": FAST32}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p


class Star(ctypes.Structure):
    _fields_ = [("grid", ctypes.c_int), ("period", ctypes.c_double), ("omega_ratio", ctypes.c_double),
                ("incl", ctypes.c_double), ("radius_km", ctypes.c_double), ("u1", ctypes.c_double),
                ("u2", ctypes.c_double), ("lb", ctypes.c_double * 4)]


class Maps(ctypes.Structure):
    _fields_ = [("delta", _vp), ("limb", _vp), ("mu", _vp), ("region", _vp), ("lb", _vp)]


class Cubes(ctypes.Structure):
    _fields_ = [("q_norm", _vp), ("q_sed", _vp), ("spot_norm", _vp), ("fac_norm", _vp), ("spot_sed", _vp),
                ("fac_sed", _vp), ("n_mu", ctypes.c_int)]


class Activity(ctypes.Structure):
    _fields_ = [("t_star", ctypes.c_int), ("t_diff_spot", ctypes.c_int), ("t_diff_fac", ctypes.c_int),
                ("nrho", ctypes.c_int), ("solar", ctypes.c_int)]


class BatchDesc(ctypes.Structure):
    _fields_ = [("form", ctypes.c_int), ("n", ctypes.c_int), ("n_eff", ctypes.c_int), ("wave", _vp),
                ("cubes", ctypes.POINTER(Cubes)), ("mu_boundary", _vp), ("step", ctypes.c_double),
                ("act", Activity), ("sigma_v", ctypes.c_double), ("conv_step", ctypes.c_double),
                ("sentinel", ctypes.c_double), ("n_star", ctypes.c_int), ("stars", ctypes.POINTER(Star)),
                ("phase_offsets", _vp), ("phases", _vp), ("reg_offsets", _vp), ("regions", _vp),
                ("chunk", ctypes.c_int), ("blocks_per_sm", ctypes.c_int)]


# (name, restype, argtypes) for every entry point declared in include/soapgb.h
SIGNATURES = [
    ("soapgb_ctx_create", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_vp)]),
    ("soapgb_ctx_destroy", ctypes.c_int, [_vp]),
    ("soapgb_last_error", ctypes.c_char_p, [_vp]),
    ("soapgb_set_stream", ctypes.c_int, [_vp, _vp]),
    ("soapgb_synchronize", ctypes.c_int, [_vp]),
    ("soapgb_launch_count", ctypes.c_longlong, [_vp]),
    ("soapgb_set_compensated", ctypes.c_int, [_vp, ctypes.c_int]),
    ("soapgb_version", ctypes.c_char_p, []),
    ("soapgb_trace_enable", ctypes.c_int, [_vp, ctypes.c_int]),
    ("soapgb_trace_report", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_size_t]),
    ("soapgb_disk_maps", ctypes.c_int, [_vp, ctypes.POINTER(Star), ctypes.c_int, _vp, ctypes.c_int,
                                        ctypes.POINTER(Maps)]),
    ("soapgb_quiet_disk", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.c_int,
                                         ctypes.c_int, _vp, _vp, _vp, ctypes.c_double, ctypes.c_int, _vp]),
    ("soapgb_lower_resolution", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp,
                                               _vp, _vp] + [ctypes.c_double] * 5 + [ctypes.c_int, _vp, _vp]),
    ("soapgb_lower_resolution_adjoint", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]
     + [ctypes.c_double] * 5 + [_vp, ctypes.c_int, _vp, _vp]),
    ("soapgb_phase_maps", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, _vp, _vp, _vp,
                                         ctypes.POINTER(Activity), ctypes.c_int, _vp, _vp]),
    ("soapgb_phase_integrate", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_int,
                                              ctypes.c_int, _vp, _vp, ctypes.POINTER(Maps), ctypes.POINTER(Cubes),
                                              ctypes.c_double, ctypes.POINTER(Activity), ctypes.c_int, _vp, _vp,
                                              _vp]),
    ("soapgb_phase_integrate_adjoint", ctypes.c_int,
     [_vp, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.POINTER(Maps),
      ctypes.POINTER(Cubes), ctypes.c_double, ctypes.POINTER(Activity), _vp, _vp, _vp, ctypes.c_int, _vp, _vp, _vp,
      _vp, _vp, _vp, _vp, _vp]),
    ("soapgb_ccf", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_int, _vp, _vp, ctypes.c_int, _vp,
                                  ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                  _vp, ctypes.c_int, ctypes.c_int, _vp]),
    ("soapgb_ccf_adjoint", ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int, _vp, _vp, ctypes.c_int, _vp,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_int, _vp, ctypes.c_int, _vp, ctypes.c_int, _vp]),
    ("soapgb_gauss_fit_adjoint", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp,
                                                ctypes.c_int, _vp]),
    ("soapgb_gauss_bis", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int, _vp, _vp, _vp,
                                        _vp, _vp]),
    ("soapgb_phase_pipeline", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp,
                                             ctypes.POINTER(Star), ctypes.POINTER(Maps), ctypes.POINTER(Cubes),
                                             ctypes.c_double, ctypes.POINTER(Activity), ctypes.c_int, _vp, _vp, _vp,
                                             _vp, _vp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_int, _vp, _vp]),
    ("soapgb_bisector_inject", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp,
                                              _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_double, ctypes.c_int, _vp]),
    ("soapgb_batch_create", ctypes.c_int, [_vp, ctypes.POINTER(BatchDesc), ctypes.POINTER(_vp)]),
    ("soapgb_batch_run", ctypes.c_int, [_vp, _vp, _vp, _vp]),
    ("soapgb_batch_tune", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    ("soapgb_batch_device_bytes", ctypes.c_size_t, [_vp]),
    ("soapgb_batch_items", ctypes.c_longlong, [_vp]),
    ("soapgb_batch_destroy", ctypes.c_int, [_vp]),
    ("soapgb_noalloc_capacity", ctypes.c_size_t, [ctypes.c_int]),
    ("soapgb_lower_resolution_noalloc", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]
     + [ctypes.c_double] * 5 + [_vp, _vp]),
]

_lib = None


class SoapError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libsoapgb error %d: %s" % (code, msg))
        self.code = code


def load():
    """Load libsoapgb.so (raises if absent: there is no fallback path)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libsoapgb.so not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib
