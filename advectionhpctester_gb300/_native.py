"""ctypes binding of the C ABI in include/mpdata.h.

The library is loaded from the package's in-tree build
(advectionhpctester_gb300/_lib/libmpdata_gb300.so).  There is no fallback: if
the library is missing, loading raises, and every MPDATA call fails loudly.
"""
import ctypes
import os
import re

from . import build as _build

_lib = None

P = ctypes.c_void_p
I = ctypes.c_int
D = ctypes.c_double
F = ctypes.c_float


class MpdataGrid(ctypes.Structure):
    _fields_ = [("np", I), ("mp", I), ("lp", I), ("ih", I), ("ibcx", I), ("ibcy", I), ("ibcz", I)]


class MpdataProblem(ctypes.Structure):
    _fields_ = [("np", I), ("mp", I), ("lp", I), ("ibcx", I), ("ibcy", I), ("ibcz", I),
                ("gauge", I), ("velocity_group", I)]


class MpdataOpts(ctypes.Structure):
    _fields_ = [("iord", I), ("nonos", I), ("gauge", I), ("precision", I), ("predictor", I)]


# (name, argtypes, restype) for every symbol include/mpdata.h declares
SIGNATURES = {
    "mpdata_ws_create": ([ctypes.POINTER(MpdataGrid), ctypes.POINTER(MpdataOpts), ctypes.POINTER(P)], I),
    "mpdata_ws_destroy": ([P], I),
    "mpdata_step_f64": ([P] * 10, I),
    "mpdata_step_f32": ([P] * 10, I),
    "mpdata_advec_dwarf_f64": ([I] * 12 + [P] * 8 + [I, I, P], I),
    "mpdata_advec_dwarf_f32": ([I] * 12 + [P] * 8 + [I, I, P], I),
    "mpdata_release_cached": ([], I),
    "mpdata_velprd_f64": ([P] * 8 + [D] * 5 + [P] * 4, I),
    "mpdata_velprd_f32": ([P] * 8 + [F] * 5 + [P] * 4, I),
    "mpdata_velprd_adjoint_f64": ([P, P] + [D] * 5 + [P] * 7, I),
    "mpdata_velprd_adjoint_f32": ([P, P] + [F] * 5 + [P] * 7, I),
    "mpdata_rho_gauge_f64": ([P] * 20 + [D] * 5 + [I, P], I),
    "mpdata_rho_gauge_f32": ([P] * 20 + [F] * 5 + [I, P], I),
    "mpdata_rho_gauge_adjoint_f64": ([P] * 24, I),
    "mpdata_rho_gauge_adjoint_f32": ([P] * 24, I),
    "mpdata_step_adjoint_f64": ([P] * 14, I),
    "mpdata_step_adjoint_f32": ([P] * 14, I),
    "mpdata_adjoint_run_f64": ([P, I, I] + [P] * 9 + [ctypes.POINTER(D)] + [P] * 4 +
                               [ctypes.POINTER(ctypes.c_longlong), P], I),
    "mpdata_adjoint_run_f32": ([P, I, I] + [P] * 9 + [ctypes.POINTER(D)] + [P] * 4 +
                               [ctypes.POINTER(ctypes.c_longlong), P], I),
    "mpdata_ws_error": ([P, ctypes.POINTER(I)], I),
    "mpdata_ws_bound_violations": ([P, P, D, ctypes.POINTER(ctypes.c_longlong), P], I),
    "mpdata_launch_count": ([], ctypes.c_longlong),
    "mpdata_ws_profile": ([P, I], I),
    "mpdata_ws_stage_times": ([P, I, ctypes.POINTER(D), ctypes.POINTER(ctypes.c_longlong)], I),
    "mpdata_stage_name": ([I], ctypes.c_char_p),
    "mpdata_batch_create": ([I, ctypes.POINTER(MpdataProblem), I, I, I, I, ctypes.POINTER(P)], I),
    "mpdata_batch_destroy": ([P], I),
    "mpdata_batch_set": ([P, I] + [P] * 8, I),
    "mpdata_batch_step": ([P, P], I),
    "mpdata_batch_graph": ([P, I], I),
    "mpdata_batch_tune": ([P, P, ctypes.POINTER(I), ctypes.POINTER(I)], I),
    "mpdata_batch_set_shape": ([P, I, I, P], I),
    "mpdata_batch_profile": ([P, I], I),
    "mpdata_batch_stage_times": ([P, I, ctypes.POINTER(D), ctypes.POINTER(ctypes.c_longlong)], I),
    "mpdata_mass_f64": ([ctypes.POINTER(MpdataGrid), P, P, P, ctypes.POINTER(D), P], I),
    "mpdata_mass_f32": ([ctypes.POINTER(MpdataGrid), P, P, P, ctypes.POINTER(D), P], I),
    "mpdata_error_norms": ([ctypes.POINTER(MpdataGrid), P, I, P, I, ctypes.POINTER(D), P], I),
    "mpdata_compute_courants_f64": ([P] * 5 + [I] + [D] * 4 + [I] * 4 + [P], I),
    "mpdata_compute_courants_f32": ([P] * 5 + [I] + [F] * 4 + [I] * 4 + [P], I),
    "mpdata_velprd_driver_f64": ([ctypes.POINTER(I), ctypes.POINTER(I), I, ctypes.POINTER(D), ctypes.POINTER(D),
                                  I, I, I, D, D] + [P] * 10 + [I] * 8 + [D] * 4 + [P, P], I),
    "mpdata_velprd_driver_f32": ([ctypes.POINTER(I), ctypes.POINTER(I), I, ctypes.POINTER(F), ctypes.POINTER(F),
                                  I, I, I, F, F] + [P] * 10 + [I] * 8 + [F] * 4 + [P, P], I),
    "mpdata_pnet_out_chunk_f64": ([ctypes.c_char_p, ctypes.c_char_p] + [I] * 6 + [P] + [I] * 5 + [P], I),
    "mpdata_pnet_out_chunk_f32": ([ctypes.c_char_p, ctypes.c_char_p] + [I] * 6 + [P] + [I] * 5 + [P], I),
    "mpdata_pnet_in_chunk_f64": ([ctypes.c_char_p, ctypes.c_char_p, I, P] + [I] * 5 + [P], I),
    "mpdata_pnet_in_chunk_f32": ([ctypes.c_char_p, ctypes.c_char_p, I, P] + [I] * 5 + [P], I),
    "mpdata_step_noalloc_f64": ([ctypes.POINTER(MpdataGrid), ctypes.POINTER(MpdataOpts)] + [P] * 9, I),
    "mpdata_strerror": ([I], ctypes.c_char_p),
    "mpdata_version": ([], ctypes.c_char_p),
}


def header_symbols():
    """Function names declared in include/mpdata.h."""
    with open(os.path.join(_build.INCLUDE, "mpdata.h")) as fh:
        text = fh.read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_ ]+\*?\s*\b(mpdata_[a-z0-9_]+)\s*\(", text, re.M)))


def lib_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load the library (optionally building it first)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError("MPDATA CUDA library not built (%s); run "
                               "advectionhpctester_gb300.build.build() first" % path)
    lib = ctypes.CDLL(path)
    for name, (argt, rest) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argt
        fn.restype = rest
    _lib = lib
    return lib


class MpdataError(RuntimeError):
    def __init__(self, code, where=""):
        msg = load().mpdata_strerror(code).decode()
        super().__init__("%s failed: %s (code %d)" % (where or "mpdata call", msg, code))
        self.code = code


def check(code, where=""):
    if code != 0:
        raise MpdataError(code, where)
    return code
