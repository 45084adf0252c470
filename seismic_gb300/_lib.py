"""ctypes binding of libseismic_gb300.so (the C ABI in include/seismic_gb300.h).

The library is loaded from this package directory (built in-tree by
``seismic_gb300.build``).  There is no fallback: if the shared library is
missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("SEISMIC_GB300_LIB", os.path.join(PKG, "libseismic_gb300.so"))
HEADER = os.path.join(os.path.dirname(PKG), "include", "seismic_gb300.h")

c_float_p = ctypes.POINTER(ctypes.c_float)
c_int_p = ctypes.POINTER(ctypes.c_int)
c_ll = ctypes.c_longlong

SEISMIC_OK = 0
FORMS = {"fp32": 0, "fp16": 1, "laggemm": 2, "bf16": 3, "laggemm16": 4}

_lib = None


class SeismicError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"seismic_gb300 status {status}: {message}")
        self.status = status


def _declare(lib):
    vp = ctypes.c_void_p
    sig = {
        "correlationCPP": (None, [c_float_p, c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                  ctypes.c_int, c_float_p, c_int_p, c_float_p, c_int_p, c_int_p,
                                  c_int_p]),
        "correlationCUDA": (None, [c_float_p, c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_float, c_float_p, c_int_p,
                                   c_float_p, c_int_p]),
        "initialiseCUDA": (None, []),
        "seismic_last_error": (ctypes.c_int, []),
        "seismic_last_error_message": (ctypes.c_char_p, []),
        "seismic_status_string": (ctypes.c_char_p, [ctypes.c_int]),
        "seismic_resolve_padded_size": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
        "seismic_xcorr_workspace_bytes": (ctypes.c_size_t, [c_ll, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                            ctypes.c_int, ctypes.c_int]),
        "seismic_check_device_error": (ctypes.c_int, []),
        "seismic_fft_plan": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            c_int_p, c_int_p, c_int_p]),
        "seismic_xcorr_device": (ctypes.c_int, [vp, c_ll, ctypes.c_int, ctypes.c_int, c_ll, c_ll,
                                                ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, vp,
                                                vp, ctypes.c_size_t, vp]),
        "seismic_xcorr_device_stages": (ctypes.c_int, [vp, c_ll, ctypes.c_int, ctypes.c_int, c_ll, c_ll,
                                                       ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                       ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, vp,
                                                       vp, ctypes.c_size_t, vp, ctypes.c_int]),
        "seismic_xcorr_host": (ctypes.c_int, [vp, c_ll, ctypes.c_int, ctypes.c_int, c_ll, c_ll,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                              ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, vp]),
        "seismic_spectra_device": (ctypes.c_int, [vp, c_ll, ctypes.c_int, ctypes.c_int, c_ll, c_ll,
                                                  ctypes.c_int, ctypes.c_int, vp, vp, vp]),
        "seismic_pairs_device": (ctypes.c_int, [vp, vp, c_ll, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                                                vp, vp, vp, vp, vp, vp, vp]),
        "seismic_pairs_device_range": (ctypes.c_int, [vp, vp, c_ll, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                      ctypes.c_int, ctypes.c_float, ctypes.c_int, c_ll, c_ll,
                                                      vp, vp, vp, vp, vp, vp, vp]),
        "seismic_pair_couples": (c_ll, [c_ll, ctypes.c_int, ctypes.c_int]),
        "seismic_xcorr_device_noalloc": (ctypes.c_int, [vp, c_ll, ctypes.c_int, ctypes.c_int, c_ll, c_ll,
                                                        ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                        ctypes.c_int, vp, vp, vp, vp, vp, vp, vp]),
        "seismic_noalloc_scratch_bytes": (ctypes.c_size_t, []),
        "seismic_compact_workspace_bytes": (ctypes.c_size_t, [c_ll]),
        "seismic_compact_pairs_device": (ctypes.c_int, [vp, vp, vp, vp, c_ll, ctypes.c_float, c_ll,
                                                        vp, vp, vp, vp, vp, vp, vp, vp, ctypes.c_size_t, vp]),
        "seismic_histogram_device": (ctypes.c_int, [vp, vp, c_ll, ctypes.c_int, vp, vp, vp]),
        "seismic_launch_count": (ctypes.c_ulonglong, []),
        "seismic_release_cached_memory": (ctypes.c_int, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def lib():
    """The loaded library (raises if it is not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SeismicError(-1, f"{LIB_PATH} is not built; run python -m seismic_gb300.build")
        _lib = _declare(ctypes.CDLL(LIB_PATH))
    return _lib


def check(status: int) -> None:
    if status != SEISMIC_OK:
        msg = lib().seismic_last_error_message().decode(errors="replace")
        raise SeismicError(status, msg)


def header_symbols(path: str = HEADER) -> list[str]:
    """Function names declared in the public header."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b([A-Za-z_]\w*)\s*\(", text, flags=re.M)
    return [n for n in names if n not in ("defined",)]
