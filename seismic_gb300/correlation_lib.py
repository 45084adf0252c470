"""Drop-in replacement for the reference's OpenMP ``correlation_lib.py``.

Same function names, arguments, array layouts and return tuple as
Correlation_in_OMP/correlation_lib.py:31-113:
``compute_correlation(events, shift, num_threads, chunk_size, threshold,
n_classes_hist)`` -> (xcm_pos, xclags_pos, xcm_neg, xclags_neg, max_hist,
min_hist), through the C symbol ``correlationCPP``.  The reference's CUDA
wrapper (same module name, other signature) is ``seismic_gb300.cuda.
correlation_lib``; ``compute_correlation_cuda`` here is the same function.

``events`` may be what the reference expects (an object array of traces with a
``.data`` attribute) or a plain (N, L) array.  As in the reference, L is the
length of the FIRST event (correlation_lib.py:43-51), the padded size is
``1 << L.bit_length()`` (:54) and every event is zero-padded to it.  The
reversed copy the reference builds (:65-66) is not built: the padded array is
passed for both pointers, and the library reads only the first.  Outputs are
the packed upper triangle of N(N+1)/2 entries.  Unlike the reference, a
library that fails to load raises instead of calling ``sys.exit(1)``
(:26-28).  The module also imports as the top-level ``correlation_lib``
with this directory on ``sys.path``.
"""
from __future__ import annotations

import os
import sys

import numpy as np

try:
    from . import _dropin, _lib
except ImportError:  # imported as the top-level module ``correlation_lib``
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from seismic_gb300 import _dropin, _lib


def initialize_library():
    """Load libseismic_gb300.so (reference: correlation_lib.py:17-29)."""
    return _lib.lib()


initialise_library = initialize_library


def compute_correlation(events, shift, num_threads, chunk_size, threshold, n_classes_hist):
    """OMP-signature entry point (Correlation_in_OMP/correlation_lib.py:31)."""
    library = initialize_library()
    max_hist = np.zeros(n_classes_hist, dtype=np.int32)
    min_hist = np.zeros(n_classes_hist, dtype=np.int32)
    n_events, length, max_pad, padded = _dropin.pad_events(events)
    n_elements = n_events * (n_events + 1) // 2
    xcm_pos = np.zeros(n_elements, dtype=np.float32)
    xclags_pos = np.zeros(n_elements, dtype=np.int32)
    xcm_neg = np.zeros(n_elements, dtype=np.float32)
    xclags_neg = np.zeros(n_elements, dtype=np.int32)
    fp, ip = _lib.c_float_p, _lib.c_int_p
    ev = padded.ctypes.data_as(fp)
    library.correlationCPP(ev, ev, n_events, length, shift, max_pad, num_threads, chunk_size, float(threshold),
                           n_classes_hist, xcm_pos.ctypes.data_as(fp), xclags_pos.ctypes.data_as(ip),
                           xcm_neg.ctypes.data_as(fp), xclags_neg.ctypes.data_as(ip),
                           max_hist.ctypes.data_as(ip), min_hist.ctypes.data_as(ip))
    _lib.check(library.seismic_last_error())
    return xcm_pos, xclags_pos, xcm_neg, xclags_neg, max_hist, min_hist


def compute_correlation_cuda(events, shift, num_threads, threshold):
    """CUDA-signature entry point (Correlation_in_CUDA/correlation_lib.py:31); the
    same function as ``seismic_gb300.cuda.correlation_lib.compute_correlation``."""
    from seismic_gb300.cuda import correlation_lib as cuda_lib
    return cuda_lib.compute_correlation(events, shift, num_threads, threshold)


def initialiseRunTime():  # noqa: N802 (the reference's name)
    """Reference: Correlation_in_CUDA/correlation_lib.py:101-106."""
    library = initialize_library()
    library.initialiseCUDA()
    _lib.check(library.seismic_last_error())
