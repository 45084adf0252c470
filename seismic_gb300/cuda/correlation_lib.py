"""Drop-in replacement for the reference's CUDA ``correlation_lib.py``.

Same module name, function names, arguments and return tuple as
Correlation_in_CUDA/correlation_lib.py:

* ``compute_correlation(events, shift, num_threads, threshold)`` (:31) ->
  (xcm_pos, xclags_pos, xcm_neg, xclags_neg), the packed upper triangle of
  N(N+1)/2 entries each, through the C symbol ``correlationCUDA``;
* ``initialiseRunTime()`` (:101) -> None, through ``initialiseCUDA``;
* ``initialise_library()`` (:17) -> the loaded library.

A driver written for the reference (``from correlation_lib import
compute_correlation, initialiseRunTime``, Correlation_in_CUDA/test_cuda.py:15)
runs unchanged with this directory on ``sys.path``; inside the package it is
``seismic_gb300.cuda.correlation_lib``.  Results follow the reference's CPU
(OpenMP) semantics: every pair below the threshold is written as 0 / lag 0,
the lag window is the full [-shift, shift) and ties go to the first lag.
Unlike the reference, a library that fails to load raises instead of
calling ``sys.exit(1)`` (:26-28).
"""
from __future__ import annotations

import os
import sys

import numpy as np

try:
    from .. import _dropin, _lib
except ImportError:  # imported as the top-level module ``correlation_lib``
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    from seismic_gb300 import _dropin, _lib


def initialise_library():
    """Load libseismic_gb300.so (reference: correlation_lib.py:17-29)."""
    return _lib.lib()


def compute_correlation(events, shift, num_threads, threshold):
    """All-pairs normalised cross-correlation (reference: correlation_lib.py:31-99)."""
    library = initialise_library()
    n_events, length, max_pad, padded = _dropin.pad_events(events)
    n_elements = n_events * (n_events + 1) // 2
    xcm_pos = np.zeros(n_elements, dtype=np.float32)
    xclags_pos = np.zeros(n_elements, dtype=np.int32)
    xcm_neg = np.zeros(n_elements, dtype=np.float32)
    xclags_neg = np.zeros(n_elements, dtype=np.int32)
    fp, ip = _lib.c_float_p, _lib.c_int_p
    ev = padded.ctypes.data_as(fp)
    library.correlationCUDA(ev, ev, n_events, length, shift, max_pad, num_threads, float(threshold),
                            xcm_pos.ctypes.data_as(fp), xclags_pos.ctypes.data_as(ip),
                            xcm_neg.ctypes.data_as(fp), xclags_neg.ctypes.data_as(ip))
    _lib.check(library.seismic_last_error())
    return xcm_pos, xclags_pos, xcm_neg, xclags_neg


def initialiseRunTime():  # noqa: N802 (the reference's name)
    """Create the CUDA context and load the kernels (reference: correlation_lib.py:101-106)."""
    library = initialise_library()
    library.initialiseCUDA()
    _lib.check(library.seismic_last_error())
