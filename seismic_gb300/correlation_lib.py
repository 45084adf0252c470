"""Drop-in replacement for the reference's ``correlation_lib.py``.

Same function names, arguments, array layouts and return tuples as

* Correlation_in_OMP/correlation_lib.py:31-113
  ``compute_correlation(events, shift, num_threads, chunk_size, threshold,
  n_classes_hist)`` -> (xcm_pos, xclags_pos, xcm_neg, xclags_neg, max_hist,
  min_hist), via the C symbol ``correlationCPP``;
* Correlation_in_CUDA/correlation_lib.py:31-106
  ``compute_correlation_cuda(events, shift, num_threads, threshold)`` ->
  (xcm_pos, xclags_pos, xcm_neg, xclags_neg) and ``initialiseRunTime()``,
  via ``correlationCUDA`` / ``initialiseCUDA``.

``events`` may be what the reference expects (an object array of traces with a
``.data`` attribute) or a plain (N, L) array.  As in the reference, L is the
length of the FIRST event (correlation_lib.py:43-51), the padded size is
``1 << L.bit_length()`` (:54) and every event is zero-padded to it; the
reversed copy the reference builds (:65-66) is still passed through the ABI
but the library does not need it.  Outputs are the packed upper triangle of
N(N+1)/2 entries.  Unlike the reference, a library that fails to load raises
instead of calling ``sys.exit(1)`` (:26-28).
"""
from __future__ import annotations

import numpy as np

from . import _lib


def initialize_library():
    """Load libseismic_gb300.so (reference: correlation_lib.py:17-29)."""
    return _lib.lib()


initialise_library = initialize_library


def _event_data(ev):
    return ev.data if hasattr(ev, "data") else ev


def _pad(events):
    n_events = events.shape[0] if hasattr(events, "shape") else len(events)
    length = int(np.asarray(_event_data(events[0])).shape[0])
    max_pad = 1 << length.bit_length()
    padded = np.zeros((n_events, max_pad), dtype=np.float32)
    padded_rev = np.zeros((n_events, max_pad), dtype=np.float32)
    for i in range(n_events):
        d = np.asarray(_event_data(events[i]), dtype=np.float32)
        if d.shape[0] > max_pad:
            raise ValueError(f"event {i} has {d.shape[0]} samples, more than the padded size {max_pad}")
        padded[i, :d.shape[0]] = d
        padded_rev[i, :d.shape[0]] = d[::-1]
    return n_events, length, max_pad, padded, padded_rev


def compute_correlation(events, shift, num_threads, chunk_size, threshold, n_classes_hist):
    """OMP-signature entry point (Correlation_in_OMP/correlation_lib.py:31)."""
    library = initialize_library()
    max_hist = np.zeros(n_classes_hist, dtype=np.int32)
    min_hist = np.zeros(n_classes_hist, dtype=np.int32)
    n_events, length, max_pad, padded, padded_rev = _pad(events)
    n_elements = n_events * (n_events + 1) // 2
    xcm_pos = np.zeros(n_elements, dtype=np.float32)
    xclags_pos = np.zeros(n_elements, dtype=np.int32)
    xcm_neg = np.zeros(n_elements, dtype=np.float32)
    xclags_neg = np.zeros(n_elements, dtype=np.int32)
    fp, ip = _lib.c_float_p, _lib.c_int_p
    library.correlationCPP(padded.ctypes.data_as(fp), padded_rev.ctypes.data_as(fp), n_events, length,
                           shift, max_pad, num_threads, chunk_size, float(threshold), n_classes_hist,
                           xcm_pos.ctypes.data_as(fp), xclags_pos.ctypes.data_as(ip),
                           xcm_neg.ctypes.data_as(fp), xclags_neg.ctypes.data_as(ip),
                           max_hist.ctypes.data_as(ip), min_hist.ctypes.data_as(ip))
    _lib.check(library.seismic_last_error())
    return xcm_pos, xclags_pos, xcm_neg, xclags_neg, max_hist, min_hist


def compute_correlation_cuda(events, shift, num_threads, threshold):
    """CUDA-signature entry point (Correlation_in_CUDA/correlation_lib.py:31)."""
    library = initialize_library()
    n_events, length, max_pad, padded, padded_rev = _pad(events)
    n_elements = n_events * (n_events + 1) // 2
    xcm_pos = np.zeros(n_elements, dtype=np.float32)
    xclags_pos = np.zeros(n_elements, dtype=np.int32)
    xcm_neg = np.zeros(n_elements, dtype=np.float32)
    xclags_neg = np.zeros(n_elements, dtype=np.int32)
    fp, ip = _lib.c_float_p, _lib.c_int_p
    library.correlationCUDA(padded.ctypes.data_as(fp), padded_rev.ctypes.data_as(fp), n_events, length,
                            shift, max_pad, num_threads, float(threshold), xcm_pos.ctypes.data_as(fp),
                            xclags_pos.ctypes.data_as(ip), xcm_neg.ctypes.data_as(fp),
                            xclags_neg.ctypes.data_as(ip))
    _lib.check(library.seismic_last_error())
    return xcm_pos, xclags_pos, xcm_neg, xclags_neg


def initialiseRunTime():
    """Reference: Correlation_in_CUDA/correlation_lib.py:101-106."""
    library = initialize_library()
    library.initialiseCUDA()
    _lib.check(library.seismic_last_error())
