"""Event padding shared by the two drop-in wrappers (correlation_lib.py for
the OpenMP signature, cuda/correlation_lib.py for the CUDA one).

The reference wrappers take L from the FIRST event
(Correlation_in_OMP/correlation_lib.py:43-51, Correlation_in_CUDA/
correlation_lib.py:40-48), pad every event with zeros to
P = 1 << L.bit_length() (:54 / :51) and build a time-reversed copy as well
(:65-66 / :61-62).  The library forms the reversed spectra by conjugation,
so no reversed copy is built here: the padded array is passed for both
pointers of the C ABI, which reads only the first one.
"""
from __future__ import annotations

import numpy as np


def event_data(ev):
    """A trace's samples: ``ev.data`` for obspy-style objects, else ``ev``."""
    return ev.data if hasattr(ev, "data") else ev


def pad_events(events):
    """(n_events, L, P, padded float32 [n_events][P])."""
    arr = events if isinstance(events, np.ndarray) and events.dtype != object and events.ndim == 2 else None
    n_events = events.shape[0] if hasattr(events, "shape") else len(events)
    length = int(arr.shape[1]) if arr is not None else int(np.asarray(event_data(events[0])).shape[0])
    max_pad = 1 << length.bit_length()
    padded = np.zeros((n_events, max_pad), dtype=np.float32)
    if arr is not None:
        padded[:, :length] = arr
        return n_events, length, max_pad, padded
    for i in range(n_events):
        d = np.asarray(event_data(events[i]), dtype=np.float32)
        if d.shape[0] > max_pad:
            raise ValueError(f"event {i} has {d.shape[0]} samples, more than the padded size {max_pad}")
        padded[i, :d.shape[0]] = d
    return n_events, length, max_pad, padded
