"""Native Python API over the C ABI: multichannel events, host or device.

``xcorr(events, shift, ...)`` correlates every pair (i, j >= i) of the
events of one catalog and returns the packed upper-triangle outputs.

* numpy input  -> ``seismic_xcorr_host`` (copies in, runs, copies back);
* torch CUDA tensor input -> ``seismic_xcorr_device`` on torch's current
  stream, outputs are CUDA tensors (nothing leaves the device).

events are float32 shaped (N, L) or (N, C, L); with C > 1 the coefficient
series is the mean over channels of the per-channel normalised series.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class XcorrResult:
    vals_pos: object
    lags_pos: object
    vals_neg: object
    lags_neg: object
    max_hist: object = None
    min_hist: object = None


def n_pairs(n_events: int) -> int:
    return n_events * (n_events + 1) // 2


def packed_index(i, j, n_events):
    """Index of pair (i, j >= i) in the packed outputs
    (Correlation_in_OMP/correlation_c.cpp:269), in 64-bit."""
    i = np.asarray(i, np.int64)
    j = np.asarray(j, np.int64)
    return i * n_events - i * (i - 1) // 2 + (j - i)


def resolve_padded_size(event_length: int, shift: int) -> int:
    return int(_lib.lib().seismic_resolve_padded_size(int(event_length), int(shift)))


def _shape3(events):
    if events.ndim == 2:
        return events.shape[0], 1, events.shape[1]
    if events.ndim == 3:
        return events.shape
    raise ValueError("events must be (N, L) or (N, C, L)")


def xcorr(events, shift: int, threshold: float = 0.0, n_classes_hist: int = 0, padded_size: int = 0,
          form: str = "fp32", stream=None, workspace=None) -> XcorrResult:
    lib = _lib.lib()
    f = _lib.FORMS[form]
    try:
        import torch
        is_torch = isinstance(events, torch.Tensor)
    except ImportError:  # pragma: no cover
        is_torch = False
    if is_torch:
        if not events.is_cuda or events.dtype != torch.float32:
            raise ValueError("torch events must be a float32 CUDA tensor")
        ev = events.contiguous()
        n, c, length = _shape3(ev)
        m = n_pairs(n)
        dev = ev.device
        vp = torch.empty(m, dtype=torch.float32, device=dev)
        lp = torch.empty(m, dtype=torch.int32, device=dev)
        vn = torch.empty(m, dtype=torch.float32, device=dev)
        ln = torch.empty(m, dtype=torch.int32, device=dev)
        hmax = torch.zeros(max(n_classes_hist, 1), dtype=torch.int32, device=dev)
        hmin = torch.zeros(max(n_classes_hist, 1), dtype=torch.int32, device=dev)
        s = stream if stream is not None else torch.cuda.current_stream(dev)
        ws_ptr, ws_bytes = (None, 0) if workspace is None else (workspace.data_ptr(),
                                                                  workspace.numel() * workspace.element_size())
        with torch.cuda.device(dev):
            st = lib.seismic_xcorr_device(ev.data_ptr(), n, c, length, c * length, length, padded_size, shift,
                                          float(threshold), n_classes_hist, f, vp.data_ptr(), lp.data_ptr(),
                                          vn.data_ptr(), ln.data_ptr(), hmax.data_ptr(), hmin.data_ptr(),
                                          ws_ptr, ws_bytes, ctypes.c_void_p(s.cuda_stream))
        _lib.check(st)
        return XcorrResult(vp, lp, vn, ln, hmax[:n_classes_hist], hmin[:n_classes_hist])

    ev = np.ascontiguousarray(events, dtype=np.float32)
    n, c, length = _shape3(ev)
    m = n_pairs(n)
    vp = np.empty(m, np.float32)
    lp = np.empty(m, np.int32)
    vn = np.empty(m, np.float32)
    ln = np.empty(m, np.int32)
    hmax = np.zeros(max(n_classes_hist, 1), np.int32)
    hmin = np.zeros(max(n_classes_hist, 1), np.int32)
    st = lib.seismic_xcorr_host(ev.ctypes.data, n, c, length, c * length, length, padded_size, shift,
                                float(threshold), n_classes_hist, f, vp.ctypes.data, lp.ctypes.data,
                                vn.ctypes.data, ln.ctypes.data, hmax.ctypes.data, hmin.ctypes.data)
    _lib.check(st)
    return XcorrResult(vp, lp, vn, ln, hmax[:n_classes_hist], hmin[:n_classes_hist])
