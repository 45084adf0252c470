"""Batched form: many independent catalogs in one graph replay, plus the
autotuner.  Thin ctypes layer over seismic_batch_* / seismic_autotune of
include/seismic_gb300.h; catalogs are float32 CUDA tensors (N, C, L)."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

from . import _lib


class CCatalog(ctypes.Structure):
    _fields_ = [("events", ctypes.c_void_p), ("n_events", ctypes.c_longlong), ("n_channels", ctypes.c_int),
                ("event_length", ctypes.c_int), ("event_stride", ctypes.c_longlong),
                ("channel_stride", ctypes.c_longlong), ("shift", ctypes.c_int), ("threshold", ctypes.c_float),
                ("n_classes_hist", ctypes.c_int), ("vals_pos", ctypes.c_void_p), ("lags_pos", ctypes.c_void_p),
                ("vals_neg", ctypes.c_void_p), ("lags_neg", ctypes.c_void_p), ("max_hist", ctypes.c_void_p),
                ("min_hist", ctypes.c_void_p)]


NO_GRAPH = 1
PER_SIZE = 2  # one persistent pair launch per transform size instead of one over all sizes


def _declare(lib):
    if getattr(lib, "_batch_declared", False):
        return lib
    vp = ctypes.c_void_p
    lib.seismic_batch_create.restype = ctypes.c_int
    lib.seismic_batch_create.argtypes = [ctypes.POINTER(CCatalog), ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(vp)]
    lib.seismic_batch_run.restype = ctypes.c_int
    lib.seismic_batch_run.argtypes = [vp, vp]
    lib.seismic_batch_destroy.restype = ctypes.c_int
    lib.seismic_batch_destroy.argtypes = [vp]
    lib.seismic_batch_pairs.restype = ctypes.c_longlong
    lib.seismic_batch_pairs.argtypes = [vp]
    lib.seismic_batch_kernels_per_run.restype = ctypes.c_int
    lib.seismic_batch_kernels_per_run.argtypes = [vp]
    lib.seismic_autotune.restype = ctypes.c_int
    lib.seismic_autotune.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_char_p]
    lib.seismic_tuning.restype = ctypes.c_int
    lib.seismic_tuning.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                   ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    lib.seismic_tuning_staged.restype = ctypes.c_int
    lib.seismic_tuning_staged.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_int)]
    lib._batch_declared = True
    return lib


@dataclass
class CatalogOutputs:
    vals_pos: object
    lags_pos: object
    vals_neg: object
    lags_neg: object
    max_hist: object
    min_hist: object


class Batch:
    """Plan + outputs for a list of catalogs (float32 CUDA tensors (N, C, L)
    or (N, L)); run() replays the captured graph on a stream."""

    def __init__(self, events, shifts, thresholds=None, n_classes_hist=0, use_graph=True, per_size=False):
        import torch
        self.lib = _declare(_lib.lib())
        self.events = [e.contiguous() if e.dim() == 3 else e.contiguous()[:, None, :] for e in events]
        n = len(self.events)
        thresholds = thresholds if thresholds is not None else [0.0] * n
        self.outputs = []
        arr = (CCatalog * n)()
        for k, ev in enumerate(self.events):
            if not ev.is_cuda or ev.dtype != torch.float32:
                raise ValueError("catalog events must be float32 CUDA tensors")
            ne, c, length = ev.shape
            m = ne * (ne + 1) // 2
            dev = ev.device
            o = CatalogOutputs(torch.empty(m, device=dev), torch.empty(m, dtype=torch.int32, device=dev),
                               torch.empty(m, device=dev), torch.empty(m, dtype=torch.int32, device=dev),
                               torch.zeros(max(1, n_classes_hist), dtype=torch.int32, device=dev),
                               torch.zeros(max(1, n_classes_hist), dtype=torch.int32, device=dev))
            self.outputs.append(o)
            arr[k] = CCatalog(ev.data_ptr(), ne, c, length, c * length, length, int(shifts[k]),
                              float(thresholds[k]), n_classes_hist, o.vals_pos.data_ptr(), o.lags_pos.data_ptr(),
                              o.vals_neg.data_ptr(), o.lags_neg.data_ptr(),
                              o.max_hist.data_ptr() if n_classes_hist else None,
                              o.min_hist.data_ptr() if n_classes_hist else None)
        self._arr = arr
        h = ctypes.c_void_p()
        flags = (0 if use_graph else NO_GRAPH) | (PER_SIZE if per_size else 0)
        _lib.check(self.lib.seismic_batch_create(arr, n, flags, ctypes.byref(h)))
        self.handle = h
        self.pairs = int(self.lib.seismic_batch_pairs(h))
        self.kernels_per_run = int(self.lib.seismic_batch_kernels_per_run(h))

    def run(self, stream=None):
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        _lib.check(self.lib.seismic_batch_run(self.handle, ctypes.c_void_p(s.cuda_stream)))

    def close(self):
        if self.handle:
            self.lib.seismic_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # pragma: no cover - interpreter teardown
            pass


def autotune(padded_size: int, n_channels: int, cache_path: str | None = None) -> dict:
    lib = _declare(_lib.lib())
    _lib.check(lib.seismic_autotune(padded_size, n_channels, cache_path.encode() if cache_path else None))
    return tuning(padded_size, n_channels)


def tuning(padded_size: int, n_channels: int) -> dict:
    lib = _declare(_lib.lib())
    t, c, i = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _lib.check(lib.seismic_tuning(padded_size, n_channels, ctypes.byref(t), ctypes.byref(c), ctypes.byref(i)))
    w, r = ctypes.c_int(), ctypes.c_int()
    _lib.check(lib.seismic_tuning_staged(padded_size, n_channels, ctypes.byref(w), ctypes.byref(r)))
    return {"tile": t.value, "ctas_per_sm": c.value, "item_groups": i.value, "staged_warps": w.value,
            "staged_ru": r.value}
