"""Serving loop over a device-resident catalog (ctypes layer over
seismic_server_* of include/seismic_gb300.h).

    srv = Server(catalog, shift=256, form="fp16", n_slots=4, topk=16)
    t = srv.submit(query_events, subset=(0, 50000))   # returns at once; events of
                                                      # any length up to the catalog's
    res = srv.wait(t)                                 # results + latency

Forms: "fp32" / "fp16" (catalog spectra, any lag window), "laggemm" /
"laggemm16" (catalog 16-bit sample planes and tensor-core lag sums, lag
windows up to +-256; "laggemm16" is the fastest of them).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib


def _declare(lib):
    if getattr(lib, "_server_declared", False):
        return lib
    vp = ctypes.c_void_p
    ll = ctypes.c_longlong
    lib.seismic_server_create.restype = ctypes.c_int
    lib.seismic_server_create.argtypes = [vp, ll, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(vp)]
    lib.seismic_server_submit.restype = ctypes.c_int
    lib.seismic_server_submit.argtypes = [vp, vp, ctypes.c_int, ll, ll, vp, vp, vp, vp, vp, vp,
                                          ctypes.POINTER(ll)]
    lib.seismic_server_submit_len.restype = ctypes.c_int
    lib.seismic_server_submit_len.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ll, ll, vp, vp, vp, vp, vp, vp,
                                              ctypes.POINTER(ll)]
    lib.seismic_server_wait.restype = ctypes.c_int
    lib.seismic_server_wait.argtypes = [vp, ll, ctypes.POINTER(ctypes.c_double)]
    lib.seismic_server_stats.restype = ctypes.c_int
    lib.seismic_server_stats.argtypes = [vp, ctypes.POINTER(ll), ctypes.POINTER(ll), ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_int)]
    lib.seismic_server_destroy.restype = ctypes.c_int
    lib.seismic_server_destroy.argtypes = [vp]
    lib._server_declared = True
    return lib


@dataclass
class Result:
    vals_pos: np.ndarray   # [n_query][subset]
    lags_pos: np.ndarray
    vals_neg: np.ndarray
    lags_neg: np.ndarray
    topk_vals: np.ndarray  # [n_query][topk]
    topk_index: np.ndarray
    latency_ms: float


class Server:
    def __init__(self, catalog: np.ndarray, shift: int, threshold: float = 0.0, form: str = "fp16",
                 n_slots: int = 4, hbm_budget_bytes: int = 0, max_query_events: int = 64, topk: int = 16):
        self.lib = _declare(_lib.lib())
        cat = np.ascontiguousarray(catalog, dtype=np.float32)
        if cat.ndim == 2:
            cat = cat[:, None, :]
        self.n_catalog, self.n_channels, self.event_length = cat.shape
        self.topk = topk
        h = ctypes.c_void_p()
        _lib.check(self.lib.seismic_server_create(cat.ctypes.data, self.n_catalog, self.n_channels,
                                                  self.event_length, shift, float(threshold), _lib.FORMS[form],
                                                  n_slots, hbm_budget_bytes, max_query_events, topk,
                                                  ctypes.byref(h)))
        self.handle = h
        self._live = {}

    def submit(self, query: np.ndarray, subset=None) -> int:
        """query: (n, C, Lq) or (n, Lq) float32 with Lq <= the catalog's event
        length (shorter events are zero-padded on the device)."""
        import torch
        q = np.ascontiguousarray(query, dtype=np.float32)
        if q.ndim == 2:
            q = q[:, None, :]
        nq, ql = q.shape[0], q.shape[-1]
        b, e = subset if subset is not None else (0, self.n_catalog)
        m = nq * (e - b)
        # pinned host buffers keep the device->host copies asynchronous
        qh = torch.from_numpy(q).pin_memory()
        outs = [torch.empty(m, dtype=torch.float32, pin_memory=True), torch.empty(m, dtype=torch.int32, pin_memory=True),
                torch.empty(m, dtype=torch.float32, pin_memory=True), torch.empty(m, dtype=torch.int32, pin_memory=True),
                torch.empty(max(1, nq * self.topk), dtype=torch.float32, pin_memory=True),
                torch.empty(max(1, nq * self.topk), dtype=torch.int64, pin_memory=True)]
        t = ctypes.c_longlong()
        _lib.check(self.lib.seismic_server_submit_len(self.handle, qh.data_ptr(), nq, ql, b, e,
                                                      *(o.data_ptr() for o in outs), ctypes.byref(t)))
        self._live[t.value] = (qh, outs, nq, e - b)
        return t.value

    def wait(self, ticket: int) -> Result:
        lat = ctypes.c_double()
        _lib.check(self.lib.seismic_server_wait(self.handle, ticket, ctypes.byref(lat)))
        qh, outs, nq, ns = self._live.pop(ticket)
        v = [o.numpy() for o in outs]
        return Result(v[0].reshape(nq, ns), v[1].reshape(nq, ns), v[2].reshape(nq, ns), v[3].reshape(nq, ns),
                      v[4][:nq * self.topk].reshape(nq, self.topk), v[5][:nq * self.topk].reshape(nq, self.topk),
                      float(lat.value))

    def stats(self) -> dict:
        c, p = ctypes.c_longlong(), ctypes.c_longlong()
        f, q = ctypes.c_int(), ctypes.c_int()
        _lib.check(self.lib.seismic_server_stats(self.handle, ctypes.byref(c), ctypes.byref(p), ctypes.byref(f),
                                                 ctypes.byref(q)))
        return {"completed": c.value, "pairs": p.value, "in_flight": f.value, "pending": q.value}

    def close(self):
        if self.handle:
            self.lib.seismic_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # pragma: no cover
            pass
