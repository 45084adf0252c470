"""Sparse output and standalone histograms of the packed correlation outputs.

The reference's driver thresholds inside the pair loop, then stores each
packed array as a 1 x N(N+1)/2 scipy CSR matrix of its nonzeros
(Correlation_in_OMP/test_c.py:43-55).  Here the correlation can run once with
threshold 0 on the device; `histogram` bins the stored coefficients (to pick a
threshold), `compact` keeps the pairs above it on the device
(seismic_compact_pairs_device), and `to_csr` / `save_npz` give the same
matrices and files the reference writes, with only the kept pairs crossing
PCIe.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class SparsePairs:
    """Pairs above a threshold, in packed order (CUDA tensors)."""
    n_pairs: int            # N (N + 1) / 2 of the packed arrays they came from
    index_pos: object       # int64 packed indices with vals_pos > threshold
    value_pos: object       # float32
    lag_pos: object         # int32
    index_neg: object       # int64 packed indices with vals_neg < -threshold
    value_neg: object
    lag_neg: object


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def histogram(vals_pos, vals_neg, n_classes_hist: int):
    """Max / min histograms (int32 CUDA tensors) of stored coefficients, with
    the pair kernel's binning rule, on the current stream."""
    import torch
    dev = vals_pos.device
    hmax = torch.zeros(n_classes_hist, dtype=torch.int32, device=dev)
    hmin = torch.zeros(n_classes_hist, dtype=torch.int32, device=dev)
    _lib.check(_lib.lib().seismic_histogram_device(_ptr(vals_pos), _ptr(vals_neg), vals_pos.numel(),
                                                   n_classes_hist, _ptr(hmax), _ptr(hmin), _stream()))
    return hmax, hmin


def compact(vals_pos, lags_pos, vals_neg, lags_neg, threshold: float = 0.0) -> SparsePairs:
    """Pairs with vals_pos > threshold and vals_neg < -threshold, in packed
    order, from packed CUDA tensors (one count pass, then the write pass)."""
    import torch
    lib = _lib.lib()
    dev = vals_pos.device
    n = vals_pos.numel()
    ws = torch.empty(max(16, lib.seismic_compact_workspace_bytes(n)), dtype=torch.uint8, device=dev)
    counts = torch.zeros(2, dtype=torch.int64, device=dev)
    args = [_ptr(vals_pos), _ptr(lags_pos), _ptr(vals_neg), _ptr(lags_neg), n, ctypes.c_float(threshold)]
    _lib.check(lib.seismic_compact_pairs_device(*args, 0, None, None, None, None, None, None, _ptr(counts),
                                                _ptr(ws), ws.numel(), _stream()))
    cp, cn = (int(x) for x in counts.cpu())
    cap = max(cp, cn, 1)
    out = [torch.empty(cap, dtype=torch.int64, device=dev), torch.empty(cap, dtype=torch.float32, device=dev),
           torch.empty(cap, dtype=torch.int32, device=dev), torch.empty(cap, dtype=torch.int64, device=dev),
           torch.empty(cap, dtype=torch.float32, device=dev), torch.empty(cap, dtype=torch.int32, device=dev)]
    _lib.check(lib.seismic_compact_pairs_device(*args, cap, *(_ptr(t) for t in out), _ptr(counts), _ptr(ws),
                                                ws.numel(), _stream()))
    return SparsePairs(n, out[0][:cp], out[1][:cp], out[2][:cp], out[3][:cn], out[4][:cn], out[5][:cn])


def to_csr(sp: SparsePairs) -> dict:
    """The four 1 x n_pairs CSR matrices the reference builds with
    csr_matrix(dense) (test_c.py:43-46): entries where the value (or lag) is
    nonzero."""
    from scipy.sparse import csr_matrix

    def one(index, data, dtype):
        index = index.cpu().numpy()
        data = data.cpu().numpy().astype(dtype)
        keep = data != 0
        index, data = index[keep], data[keep]
        return csr_matrix((data, index.astype(np.int64), np.array([0, index.size], dtype=np.int64)),
                          shape=(1, sp.n_pairs), dtype=dtype)

    return {"xcm_pos": one(sp.index_pos, sp.value_pos, np.float32),
            "xclags_pos": one(sp.index_pos, sp.lag_pos, np.int32),
            "xcm_neg": one(sp.index_neg, sp.value_neg, np.float32),
            "xclags_neg": one(sp.index_neg, sp.lag_neg, np.int32)}


def save_npz(directory: str, sp: SparsePairs, max_hist=None, min_hist=None) -> list[str]:
    """Writes the reference's output files (test_c.py:50-55) into `directory`."""
    from scipy.sparse import csr_matrix, save_npz as _save

    m = to_csr(sp)
    names = {"xcm_pos": "out_xcm_pos.npz", "xclags_pos": "out_xcl_pos.npz", "xcm_neg": "out_xcm_neg.npz",
             "xclags_neg": "out_xcl_neg.npz"}
    paths = []
    for k, fname in names.items():
        paths.append(os.path.join(directory, fname))
        _save(paths[-1], m[k], compressed=True)
    for h, fname in ((max_hist, "out_xmax_hist.npz"), (min_hist, "out_xmin_hist.npz")):
        if h is not None:
            h = h.cpu().numpy() if hasattr(h, "cpu") else np.asarray(h)
            paths.append(os.path.join(directory, fname))
            _save(paths[-1], csr_matrix(h, dtype=np.int32), compressed=True)
    return paths
