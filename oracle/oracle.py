"""TEST INFRASTRUCTURE ONLY: CPU oracles for the all-pairs normalised
cross-correlation of Correlation_in_OMP/correlation_c.cpp.

Three oracles live here:

* ``port_correlation_cpp`` -- ctypes call into ``liboracle_port.so``
  (``xcorr_port.c``), a plain-C restatement of the reference's OpenMP path in
  its own float operation order, using the FFTW-API shim.  It takes exactly
  the arguments of the reference's ``correlationCPP``
  (Correlation_in_OMP/correlation_c.cpp:210-213).
* ``ref_correlation_cpp`` -- the same call into the reference's own source
  compiled against the same shim (``oracle/_ref``), available only where the
  reference tree exists.  It pins the port (they must agree bit for bit).
* ``fp64_xcorr`` -- an FP64 numpy restatement of the maths, used to state the
  max/mean coefficient error of every GPU form and the lag-agreement
  exemptions (top-two peaks closer than 1e-6).

Nothing here is shipped or used by the product path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle_port.so")
REF_SO = os.path.join(HERE, "_ref", "libcorrelation_omp_ref.so")

_c_float_p = ctypes.POINTER(ctypes.c_float)
_c_int_p = ctypes.POINTER(ctypes.c_int)
_ARGTYPES_CPP = [_c_float_p, _c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                 ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int, _c_float_p, _c_int_p,
                 _c_float_p, _c_int_p, _c_int_p, _c_int_p]

_libs: dict = {}


def build_port() -> str:
    """Compile the C restatement (make -C oracle port); returns the .so path."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def ref_root() -> str | None:
    """The reference source tree this recipe compiles: $SEISMIC_REF_ROOT, else
    the read-only checkout at /root/reference; None where neither holds
    Correlation_in_OMP/correlation_c.cpp (the GPU machine has no reference tree)."""
    for cand in (os.environ.get("SEISMIC_REF_ROOT"), "/root/reference"):
        if cand and os.path.exists(os.path.join(cand, "Correlation_in_OMP", "correlation_c.cpp")):
            return cand
    return None


def build_ref(root: str | None = None) -> str | None:
    """Compile the reference's own OMP source against the shim, if present."""
    root = root or ref_root()
    if root is None:
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={root}"], check=True)
    return REF_SO


def _load(path: str, symbol: str):
    if path in _libs:
        return _libs[path]
    lib = ctypes.CDLL(path)
    fn = getattr(lib, symbol)
    fn.restype = None
    fn.argtypes = _ARGTYPES_CPP
    _libs[path] = lib
    return lib


def port_lib():
    if not os.path.exists(PORT_SO):
        build_port()
    return _load(PORT_SO, "port_correlationCPP")


def ref_lib():
    if not os.path.exists(REF_SO):
        if build_ref() is None:
            return None
    return _load(REF_SO, "correlationCPP")


def pad_events(events: np.ndarray, padded: int | None = None):
    """Zero-pad (N, L) float32 events to (N, P) and build the reversed copy,
    as the reference wrapper does (Correlation_in_OMP/correlation_lib.py:54-66).
    P defaults to the reference rule 1 << L.bit_length()."""
    events = np.asarray(events, dtype=np.float32)
    n, length = events.shape
    p = padded if padded is not None else (1 << int(length).bit_length())
    fwd = np.zeros((n, p), np.float32)
    rev = np.zeros((n, p), np.float32)
    fwd[:, :length] = events
    rev[:, :length] = events[:, ::-1]
    return fwd, rev, p


@dataclass
class PairOutputs:
    vals_pos: np.ndarray
    lags_pos: np.ndarray
    vals_neg: np.ndarray
    lags_neg: np.ndarray
    max_hist: np.ndarray | None = None
    min_hist: np.ndarray | None = None


def _call_cpp(fn, events, shift, threshold, n_classes_hist, num_threads, chunk_size, padded):
    fwd, rev, p = pad_events(events, padded)
    n, length = np.asarray(events).shape
    m = n * (n + 1) // 2
    out = PairOutputs(np.zeros(m, np.float32), np.zeros(m, np.int32), np.zeros(m, np.float32),
                      np.zeros(m, np.int32), np.zeros(n_classes_hist, np.int32),
                      np.zeros(n_classes_hist, np.int32))
    fn(fwd.ctypes.data_as(_c_float_p), rev.ctypes.data_as(_c_float_p), n, length, shift, p,
       num_threads, chunk_size, ctypes.c_float(threshold), n_classes_hist,
       out.vals_pos.ctypes.data_as(_c_float_p), out.lags_pos.ctypes.data_as(_c_int_p),
       out.vals_neg.ctypes.data_as(_c_float_p), out.lags_neg.ctypes.data_as(_c_int_p),
       out.max_hist.ctypes.data_as(_c_int_p), out.min_hist.ctypes.data_as(_c_int_p))
    return out


def port_correlation_cpp(events, shift, threshold=0.0, n_classes_hist=20, num_threads=0,
                         chunk_size=4, padded=None) -> PairOutputs:
    """The C restatement on (N, L) events; outputs are the packed triangle."""
    return _call_cpp(port_lib().port_correlationCPP, events, shift, threshold, n_classes_hist,
                     num_threads, chunk_size, padded)


def ref_correlation_cpp(events, shift, threshold=0.0, n_classes_hist=20, num_threads=0,
                        chunk_size=4, padded=None) -> PairOutputs | None:
    """The reference's own source (built against the shim), if available."""
    lib = ref_lib()
    if lib is None:
        return None
    return _call_cpp(lib.correlationCPP, events, shift, threshold, n_classes_hist,
                     num_threads if num_threads > 0 else os.cpu_count(), chunk_size, padded)


def port_threads() -> int:
    lib = port_lib()
    lib.port_threads_available.restype = ctypes.c_int
    return int(lib.port_threads_available())


# ---------------------------------------------------------------------------
# FP64 oracle
# ---------------------------------------------------------------------------

def triu_pairs(n: int):
    """(i, j) of the packed upper triangle incl. the diagonal, in packed order
    index(i, j) = i*N - i(i-1)/2 + (j-i) (Correlation_in_OMP/correlation_c.cpp:269)."""
    i, j = np.triu_indices(n)
    return i.astype(np.int64), j.astype(np.int64)


def packed_index(i, j, n):
    i = np.asarray(i, np.int64)
    j = np.asarray(j, np.int64)
    return i * n - i * (i - 1) // 2 + (j - i)


@dataclass
class Fp64Result:
    val_pos: np.ndarray   # un-thresholded max coefficient (0 if no positive value)
    lag_pos: np.ndarray
    val_neg: np.ndarray
    lag_neg: np.ndarray
    gap_pos: np.ndarray   # top-1 minus top-2 (different lags) of the positive scan
    gap_neg: np.ndarray


def fp64_xcorr(events, shift: int, pairs_i, pairs_j, padded: int | None = None,
               chunk: int = 4096) -> Fp64Result:
    """FP64 restatement of the pair reduction.

    events: (N, L) or (N, C, L).  For C > 1 the series is the mean over channels
    of the per-channel normalised series (the reference has no channel axis).
    The series is the circular correlation of size P (reference rule when
    ``padded`` is None), read at lags d = 1-shift .. shift in increasing order
    (Correlation_in_OMP/correlation_c.cpp:102-111); the reported value is the
    first strict maximum above 0 (minimum below 0) and its lag, else 0 / 0.
    A zero-norm channel contributes nothing.
    """
    ev = np.asarray(events, dtype=np.float64)
    if ev.ndim == 2:
        ev = ev[:, None, :]
    n, c, length = ev.shape
    p = padded if padded is not None else (1 << int(length).bit_length())
    spec = np.fft.rfft(ev, n=p, axis=-1)                       # (N, C, F)
    norms = np.sqrt(np.sum(ev * ev, axis=-1))                  # (N, C)
    inv = np.where(norms > 0, 1.0 / np.where(norms > 0, norms, 1.0), 0.0)
    lags = np.arange(1 - shift, shift + 1, dtype=np.int64)
    idx = np.mod(lags, p)
    pi = np.asarray(pairs_i, np.int64)
    pj = np.asarray(pairs_j, np.int64)
    m = pi.size
    res = Fp64Result(np.zeros(m), np.zeros(m, np.int64), np.zeros(m), np.zeros(m, np.int64),
                     np.zeros(m), np.zeros(m))
    for s in range(0, m, chunk):
        a = pi[s:s + chunk]
        b = pj[s:s + chunk]
        w = (inv[a] * inv[b])[..., None]                         # (B, C, 1)
        prod = (spec[a] * np.conj(spec[b]) * w).sum(axis=1) / c  # (B, F)
        series = np.fft.irfft(prod, n=p, axis=-1)[:, idx]        # (B, W), normalised
        amax = np.argmax(series, axis=1)
        vmax = series[np.arange(series.shape[0]), amax]
        amin = np.argmin(series, axis=1)
        vmin = series[np.arange(series.shape[0]), amin]
        top2 = np.partition(series, -2, axis=1)[:, -2:]
        bot2 = np.partition(series, 1, axis=1)[:, :2]
        posmask = vmax > 0
        negmask = vmin < 0
        res.val_pos[s:s + chunk] = np.where(posmask, vmax, 0.0)
        res.lag_pos[s:s + chunk] = np.where(posmask, lags[amax], 0)
        res.val_neg[s:s + chunk] = np.where(negmask, vmin, 0.0)
        res.lag_neg[s:s + chunk] = np.where(negmask, lags[amin], 0)
        res.gap_pos[s:s + chunk] = top2[:, 1] - top2[:, 0]
        res.gap_neg[s:s + chunk] = bot2[:, 1] - bot2[:, 0]
    return res


def hist_bins(vals: np.ndarray, n_classes_hist: int, negative: bool) -> np.ndarray:
    """Histogram counting rule of Correlation_in_OMP/correlation_c.cpp:116-117,128-129,
    in float32 arithmetic, NaN counted nowhere, index clamped to the last bin."""
    v = np.asarray(vals, np.float32)
    if negative:
        v = -v
    delta = np.float32(1.0 / n_classes_hist)
    ok = ~np.isnan(v)
    v = v[ok]
    b = np.where(v >= 1.0, n_classes_hist - 1,
                 np.clip((v / delta).astype(np.int64), 0, n_classes_hist - 1))
    return np.bincount(b, minlength=n_classes_hist).astype(np.int64)


@dataclass
class Agreement:
    n: int
    max_err_pos: float
    max_err_neg: float
    mean_err: float
    lag_mismatch: int          # mismatches that are NOT exempt
    lag_exempt: int            # mismatches exempt by the top-two-peaks rule
    lag_agree_frac: float      # raw agreement over all max and min lags
    lag_agree_frac_untied: float = 1.0  # agreement where the FP64 extremum is unique (gap > 1e-9)

    def as_dict(self):
        return dict(self.__dict__)


def agreement(vals_pos, lags_pos, vals_neg, lags_neg, ref: Fp64Result, gap_tol: float = 1e-6,
              threshold: float | None = None) -> Agreement:
    """Compare an implementation's (un-thresholded unless ``threshold`` given)
    outputs with the FP64 oracle: coefficient errors and lag agreement, with
    lags exempt where the FP64 top-two peaks differ by less than ``gap_tol``."""
    vp = np.asarray(vals_pos, np.float64)
    vn = np.asarray(vals_neg, np.float64)
    rp, rn = ref.val_pos.copy(), ref.val_neg.copy()
    rlp, rln = ref.lag_pos.copy(), ref.lag_neg.copy()
    if threshold is not None:
        keep_p = rp > threshold
        keep_n = rn < -threshold
        rp = np.where(keep_p, rp, 0.0)
        rn = np.where(keep_n, rn, 0.0)
        rlp = np.where(keep_p, rlp, 0)
        rln = np.where(keep_n, rln, 0)
    ep = np.abs(vp - rp)
    en = np.abs(vn - rn)
    mis_p = np.asarray(lags_pos) != rlp
    mis_n = np.asarray(lags_neg) != rln
    ex_p = mis_p & (ref.gap_pos < gap_tol)
    ex_n = mis_n & (ref.gap_neg < gap_tol)
    n = vp.size
    bad = int((mis_p & ~ex_p).sum() + (mis_n & ~ex_n).sum())
    agree = 1.0 - (mis_p.sum() + mis_n.sum()) / max(1, 2 * n)
    untied_p = ref.gap_pos > 1e-9
    untied_n = ref.gap_neg > 1e-9
    n_untied = int(untied_p.sum() + untied_n.sum())
    agree_untied = 1.0 - ((mis_p & untied_p).sum() + (mis_n & untied_n).sum()) / max(1, n_untied)
    return Agreement(n, float(ep.max(initial=0.0)), float(en.max(initial=0.0)),
                     float(np.concatenate([ep, en]).mean()) if n else 0.0, bad,
                     int(ex_p.sum() + ex_n.sum()), float(agree), float(agree_untied))
