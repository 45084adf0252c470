"""Generate the golden fixtures in this directory from the reference itself.

The reference ships no test vectors (its drivers need a dataset that is not
distributed), so the fixtures are produced by running the reference's own
code here:

* its unmodified OpenMP source, Correlation_in_OMP/correlation_c.cpp, compiled
  against this repository's FFTW-API shim (``make -C oracle ref``), and
* its own Python wrapper, Correlation_in_OMP/correlation_lib.py, imported from
  the reference tree with only ``initialize_library`` redirected to that build
  (the original loads a hard-coded path, correlation_lib.py:24) and the events
  wrapped as objects with a ``.data`` attribute (the wrapper expects obspy
  traces, correlation_lib.py:50,64).

Run:  python tests/golden/make_golden.py [/path/to/reference]
Each case is written as <name>.npz holding the (N, L) float32 events, the
call parameters and the wrapper's six outputs.
"""
from __future__ import annotations

import contextlib
import ctypes
import importlib.util
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O          # noqa: E402
from seismic_gb300 import synth         # noqa: E402


class _Trace:
    def __init__(self, data):
        self.data = data


def _load_reference_wrapper(ref_root: str):
    path = os.path.join(ref_root, "Correlation_in_OMP", "correlation_lib.py")
    spec = importlib.util.spec_from_file_location("reference_correlation_lib", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    so = O.build_ref(ref_root)
    lib = ctypes.CDLL(so)
    mod.initialize_library = lambda: lib
    return mod


CASES = {
    # name: (events builder, shift, num_threads, chunk_size, threshold, n_classes_hist)
    "ricker_n64_l512_full": (lambda: synth.ricker_catalog(64, 512, seed=101)[:, 0], 512, 4, 1, 0.0, 20),
    "ricker_n40_l512_s256_thr": (lambda: synth.ricker_catalog(40, 512, seed=102)[:, 0], 256, 3, 4, 0.3, 10),
    "ragged_n37_l300_s200": (lambda: synth.ricker_catalog(37, 300, seed=103)[:, 0], 200, 2, 2, 0.1, 7),
    "family_n48_l1024_s128": (lambda: synth.family_catalog(48, 1, 1024, n_families=4, seed=104)[:, 0],
                              128, 4, 16, 0.2, 20),
    "family_n20_l2048_full": (lambda: synth.family_catalog(20, 1, 2048, n_families=2, seed=105)[:, 0],
                              2048, 4, 1, 0.0, 20),
    "tiny_n1_l64": (lambda: synth.ricker_catalog(1, 64, seed=106)[:, 0], 32, 1, 1, 0.0, 4),
    "tiny_n2_l100": (lambda: synth.ricker_catalog(2, 100, seed=107)[:, 0], 28, 1, 1, 0.0, 4),
    "tiny_n3_l256_s8": (lambda: synth.ricker_catalog(3, 256, seed=108)[:, 0], 8, 1, 1, 0.05, 3),
}


def main(ref_root: str | None = None) -> None:
    ref_root = ref_root or O.ref_root()
    if ref_root is None:
        raise SystemExit("reference tree not found: set SEISMIC_REF_ROOT")
    mod = _load_reference_wrapper(ref_root)
    for name, (build, shift, nthreads, chunk, thr, nh) in CASES.items():
        events = np.ascontiguousarray(build(), dtype=np.float32)
        traces = np.empty(events.shape[0], dtype=object)
        for i in range(events.shape[0]):
            traces[i] = _Trace(events[i])
        with contextlib.redirect_stdout(io.StringIO()):
            out = mod.compute_correlation(traces, shift, nthreads, chunk, thr, nh)
        xcm_pos, xcl_pos, xcm_neg, xcl_neg, hmax, hmin = out
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"), events=events, shift=shift, num_threads=nthreads,
            chunk_size=chunk, threshold=np.float32(thr), n_classes_hist=nh,
            padded=1 << int(events.shape[1]).bit_length(), xcm_pos=xcm_pos, xclags_pos=xcl_pos,
            xcm_neg=xcm_neg, xclags_neg=xcl_neg, max_hist=hmax, min_hist=hmin)
        print(f"{name}: N={events.shape[0]} L={events.shape[1]} pairs={xcm_pos.size}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
