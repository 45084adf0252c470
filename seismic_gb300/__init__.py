"""seismic_gb300: all-pairs normalised cross-correlation of seismic event
waveforms on one GB300 GPU (sm_103a), behind the reference's ctypes ABI.

Modules:
  correlation_lib -- drop-in for the reference's correlation_lib.py
  xcorr           -- native multichannel API (host or CUDA-tensor inputs)
  synth           -- seeded synthetic catalogs
  build           -- in-tree nvcc build of libseismic_gb300.so
"""
from ._lib import SeismicError, lib  # noqa: F401
