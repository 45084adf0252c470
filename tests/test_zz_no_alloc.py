"""The allocation-free entry point, seismic_xcorr_device_noalloc.

It serves callers that may not allocate device memory themselves through
this library (a framework that owns the whole GPU memory pool, a fixed
device-memory quota, a loop where an allocation's synchronisation is not
acceptable).  The test calls it through the C ABI twice in a row, on two
different catalogs so that whatever the shared scratch array kept from the
first call must not leak into the second, and checks every output against
the regular seismic_xcorr_device entry point with the parity tolerance of
the other tests (1e-5 on coefficients, identical lags and histograms).  It
also checks that a catalog too large for the fixed scratch is refused with
a clear error before anything runs.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from seismic_gb300 import synth

pytestmark = pytest.mark.gpu

COEF_TOL = 1e-5


def _run(lib, fn_name, t_ev, shift, thr, nh, stream):
    import torch
    n, c, length = t_ev.shape
    m = n * (n + 1) // 2
    # sentinels no pair can produce: NaN coefficients, INT_MIN lags
    out = [torch.full((m,), float("nan"), device="cuda"), torch.full((m,), -2**31, dtype=torch.int32, device="cuda"),
           torch.full((m,), float("nan"), device="cuda"), torch.full((m,), -2**31, dtype=torch.int32, device="cuda")]
    hist = torch.zeros(2, nh, dtype=torch.int32, device="cuda")
    args = [t_ev.data_ptr(), n, c, length, c * length, length, 0, shift, ctypes.c_float(thr), nh]
    if fn_name == "seismic_xcorr_device":
        st = lib.seismic_xcorr_device(*args, 0, *(o.data_ptr() for o in out), hist[0].data_ptr(),
                                      hist[1].data_ptr(), None, 0, ctypes.c_void_p(stream.cuda_stream))
    else:
        st = lib.seismic_xcorr_device_noalloc(*args, *(o.data_ptr() for o in out), hist[0].data_ptr(),
                                              hist[1].data_ptr(), ctypes.c_void_p(stream.cuda_stream))
    assert st == 0, lib.seismic_last_error_message()
    stream.synchronize()
    return [o.cpu().numpy() for o in out], hist.cpu().numpy()


def test_noalloc_matches_regular_entry_point_twice(cuda_ok):
    import torch
    lib = cuda_ok
    stream = torch.cuda.Stream()
    cases = [
        (synth.family_catalog(96, 3, 1000, n_families=4, seed=301), 1000, 0.1, 12),
        (synth.ricker_catalog(150, 512, seed=302), 512, 0.0, 20),
        # padded size 256: the direct-load pair form, whose row bands are
        # planned inside the launch, through the same fixed scratch
        (synth.family_catalog(70, 1, 200, n_families=3, seed=303), 50, 0.0, 10),
    ]
    for ev, shift, thr, nh in cases:
        t_ev = torch.from_numpy(ev).cuda()
        got, got_h = _run(lib, "seismic_xcorr_device_noalloc", t_ev, shift, thr, nh, stream)
        exp, exp_h = _run(lib, "seismic_xcorr_device", t_ev, shift, thr, nh, stream)
        assert np.abs(got[0] - exp[0]).max() <= COEF_TOL
        assert np.abs(got[2] - exp[2]).max() <= COEF_TOL
        np.testing.assert_array_equal(got[1], exp[1])
        np.testing.assert_array_equal(got[3], exp[3])
        np.testing.assert_array_equal(got_h, exp_h)
        assert not np.isnan(got[0]).any() and not np.isnan(got[2]).any()  # every pair written
        assert not np.any(got[1] == -2**31) and not np.any(got[3] == -2**31)


def test_noalloc_accepts_catalog_filling_the_scratch_exactly(cuda_ok):
    """One channel at padded size 4096: 16 KiB of spectra + 16 B of FP64 norm
    and inverse norm per event, each part rounded up to 256 B.  4092 events
    need 4092*16384 + 65536 bytes = exactly 64 MiB: accepted, same results
    as the regular entry point, and the check call reports no timeout."""
    import torch
    lib = cuda_ok
    cap = lib.seismic_noalloc_scratch_bytes()
    n = 4092
    assert n * 16384 + ((16 * n + 255) // 256) * 256 == cap
    ev = synth.family_catalog(n, 1, 2048, n_families=16, seed=304)
    t_ev = torch.from_numpy(ev).cuda()
    stream = torch.cuda.Stream()
    got, got_h = _run(lib, "seismic_xcorr_device_noalloc", t_ev, 2048, 0.0, 20, stream)
    assert lib.seismic_check_device_error() == 0
    exp, exp_h = _run(lib, "seismic_xcorr_device", t_ev, 2048, 0.0, 20, stream)
    assert np.abs(got[0] - exp[0]).max() <= COEF_TOL
    assert np.abs(got[2] - exp[2]).max() <= COEF_TOL
    np.testing.assert_array_equal(got[1], exp[1])
    np.testing.assert_array_equal(got[3], exp[3])
    np.testing.assert_array_equal(got_h, exp_h)


def test_noalloc_rejects_catalog_beyond_scratch(cuda_ok):
    import torch
    lib = cuda_ok
    cap = lib.seismic_noalloc_scratch_bytes()
    assert cap == 64 << 20
    n = 4093                            # one event more than fills the scratch exactly
    m = n * (n + 1) // 2
    ev = torch.zeros(n, 2048, device="cuda")       # real buffers of the full size
    outs = [torch.zeros(m, device="cuda"), torch.zeros(m, dtype=torch.int32, device="cuda"),
            torch.zeros(m, device="cuda"), torch.zeros(m, dtype=torch.int32, device="cuda")]
    st = lib.seismic_xcorr_device_noalloc(ev.data_ptr(), n, 1, 2048, 2048, 2048, 4096, 2048,
                                          ctypes.c_float(0.0), 0, *(o.data_ptr() for o in outs), None, None,
                                          None)
    assert st == 6  # SEISMIC_ERR_WORKSPACE_TOO_SMALL, refused before any launch
    assert b"scratch" in lib.seismic_last_error_message()
