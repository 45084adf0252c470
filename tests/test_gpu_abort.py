"""The staged pair kernel's bounded waits and abort path, on a healthy GPU.

SEISMIC_DEVICE_WAIT_POLLS set to a few polls makes the producer's waits for
a free ring slot run out while the FFT threads are still busy (nothing is
wrong with the GPU; the limit is just too short).  The kernel must then
raise the device error flag, stop issuing, wait for the copies it already
issued, and leave without a hang or a fault.  The host sees
SEISMIC_ERR_DEVICE_TIMEOUT (from seismic_check_device_error after a device
call, from the host call itself), and the next call without the knob is
correct against the C port of the reference's CPU path.  No test here makes
a GPU fault, trap or hang.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from seismic_gb300 import _lib, synth, xcorr
from tolerances import check_pairs

pytestmark = pytest.mark.gpu

TIMEOUT = 7  # SEISMIC_ERR_DEVICE_TIMEOUT


def _events():
    # 96 events of 1024 samples, lags -127..128: padded size 2048 (staged
    # form, 14 FFT warps, a ring of a few slots, several items per CTA)
    return synth.family_catalog(96, 1, 1024, n_families=4, seed=811)[:, 0]


def _with_polls(polls, fn):
    old = os.environ.get("SEISMIC_DEVICE_WAIT_POLLS")
    os.environ["SEISMIC_DEVICE_WAIT_POLLS"] = str(polls)
    try:
        return fn()
    finally:
        if old is None:
            del os.environ["SEISMIC_DEVICE_WAIT_POLLS"]
        else:
            os.environ["SEISMIC_DEVICE_WAIT_POLLS"] = old


def test_short_wait_limit_reports_timeout_then_recovers(cuda_ok):
    import torch
    lib = cuda_ok
    ev = _events()
    assert lib.seismic_check_device_error() == 0      # nothing pending from earlier tests
    t_ev = torch.from_numpy(ev).cuda()
    # device entry point: the call itself is asynchronous and returns OK;
    # the check call sees the flag and clears it
    _with_polls(2, lambda: xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10))
    torch.cuda.synchronize()
    assert lib.seismic_check_device_error() == TIMEOUT
    assert lib.seismic_check_device_error() == 0      # cleared
    # host entry point: reads the flag itself
    with pytest.raises(_lib.SeismicError) as exc:
        _with_polls(2, lambda: xcorr.xcorr(ev, 128, threshold=0.0, n_classes_hist=10))
    assert exc.value.status == TIMEOUT
    assert lib.seismic_check_device_error() == 0
    # the same process, no knob: correct against the C port
    got = xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10)
    torch.cuda.synchronize()
    assert lib.seismic_check_device_error() == 0
    exp = O.port_correlation_cpp(ev, 128, 0.0, 10, padded=2048)
    i, j = O.triu_pairs(ev.shape[0])
    r = O.fp64_xcorr(ev, 128, i, j, padded=2048)
    check_pairs((got.vals_pos.cpu().numpy(), got.lags_pos.cpu().numpy(), got.vals_neg.cpu().numpy(),
                 got.lags_neg.cpu().numpy()), (exp.vals_pos, exp.lags_pos, exp.vals_neg, exp.lags_neg), r, 0.0,
                label="after abort")


def test_generous_wait_limit_changes_nothing(cuda_ok):
    """A limit that never runs out on a healthy GPU: bit-identical to the default."""
    import torch
    lib = cuda_ok
    t_ev = torch.from_numpy(_events()).cuda()
    a = xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10)
    b = _with_polls(1 << 26, lambda: xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10))
    torch.cuda.synchronize()
    assert lib.seismic_check_device_error() == 0
    for x, y in zip((a.vals_pos, a.lags_pos, a.vals_neg, a.lags_neg), (b.vals_pos, b.lags_pos, b.vals_neg,
                                                                        b.lags_neg)):
        np.testing.assert_array_equal(x.cpu().numpy(), y.cpu().numpy())


@pytest.mark.parametrize("form", ["laggemm16", "laggemm"])
def test_lag_gemm_short_wait_limit_reports_timeout_then_recovers(cuda_ok, form):
    """The tensor-core lag-GEMM's roles (TMA, MMA, strip builders, epilogue)
    leave their loops together after a wait runs out, wait for their copies
    and MMAs, free TMEM and return; the next call is correct."""
    import torch
    lib = cuda_ok
    ev = _events()
    t_ev = torch.from_numpy(ev).cuda()
    assert lib.seismic_check_device_error() == 0
    _with_polls(2, lambda: xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10, form=form))
    torch.cuda.synchronize()
    assert lib.seismic_check_device_error() == TIMEOUT
    got = xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10, form=form)
    torch.cuda.synchronize()
    assert lib.seismic_check_device_error() == 0
    i, j = O.triu_pairs(ev.shape[0])
    r = O.fp64_xcorr(ev, 128, i, j, padded=2048)
    err = max(np.abs(got.vals_pos.cpu().numpy() - r.val_pos).max(),
              np.abs(got.vals_neg.cpu().numpy() - r.val_neg).max())
    assert err < (2e-3 if form == "laggemm16" else 1e-4), err
