"""The bounded waits and the abort path of the pair kernels, on a healthy GPU.

SEISMIC_DEVICE_WAIT_PROBE makes the producer's first wait (the staged FFT
pair kernel's ring producer, the lag-GEMM's TMA warp) a wait on an mbarrier
that nothing ever completes, and SEISMIC_DEVICE_WAIT_POLLS shortens every
wait to a few polls: the probe then runs out for certain.  The kernel must
raise the device error flag, stop, wait for whatever it already issued, free
its tensor memory and return -- no hang, no fault.  The host sees
SEISMIC_ERR_DEVICE_TIMEOUT (from seismic_check_device_error after a device
call, from the host call itself), and the next call without the knobs is
correct against the C port of the reference's CPU path.  Short poll limits
alone make waits run out at whatever point the timing gives; those runs
must end cleanly too, with either status.  No test here makes a GPU fault,
trap or hang.
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
    # 96 events of 1024 samples, lags -127..128: the staged form (a ring of a
    # few slots, several items per CTA) and the lag-GEMM forms
    return synth.family_catalog(96, 1, 1024, n_families=4, seed=811)[:, 0]


def _with_env(env, fn):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update({k: str(v) for k, v in env.items()})
    try:
        return fn()
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


PROBE = {"SEISMIC_DEVICE_WAIT_POLLS": 4, "SEISMIC_DEVICE_WAIT_PROBE": 1}


def _check_fp32(got, ev):
    exp = O.port_correlation_cpp(ev, 128, 0.0, 10, padded=2048)
    i, j = O.triu_pairs(ev.shape[0])
    r = O.fp64_xcorr(ev, 128, i, j, padded=2048)
    check_pairs((got.vals_pos.cpu().numpy(), got.lags_pos.cpu().numpy(), got.vals_neg.cpu().numpy(),
                 got.lags_neg.cpu().numpy()), (exp.vals_pos, exp.lags_pos, exp.vals_neg, exp.lags_neg), r, 0.0,
                label="after abort")


@pytest.mark.parametrize("block", ["on", "off"])  # the overlap-save and the plain transform
def test_staged_probe_reports_timeout_then_recovers(cuda_ok, monkeypatch, block):
    import torch
    lib = cuda_ok
    if block == "off":
        monkeypatch.setenv("SEISMIC_BLOCK_FORM", "off")
    ev = _events()
    assert lib.seismic_check_device_error() == 0      # nothing pending from earlier tests
    t_ev = torch.from_numpy(ev).cuda()
    # device entry point: asynchronous, returns OK; the check call sees the flag and clears it
    _with_env(PROBE, lambda: xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10))
    torch.cuda.synchronize()
    assert lib.seismic_check_device_error() == TIMEOUT
    assert lib.seismic_check_device_error() == 0      # cleared
    # host entry point: reads the flag itself
    with pytest.raises(_lib.SeismicError) as exc:
        _with_env(PROBE, lambda: xcorr.xcorr(ev, 128, threshold=0.0, n_classes_hist=10))
    assert exc.value.status == TIMEOUT
    assert lib.seismic_check_device_error() == 0
    # the same process, no knobs: correct against the C port
    got = xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10)
    torch.cuda.synchronize()
    assert lib.seismic_check_device_error() == 0
    _check_fp32(got, ev)


@pytest.mark.parametrize("form", ["laggemm16", "laggemm"])
def test_lag_gemm_probe_reports_timeout_then_recovers(cuda_ok, form):
    """The tensor-core lag-GEMM's roles (TMA, MMA, strip builders, epilogue)
    leave their loops together after the TMA warp's wait runs out, wait for
    their copies and MMAs, free TMEM and return; the next call is correct."""
    import torch
    lib = cuda_ok
    ev = _events()
    t_ev = torch.from_numpy(ev).cuda()
    assert lib.seismic_check_device_error() == 0
    _with_env(PROBE, lambda: xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10, form=form))
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


@pytest.mark.parametrize("form", ["fp32", "laggemm16", "laggemm"])
def test_short_poll_limit_ends_cleanly(cuda_ok, form):
    """Two polls per wait and no probe: waits run out wherever the timing
    makes them (or nowhere).  Every such run ends, the status is OK or
    SEISMIC_ERR_DEVICE_TIMEOUT, and the next call is correct."""
    import torch
    lib = cuda_ok
    ev = _events()
    t_ev = torch.from_numpy(ev).cuda()
    statuses = set()
    for _ in range(3):
        _with_env({"SEISMIC_DEVICE_WAIT_POLLS": 2},
                  lambda: xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10, form=form))
        torch.cuda.synchronize()
        statuses.add(lib.seismic_check_device_error())
    assert statuses <= {0, TIMEOUT}, statuses
    got = xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10, form=form)
    torch.cuda.synchronize()
    assert lib.seismic_check_device_error() == 0
    if form == "fp32":
        _check_fp32(got, ev)
    print(f"{form}: statuses under two polls {sorted(statuses)}")


def test_generous_wait_limit_changes_nothing(cuda_ok):
    """A limit that never runs out on a healthy GPU: bit-identical to the default."""
    import torch
    lib = cuda_ok
    t_ev = torch.from_numpy(_events()).cuda()
    a = xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10)
    b = _with_env({"SEISMIC_DEVICE_WAIT_POLLS": 1 << 26},
                  lambda: xcorr.xcorr(t_ev, 128, threshold=0.0, n_classes_hist=10))
    torch.cuda.synchronize()
    assert lib.seismic_check_device_error() == 0
    for x, y in zip((a.vals_pos, a.lags_pos, a.vals_neg, a.lags_neg), (b.vals_pos, b.lags_pos, b.vals_neg,
                                                                        b.lags_neg)):
        np.testing.assert_array_equal(x.cpu().numpy(), y.cpu().numpy())
