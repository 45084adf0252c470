"""GPU tests of the tensor-core lag-GEMM forms (SEISMIC_FORM_LAGGEMM_BF16X3
and SEISMIC_FORM_LAGGEMM_FP16).

They compute the linear correlation over lags 1-shift .. shift directly in
the time domain (BF16 hi+lo split with three products, or one FP16 product;
FP32 accumulation), so they are compared with the FP64 oracle and with the
FP32 FFT form run at a padded size >= L + shift (where the FFT form is also
linear).  Bar for the three-product form: coefficients within 1e-4 of FP64
(the stated target is 1e-3), lags identical except where the FP64 top-two
peaks are closer than the form's own error, agreement >= 99.9 %.  The
one-product form: within 2e-3.  Lengths whose 64-sample chunk count is not a
multiple of the MMA group (4 or 2 chunks) take the kernel's tail path.
"""
import numpy as np
import pytest

from oracle import oracle as O
from seismic_gb300 import synth, xcorr

pytestmark = pytest.mark.gpu

COEF_TOL = 1e-4


def _check(ev, shift, thr=0.0, nh=20):
    n = ev.shape[0]
    res = xcorr.xcorr(ev, shift, threshold=thr, n_classes_hist=nh, form="laggemm")
    i, j = O.triu_pairs(n)
    p = xcorr.resolve_padded_size(ev.shape[-1], shift)
    r = O.fp64_xcorr(ev, shift, i, j, padded=p)
    ag = O.agreement(res.vals_pos, res.lags_pos, res.vals_neg, res.lags_neg, r,
                     gap_tol=2 * COEF_TOL, threshold=thr)
    assert ag.max_err_pos < COEF_TOL and ag.max_err_neg < COEF_TOL, ag
    near_thr = int((np.abs(r.val_pos - thr) < COEF_TOL).sum() + (np.abs(r.val_neg + thr) < COEF_TOL).sum())
    assert ag.lag_mismatch <= near_thr, ag
    # exact FP64 ties (e.g. the +-d symmetric minima of an autocorrelation)
    # may resolve either way at reduced precision; agreement is stated
    # over pairs whose FP64 extremum is unique
    assert ag.lag_agree_frac_untied >= 0.999, ag
    fft = xcorr.xcorr(ev, shift, threshold=thr, n_classes_hist=nh, padded_size=p)
    assert np.abs(res.vals_pos - fft.vals_pos).max() < COEF_TOL
    assert np.abs(res.vals_neg - fft.vals_neg).max() < COEF_TOL
    if nh:
        assert int(res.max_hist.sum()) == i.size and int(res.min_hist.sum()) == i.size
        assert np.abs(res.max_hist.astype(int) - fft.max_hist).sum() <= 2 * near_thr + 2 * max(
            1, int(0.001 * i.size))
    return ag


def test_laggemm_precision_shape_small(cuda_ok):
    """L=1024, +-128 lags (the precision workload's shape), N across 3 event blocks."""
    ev = synth.family_catalog(300, 1, 1024, n_families=8, seed=51)
    _check(ev, 128)


def test_laggemm_ragged(cuda_ok):
    """N < one 128-event block, L not a multiple of 64, 2*shift not a multiple of 16."""
    ev = synth.ricker_catalog(37, 300, seed=52)
    _check(ev, 50, thr=0.2, nh=7)


def test_laggemm_two_ntiles_per_event(cuda_ok):
    """2*shift = 512: two N-tiles of 256 lags, one event j per pass."""
    ev = synth.family_catalog(140, 1, 1024, n_families=4, seed=53)
    _check(ev, 256)


def test_laggemm_multichannel(cuda_ok):
    """3 channels (mean of per-channel normalised series), 2*shift = 400."""
    ev = synth.family_catalog(150, 3, 512, n_families=4, seed=54)
    _check(ev, 200, thr=0.1, nh=10)


def test_laggemm_zero_event_and_device_api(cuda_ok):
    import torch
    ev = synth.family_catalog(130, 1, 256, n_families=2, seed=55).copy()
    ev[5] = 0.0
    t = torch.from_numpy(ev).cuda()
    res = xcorr.xcorr(t, 64, threshold=0.0, n_classes_hist=5, form="laggemm")
    torch.cuda.synchronize()
    n = ev.shape[0]
    vp = res.vals_pos.cpu().numpy()
    lp = res.lags_pos.cpu().numpy()
    rows = xcorr.packed_index(np.minimum(5, np.arange(n)), np.maximum(5, np.arange(n)), n)
    assert np.all(vp[rows] == 0) and np.all(lp[rows] == 0)
    assert int(res.max_hist.sum()) == n * (n + 1) // 2 - n
    from seismic_gb300 import _lib
    assert _lib.lib().seismic_check_device_error() == 0


def test_laggemm_rejects_long_windows(cuda_ok):
    from seismic_gb300 import _lib
    ev = synth.ricker_catalog(4, 1024, seed=56)
    with pytest.raises(_lib.SeismicError):
        xcorr.xcorr(ev, 300, form="laggemm")


@pytest.mark.parametrize("n,c,length,shift", [(300, 1, 1024, 128), (140, 3, 512, 256),
                                              (37, 1, 300, 50), (150, 3, 600, 200)])
def test_laggemm_fp16_one_product(cuda_ok, n, c, length, shift):
    """SEISMIC_FORM_LAGGEMM_FP16: one FP16 product per lag sum.  Bar for this
    form: coefficients within 2e-3 of FP64, lags identical where the FP64 top
    two peaks are further apart than twice that, histogram totals exact."""
    tol = 2e-3
    ev = synth.family_catalog(n, c, length, n_families=8, seed=n + c)
    res = xcorr.xcorr(ev, shift, threshold=0.0, n_classes_hist=16, form="laggemm16")
    i, j = O.triu_pairs(n)
    r = O.fp64_xcorr(ev, shift, i, j, padded=xcorr.resolve_padded_size(length, shift))
    ag = O.agreement(res.vals_pos, res.lags_pos, res.vals_neg, res.lags_neg, r, gap_tol=2 * tol)
    assert ag.max_err_pos < tol and ag.max_err_neg < tol, ag
    assert ag.lag_mismatch == 0, ag
    assert int(res.max_hist.sum()) == i.size and int(res.min_hist.sum()) == i.size


@pytest.mark.parametrize("form,tol", [("laggemm16", 2e-3), ("laggemm", 1e-4)])
@pytest.mark.parametrize("amplitude", [3e5, 1e-6, 1e-25, 1e25])
def test_laggemm_amplitude_range(cuda_ok, form, tol, amplitude):
    """One-channel catalogs far outside FP16's range (max 65504, normal floor
    6.1e-5) and near the ends of FP32's: the FP16 planes hold samples scaled
    by 1/norm, the BF16 planes keep FP32's exponent range, and the norms are
    exact float-pair sums of power-of-two-scaled samples, so the result is the
    same as at unit amplitude."""
    n, length, shift = 96, 512, 64
    ev = synth.family_catalog(n, 1, length, n_families=6, seed=7).astype(np.float32)
    ev = (ev / np.abs(ev).max() * amplitude).astype(np.float32)
    res = xcorr.xcorr(ev, shift, threshold=0.0, n_classes_hist=16, form=form)
    i, j = O.triu_pairs(n)
    r = O.fp64_xcorr(ev, shift, i, j, padded=xcorr.resolve_padded_size(length, shift))
    assert np.all(np.isfinite(res.vals_pos)) and np.all(np.isfinite(res.vals_neg))
    ag = O.agreement(res.vals_pos, res.lags_pos, res.vals_neg, res.lags_neg, r, gap_tol=2 * tol)
    assert ag.max_err_pos < tol and ag.max_err_neg < tol, ag
    assert ag.lag_mismatch == 0, ag


@pytest.mark.parametrize("form", ["laggemm", "laggemm16"])
def test_laggemm_host_chunks_match_device_call(cuda_ok, form):
    """The host entry point runs the lag-GEMM in chunks of 128-event blocks
    (copies of one chunk overlap the next): bit-identical to one device call."""
    import torch
    ev = synth.family_catalog(1100, 1, 256, n_families=6, seed=57)
    host = xcorr.xcorr(ev, 64, threshold=0.05, n_classes_hist=12, form=form)
    dev = xcorr.xcorr(torch.from_numpy(ev).cuda(), 64, threshold=0.05, n_classes_hist=12, form=form)
    torch.cuda.synchronize()
    for f in ("vals_pos", "lags_pos", "vals_neg", "lags_neg", "max_hist", "min_hist"):
        np.testing.assert_array_equal(getattr(host, f), getattr(dev, f).cpu().numpy())


def _hist_from_outputs(vp, vn, nh):
    """The kernel's binning rule (before the threshold) applied to threshold-0
    outputs: value >= 1 -> last bin, else int(value / float32(1/nh))."""
    delta = np.float32(1.0 / nh)
    out = []
    for v in (vp.astype(np.float32), (-vn).astype(np.float32)):
        b = np.floor(v / delta).astype(np.int64)
        b = np.where(v >= 1.0, nh - 1, np.clip(b, 0, nh - 1))
        out.append(np.bincount(b, minlength=nh))
    return out


@pytest.mark.parametrize("form", ["laggemm", "laggemm16"])
def test_laggemm_large_histogram_global_atomics(cuda_ok, form):
    """More classes than the kernel's shared-memory histogram holds (1024):
    counts go to global atomics and still match the outputs bin by bin."""
    ev = synth.family_catalog(200, 1, 512, n_families=5, seed=58)
    nh = 1500
    res = xcorr.xcorr(ev, 100, threshold=0.0, n_classes_hist=nh, form=form)
    hmax, hmin = _hist_from_outputs(res.vals_pos, res.vals_neg, nh)
    np.testing.assert_array_equal(res.max_hist, hmax)
    np.testing.assert_array_equal(res.min_hist, hmin)


@pytest.mark.parametrize("form", ["laggemm", "laggemm16"])
def test_laggemm_single_event(cuda_ok, form):
    """N = 1: the one pair (0, 0) peaks at 1 at lag 0."""
    ev = synth.family_catalog(1, 1, 700, n_families=1, seed=59)
    res = xcorr.xcorr(ev, 50, threshold=0.0, n_classes_hist=4, form=form)
    assert res.vals_pos.shape == (1,)
    assert abs(res.vals_pos[0] - 1.0) < 2e-3 and res.lags_pos[0] == 0
    assert int(res.max_hist.sum()) == 1
