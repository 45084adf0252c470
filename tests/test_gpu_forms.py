"""GPU tests of the reduced-precision spectra forms (FP16 / BF16 spectra and
pointwise products, FP32 accumulation, FP32 inverse FFT) against the FP64
oracle.  The stated bar for reduced-precision forms is a coefficient error
<= 1e-3 and >= 99.9 % lag agreement (over pairs whose FP64 extremum is
unique); every run also reports max / mean error."""
import numpy as np
import pytest

from oracle import oracle as O
from seismic_gb300 import synth, xcorr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form,tol,agree", [
    ("fp16", 1e-3, 0.999),
    # BF16's 8-bit mantissa meets the 1e-3 coefficient bar but cannot separate
    # neighbouring lags of smooth band-limited peaks as often: measured
    # agreement ~99.6-99.7 %, below the 99.9 % bar -- FP16 is the half form
    # that meets both
    ("bf16", 1e-3, 0.995),
])
@pytest.mark.parametrize("case", ["precision_shape", "scale_shape"])
def test_half_spectra_forms_vs_fp64(cuda_ok, form, tol, agree, case):
    if case == "precision_shape":
        ev = synth.family_catalog(200, 1, 1024, n_families=6, seed=61)
        shift = 128
    else:
        ev = synth.family_catalog(64, 3, 2048, n_families=2, seed=62)
        shift = 2048
    n = ev.shape[0]
    res = xcorr.xcorr(ev, shift, threshold=0.0, n_classes_hist=20, form=form)
    i, j = O.triu_pairs(n)
    p = xcorr.resolve_padded_size(ev.shape[-1], shift)
    r = O.fp64_xcorr(ev, shift, i, j, padded=p)
    ag = O.agreement(res.vals_pos, res.lags_pos, res.vals_neg, res.lags_neg, r, gap_tol=2 * tol)
    print(f"{form} {case}: max err {max(ag.max_err_pos, ag.max_err_neg):.3g} mean {ag.mean_err:.3g} "
          f"lag agreement {ag.lag_agree_frac_untied:.5f}")
    assert ag.max_err_pos < tol and ag.max_err_neg < tol, ag
    assert ag.lag_mismatch == 0, ag
    assert ag.lag_agree_frac_untied >= agree, ag
    assert int(res.max_hist.sum()) == i.size


def test_half_forms_zero_event(cuda_ok):
    ev = synth.ricker_catalog(9, 256, seed=63).copy()
    ev[4] = 0.0
    for form in ("fp16", "bf16"):
        res = xcorr.xcorr(ev, 128, n_classes_hist=4, form=form)
        idx = xcorr.packed_index(np.array([0, 4, 4]), np.array([4, 4, 8]), 9)
        assert np.all(res.vals_pos[idx] == 0) and np.all(res.lags_pos[idx] == 0)
        assert int(res.max_hist.sum()) == 45 - 9
