"""CPU tests of the measurement code in bench.py: the algorithmic work
figures the roofline is computed from, the FP64 error statistics, the
workload descriptions, the traffic file and the CPU-baseline arm on a tiny
sample (no GPU)."""
import importlib.util
import os

import numpy as np
import pytest

from oracle import oracle as O
from seismic_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_fft_flops_per_pair_is_the_stated_count(bench):
    # 2.5 P log2 P (one size-P inverse FFT) + 6 C (P/2 + 1) (conj-products)
    assert bench.fft_flops_per_pair(4096, 3) == pytest.approx(2.5 * 4096 * 12 + 6 * 3 * 2049)
    assert bench.fft_flops_per_pair(2048, 1) == pytest.approx(2.5 * 2048 * 11 + 6 * 1025)


def test_linear_padding_rule(bench):
    # the FP64 check pads to a power of two >= L + shift (linear correlation)
    assert bench.xcorr_padded(1024, 128) == 2048
    assert bench.xcorr_padded(2048, 2048) == 4096
    assert bench.xcorr_padded(100, 28) == 128


def test_workload_text_names_the_form(bench):
    t = bench.workload_text("precision", "laggemm16")
    assert "lag-GEMM" in t and "padded FFT" not in t and "FP16" in t
    t = bench.workload_text("scale", "fp32")
    assert t.endswith("FP32 fused FFT form") and "padded FFT 4096" in t
    assert "FP16-spectra" in bench.workload_text("scale", "fp16")
    assert bench.FORM_DTYPE["laggemm16"] == "f16"


def test_traffic_file_entries(bench):
    for w in ("scale", "precision", "precision/laggemm", "precision/laggemm16"):
        v = bench.read_traffic(w)
        assert v is not None and 10.0 < v < 200.0, (w, v)
    assert bench.read_traffic("no-such-workload") is None


def test_fp64_sample_error_is_zero_on_exact_outputs(bench):
    """Outputs taken from the FP64 oracle itself give zero error and full
    agreement up to exempt ties; a planted lag error on a well-separated peak
    is counted."""
    ev = synth.family_catalog(30, 1, 256, n_families=3, seed=11)
    shift, p = 64, bench.xcorr_padded(256, 64)
    n = ev.shape[0]
    i, j = O.triu_pairs(n)
    r = O.fp64_xcorr(ev, shift, i, j, padded=p)
    vp, lp = r.val_pos.astype(np.float32), r.lag_pos.astype(np.int32)
    vn, ln = r.val_neg.astype(np.float32), r.lag_neg.astype(np.int32)
    e = bench.fp64_sample_error(ev, shift, p, vp, lp, vn, ln, n_sample=200, seed=1)
    # two FP64 evaluations may order exact or 1e-12 ties differently: those are
    # exempt (top-two gap < 1e-6), every other lag agrees
    assert e["max_abs"] < 1e-6 and e["lag_mismatch_not_exempt"] == 0 and e["lag_agreement"] >= 0.99
    # plant a wrong lag on the pair with the clearest positive peak
    k = int(np.argmax(r.gap_pos))
    lp_bad = lp.copy()
    lp_bad[k] += 1
    rng = np.random.default_rng(1)
    ii = rng.integers(0, n, 5000)
    jj = rng.integers(0, n, 5000)
    e2 = bench.fp64_sample_error(ev, shift, p, vp, lp_bad, vn, ln, n_sample=5000, seed=1)
    sampled = np.minimum(ii, jj) * n - np.minimum(ii, jj) * (np.minimum(ii, jj) - 1) // 2 + (
        np.maximum(ii, jj) - np.minimum(ii, jj))
    if k in set(sampled.tolist()):
        assert e2["lag_mismatch_not_exempt"] >= 1


def test_cpu_baseline_arm_on_a_tiny_sample(bench):
    ev = synth.family_catalog(24, 2, 128, n_families=2, seed=12)
    base, times = bench.cpu_baseline("small", ev, 64, n_sample=24)
    assert base["unit"] == "pairs/s" and base["value"] > 0
    assert base["kind"] in ("port", "reference") and base["cores"] >= 1
    assert "24 events" in base["sample"] and len(times) == 1
