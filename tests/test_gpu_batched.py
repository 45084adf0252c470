"""GPU tests of the batched form (many catalogs, one persistent pair launch
over every transform size or one per size, captured CUDA graph) and of the
autotuner.  Each catalog of a batch must give exactly what the
single-catalog FP32 path gives with the same plain size-P transform (the
batched form never takes the overlap-save form), on every replay, with and
without the graph."""
import os

import numpy as np
import pytest

from seismic_gb300 import synth, xcorr

pytestmark = pytest.mark.gpu


def _catalogs():
    rng = np.random.default_rng(7)
    specs = [(17, 1, 256), (120, 3, 512), (1, 1, 1000), (64, 1, 2048), (33, 3, 3000), (5, 1, 4096),
             (200, 1, 256), (90, 3, 1000), (2, 1, 512), (150, 1, 1000), (40, 3, 2048), (9, 3, 256)]
    out = []
    for k, (n, c, length) in enumerate(specs):
        ev = synth.family_catalog(n, c, length, n_families=max(1, n // 32), seed=500 + k)
        shift = length if k % 3 else int(rng.integers(8, length // 2))   # mostly the full lag range
        out.append((ev, shift))
    return out


@pytest.mark.parametrize("use_graph,per_size", [(True, False), (False, False), (True, True)])
def test_batch_matches_single_catalog_path(cuda_ok, monkeypatch, use_graph, per_size):
    import torch
    from seismic_gb300.batch import Batch
    monkeypatch.setenv("SEISMIC_BLOCK_FORM", "off")  # the single-catalog path's plain transform
    cats = _catalogs()
    tens = [torch.from_numpy(ev).cuda() for ev, _ in cats]
    b = Batch(tens, [s for _, s in cats], thresholds=[0.05] * len(cats), n_classes_hist=9, use_graph=use_graph,
              per_size=per_size)
    assert b.pairs == sum(ev.shape[0] * (ev.shape[0] + 1) // 2 for ev, _ in cats)
    assert b.kernels_per_run == (1 + 5 if per_size else 2)  # sizes 512 .. 8192 present, or one mixed launch
    for rep in range(2):  # replay twice: same results (histograms accumulate)
        b.run()
        torch.cuda.synchronize()
        for k, (ev, shift) in enumerate(cats):
            single = xcorr.xcorr(tens[k], shift, threshold=0.05, n_classes_hist=9)
            o = b.outputs[k]
            for got, exp in ((o.vals_pos, single.vals_pos), (o.lags_pos, single.lags_pos),
                             (o.vals_neg, single.vals_neg), (o.lags_neg, single.lags_neg)):
                assert torch.equal(got, exp), f"catalog {k} replay {rep}"
            np.testing.assert_array_equal(o.max_hist.cpu().numpy(), (rep + 1) * single.max_hist.cpu().numpy())
            np.testing.assert_array_equal(o.min_hist.cpu().numpy(), (rep + 1) * single.min_hist.cpu().numpy())
    b.close()


def test_autotuner_writes_cache_and_is_used(cuda_ok, tmp_path):
    from seismic_gb300 import batch
    path = os.path.join(tmp_path, "tune.txt")
    t = batch.autotune(1024, 1, path)
    assert t["tile"] in (2, 4, 8, 16) and t["ctas_per_sm"] >= 1 and t["item_groups"] in (4, 16, 64)
    assert t["staged_warps"] in (12, 99) and t["staged_ru"] in (2, 4)   # the staged form's CTA shape
    line = open(path).read()
    assert f"P=1024 C=1 tile={t['tile']}" in line and f"warps={t['staged_warps']} ru={t['staged_ru']}" in line
    assert batch.tuning(1024, 1) == t
    # results do not depend on the tuned parameters
    ev = synth.ricker_catalog(70, 512, seed=9)
    r = xcorr.xcorr(ev, 512, n_classes_hist=5)
    from oracle import oracle as O
    exp = O.port_correlation_cpp(ev[:, 0], 512, 0.0, 5)
    assert np.abs(r.vals_pos - exp.vals_pos).max() < 1e-5
