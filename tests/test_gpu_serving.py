"""GPU tests of the serving loop: query x resident-catalog results against
the FP64 oracle, the top-K selection, continuous batching under a small HBM
budget, and the same result alone and in the mix of concurrent requests."""
import threading

import numpy as np
import pytest

from oracle import oracle as O
from seismic_gb300 import synth, xcorr

pytestmark = pytest.mark.gpu


def _catalog():
    return synth.family_catalog(600, 3, 512, n_families=12, seed=71)


def _fp64_block(cat, query, shift, b, e):
    ev = np.concatenate([query, cat[b:e]])
    nq = query.shape[0]
    i = np.repeat(np.arange(nq), e - b)
    j = nq + np.tile(np.arange(e - b), nq)
    return O.fp64_xcorr(ev, shift, i, j, padded=xcorr.resolve_padded_size(cat.shape[-1], shift))


@pytest.mark.parametrize("form,tol", [("fp32", 1e-5), ("fp16", 1e-3), ("laggemm", 1e-4), ("laggemm16", 2e-3)])
def test_server_results_vs_fp64(cuda_ok, form, tol):
    from seismic_gb300.serving import Server
    cat = _catalog()
    srv = Server(cat, shift=100, form=form, n_slots=3, max_query_events=16, topk=8)
    query = synth.family_catalog(5, 3, 512, n_families=2, seed=72)
    t = srv.submit(query, subset=(50, 480))
    res = srv.wait(t)
    r = _fp64_block(cat, query, 100, 50, 480)
    ag = O.agreement(res.vals_pos.ravel(), res.lags_pos.ravel(), res.vals_neg.ravel(), res.lags_neg.ravel(), r,
                     gap_tol=2 * tol)
    assert ag.max_err_pos < tol and ag.max_err_neg < tol, ag
    assert ag.lag_mismatch == 0, ag
    # top-K: the K largest max-coefficients per query, ties to the lower index
    for q in range(5):
        order = np.lexsort((np.arange(430), -res.vals_pos[q]))[:8]
        np.testing.assert_array_equal(res.topk_index[q], 50 + order)
        np.testing.assert_array_equal(res.topk_vals[q], res.vals_pos[q][order])
    assert res.latency_ms > 0
    srv.close()


def test_server_item_shapes_agree_bitwise(cuda_ok, monkeypatch):
    """Rectangle work items of TI queries x TJ catalog events: TI = 1, 2 and
    3 over a 7-event request (query blocks padded past the last query) give
    the same results bit for bit."""
    from seismic_gb300.serving import Server
    cat = _catalog()
    query = synth.family_catalog(7, 3, 512, n_families=2, seed=74)
    got = {}
    for ti in ("1", "2", "3"):
        monkeypatch.setenv("SEISMIC_STAGED_TI", ti)
        srv = Server(cat, shift=100, form="fp32", n_slots=2, max_query_events=8, topk=4)
        res = srv.wait(srv.submit(query, subset=(3, 557)))
        got[ti] = [res.vals_pos, res.lags_pos, res.vals_neg, res.lags_neg, res.topk_index]
        srv.close()
    for ti in ("2", "3"):
        for a, b in zip(got["1"], got[ti]):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("form", ["fp16", "laggemm16"])
def test_server_same_result_alone_and_in_the_mix(cuda_ok, form):
    """A request gives bit-identical results alone and when it is admitted
    while many other requests of different sizes are on the device."""
    from seismic_gb300.serving import Server
    cat = _catalog()
    srv = Server(cat, shift=128, form=form, n_slots=4, max_query_events=32, topk=16)
    probe = synth.family_catalog(7, 3, 512, n_families=2, seed=73)
    alone = srv.wait(srv.submit(probe, subset=(10, 590)))
    rng = np.random.default_rng(5)
    tickets = []
    lock = threading.Lock()

    def burst(seed):
        r = np.random.default_rng(seed)
        for _ in range(6):
            nq = int(r.integers(1, 33))
            ql = int(r.choice([200, 350, 512]))  # query events of different lengths
            b = int(r.integers(0, 300))
            e = int(r.integers(b + 1, 600))
            t = srv.submit(synth.family_catalog(nq, 3, ql, n_families=1, seed=int(r.integers(1 << 30))), (b, e))
            with lock:
                tickets.append(t)

    threads = [threading.Thread(target=burst, args=(s,)) for s in range(3)]
    for th in threads:
        th.start()
    mid = srv.submit(probe, subset=(10, 590))
    for th in threads:
        th.join()
    mixed = srv.wait(mid)
    others = [srv.wait(t) for t in tickets]
    assert len(others) == 18
    for f in ("vals_pos", "lags_pos", "vals_neg", "lags_neg", "topk_vals", "topk_index"):
        np.testing.assert_array_equal(getattr(alone, f), getattr(mixed, f))
    assert srv.stats()["completed"] == 20
    srv.close()
    del rng


@pytest.mark.parametrize("form,tol", [("fp32", 1e-5), ("laggemm16", 2e-3)])
def test_server_shorter_queries(cuda_ok, form, tol):
    """Query events shorter than the catalog's are zero-padded on the device:
    the same results as submitting them padded on the host, and within the
    form's tolerance of FP64.  Longer ones are rejected."""
    from seismic_gb300 import _lib
    from seismic_gb300.serving import Server
    cat = _catalog()
    srv = Server(cat, shift=100, form=form, n_slots=2, max_query_events=8, topk=4)
    short = synth.family_catalog(4, 3, 300, n_families=2, seed=74)
    padded = np.zeros((4, 3, cat.shape[-1]), np.float32)
    padded[..., :300] = short
    a = srv.wait(srv.submit(short, subset=(0, 256)))
    b = srv.wait(srv.submit(padded, subset=(0, 256)))
    for f in ("vals_pos", "lags_pos", "vals_neg", "lags_neg"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f))
    r = _fp64_block(cat, padded, 100, 0, 256)
    ag = O.agreement(a.vals_pos.ravel(), a.lags_pos.ravel(), a.vals_neg.ravel(), a.lags_neg.ravel(), r,
                     gap_tol=2 * tol)
    assert ag.max_err_pos < tol and ag.max_err_neg < tol, ag
    assert ag.lag_mismatch == 0, ag
    with pytest.raises(_lib.SeismicError):
        srv.submit(synth.family_catalog(1, 3, cat.shape[-1] + 1, n_families=1, seed=75))
    srv.close()


def test_server_admission_by_hbm_budget(cuda_ok):
    """With a pool that fits about one large request, requests still all
    complete (admitted as memory frees up); one larger than the pool is
    refused at submit."""
    from seismic_gb300 import _lib
    from seismic_gb300.serving import Server
    cat = _catalog()
    one = 2 * 8 * 600 * 16 + 3 * 8 * 3 * 512 * 4 * 3   # rough size of one 8-event full-catalog request, x2
    srv = Server(cat, shift=64, form="fp32", n_slots=4, hbm_budget_bytes=one, max_query_events=64, topk=4)
    ts = [srv.submit(synth.family_catalog(8, 3, 512, n_families=1, seed=80 + k)) for k in range(6)]
    for t in ts:
        srv.wait(t)
    with pytest.raises(_lib.SeismicError):
        srv.submit(synth.family_catalog(64, 3, 512, n_families=2, seed=90))
    srv.close()
