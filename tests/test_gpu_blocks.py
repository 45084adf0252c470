"""The overlap-save form of the FFT path for short lag windows.

For lags 1-shift .. shift much shorter than the events, the library splits
every event into nb blocks of B samples and correlates each block (A frame)
with the block widened by `shift` on both sides (W frame) at a transform
size Q < P; the block correlations sum to the linear correlation the plain
size-P form computes wherever the reference is defined (L + shift <= P,
Correlation_in_OMP/correlation_c.cpp:102-103).  These tests check the plan
the library reports, the results against the C port of the reference's CPU
path and the FP64 oracle at the parity bar, the plain form
(SEISMIC_BLOCK_FORM=off) at the same bar, and the host entry point's chunked
launches against the device entry point bit for bit.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from seismic_gb300 import _lib, synth, xcorr
from tolerances import check_hist, check_pairs

pytestmark = pytest.mark.gpu

CASES = [  # n, channels, L, shift, expected transform size
    (90, 1, 1024, 128, 512),    # the precision shape: 4 blocks of 256
    (61, 1, 2048, 100, 512),    # P = 4096 -> 7 blocks of 312
    (77, 3, 1024, 256, 1024),   # the serving shape: 2 blocks of 512, three channels
    (40, 2, 700, 30, 512),      # ragged last block, two channels
]


def _plan(lib, length, shift, c):
    q, b, bl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _lib.check(lib.seismic_fft_plan(length, shift, 0, c, 0, ctypes.byref(q), ctypes.byref(b), ctypes.byref(bl)))
    return q.value, b.value, bl.value


@pytest.mark.parametrize("n,c,length,shift,q", CASES)
def test_block_form_plan_and_parity(cuda_ok, monkeypatch, n, c, length, shift, q):
    import torch
    lib = cuda_ok
    tq, nb, bl = _plan(lib, length, shift, c)
    assert (tq, bl) == (q, q - 2 * shift) and nb == -(-length // bl), (tq, nb, bl)
    ev = synth.family_catalog(n, c, length, n_families=max(1, n // 12), seed=700 + n)
    ev[n // 2] = 0.0                                   # a zero-norm event
    t = torch.from_numpy(ev).cuda()
    thr = 0.2
    got = xcorr.xcorr(t, shift, threshold=thr, n_classes_hist=12)
    torch.cuda.synchronize()
    g = [x.cpu().numpy() for x in (got.vals_pos, got.lags_pos, got.vals_neg, got.lags_neg)]
    i, j = O.triu_pairs(n)
    p = xcorr.resolve_padded_size(length, shift)
    r = O.fp64_xcorr(ev, shift, i, j, padded=p)
    ag = O.agreement(*g, r, threshold=thr)
    # coefficients within 1e-5 of FP64 and lags identical outside the tie rule
    exp_fp64 = (np.where(r.val_pos > thr, r.val_pos, 0.0), np.where(r.val_pos > thr, r.lag_pos, 0),
                np.where(r.val_neg < -thr, r.val_neg, 0.0), np.where(r.val_neg < -thr, r.lag_neg, 0))
    check_pairs(g, exp_fp64, r, thr, label="block form vs FP64")
    if c == 1:  # the reference's own CPU path (one channel), through the C port
        exp = O.port_correlation_cpp(ev[:, 0], shift, thr, 12, padded=p)
        check_pairs(g, (exp.vals_pos, exp.lags_pos, exp.vals_neg, exp.lags_neg), r, thr, label="block vs port")
        check_hist(got.max_hist.cpu().numpy(), got.min_hist.cpu().numpy(), exp.max_hist, exp.min_hist, r, 12)
    # the plain size-P form, same bar
    monkeypatch.setenv("SEISMIC_BLOCK_FORM", "off")
    assert _plan(lib, length, shift, c)[1] == 0
    plain = xcorr.xcorr(t, shift, threshold=thr, n_classes_hist=12)
    torch.cuda.synchronize()
    pl = [x.cpu().numpy() for x in (plain.vals_pos, plain.lags_pos, plain.vals_neg, plain.lags_neg)]
    check_pairs(g, pl, r, thr, label="block vs plain")
    print(f"n={n} c={c} L={length} shift={shift}: Q={tq} nb={nb} B={bl}, max err vs FP64 "
          f"{max(ag.max_err_pos, ag.max_err_neg):.3g}")


def test_block_form_host_entry_matches_device_entry(cuda_ok):
    """seismic_xcorr_host launches the pair kernel in chunks of L2 bands (the
    copy-back of one chunk overlaps the next); the overlap-save form gives the
    same bits as one device call."""
    import torch
    ev = synth.family_catalog(700, 1, 1024, n_families=20, seed=731)
    dev = xcorr.xcorr(torch.from_numpy(ev).cuda(), 128, threshold=0.0, n_classes_hist=20)
    torch.cuda.synchronize()
    host = xcorr.xcorr(ev, 128, threshold=0.0, n_classes_hist=20)
    for a, b in zip((dev.vals_pos, dev.lags_pos, dev.vals_neg, dev.lags_neg, dev.max_hist, dev.min_hist),
                    (host.vals_pos, host.lags_pos, host.vals_neg, host.lags_neg, host.max_hist, host.min_hist)):
        np.testing.assert_array_equal(a.cpu().numpy(), b)


def test_stage_entry_point_equals_one_call(cuda_ok):
    """seismic_xcorr_device_stages 1 then 2 (the transforms, then the pairs)
    gives the bits of one seismic_xcorr_device call, for an FFT form with
    the overlap-save plan and for a lag-GEMM form; one stage-1 result serves
    two stage-2 calls with other thresholds."""
    import torch
    lib = cuda_ok
    ev = synth.family_catalog(150, 1, 1024, n_families=6, seed=741)
    t = torch.from_numpy(ev).cuda()
    n = ev.shape[0]
    m = n * (n + 1) // 2
    for form in (0, 4):
        wsb = lib.seismic_xcorr_workspace_bytes(n, 1, 1024, 128, 0, form)
        ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
        outs = {}
        for key, stages, thr in (("one", [3], 0.0), ("split", [1, 2], 0.0), ("thr", [2], 0.3)):
            o = [torch.zeros(m, device="cuda"), torch.zeros(m, dtype=torch.int32, device="cuda"),
                 torch.zeros(m, device="cuda"), torch.zeros(m, dtype=torch.int32, device="cuda")]
            h = torch.zeros(2, 10, dtype=torch.int32, device="cuda")
            for st in stages:
                _lib.check(lib.seismic_xcorr_device_stages(t.data_ptr(), n, 1, 1024, 1024, 1024, 0, 128,
                                                           ctypes.c_float(thr), 10, form,
                                                           *(x.data_ptr() for x in o), h[0].data_ptr(),
                                                           h[1].data_ptr(), ws.data_ptr(), wsb, None, st))
            torch.cuda.synchronize()
            outs[key] = [x.cpu().numpy() for x in o] + [h.cpu().numpy()]
        for a, b in zip(outs["one"], outs["split"]):
            np.testing.assert_array_equal(a, b)
        keep = outs["one"][0] > 0.3
        np.testing.assert_array_equal(outs["thr"][0], np.where(keep, outs["one"][0], 0.0))
        np.testing.assert_array_equal(outs["thr"][4], outs["one"][4])  # histograms come before the threshold
    assert lib.seismic_xcorr_device_stages(t.data_ptr(), n, 1, 1024, 1024, 1024, 0, 128, ctypes.c_float(0.0), 0, 0,
                                           *(0 for _ in range(4)), None, None, None, 0, None, 2) == 1
