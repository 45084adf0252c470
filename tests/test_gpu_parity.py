"""GPU parity tests of the FP32 fused path, through the C ABI.

Reference outputs come from the golden fixtures (the reference's own OMP
source + wrapper), from the C restatement (pinned bit-exact to those
fixtures by test_oracle.py) on larger seeded inputs, and from the FP64
oracle.  Tolerances: see tolerances.py.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from oracle import oracle as O
from seismic_gb300 import _lib, correlation_lib, synth, xcorr
from tolerances import check_hist, check_pairs

pytestmark = pytest.mark.gpu


class _Trace:
    def __init__(self, d):
        self.data = d


def _traces(ev):
    out = np.empty(ev.shape[0], dtype=object)
    for k in range(ev.shape[0]):
        out[k] = _Trace(ev[k])
    return out


@pytest.mark.parametrize("name", golden_cases())
def test_dropin_cpp_matches_reference_golden(cuda_ok, name):
    g = load_golden(name)
    ev = g["events"]
    n = ev.shape[0]
    thr = float(g["threshold"])
    nh = int(g["n_classes_hist"])
    got = correlation_lib.compute_correlation(_traces(ev), int(g["shift"]), 4, 1, thr, nh)
    i, j = O.triu_pairs(n)
    r = O.fp64_xcorr(ev, int(g["shift"]), i, j, padded=int(g["padded"]))
    check_pairs(got[:4], (g["xcm_pos"], g["xclags_pos"], g["xcm_neg"], g["xclags_neg"]), r, thr, label=name)
    check_hist(got[4], got[5], g["max_hist"], g["min_hist"], r, nh)


@pytest.mark.parametrize("name", ["ricker_n64_l512_full", "family_n48_l1024_s128", "ragged_n37_l300_s200"])
def test_dropin_cuda_signature_matches_golden(cuda_ok, name):
    g = load_golden(name)
    ev = g["events"]
    thr = float(g["threshold"])
    correlation_lib.initialiseRunTime()
    got = correlation_lib.compute_correlation_cuda(ev, int(g["shift"]), 8, thr)
    i, j = O.triu_pairs(ev.shape[0])
    r = O.fp64_xcorr(ev, int(g["shift"]), i, j, padded=int(g["padded"]))
    check_pairs(got, (g["xcm_pos"], g["xclags_pos"], g["xcm_neg"], g["xclags_neg"]), r, thr, label=name)


def test_cuda_dropin_module_as_the_reference_driver_imports_it(cuda_ok, tmp_path):
    """The CUDA drop-in module run the way Correlation_in_CUDA/test_cuda.py:15,32
    uses the reference's: ``from correlation_lib import compute_correlation,
    initialiseRunTime`` with the module's directory on sys.path, in a fresh
    process, compared with the golden fixture the reference made."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    g = load_golden("family_n48_l1024_s128")
    np.save(tmp_path / "events.npy", g["events"])
    script = (
        "import sys, numpy as np\n"
        f"sys.path.insert(0, {os.path.join(root, 'seismic_gb300', 'cuda')!r})\n"
        "from correlation_lib import compute_correlation, initialiseRunTime\n"
        "initialiseRunTime()\n"
        f"ev = np.load({str(tmp_path / 'events.npy')!r})\n"
        f"out = compute_correlation(ev, {int(g['shift'])}, 8, {float(g['threshold'])!r})\n"
        f"np.savez({str(tmp_path / 'out.npz')!r}, *out)\n")
    subprocess.run([sys.executable, "-c", script], check=True, cwd=str(tmp_path), timeout=300)
    z = np.load(tmp_path / "out.npz")
    got = tuple(z[f"arr_{k}"] for k in range(4))
    ev = g["events"]
    i, j = O.triu_pairs(ev.shape[0])
    r = O.fp64_xcorr(ev, int(g["shift"]), i, j, padded=int(g["padded"]))
    check_pairs(got, (g["xcm_pos"], g["xclags_pos"], g["xcm_neg"], g["xclags_neg"]), r, float(g["threshold"]),
                label="cuda drop-in module")


def test_small_workload_full_triangle_vs_port(cuda_ok):
    """N=200 Ricker events, L=512, lags -511..512, full triangle."""
    ev, shift = synth.make_workload("small")
    ev = ev[:, 0]
    exp = O.port_correlation_cpp(ev, shift, 0.0, 20)
    got = correlation_lib.compute_correlation(ev, shift, 4, 4, 0.0, 20)
    i, j = O.triu_pairs(ev.shape[0])
    r = O.fp64_xcorr(ev, shift, i, j)
    stats = check_pairs(got[:4], (exp.vals_pos, exp.lags_pos, exp.vals_neg, exp.lags_neg), r, 0.0)
    check_hist(got[4], got[5], exp.max_hist, exp.min_hist, r, 20)
    ag = O.agreement(*got[:4], r)
    assert ag.max_err_pos < 1e-5 and ag.max_err_neg < 1e-5
    assert ag.lag_mismatch == 0, (ag, stats)


@pytest.mark.parametrize("n,length,shift,thr,nh", [
    (13, 2048, 2048, 0.0, 20),     # P = 4096, ragged tile
    (9, 4096, 4096, 0.25, 10),     # P = 8192
    (11, 32, 32, 0.0, 4),          # P = 64
    (21, 200, 56, 0.1, 6),         # P = 256
    (70, 700, 300, 0.05, 17),      # P = 1024, non-power-of-two L
    (6, 9000, 9000, 0.0, 10),      # P = 16384: one 512-thread FFT group per CTA
    (5, 17000, 300, 0.1, 8),       # padded 32768: beyond the plain transform, the overlap-save form
])
def test_sizes_vs_port(cuda_ok, n, length, shift, thr, nh):
    ev = synth.family_catalog(n, 1, length, n_families=max(1, n // 4), seed=n + length)[:, 0]
    exp = O.port_correlation_cpp(ev, shift, thr, nh)
    got = correlation_lib.compute_correlation(ev, shift, 2, 1, thr, nh)
    i, j = O.triu_pairs(n)
    r = O.fp64_xcorr(ev, shift, i, j)
    check_pairs(got[:4], (exp.vals_pos, exp.lags_pos, exp.vals_neg, exp.lags_neg), r, thr)
    check_hist(got[4], got[5], exp.max_hist, exp.min_hist, r, nh)


def test_non_power_of_two_padded_size_dropin(cuda_ok):
    """The reference's C entry point with a paddedSize that is not a power of
    two but holds the lag window: the size-3000 circular correlation the
    reference computes is the linear one, against FP64 at that size."""
    n, length, shift, padded = 23, 1000, 900, 3000
    ev = synth.family_catalog(n, 1, length, n_families=3, seed=41)[:, 0]
    lay = np.zeros((n, padded), np.float32)  # the reference's padded layout, rows of paddedSize
    lay[:, :length] = ev
    m = n * (n + 1) // 2
    got = [np.zeros(m, np.float32), np.zeros(m, np.int32), np.zeros(m, np.float32), np.zeros(m, np.int32)]
    hmax, hmin = np.zeros(10, np.int32), np.zeros(10, np.int32)
    lib = _lib.lib()
    fp, ip = _lib.c_float_p, _lib.c_int_p
    lib.correlationCPP(lay.ctypes.data_as(fp), lay.ctypes.data_as(fp), n, length, shift, padded, 2, 1, 0.0, 10,
                       got[0].ctypes.data_as(fp), got[1].ctypes.data_as(ip), got[2].ctypes.data_as(fp),
                       got[3].ctypes.data_as(ip), hmax.ctypes.data_as(ip), hmin.ctypes.data_as(ip))
    _lib.check(lib.seismic_last_error())
    assert int(hmax.sum()) == m
    i, j = O.triu_pairs(n)
    ref = O.fp64_xcorr(ev, shift, i, j, padded=3000)
    ag = O.agreement(*got[:4], ref)
    assert ag.max_err_pos < 1e-5 and ag.max_err_neg < 1e-5, ag
    assert ag.lag_mismatch == 0, ag


def test_large_padded_sizes_native(cuda_ok):
    """The native entry point on long events: P = 16384 (plain, three channels)
    and a 2^17 padded size with a short lag window (overlap-save frames), each
    against FP64; a padded size beyond the plain transform whose lag window
    the overlap-save form cannot take is refused."""
    import ctypes
    import torch
    lib = _lib.lib()
    for n, c, length, shift in ((7, 3, 6000, 5000), (4, 1, 70000, 1000)):
        ev = synth.family_catalog(n, c, length, n_families=2, seed=length)
        r = xcorr.xcorr(torch.from_numpy(ev).cuda(), shift, threshold=0.0, n_classes_hist=8)
        torch.cuda.synchronize()
        P = xcorr.resolve_padded_size(length, shift)
        i, j = O.triu_pairs(n)
        ref = O.fp64_xcorr(ev, shift, i, j, padded=P)
        ag = O.agreement(r.vals_pos.cpu().numpy(), r.lags_pos.cpu().numpy(), r.vals_neg.cpu().numpy(),
                         r.lags_neg.cpu().numpy(), ref)
        assert ag.max_err_pos < 1e-5 and ag.max_err_neg < 1e-5, (length, ag)
        assert ag.lag_mismatch == 0, (length, ag)
    P, nb, bl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _lib.check(lib.seismic_fft_plan(70000, 1000, 0, 1, 0, ctypes.byref(P), ctypes.byref(nb), ctypes.byref(bl)))
    assert nb.value > 0 and P.value <= 4096
    assert lib.seismic_fft_plan(20000, 3000, 32768, 1, 0, ctypes.byref(P), ctypes.byref(nb), ctypes.byref(bl)) == 2
    assert lib.seismic_xcorr_workspace_bytes(4, 1, 20000, 3000, 32768, 0) == 0


@pytest.mark.parametrize("n,c,length,shift", [
    (11, 3, 700, 300),    # P = 1024, three channels: the lane vote
    (9, 40, 400, 200),    # P = 1024, forty channels: lanes 0..31 vote, thread 0 checks the rest
    (8, 3, 2048, 1500),   # P = 4096, the split exchange
])
def test_multichannel_zero_norms(cuda_ok, monkeypatch, n, c, length, shift):
    """Multichannel (prescaled) pairs with zero-norm channels: a pair is live
    when some channel has both norms nonzero, zero channels add nothing to the
    mean, an all-zero event gives zeros.  Against FP64, and the staged form
    bit-identical to the direct form."""
    import torch
    ev = synth.family_catalog(n, c, length, n_families=2, seed=n + c)
    ev[2, 1] = 0.0            # one channel of event 2
    ev[5] = 0.0               # all of event 5
    ev[6, :c - 1] = 0.0       # event 6 keeps only its last channel
    ev[7, c - 1] = 0.0        # event 7 lacks exactly that one: (6, 7) has no common channel
    t = torch.from_numpy(ev).cuda()
    i, j = O.triu_pairs(n)
    ref = O.fp64_xcorr(ev, shift, i, j, padded=xcorr.resolve_padded_size(length, shift))
    got = {}
    for kind in ("staged", "direct"):
        monkeypatch.setenv("SEISMIC_PAIR_KERNEL", kind)
        r = xcorr.xcorr(t, shift, threshold=0.0, n_classes_hist=8)
        torch.cuda.synchronize()
        got[kind] = [x.cpu().numpy() for x in (r.vals_pos, r.lags_pos, r.vals_neg, r.lags_neg)] + \
                    [r.max_hist.cpu().numpy(), r.min_hist.cpu().numpy()]
        ag = O.agreement(*got[kind][:4], ref)
        assert ag.max_err_pos < 1e-5 and ag.max_err_neg < 1e-5, (kind, ag)
        assert ag.lag_mismatch == 0, (kind, ag)
        for e in range(n):  # the all-zero event: zeros everywhere
            k = xcorr.packed_index(np.array([min(e, 5)]), np.array([max(e, 5)]), n)[0]
            assert got[kind][0][k] == 0 and got[kind][2][k] == 0 and got[kind][1][k] == 0
        k = xcorr.packed_index(np.array([6]), np.array([7]), n)[0]
        assert got[kind][0][k] == 0 and got[kind][2][k] == 0  # no channel in common
    for a, b in zip(got["staged"], got["direct"]):
        np.testing.assert_array_equal(a, b)


def test_zero_norm_event_defined(cuda_ok):
    ev = synth.ricker_catalog(6, 256, seed=31)[:, 0].copy()
    ev[3] = 0.0
    got = correlation_lib.compute_correlation(ev, 128, 1, 1, 0.0, 8)
    exp = O.port_correlation_cpp(ev, 128, 0.0, 8)
    np.testing.assert_array_equal(got[4], exp.max_hist)
    np.testing.assert_array_equal(got[5], exp.min_hist)
    idx = xcorr.packed_index(np.array([0, 1, 2, 3, 3, 3]), np.array([3, 3, 3, 3, 4, 5]), 6)
    for a in got[:4]:
        assert np.all(a[idx] == 0)


def test_shift_zero_and_single_event(cuda_ok):
    ev = synth.ricker_catalog(1, 100, seed=1)[:, 0]
    got = correlation_lib.compute_correlation(ev, 50, 1, 1, 0.0, 4)
    assert got[1][0] == 0 and abs(got[0][0] - 1.0) < 1e-5
    ev = synth.ricker_catalog(5, 100, seed=2)[:, 0]
    got = correlation_lib.compute_correlation(ev, 0, 1, 1, 0.0, 4)
    for a in got[:4]:
        assert np.all(a == 0)
    assert got[4][0] == 15 and got[5][0] == 15   # every pair counted in bin 0


def test_multichannel_vs_fp64(cuda_ok):
    """3 channels, mean of per-channel normalised series, full lag range."""
    ev = synth.family_catalog(40, 3, 1024, n_families=3, seed=41)
    shift = 1024
    res = xcorr.xcorr(ev, shift, threshold=0.0, n_classes_hist=20)
    i, j = O.triu_pairs(40)
    r = O.fp64_xcorr(ev, shift, i, j, padded=xcorr.resolve_padded_size(1024, shift))
    ag = O.agreement(res.vals_pos, res.lags_pos, res.vals_neg, res.lags_neg, r)
    assert ag.max_err_pos < 1e-5 and ag.max_err_neg < 1e-5, ag
    assert ag.lag_mismatch == 0, ag
    assert res.max_hist.sum() == i.size and res.min_hist.sum() == i.size


def test_device_api_torch_stream_and_workspace(cuda_ok):
    import torch
    from seismic_gb300 import _lib
    ev = synth.family_catalog(50, 2, 600, n_families=2, seed=5)
    t = torch.from_numpy(ev).cuda()
    host = xcorr.xcorr(ev, 200, threshold=0.1, n_classes_hist=10)
    lib = _lib.lib()
    p = xcorr.resolve_padded_size(600, 200)
    ws = torch.empty(lib.seismic_xcorr_workspace_bytes(50, 2, 600, 200, p, 0), dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        dev = xcorr.xcorr(t, 200, threshold=0.1, n_classes_hist=10, workspace=ws)
    s.synchronize()
    np.testing.assert_array_equal(dev.vals_pos.cpu().numpy(), host.vals_pos)
    np.testing.assert_array_equal(dev.lags_neg.cpu().numpy(), host.lags_neg)
    np.testing.assert_array_equal(dev.max_hist.cpu().numpy(), host.max_hist)
    small = torch.empty(16, dtype=torch.uint8, device="cuda")
    with pytest.raises(_lib.SeismicError):
        xcorr.xcorr(t, 200, workspace=small)
    big = torch.empty(ws.numel() + 256, dtype=torch.uint8, device="cuda")
    with pytest.raises(_lib.SeismicError, match="aligned"):
        xcorr.xcorr(t, 200, workspace=big[16:])  # enough bytes, not 256-byte aligned


@pytest.mark.parametrize("n,length,shift", [(150, 200, 56), (70, 2048, 2048)])  # direct form (P=256), staged form
def test_pair_ranges_on_streams_compose_the_triangle(cuda_ok, n, length, shift):
    """Disjoint work-item ranges (how ranks or streams share one catalog)
    write exactly what one full launch writes."""
    import ctypes
    import torch
    from seismic_gb300 import _lib
    from seismic_gb300.shard import couple_range
    lib = _lib.lib()
    ev = synth.family_catalog(n, 3, length, n_families=5, seed=91)
    n, c, length = ev.shape
    p = xcorr.resolve_padded_size(length, shift)
    t = torch.from_numpy(ev).cuda()
    rows = n * c
    spec = torch.empty(rows * p // 2 * 2, device="cuda")
    norms = torch.empty(2 * rows, dtype=torch.float64, device="cuda")
    _lib.check(lib.seismic_spectra_device(t.data_ptr(), n, c, length, c * length, length, p, 1, spec.data_ptr(),
                                          norms.data_ptr(), None))
    m = n * (n + 1) // 2
    full = [torch.zeros(m, device="cuda"), torch.zeros(m, dtype=torch.int32, device="cuda"),
            torch.zeros(m, device="cuda"), torch.zeros(m, dtype=torch.int32, device="cuda")]
    parts = [torch.full((m,), float("nan"), device="cuda"), torch.zeros(m, dtype=torch.int32, device="cuda"),
             torch.full((m,), float("nan"), device="cuda"), torch.zeros(m, dtype=torch.int32, device="cuda")]
    _lib.check(lib.seismic_pairs_device(spec.data_ptr(), norms.data_ptr(), n, c, p, 1, shift, 0.0, 0, 0,
                                        *(x.data_ptr() for x in full), None, None, None))
    total = lib.seismic_pair_couples(n, p, c)
    streams = [torch.cuda.Stream() for _ in range(3)]
    for r, s in enumerate(streams):
        b, e = couple_range(total, 3, r)
        _lib.check(lib.seismic_pairs_device_range(spec.data_ptr(), norms.data_ptr(), n, c, p, 1, shift, 0.0, 0, b, e,
                                                  *(x.data_ptr() for x in parts), None, None,
                                                  ctypes.c_void_p(s.cuda_stream)))
    torch.cuda.synchronize()
    for a, b in zip(full, parts):
        assert torch.equal(a, b)


@pytest.mark.parametrize("n,c,length,shift", [
    (150, 3, 700, 300),    # P = 1024, ragged last tile
    (61, 1, 2048, 2048),   # P = 4096
    (130, 3, 2048, 1500),  # P = 4096, three channels
    (200, 2, 300, 44),     # P = 512
    (77, 3, 1024, 256),    # P = 2048, the serving shape
    (90, 1, 1024, 128),    # P = 2048, one channel: the wide (14 FFT warp) CTA
])
def test_staged_and_direct_forms_agree_bitwise(cuda_ok, monkeypatch, n, c, length, shift):
    """The TMA-staged pair form and the direct-load form compute the same
    couples (i; j, j+1), j even, in the same arithmetic order: identical
    outputs and histograms, both within the FP64 bar."""
    import torch
    ev = synth.family_catalog(n, c, length, n_families=max(1, n // 10), seed=n + c)
    t = torch.from_numpy(ev).cuda()
    i, j = O.triu_pairs(n)
    ref = O.fp64_xcorr(ev, shift, i, j, padded=xcorr.resolve_padded_size(length, shift))
    got = {}
    monkeypatch.setenv("SEISMIC_BLOCK_FORM", "off")  # the plain transform in both forms
    for kind in ("staged", "direct"):
        monkeypatch.setenv("SEISMIC_PAIR_KERNEL", kind)
        r = xcorr.xcorr(t, shift, threshold=0.0, n_classes_hist=16)
        torch.cuda.synchronize()
        got[kind] = [x.cpu().numpy() for x in (r.vals_pos, r.lags_pos, r.vals_neg, r.lags_neg)] + \
                    [r.max_hist.cpu().numpy(), r.min_hist.cpu().numpy()]
        ag = O.agreement(*got[kind][:4], ref)
        assert ag.max_err_pos < 1e-5 and ag.max_err_neg < 1e-5, (kind, ag)
        assert ag.lag_mismatch == 0, (kind, ag)
    for a, b in zip(got["staged"], got["direct"]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("n,c,length,shift,block", [
    (203, 1, 1024, 128, "on"),    # overlap-save frames Q = 512 x 4: 24 groups, TI = 6
    (150, 3, 700, 300, "off"),    # P = 1024, ragged last tile: 12 groups
    (130, 3, 2048, 1500, "off"),  # P = 4096: 3 groups, TI = 3
    (90, 1, 1024, 128, "off"),    # P = 2048, the wide CTA: 7 groups, TI = 7
])
def test_staged_item_shapes_agree_bitwise(cuda_ok, monkeypatch, n, c, length, shift, block):
    """Staged work items of TI i events x TJ j events -- the automatic TI,
    one i per item, and other divisors of the group count -- run the same
    couples in the same arithmetic: identical outputs and histograms, and
    the automatic one within the FP64 bar."""
    import torch
    ev = synth.family_catalog(n, c, length, n_families=max(1, n // 10), seed=n + 3 * c)
    t = torch.from_numpy(ev).cuda()
    monkeypatch.setenv("SEISMIC_BLOCK_FORM", block)
    got = {}
    for ti in ("", "1", "2", "3"):
        monkeypatch.setenv("SEISMIC_STAGED_TI", ti)
        r = xcorr.xcorr(t, shift, threshold=0.0, n_classes_hist=16)
        torch.cuda.synchronize()
        got[ti] = [x.cpu().numpy() for x in (r.vals_pos, r.lags_pos, r.vals_neg, r.lags_neg)] + \
                  [r.max_hist.cpu().numpy(), r.min_hist.cpu().numpy()]
    i, j = O.triu_pairs(n)
    ref = O.fp64_xcorr(ev, shift, i, j, padded=xcorr.resolve_padded_size(length, shift))
    ag = O.agreement(*got[""][:4], ref)
    assert ag.max_err_pos < 1e-5 and ag.max_err_neg < 1e-5, ag
    assert ag.lag_mismatch == 0, ag
    for ti in ("1", "2", "3"):
        for a, b in zip(got[""], got[ti]):
            np.testing.assert_array_equal(a, b)


def test_precision_workload_size_properties(cuda_ok):
    """Full-size N=16384, L=1024, +-128 lags: properties that hold at any size
    (diagonal coefficient 1 at lag 0, |coef| <= 1, histogram totals) and an
    FP64 check of a random sample of pairs."""
    import torch
    ev, shift = synth.make_workload("precision")
    n = ev.shape[0]
    t = torch.from_numpy(ev).cuda()
    res = xcorr.xcorr(t, shift, threshold=0.0, n_classes_hist=20)
    vp = res.vals_pos.cpu().numpy()
    lp = res.lags_pos.cpu().numpy()
    vn = res.vals_neg.cpu().numpy()
    ln = res.lags_neg.cpu().numpy()
    diag = xcorr.packed_index(np.arange(n), np.arange(n), n)
    assert np.abs(vp[diag] - 1.0).max() < 1e-5
    assert np.all(lp[diag] == 0)
    assert vp.max() <= 1.0 + 1e-5 and vn.min() >= -1.0 - 1e-5
    assert int(res.max_hist.sum()) == vp.size and int(res.min_hist.sum()) == vp.size
    rng = np.random.default_rng(0)
    i = rng.integers(0, n, 3000)
    j = rng.integers(0, n, 3000)
    i, j = np.minimum(i, j), np.maximum(i, j)
    idx = xcorr.packed_index(i, j, n)
    r = O.fp64_xcorr(ev, shift, i, j)
    ag = O.agreement(vp[idx], lp[idx], vn[idx], ln[idx], r)
    assert ag.max_err_pos < 1e-5 and ag.max_err_neg < 1e-5, ag
    assert ag.lag_mismatch == 0, ag


@pytest.mark.parametrize("length", [200, 1000, 4096])
def test_spectra_norms_fp64_over_amplitude_range(cuda_ok, length):
    """Kernel (a)'s norms against numpy FP64 sums of squares, for rows from
    1e-30 to 1e30 in amplitude, a row with one large spike, and a zero row:
    relative error at the FP64 level; the inverse norms, kept as hi + lo
    floats, equal the FP64 inverse to 2^-46 relative with hi rounded once."""
    import torch
    from seismic_gb300 import _lib
    lib = _lib.lib()
    rng = np.random.default_rng(92)
    amps = [1e-30, 1e-12, 1e-3, 1.0, 7.5e4, 1e12, 1e30]
    ev = np.stack([rng.standard_normal(length) * a for a in amps]
                  + [np.r_[1e20, rng.standard_normal(length - 1) * 1e-3], np.zeros(length)]).astype(np.float32)
    n = ev.shape[0]
    p = xcorr.resolve_padded_size(length, length)
    t = torch.from_numpy(ev).cuda()
    spec = torch.empty(n * p // 2 * 2, device="cuda")
    norms = torch.empty(2 * n, dtype=torch.float64, device="cuda")
    _lib.check(lib.seismic_spectra_device(t.data_ptr(), n, 1, length, length, length, p, 0, spec.data_ptr(),
                                          norms.data_ptr(), None))
    torch.cuda.synchronize()
    got = norms[:n].cpu().numpy()
    pair = norms[n:].cpu().numpy().view(np.float32).reshape(n, 2)
    want = np.sqrt((ev.astype(np.float64) ** 2).sum(axis=1))
    np.testing.assert_allclose(got[:-1], want[:-1], rtol=1e-12)
    assert got[-1] == 0.0 and pair[-1, 0] == 0.0 and pair[-1, 1] == 0.0
    np.testing.assert_array_equal(pair[:-1, 0], (1.0 / got[:-1]).astype(np.float32))
    inv = pair[:, 0].astype(np.float64) + pair[:, 1].astype(np.float64)
    # 48 bits while the low part stays a normal float (1/norm > ~2^-102);
    # below that it loses bits to FP32's subnormal range
    normal = pair[:-1, 0] > 2.0 ** -102
    np.testing.assert_allclose(inv[:-1][normal], (1.0 / got[:-1])[normal], rtol=2.0 ** -46)
    np.testing.assert_allclose(inv[:-1], 1.0 / got[:-1], rtol=2.0 ** -40)


@pytest.mark.parametrize("n,c,length,shift,form", [(600, 3, 1024, 1024, "fp32"),   # staged form, P=2048
                                                   (500, 1, 2048, 1024, "fp16"),   # staged, half spectra, P=4096
                                                   (100, 1, 4096, 4096, "fp32"),   # direct form, P=8192
                                                   (2000, 1, 128, 128, "fp32")])   # direct form, P=256
def test_host_chunks_by_row_band_match_device_call(cuda_ok, monkeypatch, n, c, length, shift, form):
    """With 1 MB L2 bands the host entry point runs the pair kernel in several
    chunks of row bands, each copied back while the next runs: bit-identical
    to one device call over the same tiles."""
    import torch
    monkeypatch.setenv("SEISMIC_L2_BAND_MB", "1")
    ev = synth.family_catalog(n, c, length, n_families=4, seed=93)
    host = xcorr.xcorr(ev, shift, threshold=0.1, n_classes_hist=12, form=form)
    dev = xcorr.xcorr(torch.from_numpy(ev).cuda(), shift, threshold=0.1, n_classes_hist=12, form=form)
    torch.cuda.synchronize()
    for f in ("vals_pos", "lags_pos", "vals_neg", "lags_neg", "max_hist", "min_hist"):
        np.testing.assert_array_equal(getattr(host, f), getattr(dev, f).cpu().numpy())
