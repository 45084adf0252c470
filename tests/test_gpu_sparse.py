"""GPU tests of the consumers of the packed outputs: on-device compaction of
the pairs above a threshold (the reference's sparse CSR output,
Correlation_in_OMP/test_c.py:43-55) and the standalone histogram."""
import numpy as np
import pytest

from seismic_gb300 import synth, xcorr

pytestmark = pytest.mark.gpu


def _dense_csr(a, dtype):
    from scipy.sparse import csr_matrix
    return csr_matrix(np.asarray(a)[None, :], dtype=dtype)


def _same_csr(got, exp):
    assert got.shape == exp.shape
    np.testing.assert_array_equal(got.indices, exp.indices)
    np.testing.assert_array_equal(got.indptr, exp.indptr)
    np.testing.assert_array_equal(got.data, exp.data)


@pytest.mark.parametrize("n,c,length,shift,thr", [(300, 1, 512, 512, 0.3), (130, 3, 2048, 1500, 0.5),
                                                  (77, 3, 1024, 256, 0.0), (1, 1, 64, 32, 0.1)])
def test_compaction_equals_reference_csr_of_thresholded_run(cuda_ok, n, c, length, shift, thr):
    """Compacting threshold-0 outputs at `thr` gives the CSR matrices the
    reference builds from a run with threshold `thr`."""
    import torch
    from seismic_gb300 import sparse
    ev = synth.family_catalog(n, c, length, n_families=max(1, n // 20), seed=n + 3)
    t = torch.from_numpy(ev).cuda()
    r0 = xcorr.xcorr(t, shift, threshold=0.0)
    rt = xcorr.xcorr(t, shift, threshold=thr)
    sp = sparse.compact(r0.vals_pos, r0.lags_pos, r0.vals_neg, r0.lags_neg, thr)
    torch.cuda.synchronize()
    m = sparse.to_csr(sp)
    _same_csr(m["xcm_pos"], _dense_csr(rt.vals_pos.cpu().numpy(), np.float32))
    _same_csr(m["xclags_pos"], _dense_csr(rt.lags_pos.cpu().numpy(), np.int32))
    _same_csr(m["xcm_neg"], _dense_csr(rt.vals_neg.cpu().numpy(), np.float32))
    _same_csr(m["xclags_neg"], _dense_csr(rt.lags_neg.cpu().numpy(), np.int32))
    # packed order, and exact counts
    idx = sp.index_pos.cpu().numpy()
    assert np.all(np.diff(idx) > 0)
    assert idx.size == int((r0.vals_pos.cpu().numpy() > thr).sum())


def test_compaction_capacity_and_counts(cuda_ok):
    """A capacity below the count writes a prefix and still reports the count."""
    import ctypes
    import torch
    from seismic_gb300 import _lib
    lib = _lib.lib()
    n = 10_000
    g = torch.Generator(device="cuda").manual_seed(3)
    vp = torch.rand(n, device="cuda", generator=g)
    vn = -torch.rand(n, device="cuda", generator=g)
    lp = torch.arange(n, dtype=torch.int32, device="cuda")
    ln = -lp
    ws = torch.empty(lib.seismic_compact_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    counts = torch.zeros(2, dtype=torch.int64, device="cuda")
    cap = 100
    out = [torch.full((cap,), -1, dtype=torch.int64, device="cuda"), torch.zeros(cap, device="cuda"),
           torch.zeros(cap, dtype=torch.int32, device="cuda"), torch.full((cap,), -1, dtype=torch.int64, device="cuda"),
           torch.zeros(cap, device="cuda"), torch.zeros(cap, dtype=torch.int32, device="cuda")]
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    _lib.check(lib.seismic_compact_pairs_device(p(vp), p(lp), p(vn), p(ln), n, ctypes.c_float(0.5), cap,
                                                *(p(o) for o in out), p(counts), p(ws), ws.numel(), None))
    torch.cuda.synchronize()
    keep_p = np.nonzero(vp.cpu().numpy() > 0.5)[0]
    keep_n = np.nonzero(vn.cpu().numpy() < -0.5)[0]
    assert counts.cpu().tolist() == [keep_p.size, keep_n.size]
    np.testing.assert_array_equal(out[0].cpu().numpy(), keep_p[:cap])
    np.testing.assert_array_equal(out[2].cpu().numpy(), keep_p[:cap])      # lags = index here
    np.testing.assert_array_equal(out[3].cpu().numpy(), keep_n[:cap])
    np.testing.assert_array_equal(out[5].cpu().numpy(), -keep_n[:cap])
    with pytest.raises(_lib.SeismicError):
        _lib.check(lib.seismic_compact_pairs_device(p(vp), p(lp), p(vn), p(ln), n, ctypes.c_float(0.5), 0,
                                                    None, None, None, None, None, None, p(counts), p(ws), 8,
                                                    None))


@pytest.mark.parametrize("n_hist", [7, 20, 5000])
def test_standalone_histogram_equals_pair_kernel_histogram(cuda_ok, n_hist):
    import torch
    from seismic_gb300 import sparse
    ev = synth.family_catalog(200, 2, 700, n_families=6, seed=17)
    r = xcorr.xcorr(torch.from_numpy(ev).cuda(), 300, threshold=0.0, n_classes_hist=n_hist)
    hmax, hmin = sparse.histogram(r.vals_pos, r.vals_neg, n_hist)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(hmax.cpu().numpy(), r.max_hist.cpu().numpy())
    np.testing.assert_array_equal(hmin.cpu().numpy(), r.min_hist.cpu().numpy())


def test_save_npz_writes_reference_files(cuda_ok, tmp_path):
    import torch
    from scipy.sparse import load_npz
    from seismic_gb300 import sparse
    ev = synth.ricker_catalog(50, 256, seed=4)
    r = xcorr.xcorr(torch.from_numpy(ev).cuda(), 128, threshold=0.0, n_classes_hist=10)
    sp = sparse.compact(r.vals_pos, r.lags_pos, r.vals_neg, r.lags_neg, 0.2)
    paths = sparse.save_npz(str(tmp_path), sp, r.max_hist, r.min_hist)
    assert sorted(p.split("/")[-1] for p in paths) == sorted(
        ["out_xcm_pos.npz", "out_xcl_pos.npz", "out_xcm_neg.npz", "out_xcl_neg.npz", "out_xmax_hist.npz",
         "out_xmin_hist.npz"])
    m = load_npz(paths[0])
    assert m.shape == (1, 50 * 51 // 2) and np.all(m.data > 0.2)
