"""CPU tests of the host-side logic: the C ABI library loads and exports every
symbol the public header declares, host-only entry points, the Python
drop-in's padding, and the pair scheduler's coverage of the triangle."""
import ctypes
import importlib.util
import os
import math
import subprocess

import numpy as np
import pytest

from seismic_gb300 import _dropin, _lib, xcorr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_header_symbol(built_lib):
    names = _lib.header_symbols()
    assert {"correlationCPP", "correlationCUDA", "initialiseCUDA"} <= set(names)
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, f"declared in the header but not exported: {missing}"
    for n in names:
        assert hasattr(built_lib, n)


def test_resolve_padded_size(built_lib):
    assert xcorr.resolve_padded_size(512, 512) == 1024
    assert xcorr.resolve_padded_size(1024, 128) == 2048
    assert xcorr.resolve_padded_size(1000, 1000) == 2048
    assert xcorr.resolve_padded_size(3000, 3000) == 8192
    assert xcorr.resolve_padded_size(5000, 5000) == 16384
    assert xcorr.resolve_padded_size(9000, 9000) == 0       # beyond the plain transform, lag window too wide
    assert xcorr.resolve_padded_size(20000, 300) == 32768   # the overlap-save form's sizes
    assert xcorr.resolve_padded_size(20000, 1792) == 32768
    assert xcorr.resolve_padded_size(20000, 1793) == 0
    assert xcorr.resolve_padded_size(10, 5) == 64


def test_status_strings(built_lib):
    assert built_lib.seismic_status_string(0) == b"ok"
    assert built_lib.seismic_status_string(2) == b"unsupported size"


def test_workspace_bytes(built_lib):
    b = built_lib.seismic_xcorr_workspace_bytes(1000, 3, 1024, 1024, 2048, 0)
    assert b >= 1000 * 3 * 1024 * 8 + 1000 * 3 * 8
    assert built_lib.seismic_xcorr_workspace_bytes(1000, 3, 1024, 1024, 1000, 0) == 0
    # lag-GEMM form: two BF16 copies (hi, lo) of the events + FP64 norms
    b = built_lib.seismic_xcorr_workspace_bytes(1000, 1, 1024, 128, 0, 2)
    assert b >= 2 * 1000 * 1024 * 2 + 1000 * 8
    assert built_lib.seismic_xcorr_workspace_bytes(1000, 1, 1024, 300, 0, 2) == 0  # 2*shift > 512


def test_dropin_padding_matches_reference_rule():
    class Tr:
        def __init__(self, d):
            self.data = d
    rng = np.random.default_rng(0)
    evs = np.empty(3, dtype=object)
    for k, length in enumerate((300, 300, 250)):
        evs[k] = Tr(rng.standard_normal(length).astype(np.float32))
    n, length, p, padded = _dropin.pad_events(evs)
    assert (n, length, p) == (3, 300, 512)          # L from events[0], P = 1 << L.bit_length()
    np.testing.assert_array_equal(padded[2, :250], evs[2].data)
    assert np.all(padded[2, 250:] == 0)
    # a plain (N, L) array takes the vectorised path, same result
    plain = rng.standard_normal((4, 100)).astype(np.float32)
    n, length, p, padded = _dropin.pad_events(plain)
    assert (n, length, p) == (4, 100, 128)
    np.testing.assert_array_equal(padded[:, :100], plain)
    assert np.all(padded[:, 100:] == 0)


def test_cuda_dropin_imports_under_the_reference_module_name():
    """Correlation_in_CUDA/test_cuda.py:15 does ``from correlation_lib import
    compute_correlation, initialiseRunTime``: the CUDA drop-in must import
    under that name with its directory on sys.path, with the reference's
    signatures (Correlation_in_CUDA/correlation_lib.py:31,101)."""
    import inspect
    spec = importlib.util.spec_from_file_location(
        "correlation_lib", os.path.join(ROOT, "seismic_gb300", "cuda", "correlation_lib.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    assert list(inspect.signature(mod.compute_correlation).parameters) == ["events", "shift", "num_threads",
                                                                            "threshold"]
    assert list(inspect.signature(mod.initialiseRunTime).parameters) == []
    assert callable(mod.initialise_library)


def test_packed_index():
    n = 7
    i, j = np.triu_indices(n)
    np.testing.assert_array_equal(xcorr.packed_index(i, j, n), np.arange(n * (n + 1) // 2))
    big = 100_000
    assert xcorr.packed_index(big - 1, big - 1, big) == big * (big + 1) // 2 - 1


def _band_tile(x, nb, band):
    """Python restatement of band_tile (pair_core.cuh): tile x of the upper
    triangle of nb x nb tiles in row bands of `band` tiles (0 = one band),
    each band column by column from its diagonal, top to bottom."""
    band = band if 0 < band <= nb else nb
    r0 = 0
    while True:
        re = min(r0 + band, nb)
        wb = re - r0
        tri = wb * (wb + 1) // 2
        cnt = tri + wb * (nb - re)
        if x < cnt or re >= nb:
            if x < tri:
                c = 0
                while (c + 1) * (c + 2) // 2 <= x:
                    c += 1
                return r0 + (x - c * (c + 1) // 2), r0 + c
            q, rem = divmod(x - tri, wb)
            return r0 + rem, re + q
        x -= cnt
        r0 = re


@pytest.mark.parametrize("nb,band", [(1, 0), (7, 0), (7, 3), (12, 5), (30, 4), (30, 30), (9, 1)])
def test_row_bands_are_contiguous_rows(nb, band):
    """Tiles of row band k are the consecutive tile indices from
    band_first_tile(k) (rows 0 .. r0 - 1 of the triangle before it) and hold
    exactly the tile rows of the band: the band's outputs are a contiguous
    range of packed rows (what the host entry point copies chunk by chunk)."""
    b = band if 0 < band <= nb else nb
    bands = (nb + b - 1) // b
    first = [min(k * b, nb) * nb - min(k * b, nb) * (min(k * b, nb) - 1) // 2 for k in range(bands + 1)]
    assert first[-1] == nb * (nb + 1) // 2
    for k in range(bands):
        rows = {_band_tile(x, nb, band)[0] for x in range(first[k], first[k + 1])}
        assert rows == set(range(k * b, min((k + 1) * b, nb)))


def _scheduler_pairs(n, tile, band=0):
    """Python restatement of the direct pair kernel's work decomposition
    (band_tile + couple split in pairs.cu) to check coverage."""
    nb = (n + tile - 1) // tile
    return _scheduler_pairs_range(n, tile, 0, nb * (nb + 1) // 2 * (tile * tile // 2), band)


def _scheduler_pairs_range(n, tile, begin, end, band=0):
    """Pairs produced by work items [begin, end) of the triangle of n events."""
    nb = (n + tile - 1) // tile
    cpt = tile * tile // 2
    seen = []
    for w in range(begin, end):
        tl, lc = divmod(w, cpt)
        bi, bj = _band_tile(tl, nb, band)
        ii, jj = divmod(2 * lc, tile)
        i = bi * tile + ii
        for j in (bj * tile + jj, bj * tile + jj + 1):
            if i < n and j < n and j >= i:
                seen.append((i, j))
    return seen


@pytest.mark.parametrize("n,tile,band", [(1, 8, 0), (2, 8, 0), (13, 8, 0), (37, 4, 0), (64, 8, 0), (9, 2, 0),
                                         (50, 2, 0), (37, 4, 3), (64, 8, 1), (50, 2, 7)])
def test_scheduler_covers_triangle_exactly_once(n, tile, band):
    seen = _scheduler_pairs(n, tile, band)
    assert len(seen) == len(set(seen)) == n * (n + 1) // 2


def _staged_pairs(n, t, band, begin=0, end=None):
    """Pairs written by items [begin, end) of the staged form with one i per
    item (TI = 1 in staged_core.cuh): item w is tile w // t in band order and
    its row w % t; group g takes j0 + 2g and j0 + 2g + 1, t = 2 * groups."""
    nb = (n + t - 1) // t
    end = t * nb * (nb + 1) // 2 if end is None else end
    seen = []
    for w in range(begin, end):
        bi, bj = _band_tile(w // t, nb, band)
        i, j0 = bi * t + w % t, bj * t
        for j in range(j0, j0 + t):
            if i < n and j < n and j >= i:
                seen.append((i, j))
    return seen


@pytest.mark.parametrize("n,t,band", [(1, 6, 0), (5, 6, 0), (37, 6, 0), (37, 6, 2), (100, 12, 1), (100, 12, 3),
                                      (97, 24, 2), (300, 48, 2), (61, 6, 4)])
def test_staged_scheduler_covers_triangle_exactly_once(n, t, band):
    seen = _staged_pairs(n, t, band)
    assert len(seen) == len(set(seen)) == n * (n + 1) // 2


def _staged_geom(ng, ti):
    """Item geometry of the staged form (staged_core.cuh staged_geom): TI i
    events x TJ = 2 ng / TI j events, square tiles of TS = lcm(TI, TJ)."""
    tj = 2 * ng // ti
    ts = ti // math.gcd(ti, tj) * tj
    jpt = ts // tj
    return ti, tj, ts, jpt, (ts // ti) * jpt


def _staged_geom_pairs(n, ng, ti, band, begin=0, end=None):
    """Pairs written by items [begin, end) of the triangle (staged_decode):
    item w is tile w // ipt in band order, item k = w % ipt at tile row
    k // jpt and column k % jpt; group g takes i0 + g // (TJ/2) and the
    couple j0 + 2 (g % (TJ/2)), +1."""
    ti, tj, ts, jpt, ipt = _staged_geom(ng, ti)
    nb = (n + ts - 1) // ts
    end = ipt * nb * (nb + 1) // 2 if end is None else end
    seen = []
    for w in range(begin, end):
        x, k = divmod(w, ipt)
        bi, bj = _band_tile(x, nb, band)
        i0, j0 = bi * ts + (k // jpt) * ti, bj * ts + (k % jpt) * tj
        for g in range(ng):
            gi, gc = divmod(g, tj // 2)
            for j in (j0 + 2 * gc, j0 + 2 * gc + 1):
                if i0 + gi < n and j < n and j >= i0 + gi:
                    seen.append((i0 + gi, j))
    return seen


@pytest.mark.parametrize("n,ng,ti,band", [(1, 24, 6, 0), (7, 24, 6, 0), (203, 24, 6, 2), (203, 30, 6, 3),
                                          (100, 15, 5, 1), (61, 3, 3, 4), (90, 7, 7, 2), (50, 6, 3, 0),
                                          (77, 12, 4, 5), (33, 24, 1, 2), (45, 12, 12, 1)])
def test_staged_items_cover_triangle_exactly_once(n, ng, ti, band):
    """TI x TJ work items (any TI dividing the group count) write every pair
    of the triangle once, and the items of row band k (band_first_tile(k) x
    items per tile onwards) write exactly the band's packed rows, which the
    host entry point copies back chunk by chunk."""
    seen = _staged_geom_pairs(n, ng, ti, band)
    assert len(seen) == len(set(seen)) == n * (n + 1) // 2
    _, _, ts, _, ipt = _staged_geom(ng, ti)
    nb = (n + ts - 1) // ts
    b = band if 0 < band <= nb else nb
    for k in range((nb + b - 1) // b):
        r0, r1 = min(k * b, nb), min((k + 1) * b, nb)
        first = lambda r: r * nb - r * (r - 1) // 2
        rows = {i for i, _ in _staged_geom_pairs(n, ng, ti, band, first(r0) * ipt, first(r1) * ipt)}
        assert rows == set(range(r0 * ts, min(r1 * ts, n)))


@pytest.mark.parametrize("nq,ncols,ng,ti", [(1, 50, 24, 1), (7, 113, 24, 2), (7, 113, 24, 3), (64, 200, 15, 5),
                                            (5, 9, 6, 3), (13, 31, 30, 6)])
def test_staged_rect_items_cover_rectangle_exactly_once(nq, ncols, ng, ti):
    """Rectangle items: column block w // ceil(nq / TI) of TJ catalog events,
    query block w % that of TI queries (queries past the last are idle)."""
    ti, tj, _, _, _ = _staged_geom(ng, ti)
    nqb = (nq + ti - 1) // ti
    seen = []
    for w in range(nqb * ((ncols + tj - 1) // tj)):
        blk, qb = divmod(w, nqb)
        for g in range(ng):
            gi, gc = divmod(g, tj // 2)
            i, ja = qb * ti + gi, blk * tj + 2 * gc
            if i < nq and ja < ncols:
                seen.append((i, ja))
                if ja + 1 < ncols:
                    seen.append((i, ja + 1))
    assert len(seen) == len(set(seen)) == nq * ncols


def test_staged_item_row_division():
    """A group's item row g // (TJ/2) as (g * ceil(2^16 / (TJ/2))) >> 16."""
    for d in range(1, 65):
        m = (65536 + d - 1) // d
        assert all((g * m) >> 16 == g // d for g in range(64))


def test_non_power_of_two_padded_sizes(built_lib):
    """A padded size that is not a power of two but holds the lag window
    (the circular series is then the linear one) gets the workspace of the
    next power of two; an aliasing one is refused."""
    ws = built_lib.seismic_xcorr_workspace_bytes
    assert ws(8, 1, 1000, 1000, 3000, 0) == ws(8, 1, 1000, 1000, 4096, 0) > 0
    assert ws(8, 1, 1000, 1000, 1999, 0) == 0       # 1000 + 1000 > 1999: aliasing
    assert ws(8, 3, 700, 300, 1000, 0) == ws(8, 3, 700, 300, 1024, 0) > 0


def test_native_api_rejects_bad_sizes_without_gpu(built_lib):
    """Argument validation runs before any CUDA call."""
    st = built_lib.seismic_xcorr_host(ctypes.c_void_p(1), 4, 1, 100, 100, 100, 96, 10, 0.0, 0, 0,
                                      ctypes.c_void_p(1), ctypes.c_void_p(1), ctypes.c_void_p(1),
                                      ctypes.c_void_p(1), None, None)
    assert st == 2  # unsupported padded size
    assert b"unsupported" in built_lib.seismic_last_error_message()
    st = built_lib.seismic_xcorr_host(ctypes.c_void_p(1), 0, 1, 100, 100, 100, 128, 10, 0.0, 0, 0,
                                      ctypes.c_void_p(1), ctypes.c_void_p(1), ctypes.c_void_p(1),
                                      ctypes.c_void_p(1), None, None)
    assert st == 1
