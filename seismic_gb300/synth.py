"""Seeded synthetic seismic waveforms.

The reference's own dataset (``events_eruption_v8.npy``, loaded by every driver,
e.g. Correlation_in_OMP/test_c.py:27) is not distributed, so workloads are
built from seeded generators with the shapes and value distributions of the
five workloads this library is measured on:

* ``ricker_catalog``  -- Ricker wavelets, centre frequency U(2, 10) Hz at
  100 Hz sampling, onset jitter U(+-50) samples, amplitude log-uniform in
  [0.1, 10], random polarity, white noise at SNR U(5, 20) dB.
* ``family_catalog``  -- events grouped in families; each family shares a
  band-limited (2-15 Hz) Gaussian-noise template with cosine tapers of up to
  400 samples; members are time-shifted U(+-100) samples, amplitude-scaled,
  polarity-flipped, perturbed by 10 % independent band-limited noise and
  buried in white noise at SNR U(0, 20) dB.

All arrays are float32, shaped (N, C, L).
"""
from __future__ import annotations

import numpy as np

FS_HZ = 100.0


def ricker_catalog(n_events: int, length: int, seed: int = 1, n_channels: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    t = (np.arange(length) - length / 2.0) / FS_HZ
    out = np.empty((n_events, n_channels, length), np.float32)
    for e in range(n_events):
        for c in range(n_channels):
            f = rng.uniform(2.0, 10.0)
            onset = rng.uniform(-50.0, 50.0) / FS_HZ
            amp = 10.0 ** rng.uniform(-1.0, 1.0)
            pol = 1.0 if rng.random() < 0.5 else -1.0
            tt = t - onset
            a = (np.pi * f * tt) ** 2
            w = (1.0 - 2.0 * a) * np.exp(-a) * amp * pol
            snr_db = rng.uniform(5.0, 20.0)
            rms = np.sqrt(np.mean(w * w))
            noise = rng.standard_normal(length) * rms / (10.0 ** (snr_db / 20.0))
            out[e, c] = (w + noise).astype(np.float32)
    return out


def _bandpass_noise(rng, shape, length, lo=2.0, hi=15.0):
    x = rng.standard_normal(tuple(shape) + (length,))
    spec = np.fft.rfft(x, axis=-1)
    f = np.fft.rfftfreq(length, d=1.0 / FS_HZ)
    spec[..., (f < lo) | (f > hi)] = 0.0
    y = np.fft.irfft(spec, n=length, axis=-1)
    y /= np.sqrt(np.mean(y * y, axis=-1, keepdims=True)) + 1e-30
    return y


def _taper(length, width=400):
    w = min(width, length // 4)
    tap = np.ones(length)
    if w > 0:
        ramp = 0.5 - 0.5 * np.cos(np.pi * np.arange(w) / w)
        tap[:w] = ramp
        tap[length - w:] = ramp[::-1]
    return tap


def family_catalog(n_events: int, n_channels: int, length: int, n_families: int | None = None,
                   seed: int = 2) -> np.ndarray:
    """Family-based generator; ``n_families`` defaults to max(1, N // 32)."""
    rng = np.random.default_rng(seed)
    if n_families is None:
        n_families = max(1, n_events // 32)
    tap = _taper(length)
    templates = _bandpass_noise(rng, (n_families, n_channels), length) * tap
    fam = rng.integers(0, n_families, size=n_events)
    shifts = np.clip(rng.integers(-100, 101, size=n_events), -(length // 2), length // 2)
    amp = 10.0 ** rng.uniform(-0.5, 0.5, size=n_events)
    pol = np.where(rng.random(n_events) < 0.5, -1.0, 1.0)
    snr_db = rng.uniform(0.0, 20.0, size=n_events)
    out = np.empty((n_events, n_channels, length), np.float32)
    # 10 % waveform perturbation: band-limited traces drawn from a bank of
    # 64 per catalog, each use with its own circular shift and sign
    bank = (_bandpass_noise(rng, (min(64, n_events), n_channels), length) * tap).astype(np.float32)
    bank2 = np.concatenate([bank, bank], axis=-1)                  # circular windows by slicing
    windows = np.lib.stride_tricks.sliding_window_view(bank2, length, axis=-1)  # (K, C, 2L-?, L)
    # templates shifted by s in [-L/2, L/2] with zero fill: slice a zero-padded copy
    half = length // 2
    tpad = np.zeros((n_families, n_channels, length + 2 * half), np.float32)
    tpad[:, :, half:half + length] = templates
    twin = np.lib.stride_tricks.sliding_window_view(tpad, length, axis=-1)     # (F, C, 2*half+1, L)
    block = 2048
    for s in range(0, n_events, block):
        e = np.arange(s, min(n_events, s + block))
        # event shifted right by sh: x[t] = template[t - sh]  ->  window starting at half - sh
        shifted = twin[fam[e], :, half - shifts[e], :]                 # (B, C, L)
        pick = rng.integers(0, bank.shape[0], size=e.size)
        roll = rng.integers(0, length, size=e.size)
        sign = np.where(rng.random(e.size) < 0.5, -1.0, 1.0).astype(np.float32)
        pert = windows[pick, :, roll, :] * sign[:, None, None]
        sig = shifted + np.float32(0.1) * pert
        sig *= (amp[e] * pol[e]).astype(np.float32)[:, None, None]
        rms = np.sqrt(np.mean(sig * sig, axis=-1, keepdims=True))
        scale = (rms / (10.0 ** (snr_db[e] / 20.0))[:, None, None]).astype(np.float32)
        noise = rng.standard_normal(sig.shape, dtype=np.float32)
        noise *= scale
        out[e] = sig + noise
    return out


WORKLOADS = {
    # name: (description, builder kwargs)
    "small": dict(kind="ricker", n_events=200, n_channels=1, length=512, shift=512, seed=11),
    "scale": dict(kind="family", n_events=4096, n_channels=3, length=2048, shift=2048,
                  n_families=32, seed=12),
    "precision": dict(kind="family", n_events=16384, n_channels=1, length=1024, shift=128,
                      n_families=128, seed=13),
}


def make_workload(name: str, n_events: int | None = None) -> tuple[np.ndarray, int]:
    """Events (N, C, L) and lag half-window ``shift`` of a named workload;
    ``n_events`` overrides N (for bounded samples and small test cases)."""
    w = WORKLOADS[name]
    n = n_events if n_events is not None else w["n_events"]
    if w["kind"] == "ricker":
        ev = ricker_catalog(n, w["length"], seed=w["seed"], n_channels=w["n_channels"])
    else:
        ev = family_catalog(n, w["n_channels"], w["length"],
                            n_families=max(1, min(w["n_families"], n // 32 or 1)), seed=w["seed"])
    return ev, w["shift"]


def _family_job(job):
    n, c, length, seed = job
    return family_catalog(n, c, length, n_families=max(1, n // 32), seed=seed)


def _pool_map(jobs):
    """family_catalog over jobs in a spawn-context process pool (each job has
    its own seed, so the result does not depend on the pool)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import os
    workers = max(1, min(16, len(os.sched_getaffinity(0)), len(jobs)))
    if workers == 1:
        return [_family_job(j) for j in jobs]
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_family_job, jobs, chunksize=4))


def batched_catalogs(n_catalogs: int = 256, seed: int = 4000) -> list[tuple[np.ndarray, int]]:
    """The batched workload: independent catalogs with N log-uniform in
    16..2048, L from {256, 512, 1000, 2048, 3000, 4096}, 1 or 3 channels,
    families = max(1, N // 32), full lag range (shift = L).  Returns
    [(events (N, C, L), shift)]."""
    rng = np.random.default_rng(seed)
    lengths = [256, 512, 1000, 2048, 3000, 4096]
    jobs = []
    for k in range(n_catalogs):
        n = int(round(np.exp(rng.uniform(np.log(16), np.log(2048)))))
        length = int(rng.choice(lengths))
        c = int(rng.choice([1, 3]))
        jobs.append((n, c, length, seed + 1 + k))
    return [(ev, job[2]) for ev, job in zip(_pool_map(jobs), jobs)]


def serving_catalog(n_events: int = 50000, seed: int = 9000) -> np.ndarray:
    """The serving workload's resident catalog: family events of 3 channels
    x 1024 samples, generated in blocks of 2500 (block b seeded seed + b)."""
    jobs = [(min(2500, n_events - b), 3, 1024, seed + b) for b in range(0, n_events, 2500)]
    return np.concatenate(_pool_map(jobs))
