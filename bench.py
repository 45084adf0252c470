"""Throughput benchmark of the all-pairs normalised cross-correlation.

One step = the whole hot path over one catalog already resident in HBM:
kernel (a) (spectra + FP64 norms of every event/channel) then kernel (b)
(every pair of the upper triangle: conj-products, inverse FFT, window
max/min, normalisation, histograms, threshold, packed outputs).

Default workload ("precision"): N=16384 events, 1 channel, L=1024 float32
samples, lags -127..128 (padded size 2048), FP32 fused FFT form, seeded
family-based synthetic waveforms (128 families).  The same line carries the
reduced-precision forms of that workload (the tensor-core lag-GEMM with one
FP16 product and with three BF16 hi/lo products) at full size: their
pairs/s, end-to-end pairs/s, FP64 error and lag agreement, roofline
fraction and ratio to the FP32 form.  Other workloads: --workload scale
(N=4096, 3 channels, L=2048, full lags), --workload small (N=200, L=512,
full lags), --workload batched, --workload serving.

Prints ONE JSON line (rank 0).  With --impl reference the CPU path of the
reference (its OpenMP source where it was built here, else the C
restatement of it) is timed on the host cores on a bounded sample of the
same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from seismic_gb300 import synth  # noqa: E402

METRIC = "normalized xcorr pairs/sec at stated FP64-oracle error"
WORKLOAD_TEXT = {
    "scale": "N=4096 events x 3 channels x L=2048 float32, lags -2047..2048, padded FFT 4096, FP32 fused FFT form",
    "precision": "N=16384 events x 1 channel x L=1024 float32, lags -127..128, padded FFT 2048, FP32 fused FFT form",
    "small": "N=200 events x 1 channel x L=512 float32 (Ricker), lags -511..512, padded FFT 1024, FP32 fused FFT form",
    "serving": "50,000-event resident catalog x 3 channels x L=1024, lags -255..256, Poisson query stream "
               "(1..64 events of 256..1024 samples per request)",
    "batched": "256 independent catalogs, N log-uniform in 16..2048, L in {256,512,1000,2048,3000,4096}, "
               "1 or 3 channels, full lag range each, padded FFT = next power of two >= 2L, FP32 fused FFT form, "
               "one captured CUDA graph (a spectra launch + one persistent pair launch over every FFT size)",
}
CPU_SAMPLE_EVENTS = {"scale": 640, "precision": 1024, "small": 200}
FORM_TEXT = {"fp32": "FP32 fused FFT form", "fp16": "FP16-spectra fused FFT form",
             "bf16": "BF16-spectra fused FFT form",
             "laggemm": "tensor-core lag-GEMM form (BF16 hi/lo, three products, FP32 accumulation)",
             "laggemm16": "tensor-core lag-GEMM form (FP16 samples scaled by 1/norm, one product, FP32 accumulation)"}


def workload_text(workload: str, form: str) -> str:
    """Workload description with the form that ran it (the lag-GEMM forms use
    no padded FFT)."""
    text = WORKLOAD_TEXT[workload]
    if "FP32 fused FFT form" not in text:
        return text
    if form.startswith("laggemm"):
        text = text.split(", padded FFT")[0]
    else:
        text = text.replace(", FP32 fused FFT form", "")
    return text + ", " + FORM_TEXT.get(form, form)


def pair_kernel_name(p: int, c: int) -> str:
    """The pair form the library dispatches for FP32 spectra of size p, c channels."""
    if os.environ.get("SEISMIC_PAIR_KERNEL") == "direct":
        return "pair_kernel (direct-load form)"
    if 512 <= p <= 4096:
        return "staged_pair_kernel (TMA-staged form)"
    return "pair_kernel (direct-load form)"


def fft_flops_per_pair(p: int, c: int) -> float:
    """Algorithmic work per pair of the FFT form: one size-P inverse FFT
    (2.5 P log2 P) plus C conj-products of P/2+1 bins (6 flops each)."""
    return 2.5 * p * np.log2(p) + 6.0 * c * (p // 2 + 1)


def fft_plan(lib, length: int, shift: int, p: int, c: int, form_code: int) -> dict:
    """The transform the library runs for these sizes (seismic_fft_plan):
    the plain size-P form (blocks 0) or the overlap-save frames."""
    q, b, bl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    from seismic_gb300 import _lib
    _lib.check(lib.seismic_fft_plan(length, shift, p, c, form_code, ctypes.byref(q), ctypes.byref(b),
                                    ctypes.byref(bl)))
    return {"transform_size": q.value, "blocks": b.value, "block_length": bl.value}


def executed_flops_per_pair(plan: dict, p: int, c: int) -> float:
    """FLOPs per pair of the transform the kernel runs: the plain count, or
    one size-Q inverse FFT plus C x blocks conj-products of Q/2+1 bins."""
    if not plan or plan["blocks"] == 0:
        return fft_flops_per_pair(p, c)
    q = plan["transform_size"]
    return 2.5 * q * np.log2(q) + 6.0 * c * plan["blocks"] * (q // 2 + 1)


# arithmetic type of each form's products (accumulation is FP32 in all of them)
FORM_DTYPE = {"fp32": "f32", "fp16": "f16", "bf16": "bf16", "laggemm": "bf16x3 (hi+lo)", "laggemm16": "f16"}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", self.gpu_id], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "power_w_max": float(max(power)),
                "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------- FP64 check
def fp64_sample_error(ev: np.ndarray, shift: int, p: int, vp, lp, vn, ln, n_sample: int = 2000, seed: int = 0):
    """Max/mean |coef - FP64| and lag agreement on a random sample of pairs,
    FP64 computed here with numpy (mean over channels of the per-channel
    normalised circular correlation, lags 1-shift..shift, first maximum)."""
    n = ev.shape[0]
    rng = np.random.default_rng(seed)
    i = rng.integers(0, n, n_sample)
    j = rng.integers(0, n, n_sample)
    i, j = np.minimum(i, j), np.maximum(i, j)
    idx = i * n - i * (i - 1) // 2 + (j - i)
    x = ev.astype(np.float64)
    if x.ndim == 2:
        x = x[:, None, :]
    norms = np.sqrt((x * x).sum(-1))
    inv = np.where(norms > 0, 1.0 / np.where(norms > 0, norms, 1), 0.0)
    spec_i = np.fft.rfft(x[i], n=p, axis=-1) * inv[i][..., None]
    spec_j = np.fft.rfft(x[j], n=p, axis=-1) * inv[j][..., None]
    series = np.fft.irfft((spec_i * np.conj(spec_j)).mean(axis=1), n=p, axis=-1)
    lags = np.arange(1 - shift, shift + 1)
    s = series[:, np.mod(lags, p)]
    amax, amin = s.argmax(1), s.argmin(1)
    rvp = np.maximum(s.max(1), 0.0)
    rvn = np.minimum(s.min(1), 0.0)
    rlp = np.where(rvp > 0, lags[amax], 0)
    rln = np.where(rvn < 0, lags[amin], 0)
    top2 = np.partition(s, -2, axis=1)[:, -2:]
    bot2 = np.partition(s, 1, axis=1)[:, :2]
    gp, gn = top2[:, 1] - top2[:, 0], bot2[:, 1] - bot2[:, 0]
    e = np.concatenate([np.abs(vp[idx] - rvp), np.abs(vn[idx] - rvn)])
    mis = np.concatenate([(lp[idx] != rlp), (ln[idx] != rln)])
    exempt = np.concatenate([gp < 1e-6, gn < 1e-6])
    # a reduced-precision form can swap two peaks closer than its own error
    within = np.concatenate([gp, gn]) < 2 * e.max()
    return {"max_abs": float(e.max()), "mean_abs": float(e.mean()),
            "lag_agreement": float(1.0 - mis.mean()),
            "lag_mismatch_not_exempt": int((mis & ~exempt).sum()),
            "lag_mismatch_beyond_2x_max_err": int((mis & ~within).sum()), "pairs_sampled": int(n_sample)}


# ----------------------------------------------------------- CPU baseline
def cpu_baseline(workload: str, ev: np.ndarray, shift: int, n_sample: int | None = None, repeats: int = 1):
    """The reference's CPU path on a bounded sample of the workload: its own
    OpenMP source (built against the FFT shim) where available, else the C
    restatement; one single-channel call per channel, all host cores."""
    from oracle import oracle as O
    n_s = n_sample or CPU_SAMPLE_EVENTS[workload]
    sample = ev[:n_s]
    cores = len(os.sched_getaffinity(0))
    kind = "port"
    fn = O.port_correlation_cpp
    try:
        if O.ref_lib() is not None:
            kind, fn = "reference", O.ref_correlation_cpp
    except OSError:
        pass
    p = 1 << int(sample.shape[-1]).bit_length()
    c = sample.shape[1]
    chans = [np.ascontiguousarray(sample[:, ch]) for ch in range(c)]
    times = []
    sys.stdout.flush()
    saved = os.dup(1)
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)  # the reference's C code prints its parameters on stdout
    try:
        for _ in range(repeats):
            t0 = time.perf_counter()
            for x in chans:
                fn(x, shift, 0.0, 20, num_threads=cores, chunk_size=4, padded=p)
            times.append(time.perf_counter() - t0)
    finally:
        ctypes.CDLL(None).fflush(None)  # drain C stdio buffers while fd 1 is still /dev/null
        os.dup2(saved, 1)
        os.close(saved)
        os.close(devnull)
    pairs = n_s * (n_s + 1) // 2
    return {"value": pairs / float(np.median(times)), "unit": "pairs/s", "cores": cores, "kind": kind,
            "sample": f"first {n_s} events of the same workload ({pairs} pairs x {c} channel(s), "
                      f"one single-channel call per channel), median of {repeats}"}, times


# --------------------------------------------------------------- the arms
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return ws, rank, local


def run_reference(args):
    ws, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return
    if args.workload == "batched":  # a catalog of the batch where the reference is defined (power-of-two L)
        ev, shift = next((e, s) for e, s in batched_catalogs(64) if e.shape[-1] in (512, 2048) and e.shape[0] >= 200)
        CPU_SAMPLE_EVENTS["batched"] = min(ev.shape[0], 400)
        ev = ev[:CPU_SAMPLE_EVENTS["batched"]]
    elif args.workload == "serving":  # events of the serving shape: 3 x 1024, lags -255..256
        CPU_SAMPLE_EVENTS["serving"] = 400
        ev, shift = synth.family_catalog(400, 3, 1024, n_families=12, seed=9000), 256
    else:
        ev, shift = synth.make_workload(args.workload, n_events=CPU_SAMPLE_EVENTS[args.workload])
    for _ in range(args.warmup):
        cpu_baseline(args.workload, ev, shift)
    base, times = cpu_baseline(args.workload, ev, shift, repeats=args.steps)
    n_s = CPU_SAMPLE_EVENTS[args.workload]
    pairs = n_s * (n_s + 1) // 2
    ms = float(np.mean(times)) * 1e3
    out = {"metric": METRIC, "value": base["value"], "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "impl": "reference",
           "data": "synthetic: seeded family-based waveforms (no public dataset; the reference's is not distributed)",
           "config": {"workload": args.workload + ": " + WORKLOAD_TEXT[args.workload],
                      "cpu_sample_events": n_s, "pairs_per_step": pairs},
           "cpu_baseline": base, "e2e": {"value": base["value"], "unit": "pairs/s", "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def read_traffic(workload: str):
    path = os.path.join(ROOT, "profiles", "pair_kernel_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        f = dict(kv.split("=", 1) for kv in line.split() if "=" in kv)
        if f.get("workload") == workload and "dram_bytes_per_pair" in f:
            return float(f["dram_bytes_per_pair"])
    return None


class HostBuffers:
    """Pinned host copies of one workload's events and outputs, for the
    end-to-end measurement through seismic_xcorr_host (the C-ABI host call:
    H2D of the events, the kernels, D2H of the four packed outputs and the
    histograms, all inside the timed call)."""

    def __init__(self, ev: np.ndarray, npairs: int):
        import torch
        self.ev = torch.empty(ev.shape, dtype=torch.float32, pin_memory=True)
        self.ev.numpy()[...] = ev
        self.out = [torch.empty(npairs, dtype=torch.float32 if k % 2 == 0 else torch.int32, pin_memory=True)
                    for k in range(4)]
        self.hist = [np.zeros(20, np.int32), np.zeros(20, np.int32)]
        self.npairs = npairs
        self.h2d = int(ev.nbytes)

    def e2e(self, lib, n, c, length, padded, shift, form_code, steps, ws, dev):
        import torch
        from seismic_gb300 import _lib

        def host_call():
            _lib.check(lib.seismic_xcorr_host(self.ev.data_ptr(), n, c, length, c * length, length, padded, shift,
                                              0.0, 20, form_code, *(t.data_ptr() for t in self.out),
                                              self.hist[0].ctypes.data, self.hist[1].ctypes.data))
        torch.cuda.set_device(dev)
        host_call()
        walls = []
        for _ in range(max(3, min(steps, 10))):
            t0 = time.perf_counter()
            host_call()
            walls.append(time.perf_counter() - t0)
        e2e_t = float(np.median(walls))  # per-call wall time: median of the calls (mean and min beside it)
        if ws > 1:
            import torch.distributed as dist
            tt = torch.tensor([e2e_t], device=dev, dtype=torch.float64)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            e2e_t = float(tt.item())
        self.walls_ms = [round(w * 1e3, 3) for w in walls]
        return {"value": ws * self.npairs / e2e_t, "unit": "pairs/s", "h2d_bytes_per_step": self.h2d,
                "d2h_bytes_per_step": int(4 * 4 * self.npairs + 2 * 20 * 4),
                "entry_point": "seismic_xcorr_host (C ABI), pinned host buffers, wall clock per call (median)",
                "call_ms": {"median": e2e_t * 1e3, "mean": float(np.mean(walls)) * 1e3,
                            "min": float(np.min(walls)) * 1e3, "calls": len(walls)}}


def measure_lag_form(lib, form, d_ev, ev, shift, outs, hist, flush, stream, args, dev, peaks, fp32_value, host, ws,
                     clocks=None):
    """One reduced-precision form of the same workload at full size: the
    tensor-core lag-GEMM (prep + lag_gemm_kernel) timed with CUDA events on
    its stream over the same number of steps, L2 flushed between steps; FP64
    error on a sample of pairs; end to end through seismic_xcorr_host."""
    import torch
    from seismic_gb300 import _lib
    n, c, length = ev.shape
    npairs = n * (n + 1) // 2
    code = _lib.FORMS[form]
    wsb = lib.seismic_xcorr_workspace_bytes(n, c, length, shift, 0, code)
    if wsb == 0:
        return {"unavailable": f"form {form} does not support this workload"}
    lag_ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    vp, lp, vn, ln = outs

    def call(stage):  # 1: prep (16-bit planes + FP64 norms), 2: the lag-GEMM
        _lib.check(lib.seismic_xcorr_device_stages(d_ev.data_ptr(), n, c, length, c * length, length, 0, shift, 0.0,
                                                   20, code, vp.data_ptr(), lp.data_ptr(), vn.data_ptr(),
                                                   ln.data_ptr(), hist[0].data_ptr(), hist[1].data_ptr(),
                                                   lag_ws.data_ptr(), wsb, ctypes.c_void_p(stream.cuda_stream),
                                                   stage))
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            call(1)
            call(2)
    torch.cuda.synchronize(dev)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(3 * args.steps)]
    launches0 = lib.seismic_launch_count()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            hist.zero_()
            evs[3 * k].record(stream)
            call(1)
            evs[3 * k + 1].record(stream)
            call(2)
            evs[3 * k + 2].record(stream)
    torch.cuda.synchronize(dev)
    launches = lib.seismic_launch_count() - launches0
    t = np.array([evs[3 * k].elapsed_time(evs[3 * k + 2]) for k in range(args.steps)]) * 1e-3
    t_gemm = float(np.mean([evs[3 * k + 1].elapsed_time(evs[3 * k + 2]) for k in range(args.steps)])) * 1e-3
    step = float(t.mean())
    if ws > 1:
        import torch.distributed as dist
        tt = torch.tensor([step], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        step = float(tt.item())
    value = ws * npairs / step
    p_lin = xcorr_padded(length, shift)
    fp64 = fp64_sample_error(ev, shift, p_lin, vp.cpu().numpy(), lp.cpu().numpy(), vn.cpu().numpy(),
                             ln.cpu().numpy(), n_sample=4000)
    flops = npairs * c * 2.0 * length * (2 * shift)
    achieved = flops / t_gemm / 1e12
    peak = peaks.get("bf16_tflops_sustained", 1700.0)
    products = 3 if form == "laggemm" else 1
    out = {"form": FORM_TEXT[form], "dtype": FORM_DTYPE[form], "value": value, "unit": "pairs/s",
           "ms_per_step": step * 1e3, "ratio_to_fp32_form": value / fp32_value if fp32_value else None,
           "fp64_error": fp64,
           "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                        "frac": achieved / peak, "tensor_products_per_lag_sum": products,
                        "issued_frac": products * achieved / peak,
                        "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (of measured): a kernel timed "
                                       "inside a step of tens of ms" if "bf16_tflops_sustained" in peaks
                        else "fallback 1.7 PFLOP/s sustained",
                        "kernel": "lag_gemm_kernel, timed alone", "kernel_ms": t_gemm * 1e3,
                        "kernel_share_of_step": t_gemm / step,
                        "work": f"{npairs} pairs x {c} ch x 2 L (2 shift) flop, L={length}, shift={shift}"},
           "gpu_launches": int(launches), "e2e": None}
    out["clocks"] = clocks.stop() if clocks is not None else None  # the timed region only
    if host is not None:
        out["e2e"] = host.e2e(lib, n, c, length, 0, shift, code, args.steps, ws, dev)
    del lag_ws
    return out


def run_ours(args):
    import torch
    from seismic_gb300 import _lib

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.lib()
    ev, shift = synth.make_workload(args.workload, n_events=args.n_events)
    if ws > 1:  # weak scaling: every rank its own catalog of the same shape
        ev = synth.family_catalog(ev.shape[0], ev.shape[1], ev.shape[2], seed=1000 + rank) \
            if args.workload != "small" else ev
    n, c, length = ev.shape
    p = 1 << int(length).bit_length()
    npairs = n * (n + 1) // 2
    rows = n * c

    d_ev = torch.from_numpy(ev).to(dev)
    vp = torch.empty(npairs, dtype=torch.float32, device=dev)
    lp = torch.empty(npairs, dtype=torch.int32, device=dev)
    vn = torch.empty(npairs, dtype=torch.float32, device=dev)
    ln = torch.empty(npairs, dtype=torch.int32, device=dev)
    hist = torch.zeros(2, 20, dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2
    stream = torch.cuda.Stream(dev)
    sh = ctypes.c_void_p(stream.cuda_stream)

    form_code = _lib.FORMS[args.form]
    lag = args.form.startswith("laggemm")
    p_arg = 0 if lag else p
    wsb = lib.seismic_xcorr_workspace_bytes(n, c, length, shift, p_arg, form_code)
    if wsb == 0:
        raise SystemExit(f"form {args.form} does not support this workload")
    ws_t = torch.empty(wsb, dtype=torch.uint8, device=dev)
    plan = None if lag else fft_plan(lib, length, shift, p, c, form_code)

    # the two halves of seismic_xcorr_device, timed apart: kernel (a) (spectra
    # + FP64 norms, or the lag form's planes) and kernel (b) (all pairs)
    def stage_call(stage):
        _lib.check(lib.seismic_xcorr_device_stages(d_ev.data_ptr(), n, c, length, c * length, length, p_arg, shift,
                                                   0.0, 20, form_code, vp.data_ptr(), lp.data_ptr(), vn.data_ptr(),
                                                   ln.data_ptr(), hist[0].data_ptr(), hist[1].data_ptr(),
                                                   ws_t.data_ptr(), wsb, sh, stage))

    def spectra_call():
        stage_call(1)

    def pairs_call():
        stage_call(2)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            hist.zero_()
            spectra_call()
            pairs_call()
    torch.cuda.synchronize(dev)

    gpu_id = "0"
    try:
        props = torch.cuda.get_device_properties(dev)
        gpu_id = f"{props.pci_domain_id:08x}:{props.pci_bus_id:02x}:{props.pci_device_id:02x}.0"
    except Exception:
        gpu_id = str(local)
    clocks = ClockSampler(gpu_id)
    ev_s = [torch.cuda.Event(enable_timing=True) for _ in range(3 * args.steps)]
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    launches0 = lib.seismic_launch_count()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()                      # L2 flush between steps, outside the timed events
            hist.zero_()
            ev_s[3 * k].record(stream)
            spectra_call()
            ev_s[3 * k + 1].record(stream)
            pairs_call()
            ev_s[3 * k + 2].record(stream)
    torch.cuda.synchronize(dev)
    launches = lib.seismic_launch_count() - launches0
    clk = clocks.stop()
    t_spec = np.array([ev_s[3 * k].elapsed_time(ev_s[3 * k + 1]) for k in range(args.steps)]) * 1e-3
    t_pair = np.array([ev_s[3 * k + 1].elapsed_time(ev_s[3 * k + 2]) for k in range(args.steps)]) * 1e-3
    t_step = t_spec + t_pair
    step_mean = float(t_step.mean())
    if ws > 1:
        import torch.distributed as dist
        tt = torch.tensor([step_mean], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        step_mean = float(tt.item())
    value = ws * npairs / step_mean

    fp64 = fp64_sample_error(ev, shift, p, vp.cpu().numpy(), lp.cpu().numpy(), vn.cpu().numpy(),
                             ln.cpu().numpy())

    # ---- end-to-end through the public host entry point, pinned host buffers
    e2e = None
    host = None
    if not args.skip_e2e:
        host = HostBuffers(ev, npairs)
        e2e = host.e2e(lib, n, c, length, p if args.form == "fp32" else 0, shift, form_code, args.steps, ws, dev)

    # ---- roofline of the dominant kernel
    t_pair_mean = float(t_pair.mean())
    traffic_pp = read_traffic(args.workload + ("" if args.form == "fp32" else "/" + args.form))
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        peaks = {}
    if not args.form.startswith("laggemm"):  # FFT forms: pair kernel on the FP32 pipe
        flops = npairs * fft_flops_per_pair(p, c)
        achieved_tf = flops / t_pair_mean / 1e12
        sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
        sm_mhz = clk.get("sm_mhz") or 2070.0
        peak_tf = sm_count * 128 * 2 * sm_mhz * 1e6 / 1e12
        executed_tf = npairs * executed_flops_per_pair(plan, p, c) / t_pair_mean / 1e12
        roofline = {"bound": "fp32", "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
                    "frac": achieved_tf / peak_tf,
                    "traffic": (traffic_pp * npairs) if traffic_pp is not None else None,
                    "kernel": pair_kernel_name(p, c),
                    "peak_source": f"nominal FP32 FMA rate: {sm_count} SMs x 128 lanes x 2 flop x median SM clock "
                                   f"{sm_mhz:.0f} MHz under load (MEASURED_PEAKS.json has no FP32 figure)",
                    "work": f"{npairs} pairs x (2.5 P log2 P + 6 C (P/2+1)) flop, P={p}, C={c} (the reference's "
                            "size-P transform per pair, counted whatever transform runs)",
                    "transform": plan,
                    "executed_work": "as work" if not plan["blocks"] else
                    f"{npairs} pairs x (2.5 Q log2 Q + 6 C nb (Q/2+1)) flop, Q={plan['transform_size']}, "
                    f"nb={plan['blocks']} overlap-save frames of {plan['block_length']} samples",
                    "executed_achieved": executed_tf, "executed_frac": executed_tf / peak_tf,
                    "pair_kernel_ms": t_pair_mean * 1e3, "pair_kernel_share_of_step": t_pair_mean / step_mean}
    else:  # lag-GEMM: tensor pipe; algorithmic work 2 L (2 shift) per channel-pair, hi/lo extras not counted
        flops = npairs * c * 2.0 * length * (2 * shift)
        achieved_tf = flops / t_pair_mean / 1e12
        peak_tf = peaks.get("bf16_tflops", 1900.0)
        roofline = {"bound": "tensor", "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
                    "frac": achieved_tf / peak_tf,
                    "traffic": (traffic_pp * npairs) if traffic_pp is not None else None,
                    "kernel": "lag_gemm_kernel (timed alone; lag_prep_kernel is the step's other launch)",
                    "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst) of measured" if "bf16_tflops" in peaks
                    else "fallback 1.9 PFLOP/s",
                    "work": f"{npairs} pairs x {c} ch x 2 L (2 shift) flop, L={length}, shift={shift}; "
                            + ("the three BF16 hi/lo products issue 3x this on the tensor pipe"
                               if args.form == "laggemm" else "one FP16 product per lag sum"),
                    "pair_kernel_ms": t_pair_mean * 1e3, "pair_kernel_share_of_step": t_pair_mean / step_mean}
    # kernel (a): samples in, spectra (plain, or A + W frames) and 16 B of norms out
    spec_out = (p // 2) * 8 if not plan or not plan["blocks"] else 2 * plan["blocks"] * (plan["transform_size"] // 2) * 8
    spec_bytes = rows * (length * 4 + spec_out + 16)
    spectra_roof = None
    if args.form == "fp32":
        spectra_roof = {"bound": "hbm", "achieved": spec_bytes / float(t_spec.mean()) / 1e9, "unit": "GB/s",
                        "ms": float(t_spec.mean()) * 1e3, "bytes": int(spec_bytes)}
        spectra_roof["peak"] = peaks.get("hbm_gbs", 6800.0)
        spectra_roof["frac"] = spectra_roof["achieved"] / spectra_roof["peak"]
        if "hbm_gbs" not in peaks:
            spectra_roof["peak_source"] = "fallback"

    out = {"metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": step_mean * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": FORM_DTYPE.get(args.form, "f32"),
           "data": "synthetic: seeded family-based waveforms (no public dataset; the reference's is not distributed)",
           "config": {"workload": args.workload + ": " + workload_text(args.workload, args.form), "n_events": n,
                      "n_channels": c, "event_length": length, "shift": shift, "padded_size": p,
                      "pairs_per_step": npairs, "form": args.form, "transform": plan,
                      "l2": "L2 flushed (256 MB write) between timed steps; spectra > L2 for this workload"
                      if rows * p * 4 > 129e6 else "L2 flushed (256 MB write) between timed steps"},
           "fp64_error": fp64, "roofline": roofline, "spectra_kernel": spectra_roof, "e2e": e2e,
           "clocks": clk, "gpu_launches": int(launches)}
    if args.workload == "precision" and args.form == "fp32" and not args.no_extra_forms:
        # the reduced-precision forms of the same workload, full size, same outputs buffers
        forms = {}
        for form in ("laggemm16", "laggemm"):
            clocks_f = ClockSampler(gpu_id)
            clocks_f.start()
            forms[form] = measure_lag_form(lib, form, d_ev, ev, shift, (vp, lp, vn, ln), hist, flush, stream, args,
                                           dev, peaks, value, host, ws, clocks_f)
        best = max((f for f in forms.values() if "value" in f), key=lambda f: f["value"], default=None)
        out["reduced_precision_forms"] = forms
        if best is not None:
            fe = best["fp64_error"]
            out["precision_target"] = {
                "rule": "reduced-precision form >= 3x the FP32 fused form at N=16384, L=1024, +-128 lags, "
                        "coefficient error <= 1e-3 vs FP64, lag agreement >= 0.999",
                "form": best["form"], "ratio": best["value"] / value,
                "max_abs_err": fe["max_abs"], "lag_agreement": fe["lag_agreement"],
                "met": bool(best["value"] / value >= 3.0 and fe["max_abs"] <= 1e-3 and fe["lag_agreement"] >= 0.999)}
    if rank == 0 and not args.no_cpu_baseline:
        base, _ = cpu_baseline(args.workload, ev, shift, repeats=5)  # about 1-4 s of host work
        out["cpu_baseline"] = base
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def batched_catalogs(n_catalogs: int = 256, seed: int = 4000):
    """Seeded catalogs of the batched workload: [(events (N, C, L), shift)]."""
    return synth.batched_catalogs(n_catalogs, seed)


def run_batched(args):
    import torch
    from seismic_gb300 import _lib
    from seismic_gb300.batch import Batch

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.lib()
    t_gen = time.perf_counter()
    cats = batched_catalogs(seed=4000 + 1000 * rank)
    t_gen = time.perf_counter() - t_gen
    tens = [torch.from_numpy(ev).to(dev) for ev, _ in cats]
    b = Batch(tens, [s for _, s in cats], n_classes_hist=20, use_graph=True, per_size=args.batch_per_size)
    npairs = b.pairs
    flops = 0.0
    for ev, shift in cats:
        n, c, length = ev.shape
        p = xcorr_padded(length, shift)
        flops += n * (n + 1) / 2 * fft_flops_per_pair(p, c)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)
    for _ in range(args.warmup):
        b.run(stream)
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(_gpu_id(dev, local))
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps)]
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    launches0 = lib.seismic_launch_count()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            evs[2 * k].record(stream)
            b.run(stream)
            evs[2 * k + 1].record(stream)
    torch.cuda.synchronize(dev)
    launches = lib.seismic_launch_count() - launches0
    clk = clocks.stop()
    t = np.array([evs[2 * k].elapsed_time(evs[2 * k + 1]) for k in range(args.steps)]) * 1e-3
    step = float(t.mean())
    if ws > 1:
        import torch.distributed as dist
        tt = torch.tensor([step], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        step = float(tt.item())
    # FP64 error on a sample of pairs of a few catalogs
    errs = []
    for k in range(0, len(cats), 51):
        ev, shift = cats[k]
        o = b.outputs[k]
        errs.append(fp64_sample_error(ev, shift, xcorr_padded(ev.shape[-1], shift), o.vals_pos.cpu().numpy(),
                                      o.lags_pos.cpu().numpy(), o.vals_neg.cpu().numpy(),
                                      o.lags_neg.cpu().numpy(), n_sample=300))
    fp64 = {"max_abs": max(e["max_abs"] for e in errs), "mean_abs": float(np.mean([e["mean_abs"] for e in errs])),
            "lag_agreement": float(np.mean([e["lag_agreement"] for e in errs])),
            "lag_mismatch_not_exempt": int(sum(e["lag_mismatch_not_exempt"] for e in errs)),
            "pairs_sampled": int(sum(e["pairs_sampled"] for e in errs))}
    # end to end: events in from pinned host memory, graph replay, outputs back
    e2e = None
    if not args.skip_e2e:
        h_in = [torch.empty(ev.shape, dtype=torch.float32, pin_memory=True) for ev, _ in cats]
        for h, (ev, _) in zip(h_in, cats):
            h.numpy()[...] = ev
        h_out = [[torch.empty_like(x, device="cpu", pin_memory=True) for x in (o.vals_pos, o.lags_pos, o.vals_neg,
                                                                               o.lags_neg)] for o in b.outputs]
        walls = []
        for k in range(4):  # one untimed warm-up pass of the copies, then 3 timed
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            with torch.cuda.stream(stream):
                for h, d in zip(h_in, tens):
                    d.copy_(h, non_blocking=True)
                b.run(stream)
                for o, ho in zip(b.outputs, h_out):
                    for x, hx in zip((o.vals_pos, o.lags_pos, o.vals_neg, o.lags_neg), ho):
                        hx.copy_(x, non_blocking=True)
            stream.synchronize()
            if k > 0:
                walls.append(time.perf_counter() - t0)
        e2e = {"value": ws * npairs / float(np.mean(walls)), "unit": "pairs/s", "walls_ms": [1e3 * w for w in walls],
               "h2d_bytes_per_step": int(sum(ev.nbytes for ev, _ in cats)),
               "d2h_bytes_per_step": int(16 * npairs),
               "entry_point": "seismic_batch_run (C ABI) with host<->device copies of every catalog"}
    peaks_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_mhz = clk.get("sm_mhz") or 2070.0
    peak_tf = peaks_sm * 128 * 2 * sm_mhz * 1e6 / 1e12
    achieved = flops / step / 1e12
    sizes = {}
    for ev, shift in cats:
        p = xcorr_padded(ev.shape[-1], shift)
        sizes[p] = sizes.get(p, 0) + 1
    out = {"metric": METRIC, "value": ws * npairs / step, "unit": "pairs/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": step * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32",
           "data": "synthetic: seeded family-based waveforms (no public dataset; the reference's is not distributed)",
           "config": {"workload": "batched: " + WORKLOAD_TEXT["batched"], "n_catalogs": len(cats),
                      "pairs_per_step": npairs, "catalogs_per_fft_size": sizes,
                      "events_total": int(sum(ev.shape[0] for ev, _ in cats)),
                      "kernels_per_step": b.kernels_per_run, "generation_s": round(t_gen, 1),
                      "pair_launch": "one per transform size" if args.batch_per_size else "one over all sizes",
                      "l2": "L2 flushed (256 MB write) between timed steps"},
           "fp64_error": fp64,
           "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_tf, "unit": "TFLOP/s",
                        "frac": achieved / peak_tf, "traffic": None,
                        "kernel": "whole graph (batched_spectra_kernel + batched_pair_kernel<P> per size)",
                        "peak_source": f"nominal FP32 FMA rate at the median SM clock {sm_mhz:.0f} MHz",
                        "work": "sum over catalogs of pairs x (2.5 P log2 P + 6 C (P/2+1)) flop"},
           "e2e": e2e, "clocks": clk, "gpu_launches": int(launches)}
    if rank == 0 and not args.no_cpu_baseline:
        # the reference's CPU path on catalogs where it is defined (power-of-two L, full lags)
        from oracle import oracle as O  # noqa: F401  (cpu_baseline imports it)
        sample = [(ev, s) for ev, s in cats if (ev.shape[-1] & (ev.shape[-1] - 1)) == 0 and ev.shape[0] <= 300][:6]
        tot_pairs, tot_t = 0, 0.0
        base = None
        for ev, s in sample:
            base, times = cpu_baseline("batched", ev, s, n_sample=ev.shape[0])
            tot_pairs += ev.shape[0] * (ev.shape[0] + 1) // 2
            tot_t += float(np.median(times))
        if base is not None:
            base["value"] = tot_pairs / tot_t
            base["sample"] = (f"{len(sample)} catalogs of the batch with power-of-two L and N <= 300 "
                              f"({tot_pairs} pairs; one single-channel call per channel)")
            out["cpu_baseline"] = base
    if rank == 0:
        print(json.dumps(out), flush=True)
    b.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_serving(args):
    """Serving form: 50,000 x 3 x 1024 resident catalog, lags -255..256,
    Poisson query stream; reports latency percentiles and pairs/s."""
    import torch
    from seismic_gb300 import _lib
    from seismic_gb300.serving import Server

    n_cat = args.n_events or 50000
    cat = synth.serving_catalog(n_cat)  # process pool: before the first GPU call
    torch.cuda.set_device(0)
    shift = 256
    form = args.form if args.form in ("fp32", "fp16", "laggemm", "laggemm16") else "fp16"
    lib = _lib.lib()
    srv = Server(cat, shift=shift, form=form, n_slots=args.slots, max_query_events=64, topk=16)
    rng = np.random.default_rng(77)

    def query(nq, seed, length=1024):
        return synth.family_catalog(nq, 3, length, n_families=1, seed=seed)

    for k in range(args.warmup):
        srv.wait(srv.submit(query(64, 100 + k)))
    # isolated latency: 64-event queries against the whole catalog, one at a time
    clocks = ClockSampler(_gpu_id(torch.device("cuda", 0), 0))
    clocks.start()
    launches0 = lib.seismic_launch_count()
    iso = []
    t0 = time.perf_counter()
    iso_q = [query(64, 200 + k) for k in range(max(args.steps, 10))]
    for q in iso_q:
        iso.append(srv.wait(srv.submit(q)).latency_ms)
    iso_wall = time.perf_counter() - t0
    iso_pairs = 64 * n_cat * len(iso)
    # Poisson load sweep: 1..64 events of 256..1024 samples, full catalog or a
    # station subset of 1,000..50,000
    levels = []
    for rate in (100, 300, 1000):
        n_req = {100: 200, 300: 300, 1000: 200}[rate]  # 2 s, 1 s and 0.2 s of offered load
        gaps = rng.exponential(1.0 / rate, size=n_req)
        reqs = []
        for k in range(n_req):
            nq = int(rng.integers(1, 65))
            if rng.random() < 0.5:
                b, e = 0, n_cat
            else:
                size = int(rng.integers(min(1000, n_cat), n_cat + 1))
                b = int(rng.integers(0, n_cat - size + 1))
                e = b + size
            ql = int(rng.integers(256, 1025))
            reqs.append((query(nq, 1000 + rate * 100 + k, ql), (b, e), nq * (e - b)))
        tickets = []
        start = time.perf_counter()
        due = start
        for (q, sub, _), g in zip(reqs, gaps):
            due += g
            dt = due - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            tickets.append(srv.submit(q, sub))
        lat = [srv.wait(t).latency_ms for t in tickets]
        wall = time.perf_counter() - start
        pairs = sum(p for _, _, p in reqs)
        levels.append({"offered_req_per_s": rate, "requests": n_req, "p50_ms": float(np.percentile(lat, 50)),
                       "p99_ms": float(np.percentile(lat, 99)), "pairs_per_s": pairs / wall})
    launches = lib.seismic_launch_count() - launches0
    clk = clocks.stop()
    # FP64 check on a sample of one isolated request's pairs
    res = srv.wait(srv.submit(iso_q[0]))
    sel = rng.integers(0, n_cat, 400)
    ev = np.concatenate([iso_q[0][:4], cat[sel]])
    fp = fp64_sample_error_rect(ev, 4, shift, res, sel)
    srv.close()
    out = {"metric": METRIC + "; serving p50/p99 latency", "value": iso_pairs / iso_wall, "unit": "pairs/s",
           "n_gpus": 1, "steps": len(iso), "warmup": args.warmup,
           "ms_per_step": float(np.mean(iso)), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": FORM_DTYPE.get(form, "f32"),
           "data": "synthetic: seeded family-based waveforms (no public dataset; the reference's is not distributed)",
           "config": {"workload": "serving: 50,000-event resident catalog x 3 channels x L=1024, lags -255..256, "
                                  f"{form} catalog " + ("16-bit sample planes" if form.startswith("laggemm")
                                                         else "spectra") + f" + FP64 norms on device, {args.slots} "
                                  "request slots, top-16; Poisson requests of 1..64 events of 256..1024 samples",
                      "n_catalog": n_cat},
           "serving": {"isolated_64_event_full_catalog": {"p50_ms": float(np.percentile(iso, 50)),
                                                          "p99_ms": float(np.percentile(iso, 99)),
                                                          "requests": len(iso), "pairs_per_request": 64 * n_cat},
                       "poisson_load": levels},
           "fp64_error": fp, "clocks": clk, "gpu_launches": int(launches),
           "e2e": {"value": iso_pairs / iso_wall, "unit": "pairs/s",
                   "h2d_bytes_per_step": 64 * 3 * 1024 * 4, "d2h_bytes_per_step": 64 * n_cat * 16 + 64 * 16 * 12,
                   "entry_point": "seismic_server_submit/wait (C ABI), query in, all pair outputs + top-16 out"}}
    print(json.dumps(out), flush=True)


def fp64_sample_error_rect(ev, nq, shift, res, sel):
    """FP64 error of query rows 0..nq-1 against catalog columns `sel`."""
    x = ev.astype(np.float64)
    p = xcorr_padded(x.shape[-1], shift)
    norms = np.sqrt((x * x).sum(-1))
    inv = np.where(norms > 0, 1.0 / np.where(norms > 0, norms, 1), 0.0)
    spec = np.fft.rfft(x, n=p, axis=-1) * inv[..., None]
    lags = np.arange(1 - shift, shift + 1)
    errs, mis, gaps = [], [], []
    for q in range(nq):
        series = np.fft.irfft((spec[q][None] * np.conj(spec[nq:])).mean(axis=1), n=p, axis=-1)[:, np.mod(lags, p)]
        vp = np.maximum(series.max(1), 0.0)
        vn = np.minimum(series.min(1), 0.0)
        errs.append(np.abs(res.vals_pos[q][sel] - vp))
        errs.append(np.abs(res.vals_neg[q][sel] - vn))
        lp = np.where(vp > 0, lags[series.argmax(1)], 0)
        mis.append(res.lags_pos[q][sel] != lp)
        top2 = np.partition(series, -2, axis=1)[:, -2:]
        gaps.append(top2[:, 1] - top2[:, 0])
    e = np.concatenate(errs)
    mis, gaps = np.concatenate(mis), np.concatenate(gaps)
    return {"max_abs": float(e.max()), "mean_abs": float(e.mean()),
            "lag_agreement": float(1.0 - mis.mean()),
            "lag_mismatch_not_exempt": int((mis & (gaps >= 1e-6)).sum()),
            "lag_mismatch_beyond_2x_max_err": int((mis & (gaps >= 2 * e.max())).sum()),
            "pairs_sampled": int(mis.size)}


def xcorr_padded(length: int, shift: int) -> int:
    p = 64
    while p < length + shift:
        p <<= 1
    return p


def _gpu_id(dev, local):
    import torch
    try:
        props = torch.cuda.get_device_properties(dev)
        return f"{props.pci_domain_id:08x}:{props.pci_bus_id:02x}:{props.pci_device_id:02x}.0"
    except Exception:
        return str(local)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOAD_TEXT), default="precision")
    ap.add_argument("--form", choices=["fp32", "fp16", "bf16", "laggemm", "laggemm16"], default="fp32",
                    help="fp32: fused FFT form; fp16/bf16: half-precision spectra and products; "
                         "laggemm: tensor-core lag-GEMM (short windows)")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--n-events", type=int, default=None, help="override N (small profiling cases only)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra-forms", action="store_true",
                    help="precision workload: skip the reduced-precision forms carried in the FP32 line")
    ap.add_argument("--slots", type=int, default=4, help="serving: request slots (concurrent requests)")
    ap.add_argument("--batch-per-size", action="store_true",
                    help="batched: one persistent pair launch per transform size instead of one over all sizes")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "serving":
        run_serving(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
