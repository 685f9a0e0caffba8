#!/usr/bin/env python
"""Benchmark: equilibrium LDM spectra/s on the 5M-line CO2-like workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload co2_5M|h2o_100M]

One step = one spectrum (scatter -> FFT/Voigt reduce -> IFFT) of the 5M-line
CO2-like list over 2000-2400 cm-1 at 0.001 cm-1 (400 001 points), 8 x 16 LDM
nodes, T = 1500 K, p = 1 bar, x = 0.1.  ``value``: spectra/s with the line list
resident in HBM, timed with CUDA events on the launching stream (no per-stage
events inside that region; a separate pass records them for the stage table
and the roofline).  ``e2e``: the same through the host API
(rg_synthesize_host: conditions in, float32 spectrum copied back to pinned
host memory, synchronous), plus the cold path (upload from host arrays + plan
+ spectrum) reported beside it.  ``error``: the timed spectrum's
abscoeff, absorbance, emissivity, transmittance and radiance against the
reference's CPU path run on the whole workload (the same run is the
``cpu_baseline`` timing).  ``c3``: the 100M-line H2O-like workload (1 500 001
points, 12 x 24 nodes): stage times, scatter roofline and error against the
oracle over the full spectrum.  ``fft_vs_cufft``: cuFFT (through torch) on
the same batched rows as this library's FFT stages.  N > 1 runs independent
replicas, one per GPU (the path needs no exchange between GPUs).

``--impl reference`` runs the reference's CPU LDM path, restated in FP64
numpy by the oracle (the reference itself needs pandas/astropy/numba and its
GPU path needs Vulkan, neither of which exists here), on the whole workload
every step, on rank 0 only; it imports nothing of this library.

``--ingest-only`` times the host-side HITRAN-160 ingestion instead (no GPU).
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "spectra/s and p50/p99 latency at <=1e-4 rel err: served vs plain GPU LDM"
WORKLOAD = "co2_5M"
KERNELS_PER_STEP = 5   # plain layout: scatter, column FFT, row FFT + Voigt, inverse row, inverse column


def inverse_fused(info):
    """The inverse row DFT runs inside the forward row kernel when one CTA
    holds a row's whole pair sum (at most 16 pairs, i.e. 32 FFT rows)."""
    return int(info.fft_rows) // 2 <= 16


def kernels_per_step(info):
    """Kernels one spectrum launches: scatter, column FFT, row FFT + Voigt,
    inverse row FFT (unless fused into the row kernel) and inverse column
    FFT; with the skeleton layout the projection in addition (none when the
    scatter projects); with the merged layout the Gaussian stage and the
    merged-row column FFT instead of the column FFT, plus a column FFT of the
    narrow-node rows when there are any."""
    base = KERNELS_PER_STEP - (1 if inverse_fused(info) else 0)
    if int(info.layout) == 3:
        return base + 1
    if int(info.layout) == 4 or not info.merged_rows:
        return base
    nlv = info.merged_rows + (info.merged_rows & 1)
    return base + 1 + (1 if info.fft_rows > nlv else 0)
STAGES = ["k_scatter", "k_col_fft_fwd", "k_row_fft_voigt", "k_row_ifft", "k_col_ifft"]
LAYOUT_NAMES = {1: "node rows", 2: "merged rows", 3: "skeleton rows", 4: "skeleton rows, projected in the scatter"}


# name: (label, lines factory, molar mass, vmin, vmax, wstep, T, p_bar, x, n_G, n_L)
WORKLOADS = {
    "co2_5M": ("CO2-like", "co2_like", 44.0, 2000.0, 2400.0, 0.001, 1500.0, 1.0, 0.1, 8, 16),
    "h2o_100M": ("H2O-like", "h2o_like", 18.0, 500.0, 8000.0, 0.005, 2000.0, 1.0, 0.2, 12, 24),
}


def line_record_bytes(lines):
    """Bytes the scatter reads per line: v0 as an FP32 (hi, lo) pair, then
    log2 S', E_low, gamma_air, gamma_self, n_air (4 B each), the pressure
    shift (4 B) and the isotopologue slot (1 B) only when the list has them."""
    import numpy as np
    b = 8 + 5 * 4
    if lines.get("delta") is not None:
        b += 4
    if lines.get("iso") is not None and np.unique(np.asarray(lines["iso"])).size > 1:
        b += 1
    return b


def workload_desc(name, n_lines, n_v, line_bytes):
    """The workload a bench line measures (identical in both arms)."""
    label, _, _, vmin, vmax, ws, T, p, x, nG, nL = WORKLOADS[name]
    return {
        "workload": (f"{label} synthetic list, {n_lines} lines, {vmin:g}-{vmax:g} cm-1 at {ws:g} cm-1 "
                     f"({n_v} points), {nG}x{nL} LDM nodes, T={T:g} K, p={p:g} bar, x={x:g}"),
        "n_lines": n_lines, "n_v": n_v, "ldm_nodes": [nG, nL],
        "l2": ("inputs larger than L2 (129 MB): resident line list %d MB (%d B/line), LDM %d MB"
               % (n_lines * line_bytes // 1000000, line_bytes, nG * nL * n_v * 4 // 1000000)),
        "parallelism": "replicas",
    }


def max_over_ranks(x, ws, device):
    """The slowest rank's time (the job's time): all-reduce MAX over the
    process group (NCCL on the GPUs; any backend works, the CPU tests use gloo)."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.path:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(n_lines_read, line_bytes, n_nodes, n_v, n_ft, info):
    """Bytes each kernel must move once (per spectrum): the line records
    (``line_bytes`` each) and the LDM written once (n_v columns, no zero
    padding); the column FFT reads its node rows and writes the packed complex
    rows; the row stage reads them (its accumulator G is stored once); the
    inverse stages read/write G and the output.  With the merged layout the
    Gaussian stage reads the wide-node LDM rows and writes the n_L merged rows
    (n_v + 2 ext points), and the column FFT reads those and the narrow-node
    rows.  With the skeleton layout the projection reads the node rows and
    writes the skeleton rows, which the column FFT reads; projected in the
    scatter's flush, the scatter writes only the skeleton rows."""
    pairs = int(info.fft_rows or n_nodes) // 2
    out = {
        "k_scatter": n_lines_read * line_bytes + n_nodes * n_v * 4,
        "k_col_fft_fwd": n_nodes * n_v * 4 + pairs * n_ft * 8,
        "k_row_fft_voigt": pairs * n_ft * 8 + n_ft * 8,
        "k_row_ifft": 2 * n_ft * 8,
        "k_col_ifft": n_ft * 8 + n_v * 4,
    }
    if inverse_fused(info):   # G written once, after the inverse part
        out.pop("k_row_ifft")
    NL = int(info.merged_rows)
    if NL:
        nlv = NL + (NL & 1)
        n_narrow = int(info.fft_rows) // nlv - 1
        wide_rows = (int(info.grid.n_G) - n_narrow) * NL
        merged = NL * (n_v + 2 * int(info.merged_ext)) * 4
        out["k_gauss_merge"] = wide_rows * n_v * 4 + merged
        out["k_col_fft_fwd"] = merged + n_narrow * NL * n_v * 4 + pairs * n_ft * 8
    if int(info.layout) in (3, 4):
        rows = int(info.fft_rows)
        real_nodes = int(info.grid.n_G) * int(info.grid.n_L)
        out["k_col_fft_fwd"] = rows * n_v * 4 + pairs * n_ft * 8
        if int(info.layout) == 3:
            out["k_node_project"] = real_nodes * n_v * 4 + rows * n_v * 4
        else:   # projected by the scatter's flush: only the skeleton rows are written
            out["k_scatter"] = n_lines_read * line_bytes + rows * n_v * 4
    return out


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(workload):
    """Per-launch DRAM traffic (bytes) per kernel from the committed ncu
    summary profiles/traffic_<workload>.txt ("kernel bytes" lines), if
    present."""
    p = os.path.join(ROOT, "profiles", f"traffic_{workload}.txt")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            f = line.split()
            if len(f) == 2 and not line.startswith("#"):
                out[f[0]] = int(f[1])
    return out


def _synthetic():
    """The seeded workload generators (radis_gb300/synthetic.py, numpy only),
    loaded from their file so that the reference arm imports nothing of the
    library package."""
    spec = importlib.util.spec_from_file_location("rg_bench_synthetic",
                                                  os.path.join(ROOT, "radis_gb300", "synthetic.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def load_workload(wl, n_lines=None):
    """The workload's seeded line list (its own size, or the first draw of
    ``n_lines`` lines of the same generator: same geometry, fewer lines, for
    small profiling cases) and its grid."""
    S = _synthetic()
    _, fac, M, vmin, vmax, ws, T, p, x, nG, nL = WORKLOADS[wl]
    lines = getattr(S, fac)() if not n_lines else getattr(S, fac)(n=int(n_lines))
    return lines, M, vmin, ws, S.grid_points(vmin, vmax, ws), T, p, x, nG, nL


def reference_spectrum(wl, lines, workers, axes=None, n_ft=None, line_chunk=None):
    """The reference's CPU LDM path (broadening_method='fft') on the whole
    line list, as the oracle restates it in FP64 numpy: per-line scaling, the
    8 np.add.at of radis/lbl/broadening.py:2478-2485 (single-threaded, as in
    the reference), per-node rfft x folded Voigt FT and one irfft
    (:2521-2530; FFTs through scipy.fft on ``workers`` host threads), x the
    number density.  Node axes from the oracle's own restatement of the
    reference's envelope rule unless ``axes`` is given; the FFT length is the
    CPU path's 2 n_v (broadening.py:2340) unless ``n_ft`` is given.  Returns
    (abscoeff cm-1, seconds for scaling + scatter, seconds for the FFT stage)."""
    import numpy as np

    from oracle import ldm_oracle as O
    _, _, M, vmin, vmax, ws, T, p, x, nG, nL = WORKLOADS[wl]
    n_v = int(round((vmax - vmin) / ws)) + 1
    if axes is None:
        axes = O.envelope_axes(lines, T, p, x, NG=nG, NL=nL, molar_mass=M)
    n_ft = 2 * n_v if n_ft is None else int(n_ft)
    n = len(lines["v0"])
    step = n if not line_chunk else int(line_chunk)
    t0 = time.perf_counter()
    LDM = None
    for a in range(0, n, step):
        part = lines if step >= n else {k: (np.asarray(v)[a:a + step] if np.ndim(v) == 1 else v)
                                        for k, v in lines.items()}
        kpos, lgG, lgL, S = O.line_quantities(part, T, p, x, vmin, ws, molar_mass=M)
        LDM = O.ldm_scatter(kpos, lgG, lgL, S, n_v, axes, out=LDM)
        del kpos, lgG, lgL, S
    t1 = time.perf_counter()
    spec = O.ldm_convolve(LDM, n_v, ws, axes, n_ft, fft_workers=workers)
    t2 = time.perf_counter()
    return spec * O.number_density(p, T, x), t1 - t0, t2 - t1


def run_reference(args):
    ws_, rank, _ = dist_env()
    if rank != 0:
        return 0
    wl = args.workload
    lines, M, vmin, dv, n_v, T, p, x, nG, nL = load_workload(wl)
    workers = os.cpu_count() or 1
    times, parts = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _, tl, tc = reference_spectrum(wl, lines, workers)
        t = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(t)
            parts.append((tl, tc))
    step = statistics.mean(times)
    value = 1.0 / step
    n = len(lines["v0"])
    sample = (f"whole workload every step: all {n} lines scaled and scattered (8 np.add.at, one host thread, "
              f"as the reference), {nG * nL} node rows of rfft length {2 * n_v} x folded Voigt FT + one irfft "
              f"(scipy.fft, {workers} host threads); FP64")
    out = {
        "metric": METRIC, "value": value, "unit": "spectra/s", "n_gpus": ws_, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": workload_desc(wl, n, n_v, line_record_bytes(lines)),
        "cpu_baseline": {"value": value, "unit": "spectra/s", "cores": workers, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "spectra/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "stage_s": {"lines_scaled_scattered": statistics.mean(q[0] for q in parts),
                    "fft_voigt": statistics.mean(q[1] for q in parts)},
    }
    print(json.dumps(out))
    return 0


def serving_requests(lists, n, seed):
    """Seeded request stream of the serving configuration: list uniform, window
    width log-uniform 50-2000 cm-1 (clipped to the list), wstep in
    {0.001, 0.002, 0.005, 0.01}, T log-U[300, 3000] K, p log-U[0.1, 10] bar,
    x log-U[0.01, 1]."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        name = list(lists)[int(rng.integers(len(lists)))]
        lines, lo, hi = lists[name]
        dv = float(rng.choice([0.001, 0.002, 0.005, 0.01]))
        width = min(float(np.exp(rng.uniform(np.log(50.0), np.log(2000.0)))), hi - lo)
        vmin = float(np.floor(rng.uniform(lo, hi - width) / dv) * dv)
        n_v = int(width / dv) + 1
        T = float(np.exp(rng.uniform(np.log(300.0), np.log(3000.0))))
        p = float(np.exp(rng.uniform(np.log(0.1), np.log(10.0))))
        x = float(np.exp(rng.uniform(np.log(0.01), np.log(1.0))))
        out.append((name, lines, vmin, dv, n_v, T, p, x))
    return out


def run_serving(ctx, L, lists, n_req, slots, seed=11):
    """Served (continuous batching, rg_server) vs plain per-request form (a
    fresh plan per request, synchronous), on the same request stream:
    capacity with every request queued at t = 0, then latency under Poisson
    arrivals at 0.8 x the plain capacity.  Both forms are warmed up with one
    untimed pass of the stream first: the plain form's stream-ordered
    allocations then come from a warm pool, and the server -- one long-lived
    instance, as a deployed service -- has grown its slots' workspaces to the
    stream's sizes."""
    import threading

    import numpy as np
    import torch
    from radis_gb300 import synthetic as S
    reqs = serving_requests(lists, n_req, seed)
    # one page-locked output buffer per request, the same in both forms: the
    # spectrum's last kernel writes it directly (no staging copy)
    bufs = [torch.empty(r[4], dtype=torch.float32, pin_memory=True).numpy() for r in reqs]
    # node spacing of the reference's defaults; the Gaussian axis spans the
    # lines that can reach each request's window (as the reference's factory
    # loads only those), in both forms
    dx = dict(dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT, axes_window=True)

    def plain(arrivals):
        outs, lat = [], []
        t0 = time.perf_counter()
        for i, ((name, lines, vmin, dv, n_v, T, p, x), ta) in enumerate(zip(reqs, arrivals)):
            now = time.perf_counter() - t0
            if ta > now:
                time.sleep(ta - now)
            plan = L.Plan(lines, vmin, dv, n_v, **dx)
            o, info = plan.synthesize_host(T, p, x, out=bufs[i])
            plan.close()
            outs.append((o, info.log_scale))
            lat.append(time.perf_counter() - t0 - ta)
        total = time.perf_counter() - t0
        return [o.astype(np.float64) * np.exp(ls) for o, ls in outs], lat, total

    worker_ms = {}
    srv = L.Server(ctx, slots=slots, mem_budget=96 << 30)

    def served(arrivals):
        st0 = srv.stats()
        tickets = [None] * len(reqs)
        t0 = time.perf_counter()

        def submitter():
            for i, ((name, lines, vmin, dv, n_v, T, p, x), ta) in enumerate(zip(reqs, arrivals)):
                now = time.perf_counter() - t0
                if ta > now:
                    time.sleep(ta - now)
                tickets[i] = srv.submit(lines, vmin, dv, n_v, T, p, x, out=bufs[i], **dx)
        th = threading.Thread(target=submitter)
        th.start()
        outs, lat = [], []
        for i in range(len(reqs)):
            while tickets[i] is None:
                time.sleep(1e-5)
            o, info, (ts, t_start, t_done) = srv.wait(tickets[i])
            lat.append(time.perf_counter() - t0 - arrivals[i])
            outs.append((o, info.log_scale))
        th.join()
        total = time.perf_counter() - t0
        st = srv.stats()
        worker_ms.update(need=st.host_need_ms - st0.host_need_ms, launch=st.host_launch_ms - st0.host_launch_ms,
                         copy=st.host_copy_ms - st0.host_copy_ms)
        return [o.astype(np.float64) * np.exp(ls) for o, ls in outs], lat, total

    zero = [0.0] * len(reqs)
    plain(zero)                          # warm-up (allocator pools)
    served(zero)                         # warm-up (slot workspaces)
    p_out, _, p_total = plain(zero)
    s_out, _, s_total = served(zero)
    worker_capacity_ms = dict(worker_ms)
    plain_sps, served_sps = len(reqs) / p_total, len(reqs) / s_total
    err = max(float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)) for a, b in zip(s_out, p_out))
    rate = 0.8 * plain_sps
    rng = np.random.default_rng(seed + 1)
    arrivals = list(np.cumsum(rng.exponential(1.0 / rate, len(reqs))))
    _, p_lat, _ = plain(arrivals)
    _, s_lat, _ = served(arrivals)
    srv.close()
    pct = lambda v, q: float(np.percentile(np.asarray(v) * 1e3, q))
    npts = [r[4] for r in reqs]
    # where the plain time goes, per line list: plan creation (host clock,
    # includes its device work and synchronisation) and the spectrum's device
    # time (stage events)
    brk = {}
    for (name, lines, vmin, dv, n_v, T, p, x) in reqs:
        t_a = time.perf_counter()
        plan = L.Plan(lines, vmin, dv, n_v, **dx)
        t_b = time.perf_counter()
        _, info = plan.synthesize_host(T, p, x, timing=True)
        plan.close()
        b = brk.setdefault(name, {"requests": 0, "plan_ms": 0.0, "spectrum_gpu_ms": 0.0, "points": 0,
                                  "stage_ms": [0.0] * 5, "merged": 0, "fft_rows": 0, "nodes": 0})
        b["requests"] += 1
        b["plan_ms"] += (t_b - t_a) * 1e3
        b["spectrum_gpu_ms"] += float(info.stage_ms[5])
        b["points"] += n_v
        for i in range(5):
            b["stage_ms"][i] += float(info.stage_ms[i])
        b["merged"] += int(info.merged_rows > 0)
        b["fft_rows"] += int(info.fft_rows)
        b["nodes"] += int(info.grid.n_G * info.grid.n_L)
    return {
        "requests": len(reqs), "slots": slots,
        "served_spectra_per_s": served_sps, "plain_spectra_per_s": plain_sps,
        "served_over_plain": served_sps / plain_sps,
        "max_rel_err_served_vs_alone": err,
        "poisson_rate_per_s": rate,
        "latency_ms": {"served_p50": pct(s_lat, 50), "served_p99": pct(s_lat, 99),
                       "plain_p50": pct(p_lat, 50), "plain_p99": pct(p_lat, 99)},
        "request_points": {"min": int(min(npts)), "median": int(np.median(npts)), "max": int(max(npts))},
        "plain_form": "fresh plan (FFT tables, line index, workspace) + synchronous spectrum per request",
        "plain_breakdown": brk,
        "served_worker_host_ms": worker_capacity_ms,
    }


def run_slit(ctx, abscoeff_dev, vmin, dv, path_length=1.0, fwhm=0.5, reps=20):
    """Instrument slit on the spectrum of the bench workload: transmittance
    exp(-abscoeff L) convolved with a triangular slit of ``fwhm`` cm-1
    (generated and resampled on the host as the reference does), the
    convolution on the GPU (rg_slit_convolve).  Times the device convolution
    with CUDA events and, for comparison, the reference's own CPU algorithm
    for it (scipy.signal.oaconvolve, radis/tools/slit.py:737) on the host."""
    import numpy as np
    import torch
    from scipy.signal import oaconvolve

    from radis_gb300 import slit as S
    n = abscoeff_dev.numel()
    wstep = dv
    w_s, I_s = S.triangular_slit(fwhm, wstep, center=vmin + dv * (n // 2))
    taps = S.slit_on_grid(w_s, I_s, wstep)
    tr = torch.exp(-abscoeff_dev.double() * path_length).float()
    out = torch.empty_like(tr)
    st = torch.cuda.current_stream()
    for _ in range(3):
        S.convolve_device(tr, taps, wstep, mode="valid", out=out, ctx=ctx)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        S.convolve_device(tr, taps, wstep, mode="valid", out=out, ctx=ctx)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    host = tr.double().cpu().numpy()
    t0 = time.perf_counter()
    ref = oaconvolve(host, taps, mode="same") * wstep
    cpu_ms = (time.perf_counter() - t0) * 1e3
    got = out.double().cpu().numpy()
    ok = ~np.isnan(got)
    err = float(np.max(np.abs(got[ok] - ref[ok])) / np.max(np.abs(ref[ok])))
    return {"workload": f"transmittance of the bench spectrum ({n} points, L = {path_length} cm) with a "
                        f"triangular slit of FWHM {fwhm} cm-1 ({len(taps)} taps on the {dv} cm-1 step), "
                        "mode 'valid'",
            "taps": int(len(taps)), "gpu_ms": ms, "gflop_s": 2.0 * n * len(taps) / (ms * 1e-3) / 1e9,
            "cpu_reference_ms": cpu_ms, "cpu_reference": "scipy.signal.oaconvolve (FFT overlap-add), 1 core",
            "max_rel_err_vs_cpu": err}


def run_autodiff(ctx, L, n_cond=64, seed=12):
    """Derivative configuration: 64 seeded conditions on the CO-like 10k list
    at 0.001 cm-1 (1900-2300, 400 001 points), T log-U[300, 3000] K, p
    log-U[0.1, 10] bar, x log-U[0.01, 1].  Times, per condition, the FP32
    forward, forward + adjoint (gradient of a scalar loss, through the
    library's API and through the torch.autograd wrapper), forward + the
    three tangent spectra, and finite differences by forward runs (a central
    difference per parameter: 6 extra spectra)."""
    import numpy as np
    import torch

    from radis_gb300 import synthetic as S
    from radis_gb300.autodiff import absorbance, jacobian
    rng = np.random.default_rng(seed)
    conds = [(float(np.exp(rng.uniform(np.log(300), np.log(3000)))),
              float(np.exp(rng.uniform(np.log(0.1), np.log(10.0)))),
              float(np.exp(rng.uniform(np.log(0.01), np.log(1.0))))) for _ in range(n_cond)]
    ln = L.Lines(ctx, S.co_like(), 28.0)
    n_v = 400001
    plan = L.Plan(ln, 1900.0, 0.001, n_v, dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT)
    out = torch.empty(n_v, dtype=torch.float32, device="cuda")
    w = torch.rand(n_v, device="cuda")

    def fwd(c):
        plan.synthesize_device(*c, out.data_ptr(), torch.cuda.current_stream().cuda_stream or 1)

    st = torch.cuda.current_stream().cuda_stream or 1

    def fwd_bwd(c):   # the library's adjoint: spectrum, then the gradient of sum(w A) by rg_backward
        plan.synthesize_device(*c, out.data_ptr(), st)
        plan.backward(*c, w.data_ptr(), stream_ptr=st)

    def fwd_bwd_autograd(c):   # the same through the torch.autograd.Function wrapper
        T, p, x = (torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in c)
        (absorbance(plan, T, p, x) * w).sum().backward()

    def fwd_jvp(c):
        jacobian(plan, *c)

    def fd(c):
        fwd(c)
        for i in range(3):
            for sgn in (1.0, -1.0):
                cc = list(c)
                cc[i] *= 1.0 + sgn * 1e-4
                fwd(tuple(cc))

    res = {"workload": ("CO-like synthetic list, 10000 lines, 1900-2300 cm-1 at 0.001 cm-1 (400001 points), "
                        f"{n_cond} conditions T log-U[300,3000] K, p log-U[0.1,10] bar, x log-U[0.01,1]"),
           "conditions": n_cond}
    for name, f in (("forward", fwd), ("forward_adjoint", fwd_bwd), ("forward_adjoint_autograd", fwd_bwd_autograd),
                    ("forward_tangent3", fwd_jvp), ("fd_by_forward", fd)):
        for c in conds[:3]:
            f(c)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for c in conds:
            f(c)
        torch.cuda.synchronize()
        res[name + "_ms"] = (time.perf_counter() - t0) * 1e3 / n_cond
    res["adjoint_speedup_vs_fd"] = res["fd_by_forward_ms"] / res["forward_adjoint_ms"]
    res["tangent_speedup_vs_fd"] = res["fd_by_forward_ms"] / res["forward_tangent3_ms"]
    res["note"] = ("per-condition wall time through the library's API (forward: rg_synthesize; adjoint: "
                   "rg_synthesize + rg_backward of sum(w A), which returns the three sums to the host; tangents: "
                   "rg_synthesize + rg_jvp; FD: 7 forwards), device work synchronised per batch; "
                   "forward_adjoint_autograd is the same gradient through the torch.autograd.Function wrapper "
                   "(its graph, small torch kernels and engine hand-off included); node axes follow each "
                   "condition; accuracy vs central FD of the FP64 oracle is checked in tests/test_gpu_autodiff.py")
    plan.close()
    ln.close()
    return res


def rel_err(got, ref):
    """max |got - ref| / max |ref| (0 for an all-zero reference and result)."""
    import numpy as np
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    den = float(np.max(np.abs(ref))) if ref.size else 0.0
    num = float(np.max(np.abs(got - ref))) if ref.size else 0.0
    return num / den if den > 0 else num


def quantity_errors(plan, T, p, x, vmin, dv, n_v, ref_abscoeff, path_length=1.0):
    """The spectrum at (T, p, x) with the device post-processing
    (rg_synthesize_quantities: abscoeff, absorbance, emissivity,
    transmittance, radiance) against the same quantities derived from the
    reference abscoeff on the host in FP64; max |d| / max |ref| per output."""
    import numpy as np
    import torch

    from oracle import ldm_oracle as O
    buf = torch.empty(5 * n_v, dtype=torch.float32, device="cuda")
    info = plan.synthesize_quantities(T, p, x, path_length, buf.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream or 1)
    torch.cuda.synchronize()
    rows = buf.double().cpu().numpy().reshape(5, n_v)
    sc = math.exp(info.log_scale)
    got = {"abscoeff": rows[0] * sc, "absorbance": rows[1] * sc, "emissivity_noslit": rows[2],
           "transmittance_noslit": rows[3], "radiance_noslit": rows[4]}
    ref = O.quantities(ref_abscoeff, vmin, dv, T, path_length)
    return {k: rel_err(got[k], ref[k]) for k in got}


def run_fft_compare(n_ft, rows, our_fwd_ms, our_inv_ms, reps=10, inverse_row_in_forward=False):
    """cuFFT, through torch.fft, on the batched rows this library's FFT stages
    transform: R2C of ``rows`` real rows of length n_ft (the reference's
    per-node rfft, radis/lbl/broadening.py:2521-2530), C2C of the rows packed
    in complex pairs (what the four-step kernels transform), and the one C2R
    of the summed spectrum.  Library calls, timed with CUDA events on the
    current stream; outside the product path."""
    import torch
    st = torch.cuda.current_stream()
    x = torch.randn(rows, n_ft, device="cuda", dtype=torch.float32)
    z = torch.randn(max(rows // 2, 1), n_ft, device="cuda", dtype=torch.complex64)
    h = torch.randn(n_ft // 2 + 1, device="cuda", dtype=torch.complex64)

    def timed(fn):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    r2c = timed(lambda: torch.fft.rfft(x, dim=1))
    c2c = timed(lambda: torch.fft.fft(z, dim=1))
    c2r = timed(lambda: torch.fft.irfft(h, n=n_ft))
    gbs = lambda b, ms: b / (ms * 1e-3) / 1e9
    half = n_ft // 2 + 1
    out = {
        "rows": rows, "n_ft": n_ft,
        "cufft_r2c_rows_ms": r2c, "cufft_r2c_GB/s": gbs(rows * n_ft * 4 + rows * half * 8, r2c),
        "cufft_c2c_pairs_ms": c2c, "cufft_c2c_GB/s": gbs(2 * (rows // 2) * n_ft * 8, c2c),
        "cufft_c2r_ms": c2r,
        "ours_forward_fft_voigt_ms": our_fwd_ms,
        "ours_inverse_ms": our_inv_ms,
        "note": ("ours = column FFT (+ twiddle) + row FFT fused with the Voigt multiply and the sum over "
                 "nodes, on the same packed rows; cuFFT's figures exclude the Voigt multiply and node sum"
                 + ("; the inverse row DFT runs inside our row kernel, so ours_forward includes it and "
                    "ours_inverse is the inverse column DFT alone" if inverse_row_in_forward else "")),
    }
    del x, z, h
    torch.cuda.empty_cache()
    return out


def time_plan(plan, T, p, x, n_v, K, stream, warm=3):
    """(ms per spectrum over K spectra with no stage events, per-stage average
    ms over a second pass with stage events, Gaussian-stage ms, info with the
    lines in the window)."""
    import torch
    out = torch.empty(n_v, dtype=torch.float32, device="cuda")
    sptr = stream.cuda_stream
    for _ in range(warm):
        plan.synthesize_device(T, p, x, out.data_ptr(), sptr)
    info = plan.synthesize_device(T, p, x, out.data_ptr(), sptr, timing=1)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(K):
        plan.synthesize_device(T, p, x, out.data_ptr(), sptr)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / K
    for _ in range(min(K, 200)):
        plan.synthesize_device(T, p, x, out.data_ptr(), sptr, timing=2)
    stage_sum, stage_n = plan.stage_times()
    stage_avg = [v / max(stage_n, 1) for v in stage_sum]
    gauss = plan.gauss_time() / max(stage_n, 1)
    return ms, stage_avg, gauss, info


def kernel_times(stage_avg, gauss, info):
    """Per-kernel ms from the stage events: with the merged layout the column
    stage is the Gaussian stage (its own event) followed by the column FFT,
    with the skeleton layout the projection followed by the column FFT."""
    kt = {STAGES[i]: stage_avg[i] for i in range(5)}
    if inverse_fused(info):   # one kernel: its stage ends after its inverse part
        kt["k_row_fft_voigt"] += kt.pop("k_row_ifft")
    if int(info.layout) == 3:
        kt["k_node_project"] = gauss
        kt["k_col_fft_fwd"] = stage_avg[1] - gauss
    elif info.merged_rows:
        kt["k_gauss_merge"] = gauss
        kt["k_col_fft_fwd"] = stage_avg[1] - gauss
    return kt


def run_c3(ctx, L, h2o_host, h2o, K, peak, peak_kind, workers, check=True):
    """The 100M-line H2O-like workload (1 500 001 points at 0.005 cm-1,
    12 x 24 nodes, T = 2000 K, p = 1 bar, x = 0.2) on the resident list:
    spectra/s, stage times, the scatter's HBM roofline, and the error of the
    full spectrum against the oracle (FP64, on the plan's node axes and FFT
    length, lines scaled and scattered in blocks of 10M)."""
    import torch
    _, _, M, vmin, vmax, dv, T, p, x, nG, nL = WORKLOADS["h2o_100M"]
    n_v = int(round((vmax - vmin) / dv)) + 1
    plan = L.Plan(h2o, vmin, dv, n_v, n_G=nG, n_L=nL)
    stream = torch.cuda.Stream()
    ms, stage_avg, gauss, info = time_plan(plan, T, p, x, n_v, K, stream)
    g = info.grid
    n_nodes = g.n_G * g.n_L + (g.n_G * g.n_L) % 2
    lb = line_record_bytes(h2o_host)
    ab = algorithmic_bytes(info.lines_in_window, lb, n_nodes, n_v, g.n_ft, info)
    kt = kernel_times(stage_avg, gauss, info)
    stages = {k: {"ms": t, "algorithmic_bytes": ab[k], "GB/s": ab[k] / (t * 1e-3) / 1e9 if t > 0 else None}
              for k, t in kt.items()}
    sc_gbs = stages["k_scatter"]["GB/s"]
    res = {
        "workload": workload_desc("h2o_100M", len(h2o_host["v0"]), n_v, lb)["workload"],
        "spectra_per_s": 1000.0 / ms, "ms_per_spectrum": ms, "spectra_timed": K,
        "stages": stages,
        "scatter_roofline": {"achieved": sc_gbs, "peak": peak, "unit": "GB/s", "frac": sc_gbs / peak,
                             "peak_kind": peak_kind, "bytes_per_line": lb,
                             "lines_read": int(info.lines_in_window)},
        "fft_layout": {"layout": LAYOUT_NAMES.get(int(info.layout)),
                       "fft_rows": int(info.fft_rows), "merged_rows": int(info.merged_rows),
                       "n_ft": int(g.n_ft), "skeleton_sampled_err": float(info.layout_err)},
        "scatter_accumulator_bits": int(info.accum_bits),
    }
    if check:
        import numpy as np

        from oracle import ldm_oracle as O
        host = np.empty(n_v, dtype=np.float32)
        o, inf2 = plan.synthesize_host(T, p, x, out=host)
        gpu = o.astype(np.float64) * math.exp(inf2.log_scale)
        t0 = time.perf_counter()
        ref = O.synthesize(h2o_host, T, p, x, vmin, dv, n_v, g.axes(), g.n_ft, molar_mass=M,
                           fft_workers=workers, line_chunk=10_000_000)
        res["error"] = {"abscoeff_max_rel": rel_err(gpu, ref),
                        "vs": "FP64 oracle over the full 1 500 001-point spectrum, all lines",
                        "oracle_s": time.perf_counter() - t0}
    plan.close()
    return res


def run_ours(args):
    import numpy as np
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from radis_gb300 import _build
    if rank == 0:
        _build.build()
    if ws > 1:
        dist.barrier()
    from radis_gb300 import _lib as L, synthetic as S

    wl = args.workload
    lines, M, vmin, dv, n_v, T, p, x, nG, nL = load_workload(wl, args.lines)
    n_lines = len(lines["v0"])
    lb = line_record_bytes(lines)
    ctx = L.Context(local)
    t0 = time.perf_counter()
    ln = L.Lines(ctx, lines, M)
    plan = L.Plan(ln, vmin, dv, n_v, n_G=nG, n_L=nL, layout=args.layout)
    setup_s = time.perf_counter() - t0
    g = plan.grid(T, p, x)
    n_nodes = g.n_G * g.n_L + (g.n_G * g.n_L) % 2
    stream = torch.cuda.Stream()
    out = torch.empty(n_v, dtype=torch.float32, device="cuda")
    sptr = stream.cuda_stream
    W = max(args.warmup, 3)

    for _ in range(W):
        plan.synthesize_device(T, p, x, out.data_ptr(), sptr)
    torch.cuda.synchronize()
    # lines actually read by the scatter (window + shift margins): all of them here
    info = plan.synthesize_device(T, p, x, out.data_ptr(), sptr, timing=1)
    lines_in_window = info.lines_in_window
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()

    K = args.steps
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        if ws > 1:
            dist.barrier()
        e0.record(stream)
        for i in range(K):
            plan.synthesize_device(T, p, x, out.data_ptr(), sptr)
        e1.record(stream)
        torch.cuda.synchronize()
        if ws > 1:
            dist.barrier()
    ms = e0.elapsed_time(e1) / K
    ms = max_over_ranks(ms, ws, "cuda")
    value = ws * 1000.0 / ms   # replicas: every rank synthesises one spectrum per step
    # per-stage times: a separate pass with stage events (not in the timed region above)
    for _ in range(min(K, 200)):
        plan.synthesize_device(T, p, x, out.data_ptr(), sptr, timing=2)
    stage_sum, stage_n = plan.stage_times()
    stage_avg = [s / max(stage_n, 1) for s in stage_sum]
    gauss_avg = plan.gauss_time() / max(stage_n, 1)

    # e2e through the host API: conditions in, spectrum out to pinned memory
    host = torch.empty(n_v, dtype=torch.float32, pin_memory=True).numpy()
    lat = []
    for i in range(W + K):
        t0 = time.perf_counter()
        plan.synthesize_host(T, p, x, out=host)
        if i >= W:
            lat.append(time.perf_counter() - t0)
    e2e_ms = statistics.mean(lat) * 1e3
    lat_ms = sorted(v * 1e3 for v in lat)
    p50 = lat_ms[len(lat_ms) // 2]
    p99 = lat_ms[min(len(lat_ms) - 1, int(math.ceil(0.99 * len(lat_ms))) - 1)]
    e2e_ms = max_over_ranks(e2e_ms, ws, "cuda")
    # the same with T stepped by 0.1 K per spectrum: new node axes every step,
    # so every per-grid host step (envelopes, skeleton decomposition) reruns
    lat_v = []
    for i in range(W + K):
        t0 = time.perf_counter()
        plan.synthesize_host(T + 0.1 * (i + 1), p, x, out=host)
        if i >= W:
            lat_v.append(time.perf_counter() - t0)
    e2e_var_ms = max_over_ranks(statistics.mean(lat_v) * 1e3, ws, "cuda")
    # cold path: upload from host arrays + plan + one spectrum (eq_spectrum_gpu with exit_gpu)
    cold = []
    for _ in range(2 if n_lines <= 10_000_000 else 1):
        t0 = time.perf_counter()
        ln2 = L.Lines(ctx, lines, M)
        pl2 = L.Plan(ln2, vmin, dv, n_v, n_G=nG, n_L=nL, layout=args.layout)
        pl2.synthesize_host(T, p, x, out=host)
        cold.append(time.perf_counter() - t0)
        pl2.close()
        ln2.close()

    peak, peak_kind = load_peaks()
    ab = algorithmic_bytes(lines_in_window, lb, n_nodes, n_v, g.n_ft, info)
    kt = kernel_times(stage_avg, gauss_avg, info)
    name = max(kt, key=kt.get)   # the dominant kernel
    achieved = ab[name] / (kt[name] * 1e-3) / 1e9
    traffic = load_traffic(wl).get(name)
    stages = {k: {"ms": t, "algorithmic_bytes": ab[k], "GB/s": ab[k] / (t * 1e-3) / 1e9 if t > 0 else None}
              for k, t in kt.items()}

    res = None
    if rank == 0:
        res = {
            "metric": METRIC, "value": value, "unit": "spectra/s", "n_gpus": ws, "steps": K,
            "warmup": W, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_desc(wl, n_lines, n_v, lb),
            "clocks": clk.summary(),
            "gpu_launches": kernels_per_step(info) * K,
            "e2e": {"value": ws * 1000.0 / e2e_ms, "unit": "spectra/s",
                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": n_v * 4,
                    "note": ("resident line list (as the reference's gpuApp.iterate); per step the conditions "
                             "travel as kernel parameters and the spectrum's last kernel writes the float32 "
                             "spectrum into the caller's pinned host buffer (over NVLink-C2C)")},
            "e2e_varied_T": {"value": ws * 1000.0 / e2e_var_ms, "unit": "spectra/s",
                             "h2d_bytes_per_step": 0, "d2h_bytes_per_step": n_v * 4,
                             "note": ("as e2e with T raised by 0.1 K every step: new node axes each step, so the "
                                      "host recomputes the grid and the skeleton decomposition every step (a fit "
                                      "over temperature)")},
            "e2e_cold": {"value": 1.0 / statistics.mean(cold), "unit": "spectra/s",
                         "h2d_bytes_per_step": n_lines * (8 + 8 + 4 * 4), "d2h_bytes_per_step": n_v * 4,
                         "note": "line upload from host arrays + envelopes + plan + one spectrum"},
            "latency_ms": {"p50": p50, "p99": p99, "of": "host API call, plain per-request"},
            "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": traffic, "algorithmic_bytes_per_launch": ab[name],
                         "avg_launch_ms": kt[name]},
            "stages": stages,
            "scatter_accumulator_bits": int(info.accum_bits),
            "fft_layout": {"layout": LAYOUT_NAMES.get(int(info.layout)),
                           "fft_rows": int(info.fft_rows), "merged_rows": int(info.merged_rows),
                           "gauss_halfwidth": int(info.merged_ext), "n_ft": int(g.n_ft),
                           "skeleton_sampled_err": float(info.layout_err)},
            "setup_s": setup_s,
        }
        if name == "k_scatter" and int(info.layout) == 4:
            res["roofline"]["note"] = (
                "the scatter writes only the skeleton rows: each finished tile is projected onto them in shared "
                f"memory ({g.n_G * g.n_L} x {int(info.fft_rows)} FMA per grid column), so the kernel moves "
                f"{ab[name] / 1e6:.0f} MB instead of {(lines_in_window * lb + n_nodes * n_v * 4) / 1e6:.0f} MB "
                "and is bound by its instruction issue, not HBM; frac is the HBM fraction of the bytes it must "
                "move")
        if name == "k_gauss_merge":
            res["roofline"]["note"] = ("the real-space Gaussian stage is FP32-FMA-bound (a banded convolution of "
                                       "each wide-node row with its residual Gaussian, ~200 FMA per merged "
                                       "output point on the 8 wide nodes of this grid): frac is the HBM fraction "
                                       "of the bytes it must move")
        workers = os.cpu_count() or 1
        if ws == 1 and not args.no_cpu_baseline:
            # the reference's CPU path on the whole workload, once: its time is the
            # CPU baseline and its spectrum the reference for the timed spectrum's error
            t0 = time.perf_counter()
            ref, tl, tc = reference_spectrum(wl, lines, workers)
            t = time.perf_counter() - t0
            res["cpu_baseline"] = {
                "value": 1.0 / t, "unit": "spectra/s", "cores": workers, "kind": "port",
                "sample": (f"one spectrum of the whole workload: all {n_lines} lines scaled and scattered "
                           f"(8 np.add.at, one host thread, as the reference; {tl:.2f} s), {nG * nL} node rows "
                           f"of rfft length {2 * n_v} x folded Voigt FT + one irfft (scipy.fft, {workers} host "
                           f"threads; {tc:.2f} s); FP64 oracle restatement of the reference's CPU path")}
            # a path length that puts the peak absorbance at 5, so that
            # transmittance and emissivity span (0, 1) instead of saturating
            Lp = 5.0 / float(np.max(ref))
            res["error"] = quantity_errors(plan, T, p, x, vmin, dv, n_v, ref, path_length=Lp)
            res["error"]["vs"] = ("reference CPU path (FP64 oracle) on the same workload, n_ft = 2 n_v as the "
                                  "reference; max |gpu - ref| / max |ref| per output; quantities from the "
                                  "post-processing fused into the last kernel")
            res["error"]["path_length_cm"] = Lp
            del ref
        if ws == 1 and not args.no_fft_compare:
            fwd = kt["k_col_fft_fwd"] + kt["k_row_fft_voigt"]
            res["fft_vs_cufft"] = {wl: run_fft_compare(int(g.n_ft), int(info.fft_rows or n_nodes), fwd,
                                                       kt.get("k_row_ifft", 0.0) + kt["k_col_ifft"],
                                                       inverse_row_in_forward="k_row_ifft" not in kt)}
        if ws == 1 and not args.no_slit:
            plan.synthesize_device(T, p, x, out.data_ptr(), torch.cuda.current_stream().cuda_stream or 1)
            res["slit"] = run_slit(ctx, out, vmin, dv)
        if ws == 1 and not args.no_autodiff:
            res["autodiff"] = run_autodiff(ctx, L)
        h2o = h2o_host = None
        if ws == 1 and (not args.no_serving or not args.no_c3):
            h2o_host = S.h2o_like(args.serve_h2o_lines)
            h2o = L.Lines(ctx, h2o_host, 18.0)
        if ws == 1 and not args.no_c3 and args.serve_h2o_lines == 100_000_000:
            c3 = run_c3(ctx, L, h2o_host, h2o, 10, peak, peak_kind, workers, check=not args.no_c3_check)
            if not args.no_fft_compare:
                kt3 = {k: v["ms"] for k, v in c3["stages"].items()}
                c3_rows = c3["fft_layout"]["fft_rows"]
                res.setdefault("fft_vs_cufft", {})["h2o_100M"] = run_fft_compare(
                    c3["fft_layout"]["n_ft"], c3_rows, kt3["k_col_fft_fwd"] + kt3["k_row_fft_voigt"],
                    kt3.get("k_row_ifft", 0.0) + kt3["k_col_ifft"], reps=5,
                    inverse_row_in_forward="k_row_ifft" not in kt3)
            res["c3"] = c3
        if h2o_host is not None:
            h2o_host = None
        if ws == 1 and not args.no_serving:
            co = L.Lines(ctx, S.co_like(), 28.0)
            lists = {"co_10k": (co, 1900.0, 2300.0), "co2_5M": (ln, 2000.0, 2400.0),
                     "h2o": (h2o, 500.0, 8000.0)}
            sv = run_serving(ctx, L, lists, args.serve_requests, args.serve_slots)
            sv["lists"] = {"co_10k": 10_000, "co2_5M": n_lines, "h2o": args.serve_h2o_lines}
            res["serving"] = sv
            co.close()
        if h2o is not None:
            h2o.close()
        print(json.dumps(res))
    plan.close()
    ln.close()
    ctx.close()
    if ws > 1:
        dist.destroy_process_group()
    return 0


def run_ingest(args):
    """``--ingest-only`` (host only, no GPU): HITRAN-160 ingestion of a seeded
    synthetic file of ``--ingest-records`` CO-like records.  Times the
    library's parser (all host threads, and one), the numpy fixed-record
    restatement of the reference's parse (parse_hitran_file:
    numpy.fromfile + cast, radis/api/tools.py:25-78) as the CPU baseline,
    and the columnar cache (first load: parse + write; later loads:
    memory-mapped).  Checks the parser against the baseline bit for bit."""
    import numpy as np
    from oracle import hitran_oracle as HO
    from radis_gb300 import hitran as H
    n = args.ingest_records
    rng = np.random.default_rng(31)
    lines = {"v0": np.sort(rng.uniform(1900.0, 2400.0, n)), "S_ref": 10 ** rng.uniform(-30, -18, n),
             "A": 10 ** rng.uniform(-3, 2, n), "g_air": rng.uniform(0.03, 0.09, n),
             "g_self": rng.uniform(0.05, 0.11, n), "El": np.minimum(rng.exponential(3000.0, n), 40000.0),
             "n_air": rng.uniform(0.5, 0.8, n), "delta": rng.uniform(-0.008, 0.004, n),
             "iso": rng.integers(1, 10, n), "gp": rng.integers(1, 200, n).astype(float),
             "gpp": rng.integers(1, 200, n).astype(float)}
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "lines.par")
        H.write_hitran160(p, lines)
        size = os.path.getsize(p)
        text = open(p, "rb").read()

        def best(fn, reps=3):
            t = []
            for _ in range(reps):
                t0 = time.perf_counter()
                r = fn()
                t.append(time.perf_counter() - t0)
            return min(t), r

        cores = os.cpu_count() or 1
        t_all, cols = best(lambda: H.read_hitran160(p, threads=0))
        t_one, _ = best(lambda: H.read_hitran160(p, threads=1))
        t_ref, ref = best(lambda: HO.read_fixed_records(text), reps=1)
        exact = all(np.array_equal(cols[k].view(np.int64) if cols[k].dtype == np.float64 else cols[k],
                                   ref[k].view(np.int64) if ref[k].dtype == np.float64 else ref[k]) for k in ref)
        t_first, _ = best(lambda: H.load_hitran(p, cache="regen"), reps=1)

        def cached():
            c = H.load_hitran(p)
            return float(np.asarray(c["v0"]).sum() + np.asarray(c["S_ref"]).sum())
        t_cached, _ = best(cached)
    rate = lambda t: n / t / 1e6
    print(json.dumps({
        "metric": "HITRAN-160 ingestion (records parsed to columns)", "value": rate(t_all), "unit": "M records/s",
        "higher_is_better": True, "records": n, "bytes": size, "GB/s": size / t_all / 1e9, "threads": cores,
        "ms": t_all * 1e3, "single_thread": {"value": rate(t_one), "ms": t_one * 1e3},
        "bit_exact_vs_baseline": bool(exact),
        "cpu_baseline": {"value": rate(t_ref), "unit": "M records/s", "cores": 1, "kind": "port",
                         "ms": t_ref * 1e3,
                         "sample": "numpy fixed-record parse of the same file (the reference's fromfile + cast)"},
        "cache": {"first_load_ms": t_first * 1e3, "cached_load_ms": t_cached * 1e3,
                  "note": "first load = parse + write of the columnar cache; cached = memory-mapped, "
                          "v0 and S_ref read"},
        "data": "synthetic", "config": {"workload": f"CO-like HITRAN-160 file, {n} records, "
                                                    f"{size / 1e6:.0f} MB, isotopologues 1-9"}}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-autodiff", action="store_true")
    ap.add_argument("--no-slit", action="store_true")
    ap.add_argument("--no-c3", action="store_true", help="skip the 100M-line H2O-like section")
    ap.add_argument("--no-c3-check", action="store_true", help="skip its full-size oracle comparison")
    ap.add_argument("--no-fft-compare", action="store_true", help="skip the cuFFT comparison")
    ap.add_argument("--layout", type=int, default=0, choices=[0, 1, 2, 3],
                    help="FFT-stage layout of the timed plan (0: the fewest rows; 1 node, 2 merged, 3 skeleton)")
    ap.add_argument("--lines", type=int, default=0,
                    help="profiling cases: the workload's geometry with this many lines of its generator")
    ap.add_argument("--serve-requests", type=int, default=120)
    ap.add_argument("--serve-slots", type=int, default=8)
    ap.add_argument("--serve-h2o-lines", type=int, default=100_000_000)
    ap.add_argument("--ingest-only", action="store_true",
                    help="host only: time HITRAN-160 ingestion (parser, baseline, cache) and exit")
    ap.add_argument("--ingest-records", type=int, default=1_000_000)
    args = ap.parse_args()
    if args.ingest_only:
        return run_ingest(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
