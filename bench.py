"""Benchmark: batched all-pairs PCC2 on one GB300 (correlations/s), with the plain
per-pair drop-in, end-to-end host-buffer throughput, latency, roofline and the
CPU baseline on the same line.

Workload (all-pairs): 64 synthetic stations x 48 windows of 18,000 float32
samples (noise + a shared band-passed component with per-station delays), all
2016 station pairs x 48 windows = 96,768 PCC2 correlations per step, lags
+-2000 (4001 lags).  One step = station stage (phase spectra of the 3072 station
windows) + pair stage (96,768 fused cross-spectrum / inverse-transform / lag
kernels), inputs resident in HBM.  Inputs (221 MB) and outputs (1.55 GB) exceed
the 129 MB L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PCC2 correlations/s + p99 latency, served-batched vs plain, 1 GB300, err≤1e-4"
UNIT = "correlations/s"
N_STA, N_WIN, N_SAMP, LAG = 64, 48, 18000, 2000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--stations", type=int, default=N_STA)
    ap.add_argument("--windows", type=int, default=N_WIN)
    ap.add_argument("--fmt", default="f32", choices=["f32", "f16", "i16"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-served", action="store_true", help="skip the served (request loop) leg")
    ap.add_argument("--no-mixed", action="store_true", help="skip the uneven-batch and request-stream legs")
    ap.add_argument("--no-config1", action="store_true", help="skip the plain-config leg (24 x 36000, +-3000)")
    ap.add_argument("--mixed-only", action="store_true", help="run only the uneven-batch and request-stream legs")
    ap.add_argument("--multi-only", action="store_true",
                    help="run only the packed analytic-signal stage leg (profiling); --windows sets its count")
    ap.add_argument("--profile-uneven", metavar="TRACE_JSON",
                    help="profile one cold pass of the uneven batch (torch profiler), write its chrome trace "
                         "to TRACE_JSON and print the kernel and stream summary")
    ap.add_argument("--stack-only", action="store_true",
                    help="run one all-pairs step, then only the stacking leg (profiling of the stacks)")
    ap.add_argument("--wpcc-only", action="store_true",
                    help="run only the wavelet leg (profiling); --windows sets its windows per pair (24 by default)")
    ap.add_argument("--methods-only", action="store_true",
                    help="run the warm-up steps, then only the per-method kernel leg (profiling of one method's "
                         "kernel: ncu -k)")
    return ap.parse_args()


def host_link_leg(torch, dev, hx, hy, d_x, d_y, t_e2e):
    """The end-to-end roofline: copy rates between pinned host memory and the
    device for the step's own buffers (uploads alone, downloads alone, both at
    once on two streams), and the time the step's copies alone would take."""
    up = torch.cuda.Stream(device=dev)
    down = torch.cuda.Stream(device=dev)
    dy = d_y.view(-1)[: hy.numel()]
    hyv = hy.view(-1)

    def run(h2d, d2h, reps=3):
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        for _ in range(reps):
            if h2d:
                with torch.cuda.stream(up):
                    d_x.copy_(hx, non_blocking=True)
            if d2h:
                with torch.cuda.stream(down):
                    hyv.copy_(dy, non_blocking=True)
        torch.cuda.synchronize(dev)
        return (time.perf_counter() - t) / reps

    run(True, True, 1)
    bi, bo = hx.numel() * 4, hy.numel() * 4
    t_up, t_down, t_both = run(True, False), run(False, True), run(True, True)
    return {"h2d_GBs": bi / t_up / 1e9, "d2h_GBs": bo / t_down / 1e9, "both_GBs": (bi + bo) / t_both / 1e9,
            "copies_ms": t_both * 1e3, "frac": t_both / t_e2e,
            "what": "the step's upload and download alone (pinned, both directions at once on two streams): "
                    "frac = their time / the end-to-end step"}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def all_pairs_index(n_sta, n_win):
    """(station-window row of station 1, of station 2) for all i<j pairs, window-major;
    station-window rows are station*n_win + window."""
    iu, ju = np.triu_indices(n_sta, k=1)
    w = np.repeat(np.arange(n_win), iu.size)
    a = np.tile(iu, n_win) * n_win + w
    b = np.tile(ju, n_win) * n_win + w
    return np.ascontiguousarray(np.stack([a, b], axis=1).astype(np.int32))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """Per-launch DRAM bytes of the pair kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "pcc2_pairs_allpairs.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_full_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def served_leg(F, x, pairs, n_win, L, rate_frac=0.5, poisson_max=60000):
    """The same requests through the continuous-batching server: saturation
    throughput with station products resident, then p50/p99 latency at a
    Poisson offered load of rate_frac x saturation."""
    srv = F.Server(hbm_budget=150 << 30, max_batch=8192)
    for row in range(x.shape[0]):
        srv.put(row // n_win, row % n_win, x[row])
    P = pairs.shape[0]
    out = np.zeros((P, L), np.float32)
    reqs = F.Server.request_array(
        [F.Server.request(F.PCC2, int(a // n_win), int(b // n_win), int(a % n_win), -LAG, LAG, out[i])
         for i, (a, b) in enumerate(pairs)])
    t0 = time.perf_counter()
    srv.submit_many(reqs)
    srv.drain()
    t_cold = time.perf_counter() - t0
    # results into ordinary (pageable) arrays: device -> pinned block -> host copy threads
    srv.reset_stats()
    t0 = time.perf_counter()
    srv.submit_many(reqs)
    srv.drain()
    t_pageable = time.perf_counter() - t0
    st_pg = srv.stats()
    # results straight into the registered output array (fpcc_server_register_output)
    srv.register_output(out)
    srv.submit_many(reqs)
    srv.drain()
    srv.reset_stats()
    t0 = time.perf_counter()
    srv.submit_many(reqs)
    srv.drain()
    t_warm = time.perf_counter() - t0
    st_sat = srv.stats()
    sat = P / t_warm
    rate = rate_frac * sat
    n_p = min(P, poisson_max, int(rate * 3.0) + 1)
    srv.reset_stats()
    t0 = time.perf_counter()
    srv.submit_many(reqs, poisson_rate=rate, seed=7, count=n_p)
    srv.drain()
    t_p = time.perf_counter() - t0
    st_p = srv.stats()
    srv.close()
    srv_err = None
    from oracle import oracle as O
    sel = np.random.default_rng(6).choice(P, 4, replace=False)
    srv_err = float(O.relerr(out[sel], O.pcc2(x[pairs[sel, 0]], x[pairs[sel, 1]], -LAG, LAG)).max())
    return {
        "saturation": {"value": sat, "unit": UNIT, "batches": st_sat["batches"],
                       "p50_ms": st_sat["p50_ms"], "p99_ms": st_sat["p99_ms"], "wall_ms": t_warm * 1e3,
                       "worker_ms": st_sat["worker_ms"], "deliver_ms": st_sat["deliver_ms"],
                       "what": f"{P} requests submitted at once, station products resident, results copied "
                               f"straight into the caller's registered output array"},
        "saturation_pageable": {"value": P / t_pageable, "unit": UNIT, "batches": st_pg["batches"],
                                "p50_ms": st_pg["p50_ms"], "p99_ms": st_pg["p99_ms"], "wall_ms": t_pageable * 1e3,
                                "worker_ms": st_pg["worker_ms"], "deliver_ms": st_pg["deliver_ms"],
                                "what": "the same with results delivered into unregistered (pageable) arrays by "
                                        "host copy threads"},
        "max_rel_err": srv_err,
        "cold": {"value": P / t_cold, "unit": UNIT, "what": "first pass, station products computed on demand"},
        "poisson": {"offered": rate, "achieved": n_p / t_p, "requests": n_p, "p50_ms": st_p["p50_ms"],
                    "p99_ms": st_p["p99_ms"], "max_ms": st_p["max_ms"], "batches": st_p["batches"]},
        "hbm_used_bytes": st_sat["hbm_used"],
    }


# mixed workloads: method shares of the uneven batch and of the request stream
MIX_BATCH = {0: 0.40, 2: 0.30, 1: 0.20, 4: 0.10}                        # PCC2, 1-bit, GNCC, PCC1
MIX_STREAM = {0: 0.38, 2: 0.285, 1: 0.19, 4: 0.095, 6: 0.05}            # ... and 5 % wavelet PCC
WAVELET = dict(pmin=4.0, pmax=1000.0, V=5, type=-1)                      # Morlet, 40 scales
METHOD_NAME = {0: "pcc2", 1: "gncc", 2: "cc1b", 3: "cc1b_popcount", 4: "pcc1", 6: "wpcc"}


def _plain_call(F, m, a, b, l1, l2):
    """One request through the plain drop-in of its method (own launch sequence)."""
    if m == F.WPCC:
        return F.wpcc_set(a, b, l1, l2, WAVELET["pmin"], WAVELET["pmax"], V=WAVELET["V"], type=WAVELET["type"])[0]
    return F.correlate(m, a, b, l1, l2, plain=True)[0]


def _oracle_call(O, m, a, b, l1, l2):
    a, b = a[None], b[None]
    if m == 0:
        return O.pcc2(a, b, l1, l2)[0]
    if m == 1:
        return O.gncc(a, b, l1, l2)[0]
    if m == 2:
        return O.cc1b(a, b, l1, l2)[0]
    if m == 4:
        return O.pcc1(a, b, l1, l2)[0]
    return O.wpcc(a, b, l1, l2, WAVELET["pmin"], WAVELET["pmax"], V=WAVELET["V"], wtype=WAVELET["type"])[0]


def _serve_requests(F, srv, reqs, sta_of, outs=None):
    """A Request array over reqs = [(method, s1, s2, window, Lag1, Lag2)] and its outputs."""
    if outs is None:
        outs = [np.zeros(abs(l2 - l1) + 1, np.float32) for (_, _, _, _, l1, l2) in reqs]
    arr = F.Server.request_array([F.Server.request(m, sta_of(s1, w), sta_of(s2, w), w, l1, l2, o)
                                  for (m, s1, s2, w, l1, l2), o in zip(reqs, outs)])
    return arr, outs


def _errors(O, F, reqs, outs, win, n_max, per_method=2):
    """Max relative error per method over a few requests with short windows."""
    err = {}
    for (m, s1, s2, w, l1, l2), o in zip(reqs, outs):
        N = win[w].shape[1]
        name = METHOD_NAME[m]
        if N > n_max or len(err.get(name, [])) >= per_method:
            continue
        y64 = _oracle_call(O, m, win[w][s1], win[w][s2], l1, l2)
        err.setdefault(name, []).append(float(O.relerr(o[None], y64[None]).max()))
    return {k: max(v) for k, v in err.items()}


def autotune(F, max_nz=1 << 20):
    """Measured padded-length table on this GPU (fpcc_autotune), outside any timed region."""
    ctx = F.Context(0)
    t0 = time.perf_counter()
    import tempfile
    with tempfile.TemporaryDirectory(prefix="fpcc-tune-") as d:
        table = ctx.autotune(min_nz=512, max_nz=max_nz, reuse=8.0, path=os.path.join(d, "autotune.json"))
    ctx.close()
    return {"lengths_timed": len(table) if table else None, "seconds": time.perf_counter() - t0}


def _uneven_case(n, seed, tag):
    """n pairs of windows (log-uniform lengths 2^12-2^17, 5 % gaps) and their
    requests [(method, s1, s2, window, Lag1, Lag2)]."""
    from fastpcc_gb300 import synth
    rng = np.random.default_rng(seed)
    lengths = np.round(2.0 ** rng.uniform(12, 17, n)).astype(int)
    win = synth.uneven_windows(lengths, 2, gap_frac=0.05, tag=tag)
    methods = rng.choice(list(MIX_BATCH), size=n, p=list(MIX_BATCH.values()))
    reqs = []
    for i in range(n):
        M = max(1, int(rng.uniform(0.01, 0.10) * lengths[i]))
        reqs.append((int(methods[i]), 0, 1, i, -M, M))
    return win, reqs


def _uneven_server(F, win, fmt, nz_mode):
    srv = F.Server(hbm_budget=150 << 30, max_batch=8192, fmt=fmt, nz_mode=nz_mode)
    for w in range(len(win)):
        srv.put(0, w, win[w][0])
        srv.put(1, w, win[w][1])
    return srv


def uneven_profile(F, path, n_pairs=500, fmt=2, nz_mode=1):
    """One cold pass of the uneven batch under the torch profiler (CUDA
    activity): the chrome trace goes to `path`; returns the kernel table (launches,
    total time, share of kernel time) and the overlap of the server's streams
    (busy time per stream, the union over streams, idle time of the span)."""
    import collections
    import re
    import torch
    from torch.profiler import profile, ProfilerActivity
    wwin, wreqs = _uneven_case(60, 141, "uneven-batch-warmup")
    srv = _uneven_server(F, wwin, fmt, nz_mode)
    arr, _ = _serve_requests(F, srv, wreqs, lambda s, w: s)
    srv.submit_many(arr)
    srv.drain()
    srv.close()
    win, reqs = _uneven_case(n_pairs, 41, "uneven-batch")
    for rep in range(2):   # the profiler's first session records no device activity
        srv = _uneven_server(F, win if rep else wwin, fmt, nz_mode)
        arr, _ = _serve_requests(F, srv, reqs if rep else wreqs, lambda s, w: s)
        torch.cuda.synchronize()
        with profile(activities=[ProfilerActivity.CPU, ProfilerActivity.CUDA]) as prof:
            t0 = time.perf_counter()
            srv.submit_many(arr)
            srv.drain()
            wall = time.perf_counter() - t0
        srv.close()
    prof.export_chrome_trace(path)
    with open(path) as f:
        ev = json.load(f)["traceEvents"]
    ops = sorted([e for e in ev if e.get("cat") in ("kernel", "gpu_memcpy", "gpu_memset") and "dur" in e],
                 key=lambda e: e["ts"])
    t_a, t_b = ops[0]["ts"], max(e["ts"] + e["dur"] for e in ops)
    busy, cur_s, cur_e = 0.0, None, None
    for e in ops:
        s, en = e["ts"], e["ts"] + e["dur"]
        if cur_e is None or s > cur_e:
            if cur_e is not None:
                busy += cur_e - cur_s
            cur_s, cur_e = s, en
        else:
            cur_e = max(cur_e, en)
    busy += cur_e - cur_s
    per_stream = collections.defaultdict(float)
    table = collections.defaultdict(lambda: [0, 0.0])
    for e in ops:
        per_stream[e["args"].get("stream")] += e["dur"]
        name = re.sub(r"\(.*$", "", e["name"].replace("(anonymous namespace)::", "").replace("fpcc::", "")
                      .replace("void ", ""))
        name = re.sub(r"Radices<[^>]*>", "R", name)
        table[name][0] += 1
        table[name][1] += e["dur"]
    total = sum(v[1] for v in table.values())
    top = sorted(table.items(), key=lambda kv: -kv[1][1])[:25]
    return {"wall_ms": wall * 1e3, "gpu_span_ms": (t_b - t_a) / 1e3, "gpu_busy_union_ms": busy / 1e3,
            "gpu_idle_ms": (t_b - t_a - busy) / 1e3, "operations": len(ops),
            "busy_ms_per_stream": {str(k): round(v / 1e3, 3) for k, v in per_stream.items()},
            "kernels": [{"name": k, "launches": v[0], "total_ms": round(v[1] / 1e3, 3),
                         "share": round(v[1] / total, 4)} for k, v in top],
            "note": "times under the profiler; wall time of the same pass without it is the bench's batched leg"}


def uneven_batch_leg(F, n_pairs=500, fmt=2, nz_mode=1):
    """500 pairs with window lengths log-uniform in 2^12-2^17 (5 % of samples in
    gaps), lags +-(1-10 %) of the length, methods 40/30/20/10 % PCC2 / 1-bit /
    GNCC / PCC1: the whole batch through the server (products computed on
    demand, pair stages packed per method and padded length) against the plain
    per-pair drop-in."""
    from oracle import oracle as O
    from fastpcc_gb300 import synth

    case = _uneven_case

    def server(win):
        return _uneven_server(F, win, fmt, nz_mode)

    # warm-up on another batch of the same distribution (other lengths), through
    # both arms: loads every kernel once in this process; each timed arm below
    # still starts with its own per-length caches empty (new lengths, new server)
    wwin, wreqs = case(60, 141, "uneven-batch-warmup")
    for (m, s1, s2, w, l1, l2) in wreqs:
        _plain_call(F, m, wwin[w][s1][None], wwin[w][s2][None], l1, l2)
    wsrv = server(wwin)
    warr, _ = _serve_requests(F, wsrv, wreqs, lambda s, w: s)
    wsrv.submit_many(warr)
    wsrv.drain()
    wsrv.close()
    win, reqs = case(n_pairs, 41, "uneven-batch")
    # plain: every pair through its method's plain drop-in
    t0 = time.perf_counter()
    for (m, s1, s2, w, l1, l2) in reqs:
        _plain_call(F, m, win[w][s1][None], win[w][s2][None], l1, l2)
    t_plain = time.perf_counter() - t0
    # batched: three cold passes, each on a fresh server (no products, no cached
    # lengths), the median reported; then a resident pass on the last server
    colds = []
    for rep in range(3):
        srv = server(win)
        arr, outs = _serve_requests(F, srv, reqs, lambda s, w: s)
        t0 = time.perf_counter()
        srv.submit_many(arr)
        srv.drain()
        colds.append(time.perf_counter() - t0)
        if rep < 2:
            srv.close()
    t_cold = statistics.median(colds)
    st = srv.stats()
    srv.reset_stats()
    t0 = time.perf_counter()
    srv.submit_many(arr)
    srv.drain()
    t_warm = time.perf_counter() - t0
    srv.close()
    err = _errors(O, F, reqs, outs, win, n_max=1 << 14)
    return {"workload": f"{n_pairs} pairs, window lengths log-uniform 2^12-2^17, 5 % gaps, lags +-(1-10 %), "
                        "methods 40/30/20/10 % PCC2/1-bit/GNCC/PCC1",
            "plain": {"value": n_pairs / t_plain, "unit": UNIT},
            "batched": {"value": n_pairs / t_cold, "unit": UNIT, "batches": st["batches"],
                        "cold_passes_s": colds,
                        "what": "station products computed on demand, pair stages packed (median of 3 fresh servers)"},
            "batched_resident": {"value": n_pairs / t_warm, "unit": UNIT, "what": "second pass, products resident"},
            "speedup_vs_plain": t_plain / t_cold, "spectra": ("f32", "f16", "i16")[fmt],
            "warmup": "60 pairs of another seed through both arms first (kernels loaded; no cached lengths)",
            "max_rel_err": err, "err_sample": "2 requests per method with N <= 2^14 against the FP64 oracle"}


def serving_leg(F, n_sta=200, n_win=8, n_req=4000, fmt=2, rates=(1e3, 1e4, 1e5, 1e6), nz_mode=1):
    """Request stream over a 200-station pool: window lengths lognormal (median
    2^15, sigma 1) clipped to 2^12-2^18, lags +-(1-10 %), methods 38/28.5/19/9.5/5 %
    PCC2 / 1-bit / GNCC / PCC1 / wavelet PCC; Poisson arrivals swept over the
    offered rates, products cached under a 150 GB budget; the plain per-request
    drop-in timed on a sample of the same requests."""
    from oracle import oracle as O
    from fastpcc_gb300 import synth
    rng = np.random.default_rng(43)
    lengths = np.clip(np.round(np.exp(rng.normal(np.log(2.0 ** 15), 1.0, n_win))), 2 ** 12, 2 ** 18).astype(int)
    win = synth.uneven_windows(lengths, n_sta, tag="serving")
    reqs = synth.mixed_requests(n_req, n_sta, lengths, MIX_STREAM, seed=6)
    n_plain = 150
    # warm-up on a small pool of other lengths through both arms (kernels loaded;
    # the timed server starts with no products and no cached lengths)
    wl = np.array([5003, 12007, 30011])
    wwin = synth.uneven_windows(wl, 8, tag="serving-warmup")
    wreqs = synth.mixed_requests(60, 8, wl, MIX_STREAM, seed=61)
    for (m, s1, s2, w, l1, l2) in wreqs:
        _plain_call(F, m, wwin[w][s1][None], wwin[w][s2][None], l1, l2)
    wsrv = F.Server(hbm_budget=8 << 30, max_batch=8192, fmt=fmt, wavelet=WAVELET, nz_mode=nz_mode)
    for w in range(len(wl)):
        for k in range(8):
            wsrv.put(k, w, wwin[w][k])
    warr, _ = _serve_requests(F, wsrv, wreqs, lambda s, w: s)
    wsrv.submit_many(warr)
    wsrv.drain()
    wsrv.close()
    t0 = time.perf_counter()
    for (m, s1, s2, w, l1, l2) in reqs[:n_plain]:
        _plain_call(F, m, win[w][s1][None], win[w][s2][None], l1, l2)
    t_plain = time.perf_counter() - t0
    srv = F.Server(hbm_budget=150 << 30, max_batch=8192, fmt=fmt, wavelet=WAVELET, nz_mode=nz_mode)
    for w in range(n_win):
        for k in range(n_sta):
            srv.put(k, w, win[w][k])
    arr, outs = _serve_requests(F, srv, reqs, lambda s, w: s)
    t0 = time.perf_counter()
    srv.submit_many(arr)
    srv.drain()
    t_cold = time.perf_counter() - t0
    srv.reset_stats()
    t0 = time.perf_counter()
    srv.submit_many(arr)
    srv.drain()
    t_warm = time.perf_counter() - t0
    st_w = srv.stats()
    sweep = []
    for r in rates:
        cnt = int(min(n_req, max(500, r * 1.0)))
        srv.reset_stats()
        t0 = time.perf_counter()
        srv.submit_many(arr, poisson_rate=r, seed=int(r), count=cnt)
        srv.drain()
        dt = time.perf_counter() - t0
        st = srv.stats()
        sweep.append({"offered": r, "requests": cnt, "achieved": cnt / dt, "p50_ms": st["p50_ms"],
                      "p99_ms": st["p99_ms"], "max_ms": st["max_ms"], "batches": st["batches"]})
    hbm = srv.stats()["hbm_used"]
    srv.close()
    err = _errors(O, F, reqs, outs, win, n_max=20000)
    plain = n_plain / t_plain
    return {"workload": f"{n_req} requests, {n_sta} stations x {n_win} windows, lengths {sorted(lengths.tolist())}, "
                        "lags +-(1-10 %), methods 38/28.5/19/9.5/5 % PCC2/1-bit/GNCC/PCC1/WPCC",
            "plain": {"value": plain, "unit": UNIT, "sample": f"first {n_plain} requests"},
            "served_saturation": {"value": n_req / t_warm, "unit": UNIT, "p50_ms": st_w["p50_ms"],
                                  "p99_ms": st_w["p99_ms"], "batches": st_w["batches"],
                                  "what": "all requests at once, products resident"},
            "served_cold": {"value": n_req / t_cold, "unit": UNIT, "what": "products computed on demand"},
            "speedup_vs_plain": (n_req / t_warm) / plain, "poisson": sweep, "hbm_used_bytes": hbm,
            "warmup": "60 requests over 8 stations x 3 other lengths through both arms first",
            "spectra": ("f32", "f16", "i16")[fmt], "max_rel_err": err,
            "err_sample": "2 requests per method with N <= 20000 against the FP64 oracle"}


def _time_ms(torch, stream, fn, reps=3):
    """Average CUDA-event time of fn() on `stream` after one untimed call."""
    fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def method_legs(F, torch, ctx, stream, dev, x, d_x, pairs, Nz, peak):
    """Pair-stage (and station-stage) kernels of every method on the all-pairs
    workload, timed with CUDA events, against their rooflines: HBM bytes for the
    FFT methods, sqrt throughput for PCC1, bit operations for the popcount form."""
    N, L, rows, P = N_SAMP, 2 * LAG + 1, x.shape[0], pairs.shape[0]
    d_pairs = torch.from_numpy(pairs).to(dev)
    d_y = torch.empty((P, L), dtype=torch.float32, device=dev)
    out = {}

    def hbm(name, ms, alg_bytes, units):
        out[name] = {"kernel_ms": ms, "alg_bytes": alg_bytes, "achieved_GBs": alg_bytes / ms / 1e6,
                     "frac_of_measured_hbm": alg_bytes / ms / 1e6 / peak, "correlations": units}

    # PCC2 station stage (fused analytic + normalisation + DFT_Nz), F32 and F16 spectra
    for fmt, esz, tag in ((F.F32, 8, "f32"), (F.F16, 4, "f16"), (F.I16, 4, "i16")):
        lds = Nz + 4 if fmt == F.I16 else Nz
        spec = torch.empty((rows, lds * esz // 4), dtype=torch.float32, device=dev)
        ms = _time_ms(torch, stream, lambda: ctx.station_stage(F.PCC2, d_x.data_ptr(), N, rows, N, Nz, fmt,
                                                               F.AMP_F_REG, spec.data_ptr(), lds))
        out[f"pcc2_station_{tag}"] = {"kernel_ms": ms, "alg_bytes": rows * (4 * N + esz * lds),
                                      "achieved_GBs": rows * (4 * N + esz * lds) / ms / 1e6, "windows": rows}
        if fmt != F.F32:
            ms = _time_ms(torch, stream, lambda: ctx.pair_stage(F.PCC2, spec.data_ptr(), lds, fmt, d_pairs.data_ptr(),
                                                                P, N, Nz, -LAG, LAG, d_y=d_y.data_ptr(), ldy=L))
            hbm(f"pcc2_pairs_{tag}", ms, P * (2 * lds * esz + 4 * L), P)
            from oracle import oracle as O
            sel = np.random.default_rng(4).choice(P, 6, replace=False)
            y64 = O.pcc2(x[pairs[sel, 0]], x[pairs[sel, 1]], -LAG, LAG)
            out[f"pcc2_pairs_{tag}"]["max_rel_err"] = float(
                O.relerr(d_y[torch.from_numpy(sel).to(dev)].cpu().numpy(), y64).max())
        del spec
    # GNCC: half spectra + energy rows (FP64 prefix sums and the float
    # normalisation tables: two 4-byte table entries per lag); the same pairs
    # with rows of prefix sums only (two FP64 sums per lag) beside it
    H = Nz // 2 + 1
    half = torch.empty((rows, 2 * H), dtype=torch.float32, device=dev)
    E = torch.empty((rows, 2 * (N + 1)), dtype=torch.float64, device=dev)
    ctx.station_stage(F.GNCC, d_x.data_ptr(), N, rows, N, Nz, F.F32, 0, half.data_ptr(), H)
    for name, ldE, per_lag in (("gncc_pairs", 2 * (N + 1), 8), ("gncc_pairs_sums_only", N + 1, 16)):
        ctx.energy_stage(d_x.data_ptr(), N, rows, N, E.data_ptr(), ldE)
        ms = _time_ms(torch, stream, lambda: ctx.pair_stage(F.GNCC, half.data_ptr(), H, F.F32, d_pairs.data_ptr(),
                                                            P, N, Nz, -LAG, LAG, d_E=E.data_ptr(), ldE=ldE,
                                                            d_y=d_y.data_ptr(), ldy=L))
        hbm(name, ms, P * (2 * H * 8 + per_lag * L + 4 * L), P)
    del E
    # 1-bit, DFT form: station 1 signs x >= 0, station 2 signs x > 0 (rows offset by `rows`)
    half2 = torch.empty((2 * rows, 2 * H), dtype=torch.float32, device=dev)
    ctx.station_stage(F.CC1B, d_x.data_ptr(), N, rows, N, Nz, F.F32, F.SIGN_GE, half2.data_ptr(), H)
    ctx.station_stage(F.CC1B, d_x.data_ptr(), N, rows, N, Nz, F.F32, F.SIGN_GT, half2[rows:].data_ptr(), H)
    p2 = pairs.copy()
    p2[:, 1] += rows
    d_p2 = torch.from_numpy(p2).to(dev)
    ms = _time_ms(torch, stream, lambda: ctx.pair_stage(F.CC1B, half2.data_ptr(), H, F.F32, d_p2.data_ptr(), P, N, Nz,
                                                        -LAG, LAG, d_y=d_y.data_ptr(), ldy=L))
    hbm("cc1b_pairs_dft", ms, P * (2 * H * 8 + 4 * L), P)
    del half, half2
    # 1-bit, exact popcount form: XOR + popcount of 32-bit words over every overlap
    nw = (N + 31) // 32
    bits = torch.empty((2 * rows, nw), dtype=torch.int32, device=dev)
    ctx.station_stage(F.CC1B_POPCOUNT, d_x.data_ptr(), N, rows, N, 0, F.F32, F.SIGN_GE, bits.data_ptr(), nw)
    ctx.station_stage(F.CC1B_POPCOUNT, d_x.data_ptr(), N, rows, N, 0, F.F32, F.SIGN_GT, bits[rows:].data_ptr(), nw)
    ms = _time_ms(torch, stream, lambda: ctx.pair_stage(F.CC1B_POPCOUNT, bits.data_ptr(), nw, F.F32, d_p2.data_ptr(),
                                                        P, N, 0, -LAG, LAG, d_y=d_y.data_ptr(), ldy=L))
    words = P * sum((N - abs(l) + 31) // 32 for l in range(-LAG, LAG + 1))
    out["cc1b_pairs_popcount"] = {"kernel_ms": ms, "word_ops": words, "Gword_ops_per_s": words / ms / 1e6,
                                  "correlations": P}
    del bits
    # PCC1 by direct lag sums, one window (2016 pairs): two square roots per term
    ph = torch.empty((rows, 2 * N), dtype=torch.float32, device=dev)
    ctx.station_stage(F.PCC1, d_x.data_ptr(), N, rows, N, 0, F.F32, F.AMP_F_REG, ph.data_ptr(), N)
    P1 = N_STA * (N_STA - 1) // 2
    ms = _time_ms(torch, stream, lambda: ctx.pair_stage(F.PCC1, ph.data_ptr(), N, F.F32, d_pairs.data_ptr(), P1, N,
                                                        0, -LAG, LAG, d_y=d_y.data_ptr(), ldy=L), reps=1)
    terms = P1 * sum(N - abs(l) for l in range(-LAG, LAG + 1))
    clk = 2.07e9
    sfu_peak = 152 * 16 * clk / 2.0    # 16 special-function results per SM per clock, 2 per term
    out["pcc1_pairs"] = {"kernel_ms": ms, "terms": terms, "Gterms_per_s": terms / ms / 1e6,
                         "frac_of_sfu_peak": terms / ms * 1e3 / sfu_peak, "correlations": P1,
                         "rule": "AmpNormf (regularised moduli): two square roots per term",
                         "sfu_peak_assumed": "152 SMs x 16 sqrt/clk x 2.07 GHz, 2 sqrt per term"}
    # the same pairs with the pure-phase rule of the reference GPU path: one
    # reciprocal square root per term
    ctx.station_stage(F.PCC1, d_x.data_ptr(), N, rows, N, 0, F.F32, F.AMP_PURE, ph.data_ptr(), N)
    ms = _time_ms(torch, stream, lambda: ctx.pair_stage(F.PCC1, ph.data_ptr(), N, F.F32, d_pairs.data_ptr(), P1, N,
                                                        0, -LAG, LAG, d_y=d_y.data_ptr(), ldy=L), reps=1)
    from oracle import oracle as O
    y64 = O.pcc1(x[pairs[:2, 0]], x[pairs[:2, 1]], -LAG, LAG, rule=O.AMP_PURE)
    out["pcc1_pairs_pure_rule"] = {"kernel_ms": ms, "terms": terms, "Gterms_per_s": terms / ms / 1e6,
                                   "frac_of_sfu_peak": terms / ms * 1e3 / (2 * sfu_peak), "correlations": P1,
                                   "rule": "pure phase x/|x| (reference GPU path): one reciprocal square root "
                                           "per term",
                                   "max_rel_err": float(O.relerr(d_y[:2].cpu().numpy(), y64).max())}
    del ph, d_y
    return out


def wpcc_leg(F, torch, ctx, stream, dev, peak, n_pairs=16, n_win=24, N=65536, lag=4000):
    """Wavelet PCC on its configuration (16 station pairs x 24 windows x 65536
    samples at 20 Hz, Morlet, 40 scales over 0.02-5 Hz, lags +-4000): station
    and pair stages timed, pair stage against the HBM roofline."""
    from fastpcc_gb300 import synth
    a, b, _ = synth.wavelet_pairs(n_pairs=n_pairs, n_windows=n_win, N=N, tag="bench/wpcc")
    x = np.ascontiguousarray(np.concatenate([a.reshape(-1, N), b.reshape(-1, N)]))
    P = n_pairs * n_win
    plan = F.WpccPlan(ctx, N, -lag, lag, WAVELET["pmin"], WAVELET["pmax"], V=WAVELET["V"], type=WAVELET["type"])
    S, Nz, L = plan.S, plan.Nz, plan.L
    d_x = torch.from_numpy(x).to(dev)
    d_P = torch.empty((2 * P, S * Nz * 2), dtype=torch.float32, device=dev)
    pairs = np.stack([np.arange(P), P + np.arange(P)], 1).astype(np.int32)
    d_pairs = torch.from_numpy(pairs).to(dev)
    d_y = torch.empty((P, L), dtype=torch.float32, device=dev)
    ms_st = _time_ms(torch, stream, lambda: plan.station_stage(d_x.data_ptr(), N, 2 * P, d_P.data_ptr()), reps=1)
    ms = _time_ms(torch, stream, lambda: plan.pair_stage(d_P.data_ptr(), d_pairs.data_ptr(), P, d_y.data_ptr(), L))
    alg = P * (2 * S * Nz * 8 + 4 * L)
    from oracle import oracle as O
    k = 0
    y64 = O.wpcc(x[k][None], x[P + k][None], -lag, lag, WAVELET["pmin"], WAVELET["pmax"], V=WAVELET["V"],
                 wtype=WAVELET["type"])
    err = float(O.relerr(d_y[k:k + 1].cpu().numpy(), y64).max())
    plan.close()
    return {"workload": f"{n_pairs} pairs x {n_win} windows x {N} samples, S={S}, Nz={Nz}, lags +-{lag}",
            "station_ms": ms_st, "station_windows": 2 * P, "pair_kernel_ms": ms, "correlations": P,
            "correlations_per_s_device": P / ((ms + ms_st) / 1e3), "alg_bytes": alg,
            "achieved_GBs": alg / ms / 1e6, "frac_of_measured_hbm": alg / ms / 1e6 / peak, "max_rel_err": err}


def multi_station_leg(F, torch, ctx, stream, dev, peak, n=512, lo=24000, hi=32000):
    """The packed analytic-signal stage (fpcc_station_stage_multi, PCC1 phase
    signals) on n windows of lengths uniform in [lo, hi) with 5 % of samples in
    gaps: double-float transforms (the gapped path) and FP32 transforms on the
    same windows; kernel spectra cached (a second call, as in serving).  The
    class length is 65536 for these lengths: per window 1.5 transforms of four
    radix-16 passes, each pass moving 32 bytes per point (double-float) or 16
    (FP32), the rate reported against the measured copy bandwidth."""
    from fastpcc_gb300 import synth
    rng = np.random.default_rng(17)
    lengths = np.sort(rng.integers(lo, hi, n))
    win = synth.uneven_windows(lengths, 1, gap_frac=0.05, tag="multi-station")
    Nmax = int(lengths.max())
    x = np.zeros((n, Nmax), np.float32)
    for i in range(n):
        x[i, :lengths[i]] = win[i][0]
    d_x = torch.from_numpy(x).to(dev)
    d_o = torch.empty((n, 2 * Nmax), dtype=torch.float32, device=dev)
    M = 65536
    out = {"workload": f"{n} windows, lengths {lo}-{hi} (class length {M}), 5 % gaps, PCC1 phase signals"}
    for name, f64 in (("double_float", 1), ("fp32", 0)):
        rows = [(d_x.data_ptr() + i * Nmax * 4, int(lengths[i]), 0, f64) for i in range(n)]
        ms = _time_ms(torch, stream, lambda: ctx.station_stage_multi(F.PCC1, rows, F.F32, F.AMP_F_REG,
                                                                     d_o.data_ptr(), Nmax), reps=3)
        esz = 32 if f64 else 16             # bytes a point-pass reads and writes
        pp = n * 1.5 * M * 4                # point-passes: 1.5 transforms x 4 radix-16 passes per window
        out[name] = {"kernel_ms": ms, "windows_per_s": n / ms * 1e3, "point_passes_per_s": pp / ms * 1e3,
                     "pass_bytes_GBs": pp * esz / ms / 1e6, "pass_frac_of_measured_hbm": pp * esz / ms / 1e6 / peak,
                     "note": "the whole stage (load, split, store, row statistics, phase store) over the pass bytes"}
    return out


def stack_leg(F, torch, ctx, stream, dev, d_y, n_sta, n_win, L, peak):
    """Stacks over the windows of every channel pair, read in place from the
    window-major rows of the all-pairs pair stage (row w * P + p): linear,
    phase-weighted and time-scale phase-weighted (Morlet, 4 voices, periods
    8-1000 samples, 28 scales, nu = 2), timed with CUDA events; the linear stack
    against the HBM roofline (it reads every correlation once)."""
    from oracle import oracle as O
    P = n_sta * (n_sta - 1) // 2
    K = n_win
    d_o = torch.empty((P, L), dtype=torch.float32, device=dev)
    kw = dict(ldg=L, ldj=P * L, nu=2.0, pmin=8.0, pmax=1000.0, V=4, type=-1)
    out = {"workload": f"{P} channel pairs x {K} windows x {L} lags (the all-pairs output, in place)"}
    for name, mode, reps in (("linear", F.STACK_LINEAR, 3), ("pws", F.STACK_PWS, 3), ("tspws", F.STACK_TSPWS, 1)):
        ms = _time_ms(torch, stream, lambda: ctx.stack(mode, d_y.data_ptr(), L, K, L, P, d_o.data_ptr(), L, **kw),
                      reps=reps)
        out[name] = {"kernel_ms": ms, "stacks_per_s": P / ms * 1e3, "traces_per_s": P * K / ms * 1e3}
        if mode != F.STACK_TSPWS:
            y = d_o[:2].cpu().numpy()
            yy = d_y.view(K, P, L)[:, :2].cpu().numpy()
            out[name]["max_rel_err"] = max(float(O.relerr(y[k][None], O.stack(yy[:, k], mode, 2.0)[None])[0])
                                           for k in range(2))
    alg = P * K * L * 4 + P * L * 4
    out["linear"].update({"alg_bytes": alg, "achieved_GBs": alg / out["linear"]["kernel_ms"] / 1e6,
                          "frac_of_measured_hbm": alg / out["linear"]["kernel_ms"] / 1e6 / peak})
    out["tspws"]["scales"] = 28
    return out


def _cpu_rate(fn, x1, x2, l1, l2, budget_s, batch):
    """Correlations/s of fn over batches of (x1, x2) rows until budget_s has passed
    (at least one batch); x1, x2 are callables giving the next batch."""
    done, t0 = 0, time.perf_counter()
    while True:
        a, b = x1(), x2()
        fn(a, b, l1, l2)
        done += a.shape[0]
        dt = time.perf_counter() - t0
        if dt >= budget_s:
            return done / dt, done, dt


def cpu_baseline(x, pairs, budget_s=10.0):
    """The reference's pcc2_set arithmetic (single-precision transforms, seven per
    correlation; oracle/cpuref.py) on the host cores over random pair-windows of
    the all-pairs workload."""
    from oracle import cpuref
    threads = cpuref.threads()
    rng = np.random.default_rng(7)
    sel = []
    batch = 16 * threads          # as the reference arm's steps

    def take(col):
        if col == 0:
            sel.append(rng.choice(pairs.shape[0], batch, replace=False))
        return x[pairs[sel[-1], col]]

    cpuref.pcc2_set(x[pairs[:batch, 0]], x[pairs[:batch, 1]], -LAG, LAG)    # warm: thread pool, FFT plans
    rate, done, dt = _cpu_rate(cpuref.pcc2_set, lambda: take(0), lambda: take(1), -LAG, LAG, budget_s, batch)
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "dtype": "f32",
            "cpu_model": cpuref.cpu_model(),
            "sample": f"{done} random pair-windows of the all-pairs workload, {dt:.1f} s: the reference's pcc2_set "
                      f"steps (src/FFTapps.c:785-881) in single precision, seven transforms per correlation at the "
                      f"reference padding 2^ceil(log2(N+M)), scipy FFT on {threads} threads in place of FFTW"}


def cpu_methods_leg(x, pairs, budget_s=4.0):
    """Per-method CPU rates of the reference's arithmetic (oracle/cpuref.py): the plain config (24 windows x 36,000, +-3000, every
    window) and sampled pair-windows of the all-pairs config."""
    from fastpcc_gb300 import synth
    from oracle import cpuref
    threads = cpuref.threads()
    out = {"cores": threads, "cpu_model": cpuref.cpu_model(), "unit": UNIT,
           "note": "single precision for PCC2, 1-bit and PCC1 (double sums), double for GNCC and WPCC, as the "
                   "reference's CPU paths; scipy FFT in place of FFTW"}
    a, b = synth.plain_pair(N=36000, n_windows=24, delay=150, tag="config1")
    c1 = {}
    for name, fn in cpuref.METHODS.items():
        t0 = time.perf_counter()
        fn(a, b, -3000, 3000)
        c1[name] = 24 / (time.perf_counter() - t0)
    out["config1"] = {"workload": "24 windows x 36000 samples, lags +-3000, every window", **c1}
    rng = np.random.default_rng(9)
    c2 = {}
    for name, fn in cpuref.METHODS.items():
        batch = threads if name == "pcc1" else 16 * threads
        sel = []

        def take(col):
            if col == 0:
                sel.append(rng.choice(pairs.shape[0], batch, replace=False))
            return x[pairs[sel[-1], col]]

        rate, done, dt = _cpu_rate(fn, lambda: take(0), lambda: take(1), -LAG, LAG, budget_s, batch)
        c2[name] = {"value": rate, "sample": f"{done} random pair-windows, {dt:.1f} s"}
    out["allpairs"] = {"workload": f"all-pairs: {N_SAMP} samples, lags +-{LAG}, random pair-windows", **c2}
    nw = max(2, threads)
    w1, w2, _ = synth.wavelet_pairs(n_pairs=nw, n_windows=1, N=65536, tag="bench/wpcc-cpu")
    w1, w2 = w1.reshape(-1, 65536), w2.reshape(-1, 65536)
    kw = dict(pmin=WAVELET["pmin"], pmax=WAVELET["pmax"], V=WAVELET["V"], wtype=WAVELET["type"])
    cpuref.wpcc_set(w1[:1], w2[:1], -4000, 4000, **kw)        # wavelet spectra built outside the timing
    t0 = time.perf_counter()
    cpuref.wpcc_set(w1, w2, -4000, 4000, **kw)
    dt = time.perf_counter() - t0
    out["wpcc"] = {"value": nw / dt, "sample": f"{nw} pair-windows of the wavelet config (65536 samples, 40 scales, "
                                               f"+-4000), double precision, {dt:.1f} s"}
    return out


def config1_leg(F, cpu=None):
    """The plain config: stations A and B, 24 windows of 36,000 samples, lags
    +-3000, padded length 2^17; GNCC, 1-bit, PCC2 and PCC1 for the 24 same-index
    window pairs through the batched host entry point and the plain per-pair
    drop-in, each against the FP64 oracle."""
    from fastpcc_gb300 import synth
    from oracle import oracle as O
    a, b = synth.plain_pair(N=36000, n_windows=24, delay=150, tag="config1")
    l1, l2, nz = -3000, 3000, 1 << 17
    calls = {"gncc": (F.GNCC, O.gncc), "cc1b": (F.CC1B, O.cc1b), "pcc2": (F.PCC2, O.pcc2), "pcc1": (F.PCC1, O.pcc1)}
    out = {"workload": "24 windows x 36000 samples, lags +-3000, Nz = 131072 (FFT methods)", "unit": UNIT}
    for name, (m, orc) in calls.items():
        mode = nz if m != F.PCC1 else F.NZ_FAST
        r = {}
        for arm, plain in (("batched", False), ("plain", True)):
            # warm at the full size (kernels, plans and the buffers of 24 windows),
            # then the median of three calls
            F.correlate(m, a, b, l1, l2, plain=plain, nz_mode=mode)
            ts = []
            for _ in range(3):
                t0 = time.perf_counter()
                y = F.correlate(m, a, b, l1, l2, plain=plain, nz_mode=mode)
                ts.append(time.perf_counter() - t0)
            r[arm] = 24 / float(np.median(ts))
            k = 24 if m != F.PCC1 else 3
            r[f"max_rel_err_{arm}"] = float(O.relerr(y[:k], orc(a[:k], b[:k], l1, l2)).max())
        r["err_sample"] = "all 24 windows" if m != F.PCC1 else "3 windows"
        if cpu is not None:
            r["cpu"] = cpu["config1"].get(name)
        out[name] = r
    return out


def run_reference(args):
    """The reference arm: the reference's pcc2_set arithmetic on the host cores
    (oracle/cpuref.py: single-precision transforms, seven per correlation, all
    host threads), random pair-windows of the same all-pairs workload."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from fastpcc_gb300 import synth
    from oracle import cpuref
    n_sta, n_win = args.stations, args.windows
    x, _ = synth.all_pairs(n_stations=n_sta, n_windows=n_win, N=N_SAMP)
    x = x.reshape(n_sta * n_win, N_SAMP)
    pairs = all_pairs_index(n_sta, n_win)
    threads = cpuref.threads()
    rng = np.random.default_rng(11)
    per_step = 16 * threads
    for _ in range(args.warmup):
        sel = rng.choice(pairs.shape[0], threads, replace=False)
        cpuref.pcc2_set(x[pairs[sel, 0]], x[pairs[sel, 1]], -LAG, LAG)
    times = []
    for _ in range(args.steps):
        sel = rng.choice(pairs.shape[0], per_step, replace=False)
        t0 = time.perf_counter()
        cpuref.pcc2_set(x[pairs[sel, 0]], x[pairs[sel, 1]], -LAG, LAG)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = per_step * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded noise + shared band-passed component)",
        "config": {"workload": f"all-pairs PCC2: {n_sta} stations x {n_win} windows x {N_SAMP} samples, "
                               f"lags +-{LAG}", "sample_per_step": per_step},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "dtype": "f32",
                         "cpu_model": cpuref.cpu_model(),
                         "sample": f"{per_step} random pair-windows per step: the reference's pcc2_set steps "
                                   f"(src/FFTapps.c:785-881) in single precision, seven transforms per "
                                   f"correlation, scipy FFT on {threads} threads in place of FFTW (the reference's "
                                   f"own sources are not on this host)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import fastpcc_gb300 as F

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    F.build()
    if args.wpcc_only:
        stream = torch.cuda.Stream(device=torch.device("cuda", local))
        ctx = F.Context(local)
        ctx.set_stream(stream.cuda_stream)
        n_win = args.windows if args.windows != N_WIN else 24
        print(json.dumps({"wpcc": wpcc_leg(F, torch, ctx, stream, torch.device("cuda", local), measured_peaks()[0],
                                           n_win=n_win)}), flush=True)
        ctx.close()
        return
    if args.multi_only:
        stream = torch.cuda.Stream(device=torch.device("cuda", local))
        ctx = F.Context(local)
        ctx.set_stream(stream.cuda_stream)
        print(json.dumps({"multi_station": multi_station_leg(F, torch, ctx, stream, torch.device("cuda", local),
                                                             measured_peaks()[0], n=args.windows * 8)}), flush=True)
        ctx.close()
        return
    if args.profile_uneven:
        autotune(F)
        fmt = {"f32": F.F32, "f16": F.F16, "i16": F.I16}[args.fmt]
        print(json.dumps({"uneven_profile": uneven_profile(F, args.profile_uneven, fmt=fmt, nz_mode=F.NZ_TUNED)}),
              flush=True)
        return
    if args.mixed_only:
        fmt = {"f32": F.F32, "f16": F.F16, "i16": F.I16}[args.fmt]
        tune = autotune(F)
        print(json.dumps({"autotune": tune,
                          "uneven_batch": uneven_batch_leg(F, fmt=fmt, nz_mode=F.NZ_TUNED),
                          "uneven_batch_fast_nz": uneven_batch_leg(F, fmt=fmt, nz_mode=F.NZ_FAST),
                          "serving": serving_leg(F, fmt=fmt, nz_mode=F.NZ_TUNED)}), flush=True)
        return
    n_sta, n_win = args.stations, args.windows
    from fastpcc_gb300 import partition, synth
    # weak scaling: the job is n_sta stations x (n_win x world) windows, and the
    # partitioner deals each rank n_win of them (no product computed twice, no
    # data-path collective); the rank synthesises and correlates its own windows
    shard = partition.shard_all_pairs(n_sta, n_win * world, world)[rank]
    x, _ = synth.all_pairs(n_stations=n_sta, n_windows=len(shard.windows), N=N_SAMP, tag=f"all-pairs/rank{rank}")
    x = np.ascontiguousarray(x.reshape(n_sta * len(shard.windows), N_SAMP))
    pairs = partition.shard_rows(shard, n_sta)
    assert world > 1 or np.array_equal(pairs, all_pairs_index(n_sta, n_win))
    P = pairs.shape[0]
    L = 2 * LAG + 1
    fmt = {"f32": F.F32, "f16": F.F16, "i16": F.I16}[args.fmt]
    Nz = F.choose_nz(N_SAMP, -LAG, LAG, F.NZ_FAST)
    esz = 8 if fmt == F.F32 else 4

    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    ctx = F.Context(local)
    ctx.set_stream(stream.cuda_stream)
    d_x = torch.from_numpy(x).to(dev)
    d_pairs = torch.from_numpy(pairs).to(dev)
    lds = Nz + 4 if fmt == F.I16 else Nz     # int16 rows carry a 16-byte scale header
    d_spec = torch.empty((x.shape[0], lds * esz // 4), dtype=torch.float32, device=dev)
    d_y = torch.empty((P, L), dtype=torch.float32, device=dev)

    def step():
        ctx.station_stage(F.PCC2, d_x.data_ptr(), N_SAMP, x.shape[0], N_SAMP, Nz, fmt, F.AMP_F_REG,
                          d_spec.data_ptr(), lds)
        ctx.pair_stage(F.PCC2, d_spec.data_ptr(), lds, fmt, d_pairs.data_ptr(), P, N_SAMP, Nz, -LAG, LAG,
                       d_y=d_y.data_ptr(), ldy=L)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(args.warmup):
        step()
    barrier()
    if args.methods_only:
        print(json.dumps({"methods": method_legs(F, torch, ctx, stream, dev, x, d_x, pairs, Nz,
                                                 measured_peaks()[0])}), flush=True)
        ctx.close()
        return
    if args.stack_only:
        print(json.dumps({"stacks": stack_leg(F, torch, ctx, stream, dev, d_y, n_sta, n_win, L,
                                              measured_peaks()[0])}), flush=True)
        ctx.close()
        return
    # --- timed: device-resident step ---
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        # untimed load of about a second so that the clock sampler sees the GPU under load
        t_soak = time.perf_counter()
        while time.perf_counter() - t_soak < 1.0:
            step()
            torch.cuda.synchronize(dev)
        launches0 = F.launch_count()
        barrier()
        for i in range(args.steps):
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        barrier()
        launches = F.launch_count() - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_total = sum(step_ms) / 1e3
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_total], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_total = float(tt.item())
    value = P * world * args.steps / t_total

    # --- roofline: the pair kernel alone, timed on its stream ---
    ctx.station_stage(F.PCC2, d_x.data_ptr(), N_SAMP, x.shape[0], N_SAMP, Nz, fmt, F.AMP_F_REG,
                      d_spec.data_ptr(), lds)
    reps = max(3, args.steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(reps):
        ctx.pair_stage(F.PCC2, d_spec.data_ptr(), lds, fmt, d_pairs.data_ptr(), P, N_SAMP, Nz, -LAG, LAG,
                       d_y=d_y.data_ptr(), ldy=L)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    t_pair = e0.elapsed_time(e1) / 1e3 / reps
    alg_bytes = P * (2 * Nz * esz + 4 * L)
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / t_pair / 1e9
    traffic = profiled_traffic()
    if traffic is not None:
        # the profile is of the default workload with F32 spectra
        traffic = traffic * P / float(N_STA * (N_STA - 1) // 2 * N_WIN) if fmt == F.F32 else None
    # FP32 work of the pair kernel per correlation: the Nz/2-point inverse
    # transform (5 H log2 H) and the cross-spectrum packing (4 complex products
    # and 13 further operations per two packed points: 19 per point of Nz/2)
    H = Nz // 2
    flops = P * (5.0 * H * np.log2(H) + 19.0 * H)
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12      # nominal: 152 SMs x 128 FP32 lanes x FMA x 2.07 GHz

    # --- parity spot check against the oracle ---
    err = None
    if rank == 0:
        from oracle import oracle as O
        sel = np.random.default_rng(3).choice(P, 8, replace=False)
        y_gpu = d_y[torch.from_numpy(sel).to(dev)].cpu().numpy()
        y64 = O.pcc2(x[pairs[sel, 0]], x[pairs[sel, 1]], -LAG, LAG)
        err = float(O.relerr(y_gpu, y64).max())

    # --- end to end through the C ABI with host buffers (pinned) ---
    hx = torch.from_numpy(x).pin_memory()
    hp = torch.from_numpy(pairs).pin_memory()
    hy = torch.empty((P, L), dtype=torch.float32).pin_memory()
    hxn, hpn, hyn = hx.numpy(), hp.numpy(), hy.numpy()
    for _ in range(max(3, args.warmup)):   # warm: buffers allocated, GPU under load
        step()
        ctx.allpairs_host(F.PCC2, hxn, hpn, -LAG, LAG, hyn, fmt=fmt)
    e2e_steps = max(5, args.steps)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.allpairs_host(F.PCC2, hxn, hpn, -LAG, LAG, hyn, fmt=fmt)
    barrier()
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": P * world / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(hxn.nbytes + hpn.nbytes),
           "d2h_bytes_per_step": int(hyn.nbytes), "ms_per_step": t_e2e * 1e3}
    if rank == 0:
        e2e["host_link"] = host_link_leg(torch, dev, hx, hy, d_x, d_y, t_e2e)

    # --- plain per-pair drop-in (one launch sequence per pair-window), bounded sample ---
    plain = None
    if rank == 0:
        n_plain = 256
        sel = np.random.default_rng(5).choice(P, n_plain, replace=False)
        a, b = x[pairs[sel, 0]], x[pairs[sel, 1]]
        F.pcc2_highlevel(a[:4], b[:4], -LAG, LAG)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        F.pcc2_highlevel(a, b, -LAG, LAG)
        dt = time.perf_counter() - t0
        plain = {"value": n_plain / dt, "unit": UNIT, "sample": f"{n_plain} pair-windows through pcc2_highlevel"}

    served = None
    if rank == 0 and not args.no_served:
        served = served_leg(F, x, pairs, n_win, L)

    methods = None
    if rank == 0 and not args.no_mixed:
        methods = method_legs(F, torch, ctx, stream, dev, x, d_x, pairs, Nz, peak)
        methods["wpcc_config"] = wpcc_leg(F, torch, ctx, stream, dev, peak)
        methods["multi_station"] = multi_station_leg(F, torch, ctx, stream, dev, peak)

    stacks = None
    if rank == 0 and not args.no_mixed:
        ctx.pair_stage(F.PCC2, d_spec.data_ptr(), lds, fmt, d_pairs.data_ptr(), P, N_SAMP, Nz, -LAG, LAG,
                       d_y=d_y.data_ptr(), ldy=L)
        stacks = stack_leg(F, torch, ctx, stream, dev, d_y, n_sta, n_win, L, peak)

    mixed = None
    if rank == 0 and not args.no_mixed:
        mixed = {"autotune": autotune(F), "uneven_batch": uneven_batch_leg(F, nz_mode=F.NZ_TUNED),
                 "serving": serving_leg(F, nz_mode=F.NZ_TUNED)}

    cpu = None
    cpu_methods = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(x, pairs)
        cpu_methods = cpu_methods_leg(x, pairs)

    config1 = None
    if rank == 0 and not args.no_config1:
        config1 = config1_leg(F, cpu_methods)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if fmt == F.F32 else f"f32 ({args.fmt} spectra)",
            "data": "synthetic (seeded noise + shared band-passed component, per-station delays)",
            "config": {"workload": f"all-pairs PCC2: {n_sta} stations x {n_win} windows x {N_SAMP} samples, "
                                   f"{P} pair-windows per step, lags +-{LAG}",
                       "Nz": Nz, "spectra": args.fmt, "l2": f"inputs {x.nbytes / 1e6:.0f} MB and outputs {P * L * 4 / 1e9:.2f} GB exceed L2; no flush",
                       "parallelism": f"window shards x{world}"},
            "max_rel_err": err,
            "latency_ms": {"p50": statistics.median(step_ms), "p99": float(np.percentile(step_ms, 99)),
                           "what": f"batched step ({x.shape[0]} station windows + {P} correlations)"},
            "plain": plain,
            "served": served,
            "methods": methods,
            "stacks": stacks,
            "mixed": mixed,
            "gpu_launches": int(launches),
            "e2e": e2e,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "traffic_source": "profiles/pcc2_pairs_allpairs.txt (ncu dram__bytes of the pair kernel "
                                           "on 16 windows, scaled by windows); not measured in this run",
                         "kernel": f"PCC2 pair stage ({'tiled' if F.pair_form(Nz) == F.PAIR_TILED else 'block'} "
                                   f"kernel)", "kernel_ms": t_pair * 1e3,
                         "alg_bytes_per_launch": alg_bytes,
                         "fp32": {"flops_per_launch": flops, "achieved_tflops": flops / t_pair / 1e12,
                                  "peak_tflops": fp32_peak, "peak_kind": "nominal",
                                  "frac": flops / t_pair / 1e12 / fp32_peak}},
            "cpu_baseline": cpu,
            "cpu_methods": cpu_methods,
            "config1": config1,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
