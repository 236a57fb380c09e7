"""Benchmark: galaxies/s of the shape-measurement hot path on one GB300.

Workload (default c4_ska_mid_64ch, the configuration the throughput target is stated on): 197
antennas (19,306 baselines) x 960 times at 30 s x 64 channels = 1.19e9 visibilities, 50,000
galaxies at 5-200 uJy with shear g = (0.02, 0.01), seeded synthetic array, catalogue and noise
(no public dataset exists for this path).

A step is one window of consecutive galaxies of the flux-ordered catalogue (default 500)
through the whole path: extraction, fit and removal of every galaxy of the window in catalogue
order, then the re-fit pass over the window's bad galaxies (RadioLensfit2.cpp:597-606 applied to
the window).  Steps walk down the catalogue and the data carry every earlier window's removals,
as one long run does; when the catalogue is exhausted the data are restored and the walk starts
again.  W warm-up windows, then K timed windows.

  value : device-resident run (rlf_obs_process) of the batched mixed-precision path, CUDA events
          on the library's stream around each window, inputs (FP32 data and sky model, larger than
          L2) resident in HBM
  e2e   : windows through the reference-facing C entry point data_processing() with host
          complex128 buffers (catalogue pass + re-fit pass per window), copies inside the timing
  plain : the one-launch-chain-per-galaxy path (batch 1) on a prefix of the catalogue against the
          batched path on the same prefix from the same data: galaxies/s of both and per-galaxy |de|
  cpu_baseline : the oracle (the reference's arithmetic, OpenMP on all host cores) on the first
          galaxies of the same data, both passes, with its fitted e against the GPU's
  --impl reference : the oracle on a bounded sample of the workload, nothing on the GPU
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from radiolensfit2_gb300 import constants as K, synth  # noqa: E402

METRIC = "galaxies/s on 1 GB300: learned+batched vs plain GPU fit at |Δe|≤1e-3; HBM GB/s"
DEFAULT_WORKLOAD = "c4_ska_mid_64ch"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--galaxies", type=int, default=0, help="catalogue size (0 = the workload's)")
    ap.add_argument("--window", type=int, default=500, help="galaxies per step (at most the catalogue)")
    ap.add_argument("--proposal", default="report", choices=["report", "on", "none"],
                    help="learned simplex-start proposal: report = measured path with the reference's start, the "
                         "proposal's effect measured on the prefix beside it; on = measured path with the proposal")
    ap.add_argument("--tune", default="auto", choices=["auto", "none"],
                    help="autotune the batched launch shapes on the first window before the warm-up")
    ap.add_argument("--graphs", type=int, default=0, choices=[0, 1],
                    help="capture each sub-batch's rounds and removal as one CUDA graph")
    ap.add_argument("--batch", type=int, default=1000)
    ap.add_argument("--rounds", type=int, default=0,
                    help="extraction + fit rounds per batch (0 = library default)")
    ap.add_argument("--fit-precision", default="f64", choices=["f64", "mixed"],
                    help="arithmetic of the fit (visibility passes are always mixed)")
    ap.add_argument("--plain-prefix", type=int, default=400,
                    help="galaxies of the plain-vs-batched comparison (0 = none)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5, help="timed e2e windows (at most --steps)")
    ap.add_argument("--cpu-sample-galaxies", type=int, default=-1,
                    help="oracle galaxies of the CPU baseline (-1 = by workload size, 0 = none)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs."""

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap")
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", os.environ.get("RLF_GPU_INDEX", "0")],
                                         capture_output=True, text=True, timeout=5).stdout.strip()
                    if out:
                        self.samples.append([x.strip() for x in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def workload(args):
    w = dict(synth.WORKLOADS[args.workload])
    if args.galaxies:
        w["n_gal"] = args.galaxies
    obs = synth.make_observation(**w)
    cat = synth.make_catalogue(w["n_gal"], w["fmin"], w["fmax"], g=w["g"])
    return w, obs, cat


def window_size(args, n_gal):
    w = min(max(1, args.window), n_gal)
    return w + (w % 2) if w < n_gal else w  # keep the opposite-orientation pairs together


def windows(n_gal, w, count):
    """(start, stop, restore_before) of `count` consecutive windows, wrapping at the end."""
    per = -(-n_gal // w)
    out = []
    for k in range(count):
        j = k % per
        out.append((j * w, min(n_gal, (j + 1) * w), k > 0 and j == 0))
    return out


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def snr_of(obs, cat):
    """Signal-to-noise of each galaxy's round model, sqrt(sum over visibilities of |V|^2) / sigma
    (the sum data_simulation.c:79-98 accumulates), from a radial histogram of the uv coverage: used
    only for the shear estimator's SNR >= 10 selection (shear.py:58)."""
    q = obs.uu * obs.uu + obs.vv * obs.vv
    hist, edges = np.histogram(q, bins=1024)
    qc = 0.5 * (edges[1:] + edges[:-1])
    sc = cat.scale * K.ARCS2RAD
    tot = np.zeros(cat.n)
    for c in range(obs.n_ch):
        x = (sc * sc)[:, None] * (obs.wavenumbers[c] ** 2 * qc)[None, :]
        tot += (cat.flux * obs.spec[c]) ** 2 * ((1.0 + x) ** -3.0 @ hist)
    return np.sqrt(tot) / obs.sigma


def shear_block(cat, res, snr, label):
    """Recovered shear (the estimator of shear.py:32-145, radiolensfit2_gb300.shear) against the
    input shear of the field."""
    from radiolensfit2_gb300 import shear as SH
    err1 = np.sqrt(np.maximum(res["var_e1"], 0.0))
    err2 = np.sqrt(np.maximum(res["var_e2"], 0.0))
    est = SH.estimate_shear(res["e1"], res["e2"], err1, err2, res["oneDimvar"], snr)
    g1, g2 = cat.g
    return {"fit": label, "g_true": [g1, g2], "g": [est.g1, est.g2], "g_err": [est.g1_err, est.g2_err],
            "bias": [est.g1 - g1, est.g2 - g2], "galaxies_used": est.n_used,
            "within_1sigma": bool(abs(est.g1 - g1) <= est.g1_err and abs(est.g2 - g2) <= est.g2_err)
            if est.n_used else None}


def cpu_sample_size(args, obs):
    if args.cpu_sample_galaxies >= 0:
        return args.cpu_sample_galaxies
    # about 10-30 s of oracle work on 16 host cores (~1.3 s per galaxy per 1.5e8 visibilities)
    return max(1, min(16, int(3e9 // max(obs.n_vis, 1))))


def oracle_two_passes(O, orc, obs, sub, d, s, gal, sigma2, flag, ro, fmax):
    """data_processing (oracle) over `sub`: catalogue pass, then the re-fit pass of its bad galaxies;
    results [(e1, e2, error)] after both passes (bad ones written with e = 0)."""
    out = (O.OrcFitResult * sub.n)()
    bl = np.zeros(sub.n, np.uint32)
    bad = C.c_int(0)
    sumw = np.zeros(fmax * fmax)
    tail = (obs.len_lambda, obs.n_rows, obs.n_ch, O.dp(obs.spec), O.dp(obs.wavenumbers), len(ro), O.dp(ro),
            O.dp(sub.l), O.dp(sub.m), O.dp(sub.flux), O.dp(sub.scale), O.dp(sumw), O.cp(gal), O.cp(s), O.cp(d),
            O.fp(sigma2), O.bp(flag), O.dp(obs.uu), O.dp(obs.vv), O.dp(obs.ww), 0)
    orc.orc_data_processing(0, bl.ctypes.data_as(O.PU), sub.n, *tail, out, C.byref(bad))
    res = np.array([(r.e1, r.e2, r.error) for r in out])
    nb = bad.value
    if nb:
        out2 = (O.OrcFitResult * sub.n)()
        bad2 = C.c_int(0)
        orc.orc_data_processing(1, bl.ctypes.data_as(O.PU), nb, *tail, out2, C.byref(bad2))
        for k in range(nb):
            r = out2[k]
            res[int(bl[k])] = (0.0, 0.0, 1) if r.error else (r.e1, r.e2, 0)
        nb = bad2.value
    return res, nb


def run_reference(args):
    """Reference arm: the oracle restatement of the reference's data_processing (its arithmetic and
    order, OpenMP over scalelength nodes and channels as the reference) on the host cores, on a
    bounded sample of the workload: the first galaxies of the catalogue, both passes, on data holding
    those galaxies' models plus noise.  Nothing runs on the GPU."""
    w, obs, cat = workload(args)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O
    orc = O.load_oracle()
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    n = cpu_sample_size(args, obs) if args.cpu_sample_galaxies < 0 else max(1, args.cpu_sample_galaxies)
    # each step stays a bounded sample (a few seconds of host work at the largest workload)
    n = max(1, min(n, int(1.5e9 // max(obs.n_vis, 1)) or 1))
    sub = cat.subset(range(n))
    sky = np.zeros(obs.n_vis, np.complex128)
    gal = np.zeros(obs.n_vis, np.complex128)
    orc.orc_sky_model(O.dp(obs.wavenumbers), O.dp(obs.spec), obs.n_ch, sub.n, O.dp(sub.flux), O.dp(sub.scale),
                      O.dp(sub.l), O.dp(sub.m), obs.n_rows, O.dp(obs.uu), O.dp(obs.vv), O.dp(obs.ww), O.cp(gal),
                      O.cp(sky), 0)
    # noise: a seeded block of up to 2^24 complex samples tiled over the visibilities (a timing sample)
    rng = np.random.default_rng(synth.NOISE_SEED)
    blk = min(obs.n_vis, 1 << 24)
    noise = obs.sigma * (rng.standard_normal(blk) + 1j * rng.standard_normal(blk))
    data = sky.copy()
    for i0 in range(0, obs.n_vis, blk):
        i1 = min(obs.n_vis, i0 + blk)
        data[i0:i1] += noise[:i1 - i0]
    del noise
    sigma2 = np.full(obs.n_vis, np.float32(obs.sigma2), np.float32)
    flag = np.zeros(obs.n_vis, np.uint8)
    ro = np.array(K.ro_grid())
    fmax = K.facet_size(K.RMAX, obs.len_lambda)
    d = np.empty_like(data)
    s = np.empty_like(sky)
    times = []
    steps = max(1, args.steps)
    warm = max(0, min(args.warmup, 1))
    for it in range(warm + steps):
        np.copyto(d, data)
        np.copyto(s, sky)
        t0 = time.perf_counter()
        oracle_two_passes(O, orc, obs, sub, d, s, gal, sigma2, flag, ro, fmax)
        dt = time.perf_counter() - t0
        if it >= warm:
            times.append(dt)
    t = float(np.mean(times))
    value = sub.n / t
    sample = (f"first {sub.n} galaxies of {w['n_gal']} (flux {sub.flux.min():.0f}-{sub.flux.max():.0f} uJy) on the "
              f"full {obs.n_vis}-visibility arrays holding those galaxies plus noise, both passes")
    line = {"metric": METRIC, "value": value, "unit": "galaxies/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": warm, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded array, catalogue and noise)",
            "config": {"workload": args.workload, "n_vis": obs.n_vis, "galaxies": w["n_gal"],
                       "sample_galaxies": sub.n},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "galaxies/s", "cores": int(os.environ["OMP_NUM_THREADS"]),
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "galaxies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def e2e_data_processing(lib, obs, cat, data_h, sky_h, B, win, steps, fit_prec, extra=None):
    """Galaxies/s through the reference-facing entry point data_processing() with pinned host
    complex128 buffers, one window per step: catalogue pass + re-fit pass of the window (two calls),
    copies inside the timing.  rlf_options.reuse_obs keeps uvw, variances, flags and the facet tables
    on the device between calls (the arrays are the same); visibilities and sky model cross the
    boundary on every call.  One warm-up window (it builds the observation), then `steps` windows.
    Bytes per step are the library's own copy counters."""
    import torch
    from radiolensfit2_gb300 import _lib
    from radiolensfit2_gb300.abi import LikelihoodParams, dptr, fptr, cptr, bptr
    opt = _lib.Options()
    opt.precision, opt.batch, opt.refit, opt.fit_precision = _lib.RLF_MIXED, B, 1, fit_prec
    opt.reuse_obs = 1  # the two passes and the windows pass the same uvw, variances and flags
    for k, v in (extra or {}).items():  # proposal and tuned launch shapes, as the device-resident run
        setattr(opt, k, int(v))
    lib.rlf_configure(C.byref(opt))
    n_vis = obs.n_vis
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    d, s = pin(data_h), pin(sky_h)
    sigma2 = pin(np.full(n_vis, np.float32(obs.sigma2), np.float32))
    flag = pin(np.zeros(n_vis, np.uint8))
    uu, vv, ww = pin(obs.uu), pin(obs.vv), pin(obs.ww)
    gal = np.zeros(1, np.complex128)
    ro = np.array(K.ro_grid())
    rprior = np.zeros(len(ro))
    p = LikelihoodParams()
    p.numr, p.ro, p.rprior, p.nchannels = len(ro), dptr(ro), dptr(rprior), obs.n_ch
    p.spec, p.wavenumbers = dptr(obs.spec), dptr(obs.wavenumbers)
    fmax = K.facet_size(K.RMAX, obs.len_lambda)
    sumw = np.zeros(fmax * fmax)
    times, h2d, d2h, ngal = [], [], [], []
    cold_ms = None
    c_in, c_out = C.c_ulonglong(0), C.c_ulonglong(0)
    lib.rlf_release()
    for it, (a, b, restore) in enumerate(windows(cat.n, win, 1 + steps)):
        if restore:
            np.copyto(d, data_h)
            np.copyto(s, sky_h)
        l, m, flux, scale, e1, e2 = (np.ascontiguousarray(x[a:b]) for x in
                                    (cat.l, cat.m, cat.flux, cat.scale, cat.e1, cat.e2))
        snr = np.zeros(b - a)
        bad_list = np.zeros(b - a, np.uint32)
        bad = C.c_int(0)
        ft = C.c_double(0)
        args = [C.byref(p), dptr(l), dptr(m), dptr(flux), dptr(scale), dptr(e1), dptr(e2), dptr(snr), dptr(sumw),
                cptr(gal), cptr(s), cptr(d), fptr(sigma2), bptr(flag), dptr(uu), dptr(vv), dptr(ww), C.byref(ft),
                C.byref(bad)]
        lib.rlf_transfer_bytes(C.byref(c_in), C.byref(c_out))
        b_in, b_out = c_in.value, c_out.value
        t0 = time.perf_counter()
        lib.data_processing(False, bad_list.ctypes.data_as(_lib.PU), b - a, obs.len_lambda, obs.n_rows, None, *args)
        nb = bad.value
        lib.data_processing(True, bad_list.ctypes.data_as(_lib.PU), nb, obs.len_lambda, obs.n_rows, None, *args)
        dt = time.perf_counter() - t0
        lib.rlf_transfer_bytes(C.byref(c_in), C.byref(c_out))
        if it == 0:
            cold_ms = dt * 1e3
        else:
            times.append(dt)
            ngal.append(b - a)
            h2d.append(c_in.value - b_in)
            d2h.append(c_out.value - b_out)
    lib.rlf_release()
    t = float(np.sum(times))
    return {"value": float(np.sum(ngal)) / t, "unit": "galaxies/s", "h2d_bytes_per_step": int(np.mean(h2d)),
            "d2h_bytes_per_step": int(np.mean(d2h)), "ms_per_step": t / len(times) * 1e3, "steps": len(times),
            "warmup": 1, "cold_ms": cold_ms,
            "path": ("data_processing() x2 per window (catalogue + re-fit pass), pinned host complex128 buffers, "
                     "mixed, batch %d, windows 2..%d of %d galaxies" % (B, steps + 1, win))}


def cpu_baseline(obs, cat, data_h, sky_h, n_sample, gpu_first):
    """The oracle (reference arithmetic, OpenMP over all host cores as the reference) on the first
    n_sample galaxies of the same data, both passes, run in place on data_h / sky_h; its fitted e
    against the GPU's for the same galaxies (the first galaxies' results do not depend on the rest
    of the catalogue)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O
    orc = O.load_oracle()
    sub = cat.subset(range(n_sample))
    gal = np.zeros(obs.n_vis, np.complex128)
    sigma2 = np.full(obs.n_vis, np.float32(obs.sigma2), np.float32)
    flag = np.zeros(obs.n_vis, np.uint8)
    ro = np.array(K.ro_grid())
    fmax = K.facet_size(K.RMAX, obs.len_lambda)
    t0 = time.perf_counter()
    res, nb = oracle_two_passes(O, orc, obs, sub, data_h, sky_h, gal, sigma2, flag, ro, fmax)
    dt = time.perf_counter() - t0
    g = gpu_first[:n_sample]
    ok = (res[:, 2] == 0) & (g["error"] == 0)
    de = np.maximum(np.abs(res[ok, 0] - g["e1"][ok]), np.abs(res[ok, 1] - g["e2"][ok]))
    parity = {"galaxies": int(n_sample), "good_in_both": int(ok.sum()),
              "error_flags_equal": bool(np.array_equal(res[:, 2].astype(int), g["error"])),
              "error_flags_differ": int(np.sum(res[:, 2].astype(int) != g["error"])),
              "max_abs_de": float(de.max()) if de.size else None,
              "frac_le_1e-4": float(np.mean(de <= 1e-4)) if de.size else None,
              "gpu_path": "batched mixed-precision, both passes, same data"}
    return sub.n / dt, dt, parity


# DRAM bytes of one k_extract_seq launch per algorithmic byte, from the ncu capture of
# profiles/k_extract_seq_mid_128ant_64ch.md (the full-scale channel layout; the mean of its first
# round and two correction rounds): dram__bytes_read.sum + dram__bytes_write.sum = 1214.0 MB + 16.3 MB
# against 16 B per visibility (975,360 rows x 64 channels) + 32 B per row.  A launch reads data and
# sky model once per visibility and the row table, work items and run descriptors once per (row,
# 16-channel chunk), so its traffic grows with those units.
EXTRACT_DRAM_PER_ALG_BYTE = (1214.021e6 + 16.319915e6) / (975360 * 64 * 16 + 975360 * 32)
EXTRACT_TRAFFIC_SOURCE = ("ncu DRAM bytes of one k_extract_seq launch on mid_128ant_64ch "
                          "(profiles/k_extract_seq_mid_128ant_64ch.md) per algorithmic byte, times this "
                          "launch's algorithmic bytes")


def roofline_of(obs, st, steps, hbm_peak, peak_kind, fp32_peak):
    """Roofline of the dominant kernel, k_extract_seq (the sequential batch extraction).

    Algorithmic bytes per launch: data and sky model (2 x 8 B FP32 complex) per visibility and the
    32 B row-table entry per row.  Algorithmic FP32 work per galaxy-visibility pair (FMA = 2): 15
    FLOP in a first round (Horner step 8, round-model profile 5, spectral sum 2) and 33 FLOP in a
    correction round (phase recurrence 6, rotation 8, two profiles 10, model difference and residual
    update 9).  Time: the kernel's own launches, CUDA events on the launching stream
    (RLF_STAT_EXTRACT_SEQ_US), summed over the timed steps."""
    n_vis, n_rows = float(obs.n_vis), float(obs.n_rows)
    launches = st["extract_passes"]
    t = st["extract_seq_us"] * 1e-6
    per_launch = 16.0 * n_vis + 32.0 * n_rows
    first = st["extract_gal_first"]
    flops = n_vis * (15.0 * first + 33.0 * (st["extract_gal"] - first))
    achieved = per_launch * launches / t / 1e9 if t > 0 and launches else None
    r = {"kernel": "k_extract_seq", "bound": "hbm", "unit": "GB/s", "achieved": achieved, "peak": hbm_peak,
         "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
         "frac": achieved / hbm_peak if achieved else None,
         "traffic": EXTRACT_DRAM_PER_ALG_BYTE * per_launch, "traffic_algorithmic": per_launch,
         "traffic_source": EXTRACT_TRAFFIC_SOURCE, "launches": int(launches),
         "avg_launch_ms": t / launches * 1e3 if launches else None, "kernel_ms_per_step": t * 1e3 / steps}
    if t > 0:
        # the batched passes are FP32-pipe bound (profiles, phase recurrences), not HBM bound
        r["compute"] = {"bound": "fp32", "unit": "TFLOP/s", "achieved": flops / t / 1e12,
                        "peak": fp32_peak / 1e3, "peak_kind": "measured FP32 FMA probe kernel",
                        "frac": flops / t / 1e12 / (fp32_peak / 1e3)}
    return r


def run_sharded(args, rank, world, local):
    """N > 1: the reference's MPI decomposition (data_processing-mpi.c:65-216) across GPUs.  Rank r
    holds channels channel_shards(n_ch, N)[r] of the observation (the same facet extent len on every
    rank); per window every rank extracts un-averaged facet partials of the window's galaxies over its
    channels, the partials are all-reduced over NCCL, each rank fits the galaxies it owns
    (round-robin), the results are all-reduced, and every rank removes the good fits from its
    channels; then the window's re-fit pass.  Windows play the reference's rounds (all galaxies of a
    window extracted from the same data).  The total work is fixed as N grows (strong scaling);
    timing: wall clock between barriers after CUDA synchronisation, max over ranks."""
    import torch
    import torch.distributed as dist
    from radiolensfit2_gb300 import _lib, shard
    from radiolensfit2_gb300.pipeline import DeviceObservation
    w, obs, cat = workload(args)
    so, (lo, hi) = shard.shard_observation(obs, world, rank)
    dev = DeviceObservation(so, precision=_lib.RLF_MIXED)
    dev.simulate(cat, so.sigma, seed=synth.NOISE_SEED + rank)
    dev.sky_model(cat)
    win = window_size(args, cat.n)
    plan = windows(cat.n, win, args.warmup + args.steps)
    dev.snapshot()
    pipe = shard.ShardPipeline([dev], shard.TorchExchange(device=torch.device("cuda", local)), world=world, rank=rank,
                               fit_precision=_lib.RLF_F64 if args.fit_precision == "f64" else _lib.RLF_MIXED)

    def step(a, b, restore):
        if restore:
            dev.restore()
        return pipe.process(cat.subset(range(a, b)), round_size=b - a, refit=True)

    for (a, b, restore) in plan[:args.warmup]:
        step(a, b, restore)
    torch.cuda.synchronize()
    dist.barrier()
    lib = _lib.load()
    l0 = lib.rlf_launch_count()
    t0 = time.perf_counter()
    n_timed = 0
    for (a, b, restore) in plan[args.warmup:]:
        step(a, b, restore)
        n_timed += b - a
    torch.cuda.synchronize()
    dist.barrier()
    t = torch.tensor([time.perf_counter() - t0], device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    elapsed = float(t.item())
    if rank == 0:
        print(json.dumps({"metric": METRIC, "value": n_timed / elapsed, "unit": "galaxies/s", "n_gpus": world,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
                          "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
                          "dtype": "fp32 visibilities (FP64 phase argument), %s fit" % args.fit_precision,
                          "data": "synthetic (seeded array, catalogue and noise)",
                          "config": {"workload": args.workload, "n_vis": obs.n_vis, "galaxies": cat.n, "window": win,
                                     "parallelism": "channel shards x%d (data_processing-mpi decomposition)" % world,
                                     "channels_rank0": [lo, hi]},
                          "gpu_launches": int(lib.rlf_launch_count() - l0)}), flush=True)
    dev.close()


def main():
    args = parse()
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) == 0:
            run_reference(args)
        return
    import torch
    from radiolensfit2_gb300 import _lib
    from radiolensfit2_gb300.pipeline import DeviceObservation, RESULT_DTYPE

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
        return run_sharded(args, rank, world, local)
    lib = _lib.load()
    t_setup = time.perf_counter()
    w, obs, cat = workload(args)
    dev = DeviceObservation(obs, precision=_lib.RLF_MIXED)
    dev.simulate(cat, obs.sigma, seed=synth.NOISE_SEED + rank)
    dev.sky_model(cat)
    dev.snapshot()
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    B = max(1, args.batch)
    fit_prec = _lib.RLF_F64 if args.fit_precision == "f64" else _lib.RLF_MIXED
    win = window_size(args, cat.n)
    plan = windows(cat.n, win, args.warmup + args.steps)
    # the learned proposal of the simplex starts (trained network shipped with the package)
    from radiolensfit2_gb300 import proposal as PR, autotune as AT
    use_prop = 0
    prop_desc = "none (the reference's simplex start (0, 0), step 0.1)"
    have_prop = args.proposal != "none" and os.path.exists(PR.WEIGHTS)
    if have_prop:
        PR.load()
    if args.proposal == "on" and have_prop:
        use_prop = 1
        prop_desc = "learned (radiolensfit2_gb300/proposal_weights.npz, rlf_options.proposal = 1)"
    # launch shapes tuned on the first window, from the snapshot (restored after every candidate)
    shapes, tune_ms = {}, None
    if args.tune == "auto" and B > 1:
        a0, b0, _ = plan[0]
        shapes, tune_ms = AT.tune(dev, cat.subset(range(a0, b0)), batch=B, fit_precision=fit_prec,
                                  rounds=args.rounds, proposal=use_prop)
    if args.graphs:
        shapes = dict(shapes, graphs=1)
    # the first walk over the catalogue: its results (shear) and device time (whole-job throughput)
    full = np.zeros(cat.n, RESULT_DTYPE)
    seen = np.zeros(cat.n, bool)
    walk = {"ms": 0.0}

    def step(a, b, restore):
        if restore:
            dev.restore()
        r = dev.process(cat.subset(range(a, b)), batch=B, refit=True, fit_precision=fit_prec, rounds=args.rounds,
                        proposal=use_prop, **shapes)
        if not seen[a:b].any():
            full[a:b] = r.results
            seen[a:b] = True
            walk["ms"] += r.ms[0]
        return r

    for (a, b, restore) in plan[:args.warmup]:
        step(a, b, restore)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler()
    clocks.start()
    l0 = lib.rlf_launch_count()
    t0 = time.perf_counter()
    stage = np.zeros(4)  # device time from CUDA events on the library's stream: total, extract, fit, remove
    stats = None
    n_timed = n_bad = 0
    for (a, b, restore) in plan[args.warmup:]:
        r = step(a, b, restore)
        stage += np.array(r.ms)
        n_timed += b - a
        n_bad += r.n_bad
        stats = dict(r.stats) if stats is None else {k: stats[k] + r.stats[k] for k in stats}
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    wall = time.perf_counter() - t0
    launches = int(lib.rlf_launch_count() - l0)
    ck = clocks.stop()
    elapsed = stage[0] * 1e-3  # seconds of device time over the K timed steps
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed = float(t.item())
    value = n_timed * world / elapsed
    stage_ms = {"extract": stage[1] / args.steps, "fit": stage[2] / args.steps, "remove": stage[3] / args.steps}
    peaks, peak_kind = measured_peaks()
    hbm_peak = float(peaks.get("hbm_gbs") or 6800.0)
    fp32_peak = float(lib.rlf_fp32_peak_gflops())  # measured here by an FMA probe kernel, GFLOP/s
    out = {"metric": METRIC, "value": value, "unit": "galaxies/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": "fp32 visibilities (FP64 phase argument), %s fit" % args.fit_precision,
           "data": "synthetic (seeded array, catalogue and noise)",
           "config": {"workload": args.workload, "antennas": w["n_ant"], "rows": obs.n_rows, "channels": obs.n_ch,
                      "n_vis": obs.n_vis, "galaxies": cat.n, "window": win, "timed_galaxies": n_timed,
                      "batch": B, "precision": "mixed", "fit_precision": args.fit_precision,
                      "proposal": prop_desc, "tuned_shapes": shapes or "defaults",
                      "l2_policy": "inputs larger than L2 (data + sky model %.1f GB)" % (16 * obs.n_vis / 1e9),
                      "timing": "CUDA events on the library stream around both passes of each window"},
           "setup_s": setup_s, "wall_ms_per_step": wall / args.steps * 1e3, "stage_ms_per_step": stage_ms,
           "bad_galaxies_timed": int(n_bad), "gpu_launches": launches, "work": stats, "autotune_ms": tune_ms,
           "roofline": roofline_of(obs, stats, args.steps, hbm_peak, peak_kind, fp32_peak),
           "clocks": ck, "peaks": peak_kind}
    snr = None
    if seen.all():
        out["catalogue_walk"] = {"galaxies": cat.n, "device_s": walk["ms"] * 1e-3,
                                 "galaxies_per_s": cat.n / (walk["ms"] * 1e-3),
                                 "note": "the W+K windows covered the catalogue: whole-job throughput"}
        if rank == 0:
            snr = snr_of(obs, cat)
            out["shear"] = [shear_block(cat, full, snr, "batched, whole catalogue")]
    gpu_first = None
    if rank == 0 and args.plain_prefix > 0:
        P = min(args.plain_prefix, cat.n)
        pre = cat.subset(range(P))
        # the same prefix from the same data: batched with the learned start, batched with the
        # reference's simplex start, and the plain one-galaxy-at-a-time fit
        rl = None
        if have_prop:
            dev.restore()
            rl = dev.process(pre, batch=B, refit=True, fit_precision=fit_prec, rounds=args.rounds, proposal=1,
                             **shapes)
        dev.restore()
        rn = dev.process(pre, batch=B, refit=True, fit_precision=fit_prec, rounds=args.rounds, **shapes)
        dev.restore()
        rp = dev.process(pre, batch=1, refit=True, fit_precision=fit_prec)
        rb = rl if use_prop else rn  # the measured path
        bt, bn, pl = rb.results, rn.results, rp.results
        gpu_first = bt

        def dev_of(a, b):
            ok = (a["error"] == 0) & (b["error"] == 0)
            de = np.maximum(np.abs(a["e1"][ok] - b["e1"][ok]), np.abs(a["e2"][ok] - b["e2"][ok]))
            return {"max": float(de.max()) if de.size else None, "median": float(np.median(de)) if de.size else None,
                    "frac_le_1e-3": float(np.mean(de <= 1e-3)) if de.size else None,
                    "frac_le_1e-4": float(np.mean(de <= 1e-4)) if de.size else None, "n": int(de.size),
                    "error_flags_differ": int(np.sum(a["error"] != b["error"]))}

        plain_rate = P / (rp.ms[0] * 1e-3)
        out["plain_gpu"] = {"value": plain_rate, "unit": "galaxies/s", "prefix_galaxies": P, "ms": rp.ms[0],
                            "stage_ms": dict(zip(("extract", "fit", "remove"), rp.ms[1:])),
                            "evals_per_galaxy": float(np.mean(pl["nevals"])),
                            "measured_path_on_prefix": {"value": P / (rb.ms[0] * 1e-3), "ms": rb.ms[0],
                                                        "evals_per_galaxy": float(np.mean(bt["nevals"]))},
                            "speedup_measured_path_vs_plain_same_prefix": rp.ms[0] / rb.ms[0],
                            "speedup_value_vs_plain": value / plain_rate,
                            "abs_de_measured_vs_plain": dev_of(bt, pl)}
        if rl is not None:
            lr = rl.results
            out["learned_proposal"] = {
                "prefix_galaxies": P, "gate_max_sigma": 0.05,
                "evals_per_galaxy": {"reference_start": float(np.mean(bn["nevals"])),
                                     "learned_start": float(np.mean(lr["nevals"]))},
                "ms": {"reference_start": rn.ms[0], "learned_start": rl.ms[0]},
                "fit_ms": {"reference_start": rn.ms[2], "learned_start": rl.ms[2]},
                "abs_de_learned_vs_reference_start": dev_of(lr, bn), "abs_de_learned_vs_plain": dev_of(lr, pl),
                "in_measured_path": bool(use_prop)}
        if snr is not None:
            out["shear"].append(shear_block(pre, bt, snr[:P], "measured path, prefix"))
            out["shear"].append(shear_block(pre, pl, snr[:P], "plain, prefix"))
    n_cpu = cpu_sample_size(args, obs) if gpu_first is not None else 0
    data_h = sky_h = None
    if rank == 0 and (not args.no_e2e or n_cpu > 0):
        dev.restore()
        data_h, sky_h = dev.get_vis()
    dev.close()
    if rank == 0 and not args.no_e2e:
        out["e2e"] = e2e_data_processing(lib, obs, cat, data_h, sky_h, B, win, max(1, min(args.steps, args.e2e_steps)),
                                         fit_prec, dict(shapes, proposal=use_prop))
    if rank == 0 and n_cpu > 0:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
        n_cpu = min(n_cpu, len(gpu_first))
        v, dt, parity = cpu_baseline(obs, cat, data_h, sky_h, n_cpu, gpu_first)
        out["cpu_baseline"] = {"value": v, "unit": "galaxies/s", "cores": int(os.environ["OMP_NUM_THREADS"]),
                               "kind": "port",
                               "sample": f"first {n_cpu} galaxies of {cat.n} (the brightest), full "
                                         f"{obs.n_vis}-visibility arrays, extraction+fit+removal, both passes "
                                         f"({dt:.1f} s)"}
        out["parity"] = {"vs_cpu_oracle": parity}
    if rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
