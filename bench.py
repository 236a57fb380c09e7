"""Benchmark: galaxies/s of the shape-measurement hot path on one GB300.

A step is one full pass of the path over the synthetic observation: extraction, fit and
removal of every galaxy in catalogue order, then the re-fit pass over the bad ones
(RadioLensfit2.cpp:597-606), starting from the same data and sky model each step.

  value : device-resident run (rlf_obs_process) of the batched mixed-precision path
  e2e   : the same work through the reference-facing C entry point data_processing() with host
          buffers (two calls: catalogue pass and re-fit pass), H2D/D2H copies inside the timing
  plain : the one-launch-chain-per-galaxy mixed-precision path (batch 1), per-galaxy |de| of the
          batched result against it
  --impl reference : the CPU oracle (restatement of the reference, OpenMP on all host cores) on a
          bounded sample of the same workload

Workload (default): 197 antennas (19,306 baselines) x 480 times x 16 channels = 148M
visibilities, 1,000 galaxies at 10-200 uJy, seeded synthetic data (no public dataset exists).
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

METRIC = "galaxies/s on 1 GB300 (extract+fit+remove, both passes)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c1_ska_mid_16ch")
    ap.add_argument("--galaxies", type=int, default=0)
    ap.add_argument("--batch", type=int, default=1000)
    ap.add_argument("--rounds", type=int, default=0,
                    help="extraction + fit rounds per batch (0 = library default)")
    ap.add_argument("--fit-precision", default="f64", choices=["f64", "mixed"],
                    help="arithmetic of the fit (visibility passes are always mixed)")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-sample-galaxies", type=int, default=2)
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


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def run_reference(args):
    """CPU baseline: the oracle restatement (reference arithmetic, OpenMP over scalelength nodes and
    channels as the reference) on a bounded sample of the workload."""
    w, obs, cat = workload(args)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O
    orc = O.load_oracle()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    n = max(1, args.cpu_sample_galaxies)
    # data for the sample: the sample galaxies' models + noise; sky model of the sample
    sub = cat.subset(range(n))
    rng = np.random.default_rng(synth.NOISE_SEED)
    data = np.zeros(obs.n_vis, np.complex128)
    sky = np.zeros(obs.n_vis, np.complex128)
    gal = np.zeros(obs.n_vis, np.complex128)
    orc.orc_sky_model(O.dp(obs.wavenumbers), O.dp(obs.spec), obs.n_ch, sub.n, O.dp(sub.flux), O.dp(sub.scale),
                      O.dp(sub.l), O.dp(sub.m), obs.n_rows, O.dp(obs.uu), O.dp(obs.vv), O.dp(obs.ww), O.cp(gal),
                      O.cp(sky), 0)
    data[:] = sky
    data += obs.sigma * (rng.standard_normal(obs.n_vis) + 1j * rng.standard_normal(obs.n_vis))
    sigma2 = np.full(obs.n_vis, np.float32(obs.sigma2), np.float32)
    flag = np.zeros(obs.n_vis, np.uint8)
    ro = np.array(K.ro_grid())
    fmax = K.facet_size(K.RMAX, obs.len_lambda)
    times = []
    steps = max(1, args.steps)
    for it in range(max(0, min(args.warmup, 1)) + steps):
        d, s = data.copy(), sky.copy()
        out = (O.OrcFitResult * sub.n)()
        bl = np.zeros(sub.n, np.uint32)
        bad = C.c_int(0)
        sumw = np.zeros(fmax * fmax)
        t0 = time.perf_counter()
        orc.orc_data_processing(0, bl.ctypes.data_as(O.PU), sub.n, obs.len_lambda, obs.n_rows, obs.n_ch,
                                O.dp(obs.spec), O.dp(obs.wavenumbers), len(ro), O.dp(ro), O.dp(sub.l), O.dp(sub.m),
                                O.dp(sub.flux), O.dp(sub.scale), O.dp(sumw), O.cp(gal), O.cp(s), O.cp(d),
                                O.fp(sigma2), O.bp(flag), O.dp(obs.uu), O.dp(obs.vv), O.dp(obs.ww), 0, out,
                                C.byref(bad))
        dt = time.perf_counter() - t0
        if it >= min(args.warmup, 1):
            times.append(dt)
    t = float(np.mean(times))
    value = sub.n / t
    line = {"metric": METRIC, "value": value, "unit": "galaxies/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": min(args.warmup, 1), "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "n_vis": obs.n_vis, "galaxies": w["n_gal"],
                       "sample_galaxies": sub.n},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "galaxies/s", "cores": int(os.environ["OMP_NUM_THREADS"]),
                             "kind": "port", "sample": f"{sub.n} galaxies of {w['n_gal']} on the full "
                                                       f"{obs.n_vis}-visibility array, first pass"},
            "e2e": {"value": value, "unit": "galaxies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def e2e_data_processing(lib, obs, cat, data_h, sky_h, B, steps, warmup, fit_prec):
    """Galaxies/s through the reference-facing entry point data_processing() with pinned host
    buffers: catalogue pass + re-fit pass (RadioLensfit2.cpp:597-606), copies inside the timing.
    The library keeps the observation (uvw, variances, flags, facet tables) between calls that
    pass the same arrays, as the reference driver's do; visibilities and sky model cross the
    boundary on every call.  Bytes per step are the library's own copy counters; cold_ms is the
    first call pair, which builds the observation."""
    import torch
    from radiolensfit2_gb300 import _lib
    from radiolensfit2_gb300.abi import LikelihoodParams, dptr, fptr, cptr, bptr
    opt = _lib.Options()
    opt.precision, opt.batch, opt.refit, opt.fit_precision = _lib.RLF_MIXED, B, 1, fit_prec
    opt.reuse_obs = 1  # the two passes pass the same uvw, variances and flags
    lib.rlf_configure(C.byref(opt))
    n_vis = obs.n_vis
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    d0, s0 = pin(data_h), pin(sky_h)
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
    snr = np.zeros(cat.n)
    flux, scale, l, m, e1, e2 = (np.ascontiguousarray(x) for x in (cat.flux, cat.scale, cat.l, cat.m, cat.e1, cat.e2))
    times, h2d, d2h = [], [], []
    cold_ms = None
    nbad_final = 0
    c_in, c_out = C.c_ulonglong(0), C.c_ulonglong(0)
    lib.rlf_release()
    for it in range(warmup + steps):
        np.copyto(d, d0)
        np.copyto(s, s0)
        bad_list = np.zeros(cat.n, np.uint32)
        bad = C.c_int(0)
        ft = C.c_double(0)
        args = [C.byref(p), dptr(l), dptr(m), dptr(flux), dptr(scale), dptr(e1), dptr(e2), dptr(snr), dptr(sumw),
                cptr(gal), cptr(s), cptr(d), fptr(sigma2), bptr(flag), dptr(uu), dptr(vv), dptr(ww), C.byref(ft),
                C.byref(bad)]
        lib.rlf_transfer_bytes(C.byref(c_in), C.byref(c_out))
        b_in, b_out = c_in.value, c_out.value
        t0 = time.perf_counter()
        lib.data_processing(False, bad_list.ctypes.data_as(_lib.PU), cat.n, obs.len_lambda, obs.n_rows, None, *args)
        nb = bad.value
        lib.data_processing(True, bad_list.ctypes.data_as(_lib.PU), nb, obs.len_lambda, obs.n_rows, None, *args)
        dt = time.perf_counter() - t0
        lib.rlf_transfer_bytes(C.byref(c_in), C.byref(c_out))
        nbad_final = bad.value
        if it == 0:
            cold_ms = dt * 1e3
        if it >= warmup:
            times.append(dt)
            h2d.append(c_in.value - b_in)
            d2h.append(c_out.value - b_out)
    lib.rlf_release()
    t = float(np.mean(times))
    return {"value": cat.n / t, "unit": "galaxies/s", "h2d_bytes_per_step": int(np.mean(h2d)),
            "d2h_bytes_per_step": int(np.mean(d2h)), "ms_per_step": t * 1e3, "cold_ms": cold_ms,
            "path": "data_processing() x2 (catalogue + re-fit pass), host complex128 buffers, mixed, batch %d" % B,
            "bad_after_refit": nbad_final}


def cpu_baseline(obs, cat, data_h, sky_h, n_sample):
    """The oracle (reference arithmetic, OpenMP over all host cores as the reference) on the
    first n_sample galaxies of the workload: extraction + fit + removal, first pass."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O
    orc = O.load_oracle()
    sub = cat.subset(range(n_sample))
    d, s = data_h.copy(), sky_h.copy()
    gal = np.zeros(obs.n_vis, np.complex128)
    sigma2 = np.full(obs.n_vis, np.float32(obs.sigma2), np.float32)
    flag = np.zeros(obs.n_vis, np.uint8)
    ro = np.array(K.ro_grid())
    fmax = K.facet_size(K.RMAX, obs.len_lambda)
    out = (O.OrcFitResult * sub.n)()
    bl = np.zeros(sub.n, np.uint32)
    bad = C.c_int(0)
    t0 = time.perf_counter()
    orc.orc_data_processing(0, bl.ctypes.data_as(O.PU), sub.n, obs.len_lambda, obs.n_rows, obs.n_ch, O.dp(obs.spec),
                            O.dp(obs.wavenumbers), len(ro), O.dp(ro), O.dp(sub.l), O.dp(sub.m), O.dp(sub.flux),
                            O.dp(sub.scale), O.dp(np.zeros(fmax * fmax)), O.cp(gal), O.cp(s), O.cp(d), O.fp(sigma2),
                            O.bp(flag), O.dp(obs.uu), O.dp(obs.vv), O.dp(obs.ww), 0, out, C.byref(bad))
    dt = time.perf_counter() - t0
    res = np.array([(r.e1, r.e2, r.error) for r in out])
    return sub.n / dt, dt, res


# DRAM bytes of one k_extract_seq launch per row of the observation, from the ncu capture of
# profiles/k_extract_seq_mid_128ant_16ch.md (dram__bytes_read.sum + dram__bytes_write.sum =
# 335.9 MB + 7.7 MB over 975,360 rows); a launch reads data, sky model, the row table, the
# work-item list and the run descriptors once per row, so the traffic of a launch grows with the
# rows
EXTRACT_DRAM_BYTES_PER_ROW = (335.856384e6 + 7.741184e6) / 975360


def roofline_of(obs, cat, batched, res, B, stage_ms, hbm_peak, peak_kind, fp32_peak):
    """Roofline of the dominant stage of a step.

    Algorithmic bytes of the streaming passes: a sequential batch extraction pass reads data and
    sky model (2 x 8 B FP32 complex) per visibility and the 32 B row table entry per row; a removal
    pass reads and writes data and sky model (32 B) per visibility and reads the row table.
    Algorithmic FP32 work per galaxy-visibility pair (FMA = 2): extraction 15 FLOP in a first round
    (Horner step 8, round-model profile 5, spectral sum 2) and 33 FLOP in a correction round (phase
    recurrence 6, rotation 8, two profiles 10, model difference and residual update 9); removal
    40 FLOP.  The fit reads only facets (kilobytes) and has no streaming roofline."""
    n_vis, n_rows = float(obs.n_vis), float(obs.n_rows)
    good = int(np.sum(batched["error"] == 0))
    st = res.stats  # passes of the last step (both passes), counted by the library
    dominant = max(stage_ms, key=stage_ms.get)
    t = stage_ms[dominant] * 1e-3
    if dominant == "extract":
        nbytes = (st["extract_passes"] + st["extract_single"]) * (16.0 * n_vis + 32.0 * n_rows)
        first = st["extract_gal_first"]
        flops = n_vis * (15.0 * first + 33.0 * (st["extract_gal"] - first))
    elif dominant == "remove":
        nbytes = (st["remove_batches"] + st["remove_single"]) * (32.0 * n_vis + 32.0 * n_rows)
        flops = 40.0 * n_vis * good
    else:
        nbytes, flops = None, None
    kernel = {"remove": "k_remove_batch", "extract": "k_extract_seq", "fit": "k_fit"}[dominant]
    r = {"kernel": kernel, "bound": "hbm", "unit": "GB/s",
         "achieved": nbytes / t / 1e9 if nbytes else None, "peak": hbm_peak,
         "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
         "traffic": None, "time_ms_per_step": stage_ms[dominant], "passes": st}
    r["frac"] = r["achieved"] / hbm_peak if r["achieved"] else None
    if dominant == "extract":
        # per launch, from the mid-size capture scaled by rows (this workload is too large for a
        # multi-pass capture); algorithmic bytes per launch beside it
        r["traffic"] = EXTRACT_DRAM_BYTES_PER_ROW * n_rows
        r["traffic_algorithmic"] = 16.0 * n_vis + 32.0 * n_rows
        r["traffic_source"] = ("ncu DRAM bytes of one k_extract_seq launch on mid_128ant_16ch "
                               "(profiles/k_extract_seq_mid_128ant_16ch.md), scaled by rows")
    if flops:
        # the batched passes are FP32-pipe bound (profiles, phase recurrences), not HBM bound
        r["compute"] = {"bound": "fp32", "unit": "TFLOP/s", "achieved": flops / t / 1e12,
                        "peak": fp32_peak / 1e3, "peak_kind": "measured FP32 FMA probe kernel",
                        "frac": flops / t / 1e12 / (fp32_peak / 1e3)}
    return r

def main():
    args = parse()
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        if rank == 0:
            run_reference(args)
        return
    import torch
    from radiolensfit2_gb300 import _lib
    from radiolensfit2_gb300.pipeline import DeviceObservation

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    lib = _lib.load()
    w, obs, cat = workload(args)
    dev = DeviceObservation(obs, precision=_lib.RLF_MIXED)
    dev.simulate(cat, obs.sigma, seed=synth.NOISE_SEED + rank)
    dev.sky_model(cat)
    dev.snapshot()
    B = max(1, args.batch)
    fit_prec = _lib.RLF_F64 if args.fit_precision == "f64" else _lib.RLF_MIXED

    def step():
        dev.restore()
        return dev.process(cat, batch=B, refit=True, fit_precision=fit_prec, rounds=args.rounds)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler()
    clocks.start()
    l0 = lib.rlf_launch_count()
    t0 = time.perf_counter()
    stage = np.zeros(4)  # device time from CUDA events on the library's stream: total, extract, fit, remove
    res = None
    for _ in range(args.steps):
        res = step()
        stage += np.array(res.ms)
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
    value = cat.n * args.steps * world / elapsed
    batched = res.results
    stage_ms = {"extract": stage[1] / args.steps, "fit": stage[2] / args.steps, "remove": stage[3] / args.steps}
    peaks, peak_kind = measured_peaks()
    hbm_peak = float(peaks.get("hbm_gbs") or 6800.0)
    fp32_peak = float(lib.rlf_fp32_peak_gflops())  # measured here by an FMA probe kernel, GFLOP/s
    roofline = roofline_of(obs, cat, batched, res, B, stage_ms, hbm_peak, peak_kind, fp32_peak)
    out = {"metric": METRIC, "value": value, "unit": "galaxies/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp32 visibilities (FP64 phase argument), %s fit" % args.fit_precision,
           "data": "synthetic (seeded array, catalogue and noise)",
           "config": {"workload": args.workload, "antennas": w["n_ant"], "rows": obs.n_rows, "channels": obs.n_ch,
                      "n_vis": obs.n_vis, "galaxies": cat.n, "batch": B, "precision": "mixed",
                      "fit_precision": args.fit_precision,
                      "l2_policy": "inputs larger than L2 (data + sky model %.1f GB)" % (16 * obs.n_vis / 1e9),
                      "timing": "CUDA events on the library stream around both passes of each step"},
           "wall_ms_per_step": wall / args.steps * 1e3,
           "stage_ms_per_step": stage_ms, "bad_galaxies": int(res.n_bad), "gpu_launches": launches,
           "roofline": roofline, "clocks": ck, "peaks": peak_kind}
    if rank == 0 and not args.no_plain:
        dev.restore()
        t1 = time.perf_counter()
        pr = dev.process(cat, batch=1, refit=True, fit_precision=fit_prec)
        tp = time.perf_counter() - t1
        pl = pr.results
        ok = (pl["error"] == 0) & (batched["error"] == 0)
        de = np.maximum(np.abs(pl["e1"][ok] - batched["e1"][ok]), np.abs(pl["e2"][ok] - batched["e2"][ok]))
        out["plain_gpu"] = {"value": cat.n / tp, "unit": "galaxies/s", "ms": tp * 1e3,
                            "stage_ms": dict(zip(("extract", "fit", "remove"), pr.ms[1:])),
                            "speedup_batched_vs_plain": value / (cat.n / tp),
                            "abs_de_vs_batched": {"max": float(de.max()) if de.size else None,
                                                  "median": float(np.median(de)) if de.size else None,
                                                  "frac_le_1e-3": float(np.mean(de <= 1e-3)) if de.size else None,
                                                  "n": int(de.size)}}
    data_h = sky_h = None
    if rank == 0 and (not args.no_e2e or args.cpu_sample_galaxies > 0):
        dev.restore()
        data_h, sky_h = dev.get_vis()
    if rank == 0 and not args.no_e2e:
        out["e2e"] = e2e_data_processing(lib, obs, cat, data_h, sky_h, B, steps=1, warmup=1, fit_prec=fit_prec)
    if rank == 0 and args.cpu_sample_galaxies > 0:
        v, dt, _ = cpu_baseline(obs, cat, data_h, sky_h, args.cpu_sample_galaxies)
        out["cpu_baseline"] = {"value": v, "unit": "galaxies/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": f"first {args.cpu_sample_galaxies} galaxies of {cat.n}, full "
                                         f"{obs.n_vis}-visibility arrays, extraction+fit+removal, first pass "
                                         f"({dt:.1f} s)"}
    if rank == 0:
        print(json.dumps(out), flush=True)
    dev.close()


if __name__ == "__main__":
    main()
