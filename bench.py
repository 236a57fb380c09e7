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


def cpu_baseline_sample(obs, cat, galaxies=1):
    """Time the oracle (OpenMP, all cores) on `galaxies` galaxies of the workload (first pass)."""
    ns = argparse.Namespace(workload=None, galaxies=0, steps=1, warmup=0, cpu_sample_galaxies=galaxies, gpus=1)
    return ns


def main():
    args = parse()
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        if rank == 0:
            run_reference(args)
        return
    import torch
    from radiolensfit2_gb300 import _lib
    from radiolensfit2_gb300.pipeline import DeviceObservation, RESULT_DTYPE
    from radiolensfit2_gb300.abi import LikelihoodParams, dptr, fptr, cptr, bptr

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

    def step():
        dev.restore()
        return dev.process(cat, batch=B, refit=True)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler()
    clocks.start()
    t0 = time.perf_counter()
    stage = np.zeros(4)
    res = None
    for _ in range(args.steps):
        res = step()
        stage += np.array(res.ms)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    elapsed = time.perf_counter() - t0
    ck = clocks.stop()
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed = float(t.item())
    value = cat.n * args.steps * world / elapsed
    out = {"metric": METRIC, "value": value, "unit": "galaxies/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (FP64 phase argument)",
           "data": "synthetic (seeded array, catalogue and noise)",
           "config": {"workload": args.workload, "antennas": w["n_ant"], "rows": obs.n_rows, "channels": obs.n_ch,
                      "n_vis": obs.n_vis, "galaxies": cat.n, "batch": B, "precision": "mixed",
                      "l2_policy": "inputs larger than L2 (data + sky model 2.4 GB)"},
           "stage_ms_per_step": {"extract": stage[1] / args.steps, "fit": stage[2] / args.steps,
                                 "remove": stage[3] / args.steps},
           "bad_galaxies": int(res.n_bad), "clocks": ck}
    batched = res.results
    if rank == 0:
        print(json.dumps(out), flush=True)
    dev.close()


if __name__ == "__main__":
    main()
