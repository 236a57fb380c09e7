"""Train the learned simplex-start proposal on the GPU and evaluate it on held-out galaxies.

  python -m radiolensfit2_gb300.train_proposal [--train 200000] [--heldout 10000] [--out FILE]

Training set: galaxies drawn from the small configuration's distributions (flux 10-200 uJy,
scalelength and ellipticity distributions of synth.make_catalogue, shear (0.03, -0.02)) through the
project's visibility simulator on the 32-channel SKA-MID-like array (197 antennas, 480 times),
10,000 per simulated observation, their facets extracted by the batched extraction.  A tenth is
kept for validation.  Held-out evaluation: another catalogue (other seeds) on the same array,
processed by the batched pipeline with and without the proposal: likelihood evaluations per
galaxy and per-galaxy |de| between the two.  Writes the parameters (--out, default the package's
proposal_weights.npz) and a JSON report next to them.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import proposal as PR, synth
from .pipeline import DeviceObservation


def evaluate(obs, n_gal, seed=11, batch=1000, fmin=10.0, fmax=200.0, g=(0.03, -0.02), gates=(0.02, 0.03, 0.05)):
    """Held-out galaxies through the batched pipeline with the reference's start and with the
    proposal at each gate (galaxies whose predicted sigma exceeds the gate keep the reference's
    start)."""
    from . import _lib
    cat = synth.make_catalogue(n_gal, fmin, fmax, g=g, seed=seed)
    dev = DeviceObservation(obs)
    dev.simulate(cat, obs.sigma, seed=seed)
    dev.sky_model(cat)
    dev.snapshot()
    dev.restore()
    t0 = time.time()
    base = dev.process(cat, batch=batch, refit=True, proposal=0)
    base_wall = time.time() - t0
    out = {}
    for gate in gates:
        _lib.load().rlf_proposal_set_max_sigma(float(gate))
        dev.restore()
        t0 = time.time()
        r = dev.process(cat, batch=batch, refit=True, proposal=1)
        out[f"gate_{gate}"] = compare(n_gal, (base, base_wall), (r, time.time() - t0))
    dev.close()
    return out


def compare(n_gal, base, learned):
    runs = {"plain_start": base, "learned_start": learned}
    a, b = runs["plain_start"][0].results, runs["learned_start"][0].results
    ok = (a["error"] == 0) & (b["error"] == 0)
    de = np.maximum(np.abs(a["e1"] - b["e1"]), np.abs(a["e2"] - b["e2"]))[ok]
    rep = {"galaxies": n_gal, "good_in_both": int(ok.sum()),
           "error_flags_differ": int(np.sum(a["error"] != b["error"])),
           "abs_de": {"max": float(de.max()) if de.size else None, "median": float(np.median(de)) if de.size else None,
                      "frac_le_1e-3": float(np.mean(de <= 1e-3)) if de.size else None,
                      "frac_le_1e-4": float(np.mean(de <= 1e-4)) if de.size else None}}
    for name, (r, wall) in runs.items():
        res = r.results
        rep[name] = {"evals_per_galaxy": float(np.mean(res["nevals"])),
                     "evals_per_good_galaxy": float(np.mean(res["nevals"][res["error"] == 0])),
                     "simplex_iters_per_galaxy": float(np.mean(res["iters"])),
                     "fit_ms": r.ms[2], "total_ms": r.ms[0], "wall_s": wall, "bad": int(r.n_bad)}
    rep["eval_reduction"] = 1.0 - rep["learned_start"]["evals_per_galaxy"] / rep["plain_start"]["evals_per_galaxy"]
    # the galaxies the proposal started (predicted sigma <= 0.05): evaluations and |de| there
    a_it, b_it = a["nevals"], b["nevals"]
    moved = (a["iters"] != b["iters"]) | (a_it != b_it)
    rep["galaxies_with_changed_path"] = int(moved.sum())
    if moved.any():
        rep["changed_path"] = {"evals_reference_start": float(np.mean(a_it[moved])),
                               "evals_learned_start": float(np.mean(b_it[moved]))}
    return rep


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=200000)
    ap.add_argument("--heldout", type=int, default=10000)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--workload", default="c2_ska_mid_32ch")
    ap.add_argument("--out", default=PR.WEIGHTS)
    ap.add_argument("--eval-only", action="store_true", help="evaluate the parameters in --out on held-out galaxies")
    a = ap.parse_args()
    if a.eval_only:
        PR.load(a.out)
        obs = synth.make_observation(**synth.WORKLOADS[a.workload])
        print(json.dumps({"heldout": evaluate(obs, a.heldout)}), flush=True)
        return
    n_val = max(256, a.train // 10)
    n_all = a.train + n_val
    t0 = time.time()
    net = PR.ProposalNet(max_batch=256, capacity=n_all)
    obs, cats = PR.training_set(net, n_all, workload=a.workload, seed=10)
    t_data = time.time() - t0
    t1 = time.time()
    params, hist = PR.train(net, a.train, n_val, epochs=a.epochs)
    t_train = time.time() - t1
    # accuracy of the proposal on the validation images
    net.set_params(params)
    out = net.predict(a.train, n_val)
    cat_all = np.concatenate([np.stack([c.e1, c.e2, c.flux], 1) for c in cats])[a.train:a.train + n_val]
    de = np.hypot(out[:, 0] - cat_all[:, 0], out[:, 1] - cat_all[:, 1])
    bright = cat_all[:, 2] > 50
    net.close()
    PR.save(params, a.out)
    PR.load(a.out)
    rep = {"train_galaxies": a.train, "val_galaxies": n_val, "workload": a.workload, "epochs": a.epochs,
           "data_s": t_data, "train_s": t_train, "history": hist,
           "val_abs_e_error": {"median": float(np.median(de)), "median_flux_gt_50uJy": float(np.median(de[bright])),
                               "median_predicted_sigma": float(np.median(np.exp(out[:, 3])))},
           "heldout": evaluate(obs, a.heldout) if a.heldout > 0 else None}
    with open(os.path.splitext(a.out)[0] + "_report.json", "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps(rep), flush=True)


if __name__ == "__main__":
    main()
