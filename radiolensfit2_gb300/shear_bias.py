"""Multiplicative and additive shear bias of the fit over fields of different input shear.

  python -m radiolensfit2_gb300.shear_bias [--workload c1_ska_mid_16ch] [--galaxies 1000]
                                           [--noise-scale 1] [--snr-cuts 10,20,40]

For each input shear g of a set of fields (same array and catalogue distributions, a different
catalogue and noise seed per field), the observation is simulated on the GPU and processed both by
the batched mixed-precision path and by the plain one-galaxy-at-a-time path (both passes); the
shear of each field is estimated with the reference's estimator (shear.py:32-145,
radiolensfit2_gb300.shear), and g_measured = (1 + m) g_true + c is fitted per component
(shear.multiplicative_additive_bias).  The same fit is repeated for stricter SNR cuts than the
reference's 10, and per SNR band the fitted ellipticities are regressed on the true (sheared) ones
(slope and offset of e_fit = s e_true + o, the per-galaxy response behind m and c).  --noise-scale
multiplies the simulated noise (0: noise-free data, the likelihood still weighted by the
observation's sigma).  Prints one JSON object.
"""
from __future__ import annotations

import argparse
import json
import math

import numpy as np

from . import _lib, shear, synth

FIELDS = ((0.03, -0.02), (-0.03, 0.02), (0.02, 0.03), (-0.02, -0.03))


def snr_of(obs, cat):
    """sqrt(sum over visibilities of |V|^2) / sigma of each galaxy's round model (the sum
    data_simulation.c:79-98 accumulates), from a radial histogram of the uv coverage: used only for
    the estimator's SNR >= 10 selection (shear.py:58)."""
    q = obs.uu * obs.uu + obs.vv * obs.vv
    hist, edges = np.histogram(q, bins=1024)
    qc = 0.5 * (edges[1:] + edges[:-1])
    sc = cat.scale * math.pi / 648000.0
    tot = np.zeros(cat.n)
    for c in range(obs.n_ch):
        x = (sc * sc)[:, None] * (obs.wavenumbers[c] ** 2 * qc)[None, :]
        tot += (cat.flux * obs.spec[c]) ** 2 * ((1.0 + x) ** -3.0 @ hist)
    return np.sqrt(tot) / obs.sigma


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="c1_ska_mid_16ch")
    ap.add_argument("--galaxies", type=int, default=0)
    ap.add_argument("--batch", type=int, default=1000)
    ap.add_argument("--noise-scale", type=float, default=1.0)
    ap.add_argument("--snr-cuts", default="10,20,40")
    a = ap.parse_args()
    cuts = [float(x) for x in a.snr_cuts.split(",")]
    from .pipeline import DeviceObservation
    w = dict(synth.WORKLOADS[a.workload])
    n = a.galaxies or w["n_gal"]
    obs = synth.make_observation(**w)
    rows = {(cut, name): [] for cut in cuts for name in ("batched", "plain")}
    per_galaxy = []
    fits = []  # (snr, e_true 1, e_true 2, e_fit 1, e_fit 2) of the batched path's good galaxies
    for k, g in enumerate(FIELDS):
        cat = synth.make_catalogue(n, w["fmin"], w["fmax"], g=g, seed=100 + k)
        dev = DeviceObservation(obs, precision=_lib.RLF_MIXED)
        dev.simulate(cat, obs.sigma * a.noise_scale, seed=200 + k)
        dev.sky_model(cat)
        dev.snapshot()
        res = {}
        for name, batch in (("batched", a.batch), ("plain", 1)):
            dev.restore()
            res[name] = dev.process(cat, batch=batch, refit=True).results
        dev.close()
        snr = snr_of(obs, cat)
        for cut in cuts:
            for name, r in res.items():
                est = shear.estimate_shear(r["e1"], r["e2"], np.sqrt(np.maximum(r["var_e1"], 0)),
                                           np.sqrt(np.maximum(r["var_e2"], 0)), r["oneDimvar"], snr, snr_min=cut)
                rows[(cut, name)].append((g[0], g[1], est.g1, est.g2, est.g1_err, est.g2_err, est.n_used))
        rb = res["batched"]
        gb = rb["error"] == 0
        fits.append(np.stack([snr[gb], cat.e1[gb], cat.e2[gb], rb["e1"][gb], rb["e2"][gb]], axis=1))
        ok = (res["batched"]["error"] == 0) & (res["plain"]["error"] == 0)
        de = np.maximum(np.abs(res["batched"]["e1"] - res["plain"]["e1"]),
                        np.abs(res["batched"]["e2"] - res["plain"]["e2"]))[ok]
        per_galaxy.append({"field": list(g), "good": int(ok.sum()), "frac_le_1e-3": float(np.mean(de <= 1e-3)),
                           "frac_le_1e-4": float(np.mean(de <= 1e-4)), "max": float(de.max())})
    out = {"workload": a.workload, "galaxies_per_field": n, "noise_scale": a.noise_scale,
           "fields": [list(g) for g in FIELDS], "abs_de_batched_vs_plain": per_galaxy}

    def bias(rr):
        t = np.array(rr)
        if not np.isfinite(t[:, 4:6]).all() or (t[:, 4:6] <= 0).any():  # a field with no pair left
            nan = float("nan")
            return {"g_measured": t[:, 2:4].tolist(), "galaxies_used": t[:, 6].tolist(),
                    **{k: nan for k in ("m1", "m1_err", "c1", "c1_err", "m2", "m2_err", "c2", "c2_err")}}
        m1, c1, m1e, c1e = shear.multiplicative_additive_bias(t[:, 0], t[:, 2], t[:, 4])
        m2, c2, m2e, c2e = shear.multiplicative_additive_bias(t[:, 1], t[:, 3], t[:, 5])
        return {"g_measured": t[:, 2:4].tolist(), "g_err": t[:, 4:6].tolist(), "galaxies_used": t[:, 6].tolist(),
                "m1": m1, "m1_err": m1e, "c1": c1, "c1_err": c1e, "m2": m2, "m2_err": m2e, "c2": c2, "c2_err": c2e}

    for name in ("batched", "plain"):
        out[name] = bias(rows[(cuts[0], name)])
    out["by_snr_cut"] = {f"{cut:g}": {name: {k: v for k, v in bias(rows[(cut, name)]).items()
                                             if k[0] in "mc" or k == "galaxies_used"}
                                      for name in ("batched", "plain")} for cut in cuts}
    f = np.concatenate(fits)
    edges = [0.0] + cuts + [np.inf]
    bands = []
    for lo, hi in zip(edges[:-1], edges[1:]):
        sel = (f[:, 0] >= lo) & (f[:, 0] < hi)
        if sel.sum() < 3:
            continue
        band = {"snr": [lo, hi if np.isfinite(hi) else None], "galaxies": int(sel.sum())}
        for c in (1, 2):
            s_, o_ = np.polyfit(f[sel, c], f[sel, c + 2], 1)
            band[f"slope{c}"], band[f"offset{c}"] = float(s_), float(o_)
        bands.append(band)
    out["response_by_snr"] = bands
    b, p = out["batched"], out["plain"]
    out["batched_minus_plain"] = {k: b[k] - p[k] for k in ("m1", "c1", "m2", "c2")}
    out["consistent_within_1sigma"] = bool(all(abs(b[k] - p[k]) <= b[k + "_err"] for k in ("m1", "c1", "m2", "c2")))
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
