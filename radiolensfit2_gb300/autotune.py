"""Autotuner of the batched pipeline's launch shapes.

Two shapes of the batched path are left to tuning (rlf_options):

* ``seq_facet_kb``: the shared memory of one sequential-extraction sub-batch's compensated facet
  accumulators, which sets how many consecutive galaxies one extraction pass over the visibilities
  carries (more galaxies per pass, fewer passes and fit launches; fewer, smaller and better-filled
  fit launches at the end of a window);
* ``fit_ctas_per_sm``: persistent fit thread blocks per SM (one block fits one galaxy; more
  blocks share an SM's FP64 pipes and shared memory, fewer leave helpers idle).

``tune`` times every candidate on one window of galaxies from the same device data (the data are
restored from the observation's snapshot before each run), CUDA-event device time of both passes,
and keeps the fastest.  Results are cached per (rows, channels, histogram of facet sizes in the
window), in memory and, when RLF_TUNE_CACHE names a JSON file, on disk.  Every candidate gives the
FP64 path's results unchanged (tests/test_gpu_autotune.py); the FP32 batched path's results move
only at its FP32 rounding level, as sub-batch boundaries move.
"""
from __future__ import annotations

import json
import os

import numpy as np

from . import constants as K

CANDIDATES = tuple(dict(seq_facet_kb=kb, fit_ctas_per_sm=c) for kb in (96, 128, 160, 192) for c in (2, 3))
_cache: dict = {}


def _key(obs, cat) -> str:
    fmax = K.facet_size(K.RMAX, obs.len_lambda)
    sizes = [min(max(K.facet_size(s, obs.len_lambda), 2), fmax) for s in cat.scale]
    hist = np.bincount(np.array(sizes) // 2, minlength=fmax // 2 + 1)
    frac = np.round(hist / max(1, len(sizes)), 1)  # coarse: windows of the same kind share a key
    return f"{obs.n_rows}x{obs.n_ch}:" + ",".join(f"{x:.1f}" for x in frac)


def _load_disk():
    path = os.environ.get("RLF_TUNE_CACHE")
    if path and os.path.exists(path):
        try:
            with open(path) as f:
                _cache.update(json.load(f))
        except (OSError, ValueError):
            pass


def _save_disk():
    path = os.environ.get("RLF_TUNE_CACHE")
    if path:
        with open(path, "w") as f:
            json.dump(_cache, f, indent=1)


def tune(dev, cat, *, batch=1000, fit_precision=0, rounds=0, proposal=0, candidates=CANDIDATES,
         restore=True, force=False):
    """Fastest candidate for this window of galaxies on this observation.  `dev` must hold a snapshot
    (DeviceObservation.snapshot) of the data the window starts from; it is restored before every
    candidate and left restored.  Returns (choice dict, {candidate: device ms})."""
    _load_disk()
    key = _key(dev.obs, cat)
    if key in _cache and not force:
        return dict(_cache[key]["choice"]), _cache[key]["ms"]
    timings = {}
    for cand in candidates:
        if restore:
            dev.restore()
        r = dev.process(cat, batch=batch, refit=True, fit_precision=fit_precision, rounds=rounds,
                        proposal=proposal, **cand)
        timings[json.dumps(cand, sort_keys=True)] = float(r.ms[0])
    if restore:
        dev.restore()
    best = min(timings, key=timings.get)
    _cache[key] = {"choice": json.loads(best), "ms": timings}
    _save_disk()
    return json.loads(best), timings
