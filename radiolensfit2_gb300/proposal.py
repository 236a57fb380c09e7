"""Learned proposal of the simplex start: training on simulated galaxies and use in the pipeline.

The network and its training and inference kernels are CUDA code of librlf_gb300.so
(csrc/rlf_proposal.cu: bf16 convolutions on the tcgen05 tensor cores, FP32 head, loss and Adam);
this module drives them:

* ``training_set`` simulates galaxies with the project's own visibility simulator on an array
  (rlf_obs_simulate + rlf_obs_sky_model) and extracts their facets with the batched extraction
  (rlf_obs_extract), which the library resamples to 64 x 64 x 4 images in the network's device
  store; targets are where the plain fit's simplex ends (its maximum) and ln scalelength;
* ``train`` runs Adam over the store (rlf_cnn_train_step) and keeps the parameters of the best
  validation loss;
* ``load`` hands a trained network to the pipeline (rlf_proposal_set_params), after which
  ``DeviceObservation.process(..., proposal=1)`` starts every fit at the proposal.

The reference's fit starts every galaxy at (0, 0) with step 0.1 (galaxy_fitting.c:59-65); the
fit itself is unchanged and has the last word on every proposal.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import time

import numpy as np

from . import _lib, constants as K, synth

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "proposal_weights.npz")
N_CONV_IN = (4, 32, 32, 32)


def param_count() -> int:
    return int(_lib.load().rlf_cnn_param_count())


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights, small biases, in the library's parameter layout."""
    rng = np.random.default_rng(seed)
    out = []
    for cin in N_CONV_IN:
        out.append(rng.standard_normal(32 * 9 * cin) * math.sqrt(2.0 / (9 * cin)))
        out.append(np.zeros(32))
    out.append(rng.standard_normal(4 * 512) * math.sqrt(1.0 / 512) * 0.1)
    out.append(np.array([0.0, 0.0, -0.5, -1.5]))
    p = np.concatenate(out).astype(np.float32)
    assert p.size == param_count()
    return p


class ProposalNet:
    """A network on the GPU with a device store of training images (rlf_cnn)."""

    def __init__(self, max_batch: int = 256, capacity: int = 0, params: np.ndarray | None = None):
        self.lib = _lib.load()
        self.h = self.lib.rlf_cnn_create(int(max_batch), int(capacity))
        if not self.h:
            raise RuntimeError("rlf_cnn_create failed")
        self.max_batch, self.capacity = max_batch, capacity
        self.set_params(init_params() if params is None else params)

    def close(self):
        if getattr(self, "h", None):
            self.lib.rlf_cnn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        if self.lib.rlf_cnn_set_params(self.h, p.ctypes.data_as(_lib.PF)):
            raise RuntimeError("rlf_cnn_set_params failed")

    def get_params(self) -> np.ndarray:
        p = np.zeros(param_count(), np.float32)
        if self.lib.rlf_cnn_get_params(self.h, p.ctypes.data_as(_lib.PF)):
            raise RuntimeError("rlf_cnn_get_params failed")
        return p

    def store_facets(self, first, facets, ncoords, facet, flux, length):
        facets = np.ascontiguousarray(facets, np.float64)
        n, five, stride = facets.shape
        assert five == 5
        nc = np.ascontiguousarray(ncoords, np.int32)
        fa = np.ascontiguousarray(facet, np.int32)
        fl = np.ascontiguousarray(flux, np.float64)
        if self.lib.rlf_cnn_store_facets(self.h, int(first), n, facets.ctypes.data_as(_lib.PD), stride,
                                         nc.ctypes.data_as(_lib.PI), fa.ctypes.data_as(_lib.PI),
                                         fl.ctypes.data_as(_lib.PD), float(length)):
            raise RuntimeError("rlf_cnn_store_facets failed")

    def set_targets(self, first, targets):
        t = np.ascontiguousarray(targets, np.float32)
        if self.lib.rlf_cnn_set_targets(self.h, int(first), len(t), t.ctypes.data_as(_lib.PF)):
            raise RuntimeError("rlf_cnn_set_targets failed")

    def train_step(self, idx, lr) -> float:
        idx = np.ascontiguousarray(idx, np.int32)
        loss = np.zeros(1, np.float32)
        if self.lib.rlf_cnn_train_step(self.h, idx.ctypes.data_as(_lib.PI), len(idx), float(lr),
                                       loss.ctypes.data_as(_lib.PF)):
            raise RuntimeError("rlf_cnn_train_step failed")
        return float(loss[0])

    def loss_of(self, idx) -> float:
        idx = np.ascontiguousarray(idx, np.int32)
        loss = np.zeros(1, np.float32)
        if self.lib.rlf_cnn_grads(self.h, idx.ctypes.data_as(_lib.PI), len(idx), None, loss.ctypes.data_as(_lib.PF),
                                  None):
            raise RuntimeError("rlf_cnn_grads failed")
        return float(loss[0])

    def predict(self, first, n) -> np.ndarray:
        out = np.zeros((n, 4), np.float32)
        if self.lib.rlf_cnn_predict(self.h, int(first), int(n), out.ctypes.data_as(_lib.PF)):
            raise RuntimeError("rlf_cnn_predict failed")
        return out


def facet_sizes(cat, length) -> np.ndarray:
    """facet side of each galaxy as the pipeline chooses it (facet_size of the catalogue scale,
    at most facet_size(RMAX) and at least 2)"""
    fmax = K.facet_size(K.RMAX, length)
    return np.array([min(max(K.facet_size(s, length), 2), fmax) for s in cat.scale], np.int32)


def extract_raw(dev, cat, batch=1000):
    """rlf_obs_extract into [n][5][stride] doubles (u, v, vis/sigma^2 re, im, sigma^2) and cell counts"""
    lib = _lib.load()
    length = dev.obs.len_lambda
    stride = K.facet_size(K.RMAX, length) ** 2
    arrs = [np.ascontiguousarray(x, np.float64) for x in (cat.flux, cat.scale, cat.l, cat.m)]
    buf = np.zeros((cat.n, 5, stride))
    nc = np.zeros(cat.n, np.int32)
    if lib.rlf_obs_extract(dev.h, cat.n, *[a.ctypes.data_as(_lib.PD) for a in arrs], int(batch),
                           buf.ctypes.data_as(_lib.PD), stride, nc.ctypes.data_as(_lib.PI)):
        raise RuntimeError("rlf_obs_extract failed")
    return buf, nc


def training_set(net: ProposalNet, n_gal: int, *, workload="c2_ska_mid_32ch", per_obs=10000, seed=10,
                 fmin=10.0, fmax=200.0, g=(0.03, -0.02), first=0, verbose=True):
    """Simulate n_gal galaxies (catalogue distributions of the small CPU configuration: flux 10-200 uJy,
    shear g) on `workload`'s array, per_obs per simulated observation, extract their facets and
    store images and targets in the network's store from `first`.  Targets: the maximum of the
    plain fit's simplex (where the proposal should start it), else the true sheared ellipticity, and
    ln scalelength.  Returns the observation and the catalogues."""
    from .pipeline import DeviceObservation
    w = dict(synth.WORKLOADS[workload])
    obs = synth.make_observation(**w)
    cats = []
    done = 0
    k = 0
    while done < n_gal:
        m = min(per_obs, n_gal - done)
        t0 = time.time()
        cat = synth.make_catalogue(m, fmin, fmax, g=g, seed=seed * 1000 + k)
        dev = DeviceObservation(obs)
        dev.simulate(cat, obs.sigma, seed=seed * 1000 + k)
        dev.sky_model(cat)
        buf, nc = extract_raw(dev, cat)
        fit = dev.process(cat, batch=1000, refit=False).results
        dev.close()
        me1, me2 = fit["max_e1"], fit["max_e2"]
        ok = np.isfinite(me1) & np.isfinite(me2) & (me1 * me1 + me2 * me2 < 0.65)
        t1 = np.where(ok, me1, cat.e1)
        t2 = np.where(ok, me2, cat.e2)
        net.store_facets(first + done, buf, nc, facet_sizes(cat, obs.len_lambda), cat.flux, obs.len_lambda)
        net.set_targets(first + done, np.stack([t1, t2, np.log(cat.scale)], 1))
        cats.append(cat)
        done += m
        k += 1
        if verbose:
            print(f"  training set: {done}/{n_gal} galaxies ({time.time() - t0:.1f} s for {m})", flush=True)
    return obs, cats


def train(net: ProposalNet, n_train: int, n_val: int, *, epochs=12, batch=256, lr=2e-3, seed=0, verbose=True):
    """Adam over store images [0, n_train), validation on [n_train, n_train + n_val); cosine
    learning-rate decay; returns (best params, history)."""
    rng = np.random.default_rng(seed)
    steps_per_epoch = max(1, n_train // batch)
    total = epochs * steps_per_epoch
    val_idx = np.arange(n_train, n_train + n_val, dtype=np.int32)
    best, best_p, hist = math.inf, net.get_params(), []
    step = 0
    for ep in range(epochs):
        perm = rng.permutation(n_train).astype(np.int32)
        t0 = time.time()
        tl = []
        for s in range(steps_per_epoch):
            cur = lr * 0.5 * (1.0 + math.cos(math.pi * step / total))
            tl.append(net.train_step(perm[s * batch:(s + 1) * batch], cur))
            step += 1
        vl = float(np.mean([net.loss_of(val_idx[i:i + batch]) for i in range(0, n_val, batch)
                            if len(val_idx[i:i + batch]) > 0]))
        hist.append((ep, float(np.mean(tl)), vl, time.time() - t0))
        if verbose:
            print(f"  epoch {ep}: train loss {np.mean(tl):.4f} val loss {vl:.4f} ({time.time() - t0:.1f} s)", flush=True)
        if vl < best:
            best, best_p = vl, net.get_params()
    return best_p, hist


def save(params, path=WEIGHTS, **meta):
    np.savez(path, params=np.asarray(params, np.float32), **{k: np.asarray(v) for k, v in meta.items()})


def load(path=WEIGHTS, max_sigma: float | None = None) -> np.ndarray:
    """Load trained parameters and hand them to the pipeline (rlf_proposal_set_params); max_sigma:
    the gate above which a galaxy keeps the reference's start (default: the stored one, else 0.05)."""
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path}: no trained proposal network")
    p = np.ascontiguousarray(np.load(path)["params"], np.float32)
    if p.size != param_count():
        raise ValueError("proposal parameters of another layout")
    lib = _lib.load()
    if lib.rlf_proposal_set_params(p.ctypes.data_as(_lib.PF)):
        raise RuntimeError("rlf_proposal_set_params failed")
    if max_sigma is None:
        z = np.load(path)
        max_sigma = float(z["max_sigma"]) if "max_sigma" in z else 0.05
    if lib.rlf_proposal_set_max_sigma(float(max_sigma)):
        raise RuntimeError("rlf_proposal_set_max_sigma failed")
    return p


def unload():
    _lib.load().rlf_proposal_set_params(None)
