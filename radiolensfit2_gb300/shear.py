"""Shear estimation from measured ellipticities (the reference's shear.py:32-145, restated).

The shear is the weighted mean of the measured ellipticities of galaxies whose simulated
intrinsic shapes come in opposite pairs (consecutive rows), with

  * selection: 1-D variance > 1e-5, both per-component errors > 1e-3, SNR >= snr_min; when a
    measurement is rejected its opposite partner is rejected too (shear.py:58-89);
  * shape noise sigma_e from the prior-weighted second moments of the measurements
    (shear.py:103-115), prior p(e) of shear.py:30-32;
  * weight w = 1 / (v e_max^2 / (e_max^2 - 2 v) + sigma_e), v the 1-D variance (shear.py:69,120);
  * bootstrap over pairs for the errors (shear.py:125-145), seeded for reproducibility.

With several fields of different input shear, `multiplicative_additive_bias` fits
g_measured = (1 + m) g_true + c per component.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

E_MAX = 0.804
E_0 = 0.0256
DISP = 0.2539
NORM = 2.43180252985281


def prior_ellipticity(e1, e2):
    emod = np.sqrt(e1 * e1 + e2 * e2)
    return NORM * emod * (1.0 - np.exp((emod - E_MAX) / DISP)) / ((1.0 + emod) * np.sqrt(emod * emod + E_0 * E_0))


@dataclass
class ShearEstimate:
    g1: float
    g2: float
    g1_err: float
    g2_err: float
    n_used: int
    n_rejected: int
    shape_noise: float


def select_pairs(err1, err2, onedvar, snr, snr_min=10.0):
    """Boolean mask of accepted rows; a rejected row also rejects its opposite partner."""
    n = len(onedvar)
    ok = (onedvar > 1e-5) & (err1 > 1e-3) & (err2 > 1e-3) & (snr >= snr_min)
    ok = np.asarray(ok, dtype=bool).copy()
    n2 = n - (n % 2)
    pair_ok = ok[0:n2:2] & ok[1:n2:2]
    ok[:] = False
    ok[0:n2:2] = pair_ok
    ok[1:n2:2] = pair_ok
    return ok


def estimate_shear(me1, me2, err1, err2, onedvar, snr=None, *, snr_min=10.0, bootnum=1000,
                   seed=0) -> ShearEstimate:
    me1, me2 = np.asarray(me1, float), np.asarray(me2, float)
    err1, err2 = np.asarray(err1, float), np.asarray(err2, float)
    var = np.asarray(onedvar, float)
    snr = np.full(len(me1), np.inf) if snr is None else np.asarray(snr, float)
    ok = select_pairs(err1, err2, var, snr, snr_min)
    e1, e2, v = me1[ok], me2[ok], var[ok]
    pe = prior_ellipticity(e1, e2)
    m1, m2 = np.average(e1, weights=pe), np.average(e2, weights=pe)
    v12 = np.average(e1 * e2, weights=pe) - m1 * m2
    v1 = np.average(e1 * e1, weights=pe) - m1 * m1
    v2 = np.average(e2 * e2, weights=pe) - m2 * m2
    sigma_shape = float(np.sqrt(max(v1 * v2 - v12 * v12, 0.0)))
    wvar = v * E_MAX * E_MAX / (E_MAX * E_MAX - 2 * v)
    w = 1.0 / (wvar + sigma_shape)
    npair = len(e1) // 2
    e1p, e2p, wp = e1[:2 * npair].reshape(npair, 2), e2[:2 * npair].reshape(npair, 2), w[:2 * npair].reshape(npair, 2)
    g1 = float(np.sum(e1p * wp) / np.sum(wp))
    g2 = float(np.sum(e2p * wp) / np.sum(wp))
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, npair, size=(bootnum, npair))
    ws = wp[idx]
    b1 = np.sum(e1p[idx] * ws, axis=(1, 2)) / np.sum(ws, axis=(1, 2))
    b2 = np.sum(e2p[idx] * ws, axis=(1, 2)) / np.sum(ws, axis=(1, 2))
    return ShearEstimate(g1=g1, g2=g2, g1_err=float(np.std(b1)), g2_err=float(np.std(b2)),
                         n_used=int(2 * npair), n_rejected=int(len(me1) - 2 * npair), shape_noise=sigma_shape)


def multiplicative_additive_bias(g_true, g_meas, g_err):
    """Weighted least squares of g_meas = (1 + m) g_true + c for one component over fields.
    Returns (m, c, m_err, c_err)."""
    g_true, g_meas, g_err = map(lambda a: np.asarray(a, float), (g_true, g_meas, g_err))
    W = 1.0 / g_err ** 2
    A = np.stack([g_true, np.ones_like(g_true)], axis=1)
    cov = np.linalg.inv(A.T @ (A * W[:, None]))
    slope, c = cov @ (A.T @ (W * g_meas))
    return float(slope - 1.0), float(c), float(np.sqrt(cov[0, 0])), float(np.sqrt(cov[1, 1]))


def read_table(path):
    """Read an output table written by data_processing (data_processing.c:101,136)."""
    rows = []
    with open(path) as f:
        for line in f:
            parts = [p.strip() for p in line.split("|")]
            if len(parts) < 11:
                continue
            try:
                rows.append([float(p) for p in parts[:11]])
            except ValueError:
                continue
    a = np.array(rows)
    cols = ["flux", "e1", "m_e1", "err1", "e2", "m_e2", "err2", "onedvar", "snr", "l", "m"]
    return {c: a[:, i] for i, c in enumerate(cols)} if len(a) else {c: np.zeros(0) for c in cols}
