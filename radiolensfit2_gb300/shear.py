"""Shear estimation from measured ellipticities (the reference's shear.py:32-145, restated).

The shear is the weighted mean of the measured ellipticities of galaxies whose simulated
intrinsic shapes come in opposite pairs (consecutive rows), with

  * selection: 1-D variance > 1e-5, both per-component errors > 1e-3, SNR >= snr_min; when a
    measurement is rejected its opposite partner is rejected too (shear.py:58-99, with the
    reference's slip at the end of a table reproduced);
  * shape noise sigma_e from the second moments of the measurements (shear.py:103-115); the
    reference's prior_ellipticity (shear.py:30-32) returns nothing, so its moments are unweighted,
    as here by default;
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


def reference_selection(err1, err2, onedvar, snr, snr_min=10.0):
    """Rows kept by the reference's reading loop (shear.py:58-99), in its order, and its count of
    bad measurements.  A row is good when var > 1e-5, both errors > 1e-3 and SNR >= snr_min.  A bad
    even row (0-based) also drops the next row unread; a bad odd row drops the kept previous row
    (the next good row overwrites its slot).  When the last row read is a bad odd row, the
    reference deletes the element before the dropped one instead of the dropped one
    (shear.py:93-99: k is decremented twice); that is reproduced so that results agree.  Returns
    (indices of the kept rows in list order, number of bad measurements)."""
    n = len(onedvar)
    kept = []
    remove = False
    bad = 0
    i = 0
    while i < n:
        good = onedvar[i] > 1e-5 and err1[i] > 1e-3 and err2[i] > 1e-3 and snr[i] >= snr_min
        if good:
            if remove:
                kept[-1] = i
            else:
                kept.append(i)
            remove = False
        else:
            if i % 2 != 0:
                remove = True
            else:
                i += 1
            bad += 1
        i += 1
    if remove:
        # shear.py:93-99: the slot of the dropped row is the last one; the reference deletes the one
        # before it
        if len(kept) >= 2:
            del kept[-2]
        elif kept:
            del kept[-1]
    return np.array(kept, dtype=np.int64), bad


def select_pairs(err1, err2, onedvar, snr, snr_min=10.0):
    """Boolean mask of accepted rows; a rejected row also rejects its opposite partner (the
    reference's rule without its end-of-file slip)."""
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
                   seed=0, prior_weighted_moments=False) -> ShearEstimate:
    """The reference's estimator (shear.py:58-145).  Its shape-noise moments are unweighted: its
    prior_ellipticity (:30-32) returns nothing, so np.average receives weights=None; pass
    prior_weighted_moments=True for the prior-weighted moments that function describes.  The
    errors come from a seeded bootstrap over the pairs (the reference's astropy bootstrap is
    unseeded)."""
    me1, me2 = np.asarray(me1, float), np.asarray(me2, float)
    err1, err2 = np.asarray(err1, float), np.asarray(err2, float)
    var = np.asarray(onedvar, float)
    snr = np.full(len(me1), np.inf) if snr is None else np.asarray(snr, float)
    kept, bad = reference_selection(err1, err2, var, snr, snr_min)
    if len(kept) < 2:  # no pair left: no estimate (the reference's script fails on an empty sample)
        nan = float("nan")
        return ShearEstimate(g1=nan, g2=nan, g1_err=nan, g2_err=nan, n_used=int(len(kept)), n_rejected=int(bad),
                             shape_noise=nan)
    e1, e2, v = me1[kept], me2[kept], var[kept]
    pe = prior_ellipticity(e1, e2) if prior_weighted_moments else None
    m1, m2 = np.average(e1, weights=pe), np.average(e2, weights=pe)
    v12 = np.average(e1 * e2, weights=pe) - m1 * m2
    v1 = np.average(e1 * e1, weights=pe) - m1 * m1
    v2 = np.average(e2 * e2, weights=pe) - m2 * m2
    sigma_shape = float(np.sqrt(max(v1 * v2 - v12 * v12, 0.0)))
    wvar = v * E_MAX * E_MAX / (E_MAX * E_MAX - 2 * v)
    w = 1.0 / (wvar + sigma_shape)
    npair = len(e1) // 2
    e1p, e2p, wp = e1[:2 * npair].reshape(npair, 2), e2[:2 * npair].reshape(npair, 2), w[:2 * npair].reshape(npair, 2)
    g1 = float(np.average(e1p, weights=wp))
    g2 = float(np.average(e2p, weights=wp))
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, npair, size=(bootnum, npair))
    ws = wp[idx]
    b1 = np.sum(e1p[idx] * ws, axis=(1, 2)) / np.sum(ws, axis=(1, 2))
    b2 = np.sum(e2p[idx] * ws, axis=(1, 2)) / np.sum(ws, axis=(1, 2))
    return ShearEstimate(g1=g1, g2=g2, g1_err=float(np.std(b1)), g2_err=float(np.std(b2)),
                         n_used=int(len(e1)), n_rejected=int(bad), shape_noise=sigma_shape)


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
