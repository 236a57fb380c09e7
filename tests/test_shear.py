"""Shear estimator (shear.py restated): unbiased on a noiseless ring test, pair rejection, m/c fit."""
import numpy as np

from radiolensfit2_gb300 import shear, synth


def test_ring_test_recovers_shear():
    cat = synth.make_catalogue(2000, 10.0, 200.0, g=(0.03, -0.02), seed=5)
    n = cat.n
    est = shear.estimate_shear(cat.e1, cat.e2, np.full(n, 0.1), np.full(n, 0.1), np.full(n, 0.01), bootnum=200)
    # opposite-pair ring cancels the intrinsic shapes: the weighted mean is the shear to O(g^2 e^2)
    assert abs(est.g1 - 0.03) < 3e-3 and abs(est.g2 + 0.02) < 3e-3
    assert est.n_used == n


def test_pair_rejection():
    v = np.full(8, 0.01)
    v[3] = 0.0  # rejects row 3 and its partner 2
    ok = shear.select_pairs(np.full(8, 0.1), np.full(8, 0.1), v, np.full(8, 50.0))
    assert ok.tolist() == [True, True, False, False, True, True, True, True]


def test_bias_fit():
    gt = np.array([-0.04, -0.02, 0.0, 0.02, 0.04])
    gm = 1.05 * gt + 0.001
    m, c, me, ce = shear.multiplicative_additive_bias(gt, gm, np.full(5, 1e-3))
    assert abs(m - 0.05) < 1e-9 and abs(c - 0.001) < 1e-9
