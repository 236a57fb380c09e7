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


def test_against_reference_script_fixtures():
    """The reference's own shear.py run on fixed tables (tests/golden/make_shear_golden.py: its
    prints made calls, its bootstrap the identity so that the printed shear is the full-sample
    weighted mean): galaxies kept, bad count, shape noise and shear agree, including a table
    whose last row is a bad odd row (the reference's end-of-file slip)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "shear_golden.npz"))
    for name in ("clean", "bad_even_and_odd", "last_odd_bad"):
        t, ref = g[name + "_table"], g[name + "_out"]
        est = shear.estimate_shear(t[:, 2], t[:, 5], t[:, 3], t[:, 6], t[:, 7], t[:, 8], bootnum=50)
        ngal, bad, sigma, g1, g2 = ref[:5]
        assert est.n_used == int(ngal) and est.n_rejected == int(bad), name
        assert abs(est.shape_noise - sigma) <= 1e-12 * abs(sigma), name
        assert abs(est.g1 - g1) <= 1e-12 * abs(g1) and abs(est.g2 - g2) <= 1e-12 * abs(g2), name


def test_reference_selection_rules():
    n = 10
    ok = np.full(n, 0.01)
    v = ok.copy()
    v[3] = 0.0   # odd: drops row 2 (kept) and itself
    v[6] = 0.0   # even: drops itself and row 7 unread
    kept, bad = shear.reference_selection(np.full(n, 0.1), np.full(n, 0.1), v, np.full(n, 50.0))
    assert kept.tolist() == [0, 1, 4, 5, 8, 9] and bad == 2
    v = ok.copy()
    v[9] = 0.0   # the last row, odd: the reference deletes row 7 instead of row 8
    kept, bad = shear.reference_selection(np.full(n, 0.1), np.full(n, 0.1), v, np.full(n, 50.0))
    assert kept.tolist() == [0, 1, 2, 3, 4, 5, 6, 8] and bad == 1


def test_no_pair_left_gives_no_estimate():
    n = 6
    est = shear.estimate_shear(np.zeros(n), np.zeros(n), np.full(n, 0.1), np.full(n, 0.1), np.zeros(n))
    assert est.n_used == 0 and np.isnan(est.g1) and np.isnan(est.g2)
