"""Synthetic array / catalogue generators: shapes and distributions of the measured workloads."""
import math

import numpy as np

from radiolensfit2_gb300 import constants as K, synth


def test_array_shapes_match_workloads():
    o = synth.make_observation(n_ant=64, ha_hours=2.0, dt_s=120.0, n_ch=4)
    assert o.n_rows == 2016 * 120 and o.n_vis == 2016 * 120 * 4
    assert o.len_metres == math.ceil(max(np.abs(o.uu).max(), np.abs(o.vv).max()))
    assert np.all(np.diff(o.wavenumbers) > 0)
    f0 = 950e6 + 120e3
    assert o.wavenumbers[0] == 2.0 * K.PI * f0 / K.C0
    assert o.spec[0] == math.pow(f0 / 1.4e9, -0.7)
    assert abs(o.sigma - 400e6 / math.sqrt(2 * 120 * 240e3)) < 1e-9
    # facet sizes quoted for the SKA-MID-like array: 4 at 0.3", 34 at 3.5"
    big = synth.make_observation(n_ant=197, ha_hours=0.05, dt_s=60.0, n_ch=16)
    assert 30 <= K.facet_size(K.RMAX, big.len_lambda) <= 36


def test_catalogue_distributions():
    c = synth.make_catalogue(10000, 10.0, 200.0, g=(0.03, -0.02))
    assert c.n == 10000
    assert np.all(np.diff(c.flux) <= 0) and c.flux.min() >= 10.0 and c.flux.max() <= 200.0
    r = np.hypot(c.l, c.m)
    assert r.max() <= math.radians(0.5)
    e = np.hypot(c.e1_int, c.e2_int)
    assert e.max() < K.E_MAX
    # ring construction: each group of 2*NUM_ORIENT shares |e|, and the intrinsic ellipticities cancel
    grp = e[:10]
    assert np.allclose(grp, grp[0])
    assert abs(c.e1_int[:10].sum()) < 1e-12
    # shear shifts the mean ellipticity by ~g
    assert abs(c.e1.mean() - 0.03) < 0.01 and abs(c.e2.mean() + 0.02) < 0.01
    med = np.median(c.scale[c.flux < 12.0])
    assert 0.2 < med < 0.45
