"""The reference's CPU-runnable configuration, whole catalogue, against the oracle.

c0_small_cpu: 64 antennas (2,016 baselines) x 120 times x 4 channels = 967,680 visibilities, 100
galaxies at 10-200 uJy with the configuration's noise (SEFD 400 Jy: most fits fail, as they do in
the reference), both passes of data_processing (RadioLensfit2.cpp:597-606).  The data are the
device simulator's FP32 visibilities, handed to the oracle and to every GPU path as the same doubles.

Bounds: the F64 paths (one galaxy at a time and batched) follow the reference's arithmetic: error
flags equal for every galaxy, fitted e within 1e-9.  The batched mixed-precision path: error flags
equal, fitted e within 1e-4 (the FP32 visibility passes' bound).
"""
import types

import numpy as np
import pytest

from radiolensfit2_gb300 import _lib, synth
from radiolensfit2_gb300 import constants as K
from radiolensfit2_gb300.pipeline import DeviceObservation

import _oracle as O
from _cases import oracle_data_processing

pytestmark = pytest.mark.gpu


def test_whole_catalogue_c0():
    w = dict(synth.WORKLOADS["c0_small_cpu"])
    obs = synth.make_observation(**w)
    cat = synth.make_catalogue(w["n_gal"], w["fmin"], w["fmax"], g=w["g"])
    mixed = DeviceObservation(obs, precision=_lib.RLF_MIXED)
    mixed.simulate(cat, obs.sigma, seed=3)
    mixed.sky_model(cat)
    mixed.snapshot()
    data, sky = mixed.get_vis()
    case = types.SimpleNamespace(obs=obs, cat=cat, sigma2=np.full(obs.n_vis, np.float32(obs.sigma2), np.float32),
                                 flag=np.zeros(obs.n_vis, np.uint8), ro=np.array(K.ro_grid()), gaussian=0,
                                 len=obs.len_lambda)
    case.numr = len(case.ro)
    orc = O.load_oracle()
    d1, s1, nbad, bl, res1 = oracle_data_processing(orc, case, data, sky)
    _, _, _, _, res2 = oracle_data_processing(orc, case, d1, s1, re_fitting=True, bad_list=bl[:nbad])
    final = list(res1)
    for g in bl[:nbad]:
        final[int(g)] = res2[int(g)]
    ref_err = np.array([r[6] for r in final])
    ref_e = np.array([(r[0], r[1]) for r in final])
    assert 0 < int((ref_err == 0).sum()) < cat.n

    f64 = DeviceObservation(obs, precision=_lib.RLF_F64)
    runs = []
    for batch in (1, 1000):
        f64.set_vis(data, sky)
        runs.append((f"f64 batch {batch}", f64.process(cat, batch=batch, refit=True).results, 1e-9))
    f64.close()
    mixed.restore()
    runs.append(("mixed batched", mixed.process(cat, batch=1000, refit=True).results, 1e-4))
    mixed.close()
    for name, r, tol in runs:
        assert np.array_equal(r["error"], ref_err), name
        good = ref_err == 0
        de = np.maximum(np.abs(r["e1"][good] - ref_e[good, 0]), np.abs(r["e2"][good] - ref_e[good, 1]))
        print(f"{name}: {int(good.sum())} good of {cat.n}, |de| max {de.max():.2e}")
        assert de.max() <= tol, name
