"""The autotuner's candidate launch shapes: every candidate gives the FP64 path's results to 1e-11
relative, with equal error flags and evaluation counts (the FP64 path takes galaxies one at a time;
the number of fit thread blocks changes which block evaluates each sampling-grid point, and the
results are not bit-identical across candidates), the batched FP32 path stays within its accuracy
against the FP64 path for every candidate, and the tuner returns one of the candidates with a
timing for each."""
import numpy as np
import pytest

from radiolensfit2_gb300 import _lib, autotune
from radiolensfit2_gb300.pipeline import DeviceObservation

import _oracle as O
from _cases import Case, oracle_sky_model

pytestmark = pytest.mark.gpu


def test_candidates_keep_f64_results_identical():
    orc = O.load_oracle()
    case = Case(n_ant=40, n_gal=10, fmin=30.0, fmax=200.0, noise=900.0, flag_frac=0.02)
    sky = oracle_sky_model(orc, case)
    f64 = DeviceObservation(case.obs, precision=_lib.RLF_F64, sigma2=case.sigma2, flag=case.flag)
    f64.set_vis(case.data, sky)
    f64.snapshot()
    base = None
    for cand in autotune.CANDIDATES:
        f64.restore()
        r = f64.process(case.cat, batch=1, refit=True, **cand).results
        if base is None:
            base = r
        else:
            for k in ("error", "nevals"):
                assert np.array_equal(r[k], base[k]), (cand, k)
            for k in ("e1", "e2", "var_e1", "var_e2", "maxL"):
                d = np.max(np.abs(r[k] - base[k]) / np.maximum(np.abs(base[k]), 1e-3))
                print(cand, k, f"{d:.1e}")
                assert d < 1e-11, (cand, k, d)
    f64.close()
    mixed = DeviceObservation(case.obs, precision=_lib.RLF_MIXED, sigma2=case.sigma2, flag=case.flag)
    mixed.set_vis(case.data, sky)
    mixed.snapshot()
    good = base["error"] == 0
    for cand in autotune.CANDIDATES:
        mixed.restore()
        r = mixed.process(case.cat, batch=64, refit=True, **cand).results
        assert np.array_equal(r["error"], base["error"]), cand
        de = np.maximum(np.abs(r["e1"] - base["e1"]), np.abs(r["e2"] - base["e2"]))[good]
        assert de.max() < 1e-4, (cand, de.max())
    choice, ms = autotune.tune(mixed, case.cat, batch=64, force=True)
    mixed.close()
    assert choice in [dict(c) for c in autotune.CANDIDATES]
    assert len(ms) == len(autotune.CANDIDATES) and all(v > 0 for v in ms.values())
