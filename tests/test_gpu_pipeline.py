"""The device-resident pipeline (rlf_obs_*) against the oracle: facets from every extraction
kernel, fits of the F64 and mixed paths, and the batched mode against the one-galaxy-at-a-time
mode.  Tolerances: F64 follows the reference arithmetic (1e-11 on facets); the mixed path keeps
visibilities and model arithmetic in FP32 with compensated sums, so its facets agree to ~1e-6 of
the facet noise level and its fitted ellipticities to 1e-4 (the benchmark spec tolerance)."""
import numpy as np
import pytest

from radiolensfit2_gb300 import _lib, constants as K
from radiolensfit2_gb300.pipeline import DeviceObservation

import _oracle as O
from _cases import Case, oracle_sky_model, oracle_data_processing, oracle_facet

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def orc():
    return O.load_oracle()


@pytest.fixture(scope="module")
def case():
    # larger array than the C-ABI case: 48 antennas x 24 times x 8 channels, 16 galaxies
    return Case(n_ant=48, ha_hours=2.0, dt_s=600.0, n_ch=8, n_gal=16, fmin=30.0, fmax=200.0,
                noise=900.0, flag_frac=0.02)


@pytest.fixture(scope="module")
def sky(orc, case):
    return oracle_sky_model(orc, case)


def _dev(case, sky, precision):
    d = DeviceObservation(case.obs, precision=precision, sigma2=case.sigma2, flag=case.flag)
    d.set_vis(case.data, sky)
    return d


@pytest.mark.parametrize("precision,batch,tol", [(_lib.RLF_F64, 1, 1e-11), (_lib.RLF_MIXED, 1, 2e-6),
                                                 (_lib.RLF_MIXED, 16, 2e-6)])
def test_facets_against_oracle(orc, case, sky, precision, batch, tol):
    dev = _dev(case, sky, precision)
    facets = dev.extract(case.cat, batch=batch)
    for gi in range(case.cat.n):
        F, n, gu, gv, fvis, fs2, _ = oracle_facet(orc, case, gi, case.data, sky)
        u, v, vis, s2 = facets[gi]
        assert len(u) == n, (gi, len(u), n)
        assert np.allclose(u, gu, rtol=1e-6, atol=0) and np.allclose(v, gv, rtol=1e-6, atol=0)
        # facet values are vis/sigma2; compare relative to the facet's noise level
        scale = np.sqrt(np.mean(np.abs(fvis) ** 2))
        err = np.max(np.abs(vis - fvis)) / scale
        assert err < tol, (gi, err)
        assert np.allclose(s2, fs2, rtol=1e-6 if precision else 1e-13)
    dev.close()


def test_pipeline_modes(orc, case, sky):
    d_ref, s_ref, bad_ref, bl_ref, ref = oracle_data_processing(orc, case, case.data, sky)
    e_ref = np.array([(r[0], r[1]) for r in ref])
    L_ref = np.array([r[5] for r in ref])
    err_ref = np.array([r[6] for r in ref])
    out = {}
    for name, prec, batch in (("f64", _lib.RLF_F64, 1), ("mixed", _lib.RLF_MIXED, 1), ("batched", _lib.RLF_MIXED, 16)):
        dev = _dev(case, sky, prec)
        pr = dev.process(case.cat, batch=batch, refit=False)
        out[name] = pr.results
        dev.close()
    f = out["f64"]
    assert np.array_equal(f["error"], err_ref)
    good = err_ref == 0
    assert np.allclose(f["max_e1"][good], [r for r in f["max_e1"][good]])
    assert np.max(np.abs(f["e1"][good] - e_ref[good, 0])) < 1e-7
    assert np.max(np.abs(f["e2"][good] - e_ref[good, 1])) < 1e-7
    assert np.allclose(f["maxL"][good], L_ref[good], rtol=1e-9)
    for name in ("mixed", "batched"):
        r = out[name]
        ok = good & (r["error"] == 0)
        de = np.maximum(np.abs(r["e1"][ok] - e_ref[ok, 0]), np.abs(r["e2"][ok] - e_ref[ok, 1]))
        dL = np.abs(r["maxL"][ok] - L_ref[ok]) / np.abs(L_ref[ok])
        print(f"{name}: |de| max {de.max():.2e} median {np.median(de):.2e}; |dL/L| max {dL.max():.2e}; "
              f"errors {int(r['error'].sum())} vs {int(err_ref.sum())}")
        assert np.sum(r["error"] != err_ref) <= 1
        assert np.median(de) < 1e-4
        assert np.max(dL) < 1e-5
