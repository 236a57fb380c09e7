"""The device-resident pipeline (rlf_obs_*) against the oracle: facets from every extraction
kernel, fits of the F64 and mixed paths, and the batched mode against the one-galaxy-at-a-time
mode.  Tolerances: F64 follows the reference arithmetic (1e-11 on facets); the mixed path keeps
visibilities and model arithmetic in FP32 with compensated sums, so its facets agree to ~1e-6 of
the facet noise level and its fitted ellipticities to 1e-4 (the accuracy required of it)."""
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
    """Sequential modes against the oracle's data_processing (first pass, catalogue order).

    f64        FP64 everywhere: the reference's arithmetic, bit-for-bit simplex path.
    mixed      FP32 visibility passes, FP64 fit: the FP32 facet error is a smooth perturbation of
               the likelihood surface, so the fit follows the reference's simplex path and the
               fitted ellipticities stay within 1e-4 (log-likelihood within 1e-6 relative).
    mixed-fit  FP32 visibility passes and FP32 fit cells (rlf_options.fit_precision = RLF_MIXED):
               this mode does NOT meet the required bounds (|dL/L| <= 1e-6, |de| <= 1e-4).  Its
               log-likelihood is within ~4e-6 relative, and the rounding noise varies with
               (e1, e2) and changes nmsimplex2 decisions, so e agrees only statistically.  It is
               not the default and neither the bench nor the drop-in entry points select it; the
               asserts below pin what it achieves (median |de| < 1e-3, |dL/L| < 1e-5).
    """
    d_ref, s_ref, bad_ref, bl_ref, ref = oracle_data_processing(orc, case, case.data, sky)
    e_ref = np.array([(r[0], r[1]) for r in ref])
    L_ref = np.array([r[5] for r in ref])
    err_ref = np.array([r[6] for r in ref])
    out = {}
    modes = (("f64", _lib.RLF_F64, _lib.RLF_F64, 1, 0), ("mixed", _lib.RLF_MIXED, _lib.RLF_F64, 1, 0),
             ("mixed-fit", _lib.RLF_MIXED, _lib.RLF_MIXED, 1, 0), ("batched", _lib.RLF_MIXED, _lib.RLF_F64, 16, 3),
             ("batched-1round", _lib.RLF_MIXED, _lib.RLF_F64, 16, 1))
    changed = {}
    for name, prec, fprec, batch, rounds in modes:
        dev = _dev(case, sky, prec)
        pr = dev.process(case.cat, batch=batch, refit=False, fit_precision=fprec, rounds=rounds)
        out[name] = pr.results
        changed[name] = pr.stats["changed"]
        dev.close()
    f = out["f64"]
    assert np.array_equal(f["error"], err_ref)
    good = err_ref == 0
    # simplex maxima before the sampling step: same iterates as the oracle's nmsimplex2
    assert np.max(np.abs(f["max_e1"][good] - np.array([r[8] for r in ref])[good])) < 1e-9
    assert np.max(np.abs(f["max_e2"][good] - np.array([r[9] for r in ref])[good])) < 1e-9
    assert np.max(np.abs(f["e1"][good] - e_ref[good, 0])) < 1e-7
    assert np.max(np.abs(f["e2"][good] - e_ref[good, 1])) < 1e-7
    assert np.allclose(f["maxL"][good], L_ref[good], rtol=1e-9)
    de64 = np.maximum(np.abs(f["e1"][good] - e_ref[good, 0]), np.abs(f["e2"][good] - e_ref[good, 1]))
    print(f"f64: |de| max {de64.max():.2e}; |dL/L| max "
          f"{np.max(np.abs(f['maxL'][good] - L_ref[good]) / np.abs(L_ref[good])):.2e}")
    stats = {}
    for name in ("mixed", "mixed-fit", "batched", "batched-1round"):
        r = out[name]
        ok = good & (r["error"] == 0)
        de = np.maximum(np.abs(r["e1"][ok] - e_ref[ok, 0]), np.abs(r["e2"][ok] - e_ref[ok, 1]))
        dL = np.abs(r["maxL"][ok] - L_ref[ok]) / np.abs(L_ref[ok])
        stats[name] = (de, dL, int(np.sum(r["error"] != err_ref)))
        print(f"{name}: |de| max {de.max():.2e} median {np.median(de):.2e}; |dL/L| max {dL.max():.2e}; "
              f"errors {int(r['error'].sum())} vs {int(err_ref.sum())}; changed in last round {changed[name]}")
    de, dL, nerr = stats["mixed"]
    assert nerr == 0
    assert de.max() < 1e-4 and dL.max() < 1e-6
    de, dL, nerr = stats["mixed-fit"]
    # below the required bounds by design (see the docstring): a statistical check only
    assert nerr <= 1
    assert np.median(de) < 1e-3 and dL.max() < 1e-5
