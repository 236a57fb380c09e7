"""Further modes of the device pipeline against the oracle's data_processing:

* the Gaussian profile (the reference's -DGAUSSIAN build), F64 one galaxy at a time and batched;
* a batch holding a galaxy whose facet is larger than the batched kernels take (F > 28): it is
  extracted, fitted and removed on its own at its place in the catalogue order;
* both passes (catalogue pass, then the re-fit of the bad galaxies, RadioLensfit2.cpp:597-606)
  through the batched path, including the final data and sky model.

Tolerances: the F64 path follows the reference arithmetic (fitted e within 1e-7); the batched
path (FP32 visibility passes, FP64 fit, 3 rounds) within 1e-4 in e, the accuracy required of it.
"""
import numpy as np
import pytest

from radiolensfit2_gb300 import _lib
from radiolensfit2_gb300.pipeline import DeviceObservation

import _oracle as O
from _cases import Case, oracle_sky_model, oracle_data_processing

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def orc():
    return O.load_oracle()


def _dev(case, sky, precision):
    d = DeviceObservation(case.obs, precision=precision, sigma2=case.sigma2, flag=case.flag)
    d.set_vis(case.data, sky)
    return d


def _compare(results, ref, tol, name):
    err_ref = np.array([r[6] for r in ref])
    e_ref = np.array([(r[0], r[1]) for r in ref])
    assert np.array_equal(results["error"], err_ref), name
    good = err_ref == 0
    assert good.any(), name
    de = np.maximum(np.abs(results["e1"][good] - e_ref[good, 0]), np.abs(results["e2"][good] - e_ref[good, 1]))
    print(f"{name}: |de| max {de.max():.2e} median {np.median(de):.2e} over {int(good.sum())} galaxies")
    assert de.max() < tol, name


def test_gaussian_profile(orc):
    case = Case(n_ant=48, ha_hours=2.0, dt_s=600.0, n_ch=8, n_gal=12, fmin=30.0, fmax=200.0, noise=900.0,
                flag_frac=0.02, gaussian=True)
    sky = oracle_sky_model(orc, case)
    _, _, _, _, ref = oracle_data_processing(orc, case, case.data, sky)
    for name, prec, batch, tol in (("gaussian f64", _lib.RLF_F64, 1, 1e-7),
                                   ("gaussian batched", _lib.RLF_MIXED, 12, 1e-4)):
        dev = _dev(case, sky, prec)
        pr = dev.process(case.cat, batch=batch, refit=False, gaussian=1, rounds=3)
        dev.close()
        _compare(pr.results, ref, tol, name)


def test_batch_with_large_facet(orc):
    # galaxy 5 gets a 30-cell facet: a one-galaxy unit between two sequential sub-batches
    case = Case(n_ant=48, ha_hours=2.0, dt_s=600.0, n_ch=8, n_gal=12, fmin=30.0, fmax=200.0, noise=900.0,
                flag_frac=0.02, scale_override={5: 3.3})
    sky = oracle_sky_model(orc, case)
    _, _, _, _, ref = oracle_data_processing(orc, case, case.data, sky)
    dev = _dev(case, sky, _lib.RLF_MIXED)
    pr = dev.process(case.cat, batch=12, refit=False, rounds=3)
    dev.close()
    assert pr.stats["extract_single"] >= 1 and pr.stats["extract_passes"] >= 2
    _compare(pr.results, ref, 1e-4, "large facet")


@pytest.mark.parametrize("n_ch", [8, 64])
def test_batched_two_passes(orc, n_ch):
    # 64 channels: four full chunks, the extraction and removal code compiled per chunk
    case = Case(n_ant=48, ha_hours=2.0, dt_s=600.0, n_ch=n_ch, n_gal=16, fmin=10.0, fmax=200.0, noise=1500.0,
                flag_frac=0.02)
    sky = oracle_sky_model(orc, case)
    d1, s1, nbad, bl, res1 = oracle_data_processing(orc, case, case.data, sky)
    assert nbad > 0
    d2, s2, nbad2, _, res2 = oracle_data_processing(orc, case, d1, s1, re_fitting=True, bad_list=bl[:nbad])
    final = list(res1)
    for g in bl[:nbad]:
        final[int(g)] = res2[int(g)]
    dev = _dev(case, sky, _lib.RLF_MIXED)
    pr = dev.process(case.cat, batch=16, refit=True, rounds=3)
    d, s = dev.get_vis()
    dev.close()
    assert pr.n_bad == nbad2
    _compare(pr.results, final, 1e-4, "two passes")
    # bad galaxies of the re-fit pass are written with e = 0 (data_processing.c:97-103)
    for g in np.nonzero(pr.results["error"])[0]:
        assert pr.results["e1"][g] == 0.0 and pr.results["e2"][g] == 0.0
    # data and sky model after both passes: FP32 storage, relative to their scale
    assert np.max(np.abs(d - d2)) < 1e-5 * np.max(np.abs(d2))
    assert np.max(np.abs(s - s2)) < 1e-5 * np.max(np.abs(sky))


@pytest.mark.parametrize("gaussian,n_ch", [(0, 8), (1, 8), (0, 16), (1, 16)])
def test_sky_model_and_simulator(orc, gaussian, n_ch):
    """rlf_obs_sky_model (round models, data_simulation.c:131-165) and the noise-free
    rlf_obs_simulate (sheared models) against the oracle's per-galaxy, per-channel model
    visibilities (galaxy_visibilities.c:154-190); 16 channels take the single-chunk kernels."""
    case = Case(n_ant=48, ha_hours=2.0, dt_s=600.0, n_ch=n_ch, n_gal=12, fmin=30.0, fmax=200.0, noise=0.0,
                gaussian=bool(gaussian))
    o, c = case.obs, case.cat
    sky_ref = oracle_sky_model(orc, case)
    data_ref = np.zeros(o.n_vis, np.complex128)
    one = np.zeros(o.n_rows, np.complex128)
    for gi in range(c.n):
        for ch in range(o.n_ch):
            orc.orc_data_galaxy_vis(o.spec[ch], o.wavenumbers[ch], c.e1[gi], c.e2[gi], c.scale[gi], c.flux[gi],
                                    c.l[gi], c.m[gi], o.n_rows, O.dp(o.uu), O.dp(o.vv), O.dp(o.ww), O.cp(one),
                                    gaussian)
            data_ref[ch * o.n_rows:(ch + 1) * o.n_rows] += one
    # F64 observations follow the reference arithmetic; FP32 ones carry the phase argument as
    # double-float and round every visibility to FP32
    for prec, tol in ((_lib.RLF_F64, 1e-12), (_lib.RLF_MIXED, 2e-6)):
        dev = DeviceObservation(o, precision=prec, sigma2=case.sigma2, flag=case.flag)
        dev.set_vis(np.zeros(o.n_vis, np.complex128), np.zeros(o.n_vis, np.complex128))
        dev.sky_model(c, gaussian=gaussian)
        dev.simulate(c, 0.0, gaussian=gaussian)
        d, s = dev.get_vis()
        dev.close()
        es = np.max(np.abs(s - sky_ref)) / np.max(np.abs(sky_ref))
        ed = np.max(np.abs(d - data_ref)) / np.max(np.abs(data_ref))
        print(f"precision {prec} gaussian {gaussian}: sky model {es:.2e}, simulated data {ed:.2e}")
        assert es < tol and ed < tol


@pytest.mark.parametrize("n_ch,gaussian", [(16, 0), (32, 0), (16, 1), (48, 1), (64, 0)])
def test_batched_full_chunks(orc, n_ch, gaussian):
    """The batched path on 16 to 64 channels, where most work items are single-run 16-channel
    chunks (the kernels' fast path; 16 channels: the single-chunk variant with compile-time channel
    constants; 32-64 channels: the item code compiled for each chunk) and the galaxy profiles come
    from the chunk polynomials, against the oracle's one-galaxy-at-a-time data_processing."""
    case = Case(n_ant=40, ha_hours=2.0, dt_s=600.0, n_ch=n_ch, n_gal=12, fmin=30.0, fmax=200.0, noise=1500.0,
                flag_frac=0.01, gaussian=bool(gaussian))
    sky = oracle_sky_model(orc, case)
    _, _, _, _, ref = oracle_data_processing(orc, case, case.data, sky)
    dev = _dev(case, sky, _lib.RLF_MIXED)
    pr = dev.process(case.cat, batch=12, refit=False, gaussian=gaussian, rounds=3)
    dev.close()
    _compare(pr.results, ref, 1e-4, f"{n_ch} channels, gaussian {gaussian}")
