"""Edge cases of the device pipeline against the oracle's data_processing: an empty catalogue, a
single galaxy through a batch, every visibility flagged (empty facets: every fit is bad and nothing
is removed), a batch larger than the catalogue, four rounds, and the fit's bounded wait for
sampling-grid points running out."""
import dataclasses

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


def _check(results, ref, tol):
    err_ref = np.array([r[6] for r in ref])
    assert np.array_equal(results["error"], err_ref)
    good = err_ref == 0
    if good.any():
        e_ref = np.array([(r[0], r[1]) for r in ref])
        de = np.maximum(np.abs(results["e1"][good] - e_ref[good, 0]), np.abs(results["e2"][good] - e_ref[good, 1]))
        assert de.max() < tol


def test_empty_catalogue():
    case = Case(n_gal=3)
    cat = dataclasses.replace(case.cat, **{f: getattr(case.cat, f)[:0] for f in
                                           ("flux", "scale", "e1", "e2", "e1_int", "e2_int", "l", "m")})
    for prec, batch in ((_lib.RLF_F64, 1), (_lib.RLF_MIXED, 16)):
        dev = _dev(case, np.zeros(case.obs.n_vis, np.complex128), prec)
        pr = dev.process(cat, batch=batch, refit=True, rounds=3)
        d, _ = dev.get_vis()
        dev.close()
        assert len(pr.results) == 0 and pr.n_bad == 0
        assert np.array_equal(d.astype(np.complex64), case.data.astype(np.complex64))


@pytest.mark.parametrize("prec,batch,tol", [(_lib.RLF_F64, 1, 1e-7), (_lib.RLF_MIXED, 16, 1e-4)])
def test_single_galaxy(orc, prec, batch, tol):
    case = Case(n_gal=1, fmin=150.0, fmax=200.0, noise=300.0)
    sky = oracle_sky_model(orc, case)
    _, _, _, _, ref = oracle_data_processing(orc, case, case.data, sky)
    dev = _dev(case, sky, prec)
    pr = dev.process(case.cat, batch=batch, refit=False, rounds=3)
    dev.close()
    _check(pr.results, ref, tol)


@pytest.mark.parametrize("prec,batch", [(_lib.RLF_F64, 1), (_lib.RLF_MIXED, 8)])
def test_all_flagged(orc, prec, batch):
    case = Case(n_gal=5, flag_frac=1.0)
    assert case.flag.all()
    sky = oracle_sky_model(orc, case)
    d_ref, s_ref, nbad, _, ref = oracle_data_processing(orc, case, case.data, sky)
    assert nbad == case.cat.n
    dev = _dev(case, sky, prec)
    pr = dev.process(case.cat, batch=batch, refit=True, rounds=3)
    d, s = dev.get_vis()
    dev.close()
    _check(pr.results, ref, 1e-7)
    assert pr.n_bad == case.cat.n and np.all(pr.results["ncoords"] == 0)
    # nothing removed
    scale = np.max(np.abs(case.data))
    assert np.max(np.abs(d - d_ref)) < 1e-6 * scale and np.max(np.abs(s - s_ref)) < 1e-6 * max(np.max(np.abs(sky)), 1.0)


@pytest.mark.parametrize("batch,rounds", [(64, 3), (7, 4)])
def test_batch_shapes(orc, batch, rounds):
    case = Case(n_ant=40, n_gal=7, fmin=30.0, fmax=200.0, noise=900.0, flag_frac=0.02)
    sky = oracle_sky_model(orc, case)
    _, _, _, _, ref = oracle_data_processing(orc, case, case.data, sky)
    dev = _dev(case, sky, _lib.RLF_MIXED)
    pr = dev.process(case.cat, batch=batch, refit=False, rounds=rounds)
    dev.close()
    _check(pr.results, ref, 1e-4)


def test_board_wait_runs_out(orc):
    """The fit's wait for sampling-grid points claimed by other thread blocks is bounded: with a
    1 us limit (rlf_options.board_wait_us) the owners give up on points still in flight, count
    them as failed evaluations and set status bit 8, and the launch returns instead of waiting.
    The GPU stays usable: the next call with the default limit matches the oracle."""
    case = Case(n_gal=6, fmin=150.0, fmax=200.0, noise=300.0)
    sky = oracle_sky_model(orc, case)
    _, _, _, _, ref = oracle_data_processing(orc, case, case.data, sky)
    dev = _dev(case, sky, _lib.RLF_F64)
    dev.snapshot()
    hit = 0
    for _ in range(3):
        dev.restore()
        pr = dev.process(case.cat, batch=1, refit=False, board_wait_us=1)
        hit += int(np.count_nonzero(pr.results["status"] & 8))
        if hit:
            break
    assert hit > 0
    dev.restore()
    pr = dev.process(case.cat, batch=1, refit=False)
    dev.close()
    assert not np.any(pr.results["status"] & 8)
    _check(pr.results, ref, 1e-7)
