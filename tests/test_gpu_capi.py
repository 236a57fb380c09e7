"""Parity of the CUDA path, called through the reference-named C ABI, against the oracle.

Tolerances: the F64 path computes the reference's arithmetic in a different summation order
(parallel reductions, fused multiply-adds), so array results agree to ~1e-12 relative and the
fitted ellipticities to 1e-7; cell indices and counts are integer work and must be identical.
"""
import ctypes as C

import numpy as np
import pytest

from radiolensfit2_gb300 import _lib, constants as K
from radiolensfit2_gb300.abi import Complexd, LikelihoodParams, GslVector, dptr, fptr, cptr, bptr

import _oracle as O
from _cases import Case, oracle_sky_model, oracle_data_processing, oracle_facet, rprior_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


@pytest.fixture(scope="module")
def orc():
    return O.load_oracle()


@pytest.fixture(scope="module")
def case():
    return Case(flag_frac=0.03)


@pytest.fixture(scope="module")
def sky(orc, case):
    return oracle_sky_model(orc, case)


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_scalar_helpers(lib, orc):
    for th in (0.05, 0.3, 1.0, 3.5):
        for L in (1.0e3, 2.48e4, 1.0e5):
            assert lib.facet_size(th, L) == orc.orc_facet_size(th, L)
    for k1, k2, sf, wf in [(1e3, -2e3, 1e-11, 400.0), (0.0, 0.0, 1.0, 1.0), (5e4, 1e4, 3e-12, 420.0)]:
        assert lib.sersic_shape(k1, k2, sf, wf) == pytest.approx(orc.orc_sersic_shape(k1, k2, sf, wf), rel=1e-15)
        assert lib.gaussian_shape(k1, k2, sf, wf) == pytest.approx(orc.orc_gaussian_shape(k1, k2, sf, wf), rel=1e-15)
    for x in (1.0, 2.9955, 2.9956, 3.5, 10.0, 39.9, 40.1, 77.7, 100.0, 150.0):
        a = lib.marginalise_over_position_shift(x)
        b = orc.orc_marginalise_over_position_shift(x)
        assert a == pytest.approx(b, rel=1e-14, abs=1e-14)


def test_uv_grid_size_bit_exact(lib, orc, case):
    o = case.obs
    for F in (2, 4, 10, 34):
        a = lib.evaluate_uv_grid_size(0, 1, case.len, dptr(o.wavenumbers), o.n_ch, o.n_rows, dptr(o.uu),
                                      dptr(o.vv), F, bptr(case.flag))
        b = orc.orc_uv_grid_size(case.len, O.dp(o.wavenumbers), o.n_ch, o.n_rows, O.dp(o.uu), O.dp(o.vv), F,
                                 O.bp(case.flag))
        assert a == b


def test_gridding_and_facet_coords(lib, orc, case):
    o = case.obs
    vis = case.data.copy()
    for F in (4, 10):
        nc = F * F
        gv1, gs1, sw1 = np.zeros(nc, np.complex128), np.zeros(nc), np.zeros(nc)
        gv2, gs2, sw2 = np.zeros(nc, np.complex128), np.zeros(nc), np.zeros(nc)
        lib.gridding_visibilities(dptr(o.wavenumbers), o.n_ch, o.n_rows, dptr(o.uu), dptr(o.vv), cptr(vis),
                                  fptr(case.sigma2), case.len, F, cptr(gv1), dptr(gs1), bptr(case.flag), dptr(sw1))
        orc.orc_gridding(O.dp(o.wavenumbers), o.n_ch, o.n_rows, O.dp(o.uu), O.dp(o.vv), O.cp(vis), O.fp(case.sigma2),
                         case.len, F, O.cp(gv2), O.dp(gs2), O.bp(case.flag), O.dp(sw2))
        assert np.array_equal(sw1, sw2)  # counts: exact
        n = int(np.count_nonzero(sw2))
        assert rel(gv1[:n], gv2[:n]) < 1e-12
        assert rel(gs1[:n], gs2[:n]) < 1e-13
        u1, v1, u2, v2 = np.zeros(nc), np.zeros(nc), np.zeros(nc), np.zeros(nc)
        n1 = lib.evaluate_facet_coords(dptr(u1), dptr(v1), case.len, F, dptr(sw1))
        n2 = orc.orc_facet_coords(O.dp(u2), O.dp(v2), case.len, F, O.dp(sw2))
        assert n1 == n2 == n
        assert np.array_equal(u1[:n], u2[:n]) and np.array_equal(v1[:n], v2[:n])

def test_average_facets(lib, orc):
    """average_facets (evaluate_uv_grid.c:216-230): compaction of summed facets to the non-empty
    cells, visibilities times the weight over the variance, variances over the weight squared.
    Every cell's result is one product and one quotient of the same operands: bit-equal."""
    rng = np.random.default_rng(5)
    for F in (4, 10, 34):
        nc = F * F
        sw = rng.integers(0, 50, nc).astype(np.float64)
        sw[rng.random(nc) < 0.3] = 0.0
        sw[0] = 0.0
        sw[-1] = 7.0
        vis = (rng.standard_normal(nc) + 1j * rng.standard_normal(nc)) * 1e5
        s2 = rng.random(nc) * 1e9 + 1e6
        v1, s1 = vis.copy(), s2.copy()
        v2, s2o = vis.copy(), s2.copy()
        lib.average_facets(nc, cptr(v1), dptr(s1), dptr(sw))
        orc.orc_average_facets(nc, O.cp(v2), O.dp(s2o), O.dp(sw))
        n = int(np.count_nonzero(sw))
        assert np.array_equal(v1[:n], v2[:n])
        assert np.array_equal(s1[:n], s2o[:n])
        # cells beyond the compacted ones keep their inputs, as in the reference's in-place loop
        assert np.array_equal(v1[n:], v2[n:]) and np.array_equal(s1[n:], s2o[n:])
    # an all-empty facet leaves the arrays unchanged
    z = np.ones(16, np.complex128)
    zs = np.ones(16)
    lib.average_facets(16, cptr(z), dptr(zs), dptr(np.zeros(16)))
    assert np.all(z == 1) and np.all(zs == 1)


def test_model_and_visibility_kernels(lib, orc, case):
    o = case.obs
    gu = np.linspace(-2e4, 2e4, 37)
    gv = np.linspace(1e4, -1.5e4, 37)
    s2 = np.linspace(1.0, 2.0, 37)
    m1, m2 = np.zeros(37), np.zeros(37)
    lib.model_galaxy_visibilities_at_zero(0.2, -0.3, 0.8, 37, dptr(gu), dptr(gv), dptr(s2), dptr(m1))
    orc.orc_model_at_zero(0.2, -0.3, 0.8, 37, O.dp(gu), O.dp(gv), O.dp(s2), O.dp(m2), 0)
    assert rel(m1, m2) < 1e-13
    n = o.n_rows
    v1, v2 = np.zeros(n, np.complex128), np.zeros(n, np.complex128)
    lib.data_galaxy_visibilities(o.spec[1], o.wavenumbers[1], 0.0, 0.0, 0.3, 0.1, 0.7, 120.0, 1e-3, -2e-3, n,
                                 dptr(o.uu), dptr(o.vv), dptr(o.ww), cptr(v1))
    orc.orc_data_galaxy_vis(o.spec[1], o.wavenumbers[1], 0.3, 0.1, 0.7, 120.0, 1e-3, -2e-3, n, O.dp(o.uu),
                            O.dp(o.vv), O.dp(o.ww), O.cp(v2), 0)
    assert rel(v1, v2) < 1e-12
    lib.data_visibilities_phase_shift(o.wavenumbers[2], 1e-3, -2e-3, n, dptr(o.uu), dptr(o.vv), dptr(o.ww), cptr(v1))
    orc.orc_phase_shift(o.wavenumbers[2], 1e-3, -2e-3, n, O.dp(o.uu), O.dp(o.vv), O.dp(o.ww), O.cp(v2))
    assert rel(v1, v2) < 1e-12


def test_sky_model(lib, orc, case, sky):
    o, c = case.obs, case.cat
    s1 = np.zeros(o.n_vis, np.complex128)
    gal = np.zeros(o.n_vis, np.complex128)
    lib.sky_model(dptr(o.wavenumbers), dptr(o.spec), o.df_hz, int(o.dt_s), o.n_ch, c.n, dptr(c.flux),
                  dptr(c.scale), dptr(c.l), dptr(c.m), o.n_rows, dptr(o.uu), dptr(o.vv), dptr(o.ww), cptr(gal),
                  cptr(s1))
    assert rel(s1, sky) < 1e-12


def _params(case, gi, F, n, gu, gv, fvis, fs2):
    ro = case.ro
    pr = rprior_for(case.cat.flux[gi], ro)
    mod = np.zeros((case.numr - 1) * max(n, 1))
    keep = [ro, pr, gu, gv, fvis, fs2, mod]
    p = LikelihoodParams()
    p.numr = case.numr
    p.ro = dptr(ro)
    p.rprior = dptr(pr)
    p.nchannels = case.obs.n_ch
    p.spec = dptr(case.obs.spec)
    p.wavenumbers = dptr(case.obs.wavenumbers)
    p.uu = dptr(gu)
    p.vv = dptr(gv)
    p.data = cptr(fvis)
    p.sigma2 = dptr(fs2)
    p.mod = dptr(mod)
    p.facet = F
    p.ncoords = n
    op = O.OrcParams()
    op.numr = case.numr
    op.ro = O.dp(ro)
    op.rprior = O.dp(pr)
    op.ncoords = n
    op.uu = O.dp(gu)
    op.vv = O.dp(gv)
    op.data = O.cp(fvis)
    op.sigma2 = O.dp(fs2)
    # a struct field keeps only the address: the scratch array itself must stay referenced
    omod = np.zeros_like(mod)
    keep.append(omod)
    op.mod = O.dp(omod)
    return p, op, keep


def test_source_extraction(lib, orc, case, sky):
    o, c = case.obs, case.cat
    for gi in (0, 5):
        F, n, gu, gv, fvis, fs2, sumw = oracle_facet(orc, case, gi, case.data, sky)
        nc = F * F
        f1, s1, w1 = np.zeros(nc, np.complex128), np.zeros(nc), np.zeros(nc)
        p, _, keep = _params(case, gi, F, n, gu, gv, fvis, fs2)
        gal = np.zeros(o.n_vis, np.complex128)
        lib.source_extraction(0, F, C.byref(p), cptr(f1), dptr(s1), dptr(w1), c.l[gi], c.m[gi], c.flux[gi],
                              c.scale[gi], 0.0, 0.0, cptr(sky), cptr(case.data), cptr(gal), fptr(case.sigma2),
                              bptr(case.flag), o.n_rows, dptr(o.uu), dptr(o.vv), dptr(o.ww), case.len)
        assert np.array_equal(w1, sumw)
        assert rel(f1[:n], fvis) < 1e-11
        assert rel(s1[:n], fs2) < 1e-13


def test_likelihood_functions(lib, orc, case, sky):
    gi = 0
    F, n, gu, gv, fvis, fs2, _ = oracle_facet(orc, case, gi, case.data, sky)
    p, op, keep = _params(case, gi, F, n, gu, gv, fvis, fs2)
    # loglikelihood_r and cross_correlation
    for r in (0.3, 0.9, 2.1):
        m1, m2 = np.zeros(n), np.zeros(n)
        it = C.c_int(0)
        a = lib.loglikelihood_r(0.1, -0.2, r, n, dptr(fs2), dptr(gu), dptr(gv), cptr(fvis), dptr(m1))
        b = orc.orc_loglikelihood_r(0.1, -0.2, r, n, O.dp(fs2), O.dp(gu), O.dp(gv), O.cp(fvis), O.dp(m2), 0,
                                    C.byref(it))
        assert a == pytest.approx(b, rel=1e-10, abs=1e-9)
        assert rel(m1, m2) < 1e-13
        ho1, d1, ho2, d2 = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        e1 = lib.cross_correlation(n, dptr(gu), dptr(gv), cptr(fvis), dptr(m2), C.byref(ho1), C.byref(d1))
        e2 = orc.orc_cross_correlation(n, O.dp(gu), O.dp(gv), O.cp(fvis), O.dp(m2), C.byref(ho2), C.byref(d2), None)
        assert e1 == e2
        assert ho1.value == pytest.approx(ho2.value, rel=1e-11)
        assert d1.value == pytest.approx(d2.value, rel=1e-10)
    # loglikelihood and f_likelihood
    for e1, e2 in [(0.0, 0.0), (0.1, 0.05), (-0.3, 0.2), (0.5, 0.5)]:
        err1, err2 = C.c_int(0), C.c_int(0)
        a = lib.loglikelihood(C.c_void_p(C.addressof(p)), e1, e2, C.byref(err1))
        b = orc.orc_loglikelihood(C.byref(op), e1, e2, C.byref(err2))
        assert err1.value == err2.value
        assert a == pytest.approx(b, rel=1e-10, abs=1e-9)
        x = np.array([e1, e2])
        v = GslVector(2, 1, dptr(x), None, 0)
        assert lib.f_likelihood(C.byref(v), C.c_void_p(C.addressof(p))) == pytest.approx(-b, rel=1e-10, abs=1e-9)


def test_marginalise_posterior(lib, orc):
    rng = np.random.default_rng(5)
    ro = np.array(K.ro_grid())
    for trial in range(6):
        n = 23 - trial * 3
        x = ro[1:n + 1].copy()
        y = -0.5 * ((np.log(x) - np.log(0.8 + 0.3 * trial)) / 0.4) ** 2 * (5 + 40 * trial) + rng.normal(0, 0.1, n)
        y1, y2 = y.copy(), y.copy()
        a = lib.rlf_marginalise_posterior_r(n, dptr(x), dptr(y1))
        b = orc.orc_marginalise_posterior_r(n, O.dp(x), O.dp(y2))
        assert a == pytest.approx(b, rel=1e-12, abs=1e-12)
        assert np.allclose(y1, y2, rtol=0, atol=1e-13)
    Lr = np.array([0.0, -1e10, 3.0, 4.0, -1e10, 6.0, 7.0, 8.0])
    pr = np.linspace(0, -1, 8)
    rr = np.linspace(0, 2, 8)
    x1, y1, x2, y2 = np.zeros(8), np.zeros(8), np.zeros(8), np.zeros(8)
    n1, n2 = C.c_int(), C.c_int()
    lib.rlf_set_posterior_values(8, dptr(Lr), dptr(pr), dptr(rr), dptr(x1), dptr(y1), C.byref(n1))
    orc.orc_set_posterior_values(8, O.dp(Lr), O.dp(pr), O.dp(rr), O.dp(x2), O.dp(y2), C.byref(n2))
    assert n1.value == n2.value == 5
    assert np.array_equal(x1[:5], x2[:5]) and np.array_equal(y1[:5], y2[:5])


def test_source_fitting_and_sampling(lib, orc, case, sky):
    for gi in (0, 3):
        F, n, gu, gv, fvis, fs2, _ = oracle_facet(orc, case, gi, case.data, sky)
        p, op, keep = _params(case, gi, F, n, gu, gv, fvis, fs2)
        out = [C.c_double() for _ in range(6)]
        err = lib.source_fitting(0, C.byref(p), *[C.byref(x) for x in out])
        r = O.OrcFitResult()
        err2 = orc.orc_source_fitting(C.byref(op), 0.0, 0.0, 0.1, C.byref(r))
        assert err == err2
        got = [x.value for x in out]
        want = [r.e1, r.e2, r.var_e1, r.var_e2, r.oneDimvar, r.maxL]
        assert got[0] == pytest.approx(want[0], abs=1e-7)
        assert got[1] == pytest.approx(want[1], abs=1e-7)
        assert got[5] == pytest.approx(want[5], rel=1e-9)
        for k in (2, 3, 4):
            assert got[k] == pytest.approx(want[k], rel=1e-6)
        # likelihood_sampling alone from the oracle's maximum
        m1 = [C.c_double(0.05), C.c_double(-0.02)]
        m2 = [C.c_double(0.05), C.c_double(-0.02)]
        v1 = [C.c_double() for _ in range(3)]
        v2 = [C.c_double() for _ in range(3)]
        maxL = orc.orc_loglikelihood(C.byref(op), 0.05, -0.02, C.byref(C.c_int()))
        lib.likelihood_sampling(C.byref(m1[0]), C.byref(m1[1]), maxL, C.c_void_p(C.addressof(p)), 30,
                                *[C.byref(x) for x in v1])
        orc.orc_likelihood_sampling(C.byref(m2[0]), C.byref(m2[1]), maxL, C.byref(op), 30, *[C.byref(x) for x in v2])
        assert m1[0].value == pytest.approx(m2[0].value, abs=1e-9)
        assert m1[1].value == pytest.approx(m2[1].value, abs=1e-9)
        for a, b in zip(v1, v2):
            assert a.value == pytest.approx(b.value, rel=1e-7)


def test_data_processing_f64(lib, orc, case, sky):
    """Both passes of the reference loop (RadioLensfit2.cpp:597-606) through the drop-in."""
    o, c = case.obs, case.cat
    d_ref, s_ref, bad_ref, bl_ref, res_ref = oracle_data_processing(orc, case, case.data, sky)
    opt = _lib.Options()
    opt.precision, opt.batch, opt.refit = _lib.RLF_F64, 1, 1
    lib.rlf_configure(C.byref(opt))
    data = case.data.copy()
    skym = sky.copy()
    fmax = K.facet_size(K.RMAX, case.len)
    p = LikelihoodParams()
    ro = case.ro.copy()
    pr = np.zeros(case.numr)
    p.numr, p.ro, p.rprior, p.nchannels = case.numr, dptr(ro), dptr(pr), o.n_ch
    p.spec, p.wavenumbers = dptr(o.spec), dptr(o.wavenumbers)
    bad_list = np.zeros(c.n, np.uint32)
    bad = C.c_int(0)
    ft = C.c_double(0)
    snr = np.zeros(c.n)
    sumw = np.zeros(fmax * fmax)
    gal = np.zeros(o.n_vis, np.complex128)
    lib.data_processing(False, bad_list.ctypes.data_as(_lib.PU), c.n, case.len, o.n_rows, None, C.byref(p),
                        dptr(c.l), dptr(c.m), dptr(c.flux), dptr(c.scale), dptr(c.e1), dptr(c.e2), dptr(snr),
                        dptr(sumw), cptr(gal), cptr(skym), cptr(data), fptr(case.sigma2), bptr(case.flag),
                        dptr(o.uu), dptr(o.vv), dptr(o.ww), C.byref(ft), C.byref(bad))
    assert bad.value == bad_ref
    assert np.array_equal(bad_list[:bad_ref], bl_ref[:bad_ref])
    assert rel(data, d_ref) < 1e-11
    # every galaxy's round model has been subtracted: both sky models are left at rounding level,
    # so the difference is measured against the scale of the sky model before the loop
    assert np.max(np.abs(skym - s_ref)) < 1e-11 * np.max(np.abs(sky))


def test_device_pipeline_f64_matches_oracle(orc, case, sky):
    from radiolensfit2_gb300.pipeline import DeviceObservation
    d_ref, s_ref, bad_ref, bl_ref, res_ref = oracle_data_processing(orc, case, case.data, sky)
    dev = DeviceObservation(case.obs, precision=_lib.RLF_F64, sigma2=case.sigma2, flag=case.flag)
    dev.set_vis(case.data, sky)
    pr = dev.process(case.cat, batch=1, refit=False)
    for gi, r in enumerate(res_ref):
        assert pr.results["error"][gi] == r[6]
        assert pr.results["e1"][gi] == pytest.approx(r[0], abs=1e-7)
        assert pr.results["e2"][gi] == pytest.approx(r[1], abs=1e-7)
        assert pr.results["maxL"][gi] == pytest.approx(r[5], rel=1e-9, abs=1e-9)
        assert pr.results["nevals"][gi] == r[7]
    d, s = dev.get_vis()
    assert rel(d, d_ref) < 1e-11
    assert np.max(np.abs(s - s_ref)) < 1e-11 * np.max(np.abs(sky))


def _data_processing(lib, case, data, skym, uu, vv, ww, sigma2, flag):
    """one catalogue pass of the drop-in data_processing on the given host arrays"""
    o, c = case.obs, case.cat
    fmax = K.facet_size(K.RMAX, case.len)
    p = LikelihoodParams()
    ro = case.ro.copy()
    pr = np.zeros(case.numr)
    p.numr, p.ro, p.rprior, p.nchannels = case.numr, dptr(ro), dptr(pr), o.n_ch
    p.spec, p.wavenumbers = dptr(o.spec), dptr(o.wavenumbers)
    bad_list = np.zeros(c.n, np.uint32)
    bad = C.c_int(0)
    ft = C.c_double(0)
    snr = np.zeros(c.n)
    sumw = np.zeros(fmax * fmax)
    gal = np.zeros(1, np.complex128)
    lib.data_processing(False, bad_list.ctypes.data_as(_lib.PU), c.n, case.len, o.n_rows, None, C.byref(p),
                        dptr(c.l), dptr(c.m), dptr(c.flux), dptr(c.scale), dptr(c.e1), dptr(c.e2), dptr(snr),
                        dptr(sumw), cptr(gal), cptr(skym), cptr(data), fptr(sigma2), bptr(flag),
                        dptr(uu), dptr(vv), dptr(ww), C.byref(ft), C.byref(bad))
    return bad.value, bad_list


def test_data_processing_keeps_observation(lib, orc):
    """data_processing keeps the observation (device uvw, variances, flags, facet tables) between
    calls that pass the same arrays, uploading only visibilities and sky model, and rebuilds it
    when the contents at the same addresses change (here: uvw scaled, other variances and flags)."""
    A = Case(flag_frac=0.03, n_gal=6)
    B = Case(seed=5, flag_frac=0.05, noise=700.0, n_gal=6)
    opt = _lib.Options()
    opt.precision, opt.batch, opt.refit, opt.reuse_obs = _lib.RLF_F64, 1, 1, 1
    lib.rlf_configure(C.byref(opt))
    lib.rlf_release()
    uu, vv, ww = A.obs.uu.copy(), A.obs.vv.copy(), A.obs.ww.copy()
    sigma2, flag = A.sigma2.copy(), A.flag.copy()
    sky_a = oracle_sky_model(orc, A)
    d_ref, s_ref, bad_ref, bl_ref, _ = oracle_data_processing(orc, A, A.data, sky_a)
    h0, o0 = C.c_ulonglong(0), C.c_ulonglong(0)
    h1, o1 = C.c_ulonglong(0), C.c_ulonglong(0)
    moved = []
    for _ in range(2):
        data, skym = A.data.copy(), sky_a.copy()
        lib.rlf_transfer_bytes(C.byref(h0), C.byref(o0))
        bad, bl = _data_processing(lib, A, data, skym, uu, vv, ww, sigma2, flag)
        lib.rlf_transfer_bytes(C.byref(h1), C.byref(o1))
        moved.append(h1.value - h0.value)
        assert bad == bad_ref and np.array_equal(bl[:bad], bl_ref[:bad])
        assert rel(data, d_ref) < 1e-11
        assert np.max(np.abs(skym - s_ref)) < 1e-11 * np.max(np.abs(sky_a))
    vis_bytes = 2 * 16 * A.obs.n_vis
    # the second call moved the visibilities and sky model and the per-call galaxy tables only
    assert moved[1] < moved[0]
    assert vis_bytes <= moved[1] < vis_bytes + (1 << 20)
    # another observation in the same host buffers
    np.copyto(uu, A.obs.uu * 1.001)
    np.copyto(vv, A.obs.vv * 1.001)
    np.copyto(ww, A.obs.ww * 1.001)
    np.copyto(sigma2, B.sigma2)
    np.copyto(flag, B.flag)
    B.obs.uu, B.obs.vv, B.obs.ww = uu.copy(), vv.copy(), ww.copy()
    B.flag = flag.copy()
    sky_b = oracle_sky_model(orc, B)
    d_ref, s_ref, bad_ref, bl_ref, _ = oracle_data_processing(orc, B, B.data, sky_b)
    data, skym = B.data.copy(), sky_b.copy()
    bad, bl = _data_processing(lib, B, data, skym, uu, vv, ww, sigma2, flag)
    assert bad == bad_ref and np.array_equal(bl[:bad], bl_ref[:bad])
    assert rel(data, d_ref) < 1e-11
    assert np.max(np.abs(skym - s_ref)) < 1e-11 * np.max(np.abs(sky_b))
    lib.rlf_release()


def test_data_processing_reads_arrays_every_call(lib, orc):
    """Default mode (reuse_obs = 0): a flag changed in place between two calls, at a position the
    kept observation's sampled fingerprint does not look at, is seen by the second call, which
    gives the oracle's result with the new flags (the reference reads its arrays on every call,
    data_processing.c:82-84)."""
    A = Case(flag_frac=0.03, n_gal=6)
    opt = _lib.Options()
    opt.precision, opt.batch, opt.refit, opt.reuse_obs = _lib.RLF_F64, 1, 1, 0
    lib.rlf_configure(C.byref(opt))
    lib.rlf_release()
    sky_a = oracle_sky_model(orc, A)
    flag = A.flag.copy()
    nv = A.obs.n_vis
    sampled = {(nv - 1) * i // 4096 for i in range(4097)}
    # unsampled, unflagged visibilities of the first channel: flag a run of them
    idx = [i for i in range(A.obs.n_rows) if i not in sampled and not flag[i]][:40]
    assert len(idx) == 40
    data, skym = A.data.copy(), sky_a.copy()
    _data_processing(lib, A, data, skym, A.obs.uu, A.obs.vv, A.obs.ww, A.sigma2, flag)
    flag[idx] = 1
    A.flag = flag.copy()
    d_ref, s_ref, bad_ref, bl_ref, _ = oracle_data_processing(orc, A, A.data, sky_a)
    data, skym = A.data.copy(), sky_a.copy()
    bad, bl = _data_processing(lib, A, data, skym, A.obs.uu, A.obs.vv, A.obs.ww, A.sigma2, flag)
    assert bad == bad_ref and np.array_equal(bl[:bad], bl_ref[:bad])
    assert rel(data, d_ref) < 1e-11
    assert np.max(np.abs(skym - s_ref)) < 1e-11 * np.max(np.abs(sky_a))
    lib.rlf_release()


def test_data_processing_pinned_buffers(lib, orc):
    """Page-locked host buffers (converted by kernels reading and writing them directly) give the
    same data, sky model and bad list as pageable ones (staged copies)."""
    torch = pytest.importorskip("torch")
    A = Case(flag_frac=0.03, n_gal=6)
    opt = _lib.Options()
    opt.precision, opt.batch, opt.refit, opt.reuse_obs = _lib.RLF_MIXED, 6, 1, 1
    lib.rlf_configure(C.byref(opt))
    lib.rlf_release()
    sky_a = oracle_sky_model(orc, A)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    out = []
    for make in (np.copy, np.copy, pin):
        data, skym = make(A.data), make(sky_a)
        bad, bl = _data_processing(lib, A, data, skym, A.obs.uu, A.obs.vv, A.obs.ww, A.sigma2, A.flag)
        out.append((bad, bl[:bad].copy(), np.array(data), np.array(skym)))
    lib.rlf_release()
    rep = np.max(np.abs(out[0][2] - out[1][2])) / np.max(np.abs(out[0][2]))
    pinned = np.max(np.abs(out[0][2] - out[2][2])) / np.max(np.abs(out[0][2]))
    print(f"pageable twice: {rep:.2e}; pinned vs pageable: {pinned:.2e}")
    assert out[0][0] == out[2][0] and np.array_equal(out[0][1], out[2][1])
    assert pinned < 1e-6 and np.max(np.abs(out[0][3] - out[2][3])) < 1e-6 * np.max(np.abs(sky_a))
