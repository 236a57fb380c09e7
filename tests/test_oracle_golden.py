"""The oracle (CPU restatement, oracle/rlf_oracle.c) against the golden vectors produced by the
reference's own code (tests/golden/golden_small.npz).  This pins the oracle; the GPU tests then
use the oracle and the same vectors as their checker."""
import ctypes as C

import numpy as np
import pytest

from radiolensfit2_gb300 import constants as K

import _oracle as O
from _golden import Golden, SUB, rows_from_results


@pytest.fixture(scope="module")
def g():
    return Golden()


@pytest.fixture(scope="module")
def orc():
    return O.load_oracle()


def _sky(orc, g):
    o, c = g.obs, g.cat
    sky = np.zeros(o.n_vis, np.complex128)
    gal = np.zeros(o.n_vis, np.complex128)
    orc.orc_sky_model(O.dp(o.wavenumbers), O.dp(o.spec), o.n_ch, c.n, O.dp(c.flux), O.dp(c.scale), O.dp(c.l),
                      O.dp(c.m), o.n_rows, O.dp(o.uu), O.dp(o.vv), O.dp(o.ww), O.cp(gal), O.cp(sky), 0)
    return sky


def test_sky_model_and_grid_size(orc, g):
    sky = _sky(orc, g)
    assert np.array_equal(sky[::SUB], g["sky_sub"])  # same arithmetic, same order: bit-exact
    o = g.obs
    F = orc.orc_facet_size(K.RMAX, g.len)
    assert F == int(g["facet_rmax"])
    n = orc.orc_uv_grid_size(g.len, O.dp(o.wavenumbers), o.n_ch, o.n_rows, O.dp(o.uu), O.dp(o.vv), F, O.bp(g.flag))
    assert n == int(g["uv_grid_size_rmax"])


def _facet(orc, g, gi, sky):
    o, c = g.obs, g.cat
    F = int(g[f"g{gi}_facet"])
    assert F == orc.orc_facet_size(c.scale[gi], g.len)
    nc = F * F
    fvis, fs2, sumw = np.zeros(nc, np.complex128), np.zeros(nc), np.zeros(nc)
    gal = np.zeros(o.n_vis, np.complex128)
    orc.orc_source_extraction(o.n_ch, O.dp(o.spec), O.dp(o.wavenumbers), F, O.cp(fvis), O.dp(fs2), O.dp(sumw),
                              c.l[gi], c.m[gi], c.flux[gi], c.scale[gi], 0.0, 0.0, O.cp(sky), O.cp(g.data),
                              O.cp(gal), O.fp(g.sigma2), O.bp(g.flag), o.n_rows, O.dp(o.uu), O.dp(o.vv), O.dp(o.ww),
                              g.len, 0)
    gu, gv = np.zeros(nc), np.zeros(nc)
    n = orc.orc_facet_coords(O.dp(gu), O.dp(gv), g.len, F, O.dp(sumw))
    return F, n, sumw, gu[:n].copy(), gv[:n].copy(), fvis[:n].copy(), fs2[:n].copy()


def test_facets_likelihoods_fits(orc, g):
    sky = _sky(orc, g)
    fits = g["fit_independent"]
    for gi in range(g.cat.n):
        F, n, sumw, gu, gv, fvis, fs2 = _facet(orc, g, gi, sky)
        assert np.array_equal(sumw, g[f"g{gi}_sumw"])
        assert np.array_equal(gu, g[f"g{gi}_gu"]) and np.array_equal(gv, g[f"g{gi}_gv"])
        assert np.array_equal(fvis, g[f"g{gi}_vis"])
        assert np.array_equal(fs2, g[f"g{gi}_sigma2"])
        p = O.OrcParams()
        pr = np.ascontiguousarray(g[f"g{gi}_rprior"])
        ro = np.ascontiguousarray(g.ro)
        mod = np.zeros((g.numr - 1) * n)
        p.numr, p.ro, p.rprior, p.ncoords = g.numr, O.dp(ro), O.dp(pr), n
        p.uu, p.vv, p.data, p.sigma2, p.mod = O.dp(gu), O.dp(gv), O.cp(fvis), O.dp(fs2), O.dp(mod)
        nodes = np.zeros(g.numr)
        m1 = np.zeros(n)
        for r in range(1, g.numr):
            nodes[r] = orc.orc_loglikelihood_r(0.1, -0.05, ro[r], n, O.dp(fs2), O.dp(gu), O.dp(gv), O.cp(fvis),
                                               O.dp(m1), 0, None)
        assert np.array_equal(nodes, g[f"g{gi}_Lr"])
        for k, (a, b) in enumerate(g[f"g{gi}_Le_points"]):
            err = C.c_int(0)
            L = orc.orc_loglikelihood(C.byref(p), a, b, C.byref(err))
            assert err.value == g[f"g{gi}_Le_err"][k]
            assert L == g[f"g{gi}_Le"][k]
        r = O.OrcFitResult()
        e = orc.orc_source_fitting(C.byref(p), 0.0, 0.0, 0.1, C.byref(r))
        want = fits[gi]
        assert e == int(want[6])
        np.testing.assert_array_equal([r.e1, r.e2, r.var_e1, r.var_e2, r.oneDimvar, r.maxL], want[:6])


def test_data_processing_two_passes(orc, g):
    """Sequential extraction -> fit -> removal (data_processing.c:61-138), then the re-fit pass."""
    o, c = g.obs, g.cat
    sky = _sky(orc, g)
    data = g.data.copy()
    sumw = np.zeros(int(g["facet_rmax"]) ** 2)
    gal = np.zeros(o.n_vis, np.complex128)
    ro = np.ascontiguousarray(g.ro)
    out1 = (O.OrcFitResult * c.n)()
    bad_list = np.zeros(c.n, np.uint32)
    bad = C.c_int(0)
    common = [g.len, o.n_rows, o.n_ch, O.dp(o.spec), O.dp(o.wavenumbers), g.numr, O.dp(ro), O.dp(c.l),
              O.dp(c.m), O.dp(c.flux), O.dp(c.scale), O.dp(sumw), O.cp(gal), O.cp(sky), O.cp(data),
              O.fp(g.sigma2), O.bp(g.flag), O.dp(o.uu), O.dp(o.vv), O.dp(o.ww), 0]
    orc.orc_data_processing(0, bad_list.ctypes.data_as(O.PU), c.n, *common, out1, C.byref(bad))
    nbad = bad.value
    assert np.array_equal(bad_list[:nbad], g["dp_bad_list"])
    assert np.array_equal(data[::SUB], g["dp_data1_sub"])
    assert np.array_equal(sky[::SUB], g["dp_sky1_sub"])
    good1 = [i for i in range(c.n) if not out1[i].error]
    res = {i: (out1[i].e1, out1[i].e2, out1[i].var_e1, out1[i].var_e2, out1[i].oneDimvar) for i in good1}
    out2 = (O.OrcFitResult * c.n)()
    orc.orc_data_processing(1, bad_list.ctypes.data_as(O.PU), nbad, *common, out2, C.byref(bad))
    assert bad.value == int(g["dp_nbad_final"])
    assert np.array_equal(data[::SUB], g["dp_data2_sub"])
    assert np.array_equal(sky[::SUB], g["dp_sky2_sub"])
    for i in bad_list[:nbad]:
        r = out2[i]
        res[int(i)] = (r.e1, r.e2, r.var_e1, r.var_e2, r.oneDimvar)
    rows = rows_from_results(g, good1 + [int(i) for i in bad_list[:nbad]], res)
    assert rows == list(g["dp_rows"])
