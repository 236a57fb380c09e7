"""Seeded small cases shared by the oracle, golden and GPU tests (test infrastructure)."""
import ctypes as C

import numpy as np

from radiolensfit2_gb300 import constants as K
from radiolensfit2_gb300 import synth

import _oracle as O


class Case:
    """A small observation with its catalogue, data, variances and flags (host arrays)."""

    def __init__(self, n_ant=24, ha_hours=2.0, dt_s=600.0, n_ch=4, n_gal=8, fmin=50.0, fmax=200.0,
                 noise=600.0, g=(0.03, -0.02), seed=2, flag_frac=0.0, scale_mult=1.0, gaussian=False,
                 scale_override=None):
        self.obs = synth.make_observation(n_ant=n_ant, ha_hours=ha_hours, dt_s=dt_s, n_ch=n_ch)
        self.cat = synth.make_catalogue(n_gal, fmin, fmax, g=g, seed=seed)
        self.cat.scale = np.clip(self.cat.scale * scale_mult, 0.05, K.RMAX)
        for gi, sc in (scale_override or {}).items():
            self.cat.scale[gi] = sc
        self.gaussian = int(bool(gaussian))
        self.noise = noise
        self.data = synth.simulate_visibilities_np(self.obs, self.cat, noise_sigma=noise, seed=seed + 1,
                                                   gaussian=bool(gaussian)).astype(np.complex128)
        self.sigma2 = np.full(self.obs.n_vis, np.float32(noise * noise), dtype=np.float32)
        rng = np.random.default_rng(seed + 7)
        self.flag = (rng.random(self.obs.n_vis) < flag_frac).astype(np.uint8)
        self.ro = np.array(K.ro_grid())
        self.numr = len(self.ro)

    @property
    def len(self):
        return self.obs.len_lambda


def oracle_sky_model(orc, case):
    o, c = case.obs, case.cat
    sky = np.zeros(o.n_vis, np.complex128)
    gal = np.zeros(o.n_vis, np.complex128)
    orc.orc_sky_model(O.dp(o.wavenumbers), O.dp(o.spec), o.n_ch, c.n, O.dp(c.flux), O.dp(c.scale),
                      O.dp(c.l), O.dp(c.m), o.n_rows, O.dp(o.uu), O.dp(o.vv), O.dp(o.ww), O.cp(gal),
                      O.cp(sky), case.gaussian)
    return sky


def oracle_data_processing(orc, case, data, sky, re_fitting=False, bad_list=None):
    o, c = case.obs, case.cat
    data = data.copy()
    sky = sky.copy()
    gal = np.zeros(o.n_vis, np.complex128)
    fmax = K.facet_size(K.RMAX, case.len)
    sumw = np.zeros(fmax * fmax)
    out = (O.OrcFitResult * c.n)()
    if bad_list is None:
        bad_list = np.zeros(c.n, np.uint32)
    else:
        bad_list = np.ascontiguousarray(bad_list, dtype=np.uint32).copy()
    nsrc = c.n if not re_fitting else len(bad_list)
    bad = C.c_int(0)
    orc.orc_data_processing(1 if re_fitting else 0, bad_list.ctypes.data_as(O.PU), nsrc, case.len,
                            o.n_rows, o.n_ch, O.dp(o.spec), O.dp(o.wavenumbers), case.numr,
                            O.dp(case.ro), O.dp(c.l), O.dp(c.m), O.dp(c.flux), O.dp(c.scale),
                            O.dp(sumw), O.cp(gal), O.cp(sky), O.cp(data), O.fp(case.sigma2),
                            O.bp(case.flag), O.dp(o.uu), O.dp(o.vv), O.dp(o.ww), case.gaussian, out,
                            C.byref(bad))
    res = [(r.e1, r.e2, r.var_e1, r.var_e2, r.oneDimvar, r.maxL, r.error, r.nevals, r.max_e1, r.max_e2)
           for r in out]
    return data, sky, bad.value, bad_list, res


def oracle_facet(orc, case, gi, data, sky):
    """source_extraction + evaluate_facet_coords of galaxy gi (oracle)."""
    o, c = case.obs, case.cat
    F = K.facet_size(c.scale[gi], case.len)
    nc = F * F
    fvis = np.zeros(nc, np.complex128)
    fs2 = np.zeros(nc)
    sumw = np.zeros(nc)
    gal = np.zeros(o.n_vis, np.complex128)
    orc.orc_source_extraction(o.n_ch, O.dp(o.spec), O.dp(o.wavenumbers), F, O.cp(fvis), O.dp(fs2),
                              O.dp(sumw), c.l[gi], c.m[gi], c.flux[gi], c.scale[gi], 0.0, 0.0,
                              O.cp(sky), O.cp(data), O.cp(gal), O.fp(case.sigma2), O.bp(case.flag),
                              o.n_rows, O.dp(o.uu), O.dp(o.vv), O.dp(o.ww), case.len, case.gaussian)
    gu = np.zeros(nc)
    gv = np.zeros(nc)
    n = orc.orc_facet_coords(O.dp(gu), O.dp(gv), case.len, F, O.dp(sumw))
    return F, n, gu[:n].copy(), gv[:n].copy(), fvis[:n].copy(), fs2[:n].copy(), sumw


def rprior_for(flux, ro):
    mu = K.scale_mean(flux)
    pr = np.zeros(len(ro))
    for r in range(1, len(ro)):
        pr[r] = K.rfunc(mu, K.R_STD, ro[r])
    return pr
