"""Generate the golden fixtures in this directory from the reference's own code.

Runs oracle/_ref/librlf_ref.so (the reference's hot-path sources compiled against the project's
GSL-subset shim by `make -C oracle ref REF=<reference checkout>`) on seeded small cases and
stores inputs and outputs:

  golden_small.npz   one small observation (16 antennas, 24 times, 4 channels, 7 galaxies, one too faint
                     to measure):
                     uvw, data, variances, flags, catalogue; the reference's sky model (every 7th
                     visibility), per-galaxy facets, node likelihoods L_r, loglikelihood at fixed
                     ellipticities, source_fitting results on independent facets, and the
                     sequential data_processing pass (per-galaxy results in full precision,
                     residual visibilities every 7th value, the output table rows).

Usage:  python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from radiolensfit2_gb300 import constants as K, synth  # noqa: E402
from radiolensfit2_gb300.abi import Complexd, LikelihoodParams, GslVector  # noqa: E402
import _oracle as O  # noqa: E402

SUB = 7  # stride of the stored visibility subsets


def cptr(a):
    return a.ctypes.data_as(C.POINTER(Complexd))


def make_case():
    obs = synth.make_observation(n_ant=16, ha_hours=2.0, dt_s=600.0, n_ch=4)
    cat = synth.make_catalogue(7, 60.0, 200.0, g=(0.03, -0.02), seed=12)
    cat.flux[-1] = 6.0  # a faint source that the fit rejects, so the re-fit pass runs
    noise = 250.0
    data = synth.simulate_visibilities_np(obs, cat, noise_sigma=noise, seed=13)  # complex64
    rng = np.random.default_rng(14)
    flag = (rng.random(obs.n_vis) < 0.02).astype(np.uint8)
    sigma2 = np.full(obs.n_vis, np.float32(noise * noise), dtype=np.float32)
    return obs, cat, data, sigma2, flag


def main():
    if not O.have_ref():
        raise SystemExit("oracle/_ref/librlf_ref.so missing: run make -C oracle ref")
    ref = O.load_ref()
    obs, cat, data64, sigma2, flag = make_case()
    data = data64.astype(np.complex128)
    ro = np.array(K.ro_grid())
    numr = len(ro)
    L = obs.len_lambda
    out = dict(uu=obs.uu, vv=obs.vv, ww=obs.ww, wavenumbers=obs.wavenumbers, spec=obs.spec,
               len_lambda=np.float64(L), n_rows=np.int64(obs.n_rows), n_ch=np.int64(obs.n_ch),
               data=data64, sigma2=sigma2, flag=flag, flux=cat.flux, scale=cat.scale, e1=cat.e1,
               e2=cat.e2, l=cat.l, m=cat.m, ro=ro)
    # sky model (data_simulation.c:131-165)
    sky = np.zeros(obs.n_vis, np.complex128)
    gal = np.zeros(obs.n_vis, np.complex128)
    ref.sky_model(O.dp(obs.wavenumbers), O.dp(obs.spec), obs.df_hz, int(obs.dt_s), obs.n_ch, cat.n,
                  O.dp(cat.flux), O.dp(cat.scale), O.dp(cat.l), O.dp(cat.m), obs.n_rows, O.dp(obs.uu),
                  O.dp(obs.vv), O.dp(obs.ww), cptr(gal), cptr(sky))
    out["sky_sub"] = sky[::SUB].copy()
    fmax = ref.facet_size(K.RMAX, L)
    out["facet_rmax"] = np.int64(fmax)
    out["uv_grid_size_rmax"] = np.int64(ref.evaluate_uv_grid_size(
        0, 1, L, O.dp(obs.wavenumbers), obs.n_ch, obs.n_rows, O.dp(obs.uu), O.dp(obs.vv), fmax, O.bp(flag)))
    # independent facets of every galaxy against the full sky model, and their fits
    fits = []
    for gi in range(cat.n):
        F = ref.facet_size(cat.scale[gi], L)
        nc = F * F
        fvis = np.zeros(nc, np.complex128)
        fs2 = np.zeros(nc)
        sumw = np.zeros(nc)
        par = LikelihoodParams()
        rprior = np.zeros(numr)
        mu = ref.scale_mean(cat.flux[gi])
        for r in range(1, numr):
            rprior[r] = ref.rfunc(mu, K.R_STD, ro[r])
        par.numr = numr
        par.ro = O.dp(ro)
        par.rprior = O.dp(rprior)
        par.nchannels = obs.n_ch
        par.spec = O.dp(obs.spec)
        par.wavenumbers = O.dp(obs.wavenumbers)
        g2 = np.zeros(obs.n_vis, np.complex128)
        ref.source_extraction(0, F, C.byref(par), cptr(fvis), O.dp(fs2), O.dp(sumw), cat.l[gi], cat.m[gi],
                              cat.flux[gi], cat.scale[gi], 0.0, 0.0, cptr(sky), cptr(data), cptr(g2),
                              O.fp(sigma2), O.bp(flag), obs.n_rows, O.dp(obs.uu), O.dp(obs.vv), O.dp(obs.ww), L)
        gu = np.zeros(nc)
        gv = np.zeros(nc)
        n = ref.evaluate_facet_coords(O.dp(gu), O.dp(gv), L, F, O.dp(sumw))
        out[f"g{gi}_facet"] = np.int64(F)
        out[f"g{gi}_sumw"] = sumw
        out[f"g{gi}_gu"] = gu[:n].copy()
        out[f"g{gi}_gv"] = gv[:n].copy()
        out[f"g{gi}_vis"] = fvis[:n].copy()
        out[f"g{gi}_sigma2"] = fs2[:n].copy()
        out[f"g{gi}_rprior"] = rprior
        gu, gv, fvis, fs2 = gu[:n].copy(), gv[:n].copy(), fvis[:n].copy(), fs2[:n].copy()
        mod = np.zeros((numr - 1) * n)
        par.uu, par.vv, par.data, par.sigma2, par.mod = O.dp(gu), O.dp(gv), cptr(fvis), O.dp(fs2), O.dp(mod)
        par.facet, par.ncoords = F, n
        # node likelihoods at e = (0.1, -0.05)
        Lr = np.zeros(numr)
        m1 = np.zeros(n)
        for r in range(1, numr):
            Lr[r] = ref.loglikelihood_r(0.1, -0.05, ro[r], n, O.dp(fs2), O.dp(gu), O.dp(gv), cptr(fvis), O.dp(m1))
        out[f"g{gi}_Lr"] = Lr
        pts = np.array([[0.0, 0.0], [0.1, -0.05], [-0.2, 0.3], [0.4, 0.1]])
        Le = np.zeros(len(pts))
        errs = np.zeros(len(pts), np.int64)
        for k, (a, b) in enumerate(pts):
            e = C.c_int(0)
            Le[k] = ref.loglikelihood(C.cast(C.byref(par), C.c_void_p), a, b, C.byref(e))
            errs[k] = e.value
        out[f"g{gi}_Le_points"] = pts
        out[f"g{gi}_Le"] = Le
        out[f"g{gi}_Le_err"] = errs
        res = [C.c_double() for _ in range(6)]
        err = ref.source_fitting(0, C.byref(par), *[C.byref(x) for x in res])
        fits.append([x.value for x in res] + [err])
    out["fit_independent"] = np.array(fits)  # e1, e2, var1, var2, 1Dvar, maxL, error
    # data_processing (data_processing.c:47-147), both passes, through the reference itself
    d = data.copy()
    s = sky.copy()
    nc = fmax * fmax
    nfc = int(out["uv_grid_size_rmax"])
    fvis = np.zeros(nc, np.complex128)
    fs2 = np.zeros(nc)
    fu = np.zeros(nfc)
    fv = np.zeros(nfc)
    mod = np.zeros((numr - 1) * nfc)
    rprior = np.zeros(numr)
    sumw = np.zeros(nc)
    par = LikelihoodParams()
    par.numr, par.ro, par.rprior, par.nchannels = numr, O.dp(ro), O.dp(rprior), obs.n_ch
    par.band_factor, par.acc_time = obs.df_hz * K.PI / K.C0, obs.dt_s
    par.spec, par.wavenumbers = O.dp(obs.spec), O.dp(obs.wavenumbers)
    par.uu, par.vv, par.data, par.sigma2, par.mod = O.dp(fu), O.dp(fv), cptr(fvis), O.dp(fs2), O.dp(mod)
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    tmp = tempfile.NamedTemporaryFile(delete=False, suffix=".txt")
    tmp.close()
    fp = libc.fopen(tmp.name.encode(), b"w")
    bad_list = np.zeros(cat.n, np.uint32)
    bad = C.c_int(0)
    ft = C.c_double(0)
    snr = np.zeros(cat.n)
    g2 = np.zeros(obs.n_vis, np.complex128)
    args = [C.byref(par), O.dp(cat.l), O.dp(cat.m), O.dp(cat.flux), O.dp(cat.scale), O.dp(cat.e1), O.dp(cat.e2),
            O.dp(snr), O.dp(sumw), cptr(g2), cptr(s), cptr(d), O.fp(sigma2), O.bp(flag), O.dp(obs.uu), O.dp(obs.vv),
            O.dp(obs.ww), C.byref(ft), C.byref(bad)]
    ref.data_processing(False, bad_list.ctypes.data_as(O.PU), cat.n, L, obs.n_rows, fp, *args)
    nbad1 = bad.value
    out["dp_bad_list"] = bad_list[:nbad1].copy()
    out["dp_data1_sub"] = d[::SUB].copy()
    out["dp_sky1_sub"] = s[::SUB].copy()
    ref.data_processing(True, bad_list.ctypes.data_as(O.PU), nbad1, L, obs.n_rows, fp, *args)
    libc.fclose(fp)
    out["dp_nbad_final"] = np.int64(bad.value)
    out["dp_data2_sub"] = d[::SUB].copy()
    out["dp_sky2_sub"] = s[::SUB].copy()
    with open(tmp.name) as f:
        rows = [line.strip() for line in f if line.strip()]
    os.unlink(tmp.name)
    out["dp_rows"] = np.array(rows)
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **out)
    print(f"wrote golden_small.npz: {cat.n} galaxies, {obs.n_vis} visibilities, bad after pass 1: {nbad1}, "
          f"rows: {len(rows)}")


if __name__ == "__main__":
    main()
