"""Seeded synthetic interferometer arrays and galaxy catalogues.

The reference reads a Measurement Set (measurement_set.cpp) and a catalogue file
(read_catalog.c); neither ships with it, and no public dataset is named for this path.  These
generators produce inputs with the shapes, sizes and distributions of the workloads the path
is measured on:

* array: antennas at radius sqrt(U)*R with uniform angle, baselines i<j, hour angles evenly
  spaced over +-H, standard ENU -> equatorial -> (u,v,w) rotation; rows are time-major x
  baseline, uvw in metres (FP64), as ms_read_coords returns them (measurement_set.cpp:204-241);
* channels: centre frequencies f0 + (ch+1/2) df, wavenumber 2 pi f / c and spectral factor
  (f / 1.4 GHz)^-0.7 (RadioLensfit2.cpp:342-351);
* catalogue: flux dN/dS ~ S^-1.34 by inverse CDF, sorted by decreasing flux and repeated in
  rings of 2*NUM_ORIENT orientations as generate_catalog.c:60-112 does; ln r ~ N(ln(0.3''
  (S/10uJy)^0.33), 0.3); |e| from p(e) ~ e(1-exp((e-0.804)/0.254))/((1+e) sqrt(e^2+0.0732^2))
  by inverse CDF on 1000 points; positions uniform in a disk; shear applied as
  e' = (e+g)/(1+g* e) (data_simulation.c:69-74);
* noise: complex Gaussian with sigma = SEFD/sqrt(2 dt df) per component (uJy), uniform weights.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import constants as K


@dataclass
class Observation:
    uu: np.ndarray            # [n_rows] metres, float64
    vv: np.ndarray
    ww: np.ndarray
    wavenumbers: np.ndarray   # [n_ch] rad/m
    spec: np.ndarray          # [n_ch]
    n_rows: int
    n_ch: int
    dt_s: float
    df_hz: float
    f_start_hz: float
    sigma: float              # noise rms per real/imag component, uJy
    len_metres: float         # ceil(max(|u|,|v|)) as ms_read_coords returns it
    len_lambda: float         # len_metres * wavenumbers[-1] / (2 pi) (RadioLensfit2.cpp:406)

    @property
    def n_vis(self) -> int:
        return self.n_rows * self.n_ch

    @property
    def sigma2(self) -> float:
        return float(np.float32(self.sigma * self.sigma))


@dataclass
class Catalogue:
    flux: np.ndarray
    scale: np.ndarray
    e1: np.ndarray            # sheared ellipticity (what the visibilities contain)
    e2: np.ndarray
    e1_int: np.ndarray        # intrinsic ellipticity before shear
    e2_int: np.ndarray
    l: np.ndarray             # direction cosines (rad)
    m: np.ndarray
    g: tuple = (0.0, 0.0)

    @property
    def n(self) -> int:
        return int(self.flux.shape[0])

    def subset(self, idx) -> "Catalogue":
        idx = np.asarray(idx)
        return Catalogue(self.flux[idx], self.scale[idx], self.e1[idx], self.e2[idx],
                         self.e1_int[idx], self.e2_int[idx], self.l[idx], self.m[idx], self.g)


# Workloads: the reference's CPU-sized case and the GPU-sized cases.
WORKLOADS = {
    "c0_small_cpu": dict(n_ant=64, ha_hours=2.0, dt_s=120.0, n_ch=4, n_gal=100, fmin=10.0,
                         fmax=200.0, g=(0.03, -0.02)),
    "c1_ska_mid_16ch": dict(n_ant=197, ha_hours=4.0, dt_s=60.0, n_ch=16, n_gal=1000,
                            fmin=10.0, fmax=200.0, g=(0.03, -0.02)),
    "c2_ska_mid_32ch": dict(n_ant=197, ha_hours=4.0, dt_s=60.0, n_ch=32, n_gal=10000,
                            fmin=5.0, fmax=200.0, g=(0.03, -0.02)),
    "c4_ska_mid_64ch": dict(n_ant=197, ha_hours=4.0, dt_s=30.0, n_ch=64, n_gal=50000,
                            fmin=5.0, fmax=200.0, g=(0.02, 0.01)),
    # profiling case: C1's channel layout on a smaller array, 15.6M visibilities (250 MB of FP32
    # data and sky model, larger than the 129 MB L2), 64 galaxies
    "mid_128ant_16ch": dict(n_ant=128, ha_hours=1.0, dt_s=60.0, n_ch=16, n_gal=64,
                            fmin=10.0, fmax=200.0, g=(0.03, -0.02)),
    # profiling case with the full-scale channel layout (64 channels): 62M visibilities (1 GB of
    # FP32 data and sky model, larger than the 129 MB L2), 64 galaxies of the full-scale flux range
    "mid_128ant_64ch": dict(n_ant=128, ha_hours=0.5, dt_s=30.0, n_ch=64, n_gal=64,
                            fmin=5.0, fmax=200.0, g=(0.02, 0.01)),
}

ARRAY_SEED, CATALOGUE_SEED, NOISE_SEED = 1, 2, 3


def make_observation(n_ant: int, ha_hours: float, dt_s: float, n_ch: int, *,
                     radius_m: float = 4000.0, dec_deg: float = -30.0, lat_deg: float = -30.0,
                     f_start_hz: float = 950e6, df_hz: float = 240e3, sefd_ujy: float = K.SEFD_SKA,
                     seed: int = ARRAY_SEED, **_ignored) -> Observation:
    rng = np.random.default_rng(seed)
    r = np.sqrt(rng.random(n_ant)) * radius_m
    th = rng.random(n_ant) * 2 * math.pi
    east, north = r * np.cos(th), r * np.sin(th)
    lat = math.radians(lat_deg)
    # local ENU (up = 0) to equatorial XYZ
    X = -math.sin(lat) * north
    Y = east
    Z = math.cos(lat) * north
    i, j = np.triu_indices(n_ant, k=1)
    bx, by, bz = X[j] - X[i], Y[j] - Y[i], Z[j] - Z[i]
    n_times = int(round(2 * ha_hours * 3600.0 / dt_s))
    ha = (-ha_hours * 3600.0 + (np.arange(n_times) + 0.5) * dt_s) / 86164.0905 * 2 * math.pi
    dec = math.radians(dec_deg)
    sh, ch_ = np.sin(ha)[:, None], np.cos(ha)[:, None]
    sd, cd = math.sin(dec), math.cos(dec)
    uu = (sh * bx + ch_ * by).reshape(-1)
    vv = (-sd * ch_ * bx + sd * sh * by + cd * bz).reshape(-1)
    ww = (cd * ch_ * bx - cd * sh * by + sd * bz).reshape(-1)
    freqs = f_start_hz + 0.5 * df_hz + np.arange(n_ch) * df_hz
    # RadioLensfit2.cpp:344-351 accumulates ch_freq += df; reproduce that summation order
    wn = np.empty(n_ch)
    sp = np.empty(n_ch)
    f = f_start_hz + 0.5 * df_hz
    for c in range(n_ch):
        wn[c] = 2.0 * K.PI * f / K.C0
        sp[c] = math.pow(f / K.REF_FREQ, -0.7)
        f += df_hz
    del freqs
    len_m = float(math.ceil(max(np.abs(uu).max(), np.abs(vv).max())))
    len_lambda = len_m * wn[-1] / (2 * K.PI)
    sigma = sefd_ujy / math.sqrt(2.0 * dt_s * df_hz)
    return Observation(uu=np.ascontiguousarray(uu), vv=np.ascontiguousarray(vv),
                       ww=np.ascontiguousarray(ww), wavenumbers=wn, spec=sp,
                       n_rows=int(uu.shape[0]), n_ch=n_ch, dt_s=dt_s, df_hz=df_hz,
                       f_start_hz=f_start_hz, sigma=sigma, len_metres=len_m,
                       len_lambda=len_lambda)


def _e_pdf(e, disp=0.254):
    return e * (1.0 - np.exp((e - K.E_MAX) / disp)) / ((1.0 + e) * np.sqrt(e * e + K.E_0 * K.E_0))


def make_catalogue(n_gal: int, fmin: float, fmax: float, g=(0.0, 0.0), *,
                   radius_deg: float = 0.5, seed: int = CATALOGUE_SEED,
                   rings: bool = True, r_median_10ujy: float = 0.3, r_sigma_ln: float = 0.3,
                   r_max: float = K.RMAX, **_ignored) -> Catalogue:
    rng = np.random.default_rng(seed)
    per = 2 * K.NUM_ORIENT if rings else 1
    n_distinct = max(1, -(-n_gal // per))
    a = -1.34 + 1.0  # exponent of the integrated power law dN/dS ~ S^-1.34
    u = rng.random(n_distinct)
    flux = (fmin ** a + u * (fmax ** a - fmin ** a)) ** (1.0 / a)
    flux = np.sort(flux)[::-1]
    mu = np.log(r_median_10ujy * (flux / 10.0) ** 0.33)
    scale = np.exp(mu + r_sigma_ln * rng.standard_normal(n_distinct))
    scale = np.clip(scale, 0.05, r_max)
    # |e| by inverse CDF on 1000 points
    ee = np.linspace(0.0, K.E_MAX, 1001)
    pdf = _e_pdf(ee)
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (pdf[1:] + pdf[:-1]) * np.diff(ee))])
    cdf /= cdf[-1]
    emod = np.interp(rng.random(n_distinct), cdf, ee)
    phi0 = rng.random(n_distinct) * 2 * math.pi
    e1 = np.empty(n_distinct * per)
    e2 = np.empty(n_distinct * per)
    fl = np.repeat(flux, per)
    sc = np.repeat(scale, per)
    if rings:
        k = np.arange(K.NUM_ORIENT)
        phi = phi0[:, None] + k[None, :] * (math.pi / K.NUM_ORIENT)
        c1, c2 = emod[:, None] * np.cos(phi), emod[:, None] * np.sin(phi)
        e1 = np.stack([c1, -c1], axis=2).reshape(-1)
        e2 = np.stack([c2, -c2], axis=2).reshape(-1)
    else:
        e1 = emod * np.cos(phi0)
        e2 = emod * np.sin(phi0)
    e1, e2, fl, sc = e1[:n_gal], e2[:n_gal], fl[:n_gal], sc[:n_gal]
    # shear: e' = (e + g) / (1 + conj(g) e)  (data_simulation.c:69-74)
    g1, g2 = g
    z1r, z1i = e1 + g1, e2 + g2
    z2r, z2i = 1.0 + e1 * g1 + e2 * g2, e2 * g1 - e1 * g2
    den = z2r * z2r + z2i * z2i
    se1 = (z1r * z2r + z1i * z2i) / den
    se2 = (z1i * z2r - z1r * z2i) / den
    rad = np.sqrt(rng.random(n_gal)) * math.radians(radius_deg)
    ori = rng.random(n_gal) * 2 * math.pi
    return Catalogue(flux=np.ascontiguousarray(fl), scale=np.ascontiguousarray(sc),
                     e1=se1, e2=se2, e1_int=e1.copy(), e2_int=e2.copy(),
                     l=rad * np.cos(ori), m=rad * np.sin(ori), g=(g1, g2))


def galaxy_visibilities_np(obs: Observation, e1, e2, scale, flux, l, m, gaussian=False):
    """Host (numpy) model visibilities of one galaxy over all channels, [n_ch, n_rows] complex128.
    Same formula as galaxy_visibilities.c:154-190; used only to build small test inputs."""
    detA = 1.0 - e1 * e1 - e2 * e2
    sc = scale * (K.PI / 648000.0)
    sf = (sc * sc) / (detA * detA)
    n = math.sqrt(1.0 - l * l - m * m) - 1.0
    p = obs.uu * l + obs.vv * m + obs.ww * n
    k1 = (1.0 + e1) * obs.uu + e2 * obs.vv
    k2 = e2 * obs.uu + (1.0 - e1) * obs.vv
    kk = k1 * k1 + k2 * k2
    out = np.empty((obs.n_ch, obs.n_rows), dtype=np.complex128)
    for c in range(obs.n_ch):
        wn = obs.wavenumbers[c]
        if gaussian:
            shape = np.exp(-0.5 * sf * (wn * wn) * kk)
        else:
            den = 1.0 + sf * (wn * wn) * kk
            shape = 1.0 / (den * np.sqrt(den))
        shape = shape * (obs.spec[c] * flux)
        ph = wn * p
        out[c] = shape * np.cos(ph) + 1j * shape * np.sin(ph)
    return out


def simulate_visibilities_np(obs: Observation, cat: Catalogue, *, noise_sigma=None,
                             seed: int = NOISE_SEED, gaussian=False) -> np.ndarray:
    """Data visibilities (sum of sheared galaxy models plus noise) as complex64 [n_ch*n_rows].
    numpy version for small test inputs; the GPU simulator covers the large workloads."""
    vis = np.zeros((obs.n_ch, obs.n_rows), dtype=np.complex128)
    for gi in range(cat.n):
        vis += galaxy_visibilities_np(obs, cat.e1[gi], cat.e2[gi], cat.scale[gi], cat.flux[gi],
                                      cat.l[gi], cat.m[gi], gaussian)
    s = obs.sigma if noise_sigma is None else noise_sigma
    if s > 0:
        rng = np.random.default_rng(seed)
        vis += s * (rng.standard_normal(vis.shape) + 1j * rng.standard_normal(vis.shape))
    return vis.reshape(-1).astype(np.complex64)
