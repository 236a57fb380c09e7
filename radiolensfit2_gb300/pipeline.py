"""Python host layer over the device-resident API of librlf_gb300.so (include/rlf_gb300.h).

DeviceObservation keeps uvw, variances, flags, data and sky model in GPU memory and runs the
per-galaxy pipeline (extraction -> fit -> removal, then the re-fit pass) in native code.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from . import constants as K
from .synth import Catalogue, Observation


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_lib.PD)


RESULT_DTYPE = np.dtype([("e1", "f8"), ("e2", "f8"), ("var_e1", "f8"), ("var_e2", "f8"),
                         ("oneDimvar", "f8"), ("maxL", "f8"), ("error", "i4"), ("iters", "i4"),
                         ("nevals", "i4"), ("newton_iters", "i4"), ("status", "i4"),
                         ("ncoords", "i4"), ("max_e1", "f8"), ("max_e2", "f8")])


@dataclass
class ProcessResult:
    results: np.ndarray       # RESULT_DTYPE [n_gal]
    n_bad: int
    ms: tuple                 # (total, extract, fit, remove) milliseconds, CUDA events
    stats: dict = None        # streaming passes and fitted galaxies (rlf_obs_last_stats)


class DeviceObservation:
    def __init__(self, obs: Observation, precision: int = _lib.RLF_MIXED, sigma2=None, flag=None):
        self.lib = _lib.load()
        self.obs = obs
        self.precision = precision
        n_vis = obs.n_vis
        if sigma2 is None:
            sigma2 = np.full(n_vis, np.float32(obs.sigma2), dtype=np.float32)
        self._keep = []
        uu, puu = _d(obs.uu)
        vv, pvv = _d(obs.vv)
        ww, pww = _d(obs.ww)
        wn, pwn = _d(obs.wavenumbers)
        sp, psp = _d(obs.spec)
        s2 = np.ascontiguousarray(sigma2, dtype=np.float32)
        fl = None if flag is None else np.ascontiguousarray(flag, dtype=np.uint8)
        h = self.lib.rlf_obs_create(obs.n_rows, obs.n_ch, puu, pvv, pww, pwn, psp, obs.len_lambda,
                                    s2.ctypes.data_as(_lib.PF),
                                    None if fl is None else fl.ctypes.data_as(_lib.PU8), precision)
        if not h:
            raise RuntimeError("rlf_obs_create failed")
        self.h = C.c_void_p(h)

    def set_data_ms(self, data_block, num_pols: int):
        """Data from a Measurement Set DATA block [n_rows][n_ch][num_pols] complex64 in Jy, converted
        on the GPU as ms_read_vis does (measurement_set.cpp:345-400): Stokes I in uJy, channel-major."""
        b = np.ascontiguousarray(data_block, dtype=np.complex64).reshape(-1)
        if b.size != self.obs.n_vis * num_pols:
            raise ValueError("DATA block size does not match the observation")
        if self.lib.rlf_obs_set_data_ms(self.h, b.view(np.float32).ctypes.data_as(_lib.PF), num_pols):
            raise RuntimeError("rlf_obs_set_data_ms failed")

    def close(self):
        if getattr(self, "h", None):
            self.lib.rlf_obs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed ({rc})")

    def set_vis(self, data=None, sky=None):
        d = None if data is None else np.ascontiguousarray(data, dtype=np.complex128)
        s = None if sky is None else np.ascontiguousarray(sky, dtype=np.complex128)
        self._check(self.lib.rlf_obs_set_vis(
            self.h, None if d is None else d.ctypes.data_as(_lib.PD),
            None if s is None else s.ctypes.data_as(_lib.PD)), "rlf_obs_set_vis")

    def set_data_c64(self, data):
        d = np.ascontiguousarray(data, dtype=np.complex64)
        self._check(self.lib.rlf_obs_set_data_c64(self.h, d.ctypes.data_as(_lib.PF)), "rlf_obs_set_data_c64")

    def get_vis(self):
        n = self.obs.n_vis
        d = np.empty(n, np.complex128)
        s = np.empty(n, np.complex128)
        self._check(self.lib.rlf_obs_get_vis(self.h, d.ctypes.data_as(_lib.PD), s.ctypes.data_as(_lib.PD)),
                    "rlf_obs_get_vis")
        return d, s

    def simulate(self, cat: Catalogue, noise_sigma: float, seed: int = 3, gaussian: int = 0):
        arrs = [_d(x) for x in (cat.flux, cat.scale, cat.e1, cat.e2, cat.l, cat.m)]
        self._check(self.lib.rlf_obs_simulate(self.h, cat.n, *[p for _, p in arrs], float(noise_sigma),
                                              int(seed), gaussian), "rlf_obs_simulate")

    def sky_model(self, cat: Catalogue, gaussian: int = 0):
        arrs = [_d(x) for x in (cat.flux, cat.scale, cat.l, cat.m)]
        self._check(self.lib.rlf_obs_sky_model(self.h, cat.n, *[p for _, p in arrs], gaussian),
                    "rlf_obs_sky_model")

    def snapshot(self):
        self._check(self.lib.rlf_obs_snapshot(self.h), "rlf_obs_snapshot")

    def restore(self):
        self._check(self.lib.rlf_obs_restore(self.h), "rlf_obs_restore")

    def process(self, cat: Catalogue, *, batch: int = 1, refit: bool = True, gaussian: int = 0,
                start=None, verbose: int = 0, fit_precision: int = _lib.RLF_F64, rounds: int = 0,
                board_wait_us: int = 0, proposal: int = 0, seq_facet_kb: int = 0,
                fit_ctas_per_sm: int = 0, graphs: int = 0) -> ProcessResult:
        ro, pro = _d(K.ro_grid())
        arrs = [_d(x) for x in (cat.flux, cat.scale, cat.l, cat.m)]
        opt = _lib.Options()
        opt.precision = self.precision
        opt.batch = int(batch)
        opt.gaussian = gaussian
        opt.refit = 1 if refit else 0
        opt.verbose = verbose
        opt.fit_precision = int(fit_precision)
        opt.rounds = int(rounds)
        opt.board_wait_us = int(board_wait_us)
        opt.proposal = int(proposal)
        opt.seq_facet_kb = int(seq_facet_kb)
        opt.fit_ctas_per_sm = int(fit_ctas_per_sm)
        opt.graphs = int(graphs)
        st = None
        if start is not None:
            st = np.ascontiguousarray(start, dtype=np.float64).reshape(-1)
            opt.start = st.ctypes.data_as(_lib.PD)
        out = (_lib.FitResult * cat.n)()
        nbad = C.c_int(0)
        self._check(self.lib.rlf_obs_process(self.h, cat.n, *[p for _, p in arrs], len(ro), pro, C.byref(opt),
                                             out, C.byref(nbad)), "rlf_obs_process")
        res = np.frombuffer(out, dtype=RESULT_DTYPE, count=cat.n).copy()
        ms = (C.c_double * 4)()
        self.lib.rlf_obs_last_timing(self.h, ms)
        names = ("extract_passes", "extract_single", "remove_batches", "remove_single", "fitted",
                 "extract_gal", "changed", "extract_gal_first", "skipped_gal",
                 "extract_seq_us", "graphs")  # RLF_NSTATS entries
        sv = (C.c_longlong * len(names))()
        self.lib.rlf_obs_last_stats(self.h, sv)
        stats = dict(zip(names, (int(x) for x in sv)))
        return ProcessResult(res, nbad.value, tuple(ms), stats)

    def facet_partials(self, cat: Catalogue, stride: int) -> np.ndarray:
        """Un-averaged facet sums of every galaxy over this observation's channels,
        [n][4][stride]: sum vis re, sum vis im, sum sigma^2, sum of weights per cell
        (rlf_obs_facet_partials)."""
        arrs = [_d(x) for x in (cat.flux, cat.scale, cat.l, cat.m)]
        out = np.zeros((cat.n, 4, stride))
        self._check(self.lib.rlf_obs_facet_partials(self.h, cat.n, *[p for _, p in arrs],
                                                    out.ctypes.data_as(_lib.PD), int(stride)),
                    "rlf_obs_facet_partials")
        return out

    def remove(self, cat: Catalogue, results: np.ndarray):
        """Removal of the given fits (RESULT_DTYPE rows; error != 0 skipped) from the data and sky
        model, in catalogue order (rlf_obs_remove)."""
        arrs = [_d(x) for x in (cat.flux, cat.scale, cat.l, cat.m)]
        r = np.ascontiguousarray(results, RESULT_DTYPE)
        buf = (_lib.FitResult * cat.n).from_buffer_copy(r.tobytes()) if cat.n else (_lib.FitResult * 1)()
        self._check(self.lib.rlf_obs_remove(self.h, cat.n, *[p for _, p in arrs], buf), "rlf_obs_remove")

    def extract(self, cat: Catalogue, *, batch: int = 1):
        """Facets of every galaxy against the current data and sky model (no fit, no removal).
        Returns a list of (u, v, vis/sigma2, sigma2) arrays per galaxy."""
        fmax = K.facet_size(K.RMAX, self.obs.len_lambda)
        stride = fmax * fmax
        arrs = [_d(x) for x in (cat.flux, cat.scale, cat.l, cat.m)]
        buf = np.zeros((cat.n, 5, stride))
        nc = np.zeros(cat.n, np.int32)
        self._check(self.lib.rlf_obs_extract(self.h, cat.n, *[p for _, p in arrs], int(batch),
                                             buf.ctypes.data_as(_lib.PD), stride, nc.ctypes.data_as(_lib.PI)),
                    "rlf_obs_extract")
        out = []
        for g in range(cat.n):
            n = int(nc[g])
            out.append((buf[g, 0, :n].copy(), buf[g, 1, :n].copy(), buf[g, 2, :n] + 1j * buf[g, 3, :n],
                        buf[g, 4, :n].copy()))
        return out
