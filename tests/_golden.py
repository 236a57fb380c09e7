"""Loader of tests/golden/golden_small.npz (made by tests/golden/make_golden.py from the
reference's own compiled code) and helpers shared by the CPU and GPU golden tests."""
import ctypes as C
import math
import os

import numpy as np

from radiolensfit2_gb300 import constants as K
from radiolensfit2_gb300.synth import Observation, Catalogue

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "golden", "golden_small.npz")
SUB = 7


class Golden:
    def __init__(self, path=PATH):
        z = np.load(path)
        self.z = z
        n_rows, n_ch = int(z["n_rows"]), int(z["n_ch"])
        self.obs = Observation(uu=z["uu"], vv=z["vv"], ww=z["ww"], wavenumbers=z["wavenumbers"],
                               spec=z["spec"], n_rows=n_rows, n_ch=n_ch, dt_s=600.0, df_hz=240e3,
                               f_start_hz=950e6, sigma=250.0, len_metres=0.0,
                               len_lambda=float(z["len_lambda"]))
        self.cat = Catalogue(flux=z["flux"], scale=z["scale"], e1=z["e1"], e2=z["e2"], e1_int=z["e1"],
                             e2_int=z["e2"], l=z["l"], m=z["m"])
        self.data = z["data"].astype(np.complex128)
        self.sigma2 = z["sigma2"]
        self.flag = z["flag"]
        self.ro = z["ro"]
        self.numr = len(self.ro)
        self.len = float(z["len_lambda"])

    def __getitem__(self, k):
        return self.z[k]


def _cf(x):
    """printf("%f") as glibc prints it, including the sign of a NaN."""
    if math.isnan(x):
        return "-nan" if math.copysign(1.0, x) < 0 else "nan"
    return "%f" % x


def _csqrt(x):
    """C sqrt: a negative argument gives -nan on x86-64 and aarch64 glibc."""
    return math.sqrt(x) if x >= 0 else (x if math.isnan(x) else -float("nan"))


def format_row(flux, ge1, e1, var1, ge2, e2, var2, onedvar, snr, l, m):
    """The output row of data_processing.c:101,136."""
    a = K.PI / 648000.0
    vals = (flux, ge1, e1, _csqrt(var1), ge2, e2, _csqrt(var2), onedvar, snr, l / a, m / a)
    return " | ".join(_cf(v) for v in vals)


def rows_from_results(g, order, results):
    """Rows in processing order: results[gal] = (e1, e2, var1, var2, onedvar)."""
    c = g.cat
    return [format_row(c.flux[i], c.e1[i], results[i][0], results[i][2], c.e2[i], results[i][1],
                       results[i][3], results[i][4], 0.0, c.l[i], c.m[i]) for i in order]
