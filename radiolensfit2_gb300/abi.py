"""ctypes mirrors of the reference's C data types (datatype.h:44-74, FACET branch) and of the
GSL vector the simplex objective receives (galaxy_fitting.c:45-48).  The drop-in library takes
exactly these layouts, so a caller built against the reference headers needs no change."""
import ctypes as C

import numpy as np


class Complexd(C.Structure):
    """datatype.h:44-47"""
    _fields_ = [("real", C.c_double), ("imag", C.c_double)]


class LikelihoodParams(C.Structure):
    """datatype.h:49-74 with -DFACET (always on, Makefile:10)."""
    _fields_ = [
        ("numr", C.c_int),
        ("ro", C.POINTER(C.c_double)),
        ("rprior", C.POINTER(C.c_double)),
        ("nchannels", C.c_uint),
        ("band_factor", C.c_double),
        ("acc_time", C.c_double),
        ("spec", C.POINTER(C.c_double)),
        ("wavenumbers", C.POINTER(C.c_double)),
        ("uu", C.POINTER(C.c_double)),
        ("vv", C.POINTER(C.c_double)),
        ("l0", C.c_double),
        ("m0", C.c_double),
        ("data", C.POINTER(Complexd)),
        ("sigma2", C.POINTER(C.c_double)),
        ("mod", C.POINTER(C.c_double)),
        ("facet", C.c_uint),
        ("ncoords", C.c_uint),
    ]


class GslVector(C.Structure):
    """GSL's public gsl_vector layout (size, stride, data, block, owner)."""
    _fields_ = [("size", C.c_size_t), ("stride", C.c_size_t), ("data", C.POINTER(C.c_double)),
                ("block", C.c_void_p), ("owner", C.c_int)]


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_float))


def cptr(a: np.ndarray):
    """complex128 array -> complexd*"""
    assert a.dtype == np.complex128 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(Complexd))


def bptr(a: np.ndarray):
    assert a.dtype in (np.bool_, np.uint8) and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def uptr(a: np.ndarray):
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_uint))


def make_params(ro, rprior, uu, vv, data, sigma2, mod, ncoords, facet=0, nchannels=0,
                spec=None, wavenumbers=None):
    """Fill a LikelihoodParams from numpy arrays (the arrays must outlive the struct)."""
    p = LikelihoodParams()
    p.numr = len(ro)
    p.ro = dptr(ro)
    p.rprior = dptr(rprior)
    p.nchannels = nchannels
    p.band_factor = 0.0
    p.acc_time = 0.0
    p.spec = dptr(spec) if spec is not None else None
    p.wavenumbers = dptr(wavenumbers) if wavenumbers is not None else None
    p.uu = dptr(uu)
    p.vv = dptr(vv)
    p.l0 = 0.0
    p.m0 = 0.0
    p.data = cptr(data)
    p.sigma2 = dptr(sigma2)
    p.mod = dptr(mod)
    p.facet = facet
    p.ncoords = ncoords
    return p
