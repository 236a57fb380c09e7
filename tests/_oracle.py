"""ctypes bindings to the oracle (test infrastructure only).

* ``orc``: oracle/_build/librlf_oracle.so, the CPU restatement, built by ``make -C oracle``
  (``__graft_entry__.build()`` runs it);
* ``ref``: oracle/_ref/librlf_ref.so, the reference's own sources compiled against the GSL
  shim; present only where the reference checkout exists (never on the GPU machine).
"""
import ctypes as C
import os
import subprocess

import numpy as np

from radiolensfit2_gb300.abi import LikelihoodParams, GslVector, Complexd  # noqa: F401

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORC_PATH = os.path.join(ORACLE_DIR, "_build", "librlf_oracle.so")
REF_PATH = os.path.join(ORACLE_DIR, "_ref", "librlf_ref.so")
REF_FAST_PATH = os.path.join(ORACLE_DIR, "_ref", "librlf_ref_fastmath.so")

D = C.c_double
PD = C.POINTER(C.c_double)
PF = C.POINTER(C.c_float)
PU8 = C.POINTER(C.c_uint8)
PU = C.POINTER(C.c_uint)


class OrcComplex(C.Structure):
    _fields_ = [("real", D), ("imag", D)]


PC = C.POINTER(OrcComplex)


class OrcParams(C.Structure):
    _fields_ = [("numr", C.c_int), ("ro", PD), ("rprior", PD), ("ncoords", C.c_uint),
                ("uu", PD), ("vv", PD), ("data", PC), ("sigma2", PD), ("mod", PD),
                ("gaussian", C.c_int), ("nevals", C.c_long), ("newton_iters", C.c_long),
                ("trace", PD), ("trace_cap", C.c_long)]


class OrcFitResult(C.Structure):
    _fields_ = [("e1", D), ("e2", D), ("var_e1", D), ("var_e2", D), ("oneDimvar", D),
                ("maxL", D), ("error", C.c_int), ("iters", C.c_int), ("nevals", C.c_long),
                ("max_e1", D), ("max_e2", D)]


def _build_oracle():
    if not os.path.exists(ORC_PATH):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "oracle"], check=True)


def load_oracle():
    _build_oracle()
    lib = C.CDLL(ORC_PATH)
    lib.orc_facet_size.restype = C.c_uint
    lib.orc_facet_size.argtypes = [D, D]
    lib.orc_uv_grid_size.restype = C.c_uint
    lib.orc_uv_grid_size.argtypes = [D, PD, C.c_uint, C.c_uint, PD, PD, C.c_uint, PU8]
    lib.orc_facet_coords.restype = C.c_uint
    lib.orc_facet_coords.argtypes = [PD, PD, D, C.c_uint, PD]
    lib.orc_gridding.restype = None
    lib.orc_gridding.argtypes = [PD, C.c_uint, C.c_uint, PD, PD, PC, PF, D, C.c_uint, PC, PD, PU8, PD]
    lib.orc_average_facets.restype = None
    lib.orc_average_facets.argtypes = [C.c_ulong, PC, PD, PD]
    lib.orc_ms_read_coords.restype = D
    lib.orc_ms_read_coords.argtypes = [PD, C.c_uint, PD, PD, PD]
    lib.orc_ms_read_flag.restype = C.c_ulong
    lib.orc_ms_read_flag.argtypes = [PU8, C.c_uint, C.c_uint, C.c_uint, PU8]
    lib.orc_ms_read_vis.restype = None
    lib.orc_ms_read_vis.argtypes = [PF, C.c_uint, C.c_uint, C.c_uint, PC]
    lib.orc_ms_read_sigma2.restype = None
    lib.orc_ms_read_sigma2.argtypes = [PF, C.c_uint, C.c_uint, C.c_float, PF]
    lib.orc_ms_write_vis.restype = None
    lib.orc_ms_write_vis.argtypes = [PC, C.c_uint, C.c_uint, PF]
    for nm in ("orc_sersic_shape", "orc_gaussian_shape"):
        getattr(lib, nm).restype = D
        getattr(lib, nm).argtypes = [D, D, D, D]
    lib.orc_model_at_zero.restype = None
    lib.orc_model_at_zero.argtypes = [D, D, D, C.c_uint, PD, PD, PD, PD, C.c_int]
    lib.orc_data_galaxy_vis.restype = None
    lib.orc_data_galaxy_vis.argtypes = [D, D, D, D, D, D, D, D, C.c_uint, PD, PD, PD, PC, C.c_int]
    lib.orc_phase_shift.restype = None
    lib.orc_phase_shift.argtypes = [D, D, D, C.c_uint, PD, PD, PD, PC]
    lib.orc_source_extraction.restype = None
    lib.orc_source_extraction.argtypes = [C.c_uint, PD, PD, C.c_uint, PC, PD, PD, D, D, D, D, D, D,
                                          PC, PC, PC, PF, PU8, C.c_ulong, PD, PD, PD, D, C.c_int]
    lib.orc_cross_correlation.restype = C.c_int
    lib.orc_cross_correlation.argtypes = [C.c_ulong, PD, PD, PC, PD, PD, PD, C.POINTER(C.c_int)]
    lib.orc_ei.restype = D
    lib.orc_ei.argtypes = [D]
    lib.orc_marginalise_over_position_shift.restype = D
    lib.orc_marginalise_over_position_shift.argtypes = [D]
    lib.orc_loglikelihood_r.restype = D
    lib.orc_loglikelihood_r.argtypes = [D, D, D, C.c_ulong, PD, PD, PD, PC, PD, C.c_int, C.POINTER(C.c_int)]
    lib.orc_loglikelihood.restype = D
    lib.orc_loglikelihood.argtypes = [C.POINTER(OrcParams), D, D, C.POINTER(C.c_int)]
    lib.orc_loglikelihood_nodes.restype = D
    lib.orc_loglikelihood_nodes.argtypes = [C.POINTER(OrcParams), D, D, PD]
    lib.orc_set_posterior_values.restype = None
    lib.orc_set_posterior_values.argtypes = [C.c_int, PD, PD, PD, PD, PD, C.POINTER(C.c_int)]
    lib.orc_marginalise_posterior_r.restype = D
    lib.orc_marginalise_posterior_r.argtypes = [C.c_int, PD, PD]
    lib.orc_likelihood_sampling.restype = None
    lib.orc_likelihood_sampling.argtypes = [PD, PD, D, C.POINTER(OrcParams), C.c_int, PD, PD, PD]
    lib.orc_source_fitting.restype = C.c_int
    lib.orc_source_fitting.argtypes = [C.POINTER(OrcParams), D, D, D, C.POINTER(OrcFitResult)]
    lib.orc_scale_mean.restype = D
    lib.orc_scale_mean.argtypes = [D]
    lib.orc_rfunc.restype = D
    lib.orc_rfunc.argtypes = [D, D, D]
    lib.orc_ro_grid.restype = C.c_int
    lib.orc_ro_grid.argtypes = [PD, C.c_int]
    lib.orc_sky_model.restype = None
    lib.orc_sky_model.argtypes = [PD, PD, C.c_uint, C.c_uint, PD, PD, PD, PD, C.c_ulong, PD, PD, PD,
                                  PC, PC, C.c_int]
    lib.orc_data_processing.restype = None
    lib.orc_data_processing.argtypes = [C.c_int, PU, C.c_int, D, C.c_uint, C.c_uint, PD, PD, C.c_int,
                                        PD, PD, PD, PD, PD, PD, PC, PC, PC, PF, PU8, PD, PD, PD,
                                        C.c_int, C.POINTER(OrcFitResult), C.POINTER(C.c_int)]
    return lib


def have_ref():
    return os.path.exists(REF_PATH)


def load_ref(fastmath=False):
    lib = C.CDLL(REF_FAST_PATH if fastmath else REF_PATH)
    P = C.POINTER(LikelihoodParams)
    PCd = C.POINTER(Complexd)
    lib.facet_size.restype = C.c_uint
    lib.facet_size.argtypes = [D, D]
    lib.evaluate_uv_grid_size.restype = C.c_uint
    lib.evaluate_uv_grid_size.argtypes = [C.c_int, C.c_int, D, PD, C.c_uint, C.c_uint, PD, PD, C.c_uint, PU8]
    lib.evaluate_facet_coords.restype = C.c_uint
    lib.evaluate_facet_coords.argtypes = [PD, PD, D, C.c_uint, PD]
    lib.gridding_visibilities.restype = None
    lib.gridding_visibilities.argtypes = [PD, C.c_uint, C.c_uint, PD, PD, PCd, PF, D, C.c_uint, PCd, PD, PU8, PD]
    lib.average_facets.restype = None
    lib.average_facets.argtypes = [C.c_ulong, PCd, PD, PD]
    lib.sersic_shape.restype = D
    lib.sersic_shape.argtypes = [D, D, D, D]
    lib.gaussian_shape.restype = D
    lib.gaussian_shape.argtypes = [D, D, D, D]
    lib.model_galaxy_visibilities_at_zero.restype = None
    lib.model_galaxy_visibilities_at_zero.argtypes = [D, D, D, C.c_uint, PD, PD, PD, PD]
    lib.data_galaxy_visibilities.restype = None
    lib.data_galaxy_visibilities.argtypes = [D, D, D, D, D, D, D, D, D, D, C.c_uint, PD, PD, PD, PCd]
    lib.data_visibilities_phase_shift.restype = None
    lib.data_visibilities_phase_shift.argtypes = [D, D, D, C.c_uint, PD, PD, PD, PCd]
    lib.source_extraction.restype = None
    lib.source_extraction.argtypes = [C.c_int, C.c_uint, P, PCd, PD, PD, D, D, D, D, D, D, PCd, PCd, PCd,
                                      PF, PU8, C.c_ulong, PD, PD, PD, D]
    lib.cross_correlation.restype = C.c_int
    lib.cross_correlation.argtypes = [C.c_ulong, PD, PD, PCd, PD, PD, PD]
    lib.marginalise_over_position_shift.restype = D
    lib.marginalise_over_position_shift.argtypes = [D]
    lib.loglikelihood_r.restype = D
    lib.loglikelihood_r.argtypes = [D, D, D, C.c_ulong, PD, PD, PD, PCd, PD]
    lib.loglikelihood.restype = D
    lib.loglikelihood.argtypes = [C.c_void_p, D, D, C.POINTER(C.c_int)]
    lib.f_likelihood.restype = D
    lib.f_likelihood.argtypes = [C.POINTER(GslVector), C.c_void_p]
    lib.likelihood_sampling.restype = None
    lib.likelihood_sampling.argtypes = [PD, PD, D, C.c_void_p, C.c_int, PD, PD, PD]
    lib.source_fitting.restype = C.c_int
    lib.source_fitting.argtypes = [C.c_int, P, PD, PD, PD, PD, PD, PD]
    lib.rlfref_set_posterior_values.restype = None
    lib.rlfref_set_posterior_values.argtypes = [C.c_int, PD, PD, PD, PD, PD, C.POINTER(C.c_int)]
    lib.rlfref_marginalise_posterior_r.restype = D
    lib.rlfref_marginalise_posterior_r.argtypes = [C.c_int, PD, PD]
    lib.rfunc.restype = D
    lib.rfunc.argtypes = [D, D, D]
    lib.scale_mean.restype = D
    lib.scale_mean.argtypes = [D]
    lib.sky_model.restype = None
    lib.sky_model.argtypes = [PD, PD, D, C.c_int, C.c_uint, C.c_uint, PD, PD, PD, PD, C.c_ulong, PD, PD,
                              PD, PCd, PCd]
    lib.data_processing.restype = None
    lib.data_processing.argtypes = [C.c_bool, PU, C.c_int, D, C.c_uint, C.c_void_p, P, PD, PD, PD, PD,
                                    PD, PD, PD, PD, PCd, PCd, PCd, PF, PU8, PD, PD, PD, PD,
                                    C.POINTER(C.c_int)]
    return lib


def dp(a):
    return a.ctypes.data_as(PD)


def fp(a):
    return a.ctypes.data_as(PF)


def cp(a):
    assert a.dtype == np.complex128
    return a.ctypes.data_as(PC)


def bp(a):
    return a.ctypes.data_as(PU8)
