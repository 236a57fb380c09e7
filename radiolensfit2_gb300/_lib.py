"""ctypes binding of librlf_gb300.so.

The library is built in-tree by radiolensfit2_gb300.build; load() raises if it is missing so
that no caller silently runs without the CUDA path.
"""
from __future__ import annotations

import ctypes as C
import os

from .abi import Complexd, LikelihoodParams, GslVector
from .build import LIB

D = C.c_double
PD = C.POINTER(C.c_double)
PF = C.POINTER(C.c_float)
PU8 = C.POINTER(C.c_uint8)
PU = C.POINTER(C.c_uint)
PI = C.POINTER(C.c_int)
PCd = C.POINTER(Complexd)

RLF_F64 = 0
RLF_MIXED = 1


class FitResult(C.Structure):
    """rlf_fit_result (include/rlf_gb300.h)"""
    _fields_ = [("e1", D), ("e2", D), ("var_e1", D), ("var_e2", D), ("oneDimvar", D), ("maxL", D),
                ("error", C.c_int), ("iters", C.c_int), ("nevals", C.c_int),
                ("newton_iters", C.c_int), ("status", C.c_int), ("ncoords", C.c_int),
                ("max_e1", D), ("max_e2", D)]


class Options(C.Structure):
    """rlf_options (include/rlf_gb300.h)"""
    _fields_ = [("precision", C.c_int), ("batch", C.c_int), ("gaussian", C.c_int),
                ("refit", C.c_int), ("verbose", C.c_int), ("start", PD), ("fit_precision", C.c_int),
                ("rounds", C.c_int), ("reuse_obs", C.c_int),
                ("board_wait_us", C.c_int), ("proposal", C.c_int), ("seq_facet_kb", C.c_int),
                ("fit_ctas_per_sm", C.c_int), ("graphs", C.c_int)]


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise RuntimeError(f"{LIB} is missing: run radiolensfit2_gb300.build.build() "
                           "(the CUDA library is required; there is no CPU fallback)")
    lib = C.CDLL(LIB)
    sig = {
        "rlf_version": (C.c_char_p, []),
        "rlf_device_count": (C.c_int, []),
        "rlf_launch_count": (C.c_longlong, []),
        "rlf_release": (None, []),
        "rlf_obs_set_data_ms": (C.c_int, [C.c_void_p, PF, C.c_uint]),
        "rlf_ms_read_coords": (D, [PD, C.c_uint, PD, PD, PD]),
        "rlf_ms_read_flag": (C.c_ulong, [PU8, C.c_uint, C.c_uint, C.c_uint, PU8]),
        "rlf_ms_read_vis": (C.c_int, [PF, C.c_uint, C.c_uint, C.c_uint, PD]),
        "rlf_ms_read_sigma2": (C.c_int, [PF, C.c_uint, C.c_uint, C.c_float, PF]),
        "rlf_ms_write_vis": (C.c_int, [PD, C.c_uint, C.c_uint, PF]),
        "rlf_transfer_bytes": (None, [C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong)]),
        "rlf_fp32_peak_gflops": (D, []),
        "rlf_configure": (C.c_int, [C.POINTER(Options)]),
        "rlf_obs_create": (C.c_void_p, [C.c_int, C.c_int, PD, PD, PD, PD, PD, D, PF, PU8, C.c_int]),
        "rlf_obs_destroy": (None, [C.c_void_p]),
        "rlf_obs_set_vis": (C.c_int, [C.c_void_p, PD, PD]),
        "rlf_obs_set_data_c64": (C.c_int, [C.c_void_p, PF]),
        "rlf_obs_get_vis": (C.c_int, [C.c_void_p, PD, PD]),
        "rlf_obs_simulate": (C.c_int, [C.c_void_p, C.c_int, PD, PD, PD, PD, PD, PD, D, C.c_uint64, C.c_int]),
        "rlf_obs_sky_model": (C.c_int, [C.c_void_p, C.c_int, PD, PD, PD, PD, C.c_int]),
        "rlf_obs_snapshot": (C.c_int, [C.c_void_p]),
        "rlf_obs_restore": (C.c_int, [C.c_void_p]),
        "rlf_obs_process": (C.c_int, [C.c_void_p, C.c_int, PD, PD, PD, PD, C.c_int, PD,
                                      C.POINTER(Options), C.POINTER(FitResult), PI]),
        "rlf_obs_last_timing": (C.c_int, [C.c_void_p, PD]),
        "rlf_obs_last_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
        "rlf_obs_extract": (C.c_int, [C.c_void_p, C.c_int, PD, PD, PD, PD, C.c_int, PD, C.c_int, PI]),
        "rlf_debug_fit_trace": (C.c_int, [C.c_void_p, PD, C.c_int, PD, C.c_int]),
        "rlf_debug_loglike_nodes": (C.c_int, [C.c_void_p, D, D, C.c_int, PD, PD]),
        "rlf_debug_df_math": (C.c_int, [C.c_int, C.c_int, PD, PD, PD]),
        "rlf_gridding_visibilities_noalloc": (C.c_int, [PD, C.c_uint, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p,
                                                        C.c_void_p, C.c_void_p, D, C.c_uint, C.c_void_p,
                                                        C.c_void_p, C.c_void_p, C.c_void_p]),
        "rlf_obs_facet_partials": (C.c_int, [C.c_void_p, C.c_int, PD, PD, PD, PD, PD, C.c_int]),
        "rlf_fit_partials": (C.c_int, [C.c_int, PD, C.c_int, PD, PD, D, C.c_int, PD, C.POINTER(Options),
                                       C.POINTER(FitResult)]),
        "rlf_obs_remove": (C.c_int, [C.c_void_p, C.c_int, PD, PD, PD, PD, C.POINTER(FitResult)]),
        "rlf_cnn_param_count": (C.c_int, []),
        "rlf_cnn_create": (C.c_void_p, [C.c_int, C.c_int]),
        "rlf_cnn_destroy": (None, [C.c_void_p]),
        "rlf_cnn_set_params": (C.c_int, [C.c_void_p, PF]),
        "rlf_cnn_get_params": (C.c_int, [C.c_void_p, PF]),
        "rlf_cnn_store_facets": (C.c_int, [C.c_void_p, C.c_int, C.c_int, PD, C.c_int, PI, PI, PD, D]),
        "rlf_cnn_set_targets": (C.c_int, [C.c_void_p, C.c_int, C.c_int, PF]),
        "rlf_cnn_read_images": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_uint16)]),
        "rlf_cnn_set_images": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_uint16)]),
        "rlf_cnn_grads": (C.c_int, [C.c_void_p, PI, C.c_int, PF, PF, PF]),
        "rlf_cnn_train_step": (C.c_int, [C.c_void_p, PI, C.c_int, C.c_float, PF]),
        "rlf_cnn_predict": (C.c_int, [C.c_void_p, C.c_int, C.c_int, PF]),
        "rlf_proposal_set_params": (C.c_int, [PF]),
        "rlf_proposal_set_max_sigma": (C.c_int, [C.c_float]),
        # reference-named drop-in entry points
        "facet_size": (C.c_uint, [D, D]),
        "evaluate_uv_grid_size": (C.c_uint, [C.c_int, C.c_int, D, PD, C.c_uint, C.c_uint, PD, PD, C.c_uint, PU8]),
        "evaluate_facet_coords": (C.c_uint, [PD, PD, D, C.c_uint, PD]),
        "gridding_visibilities": (None, [PD, C.c_uint, C.c_uint, PD, PD, PCd, PF, D, C.c_uint, PCd, PD, PU8, PD]),
        "average_facets": (None, [C.c_ulong, PCd, PD, PD]),
        "gaussian_shape": (D, [D, D, D, D]),
        "sersic_shape": (D, [D, D, D, D]),
        "model_galaxy_visibilities_at_zero": (None, [D, D, D, C.c_uint, PD, PD, PD, PD]),
        "data_galaxy_visibilities": (None, [D, D, D, D, D, D, D, D, D, D, C.c_uint, PD, PD, PD, PCd]),
        "data_visibilities_phase_shift": (None, [D, D, D, C.c_uint, PD, PD, PD, PCd]),
        "f_likelihood": (D, [C.POINTER(GslVector), C.c_void_p]),
        "loglikelihood": (D, [C.c_void_p, D, D, PI]),
        "loglikelihood_r": (D, [D, D, D, C.c_ulong, PD, PD, PD, PCd, PD]),
        "cross_correlation": (C.c_int, [C.c_ulong, PD, PD, PCd, PD, PD, PD]),
        "marginalise_over_position_shift": (D, [D]),
        "likelihood_sampling": (None, [PD, PD, D, C.c_void_p, C.c_int, PD, PD, PD]),
        "source_extraction": (None, [C.c_int, C.c_uint, C.POINTER(LikelihoodParams), PCd, PD, PD, D, D, D, D,
                                     D, D, PCd, PCd, PCd, PF, PU8, C.c_ulong, PD, PD, PD, D]),
        "source_fitting": (C.c_int, [C.c_int, C.POINTER(LikelihoodParams), PD, PD, PD, PD, PD, PD]),
        "data_processing": (None, [C.c_bool, PU, C.c_int, D, C.c_uint, C.c_void_p,
                                   C.POINTER(LikelihoodParams), PD, PD, PD, PD, PD, PD, PD, PD, PCd, PCd,
                                   PCd, PF, PU8, PD, PD, PD, PD, PI]),
        "sky_model": (None, [PD, PD, D, C.c_int, C.c_uint, C.c_uint, PD, PD, PD, PD, C.c_ulong, PD, PD, PD,
                             PCd, PCd]),
        "rfunc": (D, [D, D, D]),
        "scale_mean": (D, [D]),
        "rlf_set_posterior_values": (None, [C.c_int, PD, PD, PD, PD, PD, PI]),
        "rlf_marginalise_posterior_r": (D, [C.c_int, PD, PD]),
        "rlf_marf": (D, [D, C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


EXPORTED = [
    "rlf_version", "rlf_device_count", "rlf_launch_count", "rlf_fp32_peak_gflops", "rlf_configure", "rlf_release",
    "rlf_transfer_bytes", "rlf_obs_create", "rlf_obs_destroy", "rlf_obs_set_data_ms", "rlf_ms_read_coords",
    "rlf_ms_read_flag", "rlf_ms_read_vis", "rlf_ms_read_sigma2", "rlf_ms_write_vis",
    "rlf_obs_set_vis", "rlf_obs_set_data_c64", "rlf_obs_get_vis", "rlf_obs_simulate",
    "rlf_obs_sky_model", "rlf_obs_snapshot", "rlf_obs_restore", "rlf_obs_process",
    "rlf_obs_last_timing", "rlf_obs_last_stats", "rlf_obs_extract", "rlf_debug_fit_trace", "rlf_debug_loglike_nodes", "rlf_debug_df_math", "rlf_gridding_visibilities_noalloc", "facet_size", "evaluate_uv_grid_size", "evaluate_facet_coords",
    "gridding_visibilities", "average_facets", "gaussian_shape", "sersic_shape",
    "model_galaxy_visibilities_at_zero", "data_galaxy_visibilities", "data_visibilities_phase_shift",
    "f_likelihood", "loglikelihood", "loglikelihood_r", "cross_correlation",
    "marginalise_over_position_shift", "likelihood_sampling", "source_extraction", "source_fitting",
    "data_processing", "sky_model", "rfunc", "scale_mean", "rlf_set_posterior_values",
    "rlf_marginalise_posterior_r", "rlf_marf", "rlf_obs_facet_partials", "rlf_fit_partials", "rlf_obs_remove",
    "rlf_cnn_param_count", "rlf_cnn_create", "rlf_cnn_destroy",
    "rlf_cnn_set_params", "rlf_cnn_get_params", "rlf_cnn_store_facets", "rlf_cnn_set_targets",
    "rlf_cnn_read_images", "rlf_cnn_set_images", "rlf_cnn_grads", "rlf_cnn_train_step", "rlf_cnn_predict", "rlf_proposal_set_params",
    "rlf_proposal_set_max_sigma",
]
