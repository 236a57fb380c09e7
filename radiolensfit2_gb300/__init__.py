"""GB300-native shape measurement for radio weak lensing: the per-galaxy hot path of
RadioLensfit2 (source extraction, uv faceting, model visibilities, marginalised likelihood,
scalelength marginalisation, simplex and sampling fit) as sm_103a CUDA kernels behind the
reference's own C entry points (include/rlf_reference_abi.h) and a batched, device-resident
API (include/rlf_gb300.h)."""
from . import constants  # noqa: F401

__all__ = ["constants", "synth", "pipeline", "build"]
