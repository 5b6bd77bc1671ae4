"""GB300-native Parallel Toplesets Propagation (PTP) geodesics.

A drop-in for gproshan's PTP_GPU path: the same geodesics API
(``geodesics.PTP_GPU``, ``parallel_toplesets_propagation_gpu``, ``ptp_out_t``,
``toplesets_t``) over hand-written sm_103a CUDA in ``libgp_ptp.so``, reached
through the C ABI declared in ``include/gp_ptp.h``.
"""
from .che import che, che_off, NIL
from .geodesics import (
    PTP_TOL,
    farthest_point_sampling_ptp_gpu,
    geodesics,
    normalize_ptp,
    parallel_toplesets_propagation_coalescence_gpu,
    parallel_toplesets_propagation_gpu,
    ptp_out_t,
    toplesets_t,
)
from . import _capi as capi

__all__ = [
    "che", "che_off", "NIL", "PTP_TOL", "geodesics", "ptp_out_t", "toplesets_t",
    "parallel_toplesets_propagation_gpu", "parallel_toplesets_propagation_coalescence_gpu",
    "farthest_point_sampling_ptp_gpu", "normalize_ptp", "capi",
]
