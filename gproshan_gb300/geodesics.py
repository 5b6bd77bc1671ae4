"""Host mirror of gproshan's geodesics API for the PTP_GPU path.

Names, argument meanings and return values follow the reference:

* ``PTP_TOL``, ``ptp_out_t``, ``toplesets_t`` (include/geodesics_ptp.h:11-30);
* ``parallel_toplesets_propagation_gpu`` and
  ``parallel_toplesets_propagation_coalescence_gpu``
  (include/geodesics_ptp.h:34-36): fill ``ptp_out.dist`` (and
  ``ptp_out.clusters``) in place and return the elapsed seconds;
* ``farthest_point_sampling_ptp_gpu`` (include/geodesics_ptp.h:42): extends
  ``samples`` in place, returns the last farthest distance (and the time);
* ``normalize_ptp`` (include/geodesics_ptp.h:46);
* class ``geodesics`` with ``option_t`` (include/geodesics.h:19-48).

Everything runs through libgp_ptp.so; there is no CPU code path.
"""
from __future__ import annotations

import enum
import math

import numpy as np

from . import _capi
from .che import che, NIL

PTP_TOL = 1e-3


class ptp_out_t:
    """Output of a PTP call: ``dist`` (n_vertices) and optional ``clusters``."""

    def __init__(self, dist, clusters=None):
        self.dist = dist
        self.clusters = clusters


class toplesets_t:
    """``limits`` (start of each ring, then the end) and ``index`` (the sorted vertices)."""

    def __init__(self, limits, index):
        self.limits = limits
        self.index = index


def _dtype_of(a) -> np.dtype:
    return np.dtype(np.float64) if np.asarray(a).dtype == np.float64 else np.dtype(np.float32)


def _check_out(ptp_out: ptp_out_t, n: int):
    if not isinstance(ptp_out.dist, np.ndarray) or ptp_out.dist.shape != (n,) or not ptp_out.dist.flags.c_contiguous:
        raise ValueError("ptp_out.dist must be a contiguous numpy array of n_vertices elements")
    if ptp_out.dist.dtype not in (np.float32, np.float64):
        raise ValueError("ptp_out.dist must be float32 or float64")
    if ptp_out.clusters is not None:
        c = ptp_out.clusters
        if not isinstance(c, np.ndarray) or c.dtype != np.uint32 or c.shape != (n,):
            raise ValueError("ptp_out.clusters must be a uint32 numpy array of n_vertices elements")


def _run(ptp_out, mesh, sources, toplesets, precision, ctx):
    n = mesh.n_vertices()
    _check_out(ptp_out, n)
    limits = index = None
    if toplesets is not None:
        limits = np.ascontiguousarray(toplesets.limits, dtype=np.uint32)
        index = np.ascontiguousarray(toplesets.index, dtype=np.uint32)[: int(limits[-1])]
    dist, cl, stats = _capi.ptp(mesh.device(ctx), sources, limits, index, dtype=ptp_out.dist.dtype,
                                precision=precision, clusters=ptp_out.clusters)
    ptp_out.dist[:] = dist
    if ptp_out.clusters is not None:
        ptp_out.clusters[:] = cl
    return stats.seconds


def parallel_toplesets_propagation_gpu(ptp_out: ptp_out_t, mesh: che, sources, toplesets: toplesets_t | None,
                                       precision: int = _capi.GP_F32, ctx=None) -> float:
    """PTP from ``sources`` with the caller's toplesets (or GPU-built ones when
    ``toplesets`` is None).  Writes ``ptp_out.dist`` (INF where unreached) and,
    if given, ``ptp_out.clusters`` (source k's region gets k+1; the array's
    values are the initial labels).  Returns device seconds.
    (src/cuda/geodesics_ptp.cu:20-85)"""
    return _run(ptp_out, mesh, sources, toplesets, precision, ctx)


def parallel_toplesets_propagation_coalescence_gpu(ptp_out: ptp_out_t, mesh: che, sources,
                                                   toplesets: toplesets_t | None, set_inf: bool = True,
                                                   precision: int = _capi.GP_F32, ctx=None) -> float:
    """Ring-renumbered PTP (src/cuda/geodesics_ptp_coalescence.cu:21-100).  This
    build always works on the ring-renumbered layout, so this is the same call
    as parallel_toplesets_propagation_gpu; ``set_inf`` is accepted and, like in
    the reference, has no effect."""
    return _run(ptp_out, mesh, sources, toplesets, precision, ctx)


def farthest_point_sampling_ptp_gpu(mesh: che, samples: list, n: int, radio: float = 0.0,
                                    precision: int = _capi.GP_F32, ctx=None):
    """Farthest-point sampling by multi-source PTP
    (src/cuda/geodesics_ptp.cu:87-172).  ``samples`` (a list, at least one
    seed; the reference's loader seeds vertex 0) is extended in place.
    Returns (max_dist, time_fps)."""
    seeds = list(samples) if len(samples) else [0]
    s, md, sec = _capi.fps(mesh.device(ctx), n, seeds, radio, precision)
    samples[:] = [int(x) for x in s]
    return md, sec


def normalize_ptp(dist, ctx=None):
    """dist /= max finite dist, in place (src/geodesics_ptp.cpp:264-276)."""
    d = np.ascontiguousarray(dist)
    out = _capi.normalize_ptp(ctx or _capi.default_context(), d.copy())
    dist[:] = out
    return dist


class geodesics:
    """Geodesic distances from a source set (include/geodesics.h:19-78).

    Only the PTP_GPU option is built here; the other options of the reference
    (Fast Marching, heat flow, PTP on the CPU) raise NotImplementedError."""

    class option_t(enum.IntEnum):
        FM = 0
        PTP_GPU = 1
        HEAT_FLOW_GPU = 2
        PTP_CPU = 3
        HEAT_FLOW = 4

    FM = option_t.FM
    PTP_GPU = option_t.PTP_GPU
    HEAT_FLOW_GPU = option_t.HEAT_FLOW_GPU
    PTP_CPU = option_t.PTP_CPU
    HEAT_FLOW = option_t.HEAT_FLOW

    def __init__(self, mesh: che, sources, opt=option_t.FM, e_dist=None, cluster: bool = False,
                 n_iter: int = 0, radio: float = math.inf, precision: int = _capi.GP_F32, ctx=None):
        n = mesh.n_vertices()
        assert n > 0
        self.n_vertices = n
        self.free_dist = e_dist is None
        self.dist = np.full(n, np.inf, dtype=np.float64) if e_dist is None else e_dist
        if not self.free_dist:
            self.dist[:] = np.inf
        self.clusters = np.zeros(n, np.uint32) if cluster else None
        self.sorted_index = np.full(n, NIL, np.uint32)
        self.n_sorted = 0
        assert len(sources) > 0
        if opt != geodesics.PTP_GPU:
            raise NotImplementedError(f"{geodesics.option_t(opt).name} is outside this build (PTP_GPU only)")
        self._run_ptp_gpu(mesh, sources, precision, ctx)

    def _run_ptp_gpu(self, mesh, sources, precision, ctx):
        # geodesics::run_parallel_toplesets_propagation_gpu (src/geodesics.cpp:225-240);
        # n_iter and radio are ignored there too
        rings, srt, limits = mesh.compute_toplesets(sources, ctx=ctx)
        self.sorted_index[: min(len(srt), self.n_vertices)] = srt[: self.n_vertices]
        out = ptp_out_t(self.dist, self.clusters)
        self.time_ptp = parallel_toplesets_propagation_gpu(out, mesh, sources, toplesets_t(limits, srt),
                                                           precision=precision, ctx=ctx)

    def __getitem__(self, i: int):
        return self.dist[i]

    def __call__(self, i: int) -> int:
        return int(self.sorted_index[i])

    def n_sorted_index(self) -> int:
        return self.n_sorted

    def normalize(self):
        """geodesics::normalize (src/geodesics.cpp:75-90): with no FM order,
        normalize_ptp over all vertices."""
        normalize_ptp(self.dist)
