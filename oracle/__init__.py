"""CPU oracle for the PTP geodesics path -- TEST INFRASTRUCTURE ONLY.

Two checkers live here:

* ``liboracle.so`` -- the project's plain-C restatement of the reference
  algorithm (``ptp_oracle.c``), built on any machine;
* ``_ref/libref_f64.so`` / ``_ref/libref_f32.so`` -- the reference's own CPU code
  (src/che.cpp, src/geodesics_ptp.cpp, ...) compiled where it lies, built only
  where the reference checkout is present (``make ref``).

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this package.  The product path (``gproshan_gb300``) never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NIL = 0xFFFFFFFF
PTP_TOL = 1e-3

_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


STAGED_REF = os.path.join(HERE, "..", "baseline", "_ref")


def reference_sources() -> str | None:
    """Where the reference's CPU sources are: a checkout named by the
    GPROSHAN_REF environment variable, else the staged copy under
    baseline/_ref/ (see the Makefile's ``stage`` target), else None."""
    env = os.environ.get("GPROSHAN_REF")
    for d in (env, STAGED_REF):
        if d and os.path.isfile(os.path.join(d, "src", "geodesics_ptp.cpp")):
            return os.path.abspath(d)
    return None


def build(ref: bool | None = None, ref_dir: str | None = None) -> None:
    """Compile the oracle and, when the reference's sources are at hand
    (``ref_dir``, GPROSHAN_REF or the staged copy), the reference's own CPU
    code into _ref/.  With GPROSHAN_REF set -- or, without a staged copy, with
    the Makefile's default checkout present -- its sources are first staged
    into baseline/_ref/ so that they travel with the working tree."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    env = os.environ.get("GPROSHAN_REF")
    if env and os.path.isfile(os.path.join(env, "src", "geodesics_ptp.cpp")):
        subprocess.run(["make", "-s", "-C", HERE, "stage", f"GPROSHAN_REF={env}"], check=True)
    elif not os.path.isfile(os.path.join(STAGED_REF, "src", "geodesics_ptp.cpp")):
        # no staged copy: stage from the recipe's default checkout if there is one
        subprocess.run(["make", "-s", "-C", HERE, "stage"], capture_output=True)
    src = ref_dir or reference_sources()
    if ref is None:
        ref = src is not None
    if ref and src:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={src}"], check=True)


def build_ref_gpu() -> str:
    """Compile _ref/libref_gpu_f64.so: the reference's own GPU PTP (sm_103a)
    with its CPU che, from the reference sources (see reference_sources()).
    Returns its path.  It resets the device on every call: load it only in a
    process that uses no other GPU code."""
    src = reference_sources()
    if src is None:
        raise FileNotFoundError("reference sources not present (GPROSHAN_REF or the staged copy)")
    subprocess.run(["make", "-s", "-C", HERE, "ref_gpu", f"REF={src}"], check=True)
    return os.path.join(HERE, "_ref", "libref_gpu_f64.so")


class RefGpuLib:
    """ctypes view of _ref/libref_gpu_f64.so (ref_wrap.cpp built with REF_GPU)."""

    def __init__(self, path: str):
        L = C.CDLL(path)
        self.create = L.refg_f64_che_create
        self.create.restype = C.c_void_p
        self.create.argtypes = [_f64p, C.c_uint, _u32p, C.c_uint]
        self.free = L.refg_f64_che_free
        self.free.argtypes = [C.c_void_p]
        self.geod = L.refg_f64_geodesics_ptp_gpu
        self.geod.restype = C.c_double
        self.geod.argtypes = [C.c_void_p, _u32p, C.c_uint, _f64p]


class _OrcInfo(C.Structure):
    _fields_ = [("n_iter", C.c_uint32), ("last", C.c_uint32), ("relaxations", C.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.orc_che_build.restype = C.c_int
        L.orc_che_build.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p, _u32p]
        L.orc_toplesets.restype = C.c_uint32
        L.orc_toplesets.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p, _u32p, _u32p, C.c_uint32,
                                    _u32p, _u32p, C.c_uint32, _u32p, C.c_uint32]
        L.orc_update_step.restype = C.c_double
        L.orc_update_step.argtypes = [_f64p, _u32p, _f64p, C.c_uint32]
        L.orc_ptp.restype = _OrcInfo
        L.orc_ptp.argtypes = [C.c_uint32, _f64p, _u32p, _u32p, _u32p, _u32p, C.c_uint32,
                              _u32p, C.c_uint32, _u32p, _f64p, _f64p, C.c_void_p, C.c_void_p,
                              C.c_void_p, C.c_uint32, C.c_int]
        L.orc_ptp_replay.restype = _OrcInfo
        L.orc_ptp_replay.argtypes = [C.c_uint32, _f64p, _u32p, _u32p, _u32p, _u32p, C.c_uint32,
                                     _u32p, C.c_uint32, _u32p, _u32p, C.c_uint32, _f64p, _f64p,
                                     C.c_int]
        L.orc_normalize_ptp.restype = None
        L.orc_normalize_ptp.argtypes = [_f64p, C.c_uint64]
        L.orc_fps.restype = C.c_uint32
        L.orc_fps.argtypes = [C.c_uint32, _f64p, _u32p, _u32p, _u32p, _u32p, C.c_uint32, C.c_uint32,
                              C.c_uint64, C.c_double, C.POINTER(C.c_double), C.c_int]
        _lib = L
    return _lib


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


class Mesh:
    """CHE tables of a triangle mesh as built by the oracle (che::update_evt_ot_et)."""

    def __init__(self, xyz, tri):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self.VT = _u32(tri).reshape(-1)
        self.nv = len(self.xyz)
        self.nf = len(self.VT) // 3
        self.OT = np.empty(3 * self.nf, np.uint32)
        self.EVT = np.empty(self.nv, np.uint32)
        self.manifold = lib().orc_che_build(self.nv, self.nf, self.VT, self.OT, self.EVT)
        if self.manifold < 0:
            raise ValueError("triangle references a vertex out of range")


def toplesets(mesh: Mesh, sources):
    """(rings, sorted, limits) exactly as che::compute_toplesets returns them."""
    src = _u32(sources)
    rings = np.empty(mesh.nv, np.uint32)
    sorted_ = np.empty(mesh.nv + len(src), np.uint32)
    limits = np.empty(mesh.nv + 2, np.uint32)
    nl = lib().orc_toplesets(mesh.nv, 3 * mesh.nf, mesh.VT, mesh.OT, mesh.EVT, src, len(src),
                             rings, sorted_, len(sorted_), limits, len(limits))
    if nl == 0:
        raise ValueError("toplesets failed (no sources or source out of range)")
    return rings, sorted_[:limits[nl - 1]].copy(), limits[:nl].copy()


def ptp(mesh: Mesh, sources, limits=None, sorted_=None, xyz=None, clusters=False,
        trace=False, nthreads=0):
    """FP64 PTP with the GPU entry points' schedule.

    Returns a dict with ``dist`` (what parallel_toplesets_propagation_gpu
    returns), ``dist_cpu`` (what the reference CPU entry points return: the
    other Jacobi buffer), ``n_iter``, ``relaxations`` and optionally
    ``clusters`` and ``trace`` ((n_iter, 2) array of (i, j)).
    ``xyz`` overrides the coordinates (e.g. float32-rounded ones)."""
    src = _u32(sources)
    if limits is None:
        _, sorted_, limits = toplesets(mesh, src)
    limits = _u32(limits)
    sorted_ = _u32(sorted_)
    g = mesh.xyz if xyz is None else np.ascontiguousarray(xyz, dtype=np.float64)
    b0 = np.empty(mesh.nv, np.float64)
    b1 = np.empty(mesh.nv, np.float64)
    c0 = c1 = None
    if clusters:
        c0 = np.zeros(mesh.nv, np.uint32)
        c1 = np.zeros(mesh.nv, np.uint32)
    cap = 2 * len(limits) + 2 if trace else 0
    tr = np.zeros(2 * max(cap, 1), np.uint32)
    info = lib().orc_ptp(mesh.nv, g, mesh.VT, mesh.OT, mesh.EVT, src, len(src), limits, len(limits),
                         sorted_, b0, b1,
                         c0.ctypes.data if c0 is not None else None,
                         c1.ctypes.data if c1 is not None else None,
                         tr.ctypes.data if trace else None, cap, nthreads)
    bufs = (b0, b1)
    out = {
        "dist": bufs[info.last],
        "dist_cpu": bufs[1 - info.last],
        "n_iter": info.n_iter,
        "relaxations": int(info.relaxations),
    }
    if clusters:
        out["clusters"] = (c0, c1)[info.last]
    if trace:
        out["trace"] = tr[:2 * info.n_iter].reshape(-1, 2).copy()
    return out


def ptp_replay(mesh: Mesh, sources, limits, sorted_, trace, xyz=None, nthreads=0):
    """FP64 sweeps following a given (i, j) schedule; returns the last buffer."""
    src = _u32(sources)
    g = mesh.xyz if xyz is None else np.ascontiguousarray(xyz, dtype=np.float64)
    b0 = np.empty(mesh.nv, np.float64)
    b1 = np.empty(mesh.nv, np.float64)
    tr = _u32(trace).reshape(-1)
    info = lib().orc_ptp_replay(mesh.nv, g, mesh.VT, mesh.OT, mesh.EVT, src, len(src), _u32(limits),
                                len(limits), _u32(sorted_), tr, len(tr) // 2, b0, b1, nthreads)
    return (b0, b1)[info.last]


def normalize_ptp(dist):
    d = np.ascontiguousarray(dist, dtype=np.float64).copy()
    lib().orc_normalize_ptp(d, len(d))
    return d


def fps(mesh: Mesh, n: int, seeds=(0,), radio: float = 0.0, nthreads=0):
    """farthest_point_sampling_ptp_gpu: returns (samples, max_dist)."""
    cap = max(int(n), len(seeds)) + 1
    s = np.zeros(cap, np.uint32)
    s[:len(seeds)] = seeds
    md = C.c_double(0.0)
    ns = lib().orc_fps(mesh.nv, mesh.xyz, mesh.VT, mesh.OT, mesh.EVT, s, len(seeds), cap, int(n),
                       float(radio), C.byref(md), nthreads)
    return s[:ns].copy(), md.value


def max_rel_err(d, ref):
    """Largest |d - ref| / ref over vertices with 0 < ref < inf; INF/finite
    disagreements count as an infinite error."""
    d = np.asarray(d, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    fin = np.isfinite(ref)
    if np.any(np.isfinite(d) != fin):
        return float("inf")
    m = fin & (ref > 0)
    if not np.any(m):
        return 0.0 if np.array_equal(d[fin], ref[fin]) else float("inf")
    bad0 = fin & (ref == 0) & (d != 0)
    if np.any(bad0):
        return float("inf")
    return float(np.max(np.abs(d[m] - ref[m]) / ref[m]))


# --------------------------------------------------------------------------
# The reference's own compiled CPU code (present only where it was built).
# --------------------------------------------------------------------------

class RefLib:
    """ctypes view of oracle/_ref/libref_{f64,f32}.so (see ref_wrap.cpp)."""

    def __init__(self, precision: str = "f64"):
        path = os.path.join(HERE, "_ref", f"libref_{precision}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.prec = precision
        self.real = np.float64 if precision == "f64" else np.float32
        rp = _f64p if precision == "f64" else _f32p
        L = C.CDLL(path)
        p = f"refw_{precision}_"
        self.create = getattr(L, p + "che_create")
        self.create.restype = C.c_void_p
        self.create.argtypes = [_f64p, C.c_uint, _u32p, C.c_uint]
        self.free = getattr(L, p + "che_free")
        self.free.argtypes = [C.c_void_p]
        self.nhe = getattr(L, p + "che_n_half_edges")
        self.nhe.restype = C.c_uint
        self.nhe.argtypes = [C.c_void_p]
        self.tables = getattr(L, p + "che_tables")
        self.tables.argtypes = [C.c_void_p, _u32p, _u32p, _u32p]
        self.tops = getattr(L, p + "toplesets")
        self.tops.restype = C.c_uint
        self.tops.argtypes = [C.c_void_p, _u32p, C.c_uint, _u32p, _u32p, C.c_uint, _u32p, C.c_uint]
        self.ptp_cpu = getattr(L, p + "ptp_cpu")
        self.ptp_cpu.argtypes = [C.c_void_p, _u32p, C.c_uint, _u32p, C.c_uint, _u32p, rp,
                                 C.c_void_p, C.c_int]
        self.upd = getattr(L, p + "update_step")
        self.upd.restype = C.c_double if precision == "f64" else C.c_float
        self.upd.argtypes = [C.c_void_p, rp, C.c_uint]
        self.geod = getattr(L, p + "geodesics_ptp_cpu")
        self.geod.restype = C.c_uint
        self.geod.argtypes = [C.c_void_p, _u32p, C.c_uint, rp]
        self.norm = getattr(L, p + "normalize_ptp")
        self.norm.argtypes = [rp, C.c_ulonglong]
        self.off_open = getattr(L, p + "off_open")
        self.off_open.restype = C.c_void_p
        self.off_open.argtypes = [C.c_char_p]
        self.nv = getattr(L, p + "che_n_vertices")
        self.nv.restype = C.c_uint
        self.nv.argtypes = [C.c_void_p]
        self.xyz = getattr(L, p + "che_xyz")
        self.xyz.argtypes = [C.c_void_p, _f64p]

    def read_off(self, path: str):
        """(xyz, VT, OT, EVT) of an OFF file read by the reference's che_off."""
        h = self.off_open(path.encode())
        try:
            nv, nhe = self.nv(h), self.nhe(h)
            xyz = np.empty(3 * nv, np.float64)
            VT = np.empty(nhe, np.uint32)
            OT = np.empty(nhe, np.uint32)
            EVT = np.empty(nv, np.uint32)
            self.xyz(h, xyz)
            self.tables(h, VT, OT, EVT)
        finally:
            self.free(h)
        return xyz.reshape(-1, 3), VT, OT, EVT


class RefMesh:
    """A reference ``che`` built by the reference's own constructor."""

    def __init__(self, reflib: RefLib, xyz, tri):
        self.L = reflib
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self.tri = _u32(tri).reshape(-1)
        self.nv = len(self.xyz)
        self.nf = len(self.tri) // 3
        self.h = reflib.create(self.xyz.reshape(-1), self.nv, self.tri, self.nf)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.free(self.h)
            self.h = None

    def tables(self):
        nhe = self.L.nhe(self.h)
        VT = np.empty(nhe, np.uint32)
        OT = np.empty(nhe, np.uint32)
        EVT = np.empty(self.nv, np.uint32)
        self.L.tables(self.h, VT, OT, EVT)
        return VT, OT, EVT

    def toplesets(self, sources):
        src = _u32(sources)
        rings = np.empty(self.nv, np.uint32)
        srt = np.empty(self.nv + len(src), np.uint32)
        lim = np.empty(self.nv + 2, np.uint32)
        nl = self.L.tops(self.h, src, len(src), rings, srt, len(srt), lim, len(lim))
        if nl == 0:
            raise ValueError("reference toplesets failed")
        return rings, srt[:lim[nl - 1]].copy(), lim[:nl].copy()

    def ptp_cpu(self, sources, limits, sorted_, coalescence=False, clusters=None):
        src = _u32(sources)
        dist = np.empty(self.nv, self.L.real)
        cl = None
        if clusters is not None:
            cl = np.ascontiguousarray(clusters, dtype=np.uint32).copy()
        self.L.ptp_cpu(self.h, src, len(src), _u32(limits), len(limits), _u32(sorted_), dist,
                       cl.ctypes.data if cl is not None else None, int(coalescence))
        return (dist, cl) if clusters is not None else dist

    def geodesics_ptp_cpu(self, sources, out=None):
        """One field as geodesics(mesh, sources, PTP_CPU) computes it:
        toplesets + the coalescence CPU PTP (the reference's CPU timing unit)."""
        src = _u32(sources)
        dist = np.empty(self.nv, self.L.real) if out is None else out
        self.L.geod(self.h, src, len(src), dist)
        return dist

    def update_step(self, dist, he):
        return self.L.upd(self.h, np.ascontiguousarray(dist, dtype=self.L.real), he)
