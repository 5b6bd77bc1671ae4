"""ctypes binding of libgp_ptp.so (the C ABI declared in include/gp_ptp.h).

The library is built in-tree by ``gproshan_gb300.build``.  There is no
fallback: if the shared library is missing or no GB300 is visible, every
call raises.
"""
from __future__ import annotations

import atexit
import ctypes as C
import os
import threading
import weakref

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgp_ptp.so")

GP_OK = 0
GP_ERR_INVALID_ARG = 1
GP_ERR_DEVICE_TIMEOUT = 4
GP_ERR_CAPACITY = 8
GP_F32 = 0
GP_F64 = 1
GP_BATCH_DEVICE_POINTERS = 1
NIL = 0xFFFFFFFF

STATUS = {
    0: "GP_OK", 1: "GP_ERR_INVALID_ARG", 2: "GP_ERR_NONMANIFOLD", 3: "GP_ERR_NO_CONVERGENCE",
    4: "GP_ERR_DEVICE_TIMEOUT", 5: "GP_ERR_CUDA", 6: "GP_ERR_NO_DEVICE", 7: "GP_ERR_OUT_OF_MEMORY",
    8: "GP_ERR_CAPACITY",
}


class GPError(RuntimeError):
    """A libgp_ptp call returned a status other than GP_OK."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {message}")


class gp_ptp_opts(C.Structure):
    _fields_ = [("precision", C.c_uint32), ("max_iter", C.c_uint32), ("tol", C.c_double),
                ("threads", C.c_uint32), ("ctas", C.c_uint32), ("local_window", C.c_uint32),
                ("round_coords", C.c_uint32), ("schedule", C.c_uint32), ("grid_kernel", C.c_uint32),
                ("queue_min", C.c_uint32), ("queue_tile", C.c_uint32), ("normalize", C.c_uint32),
                ("stream_min", C.c_uint32)]


class gp_ptp_stats(C.Structure):
    _fields_ = [("n_iter", C.c_uint32), ("n_limits", C.c_uint32), ("relaxations", C.c_uint64),
                ("seconds", C.c_double)]


class gp_call_stats(C.Structure):
    _fields_ = [("launches", C.c_uint32), ("n_fields", C.c_uint32), ("fields_grid", C.c_uint32),
                ("sweeps_grid", C.c_uint32), ("grid_kernel", C.c_uint32),
                ("fields_streamed", C.c_uint32), ("ms_toplesets", C.c_double), ("ms_renumber", C.c_double),
                ("ms_local", C.c_double), ("ms_grid", C.c_double), ("ms_gather", C.c_double),
                ("relax_local", C.c_uint64), ("relax_grid", C.c_uint64), ("h2d_bytes", C.c_uint64),
                ("d2h_bytes", C.c_uint64), ("skip_grid", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class gp_field(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("sources", C.c_void_p), ("n_sources", C.c_uint32),
                ("dist", C.c_void_p), ("clusters", C.c_void_p), ("stats", C.c_void_p)]


# every symbol declared in include/gp_ptp.h, with (restype, argtypes)
_u32p = C.POINTER(C.c_uint32)
SIGNATURES = {
    "gp_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "gp_ctx_destroy": (None, [C.c_void_p]),
    "gp_ctx_last_error": (C.c_char_p, [C.c_void_p]),
    "gp_status_str": (C.c_char_p, [C.c_int]),
    "gp_ctx_stream": (C.c_void_p, [C.c_void_p]),
    "gp_ctx_workspace_bytes": (C.c_size_t, [C.c_void_p]),
    "gp_ctx_valid": (C.c_int, [C.c_void_p]),
    "gp_ctx_device_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "gp_che_build": (C.c_int, [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.POINTER(C.c_int)]),
    "gp_mesh_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.POINTER(C.c_void_p)]),
    "gp_mesh_destroy": (None, [C.c_void_p]),
    "gp_mesh_n_vertices": (C.c_uint32, [C.c_void_p]),
    "gp_mesh_n_faces": (C.c_uint32, [C.c_void_p]),
    "gp_toplesets": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                               C.c_uint32, C.c_void_p, C.c_uint32, _u32p]),
    "gp_ptp": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                         C.c_void_p, C.POINTER(gp_ptp_opts), C.c_void_p, C.c_int, C.c_void_p,
                         C.POINTER(gp_ptp_stats)]),
    "gp_ptp_batch": (C.c_int, [C.c_void_p, C.POINTER(gp_field), C.c_uint32, C.POINTER(gp_ptp_opts),
                               C.c_int, C.c_uint32, C.POINTER(C.c_double)]),
    "gp_normalize_ptp": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_uint64]),
    "gp_ctx_call_stats": (C.c_int, [C.c_void_p, C.POINTER(gp_call_stats)]),
    "gp_ctx_step_trace": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_uint32)]),
    "gp_toplesets_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
                                       C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "gp_mlp_n_params": (C.c_uint32, []),
    "gp_mlp_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                              C.c_void_p]),
    "gp_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                               C.c_float, C.c_void_p]),
    "gp_mlp_infer": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int]),
    "gp_ctx_set_cost_model": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gp_field_features": (C.c_int, [C.c_void_p, C.POINTER(gp_field), C.c_uint32, C.c_void_p]),
    "gp_ptp_autotune": (C.c_int, [C.c_void_p, C.POINTER(gp_field), C.c_uint32, C.c_int, C.c_uint32,
                                  C.POINTER(gp_ptp_opts), C.c_uint32]),
    "gp_plan_create": (C.c_int, [C.c_void_p, C.POINTER(gp_field), C.c_uint32, C.POINTER(gp_ptp_opts), C.c_int,
                                 C.POINTER(C.c_void_p)]),
    "gp_plan_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gp_plan_wait": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(gp_ptp_stats)]),
    "gp_plan_destroy": (None, [C.c_void_p]),
    "gp_off_read": (C.c_int, [C.c_char_p, _u32p, _u32p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
    "gp_mesh_create_off": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "gp_che_build_device": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.POINTER(C.c_int)]),
    "gp_ctx_debug_barrier": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "gp_fps": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64,
                         C.c_double, C.POINTER(gp_ptp_opts), _u32p, C.POINTER(C.c_double),
                         C.POINTER(C.c_double)]),
}

_lib = None
_lock = threading.Lock()
_live_meshes = weakref.WeakSet()
_live_contexts = weakref.WeakSet()
_live_plans = weakref.WeakSet()


@atexit.register
def _release_all():
    # free plans and device meshes, then contexts, while the CUDA runtime is still up
    for p in list(_live_plans):
        p.close()
    for m in list(_live_meshes):
        m.close()
    for c in list(_live_contexts):
        c.close()


def lib():
    """Load libgp_ptp.so (raises if it was not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"{LIB_PATH} is missing: build it with gproshan_gb300.build.build()")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def che_build(n_vertices: int, tri):
    """(OT, EVT, manifold) of a triangle list (host only, no GPU needed)."""
    VT = _u32(tri).reshape(-1)
    nf = len(VT) // 3
    OT = np.empty(3 * nf, np.uint32)
    EVT = np.empty(n_vertices, np.uint32)
    man = C.c_int(0)
    st = lib().gp_che_build(n_vertices, nf, _ptr(VT), _ptr(OT), _ptr(EVT), C.byref(man))
    if st != GP_OK:
        raise GPError(st, "gp_che_build: triangle index out of range")
    return OT, EVT, bool(man.value)


def off_read(path: str):
    """(xyz, tri) of an OFF file (gp_off_read; quads split as the reference does)."""
    nv, nf = C.c_uint32(0), C.c_uint32(0)
    st = lib().gp_off_read(path.encode(), C.byref(nv), C.byref(nf), None, 0, None, 0)
    if st != GP_OK:
        raise GPError(st, f"gp_off_read({path})")
    xyz = np.empty((nv.value, 3), np.float64)
    tri = np.empty((nf.value, 3), np.uint32)
    st = lib().gp_off_read(path.encode(), C.byref(nv), C.byref(nf), _ptr(xyz), nv.value, _ptr(tri), nf.value)
    if st != GP_OK:
        raise GPError(st, f"gp_off_read({path})")
    return xyz, tri


class Context:
    """A gp_ctx: one CUDA stream and a reusable device workspace."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        st = lib().gp_ctx_create(device, C.byref(self._h))
        if st != GP_OK:
            raise GPError(st, f"gp_ctx_create(device={device}) failed")
        self.device = device
        _live_contexts.add(self)

    @property
    def handle(self):
        return self._h

    def check(self, st: int, what: str):
        if st != GP_OK:
            raise GPError(st, f"{what}: {lib().gp_ctx_last_error(self._h).decode()}")

    def workspace_bytes(self) -> int:
        return int(lib().gp_ctx_workspace_bytes(self._h))

    def call_stats(self) -> gp_call_stats:
        cs = gp_call_stats()
        self.check(lib().gp_ctx_call_stats(self._h, C.byref(cs)), "gp_ctx_call_stats")
        return cs

    def device_info(self):
        """(compute capability, binary version of the loaded sweep kernel, SMs)."""
        cc, bv, ns = C.c_int(), C.c_int(), C.c_int()
        self.check(lib().gp_ctx_device_info(self._h, C.byref(cc), C.byref(bv), C.byref(ns)), "gp_ctx_device_info")
        return cc.value, bv.value, ns.value

    def arm_step_trace(self, cap: int):
        self.check(lib().gp_ctx_step_trace(self._h, cap, None, None), "gp_ctx_step_trace")
        self._trace_cap = cap

    def step_trace(self):
        """(t_ns, tiles, live) per step of the last call's grid launch."""
        cap = getattr(self, "_trace_cap", 0)
        out = np.zeros(2 * max(cap, 1), np.uint64)
        n = C.c_uint32(0)
        self.check(lib().gp_ctx_step_trace(self._h, cap, out.ctypes.data_as(C.c_void_p), C.byref(n)),
                   "gp_ctx_step_trace")
        w = out[:2 * n.value].reshape(-1, 2)
        return w[:, 0].astype(np.int64), (w[:, 1] >> np.uint64(32)).astype(np.int64), \
            (w[:, 1] & np.uint64(0xffffffff)).astype(np.int64)

    @property
    def stream(self) -> int:
        return int(lib().gp_ctx_stream(self._h) or 0)

    def close(self):
        if self._h:
            lib().gp_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = {}


def default_context(device: int = 0) -> Context:
    if device not in _default:
        _default[device] = Context(device)
    return _default[device]


class DeviceMesh:
    """A gp_mesh: CHE tables uploaded once, star lists built on the device."""

    def __init__(self, ctx: Context, xyz, VT, OT=None, EVT=None):
        self.ctx = ctx
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        VT = _u32(VT).reshape(-1)
        self.n_vertices = len(xyz)
        self.n_faces = len(VT) // 3
        self._h = C.c_void_p()
        st = lib().gp_mesh_create(ctx.handle, self.n_vertices, _ptr(xyz), self.n_faces, _ptr(VT),
                                  _ptr(None if OT is None else _u32(OT)),
                                  _ptr(None if EVT is None else _u32(EVT)), C.byref(self._h))
        ctx.check(st, "gp_mesh_create")
        _live_meshes.add(self)

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().gp_mesh_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mesh_from_off(ctx: Context, path: str) -> DeviceMesh:
    """gp_mesh_create_off: an OFF file to a device mesh (tables built on the GPU)."""
    m = DeviceMesh.__new__(DeviceMesh)
    m.ctx = ctx
    m._h = C.c_void_p()
    ctx.check(lib().gp_mesh_create_off(ctx.handle, path.encode(), C.byref(m._h)), "gp_mesh_create_off")
    m.n_vertices = int(lib().gp_mesh_n_vertices(m._h))
    m.n_faces = int(lib().gp_mesh_n_faces(m._h))
    _live_meshes.add(m)
    return m


def che_build_device(ctx: Context, n_vertices: int, tri):
    """(OT, EVT, manifold) computed on the GPU (gp_che_build_device)."""
    VT = _u32(tri).reshape(-1)
    nf = len(VT) // 3
    OT = np.empty(3 * nf, np.uint32)
    EVT = np.empty(n_vertices, np.uint32)
    man = C.c_int(0)
    ctx.check(lib().gp_che_build_device(ctx.handle, n_vertices, nf, _ptr(VT), _ptr(OT), _ptr(EVT), C.byref(man)),
              "gp_che_build_device")
    return OT, EVT, bool(man.value)


def toplesets(mesh: DeviceMesh, sources):
    """(rings, sorted, limits) computed on the GPU (gp_toplesets)."""
    src = _u32(sources)
    nv = mesh.n_vertices
    rings = np.empty(nv, np.uint32)
    srt = np.empty(nv + len(src), np.uint32)
    lim = np.empty(nv + 2, np.uint32)
    nl = C.c_uint32(0)
    st = lib().gp_toplesets(mesh.ctx.handle, mesh.handle, _ptr(src), len(src), _ptr(rings), _ptr(srt),
                            len(srt), _ptr(lim), len(lim), C.byref(nl))
    mesh.ctx.check(st, "gp_toplesets")
    lim = lim[:nl.value].copy()
    return rings, srt[:lim[-1]].copy() if len(lim) else srt[:0].copy(), lim


GP_SCHED_REACTIVE = 0
GP_SCHED_LEARNED = 1


GP_GRID_AUTO = 0
GP_GRID_LOCKSTEP = 1
GP_GRID_QUEUE = 2


def make_opts(precision: int = GP_F32, max_iter: int = 0, tol: float = 0.0, ctas: int = 0,
              local_window: int = 0, round_coords: bool = False, schedule: int = GP_SCHED_REACTIVE,
              grid_kernel: int = GP_GRID_AUTO, queue_min: int = 0, queue_tile: int = 0,
              normalize: bool = False, stream_min: int = 0) -> gp_ptp_opts:
    o = gp_ptp_opts()
    o.stream_min = stream_min
    o.normalize = int(bool(normalize))
    o.queue_tile = queue_tile
    o.schedule = schedule
    o.grid_kernel = grid_kernel
    o.queue_min = queue_min
    o.round_coords = int(bool(round_coords))
    o.precision = precision
    o.max_iter = max_iter
    o.tol = tol
    o.ctas = ctas
    o.local_window = local_window
    return o


def ptp(mesh: DeviceMesh, sources, limits=None, sorted_=None, dtype=np.float32, precision=None,
        clusters=None, opts: gp_ptp_opts | None = None):
    """Distances (and labels if ``clusters`` is an initial label array) on the GPU.
    Returns (dist, clusters_or_None, stats)."""
    src = _u32(sources)
    out_t = GP_F64 if np.dtype(dtype) == np.float64 else GP_F32
    if opts is None:
        opts = make_opts(GP_F32 if precision is None else precision)
    elif precision is not None:
        opts.precision = precision
    dist = np.empty(mesh.n_vertices, dtype=np.float64 if out_t == GP_F64 else np.float32)
    cl = None if clusters is None else _u32(clusters).copy()
    lim = None if limits is None else _u32(limits)
    srt = None if sorted_ is None else _u32(sorted_)
    stats = gp_ptp_stats()
    st = lib().gp_ptp(mesh.ctx.handle, mesh.handle, _ptr(src), len(src), _ptr(lim),
                      0 if lim is None else len(lim), _ptr(srt), C.byref(opts), _ptr(dist), out_t, _ptr(cl),
                      C.byref(stats))
    mesh.ctx.check(st, "gp_ptp")
    return dist, cl, stats


def ptp_batch(ctx: Context, meshes, sources_list, dtype=np.float32, precision=GP_F32, ctas: int = 0,
              with_stats: bool = True, local_window: int = 0, round_coords: bool = False,
              schedule: int = GP_SCHED_REACTIVE, grid_kernel: int = GP_GRID_AUTO, queue_min: int = 0,
              queue_tile: int = 0, clusters=None, stream_min: int = 0):
    """Solve many fields together (host arrays).  Returns (dists, stats, seconds).
    ``clusters``: optional list of per-field uint32 label arrays (initial labels
    in, labels out, updated in place)."""
    n = len(sources_list)
    out_t = GP_F64 if np.dtype(dtype) == np.float64 else GP_F32
    fields = (gp_field * n)()
    keep = []
    dists = []
    stats = [gp_ptp_stats() for _ in range(n)]
    for k in range(n):
        src = _u32(sources_list[k])
        d = np.empty(meshes[k].n_vertices, dtype=np.float64 if out_t == GP_F64 else np.float32)
        keep.append(src)
        dists.append(d)
        fields[k].mesh = meshes[k].handle
        fields[k].sources = src.ctypes.data
        fields[k].n_sources = len(src)
        fields[k].dist = d.ctypes.data
        fields[k].clusters = None
        if clusters is not None and clusters[k] is not None:
            lab = clusters[k]
            if lab.dtype != np.uint32 or not lab.flags.c_contiguous or len(lab) != meshes[k].n_vertices:
                raise ValueError("clusters[k] must be a contiguous uint32 array of n_vertices labels")
            fields[k].clusters = lab.ctypes.data
        fields[k].stats = C.addressof(stats[k]) if with_stats else None
    sec = C.c_double(0)
    opts = make_opts(precision, ctas=ctas, local_window=local_window, round_coords=round_coords,
                     schedule=schedule, grid_kernel=grid_kernel, queue_min=queue_min, queue_tile=queue_tile,
                     stream_min=stream_min)
    st = lib().gp_ptp_batch(ctx.handle, fields, n, C.byref(opts), out_t, 0, C.byref(sec))
    ctx.check(st, "gp_ptp_batch")
    return dists, stats, sec.value


def normalize_ptp(ctx: Context, dist):
    d = np.ascontiguousarray(dist)
    t = GP_F64 if d.dtype == np.float64 else GP_F32
    st = lib().gp_normalize_ptp(ctx.handle, _ptr(d), t, len(d))
    ctx.check(st, "gp_normalize_ptp")
    return d


def fps(mesh: DeviceMesh, n: int, seeds=(0,), radio: float = 0.0, precision=GP_F32):
    """farthest_point_sampling_ptp_gpu: (samples, max_dist, seconds)."""
    cap = max(int(n), len(seeds)) + 1
    s = np.zeros(cap, np.uint32)
    s[:len(seeds)] = seeds
    n_out = C.c_uint32(0)
    md = C.c_double(0)
    sec = C.c_double(0)
    opts = make_opts(precision)
    st = lib().gp_fps(mesh.ctx.handle, mesh.handle, _ptr(s), len(seeds), cap, int(n), float(radio),
                      C.byref(opts), C.byref(n_out), C.byref(md), C.byref(sec))
    mesh.ctx.check(st, "gp_fps")
    return s[:n_out.value].copy(), md.value, sec.value


# ---- sweep-cost model (3-layer MLP) ----------------------------------------
MLP_IN = 16


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def mlp_n_params() -> int:
    return int(lib().gp_mlp_n_params())


def mlp_grad(ctx: Context, X, T, params):
    """(grads, loss) of the mean squared error, FP32 kernels."""
    X, T, p = _f32(X), _f32(T), _f32(params)
    g = np.empty(mlp_n_params(), np.float32)
    loss = C.c_float(0)
    ctx.check(lib().gp_mlp_grad(ctx.handle, _ptr(X), _ptr(T), len(X), _ptr(p), _ptr(g), C.byref(loss)),
              "gp_mlp_grad")
    return g, float(loss.value)


def mlp_train(ctx: Context, X, T, params, epochs: int, lr: float):
    """Full-batch Adam on the GPU; returns (params, losses)."""
    X, T = _f32(X), _f32(T)
    p = _f32(params).copy()
    losses = np.empty(epochs, np.float32)
    ctx.check(lib().gp_mlp_train(ctx.handle, _ptr(X), _ptr(T), len(X), _ptr(p), epochs, float(lr),
                                 _ptr(losses)), "gp_mlp_train")
    return p, losses


def mlp_infer(ctx: Context, X, params, bf16: bool = True):
    X, p = _f32(X), _f32(params)
    Y = np.empty((len(X), 2), np.float32)
    ctx.check(lib().gp_mlp_infer(ctx.handle, _ptr(X), len(X), _ptr(p), _ptr(Y), int(bool(bf16))),
              "gp_mlp_infer")
    return Y


def set_cost_model(ctx: Context, params):
    p = None if params is None else _f32(params)
    ctx.check(lib().gp_ctx_set_cost_model(ctx.handle, _ptr(p)), "gp_ctx_set_cost_model")


def field_features(ctx: Context, meshes, sources_list):
    """features[n][MLP_IN] of each field (toplesets on the GPU, no sweep)."""
    n = len(sources_list)
    fields = (gp_field * n)()
    keep = []
    for k in range(n):
        src = _u32(sources_list[k])
        keep.append(src)
        fields[k].mesh = meshes[k].handle
        fields[k].sources = src.ctypes.data
        fields[k].n_sources = len(src)
    out = np.empty((n, MLP_IN), np.float32)
    ctx.check(lib().gp_field_features(ctx.handle, fields, n, _ptr(out)), "gp_field_features")
    return out


# ---- autotuner and CUDA-graph plans -------------------------------------------

def _fields(meshes, sources, dists):
    """gp_field array from raw pointers (ints) or host arrays."""
    n = len(meshes)
    fields = (gp_field * n)()
    keep = []
    for k in range(n):
        src = sources[k]
        if isinstance(src, tuple) and len(src) == 2 and isinstance(src[0], int) and src[0] > 0xFFFFFFFF:
            fields[k].sources, fields[k].n_sources = src  # (device pointer, count)
        else:
            src = _u32(src)
            keep.append(src)
            fields[k].sources = src.ctypes.data
            fields[k].n_sources = len(src)
        d = dists[k]
        fields[k].dist = d.ctypes.data if isinstance(d, np.ndarray) else d
        fields[k].mesh = meshes[k].handle
    return fields, keep


def autotune(ctx: Context, meshes, sources_list, dtype=np.float32, opts: gp_ptp_opts | None = None, reps: int = 2):
    """Best gp_ptp_opts for this batch (host arrays); see gp_ptp_autotune."""
    out_t = GP_F64 if np.dtype(dtype) == np.float64 else GP_F32
    dists = [np.empty(m.n_vertices, dtype=np.float64 if out_t == GP_F64 else np.float32) for m in meshes]
    fields, keep = _fields(meshes, sources_list, dists)
    o = make_opts(GP_F64 if out_t == GP_F64 else GP_F32) if opts is None else opts
    ctx.check(lib().gp_ptp_autotune(ctx.handle, fields, len(meshes), out_t, 0, C.byref(o), reps), "gp_ptp_autotune")
    return o


class Plan:
    """A batched call captured in a CUDA graph (gp_plan_*).  ``sources`` are
    (device pointer, count) pairs and ``dists`` device pointers that stay valid
    while the plan lives."""

    def __init__(self, ctx: Context, meshes, sources, dists, opts: gp_ptp_opts | None = None, dtype=np.float32):
        self.ctx = ctx
        self._h = C.c_void_p()
        out_t = GP_F64 if np.dtype(dtype) == np.float64 else GP_F32
        fields, _ = _fields(meshes, sources, dists)
        o = make_opts(GP_F64 if out_t == GP_F64 else GP_F32) if opts is None else opts
        ctx.check(lib().gp_plan_create(ctx.handle, fields, len(meshes), C.byref(o), out_t, C.byref(self._h)),
                  "gp_plan_create")
        self.n = len(meshes)
        _live_plans.add(self)

    def launch(self, stream: int = 0):
        self.ctx.check(lib().gp_plan_launch(self._h, C.c_void_p(stream or None)), "gp_plan_launch")

    def wait(self, stream: int = 0):
        stats = (gp_ptp_stats * self.n)()
        self.ctx.check(lib().gp_plan_wait(self._h, C.c_void_p(stream or None), stats), "gp_plan_wait")
        return list(stats)

    def close(self):
        if self._h:
            lib().gp_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
