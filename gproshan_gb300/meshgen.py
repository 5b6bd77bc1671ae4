"""Seeded synthetic triangle meshes for the PTP geodesics workloads.

Every generator returns ``(xyz, tri)``: ``xyz`` is a float64 ``(n_v, 3)`` array and
``tri`` a uint32 ``(n_f, 3)`` array of consistently oriented triangles.  The meshes
stand in for the ``.off`` files the reference's geodesics harness reads
(src/test_geodesics_ptp.cpp:44-64), which are not distributed with it.

Workloads (sizes as used by the tests and the benchmark):

* icosphere: unit icosahedron, midpoint-subdivided ``level`` times and re-projected
  to radius 1 (level 6: 40,962 vertices, 81,920 faces), vertices jittered
  tangentially by seeded uniform noise of ``jitter`` x mean edge length;
* height field: ``n x n`` grid on the unit square, two triangles per cell,
  ``z = sum of 8 seeded sinusoids`` of amplitude 0.05 and frequencies 1-16;
* torus: R=1, r=0.3, anisotropic sampling along the major circle;
* bumps: height field of seeded Gaussian bumps with a fraction of vertices
  displaced along the normal.
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "icosphere",
    "height_field",
    "torus",
    "bump_field",
    "batch_mix",
    "mean_edge",
]


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array(
        [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
         [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(
        [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
         [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
         [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
         [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v, f


def _subdivide(v, f):
    """One midpoint subdivision; new vertices are re-projected to the unit sphere."""
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
    e.sort(axis=1)
    key = e[:, 0] * (len(v) + 1) + e[:, 1]
    uniq, inv = np.unique(key, return_inverse=True)
    a = uniq // (len(v) + 1)
    b = uniq % (len(v) + 1)
    mid = v[a] + v[b]
    mid /= np.linalg.norm(mid, axis=1, keepdims=True)
    nf = len(f)
    m01 = inv[:nf] + len(v)
    m12 = inv[nf:2 * nf] + len(v)
    m20 = inv[2 * nf:] + len(v)
    f2 = np.concatenate([
        np.stack([f[:, 0], m01, m20], 1),
        np.stack([f[:, 1], m12, m01], 1),
        np.stack([f[:, 2], m20, m12], 1),
        np.stack([m01, m12, m20], 1),
    ], axis=0)
    return np.concatenate([v, mid], axis=0), f2


def mean_edge(xyz, tri):
    """Mean length over the unique undirected edges (che::mean_edge, src/che.cpp:334-343)."""
    tri = np.asarray(tri, dtype=np.int64)
    e = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]], axis=0)
    e.sort(axis=1)
    e = np.unique(e, axis=0)
    return float(np.linalg.norm(xyz[e[:, 0]] - xyz[e[:, 1]], axis=1).mean())


def icosphere(level: int = 6, jitter: float = 0.1, seed: int = 0):
    """Unit icosphere subdivided ``level`` times, tangentially jittered, on radius 1."""
    v, f = _icosahedron()
    for _ in range(level):
        v, f = _subdivide(v, f)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        me = mean_edge(v, f)
        # two tangent axes per vertex
        ref = np.where(np.abs(v[:, 2:3]) < 0.9, np.array([[0.0, 0.0, 1.0]]), np.array([[1.0, 0.0, 0.0]]))
        t1 = np.cross(v, ref)
        t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
        t2 = np.cross(v, t1)
        u = rng.uniform(-1.0, 1.0, size=(len(v), 2)) * (jitter * me)
        v = v + u[:, :1] * t1 + u[:, 1:] * t2
        v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v.astype(np.float64), f.astype(np.uint32)


def _grid_faces(nr: int, nc: int):
    r, c = np.meshgrid(np.arange(nr - 1), np.arange(nc - 1), indexing="ij")
    a = (r * nc + c).ravel()
    b = a + 1
    d = a + nc
    e = d + 1
    t1 = np.stack([a, b, e], 1)
    t2 = np.stack([a, e, d], 1)
    f = np.empty((2 * len(a), 3), dtype=np.int64)
    f[0::2] = t1
    f[1::2] = t2
    return f.astype(np.uint32)


def height_field(n: int = 2048, seed: int = 0, n_waves: int = 8, amp: float = 0.05,
                 fmin: float = 1.0, fmax: float = 16.0, cols: int | None = None):
    """``n x n`` grid on [0,1]^2 (``n x cols`` on [0,cols/n]x[0,1] when ``cols`` is
    given: a strip), z = sum of ``n_waves`` seeded sinusoids."""
    rng = np.random.default_rng(seed)
    fx = rng.uniform(fmin, fmax, n_waves) * rng.choice([-1.0, 1.0], n_waves)
    fy = rng.uniform(fmin, fmax, n_waves) * rng.choice([-1.0, 1.0], n_waves)
    ph = rng.uniform(0.0, 2.0 * np.pi, n_waves)
    nc = n if cols is None else int(cols)
    u = np.linspace(0.0, 1.0, n)
    uc = u if cols is None else np.arange(nc) / max(n - 1, 1)
    U, V = np.meshgrid(uc, u, indexing="xy")  # row r -> y, column c -> x
    Z = np.zeros_like(U)
    for k in range(n_waves):
        Z += amp * np.sin(2.0 * np.pi * (fx[k] * U + fy[k] * V) + ph[k])
    xyz = np.stack([U.ravel(), V.ravel(), Z.ravel()], 1)
    return xyz.astype(np.float64), _grid_faces(n, nc)


def torus(n_major: int = 400, n_minor: int = 2500, R: float = 1.0, r: float = 0.3,
          warp: float = 0.6, seed: int = 0):
    """Torus sampled anisotropically: edges along the major circle are up to ~20x
    longer than edges along the minor circle, and the major-angle spacing varies
    smoothly (``warp``) around the ring."""
    rng = np.random.default_rng(seed)
    k = np.arange(n_major) / n_major
    ph = rng.uniform(0.0, 2.0 * np.pi)
    # theta(k) monotone with derivative 2*pi*(1 + warp*cos(2*pi*k + ph)) / (1)
    theta = 2.0 * np.pi * k + warp * np.sin(2.0 * np.pi * k + ph) - warp * np.sin(ph)
    phi = 2.0 * np.pi * np.arange(n_minor) / n_minor
    T, P = np.meshgrid(theta, phi, indexing="ij")
    x = (R + r * np.cos(P)) * np.cos(T)
    y = (R + r * np.cos(P)) * np.sin(T)
    z = r * np.sin(P)
    xyz = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)
    # periodic grid faces
    i, j = np.meshgrid(np.arange(n_major), np.arange(n_minor), indexing="ij")
    a = (i * n_minor + j).ravel()
    b = (i * n_minor + (j + 1) % n_minor).ravel()
    d = (((i + 1) % n_major) * n_minor + j).ravel()
    e = (((i + 1) % n_major) * n_minor + (j + 1) % n_minor).ravel()
    f = np.empty((2 * len(a), 3), dtype=np.int64)
    f[0::2] = np.stack([a, d, e], 1)
    f[1::2] = np.stack([a, e, b], 1)
    return xyz.astype(np.float64), f.astype(np.uint32)


def bump_field(n: int = 1414, seed: int = 0, n_bumps: int = 64, displaced: float = 0.05,
               disp_scale: float = 0.2):
    """Grid with seeded Gaussian bumps (sigma in [0.01, 0.1]); a fraction
    ``displaced`` of the vertices is moved along the normal by
    ``disp_scale`` x the grid edge length."""
    rng = np.random.default_rng(seed)
    u = np.linspace(0.0, 1.0, n)
    U, V = np.meshgrid(u, u, indexing="xy")
    Z = np.zeros_like(U)
    cx = rng.uniform(0, 1, n_bumps)
    cy = rng.uniform(0, 1, n_bumps)
    sg = rng.uniform(0.01, 0.1, n_bumps)
    hh = rng.uniform(-0.1, 0.1, n_bumps)
    for k in range(n_bumps):
        Z += hh[k] * np.exp(-((U - cx[k]) ** 2 + (V - cy[k]) ** 2) / (2.0 * sg[k] ** 2))
    xyz = np.stack([U.ravel(), V.ravel(), Z.ravel()], 1)
    h = 1.0 / (n - 1)
    gy, gx = np.gradient(Z, h)
    nrm = np.stack([-gx.ravel(), -gy.ravel(), np.ones(n * n)], 1)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    sel = rng.random(n * n) < displaced
    sgn = rng.choice([-1.0, 1.0], n * n)
    xyz[sel] += (disp_scale * h * sgn[sel])[:, None] * nrm[sel]
    return xyz.astype(np.float64), _grid_faces(n, n)


def batch_mix(n_meshes: int = 64, seed: int = 0, ico_levels=(3, 7), grid_sizes=(64, 1024)):
    """Seeded mix of icospheres (levels in ``ico_levels``) and height-field grids
    (sides in ``grid_sizes``, log-uniform): the many-mesh batched workload.
    Returns a list of ``(name, xyz, tri)``."""
    rng = np.random.default_rng(seed)
    out = []
    for m in range(n_meshes):
        s = int(rng.integers(0, 1 << 30))
        if rng.random() < 0.5:
            lv = int(rng.integers(ico_levels[0], ico_levels[1] + 1))
            xyz, tri = icosphere(lv, 0.1, s)
            out.append((f"ico{lv}_s{s}", xyz, tri))
        else:
            lo, hi = np.log2(grid_sizes[0]), np.log2(grid_sizes[1])
            n = int(round(2.0 ** rng.uniform(lo, hi)))
            xyz, tri = height_field(n, s)
            out.append((f"grid{n}_s{s}", xyz, tri))
    return out
