"""Test oracle for the sweep-cost model (test infrastructure only).

The reference has no learned component: gproshan runs a fixed convergence
loop per field (src/cuda/geodesics_ptp.cu:206-229).  This module restates, in
FP64 numpy, what the library's cost model computes, so that the GPU kernels
can be checked:

* ``forward`` / ``grad``: the 3-layer MLP (16 -> 64 -> 64 -> 2, ReLU) with the
  mean squared error over all outputs, and its exact gradient;
* ``field_features``: the 16 per-field features, from the field's toplesets
  (``limits`` as che::compute_toplesets returns them, src/che.cpp:470-505) and
  the mesh's edge/triangle statistics.

Parameter layout (flat float array): W1[16][64] b1[64] W2[64][64] b2[64]
W3[64][2] b3[2].
"""
from __future__ import annotations

import numpy as np

N_IN, N_H, N_OUT = 16, 64, 2
SHAPES = [("W1", (N_IN, N_H)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)),
          ("W3", (N_H, N_OUT)), ("b3", (N_OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = p[o:o + n].reshape(shp)
        o += n
    return out


def pack(d) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SHAPES])


def forward(p, X):
    w = unpack(p)
    X = np.asarray(X, np.float64)
    H1 = np.maximum(X @ w["W1"] + w["b1"], 0.0)
    H2 = np.maximum(H1 @ w["W2"] + w["b2"], 0.0)
    return H2 @ w["W3"] + w["b3"]


def loss(p, X, T):
    Y = forward(p, X)
    return float(np.mean((Y - np.asarray(T, np.float64)) ** 2))


def grad(p, X, T):
    """(gradient, loss) of mean((Y - T)^2) over all n * 2 outputs."""
    w = unpack(p)
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    Z1 = X @ w["W1"] + w["b1"]
    H1 = np.maximum(Z1, 0.0)
    Z2 = H1 @ w["W2"] + w["b2"]
    H2 = np.maximum(Z2, 0.0)
    Y = H2 @ w["W3"] + w["b3"]
    E = Y - T
    dY = 2.0 * E / E.size
    g = {"W3": H2.T @ dY, "b3": dY.sum(0)}
    dH2 = (dY @ w["W3"].T) * (Z2 > 0)
    g["W2"] = H1.T @ dH2
    g["b2"] = dH2.sum(0)
    dH1 = (dH2 @ w["W2"].T) * (Z1 > 0)
    g["W1"] = X.T @ dH1
    g["b1"] = dH1.sum(0)
    return pack(g), float(np.mean(E ** 2))


def init_params(seed: int = 0) -> np.ndarray:
    """He-uniform weights, zero biases."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shp in SHAPES:
        if name.startswith("W"):
            lim = np.sqrt(6.0 / shp[0])
            d[name] = rng.uniform(-lim, lim, shp)
        else:
            d[name] = np.zeros(shp)
    return pack(d)


def mesh_stats(xyz, tri, OT):
    """The five geometry statistics of a mesh: log mean edge length, edge
    length coefficient of variation, std of log edge length, fraction of obtuse
    triangles, mean (1 - cos) of the dihedral angle over interior edges.
    Edges are counted once per triangle side (interior edges twice)."""
    P = np.asarray(xyz, np.float64)[np.asarray(tri, np.int64)]
    E = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 1], P[:, 0] - P[:, 2]], 1)
    q = (E ** 2).sum(-1)
    ln = np.sqrt(q[q > 0])
    mean = ln.mean()
    cv = ln.std() / mean
    glog = np.log(ln).std()
    obt = float(np.mean(2.0 * q.max(1) > q.sum(1)))
    n = np.cross(E[:, 0], E[:, 1])
    nn = np.linalg.norm(n, axis=1)
    OT = np.asarray(OT, np.int64).reshape(-1, 3)
    t = np.repeat(np.arange(len(tri)), 3)
    o = OT.ravel()
    nil = np.uint32(0xFFFFFFFF).astype(np.int64)
    sel = (o != nil) & (o >= 0)
    u = np.where(sel, o // 3, 0)
    sel &= (u >= t) & (nn[t] > 0) & (nn[u] > 0)
    cosang = (n[t[sel]] * n[u[sel]]).sum(1) / (nn[t[sel]] * nn[u[sel]])
    dih = float(np.mean(1.0 - cosang)) if sel.any() else 0.0
    return np.array([np.log(mean), cv, glog, obt, dih])


def field_features(limits, n_vertices: int, n_sources: int, stats):
    """The 16 cost-model features of one field (the library computes them in
    FP32 on the GPU)."""
    lim = np.asarray(limits, np.int64)
    nl = len(lim)
    L = max(nl - 1, 0)
    rings = np.diff(lim) if L else np.zeros(0, np.int64)
    rmax = int(rings.max()) if L else 0
    amax = int(np.argmax(rings)) if L else 0
    bound = max((int(lim[j] - lim[j >> 1]) for j in range(2, nl)), default=0)
    nr = int(lim[-1]) if nl else 0
    Lf = float(max(L, 1))

    def ring(k):
        return float(rings[k]) if k < L else 0.0

    x = np.empty(N_IN)
    x[0] = np.log(max(n_vertices, 1))
    x[1] = np.log(Lf)
    x[2] = np.log(max(n_sources, 1))
    x[3] = np.log(max(rmax, 1))
    x[4] = np.log(max(nr / Lf, 1.0))
    x[5] = amax / Lf
    x[6] = np.log(bound + 1.0)
    x[7] = np.log(ring(L // 4) + 1.0)
    x[8] = np.log(ring(L // 2) + 1.0)
    x[9] = np.log(ring(3 * L // 4) + 1.0)
    x[10:15] = stats
    x[15] = nr / max(n_vertices, 1)
    return x
