"""Learned sweep-cost model for batch scheduling.

gproshan sweeps each field until its toplesets converge
(src/cuda/geodesics_ptp.cu:206-229); how many sweeps that takes, and how many
vertex relaxations, is only known afterwards.  When many fields are solved in
one call (``gp_ptp_batch``), the library runs every field on one CTA and
hands the ones whose windows outgrow a CTA to the grid-wide launch.  With a
cost model installed and ``schedule=GP_SCHED_LEARNED``, it predicts both
numbers from the field's toplesets before the first sweep, starts the fields
expected to outgrow one CTA on the grid launch right away, and takes the
others longest-predicted-first.  Which sweeps run never changes, so the
distances are bit-identical with and without the model.

The model is a 3-layer MLP (16 features -> 64 -> 64 -> 2, ReLU) trained by the
library's own FP32 kernels (``gp_mlp_train``) and evaluated in the batch call
by its BF16 tensor-core kernel.  Targets: ``log(sweeps / rings)`` and
``log(relaxations / vertices)``.  Input standardisation is folded into the
first layer, so the installed parameters take the raw features.

``python -m gproshan_gb300.learned --out gproshan_gb300/cost_model.npz``
regenerates the shipped model (needs a GPU).
"""
from __future__ import annotations

import argparse
import os

import numpy as np

from . import _capi, meshgen

FEATURES = [
    "log_vertices", "log_rings", "log_sources", "log_max_ring", "log_mean_ring", "argmax_ring_frac",
    "log_max_window", "log_ring_q1", "log_ring_mid", "log_ring_q3", "log_mean_edge", "edge_cv",
    "log_edge_std", "obtuse_frac", "dihedral", "reached_frac",
]
N_IN = len(FEATURES)
DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cost_model.npz")


def targets(stats, n_vertices):
    """(T[n][2], mask) from per-field gp_ptp_stats: fields with fewer than
    three toplesets limits run no sweep and are masked out."""
    T = np.zeros((len(stats), 2), np.float32)
    ok = np.zeros(len(stats), bool)
    for k, s in enumerate(stats):
        L = int(s.n_limits) - 1
        if s.n_iter > 0 and L >= 2:
            T[k, 0] = np.log(s.n_iter / L)
            T[k, 1] = np.log(max(s.relaxations, 1) / max(n_vertices[k], 1))
            ok[k] = True
    return T, ok


def fold_standardisation(params, mean, std):
    """Parameters taking raw x from parameters trained on (x - mean) / std."""
    p = np.asarray(params, np.float64).copy()
    W1 = p[:N_IN * 64].reshape(N_IN, 64)
    b1 = p[N_IN * 64:N_IN * 64 + 64]
    W1n = W1 / std[:, None]
    b1n = b1 - (mean / std) @ W1
    p[:N_IN * 64] = W1n.ravel()
    p[N_IN * 64:N_IN * 64 + 64] = b1n
    return p.astype(np.float32)


def init_params(seed: int = 0) -> np.ndarray:
    """He-uniform weights, zero biases (layout W1 b1 W2 b2 W3 b3)."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((N_IN, 64), (64, 64), (64, 2)):
        lim = np.sqrt(6.0 / fan_in)
        parts += [rng.uniform(-lim, lim, fan_in * fan_out), np.zeros(fan_out)]
    return np.concatenate(parts).astype(np.float32)


def fit(ctx, X, T, epochs: int = 4000, lr: float = 3e-3, seed: int = 0):
    """Train on the GPU; returns (params for raw features, losses)."""
    X = np.asarray(X, np.float64)
    mean = X.mean(0)
    std = X.std(0)
    std[std < 1e-6] = 1.0
    Xs = ((X - mean) / std).astype(np.float32)
    p, losses = _capi.mlp_train(ctx, Xs, np.asarray(T, np.float32), init_params(seed), epochs, lr)
    return fold_standardisation(p, mean, std), losses


def save(path, params, **meta):
    np.savez(path, params=np.asarray(params, np.float32), features=np.array(FEATURES), **meta)


def load(path: str = DEFAULT_MODEL) -> np.ndarray:
    with np.load(path) as z:
        p = z["params"].astype(np.float32)
    if len(p) != _capi.mlp_n_params():
        raise ValueError(f"{path}: {len(p)} parameters, the library expects {_capi.mlp_n_params()}")
    return p


def install(ctx, params=None):
    """Install ``params`` (default: the shipped model) as ctx's cost model."""
    _capi.set_cost_model(ctx, load() if params is None else params)


def predict(ctx, features, params, bf16: bool = True):
    return _capi.mlp_infer(ctx, features, params, bf16=bf16)


# ---- training workload --------------------------------------------------------

def training_meshes(seed: int = 0, n: int = 48, families: str = "mixed"):
    """Seeded meshes, one at a time.  ``mixed``: icospheres, height fields,
    strips, tori and bump fields (a few hundred to ~250k vertices);
    ``configs``: the families of the benchmark configurations, icospheres
    subdivided 3-6 times and height fields 64^2-512^2."""
    rng = np.random.default_rng(seed)
    for k in range(n):
        s = int(rng.integers(0, 1 << 30))
        if families == "configs":
            if k % 2 == 0:
                lv = int(rng.integers(3, 7))
                yield (f"ico{lv}", *meshgen.icosphere(lv, 0.1, s))
            else:
                m = int(round(2.0 ** rng.uniform(6, 9)))
                yield (f"grid{m}", *meshgen.height_field(m, s))
            continue
        kind = k % 5
        if kind == 0:
            lv = int(rng.integers(2, 8))
            yield (f"ico{lv}", *meshgen.icosphere(lv, 0.1, s))
        elif kind == 1:
            m = int(round(2.0 ** rng.uniform(4, 9)))
            yield (f"grid{m}", *meshgen.height_field(m, s))
        elif kind == 2:
            w = int(rng.integers(3, 17))
            ln = int(round(2.0 ** rng.uniform(6, 12)))
            yield (f"strip{w}x{ln}", *meshgen.height_field(w, s, cols=ln))
        elif kind == 3:
            a = int(round(2.0 ** rng.uniform(4, 8)))
            b = int(round(2.0 ** rng.uniform(4, 9)))
            yield (f"torus{a}x{b}", *meshgen.torus(a, b, seed=s))
        else:
            m = int(round(2.0 ** rng.uniform(4, 9)))
            yield (f"bump{m}", *meshgen.bump_field(m, s))


def random_sources(rng, nv: int):
    ns = int(min(nv, 2 ** rng.uniform(0, 5)))
    return np.unique(rng.integers(0, nv, ns)).astype(np.uint32)


def collect(ctx, meshes, sources_list):
    """(X, T, mask) over the fields: features from gp_field_features, targets
    from a reactive gp_ptp_batch run."""
    X = _capi.field_features(ctx, meshes, sources_list)
    _, stats, _ = _capi.ptp_batch(ctx, meshes, sources_list)
    T, ok = targets(stats, [m.n_vertices for m in meshes])
    return X, T, ok


def build_dataset(ctx, seed: int = 0, n_meshes: int = 48, fields_per_mesh: int = 16, families: str = "mixed",
                  chunk: int = 32):
    """(X, T, mesh index) of the fields that ran sweeps; meshes are generated,
    uploaded, solved and freed `chunk` at a time."""
    rng = np.random.default_rng(seed + 1)
    Xs, Ts, Gs = [], [], []
    dms, srcs, gid = [], [], []

    def flush():
        if srcs:
            X, T, ok = collect(ctx, dms, srcs)
            Xs.append(X[ok])
            Ts.append(T[ok])
            Gs.append(np.asarray(gid)[ok])
        for m in {id(d): d for d in dms}.values():
            m.close()
        dms.clear()
        srcs.clear()
        gid.clear()

    for g, (_, xyz, tri) in enumerate(training_meshes(seed, n_meshes, families)):
        dm = _capi.DeviceMesh(ctx, xyz, tri)
        for _ in range(fields_per_mesh):
            dms.append(dm)
            srcs.append(random_sources(rng, dm.n_vertices))
            gid.append(g)
        if (g + 1) % chunk == 0:
            flush()
    flush()
    return np.concatenate(Xs), np.concatenate(Ts), np.concatenate(Gs)


def torus_eval(ctx, params):
    """Mean |error| (log-sweeps, log-relaxations) on the 1M-vertex anisotropic
    torus: 16 single-source fields and one field with all 16 sources."""
    xyz, tri = meshgen.torus(400, 2500, seed=0)
    m = _capi.DeviceMesh(ctx, xyz, tri)
    s16 = np.random.default_rng(4).choice(len(xyz), 16, replace=False).astype(np.uint32)
    srcs = [[int(x)] for x in s16] + [s16]
    X, T, ok = collect(ctx, [m] * len(srcs), srcs)
    m.close()
    Y = predict(ctx, X[ok], params)
    return np.abs(Y - T[ok]).mean(0)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=DEFAULT_MODEL)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--config-meshes", type=int, default=2000,
                    help="meshes of the benchmark families (icospheres, height fields)")
    ap.add_argument("--config-fields", type=int, default=4)
    ap.add_argument("--mixed-meshes", type=int, default=60, help="meshes of the wider mix (strips, tori, bumps, ...)")
    ap.add_argument("--mixed-fields", type=int, default=16)
    ap.add_argument("--epochs", type=int, default=6000)
    ap.add_argument("--lr", type=float, default=3e-3)
    a = ap.parse_args(argv)
    ctx = _capi.Context(0)
    X1, T1, g1 = build_dataset(ctx, a.seed, a.config_meshes, a.config_fields, "configs")
    X2, T2, g2 = build_dataset(ctx, a.seed + 7, a.mixed_meshes, a.mixed_fields, "mixed")
    X = np.concatenate([X1, X2])
    T = np.concatenate([T1, T2])
    g = np.concatenate([g1, g2 + a.config_meshes])
    # validation on whole held-out meshes (one group of five in five), not on
    # other fields of training meshes
    held = (g // 5) % 5 == 4
    va, tr = np.flatnonzero(held), np.flatnonzero(~held)
    params, losses = fit(ctx, X[tr], T[tr], a.epochs, a.lr, a.seed)
    Y = predict(ctx, X[va], params)
    mae = np.abs(Y - T[va]).mean(0)
    tmae = torus_eval(ctx, params)
    print(f"meshes {a.config_meshes} + {a.mixed_meshes}; samples train {len(tr)} val {len(va)}; "
          f"final train loss {losses[-1]:.4f}; val mean |err| log-sweeps {mae[0]:.3f} log-relax {mae[1]:.3f}; "
          f"torus (held-out family) {tmae[0]:.3f} / {tmae[1]:.3f}")
    save(a.out, params, val_mae=mae, torus_mae=tmae, n_train=len(tr), n_val=len(va), seed=a.seed,
         meshes=np.array([a.config_meshes, a.mixed_meshes]))
    print(a.out)


if __name__ == "__main__":
    main()
