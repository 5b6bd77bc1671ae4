"""The learned sweep-cost model: FP32 training kernels against the FP64 numpy
oracle (which is itself checked by finite differences), BF16 tensor-core
inference against FP32, the GPU field features against their restatement,
and the learned batch schedule: results bit-identical to the reactive
schedule, and a faster batch on a workload where the order matters."""
import os

import numpy as np
import pytest

import oracle.mlp as om


def _data(n=300, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, om.N_IN))
    T = np.stack([np.sin(X[:, 0]) + 0.5 * X[:, 1], X[:, 2] * X[:, 3] - 0.3], 1)
    return X.astype(np.float32), T.astype(np.float32)


# ---- CPU: the oracle and the host logic --------------------------------------

def test_oracle_gradient_matches_finite_differences():
    X, T = _data(40, 1)
    p = om.init_params(3)
    g, _ = om.grad(p, X, T)
    rng = np.random.default_rng(5)
    idx = rng.choice(om.N_PARAMS, 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros(om.N_PARAMS)
        e[i] = h
        fd = (om.loss(p + e, X, T) - om.loss(p - e, X, T)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), i


def test_param_count_and_layout_agree_with_library_constants():
    from gproshan_gb300 import learned
    assert om.N_PARAMS == 16 * 64 + 64 + 64 * 64 + 64 + 64 * 2 + 2
    assert len(learned.init_params(0)) == om.N_PARAMS
    assert learned.N_IN == om.N_IN


def test_folded_standardisation_is_exact():
    from gproshan_gb300 import learned
    X, _ = _data(50, 2)
    X = X.astype(np.float64) * 7.0 + 3.0
    mean, std = X.mean(0), X.std(0)
    p = learned.init_params(4).astype(np.float64)
    want = om.forward(p, (X - mean) / std)
    got = om.forward(learned.fold_standardisation(p, mean, std).astype(np.float64), X)
    assert np.allclose(got, want, rtol=1e-4, atol=1e-4)


def test_targets_mask_fields_without_sweeps():
    from gproshan_gb300 import _capi, learned
    s = [_capi.gp_ptp_stats(), _capi.gp_ptp_stats()]
    s[0].n_iter, s[0].n_limits, s[0].relaxations = 20, 11, 5000
    s[1].n_iter, s[1].n_limits, s[1].relaxations = 0, 2, 0
    T, ok = learned.targets(s, [1000, 10])
    assert ok.tolist() == [True, False]
    assert np.allclose(T[0], [np.log(2.0), np.log(5.0)])


def test_shipped_model_has_the_library_layout():
    from gproshan_gb300 import learned
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no shipped cost model")
    with np.load(learned.DEFAULT_MODEL) as z:
        assert len(z["params"]) == om.N_PARAMS
        assert list(z["features"]) == learned.FEATURES
        assert np.all(np.isfinite(z["params"]))


# ---- GPU --------------------------------------------------------------------

@pytest.mark.gpu
def test_gpu_gradient_matches_oracle(gpu_ctx):
    from gproshan_gb300 import _capi
    X, T = _data(257, 7)
    p = om.init_params(8).astype(np.float32)
    g, loss = _capi.mlp_grad(gpu_ctx, X, T, p)
    gr, lr = om.grad(p.astype(np.float64), X, T)
    assert abs(loss - lr) <= 1e-5 * max(1.0, lr)
    assert np.max(np.abs(g - gr)) <= 1e-4 * max(1e-3, np.max(np.abs(gr)))


@pytest.mark.gpu
def test_gpu_inference_fp32_and_bf16(gpu_ctx):
    from gproshan_gb300 import _capi
    X, _ = _data(1000, 9)  # not a multiple of 16: ragged last warp
    p = om.init_params(10).astype(np.float32)
    ref = om.forward(p.astype(np.float64), X)
    y32 = _capi.mlp_infer(gpu_ctx, X, p, bf16=False)
    y16 = _capi.mlp_infer(gpu_ctx, X, p, bf16=True)
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(y32 - ref)) <= 1e-5 * scale
    # BF16 operands (8-bit mantissa) with FP32 accumulation over three layers
    assert np.max(np.abs(y16 - ref)) <= 3e-2 * scale
    assert np.mean(np.abs(y16 - ref)) <= 5e-3 * scale


@pytest.mark.gpu
def test_gpu_training_reduces_loss(gpu_ctx):
    from gproshan_gb300 import _capi
    X, T = _data(512, 11)
    p0 = om.init_params(12).astype(np.float32)
    p, losses = _capi.mlp_train(gpu_ctx, X, T, p0, 400, 3e-3)
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.1 * losses[0]
    assert abs(om.loss(p.astype(np.float64), X, T) - losses[-1]) < 0.05 * losses[0]


def _meshes():
    from gproshan_gb300 import meshgen
    return [meshgen.icosphere(4, 0.1, 1), meshgen.torus(40, 90, seed=2), meshgen.height_field(8, 3, cols=300),
            meshgen.bump_field(60, 4)]


@pytest.mark.gpu
def test_gpu_field_features_match_restatement(gpu_ctx, oracle_lib):
    from gproshan_gb300 import _capi
    rng = np.random.default_rng(13)
    dms, srcs, want = [], [], []
    for xyz, tri in _meshes():
        dm = _capi.DeviceMesh(gpu_ctx, xyz, tri)
        m = oracle_lib.Mesh(xyz, tri)
        stats = om.mesh_stats(xyz, tri, m.OT)
        for ns in (1, 3, 9):
            s = rng.choice(len(xyz), ns, replace=False).astype(np.uint32)
            _, _, lim = oracle_lib.toplesets(m, s)
            dms.append(dm)
            srcs.append(s)
            want.append(om.field_features(lim, len(xyz), ns, stats))
    got = _capi.field_features(gpu_ctx, dms, srcs)
    want = np.array(want)
    # toplesets-derived features are exact up to FP32 logs; the geometry
    # statistics are accumulated from FP32 coordinates
    assert np.allclose(got[:, :10], want[:, :10], rtol=1e-5, atol=1e-5)
    assert np.allclose(got[:, 15], want[:, 15], rtol=1e-6, atol=1e-6)
    assert np.allclose(got[:, 10:15], want[:, 10:15], rtol=1e-3, atol=2e-3)


def _order_workload(gpu_ctx):
    """Short fields listed first, long ones last: many more fields than CTAs
    of the one-CTA kernel, every window within one CTA."""
    from gproshan_gb300 import _capi, meshgen
    short = _capi.DeviceMesh(gpu_ctx, *meshgen.height_field(6, 5, cols=240))
    long_ = _capi.DeviceMesh(gpu_ctx, *meshgen.height_field(6, 6, cols=1600))
    ms, srcs = [], []
    for k in range(1200):
        ms.append(short)
        srcs.append(np.array([k % short.n_vertices], np.uint32))
    for k in range(160):
        ms.append(long_)
        srcs.append(np.array([k % 6], np.uint32))  # one end of the strip
    return ms, srcs


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_learned_schedule_results_identical(gpu_ctx, precision):
    from gproshan_gb300 import _capi, learned, meshgen
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no shipped cost model")
    learned.install(gpu_ctx)
    try:
        meshes = [_capi.DeviceMesh(gpu_ctx, *m) for m in _meshes()]
        meshes.append(_capi.DeviceMesh(gpu_ctx, *meshgen.height_field(200, 8)))
        rng = np.random.default_rng(precision)
        ms, srcs = [], []
        for k in range(41):
            mm = meshes[k % len(meshes)]
            ms.append(mm)
            srcs.append(rng.choice(mm.n_vertices, size=1 + k % 4, replace=False))
        dt = np.float64 if precision else np.float32
        d0, s0, _ = _capi.ptp_batch(gpu_ctx, ms, srcs, dtype=dt, precision=precision)
        d1, s1, _ = _capi.ptp_batch(gpu_ctx, ms, srcs, dtype=dt, precision=precision,
                                    schedule=_capi.GP_SCHED_LEARNED)
        cs = gpu_ctx.call_stats()
        assert cs.fields_grid >= 1
        for k in range(len(ms)):
            assert np.array_equal(d0[k], d1[k]), k
            assert s0[k].n_iter == s1[k].n_iter and s0[k].relaxations == s1[k].relaxations
    finally:
        _capi.set_cost_model(gpu_ctx, None)


@pytest.mark.gpu
def test_learned_schedule_is_faster_when_order_matters(gpu_ctx):
    """The reactive schedule takes fields in the order given; with the short
    fields first, the long chains start last and set the makespan.  The cost
    model ranks them first."""
    from gproshan_gb300 import _capi, learned
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no shipped cost model")
    ms, srcs = _order_workload(gpu_ctx)
    learned.install(gpu_ctx)
    try:
        def timed(schedule):
            best, out = None, None
            for _ in range(3):
                d, _, _ = _capi.ptp_batch(gpu_ctx, ms, srcs, schedule=schedule, with_stats=False)
                cs = gpu_ctx.call_stats()
                t = cs.ms_local + cs.ms_grid
                if best is None or t < best:
                    best, out = t, d
            return best, out
        t0, d0 = timed(_capi.GP_SCHED_REACTIVE)
        t1, d1 = timed(_capi.GP_SCHED_LEARNED)
        for k in range(len(ms)):
            assert np.array_equal(d0[k], d1[k]), k
        print(f"sweep phases: reactive {t0:.3f} ms, learned {t1:.3f} ms ({t0 / t1:.2f}x)")
        assert t1 < 0.85 * t0
    finally:
        _capi.set_cost_model(gpu_ctx, None)
