"""GPU parity: the CUDA path through the C ABI against the CPU oracle and the
golden vectors of the reference's own code.

Bars: integer outputs (rings, sorted, limits, labels, samples) bit-exact; the
FP64 path (reference formula) bit-exact with the FP64 oracle; the FP32 path
within max relative error 1e-5 of the FP64 oracle run on the same
float-rounded coordinates, with the same number of sweeps."""
import numpy as np
import pytest

from conftest import golden_cases

pytestmark = pytest.mark.gpu

CASES = golden_cases()
REL_TOL_F32 = 1e-5


def dev_mesh(ctx, xyz, tri):
    from gproshan_gb300 import _capi
    return _capi.DeviceMesh(ctx, xyz, tri)


def test_loaded_code_is_native_sm103(gpu_ctx):
    """The kernels run from native sm_103 code built by build(), not from PTX
    JIT-compiled by the driver: the binary version of the loaded sweep kernel
    (cudaFuncGetAttributes) is 103 on a compute capability 10.3 device."""
    cc, bv, n_sm = gpu_ctx.device_info()
    assert cc == 103 and bv == 103 and n_sm > 0


@pytest.mark.parametrize("name,g", CASES, ids=[c[0] for c in CASES])
def test_toplesets_bit_exact_golden(gpu_ctx, name, g):
    from gproshan_gb300 import _capi
    m = _capi.DeviceMesh(gpu_ctx, g["xyz"], g["VT"], g["OT"], g["EVT"])
    for k in range(int(g["n_sets"])):
        rings, srt, lim = _capi.toplesets(m, g[f"src{k}"])
        assert np.array_equal(rings, g[f"rings{k}"]), (name, k)
        assert np.array_equal(lim, g[f"limits{k}"]), (name, k)
        assert np.array_equal(srt, g[f"sorted{k}"]), (name, k)


@pytest.mark.parametrize("name,g", CASES, ids=[c[0] for c in CASES])
def test_ptp_f64_bit_exact_oracle(gpu_ctx, oracle_lib, name, g):
    from gproshan_gb300 import _capi
    m = dev_mesh(gpu_ctx, g["xyz"], g["tri"])
    om = oracle_lib.Mesh(g["xyz"], g["tri"])
    for k in range(int(g["n_sets"])):
        src = g[f"src{k}"]
        ref = oracle_lib.ptp(om, src, g[f"limits{k}"], g[f"sorted{k}"])
        d, _, st = _capi.ptp(m, src, dtype=np.float64, precision=_capi.GP_F64)
        assert st.n_iter == ref["n_iter"], (name, k)
        assert st.relaxations == ref["relaxations"], (name, k)
        assert np.array_equal(d, ref["dist"]), (name, k, np.nanmax(np.abs(d - ref["dist"])))


@pytest.mark.parametrize("name,g", CASES, ids=[c[0] for c in CASES])
def test_ptp_f32_within_tolerance(gpu_ctx, oracle_lib, name, g):
    from gproshan_gb300 import _capi
    m = dev_mesh(gpu_ctx, g["xyz"], g["tri"])
    om = oracle_lib.Mesh(g["xyz"], g["tri"])
    x32 = g["xyz"].astype(np.float32).astype(np.float64)
    for k in range(int(g["n_sets"])):
        src = g[f"src{k}"]
        ref = oracle_lib.ptp(om, src, g[f"limits{k}"], g[f"sorted{k}"], xyz=x32)
        d, _, st = _capi.ptp(m, src)
        assert st.n_iter == ref["n_iter"], (name, k)
        err = oracle_lib.max_rel_err(d, ref["dist"])
        assert err <= REL_TOL_F32, (name, k, err)


def test_caller_toplesets_equal_gpu_toplesets(gpu_ctx):
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = meshgen.height_field(48, 5)
    m = dev_mesh(gpu_ctx, xyz, tri)
    rings, srt, lim = _capi.toplesets(m, [7, 1500])
    a, _, sa = _capi.ptp(m, [7, 1500], lim, srt)
    b, _, sb = _capi.ptp(m, [7, 1500])
    assert np.array_equal(a, b) and sa.n_iter == sb.n_iter


@pytest.mark.parametrize("maker,src", [
    (lambda mg: mg.icosphere(5, 0.1, 3), [0]),
    (lambda mg: mg.height_field(160, 9), [0, 12345, 20000]),
    (lambda mg: mg.torus(120, 40, seed=2), [5]),
    (lambda mg: mg.bump_field(90, 4), [77]),
    # anisotropic torus, edge ratio ~20:1 (needle triangles): the FP32 path
    # forms each new distance exactly from its candidate's operands, which
    # keeps it at ~2e-7 here (rounded candidates drifted to ~3e-5)
    (lambda mg: mg.torus(100, 600, seed=0), [43584, 56581, 52882, 30679]),
])
def test_larger_meshes_against_oracle(gpu_ctx, oracle_lib, maker, src):
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = maker(meshgen)
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    r_o, s_o, l_o = oracle_lib.toplesets(om, src)
    rings, srt, lim = _capi.toplesets(m, src)
    assert np.array_equal(rings, r_o) and np.array_equal(srt, s_o) and np.array_equal(lim, l_o)
    ref64 = oracle_lib.ptp(om, src, l_o, s_o)
    d64, _, st = _capi.ptp(m, src, dtype=np.float64, precision=_capi.GP_F64)
    assert st.n_iter == ref64["n_iter"] and np.array_equal(d64, ref64["dist"])
    ref = oracle_lib.ptp(om, src, l_o, s_o, xyz=xyz.astype(np.float32).astype(np.float64))
    d32, _, st32 = _capi.ptp(m, src)
    assert st32.n_iter == ref["n_iter"]
    assert oracle_lib.max_rel_err(d32, ref["dist"]) <= REL_TOL_F32


def _degenerate_mesh():
    """A height field with collinear vertices (zero-area triangles) and
    coincident vertices (zero-length edges)."""
    from gproshan_gb300 import meshgen
    xyz, tri = meshgen.height_field(40, 3)
    n = 40
    for r in range(5, 35, 6):
        for c in range(5, 35, 7):
            v = r * n + c
            xyz[v] = 0.5 * (xyz[v - 1] + xyz[v + 1])
    for r in range(8, 32, 9):
        v = r * n + 20
        xyz[v] = xyz[v + n]
    return xyz, tri


def test_degenerate_triangles_follow_the_reference(gpu_ctx, oracle_lib):
    """Zero-area triangles give NaN candidates that the reference ignores (INF
    inputs still take the edge fallback), zero-length edges give zero
    fallbacks: the FP64 path matches bit for bit, the FP32 path within tol."""
    from gproshan_gb300 import _capi
    xyz, tri = _degenerate_mesh()
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    src = [0, 777]
    _, s_o, l_o = oracle_lib.toplesets(om, src)
    ref64 = oracle_lib.ptp(om, src, l_o, s_o)
    d64, _, st = _capi.ptp(m, src, dtype=np.float64, precision=_capi.GP_F64)
    assert st.n_iter == ref64["n_iter"] and np.array_equal(d64, ref64["dist"])
    ref = oracle_lib.ptp(om, src, l_o, s_o, xyz=xyz.astype(np.float32).astype(np.float64))
    d32, _, st32 = _capi.ptp(m, src)
    assert np.isfinite(d32).all() and st32.n_iter == ref["n_iter"]
    assert oracle_lib.max_rel_err(d32, ref["dist"]) <= REL_TOL_F32


def test_batches_longer_than_one_device_pass(gpu_ctx):
    """More fields than one device pass holds (2048): the call is chunked and
    every field equals its single-field result."""
    from gproshan_gb300 import _capi, meshgen
    m = dev_mesh(gpu_ctx, *meshgen.icosphere(2, 0.1, 4))
    rng = np.random.default_rng(3)
    srcs = [rng.choice(m.n_vertices, size=1 + k % 2, replace=False) for k in range(2100)]
    d, st, _ = _capi.ptp_batch(gpu_ctx, [m] * len(srcs), srcs)
    for k in (0, 1, 2047, 2048, 2099):
        d1, _, s1 = _capi.ptp(m, srcs[k])
        assert np.array_equal(d1, d[k]) and s1.n_iter == st[k].n_iter, k


def test_duplicate_and_isolated_sources(gpu_ctx, oracle_lib):
    from gproshan_gb300 import _capi
    g = dict(np.load(__import__("os").path.join(__import__("conftest").GOLDEN, "grid_hole.npz")))
    m = dev_mesh(gpu_ctx, g["xyz"], g["tri"])
    om = oracle_lib.Mesh(g["xyz"], g["tri"])
    # isolated source: no sweep, the source at 0, everything else INF
    d, _, st = _capi.ptp(m, g["src2"], dtype=np.float64, precision=_capi.GP_F64)
    assert st.n_iter == 0 and d[g["src2"][0]] == 0 and np.isinf(np.delete(d, g["src2"][0])).all()
    # repeated sources: defined here (every sorted entry is relaxed)
    src = [168, 5, 168]
    ref = oracle_lib.ptp(om, src)
    d, _, st = _capi.ptp(m, src, dtype=np.float64, precision=_capi.GP_F64)
    assert st.n_iter == ref["n_iter"] and np.array_equal(d, ref["dist"])


def test_icosphere_l6_workload_exact(gpu_ctx, oracle_lib):
    """The single-field workload exactly as specified: icosphere subdivided 6
    times (40,962 vertices, 81,920 faces, unit radius), vertices jittered
    tangentially by seeded uniform noise of 0.1 x mean edge, source vertex 0.
    FP64: the same sweeps, relaxations and distance bits as the oracle; FP32:
    within 1e-5 of the FP64 oracle on the same float-rounded coordinates, with
    the same sweep count.  Where the reference's own CPU build is present, the
    oracle's CPU-returned buffer equals its output bit for bit as well."""
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = meshgen.icosphere(6, 0.1, 0)
    assert len(xyz) == 40962 and len(tri) == 81920
    assert np.allclose(np.linalg.norm(xyz, axis=1), 1.0)
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    r_o, s_o, l_o = oracle_lib.toplesets(om, [0])
    rings, srt, lim = _capi.toplesets(m, [0])
    assert np.array_equal(rings, r_o) and np.array_equal(srt, s_o) and np.array_equal(lim, l_o)
    ref64 = oracle_lib.ptp(om, [0], l_o, s_o)
    d64, _, st64 = _capi.ptp(m, [0], dtype=np.float64, precision=_capi.GP_F64)
    assert st64.n_iter == ref64["n_iter"] == 194 and st64.relaxations == ref64["relaxations"]
    assert np.array_equal(d64, ref64["dist"])
    x32 = xyz.astype(np.float32).astype(np.float64)
    ref32 = oracle_lib.ptp(om, [0], l_o, s_o, xyz=x32)
    d32, _, st32 = _capi.ptp(m, [0])
    assert st32.n_iter == ref32["n_iter"]
    assert oracle_lib.max_rel_err(d32, ref32["dist"]) <= REL_TOL_F32
    try:
        rl = oracle_lib.RefLib("f64")
    except (FileNotFoundError, OSError):
        return
    rm = oracle_lib.RefMesh(rl, xyz, tri)
    assert np.array_equal(rm.geodesics_ptp_cpu([0]), ref64["dist_cpu"])


@pytest.mark.parametrize("maker,src", [
    (lambda mg: mg.icosphere(4, 0.1, 2), [0, 1000, 2000]),
    (lambda mg: mg.icosphere(5, 0.1, 7), [3, 500, 4000, 9000, 10000]),
    (lambda mg: mg.height_field(90, 4), [0, 4000, 8099]),
    (lambda mg: mg.torus(80, 200, seed=1), [10, 5000, 11000, 15999]),
])
def test_fp32_labels_follow_the_reference_rule(gpu_ctx, oracle_lib, maker, src):
    """FP32 labels are integer output: the label of the first strictly smaller
    candidate in the reference's star order, taken from the nearer of the
    triangle's two other vertices (src/cuda/geodesics_ptp.cu:257-282).  They
    equal the FP64 oracle's labels bit for bit (same float-rounded
    coordinates), every source labelled with its 1-based index, on every launch
    kind.  The labelled sweeps solve the star triangle by triangle (the label
    rule needs the reference's order); the unlabelled ones take each edge value
    once per neighbour: both within the FP32 bar, with the same sweeps."""
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = maker(meshgen)
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    ref = oracle_lib.ptp(om, src, clusters=True, xyz=xyz.astype(np.float32).astype(np.float64))
    plain, _, _ = _capi.ptp(m, src)
    for kw in (dict(local_window=1 << 30), dict(local_window=1, grid_kernel=_capi.GP_GRID_LOCKSTEP),
               dict(local_window=1, grid_kernel=_capi.GP_GRID_QUEUE, queue_min=1)):
        d, cl, st = _capi.ptp(m, src, clusters=np.zeros(len(xyz), np.uint32), opts=_capi.make_opts(0, **kw))
        assert st.n_iter == ref["n_iter"]
        assert np.array_equal(cl, ref["clusters"]), (kw, int(np.sum(cl != ref["clusters"])))
        assert oracle_lib.max_rel_err(d, ref["dist"]) <= REL_TOL_F32
        assert oracle_lib.max_rel_err(plain, d.astype(np.float64)) <= REL_TOL_F32
    assert [int(cl[s]) for s in src] == list(range(1, len(src) + 1))


def test_clusters_gpu_rule(gpu_ctx, oracle_lib):
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = meshgen.icosphere(4, 0.1, 2)
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    src = [0, 1000, 2000]
    ref = oracle_lib.ptp(om, src, clusters=True)
    d, cl, _ = _capi.ptp(m, src, dtype=np.float64, precision=_capi.GP_F64,
                         clusters=np.zeros(len(xyz), np.uint32))
    assert np.array_equal(d, ref["dist"])
    assert np.array_equal(cl, ref["clusters"])
    assert set(np.unique(cl)) == {1, 2, 3}


@pytest.mark.parametrize("n_fields", [12, 13, 40])
def test_batch_equals_single_fields(gpu_ctx, n_fields):
    """Batched fields (some swept by one CTA, some handed to the grid-wide
    launch: the 200^2 height field's windows outgrow one CTA) equal the same
    fields solved alone, bit for bit; odd and even batch sizes."""
    from gproshan_gb300 import _capi, meshgen
    meshes = [dev_mesh(gpu_ctx, *meshgen.icosphere(3, 0.1, 1)), dev_mesh(gpu_ctx, *meshgen.height_field(70, 2)),
              dev_mesh(gpu_ctx, *meshgen.icosphere(5, 0.1, 3)), dev_mesh(gpu_ctx, *meshgen.height_field(200, 8))]
    rng = np.random.default_rng(n_fields)
    ms, srcs = [], []
    for k in range(n_fields):
        mm = meshes[k % len(meshes)]
        ms.append(mm)
        srcs.append(rng.choice(mm.n_vertices, size=1 + k % 3, replace=False))
    dists, stats, sec = _capi.ptp_batch(gpu_ctx, ms, srcs)
    assert sec > 0
    assert gpu_ctx.call_stats().fields_grid >= 1  # the grid-wide launch did run
    for k in range(n_fields):
        d, _, st = _capi.ptp(ms[k], srcs[k])
        assert np.array_equal(d, dists[k]), k
        assert st.n_iter == stats[k].n_iter


def test_fps_matches_oracle(gpu_ctx, oracle_lib):
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = meshgen.icosphere(3, 0.1, 5)
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    s_ref, md_ref = oracle_lib.fps(om, 12, [0])
    s, md, _ = _capi.fps(m, 12, [0], precision=_capi.GP_F64)
    assert np.array_equal(s, s_ref) and md == md_ref


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_normalize_option_in_the_call(gpu_ctx, oracle_lib, precision):
    """gp_ptp_opts.normalize divides every field's output by its largest finite
    distance on the device (the maximum reduced in the output gather): bit for
    bit normalize_ptp of the unnormalized output, in a batch with an
    unreached component (INF stays INF) and fields on several meshes."""
    from gproshan_gb300 import _capi, meshgen
    x1, t1 = meshgen.icosphere(3, 0.1, 1)
    x2, t2 = meshgen.height_field(20, 2)
    xyz = np.concatenate([x1, x2 + np.array([3.0, 0.0, 0.0])])
    tri = np.concatenate([t1, t2 + len(x1)]).astype(np.uint32)
    ms = [dev_mesh(gpu_ctx, xyz, tri), dev_mesh(gpu_ctx, *meshgen.height_field(150, 4))]
    prec, dt = (_capi.GP_F64, np.float64) if precision == "f64" else (_capi.GP_F32, np.float32)
    meshes, srcs = [ms[0], ms[1], ms[1]], [[5], [0], [100, 9000]]
    plain, _, _ = _capi.ptp_batch(gpu_ctx, meshes, srcs, dtype=dt, precision=prec)
    L = _capi.lib()
    outs = [np.empty(m.n_vertices, dt) for m in meshes]
    fields, keep = _capi._fields(meshes, srcs, outs)
    o = _capi.make_opts(prec, normalize=True)
    sec = _capi.C.c_double()
    gpu_ctx.check(L.gp_ptp_batch(gpu_ctx.handle, fields, len(meshes), _capi.C.byref(o),
                                 _capi.GP_F64 if dt == np.float64 else _capi.GP_F32, 0, _capi.C.byref(sec)), "batch")
    for a, b in zip(outs, plain):
        ref = b.copy()
        m = np.max(ref[np.isfinite(ref)])
        ref /= dt(m)
        assert np.array_equal(a, ref)
        if dt == np.float64:
            assert np.array_equal(a, oracle_lib.normalize_ptp(b))
    assert np.isinf(outs[0][len(x1):]).all() and np.max(outs[1]) == 1.0


def test_fps_device_loop_matches_oracle_longer_runs(gpu_ctx, oracle_lib):
    """The device-resident sample loop: 40 samples on a height field and a
    radius-limited run (the loop stops on the device at the first field whose
    farthest distance is within the radius), both equal to the oracle's FPS."""
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = meshgen.height_field(60, 3)
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    s_ref, md_ref = oracle_lib.fps(om, 40, [7])
    s, md, sec = _capi.fps(m, 40, [7], precision=_capi.GP_F64)
    assert np.array_equal(s, s_ref) and md == md_ref and sec > 0
    s_ref, md_ref = oracle_lib.fps(om, 200, [7], radio=0.4)
    s, md, _ = _capi.fps(m, 200, [7], radio=0.4, precision=_capi.GP_F64)
    assert 1 < len(s_ref) < 200 and np.array_equal(s, s_ref) and md == md_ref
    # FP32: same samples while the farthest distances are well separated
    s32, _, _ = _capi.fps(m, 12, [7])
    assert np.array_equal(s32, oracle_lib.fps(om, 12, [7])[0])


def test_normalize_matches_oracle(gpu_ctx, oracle_lib):
    from gproshan_gb300 import _capi
    rng = np.random.default_rng(3)
    d = rng.random(1000) * 5
    d[7] = np.inf
    out = _capi.normalize_ptp(gpu_ctx, d.copy())
    ref = oracle_lib.normalize_ptp(d)
    assert np.array_equal(out, ref)


def test_geodesics_api_end_to_end(gpu_ctx, oracle_lib):
    from gproshan_gb300 import che, geodesics, meshgen, parallel_toplesets_propagation_gpu, ptp_out_t, toplesets_t
    xyz, tri = meshgen.icosphere(4, 0.1, 9)
    mesh = che(xyz, tri)
    g = geodesics(mesh, [3], geodesics.PTP_GPU, ctx=gpu_ctx)
    om = oracle_lib.Mesh(xyz, tri)
    ref = oracle_lib.ptp(om, [3], xyz=xyz.astype(np.float32).astype(np.float64))
    assert oracle_lib.max_rel_err(g.dist, ref["dist"]) <= REL_TOL_F32
    assert g[3] == 0.0
    rings, srt, lim = mesh.compute_toplesets([3], ctx=gpu_ctx)
    out = ptp_out_t(np.empty(mesh.n_vertices(), np.float64))
    t = parallel_toplesets_propagation_gpu(out, mesh, [3], toplesets_t(lim, srt), ctx=gpu_ctx)
    assert t > 0 and np.array_equal(out.dist, g.dist)


def test_invalid_source_is_an_error_and_context_survives(gpu_ctx):
    from gproshan_gb300 import _capi, meshgen
    m = dev_mesh(gpu_ctx, *meshgen.icosphere(2, 0.0, 0))
    with pytest.raises(_capi.GPError) as e:
        _capi.ptp(m, [m.n_vertices + 5])
    assert e.value.status == 1
    d, _, _ = _capi.ptp(m, [0])
    assert d[0] == 0 and np.isfinite(d).all()


def test_grid_barrier_wait_is_bounded_and_reported(gpu_ctx):
    """A grid barrier that cannot complete (it waits for one arrival more
    than the launch has CTAs, set through the test hook) gives up after its
    poll limit: the call returns GP_ERR_DEVICE_TIMEOUT, nothing hangs, and the
    context keeps working."""
    from gproshan_gb300 import _capi, meshgen
    m = dev_mesh(gpu_ctx, *meshgen.height_field(150, 2))
    ref, _, _ = _capi.ptp(m, [0])
    L = _capi.lib()
    gpu_ctx.check(L.gp_ctx_debug_barrier(gpu_ctx.handle, 4000, 1), "gp_ctx_debug_barrier")
    try:
        with pytest.raises(_capi.GPError) as e:
            _capi.ptp(m, [0], opts=_capi.make_opts(grid_kernel=_capi.GP_GRID_LOCKSTEP))
        assert e.value.status == _capi.GP_ERR_DEVICE_TIMEOUT
    finally:
        gpu_ctx.check(L.gp_ctx_debug_barrier(gpu_ctx.handle, 0, 0), "gp_ctx_debug_barrier")
    d, _, _ = _capi.ptp(m, [0])
    assert np.array_equal(d, ref)


@pytest.mark.parametrize("maker,src", [
    (lambda mg: mg.icosphere(4, 0.1, 1), [0]),
    (lambda mg: mg.height_field(96, 6), [5, 4000]),
])
@pytest.mark.parametrize("precision", [0, 1])
def test_one_cta_and_grid_paths_agree(gpu_ctx, maker, src, precision):
    """A field swept by one CTA and the same field swept by the grid-wide
    launch give identical bits (same arithmetic, same schedule)."""
    from gproshan_gb300 import _capi, meshgen
    m = dev_mesh(gpu_ctx, *maker(meshgen))
    dt = np.float64 if precision else np.float32
    a, _, sa = _capi.ptp(m, src, dtype=dt, opts=_capi.make_opts(precision, local_window=1 << 30))
    b, _, sb = _capi.ptp(m, src, dtype=dt, opts=_capi.make_opts(precision, local_window=1))
    assert sa.n_iter == sb.n_iter and sa.relaxations == sb.relaxations
    assert np.array_equal(a, b)


@pytest.mark.parametrize("precision,clusters", [(0, False), (1, False), (0, True)])
def test_queue_and_lockstep_grid_kernels_agree(gpu_ctx, precision, clusters):
    """The work-queue launch (no grid barrier) and the lockstep launch sweep
    the same windows of every field, so distances, labels and sweep counts are
    identical; both are also checked against the fields solved alone."""
    from gproshan_gb300 import _capi, meshgen
    meshes = [dev_mesh(gpu_ctx, *meshgen.icosphere(5, 0.1, 3)), dev_mesh(gpu_ctx, *meshgen.height_field(200, 8)),
              dev_mesh(gpu_ctx, *meshgen.height_field(8, 5, cols=900)), dev_mesh(gpu_ctx, *meshgen.icosphere(3, 0.1, 1))]
    rng = np.random.default_rng(7 + precision)
    ms, srcs = [], []
    for k in range(23):
        mm = meshes[k % len(meshes)]
        ms.append(mm)
        srcs.append(rng.choice(mm.n_vertices, size=1 + k % 3, replace=False))
    dt = np.float64 if precision else np.float32
    out = {}
    for gk in (_capi.GP_GRID_LOCKSTEP, _capi.GP_GRID_QUEUE):
        fields = (_capi.gp_field * len(ms))()
        keep, dists, labs, stats = [], [], [], [_capi.gp_ptp_stats() for _ in ms]
        for k, (mm, sr) in enumerate(zip(ms, srcs)):
            sr = np.ascontiguousarray(sr, np.uint32)
            d = np.empty(mm.n_vertices, dt)
            lab = np.zeros(mm.n_vertices, np.uint32) if clusters else None
            keep.append(sr)
            dists.append(d)
            labs.append(lab)
            fields[k].mesh = mm.handle
            fields[k].sources = sr.ctypes.data
            fields[k].n_sources = len(sr)
            fields[k].dist = d.ctypes.data
            fields[k].clusters = None if lab is None else lab.ctypes.data
            import ctypes
            fields[k].stats = ctypes.addressof(stats[k])
        opts = _capi.make_opts(precision, local_window=256, grid_kernel=gk)
        sec = _capi.C.c_double(0)
        gpu_ctx.check(_capi.lib().gp_ptp_batch(gpu_ctx.handle, fields, len(ms), _capi.C.byref(opts),
                                               _capi.GP_F64 if precision else _capi.GP_F32, 0,
                                               _capi.C.byref(sec)), "gp_ptp_batch")
        cs = gpu_ctx.call_stats()
        assert cs.grid_kernel == gk and cs.fields_grid >= 10
        out[gk] = (dists, labs, [(s.n_iter, s.relaxations) for s in stats])
    a, b = out[_capi.GP_GRID_LOCKSTEP], out[_capi.GP_GRID_QUEUE]
    assert a[2] == b[2]
    for k in range(len(ms)):
        assert np.array_equal(a[0][k], b[0][k]), k
        if clusters:
            assert np.array_equal(a[1][k], b[1][k]), k
    for k in range(0, len(ms), 5):
        lab = np.zeros(ms[k].n_vertices, np.uint32) if clusters else None
        d, cl, st = _capi.ptp(ms[k], srcs[k], dtype=dt, precision=precision, clusters=lab)
        assert np.array_equal(d, b[0][k]) and st.n_iter == b[2][k][0], k
        if clusters:
            assert np.array_equal(cl, b[1][k]), k


@pytest.mark.parametrize("launch", ["cta", "lockstep", "queue"])
def test_change_flags_leave_distances_unchanged(gpu_ctx, oracle_lib, launch):
    """The FP32 sweeps without labels keep a change flag in the sign bit of
    every stored distance.  No flag reaches the output, every launch kind gives
    the one-CTA launch's distance bits, and the labelled sweeps (no flags,
    triangle-by-triangle solves) agree within the FP32 bar with the same sweep
    and relaxation counts."""
    from gproshan_gb300 import _capi, meshgen
    kw = {"cta": dict(local_window=1 << 30), "lockstep": dict(local_window=1, grid_kernel=_capi.GP_GRID_LOCKSTEP),
          "queue": dict(local_window=1, grid_kernel=_capi.GP_GRID_QUEUE, queue_min=1)}[launch]
    cases = [(meshgen.height_field(150, 3), [7]), (meshgen.torus(60, 300, seed=2), [0, 9000])]
    for (xyz, tri), src in cases:
        m = dev_mesh(gpu_ctx, xyz, tri)
        a, _, sa = _capi.ptp(m, src, opts=_capi.make_opts(0, **kw))
        c, _, _ = _capi.ptp(m, src, opts=_capi.make_opts(0, local_window=1 << 30))
        b, _, sb = _capi.ptp(m, src, clusters=np.zeros(len(xyz), np.uint32), opts=_capi.make_opts(0, **kw))
        assert sa.n_iter == sb.n_iter and sa.relaxations == sb.relaxations
        assert np.array_equal(a, c), np.max(np.abs(a.astype(np.float64) - c))
        assert oracle_lib.max_rel_err(a, b) <= REL_TOL_F32
        assert np.all(a >= 0)  # no flag leaks into the output


def test_unchanged_input_skip_is_exact(gpu_ctx, oracle_lib):
    """In steps of the lockstep launch with at least one tile per warp, a warp
    whose vertices and their neighbours did not change in the previous sweep
    skips the solves.  The skip happens (counted) and changes nothing: the
    distances equal those of the one-CTA launch (which never skips) bit for
    bit, and a sample matches the FP64 oracle within the FP32 bar."""
    from gproshan_gb300 import _capi, meshgen
    meshes = [meshgen.height_field(256, 11), meshgen.torus(60, 300, seed=2)]
    dms = [dev_mesh(gpu_ctx, x, t) for x, t in meshes]
    rng = np.random.default_rng(5)
    ms, srcs, mi = [], [], []
    for k in range(40):
        q = k % 2
        ms.append(dms[q])
        mi.append(q)
        srcs.append(rng.choice(dms[q].n_vertices, size=1 + k % 2, replace=False))
    kw = dict(local_window=1, grid_kernel=_capi.GP_GRID_LOCKSTEP)
    a, sa, _ = _capi.ptp_batch(gpu_ctx, ms, srcs, **kw)
    cs = gpu_ctx.call_stats()
    assert cs.grid_kernel == _capi.GP_GRID_LOCKSTEP and cs.fields_grid == len(ms)
    assert cs.skip_grid > 0.02 * cs.relax_grid, (cs.skip_grid, cs.relax_grid)
    b, sb, _ = _capi.ptp_batch(gpu_ctx, ms, srcs, local_window=1 << 30)
    cs = gpu_ctx.call_stats()
    assert cs.fields_grid == 0 and cs.skip_grid == 0
    for k in range(len(ms)):
        assert sa[k].n_iter == sb[k].n_iter, k
        assert np.array_equal(a[k], b[k]), k
    for k in (0, 1, 6):
        x, t = meshes[mi[k]]
        om = oracle_lib.Mesh(x, t)
        _, s_o, l_o = oracle_lib.toplesets(om, srcs[k])
        ref = oracle_lib.ptp(om, srcs[k], l_o, s_o, xyz=x.astype(np.float32).astype(np.float64))
        assert sa[k].n_iter == ref["n_iter"]
        assert oracle_lib.max_rel_err(a[k], ref["dist"]) <= REL_TOL_F32


def test_queue_kernel_auto_choice(gpu_ctx):
    """GP_GRID_AUTO takes the lockstep launch below queue_min grid fields and
    the work queue from there on."""
    from gproshan_gb300 import _capi, meshgen
    m = dev_mesh(gpu_ctx, *meshgen.height_field(150, 2))
    _capi.ptp_batch(gpu_ctx, [m], [[0]], queue_min=2)
    assert gpu_ctx.call_stats().grid_kernel == _capi.GP_GRID_LOCKSTEP
    _capi.ptp_batch(gpu_ctx, [m] * 5, [[0], [1], [2], [300], [5000]], queue_min=2)
    assert gpu_ctx.call_stats().grid_kernel == _capi.GP_GRID_QUEUE


@pytest.mark.parametrize("n_src", [1, 7, 300])
def test_wide_toplesets_match_oracle(gpu_ctx, oracle_lib, n_src):
    """A field on a mesh of >= 2^18 vertices in a call of few fields takes
    the whole-GPU BFS (all CTAs on each level); its rings, sorted order and
    limits still equal the reference's, and so do the distances."""
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = meshgen.height_field(520, 11)
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    src = np.random.default_rng(n_src).choice(len(xyz), n_src, replace=False)
    r_o, s_o, l_o = oracle_lib.toplesets(om, src)
    rings, srt, lim = _capi.toplesets(m, src)
    assert np.array_equal(lim, l_o) and np.array_equal(srt, s_o) and np.array_equal(rings, r_o)
    # the same field in a batch of two (both wide) and alone through gp_ptp agree
    d2, st2, _ = _capi.ptp_batch(gpu_ctx, [m, m], [src, src[:1]])
    d1, _, st1 = _capi.ptp(m, src)
    assert np.array_equal(d1, d2[0]) and st1.n_iter == st2[0].n_iter and st2[0].n_limits == len(l_o)


@pytest.mark.parametrize("src", [[0, 1, 2], [64, 65, 128, 0], [5, 5, 6], [4095, 4094]])
def test_toplesets_adjacent_and_repeated_sources(gpu_ctx, oracle_lib, src):
    """Sources next to each other (and repeated) stay in ring 0 and keep the
    reference's order: a source is never re-discovered from a neighbour."""
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = meshgen.height_field(64, 3)
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    r_o, s_o, l_o = oracle_lib.toplesets(om, src)
    rings, srt, lim = _capi.toplesets(m, src)
    assert np.array_equal(rings, r_o) and np.array_equal(lim, l_o) and np.array_equal(srt, s_o)


def test_toplesets_high_valence_vertex(gpu_ctx, oracle_lib):
    """A fan of more than 8 triangles (link read from the CSR lists)."""
    from gproshan_gb300 import _capi
    k = 13
    ang = np.linspace(0, 2 * np.pi, k, endpoint=False)
    ring1 = np.stack([np.cos(ang), np.sin(ang), np.zeros(k)], 1)
    ring2 = 2.1 * np.stack([np.cos(ang + 0.2), np.sin(ang + 0.2), 0.1 * np.ones(k)], 1)
    xyz = np.concatenate([[[0.0, 0.0, 0.3]], ring1, ring2])
    tri = []
    for i in range(k):
        a, b = 1 + i, 1 + (i + 1) % k
        c, d = 1 + k + i, 1 + k + (i + 1) % k
        tri += [[0, a, b], [a, c, b], [b, c, d]]
    tri = np.array(tri, np.uint32)
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    for src in ([0], [1 + k], [3, 0]):
        r_o, s_o, l_o = oracle_lib.toplesets(om, src)
        rings, srt, lim = _capi.toplesets(m, src)
        assert np.array_equal(rings, r_o) and np.array_equal(lim, l_o) and np.array_equal(srt, s_o)
        ref = oracle_lib.ptp(om, src, l_o, s_o)
        d, _, st = _capi.ptp(m, src, dtype=np.float64, precision=_capi.GP_F64)
        assert st.n_iter == ref["n_iter"] and np.array_equal(d, ref["dist"])
        ref32 = oracle_lib.ptp(om, src, l_o, s_o, xyz=xyz.astype(np.float32).astype(np.float64))
        d32, _, _ = _capi.ptp(m, src)
        assert oracle_lib.max_rel_err(d32, ref32["dist"]) <= REL_TOL_F32


@pytest.mark.parametrize("case", [0, 1], ids=["flat101", "sphere_L5"])
def test_accuracy_against_closed_form_matches_oracle(gpu_ctx, oracle_lib, case):
    """Against exact geodesics (flat grid: Euclidean; unit sphere:
    great-circle), the FP32 GPU path has the algorithm's own error profile:
    the mean relative error the reference's harness reports equals the FP64
    oracle's to within 1e-3 percentage points."""
    from gproshan_gb300 import _capi
    from test_oracle import _closed_form_cases, mean_rel_err_pct
    name, xyz, tri, src, exact = _closed_form_cases()[case]
    m = dev_mesh(gpu_ctx, xyz, tri)
    d, _, st = _capi.ptp(m, [src])
    om = oracle_lib.Mesh(xyz, tri)
    ref = oracle_lib.ptp(om, [src], xyz=xyz.astype(np.float32).astype(np.float64))
    assert st.n_iter == ref["n_iter"]
    e_gpu = mean_rel_err_pct(d.astype(np.float64), exact)
    e_ref = mean_rel_err_pct(ref["dist"], exact)
    assert abs(e_gpu - e_ref) < 1e-3, (name, e_gpu, e_ref)


def _uv_sphere(n_lon=64, n_lat=48):
    """Latitude-longitude sphere: two poles of valence n_lon (rows past 8
    entries, read from the CSR lists) surrounded by needle triangles."""
    th = np.linspace(0, np.pi, n_lat + 1)[1:-1]
    ph = np.linspace(0, 2 * np.pi, n_lon, endpoint=False)
    T, P = np.meshgrid(th, ph, indexing="ij")
    ring = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1).reshape(-1, 3)
    xyz = np.concatenate([[[0.0, 0.0, 1.0]], ring, [[0.0, 0.0, -1.0]]])
    south = len(xyz) - 1
    idx = lambda r, c: 1 + r * n_lon + c % n_lon
    tri = []
    for c in range(n_lon):
        tri.append([0, idx(0, c), idx(0, c + 1)])
        tri.append([south, idx(n_lat - 2, c + 1), idx(n_lat - 2, c)])
        for r in range(n_lat - 2):
            a, b, cc, d = idx(r, c), idx(r, c + 1), idx(r + 1, c), idx(r + 1, c + 1)
            tri += [[a, cc, b], [b, cc, d]]
    return xyz, np.array(tri, np.uint32)


@pytest.mark.parametrize("src", [[0], [1000], [0, 1500]])
def test_high_valence_poles_on_the_grid_launch(gpu_ctx, oracle_lib, src):
    """Vertices of valence 64 swept by the grid-wide lockstep launch: FP64
    bit-exact with the oracle, FP32 within the bar with the same sweeps, with
    and without labels."""
    from gproshan_gb300 import _capi
    xyz, tri = _uv_sphere()
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    _, s_o, l_o = oracle_lib.toplesets(om, src)
    kw = dict(local_window=1, grid_kernel=_capi.GP_GRID_LOCKSTEP)
    ref = oracle_lib.ptp(om, src, l_o, s_o)
    d64, _, st = _capi.ptp(m, src, dtype=np.float64, opts=_capi.make_opts(_capi.GP_F64, **kw))
    assert gpu_ctx.call_stats().fields_grid == 1
    assert st.n_iter == ref["n_iter"] and np.array_equal(d64, ref["dist"])
    ref32 = oracle_lib.ptp(om, src, l_o, s_o, xyz=xyz.astype(np.float32).astype(np.float64))
    d32, _, st32 = _capi.ptp(m, src, opts=_capi.make_opts(_capi.GP_F32, **kw))
    assert st32.n_iter == ref32["n_iter"]
    assert oracle_lib.max_rel_err(d32, ref32["dist"]) <= REL_TOL_F32
    d32c, _, st32c = _capi.ptp(m, src, clusters=np.zeros(len(xyz), np.uint32), opts=_capi.make_opts(_capi.GP_F32, **kw))
    assert st32c.n_iter == ref32["n_iter"]
    assert oracle_lib.max_rel_err(d32c, ref32["dist"]) <= REL_TOL_F32


@pytest.mark.parametrize("n,seeds,radio", [(10000, [0, 50], 0.0), (20, [3], 10.0), (1, [3], 0.0), (30, [7, 7], 0.0)],
                         ids=["n_above_vertices", "radius_at_first", "no_new_sample", "repeated_seed"])
def test_fps_device_loop_edge_cases(gpu_ctx, oracle_lib, n, seeds, radio):
    """The device sample loop at its edges, against the oracle (FP64 path):
    n at or above the vertex count is clamped to half of it, as the reference
    does; a radius larger than the first field's farthest distance stops after
    one new sample; n not above the seeds adds nothing; a repeated seed."""
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = meshgen.icosphere(2, 0.1, 5)
    m = dev_mesh(gpu_ctx, xyz, tri)
    om = oracle_lib.Mesh(xyz, tri)
    s_ref, md_ref = oracle_lib.fps(om, n, seeds, radio=radio)
    s, md, _ = _capi.fps(m, n, seeds, radio=radio, precision=_capi.GP_F64)
    assert np.array_equal(s, s_ref)
    assert md == md_ref or (np.isinf(md) and np.isinf(md_ref))


def test_normalize_option_with_labels(gpu_ctx, oracle_lib):
    """normalize and cluster labels in one FP64 call: distances are
    normalize_ptp of the plain ones, labels unchanged, bit for bit."""
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = meshgen.icosphere(4, 0.1, 2)
    m = dev_mesh(gpu_ctx, xyz, tri)
    src = [0, 1000, 2000]
    d0, c0, _ = _capi.ptp(m, src, dtype=np.float64, precision=_capi.GP_F64, clusters=np.zeros(len(xyz), np.uint32))
    d1, c1, _ = _capi.ptp(m, src, dtype=np.float64, clusters=np.zeros(len(xyz), np.uint32),
                          opts=_capi.make_opts(_capi.GP_F64, normalize=True))
    assert np.array_equal(c0, c1)
    assert np.array_equal(d1, oracle_lib.normalize_ptp(d0))
