"""Toplesets built inside the lockstep sweep launch (gp_ptp_opts.stream_min).

Worker CTAs of the grid-wide launch build the BFS and the ring renumbering of
the streamed fields while the other CTAs sweep; a streamed field opens each
window once the rings it reads are renumbered.  The sweeps are the same sweeps
in the same order, so every output -- distances, sweep counts, relaxations --
equals bit for bit the launch that builds every field's toplesets first
(stream_min = 0xFFFFFFFF), and the FP32 bar against the FP64 oracle holds.
"""
import numpy as np
import pytest

from conftest import golden_cases

pytestmark = pytest.mark.gpu

NEVER = 0xFFFFFFFF
REL_TOL_F32 = 1e-5


def _run(ctx, ms, srcs, stream_min, **kw):
    from gproshan_gb300 import _capi
    d, st, _ = _capi.ptp_batch(ctx, ms, srcs, grid_kernel=_capi.GP_GRID_LOCKSTEP, stream_min=stream_min, **kw)
    return d, [(s.n_iter, s.relaxations) for s in st], ctx.call_stats()


def _meshes(ctx):
    from gproshan_gb300 import _capi, meshgen
    gen = [meshgen.icosphere(5, 0.1, 3), meshgen.height_field(200, 8), meshgen.height_field(8, 5, cols=900),
           meshgen.torus(80, 200, seed=1), meshgen.icosphere(3, 0.1, 1)]
    gen += [(g["xyz"], g["tri"]) for n, g in golden_cases() if n in ("grid_hole", "two_components", "grid24")]
    return gen, [_capi.DeviceMesh(ctx, x, t) for x, t in gen]


@pytest.mark.parametrize("stream_min,local_window", [(1, 1), (1, 0), (3000, 1)])
def test_streamed_fields_bit_identical(gpu_ctx, oracle_lib, stream_min, local_window):
    gen, dms = _meshes(gpu_ctx)
    rng = np.random.default_rng(11 + stream_min)
    ms, srcs, mi = [], [], []
    for k in range(40):
        q = k % len(dms)
        ms.append(dms[q])
        mi.append(q)
        s = rng.choice(dms[q].n_vertices, size=1 + k % 3, replace=False)
        if k % 7 == 3:
            s = np.concatenate([s, s[:1]])  # a repeated source
        srcs.append(s)
    a, sa, ca = _run(gpu_ctx, ms, srcs, stream_min, local_window=local_window)
    b, sb, cb = _run(gpu_ctx, ms, srcs, NEVER, local_window=local_window)
    assert ca.fields_streamed > 0 and cb.fields_streamed == 0
    assert sa == sb
    for k in range(len(ms)):
        assert np.array_equal(a[k], b[k]), k
    for k in (0, 3, 5, 6, 7):  # icosphere, torus, mesh with a hole, two components (unreached vertices)
        x, t = gen[mi[k]]
        om = oracle_lib.Mesh(x, t)
        ref = oracle_lib.ptp(om, srcs[k], xyz=x.astype(np.float32).astype(np.float64))
        assert sa[k][0] == ref["n_iter"], k
        assert oracle_lib.max_rel_err(a[k], ref["dist"]) <= REL_TOL_F32, k


def test_single_streamed_field_and_learned_schedule(gpu_ctx):
    """One large field alone (one worker CTA, the rest sweeping), and a batch
    under the learned schedule: same bits as without streaming."""
    from gproshan_gb300 import _capi, learned, meshgen
    m = _capi.DeviceMesh(gpu_ctx, *meshgen.height_field(400, 3))
    for src in ([0], [12345, 160000 - 1]):
        a, sa, ca = _run(gpu_ctx, [m], [src], 1)
        b, sb, _ = _run(gpu_ctx, [m], [src], NEVER)
        assert ca.fields_streamed == 1 and sa == sb and np.array_equal(a[0], b[0])
    learned.install(gpu_ctx)
    try:
        _, dms = _meshes(gpu_ctx)
        rng = np.random.default_rng(3)
        ms = [dms[k % len(dms)] for k in range(24)]
        srcs = [rng.choice(x.n_vertices, size=1, replace=False) for x in ms]
        a, sa, ca = _run(gpu_ctx, ms, srcs, 1, schedule=_capi.GP_SCHED_LEARNED)
        b, sb, _ = _run(gpu_ctx, ms, srcs, NEVER, schedule=_capi.GP_SCHED_LEARNED)
        assert ca.fields_streamed > 0 and sa == sb
        assert all(np.array_equal(x, y) for x, y in zip(a, b))
    finally:
        _capi.set_cost_model(gpu_ctx, None)


def test_streaming_off_where_it_does_not_apply(gpu_ctx):
    """The default (stream_min 0), labels, FP64 and the work-queue launch
    stream nothing; a threshold streams only the meshes at or above it."""
    from gproshan_gb300 import _capi, meshgen
    small = _capi.DeviceMesh(gpu_ctx, *meshgen.icosphere(4, 0.1, 2))
    _run(gpu_ctx, [small, small], [[0], [5]], 0)
    assert gpu_ctx.call_stats().fields_streamed == 0
    _capi.ptp_batch(gpu_ctx, [small], [[0]], grid_kernel=_capi.GP_GRID_QUEUE, queue_min=1, stream_min=1)
    assert gpu_ctx.call_stats().fields_streamed == 0
    _capi.ptp_batch(gpu_ctx, [small], [[0]], dtype=np.float64, precision=_capi.GP_F64, stream_min=1)
    assert gpu_ctx.call_stats().fields_streamed == 0
    _capi.ptp_batch(gpu_ctx, [small], [[0]], clusters=[np.zeros(small.n_vertices, np.uint32)], stream_min=1)
    assert gpu_ctx.call_stats().fields_streamed == 0
    big = _capi.DeviceMesh(gpu_ctx, *meshgen.height_field(520, 1))
    _run(gpu_ctx, [big, small], [[7], [0]], 0)
    assert gpu_ctx.call_stats().fields_streamed == 0
    _run(gpu_ctx, [big, small], [[7], [0]], 1 << 18)
    assert gpu_ctx.call_stats().fields_streamed == 1


def test_default_streams_large_fields_of_larger_calls(gpu_ctx):
    """stream_min 0 (the default) streams the fields on meshes of at least
    2^18 vertices once a call has more than 8 fields, and never in smaller
    calls, whose large fields build their toplesets with the whole GPU; once
    the streamed fields' toplesets are done the streaming launch ends and a
    launch of the plain kernel sweeps the rest, and every output equals the
    unstreamed call's."""
    from gproshan_gb300 import _capi, meshgen
    big = _capi.DeviceMesh(gpu_ctx, *meshgen.height_field(520, 1))
    big2 = _capi.DeviceMesh(gpu_ctx, *meshgen.torus(200, 1400, seed=2))
    _, dms = _meshes(gpu_ctx)
    rng = np.random.default_rng(5)
    ms = [big, big2, big] + [dms[k % len(dms)] for k in range(9)]
    srcs = [rng.choice(m.n_vertices, size=1 + k % 2, replace=False) for k, m in enumerate(ms)]
    a, sa, ca = _run(gpu_ctx, ms, srcs, 0)
    assert ca.fields_streamed == 3
    b, sb, cb = _run(gpu_ctx, ms, srcs, NEVER)
    assert cb.fields_streamed == 0 and sa == sb
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    _run(gpu_ctx, ms[:8], srcs[:8], 0)
    assert gpu_ctx.call_stats().fields_streamed == 0


def test_streamed_fields_with_normalize(gpu_ctx):
    """normalize in a call with streamed fields (the maximum reduced in the
    output gather, after both grid launches): the same bits as the unstreamed
    normalized call, and each field is its plain output over its largest
    finite distance."""
    from gproshan_gb300 import _capi, meshgen
    big = _capi.DeviceMesh(gpu_ctx, *meshgen.height_field(520, 1))
    _, dms = _meshes(gpu_ctx)
    ms = [big, dms[0], big] + dms[1:8]
    srcs = [[3], [0], [200000]] + [[1]] * 7
    plain, _, _ = _run(gpu_ctx, ms, srcs, NEVER)
    L = _capi.lib()
    got = {}
    for smin in (1 << 18, NEVER):
        outs = [np.empty(m.n_vertices, np.float32) for m in ms]
        fields, keep = _capi._fields(ms, srcs, outs)
        o = _capi.make_opts(_capi.GP_F32, normalize=True, grid_kernel=_capi.GP_GRID_LOCKSTEP, stream_min=smin)
        sec = _capi.C.c_double()
        gpu_ctx.check(L.gp_ptp_batch(gpu_ctx.handle, fields, len(ms), _capi.C.byref(o), _capi.GP_F32, 0,
                                     _capi.C.byref(sec)), "batch")
        got[smin] = (outs, gpu_ctx.call_stats().fields_streamed)
    assert got[1 << 18][1] == 2 and got[NEVER][1] == 0
    for a, b, p in zip(got[1 << 18][0], got[NEVER][0], plain):
        assert np.array_equal(a, b)
        ref = p.copy()
        ref /= np.float32(np.max(ref[np.isfinite(ref)]))
        assert np.array_equal(a, ref)


def test_streaming_launch_gives_up_cleanly(gpu_ctx):
    """A grid barrier that cannot complete (test hook: one arrival more than
    the launch has) with streamed fields in the launch: the sweeping CTAs give
    up after their poll limit, the workers leave their BFS on the abort flag,
    the launch that would resume the sweeps sees it and returns, the call
    reports GP_ERR_DEVICE_TIMEOUT, and the context then gives the unstreamed
    call's bits."""
    from gproshan_gb300 import _capi, meshgen
    big = _capi.DeviceMesh(gpu_ctx, *meshgen.height_field(520, 1))
    _, dms = _meshes(gpu_ctx)
    ms = [big, big] + dms[:8]
    srcs = [[7], [1000]] + [[0]] * 8
    ref, rst, _ = _run(gpu_ctx, ms, srcs, NEVER)
    L = _capi.lib()
    gpu_ctx.check(L.gp_ctx_debug_barrier(gpu_ctx.handle, 4000, 1), "gp_ctx_debug_barrier")
    try:
        with pytest.raises(_capi.GPError) as e:
            _run(gpu_ctx, ms, srcs, 1)
        assert e.value.status == _capi.GP_ERR_DEVICE_TIMEOUT
    finally:
        gpu_ctx.check(L.gp_ctx_debug_barrier(gpu_ctx.handle, 0, 0), "gp_ctx_debug_barrier")
    d, st, cs = _run(gpu_ctx, ms, srcs, 1)
    assert cs.fields_streamed >= 2 and st == rst
    assert all(np.array_equal(x, y) for x, y in zip(d, ref))


def test_streamed_plan_replays_bit_exact(gpu_ctx):
    """A captured plan (CUDA graph) with streamed fields: every replay, with
    sources rewritten in place between launches, gives the bits of the
    unstreamed batched call, including a source outside the mesh, which the
    device reports and which leaves that field empty."""
    torch = pytest.importorskip("torch")
    from gproshan_gb300 import _capi
    _, dms = _meshes(gpu_ctx)
    ms = [dms[k % len(dms)] for k in range(12)]
    rng = np.random.default_rng(21)
    srcs = [rng.choice(m.n_vertices, size=1 + k % 2, replace=False).astype(np.uint32) for k, m in enumerate(ms)]
    soff = np.concatenate([[0], np.cumsum([len(s) for s in srcs])])
    voff = np.concatenate([[0], np.cumsum([m.n_vertices for m in ms])])
    src_dev = torch.from_numpy(np.concatenate(srcs).astype(np.int32)).cuda()
    dist_dev = torch.empty(int(voff[-1]), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    sp, dp = src_dev.data_ptr(), dist_dev.data_ptr()
    plan = _capi.Plan(gpu_ctx, ms, [(sp + 4 * int(soff[k]), len(srcs[k])) for k in range(len(ms))],
                      [dp + 4 * int(voff[k]) for k in range(len(ms))],
                      opts=_capi.make_opts(grid_kernel=_capi.GP_GRID_LOCKSTEP, stream_min=1))
    try:
        for rnd in range(3):
            plan.launch()
            st = plan.wait()
            got = dist_dev.cpu().numpy()
            ref, rst, _ = _capi.ptp_batch(gpu_ctx, ms, srcs, grid_kernel=_capi.GP_GRID_LOCKSTEP, stream_min=NEVER)
            for k in range(len(ms)):
                assert np.array_equal(got[voff[k]:voff[k + 1]], ref[k]), (rnd, k)
                assert st[k].n_iter == rst[k].n_iter and st[k].relaxations == rst[k].relaxations
            srcs = [rng.choice(m.n_vertices, size=len(s), replace=False).astype(np.uint32) for m, s in zip(ms, srcs)]
            src_dev.copy_(torch.from_numpy(np.concatenate(srcs).astype(np.int32)))
            torch.cuda.synchronize()
        # a source outside the mesh in a streamed field: reported, the rest unaffected
        bad = np.concatenate(srcs).astype(np.int64)
        bad[0] = ms[0].n_vertices + 3
        src_dev.copy_(torch.from_numpy(bad.astype(np.int32)))
        torch.cuda.synchronize()
        plan.launch()
        with pytest.raises(_capi.GPError):
            plan.wait()
    finally:
        plan.close()
    d, _, _ = _capi.ptp(ms[1], srcs[1])  # the context still works
    assert np.isfinite(d).any()
