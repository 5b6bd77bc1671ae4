"""CUDA-graph plans and the autotuner: a captured batch replays to the same
bits as gp_ptp_batch, picks up new sources written in place between launches,
and the autotuner's choice changes speed only, never results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _workload(ctx, seed):
    from gproshan_gb300 import _capi, meshgen
    meshes = [_capi.DeviceMesh(ctx, *meshgen.icosphere(4, 0.1, 1)),
              _capi.DeviceMesh(ctx, *meshgen.height_field(150, 2)),
              _capi.DeviceMesh(ctx, *meshgen.height_field(6, 3, cols=500)),
              _capi.DeviceMesh(ctx, *meshgen.torus(40, 90, seed=2))]
    rng = np.random.default_rng(seed)
    ms, srcs = [], []
    for k in range(11):
        m = meshes[k % len(meshes)]
        ms.append(m)
        srcs.append(rng.choice(m.n_vertices, size=1 + k % 3, replace=False).astype(np.uint32))
    return meshes, ms, srcs


@pytest.mark.parametrize("learned", [False, True])
def test_plan_replays_batch_bit_exact(gpu_ctx, learned):
    torch = pytest.importorskip("torch")
    from gproshan_gb300 import _capi
    from gproshan_gb300 import learned as L
    meshes, ms, srcs = _workload(gpu_ctx, 5)
    sched = _capi.GP_SCHED_LEARNED if learned else _capi.GP_SCHED_REACTIVE
    if learned:
        L.install(gpu_ctx)
    try:
        soff = np.concatenate([[0], np.cumsum([len(s) for s in srcs])])
        voff = np.concatenate([[0], np.cumsum([m.n_vertices for m in ms])])
        src_dev = torch.from_numpy(np.concatenate(srcs).astype(np.int32)).cuda()
        dist_dev = torch.empty(int(voff[-1]), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        sp, dp = src_dev.data_ptr(), dist_dev.data_ptr()
        plan = _capi.Plan(gpu_ctx, ms, [(sp + 4 * int(soff[k]), len(srcs[k])) for k in range(len(ms))],
                          [dp + 4 * int(voff[k]) for k in range(len(ms))],
                          opts=_capi.make_opts(schedule=sched))
        for rnd in range(3):
            plan.launch()
            st = plan.wait()
            got = dist_dev.cpu().numpy()
            ref, rst, _ = _capi.ptp_batch(gpu_ctx, ms, srcs, schedule=sched)
            for k in range(len(ms)):
                assert np.array_equal(got[voff[k]:voff[k + 1]], ref[k]), (rnd, k)
                assert st[k].n_iter == rst[k].n_iter and st[k].relaxations == rst[k].relaxations
            # new sources, same counts, written in place
            rng = np.random.default_rng(100 + rnd)
            srcs = [rng.choice(m.n_vertices, size=len(s), replace=False).astype(np.uint32) for m, s in zip(ms, srcs)]
            src_dev.copy_(torch.from_numpy(np.concatenate(srcs).astype(np.int32)))
            torch.cuda.synchronize()
        plan.close()
    finally:
        _capi.set_cost_model(gpu_ctx, None)


def test_plan_rejects_labels_and_bad_sources(gpu_ctx):
    torch = pytest.importorskip("torch")
    from gproshan_gb300 import _capi, meshgen
    m = _capi.DeviceMesh(gpu_ctx, *meshgen.icosphere(3, 0.1, 1))
    src = torch.tensor([0, m.n_vertices + 5], dtype=torch.int32, device="cuda")
    dist = torch.empty(m.n_vertices, dtype=torch.float32, device="cuda")
    lab = torch.zeros(m.n_vertices, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    fields = (_capi.gp_field * 1)()
    fields[0].mesh = m.handle
    fields[0].sources = src.data_ptr()
    fields[0].n_sources = 1
    fields[0].dist = dist.data_ptr()
    fields[0].clusters = lab.data_ptr()
    h = _capi.C.c_void_p()
    o = _capi.make_opts()
    st = _capi.lib().gp_plan_create(gpu_ctx.handle, fields, 1, _capi.C.byref(o), _capi.GP_F32, _capi.C.byref(h))
    assert st == _capi.GP_ERR_INVALID_ARG and not h.value
    # an out-of-range source id found on the device is reported by wait()
    plan = _capi.Plan(gpu_ctx, [m], [(src.data_ptr() + 4, 1)], [dist.data_ptr()])
    plan.launch()
    with pytest.raises(_capi.GPError):
        plan.wait()
    plan.close()
    # the context still works
    d, _, _ = _capi.ptp(m, [0])
    assert d[0] == 0


def test_autotune_choice_keeps_results(gpu_ctx):
    from gproshan_gb300 import _capi
    meshes, ms, srcs = _workload(gpu_ctx, 9)
    o = _capi.autotune(gpu_ctx, ms, srcs, reps=1)
    assert o.local_window in (1024, 2048, 4096, 8192, 16384)
    assert o.grid_kernel in (_capi.GP_GRID_LOCKSTEP, _capi.GP_GRID_QUEUE)
    if o.grid_kernel == _capi.GP_GRID_QUEUE:
        assert o.queue_tile in (64, 128, 256)
    ref, rst, _ = _capi.ptp_batch(gpu_ctx, ms, srcs)
    outs = [np.empty(m.n_vertices, np.float32) for m in ms]
    fields, keep = _capi._fields(ms, srcs, outs)
    sec = _capi.C.c_double()
    gpu_ctx.check(_capi.lib().gp_ptp_batch(gpu_ctx.handle, fields, len(ms), _capi.C.byref(o), _capi.GP_F32, 0,
                                           _capi.C.byref(sec)), "gp_ptp_batch")
    for k in range(len(ms)):
        assert np.array_equal(outs[k], ref[k]), k


def test_sharded_front_end_on_one_rank(gpu_ctx):
    """gproshan_gb300.shard on a single process: the cost model's predicted
    relaxations come from the GPU (toplesets features + BF16 MLP), are positive
    and grow with the mesh, and ptp_sharded returns every field, in the
    caller's order, bit for bit equal to one gp_ptp_batch call."""
    from gproshan_gb300 import _capi, meshgen, shard
    ms = [_capi.DeviceMesh(gpu_ctx, *meshgen.icosphere(3, 0.1, 1)),
          _capi.DeviceMesh(gpu_ctx, *meshgen.height_field(120, 2)),
          _capi.DeviceMesh(gpu_ctx, *meshgen.icosphere(5, 0.1, 3))]
    meshes = [ms[0], ms[1], ms[2], ms[1], ms[0]]
    srcs = [[0], [5], [17], [9000, 3], [600]]
    c = shard.predicted_costs(gpu_ctx, meshes, srcs)
    assert c.shape == (5,) and np.all(c > 0) and c[2] > c[0]
    full, mine, parts = shard.ptp_sharded(gpu_ctx, meshes, srcs)
    assert parts == [list(range(5))] and mine == list(range(5))
    ref, _, _ = _capi.ptp_batch(gpu_ctx, meshes, srcs)
    for a, b in zip(full, ref):
        assert np.array_equal(a, b)


def test_host_outputs_back_to_back_and_scattered(gpu_ctx):
    """Host output arrays that lie back to back in one buffer (downloaded in
    merged copies) and arrays scattered in memory give the same distances."""
    import ctypes as C
    from gproshan_gb300 import _capi, meshgen
    ms = [_capi.DeviceMesh(gpu_ctx, *meshgen.icosphere(3, 0.1, 1)),
          _capi.DeviceMesh(gpu_ctx, *meshgen.height_field(90, 2))]
    meshes = [ms[0], ms[1], ms[1], ms[0], ms[1]]
    srcs = [[0], [5], [70], [9], [8000]]
    ref, _, _ = _capi.ptp_batch(gpu_ctx, meshes, srcs)
    nv = [m.n_vertices for m in meshes]
    buf = np.full(sum(nv) + 7, -1.0, np.float32)
    off = np.concatenate([[0], np.cumsum(nv)])
    # fields 0-2 back to back, field 3 after a gap, field 4 in its own array
    views = [buf[off[0]:off[1]], buf[off[1]:off[2]], buf[off[2]:off[3]], buf[off[3] + 7:off[4] + 7],
             np.empty(nv[4], np.float32)]
    fields, keep = _capi._fields(meshes, srcs, views)
    o = _capi.make_opts(_capi.GP_F32)
    sec = C.c_double()
    gpu_ctx.check(_capi.lib().gp_ptp_batch(gpu_ctx.handle, fields, len(meshes), C.byref(o), _capi.GP_F32, 0,
                                           C.byref(sec)), "gp_ptp_batch")
    for a, b in zip(views, ref):
        assert np.array_equal(a, b)
    assert (buf[off[3]:off[3] + 7] == -1.0).all()  # the gap is left alone
