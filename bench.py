"""Benchmark: distance fields/s of batched PTP geodesics on GB300.

Workload (the batched configuration): 64 seeded meshes of uneven size
(icospheres subdivided 3-7 times, tangentially jittered, and sinusoid height
fields with sides 64-1024, log-uniform) carrying 256 independent single-source
fields (4 seeded sources per mesh), FP32.  Synthetic meshes stand in for the
reference's .off inputs.

One step = every field of the workload solved once: GPU toplesets, ring
renumbering, sweeps, gather.  The timed region brackets K steps with CUDA
events on the library's stream.

* value   -- batched: all 256 fields in one gp_ptp_batch call, sources and
             outputs resident in HBM;
* plain   -- the same fields one gp_ptp_batch call each (the single-field GPU
             PTP), same GPU, same kernels;
* e2e     -- batched through the C ABI with HOST buffers (page-locked): sources copied in,
             distances copied out every step (meshes stay resident, as a
             reference `che` does between calls);
* roofline -- the sweep launch's algorithmic bytes (48 per relaxation) over
             its CUDA-event time, against the measured HBM copy bandwidth;
* cpu_baseline -- the reference's own CPU PTP (FP64, every host core) on one
             field of every mesh up to 400k vertices, scaled by the GPU-counted
             relaxations of each mesh's fields; the same fields also check the
             GPU result against the FP64 oracle (oracle_check);
* clocks, gpu_launches -- SM clocks sampled during the timed region, and the
             library's kernel launches inside it.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
``--impl reference`` times the reference's own CPU PTP (geodesics PTP_CPU:
toplesets + parallel_toplesets_propagation_coalescence_cpu) on every host
core over the whole workload: the K timed steps take the fields in a seeded
order, 256 / K each, so together they solve every field exactly once.
Under torchrun each rank solves its own 256-field workload (seed offset by
rank; weak scaling), and rank 0 prints one JSON line.

``--config single|grid2048|torus|fps`` instead measures one of the other
workloads (a single 40,962-vertex icosphere field in FP32 and FP64; one
2048^2 height field with 4 sources; a 1M-vertex anisotropic torus, one field
with 16 sources and 16 single-source fields batched vs plain; farthest-point
sampling of 512 points on a 2M-vertex bump field) and prints one JSON line
for it.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_MESHES = 64
FIELDS_PER_MESH = 4
ALGO_BYTES_PER_RELAX = 48  # per interior vertex relaxation, FP32 values + 32-bit indices
METRIC = "distance fields/s, batched vs plain PTP on same GB300 at max rel err <=1e-5"
WORKLOAD = "batch_mix64: 256 single-source fields on 64 seeded meshes (icospheres L3-7, height fields 64^2-1024^2)"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def shard_seed(base: int, rank: int) -> int:
    """Seed of a rank's workload: weak scaling, every rank has its own fields."""
    return base + 1000003 * rank


def make_workload(seed: int, n_meshes: int = N_MESHES):
    from gproshan_gb300 import meshgen
    meshes = meshgen.batch_mix(n_meshes, seed)
    rng = np.random.default_rng(seed + 17)
    fields = []
    for mi, (name, xyz, tri) in enumerate(meshes):
        for _ in range(FIELDS_PER_MESH):
            fields.append((mi, int(rng.integers(0, len(xyz)))))
    return meshes, fields


# --------------------------------------------------------------------------
# clocks sampled during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------
# the GPU arm
# --------------------------------------------------------------------------
def run_gpu(args, rank, world, local):
    import torch
    from gproshan_gb300 import _capi, build, learned

    build.build()
    torch.cuda.set_device(local)
    ctx = _capi.Context(local)
    L = _capi.lib()
    meshes, fields = make_workload(shard_seed(args.seed, rank), args.meshes)
    dmesh = [_capi.DeviceMesh(ctx, xyz, tri) for _, xyz, tri in meshes]
    F = len(fields)
    nv = [dmesh[mi].n_vertices for mi, _ in fields]

    # device-resident sources and outputs (one buffer, per-field views)
    src_host = np.array([s for _, s in fields], dtype=np.uint32)
    src_dev = torch.from_numpy(src_host.astype(np.int32)).cuda()
    voff = np.concatenate([[0], np.cumsum(nv)]).astype(np.int64)
    dist_dev = torch.empty(int(voff[-1]), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    def field_array(device: bool, host_out=None, host_src=None):
        arr = (_capi.gp_field * F)()
        for k, (mi, s) in enumerate(fields):
            arr[k].mesh = dmesh[mi].handle
            if device:
                arr[k].sources = src_dev.data_ptr() + 4 * k
                arr[k].dist = dist_dev.data_ptr() + 4 * int(voff[k])
            else:
                arr[k].sources = host_src.ctypes.data + 4 * k
                arr[k].dist = host_out[k].ctypes.data
            arr[k].n_sources = 1
        return arr

    dev_fields = field_array(True)
    sched = _capi.GP_SCHED_LEARNED if args.schedule == "learned" else _capi.GP_SCHED_REACTIVE
    if sched == _capi.GP_SCHED_LEARNED:
        learned.install(ctx)
    gk = {"auto": _capi.GP_GRID_AUTO, "lockstep": _capi.GP_GRID_LOCKSTEP, "queue": _capi.GP_GRID_QUEUE}
    opts = _capi.make_opts(_capi.GP_F32, schedule=sched, grid_kernel=gk[args.grid_kernel],
                           queue_tile=args.queue_tile)
    tuned = None
    if args.autotune and args.grid_kernel == "auto":
        # the library's autotuner picks the one-CTA window and the grid launch
        # for this workload (untimed; every candidate gives the same results;
        # best of 3 per candidate: the windows' times differ by ~1 %)
        opts = _capi.autotune(ctx, [dmesh[mi] for mi, _ in fields], [[s] for _, s in fields], opts=opts, reps=3)
        tuned = {"local_window": opts.local_window, "grid_kernel": {1: "lockstep", 2: "queue"}[opts.grid_kernel],
                 "queue_tile": opts.queue_tile}
    sec = C.c_double()
    stream = torch.cuda.ExternalStream(ctx.stream)

    def batched_call():
        ctx.check(L.gp_ptp_batch(ctx.handle, dev_fields, F, C.byref(opts), _capi.GP_F32,
                                 _capi.GP_BATCH_DEVICE_POINTERS, C.byref(sec)), "gp_ptp_batch")
        return ctx.call_stats()

    plan = None
    if args.graph:
        # the whole batched call captured once in a CUDA graph, replayed per step
        plan = _capi.Plan(ctx, [dmesh[mi] for mi, _ in fields],
                          [(src_dev.data_ptr() + 4 * k, 1) for k in range(F)],
                          [dist_dev.data_ptr() + 4 * int(voff[k]) for k in range(F)], opts=opts)

        def batched():
            plan.launch()
            return None
    else:
        batched = batched_call

    plain_opts = _capi.make_opts(_capi.GP_F32)

    def plain():
        st = []
        for k in range(F):
            ctx.check(L.gp_ptp_batch(ctx.handle, C.byref(dev_fields[k]), 1, C.byref(plain_opts), _capi.GP_F32,
                                     _capi.GP_BATCH_DEVICE_POINTERS, C.byref(sec)), "gp_ptp_batch")
            st.append(ctx.call_stats())
        return st

    def timed(fn, steps, warmup, tag):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        outs = []
        torch.cuda.nvtx.range_push(tag)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(steps):
                outs.append(fn())
            e1.record(stream)
        e1.synchronize()
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if world > 1:
            t = torch.tensor([ms], dtype=torch.float64, device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms / steps, outs

    with ClockSampler(local) as clk:
        ms_batched, stats = timed(batched, args.steps, args.warmup, "batched")
    clocks = clk.summary()
    if plan is not None:
        plan.wait()  # device-side errors of the replays
        # phase times and counts of the same call (the graph carries no events)
        stats = [batched_call() for _ in range(2)]

    # the same batch with the reactive schedule (every field starts on one CTA;
    # no cost model), otherwise the same options, timed the same way: what the
    # learned schedule buys on this workload, with bit-identical distances
    dist_learned = dist_dev.cpu().numpy().copy()
    learned_over_reactive = None
    if plan is not None and sched == _capi.GP_SCHED_LEARNED and not args.only_batched:
        ropts = _capi.make_opts(_capi.GP_F32, schedule=_capi.GP_SCHED_REACTIVE, grid_kernel=opts.grid_kernel,
                                queue_tile=opts.queue_tile, local_window=opts.local_window)
        rplan = _capi.Plan(ctx, [dmesh[mi] for mi, _ in fields],
                           [(src_dev.data_ptr() + 4 * k, 1) for k in range(F)],
                           [dist_dev.data_ptr() + 4 * int(voff[k]) for k in range(F)], opts=ropts)

        def reactive():
            rplan.launch()
            return None

        ms_reactive, _ = timed(reactive, args.steps, args.warmup, "reactive")
        rplan.wait()
        learned_over_reactive = {"ratio": ms_reactive / ms_batched, "ms_reactive": ms_reactive,
                                 "ms_learned": ms_batched,
                                 "bit_identical": bool(np.array_equal(dist_dev.cpu().numpy(), dist_learned))}
        del rplan

    # accuracy of the batched result vs the FP64 path of the same library on
    # every field, on the same float-rounded coordinates (the FP64 path is
    # bit-exact with the CPU oracle in the tests)
    dist32 = dist_dev.cpu().numpy()
    err = 0.0
    sched_equal = None
    field_relax = None
    if not args.skip_check:
        fm = [dmesh[mi] for mi, _ in fields]
        fsrc = [[s] for _, s in fields]
        d64s, st64, _ = _capi.ptp_batch(ctx, fm, fsrc, dtype=np.float64, precision=_capi.GP_F64, round_coords=True)
        d32s, st32, _ = _capi.ptp_batch(ctx, fm, fsrc, dtype=np.float32, precision=_capi.GP_F32)
        sched_equal = sum(int(a.n_iter == b.n_iter) for a, b in zip(st32, st64))
        field_relax = [(int(a.relaxations), int(a.n_iter)) for a in st32]
        for k in range(len(fields)):
            ref = d64s[k]
            a = dist32[voff[k]:voff[k + 1]].astype(np.float64)
            if not np.array_equal(d32s[k], dist32[voff[k]:voff[k + 1]]):
                err = float("inf")  # device-pointer and host-pointer runs must agree bit for bit
                break
            fin = np.isfinite(ref) & (ref > 0)
            if np.any(np.isfinite(a) != np.isfinite(ref)):
                err = float("inf")
                break
            if fin.any():
                err = max(err, float(np.max(np.abs(a[fin] - ref[fin]) / ref[fin])))

    # plain single-field GPU PTP over the same fields (5 timed passes after 2
    # warm-ups: each pass is ~0.8 s)
    plain_steps = max(1, min(args.steps, 5))
    if args.only_batched:
        ms_plain, pstats = float("nan"), [[]]
    else:
        ms_plain, pstats = timed(plain, plain_steps, 2, "plain")

    # e2e with host buffers through the same C entry point
    src_pinned = torch.from_numpy(src_host.view(np.int32)).pin_memory()
    # results land in page-locked host memory (one buffer, per-field views)
    out_pinned = torch.empty(int(voff[-1]), dtype=torch.float32).pin_memory()
    out_np = out_pinned.numpy()
    host_out = [out_np[voff[k]:voff[k + 1]] for k in range(F)]
    host_fields = field_array(False, host_out, src_pinned.numpy().view(np.uint32))

    def e2e():
        ctx.check(L.gp_ptp_batch(ctx.handle, host_fields, F, C.byref(opts), _capi.GP_F32, 0, C.byref(sec)),
                  "gp_ptp_batch(host)")
        return ctx.call_stats()

    if args.only_batched:
        ms_e2e, estats = float("nan"), [stats[-1]]
    else:
        ms_e2e, estats = timed(e2e, args.steps, args.warmup, "e2e")
    same = all(np.array_equal(host_out[k], dist32[voff[k]:voff[k + 1]]) for k in range(F))

    strong = None
    if world > 1:
        try:
            strong = strong_scaling(args, ctx, rank, world, timed)
        except Exception as exc:  # the weak-scaling line must survive a failure of this extra leg
            strong = {"error": f"{type(exc).__name__}: {exc}"}

    s0 = stats[-1]
    relax_total = int(s0.relax_local + s0.relax_grid)
    return {
        "ms_batched": ms_batched, "ms_plain": ms_plain, "ms_e2e": ms_e2e, "stats": [x.as_dict() for x in stats],
        "sched_equal": sched_equal,
        "e2e_stats": estats[-1].as_dict(), "err": err, "e2e_equal": same, "clocks": clocks, "F": F,
        "relax_total": relax_total, "nv_total": int(voff[-1]), "meshes": meshes, "fields": fields,
        "field_relax": field_relax, "gpu_dists": [dist32[voff[k]:voff[k + 1]] for k in range(F)],
        "plain_launches": sum(p.launches for p in pstats[-1]), "plain_steps": plain_steps,
        "grid_kernel": {0: "none", 1: "lockstep", 2: "queue"}.get(int(s0.grid_kernel), "?"),
        "fields_streamed": int(s0.fields_streamed),
        "tuned": tuned, "graph": plan is not None, "launches_per_step": int(s0.launches),
        "strong": strong, "learned_over_reactive": learned_over_reactive,
    }


def strong_scaling(args, ctx, rank, world, timed):
    """Strong scaling: the fixed workload of rank 0's seed split across the
    ranks by the sweep-cost model (gproshan_gb300.shard: strided cost
    predictions, one all-gather of the costs, longest-predicted-first split),
    each rank solving its share in one batched call per step with inputs
    resident; time = max over ranks."""
    import ctypes as C
    import torch
    import torch.distributed as dist
    from gproshan_gb300 import _capi, shard
    meshes, fields = make_workload(shard_seed(args.seed, 0), args.meshes)
    F = len(fields)
    share = list(range(rank, F, world))
    dm = {}

    def mesh(mi):
        if mi not in dm:
            dm[mi] = _capi.DeviceMesh(ctx, meshes[mi][1], meshes[mi][2])
        return dm[mi]

    pc = shard.predicted_costs(ctx, [mesh(fields[k][0]) for k in share], [[fields[k][1]] for k in share])
    got = [None] * world
    dist.all_gather_object(got, (share, [float(x) for x in pc]))
    costs = np.zeros(F)
    for idx, cs in got:
        costs[idx] = cs
    parts = shard.lpt_partition(costs, world)
    mine = parts[rank]
    dm = {mi: dm[mi] for mi in {fields[k][0] for k in mine} if mi in dm}
    n = len(mine)
    src = torch.tensor([fields[k][1] for k in mine] or [0], dtype=torch.int32, device="cuda")
    nvs = [mesh(fields[k][0]).n_vertices for k in mine]
    off = np.concatenate([[0], np.cumsum(nvs)]).astype(np.int64)
    out = torch.empty(max(int(off[-1]), 1), dtype=torch.float32, device="cuda")
    arr = (_capi.gp_field * max(n, 1))()
    for q, k in enumerate(mine):
        arr[q].mesh = mesh(fields[k][0]).handle
        arr[q].sources = src.data_ptr() + 4 * q
        arr[q].dist = out.data_ptr() + 4 * int(off[q])
        arr[q].n_sources = 1
    opts = _capi.make_opts(_capi.GP_F32, schedule=_capi.GP_SCHED_LEARNED)
    sec = C.c_double()

    def step():
        if n:
            ctx.check(_capi.lib().gp_ptp_batch(ctx.handle, arr, n, C.byref(opts), _capi.GP_F32,
                                               _capi.GP_BATCH_DEVICE_POINTERS, C.byref(sec)), "gp_ptp_batch")
        return None

    ms, _ = timed(step, args.steps, args.warmup, "strong")
    return {"value": F / (ms * 1e-3), "unit": "fields/s", "ms_per_step": ms, "fields": F,
            "fields_per_rank": [len(p) for p in parts],
            "predicted_relaxations_per_rank": [float(sum(costs[k] for k in p)) for p in parts],
            "what": "the fixed workload (rank 0's seed) split across the ranks by predicted cost, "
                    "longest-predicted-first; max time over ranks"}


# --------------------------------------------------------------------------
# CPU: the reference's own CPU PTP (or, without its sources, the oracle port)
# --------------------------------------------------------------------------
class CpuPtp:
    """One field on the host cores the way geodesics(mesh, sources, PTP_CPU)
    computes it: toplesets, then parallel_toplesets_propagation_coalescence_cpu
    (reference src/geodesics.cpp:192-207, src/geodesics_ptp.cpp:40-120), FP64,
    OpenMP on every host core.  kind "reference": the reference's own code
    compiled by oracle/Makefile (oracle/_ref); kind "port": the oracle's C
    restatement when the reference's sources are not at hand.  Meshes are
    built once, outside any timed region, on the float-rounded coordinates the
    FP32 GPU path reads."""

    def __init__(self, meshes):
        import oracle
        oracle.build()
        self.threads = os.cpu_count() or 1
        self.meshes = meshes
        self.cache = {}
        try:
            self.L = oracle.RefLib("f64")
            self.kind = "reference"
        except (FileNotFoundError, OSError):
            self.L = None
            self.kind = "port"

    def mesh(self, mi):
        import oracle
        if mi not in self.cache:
            _, xyz, tri = self.meshes[mi]
            x = np.asarray(xyz, dtype=np.float32).astype(np.float64)
            self.cache[mi] = oracle.RefMesh(self.L, x, tri) if self.L else oracle.Mesh(x, tri)
        return self.cache[mi]

    def solve(self, mi, src):
        """One field; src is a vertex or a list of vertices."""
        import oracle
        m = self.mesh(mi)
        srcs = [int(x) for x in src] if hasattr(src, "__len__") else [int(src)]
        if self.L:
            return m.geodesics_ptp_cpu(srcs)
        _, srt, lim = oracle.toplesets(m, srcs)
        return oracle.ptp(m, srcs, lim, srt, nthreads=self.threads)["dist_cpu"]


def reference_order(n_fields: int, seed: int):
    """The order in which the reference arm's steps take the workload's
    fields: a seeded permutation, so every step mixes mesh sizes."""
    return np.random.default_rng(seed + 99).permutation(n_fields)


def cpu_baseline_sample(meshes, fields, field_relax, gpu_dists, max_nv: int = 400_000):
    """The GPU arm's CPU baseline and oracle check, on a bounded sample:
    one field of every mesh with at most max_nv vertices (every family and
    size class of the workload up to the 587^2 height field).

    * baseline: each sampled field is timed on the reference's CPU PTP; the
      mesh's measured rate (relaxations/s, relaxations counted on the GPU,
      which runs the same schedule) times the GPU-counted relaxations of all
      of that mesh's fields gives the mesh's CPU time; the few larger meshes
      take the rate of the largest sampled mesh of their family.
    * oracle check: every field of those meshes (all four per mesh, 244 on
      the benchmark batch) on the oracle port (FP64, float-rounded
      coordinates): the GPU FP32 result against the GPU-returned buffer (max
      rel. error, sweep counts); on the timed fields also the port's
      CPU-returned buffer against the reference's output bit for bit."""
    import oracle
    cpu = CpuPtp(meshes)
    first = {}
    for k, (mi, s) in enumerate(fields):
        first.setdefault(mi, k)
    sampled = [k for mi, k in sorted(first.items()) if len(meshes[mi][1]) <= max_nv]
    rate = {}
    t_sample = 0.0
    r_sample = 0
    err = 0.0
    same_ref = 0
    sweeps_equal = 0
    checked = 0
    timed = set(sampled)
    for k0 in sampled:
        mi = fields[k0][0]
        cpu.mesh(mi)
        om = oracle.Mesh(np.asarray(meshes[mi][1], np.float32).astype(np.float64), meshes[mi][2])
        for k in [k for k, (m, _) in enumerate(fields) if m == mi]:
            s = fields[k][1]
            if k in timed:
                t = time.perf_counter()
                d_cpu = cpu.solve(mi, s)
                dt = time.perf_counter() - t
                t_sample += dt
                r_sample += field_relax[k][0]
                rate[mi] = field_relax[k][0] / dt if dt > 0 else float("inf")
            _, srt, lim = oracle.toplesets(om, [s])
            o = oracle.ptp(om, [s], lim, srt, nthreads=cpu.threads)
            err = max(err, oracle.max_rel_err(gpu_dists[k], o["dist"]))
            sweeps_equal += int(o["n_iter"] == field_relax[k][1])
            checked += 1
            if k in timed:
                same_ref += int(np.array_equal(o["dist_cpu"], d_cpu))
        cpu.cache.pop(mi, None)
    fam_rate = {}
    for mi in rate:  # the largest sampled mesh of each family
        fam = meshes[mi][0][:3]
        if fam not in fam_rate or len(meshes[mi][1]) > len(meshes[fam_rate[fam]][1]):
            fam_rate[fam] = mi
    t_total = 0.0
    scaled = set()
    for k, (mi, _) in enumerate(fields):
        r = rate.get(mi)
        if r is None:
            r = rate[fam_rate[meshes[mi][0][:3]]]
            scaled.add(mi)
        t_total += field_relax[k][0] / r
    v = len(fields) / t_total if t_total else 0.0
    big = ", ".join(f"{meshes[mi][0].split('_')[0]}" for mi in sorted(scaled))
    base = {"value": v, "unit": "fields/s", "cores": cpu.threads, "kind": cpu.kind,
            "sample": f"{len(sampled)} fields, one per mesh of <= {max_nv} vertices ({r_sample} relaxations, "
                      f"{t_sample:.1f} s timed); each mesh's measured rate x the GPU-counted relaxations of its "
                      f"fields; {len(scaled)} larger meshes ({big}) at the rate of the largest sampled mesh of "
                      f"their family",
            "estimate": True}
    check = {"fields": checked, "max_rel_err_vs_oracle": err, "sweeps_equal_oracle": sweeps_equal,
             "oracle_cpu_buffer_equals_reference": same_ref if cpu.kind == "reference" else None,
             "reference_compared_fields": len(sampled),
             "what": f"GPU FP32 result vs the FP64 oracle on the same float-rounded coordinates, every field of the "
                     f"meshes of <= {max_nv} vertices; the oracle's CPU-returned buffer vs the reference's own CPU "
                     f"PTP output (bit for bit) on the {len(sampled)} timed fields"}
    return base, check


def reference_arm(args):
    """`--impl reference`: the reference's CPU PTP on the host cores over the
    whole workload.  The timed steps take the workload's fields in a seeded
    order, step k the fields [k F / K, (k + 1) F / K) of it, so the K timed
    steps together solve every field exactly once; value = fields / total
    time.  Warm-up steps solve one small field each."""
    meshes, fields = make_workload(shard_seed(args.seed, 0), args.meshes)
    cpu = CpuPtp(meshes)
    for mi in range(len(meshes)):
        cpu.mesh(mi)
    F = len(fields)
    order = reference_order(F, args.seed)
    small = min(range(F), key=lambda k: len(meshes[fields[k][0]][1]))
    for _ in range(args.warmup):
        cpu.solve(*fields[small])
    K = max(args.steps, 1)
    times = []
    n = 0
    for step in range(K):
        ks = [int(order[q]) for q in range(step * F // K, (step + 1) * F // K)]
        t = time.perf_counter()
        for k in ks:
            cpu.solve(*fields[k])
        times.append(time.perf_counter() - t)
        n += len(ks)
    T = sum(times)
    v = n / T if T else 0.0
    desc = ("the reference's own parallel_toplesets_propagation_coalescence_cpu + che::compute_toplesets "
            "(oracle/_ref, built from its unmodified sources)" if cpu.kind == "reference" else
            "the oracle's C restatement of the reference CPU PTP (reference sources not present)")
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "fields/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * T / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "fields": F, "vertices_per_step": int(sum(len(meshes[mi][1])
                                                                                        for mi, _ in fields)),
                       "parallelism": f"cpu x{cpu.threads} threads"},
            "cpu_baseline": {"value": v, "unit": "fields/s", "cores": cpu.threads, "kind": cpu.kind,
                             "sample": f"all {F} fields of the workload, about {F // K} per timed step ({n} solved in "
                                       f"{T:.1f} s): {desc}, FP64, OpenMP on every host core"},
            "e2e": {"value": v, "unit": "fields/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def reference_gpu_arm(args):
    """`--impl reference_gpu` (not part of the driver's arms): the reference's
    own GPU PTP -- geodesics(mesh, sources, PTP_GPU), i.e. che::compute_toplesets
    on the host, then parallel_toplesets_propagation_coalescence_gpu
    (src/cuda/geodesics_ptp_coalescence.cu, one source) -- built unmodified for
    sm_103a, over every field of the workload, one call per field as its
    callers make them.  Each call resets the device, so this mode runs no other
    GPU code in its process.  Reports wall-clock fields/s and the GPU time the
    reference's own event timer reports; fields on meshes of at most 50k
    vertices are checked against the FP64 oracle."""
    import oracle
    L = oracle.RefGpuLib(oracle.build_ref_gpu())
    meshes, fields = make_workload(shard_seed(args.seed, 0), args.meshes)
    hs = []
    for _, xyz, tri in meshes:
        x = np.ascontiguousarray(np.asarray(xyz, np.float32).astype(np.float64).reshape(-1))
        t = np.ascontiguousarray(np.asarray(tri, np.uint32).reshape(-1))
        hs.append(L.create(x, len(x) // 3, t, len(t) // 3))
    small = min(range(len(fields)), key=lambda k: len(meshes[fields[k][0]][1]))
    for _ in range(max(args.warmup, 1)):
        mi, s = fields[small]
        L.geod(hs[mi], np.array([s], np.uint32), 1, np.empty(len(meshes[mi][1])))
    wall, rep, err, checked = 0.0, 0.0, 0.0, 0
    for mi, s in fields:
        d = np.empty(len(meshes[mi][1]))
        t0 = time.perf_counter()
        rep += L.geod(hs[mi], np.array([s], np.uint32), 1, d)
        wall += time.perf_counter() - t0
        if len(d) <= 50_000:
            om = oracle.Mesh(np.asarray(meshes[mi][1], np.float32).astype(np.float64), meshes[mi][2])
            err = max(err, oracle.max_rel_err(d, oracle.ptp(om, [s])["dist"]))
            checked += 1
    for h in hs:
        L.free(h)
    F = len(fields)
    return {"impl": "reference_gpu", "metric": METRIC, "value": F / wall, "unit": "fields/s", "n_gpus": 1,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "wall_s": wall, "reference_reported_gpu_s": rep, "reported_fields_per_s": F / rep if rep else None,
            "oracle_check": {"fields": checked, "max_rel_err_vs_oracle": err},
            "config": {"workload": WORKLOAD, "fields": F},
            "what": "the reference's own GPU PTP (geodesics PTP_GPU: host toplesets + "
                    "parallel_toplesets_propagation_coalescence_gpu, FP64, built for sm_103a), one call per field; "
                    "wall clock per call, and the time its own event timer reports (device reset to download)"}


def emit(obj):
    print(json.dumps(obj), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference", "reference_gpu"])
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--skip-check", action="store_true")
    ap.add_argument("--meshes", type=int, default=N_MESHES, help="meshes in the workload (profiling runs)")
    ap.add_argument("--only-batched", action="store_true", help="skip the plain, e2e and CPU legs (profiling runs)")
    ap.add_argument("--schedule", default="learned", choices=["learned", "reactive"],
                    help="batch schedule: the shipped sweep-cost model, or every field starting on one CTA")
    ap.add_argument("--grid-kernel", default="auto", choices=["auto", "lockstep", "queue"])
    ap.add_argument("--queue-tile", type=int, default=0, help="work-queue tile (vertices, multiple of 32)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip the autotuner (default: tune the one-CTA window and grid launch first)")
    ap.add_argument("--no-graph", dest="graph", action="store_false",
                    help="time gp_ptp_batch calls instead of replaying the captured CUDA graph")
    ap.add_argument("--config", default="batch", choices=["batch", "single", "grid2048", "torus", "fps"])
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.config != "batch":
        if rank == 0:
            emit(run_config(args))
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)

    if args.impl == "reference":
        if rank == 0:
            emit(reference_arm(args))
        return
    if args.impl == "reference_gpu":
        if rank == 0:
            emit(reference_gpu_arm(args))
        return

    res = run_gpu(args, rank, world, local)
    if rank != 0:
        return
    F = res["F"] * world
    value = F / (res["ms_batched"] * 1e-3)
    plain = F / (res["ms_plain"] * 1e-3)
    e2e = F / (res["ms_e2e"] * 1e-3)
    st = res["stats"]
    ms_grid = statistics.mean(s["ms_grid"] for s in st)
    ms_local = statistics.mean(s["ms_local"] for s in st)
    relax_grid = st[-1]["relax_grid"]
    relax_local = st[-1]["relax_local"]
    # dominant sweep launch: the one with the larger device time
    if ms_grid >= ms_local:
        kname, kms, krelax = "ptp_kernel (grid-wide sweeps)", ms_grid, relax_grid
    else:
        kname, kms, krelax = "ptp_local_kernel (one CTA per field)", ms_local, relax_local
    peak, pkind = peaks()
    achieved = ALGO_BYTES_PER_RELAX * krelax / (kms * 1e-3) / 1e9 if kms > 0 else 0.0
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        t = json.load(open(tp)).get(kname.split()[0])
        if t and t.get("dram_bytes_per_relax"):
            traffic = t["dram_bytes_per_relax"] * krelax
    # CPU baseline and oracle check on a bounded sample (rank 0, N=1 only)
    cpu, ocheck = None, None
    if world == 1 and not args.only_batched and res["field_relax"] is not None:
        cpu, ocheck = cpu_baseline_sample(res["meshes"], res["fields"], res["field_relax"], res["gpu_dists"])
    launches = res["launches_per_step"] * args.steps
    out = {
        "metric": METRIC, "value": value, "unit": "fields/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["ms_batched"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "fields": F, "vertices_per_step": res["nv_total"] * world,
                   "relaxations_per_step": res["relax_total"] * world,
                   "relaxations_per_s": res["relax_total"] * world / (res["ms_batched"] * 1e-3)
                   if res["ms_batched"] else None,
                   "parallelism": f"fields x{world}",
                   "schedule": args.schedule, "grid_kernel": res["grid_kernel"], "autotuned": res["tuned"],
                   "fields_streamed": res["fields_streamed"],
                   "cuda_graph": res["graph"],
                   "l2": "inputs larger than L2 (129 MB): the step touches every mesh and field buffer"},
        "plain": {"value": plain, "unit": "fields/s", "ms_per_step": res["ms_plain"], "steps": res["plain_steps"],
                  "what": "same fields, one gp_ptp_batch call per field (single-field GPU PTP)"},
        "batched_over_plain": value / plain,
        "max_rel_err": res["err"],
        "max_rel_err_vs": "FP64 reference-formula run of the same fields on the same float-rounded coordinates",
        "fields_same_sweep_count": res["sched_equal"],
        "oracle_check": ocheck,
        "e2e": {"value": e2e, "unit": "fields/s", "h2d_bytes_per_step": res["e2e_stats"]["h2d_bytes"],
                "d2h_bytes_per_step": res["e2e_stats"]["d2h_bytes"], "ms_per_step": res["ms_e2e"],
                "equal_to_device_run": res["e2e_equal"]},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "peak_kind": pkind,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "bytes_per_relaxation": ALGO_BYTES_PER_RELAX, "relaxations_per_launch": krelax,
                     "ms_per_launch": kms}
        | ({"launch_also": f"the grid phase is two launches: the streaming launch, which also builds the "
                           f"toplesets of the {res['fields_streamed']} streamed fields (their BFS and renumbering "
                           f"bytes are not counted above), then the plain launch that resumes after it; "
                           f"ms_per_launch covers both"} if res["fields_streamed"] else {}),
        "phases_ms": {k: statistics.mean(s[k] for s in st) for k in
                      ("ms_toplesets", "ms_renumber", "ms_local", "ms_grid", "ms_gather")},
        "cpu_baseline": cpu,
        "strong_scaling": res["strong"],
        "learned_over_reactive": res["learned_over_reactive"],
        "clocks": res["clocks"],
        "gpu_launches": launches,
    }
    emit(out)


def sweep_roofline(cs, peak, pkind):
    """Roofline of a call's dominant sweep launch from its call statistics:
    48 algorithmic bytes per relaxation over the launch's CUDA-event time."""
    if cs["ms_grid"] >= cs["ms_local"]:
        name, ms, relax = "ptp_kernel (grid-wide sweeps)", cs["ms_grid"], cs["relax_grid"]
    else:
        name, ms, relax = "ptp_local_kernel (one CTA per field)", cs["ms_local"], cs["relax_local"]
    ach = ALGO_BYTES_PER_RELAX * relax / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
    return {"bound": "hbm", "kernel": name, "achieved": ach, "peak": peak, "peak_kind": pkind, "unit": "GB/s",
            "frac": ach / peak, "traffic": None, "bytes_per_relaxation": ALGO_BYTES_PER_RELAX,
            "relaxations_per_launch": relax, "ms_per_launch": ms}


def cpu_fields(xyz, tri, fields, relax_of=None, budget_fields=None):
    """The reference's CPU PTP (geodesics PTP_CPU: toplesets + coalescence CPU
    PTP, FP64, every host core) timed on fields of one mesh.  With relax_of
    (GPU-counted relaxations per field, same schedule) and budget_fields, only
    the first budget_fields fields are timed and the rest are scaled by
    relaxations.  Returns (seconds for all fields, timed fields, kind, cores,
    estimate?)."""
    cpu = CpuPtp([("mesh", xyz, tri)])
    cpu.mesh(0)
    k = len(fields) if budget_fields is None else min(budget_fields, len(fields))
    t = 0.0
    for src in fields[:k]:
        t0 = time.perf_counter()
        cpu.solve(0, src)
        t += time.perf_counter() - t0
    est = k < len(fields)
    if est:
        t *= sum(relax_of) / sum(relax_of[:k])
    return t, k, cpu.kind, cpu.threads, est


def run_config(args):
    """One of the non-headline workloads; returns its JSON record: the GPU
    number, the dominant sweep launch's roofline, the reference's CPU PTP on the
    same workload (timed, or where a full run takes minutes a timed part scaled
    by the GPU-counted relaxations, marked as an estimate), and the GPU result
    checked against the FP64 oracle on the same float-rounded coordinates."""
    import oracle
    from gproshan_gb300 import _capi, build, learned, meshgen

    build.build()
    ctx = _capi.Context(0)
    learned.install(ctx)
    peak, pkind = peaks()

    def best_of(fn, reps):
        best = None
        for _ in range(max(1, args.warmup)):
            fn()
        for _ in range(reps):
            r = fn()
            if best is None or r[2] < best[2]:
                best = r + (ctx.call_stats().as_dict(),)
        return best

    def oracle_check(xyz, tri, srcs, dists, iters):
        om = oracle.Mesh(xyz, tri)
        x32 = np.asarray(xyz, np.float32).astype(np.float64)
        err, same = 0.0, 0
        for src, d, it in zip(srcs, dists, iters):
            ref = oracle.ptp(om, src, xyz=x32, nthreads=os.cpu_count() or 1)
            err = max(err, oracle.max_rel_err(d, ref["dist"]))
            same += int(ref["n_iter"] == it)
        return {"fields": len(srcs), "max_rel_err_vs_oracle": err, "sweeps_equal_oracle": same,
                "what": "GPU FP32 vs the FP64 oracle on the same float-rounded coordinates"}

    rec = {"config": {"workload": args.config}, "data": "synthetic", "n_gpus": 1, "dtype": "f32"}
    if args.config == "single":
        xyz, tri = meshgen.icosphere(6, 0.1, 0)
        m = _capi.DeviceMesh(ctx, xyz, tri)
        d32, st32, s32, cs = best_of(lambda: _capi.ptp_batch(ctx, [m], [[0]]), args.steps)
        d64, st64, s64, _ = best_of(lambda: _capi.ptp_batch(ctx, [m], [[0]], dtype=np.float64, precision=1,
                                                               round_coords=True), max(1, args.steps // 2))
        t_cpu, nk, kind, cores, est = cpu_fields(xyz, tri, [0])
        rec.update({"metric": "ms per field (plain single-field PTP)", "value": s32 * 1e3, "unit": "ms",
                    "higher_is_better": False, "ms_f64": s64 * 1e3, "n_iter": st32[0].n_iter,
                    "relaxations": st32[0].relaxations,
                    "oracle_check": oracle_check(xyz, tri, [[0]], [d32[0]], [st32[0].n_iter]),
                    "roofline": sweep_roofline(cs, peak, pkind),
                    "cpu_baseline": {"value": t_cpu * 1e3, "unit": "ms", "cores": cores, "kind": kind,
                                     "sample": "the same field (toplesets + coalescence CPU PTP, FP64)"},
                    "config": {"workload": "icosphere L6 (40,962 vertices, jitter 0.1 x mean edge, seed 0), "
                                           "source 0"}})
    elif args.config == "grid2048":
        xyz, tri = meshgen.height_field(2048, 0)
        src = np.random.default_rng(0).choice(len(xyz), 4, replace=False).astype(np.uint32)
        m = _capi.DeviceMesh(ctx, xyz, tri)
        d32, st32, s32, cs = best_of(lambda: _capi.ptp_batch(ctx, [m], [src]), args.steps)
        # the reference's CPU PTP on the same family at 512^2 (same seed, 4
        # sources), scaled by the GPU-counted relaxations of both fields: a
        # full 2048^2 run takes minutes
        sx, stri = meshgen.height_field(512, 0)
        ssrc = np.random.default_rng(0).choice(len(sx), 4, replace=False).astype(np.uint32)
        sm = _capi.DeviceMesh(ctx, sx, stri)
        _, sst, _ = _capi.ptp_batch(ctx, [sm], [ssrc])
        cpu = CpuPtp([("mesh", sx, stri)])
        cpu.mesh(0)
        t0 = time.perf_counter()
        cpu.solve(0, ssrc)
        t_small = time.perf_counter() - t0
        t_cpu = t_small * st32[0].relaxations / max(sst[0].relaxations, 1)
        rec.update({"metric": "ms per field", "value": s32 * 1e3, "unit": "ms", "higher_is_better": False,
                    "n_iter": st32[0].n_iter, "relaxations": st32[0].relaxations,
                    "relaxations_per_s": st32[0].relaxations / s32,
                    "oracle_check": oracle_check(xyz, tri, [src], [d32[0]], [st32[0].n_iter]),
                    "roofline": sweep_roofline(cs, peak, pkind),
                    "phases_ms": {k: cs[k] for k in ("ms_toplesets", "ms_renumber", "ms_local", "ms_grid")},
                    "cpu_baseline": {"value": t_cpu * 1e3, "unit": "ms", "cores": cpu.threads, "kind": cpu.kind,
                                     "estimate": True,
                                     "sample": f"the 512^2 field of the same family ({sst[0].relaxations} "
                                               f"relaxations, {t_small:.2f} s), scaled by relaxations"},
                    "config": {"workload": "height field 2048^2 (4,194,304 vertices), 4 seeded sources"}})
    elif args.config == "torus":
        xyz, tri = meshgen.torus(400, 2500, seed=0)
        m = _capi.DeviceMesh(ctx, xyz, tri)
        s16 = np.random.default_rng(4).choice(len(xyz), 16, replace=False).astype(np.uint32)
        d1, st1, s1, _ = best_of(lambda: _capi.ptp_batch(ctx, [m], [s16]), args.steps)
        fs = [[int(x)] for x in s16]
        d16, st16, sl, csl = best_of(lambda: _capi.ptp_batch(ctx, [m] * 16, fs, schedule=_capi.GP_SCHED_LEARNED),
                                     args.steps)
        _, _, sr, csr = best_of(lambda: _capi.ptp_batch(ctx, [m] * 16, fs), args.steps)
        t_plain = 0.0
        for f in fs:
            t_plain += _capi.ptp_batch(ctx, [m], [f])[2]
        relax16 = [int(x.relaxations) for x in st16]
        t_cpu, nk, kind, cores, est = cpu_fields(xyz, tri, [f[0] for f in fs], relax16, budget_fields=1)
        rec.update({"metric": "distance fields/s (16 single-source fields, learned schedule)", "value": 16 / sl,
                    "unit": "fields/s", "higher_is_better": True, "reactive_fields_per_s": 16 / sr,
                    "learned_over_reactive": sr / sl,
                    "plain_fields_per_s": 16 / t_plain, "batched_over_plain": t_plain / sl,
                    "oracle_check": oracle_check(xyz, tri, fs[:3], d16[:3], [x.n_iter for x in st16[:3]]),
                    "roofline": sweep_roofline(csl, peak, pkind),
                    "cpu_baseline": {"value": 16 / t_cpu, "unit": "fields/s", "cores": cores, "kind": kind,
                                     "estimate": est,
                                     "sample": f"{nk} of the 16 fields timed, the rest scaled by their "
                                               f"GPU-counted relaxations"},
                    "one_field_16_sources": {"ms": s1 * 1e3, "n_iter": st1[0].n_iter,
                                             "relaxations": st1[0].relaxations,
                                             "oracle_check": oracle_check(xyz, tri, [s16], [d1[0]],
                                                                          [st1[0].n_iter])},
                    "config": {"workload": "torus R=1 r=0.3, 400x2500 (1M vertices), anisotropic (edge ratio "
                                           "up to ~20:1), 16 seeded sources"}})
    else:
        xyz, tri = meshgen.bump_field(1414, 0)
        m = _capi.DeviceMesh(ctx, xyz, tri)
        _capi.fps(m, 8, seeds=(0,))  # warm-up
        t0 = time.perf_counter()
        smp, md, sec = _capi.fps(m, 512, seeds=(0,))
        wall = time.perf_counter() - t0
        cs = ctx.call_stats().as_dict()
        # the oracle's FPS (FP64) over the first samples: FP32 picks the same
        # farthest vertices while the maxima are separated by more than its
        # rounding
        om = oracle.Mesh(xyz, tri)
        k = 8
        s_ref, _ = oracle.fps(om, k, [0], nthreads=os.cpu_count() or 1)
        agree = 0
        while agree < min(k, len(smp)) and smp[agree] == s_ref[agree]:
            agree += 1
        # CPU: the reference has no CPU farthest-point sampling on PTP; its CPU
        # PTP (toplesets + coalescence CPU PTP) is timed on four of the loop's
        # fields, the sample sets of 64, 128, 256 and 511 samples the GPU chose
        # (early fields, with one or a few sources, take minutes each on the CPU)
        t_cpu, nk, kind, cores, _ = cpu_fields(xyz, tri, [list(smp[:q]) for q in (64, 128, 256, 511)])
        rec.update({"metric": "FPS fields/s (512 sequential geodesic fields)", "value": (len(smp) - 1) / wall,
                    "unit": "fields/s", "higher_is_better": True, "device_s": sec, "wall_s": wall,
                    "samples": len(smp), "max_dist": md,
                    "oracle_check": {"samples_compared": k, "leading_samples_equal": agree,
                                     "what": "GPU FP32 samples vs the FP64 oracle's farthest-point samples"},
                    "roofline": sweep_roofline(cs, peak, pkind) | {"note": "last sample's field"},
                    "cpu_baseline": {"value": nk / t_cpu, "unit": "fields/s", "cores": cores, "kind": kind,
                                     "estimate": True,
                                     "sample": "the reference's CPU PTP on the loop's fields of 64, 128, 256 and "
                                               "511 sources; these are the cheapest fields of the loop (more "
                                               "sources, fewer rings), so this overstates the CPU's rate"},
                    "config": {"workload": "bump field 1414^2 (1,999,396 vertices), 64 Gaussian bumps, 5% "
                                           "displaced vertices; farthest-point sampling from vertex 0"}})
    return rec


if __name__ == "__main__":
    main()
