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
* cpu_baseline -- the FP64 CPU restatement on all host cores, on a bounded
             sample of the same fields, scaled by relaxations;
* clocks, gpu_launches -- SM clocks sampled during the timed region, and the
             library's kernel launches inside it.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
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
        # for this workload (untimed; every candidate gives the same results)
        opts = _capi.autotune(ctx, [dmesh[mi] for mi, _ in fields], [[s] for _, s in fields], opts=opts, reps=1)
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

    # accuracy of the batched result vs the FP64 path of the same library on
    # every field, on the same float-rounded coordinates (the FP64 path is
    # bit-exact with the CPU oracle in the tests)
    dist32 = dist_dev.cpu().numpy()
    err = 0.0
    sched_equal = None
    if not args.skip_check:
        fm = [dmesh[mi] for mi, _ in fields]
        fsrc = [[s] for _, s in fields]
        d64s, st64, _ = _capi.ptp_batch(ctx, fm, fsrc, dtype=np.float64, precision=_capi.GP_F64, round_coords=True)
        d32s, st32, _ = _capi.ptp_batch(ctx, fm, fsrc, dtype=np.float32, precision=_capi.GP_F32)
        sched_equal = sum(int(a.n_iter == b.n_iter) for a, b in zip(st32, st64))
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

    # plain single-field GPU PTP over the same fields (fewer steps: it is slow)
    plain_steps = max(1, min(args.steps, 2))
    if args.only_batched:
        ms_plain, pstats = float("nan"), [[]]
    else:
        ms_plain, pstats = timed(plain, plain_steps, 1, "plain")

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

    s0 = stats[-1]
    relax_total = int(s0.relax_local + s0.relax_grid)
    return {
        "ms_batched": ms_batched, "ms_plain": ms_plain, "ms_e2e": ms_e2e, "stats": [x.as_dict() for x in stats],
        "sched_equal": sched_equal,
        "e2e_stats": estats[-1].as_dict(), "err": err, "e2e_equal": same, "clocks": clocks, "F": F,
        "relax_total": relax_total, "nv_total": int(voff[-1]), "meshes": meshes, "fields": fields,
        "plain_launches": sum(p.launches for p in pstats[-1]),
        "grid_kernel": {0: "none", 1: "lockstep", 2: "queue"}.get(int(s0.grid_kernel), "?"),
        "tuned": tuned, "graph": plan is not None, "launches_per_step": int(s0.launches),
    }


# --------------------------------------------------------------------------
# CPU: the oracle port (or the reference build) on a bounded sample
# --------------------------------------------------------------------------
def cpu_sample(meshes, fields, budget_s: float, max_nv: int = 300_000, start: int = 0):
    """Time the CPU PTP (the FP64 oracle port, OpenMP on every host core) on
    fields in workload order, skipping meshes above max_nv so that one field
    stays within the budget, until budget_s elapses.
    Returns (relaxations, seconds, n_fields, kind, threads)."""
    import oracle
    threads = os.cpu_count() or 1
    relax = 0
    t_total = 0.0
    n = 0
    cache = {}
    k = start
    tried = 0
    while t_total < budget_s and tried < len(fields):
        mi, s = fields[k % len(fields)]
        k += 1
        tried += 1
        name, xyz, tri = meshes[mi]
        if len(xyz) > max_nv:
            continue
        if mi not in cache:
            cache[mi] = oracle.Mesh(xyz, tri)
        m = cache[mi]
        _, srt, lim = oracle.toplesets(m, [s])
        t = time.perf_counter()
        out = oracle.ptp(m, [s], lim, srt, nthreads=threads)
        t_total += time.perf_counter() - t
        relax += out["relaxations"]
        n += 1
    return relax, t_total, n, "port", threads


def emit(obj):
    print(json.dumps(obj), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
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
        if rank != 0:
            return
        meshes, fields = make_workload(shard_seed(args.seed, 0), args.meshes)
        # total relaxations of the workload, from the oracle's schedule on the
        # fields the sample covers, scaled by vertex count for the rest
        per_step = []
        kinds = None
        start = 0
        for step in range(args.warmup + args.steps):
            r, t, n, kind, thr = cpu_sample(meshes, fields, args.cpu_budget / 3, start=start)
            start += n
            kinds = (kind, thr, n)
            if step >= args.warmup:
                per_step.append((r, t))
        R = sum(r for r, _ in per_step)
        T = sum(t for _, t in per_step)
        rate = R / T if T else 0.0
        est_total = estimate_total_relax(meshes, fields)
        v = len(fields) * rate / est_total if est_total else 0.0
        emit({"impl": "reference", "metric": METRIC, "value": v, "unit": "fields/s", "n_gpus": args.gpus,
              "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * len(fields) / v if v else None,
              "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
              "data": "synthetic", "config": {"workload": WORKLOAD, "fields": len(fields), "parallelism": "cpu"},
              "cpu_baseline": {"value": v, "unit": "fields/s", "cores": kinds[1], "kind": kinds[0],
                               "sample": f"{R} vertex relaxations over {T:.1f} s on fields of meshes <=300k "
                                         f"vertices, scaled to the workload's estimated {est_total:.3g}"},
              "e2e": {"value": v, "unit": "fields/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
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
    # CPU baseline on a bounded sample (rank 0, N=1 only)
    cpu = None
    if world == 1 and not args.only_batched:
        r, t, n, kind, thr = cpu_sample(res["meshes"], res["fields"], args.cpu_budget)
        rate = r / t if t else 0.0
        cpu_v = res["F"] * rate / res["relax_total"] if res["relax_total"] else 0.0
        cpu = {"value": cpu_v, "unit": "fields/s", "cores": thr, "kind": kind,
               "sample": f"{n} fields of meshes <=300k vertices ({r} relaxations, {t:.1f} s, FP64 oracle port "
                         f"with OpenMP); rate scaled to the workload's {res['relax_total']} relaxations"}
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
                   "cuda_graph": res["graph"],
                   "l2": "inputs larger than L2 (129 MB): the step touches every mesh and field buffer"},
        "plain": {"value": plain, "unit": "fields/s", "ms_per_step": res["ms_plain"],
                  "what": "same fields, one gp_ptp_batch call per field (single-field GPU PTP)"},
        "batched_over_plain": value / plain,
        "max_rel_err": res["err"],
        "max_rel_err_vs": "FP64 reference-formula run of the same fields on the same float-rounded coordinates",
        "fields_same_sweep_count": res["sched_equal"],
        "e2e": {"value": e2e, "unit": "fields/s", "h2d_bytes_per_step": res["e2e_stats"]["h2d_bytes"],
                "d2h_bytes_per_step": res["e2e_stats"]["d2h_bytes"], "ms_per_step": res["ms_e2e"],
                "equal_to_device_run": res["e2e_equal"]},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "peak_kind": pkind,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "bytes_per_relaxation": ALGO_BYTES_PER_RELAX, "relaxations_per_launch": krelax,
                     "ms_per_launch": kms},
        "phases_ms": {k: statistics.mean(s[k] for s in st) for k in
                      ("ms_toplesets", "ms_renumber", "ms_local", "ms_grid", "ms_gather")},
        "cpu_baseline": cpu,
        "clocks": res["clocks"],
        "gpu_launches": launches,
    }
    emit(out)


def run_config(args):
    """One of the non-headline workloads; returns its JSON record."""
    from gproshan_gb300 import _capi, build, learned, meshgen

    build.build()
    ctx = _capi.Context(0)
    learned.install(ctx)

    def relerr(a, ref):
        fin = np.isfinite(ref) & (ref > 0)
        return float(np.max(np.abs(a[fin].astype(np.float64) - ref[fin]) / ref[fin])) if fin.any() else 0.0

    def best_of(fn, reps):
        best = None
        for _ in range(max(1, args.warmup)):
            fn()
        for _ in range(reps):
            r = fn()
            if best is None or r[2] < best[2]:
                best = r + (ctx.call_stats().as_dict(),)
        return best

    rec = {"config": {"workload": args.config}, "data": "synthetic", "n_gpus": 1, "dtype": "f32"}
    if args.config == "single":
        xyz, tri = meshgen.icosphere(6, 0.1, 0)
        m = _capi.DeviceMesh(ctx, xyz, tri)
        d32, st32, s32, _ = best_of(lambda: _capi.ptp_batch(ctx, [m], [[0]]), args.steps)
        d64, st64, s64, _ = best_of(lambda: _capi.ptp_batch(ctx, [m], [[0]], dtype=np.float64, precision=1,
                                                               round_coords=True), max(1, args.steps // 2))
        rec.update({"metric": "ms per field (plain single-field PTP)", "value": s32 * 1e3, "unit": "ms",
                    "higher_is_better": False, "ms_f64": s64 * 1e3, "n_iter": st32[0].n_iter,
                    "relaxations": st32[0].relaxations, "max_rel_err": relerr(d32[0], d64[0]),
                    "config": {"workload": "icosphere L6 (40,962 vertices), source 0"}})
    elif args.config == "grid2048":
        xyz, tri = meshgen.height_field(2048, 0)
        src = np.random.default_rng(0).choice(len(xyz), 4, replace=False).astype(np.uint32)
        m = _capi.DeviceMesh(ctx, xyz, tri)
        d32, st32, s32, cs = best_of(lambda: _capi.ptp_batch(ctx, [m], [src]), args.steps)
        d64, st64, _ = _capi.ptp_batch(ctx, [m], [src], dtype=np.float64, precision=1, round_coords=True)
        rec.update({"metric": "ms per field", "value": s32 * 1e3, "unit": "ms", "higher_is_better": False,
                    "n_iter": st32[0].n_iter, "n_iter_f64": st64[0].n_iter, "relaxations": st32[0].relaxations,
                    "relaxations_per_s": st32[0].relaxations / s32, "max_rel_err": relerr(d32[0], d64[0]),
                    "phases_ms": {k: cs[k] for k in ("ms_toplesets", "ms_renumber", "ms_local", "ms_grid")},
                    "config": {"workload": "height field 2048^2 (4,194,304 vertices), 4 seeded sources"}})
    elif args.config == "torus":
        xyz, tri = meshgen.torus(400, 2500, seed=0)
        m = _capi.DeviceMesh(ctx, xyz, tri)
        s16 = np.random.default_rng(4).choice(len(xyz), 16, replace=False).astype(np.uint32)
        d1, st1, s1, _ = best_of(lambda: _capi.ptp_batch(ctx, [m], [s16]), args.steps)
        d64, st64, _ = _capi.ptp_batch(ctx, [m], [s16], dtype=np.float64, precision=1, round_coords=True)
        fs = [[int(x)] for x in s16]
        _, _, sl, csl = best_of(lambda: _capi.ptp_batch(ctx, [m] * 16, fs, schedule=_capi.GP_SCHED_LEARNED),
                                args.steps)
        _, _, sr, csr = best_of(lambda: _capi.ptp_batch(ctx, [m] * 16, fs), args.steps)
        t_plain = 0.0
        for f in fs:
            t_plain += _capi.ptp_batch(ctx, [m], [f])[2]
        d16, _, _ = _capi.ptp_batch(ctx, [m] * 16, fs, schedule=_capi.GP_SCHED_LEARNED)
        d16r, _, _ = _capi.ptp_batch(ctx, [m] * 16, fs, dtype=np.float64, precision=1, round_coords=True)
        rec.update({"metric": "distance fields/s (16 single-source fields, learned schedule)", "value": 16 / sl,
                    "unit": "fields/s", "higher_is_better": True, "reactive_fields_per_s": 16 / sr,
                    "plain_fields_per_s": 16 / t_plain, "batched_over_plain": t_plain / sl,
                    "max_rel_err_16_fields": max(relerr(a, b) for a, b in zip(d16, d16r)),
                    "one_field_16_sources": {"ms": s1 * 1e3, "n_iter": st1[0].n_iter, "n_iter_f64": st64[0].n_iter,
                                             "relaxations": st1[0].relaxations,
                                             "max_rel_err": relerr(d1[0], d64[0])},
                    "config": {"workload": "torus R=1 r=0.3, 400x2500 (1M vertices), anisotropic (edge ratio "
                                           "up to ~20:1), 16 seeded sources"}})
    else:
        xyz, tri = meshgen.bump_field(1414, 0)
        m = _capi.DeviceMesh(ctx, xyz, tri)
        t0 = time.perf_counter()
        smp, md, sec = _capi.fps(m, 512, seeds=(0,))
        wall = time.perf_counter() - t0
        rec.update({"metric": "FPS fields/s (512 sequential geodesic fields)", "value": (len(smp) - 1) / wall,
                    "unit": "fields/s", "higher_is_better": True, "device_s": sec, "wall_s": wall,
                    "samples": len(smp), "max_dist": md,
                    "config": {"workload": "bump field 1414^2 (1,999,396 vertices), 64 Gaussian bumps, 5% "
                                           "displaced vertices; farthest-point sampling from vertex 0"}})
    return rec


def estimate_total_relax(meshes, fields):
    """Relaxations of the whole workload from a schedule model fitted to the
    oracle on small meshes: about 3 V per icosphere field and 0.27 V^1.5 per
    height-field field (fits the reference schedule within tens of percent)."""
    tot = 0.0
    for mi, _ in fields:
        name, xyz, _ = meshes[mi]
        n = len(xyz)
        tot += 3.0 * n if name.startswith("ico") else 0.27 * n ** 1.5
    return tot


if __name__ == "__main__":
    main()
