"""Benchmark of the pore-throat + geodesic pipeline on one GB300.

One step = the full pipeline over one synthetic volume: EDT -> containing balls -> seeds and
pore propagation -> empty-pore removal -> watershed, plus float64 geodesics
(EuclideanDistanceComputer .. WatershedComputer and ShortestPathComputer of the reference).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload spinodal1024|spinodal384|grf512|grf320|union128]
  python bench.py --serve [--serve-requests R]   the serving loop (its own JSON line)
  python bench.py --impl reference ...           the CPU restatement (oracle) on bounded samples

Prints one JSON line. `value` is Gvoxel/s with the volume resident in HBM (default: the 1024^3
leveled-wave spinodal); `e2e` is the same metric through pma_pipeline_host with pinned host
buffers (volume in, watershed labels and float64 geodesics out, copies inside the timed
region). `batch` holds the batched form against the plain form on the 256-volume sphere-pack
batch. The working set (GBs of fields) exceeds the 129 MB L2 between steps. With N > 1
(torchrun), each rank runs its own replica on its own GPU: the path has no exchange step, so
scaling is weak and value sums the ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "grf512": dict(kind="grf", shape=(512, 512, 512), sigma=3.0, porosity=0.65, seed=2,
                   desc="512^3 thresholded Gaussian random field, sigma 3, porosity 0.65"),
    "grf320": dict(kind="grf", shape=(320, 320, 320), sigma=3.0, porosity=0.65, seed=2,
                   desc="320^3 thresholded Gaussian random field, sigma 3, porosity 0.65 (profiling size)"),
    "spinodal1024": dict(kind="spinodal", shape=(1024, 1024, 1024), seed=3,
                         desc="1024^3 leveled-wave spinodal, 1000 waves, wavelength 48, porosity 0.70"),
    "spinodal384": dict(kind="spinodal", shape=(384, 384, 384), seed=3,
                        desc="384^3 leveled-wave spinodal, 1000 waves, wavelength 48, porosity 0.70 (profiling size)"),
    "spinodal256": dict(kind="spinodal", shape=(256, 256, 256), seed=3,
                        desc="256^3 leveled-wave spinodal, 1000 waves, wavelength 48, porosity 0.70 (profiling size)"),
    "union128": dict(kind="union", shape=(128, 128, 128), seed=1,
                     desc="128^3 union of 300 spheres, radii U[5,10]"),
}

# DRAM bytes per voxel measured by ncu over all launches of a kernel in one step of a 320^3
# GRF, used as the roofline's `traffic` when that kernel dominates.
TRAFFIC_PER_VOXEL = {
    "ws_generations": (156.2, "ncu dram__bytes_read+write of the 107 ws_generations launches of one "
                              "320^3 GRF step (4683 MB read, 436 MB written), scaled by voxels"),
}

# Algorithmic HBM bytes per voxel of the timed kernels (reads + writes each kernel must do).
ALGO_BYTES = {
    "edt_pass_x": 5.0,          # 1 B mask read + 4 B write
    "edt_pass_y": 8.0,          # 4 B read + 4 B write
    "edt_pass_z": 8.0,          # 4 B read + 4 B write
    "balls_candidates": 16.0,   # 2 x (4 B EDT read) + 8 B key init write
    "balls_tile_gather": 20.0,  # 4 B EDT read + 16 B (radius, centre x, y, z) written
    "uf_hook": 12.0,            # 4 B crad read + 4 B parent read + 4 B parent write
    "geo_bucket": 17.0,         # per settled voxel: 1 B mask + 8 B read + 8 B write (float64)
    "level_sets": 0.0,          # plateau graph work, not per voxel
    "ws_generations": 24.0,     # 4 B crad read + 4 B claim write + 2 x 8 B frontier entry
}


def make_volume(name, device):
    import torch
    from porousmediaanalysis_gb300 import synth
    w = WORKLOADS[name]
    if w["kind"] == "grf":
        return synth.grf(w["shape"], sigma=w["sigma"], porosity=w["porosity"], seed=w["seed"], device=device)
    if w["kind"] == "spinodal":
        return synth.spinodal(w["shape"], seed=w["seed"], device=device)
    return torch.from_numpy(synth.sphere_union(w["shape"], seed=w["seed"])).to(device)


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        cmd = ["nvidia-smi", "-i", str(self.index),
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
               "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
               "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[0]) for r in self.rows if num(r[0])]
        mx = [num(r[1]) for r in self.rows if num(r[1])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def device_step(pma, ctx, solid):
    edt2, mx, _ = pma.compute_euclidean_distances(ctx, solid)
    crad2, cx, cy, cz, mask, nb = pma.set_containing_balls(ctx, edt2, mx)
    labels, table = pma.assign_pore_and_throat_ids(ctx, mask, edt2, crad2)
    pma.remove_empty_pores(ctx, table, labels)
    ws, ws_table = pma.assign_watershed_ids(ctx, table, crad2, mx)
    dist, cav, cavities = pma.compute_shortest_path_distances(ctx, solid, fp64=True)
    return dict(max_edt2=mx, maximum_balls=nb, pores=table.counts()[0],
                ws_throats=ws_table.counts()[1], cavities=len(cavities))


def replica_max(x, world, device):
    """The slowest rank's time: every rank runs its own replica, and the job ends with the last."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(voxels_per_rank, steps, world, seconds):
    """Whole-job Gvoxel/s of `world` replicas that each processed `steps` volumes."""
    return world * voxels_per_rank * steps / seconds / 1e9


def batch_volumes(count=256, seed=4):
    """The 256-volume batch: axis lengths log-uniform in [32, 192], sphere packs with radii
    U[3, 12] added until the solid fraction reaches 0.40."""
    from porousmediaanalysis_gb300 import synth
    shapes = synth.batch_shapes(count, lo=32, hi=192, seed=seed)
    return [synth.sphere_pack(s, rmin=3.0, rmax=12.0, solid_fraction=0.40, seed=seed * 1000 + i)
            for i, s in enumerate(shapes)]


def run_batch(pma, ctx, dev, lanes, reps):
    """Batched form against the plain form (one volume after another) on the same batch:
    Gvoxel/s of each with volumes resident, the batched form end to end from host buffers,
    and a bitwise comparison of every volume's watershed labels and float64 geodesics."""
    import torch
    vols = batch_volumes()
    nvox = sum(v.size for v in vols)
    dvols = [torch.from_numpy(v).to(dev) for v in vols]
    fields = ("watershed_labels", "dist_f64")

    def outputs():  # allocated before timing, so that no run pays for device allocations
        return [{"watershed_labels": torch.empty(v.shape, dtype=torch.int32, device=dev),
                 "dist_f64": torch.empty(v.shape, dtype=torch.float64, device=dev)} for v in dvols]

    def timed(fn, n):
        fn()  # warm-up: scratch sized, lanes created
        torch.cuda.synchronize()
        best = None
        for _ in range(n):
            t0 = time.perf_counter()
            out = fn()
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        return out, best

    out_b, out_p = outputs(), outputs()
    launches0 = ctx.launch_count
    batched, t_batch = timed(lambda: pma.pipeline_batch(ctx, dvols, fp64=True, fields=fields, resident=True,
                                                        lanes=lanes, out_arrays=out_b), reps)
    launches = (ctx.launch_count - launches0) // (reps + 1)
    # plain form: the same call with one lane, one volume after another (warmed up the same way)
    plain, t_plain = timed(lambda: pma.pipeline_batch(ctx, dvols, fp64=True, fields=fields, resident=True,
                                                      lanes=1, out_arrays=out_p), 1)
    same = all(torch.equal(a["watershed_labels"], b["watershed_labels"]) and
               torch.equal(a["dist_f64"].view(torch.int64), b["dist_f64"].view(torch.int64)) and
               a["watershed"].counts() == b["watershed"].counts()
               for a, b in zip(plain, batched))
    t0 = time.perf_counter()
    pma.pipeline_batch(ctx, vols, fp64=True, fields=fields, lanes=lanes)
    t_e2e = time.perf_counter() - t0
    return {"volumes": len(vols), "voxels": nvox, "lanes": lanes, "batched_repeats": reps,
            "value": nvox / t_batch / 1e9, "plain_value": nvox / t_plain / 1e9,
            "speedup_vs_plain": t_plain / t_batch, "e2e_value": nvox / t_e2e / 1e9,
            "unit": "Gvoxel/s", "bitwise_equal_to_plain": bool(same),
            "gpu_launches_per_pass": launches,
            "desc": "256 sphere packs, axes log-uniform [32,192], radii U[3,12], solid 0.40; "
                    "wall clock of the whole batch with volumes resident and outputs preallocated "
                    "(batched: best of repeats; plain: one lane, one volume after another, after a "
                    "warm-up pass); e2e: batched from host buffers, copies included"}


SERVE_SIDES = (64, 128, 256, 384, 512, 768)


def run_serving(args, pma, ctx, requests, sides=SERVE_SIDES, variants=2):
    """Serving: Poisson arrivals of cubic requests (side uniform in `sides`, structure
    alternating between a Gaussian random field with sigma U[2,6], porosity U[0.5,0.8] and a
    sphere pack with radii U[3,12], solid 0.40) at args.serve_load of the plain form's
    throughput, admitted under args.serve_budget_gb of device memory. `variants` distinct
    volumes per (side, structure) are generated up front and drawn at random. Returns the JSON
    object with p50/p99 latency and throughput."""
    import numpy as np
    import torch
    from porousmediaanalysis_gb300 import synth
    rng = np.random.default_rng(5)
    reqs = []
    for i in range(requests):
        side = int(rng.choice(sides))
        reqs.append((side, "grf" if i % 2 == 0 else "pack", int(rng.integers(0, variants))))
    templates = {}
    for key in sorted(set(reqs)):
        side, kind, var = key
        trng = np.random.default_rng(side * 1000 + (500 if kind == "grf" else 0) + var)
        if kind == "grf":
            v = synth.grf((side,) * 3, sigma=float(trng.uniform(2, 6)), porosity=float(trng.uniform(0.5, 0.8)),
                          seed=int(trng.integers(1 << 30)), device="cuda")
        else:
            v = synth.sphere_pack_gpu((side,) * 3, ctx, seed=int(trng.integers(1 << 30)))
        templates[key] = v.cpu().numpy()
        del v
    torch.cuda.empty_cache()
    fields = ("watershed_labels",)
    # plain form: each distinct volume alone, one after another (a warm-up run first)
    alone = {}
    for key, vol in templates.items():
        pma.pipeline_host(ctx, vol, fp64=True, fields=fields)
        t0 = time.perf_counter()
        pma.pipeline_host(ctx, vol, fp64=True, fields=fields)
        alone[key] = time.perf_counter() - t0
    total_vox = sum(r[0] ** 3 for r in reqs)
    plain_seconds = sum(alone[r] for r in reqs)
    plain_tput = total_vox / plain_seconds
    rate = args.serve_load * plain_tput / (total_vox / len(reqs))  # requests per second
    gaps = rng.exponential(1.0 / rate, len(reqs))
    budget = int(args.serve_budget_gb * 10 ** 9)
    ctx.trim()  # the plain runs' scratch goes back before the server's lanes take theirs
    srv = pma.Server(ctx, lanes=args.serve_lanes, memory_budget=budget, fp64=True)
    tickets = [None] * len(reqs)
    t_start = time.perf_counter()

    def feeder():
        t = t_start
        for i, r in enumerate(reqs):
            t += gaps[i]
            dt = t - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            tickets[i] = srv.submit(templates[r], fields=fields)

    th = threading.Thread(target=feeder)
    th.start()
    lat = []
    for i in range(len(reqs)):
        while tickets[i] is None:
            time.sleep(0.0005)
        _, ms = srv.wait(tickets[i])
        lat.append(ms)
    t_end = time.perf_counter()
    th.join()
    st = srv.stats()
    srv.close()
    ctx.trim()
    lat_sorted = sorted(lat)
    pct = lambda q: lat_sorted[min(len(lat_sorted) - 1, int(math.ceil(q * len(lat_sorted))) - 1)]
    return {
        "metric": "serving", "value": total_vox / (t_end - t_start) / 1e9, "unit": "Gvoxel/s",
        "p50_ms": pct(0.50), "p99_ms": pct(0.99), "mean_ms": sum(lat) / len(lat),
        "plain_value": plain_tput / 1e9, "offered_load": args.serve_load, "requests": len(reqs),
        "distinct_volumes": len(templates), "arrival_rate_per_s": rate, "lanes": args.serve_lanes,
        "memory_budget_bytes": budget, "max_in_flight": st["max_in_flight"],
        "peak_reserved_bytes": st["peak_reserved_bytes"], "bytes_per_voxel": st["bytes_per_voxel"],
        "rejected": st["rejected"], "failed": st["failed"], "sides": list(sides),
        "desc": "Poisson arrivals at %.0f%% of the plain form's throughput; outputs: watershed labels to "
                "host, float64 geodesics kept on the device" % (100 * args.serve_load)}


def serve_main(args):
    """The configured serving benchmark as its own JSON line."""
    import torch
    import porousmediaanalysis_gb300 as pma
    from porousmediaanalysis_gb300 import build as pbuild
    pbuild.build()
    torch.cuda.set_device(0)
    ctx = pma.Context(0)
    res = run_serving(args, pma, ctx, args.serve_requests, variants=args.serve_variants)
    line = dict(res)
    line.update({"n_gpus": 1, "higher_is_better": True, "data": "synthetic", "dtype": "u32+f64",
                 "config": {"workload": "serving", "sides": list(SERVE_SIDES)}})
    print(json.dumps(line))
    ctx.close()


CPU_BLOCK = 128  # side of the workload blocks the CPU restatement is timed on


def cpu_blocks(name, count, size=CPU_BLOCK):
    """Bounded CPU samples of the workload: `count` blocks of size^3 voxels cut from the
    workload's own volume (generated on the GPU, so the blocks carry its threshold and
    structure) at offsets spread over the volume. Without a GPU (CPU tests only) the blocks are
    64^3 volumes of the same generator, thresholded on their own. Returns (blocks, description)."""
    import numpy as np
    import torch
    from porousmediaanalysis_gb300 import synth
    w = WORKLOADS[name]
    if not torch.cuda.is_available():
        if w["kind"] == "union":
            v = synth.sphere_union((64, 64, 64), count=38, seed=w["seed"])
        elif w["kind"] == "grf":
            v = synth.grf((64, 64, 64), sigma=w["sigma"], porosity=w["porosity"], seed=w["seed"])
        else:
            v = np.ascontiguousarray(synth.spinodal((64, 64, 64), seed=w["seed"], device="cpu").numpy())
        return [v] * count, "64^3 volume of the same generator (no GPU to build the workload)"
    vol = make_volume(name, "cuda")
    n = [int(s) for s in vol.shape]
    b = [min(size, s) for s in n]
    blocks = []
    for k in range(count):
        o = [((k * m) % max(count, 1)) * (s - e) // max(count - 1, 1) for m, s, e in zip((1, 5, 11), n, b)]
        blk = vol[o[0]:o[0] + b[0], o[1]:o[1] + b[1], o[2]:o[2] + b[2]]
        blocks.append(np.ascontiguousarray(blk.cpu().numpy()))
    del vol
    torch.cuda.empty_cache()
    return blocks, "%dx%dx%d blocks cut from the %s volume at spread offsets" % (b[0], b[1], b[2], name)


def time_oracle(vol):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    t0 = time.perf_counter()
    oracle.full(vol, geodesic_too=False)
    oracle.geodesic(vol, fp64=True)
    return time.perf_counter() - t0


def _oracle_worker(vol):
    return vol.size, time_oracle(vol)


def run_reference(args, workload):
    """CPU restatement of the reference on bounded samples, on all host cores."""
    import multiprocessing as mp
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    blocks, desc = cpu_blocks(workload, cores)  # built before the timed region
    ctxm = mp.get_context("spawn")
    with ctxm.Pool(cores) as pool:
        for _ in range(args.warmup):
            pool.map(_oracle_worker, blocks, chunksize=1)
        t0 = time.perf_counter()
        voxels = 0
        for _ in range(args.steps):
            res = pool.map(_oracle_worker, blocks, chunksize=1)
            voxels += sum(r[0] for r in res)
        wall = time.perf_counter() - t0
    value = voxels / wall / 1e9
    line = {
        "impl": "reference", "metric": "pipeline_throughput", "value": value, "unit": "Gvoxel/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32+f64", "data": "synthetic",
        "config": {"workload": workload, "desc": WORKLOADS[workload]["desc"],
                   "cpu_sample": desc + ", one per core per step"},
        "cpu_baseline": {"value": value, "unit": "Gvoxel/s", "cores": cores, "kind": "port",
                         "sample": desc + ", one per core per step, full pipeline + float64 geodesics "
                                   "(the oracle built -O3 -funroll-loops, as the reference's release build)"},
        "e2e": {"value": value, "unit": "Gvoxel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="spinodal1024", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="pma", choices=["pma", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-lanes", type=int, default=16,
                    help="lanes of the batched-form measurement (0: leave it out)")
    ap.add_argument("--batch-repeats", type=int, default=2)
    ap.add_argument("--serve", action="store_true", help="run the serving benchmark instead")
    ap.add_argument("--serve-requests", type=int, default=2000)
    ap.add_argument("--serve-variants", type=int, default=8, help="distinct volumes per (side, structure)")
    ap.add_argument("--serve-lanes", type=int, default=8)
    ap.add_argument("--serve-budget-gb", type=float, default=120.0)
    ap.add_argument("--serve-load", type=float, default=0.8)
    ap.add_argument("--serve-short", type=int, default=48,
                    help="requests of the short serving run in the default line (0: leave it out)")
    args = ap.parse_args()
    if args.serve:
        return serve_main(args)
    if args.impl == "reference":
        return run_reference(args, args.workload)

    import torch
    import torch.distributed as dist
    import porousmediaanalysis_gb300 as pma
    from porousmediaanalysis_gb300 import build as pbuild
    pbuild.build()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    solid = make_volume(args.workload, dev)
    torch.cuda.synchronize()
    nvox = solid.numel()
    ctx = pma.Context(local)

    for _ in range(args.warmup):
        info = device_step(pma, ctx, solid)
    torch.cuda.synchronize()

    # Device-resident timed region (CUDA events on the context's stream).
    ctx.set_timing(True)
    ctx.timing_report()
    launches0 = ctx.launch_count
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("bench_timed")  # lets ncu --nvtx-include select these launches
        start.record()
        for _ in range(args.steps):
            info = device_step(pma, ctx, solid)
        stop.record()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    if world > 1:
        dist.barrier()
    launches = ctx.launch_count - launches0
    ms = start.elapsed_time(stop)
    kern = ctx.timing_report()
    ctx.set_timing(False)
    ms_max = replica_max(ms, world, dev)
    value = replica_throughput(nvox, args.steps, world, ms_max / 1e3)

    # End-to-end through the C ABI with pinned host buffers.
    import numpy as np
    h_solid = solid.cpu().pin_memory()
    h_ws = torch.empty(solid.shape, dtype=torch.int32).pin_memory()
    h_dist = torch.empty(solid.shape, dtype=torch.float64).pin_memory()
    outs = {"watershed_labels": h_ws.numpy().view(np.uint32), "dist_f64": h_dist.numpy()}
    pma.pipeline_host(ctx, h_solid.numpy(), fp64=True, fields=("watershed_labels", "dist_f64"),
                      out_arrays=outs)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pma.pipeline_host(ctx, h_solid.numpy(), fp64=True, fields=("watershed_labels", "dist_f64"),
                          out_arrays=outs)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = replica_throughput(nvox, args.steps, world, replica_max(e2e_s, world, dev))

    # Roofline of the dominant timed kernel.
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    # the dominant region among the kernels whose algorithmic bytes are stated (whole-stage
    # regions stage_* and host-side regions bracket several kernels; count.* are work counters)
    counters = {k[len("count."):]: v[0] / args.steps for k, v in kern.items() if k.startswith("count.")}
    kern = {k: v for k, v in kern.items() if not k.startswith("count.")}
    kk = {k: v for k, v in kern.items() if k in ALGO_BYTES}
    dom = max(kk.items(), key=lambda kv: kv[1][0]) if kk else ("none", (0.0, 1))
    name, (tot_ms, nlaunch) = dom
    per_launch_ms = tot_ms / max(nlaunch, 1)
    units_per_launch = nvox * args.steps / max(nlaunch, 1)
    algo = ALGO_BYTES.get(name, 0.0) * units_per_launch
    achieved = algo / (per_launch_ms / 1e3) / 1e9 if per_launch_ms > 0 else 0.0
    traffic, traffic_src = None, None
    if name in TRAFFIC_PER_VOXEL:
        traffic = TRAFFIC_PER_VOXEL[name][0] * units_per_launch
        traffic_src = TRAFFIC_PER_VOXEL[name][1]
    roofline = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_src, "traffic": traffic,
                "traffic_unit": "bytes per launch", "traffic_source": traffic_src,
                "algorithmic_bytes_per_launch": algo,
                "kernel_ms_per_step": tot_ms / args.steps,
                "kernels_ms_per_step": {k: v[0] / args.steps for k, v in sorted(kern.items())},
                "counters_per_step": counters}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        oracle.build()
        c = [int(v) // 2 - CPU_BLOCK // 2 for v in solid.shape]
        vol = np.ascontiguousarray(solid[max(c[0], 0):max(c[0], 0) + CPU_BLOCK, max(c[1], 0):max(c[1], 0) + CPU_BLOCK,
                                         max(c[2], 0):max(c[2], 0) + CPU_BLOCK].cpu().numpy())
        secs = time_oracle(vol)
        cpu = {"value": vol.size / secs / 1e9, "unit": "Gvoxel/s", "cores": 1, "kind": "port",
               "sample": "the central %s block of the workload's volume, full pipeline + float64 geodesics "
                         "(the oracle built -O3 -funroll-loops)" % ("x".join(map(str, vol.shape)))}

    batch = None
    if args.batch_lanes > 0:
        batch = run_batch(pma, ctx, dev, args.batch_lanes, args.batch_repeats)

    serving = None
    if args.serve_short > 0 and rank == 0:
        del solid
        torch.cuda.empty_cache()
        ctx.trim()
        # a short run of the serving loop (the configured 2000-request run: bench.py --serve)
        serving = run_serving(args, pma, ctx, args.serve_short, sides=(64, 128, 256, 384), variants=2)

    if rank == 0:
        line = {
            "metric": "pipeline_throughput", "value": value, "unit": "Gvoxel/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32+f64",
            "data": "synthetic",
            "config": {"workload": args.workload, "desc": WORKLOADS[args.workload]["desc"],
                       "voxels": nvox, "l2": "working set of several GB exceeds L2 between steps",
                       "stages": "edt, containing balls, pores, removal, watershed, fp64 geodesics",
                       "result": info},
            "e2e": {"value": e2e_value, "unit": "Gvoxel/s", "h2d_bytes_per_step": nvox,
                    "d2h_bytes_per_step": nvox * 12},
            "gpu_launches": launches,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "batch": batch,
            "serving": serving,
        }
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
