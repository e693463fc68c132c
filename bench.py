#!/usr/bin/env python3
"""Scan-insertion benchmark: rays/s and voxel-updates/s on the dense street workload.

One step = one insertPointCloud of a 262,144-point 128x2048 LiDAR scan
(pcl::PointXYZ layout) into one resident map at 0.05 m voxels, max range 60 m,
through the C ABI of libvdb_gb300.so. The scans come from the seeded
synthetic street of vdb_mapping_gb300.workloads ("dense").

  value  rays/s with the scans already in HBM (device pointers), CUDA events
         on the map's stream around each insert, L2 flushed between steps.
  e2e    the same through the public API with pinned HOST buffers: the
         host-to-device copy of the scan and the device-to-host read of the
         call's status are inside the timed region (wall clock per call).

`--impl reference` times the reference's CPU path (the C++ oracle restating
it: VDBMapping::raycastPointCloud + updateMap) on all host cores, as
independent map replicas, for the same metric.

With --gpus N > 1 (torchrun, one rank per GPU) each rank inserts the same
scan sequence into its own map: replicas only, no collective on the data path.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "rays/s & voxel-updates/s, batched vs plain GPU, bit-exact; p99 insert latency"
UNIT = "rays/s"
FALLBACK_HBM_GBS = 6800.0
L2_FLUSH_BYTES = 256 << 20
PCL_POINT_BYTES = 16
STATUS_BYTES = 80  # device status block (DevStatus) read back by every call

# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per launch of
# each kernel on a steady-state dense scan, from one ncu capture of the
# default workload's launch list (the last of three inserts; prep = k_prep +
# k_scatter). Only meaningful for the dense workload; other workloads report
# None.
NCU_TRAFFIC_BYTES = {"k_dda_mark": 429.4e6, "k_apply_runs": 804.0e6, "k_sweep": 1986.8e6,
                     "prep (k_prep+k_scan+k_scatter)": 8.4e6}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="dense")
    ap.add_argument("--cpu-scans", type=int, default=2, help="scans in the single-thread CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--points", type=int, default=0,
                    help="use an evenly strided subset of N points of each scan (small profiling cases)")
    ap.add_argument("--serve-seconds", type=float, default=10.0, help="simulated traffic for --workload serving")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0, help="device-memory admission budget")
    ap.add_argument("--serve-drift", default="",
                    help="serving: metres per scan that LiDAR and depth scans move along their heading, 'L,D' "
                         "(maps keep growing); empty: scans cycle in place")
    ap.add_argument("--no-autotune", action="store_true", help="batched mode: keep the library's default tuning")
    ap.add_argument("--tuning", default=None,
                    help='dense mode: kernel tuning as JSON, e.g. \'{"apply_chunk_runs": 1024}\' (speed only)')
    ap.add_argument("--no-graph", action="store_true",
                    help="batched and serving modes: separate launches instead of the captured step")
    ap.add_argument("--batch-maps", type=int, default=32,
                    help="--workload batched: maps per step (the first N maps of the 32-map workload; smaller "
                         "cases for profiling)")
    ap.add_argument("--batch-steps", type=int, default=4,
                    help="distinct steps generated for --workload batched (cycled)")
    ap.add_argument("--leaf-capacity", type=int, default=0,
                    help="leaf pool slots reserved up front (default: sized for the workload)")
    ap.add_argument("--fast-mode", action="store_true",
                    help="dense mode: timed inserts in fast mode (castRayIntoGridFast); the warm-up inserts are normal ones but the last two")
    ap.add_argument("--queries", type=int, default=1 << 20, help="--workload raytrace: queries per step")
    ap.add_argument("--map-scans", type=int, default=6, help="--workload raytrace: dense scans forming the map")
    ap.add_argument("--no-trajectory", action="store_true",
                    help="dense mode: skip timing the whole 100-scan trajectory into one map")
    ap.add_argument("--profile-range", action="store_true",
                    help="bracket the timed steps (batched: the batched arm's) with cudaProfilerStart/Stop, for "
                         "ncu --profile-from-start off")
    ap.add_argument("--peaks", action="store_true",
                    help="print the roofline denominators of this GPU (HBM copy rate and measured L2 atomic rates)")
    ap.add_argument("--no-extras", action="store_true",
                    help="dense mode: skip the short batched and serving runs whose figures join the line")
    ap.add_argument("--extras-serve-seconds", type=float, default=4.0,
                    help="seconds of simulated traffic of the serving figures in the dense line")
    return ap.parse_args()


class ProfileRange:
    """cudaProfilerStart/Stop around a region when enabled (ncu
    --profile-from-start off then captures only that region)."""

    def __init__(self, enabled):
        self.enabled = enabled

    def __enter__(self):
        if self.enabled:
            import torch

            torch.cuda.synchronize()
            torch.cuda.cudart().cudaProfilerStart()
        return self

    def __exit__(self, *exc):
        if self.enabled:
            import torch

            torch.cuda.synchronize()
            torch.cuda.cudart().cudaProfilerStop()


def l2_atomic_rates(device):
    """Measured L2 reduction rates of this GPU (ops/s), or None."""
    import ctypes as C

    from vdb_mapping_gb300 import _lib

    lib = _lib.load()
    out = {}
    for name, pattern in (("coalesced", 0), ("random", 1)):
        r = C.c_double()
        if lib.vdbg_l2_atomic_rate(int(device), pattern, C.byref(r)) != 0 or r.value <= 0:
            return None
        out[name] = r.value
    return out


def measured_peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def max_over_ranks(seconds, dist):
    """The slowest rank's time (the job's time), on any backend (NCCL on GPU
    tensors, gloo on CPU tensors); `dist` None for one rank."""
    if dist is None:
        return seconds
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def host_cpu():
    """The host's CPU model and logical core count."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip().lower() == "model name" and ":" in line:
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if model:
                    break
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "hardware") and ":" in line:
                    model = line.split(":", 1)[1].strip()
    except OSError:
        pass
    if not model:
        import platform

        model = platform.processor() or platform.machine()
    return {"model": model, "logical_cores": os.cpu_count()}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


DESCRIPTIONS = {
    "dense": "128x2048 LiDAR scans of a seeded 200x200x20 m street",
    "small": "64x1024 LiDAR scans of a seeded 40x40x6 m room with 20 boxes",
    "stress": "65,536 random rays of 0.5-200 m from (5000,-3000,40) m",
}
DEFAULT_CAPACITY = {"dense": 1 << 23, "small": 1 << 18, "stress": 1 << 25}


def config_block(wl, args, world):
    return {
        "workload": f"{wl.name}: {wl.points_per_scan} pts/scan, {DESCRIPTIONS.get(wl.name, wl.name)}, "
                    f"voxel {wl.resolution} m, max_range {wl.max_range} m",
        "points_per_scan": wl.points_per_scan,
        "voxel_m": wl.resolution,
        "max_range_m": wl.max_range,
        "scans_timed": args.steps,
        "scans_warmup": args.warmup,
        "point_layout": "pcl::PointXYZ 16 B",
        "l2": "flushed between steps (256 MiB write)",
        "parallelism": f"replicas x{world}" if world > 1 else "single map",
        "leaf_pool_slots": args.leaf_capacity or DEFAULT_CAPACITY.get(wl.name, 1 << 20),
        "tuning": json.loads(args.tuning) if getattr(args, "tuning", None) else "library defaults",
        "fast_mode": bool(getattr(args, "fast_mode", False)),
    }


# --------------------------------------------------------------------------
# Reference arm: the CPU path on all host cores
# --------------------------------------------------------------------------

def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import numpy as np
    import oracle as O

    from vdb_mapping_gb300 import workloads as W

    wl = W.get(args.workload)
    threads = os.cpu_count() or 1
    slice_rays = 32768  # bounded sample per thread and step
    n_src = max(1, min(args.steps + args.warmup, 4))
    scans = [wl.scan(k) for k in range(n_src)]
    times, rays = [], 0
    for step in range(args.warmup + args.steps):
        pts, org = scans[step % n_src]
        off = (step * 7919) % max(1, pts.shape[0] - slice_rays)
        sample = pts[off:off + slice_rays][None, :, :3]
        sec, _ = O.bench_replicas(wl.resolution, wl.config, sample, np.asarray([org]), threads)
        if step >= args.warmup:
            times.append(sec)
            rays += threads * slice_rays
    total = sum(times)
    value = rays / total
    config = config_block(wl, args, world)
    config["parallelism"] = (f"{threads} CPU replicas (one map per host thread), each inserting a "
                             f"{slice_rays}-ray slice of the step's scan into a fresh map per step")
    config["host_cpu"] = host_cpu()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded street scene, no dataset)",
        "config": config,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "host_cpu": host_cpu(),
                         "sample": f"{threads} independent CPU maps (one per thread), each inserting a "
                                   f"{slice_rays}-ray slice of a {wl.name} scan per step; the C++ oracle "
                                   f"restating raycastPointCloud+updateMap, -O2, single-threaded per map like "
                                   f"the reference"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# --------------------------------------------------------------------------
# Our arm
# --------------------------------------------------------------------------

def cpu_baseline_single(wl, scans, n, fast_after=0):
    """The oracle inserting scans 0..n-1 on one thread; with fast_after > 0 the
    first fast_after scans build the map (untimed, normal mode) and the n scans
    after them are timed in fast mode."""
    import dataclasses

    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as O

    m = O.OracleMap(wl.resolution)
    m.setConfig(wl.config)
    m.addInputSource("lidar", wl.max_range, 0)
    for pts, org in scans[:fast_after]:
        m.insertPointCloud(pts, org, "lidar")
    if fast_after:
        m.setConfig(dataclasses.replace(wl.config, fast_mode=True))
    timed = scans[fast_after:fast_after + n]
    t0 = time.perf_counter()
    rays = 0
    for pts, org in timed:
        m.insertPointCloud(pts, org, "lidar")
        rays += pts.shape[0]
    sec = time.perf_counter() - t0
    what = (f"{wl.name} scans {fast_after}-{fast_after + len(timed) - 1} ({rays} rays) in fast mode into a map of "
            f"scans 0-{fast_after - 1}") if fast_after else f"{wl.name} scans 0-{n - 1} ({rays} rays) into a fresh map"
    return {"value": rays / sec, "unit": UNIT, "cores": 1, "kind": "port", "host_cpu": host_cpu(),
            "sample": f"{what}, one thread, C++ oracle restating the reference path (-O2, no FMA contraction)"}


def time_trajectory(wl, scans, new_map, flush, stream, sh):
    """Every scan of the trajectory inserted into one fresh map, each timed
    with CUDA events on the map's stream (device-resident points, L2 flushed
    before each): the latency distribution over the map's whole growth,
    including the pool extensions it needs on the way."""
    import numpy as np
    import torch

    dev = [torch.from_numpy(p).cuda() for p, _ in scans]
    m = new_map()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in scans]
    updates = 0
    torch.cuda.synchronize()
    for k, (_, org) in enumerate(scans):
        flush.zero_()
        ev[k][0].record(stream)
        m.insertPointCloud(dev[k], org, "lidar", stream=sh)
        ev[k][1].record(stream)
        updates += m.last_stats["updates"]
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in ev]
    n_rays = sum(p.shape[0] for p, _ in scans)
    out = {"scans": len(scans), "ms_per_insert": statistics.mean(ms),
           "rays_per_s": n_rays / (sum(ms) / 1000.0), "voxel_updates_per_s": updates / (sum(ms) / 1000.0),
           "latency_ms": {"p50": float(np.percentile(ms, 50)), "p99": float(np.percentile(ms, 99)),
                          "max": max(ms), "argmax": int(np.argmax(ms))},
           "map_leaves": m.leafCount(), "pool": m.poolInfo(), "device_bytes": m.deviceBytes()}
    del m, dev
    torch.cuda.synchronize()
    return out


def run_ours(args):
    import numpy as np
    import torch

    from vdb_mapping_gb300 import OccupancyVDBMapping
    from vdb_mapping_gb300 import workloads as W

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    wl = W.get(args.workload)
    n_scans = args.warmup + args.steps
    want_traj = wl.name == "dense" and not args.no_trajectory and not args.points and not args.fast_mode
    n_gen = max(n_scans, wl.n_scans) if want_traj else n_scans
    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        all_scans = list(ex.map(lambda k: wl.scan(k % wl.n_scans), range(n_gen)))
    scans = all_scans[:n_scans]
    if args.points:
        # an evenly strided subset keeps the scan's geometry (all elevations)
        scans = [(np.ascontiguousarray(p[::max(1, p.shape[0] // args.points)][:args.points]), o) for p, o in scans]
    n_pts = scans[0][0].shape[0]
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    cap = args.leaf_capacity or DEFAULT_CAPACITY.get(wl.name, 1 << 20)

    def new_map():
        m = OccupancyVDBMapping(wl.resolution, initial_leaf_capacity=cap, device=local)
        if args.tuning:
            m.setTuning({**m.tuning(), **json.loads(args.tuning)})
        m.setConfig(wl.config)
        m.addInputSource("lidar", wl.max_range, 0)
        return m

    # ---- device-resident run -------------------------------------------------
    dev_pts = [torch.from_numpy(p).cuda() for p, _ in scans]
    torch.cuda.synchronize()
    m = new_map()
    warmup_passes = []
    # Fast mode: the map is built by normal inserts, and the last two warm-up
    # inserts already run in fast mode (its buffers exist when timing starts).
    fast_from = max(1, args.warmup - 2) if args.fast_mode else args.warmup
    for k in range(args.warmup):
        if k == fast_from:
            m.setConfig(dataclasses.replace(wl.config, fast_mode=True))
        m.insertPointCloud(dev_pts[k], scans[k][1], "lidar", stream=sh)
        warmup_passes.append(m.timings()["passes"])
    if args.fast_mode:
        m.setConfig(dataclasses.replace(wl.config, fast_mode=True))
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats, phases = [], []
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    wall0 = time.perf_counter()
    with ProfileRange(args.profile_range):
        for i in range(args.steps):
            k = args.warmup + i
            flush.zero_()
            ev[i][0].record(stream)
            m.insertPointCloud(dev_pts[k], scans[k][1], "lidar", stream=sh)
            ev[i][1].record(stream)
            stats.append(dict(m.last_stats))
            phases.append(m.timings())
        torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_s = sum(step_ms) / 1000.0
    total_s = max_over_ranks(total_s, dist)
    rays = args.steps * n_pts * world
    updates = sum(s["updates"] for s in stats) * world
    value = rays / total_s
    launches = sum(p["launches"] for p in phases)

    # ---- roofline (live event times) ------------------------------------------
    # Algorithmic work per scan of N points, U updated voxels, Lt touched
    # leaves and V visits:
    #   HBM bytes of the window = 12 N (points) + 8.25 U (FP32 read+write and
    #     the active bit per updated voxel) + 128 Lt (visited and hit masks
    #     read once per touched leaf), over the whole insertion's kernels;
    #   atomics of the marking = V (one visited-bit OR per DDA visit and one
    #     hit-bit OR per unclipped ray, before any merging), over the marking
    #     kernels (k_mark_hits, k_dda_mark, k_apply_runs), against the L2
    #     atomic rate measured on this GPU (vdbg_l2_atomic_rate).
    # Intermediates this design chose (ray records, the DDA run buffer) are
    # not algorithmic: they show up in `traffic` (ncu DRAM bytes).
    hbm_peak, peak_kind = measured_peaks()
    mean = lambda key: statistics.mean(p[key] for p in phases)  # noqa: E731
    dda = mean("dda_ms")
    apply_ms = mean("apply_ms")
    sweep = mean("sweep_ms")
    prep = mean("prep_ms")
    mean_u = statistics.mean(s["updates"] for s in stats)
    mean_lt = statistics.mean(s["touched_leaves"] for s in stats)
    mean_v = statistics.mean(s["visits"] for s in stats)
    mean_runs = mean("runs")
    mean_total_ms = mean("total_ms")
    window_bytes = 12.0 * n_pts + 8.25 * mean_u + 128.0 * mean_lt
    traffic = NCU_TRAFFIC_BYTES if (wl.name == "dense" and not args.points and not args.fast_mode) else {}
    hbm_achieved = window_bytes / (mean_total_ms / 1000.0) / 1e9
    hbm = {"achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_achieved / hbm_peak,
           "peak_kind": peak_kind, "algorithmic_bytes_per_launch": window_bytes, "launch_ms": mean_total_ms,
           "scope": "the whole insertion (prep, marking, sweep)",
           "traffic": sum(traffic.values()) if traffic else None}
    atomic_rate = l2_atomic_rates(local)
    atomic = None
    if atomic_rate and not args.fast_mode:
        a_achieved = mean_v / (dda / 1000.0) / 1e9
        atomic = {"achieved": a_achieved, "peak": atomic_rate["random"] / 1e9, "unit": "G atomics/s",
                  "frac": a_achieved / (atomic_rate["random"] / 1e9), "peak_kind": "measured (vdbg_l2_atomic_rate)",
                  "peak_coalesced": atomic_rate["coalesced"] / 1e9, "algorithmic_atomics_per_launch": mean_v,
                  "launch_ms": dda, "scope": "the marking (k_mark_hits, k_dda_mark, k_apply_runs)",
                  "note": "the marking merges visits into z-plane runs and leaf masks before its ORs reach L2, so "
                          "it issues far fewer atomics than V"}
    top = atomic if atomic and atomic["frac"] > hbm["frac"] else hbm
    per_kernel = {
        "prep (k_prep+k_scan+k_scatter)": {"ms": prep, "algorithmic_bytes": 12.0 * n_pts,
                                           "traffic": traffic.get("prep (k_prep+k_scan+k_scatter)")},
        "marking (k_mark_hits+k_dda_mark+k_apply_runs)": {
            "ms": dda, "algorithmic_atomics": mean_v,
            "traffic": (traffic["k_dda_mark"] + traffic["k_apply_runs"]) if traffic else None},
        "sweep (k_compact+k_sweep)": {"ms": sweep, "algorithmic_bytes": 8.25 * mean_u + 128.0 * mean_lt,
                                      "GBps": (8.25 * mean_u + 128.0 * mean_lt) / (sweep / 1000.0) / 1e9,
                                      "traffic": traffic.get("k_sweep")},
    }

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 DDA / f32 log-odds",
        "data": "synthetic (seeded street scene, no dataset)",
        "config": config_block(wl, args, world),
        "voxel_updates_per_s": updates / total_s,
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                       "max": max(step_ms)},
        "phases_ms": {"prep": prep, "traversal (k_mark_hits+k_dda_mark)": dda - apply_ms, "k_apply_runs": apply_ms,
                      "sweep (k_compact+k_sweep)": sweep, "kernels_total": mean_total_ms},
        "per_scan": {"rays": n_pts, "visits": statistics.mean(s["visits"] for s in stats),
                     "runs": mean_runs, "updates": mean_u, "touched_leaves": mean_lt,
                     "new_leaves": statistics.mean(s["new_leaves"] for s in stats),
                     "dda_passes": [p["passes"] for p in phases], "warmup_dda_passes": warmup_passes},
        "roofline": {"bound": "l2_atomic" if top is atomic else "hbm",
                     "kernel": "marking (k_mark_hits+k_dda_mark+k_apply_runs)" if top is atomic else
                               "the whole insertion",
                     "achieved": top["achieved"], "peak": top["peak"], "unit": top["unit"], "frac": top["frac"],
                     "traffic": hbm["traffic"], "hbm": hbm, "atomic": atomic, "per_kernel": per_kernel},
        "gpu_launches": launches,
        "wall_s_timed_region": wall,
        "map_leaves": m.leafCount(),
        "pool": m.poolInfo(),
    }
    if clk:
        line["clocks"] = clk

    # ---- end to end through the public API with pinned host buffers ----------
    if not args.no_e2e:
        host_pts = [torch.from_numpy(p).pin_memory() for p, _ in scans]
        del m
        torch.cuda.synchronize()
        m2 = new_map()
        for k in range(args.warmup):
            m2.insertPointCloud(host_pts[k].numpy(), scans[k][1], "lidar")
        if args.fast_mode:
            m2.setConfig(dataclasses.replace(wl.config, fast_mode=True))
        e2e_t = []
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        for i in range(args.steps):
            k = args.warmup + i
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            m2.insertPointCloud(host_pts[k].numpy(), scans[k][1], "lidar")
            e2e_t.append(time.perf_counter() - t0)
        e2e_s = sum(e2e_t)
        e2e_s = max_over_ranks(e2e_s, dist)
        line["e2e"] = {"value": rays / e2e_s, "unit": UNIT, "h2d_bytes_per_step": n_pts * PCL_POINT_BYTES,
                       "d2h_bytes_per_step": STATUS_BYTES,
                       "latency_ms": {"p50": 1000 * float(np.percentile(e2e_t, 50)),
                                      "p99": 1000 * float(np.percentile(e2e_t, 99))}}
        del m2

    if want_traj:
        line["trajectory"] = time_trajectory(wl, all_scans[:wl.n_scans], new_map, flush, stream, sh)

    # The rest of the metric (batched vs plain GPU, serving latency), from
    # short runs of those workloads on the same GPU; `value` stays the dense
    # insertion rate.
    if wl.name == "dense" and world == 1 and not args.no_extras and not args.points and not args.fast_mode:
        del flush
        torch.cuda.synchronize()
        bl = measure_batched(local, steps_timed=5, warmup=2, n_distinct=2, autotune=True)
        sv = measure_serving(local, args.extras_serve_seconds, args.serve_budget_gb)
        line["batched_over_plain"] = bl["batched_over_plain"]
        line["batched_voxel_updates_per_s"] = bl["batched"]["voxel_updates_per_s"]
        line["plain_per_map_voxel_updates_per_s"] = bl["plain_per_map"]["voxel_updates_per_s"]
        line["batched_maps_bit_identical"] = bl["maps_bit_identical"]
        line["serving_p50_ms"] = sv["latency_ms_all"]["p50"]
        line["serving_p99_ms"] = sv["latency_ms_all"]["p99"]
        line["extras"] = {
            "batched": {k: bl[k] for k in ("config", "batched", "plain_per_map", "tuning", "gpu_launches_per_step",
                                           "steps", "warmup")},
            "serving": {k: sv[k] for k in ("config", "latency_ms", "latency_ms_all", "rays_per_s",
                                           "voxel_updates_per_s", "mean_scans_per_step", "gpu_busy_frac", "overlapped_steps",
                                           "statuses")},
        }

    if rank == 0 and not args.no_cpu_baseline:
        fa = min(args.warmup, len(scans) - 1) if args.fast_mode else 0
        line["cpu_baseline"] = cpu_baseline_single(wl, scans, min(args.cpu_scans, len(scans) - fa), fast_after=fa)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


# --------------------------------------------------------------------------
# Batched maps: one call per step for all maps vs one call per map
# --------------------------------------------------------------------------

def measure_batched(local, steps_timed, warmup, n_distinct, autotune=True, use_graph=True, profile=False,
                    n_maps=32, leaf_capacity=1 << 22):
    """32 independent maps, one scan each per step: the batched entry point
    (one pass of the kernels for all maps) against the plain per-map path on
    the same scans, both on device-resident points with CUDA events, plus a
    comparison of every map between the two (map digests, vdbg_map_digest:
    every leaf, value bit pattern and active bit). Returns the line."""
    import numpy as np
    import torch

    from vdb_mapping_gb300 import MapBatch, OccupancyVDBMapping
    from vdb_mapping_gb300 import workloads as W

    wl = W.get("batched") if n_maps == 32 else W.BatchedWorkload(n_maps=n_maps)
    n_distinct = max(1, min(warmup + steps_timed, n_distinct))
    steps = [wl.step(k) for k in range(n_distinct)]
    counts = [p.shape[0] for p, _ in steps[0]]
    packed = [torch.from_numpy(np.concatenate([p for p, _ in st])).cuda() for st in steps]
    origins = [[o for _, o in st] for st in steps]
    offs = np.concatenate([[0], np.cumsum(counts)])
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    tuned = None
    if autotune:
        # Autotuned launch parameters on the first sample steps (speed only;
        # both arms use them).
        from vdb_mapping_gb300 import autotune

        tuned, _ = autotune.tune_batch(wl.resolutions, wl.configs, steps[:min(3, n_distinct)], warmup=1)
    b = MapBatch(wl.resolutions, initial_leaf_capacity=leaf_capacity, device=local)
    if tuned:
        b.setTuning(tuned)
    b.useGraph(use_graph)
    for i, c in enumerate(wl.configs):
        b.setConfig(i, c)
    plain = []
    for i, c in enumerate(wl.configs):
        g = OccupancyVDBMapping(wl.resolutions[i], initial_leaf_capacity=1 << 17, device=local)
        if tuned:
            g.setTuning(tuned)
        g.setConfig(c)
        g.addInputSource("s", c.max_range, 0)
        plain.append(g)

    def batched_step(k):
        return b.insert_packed(packed[k % n_distinct], counts, origins[k % n_distinct], stream=sh)

    def plain_step(k):
        x = packed[k % n_distinct]
        upd = 0
        for i, g in enumerate(plain):
            if counts[i]:
                g.insertPointCloud(x[offs[i]:offs[i + 1]], origins[k % n_distinct][i], "s", stream=sh)
                upd += g.last_stats["updates"]
        return {"updates": upd, "rays": int(sum(counts))}

    phase = []
    passes = []

    def timed(fn):
        for k in range(warmup):
            fn(k)
        torch.cuda.synchronize()
        phase.clear()
        passes.clear()
        ms, upd, rays = [], 0, 0
        with ProfileRange(profile and fn is batched_step):
            for i in range(steps_timed):
                k = warmup + i
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                st = fn(k)
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
                upd += st["updates"]
                rays += st["rays"]
                if fn is batched_step:
                    phase.append(b.timings())
                    passes.append(b.timings()["passes"])
        return ms, upd, rays

    clocks = ClockSampler(local)
    clocks.start()
    b_ms, b_upd, b_rays = timed(batched_step)
    b_phase = {k: float(np.mean([p[k] for p in phase])) for k in ("prep_ms", "dda_ms", "sweep_ms", "total_ms")}
    b_passes = list(passes)
    p_ms, p_upd, p_rays = timed(plain_step)
    clk = clocks.stop()
    same = all(b.mapDigest(i) == plain[i].mapDigest() for i in range(len(plain)))
    b_s, p_s = sum(b_ms) / 1000.0, sum(p_ms) / 1000.0
    line = {
        "metric": "voxel-updates/s, 32 independent maps per step: batched call vs one call per map",
        "value": b_upd / b_s, "unit": "voxel-updates/s", "n_gpus": 1, "steps": steps_timed,
        "warmup": warmup, "ms_per_step": 1000.0 * b_s / steps_timed, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 DDA / f32 log-odds",
        "data": f"synthetic (seeded batched workload, {n_distinct} distinct steps cycled)",
        "config": {**wl.describe(), "l2": "flushed between steps (256 MiB write)"},
        "batched": {"voxel_updates_per_s": b_upd / b_s, "rays_per_s": b_rays / b_s, "phases_ms": b_phase,
                    "dda_passes": b_passes,
                    "updates_per_step": b_upd / steps_timed,
                    "ms_per_step": {"p50": float(np.percentile(b_ms, 50)), "p99": float(np.percentile(b_ms, 99))}},
        "plain_per_map": {"voxel_updates_per_s": p_upd / p_s, "rays_per_s": p_rays / p_s,
                          "ms_per_step": {"p50": float(np.percentile(p_ms, 50)),
                                          "p99": float(np.percentile(p_ms, 99))}},
        "batched_over_plain": (b_upd / b_s) / (p_upd / p_s),
        "maps_bit_identical": bool(same),
        "tuning": tuned or "library defaults",
        "gpu_launches_per_step": {"batched": b.timings()["launches"],
                                  "plain": sum(g.timings()["launches"] for g in plain)},
        "cuda_graph": {**b.graphStats(), "enabled": use_graph,
                       "steps": warmup + steps_timed},
    }
    if clk:
        line["clocks"] = clk
    b.close()
    for g in plain:
        g.close()
    torch.cuda.synchronize()
    return line


def run_batched(args):
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    line = measure_batched(local, args.steps, args.warmup, args.batch_steps, autotune=not args.no_autotune,
                           use_graph=not args.no_graph, profile=args.profile_range, n_maps=args.batch_maps,
                           leaf_capacity=args.leaf_capacity or (1 << 22))
    print(json.dumps(line))
    return 0


# --------------------------------------------------------------------------
# Serving: Poisson sensor streams through the continuous-batching loop
# --------------------------------------------------------------------------

def measure_serving(local, seconds, budget_gb, use_graph=True, drift=None):
    """16 sensor streams with Poisson arrivals in real time for `seconds`
    through MapServer; returns p50/p99 latency (submit to done) per sensor
    class next to rays/s and voxel-updates/s. With `drift` (metres per scan,
    LiDAR and depth) every scan is the stream's base scan carried along the
    stream's heading by drift x its scan number, scene and sensor together,
    so the maps keep growing as on a long trajectory; the line reports the
    maps' sizes."""
    import threading
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np
    import torch

    from vdb_mapping_gb300 import MapBatch, MapServer
    from vdb_mapping_gb300 import workloads as W

    wl = W.get("serving")
    K = wl.distinct_scans
    keys = [(i, k) for i in range(len(wl.streams)) for k in range(K)]
    with ThreadPoolExecutor(max_workers=8) as ex:
        scans = dict(zip(keys, ex.map(lambda ik: wl.scan(*ik), keys)))
    batch = MapBatch(wl.resolutions, initial_leaf_capacity=1 << 23, device=local)
    batch.useGraph(use_graph)
    for i, c in enumerate(wl.configs):
        batch.setConfig(i, c)
    # Warm the scratch and run buffers with one scan per map (not timed).
    batch.insert([scans[(i, 0)][0] for i in range(len(wl.streams))],
                 [scans[(i, 0)][1] for i in range(len(wl.streams))])
    budget = int(budget_gb * (1 << 30))
    server = MapServer(batch, memory_budget_bytes=budget)
    arrivals = wl.arrivals(seconds)
    results, busy = [], 0
    counter = [0] * len(wl.streams)
    t_start = time.perf_counter()

    def producer():
        nonlocal busy
        for j, (t, i) in enumerate(arrivals):
            delay = t_start + t - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            k = counter[i]
            counter[i] += 1
            pts, org = scans[(i, k % K)]
            if drift:
                s_ = wl.streams[i]
                d = (drift[1] if s_["depth"] else drift[0]) * k
                off = np.array([d * np.cos(s_["heading"]), d * np.sin(s_["heading"]), 0.0])
                pts = pts.copy()
                pts[:, :3] += off.astype(np.float32)
                org = org + off
            while server.submit(i, pts, org, tag=j) != 0:
                busy += 1
                time.sleep(0.0005)

    clocks = ClockSampler(local)
    clocks.start()
    th = threading.Thread(target=producer)
    th.start()
    while th.is_alive() or len(results) < len(arrivals):
        results += server.poll(512, wait_ms=50)
        if not th.is_alive() and len(results) >= len(arrivals):
            break
    th.join()
    server.drain()
    results += server.poll(4096)
    clk = clocks.stop()
    st = server.stats()
    server.close()
    leaf_bytes = 512 * 4 + 8 * 8 + 16 + 4 + 16 * 8 + 4
    map_gb = [batch.leafCount(i) * leaf_bytes / 1e9 for i in range(len(wl.streams))]
    lat = {"lidar": [], "depth": []}
    for r in results:
        lat["depth" if wl.streams[r["map"]]["depth"] else "lidar"].append((r["done_ns"] - r["submit_ns"]) / 1e6)
    span_s = (max(r["done_ns"] for r in results) - min(r["submit_ns"] for r in results)) / 1e9
    allv = lat["lidar"] + lat["depth"]
    line = {
        "metric": "serving: insert latency p50/p99 (submit to map updated) and rays/s, 16 Poisson sensor streams",
        "value": float(np.percentile(allv, 99)), "unit": "ms (p99 latency)", "n_gpus": 1,
        "steps": st["steps"], "warmup": 1, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 DDA / f32 log-odds",
        "data": f"synthetic (seeded rooms; {K} distinct scans per stream cycled, sensor moving"
                + (", carried along the heading" if drift else "") + ")",
        "config": {**wl.describe(), "seconds": seconds, "memory_budget_gb": budget_gb,
                   "arrivals": "Poisson, real time (not compressed)",
                   "drift_m_per_scan": {"lidar": drift[0], "depth": drift[1]} if drift else None},
        "map_gb": {"lidar": [round(g, 3) for i, g in enumerate(map_gb) if not wl.streams[i]["depth"]],
                   "depth": [round(g, 3) for i, g in enumerate(map_gb) if wl.streams[i]["depth"]],
                   "device_gb": st["device_bytes"] / 1e9},
        "latency_ms_all": {"p50": float(np.percentile(allv, 50)), "p99": float(np.percentile(allv, 99)),
                           "max": float(max(allv)), "n": len(allv)},
        "latency_ms": {c: {"p50": float(np.percentile(v, 50)), "p99": float(np.percentile(v, 99)),
                           "max": float(max(v)), "n": len(v),
                           "sensor_period_ms": 1000.0 / (wl.streams[-1]["hz"] if c == "depth" else wl.streams[0]["hz"])}
                       for c, v in lat.items() if v},
        "rays_per_s": st["rays"] / span_s, "voxel_updates_per_s": st["updates"] / span_s,
        "offered_points_per_s": sum(s["n"] * s["hz"] for s in wl.streams),
        "steps": st["steps"], "mean_scans_per_step": st["requests_done"] / max(1, st["steps"]),
        "max_scans_per_step": st["max_step_maps"], "gpu_busy_frac": st["busy_ns"] / 1e9 / span_s,
        "overlapped_steps": st["overlapped_steps"],
        "overlap": "the next step's upload and ray preparation run on a second stream while a step is marked "
                   "and swept",
        "rejected": st["rejected"], "max_queued": st["max_queued"], "submit_retries_busy": busy,
        "device_bytes": st["device_bytes"],
        "statuses": sorted({r["status"] for r in results}),
        "cuda_graph": {**batch.graphStats(), "enabled": use_graph},
    }
    if clk:
        line["clocks"] = clk
    batch.close()
    torch.cuda.synchronize()
    return line


def run_serving(args):
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    drift = tuple(float(v) for v in args.serve_drift.split(",")) if args.serve_drift else None
    print(json.dumps(measure_serving(local, args.serve_seconds, args.serve_budget_gb, use_graph=not args.no_graph,
                                     drift=drift)))
    return 0


# --------------------------------------------------------------------------
# raytrace queries against the dense street map
# --------------------------------------------------------------------------

def run_raytrace(args):
    """raytrace (VDBMapping.hpp:675-721) against a map of the first dense
    street scans: queries/s of the query kernels (CUDA events of the
    library) and end to end through the public API with host buffers (the
    queries go in and the results come out in every call), the oracle timed on
    a sample of the same queries."""
    import numpy as np
    import torch

    from vdb_mapping_gb300 import OccupancyVDBMapping
    from vdb_mapping_gb300 import workloads as W

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    wl = W.get("dense")
    map_scans = [wl.scan(k) for k in range(args.map_scans)]
    m = OccupancyVDBMapping(wl.resolution, initial_leaf_capacity=DEFAULT_CAPACITY.get("dense", 1 << 20),
                            device=local)
    m.setConfig(wl.config)
    m.addInputSource("lidar", wl.max_range, 0)
    for p, o in map_scans:
        m.insertPointCloud(p, o, "lidar")
    n = args.queries
    rng = np.random.default_rng(12)
    sensors = np.array([o for _, o in map_scans], np.float64)
    org = sensors[rng.integers(0, len(sensors), n)] + rng.normal(0, 0.5, (n, 3))
    d = rng.normal(0, 1, (n, 3))
    d[:, 2] *= 0.3
    ln = np.full(n, wl.max_range)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        m.raytrace(org, d, ln)
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    wall, kern, intersector = [], [], []
    launches = 0
    ok = None
    with ProfileRange(args.profile_range):
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ok, ends = m.raytrace(org, d, ln)
            wall.append(time.perf_counter() - t0)
            t = m.timings()
            kern.append(t["dda_ms"] / 1000.0)
            intersector.append(t["prep_ms"] / 1000.0)
            launches += t["launches"]
    clk = clocks.stop()
    hbm_peak, peak_kind = measured_peaks()
    per_query = 7 * 8 + 3 * 8 + 1  # query in, end point and flag out
    k_s = statistics.mean(kern)
    achieved = n * per_query / k_s / 1e9
    line = {
        "metric": "raytrace queries/s", "value": n / k_s, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * statistics.mean(wall),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded street scene, no dataset)",
        "config": {"workload": f"raytrace: {n} queries per step from the sensor positions (+-0.5 m), random "
                               f"directions (z scaled by 0.3), length {wl.max_range} m, into the map of dense "
                               f"scans 0-{args.map_scans - 1}", "map_leaves": m.leafCount(),
                   "voxel_m": wl.resolution, "l2": "flushed between steps (256 MiB write)"},
        "success_fraction": float(ok.mean()),
        "phases_ms": {"copies in + intersector (k_topo_build)": 1000 * statistics.mean(intersector),
                      "queries (k_trace_spans, span sort, k_trace_walk)": 1000 * k_s},
        "roofline": {"bound": "hbm", "kernel": "k_trace_spans + k_trace_walk", "achieved": achieved,
                     "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                     "traffic": None, "algorithmic_bytes_per_launch": n * per_query, "launch_ms": 1000 * k_s,
                     "note": "one thread per query's coarse walk, then one per span's voxel walk: "
                             "latency-bound lookups of the node sets and leaves"},
        "gpu_launches": launches,
        "e2e": {"value": n / statistics.mean(wall), "unit": "queries/s", "h2d_bytes_per_step": n * 56,
                "d2h_bytes_per_step": n * 25},
    }
    if clk:
        line["clocks"] = clk
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(HERE, "oracle"))
        import oracle as O

        om = O.OracleMap(wl.resolution)
        om.setConfig(wl.config)
        om.addInputSource("lidar", wl.max_range, 0)
        for p, o in map_scans:
            om.insertPointCloud(p, o, "lidar")
        ns = min(n, 1 << 16)
        t0 = time.perf_counter()
        r, ook, oends = om.raytrace(org[:ns], d[:ns], ln[:ns])
        sec = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": ns / sec, "unit": "queries/s", "cores": 1, "kind": "port",
                                "sample": f"the first {ns} queries on one thread, C++ oracle (-O2)"}
        line["parity_sample"] = bool(r == 0 and np.array_equal(ook, ok[:ns]) and
                                     np.array_equal(oends.view(np.uint64), ends[:ns].view(np.uint64)))
    if rank == 0:
        print(json.dumps(line))
    return 0


# --------------------------------------------------------------------------
# Precision stress: long rays far from the world origin at 0.02 m
# --------------------------------------------------------------------------

def run_stress(args):
    """The 20 stress scans (65,536 rays each, log-uniform 0.5-200 m from
    (5000,-3000,40) m, 0.02 m voxels, 1% of the endpoints on voxel faces and
    DDA tie directions), each inserted into the map after a resetMap (one scan
    makes about 16.5M leaves, so the 20 do not fit one GPU together): rays/s
    and voxel-updates/s from CUDA events around each insert, and the voxel
    mismatch count of the traversal against the oracle's FP64 DDA over every
    ray of the config (per-ray path digests)."""
    import numpy as np
    import torch

    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as O

    from vdb_mapping_gb300 import OccupancyVDBMapping
    from vdb_mapping_gb300 import workloads as W

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    wl = W.get("stress")
    scans = [wl.scan(k) for k in range(wl.n_scans)]
    dev = [torch.from_numpy(p).cuda() for p, _ in scans]
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    m = OccupancyVDBMapping(wl.resolution, initial_leaf_capacity=args.leaf_capacity or (1 << 25), device=local)
    m.setConfig(wl.config)
    m.addInputSource("s", wl.max_range, 0)
    order = [k % wl.n_scans for k in range(args.warmup + args.steps)]
    ms, updates, rays, visits, leaves, launches = [], 0, 0, 0, [], 0
    clocks = ClockSampler(local)
    clocks.start()
    for j, k in enumerate(order):
        m.resetMap()
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        m.insertPointCloud(dev[k], scans[k][1], "s", stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        if j >= args.warmup:
            ms.append(e0.elapsed_time(e1))
            st = m.last_stats
            updates += st["updates"]
            rays += st["rays"]
            visits += st["visits"]
            leaves.append(m.leafCount())
            launches += m.timings()["launches"]
    clk = clocks.stop()
    # Traversal parity over the whole config: every ray of every scan.
    mismatched, checked = 0, 0
    t0 = time.perf_counter()
    for k in range(wl.n_scans):
        pts, org = scans[k]
        dg = m.rayDigests(dev[k], org, wl.max_range)
        do = O.ray_digests(pts, org, wl.max_range, wl.resolution)
        mismatched += int(np.any(dg != do, axis=1).sum())
        checked += pts.shape[0]
    parity_s = time.perf_counter() - t0
    total_s = sum(ms) / 1000.0
    line = {
        "metric": "precision stress: rays/s and voxel mismatch count of the FP64 traversal against the oracle",
        "value": rays / total_s, "unit": "rays/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 DDA / f32 log-odds",
        "data": "synthetic (seeded random rays, no dataset)",
        "config": {"workload": "stress: 20 scans x 65,536 rays, log-uniform 0.5-200 m from (5000,-3000,40) m, "
                               "voxel 0.02 m, max_range 250 m, 1% of endpoints on voxel faces and DDA ties",
                   "map": "resetMap before every scan (one scan is ~16.5M leaves)",
                   "l2": "flushed between steps (256 MiB write)"},
        "voxel_updates_per_s": updates / total_s,
        "latency_ms": {"p50": float(np.percentile(ms, 50)), "p99": float(np.percentile(ms, 99)), "max": max(ms)},
        "per_scan": {"rays": rays / len(ms), "visits": visits / len(ms), "updates": updates / len(ms),
                     "leaves": float(np.mean(leaves))},
        "voxel_mismatch_count": mismatched,
        "parity": {"rays_checked": checked, "rays_with_a_different_path": mismatched,
                   "method": "per-ray path digests (visit count, voxel sequence hash, end voxel, clip flag): "
                             "vdbg_ray_digests against the oracle's FP64 DDA, every ray of the 20 scans",
                   "seconds": parity_s},
        "traversal": "FP64 (no FP32 variant is shipped; the mismatch count is of the FP64 path)",
        "gpu_launches": launches,
    }
    if clk:
        line["clocks"] = clk
    if not args.no_cpu_baseline:
        om = O.OracleMap(wl.resolution)
        om.setConfig(wl.config)
        om.addInputSource("s", wl.max_range, 0)
        pts, org = scans[0]
        sample = np.ascontiguousarray(pts[:4096])
        t0 = time.perf_counter()
        om.insertPointCloud(sample, org, "s")
        sec = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": sample.shape[0] / sec, "unit": "rays/s", "cores": 1, "kind": "port",
                                "sample": "the first 4096 rays of stress scan 0 into a fresh map, one thread, "
                                          "C++ oracle (-O2, no FMA contraction)"}
    print(json.dumps(line))
    m.close()
    return 0


def run_peaks(args):
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    hbm, kind = measured_peaks()
    rates = l2_atomic_rates(local)
    line = {"metric": "roofline denominators", "hbm_gbs": hbm, "hbm_kind": kind,
            "l2_atomic_ops_per_s": rates, "device": torch.cuda.get_device_name(local),
            "how": "vdbg_l2_atomic_rate: 64-bit ORs with unused results on a 32 MiB buffer, best of 3 launches "
                   "of (SMs x 8) blocks x 256 threads x 512 ops, CUDA events"}
    print(json.dumps(line))
    return 0


def main():
    args = parse_args()
    if args.peaks:
        return run_peaks(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "raytrace":
        return run_raytrace(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "stress":
        return run_stress(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
