#!/usr/bin/env python3
"""Benchmark of the GB300 LOD octree builder on the reference's headline
workload: 119,701,547 points, float64 coordinates in 27-byte records, scale
0.01, grids 512/128, inter-cell colour averaging, output factor 2.2, on a
seeded synthetic 3 km x 3 km terrain with Zipf-clustered density.

A step is one LOD build (ocpi_generate_octree) of that cloud.

  value        Mpts/s of the build with the cloud resident in HBM, timed with
               CUDA events on the builder's stream (sum of its stage events)
  e2e          Mpts/s through the public C ABI with host buffers: upload
               (ocpi_init_octree), build, and the read-back of hierarchy and
               octree records, timed on the host around the synchronous calls
  roofline     the dominant stage's algorithmic bytes / its event time vs the
               measured HBM copy bandwidth
  cpu_baseline the multithreaded CPU oracle on a bounded sample of the cloud

`--impl reference` times the CPU implementation of the same algorithm (the
oracle port: the reference has no CPU implementation of this path) on the
host cores with all threads.  Multi-GPU runs are independent replicas (the
path has no exchange step): every rank builds its own cloud.
"""
import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "octree-cuda_gb300"))

# The plain workloads (seeded synthetic clouds of the reference datasets'
# sizes and types); C is the headline.  Scales are float values widened to
# double, as the CLI passes them (src/argparser.h:12).
BASE_CFG = dict(chunk_grid=512, merge_threshold=10000, output_factor=2.2, sub_grid=128, replacement=True)
WORKLOADS = {
    "C": dict(name="lod_build_120M_f64_terrain_zipf", n=119_701_547, kind=2, cloud_type=1, stride=27, scale=0.01,
              seed=20240601, cpu_sample=12_000_000, modes=dict(inter=True)),
    "A": dict(name="lod_build_5M_f32_heightfield_boxes", n=5_138_448, kind=0, cloud_type=0, stride=15, scale=0.001,
              seed=20240602, cpu_sample=5_138_448, modes=dict(inter=True)),
    "B1": dict(name="lod_build_26M_f32_planes_random_intra", n=25_836_417, kind=1, cloud_type=0, stride=15,
               scale=0.001, seed=20240603, cpu_sample=8_000_000, modes=dict(random=True, intra=True)),
    "B2": dict(name="lod_build_26M_f32_planes_random_inter_weighted", n=25_836_417, kind=1, cloud_type=0, stride=15,
               scale=0.001, seed=20240603, cpu_sample=4_000_000, modes=dict(random=True, inter=True, weighting=True)),
}


def metric_name():
    return "Mpts/s octree build @120M pts" if WORKLOAD == WORKLOADS["C"]["name"] else "Mpts/s octree build @" + WORKLOAD


def select_workload(key):
    """Sets the module's workload constants (N_POINTS, STRIDE, ...)."""
    global N_POINTS, STRIDE, CLOUD_TYPE, SCALE, SEED, CFG, WORKLOAD, CPU_SAMPLE, KIND
    w = WORKLOADS[key]
    N_POINTS, STRIDE, CLOUD_TYPE, KIND = w["n"], w["stride"], w["cloud_type"], w["kind"]
    SCALE, SEED, WORKLOAD, CPU_SAMPLE = float(np.float32(w["scale"])), w["seed"], w["name"], w["cpu_sample"]
    CFG = dict(BASE_CFG, **w["modes"])


select_workload("C")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def replica_max(value, pg):
    """The largest value over the ranks of the process group `pg` (the
    torch.distributed module after init_process_group), or `value` alone."""
    if not pg:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def replicas_throughput(points_per_rank, ranks, ms):
    """Mpts/s of `ranks` independent replicas of a build of points_per_rank
    points timed at `ms` (the slowest rank)."""
    return points_per_rank * ranks / (ms * 1e-3) / 1e6


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def stage_bytes(st, n, stride, timings):
    """Algorithmic HBM bytes per stage (minimal unique traffic of the algorithm)."""
    p_in, p_out = st["p_in"], st["p_out"]
    return {
        "count": n * stride,
        "distribute": n * stride + n * (4 + 18),
        "subsample": p_in * (4 + stride) + p_out * (4 + 18),
    }


def pinned_bytes(nbytes):
    """uint8 numpy view of page-locked host memory."""
    import torch

    return torch.empty(nbytes, dtype=torch.uint8, pin_memory=True).numpy()


def make_cloud(n, threads):
    import octree_api

    t = time.time()
    cloud = octree_api.synthetic_cloud(KIND, CLOUD_TYPE, n, SEED, STRIDE, threads)
    bb = octree_api.cubic_bbox(cloud, n, STRIDE, CLOUD_TYPE, threads)
    return cloud, bb, time.time() - t


def cpu_oracle_time(cloud, bb, n_sample, threads):
    return cpu_oracle_run(cloud, bb, n_sample, threads)[0]


def export_timing(s, points_total):
    """Wall time of one ocpi_export_potree of the session's build (hierarchy.bin,
    octree.bin, metadata.json) into a scratch directory, and the bytes it
    wrote; the files are removed afterwards.  Skipped when the scratch file
    system lacks twice the room."""
    import shutil
    import tempfile

    need = points_total * 18
    free = shutil.disk_usage(tempfile.gettempdir()).free
    if free < 2 * need:
        return {"skipped": "%.1f GB free in %s, %.1f GB to write" % (free / 1e9, tempfile.gettempdir(), need / 1e9)}
    d = tempfile.mkdtemp(prefix="ocpi_export_")
    try:
        t0 = time.perf_counter()
        s.export_potree(d)
        dt = time.perf_counter() - t0
        nbytes = sum(os.path.getsize(os.path.join(d, f)) for f in os.listdir(d))
        return {"ms": round(dt * 1e3, 1), "bytes": nbytes, "gbs": round(nbytes / dt / 1e9, 2)}
    except Exception as e:   # a full or read-only scratch disk: reported, not fatal
        return {"error": str(e)[:200]}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def cpu_oracle_run(cloud, bb, n_sample, threads):
    """Seconds of one oracle build of the first n_sample points, and its result."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    sample = cloud[: n_sample * STRIDE]
    flags = oracle.F_REPLACE
    for key, bit in (("intra", oracle.F_INTRA), ("inter", oracle.F_INTER), ("random", oracle.F_RANDOM),
                     ("weighting", oracle.F_WEIGHT)):
        if CFG.get(key):
            flags |= bit
    t = time.perf_counter()
    r = oracle.run(sample, n=n_sample, stride=STRIDE, cloud_type=CLOUD_TYPE, scale=[SCALE] * 3, bb_min=bb[:3],
                   bb_max=bb[3:], chunk_grid=CFG["chunk_grid"], sub_grid=CFG["sub_grid"],
                   merge_threshold=CFG["merge_threshold"], output_factor=CFG["output_factor"], flags=flags,
                   threads=threads, keep_levels=False)
    dt = time.perf_counter() - t
    if r.stats["error"]:
        raise RuntimeError("oracle failed: %s" % r.stats)
    return dt, r


def link_probe(device, nbytes=1 << 30):
    """Host link bandwidth in GB/s (best of three 1 GiB pinned copies each
    way, CUDA events), measured outside every timed region: it tells a slow
    host link from a slow build in the end-to-end figure."""
    import torch

    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    dev = torch.empty(nbytes, dtype=torch.uint8, device="cuda:%d" % device)
    out = {}
    for name, dst, src in (("h2d_gbs", dev, host), ("d2h_gbs", host, dev)):
        best = None
        for _ in range(4):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[name] = round(nbytes / (best * 1e-3) / 1e9, 1)
    del host, dev
    return out


STAT_KEYS = ["points_total", "p_out", "depth", "tree_nodes", "leaf_nodes", "internal_nodes", "sparse_nodes",
             "dense_nodes", "max_leaf_depth", "min_leaf_points", "max_leaf_points", "mean_leaf_points",
             "stdev_leaf_points", "out_capacity"]


def run_reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    cloud, bb, _ = make_cloud(N_POINTS, threads)
    sample = CPU_SAMPLE
    for _ in range(args.warmup):
        cpu_oracle_time(cloud, bb, sample // 4, threads)
    times = [cpu_oracle_time(cloud, bb, sample, threads) for _ in range(args.steps)]
    t = statistics.median(times)
    v = sample / t / 1e6
    line = {
        "impl": "reference", "metric": metric_name(), "value": round(v, 3), "unit": "Mpts/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if CLOUD_TYPE == 1 else "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "points": N_POINTS, "sample_points": sample, **CFG},
        "cpu_baseline": {"value": round(v, 3), "unit": "Mpts/s", "cores": threads, "kind": "port",
                         "sample": "first %d points of the seeded %.1fM-point cloud, same bbox and settings" %
                                   (sample, N_POINTS / 1e6)},
        "e2e": {"value": round(v, 3), "unit": "Mpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- forms
# Batched (256 independent clouds at once) and served (a Poisson stream of
# build requests) forms through ocpi_batch_build / ocpi_server_*, each beside
# the same builds run one at a time through the plain session calls.

# per generator kind: subsampling options and scale of the plain workloads
# (heightfield: implicit + inter, scale 0.001; planes and cylinders: explicit
# random + inter + weighting, scale 0.001; Zipf terrain: inter, scale 0.01)
KIND_MODES = {0: dict(inter=True), 1: dict(random=True, inter=True, weighting=True), 2: dict(inter=True)}
KIND_SCALE = {0: float(np.float32(0.001)), 1: float(np.float32(0.001)), 2: float(np.float32(0.01))}
FORM_SEED = 20240701
L2_BYTES = 129 << 20


def mode_flags(m):
    import octree_api

    return ((octree_api.SUB_INTRA if m.get("intra") else 0) | (octree_api.SUB_INTER if m.get("inter") else 0) |
            (octree_api.SUB_RANDOM if m.get("random") else 0) | (octree_api.SUB_WEIGHTING if m.get("weighting") else 0))


def host_memory_available():
    try:
        with open("/proc/meminfo") as f:
            for ln in f:
                if ln.startswith("MemAvailable:"):
                    return int(ln.split()[1]) * 1024
    except Exception:
        pass
    return None


def check_host_memory(nbytes):
    """Refuses a workload whose pinned buffers would take more than half of
    the host memory still available."""
    avail = host_memory_available()
    if avail is not None and nbytes > avail // 2:
        raise SystemExit("workload needs %.1f GB of pinned host memory, %.1f GB available: reduce it" %
                         (nbytes / 1e9, avail / 1e9))


class FormCloud:
    """One seeded cloud of a form workload, held in pinned host memory."""

    def __init__(self, i, kind, cloud_type, n, seed, threads):
        import octree_api

        self.i, self.kind, self.cloud_type, self.n, self.seed = i, kind, cloud_type, n, seed
        self.stride = 15 if cloud_type == 0 else 27
        c = octree_api.synthetic_cloud(kind, cloud_type, n, seed, self.stride, threads)
        self.bb = octree_api.cubic_bbox(c, n, self.stride, cloud_type, threads)
        self.host = pinned_bytes(c.nbytes)
        self.host[:] = c
        self.scale = KIND_SCALE[kind]


def plain_build(s, c, grids, mode, rec, hier_out=None):
    """One build through the plain session calls, results into host arrays;
    returns (points_total, node count)."""
    import octree_api

    s.set_cloud(c.host, n=c.n, stride=c.stride, cloud_type=c.cloud_type, scale=[c.scale] * 3, bb_min=c.bb[:3],
                bb_max=c.bb[3:])
    s.configure(chunk_grid=grids[0], merge_threshold=10000, output_factor=2.2, sub_grid=grids[1], seed=c.seed, **mode)
    if rec is not None:
        s.set_output_host(rec)
    s.init()
    s.generate()
    L = octree_api.load_library()
    nodes = ctypes_u64()
    octree_api._check(L.ocpi_get_node_count(s._h, nodes), "ocpi_get_node_count")
    if hier_out is not None:
        octree_api._check(L.ocpi_get_hierarchy(s._h, hier_out.ctypes.data), "ocpi_get_hierarchy")
    if rec is not None:
        octree_api._check(L.ocpi_get_records(s._h, rec.ctypes.data), "ocpi_get_records")
    return s.stats()["points_total"], nodes.value


def ctypes_u64():
    import ctypes

    return ctypes.c_uint64()


def form_job(c, grids, mode, rec, hier, cloud_id=0):
    import octree_api

    return octree_api.make_job(c.host, n=c.n, stride=c.stride, cloud_type=c.cloud_type, scale=[c.scale] * 3,
                               bb_min=c.bb[:3], bb_max=c.bb[3:], chunk_grid=grids[0], merge_threshold=10000,
                               output_factor=2.2, sub_grid=grids[1], flags=mode_flags(mode), seed=c.seed,
                               records=rec, hierarchy=hier, cloud_id=cloud_id)


def form_line(args, metric, value, unit, extra):
    line = {"metric": metric, "value": round(value, 3), "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32/f64", "data": "synthetic"}
    line.update(extra)
    return line


def run_batched(args):
    """256 clouds, sizes log-uniform 50k-4M (seeded), 80% float32, grids
    128/64 or 512/128 at random, generators in turn; per-cloud seeds."""
    import octree_api

    threads = os.cpu_count() or 1
    rng = np.random.default_rng(FORM_SEED)
    count = args.clouds
    sizes = np.exp(rng.uniform(np.log(50_000), np.log(4_000_000), count)).astype(np.int64)
    types = (rng.random(count) >= 0.8).astype(int)
    grid_pick = rng.random(count) < 0.5
    t0 = time.time()
    clouds = [FormCloud(i, i % 3, int(types[i]), int(sizes[i]), FORM_SEED + i, threads) for i in range(count)]
    gen_s = time.time() - t0
    grids = [(128, 64) if g else (512, 128) for g in grid_pick]
    modes = [KIND_MODES[c.kind] for c in clouds]
    total_pts = int(sizes.sum())

    # output sizes from one plain pass (warm-up), then exact pinned outputs;
    # --no-plain: results stay on the device (no plain builds at all)
    s = octree_api.OctreeSession(0)
    in_bytes = sum(c.n * c.stride for c in clouds)
    if args.no_plain:
        recs = [None] * count
        hiers = [None] * count
        out_bytes = 0
    else:
        shapes = []
        for c, g, m in zip(clouds, grids, modes):
            shapes.append(plain_build(s, c, g, m, None))
        need = sum(max(p, 1) * 18 for p, _ in shapes)
        check_host_memory(need + sum(c.host.nbytes for c in clouds))
        recs = [pinned_bytes(max(p, 1) * 18) for p, _ in shapes]
        hiers = [np.zeros(nn * 22, np.uint8) for _, nn in shapes]
        out_bytes = sum(p * 18 + nn * 22 for p, nn in shapes)

    def plain_pass():
        t = time.perf_counter()
        for c, g, m, r, h in zip(clouds, grids, modes, recs, hiers):
            plain_build(s, c, g, m, r, h)
        return time.perf_counter() - t

    jobs = [form_job(c, g, m, r, h) for c, g, m, r, h in zip(clouds, grids, modes, recs, hiers)]
    tuning = None
    tune_s = None
    if args.waves == "auto":
        # the autotuner's trials run on a sample of this batch, outside the
        # timed region
        t0 = time.perf_counter()
        tuning = octree_api.batch_autotune(jobs, memory_budget=args.budget_gb << 30)
        tune_s = time.perf_counter() - t0

    def batch_pass():
        t = time.perf_counter()
        if tuning is not None:
            res = octree_api.batch_build_tuned(jobs, tuning, memory_budget=args.budget_gb << 30)
        elif args.waves != "lanes":
            res = octree_api.batch_build_wave(jobs, wave_size=int(args.waves), memory_budget=args.budget_gb << 30)
        else:
            res = octree_api.batch_build(jobs, lanes=args.lanes, memory_budget=args.budget_gb << 30)
        dt = time.perf_counter() - t
        bad = [r.error.decode() for r in res if r.status != 0]
        if bad:
            raise RuntimeError("batched build failed: %s" % bad[0])
        if not args.no_plain:
            # every build of the batch has the shape of the same build run alone
            for i, (r, (p, nn)) in enumerate(zip(res, shapes)):
                if (r.pointsTotal, r.nodeCount) != (p, nn):
                    raise RuntimeError("cloud %d: batched build differs from the plain build" % i)
        return dt, res

    if not args.no_plain:
        for _ in range(max(1, args.warmup - 1)):
            plain_pass()
    plain_s = [plain_pass() for _ in range(args.steps)] if not args.no_plain else [float("nan")]
    for _ in range(args.warmup):
        batch_pass()
    clocks = ClockSampler(0)
    clocks.start()
    batch = [batch_pass() for _ in range(args.steps)]
    clk = clocks.stop()
    s.close()
    b_s = statistics.median(d for d, _ in batch)
    p_s = statistics.median(plain_s)
    res = batch[-1][1]
    line = form_line(args, "Mpts/s batched build, %d clouds" % count, total_pts / b_s / 1e6, "Mpts/s", {
        "form": "batched", "ms_per_step": round(b_s * 1e3, 2),
        "config": {"workload": "batched_%d_clouds_50k_4M" % count, "clouds": count, "points": total_pts,
                   "float32_clouds": int((types == 0).sum()), "grids_128_64": int(grid_pick.sum()),
                   "lanes": args.lanes if args.waves == "lanes" else None, "waves": args.waves,
                   "tuning": tuning.as_dict() if tuning is not None else None,
                   "autotune_s": round(tune_s, 2) if tune_s is not None else None,
                   "memory_budget_gb": args.budget_gb,
                   "generator_seed": FORM_SEED,
                   "l2": "inputs larger than L2 (%.1f GB of clouds per step)" % (in_bytes / 1e9)},
        "e2e": {"value": round(total_pts / b_s / 1e6, 3), "unit": "Mpts/s", "h2d_bytes_per_step": in_bytes,
                "d2h_bytes_per_step": out_bytes, "ms": round(b_s * 1e3, 2)},
        "plain_sequential": None if args.no_plain else
        {"value": round(total_pts / p_s / 1e6, 3), "unit": "Mpts/s", "ms": round(p_s * 1e3, 2)},
        "speedup_vs_plain": None if args.no_plain else round(p_s / b_s, 3),
        "per_build_ms": {"p50": round(float(np.percentile([r.runMs for r in res], 50)), 3),
                         "p99": round(float(np.percentile([r.runMs for r in res], 99)), 3)},
        "gen_s": round(gen_s, 1), "clocks": clk})
    print(json.dumps(line))
    return 0


def run_served(args):
    """A Poisson stream of build requests (sizes log-uniform 100k-30M over a
    pool of distinct seeded clouds, mixed float32/float64, mixed grids and
    subsampling options) against a server with a 150 GB device budget."""
    import concurrent.futures
    import octree_api
    import queue

    threads = os.cpu_count() or 1
    rng = np.random.default_rng(FORM_SEED + 1)
    pool_n = args.pool
    sizes = np.exp(rng.uniform(np.log(100_000), np.log(30_000_000), pool_n)).astype(np.int64)
    types = (rng.random(pool_n) >= 0.8).astype(int)
    t0 = time.time()
    pool = [FormCloud(i, i % 3, int(types[i]), int(sizes[i]), FORM_SEED + 1000 + i, threads) for i in range(pool_n)]
    gen_s = time.time() - t0
    options = [((512, 128), None), ((128, 64), None), ((512, 128), dict(random=True, intra=True)),
               ((256, 64), dict(inter=True))]
    nreq = args.requests
    req_cloud = rng.integers(0, pool_n, nreq)
    req_opt = rng.integers(0, len(options), nreq)

    def req_mode(k):
        o = options[req_opt[k]][1]
        return o if o is not None else KIND_MODES[pool[req_cloud[k]].kind]

    # shapes of every (cloud, option) pair from plain builds (warm-up)
    s = octree_api.OctreeSession(0)
    shape = {}
    for k in range(nreq):
        key = (int(req_cloud[k]), int(req_opt[k]))
        if key not in shape:
            shape[key] = plain_build(s, pool[key[0]], options[key[1]][0], req_mode(k), None)
    max_rec = max(p for p, _ in shape.values())
    max_nodes = max(nn for _, nn in shape.values())
    slots = args.lanes * 2
    check_host_memory(slots * max_rec * 18 + sum(c.host.nbytes for c in pool))
    slot_rec = [pinned_bytes(max_rec * 18) for _ in range(slots)]
    slot_hier = [np.zeros(max_nodes * 22, np.uint8) for _ in range(slots)]
    req_pts = np.array([pool[c].n for c in req_cloud], np.int64)
    total_pts = int(req_pts.sum())

    # plain: every request one at a time (service times, no queueing)
    plain_ms = []
    t = time.perf_counter()
    for k in range(nreq):
        c = pool[req_cloud[k]]
        t1 = time.perf_counter()
        plain_build(s, c, options[req_opt[k]][0], req_mode(k), slot_rec[0], slot_hier[0])
        plain_ms.append((time.perf_counter() - t1) * 1e3)
    plain_s = time.perf_counter() - t
    s.close()

    srv = octree_api.Server(lanes=args.lanes, memory_budget=args.budget_gb << 30)

    def stream(arrivals):
        """Submits request k at arrivals[k] (seconds from the start) on a free
        result slot; returns per-request latency (arrival to completion) and
        the makespan."""
        free = queue.Queue()
        for i in range(slots):
            free.put(i)
        lat = np.zeros(nreq)
        done_at = np.zeros(nreq)
        reused = np.zeros(nreq, np.int64)

        def waiter(k, ticket, slot, t_arr):
            r = srv.wait(ticket)
            done_at[k] = time.perf_counter()
            reused[k] = r.reused
            srv.release(ticket)
            free.put(slot)
            if r.status != 0:
                raise RuntimeError("request %d failed: %s" % (k, r.error.decode()))
            if (r.pointsTotal, r.nodeCount) != shape[(int(req_cloud[k]), int(req_opt[k]))]:
                raise RuntimeError("request %d: served build differs from the plain build" % k)
            lat[k] = done_at[k] - t_arr

        with concurrent.futures.ThreadPoolExecutor(max_workers=slots) as ex:
            futs = []
            start = time.perf_counter()
            for k in range(nreq):
                t_arr = start + arrivals[k]
                now = time.perf_counter()
                if t_arr > now:
                    time.sleep(t_arr - now)
                slot = free.get()
                c = pool[req_cloud[k]]
                job = form_job(c, options[req_opt[k]][0], req_mode(k), slot_rec[slot], slot_hier[slot],
                               cloud_id=0 if args.no_resident else int(req_cloud[k]) + 1)
                futs.append(ex.submit(waiter, k, srv.submit(job), slot, t_arr))
            for f in futs:
                f.result()
        return lat, float(done_at.max() - start), int(reused.sum())

    # saturation: every request arrives at once
    stream(np.zeros(nreq))   # warm-up: lanes grow their buffers
    sat_lat, sat_s, sat_reused = stream(np.zeros(nreq))
    capacity = total_pts / sat_s
    # Poisson arrivals at a fraction of the saturation throughput
    rate = args.load * capacity / (total_pts / nreq)   # requests per second
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    clocks = ClockSampler(0)
    clocks.start()
    lat, span, reused = stream(arrivals)
    clk = clocks.stop()
    srv.close()
    def pct(a_ms, q):
        return round(float(np.percentile(a_ms, q)), 3)

    lat, sat_lat = lat * 1e3, sat_lat * 1e3
    line = form_line(args, "Mpts/s served builds, %d Poisson requests" % nreq, total_pts / span / 1e6, "Mpts/s", {
        "form": "served", "ms_per_step": round(span * 1e3, 2),
        "config": {"workload": "served_%d_requests_100k_30M" % nreq, "requests": nreq, "points": total_pts,
                   "distinct_clouds": pool_n, "lanes": args.lanes, "result_slots": slots,
                   "memory_budget_gb": args.budget_gb, "offered_load": args.load,
                   "cloud_ids": not args.no_resident,
                   "arrival_rate_per_s": round(rate, 2), "generator_seed": FORM_SEED + 1},
        "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99)},
        "resident_reuse": {"poisson": reused, "saturation": sat_reused, "requests": nreq},
        "saturation": {"value": round(capacity / 1e6, 3), "unit": "Mpts/s", "ms": round(sat_s * 1e3, 2),
                       "latency_p50_ms": pct(sat_lat, 50), "latency_p99_ms": pct(sat_lat, 99)},
        "plain_sequential": {"value": round(total_pts / plain_s / 1e6, 3), "unit": "Mpts/s",
                             "ms": round(plain_s * 1e3, 2), "service_p50_ms": pct(plain_ms, 50),
                             "service_p99_ms": pct(plain_ms, 99)},
        "speedup_vs_plain": round(plain_s / sat_s, 3),
        "e2e": {"value": round(total_pts / span / 1e6, 3), "unit": "Mpts/s",
                "h2d_bytes_per_step": int(sum(pool[c].n * pool[c].stride for c in req_cloud)),
                "d2h_bytes_per_step": None},
        "gen_s": round(gen_s, 1), "clocks": clk})
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="C", choices=sorted(WORKLOADS),
                    help="C: the headline 119.7M-point float64 build; A, B1, B2: the other plain workloads")
    ap.add_argument("--points", type=int, default=None, help="point amount (default: the workload's)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--form", default="plain", choices=["plain", "batched", "served"],
                    help="plain: the 120M-point build; batched / served: many independent builds at once")
    ap.add_argument("--lanes", type=int, default=None,
                    help="concurrent builds of the batched and served forms (default 4)")
    ap.add_argument("--budget-gb", type=int, default=150, help="device memory budget of the batched / served forms")
    ap.add_argument("--waves", default="auto",
                    help="batched form: 'auto' (subsampling waves with the autotuned size, cluster caps and graph "
                         "capture: ocpi_batch_autotune + ocpi_batch_build_tuned), a wave size "
                         "(ocpi_batch_build_wave), or 'lanes' (the lane executor, ocpi_batch_build)")
    ap.add_argument("--clouds", type=int, default=256, help="clouds of the batched form")
    ap.add_argument("--requests", type=int, default=2000, help="requests of the served form")
    ap.add_argument("--pool", type=int, default=24, help="distinct clouds the served requests draw from")
    ap.add_argument("--load", type=float, default=0.8, help="served offered load, fraction of saturation")
    ap.add_argument("--no-resident", action="store_true",
                    help="served form: requests carry no cloud id, so no lane reuses a resident cloud")
    ap.add_argument("--no-plain", action="store_true",
                    help="batched form only: no plain comparison and no host outputs (for profiling)")
    args = ap.parse_args()
    select_workload(args.workload)
    if args.points is None:
        args.points = N_POINTS
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.form == "batched":
        args.lanes = args.lanes or 4
        return run_batched(args)
    if args.form == "served":
        args.lanes = args.lanes or 4
        return run_served(args)

    import octree_api

    ws, rank, local = dist_env()
    pg = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        pg = dist
    device = local
    threads = os.cpu_count() or 1
    n = args.points
    cloud, bb, gen_s = make_cloud(n, threads)

    def barrier():
        if pg:
            pg.barrier()

    # the cloud lives in pinned host memory (the upload in ocpi_init_octree is
    # a DMA from it) and results are read back into pinned memory
    cloud_host = pinned_bytes(cloud.nbytes)
    cloud_host[:] = cloud
    del cloud
    s = octree_api.OctreeSession(device)
    s.set_cloud(cloud_host, n=n, stride=STRIDE, cloud_type=CLOUD_TYPE, scale=[SCALE] * 3, bb_min=bb[:3],
                bb_max=bb[3:])
    s.configure(**CFG)
    s.init()
    for _ in range(args.warmup):
        s.generate()

    # ---- device-resident build: CUDA events of the builder stream.  A cloud
    # smaller than twice the L2 is evicted before every timed build by
    # writing a 512 MB buffer (outside the timed events).
    cloud_bytes = n * STRIDE
    flush = None
    if cloud_bytes < 2 * L2_BYTES:
        import torch

        flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda:%d" % device)
        l2_note = "L2 flushed before every timed build (512 MB write; %.0f MB cloud)" % (cloud_bytes / 1e6)
    else:
        l2_note = "inputs larger than L2 (%.1f GB cloud)" % (cloud_bytes / 1e9)
    import torch

    torch.cuda.set_device(device)
    clocks = ClockSampler(device)
    clocks.start()
    barrier()
    torch.cuda.synchronize(device)
    stage_sum = {}
    gen_ms = []
    step_ms = []
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        if flush is not None:
            flush.zero_()
            torch.cuda.synchronize(device)
        # ocpi_generate_octree returns when the build's streams are done, so
        # events on either side of it bracket the whole build, host gaps
        # included
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        s.generate()
        e1.record()
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        t = s.timings()
        gen_ms.append(sum(t.values()))
        for k, v in t.items():
            stage_sum[k] = stage_sum.get(k, 0.0) + v
    torch.cuda.synchronize(device)
    barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    st = s.stats()
    ms_step = statistics.mean(step_ms)
    ms_step = replica_max(ms_step, pg)
    value = replicas_throughput(n, ws, ms_step)
    stage_avg = {k: v / args.steps for k, v in stage_sum.items()}

    # ---- end to end through the C ABI with host buffers
    e2e_times = []
    hier_bytes = st["tree_nodes"] * 22
    rec_bytes = st["points_total"] * 18
    # results land in pinned host arrays registered with the session: the
    # leaf records stream back while the upper levels are subsampled
    recs = pinned_bytes(max(int(np.float32(n) * np.float32(CFG["output_factor"])), st["points_total"]) * 18)
    s.set_output_host(recs)
    L = octree_api.load_library()
    init_times = []
    for i in range(args.steps + 1):   # the first is a warm-up of the result arrays
        barrier()
        t0 = time.perf_counter()
        s.init()
        t1 = time.perf_counter()
        s.generate()
        h = s.hierarchy()
        octree_api._check(L.ocpi_get_records(s._h, recs.ctypes.data), "ocpi_get_records")
        if i:
            init_times.append(t1 - t0)
            e2e_times.append(time.perf_counter() - t0)
    # the median: the host link is shared with the machine's other GPUs, and
    # a step now and then waits on it (every step is listed in the line)
    e2e_s = statistics.median(e2e_times)
    e2e_s = replica_max(e2e_s, pg)
    link = link_probe(device)
    # ocpi_init_octree inside the end-to-end steps: the chunked upload, with
    # the cloud binned as its chunks land (the call returns when the copy is
    # done)
    upload_ms = round(statistics.median(init_times) * 1e3, 3)

    # ---- roofline of the dominant stage
    peak, peak_kind = peaks()
    sb = stage_bytes(st, n, STRIDE, stage_avg)
    sub_ms = sum(v for k, v in stage_avg.items() if k.startswith("sub_l"))
    stage_ms = {"count": stage_avg.get("count", 0), "distribute": stage_avg.get("distribute", 0),
                "subsample": sub_ms}
    dom = max(stage_ms, key=stage_ms.get)
    achieved = sb[dom] / (stage_ms[dom] * 1e-3) / 1e9
    traffic = None
    try:
        if WORKLOAD != WORKLOADS["C"]["name"]:
            raise KeyError("the DRAM capture covers the headline workload only")
        # DRAM bytes per point of the stage, from one ncu capture of this
        # workload (profiles/dram_traffic_lod_build_120M_f64.md), scaled to n
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            tr = json.load(f)["stages"].get(dom)
            if tr:
                traffic = int(tr["bytes_per_point"] * n)
    except Exception:
        pass
    total_alg = sum(sb.values())
    line = {
        "metric": metric_name(), "value": round(value, 3), "unit": "Mpts/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if CLOUD_TYPE == 1 else "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "points": n, "record_bytes": STRIDE, "scale": SCALE, **CFG,
                   "l2": l2_note, "generator_seed": SEED},
        "gpu_launches": int(st.get("kernel_launches", 0)) * args.steps,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes": sb[dom]},
        "build": {"stage_ms": {k: round(v, 3) for k, v in stage_avg.items()},
                  "alg_bytes_total": total_alg,
                  "whole_build_gbs": round(total_alg / (ms_step * 1e-3) / 1e9, 1),
                  "tree_nodes": st["tree_nodes"], "internal_nodes": st["internal_nodes"], "p_in": st["p_in"],
                  "p_out": st["p_out"], "wall_s": round(wall, 3), "wall_ms_per_step": round(wall * 1e3 / args.steps, 3),
                  "device_ms_per_step": round(statistics.mean(gen_ms), 3), "upload_ms": upload_ms},
        "e2e": {"value": round(n * ws / e2e_s / 1e6, 3), "unit": "Mpts/s", "h2d_bytes_per_step": n * STRIDE,
                "d2h_bytes_per_step": hier_bytes + rec_bytes, "ms": round(e2e_s * 1e3, 2),
                "ms_mean": round(statistics.mean(e2e_times) * 1e3, 2), "steps": len(e2e_times),
                "step_ms": [round(x * 1e3, 2) for x in e2e_times],
                "init_ms": [round(x * 1e3, 2) for x in init_times], **link},
        "clocks": clk,
        "reference_cuda": {"available": False,
                           "reason": "the reference's own CUDA pipeline, compiled unmodified for sm_103a, did not "
                                     "complete on this GPU: its subsampling reads node fields that nothing "
                                     "initialises and accesses memory outside its buffers on every cloud it was "
                                     "given; it is not run again"},
    }
    if rank == 0:
        # Potree export of the last build, outside every timed region
        line["export"] = export_timing(s, int(st["points_total"]))
    if rank == 0 and not args.no_cpu_baseline:
        # the oracle builds the same whole cloud on the host cores; its result
        # is the check of the GPU build (outside every timed region)
        hier_gpu = s.hierarchy().tobytes()
        s.close()
        t, r = cpu_oracle_run(cloud_host, bb, n, threads)
        line["cpu_baseline"] = {"value": round(n / t / 1e6, 3), "unit": "Mpts/s", "cores": threads,
                                "kind": "port", "sample": "the whole %d-point cloud, same bbox and settings" % n}
        stats_equal = all(st[k] == r.stats[k] for k in STAT_KEYS)
        line["verified"] = {"by": "CPU oracle, same cloud", "hierarchy_equal": hier_gpu == r.hierarchy.tobytes(),
                            "stats_equal": stats_equal,
                            "hierarchy_sha256": hashlib.sha256(hier_gpu).hexdigest(),
                            "packed_colour_overflow_cells": int(r.stats["guard_color_overflow"]),
                            "reference_guards": {k: int(r.stats[k]) for k in
                                                 ("guard_capacity", "guard_truncation", "guard_root_leaf")}}
        line["verified"]["ok"] = line["verified"]["hierarchy_equal"] and stats_equal
        del r
    else:
        s.close()
    if rank == 0:
        print(json.dumps(line))
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
