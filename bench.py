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

N_POINTS = 119_701_547
STRIDE = 27
CLOUD_TYPE = 1
SCALE = float(np.float32(0.01))   # the CLI passes the scale through a float (src/argparser.h:12)
SEED = 20240601
CFG = dict(chunk_grid=512, merge_threshold=10000, output_factor=2.2, sub_grid=128, inter=True, replacement=True)
WORKLOAD = "lod_build_120M_f64_terrain_zipf"
CPU_SAMPLE = 12_000_000   # points of the same cloud timed on the CPU oracle


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


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
                                          "--format=csv,noheader,nounits", "-lms", "200"],
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
    cloud = octree_api.synthetic_cloud(2, CLOUD_TYPE, n, SEED, STRIDE, threads)
    bb = octree_api.cubic_bbox(cloud, n, STRIDE, CLOUD_TYPE, threads)
    return cloud, bb, time.time() - t


def cpu_oracle_time(cloud, bb, n_sample, threads):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    sample = cloud[: n_sample * STRIDE]
    flags = oracle.F_INTER | oracle.F_REPLACE
    t = time.perf_counter()
    r = oracle.run(sample, n=n_sample, stride=STRIDE, cloud_type=CLOUD_TYPE, scale=[SCALE] * 3, bb_min=bb[:3],
                   bb_max=bb[3:], chunk_grid=CFG["chunk_grid"], sub_grid=CFG["sub_grid"],
                   merge_threshold=CFG["merge_threshold"], output_factor=CFG["output_factor"], flags=flags,
                   threads=threads, keep_levels=False)
    dt = time.perf_counter() - t
    if r.stats["error"]:
        raise RuntimeError("oracle failed: %s" % r.stats)
    return dt


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
        "impl": "reference", "metric": "Mpts/s octree build @120M pts", "value": round(v, 3), "unit": "Mpts/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "points": N_POINTS, "sample_points": sample, **CFG},
        "cpu_baseline": {"value": round(v, 3), "unit": "Mpts/s", "cores": threads, "kind": "port",
                         "sample": "first %d points of the seeded 119.7M-point cloud, same bbox and settings" % sample},
        "e2e": {"value": round(v, 3), "unit": "Mpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--points", type=int, default=N_POINTS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)

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

    # ---- device-resident build: CUDA events of the builder stream
    clocks = ClockSampler(device)
    clocks.start()
    barrier()
    stage_sum = {}
    gen_ms = []
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        s.generate()
        t = s.timings()
        gen_ms.append(sum(t.values()))
        for k, v in t.items():
            stage_sum[k] = stage_sum.get(k, 0.0) + v
    barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    st = s.stats()
    ms_step = statistics.mean(gen_ms)
    if pg:
        import torch

        tt = torch.tensor([ms_step], dtype=torch.float64)
        pg.all_reduce(tt, op=pg.ReduceOp.MAX)
        ms_step = float(tt.item())
    value = n * ws / (ms_step * 1e-3) / 1e6
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
    for i in range(max(2, min(args.steps, 3))):
        barrier()
        t0 = time.perf_counter()
        s.init()
        s.generate()
        h = s.hierarchy()
        octree_api._check(L.ocpi_get_records(s._h, recs.ctypes.data), "ocpi_get_records")
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_times)
    if pg:
        import torch

        tt = torch.tensor([e2e_s], dtype=torch.float64)
        pg.all_reduce(tt, op=pg.ReduceOp.MAX)
        e2e_s = float(tt.item())
    upload_ms = None
    try:
        s.init()
        upload_ms = s.timings().get("upload")
    except Exception:
        pass

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
        "metric": "Mpts/s octree build @120M pts", "value": round(value, 3), "unit": "Mpts/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "points": n, "record_bytes": STRIDE, "scale": SCALE, **CFG,
                   "l2": "inputs larger than L2 (3.2 GB cloud)", "generator_seed": SEED},
        "gpu_launches": int(st.get("kernel_launches", 0)) * args.steps,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes": sb[dom]},
        "build": {"stage_ms": {k: round(v, 3) for k, v in stage_avg.items()},
                  "alg_bytes_total": total_alg,
                  "whole_build_gbs": round(total_alg / (ms_step * 1e-3) / 1e9, 1),
                  "tree_nodes": st["tree_nodes"], "internal_nodes": st["internal_nodes"], "p_in": st["p_in"],
                  "p_out": st["p_out"], "wall_s": round(wall, 3), "upload_ms": upload_ms},
        "e2e": {"value": round(n * ws / e2e_s / 1e6, 3), "unit": "Mpts/s", "h2d_bytes_per_step": n * STRIDE,
                "d2h_bytes_per_step": hier_bytes + rec_bytes, "ms": round(e2e_s * 1e3, 2)},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        sample = min(CPU_SAMPLE, n)
        t = cpu_oracle_time(cloud_host, bb, sample, threads)
        line["cpu_baseline"] = {"value": round(sample / t / 1e6, 3), "unit": "Mpts/s", "cores": threads,
                                "kind": "port",
                                "sample": "first %d points of the same cloud, same bbox and settings" % sample}
    s.close()
    if rank == 0:
        print(json.dumps(line))
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
