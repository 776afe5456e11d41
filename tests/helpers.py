"""Shared test helpers: synthetic cases, oracle runs, GPU runs and the parity
comparison.

Parity contract (GPU result vs the CPU oracle):
  * hierarchy.bin bytes are identical (BFS order, types, masks, point counts,
    byte offsets and sizes of every node);
  * inside every node the 18-byte records -- and the cloud indices they come
    from -- are equal as multisets (the order of records inside one node is
    not part of the contract: the reference fills nodes in atomic order);
  * the tree statistics are equal.
"""
import os
import sys
from dataclasses import dataclass

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "octree-cuda_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import octree_api  # noqa: E402


@dataclass
class Case:
    cloud: np.ndarray
    n: int
    stride: int
    cloud_type: int
    scale: tuple
    bb_min: tuple
    bb_max: tuple


# scale as the reference CLI passes it: a float32 value widened to double
# (src/argparser.h:12, src/main.cpp:86)
def cli_scale(s):
    return float(np.float32(s))


def make_case(kind, cloud_type, n, seed, scale=0.001, stride=None):
    stride = stride or (15 if cloud_type == 0 else 27)
    cloud = octree_api.synthetic_cloud(kind, cloud_type, n, seed, stride)
    bb = octree_api.cubic_bbox(cloud, n, stride, cloud_type)
    sc = cli_scale(scale)
    return Case(cloud, n, stride, cloud_type, (sc, sc, sc), tuple(bb[:3]), tuple(bb[3:]))


def case_from_points(xyz, rgb, cloud_type, scale=0.001, bbox=None):
    """Interleaved records from arrays (xyz: (n,3) float, rgb: (n,3) uint8)."""
    n = len(xyz)
    ft = np.float32 if cloud_type == 0 else np.float64
    dt = np.dtype([("p", ft, 3), ("c", np.uint8, 3)])
    rec = np.zeros(n, dt)
    rec["p"] = xyz
    rec["c"] = rgb
    cloud = rec.view(np.uint8).reshape(-1)
    stride = dt.itemsize
    if bbox is None:
        bb = octree_api.cubic_bbox(cloud, n, stride, cloud_type)
    else:
        bb = np.asarray(bbox, np.float64)
    sc = cli_scale(scale)
    return Case(cloud, n, stride, cloud_type, (sc, sc, sc), tuple(bb[:3]), tuple(bb[3:]))


def flags_of(cfg):
    import oracle

    f = 0
    if cfg.get("intra"):
        f |= oracle.F_INTRA
    if cfg.get("inter"):
        f |= oracle.F_INTER
    if cfg.get("replacement", True):
        f |= oracle.F_REPLACE
    if cfg.get("random"):
        f |= oracle.F_RANDOM
    if cfg.get("weighting"):
        f |= oracle.F_WEIGHT
    if cfg.get("weight_literal"):
        f |= oracle.F_WEIGHT_LITERAL
    if cfg.get("weight_local"):
        f |= oracle.F_WEIGHT_LOCAL
    if cfg.get("weight_reverse"):
        f |= oracle.F_WEIGHT_REVERSE
    return f


def run_oracle(case, cfg, threads=None, keep_levels=False):
    import oracle

    return oracle.run(case.cloud, n=case.n, stride=case.stride, cloud_type=case.cloud_type, scale=case.scale,
                      bb_min=case.bb_min, bb_max=case.bb_max, chunk_grid=cfg.get("chunk_grid", 512),
                      sub_grid=cfg.get("sub_grid", 128), merge_threshold=cfg.get("merge_threshold", 10000),
                      output_factor=cfg.get("output_factor", 2.2), flags=flags_of(cfg),
                      seed=cfg.get("seed", 0x5EED), threads=threads, keep_levels=keep_levels)


def run_gpu(case, cfg, device=0):
    s = octree_api.OctreeSession(device)
    s.set_cloud(case.cloud, n=case.n, stride=case.stride, cloud_type=case.cloud_type, scale=case.scale,
                bb_min=case.bb_min, bb_max=case.bb_max)
    s.configure(**cfg)
    s.init()
    s.generate()
    return s


def node_sorted(hier, records, lut):
    """Records and LUT entries sorted inside each node (BFS node order)."""
    idx = np.concatenate([np.arange(o // 18, o // 18 + p, dtype=np.int64)
                          for o, p in zip(hier["byte_offset"], hier["points"])]) if len(hier) else np.zeros(0, np.int64)
    node = np.repeat(np.arange(len(hier)), hier["points"].astype(np.int64))
    r = records[idx]
    l = lut[idx]
    order = np.lexsort((r["b"], r["g"], r["r"], r["z"], r["y"], r["x"], node))
    lorder = np.lexsort((l, node))
    return r[order], l[lorder]


STAT_KEYS = ["points_total", "p_out", "depth", "tree_nodes", "leaf_nodes", "internal_nodes", "sparse_nodes",
             "dense_nodes", "max_leaf_depth", "min_leaf_points", "max_leaf_points", "mean_leaf_points",
             "stdev_leaf_points", "out_capacity"]


def compare_results(ref, session):
    """Assert GPU == oracle under the parity contract."""
    assert ref.stats["error"] == 0, ref.stats
    st = session.stats()
    for k in STAT_KEYS:
        assert st[k] == ref.stats[k], (k, st[k], ref.stats[k])
    hier = session.hierarchy()
    assert hier.tobytes() == ref.hierarchy.tobytes(), "hierarchy.bin differs"
    rec = session.records()
    lut = session.lut()
    assert len(rec) == len(ref.records)
    g_r, g_l = node_sorted(hier, rec, lut)
    o_r, o_l = node_sorted(ref.hierarchy, ref.records, ref.lut)
    assert np.array_equal(g_l, o_l), "per-node point sets differ"
    assert g_r.tobytes() == o_r.tobytes(), "per-node records differ"
    return st
