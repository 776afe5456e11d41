"""Writes golden.json beside this script: small seeded LOD builds computed by
the CPU oracle, as regression fixtures for the oracle and the CUDA path.

Each case records the cloud's parameters and a digest of its bytes (so a
change of the cloud construction is caught separately), the exact
hierarchy.bin bytes, a digest of every node's 18-byte records and source
indices sorted inside the node (the contract compares them as multisets),
and the tree statistics.

The reference's own tests hold no golden output files; its known answers
are pinned in test_oracle_kat.py.  These fixtures pin this project's oracle
(and, through test_golden.py, the GPU path) to the outputs it produced when
they were generated.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))

CASES = [
    dict(name="heightfield_f32_inter", shape="heightfield", cloud_type=0, n=20000, seed=101, scale=0.001,
         chunk_grid=64, sub_grid=32, merge_threshold=500, modes=dict(inter=True)),
    dict(name="planes_f32_random_intra", shape="planes", cloud_type=0, n=20000, seed=102, scale=0.001,
         chunk_grid=64, sub_grid=16, merge_threshold=500, modes=dict(random=True, intra=True)),
    dict(name="clusters_f64_random_inter_weighted", shape="clusters", cloud_type=1, n=20000, seed=103, scale=0.01,
         chunk_grid=32, sub_grid=16, merge_threshold=300, modes=dict(random=True, inter=True, weighting=True)),
    dict(name="lattice_f64_first_point", shape="lattice", cloud_type=1, n=8000, seed=104, scale=0.001,
         chunk_grid=32, sub_grid=32, merge_threshold=200, modes=dict()),
]
SEED = 0x5EED


def golden_cloud(shape, cloud_type, n, seed):
    """Interleaved records (x, y, z float32 or float64, then r, g, b bytes)
    built from numpy's integer generator with exact arithmetic only
    (dyadic fractions, float adds and multiplies), so that the bytes are the
    same on every platform."""
    rng = np.random.default_rng(seed)
    u = lambda k: rng.integers(0, 1 << 20, size=k).astype(np.float64) / float(1 << 20)   # exact
    if shape == "heightfield":   # 10 m x 10 m, a polynomial surface plus 20 flat boxes
        x, y = u(n) * 10.0, u(n) * 10.0
        xn, yn = x / 16.0, y / 16.0
        z = (xn * (1.0 - xn) + yn * yn * (1.0 - yn)) * 2.0 + (u(n) - 0.5) / 512.0
        box = rng.integers(0, 20, size=n)
        on_box = u(n) < 0.3
        z = np.where(on_box, 0.25 + box.astype(np.float64) / 64.0, z)
    elif shape == "planes":   # three axis planes with density varying along them
        k = rng.integers(0, 3, size=n)
        a, b = u(n) * 30.0, u(n) * u(n) * 30.0
        c = 7.5 + (u(n) - 0.5) / 256.0
        x = np.where(k == 0, c, a)
        y = np.where(k == 1, c, np.where(k == 0, a, b))
        z = np.where(k == 2, c, b)
    elif shape == "clusters":   # hot spots: Irwin-Hall sums around 12 centres in 3 km
        centre = rng.integers(0, 12, size=n).astype(np.float64)
        spread = sum(u(n) for _ in range(4)) - 2.0
        x = 250.0 * centre + spread * 40.0
        y = 3000.0 - 200.0 * centre + (sum(u(n) for _ in range(4)) - 2.0) * 40.0
        z = 100.0 + centre * 2.5 + u(n) * 3.0
    elif shape == "lattice":   # a 20^3 lattice, cell boundaries hit exactly
        i = np.arange(n)
        x, y, z = (i % 20) * 0.25, ((i // 20) % 20) * 0.25, (i // 400) * 0.25
    else:
        raise ValueError(shape)
    ft = np.float32 if cloud_type == 0 else np.float64
    rec = np.zeros(n, np.dtype([("p", ft, 3), ("c", np.uint8, 3)]))
    rec["p"][:, 0], rec["p"][:, 1], rec["p"][:, 2] = x, y, z
    rgb = (np.stack([x * 7.0, y * 11.0, z * 13.0], axis=1).astype(np.int64) + rng.integers(0, 20, size=(n, 3))) % 256
    rec["c"] = rgb.astype(np.uint8)
    return rec.view(np.uint8).reshape(-1)


def case_cloud(c):
    from helpers import cli_scale, octree_api

    cloud = golden_cloud(c["shape"], c["cloud_type"], c["n"], c["seed"])
    stride = 15 if c["cloud_type"] == 0 else 27
    bb = octree_api.cubic_bbox(cloud, c["n"], stride, c["cloud_type"])
    return cloud, stride, bb, cli_scale(c["scale"])


def records_digest(hier, records, lut):
    from helpers import node_sorted

    r, l = node_sorted(hier, records, lut)
    return hashlib.sha256(r.tobytes() + l.astype("<u4").tobytes()).hexdigest()


STAT_KEYS = ["points_total", "p_out", "depth", "tree_nodes", "leaf_nodes", "internal_nodes"]


def oracle_case(c):
    from helpers import flags_of
    import oracle

    cloud, stride, bb, sc = case_cloud(c)
    r = oracle.run(cloud, n=c["n"], stride=stride, cloud_type=c["cloud_type"], scale=[sc] * 3, bb_min=bb[:3],
                   bb_max=bb[3:], chunk_grid=c["chunk_grid"], sub_grid=c["sub_grid"],
                   merge_threshold=c["merge_threshold"], flags=flags_of(c["modes"]), seed=SEED, keep_levels=False)
    assert r.stats["error"] == 0, r.stats
    return cloud, r


def main():
    out = {"seed": SEED, "cases": []}
    for c in CASES:
        cloud, r = oracle_case(c)
        out["cases"].append(dict(
            c, cloud_sha256=hashlib.sha256(np.ascontiguousarray(cloud).tobytes()).hexdigest(),
            hierarchy_hex=r.hierarchy.tobytes().hex(),
            records_sha256=records_digest(r.hierarchy, r.records, r.lut),
            stats={k: int(r.stats[k]) for k in STAT_KEYS}))
        print(c["name"], len(r.hierarchy), "nodes", int(r.stats["points_total"]), "records")
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
