"""CPU tests of the oracle against the known answers held by the reference's
own tests (OctreeApi/OctreeLibrary/Tests/), re-derived for a 15-byte record
layout where the reference fixture used 12-byte records."""
import ctypes

import numpy as np
import pytest

import oracle
from helpers import case_from_points, make_case, run_oracle


def test_level_tables_512():
    """test_octree.cu:46-135: dense node total and per-level sizes/offsets of a
    512 chunking grid."""
    xyz = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]])
    case = case_from_points(xyz, np.zeros((2, 3), np.uint8), 0, bbox=[0, 0, 0, 1, 1, 1])
    r = run_oracle(case, dict(chunk_grid=512, sub_grid=128, merge_threshold=10000), keep_levels=True)
    assert r.stats["dense_nodes"] == 153_391_689
    assert r.stats["depth"] == 9
    sizes = [len(c) for c in r.level_counts]
    assert sizes == [512 ** 3, 256 ** 3, 128 ** 3, 64 ** 3, 32 ** 3, 16 ** 3, 8 ** 3, 4 ** 3, 2 ** 3, 1]
    offsets = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    assert list(offsets) == [0, 134217728, 150994944, 153092096, 153354240, 153387008, 153391104, 153391616,
                             153391680, 153391688]


def test_cuboid_merging_known_answers():
    """test_merging_sparse.cpp:32-157: a 128^3 unit lattice with threshold
    10000: every level-0 cell holds one point, 2,396,745 occupied cells, root
    count 2,097,152, the 8^3 level is the first finished level."""
    case = make_case(3, 0, 128 ** 3, seed=0, scale=1.0)
    assert case.bb_min == (0.5, 0.5, 0.5) and case.bb_max == (127.5, 127.5, 127.5)
    r = run_oracle(case, dict(chunk_grid=128, sub_grid=128, merge_threshold=10000), keep_levels=True)
    assert r.stats["error"] == 0
    assert r.stats["sparse_nodes"] == 2_396_745
    for lvl in range(8):
        assert np.all(r.level_counts[lvl] == 8 ** lvl), lvl
    assert r.level_counts[7][0] == 2_097_152
    nodes = r.nodes
    # levels 7..5 internal, 8^3 level (level 4) leaves with 4096 points
    for lvl, internal, count in [(7, 1, 1), (6, 1, 8), (5, 1, 64), (4, 0, 512)]:
        m = nodes["level"] == lvl
        assert m.sum() == count and np.all(nodes["internal"][m] == internal)
    leaves = nodes["internal"] == 0
    assert np.all(nodes["points"][leaves] == 4096)
    # test_point_distribution_sparse.cpp:10-93: every point lies inside its leaf
    # cube and the leaves hold all points
    assert nodes["points"][leaves].sum() == 128 ** 3
    pts = case.cloud.view(np.dtype([("p", "<f4", 3), ("c", "u1", 3)]))["p"]
    for k in np.flatnonzero(leaves)[:64]:
        node = nodes[k]
        idx = r.lut[node["data_idx"]: node["data_idx"] + node["points"]]
        m = int(node["morton"])
        cx = cy = cz = 0
        for b in range(3):   # leaf level 4 in a 128 grid: 3 bits per axis
            cx |= ((m >> (3 * b + 2)) & 1) << b
            cy |= ((m >> (3 * b + 1)) & 1) << b
            cz |= ((m >> (3 * b)) & 1) << b
        p = pts[idx]
        for a, c in enumerate((cx, cy, cz)):
            assert np.all(p[:, a] > c * 16) and np.all(p[:, a] < (c + 1) * 16)


def test_cuboid_subsampling_known_answers():
    """test_subsampling_sparse.cpp:17-33,64: subsample sizes 128^3 (root),
    64^3 (2^3 level) and 32^3 (4^3 level)."""
    case = make_case(3, 0, 128 ** 3, seed=0, scale=1.0)
    r = run_oracle(case, dict(chunk_grid=128, sub_grid=128, merge_threshold=10000))
    nodes = r.nodes
    assert nodes["points"][nodes["level"] == 7][0] == 128 ** 3
    assert np.all(nodes["points"][nodes["level"] == 6] == 64 ** 3)
    assert np.all(nodes["points"][nodes["level"] == 5] == 32 ** 3)
    # one subsampled point per occupied cell: points_total = N + internal points
    assert r.stats["points_total"] == 128 ** 3 + 128 ** 3 + 8 * 64 ** 3 + 64 * 32 ** 3


def test_node_statistics_dummy_tree():
    """test_octree.cu:4-42,155-178: root with leaves of 100, 350, 800, 1300, 700
    and 250 points (slots 0,1,3,4,6,7): 6 leaves, 1 internal node, min 100,
    max 1300, mean 583.3, max leaf depth 1."""
    counts = {0: 100, 1: 350, 3: 800, 4: 1300, 6: 700, 7: 250}
    xyz = []
    for slot, c in counts.items():
        ox, oy, oz = (slot >> 2) & 1, (slot >> 1) & 1, slot & 1
        xyz.append(np.tile([[0.25 + ox, 0.25 + oy, 0.25 + oz]], (c, 1)))
    xyz = np.concatenate(xyz)
    case = case_from_points(xyz, np.zeros((len(xyz), 3), np.uint8), 0, bbox=[0, 0, 0, 2, 2, 2])
    r = run_oracle(case, dict(chunk_grid=2, sub_grid=4, merge_threshold=3000))
    st = r.stats
    assert st["internal_nodes"] == 1 and st["leaf_nodes"] == 6
    assert st["min_leaf_points"] == 100 and st["max_leaf_points"] == 1300
    assert st["mean_leaf_points"] == pytest.approx(583.3, rel=1e-3)
    assert st["max_leaf_depth"] == 1
    assert r.hierarchy["mask"][0] == 0b11011011


def test_reference_cell_formula():
    """mapPointToGrid (kernel_helpers.cuh:10-25): fmin clamp at the maximum,
    truncation toward zero just below the minimum, negative index below."""
    assert oracle.cell_axis(10.0, 0.0, 10.0, 512) == 511
    assert oracle.cell_axis(-0.001, 0.0, 10.0, 512) == 0
    assert oracle.cell_axis(-0.05, 0.0, 10.0, 512) == -1
    assert oracle.cell_axis(float("nan"), 0.0, 10.0, 512) == 511
    assert oracle.out_coord(1.2345, 1.0, 0.001) == 234


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors (Salmon et al., SC'11 / Random123)."""
    lib = oracle.lib()
    lib.oracle_philox.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3
    vectors = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in vectors:
        c = (ctypes.c_uint32 * 4)(*ctr)
        k = (ctypes.c_uint32 * 2)(*key)
        out = (ctypes.c_uint32 * 4)()
        lib.oracle_philox(c, k, out)
        assert list(out) == want


def test_weight_function():
    """Fixed-point weights: exp(-10 (d/r)^2) * 2^28 against numpy in double."""
    lib = oracle.lib()
    rng = np.random.default_rng(1)
    for _ in range(2000):
        u = rng.random(3).astype(np.float32) * 4 + 10
        n = np.floor(u).astype(np.int32) + rng.integers(-1, 2, 3)
        d2 = np.sum(((n + 0.5) - u.astype(np.float64)) ** 2)
        want = np.exp(-10 * min(d2 * 4 / 27, 1.5)) * 2 ** 28
        got = lib.oracle_weight_q(float(u[0]), float(u[1]), float(u[2]), int(n[0]), int(n[1]), int(n[2]))
        assert abs(got - want) <= 1 + 4e-6 * want
    for x in np.linspace(-15, 0, 301):
        assert lib.oracle_exp_neg(float(x)) == pytest.approx(np.exp(x), rel=2e-6)


def test_invalid_configurations_rejected():
    case = make_case(0, 0, 1000, seed=1)
    for cfg in (dict(chunk_grid=500), dict(chunk_grid=1), dict(intra=True, weighting=True), dict(sub_grid=0)):
        r = run_oracle(case, cfg)
        assert r.stats["error"] == 1, cfg


def _colour_dev(a, b, n):
    a, b = a[n:], b[n:]
    assert np.array_equal(a[["x", "y", "z"]], b[["x", "y", "z"]])
    dev = np.abs(np.stack([a["r"], a["g"], a["b"]]).astype(np.int64) - np.stack([b["r"], b["g"], b["b"]]))
    return int(dev.max(initial=0)), np.bincount(np.minimum(dev.ravel(), 3), minlength=4).tolist()


@pytest.mark.parametrize("kind,cloud_type,scale,modes", [
    (1, 0, 0.001, dict(random=True, inter=True, weighting=True)),
    (0, 0, 0.001, dict(inter=True, weighting=True)),
    (2, 1, 0.01, dict(inter=True, weighting=True)),
])
def test_weighted_rule_against_reference_arithmetic(kind, cloud_type, scale, modes):
    """The canonical distance-weighted colours (fixed-point weights from the
    point's own position, exact integer sums) against the reference's own
    arithmetic restated literally (binary64 distances, float exp, float sums,
    truncating division; kernel_inter_cell_filtering.cuh:137-189,
    fp_subsampling.cuh:209-217), at the reference grids 512/128.

    * Per node, from the same children's colours: every channel within 1.
    * Whole builds, where each level averages the level below: the
      reference's truncating float average of colours whose exact average is
      an integer c lands on c - 1 whenever rounding leaves it a little low, and
      that loss compounds from level to level.  Every channel stays within 2,
      and fewer than 1 in 100,000 differ by 2.  The reference against itself
      with its float sums in the reverse order (its atomics have no fixed
      order) is printed beside it."""
    case = make_case(kind, cloud_type, 400_000, seed=31 + kind, scale=scale)
    cfg = dict(chunk_grid=512, sub_grid=128, merge_threshold=10000, **modes)
    canon = run_oracle(case, cfg, threads=8)
    local = run_oracle(case, dict(cfg, weight_literal=True, weight_local=True), threads=8)
    lit = run_oracle(case, dict(cfg, weight_literal=True), threads=8)
    rev = run_oracle(case, dict(cfg, weight_literal=True, weight_reverse=True), threads=8)
    for r in (local, lit, rev):
        assert canon.hierarchy.tobytes() == r.hierarchy.tobytes()
        assert np.array_equal(canon.lut, r.lut)
    assert len(canon.records) - case.n > 1000
    m_local, h_local = _colour_dev(canon.records, local.records, case.n)
    m_lit, h_lit = _colour_dev(canon.records, lit.records, case.n)
    m_self, h_self = _colour_dev(lit.records, rev.records, case.n)
    print("weighted colours vs the reference arithmetic: per node max %d %s; whole build max %d %s; "
          "reference vs itself reversed max %d %s" % (m_local, h_local, m_lit, h_lit, m_self, h_self))
    assert m_local <= 1
    assert m_lit <= 2 and h_lit[2] * 100_000 < sum(h_lit)
