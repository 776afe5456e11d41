"""ocpi_subsample_node_noalloc against the session path.

The allocation-free entry point subsamples one node in the library's fixed
scratch array.  For nodes of an octree built by ocpi_generate_octree, it is
fed the node's candidates (its children's records and LUT entries, read back
from the session) and must reproduce the node's records and source indices
exactly, as a multiset, on two calls in a row that share the scratch.

The file is named to be collected last, so that it also runs after every
other GPU test in one process; it passes alone as well.
"""
import ctypes

import numpy as np
import pytest

from helpers import make_case, run_gpu, octree_api

pytestmark = pytest.mark.gpu

SEED = 0x1234ABCD


def tree_nodes(hier, depth, bb_min, cubic):
    """Level, Morton key, bbox minimum and side of every hierarchy node (BFS),
    and the BFS indices of its children.  Child minima follow the builder:
    parent minimum + half the parent side per set slot bit (x = bit 2)."""
    n = len(hier)
    level = np.zeros(n, np.int64)
    key = np.zeros(n, np.int64)
    mn = np.zeros((n, 3), np.float64)
    children = [[] for _ in range(n)]
    level[0] = depth
    mn[0] = bb_min
    nxt = 1
    for i in range(n):
        m = int(hier["mask"][i])
        if not m:
            continue
        side = cubic / 2.0 ** (depth - level[i])
        cside = side / 2.0
        for s in range(8):
            if not m & (1 << s):
                continue
            c = nxt
            nxt += 1
            children[i].append(c)
            level[c] = level[i] - 1
            key[c] = key[i] * 8 + s
            mn[c, 0] = mn[i, 0] + cside if s & 4 else mn[i, 0]
            mn[c, 1] = mn[i, 1] + cside if s & 2 else mn[i, 1]
            mn[c, 2] = mn[i, 2] + cside if s & 1 else mn[i, 2]
    assert nxt == n
    return level, key, mn, children


def node_slice(hier, i):
    first = int(hier["byte_offset"][i]) // 18
    return first, first + int(hier["points"][i])


def run_noalloc(torch, case, cfg, flags, sess, hier, level, key, mn, children, i, cloud_dev):
    L = octree_api.load_library()
    rec = sess.records().view(np.uint8).reshape(-1, 18)
    lut = sess.lut()
    parts = [node_slice(hier, c) for c in children[i]]
    cand_rec = np.concatenate([rec[a:b] for a, b in parts])
    cand_lut = np.concatenate([lut[a:b] for a, b in parts]).astype(np.uint32)
    n = len(cand_lut)
    assert 0 < n <= octree_api.NOALLOC_MAX_CANDIDATES
    # 16 readable bytes past the last candidate record
    d_rec = torch.from_numpy(np.concatenate([np.ascontiguousarray(cand_rec).reshape(-1), np.zeros(16, np.uint8)])).cuda()
    d_lut = torch.from_numpy(cand_lut.view(np.int32)).cuda()
    o_rec = torch.full((n * 18,), 0xAB, dtype=torch.uint8, device="cuda")
    o_lut = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    status = torch.full((2,), -1, dtype=torch.int32, device="cuda")
    D3 = ctypes.c_double * 3
    cubic = case.bb_max[0] - case.bb_min[0]
    side = cubic / 2.0 ** (stats_depth(sess) - level[i])
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.ocpi_subsample_node_noalloc(
        ctypes.c_void_p(cloud_dev.data_ptr()), case.cloud_type, case.stride, D3(*case.scale), D3(*case.bb_min),
        D3(*mn[i]), side, int(level[i]), int(key[i]), cfg["sub_grid"], flags, SEED,
        ctypes.c_void_p(d_lut.data_ptr()), ctypes.c_void_p(d_rec.data_ptr()), n,
        ctypes.c_void_p(o_lut.data_ptr()), ctypes.c_void_p(o_rec.data_ptr()), ctypes.c_void_p(status.data_ptr()),
        ctypes.c_void_p(stream))
    assert rc == 0, L.ocpi_last_error()
    torch.cuda.synchronize()
    st = status.cpu().numpy().view(np.uint32)
    assert st[1] == 0, "device error bits %#x" % st[1]
    a, b = node_slice(hier, i)
    assert st[0] == b - a, (st[0], b - a)
    got_lut = o_lut.cpu().numpy().view(np.uint32)[: st[0]]
    got_rec = o_rec.cpu().numpy().reshape(-1, 18)[: st[0]]
    want_lut, want_rec = lut[a:b], rec[a:b]
    go, wo = np.argsort(got_lut, kind="stable"), np.argsort(want_lut, kind="stable")
    assert np.array_equal(got_lut[go], want_lut[wo]), "selected points differ"
    assert got_rec[go].tobytes() == want_rec[wo].tobytes(), "records differ"
    return n


def stats_depth(sess):
    return sess.stats()["depth"]


CASES = [
    # kind, cloud type, session flags, entry-point flags
    ("heightfield", 1, dict(inter=True), octree_api.SUB_INTER),
    ("planes", 0, dict(inter=True, random=True, weighting=True),
     octree_api.SUB_INTER | octree_api.SUB_RANDOM | octree_api.SUB_WEIGHTING),
    ("terrain", 1, dict(intra=True), octree_api.SUB_INTRA),
]


@pytest.mark.parametrize("kind,cloud_type,mode,flags", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_session_two_calls(kind, cloud_type, mode, flags):
    torch = pytest.importorskip("torch")
    kinds = {"heightfield": 0, "planes": 1, "terrain": 2}
    case = make_case(kinds[kind], cloud_type, 400_000, seed=77 + kinds[kind])
    cfg = dict(chunk_grid=64, merge_threshold=3000, sub_grid=32, seed=SEED, **mode)
    sess = run_gpu(case, cfg)
    hier = sess.hierarchy()
    depth = stats_depth(sess)
    cubic = case.bb_max[0] - case.bb_min[0]
    level, key, mn, children = tree_nodes(hier, depth, np.asarray(case.bb_min), cubic)
    p_in = np.array([sum(int(hier["points"][c]) for c in ch) for ch in children])
    eligible = [i for i in range(len(hier)) if children[i] and p_in[i] <= octree_api.NOALLOC_MAX_CANDIDATES]
    assert len(eligible) >= 2
    big = max(eligible, key=lambda i: p_in[i])
    small = min((i for i in eligible if level[i] != level[big]), key=lambda i: p_in[i],
                default=min(eligible, key=lambda i: p_in[i]))
    cloud = np.concatenate([case.cloud, np.zeros(64, np.uint8)])
    cloud_dev = torch.from_numpy(cloud).cuda()
    # two calls in a row on the shared scratch: the larger node, then a smaller one
    n1 = run_noalloc(torch, case, cfg, flags, sess, hier, level, key, mn, children, big, cloud_dev)
    n2 = run_noalloc(torch, case, cfg, flags, sess, hier, level, key, mn, children, small, cloud_dev)
    assert n1 >= n2
