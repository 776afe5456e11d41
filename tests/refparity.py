"""Parity of this library's build against the reference's own CUDA build.

The reference (oracle/refcuda.py runs it) and this library build the same
cloud; their Potree exports are compared under the parity contract:

  * hierarchy.bin: same number of entries in the same BFS order; type, child
    mask, point count and byte size of every entry identical; byte offsets of
    internal nodes identical (the reference places them in DFS post-order after
    the N leaf points, kernel_helpers.cuh:55-59);
  * leaf byte offsets: the reference assigns them in atomic order
    (hierarchical_merging.cuh:110), so they are compared as a tiling of
    [0, 18 N) with each leaf's records equal as a multiset;
  * internal nodes: every record is one point of the node's subtree, lying in
    an occupied cell of the node's subsampling grid, one record per occupied
    cell, the same cells as this library's records.  The identity of the point
    chosen in a cell is racy in the reference (first atomicExch winner,
    fp_subsampling.cuh:72; arrival order, rp_subsampling.cuh:108-114), so it
    is not compared.  Colours, matched by cell: identical for intra- and
    inter-cell averaging, within `weighted_tol` per channel for distance-weighted
    averaging, and the chosen point's own colour without averaging;
  * octree.bin: the reference writes its whole output capacity, of which only
    the first (N + P_out) records are referenced; those are compared;
  * metadata.json: identical.

A record's cell is found from its quantised coordinate: every cloud point whose
quantised coordinate floor((p - min) / scale) equals the record's is a
candidate, and the candidate inside the node's subtree gives the cell (the
reference's cell formula, mapPointToGrid, kernel_helpers.cuh:10-25, over the
node box of the calculateChildMinBB chain, tools.cu:29-61).  Records whose
candidates disagree on the cell are counted as ambiguous and left out of the
cell match; the tests bound their number.
"""
import numpy as np

HIER_LEAF = 1


def load_xyz(cloud, n, stride, cloud_type):
    """(n, 3) float64 coordinates and (n, 3) colours of interleaved records."""
    ft = np.float32 if cloud_type == 0 else np.float64
    w = 4 if cloud_type == 0 else 8
    rec = np.ascontiguousarray(cloud[: n * stride]).reshape(n, stride)
    xyz = rec[:, : 3 * w].copy().view(ft).astype(np.float64)
    rgb = rec[:, 3 * w: 3 * w + 3].astype(np.uint16)
    return xyz, rgb


def quantised(xyz, bb_min, scale):
    """floor((p - min) * (1 / scale)) per axis, in binary64 as the reference
    evaluates it (point_distributing.cuh:245-247)."""
    sf = np.array([1.0 / s for s in scale])
    return np.floor((xyz - np.asarray(bb_min)) * sf).astype(np.int64)


def qkey(q):
    return (q[:, 0] & 0x1FFFFF) | ((q[:, 1] & 0x1FFFFF) << 21) | ((q[:, 2] & 0x1FFFFF) << 42)


def node_geometry(hier, depth, bb_min, cubic):
    """Per hierarchy entry (BFS): level, integer cell coordinates at that level,
    node box minimum (the reference's chain) and the node grid's cell size."""
    n = len(hier)
    level = np.zeros(n, np.int64)
    ijk = np.zeros((n, 3), np.int64)
    mn = np.zeros((n, 3), np.float64)
    level[0] = depth
    mn[0] = bb_min
    nxt = 1
    for i in range(n):
        m = int(hier["mask"][i])
        if m == 0:
            continue
        side = cubic / 2.0 ** (depth - level[i])
        cside = side / 2.0
        for s in range(8):
            if not (m >> s) & 1:
                continue
            level[nxt] = level[i] - 1
            bits = np.array([(s >> 2) & 1, (s >> 1) & 1, s & 1])
            ijk[nxt] = 2 * ijk[i] + bits
            mn[nxt] = [mn[i][a] + cside if bits[a] else mn[i][a] for a in range(3)]
            nxt += 1
    assert nxt == n, "hierarchy masks do not describe a BFS tree"
    side = cubic / 2.0 ** (depth - level)
    return level, ijk, mn, side


def cells_of(xyz, mn, side, grid):
    """mapPointToGrid over a node box (kernel_helpers.cuh:14-24); the grid
    extent is the node box's cubicSize, (min.x + side) - min.x."""
    t = ((mn[0] + side) - mn[0]) / grid
    u = (xyz - mn) / t
    i = np.fmin(u, grid - 1.0).astype(np.int64)
    return i[:, 0] + i[:, 1] * grid + i[:, 2] * grid * grid


def guards(hier, n, output_factor):
    """The reference-bug guards from a hierarchy: (capacity, truncation)."""
    total = int(hier["points"].astype(np.int64).sum())
    cap = total > int(np.float32(n) * np.float32(output_factor))
    leaf = hier["mask"] == 0
    max_leaf = int(hier["points"][leaf].max()) if leaf.any() else 0
    blocks = np.ceil(max_leaf * 8 / 128.0)
    gx = min(blocks, 65535)
    gy = np.ceil(blocks / 65535)
    extent = int(gx) * int(gy) * 128
    trunc = bool((hier["points"][1:] > extent).any())
    return cap, trunc


def compare_exports(case, cfg, mine, ref, depth, weighted_tol=1):
    """Assert the parity contract between this library's export `mine` and the
    reference's `ref` (dicts with 'hierarchy', 'octree', 'metadata'), and
    return a report dict (ambiguous records, weighted deviation histogram)."""
    sub = cfg.get("sub_grid", 128)
    intra, inter = bool(cfg.get("intra")), bool(cfg.get("inter"))
    weighted = inter and bool(cfg.get("weighting"))
    hm, hr = mine["hierarchy"], ref["hierarchy"]
    assert len(hm) == len(hr), ("node count", len(hm), len(hr))
    for f in ("type", "mask", "points", "byte_size"):
        assert np.array_equal(hm[f], hr[f]), "hierarchy field %s differs" % f
    internal = hm["mask"] != 0
    assert np.array_equal(hm["byte_offset"][internal], hr["byte_offset"][internal]), "internal byte offsets differ"
    n = case.n
    leaf = ~internal
    lo = hr["byte_offset"][leaf].astype(np.int64)
    sz = hr["byte_size"][leaf].astype(np.int64)
    order = np.argsort(lo)
    assert lo[order][0] == 0 if len(lo) else True
    assert np.array_equal(lo[order][1:], (lo[order] + sz[order])[:-1]), "reference leaves do not tile"
    assert int((lo + sz).max()) == 18 * n, "reference leaves do not cover the N points"
    total = int(hm["points"].astype(np.int64).sum())
    rec_dt = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4"), ("r", "<u2"), ("g", "<u2"), ("b", "<u2")])
    assert len(ref["octree"]) >= 18 * total, "reference octree.bin shorter than the referenced records"
    rr = np.frombuffer(ref["octree"][: 18 * total].tobytes(), rec_dt)
    rm = np.frombuffer(mine["octree"][: 18 * total].tobytes(), rec_dt)
    assert len(mine["octree"]) == 18 * total
    assert mine["metadata"] == ref["metadata"], "metadata.json differs"

    def node_slice(h, i):
        o = int(h["byte_offset"][i]) // 18
        return slice(o, o + int(h["points"][i]))

    def as_void(a):
        return np.sort(np.ascontiguousarray(a).view("V18").ravel())

    # leaves: records equal as multisets
    for i in np.nonzero(leaf)[0]:
        a = rm[node_slice(hm, i)]
        b = rr[node_slice(hr, i)]
        assert as_void(a).tobytes() == as_void(b).tobytes(), "leaf %d records differ" % i

    # internal nodes: one record per occupied cell, matched by (node, cell)
    xyz, rgb = load_xyz(case.cloud, n, case.stride, case.cloud_type)
    q = quantised(xyz, case.bb_min, case.scale)
    keys = qkey(q)
    korder = np.argsort(keys, kind="stable")
    ksorted = keys[korder]
    cubic = case.bb_max[0] - case.bb_min[0]
    level, ijk, mn, side = node_geometry(hm, depth, case.bb_min, cubic)
    # leaf of every cloud point (from this library's leaf LUT), as level + cell
    lut = mine["lut"]
    pt_level = np.empty(n, np.int64)
    pt_ijk = np.empty((n, 3), np.int64)
    for i in np.nonzero(leaf)[0]:
        idx = lut[node_slice(hm, i)]
        pt_level[idx] = level[i]
        pt_ijk[idx] = ijk[i]
    inodes = np.nonzero(internal)[0]
    S3 = sub ** 3

    def gather(h, recs):
        sel = np.concatenate([np.arange(int(h["byte_offset"][i]) // 18, int(h["byte_offset"][i]) // 18
                                        + int(h["points"][i])) for i in inodes])
        node = np.repeat(inodes, h["points"][inodes].astype(np.int64))
        return sel, node

    def cells(pts, node):
        m = mn[node]
        t = ((m[:, 0] + side[node]) - m[:, 0]) / sub
        u = (xyz[pts] - m) / t[:, None]
        c = np.fmin(u, sub - 1.0).astype(np.int64)
        return c[:, 0] + c[:, 1] * sub + c[:, 2] * sub * sub

    def in_subtree(pts, node):
        d = level[node] - pt_level[pts]
        return np.all((pt_ijk[pts] >> d[:, None]) == ijk[node], axis=1)

    msel, mnode = gather(hm, rm)
    mkey = mnode * S3 + cells(lut[msel], mnode)
    assert len(np.unique(mkey)) == len(mkey), "two of this library's records share a cell"
    rsel, rnode = gather(hr, rr)
    ref_rec = rr[rsel]
    rk = qkey(np.stack([ref_rec["x"], ref_rec["y"], ref_rec["z"]], 1).astype(np.int64))
    a = np.searchsorted(ksorted, rk, "left")
    b = np.searchsorted(ksorted, rk, "right")
    assert np.all(b > a), "a reference record matches no cloud point"
    rpt = np.full(len(rk), -1, np.int64)
    rkey = np.full(len(rk), -1, np.int64)
    one = (b - a) == 1
    cand = korder[a[one]]
    ins = in_subtree(cand, rnode[one])
    assert ins.all(), "a reference record is no point of its node's subtree"
    rpt[one] = cand
    rkey[one] = rnode[one] * S3 + cells(cand, rnode[one])
    ambiguous = 0
    for j in np.nonzero(~one)[0]:
        cs = korder[a[j]:b[j]]
        nodes = np.full(len(cs), rnode[j])
        cs = cs[in_subtree(cs, nodes)]
        assert len(cs), "a reference record is no point of its node's subtree"
        ck = np.unique(rnode[j] * S3 + cells(cs, np.full(len(cs), rnode[j])))
        if len(ck) == 1:
            rkey[j] = ck[0]
            rpt[j] = cs[0]
        else:
            ambiguous += 1
    ok = rkey >= 0
    assert len(np.unique(rkey[ok])) == ok.sum(), "two reference records share a cell"
    morder = np.argsort(mkey)
    ms = mkey[morder]
    pos = np.searchsorted(ms, rkey[ok])
    assert np.all(pos < len(ms)) and np.array_equal(ms[np.minimum(pos, len(ms) - 1)], rkey[ok]), \
        "the reference occupies a cell this library does not"
    mrec = rm[msel][morder][pos]
    mcol = np.stack([mrec["r"], mrec["g"], mrec["b"]], 1).astype(np.int64)
    rcol = np.stack([ref_rec["r"], ref_rec["g"], ref_rec["b"]], 1)[ok].astype(np.int64)
    max_dev = 0
    dev_hist = [0, 0, 0, 0]
    if not (intra or inter):
        # no averaging: the chosen point's own colour
        assert np.array_equal(rcol, rgb[rpt[ok]].astype(np.int64)), "a reference colour is not its point's"
    elif weighted:
        dev = np.abs(rcol - mcol)
        max_dev = int(dev.max(initial=0))
        dev_hist = np.bincount(np.minimum(dev.ravel(), 3), minlength=4).tolist()
        assert max_dev <= weighted_tol, ("weighted colour deviation", max_dev, dev_hist)
    else:
        assert np.array_equal(rcol, mcol), "averaged colours differ"
    return dict(ambiguous=ambiguous, records=total, internal_records=int(len(rk)), weighted_max_dev=max_dev,
                weighted_dev_hist=dev_hist)
