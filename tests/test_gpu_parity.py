"""GPU parity tests: the LOD build through the C ABI (libOctreeApi.so on the
GPU) against the CPU oracle, on seeded synthetic clouds, for every
subsampling / colour-filtering mode and both record layouts."""
import numpy as np
import pytest

from helpers import case_from_points, compare_results, make_case, octree_api, run_gpu, run_oracle

pytestmark = pytest.mark.gpu

MODES = {
    "fp_none": dict(),
    "fp_intra": dict(intra=True),
    "fp_inter": dict(inter=True),
    "fp_inter_w": dict(inter=True, weighting=True),
    "rp_none": dict(random=True),
    "rp_intra": dict(random=True, intra=True),
    "rp_inter": dict(random=True, inter=True),
    "rp_inter_w": dict(random=True, inter=True, weighting=True),
}


@pytest.mark.parametrize("mode", sorted(MODES))
@pytest.mark.parametrize("kind,cloud_type", [(0, 0), (1, 0), (2, 1)])
def test_modes_small_grids(kind, cloud_type, mode):
    case = make_case(kind, cloud_type, 120_000, seed=11 + kind, scale=0.001 if cloud_type == 0 else 0.01)
    cfg = dict(chunk_grid=64, sub_grid=32, merge_threshold=1500, **MODES[mode])
    ref = run_oracle(case, cfg)
    s = run_gpu(case, cfg)
    compare_results(ref, s)
    s.close()


@pytest.mark.parametrize("kind,cloud_type,mode", [(0, 0, "fp_inter"), (1, 0, "rp_intra"), (1, 0, "rp_inter_w"),
                                                  (2, 1, "fp_inter"), (2, 1, "rp_none")])
def test_reference_grids(kind, cloud_type, mode):
    """Grids 512/128 and threshold 10000 as in the reference's run commands."""
    case = make_case(kind, cloud_type, 1_500_000, seed=101 + kind, scale=0.001 if cloud_type == 0 else 0.01)
    cfg = dict(chunk_grid=512, sub_grid=128, merge_threshold=10000, **MODES[mode])
    ref = run_oracle(case, cfg)
    s = run_gpu(case, cfg)
    compare_results(ref, s)
    s.close()


def test_cuboid_known_answers():
    """Known answers of the reference's 128^3 unit-cuboid tests
    (Tests/test_merging_sparse.cpp:32-157, test_subsampling_sparse.cpp:17-33),
    with a 15-byte record layout."""
    case = make_case(3, 0, 128 ** 3, seed=0, scale=1.0)
    assert case.bb_min == (0.5, 0.5, 0.5) and case.bb_max == (127.5, 127.5, 127.5)
    cfg = dict(chunk_grid=128, sub_grid=128, merge_threshold=10000, debug=1)
    s = run_gpu(case, cfg)
    st = s.stats()
    assert st["sparse_nodes"] == 2_396_745
    for lvl, grid in enumerate([128, 64, 32, 16, 8, 4, 2, 1]):
        counts = s.level_counts(lvl, grid)
        assert np.all(counts == 8 ** lvl), lvl
    hier = s.hierarchy()
    # root: 128^3 subsampled points; 2^3 level: 64^3 each; 4^3 level: 32^3 each
    assert hier["points"][0] == 128 ** 3
    assert np.all(hier["points"][1:9] == 64 ** 3)
    assert np.all(hier["points"][9:73] == 32 ** 3)
    leaves = hier["type"] == 1
    assert leaves.sum() == 512 and np.all(hier["points"][leaves] == 4096)
    ref = run_oracle(case, {k: v for k, v in cfg.items() if k != "debug"})
    compare_results(ref, s)
    s.close()


def test_root_below_threshold():
    case = make_case(0, 0, 5_000, seed=3)
    cfg = dict(chunk_grid=512, sub_grid=128, merge_threshold=10000, inter=True)
    ref = run_oracle(case, cfg)
    s = run_gpu(case, cfg)
    compare_results(ref, s)
    hier = s.hierarchy()
    assert len(hier) == 1 and hier["type"][0] == 1 and hier["points"][0] == 5_000
    s.close()


def test_single_point_and_identical_points():
    for n in (1, 40_000):
        xyz = np.tile(np.array([[1.25, -3.5, 7.0]]), (n, 1))
        rgb = np.full((n, 3), 200, np.uint8)
        case = case_from_points(xyz, rgb, 0, bbox=[0, -4, 6, 2, -2, 8])
        cfg = dict(chunk_grid=64, sub_grid=32, merge_threshold=100, intra=True)
        ref = run_oracle(case, cfg)
        s = run_gpu(case, cfg)
        compare_results(ref, s)
        s.close()


@pytest.mark.parametrize("cloud_type", [0, 1])
def test_cell_boundaries(cloud_type):
    """Points on and one ulp around every cell boundary of the chunking grid and
    of the subsampling grids, plus points on the bbox maximum."""
    rng = np.random.default_rng(5)
    ft = np.float32 if cloud_type == 0 else np.float64
    lo, side, G = 3.0, 7.0, 64
    t = side / G
    k = np.arange(G + 1)
    edges = (lo + k * t).astype(ft)
    cand = np.concatenate([edges, np.nextafter(edges, ft(-np.inf)), np.nextafter(edges, ft(np.inf)),
                           (lo + k * t / 8).astype(ft), (lo + (k + 0.5) * t / 4).astype(ft)])
    cand = cand[(cand >= lo) & (cand <= lo + side)]
    n = 60_000
    xyz = np.stack([rng.choice(cand, n), rng.choice(cand, n), rng.choice(cand, n)], axis=1).astype(np.float64)
    xyz[:100] = lo + side
    rgb = rng.integers(0, 256, (n, 3), dtype=np.uint8)
    case = case_from_points(xyz, rgb, cloud_type, scale=0.001, bbox=[lo, lo, lo, lo + side, lo + side, lo + side])
    for mode in ("fp_inter", "rp_intra"):
        cfg = dict(chunk_grid=G, sub_grid=16, merge_threshold=500, **MODES[mode])
        ref = run_oracle(case, cfg)
        s = run_gpu(case, cfg)
        compare_results(ref, s)
        s.close()


def test_large_coordinates_double():
    """UTM-like coordinates with a 27-byte layout: the fp32 fast path must fall
    back to binary64 near boundaries."""
    rng = np.random.default_rng(9)
    n = 200_000
    base = np.array([512345.678, 4501234.567, 250.0])
    xyz = base + rng.random((n, 3)) * np.array([100.0, 100.0, 5.0])
    xyz[: n // 10] = np.round(xyz[: n // 10], 2)   # coordinates on a 1 cm lattice
    rgb = rng.integers(0, 256, (n, 3), dtype=np.uint8)
    case = case_from_points(xyz, rgb, 1, scale=0.01)
    cfg = dict(chunk_grid=128, sub_grid=64, merge_threshold=2000, inter=True)
    ref = run_oracle(case, cfg)
    s = run_gpu(case, cfg)
    compare_results(ref, s)
    s.close()


def test_repeat_generate_same_session():
    """Two generate calls on one session give identical hierarchies and records."""
    case = make_case(0, 0, 200_000, seed=21)
    cfg = dict(chunk_grid=128, sub_grid=64, merge_threshold=2000, random=True, inter=True)
    s = run_gpu(case, cfg)
    h1 = s.hierarchy().tobytes()
    from helpers import node_sorted
    r1, l1 = node_sorted(s.hierarchy(), s.records(), s.lut())
    s.init()
    s.generate()
    assert s.hierarchy().tobytes() == h1
    r2, l2 = node_sorted(s.hierarchy(), s.records(), s.lut())
    assert np.array_equal(l1, l2) and r1.tobytes() == r2.tobytes()
    s.close()


@pytest.mark.parametrize("cloud_type", [0, 1])
def test_shuffled_point_order(cloud_type):
    """Points in random order: warps see many cells and leaves at once, so the
    per-point paths of counting and distribution (no runs of equal keys) are
    exercised."""
    from helpers import Case

    case = make_case(1, cloud_type, 300_000, seed=33)
    perm = np.random.default_rng(5).permutation(case.n)
    recs = case.cloud[: case.n * case.stride].reshape(case.n, case.stride)[perm].reshape(-1)
    case = Case(np.ascontiguousarray(recs), case.n, case.stride, case.cloud_type, case.scale, case.bb_min, case.bb_max)
    cfg = dict(chunk_grid=128, sub_grid=64, merge_threshold=3000, inter=True)
    compare_results(run_oracle(case, cfg), run_gpu(case, cfg))


def test_output_host_arrays():
    """Records and LUT streamed into registered host arrays during generate
    equal the ones read back afterwards; a too-small array is an error."""
    torch = pytest.importorskip("torch")
    case = make_case(0, 1, 400_000, seed=41)
    cfg = dict(chunk_grid=128, sub_grid=64, merge_threshold=3000, inter=True)
    s = run_gpu(case, cfg)
    n = s.stats()["points_total"]
    cap = n + 100
    rec = torch.empty(cap * 18, dtype=torch.uint8, pin_memory=True).numpy()
    lut = torch.empty(cap, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    s.set_output_host(rec, lut)
    for _ in range(2):
        rec[:] = 0xAB
        lut[:] = 0xFFFFFFFF
        s.init()
        s.generate()
        # the same build read back by a fresh copy from the device
        want_rec = s.records().view(np.uint8).reshape(-1)
        want_lut = np.empty(n, np.uint32)
        octree_api._check(octree_api.load_library().ocpi_get_lut(s._h, want_lut.ctypes.data), "ocpi_get_lut")
        assert rec[: n * 18].tobytes() == want_rec.tobytes()
        assert np.array_equal(lut[:n], want_lut)
        assert (rec[n * 18:] == 0xAB).all()
    small = torch.empty((case.n + 1) * 18, dtype=torch.uint8, pin_memory=True).numpy()
    s.set_output_host(small)
    s.init()
    with pytest.raises(octree_api.OctreeError, match="too small"):
        s.generate()
    s.close()


@pytest.mark.parametrize("kind,cloud_type", [(0, 0), (2, 1)])
def test_device_bounding_box(kind, cloud_type):
    """ocpi_compute_cloud_bb equals the CLI's host computation exactly (NaN
    coordinates skipped), and a build on it equals the oracle's."""
    from helpers import Case

    case = make_case(kind, cloud_type, 300_000, seed=51)
    cfg = dict(chunk_grid=128, sub_grid=64, merge_threshold=3000, inter=True)
    ft = np.float32 if cloud_type == 0 else np.float64

    def device_box(cloud):
        s = octree_api.OctreeSession(0)
        s.set_cloud(cloud, n=case.n, stride=case.stride, cloud_type=cloud_type, scale=case.scale)
        s.configure(**cfg)
        s.init()
        real, cubic = s.compute_cloud_bb()
        return s, cubic

    # a NaN coordinate: fmin / fmax skip it
    nan_cloud = case.cloud.copy()
    nan_cloud[7 * case.stride: 7 * case.stride + 3 * np.dtype(ft).itemsize].view(ft)[1] = np.nan
    s, cubic = device_box(nan_cloud)
    want = octree_api.cubic_bbox(nan_cloud, case.n, case.stride, cloud_type)
    assert cubic.tobytes() == np.asarray(want, np.float64).tobytes(), (cubic, want)
    s.close()

    s, cubic = device_box(case.cloud)
    want = octree_api.cubic_bbox(case.cloud, case.n, case.stride, cloud_type)
    assert cubic.tobytes() == np.asarray(want, np.float64).tobytes(), (cubic, want)
    s.generate()
    ref = run_oracle(Case(case.cloud, case.n, case.stride, cloud_type, case.scale, tuple(want[:3]), tuple(want[3:])),
                     cfg)
    compare_results(ref, s)
    s.close()


@pytest.mark.parametrize("mode,flags", [(dict(inter=True), 2), (dict(random=True, inter=True, weighting=True), 26),
                                        (dict(intra=True), 1)])
def test_memory_estimate_bounds_allocations(tmp_path, mode, flags):
    """After a build, the session's device allocations stay within
    ocpi_estimate_memory's bound, and the memory report lists them."""
    case = make_case(1, 0, 400_000, seed=61)
    cfg = dict(chunk_grid=128, sub_grid=64, merge_threshold=3000, **mode)
    s = run_gpu(case, cfg)
    used = s.device_memory()
    bound, ref = octree_api.estimate_memory(case.n, case.stride, case.cloud_type, 128, 3000, 2.2, 64, flags)
    assert 0 < used <= bound, (used, bound)
    report = tmp_path / "memory_report.html"
    octree_api._check(octree_api.load_library().ocpi_export_memory_report(s._h, str(report).encode()), "report")
    s.close()
    text = report.read_text()
    assert "count pyramid" in text and str(used) in text


def test_potree_export_reader(tmp_path):
    """An independent reader of the exported Potree 2.0 files: metadata,
    hierarchy.bin entries (22 bytes, breadth-first), byte ranges that tile
    octree.bin, and every record inside its node's cube."""
    import json

    case = make_case(0, 1, 300_000, seed=71)
    cfg = dict(chunk_grid=128, sub_grid=64, merge_threshold=3000, inter=True)
    s = run_gpu(case, cfg)
    s.export_potree(str(tmp_path))
    st = s.stats()
    s.close()
    meta = json.loads((tmp_path / "metadata.json").read_text())
    hier = np.fromfile(tmp_path / "hierarchy.bin", dtype=octree_api.HIER_DTYPE)
    recs = np.fromfile(tmp_path / "octree.bin", dtype=octree_api.RECORD_DTYPE)
    assert octree_api.HIER_DTYPE.itemsize == 22 and octree_api.RECORD_DTYPE.itemsize == 18
    assert meta["version"] == "2.0" and meta["points"] == st["points_total"] == len(recs)
    assert meta["hierarchy"]["firstChunkSize"] == len(hier) * 22 == st["tree_nodes"] * 22
    assert [a["name"] for a in meta["attributes"]] == ["position", "rgb"]
    # node types: 0 = inner node with children, 1 = leaf
    assert ((hier["mask"] != 0) == (hier["type"] == 0)).all() and ((hier["mask"] == 0) == (hier["type"] == 1)).all()
    assert (hier["byte_size"] == hier["points"].astype(np.uint64) * 18).all()
    ranges = sorted((int(o), int(o + z)) for o, z in zip(hier["byte_offset"], hier["byte_size"]) if z)
    end = 0
    for a, b in ranges:
        assert a == end
        end = b
    assert end == len(recs) * 18
    # breadth-first walk: node cubes relative to the bounding-box minimum
    scale = meta["scale"][0]
    side0 = meta["boundingBox"]["max"][0]
    mins = np.zeros((len(hier), 3))
    sides = np.zeros(len(hier))
    sides[0] = side0
    nxt = 1
    for i in range(len(hier)):
        for sl in range(8):
            if int(hier["mask"][i]) & (1 << sl):
                sides[nxt] = sides[i] / 2
                mins[nxt] = mins[i] + sides[nxt] * np.array([(sl >> 2) & 1, (sl >> 1) & 1, sl & 1])
                nxt += 1
    assert nxt == len(hier)
    xyz = np.stack([recs["x"], recs["y"], recs["z"]], axis=1).astype(np.float64) * scale
    for i in range(len(hier)):
        a = int(hier["byte_offset"][i]) // 18
        p = xyz[a: a + int(hier["points"][i])]
        assert (p >= mins[i] - 2 * scale).all() and (p <= mins[i] + sides[i] + 2 * scale).all(), i


def test_reference_reader_reads_export(tmp_path):
    """The reference's own Potree reader (tools/potree_to_ply.py:51-248,
    standard-library Python; staged into oracle/_ref/tools by
    oracle/build_ref.py) reads this library's export: it walks hierarchy.bin
    breadth first, reads every node's byte range of octree.bin and writes one
    PLY file per level plus one of all leaves.  Each file must hold exactly
    the records of its level's nodes, in breadth-first order."""
    import re
    import subprocess
    import sys

    import build_ref

    reader = build_ref.reader()
    if reader is None:
        pytest.skip("reference reader not staged (oracle/build_ref.py)")
    case = make_case(0, 0, 400_000, seed=73)
    cfg = dict(chunk_grid=128, sub_grid=64, merge_threshold=3000, inter=True)
    s = run_gpu(case, cfg)
    out = tmp_path / "potree"
    out.mkdir()
    s.export_potree(str(out))
    hier = s.hierarchy()
    recs = s.records()
    s.close()
    ply = tmp_path / "ply"
    ply.mkdir()
    r = subprocess.run([sys.executable, reader, "-i", str(out) + "/", "-o", str(ply)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    counts = [int(v) for v in re.findall(r"Exported points: (\d+)", r.stdout)]
    # node levels from the breadth-first masks
    level = np.zeros(len(hier), np.int64)
    nxt = 1
    for i in range(len(hier)):
        for _ in range(bin(int(hier["mask"][i])).count("1")):
            level[nxt] = level[i] + 1
            nxt += 1
    assert nxt == len(hier)
    depth = int(level.max()) + 1
    assert len(counts) == depth + 1
    raw = recs.view(np.uint8).reshape(-1, 18)

    def node_bytes(idx):
        parts = [raw[int(hier["byte_offset"][i]) // 18: int(hier["byte_offset"][i]) // 18 + int(hier["points"][i])]
                 for i in idx]
        return np.concatenate(parts).tobytes() if parts else b""

    def ply_body(name):
        data = (ply / name).read_bytes()
        head, body = data.split(b"end_header\n", 1)
        n = int(re.search(rb"element vertex (\d+)", head).group(1))
        assert len(body) == 18 * n
        return n, body

    for lv in range(depth):
        idx = np.nonzero(level == lv)[0]
        n, body = ply_body("converted_level_%d.ply" % lv)
        assert n == counts[lv] == int(hier["points"][idx].sum())
        assert body == node_bytes(idx), lv
    leaves = np.nonzero(hier["mask"] == 0)[0]
    n, body = ply_body("converted_level_leaf.ply")
    assert n == counts[-1] == case.n
    assert body == node_bytes(leaves)


# statistics.json of OctreeApi/src/json_exporter.h:14-99: top-level keys in
# order, and the keys of each section ("averaging" only with averaging)
STATISTICS_SCHEMA = {
    "depth": None,
    "chunking": ["grid", "mergingThreshold"],
    "subsampling": ["grid", "strategy", "averaging"],
    "resultNodes": ["octreeNodes", "leafNodeAmount", "internalNodeAmount", "maxLeafDepth"],
    "overallNodes": ["sparseOctreeNodes", "denseOctreeNodes", "memorySaving"],
    "pointDistribution": ["meanPointsPerLeafNode", "stdevPointsPerLeafNode", "minPointsPerNode", "maxPointsPerNode"],
    "timings": ["kernel", "memcpy", "cudamalloc", "process", "accumulatedKernelTime", "accumulatedMemCpyTime",
                "accumulatedMallocTime", "accumulatedProcessTimings"],
    "memory": ["peak", "reserveEvents", "cumulatedReserved", "events"],
}


@pytest.mark.parametrize("mode", [dict(inter=True), dict(random=True)])
def test_statistics_json_schema(tmp_path, mode):
    """ocpi_export_json_report keeps the reference's statistics.json schema,
    with the build's node statistics, stage and process timings and device
    allocations."""
    import json

    case = make_case(1, 0, 300_000, seed=75)
    cfg = dict(chunk_grid=128, sub_grid=64, merge_threshold=3000, **mode)
    ref = run_oracle(case, cfg)
    s = run_gpu(case, cfg)
    s.export_potree(str(tmp_path))
    path = tmp_path / "statistics.json"
    s.export_json_report(str(path))
    used = s.device_memory()
    s.close()
    st = json.loads(path.read_text())
    assert list(st.keys()) == list(STATISTICS_SCHEMA)
    for k, keys in STATISTICS_SCHEMA.items():
        if keys is None:
            continue
        want = [x for x in keys if x != "averaging" or mode.get("inter") or mode.get("intra")]
        assert list(st[k].keys()) == want, k
    S = ref.stats
    assert st["depth"] == S["depth"]
    assert st["chunking"] == {"grid": 128, "mergingThreshold": 3000}
    assert st["subsampling"]["strategy"] == ("EXPLICIT RANDOM SUBSAMPLING" if mode.get("random")
                                             else "IMPLICIT RANDOM SUBSAMPLING")
    assert st["resultNodes"] == {"octreeNodes": S["leaf_nodes"] + S["internal_nodes"], "leafNodeAmount": S["leaf_nodes"],
                                 "internalNodeAmount": S["internal_nodes"], "maxLeafDepth": S["max_leaf_depth"]}
    assert st["overallNodes"]["sparseOctreeNodes"] == S["sparse_nodes"]
    assert st["overallNodes"]["denseOctreeNodes"] == S["dense_nodes"]
    pd = st["pointDistribution"]
    assert pd["minPointsPerNode"] == S["min_leaf_points"] and pd["maxPointsPerNode"] == S["max_leaf_points"]
    assert pd["meanPointsPerLeafNode"] == pytest.approx(S["mean_leaf_points"], rel=1e-6)
    tm = st["timings"]
    assert "upload_count" in tm["memcpy"] or "upload" in tm["memcpy"]
    assert all(v["duration"] >= 0 and v["invocations"] == 1 for v in tm["kernel"].values())
    assert tm["accumulatedKernelTime"] == pytest.approx(sum(v["duration"] for v in tm["kernel"].values()), rel=1e-5)
    assert set(tm["process"]) == {"Initialising octree", "Generating octree", "Exporting octree"}
    assert tm["accumulatedMallocTime"] > 0
    mem = st["memory"]
    assert mem["peak"] == used == sum(mem["events"].values())
    assert mem["reserveEvents"] > 0 and mem["cumulatedReserved"] >= mem["peak"]


def test_distribution_histogram(tmp_path):
    """ocpi_export_distribution_histogram writes the point-distribution page of
    octree_processor_impl/histogram.cu:39-119: the reference's automatic bin
    width (3.5 stdev / leaves^(1/3), in float), bins from the smallest leaf,
    every leaf counted once.  The reference sizes its bins so that the
    largest leaf falls one bin past the end of its vector (histogram.cu:58-63);
    this library adds that bin."""
    import math
    import re

    case = make_case(0, 0, 600_000, seed=77)
    cfg = dict(chunk_grid=256, sub_grid=64, merge_threshold=2000, inter=True)
    s = run_gpu(case, cfg)
    st = s.stats()
    path = tmp_path / "hist.html"
    s.export_histogram(str(path), 0)
    html = path.read_text()
    width = int(re.search(r"binWidth\((\d+)\)", html).group(1))
    f32 = np.float32
    expect = math.ceil(f32(3.5) * (f32(st["stdev_leaf_points"]) / f32(st["leaf_nodes"]) ** f32(1.0 / 3.0)))
    assert width == max(1, expect)
    data = [int(v) for v in re.search(r"data:\[([0-9,]*)\]", html).group(1).split(",")]
    assert sum(data) == st["leaf_nodes"]
    hier = s.hierarchy()
    pts = hier["points"][hier["mask"] == 0].astype(np.int64)
    bins = np.minimum((pts - st["min_leaf_points"]) // width, len(data) - 1)
    assert np.array_equal(np.bincount(bins, minlength=len(data)), data)
    assert "mergingThreshold(2000), points(%d)" % case.n in html
    s.export_histogram(str(path), 50)
    assert "binWidth(50)" in path.read_text()
    s.close()


# The plain workloads at full size: seeded clouds of the reference datasets'
# sizes (coin 5,138,448 float; heidentor 25,836,417 float), grids 512/128.
FULL_SIZE = {
    "A_5M_f32_inter": (0, 0, 5_138_448, 20240602, 0.001, dict(inter=True)),
    "B1_26M_f32_random_intra": (1, 0, 25_836_417, 20240603, 0.001, dict(random=True, intra=True)),
    "B2_26M_f32_random_inter_weighted": (1, 0, 25_836_417, 20240603, 0.001,
                                          dict(random=True, inter=True, weighting=True)),
}


@pytest.mark.parametrize("name", sorted(FULL_SIZE))
def test_workloads_full_size(name):
    kind, cloud_type, n, seed, scale, modes = FULL_SIZE[name]
    case = make_case(kind, cloud_type, n, seed=seed, scale=scale)
    cfg = dict(chunk_grid=512, sub_grid=128, merge_threshold=10000, output_factor=2.2, **modes)
    ref = run_oracle(case, cfg)
    s = run_gpu(case, cfg)
    compare_results(ref, s)
    s.close()
