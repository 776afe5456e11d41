"""GPU parity against the reference's own CUDA pipeline.

The reference (PotreeConverterGPU's OctreeApi, compiled unmodified for sm_103a
by oracle/build_ref.py) and this library build the same seeded clouds on the
same GPU; their Potree exports are compared under the parity contract of
tests/refparity.py.  The tests skip when the reference runner is not built
(no staged reference sources).

Every case is checked first against the reference-bug guards (output
capacity, launch-extent truncation, root below the threshold): the reference
writes past its output buffers when the capacity guard trips, so it is never
run on such a cloud.
"""
import json
import os
import tempfile

import numpy as np
import pytest

from helpers import make_case, octree_api, run_gpu

import refcuda  # noqa: E402  (oracle/, test infrastructure)
from refparity import compare_exports, guards

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refcuda.available(), reason="reference runner not built (oracle/build_ref.py)")]

CASES = {
    # name: (kind, cloud_type, n, seed, scale, modes)
    "heightfield_f32_inter": (0, 0, 1_500_000, 101, 0.001, dict(inter=True)),
    "planes_f32_random_intra": (1, 0, 1_500_000, 102, 0.001, dict(random=True, intra=True)),
    "zipf_f64_first_point": (2, 1, 1_500_000, 103, 0.01, dict()),
    "zipf_f64_intra": (2, 1, 1_500_000, 104, 0.01, dict(intra=True)),
    "planes_f32_random_plain": (1, 0, 1_000_000, 105, 0.001, dict(random=True)),
    "planes_f32_random_inter_weighted": (1, 0, 1_500_000, 106, 0.001, dict(random=True, inter=True,
                                                                            weighting=True)),
    "heightfield_f32_inter_weighted": (0, 0, 1_500_000, 107, 0.001, dict(inter=True, weighting=True)),
    # the 5,138,448-point heightfield workload at full size
    "workload_5M_f32_inter": (0, 0, 5_138_448, 20240602, 0.001, dict(inter=True)),
}


def export_mine(session, tmp):
    d = os.path.join(tmp, "mine")
    os.makedirs(d, exist_ok=True)
    session.export_potree(d)
    hier = np.fromfile(os.path.join(d, "hierarchy.bin"), refcuda.HIER_DTYPE)
    octree = np.fromfile(os.path.join(d, "octree.bin"), np.uint8)
    with open(os.path.join(d, "metadata.json")) as fh:
        meta = json.load(fh)
    return dict(hierarchy=hier, octree=octree, metadata=meta, lut=session.lut())


def build_both(name, tmp):
    kind, cloud_type, n, seed, scale, modes = CASES[name]
    case = make_case(kind, cloud_type, n, seed=seed, scale=scale)
    cfg = dict(chunk_grid=512, sub_grid=128, merge_threshold=10000, output_factor=2.2, **modes)
    s = run_gpu(case, cfg)
    mine = export_mine(s, tmp)
    depth = s.stats()["depth"]
    cap, trunc = guards(mine["hierarchy"], n, cfg["output_factor"])
    assert not cap, "capacity guard: the reference would overflow its output buffer on this cloud"
    assert not trunc, "truncation guard: the reference would cut a child's points on this cloud"
    ref = refcuda.run(case.cloud, n, case.stride, cloud_type, case.scale[0], report=True, **cfg)
    assert tuple(ref["bb"]) == tuple(case.bb_min) + tuple(case.bb_max), "bounding boxes differ"
    return case, cfg, s, mine, ref, depth


@pytest.mark.parametrize("name", sorted(CASES))
def test_export_equals_reference(name):
    with tempfile.TemporaryDirectory() as tmp:
        case, cfg, s, mine, ref, depth = build_both(name, tmp)
        rep = compare_exports(case, cfg, mine, ref, depth, weighted_tol=1)
        print(name, rep)
        assert rep["ambiguous"] <= max(10, rep["internal_records"] // 10000), rep
        s.close()


def _keys(d, prefix=""):
    out = set()
    for k, v in d.items():
        out.add(prefix + k)
        if isinstance(v, dict) and k not in ("timings", "memory"):
            out |= _keys(v, prefix + k + ".")
    return out


def test_statistics_json_schema_and_values():
    """statistics.json keeps the reference's schema (OctreeApi/src/json_exporter.h:14-99),
    and its node statistics equal the reference's for the same build."""
    with tempfile.TemporaryDirectory() as tmp:
        case, cfg, s, mine, ref, depth = build_both("heightfield_f32_inter", tmp)
        path = os.path.join(tmp, "statistics.json")
        s.export_json_report(path)
        with open(path) as fh:
            st = json.load(fh)
        rs = ref["statistics"]
        assert list(st.keys()) == list(rs.keys())
        assert _keys(st) == _keys(rs)
        for k in ("depth", "chunking", "subsampling", "resultNodes", "overallNodes"):
            assert st[k] == rs[k], k
        for k in ("meanPointsPerLeafNode", "stdevPointsPerLeafNode", "minPointsPerNode", "maxPointsPerNode"):
            assert st["pointDistribution"][k] == pytest.approx(rs["pointDistribution"][k], rel=1e-6), k
        for k in ("accumulatedKernelTime", "accumulatedMemCpyTime", "accumulatedMallocTime",
                  "accumulatedProcessTimings"):
            assert k in st["timings"]
        for k in ("peak", "reserveEvents", "cumulatedReserved"):
            assert k in st["memory"]
        s.close()


def test_distribution_histogram_written():
    """ocpi_export_distribution_histogram writes the point distribution page of
    octree_processor_impl/histogram.cu:39-119: the reference's automatic bin
    width, bins from the smallest leaf, every leaf counted once.  The
    reference's own page is not produced here: it increments one bin past
    the end of its vector for the largest leaf (histogram.cu:58-63), where
    this library adds that bin."""
    import math
    import re

    with tempfile.TemporaryDirectory() as tmp:
        kind, cloud_type, n, seed, scale, modes = CASES["heightfield_f32_inter"]
        case = make_case(kind, cloud_type, n, seed=seed, scale=scale)
        cfg = dict(chunk_grid=512, sub_grid=128, merge_threshold=10000, **modes)
        s = run_gpu(case, cfg)
        st = s.stats()
        path = os.path.join(tmp, "hist.html")
        s.export_histogram(path, 0)
        html = open(path).read()
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
        assert "mergingThreshold(10000), points(%d)" % n in html
        s.close()
