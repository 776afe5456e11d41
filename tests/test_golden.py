"""Regression fixtures (tests/golden/golden.json, written by
tests/golden/make_golden.py from the CPU oracle): the oracle and the CUDA
path must reproduce each case's hierarchy.bin bytes, the digest of every
node's records and source indices (sorted inside the node) and the tree
statistics."""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402
from helpers import octree_api  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))
CASES = GOLDEN["cases"]
IDS = [c["name"] for c in CASES]


def check_cloud(c, cloud):
    got = hashlib.sha256(np.ascontiguousarray(cloud).tobytes()).hexdigest()
    assert got == c["cloud_sha256"], "the synthetic cloud generator changed; regenerate the fixtures"


@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_oracle_reproduces_golden(c):
    cloud, r = make_golden.oracle_case(c)
    check_cloud(c, cloud)
    assert r.hierarchy.tobytes().hex() == c["hierarchy_hex"]
    assert make_golden.records_digest(r.hierarchy, r.records, r.lut) == c["records_sha256"]
    assert {k: int(r.stats[k]) for k in c["stats"]} == c["stats"]


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_gpu_reproduces_golden(c):
    cloud, stride, bb, sc = make_golden.case_cloud(c)
    check_cloud(c, cloud)
    with octree_api.OctreeSession(0) as s:
        s.set_cloud(cloud, n=c["n"], stride=stride, cloud_type=c["cloud_type"], scale=[sc] * 3, bb_min=bb[:3],
                    bb_max=bb[3:])
        s.configure(chunk_grid=c["chunk_grid"], sub_grid=c["sub_grid"], merge_threshold=c["merge_threshold"],
                    seed=GOLDEN["seed"], **c["modes"])
        s.init()
        s.generate()
        h = s.hierarchy()
        assert h.tobytes().hex() == c["hierarchy_hex"]
        assert make_golden.records_digest(h, s.records(), s.lut()) == c["records_sha256"]
        st = s.stats()
        assert {k: int(st[k]) for k in c["stats"]} == c["stats"]
