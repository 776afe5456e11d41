"""Batched and served forms (ocpi_batch_build, ocpi_server_*): every build
run in the mix equals the same build run alone through the session API --
hierarchy.bin byte-identical, each node's records equal as a multiset."""
import numpy as np
import pytest

from helpers import make_case, node_sorted, octree_api, run_gpu

pytestmark = pytest.mark.gpu

MODES = [dict(inter=True), dict(random=True, intra=True), dict(random=True, inter=True, weighting=True), dict()]
FLAGS = [octree_api.SUB_INTER, octree_api.SUB_RANDOM | octree_api.SUB_INTRA,
         octree_api.SUB_RANDOM | octree_api.SUB_INTER | octree_api.SUB_WEIGHTING, 0]


def mixed_cases(count):
    rng = np.random.default_rng(7)
    out = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(20_000), np.log(400_000))))
        cloud_type = 0 if rng.random() < 0.8 else 1
        grids = (64, 32) if rng.random() < 0.5 else (128, 64)
        m = int(rng.integers(len(MODES)))
        out.append((make_case(i % 3, cloud_type, n, seed=1000 + i), grids, m))
    return out


def alone(case, grids, m):
    cfg = dict(chunk_grid=grids[0], sub_grid=grids[1], merge_threshold=2000, seed=99, **MODES[m])
    s = run_gpu(case, cfg)
    h, r, l = s.hierarchy(), s.records(), s.lut()
    s.close()
    return h, r, l


def job_for(case, grids, m, rec, lut, hier, device_bbox=False, cloud_id=0):
    kw = {} if device_bbox else dict(bb_min=case.bb_min, bb_max=case.bb_max)
    return octree_api.make_job(case.cloud, n=case.n, stride=case.stride, cloud_type=case.cloud_type, scale=case.scale,
                               chunk_grid=grids[0], sub_grid=grids[1], merge_threshold=2000, flags=FLAGS[m], seed=99,
                               records=rec, lut=lut, hierarchy=hier, cloud_id=cloud_id, **kw)


def check_same(want, res, rec, lut, hier):
    wh, wr, wl = want
    assert res.status == 0, res.error
    assert res.nodeCount == len(wh) and res.pointsTotal == len(wr)
    got_h = hier[: res.nodeCount * 22].view(octree_api.HIER_DTYPE)
    assert got_h.tobytes() == wh.tobytes(), "hierarchy differs from the build run alone"
    got_r = rec[: res.pointsTotal * 18].view(octree_api.RECORD_DTYPE)
    a_r, a_l = node_sorted(wh, wr, wl)
    b_r, b_l = node_sorted(got_h, got_r, lut[: res.pointsTotal])
    assert np.array_equal(a_l, b_l) and a_r.tobytes() == b_r.tobytes(), "records differ from the build run alone"


def buffers(want):
    """Host outputs holding exactly the records and nodes of the build."""
    h, r, _ = want
    return np.zeros(len(r) * 18, np.uint8), np.zeros(len(r), np.uint32), np.zeros(len(h) * 22, np.uint8)


def test_batch_equals_builds_alone():
    cases = mixed_cases(12)
    want = [alone(c, g, m) for c, g, m in cases]
    bufs = [buffers(w) for w in want]
    jobs = [job_for(c, g, m, *b, device_bbox=(i % 4 == 0)) for i, ((c, g, m), b) in enumerate(zip(cases, bufs))]
    results = octree_api.batch_build(jobs, lanes=4)
    for w, r, b in zip(want, results, bufs):
        check_same(w, r, *b)


def test_wave_batch_equals_builds_alone():
    """The batch in subsampling waves (one launch per level over a wave's
    builds): several record-type and mode groups, waves of 5, some boxes
    computed on the device; every result equals its build alone."""
    cases = mixed_cases(14)
    want = [alone(c, g, m) for c, g, m in cases]
    bufs = [buffers(w) for w in want]
    jobs = [job_for(c, g, m, *b, device_bbox=(i % 4 == 0)) for i, ((c, g, m), b) in enumerate(zip(cases, bufs))]
    results = octree_api.batch_build_wave(jobs, wave_size=5)
    for w, r, b in zip(want, results, bufs):
        check_same(w, r, *b)


def test_wave_build_that_outgrows_its_buffers_repeats_alone():
    """A wave build whose records outgrow its buffers leaves the wave's
    schedule and repeats its subsampling pass alone with larger buffers.
    Output factor 1.0 sizes the records for N only, and the 1.5M-point cloud
    is larger than any cloud the wave builders of this process have held, so
    its first pass overflows.  Every build of the wave equals its build
    alone, and the large one took a second pass."""
    cases = [make_case(1, 0, n, seed=3100 + i) for i, n in enumerate((1_500_000, 60_000, 90_000))]
    grids = (128, 64)
    want, passes = [], []
    for c in cases:
        s = run_gpu(c, dict(chunk_grid=grids[0], sub_grid=grids[1], merge_threshold=2000, seed=99,
                            output_factor=1.0, **MODES[0]))
        want.append((s.hierarchy(), s.records(), s.lut()))
        passes.append(s.stats()["subsample_passes"])
        s.close()
    assert passes[0] >= 2, "the session build did not outgrow its buffers"
    bufs = [buffers(w) for w in want]
    jobs = [octree_api.make_job(c.cloud, n=c.n, stride=c.stride, cloud_type=c.cloud_type, scale=c.scale,
                                bb_min=c.bb_min, bb_max=c.bb_max, chunk_grid=grids[0], sub_grid=grids[1],
                                merge_threshold=2000, output_factor=1.0, flags=FLAGS[0], seed=99,
                                records=b[0], lut=b[1], hierarchy=b[2]) for c, b in zip(cases, bufs)]
    results = octree_api.batch_build_wave(jobs, wave_size=3)
    for w, r, b in zip(want, results, bufs):
        check_same(w, r, *b)
    assert results[0].subsamplePasses >= 2


@pytest.mark.parametrize("graphs,lanes", [(1, 0), (0, 0), (0, 3)])
def test_tuned_waves_equal_builds_alone(graphs, lanes):
    """An explicit tuning: waves of 6, cluster caps 2/8, each wave's
    subsampling captured into one CUDA graph (or launched directly), or the
    lane executor with 3 lanes; the last wave ran the way it was asked to, and
    every result equals its build alone."""
    cases = mixed_cases(13)
    want = [alone(c, g, m) for c, g, m in cases]
    bufs = [buffers(w) for w in want]
    jobs = [job_for(c, g, m, *b, device_bbox=(i % 5 == 0)) for i, ((c, g, m), b) in enumerate(zip(cases, bufs))]
    tuning = octree_api.OcpiBatchTuning(waveSize=6, clusterCap=2, weightedClusterCap=8, useGraphs=graphs, lanes=lanes)
    results = octree_api.batch_build_tuned(jobs, tuning)
    assert tuning.lastIssue == graphs
    for w, r, b in zip(want, results, bufs):
        check_same(w, r, *b)


def test_autotune_chooses_and_caches(tmp_path):
    """ocpi_batch_autotune measures a sweep on a sample of the batch and
    returns a valid choice; the choice is kept for the batch's signature (a
    second call measures nothing) and written to the cache file, and a batch
    built with wave size 0 uses it and equals its builds alone."""
    cases = mixed_cases(10)
    want = [alone(c, g, m) for c, g, m in cases]
    bufs = [buffers(w) for w in want]
    jobs = [job_for(c, g, m, *b) for (c, g, m), b in zip(cases, bufs)]
    cache = tmp_path / "tuning.txt"
    t = octree_api.batch_autotune(jobs, sample_jobs=10, cache_path=str(cache))
    assert t.trials >= 5 and t.trialMs > 0
    assert 1 <= t.waveSize <= 10 and t.clusterCap in (2, 4, 8) and t.weightedClusterCap in (8, 16)
    assert t.lanes in (0, 4)
    again = octree_api.batch_autotune(jobs, sample_jobs=10, cache_path=str(cache))
    assert again.as_dict() == t.as_dict()
    line = cache.read_text().split()
    assert int(line[1]) == t.waveSize and int(line[4]) == t.useGraphs and int(line[7]) == t.lanes
    results = octree_api.batch_build_wave(jobs, wave_size=0)
    for w, r, b in zip(want, results, bufs):
        check_same(w, r, *b)


def test_wave_with_a_failing_job():
    """A job whose box leaves points below it fails in its wave; the wave's
    other builds do not wait for it and equal their builds alone."""
    cases = [(c, g, 0) for c, g, _ in mixed_cases(6)]
    want = [alone(c, g, m) for c, g, m in cases]
    bufs = [buffers(w) for w in want]
    jobs = [job_for(c, g, m, *b) for (c, g, m), b in zip(cases, bufs)]
    bad, g, m = cases[2]
    shift = (bad.bb_max[0] - bad.bb_min[0]) / 4
    jobs[2] = octree_api.make_job(bad.cloud, n=bad.n, stride=bad.stride, cloud_type=bad.cloud_type, scale=bad.scale,
                                  bb_min=[v + shift for v in bad.bb_min], bb_max=[v + shift for v in bad.bb_max],
                                  chunk_grid=g[0], sub_grid=g[1], merge_threshold=2000, flags=FLAGS[m], seed=99)
    results = octree_api.batch_build_wave(jobs, wave_size=8)
    assert results[2].status == -1 and b"below the bounding box" in results[2].error
    for i, (w, r, b) in enumerate(zip(want, results, bufs)):
        if i != 2:
            check_same(w, r, *b)


def test_server_admission_under_a_small_budget():
    """A budget that holds about two builds at a time: jobs queue, every one
    completes, results equal the builds alone; an oversized job is refused."""
    cases = mixed_cases(8)
    bounds = [octree_api.estimate_memory(c.n, c.stride, c.cloud_type, g[0], 2000, 2.2, g[1], FLAGS[m])[0]
              for c, g, m in cases]
    budget = int(2.2 * max(bounds))
    want = [alone(c, g, m) for c, g, m in cases]
    srv = octree_api.Server(lanes=4, memory_budget=budget)
    bufs = [buffers(w) for w in want]
    tickets = [srv.submit(job_for(c, g, m, *b)) for (c, g, m), b in zip(cases, bufs)]
    results = [srv.wait(t) for t in tickets]
    for w, r, b in zip(want, results, bufs):
        check_same(w, r, *b)
    assert max(r.queuedMs for r in results) > 0
    big = make_case(0, 0, 2_000_000, seed=5)
    with pytest.raises(octree_api.OctreeError, match="budget"):
        srv.submit(job_for(big, (512, 128), 0, None, None, None))
    srv.close()


def test_failed_job_leaves_the_batch_intact():
    """One job whose box leaves points below it fails with the device's
    error; the other jobs of the batch still equal their builds alone."""
    cases = mixed_cases(6)
    want = [alone(c, g, m) for c, g, m in cases]
    bufs = [buffers(w) for w in want]
    jobs = [job_for(c, g, m, *b) for (c, g, m), b in zip(cases, bufs)]
    bad, g, m = cases[2]
    shift = (bad.bb_max[0] - bad.bb_min[0]) / 4
    jobs[2] = octree_api.make_job(bad.cloud, n=bad.n, stride=bad.stride, cloud_type=bad.cloud_type, scale=bad.scale,
                                  bb_min=[v + shift for v in bad.bb_min], bb_max=[v + shift for v in bad.bb_max],
                                  chunk_grid=g[0], sub_grid=g[1], merge_threshold=2000, flags=FLAGS[m], seed=99)
    results = octree_api.batch_build(jobs, lanes=3)
    assert results[2].status == -1 and b"below the bounding box" in results[2].error
    for i, (w, r, b) in enumerate(zip(want, results, bufs)):
        if i != 2:
            check_same(w, r, *b)


def test_batch_refuses_an_invalid_job_before_starting_any():
    cases = mixed_cases(3)
    want = [alone(c, g, m) for c, g, m in cases]
    bufs = [buffers(w) for w in want]
    jobs = [job_for(c, g, m, *b) for (c, g, m), b in zip(cases, bufs)]
    jobs[1].chunkingGrid = 96   # not a power of two
    with pytest.raises(octree_api.OctreeError, match="job 1 of the batch"):
        octree_api.batch_build(jobs, lanes=2)
    assert all(not np.any(b[0]) for b in bufs), "a job ran although the batch was refused"


def test_server_reuses_resident_cloud_state():
    """Jobs naming the same cloud (cloudId) and chunking settings rerun only
    subsampling on the lane's resident state; every result still equals the
    build run alone, and state is not reused across clouds, chunking grids or
    an explicit / device-computed bounding box."""
    a = make_case(0, 0, 300_000, seed=41)
    b = make_case(1, 1, 200_000, seed=42)
    steps = [   # case, grids, mode, cloud id, device box, expected reuse
        (a, (128, 64), 0, 1, False, 0),
        (a, (128, 64), 1, 1, False, 1),
        (a, (128, 64), 2, 1, False, 1),
        (a, (64, 32), 0, 1, False, 0),
        (a, (64, 16), 3, 1, False, 1),
        (b, (128, 64), 0, 2, False, 0),
        (a, (128, 64), 0, 1, False, 0),
        (a, (128, 64), 1, 1, True, 0),
        (a, (128, 64), 2, 1, True, 1),
        (a, (128, 64), 0, 0, False, 0),
    ]
    srv = octree_api.Server(lanes=1, memory_budget=64 << 30)
    for case, grids, m, cid, dev, expect in steps:
        want = alone(case, grids, m)
        buf = buffers(want)
        t = srv.submit(job_for(case, grids, m, *buf, device_bbox=dev, cloud_id=cid))
        r = srv.wait(t)
        srv.release(t)
        check_same(want, r, *buf)
        assert r.reused == expect, (grids, m, cid, dev)
    srv.close()


def test_injected_allocation_failure_fails_one_job_only():
    case = make_case(0, 0, 200_000, seed=61)
    want = alone(case, (128, 64), 0)
    srv = octree_api.Server(lanes=1, memory_budget=64 << 30)
    try:
        octree_api.inject_failures(octree_api.INJECT_ALLOCATION, 1)
        buf = buffers(want)
        t = srv.submit(job_for(case, (128, 64), 0, *buf))
        r = srv.wait(t)
        srv.release(t)
        assert r.status == -1 and b"injected allocation failure" in r.error
        buf = buffers(want)
        t = srv.submit(job_for(case, (128, 64), 0, *buf))
        r = srv.wait(t)
        srv.release(t)
        check_same(want, r, *buf)
    finally:
        octree_api.inject_failures(octree_api.INJECT_ALLOCATION, 0)
        srv.close()


def test_injected_allocation_failure_in_a_session():
    """A session whose reconfiguration fails part-way drops its builder; the
    next ocpi_init_octree starts over and the build is correct."""
    a = make_case(0, 0, 150_000, seed=62)
    b = make_case(1, 0, 400_000, seed=63)
    want = alone(b, (128, 64), 0)
    s = octree_api.OctreeSession(0)
    try:
        cfg = dict(chunk_grid=64, sub_grid=32, merge_threshold=2000, seed=99, **MODES[0])
        s.set_cloud(a.cloud, n=a.n, stride=a.stride, cloud_type=a.cloud_type, scale=a.scale, bb_min=a.bb_min,
                    bb_max=a.bb_max)
        s.configure(**cfg)
        s.init()
        s.generate()
        # a larger cloud and grid: the buffers must grow, and the first growth fails
        cfg = dict(chunk_grid=128, sub_grid=64, merge_threshold=2000, seed=99, **MODES[0])
        s.set_cloud(b.cloud, n=b.n, stride=b.stride, cloud_type=b.cloud_type, scale=b.scale, bb_min=b.bb_min,
                    bb_max=b.bb_max)
        s.configure(**cfg)
        octree_api.inject_failures(octree_api.INJECT_ALLOCATION, 1)
        with pytest.raises(octree_api.OctreeError, match="injected allocation failure"):
            s.init()
        s.init()
        s.generate()
        a_r, a_l = node_sorted(want[0], want[1], want[2])
        h = s.hierarchy()
        assert h.tobytes() == want[0].tobytes()
        b_r, b_l = node_sorted(h, s.records(), s.lut())
        assert np.array_equal(a_l, b_l) and a_r.tobytes() == b_r.tobytes()
    finally:
        octree_api.inject_failures(octree_api.INJECT_ALLOCATION, 0)
        s.close()


def test_lane_restarts_after_losing_its_worker():
    case = make_case(2, 1, 200_000, seed=64)
    want = alone(case, (128, 64), 0)
    srv = octree_api.Server(lanes=2, memory_budget=64 << 30)
    try:
        octree_api.inject_failures(octree_api.INJECT_LANE_LOSS, 1)
        buf = buffers(want)
        t = srv.submit(job_for(case, (128, 64), 0, *buf))
        r = srv.wait(t)
        srv.release(t)
        assert r.status == -1 and b"worker lost" in r.error
        assert srv.lane_restarts() == 1
        results = []
        for _ in range(4):   # both lanes serve again
            buf = buffers(want)
            t = srv.submit(job_for(case, (128, 64), 0, *buf))
            results.append((srv.wait(t), buf))
            srv.release(t)
        for r, buf in results:
            check_same(want, r, *buf)
    finally:
        octree_api.inject_failures(octree_api.INJECT_LANE_LOSS, 0)
        srv.close()


def test_cancel_a_waiting_job():
    """A budget that holds one job at a time: the second job waits behind the
    first and can be cancelled; the running one cannot."""
    big = make_case(0, 0, 3_000_000, seed=65)
    small = make_case(1, 0, 100_000, seed=66)
    want_big = alone(big, (128, 64), 0)
    bound = octree_api.estimate_memory(big.n, big.stride, big.cloud_type, 128, 2000, 2.2, 64, FLAGS[0])[0]
    srv = octree_api.Server(lanes=2, memory_budget=int(bound * 1.05))
    try:
        buf = buffers(want_big)
        t1 = srv.submit(job_for(big, (128, 64), 0, *buf))
        t2 = srv.submit(job_for(small, (128, 64), 0, None, None, None))
        srv.cancel(t2)
        r2 = srv.wait(t2)
        assert r2.status == -1 and r2.error == b"cancelled"
        with pytest.raises(octree_api.OctreeError, match="completed"):
            srv.cancel(t2)
        r1 = srv.wait(t1)
        check_same(want_big, r1, *buf)
        with pytest.raises(octree_api.OctreeError, match="completed"):
            srv.cancel(t1)
    finally:
        srv.close()


def test_backlog_on_one_lane_with_held_jobs():
    """One lane and a backlog: while a build runs, the lane holds the next job
    and copies its cloud ahead.  Jobs share clouds in turn (each job's cloud
    differs from the one before it), one waiting job is cancelled whether it
    is held or still queued, and every other result equals its build alone."""
    cases = [make_case(k % 3, k % 2, n, seed=80 + k) for k, n in enumerate((900_000, 300_000, 150_000, 250_000))]
    order = [0, 1, 2, 3, 1, 0, 2, 1]
    want = {k: alone(cases[k], (128, 64), 2 * (k % 2)) for k in set(order)}
    srv = octree_api.Server(lanes=1, memory_budget=64 << 30)
    try:
        bufs = [buffers(want[k]) for k in order]
        tickets = [srv.submit(job_for(cases[k], (128, 64), 2 * (k % 2), *b)) for k, b in zip(order, bufs)]
        srv.cancel(tickets[2])
        for i, (k, t) in enumerate(zip(order, tickets)):
            r = srv.wait(t)
            if i == 2:
                assert r.status == -1 and r.error == b"cancelled"
            else:
                check_same(want[k], r, *bufs[i])
            srv.release(t)
    finally:
        srv.close()


def test_session_sparse_builds_after_a_dense_build_on_other_grids():
    """One session through a dense build on a 64 grid, a sparse build on a
    32 grid, then a sparse build on the 64 grid (the first grid's finest
    level must be clean again): every build equals the same build on a new
    session."""
    steps = [(make_case(0, 0, 100_000, seed=71), (64, 32)),   # dense: 100k points > 64^3 / 16
             (make_case(1, 0, 1_500, seed=72), (32, 16)),      # sparse on the smaller grid
             (make_case(2, 1, 10_000, seed=73), (64, 32))]     # sparse on the larger grid
    s = octree_api.OctreeSession(0)
    try:
        for case, grids in steps:
            want = alone(case, grids, 0)
            s.set_cloud(case.cloud, n=case.n, stride=case.stride, cloud_type=case.cloud_type, scale=case.scale,
                        bb_min=case.bb_min, bb_max=case.bb_max)
            s.configure(chunk_grid=grids[0], sub_grid=grids[1], merge_threshold=2000, seed=99, **MODES[0])
            s.init()
            s.generate()
            h = s.hierarchy()
            assert h.tobytes() == want[0].tobytes(), grids
            a_r, a_l = node_sorted(want[0], want[1], want[2])
            b_r, b_l = node_sorted(h, s.records(), s.lut())
            assert np.array_equal(a_l, b_l) and a_r.tobytes() == b_r.tobytes()
    finally:
        s.close()


def test_session_random_sequence_equals_fresh_builds():
    """Twelve builds on one session, seeded at random: grids 32 to 128, point
    amounts on both sides of the sparse-pyramid threshold (one point per 16
    finest cells), all four subsampling modes.  Every build equals the same
    build on a fresh session, whatever state the previous build left."""
    rng = np.random.default_rng(2026)
    s = octree_api.OctreeSession(0)
    try:
        for step in range(12):
            g0 = int(rng.choice([32, 64, 128]))
            g1 = int(rng.choice([16, 32])) if g0 > 32 else 16
            cells = g0 ** 3
            n = int(cells // 16 * rng.choice([0.3, 0.9, 1.5, 6.0]))
            n = max(n, 2500)
            m = int(rng.integers(0, len(MODES)))
            case = make_case(int(rng.integers(0, 3)), int(rng.integers(0, 2)), n, seed=500 + step)
            want = alone(case, (g0, g1), m)
            s.set_cloud(case.cloud, n=case.n, stride=case.stride, cloud_type=case.cloud_type, scale=case.scale,
                        bb_min=case.bb_min, bb_max=case.bb_max)
            s.configure(chunk_grid=g0, sub_grid=g1, merge_threshold=2000, seed=99, **MODES[m])
            s.init()
            s.generate()
            h = s.hierarchy()
            assert h.tobytes() == want[0].tobytes(), (step, g0, n, m)
            a_r, a_l = node_sorted(want[0], want[1], want[2])
            b_r, b_l = node_sorted(h, s.records(), s.lut())
            assert np.array_equal(a_l, b_l) and a_r.tobytes() == b_r.tobytes(), (step, g0, n, m)
    finally:
        s.close()
