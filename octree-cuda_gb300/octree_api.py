"""Python binding of libOctreeApi.so (ctypes over the C ABI in include/octreeApi.h).

The session object mirrors the reference's OctreeApi call sequence
(src/main.cpp:83-107 of PotreeConverterGPU): create a session, describe the
cloud, configure chunking and subsampling, init (upload), generate, export.
Every call raises OctreeError when the C entry point returns -1.

Loading fails loudly when the native library is missing: there is no Python or
CPU fallback for any stage.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libOctreeApi.so")
SYNTH_PATH = os.path.join(HERE, "libocsynth.so")

# The 18 entry points of the reference API (OctreeApi/include/octreeApi.h:42-72).
REFERENCE_SYMBOLS = [
    "ocpi_create_session", "ocpi_destroy_session", "ocpi_set_logging_level",
    "ocpi_set_cloud_type", "ocpi_set_cloud_point_amount", "ocpi_set_cloud_data_stride",
    "ocpi_set_cloud_scale", "ocpi_set_cloud_offset", "ocpi_set_cloud_bb",
    "ocpi_set_point_cloud_host", "ocpi_configure_chunking", "ocpi_configure_subsampling",
    "ocpi_export_memory_report", "ocpi_export_distribution_histogram", "ocpi_export_json_report",
    "ocpi_export_potree", "ocpi_init_octree", "ocpi_generate_octree",
]
ADDED_SYMBOLS = [
    "ocpi_last_error", "ocpi_set_random_seed", "ocpi_set_debug_flags", "ocpi_get_stats",
    "ocpi_get_node_count", "ocpi_get_hierarchy", "ocpi_get_records", "ocpi_get_lut",
    "ocpi_get_level_counts", "ocpi_get_timings", "ocpi_subsample_node_noalloc", "ocpi_set_output_host",
    "ocpi_compute_cloud_bb", "ocpi_get_device_memory", "ocpi_estimate_memory",
    "ocpi_server_create", "ocpi_server_destroy", "ocpi_server_submit", "ocpi_server_wait",
    "ocpi_server_get_hierarchy", "ocpi_server_release", "ocpi_batch_build", "ocpi_batch_build_wave",
    "ocpi_server_cancel",
    "ocpi_server_lane_restarts", "ocpi_debug_inject_failures", "ocpi_batch_autotune", "ocpi_batch_build_tuned",
]

HIER_DTYPE = np.dtype([("type", "u1"), ("mask", "u1"), ("points", "<u4"),
                       ("byte_offset", "<u8"), ("byte_size", "<u8")])
RECORD_DTYPE = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4"),
                         ("r", "<u2"), ("g", "<u2"), ("b", "<u2")])


# ocpi_subsample_node_noalloc: mode bits and the fixed scratch limit
SUB_INTRA, SUB_INTER, SUB_RANDOM, SUB_WEIGHTING = 1, 2, 8, 16
NOALLOC_MAX_CANDIDATES = 131072


class OctreeError(RuntimeError):
    pass


class OcpiStats(ctypes.Structure):
    _fields_ = [
        ("points_total", ctypes.c_uint64), ("p_out", ctypes.c_uint64), ("p_in", ctypes.c_uint64),
        ("out_capacity", ctypes.c_uint64), ("depth", ctypes.c_uint32), ("tree_nodes", ctypes.c_uint32),
        ("leaf_nodes", ctypes.c_uint32), ("internal_nodes", ctypes.c_uint32), ("sparse_nodes", ctypes.c_uint32),
        ("dense_nodes", ctypes.c_uint32), ("max_leaf_depth", ctypes.c_uint32), ("min_leaf_points", ctypes.c_uint32),
        ("max_leaf_points", ctypes.c_uint32), ("mean_leaf_points", ctypes.c_float),
        ("stdev_leaf_points", ctypes.c_float), ("kernel_launches", ctypes.c_uint32),
        ("subsample_passes", ctypes.c_uint32),
    ]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "reserved"}


class OcpiJob(ctypes.Structure):
    _fields_ = [
        ("cloud", ctypes.c_void_p), ("pointAmount", ctypes.c_uint32), ("dataStride", ctypes.c_uint32),
        ("cloudType", ctypes.c_uint8), ("scale", ctypes.c_double * 3), ("bbMin", ctypes.c_double * 3),
        ("bbMax", ctypes.c_double * 3), ("chunkingGrid", ctypes.c_uint32), ("mergingThreshold", ctypes.c_uint32),
        ("outputFactor", ctypes.c_float), ("subsamplingGrid", ctypes.c_uint32), ("modeFlags", ctypes.c_uint32),
        ("seed", ctypes.c_uint64), ("outRecords", ctypes.c_void_p), ("outLut", ctypes.c_void_p),
        ("outCapacity", ctypes.c_uint64), ("outHierarchy", ctypes.c_void_p), ("outHierarchyCapacity", ctypes.c_uint64),
        ("cloudId", ctypes.c_uint64),
    ]


class OcpiJobResult(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int32), ("lane", ctypes.c_uint32), ("nodeCount", ctypes.c_uint32),
        ("reused", ctypes.c_uint32), ("pointsTotal", ctypes.c_uint64), ("queuedMs", ctypes.c_double), ("runMs", ctypes.c_double),
        ("totalMs", ctypes.c_double), ("deviceMs", ctypes.c_double), ("error", ctypes.c_char * 128),
        ("subsamplePasses", ctypes.c_uint32),
    ]


class OcpiBatchTuning(ctypes.Structure):
    _fields_ = [
        ("waveSize", ctypes.c_uint32), ("clusterCap", ctypes.c_uint32), ("weightedClusterCap", ctypes.c_uint32),
        ("useGraphs", ctypes.c_uint32), ("trialMs", ctypes.c_double), ("trials", ctypes.c_uint32),
        ("lastIssue", ctypes.c_uint32), ("lanes", ctypes.c_uint32),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None
_synth = None


def load_library(path=LIB_PATH):
    """Load libOctreeApi.so and declare the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OctreeError("libOctreeApi.so not built (run __graft_entry__.build()): %s" % path)
    L = ctypes.CDLL(path)
    vp, u8, u32, u64, d, b = (ctypes.c_void_p, ctypes.c_uint8, ctypes.c_uint32, ctypes.c_uint64,
                              ctypes.c_double, ctypes.c_bool)
    sig = {
        "ocpi_create_session": [ctypes.POINTER(vp), ctypes.c_int],
        "ocpi_destroy_session": [vp],
        "ocpi_set_logging_level": [ctypes.c_int],
        "ocpi_set_cloud_type": [vp, u8],
        "ocpi_set_cloud_point_amount": [vp, u32],
        "ocpi_set_cloud_data_stride": [vp, u32],
        "ocpi_set_cloud_scale": [vp, d, d, d],
        "ocpi_set_cloud_offset": [vp, d, d, d],
        "ocpi_set_cloud_bb": [vp, d, d, d, d, d, d],
        "ocpi_set_point_cloud_host": [vp, vp],
        "ocpi_configure_chunking": [vp, u32, u32, ctypes.c_float],
        "ocpi_configure_subsampling": [vp, u32, b, b, b, b, b],
        "ocpi_export_memory_report": [vp, ctypes.c_char_p],
        "ocpi_export_distribution_histogram": [vp, ctypes.c_char_p, u32],
        "ocpi_export_json_report": [vp, ctypes.c_char_p],
        "ocpi_export_potree": [vp, ctypes.c_char_p],
        "ocpi_init_octree": [vp],
        "ocpi_generate_octree": [vp],
        "ocpi_set_random_seed": [vp, u64],
        "ocpi_set_debug_flags": [vp, u32],
        "ocpi_get_stats": [vp, ctypes.POINTER(OcpiStats)],
        "ocpi_get_node_count": [vp, ctypes.POINTER(u64)],
        "ocpi_get_hierarchy": [vp, vp],
        "ocpi_get_records": [vp, vp],
        "ocpi_get_lut": [vp, vp],
        "ocpi_get_level_counts": [vp, u32, vp],
        "ocpi_get_timings": [vp, ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_char_p, ctypes.c_int,
                             ctypes.POINTER(ctypes.c_int)],
        "ocpi_set_output_host": [vp, vp, vp, u64],
        "ocpi_compute_cloud_bb": [vp, vp, vp],
        "ocpi_get_device_memory": [vp, ctypes.POINTER(u64)],
        "ocpi_server_create": [ctypes.POINTER(vp), ctypes.c_int, u32, u64],
        "ocpi_server_destroy": [vp],
        "ocpi_server_submit": [vp, ctypes.POINTER(OcpiJob), ctypes.POINTER(u64)],
        "ocpi_server_wait": [vp, u64, ctypes.POINTER(OcpiJobResult)],
        "ocpi_server_get_hierarchy": [vp, u64, vp],
        "ocpi_server_release": [vp, u64],
        "ocpi_server_cancel": [vp, u64],
        "ocpi_server_lane_restarts": [vp, ctypes.POINTER(u64)],
        "ocpi_debug_inject_failures": [ctypes.c_int, u32],
        "ocpi_batch_build": [ctypes.c_int, u32, u64, ctypes.POINTER(OcpiJob), u32, ctypes.POINTER(OcpiJobResult)],
        "ocpi_batch_build_wave": [ctypes.c_int, u32, u64, ctypes.POINTER(OcpiJob), u32, ctypes.POINTER(OcpiJobResult)],
        "ocpi_batch_autotune": [ctypes.c_int, u64, ctypes.POINTER(OcpiJob), u32, u32, ctypes.c_char_p,
                                ctypes.POINTER(OcpiBatchTuning)],
        "ocpi_batch_build_tuned": [ctypes.c_int, u64, ctypes.POINTER(OcpiBatchTuning), ctypes.POINTER(OcpiJob), u32,
                                   ctypes.POINTER(OcpiJobResult)],
        "ocpi_estimate_memory": [u32, u32, u8, u32, u32, ctypes.c_float, u32, u32, ctypes.POINTER(u64),
                                 ctypes.POINTER(u64)],
        "ocpi_subsample_node_noalloc": [vp, u8, u32, ctypes.POINTER(d), ctypes.POINTER(d), ctypes.POINTER(d), d,
                                        u32, u64, u32, u32, u64, vp, vp, u32, vp, vp, vp, vp],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.ocpi_last_error.restype = ctypes.c_char_p
    L.ocpi_last_error.argtypes = []
    _lib = L
    return L


def load_synthetic(path=SYNTH_PATH):
    global _synth
    if _synth is None:
        if not os.path.exists(path):
            raise OctreeError("libocsynth.so not built: %s" % path)
        S = ctypes.CDLL(path)
        S.ocsynth_generate.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32,
                                       ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int]
        S.ocsynth_generate.restype = ctypes.c_int
        S.ocsynth_cubic_bbox.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_int]
        S.ocsynth_cubic_bbox.restype = None
        _synth = S
    return _synth


def estimate_memory(n, stride, cloud_type, chunk_grid=512, merge_threshold=10000, output_factor=2.2, sub_grid=128,
                    flags=0):
    """(upper bound of this library's device bytes, the reference's estimate)."""
    a, b = ctypes.c_uint64(), ctypes.c_uint64()
    _check(load_library().ocpi_estimate_memory(n, stride, cloud_type, chunk_grid, merge_threshold, output_factor,
                                               sub_grid, flags, ctypes.byref(a), ctypes.byref(b)),
           "ocpi_estimate_memory")
    return a.value, b.value


def _check(rc, what):
    if rc != 0:
        msg = load_library().ocpi_last_error().decode(errors="replace")
        raise OctreeError("%s failed: %s" % (what, msg))


def synthetic_cloud(kind, cloud_type, n, seed, stride=None, threads=None):
    """Seeded synthetic cloud as a numpy uint8 buffer (kinds: 0 heightfield+boxes,
    1 planes+cylinders, 2 Zipf terrain, 3 unit cuboid)."""
    stride = stride or (15 if cloud_type == 0 else 27)
    buf = np.empty(n * stride + 64, np.uint8)
    rc = load_synthetic().ocsynth_generate(kind, cloud_type, n, stride, seed, buf.ctypes.data,
                                           threads or os.cpu_count() or 1)
    if rc != 0:
        raise OctreeError("synthetic generation failed")
    return buf[: n * stride]


def cubic_bbox(cloud, n, stride, cloud_type, threads=None):
    """The CLI's cubic bounding box (src/boundingbox.h:11-52)."""
    out = np.zeros(6, np.float64)
    buf = np.ascontiguousarray(cloud)
    load_synthetic().ocsynth_cubic_bbox(buf.ctypes.data, n, stride, cloud_type, out.ctypes.data,
                                        threads or os.cpu_count() or 1)
    return out


class OctreeSession:
    """One OctreeApi session on one GPU."""

    def __init__(self, device=0):
        L = load_library()
        h = ctypes.c_void_p()
        _check(L.ocpi_create_session(ctypes.byref(h), device), "ocpi_create_session")
        self._h = h
        self._cloud = None

    def close(self):
        if self._h:
            load_library().ocpi_destroy_session(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- reference call sequence
    def set_cloud(self, cloud, *, n, stride, cloud_type, scale, bb_min=None, bb_max=None, offset=None):
        """bb_min / bb_max None: compute the box on the device after init()
        (compute_cloud_bb)."""
        L = load_library()
        h = self._h
        _check(L.ocpi_set_cloud_type(h, cloud_type), "ocpi_set_cloud_type")
        _check(L.ocpi_set_cloud_point_amount(h, n), "ocpi_set_cloud_point_amount")
        _check(L.ocpi_set_cloud_data_stride(h, stride), "ocpi_set_cloud_data_stride")
        _check(L.ocpi_set_cloud_scale(h, *map(float, scale)), "ocpi_set_cloud_scale")
        off = offset if offset is not None else (bb_min if bb_min is not None else (0.0, 0.0, 0.0))
        _check(L.ocpi_set_cloud_offset(h, *map(float, off)), "ocpi_set_cloud_offset")
        if bb_min is not None:
            _check(L.ocpi_set_cloud_bb(h, *map(float, bb_min), *map(float, bb_max)), "ocpi_set_cloud_bb")
        self._cloud = np.ascontiguousarray(cloud)
        _check(L.ocpi_set_point_cloud_host(h, self._cloud.ctypes.data), "ocpi_set_point_cloud_host")

    def configure(self, *, chunk_grid=512, merge_threshold=10000, output_factor=2.2, sub_grid=128, intra=False,
                  inter=False, replacement=True, random=False, weighting=False, seed=None, debug=0):
        L = load_library()
        h = self._h
        _check(L.ocpi_configure_chunking(h, chunk_grid, merge_threshold, output_factor), "ocpi_configure_chunking")
        _check(L.ocpi_configure_subsampling(h, sub_grid, intra, inter, replacement, random, weighting),
               "ocpi_configure_subsampling")
        if seed is not None:
            _check(L.ocpi_set_random_seed(h, seed), "ocpi_set_random_seed")
        _check(L.ocpi_set_debug_flags(h, debug), "ocpi_set_debug_flags")

    def set_output_host(self, records, lut=None):
        """Arrays (uint8 of 18-byte records, optional uint32 LUT) that every
        generate fills; keep them alive (and preferably pinned)."""
        cap = len(records) // 18
        self._out = (records, lut)
        _check(load_library().ocpi_set_output_host(self._h, records.ctypes.data,
                                                   lut.ctypes.data if lut is not None else None, cap),
               "ocpi_set_output_host")

    def compute_cloud_bb(self):
        """(real, cubic) bounding boxes computed on the device after init();
        the cubic one becomes the session's bounding box."""
        real = np.zeros(6)
        cubic = np.zeros(6)
        _check(load_library().ocpi_compute_cloud_bb(self._h, real.ctypes.data, cubic.ctypes.data),
               "ocpi_compute_cloud_bb")
        return real, cubic

    def device_memory(self):
        v = ctypes.c_uint64()
        _check(load_library().ocpi_get_device_memory(self._h, ctypes.byref(v)), "ocpi_get_device_memory")
        return v.value

    def init(self):
        _check(load_library().ocpi_init_octree(self._h), "ocpi_init_octree")

    def generate(self):
        _check(load_library().ocpi_generate_octree(self._h), "ocpi_generate_octree")

    def export_potree(self, directory):
        _check(load_library().ocpi_export_potree(self._h, directory.encode()), "ocpi_export_potree")

    def export_json_report(self, filename):
        _check(load_library().ocpi_export_json_report(self._h, filename.encode()), "ocpi_export_json_report")

    def export_histogram(self, filename, bin_width=0):
        _check(load_library().ocpi_export_distribution_histogram(self._h, filename.encode(), bin_width),
               "ocpi_export_distribution_histogram")

    # ---- results
    def stats(self):
        st = OcpiStats()
        _check(load_library().ocpi_get_stats(self._h, ctypes.byref(st)), "ocpi_get_stats")
        return st.as_dict()

    def hierarchy(self):
        n = ctypes.c_uint64()
        L = load_library()
        _check(L.ocpi_get_node_count(self._h, ctypes.byref(n)), "ocpi_get_node_count")
        out = np.zeros(n.value, HIER_DTYPE)
        _check(L.ocpi_get_hierarchy(self._h, out.ctypes.data), "ocpi_get_hierarchy")
        return out

    def records(self):
        total = self.stats()["points_total"]
        out = np.zeros(total, RECORD_DTYPE)
        _check(load_library().ocpi_get_records(self._h, out.ctypes.data), "ocpi_get_records")
        return out

    def lut(self):
        total = self.stats()["points_total"]
        out = np.zeros(total, np.uint32)
        _check(load_library().ocpi_get_lut(self._h, out.ctypes.data), "ocpi_get_lut")
        return out

    def level_counts(self, level, grid):
        out = np.zeros(grid ** 3, np.uint32)
        _check(load_library().ocpi_get_level_counts(self._h, level, out.ctypes.data), "ocpi_get_level_counts")
        return out

    def timings(self):
        ms = (ctypes.c_double * 64)()
        names = ctypes.create_string_buffer(4096)
        cnt = ctypes.c_int()
        _check(load_library().ocpi_get_timings(self._h, ms, 64, names, 4096, ctypes.byref(cnt)), "ocpi_get_timings")
        keys = names.value.decode().split(",") if cnt.value else []
        return {k: ms[i] for i, k in enumerate(keys)}


def build_octree(cloud, *, n, stride, cloud_type, scale, bb_min, bb_max, device=0, **cfg):
    """One-shot build; returns (session, stats).  The session holds the result."""
    s = OctreeSession(device)
    s.set_cloud(cloud, n=n, stride=stride, cloud_type=cloud_type, scale=scale, bb_min=bb_min, bb_max=bb_max)
    s.configure(**cfg)
    s.init()
    s.generate()
    return s, s.stats()


def make_job(cloud, *, n, stride, cloud_type, scale, bb_min=None, bb_max=None, chunk_grid=512, merge_threshold=10000,
             output_factor=2.2, sub_grid=128, flags=SUB_INTER, seed=0x5EED, records=None, lut=None, hierarchy=None,
             cloud_id=0):
    """OcpiJob for Server.submit / batch_build.  bb_min None: the box is
    computed on the device.  records / lut / hierarchy: optional host arrays
    the build fills (keep them, and the cloud, alive until it completes)."""
    j = OcpiJob()
    j.cloud = cloud.ctypes.data
    j.pointAmount, j.dataStride, j.cloudType = n, stride, cloud_type
    j.scale[:] = [float(v) for v in scale]
    if bb_min is not None:
        j.bbMin[:] = [float(v) for v in bb_min]
        j.bbMax[:] = [float(v) for v in bb_max]
    j.chunkingGrid, j.mergingThreshold, j.outputFactor, j.subsamplingGrid = chunk_grid, merge_threshold, output_factor, sub_grid
    j.modeFlags, j.seed, j.cloudId = flags, seed, cloud_id
    if records is not None:
        j.outRecords, j.outCapacity = records.ctypes.data, len(records) // 18
        j.outLut = lut.ctypes.data if lut is not None else None
    if hierarchy is not None:
        j.outHierarchy, j.outHierarchyCapacity = hierarchy.ctypes.data, len(hierarchy)
    return j


class Server:
    """Executor of independent builds on one GPU (ocpi_server_*)."""

    def __init__(self, device=0, lanes=4, memory_budget=150 << 30):
        L = load_library()
        h = ctypes.c_void_p()
        _check(L.ocpi_server_create(ctypes.byref(h), device, lanes, memory_budget), "ocpi_server_create")
        self._h = h

    def submit(self, job):
        t = ctypes.c_uint64()
        _check(load_library().ocpi_server_submit(self._h, ctypes.byref(job), ctypes.byref(t)), "ocpi_server_submit")
        return t.value

    def wait(self, ticket):
        r = OcpiJobResult()
        _check(load_library().ocpi_server_wait(self._h, ticket, ctypes.byref(r)), "ocpi_server_wait")
        return r

    def hierarchy(self, ticket, node_count):
        out = np.zeros(node_count, HIER_DTYPE)
        _check(load_library().ocpi_server_get_hierarchy(self._h, ticket, out.ctypes.data), "ocpi_server_get_hierarchy")
        return out

    def release(self, ticket):
        _check(load_library().ocpi_server_release(self._h, ticket), "ocpi_server_release")

    def cancel(self, ticket):
        _check(load_library().ocpi_server_cancel(self._h, ticket), "ocpi_server_cancel")

    def lane_restarts(self):
        v = ctypes.c_uint64()
        _check(load_library().ocpi_server_lane_restarts(self._h, ctypes.byref(v)), "ocpi_server_lane_restarts")
        return v.value

    def close(self):
        if self._h:
            load_library().ocpi_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


INJECT_ALLOCATION, INJECT_LANE_LOSS = 1, 2


def inject_failures(kind, count):
    """Host-side fault injection for tests: the next `count` events of a kind
    (INJECT_ALLOCATION, INJECT_LANE_LOSS) fail; 0 clears."""
    _check(load_library().ocpi_debug_inject_failures(kind, count), "ocpi_debug_inject_failures")


def batch_build(jobs, device=0, lanes=4, memory_budget=150 << 30):
    """Builds every job of a list at once; returns their OcpiJobResults
    (per-build failures are reported there, not raised)."""
    arr = (OcpiJob * len(jobs))(*jobs)
    res = (OcpiJobResult * len(jobs))()
    rc = load_library().ocpi_batch_build(device, lanes, memory_budget, arr, len(jobs), res)
    if rc != 0 and all(r.status == 0 for r in res):
        _check(rc, "ocpi_batch_build")   # rejected before any build ran
    return list(res)   # a failed build has status -1 and its message in .error


def batch_build_wave(jobs, device=0, wave_size=32, memory_budget=150 << 30):
    """batch_build in subsampling waves (ocpi_batch_build_wave): jobs of the
    same record type and mode, wave_size at a time, each subsampling level
    of a wave in one launch, a wave's subsampling in one CUDA graph.
    wave_size 0: the autotuned choice.  Returns the OcpiJobResults."""
    arr = (OcpiJob * len(jobs))(*jobs)
    res = (OcpiJobResult * len(jobs))()
    rc = load_library().ocpi_batch_build_wave(device, wave_size, memory_budget, arr, len(jobs), res)
    if rc != 0 and all(r.status == 0 for r in res):
        _check(rc, "ocpi_batch_build_wave")   # rejected before any build ran
    return list(res)


def batch_autotune(jobs, device=0, memory_budget=150 << 30, sample_jobs=0, cache_path=None):
    """ocpi_batch_autotune: the fastest tuning of the batched form for a batch
    like `jobs` (measured on a sample of it, whose outputs it writes)."""
    arr = (OcpiJob * len(jobs))(*jobs)
    t = OcpiBatchTuning()
    _check(load_library().ocpi_batch_autotune(device, memory_budget, arr, len(jobs), sample_jobs,
                                              cache_path.encode() if cache_path else None, ctypes.byref(t)),
           "ocpi_batch_autotune")
    return t


def batch_build_tuned(jobs, tuning, device=0, memory_budget=150 << 30):
    """ocpi_batch_build_tuned: the batched form with an explicit tuning
    (tuning.lastIssue tells whether the last wave ran as one graph launch).
    Returns the OcpiJobResults."""
    arr = (OcpiJob * len(jobs))(*jobs)
    res = (OcpiJobResult * len(jobs))()
    rc = load_library().ocpi_batch_build_tuned(device, memory_budget, ctypes.byref(tuning), arr, len(jobs), res)
    if rc != 0 and all(r.status == 0 for r in res):
        _check(rc, "ocpi_batch_build_tuned")
    return list(res)
