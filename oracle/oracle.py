"""ctypes binding of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py`` (its cpu_baseline leg
and its ``--impl reference`` arm) may import this module, and only as the
checker or the timed CPU baseline.  The product path never imports it.

The oracle restates the OctreeApi LOD build of PotreeConverterGPU on the CPU;
see oracle.cpp for the per-stage citations of the reference and the canonical
rules that replace the reference's races.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

F_INTRA, F_INTER, F_REPLACE, F_RANDOM, F_WEIGHT = 1, 2, 4, 8, 16
# test variants of distance weighting (oracle.cpp): the reference's float
# arithmetic propagated up the levels, per node only, and with reversed sums
F_WEIGHT_LITERAL, F_WEIGHT_LOCAL, F_WEIGHT_REVERSE = 32, 64, 128


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("scale", ctypes.c_double * 3),
        ("bb_min", ctypes.c_double * 3),
        ("bb_max", ctypes.c_double * 3),
        ("seed", ctypes.c_uint64),
        ("n", ctypes.c_uint32),
        ("stride", ctypes.c_uint32),
        ("cloud_type", ctypes.c_uint32),
        ("chunk_grid", ctypes.c_uint32),
        ("sub_grid", ctypes.c_uint32),
        ("merge_threshold", ctypes.c_uint32),
        ("output_factor", ctypes.c_float),
        ("flags", ctypes.c_uint32),
        ("threads", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
    ]


class OracleStats(ctypes.Structure):
    _fields_ = [
        ("points_total", ctypes.c_uint64),
        ("p_out", ctypes.c_uint64),
        ("p_in", ctypes.c_uint64),
        ("out_capacity", ctypes.c_uint64),
        ("depth", ctypes.c_uint32),
        ("tree_nodes", ctypes.c_uint32),
        ("leaf_nodes", ctypes.c_uint32),
        ("internal_nodes", ctypes.c_uint32),
        ("sparse_nodes", ctypes.c_uint32),
        ("dense_nodes", ctypes.c_uint32),
        ("max_leaf_depth", ctypes.c_uint32),
        ("min_leaf_points", ctypes.c_uint32),
        ("max_leaf_points", ctypes.c_uint32),
        ("mean_leaf_points", ctypes.c_float),
        ("stdev_leaf_points", ctypes.c_float),
        ("guard_truncation", ctypes.c_uint32),
        ("guard_capacity", ctypes.c_uint32),
        ("guard_color_overflow", ctypes.c_uint32),
        ("guard_root_leaf", ctypes.c_uint32),
        ("guard_div0", ctypes.c_uint32),
        ("error", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class OracleNodeInfo(ctypes.Structure):
    _fields_ = [
        ("morton", ctypes.c_uint64),
        ("data_idx", ctypes.c_uint64),
        ("level", ctypes.c_uint32),
        ("points", ctypes.c_uint32),
        ("sub_count", ctypes.c_uint32),
        ("internal", ctypes.c_uint32),
    ]


NODE_DTYPE = np.dtype([("morton", "<u8"), ("data_idx", "<u8"), ("level", "<u4"),
                       ("points", "<u4"), ("sub_count", "<u4"), ("internal", "<u4")])
HIER_DTYPE = np.dtype([("type", "u1"), ("mask", "u1"), ("points", "<u4"),
                       ("byte_offset", "<u8"), ("byte_size", "<u8")])
RECORD_DTYPE = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4"),
                         ("r", "<u2"), ("g", "<u2"), ("b", "<u2")])

_lib = None


def build_library(force=False):
    """Compile liboracle.so from oracle.cpp with the host compiler."""
    src = os.path.join(HERE, "oracle.cpp")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
           src, "-o", LIB_PATH]
    subprocess.run(cmd, check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build_library()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_build.restype = ctypes.c_void_p
        L.oracle_build.argtypes = [ctypes.c_void_p, ctypes.POINTER(OracleParams)]
        L.oracle_free.argtypes = [ctypes.c_void_p]
        L.oracle_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(OracleStats)]
        L.oracle_node_count.restype = ctypes.c_uint64
        L.oracle_node_count.argtypes = [ctypes.c_void_p]
        L.oracle_hierarchy.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_record_count.restype = ctypes.c_uint64
        L.oracle_record_count.argtypes = [ctypes.c_void_p]
        L.oracle_records.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_lut.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_nodes.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_level_size.restype = ctypes.c_uint64
        L.oracle_level_size.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        L.oracle_level_counts.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
        L.oracle_cell_axis.restype = ctypes.c_int64
        L.oracle_cell_axis.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_uint32]
        L.oracle_out_coord.restype = ctypes.c_int32
        L.oracle_out_coord.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.oracle_rp_priority.restype = ctypes.c_uint32
        L.oracle_rp_priority.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32]
        L.oracle_weight_q.restype = ctypes.c_uint32
        L.oracle_weight_q.argtypes = [ctypes.c_float] * 3 + [ctypes.c_int32] * 3
        L.oracle_exp_neg.restype = ctypes.c_float
        L.oracle_exp_neg.argtypes = [ctypes.c_float]
        _lib = L
    return _lib


class OracleResult:
    """Everything the oracle built, copied into numpy arrays."""

    def __init__(self, handle):
        L = lib()
        st = OracleStats()
        L.oracle_stats(handle, ctypes.byref(st))
        self.stats = st.as_dict()
        n_nodes = L.oracle_node_count(handle)
        self.hierarchy = np.zeros(n_nodes, HIER_DTYPE)
        self.nodes = np.zeros(n_nodes, NODE_DTYPE)
        n_rec = L.oracle_record_count(handle)
        self.records = np.zeros(n_rec, RECORD_DTYPE)
        self.lut = np.zeros(n_rec, np.uint32)
        if self.stats["error"] == 0:
            L.oracle_hierarchy(handle, self.hierarchy.ctypes.data)
            L.oracle_nodes(handle, self.nodes.ctypes.data)
            L.oracle_records(handle, self.records.ctypes.data)
            L.oracle_lut(handle, self.lut.ctypes.data)
        self.depth = self.stats["depth"]
        self.level_counts = []
        if self.stats["error"] == 0:
            for lvl in range(self.depth + 1):
                size = L.oracle_level_size(handle, lvl)
                arr = np.zeros(size, np.uint32)
                if size:
                    L.oracle_level_counts(handle, lvl, arr.ctypes.data)
                self.level_counts.append(arr)


def run(cloud, *, n, stride, cloud_type, scale, bb_min, bb_max, chunk_grid=512, sub_grid=128,
        merge_threshold=10000, output_factor=2.2, flags=0, seed=0x5EED, threads=None,
        keep_levels=True):
    """Build the LOD octree of `cloud` (a bytes-like/numpy uint8 buffer) on the CPU."""
    L = lib()
    p = OracleParams()
    p.scale[:] = list(scale)
    p.bb_min[:] = list(bb_min)
    p.bb_max[:] = list(bb_max)
    p.seed = seed
    p.n = n
    p.stride = stride
    p.cloud_type = cloud_type
    p.chunk_grid = chunk_grid
    p.sub_grid = sub_grid
    p.merge_threshold = merge_threshold
    p.output_factor = output_factor
    p.flags = flags
    p.threads = threads or os.cpu_count() or 1
    buf = np.ascontiguousarray(np.frombuffer(cloud, dtype=np.uint8))
    h = L.oracle_build(buf.ctypes.data, ctypes.byref(p))
    try:
        res = OracleResult(h)
    finally:
        L.oracle_free(h)
    if not keep_levels:
        res.level_counts = []
    return res


def cell_axis(p, mn, size, grid):
    return lib().oracle_cell_axis(p, mn, size, grid)


def out_coord(p, mn, scale):
    return lib().oracle_out_coord(p, mn, scale)
