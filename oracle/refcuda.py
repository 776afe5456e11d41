"""The reference's own CUDA pipeline as a subprocess -- TEST INFRASTRUCTURE ONLY.

Only tests/ and bench.py's reference arm use this module.  It runs
oracle/_ref/ref_runner (built by oracle/build_ref.py from the reference's
unmodified sources) on a cloud written to a temporary file, and reads back the
runner's timings and, when asked, the reference's Potree export.

The runner is a separate process, so the reference's process-global state
(trackers, spdlog, cudaDeviceScheduleBlockingSync) and its exit() on a CUDA
error never touch the caller.
"""
import json
import os
import subprocess
import tempfile

import numpy as np

import build_ref

HIER_DTYPE = np.dtype([("type", "u1"), ("mask", "u1"), ("points", "<u4"), ("byte_offset", "<u8"),
                       ("byte_size", "<u8")])
REC_DTYPE = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4"), ("r", "<u2"), ("g", "<u2"), ("b", "<u2")])


def available():
    """True when the reference runner is built."""
    return build_ref.runner() is not None


def guards_ok(stats):
    """The reference-bug guards of the parity contract, from an oracle or
    product build's statistics: the reference run is meaningful (and safe:
    no output-buffer overflow) only when none of them trips.

    - guard_capacity: N + P_out exceeds outputFactor * N records; the
      reference would write past its output buffers
      (octree_processor_impl.cu:24-31, kernel_helpers.cuh:55-59);
    - guard_truncation: a child holds more points than the reference's launch
      extent (max leaf points * 8, fp_subsampling.cuh:317-330) and would be cut;
    - guard_root_leaf: N below the merge threshold; the reference's
      distribution reads an unset parent (hierarchical_merging.cuh:80-85).
    """
    return not (stats.get("guard_capacity") or stats.get("guard_truncation") or stats.get("guard_root_leaf"))


def run(cloud, n, stride, cloud_type, scale, chunk_grid=512, sub_grid=128, merge_threshold=10000,
        output_factor=2.2, intra=False, inter=False, replacement=True, random=False, weighting=False,
        reps=1, export=True, report=False, workdir=None, timeout=1800, pageable=False):
    """Build `cloud` with the reference.  Returns a dict with the runner's JSON
    (rc, bb, init_ms, generate_ms, export_ms) and, with export=True, the parsed
    Potree files: 'hierarchy' (HIER_DTYPE), 'octree' (raw bytes) and
    'metadata' (dict).  report=True adds 'statistics' (the parsed
    statistics.json).

    The reference's distribution histogram is not run: histogram.cu:58-63
    sizes its bins so that the largest leaf falls one bin past the end of the
    vector it increments, a write out of bounds on the host."""
    exe = build_ref.runner()
    if exe is None:
        raise RuntimeError("reference runner not built (oracle/build_ref.py)")
    if intra and weighting:
        raise ValueError("intra-cell averaging with weighting dereferences an unallocated grid in the reference")
    own = workdir is None
    tmp = tempfile.mkdtemp(prefix="ocref_") if own else workdir
    try:
        path = os.path.join(tmp, "cloud.bin")
        np.ascontiguousarray(cloud, dtype=np.uint8)[: n * stride].tofile(path)
        out = os.path.join(tmp, "potree")
        os.makedirs(out, exist_ok=True)
        cmd = [exe, "--cloud", path, "--points", str(n), "--stride", str(stride),
               "--type", "double" if cloud_type == 1 else "float", "--scale", repr(float(scale)),
               "--chunk", str(chunk_grid), "--sub", str(sub_grid), "--threshold", str(merge_threshold),
               "--factor", repr(float(output_factor)), "--reps", str(reps), "--log", "3"]
        for flag, on in (("--intra", intra), ("--inter", inter), ("--replace", replacement),
                         ("--random", random), ("--weight", weighting), ("--pageable", pageable)):
            if on:
                cmd.append(flag)
        if export:
            cmd += ["--out", out]
        if report:
            cmd += ["--report", os.path.join(tmp, "statistics.json")]
        p = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
        line = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
        if p.returncode != 0 or not line:
            raise RuntimeError("reference runner failed (rc %d): %s %s" % (p.returncode, p.stdout[-2000:],
                                                                           p.stderr[-2000:]))
        res = json.loads(line[-1])
        if export:
            res["hierarchy"] = np.fromfile(os.path.join(out, "hierarchy.bin"), HIER_DTYPE)
            res["octree"] = np.fromfile(os.path.join(out, "octree.bin"), np.uint8)
            with open(os.path.join(out, "metadata.json")) as fh:
                res["metadata"] = json.load(fh)
            if not own:
                res["export_dir"] = out
        if report:
            with open(os.path.join(tmp, "statistics.json")) as fh:
                res["statistics"] = json.load(fh)
        return res
    finally:
        if own:
            import shutil

            shutil.rmtree(tmp, ignore_errors=True)
