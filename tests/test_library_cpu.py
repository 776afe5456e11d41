"""CPU checks of the C-ABI library: it loads, exports every entry point that
include/octreeApi.h declares, and reports errors through the return code
(no GPU work is issued here)."""
import ctypes
import os
import re

import numpy as np
import pytest

import octree_api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "octreeApi.h")).read()
    return re.findall(r"OCPI_EXPORT\s+[\w\s\*]+?\b(ocpi_\w+)\s*\(", text)


def test_header_declares_reference_api():
    names = declared_symbols()
    for s in octree_api.REFERENCE_SYMBOLS:
        assert s in names, s
    assert len(octree_api.REFERENCE_SYMBOLS) == 18


def test_library_exports_every_declared_symbol():
    L = octree_api.load_library()
    for name in declared_symbols():
        assert hasattr(L, name), name


def test_errors_are_return_codes():
    L = octree_api.load_library()
    assert L.ocpi_destroy_session(None) == -1
    assert b"No Session" in L.ocpi_last_error()
    assert L.ocpi_set_cloud_type(None, 0) == -1
    assert L.ocpi_generate_octree(None) == -1
    assert L.ocpi_set_logging_level(2) == 0


def test_python_session_raises():
    with pytest.raises(octree_api.OctreeError):
        octree_api._check(-1, "probe")


def test_noalloc_rejects_oversized_node_without_gpu():
    # the size limit is checked before any CUDA call
    L = octree_api.load_library()
    n = octree_api.NOALLOC_MAX_CANDIDATES + 1
    rc = L.ocpi_subsample_node_noalloc(None, 1, 27, None, None, None, 1.0, 0, 0, 32, 0, 0, None, None, n, None,
                                       None, None, None)
    assert rc == -1
    assert b"exceed the fixed scratch limit" in L.ocpi_last_error()


def test_memory_estimate_reference_formula():
    """The reference estimate restates tools/memory_consumption.py:30-75 (with
    the configured chunking grid) plus sparse nodes, counters and the RGBA
    grid; this library's bound exceeds the data it must hold."""
    n, stride = 119_701_547, 27
    gb300, ref = octree_api.estimate_memory(n, stride, 1, 512, 10000, 2.2, 128, octree_api.SUB_INTER)
    cells = sum((512 >> i) ** 3 for i in range(10))
    s3 = 128 ** 3
    f = float(np.float32(2.2))   # outputFactor is a float in the API
    want = (2 * cells * 4 + 4 + 4 * s3 + 48 * 1024 + 8 * s3 + n * 18 * f + n * stride + n * f * 4
            + min(cells, n) * 68)
    assert abs(ref - want) <= 16, (ref, want)
    out_cap = int(np.float32(n) * np.float32(2.2))
    must_hold = n * stride + cells * 4 + 2 * out_cap * 22
    assert must_hold < gb300 < 3 * must_hold
    # more points never need less memory
    g2, r2 = octree_api.estimate_memory(2 * n, stride, 1, 512, 10000, 2.2, 128, octree_api.SUB_INTER)
    assert g2 > gb300 and r2 > ref
    with pytest.raises(octree_api.OctreeError):
        octree_api.estimate_memory(n, stride, 1, 500, 10000, 2.2, 128, 0)   # grid not a power of two


def test_server_and_batch_argument_errors_without_gpu():
    """The batched and served entry points check their arguments before any
    CUDA call and report through the return code."""
    L = octree_api.load_library()
    assert L.ocpi_server_create(None, 0, 4, 1 << 30) == -1
    assert b"null server pointer" in L.ocpi_last_error()
    h = ctypes.c_void_p()
    assert L.ocpi_server_create(ctypes.byref(h), 0, 0, 1 << 30) == -1
    assert b"lanes" in L.ocpi_last_error()
    assert L.ocpi_batch_build(0, 4, 1 << 30, None, 0, None) == -1
    assert b"null argument" in L.ocpi_last_error()
    assert L.ocpi_batch_build_wave(0, 16, 1 << 30, None, 0, None) == -1
    assert b"null argument" in L.ocpi_last_error()
    jobs, res = (octree_api.OcpiJob * 1)(), (octree_api.OcpiJobResult * 1)()
    assert L.ocpi_batch_build_wave(0, 0, 1 << 30, jobs, 1, res) == -1
    assert b"waveSize" in L.ocpi_last_error()
    t = ctypes.c_uint64()
    assert L.ocpi_server_submit(None, ctypes.byref(octree_api.OcpiJob()), ctypes.byref(t)) == -1
    assert L.ocpi_server_wait(None, 1, None) == -1
    assert L.ocpi_server_release(None, 1) == -1


def test_job_structs_match_the_header(tmp_path):
    """ctypes layouts of OcpiJob / OcpiJobResult against the C compiler's."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    fields = {"OcpiJob": [f for f, _ in octree_api.OcpiJob._fields_],
              "OcpiJobResult": [f for f, _ in octree_api.OcpiJobResult._fields_]}
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "octreeApi.h"', 'int main(void) {']
    for st, fs in fields.items():
        src.append('printf("%%zu\\n", sizeof(%s));' % st)
        src += ['printf("%%zu\\n", offsetof(%s, %s));' % (st, f) for f in fs]
    src.append("return 0; }")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    want = []
    for st in (octree_api.OcpiJob, octree_api.OcpiJobResult):
        want.append(ctypes.sizeof(st))
        want += [getattr(st, f).offset for f, _ in st._fields_]
    assert got == want


def test_fault_injection_kinds():
    L = octree_api.load_library()
    assert L.ocpi_debug_inject_failures(7, 1) == -1
    assert b"unknown fault kind" in L.ocpi_last_error()
    assert L.ocpi_debug_inject_failures(octree_api.INJECT_ALLOCATION, 0) == 0
    assert L.ocpi_debug_inject_failures(octree_api.INJECT_LANE_LOSS, 0) == 0
