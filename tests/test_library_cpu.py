"""CPU checks of the C-ABI library: it loads, exports every entry point that
include/octreeApi.h declares, and reports errors through the return code
(no GPU work is issued here)."""
import ctypes
import os
import re

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
