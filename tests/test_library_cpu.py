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
    assert L.ocpi_batch_build_wave(0, 300, 1 << 30, jobs, 1, res) == -1
    assert b"waveSize" in L.ocpi_last_error()
    assert L.ocpi_batch_autotune(0, 1 << 30, None, 0, 0, None, None) == -1
    assert b"null argument" in L.ocpi_last_error()
    tuning = octree_api.OcpiBatchTuning(waveSize=16, clusterCap=3, weightedClusterCap=16, useGraphs=1)
    assert L.ocpi_batch_build_tuned(0, 1 << 30, ctypes.byref(tuning), jobs, 1, res) == -1
    assert b"clusterCap" in L.ocpi_last_error()
    tuning.clusterCap, tuning.weightedClusterCap = 4, 32
    assert L.ocpi_batch_build_tuned(0, 1 << 30, ctypes.byref(tuning), jobs, 1, res) == -1
    assert b"weightedClusterCap" in L.ocpi_last_error()
    tuning.lanes = 65
    assert L.ocpi_batch_build_tuned(0, 1 << 30, ctypes.byref(tuning), jobs, 1, res) == -1
    assert b"lanes" in L.ocpi_last_error()
    t = ctypes.c_uint64()
    assert L.ocpi_server_submit(None, ctypes.byref(octree_api.OcpiJob()), ctypes.byref(t)) == -1
    assert L.ocpi_server_wait(None, 1, None) == -1
    assert L.ocpi_server_release(None, 1) == -1


def test_job_structs_match_the_header(tmp_path):
    """ctypes layouts of OcpiJob / OcpiJobResult / OcpiBatchTuning / OcpiStats
    against the C compiler's."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    fields = {"OcpiJob": [f for f, _ in octree_api.OcpiJob._fields_],
              "OcpiJobResult": [f for f, _ in octree_api.OcpiJobResult._fields_],
              "OcpiBatchTuning": [f for f, _ in octree_api.OcpiBatchTuning._fields_],
              "OcpiStats": [f for f, _ in octree_api.OcpiStats._fields_]}
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
    for st in (octree_api.OcpiJob, octree_api.OcpiJobResult, octree_api.OcpiBatchTuning, octree_api.OcpiStats):
        want.append(ctypes.sizeof(st))
        want += [getattr(st, f).offset for f, _ in st._fields_]
    assert got == want


def test_fault_injection_kinds():
    L = octree_api.load_library()
    assert L.ocpi_debug_inject_failures(7, 1) == -1
    assert b"unknown fault kind" in L.ocpi_last_error()
    assert L.ocpi_debug_inject_failures(octree_api.INJECT_ALLOCATION, 0) == 0
    assert L.ocpi_debug_inject_failures(octree_api.INJECT_LANE_LOSS, 0) == 0


# The reference CLI's call sequence (src/main.cpp:54-107): a session, the
# cloud setters, the two configuration calls, init, generate, export and the
# three reports, then destroy.
CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "octreeApi.h"

int main(int argc, char** argv)
{
    const char* out = argc > 1 ? argv[1] : ".";
    static unsigned char cloud[15 * 4];
    char path[4096];
    void* session = 0;
    int rc[19], k = 0;
    rc[k++] = ocpi_set_logging_level(1);
    rc[k++] = ocpi_create_session(&session, 0);
    rc[k++] = ocpi_set_cloud_type(session, 0);
    rc[k++] = ocpi_set_cloud_point_amount(session, 4);
    rc[k++] = ocpi_set_cloud_data_stride(session, 15);
    rc[k++] = ocpi_set_cloud_scale(session, 0.001, 0.001, 0.001);
    rc[k++] = ocpi_set_cloud_offset(session, 0.0, 0.0, 0.0);
    rc[k++] = ocpi_set_cloud_bb(session, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0);
    rc[k++] = ocpi_set_point_cloud_host(session, cloud);
    rc[k++] = ocpi_configure_chunking(session, 512, 10000, 2.2f);
    rc[k++] = ocpi_configure_subsampling(session, 128, 0, 1, 1, 0, 0);
    rc[k++] = ocpi_init_octree(session);
    rc[k++] = ocpi_generate_octree(session);
    rc[k++] = ocpi_export_potree(session, out);
    snprintf(path, sizeof path, "%s/point_distribution.html", out);
    rc[k++] = ocpi_export_distribution_histogram(session, path, 0);
    snprintf(path, sizeof path, "%s/statistics.json", out);
    rc[k++] = ocpi_export_json_report(session, path);
    snprintf(path, sizeof path, "%s/memory_report.html", out);
    rc[k++] = ocpi_export_memory_report(session, path);
    rc[k++] = ocpi_destroy_session(session);
    for (int i = 0; i < k; ++i) printf("%d ", rc[i]);
    printf("\n%s\n", ocpi_last_error ? "linked" : "");
    return 0;
}
"""


def _compile_and_run(tmp_path, compiler, source, include_dir, lang):
    import shutil
    import subprocess

    cc = shutil.which(compiler)
    if not cc:
        pytest.skip("no %s" % compiler)
    lib_dir = os.path.dirname(octree_api.LIB_PATH)
    src = tmp_path / ("caller." + lang)
    src.write_text(source)
    exe = tmp_path / "caller"
    subprocess.run([cc, "-I", include_dir, str(src), "-o", str(exe), "-L", lib_dir, "-lOctreeApi",
                    "-Wl,-rpath," + lib_dir], check=True)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return [int(v) for v in r.stdout.split("\n")[0].split()]


def _check_codes(codes):
    assert len(codes) == 18
    assert codes[0] == 0   # logging level
    try:
        import torch

        gpu = torch.cuda.is_available()
    except ImportError:
        gpu = False
    if not gpu:
        # no device: the session cannot be created, and every call on the
        # missing session returns UNEXPECTED_ERROR instead of faulting
        assert codes[1] == -1
        assert all(c == -1 for c in codes[2:]), codes


def test_c_caller_links_and_runs(tmp_path):
    """A C program making the reference CLI's calls compiles against
    include/octreeApi.h (as C11), links against libOctreeApi.so and runs."""
    codes = _compile_and_run(tmp_path, "gcc", "#include <stdbool.h>\n" + CALLER,
                             os.path.join(ROOT, "include"), "c")
    _check_codes(codes)


def test_caller_against_reference_header_links(tmp_path):
    """The same caller compiled as C++ against the reference's own declarations
    (OctreeApi/include/octreeApi.h, whose EXPORTED macro is extern "C" on this
    platform) resolves every call in libOctreeApi.so."""
    ref_inc = os.path.join(os.environ.get("OC_REFERENCE_DIR", "/root/reference"), "OctreeApi", "include")
    if not os.path.exists(os.path.join(ref_inc, "octreeApi.h")):
        pytest.skip("reference checkout not present")
    src = CALLER.replace('printf("\\n%s\\n", ocpi_last_error ? "linked" : "");', 'printf("\\nlinked\\n");')
    codes = _compile_and_run(tmp_path, "g++", src, ref_inc, "cpp")
    _check_codes(codes)
