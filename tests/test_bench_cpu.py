"""bench.py without a GPU: the reference arm (the multithreaded CPU oracle on
a bounded sample of the headline cloud) prints one JSON line with the keys of
the measurement contract, and the export timing of the GPU arm counts and
removes what it wrote."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, out.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == "Mpts/s octree build @120M pts" and line["unit"] == "Mpts/s"
    assert line["higher_is_better"] is True and line["n_gpus"] == 1
    assert line["steps"] == 1 and line["warmup"] == 3
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["workload"] == "lod_build_120M_f64_terrain_zipf"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_export_timing_reports_bytes_and_removes_the_files(tmp_path, monkeypatch):
    """bench.py's export field: one export into a scratch directory, its
    bytes counted and the files removed; skipped when the scratch file
    system cannot hold twice the records."""
    import tempfile

    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setattr(tempfile, "tempdir", str(tmp_path))

    class FakeSession:
        def export_potree(self, directory):
            for name, size in (("hierarchy.bin", 44), ("octree.bin", 1800), ("metadata.json", 10)):
                with open(os.path.join(directory, name), "wb") as f:
                    f.write(b"\0" * size)

    r = bench.export_timing(FakeSession(), 100)
    assert r["bytes"] == 1854 and r["ms"] >= 0 and r["gbs"] >= 0
    assert os.listdir(tmp_path) == []
    assert "skipped" in bench.export_timing(FakeSession(), 10 ** 18)
