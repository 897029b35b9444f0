"""The benchmark's reference arm (the oracle port timed on the host cores) prints one JSON line
with the fields the measurement contract names; run here on a small orchard."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--trees", "2", "2",
                          "--steps", "1", "--warmup", "1", "--ref-seconds", "0.5"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["unit"] == "rays/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["config"]["workload"].startswith("orchard-")
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_counter_digest_ignores_comments(tmp_path):
    """The ncu counters in the bench line are tied to a digest of the kernel code: a comment
    edit keeps it, a code edit changes it."""
    sys.path.insert(0, ROOT)
    import bench

    a, b, c = tmp_path / "a.cuh", tmp_path / "b.cuh", tmp_path / "c.cuh"
    a.write_text("int f(int x) {\n    return x + 1;  // one\n}\n")
    b.write_text("// header\nint f(int x) {\n\n    /* the sum */ return x + 1;   // plus one\n}\n")
    c.write_text("int f(int x) {\n    return x + 2;\n}\n")
    assert bench.code_digest([a]) == bench.code_digest([b])
    assert bench.code_digest([a]) != bench.code_digest([c])
    assert len(bench.kernel_sources_digest()) == 12
