"""bench.py on the CPU: the reference arm's JSON line (the CPU restatement of the reference step,
timed on the host's cores) carries every key of the bench contract, and the committed ncu
traffic files match only their own size, variant and tile."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_reference_arm_json_contract():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "small_plain", "--steps", "1", "--warmup", "1"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == "ion-steps/s" and line["value"] > 0
    assert line["steps"] == 1 and line["warmup"] == 1 and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert "workload" in line["config"]


def test_traffic_files_match_their_capture_only():
    import bench

    # the fixed-point accumulators leave positions and sums in L2: tens of MB per evaluation
    assert 1e7 < bench.load_traffic(2**20, {"variant": 7, "jsplit": 2048}) < 1e9
    assert bench.load_traffic(2**19, {"variant": 7, "jsplit": 2048}) is None
    assert 1e7 < bench.load_traffic(2**19, {"variant": 3, "jsplit": 512}, cutoff=True) < 1e9
    assert bench.load_traffic(2**19, {"variant": 3, "jsplit": 1024}, cutoff=True) is None
