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


def test_cutoff_scaling_workload_matches_reference_benchmark():
    # performance/CutOff-Performance/benchmark.py:14-75 at scale k, with simulate(cutOff=True)
    import bench
    from opendust_gb300 import build_simulation, workloads

    for k in (1, 8, 32):
        plasma, sim, grains, d, ext = workloads.cutoff_scaling(k=k)
        lam = plasma.r_D_e
        assert sim.N == k * 2**15 and sim.n == 3
        assert abs(sim.R / lam - 3) < 1e-12 and abs(sim.H / lam - 6 * k) < 1e-9
        assert abs(sim.d_t - 3.5148240854e-09) < 1e-20 and d == "Maxwellian"
        assert len(grains) == 1 and grains[0].chargeCalculationMethod == "given"
        assert abs(grains[0].q / (392500.0 * plasma.e) - 1) < 1e-15
        assert abs(grains[0].z / lam + 1) < 1e-12 and ext == {"cutOff": True}
        desc = bench.describe("cutoff_scaling", sim, ext)
        assert desc["n_ions"] == k * 2**15 and desc["steps_in_workload"] == 3
    holder, _ = build_simulation(plasma, sim, grains, d, trap=[0.0] * 15, **ext)
    assert abs(holder.cfg.cutoff / lam - 3.2) < 1e-12 and abs(holder.cfg.switch_dist / lam - 3.0) < 1e-12
    assert set(bench.CUTOFF_SCRIPT_PUBLISHED_S) == {1, 2, 4, 8, 32}


def test_reference_arm_cutoff_workloads():
    # the reference arm on the cutoff workloads (the oracle's cell list), switching and hard
    for extra in ([], ["--hard-cutoff"]):
        out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                              "--workload", "cutoff_scaling", "--scale", "1", "--steps", "1",
                              "--warmup", "1"] + extra,
                             capture_output=True, text=True, timeout=600, cwd=ROOT)
        assert out.returncode == 0, out.stderr[-2000:]
        line = json.loads(out.stdout.strip().splitlines()[-1])
        assert line["impl"] == "reference" and line["value"] > 0
        assert line["config"]["n_ions"] == 2**15 and line["config"]["steps_in_workload"] == 3
        assert ("hard" in line["config"]["force"]) == bool(extra)
        assert "within the cutoff" in line["cpu_baseline"]["sample"]
