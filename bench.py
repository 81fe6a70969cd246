#!/usr/bin/env python
"""Benchmark of the per-timestep superion update (one JSON line on stdout).

Workload (default "full_plain"): Ar+ plasma at Mach 1 around one grain, R = 3 lambda,
H = 6 lambda, N = 2^20 superions, all-pairs screened ion–ion forces, charge-exchange
collisions with a 2 lambda mean free path, d_t = 1e-10 s (opendust_gb300.workloads).
One "step" is one pass of the superion update over all N ions (kick, drift, N^2 force,
kick, flags, ordered compaction, re-injection, grain sums, FP64 tail).

  value      ion-steps/s from CUDA events on the library's stream over K timed steps, inputs
             resident in HBM, L2 flushed (512 MB write) before every timed step.
  e2e        the same metric through the C ABI with host arrays: od_set_state (host->device,
             including the initial force evaluation), then per step od_step and od_get_series of
             that step (device->host), then od_get_state (device->host); wall clock.
  roofline   the all-pairs force evaluation: N(N-1) directed pair interactions x 25 FP32 flops
             per launch over its CUDA-event duration, against the larger of the FP32 FMA probe
             and the SMs' FP32 rate at the sampled clock. The default kernel from 2^14 ions
             (variant 7) evaluates each unordered pair once and applies it to both ions, so it
             does about half those flops (executed_frac). Cutoff workloads credit the pairs
             inside r_c, counted by one more, untimed step.
Other workloads (--workload): small_plain (C1, 16384 ions), field_chain (C3, 2^19 ions, 2 lambda
cutoff; --hard-cutoff without the switching function), cutoff_scaling (the reference's cutoff
benchmark, N = k*2^15 with --scale k, plus the wall time of its script through simulate()),
sweep (C4: 64 simulations batched against the plain path back to back) and serve (C5: a Poisson
request stream through the continuous-batching server against the plain path).
  cpu_baseline  the CPU oracle (FP64 C restatement of the reference step, OpenMP over all host
             cores) on a bounded sample: the reference's two ion–ion evaluations per step for T
             target ions against all N sources plus one linear pass over all N ions.

--impl reference times that CPU restatement alone (the reference's own OpenMM/CuPy path
cannot be installed or run on this machine) and prints the same metric.
Multi-GPU (torchrun, N > 1): independent replicas, one per GPU (one simulation sharded over
GPUs is opendust_gb300.shard, not this benchmark); value = ion-steps of all ranks / max over
ranks of the timed duration.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOPS_PER_PAIR = 25
KERNELS_PER_STEP = 5          # all pairs: kick/drift, pairs, kick/flag (takes the fixed-point
                              # sums), collect/inject, correct/orbit (its last block runs the
                              # FP64 tail)
KERNELS_PER_STEP_CUTOFF = 11  # + cell clear, count, scan, scatter, sort, chunk scan
KERNELS_PER_STEP_CUTOFF_TILES = 15  # + clear, count, scan, scatter, sort, boxes, pairs,
                                    # scan, list, tile-pair kernel, slot take (cutoff variant 3)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="full_plain",
                    choices=["full_plain", "small_plain", "field_chain", "cutoff_scaling", "sweep",
                             "serve"])
    ap.add_argument("--scale", type=int, default=8,
                    help="cutoff_scaling: k in N = k*2^15 ions, H = k*6 lambda")
    ap.add_argument("--hard-cutoff", action="store_true",
                    help="cutoff workloads: no switching polynomial (pairs at r_c decided in FP64 "
                         "as the oracle decides them)")
    ap.add_argument("--sweep-sims", type=int, default=64)
    ap.add_argument("--sweep-exact", action="store_true")
    ap.add_argument("--pilot-steps", type=int, default=100)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--duration", type=float, default=10.0)
    ap.add_argument("--window", type=int, default=50)
    ap.add_argument("--log2n", default="14,19")
    ap.add_argument("--serve-exact", action="store_true")
    ap.add_argument("--cpu-sample-targets", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


class Dist:
    def __init__(self, backend):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            if backend == "nccl":
                import torch

                torch.cuda.set_device(self.local)
            dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def reduce(self, x: float, op: str) -> float:
        if self.world == 1:
            return x
        import torch

        dev = f"cuda:{self.local}" if self.dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX if op == "max" else self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        # raw samples: $OD_CLOCKS_DIR if set (to keep them), else the system temp directory
        self.path = os.path.join(os.environ.get("OD_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"opendust_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.fh.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        mhz = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(mhz) if mhz else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def workload(name: str, n_total: int, scale: int = 8, hard: bool = False):
    from opendust_gb300 import workloads

    if name == "cutoff_scaling":
        w = workloads.cutoff_scaling(k=scale, n=n_total)
    elif name == "full_plain":
        w = workloads.full_plain(n=n_total)
    elif name == "field_chain":
        w = workloads.field_chain(n=n_total)
    else:
        w = workloads.small_plain(n=n_total)
    if hard:
        if name not in ("cutoff_scaling", "field_chain"):
            raise SystemExit("--hard-cutoff applies to the cutoff workloads")
        w[4]["switch_distance"] = 0.0
    return w


def describe(name, sim, ext):
    w = {"cutoff_scaling": "",
         "full_plain": "Ar+ Mach 1 flow past one grain (r=10 um, consistent charging), "
                       "N=2^20 superions, all-pairs Yukawa, charge-exchange mfp 2 lambda, d_t=1e-10 s",
         "small_plain": "Ar+ Mach 1 flow past one grain, N=16384, all-pairs Yukawa, no collisions, "
                        "d_t=1e-10 s",
         "field_chain": "field-driven Ar+ (Mach 0.5, charge-exchange mfp 1 lambda) past a chain of 5 "
                        "grains (r=5 um, 1 lambda apart), N=2^19, cutoff 2 lambda over a device cell "
                        "list, d_t=1e-10 s"}[name]
    if name == "cutoff_scaling":
        k = int(sim.N) // 2**15
        w = (f"the reference's cutoff benchmark at k={k}: Ar+ Mach 1 (T_e=29011 K, T_i=290.11 K), "
             f"R=3 lambda, H={6 * k} lambda, N={k}*2^15, cutoff 3.2 lambda with switching from "
             "3.0 lambda, one grain of given charge, d_t=3.5148e-9 s")
    cut = "cutoff_distance" in ext or ext.get("cutOff", False)
    force = "all-pairs"
    if cut:
        force = "cutoff (Hilbert-sorted tile pairs), " + (
            "hard: no switching, pairs within FP32 rounding of r_c decided in FP64"
            if ext.get("switch_distance") == 0.0 else "OpenMM switching from 15/16 of r_c")
    return {"workload": f"{name}: {w}", "n_ions": int(sim.N), "grains": len(sim_grains(name)),
            "force": force,
            "collisions": ext.get("collisions", "none"),
            "l2": "flushed (512 MB write) before every timed step",
            "steps_in_workload": {"full_plain": 20000, "small_plain": 2000, "field_chain": 30000,
                                  "cutoff_scaling": 3}[name]}


def sim_grains(name):
    return [0] * (5 if name == "field_chain" else 1)


def cpu_sample(holder, pos, targets: int, repeats: int = 2):
    """Seconds per full reference step on the host, estimated from a bounded sample."""
    import numpy as np

    from oracle import oracle

    n = pos.shape[0]
    idx = np.linspace(0, n - 1, targets).astype(np.int64)
    best = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        oracle.force_targets(holder, pos, idx)  # ion–ion evaluation A (opendust.py:864)
        oracle.force_targets(holder, pos, idx)  # ion–ion evaluation B (opendust.py:866)
        t1 = time.perf_counter()
        oracle.collect_flags(holder, pos)       # one linear pass over all N ions
        t2 = time.perf_counter()
        est = (t1 - t0) * (n / targets) + (t2 - t1)
        best = est if best is None else min(best, est)
    return best, oracle.max_threads()


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return 0
    import numpy as np

    from opendust_gb300 import build_simulation, setup_host
    from oracle import oracle

    plasma, sim, grains, d, ext = workload(args.workload, 10, args.scale, args.hard_cutoff)
    holder, _ = build_simulation(plasma, sim, grains, d, seed=1, trap=np.zeros(15), **ext)
    pos, vel = setup_host.initial_state(sim.N, sim.R, sim.H, [(g.x, g.y, g.z, g.r) for g in grains],
                                        plasma.v_fl, plasma.v_T, d, 1)
    T = args.cpu_sample_targets or (256 if sim.N > 100000 else 4096)
    oracle.set_threads(os.cpu_count() or 1)
    for _ in range(max(args.warmup, 0)):
        cpu_sample(holder, pos, T, repeats=1)
    per_step = []
    for _ in range(args.steps):
        s, cores = cpu_sample(holder, pos, T, repeats=1)
        per_step.append(s)
    sec = sum(per_step) / len(per_step)
    value = sim.N / sec
    srcs = "the sources within the cutoff (cell list)" if holder.cfg.cutoff > 0 else "all sources"
    sample = (f"{T} of {sim.N} target ions x 2 ion-ion evaluations against {srcs} + one "
              f"linear pass over all ions per step; time per full step extrapolated by N/T")
    line = {
        "impl": "reference", "metric": "ion-steps/s", "value": value, "unit": "ion-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": describe(args.workload, sim, ext),
        "cpu_baseline": {"value": value, "unit": "ion-steps/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "ion-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's OpenMM/CuPy path cannot be installed here; this is the FP64 C "
                "restatement of its step (oracle/od_oracle.c) on the host cores",
    }
    print(json.dumps(line), flush=True)
    return 0


def load_traffic(n_ions: int, plan: dict, cutoff: bool = False):
    """DRAM bytes per force evaluation from the committed ncu capture of the same size and
    kernel variant (all-pairs kernel, or the cutoff force chain with its tile size)."""
    name = "cutoff_traffic.json" if cutoff else "allpairs_traffic.json"
    try:
        d = json.load(open(os.path.join(ROOT, "profiles", name)))
    except (OSError, ValueError):
        return None
    ok = d.get("n_ions") == n_ions and d.get("variant") == plan["variant"]
    if "tile" in d:
        ok = ok and d["tile"] == plan["jsplit"]
    return d.get("dram_bytes_per_launch") if ok else None


def run_ours(args, dist: Dist):
    import numpy as np
    import torch

    from opendust_gb300 import _lib, build_simulation, setup_host

    device = dist.local
    torch.cuda.set_device(device)
    K, W = args.steps, args.warmup
    K_e2e = max(2, K)
    n_total = W + K + K_e2e + 5
    plasma, sim, grains, d, ext = workload(args.workload, n_total, args.scale, args.hard_cutoff)
    seed = 1000 + dist.rank
    holder, _ = build_simulation(plasma, sim, grains, d, seed=seed, device=device, **ext)
    pos, vel = setup_host.initial_state(sim.N, sim.R, sim.H, [(g.x, g.y, g.z, g.r) for g in grains],
                                        plasma.v_fl, plasma.v_T, d, seed)
    N = int(sim.N)
    peak = _lib.fp32_peak_tflops(device)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device}")
    eng = _lib.Engine(holder, device)
    plan = eng.pair_plan()
    eng.set_state(pos, vel)
    eng.step(W)  # warm-up (graph replay path)
    eng.set_timing(True, count_pairs=False)
    clocks = Clocks(device)
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    for _ in range(K):
        flush.zero_()
        torch.cuda.synchronize()
        eng.step(1)
    torch.cuda.synchronize()
    clk = clocks.stop()
    dist.barrier()
    step_ms, nsteps, pair_ms, pair_launches = eng.timing()
    cut_pairs = 0
    if holder.cfg.force_method == _lib.OD_FORCE_CUTOFF:
        # one more (untimed) step with the counting kernel: pairs inside the cutoff per launch
        eng.set_timing(True, count_pairs=True)
        eng.step(1)
        cut_pairs = eng.cutoff_pairs() * pair_launches / max(eng.timing()[3], 1)
    eng.set_timing(False)
    t_max = dist.reduce(step_ms, "max")
    ions_all = dist.reduce(float(N * K), "sum")
    value = ions_all / (t_max * 1e-3)
    pair_avg_s = pair_ms / pair_launches * 1e-3
    cutoff = cut_pairs > 0
    pairs_per_launch = cut_pairs / pair_launches if cutoff else N * (N - 1)
    achieved = pairs_per_launch * FLOPS_PER_PAIR / pair_avg_s / 1e12
    # the larger of the probe and the FP32 rate of the SMs at the sampled clock (128 FP32 lanes,
    # 2 flops per FMA), so that a soft probe cannot inflate the fraction
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    theo = sms * 128 * 2 * (clk.get("sm_mhz") or 0.0) * 1e6 / 1e12
    peak_used = max(peak, theo)
    n3 = not cutoff and plan["variant"] == 7
    traffic = load_traffic(N, plan, cutoff)
    if cutoff and plan["variant"] == 3:
        kernel = (f"Hilbert-order sort + tile-pair list + k_pairs_cutn3 (each pair once, {plan['jsplit']}-ion "
                  "tiles, 64-ion group pairs beyond r_c skipped; pairs inside the cutoff credited)")
    elif cutoff:
        kernel = "cell-list build + k_pairs_cut (pairs inside the cutoff)"
    elif n3:
        kernel = (f"k_pairs_n3 + k_n3_take (each unordered pair once, {plan['jsplit']}-ion tiles, "
                  "fixed-point atomic sums; "
                  "credited with the N(N-1) directed pair terms it replaces)")
    else:
        kernel = f"k_pairs_x2 variant {plan['variant']} (all-pairs ion-ion)"
    if cutoff:
        launches = KERNELS_PER_STEP_CUTOFF_TILES if plan["variant"] == 3 else KERNELS_PER_STEP_CUTOFF
    else:
        launches = KERNELS_PER_STEP

    # e2e through the C ABI with host buffers (the calls simulate() makes)
    eng.close()
    eng = _lib.Engine(holder, device)
    dist.barrier()
    t0 = time.perf_counter()
    eng.set_state(pos, vel)
    rows = []
    for i in range(K_e2e):  # each step's grain results read back as the reference does per step
        eng.step(1)
        rows.append(eng.series(i, 1))
    ser = {k: np.concatenate([r[k] for r in rows]) for k in rows[0]}
    p_out, v_out = eng.get_state()
    t1 = time.perf_counter()
    e2e_t = dist.reduce(t1 - t0, "max")
    e2e_value = dist.reduce(float(N * K_e2e), "sum") / e2e_t
    h2d = 2 * N * 16
    d2h = sum(a.nbytes for a in ser.values()) // 2 + 2 * N * 16  # float4 state copies
    eng.close()
    assert np.isfinite(ser["q"]).all() and np.isfinite(p_out).all()

    script = None
    if args.workload == "cutoff_scaling" and dist.rank == 0:
        script = time_reference_script(args.scale, device)
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        from oracle import oracle

        oracle.set_threads(os.cpu_count() or 1)
        T = args.cpu_sample_targets or (512 if N > 100000 else 4096)
        sec, cores = cpu_sample(holder, pos, T, repeats=2)
        cpu = {"value": N / sec, "unit": "ion-steps/s", "cores": cores, "kind": "port",
               "sample": f"{T} of {N} target ions x 2 ion-ion evaluations + one linear pass; "
                         f"full-step time extrapolated by N/T (FP64 C oracle, OpenMP)"}
    if dist.rank == 0:
        line = {
            "metric": "ion-steps/s", "value": value, "unit": "ion-steps/s", "n_gpus": dist.world,
            "steps": K, "warmup": W, "ms_per_step": t_max / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded initial state and Philox streams)",
            "config": {**describe(args.workload, sim, ext),
                       "parallelism": f"replicas x{dist.world}" if dist.world > 1 else "1 GPU"},
            "pair_interactions_per_s": (pairs_per_launch * K * dist.world / (t_max * 1e-3)),
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_used, "unit": "TFLOP/s",
                         "frac": achieved / peak_used, "traffic": traffic, "kernel": kernel,
                         "peak_source": ("max of the FP32 FMA probe measured in this run "
                                         f"({peak:.1f}) and {sms} SMs x 128 lanes x 2 flops at the "
                                         f"median sampled SM clock ({theo:.1f})"),
                         "peak_probe": peak, "peak_sm_clock": theo,
                         # each unordered pair evaluated once: its 25 flops plus the 6 of the
                         # reaction sum, against the directed-pair credit above
                         "executed_frac": (None if not n3 else
                                           N * (N - 1) / 2 * (FLOPS_PER_PAIR + 6) / pair_avg_s / 1e12
                                           / peak_used),
                         "flops_per_pair": FLOPS_PER_PAIR, "pair_ms_avg": pair_avg_s * 1e3},
            "e2e": {"value": e2e_value, "unit": "ion-steps/s", "h2d_bytes_per_step": h2d // K_e2e,
                    "d2h_bytes_per_step": d2h // K_e2e},
            "gpu_launches": launches * K,
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        if script is not None:
            line["reference_script"] = script
        print(json.dumps(line), flush=True)
    return 0


# wall seconds of one run of performance/CutOff-Performance/benchmark.py per scale k, as logged
# in performance/CutOff-Performance/time.txt (V100-class GPU; setup + 3 steps)
CUTOFF_SCRIPT_PUBLISHED_S = {1: 80.17, 2: 174.09, 4: 388.38, 8: 886.01, 32: 1316.75}


def time_reference_script(k: int, device: int):
    """The reference's cutoff benchmark script through the drop-in API: OpenDust(...) with its
    parameters and simulate(deviceIndex, cutOff=True), 3 steps; wall clock around simulate() as
    the script times it (setup of tables, trap fit and initial state included)."""
    from opendust_gb300 import OpenDust, OutputParameters, workloads

    plasma, sim, grains, d, _ = workloads.cutoff_scaling(k=k, n=3)
    od = OpenDust(plasma, sim, OutputParameters(2999, 2999), grains, d)
    t0 = time.perf_counter()
    od.simulate(deviceIndex=str(device), cutOff=True, quiet=True)
    t1 = time.perf_counter()
    pub = CUTOFF_SCRIPT_PUBLISHED_S.get(k)
    return {"k": k, "n_ions": int(sim.N), "steps": 3, "simulate_s": t1 - t0, "published_s": pub,
            "published_hw": "V100-class (reference log)",
            "source": "performance/CutOff-Performance/benchmark.py, time.txt"}


def run_sweep(args, dist: Dist):
    """Batched sweep (64 independent simulations drawn from seeds) against the same
    simulations run back to back on the plain path; K steps each, wall clock, same GPU.

    The batched arm first picks each member's ion–ion force interval k with
    tuning.choose_force_interval (a pilot window of --pilot-steps steps from the member's own
    initial state, error bound 1 % on the time-averaged grain charge and ion force), then runs
    all members in one batch. With --sweep-exact every member keeps k = 1 (the reference's
    integrator) and members whose plan matches the plain default are compared bitwise."""
    import numpy as np

    from opendust_gb300 import _lib, build_simulation, setup_host, tuning, workloads

    if dist.rank != 0:
        return 0
    K, W, S = args.steps, args.warmup, args.sweep_sims
    window = 5000
    members = []
    t_setup = time.perf_counter()
    for k in range(S):
        plasma, sim, grains, d, ext = workloads.sweep_member(seed=k, n_steps=K + W)
        holder, _ = build_simulation(plasma, sim, grains, d, seed=k, **ext)
        pos, vel = setup_host.initial_state(sim.N, sim.R, sim.H, [(g.x, g.y, g.z, g.r) for g in grains],
                                            plasma.v_fl, plasma.v_T, d, k)
        members.append((holder, pos, vel, sim.N))
    t_setup = time.perf_counter() - t_setup
    ion_steps = sum(m[3] for m in members) * K
    # plain path, back to back, each simulation with its own default all-pairs plan
    plain_s = 0.0
    plain_series, same_plan = [], []
    for holder, pos, vel, n in members:
        with _lib.Engine(holder) as eng:
            pl = eng.pair_plan()
            bp = _lib.batch_pair_plan(n)
            same_plan.append((pl["threads"], pl["targets_per_thread"], pl["variant"]) == bp[:3] and
                             (bp[2] != 7 or pl["jsplit"] == bp[3]))
            eng.set_state(pos, vel)
            eng.step(W)
            t0 = time.perf_counter()
            eng.step(K)
            plain_s += time.perf_counter() - t0
            plain_series.append(eng.series(0, K + W))
    # force interval per member (pilot windows), unless the exact sweep is asked for
    t_tune = time.perf_counter()
    intervals, pilot_err, shapes = [], [], []
    cache = tuning.PlanCache(os.path.join(tempfile.gettempdir(), f"od_plans_{os.getpid()}.json"))
    for holder, pos, vel, n in members:
        if args.sweep_exact:
            intervals.append(1)
            shapes.append(None)
            continue
        # each-pair-once shape per size bucket, measured once per bucket in this run
        shapes.append(tuning.batch_plan_for(int(n), cache=cache))
        r = tuning.choose_force_interval(holder, pos, vel, max_rel_err=0.01,
                                         pilot_steps=args.pilot_steps)
        intervals.append(r["force_every"])
        pilot_err.append(max(r["errors"].values()))
    t_tune = time.perf_counter() - t_tune
    # batched
    with _lib.Batch() as batch:
        slots = []
        for (h, p, v, _), k, sh in zip(members, intervals, shapes):
            h.cfg.force_every = k
            slots.append(batch.add(h, p, v))
            if sh is not None:
                batch.set_plan(slots[-1], *sh)
        batch.step(W)
        t0 = time.perf_counter()
        batch.step(K)
        batch_s = time.perf_counter() - t0
        batch_dev_ms = batch.last_step_ms()
        same, qdiff = True, 0.0
        win_q, win_f = [], []
        for s, ps, sp, k in zip(slots, plain_series, same_plan, intervals):
            bs = batch.member(s).series(0, K + W)
            if k == 1 and sp:
                same = same and all(np.array_equal(bs[q], ps[q]) for q in ps)
            elif k == 1:
                qdiff = max(qdiff, float(np.max(np.abs(bs["q"] - ps["q"]) /
                                                np.maximum(np.abs(ps["q"]), 1e-30))))
            # time averages over the second half of the run, batched against plain
            h0 = (K + W) // 2
            qb, qp = bs["q"][h0:].mean(0), ps["q"][h0:].mean(0)
            fb = (bs["orbit"] + bs["collect"])[h0:].mean(0)
            fp = (ps["orbit"] + ps["collect"])[h0:].mean(0)
            win_q.append(float(np.max(np.abs(qb - qp) / np.maximum(np.abs(qp), 1e-300))))
            win_f.append(float(np.linalg.norm(fb - fp) / max(np.linalg.norm(fp), 1e-300)))
    for h, *_ in members:
        h.cfg.force_every = 1
    per_window = lambda sec: sec / K * window / S
    tune_per_sim = t_tune / S
    ks, counts = np.unique(intervals, return_counts=True)
    line = {"metric": "sweep sims/hour", "unit": "simulations/hour (5000-step windows, 64 seeded members)",
            "value": 3600.0 / (per_window(batch_s) + tune_per_sim),
            "plain_value": 3600.0 / per_window(plain_s),
            "ratio_batched_vs_plain": per_window(plain_s) / (per_window(batch_s) + tune_per_sim),
            "ratio_steps_only": plain_s / batch_s,
            "steps": K, "warmup": W, "batched_step_ms": batch_s / K * 1e3,
            "batched_device_step_ms": batch_dev_ms / K, "plain_step_ms_sum": plain_s / K * 1e3,
            "ion_steps_per_s_batched": ion_steps / batch_s, "ion_steps_per_s_plain": ion_steps / plain_s,
            "tuning_s": t_tune, "pilot_steps": args.pilot_steps,
            "force_every": {str(int(a)): int(b) for a, b in zip(ks, counts)},
            "batch_shapes": {f"{a}x{b}": sum(1 for sh in shapes if sh == (a, b))
                             for a, b in tuning.BATCH_SHAPES},
            "pilot_max_rel_err": max(pilot_err) if pilot_err else 0.0,
            "window_rel_err_vs_plain": {"q_max": max(win_q), "force_max": max(win_f),
                                        "force_median": float(np.median(win_f)),
                                        "steps_averaged": (K + W) - (K + W) // 2},
            "results_equal_bitwise_k1": bool(same),
            "bitwise_members": f"{sum(sp and k == 1 for sp, k in zip(same_plan, intervals))} of {S}",
            "q_rel_diff_other_k1_members": qdiff,
            "host_setup_s": t_setup, "n_ions": [int(m[3]) for m in members],
            "config": {"workload": "sweep: 64 members, N log-uniform 2^14-2^18, Mach 0.1-2, grain radius "
                                   "1-20 um log-uniform, 1-4 grains, mfp collisions with p=0.5",
                       "batched": "exact (k = 1)" if args.sweep_exact else
                                  "ion-ion force interval per member (pilot-tuned, 1 % bound)"}}
    print(json.dumps(line), flush=True)
    return 0


def run_serve(args, dist: Dist):
    """Poisson request stream through the continuous-batching server vs the plain path. Both
    arms get the same process pool for the host part of each request's setup, so the ratio
    measures what the GPU co-scheduling buys. The server runs every request with the ion–ion
    force interval of serve.interval_by_size (or every step with --serve-exact); each request's
    time-averaged charge and ion force are compared with the plain path's."""
    import copy

    import numpy as np

    from opendust_gb300 import serve

    if dist.rank != 0:
        return 0
    lo, hi = (float(x) for x in args.log2n.split(","))
    reqs = serve.poisson_requests(rate=args.rate, duration=args.duration, seed=7, log2n=(lo, hi),
                                  window=args.window)
    pool = serve.start_pool(8)
    list(pool.map(int, range(8)))  # start the workers before the timed runs
    interval = None if args.serve_exact else serve.interval_by_size
    served = copy.deepcopy(reqs)
    s = serve.Server(chunk=10, interval=interval).run(served, pool=pool)
    plain_reqs = copy.deepcopy(reqs)
    p = serve.run_plain(plain_reqs, pool=pool)
    pool.shutdown()
    eq, dq, df = True, [], []
    for a, b in zip(sorted(served, key=lambda r: r.rid), sorted(plain_reqs, key=lambda r: r.rid)):
        qa, qb = a.averages[:, 0], b.averages[:, 0]
        fa, fb = a.averages[:, 1:4] + a.averages[:, 4:7], b.averages[:, 1:4] + b.averages[:, 4:7]
        dq.append(float(np.max(np.abs(qa - qb) / np.maximum(np.abs(qb), 1e-300))))
        df.append(float(np.linalg.norm(fa - fb) / max(np.linalg.norm(fb), 1e-300)))
        eq = eq and all(np.array_equal(a.series[k], b.series[k]) for k in a.series)
    ks = [interval(int(r.sim.N)) if interval else 1 for r in reqs]
    line = {"metric": "request latency p99 (s)", "value": s["latency_p99_s"], "unit": "s",
            "higher_is_better": False, "server": s, "plain": p,
            "throughput_ratio_server_vs_plain": s["throughput_req_per_s"] / p["throughput_req_per_s"],
            "ion_steps_ratio_server_vs_plain": s["ion_steps_per_s"] / p["ion_steps_per_s"],
            "rel_err_vs_plain": {"q_max": max(dq), "force_max": max(df),
                                 "force_median": float(np.median(df))},
            "results_equal_bitwise": bool(eq),
            "force_every": {str(k): ks.count(k) for k in sorted(set(ks))},
            "n_ions": [int(r.sim.N) for r in reqs],
            "config": {"workload": f"serve: Poisson {args.rate}/s for {args.duration} s, N log-uniform "
                                   f"2^{lo:g}-2^{hi:g}, 1-8 grains, Mach 0.1-2, Maxwellian or "
                                   f"field-driven, {args.window}-step windows (averages over the "
                                   f"second half), 80% HBM budget; host setup in an 8-process pool "
                                   f"for both arms",
                       "served": "every step" if args.serve_exact else
                                 "ion-ion force interval by size (serve.interval_by_size)"}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    dist = Dist("gloo" if args.impl == "reference" else "nccl")
    try:
        if args.workload in ("sweep", "serve") and args.impl == "ours":
            return run_sweep(args, dist) if args.workload == "sweep" else run_serve(args, dist)
        rc = run_reference(args, dist) if args.impl == "reference" else run_ours(args, dist)
    finally:
        dist.close()
    return rc


if __name__ == "__main__":
    sys.exit(main())
