"""Accuracy-bounded choice between the all-pairs and the cutoff ion–ion force.

The reference leaves the choice to the user (``simulate(cutOff=...)``, opendust.py:469-485): a
cutoff truncates the screened potential, so it changes the physics, and how much depends on the
density and the domain. ``choose_force_method`` makes the choice measurable: on the caller's
own ion snapshot it evaluates the all-pairs force and the cutoff force at each candidate cutoff
(OpenMM's switching from 15/16 of it, as the reference's 3.0/3.2 lambda), times a few steps of
each on the GPU, and returns the fastest method whose force error stays within the given bound.

The error is the global relative error of the ion–ion force on the snapshot,
sqrt(sum |F_cut - F_all|^2 / sum |F_all|^2). It is a proxy: what a study needs to bound is the
error of the time-averaged grain charge and force, which the snapshot error bounds only loosely
(the orbit force is a sum over ions; the ion–ion force enters it through the trajectories). With
max_rel_err = 0 the answer is always the all-pairs force.
"""
from __future__ import annotations

import numpy as np

from . import _lib


def _variant(holder: _lib.ConfigHolder, rc: float | None, n_steps: int) -> _lib.ConfigHolder:
    cfg = _lib.od_config.from_buffer_copy(holder.cfg)
    if rc is None:
        cfg.force_method = _lib.OD_FORCE_ALLPAIRS
        cfg.cutoff = cfg.switch_dist = 0.0
    else:
        cfg.force_method = _lib.OD_FORCE_CUTOFF
        cfg.cutoff = rc
        cfg.switch_dist = rc * (3.0 / 3.2)
    cfg.n_steps = n_steps
    cfg.avg_start = 0
    return _lib.ConfigHolder(cfg, holder._keep)


def _measure(holder, rc, pos, vel, steps, device):
    with _lib.Engine(_variant(holder, rc, steps + 2), device) as eng:
        f = eng.force_snapshot(pos)
        eng.set_state(pos, vel)
        eng.step(1)
        eng.set_timing(True, count_pairs=False)
        eng.step(steps)
        step_ms, n, _, _ = eng.timing()
        eng.set_timing(False)
        plan = eng.pair_plan()
    return f, step_ms / max(n, 1), plan


def choose_force_method(holder: _lib.ConfigHolder, pos: np.ndarray, vel: np.ndarray,
                        max_rel_err: float = 1e-2, cutoffs_lambda=(2.0, 3.0, 4.0),
                        steps: int = 2, device: int = 0) -> dict:
    """Fastest force method whose snapshot error is within max_rel_err.

    holder: the simulation's configuration (build_simulation); pos, vel: an ion state in SI
    units (N x 3), e.g. the initial state or one taken from a running simulation.
    cutoffs_lambda: candidate cutoffs in units of r_D_e.
    Returns {"method": "allpairs" | "cutoff", "cutoff": r_c in m or None, "rel_err": e,
    "step_ms": t, "candidates": [{"cutoff", "rel_err", "step_ms", "plan"}, ...]}.
    """
    lam = float(holder.cfg.r_D_e)
    f_all, t_all, plan_all = _measure(holder, None, pos, vel, steps, device)
    norm = float(np.sqrt(np.sum(f_all ** 2)))
    cands = [{"cutoff": None, "rel_err": 0.0, "step_ms": t_all, "plan": plan_all}]
    for c in cutoffs_lambda:
        rc = float(c) * lam
        f, t, plan = _measure(holder, rc, pos, vel, steps, device)
        err = float(np.sqrt(np.sum((f - f_all) ** 2))) / norm
        cands.append({"cutoff": rc, "rel_err": err, "step_ms": t, "plan": plan})
    ok = [c for c in cands if c["rel_err"] <= max_rel_err]
    best = min(ok, key=lambda c: c["step_ms"])
    return {"method": "allpairs" if best["cutoff"] is None else "cutoff", "cutoff": best["cutoff"],
            "rel_err": best["rel_err"], "step_ms": best["step_ms"], "candidates": cands}


def _averages(holder, k, pos, vel, steps, device):
    cfg = _lib.od_config.from_buffer_copy(holder.cfg)
    cfg.force_every = int(k)
    cfg.n_steps = steps
    cfg.avg_start = steps // 2
    with _lib.Engine(_lib.ConfigHolder(cfg, holder._keep), device) as eng:
        eng.set_state(pos, vel)
        eng.set_timing(True, count_pairs=False)
        eng.step(steps)
        step_ms, n, _, _ = eng.timing()
        eng.set_timing(False)
        avg, _ = eng.averages()
    return avg, step_ms / max(n, 1)


def interval_errors(avg, ref) -> dict:
    """Relative errors of time averages (rows of od_get_averages: q, orbit, collect, dust,
    field) against a reference run: charge max_p |dq_p|/|q_p|; ion force (orbit + collect) as
    one norm over the grains, |dF| / |F|."""
    dq = float(np.max(np.abs(avg[:, 0] - ref[:, 0]) / np.maximum(np.abs(ref[:, 0]), 1e-300)))
    f = avg[:, 1:4] + avg[:, 4:7]
    fr = ref[:, 1:4] + ref[:, 4:7]
    df = float(np.linalg.norm(f - fr) / max(np.linalg.norm(fr), 1e-300))
    return {"q": dq, "force": df}


def choose_force_interval(holder: _lib.ConfigHolder, pos: np.ndarray, vel: np.ndarray,
                          max_rel_err: float = 1e-2, intervals=(2, 4, 8, 16),
                          pilot_steps: int = 100, device: int = 0) -> dict:
    """Largest ion–ion force interval k (od_config.force_every) whose error on the grains'
    time-averaged charge and ion force stays within max_rel_err on a pilot window.

    The pilot runs pilot_steps steps from the caller's state (pos, vel in SI units) with k = 1
    (the reference's integrator) and with each candidate k; every run uses the same seed, so
    the Philox streams of collisions and re-injection are the same and the runs differ only by
    the integrator. Errors are those of interval_errors over the window's second half. The
    search stops at the first candidate that fails (errors grow with k).
    Returns {"force_every": k, "errors": {...}, "step_ms": t, "candidates": [...]}.
    """
    ref, t1 = _averages(holder, 1, pos, vel, pilot_steps, device)
    best = {"force_every": 1, "errors": {"q": 0.0, "force": 0.0}, "step_ms": t1}
    cands = [dict(best)]
    for k in sorted(int(x) for x in intervals):
        if k <= 1:
            continue
        avg, t = _averages(holder, k, pos, vel, pilot_steps, device)
        err = interval_errors(avg, ref)
        c = {"force_every": k, "errors": err, "step_ms": t}
        cands.append(c)
        if max(err.values()) > max_rel_err:
            break
        best = c
    return {**best, "candidates": cands}


# ---------------------------------------------------------------- persisted plan choices
# Plans chosen by measurement are kept per (GPU model, size bucket) in a JSON file, so that a
# later process (a sweep, a server) reuses them without timing again. The bucket of N ions is
# round(2 log2 N) / 2: half-octave classes.

def plan_cache_path() -> str:
    import os

    return os.environ.get("OD_PLAN_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "opendust_gb300", "plans.json")


def size_bucket(n: int) -> float:
    return round(2.0 * np.log2(max(int(n), 2))) / 2.0


def gpu_model(device: int = 0) -> str:
    try:
        import torch

        return torch.cuda.get_device_name(device)
    except Exception:  # no torch / no device name: one class for every GPU
        return "gpu"


class PlanCache:
    """{key: plan} in a JSON file; key = "<kind>|<GPU model>|<size bucket>"."""

    def __init__(self, path: str | None = None):
        import json
        import os

        self.path = path or plan_cache_path()
        self.data = {}
        if os.path.exists(self.path):
            try:
                with open(self.path) as f:
                    self.data = json.load(f)
            except (OSError, ValueError):
                self.data = {}

    @staticmethod
    def key(kind: str, model: str, n: int) -> str:
        return f"{kind}|{model}|{size_bucket(n):g}"

    def get(self, kind, model, n):
        v = self.data.get(self.key(kind, model, n))
        return tuple(v) if v is not None else None

    def put(self, kind, model, n, plan):
        import json
        import os

        self.data[self.key(kind, model, n)] = list(plan)
        os.makedirs(os.path.dirname(self.path) or ".", exist_ok=True)
        tmp = self.path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def tuned_plan(eng: _lib.Engine, device: int = 0, cache: PlanCache | None = None) -> tuple:
    """The autotuner's all-pairs plan for this engine's size, from the persisted cache or, on a
    miss, by od_autotune on the engine's current positions (then stored). Applies it."""
    cache = cache or PlanCache()
    model = gpu_model(device)
    plan = cache.get("single", model, eng.n)
    if plan is None:
        eng.autotune(use_cache=False)
        p = eng.pair_plan()
        plan = (p["threads"], p["targets_per_thread"], p["variant"], p["jsplit"])
        cache.put("single", model, eng.n, plan)
    eng.set_pair_plan(*plan)
    return plan


BATCH_SHAPES = ((4, 1024), (8, 2048))


def batch_plan_for(n: int, device: int = 0, cache: PlanCache | None = None,
                   time_plan=None) -> tuple:
    """Each-pair-once shape (ions per lane, tile) for a batch member of n ions, chosen per size
    bucket by timing both batch shapes on a member-sized simulation; persisted. time_plan(n,
    shape) -> ms per evaluation (default: two timed steps of a small_plain simulation)."""
    cache = cache or PlanCache()
    model = gpu_model(device)
    plan = cache.get("batch", model, n)
    if plan is not None:
        return plan
    time_plan = time_plan or (lambda nn, sh: _time_batch_shape(nn, sh, device))
    best = min(BATCH_SHAPES, key=lambda sh: time_plan(n, sh))
    cache.put("batch", model, n, best)
    return best


def _time_batch_shape(n: int, shape, device: int) -> float:
    from . import build_simulation, workloads

    plasma, sim, grains, dist, ext = workloads.small_plain(N=int(n), n=8)
    holder, _ = build_simulation(plasma, sim, grains, dist, seed=1, device=device, **ext)
    with _lib.Engine(holder, device) as eng:
        eng.set_pair_plan(256, shape[0], 7, shape[1])
        eng.init_state()
        eng.step(1)
        eng.set_timing(True, count_pairs=False)
        eng.step(3)
        _, _, pair_ms, launches = eng.timing()
        eng.set_timing(False)
    return pair_ms / max(launches, 1)
