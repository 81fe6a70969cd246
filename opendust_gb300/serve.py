"""Continuous-batching request server for force/charge solves.

A request is one simulation (plasma, domain, grains, seed) to run for a fixed window of steps;
its answer is the time-averaged grain charge and forces over the second half of the window
(the steady-state window) and the per-step series. The server keeps every admitted request's
ion state resident on the GPU as a member of one ``od_batch`` and steps all members together;
between chunks of steps it admits arrived requests while the device-memory budget allows and
retires members whose window is complete. The host part of a request's setup (injection
tables; the initial state of field-driven requests) runs in a worker process pool, overlapping
the GPU steps; the trap fit and Maxwellian initial states run on the GPU when the request is
admitted.

``run_plain`` is the baseline: the same requests served one at a time through the plain
single-simulation path, in arrival order.

There is no counterpart in the reference, which runs one simulate() per parameter point
(e.g. examples/Piel2017/Figure5/launchPiel2017Figure5.py:32-106).
"""
from __future__ import annotations

import ctypes
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from . import _lib, setup_host
from .opendust import build_simulation


@dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the run
    plasma: object
    sim: object
    grains: list
    dist: str
    ext: dict
    seed: int
    window: int             # steps
    done: float | None = None
    averages: np.ndarray | None = None
    series: dict | None = field(default=None, repr=False)


def host_prepare(req: Request):
    """CPU part of a request's setup (picklable): injection tables and, for field-driven
    requests, the initial ion state (Maxwellian ones are sampled on the device)."""
    inj = setup_host.injection_setup(req.plasma.v_fl, req.plasma.v_T, req.sim.R, req.sim.H, req.dist)
    if req.dist == "Maxwellian":
        return inj, None, None
    pos, vel = setup_host.initial_state(req.sim.N, req.sim.R, req.sim.H,
                                        [(g.x, g.y, g.z, g.r) for g in req.grains],
                                        req.plasma.v_fl, req.plasma.v_T, req.dist, req.seed)
    return inj, pos, vel


def finish_prepare(req: Request, host, device: int = 0):
    """GPU part (trap fit) and the od_config; returns (holder, pos, vel)."""
    inj, pos, vel = host
    holder, _ = build_simulation(req.plasma, req.sim, req.grains, req.dist, seed=req.seed,
                                 device=device, n_steps=req.window, avg_start=req.window // 2,
                                 injection=inj, **req.ext)
    return holder, pos, vel


def prepare(req: Request, device: int = 0):
    """Whole setup of one request, in this process."""
    return finish_prepare(req, host_prepare(req), device)


def start_pool(workers: int = 8):
    """Process pool for host_prepare; uses 'spawn' so that workers never inherit a CUDA context.
    Start it before the first GPU call."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    return ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn"))


def device_memory(device: int = 0):
    """(free, total) bytes of the device."""
    lib = _lib.load()
    free, total = ctypes.c_int64(), ctypes.c_int64()
    _lib.check(lib.od_device_memory(int(device), ctypes.byref(free), ctypes.byref(total)), None)
    return free.value, total.value


def interval_by_size(N: int) -> int:
    """Ion–ion force interval for a served request of N ions: 8 from 2^16 ions, 4 from 2^15,
    every step below (where the pair work no longer dominates the step). The rule follows the
    pilot-window tuning of the sweep (tuning.choose_force_interval, 1 % bound on the grains'
    time-averaged charge and ion force); the served results are compared with the plain path's
    per request."""
    return 8 if N >= 2**16 else (4 if N >= 2**15 else 1)


class Server:
    def __init__(self, device: int = 0, budget_frac: float = 0.8, chunk: int = 25,
                 max_members: int = 512, interval=None):
        """interval: None (every step, the reference's integrator) or a function N -> force
        interval k (od_config.force_every), e.g. interval_by_size."""
        self.device = device
        self.chunk = chunk
        self.max_members = max_members
        self.interval = interval
        free, total = device_memory(device)
        self.budget = int(budget_frac * total) - (total - free)  # of what is free now

    def run(self, requests: list[Request], pool=None) -> dict:
        """Serve the requests (arrival times relative to now). pool: a process pool from
        start_pool() for the host part of each request's setup (else a thread)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        own = pool is None
        if own:
            pool = ThreadPoolExecutor(max_workers=1)
        futures = {r.rid: pool.submit(host_prepare, r) for r in reqs}
        batch = _lib.Batch(self.device)
        live = {}          # slot -> (request, bytes)
        used = 0
        pending = list(reqs)
        t0 = time.perf_counter()
        gpu_ms = 0.0
        steps_done = 0
        try:
            while pending or live:
                now = time.perf_counter() - t0
                # admit arrived requests while the budget and slots allow
                while pending and pending[0].arrival <= now and len(live) < self.max_members:
                    r = pending[0]
                    if not futures[r.rid].done() and live:
                        break  # its host setup is still running: keep stepping the others
                    holder, pos, vel = finish_prepare(r, futures[r.rid].result(), self.device)
                    if self.interval is not None:
                        holder.cfg.force_every = int(self.interval(int(r.sim.N)))
                    need = _lib.config_device_bytes(holder)
                    if live and used + need > self.budget:
                        break
                    slot = batch.add(holder, pos, vel)
                    live[slot] = (r, need, holder)
                    used += need
                    pending.pop(0)
                if not live:
                    wait = pending[0].arrival - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(wait)
                    continue
                remaining = min(r.window - batch.member(s).step_index for s, (r, _, _) in live.items())
                k = max(1, min(self.chunk, remaining))
                batch.step(k)
                gpu_ms += batch.last_step_ms()
                steps_done += k
                for s in list(live):
                    r, need, holder = live[s]
                    m = batch.member(s)
                    if m.step_index >= r.window:
                        r.averages, _ = m.averages()
                        r.series = m.series(0, r.window)
                        r.done = time.perf_counter() - t0
                        batch.remove(s)
                        used -= need
                        del live[s]
        finally:
            batch.close()
            if own:
                pool.shutdown(wait=True)
        wall = time.perf_counter() - t0
        return summarize(reqs, wall, gpu_ms)


def run_plain(requests: list[Request], device: int = 0, batch_plan: bool = False,
              pool=None, interval=None) -> dict:
    """Baseline: the same requests, one at a time through the single-simulation path (its
    default all-pairs plan, or with batch_plan the plan the server's batch gives each request,
    so that results are bitwise comparable). pool: the server's process pool, so that the host
    part of every request's setup overlaps the GPU work here as it does in the server.
    interval: as Server's (None: every step)."""
    reqs = sorted(requests, key=lambda r: r.arrival)
    futures = {r.rid: pool.submit(host_prepare, r) for r in reqs} if pool is not None else None
    t0 = time.perf_counter()
    gpu_ms = 0.0
    for r in reqs:
        wait = r.arrival - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        if futures is not None:
            holder, pos, vel = finish_prepare(r, futures[r.rid].result(), device)
        else:
            holder, pos, vel = prepare(r, device)
        if interval is not None:
            holder.cfg.force_every = int(interval(int(r.sim.N)))
        with _lib.Engine(holder, device) as eng:
            if batch_plan:
                eng.set_pair_plan(*_lib.batch_pair_plan(r.sim.N))
            if pos is None:
                eng.init_state()
            else:
                eng.set_state(pos, vel)
            t1 = time.perf_counter()
            eng.step(r.window)
            gpu_ms += (time.perf_counter() - t1) * 1e3
            r.averages, _ = eng.averages()
            r.series = eng.series(0, r.window)
        r.done = time.perf_counter() - t0
    wall = time.perf_counter() - t0
    return summarize(reqs, wall, gpu_ms)


def summarize(reqs, wall, gpu_ms) -> dict:
    lat = np.array([r.done - r.arrival for r in reqs])
    ion_steps = sum(r.sim.N * r.window for r in reqs)
    return {"requests": len(reqs), "wall_s": wall, "gpu_ms": gpu_ms,
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "throughput_req_per_s": len(reqs) / wall, "ion_steps_per_s": ion_steps / wall}


def poisson_requests(rate: float, duration: float, seed: int, log2n=(14, 16), window: int = 50,
                     max_grains: int = 8):
    """Poisson arrivals at `rate` per second for `duration` seconds; each request draws from its
    seed: N log-uniform over 2^log2n, 1..max_grains grains on an axial chain, Mach 0.1-2,
    Maxwellian or field-driven inflow."""
    from . import workloads

    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    rid = 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        N = int(round(2 ** rng.uniform(*log2n)))
        P = int(rng.integers(1, max_grains + 1))
        M = float(rng.uniform(0.1, 2.0))
        if rng.uniform() < 0.5:
            plasma = workloads.PlasmaParametersInSIUnitsMaxwell(workloads.T_I, workloads.T_E, workloads.N_INF, M,
                                                                workloads.M_AR)
            dist, ext = "Maxwellian", {}
        else:
            k_B = 1.380649e-23
            v_B = np.sqrt(k_B * workloads.T_E / workloads.M_AR)
            v_T = np.sqrt(k_B * workloads.T_I / workloads.M_AR)
            lam = np.sqrt(8.85418781762039e-12 * k_B * workloads.T_E / ((1.60217662e-19) ** 2 * workloads.N_INF))
            v_fl = M * v_B
            w_c = np.sqrt(v_fl**2 + 8 * v_T**2 / np.pi) / (2 * lam)
            E = v_fl * workloads.M_AR * w_c / 1.60217662e-19
            plasma = workloads.PlasmaParametersInSIUnitsFieldDriven(workloads.T_I, workloads.T_E, workloads.N_INF,
                                                                    E, w_c, workloads.M_AR)
            dist, ext = "fieldDriven", {}
        lam = plasma.r_D_e
        sim = workloads.SimulationParametersInSIUnits(3 * lam, 6 * lam, N, window, 1e-10, plasma)
        zs = (np.arange(P) - (P - 1) / 2.0) * 0.6 * lam
        grains = [workloads.DustParticle(0.0, 0.0, z, 5e-6, "consistent", 0.0) for z in zs]
        out.append(Request(rid, t, plasma, sim, grains, dist, ext, seed * 100003 + rid, window))
        rid += 1
    return out
