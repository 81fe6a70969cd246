"""Shared helpers for the test suite (seeded synthetic inputs)."""
from __future__ import annotations

import numpy as np

from opendust_gb300 import build_simulation, setup_host, workloads


def oracle_trap(n_points_cap: int = 200_000):
    """Trap-potential callable backed by the CPU oracle with a capped sample count."""
    from oracle import oracle

    def f(Rh, Hh, n_r, n_h, n_points, seed):
        return oracle.trap_potential(Rh, Hh, n_r, n_h, min(n_points, n_points_cap), seed)

    return f


def case(N=2048, n=16, seed=3, trap=None, builder=workloads.small_plain, state_seed=None, q0=-2e-15,
         **kw):
    """(holder, pos, vel, plasma, sim, grains) for a small seeded case; grains start at charge q0
    (non-zero, so that the orbit force of the first step is non-zero)."""
    plasma, sim, grains, dist, ext = builder(N=N, n=n)
    for g in grains:
        g.q = q0
    ext = {**ext, **kw}
    holder, info = build_simulation(plasma, sim, grains, dist, seed=seed, trap=trap, **ext)
    pos, vel = setup_host.initial_state(sim.N, sim.R, sim.H, [(g.x, g.y, g.z, g.r) for g in grains],
                                        plasma.v_fl, plasma.v_T, dist,
                                        seed if state_seed is None else state_seed)
    return holder, pos, vel, plasma, sim, grains


def rel_err_per_ion(f, ref, floor_frac=0.0):
    """|f - ref| / max(|ref|, floor_frac * rms|ref|) per ion."""
    nr = np.linalg.norm(ref, axis=1)
    floor = floor_frac * np.sqrt(np.mean(nr**2))
    return np.linalg.norm(f - ref, axis=1) / np.maximum(nr, floor)


def plant_close_pairs(pos, lam, rng, n_pairs=16, dmin=1e-3, dmax=5e-2):
    """Move pairs of ions to within [dmin, dmax] lambda of each other."""
    p = pos.copy()
    for k in range(n_pairs):
        i, j = 2 * k + 100, 2 * k + 101
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        p[j] = p[i] + d * lam * 10 ** rng.uniform(np.log10(dmin), np.log10(dmax))
    return p
