"""Generate tests/golden/c1_oracle.npz: the small_plain workload (N = 16384 superions, 2000 steps,
d_t = 1e-10 s, one self-consistently charging grain) run in full by the FP64 CPU oracle.

The fixture holds the trap coefficients and the initial state it used (so the GPU run in
tests/test_gpu_golden_c1.py starts from identical inputs) and the oracle's per-step grain charge
and forces. Runtime: about an hour on 8 cores (two all-pairs evaluations per step in FP64).

Usage: python tests/golden/make_c1_fixture.py [threads]
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from opendust_gb300 import build_simulation, setup_host, workloads  # noqa: E402
from oracle import oracle  # noqa: E402

SEED = 0


def inputs():
    """The fixture's configuration (trap from the FP64 oracle grid) and initial state."""
    plasma, sim, grains, dist, ext = workloads.small_plain()
    Rh, Hh, n_r, n_h, n_points = setup_host.trap_grid(sim.R, sim.H, plasma.r_D_e)
    pot = oracle.trap_potential(Rh, Hh, n_r, n_h, n_points, 12345)
    alpha = setup_host.fit_trap(pot, Rh, Hh, sim.N)
    holder, _ = build_simulation(plasma, sim, grains, dist, seed=SEED, trap=alpha, **ext)
    pos, vel = setup_host.initial_state(sim.N, sim.R, sim.H, [(g.x, g.y, g.z, g.r) for g in grains],
                                        plasma.v_fl, plasma.v_T, dist, SEED)
    return plasma, sim, grains, dist, ext, alpha, holder, pos, vel


def main():
    if len(sys.argv) > 1:
        oracle.set_threads(int(sys.argv[1]))
    plasma, sim, grains, dist, ext, alpha, holder, pos, vel = inputs()
    t0 = time.time()
    r = oracle.run(holder, pos, vel, 0, sim.n, round32=True)
    dt = time.time() - t0
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c1_oracle.npz")
    np.savez_compressed(out, alpha=alpha, pos0=pos, vel0=vel, q=r["q"], orbit=r["orbit"],
                        collect=r["collect"], dust=r["dust"], n_inj=r["n_inj"], dN=r["dN"],
                        seconds=dt, threads=oracle.max_threads())
    print(f"wrote {out} in {dt:.0f} s")


if __name__ == "__main__":
    main()
