"""Cell-relative position state (od_set_state / od_get_state, od_rel_* in od_common.cuh): each
ion's position is a cell index on a grid of side s (a power of two, 1/256 to 1/128 of the
domain's half extent) plus an FP32 offset in that cell, so the drift keeps 24 bits below the
cell size wherever the ion is; the force kernels read the absolute FP32 position derived from
it once per step.

  * set_state -> get_state returns every coordinate within half an FP32 ulp of the cell size
    (an absolute FP32 position is only good to half an ulp of |x|);
  * trajectories against the FP64 oracle started from the unrounded state: the positions after
    40 steps (2048 ions) and after the reference cutoff script's 3 steps on a 12 lambda high
    domain stay within the bounds below, set from the measured errors with a margin; with FP32
    absolute positions the rounding of every drift alone is up to half an ulp of |x| per step.
"""
import numpy as np
import pytest

from opendust_gb300 import _lib, build_simulation, setup_host, workloads
from oracle import oracle
from tests._util import case

pytestmark = pytest.mark.gpu


def _cell(lam_units_half_extent):
    return 2.0 ** np.ceil(np.log2(lam_units_half_extent / 256.0))


def test_state_roundtrip_within_cell_ulp(gpu_lib):
    holder, pos, vel, plasma, sim, grains = case(N=4096, n=4, seed=51)
    lam = plasma.r_D_e
    s = _cell(max(sim.R, sim.H / 2) / lam)
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        p2, v2 = eng.get_state()
    err = np.max(np.abs(p2 - pos)) / lam
    err32 = np.max(np.abs(pos / lam - (pos / lam).astype(np.float32)))
    print(f"state roundtrip: max |dx| {err:.3e} lambda (cell {s}, FP32 absolute {err32:.3e})")
    assert err <= s * 2.0**-24 * 1.0001
    assert err < err32 / 4


def _traj_err(holder, pos, vel, steps, lam):
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(steps)
        p, _ = eng.get_state()
    ref = oracle.run(holder, pos, vel, 0, steps, round32=False)
    return np.max(np.abs(p - ref["pos"])) / lam


def test_trajectory_against_fp64_oracle(gpu_lib):
    holder, pos, vel, plasma, sim, grains = case(N=2048, n=40, seed=52)
    err = _traj_err(holder, pos, vel, 40, plasma.r_D_e)
    print(f"40 steps, 2048 ions, FP64 initial state: max |dx| {err:.3e} lambda")
    assert err < 1e-5


def test_tall_domain_against_fp64_oracle(gpu_lib):
    plasma, sim, grains, d, ext = workloads.cutoff_scaling(k=2, n=3)
    holder, _ = build_simulation(plasma, sim, grains, d, seed=53, **ext)
    pos, vel = setup_host.initial_state(sim.N, sim.R, sim.H, [(g.x, g.y, g.z, g.r) for g in grains],
                                        plasma.v_fl, plasma.v_T, d, 53)
    err = _traj_err(holder, pos, vel, 3, plasma.r_D_e)
    print(f"reference cutoff script k=2 (H = 12 lambda), 3 steps: max |dx| {err:.3e} lambda")
    assert err < 1e-5
