"""Cell-relative position state (od_set_state / od_get_state, od_rel_* in od_common.cuh): each
ion's position is a cell index on a grid of side s (a power of two, 1/256 to 1/128 of the
domain's half extent) plus an FP32 offset in that cell, so the drift keeps 24 bits below the
cell size wherever the ion is; the force kernels read the absolute FP32 position derived from
it once per step.

  * set_state -> get_state returns every coordinate within half an FP32 ulp of the cell size
    (an absolute FP32 position is only good to half an ulp of |x|);
  * trajectories against the FP64 oracle started from the device's exact state: the positions
    of the ions that were not re-injected, after 40 steps (2048 ions) and after the reference
    cutoff script's 3 steps on a 12 lambda high domain, stay within the bounds below (measured
    errors with a margin), below what a single rounding of an FP32 absolute position can
    lose.
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
    """Max |dx| / lambda against the oracle started from the device's exact state: over all ions,
    and over the ions that neither run re-injected (both moved less than 0.05 lambda; a
    re-injected ion restarts from a float position drawn in FP32 on the device and in FP64 in
    the oracle)."""
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(steps)
        p, _ = eng.get_state()
    ref = oracle.run(holder, pos, vel, 0, steps, round32=oracle.DEVICE_STATE)
    d = np.max(np.abs(p - ref["pos"]), axis=1) / lam
    stay = (np.linalg.norm(p - pos, axis=1) < 0.05 * lam) & \
           (np.linalg.norm(ref["pos"] - pos, axis=1) < 0.05 * lam)
    return d.max(), d[stay].max(), int(stay.sum())


def test_trajectory_against_fp64_oracle(gpu_lib):
    holder, pos, vel, plasma, sim, grains = case(N=2048, n=40, seed=52)
    err, err_stay, n_stay = _traj_err(holder, pos, vel, 40, plasma.r_D_e)
    print(f"40 steps, 2048 ions: max |dx| {err:.3e} lambda; {n_stay} ions not re-injected "
          f"{err_stay:.3e}")
    assert n_stay > 1800
    assert err < 1e-5
    # measured 2.0e-8 (a single FP32 absolute rounding at |x| = 3 lambda is up to 1.2e-7)
    assert err_stay < 6e-8


def test_tall_domain_against_fp64_oracle(gpu_lib):
    plasma, sim, grains, d, ext = workloads.cutoff_scaling(k=2, n=3)
    holder, _ = build_simulation(plasma, sim, grains, d, seed=53, **ext)
    pos, vel = setup_host.initial_state(sim.N, sim.R, sim.H, [(g.x, g.y, g.z, g.r) for g in grains],
                                        plasma.v_fl, plasma.v_T, d, 53)
    err, err_stay, n_stay = _traj_err(holder, pos, vel, 3, plasma.r_D_e)
    print(f"reference cutoff script k=2 (H = 12 lambda), 3 steps: max |dx| {err:.3e} lambda; "
          f"{n_stay} ions not re-injected {err_stay:.3e}")
    assert err < 1e-5
    # measured 6.3e-8 (a single FP32 absolute rounding at |z| = 6 lambda is up to 2.4e-7)
    assert err_stay < 1.5e-7
