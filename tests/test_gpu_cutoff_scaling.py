"""GPU tests at the reference's own cutoff benchmark configuration
(performance/CutOff-Performance/benchmark.py:14-75 with simulate(cutOff=True): N = k*2^15 ions in
a cylinder of radius 3 lambda and height k*6 lambda, cutoff 3.2 lambda with OpenMM's switching
from 3.0 lambda, one grain of given charge, d_t = 3.5148e-9 s, 3 steps).

  * forces on 2048 random targets against the FP64 oracle over all sources at k = 1 and k = 8;
    the switched force goes to zero smoothly at r_c, so the bound is the all-pairs one: per-ion
    relative error <= 1e-5;
  * the reference script's 3 steps at k = 1 against the oracle's run (positions, velocities and
    the per-step grain series), and the number of pairs inside the cutoff against a KD-tree
    count.
"""
import numpy as np
import pytest

from opendust_gb300 import _lib, build_simulation, setup_host, workloads
from oracle import oracle
from tests._util import rel_err_per_ion

pytestmark = pytest.mark.gpu


def _scaling_case(k, seed, n=3):
    plasma, sim, grains, d, ext = workloads.cutoff_scaling(k=k, n=n)
    holder, _ = build_simulation(plasma, sim, grains, d, seed=seed, **ext)
    pos, vel = setup_host.initial_state(sim.N, sim.R, sim.H, [(g.x, g.y, g.z, g.r) for g in grains],
                                        plasma.v_fl, plasma.v_T, d, seed)
    return holder, pos, vel, plasma, sim


@pytest.mark.parametrize("k", [1, 8])
def test_reference_cutoff_config_snapshot(gpu_lib, k):
    holder, pos, vel, plasma, sim = _scaling_case(k, 30 + k)
    lam = plasma.r_D_e
    assert holder.cfg.force_method == _lib.OD_FORCE_CUTOFF
    assert holder.cfg.cutoff == pytest.approx(3.2 * lam)
    assert holder.cfg.switch_dist == pytest.approx(3.0 * lam)
    assert sim.N == k * 2**15 and sim.H == pytest.approx(6 * k * lam)
    with _lib.Engine(holder) as eng:
        assert eng.pair_plan()["variant"] == 3
        f = eng.force_snapshot(pos)
    idx = np.sort(np.random.default_rng(k).choice(sim.N, 2048, replace=False))
    ref = oracle.force_targets(holder, pos, idx, round32=True)
    err = rel_err_per_ion(f[idx], ref)
    print(f"reference cutoff config k={k} (N={sim.N}): per-ion rel err max {err.max():.3e} "
          f"p99 {np.quantile(err, 0.99):.3e}")
    assert err.max() <= 1e-5


def test_reference_cutoff_script_three_steps(gpu_lib):
    spatial = pytest.importorskip("scipy.spatial")
    holder, pos, vel, plasma, sim = _scaling_case(1, 41, n=4)  # 3 steps + 1 counted step
    lam = plasma.r_D_e
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(3)
        s = eng.series(0, 3)
        p, v = eng.get_state()
        eng.set_state(pos, vel)
        eng.set_timing(True, count_pairs=True)
        eng.step(1)
        pairs = eng.cutoff_pairs()
        eng.set_timing(False)
        p1, _ = eng.get_state()
    ref = oracle.run(holder, pos, vel, 0, 3, round32=True)
    dpos = np.max(np.abs(p - ref["pos"])) / lam
    dvel = np.max(np.abs(v - ref["vel"])) / plasma.v_T
    assert np.all(s["q"] == ref["q"])  # given charge: held at its value
    do = np.max(np.linalg.norm(s["orbit"] - ref["orbit"], axis=-1) / np.linalg.norm(ref["orbit"], axis=-1))
    print(f"reference cutoff script k=1, 3 steps: max |dx| {dpos:.3e} lambda, max |dv| {dvel:.3e} v_T, "
          f"orbit rel {do:.3e}, pairs {pairs}")
    assert dpos < 1e-5
    assert dvel < 1e-3
    assert do < 1e-3
    # directed pairs inside r_c at the positions the first step evaluates (after its drift)
    tree = spatial.cKDTree(p1 / lam)
    approx = tree.count_neighbors(tree, holder.cfg.cutoff / lam) - sim.N
    assert abs(pairs - approx) / approx < 0.01
