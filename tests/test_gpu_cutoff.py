"""GPU tests of the cutoff force path against the CPU oracle: variants 0 and 2 walk a stencil
of cells per target cell; variant 3 (the default) sorts the ions along a Hilbert curve and
evaluates each unordered pair once over tile pairs whose bounding boxes come within r_c.

Tolerances:
  * with OpenMM's switching polynomial (the reference's cutOff=True: cutoff 3.2 lambda, switch
    from 3.0 lambda) the pair force goes to zero smoothly at the cutoff, so FP32 and FP64 may
    disagree on the inclusion of a pair at r = r_c without changing the force: per-ion relative
    error <= 1e-5, as for all pairs;
  * with a hard cutoff (no switching) a pair within rounding of r_c can be included on one side
    only; the bound is 1e-5 for 99.9 % of ions and 1e-3 for all.
"""
import numpy as np
import pytest

from opendust_gb300 import _lib, workloads
from oracle import oracle
from tests._util import case, plant_close_pairs, rel_err_per_ion

pytestmark = pytest.mark.gpu


def _cut_case(N, seed, **kw):
    return case(N=N, n=4, seed=seed, **kw)


# 3: 1024-ion tiles with 4 x 4 targets x sources per lane (staggered tile pairs); 32: 512-ion
# tiles with 2 x 2 (balanced group-pair lists, the default)
PLANS = {0: (128, 1, 0), 2: (128, 1, 2), 3: (256, 4, 3), 32: (256, 2, 3)}


@pytest.mark.parametrize("variant", [0, 2, 3, 32])
def test_cutoff_switching_snapshot(gpu_lib, variant):
    holder, pos, vel, plasma, sim, grains = _cut_case(4096, 21, cutOff=True)
    assert holder.cfg.force_method == _lib.OD_FORCE_CUTOFF
    pos = plant_close_pairs(pos, plasma.r_D_e, np.random.default_rng(3), n_pairs=32, dmin=2e-4)
    with _lib.Engine(holder) as eng:
        eng.set_pair_plan(*PLANS[variant])
        assert eng.pair_plan()["variant"] == PLANS[variant][2]
        f = eng.force_snapshot(pos)
    ref = oracle.force_snapshot(holder, pos, round32=True)
    err = rel_err_per_ion(f, ref)
    print(f"variant {variant} cutoff 3.2/3.0: per-ion rel err max {err.max():.3e} p99 {np.quantile(err, 0.99):.3e}")
    assert err.max() <= 1e-5


@pytest.mark.parametrize("N,variant", [(4096, 0), (4096, 2), (2**17, 2), (4096, 3), (2**17, 3),
                                       (2**17, 32), (4096, 32)])
def test_cutoff_hard_snapshot_and_pair_count(gpu_lib, N, variant):
    spatial = pytest.importorskip("scipy.spatial")
    holder, pos, vel, plasma, sim, grains = case(N=N, n=4, seed=22, builder=workloads.field_chain,
                                                 switch_distance=0.0)
    assert holder.cfg.switch_dist == 0.0
    with _lib.Engine(holder) as eng:
        eng.set_pair_plan(*PLANS[variant])
        f = eng.force_snapshot(pos)
        eng.set_state(pos, vel)
        eng.set_timing(True)
        eng.step(1)
        pairs = eng.cutoff_pairs()
        eng.set_timing(False)
    idx = np.arange(N) if N <= 4096 else np.sort(np.random.default_rng(0).choice(N, 2048, replace=False))
    ref = oracle.force_targets(holder, pos, idx, round32=True)
    err = rel_err_per_ion(f[idx], ref)
    print(f"variant {variant} hard cutoff N={N}: max {err.max():.3e} p99.9 {np.quantile(err, 0.999):.3e}, pairs {pairs}")
    assert np.quantile(err, 0.999) <= 1e-5
    # the tile-pair kernels decide pairs within FP32 rounding of r_c in FP64 as the oracle does
    # (no pair is included on one side only); the 4 x 4 staggered one sums 1024-ion tiles in
    # FP32 before the accumulators (its worst ion here: 1.1e-5). The cell-stencil kernels decide
    # in FP32 on cell-relative offsets.
    assert err.max() <= {32: 1e-5, 3: 2e-5}.get(variant, 1e-3)
    # directed pairs inside the cutoff at the step's drifted positions, within rounding
    lam = plasma.r_D_e
    assert pairs > 0
    tree = spatial.cKDTree(pos / lam)
    approx = tree.count_neighbors(tree, holder.cfg.cutoff / lam) - N  # directed, self excluded
    assert abs(pairs - approx) / approx < 0.01


@pytest.mark.parametrize("variant", [3, 32])
def test_hard_cutoff_pairs_at_the_cutoff(gpu_lib, variant):
    # pairs planted within a few FP32 ulps of r_c on both sides: the tile-pair kernel must
    # include exactly the pairs the FP64 oracle includes (sqrt(dx^2 + dy^2 + dz^2) < r_c on the
    # float positions), so every ion's force stays within 1e-5 of the oracle's
    holder, pos, vel, plasma, sim, grains = case(N=4096, n=4, seed=27, builder=workloads.field_chain,
                                                 switch_distance=0.0)
    lam = plasma.r_D_e
    rc = holder.cfg.cutoff
    rng = np.random.default_rng(5)
    p = pos.copy()
    for k in range(200):
        i, j = 2 * k + 7, 2 * k + 8
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        p[j] = p[i] + d * rc * (1 + (k % 9 - 4) * 4e-8)
    # round to the device's float positions and keep the pairs whose exact distance is within
    # 2e-7 of r_c (both sides), so that the test exercises the exact decision
    x = (p / lam).astype(np.float32).astype(np.float64)
    r = np.linalg.norm(x[8:408:2] - x[7:407:2], axis=1) / (rc / lam)
    assert np.sum(np.abs(r - 1) < 2e-7) >= 100 and np.any(r < 1) and np.any(r >= 1)
    with _lib.Engine(holder) as eng:
        eng.set_pair_plan(*PLANS[variant])
        f = eng.force_snapshot(p)
    ref = oracle.force_snapshot(holder, p, round32=True)
    # (a planted ion with no other ion within r_c has no force at all: floor the denominator)
    err = rel_err_per_ion(f, ref, floor_frac=1e-6)
    print(f"variant {variant} hard cutoff, 200 pairs at r_c: per-ion rel err max {err.max():.3e}")
    assert err.max() <= {32: 1e-5, 3: 2e-5}[variant]


def test_cutoff_deterministic_and_one_step(gpu_lib):
    holder, pos, vel, plasma, sim, grains = _cut_case(4096, 23, cutOff=True)
    runs = []
    for _ in range(2):
        with _lib.Engine(holder) as eng:
            eng.set_state(pos, vel)
            eng.step(1)
            s = eng.series(0, 1)
            p, v = eng.get_state()
        runs.append((s, p, v))
    assert np.array_equal(runs[0][1], runs[1][1]) and np.array_equal(runs[0][2], runs[1][2])
    ref = oracle.run(holder, pos, vel, 0, 1, round32=True)
    dpos = np.max(np.abs(runs[0][1] - ref["pos"])) / plasma.r_D_e
    dvel = np.max(np.abs(runs[0][2] - ref["vel"])) / plasma.v_T
    print(f"cutoff one step: max |dx| {dpos:.3e} lambda, max |dv| {dvel:.3e} v_T")
    assert dpos < 1e-5
    assert dvel < 1e-4


def test_timing_modes_count_pairs_only_when_asked(gpu_lib):
    # timing mode 2 runs the production kernel (no counter); mode 1 counts; other modes are rejected
    holder, pos, vel, plasma, sim, grains = _cut_case(4096, 24, cutOff=True)
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.set_timing(True, count_pairs=False)
        eng.step(1)
        assert eng.cutoff_pairs() == 0 and eng.timing()[1] == 1
        eng.set_timing(True, count_pairs=True)
        eng.step(1)
        assert eng.cutoff_pairs() > 0
        assert eng._lib.od_set_timing(eng.h, 3) == 1  # OD_ERR_INVALID
        eng.set_timing(False)


def test_cutoff_time_averages(gpu_lib):
    # field-driven chain of 5 grains with the 2 lambda cutoff (the C3 physics at 2048 ions):
    # time-averaged charges and orbit forces over the last 150 of 300 steps within 1 % of the
    # oracle's (orbit forces as one norm over the chain: inner grains are shielded and carry
    # small net forces)
    holder, pos, vel, plasma, *_ = case(N=2048, n=300, seed=25, builder=workloads.field_chain,
                                        avg_start=150)
    with _lib.Engine(holder) as eng:
        assert eng.pair_plan()["variant"] == 3
        eng.set_state(pos, vel)
        eng.step(300)
        avg, navg = eng.averages()
    ref = oracle.run(holder, pos, vel, 0, 300, round32=True)
    assert navg == 150
    q_ref = ref["q"][150:].mean(0)
    o_ref = ref["orbit"][150:].mean(0)
    dq = np.max(np.abs(avg[:, 0] - q_ref) / np.abs(q_ref))
    do = np.linalg.norm(avg[:, 1:4] - o_ref) / np.linalg.norm(o_ref)
    print(f"cutoff time averages (5 grains): q rel {dq:.3e}, orbit rel {do:.3e}")
    assert dq < 0.01
    assert do < 0.01


@pytest.mark.parametrize("N", [200, 3000, 70001])
def test_cutoff_ragged_sizes(gpu_lib, N):
    # ion counts that leave the last 512-ion tile partly empty (sentinel slots), a single tile,
    # and an odd count with many tiles: the default kernel against the oracle, switching on
    holder, pos, vel, plasma, sim, grains = case(N=N, n=4, seed=26, builder=workloads.field_chain)
    with _lib.Engine(holder) as eng:
        assert eng.pair_plan()["variant"] == 3
        f = eng.force_snapshot(pos)
    idx = np.arange(N) if N <= 4096 else np.sort(np.random.default_rng(1).choice(N, 2048, replace=False))
    ref = oracle.force_targets(holder, pos, idx, round32=True)
    err = rel_err_per_ion(f[idx], ref)
    print(f"cutoff N={N}: per-ion rel err max {err.max():.3e}")
    assert err.max() <= 1e-5
