"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle.

Tolerances (stated per test):
  * ion–ion force on an identical snapshot: per-ion |dF|/|F| <= 1e-5 (FP32 pair terms with
    two-float accumulation against FP64);
  * collected-ion sets and counts on identical positions: bit-exact;
  * one step from an identical state: positions within 1e-5 lambda, grain charge within
    1e-9 relative, orbit force within 1e-4 relative;
  * time averages over a seeded window: within 1 %.
"""
import numpy as np
import pytest

from opendust_gb300 import _lib, workloads
from oracle import oracle
from tests._util import case, plant_close_pairs, rel_err_per_ion

pytestmark = pytest.mark.gpu


PLANS = [(256, 1, 0), (128, 2, 0), (256, 1, 1), (128, 2, 2), (256, 2, 2), (128, 2, 3), (256, 2, 3),
         (256, 2, 4), (256, 1, 5), (128, 1, 6), (256, 1, 6), (256, 2, 7), (256, 2, 7, 512),
         (256, 4, 7), (256, 8, 7)]


@pytest.mark.parametrize("plan", PLANS)
def test_force_snapshot_all_targets(gpu_lib, plan):
    holder, pos, vel, plasma, sim, grains = case(N=4096, n=4, seed=11)
    rng = np.random.default_rng(5)
    pos = plant_close_pairs(pos, plasma.r_D_e, rng, n_pairs=64, dmin=2e-4)
    with _lib.Engine(holder) as eng:
        eng.set_pair_plan(*plan)
        f = eng.force_snapshot(pos)
    ref = oracle.force_snapshot(holder, pos, round32=True)
    err = rel_err_per_ion(f, ref)
    print(f"plan {plan} N=4096 per-ion rel err: max {err.max():.3e} p99 {np.quantile(err, 0.99):.3e}")
    assert err.max() <= 1e-5


@pytest.mark.parametrize("N,plan", [(2**14, None), (2**18, None), (2**20, None), (2**20, (256, 2, 3)),
                                    (2**20, (256, 1, 5)), (2**18, (256, 2, 7)),
                                    (2**20, (256, 4, 7, 4096)), (2**18, (256, 4, 7, 2048))])
def test_force_snapshot_large(gpu_lib, N, plan):
    holder, pos, vel, plasma, sim, grains = case(N=N, n=4, seed=12)
    with _lib.Engine(holder) as eng:
        if plan:
            eng.set_pair_plan(*plan)
        f = eng.force_snapshot(pos)
    rng = np.random.default_rng(1)
    idx = np.sort(rng.choice(N, 1024 if N > 2**18 else 2048, replace=False))
    ref = oracle.force_targets(holder, pos, idx, round32=True)
    err = rel_err_per_ion(f[idx], ref)
    print(f"N={N} per-ion rel err: max {err.max():.3e} p99 {np.quantile(err, 0.99):.3e}")
    assert err.max() <= 1e-5


@pytest.mark.parametrize("N,plan", [(5000, (256, 2, 7, 512)), (5000, (256, 4, 7, 2048)), (5000, (256, 4, 7, 4096)),
                                    (5000, (256, 2, 7, 4096)), (9000, (256, 2, 7, 1024)),
                                    (5000, (256, 8, 7, 2048)), (9000, (256, 8, 7, 4096))])
def test_each_pair_once_ragged_tiles(gpu_lib, N, plan):
    # variant 7 with tiles that the padded ion count does not fill: the last tile holds fewer
    # groups than the others (and padding sentinels inside the last group)
    holder, pos, vel, plasma, sim, grains = case(N=N, n=4, seed=18)
    rng = np.random.default_rng(8)
    pos = plant_close_pairs(pos, plasma.r_D_e, rng, n_pairs=32, dmin=2e-4)
    with _lib.Engine(holder) as eng:
        eng.set_pair_plan(*plan)
        pl = eng.pair_plan()
        assert pl["variant"] == 7 and pl["jsplit"] == plan[3]
        f = eng.force_snapshot(pos)
        f2 = eng.force_snapshot(pos)
    assert np.array_equal(f, f2)
    ref = oracle.force_snapshot(holder, pos, round32=True)
    err = rel_err_per_ion(f, ref)
    print(f"variant 7 {plan} N={N} per-ion rel err: max {err.max():.3e}")
    assert err.max() <= 1e-5


def test_each_pair_once_steps_match_directed(gpu_lib):
    # 30 full steps with variant 7 against the directed-pair default on the same state: the two
    # sum the same terms in a different order, so trajectories agree to FP32 rounding growth
    holder, pos, vel, plasma, *_ = case(N=8192, n=30, seed=19)
    out = {}
    for plan in [(256, 1, 5, 0), (256, 4, 7, 0)]:
        with _lib.Engine(holder) as eng:
            eng.set_pair_plan(*plan)
            eng.set_state(pos, vel)
            eng.step(30)
            out[plan[2]] = (eng.series(), eng.get_state()[0])
    dpos = np.max(np.abs(out[5][1] - out[7][1])) / plasma.r_D_e
    dq = np.max(np.abs(out[5][0]["q"] - out[7][0]["q"]) / np.maximum(np.abs(out[5][0]["q"]), 1e-30))
    print(f"variant 7 vs 5 after 30 steps: max |dx| {dpos:.3e} lambda, q rel {dq:.3e}")
    assert dpos < 1e-4
    assert dq < 1e-6


def test_collect_flags_bit_exact(gpu_lib):
    holder, pos, vel, plasma, sim, grains = case(N=4096, n=4, seed=13)
    p = pos.copy()
    g = grains[0]
    r = g.r
    rng = np.random.default_rng(2)
    # ions exactly on / just inside / just outside the grain surface and the domain walls
    for k in range(64):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        p[k] = np.array([g.x, g.y, g.z]) + d * r * (1 + (k % 3 - 1) * 1e-7)
    p[64] = [r, 0, 0]
    p[65] = [sim.R, 0, 0]
    p[66] = [0, sim.R, 0]
    p[67] = [0, 0, sim.H / 2]
    p[68] = [0, 0, -sim.H / 2]
    p[69] = [sim.R * np.cos(0.3), sim.R * np.sin(0.3), 0]
    p[70] = [np.nextafter(sim.R, 0), 0, 0]
    with _lib.Engine(holder) as eng:
        idx, cnt, gc = eng.collect_flags(p)
    ridx, rcnt, rgc = oracle.collect_flags(holder, p, round32=True)
    assert cnt == rcnt
    assert np.array_equal(idx, ridx)
    assert np.array_equal(gc, rgc)
    assert cnt > 20


def test_one_step(gpu_lib):
    holder, pos, vel, plasma, sim, grains = case(N=2048, n=4, seed=14)
    lam = plasma.r_D_e
    # ions just inside the downstream wall moving out, and ions falling into the grain
    for k in range(20):
        pos[k] = [0.1 * lam * k / 20, 0.0, sim.H / 2 - 1e-6 * lam]
        vel[k] = [0.0, 0.0, 3 * plasma.v_B]
    g = grains[0]
    for k in range(20, 30):
        th = 2 * np.pi * (k - 20) / 10
        pos[k] = [g.x + 0.5 * g.r * np.cos(th), g.y + 0.5 * g.r * np.sin(th), g.z + g.r * 1.001]
        vel[k] = [0.0, 0.0, -3 * plasma.v_B]
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(1)
        ser = eng.series(0, 1)
        gp, gv = eng.get_state()
    ref = oracle.run(holder, pos, vel, 0, 1, round32=True)
    lam = plasma.r_D_e
    assert ref["n_inj"][0] > 0
    dpos = np.max(np.abs(gp - ref["pos"])) / lam
    print(f"one step: re-injected {ref['n_inj'][0]}, max |dx| {dpos:.3e} lambda")
    assert dpos < 1e-5
    np.testing.assert_allclose(ser["q"], ref["q"], rtol=1e-9)
    o_err = np.linalg.norm(ser["orbit"] - ref["orbit"]) / np.linalg.norm(ref["orbit"])
    assert o_err < 1e-4


def test_multi_step(gpu_lib):
    holder, pos, vel, plasma, sim, grains = case(N=2048, n=40, seed=15)
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(40)
        ser = eng.series()
        gp, gv = eng.get_state()
    ref = oracle.run(holder, pos, vel, 0, 40, round32=True)
    lam = plasma.r_D_e
    dpos = np.max(np.abs(gp - ref["pos"])) / lam
    qerr = np.max(np.abs(ser["q"] - ref["q"]) / np.maximum(np.abs(ref["q"]), 1e-30))
    oerr = np.max(np.linalg.norm(ser["orbit"] - ref["orbit"], axis=2) /
                  np.linalg.norm(ref["orbit"], axis=2))
    print(f"40 steps: max |dx| {dpos:.3e} lambda, q rel {qerr:.3e}, orbit rel {oerr:.3e}, "
          f"injected {ref['n_inj'].sum()}")
    assert dpos < 1e-3
    assert qerr < 1e-6
    assert oerr < 1e-3


@pytest.mark.parametrize("plan", [None, (256, 4, 7, 1024)])
def test_deterministic(gpu_lib, plan):
    holder, pos, vel, *_ = case(N=4096, n=20, seed=16)
    out = []
    for _ in range(2):
        with _lib.Engine(holder) as eng:
            if plan:
                eng.set_pair_plan(*plan)
            eng.set_state(pos, vel)
            eng.step(20)
            s = eng.series()
            p, v = eng.get_state()
        out.append((s, p, v))
    for k in out[0][0]:
        assert np.array_equal(out[0][0][k], out[1][0][k]), k
    assert np.array_equal(out[0][1], out[1][1])


def test_trap_potential(gpu_lib):
    from opendust_gb300 import setup_host as sh

    Rh, Hh, n_r, n_h, _ = sh.trap_grid(3.0, 6.0, 1.0)
    g = _lib.trap_potential(Rh, Hh, n_r, n_h, 100_000, 99)
    o = oracle.trap_potential(Rh, Hh, n_r, n_h, 100_000, 99)
    rel = np.max(np.abs(g - o) / np.abs(o))
    print(f"trap grid rel diff {rel:.3e}")
    assert rel < 1e-5


def test_time_averages(gpu_lib):
    holder, pos, vel, plasma, *_ = case(N=2048, n=300, seed=17, avg_start=150)
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(300)
        avg, navg = eng.averages()
    ref = oracle.run(holder, pos, vel, 0, 300, round32=True)
    assert navg == 150
    q_ref = ref["q"][150:].mean(0)
    o_ref = ref["orbit"][150:].mean(0)
    dq = abs(avg[0, 0] - q_ref[0]) / abs(q_ref[0])
    do = np.linalg.norm(avg[0, 1:4] - o_ref[0]) / np.linalg.norm(o_ref[0])
    print(f"time averages: q rel {dq:.3e}, orbit rel {do:.3e}")
    assert dq < 0.01
    assert do < 0.01


def test_autotune_picks_a_correct_plan(gpu_lib):
    holder, pos, vel, plasma, *_ = case(N=2**16, n=4, seed=41)
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        rate = eng.autotune(use_cache=False)
        plan = eng.pair_plan()
        f = eng.force_snapshot(pos)
        eng.step(2)
    print(f"autotuned plan {plan}, {rate:.3e} pairs/s")
    assert rate > 1e11
    idx = np.arange(0, 2**16, 64)
    ref = oracle.force_targets(holder, pos, idx, round32=True)
    assert rel_err_per_ion(f[idx], ref).max() <= 1e-5
