"""Batched simulations: results in a batch equal the same simulations stepped alone.

Each batch member keeps its own buffers and partial sums, and the batched kernels run the same
device code as the single-simulation kernels with the member's all-pairs plan
(_lib.batch_pair_plan), so the comparison with a single simulation given that plan is bitwise
(tolerance 0) — alone, in a fixed mix, and with members joining and leaving between steps
(continuous batching).
"""
import numpy as np
import pytest

from opendust_gb300 import _lib, build_simulation, setup_host, workloads

pytestmark = pytest.mark.gpu


def member(N, P, seed, collisions, n=24):
    plasma, sim, grains, dist, ext = workloads.small_plain(N=N, n=n)
    lam = plasma.r_D_e
    grains = [workloads.DustParticle(0.0, 0.0, (k - (P - 1) / 2) * lam, 1e-5, "consistent", -1e-15)
              for k in range(P)]
    ext = {"collisions": "mfp", "mean_free_path": 2 * lam} if collisions else {}
    holder, _ = build_simulation(plasma, sim, grains, dist, seed=seed, **ext)
    pos, vel = setup_host.initial_state(N, sim.R, sim.H, [(g.x, g.y, g.z, g.r) for g in grains],
                                        plasma.v_fl, plasma.v_T, dist, seed)
    return holder, pos, vel


def alone(holder, pos, vel, steps):
    with _lib.Engine(holder) as eng:
        eng.set_pair_plan(*_lib.batch_pair_plan(eng.n))
        eng.set_state(pos, vel)
        eng.step(steps)
        s = eng.series(0, steps)
        p, v = eng.get_state()
    return s, p, v


def same(a, b):
    s1, p1, v1 = a
    s2, p2, v2 = b
    for k in s1:
        assert np.array_equal(s1[k], s2[k]), k
    assert np.array_equal(p1, p2) and np.array_equal(v1, v2)


def test_batch_equals_alone(gpu_lib):
    specs = [(2048, 1, 1, False), (5000, 2, 2, True), (9000, 3, 3, False), (16384, 4, 4, True)]
    cases = [member(*s) for s in specs]
    ref = [alone(h, p, v, 12) for h, p, v in cases]
    with _lib.Batch() as b:
        slots = [b.add(h, p, v) for h, p, v in cases]
        assert len(b) == 4
        b.step(5)
        b.step(7)
        assert b.last_step_ms() > 0
        for slot, r in zip(slots, ref):
            m = b.member(slot)
            p, v = m.get_state()
            same(r, (m.series(0, 12), p, v))


def test_batch_continuous_membership(gpu_lib):
    a = member(3000, 1, 11, True)
    c = member(7000, 2, 12, False)
    ref_c = alone(*c, 8)
    with _lib.Batch() as b:
        sa = b.add(*a)
        b.step(4)
        sc = b.add(*c)          # joins while the other member is mid-run
        b.step(4)
        b.remove(sa)            # leaves; the remaining member continues
        b.step(4)
        m = b.member(sc)
        assert m.step_index == 8
        p, v = m.get_state()
        # the later member's first 8 steps equal its solo run
        s = m.series(0, 8)
    with _lib.Engine(c[0]) as eng:
        eng.set_pair_plan(*_lib.batch_pair_plan(eng.n))
        eng.set_state(c[1], c[2])
        eng.step(8)
        s8 = eng.series(0, 8)
    for k in s8:
        assert np.array_equal(s8[k], s[k]), k
    for k in ref_c[0]:
        assert np.array_equal(ref_c[0][k], s8[k]), k


def test_batch_rejects_overflow_and_cutoff(gpu_lib):
    h, p, v = member(2048, 1, 5, False, n=4)
    with _lib.Batch() as b:
        b.add(h, p, v)
        b.step(4)
        with pytest.raises(_lib.OpenDustError) as e:
            b.step(1)
        assert e.value.status == 4
    plasma, sim, grains, dist, ext = workloads.small_plain(N=2048, n=4)
    hc, _ = build_simulation(plasma, sim, grains, dist, seed=1, cutOff=True)
    with _lib.Batch() as b:
        with pytest.raises(_lib.OpenDustError) as e:
            b.add(hc, p, v)
        assert e.value.status == 6


def test_batch_member_plan_can_be_set(gpu_lib):
    # a member moved to the other batch shape (8 x 2 with 2048-ion tiles below 2^16 ions) after
    # it joined equals the same simulation stepped alone with the same plan change, bitwise (its
    # initial sums come from the plan it joined with)
    h, p, v = member(9000, 2, 5, True)
    with _lib.Engine(h) as eng:
        eng.set_pair_plan(*_lib.batch_pair_plan(eng.n))
        eng.set_state(p, v)
        eng.set_pair_plan(256, 8, 7, 2048)
        eng.step(8)
        ref = (eng.series(0, 8), *eng.get_state())
    with _lib.Batch() as b:
        s = b.add(h, p, v)
        b.set_plan(s, 8, 2048)
        b.step(8)
        m = b.member(s)
        assert m.pair_plan()["targets_per_thread"] == 8
        same(ref, (m.series(0, 8), *m.get_state()))
        with pytest.raises(_lib.OpenDustError):
            b.set_plan(s, 4, 2048)
