"""GPU parity at the stated workload sizes, against the FP64 CPU oracle.

* Plain method at full size (2^20 ions, mean-free-path collisions): ten independent
  simulations with seeds 0-9, each stepped 2, 4, ..., 20 steps from a device-sampled initial
  state; every snapshot is checked on 4096 random target ions x all 2^20 sources, per-ion
  |dF|/|F| <= 1e-5.
* Field-driven chain of 5 grains at full size (2^19 ions, 2 lambda cutoff with switching):
  snapshot forces on 2048 random targets (per-ion <= 1e-5) from a running simulation, and the
  collected-ion set bit-exact with ions planted on, just inside and just outside every grain.
* Grain series over a few hundred steps (charge, dust-dust, collection, external field and
  orbit forces) against the oracle's per-step series, for the 5-grain field-driven chain and a
  two-grain Maxwellian case (opendust.py:1205-1235 dust-dust, :1333-1383 collection and field).
"""
import numpy as np
import pytest

from opendust_gb300 import _lib, build_simulation, setup_host, workloads
from oracle import oracle
from tests._util import case, rel_err_per_ion

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", range(10))
def test_full_size_plain_seeded_snapshots(gpu_lib, seed):
    plasma, sim, grains, dist, ext = workloads.full_plain(n=24)
    holder, _ = build_simulation(plasma, sim, grains, dist, seed=seed, **ext)
    N = int(sim.N)
    with _lib.Engine(holder) as eng:
        eng.init_state()
        eng.step(2 * (seed + 1))
        pos, _ = eng.get_state()
        f = eng.force_snapshot(pos)
    idx = np.sort(np.random.default_rng(1000 + seed).choice(N, 4096, replace=False))
    ref = oracle.force_targets(holder, pos, idx, round32=True)
    err = rel_err_per_ion(f[idx], ref)
    print(f"2^20 ions, seed {seed}, step {2 * (seed + 1)}: 4096 targets, per-ion rel err max "
          f"{err.max():.3e} p99 {np.quantile(err, 0.99):.3e}")
    assert err.max() <= 1e-5


def _plant_on_grains(pos, grains, sim, rng, per_grain=64):
    p = pos.copy()
    k = 0
    for g in grains:
        c = np.array([g.x, g.y, g.z])
        for m in range(per_grain):
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            p[k] = c + d * g.r * (1 + (m % 3 - 1) * 1e-7)   # just inside, on, just outside
            k += 1
        p[k] = c + np.array([g.r, 0.0, 0.0])                # exactly on the surface along x
        p[k + 1] = c - np.array([0.0, 0.0, g.r])
        k += 2
    p[k:k + 4] = [[sim.R, 0, 0], [0, 0, sim.H / 2], [0, 0, -sim.H / 2], [0, np.nextafter(sim.R, 0), 0]]
    return p


def test_full_size_field_chain_snapshot_and_collected_set(gpu_lib):
    plasma, sim, grains, dist, ext = workloads.field_chain(n=16)
    holder, _ = build_simulation(plasma, sim, grains, dist, seed=7, **ext)
    N = int(sim.N)
    assert N == 2**19 and len(grains) == 5 and holder.cfg.force_method == _lib.OD_FORCE_CUTOFF
    assert abs(holder.cfg.cutoff / plasma.r_D_e - 2.0) < 1e-12
    with _lib.Engine(holder) as eng:
        eng.init_state(setup_host.field_driven_vz_table(plasma.v_fl, plasma.v_T))
        eng.step(12)
        pos, _ = eng.get_state()
        f = eng.force_snapshot(pos)
        planted = _plant_on_grains(pos, grains, sim, np.random.default_rng(9))
        idx_c, cnt, gc = eng.collect_flags(planted)
    idx = np.sort(np.random.default_rng(77).choice(N, 2048, replace=False))
    ref = oracle.force_targets(holder, pos, idx, round32=True)
    err = rel_err_per_ion(f[idx], ref)
    print(f"2^19-ion 5-grain chain, 2 lambda cutoff: 2048 targets, per-ion rel err max "
          f"{err.max():.3e} p99 {np.quantile(err, 0.99):.3e}")
    assert err.max() <= 1e-5
    ridx, rcnt, rgc = oracle.collect_flags(holder, planted, round32=True)
    print(f"collected/exited at 2^19: {cnt} ions, per grain {list(gc)}")
    assert cnt == rcnt
    assert np.array_equal(idx_c, ridx)
    assert np.array_equal(gc, rgc)
    assert np.all(gc >= 20)            # at least the ions planted just inside every grain


def _two_grain_maxwell(N, n):
    plasma, sim, grains, dist, ext = workloads.small_plain(N=N, n=n)
    lam = plasma.r_D_e
    from opendust_gb300.opendust import DustParticle
    grains = [DustParticle(0.0, 0.0, -0.5 * lam, 1e-5, "oml", -2e-15),
              DustParticle(0.0, 0.0, 0.5 * lam, 1e-5, "consistent", -2e-15)]
    return plasma, sim, grains, dist, ext


@pytest.mark.parametrize("builder,N,n", [(workloads.field_chain, 2048, 300),
                                         (_two_grain_maxwell, 2048, 200)])
def test_grain_series_against_oracle(gpu_lib, builder, N, n):
    holder, pos, vel, plasma, sim, grains = case(N=N, n=n, seed=51, builder=builder)
    P = len(grains)
    assert P >= 2
    # ions aimed at every grain, so that each collects within the first steps
    rng = np.random.default_rng(52)
    k = 0
    for g in grains:
        c = np.array([g.x, g.y, g.z])
        for _ in range(8):
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            pos[k] = c + 1.5 * g.r * d
            vel[k] = -3.0 * plasma.v_B * d
            k += 1
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(n)
        ser = eng.series()
    ref = oracle.run(holder, pos, vel, 0, n, round32=True)

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

    dq = rel(ser["q"], ref["q"])
    dd = rel(ser["dust"], ref["dust"])
    dc = rel(ser["collect"], ref["collect"])
    do = rel(ser["orbit"], ref["orbit"])
    print(f"{P} grains, {n} steps: q {dq:.2e}, dust-dust {dd:.2e}, collect {dc:.2e}, "
          f"orbit {do:.2e}, collected {ref['dN'].sum()}")
    assert np.all(ref["dN"].sum(0) > 0) and np.abs(ref["dust"]).max() > 0
    # charges follow from integer collection counts: equal counts give charges equal to FP64
    # rounding, and the dust-dust force is a function of the charges and grain positions
    assert dq <= 1e-9
    assert dd <= 1e-8
    # collection force: sum of FP32 velocities of the same collected ions
    assert dc <= 1e-4
    assert do <= 1e-3
    if np.abs(ref["field"]).max() > 0:
        assert rel(ser["field"], ref["field"]) <= 1e-9
