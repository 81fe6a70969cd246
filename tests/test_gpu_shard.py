"""Shards of one simulation (od_shard_*) against a single handle, on one GPU.

The shards own contiguous ion ranges and exchange positions, re-injection lists and orbit
partial sums between the phases of a step (here by host copies, opendust_gb300.shard.step_local).
Every sum keeps the single-simulation order, so with the single handle on the same directed
all-pairs plan the comparison is bitwise (tolerance 0): the charge and force series, and each
shard's ion state against its slice of the single handle's state.
"""
import numpy as np
import pytest

from opendust_gb300 import _lib, shard, workloads
from tests._util import case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,world,builder,coll", [(5000, 2, workloads.small_plain, True),
                                                  (9000, 3, workloads.field_chain, False)])
def test_shards_equal_single_handle(gpu_lib, N, world, builder, coll):
    kw = {"collisions": "mfp", "mean_free_path": 2 * 1.17541e-3} if coll else {}
    holder, pos, vel, plasma, sim, grains = case(N=N, n=12, seed=71, builder=builder, **kw)
    if builder is workloads.field_chain:      # a hard cutoff has no shard form: all pairs here
        holder.cfg.force_method = _lib.OD_FORCE_ALLPAIRS
        holder.cfg.cutoff = holder.cfg.switch_dist = 0.0
    # ions leaving through the downstream wall and falling into grain 0 in every shard
    lam = plasma.r_D_e
    g = grains[0]
    for r, (first, count) in enumerate(shard.split(N, world)):
        for m in range(6):
            i = first + m
            pos[i] = [0.05 * lam * m, 0.0, sim.H / 2 - (m + 0.5) * 1e-3 * lam]
            vel[i] = [0.0, 0.0, 3 * plasma.v_B]
            j = first + 6 + m
            pos[j] = [g.x, g.y + 0.3 * g.r, g.z + g.r * (1.2 + 0.5 * m)]
            vel[j] = [0.0, 0.0, -3 * plasma.v_B]
    jsplit = 4
    with _lib.Engine(holder) as eng:
        eng.set_pair_plan(256, 1, 5, jsplit)
        eng.set_state(pos, vel)
        eng.step(12)
        ref = eng.series()
        rp, rv = eng.get_state()
    shards = [shard.Shard(holder, f, c, 0, jsplit) for f, c in shard.split(N, world)]
    try:
        for s in shards:
            s.set_state(pos, vel[s.first:s.first + s.count])
        shard.step_local(shards, 12)
        for s in shards:
            got = s.series()
            for k in ref:
                assert np.array_equal(got[k], ref[k]), (s.first, k)
            p, v = s.get_state()
            assert np.array_equal(p, rp[s.first:s.first + s.count])
            assert np.array_equal(v, rv[s.first:s.first + s.count])
    finally:
        for s in shards:
            s.close()
    print(f"{world} shards of {N} ions: 12 steps bitwise equal to one handle")


def test_shard_rejects_bad_ranges_and_order(gpu_lib):
    holder, pos, vel, *_ = case(N=2048, n=4, seed=72)
    with pytest.raises(_lib.OpenDustError):
        shard.Shard(holder, 100, 1000)           # not on a 512-ion boundary
    with pytest.raises(_lib.OpenDustError):
        shard.Shard(holder, 0, 1000)             # not the last shard, not a multiple of 512
    with shard.Shard(holder, 0, 1024) as s:
        s.set_state(pos, vel[:1024])
        with pytest.raises(_lib.OpenDustError):
            s.finish(np.zeros((8, 1, 3)))        # out of order
