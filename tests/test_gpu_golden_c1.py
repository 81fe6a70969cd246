"""C1 (small_plain: N = 16384, 2000 steps, d_t = 1e-10 s, one grain charging from 0) on the GPU
against the full FP64 run of the CPU oracle stored in tests/golden/c1_oracle.npz (made by
tests/golden/make_c1_fixture.py from the same trap coefficients and initial state).

Tolerance: the time averages over the steady-state window (the last 50 % of steps) agree within
1 % for the grain charge and the orbit force; the collection force, which at this size is a
handful of discrete events, agrees within 1 % of the orbit force."""
import os

import numpy as np
import pytest

from opendust_gb300 import _lib, build_simulation, workloads

pytestmark = pytest.mark.gpu
FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c1_oracle.npz")


@pytest.mark.skipif(not os.path.exists(FIX), reason="c1_oracle.npz not generated")
def test_c1_time_averages_match_fp64_oracle(gpu_lib):
    f = np.load(FIX)
    plasma, sim, grains, dist, ext = workloads.small_plain()
    holder, _ = build_simulation(plasma, sim, grains, dist, seed=0, trap=f["alpha"], **ext)
    with _lib.Engine(holder) as eng:
        eng.set_state(f["pos0"], f["vel0"])
        eng.step(sim.n)
        s = eng.series()
        avg, navg = eng.averages()
    h = sim.n // 2
    assert navg == sim.n - h
    q_ref = f["q"][h:, 0].mean()
    o_ref = f["orbit"][h:, 0, :].mean(0)
    c_ref = f["collect"][h:, 0, :].mean(0)
    dq = abs(avg[0, 0] - q_ref) / abs(q_ref)
    do = np.linalg.norm(avg[0, 1:4] - o_ref) / np.linalg.norm(o_ref)
    dc = np.linalg.norm(avg[0, 4:7] - c_ref) / np.linalg.norm(o_ref)
    qmax = np.max(np.abs(s["q"][:, 0] - f["q"][:, 0]) / np.maximum(np.abs(f["q"][:, 0]), 1e-30))
    print(f"C1: q {avg[0, 0]:.4e} vs {q_ref:.4e} ({dq:.2e}), orbit rel {do:.2e}, collect rel {dc:.2e}, "
          f"max per-step q rel {qmax:.2e}, collected {int(f['dN'].sum())} (oracle)")
    assert dq < 0.01
    assert do < 0.01
    assert dc < 0.01
