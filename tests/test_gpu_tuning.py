"""Accuracy-bounded choice between the all-pairs and the cutoff force (opendust_gb300.tuning) on
the GPU: the snapshot error falls as the cutoff grows, the choice never exceeds the bound, a zero
bound keeps the all-pairs force, and among the admissible methods the fastest is chosen."""
import numpy as np
import pytest

from opendust_gb300 import tuning, workloads
from tests._util import case

pytestmark = pytest.mark.gpu


def test_choose_force_method(gpu_lib):
    holder, pos, vel, plasma, sim, grains = case(N=32768, n=4, seed=31, builder=workloads.small_plain)
    r = tuning.choose_force_method(holder, pos, vel, max_rel_err=1.0)
    c = r["candidates"]
    assert c[0]["cutoff"] is None and c[0]["rel_err"] == 0.0
    errs = [x["rel_err"] for x in c[1:]]
    print("cutoff candidates:", [(round(x["cutoff"] / plasma.r_D_e, 2), f"{x['rel_err']:.3e}",
                                  f"{x['step_ms']:.3f} ms") for x in c[1:]], "all-pairs",
          f"{c[0]['step_ms']:.3f} ms")
    assert errs[0] > errs[1] > errs[2] > 0
    assert r["step_ms"] == min(x["step_ms"] for x in c)
    assert all(x["plan"]["variant"] == 3 for x in c[1:])
    strict = tuning.choose_force_method(holder, pos, vel, max_rel_err=0.0, cutoffs_lambda=(2.0,))
    assert strict["method"] == "allpairs" and strict["cutoff"] is None
    mid = tuning.choose_force_method(holder, pos, vel, max_rel_err=errs[1] * 1.0001)
    assert mid["rel_err"] <= errs[1] * 1.0001


def test_simulate_with_the_tuned_plan_cache(gpu_lib, tmp_path, monkeypatch):
    # pair_plan="tuned": the first run measures and stores the plan for this GPU model and size
    # bucket; a second run reuses it without timing again
    import json

    from opendust.opendust import (DustParticle, OpenDust, OutputParameters,
                                   PlasmaParametersInSIUnitsMaxwell, SimulationParametersInSIUnits)

    cache = tmp_path / "plans.json"
    monkeypatch.setenv("OD_PLAN_CACHE", str(cache))
    p = PlasmaParametersInSIUnitsMaxwell(300, 29011.3, 1e14, 1.0, 6.6335e-26)
    for _ in range(2):
        s = SimulationParametersInSIUnits(3 * p.r_D_e, 6 * p.r_D_e, 8192, 4, 1e-10, p)
        od = OpenDust(p, s, OutputParameters(100, 100), [DustParticle(0, 0, 0, 1e-5, "consistent", 0.0)],
                      "Maxwellian")
        q, forces = od.simulate("0", quiet=True, pair_plan="tuned")
        assert np.isfinite(q).all() and np.isfinite(forces["orbit"]).all()
    data = json.loads(cache.read_text())
    assert len(data) == 1 and next(iter(data)).startswith("single|")
