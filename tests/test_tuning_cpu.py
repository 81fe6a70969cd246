"""Selection logic of opendust_gb300.tuning.choose_force_method on the CPU, with the GPU
measurements replaced by fakes: the fastest method within the error bound wins, the all-pairs
force is always admissible, and the global relative error is measured against it."""
import types

import numpy as np

from opendust_gb300 import tuning


def test_choose_force_method_logic(monkeypatch):
    lam = 1e-3
    holder = types.SimpleNamespace(cfg=types.SimpleNamespace(r_D_e=lam))
    f_all = np.array([[1.0, 0.0, 0.0], [0.0, 2.0, 0.0]])
    # cutoff rc (in lambda) -> (relative error it introduces, step ms)
    fake = {None: (0.0, 10.0), 2.0: (0.10, 4.0), 3.0: (0.02, 6.0), 4.0: (0.005, 9.0)}

    def measure(h, rc, pos, vel, steps, device):
        err, ms = fake[None if rc is None else round(rc / lam, 6)]
        f = f_all * (1 + err)  # |f - f_all| / |f_all| = err
        return f, ms, {"variant": 7 if rc is None else 3}

    monkeypatch.setattr(tuning, "_measure", measure)
    pos = vel = np.zeros((2, 3))
    r = tuning.choose_force_method(holder, pos, vel, max_rel_err=0.03)
    assert r["method"] == "cutoff" and np.isclose(r["cutoff"], 3 * lam) and r["step_ms"] == 6.0
    assert np.isclose(r["rel_err"], 0.02)
    r = tuning.choose_force_method(holder, pos, vel, max_rel_err=0.2)
    assert np.isclose(r["cutoff"], 2 * lam)
    r = tuning.choose_force_method(holder, pos, vel, max_rel_err=0.001)
    assert r["method"] == "allpairs" and r["cutoff"] is None and r["rel_err"] == 0.0
    assert [c["cutoff"] for c in r["candidates"]] == [None, 2 * lam, 3 * lam, 4 * lam]


def test_plan_cache_persists_per_model_and_bucket(tmp_path):
    from opendust_gb300 import tuning

    path = str(tmp_path / "plans.json")
    calls = []

    def fake_time(n, shape):
        calls.append((n, shape))
        return 1.0 if shape == (8, 2048) else 2.0     # the 8 x 2 shape measures faster

    c = tuning.PlanCache(path)
    assert tuning.batch_plan_for(100_000, cache=c, time_plan=fake_time) == (8, 2048)
    assert len(calls) == 2
    # same half-octave bucket: no timing, from memory and from a fresh load of the file
    assert tuning.batch_plan_for(110_000, cache=c, time_plan=fake_time) == (8, 2048)
    assert tuning.batch_plan_for(100_000, cache=tuning.PlanCache(path), time_plan=fake_time) == (8, 2048)
    assert len(calls) == 2
    # another bucket is timed again
    tuning.batch_plan_for(20_000, cache=c, time_plan=fake_time)
    assert len(calls) == 4
    assert tuning.size_bucket(2**16) == 16.0 and tuning.size_bucket(int(2**16.3)) == 16.5
    assert any(k.startswith("batch|") for k in tuning.PlanCache(path).data)
