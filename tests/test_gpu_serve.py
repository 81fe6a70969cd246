"""The continuous-batching server: each request's result is the same alone and in the mix.

Requests arrive at staggered times, are admitted as members of one batch between chunks of
steps, and retire when their window is complete. Each request's series is compared with the
same request served alone by the plain path; batch members run the same device code on their
own buffers, so the tolerance is 0 (bitwise).
"""
import copy

import numpy as np
import pytest

from opendust_gb300 import serve

pytestmark = pytest.mark.gpu


def test_server_results_equal_alone(gpu_lib):
    reqs = serve.poisson_requests(rate=40.0, duration=0.2, seed=3, log2n=(11, 13), window=20, max_grains=3)
    assert len(reqs) >= 3
    mixed = copy.deepcopy(reqs)
    stats = serve.Server(chunk=6).run(mixed)
    alone = copy.deepcopy(reqs)
    base = serve.run_plain(alone, batch_plan=True)
    print(f"server: {stats}\nplain: {base}")
    for a, b in zip(sorted(mixed, key=lambda r: r.rid), sorted(alone, key=lambda r: r.rid)):
        for k in a.series:
            assert np.array_equal(a.series[k], b.series[k]), (a.rid, k)
        assert np.array_equal(a.averages, b.averages)
    assert stats["latency_p99_s"] >= stats["latency_p50_s"] > 0


def test_server_with_force_interval_equals_alone(gpu_lib):
    # requests served with a force interval (members at different step phases in the mix) equal
    # the same requests run alone with the same interval and plan, bitwise
    rule = lambda n: 4 if n >= 4096 else 2
    reqs = serve.poisson_requests(rate=40.0, duration=0.2, seed=5, log2n=(11, 13), window=21, max_grains=2)
    mixed = copy.deepcopy(reqs)
    serve.Server(chunk=5, interval=rule).run(mixed)
    alone = copy.deepcopy(reqs)
    serve.run_plain(alone, batch_plan=True, interval=rule)
    for a, b in zip(sorted(mixed, key=lambda r: r.rid), sorted(alone, key=lambda r: r.rid)):
        for k in a.series:
            assert np.array_equal(a.series[k], b.series[k]), (a.rid, k)
