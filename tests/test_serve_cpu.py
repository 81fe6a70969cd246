"""Host logic of the continuous-batching server (opendust_gb300/serve.py) on the CPU, with the
device, the batch and the setup replaced by fakes: requests are admitted in arrival order while
their device bytes fit the budget (a request larger than the budget runs alone), stepped
together, and retired after exactly their window of steps."""
import types

import numpy as np

from opendust_gb300 import serve


class FakeMember:
    def __init__(self, need):
        self.step_index = 0
        self.need = need

    def averages(self):
        return np.full((1, 4), float(self.step_index)), self.step_index

    def series(self, start, n):
        return {"q": np.zeros((n, 1))}


class FakeBatch:
    def __init__(self, device=0):
        self.members, self.next, self.used, self.max_used = {}, 0, 0, 0
        self.order, self.alone = [], []

    def add(self, holder, pos, vel):
        slot = self.next
        self.next += 1
        self.members[slot] = FakeMember(holder.need)
        self.used += holder.need
        self.max_used = max(self.max_used, self.used if len(self.members) > 1 else 0)
        self.order.append(holder.rid)
        if len(self.members) == 1:
            self.alone.append(holder.rid)
        return slot

    def step(self, k):
        for m in self.members.values():
            m.step_index += k

    def last_step_ms(self):
        return 0.01

    def member(self, slot):
        return self.members[slot]

    def remove(self, slot):
        self.used -= self.members.pop(slot).need

    def close(self):
        pass


def test_server_admission_budget_and_windows(monkeypatch):
    batches = []

    def make_batch(device=0):
        batches.append(FakeBatch(device))
        return batches[-1]

    monkeypatch.setattr(serve, "device_memory", lambda device=0: (1000, 1000))
    monkeypatch.setattr(serve._lib, "Batch", make_batch)
    monkeypatch.setattr(serve._lib, "config_device_bytes", lambda holder: holder.need)
    monkeypatch.setattr(serve, "host_prepare", lambda r: None)
    monkeypatch.setattr(serve, "finish_prepare",
                        lambda r, host, device=0: (types.SimpleNamespace(need=r.ext["need"], rid=r.rid),
                                                   None, None))
    needs = [300, 300, 300, 900, 100, 450, 450, 200]
    windows = [40, 10, 25, 30, 5, 60, 15, 20]
    reqs = [serve.Request(rid=i, arrival=0.002 * i, plasma=None, sim=types.SimpleNamespace(N=1000),
                          grains=[], dist="Maxwellian", ext={"need": n}, seed=i, window=w)
            for i, (n, w) in enumerate(zip(needs, windows))]
    stats = serve.Server(budget_frac=0.8, chunk=7).run(reqs)
    b = batches[0]
    assert stats["requests"] == 8 and all(r.done is not None for r in reqs)
    assert b.order == sorted(b.order)            # admitted in arrival order
    assert b.max_used <= 800                     # shared admissions stay within the budget
    assert 3 in b.alone                          # the 900-byte request ran alone
    for r in reqs:                               # retired after exactly its window
        assert r.averages[0, 0] == r.window and r.series["q"].shape == (r.window, 1)
    assert not b.members and b.used == 0
