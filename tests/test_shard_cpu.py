"""Host logic of the sharded step on CPU: shard ranges and the exchange pattern.

run over torch.distributed gloo with world size 2 (processes on this host), the orchestration of
opendust_gb300.shard (step_shard with TorchAllGather) drives a toy shard that has the CUDA
shard's data dependencies: forces over every shard's positions, a re-injection list that every
shard needs in global order, and orbit partial sums over 256-ion blocks combined by one tail.
The sharded run must equal the single-shard run bit for bit.
"""
import os

import numpy as np
import pytest

from opendust_gb300 import shard


def test_split_ranges():
    assert shard.split(5000, 2) == [(0, 2560), (2560, 2440)]
    assert shard.split(1024, 2) == [(0, 512), (512, 512)]
    assert shard.split(9000, 3) == [(0, 3072), (3072, 3072), (6144, 2856)]
    for n, w in ((2**20, 8), (100_000, 7), (513, 2)):
        r = shard.split(n, w)
        assert r[0][0] == 0 and sum(c for _, c in r) == n
        assert all(f % 512 == 0 for f, _ in r)
        assert all(c % 512 == 0 for _, c in r[:-1])
        assert all(r[k][0] + r[k][1] == r[k + 1][0] for k in range(w - 1))
    with pytest.raises(ValueError):
        shard.split(600, 3)


class ToyShard:
    """Toy dynamics with the exchange pattern of the CUDA shard (FP64 numpy)."""

    L = 1.0

    def __init__(self, pos_all, vel_own, first, count):
        self.first, self.count, self.n = first, count, pos_all.shape[0]
        self.x = pos_all[first:first + count].copy()
        self.v = vel_own.copy()
        self.src = pos_all.copy()
        self.f = self._force(self.x, self.src)
        self.step = 0
        self.q = 0.0
        self.series = []

    @staticmethod
    def _force(x, src):
        d = x[:, None, :] - src[None, :, :]
        r2 = (d ** 2).sum(-1) + 1e-2
        return (d / r2[..., None] ** 1.5).sum(1) * 1e-4

    def begin(self):
        self.v += 0.5 * self.f
        self.x += self.v
        return self.x.T.copy()

    def forces(self, xyz_all):
        self.src = xyz_all.T.copy()
        self.f = self._force(self.x, self.src)
        self.v += 0.5 * self.f
        out = np.flatnonzero(np.abs(self.x).max(1) > self.L)
        self._list = {"idx": (out + self.first).astype(np.int32),
                      "bits": np.ones(len(out), np.int32),
                      "old": self.x[out].copy(), "v": self.v[out].copy()}
        rng = [np.random.default_rng([int(i), self.step]) for i in self._list["idx"]]
        new = np.array([g.uniform(-0.5, 0.5, 3) for g in rng]).reshape(-1, 3)
        self.x[out] = new
        self.v[out] = 0.0
        self._list["new"] = new
        return len(out)

    def get_list(self):
        return self._list

    def set_list(self, lst):
        self.M = lst["v"].sum(0)                       # global sums in global list order
        self.n_inj = getattr(self, "n_inj", 0) + len(lst["idx"])
        self.src[lst["idx"]] = lst["new"]
        mine = (lst["idx"] >= self.first) & (lst["idx"] < self.first + self.count)
        self.f = self._force(self.x, self.src)         # forces after re-injection
        self.f[lst["idx"][mine] - self.first] *= 0.5   # the shard's own re-injected ions
        nb = (self.count + 255) // 256
        part = np.zeros((nb, 1, 3))
        for b in range(nb):
            part[b, 0] = self.x[b * 256:(b + 1) * 256].sum(0)
        return part

    def finish(self, orbit_all):
        self.q += len(self.M) + orbit_all.sum()
        self.series.append((self.q, *self.M, *orbit_all.sum((0, 1))))
        self.step += 1


def _state(n):
    rng = np.random.default_rng(3)
    return rng.uniform(-0.9, 0.9, (n, 3)), rng.normal(0, 0.05, (n, 3))


def _worker(rank, world, port, n, steps, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pos, vel = _state(n)
    first, count = shard.split(n, world)[rank]
    s = ToyShard(pos, vel[first:first + count], first, count)
    shard.step_shard(s, shard.TorchAllGather(), steps)
    np.save(os.path.join(out, f"r{rank}.npy"),
            {"series": np.array(s.series), "x": s.x, "v": s.v}, allow_pickle=True)
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_step_equals_single_rank_gloo(tmp_path):
    pytest.importorskip("torch.distributed")
    import socket

    import torch.multiprocessing as mp

    n, steps = 1300, 6
    pos, vel = _state(n)
    single = ToyShard(pos, vel, 0, n)
    shard.step_shard(single, lambda obj: [obj], steps)
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    mp.start_processes(_worker, args=(2, port, n, steps, str(tmp_path)), nprocs=2,
                       start_method="spawn")
    xs, vs = [], []
    for r in range(2):
        d = np.load(tmp_path / f"r{r}.npy", allow_pickle=True).item()
        assert np.array_equal(d["series"], np.array(single.series)), r
        xs.append(d["x"])
        vs.append(d["v"])
    assert np.array_equal(np.concatenate(xs), single.x)
    assert np.array_equal(np.concatenate(vs), single.v)
    assert len(single.series) == steps and single.n_inj > 20
