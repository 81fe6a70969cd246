"""One simulation split over several GPUs: shards of contiguous ion ranges.

The reference runs one simulation on several GPUs through OpenMM's multi-device context
(Platform property ``DeviceIndex`` "0,1,...", opendust.py:1040-1042; timed by
performance/MultipleGPU/benchmark.py:83). Here every GPU holds one :class:`Shard` (an
``od_shard_*`` handle) that owns ions [first, first + count) and keeps all positions as sources.
A step is five calls per shard with three all-gathers between them:

1. ``begin``: kick and drift of the shard's ions -> their positions (3 x count float32);
2. all-gather of the positions (shards in order) -> ``forces``: ion–ion sums of the shard's ions
   over all positions, kick, flags, ordered compaction and re-injection of the shard's ions;
3. all-gather of the re-injection lists (shards in order = increasing global index) ->
   ``set_list``: grain sums over the run's list, correction and orbit sums of the shard's ions;
4. all-gather of the orbit partial sums -> ``finish``: the FP64 tail (every shard holds the
   charge and force series).

Every sum keeps the order of a single simulation, so the shards reproduce a single handle with
the same directed all-pairs plan bit for bit. The data moved per step is 12 bytes per ion
(positions), 56 bytes per re-injected ion and 24 P bytes per 256 ions; no reduction is taken
across GPUs, so no FP64 all-reduce is needed.

:func:`run_sharded` drives one shard per rank with any ``allgather(obj) -> list`` (e.g.
:class:`TorchAllGather` over ``torch.distributed``, NCCL or gloo); :func:`step_local` drives
several shards in one process (host copies between them).
"""
from __future__ import annotations

import ctypes
from ctypes import c_int64, c_void_p

import numpy as np

from . import _lib


def _ptr(a: np.ndarray):
    return c_void_p(a.ctypes.data)


def split(n_total: int, world: int, pad: int = 512):
    """Contiguous shard ranges [(first, count)]: multiples of `pad` ions, the last takes the rest."""
    blocks = (n_total + pad - 1) // pad
    per = blocks // world
    extra = blocks % world
    out, b0 = [], 0
    for r in range(world):
        nb = per + (1 if r < extra else 0)
        first = b0 * pad
        count = min(nb * pad, n_total - first)
        out.append((first, max(count, 0)))
        b0 += nb
    if any(c <= 0 for _, c in out):
        raise ValueError("more shards than 512-ion blocks")
    return out


class Shard:
    """The ions [first, first + count) of a simulation configured for all its ions."""

    def __init__(self, holder: _lib.ConfigHolder, first: int, count: int, device: int = 0,
                 jsplit: int = 0):
        lib = _lib.load()
        self._lib = lib
        self.holder = holder
        h = c_void_p()
        _lib.check(lib.od_shard_create(holder.ptr(), int(first), int(count), int(jsplit),
                                       int(device), ctypes.byref(h)), None)
        self.h = h
        f, c, n, nb = c_int64(), c_int64(), c_int64(), c_int64()
        _lib.check(lib.od_shard_info(h, ctypes.byref(f), ctypes.byref(c), ctypes.byref(n),
                                     ctypes.byref(nb)), h)
        self.first, self.count, self.n_total, self.orbit_blocks = f.value, c.value, n.value, nb.value
        self.P = max(int(holder.cfg.n_grains), 1)
        self.engine = _lib.Engine(holder, device, _handle=h.value)  # series, state readers
        self.engine.n = self.count
        self.engine._owned = False

    def close(self):
        if getattr(self, "h", None):
            self._lib.od_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, st):
        _lib.check(st, self.h)

    def set_state(self, pos_all: np.ndarray, vel_own: np.ndarray):
        pos_all = np.ascontiguousarray(pos_all, dtype=np.float64)
        vel_own = np.ascontiguousarray(vel_own, dtype=np.float64)
        assert pos_all.shape == (self.n_total, 3) and vel_own.shape == (self.count, 3)
        self._ck(self._lib.od_shard_set_state(self.h, _lib._dptr(pos_all), _lib._dptr(vel_own)))

    def begin(self) -> np.ndarray:
        out = np.empty(3 * self.count, dtype=np.float32)
        self._ck(self._lib.od_shard_begin(self.h, _ptr(out)))
        return out.reshape(3, self.count)

    def forces(self, xyz_all: np.ndarray) -> int:
        xyz_all = np.ascontiguousarray(xyz_all, dtype=np.float32)
        assert xyz_all.shape == (3, self.n_total)
        n = c_int64()
        self._ck(self._lib.od_shard_forces(self.h, _ptr(xyz_all), ctypes.byref(n)))
        self._n_list = n.value
        return n.value

    def get_list(self) -> dict:
        n = self._n_list
        lst = {"idx": np.empty(n, np.int32), "bits": np.empty(n, np.int32),
               "old": np.empty((n, 4), np.float32), "new": np.empty((n, 4), np.float32),
               "v": np.empty((n, 4), np.float32)}
        if n:
            self._ck(self._lib.od_shard_get_list(self.h, *(_ptr(lst[k]) for k in
                                                          ("idx", "bits", "old", "new", "v"))))
        return lst

    def set_list(self, lst: dict) -> np.ndarray:
        n = int(lst["idx"].shape[0])
        arrs = [np.ascontiguousarray(lst[k]) for k in ("idx", "bits", "old", "new", "v")]
        out = np.empty((self.orbit_blocks, self.P, 3))
        self._ck(self._lib.od_shard_set_list(self.h, n, *(_ptr(a) for a in arrs), _ptr(out)))
        return out

    def finish(self, orbit_all: np.ndarray):
        orbit_all = np.ascontiguousarray(orbit_all, dtype=np.float64)
        self._ck(self._lib.od_shard_finish(self.h, _ptr(orbit_all)))

    def series(self, first: int = 0, count: int | None = None):
        return self.engine.series(first, count)

    def get_state(self):
        return self.engine.get_state()


def concat_lists(lists) -> dict:
    """The run's re-injection list from the shards' lists, in shard order."""
    return {k: np.concatenate([l[k] for l in lists]) for k in ("idx", "bits", "old", "new", "v")}


def step_shard(shard, allgather, nsteps: int = 1):
    """Advance one shard of a run by nsteps; allgather(obj) returns every rank's obj in rank
    order (the shards' order). Works with any object offering begin / forces / get_list /
    set_list / finish."""
    for _ in range(nsteps):
        xyz = shard.begin()
        shard.forces(np.concatenate(allgather(xyz), axis=1))
        lst = concat_lists(allgather(shard.get_list()))
        part = shard.set_list(lst)
        shard.finish(np.concatenate(allgather(part), axis=0))


def step_local(shards, nsteps: int = 1):
    """Advance several shards of one run held in this process (host copies between them)."""
    for _ in range(nsteps):
        xyz = np.concatenate([s.begin() for s in shards], axis=1)
        for s in shards:
            s.forces(xyz)
        lst = concat_lists([s.get_list() for s in shards])
        part = np.concatenate([s.set_list(lst) for s in shards], axis=0)
        for s in shards:
            s.finish(part)


class TorchAllGather:
    """allgather(obj) over a torch.distributed process group (gloo or NCCL)."""

    def __init__(self, group=None):
        import torch.distributed as dist

        self.dist = dist
        self.group = group

    def __call__(self, obj):
        out = [None] * self.dist.get_world_size(self.group)
        self.dist.all_gather_object(out, obj, group=self.group)
        return out


def run_sharded(holder: _lib.ConfigHolder, pos_all: np.ndarray, vel_all: np.ndarray, nsteps: int,
                rank: int, world: int, allgather, device: int = 0, jsplit: int = 0):
    """Create this rank's shard, set its state from the whole run's state and step it; returns
    the shard (its series hold the whole run's grain results)."""
    first, count = split(int(holder.cfg.n_ions), world)[rank]
    sh = Shard(holder, first, count, device, jsplit)
    sh.set_state(pos_all, vel_all[first:first + count])
    step_shard(sh, allgather, nsteps)
    return sh
