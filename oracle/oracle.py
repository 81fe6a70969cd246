"""CPU ORACLE wrapper — test infrastructure only.

ctypes access to oracle/_build/libod_oracle.so, the plain-C FP64 restatement of
OpenDust's per-timestep superion update (oracle/od_oracle.c). Only tests/,
__graft_entry__.smoke() and bench.py's cpu_baseline / reference arm use it, always as
the checker or the timed CPU baseline, never as part of the product path.

Parity status: the restatement is pinned by (1) the Philox4x32-10 known-answer vectors
of Random123 (tests/test_oracle.py), (2) analytic known-answer cases written for this
project (2- and 3-ion Yukawa forces, ion–grain Coulomb, surface flags, charge-update
closed forms), and (3) statistically, through the GPU path, against the time-averaged
forces printed by the reference's own example runs (tests/golden/). The reference's
OpenMM/CuPy code cannot run here, so bit-level parity with it is unpinned.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_int, c_int64, c_uint32, c_uint64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libod_oracle.so")
_DP = POINTER(c_double)
_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "od_oracle.c")
    hdr = os.path.join(os.path.dirname(HERE), "include", "opendust_gb300.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        lib.odo_philox.argtypes = [POINTER(c_uint32), POINTER(c_uint32), POINTER(c_uint32)]
        lib.odo_force_snapshot.argtypes = [c_void_p, _DP, c_int64, c_int, _DP]
        lib.odo_collect_flags.argtypes = [c_void_p, _DP, c_int64, c_int, POINTER(c_int64), c_int64,
                                          POINTER(c_int64), POINTER(c_int64)]
        lib.odo_trap_potential.argtypes = [c_double, c_double, c_int, c_int, c_int64, c_uint64, _DP]
        lib.odo_inject.argtypes = [c_void_p, c_int64, c_int64, _DP, _DP]
        lib.odo_run.argtypes = [c_void_p, _DP, _DP, c_int64, c_int, c_int64, c_int64, c_int64, _DP,
                                _DP, _DP, _DP, _DP, _DP, POINTER(c_int64), POINTER(c_int64)]
        lib.odo_accel.argtypes = [c_void_p, _DP, c_int64, c_int, _DP, _DP]
        lib.odo_force_targets.argtypes = [c_void_p, _DP, c_int64, c_int, POINTER(c_int64), c_int64,
                                          _DP]
        lib.odo_ion_potential_grid.argtypes = [c_void_p, _DP, c_int64, c_int, _DP, _DP, c_int, c_int,
                                               _DP]
        lib.odo_set_threads.argtypes = [c_int]
        lib.odo_max_threads.restype = c_int
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(_DP)


def _cfg(holder):
    return ctypes.cast(ctypes.byref(holder.cfg), c_void_p)


def set_threads(n: int):
    load().odo_set_threads(int(n))


def max_threads() -> int:
    return int(load().odo_max_threads())


def philox(ctr, key):
    c = (c_uint32 * 4)(*ctr)
    k = (c_uint32 * 2)(*key)
    o = (c_uint32 * 4)()
    load().odo_philox(c, k, o)
    return [int(x) for x in o]


# round32 values: True rounds positions to float (what the snapshot calls consume);
# DEVICE_STATE takes the device's cell-relative position state of od_set_state (od_run: the state
# exactly; the snapshot functions: the absolute float positions the device derives from it)
DEVICE_STATE = 2


def force_snapshot(holder, pos, round32=True):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    f = np.empty_like(pos)
    rc = load().odo_force_snapshot(_cfg(holder), _p(pos), pos.shape[0], int(round32), _p(f))
    assert rc == 0
    return f


def accel(holder, pos, q, round32=True):
    """Total acceleration [m/s^2] with grain charges q [C]."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    a = np.empty_like(pos)
    assert load().odo_accel(_cfg(holder), _p(pos), pos.shape[0], int(round32), _p(q), _p(a)) == 0
    return a


def force_targets(holder, pos, idx, round32=True):
    """Ion–ion force [N] on the ions idx only."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    f = np.empty((idx.shape[0], 3))
    rc = load().odo_force_targets(_cfg(holder), _p(pos), pos.shape[0], int(round32),
                                  idx.ctypes.data_as(POINTER(c_int64)), idx.shape[0], _p(f))
    assert rc == 0
    return f


def collect_flags(holder, pos, round32=True):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    n = pos.shape[0]
    idx = np.empty(n, dtype=np.int64)
    cnt = c_int64()
    gc = np.zeros(16, dtype=np.int64)
    rc = load().odo_collect_flags(_cfg(holder), _p(pos), n, int(round32),
                                  idx.ctypes.data_as(POINTER(c_int64)), n, ctypes.byref(cnt),
                                  gc.ctypes.data_as(POINTER(c_int64)))
    assert rc == 0
    return idx[: cnt.value].copy(), int(cnt.value), gc[: holder.cfg.n_grains].copy()


def trap_potential(Rh, Hh, n_r, n_h, n_points, seed):
    pot = np.empty(n_r * n_h)
    rc = load().odo_trap_potential(Rh, Hh, n_r, n_h, n_points, seed, _p(pot))
    assert rc == 0
    return pot.reshape(n_r, n_h)


def inject(holder, ion, step):
    x = np.empty(3)
    v = np.empty(3)
    assert load().odo_inject(_cfg(holder), ion, step, _p(x), _p(v)) == 0
    return x, v


def run(holder, pos, vel, first_step, nsteps, q_param=None, round32=True, rng_base=0):
    """Run steps [first_step, first_step+nsteps) of the reference program. Returns a dict
    with the final state and the per-step series. rng_base: Philox step counter of step 0 (a
    later window of a simulation whose random streams continue)."""
    c = holder.cfg
    P = c.n_grains
    pos = np.array(pos, dtype=np.float64, order="C")
    vel = np.array(vel, dtype=np.float64, order="C")
    if q_param is None:
        q_param = np.array([c.grain_q0[g] for g in range(P)], dtype=np.float64)
    qp = np.array(q_param, dtype=np.float64)
    Pm = max(P, 1)
    q = np.zeros((nsteps, Pm))
    fo, fc, fd, ff = (np.zeros((nsteps, Pm, 3)) for _ in range(4))
    ninj = np.zeros(nsteps, dtype=np.int64)
    dN = np.zeros((nsteps, Pm), dtype=np.int64)
    rc = load().odo_run(_cfg(holder), _p(pos), _p(vel), pos.shape[0], int(round32), first_step,
                        nsteps, int(rng_base), _p(qp), _p(q), _p(fo), _p(fc), _p(fd), _p(ff),
                        ninj.ctypes.data_as(POINTER(c_int64)), dN.ctypes.data_as(POINTER(c_int64)))
    assert rc == 0
    return {"pos": pos, "vel": vel, "q_param": qp, "q": q[:, :P], "orbit": fo[:, :P],
            "collect": fc[:, :P], "dust": fd[:, :P], "field": ff[:, :P], "n_inj": ninj,
            "dN": dN[:, :P]}


def ion_potential_grid(holder, pos, gr, gz, round32=True):
    """(len(gz), len(gr)) sum over ions of exp(-r)/(r + r_0) at (gr[i], 0, gz[j]) (units of r_D_e)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    gr = np.ascontiguousarray(gr, dtype=np.float64)
    gz = np.ascontiguousarray(gz, dtype=np.float64)
    pot = np.empty((len(gz), len(gr)))
    rc = load().odo_ion_potential_grid(_cfg(holder), _p(pos), len(pos), int(round32), _p(gr), _p(gz),
                                       len(gr), len(gz), _p(pot))
    if rc:
        raise ValueError("oracle rejected the configuration")
    return pot
