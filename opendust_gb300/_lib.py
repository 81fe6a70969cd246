"""ctypes binding of libopendust_gb300.so (the C ABI of include/opendust_gb300.h).

The library is built in-tree by ``opendust_gb300._build.build()``. There is no CPU
fallback: if the shared library is missing or no CUDA device is visible, the calls
below raise ``OpenDustError``.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int32, c_int64, c_uint32, c_uint64, c_void_p

import numpy as np

OD_ABI_VERSION = 3
OD_MAX_GRAINS = 16
OD_MAX_TABLE = 256
OD_NTAB = 4
OD_TAB_TOP, OD_TAB_BOTTOM, OD_TAB_SIDE, OD_TAB_VZ = 0, 1, 2, 3
OD_DIST_MAXWELLIAN, OD_DIST_FIELD_DRIVEN, OD_DIST_MATTHEWS = 0, 1, 2
OD_TRAP_POLY, OD_TRAP_TABLE, OD_TRAP_NONE = 0, 1, 2
OD_MAX_TRAP = 128
OD_CHARGE = {"given": 0, "consistent": 1, "oml": 2}
OD_COLL_NONE, OD_COLL_PER_DOF, OD_COLL_MFP = 0, 1, 2
OD_FORCE_ALLPAIRS, OD_FORCE_CUTOFF = 0, 1

STATUS = {
    0: "OD_OK",
    1: "OD_ERR_INVALID",
    2: "OD_ERR_CUDA",
    3: "OD_ERR_OOM",
    4: "OD_ERR_STATE",
    5: "OD_ERR_TIMEOUT",
    6: "OD_ERR_UNSUPPORTED",
    7: "OD_ERR_CAPACITY",
}

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libopendust_gb300.so")

_DP = POINTER(c_double)


class od_config(ctypes.Structure):
    """Mirror of ``od_config`` in include/opendust_gb300.h (field order matters)."""

    _fields_ = [
        ("abi_version", c_int32),
        ("distribution", c_int32),
        ("collision_model", c_int32),
        ("force_method", c_int32),
        ("n_ions", c_int64),
        ("n_steps", c_int64),
        ("avg_start", c_int64),
        ("n_grains", c_int32),
        ("sim_id", c_int32),
        ("seed", c_uint64),
        ("k_B", c_double),
        ("e", c_double),
        ("eps_0", c_double),
        ("m_e", c_double),
        ("T_e", c_double),
        ("T_n", c_double),
        ("n_inf", c_double),
        ("m_i", c_double),
        ("r_D_e", c_double),
        ("v_T", c_double),
        ("v_fl", c_double),
        ("E", c_double),
        ("w_c", c_double),
        ("mfp", c_double),
        ("R", c_double),
        ("H", c_double),
        ("d_t", c_double),
        ("r_0", c_double),
        ("N_s", c_double),
        ("cutoff", c_double),
        ("switch_dist", c_double),
        ("alpha", c_double * 15),
        ("p_top", c_double),
        ("p_side", c_double),
        ("p_bottom", c_double),
        ("tab_n", c_int32 * OD_NTAB),
        ("tab_v", _DP * OD_NTAB),
        ("tab_xi", _DP * OD_NTAB),
        ("tab_slope", _DP * OD_NTAB),
        ("grain_x", _DP),
        ("grain_y", _DP),
        ("grain_z", _DP),
        ("grain_r", _DP),
        ("grain_q0", _DP),
        ("grain_method", POINTER(c_int32)),
        ("field_order", c_int32),
        ("trap_kind", c_int32),
        ("field_alpha", c_double),
        ("field_beta", c_double),
        ("field_z1", c_double),
        ("field_z7", c_double),
        ("trap_n", c_int32),
        ("trap_tab", _DP),
        ("grain_field", _DP),
        ("grain_out", _DP),
        ("force_every", c_int32),
    ]


class OpenDustError(RuntimeError):
    """Raised when a C-ABI call returns a non-OK status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


_lib = None


def load(path: str | None = None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OpenDustError(
            6, f"{p} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
        )
    lib = ctypes.CDLL(p)
    H = c_void_p
    sig = {
        "od_abi_version": (c_int32, []),
        "od_version": (c_char_p, []),
        "od_device_count": (c_int32, []),
        "od_create": (c_int32, [POINTER(od_config), c_int32, POINTER(H)]),
        "od_destroy": (c_int32, [H]),
        "od_last_error": (c_char_p, [H]),
        "od_set_state": (c_int32, [H, _DP, _DP, c_int64]),
        "od_get_state": (c_int32, [H, _DP, _DP, c_int64]),
        "od_init_state": (c_int32, [H, _DP, _DP, c_int32]),
        "od_step": (c_int32, [H, c_int64]),
        "od_step_index": (c_int64, [H]),
        "od_get_series": (c_int32, [H, c_int64, c_int64, _DP, _DP, _DP, _DP, _DP]),
        "od_get_averages": (c_int32, [H, _DP, POINTER(c_int64)]),
        "od_force_snapshot": (c_int32, [H, _DP, c_int64, _DP]),
        "od_snapshot_positions": (c_int32, [H, _DP, c_int64, _DP]),
        "od_collect_flags": (
            c_int32,
            [H, _DP, c_int64, POINTER(c_int64), c_int64, POINTER(c_int64), POINTER(c_int64)],
        ),
        "od_set_timing": (c_int32, [H, c_int32]),
        "od_get_timing": (c_int32, [H, _DP, POINTER(c_int64), _DP, POINTER(c_int64)]),
        "od_set_graph": (c_int32, [H, c_int32]),
        "od_get_cutoff_pairs": (c_int32, [H, POINTER(c_int64)]),
        "od_probe_fp32_peak": (c_int32, [c_int32, _DP]),
        "od_selftest_wait": (c_int32, [c_int32, c_uint32, c_int32]),
        "od_shard_create": (c_int32, [POINTER(od_config), c_int64, c_int64, c_int32, c_int32,
                                      POINTER(c_void_p)]),
        "od_shard_set_state": (c_int32, [H, _DP, _DP]),
        "od_shard_begin": (c_int32, [H, c_void_p]),
        "od_shard_forces": (c_int32, [H, c_void_p, POINTER(c_int64)]),
        "od_shard_get_list": (c_int32, [H, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
        "od_shard_set_list": (c_int32, [H, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                        c_void_p, c_void_p]),
        "od_shard_finish": (c_int32, [H, c_void_p]),
        "od_shard_info": (c_int32, [H, POINTER(c_int64), POINTER(c_int64), POINTER(c_int64),
                                    POINTER(c_int64)]),
        "od_set_pair_plan": (c_int32, [H, c_int32, c_int32, c_int32, c_int32]),
        "od_get_pair_plan": (c_int32, [H, POINTER(c_int32)]),
        "od_autotune": (c_int32, [H, c_int32, _DP]),
        "od_batch_create": (c_int32, [c_int32, POINTER(c_void_p)]),
        "od_batch_add": (c_int32, [c_void_p, POINTER(od_config), _DP, _DP, POINTER(c_int32)]),
        "od_batch_remove": (c_int32, [c_void_p, c_int32]),
        "od_batch_set_plan": (c_int32, [c_void_p, c_int32, c_int32, c_int32]),
        "od_batch_member": (c_void_p, [c_void_p, c_int32]),
        "od_batch_size": (c_int32, [c_void_p]),
        "od_batch_step": (c_int32, [c_void_p, c_int64]),
        "od_batch_last_step_ms": (c_int32, [c_void_p, _DP]),
        "od_batch_pair_plan": (c_int32, [c_int64, POINTER(c_int32)]),
        "od_ion_potential_grid": (c_int32, [H, _DP, _DP, c_int32, c_int32, _DP]),
        "od_set_trap_table": (c_int32, [H, _DP, c_int32, _DP]),
        "od_set_grains": (c_int32, [H, _DP, _DP, _DP, _DP, _DP, _DP]),
        "od_begin_window": (c_int32, [H]),
        "od_batch_destroy": (c_int32, [c_void_p]),
        "od_batch_last_error": (c_char_p, [c_void_p]),
        "od_config_device_bytes": (c_int32, [POINTER(od_config), POINTER(c_int64)]),
        "od_device_memory": (c_int32, [c_int32, POINTER(c_int64), POINTER(c_int64)]),
        "od_ion_forces_static": (c_int32, [c_void_p, c_int64, c_double, c_double, c_double, c_void_p,
                                           c_void_p]),
        "od_trap_potential": (
            c_int32,
            [c_double, c_double, c_int32, c_int32, c_int64, c_uint64, c_int32, _DP],
        ),
        "od_write_xyz_frame": (c_int32, [c_char_p, _DP, c_int64, c_int64]),
        "od_write_csv_frame": (c_int32, [c_char_p, _DP, c_int64, c_double, c_double]),
        "od_format_double": (c_int32, [c_double, c_char_p]),
        "od_write_restart": (c_int32, [c_char_p, _DP, _DP, c_int64]),
        "od_read_restart": (c_int32, [c_char_p, c_int64, _DP, _DP]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if lib.od_abi_version() != OD_ABI_VERSION:
        raise OpenDustError(1, "library ABI version does not match the Python binding")
    _lib = lib
    return lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def check(status: int, handle=None):
    if status != 0:
        lib = load()
        msg = lib.od_last_error(handle)
        raise OpenDustError(status, msg.decode() if msg else "")


def device_count() -> int:
    return int(load().od_device_count())


class ConfigHolder:
    """An ``od_config`` plus the numpy arrays its pointers refer to (kept alive together)."""

    def __init__(self, cfg: od_config, keep: list):
        self.cfg = cfg
        self._keep = keep

    def ptr(self):
        return ctypes.byref(self.cfg)


def make_config(
    *,
    distribution: int,
    collision_model: int,
    force_method: int,
    n_ions: int,
    n_steps: int,
    avg_start: int,
    seed: int,
    sim_id: int,
    consts: dict,
    plasma: dict,
    sim: dict,
    alpha: np.ndarray,
    probs: tuple,
    tables: list,
    grains: dict,
    field: dict | None = None,
    trap_table: np.ndarray | None = None,
    trap_none: bool = False,
    grain_field=None,
    grain_out=None,
    force_every: int = 1,
) -> ConfigHolder:
    """Fill an od_config from plain Python/numpy values (SI units). field: order-2 field of the
    chains/matthews.py fork {"order", "alpha", "beta", "z1", "z7"}; trap_table: (5, n) alpha_k
    at uniform heights over [-H/2, H/2] (OD_TRAP_TABLE); trap_none: no trap (OD_TRAP_NONE);
    grain_field [P] (V/m) and grain_out [P, 3] (N/C): per-grain tail factors."""
    c = od_config()
    c.abi_version = OD_ABI_VERSION
    c.distribution = distribution
    c.collision_model = collision_model
    c.force_method = force_method
    c.force_every = int(force_every)
    c.n_ions = int(n_ions)
    c.n_steps = int(n_steps)
    c.avg_start = int(avg_start)
    c.n_grains = len(grains["x"])
    c.sim_id = int(sim_id)
    c.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    for k in ("k_B", "e", "eps_0", "m_e"):
        setattr(c, k, float(consts[k]))
    for k in ("T_e", "T_n", "n_inf", "m_i", "r_D_e", "v_T", "v_fl", "E", "w_c", "mfp"):
        setattr(c, k, float(plasma.get(k, 0.0)))
    for k in ("R", "H", "d_t", "r_0", "N_s", "cutoff", "switch_dist"):
        setattr(c, k, float(sim.get(k, 0.0)))
    for i in range(15):
        c.alpha[i] = float(alpha[i])
    c.p_top, c.p_side, c.p_bottom = (float(x) for x in probs)
    keep = []
    for t in range(OD_NTAB):
        v, xi, sl = tables[t]
        v = np.ascontiguousarray(v, dtype=np.float64)
        xi = np.ascontiguousarray(xi, dtype=np.float64)
        sl = np.ascontiguousarray(sl, dtype=np.float64)
        if len(v) > OD_MAX_TABLE:
            raise ValueError("injection table longer than OD_MAX_TABLE")
        keep += [v, xi, sl]
        c.tab_n[t] = len(v)
        c.tab_v[t] = _dptr(v)
        c.tab_xi[t] = _dptr(xi)
        c.tab_slope[t] = _dptr(sl)
    garr = {}
    for k in ("x", "y", "z", "r", "q0"):
        garr[k] = np.ascontiguousarray(grains[k], dtype=np.float64)
        keep.append(garr[k])
    gm = np.ascontiguousarray(grains["method"], dtype=np.int32)
    keep.append(gm)
    c.grain_x, c.grain_y, c.grain_z = _dptr(garr["x"]), _dptr(garr["y"]), _dptr(garr["z"])
    c.grain_r, c.grain_q0 = _dptr(garr["r"]), _dptr(garr["q0"])
    c.grain_method = gm.ctypes.data_as(POINTER(c_int32))
    if field:
        c.field_order = int(field.get("order", 0))
        c.field_alpha = float(field.get("alpha", 0.0))
        c.field_beta = float(field.get("beta", 0.0))
        c.field_z1 = float(field.get("z1", 0.0))
        c.field_z7 = float(field.get("z7", 0.0))
    c.trap_kind = OD_TRAP_NONE if trap_none else OD_TRAP_POLY
    if trap_table is not None:
        tt = np.ascontiguousarray(trap_table, dtype=np.float64)
        if tt.ndim != 2 or tt.shape[0] != 5 or not 4 <= tt.shape[1] <= OD_MAX_TRAP:
            raise ValueError("trap table must have shape (5, n), 4 <= n <= OD_MAX_TRAP")
        keep.append(tt)
        c.trap_kind = OD_TRAP_TABLE
        c.trap_n = tt.shape[1]
        c.trap_tab = _dptr(tt)
    if grain_field is not None:
        gf = np.ascontiguousarray(grain_field, dtype=np.float64)
        keep.append(gf)
        c.grain_field = _dptr(gf)
    if grain_out is not None:
        go = np.ascontiguousarray(grain_out, dtype=np.float64).reshape(-1)
        keep.append(go)
        c.grain_out = _dptr(go)
    return ConfigHolder(c, keep)


class Engine:
    """One simulation resident on one GPU (an ``od_handle``)."""

    def __init__(self, holder: ConfigHolder, device: int = 0, _handle=None):
        lib = load()
        self._lib = lib
        self.holder = holder
        self.n = int(holder.cfg.n_ions)
        self.P = int(holder.cfg.n_grains)
        self.n_steps = int(holder.cfg.n_steps)
        self._owned = _handle is None
        if _handle is None:
            h = c_void_p()
            check(lib.od_create(holder.ptr(), int(device), ctypes.byref(h)), None)
            self.h = h
        else:
            self.h = c_void_p(_handle)

    def close(self):
        if getattr(self, "h", None):
            if self._owned:
                self._lib.od_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_state(self, pos: np.ndarray, vel: np.ndarray):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        check(self._lib.od_set_state(self.h, _dptr(pos), _dptr(vel), pos.shape[0]), self.h)

    def init_state(self, vz_table=None):
        """Sample the initial state on the device; vz_table = (v [m/s], cdf) for field-driven."""
        if vz_table is None:
            check(self._lib.od_init_state(self.h, None, None, 0), self.h)
        else:
            v = np.ascontiguousarray(vz_table[0], dtype=np.float64)
            x = np.ascontiguousarray(vz_table[1], dtype=np.float64)
            check(self._lib.od_init_state(self.h, _dptr(v), _dptr(x), len(v)), self.h)

    def get_state(self):
        pos = np.empty((self.n, 3))
        vel = np.empty((self.n, 3))
        check(self._lib.od_get_state(self.h, _dptr(pos), _dptr(vel), self.n), self.h)
        return pos, vel

    def step(self, nsteps: int):
        check(self._lib.od_step(self.h, int(nsteps)), self.h)

    @property
    def step_index(self) -> int:
        return int(self._lib.od_step_index(self.h))

    def series(self, first: int = 0, count: int | None = None):
        if count is None:
            count = self.step_index - first
        P = self.P
        q = np.empty((count, P))
        fo, fc, fd, ff = (np.empty((count, P, 3)) for _ in range(4))
        check(
            self._lib.od_get_series(
                self.h, first, count, _dptr(q), _dptr(fo), _dptr(fc), _dptr(fd), _dptr(ff)
            ),
            self.h,
        )
        return {"q": q, "orbit": fo, "collect": fc, "dust": fd, "field": ff}

    def averages(self):
        out = np.empty((self.P, 13))
        n = c_int64()
        check(self._lib.od_get_averages(self.h, _dptr(out), ctypes.byref(n)), self.h)
        return out, int(n.value)

    def set_timing(self, enable: bool = True, count_pairs: bool = True):
        """Kernel-by-kernel steps with device events; count_pairs: the cutoff kernels also
        count the pairs inside the cutoff (cutoff_pairs())."""
        mode = 0 if not enable else (1 if count_pairs else 2)
        check(self._lib.od_set_timing(self.h, mode), self.h)

    def timing(self):
        """(step_ms, steps, pair_ms, pair_launches) summed since timing was enabled."""
        sm, pm = c_double(), c_double()
        st, pl = c_int64(), c_int64()
        check(self._lib.od_get_timing(self.h, ctypes.byref(sm), ctypes.byref(st), ctypes.byref(pm),
                                      ctypes.byref(pl)), self.h)
        return sm.value, st.value, pm.value, pl.value

    def ion_potential_grid(self, gr, gz) -> np.ndarray:
        """(len(gz), len(gr)) screened potential of the current ions at (gr[i], 0, gz[j]) in
        units of r_D_e (the fork's trap-fit grid)."""
        gr = np.ascontiguousarray(gr, dtype=np.float64)
        gz = np.ascontiguousarray(gz, dtype=np.float64)
        pot = np.empty((len(gz), len(gr)))
        check(self._lib.od_ion_potential_grid(self.h, _dptr(gr), _dptr(gz), len(gr), len(gz),
                                              _dptr(pot)), self.h)
        return pot

    def set_trap_table(self, table, grain_out=None):
        """Tabulated trap (5, n) alpha_k(h) (None: no trap) and per-grain out-of-domain factors."""
        if table is None:
            check(self._lib.od_set_trap_table(self.h, None, 0, None), self.h)
            return
        t = np.ascontiguousarray(table, dtype=np.float64)
        go = None if grain_out is None else np.ascontiguousarray(grain_out, dtype=np.float64)
        check(self._lib.od_set_trap_table(self.h, _dptr(t), t.shape[1],
                                          None if go is None else _dptr(go)), self.h)

    def set_grains(self, x, y, z, q, grain_field=None, grain_out=None):
        """Move the grains and set their charges (SI); ions stay resident."""
        arr = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z, q)]
        gf = None if grain_field is None else np.ascontiguousarray(grain_field, dtype=np.float64)
        go = None if grain_out is None else np.ascontiguousarray(grain_out, dtype=np.float64)
        check(self._lib.od_set_grains(self.h, *[_dptr(a) for a in arr],
                                      None if gf is None else _dptr(gf),
                                      None if go is None else _dptr(go)), self.h)

    def begin_window(self):
        """Restart the result series at row 0 (ion state and random streams continue)."""
        check(self._lib.od_begin_window(self.h), self.h)

    def set_pair_plan(self, threads: int, targets_per_thread: int, variant: int, jsplit: int = 0):
        """All-pairs work decomposition; for variant 7 `jsplit` is the tile size in ions."""
        check(self._lib.od_set_pair_plan(self.h, threads, targets_per_thread, variant, jsplit), self.h)

    def autotune(self, use_cache: bool = True) -> float:
        """Pick the fastest all-pairs plan on the current positions; returns pairs/s measured."""
        v = c_double()
        check(self._lib.od_autotune(self.h, int(use_cache), ctypes.byref(v)), self.h)
        return v.value

    def pair_plan(self):
        a = (c_int32 * 5)()
        check(self._lib.od_get_pair_plan(self.h, a), self.h)
        return dict(zip(("threads", "targets_per_thread", "variant", "jsplit", "chunk"), list(a)))

    def cutoff_pairs(self) -> int:
        """Pairs inside the cutoff evaluated while timing was enabled."""
        v = c_int64()
        check(self._lib.od_get_cutoff_pairs(self.h, ctypes.byref(v)), self.h)
        return v.value

    def set_graph(self, enable: bool = True):
        check(self._lib.od_set_graph(self.h, int(bool(enable))), self.h)

    def force_snapshot(self, pos: np.ndarray) -> np.ndarray:
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        f = np.empty_like(pos)
        check(self._lib.od_force_snapshot(self.h, _dptr(pos), pos.shape[0], _dptr(f)), self.h)
        return f

    def snapshot_positions(self, pos: np.ndarray) -> np.ndarray:
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        out = np.empty_like(pos)
        check(self._lib.od_snapshot_positions(self.h, _dptr(pos), pos.shape[0], _dptr(out)), self.h)
        return out

    def collect_flags(self, pos: np.ndarray, cap: int | None = None):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        cap = pos.shape[0] if cap is None else cap
        idx = np.empty(max(cap, 1), dtype=np.int64)
        cnt = c_int64()
        gc = np.zeros(max(self.P, 1), dtype=np.int64)
        st = self._lib.od_collect_flags(
            self.h,
            _dptr(pos),
            pos.shape[0],
            idx.ctypes.data_as(POINTER(c_int64)),
            cap,
            ctypes.byref(cnt),
            gc.ctypes.data_as(POINTER(c_int64)),
        )
        check(st, self.h)
        return idx[: cnt.value].copy(), int(cnt.value), gc[: self.P].copy()


def config_device_bytes(holder: ConfigHolder) -> int:
    """Device bytes a simulation with this configuration allocates (admission control)."""
    v = c_int64()
    check(load().od_config_device_bytes(holder.ptr(), ctypes.byref(v)), None)
    return int(v.value)


class Batch:
    """Many independent simulations stepped together (``od_batch``)."""

    def __init__(self, device: int = 0):
        self._lib = load()
        b = c_void_p()
        self._check(self._lib.od_batch_create(int(device), ctypes.byref(b)), None)
        self.b = b
        self._holders = {}

    def _check(self, st, b):
        if st != 0:
            msg = self._lib.od_batch_last_error(b)
            raise OpenDustError(st, msg.decode() if msg else "")

    def add(self, holder: ConfigHolder, pos: np.ndarray | None = None,
            vel: np.ndarray | None = None) -> int:
        """Add a member; without pos/vel its (Maxwellian) initial state is sampled on the device."""
        slot = c_int32()
        if pos is None:
            self._check(self._lib.od_batch_add(self.b, holder.ptr(), None, None, ctypes.byref(slot)),
                        self.b)
        else:
            pos = np.ascontiguousarray(pos, dtype=np.float64)
            vel = np.ascontiguousarray(vel, dtype=np.float64)
            self._check(self._lib.od_batch_add(self.b, holder.ptr(), _dptr(pos), _dptr(vel),
                                               ctypes.byref(slot)), self.b)
        self._holders[slot.value] = holder
        return slot.value

    def set_plan(self, slot: int, ions_per_lane: int, tile: int):
        """Each-pair-once shape of a member: (4, 1024) or (8, 2048)."""
        self._check(self._lib.od_batch_set_plan(self.b, int(slot), int(ions_per_lane), int(tile)),
                    self.b)

    def remove(self, slot: int):
        self._check(self._lib.od_batch_remove(self.b, int(slot)), self.b)
        self._holders.pop(slot, None)

    def member(self, slot: int) -> Engine:
        """Non-owning view of a member (series, averages, state)."""
        h = self._lib.od_batch_member(self.b, int(slot))
        if not h:
            raise OpenDustError(1, f"no batch member in slot {slot}")
        return Engine(self._holders[slot], _handle=h)

    def step(self, nsteps: int):
        self._check(self._lib.od_batch_step(self.b, int(nsteps)), self.b)

    def last_step_ms(self) -> float:
        v = c_double()
        self._lib.od_batch_last_step_ms(self.b, ctypes.byref(v))
        return v.value

    def __len__(self):
        return int(self._lib.od_batch_size(self.b))

    def close(self):
        if getattr(self, "b", None):
            self._lib.od_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def batch_pair_plan(n_ions: int) -> tuple:
    """(threads, targets per thread, variant, jsplit or tile) a batch member of n_ions steps
    with; Engine.set_pair_plan(*plan) makes a single simulation bitwise equal to it."""
    a = (c_int32 * 5)()
    check(load().od_batch_pair_plan(int(n_ions), a), None)
    return tuple(a[:4])


def _xyz_nm(pos_nm) -> np.ndarray:
    a = np.ascontiguousarray(pos_nm, dtype=np.float64)
    if a.ndim != 2 or a.shape[1] != 3:
        raise ValueError("positions must be an (n, 3) array")
    return a


def write_xyz_frame(path: str, pos_nm, frame: int):
    """Append one XYZ frame ("n", "frame", then "Ar\tx\ty\tz" per ion, nm) as the reference's
    simulate() writes it (opendust.py:1079-1084), byte for byte."""
    a = _xyz_nm(pos_nm)
    check(load().od_write_xyz_frame(os.fsencode(path), _dptr(a), a.shape[0], int(frame)))


def write_csv_frame(path: str, pos_nm, density: float, mass: float):
    """Write one CSV frame ("x,y,z,density,mass" rows, nm) as the reference's simulate() writes
    it with csv.writer (opendust.py:1086-1097), byte for byte."""
    a = _xyz_nm(pos_nm)
    check(load().od_write_csv_frame(os.fsencode(path), _dptr(a), a.shape[0], float(density),
                                    float(mass)))


def write_restart_file(path: str, pos_nm, vel_nmps):
    """The reference's restart file (opendust.py:1099-1115): "x\ty\tz\tvx\tvy\tvz" per ion in
    nm and nm/ps, byte for byte."""
    p, v = _xyz_nm(pos_nm), _xyz_nm(vel_nmps)
    if p.shape != v.shape:
        raise ValueError("positions and velocities differ in shape")
    check(load().od_write_restart(os.fsencode(path), _dptr(p), _dptr(v), p.shape[0]))


def read_restart_file(path: str, n: int):
    """The first n ions of a restart file: (positions nm, velocities nm/ps), each (n, 3)."""
    p = np.empty((n, 3))
    v = np.empty((n, 3))
    check(load().od_read_restart(os.fsencode(path), int(n), _dptr(p), _dptr(v)))
    return p, v


def format_double(v: float) -> str:
    """The library's formatting of one double (Python's repr of a float)."""
    buf = ctypes.create_string_buffer(40)
    n = load().od_format_double(float(v), buf)
    return buf.raw[:n].decode()


def fp32_peak_tflops(device: int = 0) -> float:
    """Measured FP32 FMA throughput of the device (TFLOP/s)."""
    t = c_double()
    check(load().od_probe_fp32_peak(int(device), ctypes.byref(t)), None)
    return t.value


def trap_potential(Rh: float, Hh: float, n_r: int, n_h: int, n_points: int, seed: int, device: int = 0):
    pot = np.empty(n_r * n_h)
    check(
        load().od_trap_potential(
            float(Rh), float(Hh), int(n_r), int(n_h), int(n_points), int(seed), int(device), _dptr(pot)
        ),
        None,
    )
    return pot.reshape(n_r, n_h)
