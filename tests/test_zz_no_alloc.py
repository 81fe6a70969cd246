"""od_ion_forces_static: the allocation-free ion–ion force entry point.

Callers that cannot allocate device memory (plug-ins inside another runtime's allocator,
loops that forbid cudaMalloc after start-up, frameworks that own every device buffer) pass
their own device arrays; the library's scratch is a fixed file-scope device array. This test
plays such a caller: it owns the position and force buffers (made with torch here), calls the
entry point through the C ABI twice in a row on different inputs, and checks each result
against the handle-based od_force_snapshot and against the FP64 CPU oracle, within the
tolerance of the other force tests (per-ion relative error 1e-5). Edge sizes (2 ions and the
array's full 32768) and the r_0 floor are covered too. This file is named so that pytest
collects it last.
"""
import ctypes

import numpy as np
import pytest

from opendust_gb300 import _lib
from oracle import oracle
from tests._util import case, rel_err_per_ion

pytestmark = pytest.mark.gpu


def _static_forces(lib, pos_np, plasma, sim, torch):
    n = pos_np.shape[0]
    pos_dev = torch.tensor(pos_np, dtype=torch.float64, device="cuda")
    out_dev = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
    k = 1.0 / (4.0 * np.pi * plasma.eps_0)
    q_s = abs(plasma.e) * sim.N_s
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.od_ion_forces_static(ctypes.c_void_p(pos_dev.data_ptr()), n, plasma.r_D_e, sim.r_0,
                                  k * q_s * q_s, ctypes.c_void_p(out_dev.data_ptr()),
                                  ctypes.c_void_p(stream))
    _lib.check(st, None)
    return out_dev.cpu().numpy()


def test_static_forces_match_snapshot_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    holder, pos_a, _, plasma, sim, _ = case(N=4096, n=4, seed=31)
    _, pos_b, _, _, _, _ = case(N=4096, n=4, seed=32)
    pos_b = pos_b[:3001]  # ragged size: exercises the padding of the scratch copy
    with _lib.Engine(holder) as eng:
        ref_a = eng.force_snapshot(pos_a)
        ref_b = eng.force_snapshot(pos_b)
    lib = _lib.load()
    got_a = _static_forces(lib, pos_a, plasma, sim, torch)
    free0 = torch.cuda.mem_get_info()[0]
    got_b = _static_forces(lib, pos_b, plasma, sim, torch)
    torch.cuda.synchronize()
    err_a = rel_err_per_ion(got_a, ref_a)
    err_b = rel_err_per_ion(got_b, ref_b)
    err_o = rel_err_per_ion(got_b, oracle.force_snapshot(holder, pos_b, round32=True))
    print(f"static vs snapshot: call 1 max {err_a.max():.3e}, call 2 max {err_b.max():.3e}; "
          f"call 2 vs FP64 oracle max {err_o.max():.3e}")
    assert np.isfinite(got_a).all() and np.isfinite(got_b).all()
    assert err_a.max() <= 1e-5
    assert err_b.max() <= 1e-5
    assert err_o.max() <= 1e-5
    # the second call took no device memory beyond the caller's two tensors (freed by torch's
    # caching allocator into its own pool, so free memory can only have dropped by them)
    assert torch.cuda.mem_get_info()[0] >= free0 - 2 * 3001 * 3 * 8 - (2 << 20)


def test_static_forces_rejects_oversize(gpu_lib):
    lib = _lib.load()
    st = lib.od_ion_forces_static(ctypes.c_void_p(16), 32769, 1e-3, 1e-6, 1.0, ctypes.c_void_p(16), None)
    assert st == 1
    assert b"32768" in lib.od_last_error(None)


@pytest.mark.parametrize("n", [2, 512, 32768])
def test_static_forces_edge_sizes_against_oracle(gpu_lib, n):
    torch = pytest.importorskip("torch")
    holder, pos, _, plasma, sim, _ = case(N=max(n, 2048), n=4, seed=33)
    pos = pos[:n]
    lib = _lib.load()
    got = _static_forces(lib, pos, plasma, sim, torch)
    got2 = _static_forces(lib, pos, plasma, sim, torch)  # second call on the same array
    idx = np.arange(n) if n <= 4096 else np.sort(np.random.default_rng(2).choice(n, 2048, replace=False))
    ref = oracle.force_targets(holder, pos, idx, round32=True)
    err = rel_err_per_ion(got[idx], ref)
    print(f"static n={n} vs FP64 oracle: max {err.max():.3e}")
    assert np.isfinite(got).all()
    assert err.max() <= 1e-5
    assert np.array_equal(got, got2)


def test_static_forces_rejects_tiny_r0(gpu_lib):
    # each ion's own pair has r = 0: r_0 below 1e-9 r_D_e would overflow FP32 there
    lib = _lib.load()
    st = lib.od_ion_forces_static(ctypes.c_void_p(16), 64, 1e-3, 0.0, 1.0, ctypes.c_void_p(16), None)
    assert st == 1
    assert b"r_0" in lib.od_last_error(None)
