"""CPU tests: host-side logic of the drop-in API and the exported C ABI (no GPU calls)."""
import ctypes
import os
import re
import shutil

import numpy as np
import pytest

import opendust_gb300
from opendust_gb300 import _build, _lib, build_simulation, setup_host, workloads
from opendust_gb300.opendust import parse_device_index

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_import_paths():
    import opendust
    from opendust import OpenDust as A
    from opendust.opendust import OpenDust as B
    from opendust.opendust import SimulatioParametersInSIUnits, SimulationParametersInSIUnits

    assert A is B is opendust_gb300.OpenDust
    assert SimulatioParametersInSIUnits is SimulationParametersInSIUnits
    assert hasattr(opendust, "DustParticle")


def test_parameter_classes_derived_values():
    p = opendust_gb300.PlasmaParametersInSIUnitsMaxwell(290.11, 29011, 1e14, 1.0, 6.6335209e-26)
    # values printed by the reference run examples/Piel2017/Figure5/outputPiel2017Fig5
    assert p.r_D_e == pytest.approx(0.0011754034632131989, rel=1e-12)
    s = opendust_gb300.SimulationParametersInSIUnits(3 * p.r_D_e, 6 * p.r_D_e, 2**16, 5000, 3.5148240854e-09, p)
    assert s.R == pytest.approx(0.0035262103896395967, rel=1e-12)
    assert s.N_s == pytest.approx(420.3631132989799, rel=1e-12)
    f = opendust_gb300.PlasmaParametersInSIUnitsFieldDriven(300, 29011, 1e14, 10.0, 1e6, 6.6335209e-26)
    assert f.v_fl == pytest.approx(10.0 * 1.60217662e-19 / 6.6335209e-26 / 1e6)
    assert f.M == pytest.approx(f.v_fl / f.v_B)


@pytest.mark.parametrize("arg,dev", [("0", 0), ("1", 1), ("0,1,2", 0), ("3,4", 3), ("CUDA", 0), ("", 0), (2, 2)])
def test_device_index_parsing(arg, dev):
    assert parse_device_index(arg) == dev


def test_build_simulation_config():
    plasma, sim, grains, dist, ext = workloads.full_plain(N=4096, n=100)
    holder, info = build_simulation(plasma, sim, grains, dist, trap=np.arange(15.0), **ext)
    c = holder.cfg
    assert c.n_ions == 4096 and c.n_steps == 100 and c.avg_start == 50
    assert c.collision_model == _lib.OD_COLL_MFP and c.mfp == pytest.approx(2 * plasma.r_D_e)
    assert c.force_method == _lib.OD_FORCE_ALLPAIRS
    assert c.p_top + c.p_side + c.p_bottom == pytest.approx(1.0)
    assert list(c.alpha) == list(np.arange(15.0))
    assert c.grain_method[0] == _lib.OD_CHARGE["consistent"]
    # cutOff=True selects the reference's 3.2 / 3.0 lambda cutoff with switching
    h2, _ = build_simulation(plasma, sim, grains, dist, trap=np.zeros(15), cutOff=True)
    assert h2.cfg.force_method == _lib.OD_FORCE_CUTOFF
    assert h2.cfg.cutoff == pytest.approx(3.2 * plasma.r_D_e)
    assert h2.cfg.switch_dist == pytest.approx(3.0 * plasma.r_D_e)
    with pytest.raises(ValueError):
        build_simulation(plasma, sim, grains, "bogus", trap=np.zeros(15))


def test_initial_state_and_restart_roundtrip(tmp_path):
    plasma, sim, grains, dist, _ = workloads.small_plain(N=5000, n=10)
    g = [(x.x, x.y, x.z, x.r) for x in grains]
    pos, vel = setup_host.initial_state(sim.N, sim.R, sim.H, g, plasma.v_fl, plasma.v_T, dist, 3)
    assert pos.shape == (5000, 3)
    assert np.all(np.hypot(pos[:, 0], pos[:, 1]) <= sim.R)
    assert np.all(np.abs(pos[:, 2]) <= sim.H / 2)
    assert np.all(np.linalg.norm(pos, axis=1) > grains[0].r)
    assert abs(vel[:, 2].mean() - plasma.v_fl) < 5 * plasma.v_T / np.sqrt(5000)
    f = tmp_path / "RESTART"
    setup_host.write_restart(str(f), pos, vel)
    p2, v2 = setup_host.read_restart(str(f), 5000)
    np.testing.assert_allclose(p2, pos, rtol=1e-12)
    np.testing.assert_allclose(v2, vel, rtol=1e-12)


def _header_functions():
    src = open(os.path.join(ROOT, "include", "opendust_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(od_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def cpu_lib():
    if not os.path.exists(_build.LIB):
        if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
            pytest.skip("library not built and nvcc unavailable")
        _build.build()
    return ctypes.CDLL(_build.LIB)


def test_library_exports_every_declared_symbol(cpu_lib):
    names = _header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(cpu_lib, n), f"{n} declared in include/opendust_gb300.h but not exported"


def test_library_fails_loudly_without_gpu(cpu_lib):
    lib = _lib.load()
    assert lib.od_abi_version() == _lib.OD_ABI_VERSION
    if lib.od_device_count() > 0:
        pytest.skip("a GPU is visible")
    plasma, sim, grains, dist, ext = workloads.small_plain(N=1024, n=4)
    holder, _ = build_simulation(plasma, sim, grains, dist, trap=np.zeros(15))
    with pytest.raises(_lib.OpenDustError) as e:
        _lib.Engine(holder, 0)
    assert e.value.status == 6  # OD_ERR_UNSUPPORTED: no CUDA device, no CPU fallback
    with pytest.raises(_lib.OpenDustError):
        _lib.trap_potential(3.0, 6.0, 30, 30, 1000, 1)


def test_config_validation(cpu_lib):
    plasma, sim, grains, dist, ext = workloads.small_plain(N=1024, n=4)
    holder, _ = build_simulation(plasma, sim, grains, dist, trap=np.zeros(15))
    holder.cfg.n_grains = 17
    with pytest.raises(_lib.OpenDustError) as e:
        _lib.Engine(holder, 0)
    assert e.value.status == 1 and "n_grains" in str(e.value)
    holder.cfg.n_grains = 1
    holder.cfg.abi_version = 99
    with pytest.raises(_lib.OpenDustError) as e:
        _lib.Engine(holder, 0)
    assert e.value.status == 1


def test_batch_pair_plan_rule():
    # the plan a batch member steps with (host arithmetic only, no device call)
    assert _lib.batch_pair_plan(2048) == (256, 4, 7, 1024)
    assert _lib.batch_pair_plan(2**16) == (256, 4, 7, 1024)
    assert _lib.batch_pair_plan(2**16 + 1) == (256, 8, 7, 2048)
    assert _lib.batch_pair_plan(2**20) == (256, 8, 7, 2048)
    # the each-pair-once kernel needs 24 bytes of accumulators per ion, whatever the size
    assert _lib.batch_pair_plan(2**22) == (256, 8, 7, 2048)


def test_config_device_bytes_budget_rules():
    # host arithmetic only: the device memory od_create would allocate by default. The
    # each-pair-once kernels (all pairs and cutoff tile pairs) keep three 64-bit fixed-point
    # accumulators per ion instead of a tile-pair matrix, so no configuration needs more than
    # about 100 bytes per ion (plus the cutoff's tile-pair list, nT^2/2 entries)
    from opendust_gb300 import build_simulation, workloads

    def gb(builder, N):
        plasma, sim, grains, dist, ext = builder(N=N, n=4)
        holder, _ = build_simulation(plasma, sim, grains, dist, seed=1, trap=np.zeros(15), **ext)
        return _lib.config_device_bytes(holder) / 1e9

    assert gb(workloads.field_chain, 2**19) < 0.2
    assert gb(workloads.field_chain, 2**20) < 0.4
    assert gb(workloads.full_plain, 2**20) < 0.3
    assert gb(workloads.full_plain, 2**22) < 1.2
    assert gb(workloads.small_plain, 2**14) < 0.1
