"""The drop-in Python API end to end on the GPU: OpenDust(...).simulate() with the reference's
outputs (opendust.py:1046-1115) — console lines, XYZ frames, CSV snapshots, restart file — and a
restart from that file (opendust.py:452-466)."""
import numpy as np
import pytest

from opendust.opendust import (DustParticle, OpenDust, OutputParameters,
                               PlasmaParametersInSIUnitsMaxwell, SimulationParametersInSIUnits)

pytestmark = pytest.mark.gpu


def _objects(tmp_path, N=2048, n=6, method="consistent"):
    p = PlasmaParametersInSIUnitsMaxwell(290.11, 29011, 1e14, 1.0, 6.6335209e-26)
    s = SimulationParametersInSIUnits(3 * p.r_D_e, 6 * p.r_D_e, N, n, 3.5148240854e-09, p)
    out = OutputParameters(2, 2, str(tmp_path / "csv" / "trajectory"), str(tmp_path / "trajectory.xyz"),
                           str(tmp_path / "RESTART"))
    (tmp_path / "csv").mkdir(exist_ok=True)
    g = [DustParticle(0, 0, -p.r_D_e, 58.8e-6, method, 0.0),
         DustParticle(0, 0, p.r_D_e, 58.8e-6, "given", -1e-14)]
    return p, s, out, g


def test_simulate_outputs_and_restart(gpu_lib, tmp_path, capsys):
    p, s, out, g = _objects(tmp_path)
    od = OpenDust(p, s, out, g, "Maxwellian")
    q, forces = od.simulate("CUDA", "")          # the reference's legacy positional call
    printed = capsys.readouterr().out
    assert "Step: 0 out of 6" in printed and "Step: 4 out of 6" in printed
    assert q.shape == (6, 2) and forces["orbit"].shape == (6, 2, 3)
    assert od.dustParticles[0].q.shape == (6,) and od.dustParticles[0].forceIonsOrbit.shape == (6, 3)
    assert np.array_equal(od.dustParticles[1].q, np.full(6, -1e-14))   # "given" charge stays fixed
    assert od.dustParticles[0].q[0] == 0.0 and od.dustParticles[0].q[5] < 0  # electrons charge it
    assert od.dustParticles[0].forceDust[0, 2] == 0.0          # grain 0 uncharged at step 0
    assert np.all(od.dustParticles[0].forceDust[1:, 2] != 0)
    assert len(od.t) == 6
    xyz = (tmp_path / "trajectory.xyz").read_text().splitlines()
    assert len(xyz) == 3 * (2048 + 2) and xyz[0] == "2048" and xyz[1] == "0" and xyz[2].startswith("Ar\t")
    csv0 = (tmp_path / "csv" / "trajectory0.csv").read_text().splitlines()
    assert csv0[0] == "x,y,z,density,mass" and len(csv0) == 2049
    rs = np.loadtxt(tmp_path / "RESTART", delimiter="\t")
    assert rs.shape == (2048, 6)
    # restart from the file written above
    (tmp_path / "r2").mkdir()
    p2, s2, out2, g2 = _objects(tmp_path / "r2")
    od2 = OpenDust(p2, s2, OutputParameters(100, 100), g2, "Maxwellian")
    od2.simulate("0", toRestartFileName=str(tmp_path / "RESTART"), quiet=True)
    assert np.isfinite(od2.dustParticles[0].forceIonsOrbit).all()


def test_simulate_field_driven_and_cutoff(gpu_lib, tmp_path):
    from opendust.opendust import PlasmaParametersInSIUnitsFieldDriven

    p = PlasmaParametersInSIUnitsFieldDriven(300, 29011, 1e14, 40.0, 2e6, 6.6335209e-26)
    s = SimulationParametersInSIUnits(3 * p.r_D_e, 6 * p.r_D_e, 4096, 8, 1e-9, p)
    g = [DustParticle(0, 0, 0, 10e-6, "oml", -1e-14)]
    od = OpenDust(p, s, OutputParameters(100, 100), g, "fieldDriven")
    od.simulate("0", cutOff=True, quiet=True)
    d = od.dustParticles[0]
    assert np.allclose(d.forceExternalField[:, 2], d.q * p.E)
    assert np.isfinite(d.forceIonsOrbit).all() and np.isfinite(d.forceIonsCollect).all()


def test_bounded_wait_runs_out_and_context_survives(gpu_lib):
    # a wait that nothing completes gives up after its (test-only, short) poll limit and the
    # call reports OD_ERR_TIMEOUT; an armed-and-arrived wait returns OD_OK; the context is
    # still usable afterwards (a later engine steps normally)
    from opendust_gb300 import _lib as L
    lib = L.load()
    assert lib.od_selftest_wait(0, 1000, 0) == 5          # OD_ERR_TIMEOUT
    assert b"ran out" in lib.od_last_error(None)
    assert lib.od_selftest_wait(0, 1000, 1) == 0
    assert lib.od_selftest_wait(0, 0, 0) == 1          # OD_ERR_INVALID: limit out of range
    from tests._util import case
    holder, pos, vel, *_ = case(N=1024, n=2, seed=3)
    with L.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(2)
        assert np.isfinite(eng.series()["q"]).all()


def test_set_state_rejects_non_finite(gpu_lib):
    # a NaN or infinite position or velocity is refused before anything reaches the device, and
    # the handle keeps stepping from its last valid state
    from opendust_gb300 import _lib
    from tests._util import case

    holder, pos, vel, *_ = case(N=2048, n=2, seed=61)
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        bad = pos.copy()
        bad[17, 2] = np.nan
        with pytest.raises(_lib.OpenDustError) as e:
            eng.set_state(bad, vel)
        assert _lib.STATUS[e.value.status] == "OD_ERR_INVALID" and "not finite" in str(e.value)
        vbad = vel.copy()
        vbad[3, 0] = np.inf
        with pytest.raises(_lib.OpenDustError):
            eng.set_state(pos, vbad)
        eng.step(1)
        p, v = eng.get_state()
        assert np.isfinite(p).all() and np.isfinite(v).all()
