"""GPU parity of the chains/matthews.py fork model against the CPU oracle, through the C ABI.

Tolerances (stated per test):
  * screened potential on the trap-fit grid: relative 1e-10 (FP64 sums in different orders);
  * one step from an identical state (tabulated trap, order-2 field, two grains, ions planted
    across the side wall, inside a grain and past the end planes): positions within 1e-5
    r_D_e, reflected velocities within 1e-5 relative, collected counts equal, charges within
    1e-9 relative;
  * 25 steps: positions within 1e-3 r_D_e, charge within 1e-6 relative;
  * a second window after moving the grains (od_set_grains + od_begin_window, Philox steps
    continuing) against the oracle started from the first window's final state: the same
    bounds as 25 steps;
  * OpenDust.simulate(): fitted trap written to and read back from the trap file.
"""
import numpy as np
import pytest

from opendust_gb300 import _lib
from opendust_gb300 import matthews as mt
from opendust_gb300 import setup_host as sh
from oracle import oracle

pytestmark = pytest.mark.gpu


def fork(N, n, grains_z=(-0.5, 0.5), q0=(-1e-15, -2e-15), w_c=2e6, M=1.0, table=True, seed=7):
    phi = {"E_0": [2600.0, "V/m"], "alpha": [2.4e6, "V/m^2"], "beta": [3.0e8, "V/m^3"],
           "z1": [-1.0e-3, "m"], "z7": [1.5e-3, "m"]}
    plasma = mt.PlasmaParametersInSIUnitsMatthews(290.0, 30000.0, 1e14, 2, phi, M, w_c, 6.6335209e-26)
    lam = plasma.r_D_e
    sim = mt.SimulatioParametersInSIUnits(1.25 * lam, 5 * lam, N, n, 2e-10, plasma)
    grains = [mt.DustParticle(0.0, 0.0, z * lam, 4.4e-6, "consistent", q) for z, q in zip(grains_z, q0)]
    pos, vel = sh.initial_state(N, sim.R, sim.H, [(g.x, g.y, g.z, g.r) for g in grains], plasma.v_fl,
                                plasma.v_T, "Maxwellian", seed)
    tab = None
    if table:
        grid_R, grid_H = sh.matthews_trap_grid(sim.R, sim.H, lam)
        holder0 = mt.build_matthews(plasma, sim, grains, consider_trap=False)
        tab = sh.fit_trap_table(oracle.ion_potential_grid(holder0, pos, grid_R, grid_H), grid_R, N)
    holder = mt.build_matthews(plasma, sim, grains, trap_table=tab, seed=seed)
    return holder, plasma, sim, grains, pos, vel, tab


def plant(pos, vel, plasma, sim):
    lam, R, H, vT = plasma.r_D_e, sim.R, sim.H, plasma.v_T
    p, v = pos.copy(), vel.copy()
    p[10] = [R * 0.9995, 0.0, 0.2 * lam]; v[10] = [60 * vT, 3 * vT, vT]          # side wall
    p[11] = [0.0, R * 0.9995, -0.9 * lam]; v[11] = [2 * vT, 50 * vT, 0.0]         # side wall
    p[12] = [1e-6, 0.0, -0.5 * lam]; v[12] = [0.0, 0.0, 0.0]                      # in grain 0
    p[13] = [0.1 * lam, 0.0, H / 2 * 0.99995]; v[13] = [0.0, 0.0, 40 * vT]       # bottom plane
    p[14] = [0.0, -0.1 * lam, -H / 2 * 0.99995]; v[14] = [0.0, 0.0, -40 * vT]    # top plane
    return p, v


def test_ion_potential_grid(gpu_lib):
    holder, plasma, sim, grains, pos, vel, tab = fork(4096, 4, table=False)
    grid_R, grid_H = sh.matthews_trap_grid(sim.R, sim.H, plasma.r_D_e)
    # the device sums over the absolute float positions derived from its cell-relative state
    ref = oracle.ion_potential_grid(holder, pos, grid_R, grid_H, round32=oracle.DEVICE_STATE)
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        got = eng.ion_potential_grid(grid_R, grid_H)
    rel = np.max(np.abs(got - ref) / np.abs(ref))
    print(f"grid potential {got.shape}: max rel {rel:.2e}")
    assert rel < 1e-10


def test_fork_one_step(gpu_lib):
    holder, plasma, sim, grains, pos, vel, tab = fork(2048, 4)
    pos, vel = plant(pos, vel, plasma, sim)
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(1)
        ser = eng.series()
        gp, gv = eng.get_state()
    ref = oracle.run(holder, pos, vel, 0, 1, round32=True)
    lam = plasma.r_D_e
    dpos = np.max(np.abs(gp - ref["pos"])) / lam
    print(f"fork one step: max |dx| {dpos:.2e} lambda, re-injected/reflected {ref['n_inj'][0]}")
    assert dpos < 1e-5
    # the two side-wall ions keep their position and have their radial velocity reversed
    for i in (10, 11):
        assert np.hypot(*ref["pos"][i, :2]) >= sim.R
        np.testing.assert_allclose(gv[i], ref["vel"][i], rtol=1e-5)
        vr_in = vel[i, :2] @ pos[i, :2] / np.hypot(*pos[i, :2])
        assert ref["vel"][i, :2] @ ref["pos"][i, :2] < 0 < vr_in
    for i in (12, 13, 14):
        assert gp[i, 2] == pytest.approx(-sim.H / 2, rel=1e-6)
    assert ref["dN"][0, 0] >= 1
    np.testing.assert_allclose(ser["q"], ref["q"], rtol=1e-9)
    np.testing.assert_allclose(ser["field"], ref["field"], rtol=1e-12)
    o_err = np.linalg.norm(ser["orbit"] - ref["orbit"]) / np.linalg.norm(ref["orbit"])
    assert o_err < 1e-4


def test_fork_multi_step(gpu_lib):
    holder, plasma, sim, grains, pos, vel, tab = fork(2048, 25)
    pos, vel = plant(pos, vel, plasma, sim)
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(25)
        ser = eng.series()
        gp, gv = eng.get_state()
    ref = oracle.run(holder, pos, vel, 0, 25, round32=True)
    dpos = np.max(np.abs(gp - ref["pos"])) / plasma.r_D_e
    qerr = np.max(np.abs(ser["q"] - ref["q"]) / np.abs(ref["q"]))
    print(f"fork 25 steps: max |dx| {dpos:.2e} lambda, q rel {qerr:.2e}, "
          f"re-injected/reflected {ref['n_inj'].sum()}")
    assert dpos < 1e-3
    assert qerr < 1e-6


def test_fork_grains_move_between_windows(gpu_lib):
    holder, plasma, sim, grains, pos, vel, tab = fork(2048, 12)
    lam = plasma.r_D_e
    new_z = np.array([-0.45, 0.55]) * lam
    new_q = np.array([-1.3e-15, -2.2e-15])
    q_s = abs(plasma.e) * sim.N_s
    xyz = [(0.0, 0.0, z) for z in new_z]
    gout = sh.trap_table_out_factor(tab, sim.H, lam, plasma.eps_0, q_s, xyz)
    gfield = mt.grain_field(plasma, new_z)
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(7)
        p1, v1 = eng.get_state()
        eng.set_grains(np.zeros(2), np.zeros(2), new_z, new_q, gfield, gout)
        eng.begin_window()
        eng.step(12)
        ser = eng.series()
        gp, _ = eng.get_state()
        assert eng.step_index == 12
    moved = [mt.DustParticle(0.0, 0.0, z, g.r, g.chargeCalculationMethod, q)
             for z, g, q in zip(new_z, grains, new_q)]
    holder2 = mt.build_matthews(plasma, sim, moved, trap_table=tab, seed=7)
    ref = oracle.run(holder2, p1, v1, 0, 12, q_param=new_q, round32=True, rng_base=7)
    dpos = np.max(np.abs(gp - ref["pos"])) / lam
    qerr = np.max(np.abs(ser["q"] - ref["q"]) / np.abs(ref["q"]))
    print(f"second window: max |dx| {dpos:.2e} lambda, q rel {qerr:.2e}")
    assert dpos < 1e-3 and qerr < 1e-6
    np.testing.assert_allclose(ser["q"][0], new_q, rtol=1e-15)


def test_fork_simulate_trap_file(gpu_lib, tmp_path):
    holder, plasma, sim, grains, pos, vel, tab = fork(2048, 6, table=False)
    trap = str(tmp_path / "trapFile.txt")
    od = mt.OpenDust(plasma, sim, mt.OutputParameters(100, 100, trapFileName=trap), grains)
    q, forces = od.simulate("0", quiet=True)
    assert q.shape == (6, 2) and np.isfinite(forces["orbit"]).all()
    assert np.all(od.dustParticles[0].forceExternalField[:, 2] != 0)
    written = sh.read_trap_table(trap)
    assert written.shape == (5, int(sim.H / plasma.r_D_e * 10))
    od2 = mt.OpenDust(plasma, sim, mt.OutputParameters(100, 100), grains)
    od2.simulate("0", quiet=True, trapFileName=trap)
    np.testing.assert_allclose(od2.alphaTrap, written, rtol=1e-15)
    od3 = mt.OpenDust(plasma, sim, mt.OutputParameters(100, 100), grains)
    od3.simulate("0", quiet=True, considerTrap=False)
    assert od3.alphaTrap is None and np.isfinite(od3.dustParticles[0].forceIonsOrbit).all()


def test_dust_dynamics_iterations(gpu_lib):
    holder, plasma, sim, grains, pos, vel, tab = fork(2048, 20, table=False)
    with mt.DustDynamics(plasma, sim, grains, seed=3) as dd:
        x0 = dd.x.copy()
        for _ in range(2):
            x, v, f, q = dd.iteration()
        assert np.all(np.isfinite(x)) and np.all(np.isfinite(f)) and np.all(q < 0)
        assert not np.allclose(x, x0)
        assert dd.eng.step_index == sim.n


def test_fork_time_averages(gpu_lib):
    # 300 steps of the fork model (tabulated trap, order-2 field, collisions, reflection):
    # time-averaged charge and orbit force within 1 % of the oracle
    holder, plasma, sim, grains, pos, vel, tab = fork(2048, 300)
    with _lib.Engine(holder) as eng:
        eng.set_state(pos, vel)
        eng.step(300)
        avg, navg = eng.averages()
    ref = oracle.run(holder, pos, vel, 0, 300, round32=True)
    assert navg == 150
    for g in range(2):
        dq = abs(avg[g, 0] - ref["q"][150:, g].mean()) / abs(ref["q"][150:, g].mean())
        o_ref = ref["orbit"][150:, g].mean(0)
        do = np.linalg.norm(avg[g, 1:4] - o_ref) / np.linalg.norm(o_ref)
        print(f"fork time averages grain {g}: q rel {dq:.2e}, orbit rel {do:.2e}")
        assert dq < 0.01 and do < 0.01
