"""Drop-in replacement for the reference's ``chains/matthews.py`` fork of OpenDust.

Same classes and arguments as the fork: ``DustParticle``, ``PlasmaParametersInSIUnitsMatthews``
(matthews.py:50-112: externalFieldOrder 0 or 2 with ``Phi_parameters`` {"E_0", "alpha", "beta",
"z1", "z7"}, each [value, unit]), ``SimulatioParametersInSIUnits`` (matthews.py:123-153, also
under the corrected spelling), ``OutputParameters`` with ``trapFileName`` (matthews.py:166-191)
and ``OpenDust(plasma, simulation, output, dustParticles)`` whose
``simulate(deviceIndex, cutOff, toRestartFileName, considerTrap, trapFileName)``
(matthews.py:303-1101) runs on one GPU through the C ABI. The fork's physics, as the library
implements it (distribution OD_DIST_MATTHEWS):

* ions enter through the top face only (shifted Maxwellian flux of Mach M); ions that leave
  through |z| = H/2 or hit a grain re-enter there; ions that cross the side wall are reflected
  (radial velocity reversed, matthews.py:653-682);
* per-component charge-exchange collisions with probability d_t * w_c (matthews.py:600-607);
* the trap is a radial polynomial with height-dependent coefficients alpha_k(h), fitted per
  height from the screened potential of the simulation's own initial ions (matthews.py:397-440)
  or read from ``trapFileName`` (matthews.py:441-453), interpolated by natural cubic splines;
  ``considerTrap=False`` drops it;
* the field is uniform (order 0) or of order 2 (E_0 + alpha z + beta z^2 between z1 and z7,
  constant outside, matthews.py:484-495); every grain gets forceExternalField.

``DustDynamics`` is the GB300 form of the fork's outer loop
(examples/DustDynamics/TwoParticles/launch.py:113-224): the ions stay resident on the GPU while
the grains move between windows.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from . import setup_host as sh
from .opendust import DustParticle, OpenDust as _OpenDustBase, parse_device_index  # noqa: F401

NMPS = 1e3  # m/s per nm/ps


class PlasmaParametersInSIUnitsMatthews:
    def __init__(self, T_n, T_e, n_inf, externalFieldOrder, Phi_parameters, M, w_c, m_i):
        """Plasma of the fork (matthews.py:51-85): neutral and electron temperatures, density,
        field order and parameters, Mach number of the inflow, collision frequency, ion mass."""
        self.T_n = T_n
        self.T_e = T_e
        self.n_inf = n_inf
        self.externalFieldOrder = externalFieldOrder
        self.Phi_parameters = Phi_parameters
        self.M = M
        self.m_i = m_i
        self.k_B = 1.380649e-23
        self.e = -1.60217662e-19
        self.eps_0 = 8.85418781762039e-12
        self.m_e = 9.0938356e-31
        self.r_D_e = np.sqrt((self.eps_0 * self.k_B * self.T_e) / (self.e ** 2 * self.n_inf))
        self.v_B = np.sqrt(self.k_B * self.T_e / self.m_i)
        self.w_p_e = np.sqrt((self.n_inf * self.e ** 2) / (self.m_e * self.eps_0))
        self.w_p_i = np.sqrt((self.n_inf * self.e ** 2) / (self.m_i * self.eps_0))
        self.w_c = w_c
        self.v_T = np.sqrt(self.k_B * self.T_n / self.m_i)
        self.v_fl = M * self.v_B

    def printParameters(self):
        print("#########################################")
        print("##### Plasma parameters in SI units #####")
        print("#########################################")
        print("\n")
        print("Neutral gas temperature T_n = {} K".format(self.T_n))
        print("Electron temperature T_e = {} K".format(self.T_e))
        print("Unperturbed density of the plasma in the quasineutral plasma region = {} 1/m**3"
              .format(self.n_inf))
        print("Mach number of the ions entering the simulation domain  M = {}".format(self.M))
        print("Ion mass m_i = {} kg".format(self.m_i))
        print("Electron Debye radius r_D_e = {} m".format(self.r_D_e))
        print("Bohm velocity v_B = {} m/s".format(self.v_B))
        print("Electron plasma frequency w_p_e = {} radian/s".format(self.w_p_e))
        print("Ion plasma frequency w_p_i = {} radian/s".format(self.w_p_i))
        print("Thermal ion velocity v_T = {} m/s".format(self.v_T))
        print("Ion flow velocity v_fl = {} m/s".format(self.v_fl))
        print("Order of external electric field: {}".format(self.externalFieldOrder))
        for key in self.Phi_parameters:
            print("{} = {} ({})".format(key, self.Phi_parameters[key][0], self.Phi_parameters[key][1]))
        print("\n")


class SimulatioParametersInSIUnits:
    def __init__(self, R, H, N, n, d_t, plasmaParametersInSIUnits):
        """Domain radius and height, superion count, step count and step (matthews.py:124-141)."""
        n_inf = plasmaParametersInSIUnits.n_inf
        r_D_e = plasmaParametersInSIUnits.r_D_e
        self.R = R
        self.H = H
        self.N = N
        self.n = n
        self.N_s = np.pi * R ** 2 * H * n_inf / self.N
        self.d_t = d_t
        self.r_0 = r_D_e * 1.0e-3

    def printParameters(self):
        print("#########################################")
        print("### Simulation parameters in SI units ###")
        print("#########################################")
        print("\n")
        print("Radius of the cylindrical computational domain R = {} m".format(self.R))
        print("Height of the cylindrical computational domain H = {} m".format(self.H))
        print("Number of superions N = {}".format(self.N))
        print("Number of ions in one superion N_s = {}".format(self.N_s))
        print("Integration time step d_t = {} s".format(self.d_t))
        print("Number of time steps n = {}".format(self.n))
        print("\n")


SimulationParametersInSIUnits = SimulatioParametersInSIUnits


class OutputParameters:
    def __init__(self, nOutput=10, nFileOutput=10, csvOutputFileName="", xyzOutputFileName="",
                 restartFileName="", trapFileName=""):
        """Output frequencies and file names (matthews.py:166-191); the trap table is written
        to trapFileName at the end of a run."""
        self.nOutput = nOutput
        self.nFileOutput = nFileOutput
        self.csvOutputFileName = csvOutputFileName
        self.xyzOutputFileName = xyzOutputFileName
        self.restartFileName = restartFileName
        self.trapFileName = trapFileName


def grain_field(plasma, grains_z) -> np.ndarray:
    """Field [V/m] at each grain height as the fork's tail uses it."""
    return np.array([sh.matthews_field_at(plasma.externalFieldOrder, plasma.Phi_parameters, z)
                     for z in grains_z], dtype=np.float64)


def build_matthews(plasma, sim, dustParticles, *, cutOff=False, seed=0, sim_id=0, avg_start=None,
                   trap_table=None, consider_trap=True, n_steps=None):
    """od_config of the fork's model. trap_table: (5, n) alpha table or None (then a tabulated
    trap is set later with Engine.set_trap_table, or none when consider_trap is False)."""
    phi = plasma.Phi_parameters
    order = int(plasma.externalFieldOrder)
    if order not in (0, 2):
        raise ValueError("externalFieldOrder must be 0 or 2")
    tables, _ = sh.injection_setup(plasma.v_fl, plasma.v_T, sim.R, sim.H, "Maxwellian")
    field = {"order": order}
    if order == 2:
        field.update(alpha=phi["alpha"][0], beta=phi["beta"][0], z1=phi["z1"][0], z7=phi["z7"][0])
    q_s = abs(plasma.e) * sim.N_s
    xyz = [(g.x, g.y, g.z) for g in dustParticles]
    gout = None
    if trap_table is not None:
        gout = sh.trap_table_out_factor(trap_table, sim.H, plasma.r_D_e, plasma.eps_0, q_s, xyz)
    if cutOff:
        method, rc = _lib.OD_FORCE_CUTOFF, 3.2 * plasma.r_D_e
        rs = rc * (3.0 / 3.2)
    else:
        method, rc, rs = _lib.OD_FORCE_ALLPAIRS, 0.0, 0.0
    n = sim.n if n_steps is None else n_steps
    grains = {
        "x": [g.x for g in dustParticles], "y": [g.y for g in dustParticles],
        "z": [g.z for g in dustParticles], "r": [g.r for g in dustParticles],
        "q0": [g.q for g in dustParticles],
        "method": [_lib.OD_CHARGE[g.chargeCalculationMethod] for g in dustParticles],
    }
    return _lib.make_config(
        distribution=_lib.OD_DIST_MATTHEWS, collision_model=_lib.OD_COLL_PER_DOF,
        force_method=method, n_ions=sim.N, n_steps=n,
        avg_start=n // 2 if avg_start is None else avg_start, seed=seed, sim_id=sim_id,
        consts={"k_B": plasma.k_B, "e": plasma.e, "eps_0": plasma.eps_0, "m_e": plasma.m_e},
        plasma={"T_e": plasma.T_e, "T_n": plasma.T_n, "n_inf": plasma.n_inf, "m_i": plasma.m_i,
                "r_D_e": plasma.r_D_e, "v_T": plasma.v_T, "v_fl": plasma.v_fl,
                "E": phi["E_0"][0], "w_c": plasma.w_c},
        sim={"R": sim.R, "H": sim.H, "d_t": sim.d_t, "r_0": sim.r_0, "N_s": sim.N_s,
             "cutoff": rc, "switch_dist": rs},
        alpha=np.zeros(15), probs=(1.0, 0.0, 0.0), tables=tables, grains=grains, field=field,
        trap_table=trap_table, trap_none=trap_table is None,
        grain_field=grain_field(plasma, [g.z for g in dustParticles]), grain_out=gout)


def fit_trap(eng, plasma, sim) -> np.ndarray:
    """The fork's trap fit from the engine's current ions (matthews.py:397-440)."""
    grid_R, grid_H = sh.matthews_trap_grid(sim.R, sim.H, plasma.r_D_e)
    pot = eng.ion_potential_grid(grid_R, grid_H)
    return sh.fit_trap_table(pot, grid_R, sim.N)


class OpenDust(_OpenDustBase):
    def __init__(self, plasmaParametersInSIUnits, simulationParametersInSIUnits, outputParameters,
                 dustParticles):
        """Main object of the fork (matthews.py:197-300): every grain has forceExternalField."""
        super().__init__(plasmaParametersInSIUnits, simulationParametersInSIUnits,
                         outputParameters, dustParticles, "Maxwellian")
        self.distributionType = "Matthews"
        for g in self.dustParticles:
            g.forceExternalField = np.zeros((self.n, 3))

    def simulate(self, deviceIndex="0", cutOff=False, toRestartFileName="", considerTrap=True,
                 trapFileName="", *, seed=0, quiet=False, avg_start=None, pair_plan=None):
        """Run n steps on one GPU (matthews.py:303-1101); returns (q, forces) as
        opendust.OpenDust.simulate and fills the same attributes."""
        plasma = self.plasmaParametersInSIUnits
        sim = self.simulationParametersInSIUnits
        out = self.outputParameters
        device = parse_device_index(deviceIndex)
        table = sh.read_trap_table(trapFileName) if (considerTrap and trapFileName) else None
        holder = build_matthews(plasma, sim, self._inputParticles, cutOff=cutOff, seed=seed,
                                avg_start=avg_start, trap_table=table, consider_trap=considerTrap)
        eng = _lib.Engine(holder, device)
        try:
            if pair_plan is not None:
                eng.set_pair_plan(*pair_plan)
            if toRestartFileName != "":
                pos, vel = sh.read_restart(toRestartFileName, self.N)
                eng.set_state(pos, vel)
            else:
                eng.init_state()
            if considerTrap and table is None:
                table = fit_trap(eng, plasma, sim)
                q_s = abs(plasma.e) * sim.N_s
                xyz = [(g.x, g.y, g.z) for g in self._inputParticles]
                eng.set_trap_table(table, sh.trap_table_out_factor(table, sim.H, plasma.r_D_e,
                                                                   plasma.eps_0, q_s, xyz))
            self.alphaTrap = table
            self._run_loop(eng, out, plasma, quiet)
            ser = eng.series(0, self.n)
            self.averages, _ = eng.averages()
        finally:
            eng.close()
        if getattr(out, "trapFileName", "") and table is not None:
            sh.write_trap_table(out.trapFileName, table)
        for p, g in enumerate(self.dustParticles):
            g.q[:] = ser["q"][:, p]
            g.forceIonsOrbit[:] = ser["orbit"][:, p]
            g.forceIonsCollect[:] = ser["collect"][:, p]
            g.forceDust[:] = ser["dust"][:, p]
            g.forceExternalField[:] = ser["field"][:, p]
        return ser["q"], {k: ser[k] for k in ("orbit", "collect", "dust", "field")}


class DustDynamics:
    """Grain dynamics over plasma windows with the ions resident on the GPU (the loop of
    examples/DustDynamics/TwoParticles/launch.py:113-224, which rebuilds an OpenDust object per
    iteration and passes the ions through a restart file).

    Each ``iteration()`` runs one window of sim.n steps with the grains fixed, averages each
    grain's charge and total force over the window, relaxes them as the reference does
    (new = 0.75 old + 0.25 window average) and moves the grains by one Langevin step of length
    d_t_p with gravity g, gas damping at pressure P and thermal kicks at temperature T_p
    (launch.py:207-224). Random kicks come from a seeded numpy generator."""

    def __init__(self, plasma, sim, dustParticles, *, rho=1500.0, d_t_p=5e-5, T_p=300.0, P=18.131842,
                 g=9.8, device=0, seed=0, consider_trap=True, trap_table=None, init_state=None):
        self.plasma, self.sim = plasma, sim
        self.rho, self.d_t_p, self.T_p, self.P, self.g = rho, d_t_p, T_p, P, g
        self.grains = [DustParticle(d.x, d.y, d.z, d.r, d.chargeCalculationMethod, d.q)
                       for d in dustParticles]
        Pn = len(self.grains)
        self.x = np.array([[d.x, d.y, d.z] for d in self.grains], dtype=np.float64)
        self.v = np.zeros((Pn, 3))
        self.f = np.zeros((Pn, 3))
        self.q = np.array([d.q for d in self.grains], dtype=np.float64)
        self.t = 0.0
        self.rng = np.random.default_rng(seed)
        self.q_s = abs(plasma.e) * sim.N_s
        self.consider_trap = consider_trap
        self.table = trap_table
        holder = build_matthews(plasma, sim, self.grains, seed=seed, trap_table=trap_table,
                                consider_trap=consider_trap)
        self._holder = holder
        self.eng = _lib.Engine(holder, device)
        if init_state is not None:
            self.eng.set_state(*init_state)
        else:
            self.eng.init_state()
        if consider_trap and self.table is None:
            self.table = fit_trap(self.eng, plasma, sim)
        self._push_grains()

    def _factors(self):
        gf = grain_field(self.plasma, self.x[:, 2])
        go = None
        if self.consider_trap and self.table is not None:
            go = sh.trap_table_out_factor(self.table, self.sim.H, self.plasma.r_D_e,
                                          self.plasma.eps_0, self.q_s, [tuple(p) for p in self.x])
        return gf, go

    def _push_grains(self):
        gf, go = self._factors()
        if self.consider_trap and self.table is not None:
            self.eng.set_trap_table(self.table, go)
        self.eng.set_grains(self.x[:, 0], self.x[:, 1], self.x[:, 2], self.q, gf, go)

    def iteration(self):
        """One window and one grain step; returns (x, v, f, q) after the step."""
        self.eng.begin_window()
        self.eng.step(self.sim.n)
        s = self.eng.series(0, self.sim.n)
        q_avg = s["q"].mean(axis=0)
        f_avg = (s["orbit"] + s["collect"] + s["dust"] + s["field"]).mean(axis=0)
        self.q = 0.75 * self.q + 0.25 * q_avg
        self.f = 0.75 * self.f + 0.25 * f_avg
        kB = self.plasma.k_B
        for p, d in enumerate(self.grains):
            m_p = 4.0 / 3.0 * np.pi * d.r ** 3 * self.rho * 1.05
            gamma = 8.0 / 3.0 * np.sqrt(2.0 * np.pi) * d.r ** 2 * self.P / self.plasma.v_T / m_p
            s_p = np.sqrt(2 * kB * self.T_p * m_p * gamma / self.d_t_p)
            f_th = self.rng.normal(0, s_p, 3) - m_p * gamma * self.v[p]
            a = (f_th + self.f[p]) / m_p
            a[2] += self.g
            self.x[p] = self.x[p] + self.v[p] * self.d_t_p + 0.5 * a * self.d_t_p ** 2
            self.v[p] = self.v[p] + a * self.d_t_p
        self.t += self.d_t_p
        self._push_grains()
        return self.x.copy(), self.v.copy(), self.f.copy(), self.q.copy()

    def close(self):
        if self.eng is not None:
            self.eng.close()
            self.eng = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
