"""Drop-in replacement for OpenDust's Python API (src/opendust/opendust.py).

Same classes, constructor arguments, attributes and result arrays as the reference:
``DustParticle`` (opendust.py:25-40), ``PlasmaParametersInSIUnitsMaxwell`` (:49-103),
``PlasmaParametersInSIUnitsFieldDriven`` (:112-171), ``SimulationParametersInSIUnits``
(:181-215, also under the alias ``SimulatioParametersInSIUnits`` used by the reference's
performance scripts), ``OutputParameters`` (:225-245) and ``OpenDust`` (:254-1383).

``OpenDust.simulate()`` runs the per-timestep superion update on one GPU through the
C ABI of libopendust_gb300.so instead of an OpenMM context. It fills
``dustParticles[p].q / forceIonsOrbit / forceIonsCollect / forceDust / forceExternalField``
and ``t`` exactly as the reference does and also returns ``(q, forces)``.
"""
from __future__ import annotations

import queue
import re
import threading

import numpy as np

from . import _lib
from . import setup_host as sh


class DustParticle:
    def __init__(self, x, y, z, r, chargeCalculationMethod, q=0.0):
        """Dust grain: centre (x, y, z) [m], radius r [m], charge method
        ("given" / "consistent" / "oml") and initial charge q [C] (opendust.py:25-40)."""
        self.x = x
        self.y = y
        self.z = z
        self.chargeCalculationMethod = chargeCalculationMethod
        self.q = q
        self.r = r


class PlasmaParametersInSIUnitsMaxwell:
    def __init__(self, T_i, T_e, n_inf, M, m_i):
        """Maxwellian plasma (opendust.py:49-77)."""
        self.T_n = T_i
        self.T_e = T_e
        self.n_inf = n_inf
        self.M = M
        self.m_i = m_i

        self.k_B = 1.380649e-23
        self.e = -1.60217662e-19
        self.eps_0 = 8.85418781762039e-12
        self.m_e = 9.0938356e-31

        self.r_D_e = np.sqrt((self.eps_0 * self.k_B * self.T_e) / (self.e**2 * self.n_inf))
        self.v_B = np.sqrt(self.k_B * self.T_e / self.m_i)
        self.w_p_e = np.sqrt((self.n_inf * self.e**2) / (self.m_e * self.eps_0))
        self.w_p_i = np.sqrt((self.n_inf * self.e**2) / (self.m_i * self.eps_0))
        self.v_T = np.sqrt(self.k_B * self.T_n / self.m_i)
        self.v_fl = self.M * self.v_B

    def printParameters(self):
        print("#########################################")
        print("##### Plasma parameters in SI units #####")
        print("#########################################")
        print("\n")
        print("Ion temperature T_i = {} K".format(self.T_n))
        print("Electron temperature T_e = {} K".format(self.T_e))
        print("Unperturbed density of the plasma in the quasineutral plasma region = {} 1/m**3".format(self.n_inf))
        print("Mach number of the ion flow M = {}".format(self.M))
        print("Ion mass m_i = {} kg".format(self.m_i))
        print("Electron Debye radius r_D_e = {} m".format(self.r_D_e))
        print("Bohm velocity v_B = {} m/s".format(self.v_B))
        print("Electron plasma frequency w_p_e = {} radian/s".format(self.w_p_e))
        print("Ion plasma frequency w_p_i = {} radian/s".format(self.w_p_i))
        print("Thermal ion velocity v_T = {} m/s".format(self.v_T))
        print("Ion flow velocity v_fl = {} m/s".format(self.v_fl))
        print("\n")


class PlasmaParametersInSIUnitsFieldDriven:
    def __init__(self, T_n, T_e, n_inf, E, w_c, m_i):
        """Field-driven plasma with ion–neutral collisions (opendust.py:112-143)."""
        self.T_n = T_n
        self.T_e = T_e
        self.n_inf = n_inf
        self.E = E
        self.m_i = m_i

        self.k_B = 1.380649e-23
        self.e = -1.60217662e-19
        self.eps_0 = 8.85418781762039e-12
        self.m_e = 9.0938356e-31

        self.r_D_e = np.sqrt((self.eps_0 * self.k_B * self.T_e) / (self.e**2 * self.n_inf))
        self.v_B = np.sqrt(self.k_B * self.T_e / self.m_i)
        self.w_p_e = np.sqrt((self.n_inf * self.e**2) / (self.m_e * self.eps_0))
        self.w_p_i = np.sqrt((self.n_inf * self.e**2) / (self.m_i * self.eps_0))
        self.w_c = w_c
        self.v_T = np.sqrt(self.k_B * self.T_n / self.m_i)
        self.v_fl = self.E * abs(self.e) / self.m_i / self.w_c
        self.M = self.v_fl / self.v_B

    def printParameters(self):
        print("#########################################")
        print("##### Plasma parameters in SI units #####")
        print("#########################################")
        print("\n")
        print("Neutral gas temperature T_n = {} K".format(self.T_n))
        print("Electron temperature T_e = {} K".format(self.T_e))
        print("Unperturbed density of the plasma in the quasineutral plasma region n_inf = {} 1/m**3".format(self.n_inf))
        print("Mach number of the ion flow M = {}".format(self.M))
        print("Ion mass m_i = {} kg".format(self.m_i))
        print("Electron Debye radius r_D_e = {} m".format(self.r_D_e))
        print("Bohm velocity v_B = {} m/s".format(self.v_B))
        print("Electron plasma frequency w_p_e = {} radian/s".format(self.w_p_e))
        print("Ion plasma frequency w_p_i = {} radian/s".format(self.w_p_i))
        print("Thermal neutral gas velocity v_T = {} m/s".format(self.v_T))
        print("Ion flow velocity v_fl = {} m/s".format(self.v_fl))
        print("Ion-neutral collision frequency w_c = {} 1/s".format(self.w_c))
        print("External electric field E = {} V/m".format(self.E))
        print("\n")


class SimulationParametersInSIUnits:
    def __init__(self, R, H, N, n, d_t, plasmaParametersInSIUnits):
        """Cylinder radius R and height H [m], N superions, n steps of d_t [s] (opendust.py:181-200)."""
        n_inf = plasmaParametersInSIUnits.n_inf
        r_D_e = plasmaParametersInSIUnits.r_D_e
        self.R = R
        self.H = H
        self.N = N
        self.n = n
        self.N_s = np.pi * R**2 * H * n_inf / self.N
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


SimulatioParametersInSIUnits = SimulationParametersInSIUnits


class OutputParameters:
    def __init__(self, nOutput=10, nFileOutput=10, csvOutputFileName="", xyzOutputFileName="",
                 restartFileName=""):
        """Console/file output cadence and file names (opendust.py:225-245)."""
        self.nOutput = nOutput
        self.nFileOutput = nFileOutput
        self.csvOutputFileName = csvOutputFileName
        self.xyzOutputFileName = xyzOutputFileName
        self.restartFileName = restartFileName


def parse_device_index(deviceIndex) -> int:
    """First integer in the reference's DeviceIndex string ("0", "0,1,2"); anything
    non-numeric (the legacy positional "CUDA" / "" forms) selects device 0."""
    if isinstance(deviceIndex, int):
        return deviceIndex
    m = re.match(r"\s*(\d+)", str(deviceIndex))
    return int(m.group(1)) if m else 0


def build_simulation(plasma, sim, dustParticles, distributionType, *, cutOff=False,
                     cutoff_distance=None, switch_distance=None, collisions=None,
                     mean_free_path=None, seed=0, avg_start=None, sim_id=0, trap=None,
                     device=0, n_steps=None, injection=None, force_every=1):
    """od_config for one simulation plus the host-side setup products.

    injection: precomputed (tables, probs) of setup_host.injection_setup, or None.
    trap: None -> Monte-Carlo grid on the GPU (od_trap_potential) + host least squares;
          an array of 15 coefficients -> used as alpha;
          a callable (Rh, Hh, n_r, n_h, n_points, seed) -> potential grid.
    collisions: None -> the reference's model (per-DOF constant w_c for fieldDriven, none
          for Maxwellian); "none"; "mfp" -> constant mean free path `mean_free_path` [m].
    force_every: ion–ion force interval k (1: every step, the reference's integrator; k > 1:
          impulse multiple time stepping, od_config.force_every).
    """
    if int(force_every) < 1:
        raise ValueError("force_every must be >= 1")
    if distributionType not in ("Maxwellian", "fieldDriven"):
        raise ValueError("distributionType must be 'Maxwellian' or 'fieldDriven'")
    dist = _lib.OD_DIST_MAXWELLIAN if distributionType == "Maxwellian" else _lib.OD_DIST_FIELD_DRIVEN
    if injection is None:
        injection = sh.injection_setup(plasma.v_fl, plasma.v_T, sim.R, sim.H, distributionType)
    tables, probs = injection
    Rh, Hh, n_r, n_h, n_points = sh.trap_grid(sim.R, sim.H, plasma.r_D_e)
    trap_seed = (int(seed) * 0x9E3779B97F4A7C15 + 0x51) & 0xFFFFFFFFFFFFFFFF
    if trap is None:
        pot = _lib.trap_potential(Rh, Hh, n_r, n_h, n_points, trap_seed, device)
        alpha = sh.fit_trap(pot, Rh, Hh, sim.N)
    elif callable(trap):
        pot = trap(Rh, Hh, n_r, n_h, n_points, trap_seed)
        alpha = sh.fit_trap(np.asarray(pot).reshape(n_r, n_h), Rh, Hh, sim.N)
    else:
        alpha = np.asarray(trap, dtype=np.float64)
    w_c = getattr(plasma, "w_c", 0.0)
    if collisions is None:
        coll = _lib.OD_COLL_PER_DOF if distributionType == "fieldDriven" else _lib.OD_COLL_NONE
    elif collisions == "none":
        coll = _lib.OD_COLL_NONE
    elif collisions == "mfp":
        if not mean_free_path or mean_free_path <= 0:
            raise ValueError("collisions='mfp' needs mean_free_path > 0")
        coll = _lib.OD_COLL_MFP
    elif collisions == "per_dof":
        coll = _lib.OD_COLL_PER_DOF
    else:
        raise ValueError("collisions must be None, 'none', 'mfp' or 'per_dof'")
    if cutOff or cutoff_distance is not None:
        method = _lib.OD_FORCE_CUTOFF
        rc = cutoff_distance if cutoff_distance is not None else 3.2 * plasma.r_D_e
        rs = switch_distance if switch_distance is not None else rc * (3.0 / 3.2)
    else:
        method, rc, rs = _lib.OD_FORCE_ALLPAIRS, 0.0, 0.0
    n = sim.n if n_steps is None else n_steps
    grains = {
        "x": [g.x for g in dustParticles],
        "y": [g.y for g in dustParticles],
        "z": [g.z for g in dustParticles],
        "r": [g.r for g in dustParticles],
        "q0": [g.q for g in dustParticles],
        "method": [_lib.OD_CHARGE[g.chargeCalculationMethod] for g in dustParticles],
    }
    holder = _lib.make_config(
        distribution=dist,
        collision_model=coll,
        force_method=method,
        n_ions=sim.N,
        n_steps=n,
        avg_start=n // 2 if avg_start is None else avg_start,
        seed=seed,
        sim_id=sim_id,
        consts={"k_B": plasma.k_B, "e": plasma.e, "eps_0": plasma.eps_0, "m_e": plasma.m_e},
        plasma={
            "T_e": plasma.T_e, "T_n": plasma.T_n, "n_inf": plasma.n_inf, "m_i": plasma.m_i,
            "r_D_e": plasma.r_D_e, "v_T": plasma.v_T, "v_fl": plasma.v_fl,
            "E": getattr(plasma, "E", 0.0), "w_c": w_c, "mfp": mean_free_path or 0.0,
        },
        sim={"R": sim.R, "H": sim.H, "d_t": sim.d_t, "r_0": sim.r_0, "N_s": sim.N_s,
             "cutoff": rc, "switch_dist": rs},
        alpha=alpha,
        probs=probs,
        tables=tables,
        grains=grains,
        force_every=int(force_every),
    )
    info = {"alpha": alpha, "tables": tables, "probs": probs, "trap_grid": (Rh, Hh, n_r, n_h, n_points)}
    return holder, info


class OpenDust:
    def __init__(self, plasmaParametersInSIUnits, simulationParametersInSIUnits, outputParameters,
                 dustParticles, distributionType):
        """Main object (opendust.py:255-360): keeps the parameter objects and the per-grain
        result arrays q[n], forceIonsCollect/forceIonsOrbit/forceDust[n,3] and, for
        fieldDriven, forceExternalField[n,3]."""
        self.plasmaParametersInSIUnits = plasmaParametersInSIUnits
        self.simulationParametersInSIUnits = simulationParametersInSIUnits
        self.outputParameters = outputParameters
        self.N = simulationParametersInSIUnits.N
        self.N_s = simulationParametersInSIUnits.N_s
        self.n = simulationParametersInSIUnits.n
        self.distributionType = distributionType
        self.k = 1.0 / (plasmaParametersInSIUnits.eps_0 * 4.0 * np.pi)
        self.e = plasmaParametersInSIUnits.e
        self.q_s = abs(plasmaParametersInSIUnits.e) * self.N_s
        if distributionType == "fieldDriven":
            self.E = plasmaParametersInSIUnits.E
        self.t = np.linspace(0, self.n * simulationParametersInSIUnits.d_t, self.n)
        self._inputParticles = list(dustParticles)

        class _Grain:
            def __init__(self, p, n, distributionType):
                self.x, self.y, self.z, self.r = p.x, p.y, p.z, p.r
                self.q = np.full(n, float(p.q))
                self.chargeCalculationMethod = p.chargeCalculationMethod
                self.forceIonsCollect = np.zeros((n, 3))
                self.forceIonsOrbit = np.zeros((n, 3))
                self.forceDust = np.zeros((n, 3))
                if distributionType == "fieldDriven":
                    self.forceExternalField = np.zeros((n, 3))

        self.dustParticles = [_Grain(p, self.n, distributionType) for p in dustParticles]
        self.numberOfDustParticles = len(self.dustParticles)
        self.alphaTrap = None
        self.averages = None

    def simulate(self, deviceIndex="0", cutOff=False, toRestartFileName="", *, seed=0,
                 collisions=None, mean_free_path=None, cutoff_distance=None,
                 switch_distance=None, avg_start=None, quiet=False, init="device",
                 pair_plan=None):
        """Run n steps on one GPU (opendust.py:362-1383). Returns (q, forces): q has shape
        (n, P); forces is a dict of (n, P, 3) arrays "orbit", "collect", "dust", "field".
        init: "device" samples the initial ions on the GPU (od_init_state), "host" with numpy
        (setup_host.initial_state); a restart file overrides both. pair_plan: all-pairs work
        decomposition (threads, ions per thread, variant[, jsplit or tile]) passed to
        od_set_pair_plan; None keeps the library's default for this ion count; "tuned" takes
        the autotuner's plan for this GPU model and size bucket from the persisted plan cache
        (tuning.tuned_plan: measured once on the initial state, then reused)."""
        plasma = self.plasmaParametersInSIUnits
        sim = self.simulationParametersInSIUnits
        out = self.outputParameters
        device = parse_device_index(deviceIndex)
        holder, info = build_simulation(
            plasma, sim, self._inputParticles, self.distributionType, cutOff=cutOff,
            cutoff_distance=cutoff_distance, switch_distance=switch_distance,
            collisions=collisions, mean_free_path=mean_free_path, seed=seed,
            avg_start=avg_start, device=device)
        self.alphaTrap = info["alpha"]
        pos = vel = None
        if toRestartFileName != "":
            pos, vel = sh.read_restart(toRestartFileName, self.N)
        elif init == "host":
            grains = [(g.x, g.y, g.z, g.r) for g in self._inputParticles]
            pos, vel = sh.initial_state(self.N, sim.R, sim.H, grains, plasma.v_fl, plasma.v_T,
                                        self.distributionType, seed)
        eng = _lib.Engine(holder, device)
        try:
            if pair_plan is not None and pair_plan != "tuned":
                eng.set_pair_plan(*pair_plan)
            if pos is not None:
                eng.set_state(pos, vel)
            elif self.distributionType == "fieldDriven":
                eng.init_state(sh.field_driven_vz_table(plasma.v_fl, plasma.v_T))
            else:
                eng.init_state()
            if pair_plan == "tuned" and not cutOff and cutoff_distance is None:
                from . import tuning
                tuning.tuned_plan(eng, device)
            self._run_loop(eng, out, plasma, quiet)
            ser = eng.series(0, self.n)
            self.averages, _ = eng.averages()
        finally:
            eng.close()
        for p, g in enumerate(self.dustParticles):
            g.q[:] = ser["q"][:, p]
            g.forceIonsOrbit[:] = ser["orbit"][:, p]
            g.forceIonsCollect[:] = ser["collect"][:, p]
            g.forceDust[:] = ser["dust"][:, p]
            if self.distributionType == "fieldDriven":
                g.forceExternalField[:] = ser["field"][:, p]
        forces = {k: ser[k] for k in ("orbit", "collect", "dust", "field")}
        return ser["q"], forces

    def _run_loop(self, eng, out, plasma, quiet):
        n = self.n
        nOutput = max(int(out.nOutput), 1)
        nFileOutput = max(int(out.nFileOutput), 1)
        want_files = bool(out.xyzOutputFileName or out.csvOutputFileName)
        if out.xyzOutputFileName:
            open(out.xyzOutputFileName, "w").close()
        # stop after every step i that prints or writes (i % nOutput == 0, i % nFileOutput == 0)
        marks = set(range(0, n, nOutput))
        if want_files:
            marks |= set(range(0, n, nFileOutput))
        marks.add(n - 1)
        writer = _FrameWriter(self, out, plasma) if want_files else None
        done = 0
        try:
            for i in sorted(marks):
                eng.step(i + 1 - done)
                done = i + 1
                if i % nOutput == 0 and not quiet:
                    if i == 0:
                        print("#########################################")
                        print("###        Start simulation           ###")
                        print("#########################################")
                        print("\n")
                    print("Step: {} out of {}".format(i, n))
                if writer is not None and i % nFileOutput == 0:
                    pos, _ = eng.get_state()
                    writer.put(pos * 1e9, i // nFileOutput)
        finally:
            if writer is not None:
                writer.close()
        if out.restartFileName:
            pos, vel = eng.get_state()
            sh.write_restart(out.restartFileName, pos, vel)

    def _write_frames(self, out, plasma, pos_nm, frame):
        """XYZ and CSV dumps in nm (opendust.py:1072-1098), written by the library's formatter:
        the same bytes as the reference's Python loops."""
        if out.xyzOutputFileName:
            _lib.write_xyz_frame(out.xyzOutputFileName, pos_nm, frame)
        if out.csvOutputFileName:
            _lib.write_csv_frame(out.csvOutputFileName + "{}.csv".format(frame), pos_nm,
                                 plasma.n_inf * 1e-27, self.N_s)


class _FrameWriter:
    """Writes the XYZ/CSV frames of one simulate() call on a background thread, in order, while
    the GPU steps on (the library's writer releases the GIL). At most two frames wait in memory;
    an error in a write is raised by the next put() or by close()."""

    def __init__(self, od, out, plasma):
        self._od, self._out, self._plasma = od, out, plasma
        self._q = queue.Queue(maxsize=2)
        self._err = None
        self._t = threading.Thread(target=self._run, name="opendust-frames", daemon=True)
        self._t.start()

    def _run(self):
        while True:
            item = self._q.get()
            if item is None:
                return
            if self._err is None:
                try:
                    self._od._write_frames(self._out, self._plasma, *item)
                except BaseException as e:  # noqa: BLE001 - re-raised on the caller's thread
                    self._err = e

    def put(self, pos_nm, frame):
        if self._err is not None:
            raise self._err
        self._q.put((pos_nm, frame))

    def close(self):
        self._q.put(None)
        self._t.join()
        if self._err is not None:
            raise self._err
