"""Named synthetic workloads (seeded; SI units).

The reference measures on no public dataset: its benchmarks run OpenDust.simulate() on
synthetic plasmas (performance/*/benchmark.py). These builders give the parameter
objects for the five workloads this engine is measured on:

  small_plain   Ar+ (m=6.6335e-26 kg, T_i=300 K, T_e=2.5 eV, n_inf=1e14 m^-3), Mach 1
                Maxwellian inflow, no collisions, one grain r=1e-5 m at the origin with
                q0=0 and self-consistent charging, R=3 lambda, H=6 lambda, N=16384,
                d_t=1e-10 s, 2000 steps, all-pairs forces.
  full_plain    same physics, N=2^20, 20000 steps, charge-exchange collisions with a
                constant mean free path of 2 lambda.
  field_chain   field-driven ions, E set for Mach 0.5 with mean free path 1 lambda, five
                grains r=5e-6 m at z = -2..2 lambda on the axis, N=2^19, cutoff 2 lambda,
                30000 steps.
  cutoff_scaling  the reference's cutoff benchmark at scale k (N = k*2^15, H = k*6 lambda,
                cutoff 3.2 lambda with switching from 3.0 lambda, 3 steps).
  (the batched-sweep and serving-stream workloads draw their members from a seed; see
   sweep_member()).
"""
from __future__ import annotations

import numpy as np

from .opendust import (
    DustParticle,
    PlasmaParametersInSIUnitsFieldDriven,
    PlasmaParametersInSIUnitsMaxwell,
    SimulationParametersInSIUnits,
)

M_AR = 6.6335e-26
T_I = 300.0
T_E = 2.5 * 11604.518  # 2.5 eV in K
N_INF = 1e14


def small_plain(N: int = 16384, n: int = 2000, d_t: float = 1e-10, M: float = 1.0):
    plasma = PlasmaParametersInSIUnitsMaxwell(T_I, T_E, N_INF, M, M_AR)
    lam = plasma.r_D_e
    sim = SimulationParametersInSIUnits(3 * lam, 6 * lam, N, n, d_t, plasma)
    grains = [DustParticle(0.0, 0.0, 0.0, 1e-5, "consistent", 0.0)]
    return plasma, sim, grains, "Maxwellian", {}


def full_plain(N: int = 2**20, n: int = 20000):
    plasma, sim, grains, dist, _ = small_plain(N=N, n=n)
    return plasma, sim, grains, dist, {"collisions": "mfp", "mean_free_path": 2 * plasma.r_D_e}


def field_chain(N: int = 2**19, n: int = 30000, d_t: float = 1e-10):
    """Field-driven: the collision frequency used in v_fl = E|e|/(m_i w_c) is the mean
    charge-exchange rate <|v|>/mfp with <|v|> = sqrt(v_fl^2 + 8 v_T^2 / pi); E is solved
    for Mach 0.5 with that rate."""
    k_B = 1.380649e-23
    v_B = np.sqrt(k_B * T_E / M_AR)
    v_T = np.sqrt(k_B * T_I / M_AR)
    lam = np.sqrt((8.85418781762039e-12 * k_B * T_E) / ((1.60217662e-19) ** 2 * N_INF))
    mfp = 1.0 * lam
    v_fl = 0.5 * v_B
    w_c = np.sqrt(v_fl**2 + 8 * v_T**2 / np.pi) / mfp
    E = v_fl * M_AR * w_c / 1.60217662e-19
    plasma = PlasmaParametersInSIUnitsFieldDriven(T_I, T_E, N_INF, E, w_c, M_AR)
    sim = SimulationParametersInSIUnits(3 * lam, 6 * lam, N, n, d_t, plasma)
    grains = [DustParticle(0.0, 0.0, z * lam, 5e-6, "consistent", 0.0) for z in (-2, -1, 0, 1, 2)]
    return plasma, sim, grains, "fieldDriven", {
        "collisions": "mfp", "mean_free_path": mfp, "cutoff_distance": 2 * lam}


def cutoff_scaling(k: int = 8, n: int = 3):
    """The reference's own cutoff benchmark (performance/CutOff-Performance/benchmark.py:14-75)
    at scale k: Ar+ (m=6.6335209e-26 kg, T_i=290.11 K, T_e=29011 K, n_inf=1e14 m^-3), Mach 1
    Maxwellian inflow, R=3 lambda, H=k*6 lambda, N=k*2^15 (constant density), d_t=3.5148e-9 s,
    n=3 steps, one grain r=5.88e-6 m at z=-1 lambda with the given charge 392500 e, and
    simulate(cutOff=True): cutoff 3.2 lambda with OpenMM's switching from 3.0 lambda
    (performance/CutOff-Performance/opendust.py:480-484)."""
    plasma = PlasmaParametersInSIUnitsMaxwell(290.11, 29011.0, 1e14, 1.0, 6.6335209e-26)
    lam = plasma.r_D_e
    sim = SimulationParametersInSIUnits(3 * lam, k * 6 * lam, k * 2**15, n, 3.5148240854e-09, plasma)
    grains = [DustParticle(0.0, 0.0, -1 * lam, 58.8e-7, "given", 392500.0 * plasma.e)]
    return plasma, sim, grains, "Maxwellian", {"cutOff": True}


def sweep_member(seed: int, n_steps: int = 5000, max_log2n: int = 18):
    """One member of the batched sweep: N log-uniform in [2^14, 2^max_log2n], Mach in
    [0.1, 2], grain radius log-uniform in [1, 20] um, 1-4 grains on the axis, collisions
    on or off with p = 0.5."""
    rng = np.random.default_rng(seed)
    N = int(round(2 ** rng.uniform(14, max_log2n)))
    M = rng.uniform(0.1, 2.0)
    r = 10 ** rng.uniform(np.log10(1e-6), np.log10(20e-6))
    P = int(rng.integers(1, 5))
    plasma = PlasmaParametersInSIUnitsMaxwell(T_I, T_E, N_INF, M, M_AR)
    lam = plasma.r_D_e
    sim = SimulationParametersInSIUnits(3 * lam, 6 * lam, N, n_steps, 1e-10, plasma)
    zs = (np.arange(P) - (P - 1) / 2.0) * lam
    grains = [DustParticle(0.0, 0.0, z, r, "consistent", 0.0) for z in zs]
    ext = {"collisions": "mfp", "mean_free_path": 2 * lam} if rng.uniform() < 0.5 else {}
    return plasma, sim, grains, "Maxwellian", ext
