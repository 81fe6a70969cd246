"""Statistical parity with the reference's own published runs (tests/golden/).

The reference's example scripts print time-averaged grain forces (examples/Piel2017/...);
tests/golden/make_golden.py copied those numbers, with the run parameters, into
reference_examples.json. The GPU test re-runs a subset through the drop-in Python API
(OpenDust.simulate) with the same parameters and compares the same averages. The reference
runs are single unseeded Monte-Carlo runs, so the comparison is statistical.

Tolerances come from the seed-to-seed spread of this engine on the same runs (4 seeds each):
std(F_orbit_z) = 1.1 % (Fig. 1 consistent) and 1.2 % (Fig. 5, M = 1); std(F_collect_z) =
0.7 % of F_orbit. A difference of two independent runs has sqrt(2) times that spread, so the
bounds below (5 % of F_orbit for both forces) are about 3 sigma.

The Fig. 1 logs were printed by the current reference source (their parameter banners match
src/opendust/opendust.py:202-215). The Fig. 5 log was printed by an older version of
opendust.py (its banners read "Radius of cylindrical computational domain" and, for a
Maxwellian plasma, "Thermal neutral gas velocity"), so Fig. 5 pins the physics only loosely:
M = 1 agrees within 5 %, M = 0.5 differs by 10 % (6 sigma of our spread) and is checked at
15 %. At M = 2 the collection force is noisier: over 8 runs (seeds 1-4, with the directed-pair
and the each-pair-once all-pairs kernels, which agree) F_collect_z differs from the reference
log by +3.9 % +- 2.7 % of F_orbit and F_orbit_z by -2.6 % +- 1.6 %, so a single seed is checked
at 12 % (the mean plus 3 sigma).
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
RUNS = {r["name"]: r for r in json.load(open(os.path.join(HERE, "golden", "reference_examples.json")))["runs"]}


def test_golden_fixture_consistent():
    from opendust_gb300 import PlasmaParametersInSIUnitsMaxwell, SimulationParametersInSIUnits

    assert len(RUNS) == 46
    r = RUNS["piel2017_fig5_M2.0"]
    p = PlasmaParametersInSIUnitsMaxwell(r["T_i"], r["T_e"], r["n_inf"], r["M"], r["m_i"])
    s = SimulationParametersInSIUnits(3 * p.r_D_e, 6 * p.r_D_e, r["N"], r["n"], r["d_t"], p)
    # N_s printed by the reference run (examples/Piel2017/Figure5/outputPiel2017Fig5)
    assert s.N_s == pytest.approx(420.3631132989799, rel=1e-12)
    for run in RUNS.values():
        if run["distribution"] == "Maxwellian" and "F1" not in run:
            assert run["F_orbit_z"] > 0


def test_golden_fixture_field_driven():
    # the 13 field-driven runs of examples/Patacchini2008/Figure3 (Mach 1 at every collision
    # frequency); the parameter classes reproduce the values the reference printed in
    # examples/Patacchini2008/Figure3/outputPatacchini2008
    from opendust_gb300 import PlasmaParametersInSIUnitsFieldDriven, SimulationParametersInSIUnits

    runs = [r for r in RUNS.values() if r["distribution"] == "fieldDriven"]
    assert len(runs) == 13
    assert [r["w_c"] for r in runs] == sorted(r["w_c"] for r in runs)
    assert all(r["q"] < 0 for r in runs)
    r = runs[0]
    p = PlasmaParametersInSIUnitsFieldDriven(r["T_n"], r["T_e"], r["n_inf"], r["E"], r["w_c"], r["m_i"])
    assert p.r_D_e == pytest.approx(0.0002000000000000135, rel=1e-12)
    assert p.v_B == pytest.approx(15731.930327435968, rel=1e-12)
    assert p.M == pytest.approx(1.0000000012668968, rel=1e-12)
    s = SimulationParametersInSIUnits(3 * p.r_D_e, 6 * p.r_D_e, r["N"], r["n"], r["d_t"], p)
    assert s.N_s == pytest.approx(36.982493495016854, rel=1e-12)
    for r in runs:
        p = PlasmaParametersInSIUnitsFieldDriven(r["T_n"], r["T_e"], r["n_inf"], r["E"], r["w_c"],
                                                 r["m_i"])
        assert p.M == pytest.approx(1.0, rel=1e-6)


def test_golden_fixture_two_grains():
    # Piel 2017 Figs. 6 (7 Mach numbers) and 7 (11 lateral offsets of the second grain): two
    # grains of given charge, N = 2^17; the parameter classes reproduce the values the reference
    # printed in examples/Piel2017/Figure{6,7}/outputPiel2017Fig{6,7}
    from opendust_gb300 import PlasmaParametersInSIUnitsMaxwell, SimulationParametersInSIUnits

    two = [r for r in RUNS.values() if "F1" in r]
    assert sum(r["name"].startswith("piel2017_fig6_") for r in two) == 7
    assert sum(r["name"].startswith("piel2017_fig7_") for r in two) == 11
    for r in two:
        p = PlasmaParametersInSIUnitsMaxwell(r["T_i"], r["T_e"], r["n_inf"], r["M"], r["m_i"])
        s = SimulationParametersInSIUnits(r["R_lambda"] * p.r_D_e, r["H_lambda"] * p.r_D_e, r["N"],
                                          r["n"], r["d_t"], p)
        assert p.r_D_e == pytest.approx(0.001175403463213199, rel=1e-12)
        assert s.N_s == pytest.approx(210.18155664948995, rel=1e-12)
        assert len(r["grains_lambda"]) == 2 and r["method"] == "given"
    fig7 = sorted((r for r in two if "fig7" in r["name"]), key=lambda r: r["grains_lambda"][1][0])
    assert fig7[0]["grains_lambda"][1][0] == pytest.approx(0.00176) and fig7[-1]["grains_lambda"][1][0] == 1.0
    assert all(r["F2"][1] > r["F1"][1] > 0 for r in fig7)  # the downstream grain is pushed harder


def run_example(r, seed):
    from opendust_gb300 import (DustParticle, OpenDust, OutputParameters,
                                PlasmaParametersInSIUnitsMaxwell, SimulationParametersInSIUnits)

    p = PlasmaParametersInSIUnitsMaxwell(r["T_i"], r["T_e"], r["n_inf"], r["M"], r["m_i"])
    s = SimulationParametersInSIUnits(r["R_lambda"] * p.r_D_e, r["H_lambda"] * p.r_D_e, r["N"], r["n"],
                                      r["d_t"], p)
    g = DustParticle(0, 0, r["grain_z_lambda"] * p.r_D_e, r["grain_r"], r["method"], r["q0_e"] * p.e)
    od = OpenDust(p, s, OutputParameters(nOutput=10**9, nFileOutput=10**9), [g], "Maxwellian")
    od.simulate("0", seed=seed, quiet=True)
    k = r["avg_after"]
    d = od.dustParticles[0]
    return d.forceIonsOrbit[k + 1:, 2].mean(), d.forceIonsCollect[k + 1:, 2].mean()


@pytest.mark.gpu
@pytest.mark.parametrize("name,tol", [("piel2017_fig1_consistent", 0.05), ("piel2017_fig1_oml", 0.05),
                                      ("piel2017_fig5_M0.99598", 0.05), ("piel2017_fig5_M2.0", 0.12),
                                      ("piel2017_fig5_M0.49799", 0.15)])
def test_reference_example(gpu_lib, name, tol):
    r = RUNS[name]
    orb, col = run_example(r, seed=1)
    d_orb = (orb - r["F_orbit_z"]) / r["F_orbit_z"]
    d_col = (col - r["F_collect_z"]) / r["F_orbit_z"]
    print(f"{name}: F_orbit {orb:.4e} (ref {r['F_orbit_z']:.4e}, {100 * d_orb:+.1f}%), "
          f"F_collect {col:.4e} (ref {r['F_collect_z']:.4e}, {100 * d_col:+.1f}% of F_orbit)")
    assert abs(d_orb) < tol
    assert abs(d_col) < tol


def run_two_grains(r, seed, n=None, avg_after=None):
    """Time averages of orbit + dust-dust force (x, z) on each grain over steps > avg_after, as
    the reference's launch script computes them, and their standard errors from the means of 10
    consecutive blocks of the averaging window."""
    from opendust_gb300 import (DustParticle, OpenDust, OutputParameters,
                                PlasmaParametersInSIUnitsMaxwell, SimulationParametersInSIUnits)

    n = n or r["n"]
    avg_after = r["avg_after"] if avg_after is None else avg_after
    p = PlasmaParametersInSIUnitsMaxwell(r["T_i"], r["T_e"], r["n_inf"], r["M"], r["m_i"])
    lam = p.r_D_e
    s = SimulationParametersInSIUnits(r["R_lambda"] * lam, r["H_lambda"] * lam, r["N"], n, r["d_t"], p)
    g = [DustParticle(x * lam, y * lam, z * lam, r["grain_r"], r["method"], r["q0_e"] * p.e)
         for x, y, z in r["grains_lambda"]]
    od = OpenDust(p, s, OutputParameters(nOutput=10**9, nFileOutput=10**9), g, "Maxwellian")
    od.simulate("0", seed=seed, quiet=True)
    mean, se = [], []
    for d in od.dustParticles:
        f = (d.forceIonsOrbit + d.forceDust)[avg_after + 1:][:, [0, 2]]
        blocks = np.array([b.mean(0) for b in np.array_split(f, 10)])
        mean.append(f.mean(0))
        se.append(blocks.std(0, ddof=1) / np.sqrt(len(blocks)))
    return np.array(mean), np.array(se)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["piel2017_fig7_d_x0.00176", "piel2017_fig7_d_x0.50088"])
def test_reference_two_grain_example(gpu_lib, name):
    # Piel 2017 Fig. 7 (examples/Piel2017/Figure7): two grains of given charge, the second
    # displaced sideways by d_x; the reference's launch script protocol (5000 steps, averages
    # over steps > 2500) with seed 1. The reference's value is one unseeded run of the same
    # protocol, so the difference of the two means has about sqrt(2) times this run's standard
    # error; every component (x and z on both grains) is checked at 4 such errors.
    r = RUNS[name]
    mean, se = run_two_grains(r, seed=1)
    ref = np.array([r["F1"], r["F2"]])
    tol = 4 * np.sqrt(2) * se
    for g in range(2):
        print(f"{name} grain {g + 1}: F_x {mean[g, 0]:.3e} (ref {ref[g, 0]:.3e}, tol {tol[g, 0]:.1e}), "
              f"F_z {mean[g, 1]:.3e} (ref {ref[g, 1]:.3e}, tol {tol[g, 1]:.1e})")
    assert np.all(np.abs(mean - ref) <= tol)
    # the downstream grain is pushed harder along the flow
    assert mean[1, 1] > mean[0, 1] > 0
