"""Extract the reference's published example results into tests/golden/reference_examples.json.

Reads the run logs and result files committed with the reference (OpenDust) under its
examples/ directory and records, for each run, the time-averaged forces (and, for the
field-driven Patacchini 2008 runs, the grain charge) together with the run's parameters taken
from the launch script next to them. The reference's runs are
unseeded, so these values pin the physics statistically, not bit for bit.

Usage (only where the reference tree is available):
    python tests/golden/make_golden.py /path/to/reference
"""
from __future__ import annotations

import json
import os
import re
import sys


def _mean_forces(path):
    txt = open(path).read()
    orb = float(re.search(r"Mean force from ions orbits = ([-0-9.e+]+)", txt).group(1))
    col = float(re.search(r"Mean force from collected ions = ([-0-9.e+]+)", txt).group(1))
    return orb, col


def main(ref):
    ex = os.path.join(ref, "examples")
    out = {"source": "OpenDust examples/ run logs (kolotinsky1998/opendust)", "runs": []}
    common = {"T_e": 29011.0, "T_i": 290.11, "n_inf": 1e14, "m_i": 6.6335209e-26,
              "R_lambda": 3.0, "H_lambda": 6.0, "d_t": 3.5148240854e-09, "grain_r": 58.8e-6,
              "distribution": "Maxwellian"}
    for method, log, N, q_e in (
        ("given", "Figure1/given/outputPiel2017Fig1Given", 2**19, 392500.0),
        ("consistent", "Figure1/consistent/outputPiel2017Fig1Consistent", 2**16, 0.0),
        ("oml", "Figure1/oml/outputPiel2017Fig1OML", 2**16, 0.0),
    ):
        orb, col = _mean_forces(os.path.join(ex, "Piel2017", log))
        out["runs"].append({
            **common, "name": f"piel2017_fig1_{method}", "source": f"examples/Piel2017/{log}",
            "M": 1.0, "N": N, "n": 3000, "avg_after": 1000, "grain_z_lambda": -1.0,
            "method": method, "q0_e": q_e, "F_orbit_z": orb, "F_collect_z": col})
    log = "Figure5/outputPiel2017Fig5"
    for line in open(os.path.join(ex, "Piel2017", log)):
        m = re.match(r"^([0-9.]+)\t([-0-9.e+]+)\t([-0-9.e+]+)\s*$", line)
        if m:
            M, orb, col = (float(x) for x in m.groups())
            out["runs"].append({
                **common, "name": f"piel2017_fig5_M{M}", "source": f"examples/Piel2017/{log}",
                "M": M, "N": 2**16, "n": 5000, "avg_after": 3000, "grain_z_lambda": 0.0,
                "method": "oml", "q0_e": 392500.0, "F_orbit_z": orb, "F_collect_z": col})
    # field-driven plasma (Patacchini 2008, Fig. 3): per collision frequency, the time averages
    # over steps > 150000 written by the launch script to charge.txt and force.txt
    fig = os.path.join(ex, "Patacchini2008", "Figure3")
    script = open(os.path.join(fig, "launchPatacchini2008Figure3.py")).read()

    def _array(name):
        body = re.search(name + r"\s*=\s*np\.asarray\(\s*\[(.*?)\]", script, re.S).group(1)
        return [float(x) for x in re.findall(r"[-0-9.e+]+", body)]

    w_c, E = _array("w_c_array"), _array("E_array")
    charge = [tuple(float(x) for x in line.split()) for line in open(os.path.join(fig, "charge.txt"))
              if line.strip()]
    force = [tuple(float(x) for x in line.split()) for line in open(os.path.join(fig, "force.txt"))
             if line.strip()]
    for k, (wc, e) in enumerate(zip(w_c, E)):
        qrow = next(r for r in charge if abs(r[0] / wc - 1) < 1e-6)
        frow = next(r for r in force if abs(r[0] / wc - 1) < 1e-6)
        out["runs"].append({
            "name": f"patacchini2008_fig3_p{k + 1}", "source": "examples/Patacchini2008/Figure3",
            "distribution": "fieldDriven", "T_e": 30000.0, "T_n": 300.0, "n_inf": 3.57167962497e15,
            "m_i": 1.673557e-27, "E": e, "w_c": wc, "R_lambda": 3.0, "H_lambda": 6.0,
            "N": 2**17, "n": 200000, "d_t": 1e-11, "avg_after": 150000, "grain_r": 1e-5,
            "grain_z_lambda": -1.0, "method": "consistent", "q0_e": 0.0, "q": qrow[1],
            "F_orbit_z": frow[1], "F_collect_z": frow[2]})
    # two grains of given charge (Piel 2017, Figs. 6 and 7): per point the time averages of
    # orbit + dust-dust force on each grain, (x, z), printed by the launch script as
    # "<parameter>\t<F1x>\t<F1z>\t<F2x>\t<F2z>" after its run log
    two = {"T_e": 29011.0, "T_i": 290.11, "n_inf": 1e14, "m_i": 6.6335209e-26, "R_lambda": 3.0,
           "H_lambda": 6.0, "N": 2**17, "distribution": "Maxwellian", "method": "given"}
    for fig, log, key in (("Figure6", "outputPiel2017Fig6", "M"), ("Figure7", "outputPiel2017Fig7", "d_x")):
        script = open(os.path.join(ex, "Piel2017", fig, f"launchPiel2017{fig}.py")).read()
        par = {
            "n": int(re.search(r"\bn = (\d+)", script).group(1)),
            "d_t": float(re.search(r"d_t = ([0-9.e+-]+)", script).group(1)),
            "grain_r": float(re.search(r"\br = ([0-9.e+-]+)", script).group(1)),
            "q0_e": float(re.search(r"q = ([0-9.e+-]+) \* plasmaParametersInSIUnits\.e", script).group(1)),
            "avg_after": int(re.search(r"if i > (\d+):", script).group(1)),
        }
        for line in open(os.path.join(ex, "Piel2017", fig, log)):
            m = re.match(r"^([0-9.]+)\t([-0-9.e+]+)\t([-0-9.e+]+)\t([-0-9.e+]+)\t([-0-9.e+]+)\s*$", line)
            if not m:
                continue
            v, f1x, f1z, f2x, f2z = (float(x) for x in m.groups())
            run = {**two, **par, "name": f"piel2017_{fig.lower().replace('figure', 'fig')}_{key}{v}",
                   "source": f"examples/Piel2017/{fig}/{log}", "M": v if key == "M" else 1.0,
                   "grains_lambda": [[0.0, 0.0, -0.5], [v if key == "d_x" else 0.5, 0.0, 0.5]],
                   "F1": [f1x, f1z], "F2": [f2x, f2z]}
            out["runs"].append(run)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_examples.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(out['runs'])} runs to {dst}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the opendust source tree>")
    main(sys.argv[1])
