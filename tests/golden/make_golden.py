"""Extract the reference's published example results into tests/golden/reference_examples.json.

Reads the run logs committed with the reference (OpenDust) under its examples/ directory
and records, for each run, the printed time-averaged forces together with the run's
parameters taken from the launch script next to the log. The reference's runs are
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
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_examples.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(out['runs'])} runs to {dst}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
