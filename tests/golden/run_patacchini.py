"""Re-run field-driven points of the reference's examples/Patacchini2008/Figure3 (stored in
reference_examples.json) through the drop-in API on the GPU and print the time averages next to
the reference's. A point is 200000 steps of 2^17 ions (about 20 minutes on one GB300), too long for
the test suite; the comparison it prints is recorded with the parity evidence.

Usage: python tests/golden/run_patacchini.py <point 1-13> [seed]
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main(point: int, seed: int = 0):
    from opendust_gb300 import (DustParticle, OpenDust, OutputParameters,
                                PlasmaParametersInSIUnitsFieldDriven, SimulationParametersInSIUnits)

    runs = json.load(open(os.path.join(HERE, "reference_examples.json")))["runs"]
    r = next(x for x in runs if x["name"] == f"patacchini2008_fig3_p{point}")
    p = PlasmaParametersInSIUnitsFieldDriven(r["T_n"], r["T_e"], r["n_inf"], r["E"], r["w_c"], r["m_i"])
    lam = p.r_D_e
    s = SimulationParametersInSIUnits(r["R_lambda"] * lam, r["H_lambda"] * lam, r["N"], r["n"],
                                      r["d_t"], p)
    g = DustParticle(0, 0, r["grain_z_lambda"] * lam, r["grain_r"], r["method"], r["q0_e"] * p.e)
    od = OpenDust(p, s, OutputParameters(nOutput=10**9, nFileOutput=10**9), [g], "fieldDriven")
    t0 = time.time()
    od.simulate("0", seed=seed, quiet=True)
    k = r["avg_after"]
    d = od.dustParticles[0]
    ours = (d.q[k + 1:].mean(), d.forceIonsOrbit[k + 1:, 2].mean(), d.forceIonsCollect[k + 1:, 2].mean())
    ref = (r["q"], r["F_orbit_z"], r["F_collect_z"])
    print(f"point {point} (w_c = {r['w_c']:.4e} 1/s, seed {seed}, {time.time() - t0:.0f} s)")
    for name, a, b in zip(("q", "F_orbit_z", "F_collect_z"), ours, ref):
        print(f"  {name:12s} ours {a: .4e}  reference {b: .4e}  ({100 * (a / b - 1):+.1f} %)")


if __name__ == "__main__":
    main(int(sys.argv[1]), int(sys.argv[2]) if len(sys.argv) > 2 else 0)
