"""Small drivers for profiling one kernel of the step with ncu (or timing it with CUDA events).

    python -m opendust_gb300.profiling pairs  --n 65536  --plan 256,1,5 --steps 2
    python -m opendust_gb300.profiling cutoff --n 131072 --variant 2    --steps 2
    python -m opendust_gb300.profiling cutoff --n 524288 --variant 3 --plan 256,2,3 --steps 2
    python -m opendust_gb300.profiling sweep  --n 65536,262144,1048576 [--plans '256,1,5;256,8,7']

`pairs` steps the small_plain workload with the given all-pairs plan, `cutoff` the field_chain
workload (cutoff 2 lambda; variants 0 and 2 walk a cell stencil, variant 3 with --plan takes the
tile pairs over Hilbert-sorted ions), both launching kernel by kernel (no CUDA graph) so that
`ncu -k regex:<kernel>` sees individual launches. `sweep` times every all-pairs plan with CUDA
events and prints pairs/s (a plan may carry the tile size as a fourth number, e.g. 256,8,7,2048).
"""
from __future__ import annotations

import argparse

from . import _lib, build_simulation, setup_host, workloads

PLANS = [(256, 1, 0), (128, 1, 0), (256, 1, 1), (128, 2, 2), (256, 2, 2), (128, 2, 3), (256, 2, 3),
         (128, 2, 4), (256, 2, 4), (128, 1, 5), (256, 1, 5), (128, 1, 6), (256, 1, 6),
         (256, 2, 7), (256, 4, 7)]


def _plain(N, n):
    plasma, sim, grains, dist, ext = workloads.small_plain(N=N, n=n)
    holder, _ = build_simulation(plasma, sim, grains, dist, seed=1, **ext)
    return holder


def run_pairs(N, plan, steps):
    with _lib.Engine(_plain(N, steps + 4)) as eng:
        eng.set_graph(False)
        eng.set_pair_plan(*plan)
        eng.init_state()
        eng.step(steps)
        print("ok", eng.pair_plan(), eng.series()["q"][-1])


def run_cutoff(N, variant, steps, plan=None):
    plasma, sim, grains, dist, ext = workloads.field_chain(N=N, n=steps + 4)
    holder, _ = build_simulation(plasma, sim, grains, dist, seed=1, **ext)
    with _lib.Engine(holder) as eng:
        eng.set_graph(False)
        eng.set_pair_plan(*(plan or (128, 1, variant)))
        eng.init_state(setup_host.field_driven_vz_table(plasma.v_fl, plasma.v_T))
        eng.step(steps)
        print("ok", eng.series()["q"][-1])


def run_sweep(sizes, plans=None):
    plans = plans or PLANS
    for N in sizes:
        with _lib.Engine(_plain(N, 22 * len(plans) + 8)) as eng:
            eng.init_state()
            steps = 2 if N >= 2**20 else (4 if N >= 2**18 else 20)
            for plan in plans:
                eng.set_pair_plan(*plan)
                eng.step(1)
                eng.set_timing(True)
                eng.step(steps)
                sm, ns, pm, pl = eng.timing()
                eng.set_timing(False)
                per = pm / pl * 1e-3
                print(f"N={N} plan={plan} {eng.pair_plan()} pair {pm / pl:.3f} ms "
                      f"{N * (N - 1) / per:.3e} pairs/s {N * (N - 1) * 25 / per / 1e12:.2f} TFLOP/s",
                      flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["pairs", "cutoff", "sweep"])
    ap.add_argument("--n", default="65536")
    ap.add_argument("--plan", default="256,1,5")
    ap.add_argument("--variant", type=int, default=2)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--plans", default="", help="sweep only these plans, e.g. '256,1,5;256,4,7'")
    a = ap.parse_args()
    if a.what == "pairs":
        run_pairs(int(a.n), tuple(int(x) for x in a.plan.split(",")), a.steps)
    elif a.what == "cutoff":
        plan = tuple(int(x) for x in a.plan.split(",")) if a.variant == 3 else None
        run_cutoff(int(a.n), a.variant, a.steps, plan)
    else:
        plans = [tuple(int(x) for x in p.split(",")) for p in a.plans.split(";") if p]
        run_sweep([int(x) for x in a.n.split(",")], plans)


if __name__ == "__main__":
    main()
