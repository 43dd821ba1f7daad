"""Generate tests/golden/opcounts.json: the floating-point operations per
cell-update of the reference algorithm, counted by running the CPU
restatement with an operation-counting scalar (oracle/opcount.cpp) over the
first steps of the two small benchmark workloads, for all four Riemann
solvers.  Run from the repository root:

    make -C oracle oracle && python tests/golden/make_opcounts.py

A cell-update is one full x+y split step of one interior cell; the counts
cover the whole time loop of scripts/cpu/main_cpu.cpp:217-262 (ghost fill,
compute_dt, advance_second_order) and so include the work the reference
repeats (each cell reconstructed twice per sweep, primitives re-derived in
every flux and Riemann call).  Categories: add (add and subtract), mul, div,
sqrt, pow (floating-point arithmetic), cmp, minmax, abs (comparisons,
fmin/fmax, fabs; not arithmetic).
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

ARITH = ("add", "mul", "div", "sqrt", "pow")

# (name, grid, initial state, cfl, t_end, counted steps)
WORKLOADS = (
    ("blast_256", lambda: O.Grid(256, 256, 0.0, 2.0, 0.0, 2.0),
     lambda port, g: port.init_blast(g), 0.8, 0.25, 10),
    ("shock_bubble_1000x396",
     lambda: O.Grid(1000, 396, 0.0, 0.225, 0.0, 0.089,
                    bc=("transmissive", "transmissive", "reflective", "reflective")),
     lambda port, g: port.init_shock_bubble(g), 0.8, 0.1, 4),
)


def count(name: str, solver: str) -> dict:
    for wname, mk_grid, mk_state, cfl, t_end, steps in WORKLOADS:
        if wname == name:
            g = mk_grid()
            U = mk_state(O.Oracle("port"), g)
            r = O.op_counts(U, g, cfl, t_end, solver, max_steps=steps)
            cu = g.nx * g.ny * r["steps"]
            per = {k: v / cu for k, v in r["counts"].items()}
            return dict(steps=r["steps"], cells=g.nx * g.ny, counts=r["counts"],
                        per_cell_update={k: round(v, 4) for k, v in per.items()},
                        arith_per_cell_update=round(sum(per[k] for k in ARITH), 4))
    raise KeyError(name)


def main() -> None:
    out = {"description": "floating-point operations per cell-update of the reference algorithm "
                          "(oracle/opcount.cpp over the first steps of each workload)",
           "arith_categories": list(ARITH), "workloads": {}}
    for wname, *_ in WORKLOADS:
        out["workloads"][wname] = {s: count(wname, s) for s in ("hll", "hllc", "exact", "force")}
    with open(os.path.join(HERE, "opcounts.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    for wname, by in out["workloads"].items():
        for s, r in by.items():
            print(f"{wname:24s} {s:6s} arith/cell-update {r['arith_per_cell_update']:8.1f}  {r['per_cell_update']}")


if __name__ == "__main__":
    main()
