"""The operation-counting build of the oracle (oracle/opcount.cpp): it runs
the restatement's arithmetic unchanged (bit-identical grids) and reproduces
the committed per-cell-update counts (tests/golden/opcounts.json, made by
tests/golden/make_opcounts.py)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("solver", ["hll", "hllc", "exact", "force"])
def test_counted_run_matches_oracle_bits(port, solver):
    g = O.Grid(40, 36, 0.0, 2.0, 0.0, 2.0, bc=("transmissive", "reflective", "transmissive", "reflective"))
    U = port.init_blast(g, cx=0.9, cy=1.1, r=0.45, p_in=4.0)
    want = U.copy()
    ref = port.run(want, g, 0.8, 0.25, solver, max_steps=6)
    r = O.op_counts(U, g, 0.8, 0.25, solver, max_steps=6)
    assert r["steps"] == ref["steps"] == 6
    assert np.array_equal(U, want)
    c = r["counts"]
    assert c["add"] > 0 and c["mul"] > 0 and c["div"] > 0 and c["sqrt"] > 0
    assert (c["pow"] > 0) == (solver == "exact")


def test_blast_256_counts_match_fixture(port, golden_dir):
    with open(os.path.join(golden_dir, "opcounts.json")) as f:
        fx = json.load(f)
    g = O.Grid(256, 256, 0.0, 2.0, 0.0, 2.0)
    U = port.init_blast(g)
    want = fx["workloads"]["blast_256"]["hllc"]
    r = O.op_counts(U, g, 0.8, 0.25, "hllc", max_steps=want["steps"])
    assert r["steps"] == want["steps"]
    assert r["counts"] == want["counts"]
    # the reference HLLC path: ~820 arithmetic operations per cell-update
    assert 700 < want["arith_per_cell_update"] < 950
