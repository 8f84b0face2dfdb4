"""MPS reader semantics, and the oracle against SCIP itself on the MIPLIB instances that the reference ships
(check/instances/MIP/*.mps).  The second part runs only where the reference sources and the SCIP driver
built from them are present; the fixtures under tests/golden/miplib (written by tests/golden/make_golden.py from
those files and SCIP's results) carry the same instances to the GPU tests."""
import glob
import os

import numpy as np
import pytest

import golden_cases as G
from scip_gb300 import instances, mps
from scip_gb300.instances import INF

SMALL = """NAME          SMALL
ROWS
 N  obj
 L  c1
 G  c2
 E  c3
 E  c4
 L  c5
COLUMNS
    x         obj       1.0          c1        2.0
    x         c3        1.0
    MARKER                 'MARKER'                 'INTORG'
    y         c1        1.0          c2        1.0
    z         c2        3.0          c4        1.0
    w         c5        1.0
    b         c5        1.0
    MARKER                 'MARKER'                 'INTEND'
    u         c4        -1.0         c5        1.0
RHS
    RHS       c1        10.0         c2        2.0
    RHS       c3        4.0          c4        1.0
    RHS       c5        7.0
RANGES
    RNG       c3        2.5          c4        -1.5
    RNG       c5        3.0
BOUNDS
 UP BND       x         -2.0
 UP BND       y         5.0
 LO BND       z         -1.0
 UP BND       w         1.0
 BV BND       b
 FR BND       u
ENDATA
"""


def test_reader_semantics(tmp_path):
    p = tmp_path / "small.mps"
    p.write_text(SMALL)
    inst = mps.read_mps(str(p))
    # columns in order of appearance: x, y, z, w, b, u
    assert list(inst.isint) == [0, 1, 1, 1, 1, 0]
    # x: UP -2 with lower bound 0 -> (-inf, -2]; y: marker integer, UP 5 > 1 -> general integer [0, 5];
    # z: LO -1 on a marker integer -> general integer with an infinite upper bound; w: UP 1 keeps [0, 1];
    # b: BV; u: free
    assert list(inst.lb) == [-INF, 0.0, -1.0, 0.0, 0.0, -INF]
    assert list(inst.ub) == [-2.0, 5.0, INF, 1.0, 1.0, INF]
    # rows (objective dropped): L <= 10, G >= 2, E with range +2.5 -> [4, 6.5], E with range -1.5 -> [-0.5, 1],
    # L 7 with range 3 -> [4, 7]
    assert list(inst.lhs) == [-INF, 2.0, 4.0, -0.5, 4.0]
    assert list(inst.rhs) == [10.0, INF, 6.5, 1.0, 7.0]
    assert list(np.diff(inst.rowptr)) == [2, 2, 1, 2, 3]
    assert list(inst.colidx[:2]) == [0, 1] and list(inst.vals[:2]) == [2.0, 1.0]


def test_reader_rejects_semicontinuous(tmp_path):
    p = tmp_path / "sc.mps"
    p.write_text(SMALL.replace(" FR BND       u", " SC BND       u         4.0"))
    with pytest.raises(ValueError):
        mps.read_mps(str(p))


def _mipdir(oracle_mod):
    d = os.path.join(oracle_mod.REFDIR, "check", "instances", "MIP")
    if not os.path.isdir(d) or not os.path.exists(oracle_mod.SCIP_ORACLE):
        pytest.skip("the reference's MIPLIB instances or the SCIP driver are not available here")
    return d


MIPLIB = ["bell5", "blend2", "dcmulti", "egout", "enigma", "flugpl", "gt2", "lseu", "misc03", "p0548", "rgn"]
# continuous columns outside tolerance (root, nodes) where SCIP's one-at-a-time order stops at another valid
# fixpoint than the rounds do (everything else agrees to the bit or within tolerance)
RECORDED_CONT = {("bell5", "easy"): (0, 24), ("egout", "res"): (0, 24), ("egout", "easy"): (0, 24),
                 ("flugpl", "res"): (1, 13), ("flugpl", "easy"): (1, 13), ("misc03", "easy"): (0, 2)}


@pytest.mark.parametrize("rule", ["res", "easy"])
@pytest.mark.parametrize("name", MIPLIB)
def test_oracle_agrees_with_scip_on_miplib(oracle_mod, name, rule):
    """Root fixpoint and 100 branch-and-bound nodes on top of SCIP's root: cutoff verdicts and integer bounds
    identical to SCIP's everywhere; continuous bounds within tolerance except the recorded columns."""
    path = os.path.join(_mipdir(oracle_mod), name + ".mps")
    if not os.path.exists(path):
        pytest.skip(f"{name}.mps not shipped")
    inst = mps.read_mps(path)
    easy = rule == "easy"
    par = oracle_mod.params(1e6 if easy else 0.0)
    orc = oracle_mod.Oracle(inst)
    scut, slb, sub, _ = oracle_mod.run_scip(inst, easy=easy)
    lb, ub, r = orc.propagate(inst.lb, inst.ub, par)
    root = G.Agreement()
    root.add(inst.isint, None if r.cutoff else (lb, ub), None if scut else (slb, sub))
    assert root.cutoff_mismatch == 0 and root.int_cols_diff == 0
    rec_root, rec_nodes = RECORDED_CONT.get((name, rule), (0, 0))
    assert root.cont_cols_out_of_tol <= rec_root
    if scut:
        return
    nodes = instances.node_batch(inst, slb, sub, 100, seed=1)
    _, _, _, res = oracle_mod.run_scip(inst, nodes, easy=easy)
    out = orc.propagate_nodes(slb, sub, nodes, par, cap=inst.n)
    agg = G.Agreement()
    for k in range(nodes.nnodes):
        mine = None
        if not out["cutoff"][k]:
            L, U = slb.copy(), sub.copy()
            n = out["n"][k]
            L[out["col"][k, :n]] = out["lb"][k, :n]
            U[out["col"][k, :n]] = out["ub"][k, :n]
            mine = (L, U)
        cut, _, cols, lbs, ubs = res[k]
        theirs = None
        if not cut:
            L2, U2 = slb.copy(), sub.copy()
            L2[cols] = lbs
            U2[cols] = ubs
            theirs = (L2, U2)
        agg.add(inst.isint, mine, theirs)
    assert agg.cutoff_mismatch == 0, "cutoff verdicts differ from SCIP"
    assert agg.int_exact == agg.problems, "integer node bounds differ from SCIP"
    assert agg.cont_cols_out_of_tol <= rec_nodes
