"""Ranged-row propagation (rangedRowPropagation, cons_linear.c:5715-6695, with rangedrowartcons off) in the oracle:
the examples SCIP documents for the rule, and SCIP's own root fixpoints on seeded instances (tests/golden/ranged).

SCIP visits rows one at a time; inside tightenBounds it re-sorts a row when one of its columns becomes binary and
then resumes at a position of the old order (cons_linear.c:7100-7138), and the gcd partition of the ranged rule
depends on which columns are fixed when it runs.  The oracle evaluates every frontier row from the bounds at the
start of a round.  With sortvars off and rows that share no column these orders cannot differ, and SCIP's
results are matched exactly; otherwise the agreement recorded below must not regress.
"""
import os

import numpy as np
import pytest

import golden_cases as G
from scip_gb300.instances import INF, Instance
from test_oracle_cpu import single_rows

RANGED = os.path.join(G.GOLDEN, "ranged")

# (case, setting) -> integer columns (of 57,000 / 7,600) that differ from SCIP at the root; cutoff verdicts agree
RECORDED = {
    ("gcd_rows_indep", "nosort_res"): 0, ("gcd_rows_indep", "nosort_easy"): 0,
    ("gcd_rows_indep", "sort_res"): 9, ("gcd_rows_indep", "sort_easy"): 9,
    ("gcd_rows_shared", "nosort_res"): 26, ("gcd_rows_shared", "nosort_easy"): 7,
    ("gcd_rows_shared", "sort_res"): 44, ("gcd_rows_shared", "sort_easy"): 26,
}


def _load(name):
    z = np.load(os.path.join(RANGED, name + ".npz"))
    inst = Instance(z["rowptr"], z["colidx"], z["vals"], z["lhs"], z["rhs"], z["lb"], z["ub"], z["isint"], name=name)
    return inst, z


def _scip(oracle_mod, inst, sortvars):
    if not os.path.exists(oracle_mod.SCIP_ORACLE):
        return None
    cut, lb, ub, _ = oracle_mod.run_scip(inst, ranged=True, sortvars=sortvars)
    return cut, lb, ub


# Examples from the rule's own description (cons_linear.c:5700-5710): 12 x1 + 9 x2 - x3 = 0 with x1, x2 free
# integers and x3 in [1, 2] is infeasible (x3 must be a multiple of 3); with right-hand side 1, x3 = 2.
@pytest.mark.parametrize("sortvars", [True, False])
def test_documented_examples(oracle_mod, sortvars):
    for rhs, cutoff, x3 in ((0.0, True, None), (1.0, False, 2.0)):
        inst = single_rows([([0, 1, 2], [12.0, 9.0, -1.0], rhs, rhs)], [-INF, -INF, 1.0], [INF, INF, 2.0], [1, 1, 1])
        orc = oracle_mod.Oracle(inst)
        lb, ub, r = orc.propagate(inst.lb, inst.ub, oracle_mod.params(0.0, sortvars=sortvars, ranged=True))
        assert bool(r.cutoff) == cutoff
        if not cutoff:
            assert lb[2] == x3 and ub[2] == x3
        # without the rule the activities alone decide nothing
        lb0, ub0, r0 = orc.propagate(inst.lb, inst.ub, oracle_mod.params(0.0, sortvars=sortvars))
        assert not r0.cutoff and lb0[2] == 1.0 and ub0[2] == 2.0
        scip = _scip(oracle_mod, inst, sortvars)
        if scip is not None:
            assert bool(scip[0]) == cutoff
            if not cutoff:
                assert np.array_equal(scip[1], lb) and np.array_equal(scip[2], ub)


def test_residue_class_bounds_the_other_entry(oracle_mod):
    # 6 x1 + 10 x2 + y in [6.75, 7.25], x1, x2 in [-10, 10], y in [0, 9]: 6 x1 + 10 x2 is even, so y is odd,
    # y >= 1 (two or more feasible values, so only the bounds of y move: cons_linear.c:6296-6352)
    inst = single_rows([([0, 1, 2], [6.0, 10.0, 1.0], 6.75, 7.25)], [-10.0, -10.0, 0.0], [10.0, 10.0, 9.0], [1, 1, 1])
    lb, ub, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(0.0, ranged=True))
    assert not r.cutoff and lb[2] == 1.0 and ub[2] == 9.0
    scip = _scip(oracle_mod, inst, True)
    if scip is not None:
        assert not scip[0] and np.array_equal(scip[1], lb) and np.array_equal(scip[2], ub)


def test_forced_changes_ignore_the_minimal_improvement(oracle_mod):
    # 3 x + 3 y + z in [99.75, 100.25] with integers x, y in [0, 30] and z in [0, 100]: z = 100 - 3 (x + y) is
    # 1 mod 3, so z in [1, 100] -- a change of 1 on a range of 100, below the 5 % minimal improvement
    # (set.c:7711), accepted because the rule forces it
    inst = single_rows([([0, 1, 2], [3.0, 3.0, 1.0], 99.75, 100.25)], [0.0, 0.0, 0.0], [30.0, 30.0, 100.0], [1, 1, 1])
    lb, ub, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(0.0, ranged=True))
    assert not r.cutoff and lb[2] == 1.0 and ub[2] == 100.0
    scip = _scip(oracle_mod, inst, True)
    if scip is not None:
        assert not scip[0] and np.array_equal(scip[1], lb) and np.array_equal(scip[2], ub)


@pytest.mark.parametrize("setting", ["nosort_res", "nosort_easy", "sort_res", "sort_easy"])
@pytest.mark.parametrize("case", ["gcd_rows_indep", "gcd_rows_shared"])
def test_oracle_agrees_with_scip_ranged(oracle_mod, case, setting):
    inst, z = _load(case)
    sortvars = setting.startswith("sort")
    par = oracle_mod.params(1e6 if setting.endswith("easy") else 0.0, sortvars=sortvars, ranged=True)
    lb, ub, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, par)
    a = G.Agreement()
    a.add(inst.isint, None if r.cutoff else (lb, ub),
          None if z[f"{setting}_rootcut"] else (z[f"{setting}_rootlb"], z[f"{setting}_rootub"]))
    assert a.cutoff_mismatch == 0
    assert a.int_cols_diff <= RECORDED[(case, setting)]
    # the rule moves bounds that the activity rules alone leave: the fixture exercises it
    lb0, ub0, _ = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub,
                                                    oracle_mod.params(0.0, sortvars=sortvars))
    assert int(((lb != lb0) | (ub != ub0)).sum()) > 100


def load_tiny():
    """the 60 small instances of tests/golden/ranged/tiny_cutoffs.npz and SCIP's verdicts and bounds"""
    z = np.load(os.path.join(RANGED, "tiny_cutoffs.npz"))
    ro, co = z["row_off"], z["col_off"]
    out = []
    for k in range(len(ro) - 1):
        r0, r1, c0, c1 = ro[k], ro[k + 1], co[k], co[k + 1]
        p0, p1 = z["rowptr"][r0], z["rowptr"][r1]
        inst = Instance(z["rowptr"][r0:r1 + 1] - p0, z["colidx"][p0:p1] - c0, z["vals"][p0:p1], z["lhs"][r0:r1],
                        z["rhs"][r0:r1], z["lb"][c0:c1], z["ub"][c0:c1], z["isint"][c0:c1])
        out.append(inst)
    return out, z


def feasible(inst):
    """exact feasibility of a small instance (scipy's MILP solver), to judge verdicts that differ from SCIP's"""
    opt = pytest.importorskip("scipy.optimize")
    from scipy.sparse import csr_matrix
    A = csr_matrix((inst.vals, inst.colidx, inst.rowptr), shape=(inst.m, inst.n))
    lhs = np.where(inst.lhs <= -INF, -np.inf, inst.lhs)
    rhs = np.where(inst.rhs >= INF, np.inf, inst.rhs)
    r = opt.milp(np.zeros(inst.n), constraints=[opt.LinearConstraint(A, lhs, rhs)],
                 integrality=inst.isint.astype(int), bounds=opt.Bounds(inst.lb, inst.ub))
    assert r.status in (0, 2), r.message
    return r.status == 0


# instances that the rounds prove infeasible and SCIP's one-row-at-a-time order does not: in instance 18 one
# row's activities fix x1 = 0 while another row's ranged rule, from the same round-start bounds, fixes x1 = 1;
# SCIP applies the first before the second row runs, after which that row's entries all share the divisor 5 and
# the rule returns without looking at the sides (cons_linear.c:5958) -- yet the row, 5 | 6, is infeasible
EXTRA_CUTOFFS = {18}


@pytest.mark.parametrize("sortvars", [True, False])
def test_ranged_cutoffs_agree_with_scip(oracle_mod, sortvars):
    """Equations shifted off their residue class: the ranged rule declares many of these instances infeasible
    (cons_linear.c:6033-6045 and :6141-6153).  Every verdict equals SCIP's except the recorded instances, which
    an exact MILP check proves infeasible; every integer bound of a feasible instance equals SCIP's."""
    insts, z = load_tiny()
    tag = "sort" if sortvars else "nosort"
    co = z["col_off"]
    ncut = 0
    for k, inst in enumerate(insts):
        lb, ub, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub,
                                                      oracle_mod.params(0.0, sortvars=sortvars, ranged=True))
        ncut += int(bool(r.cutoff))
        if k in EXTRA_CUTOFFS:
            assert r.cutoff and not z[f"{tag}_cut"][k] and not feasible(inst), f"instance {k}"
            continue
        assert bool(r.cutoff) == bool(z[f"{tag}_cut"][k]), f"instance {k}"
        if not r.cutoff:
            sl = slice(co[k], co[k + 1])
            il = inst.isint != 0
            assert np.array_equal(lb[il], z[f"{tag}_lb"][sl][il]) and np.array_equal(ub[il], z[f"{tag}_ub"][sl][il])
    # without the rule fewer instances are found infeasible
    assert ncut >= 15
    without = sum(bool(oracle_mod.Oracle(i).propagate(i.lb, i.ub, oracle_mod.params(0.0, sortvars=sortvars))[2].cutoff)
                  for i in insts)
    assert without < ncut
