"""The round-based oracle (oracle/linprop_oracle.c, the checker of the CUDA round kernels) against SCIP 11's own
results (tests/golden).

SCIP applies tightenings one at a time in its constraint order; the round mode applies them in rounds.  Under
SCIP's minimal-improvement test (set.c:7711-7753) both stop at valid fixpoints of the same rule that can differ for
continuous columns, so the contract checked here is: cutoff verdicts identical, integer bounds identical on every
node, SCIP's own fixpoint is a fixpoint of the oracle's rules, and the continuous agreement recorded below does not
regress.  SCIP's own order (oracle/linprop_seq.c, the checker of the CUDA sequential node kernel) meets the exact
contract with no recorded allowance: tests/test_seq_cpu.py.
"""
import numpy as np
import pytest

import golden_cases as G

# (case, rule) -> (integer columns that differ at the root, continuous root columns outside tolerance,
#                  continuous node columns outside tolerance)
RECORDED = {
    ("knapsack", "res"): (0, 0, 0), ("knapsack", "easy"): (0, 0, 0),
    ("network", "res"): (0, 8, 2), ("network", "easy"): (0, 7, 3),
    ("node_mip_small", "res"): (2, 639, 150), ("node_mip_small", "easy"): (2, 639, 150),
    ("root_mip_s0", "res"): (0, 31, 4), ("root_mip_s0", "easy"): (0, 31, 3),
    ("root_mip_s1", "res"): (0, 22, 0), ("root_mip_s1", "easy"): (0, 22, 0),
    ("root_mip_s2", "res"): (0, 17, 0), ("root_mip_s2", "easy"): (0, 17, 0),
    ("set_cover", "res"): (0, 0, 0), ("set_cover", "easy"): (0, 0, 0),
    ("zipf_small", "res"): (0, 427, 30), ("zipf_small", "easy"): (0, 427, 30),
    ("indicator_packing", "res"): (0, 0, 0), ("indicator_packing", "easy"): (0, 0, 0),
}


def run_oracle(oracle_mod, inst, z, tag, sortvars=True):
    par = oracle_mod.params(0.0 if tag == "res" else 1e6, sortvars=sortvars)
    orc = oracle_mod.Oracle(inst)
    root = G.Agreement()
    lb, ub, r = orc.propagate(inst.lb, inst.ub, par)
    root.add(inst.isint, None if r.cutoff else (lb, ub),
             None if z[f"{tag}_rootcut"] else (z[f"{tag}_rootlb"], z[f"{tag}_rootub"]))
    nodes = G.Agreement()
    nb = G.nodes_of(z)
    if nb is not None:
        rlb, rub = z[f"{tag}_rootlb"], z[f"{tag}_rootub"]
        out = orc.propagate_nodes(rlb, rub, nb, par, cap=inst.n)
        for k in range(nb.nnodes):
            mine = None
            if not out["cutoff"][k]:
                L, U = rlb.copy(), rub.copy()
                n = out["n"][k]
                L[out["col"][k, :n]] = out["lb"][k, :n]
                U[out["col"][k, :n]] = out["ub"][k, :n]
                mine = (L, U)
            nodes.add(inst.isint, mine, G.scip_node(z, tag, k, rlb, rub))
    return root, nodes


@pytest.mark.parametrize("tag", ["res", "easy"])
@pytest.mark.parametrize("case", G.CASES)
def test_oracle_agrees_with_scip(oracle_mod, case, tag):
    inst, z = G.load(case)
    root, nodes = run_oracle(oracle_mod, inst, z, tag)
    assert root.cutoff_mismatch == 0 and nodes.cutoff_mismatch == 0, "cutoff verdicts differ from SCIP"
    assert nodes.int_exact == nodes.problems, "integer node bounds differ from SCIP"
    rec_int, rec_root_cont, rec_node_cont = RECORDED[(case, tag)]
    assert root.int_cols_diff <= rec_int
    assert root.cont_cols_out_of_tol <= rec_root_cont
    assert nodes.cont_cols_out_of_tol <= rec_node_cont


@pytest.mark.parametrize("tag", ["res", "easy"])
@pytest.mark.parametrize("case", G.CASES)
def test_scip_fixpoint_is_oracle_fixpoint(oracle_mod, case, tag):
    inst, z = G.load(case)
    if z[f"{tag}_rootcut"]:
        pytest.skip("root infeasible")
    slb, sub = z[f"{tag}_rootlb"], z[f"{tag}_rootub"]
    lb, ub, r = oracle_mod.Oracle(inst).propagate(slb, sub, oracle_mod.params(0.0 if tag == "res" else 1e6))
    assert not r.cutoff
    il = inst.isint == 1
    assert not ((lb != slb) | (ub != sub))[il].any(), "SCIP's root fixpoint admits an integer tightening"
    assert int(((lb != slb) | (ub != sub))[~il].sum()) <= 2


def test_indicator_packing_pins_the_binary_skip(oracle_mod):
    """On the indicator-packing fixture SCIP's result depends on tightenBounds ending the visit of a row's
    binaries at the first one it cannot tighten (cons_linear.c:7110-7138): trying every entry instead
    (constraints/linear/sortvars = FALSE) contradicts SCIP's own node results, with it they agree exactly."""
    inst, z = G.load("indicator_packing")
    _, with_skip = run_oracle(oracle_mod, inst, z, "res")
    _, without = run_oracle(oracle_mod, inst, z, "res", sortvars=False)
    assert with_skip.cutoff_mismatch == 0 and with_skip.int_exact == with_skip.problems
    assert without.cutoff_mismatch > 0 and without.int_exact < without.problems
