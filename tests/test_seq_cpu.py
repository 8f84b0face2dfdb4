"""The oracle's restatement of SCIP's own propagation order (oracle/linprop_seq.c) against SCIP 11's results
(tests/golden).  This is the exact parity contract, with no recorded allowance:

- root: cutoff verdicts equal and every bound equal bit for bit; each row ends in the order SCIP holds it in, and
  the rows SCIP deleted as redundant are the rows the restatement deleted;
- nodes (each from a newly transformed problem, scip_driver.c --fresh, with rows in SCIP's order): cutoff verdicts
  and every integer bound equal; continuous bounds within 1e-9 relative or feastol absolute.  Nodes start from
  activities computed afresh, where SCIP's carry the rounding of the root's incremental updates, so continuous
  bounds can differ in the last bits.
"""
import numpy as np
import pytest

import golden_cases as G
from scip_gb300.instances import Instance, scip_var_index


def _par(oracle_mod, tag):
    return oracle_mod.params(0.0 if tag == "res" else 1e6)


@pytest.mark.parametrize("tag", ["res", "easy"])
@pytest.mark.parametrize("case", G.CASES + G.MIPLIB_CASES)
def test_root_in_scip_order_equals_scip(oracle_mod, case, tag):
    inst, z = G.load(case)
    vidx = scip_var_index(inst.isint, inst.lb, inst.ub)
    lb, ub, r, order = oracle_mod.Oracle(inst, vidx).propagate_seq(inst.lb, inst.ub, _par(oracle_mod, tag))
    assert bool(r.cutoff) == bool(z[f"{tag}_rootcut"])
    if r.cutoff:
        return
    assert np.array_equal(lb, z[f"{tag}_rootlb"]) and np.array_equal(ub, z[f"{tag}_rootub"]), \
        "root bounds differ from SCIP's"
    deleted = z[f"{tag}_rowdel"].astype(bool)
    live = ~np.repeat(deleted, np.diff(inst.rowptr))
    assert np.array_equal(order[live], z[f"{tag}_order"][live]), "row orders differ from SCIP's"
    mine = oracle_mod.Oracle(inst).root_deleted_rows(lb, ub, _par(oracle_mod, tag))
    assert np.array_equal(mine, deleted), "rows deleted at the root differ from SCIP's"


@pytest.mark.parametrize("tag", ["res", "easy"])
@pytest.mark.parametrize("case", [c for c in G.CASES + G.MIPLIB_CASES if "node_ptr" in G.load(c)[1]])
def test_nodes_in_scip_order_agree_with_scip(oracle_mod, case, tag):
    inst, z = G.load(case)
    nb = G.nodes_of(z)
    order = z[f"{tag}_order"]
    rows_in_scip_order = Instance(inst.rowptr, inst.colidx[order], inst.vals[order], inst.lhs, inst.rhs, inst.lb,
                                  inst.ub, inst.isint)
    rlb, rub = z[f"{tag}_rootlb"], z[f"{tag}_rootub"]
    out = oracle_mod.Oracle(rows_in_scip_order).propagate_nodes(rlb, rub, nb, _par(oracle_mod, tag), cap=inst.n,
                                                                seq=True)
    agree = G.Agreement()
    for k in range(nb.nnodes):
        mine = None
        if not out["cutoff"][k]:
            n = out["n"][k]
            L, U = rlb.copy(), rub.copy()
            L[out["col"][k, :n]] = out["lb"][k, :n]
            U[out["col"][k, :n]] = out["ub"][k, :n]
            mine = (L, U)
        agree.add(inst.isint, mine, G.scip_node(z, tag, k, rlb, rub))
    assert agree.cutoff_mismatch == 0, "cutoff verdicts differ from SCIP's"
    assert agree.int_exact == agree.problems and agree.int_cols_diff == 0, "integer bounds differ from SCIP's"
    assert agree.cont_cols_out_of_tol == 0, "continuous bounds outside tolerance"


def test_node_workload_in_scip_order_agrees_with_scip(oracle_mod):
    """The batched-node benchmark workload itself: the oracle's root equals SCIP's bit for bit (digest), each row
    ends in SCIP's order, and on all 4,096 nodes cutoff verdicts and integer bounds equal SCIP's, continuous bounds
    within tolerance."""
    import os

    inst, ordered, rlb, rub, nodes, z = G.load_node_workload(oracle_mod)
    out = oracle_mod.Oracle(ordered).propagate_nodes(rlb, rub, nodes, _par(oracle_mod, "res"), cap=1024,
                                                     nthreads=os.cpu_count() or 1, seq=True)
    agree = G.Agreement()
    for k in range(nodes.nnodes):
        n = out["n"][k]
        mine = None if out["cutoff"][k] else (out["col"][k, :n], out["lb"][k, :n], out["ub"][k, :n])
        agree.add_sparse(inst.isint, rlb, rub, mine, G.scip_node_sparse(z, "res", k))
    assert agree.problems == 4096 and agree.cutoff_mismatch == 0
    assert agree.int_exact == agree.problems and agree.cont_cols_out_of_tol == 0


def test_scip_variable_index():
    """SCIP groups a problem's variables by type and makes room for an inserted one by moving the first variable of
    each later group to that group's end (prob.c probProvidePos); a [0,1] integer column is a binary variable."""
    isint = np.array([0, 1, 0, 1, 1, 0], dtype=np.int8)
    lb = np.zeros(6)
    ub = np.array([5.0, 1.0, 5.0, 7.0, 1.0, 5.0])
    # original problem, columns added in order:  c0 -> [c0];  b1 -> [b1 c0];  c2 -> [b1 c0 c2];
    #   i3 -> [b1 i3 c2 c0];  b4 -> [b1 b4 c2 c0 i3] (i3 moves to the integers' end: [b1 b4 i3 c0 c2])
    # transformed problem: the original variables in that order get inserted the same way
    idx = scip_var_index(isint, lb, ub)
    assert sorted(idx.tolist()) == list(range(6))
    # the groups are binaries, integers, continuous
    assert set(idx[[1, 4]].tolist()) == {0, 1}
    assert idx[3] == 2
    assert set(idx[[0, 2, 5]].tolist()) == {3, 4, 5}


def test_pinned_node_base_reproduces_scips_root_and_orders():
    """The compact base the bench's SCIP-order arm starts its nodes from (tests/golden/workload/
    node_workload_base.npz) gives SCIP's root bounds and row orders of the batched-node workload exactly."""
    import os

    from scip_gb300 import instances

    inst = instances.node_mip(seed=2)
    lb, ub, order = instances.pinned_node_base(inst, os.path.join(G.GOLDEN, "workload", "node_workload_base.npz"))
    with np.load(os.path.join(G.GOLDEN, "workload", "node_workload_scip.npz")) as f:
        z = dict(f)
    assert G._digest(lb, ub) == str(z["root_sha256"])
    deleted = np.zeros(inst.m, dtype=bool)
    deleted[z["rowdel"]] = True
    live = ~np.repeat(deleted, np.diff(inst.rowptr))
    assert G._digest(order[live]) == str(z["order_sha256"])
    nodes = instances.node_batch(inst, lb, ub, 4096, seed=3)
    assert G._digest(nodes.ptr, nodes.col, nodes.lb, nodes.ub) == str(z["nodes_sha256"])
