"""Batched branch-and-bound nodes in SCIP's own order on the GPU (GBP_FLAG_SCIPORDER, scip_gb300/csrc/gbp_seq.cu):

* against the oracle's restatement of that order (oracle/linprop_seq.c) bit for bit -- cutoff verdicts, rounds, and
  every changed column's bounds -- on every golden instance, both rules, with and without sortvars;
* against SCIP 11's own node results (tests/golden, the seeded cases and the MIPLIB instances the reference ships,
  each node from a fresh transform, rows in the order SCIP held them): cutoff verdicts and integer bounds exact,
  continuous bounds within 1e-9 relative or feastol absolute;
* edge cases: empty nodes and batches, a change outside the column range (GBP_ERR_INVALID, after which the context
  is still exact), a change that conflicts with the base domain, and the round limit.
"""
import numpy as np
import pytest

import golden_cases as G
from scip_gb300 import gbp, instances

pytestmark = pytest.mark.gpu


def _params(maxeasy, sortvars=True, maxrounds=0):
    return gbp.default_params(maxeasy=maxeasy, sortvars=sortvars, scip_order=True, maxrounds=maxrounds)


def _assert_equal_nodes(r, o, nnodes, what):
    assert np.array_equal(r.cutoff[:nnodes], o["cutoff"]), f"{what}: cutoff verdicts differ"
    assert np.array_equal(r.rounds[:nnodes], o["rounds"]), f"{what}: round counts differ"
    for k in range(nnodes):
        if r.cutoff[k]:
            continue
        c, l, u = r.node(k)
        n = o["n"][k]
        assert n >= 0
        a, b = np.argsort(c), np.argsort(o["col"][k, :n])
        assert np.array_equal(c[a], o["col"][k, :n][b]), f"{what}: node {k} changed columns differ"
        assert np.array_equal(l[a], o["lb"][k, :n][b]) and np.array_equal(u[a], o["ub"][k, :n][b]), \
            f"{what}: node {k} bounds differ"


def _scip_ordered(z, inst, tag):
    return instances.in_order(inst, z[f"{tag}_order"])


@pytest.mark.parametrize("tag", ["res", "easy"])
@pytest.mark.parametrize("case", [c for c in G.CASES + G.MIPLIB_CASES if "node_ptr" in G.load(c)[1]])
def test_nodes_in_scip_order_equal_oracle_and_scip(gpu_prop, oracle_mod, case, tag):
    inst, z = G.load(case)
    nb = G.nodes_of(z)
    maxeasy = 0.0 if tag == "res" else 1e6
    ordered = _scip_ordered(z, inst, tag)
    rlb, rub = z[f"{tag}_rootlb"], z[f"{tag}_rootub"]
    gpu_prop.set_params(_params(maxeasy))
    gpu_prop.upload(ordered)
    r = gpu_prop.propagate_nodes(rlb, rub, nb, out_cap=nb.nnodes * inst.n)
    o = oracle_mod.Oracle(ordered).propagate_nodes(rlb, rub, nb, oracle_mod.params(maxeasy), cap=inst.n, seq=True)
    _assert_equal_nodes(r, o, nb.nnodes, case)
    assert r.result.changes == o["total"].changes and r.result.rows == o["total"].rows
    # SCIP's own results: the exact contract
    agree = G.Agreement()
    for k in range(nb.nnodes):
        mine = None
        if not r.cutoff[k]:
            c, l, u = r.node(k)
            L, U = rlb.copy(), rub.copy()
            L[c], U[c] = l, u
            mine = (L, U)
        agree.add(inst.isint, mine, G.scip_node(z, tag, k, rlb, rub))
    assert agree.cutoff_mismatch == 0 and agree.int_cols_diff == 0 and agree.cont_cols_out_of_tol == 0


@pytest.mark.parametrize("sortvars", [True, False])
@pytest.mark.parametrize("case", ["zipf_small", "indicator_packing", "network"])
def test_nodes_in_scip_order_from_a_fresh_sort(gpu_prop, oracle_mod, case, sortvars):
    """Rows sorted on the base domain by the host helper (the order a synthetic workload uses), new node draws, both
    settings of sortvars: the GPU equals the oracle bit for bit."""
    inst, z = G.load(case)
    rlb, rub = z["res_rootlb"], z["res_rootub"]
    order = instances.scip_row_order(inst, rlb, rub, instances.scip_var_index(inst.isint, inst.lb, inst.ub))
    ordered = instances.in_order(inst, order)
    nb = instances.node_batch(inst, rlb, rub, 300, seed=91)
    gpu_prop.set_params(_params(0.0, sortvars=sortvars))
    gpu_prop.upload(ordered)
    r = gpu_prop.propagate_nodes(rlb, rub, nb, out_cap=nb.nnodes * inst.n)
    o = oracle_mod.Oracle(ordered).propagate_nodes(rlb, rub, nb, oracle_mod.params(0.0, sortvars=sortvars),
                                                   cap=inst.n, seq=True)
    _assert_equal_nodes(r, o, nb.nnodes, case)


def test_node_workload_in_scip_order(gpu_prop, oracle_mod):
    """The batched-node benchmark workload (200,000 x 400,000, all 4,096 nodes) in SCIP's order: equal to the oracle
    bit for bit, and to SCIP's own results within the exact contract."""
    import os

    inst, ordered, rlb, rub, nodes, z = G.load_node_workload(oracle_mod)
    gpu_prop.set_params(_params(0.0))
    gpu_prop.upload(ordered)
    r = gpu_prop.propagate_nodes(rlb, rub, nodes, out_cap=4096 * 256)
    o = oracle_mod.Oracle(ordered).propagate_nodes(rlb, rub, nodes, oracle_mod.params(0.0), cap=1024,
                                                   nthreads=os.cpu_count() or 1, seq=True)
    _assert_equal_nodes(r, o, nodes.nnodes, "node workload")
    agree = G.Agreement()
    for k in range(nodes.nnodes):
        agree.add_sparse(inst.isint, rlb, rub, None if r.cutoff[k] else r.node(k), G.scip_node_sparse(z, "res", k))
    assert agree.cutoff_mismatch == 0 and agree.int_exact == agree.problems and agree.cont_cols_out_of_tol == 0


def test_scip_order_edge_cases(gpu_prop, oracle_mod):
    inst, z = G.load("root_mip_s0")
    ordered = _scip_ordered(z, inst, "res")
    rlb, rub = z["res_rootlb"], z["res_rootub"]
    gpu_prop.set_params(_params(0.0))
    gpu_prop.upload(ordered)
    orc = oracle_mod.Oracle(ordered)
    par = oracle_mod.params(0.0)
    # an empty batch, and nodes without changes
    empty = instances.NodeBatch(np.zeros(1, np.int64), np.zeros(0, np.int32), np.zeros(0), np.zeros(0))
    r = gpu_prop.propagate_nodes(rlb, rub, empty)
    assert r.result.rows == 0
    none = instances.NodeBatch(np.zeros(4, np.int64), np.zeros(0, np.int32), np.zeros(0), np.zeros(0))
    r = gpu_prop.propagate_nodes(rlb, rub, none)
    assert not r.cutoff[:3].any() and (r.n[:3] == 0).all()
    # a change that conflicts with the base domain cuts the node off; a change outside the columns fails the call
    j = int(np.nonzero(inst.isint)[0][0])
    bad = instances.NodeBatch(np.array([0, 1, 2], np.int64), np.array([j, inst.n + 5], np.int32),
                              np.array([rub[j] + 1.0, 0.0]), np.array([rub[j] + 1.0, 0.0]))
    with pytest.raises(gbp.GbpError) as e:
        gpu_prop.propagate_nodes(rlb, rub, bad)
    assert e.value.code == gbp.GBP_ERR_INVALID
    # the context is still exact afterwards
    nb = instances.node_batch(inst, rlb, rub, 64, seed=5)
    r = gpu_prop.propagate_nodes(rlb, rub, nb, out_cap=64 * inst.n)
    _assert_equal_nodes(r, orc.propagate_nodes(rlb, rub, nb, par, cap=inst.n, seq=True), 64, "after a failed call")
    # the round limit: valid bounds, GBP_ERR_LIMIT tolerated by the binding, same as the oracle with the same cap
    gpu_prop.set_params(_params(0.0, maxrounds=1))
    r = gpu_prop.propagate_nodes(rlb, rub, nb, out_cap=64 * inst.n)
    _assert_equal_nodes(r, orc.propagate_nodes(rlb, rub, nb, oracle_mod.params(0.0, maxrounds=1), cap=inst.n,
                                               seq=True), 64, "round limit")
    gpu_prop.set_params(_params(0.0))


def _mixed_block(tag):
    """The mixed-magnitude fixture's instances with nodes and a feasible root under `tag`, rows in SCIP's order,
    as one block-diagonal problem: (kept instances, problem, col_off, base lb, base ub, nodes with global columns,
    owner (instance, node) of each node)."""
    mixed = G.load_mixed_small()
    keep = [c for c in mixed if c["nodes"] is not None and not c[tag]["root"]["cut"]]
    big, _, col_off = instances.concat_instances([instances.in_order(c["inst"], c[tag]["root"]["order"])
                                                  for c in keep])
    rlb = np.concatenate([c[tag]["root"]["lb"] for c in keep])
    rub = np.concatenate([c[tag]["root"]["ub"] for c in keep])
    ptr, col, lb, ub, owner = [0], [], [], [], []
    for k, c in enumerate(keep):
        nb = c["nodes"]
        for q in range(nb.nnodes):
            sl = slice(int(nb.ptr[q]), int(nb.ptr[q + 1]))
            col.append(nb.col[sl] + col_off[k])
            lb.append(nb.lb[sl])
            ub.append(nb.ub[sl])
            ptr.append(ptr[-1] + sl.stop - sl.start)
            owner.append((k, q))
    nodes = instances.NodeBatch(np.array(ptr, np.int64), np.concatenate(col).astype(np.int32), np.concatenate(lb),
                                np.concatenate(ub))
    return keep, big, col_off, rlb, rub, nodes, owner


@pytest.mark.parametrize("tag", ["res", "easy"])
def test_mixed_magnitude_instances_equal_oracle_and_meet_scip(gpu_prop, oracle_mod, tag):
    """300 small instances with coefficient magnitudes 1e-5..1e7 in one row, infinite bounds and equations
    (golden/fuzz/mixed_small.npz), their 1,616 nodes in one batch over the block-diagonal problem: the GPU equals
    the oracle bit for bit in SCIP's order and in rounds; against SCIP's own nodes, cutoff verdicts and integer
    bounds are exact, and continuous bounds are within tolerance on every node but the one where a row's
    coefficients span 8.3e-4..7.2e6 (seed 5056, node 4), which nodes starting from the root's activities get
    bit for bit (tests/test_seq_carry_cpu.py)."""
    keep, big, col_off, rlb, rub, nodes, owner = _mixed_block(tag)
    maxeasy = 0.0 if tag == "res" else 1e6
    cap = int(sum(keep[k]["inst"].n for k, _ in owner))
    gpu_prop.upload(big)
    for seq in (False, True):  # the SCIP-order results (the last) are then compared with SCIP's
        gpu_prop.set_params(gbp.default_params(maxeasy=maxeasy, scip_order=seq))
        r = gpu_prop.propagate_nodes(rlb, rub, nodes, out_cap=cap)
        o = oracle_mod.Oracle(big).propagate_nodes(rlb, rub, nodes, oracle_mod.params(maxeasy), cap=big.n, seq=seq)
        _assert_equal_nodes(r, o, nodes.nnodes, f"mixed_small {tag} {'SCIP order' if seq else 'rounds'}")
    outside = set()
    for q, (k, kq) in enumerate(owner):
        c = keep[k]
        c0, c1 = int(col_off[k]), int(col_off[k + 1])
        mine = None
        if not r.cutoff[q]:
            cc, l, u = r.node(q)
            L, U = rlb[c0:c1].copy(), rub[c0:c1].copy()
            L[cc - c0], U[cc - c0] = l, u
            mine = (L, U)
        cut, cols, lb, ub = c[tag]["nodes"][kq]
        theirs = None
        if not cut:
            L, U = rlb[c0:c1].copy(), rub[c0:c1].copy()
            L[cols], U[cols] = lb, ub
            theirs = (L, U)
        ag = G.Agreement()
        ag.add(c["inst"].isint, mine, theirs)
        assert ag.cutoff_mismatch == 0 and ag.int_cols_diff == 0, f"seed {c['seed']} node {kq}"
        if ag.cont_cols_out_of_tol:
            outside.add((c["seed"], kq))
    assert outside == {(5056, 4)}
