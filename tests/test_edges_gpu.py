"""Edge cases of the CUDA path against the oracle, through the C ABI: empty, free and single-entry rows, a problem
without rows, degenerate node batches (no nodes, nodes without changes, changes outside the base domain), and
bounds at the huge and infinite thresholds (numerics/hugeval 1e15, numerics/infinity 1e20)."""
import numpy as np
import pytest

from scip_gb300 import gbp, instances
from scip_gb300.instances import INF, Instance, NodeBatch
from test_parity_gpu import _nodes_equal

pytestmark = pytest.mark.gpu


def _inst(rows, lb, ub, isint):
    rowptr, cols, vals, lhs, rhs = [0], [], [], [], []
    for c, v, lo, hi in rows:
        cols += c
        vals += v
        rowptr.append(len(cols))
        lhs.append(lo)
        rhs.append(hi)
    n = len(lb)
    return Instance(np.array(rowptr, np.int64), np.array(cols, np.int32), np.array(vals, float), np.array(lhs, float),
                    np.array(rhs, float), np.array(lb, float), np.array(ub, float), np.array(isint, np.int8),
                    x0=np.zeros(n))


def _same_root(gpu_prop, oracle_mod, inst, maxeasy=0.0):
    gpu_prop.set_params(gbp.default_params(maxeasy=maxeasy))
    gpu_prop.upload(inst)
    lb, ub, cut, res = gpu_prop.propagate(inst.lb, inst.ub)
    olb, oub, ores = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(maxeasy))
    assert cut == bool(ores.cutoff)
    assert res.rounds == ores.rounds
    if not cut:
        assert np.array_equal(lb, olb) and np.array_equal(ub, oub)
    return lb, ub, cut


@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
def test_empty_free_and_single_entry_rows(gpu_prop, oracle_mod, maxeasy):
    # an empty row whose sides hold 0, a free row, two single-entry rows (SCIP forces their bounds,
    # cons_linear.c:7029): 2 x2 in [1, 3] gives x2 = 1 (integral), -x3 <= -0.5 gives x3 = 1
    inst = _inst([([], [], -1.0, 1.0), ([0, 1], [1.0, 2.0], -INF, INF), ([2], [2.0], 1.0, 3.0),
                  ([3], [-1.0], -INF, -0.5)], [0, 0, 0, 0], [10, 10, 10, 1], [1, 0, 1, 1])
    lb, ub, cut = _same_root(gpu_prop, oracle_mod, inst, maxeasy)
    assert not cut
    assert list(lb) == [0, 0, 1, 1] and list(ub) == [10, 10, 1, 1]


def test_empty_row_outside_its_sides_is_infeasible(gpu_prop, oracle_mod):
    inst = _inst([([], [], 1.0, 2.0)], [0.0], [1.0], [1])
    _, _, cut = _same_root(gpu_prop, oracle_mod, inst)
    assert cut


def test_problem_without_rows(gpu_prop, oracle_mod):
    inst = Instance(np.zeros(1, np.int64), np.zeros(0, np.int32), np.zeros(0), np.zeros(0), np.zeros(0),
                    np.zeros(3), np.full(3, 5.0), np.ones(3, np.int8), x0=np.zeros(3))
    lb, ub, cut = _same_root(gpu_prop, oracle_mod, inst)
    assert not cut and np.array_equal(lb, inst.lb) and np.array_equal(ub, inst.ub)
    # nodes: none changed, one tightened, one looser than the base (no change), one outside the base (cut off)
    nodes = NodeBatch(np.array([0, 0, 1, 2, 3], np.int64), np.array([0, 1, 2], np.int32), np.array([2.0, -3.0, 6.0]),
                      np.array([3.0, 9.0, 7.0]))
    r = gpu_prop.propagate_nodes(inst.lb, inst.ub, nodes)
    o = oracle_mod.Oracle(inst).propagate_nodes(inst.lb, inst.ub, nodes, oracle_mod.params(0.0), cap=inst.n)
    _nodes_equal(r, o, nodes.nnodes)
    assert list(r.cutoff) == [0, 0, 0, 1] and list(r.n[:3]) == [0, 1, 0]


def test_degenerate_node_batches(gpu_prop, oracle_mod):
    inst = instances.root_mip(3)
    par = oracle_mod.params(0.0)
    orc = oracle_mod.Oracle(inst)
    rlb, rub, _ = orc.propagate(inst.lb, inst.ub, par)
    gpu_prop.set_params(gbp.default_params(maxeasy=0.0))
    gpu_prop.upload(inst)
    # no nodes at all
    empty = NodeBatch(np.zeros(1, np.int64), np.zeros(0, np.int32), np.zeros(0), np.zeros(0))
    r = gpu_prop.propagate_nodes(rlb, rub, empty)
    assert len(r.cutoff) == 0 and r.result.cutoff == 0
    # nodes without changes between ordinary ones, and a change outside the base domain
    nodes = instances.node_batch(inst, rlb, rub, 40, seed=5)
    ptr = np.concatenate([[0, 0], nodes.ptr, [nodes.ptr[-1]] * 2])
    j = int(np.flatnonzero(rub < 1e19)[0])
    col = np.concatenate([nodes.col, [j]]).astype(np.int32)
    nlb = np.concatenate([nodes.lb, [rub[j] + 1.0]])
    nub = np.concatenate([nodes.ub, [rub[j] + 2.0]])
    ptr[-1] += 1
    batch = NodeBatch(ptr.astype(np.int64), col, nlb, nub)
    r = gpu_prop.propagate_nodes(rlb, rub, batch)
    o = orc.propagate_nodes(rlb, rub, batch, par, cap=inst.n)
    _nodes_equal(r, o, batch.nnodes)
    assert r.cutoff[0] == 0 and r.n[0] == 0 and r.rounds[0] == 0
    assert r.cutoff[-1] == 1


def _with_repeats(nodes, rlb, rub, rng):
    """The batch with every node's changes named again (a second, looser or tighter change on the same column in
    random order), plus nodes whose repeated changes cross."""
    ptr, col, lb, ub = [0], [], [], []
    for k in range(nodes.nnodes):
        sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
        c, l, u = list(nodes.col[sl]), list(nodes.lb[sl]), list(nodes.ub[sl])
        for j in list(c):
            lo, hi = rlb[j], rub[j]
            c.append(j)
            l.append(lo)   # a looser repeat: no effect
            u.append(hi)
        if k % 7 == 3 and c:
            j = c[0]
            c.append(j)     # a repeat that crosses the first: the node is cut off
            l.append(min(rub[j], l[0] + 1.0) if l[0] < rub[j] else rlb[j])
            u.append(min(rub[j], l[0] + 1.0) if l[0] < rub[j] else rlb[j])
        perm = rng.permutation(len(c))
        col += [c[i] for i in perm]
        lb += [l[i] for i in perm]
        ub += [u[i] for i in perm]
        ptr.append(len(col))
    return NodeBatch(np.array(ptr, np.int64), np.array(col, np.int32), np.array(lb), np.array(ub))


@pytest.mark.parametrize("scip_order", [False, True])
def test_node_changes_naming_a_column_twice(gpu_prop, oracle_mod, scip_order):
    """A node may name a column more than once: the tightest bounds apply, and crossing bounds cut it off -- the
    same as applying the changes one after the other, on the GPU and in the oracle, in both orders."""
    inst = instances.root_mip(3)
    par = oracle_mod.params(0.0)
    orc = oracle_mod.Oracle(inst)
    rlb, rub, _ = orc.propagate(inst.lb, inst.ub, par)
    if scip_order:
        order = instances.scip_row_order(inst, rlb, rub, instances.scip_var_index(inst.isint, inst.lb, inst.ub))
        inst = instances.in_order(inst, order)
        orc = oracle_mod.Oracle(inst)
    batch = _with_repeats(instances.node_batch(inst, rlb, rub, 60, seed=8), rlb, rub, np.random.default_rng(3))
    gpu_prop.set_params(gbp.default_params(maxeasy=0.0, scip_order=scip_order))
    gpu_prop.upload(inst)
    r = gpu_prop.propagate_nodes(rlb, rub, batch)
    o = orc.propagate_nodes(rlb, rub, batch, par, cap=inst.n, seq=scip_order)
    _nodes_equal(r, o, batch.nnodes)
    assert 0 < int(r.cutoff.sum()) < batch.nnodes
    gpu_prop.set_params(gbp.default_params(maxeasy=0.0))


@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
def test_bounds_at_the_huge_and_infinite_thresholds(gpu_prop, oracle_mod, maxeasy):
    """Bounds just below and at hugeval (1e15) and at infinity (1e20): the contributions move between the
    finite sums and the huge/infinite counters, the residual rule skips what SCIP skips."""
    inst = instances.root_mip(5)
    rng = np.random.default_rng(12)
    lb, ub = inst.lb.copy(), inst.ub.copy()
    cont = np.flatnonzero(inst.isint == 0)
    pick = rng.choice(cont, size=min(len(cont), 400), replace=False)
    vals = np.array([9.9e14, 1e15, 3e16, 1e20])
    ub[pick] = vals[rng.integers(0, 4, len(pick))]
    lb[pick[::3]] = -ub[pick[::3]]
    inst = Instance(inst.rowptr, inst.colidx, inst.vals, inst.lhs, inst.rhs, lb, ub, inst.isint, x0=inst.x0)
    _same_root(gpu_prop, oracle_mod, inst, maxeasy)
    gpu_prop.upload(inst)
    act, cnt = gpu_prop.activities(lb, ub)
    oact, ocnt = oracle_mod.Oracle(inst).activities(lb, ub)
    assert np.array_equal(cnt, ocnt) and np.array_equal(act, oact)
    assert (ocnt != 0).any()


def test_change_column_out_of_range_fails_and_the_context_recovers(gpu_prop, oracle_mod):
    """A node change naming no column: the kernel gives that node up and the call returns GBP_ERR_INVALID, through
    the host and the device entry points alike; the next call on the same context is exact again."""
    import torch

    inst = instances.root_mip(3)
    par = oracle_mod.params(0.0)
    orc = oracle_mod.Oracle(inst)
    rlb, rub, _ = orc.propagate(inst.lb, inst.ub, par)
    gpu_prop.set_params(gbp.default_params(maxeasy=0.0))
    gpu_prop.upload(inst)
    nodes = instances.node_batch(inst, rlb, rub, 16, seed=6)
    for bad in (inst.n, -1):
        col = nodes.col.copy()
        col[int(nodes.ptr[3])] = bad
        with pytest.raises(gbp.GbpError) as e:
            gpu_prop.propagate_nodes(rlb, rub, NodeBatch(nodes.ptr, col, nodes.lb, nodes.ub))
        assert e.value.code == gbp.GBP_ERR_INVALID
    d = torch.device("cuda:0")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(d)
    col = nodes.col.copy()
    col[0] = inst.n + 5
    cap = inst.n * 4
    out = {"cutoff": torch.zeros(16, dtype=torch.int8, device=d), "rounds": torch.zeros(16, dtype=torch.int32, device=d),
           "off": torch.zeros(16, dtype=torch.int64, device=d), "n": torch.zeros(16, dtype=torch.int32, device=d),
           "col": torch.zeros(cap, dtype=torch.int32, device=d), "lb": torch.zeros(cap, dtype=torch.float64, device=d),
           "ub": torch.zeros(cap, dtype=torch.float64, device=d)}
    args = (t(rlb), t(rub), 16, t(nodes.ptr), t(col), t(nodes.lb), t(nodes.ub), out, cap)
    torch.cuda.synchronize()  # the inputs and zeroed outputs are ready before the library's stream uses them
    with pytest.raises(gbp.GbpError) as e:
        gpu_prop.propagate_nodes_device(*args)
    assert e.value.code == gbp.GBP_ERR_INVALID
    torch.cuda.synchronize()
    r = gpu_prop.propagate_nodes(rlb, rub, nodes)
    o = orc.propagate_nodes(rlb, rub, nodes, par, cap=inst.n)
    _nodes_equal(r, o, nodes.nnodes)


def test_sparse_calls_across_uploads(gpu_prop, oracle_mod):
    """The resident bounds of the sparse call belong to one problem: an upload drops them (a call before
    gbp_set_bounds fails), and after uploads of a larger, a smaller and again the larger problem (the device
    arrays are reused) the sparse call equals the full-vector call."""
    big = instances.root_mip(6)
    small = _inst([([0, 1], [1.0, 1.0], -INF, 1.0)], [0, 0], [1, 1], [1, 1])
    gpu_prop.set_params(gbp.default_params(maxeasy=0.0))
    for inst in (big, small, big):
        gpu_prop.upload(inst)
        with pytest.raises(gbp.GbpError):
            gpu_prop.propagate_changes(np.array([0], np.int32), inst.lb[:1], inst.ub[:1])
        rlb, rub, cut, _ = gpu_prop.propagate(inst.lb, inst.ub)
        assert not cut
        gpu_prop.set_bounds(rlb, rub)
        j = int(np.flatnonzero((inst.isint == 1) & (rub > rlb))[0])
        cut, mc, ml, mu, _ = gpu_prop.propagate_changes(np.array([j], np.int32), rub[j:j + 1], rub[j:j + 1])
        lb, ub = rlb.copy(), rub.copy()
        lb[j] = rub[j]
        flb, fub, fcut, _ = gpu_prop.propagate(lb, ub, seed=(np.array([j], np.int32), rlb[j:j + 1], rub[j:j + 1]))
        assert cut == fcut
        if not cut:
            lb[mc], ub[mc] = ml, mu
            assert np.array_equal(lb, flb) and np.array_equal(ub, fub)
