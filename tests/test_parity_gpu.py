"""CUDA path vs the oracle (C restatement) on the same seeded inputs, through the C ABI.

Bit-exact comparison: both sides evaluate the same rules in the same order of floating-point operations
(libgbp is compiled with --fmad=false; activities are summed in a fixed canonical order), so bounds,
cutoff verdicts, activities and infinity counts must be identical, not merely close.
"""
import numpy as np
import pytest

from scip_gb300 import gbp, instances

pytestmark = pytest.mark.gpu


def _params(maxeasy):
    return gbp.default_params(maxeasy=maxeasy)


def _nodes_equal(r, o, nnodes):
    assert np.array_equal(r.cutoff, o["cutoff"]), "cutoff verdicts differ"
    assert np.array_equal(r.rounds[r.cutoff == 0], o["rounds"][o["cutoff"] == 0]), "round counts differ"
    for k in range(nnodes):
        if r.cutoff[k]:
            continue
        c, l, u = r.node(k)
        n = o["n"][k]
        assert n >= 0
        oc = o["col"][k, :n]
        a, b = np.argsort(c), np.argsort(oc)
        assert np.array_equal(c[a], oc[b]), f"node {k}: changed columns differ"
        assert np.array_equal(l[a], o["lb"][k, :n][b]), f"node {k}: lower bounds differ"
        assert np.array_equal(u[a], o["ub"][k, :n][b]), f"node {k}: upper bounds differ"


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
def test_root_fixpoint_matches_oracle(gpu_prop, oracle_mod, seed, maxeasy):
    inst = instances.root_mip(seed)
    gpu_prop.set_params(_params(maxeasy))
    gpu_prop.upload(inst)
    lb, ub, cut, res = gpu_prop.propagate(inst.lb, inst.ub)
    olb, oub, ores = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(maxeasy))
    assert cut == bool(ores.cutoff)
    assert res.rounds == ores.rounds
    assert res.rows == ores.rows and res.nnz == ores.nnz and res.candidates == ores.candidates
    assert np.array_equal(lb, olb) and np.array_equal(ub, oub)


def test_activities_and_counts_bit_exact(gpu_prop, oracle_mod):
    # Zipf rows (long rows take the warp path) with infinite and huge bounds
    inst = instances.zipf_mip(seed=11, m=3000, n=6000, hi=600)
    lb = inst.lb.copy()
    ub = inst.ub.copy()
    rng = np.random.default_rng(5)
    huge = rng.random(inst.n) < 0.02
    ub[huge] = 3e16
    gpu_prop.upload(inst)
    act, cnt = gpu_prop.activities(lb, ub)
    oact, ocnt = oracle_mod.Oracle(inst).activities(lb, ub)
    assert np.array_equal(cnt, ocnt)
    assert np.array_equal(act, oact)
    assert (np.diff(inst.rowptr) > 64).any()


@pytest.mark.parametrize("hostloop", [False, True])
@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
def test_zipf_root_matches_oracle(gpu_prop, oracle_mod, maxeasy, hostloop):
    """Both drivers of the plain path: the device-side graph loop and host-driven rounds."""
    inst = instances.zipf_mip(seed=3, m=20000, n=40000, hi=2000)
    p = _params(maxeasy)
    p.flags = gbp.GBP_FLAG_HOSTLOOP if hostloop else 0
    gpu_prop.set_params(p)
    gpu_prop.upload(inst)
    lb, ub, cut, res = gpu_prop.propagate(inst.lb, inst.ub)
    olb, oub, ores = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(maxeasy))
    assert cut == bool(ores.cutoff)
    if not cut:
        assert np.array_equal(lb, olb) and np.array_equal(ub, oub)
        assert res.rounds == ores.rounds
    assert res.launches <= (3 * res.rounds + 1 if hostloop else 2)
    gpu_prop.set_params(_params(maxeasy))


@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
@pytest.mark.parametrize("threads", [32, 64, 128, 256])
def test_nodes_match_oracle(gpu_prop, oracle_mod, maxeasy, threads):
    inst = instances.node_mip(seed=2, m=20000, n=40000)
    orc = oracle_mod.Oracle(inst)
    par = oracle_mod.params(maxeasy)
    rlb, rub, _ = orc.propagate(inst.lb, inst.ub, par)
    nodes = instances.node_batch(inst, rlb, rub, 512, seed=9)
    gpu_prop.set_params(_params(maxeasy))
    gpu_prop.set_batch_shape(threads, 0)
    gpu_prop.upload(inst)
    r = gpu_prop.propagate_nodes(rlb, rub, nodes)
    o = orc.propagate_nodes(rlb, rub, nodes, par, cap=inst.n)
    _nodes_equal(r, o, nodes.nnodes)
    t = o["total"]
    if o["cutoff"].sum() == 0:
        # same frontiers, same rows, same candidates (a cut-off node stops at the end of its round on the GPU
        # but at the first infeasible row in the oracle, so counts are compared only without cutoffs)
        assert (r.result.rows, r.result.nnz, r.result.candidates, r.result.changes) == (t.rows, t.nnz, t.candidates, t.changes)
    else:
        assert r.result.rows >= t.rows


def test_nodes_seeded_plain_path_equals_batched(gpu_prop, oracle_mod):
    """Each node alone through the plain path (seeded propagate) equals its result inside the batch."""
    inst = instances.root_mip(4)
    gpu_prop.set_params(_params(0.0))
    gpu_prop.upload(inst)
    rlb, rub, _, _ = gpu_prop.propagate(inst.lb, inst.ub)
    nodes = instances.node_batch(inst, rlb, rub, 40, seed=2)
    r = gpu_prop.propagate_nodes(rlb, rub, nodes)
    gpu_prop.set_global_bounds(rlb, rub)  # the nodes' global domain is the root fixpoint
    for k in range(nodes.nnodes):
        lb, ub = rlb.copy(), rub.copy()
        sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
        cols = nodes.col[sl]
        olb, oub = lb[cols].copy(), ub[cols].copy()
        lb[cols] = np.maximum(lb[cols], nodes.lb[sl])
        ub[cols] = np.minimum(ub[cols], nodes.ub[sl])
        plb, pub, cut, _ = gpu_prop.propagate(lb, ub, seed=(cols, olb, oub))
        assert cut == bool(r.cutoff[k])
        if not cut:
            c, l, u = r.node(k)
            elb, eub = rlb.copy(), rub.copy()
            elb[c] = l
            eub[c] = u
            assert np.array_equal(plb, elb) and np.array_equal(pub, eub)
    gpu_prop.set_global_bounds(None)


@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
def test_uneven_instances_in_one_problem_match_oracle_per_instance(gpu_prop, oracle_mod, maxeasy):
    """Independent instances uploaded as one block-diagonal problem: each instance's result equals the oracle
    run on that instance alone (also covering an instance that becomes infeasible)."""
    insts = instances.uneven_batch(seed=8, count=12, rmin=300, rmax=6000)
    # one infeasible instance: x + y >= 5 with x, y in [0, 2]
    from scip_gb300.instances import Instance
    bad = Instance(np.array([0, 2], np.int64), np.array([0, 1], np.int32), np.array([1.0, 1.0]), np.array([5.0]),
                   np.array([1e20]), np.zeros(2), np.full(2, 2.0), np.ones(2, np.int8), x0=np.zeros(2))
    insts.insert(5, bad)
    gpu_prop.set_params(_params(maxeasy))
    row_off, col_off = gpu_prop.upload_instances(insts)
    lb = np.concatenate([i.lb for i in insts])
    ub = np.concatenate([i.ub for i in insts])
    glb, gub, cut, res = gpu_prop.propagate_instances(lb, ub)
    assert cut[5] == 1
    for k, inst in enumerate(insts):
        olb, oub, ores = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(maxeasy))
        assert bool(cut[k]) == bool(ores.cutoff), f"instance {k}"
        if not cut[k]:
            sl = slice(col_off[k], col_off[k + 1])
            assert np.array_equal(glb[sl], olb) and np.array_equal(gub[sl], oub), f"instance {k}"


def test_instance_list_upload_equals_concatenated_upload(gpu_prop):
    """gbp_upload_instance_list (parts copied to their places, offsets fixed on the device) gives the same results
    as gbp_upload_instances of the host concatenation, with an empty part and a part of one column among them; a
    part whose column index is outside the part is rejected."""
    from scip_gb300.gbp import GbpError
    from scip_gb300.instances import Instance
    insts = instances.uneven_batch(seed=10, count=10, rmin=200, rmax=4000)
    empty = Instance(np.zeros(1, np.int64), np.zeros(0, np.int32), np.zeros(0), np.zeros(0), np.zeros(0),
                     np.zeros(0), np.zeros(0), np.zeros(0, np.int8), x0=np.zeros(0))
    lonely = Instance(np.zeros(1, np.int64), np.zeros(0, np.int32), np.zeros(0), np.zeros(0), np.zeros(0),
                      np.zeros(1), np.ones(1), np.ones(1, np.int8), x0=np.zeros(1))
    insts[3:3] = [empty, lonely]
    lb = np.concatenate([i.lb for i in insts])
    ub = np.concatenate([i.ub for i in insts])
    gpu_prop.set_params(_params(1e6))
    got = []
    for concat in (True, False):
        row_off, col_off = gpu_prop.upload_instances(insts, concat=concat)
        got.append(gpu_prop.propagate_instances(lb, ub)[:3] + (row_off, col_off))
    for a, b in zip(got[0], got[1]):
        assert np.array_equal(a, b)
    broken = Instance(np.array([0, 2], np.int64), np.array([0, 2], np.int32), np.ones(2), np.array([-1e20]),
                      np.array([1.0]), np.zeros(2), np.ones(2), np.ones(2, np.int8), x0=np.zeros(2))
    with pytest.raises(GbpError):
        gpu_prop.upload_instances(insts[:2] + [broken])
    gpu_prop.upload_instances(insts)  # the context stays usable
    assert np.array_equal(gpu_prop.propagate_instances(lb, ub)[0], got[1][0])


def test_uneven_instances_device_variant(gpu_prop, oracle_mod):
    """gbp_propagate_instances_device: bounds and per-instance cutoff flags in device memory."""
    torch = pytest.importorskip("torch")
    insts = instances.uneven_batch(seed=9, count=9, rmin=300, rmax=3000)
    gpu_prop.set_params(_params(0.0))
    row_off, col_off = gpu_prop.upload_instances(insts)
    d = torch.device("cuda", 0)
    lb = torch.from_numpy(np.concatenate([i.lb for i in insts])).to(d)
    ub = torch.from_numpy(np.concatenate([i.ub for i in insts])).to(d)
    cut = torch.full((len(insts),), 7, dtype=torch.int8, device=d)
    gpu_prop.propagate_instances_device(lb, ub, cut)
    hlb, hub, hcut = lb.cpu().numpy(), ub.cpu().numpy(), cut.cpu().numpy()
    for k, inst in enumerate(insts):
        olb, oub, ores = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(0.0))
        assert hcut[k] == int(bool(ores.cutoff))
        sl = slice(col_off[k], col_off[k + 1])
        if not hcut[k]:
            assert np.array_equal(hlb[sl], olb) and np.array_equal(hub[sl], oub)


# ---------------------------------------------------------------------------------------------------------
# binary skip of tightenBounds (cons_linear.c:7110-7138): packing rows with an indicator, where it decides
# many nodes under the residual rule; long_frac adds rows of 65..300 entries (warp path)
def _indicator(long_frac):
    return instances.indicator_packing(np.random.default_rng(7), 6000, 12000, long_frac=long_frac)


@pytest.mark.parametrize("sortvars", [True, False])
@pytest.mark.parametrize("long_frac", [0.0, 0.1])
@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
def test_indicator_nodes_match_oracle(gpu_prop, oracle_mod, maxeasy, long_frac, sortvars):
    inst = _indicator(long_frac)
    orc = oracle_mod.Oracle(inst)
    par = oracle_mod.params(maxeasy, sortvars=sortvars)
    rlb, rub, _ = orc.propagate(inst.lb, inst.ub, par)
    nodes = instances.node_batch(inst, rlb, rub, 1024, seed=4)
    gpu_prop.set_params(gbp.default_params(maxeasy=maxeasy, sortvars=sortvars))
    gpu_prop.upload(inst)
    o = orc.propagate_nodes(rlb, rub, nodes, par, cap=inst.n)
    cap = int(o["n"].sum()) + 1024  # packed output: every changed column of every node
    for threads in (32, 128, 256):
        gpu_prop.set_batch_shape(threads, 0)
        r = gpu_prop.propagate_nodes(rlb, rub, nodes, out_cap=cap)
        _nodes_equal(r, o, nodes.nnodes)
    gpu_prop.set_batch_shape(128, 0)
    gpu_prop.set_params(_params(maxeasy))


@pytest.mark.parametrize("hostloop", [False, True])
@pytest.mark.parametrize("long_frac", [0.0, 0.1])
def test_indicator_plain_path_matches_oracle(gpu_prop, oracle_mod, long_frac, hostloop):
    """Plain path, residual rule: the root and each node alone (seeded, global domain = root bounds)."""
    inst = _indicator(long_frac)
    orc = oracle_mod.Oracle(inst)
    par = oracle_mod.params(0.0)
    p = _params(0.0)
    p.flags = gbp.GBP_FLAG_HOSTLOOP if hostloop else 0
    gpu_prop.set_params(p)
    gpu_prop.upload(inst)
    lb, ub, cut, res = gpu_prop.propagate(inst.lb, inst.ub)
    olb, oub, ores = orc.propagate(inst.lb, inst.ub, par)
    assert cut == bool(ores.cutoff) and np.array_equal(lb, olb) and np.array_equal(ub, oub)
    nodes = instances.node_batch(inst, olb, oub, 60, seed=6)
    gpu_prop.set_global_bounds(olb, oub)
    for k in range(nodes.nnodes):
        sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
        cols = nodes.col[sl]
        nlb, nub = olb.copy(), oub.copy()
        old_l, old_u = nlb[cols].copy(), nub[cols].copy()
        nlb[cols] = np.maximum(old_l, nodes.lb[sl])
        nub[cols] = np.minimum(old_u, nodes.ub[sl])
        glb, gub, gcut, _ = gpu_prop.propagate(nlb, nub, seed=(cols, old_l, old_u))
        elb, eub, er = orc.propagate(nlb, nub, par, seed=(cols, old_l, old_u), glob=(olb, oub))
        assert gcut == bool(er.cutoff)
        if not gcut:
            assert np.array_equal(glb, elb) and np.array_equal(gub, eub), f"node {k}"
    gpu_prop.set_global_bounds(None)
    gpu_prop.set_params(_params(0.0))


def test_binary_test_reads_the_global_domain(gpu_prop, oracle_mod):
    """x0 + x1 + x2 - y <= 1 with x0 = x1 = 1: y rises to 1 unless the unfixed x2 counts as binary (global
    domain inside [0,1]) and, coming first, ends the visit of the binaries."""
    rowptr = np.array([0, 4], dtype=np.int64)
    inst = instances.Instance(rowptr, np.array([0, 1, 2, 3], np.int32), np.array([1.0, 1.0, 1.0, -1.0]),
                              np.array([-instances.INF]), np.array([1.0]), np.array([1.0, 1.0, 0.0, 0.0]),
                              np.ones(4), np.ones(4, dtype=np.int8))
    gpu_prop.set_params(_params(0.0))
    gpu_prop.upload(inst)
    lb, ub, _, _ = gpu_prop.propagate(inst.lb, inst.ub)
    assert lb[3] == 0.0
    gpu_prop.set_global_bounds(np.zeros(4), np.array([1.0, 1.0, 3.0, 1.0]))
    lb, ub, _, _ = gpu_prop.propagate(inst.lb, inst.ub)
    assert lb[3] == 1.0
    gpu_prop.set_global_bounds(None)
    lb, ub, _, _ = gpu_prop.propagate(inst.lb, inst.ub)
    assert lb[3] == 0.0


# ---------------------------------------------------------------------------------------------------------
# change log of the plain path (the order in which the plugin hands tightenings to SCIP for conflict analysis)
@pytest.mark.parametrize("hostloop", [False, True])
@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
def test_change_log_matches_oracle(gpu_prop, oracle_mod, maxeasy, hostloop):
    inst = instances.root_mip(1)
    p = _params(maxeasy)
    p.flags = gbp.GBP_FLAG_HOSTLOOP if hostloop else 0
    gpu_prop.set_params(p)
    gpu_prop.upload(inst)
    gpu_prop.set_change_log(8 * inst.n)
    lb, ub, cut, res = gpu_prop.propagate(inst.lb, inst.ub)
    col, rnd, llb, lub = gpu_prop.change_log()
    orc = oracle_mod.Oracle(inst)
    olb, oub, ores, olog = orc.propagate_logged(inst.lb, inst.ub, oracle_mod.params(maxeasy))
    assert not cut and np.array_equal(lb, olb) and np.array_equal(ub, oub)
    assert len(col) == len(olog[0]) > 0
    for mine, theirs in zip((col, rnd, llb, lub), olog):
        assert np.array_equal(mine, theirs)
    # replaying the log in order reproduces the fixpoint
    rl, ru = inst.lb.copy(), inst.ub.copy()
    for c, a, b in zip(col, llb, lub):  # later rounds overwrite earlier ones
        rl[c], ru[c] = a, b
    assert np.array_equal(rl, lb) and np.array_equal(ru, ub)

    # a seeded node with its global domain
    nodes = instances.node_batch(inst, lb, ub, 8, seed=5)
    gpu_prop.set_global_bounds(lb, ub)
    for k in range(nodes.nnodes):
        sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
        cols = nodes.col[sl]
        nlb, nub = lb.copy(), ub.copy()
        old_l, old_u = nlb[cols].copy(), nub[cols].copy()
        nlb[cols] = np.maximum(old_l, nodes.lb[sl])
        nub[cols] = np.minimum(old_u, nodes.ub[sl])
        _, _, gcut, _ = gpu_prop.propagate(nlb, nub, seed=(cols, old_l, old_u))
        _, _, er, elog = orc.propagate_logged(nlb, nub, oracle_mod.params(maxeasy), seed=(cols, old_l, old_u),
                                              glob=(lb, ub))
        assert gcut == bool(er.cutoff)
        if not gcut:
            for mine, theirs in zip(gpu_prop.change_log(), elog):
                assert np.array_equal(mine, theirs), f"node {k}"
    gpu_prop.set_global_bounds(None)
    gpu_prop.set_change_log(0)
    gpu_prop.set_params(_params(maxeasy))


@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
def test_sparse_plain_calls_walk_nodes_like_a_search(gpu_prop, oracle_mod, maxeasy):
    """gbp_set_bounds once, then one gbp_propagate_changes per node as a search moves between nodes: each call
    sends the previous node's columns back to the root bounds plus the node's own changes, seeded from the root
    bounds, and gets back the columns propagation moved.  Every node's result equals the oracle's batched-node
    result bit for bit; a cutoff leaves the device copy at the bounds after the changes; a too-small output
    reports the count needed."""
    inst = instances.node_mip(seed=2, m=20000, n=40000)
    orc = oracle_mod.Oracle(inst)
    par = oracle_mod.params(maxeasy)
    rlb, rub, _ = orc.propagate(inst.lb, inst.ub, par)
    nodes = instances.node_batch(inst, rlb, rub, 160, seed=12)
    o = orc.propagate_nodes(rlb, rub, nodes, par, cap=inst.n)
    gpu_prop.set_params(_params(maxeasy))
    gpu_prop.upload(inst)
    gpu_prop.set_global_bounds(rlb, rub)  # a node's global domain: the root fixpoint
    gpu_prop.set_bounds(rlb, rub)
    dirty = np.zeros(0, np.int32)  # columns that differ from the root on the device
    ncut = 0
    for k in range(nodes.nnodes):
        sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
        chg = {int(j): (rlb[j], rub[j]) for j in dirty}
        for j, l, u in zip(nodes.col[sl], nodes.lb[sl], nodes.ub[sl]):
            chg[int(j)] = (max(rlb[j], l), min(rub[j], u))
        cols = np.array(sorted(chg), np.int32)
        nlb = np.array([chg[j][0] for j in cols])
        nub = np.array([chg[j][1] for j in cols])
        alb, aub = rlb.copy(), rub.copy()  # the bounds after the changes
        alb[cols], aub[cols] = nlb, nub
        seed = (rlb[cols], rub[cols])  # tightenings relative to the root: the rows the full-vector call marks
        if o["cutoff"][k]:
            cut, mc, _, _, _ = gpu_prop.propagate_changes(cols, nlb, nub, seed=seed)
            assert cut and len(mc) == 0, f"node {k}"
            ncut += 1
            dirty = cols[(nlb != rlb[cols]) | (nub != rub[cols])]
            continue
        n = o["n"][k]
        flb, fub = rlb.copy(), rub.copy()  # the oracle's final bounds of the node
        flb[o["col"][k, :n]], fub[o["col"][k, :n]] = o["lb"][k, :n], o["ub"][k, :n]
        want = np.flatnonzero((flb != alb) | (fub != aub))  # what propagation moved
        if len(want) > 1:  # room for one moved column only: the call reports the count needed and leaves the
            with pytest.raises(gbp.GbpError) as e:  # device copy so that it can be repeated
                gpu_prop.propagate_changes(cols, nlb, nub, cap=1, seed=seed)
            assert e.value.code == gbp.GBP_ERR_OVERFLOW
        cut, mc, ml, mu, res = gpu_prop.propagate_changes(cols, nlb, nub, seed=seed)
        assert not cut and res.rounds == o["rounds"][k], f"node {k}"
        assert np.array_equal(mc, want), f"node {k}"
        assert np.array_equal(ml, flb[want]) and np.array_equal(mu, fub[want]), f"node {k}"
        dirty = np.flatnonzero((flb != rlb) | (fub != rub)).astype(np.int32)
    assert nodes.nnodes > ncut
    gpu_prop.set_global_bounds(None)
