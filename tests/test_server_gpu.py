"""libgbp's serving loop (gbp_server_*, scip_gb300/csrc/gbp_server.cu) on the GPU: node requests submitted from
several client threads at once are merged into batched launches, and every reply equals the oracle's result for
that node bit for bit; admission refuses what the HBM budget cannot hold; bad columns are refused at submission."""
import threading

import numpy as np
import pytest

from scip_gb300 import gbp, instances

pytestmark = pytest.mark.gpu


def _setup(oracle_mod, m=20000, nnodes=400):
    inst = instances.node_mip(seed=2, m=m, n=2 * m)
    orc = oracle_mod.Oracle(inst)
    par = oracle_mod.params(0.0)
    rlb, rub, _ = orc.propagate(inst.lb, inst.ub, par)
    nodes = instances.node_batch(inst, rlb, rub, nnodes, seed=31)
    want = orc.propagate_nodes(rlb, rub, nodes, par, cap=inst.n)
    return inst, rlb, rub, nodes, want


def test_served_replies_equal_the_oracle(oracle_mod):
    inst, rlb, rub, nodes, want = _setup(oracle_mod)
    srv = gbp.Server(inst, rlb, rub, params=gbp.default_params(maxeasy=0.0), workers=2, max_batch=1024)
    try:
        tickets = [None] * nodes.nnodes

        def client(part):
            for k in range(part, nodes.nnodes, 4):
                sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
                tickets[k] = srv.submit(nodes.col[sl], nodes.lb[sl], nodes.ub[sl])

        th = [threading.Thread(target=client, args=(p,)) for p in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for k in range(nodes.nnodes):
            cut, c, l, u, ts, td = srv.poll(tickets[k])
            assert cut == bool(want["cutoff"][k]), f"node {k}"
            assert td >= ts
            if cut:
                continue
            n = want["n"][k]
            o = np.argsort(want["col"][k, :n])
            assert np.array_equal(c, want["col"][k, :n][o]), f"node {k}"
            assert np.array_equal(l, want["lb"][k, :n][o]) and np.array_equal(u, want["ub"][k, :n][o]), f"node {k}"
        st = srv.stats()
        assert st["requests"] >= nodes.nnodes and st["batches"] < st["requests"]  # requests shared launches
        assert st["budget"] > 0
    finally:
        srv.close()


def test_admission_and_bad_requests(oracle_mod):
    inst, rlb, rub, nodes, want = _setup(oracle_mod, m=5000, nnodes=8)
    srv = gbp.Server(inst, rlb, rub, params=gbp.default_params(maxeasy=0.0), workers=1, hbm_cap=1000)
    try:
        sl = slice(nodes.ptr[0], nodes.ptr[1])
        with pytest.raises(gbp.GbpError) as e:  # no request fits a budget of 1,000 bytes
            srv.submit(nodes.col[sl], nodes.lb[sl], nodes.ub[sl])
        assert e.value.code == gbp.GBP_ERR_NOMEM
        assert srv.stats()["budget"] == 1000
    finally:
        srv.close()
    srv = gbp.Server(inst, rlb, rub, params=gbp.default_params(maxeasy=0.0), workers=1)
    try:
        with pytest.raises(gbp.GbpError) as e:
            srv.submit(np.array([inst.n + 3], np.int32), np.zeros(1), np.zeros(1))
        assert e.value.code == gbp.GBP_ERR_INVALID
        t = srv.submit(np.zeros(0, np.int32), np.zeros(0), np.zeros(0))  # a node without changes
        cut, c, _, _, _, _ = srv.poll(t)
        assert not cut and len(c) == 0
        sl = slice(nodes.ptr[1], nodes.ptr[2])
        t = srv.submit(nodes.col[sl], nodes.lb[sl], nodes.ub[sl])
        r = srv.poll(t, wait_ms=60000)
        assert r is not None and r[0] == bool(want["cutoff"][1])
    finally:
        srv.close()


def test_instance_requests_beside_node_requests(oracle_mod):
    """Instance requests (problems of their own) go to instance workers, which upload what is queued as one
    block-diagonal problem and propagate it in one launch; every reply equals the oracle's root fixpoint of that
    instance bit for bit, while node requests are served beside them.  A request whose column index lies outside
    its instance is answered GBP_ERR_INVALID and the rest of its batch is still served."""
    from scip_gb300.instances import Instance
    inst, rlb, rub, nodes, want = _setup(oracle_mod, m=5000, nnodes=64)
    pool = instances.uneven_batch(seed=41, count=24)
    pool = [p for p in pool if p.m <= 20000][:12]
    bad = Instance(np.array([0, 2], np.int64), np.array([0, 5], np.int32), np.array([1.0, 1.0]), np.array([1.0]),
                   np.array([1e20]), np.zeros(2), np.full(2, 2.0), np.ones(2, np.int8), x0=np.zeros(2))
    srv = gbp.Server(inst, rlb, rub, params=gbp.default_params(maxeasy=0.0), workers=1, inst_workers=2)
    try:
        tk_i = [srv.submit_instance(p) for p in pool[:6]]
        tk_bad = srv.submit_instance(bad)
        tk_i += [srv.submit_instance(p) for p in pool[6:]]
        tk_n = []
        for k in range(nodes.nnodes):
            sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
            tk_n.append(srv.submit(nodes.col[sl], nodes.lb[sl], nodes.ub[sl]))
        for p, t in zip(pool, tk_i):
            cut, c, l, u, _, _ = srv.poll(t)
            olb, oub, ores = oracle_mod.Oracle(p).propagate(p.lb, p.ub, oracle_mod.params(0.0))
            assert cut == bool(ores.cutoff)
            if not cut:
                assert np.array_equal(c, np.arange(p.n)) and np.array_equal(l, olb) and np.array_equal(u, oub)
        for k, t in enumerate(tk_n):
            cut, c, _, _, _, _ = srv.poll(t)
            assert cut == bool(want["cutoff"][k])
        with pytest.raises(gbp.GbpError) as e:
            srv.poll(tk_bad)
        assert e.value.code == gbp.GBP_ERR_INVALID
    finally:
        srv.close()

