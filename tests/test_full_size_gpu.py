"""The CUDA path at the benchmark sizes, checked through size-independent properties and, where the oracle
finishes in seconds, against the oracle itself:

* the feasible point the generator built every instance around stays inside the propagated bounds (soundness);
* propagating a fixpoint again changes nothing (idempotence);
* the 200,000 x 400,000 root and all 4,096 nodes of the batched workload equal the oracle bit for bit;
* the 1,000,000 x 2,000,000 Zipf instance (~88M nonzeros, rows up to 5,000 entries) equals the oracle.
"""
import os

import numpy as np
import pytest

from scip_gb300 import gbp, instances

pytestmark = pytest.mark.gpu


def _inside(x0, lb, ub):
    tol = 1e-6 * np.maximum(1.0, np.abs(x0))
    return bool(((x0 >= lb - tol) & (x0 <= ub + tol)).all())


@pytest.fixture(scope="module")
def node_workload(gpu_prop, oracle_mod):
    inst = instances.node_mip(seed=2)
    gpu_prop.set_params(gbp.default_params(maxeasy=0.0))
    gpu_prop.upload(inst)
    lb, ub, cut, res = gpu_prop.propagate(inst.lb, inst.ub)
    return inst, lb, ub, cut


def test_root_of_the_node_matrix(gpu_prop, oracle_mod, node_workload):
    inst, lb, ub, cut = node_workload
    assert not cut and _inside(inst.x0, lb, ub)
    olb, oub, ores = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(0.0))
    assert np.array_equal(lb, olb) and np.array_equal(ub, oub)
    # idempotence: the fixpoint propagated again from all rows
    lb2, ub2, cut2, res2 = gpu_prop.propagate(lb, ub)
    assert not cut2 and res2.changes == 0 and np.array_equal(lb2, lb) and np.array_equal(ub2, ub)


def test_all_4096_nodes_equal_the_oracle(gpu_prop, oracle_mod, node_workload):
    inst, lb, ub, _ = node_workload
    nodes = instances.node_batch(inst, lb, ub, 4096, seed=3)
    gpu_prop.set_batch_shape(128, 0)
    r = gpu_prop.propagate_nodes(lb, ub, nodes, out_cap=4096 * 256)
    o = oracle_mod.Oracle(inst).propagate_nodes(lb, ub, nodes, oracle_mod.params(0.0), cap=1024,
                                                 nthreads=os.cpu_count() or 1)
    assert np.array_equal(r.cutoff, o["cutoff"])
    for k in range(nodes.nnodes):
        if r.cutoff[k]:
            continue
        c, l, u = r.node(k)
        n = o["n"][k]
        assert n >= 0
        a, b = np.argsort(c), np.argsort(o["col"][k, :n])
        assert np.array_equal(c[a], o["col"][k, :n][b]), f"node {k}"
        assert np.array_equal(l[a], o["lb"][k, :n][b]) and np.array_equal(u[a], o["ub"][k, :n][b]), f"node {k}"


def test_large_zipf_instance(gpu_prop, oracle_mod):
    inst = instances.zipf_mip(seed=1)
    assert np.diff(inst.rowptr).max() > 1000
    gpu_prop.set_params(gbp.default_params(maxeasy=0.0))
    gpu_prop.upload(inst)
    lb, ub, cut, res = gpu_prop.propagate(inst.lb, inst.ub)
    assert not cut and _inside(inst.x0, lb, ub)
    olb, oub, ores = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(0.0))
    assert res.rounds == ores.rounds
    assert np.array_equal(lb, olb) and np.array_equal(ub, oub)


def test_uneven_instances_at_benchmark_sizes(gpu_prop, oracle_mod):
    insts = instances.uneven_batch(seed=4, count=512)[::8]  # 64 of the benchmark's instances, all sizes
    gpu_prop.set_params(gbp.default_params(maxeasy=0.0))
    row_off, col_off = gpu_prop.upload_instances(insts)
    lb = np.concatenate([i.lb for i in insts])
    ub = np.concatenate([i.ub for i in insts])
    glb, gub, cut, res = gpu_prop.propagate_instances(lb, ub)
    from concurrent.futures import ThreadPoolExecutor

    par = oracle_mod.params(0.0)
    with ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        outs = list(ex.map(lambda i: oracle_mod.Oracle(i).propagate(i.lb, i.ub, par), insts))
    for k, (inst, (olb, oub, ores)) in enumerate(zip(insts, outs)):
        assert bool(cut[k]) == bool(ores.cutoff), f"instance {k}"
        if not cut[k]:
            sl = slice(col_off[k], col_off[k + 1])
            assert np.array_equal(glb[sl], olb) and np.array_equal(gub[sl], oub), f"instance {k}"
            assert _inside(inst.x0, glb[sl], gub[sl])
