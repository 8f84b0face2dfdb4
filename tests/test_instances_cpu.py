"""Workload generators: determinism, shapes, and soundness of the oracle's fixpoints at moderate size
(every generated instance has a feasible point x0, which propagation must never cut off)."""
import numpy as np
import pytest

from scip_gb300 import instances


def test_generators_are_deterministic():
    a, b = instances.root_mip(3), instances.root_mip(3)
    for f in ("rowptr", "colidx", "vals", "lhs", "rhs", "lb", "ub", "isint"):
        assert np.array_equal(getattr(a, f), getattr(b, f))


def test_shapes_of_the_configurations():
    r = instances.root_mip(0)
    lens = np.diff(r.rowptr)
    assert r.m == 2000 and r.n == 5000 and lens.min() >= 5 and lens.max() <= 15
    assert set(np.abs(r.vals)) <= set(range(1, 11))
    z = instances.zipf_mip(seed=1, m=20000, n=40000)
    zl = np.diff(z.rowptr)
    assert zl.min() >= 2 and zl.max() <= 5000 and (zl > 64).any()
    nm = instances.node_mip(seed=2, m=10000, n=20000)
    nl = np.diff(nm.rowptr)
    assert nl.min() >= 5 and nl.max() <= 40
    assert ((nm.lb <= -1e20) | (nm.ub >= 1e20)).mean() == pytest.approx(0.1, abs=0.02)
    for inst in (r, z, nm):  # no repeated column inside a row
        rows = np.repeat(np.arange(inst.m), np.diff(inst.rowptr))
        key = rows.astype(np.int64) * inst.n + inst.colidx
        assert np.unique(key).shape[0] == inst.nnz


def test_node_batches_fix_integer_columns_inside_bounds():
    inst = instances.node_mip(seed=2, m=5000, n=10000)
    nodes = instances.node_batch(inst, inst.lb, inst.ub, 500, seed=1)
    k = np.diff(nodes.ptr)
    assert k.min() >= 1 and k.max() <= 64
    assert (inst.isint[nodes.col] == 1).all()
    assert (nodes.lb == nodes.ub).all() and (nodes.lb >= inst.lb[nodes.col]).all() and (nodes.ub <= inst.ub[nodes.col]).all()


@pytest.mark.parametrize("make", [lambda: instances.root_mip(1), lambda: instances.node_mip(seed=4, m=20000, n=40000),
                                  lambda: instances.zipf_mip(seed=5, m=20000, n=40000, hi=1000)]
                         + [(lambda i=i: instances.uneven_batch(seed=6, count=3, rmin=2000, rmax=5000)[i]) for i in range(3)])
def test_oracle_fixpoint_keeps_the_feasible_point(oracle_mod, make):
    inst = make()
    rows = np.repeat(np.arange(inst.m), np.diff(inst.rowptr))
    act = np.bincount(rows, weights=inst.vals * inst.x0[inst.colidx], minlength=inst.m)
    assert (act <= inst.rhs + 1e-7 * np.maximum(1, np.abs(inst.rhs))).all()
    assert (act >= inst.lhs - 1e-7 * np.maximum(1, np.abs(inst.lhs))).all()
    lb, ub, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(0.0))
    assert not r.cutoff
    tol = 1e-6 * np.maximum(1.0, np.abs(inst.x0))
    assert (inst.x0 >= lb - tol).all() and (inst.x0 <= ub + tol).all()


def test_node_generator_tight_option_cuts_off_about_15_percent(oracle_mod):
    """node_batch(tight=0.15) on the 200,000 x 400,000 workload: about 15 % of the nodes are infeasible (the
    workload's stated rate), against about 0.5 % for the plain generator, whose stream the option leaves alone."""
    import os

    import numpy as np

    from scip_gb300 import instances

    inst = instances.node_mip(seed=2)
    o = oracle_mod.Oracle(inst)
    par = oracle_mod.params(0.0)
    rlb, rub, _ = o.propagate(inst.lb, inst.ub, par)
    plain = instances.node_batch(inst, rlb, rub, 4096, seed=3)
    again = instances.node_batch(inst, rlb, rub, 4096, seed=3, tight=0.0)
    assert np.array_equal(plain.ptr, again.ptr) and np.array_equal(plain.col, again.col)
    assert np.array_equal(plain.lb, again.lb)
    tight = instances.node_batch(inst, rlb, rub, 4096, seed=3, tight=0.15)
    for k in range(tight.nnodes):  # every node names a column once, fixes it inside the root domain
        c = tight.col[tight.ptr[k]:tight.ptr[k + 1]]
        assert np.all(np.diff(c) > 0)
    assert np.all(tight.lb >= rlb[tight.col]) and np.all(tight.ub <= rub[tight.col])
    rate = o.propagate_nodes(rlb, rub, tight, par, cap=1, nthreads=os.cpu_count() or 1)["cutoff"].mean()
    base = o.propagate_nodes(rlb, rub, plain, par, cap=1, nthreads=os.cpu_count() or 1)["cutoff"].mean()
    assert 0.12 <= rate <= 0.18 and base < 0.02
