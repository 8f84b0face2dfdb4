"""Ranged-row propagation (GBP_FLAG_RANGEDROW) on the CUDA path against the oracle, bit for bit, through the C ABI:
the plain path (device loop and host-driven rounds, with and without explicit global bounds), batched nodes and
batched instances; and against SCIP's own results in tests/golden/ranged."""
import numpy as np
import pytest

from scip_gb300 import gbp, instances
from test_parity_gpu import _nodes_equal
from test_ranged_cpu import EXTRA_CUTOFFS, _load, load_tiny

pytestmark = pytest.mark.gpu


def _gp(maxeasy, sortvars, hostloop=False):
    p = gbp.default_params(maxeasy=maxeasy, sortvars=sortvars, ranged=True)
    if hostloop:
        p.flags |= gbp.GBP_FLAG_HOSTLOOP
    return p


def _inst(seed=40, m=4000, n=12000):
    # rows share columns; 4 % of the rows are 65..200 long (the warp path); half of them are equations
    return instances.gcd_rows(np.random.default_rng(seed), m, n, long_frac=0.04, equations=True)


@pytest.mark.parametrize("hostloop", [False, True])
@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
@pytest.mark.parametrize("sortvars", [True, False])
def test_ranged_root_matches_oracle(gpu_prop, oracle_mod, sortvars, maxeasy, hostloop):
    inst = _inst()
    gpu_prop.set_params(_gp(maxeasy, sortvars, hostloop))
    gpu_prop.upload(inst)
    lb, ub, cut, res = gpu_prop.propagate(inst.lb, inst.ub)
    par = oracle_mod.params(maxeasy, sortvars=sortvars, ranged=True)
    olb, oub, ores = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, par)
    assert cut == bool(ores.cutoff)
    assert res.rounds == ores.rounds and res.candidates == ores.candidates
    assert np.array_equal(lb, olb) and np.array_equal(ub, oub)
    # the rule changes this fixpoint
    plb, pub, _ = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(maxeasy, sortvars=sortvars))
    assert int(((plb != olb) | (pub != oub)).sum()) > 50


@pytest.mark.parametrize("sortvars", [True, False])
def test_ranged_with_global_bounds_matches_oracle(gpu_prop, oracle_mod, sortvars):
    """Explicit global bounds fix the rows' order for the call (computed before the rounds); here they are wider
    than the bounds propagated, so the order and the binary test differ from those of the local bounds."""
    inst = _inst(seed=41)
    rng = np.random.default_rng(3)
    lb, ub = inst.lb.copy(), inst.ub.copy()
    tight = (rng.random(inst.n) < 0.2) & (inst.isint == 1) & (ub >= 2)
    ub[tight] = np.maximum(np.floor(ub[tight] / 2), inst.x0[tight])  # the generator's point stays feasible
    gpu_prop.set_params(_gp(0.0, sortvars))
    gpu_prop.upload(inst)
    gpu_prop.set_global_bounds(inst.lb, inst.ub)
    glb, gub, cut, _ = gpu_prop.propagate(lb, ub)
    gpu_prop.set_global_bounds(None)
    olb, oub, ores = oracle_mod.Oracle(inst).propagate(lb, ub, oracle_mod.params(0.0, sortvars=sortvars, ranged=True),
                                                       glob=(inst.lb, inst.ub))
    assert not cut and not ores.cutoff
    assert np.array_equal(glb, olb) and np.array_equal(gub, oub)


@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
@pytest.mark.parametrize("sortvars", [True, False])
def test_ranged_nodes_match_oracle(gpu_prop, oracle_mod, sortvars, maxeasy):
    inst = _inst(seed=42)
    par = oracle_mod.params(maxeasy, sortvars=sortvars, ranged=True)
    orc = oracle_mod.Oracle(inst)
    rlb, rub, rr = orc.propagate(inst.lb, inst.ub, par)
    assert not rr.cutoff
    nodes = instances.node_batch(inst, rlb, rub, 600, seed=9)
    gpu_prop.set_params(_gp(maxeasy, sortvars))
    gpu_prop.upload(inst)
    r = gpu_prop.propagate_nodes(rlb, rub, nodes, out_cap=inst.n * 4)
    o = orc.propagate_nodes(rlb, rub, nodes, par, cap=inst.n)
    _nodes_equal(r, o, nodes.nnodes)
    assert 0 < int(r.cutoff.sum()) < nodes.nnodes


@pytest.mark.parametrize("sortvars", [True, False])
def test_ranged_instances_match_oracle_and_scip(gpu_prop, oracle_mod, sortvars):
    """The 60 small instances of tests/golden/ranged/tiny_cutoffs in one block-diagonal problem: per-instance
    cutoff verdicts and bounds equal the oracle's, and SCIP's verdicts except the recorded instances."""
    insts, z = load_tiny()
    tag = "sort" if sortvars else "nosort"
    gpu_prop.set_params(_gp(0.0, sortvars))
    row_off, col_off = gpu_prop.upload_instances(insts)
    lb = np.concatenate([i.lb for i in insts])
    ub = np.concatenate([i.ub for i in insts])
    glb, gub, cut, _ = gpu_prop.propagate_instances(lb, ub)
    for k, inst in enumerate(insts):
        olb, oub, ores = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub,
                                                           oracle_mod.params(0.0, sortvars=sortvars, ranged=True))
        assert bool(cut[k]) == bool(ores.cutoff), f"instance {k}"
        if k not in EXTRA_CUTOFFS:
            assert bool(cut[k]) == bool(z[f"{tag}_cut"][k]), f"instance {k}"
        if not cut[k]:
            sl = slice(col_off[k], col_off[k + 1])
            assert np.array_equal(glb[sl], olb) and np.array_equal(gub[sl], oub), f"instance {k}"
    assert int(cut.sum()) >= 15


@pytest.mark.parametrize("maxeasy", [0.0, 1e6])
def test_ranged_fixture_matches_scip(gpu_prop, maxeasy):
    """Rows that share no column, sortvars off: SCIP's own root fixpoint, integer bounds exactly."""
    inst, z = _load("gcd_rows_indep")
    tag = "nosort_" + ("easy" if maxeasy else "res")
    gpu_prop.set_params(_gp(maxeasy, False))
    gpu_prop.upload(inst)
    lb, ub, cut, _ = gpu_prop.propagate(inst.lb, inst.ub)
    assert cut == bool(z[f"{tag}_rootcut"])
    il = inst.isint != 0
    assert np.array_equal(lb[il], z[f"{tag}_rootlb"][il]) and np.array_equal(ub[il], z[f"{tag}_rootub"][il])


@pytest.mark.parametrize("hostloop", [False, True])
def test_ranged_records_match_oracle(gpu_prop, oracle_mod, hostloop):
    """With a change log, the rows whose ranged rule proposed bounds or found themselves infeasible are recorded
    with their round (the reasons conflict analysis asks for); records and changes equal the oracle's."""
    inst = _inst(seed=43)
    gpu_prop.set_params(_gp(0.0, True, hostloop))
    gpu_prop.upload(inst)
    gpu_prop.set_change_log(8 * inst.n)
    lb, ub, cut, _ = gpu_prop.propagate(inst.lb, inst.ub)
    mine = gpu_prop.change_log()
    rec = gpu_prop.ranged_log()
    orc = oracle_mod.Oracle(inst)
    olb, oub, ores, olog = orc.propagate_logged(inst.lb, inst.ub, oracle_mod.params(0.0, ranged=True))
    assert cut == bool(ores.cutoff) and np.array_equal(lb, olb) and np.array_equal(ub, oub)
    for a, b in zip(mine, olog):
        assert np.array_equal(a, b)
    assert len(rec[0]) > 50
    for a, b in zip(rec, orc.last_ranged):
        assert np.array_equal(a, b)
    # infeasibility found by a ranged row is recorded with column -1.  The oracle stops at the first infeasible
    # row of the round; the device evaluates the whole round, so its records hold the oracle's and may hold more
    insts, z = load_tiny()
    k = int(np.flatnonzero(z["sort_cut"])[0])
    gpu_prop.upload(insts[k])
    gpu_prop.set_change_log(1024)
    _, _, cut, _ = gpu_prop.propagate(insts[k].lb, insts[k].ub)
    orc = oracle_mod.Oracle(insts[k])
    orc.propagate_logged(insts[k].lb, insts[k].ub, oracle_mod.params(0.0, ranged=True))
    rec = set(zip(*[a.tolist() for a in gpu_prop.ranged_log()]))
    theirs = set(zip(*[a.tolist() for a in orc.last_ranged]))
    assert cut and any(c == -1 for _, c, _ in theirs)
    assert theirs <= rec
    gpu_prop.set_change_log(0)
