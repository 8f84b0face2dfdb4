"""Known-answer tests of the oracle's arithmetic and rules on hand-checkable rows."""
import numpy as np
import pytest

from scip_gb300.instances import INF, Instance, NodeBatch


def single_rows(rows, lb, ub, isint):
    """rows: list of (cols, vals, lhs, rhs)."""
    rowptr = np.zeros(len(rows) + 1, dtype=np.int64)
    cols, vals, lhs, rhs = [], [], [], []
    for i, (c, v, l, r) in enumerate(rows):
        rowptr[i + 1] = rowptr[i] + len(c)
        cols += list(c)
        vals += list(v)
        lhs.append(l)
        rhs.append(r)
    return Instance(rowptr, np.array(cols, np.int32), np.array(vals, float), np.array(lhs, float),
                    np.array(rhs, float), np.array(lb, float), np.array(ub, float), np.array(isint, np.int8))


def test_compensated_activity(oracle_mod):
    # 2^49 + 1/16 - 2^49: a plain double sum loses the 1/16 (half an ulp of 2^49), the compensated (TwoSum)
    # sum keeps it; 2^49 stays below the huge-value threshold 1e15
    big = 2.0 ** 49
    inst = single_rows([([0, 1, 2], [1.0, 1.0, -1.0], -INF, INF)], [big, 0.0625, big], [big, 0.0625, big], [0, 0, 0])
    act, cnt = oracle_mod.Oracle(inst).activities(inst.lb, inst.ub)
    assert act[0, 0] + act[0, 1] == 0.0625
    assert ((big + 0.0625) - big) == 0.0
    assert not cnt.any()


def test_double_double_sum_known_answer(oracle_mod):
    """The known answer of SCIP's own double-double test (tests/src/misc/dbldblarith.c, test "sum"): c + b + a + a
    with a = 0.000000034567, b = 2.34567, c = 12345678.9 is 1.2345681245670069507e7 when summed compensated, which a
    plain double sum misses.  A row of four unit coefficients with columns fixed at c, b, a, a sums the same terms."""
    a, b, c = 0.000000034567, 2.34567, 12345678.9
    want = 1.2345681245670069507e7
    inst = single_rows([([0, 1, 2, 3], [1.0, 1.0, 1.0, 1.0], -INF, INF)], [c, b, a, a], [c, b, a, a], [0, 0, 0, 0])
    act, cnt = oracle_mod.Oracle(inst).activities(inst.lb, inst.ub)
    assert act[0, 0] + act[0, 1] == want and act[0, 2] + act[0, 3] == want
    assert ((c + b) + a) + a != want
    assert not cnt.any()


def test_infinity_and_huge_counters(oracle_mod):
    # x0 in (-inf, 1], x1 in [0, inf), x2 in [2e15, 3e15] (huge contributions), x3 in [1, 2]
    inst = single_rows([([0, 1, 2, 3], [2.0, -3.0, 1.0, 1.0], -INF, INF)],
                       [-INF, 0.0, 2e15, 1.0], [1.0, INF, 3e15, 2.0], [0, 0, 0, 0])
    act, cnt = oracle_mod.Oracle(inst).activities(inst.lb, inst.ub)
    # min activity: 2*(-inf) -> neg inf; -3*(+inf) -> neg inf; 1*2e15 -> pos huge; 1*1 finite
    # max activity: 2*1 finite; -3*0 = 0; 1*3e15 -> pos huge; 1*2 finite
    assert list(cnt[0]) == [0, 2, 1, 0, 0, 0, 1, 0]
    assert act[0, 0] + act[0, 1] == 1.0 and act[0, 2] + act[0, 3] == 4.0


@pytest.mark.parametrize("rhs,expect_ub", [(19.0, 20.0), (18.0, 18.0)])
def test_minimal_improvement_rule(oracle_mod, rhs, expect_ub):
    # x + y <= rhs with integer x, y in [0, 20]: the upper bound 20 -> 19 improves by exactly 1.0, which SCIP's
    # bound strengthening test (0.05 * min(ub - lb, |ub|) = 1.0, strict) rejects; 20 -> 18 is accepted
    inst = single_rows([([0, 1], [1.0, 1.0], -INF, rhs)], [0.0, 0.0], [20.0, 20.0], [1, 1])
    lb, ub, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(0.0))
    assert not r.cutoff
    assert list(ub) == [expect_ub, expect_ub]


def test_integer_rounding_and_chain(oracle_mod):
    # 3x + 2y <= 7, x - z >= 1, z >= 0: x <= floor(7/3) = 2, y <= 3; x >= 1 + z >= 1 -> y <= 2
    inst = single_rows([([0, 1], [3.0, 2.0], -INF, 7.0), ([0, 2], [1.0, -1.0], 1.0, INF)],
                       [0.0, 0.0, 0.0], [10.0, 10.0, 10.0], [1, 1, 1])
    lb, ub, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(0.0))
    assert not r.cutoff
    assert list(lb) == [1.0, 0.0, 0.0] and list(ub) == [2.0, 2.0, 1.0]


def test_cutoff_detected(oracle_mod):
    # x + y >= 5 with x, y in [0, 2] is infeasible
    inst = single_rows([([0, 1], [1.0, 1.0], 5.0, INF)], [0.0, 0.0], [2.0, 2.0], [1, 1])
    _, _, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(0.0))
    assert r.cutoff == 1


def test_single_entry_row_forces(oracle_mod):
    # 4x <= 3.99 with continuous x in [0, 1]: the forced single-entry tightening accepts any improvement
    inst = single_rows([([0], [4.0], -INF, 3.99)], [0.0], [1.0], [0])
    lb, ub, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(0.0))
    assert ub[0] == pytest.approx(3.99 / 4.0, rel=1e-15)


def test_node_outside_domain_is_cut_off(oracle_mod):
    inst = single_rows([([0, 1], [1.0, 1.0], -INF, 10.0)], [0.0, 0.0], [5.0, 5.0], [1, 1])
    nodes = NodeBatch(np.array([0, 1, 2], np.int64), np.array([0, 1], np.int32), np.array([7.0, 3.0]),
                      np.array([7.0, 3.0]))
    out = oracle_mod.Oracle(inst).propagate_nodes(inst.lb, inst.ub, nodes, oracle_mod.params(0.0), cap=4)
    assert list(out["cutoff"]) == [1, 0]
    assert out["n"][1] == 1 and out["col"][1, 0] == 1 and out["lb"][1, 0] == 3.0


def _scip_or_skip(oracle_mod, inst, easy):
    import os
    if not os.path.exists(oracle_mod.SCIP_ORACLE):
        return None
    cut, lb, ub, _ = oracle_mod.run_scip(inst, easy=easy)
    return cut, lb, ub


@pytest.mark.parametrize("indicator_first,sortvars,expect_lb4", [(False, True, 0.0), (True, True, 1.0),
                                                                  (False, False, 1.0), (True, False, 1.0)])
def test_binary_skip_order(oracle_mod, indicator_first, sortvars, expect_lb4):
    # x0 + x1 + x2 + x3 - y <= 1, all binary, x0 = x1 = 1: the minimal activity equals the right-hand side.
    # Residual rule: x2 and x3 (lb 0) would drop to 0, but their residual equals rhs, which tightenVarBounds
    # refuses (cons_linear.c:6766); y would rise to 1.  tightenBounds tries the binaries by |a|, then column
    # index, and the first unfixed one it cannot tighten ends the visit (cons_linear.c:7131-7136): y is
    # tightened only if it comes before x2, i.e. if its column index is the lowest.
    cols = [1, 2, 3, 4, 0] if indicator_first else [0, 1, 2, 3, 4]
    y = cols[4]
    lb = np.zeros(5)
    ub = np.ones(5)
    lb[cols[0]] = lb[cols[1]] = 1.0
    inst = single_rows([(cols, [1.0, 1.0, 1.0, 1.0, -1.0], -INF, 1.0)], lb, ub, [1] * 5)
    plb, pub, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(0.0, sortvars=sortvars))
    assert not r.cutoff
    assert plb[y] == expect_lb4 and pub[y] == 1.0
    assert pub[cols[2]] == 1.0 and pub[cols[3]] == 1.0   # the guard keeps the members free
    if sortvars:
        scip = _scip_or_skip(oracle_mod, inst, easy=False)
        if scip is not None:
            assert not scip[0] and np.array_equal(scip[1], plb) and np.array_equal(scip[2], pub)


def test_binary_skip_leaves_the_easy_rule_alone(oracle_mod):
    # the slack rule has no residual guard: with slack 0 every free member drops to 0 and y rises to 1,
    # whatever the order
    lb = np.array([1.0, 1.0, 0.0, 0.0, 0.0])
    inst = single_rows([([0, 1, 2, 3, 4], [1.0, 1.0, 1.0, 1.0, -1.0], -INF, 1.0)], lb, np.ones(5), [1] * 5)
    plb, pub, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(1e6))
    assert list(pub) == [1.0, 1.0, 0.0, 0.0, 1.0] and plb[4] == 1.0
    scip = _scip_or_skip(oracle_mod, inst, easy=True)
    if scip is not None:
        assert np.array_equal(scip[1], plb) and np.array_equal(scip[2], pub)


def test_binary_test_uses_the_global_domain(oracle_mod):
    # x2 is integral with global domain [0, 3] but local [0, 1]: not binary, so it does not end the visit
    # of the binaries and y (after it in column order) is tightened; with global [0, 1] it does end it
    lb = np.array([1.0, 1.0, 0.0, 0.0])
    ub = np.array([1.0, 1.0, 1.0, 1.0])
    inst = single_rows([([0, 1, 2, 3], [1.0, 1.0, 1.0, -1.0], -INF, 1.0)], lb, ub, [1] * 4)
    orc = oracle_mod.Oracle(inst)
    glb = np.zeros(4)
    wide = np.array([1.0, 1.0, 3.0, 1.0])
    l1, _, _ = orc.propagate(lb, ub, oracle_mod.params(0.0), glob=(glb, wide))
    l2, _, _ = orc.propagate(lb, ub, oracle_mod.params(0.0), glob=(glb, ub))
    assert l1[3] == 1.0 and l2[3] == 0.0


def test_node_changes_naming_a_column_twice(oracle_mod):
    """A column named twice in a node takes the tightest bounds; crossing bounds cut the node off."""
    from scip_gb300.instances import NodeBatch, root_mip

    inst = root_mip(0, m=200, n=500)
    par = oracle_mod.params(0.0)
    orc = oracle_mod.Oracle(inst)
    rlb, rub, _ = orc.propagate(inst.lb, inst.ub, par)
    j = int(np.flatnonzero((inst.isint == 1) & (rub - rlb >= 4))[0])
    lo = rlb[j]
    once = NodeBatch(np.array([0, 1], np.int64), np.array([j], np.int32), np.array([lo + 1.0]), np.array([lo + 2.0]))
    twice = NodeBatch(np.array([0, 2], np.int64), np.array([j, j], np.int32), np.array([lo, lo + 1.0]),
                      np.array([lo + 2.0, lo + 3.0]))
    crossing = NodeBatch(np.array([0, 2], np.int64), np.array([j, j], np.int32), np.array([lo, lo + 3.0]),
                         np.array([lo + 1.0, lo + 3.0]))
    for seq in (False, True):
        a = orc.propagate_nodes(rlb, rub, once, par, cap=inst.n, seq=seq)
        b = orc.propagate_nodes(rlb, rub, twice, par, cap=inst.n, seq=seq)
        n = a["n"][0]
        assert not a["cutoff"][0] and not b["cutoff"][0] and b["n"][0] == n
        o1, o2 = np.argsort(a["col"][0, :n]), np.argsort(b["col"][0, :n])
        assert np.array_equal(a["col"][0, :n][o1], b["col"][0, :n][o2])
        assert np.array_equal(a["lb"][0, :n][o1], b["lb"][0, :n][o2])
        assert np.array_equal(a["ub"][0, :n][o1], b["ub"][0, :n][o2])
        assert orc.propagate_nodes(rlb, rub, crossing, par, cap=inst.n, seq=seq)["cutoff"][0] == 1
