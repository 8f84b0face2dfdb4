"""LP-format reader (scip_gb300/lpfile.py) against SCIP's own (src/scip/reader_lp.c): hand-checkable semantics, the
reference's LP files as SCIP itself reads them (oracle/_ref/scip_dump, where the SCIP sources were available to
build it), and root propagation of what was read against SCIP's."""
import glob
import os
import subprocess

import numpy as np
import pytest

import golden_cases as G
from scip_gb300 import lpfile
from scip_gb300.instances import INF

SMALL = r"""\ a comment line
Maximize
 obj: 3 x + 2 y - z + 4
Subject To
 c1: x + y + z <= 10
 c2: - x + 2 y >= -3   \ trailing comment
 c3: x - y = 0
 2 z + y + z =< 8
 r: 3 w >= 2
Bounds
 -5 <= x <= 5
 y <= 7
 z free
 w >= 1.5
 -inf <= v <= 3
General
 x
Binary
 y w
End
"""


def test_reader_semantics(tmp_path):
    p = tmp_path / "small.lp"
    p.write_text(SMALL)
    inst, obj, names, rows, maximize, offset = lpfile.read_lp(str(p))
    # columns in order of first appearance; v appears only in the bounds
    assert names == ["x", "y", "z", "w", "v"]
    assert maximize and offset == 4.0 and list(obj) == [3.0, 2.0, -1.0, 0.0, 0.0]
    # x: [-5, 5] integral; y: ub 7 clipped to 1 by BINARY; z free; w: lb 1.5 kept (BINARY clips only outside
    # [0, 1]), ub clipped to 1; v: continuous (-inf, 3]
    assert list(inst.isint) == [1, 1, 0, 1, 0]
    assert list(inst.lb) == [-5.0, 0.0, -INF, 1.5, -INF]
    assert list(inst.ub) == [5.0, 1.0, INF, 1.0, 3.0]
    assert rows == ["c1", "c2", "c3", "", "r"]
    assert list(inst.lhs) == [-INF, -3.0, 0.0, -INF, 2.0]
    assert list(inst.rhs) == [10.0, INF, 0.0, 8.0, INF]
    # the fourth row names z twice: one entry with the coefficients added
    k = inst.rowptr[3]
    assert dict(zip(inst.colidx[k:inst.rowptr[4]], inst.vals[k:inst.rowptr[4]])) == {1: 1.0, 2: 3.0}
    k = inst.rowptr[1]
    assert dict(zip(inst.colidx[k:inst.rowptr[2]], inst.vals[k:inst.rowptr[2]])) == {0: -1.0, 1: 2.0}


@pytest.mark.parametrize("text", ["Minimize\n x\nSubject To\n c: x + [ x ^2 ] <= 1\nEnd\n",
                                  "Minimize\n x\nSubject To\n c: b = 1 -> x <= 1\nBinary\n b\nEnd\n",
                                  "Minimize\n x\nSubject To\n c: x <= 1\nSOS\n s1: S1:: x:1\nEnd\n",
                                  "Minimize\n x\nSubject To\n c: x + 2 <= 1\nEnd\n"])
def test_reader_rejects_what_it_does_not_read(tmp_path, text):
    p = tmp_path / "bad.lp"
    p.write_text(text)
    with pytest.raises(ValueError):
        lpfile.read_lp(str(p))


def _dump(oracle_mod, path):
    exe = os.path.join(os.path.dirname(oracle_mod.SCIP_ORACLE), "scip_dump")
    if not os.path.exists(exe):
        pytest.skip("SCIP reader dump (oracle/_ref/scip_dump) not built here")
    r = subprocess.run([exe, path], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    cols, rows, other = {}, {}, []
    for line in r.stdout.splitlines():
        t = line.split()
        if t[0] == "var":
            cols[t[1]] = (int(t[2]), float(t[3]), float(t[4]), float(t[5]))
        elif t[0] == "row":
            ent = {}
            for q in range(int(t[4])):
                ent[t[5 + 2 * q]] = ent.get(t[5 + 2 * q], 0.0) + float(t[6 + 2 * q])
            rows[t[1]] = (float(t[2]), float(t[3]), ent)
        else:
            other.append(t[1])
    return cols, rows, other


def _lp_files(oracle_mod):
    d = os.path.join(oracle_mod.REFDIR, "check", "instances")
    files = sorted(glob.glob(os.path.join(d, "**", "*.lp"), recursive=True))
    if not files:
        pytest.skip("the reference's instance files are not available here")
    return files


def test_reader_reads_the_reference_lp_files_as_scip_does(oracle_mod):
    """Every LP file shipped in the reference's check/instances: linear ones read to exactly SCIP's columns (name,
    integrality, bounds, objective) and rows (name, sides, coefficients); the others raise where SCIP makes
    non-linear constraints (indicator, SOS, quadratic)."""
    nread = 0
    for f in _lp_files(oracle_mod):
        try:
            inst, obj, names, rnames, _, _ = lpfile.read_lp(f)
        except ValueError:
            exe = os.path.join(os.path.dirname(oracle_mod.SCIP_ORACLE), "scip_dump")
            if os.path.exists(exe):
                r = subprocess.run([exe, f], capture_output=True, text=True, timeout=120)
                assert r.returncode != 0 or "other" in r.stdout, f
            continue
        cols, rows, other = _dump(oracle_mod, f)
        assert not other, f
        assert sorted(cols) == sorted(names), f
        for j, nm in enumerate(names):
            assert cols[nm] == (int(inst.isint[j]), inst.lb[j], inst.ub[j], obj[j]), (f, nm)
        assert sorted(rows) == sorted(rnames), f
        for i, rn in enumerate(rnames):
            mine = {names[inst.colidx[p]]: inst.vals[p] for p in range(inst.rowptr[i], inst.rowptr[i + 1])}
            assert rows[rn] == (inst.lhs[i], inst.rhs[i], mine), (f, rn)
        nread += 1
    assert nread >= 20


@pytest.mark.parametrize("name", ["MANN_a9.clq", "stein27_inf", "Side", "1-FullIns_3_reopt/1-FullIns_3"])
def test_root_propagation_of_read_lp_files_agrees_with_scip(oracle_mod, name):
    d = os.path.join(oracle_mod.REFDIR, "check", "instances", "MIP")
    path = os.path.join(d, name + ".lp")
    if not os.path.exists(path) or not os.path.exists(oracle_mod.SCIP_ORACLE):
        pytest.skip("the reference's instances or the SCIP driver are not available here")
    inst = lpfile.read_lp(path)[0]
    for easy in (False, True):
        scut, slb, sub, _ = oracle_mod.run_scip(inst, easy=easy)
        lb, ub, r = oracle_mod.Oracle(inst).propagate(inst.lb, inst.ub, oracle_mod.params(1e6 if easy else 0.0))
        a = G.Agreement()
        a.add(inst.isint, None if r.cutoff else (lb, ub), None if scut else (slb, sub))
        assert a.cutoff_mismatch == 0 and a.int_cols_diff == 0 and a.cont_cols_out_of_tol == 0
