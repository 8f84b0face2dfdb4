"""MPS reader: linear rows and column bounds of a (mixed-integer) linear program, in the semantics of SCIP's
MPS reader (src/scip/reader_mps.c) for the sections that matter to propagation:

* ROWS: N (objective, ignored), L (<= rhs), G (>= rhs), E (= rhs); RHS default 0;
* COLUMNS with 'MARKER' 'INTORG'/'INTEND' integer blocks; integer columns default to [0, 1], and the first
  bound record other than BV, UP <= 1 or FX in [0, 1] turns them into general integers with an infinite
  upper bound before the record is applied (reader_mps.c:2096-2112);
* RANGES: E rows widen to [rhs, rhs+|r|] (r > 0) or [rhs-|r|, rhs] (r < 0), L rows to [rhs-|r|, rhs],
  G rows to [rhs, rhs+|r|];
* BOUNDS: UP, LO, FX, FR, MI, PL, BV, LI, UI (an UP below zero on a column with lower bound 0 makes the lower
  bound -infinity, as MPS readers conventionally do).

Semi-continuous bounds (SC) and quadratic sections are not supported (ValueError).
"""
from __future__ import annotations

from typing import Dict, List

import numpy as np

from .instances import INF, Instance


def read_mps(path: str) -> Instance:
    rows: List[str] = []
    rtype: Dict[str, str] = {}
    rindex: Dict[str, int] = {}
    cols: List[str] = []
    cindex: Dict[str, int] = {}
    isint: List[int] = []
    entries: List[List] = []  # per column: [(row, val)]
    rhs: Dict[str, float] = {}
    rng: Dict[str, float] = {}
    lb: List[float] = []
    ub: List[float] = []
    bounded: List[bool] = []
    section = None
    inint = False
    objname = None
    with open(path) as f:
        for raw in f:
            line = raw.rstrip("\n")
            if not line.strip() or line.startswith("*"):
                continue
            if not line[0].isspace():
                tok = line.split()
                section = tok[0].upper()
                if section in ("QUADOBJ", "QMATRIX", "QSECTION", "QCMATRIX", "SOS", "INDICATORS"):
                    raise ValueError(f"MPS section {section} not supported")
                continue
            tok = line.split()
            if section == "ROWS":
                t, name = tok[0].upper(), tok[1]
                if t == "N":
                    if objname is None:
                        objname = name
                    continue
                rindex[name] = len(rows)
                rows.append(name)
                rtype[name] = t
            elif section == "COLUMNS":
                if len(tok) >= 3 and tok[1].strip("'").upper() == "MARKER":
                    marker = tok[2].strip("'").upper()
                    inint = marker == "INTORG"
                    continue
                name = tok[0]
                if name not in cindex:
                    cindex[name] = len(cols)
                    cols.append(name)
                    isint.append(1 if inint else 0)
                    entries.append([])
                    lb.append(0.0)
                    ub.append(1.0 if inint else INF)
                    bounded.append(False)
                j = cindex[name]
                for k in range(1, len(tok) - 1, 2):
                    r, v = tok[k], float(tok[k + 1])
                    if r in rindex and v != 0.0:
                        entries[j].append((rindex[r], v))
            elif section in ("RHS", "RANGES"):
                pairs = tok[1:] if len(tok) % 2 == 1 else tok
                target = rhs if section == "RHS" else rng
                for k in range(0, len(pairs) - 1, 2):
                    if pairs[k] in rindex:
                        target[pairs[k]] = float(pairs[k + 1])
            elif section == "BOUNDS":
                t = tok[0].upper()
                if t in ("FR", "MI", "PL", "BV"):
                    name = tok[-1] if len(tok) <= 3 else tok[2]
                    val = 0.0
                    if len(tok) == 3 and tok[2] in cindex:
                        name = tok[2]
                    elif len(tok) == 2:
                        name = tok[1]
                else:
                    name, val = (tok[2], float(tok[3])) if len(tok) >= 4 else (tok[1], float(tok[2]))
                if t == "SC":
                    raise ValueError("semi-continuous bounds not supported")
                j = cindex[name]
                if isint[j] and not bounded[j] and not (t == "BV" or (t == "UP" and val <= 1.0)
                                                       or (t == "FX" and 0.0 <= val <= 1.0)):
                    ub[j] = INF
                bounded[j] = True
                if t in ("UP", "UI"):
                    if val < 0.0 and lb[j] == 0.0:
                        lb[j] = -INF
                    ub[j] = val
                elif t in ("LO", "LI"):
                    lb[j] = val
                elif t == "FX":
                    lb[j] = ub[j] = val
                elif t == "FR":
                    lb[j], ub[j] = -INF, INF
                elif t == "MI":
                    lb[j] = -INF
                elif t == "PL":
                    ub[j] = INF
                elif t == "BV":
                    lb[j], ub[j] = 0.0, 1.0
                    isint[j] = 1
                if t in ("LI", "UI"):
                    isint[j] = 1
            elif section in ("ENDATA",):
                break
    m, n = len(rows), len(cols)
    lhs = np.full(m, -INF)
    rh = np.full(m, INF)
    for i, name in enumerate(rows):
        b = rhs.get(name, 0.0)
        t = rtype[name]
        if t == "L":
            rh[i] = b
        elif t == "G":
            lhs[i] = b
        else:
            lhs[i] = rh[i] = b
        if name in rng:
            r = rng[name]
            if t == "E":
                if r > 0:
                    rh[i] = b + abs(r)
                else:
                    lhs[i] = b - abs(r)
            elif t == "L":
                lhs[i] = b - abs(r)
            elif t == "G":
                rh[i] = b + abs(r)
    # row-major entries in column order within each row (columns appear in file order)
    rowent: List[List] = [[] for _ in range(m)]
    for j, es in enumerate(entries):
        for i, v in es:
            rowent[i].append((j, v))
    keep = [i for i in range(m) if rowent[i]]
    rowptr = np.zeros(len(keep) + 1, dtype=np.int64)
    colidx, vals = [], []
    for k, i in enumerate(keep):
        rowptr[k + 1] = rowptr[k] + len(rowent[i])
        for j, v in rowent[i]:
            colidx.append(j)
            vals.append(v)
    return Instance(rowptr, np.array(colidx, dtype=np.int32), np.array(vals, dtype=np.float64), lhs[keep].copy(),
                    rh[keep].copy(), np.array(lb, dtype=np.float64), np.array(ub, dtype=np.float64),
                    np.array(isint, dtype=np.int8), name=path.rsplit("/", 1)[-1])


def write_mps(inst: Instance, path: str, obj=None, name: str = "INSTANCE") -> None:
    """Writes inst (and an objective, default 0) as a free-format MPS file that read_mps and SCIP's reader read back
    to the same rows, columns, integrality and bounds: rows with both sides finite and different become L rows
    with a RANGES entry; integer columns go in one MARKER block and get explicit bounds (UP 1 alone for a [0, 1]
    column, which keeps it binary)."""
    m, n = inst.m, inst.n
    obj = np.zeros(n) if obj is None else np.asarray(obj, dtype=np.float64)
    rows = [f"r{i}" for i in range(m)]
    cols = [f"x{j}" for j in range(n)]
    kind, rhs, rngs = [], [], {}
    for i in range(m):
        lo, hi = inst.lhs[i], inst.rhs[i]
        if lo <= -INF:
            kind.append("L")
            rhs.append(hi)
        elif hi >= INF:
            kind.append("G")
            rhs.append(lo)
        elif lo == hi:
            kind.append("E")
            rhs.append(hi)
        else:
            kind.append("L")
            rhs.append(hi)
            rngs[i] = hi - lo
    colrows: List[List] = [[] for _ in range(n)]
    for i in range(m):
        for p in range(inst.rowptr[i], inst.rowptr[i + 1]):
            colrows[inst.colidx[p]].append((i, inst.vals[p]))
    out = [f"NAME {name}", "ROWS", " N obj"] + [f" {kind[i]} {rows[i]}" for i in range(m)] + ["COLUMNS"]
    order = [j for j in range(n) if inst.isint[j]] + [j for j in range(n) if not inst.isint[j]]
    nint = int(np.count_nonzero(inst.isint))
    for k, j in enumerate(order):
        if k == 0 and nint:
            out.append(" MARKER 'MARKER' 'INTORG'")
        if k == nint and nint:
            out.append(" MARKER 'MARKER' 'INTEND'")
        out.append(f" {cols[j]} obj {float(obj[j])!r}")
        for i, v in colrows[j]:
            out.append(f" {cols[j]} {rows[i]} {float(v)!r}")
    if nint == n and nint:
        out.append(" MARKER 'MARKER' 'INTEND'")
    out.append("RHS")
    out += [f" rhs {rows[i]} {float(rhs[i])!r}" for i in range(m) if rhs[i] != 0.0]
    if rngs:
        out.append("RANGES")
        out += [f" rng {rows[i]} {float(r)!r}" for i, r in rngs.items()]
    out.append("BOUNDS")
    for j in range(n):
        lo, hi = inst.lb[j], inst.ub[j]
        if inst.isint[j] and lo == 0.0 and hi == 1.0:
            out.append(f" UP bnd {cols[j]} 1.0")
            continue
        if lo <= -INF and hi >= INF:
            out.append(f" FR bnd {cols[j]}")
            continue
        out.append(f" MI bnd {cols[j]}" if lo <= -INF else f" LO bnd {cols[j]} {float(lo)!r}")
        out.append(f" PL bnd {cols[j]}" if hi >= INF else f" UP bnd {cols[j]} {float(hi)!r}")
    out.append("ENDATA")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
