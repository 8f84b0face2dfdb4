"""LP-format reader: the linear rows, column bounds and integrality of a (mixed-integer) linear program, read as SCIP's
LP reader reads them (src/scip/reader_lp.c):

* text after a backslash is a comment; tokens are values (strtod syntax, INF/INFINITY), the single characters
  + - : < > = [ ] * ^ (with <=, =<, >=, =>, == folded into <, >, =), and names (anything else up to a blank or one
  of those characters);
* sections (case-insensitive): MIN/MINIMUM/MINIMIZE, MAX/MAXIMUM/MAXIMIZE, SUBJECT TO / SUCH THAT / ST / S.T. / ST.,
  LAZY CONSTRAINTS, USER CUTS, BOUND(S), GEN/GENERAL(S)/INT/INTEGER(S), BIN/BINARY/BINARIES, END; a keyword followed
  by ':' is a row name (isNewSection, reader_lp.c:508-717);
* a row is an optional "name:", terms [sign][value] name (every term after the first needs a sign, the value
  defaults to 1), a sense and a signed right-hand side; lazy constraints and user cuts are rows like the others
  (reader_lp.c:2215-2458);
* a column is created, continuous in [0, +inf), where its name first appears; a bound line is
  [value sense] name [sense value] or "name free" and changes a bound only when it differs from the default
  (reader_lp.c:2644-2818); GENERALS make columns integral; BINARIES make them integral and clip their bounds to
  [0, 1] (reader_lp.c:2821-2933).

Not supported (ValueError): quadratic terms, indicator constraints (->), SOS and semi-continuous sections.  A
column named twice in one row appears once, with the coefficients added.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np

from .instances import INF, Instance

_TOKCHARS = set("+-:<>=[]*^")


def _value_len(s: str, i: int) -> int:
    """length of the value token starting at s[i] (isValueChar, reader_lp.c:238-290), 0 if none starts there"""
    n = len(s)
    j = i
    hasdot = False
    exp = 0  # 0 none, 1 signed pending, 2 unsigned
    first = True
    while j < n:
        c = s[j]
        nc = s[j + 1] if j + 1 < n else "\0"
        if c.isdigit():
            j += 1
        elif exp == 0 and not hasdot and c == "." and (nc.isdigit() or nc.isspace() or nc in "eE\0"):
            hasdot = True
            j += 1
        elif not first and exp == 0 and c in "eE" and (nc in "+-" or nc.isdigit()):
            exp = 1 if nc in "+-" else 2
            j += 1
        elif exp == 1 and c in "+-":
            exp = 2
            j += 1
        else:
            break
        first = False
    return j - i


def _tokens(text: str):
    """the token stream with line numbers"""
    for lineno, raw in enumerate(text.splitlines(), 1):
        line = raw.split("\\", 1)[0]
        i, n = 0, len(line)
        while i < n:
            c = line[i]
            if c.isspace():
                i += 1
                continue
            k = _value_len(line, i) if (c.isdigit() or c == ".") else 0
            if k:
                yield line[i:i + k], lineno
                i += k
                continue
            if c in _TOKCHARS:
                tok = c
                i += 1
                if c in "<>=" and i < n and line[i] == "=":
                    i += 1
                elif c == "=" and i < n and line[i] in "<>":
                    tok = line[i]
                    i += 1
                elif c == "^" and i < n and line[i] == "2":
                    i += 1
                yield tok, lineno
                continue
            j = i
            while j < n and not line[j].isspace() and line[j] not in _TOKCHARS:
                j += 1
            yield line[i:j], lineno
            i = j


_SECTIONS = {
    "MIN": "obj", "MINIMUM": "obj", "MINIMIZE": "obj", "MAX": "obj", "MAXIMUM": "obj", "MAXIMIZE": "obj",
    "ST": "rows", "ST.": "rows", "S.T.": "rows", "BOUND": "bounds", "BOUNDS": "bounds",
    "GEN": "gen", "GENERAL": "gen", "GENERALS": "gen", "INT": "gen", "INTEGER": "gen", "INTEGERS": "gen",
    "BIN": "bin", "BINARY": "bin", "BINARIES": "bin", "SEMI": "semi", "SEMIS": "semi", "SEMI-CONTINUOUS": "semi",
    "SOS": "sos", "END": "end",
}
_PAIRS = {("SUBJECT", "TO"): "rows", ("SUCH", "THAT"): "rows", ("LAZY", "CONSTRAINTS"): "rows",
          ("USER", "CUTS"): "rows"}


def _value(tok: str):
    if tok.upper() in ("INF", "INFINITY"):
        return INF
    try:
        return float(tok)
    except ValueError:
        return None


class _Reader:
    def __init__(self, text: str):
        self.toks = list(_tokens(text))
        self.k = 0
        self.cols: Dict[str, int] = {}
        self.lb: List[float] = []
        self.ub: List[float] = []
        self.isint: List[int] = []
        self.obj: Dict[int, float] = {}
        self.rows: List[Tuple[str, Dict[int, float], float, float]] = []
        self.maximize = False
        self.offset = 0.0

    def peek(self, d=0):
        return self.toks[self.k + d][0] if self.k + d < len(self.toks) else None

    def error(self, msg):
        line = self.toks[min(self.k, len(self.toks) - 1)][1] if self.toks else 0
        raise ValueError(f"LP file, line {line}: {msg}")

    def section_at(self):
        """the section a keyword at the current token starts (and its length in tokens), else (None, 0)"""
        t = self.peek()
        if t is None or self.peek(1) == ":":
            return None, 0
        u = t.upper()
        if u in _SECTIONS:
            return _SECTIONS[u], 1
        nxt = self.peek(1)
        if nxt is not None and (u, nxt.upper()) in _PAIRS:
            return _PAIRS[(u, nxt.upper())], 2
        return None, 0

    def col(self, name, create=True):
        if name not in self.cols:
            if not create:
                self.error(f"unknown column {name}")
            self.cols[name] = len(self.lb)
            self.lb.append(0.0)
            self.ub.append(INF)
            self.isint.append(0)
        return self.cols[name]

    def terms(self, objective):
        """[name:] and the terms up to a sense (rows) or the next section (objective); (name, {col: coef})"""
        name = ""
        if self.peek(1) == ":" and self.section_at()[0] is None:
            name = self.peek()
            self.k += 2
        coefs: Dict[int, float] = {}
        sign, value, havesign, n = 1.0, None, False, 0
        while self.peek() is not None:
            t = self.peek()
            if t in ("+", "-"):
                if value is not None:
                    if not objective:
                        self.error("a constant in a row")
                    self.offset += sign * value  # the objective's constant
                    value = None
                sign = sign * (-1.0 if t == "-" else 1.0) if havesign else (-1.0 if t == "-" else 1.0)
                havesign = True
                self.k += 1
                continue
            v = _value(t)
            if v is not None:
                if value is not None:
                    self.error("two consecutive values")
                value = v
                self.k += 1
                continue
            if t in ("<", ">", "="):
                if objective:
                    self.error("a sense in the objective")
                if value is not None or havesign:
                    self.error("a constant or a sign without a column in a row")
                break
            if t in ("[", "]", "*", "^"):
                raise ValueError("quadratic terms are not supported")
            if objective or (not havesign and value is None):
                sec, _ = self.section_at()
                if sec is not None:
                    break
            if n > 0 and not havesign:
                self.error("expected a sign or a sense")
            j = self.col(t)
            coefs[j] = coefs.get(j, 0.0) + sign * (1.0 if value is None else value)
            sign, value, havesign = 1.0, None, False
            n += 1
            self.k += 1
        if objective and value is not None:
            self.offset += sign * value
        return name, coefs

    def row(self):
        name, coefs = self.terms(False)
        t = self.peek()
        if t not in ("<", ">", "="):
            self.error("expected a sense")
        self.k += 1
        s = 1.0
        while self.peek() in ("+", "-"):
            s *= -1.0 if self.peek() == "-" else 1.0
            self.k += 1
        v = _value(self.peek() or "")
        if v is None:
            self.error("expected a right-hand side")
        self.k += 1
        side = s * v
        if self.peek() == "-" and self.peek(1) == ">":
            raise ValueError("indicator constraints are not supported")
        lhs, rhs = {"<": (-INF, side), ">": (side, INF), "=": (side, side)}[t]
        self.rows.append((name, coefs, lhs, rhs))

    def bound(self):
        lb, ub = 0.0, INF
        left = None
        s = 1.0
        if self.peek() in ("+", "-"):
            s = -1.0 if self.peek() == "-" else 1.0
            self.k += 1
        v = _value(self.peek() or "")
        if v is not None:
            self.k += 1
            left = self.peek()
            if left not in ("<", ">", "="):
                self.error("expected a bound sense")
            self.k += 1
            if left == ">":
                ub = s * v
            elif left == "<":
                lb = s * v
            else:
                lb = ub = s * v
        j = self.col(self.peek())
        self.k += 1
        t = self.peek()
        if t in ("<", ">", "="):
            if not (left is None or left == t and t in "<>"):
                self.error("the two bound senses do not fit")
            self.k += 1
            s = 1.0
            if self.peek() in ("+", "-"):
                s = -1.0 if self.peek() == "-" else 1.0
                self.k += 1
            v = _value(self.peek() or "")
            if v is None:
                self.error("expected a bound value")
            self.k += 1
            if t == ">":
                lb = s * v
            elif t == "<":
                ub = s * v
            else:
                lb = ub = s * v
        elif t is not None and t.upper() == "FREE":
            if left is not None:
                self.error("a bounded column marked free")
            lb, ub = -INF, INF
            self.k += 1
        if lb != 0.0:
            self.lb[j] = lb
        if ub != INF:
            self.ub[j] = ub

    def run(self):
        section = None
        while self.peek() is not None:
            sec, ln = self.section_at()
            if sec is not None:
                if sec == "obj":
                    self.maximize = self.peek().upper().startswith("MAX")
                section = sec
                self.k += ln
                if sec in ("semi", "sos"):
                    raise ValueError(f"{self.toks[self.k - 1][0]} section is not supported")
                if sec == "end":
                    break
                if sec == "obj":
                    _, coefs = self.terms(True)
                    self.obj = coefs
                continue
            if section == "rows":
                self.row()
            elif section == "bounds":
                self.bound()
            elif section in ("gen", "bin"):
                j = self.col(self.peek(), create=False)
                self.k += 1
                self.isint[j] = 1
                if section == "bin":
                    if self.lb[j] < 0.0:
                        self.lb[j] = 0.0
                    if self.ub[j] > 1.0:
                        self.ub[j] = 1.0
            else:
                self.error("text outside a section")


def read_lp(path: str):
    """(Instance, objective coefficients, column names, row names, maximize, objective offset)"""
    with open(path) as f:
        r = _Reader(f.read())
    r.run()
    m, n = len(r.rows), len(r.lb)
    rowptr = np.zeros(m + 1, dtype=np.int64)
    cols, vals = [], []
    for i, (_, coefs, _, _) in enumerate(r.rows):
        items = sorted(coefs.items())
        cols += [c for c, _ in items]
        vals += [v for _, v in items]
        rowptr[i + 1] = len(cols)
    inst = Instance(rowptr, np.array(cols, dtype=np.int32), np.array(vals, dtype=np.float64),
                    np.array([x[2] for x in r.rows], dtype=np.float64), np.array([x[3] for x in r.rows], dtype=np.float64),
                    np.array(r.lb, dtype=np.float64), np.array(r.ub, dtype=np.float64), np.array(r.isint, dtype=np.int8),
                    name=path)
    obj = np.zeros(n)
    for j, v in r.obj.items():
        obj[j] = v
    names = [None] * n
    for k, j in r.cols.items():
        names[j] = k
    return inst, obj, names, [x[0] for x in r.rows], r.maximize, r.offset
