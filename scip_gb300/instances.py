"""Seeded synthetic propagation workloads (linear rows + column bounds + node bound changes).

Every instance is a set of linear rows  lhs_i <= sum_j a_ij x_j <= rhs_i  (CSR, infinite sides = +-1e20)
over columns with bounds [lb_j, ub_j] and an integrality flag, the data that SCIP's cons_linear
propagation reads from its transformed problem (struct SCIP_ConsData, cons_linear.c:187-266).

Generators (all driven by numpy's PCG64 so that this container and an aarch64 host produce the same
arrays for the same seed):

* ``root_mip``  -- 2,000 x 5,000, row length U{5..15}, integer coefficients U{-10..10}\\{0}, 70 % integer
  columns in [0,10], 30 % continuous in [0,100]; 80 % ``<=`` rows with rhs = a.x0 + U[0,5], 10 % ranged
  rows a.x0 -+ U[0,5], 10 % equalities at a.x0 for a feasible point x0.
* ``zipf_mip``  -- 1,000,000 x 2,000,000, row lengths Zipf(1.5) truncated to [2,5000] by rejection,
  |a| log-uniform in [1e-2,1e2] with random sign, 60 % integer in [0,20], 30 % continuous in [0,1e3],
  10 % continuous with one infinite bound; senses from x0 with 85 % ``<=``, 10 % ranged, 5 % equalities.
* ``node_mip``  -- 200,000 x 400,000 built like ``zipf_mip`` but with row lengths U{5..40}.
* ``node_batch`` -- branch-and-bound node bound changes: 1..64 integer columns per node (count
  log-uniform) fixed to random integer values inside the given (root) bounds.
* ``uneven_batch`` -- distinct instances of three families (set covering, multi-knapsack, network flow
  with arc-open indicators) with log-uniform row counts and columns = 2 x rows.

Sizes are parameters, so tests use the same generators at small scale.
"""
from __future__ import annotations

import dataclasses
import struct
from typing import List, Optional

import numpy as np

INF = 1e20


@dataclasses.dataclass
class Instance:
    """Rows in CSR form plus column data; the layout the C-ABI uploads (include/gbp.h)."""

    rowptr: np.ndarray  # int64 [m+1]
    colidx: np.ndarray  # int32 [nnz]
    vals: np.ndarray  # float64 [nnz]
    lhs: np.ndarray  # float64 [m]
    rhs: np.ndarray  # float64 [m]
    lb: np.ndarray  # float64 [n]
    ub: np.ndarray  # float64 [n]
    isint: np.ndarray  # int8 [n]
    name: str = ""
    x0: Optional[np.ndarray] = None  # a feasible point the generator built the sides from (if any)

    @property
    def m(self) -> int:
        return int(self.rowptr.shape[0] - 1)

    @property
    def n(self) -> int:
        return int(self.lb.shape[0])

    @property
    def nnz(self) -> int:
        return int(self.colidx.shape[0])

    def csc(self):
        """Column-major copy (colptr int64 [n+1], rowidx int32 [nnz], vals float64 [nnz])."""
        m, n = self.m, self.n
        rows = np.repeat(np.arange(m, dtype=np.int32), np.diff(self.rowptr))
        order = np.lexsort((rows, self.colidx))
        colptr = np.zeros(n + 1, dtype=np.int64)
        np.cumsum(np.bincount(self.colidx, minlength=n), out=colptr[1:])
        return colptr, rows[order].astype(np.int32), self.vals[order].copy()

    def write(self, path: str) -> None:
        """Instance file read by the SCIP oracle driver (oracle/scip_driver.c)."""
        with open(path, "wb") as f:
            f.write(b"LPINST01")
            f.write(struct.pack("<4q", self.m, self.n, self.nnz, 0))
            for arr, dt in ((self.rowptr, "<i8"), (self.colidx, "<i4"), (self.vals, "<f8"),
                            (self.lhs, "<f8"), (self.rhs, "<f8"), (self.lb, "<f8"), (self.ub, "<f8"),
                            (self.isint, "i1")):
                f.write(np.ascontiguousarray(arr, dtype=dt).tobytes())


@dataclasses.dataclass
class NodeBatch:
    """Bound changes per node: node k changes columns col[ptr[k]:ptr[k+1]] to [lb, ub]."""

    ptr: np.ndarray  # int64 [nnodes+1]
    col: np.ndarray  # int32
    lb: np.ndarray  # float64
    ub: np.ndarray  # float64

    @property
    def nnodes(self) -> int:
        return int(self.ptr.shape[0] - 1)

    def write(self, path: str) -> None:
        with open(path, "wb") as f:
            f.write(b"LPNODE01")
            f.write(struct.pack("<2q", self.nnodes, int(self.col.shape[0])))
            for arr, dt in ((self.ptr, "<i8"), (self.col, "<i4"), (self.lb, "<f8"), (self.ub, "<f8")):
                f.write(np.ascontiguousarray(arr, dtype=dt).tobytes())


# ----------------------------------------------------------------------------------------------
# Seeded draws that every machine reproduces bit for bit: numpy's generators are exact, but its vectorised
# exp / log round differently on different CPUs, so log-uniform values are built from exactly rounded operations only.
_POW_TABLES = {}


def _pow_tables(ratio: float):
    """ratio^(i/2^10) and ratio^(j/2^20) for i, j in 0..1023, each the double nearest to the exact value (decimal
    arithmetic at 40 digits, then one correctly rounded conversion)."""
    if ratio not in _POW_TABLES:
        import decimal

        ctx = decimal.Context(prec=40)
        r = decimal.Decimal(repr(ratio))
        coarse = np.array([float(ctx.power(r, decimal.Decimal(i) / 1024)) for i in range(1024)])
        fine = np.array([float(ctx.power(r, decimal.Decimal(j) / (1 << 20))) for j in range(1024)])
        _POW_TABLES[ratio] = (coarse, fine)
    return _POW_TABLES[ratio]


def log_uniform(rng: np.random.Generator, lo: float, hi: float, size: int) -> np.ndarray:
    """lo * (hi / lo)^u with u uniform on a grid of 2^20 steps in [0, 1): a product of two table entries, so the
    same on every machine."""
    coarse, fine = _pow_tables(hi / lo)
    k = rng.integers(0, 1 << 20, size=size)
    return lo * coarse[k >> 10] * fine[k & 1023]


def log_uniform_count(rng: np.random.Generator, kmax: int, size: int) -> np.ndarray:
    """floor((kmax + 1)^u) for u uniform in [0, 1), i.e. the number of j in 1..kmax with ln j / ln(kmax + 1) <= u;
    the thresholds are exact decimal quotients rounded once, so the same on every machine."""
    import decimal

    ctx = decimal.Context(prec=40)
    den = ctx.ln(decimal.Decimal(kmax + 1))
    thr = np.array([float(ctx.divide(ctx.ln(decimal.Decimal(j)), den)) for j in range(1, kmax + 1)])
    u = rng.random(size)
    return np.searchsorted(thr, u, side="right").astype(np.int64)


def _distinct_columns(rng: np.random.Generator, lengths: np.ndarray, n: int) -> np.ndarray:
    """Uniform columns per row without repeats inside a row (rows keep their sampling order)."""
    m = lengths.shape[0]
    rowptr = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(lengths, out=rowptr[1:])
    nnz = int(rowptr[-1])
    rows = np.repeat(np.arange(m, dtype=np.int64), lengths)
    cols = rng.integers(0, n, size=nnz, dtype=np.int64)
    for _ in range(100):
        key = rows * n + cols
        order = np.argsort(key, kind="stable")
        sk = key[order]
        dup = np.zeros(nnz, dtype=bool)
        dup[order[1:][sk[1:] == sk[:-1]]] = True
        nd = int(dup.sum())
        if nd == 0:
            break
        cols[dup] = rng.integers(0, n, size=nd, dtype=np.int64)
    else:  # pragma: no cover - probability ~0 for the sizes used
        raise RuntimeError("could not draw distinct columns")
    return rowptr, cols.astype(np.int32)


def _sides_from_point(rng, rowptr, colidx, vals, x0, frac_le, frac_ranged, slack_hi):
    """Row senses from a feasible point: '<=' with slack, ranged +-slack, or equality."""
    m = rowptr.shape[0] - 1
    rows = np.repeat(np.arange(m), np.diff(rowptr))
    act = np.bincount(rows, weights=vals * x0[colidx], minlength=m)
    u = rng.random(m)
    s1 = rng.uniform(0.0, slack_hi, size=m)
    s2 = rng.uniform(0.0, slack_hi, size=m)
    lhs = np.full(m, -INF)
    rhs = act + s1
    ranged = (u >= frac_le) & (u < frac_le + frac_ranged)
    eq = u >= frac_le + frac_ranged
    lhs[ranged] = act[ranged] - s2[ranged]
    lhs[eq] = act[eq]
    rhs[eq] = act[eq]
    return lhs, rhs


def root_mip(seed: int = 0, m: int = 2000, n: int = 5000) -> Instance:
    """Plain single-problem root propagation workload (2,000 x 5,000 at default size)."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    lengths = rng.integers(5, 16, size=m)
    rowptr, colidx = _distinct_columns(rng, lengths, n)
    mag = rng.integers(1, 11, size=colidx.shape[0]).astype(np.float64)
    vals = np.where(rng.random(colidx.shape[0]) < 0.5, -mag, mag)
    isint = (rng.random(n) < 0.7).astype(np.int8)
    lb = np.zeros(n)
    ub = np.where(isint == 1, 10.0, 100.0)
    x0 = np.where(isint == 1, rng.integers(0, 11, size=n).astype(np.float64), rng.uniform(0.0, 100.0, size=n))
    lhs, rhs = _sides_from_point(rng, rowptr, colidx, vals, x0, 0.8, 0.1, 5.0)
    return Instance(rowptr, colidx, vals, lhs, rhs, lb, ub, isint, name=f"root_mip(seed={seed},{m}x{n})", x0=x0)


def _general_columns(rng, n):
    """60 % integer [0,20], 30 % continuous [0,1e3], 10 % continuous with one infinite bound."""
    u = rng.random(n)
    isint = (u < 0.6).astype(np.int8)
    lb = np.zeros(n)
    ub = np.where(u < 0.6, 20.0, 1e3)
    oneinf = u >= 0.9
    lowinf = oneinf & (rng.random(n) < 0.5)
    upinf = oneinf & ~lowinf
    lb[lowinf] = -INF
    ub[upinf] = INF
    x0 = np.where(isint == 1, rng.integers(0, 21, size=n).astype(np.float64), rng.uniform(0.0, 1e3, size=n))
    return isint, lb, ub, x0  # x0 lies in [0, 1e3] for every column, inside all bounds


def _general_mip(rng, lengths, n, name):
    rowptr, colidx = _distinct_columns(rng, lengths, n)
    nnz = colidx.shape[0]
    mag = log_uniform(rng, 1e-2, 1e2, nnz)
    vals = np.where(rng.random(nnz) < 0.5, -mag, mag)
    isint, lb, ub, x0 = _general_columns(rng, n)
    lhs, rhs = _sides_from_point(rng, rowptr, colidx, vals, x0, 0.85, 0.10, 5.0)
    return Instance(rowptr, colidx, vals, lhs, rhs, lb, ub, isint, name=name, x0=x0)


def zipf_lengths(rng: np.random.Generator, m: int, a: float = 1.5, lo: int = 2, hi: int = 5000) -> np.ndarray:
    """Zipf(a) row lengths truncated to [lo, hi] by rejection."""
    out = np.empty(0, dtype=np.int64)
    while out.shape[0] < m:
        x = rng.zipf(a, size=2 * (m - out.shape[0]) + 64)
        out = np.concatenate([out, x[(x >= lo) & (x <= hi)]])
    return out[:m]


def zipf_mip(seed: int = 1, m: int = 1_000_000, n: int = 2_000_000, hi: int = 5000) -> Instance:
    """Large single instance with Zipf row lengths (load-balance stress)."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    lengths = zipf_lengths(rng, m, 1.5, 2, min(hi, n))
    return _general_mip(rng, lengths, n, f"zipf_mip(seed={seed},{m}x{n})")


def node_mip(seed: int = 2, m: int = 200_000, n: int = 400_000) -> Instance:
    """Shared matrix of the batched branch-and-bound node workload (row lengths U{5..40})."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    lengths = rng.integers(5, 41, size=m)
    return _general_mip(rng, lengths, n, f"node_mip(seed={seed},{m}x{n})")


def node_batch(inst: Instance, lb: np.ndarray, ub: np.ndarray, nnodes: int, seed: int = 3,
               kmax: int = 64, tight: float = 0.0) -> NodeBatch:
    """Nodes fixing 1..kmax integer columns (count log-uniform) to random values inside [lb, ub].

    tight > 0: that fraction of the nodes first fixes, against one row whose right-hand side the root fixpoint
    leaves reachable and whose integer columns can pass it, the row's integer columns one by one (in random order)
    at the bound that raises the row's minimal activity, up to the first fixing that carries it past the side -- a
    dive that branches one row into infeasibility -- and then makes the random fixings.  On the 200,000 x 400,000
    workload tight = 0.15 cuts off about 15 % of the nodes (0.4 % without).  The default (tight = 0) draws exactly
    the stream of the plain generator."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    intcols = np.flatnonzero((inst.isint == 1) & (ub > lb) & (ub < INF) & (lb > -INF))
    if intcols.shape[0] == 0:
        raise ValueError("no unfixed finite integer columns")
    kmax = min(kmax, intcols.shape[0])
    ks = log_uniform_count(rng, kmax, nnodes)
    chosen = []
    for k in range(nnodes):
        chosen.append(np.sort(rng.choice(intcols, size=int(ks[k]), replace=False)))
    lo_all, hi_all = lb, ub
    pushed = [None] * nnodes
    if tight > 0.0:
        trng = np.random.default_rng(np.random.PCG64(seed + 7919))
        fin = np.isfinite(lb) & np.isfinite(ub) & (np.abs(lb) < INF) & (np.abs(ub) < INF)
        a = inst.vals
        c = inst.colidx
        lo_c = np.where(a > 0, lb[c], ub[c])
        minact = np.add.reduceat(a * np.where(fin[c], lo_c, 0.0), inst.rowptr[:-1].astype(np.int64))
        rowfin = np.add.reduceat((~fin[c]).astype(np.int64), inst.rowptr[:-1].astype(np.int64)) == 0
        movable = (inst.isint[c] == 1) & (ub[c] > lb[c]) & fin[c]
        raise_int = np.add.reduceat(np.where(movable, np.abs(a) * (ub[c] - lb[c]), 0.0),
                                    inst.rowptr[:-1].astype(np.int64))
        cand = np.flatnonzero(rowfin & (inst.rhs < INF) & (np.diff(inst.rowptr) > 0) & (minact <= inst.rhs)
                              & (minact + raise_int > inst.rhs))
        for k in range(nnodes):
            if trng.random() >= tight or cand.shape[0] == 0:
                continue
            i = int(cand[trng.integers(cand.shape[0])])
            p0, p1 = int(inst.rowptr[i]), int(inst.rowptr[i + 1])
            act = float(minact[i])
            fix_c, fix_v = [], []
            for p in p0 + trng.permutation(p1 - p0):
                j = int(c[p])
                if inst.isint[j] != 1 or not (ub[j] > lb[j]):
                    continue
                v = ub[j] if a[p] > 0 else lb[j]
                step = a[p] * (v - (lb[j] if a[p] > 0 else ub[j]))
                act += step
                fix_c.append(j)
                fix_v.append(v)
                if act > inst.rhs[i]:
                    break
            if fix_c:
                pushed[k] = (np.array(fix_c, dtype=np.int64), np.array(fix_v))
    ptr = np.zeros(nnodes + 1, dtype=np.int64)
    cols_l, vals_l = [], []
    for k in range(nnodes):
        base = chosen[k]
        lo = lo_all[base]
        hi = hi_all[base]
        v = np.minimum(np.floor(lo + rng.random(base.shape[0]) * (hi - lo + 1.0)), hi)
        if pushed[k] is not None:
            pc, pv = pushed[k]
            keep = ~np.isin(base, pc)
            base, v = np.concatenate([pc, base[keep]]), np.concatenate([pv, v[keep]])
            o = np.argsort(base, kind="stable")
            base, v = base[o], v[o]
        cols_l.append(base)
        vals_l.append(v)
        ptr[k + 1] = ptr[k] + base.shape[0]
    cols = np.concatenate(cols_l).astype(np.int32) if cols_l else np.zeros(0, np.int32)
    v = np.concatenate(vals_l) if vals_l else np.zeros(0)
    return NodeBatch(ptr, cols, v.copy(), v.copy())


# ---------------------------------------------------------------- uneven instance families
def set_cover(rng: np.random.Generator, m: int, n: int) -> Instance:
    """Set covering: binary columns, rows sum_{j in S_i} x_j >= 1 with |S_i| in 3..30."""
    lengths = rng.integers(3, 31, size=m)
    lengths = np.minimum(lengths, n)
    rowptr, colidx = _distinct_columns(rng, lengths, n)
    vals = np.ones(colidx.shape[0])
    lhs = np.ones(m)
    rhs = np.full(m, INF)
    return Instance(rowptr, colidx, vals, lhs, rhs, np.zeros(n), np.ones(n), np.ones(n, dtype=np.int8),
                    name=f"set_cover({m}x{n})", x0=np.ones(n))


def indicator_packing(rng: np.random.Generator, m: int, n: int, kmin: int = 4, kmax: int = 30,
                      long_frac: float = 0.0) -> Instance:
    """Binary packing rows with one indicator: sum_{j in S_i} x_j - y_i <= 1 (|S_i| in kmin..kmax, the rows of
    a long_frac share have 65..300 entries), all columns binary.  Once two members of a row are fixed to 1 its
    minimal activity equals the right-hand side; the residual rule then leaves the free members alone
    (cons_linear.c:6766) and fixes y_i to 1 only if y_i comes before the first free member in the row's
    propagation order (larger |a| first, ties by column index).  The members carry coefficient 1 and the
    indicator 1 or 2, so both outcomes occur."""
    lengths = rng.integers(kmin, kmax + 1, size=m)
    if long_frac > 0:
        big = rng.random(m) < long_frac
        lengths[big] = rng.integers(65, 301, size=int(big.sum()))
    lengths = np.minimum(lengths, n - 1)
    rowptr, colidx = _distinct_columns(rng, lengths + 1, n)
    vals = np.ones(colidx.shape[0])
    last = rowptr[1:] - 1                      # the indicator: the last entry of each row
    vals[last] = -rng.choice([1.0, 2.0], size=m, p=[0.8, 0.2])
    lhs = np.full(m, -INF)
    rhs = np.ones(m)
    return Instance(rowptr, colidx, vals, lhs, rhs, np.zeros(n), np.ones(n), np.ones(n, dtype=np.int8),
                    name=f"indicator_packing({m}x{n})", x0=np.zeros(n))


def gcd_rows(rng: np.random.Generator, m: int, n: int, long_frac: float = 0.0, equations: bool = True,
             continuous: bool = True) -> Instance:
    """Ranged rows and equations whose integer part shares a divisor: sum_k g*c_k*x_k + (other entries) in
    [lhs, rhs] with g in {2, 3, 4, 5, 6, 7, 10, 12} per row and |c_k| in 1..4; about 1.5 other entries per row
    carry +-1, 2, +-3 or 1.5.  The first 10 % of the columns are binary, the last 5 % continuous.  The sides come from a feasible point with a
    range narrower than g (half of the rows are equations), so the other entries' activity is confined to one
    residue class modulo g -- the case rangedRowPropagation (cons_linear.c:5715-6695) works on.  Rows have 3..8
    entries, or 65..200 for a long_frac share; general integer columns lie in [0, U] with U in 2..10.

    With equations=False every row is ranged, with sides a quarter off the half-integral activities: a residual
    activity then never equals a side, so tightenVarBounds' minres/rhs != 1 guard (cons_linear.c:6766), which
    makes the fixpoint depend on the order rows are visited in, never blocks a deduction.  continuous=False makes
    the last 5 % of the columns general integers in [0, 10] instead."""
    lengths = rng.integers(3, 9, size=m)
    if long_frac > 0:
        big = rng.random(m) < long_frac
        lengths[big] = rng.integers(65, 201, size=int(big.sum()))
    lengths = np.minimum(lengths, n)
    rowptr, colidx = _distinct_columns(rng, lengths, n)
    nnz = colidx.shape[0]
    g = rng.choice([2, 3, 4, 5, 6, 7, 10, 12], size=m)
    gp = np.repeat(g, lengths).astype(np.float64)
    c = rng.integers(1, 5, size=nnz) * np.where(rng.random(nnz) < 0.5, -1, 1)
    vals = gp * c
    other = rng.random(nnz) < 1.5 / np.repeat(lengths, lengths)
    vals[other] = rng.choice([1.0, -1.0, 2.0, -3.0, 3.0, 1.5], size=int(other.sum()))
    # columns by type -- binaries, general integers, continuous -- so that SCIP's variable indices (it keeps its
    # variables sorted by type, prob.c:887) follow the column order, on which the order ties are broken here
    nb, nc = n // 10, n // 20
    isint = (np.arange(n) < n - nc).astype(np.int8) if continuous else np.ones(n, dtype=np.int8)
    ub = np.concatenate([np.ones(nb), rng.integers(2, 11, size=n - nb - nc).astype(np.float64), np.full(nc, 10.0)])
    lb = np.zeros(n)
    x0 = np.where(isint == 1, np.floor(rng.random(n) * (ub + 1)), rng.uniform(0.0, 10.0, size=n))
    rows = np.repeat(np.arange(m), lengths)
    act = np.bincount(rows, weights=vals * x0[colidx], minlength=m)
    r1 = np.floor(rng.random(m) * (g - 1))
    r2 = np.floor(rng.random(m) * (g - 1 - r1))
    if equations:
        eq = rng.random(m) < 0.5
        r1[eq] = 0.0
        r2[eq] = 0.0
    else:
        r1 += 0.25
        r2 += 0.25
    return Instance(rowptr, colidx, vals, act - r1, act + r2, lb, ub, isint, name=f"gcd_rows({m}x{n})", x0=x0)


def multi_knapsack(rng: np.random.Generator, m: int, n: int) -> Instance:
    """Multi-knapsack: integer columns in [0,5], weights U{1..100}, capacity 40 % of the row's max activity."""
    lengths = np.minimum(rng.integers(5, 41, size=m), n)
    rowptr, colidx = _distinct_columns(rng, lengths, n)
    vals = rng.integers(1, 101, size=colidx.shape[0]).astype(np.float64)
    rows = np.repeat(np.arange(m), lengths)
    maxact = np.bincount(rows, weights=vals * 5.0, minlength=m)
    rhs = np.floor(0.4 * maxact)
    lhs = np.full(m, -INF)
    return Instance(rowptr, colidx, vals, lhs, rhs, np.zeros(n), np.full(n, 5.0), np.ones(n, dtype=np.int8),
                    name=f"multi_knapsack({m}x{n})", x0=np.zeros(n))


def network_flow(rng: np.random.Generator, m: int) -> Instance:
    """Fixed-charge network flow: conservation equalities over continuous arc flows in [0, cap] plus
    linking rows flow_a - cap_a * open_a <= 0 with integer open_a in [0,1].

    With V graph nodes and A arcs there are V + A rows and 2A columns; A = 2V/... is chosen so that
    rows ~ m and the arc count matches the column budget as closely as the family allows."""
    nv = max(2, m // 3)
    na = max(1, m - nv)
    tail = rng.integers(0, nv, size=na)
    head = (tail + rng.integers(1, nv, size=na)) % nv
    cap = rng.uniform(1.0, 50.0, size=na)
    x0 = rng.uniform(0.0, 1.0, size=na) * cap * (rng.random(na) < 0.7)
    supply = np.bincount(tail, weights=x0, minlength=nv) - np.bincount(head, weights=x0, minlength=nv)
    # conservation rows: out - in = supply
    crow = np.concatenate([tail, head])
    ccol = np.concatenate([np.arange(na), np.arange(na)])
    cval = np.concatenate([np.ones(na), -np.ones(na)])
    order = np.lexsort((ccol, crow))
    crow, ccol, cval = crow[order], ccol[order], cval[order]
    cnt = np.bincount(crow, minlength=nv)
    # linking rows
    lrow = np.repeat(np.arange(na), 2) + nv
    lcol = np.stack([np.arange(na), na + np.arange(na)], axis=1).reshape(-1)
    lval = np.stack([np.ones(na), -cap], axis=1).reshape(-1)
    mm = nv + na
    rowlen = np.concatenate([cnt, np.full(na, 2)])
    rowptr = np.zeros(mm + 1, dtype=np.int64)
    np.cumsum(rowlen, out=rowptr[1:])
    colidx = np.concatenate([ccol, lcol]).astype(np.int32)
    vals = np.concatenate([cval, lval])
    lhs = np.concatenate([supply, np.full(na, -INF)])
    rhs = np.concatenate([supply, np.zeros(na)])
    n = 2 * na
    lb = np.zeros(n)
    ub = np.concatenate([cap, np.ones(na)])
    isint = np.concatenate([np.zeros(na, dtype=np.int8), np.ones(na, dtype=np.int8)])
    x0full = np.concatenate([x0, (x0 > 0).astype(np.float64)])
    return Instance(rowptr, colidx, vals, lhs, rhs, lb, ub, isint, name=f"network_flow({mm}x{n})", x0=x0full)


def uneven_batch(seed: int = 4, count: int = 512, rmin: int = 1000, rmax: int = 200_000) -> List[Instance]:
    """Distinct instances with log-uniform row counts; families cycle set cover / knapsack / network."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    rows = np.floor(log_uniform(rng, float(rmin), float(rmax), count)).astype(np.int64)
    out = []
    for k in range(count):
        m = int(rows[k])
        fam = k % 3
        if fam == 0:
            out.append(set_cover(rng, m, 2 * m))
        elif fam == 1:
            out.append(multi_knapsack(rng, m, 2 * m))
        else:
            out.append(network_flow(rng, m))
    return out


def mixed_small(rng: np.random.Generator) -> Instance:
    """A small random MIP (2..24 columns, up to twice as many rows of 1..8 entries) that mixes what makes
    activity arithmetic delicate: coefficients from small integers over normal reals to magnitudes 1e3..1e7 and
    1e-5..1e-1 in one row, infinite and huge bounds, free and half-bounded columns, equations and ranged rows.
    Sides come from a point inside the bounds, so most instances are feasible; one in ten gets one row whose sides
    cross (an infeasible instance)."""
    n = int(rng.integers(2, 25))
    m = int(rng.integers(1, 2 * n))
    style = int(rng.integers(0, 4))  # 0: small integers only; 1..3: mixed magnitudes
    rowptr, cols, vals = [0], [], []
    for _ in range(m):
        k = int(rng.integers(1, min(n, 8) + 1))
        for c in np.sort(rng.choice(n, k, replace=False)):
            t = rng.random()
            if style == 0 or t < 0.5:
                v = float(rng.integers(-9, 10)) or 1.0
            elif t < 0.7:
                v = float(rng.normal() * 10)
            elif t < 0.85:
                v = float(rng.choice([-1, 1]) * 10 ** rng.uniform(3, 7))
            else:
                v = float(rng.choice([-1, 1]) * 10 ** rng.uniform(-5, -1))
            cols.append(int(c))
            vals.append(v)
        rowptr.append(len(cols))
    isint = (rng.random(n) < (0.9, 0.5, 0.2, 0.7)[style]).astype(np.int8)
    lb, ub = np.empty(n), np.empty(n)
    for j in range(n):
        t = rng.random()
        if isint[j]:
            if t < 0.5:
                lb[j], ub[j] = 0.0, 1.0
            elif t < 0.8:
                lb[j] = float(rng.integers(-10, 5))
                ub[j] = lb[j] + float(rng.integers(0, 30))
            elif t < 0.9:
                lb[j], ub[j] = 0.0, INF
            else:
                lb[j], ub[j] = -INF, float(rng.integers(-5, 50))
        else:
            if t < 0.4:
                lb[j] = float(rng.uniform(-10, 0))
                ub[j] = lb[j] + float(rng.uniform(0, 40))
            elif t < 0.6:
                lb[j], ub[j] = 0.0, INF
            elif t < 0.7:
                lb[j], ub[j] = -INF, INF
            elif t < 0.8:
                lb[j], ub[j] = -INF, float(rng.uniform(-5, 50))
            else:
                lb[j], ub[j] = 0.0, float(10 ** rng.uniform(-3, 6))
    x = np.clip(rng.uniform(-5, 20, n), np.where(lb > -INF, lb, -50), np.where(ub < INF, ub, 50))
    x = np.where(isint == 1, np.clip(np.round(x), lb, ub), x)
    lhs, rhs = np.empty(m), np.empty(m)
    for i in range(m):
        a = np.array(vals[rowptr[i]:rowptr[i + 1]])
        act = float(a @ x[np.array(cols[rowptr[i]:rowptr[i + 1]])])
        t = rng.random()
        slack = abs(rng.normal()) * (0.0, 1.0, 5.0)[int(rng.integers(0, 3))]
        if t < 0.4:
            lhs[i], rhs[i] = -INF, act + slack
        elif t < 0.7:
            lhs[i], rhs[i] = act - slack, INF
        elif t < 0.75:
            lhs[i] = rhs[i] = act
        else:
            lhs[i], rhs[i] = act - slack, act + slack + 1.0
    if rng.random() < 0.1:
        i = int(rng.integers(0, m))
        if lhs[i] > -INF:
            rhs[i] = lhs[i] - 1e-3
    return Instance(np.array(rowptr, np.int64), np.array(cols, np.int32), np.array(vals), lhs, rhs, lb, ub, isint,
                    name="mixed_small")


def mixed_huge(rng: np.random.Generator) -> Instance:
    """mixed_small with contributions past SCIP's hugeval (1e15): a fifth of the coefficients scaled by 1e3..1e7
    (up to about 1e14) and three in ten of the bounded continuous columns widened to 1e5..1e9, so that activities
    count huge contributions (the neghuge/poshuge counters) besides infinite ones; sides again from a point inside
    the bounds."""
    inst = mixed_small(rng)
    vals = inst.vals.copy()
    sel = rng.random(len(vals)) < 0.2
    vals[sel] *= 10 ** rng.uniform(3, 7, int(sel.sum()))
    lb, ub = inst.lb.copy(), inst.ub.copy()
    wide = (inst.isint == 0) & (ub < INF) & (lb > -INF) & (rng.random(inst.n) < 0.3)
    ub[wide] = lb[wide] + 10 ** rng.uniform(5, 9, int(wide.sum()))
    x = np.clip(rng.uniform(-5, 20, inst.n), np.where(lb > -INF, lb, -50), np.where(ub < INF, ub, 50))
    x = np.where(inst.isint == 1, np.clip(np.round(x), lb, ub), x)
    lhs, rhs = inst.lhs.copy(), inst.rhs.copy()
    for i in range(inst.m):
        sl = slice(int(inst.rowptr[i]), int(inst.rowptr[i + 1]))
        act = float(vals[sl] @ x[inst.colidx[sl]])
        if lhs[i] > -INF and rhs[i] < INF:
            w = rhs[i] - lhs[i]
            lhs[i], rhs[i] = act - w / 2, act + w / 2
        elif lhs[i] > -INF:
            lhs[i] = act - abs(rng.normal())
        elif rhs[i] < INF:
            rhs[i] = act + abs(rng.normal())
    return Instance(inst.rowptr, inst.colidx, vals, lhs, rhs, lb, ub, inst.isint, name="mixed_huge")


def concat_instances(insts: List[Instance]):
    """Block-diagonal union of independent instances: (instance, row_off, col_off) with instance k owning rows
    row_off[k]:row_off[k+1] and columns col_off[k]:col_off[k+1]."""
    row_off = np.zeros(len(insts) + 1, dtype=np.int64)
    col_off = np.zeros(len(insts) + 1, dtype=np.int64)
    nnz_off = np.zeros(len(insts) + 1, dtype=np.int64)
    for k, inst in enumerate(insts):
        row_off[k + 1] = row_off[k] + inst.m
        col_off[k + 1] = col_off[k] + inst.n
        nnz_off[k + 1] = nnz_off[k] + inst.nnz
    rowptr = np.zeros(int(row_off[-1]) + 1, dtype=np.int64)
    colidx = np.empty(int(nnz_off[-1]), dtype=np.int32)
    for k, inst in enumerate(insts):
        rowptr[row_off[k] + 1:row_off[k + 1] + 1] = inst.rowptr[1:] + nnz_off[k]
        colidx[nnz_off[k]:nnz_off[k + 1]] = inst.colidx + col_off[k]
    cat = lambda f: np.concatenate([getattr(i, f) for i in insts])
    x0 = np.concatenate([i.x0 for i in insts]) if all(i.x0 is not None for i in insts) else None
    big = Instance(rowptr, colidx, cat("vals"), cat("lhs"), cat("rhs"), cat("lb"), cat("ub"), cat("isint"),
                   name=f"{len(insts)} instances", x0=x0)
    return big, row_off, col_off


# ---------------------------------------------------------------- result files of the SCIP oracle
def scip_var_index(isint: np.ndarray, lb: np.ndarray, ub: np.ndarray) -> np.ndarray:
    """SCIP's problem index of each column when the columns are added to a SCIP problem in column order and the
    problem is then transformed, as a host program (the oracle driver, or a user building the problem) does.

    SCIP keeps a problem's variables grouped by type -- binaries, integers, continuous (prob.c: probProvidePos,
    probInsertVar) -- and makes room for an inserted variable by moving the first variable of each later group to
    that group's end, so within a group the index does not follow the column.  An integral column with bounds in
    {0, 1} is created as a binary variable (var.c: SCIPvarCreateOriginal's [0,1]-integer conversion).  The
    transformed problem adds the original variables in their index order (prob.c: SCIPprobTransform).  This index
    breaks ties in the order tightenBounds visits a row's entries (cons_linear.c: consdataCompVarProp)."""
    n = len(isint)
    kind = np.where(np.asarray(isint) != 0, 1, 2)
    kind[(kind == 1) & np.isin(lb, (0.0, 1.0)) & np.isin(ub, (0.0, 1.0))] = 0

    def insert(seq):
        arr = np.empty(n, dtype=np.int64)
        nb = ni = nv = 0
        for v in seq:
            pos = nv
            t = kind[v]
            if t != 2:
                cs = nb + ni
                if pos > cs:
                    arr[pos] = arr[cs]
                    pos = cs
                if t == 0 and pos > nb:
                    arr[pos] = arr[nb]
                    pos = nb
                if t == 0:
                    nb += 1
                else:
                    ni += 1
            arr[pos] = v
            nv += 1
        return arr

    orig = insert(range(n))
    trans = insert(orig)
    idx = np.empty(n, dtype=np.int32)
    idx[trans] = np.arange(n, dtype=np.int32)
    return idx


def scip_row_order(inst: "Instance", glb: np.ndarray, gub: np.ndarray,
                   varidx: Optional[np.ndarray] = None) -> np.ndarray:
    """The order SCIP sorts each row's entries into for propagation (cons_linear.c: consdataSort with
    consdataCompVarProp), on the global domain glb/gub: binaries first (integral columns with the domain inside
    [0, 1]) by decreasing |a|, then integers by decreasing |a| * (ub - lb), then continuous columns; ties by SCIP's
    problem index (varidx, see scip_var_index; default the column).  Keys are compared exactly, where SCIP treats
    values within 1e-9 as ties.  Returns CSR positions: order[p] for p in row i's range is the position of the
    row's entry that comes at p; inst.colidx[order], inst.vals[order] is the CSR in that order, which the batched
    node path's SCIP order (GBP_FLAG_SCIPORDER) expects."""
    col = inst.colidx
    vidx = np.arange(inst.n, dtype=np.int64) if varidx is None else np.asarray(varidx, dtype=np.int64)
    isint = np.asarray(inst.isint) != 0
    binary = isint & (glb >= 0.0) & (gub <= 1.0)
    group = np.where(binary[col], 0, np.where(isint[col], 1, 2))
    absa = np.abs(inst.vals)
    key = np.where(group == 0, -absa, np.where(group == 1, -np.abs(inst.vals * (gub[col] - glb[col])), 0.0))
    rows = np.repeat(np.arange(inst.m, dtype=np.int64), np.diff(inst.rowptr))
    return np.lexsort((vidx[col], key, group, rows)).astype(np.int32)


def pinned_node_base(inst: "Instance", path: str):
    """SCIP's root fixpoint and row orders of an instance from a compact file (tests/golden/make_golden.py,
    save_node_workload_base): returns (root lb, root ub, order) with order as scip_row_order returns it, or None
    when the file is absent or belongs to another instance."""
    import hashlib
    import os

    if not os.path.exists(path):
        return None
    with np.load(path) as f:
        z = dict(f)
    h = hashlib.sha256()
    for a in (inst.rowptr, inst.colidx, inst.vals, inst.lhs, inst.rhs, inst.lb, inst.ub, inst.isint):
        a = np.ascontiguousarray(a)
        h.update((a + 0.0 if a.dtype.kind == "f" else a).tobytes())
    if h.hexdigest() != str(z["instance_sha256"]):
        return None
    lb, ub = inst.lb.copy(), inst.ub.copy()
    lb[z["root_cols"]] = z["root_lb"]
    ub[z["root_cols"]] = z["root_ub"]
    order = scip_row_order(inst, inst.lb, inst.ub, scip_var_index(inst.isint, inst.lb, inst.ub))
    at = 0
    for i in z["order_rows"]:
        p0, p1 = int(inst.rowptr[i]), int(inst.rowptr[i + 1])
        order[p0:p1] = p0 + z["order_pos"][at:at + p1 - p0].astype(np.int64)
        at += p1 - p0
    return lb, ub, order


def in_order(inst: "Instance", order: np.ndarray) -> "Instance":
    """The instance with each row's entries rearranged by order (CSR positions, as scip_row_order returns)."""
    return Instance(inst.rowptr, inst.colidx[order], inst.vals[order], inst.lhs, inst.rhs, inst.lb, inst.ub,
                    inst.isint, name=inst.name)


def read_oracle_output(path: str):
    """Parse the oracle driver's output: (rootcutoff, rootlb, rootub, nodes) where nodes is a list of
    (cutoff, seconds, cols, lb, ub) with the columns whose bounds differ from the root fixpoint."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != b"LPOUT001":
        raise ValueError("bad oracle output")
    n, nnodes = struct.unpack_from("<2q", data, 8)
    off = 24
    rootcut = data[off]
    off += 1
    (roottime,) = struct.unpack_from("<d", data, off)
    off += 8
    rootlb = np.frombuffer(data, dtype="<f8", count=n, offset=off).copy()
    off += 8 * n
    rootub = np.frombuffer(data, dtype="<f8", count=n, offset=off).copy()
    off += 8 * n
    nodes = []
    rec = np.dtype([("col", "<i4"), ("lb", "<f8"), ("ub", "<f8")])
    for _ in range(nnodes):
        cut = data[off]
        off += 1
        (secs,) = struct.unpack_from("<d", data, off)
        off += 8
        (nch,) = struct.unpack_from("<i", data, off)
        off += 4
        r = np.frombuffer(data, dtype=rec, count=nch, offset=off)
        off += rec.itemsize * nch
        nodes.append((bool(cut), secs, r["col"].copy(), r["lb"].copy(), r["ub"].copy()))
    return bool(rootcut), rootlb, rootub, nodes
