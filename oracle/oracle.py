"""Test infrastructure only: ctypes binding of the C restatement (oracle/linprop_oracle.c) and runner of the
SCIP oracle driver (oracle/_ref/scip_oracle, present only where the SCIP sources were available to build it).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module, as the checker of
the CUDA path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liblinprop_oracle.so")
SCIP_ORACLE = os.path.join(HERE, "_ref", "scip_oracle")
# the SCIP source tree the Makefile's `ref` target compiles; unset means the sources are not available and the
# tests that read them skip
REFDIR = os.environ.get("REFDIR", "")

_P = ctypes.c_void_p


class Params(ctypes.Structure):
    _fields_ = [("infinity", ctypes.c_double), ("epsilon", ctypes.c_double), ("sumepsilon", ctypes.c_double),
                ("feastol", ctypes.c_double), ("hugeval", ctypes.c_double), ("boundstreps", ctypes.c_double),
                ("recompfac", ctypes.c_double), ("maxeasyactivitydelta", ctypes.c_double),
                ("maxrounds", ctypes.c_int32), ("flags", ctypes.c_int32)]


# Params.flags: constraints/linear/sortvars = FALSE (every entry of a row is tried)
FLAG_NOSORTVARS = 1
# Params.flags: ranged-row propagation (rangedRowPropagation, cons_linear.c:5715) without artificial constraints
FLAG_RANGEDROW = 2


class Log(ctypes.Structure):
    _fields_ = [("cap", ctypes.c_int64), ("n", ctypes.c_int64), ("col", _P), ("round", _P), ("lb", _P), ("ub", _P),
                ("rcap", ctypes.c_int64), ("rn", ctypes.c_int64), ("rrow", _P), ("rcol", _P), ("rround", _P)]


class Problem(ctypes.Structure):
    _fields_ = [("m", ctypes.c_int64), ("n", ctypes.c_int64), ("rowptr", _P), ("colidx", _P), ("vals", _P),
                ("lhs", _P), ("rhs", _P), ("isint", _P), ("colptr", _P), ("rowidx", _P), ("cvals", _P),
                ("varidx", _P)]


class Result(ctypes.Structure):
    _fields_ = [("cutoff", ctypes.c_int32), ("rounds", ctypes.c_int32), ("status", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("rows", ctypes.c_int64), ("nnz", ctypes.c_int64),
                ("candidates", ctypes.c_int64), ("changes", ctypes.c_int64), ("live_rows", ctypes.c_int64)]


def build() -> str:
    """Compile the C restatement (gcc, a few seconds)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.lpo_default_params.argtypes = [ctypes.POINTER(Params)]
        L.lpo_row_activities.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(Params), _P, _P, _P,
                                         ctypes.c_int64, _P, _P]
        L.lpo_propagate.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(Params), _P, _P, ctypes.c_int64, _P,
                                    _P, _P, _P, _P, ctypes.POINTER(Result)]
        L.lpo_propagate_logged.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(Params), _P, _P, ctypes.c_int64,
                                           _P, _P, _P, _P, _P, ctypes.POINTER(Result), ctypes.POINTER(Log)]
        L.lpo_propagate_nodes.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(Params), _P, _P, ctypes.c_int64,
                                          _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.POINTER(Result)]
        L.lpo_propagate_seq.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(Params), _P, _P, _P,
                                        ctypes.POINTER(Result)]
        L.lpo_propagate_nodes_seq.argtypes = L.lpo_propagate_nodes.argtypes
        L.lpo_seq_state_bytes.argtypes = [ctypes.c_int64]
        L.lpo_seq_state_bytes.restype = ctypes.c_size_t
        L.lpo_propagate_seq_states.argtypes = L.lpo_propagate_seq.argtypes + [_P]
        L.lpo_propagate_nodes_seq_from.argtypes = L.lpo_propagate_nodes.argtypes + [_P]
        L.lpo_seq_states_deleted.argtypes = [_P, ctypes.c_int64, _P]
        L.lpo_root_deleted_rows.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(Params), _P, _P, _P]
        _lib = L
    return _lib


def params(maxeasy: float = 0.0, maxrounds: int = 0, sortvars: bool = True, ranged: bool = False) -> Params:
    p = Params()
    lib().lpo_default_params(ctypes.byref(p))
    p.maxeasyactivitydelta = maxeasy
    p.maxrounds = maxrounds
    p.flags = (0 if sortvars else FLAG_NOSORTVARS) | (FLAG_RANGEDROW if ranged else 0)
    return p


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Oracle:
    """Keeps an instance (and its CSC copy) alive for repeated oracle calls."""

    def __init__(self, inst, varidx=None):
        """varidx: SCIP's problem index of each column (instances.scip_var_index), the tie-break of the order SCIP
        sorts rows into; None uses the column index."""
        self.inst = inst
        self.varidx = None if varidx is None else np.ascontiguousarray(varidx, dtype=np.int32)
        self.rowptr = np.ascontiguousarray(inst.rowptr, dtype=np.int64)
        self.colidx = np.ascontiguousarray(inst.colidx, dtype=np.int32)
        self.vals = np.ascontiguousarray(inst.vals, dtype=np.float64)
        self.lhs = np.ascontiguousarray(inst.lhs, dtype=np.float64)
        self.rhs = np.ascontiguousarray(inst.rhs, dtype=np.float64)
        self.isint = np.ascontiguousarray(inst.isint, dtype=np.int8)
        cp, ri, cv = inst.csc()
        self.colptr, self.rowidx, self.cvals = cp, ri, cv
        self.prob = Problem(inst.m, inst.n, _ptr(self.rowptr), _ptr(self.colidx), _ptr(self.vals), _ptr(self.lhs),
                            _ptr(self.rhs), _ptr(self.isint), _ptr(self.colptr), _ptr(self.rowidx), _ptr(self.cvals),
                            _ptr(self.varidx))

    def activities(self, lb, ub, rows=None, par=None):
        par = par or params()
        lb = np.ascontiguousarray(lb, dtype=np.float64)
        ub = np.ascontiguousarray(ub, dtype=np.float64)
        nr = self.inst.m if rows is None else len(rows)
        r = None if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
        act = np.zeros((nr, 4))
        cnt = np.zeros((nr, 8), dtype=np.int32)
        lib().lpo_row_activities(ctypes.byref(self.prob), ctypes.byref(par), _ptr(lb), _ptr(ub), _ptr(r), nr,
                                 _ptr(act), _ptr(cnt))
        return act, cnt

    def propagate(self, lb, ub, par=None, seed=None, glob=None):
        """Fixpoint from all rows (seed None) or from (cols, oldlb, oldub) changes; returns (lb, ub, Result).
        glob: (glb, gub), the global domain for the binary test; None = the current bounds (root)."""
        par = par or params()
        lb = np.array(lb, dtype=np.float64)
        ub = np.array(ub, dtype=np.float64)
        res = Result()
        glb = gub = None
        if glob is not None:
            glb = np.ascontiguousarray(glob[0], dtype=np.float64)
            gub = np.ascontiguousarray(glob[1], dtype=np.float64)
        if seed is None:
            lib().lpo_propagate(ctypes.byref(self.prob), ctypes.byref(par), _ptr(lb), _ptr(ub), 0, None, None, None,
                                _ptr(glb), _ptr(gub), ctypes.byref(res))
        else:
            cols, olb, oub = (np.ascontiguousarray(x) for x in seed)
            cols = cols.astype(np.int32)
            olb = olb.astype(np.float64)
            oub = oub.astype(np.float64)
            lib().lpo_propagate(ctypes.byref(self.prob), ctypes.byref(par), _ptr(lb), _ptr(ub), len(cols), _ptr(cols),
                                _ptr(olb), _ptr(oub), _ptr(glb), _ptr(gub), ctypes.byref(res))
        return lb, ub, res

    def propagate_logged(self, lb, ub, par=None, seed=None, glob=None, cap=None):
        """propagate() plus the change log sorted by (round, column): returns (lb, ub, Result, (col, round, lb, ub))."""
        par = par or params()
        lb = np.array(lb, dtype=np.float64)
        ub = np.array(ub, dtype=np.float64)
        cap = cap or 8 * self.inst.n + 1024
        col, rnd = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
        llb, lub = np.zeros(cap), np.zeros(cap)
        rrow, rcol, rrnd = np.zeros(cap, np.int32), np.zeros(cap, np.int32), np.zeros(cap, np.int32)
        log = Log(cap, 0, _ptr(col), _ptr(rnd), _ptr(llb), _ptr(lub), cap, 0, _ptr(rrow), _ptr(rcol), _ptr(rrnd))
        res = Result()
        glb = gub = None
        if glob is not None:
            glb = np.ascontiguousarray(glob[0], dtype=np.float64)
            gub = np.ascontiguousarray(glob[1], dtype=np.float64)
        if seed is None:
            args = (0, None, None, None)
        else:
            cols, olb, oub = (np.ascontiguousarray(x) for x in seed)
            cols, olb, oub = cols.astype(np.int32), olb.astype(np.float64), oub.astype(np.float64)
            args = (len(cols), _ptr(cols), _ptr(olb), _ptr(oub))
        lib().lpo_propagate_logged(ctypes.byref(self.prob), ctypes.byref(par), _ptr(lb), _ptr(ub), *args, _ptr(glb),
                                   _ptr(gub), ctypes.byref(res), ctypes.byref(log))
        if log.n > cap or log.rn > cap:
            raise MemoryError("oracle change log capacity exceeded")
        n = log.n
        o = np.lexsort((col[:n], rnd[:n]))
        r = log.rn
        q = np.lexsort((rrow[:r], rcol[:r], rrnd[:r]))
        # the ranged-row records, sorted by (round, column, row)
        self.last_ranged = (rrnd[:r][q], rcol[:r][q], rrow[:r][q])
        return lb, ub, res, (col[:n][o], rnd[:n][o], llb[:n][o], lub[:n][o])

    def propagate_seq(self, lb, ub, par=None, states=False):
        """Root fixpoint in SCIP's own order (lpo_propagate_seq); returns (lb, ub, Result, order) where order[p]
        for p in row i's CSR range is the CSR position of the row's entries in the order SCIP holds them at the end.
        states: also return the root's final row states (opaque bytes for propagate_nodes(root_states=...))."""
        par = par or params()
        lb = np.array(lb, dtype=np.float64)
        ub = np.array(ub, dtype=np.float64)
        order = np.zeros(max(1, self.inst.nnz), dtype=np.int32)
        res = Result()
        st = np.zeros(lib().lpo_seq_state_bytes(self.inst.m), dtype=np.uint8) if states else None
        if lib().lpo_propagate_seq_states(ctypes.byref(self.prob), ctypes.byref(par), _ptr(lb), _ptr(ub),
                                          _ptr(order), ctypes.byref(res), _ptr(st)) != 0:
            raise MemoryError("oracle allocation failed")
        if states:
            return lb, ub, res, order[:self.inst.nnz], st
        return lb, ub, res, order[:self.inst.nnz]

    def states_deleted_rows(self, states):
        """The rows the root restatement deleted, from the row states of propagate_seq(..., states=True)."""
        out = np.zeros(self.inst.m, dtype=np.uint8)
        lib().lpo_seq_states_deleted(_ptr(states), self.inst.m, _ptr(out))
        return out.astype(bool)

    def root_deleted_rows(self, lb, ub, par=None):
        """Rows redundant under lb/ub: the rows SCIP's root deletes (lpo_root_deleted_rows)."""
        par = par or params()
        lb = np.ascontiguousarray(lb, dtype=np.float64)
        ub = np.ascontiguousarray(ub, dtype=np.float64)
        out = np.zeros(self.inst.m, dtype=np.uint8)
        lib().lpo_root_deleted_rows(ctypes.byref(self.prob), ctypes.byref(par), _ptr(lb), _ptr(ub), _ptr(out))
        return out.astype(bool)

    def propagate_nodes(self, baselb, baseub, nodes, par=None, cap=4096, nthreads=1, seq=False, root_states=None):
        """Node batch; returns dict with cutoff [N], rounds [N], n [N], col/lb/ub [N, cap] and totals.
        seq: SCIP's own order (lpo_propagate_nodes_seq; each row's entries in storage order are taken as the order
        SCIP holds the row in) instead of rounds.  root_states (seq only): the row states of propagate_seq(...,
        states=True) on the same rows, which each node's rows start from as SCIP's do (default: afresh)."""
        par = par or params()
        N = nodes.nnodes
        baselb = np.ascontiguousarray(baselb, dtype=np.float64)
        baseub = np.ascontiguousarray(baseub, dtype=np.float64)
        ptr = np.ascontiguousarray(nodes.ptr, dtype=np.int64)
        col = np.ascontiguousarray(nodes.col, dtype=np.int32)
        nlb = np.ascontiguousarray(nodes.lb, dtype=np.float64)
        nub = np.ascontiguousarray(nodes.ub, dtype=np.float64)
        out = dict(cutoff=np.zeros(N, dtype=np.int8), rounds=np.zeros(N, dtype=np.int32),
                   n=np.zeros(N, dtype=np.int32), col=np.zeros((N, cap), dtype=np.int32),
                   lb=np.zeros((N, cap)), ub=np.zeros((N, cap)))
        tot = Result()
        args = (ctypes.byref(self.prob), ctypes.byref(par), _ptr(baselb), _ptr(baseub), N,
                _ptr(ptr), _ptr(col), _ptr(nlb), _ptr(nub), _ptr(out["cutoff"]), _ptr(out["rounds"]), _ptr(out["n"]),
                _ptr(out["col"]), _ptr(out["lb"]), _ptr(out["ub"]), cap, nthreads, ctypes.byref(tot))
        if root_states is not None:
            if not seq or len(root_states) != lib().lpo_seq_state_bytes(self.inst.m):
                raise ValueError("root_states: the row states of propagate_seq on the same rows, seq mode only")
            rc = lib().lpo_propagate_nodes_seq_from(*args, _ptr(root_states))
        else:
            rc = (lib().lpo_propagate_nodes_seq if seq else lib().lpo_propagate_nodes)(*args)
        if rc != 0:
            raise MemoryError("oracle node batch failed")
        out["total"] = tot
        return out


def _read_order(inst, path):
    """SCIP's row order file (scip_driver.c --order) as CSR positions into inst, and the rows SCIP deleted."""
    raw = np.fromfile(path, dtype=np.int32)
    m = int(raw[:2].view(np.int64)[0])
    assert m == inst.m
    order = np.arange(inst.nnz, dtype=np.int32)
    deleted = np.zeros(m, dtype=bool)
    off = 2
    for i in range(m):
        ln = int(raw[off])
        off += 1
        if ln < 0:
            deleted[i] = True
            continue
        cols = raw[off:off + ln]
        off += ln
        p0, p1 = inst.rowptr[i], inst.rowptr[i + 1]
        pos = {int(c): p for p, c in zip(range(p0, p1), inst.colidx[p0:p1])}
        order[p0:p1] = [pos[int(c)] for c in cols]
    return order, deleted


def run_scip(inst, nodes=None, easy=False, repeat=1, workdir=None, ranged=False, sortvars=True, fresh=False,
             order=False, unmark=False):
    """Run SCIP itself (oracle/_ref/scip_oracle) on the instance; returns the parsed output of
    scip_gb300.instances.read_oracle_output, plus (with order=True) SCIP's row order after the root as a CSR
    position array (order[p] for p in row i's range: the position of the row's k-th entry; rows deleted at the
    root keep their storage order) and the mask of the rows the root deleted.  fresh: every node from a newly
    transformed problem (scip_driver.c --fresh); unmark: nodes in one probing session, each without the marks a
    cut-off node left (--unmark)."""
    from scip_gb300.instances import read_oracle_output

    if not os.path.exists(SCIP_ORACLE):
        raise FileNotFoundError("SCIP oracle driver not built (make -C oracle ref needs the SCIP sources)")
    with tempfile.TemporaryDirectory(dir=workdir) as d:
        ip = os.path.join(d, "inst.bin")
        op = os.path.join(d, "out.bin")
        inst.write(ip)
        npth = "-"
        if nodes is not None:
            npth = os.path.join(d, "nodes.bin")
            nodes.write(npth)
        cmd = ([SCIP_ORACLE, ip, npth, op] + (["--easy"] if easy else []) + (["--ranged"] if ranged else [])
               + ([] if sortvars else ["--nosort"]) + ["--repeat", str(repeat)] + (["--fresh"] if fresh else [])
               + (["--order", os.path.join(d, "order.bin")] if order else []) + (["--unmark"] if unmark else []))
        subprocess.run(cmd, check=True, capture_output=True)
        if order:
            return read_oracle_output(op) + _read_order(inst, os.path.join(d, "order.bin"))
        return read_oracle_output(op)
