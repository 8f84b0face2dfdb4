"""Python binding of libgbp's C ABI (include/gbp.h) through ctypes.

This is the host-side mirror of the propagator interface for Python callers (tests, bench, the serving
loop).  Every call goes to the CUDA library; there is no CPU fallback: if libgbp.so is missing or no
sm_103 GPU is present, construction raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from .build import LIBGBP

_P = ctypes.c_void_p

GBP_OK = 0
GBP_ERR_INVALID = -1
GBP_ERR_CUDA = -2
GBP_ERR_NOMEM = -3
GBP_ERR_NODEVICE = -4
GBP_ERR_LIMIT = -5
GBP_ERR_OVERFLOW = -6
GBP_ERR_STATE = -7
GBP_ERR_TOO_LARGE = -8
GBP_ERR_BUSY = -9
GBP_FLAG_HOSTLOOP = 1
GBP_FLAG_NOSORTVARS = 2
GBP_FLAG_RANGEDROW = 4
GBP_FLAG_SCIPORDER = 8

# every symbol include/gbp.h declares (checked by the CPU test suite)
EXPORTS = ["gbp_version", "gbp_error_string", "gbp_last_error", "gbp_create", "gbp_destroy", "gbp_default_params",
           "gbp_set_params", "gbp_get_stream", "gbp_upload_problem", "gbp_propagate", "gbp_propagate_device",
           "gbp_row_activities", "gbp_propagate_nodes", "gbp_propagate_nodes_device", "gbp_set_batch_shape",
           "gbp_propagate_nodes_noalloc", "gbp_upload_instances", "gbp_propagate_instances",
           "gbp_propagate_instances_device", "gbp_set_global_bounds", "gbp_set_change_log", "gbp_get_change_log",
           "gbp_upload_instance_list", "gbp_get_ranged_log", "gbp_set_bounds", "gbp_propagate_changes",
           "gbp_server_create", "gbp_server_submit", "gbp_server_submit_instance", "gbp_server_poll", "gbp_server_stats",
           "gbp_server_destroy"]


class GbpParams(ctypes.Structure):
    _fields_ = [("infinity", ctypes.c_double), ("epsilon", ctypes.c_double), ("sumepsilon", ctypes.c_double),
                ("feastol", ctypes.c_double), ("hugeval", ctypes.c_double), ("boundstreps", ctypes.c_double),
                ("recompfac", ctypes.c_double), ("maxeasyactivitydelta", ctypes.c_double),
                ("maxrounds", ctypes.c_int32), ("flags", ctypes.c_int32)]


class GbpResult(ctypes.Structure):
    _fields_ = [("cutoff", ctypes.c_int32), ("rounds", ctypes.c_int32), ("status", ctypes.c_int32),
                ("launches", ctypes.c_int32), ("rows", ctypes.c_int64), ("nnz", ctypes.c_int64),
                ("candidates", ctypes.c_int64), ("changes", ctypes.c_int64), ("live_rows", ctypes.c_int64),
                ("kernel_ms", ctypes.c_double)]

    def asdict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GbpError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gbp error {code}: {msg}")
        self.code = code


_lib = None


def load_library(path: Optional[str] = None):
    """Load libgbp.so (raises FileNotFoundError if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIBGBP
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} missing: build it with scip_gb300.build.build_libgbp()")
    L = ctypes.CDLL(p)
    L.gbp_version.restype = ctypes.c_int
    L.gbp_error_string.restype = ctypes.c_char_p
    L.gbp_error_string.argtypes = [ctypes.c_int]
    L.gbp_last_error.restype = ctypes.c_char_p
    L.gbp_last_error.argtypes = [_P]
    L.gbp_create.argtypes = [ctypes.POINTER(_P), ctypes.c_int, _P]
    L.gbp_destroy.argtypes = [_P]
    L.gbp_default_params.argtypes = [ctypes.POINTER(GbpParams)]
    L.gbp_default_params.restype = None
    L.gbp_set_params.argtypes = [_P, ctypes.POINTER(GbpParams)]
    L.gbp_get_stream.argtypes = [_P, ctypes.POINTER(_P)]
    L.gbp_upload_problem.argtypes = [_P, ctypes.c_int64, ctypes.c_int64, _P, _P, _P, _P, _P, _P]
    L.gbp_propagate.argtypes = [_P, _P, _P, ctypes.c_int64, _P, _P, _P, _P, ctypes.POINTER(GbpResult)]
    L.gbp_propagate_device.argtypes = L.gbp_propagate.argtypes
    L.gbp_row_activities.argtypes = [_P, _P, _P, _P, _P]
    L.gbp_set_bounds.argtypes = [_P, _P, _P]
    L.gbp_propagate_changes.argtypes = [_P, ctypes.c_int64, _P, _P, _P, _P, _P, ctypes.c_int64,
                                        ctypes.POINTER(ctypes.c_int64), _P, _P, _P, ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(GbpResult)]
    L.gbp_set_global_bounds.argtypes = [_P, _P, _P]
    L.gbp_set_change_log.argtypes = [_P, ctypes.c_int64]
    L.gbp_get_change_log.argtypes = [_P, ctypes.c_int64, _P, _P, _P, _P, ctypes.POINTER(ctypes.c_int64)]
    L.gbp_get_ranged_log.argtypes = [_P, ctypes.c_int64, _P, _P, _P, ctypes.POINTER(ctypes.c_int64)]
    L.gbp_propagate_nodes.argtypes = [_P, _P, _P, ctypes.c_int64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                      ctypes.c_int64, ctypes.POINTER(GbpResult)]
    L.gbp_propagate_nodes_device.argtypes = L.gbp_propagate_nodes.argtypes
    L.gbp_set_batch_shape.argtypes = [_P, ctypes.c_int32, ctypes.c_int32]
    L.gbp_upload_instances.argtypes = [_P, ctypes.c_int64] + [_P] * 8
    L.gbp_upload_instance_list.argtypes = [_P, ctypes.c_int64] + [_P] * 8
    L.gbp_propagate_instances.argtypes = [_P, _P, _P, _P, ctypes.POINTER(GbpResult)]
    L.gbp_propagate_instances_device.argtypes = L.gbp_propagate_instances.argtypes
    L.gbp_propagate_nodes_noalloc.argtypes = ([ctypes.c_int64, ctypes.c_int64] + [_P] * 11 + [ctypes.c_int64]
                                              + [_P] * 11 + [ctypes.c_int64, ctypes.POINTER(GbpParams), _P,
                                                              ctypes.POINTER(GbpResult)])
    declare_server(L)
    if path is None:
        _lib = L
    return L


def declare_server(L):
    """Argument types of the serving loop's calls (gbp_server_*) on a loaded library."""
    L.gbp_error_string.restype = ctypes.c_char_p
    L.gbp_error_string.argtypes = [ctypes.c_int]
    L.gbp_server_create.argtypes = [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                    ctypes.c_int64, ctypes.POINTER(GbpParams), ctypes.c_int64, ctypes.c_int64] + [_P] * 8
    L.gbp_server_submit.argtypes = [_P, ctypes.c_int64, _P, _P, _P, ctypes.POINTER(ctypes.c_int64)]
    L.gbp_server_submit_instance.argtypes = [_P, ctypes.c_int64, ctypes.c_int64] + [_P] * 8 + [
        ctypes.POINTER(ctypes.c_int64)]
    L.gbp_server_poll.argtypes = [_P, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(ctypes.c_int32), ctypes.c_int64,
                                  ctypes.POINTER(ctypes.c_int64), _P, _P, _P, ctypes.POINTER(ctypes.c_int64),
                                  ctypes.POINTER(ctypes.c_int64)]
    L.gbp_server_stats.argtypes = [_P] + [ctypes.POINTER(ctypes.c_int64)] * 4
    L.gbp_server_destroy.argtypes = [_P]


def default_params(maxeasy: Optional[float] = None, maxrounds: int = 0, sortvars: bool = True,
                   ranged: bool = False, scip_order: bool = False) -> GbpParams:
    """gbp_default_params with the given changes; scip_order: batched nodes in SCIP's own order
    (GBP_FLAG_SCIPORDER; rows must be uploaded in the order SCIP holds them, see instances.scip_row_order)."""
    p = GbpParams()
    load_library().gbp_default_params(ctypes.byref(p))
    if maxeasy is not None:
        p.maxeasyactivitydelta = maxeasy
    p.maxrounds = maxrounds
    if not sortvars:
        p.flags |= GBP_FLAG_NOSORTVARS
    if ranged:
        p.flags |= GBP_FLAG_RANGEDROW
    if scip_order:
        p.flags |= GBP_FLAG_SCIPORDER
    return p


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)
    if hasattr(a, "data_ptr"):  # torch tensor on the device
        return ctypes.c_void_p(a.data_ptr())
    return a


@dataclass
class NodeResults:
    cutoff: np.ndarray
    rounds: np.ndarray
    off: np.ndarray
    n: np.ndarray
    col: np.ndarray
    lb: np.ndarray
    ub: np.ndarray
    result: GbpResult

    def node(self, k):
        o, c = int(self.off[k]), int(self.n[k])
        return self.col[o:o + c], self.lb[o:o + c], self.ub[o:o + c]


class Propagator:
    """One GPU context with one uploaded set of rows (the state a SCIP propagator keeps between calls)."""

    def __init__(self, device: int = 0, stream=None, params: Optional[GbpParams] = None):
        self.L = load_library()
        h = _P()
        rc = self.L.gbp_create(ctypes.byref(h), device, _ptr(stream) if stream is not None else None)
        if rc != GBP_OK:
            raise GbpError(rc, self.L.gbp_error_string(rc).decode())
        self.h = h
        self.n = 0
        self.m = 0
        if params is not None:
            self.set_params(params)

    def close(self):
        if getattr(self, "h", None):
            self.L.gbp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, allow=()):
        if rc != GBP_OK and rc not in allow:
            raise GbpError(rc, f"{self.L.gbp_error_string(rc).decode()}: {self.L.gbp_last_error(self.h).decode()}")
        return rc

    def set_params(self, p: GbpParams):
        self._check(self.L.gbp_set_params(self.h, ctypes.byref(p)))

    def set_batch_shape(self, threads_per_node: int = 128, ctas_per_sm: int = 0):
        self._check(self.L.gbp_set_batch_shape(self.h, threads_per_node, ctas_per_sm))

    def stream(self):
        s = _P()
        self._check(self.L.gbp_get_stream(self.h, ctypes.byref(s)))
        return s.value

    def upload(self, inst):
        self._keep = [np.ascontiguousarray(inst.rowptr, dtype=np.int64),
                      np.ascontiguousarray(inst.colidx, dtype=np.int32),
                      np.ascontiguousarray(inst.vals, dtype=np.float64),
                      np.ascontiguousarray(inst.lhs, dtype=np.float64),
                      np.ascontiguousarray(inst.rhs, dtype=np.float64),
                      np.ascontiguousarray(inst.isint, dtype=np.int8)]
        rp, ci, va, lh, rh, ii = self._keep
        self._check(self.L.gbp_upload_problem(self.h, inst.m, inst.n, _ptr(rp), _ptr(ci), _ptr(va), _ptr(lh),
                                              _ptr(rh), _ptr(ii)))
        self._keep = None
        self.m, self.n = inst.m, inst.n

    def set_bounds(self, lb, ub):
        """the context's device copy of the bounds, for propagate_changes"""
        lb = np.ascontiguousarray(lb, dtype=np.float64)
        ub = np.ascontiguousarray(ub, dtype=np.float64)
        self._check(self.L.gbp_set_bounds(self.h, _ptr(lb), _ptr(ub)))

    def propagate_changes(self, cols, newlb, newub, cap: Optional[int] = None, seed=None):
        """Sparse plain call: the listed columns take the given bounds on the device copy, propagation runs from
        them (tightenings relative to seed = (seedlb, seedub) per change, else to the device's previous bounds).
        Returns (cutoff, moved columns sorted, their lb, their ub, GbpResult)."""
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        newlb = np.ascontiguousarray(newlb, dtype=np.float64)
        newub = np.ascontiguousarray(newub, dtype=np.float64)
        slb = sub = None
        if seed is not None:
            slb = np.ascontiguousarray(seed[0], dtype=np.float64)
            sub = np.ascontiguousarray(seed[1], dtype=np.float64)
        cap = self.n if cap is None else cap
        if getattr(self, "_chg_out", None) is None or len(self._chg_out[0]) < cap:  # reused between calls
            self._chg_out = (np.zeros(cap, np.int32), np.zeros(cap), np.zeros(cap))
        oc, ol, ou = self._chg_out
        nout, cut, res = ctypes.c_int64(0), ctypes.c_int32(0), GbpResult()
        rc = self.L.gbp_propagate_changes(self.h, len(cols), _ptr(cols), _ptr(newlb), _ptr(newub), _ptr(slb),
                                          _ptr(sub), cap, ctypes.byref(nout), _ptr(oc), _ptr(ol), _ptr(ou),
                                          ctypes.byref(cut), ctypes.byref(res))
        self._check(rc, allow=(GBP_ERR_LIMIT,))
        k = nout.value
        return bool(cut.value), oc[:k].copy(), ol[:k].copy(), ou[:k].copy(), res

    def propagate(self, lb, ub, seed=None):
        """Host arrays; returns (lb, ub, cutoff, GbpResult).  seed = (cols, oldlb, oldub) or None (all rows)."""
        lb = np.array(lb, dtype=np.float64)
        ub = np.array(ub, dtype=np.float64)
        cut = ctypes.c_int32(0)
        res = GbpResult()
        if seed is None:
            rc = self.L.gbp_propagate(self.h, _ptr(lb), _ptr(ub), -1, None, None, None, ctypes.byref(cut),
                                      ctypes.byref(res))
        else:
            cols = np.ascontiguousarray(seed[0], dtype=np.int32)
            olb = np.ascontiguousarray(seed[1], dtype=np.float64)
            oub = np.ascontiguousarray(seed[2], dtype=np.float64)
            rc = self.L.gbp_propagate(self.h, _ptr(lb), _ptr(ub), len(cols), _ptr(cols), _ptr(olb), _ptr(oub),
                                      ctypes.byref(cut), ctypes.byref(res))
        self._check(rc, allow=(GBP_ERR_LIMIT,))
        return lb, ub, bool(cut.value), res

    def upload_instances(self, insts, concat=False):
        """Upload several independent instances as one block-diagonal problem; returns (row_off, col_off).

        By default each instance's arrays go to the device as they are (gbp_upload_instance_list); concat=True
        concatenates them on the host first (gbp_upload_instances)."""
        from .instances import concat_instances

        k = len(insts)
        if concat:
            big, row_off, col_off = concat_instances(insts)
            keep = [np.ascontiguousarray(a) for a in (row_off, col_off, big.rowptr, big.colidx, big.vals, big.lhs,
                                                       big.rhs, big.isint)]
            self._check(self.L.gbp_upload_instances(self.h, k, *[_ptr(a) for a in keep]))
        else:
            row_off = np.zeros(k + 1, dtype=np.int64)
            col_off = np.zeros(k + 1, dtype=np.int64)
            np.cumsum([i.m for i in insts], out=row_off[1:])
            np.cumsum([i.n for i in insts], out=col_off[1:])
            mk = np.ascontiguousarray(np.diff(row_off))
            nk = np.ascontiguousarray(np.diff(col_off))
            fields = (("rowptr", np.int64), ("colidx", np.int32), ("vals", np.float64), ("lhs", np.float64),
                      ("rhs", np.float64), ("isint", np.int8))
            keep = [[np.ascontiguousarray(getattr(i, f), dtype=t) for i in insts] for f, t in fields]
            tables = [(ctypes.c_void_p * k)(*[a.ctypes.data for a in arrs]) for arrs in keep]
            self._check(self.L.gbp_upload_instance_list(self.h, k, _ptr(mk), _ptr(nk),
                                                        *[ctypes.cast(t, ctypes.c_void_p) for t in tables]))
        self._inst_off = (row_off, col_off)
        self.m, self.n = int(row_off[-1]), int(col_off[-1])
        return row_off, col_off

    def propagate_instances(self, lb, ub):
        """Host bound vectors of the block-diagonal problem; returns (lb, ub, cutoff per instance, GbpResult)."""
        lb = np.array(lb, dtype=np.float64)
        ub = np.array(ub, dtype=np.float64)
        cut = np.zeros(len(self._inst_off[0]) - 1, dtype=np.int8)
        res = GbpResult()
        self._check(self.L.gbp_propagate_instances(self.h, _ptr(lb), _ptr(ub), _ptr(cut), ctypes.byref(res)),
                    allow=(GBP_ERR_LIMIT,))
        return lb, ub, cut, res

    def propagate_instances_device(self, lb, ub, cut):
        """Device tensors (float64 bounds, int8 cutoff per instance); returns GbpResult."""
        res = GbpResult()
        self._check(self.L.gbp_propagate_instances_device(self.h, _ptr(lb), _ptr(ub), _ptr(cut), ctypes.byref(res)),
                    allow=(GBP_ERR_LIMIT,))
        return res

    def propagate_device(self, lb, ub):
        """Device bound vectors (torch float64 tensors), all rows seeded; returns (cutoff, GbpResult)."""
        cut = ctypes.c_int32(0)
        res = GbpResult()
        rc = self.L.gbp_propagate_device(self.h, _ptr(lb), _ptr(ub), -1, None, None, None, ctypes.byref(cut),
                                         ctypes.byref(res))
        self._check(rc, allow=(GBP_ERR_LIMIT,))
        return bool(cut.value), res

    def activities(self, lb, ub):
        lb = np.ascontiguousarray(lb, dtype=np.float64)
        ub = np.ascontiguousarray(ub, dtype=np.float64)
        act = np.zeros((self.m, 4))
        cnt = np.zeros((self.m, 8), dtype=np.int32)
        self._check(self.L.gbp_row_activities(self.h, _ptr(lb), _ptr(ub), _ptr(act), _ptr(cnt)))
        return act, cnt

    def set_change_log(self, capacity: int):
        """Record every accepted bound change of later plain-path calls (capacity entries; 0: off)."""
        self._check(self.L.gbp_set_change_log(self.h, int(capacity)))

    def change_log(self, cap: Optional[int] = None):
        """The last call's change log sorted by (round, column): (col, round, lb, ub) arrays."""
        n = ctypes.c_int64(0)
        if cap is None:
            self._check(self.L.gbp_get_change_log(self.h, 0, None, None, None, None, ctypes.byref(n)),
                        allow=(GBP_ERR_OVERFLOW,))
            cap = n.value
        col = np.zeros(cap, np.int32)
        rnd = np.zeros(cap, np.int32)
        lb = np.zeros(cap)
        ub = np.zeros(cap)
        self._check(self.L.gbp_get_change_log(self.h, cap, _ptr(col), _ptr(rnd), _ptr(lb), _ptr(ub), ctypes.byref(n)))
        return col[:n.value], rnd[:n.value], lb[:n.value], ub[:n.value]

    def ranged_log(self, cap: Optional[int] = None):
        """The last call's ranged-row records sorted by (round, column, row): (round, col, row) arrays."""
        n = ctypes.c_int64(0)
        if cap is None:
            self._check(self.L.gbp_get_ranged_log(self.h, 0, None, None, None, ctypes.byref(n)),
                        allow=(GBP_ERR_OVERFLOW,))
            cap = n.value
        rnd = np.zeros(cap, np.int32)
        col = np.zeros(cap, np.int32)
        row = np.zeros(cap, np.int32)
        self._check(self.L.gbp_get_ranged_log(self.h, cap, _ptr(rnd), _ptr(col), _ptr(row), ctypes.byref(n)))
        return rnd[:n.value], col[:n.value], row[:n.value]

    def set_global_bounds(self, glb=None, gub=None):
        """Global domain for the binary test of later propagate() calls (None: the propagated bounds, as at the
        root)."""
        if glb is None:
            self._check(self.L.gbp_set_global_bounds(self.h, None, None))
            return
        glb = np.ascontiguousarray(glb, dtype=np.float64)
        gub = np.ascontiguousarray(gub, dtype=np.float64)
        self._check(self.L.gbp_set_global_bounds(self.h, _ptr(glb), _ptr(gub)))

    @staticmethod
    def node_outputs(nnodes: int, out_cap: int, alloc=np.empty) -> NodeResults:
        """Output arrays for propagate_nodes (reusable across calls; alloc may return pinned arrays)."""
        return NodeResults(alloc(nnodes, np.int8), alloc(nnodes, np.int32), alloc(nnodes, np.int64),
                           alloc(nnodes, np.int32), alloc(out_cap, np.int32), alloc(out_cap, np.float64),
                           alloc(out_cap, np.float64), GbpResult())

    def propagate_nodes(self, baselb, baseub, nodes, out_cap: Optional[int] = None,
                        out: Optional[NodeResults] = None) -> NodeResults:
        """Host arrays: nodes is an instances.NodeBatch.  Returns packed per-node results (in `out` when given: arrays
        from node_outputs, of at least nodes.nnodes entries and out_cap packed entries)."""
        N = nodes.nnodes
        if out_cap is None:
            out_cap = max(1024, 64 * N) if out is None else len(out.col)
        baselb = np.ascontiguousarray(baselb, dtype=np.float64)
        baseub = np.ascontiguousarray(baseub, dtype=np.float64)
        ptr = np.ascontiguousarray(nodes.ptr, dtype=np.int64)
        col = np.ascontiguousarray(nodes.col, dtype=np.int32)
        nlb = np.ascontiguousarray(nodes.lb, dtype=np.float64)
        nub = np.ascontiguousarray(nodes.ub, dtype=np.float64)
        if out is None:
            r = self.node_outputs(N, out_cap)
        else:
            if len(out.cutoff) < N or len(out.col) < out_cap:
                raise ValueError("output arrays too small")
            r = out
            r.result = GbpResult()
        rc = self.L.gbp_propagate_nodes(self.h, _ptr(baselb), _ptr(baseub), N, _ptr(ptr), _ptr(col), _ptr(nlb),
                                        _ptr(nub), _ptr(r.cutoff), _ptr(r.rounds), _ptr(r.off), _ptr(r.n),
                                        _ptr(r.col), _ptr(r.lb), _ptr(r.ub), out_cap, ctypes.byref(r.result))
        self._check(rc, allow=(GBP_ERR_LIMIT,))
        return r

    def propagate_nodes_device(self, baselb, baseub, nnodes, ptr, col, nlb, nub, out, out_cap):
        """All arguments device tensors; out = dict(cutoff, rounds, off, n, col, lb, ub).  Returns GbpResult."""
        res = GbpResult()
        rc = self.L.gbp_propagate_nodes_device(self.h, _ptr(baselb), _ptr(baseub), nnodes, _ptr(ptr), _ptr(col),
                                               _ptr(nlb), _ptr(nub), _ptr(out["cutoff"]), _ptr(out["rounds"]),
                                               _ptr(out["off"]), _ptr(out["n"]), _ptr(out["col"]), _ptr(out["lb"]),
                                               _ptr(out["ub"]), out_cap, ctypes.byref(res))
        self._check(rc, allow=(GBP_ERR_LIMIT,))
        return res


class Server:
    """libgbp's serving loop (gbp_server_*): node requests against one resident problem and its root bounds, merged
    by worker threads inside libgbp into batched launches."""

    def __init__(self, inst, rootlb, rootub, params: Optional[GbpParams] = None, device: int = 0, workers: int = 2,
                 max_batch: int = 4096, hbm_cap: int = 0, inst_workers: int = 0, lib=None):
        """lib: a library exporting gbp_server_* other than libgbp (declare_server applied), e.g. a test build."""
        self.L = lib if lib is not None else load_library()
        self.n = inst.n
        self._keep = [np.ascontiguousarray(a) for a in (inst.rowptr.astype(np.int64), inst.colidx.astype(np.int32),
                                                        inst.vals, inst.lhs, inst.rhs, inst.isint.astype(np.int8),
                                                        np.asarray(rootlb, np.float64), np.asarray(rootub, np.float64))]
        h = _P()
        par = params if params is not None else default_params()
        rc = self.L.gbp_server_create(ctypes.byref(h), device, workers, inst_workers, max_batch, hbm_cap,
                                      ctypes.byref(par), inst.m, inst.n, *[_ptr(a) for a in self._keep])
        if rc != GBP_OK:
            raise GbpError(rc, self.L.gbp_error_string(rc).decode())
        self.h = h
        self._out = (np.empty(self.n, np.int32), np.empty(self.n), np.empty(self.n))
        self._borrowed = {}  # ticket -> the arrays of an instance request, alive until its reply is read

    def submit(self, cols, lb, ub) -> int:
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        lb = np.ascontiguousarray(lb, dtype=np.float64)
        ub = np.ascontiguousarray(ub, dtype=np.float64)
        t = ctypes.c_int64()
        rc = self.L.gbp_server_submit(self.h, len(cols), _ptr(cols), _ptr(lb), _ptr(ub), ctypes.byref(t))
        if rc != GBP_OK:
            raise GbpError(rc, self.L.gbp_error_string(rc).decode())
        return t.value

    def submit_instance(self, inst) -> int:
        """An instance request (a problem of its own, answered with its root fixpoint); needs inst_workers > 0.
        libgbp borrows the arrays: they are kept alive here until the reply has been read."""
        arrs = [np.ascontiguousarray(a, dtype=d) for a, d in ((inst.rowptr, np.int64), (inst.colidx, np.int32),
                                                             (inst.vals, np.float64), (inst.lhs, np.float64),
                                                             (inst.rhs, np.float64), (inst.isint, np.int8),
                                                             (inst.lb, np.float64), (inst.ub, np.float64))]
        t = ctypes.c_int64()
        rc = self.L.gbp_server_submit_instance(self.h, inst.m, inst.n, *[_ptr(a) for a in arrs], ctypes.byref(t))
        if rc != GBP_OK:
            raise GbpError(rc, self.L.gbp_error_string(rc).decode())
        self._borrowed[t.value] = arrs
        return t.value

    def poll(self, ticket: int, wait_ms: int = -1, cap: Optional[int] = None):
        """(cutoff, cols, lb, ub, t_submit_ns, t_done_ns), or None when the wait ended first.  An instance reply
        holds every column of the instance: give cap >= its columns when they exceed the resident problem's."""
        if cap is not None and cap > len(self._out[0]):
            self._out = (np.empty(cap, np.int32), np.empty(cap), np.empty(cap))
        c, l, u = self._out
        cut = ctypes.c_int32()
        n = ctypes.c_int64()
        ts = ctypes.c_int64()
        td = ctypes.c_int64()
        rc = self.L.gbp_server_poll(self.h, ticket, wait_ms, ctypes.byref(cut), len(c), ctypes.byref(n), _ptr(c),
                                    _ptr(l), _ptr(u), ctypes.byref(ts), ctypes.byref(td))
        if rc == GBP_ERR_OVERFLOW:  # the reply stays available: read it with room for every column it holds
            return self.poll(ticket, 0, n.value)
        if rc == GBP_ERR_BUSY:
            return None
        self._borrowed.pop(ticket, None)
        if rc not in (GBP_OK, GBP_ERR_LIMIT):
            raise GbpError(rc, self.L.gbp_error_string(rc).decode())
        k = n.value
        return bool(cut.value), c[:k].copy(), l[:k].copy(), u[:k].copy(), ts.value, td.value

    def stats(self):
        v = [ctypes.c_int64() for _ in range(4)]
        self.L.gbp_server_stats(self.h, *[ctypes.byref(x) for x in v])
        return {"batches": v[0].value, "requests": v[1].value, "max_batch": v[2].value, "budget": v[3].value}

    def close(self):
        if getattr(self, "h", None):
            self.L.gbp_server_destroy(self.h)  # joins the workers: nothing borrowed is read after this
            self.h = None
            self._borrowed.clear()

