"""Helpers shared by the golden-fixture tests (CPU oracle and GPU path against SCIP's own results)."""
from __future__ import annotations

import glob
import os
from dataclasses import dataclass

import numpy as np

from scip_gb300.instances import Instance, NodeBatch

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
# the MIPLIB instances the reference ships, with SCIP's results (tests/golden/make_golden.py miplib)
MIPLIB_CASES = sorted("miplib/" + os.path.splitext(os.path.basename(p))[0]
                      for p in glob.glob(os.path.join(GOLDEN, "miplib", "*.npz")))

# continuous bounds: equal within 1e-9 relative or feastol absolute
REL_TOL = 1e-9
ABS_TOL = 1e-6


def _digest(*arrays):
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        if a.dtype.kind == "f":
            a = a + 0.0  # -0.0 and +0.0 are the same bound (SCIP reports some zero bounds as -0.0)
        h.update(a.tobytes())
    return h.hexdigest()


def load_node_workload(oracle_mod, with_states=False):
    """The batched-node benchmark workload (200,000 x 400,000, 4,096 nodes) with SCIP's results
    (golden/workload/node_workload_scip.npz).  The instance is regenerated from its seed and checked against the
    fixture's digest; SCIP's root bounds and row orders come from the oracle's restatement of SCIP's order, checked
    against the digests of SCIP's own.  Returns (inst, rows in SCIP's order, root lb, root ub, nodes, fixture), and
    with_states the root's final row states after them."""
    from scip_gb300 import instances

    with np.load(os.path.join(GOLDEN, "workload", "node_workload_scip.npz")) as f:
        z = dict(f)  # an archive's arrays are decompressed on every access: read them once
    inst = instances.node_mip(seed=2)
    assert _digest(inst.rowptr, inst.colidx, inst.vals, inst.lhs, inst.rhs, inst.lb, inst.ub,
                   inst.isint) == str(z["instance_sha256"]), "the regenerated instance differs from the fixture's"
    vidx = instances.scip_var_index(inst.isint, inst.lb, inst.ub)
    lb, ub, r, order, *states = oracle_mod.Oracle(inst, vidx).propagate_seq(inst.lb, inst.ub, oracle_mod.params(0.0),
                                                                           states=with_states)
    assert not r.cutoff and _digest(lb, ub) == str(z["root_sha256"]), "root bounds differ from SCIP's"
    deleted = np.zeros(inst.m, dtype=bool)
    deleted[z["rowdel"]] = True
    live = ~np.repeat(deleted, np.diff(inst.rowptr))
    assert _digest(order[live]) == str(z["order_sha256"]), "row orders differ from SCIP's"
    nodes = instances.node_batch(inst, lb, ub, 4096, seed=3)
    assert _digest(nodes.ptr, nodes.col, nodes.lb, nodes.ub) == str(z["nodes_sha256"])
    return (inst, instances.in_order(inst, order), lb, ub, nodes, z) + tuple(states)


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        z = dict(f)  # an archive's arrays are decompressed on every access: read them once
    inst = Instance(z["rowptr"], z["colidx"], z["vals"], z["lhs"], z["rhs"], z["lb"], z["ub"], z["isint"], name=name)
    return inst, z


def nodes_of(z):
    if "node_ptr" not in z:
        return None
    return NodeBatch(z["node_ptr"], z["node_col"], z["node_lb"], z["node_ub"])


def scip_node_sparse(z, tag, k):
    """SCIP's changed columns of node k as (cols, lb, ub), or None if cut off."""
    if z[f"{tag}_ncut"][k]:
        return None
    p = z[f"{tag}_nptr"]
    sl = slice(p[k], p[k + 1])
    return z[f"{tag}_ncol"][sl], z[f"{tag}_nlb"][sl], z[f"{tag}_nub"][sl]


def scip_node(z, tag, k, rlb, rub):
    """SCIP's bounds of node k as full vectors (None if cut off)."""
    if z[f"{tag}_ncut"][k]:
        return None
    p = z[f"{tag}_nptr"]
    sl = slice(p[k], p[k + 1])
    lb, ub = rlb.copy(), rub.copy()
    lb[z[f"{tag}_ncol"][sl]] = z[f"{tag}_nlb"][sl]
    ub[z[f"{tag}_ncol"][sl]] = z[f"{tag}_nub"][sl]
    return lb, ub


@dataclass
class Agreement:
    problems: int = 0
    cutoff_mismatch: int = 0
    int_exact: int = 0            # problems whose integer bounds all equal SCIP's
    int_cols_diff: int = 0
    cont_cols: int = 0
    cont_cols_out_of_tol: int = 0

    def add_sparse(self, isint, rlb, rub, a, b):
        """add() for results given as the columns that differ from the base (cols, lb, ub), or None for cutoff: only
        the columns either side changed are compared (the rest equal the base on both sides)."""
        if a is None or b is None:
            self.add(isint, a, b)
            return
        cols = np.union1d(a[0], b[0])
        al, au = rlb[cols].copy(), rub[cols].copy()
        bl, bu = al.copy(), au.copy()
        ia, ib = np.searchsorted(cols, a[0]), np.searchsorted(cols, b[0])
        al[ia], au[ia] = a[1], a[2]
        bl[ib], bu[ib] = b[1], b[2]
        self.add(isint[cols], (al, au), (bl, bu))

    def add(self, isint, a, b):
        """a, b: (lb, ub) of ours and SCIP's, or None for cutoff."""
        self.problems += 1
        if (a is None) != (b is None):
            self.cutoff_mismatch += 1
            return
        if a is None:
            self.int_exact += 1
            return
        il = isint == 1
        d = ((a[0] != b[0]) | (a[1] != b[1])) & il
        self.int_cols_diff += int(d.sum())
        self.int_exact += int(d.sum() == 0)
        c = ~il
        tol_l = np.maximum(REL_TOL * np.abs(b[0]), ABS_TOL)
        tol_u = np.maximum(REL_TOL * np.abs(b[1]), ABS_TOL)
        out = c & ((np.abs(a[0] - b[0]) > tol_l) | (np.abs(a[1] - b[1]) > tol_u))
        self.cont_cols += int(c.sum())
        self.cont_cols_out_of_tol += int(out.sum())


def load_mixed_small():
    return load_mixed("mixed_small")


def load_mixed(name):
    """golden/fuzz/<name>.npz split into its 300 instances: per instance a dict with the instance, its seed,
    per rule and sortvars setting ("res", "easy", "res_nosort", "easy_nosort") SCIP's root (cut, lb, ub, order, rowdel) and its nodes' results (a list of
    (cutoff, cols, lb, ub) with instance-local columns that differ from that rule's root), and the nodes
    (instance-local NodeBatch, or None)."""
    with np.load(os.path.join(GOLDEN, "fuzz", f"{name}.npz")) as f:
        z = dict(f)
    ro, co = z["row_off"], z["col_off"]
    K = len(ro) - 1
    ninst = z["node_inst"]
    first = np.searchsorted(ninst, np.arange(K + 1))
    out = []
    for k in range(K):
        r0, r1, c0, c1 = int(ro[k]), int(ro[k + 1]), int(co[k]), int(co[k + 1])
        p0, p1 = int(z["rowptr"][r0]), int(z["rowptr"][r1])
        inst = Instance(z["rowptr"][r0:r1 + 1] - p0, z["colidx"][p0:p1] - c0, z["vals"][p0:p1], z["lhs"][r0:r1],
                        z["rhs"][r0:r1], z["lb"][c0:c1], z["ub"][c0:c1], z["isint"][c0:c1],
                        name=f"{name}/{int(z['seeds'][k])}")
        q0, q1 = int(first[k]), int(first[k + 1])
        nb = None
        if q1 > q0:
            ptr = z["node_ptr"][q0:q1 + 1]
            sl = slice(int(ptr[0]), int(ptr[-1]))
            nb = NodeBatch(ptr - ptr[0], z["node_col"][sl], z["node_lb"][sl], z["node_ub"][sl])
        d = {"inst": inst, "seed": int(z["seeds"][k]), "nodes": nb}
        for tag in [t for t in ("res", "easy", "res_nosort", "easy_nosort") if f"{t}_rootcut" in z]:
            root = {"cut": bool(z[f"{tag}_rootcut"][k]), "lb": z[f"{tag}_rootlb"][c0:c1],
                    "ub": z[f"{tag}_rootub"][c0:c1], "order": z[f"{tag}_order"][p0:p1],
                    "rowdel": z[f"{tag}_rowdel"][r0:r1].astype(bool)}
            res = []
            for q in range(q0, q1):
                a, b = int(z[f"{tag}_nptr"][q]), int(z[f"{tag}_nptr"][q + 1])
                res.append((bool(z[f"{tag}_ncut"][q]), z[f"{tag}_ncol"][a:b], z[f"{tag}_nlb"][a:b],
                            z[f"{tag}_nub"][a:b]))
            d[tag] = {"root": root, "nodes": res}
        out.append(d)
    return out

