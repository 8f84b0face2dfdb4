"""Helpers shared by the golden-fixture tests (CPU oracle and GPU path against SCIP's own results)."""
from __future__ import annotations

import glob
import os
from dataclasses import dataclass

import numpy as np

from scip_gb300.instances import Instance, NodeBatch

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))

# continuous bounds: equal within 1e-9 relative or feastol absolute
REL_TOL = 1e-9
ABS_TOL = 1e-6


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    inst = Instance(z["rowptr"], z["colidx"], z["vals"], z["lhs"], z["rhs"], z["lb"], z["ub"], z["isint"], name=name)
    return inst, z


def nodes_of(z):
    if "node_ptr" not in z:
        return None
    return NodeBatch(z["node_ptr"], z["node_col"], z["node_lb"], z["node_ub"])


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
