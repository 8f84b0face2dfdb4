"""Generate the golden fixtures: SCIP 11's own cons_linear propagation results on seeded instances.

Runs oracle/_ref/scip_oracle (SCIP built from the reference sources by `make -C oracle ref`) in the
probing-in-heuristic pattern described in oracle/scip_driver.c and stores, per case, the instance arrays
(so that the fixtures do not depend on numpy's generator streams), SCIP's root fixpoint, and for node cases
SCIP's per-node cutoff verdicts and changed bounds.  Cases:

  root_mip_s{0,1,2}          2,000 x 5,000 root fixpoint, residual rule (maxeasyactivitydelta 0) and easy rule
  root_mip_s0_nodes          200 branch-and-bound nodes on top of SCIP's root fixpoint
  node_mip_small             1,500 x 3,000 general rows (log-uniform coefficients, infinite bounds) + 200 nodes
  zipf_small                 1,500 x 3,000 Zipf row lengths up to 400 (rows longer than 64 entries)
  set_cover / knapsack / network   one small instance of each uneven-batch family + 100 nodes
  indicator_packing          2,000 x 4,000 binary packing rows with an indicator (3 % of rows 65..300 long)
                             + 300 nodes: SCIP's binary skip in tightenBounds decides many of them

Usage: python tests/golden/make_golden.py [case ...]   (needs the SCIP sources; writes tests/golden/*.npz;
no argument builds every case)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from scip_gb300 import instances  # noqa: E402
import oracle  # noqa: E402


def node_arrays(nodes_out):
    cut = np.array([x[0] for x in nodes_out], dtype=np.int8)
    cnt = np.array([len(x[2]) for x in nodes_out], dtype=np.int64)
    ptr = np.zeros(len(nodes_out) + 1, dtype=np.int64)
    np.cumsum(cnt, out=ptr[1:])
    col = np.concatenate([x[2] for x in nodes_out] + [np.zeros(0, np.int32)]).astype(np.int32)
    lb = np.concatenate([x[3] for x in nodes_out] + [np.zeros(0)])
    ub = np.concatenate([x[4] for x in nodes_out] + [np.zeros(0)])
    return cut, ptr, col, lb, ub


def save_case(name, inst, nnodes=0, node_seed=11):
    out = {"rowptr": inst.rowptr, "colidx": inst.colidx, "vals": inst.vals, "lhs": inst.lhs, "rhs": inst.rhs,
           "lb": inst.lb, "ub": inst.ub, "isint": inst.isint}
    for easy in (False, True):
        tag = "easy" if easy else "res"
        rcut, rlb, rub, _ = oracle.run_scip(inst, easy=easy)
        out[f"{tag}_rootcut"] = np.int8(rcut)
        out[f"{tag}_rootlb"] = rlb
        out[f"{tag}_rootub"] = rub
    if nnodes:
        # nodes start from SCIP's own root fixpoint (residual rule) so that node results compare node work only
        rlb, rub = out["res_rootlb"], out["res_rootub"]
        nodes = instances.node_batch(inst, rlb, rub, nnodes, seed=node_seed)
        out["node_ptr"], out["node_col"], out["node_lb"], out["node_ub"] = nodes.ptr, nodes.col, nodes.lb, nodes.ub
        for easy in (False, True):
            tag = "easy" if easy else "res"
            _, rlb2, rub2, res = oracle.run_scip(inst, nodes, easy=easy)
            assert np.array_equal(rlb2, out[f"{tag}_rootlb"]) and np.array_equal(rub2, out[f"{tag}_rootub"])
            cut, ptr, col, lb, ub = node_arrays(res)
            out[f"{tag}_ncut"], out[f"{tag}_nptr"], out[f"{tag}_ncol"] = cut, ptr, col
            out[f"{tag}_nlb"], out[f"{tag}_nub"] = lb, ub
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {inst.m}x{inst.n}, {inst.nnz} nnz, {nnodes} nodes, {os.path.getsize(path) // 1024} KiB")


def cases():
    """name -> (instance builder, nodes); the uneven-family cases share one generator, drawn in this order."""
    out = {}
    for s in (0, 1, 2):
        out[f"root_mip_s{s}"] = (lambda s=s: instances.root_mip(s), 200 if s == 0 else 0)
    out["node_mip_small"] = (lambda: instances.node_mip(seed=21, m=1500, n=3000), 200)
    out["zipf_small"] = (lambda: instances.zipf_mip(seed=22, m=1500, n=3000, hi=400), 100)
    rng = np.random.default_rng(np.random.PCG64(23))
    fam = {}

    def family(k):
        if not fam:
            fam["set_cover"] = instances.set_cover(rng, 1200, 2400)
            fam["knapsack"] = instances.multi_knapsack(rng, 1000, 2000)
            fam["network"] = instances.network_flow(rng, 1500)
        return fam[k]

    for k in ("set_cover", "knapsack", "network"):
        out[k] = (lambda k=k: family(k), 100)
    out["indicator_packing"] = (lambda: instances.indicator_packing(np.random.default_rng(np.random.PCG64(24)),
                                                                    2000, 4000, long_frac=0.03), 300)
    return out


def main(names):
    if not os.path.exists(oracle.SCIP_ORACLE):
        raise SystemExit("oracle/_ref/scip_oracle missing: run `make -C oracle ref` where the SCIP sources are")
    all_cases = cases()
    for name in names or list(all_cases):
        make, nnodes = all_cases[name]
        save_case(name, make(), nnodes=nnodes)


if __name__ == "__main__":
    main(sys.argv[1:])
