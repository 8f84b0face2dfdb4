"""Generate the golden fixtures: SCIP 11's own cons_linear propagation results on seeded instances.

Runs oracle/_ref/scip_oracle (SCIP built from the reference sources by `make -C oracle ref`) in the
probing-in-heuristic pattern described in oracle/scip_driver.c and stores, per case, the instance arrays
(so that the fixtures do not depend on numpy's generator streams), SCIP's root fixpoint, the order SCIP holds
each row's entries in after the root (`<rule>_order`: CSR positions) and the rows it deleted there
(`<rule>_rowdel`), and for node cases SCIP's per-node cutoff verdicts and changed bounds.  Every node starts from
a newly transformed problem (scip_driver.c --fresh), so that its result does not depend on the nodes SCIP
propagated before it.  Cases:

  root_mip_s{0,1,2}          2,000 x 5,000 root fixpoint, residual rule (maxeasyactivitydelta 0) and easy rule
  root_mip_s0_nodes          200 branch-and-bound nodes on top of SCIP's root fixpoint
  node_mip_small             1,500 x 3,000 general rows (log-uniform coefficients, infinite bounds) + 200 nodes
  zipf_small                 1,500 x 3,000 Zipf row lengths up to 400 (rows longer than 64 entries)
  set_cover / knapsack / network   one small instance of each uneven-batch family + 100 nodes
  indicator_packing          2,000 x 4,000 binary packing rows with an indicator (3 % of rows 65..300 long)
                             + 300 nodes: SCIP's binary skip in tightenBounds decides many of them
  workload/node_workload_scip  the batched-node benchmark workload itself (200,000 x 400,000, seed 2) and its 4,096
                             nodes (seed 3, drawn from SCIP's root): SCIP's node results in full, its root bounds and
                             row orders as SHA-256 digests (the test recomputes them with the oracle, whose root is
                             checked against the digests); nodes in one probing session with the marks of cut-off
                             nodes cleared (scip_driver.c --unmark), which equals --fresh on every fixture above
  ranged/gcd_rows_indep      3,000 ranged rows over 60,000 columns (rows rarely share a column; 5 % of rows
                             65..200 long) whose integer part shares a divisor: SCIP's root with ranged-row
                             propagation on (rangedrowartcons off), sortvars off and on
  ranged/gcd_rows_shared     2,000 rows over 8,000 columns, half of them equations, the same settings
  ranged/tiny_cutoffs        60 instances of 12 rows whose equations were shifted off their feasible residue, so
                             that the ranged rule finds many of them infeasible (concatenated, with offsets)
  fuzz/mixed_small           300 small random MIPs with coefficient magnitudes 1e-5..1e7 in one row, infinite
                             bounds and equations (concatenated, with offsets), SCIP's root and up to 8 nodes each
  fuzz/mixed_huge            the same with contributions past hugeval (coefficients to ~1e14, bounds to 1e9)

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
        rcut, rlb, rub, _, order, rowdel = oracle.run_scip(inst, easy=easy, order=True)
        out[f"{tag}_rootcut"] = np.int8(rcut)
        out[f"{tag}_rootlb"] = rlb
        out[f"{tag}_rootub"] = rub
        out[f"{tag}_order"] = order
        out[f"{tag}_rowdel"] = rowdel.astype(np.int8)
    if nnodes:
        # nodes start from SCIP's own root fixpoint (residual rule) so that node results compare node work only
        rlb, rub = out["res_rootlb"], out["res_rootub"]
        nodes = instances.node_batch(inst, rlb, rub, nnodes, seed=node_seed)
        out["node_ptr"], out["node_col"], out["node_lb"], out["node_ub"] = nodes.ptr, nodes.col, nodes.lb, nodes.ub
        for easy in (False, True):
            tag = "easy" if easy else "res"
            _, rlb2, rub2, res = oracle.run_scip(inst, nodes, easy=easy, fresh=True)
            assert np.array_equal(rlb2, out[f"{tag}_rootlb"]) and np.array_equal(rub2, out[f"{tag}_rootub"])
            cut, ptr, col, lb, ub = node_arrays(res)
            out[f"{tag}_ncut"], out[f"{tag}_nptr"], out[f"{tag}_ncol"] = cut, ptr, col
            out[f"{tag}_nlb"], out[f"{tag}_nub"] = lb, ub
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {inst.m}x{inst.n}, {inst.nnz} nnz, {nnodes} nodes, {os.path.getsize(path) // 1024} KiB")


MIPLIB = ["bell5", "blend2", "dcmulti", "egout", "enigma", "flugpl", "gt2", "lseu", "misc03", "p0548", "rgn"]


def save_miplib_cases():
    """The MIPLIB instances the reference ships (check/instances/MIP, read with scip_gb300/mps.py as SCIP reads
    them): SCIP's root and 100 nodes per instance, both rules, like the seeded cases, under tests/golden/miplib so
    that the GPU machine (which has no reference sources) runs them too."""
    from scip_gb300 import mps

    d = os.path.join(oracle.REFDIR, "check", "instances", "MIP")
    if not os.path.isdir(d):
        raise SystemExit("REFDIR must name the SCIP source tree (check/instances/MIP)")
    os.makedirs(os.path.join(HERE, "miplib"), exist_ok=True)
    for name in MIPLIB:
        path = os.path.join(d, name + ".mps")
        if os.path.exists(path):
            save_case(os.path.join("miplib", name), mps.read_mps(path), nnodes=100)


def save_ranged_case(name, inst):
    """SCIP's root fixpoint with ranged-row propagation, for sortvars off ("nosort") and on ("sort") and both
    rules, under tests/golden/ranged (kept apart from the cases above, whose tests run with the rule off)."""
    out = {"rowptr": inst.rowptr, "colidx": inst.colidx, "vals": inst.vals, "lhs": inst.lhs, "rhs": inst.rhs,
           "lb": inst.lb, "ub": inst.ub, "isint": inst.isint}
    for sortvars in (False, True):
        for easy in (False, True):
            tag = ("sort" if sortvars else "nosort") + ("_easy" if easy else "_res")
            rcut, rlb, rub, _ = oracle.run_scip(inst, easy=easy, ranged=True, sortvars=sortvars)
            out[f"{tag}_rootcut"] = np.int8(rcut)
            out[f"{tag}_rootlb"] = rlb
            out[f"{tag}_rootub"] = rub
    os.makedirs(os.path.join(HERE, "ranged"), exist_ok=True)
    path = os.path.join(HERE, "ranged", f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {inst.m}x{inst.n}, {inst.nnz} nnz, {os.path.getsize(path) // 1024} KiB")


def tiny_cutoff_instances():
    rng = np.random.default_rng(np.random.PCG64(32))
    out = []
    for _ in range(60):
        inst = instances.gcd_rows(rng, 12, 40, equations=True)
        shift = rng.integers(0, 3, size=inst.m).astype(np.float64)
        inst.lhs = inst.lhs + shift
        inst.rhs = inst.rhs + shift
        out.append(inst)
    return out


def save_tiny_cutoffs():
    insts = tiny_cutoff_instances()
    big, row_off, col_off = instances.concat_instances(insts)
    out = {"rowptr": big.rowptr, "colidx": big.colidx, "vals": big.vals, "lhs": big.lhs, "rhs": big.rhs,
           "lb": big.lb, "ub": big.ub, "isint": big.isint, "row_off": row_off, "col_off": col_off}
    for sortvars in (False, True):
        tag = "sort" if sortvars else "nosort"
        cut = np.zeros(len(insts), dtype=np.int8)
        lb = np.empty(big.n)
        ub = np.empty(big.n)
        for k, inst in enumerate(insts):
            c, l, u, _ = oracle.run_scip(inst, ranged=True, sortvars=sortvars)
            cut[k] = c
            lb[col_off[k]:col_off[k + 1]] = l
            ub[col_off[k]:col_off[k + 1]] = u
        out[f"{tag}_cut"], out[f"{tag}_lb"], out[f"{tag}_ub"] = cut, lb, ub
    path = os.path.join(HERE, "ranged", "tiny_cutoffs.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {len(insts)} instances, {int(out['sort_cut'].sum())} infeasible (sortvars)")


MIXED = {"mixed_small": (instances.mixed_small, range(5000, 5300)),
         "mixed_huge": (instances.mixed_huge, range(7000, 7300))}


def save_mixed(name):
    """300 small random MIPs of instances.mixed_small (seeds 5000..5299; coefficient magnitudes 1e-5..1e7 in one
    row, infinite bounds, equations) or instances.mixed_huge (seeds 7000..7299; contributions past hugeval too),
    concatenated with offsets, with SCIP's root (bounds, row orders, deleted rows) for both rules, with sortvars on
    and off (tags res, easy, res_nosort, easy_nosort), and up to 8 nodes per feasible instance (1..4 fixings, from
    SCIP's residual-rule root, every node from a newly transformed problem), under tests/golden/fuzz/<name>.npz."""
    make, MIXED_SEEDS = MIXED[name]
    insts = [make(np.random.default_rng(np.random.PCG64(s))) for s in MIXED_SEEDS]
    big, row_off, col_off = instances.concat_instances(insts)
    out = {"rowptr": big.rowptr, "colidx": big.colidx, "vals": big.vals, "lhs": big.lhs, "rhs": big.rhs,
           "lb": big.lb, "ub": big.ub, "isint": big.isint, "row_off": row_off, "col_off": col_off,
           "seeds": np.array(list(MIXED_SEEDS), np.int64)}
    K = len(insts)
    nodes = []
    tags = [(easy, sortvars) for sortvars in (True, False) for easy in (False, True)]
    for k, inst in enumerate(insts):
        for easy, sortvars in tags:
            tag = ("easy" if easy else "res") + ("" if sortvars else "_nosort")
            rcut, rlb, rub, _ = oracle.run_scip(inst, easy=easy, sortvars=sortvars)
            if rcut:
                order, rowdel = np.arange(inst.nnz, dtype=np.int32), np.zeros(inst.m, bool)
            else:
                _, _, _, _, order, rowdel = oracle.run_scip(inst, easy=easy, order=True, sortvars=sortvars)
            out.setdefault(f"{tag}_rootcut", np.zeros(K, np.int8))[k] = rcut
            out.setdefault(f"{tag}_rootlb", np.empty(big.n))[col_off[k]:col_off[k + 1]] = rlb
            out.setdefault(f"{tag}_rootub", np.empty(big.n))[col_off[k]:col_off[k + 1]] = rub
            out.setdefault(f"{tag}_order", np.empty(big.nnz, np.int32))[big.rowptr[row_off[k]]:
                                                                         big.rowptr[row_off[k + 1]]] = order
            out.setdefault(f"{tag}_rowdel", np.zeros(big.m, np.int8))[row_off[k]:row_off[k + 1]] = rowdel
        nb = None
        if not out["res_rootcut"][k]:
            rlb = out["res_rootlb"][col_off[k]:col_off[k + 1]]
            rub = out["res_rootub"][col_off[k]:col_off[k + 1]]
            try:
                nb = instances.node_batch(inst, rlb, rub, 8, seed=int(MIXED_SEEDS[k]), kmax=4)
            except ValueError:  # no unfixed integer column with finite bounds
                nb = None
        res = {}
        if nb is not None:
            for easy, sortvars in tags:
                tag = ("easy" if easy else "res") + ("" if sortvars else "_nosort")
                _, _, _, res[tag] = oracle.run_scip(inst, nb, easy=easy, fresh=True, sortvars=sortvars)
        nodes.append((nb, res))
    # nodes: node_inst[q] = the instance of node q; node columns and SCIP's changed columns are instance-local
    cnt = [0 if nb is None else nb.nnodes for nb, _ in nodes]
    out["node_inst"] = np.repeat(np.arange(K), cnt).astype(np.int32)
    parts = [nb for nb, _ in nodes if nb is not None]
    counts = np.concatenate([np.diff(nb.ptr) for nb in parts]) if parts else np.zeros(0, np.int64)
    out["node_ptr"] = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    out["node_col"] = np.concatenate([nb.col for nb in parts]).astype(np.int32)
    out["node_lb"] = np.concatenate([nb.lb for nb in parts])
    out["node_ub"] = np.concatenate([nb.ub for nb in parts])
    for tag in ("res", "easy", "res_nosort", "easy_nosort"):
        allres = [r for nb, rr in nodes if nb is not None for r in rr[tag]]
        cut, ptr, col, lb, ub = node_arrays(allres)
        out[f"{tag}_ncut"], out[f"{tag}_nptr"], out[f"{tag}_ncol"] = cut, ptr, col
        out[f"{tag}_nlb"], out[f"{tag}_nub"] = lb, ub
    os.makedirs(os.path.join(HERE, "fuzz"), exist_ok=True)
    path = os.path.join(HERE, "fuzz", f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {K} instances, {int(out['res_rootcut'].sum())} infeasible roots, {len(out['node_inst'])} nodes, "
          f"{os.path.getsize(path) // 1024} KiB")


def digest(*arrays):
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        if a.dtype.kind == "f":
            a = a + 0.0  # -0.0 and +0.0 are the same bound (SCIP reports some zero bounds as -0.0)
        h.update(a.tobytes())
    return h.hexdigest()


def save_node_workload():
    inst = instances.node_mip(seed=2)
    rcut, rlb, rub, _, order, rowdel = oracle.run_scip(inst, order=True)
    assert not rcut
    nodes = instances.node_batch(inst, rlb, rub, 4096, seed=3)
    _, rlb2, rub2, res = oracle.run_scip(inst, nodes, unmark=True)
    assert np.array_equal(rlb2, rlb) and np.array_equal(rub2, rub)
    cut, ptr, col, lb, ub = node_arrays(res)
    live = ~np.repeat(rowdel, np.diff(inst.rowptr))
    out = {"instance_sha256": digest(inst.rowptr, inst.colidx, inst.vals, inst.lhs, inst.rhs, inst.lb, inst.ub,
                                     inst.isint),
           "root_sha256": digest(rlb, rub), "order_sha256": digest(order[live]),
           "rowdel": np.nonzero(rowdel)[0].astype(np.int32),
           "nodes_sha256": digest(nodes.ptr, nodes.col, nodes.lb, nodes.ub),
           "res_ncut": cut, "res_nptr": ptr, "res_ncol": col, "res_nlb": lb, "res_nub": ub}
    os.makedirs(os.path.join(HERE, "workload"), exist_ok=True)
    path = os.path.join(HERE, "workload", "node_workload_scip.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {inst.m}x{inst.n}, {inst.nnz} nnz, {nodes.nnodes} nodes ({int(cut.sum())} cut off), "
          f"{os.path.getsize(path) // 1024} KiB")


def save_node_workload_base():
    """SCIP's root fixpoint and row orders of the batched-node workload in compact form, for the SCIP-order arm of
    bench.py (which starts its nodes from them, with no oracle): the columns the root moved, and the rows whose
    order differs from the host sort on the instance's own bounds (instances.scip_row_order), with their orders.
    Computed by the oracle's restatement of SCIP's order and checked against the digests of SCIP's own results in
    node_workload_scip.npz."""
    inst = instances.node_mip(seed=2)
    vidx = instances.scip_var_index(inst.isint, inst.lb, inst.ub)
    lb, ub, r, order = oracle.Oracle(inst, vidx).propagate_seq(inst.lb, inst.ub, oracle.params(0.0))
    with np.load(os.path.join(HERE, "workload", "node_workload_scip.npz")) as f:
        z = dict(f)
    assert not r.cutoff and digest(lb, ub) == str(z["root_sha256"])
    deleted = np.zeros(inst.m, dtype=bool)
    deleted[z["rowdel"]] = True
    live = ~np.repeat(deleted, np.diff(inst.rowptr))
    assert digest(order[live]) == str(z["order_sha256"])
    host = instances.scip_row_order(inst, inst.lb, inst.ub, vidx)
    row_of = np.repeat(np.arange(inst.m, dtype=np.int64), np.diff(inst.rowptr))
    rows = np.unique(row_of[order != host]).astype(np.int32)
    pos = np.concatenate([order[inst.rowptr[i]:inst.rowptr[i + 1]] - inst.rowptr[i] for i in rows]).astype(np.int16)
    cols = np.nonzero((lb != inst.lb) | (ub != inst.ub))[0].astype(np.int32)
    out = {"instance_sha256": digest(inst.rowptr, inst.colidx, inst.vals, inst.lhs, inst.rhs, inst.lb, inst.ub,
                                     inst.isint),
           "root_sha256": z["root_sha256"], "order_sha256": z["order_sha256"],
           "root_cols": cols, "root_lb": lb[cols], "root_ub": ub[cols], "order_rows": rows, "order_pos": pos}
    path = os.path.join(HERE, "workload", "node_workload_base.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {len(cols)} root columns, {len(rows)} reordered rows, {os.path.getsize(path) // 1024} KiB")


def ranged_cases():
    return {
        "gcd_rows_indep": lambda: instances.gcd_rows(np.random.default_rng(np.random.PCG64(30)), 3000, 60000,
                                                     long_frac=0.05, equations=False),
        "gcd_rows_shared": lambda: instances.gcd_rows(np.random.default_rng(np.random.PCG64(31)), 2000, 8000,
                                                      long_frac=0.03, equations=True),
    }


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
    ranged = ranged_cases()
    for name in names or list(all_cases) + ["ranged/" + k for k in ranged] + ["ranged/tiny_cutoffs",
                                                                             "node_workload_scip",
                                                                             "node_workload_base", "miplib",
                                                                             "fuzz/mixed_small", "fuzz/mixed_huge"]:
        if name == "node_workload_scip":
            save_node_workload()
            continue
        if name == "node_workload_base":
            save_node_workload_base()
            continue
        if name == "miplib":
            save_miplib_cases()
            continue
        if name.startswith("fuzz/"):
            save_mixed(name[len("fuzz/"):])
            continue
        if name == "ranged/tiny_cutoffs":
            save_tiny_cutoffs()
            continue
        if name.startswith("ranged/"):
            save_ranged_case(name[len("ranged/"):], ranged[name[len("ranged/"):]]())
            continue
        make, nnodes = all_cases[name]
        save_case(name, make(), nnodes=nnodes)


if __name__ == "__main__":
    main(sys.argv[1:])
