"""Test infrastructure only: the CPU baselines of the batched-node workload on this machine's cores -- SCIP 11
itself (oracle/_ref/scip_oracle: SCIPpropagateProbing per node, the probing pattern its driver documents, each
node timed inside SCIP) against the oracle's two C restatements (the Jacobi rounds of oracle/linprop_oracle.c and
SCIP's own order, oracle/linprop_seq.c), on 1 core and on all cores, on the same nodes from SCIP's root fixpoint.

    python oracle/calibrate.py [nodes] > profiles/cpu_calibration_x86.json

Needs oracle/_ref (built where the SCIP sources are, `make -C oracle ref REFDIR=...`).  bench.py reports the
SCIP/port speed ratio it prints as cpu_baseline.scip_over_port.
"""
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

import oracle  # noqa: E402
from scip_gb300 import instances  # noqa: E402


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def timed(fn):
    t0 = time.perf_counter()
    out = fn()
    return out, time.perf_counter() - t0


def main(nnodes):
    if not os.path.exists(oracle.SCIP_ORACLE):
        raise SystemExit("oracle/_ref/scip_oracle missing: run `make -C oracle ref` where the SCIP sources are")
    oracle.build()
    inst = instances.node_mip(seed=2)
    base = instances.pinned_node_base(inst, os.path.join(os.path.dirname(HERE), "tests", "golden", "workload",
                                                         "node_workload_base.npz"))
    lb, ub, order = base
    nodes = instances.node_batch(inst, lb, ub, nnodes, seed=3)
    par = oracle.params(0.0)
    # SCIP: each node's seconds as the driver measures them around SCIPnewProbingNode .. SCIPbacktrackProbing
    _, slb, sub, res = oracle.run_scip(inst, nodes, unmark=True)
    assert np.array_equal(slb, lb) and np.array_equal(sub, ub), "SCIP's root differs from the pinned base"
    scip_s = float(sum(r[1] for r in res))
    ncores = os.cpu_count() or 1
    jac, seq = oracle.Oracle(inst), oracle.Oracle(instances.in_order(inst, order))
    out = {"machine": cpu_model(), "arch": platform.machine(), "cores": ncores, "nodes": nnodes,
           "workload": "node_mip 200,000 x 400,000 (seed 2), nodes from SCIP's root fixpoint (seed 3), residual rule",
           "scip_1core": {"value": nnodes / scip_s, "unit": "node-fixpoints/s", "seconds": scip_s}}
    for name, orc, seqmode in (("port_jacobi", jac, False), ("port_scip_order", seq, True)):
        for cores in (1, ncores):
            _, s = timed(lambda: orc.propagate_nodes(lb, ub, nodes, par, cap=1024, nthreads=cores, seq=seqmode))
            out[f"{name}_{'1core' if cores == 1 else 'allcores'}"] = {"value": nnodes / s, "unit": "node-fixpoints/s",
                                                                      "seconds": s, "threads": cores}
    out["scip_over_port_jacobi_1core"] = out["scip_1core"]["value"] / out["port_jacobi_1core"]["value"]
    out["scip_over_port_scip_order_1core"] = out["scip_1core"]["value"] / out["port_scip_order_1core"]["value"]
    out["command"] = "python oracle/calibrate.py %d" % nnodes
    print(json.dumps(out, indent=2))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 1024)
