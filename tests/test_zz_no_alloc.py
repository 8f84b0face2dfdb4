"""gbp_propagate_nodes_noalloc, the entry point for callers that cannot let a library allocate device memory.

Those callers (applications that own all device memory through their own pool allocator, and callers that
must not trigger the device-wide synchronisation of cudaMalloc/cudaFree) pass every input and output as a
device pointer; the library works in a fixed __device__ scratch array.  The results must be exactly those of
the context-based gbp_propagate_nodes_device, on two calls in a row (the second call runs on the scratch the
first one left behind).  This file is collected last so that a failure here does not hide any other test.
"""
import ctypes

import numpy as np
import pytest

from scip_gb300 import gbp, instances

pytestmark = pytest.mark.gpu


def _outputs(torch, d, nnodes, cap):
    return {"cutoff": torch.zeros(nnodes, dtype=torch.int8, device=d),
            "rounds": torch.zeros(nnodes, dtype=torch.int32, device=d),
            "off": torch.zeros(nnodes, dtype=torch.int64, device=d),
            "n": torch.zeros(nnodes, dtype=torch.int32, device=d),
            "col": torch.zeros(cap, dtype=torch.int32, device=d),
            "lb": torch.zeros(cap, dtype=torch.float64, device=d),
            "ub": torch.zeros(cap, dtype=torch.float64, device=d)}


def _per_node(out):
    h = {k: v.cpu().numpy() for k, v in out.items()}
    nodes = []
    for k in range(h["cutoff"].shape[0]):
        o, c = int(h["off"][k]), int(h["n"][k])
        assert c >= 0
        cols, lbs, ubs = h["col"][o:o + c], h["lb"][o:o + c], h["ub"][o:o + c]
        order = np.argsort(cols)
        nodes.append((int(h["cutoff"][k]), int(h["rounds"][k]), cols[order], lbs[order], ubs[order]))
    return nodes


def test_noalloc_matches_context_entry_point(oracle_mod):
    torch = pytest.importorskip("torch")
    L = gbp.load_library()
    inst = instances.node_mip(seed=5, m=6000, n=12000)
    params = gbp.default_params(maxeasy=0.0)
    prop = gbp.Propagator(0, params=params)
    prop.upload(inst)
    rlb, rub, _, _ = prop.propagate(inst.lb, inst.ub)
    nodes = instances.node_batch(inst, rlb, rub, 300, seed=4)
    N = nodes.nnodes
    cap = 64 * N
    d = torch.device("cuda", 0)

    def T(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(d)

    colptr, rowidx, cvals = inst.csc()
    A = {"rowptr": T(inst.rowptr), "colidx": T(inst.colidx), "vals": T(inst.vals), "lhs": T(inst.lhs),
         "rhs": T(inst.rhs), "isint": T(inst.isint), "colptr": T(colptr), "rowidx": T(rowidx), "cvals": T(cvals),
         "lb": T(rlb), "ub": T(rub), "ptr": T(nodes.ptr), "col": T(nodes.col), "nlb": T(nodes.lb),
         "nub": T(nodes.ub)}

    ref = _outputs(torch, d, N, cap)
    rref = prop.propagate_nodes_device(A["lb"], A["ub"], N, A["ptr"], A["col"], A["nlb"], A["nub"], ref, cap)
    torch.cuda.synchronize()
    expect = _per_node(ref)
    assert sum(e[0] for e in expect) < N
    # the context entry point itself against the oracle
    o = oracle_mod.Oracle(inst).propagate_nodes(rlb, rub, nodes, oracle_mod.params(0.0), cap=inst.n)
    for k, e in enumerate(expect):
        assert e[0] == o["cutoff"][k], f"node {k}: cutoff differs from the oracle"
        if e[0]:
            continue
        n = o["n"][k]
        srt = np.argsort(o["col"][k, :n])
        assert np.array_equal(e[2], o["col"][k, :n][srt]), f"node {k}: changed columns differ from the oracle"
        assert np.array_equal(e[3], o["lb"][k, :n][srt]) and np.array_equal(e[4], o["ub"][k, :n][srt])

    p = lambda t: ctypes.c_void_p(t.data_ptr())
    for call in range(2):
        out = _outputs(torch, d, N, cap)
        res = gbp.GbpResult()
        rc = L.gbp_propagate_nodes_noalloc(inst.m, inst.n, p(A["rowptr"]), p(A["colidx"]), p(A["vals"]),
                                           p(A["lhs"]), p(A["rhs"]), p(A["isint"]), p(A["colptr"]),
                                           p(A["rowidx"]), p(A["cvals"]), p(A["lb"]), p(A["ub"]), N, p(A["ptr"]),
                                           p(A["col"]), p(A["nlb"]), p(A["nub"]), p(out["cutoff"]),
                                           p(out["rounds"]), p(out["off"]), p(out["n"]), p(out["col"]),
                                           p(out["lb"]), p(out["ub"]), cap, ctypes.byref(params), None,
                                           ctypes.byref(res))
        assert rc == gbp.GBP_OK, f"call {call}: {L.gbp_error_string(rc).decode()}"
        got = _per_node(out)
        for k, (e, g) in enumerate(zip(expect, got)):
            assert e[0] == g[0], f"call {call}, node {k}: cutoff differs"
            if e[0]:
                continue
            assert e[1] == g[1], f"call {call}, node {k}: rounds differ"
            assert np.array_equal(e[2], g[2]), f"call {call}, node {k}: changed columns differ"
            assert np.array_equal(e[3], g[3]) and np.array_equal(e[4], g[4]), f"call {call}, node {k}: bounds differ"
        assert (res.rows, res.nnz, res.candidates, res.changes, res.cutoff) == \
               (rref.rows, rref.nnz, rref.candidates, rref.changes, rref.cutoff)
        # kernels: four slot fills, the node order (two), two input checks, the nodes; the context path: the order
        # (two), the base packing, the nodes
        assert res.launches == 9 and rref.launches == 4

    # a column index outside [0, n) in the caller's rows: the checks refuse the arrays before any node reads them
    bad = A["colidx"].clone()
    bad[5] = inst.n + 7
    out = _outputs(torch, d, N, cap)
    res = gbp.GbpResult()
    rc = L.gbp_propagate_nodes_noalloc(inst.m, inst.n, p(A["rowptr"]), p(bad), p(A["vals"]), p(A["lhs"]),
                                       p(A["rhs"]), p(A["isint"]), p(A["colptr"]), p(A["rowidx"]), p(A["cvals"]),
                                       p(A["lb"]), p(A["ub"]), N, p(A["ptr"]), p(A["col"]), p(A["nlb"]), p(A["nub"]),
                                       p(out["cutoff"]), p(out["rounds"]), p(out["off"]), p(out["n"]),
                                       p(out["col"]), p(out["lb"]), p(out["ub"]), cap, ctypes.byref(params), None,
                                       ctypes.byref(res))
    assert rc == gbp.GBP_ERR_INVALID
    assert bool((out["n"] == -1).all().item())
    prop.close()


def test_noalloc_rejects_problems_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    L = gbp.load_library()
    d = torch.device("cuda", 0)
    dummy = torch.zeros(16, dtype=torch.float64, device=d)
    p = ctypes.c_void_p(dummy.data_ptr())
    res = gbp.GbpResult()
    # two million columns need ~128 MB per node slot, beyond the 64 MiB scratch: rejected before any launch
    rc = L.gbp_propagate_nodes_noalloc(1_000_000, 2_000_000, *([p] * 11), 1, *([p] * 11), 1, None, None,
                                       ctypes.byref(res))
    assert rc == gbp.GBP_ERR_TOO_LARGE
    assert L.gbp_error_string(rc).decode() == "problem too large for the no-alloc scratch"
