"""libgbp's serving loop (scip_gb300/csrc/gbp_server.cu) built for the host against the oracle test double
(tests/plugin/gbp_oracle_shim.c) with host-memory stand-ins for its own CUDA runtime calls
(tests/native/cuda_host_stub.c): the loop's host logic on a machine without a GPU -- tickets, batching of
concurrent node requests, instance requests with borrowed arrays, a bad request failing alone, admission, polling
an unknown ticket, shutdown with requests outstanding.  Every reply equals the oracle's own result for that request
(the GPU build of the same loop is checked against the oracle in tests/test_server_gpu.py)."""
import ctypes
import os
import shutil
import subprocess
import threading

import numpy as np
import pytest

from scip_gb300 import gbp, instances

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime_api.h")):
        pytest.skip("g++ or the CUDA headers missing")
    d = tmp_path_factory.mktemp("server_cpu")
    objs = [str(d / "server.o")]
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-x", "c++", "-c",
                    os.path.join(ROOT, "scip_gb300", "csrc", "gbp_server.cu"), "-I", CUDA_INC, "-o", objs[0]],
                   check=True, capture_output=True)
    for src in (os.path.join(ROOT, "tests", "plugin", "gbp_oracle_shim.c"),
                os.path.join(ROOT, "oracle", "linprop_oracle.c"), os.path.join(ROOT, "oracle", "linprop_seq.c"),
                os.path.join(ROOT, "tests", "native", "cuda_host_stub.c")):
        o = str(d / (os.path.basename(src)[:-2] + ".o"))
        subprocess.run(["gcc", "-std=c99", "-O1", "-fPIC", "-D_XOPEN_SOURCE=600", "-ffp-contract=off",
                        "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"), "-I", CUDA_INC,
                        "-c", src, "-o", o], check=True, capture_output=True)
        objs.append(o)
    so = str(d / "libgbp_server_host.so")
    # -Bsymbolic: the library's own stand-ins and test double, even where the process has loaded the CUDA runtime
    # or libgbp itself
    subprocess.run(["g++", "-shared", "-Wl,-Bsymbolic", "-o", so, *objs, "-lpthread"], check=True,
                   capture_output=True)
    L = ctypes.CDLL(so)
    gbp.declare_server(L)
    L.gbp_default_params.argtypes = [ctypes.POINTER(gbp.GbpParams)]
    L.gbp_default_params.restype = None
    return L


def _params(L):
    p = gbp.GbpParams()
    L.gbp_default_params(ctypes.byref(p))
    p.maxeasyactivitydelta = 0.0
    return p


def _setup(oracle_mod, m=2000, nnodes=200):
    inst = instances.node_mip(seed=2, m=m, n=2 * m)
    orc = oracle_mod.Oracle(inst)
    par = oracle_mod.params(0.0)
    rlb, rub, _ = orc.propagate(inst.lb, inst.ub, par)
    nodes = instances.node_batch(inst, rlb, rub, nnodes, seed=31)
    want = orc.propagate_nodes(rlb, rub, nodes, par, cap=inst.n)
    return inst, rlb, rub, nodes, want


def test_concurrent_node_requests_equal_the_oracle(lib, oracle_mod):
    inst, rlb, rub, nodes, want = _setup(oracle_mod)
    srv = gbp.Server(inst, rlb, rub, params=_params(lib), workers=2, max_batch=64, lib=lib)
    try:
        tickets = [None] * nodes.nnodes

        def client(part):
            for k in range(part, nodes.nnodes, 4):
                sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
                tickets[k] = srv.submit(nodes.col[sl], nodes.lb[sl], nodes.ub[sl])

        th = [threading.Thread(target=client, args=(p,)) for p in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert len(set(tickets)) == nodes.nnodes
        for k in range(nodes.nnodes):
            cut, c, l, u, ts, td = srv.poll(tickets[k])
            assert cut == bool(want["cutoff"][k]), f"node {k}"
            assert td >= ts
            if cut:
                continue
            n = want["n"][k]
            o = np.argsort(want["col"][k, :n])
            assert np.array_equal(c, want["col"][k, :n][o]), f"node {k}"
            assert np.array_equal(l, want["lb"][k, :n][o]) and np.array_equal(u, want["ub"][k, :n][o]), f"node {k}"
        st = srv.stats()
        assert st["requests"] >= nodes.nnodes and st["batches"] < st["requests"] and st["max_batch"] <= 64
    finally:
        srv.close()


def test_instance_requests_with_a_bad_one(lib, oracle_mod):
    """Instance requests beside node requests: each reply is every column of the instance at the oracle's root
    fixpoint of that instance alone; a request whose column index lies outside its instance is answered
    GBP_ERR_INVALID while the rest of its batch is served."""
    from scip_gb300.instances import Instance
    inst, rlb, rub, nodes, want = _setup(oracle_mod, m=1000, nnodes=40)
    pool = [p for p in instances.uneven_batch(seed=41, count=24, rmin=200, rmax=3000)][:10]
    bad = Instance(np.array([0, 2], np.int64), np.array([0, 5], np.int32), np.array([1.0, 1.0]), np.array([1.0]),
                   np.array([1e20]), np.zeros(2), np.full(2, 2.0), np.ones(2, np.int8), x0=np.zeros(2))
    srv = gbp.Server(inst, rlb, rub, params=_params(lib), workers=1, inst_workers=2, lib=lib)
    try:
        tk = [srv.submit_instance(p) for p in pool[:5]]
        tk_bad = srv.submit_instance(bad)
        tk += [srv.submit_instance(p) for p in pool[5:]]
        tk_n = []
        for k in range(nodes.nnodes):
            sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
            tk_n.append(srv.submit(nodes.col[sl], nodes.lb[sl], nodes.ub[sl]))
        for p, t in zip(pool, tk):
            cut, c, l, u, _, _ = srv.poll(t)
            olb, oub, ores = oracle_mod.Oracle(p).propagate(p.lb, p.ub, oracle_mod.params(0.0))
            assert cut == bool(ores.cutoff)
            if not cut:
                assert np.array_equal(c, np.arange(p.n)) and np.array_equal(l, olb) and np.array_equal(u, oub)
        for k, t in enumerate(tk_n):
            assert srv.poll(t)[0] == bool(want["cutoff"][k])
        with pytest.raises(gbp.GbpError) as e:
            srv.poll(tk_bad)
        assert e.value.code == gbp.GBP_ERR_INVALID
        assert not srv._borrowed  # every borrowed instance released once its reply was read
    finally:
        srv.close()


def test_admission_unknown_tickets_and_bad_columns(lib, oracle_mod):
    inst, rlb, rub, nodes, _ = _setup(oracle_mod, m=500, nnodes=4)
    srv = gbp.Server(inst, rlb, rub, params=_params(lib), workers=1, hbm_cap=1000, lib=lib)
    try:
        assert srv.stats()["budget"] == 1000
        with pytest.raises(gbp.GbpError) as e:  # one request alone needs more than the budget
            srv.submit(nodes.col[:1], nodes.lb[:1], nodes.ub[:1])
        assert e.value.code == gbp.GBP_ERR_NOMEM
    finally:
        srv.close()
    srv = gbp.Server(inst, rlb, rub, params=_params(lib), workers=1, lib=lib)
    try:
        with pytest.raises(gbp.GbpError) as e:
            srv.submit(np.array([inst.n], np.int32), np.zeros(1), np.ones(1))
        assert e.value.code == gbp.GBP_ERR_INVALID
        with pytest.raises(gbp.GbpError) as e:
            srv.poll(123456)
        assert e.value.code == gbp.GBP_ERR_INVALID
        with pytest.raises(gbp.GbpError) as e:  # no instance workers
            srv.submit_instance(inst)
        assert e.value.code == gbp.GBP_ERR_INVALID
    finally:
        srv.close()


def test_shutdown_with_requests_outstanding(lib, oracle_mod):
    """Closing the server with requests queued and none polled serves what is queued and returns."""
    inst, rlb, rub, nodes, _ = _setup(oracle_mod, m=1000, nnodes=100)
    srv = gbp.Server(inst, rlb, rub, params=_params(lib), workers=2, max_batch=8, lib=lib)
    for k in range(nodes.nnodes):
        sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
        srv.submit(nodes.col[sl], nodes.lb[sl], nodes.ub[sl])
    t = threading.Thread(target=srv.close)
    t.start()
    t.join(timeout=120)
    assert not t.is_alive()


def test_node_requests_in_scip_order(lib, oracle_mod):
    """A server created with GBP_FLAG_SCIPORDER answers node requests in SCIP's own order: rows uploaded in the order
    SCIP sorts them into on the root bounds, every reply equal to the oracle's restatement of that order."""
    inst, rlb, rub, nodes, _ = _setup(oracle_mod, m=1000, nnodes=60)
    order = instances.scip_row_order(inst, rlb, rub, instances.scip_var_index(inst.isint, inst.lb, inst.ub))
    ordered = instances.in_order(inst, order)
    want = oracle_mod.Oracle(ordered).propagate_nodes(rlb, rub, nodes, oracle_mod.params(0.0), cap=inst.n, seq=True)
    par = _params(lib)
    par.flags |= gbp.GBP_FLAG_SCIPORDER
    srv = gbp.Server(ordered, rlb, rub, params=par, workers=2, max_batch=16, lib=lib)
    try:
        tk = []
        for k in range(nodes.nnodes):
            sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
            tk.append(srv.submit(nodes.col[sl], nodes.lb[sl], nodes.ub[sl]))
        for k, t in enumerate(tk):
            cut, c, l, u, _, _ = srv.poll(t)
            assert cut == bool(want["cutoff"][k]), f"node {k}"
            if cut:
                continue
            n = want["n"][k]
            o = np.argsort(want["col"][k, :n])
            assert np.array_equal(c, want["col"][k, :n][o]), f"node {k}"
            assert np.array_equal(l, want["lb"][k, :n][o]) and np.array_equal(u, want["ub"][k, :n][o]), f"node {k}"
    finally:
        srv.close()
