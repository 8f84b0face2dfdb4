"""The served form: a mixed request stream (node requests against a resident matrix, new instances) merged
into batched launches by several workers whose batches overlap on the GPU.  Every reply must equal the reply
the plain one-request-per-call path gives for the same request alone."""
import sys

import numpy as np
import pytest

from scip_gb300 import gbp, instances, serving

pytestmark = pytest.mark.gpu


def test_each_result_is_the_same_alone_and_in_the_mix():
    sys.setswitchinterval(1e-4)
    matrix = instances.node_mip(seed=31, m=20000, n=40000)
    params = gbp.default_params(maxeasy=0.0)
    p = gbp.Propagator(0, params=params)
    p.upload(matrix)
    rlb, rub, _, _ = p.propagate(matrix.lb, matrix.ub)
    p.close()
    pool = instances.uneven_batch(seed=32, count=12, rmin=500, rmax=5000)
    stream = serving.make_stream(matrix, rlb, rub, pool, rate=3000.0, duration=0.4, seed=5)
    srv = serving.PropagationServer(matrix, rlb, rub, node_workers=2, inst_workers=2, params=params)
    try:
        mixed, lat, wall = serving.replay(srv, stream, served=True)
        batches = list(srv.batches)
    finally:
        srv.close()
    plain = serving.PlainServer(matrix, rlb, rub, params=params)
    try:
        for q, req in enumerate(stream.reqs):
            alone = plain.answer(req)
            assert serving.same_reply(mixed[q], alone), f"request {q} differs between the mix and alone"
    finally:
        plain.close()
    assert len(stream.reqs) > 500
    assert any(size > 1 for _, size, _, _ in batches), "requests were never merged"
    # batches of different workers were on the GPU at the same time
    spans = sorted((t0, t1) for _, _, t0, t1 in batches)
    assert any(spans[i + 1][0] < spans[i][1] for i in range(len(spans) - 1)), "no overlapping batches"
    assert np.isfinite(lat).all() and (lat > 0).all()


def test_hbm_cap_defers_admission():
    """With a cap that holds one instance request but never two, instance requests wait for memory to free up
    instead of being admitted together; every request is still answered."""
    matrix = instances.node_mip(seed=33, m=5000, n=10000)
    params = gbp.default_params(maxeasy=0.0)
    one = instances.uneven_batch(seed=34, count=1, rmin=2000, rmax=3000)[0]
    pool = [one] * 4
    cap = serving._inst_bytes(one)  # room for exactly one request in flight
    srv = serving.PropagationServer(matrix, matrix.lb, matrix.ub, node_workers=1, inst_workers=2, params=params,
                                    hbm_cap=cap)
    try:
        futs = [srv.submit(serving.InstanceRequest(pool[k % 4])) for k in range(12)]
        replies = [f.result(timeout=120) for f in futs]
        sizes = [size for kind, size, _, _ in srv.batches if kind == "inst"]
    finally:
        srv.close()
    assert len(replies) == 12 and max(sizes) == 1
