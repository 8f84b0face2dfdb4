"""Serving: a continuous-batching request loop over the batched propagator.

Requests arrive one at a time:
  * a node request -- bound changes against a resident matrix (a branch-and-bound node to propagate from the
    resident root bounds), answered with its cutoff verdict and the bounds that moved;
  * an instance request -- a new set of linear rows with its own bounds, answered with its root fixpoint.

The server keeps the matrix and the root bounds on the device and runs several workers, each with its own
libgbp context and CUDA stream.  Whenever a worker is free it takes *everything* queued for its kind (up to a
batch limit), merges it into one launch (one persistent node-kernel launch for node requests, one
block-diagonal instance launch for instance requests) and runs it.  Requests that arrive while other batches
are on the GPU are admitted into the next free worker's batch, so batches of different sizes overlap on the
device.  Admission is capped by an HBM budget: a batch is only formed while the bytes in flight plus its own
estimate stay below the cap; otherwise requests wait in the queue.

`PlainServer` answers the same requests one per call (gbp_propagate per request), the baseline the
served form is compared against; both must return identical results for every request.
"""
from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import gbp, instances


@dataclass
class NodeRequest:
    cols: np.ndarray
    lb: np.ndarray
    ub: np.ndarray
    t_arrive: float = 0.0


@dataclass
class InstanceRequest:
    inst: instances.Instance
    t_arrive: float = 0.0


@dataclass
class Reply:
    cutoff: bool
    cols: Optional[np.ndarray] = None   # node request: columns whose bounds moved
    lb: Optional[np.ndarray] = None     # node request: their bounds; instance request: all bounds
    ub: Optional[np.ndarray] = None
    t_done: float = 0.0
    batch: int = 0                      # requests in the launch that served it


def _node_bytes(req: NodeRequest) -> int:
    return 24 * len(req.cols) + 4096


def _inst_bytes(inst: instances.Instance) -> int:
    # CSR + CSC + per-column scratch of the plain path + bounds
    return 28 * inst.nnz + 80 * inst.n + 24 * inst.m + 4096


class PropagationServer:
    def __init__(self, matrix: instances.Instance, root_lb, root_ub, node_workers: int = 2, inst_workers: int = 2,
                 max_batch: int = 4096, hbm_cap: float = 150e9, params=None, device: int = 0,
                 node_shape=(128, 0)):
        self.matrix = matrix
        self.root_lb = np.ascontiguousarray(root_lb, dtype=np.float64)
        self.root_ub = np.ascontiguousarray(root_ub, dtype=np.float64)
        self.max_batch = max_batch
        self.hbm_cap = hbm_cap
        self.inflight = 0
        self.params = params or gbp.default_params(maxeasy=0.0)
        # one lock; each kind of request has its own condition, so that a submission wakes one worker of its kind
        self.lock = threading.Lock()
        self.ready = {"node": threading.Condition(self.lock), "inst": threading.Condition(self.lock)}
        self.queues = {"node": collections.deque(), "inst": collections.deque()}
        self.stop = False
        self.batches = []  # (kind, size, t_start, t_end)
        self.workers = []
        for kind, count in (("node", node_workers), ("inst", inst_workers)):
            for _ in range(count):
                prop = gbp.Propagator(device, params=self.params)
                if kind == "node":
                    prop.upload(matrix)
                    prop.set_batch_shape(*node_shape)
                t = threading.Thread(target=self._work, args=(kind, prop), daemon=True)
                self.workers.append((t, prop))
        for t, _ in self.workers:
            t.start()

    # ------------------------------------------------------------------ client side
    def submit(self, req) -> Future:
        fut: Future = Future()
        kind = "node" if isinstance(req, NodeRequest) else "inst"
        if not req.t_arrive:
            req.t_arrive = time.perf_counter()
        with self.lock:
            self.queues[kind].append((req, fut))
            self.ready[kind].notify()
        return fut

    def close(self):
        with self.lock:
            self.stop = True
            for cv in self.ready.values():
                cv.notify_all()
        for t, _ in self.workers:
            t.join(timeout=60)
        for _, prop in self.workers:
            prop.close()

    # ------------------------------------------------------------------ workers
    def _take(self, kind):
        """Everything queued for `kind` (up to the batch limit) that fits the HBM budget; blocks until some."""
        with self.lock:
            while True:
                if self.stop:
                    return None, 0
                q = self.queues[kind]
                batch, est = [], 0
                while q and len(batch) < self.max_batch:
                    req, fut = q[0]
                    b = _node_bytes(req) if kind == "node" else _inst_bytes(req.inst)
                    if batch and self.inflight + est + b > self.hbm_cap:
                        break
                    if not batch and self.inflight + b > self.hbm_cap and self.inflight > 0:
                        break  # wait for memory to free up
                    q.popleft()
                    batch.append((req, fut))
                    est += b
                if batch:
                    self.inflight += est
                    if q:  # more of this kind is waiting: another free worker may take it
                        self.ready[kind].notify()
                    return batch, est
                self.ready[kind].wait(timeout=0.05)

    def _release(self, est):
        with self.lock:
            self.inflight -= est
            for cv in self.ready.values():  # memory freed: waiting batches may now fit
                cv.notify_all()

    def _work(self, kind, prop):
        while True:
            batch, est = self._take(kind)
            if batch is None:
                return
            t0 = time.perf_counter()
            try:
                replies = self._run_nodes(prop, batch) if kind == "node" else self._run_instances(prop, batch)
                err = None
            except Exception as e:  # a failed launch fails its requests, the server keeps running
                replies, err = None, e
            t1 = time.perf_counter()
            self._release(est)
            self.batches.append((kind, len(batch), t0, t1))
            for k, (req, fut) in enumerate(batch):
                if err is not None:
                    fut.set_exception(err)
                else:
                    replies[k].t_done = t1
                    replies[k].batch = len(batch)
                    fut.set_result(replies[k])

    def _run_nodes(self, prop, batch):
        ks = np.array([len(r.cols) for r, _ in batch], dtype=np.int64)
        ptr = np.zeros(len(batch) + 1, dtype=np.int64)
        np.cumsum(ks, out=ptr[1:])
        col = np.concatenate([r.cols for r, _ in batch]).astype(np.int32)
        lb = np.concatenate([r.lb for r, _ in batch])
        ub = np.concatenate([r.ub for r, _ in batch])
        res = prop.propagate_nodes(self.root_lb, self.root_ub, instances.NodeBatch(ptr, col, lb, ub),
                                   out_cap=max(1024, 512 * len(batch)))
        # every node's moved columns, gathered from the packed output into node order and sorted by column
        nb = len(batch)
        live = res.cutoff[:nb] == 0
        cnt = np.where(live, res.n[:nb], 0).astype(np.int64)
        first = np.cumsum(cnt) - cnt
        idx = np.repeat(res.off[:nb] - first, cnt) + np.arange(int(cnt.sum()))
        node = np.repeat(np.arange(nb), cnt)
        c = res.col[idx]
        o = np.lexsort((c, node))
        c, l, u = c[o], res.lb[idx][o], res.ub[idx][o]
        out = []
        for k in range(nb):
            if not live[k]:
                out.append(Reply(True))
            else:
                sl = slice(first[k], first[k] + cnt[k])
                out.append(Reply(False, c[sl], l[sl], u[sl]))
        return out

    def _run_instances(self, prop, batch):
        insts = [r.inst for r, _ in batch]
        row_off, col_off = prop.upload_instances(insts)
        lb = np.concatenate([i.lb for i in insts])
        ub = np.concatenate([i.ub for i in insts])
        glb, gub, cut, res = prop.propagate_instances(lb, ub)
        return [Reply(bool(cut[k]), None, glb[col_off[k]:col_off[k + 1]].copy(), gub[col_off[k]:col_off[k + 1]].copy())
                for k in range(len(insts))]


class PlainServer:
    """One request per call, in arrival order, on one context: the baseline of the served form."""

    def __init__(self, matrix, root_lb, root_ub, params=None, device: int = 0):
        self.root_lb = np.ascontiguousarray(root_lb, dtype=np.float64)
        self.root_ub = np.ascontiguousarray(root_ub, dtype=np.float64)
        self.params = params or gbp.default_params(maxeasy=0.0)
        self.node_prop = gbp.Propagator(device, params=self.params)
        self.node_prop.upload(matrix)
        self.node_prop.set_global_bounds(self.root_lb, self.root_ub)  # a node's global domain: the root bounds
        self.inst_prop = gbp.Propagator(device, params=self.params)

    def answer(self, req):
        if isinstance(req, NodeRequest):
            lb, ub = self.root_lb.copy(), self.root_ub.copy()
            olb, oub = lb[req.cols].copy(), ub[req.cols].copy()
            if (req.lb > oub).any() or (req.ub < olb).any():
                return Reply(True)
            lb[req.cols] = np.maximum(olb, req.lb)
            ub[req.cols] = np.minimum(oub, req.ub)
            plb, pub, cut, _ = self.node_prop.propagate(lb, ub, seed=(req.cols, olb, oub))
            if cut:
                return Reply(True)
            moved = np.flatnonzero((plb != self.root_lb) | (pub != self.root_ub)).astype(np.int32)
            return Reply(False, moved, plb[moved], pub[moved])
        self.inst_prop.upload(req.inst)
        plb, pub, cut, _ = self.inst_prop.propagate(req.inst.lb, req.inst.ub)
        return Reply(bool(cut), None, plb, pub)

    def close(self):
        self.node_prop.close()
        self.inst_prop.close()


def same_reply(a: Reply, b: Reply) -> bool:
    if a.cutoff != b.cutoff:
        return False
    if a.cutoff:
        return True
    if (a.cols is None) != (b.cols is None):
        return False
    if a.cols is not None and not np.array_equal(a.cols, b.cols):
        return False
    return np.array_equal(a.lb, b.lb) and np.array_equal(a.ub, b.ub)


# ---------------------------------------------------------------------- request streams
@dataclass
class Stream:
    times: np.ndarray                # arrival offsets in seconds
    reqs: List = field(default_factory=list)


def make_stream(matrix, root_lb, root_ub, pool: List[instances.Instance], rate: float, duration: float,
                node_frac: float = 0.8, seed: int = 0) -> Stream:
    """Poisson arrivals at `rate` per second for `duration` seconds; node_frac node requests (1..64 integer
    columns fixed inside the root bounds), the rest instance requests drawn from `pool`."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    n = max(1, int(rng.poisson(rate * duration)))
    times = np.sort(rng.uniform(0.0, duration, size=n))
    isnode = rng.random(n) < node_frac
    nn = int(isnode.sum())
    nodes = instances.node_batch(matrix, root_lb, root_ub, max(nn, 1), seed=seed + 1)
    reqs, k = [], 0
    for q in range(n):
        if isnode[q]:
            sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
            reqs.append(NodeRequest(nodes.col[sl].copy(), nodes.lb[sl].copy(), nodes.ub[sl].copy()))
            k += 1
        else:
            reqs.append(InstanceRequest(pool[int(rng.integers(0, len(pool)))]))
    return Stream(times, reqs)


def _wait_until(t):
    """Wait for time t without holding the interpreter lock: a spinning client would keep the worker threads
    from running until the interpreter's switch interval (5 ms) takes the lock away from it."""
    while True:
        d = t - time.perf_counter()
        if d <= 0:
            return
        time.sleep(d if d > 2e-4 else 0)


def replay(server, stream: Stream, served: bool = True):
    """Submit the stream at its arrival times (served) or answer it one request at a time in arrival order
    (plain, which still waits for each arrival).  Returns (replies, latencies in seconds, wall seconds)."""
    t0 = time.perf_counter()
    replies, lat = [None] * len(stream.reqs), np.zeros(len(stream.reqs))
    if served:
        futs = []
        for q, req in enumerate(stream.reqs):
            due = t0 + stream.times[q]
            _wait_until(due)
            req.t_arrive = due
            futs.append(server.submit(req))
        for q, f in enumerate(futs):
            r = f.result()
            replies[q] = r
            lat[q] = r.t_done - stream.reqs[q].t_arrive
    else:
        for q, req in enumerate(stream.reqs):
            due = t0 + stream.times[q]
            _wait_until(due)
            r = server.answer(req)
            r.t_done = time.perf_counter()
            replies[q] = r
            lat[q] = r.t_done - due
    return replies, lat, time.perf_counter() - t0
