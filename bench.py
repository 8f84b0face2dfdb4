"""Benchmark: node-fixpoints/s of linear-constraint bound propagation on one GB300.

Workload (the batched branch-and-bound node case): one shared matrix of 200,000 rows x 400,000 columns
(row lengths U{5..40}, |a| log-uniform in [1e-2, 1e2], 60 % integer columns), 4,096 node subproblems that fix
1..64 integer columns each to random values inside the root fixpoint bounds, every node propagated to its
own fixpoint.  One step = one batch of 4,096 nodes.

  value      node-fixpoints/s of the batched path, inputs resident in HBM (gbp_propagate_nodes_device)
  e2e        the same through the host-pointer C ABI (gbp_propagate_nodes): node changes and base bounds
             copied host->device and results device->host inside the timed region
  plain      the plain one-node-per-launch-sequence path (gbp_propagate with seeds), on a sample of nodes
  cpu_baseline / --impl reference   the C restatement of SCIP's propagation (oracle) on the host cores

Timing: CUDA events on the library's stream around each step, W untimed warm-up steps, L2 flushed
(256 MiB write) between timed steps, nvidia-smi clocks sampled during the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0
NNODES = 4096


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


def measured_traffic(algo_bytes, shape):
    """DRAM bytes (read + write) and FP64 warp-instructions of one k_nodes launch, from the committed ncu capture of a
    small case of the same generator (profiles/k_nodes_traffic.json), scaled to this launch by its algorithmic bytes
    (both grow with the rows, nonzeros and changes a launch processes)."""
    p = os.path.join(ROOT, "profiles", "k_nodes_traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
        scale = algo_bytes / float(d["algorithmic_bytes"])
    except Exception:
        return None, None, None
    src = {"from": "profiles/k_nodes_traffic.json", "case": d["case"], "command": d["command"],
           "scaled_by": scale, "case_launch_shape": d["launch_shape"], "this_run_shape": list(shape)}
    traffic = (int(d["dram_bytes_read"]) + int(d["dram_bytes_write"])) * scale
    fp64 = float(d["fp64_warp_inst"]) * scale if "fp64_warp_inst" in d else None
    return traffic, fp64, src


def scip_calibration():
    """SCIP 11's own speed on this workload against the port's, both on one x86 core of the build container
    (profiles/cpu_calibration_x86.json, written by oracle/calibrate.py): SCIP is not built on the GPU machine, so the
    ratio is carried over to read the port's figures as SCIP's."""
    try:
        with open(os.path.join(ROOT, "profiles", "cpu_calibration_x86.json")) as f:
            d = json.load(f)
        return {"scip_over_port": d["scip_over_port_jacobi_1core"],
                "scip_over_port_source": {"from": "profiles/cpu_calibration_x86.json", "machine": d["machine"],
                                          "scip_1core": d["scip_1core"]["value"],
                                          "port_1core": d["port_jacobi_1core"]["value"],
                                          "command": d["command"]}}
    except Exception:
        return {}


def fp64_rate():
    """The GPU's FP64 issue rate in warp-instructions/s, measured by tests/native/fp64_issue.cu
    (profiles/fp64_issue.json); None when absent."""
    try:
        with open(os.path.join(ROOT, "profiles", "fp64_issue.json")) as f:
            d = json.load(f)
        return float(d["gpu_warp_inst_per_s"]), d
    except Exception:
        return None, None


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(rows, nnz, changes, avg_col_len):
    """Bytes one propagation must move: per processed nonzero 8 (value) + 4 (column) + 16 (lb, ub gather),
    per processed row 40 (row pointer, lhs, rhs, activity outputs), per accepted change 16 (bound write)
    plus 8 per entry of the changed column's CSC list (frontier expansion)."""
    return 28.0 * nnz + 40.0 * rows + 16.0 * changes + 8.0 * changes * avg_col_len


def build_workload(seed=2, nnodes=NNODES, m=200_000, n=400_000, family="mip"):
    from scip_gb300 import instances

    if family == "gcd":
        # ranged rows and equations whose integer part shares a divisor (1 % of rows 65..200 long)
        return instances.gcd_rows(np.random.default_rng(seed), m, n, long_frac=0.01, equations=True)
    inst = instances.node_mip(seed=seed, m=m, n=n)
    return inst


class CpuArm:
    """The oracle over a bounded sample of the node batch.  plan() fixes the sample once: the first nodes of the
    batch, growing until they take a quarter of budget_s or are the whole batch, and a whole batch that takes less
    than min_wall_s is repeated until it does.  run() times one sample and returns (node-fixpoints/s, sample
    description)."""

    def __init__(self, inst, rlb, rub, nodes, par, nthreads):
        import oracle as orc

        self.o = orc.Oracle(inst)
        self.rlb, self.rub, self.nodes, self.par, self.nthreads = rlb, rub, nodes, par, nthreads
        self.sub, self.k, self.reps = None, 0, 1

    def _once(self):
        t0 = time.perf_counter()
        self.o.propagate_nodes(self.rlb, self.rub, self.sub, self.par, cap=1, nthreads=self.nthreads)
        return time.perf_counter() - t0

    def plan(self, budget_s=15.0, min_wall_s=0.0):
        from scip_gb300.instances import NodeBatch

        nodes = self.nodes
        take = 256
        while True:
            k = min(take, nodes.nnodes)
            self.sub = NodeBatch(nodes.ptr[:k + 1].copy(), nodes.col[:nodes.ptr[k]], nodes.lb[:nodes.ptr[k]],
                                 nodes.ub[:nodes.ptr[k]])
            dt = self._once()
            if dt > budget_s / 4 or k == nodes.nnodes:
                break
            take *= 4
        self.k = k
        self.reps = int(np.ceil(min_wall_s / max(dt, 1e-6))) if k == nodes.nnodes and dt < min_wall_s else 1
        return self

    def run(self):
        dt = sum(self._once() for _ in range(self.reps))
        return self.k * self.reps / dt, (f"{self.reps} x {self.k} of {self.nodes.nnodes} nodes, {self.nthreads} "
                                         f"threads, {dt:.2f} s wall")


def other_workload(args):
    """Root fixpoints of the uneven-instance batch (all instances in one block-diagonal problem) or of the large
    Zipf instance (plain path); prints one JSON line."""
    import torch
    from scip_gb300 import gbp, instances
    from scip_gb300.build import build_libgbp

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    build_libgbp()
    t0 = time.perf_counter()
    if args.workload == "uneven":
        insts = instances.uneven_batch(seed=4, count=args.instances)
        big, row_off, col_off = instances.concat_instances(insts)
        units = len(insts)
        cfg = {"workload": f"{units} distinct instances (set cover / multi-knapsack / network flow), rows log-uniform "
                           "in [1e3, 2e5], all in one block-diagonal problem, every instance to its root fixpoint",
               "rows": big.m, "cols": big.n, "nnz": big.nnz}
    elif args.workload == "root":
        big = instances.root_mip(seed=0)
        units = 1
        cfg = {"workload": "one 2,000 x 5,000 instance (row lengths 5..15, integer coefficients, 10 % ranged rows and "
                           "10 % equations), root fixpoint through the plain path", "rows": big.m, "cols": big.n,
               "nnz": big.nnz}
    else:
        big = instances.zipf_mip(seed=1)
        units = 1
        cfg = {"workload": "one 1,000,000 x 2,000,000 instance, Zipf(1.5) row lengths in [2, 5000], root fixpoint "
                           "through the plain path", "rows": big.m, "cols": big.n, "nnz": big.nnz}
    gen_s = time.perf_counter() - t0
    params = gbp.default_params(maxeasy=args.maxeasy)
    if args.hostloop:  # host-driven rounds: one launch per kernel per round (kernel-level timings, ncu launch lists)
        params.flags |= gbp.GBP_FLAG_HOSTLOOP
    prop = gbp.Propagator(0, params=params)
    t0 = time.perf_counter()
    if args.workload == "uneven":
        prop.upload_instances(insts)
    else:
        prop.upload(big)
    up_s = time.perf_counter() - t0
    d = torch.device("cuda", 0)
    lb0 = torch.from_numpy(big.lb).to(d)
    ub0 = torch.from_numpy(big.ub).to(d)
    lb, ub = lb0.clone(), ub0.clone()
    cut = torch.zeros(max(units, 1), dtype=torch.int8, device=d)
    stream = torch.cuda.ExternalStream(prop.stream())

    def step():
        if args.workload == "uneven":
            return prop.propagate_instances_device(lb, ub, cut)
        return prop.propagate_device(lb, ub)[1]

    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            lb.copy_(lb0)
            ub.copy_(ub0)
        step()
    times, res = [], None
    clocks = ClockSampler()
    clocks.start()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            lb.copy_(lb0)
            ub.copy_(ub0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        res = step()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    ms = float(np.mean(times))
    algo = algorithmic_bytes(res.rows, res.nnz, res.changes, big.nnz / max(big.n, 1))
    peak, peak_kind = measured_peak()
    line = {"metric": "node-fixpoints/sec", "value": units / (ms / 1e3), "unit": "instance-fixpoints/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": cfg, "rounds": res.rounds, "cutoffs": res.cutoff, "rows_processed": res.rows,
            "nnz_per_s": res.nnz / (ms / 1e3), "launches": res.launches, "generate_s": gen_s, "upload_s": up_s,
            "roofline": {"bound": "hbm", "achieved": algo / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": algo / (ms / 1e3) / 1e9 / peak, "traffic": None, "peak_kind": peak_kind},
            "clocks": clk}
    if args.workload == "uneven" and not args.quick:
        import oracle as orc
        from concurrent.futures import ThreadPoolExecutor

        orc.build()
        par = orc.params(args.maxeasy)
        take = insts[: max(8, len(insts) // 8)]
        t0 = time.perf_counter()
        with ThreadPoolExecutor(os.cpu_count() or 1) as ex:
            list(ex.map(lambda i: orc.Oracle(i).propagate(i.lb, i.ub, par), take))
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": len(take) / dt, "unit": "instance-fixpoints/s", "cores": os.cpu_count() or 1,
                                "kind": "port", "sample": f"{len(take)} of {len(insts)} instances, {dt:.2f} s "
                                                          "(includes the oracle's CSC build per instance)"}
    if args.workload == "root" and not args.quick:
        import oracle as orc

        orc.build()
        o = orc.Oracle(big)
        par = orc.params(args.maxeasy)
        k, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < 2.0:
            o.propagate(big.lb, big.ub, par)
            k += 1
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": k / dt, "unit": "instance-fixpoints/s", "cores": 1, "kind": "port",
                                "sample": f"{k} root fixpoints in {dt:.2f} s on one thread"}
    print(json.dumps(line))
    prop.close()


def serving_workload(args):
    """Poisson request streams (80 % node requests against the resident 200,000 x 400,000 matrix, 20 % new
    instances from the uneven-instance generator) at each rate: p50/p99 latency and throughput of the served
    (continuously batched) and of the plain one-request-per-call path, with identical replies checked."""
    from scip_gb300 import gbp, instances, serving
    from scip_gb300.build import build_libgbp

    build_libgbp()
    sys.setswitchinterval(1e-4)
    matrix = build_workload()
    params = gbp.default_params(maxeasy=args.maxeasy)
    p = gbp.Propagator(0, params=params)
    p.upload(matrix)
    rlb, rub, _, _ = p.propagate(matrix.lb, matrix.ub)
    p.close()
    pool = instances.uneven_batch(seed=41, count=24)  # the uneven-instance generator: rows log-uniform in [1e3, 2e5]
    srv = serving.PropagationServer(matrix, rlb, rub, node_workers=2, inst_workers=4, params=params,
                                    hbm_cap=150e9)
    plain = serving.PlainServer(matrix, rlb, rub, params=params)
    # warm-up: both paths once over a short stream
    warm = serving.make_stream(matrix, rlb, rub, pool, rate=2000.0, duration=0.2, seed=99)
    serving.replay(srv, warm, served=True)
    for req in warm.reqs[:20]:
        plain.answer(req)
    rows = []
    for k, rate in enumerate(float(r) for r in args.rates.split(",")):
        st = serving.make_stream(matrix, rlb, rub, pool, rate=rate, duration=args.duration, seed=k)
        replies, lat, wall = serving.replay(srv, st, served=True)
        nb = len(srv.batches)
        row = {"rate": rate, "requests": len(st.reqs), "served": {
            "throughput": len(st.reqs) / wall, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
            "p99_ms": 1e3 * float(np.percentile(lat, 99)), "wall_s": wall}}
        # the plain path on the first requests of the same stream (it saturates early)
        take = min(len(st.reqs), int(400 * args.duration) + 1)
        sub = serving.Stream(st.times[:take], st.reqs[:take])
        p_replies, p_lat, p_wall = serving.replay(plain, sub, served=False)
        same = all(serving.same_reply(replies[q], p_replies[q]) for q in range(take))
        row["plain"] = {"requests": take, "throughput": take / p_wall, "p50_ms": 1e3 * float(np.percentile(p_lat, 50)),
                        "p99_ms": 1e3 * float(np.percentile(p_lat, 99)), "identical_replies": same}
        rows.append(row)
    batches = srv.batches
    srv.close()
    plain.close()
    best = max(r["served"]["throughput"] for r in rows)
    print(json.dumps({"metric": "node-fixpoints/sec", "value": best, "unit": "requests/s", "n_gpus": 1,
                      "steps": len(rows), "warmup": 1, "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
                      "config": {"workload": "served propagation: Poisson request streams, 80 % node requests "
                                             "against the resident 200,000 x 400,000 matrix, 20 % new instances "
                                             "from the uneven-instance generator", "workers": "2 node + 4 instance",
                                 "hbm_cap_gb": 150, "duration_s": args.duration},
                      "sweep": rows, "batches": len(batches),
                      "mean_batch": float(np.mean([b[1] for b in batches])) if batches else 0.0}))


def time_served(inst, rlb, rub, nodes, params, rates=(1000, 10000, 50000), duration=0.3):
    """libgbp's serving loop (gbp_server_*, C worker threads merging node requests into batched launches): open-loop
    Poisson arrivals of single-node requests (the bench's nodes in turn) at each offered rate for `duration` seconds,
    then every reply collected.  Latency = the server's time from admitting a request to finishing its batch;
    throughput = requests / (last finish - first admission)."""
    import ctypes

    from scip_gb300 import gbp

    srv = gbp.Server(inst, rlb, rub, params=params, workers=2, max_batch=4096)
    L = srv.L
    reqs = []
    for k in range(nodes.nnodes):
        sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
        arrs = (np.ascontiguousarray(nodes.col[sl], np.int32), np.ascontiguousarray(nodes.lb[sl]),
                np.ascontiguousarray(nodes.ub[sl]))
        reqs.append((len(arrs[0]), arrs, [a.ctypes.data_as(ctypes.c_void_p) for a in arrs]))
    out = {}
    t = ctypes.c_int64()
    try:
        for rate in rates:
            rng = np.random.default_rng(np.random.PCG64(rate))
            n = int(rate * duration)
            due = np.cumsum(rng.exponential(1.0 / rate, n))
            tickets = []
            t0 = time.perf_counter()
            lag = 0.0
            for i in range(n):
                while time.perf_counter() - t0 < due[i]:
                    pass
                lag = max(lag, time.perf_counter() - t0 - due[i])
                nc, _, ptrs = reqs[i % len(reqs)]
                rc = L.gbp_server_submit(srv.h, nc, ptrs[0], ptrs[1], ptrs[2], ctypes.byref(t))
                if rc != gbp.GBP_OK:
                    raise gbp.GbpError(rc, "submit")
                tickets.append(t.value)
            sub_s = time.perf_counter() - t0
            ts, td = [], []
            for tk in tickets:
                r = srv.poll(tk)
                ts.append(r[4])
                td.append(r[5])
            ts, td = np.array(ts), np.array(td)
            lat = (td - ts) / 1e6
            out[str(rate)] = {"offered_req_s": rate, "requests": n, "submitted_req_s": n / sub_s,
                              "max_submit_lag_ms": 1e3 * lag,
                              "throughput_req_s": n / ((td.max() - ts.min()) / 1e9),
                              "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}
        out["stats"] = srv.stats()
        out["call"] = "gbp_server_submit / gbp_server_poll (2 worker threads, batched node launches)"
    finally:
        srv.close()
    return out


def time_served_mix(inst, rlb, rub, nodes, params, rates=(1000, 10000, 50000), duration=0.2, node_frac=0.8,
                    inst_workers=4):
    """The served mix through libgbp's C serving loop: open-loop Poisson arrivals, node_frac of them single-node
    requests (the bench's nodes in turn) and the rest new instances drawn from 24 instances of the uneven-instance
    generator (rows log-uniform in [1e3, 2e5]), at each offered rate for `duration` seconds.  Two node workers merge
    node requests into batched k_nodes launches; inst_workers instance workers upload queued instances as one
    block-diagonal problem each and propagate it in one launch.  Instance arrays are borrowed by the server (no host copy), so each
    instance request costs its upload: host-to-device bytes bound the instance side.  Latency = the server's time
    from admitting a request to finishing its batch, per kind and overall."""
    import ctypes

    from scip_gb300 import gbp, instances

    pool = instances.uneven_batch(seed=41, count=24)
    parts = []
    for p in pool:
        arrs = [np.ascontiguousarray(a, dtype=d) for a, d in ((p.rowptr, np.int64), (p.colidx, np.int32),
                                                             (p.vals, np.float64), (p.lhs, np.float64),
                                                             (p.rhs, np.float64), (p.isint, np.int8),
                                                             (p.lb, np.float64), (p.ub, np.float64))]
        parts.append((p.m, p.n, arrs, [a.ctypes.data_as(ctypes.c_void_p) for a in arrs],
                      sum(a.nbytes for a in arrs)))
    node_reqs = []
    for k in range(nodes.nnodes):
        sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
        arrs = (np.ascontiguousarray(nodes.col[sl], np.int32), np.ascontiguousarray(nodes.lb[sl]),
                np.ascontiguousarray(nodes.ub[sl]))
        node_reqs.append((len(arrs[0]), arrs, [a.ctypes.data_as(ctypes.c_void_p) for a in arrs]))
    cap = max(max(p.n for p in pool), inst.n)
    oc, ol, ou = np.empty(cap, np.int32), np.empty(cap), np.empty(cap)
    ocp, olp, oup = (a.ctypes.data_as(ctypes.c_void_p) for a in (oc, ol, ou))
    srv = gbp.Server(inst, rlb, rub, params=params, workers=2, inst_workers=inst_workers, max_batch=4096)
    L = srv.L
    out = {}
    t = ctypes.c_int64()
    cut, nout, ts, td = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    try:
        # warm-up: every pool instance once, so that the instance workers' contexts hold a first allocation
        warm = []
        for m_, n_, _, ptrs, _ in parts:
            if L.gbp_server_submit_instance(srv.h, m_, n_, *ptrs, ctypes.byref(t)) != gbp.GBP_OK:
                raise gbp.GbpError(gbp.GBP_ERR_INVALID, "warm-up submit")
            warm.append(t.value)
        for tk in warm:
            L.gbp_server_poll(srv.h, tk, -1, ctypes.byref(cut), cap, ctypes.byref(nout), ocp, olp, oup, None, None)
        for rate in rates:
            rng = np.random.default_rng(np.random.PCG64(rate + 7))
            n = int(rate * duration)
            due = np.cumsum(rng.exponential(1.0 / rate, n))
            isnode = rng.random(n) < node_frac
            pick = rng.integers(0, len(parts), n)
            tickets, h2d = [], 0
            t0 = time.perf_counter()
            lag = 0.0
            for i in range(n):
                while time.perf_counter() - t0 < due[i]:
                    pass
                lag = max(lag, time.perf_counter() - t0 - due[i])
                if isnode[i]:
                    nc, _, ptrs = node_reqs[i % len(node_reqs)]
                    rc = L.gbp_server_submit(srv.h, nc, ptrs[0], ptrs[1], ptrs[2], ctypes.byref(t))
                else:
                    m_, n_, _, ptrs, nbytes = parts[pick[i]]
                    rc = L.gbp_server_submit_instance(srv.h, m_, n_, *ptrs, ctypes.byref(t))
                    h2d += nbytes
                if rc != gbp.GBP_OK:
                    raise gbp.GbpError(rc, "submit")
                tickets.append(t.value)
            sub_s = time.perf_counter() - t0
            tsa, tda, errs = np.zeros(n, np.int64), np.zeros(n, np.int64), 0
            for q, tk in enumerate(tickets):
                rc = L.gbp_server_poll(srv.h, tk, -1, ctypes.byref(cut), cap, ctypes.byref(nout), ocp, olp, oup,
                                       ctypes.byref(ts), ctypes.byref(td))
                errs += rc not in (gbp.GBP_OK, gbp.GBP_ERR_LIMIT)
                tsa[q], tda[q] = ts.value, td.value
            lat = (tda - tsa) / 1e6
            wall = (tda.max() - tsa.min()) / 1e9
            row = {"offered_req_s": rate, "requests": n, "instance_requests": int((~isnode).sum()),
                   "submitted_req_s": n / sub_s, "max_submit_lag_ms": 1e3 * lag, "errors": errs,
                   "throughput_req_s": n / wall, "p50_ms": float(np.percentile(lat, 50)),
                   "p99_ms": float(np.percentile(lat, 99)), "instance_h2d_gb_s": h2d / wall / 1e9}
            for kind, sel in (("node", isnode), ("instance", ~isnode)):
                if sel.any():
                    row[kind] = {"p50_ms": float(np.percentile(lat[sel], 50)),
                                 "p99_ms": float(np.percentile(lat[sel], 99)),
                                 "served_req_s": int(sel.sum()) / ((tda[sel].max() - tsa[sel].min()) / 1e9)}
            out[str(rate)] = row
        out["stats"] = srv.stats()
        out["call"] = ("gbp_server_submit / gbp_server_submit_instance / gbp_server_poll (2 node + "
                       f"{inst_workers} instance worker threads)")
        out["mix"] = f"{node_frac:.0%} node requests, the rest instances of the uneven-instance generator " \
                     f"({sum(p.m for p in pool) // len(pool):,} rows and {sum(p.nnz for p in pool) // len(pool):,} " \
                     "nonzeros on average)"
    finally:
        srv.close()
    return out


def time_scip_order(args, inst, rlb, rub, nodes, N, dev, flush, world, seed):
    """Node-fixpoints/s of the batched nodes in SCIP's own order (GBP_FLAG_SCIPORDER), inputs resident in HBM, CUDA
    events around each step, the L2 flushed between steps.  On the default instance the nodes start from SCIP's own
    root fixpoint with the rows in SCIP's orders (the compact base in tests/golden/workload, whose 4,096 nodes equal
    SCIP's results); otherwise from the same root as the Jacobi arm, with the rows in the order consdataCompVarProp
    sorts them into on it."""
    import torch
    from scip_gb300 import gbp, instances

    if args.ranged:
        return None
    base = instances.pinned_node_base(inst, os.path.join(ROOT, "tests", "golden", "workload", "node_workload_base.npz"))
    if base is not None:
        rlb, rub, order = base
        nodes = instances.node_batch(inst, rlb, rub, N, seed=seed)
        workload = (f"SCIP's root fixpoint and row orders of this instance (tests/golden/workload/node_workload_base.npz),"
                    f" {N} nodes drawn from that root (seed {seed}); at 4,096 nodes, seed 3, every node's result "
                    f"equals SCIP's (tests/test_seq_gpu.py)")
    else:
        order = instances.scip_row_order(inst, rlb, rub, instances.scip_var_index(inst.isint, inst.lb, inst.ub))
        workload = "the Jacobi arm's root fixpoint and nodes; rows sorted as consdataCompVarProp sorts them on it"
    p = gbp.Propagator(dev, params=gbp.default_params(maxeasy=args.maxeasy, scip_order=True))
    p.upload(instances.in_order(inst, order))
    d = torch.device("cuda", dev)
    t = {k: torch.from_numpy(v).to(d) for k, v in (("lb", rlb), ("ub", rub), ("ptr", nodes.ptr), ("col", nodes.col),
                                                 ("nlb", nodes.lb), ("nub", nodes.ub))}
    cap = 256 * N
    out = {"cutoff": torch.zeros(N, dtype=torch.int8, device=d), "rounds": torch.zeros(N, dtype=torch.int32, device=d),
           "off": torch.zeros(N, dtype=torch.int64, device=d), "n": torch.zeros(N, dtype=torch.int32, device=d),
           "col": torch.zeros(cap, dtype=torch.int32, device=d), "lb": torch.zeros(cap, dtype=torch.float64, device=d),
           "ub": torch.zeros(cap, dtype=torch.float64, device=d)}
    stream = torch.cuda.ExternalStream(p.stream())

    def step():
        return p.propagate_nodes_device(t["lb"], t["ub"], N, t["ptr"], t["col"], t["nlb"], t["nub"], out, cap)

    for _ in range(args.warmup):
        step()
    steps = max(3, min(args.steps, 50))
    evs, stats = [], []
    torch.cuda.synchronize()
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        res = step()
        e1.record(stream)
        evs.append((e0, e1))
        stats.append(res.asdict())
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
    p.close()
    st = stats[-1]
    from scip_gb300 import replicas

    ms = replicas.max_over_ranks(ms, device=d)
    return {"value": replicas.aggregate_rate(N, world, ms), "unit": "node-fixpoints/s", "ms_per_step": ms, "steps": steps,
            "kernel_ms": float(np.mean([x["kernel_ms"] for x in stats])), "rows_processed": st["rows"],
            "entries_visited": st["candidates"], "changes": st["changes"], "nodes_cut_off": st["cutoff"],
            "max_rounds": st["rounds"], "gpu_launches": int(sum(x["launches"] for x in stats)),
            "call": "gbp_propagate_nodes_device with GBP_FLAG_SCIPORDER (SCIP's own order; integer bounds and "
                    "cutoffs equal SCIP's)", "workload": workload}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nodes", type=int, default=NNODES)
    ap.add_argument("--maxeasy", type=float, default=0.0)
    ap.add_argument("--quick", action="store_true", help="skip the plain-path and CPU arms (profiling runs)")
    ap.add_argument("--shape", default="", help="threads_per_node,ctas_per_sm instead of autotuning (e.g. 128,0)")
    ap.add_argument("--workload", default="nodes", choices=["nodes", "uneven", "zipf", "root", "serving"],
                    help="nodes: batched B&B nodes (headline); uneven: 512 distinct instances in one problem; "
                         "zipf: one 1M x 2M instance through the plain path; root: the 2,000 x 5,000 instance "
                         "through the plain path")
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--family", default="mip", choices=["mip", "gcd"],
                    help="nodes workload matrix: mip (log-uniform coefficients) or gcd (ranged rows sharing a divisor)")
    ap.add_argument("--ranged", action="store_true", help="ranged-row propagation on (GBP_FLAG_RANGEDROW)")
    ap.add_argument("--hostloop", action="store_true",
                    help="root/zipf/uneven: host-driven rounds (GBP_FLAG_HOSTLOOP) instead of the device loop")
    ap.add_argument("--rows", type=int, default=200_000,
                    help="nodes workload: rows of the matrix (columns = 2 x rows); smaller for profiling captures")
    ap.add_argument("--rates", default="1000,5000,10000,20000,50000", help="serving: arrival rates (req/s)")
    ap.add_argument("--duration", type=float, default=1.0, help="serving: seconds of arrivals per rate")
    args = ap.parse_args()
    if args.workload == "serving":
        return serving_workload(args)
    if args.workload != "nodes":
        return other_workload(args)

    from scip_gb300 import replicas

    rank, world, local_rank = replicas.rank_env()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from scip_gb300 import instances

    size = f"{args.rows:,} x {2 * args.rows:,}"
    config = {"workload": f"batched B&B nodes: {size} rows/cols, ~{22.5 * args.rows / 1e6:.2f}M nnz, {args.nodes:,} nodes fixing 1-64 "
                          "integer columns each, every node to fixpoint" if args.family == "mip" else
                          f"batched B&B nodes: {size} gcd rows (3..8 entries, 1 % 65..200; half equations), "
                          f"{args.nodes:,} nodes fixing 1-64 integer columns each, every node to fixpoint",
              "ranged_rows": bool(args.ranged),
              "rows": args.rows, "cols": 2 * args.rows, "nodes_per_step": args.nodes, "rule": "residual (maxeasyactivitydelta="
              f"{args.maxeasy:g})", "l2": "flushed between timed steps (256 MiB write)",
              "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        import oracle as orc

        orc.build()
        inst = build_workload(family=args.family, m=args.rows, n=2 * args.rows)
        o = orc.Oracle(inst)
        par = orc.params(args.maxeasy, ranged=args.ranged)
        rlb, rub, _ = o.propagate(inst.lb, inst.ub, par)
        nodes = instances.node_batch(inst, rlb, rub, args.nodes, seed=3)
        threads = os.cpu_count() or 1
        # each step a bounded sample, sized so that the whole run takes a minute or two
        per_step = min(1.0, max(0.05, 60.0 / max(args.steps, 1)))
        arm = CpuArm(inst, rlb, rub, nodes, par, threads).plan(budget_s=4.0 * per_step, min_wall_s=per_step)
        for _ in range(args.warmup):
            arm.run()
        rates = []
        sample = ""
        for _ in range(args.steps):
            r, sample = arm.run()
            rates.append(r)
        v = float(np.mean(rates))
        print(json.dumps({"impl": "reference", "metric": "node-fixpoints/sec", "value": v, "unit": "node-fixpoints/s",
                          "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": 1e3 * args.nodes / v, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
                          "config": config,
                          "cpu_baseline": dict({"value": v, "unit": "node-fixpoints/s", "cores": threads,
                                                "kind": "port", "sample": sample}, **scip_calibration()),
                          "e2e": {"value": v, "unit": "node-fixpoints/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return

    import torch
    from scip_gb300 import gbp
    from scip_gb300.build import build_libgbp

    build_libgbp()
    if world > 1:
        torch.distributed.init_process_group("nccl")
    dev = local_rank
    torch.cuda.set_device(dev)

    inst = build_workload(family=args.family, m=args.rows, n=2 * args.rows)
    prop = gbp.Propagator(dev, params=gbp.default_params(maxeasy=args.maxeasy, ranged=args.ranged))
    prop.upload(inst)
    rlb, rub, rcut, rres = prop.propagate(inst.lb, inst.ub)
    nodes = instances.node_batch(inst, rlb, rub, args.nodes, seed=replicas.node_seed(3, rank))
    N = nodes.nnodes
    avg_col_len = inst.nnz / inst.n

    stream = torch.cuda.ExternalStream(prop.stream())
    d = torch.device("cuda", dev)
    t_lb = torch.from_numpy(rlb).to(d)
    t_ub = torch.from_numpy(rub).to(d)
    t_ptr = torch.from_numpy(nodes.ptr).to(d)
    t_col = torch.from_numpy(nodes.col).to(d)
    t_nlb = torch.from_numpy(nodes.lb).to(d)
    t_nub = torch.from_numpy(nodes.ub).to(d)
    out_cap = 256 * N
    out = {"cutoff": torch.zeros(N, dtype=torch.int8, device=d), "rounds": torch.zeros(N, dtype=torch.int32, device=d),
           "off": torch.zeros(N, dtype=torch.int64, device=d), "n": torch.zeros(N, dtype=torch.int32, device=d),
           "col": torch.zeros(out_cap, dtype=torch.int32, device=d), "lb": torch.zeros(out_cap, dtype=torch.float64, device=d),
           "ub": torch.zeros(out_cap, dtype=torch.float64, device=d)}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=d)
    torch.cuda.synchronize()

    def step():
        return prop.propagate_nodes_device(t_lb, t_ub, N, t_ptr, t_col, t_nlb, t_nub, out, out_cap)

    from scip_gb300 import autotune

    tune_log = []
    if args.shape:
        shape = tuple(int(x) for x in args.shape.split(","))
        prop.set_batch_shape(*shape)
    else:
        shape = autotune.tune_nodes(prop, step, ("nodes", inst.m, inst.n, inst.nnz, N), log=tune_log)
    config["launch_shape"] = {"threads_per_node": shape[0], "ctas_per_sm": shape[1], "tuned_over": tune_log}

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler()
    clocks.start()
    evs = []
    stats = []
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        res = step()
        e1.record(stream)
        evs.append((e0, e1))
        stats.append(res.asdict())
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms = float(np.mean(step_ms))
    ms = replicas.max_over_ranks(ms, device=d)  # the slowest replica sets the step time
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    value = replicas.aggregate_rate(N, world, ms)
    kern_ms = float(np.mean([s["kernel_ms"] for s in stats]))
    rows = stats[-1]["rows"]
    nnz = stats[-1]["nnz"]
    changes = stats[-1]["changes"]
    algo = algorithmic_bytes(rows, nnz, changes, avg_col_len)
    peak, peak_kind = measured_peak()
    achieved = algo / (ms / 1e3) / 1e9
    cutoffs = stats[-1]["cutoff"]
    traffic, fp64_inst, traffic_src = (measured_traffic(algo, shape) if args.family == "mip" and not args.ranged
                                       else (None, None, None))
    rate, _ = fp64_rate()
    fp64_issue = None
    if fp64_inst is not None and rate is not None:
        ach = fp64_inst / (kern_ms / 1e3)
        fp64_issue = {"achieved": ach, "peak": rate, "unit": "FP64 warp-instructions/s", "frac": ach / rate,
                      "fp64_warp_inst_per_launch": fp64_inst,
                      "peak_source": "profiles/fp64_issue.json (tests/native/fp64_issue.cu)"}

    # the stated generator cuts off about 0.5 % of the nodes; the workload's stated rate is about 15 %: the same
    # step on nodes of the generator's tight-row option (instances.node_batch, tight=0.15), same launch shape
    infeasible15 = None
    if args.family == "mip" and not args.ranged:
        nt = instances.node_batch(inst, rlb, rub, N, seed=replicas.node_seed(3, rank), tight=0.15)
        tt = [torch.from_numpy(a).to(d) for a in (nt.ptr, nt.col, nt.lb, nt.ub)]
        for _ in range(args.warmup):
            prop.propagate_nodes_device(t_lb, t_ub, N, tt[0], tt[1], tt[2], tt[3], out, out_cap)
        tevs, tstats = [], []
        torch.cuda.synchronize()
        for _ in range(max(3, min(args.steps, 50))):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            r_t = prop.propagate_nodes_device(t_lb, t_ub, N, tt[0], tt[1], tt[2], tt[3], out, out_cap)
            e1.record(stream)
            tevs.append((e0, e1))
            tstats.append(r_t.asdict())
        torch.cuda.synchronize()
        tms = replicas.max_over_ranks(float(np.mean([a.elapsed_time(b) for a, b in tevs])), device=d)
        infeasible15 = {"value": replicas.aggregate_rate(N, world, tms), "unit": "node-fixpoints/s", "ms_per_step": tms,
                        "steps": len(tevs), "nodes_cut_off": int(tstats[-1]["cutoff"]),
                        "rows_processed": int(tstats[-1]["rows"]),
                        "generator": "instances.node_batch(..., tight=0.15): 15 % of the nodes dive one row past "
                                     "its right-hand side first"}

    # served form: single-node requests through libgbp's C serving loop at 1k, 10k and 50k req/s offered
    served = None
    if not args.ranged and world == 1:
        served = time_served(inst, rlb, rub, nodes, gbp.default_params(maxeasy=args.maxeasy))
        # the 80 % node / 20 % instance mix through the same loop
        try:
            served["mix"] = time_served_mix(inst, rlb, rub, nodes, gbp.default_params(maxeasy=args.maxeasy))
        except gbp.GbpError as e:
            served["mix"] = {"error": str(e)}

    # the same nodes in SCIP's own order (GBP_FLAG_SCIPORDER): rows uploaded in the order SCIP sorts them into on the
    # base domain, device-resident inputs, the same timing
    scip_order = time_scip_order(args, inst, rlb, rub, nodes, N, dev, flush, world, seed=replicas.node_seed(3, rank))

    # e2e through the host-pointer C ABI (pinned host buffers), copies inside the timed region
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()
    h_lb, h_ub = pin(rlb), pin(rub)
    hn = instances.NodeBatch(pin(nodes.ptr), pin(nodes.col), pin(nodes.lb), pin(nodes.ub))
    tdt = {np.dtype(np.int8): torch.int8, np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64,
           np.dtype(np.float64): torch.float64}
    # result buffers allocated once, pinned, as a caller of the C ABI keeps them
    h_out = gbp.Propagator.node_outputs(N, out_cap, lambda k, dt: torch.empty(k, dtype=tdt[np.dtype(dt)],
                                                                              pin_memory=True).numpy())
    e2e_ms = []
    r_host = None
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r_host = prop.propagate_nodes(h_lb, h_ub, hn, out_cap=out_cap, out=h_out)
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_ms.append(1e3 * (t1 - t0))
    e2e_v = replicas.aggregate_rate(N, world, replicas.max_over_ranks(float(np.mean(e2e_ms)), device=d))
    h2d = 16 * inst.n + 8 * (N + 1) + 20 * len(nodes.col)
    used = int(r_host.n[r_host.n > 0].sum())
    d2h = N * (1 + 4 + 8 + 4) + 20 * used

    # plain path: the same nodes one at a time through the seeded single-problem call
    plain_nodes = min(8 if args.quick else 128, N)
    prop.set_global_bounds(rlb, rub)  # a node's global domain: the root fixpoint
    t0 = time.perf_counter()
    for k in range(plain_nodes):
        lb, ub = rlb.copy(), rub.copy()
        sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
        cols = nodes.col[sl]
        olb, oub = lb[cols].copy(), ub[cols].copy()
        lb[cols] = np.maximum(lb[cols], nodes.lb[sl])
        ub[cols] = np.minimum(ub[cols], nodes.ub[sl])
        prop.propagate(lb, ub, seed=(cols, olb, oub))
    plain_v = plain_nodes / (time.perf_counter() - t0)
    # the same nodes through the sparse plain call: the bounds stay on the device, each call sends the previous
    # node's columns back to the root bounds plus the node's own changes and gets back the columns that moved
    prop.set_bounds(rlb, rub)
    dirty = np.zeros(0, np.int32)
    t0 = time.perf_counter()
    for k in range(plain_nodes):
        sl = slice(nodes.ptr[k], nodes.ptr[k + 1])
        cols = np.union1d(dirty, nodes.col[sl]).astype(np.int32)
        nlb, nub = rlb[cols].copy(), rub[cols].copy()
        at = np.searchsorted(cols, nodes.col[sl])
        nlb[at] = np.maximum(nlb[at], nodes.lb[sl])
        nub[at] = np.minimum(nub[at], nodes.ub[sl])
        cut, moved, _, _, _ = prop.propagate_changes(cols, nlb, nub, seed=(rlb[cols], rub[cols]))
        dirty = nodes.col[sl] if cut else np.union1d(nodes.col[sl], moved)
    sparse_v = plain_nodes / (time.perf_counter() - t0)
    prop.set_global_bounds(None)

    line = {"metric": "node-fixpoints/sec", "value": value, "unit": "node-fixpoints/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": config,
            "e2e": {"value": e2e_v, "unit": "node-fixpoints/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(sum(st["launches"] for st in stats)),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "traffic_source": traffic_src, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_step": algo, "kernel": "k_nodes", "fp64_issue": fp64_issue},
            "clocks": clk,
            "nnz_per_s": nnz / (ms / 1e3), "kernel_ms": kern_ms, "wall_s": wall,
            "nodes_cut_off": int(cutoffs), "max_rounds": int(stats[-1]["rounds"]),
            "plain_sparse": {"value": sparse_v, "unit": "node-fixpoints/s", "sample_nodes": plain_nodes,
                             "call": "gbp_propagate_changes (bounds resident, changed columns only)"},
            "plain": {"value": plain_v, "unit": "node-fixpoints/s", "sample_nodes": plain_nodes,
                      "root_ms": rres.kernel_ms, "root_rounds": rres.rounds},
            "scip_order": scip_order,
            "infeasible_15pct": infeasible15,
            "served": served,
            }
    if rank == 0:
        if not args.quick:
            import oracle as orc

            orc.build()
            par = orc.params(args.maxeasy, ranged=args.ranged)
            cpu_v, sample = CpuArm(inst, rlb, rub, nodes, par, os.cpu_count() or 1).plan(min_wall_s=1.0).run()
            one_v, one_sample = CpuArm(inst, rlb, rub, nodes, par, 1).plan(budget_s=8.0).run()
            line["cpu_baseline"] = {"value": cpu_v, "unit": "node-fixpoints/s", "cores": os.cpu_count() or 1,
                                    "kind": "port", "sample": sample,
                                    "one_core": {"value": one_v, "sample": one_sample}}
            line["cpu_baseline"].update(scip_calibration())
            if scip_order is not None:
                # the oracle's restatement of SCIP's order on the arm's nodes (SCIP's root and orders), all host cores
                base = instances.pinned_node_base(inst, os.path.join(ROOT, "tests", "golden", "workload",
                                                                     "node_workload_base.npz"))
                if base is not None:
                    blb, bub, border = base
                    bnodes = instances.node_batch(inst, blb, bub, N, seed=replicas.node_seed(3, rank))
                    so = orc.Oracle(instances.in_order(inst, border))
                    t0 = time.perf_counter()
                    so.propagate_nodes(blb, bub, bnodes, par, cap=1, nthreads=os.cpu_count() or 1, seq=True)
                    dt = time.perf_counter() - t0
                    scip_order["cpu_baseline"] = {"value": N / dt, "unit": "node-fixpoints/s",
                                                  "cores": os.cpu_count() or 1, "kind": "port",
                                                  "sample": f"all {N} nodes once, {dt:.2f} s wall"}
        print(json.dumps(line))
    prop.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
