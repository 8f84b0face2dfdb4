"""Autotuner for the batched propagation kernel's launch shape.

The shape is (threads working on one node, register budget of the compiled kernel variant given as resident
CTAs per SM).  Row-to-thread mapping inside a CTA is
fixed by the summation order (one thread per row of up to 64 entries, one warp per longer row), so the tuner
only changes how many nodes run at once and how wide each node's CTA is -- choices that never change results.
Results are cached per problem shape for the process.
"""
from __future__ import annotations

import time
from typing import Dict, Tuple

SHAPES = [(32, 16), (32, 24), (64, 8), (64, 12), (128, 4), (128, 6), (256, 2)]

_cache: Dict[Tuple, Tuple[int, int]] = {}


def tune_nodes(prop, run_batch, key, shapes=SHAPES, reps=2, log=None) -> Tuple[int, int]:
    """Time `run_batch()` (one batched call returning a GbpResult) for every shape and keep the fastest.

    key: hashable description of the workload (sizes); a cached choice is reused."""
    if key in _cache:
        prop.set_batch_shape(*_cache[key])
        return _cache[key]
    best, best_ms = None, float("inf")
    for shape in shapes:
        prop.set_batch_shape(*shape)
        run_batch()  # allocates the slots of this shape, warms caches
        ms = min(run_batch().kernel_ms for _ in range(reps))
        if log is not None:
            log.append({"threads_per_node": shape[0], "ctas_per_sm": shape[1], "ms": ms})
        if ms < best_ms:
            best, best_ms = shape, ms
    prop.set_batch_shape(*best)
    _cache[key] = best
    return best
