"""Autotuner of the batched form's table shape.

Three knobs decide how the fused pass counts: the table load factor (``max_load``: slots per
distinct (k-mer, biedge) estimate), the largest shared-memory partition region (``part_slots``,
which also bounds every linear probe run) and the counting block's threads (``count_threads``).
None of them changes a result -- every build stays exact -- only the time.  The tuner builds a
probe subset of the samples once per candidate on the GPU, keeps the fastest, and caches the
choice under the batch's shape: a histogram of the samples' FASTQ sizes in powers of two, so a
later batch of the same shape reuses it.
"""
from __future__ import annotations

import itertools
import math
import time
from dataclasses import replace

GRID = {"max_load": (0.4, 0.5, 0.65), "part_slots": (1536, 3072), "count_threads": (256, 512, 1024)}

_cache: dict = {}


def shape_key(sizes, config) -> tuple:
    """the batch's shape: sample sizes binned by powers of two, with k and the thresholds"""
    bins: dict = {}
    for n in sizes:
        b = int(math.log2(max(1, n)))
        bins[b] = bins.get(b, 0) + 1
    return (config.k, tuple(config.thresh), config.thresholding, tuple(sorted(bins.items())))


def tune_batch(config, samples, grid=None, repeats: int = 2):
    """Times bruno_build_samples over `samples` (a probe subset of a batch) for every point of
    the grid; returns (best config, {point: graphs per second}).  Cached by shape_key."""
    from . import Graph
    grid = grid or GRID
    sizes = [len(x) if isinstance(x, (bytes, bytearray)) else int(getattr(x, "nbytes", len(x))) for x in samples]
    key = shape_key(sizes, config)
    if key in _cache:
        return _cache[key]
    results = {}
    best, best_rate = config, -1.0
    names = list(grid)
    for point in itertools.product(*(grid[n] for n in names)):
        cfg = replace(config, **dict(zip(names, point)))
        g = Graph(cfg)
        try:
            g.build_samples(samples)                 # warm-up: allocations, module load
            t = []
            for _ in range(repeats):
                t0 = time.perf_counter()
                g.build_samples(samples)
                t.append(time.perf_counter() - t0)
        finally:
            g.close()
        rate = len(samples) / min(t)
        results[point] = rate
        if rate > best_rate:
            best, best_rate = cfg, rate
    _cache[key] = (best, {",".join(f"{n}={v}" for n, v in zip(names, p)): r for p, r in results.items()})
    return _cache[key]
