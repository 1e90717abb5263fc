"""Shared comparison helpers: results are compared after sorting, as the reference's own
integration scripts do (hash-table order is not part of the contract)."""
from __future__ import annotations

import numpy as np


def sort_k2(keys, edges, counts):
    """by (k-mer, edge, count): after trimming, two filtered entries of one k-mer can share
    an edge byte, so the count breaks the tie"""
    order = np.lexsort((counts, edges) + tuple(keys.T))
    return keys[order], edges[order], counts[order]


def sort_nodes(keys, counts, flags):
    order = np.lexsort(tuple(keys.T))
    return keys[order], counts[order], flags[order]


def sort_ranked(K, rep, dist):
    order = np.lexsort(tuple(K.T))
    return K[order], rep[order], dist[order]


def chain_set(reps, offs, chars):
    b = chars.tobytes() if hasattr(chars, "tobytes") else bytes(chars)
    return sorted((tuple(int(x) for x in reps[i][::-1]), b[int(offs[i]):int(offs[i + 1])].decode())
                  for i in range(len(reps)))


def assert_same(a, b, what):
    for x, y in zip(a, b):
        assert x.shape == y.shape, f"{what}: shape {x.shape} vs {y.shape}"
        if not np.array_equal(x, y):
            bad = np.nonzero(np.any((x != y).reshape(len(x), -1), axis=1))[0]
            raise AssertionError(f"{what}: {len(bad)} rows differ, first at {bad[:5]}")
