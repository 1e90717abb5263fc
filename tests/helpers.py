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


def compress_ranked(K, rep, dist, k):
    """to_compressed_chains (debruijn_chain_graph.hpp:1778-1856) restated over listranked
    nodes: sort by chain_rep_less (rep, |dist|, K), group by rep, print the representative for
    a distance-0 node and K's last base for every other one; returned like chain_set"""
    order = np.lexsort(tuple(K.T) + (np.abs(dist),) + tuple(rep.T))
    out = {}
    for i in order:
        r = tuple(int(x) for x in rep[i][::-1])
        if dist[i] == 0:
            v = 0
            for w, x in enumerate(rep[i]):
                v |= int(x) << (64 * w)
            s = "".join("ACGT"[(v >> (2 * (k - 1 - j))) & 3] for j in range(k))
        else:
            s = "ACGT"[int(K[i][0]) & 3]
        out[r] = out.get(r, "") + s
    return sorted(out.items())
