"""Counts past the limits of the node counters and of the device's entry words.

The reference keeps raw (k+2)-mer counts in a non-saturating uint32 (K2FreqType,
debruijn_graph_map.hpp:160), caps every per-k-mer sum at the count type's maximum before
thresholding (:1401-1407) and inserts with saturating uint16 arithmetic (sat_add,
debruijn_graph_node.hpp:81-85).  Three inputs drive those paths:

  * one random read repeated 70,000 times plus its reverse complement 5,000 times: every
    (k-mer, biedge) pair is seen 75,000 times, every node counter saturates at 65535;
  * a read around a 32-base reverse-complement palindrome, 70,000 times: the (k+1)-mer
    palindrome halving of k=31 runs on saturated sums;
  * 290,000 poly-A reads of 150 bases: one pair is seen 118 x 290,000 = 34,220,000 times,
    past 2^25, where the device's entry word stops counting and its exact side table takes
    over (the raw counts must still equal the reference's).

The CPU tests pin the oracle on what these inputs must give by construction; the GPU tests
compare the CUDA path with the oracle, bit for bit."""
import numpy as np
import pytest

import bruno_gb300 as bg
from oracle import oracle
from helpers import sort_k2

COMP = bytes.maketrans(b"ACGT", b"TGCA")


def rc(s: bytes) -> bytes:
    return s.translate(COMP)[::-1]


def fastq(reads) -> bytes:
    out = bytearray()
    for i, r in enumerate(reads):
        out += b"@s%d\n%s\n+\n%s\n" % (i, r, b"I" * len(r))
    return bytes(out)


def random_bases(n: int, seed: int) -> bytes:
    return bytes(np.frombuffer(b"ACGT", np.uint8)[np.random.default_rng(seed).integers(0, 4, n)])


REPEATED_READ = random_bases(120, 7)
REPEATED = fastq([REPEATED_READ] * 70_000 + [rc(REPEATED_READ)] * 5_000)

_Z = random_bases(16, 11)
PALINDROME_READ = random_bases(40, 12) + _Z + rc(_Z) + random_bases(40, 13)
PALINDROMIC = fastq([PALINDROME_READ] * 70_000)

POLY_A_READS = 290_000
POLY_A = fastq([b"A" * 150] * POLY_A_READS)

CASES = {"repeated": REPEATED, "palindromic": PALINDROMIC, "poly_a": POLY_A}
OPTIONS = {"u": (False, ()), "tl2": (True, (2,)), "tl3_hi": (True, (3, 2, 3))}


def test_oracle_repeated_read_saturates():
    """every node of the read: 90 k-mers, each counter either 0 or 65535; raw pairs 75,000"""
    for thr_on, lo in OPTIONS.values():
        r = oracle.run(REPEATED, k=31, thresholding=thr_on, thresh=bg.thresholds(lo), keep_k2=True)
        assert r["status"] == 0
        keys, counts, flags = r["nodes"]
        assert len(keys) == 120 - 31 + 1
        assert set(np.unique(counts).tolist()) <= {0, 65535}
        assert (counts[:, 8] == 65535).all()                 # self
        _, _, k2c = r["k2"]
        assert (k2c == 75_000).all() and len(k2c) == 90
        assert r["n_chains"] == 1 and r["n_chain_nodes"] == 90


def test_oracle_poly_a_counts_past_2_to_25():
    """one poly-A node in a self loop: raw counts exact in 32 bits, node counters saturated,
    and the node leaves the chains as a cycle"""
    r = oracle.run(POLY_A, k=31, thresholding=True, thresh=bg.thresholds([2]), keep_k2=True)
    keys, edges, counts = sort_k2(*r["k2"])
    assert keys.ravel().tolist() == [0, 0, 0]
    got = dict(zip(edges.tolist(), counts.tolist()))
    assert got == {0x01: POLY_A_READS, 0x11: 118 * POLY_A_READS, 0x10: POLY_A_READS}
    assert 118 * POLY_A_READS > 2 ** 25
    nk, nc, nf = r["nodes"]
    assert nk.ravel().tolist() == [0]
    assert nc[0].tolist() == [65535, 0, 0, 0, 65535, 0, 0, 0, 65535]
    assert r["n_chains"] == 0 and r["n_cycle_nodes"] == 1


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_oracle_saturation_shard_invariant(threads):
    """the restatement's outputs do not depend on its shard count (the reference's -np)"""
    for data in (PALINDROMIC, POLY_A):
        a = oracle.run(data, k=31, thresh=bg.thresholds([2]), keep_k2=True, keep_filtered=True)
        b = oracle.run(data, k=31, thresh=bg.thresholds([2]), keep_k2=True, keep_filtered=True, threads=threads)
        for n in ("nodes", "ranked", "chains"):
            for x, y in zip(a[n], b[n]):
                assert np.array_equal(x, y), n
        for x, y in zip(sort_k2(*a["k2"]), sort_k2(*b["k2"])):
            assert np.array_equal(x, y)


@pytest.mark.gpu
@pytest.mark.parametrize("opt", sorted(OPTIONS))
@pytest.mark.parametrize("case", sorted(CASES))
def test_gpu_saturation_parity(case, opt):
    from test_gpu_parity import compare, gpu_run
    thr_on, lo = OPTIONS[opt]
    thr = bg.thresholds(lo)
    data = CASES[case]
    ref = oracle.run(data, k=31, thresholding=thr_on, thresh=thr, min_update=True, threads=8, keep_k2=True,
                     keep_filtered=True)
    compare(gpu_run(data, 31, thr_on, thr, True), ref)


@pytest.mark.gpu
def test_gpu_saturation_parity_k45():
    """the same saturation on 128-bit keys (k = 45, the whole-table counting path)"""
    from test_gpu_parity import compare, gpu_run
    thr = bg.thresholds([2])
    for data in (REPEATED, POLY_A):
        ref = oracle.run(data, k=45, thresh=thr, min_update=True, threads=8, keep_k2=True, keep_filtered=True)
        compare(gpu_run(data, 45, True, thr, True), ref)
