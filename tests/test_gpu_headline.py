"""Bit-exact parity at the benchmarked configuration itself: the plain-scale workload (50 Mbp
genome + 2% repeats, 10M x 150 bp reads at 30x, 0.5% substitutions, k = 31, -T -L 3,
list_rank_min_update), built on the GPU through one bruno_build_and_compact call and compared
with the oracle run on every host thread.  This is the configuration whose table geometry the
smaller parity cases never reach: 2^18 partitions of the k-mer table, 10 split bits per hash
bucket, 1024 partitions per bucket in the record split."""
import os

import pytest

import bruno_gb300 as bg
from bruno_gb300 import synth
from oracle import oracle
from helpers import assert_same, chain_set, sort_k2, sort_nodes, sort_ranked

pytestmark = pytest.mark.gpu


def test_plain_scale_parity():
    w = synth.WORKLOADS["plain-scale"]
    fq = synth.make_fastq(w)
    thr = bg.thresholds(w.lower)
    g = bg.Graph(k=w.k, thresholding=True, thresh=thr, min_update=True, keep_filtered=True)
    try:
        g.build_and_compact(fq)
        s = g.sizes()
        gpu = dict(filtered=sort_k2(*g.filtered()), nodes=sort_nodes(*g.nodes()), ranked=sort_ranked(*g.ranked()),
                   chains=chain_set(*g.chains()), chain_edges=g.chain_edges())
    finally:
        g.close()
    # the partition geometry of the benchmark ran: 2^18 shared-memory partitions after the split
    assert s["table_partitions"] == 1 << 18, s["table_partitions"]
    assert s["n_instances"] == w.n_reads * (w.read_len - w.k + 1)
    ref = oracle.run(fq, k=w.k, thresholding=True, thresh=thr, min_update=True, threads=os.cpu_count() or 1,
                     keep_filtered=True)
    assert ref["status"] == 0
    for n in ("n_reads", "n_reads_used", "n_instances", "n_k2", "n_nodes", "n_branch", "n_chain_nodes", "iterations",
              "n_cycle_nodes", "n_isolated", "n_ranked", "n_chains"):
        assert s[n] == ref[n], (n, s[n], ref[n])
    assert s["filter_flag_hist"] == ref["filter_flag_hist"]
    assert_same(gpu["filtered"], sort_k2(*ref["filtered"]), "filtered k2 entries")
    assert_same(gpu["nodes"], ref["nodes"], "graph nodes")
    assert_same(gpu["ranked"], ref["ranked"], "listranked chain nodes")
    assert gpu["chains"] == chain_set(*ref["chains"]), "compacted chains"
    assert_same(gpu["chain_edges"], ref["chain_edges"], "chain end edges")
    assert s["n_chain_chars"] == int(ref["chains"][1][-1])
