"""The batched form (bruno_build_samples): many samples of uneven size built in one pass of
every kernel, each counted into hash-table partitions of its own.  Every sample's results must be
exactly those of the plain path run on that sample alone (bruno_build_and_compact), and so the
oracle's: sizes, graph nodes, listranked nodes and compacted chains, bit for bit after sorting."""
import numpy as np
import pytest

import bruno_gb300 as bg
from bruno_gb300 import synth
from oracle import oracle
from conftest import fixture_bytes
from helpers import assert_same, chain_set, sort_nodes, sort_ranked

pytestmark = pytest.mark.gpu

SIZE_KEYS = ("n_reads", "n_reads_used", "n_instances", "n_k2", "n_nodes", "n_branch", "n_chain_nodes", "iterations",
             "n_cycle_nodes", "n_isolated", "n_ranked", "n_chains", "n_chain_chars")


def plain(data, **cfg):
    g = bg.Graph(**cfg)
    try:
        g.build_and_compact(data)
        return dict(sizes=g.sizes(), nodes=sort_nodes(*g.nodes()), ranked=sort_ranked(*g.ranked()),
                    chains=chain_set(*g.chains()))
    finally:
        g.close()


def batch(samples, **cfg):
    g = bg.Graph(**cfg)
    try:
        g.build_samples(samples)
        assert g.sample_count() == len(samples)
        out = [dict(sizes=g.sample_sizes(i), nodes=sort_nodes(*g.sample_nodes(i)),
                    ranked=sort_ranked(*g.sample_ranked(i)), chains=chain_set(*g.sample_chains(i)))
               for i in range(len(samples))]
        # one copy of the whole batch's chains, sliced by bruno_sample_ranges, gives the same
        for i, ch in enumerate(g.batch_chains()):
            assert chain_set(*ch) == out[i]["chains"], i
        total = g.sizes()
        return out, total
    finally:
        g.close()


def same_as_plain(b, p, what):
    for key in SIZE_KEYS:
        assert b["sizes"][key] == p["sizes"][key], (what, key, b["sizes"][key], p["sizes"][key])
    assert_same(b["nodes"], p["nodes"], f"{what}: nodes")
    assert_same(b["ranked"], p["ranked"], f"{what}: listranked nodes")
    assert b["chains"] == p["chains"], f"{what}: chains"


def mixed_samples():
    ws = synth.sample_set(10, seed=7, max_genome=150_000, min_genome=5_000)
    out = [synth.make_fastq(w) for w in ws]
    out.insert(3, fixture_bytes("natural.withN.fastq"))              # reads with N are dropped
    out.insert(5, b"")                                               # an empty sample
    out.insert(6, fixture_bytes("debruijn.shifted_cycle_chr14.fastq"))   # cycles
    out.append(fixture_bytes("debruijn.palindrome_chr14.fastq").rstrip(b"\n"))   # no final newline
    return out


@pytest.mark.parametrize("opt", ["tl2", "u", "tl2_norank"])
def test_batch_equals_plain_per_sample(opt):
    cfg = {"tl2": dict(thresholding=True, thresh=bg.thresholds([2]), min_update=True),
           "u": dict(thresholding=False, min_update=True),
           "tl2_norank": dict(thresholding=True, thresh=bg.thresholds([2]), min_update=False)}[opt]
    samples = mixed_samples()
    got, total = batch(samples, k=31, **cfg)
    n_inst = 0
    for i, data in enumerate(samples):
        p = plain(data, k=31, **cfg)
        same_as_plain(got[i], p, f"sample {i}")
        n_inst += p["sizes"]["n_instances"]
    assert total["n_instances"] == n_inst


@pytest.mark.parametrize("chunk", [1 << 12, 1 << 16, 1 << 20])
def test_batch_copied_in_groups(chunk):
    """host samples copied in groups of whole samples (h2d_chunk bytes each), every group read
    and extracted while the next is in flight: each sample as its plain build"""
    thr = bg.thresholds([2])
    cfg = dict(k=31, thresholding=True, thresh=thr, min_update=True)
    samples = mixed_samples()
    got, total = batch(samples, h2d_chunk=chunk, **cfg)
    for i, data in enumerate(samples):
        same_as_plain(got[i], plain(data, **cfg), f"sample {i}")
    assert total["n_reads"] == sum(g["sizes"]["n_reads"] for g in got)


def test_batch_equals_oracle():
    samples = mixed_samples()[:6]
    thr = bg.thresholds([2])
    got, _ = batch(samples, k=31, thresholding=True, thresh=thr, min_update=True)
    for i, data in enumerate(samples):
        ref = oracle.run(data, k=31, thresh=thr, min_update=True, threads=8)
        for key in ("n_reads", "n_reads_used", "n_instances", "n_k2", "n_nodes", "n_branch", "n_chain_nodes",
                    "iterations", "n_cycle_nodes", "n_isolated", "n_ranked", "n_chains"):
            assert got[i]["sizes"][key] == ref[key], (i, key)
        assert_same(got[i]["nodes"], ref["nodes"], f"sample {i}: nodes")
        assert_same(got[i]["ranked"], ref["ranked"], f"sample {i}: listranked nodes")
        assert got[i]["chains"] == chain_set(*ref["chains"]), f"sample {i}: chains"


def test_batch_of_many_small_samples():
    """hundreds of samples, some with a few reads only: each its own partitions"""
    ws = synth.sample_set(300, seed=11, max_genome=20_000, min_genome=2_000)
    samples = [synth.make_fastq(w) for w in ws]
    thr = bg.thresholds([2])
    got, _ = batch(samples, k=31, thresholding=True, thresh=thr, min_update=True)
    for i in (0, 1, 57, 150, 299):
        same_as_plain(got[i], plain(samples[i], k=31, thresholding=True, thresh=thr, min_update=True), f"sample {i}")


def test_batch_refuses_what_it_cannot_keep_exact():
    data = [fixture_bytes("natural.fastq")] * 2
    for cfg in (dict(k=45), dict(k=31, thresh=bg.thresholds([2, 2, 2])), dict(k=31, edge_filter=True),
                dict(k=31, keep_k2=True)):
        g = bg.Graph(**cfg)
        try:
            with pytest.raises(bg.BrunoError) as e:
                g.build_samples(data)
            assert e.value.status == 1
        finally:
            g.close()


def test_batch_then_plain_in_one_context():
    """a context that built a batch builds a single graph afterwards exactly as a fresh one"""
    thr = bg.thresholds([2])
    data = fixture_bytes("debruijn.bubble.fastq")
    g = bg.Graph(k=31, thresholding=True, thresh=thr, min_update=True)
    try:
        g.build_samples(mixed_samples()[:4])
        g.build_and_compact(data)
        got = dict(sizes=g.sizes(), nodes=sort_nodes(*g.nodes()), ranked=sort_ranked(*g.ranked()),
                   chains=chain_set(*g.chains()))
    finally:
        g.close()
    same_as_plain(got, plain(data, k=31, thresholding=True, thresh=thr, min_update=True), "after a batch")
