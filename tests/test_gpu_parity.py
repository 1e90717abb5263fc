"""Parity of the CUDA library with the CPU oracle, through the C ABI.  Integer path: every
comparison is bit-exact, after sorting (table order is not part of the contract)."""
import numpy as np
import pytest

import bruno_gb300 as bg
from bruno_gb300 import synth
from oracle import oracle
from conftest import fixture_bytes
from helpers import assert_same, chain_set, compress_ranked, sort_k2, sort_nodes, sort_ranked

pytestmark = pytest.mark.gpu

FASTQS = ["test.unitiqs.fastq", "test.star.unitiqs.fastq", "test.star2.unitiqs.fastq", "test.short.unitiqs.fastq",
          "test.debruijn.small.fastq", "test.medium.fastq", "debruijn.palindrome.fastq", "debruijn.palindrome2.fastq",
          "debruijn.palindrome_chr14.fastq", "debruijn.shifted_cycle_chr14.fastq", "debruijn.bubble.fastq",
          "debruijn.bubble2.fastq", "natural.fastq", "natural.withN.fastq"]
OPTIONS = {
    "u": (False, (), True), "tl1": (True, (1,), True), "tl2": (True, (2,), True),
    "tl2_norank": (True, (2,), False), "tl3": (True, (3,), True), "tl222": (True, (2, 2, 2), True),
}


def gpu_run(data, k, thr_on, thresh, mu, files=None, **kw):
    g = bg.Graph(k=k, thresholding=thr_on, thresh=thresh, min_update=mu, keep_k2=True, keep_filtered=True, **kw)
    g.reset()
    for f in (files or [data]):
        g.load_fastq(f)
    g.compute_biedge_freqencies()
    k2 = g.k2()
    g.local_insert_by_freqencies()
    check = g.check_index()
    g.extract_chains()
    it = g.list_rank_min_update() if mu else g.list_rank()
    g.to_compressed_chains()
    out = dict(sizes=g.sizes(), k2=k2, filtered=g.filtered(), nodes=g.nodes(), ranked=g.ranked(),
               chains=g.chains(), chain_edges=g.chain_edges(), summaries=summaries_or_none(g), iterations=it,
               check=check)
    g.close()
    return out


def summaries_or_none(g):
    """chain summaries, or None where the library declines them (inconsistent chain pointers)"""
    try:
        return g.chain_summaries()
    except bg.BrunoError as e:
        assert e.status == 6 and "mutually consistent" in e.message, e
        return None


def compare_summaries(gpu, ref):
    """to_summarized_chains: equal to the oracle's whenever the chains are consistent; the
    library declines only where the compaction had to group chains by representative"""
    if gpu["summaries"] is None:
        assert gpu["sizes"]["grouped_chains"] == 1
        return
    assert gpu["sizes"]["grouped_chains"] == 0
    assert ref["summaries"] is not None
    assert_same(gpu["summaries"], ref["summaries"], "chain summaries")


def compare(gpu, ref):
    s = gpu["sizes"]
    for n in ("n_reads", "n_reads_used", "n_instances", "n_nodes", "n_branch", "n_chain_nodes", "iterations",
              "n_cycle_nodes", "n_isolated", "n_ranked", "n_chains"):
        assert s[n] == ref[n], (n, s[n], ref[n])
    assert gpu["iterations"] == ref["iterations"]
    assert s["filter_flag_hist"] == ref["filter_flag_hist"]
    assert_same(sort_k2(*gpu["k2"]), sort_k2(*ref["k2"]), "k2 counts")
    assert_same(sort_k2(*gpu["filtered"]), sort_k2(*ref["filtered"]), "filtered k2")
    assert_same(sort_nodes(*gpu["nodes"]), ref["nodes"], "graph nodes")
    assert_same(sort_ranked(*gpu["ranked"]), ref["ranked"], "listranked chain nodes")
    assert chain_set(*gpu["chains"]) == chain_set(*ref["chains"]), "compacted chains"
    assert_same(gpu["chain_edges"], ref["chain_edges"], "chain end edges")
    compare_summaries(gpu, ref)
    # check_index on the built graph: the same counts and histogram as the oracle's, and the
    # library's verdict is the reference's assertion
    chk = dict(gpu["check"])
    ok = chk.pop("ok")
    assert chk == ref["check_index"], (chk, ref["check_index"])
    assert ok == (chk["n_absent"] == 0 and chk["n_unreferenced"] == 0)


PATHS = {"fast": {}, "round_sync": {"exact_ranking": True}, "direct_count": {"direct_count": 1},
         "l2_partitions": {"direct_count": 2}}


@pytest.mark.parametrize("path", sorted(PATHS))
@pytest.mark.parametrize("opt", sorted(OPTIONS))
@pytest.mark.parametrize("fname", FASTQS)
def test_fixture_parity(fname, opt, path):
    thr_on, lo, mu = OPTIONS[opt]
    thr = bg.thresholds(lo)
    data = fixture_bytes(fname)
    ref = oracle.run(data, k=31, thresholding=thr_on, thresh=thr, min_update=mu, keep_k2=True, keep_filtered=True)
    compare(gpu_run(data, 31, thr_on, thr, mu, **PATHS[path]), ref)


def one_call_run(data, k, thr_on, thresh, mu, **kw):
    """the whole path in one bruno_build_and_compact call, no raw-count copy-outs"""
    g = bg.Graph(k=k, thresholding=thr_on, thresh=thresh, min_update=mu, **kw)
    g.build_and_compact(data)
    out = dict(sizes=g.sizes(), nodes=g.nodes(), ranked=g.ranked(), chains=g.chains(), chain_edges=g.chain_edges(),
               summaries=summaries_or_none(g))
    g.close()
    return out


def compare_one_call(gpu, ref):
    s = gpu["sizes"]
    for n in ("n_reads", "n_reads_used", "n_instances", "n_k2", "n_nodes", "n_branch", "n_chain_nodes",
              "iterations", "n_cycle_nodes", "n_isolated", "n_ranked", "n_chains"):
        assert s[n] == ref[n], (n, s[n], ref[n])
    assert s["filter_flag_hist"] == ref["filter_flag_hist"]
    assert_same(sort_nodes(*gpu["nodes"]), ref["nodes"], "graph nodes")
    assert_same(sort_ranked(*gpu["ranked"]), ref["ranked"], "listranked chain nodes")
    assert chain_set(*gpu["chains"]) == chain_set(*ref["chains"]), "compacted chains"
    assert_same(gpu["chain_edges"], ref["chain_edges"], "chain end edges")
    compare_summaries(gpu, ref)


@pytest.mark.parametrize("opt", sorted(OPTIONS))
@pytest.mark.parametrize("fname", FASTQS)
def test_fixture_parity_one_call(fname, opt):
    thr_on, lo, mu = OPTIONS[opt]
    thr = bg.thresholds(lo)
    data = fixture_bytes(fname)
    ref = oracle.run(data, k=31, thresholding=thr_on, thresh=thr, min_update=mu, keep_k2=True)
    compare_one_call(one_call_run(data, 31, thr_on, thr, mu), ref)


def test_repeat_rich_workload_parity_one_call():
    w = synth.Workload("rep", 2_000_000, 150, 400_000, 0.005, 31, (3,), 0.02, (1000, 10000), (2, 8), (0.01, 0.01), 3)
    fq = synth.make_fastq(w)
    thr = bg.thresholds(w.lower)
    for mu in (True, False):
        ref = oracle.run(fq, k=31, thresh=thr, min_update=mu, threads=16, keep_k2=True)
        compare_one_call(one_call_run(fq, 31, True, thr, mu), ref)


def test_known_answer_on_gpu():
    g = bg.Graph(k=31, thresholding=False).run(fixture_bytes("test.unitiqs.fastq"))
    expect = sorted(l for l in fixture_bytes("test.unitiqs.fasta").decode().splitlines() if l and l[0] != ">")
    assert sorted(g.chain_strings()) == expect


def test_plain_small_workload_parity():
    """the 1 Mbp / 100k x 100 bp / 1% / k=31 / -L 2 workload, every output"""
    w = synth.WORKLOADS["plain-small"]
    fq = synth.make_fastq(w)
    thr = bg.thresholds(w.lower)
    ref = oracle.run(fq, k=31, thresh=thr, min_update=True, threads=16, keep_k2=True, keep_filtered=True)
    gpu = gpu_run(fq, 31, True, thr, True)
    compare(gpu, ref)
    # the shared-memory partition path ran (no fallback to whole-table or L2 counting)
    assert gpu["sizes"]["table_partitions"] >= 256


def test_repeat_rich_workload_parity():
    """a scaled-down plain-scale genome (repeats, 30x, -L 3), both ranking variants"""
    w = synth.Workload("rep", 2_000_000, 150, 400_000, 0.005, 31, (3,), 0.02, (1000, 10000), (2, 8), (0.01, 0.01), 3)
    fq = synth.make_fastq(w)
    thr = bg.thresholds(w.lower)
    for mu, kw in ((True, {}), (False, {}), (True, {"exact_ranking": True}), (True, {"direct_count": 1}), (True, {"direct_count": 2})):
        ref = oracle.run(fq, k=31, thresh=thr, min_update=mu, threads=16, keep_k2=True, keep_filtered=True)
        compare(gpu_run(fq, 31, True, thr, mu, **kw), ref)


def test_two_files_count_into_one_table():
    a, b = fixture_bytes("debruijn.bubble.fastq"), fixture_bytes("debruijn.palindrome_chr14.fastq")
    thr = bg.thresholds([2])
    ref = oracle.run(a + b, k=31, thresh=thr, keep_k2=True, keep_filtered=True)
    compare(gpu_run(None, 31, True, thr, True, files=[a, b]), ref)


def test_small_table_regrows():
    """a deliberately undersized table hits the probe limit, regrows and stays exact"""
    data = fixture_bytes("debruijn.palindrome_chr14.fastq")
    thr = bg.thresholds([2])
    ref = oracle.run(data, k=31, thresh=thr, keep_k2=True, keep_filtered=True)
    out = gpu_run(data, 31, True, thr, True, table_slots=1024)
    assert out["sizes"]["table_slots"] > 1024
    compare(out, ref)


def at_quality(fq: bytes) -> bytes:
    """every quality line made to start with '@' (a valid quality character): a piece boundary
    must still fall on a header, not on a quality line"""
    lines = bytes(fq).split(b"\n")
    for i in range(3, len(lines), 4):
        if lines[i]:
            lines[i] = b"@" + lines[i][1:]
    return b"\n".join(lines)


@pytest.mark.parametrize("kw", [{}, {"direct_count": 1}, {"direct_count": 2}, {"exact_ranking": True}])
def test_host_pieces_parity(kw):
    """host FASTQ copied and indexed in 64 KiB pieces (extraction under the later copies),
    one and two files, equal to the oracle"""
    w = synth.WORKLOADS["plain-small"]
    fq = at_quality(synth.make_fastq(w))
    thr = bg.thresholds(w.lower)
    ref = oracle.run(fq, k=31, thresh=thr, min_update=True, threads=16, keep_k2=True, keep_filtered=True)
    compare(gpu_run(fq, 31, True, thr, True, h2d_chunk=1 << 16, **kw), ref)
    lines = fq.split(b"\n")
    cut = sum(len(l) + 1 for l in lines[:len(lines) // 12 * 4])   # a record start, a third of the way in
    compare(gpu_run(None, 31, True, thr, True, files=[fq[:cut], fq[cut:]], h2d_chunk=1 << 16, **kw), ref)


@pytest.mark.parametrize("fname", ["test.unitiqs.fastq", "natural.withN.fastq", "debruijn.palindrome_chr14.fastq"])
def test_host_pieces_fixture_parity(fname):
    """pieces of about 1 KiB: dozens of segments, each waited on by the index"""
    data = at_quality(fixture_bytes(fname))
    for k, kw in ((31, {}), (45, {}), (31, {"edge_filter": True})):
        thr = bg.thresholds([2])
        ref = oracle.run(data, k=k, thresh=thr, min_update=True, keep_k2=True, keep_filtered=True,
                         edge_filter=kw.get("edge_filter", False))
        compare(gpu_run(data, k, True, thr, True, h2d_chunk=1024, **kw), ref)


def test_malformed_fastq_is_bad_input():
    data = fixture_bytes("test.medium.fastq").replace(b"\n+\n", b"\n-\n", 1)
    with pytest.raises(bg.BrunoError) as e:
        bg.Graph(k=31).run(data)
    assert e.value.status == 2


def test_device_resident_input():
    torch = pytest.importorskip("torch")
    data = fixture_bytes("debruijn.bubble.fastq")
    dev = torch.frombuffer(bytearray(data), dtype=torch.uint8).cuda()
    thr = bg.thresholds([2])
    g = bg.Graph(k=31, thresh=thr)
    g.build_and_compact(dev.data_ptr(), nbytes=dev.numel(), is_device=True)
    torch.cuda.synchronize()
    ref = oracle.run(data, k=31, thresh=thr)
    assert chain_set(*g.chains()) == chain_set(*ref["chains"])
    assert_same(sort_ranked(*g.ranked()), ref["ranked"], "ranked")


def test_context_reuse_gives_identical_results():
    data = fixture_bytes("debruijn.palindrome_chr14.fastq")
    g = bg.Graph(k=31, thresh=bg.thresholds([2]))
    g.build_and_compact(data)
    first = (chain_set(*g.chains()), sort_ranked(*g.ranked()))
    g.build_and_compact(data)
    assert chain_set(*g.chains()) == first[0]
    assert_same(sort_ranked(*g.ranked()), first[1], "second build")


@pytest.mark.parametrize("k", [32, 33, 45, 63])
def test_large_k_workload_parity(k):
    """128-bit keys (k >= 32): a repeat-rich 300 kbp genome at 25x, every output, both
    ranking variants and the round-synchronous ranking"""
    w = synth.Workload(f"k{k}", 300_000, 150, 50_000, 0.005, k, (3,), 0.03, (500, 4000), (2, 6), (0.01, 0.02), 7)
    fq = synth.make_fastq(w)
    thr = bg.thresholds(w.lower)
    for mu, kw in ((True, {}), (False, {}), (True, {"exact_ranking": True})):
        ref = oracle.run(fq, k=k, thresh=thr, min_update=mu, threads=16, keep_k2=True, keep_filtered=True)
        compare(gpu_run(fq, k, True, thr, mu, **kw), ref)


@pytest.mark.parametrize("k", [33, 63])
@pytest.mark.parametrize("fname", ["debruijn.palindrome_chr14.fastq", "debruijn.bubble.fastq", "natural.fastq"])
def test_large_k_fixture_parity(fname, k):
    data = fixture_bytes(fname)
    for thr_on, lo in ((False, ()), (True, (2,))):
        thr = bg.thresholds(lo)
        ref = oracle.run(data, k=k, thresholding=thr_on, thresh=thr, min_update=True, keep_k2=True,
                         keep_filtered=True)
        compare(gpu_run(data, k, thr_on, thr, True), ref)


def test_large_k_one_call_parity():
    w = synth.Workload("k63one", 300_000, 150, 50_000, 0.005, 63, (3,), 0.03, (500, 4000), (2, 6), (0.01, 0.02), 8)
    fq = synth.make_fastq(w)
    thr = bg.thresholds(w.lower)
    ref = oracle.run(fq, k=63, thresh=thr, min_update=True, threads=16, keep_k2=True)
    compare_one_call(one_call_run(fq, 63, True, thr, True), ref)


@pytest.mark.parametrize("k", [31, 45])
@pytest.mark.parametrize("seed", [3, 4, 5])
@pytest.mark.parametrize("mu", [True, False])
def test_inconsistent_chain_pointers_emission(seed, mu, k):
    """separate k and k+2 lower bounds trim some edges on one side only, so some chains have a
    representative outside the chain map (no distance-0 node) and chains can share one.  The
    reference's ranking of such maps depends on its update order (the oracle's result changes
    with its shard count, and so does the device's with its table layout), so these inputs pin
    the emission: the compacted chains must be to_compressed_chains of the listranked nodes,
    and everything before the ranking must equal the oracle's."""
    fq = synth.make_fastq(synth.sample_set(1, seed, max_genome=200_000, k=k)[0])
    thr = [2, 65536, 2, 65536, 2, 65536]
    a = gpu_run(fq, k, True, thr, mu)
    K, rep, dist = a["ranked"]
    assert a["sizes"]["n_chains"] > int((dist == 0).sum())      # the case this test is about
    assert chain_set(*a["chains"]) == compress_ranked(K, rep, dist, k)
    ref = oracle.run(fq, k=k, thresh=thr, min_update=mu, keep_k2=True, keep_filtered=True)
    assert_same(sort_nodes(*a["nodes"]), ref["nodes"], "graph nodes")
    assert a["sizes"]["n_chain_nodes"] == ref["n_chain_nodes"]


@pytest.mark.parametrize("lo", [1, 2, 3])
@pytest.mark.parametrize("fname", FASTQS)
def test_edge_filter_parity(fname, lo):
    """the blocked driver's (k+1)-mer edge-filter build: every output equals the oracle's,
    step by step and in one call"""
    thr = bg.thresholds([lo])
    data = fixture_bytes(fname)
    ref = oracle.run(data, k=31, thresh=thr, min_update=True, keep_k2=True, keep_filtered=True, edge_filter=True)
    compare(gpu_run(data, 31, True, thr, True, edge_filter=True), ref)
    compare_one_call(one_call_run(data, 31, True, thr, True, edge_filter=True), ref)


def test_edge_filter_workload_parity():
    """the 1 Mbp / 100k x 100 bp / 1% workload through the (k+1)-mer edge filter, both rankings"""
    w = synth.WORKLOADS["plain-small"]
    fq = synth.make_fastq(w)
    thr = bg.thresholds(w.lower)
    for mu in (True, False):
        ref = oracle.run(fq, k=31, thresh=thr, min_update=mu, threads=16, keep_k2=True, keep_filtered=True,
                         edge_filter=True)
        compare(gpu_run(fq, 31, True, thr, mu, edge_filter=True), ref)


@pytest.mark.parametrize("k,slots,parts", [(31, 80_000_000, 1 << 19), (63, 140_000_000, 1 << 21)])
def test_scatter_split_parity(k, slots, parts):
    """tables with more partitions than the shared-memory split handles, on a 1 Mbp genome: an
    explicit table of partitions of at most 256 slots (k = 31: 2^19 partitions, the records
    scattered in windows of four buckets) or 128 (k = 63: 2^21 partitions, 8192 a bucket, so
    the records are scattered bucket after bucket)"""
    w = synth.WORKLOADS["plain-small"]
    fq = synth.make_fastq(w)
    thr = bg.thresholds(w.lower)
    ref = oracle.run(fq, k=k, thresh=thr, min_update=True, threads=16, keep_k2=True, keep_filtered=True)
    got = gpu_run(fq, k, True, thr, True, table_slots=slots, part_slots=256)
    assert got["sizes"]["table_partitions"] == parts
    compare(got, ref)


@pytest.mark.parametrize("k", [32, 33, 63])
@pytest.mark.parametrize("fname", ["debruijn.palindrome_chr14.fastq", "debruijn.bubble.fastq", "natural.fastq",
                                   "natural.withN.fastq"])
def test_edge_filter_large_k_parity(fname, k):
    """the (k+1)-mer edge filter at k > 31: 128-bit (k+1)-mers (33..64 bases) in their own table,
    the filter applied in the partitioned count's extraction"""
    thr = bg.thresholds([2])
    data = fixture_bytes(fname)
    ref = oracle.run(data, k=k, thresh=thr, min_update=True, keep_k2=True, keep_filtered=True, edge_filter=True)
    compare(gpu_run(data, k, True, thr, True, edge_filter=True), ref)
    compare_one_call(one_call_run(data, k, True, thr, True, edge_filter=True), ref)


def test_edge_filter_large_k_workload_parity():
    """the 1 Mbp / 100k x 100 bp / 1% workload through the edge filter at k = 45"""
    w = synth.WORKLOADS["plain-small"]
    fq = synth.make_fastq(w)
    thr = bg.thresholds(w.lower)
    ref = oracle.run(fq, k=45, thresh=thr, min_update=True, threads=16, keep_k2=True, keep_filtered=True,
                     edge_filter=True)
    compare(gpu_run(fq, 45, True, thr, True, edge_filter=True), ref)


def test_edge_filter_rejects_direct_count():
    for k in (31, 45):
        with pytest.raises(bg.BrunoError):
            bg.Graph(k=k, thresh=bg.thresholds([2]), edge_filter=True, direct_count=1)


def test_large_k_mix_parity():
    """the large-k mix (5% repeats of 1-20 kbp in 2-16 copies at 1-3% divergence, 30x 150 bp,
    0.5% substitutions, k = 63, -L 3) at a hundredth of its genome: 128-bit keys through the
    whole-table count, every output against the oracle"""
    w = synth.Workload("large-k-small", 2_000_000, 150, 400_000, 0.005, 63, (3,), 0.05, (1000, 20000), (2, 16),
                       (0.01, 0.03), 9)
    fq = synth.make_fastq(w)
    thr = bg.thresholds(w.lower)
    ref = oracle.run(fq, k=63, thresh=thr, min_update=True, threads=16, keep_k2=True, keep_filtered=True)
    compare(gpu_run(fq, 63, True, thr, True, max_load=0.7), ref)
