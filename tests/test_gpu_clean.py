"""Graph cleaning on the GPU (bruno_clean_deadend_and_bubbles_naive; the _freq_clean driver's
clean_deadend_and_bubbles_naive, compact_dbg_clean.hpp:575-890) against the oracle's
restatement, bit-exact after sorting.  Without a GPU they are skipped."""
import os
import subprocess

import pytest

import bruno_gb300 as bg
from bruno_gb300 import build, synth
from oracle import oracle
from conftest import DATA, fixture_bytes
from helpers import assert_same, chain_set, sort_nodes, sort_ranked
from test_oracle import _fastq, _genome, _subst, _tiling


def _has_cuda() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not _has_cuda(), reason="needs a CUDA GPU")]


def gpu_clean(data, k, thr_on, thresh, mu=True, **kw):
    g = bg.Graph(k=k, thresholding=thr_on, thresh=thresh, min_update=mu, **kw)
    try:
        g.build_and_compact(data)
        pre = dict(sizes=g.sizes(), chains=g.chains())
        try:
            stats = g.clean_deadend_and_bubbles_naive()
        except bg.BrunoError as e:
            if getattr(e, "stats", {}).get("status") != 2:
                raise
            return dict(pre=pre, declined=True)
        return dict(pre=pre, stats=stats, sizes=g.sizes(), nodes=g.nodes(), ranked=g.ranked(), chains=g.chains(),
                    chain_edges=g.chain_edges())
    finally:
        g.close()


def compare_clean(gpu, ref):
    if ref["clean_stats"]["status"] == 2:   # a terminus case the reference throws on
        assert gpu.get("declined"), "the oracle met a case the reference throws on; the GPU did not decline"
        return
    assert not gpu.get("declined"), "the GPU declined a graph the oracle cleaned"
    c = ref["clean"]
    assert gpu["stats"] == ref["clean_stats"], (gpu["stats"], ref["clean_stats"])
    assert chain_set(*gpu["pre"]["chains"]) == chain_set(*ref["chains"]), "first compaction"
    assert gpu["sizes"]["n_nodes"] == c["n_nodes"]
    assert_same(sort_nodes(*gpu["nodes"]), c["nodes"], "cleaned nodes")
    assert_same(sort_ranked(*gpu["ranked"]), c["ranked"], "cleaned listranked nodes")
    assert chain_set(*gpu["chains"]) == chain_set(*c["chains"]), "cleaned chains"
    assert_same(gpu["chain_edges"], c["chain_edges"], "cleaned chain end edges")


def _constructed(case: str) -> bytes:
    """the oracle tests' constructions: a 10-node tip, a 100-node tip, a one-read SNP bubble"""
    if case == "tip":
        g = _genome(400, 11)
        bad = list(g[150:250]); bad[90] = _subst(bad[90])
    elif case == "long_tip":
        g = _genome(400, 12)
        bad = list(g[100:250])
        for p in (50, 80, 110, 140):
            bad[p] = _subst(bad[p])
    else:
        g = _genome(400, 13)
        bad = list(g[150:250]); bad[50] = _subst(bad[50])
    return _fastq(_tiling(g) + ["".join(bad)])


@pytest.mark.parametrize("k", [31, 45])
@pytest.mark.parametrize("case", ["tip", "long_tip", "bubble"])
def test_clean_constructed_cases(case, k):
    fq = _constructed(case)
    thr = bg.thresholds([1])
    ref = oracle.run(fq, k=k, thresh=thr, clean=True)
    compare_clean(gpu_clean(fq, k, True, thr), ref)


FIXTURE_CASES = [
    ("debruijn.bubble.fastq", ()), ("debruijn.bubble.fastq", (1,)), ("debruijn.bubble2.fastq", ()),
    ("debruijn.palindrome_chr14.fastq", ()), ("debruijn.palindrome_chr14.fastq", (1,)),
    ("debruijn.palindrome_chr14.fastq", (2,)), ("debruijn.clean1.fastq", ()), ("debruijn.clean1.fastq", (1,)),
    ("debruijn.clean2.fastq", ()), ("debruijn.clean2.fastq", (1,)), ("test.debruijn.small.fastq", ()),
    ("debruijn.shifted_cycle_chr14.fastq", (2,)), ("debruijn.palindrome.fastq", ()),
]


@pytest.mark.parametrize("fname,lo", FIXTURE_CASES)
@pytest.mark.parametrize("kw", [{}, {"exact_ranking": True}])
def test_clean_fixture_parity(fname, lo, kw):
    data = fixture_bytes(fname)
    thr = bg.thresholds(lo)
    ref = oracle.run(data, k=31, thresholding=bool(lo), thresh=thr, clean=True)
    compare_clean(gpu_clean(data, 31, bool(lo), thr, **kw), ref)


def test_clean_workload_parity():
    """the 1 Mbp / 100k x 100 bp / 1% / -L 2 workload: thousands of error tips and bubbles"""
    w = synth.WORKLOADS["plain-small"]
    fq = bytes(synth.make_fastq(w))
    thr = bg.thresholds(w.lower)
    ref = oracle.run(fq, k=31, thresh=thr, clean=True, threads=16)
    assert ref["clean_stats"]["rounds"] > 0
    compare_clean(gpu_clean(fq, 31, True, thr), ref)


def test_clean_twice_is_refused():
    data = fixture_bytes("debruijn.bubble.fastq")
    g = bg.Graph(k=31, thresh=bg.thresholds([1]))
    try:
        g.build_and_compact(data)
        g.clean_deadend_and_bubbles_naive()
        with pytest.raises(bg.BrunoError) as e:
            g.clean_deadend_and_bubbles_naive()
        assert e.value.status == 1
    finally:
        g.close()


CLEAN_OUTPUTS = [".chain.fasta", ".chain.components", ".chain.summary", ".branch.fasta", ".branch.edges",
                 ".graph.all", ".clean.chain.fasta", ".clean.chain.components", ".clean.chain.edges",
                 ".clean.branch.fasta", ".clean.branch.edges"]


@pytest.mark.parametrize("fname,flags", [("debruijn.bubble.fastq", ["-T", "-L", "1", "-R"]),
                                         ("debruijn.clean2.fastq", ["-R"]),
                                         ("debruijn.palindrome_chr14.fastq", ["-T", "-L", "2"])])
def test_clean_driver_outputs_identical(tmp_path, fname, flags):
    drv = build.build_driver()
    fq = os.path.join(DATA, fname)
    subprocess.run([drv, "--clean", *flags, "-O", str(tmp_path / "gpu"), fq], check=True, capture_output=True)
    subprocess.run([oracle.CLI, "--clean", *flags, "-O", str(tmp_path / "ref"), fq], check=True, capture_output=True)
    for ext in CLEAN_OUTPUTS:
        a = open(tmp_path / ("gpu" + ext), "rb").read()
        b = open(tmp_path / ("ref" + ext), "rb").read()
        assert a == b, f"{fname} {' '.join(flags)}: {ext} differs"
    assert not os.path.exists(tmp_path / "gpu.chain.edges")


@pytest.mark.parametrize("case", ["empty", "one_read", "circle"])
def test_clean_edge_cases(case):
    g = _genome(200, 21)
    if case == "empty":
        fq = b""
    elif case == "one_read":
        fq = _fastq([g[:150]])
    else:
        circ = g + g[:60]
        fq = _fastq([circ[i:i + 100] for i in range(0, len(g), 5)])
    thr = bg.thresholds([1])
    ref = oracle.run(fq, k=31, thresh=thr, clean=True)
    compare_clean(gpu_clean(fq, 31, True, thr), ref)
