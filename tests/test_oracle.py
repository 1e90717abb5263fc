"""The CPU oracle against the reference's own known answers and invariants (no GPU)."""
import json
import os

import numpy as np
import pytest

import bruno_gb300 as bg
from oracle import oracle
from conftest import DATA, GOLDEN, fixture_bytes

with open(os.path.join(GOLDEN, "expected.json")) as _f:
    EXPECTED = json.load(_f)


def fasta_records(text: str):
    return [l for l in text.splitlines() if l and not l.startswith(">")]


def chain_strings(r):
    reps, offs, chars = r["chains"]
    return [chars[int(offs[i]):int(offs[i + 1])].decode() for i in range(len(reps))]


def test_known_answer_unitigs():
    """test_compact_debruijn_graph_all.sh:158 -- the unthresholded compaction of
    test.unitiqs.fastq is test.unitiqs.fasta (sequence lines, sorted)."""
    r = oracle.run(fixture_bytes("test.unitiqs.fastq"), k=31, thresholding=False)
    expect = sorted(fasta_records(fixture_bytes("test.unitiqs.fasta").decode()))
    assert sorted(chain_strings(r)) == expect
    assert r["n_chains"] == 2 and r["n_cycle_nodes"] == 0


@pytest.mark.parametrize("name", ["test.star.unitiqs", "test.short.unitiqs"])
def test_star_fixtures_split_at_branches(name):
    """every unthresholded chain of the star/short fixtures lies inside one source unitig
    and every source unitig is covered by chains plus branch k-mers"""
    r = oracle.run(fixture_bytes(name + ".fastq"), k=31, thresholding=False)
    unitigs = fasta_records(fixture_bytes(name + ".fasta").decode())
    rc = str.maketrans("ACGT", "TGCA")
    for s in chain_strings(r):
        assert any(s in u or s.translate(rc)[::-1] in u for u in unitigs), s


def _make_golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


MG = _make_golden()
OPTIONS = {o[0]: o for o in MG.OPTIONS}


def _digest(result):
    return MG.digest(result)


@pytest.mark.parametrize("key", sorted(EXPECTED))
def test_oracle_matches_golden(key):
    fname, opt = key.split(":")
    name, thr_on, lo, hi, mu = OPTIONS[opt]
    r = oracle.run(fixture_bytes(fname), k=31, thresholding=thr_on, thresh=bg.thresholds(lo, hi), min_update=mu)
    exp = EXPECTED[key]
    if "status" in exp and len(exp) == 1:
        assert r["status"] == exp["status"]
        return
    assert _digest(r) == exp


@pytest.mark.parametrize("fname", ["test.star.unitiqs.fastq", "debruijn.palindrome_chr14.fastq",
                                   "debruijn.shifted_cycle_chr14.fastq", "debruijn.bubble.fastq"])
@pytest.mark.parametrize("mu", [True, False])
def test_shard_invariance(fname, mu):
    """the reference's rank-count invariance (mpirun -np 1..16) as host-shard invariance"""
    fq = fixture_bytes(fname)
    base = oracle.run(fq, k=31, thresh=bg.thresholds([2]), min_update=mu, threads=1)
    for t in (2, 3, 8, 16):
        r = oracle.run(fq, k=31, thresh=bg.thresholds([2]), min_update=mu, threads=t)
        assert _digest(r) == _digest(base), t
        assert r["collisions"] == 0


def test_compacted_files_consistent(tmp_path):
    """check_compacted_files.sh: the first k-mer of every chain is its representative in
    .chain.components; every chain is k-1 + one base per component"""
    fq = fixture_bytes("debruijn.palindrome_chr14.fastq")
    r = oracle.run(fq, k=31, thresh=bg.thresholds([2]), write_prefix=str(tmp_path / "p"))
    comps = open(tmp_path / "p.chain.components").read().splitlines()
    reps = {l.split("\t")[1] for l in comps}
    fasta = open(tmp_path / "p.chain.fasta").read().split("\n")
    seqs = [l for l in fasta if l and not l.startswith(">")]
    assert {s[:31] for s in seqs} == reps
    assert sum(len(s) - 30 for s in seqs) == len(comps)


def test_malformed_fastq_rejected():
    r = oracle.run(fixture_bytes("test.medium.fastq").replace(b"\n+\n", b"\n-\n", 1), k=31)
    assert r["status"] == 2


def test_reads_with_n_are_dropped():
    a = oracle.run(fixture_bytes("natural.withN.fastq"), k=31, thresholding=False)
    assert a["n_reads_used"] < a["n_reads"]
