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
    fname, opt, *clean = key.split(":")
    name, thr_on, lo, hi, mu = OPTIONS[opt]
    r = oracle.run(fixture_bytes(fname), k=31, thresholding=thr_on, thresh=bg.thresholds(lo, hi), min_update=mu,
                   clean=bool(clean))
    exp = EXPECTED[key]
    if "status" in exp and len(exp) == 1:
        assert r["status"] == exp["status"]
        return
    assert (dict(_digest(r["clean"]), **r["clean_stats"]) if clean else _digest(r)) == exp


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


def _ascii(words, k):
    v = 0
    for i, w in enumerate(words):
        v |= int(w) << (64 * i)
    return "".join("ACGT"[(v >> (2 * (k - 1 - j))) & 3] for j in range(k))


_RC = str.maketrans("ACGT", "TGCA")


def _rc(s):
    return s.translate(_RC)[::-1]


@pytest.mark.parametrize("fname,k,thr_on,lo,mu", [
    ("debruijn.palindrome_chr14.fastq", 31, True, (2,), True),
    ("debruijn.bubble.fastq", 31, True, (1, 2, 1), True),
    ("debruijn.shifted_cycle_chr14.fastq", 31, True, (2,), False),
    ("test.star.unitiqs.fastq", 31, False, (), True),
    ("debruijn.bubble.fastq", 45, True, (2,), True),
    ("debruijn.palindrome_chr14.fastq", 32, False, (), False),
])
def test_chain_edges_follow_chain_strings(tmp_path, fname, k, thr_on, lo, mu):
    """print_chain_frequencies (compact_dbg_stats.hpp:879-1065) derived a second way: for every
    compacted chain L is its first k-mer and R its last, on the chain's strand; L's in-edges
    and R's out-edges are the graph counters of those k-mers read on that strand; the summary
    is over the self frequencies of the chain's listranked nodes, mean = float32 sum / float32
    count, truncated.  Lines sorted by L, every value followed by a tab."""
    r = oracle.run(fixture_bytes(fname), k=k, thresholding=thr_on, thresh=bg.thresholds(lo), min_update=mu,
                   write_prefix=str(tmp_path / "p"))
    keys, counts, _ = r["nodes"]
    node = {_ascii(keys[i], k): counts[i] for i in range(len(keys))}
    K, rep, _ = r["ranked"]
    selfs = {}
    for i in range(len(K)):
        selfs.setdefault(_ascii(rep[i], k), []).append(int(node[min(_ascii(K[i], k), _rc(_ascii(K[i], k)))][8]))
    lines = []
    for s in chain_strings(r):
        L, R = s[:k], s[-k:]
        cl, cr = node[min(L, _rc(L))], node[min(R, _rc(R))]
        lin = list(cl[4:8]) if L <= _rc(L) else [cl[3], cl[2], cl[1], cl[0]]
        rout = list(cr[0:4]) if R <= _rc(R) else [cr[7], cr[6], cr[5], cr[4]]
        f = selfs[L]
        mean = int(np.float32(sum(f)) / np.float32(len(f)))
        lines.append(f"{L}\t{R}\t" + "".join(f"{int(v)}\t" for v in lin + rout + [mean, min(f), max(f)]) + "\n")
    got = open(tmp_path / "p.chain.edges").read()
    assert got == "".join(sorted(lines))
    assert len(lines) == r["n_chains"] > 0


@pytest.mark.parametrize("fname,k,thr_on,lo,mu", [
    ("debruijn.palindrome_chr14.fastq", 31, True, (2,), True),
    ("debruijn.bubble.fastq", 31, True, (1, 2, 1), False),
    ("test.star.unitiqs.fastq", 31, False, (), True),
    ("debruijn.bubble.fastq", 45, True, (2,), True),
])
def test_chain_summaries_follow_chain_strings(tmp_path, fname, k, thr_on, lo, mu):
    """to_summarized_chains (debruijn_chain_graph.hpp:1876-2005) derived a second way: one line
    per compacted chain, 5' terminus = its first k-mer (the representative), 3' = its last,
    distance = length - k; the outer neighbour of an end is the one graph edge leaving it on
    the chain's strand (flag 1), or else (flag 0) Kmer(), all A, read on the strand of the end's
    canonical k-mer -- all T where the chain runs on the other strand, since
    transform::reverse_complement turns the missing neighbour around with the rest."""
    r = oracle.run(fixture_bytes(fname), k=k, thresholding=thr_on, thresh=bg.thresholds(lo), min_update=mu,
                   write_prefix=str(tmp_path / "p"))
    assert r["summaries"] is not None
    keys, counts, _ = r["nodes"]
    node = {_ascii(keys[i], k): counts[i] for i in range(len(keys))}

    def edge(x, side):   # the bases of x's in- (side 0) or out-edges (side 1), x on its own strand
        c = node[min(x, _rc(x))]
        canon = x <= _rc(x)
        if side == 0:
            cnt = list(c[4:8]) if canon else [c[3], c[2], c[1], c[0]]
        else:
            cnt = list(c[0:4]) if canon else [c[7], c[6], c[5], c[4]]
        return ["ACGT"[b] for b in range(4) if cnt[b]]

    lines = []
    for s in chain_strings(r):
        t5, t3 = s[:k], s[-k:]
        pin, pout = edge(t5, 0), edge(t3, 1)
        assert len(pin) <= 1 and len(pout) <= 1
        prev = pin[0] + t5[:-1] if pin else ("A" if t5 <= _rc(t5) else "T") * k
        nxt = t3[1:] + pout[0] if pout else ("A" if t3 <= _rc(t3) else "T") * k
        lines.append(f"{prev} {t5} {t3} {nxt} {len(s) - k} {len(pin)} {len(pout)}\n")
    assert open(tmp_path / "p.chain.summary").read() == "".join(sorted(lines, key=lambda l: l.split()[1]))
    assert len(lines) == r["n_chains"] > 0


def test_chain_edges_select_one_terminus_per_chain():
    """IsCanonicalTerminusOrIsolated (debruijn_chain_filters.hpp:125-147) keeps exactly one
    chain-map node per chain whose representative is a chain node; with k and k+2 bounds the
    filter can trim an edge on one side only, leaving chains whose representative lies outside
    the chain map, and those get no record"""
    from bruno_gb300 import synth
    fq = synth.make_fastq(synth.sample_set(1, 3, max_genome=50_000)[0])
    r = oracle.run(fq, k=31, thresh=[2, 65536, 2, 65536, 2, 65536])
    K, rep, dist = r["ranked"]
    headed = {tuple(rep[i]) for i in range(len(K)) if dist[i] == 0}
    L = r["chain_edges"][0]
    assert len(L) == len(headed) < r["n_chains"]
    assert {tuple(x) for x in L} == headed


@pytest.mark.parametrize("seed,k", [(3, 31), (4, 45)])
def test_compress_ranked_restatement(seed, k):
    """the test helper restating to_compressed_chains over listranked nodes gives the oracle's
    own compaction, also when chains lack a distance-0 node or share a representative"""
    from bruno_gb300 import synth
    from helpers import chain_set, compress_ranked
    fq = synth.make_fastq(synth.sample_set(1, seed, max_genome=100_000, k=k)[0])
    r = oracle.run(fq, k=k, thresh=[2, 65536, 2, 65536, 2, 65536])
    assert r["n_chains"] > int((r["ranked"][2] == 0).sum())
    assert chain_set(*r["chains"]) == compress_ranked(*r["ranked"], k)


def _edge_filter_nodes(fq: bytes, k: int, lo: int, hi: int = 65536):
    """the blocked driver's build_index_thresholded restated in Python: canonical (k+1)-mer
    counts (saturating at 65535), those outside [lo, hi) erased; per read position the biedge
    loses each edge whose (k+1)-mer is gone; pairs without edges are dropped; the rest update
    their canonical node: self count and one count per present edge"""
    lines = fq.decode().split("\n")
    reads = [lines[i + 1].upper() for i in range(0, len(lines) - 3, 4) if lines[i].startswith("@")]
    reads = [r for r in reads if set(r) <= set("ACGT")]
    k1 = {}
    for r in reads:
        for p in range(len(r) - k):
            x = r[p:p + k + 1]
            c = min(x, _rc(x))
            k1[c] = min(65535, k1.get(c, 0) + 1)
    keep = {x for x, c in k1.items() if lo <= c < hi}
    nodes = {}
    comp = {"A": "T", "C": "G", "G": "C", "T": "A"}
    for r in reads:
        if len(r) < k + 2:
            continue
        for p in range(len(r) - k + 1):
            x = r[p:p + k]
            i = r[p - 1] if p > 0 else None
            o = r[p + k] if p + k < len(r) else None
            if i and min(i + x, _rc(i + x)) not in keep:
                i = None
            if o and min(x + o, _rc(x + o)) not in keep:
                o = None
            if i is None and o is None:
                continue
            if x > _rc(x) or x == _rc(x):          # lex_less keeps x only when x < rc(x)
                x, i, o = _rc(x), (comp[o] if o else None), (comp[i] if i else None)
            c = nodes.setdefault(x, [0] * 9)
            if o:
                c["ACGT".index(o)] = min(65535, c["ACGT".index(o)] + 1)
            if i:
                c[4 + "ACGT".index(i)] = min(65535, c[4 + "ACGT".index(i)] + 1)
            c[8] = min(65535, c[8] + 1)
    return nodes


@pytest.mark.parametrize("fname,lo", [("debruijn.palindrome_chr14.fastq", 2), ("debruijn.bubble.fastq", 3),
                                      ("test.star.unitiqs.fastq", 1), ("debruijn.shifted_cycle_chr14.fastq", 2)])
def test_edge_filter_nodes_restated(fname, lo):
    """the oracle's (k+1)-mer edge-filter build (compact_debruijn_graph_block_construct.cpp:
    417-470, debruijn_biedge_filters.hpp:66-75, 128-177, 331-423) against a second restatement
    of it: the same graph nodes with the same nine counters"""
    k = 31
    fq = fixture_bytes(fname)
    r = oracle.run(fq, k=k, thresh=bg.thresholds([lo]), edge_filter=True)
    keys, counts, _ = r["nodes"]
    got = {_ascii(keys[i], k): list(map(int, counts[i])) for i in range(len(keys))}
    want = _edge_filter_nodes(fq, k, lo)
    assert got == want
    assert len(got) > 0


def test_edge_filter_without_bounds_is_build_index():
    """with no (k+1)-mer erased the edge filter changes nothing: the unthresholded build"""
    fq = fixture_bytes("debruijn.bubble.fastq")
    a = oracle.run(fq, k=31, thresh=bg.thresholds([0]), edge_filter=True)
    b = oracle.run(fq, k=31, thresholding=False)
    assert MG.digest(a) == MG.digest(b)


def test_malformed_fastq_rejected():
    r = oracle.run(fixture_bytes("test.medium.fastq").replace(b"\n+\n", b"\n-\n", 1), k=31)
    assert r["status"] == 2


def test_reads_with_n_are_dropped():
    a = oracle.run(fixture_bytes("natural.withN.fastq"), k=31, thresholding=False)
    assert a["n_reads_used"] < a["n_reads"]


# ---------------------------------------------------------------- graph cleaning
# clean_deadend_and_bubbles_naive (compact_dbg_clean.hpp:575-890).  The reference ships no
# cleaned outputs, so these cases pin the restatement by construction: reads tiling a random
# genome at 20x, plus reads that add a low-coverage tip or bubble whose fate is known.

def _fastq(reads) -> bytes:
    return b"".join(b"@r%d\n%s\n+\n%s\n" % (i, r.encode(), b"I" * len(r)) for i, r in enumerate(reads))


def _genome(n, seed):
    rng = np.random.default_rng(seed)
    return "".join("ACGT"[x] for x in rng.integers(0, 4, n))


def _tiling(g, L=100, step=5):
    return [g[i:i + L] for i in range(0, len(g) - L + 1, step)]


def _canon_strings(strings):
    return sorted(min(x, _rc(x)) for x in strings)


def _subst(c):
    return "ACGT"[("ACGT".index(c) + 1) % 4]


@pytest.mark.parametrize("k", [31, 45])
def test_clean_severs_short_low_coverage_tip(k):
    """one read with an error 10 bases before its end: a 10-node tip (shorter than 2k-1) off a
    20x genome.  Cleaning severs the tip's edge of frequency 1 (below -L 1's 2): the genome
    becomes one chain again and the tip stays as a chain of its own."""
    g = _genome(400, 11)
    bad = list(g[150:250]); bad[90] = _subst(bad[90]); bad = "".join(bad)
    r = oracle.run(_fastq(_tiling(g) + [bad]), k=k, thresh=bg.thresholds([1]), clean=True)
    assert r["clean_stats"] == {"rounds": 1, "deadends": 1, "bubbles": 0, "edges": 1, "status": 0}
    # before: the genome's chains on either side of the branch k-mer g[240-k:240], and the tip
    tip = bad[90 - k + 1:]
    assert _canon_strings(chain_strings(r)) == _canon_strings([g[:239], g[241 - k:], tip])
    assert _canon_strings(chain_strings(r["clean"])) == _canon_strings([g, tip])


@pytest.mark.parametrize("k", [31, 45])
def test_clean_keeps_long_tip(k):
    """a tip of 2k-1 nodes or more is not a dead end to clean: nothing changes.  Four errors in
    one 150-base read, the first past the read's first k-mer, make every k-mer from the first
    error's on new: a 100-node tip off the genome (2k-1 is 61 at k = 31, 89 at k = 45)."""
    g = _genome(400, 12)
    bad = list(g[100:250])
    for p in (50, 80, 110, 140):
        bad[p] = _subst(bad[p])
    bad = "".join(bad)
    r = oracle.run(_fastq(_tiling(g) + [bad]), k=k, thresh=bg.thresholds([1]), clean=True)
    assert r["clean_stats"]["rounds"] == 0
    assert _canon_strings(chain_strings(r["clean"])) == _canon_strings(chain_strings(r))
    assert len(chain_strings(r)) == 3


@pytest.mark.parametrize("k", [31, 45])
def test_clean_severs_low_coverage_bubble_path(k):
    """one read with a substitution mid-read: a k-node bubble path beside the 20x genome's.  The
    two paths between the same branches have equal lengths and a low-frequency end, so both
    lose their end edges below frequency 2: only the error path's go, the genome re-joins."""
    g = _genome(400, 13)
    bad = list(g[150:250]); bad[50] = _subst(bad[50]); bad = "".join(bad)
    r = oracle.run(_fastq(_tiling(g) + [bad]), k=k, thresh=bg.thresholds([1]), clean=True)
    assert r["clean_stats"] == {"rounds": 1, "deadends": 0, "bubbles": 2, "edges": 2, "status": 0}
    assert _canon_strings(chain_strings(r["clean"])) == _canon_strings([g, bad[50 - k + 1:50 + k]])


def _node_map(nodes, k):
    keys, counts, _ = nodes
    return {_ascii(keys[i], k): counts[i].astype(int) for i in range(len(keys))}


def _edge_neighbour(x, i):
    """the node at the other end of count index i (out A C G T, in A C G T) of canonical k-mer x,
    as stored (canonical), and the count index of the same edge there"""
    code = "ACGT".index
    if i < 4:    # out-edge to y = x[1:] + c: on y an in-edge from x's first character
        y, j = x[1:] + "ACGT"[i], 4 + code(x[0])
    else:        # in-edge from y = c + x[:-1]: on y an out-edge to x's last character
        y, j = "ACGT"[i - 4] + x[:-1], code(x[-1])
    if _rc(y) < y:   # stored on the other strand: in <-> out, character complemented
        y, j = _rc(y), (4 + 3 - j) if j < 4 else 3 - (j - 4)
    return y, j


@pytest.mark.parametrize("fname,lo", [("debruijn.palindrome_chr14.fastq", ()), ("debruijn.bubble.fastq", (1,)),
                                      ("debruijn.clean2.fastq", ()), ("debruijn.clean1.fastq", (1,))])
def test_clean_only_erases_edges_in_pairs(fname, lo):
    """cleaning removes edges and edge-less nodes, never adds or changes a count, and every edge
    it removes is removed on both of its nodes (erase_edges_internal, debruijn_graph_map.hpp
    :737-747); cycle nodes and nodes left without edges leave the graph"""
    k = 31
    r = oracle.run(fixture_bytes(fname), k=k, thresholding=bool(lo), thresh=bg.thresholds(lo), clean=True)
    assert r["clean_stats"]["status"] == 0 and r["clean_stats"]["rounds"] > 0
    before, after = _node_map(r["nodes"], k), _node_map(r["clean"]["nodes"], k)
    assert set(after) <= set(before)
    removed = 0
    for x, a in after.items():
        b = before[x]
        assert a[8] == b[8]                                  # self count kept
        assert all(a[i] in (0, b[i]) for i in range(8))      # an edge is kept or erased
        assert any(a[:8])                                    # no edge-less node stays
        for i in range(8):
            if b[i] and not a[i]:
                removed += 1
                y, j = _edge_neighbour(x, i)
                if y in after and y in before and before[y][j]:
                    assert after[y][j] == 0, (x, i, y, j)
    assert removed > 0


@pytest.mark.parametrize("fname,lo", [("debruijn.palindrome_chr14.fastq", ()), ("debruijn.bubble.fastq", (1,)),
                                      ("debruijn.clean1.fastq", ()), ("debruijn.clean2.fastq", (1,))])
def test_clean_shard_invariance(fname, lo):
    """cleaning gives the same graph for any number of host shards (the reference's rank-count
    invariance, as its bubble-clean script checks across -np)"""
    fq = fixture_bytes(fname)
    kw = dict(k=31, thresholding=bool(lo), thresh=bg.thresholds(lo), clean=True)
    base = oracle.run(fq, threads=1, **kw)
    assert base["clean_stats"]["rounds"] > 0
    for t in (2, 5, 16):
        r = oracle.run(fq, threads=t, **kw)
        assert r["clean_stats"] == base["clean_stats"], t
        assert _digest(r["clean"]) == _digest(base["clean"]), t


def test_clean_files_match_arrays(tmp_path):
    """the --clean file set: first-compaction files without .chain.edges, then the .clean.*
    files of the cleaned graph, whose chains are the cleaned arrays' chains"""
    fq = fixture_bytes("debruijn.bubble.fastq")
    prefix = str(tmp_path / "o")
    r = oracle.run(fq, k=31, thresh=bg.thresholds([1]), clean=True, write_prefix=prefix)
    names = sorted(p.name[2:] for p in tmp_path.iterdir())
    assert names == sorted(["branch.edges", "branch.fasta", "chain.components", "chain.fasta", "chain.summary",
                            "graph.all", "clean.branch.edges", "clean.branch.fasta", "clean.chain.components",
                            "clean.chain.fasta", "clean.chain.edges"])
    with open(prefix + ".clean.chain.fasta") as f:
        assert sorted(fasta_records(f.read())) == sorted(chain_strings(r["clean"]))
    with open(prefix + ".chain.fasta") as f:
        assert sorted(fasta_records(f.read())) == sorted(chain_strings(r))
    with open(prefix + ".clean.branch.edges") as f:
        assert len(f.read().splitlines()) == int((r["clean"]["nodes"][2] & 1).sum())


@pytest.mark.parametrize("fname,lo", [("debruijn.bubble.fastq", (1,)), ("debruijn.palindrome_chr14.fastq", ()),
                                      ("debruijn.clean1.fastq", ()), ("debruijn.clean2.fastq", (1,))])
def test_cleaned_chains_are_a_compaction_of_the_cleaned_graph(fname, lo):
    """check_compacted_files.sh's idea on the cleaned outputs: every k-mer of every cleaned chain
    is a chain node of the cleaned node table, consecutive k-mers are joined by an edge that both
    nodes hold, and every chain node of the table lies on exactly one chain (cycles created by the
    cleaning leave the graph, as compact_dbg_clean.hpp:797-806 takes them out)"""
    k = 31
    r = oracle.run(fixture_bytes(fname), k=k, thresholding=bool(lo), thresh=bg.thresholds(lo), clean=True)
    c = r["clean"]
    nodes = _node_map(c["nodes"], k)
    flags = {_ascii(c["nodes"][0][i], k): int(c["nodes"][2][i]) for i in range(len(c["nodes"][2]))}
    canon = lambda x: min(x, _rc(x))
    seen = set()
    for s in chain_strings(c):
        kmers = [s[i:i + k] for i in range(len(s) - k + 1)]
        for x in kmers:
            assert canon(x) in nodes and flags[canon(x)] & 2, x
            assert canon(x) not in seen, x
            seen.add(canon(x))
        for a, b in zip(kmers, kmers[1:]):
            # a -> b: a's out-edge to b's last base, b's in-edge from a's first base, each on its
            # stored strand
            ca, cb = canon(a), canon(b)
            out_i = "ACGT".index(b[-1]) if ca == a else 4 + 3 - "ACGT".index(b[-1])
            in_i = 4 + "ACGT".index(a[0]) if cb == b else 3 - "ACGT".index(a[0])
            assert nodes[ca][out_i] > 0 and nodes[cb][in_i] > 0, (a, b)
    # the loop takes the cycle nodes of each recompaction out of the graph, and edge-less nodes
    # go too, so every chain node left is on exactly one chain
    assert seen == {x for x, f in flags.items() if f & 2}


def test_clean_edge_cases():
    """no input; one read (a chain whose both ends lack edges is no dead end); a circular genome
    (one cycle, which the driver takes out before cleaning, leaving nothing to clean)"""
    thr = bg.thresholds([1])
    r = oracle.run(b"", k=31, thresh=thr, clean=True)
    assert r["clean_stats"] == {"rounds": 0, "deadends": 0, "bubbles": 0, "edges": 0, "status": 0}
    assert r["clean"]["n_nodes"] == 0 and r["clean"]["n_chains"] == 0
    g = _genome(200, 21)
    r = oracle.run(_fastq([g[:150]]), k=31, thresh=thr, clean=True)
    assert r["clean_stats"]["rounds"] == 0
    assert chain_strings(r["clean"]) == chain_strings(r) and len(chain_strings(r)) == 1
    circ = g + g[:60]   # reads around a circle: every k-mer has one successor and one predecessor
    reads = [circ[i:i + 100] for i in range(0, len(g), 5)]
    r = oracle.run(_fastq(reads), k=31, thresh=thr, clean=True)
    assert r["n_cycle_nodes"] == len(g) and r["n_chains"] == 0
    assert r["clean_stats"]["rounds"] == 0 and r["clean"]["n_nodes"] == 0


@pytest.mark.parametrize("fname,lo", [("debruijn.bubble.fastq", (1,)), ("debruijn.palindrome_chr14.fastq", ()),
                                      ("debruijn.clean2.fastq", (1,))])
def test_cleaned_chain_edges_follow_chain_strings(tmp_path, fname, lo):
    """the same second derivation of .chain.edges, on the cleaned graph's .clean.chain.edges"""
    k = 31
    r = oracle.run(fixture_bytes(fname), k=k, thresholding=bool(lo), thresh=bg.thresholds(lo), clean=True,
                   write_prefix=str(tmp_path / "p"))
    c = r["clean"]
    assert r["clean_stats"]["rounds"] > 0
    keys, counts, _ = c["nodes"]
    node = {_ascii(keys[i], k): counts[i] for i in range(len(keys))}
    K, rep, _ = c["ranked"]
    selfs = {}
    for i in range(len(K)):
        selfs.setdefault(_ascii(rep[i], k), []).append(int(node[min(_ascii(K[i], k), _rc(_ascii(K[i], k)))][8]))
    lines = []
    for s in chain_strings(c):
        L, R = s[:k], s[-k:]
        cl, cr = node[min(L, _rc(L))], node[min(R, _rc(R))]
        lin = list(cl[4:8]) if L <= _rc(L) else [cl[3], cl[2], cl[1], cl[0]]
        rout = list(cr[0:4]) if R <= _rc(R) else [cr[7], cr[6], cr[5], cr[4]]
        f = selfs[L]
        mean = int(np.float32(sum(f)) / np.float32(len(f)))
        lines.append(f"{L}\t{R}\t" + "".join(f"{int(v)}\t" for v in lin + rout + [mean, min(f), max(f)]) + "\n")
    assert open(tmp_path / "p.clean.chain.edges").read() == "".join(sorted(lines))
    assert len(lines) == c["n_chains"] > 0


def test_check_index_holds_on_consistent_builds():
    """check_index (compact_dbg_stats.hpp:45-119) holds on every fixture built unthresholded or
    with -L alone (the filter trims both sides of an edge alike); it can fail only where
    separate k and k+2 bounds trim an edge on one side (the reference's debug build would
    assert there), and the edge histogram covers every node"""
    import os
    from conftest import DATA, fixture_bytes
    failed_222 = 0
    for f in sorted(os.listdir(DATA)):
        if not f.endswith(".fastq"):
            continue
        for lo in ([], [1], [2], [3], [2, 2, 2]):
            r = oracle.run(fixture_bytes(f), k=31, thresholding=bool(lo), thresh=bg.thresholds(lo))
            c = r["check_index"]
            assert sum(c["edge_hist"]) == r["n_nodes"]
            assert c["n_query"] == sum(((i // 5) + (i % 5)) * v for i, v in enumerate(c["edge_hist"]))
            if len(lo) == 3:
                failed_222 += c["n_absent"] > 0
            else:
                assert c["n_absent"] == 0 and c["n_unreferenced"] == 0 and c["n_unanswered"] == 0, (f, lo, c)
    assert failed_222 > 0
