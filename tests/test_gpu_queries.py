"""The graph and chain-map queries of the boundary against the oracle: debruijn_graph::find_if /
erase_if with the node predicates (debruijn_graph_filters.hpp), debruijn_graph_map::erase_nodes
(debruijn_graph_map.hpp:833-836), debruijn_chain_graph::find_if with the chain predicates
(debruijn_chain_filters.hpp), get_cycle_node_kmers and get_isolated, and the reference driver's
sequence between ranking and output (compact_dbg_freq_construct_clean.cpp:599-610, 794-807)
replayed through the C++ facade.

The expected results are restated here in Python over the oracle's outputs: each predicate as
the reference header defines it, erase_nodes as a snapshot of the queried nodes, their removal,
and the removal of the edges their neighbours have back to them."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import bruno_gb300 as bg
from bruno_gb300 import build
from oracle import oracle
from conftest import fixture_bytes
from helpers import sort_nodes

TM = 0x80000000
DM = 0x7FFFFFFF
FIXTURES = ["debruijn.palindrome_chr14.fastq", "debruijn.shifted_cycle_chr14.fastq", "debruijn.bubble.fastq",
            "natural.fastq", "test.star.unitiqs.fastq", "debruijn.palindrome2.fastq"]


# --------------------------------------------------------------- k-mer helpers (Python ints)
def to_int(row) -> int:
    return sum(int(x) << (64 * i) for i, x in enumerate(row))


def to_row(v: int, words: int):
    return [(v >> (64 * i)) & (2 ** 64 - 1) for i in range(words)]


def rc(x: int, k: int) -> int:
    y = 0
    for _ in range(k):
        y = (y << 2) | (3 - (x & 3))
        x >>= 2
    return y


def first(x: int, k: int) -> int:
    return (x >> (2 * (k - 1))) & 3


def canon(x: int, k: int) -> int:
    return min(x, rc(x, k))


# --------------------------------------------------------------- the node predicates
def node_pred(name: str, K: int, cnt, k: int) -> bool:
    out, inn = cnt[0:4], cnt[4:8]
    dout, din = sum(1 for c in out if c), sum(1 for c in inn if c)
    kpal = k % 2 == 0 and rc(K, k) == K
    k1pal = False
    if k % 2 == 1:
        low = K & ((1 << (2 * (k - 1))) - 1)
        high = K >> 2
        low_pal, high_pal = rc(low, k - 1) == low, rc(high, k - 1) == high
        f, l = first(K, k), K & 3
        for c in range(4):
            if out[c] and low_pal and (f == 3 - c or f == c):
                k1pal = True
            if inn[c] and high_pal and (l == 3 - c or l == c):
                k1pal = True
    return {"all": True, "IsKPalindrome": kpal, "IsKplus1Palindrome": k1pal,
            "IsBranchPoint": din >= 2 or dout >= 2 or kpal or k1pal, "IsIsolated": din == 0 and dout == 0,
            "IsChainInternalNode": din == 1 and dout == 1 and not kpal and not k1pal,
            "IsChainNode": din < 2 and dout < 2 and not kpal and not k1pal}[name]


def nodes_dict(nodes) -> dict:
    keys, counts, _ = nodes
    return {to_int(keys[i]): [int(x) for x in counts[i]] for i in range(len(keys))}


def node_arrays(d: dict, k: int, words: int):
    items = sorted(d.items())
    keys = np.array([to_row(K, words) for K, _ in items], np.uint64).reshape(-1, words)
    counts = np.array([c for _, c in items], np.uint16).reshape(-1, 9)
    flags = np.array([(1 if node_pred("IsBranchPoint", K, c, k) else 0) | (2 if node_pred("IsChainNode", K, c, k) else 0)
                      for K, c in items], np.uint8)
    return keys, counts, flags


def zero_edge(d: dict, y: int, in_c, out_c, k: int):
    """zero the edge nibbles of the pair (y, in_c, out_c) on the canonical node (lex_less)"""
    r = rc(y, k)
    if not (y < r):
        y, in_c, out_c = r, (3 - out_c if out_c is not None else None), (3 - in_c if in_c is not None else None)
    n = d.get(y)
    if n is None:
        return
    if out_c is not None:
        n[out_c] = 0
    if in_c is not None:
        n[4 + in_c] = 0


def erase_nodes(d: dict, query, k: int):
    """erase_nodes(query): snapshot the found nodes, erase them, then the remote edges"""
    mask = (1 << (2 * k)) - 1
    found = {}
    for q in query:
        K = canon(q, k)
        if K in d:
            found[K] = list(d[K])
    for K in found:
        d.pop(K, None)
    for K, cnt in found.items():
        for c in range(4):
            if cnt[c]:       # out edge to K.c: that node's in edge from first(K)
                zero_edge(d, ((K << 2) | c) & mask, first(K, k), None, k)
            if cnt[4 + c]:   # in edge from c.K: that node's out edge to last(K)
                zero_edge(d, (K >> 2) | (c << (2 * (k - 1))), None, K & 3, k)


# --------------------------------------------------------------- the chain predicates
def chain_pred(name: str, K: int, inK: int, outK: int, inD: int, outD: int, k: int) -> bool:
    ti, to = (inD & DM) == 0, (outD & DM) == 0
    ptcn = lambda x: (x ^ TM) > TM
    if name in ("IsCanonicalTerminus", "IsCanonicalTerminusOrIsolated"):
        if ti and to:
            return name == "IsCanonicalTerminusOrIsolated"
        if ti:
            return K <= rc(outK, k)
        if to:
            return rc(K, k) < inK
        return False
    return {"all": True, "IsUnitLength": ti and to, "IsIsolated": inD == TM and outD == TM, "IsTerminus": ti != to,
            "IsInternal": (inD & DM) > 0 and (outD & DM) > 0, "IsTerminusOrIsolated": ti or to,
            "PointsToTermini": not ptcn(inD) and not ptcn(outD),
            "PointsToInternalNode": ptcn(inD) or ptcn(outD)}[name]


def sort_records(rec):
    K, inK, outK, inD, outD = rec
    order = np.lexsort(tuple(K.T))
    return K[order], inK[order], outK[order], inD[order], outD[order]


def select_records(rec, name, k):
    K, inK, outK, inD, outD = rec
    keep = [i for i in range(len(K)) if chain_pred(name, to_int(K[i]), to_int(inK[i]), to_int(outK[i]), int(inD[i]),
                                                   int(outD[i]), k)]
    return tuple(a[keep] for a in rec)


def same(a, b, what):
    for x, y in zip(a, b):
        assert x.shape == y.shape, (what, x.shape, y.shape)
        assert np.array_equal(x, y), what


# --------------------------------------------------------------- CPU: the restatements
def test_chain_map_counts_consistent():
    """the oracle's chain map: one canonical terminus per chain, cycle and isolated counts"""
    for f in FIXTURES:
        r = oracle.run(fixture_bytes(f), k=31, thresh=bg.thresholds([2]))
        sel = select_records(r["chain_map"], "IsCanonicalTerminusOrIsolated", 31)
        assert len(sel[0]) == r["n_chains"], f
        assert len(r["cycle_kmers"]) == r["n_cycle_nodes"] and len(r["isolated"][0]) == r["n_isolated"]
        assert len(r["chain_map"][0]) == r["n_ranked"]


def test_erase_restatement_matches_oracle_cleaning_start():
    """erase_nodes(cycle k-mers) then erase_if(IsIsolated), restated here, equals the graph the
    oracle's cleaning starts from where no cleaning round follows (no dead end, no bubble)"""
    data = fixture_bytes("debruijn.palindrome2.fastq")
    r = oracle.run(data, k=31, thresh=bg.thresholds([3]), clean=True)
    assert r["clean_stats"]["rounds"] == 0 and r["n_cycle_nodes"] > 0
    d = nodes_dict(r["nodes"])
    erase_nodes(d, [to_int(x) for x in r["cycle_kmers"]], 31)
    d = {K: c for K, c in d.items() if not node_pred("IsIsolated", K, c, 31)}
    keys, counts, _ = node_arrays(d, 31, 1)
    assert np.array_equal(keys, r["clean"]["nodes"][0]) and np.array_equal(counts, r["clean"]["nodes"][1])


# --------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("lo", [(), (2,), (3,)])
@pytest.mark.parametrize("fname", FIXTURES)
def test_gpu_queries(fname, lo):
    data = fixture_bytes(fname)
    thr = bg.thresholds(lo)
    ref = oracle.run(data, k=31, thresholding=bool(lo), thresh=thr, min_update=True)
    g = bg.Graph(k=31, thresholding=bool(lo), thresh=thr, min_update=True)
    try:
        g.reset()
        g.load_fastq(data)
        g.compute_biedge_freqencies()
        g.local_insert_by_freqencies()
        ref_nodes = nodes_dict(ref["nodes"])
        for name in bg.NODE_FILTERS:
            want = {K: c for K, c in ref_nodes.items() if node_pred(name, K, c, 31)}
            same(sort_nodes(*g.find_if(name)), node_arrays(want, 31, 1), f"find_if({name})")
        g.extract_chains()
        g.list_rank_min_update()
        g.to_compressed_chains()
        for name in bg.CHAIN_FILTERS:
            same(sort_records(g.chain_find_if(name)), select_records(ref["chain_map"], name, 31),
                 f"chain find_if({name})")
        same(sort_records(g.get_isolated()), ref["isolated"], "get_isolated")
        cyc = g.get_cycle_node_kmers()
        assert np.array_equal(cyc[np.lexsort(tuple(cyc.T))], ref["cycle_kmers"])
        # compact_dbg_freq_construct_clean.cpp:599-604: cycles and edge-less nodes out
        d = dict(ref_nodes)
        erase_nodes(d, [to_int(x) for x in ref["cycle_kmers"]], 31)
        g.erase_nodes(cyc)
        n_iso = sum(1 for K, c in d.items() if node_pred("IsIsolated", K, c, 31))
        assert g.erase_if("IsIsolated") == n_iso
        d = {K: c for K, c in d.items() if not node_pred("IsIsolated", K, c, 31)}
        same(sort_nodes(*g.nodes()), node_arrays(d, 31, 1), "after erasing cycles and isolated nodes")
        assert g.sizes()["n_nodes"] == len(d)
        # :794-807: the internal chain nodes out, then the branch points
        internal = select_records(ref["chain_map"], "IsInternal", 31)[0]
        erase_nodes(d, [to_int(x) for x in internal], 31)
        g.erase_nodes(g.chain_find_if("IsInternal")[0])
        g.erase_if("IsBranchPoint")
        d = {K: c for K, c in d.items() if not node_pred("IsBranchPoint", K, c, 31)}
        same(sort_nodes(*g.nodes()), node_arrays(d, 31, 1), "after erasing internal nodes and branch points")
    finally:
        g.close()


REPLAY = r'''
#include "bruno_gb300.hpp"
#include <cstdio>
#include <fstream>
#include <sstream>
/* the reference driver's sequence (compact_dbg_freq_construct_clean.cpp:491-610, 794-807)
 * through the facade; prints the node table after each erasure step and the chain records */
static void dump(const char *tag, bruno_gb300::debruijn_graph &g) {
  std::vector<uint64_t> keys; std::vector<uint16_t> counts; std::vector<uint8_t> flags;
  g.get_map().to_vector(keys, counts, flags);
  printf("%s %zu\n", tag, flags.size());
  for (size_t i = 0; i < flags.size(); ++i) {
    printf("%llu", (unsigned long long)keys[i]);
    for (int q = 0; q < 9; ++q) printf(" %u", counts[i * 9 + q]);
    printf("\n");
  }
}
int main(int argc, char **argv) {
  namespace bf = bruno_gb300::filter;
  std::ifstream in(argv[1], std::ios::binary);
  std::stringstream ss; ss << in.rdbuf();
  const std::string fq = ss.str();
  bruno_cfg cfg{};
  cfg.k = 31; cfg.thresholding = 1; cfg.min_update = 1;
  auto t = bruno_gb300::thresholds({2}, {});
  for (int i = 0; i < 6; ++i) cfg.thresh[i] = t[i];
  bruno_gb300::context ctx(cfg);
  bruno_gb300::debruijn_graph idx(ctx);
  bruno_gb300::debruijn_chain_graph chainmap(ctx);
  idx.get_map().load_fastq(fq.data(), fq.size());
  idx.get_map().compute_biedge_freqencies();
  idx.get_map().local_insert_by_freqencies(t);
  chainmap.extract_chains(idx);
  chainmap.list_rank_min_update();
  auto compacted = chainmap.to_ranked_chain_nodes();
  auto cycle_kmers = chainmap.get_cycle_node_kmers();
  idx.get_map().erase_nodes(cycle_kmers);
  idx.erase_if(bf::graph::IsIsolated());
  dump("after_cycles", idx);
  auto chain_rep = chainmap.find_if(bf::chain::IsCanonicalTerminusOrIsolated());
  printf("chain_rep %zu\n", chain_rep.size());
  auto internal = chainmap.get_internal_node_kmers();
  idx.get_map().erase_nodes(internal);
  idx.erase_if(bf::graph::IsBranchPoint());
  dump("after_internal", idx);
  auto branches = idx.find_if(bf::graph::IsBranchPoint());
  printf("branches %zu\n", branches.size());
  return 0;
}
'''


def _parse_dump(text: str):
    out, lines, i = {}, text.splitlines(), 0
    while i < len(lines):
        tag, n = lines[i].split()
        if tag in ("chain_rep", "branches"):
            out[tag] = int(n)
            i += 1
            continue
        rows = [list(map(int, l.split())) for l in lines[i + 1:i + 1 + int(n)]]
        out[tag] = {r[0]: r[1:] for r in rows}
        i += 1 + int(n)
    return out


@pytest.mark.gpu
def test_gpu_driver_replay_through_facade(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host C++ compiler")
    lib = build.build_library()
    src, exe = tmp_path / "replay.cpp", tmp_path / "replay"
    src.write_text(REPLAY)
    subprocess.run([gxx, "-O1", "-std=c++17", "-I", build.INCLUDE, str(src), "-o", str(exe), "-L", os.path.dirname(lib),
                    "-lbruno_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    fname = "debruijn.shifted_cycle_chr14.fastq"
    fq = tmp_path / fname
    fq.write_bytes(fixture_bytes(fname))
    got = _parse_dump(subprocess.run([str(exe), str(fq)], capture_output=True, text=True, check=True).stdout)
    ref = oracle.run(fixture_bytes(fname), k=31, thresh=bg.thresholds([2]))
    d = nodes_dict(ref["nodes"])
    erase_nodes(d, [to_int(x) for x in ref["cycle_kmers"]], 31)
    d = {K: c for K, c in d.items() if not node_pred("IsIsolated", K, c, 31)}
    assert got["after_cycles"] == d
    assert got["chain_rep"] == ref["n_chains"]
    erase_nodes(d, [to_int(x) for x in select_records(ref["chain_map"], "IsInternal", 31)[0]], 31)
    d = {K: c for K, c in d.items() if not node_pred("IsBranchPoint", K, c, 31)}
    assert got["after_internal"] == d
    assert got["branches"] == 0
