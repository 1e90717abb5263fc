"""bruno_count_biedges_noalloc, the allocation-free pair counter, against the context path.

The context path (bruno_load_fastq + bruno_compute_biedge_freqencies + bruno_copy_k2) gives
every distinct canonical (k-mer, biedge) pair of a read set with its count.  Expanding those
counts back into the individual pairs, shuffled, and counting them again through the
allocation-free entry point must give the same multiset exactly (integer counts: the
tolerance is zero).  Each test makes two calls in a row, so the second one also checks that
the first left nothing behind in the library's scratch table.  The file name sorts last, so
it runs after every other test; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

import bruno_gb300 as bg
from bruno_gb300 import synth

pytestmark = pytest.mark.gpu

MAX_PAIRS = {31: (((32 << 20) - (64 << 10)) // 32) // 2, 63: (((32 << 20) - (64 << 10)) // 64) // 2}


def _context_k2(fq, k):
    g = bg.Graph(k=k, keep_k2=True)
    try:
        g.load_fastq(fq)
        g.compute_biedge_freqencies()
        return g.k2()
    finally:
        g.close()


def _noalloc(torch, k, keys, edges, out_cap=None):
    """one call through the C ABI with device inputs and outputs; returns (status, n, triple)"""
    lib = bg.load_library()
    words = bg.kmer_words(k)
    n = len(edges)
    dk = torch.from_numpy(np.ascontiguousarray(keys.reshape(-1), dtype=np.uint64).view(np.int64)).cuda()
    de = torch.from_numpy(np.ascontiguousarray(edges, dtype=np.uint8)).cuda()
    cap = n if out_cap is None else out_cap
    ok = torch.zeros(max(1, cap) * words, dtype=torch.int64, device="cuda")
    oe = torch.zeros(max(1, cap), dtype=torch.uint8, device="cuda")
    oc = torch.zeros(max(1, cap), dtype=torch.int32, device="cuda")
    n_out = ctypes.c_size_t(0)
    stream = torch.cuda.current_stream()
    st = lib.bruno_count_biedges_noalloc(0, k, ctypes.c_void_p(dk.data_ptr()), ctypes.c_void_p(de.data_ptr()), n,
                                         ctypes.c_void_p(ok.data_ptr()), ctypes.c_void_p(oe.data_ptr()),
                                         ctypes.c_void_p(oc.data_ptr()), cap, ctypes.byref(n_out),
                                         ctypes.c_void_p(stream.cuda_stream))
    m = min(n_out.value, cap)
    out = (ok.cpu().numpy().view(np.uint64)[: m * words].reshape(m, words), oe.cpu().numpy()[:m],
           oc.cpu().numpy().view(np.uint32)[:m])
    return st, n_out.value, out


def _sorted(keys, edges, counts):
    keys = np.asarray(keys, dtype=np.uint64)
    cols = [np.asarray(counts, np.uint64), np.asarray(edges, np.uint64)]
    cols += [keys[:, w] for w in range(keys.shape[1])] if keys.ndim == 2 else [keys]
    order = np.lexsort(cols)
    return keys[order], np.asarray(edges)[order], np.asarray(counts)[order]


def _expand(keys, edges, counts, seed):
    rng = np.random.default_rng(seed)
    idx = np.repeat(np.arange(len(edges)), np.asarray(counts, np.int64))
    rng.shuffle(idx)
    return keys[idx], edges[idx]


def _workload(k, reads, seed):
    return synth.Workload(f"noalloc-k{k}", 20_000, 100, reads, 0.01, k, (2,), seed=seed)


@pytest.mark.parametrize("k,reads", [(31, 6000), (63, 6000)])
def test_noalloc_matches_context_path(k, reads):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    for call, seed in enumerate((11, 12)):   # two calls in a row, different read sets
        fq = synth.make_fastq(_workload(k, reads, seed))
        keys, edges, counts = _context_k2(fq, k)
        pk, pe = _expand(keys, edges, counts, seed)
        assert 0 < len(pe) <= MAX_PAIRS[k]
        st, n_out, got = _noalloc(torch, k, pk, pe)
        assert st == 0, f"call {call}: status {st}"
        assert n_out == len(edges), f"call {call}: {n_out} distinct pairs, context path has {len(edges)}"
        want = _sorted(keys, edges, counts)
        have = _sorted(*got)
        for a, b in zip(want, have):
            np.testing.assert_array_equal(a, b)


def test_noalloc_limits_and_errors():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    fq = synth.make_fastq(_workload(31, 500, 13))
    keys, edges, counts = _context_k2(fq, 31)
    pk, pe = _expand(keys, edges, counts, 13)
    # output buffer one pair short: BRUNO_ERR_CAPACITY, and n_out still reports the count
    st, n_out, _ = _noalloc(torch, 31, pk, pe, out_cap=len(edges) - 1)
    assert st == 8 and n_out == len(edges)
    # an edge nibble that is not a DNA16 base: BRUNO_ERR_BAD_INPUT
    bad = pe.copy()
    bad[len(bad) // 2] = 0x33
    st, _, _ = _noalloc(torch, 31, pk, bad)
    assert st == 2
    # the next call is clean again
    st, n_out, got = _noalloc(torch, 31, pk, pe)
    assert st == 0 and n_out == len(edges)
    for a, b in zip(_sorted(keys, edges, counts), _sorted(*got)):
        np.testing.assert_array_equal(a, b)
    # more pairs than the scratch table takes: refused on the host before any launch
    lib = bg.load_library()
    n_out = ctypes.c_size_t(7)
    one = torch.zeros(2, dtype=torch.int64, device="cuda")
    st = lib.bruno_count_biedges_noalloc(0, 31, ctypes.c_void_p(one.data_ptr()), ctypes.c_void_p(one.data_ptr()),
                                         MAX_PAIRS[31] + 1, None, None, None, 0, ctypes.byref(n_out), None)
    assert st == 8 and n_out.value == 0
