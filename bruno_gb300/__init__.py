"""GB300 de Bruijn graph construction and compaction: the Python host binding.

A thin ctypes layer over the C ABI in ``include/bruno_gb300.h``; the work runs in the
CUDA library ``_lib/libbruno_gb300.so``.  There is no CPU fallback: if the library is
missing or no GPU is present, calls raise.

The step names follow ParBLiSS/bruno's src/debruijn API (debruijn_graph_map::
compute_biedge_freqencies / local_insert_by_freqencies, debruijn_chain_graph::
extract_chains / list_rank_min_update / list_rank / to_ranked_chain_nodes /
to_compressed_chains), so a driver written against the reference reads the same.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libbruno_gb300.so")

STATUS = {
    0: "OK", 1: "ARG", 2: "BAD_INPUT", 3: "OOM", 4: "TABLE_FULL", 5: "RANK_NOT_CONVERGED",
    6: "INVARIANT", 7: "CUDA", 8: "CAPACITY",
}
COUNT_MAX = 65535  # CountType = uint16 (compact_dbg_freq_construct_clean.cpp:187)


class BrunoError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"bruno_gb300 {STATUS.get(status, status)}: {message}")
        self.status = status
        self.message = message


class _Cfg(ctypes.Structure):
    _fields_ = [
        ("k", ctypes.c_int32), ("thresholding", ctypes.c_int32), ("thresh", ctypes.c_uint64 * 6),
        ("min_update", ctypes.c_int32), ("device", ctypes.c_int32), ("table_slots", ctypes.c_uint64),
        ("max_load", ctypes.c_double), ("keep_k2", ctypes.c_int32), ("keep_filtered", ctypes.c_int32),
        ("exact_ranking", ctypes.c_int32), ("direct_count", ctypes.c_int32), ("edge_filter", ctypes.c_int32),
        ("h2d_chunk", ctypes.c_uint64), ("h2d_streams", ctypes.c_int32), ("rank_fill", ctypes.c_int32),
        ("part_slots", ctypes.c_int32), ("count_threads", ctypes.c_int32),
    ]


class _Sizes(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "n_reads", "n_reads_used", "n_instances", "n_k2", "n_filtered", "n_nodes", "n_branch",
        "n_chain_nodes", "iterations", "n_cycle_nodes", "n_isolated", "n_ranked", "n_chains",
        "n_chain_chars", "table_slots", "collisions")] + [("filter_flag_hist", ctypes.c_uint64 * 16),
                                                    ("launches", ctypes.c_uint64),
                                                    ("table_partitions", ctypes.c_uint64),
                                                    ("grouped_chains", ctypes.c_uint64),
                                                    ("filter_slots_read", ctypes.c_uint64)]


class _PoolResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("worker", ctypes.c_int32), ("words", ctypes.c_int32), ("sizes", _Sizes),
                ("n_chains", ctypes.c_uint64), ("n_chars", ctypes.c_uint64), ("reps", ctypes.POINTER(ctypes.c_uint64)),
                ("offsets", ctypes.POINTER(ctypes.c_uint64)), ("chars", ctypes.POINTER(ctypes.c_char)),
                ("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double)]


class _CleanStats(ctypes.Structure):
    _fields_ = [("rounds", ctypes.c_uint64), ("deadends", ctypes.c_uint64), ("bubbles", ctypes.c_uint64),
                ("edges", ctypes.c_uint64), ("status", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class _DeviceView(ctypes.Structure):
    _fields_ = [("ranked_K", ctypes.c_void_p), ("ranked_rep", ctypes.c_void_p), ("ranked_dist", ctypes.c_void_p),
                ("chain_reps", ctypes.c_void_p), ("chain_offsets", ctypes.c_void_p), ("chain_chars", ctypes.c_void_p),
                ("n_ranked", ctypes.c_uint64), ("n_chains", ctypes.c_uint64), ("n_chain_chars", ctypes.c_uint64),
                ("words", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class _IndexCheck(ctypes.Structure):
    _fields_ = [("n_query", ctypes.c_uint64), ("n_absent", ctypes.c_uint64), ("n_unreferenced", ctypes.c_uint64),
                ("n_unanswered", ctypes.c_uint64), ("edge_hist", ctypes.c_uint64 * 25)]


_lib: Optional[ctypes.CDLL] = None

# every entry point of include/bruno_gb300.h
EXPORTS = (
    "bruno_ctx_create", "bruno_ctx_destroy", "bruno_set_stream", "bruno_last_error", "bruno_reset",
    "bruno_load_fastq", "bruno_compute_biedge_freqencies", "bruno_local_insert_by_freqencies",
    "bruno_extract_chains", "bruno_list_rank", "bruno_to_compressed_chains", "bruno_build_and_compact",
    "bruno_get_sizes", "bruno_copy_k2", "bruno_copy_filtered", "bruno_copy_nodes", "bruno_copy_ranked",
    "bruno_copy_chains", "bruno_copy_chain_edges", "bruno_copy_chain_summaries", "bruno_host_alloc", "bruno_host_free", "bruno_phase_ms",
    "bruno_count_biedges_noalloc", "bruno_pool_create", "bruno_pool_submit", "bruno_pool_wait",
    "bruno_pool_result_free", "bruno_pool_destroy", "bruno_clean_deadend_and_bubbles_naive",
    "bruno_device_results", "bruno_graph_find_if", "bruno_graph_erase_if", "bruno_graph_erase_nodes",
    "bruno_chain_find_if", "bruno_get_cycle_node_kmers", "bruno_get_isolated", "bruno_check_index",
    "bruno_build_samples", "bruno_sample_count", "bruno_sample_sizes", "bruno_sample_copy_ranked",
    "bruno_sample_copy_chains", "bruno_sample_copy_nodes", "bruno_pool_create_batched", "bruno_sample_ranges",
)

# node predicates (bliss::debruijn::filter::graph) and chain predicates
# (bliss::debruijn::filter::chain) as the C ABI numbers them
NODE_FILTERS = {"all": 0, "IsKPalindrome": 1, "IsKplus1Palindrome": 2, "IsBranchPoint": 3, "IsIsolated": 4,
                "IsChainInternalNode": 5, "IsChainNode": 6}
CHAIN_FILTERS = {"all": 0, "IsUnitLength": 1, "IsIsolated": 2, "IsTerminus": 3, "IsInternal": 4,
                 "IsTerminusOrIsolated": 5, "IsCanonicalTerminus": 6, "IsCanonicalTerminusOrIsolated": 7,
                 "PointsToTermini": 8, "PointsToInternalNode": 9}


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads the CUDA library (built by ``__graft_entry__.build()``); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise BrunoError(1, f"CUDA library not built: {path} (run __graft_entry__.build())")
    lib = ctypes.CDLL(path)
    P, U64, I32, SZ = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_size_t
    PSZ = ctypes.POINTER(ctypes.c_size_t)
    sig = {
        "bruno_ctx_create": [ctypes.POINTER(_Cfg), ctypes.POINTER(P)],
        "bruno_ctx_destroy": [P], "bruno_set_stream": [P, P], "bruno_reset": [P],
        "bruno_load_fastq": [P, P, SZ, I32], "bruno_compute_biedge_freqencies": [P],
        "bruno_local_insert_by_freqencies": [P, P], "bruno_extract_chains": [P],
        "bruno_list_rank": [P, I32, ctypes.POINTER(U64)], "bruno_to_compressed_chains": [P],
        "bruno_build_and_compact": [P, P, SZ, I32], "bruno_get_sizes": [P, ctypes.POINTER(_Sizes)],
        "bruno_copy_k2": [P, P, P, P, SZ, PSZ], "bruno_copy_filtered": [P, P, P, P, SZ, PSZ],
        "bruno_copy_nodes": [P, P, P, P, SZ, PSZ], "bruno_copy_ranked": [P, P, P, P, SZ, PSZ],
        "bruno_copy_chains": [P, P, P, P, SZ, SZ, PSZ, PSZ],
        "bruno_copy_chain_edges": [P, P, P, SZ, PSZ],
        "bruno_copy_chain_summaries": [P, P, P, P, SZ, PSZ],
        "bruno_host_alloc": [SZ, ctypes.POINTER(P)], "bruno_host_free": [P],
        "bruno_phase_ms": [P, ctypes.POINTER(ctypes.c_double), SZ],
        "bruno_count_biedges_noalloc": [I32, I32, P, P, SZ, P, P, P, SZ, PSZ, P],
        "bruno_pool_create": [ctypes.POINTER(_Cfg), I32, U64, ctypes.POINTER(P)],
        "bruno_pool_submit": [P, P, SZ, ctypes.POINTER(U64)],
        "bruno_pool_wait": [P, U64, ctypes.POINTER(_PoolResult)], "bruno_pool_result_free": [ctypes.POINTER(_PoolResult)],
        "bruno_pool_destroy": [P],
        "bruno_clean_deadend_and_bubbles_naive": [P, ctypes.POINTER(_CleanStats)],
        "bruno_device_results": [P, ctypes.POINTER(_DeviceView)],
        "bruno_graph_find_if": [P, I32, P, P, P, SZ, PSZ], "bruno_graph_erase_if": [P, I32, PSZ],
        "bruno_graph_erase_nodes": [P, P, SZ],
        "bruno_chain_find_if": [P, I32, P, P, P, P, P, SZ, PSZ],
        "bruno_get_cycle_node_kmers": [P, P, SZ, PSZ], "bruno_get_isolated": [P, P, P, P, P, P, SZ, PSZ],
        "bruno_check_index": [P, ctypes.POINTER(_IndexCheck)],
        "bruno_build_samples": [P, ctypes.POINTER(P), ctypes.POINTER(SZ), SZ, I32],
        "bruno_sample_count": [P, PSZ], "bruno_sample_sizes": [P, SZ, ctypes.POINTER(_Sizes)],
        "bruno_sample_copy_ranked": [P, SZ, P, P, P, SZ, PSZ],
        "bruno_sample_copy_chains": [P, SZ, P, P, P, SZ, SZ, PSZ, PSZ],
        "bruno_sample_copy_nodes": [P, SZ, P, P, P, SZ, PSZ],
        "bruno_pool_create_batched": [ctypes.POINTER(_Cfg), ctypes.c_uint32, U64, ctypes.POINTER(P)],
        "bruno_sample_ranges": [P, P, P, P],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    lib.bruno_last_error.argtypes = [P]
    lib.bruno_last_error.restype = ctypes.c_char_p
    _lib = lib
    return lib


def thresholds(lower: Sequence[int] = (), upper: Sequence[int] = (), count_max: int = COUNT_MAX) -> list[int]:
    """The reference driver's -L/-U handling (compact_dbg_freq_construct_clean.cpp:874,937-961):
    one value = the (k+1)-mer bound (and k / k+2 lower bounds drop to 0), three values =
    k, k+1, k+2.  Order: k_lo, k_hi, k1_lo, k1_hi, k2_lo, k2_hi."""
    t = [count_max + 1] * 6
    lower, upper = list(lower), list(upper)
    if len(lower) == 1:
        t[2] = min(lower[0], t[2])
        t[0] = t[4] = 0
    elif len(lower) == 3:
        t[0], t[2], t[4] = (min(v, c) for v, c in zip(lower, (t[0], t[2], t[4])))
    elif lower:
        raise ValueError("lower thresholds take 1 or 3 values")
    if len(upper) == 1:
        t[3] = min(upper[0], t[3])
    elif len(upper) == 3:
        t[1], t[3], t[5] = (min(v, c) for v, c in zip(upper, (t[1], t[3], t[5])))
    elif upper:
        raise ValueError("upper thresholds take 1 or 3 values")
    return t


def kmer_words(k: int) -> int:
    return 1 if k <= 31 else 2


def decode_kmers(words: np.ndarray, k: int) -> list[str]:
    """2-bit packed k-mers (n x words uint64, low word first) -> strings."""
    w = words.reshape(len(words), -1) if words.ndim == 1 else words
    out = []
    for row in w:
        v = int(row[0]) | (int(row[1]) << 64 if len(row) > 1 else 0)
        out.append("".join("ACGT"[(v >> (2 * (k - 1 - i))) & 3] for i in range(k)))
    return out


@dataclass
class GraphConfig:
    k: int = 31
    thresholding: bool = True
    thresh: list = field(default_factory=lambda: thresholds([2]))
    min_update: bool = True
    device: int = 0
    table_slots: int = 0
    max_load: float = 0.5
    keep_k2: bool = False
    keep_filtered: bool = False
    exact_ranking: bool = False
    direct_count: int = 0          # 0 automatic, 1 whole-table counting, 2 L2 partitions (k <= 31)
    edge_filter: bool = False      # the blocked driver's (k+1)-mer filter build
    h2d_chunk: int = 0             # host FASTQ copied and parsed in pieces of this many bytes (0 = 256 MiB)
    h2d_streams: int = 1           # copy streams the pieces are spread over (1..4)
    rank_fill: int = 0             # ranking's final states: 0 = second walk, 1 = one pass over the nodes
    part_slots: int = 0            # most slots of one shared-memory table partition (256..3072; 0 = 3072)
    count_threads: int = 0         # threads of a partition's counting block (256, 512, 1024; 0 = 512)

    def to_c(self) -> _Cfg:
        c = _Cfg()
        c.k, c.thresholding, c.min_update, c.device = self.k, int(self.thresholding), int(self.min_update), self.device
        for i, v in enumerate(self.thresh):
            c.thresh[i] = int(min(v, 2**64 - 1))
        c.table_slots, c.max_load = self.table_slots, self.max_load
        c.keep_k2, c.keep_filtered = int(self.keep_k2), int(self.keep_filtered)
        c.exact_ranking = int(self.exact_ranking)
        c.direct_count = int(self.direct_count)
        c.edge_filter = int(self.edge_filter)
        c.h2d_chunk = int(self.h2d_chunk)
        c.h2d_streams = int(self.h2d_streams)
        c.rank_fill = int(self.rank_fill)
        c.part_slots = int(self.part_slots)
        c.count_threads = int(self.count_threads)
        return c


class Graph:
    """One de Bruijn graph build on one GPU (a bruno_ctx)."""

    def __init__(self, config: Optional[GraphConfig] = None, **kw):
        self.lib = load_library()
        self.config = config or GraphConfig(**kw)
        self.words = kmer_words(self.config.k)
        self._cfg = self.config.to_c()
        h = ctypes.c_void_p()
        self._check(self.lib.bruno_ctx_create(ctypes.byref(self._cfg), ctypes.byref(h)), "ctx_create")
        self.ctx = h
        self._keep = []

    # ------------------------------------------------------------------ plumbing
    def _check(self, status: int, what: str) -> None:
        if status != 0:
            msg = what
            if getattr(self, "ctx", None):
                m = self.lib.bruno_last_error(self.ctx)
                msg = f"{what}: {m.decode() if m else ''}"
            raise BrunoError(status, msg)

    def close(self) -> None:
        if getattr(self, "ctx", None):
            self.lib.bruno_ctx_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int) -> None:
        """Runs later calls on an existing cudaStream_t (e.g. torch's current stream)."""
        self._check(self.lib.bruno_set_stream(self.ctx, ctypes.c_void_p(int(stream_handle))), "set_stream")

    # ------------------------------------------------------------------ steps
    def reset(self) -> None:
        self._keep.clear()
        self._check(self.lib.bruno_reset(self.ctx), "reset")

    def load_fastq(self, data, nbytes: Optional[int] = None, is_device: bool = False) -> None:
        """Adds one FASTQ file (bytes / uint8 array on the host, or a device address)."""
        if is_device:
            self._check(self.lib.bruno_load_fastq(self.ctx, ctypes.c_void_p(int(data)), int(nbytes), 1), "load_fastq")
            return
        arr = np.frombuffer(data, dtype=np.uint8) if isinstance(data, (bytes, bytearray, memoryview)) else data
        arr = np.ascontiguousarray(arr, dtype=np.uint8)
        self._keep.append(arr)
        self._check(self.lib.bruno_load_fastq(self.ctx, arr.ctypes.data_as(ctypes.c_void_p), arr.nbytes, 0),
                    "load_fastq")

    def compute_biedge_freqencies(self) -> int:
        self._check(self.lib.bruno_compute_biedge_freqencies(self.ctx), "compute_biedge_freqencies")
        return self.sizes()["n_k2"]

    def local_insert_by_freqencies(self, threshes: Optional[Sequence[int]] = None) -> int:
        p = None
        if threshes is not None:
            t = (ctypes.c_uint64 * 6)(*[int(min(v, 2**64 - 1)) for v in threshes])
            p = ctypes.cast(t, ctypes.c_void_p)
        self._check(self.lib.bruno_local_insert_by_freqencies(self.ctx, p), "local_insert_by_freqencies")
        return self.sizes()["n_nodes"]

    def extract_chains(self) -> None:
        self._check(self.lib.bruno_extract_chains(self.ctx), "extract_chains")

    def _rank(self, min_update: bool) -> int:
        it = ctypes.c_uint64()
        self._check(self.lib.bruno_list_rank(self.ctx, int(min_update), ctypes.byref(it)), "list_rank")
        return it.value

    def list_rank_min_update(self) -> int:
        return self._rank(True)

    def list_rank(self) -> int:
        return self._rank(False)

    def to_compressed_chains(self) -> None:
        self._check(self.lib.bruno_to_compressed_chains(self.ctx), "to_compressed_chains")

    def device_results(self) -> dict:
        """device addresses (ints) and sizes of the listranked nodes and compacted chains, read-only,
        valid until the context is rebuilt or changed"""
        v = _DeviceView()
        self._check(self.lib.bruno_device_results(self.ctx, ctypes.byref(v)), "device_results")
        return {n: (int(getattr(v, n) or 0)) for n, _ in _DeviceView._fields_ if n != "reserved"}

    def clean_deadend_and_bubbles_naive(self) -> dict:
        """The _freq_clean driver's graph cleaning (compact_dbg_clean.hpp:575-890) on the ranked
        graph; afterwards every copy returns the cleaned graph.  Returns the loop's tallies."""
        s = _CleanStats()
        st = self.lib.bruno_clean_deadend_and_bubbles_naive(self.ctx, ctypes.byref(s))
        out = {n: int(getattr(s, n)) for n in ("rounds", "deadends", "bubbles", "edges", "status")}
        try:
            self._check(st, "clean_deadend_and_bubbles_naive")
        except BrunoError as e:
            e.stats = out      # status 2: declined (chain pointers not mutually consistent)
            raise
        return out

    def build_and_compact(self, data, nbytes: Optional[int] = None, is_device: bool = False) -> None:
        """The whole plain path; host bytes are copied in, device bytes are read in place."""
        if is_device:
            self._check(self.lib.bruno_build_and_compact(self.ctx, ctypes.c_void_p(int(data)), int(nbytes), 1),
                        "build_and_compact")
            return
        arr = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8) if isinstance(data, (bytes, bytearray))
                                   else data, dtype=np.uint8)
        self._keep = [arr]
        self._check(self.lib.bruno_build_and_compact(self.ctx, arr.ctypes.data_as(ctypes.c_void_p), arr.nbytes, 0),
                    "build_and_compact")

    # ------------------------------------------------------------------ batched form
    def build_samples(self, samples, is_device: bool = False, nbytes=None) -> None:
        """The batched form: every sample (bytes / uint8 arrays, or device addresses with their
        sizes in nbytes) built in one pass; each sample's results are those of its plain build."""
        n = len(samples)
        ptrs = (ctypes.c_void_p * max(1, n))()
        sizes = (ctypes.c_size_t * max(1, n))()
        keep = []
        for i, x in enumerate(samples):
            if is_device:
                ptrs[i], sizes[i] = int(x), int(nbytes[i])
                continue
            arr = np.ascontiguousarray(np.frombuffer(x, dtype=np.uint8) if isinstance(x, (bytes, bytearray)) else x,
                                       dtype=np.uint8)
            keep.append(arr)
            ptrs[i], sizes[i] = arr.ctypes.data, arr.nbytes
        self._keep = keep
        self._check(self.lib.bruno_build_samples(self.ctx, ptrs, sizes, n, int(is_device)), "build_samples")

    def sample_count(self) -> int:
        n = ctypes.c_size_t()
        self._check(self.lib.bruno_sample_count(self.ctx, ctypes.byref(n)), "sample_count")
        return n.value

    def sample_sizes(self, sample: int) -> dict:
        s = _Sizes()
        self._check(self.lib.bruno_sample_sizes(self.ctx, sample, ctypes.byref(s)), "sample_sizes")
        d = {n: getattr(s, n) for n, _ in _Sizes._fields_ if n != "filter_flag_hist"}
        d["filter_flag_hist"] = list(s.filter_flag_hist)
        return d

    def batch_chains(self) -> list:
        """every sample's compacted chains (reps, offsets, chars) from one copy of the batch's chains"""
        n = self.sample_count()
        c0 = np.zeros(n + 1, np.uint64)
        ch0 = np.zeros(n + 1, np.uint64)
        self._check(self.lib.bruno_sample_ranges(self.ctx, None, self._ptr(c0), self._ptr(ch0)), "sample_ranges")
        reps, offs, chars = self.chains()
        out = []
        for i in range(n):
            a, b = int(c0[i]), int(c0[i + 1])
            base = int(ch0[i])
            out.append((reps[a:b], offs[a:b + 1] - np.uint64(base), chars[base:int(ch0[i + 1])]))
        return out

    def sample_ranked(self, sample: int):
        n = ctypes.c_size_t()
        fn = self.lib.bruno_sample_copy_ranked
        self._check(fn(self.ctx, sample, None, None, None, 0, ctypes.byref(n)), "sample_copy_ranked")
        K = np.zeros((n.value, self.words), np.uint64)
        rep = np.zeros((n.value, self.words), np.uint64)
        dist = np.zeros(n.value, np.int32)
        if n.value:
            self._check(fn(self.ctx, sample, self._ptr(K), self._ptr(rep), self._ptr(dist), n.value, ctypes.byref(n)),
                        "sample_copy_ranked")
        return K, rep, dist

    def sample_chains(self, sample: int):
        nc, nch = ctypes.c_size_t(), ctypes.c_size_t()
        fn = self.lib.bruno_sample_copy_chains
        self._check(fn(self.ctx, sample, None, None, None, 0, 0, ctypes.byref(nc), ctypes.byref(nch)),
                    "sample_copy_chains")
        reps = np.zeros((nc.value, self.words), np.uint64)
        offs = np.zeros(nc.value + 1, np.uint64)
        chars = np.zeros(max(1, nch.value), np.uint8)
        if nc.value:
            self._check(fn(self.ctx, sample, self._ptr(reps), self._ptr(offs), self._ptr(chars), nc.value, chars.size,
                           ctypes.byref(nc), ctypes.byref(nch)), "sample_copy_chains")
        return reps, offs, chars[:nch.value]

    def sample_nodes(self, sample: int):
        n = ctypes.c_size_t()
        fn = self.lib.bruno_sample_copy_nodes
        self._check(fn(self.ctx, sample, None, None, None, 0, ctypes.byref(n)), "sample_copy_nodes")
        keys = np.zeros((n.value, self.words), np.uint64)
        counts = np.zeros((n.value, 9), np.uint16)
        flags = np.zeros(n.value, np.uint8)
        if n.value:
            self._check(fn(self.ctx, sample, self._ptr(keys), self._ptr(counts), self._ptr(flags), n.value,
                           ctypes.byref(n)), "sample_copy_nodes")
        return keys, counts, flags

    def run(self, *files) -> "Graph":
        """load every file, then count, filter, extract, rank and compress"""
        self.reset()
        for f in files:
            self.load_fastq(f)
        self.compute_biedge_freqencies()
        self.local_insert_by_freqencies()
        self.extract_chains()
        self._rank(self.config.min_update)
        self.to_compressed_chains()
        return self

    # ------------------------------------------------------------------ results
    def sizes(self) -> dict:
        s = _Sizes()
        self._check(self.lib.bruno_get_sizes(self.ctx, ctypes.byref(s)), "get_sizes")
        d = {n: getattr(s, n) for n, _ in _Sizes._fields_ if n != "filter_flag_hist"}
        d["filter_flag_hist"] = list(s.filter_flag_hist)
        return d

    PHASES = ("parse", "count_k2mers", "filter_insert", "chainmap", "list_rank", "compress",
              "count_estimate", "count_table_init", "count_insert", "count_split", "h2d")

    def phase_ms(self) -> dict:
        a = (ctypes.c_double * len(self.PHASES))()
        self._check(self.lib.bruno_phase_ms(self.ctx, a, len(self.PHASES)), "phase_ms")
        return dict(zip(self.PHASES, list(a)))

    def _ptr(self, a: np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)

    def _triple(self, fn, what):
        n = ctypes.c_size_t()
        self._check(fn(self.ctx, None, None, None, 0, ctypes.byref(n)), what)
        keys = np.zeros((n.value, self.words), np.uint64)
        edges = np.zeros(n.value, np.uint8)
        counts = np.zeros(n.value, np.uint32)
        if n.value:
            self._check(fn(self.ctx, self._ptr(keys), self._ptr(edges), self._ptr(counts), n.value, ctypes.byref(n)),
                        what)
        return keys, edges, counts

    def k2(self):
        """raw canonical (k-mer, biedge) counts: keys (n, words), edges, counts"""
        return self._triple(self.lib.bruno_copy_k2, "copy_k2")

    def filtered(self):
        return self._triple(self.lib.bruno_copy_filtered, "copy_filtered")

    def nodes(self):
        """graph nodes: keys (n, words), counts (n, 9) = out ACGT, in ACGT, self; flags"""
        n = ctypes.c_size_t()
        self._check(self.lib.bruno_copy_nodes(self.ctx, None, None, None, 0, ctypes.byref(n)), "copy_nodes")
        keys = np.zeros((n.value, self.words), np.uint64)
        counts = np.zeros((n.value, 9), np.uint16)
        flags = np.zeros(n.value, np.uint8)
        if n.value:
            self._check(self.lib.bruno_copy_nodes(self.ctx, self._ptr(keys), self._ptr(counts), self._ptr(flags),
                                                  n.value, ctypes.byref(n)), "copy_nodes")
        return keys, counts, flags

    # ------------------------------------------------- graph and chain-map queries
    def check_index(self) -> dict:
        """check_index (compact_dbg_stats.hpp:45-119) and the edge-count histogram; "ok" is False
        where the reference's debug build would assert (the library returns BRUNO_ERR_INVARIANT)"""
        r = _IndexCheck()
        st = self.lib.bruno_check_index(self.ctx, ctypes.byref(r))
        if st not in (0, 6):
            self._check(st, "check_index")
        d = {n: int(getattr(r, n)) for n, _ in _IndexCheck._fields_ if n != "edge_hist"}
        d["edge_hist"] = list(r.edge_hist)
        d["ok"] = st == 0
        return d

    def find_if(self, pred: str):
        """debruijn_graph::find_if(pred): the matching nodes as nodes() gives them"""
        f = NODE_FILTERS[pred]
        n = ctypes.c_size_t()
        self._check(self.lib.bruno_graph_find_if(self.ctx, f, None, None, None, 0, ctypes.byref(n)), "graph_find_if")
        keys = np.zeros((n.value, self.words), np.uint64)
        counts = np.zeros((n.value, 9), np.uint16)
        flags = np.zeros(n.value, np.uint8)
        if n.value:
            self._check(self.lib.bruno_graph_find_if(self.ctx, f, self._ptr(keys), self._ptr(counts), self._ptr(flags),
                                                     n.value, ctypes.byref(n)), "graph_find_if")
        return keys, counts, flags

    def erase_if(self, pred: str) -> int:
        """debruijn_graph::erase_if(pred); returns the number of nodes erased"""
        n = ctypes.c_size_t()
        self._check(self.lib.bruno_graph_erase_if(self.ctx, NODE_FILTERS[pred], ctypes.byref(n)), "graph_erase_if")
        return n.value

    def erase_nodes(self, kmers) -> None:
        """debruijn_graph_map::erase_nodes(query): k-mers (n, words), either strand"""
        q = np.ascontiguousarray(np.asarray(kmers, np.uint64).reshape(-1, self.words))
        self._check(self.lib.bruno_graph_erase_nodes(self.ctx, self._ptr(q), len(q)), "graph_erase_nodes")

    def _chain_records(self, fn, what, *lead):
        n = ctypes.c_size_t()
        self._check(fn(self.ctx, *lead, None, None, None, None, None, 0, ctypes.byref(n)), what)
        K = np.zeros((n.value, self.words), np.uint64)
        inK = np.zeros((n.value, self.words), np.uint64)
        outK = np.zeros((n.value, self.words), np.uint64)
        inD = np.zeros(n.value, np.uint32)
        outD = np.zeros(n.value, np.uint32)
        if n.value:
            self._check(fn(self.ctx, *lead, self._ptr(K), self._ptr(inK), self._ptr(outK), self._ptr(inD),
                           self._ptr(outD), n.value, ctypes.byref(n)), what)
        return K, inK, outK, inD, outD

    def chain_find_if(self, pred: str):
        """debruijn_chain_graph::find_if(pred): records (K, inK, outK, inDist, outDist)"""
        return self._chain_records(self.lib.bruno_chain_find_if, "chain_find_if", CHAIN_FILTERS[pred])

    def get_isolated(self):
        """debruijn_chain_graph::get_isolated(): records as chain_find_if gives them"""
        return self._chain_records(self.lib.bruno_get_isolated, "get_isolated")

    def get_cycle_node_kmers(self):
        """debruijn_chain_graph::get_cycle_node_kmers(): k-mers (n, words)"""
        n = ctypes.c_size_t()
        self._check(self.lib.bruno_get_cycle_node_kmers(self.ctx, None, 0, ctypes.byref(n)), "get_cycle_node_kmers")
        K = np.zeros((n.value, self.words), np.uint64)
        if n.value:
            self._check(self.lib.bruno_get_cycle_node_kmers(self.ctx, self._ptr(K), n.value, ctypes.byref(n)),
                        "get_cycle_node_kmers")
        return K

    def ranked(self):
        """listranked chain nodes: K (n, words), rep (n, words), dist"""
        n = ctypes.c_size_t()
        self._check(self.lib.bruno_copy_ranked(self.ctx, None, None, None, 0, ctypes.byref(n)), "copy_ranked")
        K = np.zeros((n.value, self.words), np.uint64)
        rep = np.zeros((n.value, self.words), np.uint64)
        dist = np.zeros(n.value, np.int32)
        if n.value:
            self._check(self.lib.bruno_copy_ranked(self.ctx, self._ptr(K), self._ptr(rep), self._ptr(dist), n.value,
                                                   ctypes.byref(n)), "copy_ranked")
        return K, rep, dist

    def chains(self):
        """compacted chains: reps (n, words), offsets (n+1), chars (uint8)"""
        nc, nch = ctypes.c_size_t(), ctypes.c_size_t()
        self._check(self.lib.bruno_copy_chains(self.ctx, None, None, None, 0, 0, ctypes.byref(nc), ctypes.byref(nch)),
                    "copy_chains")
        reps = np.zeros((nc.value, self.words), np.uint64)
        offs = np.zeros(nc.value + 1, np.uint64)
        chars = np.zeros(max(1, nch.value), np.uint8)
        if nc.value:
            self._check(self.lib.bruno_copy_chains(self.ctx, self._ptr(reps), self._ptr(offs), self._ptr(chars),
                                                   nc.value, chars.size, ctypes.byref(nc), ctypes.byref(nch)),
                        "copy_chains")
        return reps, offs, chars[:nch.value]

    def chain_edges(self):
        """print_chain_frequencies records, sorted by L as the reference prints them:
        L (n, words), R (n, words), freqs (n, 11) = L in ACGT, R out ACGT, mean, min, max"""
        n = ctypes.c_size_t()
        self._check(self.lib.bruno_copy_chain_edges(self.ctx, None, None, 0, ctypes.byref(n)), "copy_chain_edges")
        ends = np.zeros((n.value, 2, self.words), np.uint64)
        freqs = np.zeros((n.value, 11), np.uint16)
        if n.value:
            self._check(self.lib.bruno_copy_chain_edges(self.ctx, self._ptr(ends), self._ptr(freqs), n.value,
                                                        ctypes.byref(n)), "copy_chain_edges")
        L, R = ends[:, 0, :], ends[:, 1, :]
        order = np.lexsort(tuple(L[:, w] for w in range(self.words)))   # last key = high word first
        return L[order], R[order], freqs[order]

    def chain_summaries(self):
        """to_summarized_chains records sorted by the 5' terminus (the representative), as the
        reference orders them: kmers (n, 4, words) = prev at 5', 5', 3', next at 3';
        dist (n,); flags (n, 2) = 5' and 3' end point to a branch"""
        n = ctypes.c_size_t()
        self._check(self.lib.bruno_copy_chain_summaries(self.ctx, None, None, None, 0, ctypes.byref(n)),
                    "copy_chain_summaries")
        kmers = np.zeros((n.value, 4, self.words), np.uint64)
        dist = np.zeros(n.value, np.uint32)
        flags = np.zeros((n.value, 2), np.uint8)
        if n.value:
            self._check(self.lib.bruno_copy_chain_summaries(self.ctx, self._ptr(kmers), self._ptr(dist),
                                                            self._ptr(flags), n.value, ctypes.byref(n)),
                        "copy_chain_summaries")
        order = np.lexsort(tuple(kmers[:, 1, w] for w in range(self.words)))
        return kmers[order], dist[order], flags[order]

    def chain_strings(self) -> list[str]:
        reps, offs, chars = self.chains()
        b = chars.tobytes()
        return [b[offs[i]:offs[i + 1]].decode() for i in range(len(reps))]


class PinnedBuffer:
    """Page-locked host memory from the library (fast host<->device copies)."""

    def __init__(self, nbytes: int):
        self.lib = load_library()
        p = ctypes.c_void_p()
        st = self.lib.bruno_host_alloc(nbytes, ctypes.byref(p))
        if st != 0:
            raise BrunoError(st, "host_alloc")
        self.ptr, self.nbytes = p.value, nbytes
        self.array = np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(p.value))

    def free(self) -> None:
        if self.ptr:
            self.lib.bruno_host_free(ctypes.c_void_p(self.ptr))
            self.ptr = None


class Pool:
    """Many graph builds at once on one GPU (bruno_pool_*): `workers` host threads, each with its
    own context and stream, run the whole plain path for submitted FASTQ buffers; every result
    equals the plain path's for that input alone.  Submit a batch and wait for each ticket, or
    submit requests as they arrive and wait for them when needed."""

    def __init__(self, config: Optional[GraphConfig] = None, workers: int = 8, mem_budget: int = 0,
                 batched: bool = False, max_samples: int = 256, **kw):
        """batched: continuous batching over the fused form (one scheduler, passes of up to
        max_samples requests that fit mem_budget) instead of `workers` side-by-side builds"""
        self.lib = load_library()
        self.config = config or GraphConfig(**kw)
        c = self.config.to_c()
        self.pool = ctypes.c_void_p()
        if batched:
            st = self.lib.bruno_pool_create_batched(ctypes.byref(c), max_samples, mem_budget, ctypes.byref(self.pool))
        else:
            st = self.lib.bruno_pool_create(ctypes.byref(c), workers, mem_budget, ctypes.byref(self.pool))
        if st != 0:
            raise BrunoError(st, "pool_create")
        self._bufs = {}

    def submit(self, data) -> int:
        """queues one FASTQ (bytes or a uint8 host array, pinned for fast copies); the buffer is
        kept alive here until its result is collected"""
        arr = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8) if isinstance(data, (bytes, bytearray))
                                   else data, dtype=np.uint8)
        t = ctypes.c_uint64()
        st = self.lib.bruno_pool_submit(self.pool, arr.ctypes.data_as(ctypes.c_void_p), arr.nbytes, ctypes.byref(t))
        if st != 0:
            raise BrunoError(st, "pool_submit")
        self._bufs[t.value] = arr
        return t.value

    def wait(self, ticket: int) -> dict:
        """the build's status, sizes, compacted chains (reps, offsets, chars) and timings"""
        r = _PoolResult()
        st = self.lib.bruno_pool_wait(self.pool, ticket, ctypes.byref(r))
        self._bufs.pop(ticket, None)
        if st != 0:
            raise BrunoError(st, "pool_wait")
        try:
            out = {"status": r.status, "worker": r.worker, "queue_ms": r.queue_ms, "run_ms": r.run_ms}
            if r.status == 0:
                nc, nch, w = int(r.n_chains), int(r.n_chars), int(r.words)
                out["sizes"] = {n: getattr(r.sizes, n) for n, _ in _Sizes._fields_ if n != "filter_flag_hist"}
                out["chains"] = (np.ctypeslib.as_array(r.reps, (max(1, nc * w),))[:nc * w].reshape(nc, w).copy(),
                                 np.ctypeslib.as_array(r.offsets, (nc + 1,)).copy(),
                                 np.frombuffer(ctypes.string_at(r.chars, nch), np.uint8).copy())
            return out
        finally:
            self.lib.bruno_pool_result_free(ctypes.byref(r))

    def close(self) -> None:
        if getattr(self, "pool", None):
            self.lib.bruno_pool_destroy(self.pool)
            self.pool = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
