"""ctypes wrapper of the CPU oracle (oracle/bruno_oracle.h).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the parity checker and by bench.py's CPU
baseline leg.  The product library never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
CLI = os.path.join(HERE, "_build", "oracle_cli")
PHASES = ("parse", "count_k2mers", "filter_insert", "chainmap", "list_rank", "compress")


class _Cfg(ctypes.Structure):
    _fields_ = [("k", ctypes.c_int32), ("thresholding", ctypes.c_int32), ("thresh", ctypes.c_uint64 * 6),
                ("min_update", ctypes.c_int32), ("threads", ctypes.c_int32), ("keep_k2", ctypes.c_int32),
                ("keep_filtered", ctypes.c_int32), ("edge_filter", ctypes.c_int32), ("clean", ctypes.c_int32)]


_U64P = ctypes.POINTER(ctypes.c_uint64)


class _Res(ctypes.Structure):
    pass


_Res._fields_ = [
        ("status", ctypes.c_int32), ("words", ctypes.c_int32), ("n_reads", ctypes.c_uint64),
        ("n_reads_used", ctypes.c_uint64), ("n_instances", ctypes.c_uint64),
        ("n_k2", ctypes.c_uint64), ("k2_keys", _U64P), ("k2_edges", ctypes.POINTER(ctypes.c_uint8)),
        ("k2_counts", ctypes.POINTER(ctypes.c_uint32)),
        ("n_filtered", ctypes.c_uint64), ("filt_keys", _U64P), ("filt_edges", ctypes.POINTER(ctypes.c_uint8)),
        ("filt_counts", ctypes.POINTER(ctypes.c_uint32)), ("filter_flag_hist", ctypes.c_uint64 * 16),
        ("n_nodes", ctypes.c_uint64), ("node_keys", _U64P), ("node_counts", ctypes.POINTER(ctypes.c_uint16)),
        ("node_flags", ctypes.POINTER(ctypes.c_uint8)), ("n_branch", ctypes.c_uint64),
        ("n_chain_nodes", ctypes.c_uint64), ("iterations", ctypes.c_uint64), ("collisions", ctypes.c_uint64),
        ("n_cycle_nodes", ctypes.c_uint64), ("n_isolated", ctypes.c_uint64),
        ("n_ranked", ctypes.c_uint64), ("ranked_K", _U64P), ("ranked_rep", _U64P),
        ("ranked_dist", ctypes.POINTER(ctypes.c_int32)),
        ("n_chains", ctypes.c_uint64), ("chain_rep", _U64P), ("chain_offsets", _U64P),
        ("chain_chars", ctypes.POINTER(ctypes.c_char)),
        ("n_chain_edges", ctypes.c_uint64), ("edge_L", _U64P), ("edge_R", _U64P),
        ("edge_freqs", ctypes.POINTER(ctypes.c_uint16)),
        ("n_summaries", ctypes.c_uint64), ("sum_kmers", _U64P), ("sum_dist", ctypes.POINTER(ctypes.c_uint32)),
        ("sum_flags", ctypes.POINTER(ctypes.c_uint8)), ("summaries_ok", ctypes.c_int32),
        ("seconds", ctypes.c_double * 6),
        ("clean_rounds", ctypes.c_uint64), ("clean_deadends", ctypes.c_uint64), ("clean_bubbles", ctypes.c_uint64),
        ("clean_edges", ctypes.c_uint64), ("clean_status", ctypes.c_int32), ("clean", ctypes.POINTER(_Res)),
        ("n_chain_map", ctypes.c_uint64), ("cm_keys", _U64P), ("cm_in", _U64P), ("cm_out", _U64P),
        ("cm_in_dist", ctypes.POINTER(ctypes.c_uint32)), ("cm_out_dist", ctypes.POINTER(ctypes.c_uint32)),
        ("n_isolated_recs", ctypes.c_uint64), ("iso_keys", _U64P), ("iso_in", _U64P), ("iso_out", _U64P),
        ("iso_in_dist", ctypes.POINTER(ctypes.c_uint32)), ("iso_out_dist", ctypes.POINTER(ctypes.c_uint32)),
        ("n_cycle_kmers", ctypes.c_uint64), ("cycle_keys", _U64P),
        ("check_query", ctypes.c_uint64), ("check_absent", ctypes.c_uint64), ("check_unreferenced", ctypes.c_uint64),
        ("check_unanswered", ctypes.c_uint64), ("edge_hist", ctypes.c_uint64 * 25),
    ]


def build(force: bool = False) -> None:
    """Same recipe as oracle/Makefile, with g++ called directly (no make needed)."""
    os.makedirs(os.path.join(HERE, "_build"), exist_ok=True)
    src = [os.path.join(HERE, "bruno_oracle.cpp"), os.path.join(HERE, "bruno_oracle.h")]
    flags = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter"]
    jobs = []
    if force or not _fresh(LIB, src):
        jobs.append(["g++", *flags, "-shared", "-o", LIB, src[0], "-lpthread"])
    if force or not _fresh(CLI, src + [os.path.join(HERE, "oracle_main.cpp")]):
        jobs.append(["g++", *flags, "-o", CLI, os.path.join(HERE, "oracle_main.cpp"), src[0], "-lpthread"])
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True) for j in jobs]
    for p, j in zip(procs, jobs):
        out, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"oracle build failed: {' '.join(j)}\n{err}")


def _fresh(target, deps) -> bool:
    return os.path.exists(target) and all(os.path.getmtime(d) <= os.path.getmtime(target) for d in deps)


_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = ctypes.CDLL(LIB)
        lib.oracle_run.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(_Cfg),
                                   ctypes.POINTER(ctypes.POINTER(_Res))]
        lib.oracle_run.restype = ctypes.c_int
        lib.oracle_free.argtypes = [ctypes.POINTER(_Res)]
        lib.oracle_write_outputs.argtypes = [ctypes.POINTER(_Res), ctypes.c_int32, ctypes.c_char_p, ctypes.c_int32]
        lib.oracle_write_outputs.restype = ctypes.c_int
        _lib = lib
    return _lib


def _arr(ptr, n, dtype, shape=None):
    if n == 0:
        return np.zeros(shape or (0,), dtype)
    a = np.ctypeslib.as_array(ptr, shape=(n,)).copy().astype(dtype, copy=False)
    return a.reshape(shape) if shape else a


def _graph(r, keep_k2: bool = False, keep_filtered: bool = False) -> dict:
    """the arrays and counters of one result (the first compaction, or the cleaned graph)"""
    out = {}
    w = r.words
    for n in ("n_reads", "n_reads_used", "n_instances", "n_k2", "n_filtered", "n_nodes", "n_branch",
              "n_chain_nodes", "iterations", "collisions", "n_cycle_nodes", "n_isolated", "n_ranked", "n_chains"):
        out[n] = int(getattr(r, n))
    out["filter_flag_hist"] = list(r.filter_flag_hist)
    out["seconds"] = dict(zip(PHASES, list(r.seconds)))
    out["k2"] = (_arr(r.k2_keys, r.n_k2 * w, np.uint64, (r.n_k2, w)), _arr(r.k2_edges, r.n_k2, np.uint8),
                 _arr(r.k2_counts, r.n_k2, np.uint32)) if keep_k2 else None
    out["filtered"] = (_arr(r.filt_keys, r.n_filtered * w, np.uint64, (r.n_filtered, w)),
                       _arr(r.filt_edges, r.n_filtered, np.uint8),
                       _arr(r.filt_counts, r.n_filtered, np.uint32)) if keep_filtered else None
    out["nodes"] = (_arr(r.node_keys, r.n_nodes * w, np.uint64, (r.n_nodes, w)),
                    _arr(r.node_counts, r.n_nodes * 9, np.uint16, (r.n_nodes, 9)),
                    _arr(r.node_flags, r.n_nodes, np.uint8))
    out["ranked"] = (_arr(r.ranked_K, r.n_ranked * w, np.uint64, (r.n_ranked, w)),
                     _arr(r.ranked_rep, r.n_ranked * w, np.uint64, (r.n_ranked, w)),
                     _arr(r.ranked_dist, r.n_ranked, np.int32))
    offs = _arr(r.chain_offsets, r.n_chains + 1, np.uint64) if r.n_chains else np.zeros(1, np.uint64)
    nchars = int(offs[-1])
    chars = ctypes.string_at(r.chain_chars, nchars) if nchars else b""
    out["chains"] = (_arr(r.chain_rep, r.n_chains * w, np.uint64, (r.n_chains, w)), offs, chars)
    ns = r.n_summaries
    out["summaries"] = (_arr(r.sum_kmers, ns * 4 * w, np.uint64, (ns, 4, w)), _arr(r.sum_dist, ns, np.uint32),
                        _arr(r.sum_flags, ns * 2, np.uint8, (ns, 2))) if r.summaries_ok else None
    ne = r.n_chain_edges
    out["chain_edges"] = (_arr(r.edge_L, ne * w, np.uint64, (ne, w)), _arr(r.edge_R, ne * w, np.uint64, (ne, w)),
                          _arr(r.edge_freqs, ne * 11, np.uint16, (ne, 11)))

    def records(n, keys, inK, outK, inD, outD):
        return (_arr(keys, n * w, np.uint64, (n, w)), _arr(inK, n * w, np.uint64, (n, w)),
                _arr(outK, n * w, np.uint64, (n, w)), _arr(inD, n, np.uint32), _arr(outD, n, np.uint32))
    # the chain map after ranking, the isolated records and the cycle k-mers, each sorted by k-mer
    out["chain_map"] = records(r.n_chain_map, r.cm_keys, r.cm_in, r.cm_out, r.cm_in_dist, r.cm_out_dist)
    out["isolated"] = records(r.n_isolated_recs, r.iso_keys, r.iso_in, r.iso_out, r.iso_in_dist, r.iso_out_dist)
    out["cycle_kmers"] = _arr(r.cycle_keys, r.n_cycle_kmers * w, np.uint64, (r.n_cycle_kmers, w))
    out["check_index"] = {"n_query": int(r.check_query), "n_absent": int(r.check_absent),
                          "n_unreferenced": int(r.check_unreferenced), "n_unanswered": int(r.check_unanswered),
                          "edge_hist": list(r.edge_hist)}
    return out


def run(fastq, k: int = 31, thresholding: bool = True, thresh=None, min_update: bool = True, threads: int = 1,
        keep_k2: bool = False, keep_filtered: bool = False, write_prefix: str | None = None,
        benchmark: bool = False, edge_filter: bool = False, clean: bool = False) -> dict:
    """Runs the oracle on FASTQ bytes (or a uint8 array); returns numpy results.  With clean,
    out["clean"] holds the cleaned graph (nodes, ranked, chains, chain_edges and the ranking
    counters of the last recompaction) and out["clean_stats"] the loop's tallies."""
    lib = _load()
    buf = np.ascontiguousarray(np.frombuffer(fastq, np.uint8) if isinstance(fastq, (bytes, bytearray)) else fastq,
                               dtype=np.uint8)
    c = _Cfg()
    c.k, c.thresholding, c.min_update, c.threads = k, int(thresholding), int(min_update), threads
    t = thresh if thresh is not None else [65536] * 6
    for i in range(6):
        c.thresh[i] = int(min(t[i], 2**64 - 1))
    c.keep_k2, c.keep_filtered, c.edge_filter = int(keep_k2), int(keep_filtered), int(edge_filter)
    c.clean = int(clean)
    rp = ctypes.POINTER(_Res)()
    rc = lib.oracle_run(buf.ctypes.data_as(ctypes.c_void_p), buf.nbytes, ctypes.byref(c), ctypes.byref(rp))
    try:
        r = rp.contents
        if rc != 0:
            return {"status": rc}
        out = {"status": rc, **_graph(r, keep_k2, keep_filtered)}
        if clean:
            out["clean_stats"] = {n: int(getattr(r, "clean_" + n))
                                  for n in ("rounds", "deadends", "bubbles", "edges", "status")}
            out["clean"] = _graph(r.clean.contents) if r.clean else None
        if write_prefix:
            lib.oracle_write_outputs(rp, k, write_prefix.encode(), int(benchmark))
        return out
    finally:
        lib.oracle_free(rp)
