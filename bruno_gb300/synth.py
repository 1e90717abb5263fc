"""Seeded synthetic FASTQ workloads (the generator lives in csrc/synth.cpp).

Each workload reproduces the shapes, sizes and value distributions of one benchmark
configuration: a uniform ACGT genome, optionally with diverged repeat families, and
fixed-length reads sampled uniformly with random strand and uniform substitutions, written
as ``@r<i>\\n<seq>\\n+\\n<'I' x L>\\n`` records.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, replace

import numpy as np

_LIB = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libbruno_synth.so")


class _SynthCfg(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("genome_len", ctypes.c_uint64), ("repeat_frac", ctypes.c_double),
                ("rep_len_min", ctypes.c_uint32), ("rep_len_max", ctypes.c_uint32),
                ("rep_copies_min", ctypes.c_uint32), ("rep_copies_max", ctypes.c_uint32),
                ("rep_div_min", ctypes.c_double), ("rep_div_max", ctypes.c_double),
                ("read_len", ctypes.c_uint32), ("n_reads", ctypes.c_uint64), ("sub_rate", ctypes.c_double),
                ("threads", ctypes.c_int32)]


@dataclass(frozen=True)
class Workload:
    name: str
    genome_len: int
    read_len: int
    n_reads: int
    sub_rate: float
    k: int
    lower: tuple
    repeat_frac: float = 0.0
    rep_len: tuple = (0, 0)
    rep_copies: tuple = (0, 0)
    rep_div: tuple = (0.0, 0.0)
    seed: int = 1

    @property
    def coverage(self) -> float:
        return self.n_reads * self.read_len / self.genome_len

    def scaled(self, reads_fraction: float) -> "Workload":
        """The same genome with a fraction of the reads (a bounded sample of the workload)."""
        return replace(self, n_reads=max(1, int(self.n_reads * reads_fraction)))


WORKLOADS = {
    # 1 Mbp uniform genome, 100k x 100 bp reads, 1% substitutions, k=31, -L 2
    "plain-small": Workload("plain-small", 1_000_000, 100, 100_000, 0.01, 31, (2,)),
    # 50 Mbp + 2% repeats (1-10 kbp, 2-8 copies, 1% divergence), 30x 150 bp, 0.5% subs, k=31, -L 3
    "plain-scale": Workload("plain-scale", 50_000_000, 150, 10_000_000, 0.005, 31, (3,), 0.02, (1000, 10000),
                            (2, 8), (0.01, 0.01)),
    # the plain-scale mix at a fifth of the genome (profiling case: 10 Mbp, 2M x 150 bp, k=31, -L 3)
    "plain-medium": Workload("plain-medium", 10_000_000, 150, 2_000_000, 0.005, 31, (3,), 0.02, (1000, 10000),
                             (2, 8), (0.01, 0.01), 5),
    # the plain-scale mix at a twelfth of the genome, sized for full ncu captures (a few GB on the
    # device, inputs still larger than L2): 4 Mbp + 2% repeats, 800k x 150 bp, k=31, -L 3
    "plain-profile": Workload("plain-profile", 4_000_000, 150, 800_000, 0.005, 31, (3,), 0.02, (1000, 10000),
                              (2, 8), (0.01, 0.01), 6),
    # 200 Mbp + 5% repeats (1-20 kbp, 2-16 copies, 1-3% divergence), 30x 150 bp, k=63, -L 3
    "large-k": Workload("large-k", 200_000_000, 150, 40_000_000, 0.005, 63, (3,), 0.05, (1000, 20000), (2, 16),
                        (0.01, 0.03)),
    # the large-k mix at a fiftieth of the genome, for full ncu captures (4 Mbp, 800k x 150 bp, k=63)
    "large-k-profile": Workload("large-k-profile", 4_000_000, 150, 800_000, 0.005, 63, (3,), 0.05, (1000, 20000),
                                (2, 16), (0.01, 0.03), 10),
}


def sample_set(n: int, seed: int, max_genome: int = 2_000_000, min_genome: int = 5_000, k: int = 31,
               lower: tuple = (2,)) -> list:
    """Independent samples of uneven size for the batched and served forms: genome length
    log-uniform in [min_genome, max_genome], coverage uniform in [20, 60]x, one read length per
    sample uniform in 100..250 bp, substitutions uniform in [0.5%, 2%]; every sample has its own
    seed.  (Batched: 256 samples up to 2 Mbp; served: the same shape up to 20 Mbp.)"""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        g = int(round(np.exp(rng.uniform(np.log(min_genome), np.log(max_genome)))))
        cov = float(rng.uniform(20.0, 60.0))
        L = int(rng.integers(100, 251))
        sub = float(rng.uniform(0.005, 0.02))
        out.append(Workload(f"sample{i}", g, L, max(1, int(round(cov * g / L))), sub, k, lower,
                            seed=int(rng.integers(1, 2**31))))
    return out


def _lib() -> ctypes.CDLL:
    if not os.path.exists(_LIB):
        raise RuntimeError(f"synthetic generator not built: {_LIB}")
    lib = ctypes.CDLL(_LIB)
    lib.synth_fastq_size.argtypes = [ctypes.POINTER(_SynthCfg)]
    lib.synth_fastq_size.restype = ctypes.c_uint64
    lib.synth_fastq.argtypes = [ctypes.POINTER(_SynthCfg), ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    lib.synth_fastq.restype = ctypes.c_int
    return lib


def _cfg(w: Workload, threads: int = 0) -> _SynthCfg:
    return _SynthCfg(w.seed, w.genome_len, w.repeat_frac, w.rep_len[0], w.rep_len[1], w.rep_copies[0],
                     w.rep_copies[1], w.rep_div[0], w.rep_div[1], w.read_len, w.n_reads, w.sub_rate, threads)


def fastq_size(w: Workload) -> int:
    c = _cfg(w)
    return int(_lib().synth_fastq_size(ctypes.byref(c)))


def make_fastq(w: Workload, out: np.ndarray | None = None, threads: int = 0, genome: bool = False):
    """Generates the workload's FASTQ into `out` (uint8, at least fastq_size(w) bytes) or a
    new array; returns the array view (and the genome when genome=True)."""
    lib = _lib()
    c = _cfg(w, threads)
    n = int(lib.synth_fastq_size(ctypes.byref(c)))
    buf = np.empty(n, np.uint8) if out is None else out
    if buf.nbytes < n:
        raise ValueError("output buffer too small")
    g = np.empty(w.genome_len, np.uint8) if genome else None
    rc = lib.synth_fastq(ctypes.byref(c), buf.ctypes.data_as(ctypes.c_void_p), n,
                         g.ctypes.data_as(ctypes.c_void_p) if genome else None)
    if rc != 0:
        raise RuntimeError(f"synth_fastq failed: {rc}")
    return (buf[:n], g) if genome else buf[:n]
