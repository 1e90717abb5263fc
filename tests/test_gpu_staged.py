"""GPU parity of code paths that have not yet run on a GPU: the ranking's one-pass final states
(cfg.rank_fill = 1).  Staged like tests/test_gpu_clean.py: marker `gpu_staged`, selected only by
`-m gpu_staged`, skipped without a GPU; moved to `gpu` once it has passed on a GB300."""
import pytest

import bruno_gb300 as bg
from bruno_gb300 import synth
from oracle import oracle
from conftest import fixture_bytes
from test_gpu_clean import _has_cuda
from test_gpu_parity import compare, gpu_run

pytestmark = [pytest.mark.gpu_staged, pytest.mark.skipif(not _has_cuda(), reason="needs a CUDA GPU")]


@pytest.mark.parametrize("fname", ["debruijn.palindrome_chr14.fastq", "debruijn.shifted_cycle_chr14.fastq",
                                   "debruijn.bubble.fastq", "natural.fastq", "test.unitiqs.fastq"])
@pytest.mark.parametrize("lo", [(), (2,)])
def test_rank_fill_fixture_parity(fname, lo):
    data = fixture_bytes(fname)
    thr = bg.thresholds(lo)
    ref = oracle.run(data, k=31, thresholding=bool(lo), thresh=thr, min_update=True, keep_k2=True,
                     keep_filtered=True)
    compare(gpu_run(data, 31, bool(lo), thr, True, rank_fill=1), ref)


@pytest.mark.parametrize("k", [31, 45])
def test_rank_fill_workload_parity(k):
    """a repeat-rich genome: long chains, cycles, many rulers per chain"""
    w = synth.Workload(f"rf{k}", 1_000_000, 150, 200_000, 0.005, k, (3,), 0.02, (1000, 10000), (2, 8),
                       (0.01, 0.01), 5)
    fq = synth.make_fastq(w)
    thr = bg.thresholds(w.lower)
    ref = oracle.run(fq, k=k, thresh=thr, min_update=True, threads=16, keep_k2=True, keep_filtered=True)
    compare(gpu_run(fq, k, True, thr, True, rank_fill=1), ref)
