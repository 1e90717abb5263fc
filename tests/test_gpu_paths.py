"""GPU parity of the optional paths: the ranking's one-pass final states (cfg.rank_fill = 1),
the zero-copy result view, and host pieces over several copy streams."""
import pytest

import bruno_gb300 as bg
from bruno_gb300 import synth
from oracle import oracle
from conftest import fixture_bytes
from test_gpu_clean import _has_cuda
from test_gpu_parity import compare, gpu_run

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not _has_cuda(), reason="needs a CUDA GPU")]


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


class _DevArray:
    """a read-only device array for torch.as_tensor (the CUDA array interface)"""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 2}


def test_device_results_zero_copy():
    """bruno_device_results: the device arrays read in place equal what the copy calls return"""
    torch = pytest.importorskip("torch")
    data = fixture_bytes("debruijn.palindrome_chr14.fastq")
    g = bg.Graph(k=31, thresh=bg.thresholds([2]))
    try:
        g.build_and_compact(data)
        v = g.device_results()
        K, rep, dist = g.ranked()
        reps, offs, chars = g.chains()
        w = v["words"]
        assert v["n_ranked"] == len(dist) and v["n_chains"] == len(reps) and v["n_chain_chars"] == len(chars)

        def read(ptr, n, typestr):
            return torch.as_tensor(_DevArray(ptr, n, typestr), device="cuda").cpu().numpy()
        assert (read(v["ranked_K"], v["n_ranked"] * w, "<u8").reshape(-1, w) == K).all()
        assert (read(v["ranked_rep"], v["n_ranked"] * w, "<u8").reshape(-1, w) == rep).all()
        assert (read(v["ranked_dist"], v["n_ranked"], "<i4") == dist).all()
        assert (read(v["chain_reps"], v["n_chains"] * w, "<u8").reshape(-1, w) == reps).all()
        assert (read(v["chain_offsets"], v["n_chains"] + 1, "<u8") == offs).all()
        assert read(v["chain_chars"], v["n_chain_chars"], "|u1").tobytes() == bytes(chars)
    finally:
        g.close()


@pytest.mark.parametrize("streams", [2, 3, 4])
def test_host_pieces_over_copy_streams(streams):
    """host FASTQ pieces spread round robin over several copy streams (cfg.h2d_streams), each
    piece waited on by its own event, with extraction under the later copies: equal to the oracle"""
    from test_gpu_parity import at_quality
    w = synth.WORKLOADS["plain-small"]
    fq = at_quality(synth.make_fastq(w))
    thr = bg.thresholds(w.lower)
    ref = oracle.run(fq, k=31, thresh=thr, min_update=True, threads=16, keep_k2=True, keep_filtered=True)
    compare(gpu_run(fq, 31, True, thr, True, h2d_chunk=1 << 16, h2d_streams=streams), ref)
    data = at_quality(fixture_bytes("natural.withN.fastq"))
    thr2 = bg.thresholds([2])
    ref2 = oracle.run(data, k=45, thresh=thr2, min_update=True, keep_k2=True, keep_filtered=True)
    compare(gpu_run(data, 45, True, thr2, True, h2d_chunk=1024, h2d_streams=streams), ref2)
