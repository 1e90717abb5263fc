"""The pool (bruno_pool_*): many builds at once on one GPU.  Every result must equal the plain
path's result for the same input built alone -- sizes and compacted chains bit for bit --
whether the requests run as a batch, arrive while others are running, or are held back by a
small memory budget."""
import threading
import time

import numpy as np
import pytest

import bruno_gb300 as bg
from bruno_gb300 import synth
from helpers import chain_set

pytestmark = pytest.mark.gpu

SIZE_KEYS = ("n_reads", "n_reads_used", "n_instances", "n_k2", "n_nodes", "n_branch", "n_chain_nodes",
             "iterations", "n_cycle_nodes", "n_isolated", "n_ranked", "n_chains", "n_chain_chars")


def _samples(n, seed, max_genome=300_000):
    return [synth.make_fastq(w) for w in synth.sample_set(n, seed, max_genome=max_genome)]


def _alone(fq, k=31):
    g = bg.Graph(k=k, thresh=bg.thresholds([2]), min_update=True)
    try:
        g.build_and_compact(fq)
        return g.sizes(), g.chains()
    finally:
        g.close()


def _same(res, alone):
    sizes, chains = alone
    assert res["status"] == 0
    for n in SIZE_KEYS:
        assert res["sizes"][n] == sizes[n], n
    assert chain_set(*res["chains"]) == chain_set(*chains)


def test_batch_equals_plain_path():
    fqs = _samples(24, 11)
    pool = bg.Pool(workers=6, thresh=bg.thresholds([2]), min_update=True)
    try:
        tickets = [pool.submit(fq) for fq in fqs]
        results = [pool.wait(t) for t in tickets]
    finally:
        pool.close()
    assert len({r["worker"] for r in results}) > 1
    for fq, r in zip(fqs, results):
        _same(r, _alone(fq))


def test_requests_arriving_during_others_equal_alone():
    """requests submitted from several threads while earlier ones run"""
    fqs = _samples(16, 12)
    alone = [_alone(fq) for fq in fqs]
    pool = bg.Pool(workers=4, thresh=bg.thresholds([2]), min_update=True)
    got = {}

    def client(idx):
        for i in idx:
            time.sleep(0.002 * (i % 3))
            t = pool.submit(fqs[i])
            got[i] = pool.wait(t)

    try:
        threads = [threading.Thread(target=client, args=(list(range(c, 16, 4)),)) for c in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    finally:
        pool.close()
    for i in range(16):
        _same(got[i], alone[i])


def test_small_memory_budget_still_exact():
    """a budget below one request's estimate: requests run one at a time, results unchanged"""
    fqs = _samples(6, 13)
    pool = bg.Pool(workers=3, mem_budget=1 << 20, thresh=bg.thresholds([2]), min_update=True)
    try:
        results = [pool.wait(t) for t in [pool.submit(fq) for fq in fqs]]
    finally:
        pool.close()
    for fq, r in zip(fqs, results):
        _same(r, _alone(fq))


def test_bad_request_reports_its_status():
    pool = bg.Pool(workers=2, thresh=bg.thresholds([2]))
    try:
        good = _samples(1, 14)[0]
        t_bad = pool.submit(b"@r\nACGT\n-\nIIII\n")
        t_good = pool.submit(good)
        assert pool.wait(t_bad)["status"] == 2          # malformed FASTQ
        _same(pool.wait(t_good), _alone(good))
    finally:
        pool.close()


# ------------------------------------------------------- continuous batching (the served form)
def test_batched_pool_equals_plain_path():
    """requests queued together are built in fused passes; each result is its plain build's"""
    fqs = _samples(24, 21)
    pool = bg.Pool(batched=True, max_samples=16, thresh=bg.thresholds([2]), min_update=True)
    try:
        results = [pool.wait(t) for t in [pool.submit(fq) for fq in fqs]]
    finally:
        pool.close()
    # requests of one pass share its run time: the 24 requests went in at most a few passes
    assert len({round(r["run_ms"], 6) for r in results}) < len(fqs)
    for fq, r in zip(fqs, results):
        _same(r, _alone(fq))


def test_batched_pool_requests_join_later_passes():
    """requests from several threads arrive while passes run and join the next pass"""
    fqs = _samples(16, 22)
    alone = [_alone(fq) for fq in fqs]
    pool = bg.Pool(batched=True, max_samples=64, thresh=bg.thresholds([2]), min_update=True)
    got = {}

    def client(idx):
        for i in idx:
            time.sleep(0.003 * (i % 3))
            got[i] = pool.wait(pool.submit(fqs[i]))

    try:
        threads = [threading.Thread(target=client, args=(list(range(c, 16, 4)),)) for c in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    finally:
        pool.close()
    for i in range(16):
        _same(got[i], alone[i])


def test_batched_pool_bad_request_falls_back_per_request():
    """a malformed request fails its pass; each request of that pass is then built alone"""
    pool = bg.Pool(batched=True, max_samples=8, thresh=bg.thresholds([2]))
    try:
        good = _samples(2, 23)
        tickets = [pool.submit(good[0]), pool.submit(b"@r\nACGT\n-\nIIII\n"), pool.submit(good[1])]
        res = [pool.wait(t) for t in tickets]
    finally:
        pool.close()
    assert res[1]["status"] == 2
    _same(res[0], _alone(good[0]))
    _same(res[2], _alone(good[1]))


def test_batched_pool_small_budget_one_request_a_pass():
    fqs = _samples(5, 24)
    pool = bg.Pool(batched=True, max_samples=8, mem_budget=1 << 20, thresh=bg.thresholds([2]), min_update=True)
    try:
        results = [pool.wait(t) for t in [pool.submit(fq) for fq in fqs]]
    finally:
        pool.close()
    for fq, r in zip(fqs, results):
        _same(r, _alone(fq))
