#!/usr/bin/env python3
"""Benchmark: k-mers/s of the plain build+compact path on the plain-scale workload.

One step = one pass of the whole path -- FASTQ parse, (k+2)-mer counting, frequency filter
and node insert, chain extraction, list ranking (list_rank_min_update) and compacted-chain
emission -- over the 50 Mbp / 30x / 150 bp / k=31 / -L 3 synthetic workload.

  value   k-mers/s with the FASTQ already resident in HBM (CUDA events on the library's
          stream, which is torch's current stream).
  e2e     the same through the C ABI with pinned host buffers: the FASTQ host->device copy
          and the device->host read of the compacted chains are inside the timed region.
  roofline  the dominant kernel (by time) against the measured HBM copy bandwidth, with the
          other large kernels beside it.
  cpu_baseline  the CPU oracle (a restatement of the reference's CPU path) on a bounded
          sample of the same workload, with every host thread.

--impl reference runs the CPU path instead and prints the same line with "impl":
"reference".  Multi-GPU runs are independent replicas (the path is one graph per GPU).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC, UNIT = "k-mers/s build+compact", "k-mers/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="plain-scale")
    ap.add_argument("--cpu-sample", type=float, default=0.2, help="fraction of reads in the CPU baseline sample")
    ap.add_argument("--ref-sample", type=float, default=0.05,
                    help="fraction of reads in each step of the reference arm (a bounded sample of the workload, "
                         "so that every step of --steps/--warmup takes a few seconds)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--samples", type=int, default=None,
                    help="batched / served: number of distinct samples (256 / 48)")
    ap.add_argument("--tune", type=int, default=1, choices=[0, 1],
                    help="batched: 1 = autotune the table shape on a probe quarter, 0 = the library's defaults")
    ap.add_argument("--rates", type=float, nargs="+", default=[10, 50, 100, 200, 500], help="served: requests/s")
    ap.add_argument("--requests", type=int, default=200, help="served: most requests per rate")
    ap.add_argument("--seconds", type=float, default=4.0, help="served: target seconds per rate")
    ap.add_argument("--h2d-streams", type=int, default=1, help="copy streams for the host FASTQ pieces (1..4)")
    ap.add_argument("--h2d-chunk", type=int, default=0, help="host FASTQ piece size in bytes (0 = the library's)")
    ap.add_argument("--e2e-workers", type=int, default=0,
                    help="e2e through a pool of this many contexts (bruno_pool_*), so that one step's host "
                         "copy overlaps the previous step's device work; 0 = one context, steps in turn")
    ap.add_argument("--part-slots", type=int, default=0,
                    help="largest shared-memory partition region in slots (0 = the library's 3072)")
    ap.add_argument("--count-threads", type=int, default=0, choices=[0, 256, 512, 1024],
                    help="threads of the shared-memory counting block (0 = the library's 512)")
    ap.add_argument("--max-load", type=float, default=0.0,
                    help="target k-mer table load (0 = the library's 0.5; the large-k workload uses 0.7 so "
                         "its 64-byte slots fit the device)")
    ap.add_argument("--rank-fill", type=int, default=0, choices=[0, 1],
                    help="ranking's final states: 0 = second walk, 1 = one pass over the nodes")
    ap.add_argument("--api", default="build", choices=["build", "steps"],
                    help="build: bruno_build_and_compact (one call); steps: the reference's call sequence "
                         "(load, compute_biedge_freqencies, local_insert_by_freqencies, extract_chains, "
                         "list_rank_min_update, to_compressed_chains)")
    return ap.parse_args()


def max_over_ranks(x: float, world: int) -> float:
    """The largest value over all ranks (the slowest rank's time); a no-op for one rank.
    Uses a device tensor under NCCL and a host tensor under gloo."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, copy burst)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s"


def workload_config(w, mu=True):
    return {"workload": f"{w.name}: {w.genome_len / 1e6:g} Mbp genome"
                        + (f" + {w.repeat_frac * 100:g}% repeats ({w.rep_len[0]}-{w.rep_len[1]} bp, "
                           f"{w.rep_copies[0]}-{w.rep_copies[1]} copies, {w.rep_div[0] * 100:g}-{w.rep_div[1] * 100:g}% "
                           f"divergence)" if w.repeat_frac else "")
                        + f", {w.n_reads} x {w.read_len} bp reads ({w.coverage:.0f}x), {w.sub_rate * 100:g}% "
                          f"substitutions, k={w.k}, -T -L {w.lower[0]}, "
                        + ("list_rank_min_update" if mu else "list_rank"),
            "genome_bp": w.genome_len, "reads": w.n_reads, "read_len": w.read_len, "k": w.k,
            "threshold_k1_lower": w.lower[0], "seed": w.seed,
            "l2": "inputs larger than L2 (FASTQ and k-mer table are GBs; no flush needed)"}


class ClockSampler:
    """nvidia-smi samples during the timed region"""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(w, frac, threads):
    """the oracle on the first `frac` of the workload's reads, all host threads.  The time is
    the sum of the oracle's six path phases (parse through compression, the steps the GPU step
    runs); the exports the oracle adds for the parity tests (sorted node, chain-map and k2
    copies, chain edges and summaries, the check_index tally) are left out of it."""
    from bruno_gb300 import synth, thresholds
    from oracle import oracle
    ws = w.scaled(frac)
    fq = synth.make_fastq(ws)
    t0 = time.perf_counter()
    r = oracle.run(fq, k=w.k, thresh=thresholds(w.lower), min_update=True, threads=threads)
    wall = time.perf_counter() - t0
    dt = sum(r["seconds"].values())
    return {"value": r["n_instances"] / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {ws.n_reads} of {w.n_reads} reads ({frac * 100:g}%), {r['n_instances']} k-mers, "
                      f"{dt:.2f} s in the six path phases ({wall:.2f} s with the oracle's test-only exports)",
            "seconds": dt, "instances": r["n_instances"],
            "phases_s": {p: round(t, 4) for p, t in r["seconds"].items()}}


def run_reference(args, w):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sample = max(args.ref_sample, 1e-4)
    for _ in range(args.warmup):
        cpu_baseline(w, sample, threads)
    vals, secs = [], []
    for _ in range(args.steps):
        b = cpu_baseline(w, sample, threads)
        vals.append(b["value"])
        secs.append(b["seconds"])
    value = statistics.mean(vals)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded generator, " + w.name + ")",
            "config": workload_config(w), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": b["sample"],
                             "phases_s": b["phases_s"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _pinned_copies(bg, fqs):
    bufs = []
    for fq in fqs:
        b = bg.PinnedBuffer(max(1, fq.nbytes))
        b.array[:fq.nbytes] = fq
        bufs.append(b)
    return bufs


def _plain_loop(bg, cfg, bufs, sizes):
    """the plain path looped over the samples: one context, one build after another"""
    g = bg.Graph(cfg)
    outs = []
    t0 = time.perf_counter()
    for b, n in zip(bufs, sizes):
        g.build_and_compact(b.array[:n])
        outs.append((g.sizes(), g.chains()))
    dt = time.perf_counter() - t0
    g.close()
    return dt, outs


def _same_as_plain(res, plain):
    sizes, chains = plain
    keys = ("n_instances", "n_k2", "n_nodes", "n_chain_nodes", "n_ranked", "n_chains", "n_chain_chars")
    if res["status"] != 0 or any(res["sizes"][k] != sizes[k] for k in keys):
        return False
    a, b = res["chains"], chains
    return (np.array_equal(np.sort(a[0], axis=0), np.sort(b[0], axis=0)) and a[1][-1] == b[1][-1]
            and sorted(bytes(a[2][a[1][i]:a[1][i + 1]]) for i in range(len(a[0])))
            == sorted(bytes(b[2][b[1][i]:b[1][i + 1]]) for i in range(len(b[0]))))


def run_batched(args):
    """Config 3: 256 independent samples of uneven size built in one fused pass of every kernel
    (bruno_build_samples: per-sample hash-table partitions; load factor, partition size and
    counting block shape chosen by the autotuner on a probe quarter of the batch), against the
    plain path looped over the same samples on the same GPU.  Both time host buffers in and
    every sample's chains out."""
    import bruno_gb300 as bg
    from bruno_gb300 import autotune, synth
    samples = synth.sample_set(args.samples or 256, seed=3, max_genome=2_000_000)
    fqs = [synth.make_fastq(w) for w in samples]
    sizes = [fq.nbytes for fq in fqs]
    bufs = _pinned_copies(bg, fqs)
    views = [b.array[:n] for b, n in zip(bufs, sizes)]
    cfg = bg.GraphConfig(k=31, thresh=bg.thresholds([2]), min_update=True, h2d_chunk=args.h2d_chunk)
    _plain_loop(bg, cfg, bufs[:8], sizes[:8])                 # warm-up
    plain_s, plain = _plain_loop(bg, cfg, bufs, sizes)
    probe = views[::4]
    best, tune = autotune.tune_batch(cfg, probe) if args.tune else (cfg, {})
    g = bg.Graph(best)
    g.build_samples(probe)                                    # warm-up of the chosen shape
    passes = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        g.build_samples(views)
        t1 = time.perf_counter()
        chains = g.batch_chains()   # one copy of every sample's chains, sliced per sample
        res = [{"status": 0, "sizes": g.sample_sizes(i), "chains": chains[i]} for i in range(len(views))]
        passes.append((time.perf_counter() - t0, t1 - t0))
    phases = g.phase_ms()
    tot = g.sizes()
    g.close()
    dt = statistics.median(p[0] for p in passes)
    exact = all(_same_as_plain(r, p) for r, p in zip(res, plain))
    line = {"metric": "graphs/s batched", "value": len(fqs) / dt, "unit": "graphs/s", "n_gpus": 1,
            "steps": len(passes), "higher_is_better": True, "data": "synthetic (seeded generator, sample_set seed 3)",
            "config": {"workload": f"batched: {len(fqs)} samples, genome log-uniform 5 kbp-2 Mbp, 20-60x, "
                                   "100-250 bp reads, 0.5-2% substitutions, k=31, -L 2",
                       "fastq_bytes": int(sum(sizes))},
            "form": "one fused pass (bruno_build_samples), host buffers in, chains out",
            "run": {"h2d_chunk": args.h2d_chunk or 256 << 20, "tune": args.tune},
            "plain_loop_graphs_per_s": len(fqs) / plain_s, "speedup_vs_plain_loop": plain_s / dt,
            "pass_ms": {"with_copy_out": 1e3 * dt, "build_only": 1e3 * statistics.median(p[1] for p in passes)},
            "phase_ms": phases,
            "sizes": {k: tot[k] for k in ("n_reads", "n_instances", "n_k2", "n_nodes", "n_chain_nodes", "n_chains",
                                          "n_ranked", "table_slots", "table_partitions")},
            "autotuned": {"max_load": best.max_load, "part_slots": best.part_slots, "count_threads": best.count_threads},
            "autotune_graphs_per_s": tune,
            "latency_ms": {"p50": 1e3 * dt, "p99": 1e3 * dt,
                           "note": "every sample of a batch completes with its pass"},
            "bit_exact_vs_plain": exact}
    print(json.dumps(line), flush=True)
    for b in bufs:
        b.free()


def run_served(args):
    """Config 4: Poisson arrivals of build-and-compact requests (samples up to 20 Mbp) admitted
    to the pool as workers and memory free up; p50/p99 latency (arrival to result on the host)
    and throughput at each arrival rate, against the plain path looped on the same GPU."""
    import threading
    import bruno_gb300 as bg
    from bruno_gb300 import synth
    samples = synth.sample_set(args.samples or 48, seed=4, max_genome=20_000_000)
    fqs = [synth.make_fastq(w) for w in samples]
    sizes = [fq.nbytes for fq in fqs]
    bufs = _pinned_copies(bg, fqs)
    cfg = bg.GraphConfig(k=31, thresh=bg.thresholds([2]), min_update=True)
    _plain_loop(bg, cfg, bufs[:4], sizes[:4])
    plain_s, plain = _plain_loop(bg, cfg, bufs, sizes)
    # continuous batching over the fused form: every pass takes what is queued
    pool = bg.Pool(cfg, batched=True, max_samples=256)
    for t in [pool.submit(bufs[i].array[:sizes[i]]) for i in range(min(8, len(bufs)))]:
        pool.wait(t)
    rng = np.random.default_rng(5)
    rates = {}
    exact = True
    for rate in args.rates:
        n = max(20, min(args.requests, int(rate * args.seconds)))
        order = rng.integers(0, len(fqs), n)
        gaps = rng.exponential(1.0 / rate, n)
        lat, got, lock = [], [], threading.Lock()

        def collect(t, i, t_arr):
            r = pool.wait(t)
            done = time.perf_counter()
            with lock:
                lat.append(1e3 * (done - t_arr))
                got.append((i, r))
        waiters = []
        t0 = time.perf_counter()
        t_next = t0
        for i, gap in zip(order, gaps):
            t_next += gap
            delay = t_next - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            t_arr = time.perf_counter()
            tk = pool.submit(bufs[i].array[:sizes[i]])
            th = threading.Thread(target=collect, args=(tk, int(i), t_arr))
            th.start()
            waiters.append(th)
        for th in waiters:
            th.join()
        wall = time.perf_counter() - t0
        lat.sort()
        bad = [int(i) for i, r in got if not _same_as_plain(r, plain[i])]   # checked after the timed run
        rates[str(rate)] = {"requests": n, "graphs_per_s": n / wall, "p50_ms": lat[len(lat) // 2],
                            "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
                            "statuses": sorted({r["status"] for _, r in got}), "mismatched": sorted(set(bad))}
        exact = exact and not bad
    pool.close()
    best = max(v["graphs_per_s"] for v in rates.values())
    line = {"metric": "graphs/s served", "value": best, "unit": "graphs/s", "n_gpus": 1, "higher_is_better": True,
            "data": "synthetic (seeded generator, sample_set seed 4)",
            "config": {"workload": f"served: Poisson arrivals, {len(fqs)} distinct requests (genome log-uniform "
                                   "5 kbp-20 Mbp, 20-60x, 100-250 bp, 0.5-2% substitutions, k=31, -L 2), "
                                   "admission by free HBM"},
            "form": "continuous batching: each fused pass (bruno_build_samples) takes every queued request that "
                    "fits the memory budget; requests arriving during a pass join the next",
            "plain_loop_graphs_per_s": len(fqs) / plain_s, "speedup_vs_plain_loop": best * plain_s / len(fqs),
            "rates": rates, "bit_exact_vs_plain": exact}
    print(json.dumps(line), flush=True)
    for b in bufs:
        b.free()


def main():
    args = parse_args()
    from bruno_gb300 import synth
    if args.workload == "batched" and args.impl != "reference":
        run_batched(args)
        return
    if args.workload == "served" and args.impl != "reference":
        run_served(args)
        return
    w = synth.WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, w)
        return
    import torch
    import bruno_gb300 as bg
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()   # a real (non-default) stream shared by the library and the events
    torch.cuda.set_stream(stream)

    # workload in pinned host memory, and a device-resident copy
    n = synth.fastq_size(w)
    host = bg.PinnedBuffer(n)
    synth.make_fastq(w, out=host.array)
    dev = torch.empty(n, dtype=torch.uint8, device="cuda")
    dev.copy_(torch.from_numpy(host.array[:n]), non_blocking=False)
    torch.cuda.synchronize()

    max_load = args.max_load or (0.7 if w.k > 31 else 0.5)
    g = bg.Graph(k=w.k, thresh=bg.thresholds(w.lower), min_update=True, device=local, max_load=max_load,
                 h2d_streams=args.h2d_streams, h2d_chunk=args.h2d_chunk, rank_fill=args.rank_fill,
                 part_slots=args.part_slots, count_threads=args.count_threads)
    g.set_stream(stream.cuda_stream)

    def step_device():
        if args.api == "build":
            g.build_and_compact(dev.data_ptr(), nbytes=n, is_device=True)
        else:
            g.reset()
            g.load_fastq(dev.data_ptr(), nbytes=n, is_device=True)
            g.compute_biedge_freqencies()
            g.local_insert_by_freqencies()
            g.extract_chains()
            g.list_rank_min_update()
            g.to_compressed_chains()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step_device()
    sizes = g.sizes()
    barrier()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kms, launches = [], 0
    with ClockSampler(local) as clk:
        start.record(stream)
        for _ in range(args.steps):
            step_device()
            kms.append(g.phase_ms())
            launches += g.sizes()["launches"]
        end.record(stream)
        barrier()
    ms = max_over_ranks(start.elapsed_time(end), world)
    inst_step = sizes["n_instances"]
    value = inst_step * args.steps * world / (ms / 1e3)

    # end to end through the C ABI: host FASTQ in, compacted chains out
    nc, nch = sizes["n_chains"], sizes["n_chain_chars"]
    out_chars = bg.PinnedBuffer(max(1, nch))
    out_offs = bg.PinnedBuffer(8 * (nc + 1))
    out_reps = bg.PinnedBuffer(8 * g.words * max(1, nc))
    import ctypes

    def step_e2e():
        g.build_and_compact(host.array[:n])
        ncs, nchs = ctypes.c_size_t(), ctypes.c_size_t()
        g._check(g.lib.bruno_copy_chains(g.ctx, ctypes.c_void_p(out_reps.ptr), ctypes.c_void_p(out_offs.ptr),
                                         ctypes.c_void_p(out_chars.ptr), nc, max(1, nch), ctypes.byref(ncs),
                                         ctypes.byref(nchs)), "copy_chains")
    e2e_phases = []
    if args.e2e_workers > 0:
        # steps streamed through a pool of contexts: each step still copies its FASTQ in and its
        # chains out, but one step's copy runs under the previous step's device work; host clock
        # between device synchronisations (the pool's workers run on streams of their own)
        pool = bg.Pool(workers=args.e2e_workers, k=w.k, thresh=bg.thresholds(w.lower), min_update=True,
                       device=local, h2d_streams=args.h2d_streams, h2d_chunk=args.h2d_chunk,
                       rank_fill=args.rank_fill)
        for t in [pool.submit(host.array[:n]) for _ in range(args.e2e_workers)]:
            assert pool.wait(t)["status"] == 0
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        tickets = [pool.submit(host.array[:n]) for _ in range(args.steps)]
        res = [pool.wait(t) for t in tickets]
        torch.cuda.synchronize()
        ems = max_over_ranks((time.perf_counter() - t0) * 1e3, world)
        pool.close()
        assert all(r["status"] == 0 and r["sizes"]["n_instances"] == inst_step for r in res)
    else:
        step_e2e()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step_e2e()
            e2e_phases.append(g.phase_ms())
        e1.record(stream)
        barrier()
        ems = max_over_ranks(e0.elapsed_time(e1), world)
    e2e_value = inst_step * args.steps * world / (ems / 1e3)
    d2h = nch + 8 * (nc + 1) + 8 * g.words * nc

    # Roofline of the dominant kernel.  Each candidate's algorithmic bytes per launch (one
    # launch per step each) and its CUDA-event time on the library's stream.  k <= 31:
    #   k_extract      FASTQ bytes + 16 B read span per read read once, 8 B per record written
    #   k_split        8 B per record read and written once
    #   k_count_local  8 B per record read once + 32 B per table slot written once + 4 B per
    #                  slot it lists for the filter
    #   k_filter       32 B per slot it reads (the listed ones) + 32 B per graph node written once
    mean = lambda key: statistics.mean(p[key] for p in kms)
    peak, peak_src = measured_peak()
    slots = sizes["table_slots"]
    listed = sizes["filter_slots_read"]
    if w.k <= 31:
        kern = {
            "k_extract": (n + 16 * sizes["n_reads"] + 8 * inst_step, mean("count_estimate")),
            "k_split": (16 * inst_step, mean("count_split")),
            "k_count_local": (8 * inst_step + 32 * slots + 4 * listed, mean("count_insert") - mean("count_split")),
            "k_filter": (32 * listed + 32 * sizes["n_nodes"], mean("filter_insert")),
        }
    elif sizes["table_partitions"] > 1:
        # k > 31, partitioned (128-bit keys, 16-byte records, 64-byte slots):
        #   k_extract      FASTQ bytes + 16 B read span per read read once, 16 B per record written
        #   k_split_scatter 16 B per record read and written once (into its partition's region)
        #   k_count_local2 16 B per record read once + 64 B per slot written once + 4 B per listed slot
        #   k_filter       64 B per slot it reads + 64 B per graph node written once
        kern = {
            "k_extract": (n + 16 * sizes["n_reads"] + 16 * inst_step, mean("count_estimate")),
            "k_split_scatter": (32 * inst_step, mean("count_split")),
            "k_count_local2": (16 * inst_step + 64 * slots + 4 * listed, mean("count_insert") - mean("count_split")),
            "k_filter": (64 * listed + 64 * sizes["n_nodes"], mean("filter_insert")),
        }
    else:
        # k > 31 counted straight into the whole table (the fallback for skewed inputs):
        #   k_hll          FASTQ bytes + 16 B read span per read read once (the distinct estimate)
        #   k_table_init   64 B per slot written once
        #   k_count        FASTQ bytes read once + one random 64-byte read-modify-write per instance
        #   k_filter       64 B per slot it reads + 64 B per graph node written once
        kern = {
            "k_hll": (n + 16 * sizes["n_reads"], mean("count_estimate")),
            "k_table_init": (64 * slots, mean("count_table_init")),
            "k_count": (n + 64 * inst_step, mean("count_insert")),
            "k_filter": (64 * listed + 64 * sizes["n_nodes"], mean("filter_insert")),
        }
    kernels = {k: {"alg_bytes_per_launch": b, "launch_ms": t, "achieved": b / (t / 1e3) / 1e9 if t > 0 else None,
                   "frac": b / (t / 1e3) / 1e9 / peak if t > 0 else None} for k, (b, t) in kern.items()}
    top = max(kernels, key=lambda k: kernels[k]["launch_ms"])
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tj = json.load(f)
        if top in tj and tj[top].get("bytes_per_record"):
            traffic = tj[top]["bytes_per_record"] * inst_step
    phases = {k: round(statistics.mean(p[k] for p in kms), 3) for k in kms[0]}

    # The whole path against the HBM roofline, with the path's algorithmic bytes:
    #   FASTQ once + one random 64-byte read-modify-write per (k-mer, biedge) instance + one
    #   scan of the distinct entries (16 B each at k <= 31, 32 B above) + one 64-byte update
    #   per kept entry + one scan of the node table (32 / 48 B a node) + three 32-byte touches
    #   per chain node + the emitted chains (sequence bytes + 24-byte listranked records),
    # over the device-resident step time.
    s2, s1 = (16, 32) if w.k <= 31 else (32, 48)
    kept = sum(sizes["filter_flag_hist"][:3])
    path_bytes = (n + 64 * inst_step + s2 * sizes["n_k2"] + 64 * kept + s1 * sizes["n_nodes"]
                  + 96 * sizes["n_chain_nodes"] + sizes["n_chain_chars"] + 24 * sizes["n_ranked"])
    path_achieved = path_bytes / (ms / args.steps / 1e3) / 1e9

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded generator, " + w.name + ")",
                "config": workload_config(w),
                "run": {"api": "bruno_build_and_compact" if args.api == "build" else "step calls",
                        "h2d_streams": args.h2d_streams, "h2d_chunk": args.h2d_chunk or 256 << 20,
                        "rank_fill": args.rank_fill, "max_load": max_load,
                        "part_slots": args.part_slots or 3072, "count_threads": args.count_threads or 512},
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n, "d2h_bytes_per_step": d2h,
                        "ms_per_step": ems / args.steps,
                        "h2d_ms": statistics.mean(p["h2d"] for p in e2e_phases) if e2e_phases else None,
                        "device_ms": statistics.mean(sum(p[k] for k in ("parse", "count_k2mers", "filter_insert",
                                                                        "chainmap", "list_rank", "compress"))
                                                     for p in e2e_phases) if e2e_phases else None,
                        "contexts": max(1, args.e2e_workers)},
                "roofline": {"bound": "hbm", "kernel": top, "achieved": kernels[top]["achieved"], "peak": peak,
                             "unit": "GB/s", "frac": kernels[top]["frac"], "peak_source": peak_src,
                             "traffic": traffic, "alg_bytes_per_launch": kernels[top]["alg_bytes_per_launch"],
                             "launch_ms": kernels[top]["launch_ms"], "kernels": kernels},
                "path_roofline": {"bound": "hbm", "alg_bytes_per_step": path_bytes, "achieved": path_achieved,
                                  "peak": peak, "unit": "GB/s", "frac": path_achieved / peak},
                "gpu_launches": launches, "clocks": clk.summary(), "phase_ms": phases,
                "sizes": {k: sizes[k] for k in ("n_reads", "n_instances", "n_k2", "n_nodes", "n_branch",
                                                "n_chain_nodes", "iterations", "n_chains", "table_slots",
                                                "table_partitions")}}
        if not args.no_cpu_baseline:
            b = cpu_baseline(w, args.cpu_sample, os.cpu_count() or 1)
            line["cpu_baseline"] = {k: b[k] for k in ("value", "unit", "cores", "kind", "sample", "phases_s")}
        print(json.dumps(line), flush=True)
    g.close()
    host.free()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
