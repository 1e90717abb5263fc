/*
 * capi.cu -- the C ABI (include/bruno_gb300.h): context lifetime, device memory, the
 * pipeline state machine and the copy-outs.  All device work is stream-ordered on the
 * context's stream; the host synchronises only to read small counters between phases.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "internal.cuh"
#include "piece_cuts.h"

namespace bg {

bruno_status set_err(Ctx *c, bruno_status s, const std::string &msg) {
  if (c) c->err = msg;
  return s;
}

bruno_status cuda_check(Ctx *c, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return BRUNO_OK;
  return set_err(c, e == cudaErrorMemoryAllocation ? BRUNO_ERR_OOM : BRUNO_ERR_CUDA,
                 std::string(what) + ": " + cudaGetErrorString(e));
}

/* Buffers grow with 1/8 headroom, so a context reused for inputs of varying size rarely
 * reallocates, and they are allocated and released in the order of the context's stream:
 * growing never waits for the work of other contexts on the device. */
bruno_status ensure(Ctx *c, Buf &b, size_t bytes, bool preserve) {
  if (bytes <= b.bytes && b.p) return BRUNO_OK;
  void *p = nullptr;
  /* an eighth more, at most 1 GiB more, so that a slightly larger rebuild keeps the buffer */
  size_t want = std::max(bytes + std::min(bytes / 8, (size_t)1 << 30), (size_t)256);
  cudaError_t e = cudaMallocFromPoolAsync(&p, want, c->pool, c->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, BRUNO_ERR_OOM, "device allocation of " + std::to_string(want) + " bytes failed");
  }
  if (preserve && b.p && b.bytes) cudaMemcpyAsync(p, b.p, b.bytes, cudaMemcpyDeviceToDevice, c->stream);
  if (b.p) cudaFreeAsync(b.p, c->stream);
  b.p = p;
  b.bytes = want;
  return BRUNO_OK;
}

/* The library's own stream-ordered pool on a device (created once, kept for the process): it
 * keeps what is freed instead of returning it at every synchronisation, so a context that
 * rebuilds with the same sizes never waits for memory to be mapped again; the device's default
 * pool, which other code in the process may use, is left as it is. */
cudaMemPool_t library_pool(int device) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  if (device < 0 || device >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!pools[device]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t p = nullptr;
    if (cudaMemPoolCreate(&p, &props) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[device] = p;
  }
  return pools[device];
}

static void release(Buf &b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

bruno_status sync_counters(Ctx *c, bool with_hll) {
  const size_t n = with_hll ? offsetof(DevCounters, big_key) : offsetof(DevCounters, hll);
  cudaError_t e = cudaMemcpyAsync(c->hctr, c->dctr, n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  return cuda_check(c, e, "device phase");
}

static void record(Ctx *c, int i) { cudaEventRecord(c->ev[i], c->stream); }

static double elapsed(Ctx *c, int a, int b) {
  float ms = 0;
  if (cudaEventElapsedTime(&ms, c->ev[a], c->ev[b]) != cudaSuccess) { cudaGetLastError(); return 0; }
  return ms;
}

}  // namespace bg

using namespace bg;

struct bruno_ctx : public Ctx {};

extern "C" {

bruno_status bruno_ctx_create(const bruno_cfg *cfg, bruno_ctx **out) {
  if (!cfg || !out) return BRUNO_ERR_ARG;
  *out = nullptr;
  if (cfg->k < 3 || cfg->k > 63) return BRUNO_ERR_ARG;
  if (cfg->edge_filter && cfg->thresholding && cfg->direct_count == 1) return BRUNO_ERR_ARG;
  bruno_ctx *c = new (std::nothrow) bruno_ctx();
  if (!c) return BRUNO_ERR_OOM;
  c->cfg = *cfg;
  if (!c->cfg.thresholding) c->cfg.edge_filter = 0;   /* build_index: no filter at all */
  c->W = cfg->k <= 31 ? 1 : 2;
  c->exact_ranking = cfg->exact_ranking != 0;
  c->force_direct_count = cfg->direct_count;
  bruno_status st = cuda_check(c, cudaSetDevice(cfg->device), "cudaSetDevice");
  if (st == BRUNO_OK && !(c->pool = library_pool(cfg->device)))
    st = set_err(c, BRUNO_ERR_CUDA, "stream-ordered memory pool");
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");
  c->own_stream = true;
  /* The k-mer table is read at random, one 32-byte slot per probe: ask L2 to fetch only
   * the sector that missed (a hint for this process's context only). */
  if (st == BRUNO_OK) { cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, 32); cudaGetLastError(); }
  if (st == BRUNO_OK) st = cuda_check(c, cudaMalloc(&c->dctr, sizeof(DevCounters)), "counters");
  if (st == BRUNO_OK) st = cuda_check(c, cudaMallocHost(&c->hctr, sizeof(DevCounters)), "pinned counters");
  for (int i = 0; i < 8 && st == BRUNO_OK; ++i) st = cuda_check(c, cudaEventCreate(&c->ev[i]), "event");
  for (int i = 0; i < 5 && st == BRUNO_OK; ++i) st = cuda_check(c, cudaEventCreate(&c->kev[i]), "event");
  if (st == BRUNO_OK) st = cuda_check(c, cudaEventCreate(&c->h2d_end), "event");
  if (st == BRUNO_OK) st = cuda_check(c, cudaEventCreateWithFlags(&c->order_ev, cudaEventDisableTiming), "event");
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking), "stream");
  c->n_copy = std::max(1, std::min(4, (int)c->cfg.h2d_streams));
  for (int i = 0; i + 1 < c->n_copy && st == BRUNO_OK; ++i) {
    st = cuda_check(c, cudaStreamCreateWithFlags(&c->copy_more[i], cudaStreamNonBlocking), "stream");
    if (st == BRUNO_OK) st = cuda_check(c, cudaEventCreateWithFlags(&c->copy_tail[i], cudaEventDisableTiming), "event");
  }
  if (st != BRUNO_OK) { bruno_ctx_destroy(c); return st; }
  cudaMemsetAsync(c->dctr, 0, sizeof(DevCounters), c->stream);
  *out = c;
  return BRUNO_OK;
}

bruno_status bruno_ctx_destroy(bruno_ctx *c) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  for (cudaStream_t s : c->copy_more) if (s) cudaStreamSynchronize(s);
  if (c->stream) cudaStreamSynchronize(c->stream);
  Buf *bufs[] = {&c->rstart, &c->rend, &c->tile_cnt, &c->tile_base, &c->table, &c->k2_keys, &c->k2_edges, &c->k2_counts,
                 &c->f_keys, &c->f_edges, &c->f_counts, &c->blk_cnt, &c->blk_base, &c->ckey, &c->cedge,
                 &c->cstate, &c->cstate2, &c->pend, &c->pay, &c->unf0, &c->unf1, &c->removed, &c->r_K, &c->r_rep, &c->r_dist,
                 &c->rep_idx, &c->head_of, &c->heads, &c->head_len, &c->head_off, &c->ch_rep, &c->ch_off, &c->ch_chars, &c->chain_list, &c->branch_list, &c->e_ends, &c->e_freqs, &c->s_kmers, &c->s_dist, &c->s_flags, &c->k1tab,
                 &c->cl_trec, &c->cl_tslot, &c->cl_sums, &c->cl_norm, &c->cl_htab, &c->cl_q, &c->cl_found,
                 &c->records, &c->bucket_cnt, &c->records2, &c->sub_cnt, &c->bigres, &c->cand, &c->scan_tmp, &c->fr_tmp,
                 &c->xsamp, &c->hllreg, &c->hsum, &c->sgeom, &c->s_tally, &c->s_inst, &c->s_used, &c->xitems,
                 &c->split_items, &c->csample, &c->r_samp, &c->h_samp, &c->grp_tmp};
  for (Buf *b : bufs) release(*b);
  for (Buf &b : c->seg_bufs) release(b);
  if (c->dctr) cudaFree(c->dctr);
  if (c->hctr) cudaFreeHost(c->hctr);
  for (int i = 0; i < 8; ++i) if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  for (int i = 0; i < 5; ++i) if (c->kev[i]) cudaEventDestroy(c->kev[i]);
  for (cudaEvent_t e : c->seg_ev) cudaEventDestroy(e);
  if (c->h2d_end) cudaEventDestroy(c->h2d_end);
  if (c->order_ev) cudaEventDestroy(c->order_ev);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  for (int i = 0; i < 3; ++i) {
    if (c->copy_more[i]) cudaStreamDestroy(c->copy_more[i]);
    if (c->copy_tail[i]) cudaEventDestroy(c->copy_tail[i]);
  }
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return BRUNO_OK;
}

bruno_status bruno_set_stream(bruno_ctx *c, void *stream) {
  if (!c) return BRUNO_ERR_ARG;
  cudaStreamSynchronize(c->stream);
  if (stream) {
    if (c->own_stream) cudaStreamDestroy(c->stream);
    c->stream = (cudaStream_t)stream;
    c->own_stream = false;
  } else if (!c->own_stream) {
    bruno_status st = cuda_check(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");
    if (st != BRUNO_OK) return st;
    c->own_stream = true;
  }
  return BRUNO_OK;
}

const char *bruno_last_error(const bruno_ctx *c) { return c ? c->err.c_str() : "null context"; }

bruno_status bruno_reset(bruno_ctx *c) {
  if (!c) return BRUNO_ERR_ARG;
  c->segs.clear();
  c->stage = 0;
  c->S = 1;   /* the plain build; bruno_build_samples sets a batch */
  c->samp_off.clear();
  c->samp_r0.clear();
  c->batch_piped = false;
  c->seg_samp.clear();
  c->n_reads = c->n_reads_used = c->n_instances = c->n_entries = 0;
  c->n_k2 = c->n_filtered = 0;
  c->k2_dumped = false;
  c->h2d_pending = false;
  c->h2d_piped = false;
  c->host_loads = 0;
  c->seg_ev_used = 0;
  /* copies still queued on the copy stream finish before the context's stream frees or reuses
   * their buffers */
  if (c->copy_stream) {
    cudaEventRecord(c->order_ev, c->copy_stream);
    cudaStreamWaitEvent(c->stream, c->order_ev, 0);
    for (int i = 0; i + 1 < c->n_copy; ++i) {
      cudaEventRecord(c->order_ev, c->copy_more[i]);
      cudaStreamWaitEvent(c->stream, c->order_ev, 0);
    }
  }
  c->n_nodes = c->n_branch = c->n_chain = c->filter_read = 0;
  c->iterations = c->n_cycle = c->n_isolated = c->multi = 0;
  c->n_ranked = c->n_heads = c->n_chain_chars = 0;
  c->chains_clean = true;
  c->n_chain_edges = 0;
  c->chain_edges_done = false;
  c->n_summaries = 0;
  c->summaries_done = false;
  c->general_emission = false;
  c->cleaned = false;
  c->launches = 0;
  std::memset(c->flag_hist, 0, sizeof(c->flag_hist));
  std::memset(c->phase_ms, 0, sizeof(c->phase_ms));
  c->err.clear();
  return BRUNO_OK;
}

bruno_status bruno_load_fastq(bruno_ctx *c, const char *buf, size_t nbytes, int32_t is_device) {
  if (!c || (!buf && nbytes)) return BRUNO_ERR_ARG;
  if (c->stage > 1) return set_err(c, BRUNO_ERR_ARG, "load_fastq after counting; call bruno_reset first");
  if (is_device) {
    c->segs.push_back({buf, nbytes});
  } else {
    const size_t i = c->host_loads++;
    if (c->seg_bufs.size() <= i) c->seg_bufs.resize(i + 1);
    const std::vector<uint64_t> cuts = piece_cuts(buf, nbytes, c->cfg.h2d_chunk ? c->cfg.h2d_chunk : (256ull << 20));
    /* each piece starts on a 16-byte boundary of the device copy, for the parser's vector loads */
    bruno_status st = ensure(c, c->seg_bufs[i], nbytes + 16 * cuts.size() + 1);
    if (st != BRUNO_OK) return st;
    char *dst = (char *)c->seg_bufs[i].p;
    if (cuts.size() < 2 && !c->h2d_piped) {   /* one piece: copied on the context's stream */
      if (!c->h2d_pending) { record(c, 7); c->h2d_pending = true; }   /* before the first host copy */
      st = cuda_check(c, cudaMemcpyAsync(dst, buf, nbytes, cudaMemcpyHostToDevice, c->stream), "H2D FASTQ");
      if (st != BRUNO_OK) return st;
      c->segs.push_back({dst, nbytes});
    } else {
      /* pieces on the copy stream, after whatever the context's stream has queued (the buffer's
       * allocation, an earlier copy); each piece is a segment with its own event, so that the
       * read index parses a piece while the next one is still in flight */
      cudaEventRecord(c->order_ev, c->stream);
      cudaStreamWaitEvent(c->copy_stream, c->order_ev, 0);
      for (int i = 0; i + 1 < c->n_copy; ++i) cudaStreamWaitEvent(c->copy_more[i], c->order_ev, 0);
      if (!c->h2d_pending) { cudaEventRecord(c->ev[7], c->copy_stream); c->h2d_pending = true; }
      uint64_t at = 0;   /* where the piece goes in the device copy */
      for (size_t j = 0; j < cuts.size(); ++j) {
        const uint64_t off = cuts[j], len = (j + 1 < cuts.size() ? cuts[j + 1] : nbytes) - off;
        const int sj = (int)(j % (size_t)c->n_copy);   /* pieces go round robin over the copy streams */
        cudaStream_t cs = sj == 0 ? c->copy_stream : c->copy_more[sj - 1];
        st = cuda_check(c, cudaMemcpyAsync(dst + at, buf + off, len, cudaMemcpyHostToDevice, cs), "H2D FASTQ");
        if (st != BRUNO_OK) return st;
        if (c->seg_ev_used == c->seg_ev.size()) {
          cudaEvent_t e;
          st = cuda_check(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
          if (st != BRUNO_OK) return st;
          c->seg_ev.push_back(e);
        }
        const int ev = (int)c->seg_ev_used++;
        cudaEventRecord(c->seg_ev[ev], cs);
        c->segs.push_back({dst + at, len, ev});
        at = (at + len + 15) & ~15ull;
      }
      for (int i = 0; i + 1 < c->n_copy; ++i) {   /* h2d_end after the last copy of every stream */
        cudaEventRecord(c->copy_tail[i], c->copy_more[i]);
        cudaStreamWaitEvent(c->copy_stream, c->copy_tail[i], 0);
      }
      cudaEventRecord(c->h2d_end, c->copy_stream);
      c->h2d_piped = true;
    }
  }
  c->stage = 1;
  return BRUNO_OK;
}

bruno_status bruno_compute_biedge_freqencies(bruno_ctx *c) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->stage != 1) return set_err(c, BRUNO_ERR_ARG, "compute_biedge_freqencies needs loaded FASTQ");
  record(c, 0);
  bruno_status st = run_index_reads(c);
  if (st != BRUNO_OK) return st;
  record(c, 1);
  st = run_count(c);
  if (st != BRUNO_OK) return st;
  record(c, 2);
  if (c->cfg.keep_k2 && (st = run_dump_k2(c)) != BRUNO_OK) return st;
  cudaEventSynchronize(c->ev[2]);
  c->phase_ms[0] = elapsed(c, 0, 1);
  if (c->h2d_pending) {   /* the copies: back to back right before this call's start event, or
                            on the copy stream beneath the read index */
    if (c->h2d_piped) {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, c->ev[7], c->h2d_end) != cudaSuccess) { cudaGetLastError(); ms = 0; }
      c->phase_ms[10] = ms;
    } else {
      c->phase_ms[10] = elapsed(c, 7, 0);
    }
    c->h2d_pending = false;
  }
  c->phase_ms[1] = elapsed(c, 1, 2);
  c->stage = 2;
  return BRUNO_OK;
}

bruno_status bruno_local_insert_by_freqencies(bruno_ctx *c, const uint64_t *thresh) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->stage != 2) return set_err(c, BRUNO_ERR_ARG, "local_insert_by_freqencies needs counted (k+2)-mers");
  record(c, 2);
  std::memcpy(c->thr_used, thresh ? thresh : c->cfg.thresh, sizeof(c->thr_used));
  bruno_status st = run_filter(c, c->thr_used);
  if (st != BRUNO_OK) return st;
  record(c, 3);
  cudaEventSynchronize(c->ev[3]);
  c->phase_ms[2] = elapsed(c, 2, 3);
  c->stage = 3;
  return BRUNO_OK;
}

bruno_status bruno_extract_chains(bruno_ctx *c) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->stage != 3) return set_err(c, BRUNO_ERR_ARG, "extract_chains needs the filtered graph");
  record(c, 3);
  bruno_status st = run_extract_chains(c);
  if (st != BRUNO_OK) return st;
  record(c, 4);
  cudaEventSynchronize(c->ev[4]);
  c->phase_ms[3] = elapsed(c, 3, 4);
  c->stage = 4;
  return BRUNO_OK;
}

bruno_status bruno_list_rank(bruno_ctx *c, int32_t min_update, uint64_t *iterations) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->stage != 4) return set_err(c, BRUNO_ERR_ARG, "list_rank needs extracted chains");
  record(c, 4);
  bruno_status st = run_list_rank(c, min_update);
  if (st != BRUNO_OK) return st;
  record(c, 5);
  cudaEventSynchronize(c->ev[5]);
  c->phase_ms[4] = elapsed(c, 4, 5);
  if (iterations) *iterations = c->iterations;
  c->stage = 5;
  return BRUNO_OK;
}

bruno_status bruno_to_compressed_chains(bruno_ctx *c) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->stage != 5) return set_err(c, BRUNO_ERR_ARG, "to_compressed_chains needs ranked chains");
  record(c, 5);
  bruno_status st = run_compress(c);
  if (st != BRUNO_OK) return st;
  record(c, 6);
  cudaEventSynchronize(c->ev[6]);
  c->phase_ms[5] = elapsed(c, 5, 6);
  c->stage = 6;
  if (!c->chains_clean)
    return set_err(c, BRUNO_ERR_INVARIANT,
                   "chain pointers are not mutually consistent (asymmetric edge filtering); the listranked "
                   "nodes are valid, the compacted sequences are not");
  return BRUNO_OK;
}

bruno_status bruno_clean_deadend_and_bubbles_naive(bruno_ctx *c, bruno_clean_stats *stats) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->S > 1) return set_err(c, BRUNO_ERR_ARG, "graph cleaning works on one graph; build it with bruno_build_and_compact");
  if (c->stage < 5) return set_err(c, BRUNO_ERR_ARG, "cleaning needs ranked chains");
  if (c->cleaned) return set_err(c, BRUNO_ERR_ARG, "the graph is cleaned already; call bruno_reset first");
  bruno_clean_stats s{};
  record(c, 5);
  bruno_status st = run_clean(c, &s.rounds, &s.deadends, &s.bubbles, &s.edges, &s.status);
  if (stats) *stats = s;
  if (st != BRUNO_OK) return st;
  record(c, 6);
  cudaEventSynchronize(c->ev[6]);
  c->phase_ms[5] = elapsed(c, 5, 6);
  c->cleaned = true;
  c->stage = 6;
  if (!c->chains_clean)
    return set_err(c, BRUNO_ERR_INVARIANT,
                   "chain pointers are not mutually consistent (asymmetric edge filtering); the listranked "
                   "nodes are valid, the compacted sequences are not");
  return BRUNO_OK;
}

bruno_status bruno_build_and_compact(bruno_ctx *c, const char *buf, size_t nbytes, int32_t is_device) {
  if (!c) return BRUNO_ERR_ARG;
  bruno_status st = bruno_reset(c);
  if (st == BRUNO_OK) st = bruno_load_fastq(c, buf, nbytes, is_device);
  if (st == BRUNO_OK) st = bruno_compute_biedge_freqencies(c);
  if (st == BRUNO_OK) st = bruno_local_insert_by_freqencies(c, nullptr);
  if (st == BRUNO_OK) st = bruno_extract_chains(c);
  if (st == BRUNO_OK) st = bruno_list_rank(c, c->cfg.min_update, nullptr);
  if (st == BRUNO_OK) st = bruno_to_compressed_chains(c);
  return st;
}

bruno_status bruno_get_sizes(bruno_ctx *c, bruno_sizes *o) {
  if (!c || !o) return BRUNO_ERR_ARG;
  std::memset(o, 0, sizeof(*o));
  o->n_reads = c->n_reads;
  o->n_reads_used = c->n_reads_used;
  o->n_instances = c->n_instances;
  o->n_k2 = c->n_entries;
  o->n_filtered = c->n_filtered;
  o->n_nodes = c->n_nodes;
  o->n_branch = c->n_branch;
  o->n_chain_nodes = c->n_chain;
  o->iterations = c->iterations;
  o->n_cycle_nodes = c->n_cycle;
  o->n_isolated = c->n_isolated;
  o->n_ranked = c->n_ranked;
  o->n_chains = c->n_heads;
  o->n_chain_chars = c->n_chain_chars;
  o->table_slots = c->nslots;
  o->collisions = c->multi;
  o->launches = c->launches;
  o->table_partitions = 1ull << c->geom.pbits;
  o->grouped_chains = c->general_emission ? 1 : 0;
  o->filter_slots_read = c->filter_read;
  for (int f = 0; f < 16; ++f) o->filter_flag_hist[f] = c->flag_hist[f];
  return BRUNO_OK;
}

static bruno_status copy_d2h(Ctx *c, void *dst, const void *src, size_t bytes) {
  if (!dst || !bytes) return BRUNO_OK;
  return cuda_check(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream), "D2H copy");
}

static bruno_status copy_triple(Ctx *c, uint64_t n, const Buf &k, const Buf &e, const Buf &cnt, uint64_t *keys,
                                uint8_t *edges, uint32_t *counts, size_t cap, size_t *out_n) {
  if (out_n) *out_n = n;
  if (!keys && !edges && !counts) return BRUNO_OK;
  if (cap < n) return set_err(c, BRUNO_ERR_CAPACITY, "copy buffer too small");
  bruno_status st = copy_d2h(c, keys, k.p, n * 8 * c->W);
  if (st == BRUNO_OK) st = copy_d2h(c, edges, e.p, n);
  if (st == BRUNO_OK) st = copy_d2h(c, counts, cnt.p, n * 4);
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  return st;
}

bruno_status bruno_copy_k2(bruno_ctx *c, uint64_t *keys, uint8_t *edges, uint32_t *counts, size_t cap, size_t *n) {
  if (!c) return BRUNO_ERR_ARG;
  if (!c->k2_dumped) return set_err(c, BRUNO_ERR_ARG, "raw (k+2)-mer counts need cfg.keep_k2 and a counted build");
  return copy_triple(c, c->n_k2, c->k2_keys, c->k2_edges, c->k2_counts, keys, edges, counts, cap, n);
}

bruno_status bruno_copy_filtered(bruno_ctx *c, uint64_t *keys, uint8_t *edges, uint32_t *counts, size_t cap, size_t *n) {
  if (!c) return BRUNO_ERR_ARG;
  if (!c->cfg.keep_filtered || c->stage < 3) return set_err(c, BRUNO_ERR_ARG, "filtered entries need cfg.keep_filtered");
  return copy_triple(c, c->n_filtered, c->f_keys, c->f_edges, c->f_counts, keys, edges, counts, cap, n);
}

bruno_status bruno_copy_nodes(bruno_ctx *c, uint64_t *keys, uint16_t *counts, uint8_t *flags, size_t cap, size_t *n) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->stage < 3) return set_err(c, BRUNO_ERR_ARG, "nodes exist after local_insert_by_freqencies");
  return run_copy_nodes(c, keys, counts, flags, cap, n);
}

bruno_status bruno_copy_ranked(bruno_ctx *c, uint64_t *K, uint64_t *rep, int32_t *dist, size_t cap, size_t *n) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->stage < 6) return set_err(c, BRUNO_ERR_ARG, "ranked nodes exist after to_compressed_chains");
  if (n) *n = c->n_ranked;
  if (!K && !rep && !dist) return BRUNO_OK;
  if (cap < c->n_ranked) return set_err(c, BRUNO_ERR_CAPACITY, "copy buffer too small");
  bruno_status st = copy_d2h(c, K, c->r_K.p, c->n_ranked * 8 * c->W);
  if (st == BRUNO_OK) st = copy_d2h(c, rep, c->r_rep.p, c->n_ranked * 8 * c->W);
  if (st == BRUNO_OK) st = copy_d2h(c, dist, c->r_dist.p, c->n_ranked * 4);
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  return st;
}

bruno_status bruno_copy_chains(bruno_ctx *c, uint64_t *reps, uint64_t *offsets, char *chars, size_t cap_chains,
                               size_t cap_chars, size_t *n_chains, size_t *n_chars) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->stage < 6) return set_err(c, BRUNO_ERR_ARG, "chains exist after to_compressed_chains");
  if (n_chains) *n_chains = c->n_heads;
  if (n_chars) *n_chars = c->n_chain_chars;
  if (!reps && !offsets && !chars) return BRUNO_OK;
  if ((reps || offsets) && cap_chains < c->n_heads) return set_err(c, BRUNO_ERR_CAPACITY, "chain buffer too small");
  if (chars && cap_chars < c->n_chain_chars) return set_err(c, BRUNO_ERR_CAPACITY, "char buffer too small");
  bruno_status st = copy_d2h(c, reps, c->ch_rep.p, c->n_heads * 8 * c->W);
  if (st == BRUNO_OK) st = copy_d2h(c, offsets, c->head_off.p, (c->n_heads + 1) * 8);
  if (st == BRUNO_OK) st = copy_d2h(c, chars, c->ch_chars.p, c->n_chain_chars);
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  return st;
}

bruno_status bruno_device_results(bruno_ctx *c, bruno_device_view *o) {
  if (!c || !o) return BRUNO_ERR_ARG;
  if (c->stage < 6) return set_err(c, BRUNO_ERR_ARG, "results exist after to_compressed_chains");
  bruno_status st = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  if (st != BRUNO_OK) return st;
  std::memset(o, 0, sizeof(*o));
  o->ranked_K = (const uint64_t *)c->r_K.p;
  o->ranked_rep = (const uint64_t *)c->r_rep.p;
  o->ranked_dist = (const int32_t *)c->r_dist.p;
  o->chain_reps = (const uint64_t *)c->ch_rep.p;
  o->chain_offsets = (const uint64_t *)c->head_off.p;
  o->chain_chars = (const char *)c->ch_chars.p;
  o->n_ranked = c->n_ranked;
  o->n_chains = c->n_heads;
  o->n_chain_chars = c->n_chain_chars;
  o->words = c->W;
  return BRUNO_OK;
}

bruno_status bruno_copy_chain_edges(bruno_ctx *c, uint64_t *ends, uint16_t *freqs, size_t cap, size_t *n) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->stage < 6) return set_err(c, BRUNO_ERR_ARG, "chain edges exist after to_compressed_chains");
  bruno_status st = BRUNO_OK;
  if (!c->chain_edges_done && (st = run_chain_edges(c)) != BRUNO_OK) return st;
  if (n) *n = c->n_chain_edges;
  if (!ends && !freqs) return BRUNO_OK;
  if (cap < c->n_chain_edges) return set_err(c, BRUNO_ERR_CAPACITY, "copy buffer too small");
  st = copy_d2h(c, ends, c->e_ends.p, c->n_chain_edges * 2 * 8 * c->W);
  if (st == BRUNO_OK) st = copy_d2h(c, freqs, c->e_freqs.p, c->n_chain_edges * 11 * 2);
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  return st;
}

bruno_status bruno_copy_chain_summaries(bruno_ctx *c, uint64_t *kmers, uint32_t *dist, uint8_t *flags, size_t cap,
                                        size_t *n) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->stage < 6) return set_err(c, BRUNO_ERR_ARG, "chain summaries exist after to_compressed_chains");
  bruno_status st = BRUNO_OK;
  if (!c->summaries_done && (st = run_chain_summaries(c)) != BRUNO_OK) return st;
  if (n) *n = c->n_summaries;
  if (!kmers && !dist && !flags) return BRUNO_OK;
  if (cap < c->n_summaries) return set_err(c, BRUNO_ERR_CAPACITY, "copy buffer too small");
  st = copy_d2h(c, kmers, c->s_kmers.p, c->n_summaries * 4 * 8 * c->W);
  if (st == BRUNO_OK) st = copy_d2h(c, dist, c->s_dist.p, c->n_summaries * 4);
  if (st == BRUNO_OK) st = copy_d2h(c, flags, c->s_flags.p, c->n_summaries * 2);
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  return st;
}

bruno_status bruno_graph_find_if(bruno_ctx *c, int32_t filter, uint64_t *keys, uint16_t *counts, uint8_t *flags,
                                 size_t cap, size_t *n) {
  if (!c || !n) return BRUNO_ERR_ARG;
  if (filter < BRUNO_NODES_ALL || filter > BRUNO_IS_CHAIN_NODE) return set_err(c, BRUNO_ERR_ARG, "unknown node filter");
  if (c->stage < 3) return set_err(c, BRUNO_ERR_ARG, "nodes exist after local_insert_by_freqencies");
  return run_node_query(c, filter, false, keys, counts, flags, cap, n);
}

bruno_status bruno_graph_erase_if(bruno_ctx *c, int32_t filter, size_t *n_erased) {
  if (!c) return BRUNO_ERR_ARG;
  if (filter < BRUNO_NODES_ALL || filter > BRUNO_IS_CHAIN_NODE) return set_err(c, BRUNO_ERR_ARG, "unknown node filter");
  if (c->stage < 3) return set_err(c, BRUNO_ERR_ARG, "nodes exist after local_insert_by_freqencies");
  size_t n = 0;
  const bruno_status st = run_node_query(c, filter, true, nullptr, nullptr, nullptr, 0, &n);
  if (n_erased) *n_erased = n;
  return st;
}

bruno_status bruno_check_index(bruno_ctx *c, bruno_index_check *out) {
  if (!c || !out) return BRUNO_ERR_ARG;
  if (c->stage < 3) return set_err(c, BRUNO_ERR_ARG, "nodes exist after local_insert_by_freqencies");
  const bruno_status st = run_check_index(c, out);
  if (st != BRUNO_OK) return st;
  if (out->n_absent || out->n_unreferenced)
    return set_err(c, BRUNO_ERR_INVARIANT, "check_index: the graph names absent neighbours or holds unnamed nodes");
  return BRUNO_OK;
}

bruno_status bruno_graph_erase_nodes(bruno_ctx *c, const uint64_t *kmers, size_t n) {
  if (!c || (!kmers && n)) return BRUNO_ERR_ARG;
  if (c->stage < 3) return set_err(c, BRUNO_ERR_ARG, "nodes exist after local_insert_by_freqencies");
  return run_erase_nodes(c, kmers, n);
}

bruno_status bruno_chain_find_if(bruno_ctx *c, int32_t filter, uint64_t *kmers, uint64_t *in_kmers,
                                 uint64_t *out_kmers, uint32_t *in_dist, uint32_t *out_dist, size_t cap, size_t *n) {
  if (!c || !n) return BRUNO_ERR_ARG;
  if (filter < BRUNO_CHAIN_ALL || filter > BRUNO_CHAIN_POINTS_TO_INTERNAL_NODE)
    return set_err(c, BRUNO_ERR_ARG, "unknown chain filter");
  if (c->stage < 4) return set_err(c, BRUNO_ERR_ARG, "the chain map exists after extract_chains");
  return run_chain_query(c, filter, 0, kmers, in_kmers, out_kmers, in_dist, out_dist, cap, n);
}

bruno_status bruno_get_cycle_node_kmers(bruno_ctx *c, uint64_t *kmers, size_t cap, size_t *n) {
  if (!c || !n) return BRUNO_ERR_ARG;
  if (c->stage < 5) return set_err(c, BRUNO_ERR_ARG, "cycle nodes are known after list_rank");
  return run_chain_query(c, BRUNO_CHAIN_ALL, 1, kmers, nullptr, nullptr, nullptr, nullptr, cap, n);
}

bruno_status bruno_get_isolated(bruno_ctx *c, uint64_t *kmers, uint64_t *in_kmers, uint64_t *out_kmers,
                                uint32_t *in_dist, uint32_t *out_dist, size_t cap, size_t *n) {
  if (!c || !n) return BRUNO_ERR_ARG;
  if (c->stage < 5) return set_err(c, BRUNO_ERR_ARG, "isolated nodes are known after list_rank");
  return run_chain_query(c, BRUNO_CHAIN_ALL, 2, kmers, in_kmers, out_kmers, in_dist, out_dist, cap, n);
}

/* ------------------------------------------------------------------ batched form */
/* dst[i] = src[idx[i]] */
__global__ void k_gather_u64(const uint64_t *src, const uint64_t *idx, uint32_t n, uint64_t *dst) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[idx[i]];
}

bruno_status bruno_build_samples(bruno_ctx *c, const char *const *bufs, const size_t *nbytes, size_t n_samples,
                                 int32_t is_device) {
  if (!c || !bufs || !nbytes || n_samples == 0) return BRUNO_ERR_ARG;
  if (n_samples > MAX_SAMPLES) return set_err(c, BRUNO_ERR_ARG, "batch: at most 16384 samples in one batch");
  for (size_t q = 0; q < n_samples; ++q)
    if (!bufs[q] && nbytes[q]) return BRUNO_ERR_ARG;
  if (c->W != 1 || c->cfg.edge_filter || c->cfg.keep_k2 || c->cfg.keep_filtered || c->force_direct_count)
    return set_err(c, BRUNO_ERR_ARG, "batch: k <= 31, the (k+2)-mer filter, no raw or filtered count copies, "
                                     "automatic counting path");
  if (c->cfg.thresholding && (c->cfg.thresh[0] != 0 || c->cfg.thresh[1] < 65536 || c->cfg.thresh[4] != 0 ||
                              c->cfg.thresh[5] < 65536))
    return set_err(c, BRUNO_ERR_ARG, "batch: only the (k+1)-mer bounds may be set (one -L / -U value)");
  bruno_status st = bruno_reset(c);
  if (st != BRUNO_OK) return st;
  /* one device copy of all samples, one after another; a sample whose last byte is not a newline
   * gets one, so that no record runs into the next sample */
  std::vector<unsigned char> last(n_samples, '\n');
  if (is_device) {
    for (size_t q = 0; q < n_samples; ++q)
      if (nbytes[q]) cudaMemcpyAsync(&last[q], bufs[q] + nbytes[q] - 1, 1, cudaMemcpyDeviceToHost, c->stream);
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "sample ends")) != BRUNO_OK) return st;
  } else {
    for (size_t q = 0; q < n_samples; ++q) if (nbytes[q]) last[q] = (unsigned char)bufs[q][nbytes[q] - 1];
  }
  /* host samples travel in groups of whole samples (about cfg.h2d_chunk bytes, each group on a
   * 16-byte boundary) on the copy stream, one event a group, so that the read index parses and
   * extracts each group while the next is in flight */
  const uint64_t group = c->cfg.h2d_chunk ? c->cfg.h2d_chunk : (256ull << 20);
  c->samp_off.assign(n_samples + 1, 0);
  c->seg_samp.assign(1, 0);
  uint64_t at = 0, in_group = 0;
  for (size_t q = 0; q < n_samples; ++q) {
    if (!is_device && in_group >= group) {
      at = (at + 15) & ~15ull;
      c->seg_samp.push_back((uint32_t)q);
      in_group = 0;
    }
    c->samp_off[q] = at;
    const uint64_t len = nbytes[q] + (nbytes[q] && last[q] != '\n' ? 1 : 0);
    at += len;
    in_group += len;
  }
  c->samp_off[n_samples] = at;
  c->seg_samp.push_back((uint32_t)n_samples);
  const uint64_t total = at;
  const size_t ngroups = c->seg_samp.size() - 1;
  if (c->seg_bufs.empty()) c->seg_bufs.resize(1);
  if ((st = ensure(c, c->seg_bufs[0], total + 16)) != BRUNO_OK) return st;
  char *dst = (char *)c->seg_bufs[0].p;
  static const char nl = '\n';
  c->batch_piped = ngroups > 1;
  if (!c->batch_piped) {   /* one copy after another on the context's stream, one segment */
    record(c, 7);
    for (size_t q = 0; q < n_samples && st == BRUNO_OK; ++q) {
      if (!nbytes[q]) continue;
      st = cuda_check(c, cudaMemcpyAsync(dst + c->samp_off[q], bufs[q], nbytes[q],
                                         is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream),
                      "sample copy");
      if (st == BRUNO_OK && last[q] != '\n')
        st = cuda_check(c, cudaMemcpyAsync(dst + c->samp_off[q] + nbytes[q], &nl, 1, cudaMemcpyHostToDevice,
                                           c->stream), "sample end");
    }
    if (st != BRUNO_OK) return st;
    c->segs.push_back({dst, total});
  } else {
    /* after whatever the context's stream has queued (the buffer's allocation) */
    cudaEventRecord(c->order_ev, c->stream);
    cudaStreamWaitEvent(c->copy_stream, c->order_ev, 0);
    cudaEventRecord(c->ev[7], c->copy_stream);
    for (size_t gi = 0; gi < ngroups && st == BRUNO_OK; ++gi) {
      const uint32_t q0 = c->seg_samp[gi], q1 = c->seg_samp[gi + 1];
      for (uint32_t q = q0; q < q1 && st == BRUNO_OK; ++q) {
        if (!nbytes[q]) continue;
        st = cuda_check(c, cudaMemcpyAsync(dst + c->samp_off[q], bufs[q], nbytes[q], cudaMemcpyHostToDevice,
                                           c->copy_stream), "sample copy");
        if (st == BRUNO_OK && last[q] != '\n')
          st = cuda_check(c, cudaMemcpyAsync(dst + c->samp_off[q] + nbytes[q], &nl, 1, cudaMemcpyHostToDevice,
                                             c->copy_stream), "sample end");
      }
      if (st == BRUNO_OK && c->seg_ev_used == c->seg_ev.size()) {
        cudaEvent_t e;
        st = cuda_check(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
        if (st == BRUNO_OK) c->seg_ev.push_back(e);
      }
      if (st != BRUNO_OK) break;
      const int ev = (int)c->seg_ev_used++;
      cudaEventRecord(c->seg_ev[ev], c->copy_stream);
      uint64_t gend = c->samp_off[q0];   /* the group's last byte: its last sample's end, before any padding */
      for (uint32_t q = q0; q < q1; ++q) gend = c->samp_off[q] + nbytes[q] + (nbytes[q] && last[q] != '\n' ? 1 : 0);
      c->segs.push_back({dst + c->samp_off[q0], gend - c->samp_off[q0], ev});
    }
    cudaEventRecord(c->h2d_end, c->copy_stream);
    if (st != BRUNO_OK) return st;
  }
  c->S = (uint32_t)n_samples;
  c->stage = 1;
  record(c, 0);
  if ((st = run_count_samples(c)) != BRUNO_OK) return st;
  record(c, 1);
  cudaEventSynchronize(c->ev[1]);
  if (c->batch_piped) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, c->ev[7], c->h2d_end) != cudaSuccess) { cudaGetLastError(); ms = 0; }
    c->phase_ms[10] = ms;
  } else {
    c->phase_ms[10] = elapsed(c, 7, 0);
  }
  c->phase_ms[1] = elapsed(c, 0, 1);
  c->stage = 2;
  if ((st = bruno_local_insert_by_freqencies(c, nullptr)) != BRUNO_OK) return st;
  if ((st = bruno_extract_chains(c)) != BRUNO_OK) return st;
  if ((st = bruno_list_rank(c, c->cfg.min_update, nullptr)) != BRUNO_OK) return st;
  if (!c->fast_ranked)
    return set_err(c, BRUNO_ERR_INVARIANT, "batch: the chain maps are not mutually consistent");
  if ((st = bruno_to_compressed_chains(c)) != BRUNO_OK) return st;
  /* per-sample tallies and ranges */
  const uint32_t S = c->S;
  c->h_tally.assign((size_t)S * T_NUM, 0);
  st = cuda_check(c, cudaMemcpyAsync(c->h_tally.data(), c->s_tally.p, (size_t)S * T_NUM * 8, cudaMemcpyDeviceToHost,
                                     c->stream), "tallies");
  /* each sample's first chain character: the chain offsets at the samples' first chains,
   * gathered on the device (S + 1 values rather than every chain's offset) */
  std::vector<uint64_t> off(S + 1, 0);
  if (st == BRUNO_OK) st = ensure(c, c->fr_tmp, (size_t)(S + 1) * 16);
  if (st == BRUNO_OK) {
    uint64_t *d = (uint64_t *)c->fr_tmp.p;
    cudaMemcpyAsync(d, c->h_head0.data(), (size_t)(S + 1) * 8, cudaMemcpyHostToDevice, c->stream);
    k_gather_u64<<<(S + 1 + 255) / 256, 256, 0, c->stream>>>((const uint64_t *)c->head_off.p, d, S + 1, d + S + 1);
    c->launches += 1;
    st = cuda_check(c, cudaMemcpyAsync(off.data(), d + S + 1, (size_t)(S + 1) * 8, cudaMemcpyDeviceToHost, c->stream),
                    "chain offsets");
  }
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamSynchronize(c->stream), "tallies");
  if (st != BRUNO_OK) return st;
  c->h_iter.assign(S, 0);
  for (uint32_t q = 0; q < S; ++q) {
    uint64_t *t = &c->h_tally[(size_t)q * T_NUM];
    const uint64_t nmax = t[T_NMAX];
    uint64_t it = 0;
    if (nmax >= 2) { uint64_t x = nmax - 1; while (x >>= 1) ++it; ++it; }   /* floor(log2(nmax-1)) + 1 */
    else if (t[T_CYCLE] > 0) it = 1;
    c->h_iter[q] = it;
    t[T_RANKED] = c->h_rank0[q + 1] - c->h_rank0[q];
    t[T_HEADS] = c->h_head0[q + 1] - c->h_head0[q];
    t[T_CHARS] = off[q + 1] - off[q];
  }
  return BRUNO_OK;
}

static bruno_status batch_sample(bruno_ctx *c, size_t sample) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->S <= 1 || c->stage < 6 || c->h_tally.empty()) return set_err(c, BRUNO_ERR_ARG, "no batch built");
  if (sample >= c->S) return set_err(c, BRUNO_ERR_ARG, "sample index out of range");
  return BRUNO_OK;
}

bruno_status bruno_sample_count(bruno_ctx *c, size_t *n_samples) {
  if (!c || !n_samples) return BRUNO_ERR_ARG;
  *n_samples = c->stage >= 6 ? c->S : 0;
  return BRUNO_OK;
}

bruno_status bruno_sample_ranges(bruno_ctx *c, uint64_t *ranked0, uint64_t *chains0, uint64_t *chars0) {
  if (!c) return BRUNO_ERR_ARG;
  if (c->S <= 1 || c->stage < 6 || c->h_tally.empty()) return set_err(c, BRUNO_ERR_ARG, "no batch built");
  uint64_t chars = 0;
  for (uint32_t q = 0; q <= c->S; ++q) {
    if (ranked0) ranked0[q] = c->h_rank0[q];
    if (chains0) chains0[q] = c->h_head0[q];
    if (chars0) chars0[q] = chars;
    if (q < c->S) chars += c->h_tally[(size_t)q * T_NUM + T_CHARS];
  }
  return BRUNO_OK;
}

bruno_status bruno_sample_sizes(bruno_ctx *c, size_t sample, bruno_sizes *o) {
  bruno_status st = batch_sample(c, sample);
  if (st != BRUNO_OK) return st;
  if (!o) return BRUNO_ERR_ARG;
  std::memset(o, 0, sizeof(*o));
  const uint64_t *t = &c->h_tally[sample * T_NUM];
  const SGeom &g = c->h_sgeom[sample];
  o->n_reads = c->samp_r0[sample + 1] - c->samp_r0[sample];
  o->n_reads_used = c->h_used[sample];
  o->n_instances = c->h_inst[sample];
  o->n_k2 = t[T_ENTRIES];
  o->n_nodes = t[T_CHAIN] + t[T_BRANCH];
  o->n_branch = t[T_BRANCH];
  o->n_chain_nodes = t[T_CHAIN];
  o->iterations = c->h_iter[sample];
  o->n_cycle_nodes = t[T_CYCLE];
  o->n_isolated = t[T_ISOLATED];
  o->n_ranked = t[T_RANKED];
  o->n_chains = t[T_HEADS];
  o->n_chain_chars = t[T_CHARS];
  o->table_slots = g.g.nslots;
  o->table_partitions = 1ull << g.g.pbits;
  o->launches = c->launches;
  return BRUNO_OK;
}

bruno_status bruno_sample_copy_ranked(bruno_ctx *c, size_t sample, uint64_t *K, uint64_t *rep, int32_t *dist,
                                      size_t cap, size_t *n) {
  bruno_status st = batch_sample(c, sample);
  if (st != BRUNO_OK) return st;
  const uint64_t a = c->h_rank0[sample], cnt = c->h_rank0[sample + 1] - a;
  if (n) *n = cnt;
  if (!K && !rep && !dist) return BRUNO_OK;
  if (cap < cnt) return set_err(c, BRUNO_ERR_CAPACITY, "copy buffer too small");
  const size_t w = 8 * c->W;
  if (K) st = copy_d2h(c, K, (const char *)c->r_K.p + a * w, cnt * w);
  if (st == BRUNO_OK && rep) st = copy_d2h(c, rep, (const char *)c->r_rep.p + a * w, cnt * w);
  if (st == BRUNO_OK && dist) st = copy_d2h(c, dist, (const char *)c->r_dist.p + a * 4, cnt * 4);
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  return st;
}

bruno_status bruno_sample_copy_chains(bruno_ctx *c, size_t sample, uint64_t *reps, uint64_t *offsets, char *chars,
                                      size_t cap_chains, size_t cap_chars, size_t *n_chains, size_t *n_chars) {
  bruno_status st = batch_sample(c, sample);
  if (st != BRUNO_OK) return st;
  const uint64_t h0 = c->h_head0[sample], h1 = c->h_head0[sample + 1], nc = h1 - h0;
  const uint64_t nch = c->h_tally[sample * T_NUM + T_CHARS];
  if (n_chains) *n_chains = nc;
  if (n_chars) *n_chars = nch;
  if (!reps && !offsets && !chars) return BRUNO_OK;
  if ((reps || offsets) && cap_chains < nc) return set_err(c, BRUNO_ERR_CAPACITY, "chain buffer too small");
  if (chars && cap_chars < nch) return set_err(c, BRUNO_ERR_CAPACITY, "char buffer too small");
  uint64_t off0 = 0;
  st = cuda_check(c, cudaMemcpyAsync(&off0, (const uint64_t *)c->head_off.p + h0, 8, cudaMemcpyDeviceToHost, c->stream),
                  "offset");
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamSynchronize(c->stream), "offset");
  const size_t w = 8 * c->W;
  if (st == BRUNO_OK && reps) st = copy_d2h(c, reps, (const char *)c->ch_rep.p + h0 * w, nc * w);
  if (st == BRUNO_OK && offsets) st = copy_d2h(c, offsets, (const uint64_t *)c->head_off.p + h0, (nc + 1) * 8);
  if (st == BRUNO_OK && chars) st = copy_d2h(c, chars, (const char *)c->ch_chars.p + off0, nch);
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  if (st == BRUNO_OK && offsets)
    for (uint64_t i = 0; i <= nc; ++i) offsets[i] -= off0;   /* offsets into this sample's chars */
  return st;
}

bruno_status bruno_sample_copy_nodes(bruno_ctx *c, size_t sample, uint64_t *keys, uint16_t *counts, uint8_t *flags,
                                     size_t cap, size_t *n) {
  bruno_status st = batch_sample(c, sample);
  if (st != BRUNO_OK) return st;
  const uint64_t *t = &c->h_tally[sample * T_NUM];
  return run_copy_nodes_range(c, c->h_sgeom[sample].g.base, c->h_sgeom[sample].g.nslots, t[T_CHAIN] + t[T_BRANCH],
                              keys, counts, flags, cap, n);
}

bruno_status bruno_host_alloc(size_t bytes, void **out) {
  if (!out) return BRUNO_ERR_ARG;
  *out = nullptr;
  cudaError_t e = cudaMallocHost(out, std::max<size_t>(bytes, 1));
  if (e != cudaSuccess) { cudaGetLastError(); return BRUNO_ERR_OOM; }
  return BRUNO_OK;
}

bruno_status bruno_host_free(void *p) {
  if (p && cudaFreeHost(p) != cudaSuccess) { cudaGetLastError(); return BRUNO_ERR_CUDA; }
  return BRUNO_OK;
}

bruno_status bruno_phase_ms(bruno_ctx *c, double *ms, size_t n) {
  if (!c || !ms) return BRUNO_ERR_ARG;
  for (size_t i = 0; i < n && i < 11; ++i) ms[i] = c->phase_ms[i];
  return BRUNO_OK;
}
}  // extern "C"
