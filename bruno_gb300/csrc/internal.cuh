/*
 * internal.cuh -- context state shared by the library's translation units.
 */
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bruno_gb300.h"
#include "kmer.cuh"

namespace bg {

/* device error word bits */
constexpr uint32_t DERR_TABLE_FULL = 1u;
constexpr uint32_t DERR_BAD_INPUT = 2u;
constexpr uint32_t DERR_INVARIANT = 4u;
constexpr uint32_t DERR_UNCLEAN_CHAINS = 8u;

/* Small counters written by kernels, read back by the host between phases. */
struct DevCounters {
  unsigned long long err;
  unsigned long long n_newlines_eff;   /* newlines before the end of the last non-blank line */
  long long last_nonws;                /* index of the last byte that is not \n or \r, -1 if none */
  unsigned long long bad_line;         /* first malformed line, ~0 if none */
  unsigned long long n_records;
  unsigned long long n_instances, n_reads_used, n_slots_claimed, n_entries;
  unsigned long long n_nodes, n_branch, n_chain, n_filtered, n_k2_dump;
  unsigned long long flag_hist[16];
  unsigned long long lr_applied, lr_remaining, lr_cycles, lr_multi;
  unsigned long long n_cycle, n_isolated, n_ranked, n_heads, n_chain_chars;
  unsigned long long n_upper;          /* k-mer positions of all reads long enough */
  unsigned long long n_chain_edges;    /* chain-end records appended */
  unsigned long long n_groups, n_hist; /* general emission: representative groups, histogram bins */
  /* graph cleaning: terminus records, those not on the all-A k-mer, merged summaries, chains
   * with both ends on branches, erase queries, edges found, dead ends, bubble chains, live
   * nodes and live branch nodes after an erasure pass */
  unsigned long long cl_term, cl_nonzero, cl_sum, cl_norm, cl_q, cl_found, cl_dead, cl_bub, cl_live, cl_live_branch;
  unsigned long long n_big, n_big_res; /* entries counted past 2^24 (keys in big_key), resolved */
  unsigned long long n_cand;           /* slots the count listed for the filter */
  unsigned long long quick_hist[16];   /* the filter flags of the entries the count dropped */
  unsigned int hll[1 << 12];           /* HyperLogLog registers, p = 12 */
  /* exact counts of (k-mer, biedge) entries past 2^24 occurrences: an entry word's count stops
   * there and sets E_BIG, and every later occurrence adds 1 here, under the entry word's
   * address (open addressing, key 0 = free); cleared before every counting pass */
  unsigned long long big_key[1024];
  unsigned long long big_cnt[1024];
};
constexpr int BIG_SLOTS = 1024;
/* an entry counted past 2^24, resolved after counting: its table key (continuation mark
 * cleared), its biedge code and its exact count (for the filtered-entry copy-out) */
struct BigRes { uint64_t k0, k1; uint32_t code, pad; unsigned long long count; };

struct Segment { const char *ptr; uint64_t n; int ev = -1; };   /* ev: copy-done event, -1 if none */

/* One sample's share of the k-mer table when the table is cut into shared-memory partitions;
 * a batch of samples (the batched form) gives every sample partitions of its own, and the
 * plain build is a batch of one.  Partition j of sample s is global partition pbase + j: its
 * slots are g.base + j * g.region onwards, its split records rec2_base + j * cap2 onwards. */
struct SGeom {
  TableGeom g;
  uint64_t pbase, rec2_base, cap2;
};
/* per-sample tallies of a batch (u64 each, T_NUM per sample) */
enum {
  T_ENTRIES = 0, T_CHAIN, T_BRANCH, T_CYCLE, T_ISOLATED, T_NMAX, T_RANKED, T_HEADS, T_CHARS, T_NUM
};
/* the largest s with sg[s].pbase <= P (partition -> sample), and likewise for a table slot */
__device__ __forceinline__ uint32_t sample_of_part(const SGeom *sg, uint32_t S, uint64_t P) {
  uint32_t lo = 0, hi = S;
  while (hi - lo > 1) { const uint32_t m = (lo + hi) >> 1; if (sg[m].pbase <= P) lo = m; else hi = m; }
  return lo;
}
__device__ __forceinline__ uint32_t sample_of_slot(const SGeom *sg, uint32_t S, uint64_t slot) {
  uint32_t lo = 0, hi = S;
  while (hi - lo > 1) { const uint32_t m = (lo + hi) >> 1; if (sg[m].g.base <= slot) lo = m; else hi = m; }
  return lo;
}
/* node flags bits 2..15 hold the node's sample in a batch */
constexpr int NF_SAMPLE_SHIFT = 2;
constexpr uint32_t MAX_SAMPLES = 1u << 14;

/* chain state of one chain node, 32 B: pointers encode a chain index (bits 0..31) plus
 * PF_FLIP (the target k-mer, on this node's strand, is the reverse complement of the
 * target's canonical key), PF_EXT (the target is the non-chain in- (PF_EXTOUT clear) or
 * out-neighbour of the chain node in bits 0..31) and PF_BLANK (Kmer(), no neighbour). */
struct ChainState { uint64_t inP, outP; uint32_t inD, outD; uint64_t pad; };
constexpr uint64_t PF_FLIP = 1ull << 32, PF_EXT = 1ull << 33, PF_EXTOUT = 1ull << 34, PF_BLANK = 1ull << 35;
struct Payload { uint64_t P; uint32_t D; uint32_t pad; };

struct Buf {
  void *p = nullptr;
  size_t bytes = 0;
};

struct Ctx {
  bruno_cfg cfg{};
  int W = 1;                     /* key words */
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaMemPool_t pool = nullptr;  /* the library's stream-ordered pool on this device */
  cudaStream_t copy_stream = nullptr;   /* host FASTQ pieces are copied here, one event each */
  cudaStream_t copy_more[3] = {nullptr, nullptr, nullptr};   /* further copy streams (cfg.h2d_streams) */
  cudaEvent_t copy_tail[3] = {nullptr, nullptr, nullptr};    /* their last copy, joined before h2d_end */
  int n_copy = 1;
  std::vector<cudaEvent_t> seg_ev;
  cudaEvent_t h2d_end = nullptr;
  cudaEvent_t order_ev = nullptr; /* orders the copy stream after the context's stream */
  size_t seg_ev_used = 0;
  size_t host_loads = 0;         /* host buffers loaded since the reset (one device buffer each) */
  bool h2d_piped = false;        /* the current graph build's copies ran on the copy stream, ending at h2d_end */
  bool pre_extracted = false;    /* the read index already extracted every segment's reads */
  uint64_t xcap = 0;             /* extraction: bucket capacity, chunk, HLL partial blocks */
  uint32_t xchunk = 1;
  int xblk = 0, xblk_max = 0;
  std::string err;
  int stage = 0;                 /* 0 empty, 1 loaded, 2 counted, 3 filtered, 4 chains, 5 ranked, 6 compressed */

  std::vector<Segment> segs;
  std::vector<Buf> seg_bufs;     /* device copies of host-loaded files */

  DevCounters *dctr = nullptr;   /* device */
  DevCounters *hctr = nullptr;   /* pinned host mirror */

  /* read index */
  Buf rstart, rend, tile_cnt, tile_base;   /* read spans as device byte addresses */
  uint64_t n_reads = 0, n_reads_used = 0, n_instances = 0;

  /* k-mer table */
  Buf table;
  TableGeom geom{0, 0, 0, 0};
  uint64_t nslots = 0, n_entries = 0, n_slots_claimed = 0;
  Buf records, bucket_cnt;       /* partitioned counting: 8-byte records per hash bucket */
  Buf xsamp, hllreg, hsum;       /* the extraction's bucket layout, HyperLogLog registers, their sums */
  /* batched form: S samples, one after another in the FASTQ; per sample its byte offset in the
   * device copy (S + 1 values), first read (S + 1), table geometry and tallies */
  uint32_t S = 1;
  std::vector<uint64_t> samp_off, samp_r0;
  /* a batch copied from the host in groups of whole samples: segment i holds samples
   * [seg_samp[i], seg_samp[i + 1]), and the read index extracts each group as it lands */
  bool batch_piped = false;
  std::vector<uint32_t> seg_samp;
  std::vector<uint64_t> x_cap, x_base;     /* per sample: bucket capacity, first record */
  Buf fr_tmp;                              /* first-read lookups of a group of samples */
  std::vector<SGeom> h_sgeom;
  Buf sgeom, s_tally, s_inst, s_used, xitems, split_items, csample, r_samp, h_samp, grp_tmp;
  std::vector<uint64_t> h_tally;           /* T_NUM per sample, after the build */
  std::vector<uint64_t> h_inst, h_used;    /* instances and reads used per sample */
  std::vector<uint64_t> h_rank0, h_head0;  /* first listranked node / chain of each sample (S + 1) */
  std::vector<uint64_t> h_iter;            /* ranking rounds per sample */
  Buf records2, sub_cnt;         /* the same records split per table partition */
  bool h2d_pending = false;      /* ev[7] marks the start of the current graph build's host-to-device copies */
  int force_direct_count = 0;    /* cfg.direct_count: 0 automatic, 1 whole table, 2 L2 partitions */
  Buf chain_list, branch_list;   /* slot indices, filled by the filter */
  Buf scan_tmp;                  /* block offsets of the multi-block scan */
  Buf bigres;                    /* BigRes per entry counted past 2^24 (n_big of them) */
  uint64_t n_big = 0;
  /* thresholded counts in shared memory list the first slots of the k-mers the filter's quick
   * rule cannot drop, and tally the flags of those it drops; the filter then reads the list */
  Buf cand;
  bool have_cand = false;
  uint64_t n_cand = 0, quick_hist[16] = {0};
  Buf k1tab;                     /* the (k+1)-mer edge filter's (key, count) table */
  uint64_t k1slots = 0;

  /* dumps */
  Buf k2_keys, k2_edges, k2_counts;
  uint64_t n_k2 = 0;
  Buf f_keys, f_edges, f_counts;
  uint64_t n_filtered = 0;
  bool k2_dumped = false;

  /* nodes */
  uint64_t n_nodes = 0, n_branch = 0, n_chain = 0;
  uint64_t filter_read = 0;      /* slots the filter read */
  uint64_t flag_hist[16] = {0};
  Buf blk_cnt, blk_base;

  /* chains */
  Buf ckey, cedge, cstate, cstate2, pend, pay, unf0, unf1, removed;
  uint64_t iterations = 0, n_cycle = 0, n_isolated = 0, multi = 0;
  bool exact_ranking = false;    /* force the round-synchronous ranking (tests) */
  bool fast_ranked = false;      /* the last ranking took the O(M) path (a batch needs it) */

  /* emission */
  Buf r_K, r_rep, r_dist, rep_idx, head_of, heads, head_len, head_off, ch_rep, ch_off, ch_chars;
  uint64_t n_ranked = 0, n_heads = 0, n_chain_chars = 0;
  bool chains_clean = true;
  bool general_emission = false; /* the compaction grouped by representative (inconsistent map) */
  Buf e_ends, e_freqs;           /* chain-end records (L, R; 11 counts each), built on demand */
  uint64_t n_chain_edges = 0;
  bool chain_edges_done = false;
  Buf s_kmers, s_dist, s_flags;  /* chain summaries, built on demand */
  uint64_t n_summaries = 0;
  bool summaries_done = false;
  /* graph cleaning: terminus records and their index per chain node, merged summaries,
   * chains between two branches, the bubble grouping table, erase queries, edges found */
  Buf cl_trec, cl_tslot, cl_sums, cl_norm, cl_htab, cl_q, cl_found;
  bool cleaned = false;
  uint64_t thr_used[6] = {0, 0, 0, 0, 0, 0};   /* the thresholds local_insert_by_freqencies used */

  cudaEvent_t ev[8] = {nullptr};
  cudaEvent_t kev[5] = {nullptr};  /* counting sub-steps */
  double phase_ms[11] = {0};       /* 6 phases, then estimate/extract, table init, count, split,
                                      and the host-to-device copies of the FASTQ input */
  uint64_t launches = 0;           /* kernels launched since the last reset */
};

/* --------------------------------------------------------------- host helpers */
bruno_status set_err(Ctx *c, bruno_status s, const std::string &msg);
bruno_status cuda_check(Ctx *c, cudaError_t e, const char *what);
bruno_status ensure(Ctx *c, Buf &b, size_t bytes, bool preserve = false);
cudaMemPool_t library_pool(int device);
bruno_status sync_counters(Ctx *c, bool with_hll = false);

/* exclusive scan of n uint64 values (in may equal out); writes the total to *total_dev (may be
 * NULL).  scratch: 1024 device words for the block offsets (NULL: one block does it all).
 * Returns the number of kernels launched. */
int scan_u64(const uint64_t *in, uint64_t *out, uint64_t n, unsigned long long *total_dev, cudaStream_t s,
             uint64_t *scratch);
/* the same on the context's stream with the context's scratch; counts its launches */
bruno_status scan_ctx(Ctx *c, const uint64_t *in, uint64_t *out, uint64_t n, unsigned long long *total_dev);

/* -------------------------------------------------------------- phase launchers */
bruno_status run_index_reads(Ctx *c);        /* FASTQ line structure -> read spans */
bruno_status run_count(Ctx *c);              /* distinct-count estimate, table, counting */
bruno_status run_count_samples(Ctx *c);      /* the same for a batch of c->S samples (read index included) */
bruno_status run_dump_k2(Ctx *c);            /* optional raw (k+2)-mer copy */
bruno_status run_filter(Ctx *c, const uint64_t *thresh);
bruno_status run_extract_chains(Ctx *c);
bruno_status run_list_rank(Ctx *c, int min_update);
bruno_status run_compress(Ctx *c);
bruno_status run_chain_edges(Ctx *c);
bruno_status run_chain_summaries(Ctx *c);
/* clean_deadend_and_bubbles_naive on the ranked chain map and the node table; leaves the
 * cleaned graph compacted (as run_compress does) */
bruno_status run_clean(Ctx *c, uint64_t *rounds, uint64_t *deadends, uint64_t *bubbles, uint64_t *edges,
                       int32_t *status);
bruno_status run_copy_nodes(Ctx *c, uint64_t *keys, uint16_t *counts, uint8_t *flags, size_t cap, size_t *n);
/* the nodes of table slots [base, base + nslots), of which there are nn */
bruno_status run_copy_nodes_range(Ctx *c, uint64_t base, uint64_t nslots, uint64_t nn, uint64_t *keys, uint16_t *counts,
                                  uint8_t *flags, size_t cap, size_t *n);
/* debruijn_graph::find_if / erase_if over the node table (filter: a bruno_node_filter); after an
 * erasure the node counts and stored classifications are brought up to date */
bruno_status run_node_query(Ctx *c, int filter, bool erase, uint64_t *keys, uint16_t *counts, uint8_t *flags,
                            size_t cap, size_t *n);
/* check_index (compact_dbg_stats.hpp:45-119) and the edge-count histogram over the node table */
bruno_status run_check_index(Ctx *c, bruno_index_check *out);
/* debruijn_graph_map::erase_nodes: host k-mers (either strand), with the edges back to them */
bruno_status run_erase_nodes(Ctx *c, const uint64_t *kmers, size_t n);
/* chain-map records of the nodes whose removed[] mark is `which` (0 chain map, 1 cycle, 2 isolated)
 * matching a bruno_chain_filter */
bruno_status run_chain_query(Ctx *c, int filter, int which, uint64_t *kmers, uint64_t *inK, uint64_t *outK,
                             uint32_t *inD, uint32_t *outD, size_t cap, size_t *n);

}  // namespace bg
