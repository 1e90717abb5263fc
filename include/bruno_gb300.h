/*
 * bruno_gb300.h -- C ABI of the GB300 de Bruijn graph-construction library.
 *
 * One context builds one graph on one GPU: FASTQ bytes -> canonical (k-mer, biedge) pairs
 * -> (k+2)-mer edge-frequency counts -> frequency filter -> graph nodes with 9 uint16 edge
 * counters -> chain nodes -> list ranking -> compacted chains.  Every entry point replaces
 * one step of ParBLiSS/bruno's src/debruijn API (cited beside it) and computes the same
 * result bit for bit; the reference's MPI distribution disappears because all tables live
 * in one device's memory.
 *
 * Conventions
 *  - Plain C types only.  A CUDA stream is passed as `void *` (a cudaStream_t).
 *  - k-mers are 2-bit packed (A0 C1 G2 T3), first base in the most significant bits.
 *    Arrays of k-mers hold `words` uint64 per k-mer: 1 for k <= 31, 2 for k >= 32 (low word
 *    first).  A biedge byte holds the DNA16 code (A1 C2 G4 T8, 0 = none) of the base before
 *    the k-mer in its high nibble and of the base after it in its low nibble.
 *  - Every call returns a bruno_status; the context keeps a message for the last failure
 *    (bruno_last_error).  Kernels never trap: device-side failures (table full, malformed
 *    input, ranking that does not converge) set a status word that the host reads.
 *  - The context owns all device memory it allocates.  Copy-out calls use the size-query
 *    pattern: pass dst == NULL to learn the element count, then pass buffers of that size.
 *  - Calls on one context are stream-ordered on the context's stream and are not
 *    thread-safe; use one context per host thread.
 */
#ifndef BRUNO_GB300_H_
#define BRUNO_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bruno_status {
  BRUNO_OK = 0,
  BRUNO_ERR_ARG = 1,              /* invalid argument or call order */
  BRUNO_ERR_BAD_INPUT = 2,        /* malformed FASTQ */
  BRUNO_ERR_OOM = 3,              /* device allocation failed */
  BRUNO_ERR_TABLE_FULL = 4,       /* hash table probe limit hit even after regrowth */
  BRUNO_ERR_RANK_NOT_CONVERGED = 5,/* not returned: the round-synchronous ranking stops at the
                                     reference's 30-round cap without an error, as the reference
                                     does (debruijn_chain_graph.hpp:923-926, 1249-1252); sizes.iterations
                                     = 30 shows it */
  BRUNO_ERR_INVARIANT = 6,        /* an internal invariant failed (reported, never trapped) */
  BRUNO_ERR_CUDA = 7,             /* a CUDA runtime call failed */
  BRUNO_ERR_CAPACITY = 8          /* caller buffer too small */
} bruno_status;

typedef struct bruno_cfg {
  int32_t k;                /* k-mer length, 3..63 (compile-time pK of the reference driver) */
  int32_t thresholding;     /* -T: 1 = build_index_thresholded, 0 = build_index */
  uint64_t thresh[6];       /* k_lo, k_hi, k1_lo, k1_hi, k2_lo, k2_hi; lower bounds inclusive,
                               upper bounds exclusive (debruijn_graph_map.hpp:1261) */
  int32_t min_update;       /* -R: 1 = list_rank_min_update, 0 = list_rank */
  int32_t device;           /* CUDA device ordinal */
  uint64_t table_slots;     /* 0 = size the k-mer table from a distinct-count estimate */
  double max_load;          /* target table load when sizing (0 = 0.5) */
  int32_t keep_k2;          /* 1: keep enough state to copy out the raw (k+2)-mer counts */
  int32_t keep_filtered;    /* 1: record the filtered (k+2)-mer entries for copy-out */
  int32_t exact_ranking;    /* 1: always run the round-synchronous ranking; 0: use the O(M)
                               ruling-set ranking whenever the chain map is consistent */
  int32_t direct_count;     /* counting path: 0 = automatic (hash-partitioned records counted
                               partition by partition in one CTA's shared memory; a skewed input
                               that overflows a partition falls back to L2-resident partitions at
                               k <= 31 and to the whole-table count at k > 31), 1 = every
                               instance straight into the whole table, 2 = the L2 partitions
                               always (k <= 31; k > 31 then counts into the whole table). */
  int32_t edge_filter;      /* with thresholding: 1 = the blocked driver's build_index_thresholded
                               (test/test/compact_debruijn_graph_block_construct.cpp:417-470):
                               canonical (k+1)-mers counted (saturating uint16) and kept in
                               [thresh[2], thresh[3]), biedge edges whose (k+1)-mer is gone
                               cleared, pairs left without edges dropped, the rest inserted
                               unthresholded; not with direct_count = 1.  0 = the
                               (k+2)-mer count filter (local_insert_by_freqencies). */
  uint64_t h2d_chunk;       /* FASTQ from host memory is copied in pieces of about this many bytes,
                               cut at record starts, and each piece is parsed (and on the k <= 31
                               counting path its k-mers extracted) as soon as it lands, while the
                               rest is still copying; inputs under two pieces are copied whole.
                               0 = 256 MiB. */
  int32_t h2d_streams;      /* copy streams the pieces are spread over, round robin (1..4; 0 = 1) */
  int32_t rank_fill;        /* the O(M) ranking's final states: 0 = a second walk of every segment
                               between rulers; 1 = the first walk records each node's place on its
                               segment and one pass over the nodes sets the final states */
  int32_t part_slots;       /* counting in shared memory: the most 32-byte slots of one table
                               partition, which also bounds every probe run (256..3072; 0 = 3072;
                               k > 31 partitions hold half as many 64-byte slots) */
  int32_t count_threads;    /* threads of a k <= 31 partition's counting block at most (256, 512 or
                               1024; 0 = 512; blocks of small partitions take fewer, at least 128) */
} bruno_cfg;

typedef struct bruno_sizes {
  uint64_t n_reads;         /* FASTQ records */
  uint64_t n_reads_used;    /* records that produced k-mers (no N, length >= k+2) */
  uint64_t n_instances;     /* (k-mer, biedge) pairs */
  uint64_t n_k2;            /* distinct canonical (k-mer, biedge) entries */
  uint64_t n_filtered;      /* entries kept by the filter */
  uint64_t n_nodes;         /* graph nodes */
  uint64_t n_branch;        /* IsBranchPoint nodes */
  uint64_t n_chain_nodes;   /* IsChainNode nodes */
  uint64_t iterations;      /* list-ranking rounds */
  uint64_t n_cycle_nodes;   /* removed as cycles */
  uint64_t n_isolated;      /* removed as isolated */
  uint64_t n_ranked;        /* listranked chain nodes */
  uint64_t n_chains;        /* compacted chains */
  uint64_t n_chain_chars;   /* total bases over all compacted chains */
  uint64_t table_slots;     /* k-mer table slots in use */
  uint64_t collisions;      /* list-ranking sides that got >1 update in one round */
  uint64_t filter_flag_hist[16]; /* k_del[] histogram (debruijn_graph_map.hpp:1568) */
  uint64_t launches;        /* kernels launched by the last build */
  uint64_t table_partitions; /* slot regions the k-mer table was filled in (1 = one region) */
  uint64_t grouped_chains;  /* 1: the chain pointers were not mutually consistent (separate k and
                               k+2 bounds can trim an edge on one side only) and the compaction
                               grouped the nodes by representative */
  uint64_t filter_slots_read; /* table slots local_insert_by_freqencies read: every slot, or only those
                                 the count listed (thresholded builds) */
} bruno_sizes;

typedef struct bruno_ctx bruno_ctx;

/* Context lifetime.  Replaces constructing debruijn_graph / debruijn_chain_graph
 * (debruijn_graph.hpp:45-60, debruijn_chain_graph.hpp:162-168) on an MPI communicator. */
bruno_status bruno_ctx_create(const bruno_cfg *cfg, bruno_ctx **out);
bruno_status bruno_ctx_destroy(bruno_ctx *ctx);
/* Runs all later calls on `stream` (a cudaStream_t; NULL = the context's own stream). */
bruno_status bruno_set_stream(bruno_ctx *ctx, void *stream);
const char *bruno_last_error(const bruno_ctx *ctx);
/* Drops all graph state so the context can build another graph (keeps allocations). */
bruno_status bruno_reset(bruno_ctx *ctx);

/* Adds one FASTQ file's bytes.  Replaces partitioned_file::read_file + parse_file_data
 * (compact_dbg_io.hpp:165-195, compact_dbg_freq_construct_clean.cpp:321-323).  If
 * is_device != 0, `buf` is a device pointer that must stay valid until
 * bruno_compute_biedge_freqencies returns; otherwise the bytes are copied to the device,
 * asynchronously (in cfg.h2d_chunk pieces on the context's copy stream when the buffer holds
 * at least two), so the host buffer too must stay valid until that call returns. */
bruno_status bruno_load_fastq(bruno_ctx *ctx, const char *buf, size_t nbytes, int32_t is_device);

/* Parses every loaded file into canonical (k-mer, biedge) pairs and counts each distinct
 * pair.  Replaces debruijn_kmer_simple_biedge_parser (debruijn_biedge_loader.hpp:393-623)
 * followed by debruijn_graph_map::compute_biedge_freqencies (debruijn_graph_map.hpp:1085). */
bruno_status bruno_compute_biedge_freqencies(bruno_ctx *ctx);

/* Frequency filter and node insertion.  Replaces
 * debruijn_graph_map::local_insert_by_freqencies(k2_counter, threshes)
 * (debruijn_graph_map.hpp:1258-1623); thresh == NULL uses cfg.thresh.  With
 * cfg.thresholding == 0 it is the unthresholded build_index insert
 * (compact_dbg_build.hpp:34-62).  Also classifies every node (IsBranchPoint / IsChainNode,
 * debruijn_graph_filters.hpp:142-220). */
bruno_status bruno_local_insert_by_freqencies(bruno_ctx *ctx, const uint64_t *thresh);

/* Builds the chain map and marks termini next to branch points.  Replaces
 * debruijn_chain_graph::extract_chains (debruijn_chain_graph.hpp:604-667). */
bruno_status bruno_extract_chains(bruno_ctx *ctx);

/* List ranking.  min_update != 0 replaces list_rank_min_update (debruijn_chain_graph.hpp:
 * 1040-1310), otherwise list_rank (:793-994); both end with separate_cycles and
 * separate_isolated.  *iterations receives the round count the reference returns. */
bruno_status bruno_list_rank(bruno_ctx *ctx, int32_t min_update, uint64_t *iterations);

/* Listranked chain nodes and compacted chain sequences on the device.  Replaces
 * to_ranked_chain_nodes (debruijn_chain_graph.hpp:1760-1773) and to_compressed_chains
 * (:1778-1856). */
bruno_status bruno_to_compressed_chains(bruno_ctx *ctx);

/* Graph cleaning of the reference driver's _freq_clean build (the _freq build defines
 * NCLEAN): clean_deadend_and_bubbles_naive (test/common/compact_dbg_clean.hpp:575-890) after
 * the first compaction (compact_dbg_freq_construct_clean.cpp:633-700).  Cycle nodes and then
 * edge-less nodes leave the graph; then, until none is found, chains shorter than 2k-1 with
 * exactly one end on a branch (dead ends, find_deadends, debruijn_topo_operations.hpp:146-175)
 * and runs of chains between the same two branches with lengths within one (bubbles,
 * find_bubbles, :285-395) lose their end edges of frequency at most thresh[2] (the thresholds
 * local_insert_by_freqencies used) on both nodes, edge-less nodes go, and the graph is
 * compacted again.  Needs ranked chains (the first compaction's outputs are to be copied out
 * before); leaves the cleaned graph compacted, so that every copy call returns the cleaned
 * graph.  BRUNO_ERR_INVARIANT with stats->status = 2 when the chain pointers are not mutually
 * consistent; stats->status = 1 when an iteration erased nothing (the reference would repeat it
 * forever), 0 otherwise.  stats may be NULL. */
typedef struct bruno_clean_stats {
  uint64_t rounds;          /* iterations of the cleaning loop */
  uint64_t deadends;        /* dead-end chains found, over all iterations */
  uint64_t bubbles;         /* bubble chains found, over all iterations */
  uint64_t edges;           /* low-frequency end edges erased (with their reverse edges) */
  int32_t status;
  int32_t reserved;
} bruno_clean_stats;
bruno_status bruno_clean_deadend_and_bubbles_naive(bruno_ctx *ctx, bruno_clean_stats *stats);

/* The whole plain path in one call: load (host or device bytes), count, filter, extract,
 * rank, compress.  Equivalent to the reference driver's build_index_thresholded ->
 * extract_chains -> list_rank[_min_update] -> to_ranked_chain_nodes sequence
 * (compact_dbg_freq_construct_clean.cpp:491-737). */
bruno_status bruno_build_and_compact(bruno_ctx *ctx, const char *buf, size_t nbytes, int32_t is_device);

bruno_status bruno_get_sizes(bruno_ctx *ctx, bruno_sizes *out);

/* Copy-outs to host memory (device order, not sorted).  `n` receives the element count;
 * dst pointers may be NULL to query it. */
/* Raw (k+2)-mer counts: LocalK2CountMapType::to_vector (debruijn_graph_map.hpp:1268).
 * Needs cfg.keep_k2 and must be called before bruno_local_insert_by_freqencies. */
bruno_status bruno_copy_k2(bruno_ctx *ctx, uint64_t *keys, uint8_t *edges, uint32_t *counts,
                           size_t cap, size_t *n);
/* Filtered entries (k2counts after :1594).  Needs cfg.keep_filtered. */
bruno_status bruno_copy_filtered(bruno_ctx *ctx, uint64_t *keys, uint8_t *edges, uint32_t *counts,
                                 size_t cap, size_t *n);
/* Graph nodes: k-mer and counts[9] = out A C G T, in A C G T, self (debruijn_graph_node.hpp:157);
 * flags bit 0 = IsBranchPoint, bit 1 = IsChainNode. */
bruno_status bruno_copy_nodes(bruno_ctx *ctx, uint64_t *keys, uint16_t *counts, uint8_t *flags,
                              size_t cap, size_t *n);
/* listranked_chain_node<K> = (K on the representative's strand, representative, distance)
 * (debruijn_chain_node.hpp:155-156). */
bruno_status bruno_copy_ranked(bruno_ctx *ctx, uint64_t *K, uint64_t *rep, int32_t *dist,
                               size_t cap, size_t *n);
/* Compacted chains: representative k-mer per chain, offsets[n_chains + 1] into `chars`. */
bruno_status bruno_copy_chains(bruno_ctx *ctx, uint64_t *reps, uint64_t *offsets, char *chars,
                               size_t cap_chains, size_t cap_chars, size_t *n_chains, size_t *n_chars);
/* Chain end edges and frequency summaries, the records print_chain_frequencies
 * (test/common/compact_dbg_stats.hpp:879-1065) prints to <prefix>.chain.edges, with the
 * summaries of compute_freq_map (:783-816).  One record per chain-map node that
 * IsCanonicalTerminusOrIsolated (src/debruijn/debruijn_chain_filters.hpp:125-147) accepts:
 * ends[2 * words] = L then R, the chain's two ends on one strand; freqs[11] = L's in-edge
 * counts A C G T, R's out-edge counts A C G T, then the mean (float sum / float count,
 * truncated), min and max of the self frequencies of the chain's nodes.  Records come in no
 * particular order (the reference sorts them by L before printing).  Computed on the device at
 * the first call after bruno_to_compressed_chains, which may pass NULL buffers to query n. */
/* Device addresses of the results, for a consumer on the same device that reads them in place
 * (zero copy): the listranked nodes as bruno_copy_ranked gives them and the compacted chains as
 * bruno_copy_chains gives them.  Read-only; valid until the next call that rebuilds or changes
 * the context (bruno_reset, a load, a build, the cleaning, bruno_ctx_destroy).  Read them on the
 * context's stream or after it has been synchronised (this call synchronises it). */
typedef struct bruno_device_view {
  const uint64_t *ranked_K;       /* n_ranked k-mers (words each) */
  const uint64_t *ranked_rep;     /* n_ranked representatives (words each) */
  const int32_t *ranked_dist;     /* n_ranked distances */
  const uint64_t *chain_reps;     /* n_chains representatives (words each) */
  const uint64_t *chain_offsets;  /* n_chains + 1 offsets into chain_chars */
  const char *chain_chars;        /* n_chain_chars bases */
  uint64_t n_ranked, n_chains, n_chain_chars;
  int32_t words;
  int32_t reserved;
} bruno_device_view;
bruno_status bruno_device_results(bruno_ctx *ctx, bruno_device_view *out);

bruno_status bruno_copy_chain_edges(bruno_ctx *ctx, uint64_t *ends, uint16_t *freqs, size_t cap, size_t *n);
/* Chain summaries: debruijn_chain_graph::to_summarized_chains()
 * (src/debruijn/debruijn_chain_graph.hpp:1876-2005), the records print_chain_summaries
 * (test/common/compact_dbg_io.hpp:528-556) prints to <prefix>.chain.summary.  One per chain:
 * kmers[4 * words] = the 5' terminus's outer neighbour, the 5' terminus (the chain's
 * representative), the 3' terminus, the 3' terminus's outer neighbour, all on the
 * representative's strand (a missing neighbour is the all-A k-mer); dist = distance between the
 * termini; flags[2] = 1 where the 5' / 3' end points to a branch node, 0 where it has no
 * neighbour.  Records come in no particular order (the reference's are sorted by the
 * representative).  BRUNO_ERR_INVARIANT when the chain pointers are not mutually consistent
 * (the compaction had to group by representative): the reference's pairing of termini then
 * depends on its sort order.  Computed at the first call after bruno_to_compressed_chains. */
bruno_status bruno_copy_chain_summaries(bruno_ctx *ctx, uint64_t *kmers, uint32_t *dist, uint8_t *flags, size_t cap,
                                        size_t *n);

/* ---------------------------------------------------------------------------------------
 * Graph and chain-map queries between the phases, as the reference driver makes them
 * (compact_dbg_freq_construct_clean.cpp:599-610, 794-807).  Predicates are tag values. */

/* Node predicates of bliss::debruijn::filter::graph (src/debruijn/debruijn_graph_filters.hpp),
 * evaluated on a node's canonical k-mer and its current edge counts. */
typedef enum bruno_node_filter {
  BRUNO_NODES_ALL = 0,              /* every node */
  BRUNO_IS_K_PALINDROME = 1,        /* IsKPalindrome (:38-55) */
  BRUNO_IS_KPLUS1_PALINDROME = 2,   /* IsKplus1Palindrome (:57-140) */
  BRUNO_IS_BRANCH_POINT = 3,        /* IsBranchPoint (:142-160) */
  BRUNO_IS_ISOLATED_NODE = 4,       /* IsIsolated (:163-172): no in and no out edge */
  BRUNO_IS_CHAIN_INTERNAL_NODE = 5, /* IsChainInternalNode (:189-203) */
  BRUNO_IS_CHAIN_NODE = 6           /* IsChainNode (:206-220) */
} bruno_node_filter;

/* debruijn_graph::find_if(pred) (debruijn_graph.hpp:193-196): the matching nodes, in the format of
 * bruno_copy_nodes (flags evaluated on the current counts).  Size-query pattern.  After
 * bruno_local_insert_by_freqencies. */
bruno_status bruno_graph_find_if(bruno_ctx *ctx, int32_t filter, uint64_t *keys, uint16_t *counts, uint8_t *flags,
                                 size_t cap, size_t *n);
/* debruijn_graph::erase_if(pred) (:247-250): the matching nodes leave the graph (their neighbours'
 * edges stay, as the reference's plain erase leaves them).  *n_erased may be NULL. */
bruno_status bruno_graph_erase_if(bruno_ctx *ctx, int32_t filter, size_t *n_erased);
/* debruijn_graph_map::erase_nodes(query) (debruijn_graph_map.hpp:833-836): each k-mer of the host
 * array (n of them, either strand, `words` uint64 each) that is a node leaves the graph, and its
 * neighbours lose their edges to it (erase_nodes_and_edges, :811-827). */
bruno_status bruno_graph_erase_nodes(bruno_ctx *ctx, const uint64_t *kmers, size_t n);

/* The reference driver's debug check of the graph, check_index (test/common/compact_dbg_stats.hpp:
 * 45-119): every neighbour k-mer that a node's edges name must be a node (n_absent = 0), and every
 * node with an edge must be named as a neighbour by some node (n_unreferenced = 0).  Also reported:
 * edges whose neighbour node lacks the edge back (n_unanswered), and the in-edge count x out-edge
 * count histogram of print_edge_histogram (compact_dbg_stats.hpp:121-135, debruijn_stats.hpp:
 * 39-74), edge_hist[in * 5 + out].  Returns BRUNO_ERR_INVARIANT, with *out filled, when either of
 * the reference's two checks fails (where the reference's debug build asserts).  After
 * bruno_local_insert_by_freqencies. */
typedef struct bruno_index_check {
  uint64_t n_query;         /* neighbour k-mers named: one per edge of every node */
  uint64_t n_absent;        /* of them, k-mers that are not nodes */
  uint64_t n_unreferenced;  /* nodes with an edge that no node names */
  uint64_t n_unanswered;    /* edges whose neighbour node has no edge back */
  uint64_t edge_hist[25];
} bruno_index_check;
bruno_status bruno_check_index(bruno_ctx *ctx, bruno_index_check *out);

/* Chain-map predicates of bliss::debruijn::filter::chain (src/debruijn/debruijn_chain_filters.hpp),
 * evaluated on a chain-map record (k-mer, in k-mer, out k-mer, in distance, out distance). */
typedef enum bruno_chain_filter {
  BRUNO_CHAIN_ALL = 0,                              /* every record */
  BRUNO_CHAIN_IS_UNIT_LENGTH = 1,                   /* IsUnitLength (:37-46) */
  BRUNO_CHAIN_IS_ISOLATED = 2,                      /* IsIsolated (:49-58) */
  BRUNO_CHAIN_IS_TERMINUS = 3,                      /* IsTerminus (:60-69) */
  BRUNO_CHAIN_IS_INTERNAL = 4,                      /* IsInternal (:71-82) */
  BRUNO_CHAIN_IS_TERMINUS_OR_ISOLATED = 5,          /* IsTerminusOrIsolated (:84-97) */
  BRUNO_CHAIN_IS_CANONICAL_TERMINUS = 6,            /* IsCanonicalTerminus (:100-122) */
  BRUNO_CHAIN_IS_CANONICAL_TERMINUS_OR_ISOLATED = 7,/* IsCanonicalTerminusOrIsolated (:125-147) */
  BRUNO_CHAIN_POINTS_TO_TERMINI = 8,                /* PointsToTermini (:153-165) */
  BRUNO_CHAIN_POINTS_TO_INTERNAL_NODE = 9           /* PointsToInternalNode (:169-186) */
} bruno_chain_filter;

/* debruijn_chain_graph::find_if(pred) (debruijn_chain_graph.hpp:306-311): the chain-map records
 * simple_biedge<K> = (inK, outK, inDist, outDist) (debruijn_chain_node.hpp:49-50) of the matching
 * nodes, keyed by the canonical k-mer; inK / outK are on the key's strand, the all-A k-mer where
 * the node has no neighbour; distances carry the terminal mark in their top bit.  After
 * bruno_extract_chains (the records before ranking) or after bruno_list_rank (the ranked
 * records; cycle and isolated nodes have left the chain map by then).  Size-query pattern; any
 * output may be NULL. */
bruno_status bruno_chain_find_if(bruno_ctx *ctx, int32_t filter, uint64_t *kmers, uint64_t *in_kmers,
                                 uint64_t *out_kmers, uint32_t *in_dist, uint32_t *out_dist, size_t cap, size_t *n);
/* get_cycle_node_kmers (debruijn_chain_graph.hpp:448-460): the k-mers separate_cycles took out of
 * the chain map in the last ranking.  Size-query pattern. */
bruno_status bruno_get_cycle_node_kmers(bruno_ctx *ctx, uint64_t *kmers, size_t cap, size_t *n);
/* get_isolated (:462-468): the chain-map records separate_isolated took out, as bruno_chain_find_if
 * gives records.  Size-query pattern. */
bruno_status bruno_get_isolated(bruno_ctx *ctx, uint64_t *kmers, uint64_t *in_kmers, uint64_t *out_kmers,
                                uint32_t *in_dist, uint32_t *out_dist, size_t cap, size_t *n);

/* Page-locked host memory, for fast host<->device copies of FASTQ input and results. */
bruno_status bruno_host_alloc(size_t bytes, void **out);
bruno_status bruno_host_free(void *p);

/* Device times of the last build, milliseconds, from CUDA events on the context's stream:
 * ms[0..5] = phases parse, count_k2mers, filter_insert, chainmap, list_rank, compress;
 * ms[6..9] = counting sub-steps: distinct-count estimate (with the record extraction on
 * the partitioned path), whole-table initialisation (direct path only), the counting
 * itself (split + per-partition counts, the L2 partition inserts, or k_count), and the
 * record split alone (shared-memory partition path only); ms[10] = the host-to-device
 * copies of FASTQ bytes given in host memory.  Writes min(n, 11) values. */
bruno_status bruno_phase_ms(bruno_ctx *ctx, double *ms, size_t n);

/* ---------------------------------------------------------------------------------------
 * Batched form: many samples built in one pass.  No counterpart in the reference (one graph per
 * MPI job there).  The n_samples FASTQ buffers (host memory, or device memory with is_device)
 * are copied one after another into one device buffer, and every kernel of the path runs once
 * over all of them: each sample counts into hash-table partitions of its own (sized from its own
 * distinct-count estimate), is filtered, chained and ranked, so that each sample's graph, chains
 * and counts are exactly what bruno_build_and_compact gives for that sample alone.  The whole
 * path of one sample is the reference driver's build_index_thresholded -> extract_chains ->
 * list_rank[_min_update] -> to_ranked_chain_nodes (compact_dbg_freq_construct_clean.cpp:
 * 295-348, 549-737).  Needs k <= 31, no edge filter, no raw or filtered count copies, and
 * thresholds on the (k+1)-mer counts only (one -L / -U value: the chain maps are then mutually
 * consistent); at most 16384 samples.  The results stay in the context, grouped by sample, until
 * the next build or reset; bruno_copy_ranked / bruno_copy_chains return all samples' results
 * (sample after sample), the calls below one sample's. */
bruno_status bruno_build_samples(bruno_ctx *ctx, const char *const *bufs, const size_t *nbytes, size_t n_samples,
                                 int32_t is_device);
/* Samples of the last batch (0 if none was built). */
bruno_status bruno_sample_count(bruno_ctx *ctx, size_t *n_samples);
/* Where each sample's results start in what bruno_copy_ranked / bruno_copy_chains return for the
 * whole batch (each array n_samples + 1 long, may be NULL): listranked nodes, chains, and chain
 * characters, so that one copy of everything serves every sample. */
bruno_status bruno_sample_ranges(bruno_ctx *ctx, uint64_t *ranked0, uint64_t *chains0, uint64_t *chars0);
/* One sample's sizes, as bruno_get_sizes gives them for a plain build of the sample alone
 * (n_filtered and filter_flag_hist are not kept per sample and read 0). */
bruno_status bruno_sample_sizes(bruno_ctx *ctx, size_t sample, bruno_sizes *out);
/* One sample's listranked nodes, compacted chains (offsets into the sample's own chars) and graph
 * nodes, in the formats of bruno_copy_ranked / bruno_copy_chains / bruno_copy_nodes. */
bruno_status bruno_sample_copy_ranked(bruno_ctx *ctx, size_t sample, uint64_t *K, uint64_t *rep, int32_t *dist,
                                      size_t cap, size_t *n);
bruno_status bruno_sample_copy_chains(bruno_ctx *ctx, size_t sample, uint64_t *reps, uint64_t *offsets, char *chars,
                                      size_t cap_chains, size_t cap_chars, size_t *n_chains, size_t *n_chars);
bruno_status bruno_sample_copy_nodes(bruno_ctx *ctx, size_t sample, uint64_t *keys, uint16_t *counts, uint8_t *flags,
                                     size_t cap, size_t *n);

/* ---------------------------------------------------------------------------------------
 * Many builds at once.  No counterpart in the reference (one graph per MPI job there): a pool
 * of `workers` host threads, each with its own context and stream, runs
 * bruno_build_and_compact for submitted FASTQ buffers, so several small graphs share the GPU.
 * Each result is exactly what the plain path gives for that input alone.  Batched use:
 * submit every sample, then wait for each.  Served use: submit requests as they arrive; a
 * request starts when a worker is free and its device-memory estimate (20 B per FASTQ byte +
 * 64 MiB) fits `mem_budget` bytes (0 = 80% of the device memory free at creation) together with
 * what the other workers hold; a request larger than the budget runs once no other is busy, and
 * one that runs out of device memory beside others is retried once on its own.
 * Buffers are host memory (pinned for fast copies) and must stay valid until the request's
 * bruno_pool_wait returns.  The pool's functions may be called from several host threads. */
typedef struct bruno_pool bruno_pool;
typedef struct bruno_pool_result {
  bruno_status status;      /* of the build */
  int32_t worker;           /* worker that ran it */
  int32_t words;            /* uint64 words per k-mer in reps */
  bruno_sizes sizes;
  uint64_t n_chains, n_chars;
  uint64_t *reps;           /* n_chains x words: representative k-mer of each compacted chain */
  uint64_t *offsets;        /* n_chains + 1 offsets into chars */
  char *chars;              /* the chain sequences */
  double queue_ms;          /* submit -> start on a worker */
  double run_ms;            /* start -> result on the host */
} bruno_pool_result;
bruno_status bruno_pool_create(const bruno_cfg *cfg, int32_t workers, uint64_t mem_budget, bruno_pool **out);
/* The same pool over the batched form (continuous batching): two scheduler threads, each with
 * its own context, repeatedly take every queued request whose estimates fit half of mem_budget
 * together (at least one, at most max_samples, 1..16384) and build them in one fused pass
 * (bruno_build_samples); requests that arrive during a pass join the next one, and one pass's
 * copies and result copy-outs run beside the other's kernels.  Results, submit / wait / free / destroy as above (run_ms
 * is the pass that built the request).  Where the batched form refuses the configuration, each
 * request is built with the plain path instead; every result equals the plain path's. */
bruno_status bruno_pool_create_batched(const bruno_cfg *cfg, uint32_t max_samples, uint64_t mem_budget,
                                       bruno_pool **out);
bruno_status bruno_pool_submit(bruno_pool *pool, const char *buf, size_t nbytes, uint64_t *ticket);
/* Blocks until the request is done; the result's arrays belong to the caller. */
bruno_status bruno_pool_wait(bruno_pool *pool, uint64_t ticket, bruno_pool_result *out);
bruno_status bruno_pool_result_free(bruno_pool_result *result);
/* Finishes every queued request, then stops the workers. */
bruno_status bruno_pool_destroy(bruno_pool *pool);

/* ---------------------------------------------------------------------------------------
 * Allocation-free pair counting.  This entry point has no counterpart in the reference; it
 * exists for callers that may not allocate device memory themselves or through this
 * library: a host application that has already handed the whole device to its own memory
 * pool, a plugin framework that only lends fixed buffers and forbids allocation calls, or a
 * latency-sensitive loop that must not stop for an allocator.  Every other entry point
 * allocates through its context, so such callers cannot use them.
 *
 * It counts the n (k-mer, biedge) pairs kmers[i], edges[i] and writes every distinct pair once
 * with its count to out_kmers, out_edges, out_counts.  A k-mer is in the packing above (`words`
 * uint64 each, bits above 2k zero) and a biedge is a DNA16 byte (base before the k-mer in the
 * high nibble, base after it in the low nibble, 0 = none).  Pairs are counted exactly as given,
 * never canonicalised: pass each k-mer as the smaller of itself and its reverse complement,
 * with its biedge oriented to match (on a flip the two nibbles swap and each is complemented);
 * a pair and its reverse complement passed as they come are counted as two different pairs.
 * The outputs go to out_kmers,
 * out_edges, out_counts (capacity out_cap pairs, in no particular order).  *n_out receives
 * the number of distinct pairs.  All five arrays are DEVICE pointers; passing NULL for all
 * three outputs only counts.  The working hash table lives in one fixed device array of
 * BRUNO_NOALLOC_SCRATCH_BYTES inside the library, so n is limited to
 * BRUNO_NOALLOC_MAX_PAIRS_K31 pairs for k <= 31 and BRUNO_NOALLOC_MAX_PAIRS_K63 for
 * 32 <= k <= 63; a larger n returns BRUNO_ERR_CAPACITY before any work is queued.  Other
 * errors: BRUNO_ERR_ARG (bad k, device or pointers), BRUNO_ERR_BAD_INPUT (an edge nibble that
 * is not 0/1/2/4/8, or k-mer bits above 2k), BRUNO_ERR_CAPACITY (more distinct pairs than
 * out_cap; *n_out still holds the count), BRUNO_ERR_CUDA.
 *
 * The work runs on `stream` (a cudaStream_t, NULL = the default stream) of `device`; the
 * call waits for it before returning and leaves the caller's current device as it was.
 * There is one scratch array per device, held by every GPU that loads the library until the
 * process exits, and it keeps the last call's contents: each call first clears its counters
 * and the table slots it uses.  Two calls whose GPU work can overlap on the same device (from
 * two host threads, or on two streams without ordering between them) use the same table at
 * the same time and corrupt each other's counts.  Serialise them.  The first call on a device
 * does a one-time set-up for that device (it looks up the array's device address); make that
 * first call before any stream capture. */
#define BRUNO_NOALLOC_SCRATCH_BYTES (32u << 20)
#define BRUNO_NOALLOC_MAX_PAIRS_K31 ((((32u << 20) - (64u << 10)) / 32u) / 2u)
#define BRUNO_NOALLOC_MAX_PAIRS_K63 ((((32u << 20) - (64u << 10)) / 64u) / 2u)
bruno_status bruno_count_biedges_noalloc(int32_t device, int32_t k, const uint64_t *kmers, const uint8_t *edges,
                                         size_t n, uint64_t *out_kmers, uint8_t *out_edges, uint32_t *out_counts,
                                         size_t out_cap, size_t *n_out, void *stream);
#ifdef __cplusplus
}
#endif

#endif /* BRUNO_GB300_H_ */
