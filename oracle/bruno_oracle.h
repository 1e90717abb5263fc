/*
 * bruno_oracle.h -- C API of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a CPU restatement of ParBLiSS/bruno's
 * graph-construction path (FASTQ -> canonical k-mer/biedge -> (k+2)-mer counting ->
 * frequency filter -> chain extraction -> list ranking -> compacted chains).  It is the
 * parity checker for the CUDA library and the timed CPU baseline; nothing in the product
 * library links or calls it.
 *
 * The reference itself cannot be compiled: its k-mer/alphabet/FASTQ/hash-map layer is the
 * un-vendored `kmerind` submodule (ext/kmerind is empty).  Every function in
 * bruno_oracle.cpp cites the reference file:line it restates.
 *
 * k-mer words: a k-mer of length k (1..63) is 2-bit packed, first character in the most
 * significant bits, A=0 C=1 G=2 T=3.  Arrays of k-mers use `words` uint64 per k-mer
 * (1 for k <= 31, 2 for k >= 32 -- the GB300 library's layout; for 2 words the low word
 * comes first).
 */
#ifndef BRUNO_ORACLE_H_
#define BRUNO_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_cfg {
  int32_t k;                /* k-mer length, 1..63 */
  int32_t thresholding;     /* -T: 1 = build_index_thresholded, 0 = build_index */
  uint64_t thresh[6];       /* k_lo, k_hi, k1_lo, k1_hi, k2_lo, k2_hi (debruijn_graph_map.hpp:1261) */
  int32_t min_update;       /* -R: 1 = list_rank_min_update, 0 = list_rank */
  int32_t threads;          /* host threads = hash shards (stand-in for MPI ranks); 0 = 1 */
  int32_t keep_k2;          /* 1: keep the unfiltered (k+2)-mer count table for output */
  int32_t keep_filtered;    /* 1: keep the filtered (k+2)-mer entries for output */
  int32_t edge_filter;      /* 1 (with thresholding): the blocked driver's build_index_thresholded
                               (compact_debruijn_graph_block_construct.cpp:417-470): (k+1)-mers
                               counted and kept in [thresh[2], thresh[3]), biedges losing the
                               edges whose (k+1)-mer is gone, then the unthresholded insert */
  int32_t clean;            /* 1: the _freq_clean driver's graph cleaning after the first
                               compaction (clean_deadend_and_bubbles_naive,
                               compact_dbg_clean.hpp:575-890): dead ends shorter than 2k-1 and
                               bubbles lose their end edges of frequency <= thresh[2], the graph
                               is recompacted, until no dead end or bubble is left */
} oracle_cfg;

/* Phase timers, seconds, named after the reference's BL_BENCH phases. */
enum {
  ORACLE_T_PARSE = 0, ORACLE_T_COUNT_K2, ORACLE_T_FILTER_INSERT, ORACLE_T_CHAINMAP,
  ORACLE_T_LIST_RANK, ORACLE_T_COMPRESS, ORACLE_T_NUM
};

typedef struct oracle_result {
  int32_t status;           /* 0 ok, 2 bad input */
  int32_t words;            /* uint64 words per k-mer in the arrays below */
  uint64_t n_reads;         /* FASTQ records */
  uint64_t n_reads_used;    /* records that produced k-mers (no N, length >= k+2) */
  uint64_t n_instances;     /* (k-mer, biedge) pairs parsed */

  uint64_t n_k2;            /* distinct canonical (k-mer, biedge) entries */
  uint64_t *k2_keys; uint8_t *k2_edges; uint32_t *k2_counts;  /* sorted by (k-mer, edge) */

  uint64_t n_filtered;      /* entries kept by the filter (edges already trimmed) */
  uint64_t *filt_keys; uint8_t *filt_edges; uint32_t *filt_counts; /* sorted by (k-mer, edge) */
  uint64_t filter_flag_hist[16];  /* k_del[] histogram (debruijn_graph_map.hpp:1568) */

  uint64_t n_nodes;         /* graph nodes after the filter */
  uint64_t *node_keys; uint16_t *node_counts; /* 9 counts per node, sorted by k-mer */
  uint8_t *node_flags;      /* bit 0: IsBranchPoint, bit 1: IsChainNode */
  uint64_t n_branch;        /* IsBranchPoint nodes */
  uint64_t n_chain_nodes;   /* IsChainNode nodes inserted into the chain map */

  uint64_t iterations;      /* list-ranking rounds */
  uint64_t collisions;      /* order-dependent collisions: a (node, side) whose updates of one
                               round give a different state applied in sequence than the
                               largest (distance, mark) update alone */
  uint64_t n_cycle_nodes;   /* removed by separate_cycles */
  uint64_t n_isolated;      /* removed by separate_isolated */

  uint64_t n_ranked;        /* listranked_chain_node records, sorted by K (chain_node_less) */
  uint64_t *ranked_K; uint64_t *ranked_rep; int32_t *ranked_dist;

  uint64_t n_chains;        /* compacted chains, sorted by rep (chain_rep_less) */
  uint64_t *chain_rep;      /* chain representative k-mer */
  uint64_t *chain_offsets;  /* n_chains + 1 offsets into chain_chars */
  char *chain_chars;        /* concatenated chain sequences (to_compressed_chains strings) */

  uint64_t n_chain_edges;   /* print_chain_frequencies records, one per chain, sorted by L */
  uint64_t *edge_L;         /* chain end on the representative's strand (the selected terminus) */
  uint64_t *edge_R;         /* the other end, same strand */
  uint16_t *edge_freqs;     /* 11 per record: L in-edges A C G T, R out-edges A C G T,
                               mean, min, max of the chain's node frequencies */

  uint64_t n_summaries;     /* to_summarized_chains records, in the reference's order (by rep) */
  uint64_t *sum_kmers;      /* 4 k-mers per record: prev at 5', 5' terminus, 3' terminus, next at 3' */
  uint32_t *sum_dist;       /* distance between the termini */
  uint8_t *sum_flags;       /* 2 per record: 5' and 3' terminal points to a branch (1) or nothing (0) */
  int32_t summaries_ok;     /* 0 when the pairing met a case the reference throws on */

  double seconds[ORACLE_T_NUM];

  /* graph cleaning (cfg.clean) */
  uint64_t clean_rounds;    /* iterations of the cleaning loop */
  uint64_t clean_deadends;  /* dead-end summaries found, over all iterations */
  uint64_t clean_bubbles;   /* bubble summaries found, over all iterations */
  uint64_t clean_edges;     /* low-frequency end edges found and erased (with their reverse edges) */
  int32_t clean_status;     /* 0 done; 1 stopped after an iteration that erased nothing (the
                               reference repeats such an iteration forever); 2 a terminus case the
                               reference throws on */
  struct oracle_result *clean;  /* the cleaned graph: node table (cycles and isolated nodes
                                   removed), ranked chain nodes, chains and chain edges */

  /* the chain map after list ranking (separate_cycles and separate_isolated have taken their
   * nodes out), sorted by k-mer: per node simple_biedge<K> = (inK, outK, inDist, outDist)
   * (debruijn_chain_node.hpp:49-50); then the records separate_isolated took out (get_isolated,
   * debruijn_chain_graph.hpp:462-468), and the k-mers separate_cycles took out
   * (get_cycle_node_kmers, :448-460), both sorted by k-mer */
  uint64_t n_chain_map;
  uint64_t *cm_keys, *cm_in, *cm_out; uint32_t *cm_in_dist, *cm_out_dist;
  uint64_t n_isolated_recs;
  uint64_t *iso_keys, *iso_in, *iso_out; uint32_t *iso_in_dist, *iso_out_dist;
  uint64_t n_cycle_kmers;
  uint64_t *cycle_keys;

  /* check_index (test/common/compact_dbg_stats.hpp:45-119) on the graph after the build:
   * neighbour k-mers named, of them absent, nodes with an edge that no node names, edges whose
   * neighbour lacks the edge back; and the in x out edge-count histogram (in * 5 + out) */
  uint64_t check_query, check_absent, check_unreferenced, check_unanswered;
  uint64_t edge_hist[25];
} oracle_result;

/* Runs the whole path on an in-memory FASTQ buffer.  Returns 0 on success. */
int oracle_run(const char *fastq, size_t nbytes, const oracle_cfg *cfg, oracle_result **out);
void oracle_free(oracle_result *r);

/* Writes the reference driver's text outputs for a finished run:
 * <prefix>.chain.fasta, <prefix>.chain.components, <prefix>.branch.fasta and, unless
 * benchmark != 0, <prefix>.chain.edges, <prefix>.chain.summary (when summaries_ok),
 * <prefix>.branch.edges and <prefix>.graph.all.  After cleaning, as the _freq_clean driver:
 * the same first-compaction files except .chain.edges, then <prefix>.clean.branch.edges,
 * .clean.branch.fasta, .clean.chain.fasta, .clean.chain.components and .clean.chain.edges of
 * the cleaned graph. */
int oracle_write_outputs(const oracle_result *r, int32_t k, const char *prefix, int32_t benchmark);

#ifdef __cplusplus
}
#endif

#endif /* BRUNO_ORACLE_H_ */
