/*
 * bruno_gb300.hpp -- header-only C++ facade over the C ABI with the class and method names
 * of ParBLiSS/bruno's src/debruijn API, so a driver written against the reference compiles
 * against the GB300 library with its types swapped:
 *
 *   reference                                              here
 *   bliss::debruijn::graph::debruijn_graph<K,uint16_t>     bruno_gb300::debruijn_graph
 *     .get_map().compute_biedge_freqencies(nodes, k2)        .get_map().compute_biedge_freqencies()
 *     .get_map().local_insert_by_freqencies(k2, threshes)    .get_map().local_insert_by_freqencies(threshes)
 *     .find_if(pred) / .erase_if(pred)                       same, pred a tag of bruno_gb300::filter::graph
 *     .get_map().erase_nodes(kmers)                          same
 *   bliss::debruijn::graph::debruijn_chain_graph<K>        bruno_gb300::debruijn_chain_graph
 *     .extract_chains(idx)                                   .extract_chains(idx)
 *     .list_rank_min_update() / .list_rank()                 same
 *     .to_ranked_chain_nodes() / .to_compressed_chains()     same
 *     .find_if(pred)                                         same, pred a tag of bruno_gb300::filter::chain
 *     .get_cycle_node_kmers() / .get_isolated()              same
 *     .get_internal_node_kmers()                             same
 *   bliss::debruijn::filter::graph::IsBranchPoint, ...     bruno_gb300::filter::graph::IsBranchPoint, ...
 *
 * The reference's (k-mer, biedge) vector and k2 counter are not materialised on the host:
 * they live in device memory inside the context.  Errors become bruno_gb300::error
 * exceptions carrying the bruno_status, as the reference throws std::logic_error.
 * k-mers are returned as uint64 words (1 word for k <= 31, 2 for k >= 32, low word first).
 */
#ifndef BRUNO_GB300_HPP_
#define BRUNO_GB300_HPP_

#include <cstdint>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "bruno_gb300.h"

namespace bruno_gb300 {

struct error : std::runtime_error {
  bruno_status status;
  error(bruno_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void check(bruno_status s, bruno_ctx *c, const char *what) {
  if (s != BRUNO_OK) throw error(s, std::string(what) + ": " + (c ? bruno_last_error(c) : ""));
}

/* -L / -U handling of compact_dbg_freq_construct_clean.cpp:937-961 (order k_lo, k_hi,
 * k1_lo, k1_hi, k2_lo, k2_hi; one value = the (k+1)-mer bound). */
inline std::vector<uint64_t> thresholds(const std::vector<uint64_t> &lower, const std::vector<uint64_t> &upper,
                                        uint64_t count_max = 65535) {
  std::vector<uint64_t> t(6, count_max + 1);
  if (lower.size() == 1) { t[2] = std::min(lower[0], t[2]); t[0] = t[4] = 0; }
  else if (lower.size() == 3) {
    t[0] = std::min(lower[0], t[0]); t[2] = std::min(lower[1], t[2]); t[4] = std::min(lower[2], t[4]);
  }
  if (upper.size() == 1) t[3] = std::min(upper[0], t[3]);
  else if (upper.size() == 3) {
    t[1] = std::min(upper[0], t[1]); t[3] = std::min(upper[1], t[3]); t[5] = std::min(upper[2], t[5]);
  }
  return t;
}

/* The reference's predicate structs as tag types: each names the C ABI's predicate number. */
namespace filter {
namespace graph {   /* bliss::debruijn::filter::graph (src/debruijn/debruijn_graph_filters.hpp) */
struct IsKPalindrome { static constexpr int32_t value = BRUNO_IS_K_PALINDROME; };
struct IsKplus1Palindrome { static constexpr int32_t value = BRUNO_IS_KPLUS1_PALINDROME; };
struct IsBranchPoint { static constexpr int32_t value = BRUNO_IS_BRANCH_POINT; };
struct IsIsolated { static constexpr int32_t value = BRUNO_IS_ISOLATED_NODE; };
struct IsChainInternalNode { static constexpr int32_t value = BRUNO_IS_CHAIN_INTERNAL_NODE; };
struct IsChainNode { static constexpr int32_t value = BRUNO_IS_CHAIN_NODE; };
}  // namespace graph
namespace chain {   /* bliss::debruijn::filter::chain (src/debruijn/debruijn_chain_filters.hpp) */
struct IsUnitLength { static constexpr int32_t value = BRUNO_CHAIN_IS_UNIT_LENGTH; };
struct IsIsolated { static constexpr int32_t value = BRUNO_CHAIN_IS_ISOLATED; };
struct IsTerminus { static constexpr int32_t value = BRUNO_CHAIN_IS_TERMINUS; };
struct IsInternal { static constexpr int32_t value = BRUNO_CHAIN_IS_INTERNAL; };
struct IsTerminusOrIsolated { static constexpr int32_t value = BRUNO_CHAIN_IS_TERMINUS_OR_ISOLATED; };
struct IsCanonicalTerminus { static constexpr int32_t value = BRUNO_CHAIN_IS_CANONICAL_TERMINUS; };
struct IsCanonicalTerminusOrIsolated { static constexpr int32_t value = BRUNO_CHAIN_IS_CANONICAL_TERMINUS_OR_ISOLATED; };
struct PointsToTermini { static constexpr int32_t value = BRUNO_CHAIN_POINTS_TO_TERMINI; };
struct PointsToInternalNode { static constexpr int32_t value = BRUNO_CHAIN_POINTS_TO_INTERNAL_NODE; };
}  // namespace chain
}  // namespace filter

/* (k-mer, compact_multi_biedge) records of find_if: keys (words each), counts (9 each), flags */
struct node_records {
  std::vector<uint64_t> keys;
  std::vector<uint16_t> counts;
  std::vector<uint8_t> flags;
  size_t size() const { return flags.size(); }
};

/* (k-mer, simple_biedge<K>) records of the chain map: K, inK, outK (words each), inDist, outDist */
struct chain_records {
  std::vector<uint64_t> K, inK, outK;
  std::vector<uint32_t> inD, outD;
  size_t size() const { return inD.size(); }
};

/* one graph build on one GPU; the graph map and the chain graph share it */
class context {
 public:
  explicit context(const bruno_cfg &cfg) : cfg_(cfg) { check(bruno_ctx_create(&cfg_, &ctx_), nullptr, "ctx_create"); }
  ~context() { if (ctx_) bruno_ctx_destroy(ctx_); }
  context(const context &) = delete;
  context &operator=(const context &) = delete;
  bruno_ctx *get() const { return ctx_; }
  const bruno_cfg &cfg() const { return cfg_; }
  int words() const { return cfg_.k <= 31 ? 1 : 2; }
  bruno_sizes sizes() const {
    bruno_sizes s;
    check(bruno_get_sizes(ctx_, &s), ctx_, "get_sizes");
    return s;
  }

 private:
  bruno_cfg cfg_;
  bruno_ctx *ctx_ = nullptr;
};

/* debruijn_graph_map (debruijn_graph_map.hpp:52-1626) */
class debruijn_graph_map {
 public:
  explicit debruijn_graph_map(context &c) : c_(c) {}
  /* parse_file_data of one file into the device-side (k-mer, biedge) stream */
  void load_fastq(const char *buf, size_t n, bool on_device = false) {
    check(bruno_load_fastq(c_.get(), buf, n, on_device ? 1 : 0), c_.get(), "load_fastq");
  }
  /* compute_biedge_freqencies (:1085-1141): returns the distinct (k+2)-mer count */
  size_t compute_biedge_freqencies() {
    check(bruno_compute_biedge_freqencies(c_.get()), c_.get(), "compute_biedge_freqencies");
    return c_.sizes().n_k2;
  }
  /* local_insert_by_freqencies (:1258-1623): returns the node count */
  size_t local_insert_by_freqencies(const std::vector<uint64_t> &threshes) {
    if (threshes.size() != 6) throw error(BRUNO_ERR_ARG, "threshes takes 6 values");
    check(bruno_local_insert_by_freqencies(c_.get(), threshes.data()), c_.get(), "local_insert_by_freqencies");
    return c_.sizes().n_nodes;
  }
  size_t local_size() const { return c_.sizes().n_nodes; }
  /* erase_nodes(query) (:833-836): the nodes (k-mers of either strand, words each) and, on their
   * neighbours, the edges back to them */
  void erase_nodes(const std::vector<uint64_t> &query) {
    check(bruno_graph_erase_nodes(c_.get(), query.data(), query.size() / c_.words()), c_.get(), "erase_nodes");
  }
  /* the node table: k-mers (words per node) and counts[9] (out ACGT, in ACGT, self) */
  void to_vector(std::vector<uint64_t> &keys, std::vector<uint16_t> &counts, std::vector<uint8_t> &flags) const {
    size_t n = 0;
    check(bruno_copy_nodes(c_.get(), nullptr, nullptr, nullptr, 0, &n), c_.get(), "copy_nodes");
    keys.resize(n * c_.words()); counts.resize(n * 9); flags.resize(n);
    check(bruno_copy_nodes(c_.get(), keys.data(), counts.data(), flags.data(), n, &n), c_.get(), "copy_nodes");
  }

 private:
  context &c_;
};

/* debruijn_graph (debruijn_graph.hpp:45-295) */
class debruijn_graph {
 public:
  explicit debruijn_graph(context &c) : c_(c), map_(c) {}
  debruijn_graph_map &get_map() { return map_; }
  size_t size() const { return map_.local_size(); }
  size_t local_size() const { return map_.local_size(); }
  context &ctx() { return c_; }
  /* find_if(pred) (debruijn_graph.hpp:193-196) */
  template <typename Pred>
  node_records find_if(const Pred &) const {
    node_records r;
    size_t n = 0;
    check(bruno_graph_find_if(c_.get(), Pred::value, nullptr, nullptr, nullptr, 0, &n), c_.get(), "find_if");
    r.keys.resize(n * c_.words()); r.counts.resize(n * 9); r.flags.resize(n);
    check(bruno_graph_find_if(c_.get(), Pred::value, r.keys.data(), r.counts.data(), r.flags.data(), n, &n), c_.get(),
          "find_if");
    return r;
  }
  /* erase_if(pred) (:247-250): the matching nodes; returns how many */
  template <typename Pred>
  size_t erase_if(const Pred &) {
    size_t n = 0;
    check(bruno_graph_erase_if(c_.get(), Pred::value, &n), c_.get(), "erase_if");
    return n;
  }

 private:
  context &c_;
  debruijn_graph_map map_;
};

/* listranked_chain_node<K> = (K on the representative's strand, representative, distance) */
struct listranked_chain_nodes {
  std::vector<uint64_t> K, rep;
  std::vector<int32_t> dist;
  size_t size() const { return dist.size(); }
};

/* debruijn_chain_graph (debruijn_chain_graph.hpp:126-2290) */
class debruijn_chain_graph {
 public:
  explicit debruijn_chain_graph(context &c) : c_(c) {}
  void extract_chains(debruijn_graph &) { check(bruno_extract_chains(c_.get()), c_.get(), "extract_chains"); }
  size_t list_rank_min_update() { return rank(1); }
  size_t list_rank() { return rank(0); }
  size_t size() const { return c_.sizes().n_ranked; }
  /* find_if(pred) (debruijn_chain_graph.hpp:306-311) over the chain map */
  template <typename Pred>
  chain_records find_if(const Pred &) const { return records(Pred::value, 0); }
  /* get_cycle_node_kmers (:448-460): words per k-mer */
  std::vector<uint64_t> get_cycle_node_kmers() const {
    size_t n = 0;
    check(bruno_get_cycle_node_kmers(c_.get(), nullptr, 0, &n), c_.get(), "get_cycle_node_kmers");
    std::vector<uint64_t> k(n * c_.words());
    check(bruno_get_cycle_node_kmers(c_.get(), k.data(), n, &n), c_.get(), "get_cycle_node_kmers");
    return k;
  }
  /* get_isolated (:462-468) */
  chain_records get_isolated() const { return records(-1, 2); }
  /* get_internal_node_kmers (:410-415): the k-mers of IsInternal records */
  std::vector<uint64_t> get_internal_node_kmers() const { return find_if(filter::chain::IsInternal()).K; }
  listranked_chain_nodes to_ranked_chain_nodes() {
    compress();
    listranked_chain_nodes r;
    size_t n = 0;
    check(bruno_copy_ranked(c_.get(), nullptr, nullptr, nullptr, 0, &n), c_.get(), "copy_ranked");
    r.K.resize(n * c_.words()); r.rep.resize(n * c_.words()); r.dist.resize(n);
    check(bruno_copy_ranked(c_.get(), r.K.data(), r.rep.data(), r.dist.data(), n, &n), c_.get(), "copy_ranked");
    return r;
  }
  /* to_compressed_chains (:1778-1856): one sequence per chain, with its representative */
  std::vector<std::pair<std::vector<uint64_t>, std::string>> to_compressed_chains() {
    compress();
    size_t nc = 0, nch = 0;
    check(bruno_copy_chains(c_.get(), nullptr, nullptr, nullptr, 0, 0, &nc, &nch), c_.get(), "copy_chains");
    std::vector<uint64_t> reps(nc * c_.words()), offs(nc + 1);
    std::string chars(nch, '\0');
    check(bruno_copy_chains(c_.get(), reps.data(), offs.data(), &chars[0], nc, nch, &nc, &nch), c_.get(),
          "copy_chains");
    std::vector<std::pair<std::vector<uint64_t>, std::string>> out(nc);
    const int w = c_.words();
    for (size_t i = 0; i < nc; ++i) {
      out[i].first.assign(reps.begin() + i * w, reps.begin() + (i + 1) * w);
      out[i].second = chars.substr(offs[i], offs[i + 1] - offs[i]);
    }
    return out;
  }
  /* print_chain_frequencies' records (compact_dbg_stats.hpp:879-1065), unordered:
   * ends = L, R per record (2 * words), freqs = 11 per record */
  size_t chain_edges(std::vector<uint64_t> &ends, std::vector<uint16_t> &freqs) {
    compress();
    size_t n = 0;
    check(bruno_copy_chain_edges(c_.get(), nullptr, nullptr, 0, &n), c_.get(), "copy_chain_edges");
    ends.resize(n * 2 * c_.words());
    freqs.resize(n * 11);
    check(bruno_copy_chain_edges(c_.get(), ends.data(), freqs.data(), n, &n), c_.get(), "copy_chain_edges");
    return n;
  }
  /* to_summarized_chains' records (debruijn_chain_graph.hpp:1876-2005), unordered:
   * kmers = prev at 5', 5', 3', next at 3' per record (4 * words), dist, flags (2 per record) */
  size_t to_summarized_chains(std::vector<uint64_t> &kmers, std::vector<uint32_t> &dist, std::vector<uint8_t> &flags) {
    compress();
    size_t n = 0;
    check(bruno_copy_chain_summaries(c_.get(), nullptr, nullptr, nullptr, 0, &n), c_.get(), "copy_chain_summaries");
    kmers.resize(n * 4 * c_.words());
    dist.resize(n);
    flags.resize(n * 2);
    check(bruno_copy_chain_summaries(c_.get(), kmers.data(), dist.data(), flags.data(), n, &n), c_.get(),
          "copy_chain_summaries");
    return n;
  }
  /* clean_deadend_and_bubbles_naive (test/common/compact_dbg_clean.hpp:575-890) on this chain
   * graph and its de Bruijn graph; afterwards both describe the cleaned graph */
  bruno_clean_stats clean_deadend_and_bubbles_naive() {
    bruno_clean_stats s{};
    check(bruno_clean_deadend_and_bubbles_naive(c_.get(), &s), c_.get(), "clean_deadend_and_bubbles_naive");
    ranked_ = true;
    return s;
  }

 private:
  size_t rank(int min_update) {
    uint64_t it = 0;
    check(bruno_list_rank(c_.get(), min_update, &it), c_.get(), "list_rank");
    ranked_ = false;
    return it;
  }
  chain_records records(int32_t filter, int which) const {
    chain_records r;
    size_t n = 0;
    auto call = [&](uint64_t *K, uint64_t *inK, uint64_t *outK, uint32_t *inD, uint32_t *outD, size_t cap) {
      return which == 2 ? bruno_get_isolated(c_.get(), K, inK, outK, inD, outD, cap, &n)
                        : bruno_chain_find_if(c_.get(), filter, K, inK, outK, inD, outD, cap, &n);
    };
    check(call(nullptr, nullptr, nullptr, nullptr, nullptr, 0), c_.get(), "chain find_if");
    const size_t w = c_.words();
    r.K.resize(n * w); r.inK.resize(n * w); r.outK.resize(n * w); r.inD.resize(n); r.outD.resize(n);
    check(call(r.K.data(), r.inK.data(), r.outK.data(), r.inD.data(), r.outD.data(), n), c_.get(), "chain find_if");
    return r;
  }
  void compress() {
    if (!ranked_) {
      check(bruno_to_compressed_chains(c_.get()), c_.get(), "to_compressed_chains");
      ranked_ = true;
    }
  }
  context &c_;
  bool ranked_ = false;
};

}  // namespace bruno_gb300

#endif /* BRUNO_GB300_HPP_ */
