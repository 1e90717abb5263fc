/*
 * bruno_oracle.cpp -- CPU restatement of ParBLiSS/bruno's de Bruijn graph-construction
 * path.  TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA library and the timed
 * CPU baseline.  The product library never links, loads or calls this file.
 *
 * Every step follows the reference file:line cited beside it.  The reference's k-mer,
 * alphabet, FASTQ-parser and distributed-hash-map layer lives in the un-vendored kmerind
 * submodule, so the semantics taken from it are restated from their use inside bruno:
 *   - 2-bit DNA codes A0 C1 G2 T3, first character in the most significant bits, last
 *     character at the LSBs (debruijn_graph_loader.hpp:87-88, debruijn_chain_operations.hpp:380,
 *     kmer_traits.hpp:79,86);
 *   - nextFromChar appends at the 3' end, nextReverseFromChar prepends at the 5' end
 *     (debruijn_graph_node.hpp:327,344);
 *   - DNA16 codes A1 C2 G4 T8 N15, gap 0 (debruijn_graph_node.hpp:118-136);
 *   - k-mer operator< is the lexicographic order of the strings, i.e. the unsigned order of
 *     the packed words;
 *   - reads containing N are dropped (compact_dbg_freq_construct_clean.cpp:210-213), and
 *     reads shorter than the k+2 window give no k-mers (debruijn_biedge_loader.hpp:402,462-505).
 * The distributed maps become per-shard open-addressing maps, one shard per host thread,
 * standing in for the reference's MPI ranks: outputs must not depend on the shard count.
 */
#include "bruno_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

typedef unsigned __int128 u128;

/* ---------------------------------------------------------------- k-mer words */

inline uint64_t rev_pairs(uint64_t x) {
  x = ((x >> 2) & 0x3333333333333333ULL) | ((x & 0x3333333333333333ULL) << 2);
  x = ((x >> 4) & 0x0F0F0F0F0F0F0F0FULL) | ((x & 0x0F0F0F0F0F0F0F0FULL) << 4);
  return __builtin_bswap64(x);
}
inline u128 rev_pairs(u128 x) {
  return ((u128)rev_pairs((uint64_t)x) << 64) | (u128)rev_pairs((uint64_t)(x >> 64));
}
inline uint64_t mix64(uint64_t x) {  /* splitmix64 finaliser */
  x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ULL;
  x ^= x >> 27; x *= 0x94d049bb133111ebULL;
  x ^= x >> 31; return x;
}
inline uint64_t hash_word(uint64_t x) { return mix64(x); }
inline uint64_t hash_word(u128 x) { return mix64((uint64_t)x ^ mix64((uint64_t)(x >> 64))); }

/* Operations of bliss::common::Kmer<k, DNA, W> for a runtime k. */
template <typename W>
struct KOps {
  static constexpr int BITS = 8 * sizeof(W);
  int k;
  W mask;
  explicit KOps(int k_) : k(k_) { mask = (2 * k >= BITS) ? ~W(0) : ((W(1) << (2 * k)) - 1); }
  /* Kmer::reverse_complement: complement = 3 - c = c ^ 3, then reverse character order. */
  W rc(W x) const { return rev_pairs(W(~x)) >> (BITS - 2 * k); }
  /* reverse complement of the (k-1)-mer held in the low 2(k-1) bits */
  W rc_km1(W x) const { return rev_pairs(W(~x)) >> (BITS - 2 * (k - 1)); }
  unsigned first(W x) const { return (unsigned)(x >> (2 * (k - 1))) & 3u; }  /* getCharsAtPos(k-1) */
  unsigned last(W x) const { return (unsigned)x & 3u; }                     /* getCharsAtPos(0) */
  W next_from_char(W x, unsigned c) const { return ((x << 2) | W(c)) & mask; }
  W next_reverse_from_char(W x, unsigned c) const { return (x >> 2) | (W(c) << (2 * (k - 1))); }
  std::string ascii(W x) const {
    static const char A[4] = {'A', 'C', 'G', 'T'};
    std::string s(k, 'A');
    for (int i = 0; i < k; ++i) s[k - 1 - i] = A[(unsigned)(x >> (2 * i)) & 3u];
    return s;
  }
};

inline void store_word(uint64_t *dst, uint64_t x, int) { dst[0] = x; }
inline void store_word(uint64_t *dst, u128 x, int words) {
  dst[0] = (uint64_t)x;
  if (words > 1) dst[1] = (uint64_t)(x >> 64);
}

/* DNA16 nibble <-> DNA code (debruijn_graph_node.hpp:118-136 FROM_DNA16 table). */
inline unsigned from_dna16(unsigned n) {
  switch (n) { case 1: return 0; case 2: return 1; case 4: return 2; case 8: return 3; default: return 8; }
}
/* DNA16 complement = bit reversal of the nibble (A1<->T8, C2<->G4, N15, gap 0). */
inline unsigned comp16(unsigned n) {
  return ((n & 1u) << 3) | ((n & 2u) << 1) | ((n & 4u) >> 1) | ((n & 8u) >> 3);
}
/* transform::reverse_complement(compact_simple_biedge) (debruijn_biedge_loader.hpp:708-712):
 * the 2-character DNA16 k-mer "in out" becomes "comp(out) comp(in)". */
inline uint8_t rc_biedge(uint8_t e) { return (uint8_t)((comp16(e & 0xFu) << 4) | comp16(e >> 4)); }

inline int char_code(unsigned char c) {
  switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return -1;
  }
}

/* ------------------------------------------------------- chain distance words */
/* debruijn_chain_node.hpp:53-80 */
constexpr uint32_t dist_mask = 0x7FFFFFFFu;
constexpr uint32_t term_mask = 0x80000000u;
inline uint32_t get_chain_dist(uint32_t x) { return x & dist_mask; }
inline bool is_chain_terminal(uint32_t x) { return (x & dist_mask) == 0; }
inline bool points_to_self(uint32_t x) { return x == term_mask; }
inline bool points_to_chain_node(uint32_t x) { return (x ^ term_mask) > term_mask; }
inline uint32_t mark_terminal(uint32_t x) { return x | term_mask; }

/* ---------------------------------------------------------- saturating counts */
/* debruijn_graph_node.hpp:81-91 */
inline uint16_t sat_add(uint16_t a, uint16_t b) {
  uint16_t c = (uint16_t)(a + b);
  return (c < a) ? (uint16_t)0xFFFF : c;
}
inline void sat_incr(uint16_t &t) { t += (t < 0xFFFF); }

/* ----------------------------------------------------- open-addressing map */
template <typename K, typename V>
struct OAMap {
  std::vector<K> keys;
  std::vector<V> vals;
  std::vector<uint8_t> state;  /* 0 empty, 1 live, 2 erased */
  size_t live = 0, used = 0, mask = 0;

  void init(size_t expected) {
    size_t cap = 16;
    while (cap < 2 * expected + 16) cap <<= 1;
    keys.assign(cap, K()); vals.assign(cap, V()); state.assign(cap, 0);
    mask = cap - 1; live = used = 0;
  }
  static uint64_t h(const K &k) { return k.hash(); }
  void grow() {
    std::vector<K> ok; std::vector<V> ov; std::vector<uint8_t> os;
    ok.swap(keys); ov.swap(vals); os.swap(state);
    init(live * 2 + 16);
    for (size_t i = 0; i < ok.size(); ++i)
      if (os[i] == 1) { bool ins; get(ok[i], &ins) = ov[i]; }
  }
  V *find(const K &k) {
    if (keys.empty()) return nullptr;
    for (size_t i = h(k) & mask;; i = (i + 1) & mask) {
      if (state[i] == 0) return nullptr;
      if (state[i] == 1 && keys[i] == k) return &vals[i];
    }
  }
  V &get(const K &k, bool *inserted) {
    if (keys.empty()) init(16);
    if (2 * (used + 1) > keys.size()) grow();
    for (size_t i = h(k) & mask;; i = (i + 1) & mask) {
      if (state[i] == 0) {
        state[i] = 1; keys[i] = k; vals[i] = V(); ++live; ++used;
        *inserted = true; return vals[i];
      }
      if (state[i] == 1 && keys[i] == k) { *inserted = false; return vals[i]; }
    }
  }
  void erase_slot(size_t i) { state[i] = 2; --live; }
};

template <typename W>
struct KmerKey {
  W v;
  bool operator==(const KmerKey &o) const { return v == o.v; }
  uint64_t hash() const { return hash_word(v); }
};
template <typename W>
struct K2Key {
  W kmer;
  uint8_t edge;
  bool operator==(const K2Key &o) const { return kmer == o.kmer && edge == o.edge; }
  uint64_t hash() const { return hash_word(kmer) ^ mix64(0x9e3779b97f4a7c15ULL * (edge + 1)); }
};

struct Node { uint16_t c[9]; };  /* compact_multi_biedge<DNA,uint16>: out ACGT, in ACGT, self */

/* Oracle bookkeeping for one side of a chain node during one list-ranking round: the
 * side's state at the start of the round, the number of updates it received, and the
 * update with the largest (distance, terminal mark).  Used to prove that applying the
 * round's updates in sequence (the reference) equals applying only that largest update
 * (the CUDA kernels); a side where the two differ is an order-dependent collision. */
template <typename W>
struct SideLog {
  uint32_t round = ~0u, n = 0;
  W snapK = 0; uint32_t snapD = 0;
  W bestK = 0; uint32_t bestD = 0;
};

template <typename W>
struct ChainNode {               /* simple_biedge<K> (debruijn_chain_node.hpp:49-50) */
  W inK, outK;
  uint32_t inD, outD;
  SideLog<W> log_in, log_out;
};

/* ------------------------------------------------------------- parallel helper */
template <typename F>
void parallel(int T, F f) {
  if (T == 1) { f(0); return; }
  std::vector<std::thread> th;
  for (int t = 0; t < T; ++t) th.emplace_back(f, t);
  for (auto &x : th) x.join();
}

/* Sorts v with T threads: T contiguous chunks are sorted at once, then T threads merge them,
 * each thread the output range between two splitters taken from the sorted chunks.  The
 * result is the order std::sort gives for a strict weak order (equal elements may come in
 * any order, as with std::sort). */
template <typename V, typename C>
void par_sort(std::vector<V> &v, C less, int T) {
  const size_t n = v.size();
  if (T <= 1 || n < (size_t)(1 << 16)) { std::sort(v.begin(), v.end(), less); return; }
  std::vector<size_t> lo(T + 1);
  for (int t = 0; t <= T; ++t) lo[t] = n * (size_t)t / (size_t)T;
  parallel(T, [&](int t) { std::sort(v.begin() + lo[t], v.begin() + lo[t + 1], less); });
  /* splitters: every chunk's elements at its T quantiles, sorted; thread t merges the
   * elements in [split[t-1], split[t]) of every chunk (by lower_bound on each side) */
  std::vector<V> sample;
  for (int t = 0; t < T; ++t)
    for (int q = 1; q < T; ++q) sample.push_back(v[lo[t] + (lo[t + 1] - lo[t]) * (size_t)q / (size_t)T]);
  std::sort(sample.begin(), sample.end(), less);
  std::vector<V> split;
  for (int q = 1; q < T; ++q) split.push_back(sample[sample.size() * (size_t)q / (size_t)T]);
  std::vector<std::vector<size_t>> cut(T, std::vector<size_t>(T + 1));   /* cut[chunk][range] */
  parallel(T, [&](int c) {
    cut[c][0] = lo[c];
    cut[c][T] = lo[c + 1];
    for (int q = 1; q < T; ++q)
      cut[c][q] = (size_t)(std::lower_bound(v.begin() + lo[c], v.begin() + lo[c + 1], split[q - 1], less) - v.begin());
  });
  std::vector<size_t> out0(T + 1, 0);
  for (int q = 0; q < T; ++q) {
    size_t m = 0;
    for (int c = 0; c < T; ++c) m += cut[c][q + 1] - cut[c][q];
    out0[q + 1] = out0[q] + m;
  }
  std::vector<V> out(n);
  parallel(T, [&](int q) {
    /* T-way merge of the chunk pieces of range q */
    std::vector<std::pair<size_t, size_t>> runs;
    for (int c = 0; c < T; ++c)
      if (cut[c][q] < cut[c][q + 1]) runs.emplace_back(cut[c][q], cut[c][q + 1]);
    size_t o = out0[q];
    while (!runs.empty()) {
      size_t best = 0;
      for (size_t r = 1; r < runs.size(); ++r)
        if (less(v[runs[r].first], v[runs[best].first])) best = r;
      out[o++] = v[runs[best].first];
      if (++runs[best].first == runs[best].second) runs.erase(runs.begin() + (long)best);
    }
  });
  v.swap(out);
}

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct ReadSpan { size_t off; uint32_t len; };

/* FASTQ record split (kmerind FASTQParser + NFilterSequencesIterator, selected at
 * compact_dbg_freq_construct_clean.cpp:195-219): records are 4 lines, '@' header,
 * sequence, '+' separator, quality; EOL characters are not part of the sequence
 * (NonEOLIter, debruijn_biedge_loader.hpp:408-410); blank lines where a record header is
 * expected are skipped.  Returns false on malformed input. */
bool split_fastq(const char *buf, size_t n, std::vector<ReadSpan> &seqs, uint64_t &records) {
  size_t pos = 0, line = 0;
  records = 0;
  while (pos < n) {
    const char *nl = (const char *)memchr(buf + pos, '\n', n - pos);
    size_t e = nl ? (size_t)(nl - buf) : n;
    size_t le = e;
    if (le > pos && buf[le - 1] == '\r') --le;
    if ((line & 3) == 0 && le == pos) { pos = e + 1; continue; }  /* blank line between records */
    switch (line & 3) {
      case 0: if (buf[pos] != '@') return false; break;
      case 1: seqs.push_back({pos, (uint32_t)(le - pos)}); break;
      case 2: if (le == pos || buf[pos] != '+') return false; break;
      default: ++records; break;
    }
    ++line;
    pos = e + 1;
  }
  return (line & 3) == 0;
}

/* ====================================================================== run */
template <typename W>
struct Run {
  const oracle_cfg cfg;
  const int T;
  const KOps<W> ko;
  oracle_result *res;

  std::vector<OAMap<K2Key<W>, uint32_t>> k2;          /* LocalK2CountMapType per shard */
  std::vector<OAMap<KmerKey<W>, Node>> nodes;         /* debruijn_graph_map per shard */
  std::vector<OAMap<KmerKey<W>, ChainNode<W>>> chain; /* debruijn_chain_graph map per shard */
  std::vector<std::vector<std::pair<K2Key<W>, uint32_t>>> filtered;

  const uint64_t clean_k1_lo;   /* threshes[2] as the driver passed it, whatever the filter used */
  std::vector<W> cycle_kmers;   /* get_cycle_node_kmers after the last list ranking */
  std::vector<std::pair<W, ChainNode<W>>> isolated_recs;   /* get_isolated after the last ranking */

  Run(const oracle_cfg &c, oracle_result *r, uint64_t k1_lo)
      : cfg(c), T(c.threads > 0 ? c.threads : 1), ko(c.k), res(r), clean_k1_lo(k1_lo) {}

  /* owning shard: the high hash bits, independent of the low bits that pick map slots */
  int shard(W kmer) const { return (int)((hash_word(kmer) >> 40) % (uint64_t)T); }

  /* lex_less<KMER>::operator()(pair) (debruijn_common.hpp:53-57): keeps the pair when
   * kmer < rc(kmer), otherwise flips the k-mer and reverse-complements the value. */
  void canonical(W &kmer, uint8_t &edge) const {
    W y = ko.rc(kmer);
    if (!(kmer < y)) { kmer = y; edge = rc_biedge(edge); }
  }

  /* ---------------------------------------------------------------- palindromes
   * kmer_traits.hpp:56-88 and debruijn_graph_filters.hpp:57-90.  DNA with odd k has no
   * k-palindromes; DNA with even k has no (k-1)-palindromes. */
  bool is_rc_palindrome(W x) const { return (ko.k & 1) ? false : (x == ko.rc(x)); }
  bool km1_high(W x) const {  /* first k-1 characters form an rc-palindrome */
    if ((ko.k & 1) == 0) return false;
    W h = x >> 2;
    return h == ko.rc_km1(h);
  }
  bool km1_low(W x) const {   /* last k-1 characters form an rc-palindrome */
    if ((ko.k & 1) == 0) return false;
    W l = x & (ko.mask >> 2);
    return l == ko.rc_km1(l);
  }
  /* is_k1_rc_palindrome(l, k, high): the (k+1)-mer l.K is its own reverse complement */
  bool k1pal_in(unsigned l, W x, bool high) const {
    if ((ko.k & 1) == 0) return false;
    if (ko.last(x) != 3u - l) return false;
    return high;
  }
  /* is_k1_rc_palindrome(k, r, low): the (k+1)-mer K.r is its own reverse complement */
  bool k1pal_out(W x, unsigned r, bool low) const {
    if ((ko.k & 1) == 0) return false;
    if (ko.first(x) != 3u - r) return false;
    return low;
  }
  /* IsKplus1Palindrome (debruijn_graph_filters.hpp:57-90) via is_k1_k1pair_rc_palindrome
   * (kmer_traits.hpp:108-125). */
  bool is_kplus1_palindrome(W x, const Node &n) const {
    if ((ko.k & 1) == 0) return false;
    bool low = km1_low(x);
    for (unsigned c = 0; c < 4; ++c)
      if (n.c[c] > 0 && low && (ko.first(x) == 3u - c || ko.first(x) == c)) return true;
    bool high = km1_high(x);
    for (unsigned c = 0; c < 4; ++c)
      if (n.c[4 + c] > 0 && high && (ko.last(x) == 3u - c || ko.last(x) == c)) return true;
    return false;
  }
  static unsigned in_count(const Node &n) {
    unsigned d = 0; for (int i = 4; i < 8; ++i) d += n.c[i] > 0; return d;
  }
  static unsigned out_count(const Node &n) {
    unsigned d = 0; for (int i = 0; i < 4; ++i) d += n.c[i] > 0; return d;
  }
  /* IsBranchPoint (debruijn_graph_filters.hpp:142-160) */
  bool is_branch(W x, const Node &n) const {
    return in_count(n) >= 2 || out_count(n) >= 2 || is_rc_palindrome(x) || is_kplus1_palindrome(x, n);
  }
  /* IsChainNode (debruijn_graph_filters.hpp:206-220) */
  bool is_chain(W x, const Node &n) const {
    return in_count(n) < 2 && out_count(n) < 2 && !is_rc_palindrome(x) && !is_kplus1_palindrome(x, n);
  }

  /* compact_multi_biedge<DNA,COUNT>::update(edges, cnt) (debruijn_graph_node.hpp:200-211) */
  static void node_update(Node &n, uint8_t edges, uint16_t cnt) {
    unsigned out = from_dna16(edges & 0xFu), in = from_dna16(edges >> 4);
    if (out < 4) n.c[out] = sat_add(n.c[out], cnt);
    if (in < 4) n.c[4 + in] = sat_add(n.c[4 + in], cnt);
    n.c[8] = sat_add(n.c[8], cnt);
  }

  /* ============================================================ parse + count */
  /* debruijn_kmer_simple_biedge_parser (debruijn_biedge_loader.hpp:393-623) with
   * biedge_generating_iterator::operator* (:356-372), then compute_biedge_freqencies
   * (debruijn_graph_map.hpp:1085-1141): transform_input = lex_less, distribute to the
   * owning shard, count into a uint32 (non-saturating) k2 counter. */
  /* ------------------------------------------------ (k+1)-mer edge filter
   * compute_edge_frequency (debruijn_biedge_filters.hpp:128-177) with KmerParser over the
   * N-filtered reads: every (k+1)-mer of a read at least k+1 long, canonical (lex_less), in a
   * saturating uint16 counter (CountType of compact_debruijn_graph_block_construct.cpp:151);
   * entries with count < lo or >= hi are erased when lo > 0 or hi < 65536 (:163-171).  The
   * keys are 128-bit so every k up to 63 fits. */
  std::vector<OAMap<KmerKey<u128>, uint32_t>> k1;

  int shard1(u128 x) const { return (int)((hash_word(x) >> 40) % (uint64_t)T); }

  void count_k1mers(const char *buf, const std::vector<ReadSpan> &seqs) {
    const int k = ko.k;
    const KOps<u128> k1o(k + 1);
    std::vector<std::vector<std::vector<u128>>> out(T, std::vector<std::vector<u128>>(T));
    parallel(T, [&](int t) {
      size_t b = seqs.size() * t / T, e = seqs.size() * (t + 1) / T;
      std::vector<int> codes;
      for (size_t r = b; r < e; ++r) {
        const unsigned char *s = (const unsigned char *)buf + seqs[r].off;
        const uint32_t L = seqs[r].len;
        codes.resize(L);
        bool ok = true;
        for (uint32_t i = 0; i < L; ++i) { codes[i] = char_code(s[i]); ok &= codes[i] >= 0; }
        if (!ok || L < (uint32_t)k + 1) continue;
        u128 x = 0;
        for (int i = 0; i < k; ++i) x = (x << 2) | (u128)codes[i];
        for (uint32_t p = 0; p + k + 1 <= L; ++p) {
          x = ((x << 2) | (u128)codes[p + k]) & k1o.mask;
          const u128 y = k1o.rc(x), c = x < y ? x : y;
          out[t][shard1(c)].push_back(c);
        }
      }
    });
    const uint64_t lo = cfg.thresh[2], hi = cfg.thresh[3];
    const bool erase = lo > 0 || hi < 65536;
    k1.resize(T);
    parallel(T, [&](int s) {
      size_t total = 0;
      for (int t = 0; t < T; ++t) total += out[t][s].size();
      k1[s].init(total / 4 + 16);
      for (int t = 0; t < T; ++t) {
        for (const u128 &x : out[t][s]) {
          bool ins;
          uint32_t &c = k1[s].get(KmerKey<u128>{x}, &ins);
          if (c < 0xFFFFu) ++c;
        }
        std::vector<u128>().swap(out[t][s]);
      }
      if (erase)
        for (size_t i = 0; i < k1[s].keys.size(); ++i)
          if (k1[s].state[i] == 1 && (k1[s].vals[i] < lo || k1[s].vals[i] >= hi)) k1[s].erase_slot(i);
    });
  }

  /* the read-orientation (k+1)-mer at codes[p..p+k] kept by the counter? */
  bool k1_exists(const std::vector<int> &codes, uint32_t p) const {
    const KOps<u128> k1o(ko.k + 1);
    u128 x = 0;
    for (int i = 0; i <= ko.k; ++i) x = (x << 2) | (u128)codes[p + i];
    const u128 y = k1o.rc(x), c = x < y ? x : y;
    return const_cast<OAMap<KmerKey<u128>, uint32_t> &>(k1[shard1(c)]).find(KmerKey<u128>{c}) != nullptr;
  }

  bool parse_and_count(const char *buf, size_t n) {
    double t0 = now();
    std::vector<ReadSpan> seqs;
    uint64_t records = 0;
    if (!split_fastq(buf, n, seqs, records)) return false;
    res->n_reads = records;
    const int k = ko.k;
    if (cfg.edge_filter) count_k1mers(buf, seqs);
    std::vector<std::vector<std::vector<std::pair<W, uint8_t>>>> out(T, std::vector<std::vector<std::pair<W, uint8_t>>>(T));
    std::vector<uint64_t> used(T, 0), inst(T, 0);
    parallel(T, [&](int t) {
      size_t b = seqs.size() * t / T, e = seqs.size() * (t + 1) / T;
      std::vector<int> codes;
      for (size_t r = b; r < e; ++r) {
        const unsigned char *s = (const unsigned char *)buf + seqs[r].off;
        uint32_t L = seqs[r].len;
        codes.resize(L);
        bool ok = true;
        for (uint32_t i = 0; i < L; ++i) { codes[i] = char_code(s[i]); ok &= codes[i] >= 0; }
        if (!ok) continue;                          /* NFilterSequencesIterator */
        if (L < (uint32_t)k + 2) continue;           /* longer_than_window */
        ++used[t];
        W km = 0;
        for (int i = 0; i < k - 1; ++i) km = (km << 2) | W(codes[i]);
        for (uint32_t p = 0; p + k <= L; ++p) {
          km = ((km << 2) | W(codes[p + k - 1])) & ko.mask;
          unsigned in = p > 0 ? (1u << codes[p - 1]) : 0u;
          unsigned o = (p + k < L) ? (1u << codes[p + k]) : 0u;
          ++inst[t];
          if (cfg.edge_filter) {
            /* transform_biedges_by_frequency (debruijn_biedge_filters.hpp:331-423): an edge
             * whose (k+1)-mer the counter lost is cleared; filter_isolated_nodes (:66-75)
             * drops a pair left without edges.  (The reference checks a k-mer's in edge
             * through the out edge of the k-mer before it in parse order: the same
             * (k+1)-mer within a read, and an empty edge at a read's start either way.) */
            if (in && !k1_exists(codes, p - 1)) in = 0;
            if (o && !k1_exists(codes, p)) o = 0;
            if (!in && !o) continue;
          }
          W ck = km; uint8_t e2 = (uint8_t)((in << 4) | o);
          canonical(ck, e2);
          out[t][shard(ck)].emplace_back(ck, e2);
        }
      }
    });
    for (int t = 0; t < T; ++t) { res->n_reads_used += used[t]; res->n_instances += inst[t]; }
    double t1 = now();
    res->seconds[ORACLE_T_PARSE] = t1 - t0;

    k2.resize(T);
    parallel(T, [&](int s) {
      size_t total = 0;
      for (int t = 0; t < T; ++t) total += out[t][s].size();
      k2[s].init(total / 4 + 16);
      for (int t = 0; t < T; ++t) {
        for (auto &x : out[t][s]) {
          bool ins;
          uint32_t &c = k2[s].get(K2Key<W>{x.first, x.second}, &ins);
          ++c;  /* insert with 1 or increment: no saturation, uint32 (:1120-1132) */
        }
        std::vector<std::pair<W, uint8_t>>().swap(out[t][s]);
      }
    });
    res->n_k2 = 0;   /* the distinct (k+2)-mer entries, whether or not the table is kept */
    for (int s = 0; s < T; ++s) res->n_k2 += k2[s].live;
    res->seconds[ORACLE_T_COUNT_K2] = now() - t1;
    return true;
  }

  /* ================================================== filter and insert nodes */
  /* local_insert_by_freqencies (debruijn_graph_map.hpp:1258-1623) per shard. */
  void filter_insert() {
    double t0 = now();
    nodes.resize(T);
    filtered.resize(T);
    std::vector<std::array<uint64_t, 16>> hist(T);
    parallel(T, [&](int s) {
      hist[s].fill(0);
      /* step 2: to_vector (:1268-1270) */
      std::vector<std::pair<K2Key<W>, uint32_t>> v;
      v.reserve(k2[s].live);
      for (size_t i = 0; i < k2[s].keys.size(); ++i)
        if (k2[s].state[i] == 1) v.emplace_back(k2[s].keys[i], k2[s].vals[i]);
      /* step 3: sort by k-mer (:1275-1279).  The edge is a secondary key only to make the
       * oracle's own output order deterministic; every per-block quantity is a sum. */
      std::sort(v.begin(), v.end(), [](const std::pair<K2Key<W>, uint32_t> &a, const std::pair<K2Key<W>, uint32_t> &b) {
        return a.first.kmer < b.first.kmer || (a.first.kmer == b.first.kmer && a.first.edge < b.first.edge);
      });
      nodes[s].init(v.size() / 2 + 16);
      std::vector<unsigned char> flag(v.size(), 0);
      const uint64_t t0_lo = cfg.thresh[0], t0_hi = cfg.thresh[1], t1_lo = cfg.thresh[2],
                     t1_hi = cfg.thresh[3], t2_lo = cfg.thresh[4], t2_hi = cfg.thresh[5];
      const uint64_t cnt_max = 0xFFFF;  /* FreqType = uint16 */
      if (cfg.thresholding) {
        size_t b = 0;
        while (b < v.size()) {
          size_t e = b;
          W km = v[b].first.kmer;
          while (e < v.size() && v[e].first.kmer == km) ++e;
          /* step 4: per-block sums (:1460-1507) */
          const bool kpal = is_rc_palindrome(km), high = km1_high(km), low = km1_low(km);
          uint64_t k_f = 0, k1in[4] = {0, 0, 0, 0}, k1out[4] = {0, 0, 0, 0};
          for (size_t i = b; i < e; ++i) {
            uint64_t c = v[i].second;
            uint8_t ed = v[i].first.edge;
            k_f += c;
            unsigned ch = ed >> 4;
            if (ch > 0) {
              ch = from_dna16(ch);
              bool split = k1pal_in(ch, km, high) && !kpal;
              k1in[ch] += split ? ((c + 1) >> 1) : c;
            }
            ch = ed & 0xFu;
            if (ch > 0) {
              ch = from_dna16(ch);
              bool split = k1pal_out(km, ch, low) && !kpal;
              k1out[ch] += split ? ((c + 1) >> 1) : c;
            }
          }
          /* caps (:1401-1407) */
          k_f = std::min(cnt_max, k_f);
          for (int c = 0; c < 4; ++c) { k1in[c] = std::min(cnt_max, k1in[c]); k1out[c] = std::min(cnt_max, k1out[c]); }
          /* step 5: per-entry flags (:1410-1448) */
          for (size_t i = b; i < e; ++i) {
            uint64_t cnt = std::min(cnt_max, (uint64_t)v[i].second);
            unsigned char f = 0;
            if (cnt < t2_lo || cnt >= t2_hi) f |= 4;
            if (k_f < t0_lo || k_f >= t0_hi) f |= 8;
            uint8_t ed = v[i].first.edge;
            uint64_t k1;
            switch (ed & 0xF0) {
              case 0x10: k1 = k1in[0]; break; case 0x20: k1 = k1in[1]; break;
              case 0x40: k1 = k1in[2]; break; case 0x80: k1 = k1in[3]; break;
              default: k1 = t1_hi; break;
            }
            if (k1 < t1_lo || k1 >= t1_hi) f |= 2;
            switch (ed & 0x0F) {
              case 0x01: k1 = k1out[0]; break; case 0x02: k1 = k1out[1]; break;
              case 0x04: k1 = k1out[2]; break; case 0x08: k1 = k1out[3]; break;
              default: k1 = t1_hi; break;
            }
            if (k1 < t1_lo || k1 >= t1_hi) f |= 1;
            flag[i] = f;
          }
          b = e;
        }
      }
      /* step 6: modify and compact (:1563-1594); flag 1 drops the out edge, 2 the in edge */
      std::vector<std::pair<K2Key<W>, uint32_t>> kept;
      kept.reserve(v.size());
      for (size_t i = 0; i < v.size(); ++i) {
        unsigned char f = flag[i];
        ++hist[s][f];
        if (f < 3) {
          auto x = v[i];
          if (f == 1) x.first.edge &= 0xF0;
          if (f == 2) x.first.edge &= 0x0F;
          kept.push_back(x);
        }
      }
      /* step 7: local_insert, frequency overload (:256-285): cap at FreqType max */
      for (auto &x : kept) {
        if (x.second == 0) continue;
        bool ins;
        Node &nd = nodes[s].get(KmerKey<W>{x.first.kmer}, &ins);
        node_update(nd, x.first.edge, (uint16_t)std::min<uint64_t>(cnt_max, x.second));
      }
      if (cfg.keep_filtered) filtered[s].swap(kept);
      if (!cfg.keep_k2) { OAMap<K2Key<W>, uint32_t> e2; std::swap(e2, k2[s]); }
    });
    for (int s = 0; s < T; ++s)
      for (int f = 0; f < 16; ++f) res->filter_flag_hist[f] += hist[s][f];
    res->seconds[ORACLE_T_FILTER_INSERT] = now() - t0;
  }

  /* =========================================================== chain extraction */
  /* debruijn_chain_graph::extract_chains (debruijn_chain_graph.hpp:604-667) with
   * to_simple_biedge (debruijn_chain_node.hpp:83-111), then setup_chain_termini (:485-596)
   * applying terminus_update (debruijn_chain_operations.hpp:57-93) through lex_less. */
  void extract_chains() {
    double t0 = now();
    chain.resize(T);
    std::vector<uint64_t> nb(T, 0), nc(T, 0);
    parallel(T, [&](int s) {
      chain[s].init(nodes[s].live / 2 + 16);
      for (size_t i = 0; i < nodes[s].keys.size(); ++i) {
        if (nodes[s].state[i] != 1) continue;
        W x = nodes[s].keys[i].v;
        const Node &n = nodes[s].vals[i];
        if (is_branch(x, n)) ++nb[s];
        if (!is_chain(x, n)) continue;
        ChainNode<W> cn{W(0), W(0), term_mask, term_mask, SideLog<W>(), SideLog<W>()};
        for (unsigned c = 0; c < 4; ++c)
          if (n.c[4 + c] > 0) { cn.inK = ko.next_reverse_from_char(x, c); cn.inD = 1; }
        for (unsigned c = 0; c < 4; ++c)
          if (n.c[c] > 0) { cn.outK = ko.next_from_char(x, c); cn.outD = 1; }
        bool ins;
        chain[s].get(KmerKey<W>{x}, &ins) = cn;
        ++nc[s];
      }
    });
    for (int s = 0; s < T; ++s) { res->n_branch += nb[s]; res->n_chain_nodes += nc[s]; }
    /* terminus updates: (neighbour, (branch, IN)) for out-neighbours, (neighbour, (branch,
     * OUT)) for in-neighbours; lex_less flips k-mer and orientation for non-canonical keys
     * (debruijn_chain_operations.hpp:494-497). */
    std::vector<std::vector<std::vector<std::pair<W, int>>>> upd(T, std::vector<std::vector<std::pair<W, int>>>(T));
    parallel(T, [&](int s) {
      for (size_t i = 0; i < nodes[s].keys.size(); ++i) {
        if (nodes[s].state[i] != 1) continue;
        W x = nodes[s].keys[i].v;
        const Node &n = nodes[s].vals[i];
        if (!is_branch(x, n)) continue;
        for (unsigned c = 0; c < 4; ++c) if (n.c[c] > 0) {
          W nbk = ko.next_from_char(x, c); int o = -1;      /* OUT neighbour gets IN */
          W y = ko.rc(nbk); if (!(nbk < y)) { nbk = y; o = -o; }
          upd[s][shard(nbk)].emplace_back(nbk, o);
        }
        for (unsigned c = 0; c < 4; ++c) if (n.c[4 + c] > 0) {
          W nbk = ko.next_reverse_from_char(x, c); int o = 1; /* IN neighbour gets OUT */
          W y = ko.rc(nbk); if (!(nbk < y)) { nbk = y; o = -o; }
          upd[s][shard(nbk)].emplace_back(nbk, o);
        }
      }
    });
    parallel(T, [&](int d) {
      for (int s = 0; s < T; ++s)
        for (auto &u : upd[s][d]) {
          ChainNode<W> *cn = chain[d].find(KmerKey<W>{u.first});
          if (!cn) continue;                 /* update only existing chain nodes */
          if (u.second < 0) cn->inD = 0; else cn->outD = 0;   /* branch_neighbor */
        }
    });
    res->seconds[ORACLE_T_CHAINMAP] = now() - t0;
  }

  /* ================================================================ list ranking */
  struct Update { W key; W kmer; uint32_t dist; int orient; };

  /* PointsToInternalNode (debruijn_chain_filters.hpp:169-186) */
  static bool unfinished(const ChainNode<W> &c) {
    return points_to_chain_node(c.inD) || points_to_chain_node(c.outD);
  }
  /* IsCycleNode (debruijn_chain_filters.hpp:189-213) */
  static bool is_cycle(const ChainNode<W> &c, uint32_t maxd) {
    return get_chain_dist(c.inD) == maxd && get_chain_dist(c.outD) == maxd;
  }

  /* order of updates in the max reduction: distance first, then the terminal mark */
  static uint64_t update_rank(uint32_t dword) {
    return ((uint64_t)get_chain_dist(dword) << 1) | (dword >> 31);
  }

  /* chain_update (debruijn_chain_operations.hpp:107-256), applied after lex_less has put
   * the update on the key's canonical strand. */
  static size_t chain_update(ChainNode<W> &x, const Update &y) {
    uint32_t dist = get_chain_dist(y.dist);
    if (y.orient < 0) {
      if (points_to_chain_node(x.inD)) {
        uint32_t dx = get_chain_dist(x.inD);
        if (dist > dx) x.inK = y.kmer;
        if (dist >= dx) { x.inD = y.dist; return 1; }
      }
    } else {
      if (points_to_chain_node(x.outD)) {
        uint32_t dx = get_chain_dist(x.outD);
        if (dist > dx) x.outK = y.kmer;
        if (dist >= dx) { x.outD = y.dist; return 1; }
      }
    }
    return 0;
  }

  /* list_rank_min_update (debruijn_chain_graph.hpp:1040-1310) when cfg.min_update,
   * list_rank (:793-994) otherwise.  Round-synchronous: every update of a round is made
   * from the state at the start of the round, then all are applied. */
  void list_rank() {
    double t0 = now();
    std::vector<std::vector<W>> unf(T);
    parallel(T, [&](int s) {
      for (size_t i = 0; i < chain[s].keys.size(); ++i)
        if (chain[s].state[i] == 1 && unfinished(chain[s].vals[i])) unf[s].push_back(chain[s].keys[i].v);
      std::sort(unf[s].begin(), unf[s].end());
    });
    size_t total_unf = 0;
    for (int s = 0; s < T; ++s) total_unf += unf[s].size();
    bool all_compacted = total_unf == 0;
    uint64_t iterations = 0;
    std::vector<std::vector<std::vector<Update>>> upd(T, std::vector<std::vector<Update>>(T));
    std::vector<uint64_t> cnt(T), cyc(T), col(T), left(T);
    while (!all_compacted) {
      const uint32_t round = (uint32_t)iterations;
      parallel(T, [&](int s) {
        for (int d = 0; d < T; ++d) upd[s][d].clear();
        for (W km : unf[s]) {
          const ChainNode<W> md = *chain[s].find(KmerKey<W>{km});
          uint32_t ldist = md.inD, rdist = md.outD;
          uint32_t dist = get_chain_dist(ldist) + get_chain_dist(rdist);
          bool send_l = cfg.min_update ? points_to_chain_node(ldist) : !is_chain_terminal(ldist);
          bool send_r = cfg.min_update ? points_to_chain_node(rdist) : !is_chain_terminal(rdist);
          if (send_l) {   /* send rr to ll, orientation OUT */
            Update u{md.inK, is_chain_terminal(rdist) ? km : md.outK,
                     points_to_chain_node(rdist) ? dist : mark_terminal(dist), 1};
            W y = ko.rc(u.key);
            if (!(u.key < y)) { u.key = y; u.kmer = ko.rc(u.kmer); u.orient = -u.orient; }
            upd[s][shard(u.key)].push_back(u);
          }
          if (send_r) {   /* send ll to rr, orientation IN */
            Update u{md.outK, is_chain_terminal(ldist) ? km : md.inK,
                     points_to_chain_node(ldist) ? dist : mark_terminal(dist), -1};
            W y = ko.rc(u.key);
            if (!(u.key < y)) { u.key = y; u.kmer = ko.rc(u.kmer); u.orient = -u.orient; }
            upd[s][shard(u.key)].push_back(u);
          }
        }
      });
      parallel(T, [&](int d) {
        uint64_t c = 0, cl = 0;
        std::vector<std::pair<ChainNode<W> *, int>> multi;
        for (int s = 0; s < T; ++s)
          for (const Update &u : upd[s][d]) {
            ChainNode<W> *x = chain[d].find(KmerKey<W>{u.key});
            if (!x) continue;                  /* updates to absent keys are dropped */
            SideLog<W> &lg = u.orient < 0 ? x->log_in : x->log_out;
            if (lg.round != round) {
              lg.round = round; lg.n = 0;
              lg.snapK = u.orient < 0 ? x->inK : x->outK;
              lg.snapD = u.orient < 0 ? x->inD : x->outD;
              lg.bestK = u.kmer; lg.bestD = u.dist;
            } else if (update_rank(u.dist) > update_rank(lg.bestD)) {
              lg.bestK = u.kmer; lg.bestD = u.dist;
            }
            if (++lg.n == 2) multi.emplace_back(x, u.orient);
            c += chain_update(*x, u);
          }
        for (auto &m : multi) {
          ChainNode<W> tmp = *m.first;
          const SideLog<W> &lg = m.second < 0 ? tmp.log_in : tmp.log_out;
          if (m.second < 0) { tmp.inK = lg.snapK; tmp.inD = lg.snapD; }
          else { tmp.outK = lg.snapK; tmp.outD = lg.snapD; }
          chain_update(tmp, Update{W(0), lg.bestK, lg.bestD, m.second});
          bool same = m.second < 0 ? (tmp.inK == m.first->inK && tmp.inD == m.first->inD)
                                   : (tmp.outK == m.first->outK && tmp.outD == m.first->outD);
          if (!same) ++cl;
        }
        cnt[d] = c; col[d] = cl;
      });
      ++iterations;
      const uint32_t maxd = 0x1u << iterations;
      parallel(T, [&](int s) {
        std::vector<W> keep;
        uint64_t cy = 0;
        for (W km : unf[s]) {
          const ChainNode<W> &x = *chain[s].find(KmerKey<W>{km});
          if (unfinished(x)) { keep.push_back(km); cy += is_cycle(x, maxd); }
        }
        unf[s].swap(keep);
        cyc[s] = cy; left[s] = unf[s].size();
      });
      uint64_t count = 0, cycles = 0, remaining = 0;
      for (int s = 0; s < T; ++s) { count += cnt[s]; cycles += cyc[s]; remaining += left[s]; res->collisions += col[s]; }
      if (iterations >= 30) all_compacted = true;
      else all_compacted = (count == 0) || (cycles == remaining);
    }
    res->iterations = iterations;

    /* separate_cycles(iterations) when anything is still unfinished (:1283-1292, :670-705),
     * then separate_isolated (:744-777). */
    bool any_unfinished = false;
    for (int s = 0; s < T; ++s)
      for (size_t i = 0; i < chain[s].keys.size(); ++i)
        if (chain[s].state[i] == 1 && unfinished(chain[s].vals[i])) any_unfinished = true;
    std::vector<uint64_t> ncy(T, 0), niso(T, 0);
    std::vector<std::vector<W>> cyk(T);
    std::vector<std::vector<std::pair<W, ChainNode<W>>>> isok(T);
    const uint32_t maxd = 0x1u << iterations;
    parallel(T, [&](int s) {
      for (size_t i = 0; i < chain[s].keys.size(); ++i) {
        if (chain[s].state[i] != 1) continue;
        if (any_unfinished && is_cycle(chain[s].vals[i], maxd)) {
          cyk[s].push_back(chain[s].keys[i].v);
          chain[s].erase_slot(i);
          ++ncy[s];
        }
      }
      for (size_t i = 0; i < chain[s].keys.size(); ++i) {
        if (chain[s].state[i] != 1) continue;
        const ChainNode<W> &x = chain[s].vals[i];
        if (points_to_self(x.inD) && points_to_self(x.outD)) {
          isok[s].push_back({chain[s].keys[i].v, x});
          chain[s].erase_slot(i);
          ++niso[s];
        }
      }
    });
    for (int s = 0; s < T; ++s) { res->n_cycle_nodes += ncy[s]; res->n_isolated += niso[s]; }
    cycle_kmers.clear();
    for (int s = 0; s < T; ++s) cycle_kmers.insert(cycle_kmers.end(), cyk[s].begin(), cyk[s].end());
    isolated_recs.clear();
    for (int s = 0; s < T; ++s) isolated_recs.insert(isolated_recs.end(), isok[s].begin(), isok[s].end());
    res->seconds[ORACLE_T_LIST_RANK] = now() - t0;
  }

  /* ============================================================== emission */
  struct Ranked { W K, rep; int32_t dist; };

  /* to_ranked_chain_nodes (debruijn_chain_graph.hpp:1760-1773) with to_listranked_chain_node
   * (debruijn_chain_operations.hpp:260-309); to_compressed_chains (:1778-1856) groups by
   * rep after sorting with chain_rep_less (:332-340) and prints each group with
   * print_chain_as_fasta(chain_only) (:359-384). */
  void emit() {
    double t0 = now();
    std::vector<std::vector<Ranked>> part(T);
    parallel(T, [&](int s) {
      for (size_t i = 0; i < chain[s].keys.size(); ++i) {
        if (chain[s].state[i] != 1) continue;
        W key = chain[s].keys[i].v;
        const ChainNode<W> &x = chain[s].vals[i];
        W L = is_chain_terminal(x.inD) ? key : x.inK;
        W R = is_chain_terminal(x.outD) ? ko.rc(key) : ko.rc(x.outK);
        bool sense = L <= R;
        part[s].push_back({sense ? key : ko.rc(key), sense ? L : R,
                           (int32_t)(sense ? get_chain_dist(x.inD) : get_chain_dist(x.outD))});
      }
    });
    std::vector<Ranked> rk;
    for (int s = 0; s < T; ++s) { rk.insert(rk.end(), part[s].begin(), part[s].end()); std::vector<Ranked>().swap(part[s]); }
    std::vector<Ranked> byrep(rk);
    par_sort(byrep, [](const Ranked &a, const Ranked &b) {
      if (a.rep != b.rep) return a.rep < b.rep;
      if (std::abs(a.dist) != std::abs(b.dist)) return std::abs(a.dist) < std::abs(b.dist);
      return a.K < b.K;
    }, T);
    std::string chars;
    std::vector<W> reps;
    std::vector<uint64_t> offs;
    for (size_t i = 0; i < byrep.size(); ++i) {
      if (i == 0 || byrep[i].rep != byrep[i - 1].rep) { reps.push_back(byrep[i].rep); offs.push_back(chars.size()); }
      if (byrep[i].dist == 0) chars += ko.ascii(byrep[i].rep);
      else chars += "ACGT"[ko.last(byrep[i].K)];
    }
    offs.push_back(chars.size());
    par_sort(rk, [](const Ranked &a, const Ranked &b) { return a.K < b.K; }, T);

    const int w = res->words;
    res->n_ranked = rk.size();
    res->ranked_K = (uint64_t *)calloc(rk.size() * w + 1, 8);
    res->ranked_rep = (uint64_t *)calloc(rk.size() * w + 1, 8);
    res->ranked_dist = (int32_t *)calloc(rk.size() + 1, 4);
    for (size_t i = 0; i < rk.size(); ++i) {
      store_word(res->ranked_K + i * w, rk[i].K, w);
      store_word(res->ranked_rep + i * w, rk[i].rep, w);
      res->ranked_dist[i] = rk[i].dist;
    }
    res->n_chains = reps.size();
    res->chain_rep = (uint64_t *)calloc(reps.size() * w + 1, 8);
    res->chain_offsets = (uint64_t *)calloc(offs.size() + 1, 8);
    res->chain_chars = (char *)malloc(chars.size() + 1);
    for (size_t i = 0; i < reps.size(); ++i) store_word(res->chain_rep + i * w, reps[i], w);
    for (size_t i = 0; i < offs.size(); ++i) res->chain_offsets[i] = offs[i];
    memcpy(res->chain_chars, chars.data(), chars.size());
    res->chain_chars[chars.size()] = 0;
    res->seconds[ORACLE_T_COMPRESS] = now() - t0;
  }

  /* ================================================== chain end edges
   * The records print_chain_frequencies (compact_dbg_stats.hpp:879-1065) prints, with the
   * frequency summaries of compute_freq_map (:783-816):
   *   - freq_map: every listranked node adds (1, f, f, f) under its chain representative,
   *     f = get_self_frequency of its canonical k-mer; keys are canonical
   *     (CanonicalHashMapParams), summaries reduce as freq_summary
   *     (debruijn_chain_operations.hpp:447-459): count and sum add, min, max;
   *   - chain_rep: the chain-map nodes IsCanonicalTerminusOrIsolated accepts
   *     (debruijn_chain_filters.hpp:125-147);
   *   - per selected node, L and R on one strand (:947-962), L's in-edges and R's out-edges
   *     taken from the canonical k-mer's counters, reversed and complemented when the end is
   *     not canonical (:973-1007), and the summary of canonical(L) with the mean as
   *     (float)sum / (float)count stored in the count type (:1009-1013);
   *   - records sorted by L (:1019-1029).
   * A chain end that is not a graph node (possible only when chain pointers are not mutually
   * consistent) gets zero counts, where the reference's lookup would fail. */
  struct FreqSum { uint64_t count = 0, sum = 0; uint16_t mn = 0xFFFF, mx = 0; };
  struct EdgeRec { W L, R; uint16_t f[11]; };

  Node *node_of(W canon) { return nodes[shard(canon)].find(KmerKey<W>{canon}); }
  W canon_of(W x) const { W y = ko.rc(x); return x < y ? x : y; }

  void chain_edges() {
    OAMap<KmerKey<W>, FreqSum> freq;
    for (int s = 0; s < T; ++s)
      for (size_t i = 0; i < chain[s].keys.size(); ++i) {
        if (chain[s].state[i] != 1) continue;
        const W key = chain[s].keys[i].v;
        const ChainNode<W> &x = chain[s].vals[i];
        const W L = is_chain_terminal(x.inD) ? key : x.inK;
        const W R = is_chain_terminal(x.outD) ? ko.rc(key) : ko.rc(x.outK);
        const W rep = L <= R ? L : R;
        const Node *nd = node_of(key);
        const uint16_t f = nd ? nd->c[8] : 0;
        bool ins;
        FreqSum &q = freq.get(KmerKey<W>{canon_of(rep)}, &ins);
        q.count += 1; q.sum += f;
        q.mn = std::min(q.mn, f); q.mx = std::max(q.mx, f);
      }
    std::vector<EdgeRec> out;
    for (int s = 0; s < T; ++s)
      for (size_t i = 0; i < chain[s].keys.size(); ++i) {
        if (chain[s].state[i] != 1) continue;
        const W K = chain[s].keys[i].v;
        const ChainNode<W> &x = chain[s].vals[i];
        const bool ti = is_chain_terminal(x.inD), to = is_chain_terminal(x.outD);
        EdgeRec e;
        if (ti && to) { e.L = K; e.R = K; }
        else if (ti) { if (!(K <= ko.rc(x.outK))) continue; e.L = K; e.R = x.outK; }
        else if (to) { if (!(ko.rc(K) < x.inK)) continue; e.L = ko.rc(K); e.R = ko.rc(x.inK); }
        else continue;
        const W cL = canon_of(e.L), cR = canon_of(e.R);
        const Node *nl = node_of(cL), *nr = node_of(cR);
        for (int b = 0; b < 4; ++b) {
          e.f[b] = !nl ? 0 : (cL == e.L ? nl->c[4 + b] : nl->c[3 - b]);
          e.f[4 + b] = !nr ? 0 : (cR == e.R ? nr->c[b] : nr->c[7 - b]);
        }
        const FreqSum *q = freq.find(KmerKey<W>{cL});
        if (q && q->count) {
          e.f[8] = (uint16_t)(static_cast<float>(q->sum) / static_cast<float>(q->count));
          e.f[9] = q->mn; e.f[10] = q->mx;
        } else {
          e.f[8] = e.f[9] = e.f[10] = 0;
        }
        out.push_back(e);
      }
    std::sort(out.begin(), out.end(), [](const EdgeRec &a, const EdgeRec &b) { return a.L < b.L; });
    const int w = res->words;
    res->n_chain_edges = out.size();
    res->edge_L = (uint64_t *)calloc(out.size() * w + 1, 8);
    res->edge_R = (uint64_t *)calloc(out.size() * w + 1, 8);
    res->edge_freqs = (uint16_t *)calloc(out.size() * 11 + 1, 2);
    for (size_t i = 0; i < out.size(); ++i) {
      store_word(res->edge_L + i * w, out[i].L, w);
      store_word(res->edge_R + i * w, out[i].R, w);
      memcpy(res->edge_freqs + i * 11, out[i].f, 22);
    }
  }

  /* ================================================== chain summaries
   * to_summarized_chains() (debruijn_chain_graph.hpp:1876-2005): the chain-map termini
   * (IsTerminusOrIsolated, debruijn_chain_filters.hpp:84-92) sorted by get_chain_rep
   * (debruijn_chain_operations.hpp:512-522); a terminus terminal on both sides makes a
   * summary with itself, two consecutive termini with one representative make one summary
   * oriented so that the 5' terminus is the representative (the four cases of :1937-2000);
   * make_summarized_chain and transform::reverse_complement (debruijn_chain_node.hpp:201-268):
   * (prev at 5', 5', 3', next at 3', dist of the 5' node, 5' and 3' ends point to a branch).
   * The single-rank run: no left shift from a next rank.  A case the reference throws on
   * leaves summaries_ok = 0. */
  struct Term { W K; ChainNode<W> x; };
  struct Summary { W prev, t5, t3, next; uint32_t dist; uint8_t f5, f3; };

  W chain_rep_of(const Term &t) const {
    const W L = is_chain_terminal(t.x.inD) ? t.K : t.x.inK;
    const W R = is_chain_terminal(t.x.outD) ? ko.rc(t.K) : ko.rc(t.x.outK);
    return L <= R ? L : R;
  }
  Term rc_term(const Term &t) const {   /* (K, biedge) -> (rc K, reverse_complement(biedge)) */
    Term r = t;
    r.K = ko.rc(t.K);
    r.x.inK = ko.rc(t.x.outK); r.x.outK = ko.rc(t.x.inK);
    r.x.inD = t.x.outD; r.x.outD = t.x.inD;
    return r;
  }
  Summary make_summary(const Term &f, const Term &s) const {
    return Summary{f.x.inK, f.K, s.K, s.x.outK, get_chain_dist(f.x.inD) + get_chain_dist(f.x.outD),
                   (uint8_t)(points_to_self(f.x.inD) ? 0 : 1), (uint8_t)(points_to_self(s.x.outD) ? 0 : 1)};
  }

  void chain_summaries() {
    std::vector<Term> termini;
    for (int s = 0; s < T; ++s)
      for (size_t i = 0; i < chain[s].keys.size(); ++i) {
        if (chain[s].state[i] != 1) continue;
        const ChainNode<W> &x = chain[s].vals[i];
        if (is_chain_terminal(x.inD) || is_chain_terminal(x.outD)) termini.push_back({chain[s].keys[i].v, x});
      }
    std::vector<std::pair<W, size_t>> order;
    for (size_t i = 0; i < termini.size(); ++i) order.emplace_back(chain_rep_of(termini[i]), i);
    std::sort(order.begin(), order.end(), [](const std::pair<W, size_t> &a, const std::pair<W, size_t> &b) {
      return a.first < b.first || (a.first == b.first && a.second < b.second);
    });
    std::vector<Summary> out;
    bool ok = true;
    auto both = [](const Term &t) { return is_chain_terminal(t.x.inD) && is_chain_terminal(t.x.outD); };
    if (!order.empty()) {
      Term first = termini[order[0].second];
      W first_rep = order[0].first;
      if (both(first)) out.push_back(make_summary(first, first));
      for (size_t i = 1; i < order.size() && ok; ++i) {
        const W rep = order[i].first;
        if (rep != first_rep) {
          first = termini[order[i].second];
          first_rep = rep;
          if (both(first)) out.push_back(make_summary(first, first));
          continue;
        }
        const Term &second = termini[order[i].second];
        const bool f2 = is_chain_terminal(first.x.inD), f3 = is_chain_terminal(first.x.outD);
        const bool s2 = is_chain_terminal(second.x.inD), s3 = is_chain_terminal(second.x.outD);
        if (f2 && s3) {
          if (first.K == rep) out.push_back(make_summary(first, second));
          else if (ko.rc(second.K) == rep) out.push_back(make_summary(rc_term(second), rc_term(first)));
          else ok = false;
        } else if (f2 && s2) {
          if (first.K == rep) out.push_back(make_summary(first, rc_term(second)));
          else if (second.K == rep) out.push_back(make_summary(second, rc_term(first)));
          else ok = false;
        } else if (f3 && s3) {
          if (ko.rc(first.K) == rep) out.push_back(make_summary(rc_term(first), second));
          else if (ko.rc(second.K) == rep) out.push_back(make_summary(rc_term(second), first));
          else ok = false;
        } else if (f3 && s2) {
          if (ko.rc(first.K) == rep) out.push_back(make_summary(rc_term(first), rc_term(second)));
          else if (second.K == rep) out.push_back(make_summary(second, first));
          else ok = false;
        } else {
          ok = false;
        }
      }
    }
    const int w = res->words;
    res->summaries_ok = ok ? 1 : 0;
    if (!ok) out.clear();
    res->n_summaries = out.size();
    res->sum_kmers = (uint64_t *)calloc(out.size() * 4 * w + 1, 8);
    res->sum_dist = (uint32_t *)calloc(out.size() + 1, 4);
    res->sum_flags = (uint8_t *)calloc(out.size() * 2 + 1, 1);
    for (size_t i = 0; i < out.size(); ++i) {
      store_word(res->sum_kmers + (i * 4 + 0) * w, out[i].prev, w);
      store_word(res->sum_kmers + (i * 4 + 1) * w, out[i].t5, w);
      store_word(res->sum_kmers + (i * 4 + 2) * w, out[i].t3, w);
      store_word(res->sum_kmers + (i * 4 + 3) * w, out[i].next, w);
      res->sum_dist[i] = out[i].dist;
      res->sum_flags[2 * i] = out[i].f5;
      res->sum_flags[2 * i + 1] = out[i].f3;
    }
  }


  /* ================================================== graph cleaning
   * clean_deadend_and_bubbles_naive (compact_dbg_clean.hpp:575-890), the cleaning of the
   * _freq_clean driver (compact_dbg_freq_construct_clean.cpp:633-700), on one rank. */
  static bool single16(unsigned n) { return n != 0 && (n & (n - 1)) == 0; }
  static uint16_t in_total(const Node &n) {   /* get_in_edge_total_frequency (debruijn_graph_node.hpp:307-313) */
    uint16_t t = 0;
    for (int c = 4; c < 8; ++c) t = sat_add(t, n.c[c]);
    return t;
  }
  static uint16_t out_total(const Node &n) {  /* get_out_edge_total_frequency (:299-305) */
    uint16_t t = 0;
    for (int c = 0; c < 4; ++c) t = sat_add(t, n.c[c]);
    return t;
  }
  static bool no_edges(const Node &n) {     /* graph::IsIsolated (debruijn_graph_filters.hpp:163-172) */
    for (int c = 0; c < 8; ++c) if (n.c[c]) return false;
    return true;
  }

  /* idx.erase_if(IsIsolated): nodes without any edge leave the graph */
  void erase_isolated() {
    parallel(T, [&](int s) {
      for (size_t i = 0; i < nodes[s].keys.size(); ++i)
        if (nodes[s].state[i] == 1 && no_edges(nodes[s].vals[i])) nodes[s].erase_slot(i);
    });
  }

  /* erase_simple_biedges (debruijn_graph_map.hpp:600-608): each (k-mer, DNA16 biedge) put on
   * the canonical strand (transform_input), then compact_multi_biedge::erase (debruijn_graph_node.hpp
   * :223-226) zeroes the count of each single-character nibble; the self count stays. */
  void erase_simple(const std::vector<std::pair<W, uint8_t>> &q) {
    for (auto e : q) {
      W x = e.first; uint8_t ed = e.second;
      canonical(x, ed);
      Node *n = node_of(x);
      if (!n) continue;
      const unsigned out = from_dna16(ed & 0xFu), in = from_dna16(ed >> 4);
      if (out < 4) n->c[out] = 0;
      if (in < 4) n->c[4 + in] = 0;
    }
  }

  /* get_remote_edges for simple biedges (:475-510): the same edge seen from the other end.
   * An in-nibble c of x is the edge from c.x[0..k-2] whose out-nibble is x's last character;
   * an out-nibble c is the edge to x[1..k-1].c whose in-nibble is x's first character. */
  std::vector<std::pair<W, uint8_t>> remote_simple(const std::vector<std::pair<W, uint8_t>> &q) const {
    std::vector<std::pair<W, uint8_t>> r;
    for (auto e : q) {
      const unsigned in = e.second >> 4, out = e.second & 0xFu;
      if (single16(in))
        r.emplace_back(ko.next_reverse_from_char(e.first, from_dna16(in)), (uint8_t)(1u << ko.last(e.first)));
      if (single16(out))
        r.emplace_back(ko.next_from_char(e.first, from_dna16(out)), (uint8_t)((1u << ko.first(e.first)) << 4));
    }
    return r;
  }

  /* get_remote_edges for whole nodes (:440-471): every in- and out-neighbour's edge back */
  void remote_multi(W x, const Node &n, std::vector<std::pair<W, uint8_t>> &r) const {
    for (unsigned c = 0; c < 4; ++c)
      if (n.c[4 + c] > 0) r.emplace_back(ko.next_reverse_from_char(x, c), (uint8_t)(1u << ko.last(x)));
    for (unsigned c = 0; c < 4; ++c)
      if (n.c[c] > 0) r.emplace_back(ko.next_from_char(x, c), (uint8_t)((1u << ko.first(x)) << 4));
  }

  /* erase_nodes(kmers) (:833-836 -> erase_nodes_and_edges :811-827): the nodes found leave
   * the graph, then their neighbours lose the edges back to them */
  void erase_graph_nodes(const std::vector<W> &kmers) {
    std::vector<std::pair<W, Node>> found;
    for (W x : kmers) {
      W y = ko.rc(x), key = x < y ? x : y;
      OAMap<KmerKey<W>, Node> &m = nodes[shard(key)];
      Node *n = m.find(KmerKey<W>{key});
      if (n) found.emplace_back(key, *n);
    }
    for (auto &f : found) {
      OAMap<KmerKey<W>, Node> &m = nodes[shard(f.first)];
      Node *n = m.find(KmerKey<W>{f.first});
      if (n) m.erase_slot((size_t)(n - m.vals.data()));
    }
    std::vector<std::pair<W, uint8_t>> rev;
    for (auto &f : found) remote_multi(f.first, f.second, rev);
    erase_simple(rev);
  }

  /* erase_edges(query, edge_freq_filter) (:770-775): find_edges with the predicate (:615-660)
   * keeps, per query, the single-character nibbles whose edge exists with a count below
   * min_freq (compact_multi_biedge::select, debruijn_graph_node.hpp:240-247), all looked up
   * before anything is erased; then the reverse edges and the edges themselves are erased
   * (erase_edges_internal, :737-747).  Returns the number of query edges kept. */
  uint64_t erase_low_edges(std::vector<std::pair<W, uint8_t>> q, uint32_t min_freq) {
    std::vector<std::pair<W, uint8_t>> found;
    for (auto &e : q) {
      W x = e.first; uint8_t ed = e.second;
      canonical(x, ed);
      const Node *n = node_of(x);
      if (!n) continue;
      const unsigned in = ed >> 4, out = ed & 0xFu;
      auto sel = [&](uint16_t v) { return (uint32_t)v < min_freq ? v : (uint16_t)0; };
      if (single16(in) && sel(n->c[4 + from_dna16(in)]) == 0) ed &= 0x0Fu;
      if (single16(out) && sel(n->c[from_dna16(out)]) == 0) ed &= 0xF0u;
      if (ed > 0) found.emplace_back(x, ed);
    }
    erase_simple(remote_simple(found));
    erase_simple(found);
    return found.size();
  }

  /* summarized_chain<K, uint16> (debruijn_chain_node.hpp:174): prev at 5', 5' terminus (the
   * chain representative), 3' terminus, next at 3', distance between the termini, and the
   * 5' / 3' end-edge frequencies */
  struct FSum { W k0, k1, k2, k3; uint32_t len; uint16_t f5, f6; };

  FSum rc_sum(const FSum &x) const {   /* transform::reverse_complement (debruijn_chain_node.hpp:257-268) */
    return FSum{ko.rc(x.k3), ko.rc(x.k2), ko.rc(x.k1), ko.rc(x.k0), x.len, x.f6, x.f5};
  }

  /* to_summarized_chains(dbg) (debruijn_chain_graph.hpp:2044-2130) over the chain map's
   * termini (IsTerminusOrIsolated): one summary per terminus oriented so that the 5' terminus
   * is the representative, the end edge's frequency the terminus node's total in- or out-edge
   * frequency; sorted by (5' terminus, next at 3'), a unit chain kept as is and two
   * consecutive termini of one chain merged (merge_summarized_chains, debruijn_chain_node.hpp
   * :176-197).  On one rank the left and right shifts deliver value-initialised summaries, so a
   * last summary whose 5' terminus is the all-A k-mer is dropped and a first one with that
   * terminus merges with the empty summary.  False where the reference throws. */
  bool freq_summaries(std::vector<FSum> &out) {
    std::vector<FSum> r;
    for (int s = 0; s < T; ++s)
      for (size_t i = 0; i < chain[s].keys.size(); ++i) {
        if (chain[s].state[i] != 1) continue;
        const ChainNode<W> &x = chain[s].vals[i];
        const W K = chain[s].keys[i].v;
        const bool t5 = is_chain_terminal(x.inD), t3 = is_chain_terminal(x.outD);
        if (!t5 && !t3) continue;
        const Node *n = node_of(K);
        if (!n) return false;
        const uint32_t d = get_chain_dist(x.inD) + get_chain_dist(x.outD);
        if (t5 && t3) {
          r.push_back(FSum{x.inK, K, K, x.outK, d, in_total(*n), out_total(*n)});
        } else if (t5) {
          const W o = ko.rc(x.outK);
          if (K < o) r.push_back(FSum{x.inK, K, x.outK, W(0), d, in_total(*n), 0});
          else if (o < K) r.push_back(FSum{W(0), o, ko.rc(K), ko.rc(x.inK), d, 0, in_total(*n)});
          else return false;
        } else {
          const W o = ko.rc(K);
          if (x.inK < o) r.push_back(FSum{W(0), x.inK, K, x.outK, d, 0, out_total(*n)});
          else if (o < x.inK) r.push_back(FSum{ko.rc(x.outK), o, ko.rc(x.inK), W(0), d, out_total(*n), 0});
          else return false;
        }
      }
    /* the reference's sort compares (5' terminus, next at 3') only; the rest of the record
     * breaks ties here, where merging is order-independent anyway */
    std::sort(r.begin(), r.end(), [](const FSum &a, const FSum &b) {
      if (a.k1 != b.k1) return a.k1 < b.k1;
      if (a.k3 != b.k3) return a.k3 < b.k3;
      if (a.k0 != b.k0) return a.k0 < b.k0;
      if (a.k2 != b.k2) return a.k2 < b.k2;
      if (a.f5 != b.f5) return a.f5 < b.f5;
      return a.f6 < b.f6;
    });
    out.clear();
    if (r.empty()) return true;
    size_t max_pos = r.size();
    if (r.back().k1 == W(0)) --max_pos;
    FSum last{W(0), W(0), W(0), W(0), 0, 0, 0};
    for (size_t pos = 0; pos < max_pos; ++pos) {
      if (r[pos].len == 0) {
        out.push_back(r[pos]);
      } else if (r[pos].k1 == last.k1) {
        FSum m = r[pos];
        if (m.f5 < last.f5) { m.k0 = last.k0; m.f5 = last.f5; }
        if (m.f6 < last.f6) { m.k3 = last.k3; m.f6 = last.f6; }
        out.push_back(m);
      }
      last = r[pos];
    }
    return true;
  }

  /* find_deadends (debruijn_topo_operations.hpp:146-175) with deadend_filter
   * (compact_dbg_clean.hpp:63-80): shorter than max_len, both end-edge frequencies below
   * min_freq, exactly one end without an edge */
  std::vector<FSum> find_deadends(const std::vector<FSum> &sums, uint32_t max_len, uint32_t min_freq) const {
    std::vector<FSum> r;
    for (const FSum &x : sums)
      if (x.len < max_len && x.f5 < min_freq && x.f6 < min_freq && ((x.f5 == 0) != (x.f6 == 0))) r.push_back(x);
    return r;
  }

  /* find_bubbles (debruijn_topo_operations.hpp:285-395) with bubble_filter
   * (compact_dbg_clean.hpp:84-112): chains with both ends on branches (find_normal_chains,
   * :251-272) put on the strand where the 5' branch is not above rc(3' branch), sorted by
   * (5' branch, 3' branch, length), then every run of two or more consecutive chains between
   * the same two branches whose neighbours differ in length by at most 1 and have some end
   * edge below min_freq.  On one rank the redistribution by 5' branch (:320-345) moves nothing
   * that could join or split a run.  Ties of the reference's sort are broken by the termini. */
  std::vector<FSum> find_bubbles(const std::vector<FSum> &sums, uint32_t min_freq) const {
    std::vector<FSum> t;
    for (const FSum &x : sums)
      if (x.len > 0 && x.f5 > 0 && x.f6 > 0) t.push_back(x.k0 > ko.rc(x.k3) ? rc_sum(x) : x);
    std::sort(t.begin(), t.end(), [](const FSum &a, const FSum &b) {
      if (a.k0 != b.k0) return a.k0 < b.k0;
      if (a.k3 != b.k3) return a.k3 < b.k3;
      if (a.len != b.len) return a.len < b.len;
      if (a.k1 != b.k1) return a.k1 < b.k1;
      return a.k2 < b.k2;
    });
    std::vector<FSum> out;
    if (t.empty()) return out;
    auto pred = [&](const FSum &l, const FSum &r) {
      const uint32_t d = l.len > r.len ? l.len - r.len : r.len - l.len;
      return d <= 1 && (l.f5 < min_freq || l.f6 < min_freq || r.f5 < min_freq || r.f6 < min_freq);
    };
    size_t first_i = 0, i = 1;
    FSum prev = t[0];
    for (; i < t.size(); ++i) {
      if (prev.k0 == t[i].k0 && prev.k3 == t[i].k3 && pred(prev, t[i])) { prev = t[i]; continue; }
      if (i - first_i > 1) out.insert(out.end(), t.begin() + first_i, t.begin() + i);
      prev = t[i];
      first_i = i;
    }
    if (i - first_i > 1) out.insert(out.end(), t.begin() + first_i, t.begin() + i);
    return out;
  }

  /* the edges to sever (compact_dbg_clean.hpp:619-640, 687-699): the 5' branch's out-edge to the
   * 5' terminus (its last character) and the 3' branch's in-edge from the 3' terminus (its first
   * character), as DNA16 biedges; a dead end contributes only the end that has an edge */
  void end_edges(const FSum &x, bool only_present, std::vector<std::pair<W, uint8_t>> &q) const {
    if (!only_present || x.f5 > 0) q.emplace_back(x.k0, (uint8_t)(1u << ko.last(x.k1)));
    if (!only_present || x.f6 > 0) q.emplace_back(x.k3, (uint8_t)((1u << ko.first(x.k2)) << 4));
  }

  void reset_graph_counters(oracle_result *r) {
    r->n_branch = r->n_chain_nodes = r->iterations = r->collisions = r->n_cycle_nodes = r->n_isolated = 0;
  }

  void clean() {
    oracle_result *top = res;
    oracle_result *cr = (oracle_result *)calloc(1, sizeof(oracle_result));
    cr->words = top->words;
    top->clean = cr;
    const uint32_t min_freq = (uint32_t)(clean_k1_lo + 1);   /* edge_freq_filter(threshes[2] + 1) */
    const uint32_t max_len = 2u * (uint32_t)ko.k - 1u;       /* deadend_filter(2 * k - 1, ...) */
    /* the driver removes cycle nodes and then edge-less nodes from the graph right after the
     * first list ranking (compact_dbg_freq_construct_clean.cpp:599-604) */
    erase_graph_nodes(cycle_kmers);
    erase_isolated();
    std::vector<FSum> sums;
    if (!freq_summaries(sums)) { top->clean_status = 2; res = top; return; }
    std::vector<FSum> dead = find_deadends(sums, max_len, min_freq), bub = find_bubbles(sums, min_freq);
    res = cr;
    reset_graph_counters(cr);
    while (!dead.empty() || !bub.empty()) {
      top->clean_deadends += dead.size();
      top->clean_bubbles += bub.size();
      std::vector<std::pair<W, uint8_t>> q;
      for (const FSum &x : dead) end_edges(x, true, q);
      uint64_t erased = erase_low_edges(q, min_freq);
      erase_isolated();
      q.clear();
      for (const FSum &x : bub) end_edges(x, false, q);
      erased += erase_low_edges(q, min_freq);
      erase_isolated();
      top->clean_edges += erased;
      ++top->clean_rounds;
      if (erased == 0) { top->clean_status = 1; break; }
      /* recompact: a new chain map from the graph, ranked, cycles and edge-less nodes out */
      reset_graph_counters(cr);
      extract_chains();
      list_rank();
      erase_graph_nodes(cycle_kmers);
      erase_isolated();
      if (!freq_summaries(sums)) { top->clean_status = 2; break; }
      dead = find_deadends(sums, max_len, min_freq);
      bub = find_bubbles(sums, min_freq);
    }
    /* the cleaned graph's outputs */
    emit();
    chain_edges();
    export_tables(true);
    res = top;
  }

  /* ====================================================== check_index
   * test/common/compact_dbg_stats.hpp:45-119, run where the driver runs it after the build
   * (compact_dbg_freq_construct_clean.cpp:515): the neighbours every node's edges name
   * (get_out_neighbors / get_in_neighbors, debruijn_graph_node.hpp:316-381) are counted in the
   * canonical index -- absent ones fail the first check; the index minus every named k-mer minus
   * IsIsolated nodes must be empty -- the second.  Also the edges whose neighbour lacks the edge
   * back, and print_compact_multi_biedge_histogram's in x out histogram (debruijn_stats.hpp:39-74). */
  void check_index() {
    std::vector<uint64_t> q(T, 0), absent(T, 0), unanswered(T, 0);
    std::vector<std::array<uint64_t, 25>> hist(T);
    std::vector<std::vector<W>> named(T);
    parallel(T, [&](int s) {
      hist[s].fill(0);
      for (size_t i = 0; i < nodes[s].keys.size(); ++i) {
        if (nodes[s].state[i] != 1) continue;
        const W K = nodes[s].keys[i].v;
        const Node &n = nodes[s].vals[i];
        unsigned din = 0, dout = 0;
        for (unsigned c = 0; c < 4; ++c) {
          for (int side = 0; side < 2; ++side) {
            if (!n.c[side ? 4 + c : c]) continue;
            ++q[s];
            side ? ++din : ++dout;
            /* K.c answers with its in edge from first(K); c.K with its out edge to last(K) */
            W y = side ? ((K >> 2) | (W(c) << (2 * (ko.k - 1)))) : (((K << 2) | W(c)) & ko.mask);
            unsigned want_in = side ? 4 : ko.first(K), want_out = side ? ko.last(K) : 4;
            const W r = ko.rc(y);
            if (!(y < r)) {   /* lex_less flips the pair: in and out swap, complemented */
              y = r;
              const unsigned wi = want_out < 4 ? 3 - want_out : 4, wo = want_in < 4 ? 3 - want_in : 4;
              want_in = wi; want_out = wo;
            }
            named[s].push_back(y);
            const Node *m = node_of(y);
            if (!m) { ++absent[s]; continue; }
            if ((want_out < 4 && !m->c[want_out]) || (want_in < 4 && !m->c[4 + want_in])) ++unanswered[s];
          }
        }
        ++hist[s][din * 5 + dout];
      }
    });
    std::vector<std::vector<uint8_t>> marks(T);
    for (int s = 0; s < T; ++s) marks[s].assign(nodes[s].keys.size(), 0);
    for (int s = 0; s < T; ++s)
      for (W y : named[s]) {
        OAMap<KmerKey<W>, Node> &m = nodes[shard(y)];
        Node *x = m.find(KmerKey<W>{y});
        if (x) marks[shard(y)][(size_t)(x - m.vals.data())] = 1;
      }
    uint64_t unref = 0;
    for (int s = 0; s < T; ++s)
      for (size_t i = 0; i < nodes[s].keys.size(); ++i) {
        if (nodes[s].state[i] != 1 || marks[s][i]) continue;
        const Node &n = nodes[s].vals[i];
        bool any = false;
        for (int c = 0; c < 8; ++c) any |= n.c[c] != 0;
        unref += any;   /* IsIsolated nodes are erased before the check */
      }
    res->check_query = res->check_absent = res->check_unanswered = 0;
    for (int i = 0; i < 25; ++i) res->edge_hist[i] = 0;
    for (int s = 0; s < T; ++s) {
      res->check_query += q[s]; res->check_absent += absent[s]; res->check_unanswered += unanswered[s];
      for (int i = 0; i < 25; ++i) res->edge_hist[i] += hist[s][i];
    }
    res->check_unreferenced = unref;
  }

  /* ====================================================== chain-map outputs */
  static void put_records(std::vector<std::pair<W, ChainNode<W>>> &v, int w, uint64_t *n, uint64_t **keys,
                          uint64_t **in, uint64_t **out, uint32_t **ind, uint32_t **outd) {
    std::sort(v.begin(), v.end(), [](const std::pair<W, ChainNode<W>> &a, const std::pair<W, ChainNode<W>> &b) {
      return a.first < b.first;
    });
    *n = v.size();
    *keys = (uint64_t *)calloc(v.size() * w + 1, 8);
    *in = (uint64_t *)calloc(v.size() * w + 1, 8);
    *out = (uint64_t *)calloc(v.size() * w + 1, 8);
    *ind = (uint32_t *)calloc(v.size() + 1, 4);
    *outd = (uint32_t *)calloc(v.size() + 1, 4);
    for (size_t i = 0; i < v.size(); ++i) {
      store_word(*keys + i * w, v[i].first, w);
      store_word(*in + i * w, v[i].second.inK, w);
      store_word(*out + i * w, v[i].second.outK, w);
      (*ind)[i] = v[i].second.inD;
      (*outd)[i] = v[i].second.outD;
    }
  }
  void export_chain_map() {
    const int w = res->words;
    std::vector<std::pair<W, ChainNode<W>>> v;
    for (int s = 0; s < T; ++s)
      for (size_t i = 0; i < chain[s].keys.size(); ++i)
        if (chain[s].state[i] == 1) v.emplace_back(chain[s].keys[i].v, chain[s].vals[i]);
    put_records(v, w, &res->n_chain_map, &res->cm_keys, &res->cm_in, &res->cm_out, &res->cm_in_dist,
                &res->cm_out_dist);
    std::vector<std::pair<W, ChainNode<W>>> iso(isolated_recs);
    put_records(iso, w, &res->n_isolated_recs, &res->iso_keys, &res->iso_in, &res->iso_out, &res->iso_in_dist,
                &res->iso_out_dist);
    std::vector<W> cyc(cycle_kmers);
    std::sort(cyc.begin(), cyc.end());
    res->n_cycle_kmers = cyc.size();
    res->cycle_keys = (uint64_t *)calloc(cyc.size() * w + 1, 8);
    for (size_t i = 0; i < cyc.size(); ++i) store_word(res->cycle_keys + i * w, cyc[i], w);
  }

  /* ====================================================== table outputs */
  void export_tables(bool graph_only = false) {
    const int w = res->words;
    if (cfg.keep_k2 && !graph_only) {
      std::vector<std::pair<K2Key<W>, uint32_t>> v;
      for (int s = 0; s < T; ++s)
        for (size_t i = 0; i < k2[s].keys.size(); ++i)
          if (k2[s].state[i] == 1) v.emplace_back(k2[s].keys[i], k2[s].vals[i]);
      export_k2(v, &res->n_k2, &res->k2_keys, &res->k2_edges, &res->k2_counts, w);
    }
    if (cfg.keep_filtered && !graph_only) {
      std::vector<std::pair<K2Key<W>, uint32_t>> v;
      for (int s = 0; s < T; ++s) v.insert(v.end(), filtered[s].begin(), filtered[s].end());
      export_k2(v, &res->n_filtered, &res->filt_keys, &res->filt_edges, &res->filt_counts, w);
    }
    std::vector<std::pair<W, Node>> nv;
    for (int s = 0; s < T; ++s)
      for (size_t i = 0; i < nodes[s].keys.size(); ++i)
        if (nodes[s].state[i] == 1) nv.emplace_back(nodes[s].keys[i].v, nodes[s].vals[i]);
    par_sort(nv, [](const std::pair<W, Node> &a, const std::pair<W, Node> &b) { return a.first < b.first; }, T);
    res->n_nodes = nv.size();
    res->node_keys = (uint64_t *)calloc(nv.size() * w + 1, 8);
    res->node_counts = (uint16_t *)calloc(nv.size() * 9 + 1, 2);
    res->node_flags = (uint8_t *)calloc(nv.size() + 1, 1);
    for (size_t i = 0; i < nv.size(); ++i) {
      store_word(res->node_keys + i * w, nv[i].first, w);
      memcpy(res->node_counts + i * 9, nv[i].second.c, 18);
      res->node_flags[i] = (uint8_t)((is_branch(nv[i].first, nv[i].second) ? 1 : 0) |
                                     (is_chain(nv[i].first, nv[i].second) ? 2 : 0));
    }
  }
  void export_k2(std::vector<std::pair<K2Key<W>, uint32_t>> &v, uint64_t *n, uint64_t **keys,
                 uint8_t **edges, uint32_t **counts, int w) {
    par_sort(v, [](const std::pair<K2Key<W>, uint32_t> &a, const std::pair<K2Key<W>, uint32_t> &b) {
      return a.first.kmer < b.first.kmer || (a.first.kmer == b.first.kmer && a.first.edge < b.first.edge);
    }, T);
    *n = v.size();
    *keys = (uint64_t *)calloc(v.size() * w + 1, 8);
    *edges = (uint8_t *)calloc(v.size() + 1, 1);
    *counts = (uint32_t *)calloc(v.size() + 1, 4);
    for (size_t i = 0; i < v.size(); ++i) {
      store_word(*keys + i * w, v[i].first.kmer, w);
      (*edges)[i] = v[i].first.edge;
      (*counts)[i] = v[i].second;
    }
  }

  int run(const char *buf, size_t n) {
    if (!parse_and_count(buf, n)) { res->status = 2; return 2; }
    /* Unthresholded build_index (compact_dbg_build.hpp:34-62) updates each node once per
     * parsed pair with sat_incr (local_insert, debruijn_graph_map.hpp:175-197, update
     * :187-198).  A sum of saturating increments equals the saturating add of the pair's
     * count, so the same insert step serves both builds; it just sets no flags. */
    filter_insert();
    check_index();
    extract_chains();
    list_rank();
    emit();
    chain_edges();
    chain_summaries();
    export_tables();
    export_chain_map();
    if (cfg.clean) clean();
    return 0;
  }
};

template <typename W>
int run_typed(const char *buf, size_t n, const oracle_cfg &cfg, oracle_result *r, uint64_t k1_lo) {
  Run<W> run(cfg, r, k1_lo);
  return run.run(buf, n);
}

/* ---------------------------------------------------------------- text output */
std::string ascii_words(const uint64_t *p, int k, int words) {
  static const char A[4] = {'A', 'C', 'G', 'T'};
  std::string s(k, 'A');
  for (int i = 0; i < k; ++i) {
    int bit = 2 * i;
    uint64_t w = (words == 1 || bit < 64) ? p[0] : p[1];
    s[k - 1 - i] = A[(w >> (bit & 63)) & 3u];
  }
  return s;
}

}  // namespace

extern "C" int oracle_run(const char *fastq, size_t nbytes, const oracle_cfg *cfg, oracle_result **out) {
  if (!cfg || !out || cfg->k < 3 || cfg->k > 63) return 1;
  oracle_result *r = (oracle_result *)calloc(1, sizeof(oracle_result));
  /* exported arrays use the GB300 library's layout (2 words from k = 32 on) so the two
   * compare directly; k = 32 still computes in one 64-bit word, as Kmer<32> does */
  r->words = cfg->k <= 31 ? 1 : 2;
  oracle_cfg c = *cfg;
  const uint64_t k1_lo = cfg->thresh[2];   /* cleaning reads threshes[2] whatever the build */
  if (c.edge_filter && !c.thresholding) c.edge_filter = 0;   /* build_index: no filter at all */
  if (c.edge_filter) {
    /* the (k+1)-mer bounds stay in thresh[2..3]; the node insert is build_index's */
    c.thresholding = 0;
    c.thresh[0] = c.thresh[4] = 0;
    c.thresh[1] = c.thresh[5] = ~0ULL;
  } else if (!c.thresholding) {
    /* build_index: no flags (every entry kept with both edges) */
    c.thresh[0] = c.thresh[2] = c.thresh[4] = 0;
    c.thresh[1] = c.thresh[3] = c.thresh[5] = ~0ULL;
  }
  int rc = (cfg->k <= 32) ? run_typed<uint64_t>(fastq, nbytes, c, r, k1_lo)
                               : run_typed<u128>(fastq, nbytes, c, r, k1_lo);
  r->status = rc;
  *out = r;
  return rc;
}

extern "C" void oracle_free(oracle_result *r) {
  if (!r) return;
  free(r->k2_keys); free(r->k2_edges); free(r->k2_counts);
  free(r->filt_keys); free(r->filt_edges); free(r->filt_counts);
  free(r->node_keys); free(r->node_counts); free(r->node_flags);
  free(r->ranked_K); free(r->ranked_rep); free(r->ranked_dist);
  free(r->chain_rep); free(r->chain_offsets); free(r->chain_chars);
  free(r->edge_L); free(r->edge_R); free(r->edge_freqs);
  free(r->sum_kmers); free(r->sum_dist); free(r->sum_flags);
  oracle_free(r->clean);
  free(r->cm_keys); free(r->cm_in); free(r->cm_out); free(r->cm_in_dist); free(r->cm_out_dist);
  free(r->iso_keys); free(r->iso_in); free(r->iso_out); free(r->iso_in_dist); free(r->iso_out_dist);
  free(r->cycle_keys);
  free(r);
}

namespace {
enum { W_CHAINS = 1, W_EDGES = 2, W_SUMMARY = 4, W_NODES = 8, W_GRAPH_ALL = 16 };

int write_parts(const oracle_result *r, int32_t k, const std::string &p, int32_t benchmark, int parts) {
  const int w = r->words;
  auto canon = [&](const uint64_t *x) {
    /* lex_less on a k-mer word: min(x, rc(x)) */
    if (w == 1) { KOps<uint64_t> ko(k); uint64_t v = x[0], y = ko.rc(v); return v < y ? v : y; }
    return (uint64_t)0;
  };
  auto canon128 = [&](const uint64_t *x) {
    KOps<u128> ko(k); u128 v = ((u128)(w > 1 ? x[1] : 0) << 64) | x[0], y = ko.rc(v); return v < y ? v : y;
  };
  auto canon_ascii = [&](const uint64_t *x) {
    if (w == 1) { uint64_t c = canon(x); return ascii_words(&c, k, 1); }
    u128 c = canon128(x); uint64_t q[2] = {(uint64_t)c, (uint64_t)(c >> 64)}; return ascii_words(q, k, 2);
  };
  auto is_canon = [&](const uint64_t *x) {
    if (w == 1) return canon(x) == x[0];
    u128 c = canon128(x); return (uint64_t)c == x[0] && (uint64_t)(c >> 64) == x[1];
  };
  auto less_words = [&](const uint64_t *a, const uint64_t *b) {
    if (w == 2 && a[1] != b[1]) return a[1] < b[1];
    return a[0] < b[0];
  };
  /* .chain.fasta: print_chain_string (compact_dbg_io.hpp:323-363), sorted by chain_rep_less;
   * the leading newline of the first record is dropped. */
  if (parts & W_CHAINS) {
    std::vector<size_t> idx(r->n_ranked);
    for (size_t i = 0; i < idx.size(); ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) {
      const uint64_t *ra = r->ranked_rep + a * w, *rb = r->ranked_rep + b * w;
      if (less_words(ra, rb)) return true;
      if (less_words(rb, ra)) return false;
      int da = std::abs(r->ranked_dist[a]), db = std::abs(r->ranked_dist[b]);
      if (da != db) return da < db;
      return less_words(r->ranked_K + a * w, r->ranked_K + b * w);
    });
    std::string s;
    for (size_t i : idx) {
      if (r->ranked_dist[i] == 0) {
        s += "\n>"; s += canon_ascii(r->ranked_K + i * w); s += "\n";
        s += ascii_words(r->ranked_rep + i * w, k, w);
      } else {
        s += ascii_words(r->ranked_K + i * w, k, w).back();
      }
    }
    FILE *f = fopen((p + ".chain.fasta").c_str(), "wb");
    if (!f) return 1;
    if (!s.empty()) fwrite(s.data() + 1, 1, s.size() - 1, f);
    fclose(f);
  }
  /* .chain.components: print_chain_nodes (compact_dbg_io.hpp:463-498) sorted by K,
   * print_chain_node (debruijn_chain_operations.hpp:434-441). */
  if ((parts & W_CHAINS) && !benchmark) {
    std::string s;
    for (size_t i = 0; i < r->n_ranked; ++i) {
      const uint64_t *K = r->ranked_K + i * w;
      s += canon_ascii(K); s += "\t"; s += ascii_words(r->ranked_rep + i * w, k, w); s += "\t";
      s += std::to_string(r->ranked_dist[i]); s += "\t"; s += is_canon(K) ? "1" : "0"; s += "\n";
    }
    FILE *f = fopen((p + ".chain.components").c_str(), "wb");
    if (!f) return 1;
    fwrite(s.data(), 1, s.size(), f);
    fclose(f);
  }
  /* .chain.edges: print_chain_frequencies (compact_dbg_stats.hpp:1034-1057), each value
   * followed by a tab, records already sorted by L. */
  if ((parts & W_EDGES) && !benchmark) {
    std::string s;
    for (size_t i = 0; i < r->n_chain_edges; ++i) {
      s += ascii_words(r->edge_L + i * w, k, w); s += "\t";
      s += ascii_words(r->edge_R + i * w, k, w); s += "\t";
      for (int j = 0; j < 11; ++j) { s += std::to_string(r->edge_freqs[i * 11 + j]); s += "\t"; }
      s += "\n";
    }
    FILE *f = fopen((p + ".chain.edges").c_str(), "wb");
    if (!f) return 1;
    fwrite(s.data(), 1, s.size(), f);
    fclose(f);
  }
  /* .chain.summary: print_chain_summaries (compact_dbg_io.hpp:528-556), space separated.
   * The reference prints the four k-mers with kmerind's Kmer stream operator, which is not part
   * of the reference sources; they are printed here as their bases. */
  if ((parts & W_SUMMARY) && !benchmark && r->summaries_ok) {
    std::string s;
    for (size_t i = 0; i < r->n_summaries; ++i) {
      for (int j = 0; j < 4; ++j) { s += ascii_words(r->sum_kmers + (i * 4 + j) * w, k, w); s += " "; }
      s += std::to_string(r->sum_dist[i]) + " " + std::to_string(r->sum_flags[2 * i]) + " " +
           std::to_string(r->sum_flags[2 * i + 1]) + "\n";
    }
    FILE *f = fopen((p + ".chain.summary").c_str(), "wb");
    if (!f) return 1;
    fwrite(s.data(), 1, s.size(), f);
    fclose(f);
  }
  /* .branch.fasta (compact_dbg_io.hpp:254-299), .branch.edges (compact_dbg_stats.hpp:219-262)
   * and .graph.all, all sorted by k-mer; node lines follow print_graph_node
   * (debruijn_graph_operations.hpp:57-78): k-mer, in A C G T, out A C G T, self. */
  if (parts & W_NODES) {
    std::string fa, be, ga;
    for (size_t i = 0; i < r->n_nodes; ++i) {
      const uint64_t *x = r->node_keys + i * w;
      const uint16_t *c = r->node_counts + i * 9;
      std::string a = ascii_words(x, k, w);
      bool br = (r->node_flags[i] & 1) != 0;
      std::string line = a;
      for (int j = 4; j < 8; ++j) line += "\t" + std::to_string(c[j]);
      for (int j = 0; j < 4; ++j) line += "\t" + std::to_string(c[j]);
      line += "\t" + std::to_string(c[8]) + "\n";
      if (br) { fa += ">" + a + "\n" + a + "\n"; be += line; }
      ga += line;
    }
    FILE *f = fopen((p + ".branch.fasta").c_str(), "wb");
    if (!f) return 1;
    fwrite(fa.data(), 1, fa.size(), f); fclose(f);
    if (!benchmark) {
      f = fopen((p + ".branch.edges").c_str(), "wb");
      if (!f) return 1;
      fwrite(be.data(), 1, be.size(), f); fclose(f);
      if (parts & W_GRAPH_ALL) {
        f = fopen((p + ".graph.all").c_str(), "wb");
        if (!f) return 1;
        fwrite(ga.data(), 1, ga.size(), f); fclose(f);
      }
    }
  }
  return 0;
}
}  // namespace

/* Without cleaning, the _freq driver's files.  With cleaning, the _freq_clean driver's: the
 * first compaction's .graph.all, .branch.*, .chain.summary, .chain.fasta and .chain.components
 * (printed inside the clean block, compact_dbg_freq_construct_clean.cpp:636-660), then, under
 * the prefix with ".clean" appended (:677), the cleaned graph's .branch.* (:680-697) and its
 * .chain.fasta, .chain.components and .chain.edges (:733-790). */
extern "C" int oracle_write_outputs(const oracle_result *r, int32_t k, const char *prefix, int32_t benchmark) {
  if (!r || r->status != 0) return 1;
  const std::string p(prefix);
  if (!r->clean) return write_parts(r, k, p, benchmark, W_CHAINS | W_EDGES | W_SUMMARY | W_NODES | W_GRAPH_ALL);
  if (write_parts(r, k, p, benchmark, W_CHAINS | W_SUMMARY | W_NODES | W_GRAPH_ALL)) return 1;
  return write_parts(r->clean, k, p + ".clean", benchmark, W_CHAINS | W_EDGES | W_NODES);
}
