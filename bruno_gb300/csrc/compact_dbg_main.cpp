/*
 * compact_dbg_main.cpp -- command-line driver on the GB300 library, with the flags and
 * output files of the reference driver test/test/compact_dbg_freq_construct_clean.cpp
 * (main :848-1030, do_work :431-840, built with -DNCLEAN):
 *
 *   -T          thresholding (build_index_thresholded), else build_index
 *   -L n [-L n -L n], -U ...  lower / upper thresholds (one value = (k+1)-mer bound,
 *               three values = k, k+1, k+2; :937-961)
 *   -R          list_rank_min_update, else list_rank
 *   -B          benchmark: only .chain.fasta and .branch.fasta
 *   -E          with -T: the (k+1)-mer edge filter of the blocked driver
 *               test/test/compact_debruijn_graph_block_construct.cpp (build_index_thresholded
 *               :417-470; -L / -U bound the (k+1)-mer counts) instead of the (k+2)-mer filter
 *   --clean     the _freq_clean build of the same driver (no NCLEAN): dead ends and bubbles
 *               cleaned after the first compaction (clean_deadend_and_bubbles_naive,
 *               test/common/compact_dbg_clean.hpp:575-890)
 *   -O prefix   output prefix
 *   -k K        k-mer length (the reference's compile-time pK)
 *   files...    FASTQ files, all counted into one table
 *
 * Outputs: <prefix>.chain.fasta (print_chain_string, compact_dbg_io.hpp:323-363),
 * <prefix>.chain.components (print_chain_nodes, :463-498), <prefix>.branch.fasta
 * (print_branch_fasta, :254-299), and unless -B <prefix>.chain.edges
 * (print_chain_frequencies, compact_dbg_stats.hpp:879-1065), <prefix>.chain.summary
 * (print_chain_summaries, compact_dbg_io.hpp:528-556; k-mers printed as bases), <prefix>.branch.edges
 * (print_branch_edge_frequencies, :219-262) and <prefix>.graph.all.
 * With --clean: the same files of the first compaction except .chain.edges, then
 * <prefix>.clean.branch.fasta, .clean.chain.fasta and unless -B .clean.branch.edges,
 * .clean.chain.components and .clean.chain.edges of the cleaned graph.
 * Like the reference, records are sorted before printing; the .chain.fasta has no newline
 * before its first record and none after its last.
 */
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "bruno_gb300.hpp"

namespace {

bool read_file(const char *fn, std::string &out) {
  FILE *f = fopen(fn, "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, n);
  fclose(f);
  return true;
}

struct Kmer {
  uint64_t w[2] = {0, 0};
  bool operator<(const Kmer &o) const { return w[1] != o.w[1] ? w[1] < o.w[1] : w[0] < o.w[0]; }
  bool operator==(const Kmer &o) const { return w[0] == o.w[0] && w[1] == o.w[1]; }
};

Kmer load(const uint64_t *p, int words) {
  Kmer k;
  k.w[0] = p[0];
  if (words > 1) k.w[1] = p[1];
  return k;
}

unsigned base(const Kmer &x, int i) {  /* i counted from the last base */
  return (unsigned)((i < 32 ? x.w[0] >> (2 * i) : x.w[1] >> (2 * (i - 32))) & 3u);
}

std::string ascii(const Kmer &x, int k) {
  std::string s(k, 'A');
  for (int i = 0; i < k; ++i) s[k - 1 - i] = "ACGT"[base(x, i)];
  return s;
}

Kmer rc(const Kmer &x, int k) {
  Kmer y;
  for (int i = 0; i < k; ++i) {
    const unsigned b = 3u - base(x, i);   /* base i from the end becomes base i from the start */
    const int pos = k - 1 - i;             /* its index from the end in the result */
    if (pos < 32) y.w[0] |= (uint64_t)b << (2 * pos); else y.w[1] |= (uint64_t)b << (2 * (pos - 32));
  }
  return y;
}

Kmer canonical(const Kmer &x, int k) {
  Kmer y = rc(x, k);
  return x < y ? x : y;
}

bool write(const std::string &fn, const std::string &s) {
  FILE *f = fopen(fn.c_str(), "wb");
  if (!f) return false;
  fwrite(s.data(), 1, s.size(), f);
  fclose(f);
  return true;
}

}  // namespace

int main(int argc, char **argv) {
  bruno_cfg cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.k = 31;
  std::vector<uint64_t> lo, hi;
  std::string prefix = "./output";
  bool benchmark = false, clean = false;
  std::vector<const char *> files;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "-T") cfg.thresholding = 1;
    else if (a == "-R") cfg.min_update = 1;
    else if (a == "-B") benchmark = true;
    else if (a == "-E") cfg.edge_filter = 1;
    else if (a == "--clean") clean = true;
    else if (a == "-L" && i + 1 < argc) lo.push_back(strtoull(argv[++i], nullptr, 10));
    else if (a == "-U" && i + 1 < argc) hi.push_back(strtoull(argv[++i], nullptr, 10));
    else if (a == "-O" && i + 1 < argc) prefix = argv[++i];
    else if (a == "-k" && i + 1 < argc) cfg.k = atoi(argv[++i]);
    else if (a == "-d" && i + 1 < argc) cfg.device = atoi(argv[++i]);
    else if (!a.empty() && a[0] == '-') { fprintf(stderr, "unknown flag %s\n", a.c_str()); return 1; }
    else files.push_back(argv[i]);
  }
  if (files.empty()) {
    fprintf(stderr, "usage: %s [-T] [-E] [--clean] [-L n].. [-U n].. [-R] [-B] [-O prefix] [-k K] reads.fastq..\n", argv[0]);
    return 1;
  }
  const std::vector<uint64_t> t = bruno_gb300::thresholds(lo, hi);
  std::copy(t.begin(), t.end(), cfg.thresh);
  const int k = cfg.k, words = k <= 31 ? 1 : 2;
  try {
    std::vector<std::string> data(files.size());
    for (size_t i = 0; i < files.size(); ++i)
      if (!read_file(files[i], data[i])) { fprintf(stderr, "cannot read %s\n", files[i]); return 1; }
    const auto t0 = std::chrono::steady_clock::now();
    bruno_gb300::context ctx(cfg);
    bruno_gb300::debruijn_graph idx(ctx);
    bruno_gb300::debruijn_chain_graph chainmap(ctx);
    for (auto &d : data) idx.get_map().load_fastq(d.data(), d.size());
    idx.get_map().compute_biedge_freqencies();                  /* build_index_thresholded */
    idx.get_map().local_insert_by_freqencies(t);
    chainmap.extract_chains(idx);                               /* do_work :549 */
    const size_t iterations = cfg.min_update ? chainmap.list_rank_min_update() : chainmap.list_rank();
    bruno_gb300::listranked_chain_nodes ranked = chainmap.to_ranked_chain_nodes();
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const bruno_sizes s = ctx.sizes();
    printf("reads %llu used %llu instances %llu nodes %llu branch %llu chain %llu iterations %zu cycle %llu "
           "isolated %llu chains %llu  (%.3f s)\n",
           (unsigned long long)s.n_reads, (unsigned long long)s.n_reads_used, (unsigned long long)s.n_instances,
           (unsigned long long)s.n_nodes, (unsigned long long)s.n_branch, (unsigned long long)s.n_chain_nodes,
           iterations, (unsigned long long)s.n_cycle_nodes, (unsigned long long)s.n_isolated,
           (unsigned long long)s.n_chains, secs);

    /* chain files of the current chain graph: .chain.fasta, and unless -B .chain.components,
     * then (when asked) .chain.edges and .chain.summary */
    auto write_chain_files = [&](const std::string &pre, const bruno_gb300::listranked_chain_nodes &ranked,
                                 bool edges, bool summary) -> bool {
      /* .chain.fasta: sorted by chain_rep_less (rep, |dist|) */
      const size_t n = ranked.size();
      std::vector<size_t> order(n);
      std::iota(order.begin(), order.end(), 0);
      std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        const Kmer ra = load(&ranked.rep[a * words], words), rb = load(&ranked.rep[b * words], words);
        if (!(ra == rb)) return ra < rb;
        const int da = std::abs(ranked.dist[a]), db = std::abs(ranked.dist[b]);
        if (da != db) return da < db;
        return load(&ranked.K[a * words], words) < load(&ranked.K[b * words], words);
      });
      std::string fa;
      for (size_t i : order) {
        const Kmer K = load(&ranked.K[i * words], words);
        if (ranked.dist[i] == 0) {
          fa += "\n>" + ascii(canonical(K, k), k) + "\n" + ascii(load(&ranked.rep[i * words], words), k);
        } else {
          fa += "ACGT"[base(K, 0)];
        }
      }
      if (!write(pre + ".chain.fasta", fa.empty() ? fa : fa.substr(1))) return false;
      if (benchmark) return true;
      /* .chain.components: sorted by K (chain_node_less) */
      std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return load(&ranked.K[a * words], words) < load(&ranked.K[b * words], words);
      });
      std::string cc;
      for (size_t i : order) {
        const Kmer K = load(&ranked.K[i * words], words), c = canonical(K, k);
        cc += ascii(c, k) + "\t" + ascii(load(&ranked.rep[i * words], words), k) + "\t" +
              std::to_string(ranked.dist[i]) + "\t" + (K == c ? "1" : "0") + "\n";
      }
      if (!write(pre + ".chain.components", cc)) return false;
      if (edges) {
        /* .chain.edges: sorted by L; every value is followed by a tab */
        std::vector<uint64_t> ends;
        std::vector<uint16_t> ef;
        const size_t ne = chainmap.chain_edges(ends, ef);
        std::vector<size_t> eo(ne);
        std::iota(eo.begin(), eo.end(), 0);
        std::sort(eo.begin(), eo.end(), [&](size_t a, size_t b) {
          return load(&ends[a * 2 * words], words) < load(&ends[b * 2 * words], words);
        });
        std::string ce;
        for (size_t i : eo) {
          ce += ascii(load(&ends[i * 2 * words], words), k) + "\t" + ascii(load(&ends[i * 2 * words + words], words), k);
          for (int j = 0; j < 11; ++j) ce += "\t" + std::to_string(ef[i * 11 + j]);
          ce += "\t\n";
        }
        if (!write(pre + ".chain.edges", ce)) return false;
      }
      if (summary) {
        /* .chain.summary: sorted by the 5' terminus (the representative), space separated; only
         * for mutually consistent chain pointers, where the reference's pairing is well defined */
        std::vector<uint64_t> sk;
        std::vector<uint32_t> sd;
        std::vector<uint8_t> sf;
        size_t ns = 0;
        bool have_summaries = true;
        try {
          ns = chainmap.to_summarized_chains(sk, sd, sf);
        } catch (const bruno_gb300::error &e) {
          if (e.status != BRUNO_ERR_INVARIANT) throw;
          fprintf(stderr, "no .chain.summary: %s\n", e.what());
          have_summaries = false;
        }
        if (have_summaries) {
          std::vector<size_t> so(ns);
          std::iota(so.begin(), so.end(), 0);
          std::sort(so.begin(), so.end(), [&](size_t a, size_t b) {
            return load(&sk[(a * 4 + 1) * words], words) < load(&sk[(b * 4 + 1) * words], words);
          });
          std::string cs;
          for (size_t i : so) {
            for (int j = 0; j < 4; ++j) cs += ascii(load(&sk[(i * 4 + j) * words], words), k) + " ";
            cs += std::to_string(sd[i]) + " " + std::to_string(sf[2 * i]) + " " + std::to_string(sf[2 * i + 1]) + "\n";
          }
          if (!write(pre + ".chain.summary", cs)) return false;
        }
      }
      return true;
    };
    /* node files of the current graph, sorted by k-mer: .branch.fasta, and unless -B
     * .branch.edges and (when asked) .graph.all */
    auto write_node_files = [&](const std::string &pre, bool graph_all) -> bool {
      std::vector<uint64_t> nkeys;
      std::vector<uint16_t> ncounts;
      std::vector<uint8_t> nflags;
      idx.get_map().to_vector(nkeys, ncounts, nflags);
      std::vector<size_t> nord(nflags.size());
      std::iota(nord.begin(), nord.end(), 0);
      std::sort(nord.begin(), nord.end(),
                [&](size_t a, size_t b) { return load(&nkeys[a * words], words) < load(&nkeys[b * words], words); });
      std::string bf, be, ga;
      for (size_t i : nord) {
        const std::string a = ascii(load(&nkeys[i * words], words), k);
        const uint16_t *c = &ncounts[i * 9];
        std::string line = a;
        for (int j = 4; j < 8; ++j) line += "\t" + std::to_string(c[j]);
        for (int j = 0; j < 4; ++j) line += "\t" + std::to_string(c[j]);
        line += "\t" + std::to_string(c[8]) + "\n";
        if (nflags[i] & 1) { bf += ">" + a + "\n" + a + "\n"; be += line; }
        ga += line;
      }
      if (!write(pre + ".branch.fasta", bf)) return false;
      if (benchmark) return true;
      return write(pre + ".branch.edges", be) && (!graph_all || write(pre + ".graph.all", ga));
    };
    if (!clean) {
      if (!write_chain_files(prefix, ranked, true, true) || !write_node_files(prefix, true)) return 1;
    } else {
      /* the _freq_clean build: the first compaction's files without .chain.edges (:513-660),
       * the cleaning (:670-674), then the cleaned graph's under <prefix>.clean (:677-790) */
      if (!write_node_files(prefix, true) || !write_chain_files(prefix, ranked, false, true)) return 1;
      const bruno_clean_stats cs = chainmap.clean_deadend_and_bubbles_naive();
      printf("cleaning: %llu rounds, %llu dead ends, %llu bubble chains, %llu edges erased%s\n",
             (unsigned long long)cs.rounds, (unsigned long long)cs.deadends, (unsigned long long)cs.bubbles,
             (unsigned long long)cs.edges, cs.status == 1 ? " (stopped: an iteration erased nothing)" : "");
      const std::string pc = prefix + ".clean";
      if (!write_node_files(pc, false) || !write_chain_files(pc, chainmap.to_ranked_chain_nodes(), true, false)) return 1;
    }
  } catch (const bruno_gb300::error &e) {
    fprintf(stderr, "error: %s\n", e.what());
    return 2;
  }
  return 0;
}
