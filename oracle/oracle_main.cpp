/*
 * oracle_main.cpp -- command-line front end of the CPU oracle (test infrastructure).
 *
 * Mirrors the flags of the reference driver test/test/compact_dbg_freq_construct_clean.cpp
 * (main :848-1030): -T thresholding, -L/-U lower/upper thresholds (one value = (k+1)-mer,
 * three values = k, k+1, k+2; :937-961), -E the (k+1)-mer edge filter of the blocked driver
 * compact_debruijn_graph_block_construct.cpp, -R list_rank_min_update, -B benchmark, -O output
 * prefix; plus -k (k-mer length, a compile-time constant in the reference), -t (host
 * threads = hash shards) and --clean (the _freq_clean build of the same driver, which cleans
 * dead ends and bubbles after the first compaction; the _freq build defines NCLEAN).  FASTQ files are concatenated into one k2 counter, as the
 * reference counts all files before filtering (build_index_thresholded :295-348).
 */
#include "bruno_oracle.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

static bool read_file(const char *fn, std::string &out) {
  FILE *f = fopen(fn, "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, n);
  fclose(f);
  return true;
}

int main(int argc, char **argv) {
  oracle_cfg cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.k = 31;
  cfg.threads = 1;
  for (int i = 0; i < 6; ++i) cfg.thresh[i] = 65536;  /* CountType max + 1 (:874) */
  std::vector<uint64_t> lo, hi;
  std::string prefix = "./output";
  int benchmark = 0;
  std::vector<const char *> files;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "-T") cfg.thresholding = 1;
    else if (a == "-R") cfg.min_update = 1;
    else if (a == "-B") benchmark = 1;
    else if (a == "-E") cfg.edge_filter = 1;   /* the blocked driver's (k+1)-mer filter build */
    else if (a == "--clean") cfg.clean = 1;
    else if (a == "-L" && i + 1 < argc) lo.push_back(strtoull(argv[++i], 0, 10));
    else if (a == "-U" && i + 1 < argc) hi.push_back(strtoull(argv[++i], 0, 10));
    else if (a == "-O" && i + 1 < argc) prefix = argv[++i];
    else if (a == "-k" && i + 1 < argc) cfg.k = atoi(argv[++i]);
    else if (a == "-t" && i + 1 < argc) cfg.threads = atoi(argv[++i]);
    else if (a[0] == '-') { fprintf(stderr, "unknown flag %s\n", a.c_str()); return 1; }
    else files.push_back(argv[i]);
  }
  if (lo.size() == 1) { cfg.thresh[2] = std::min<uint64_t>(lo[0], cfg.thresh[2]); cfg.thresh[0] = cfg.thresh[4] = 0; }
  else if (lo.size() == 3) {
    cfg.thresh[0] = std::min<uint64_t>(lo[0], cfg.thresh[0]);
    cfg.thresh[2] = std::min<uint64_t>(lo[1], cfg.thresh[2]);
    cfg.thresh[4] = std::min<uint64_t>(lo[2], cfg.thresh[4]);
  }
  if (hi.size() == 1) cfg.thresh[3] = std::min<uint64_t>(hi[0], cfg.thresh[3]);
  else if (hi.size() == 3) {
    cfg.thresh[1] = std::min<uint64_t>(hi[0], cfg.thresh[1]);
    cfg.thresh[3] = std::min<uint64_t>(hi[1], cfg.thresh[3]);
    cfg.thresh[5] = std::min<uint64_t>(hi[2], cfg.thresh[5]);
  }
  if (files.empty()) { fprintf(stderr, "usage: %s [-T] [-E] [--clean] [-L n].. [-U n].. [-R] [-B] [-O prefix] [-k K] [-t T] reads.fastq..\n", argv[0]); return 1; }
  std::string data;
  for (const char *f : files) {
    if (!read_file(f, data)) { fprintf(stderr, "cannot read %s\n", f); return 1; }
    if (!data.empty() && data.back() != '\n') data.push_back('\n');
  }
  oracle_result *r = nullptr;
  int rc = oracle_run(data.data(), data.size(), &cfg, &r);
  if (rc != 0) { fprintf(stderr, "oracle_run failed: %d\n", rc); oracle_free(r); return 1; }
  printf("reads %llu used %llu instances %llu nodes %llu branch %llu chain %llu iterations %llu "
         "cycle %llu isolated %llu chains %llu collisions %llu\n",
         (unsigned long long)r->n_reads, (unsigned long long)r->n_reads_used, (unsigned long long)r->n_instances,
         (unsigned long long)r->n_nodes, (unsigned long long)r->n_branch, (unsigned long long)r->n_chain_nodes,
         (unsigned long long)r->iterations, (unsigned long long)r->n_cycle_nodes, (unsigned long long)r->n_isolated,
         (unsigned long long)r->n_chains, (unsigned long long)r->collisions);
  rc = oracle_write_outputs(r, cfg.k, prefix.c_str(), benchmark);
  oracle_free(r);
  return rc;
}
