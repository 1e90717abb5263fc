/*
 * synth.cpp -- seeded synthetic genomes and FASTQ reads for the workloads the library is
 * measured and tested on (uniform genomes with optional diverged repeat families, reads
 * sampled uniformly with random strand and uniform substitution errors).
 *
 * The generator is deterministic for a given configuration and independent of the thread
 * count and of the host architecture: every read draws from its own counter-seeded
 * xoshiro256** stream, and only integer arithmetic decides bases.
 *
 * Output record format: "@r<i>\n<sequence>\n+\n<'I' x L>\n".
 */
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

namespace {

inline uint64_t splitmix64(uint64_t &s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

struct Rng {  /* xoshiro256** (Blackman & Vigna), seeded through splitmix64 */
  uint64_t s[4];
  explicit Rng(uint64_t seed) { for (int i = 0; i < 4; ++i) s[i] = splitmix64(seed); }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
    return r;
  }
  uint64_t below(uint64_t n) { return n ? (uint64_t)(((unsigned __int128)next() * n) >> 64) : 0; }
  /* Bernoulli(p) with p given in parts per 2^32 */
  bool chance(uint32_t p32) { return (uint32_t)(next() >> 32) < p32; }
};

inline uint32_t prob32(double p) {
  if (p <= 0) return 0;
  if (p >= 1) return 0xFFFFFFFFu;
  return (uint32_t)(p * 4294967296.0);
}

const char BASES[4] = {'A', 'C', 'G', 'T'};

inline char substitute(char c, Rng &r) {  /* uniform choice among the 3 other bases */
  int code = c == 'A' ? 0 : c == 'C' ? 1 : c == 'G' ? 2 : 3;
  return BASES[(code + 1 + (int)r.below(3)) & 3];
}
inline char complement(char c) {
  return c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : 'A';
}
inline int digits(uint64_t x) { int d = 1; while (x >= 10) { x /= 10; ++d; } return d; }

}  // namespace

extern "C" {

typedef struct synth_cfg {
  uint64_t seed;
  uint64_t genome_len;
  double repeat_frac;        /* fraction of the genome covered by repeat copies */
  uint32_t rep_len_min, rep_len_max;
  uint32_t rep_copies_min, rep_copies_max;
  double rep_div_min, rep_div_max;   /* per-copy substitution rate, uniform in [min, max] */
  uint32_t read_len;
  uint64_t n_reads;
  double sub_rate;           /* per-base substitution rate of the reads */
  int32_t threads;
} synth_cfg;

/* Byte offset of record i: records with a d-digit index are 2+d+1+L+1+2+L+1 bytes. */
static uint64_t record_offset(uint64_t i, uint64_t L) {
  uint64_t off = 0, base = 2 + 1 + L + 1 + 2 + L + 1;
  for (uint64_t lo = 0, hi = 10, d = 1; lo < i; lo = hi, hi *= 10, ++d)
    off += (std::min(i, hi) - lo) * (base + d);
  return off;
}

/* Exact size in bytes of the FASTQ that synth_fastq writes. */
uint64_t synth_fastq_size(const synth_cfg *c) { return record_offset(c->n_reads, c->read_len); }

/* Genome: uniform ACGT, then repeat families copied over it (source segment re-written at
 * `copies` further positions, each copy with its own divergence). */
int synth_genome(const synth_cfg *c, char *g) {
  Rng r(c->seed ^ 0x5eed0001ULL);
  const uint64_t G = c->genome_len;
  for (uint64_t i = 0; i < G; ++i) g[i] = BASES[r.next() >> 62];
  if (c->repeat_frac > 0 && c->rep_len_max > 0 && G > c->rep_len_max) {
    uint64_t target = (uint64_t)(c->repeat_frac * (double)G), covered = 0;
    std::vector<char> seg;
    while (covered < target) {
      uint64_t len = c->rep_len_min + r.below(c->rep_len_max - c->rep_len_min + 1);
      uint64_t copies = c->rep_copies_min + r.below(c->rep_copies_max - c->rep_copies_min + 1);
      uint64_t src = r.below(G - len);
      seg.assign(g + src, g + src + len);
      for (uint64_t cp = 1; cp < copies; ++cp) {
        double div = c->rep_div_min + (c->rep_div_max - c->rep_div_min) * ((r.next() >> 11) * 0x1.0p-53);
        uint32_t p = prob32(div);
        uint64_t dst = r.below(G - len);
        for (uint64_t i = 0; i < len; ++i) g[dst + i] = r.chance(p) ? substitute(seg[i], r) : seg[i];
      }
      covered += len * copies;
    }
  }
  return 0;
}

/* Writes the FASTQ into out (capacity cap, at least synth_fastq_size bytes).  If genome is
 * non-null it receives the genome (genome_len bytes). */
int synth_fastq(const synth_cfg *c, char *out, uint64_t cap, char *genome_out) {
  const uint64_t G = c->genome_len, L = c->read_len, R = c->n_reads;
  if (G < L || L == 0) return 1;
  if (cap < synth_fastq_size(c)) return 2;
  std::vector<char> gbuf;
  char *g = genome_out;
  if (!g) { gbuf.resize(G); g = gbuf.data(); }
  synth_genome(c, g);
  const uint32_t p = prob32(c->sub_rate);
  int T = c->threads > 0 ? c->threads : (int)std::max(1u, std::thread::hardware_concurrency());
  T = (int)std::min<uint64_t>((uint64_t)T, std::max<uint64_t>(1, R / 1024));
  std::vector<std::thread> th;
  for (int t = 0; t < T; ++t) {
    th.emplace_back([&, t]() {
      uint64_t b = R * t / T, e = R * (t + 1) / T;
      char *o = out + record_offset(b, L);
      for (uint64_t i = b; i < e; ++i) {
        Rng r(c->seed * 0x9e3779b97f4a7c15ULL + i + 1);
        uint64_t start = r.below(G - L + 1);
        bool rev = (r.next() >> 63) != 0;
        *o++ = '@'; *o++ = 'r';
        int d = digits(i);
        uint64_t v = i;
        for (int q = d - 1; q >= 0; --q) { o[q] = (char)('0' + v % 10); v /= 10; }
        o += d;
        *o++ = '\n';
        for (uint64_t j = 0; j < L; ++j) {
          char ch = rev ? complement(g[start + L - 1 - j]) : g[start + j];
          if (r.chance(p)) ch = substitute(ch, r);
          *o++ = ch;
        }
        *o++ = '\n'; *o++ = '+'; *o++ = '\n';
        memset(o, 'I', L); o += L;
        *o++ = '\n';
      }
    });
  }
  for (auto &x : th) x.join();
  return 0;
}

}  // extern "C"
