/*
 * kmer.cuh -- device k-mer words and the k-mer table slot format.
 *
 * A k-mer is 2-bit packed (A0 C1 G2 T3) with its first base in the most significant bits,
 * the layout of bliss::common::Kmer<k, DNA, uint64_t> (nextFromChar appends at the least
 * significant end, debruijn_graph_node.hpp:327; nextReverseFromChar prepends,
 * :344).  Its order (operator<) is the unsigned order of the packed value.
 *   KW1: one 64-bit word, k <= 31 (bits 62/63 stay free for table flags)
 *   KW2: two 64-bit words, 32 <= k <= 63 (the high word keeps bits 62/63 free)
 *
 * k-mer table slot (one slot per distinct canonical k-mer, linear probing):
 *   KW1: 32 B = key u64 | 6 x u32 entry words
 *   KW2: 64 B = key lo u64 | key hi u64 | 12 x u32 entry words
 * During counting an entry word is [count:26 | biedge code:5 | big:1]: the code numbers the
 * canonical (in, out) pair 1..25 (0 = free entry) and `big` is set once the count reached
 * 2^24: the word's count then stops and the rest is counted exactly in a side table (read only
 * by the raw-count copy-out; every other consumer caps at 65535).  A k-mer
 * with more distinct biedges than one slot holds continues in later slots of its probe
 * sequence, keyed k-mer | CONT.  After the filter the slot holds the graph node instead:
 *   word after the key: counts[0..3] (u16: out A C G T), then counts[4..7] (in A C G T),
 *   then counts[8] (self) | flags << 16 | aux << 32, aux = chain index.
 */
#pragma once

#include <cstdint>

namespace bg {

constexpr uint64_t KEY_EMPTY = ~0ull;          /* never claimed */
constexpr uint64_t KEY_TOMB = ~1ull;           /* removed (continuation or filtered-out node) */
constexpr uint64_t KEY_CONT = 1ull << 62;      /* continuation slot of a k-mer */
constexpr uint64_t KEY_DEAD_BIT = 1ull << 63;  /* set in EMPTY and TOMB only */

/* node flags (payload word 3, bits 16..31) */
constexpr uint32_t NF_BRANCH = 1u, NF_CHAIN = 2u;

struct KW1 { uint64_t v; };
struct KW2 { uint64_t lo, hi; };

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {  /* splitmix64 finaliser */
  x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27; x *= 0x94d049bb133111ebull;
  x ^= x >> 31; return x;
}

__device__ __forceinline__ uint64_t rev_pairs(uint64_t x) {
  x = __brevll(x);
  return ((x >> 1) & 0x5555555555555555ull) | ((x & 0x5555555555555555ull) << 1);
}

/* DNA16 complement = bit reversal of the nibble (A1<->T8, C2<->G4, gap 0). */
__device__ __forceinline__ unsigned comp16(unsigned n) {
  return ((n & 1u) << 3) | ((n & 2u) << 1) | ((n & 4u) >> 1) | ((n & 8u) >> 3);
}

template <class KT> struct KOps;

template <> struct KOps<KW1> {
  static constexpr int WORDS = 1;
  __device__ static __forceinline__ uint64_t mask(int k) { return (1ull << (2 * k)) - 1; }
  __device__ static __forceinline__ KW1 rc(KW1 x, int k) { return {rev_pairs(~x.v) >> (64 - 2 * k)}; }
  __device__ static __forceinline__ bool lt(KW1 a, KW1 b) { return a.v < b.v; }
  __device__ static __forceinline__ bool le(KW1 a, KW1 b) { return a.v <= b.v; }
  __device__ static __forceinline__ bool eq(KW1 a, KW1 b) { return a.v == b.v; }
  __device__ static __forceinline__ uint64_t hash(KW1 a) { return mix64(a.v); }
  __device__ static __forceinline__ KW1 append(KW1 x, unsigned c, int k) { return {((x.v << 2) | c) & mask(k)}; }
  __device__ static __forceinline__ KW1 prepend(unsigned c, KW1 x, int k) {
    return {(x.v >> 2) | ((uint64_t)c << (2 * (k - 1)))};
  }
  __device__ static __forceinline__ unsigned first(KW1 x, int k) { return (unsigned)(x.v >> (2 * (k - 1))) & 3u; }
  __device__ static __forceinline__ unsigned last(KW1 x) { return (unsigned)x.v & 3u; }
  /* the first k-1 bases (drop the last) and the last k-1 bases, as (k-1)-mers */
  __device__ static __forceinline__ KW1 head_km1(KW1 x) { return {x.v >> 2}; }
  __device__ static __forceinline__ KW1 tail_km1(KW1 x, int k) { return {x.v & mask(k - 1)}; }
  /* a k-mer from the packed base stream: `w` holds 2-bit bases MSB-first, 32 per word;
   * the k-mer starts at base index i (w[i/32] bit 63-2*(i%32)). */
  __device__ static __forceinline__ KW1 extract(const uint64_t *w, int i, int k) {
    int q = i >> 5, r = i & 31;
    uint64_t x = r ? ((w[q] << (2 * r)) | (w[q + 1] >> (64 - 2 * r))) : w[q];
    return {x >> (64 - 2 * k)};
  }
  /* base at index i counted from the last base (i = 0 is the last base) */
  __device__ static __forceinline__ unsigned base_lsb(KW1 x, int i) { return (unsigned)(x.v >> (2 * i)) & 3u; }
  __device__ static __forceinline__ void store(uint64_t *dst, KW1 x) { dst[0] = x.v; }
  __device__ static __forceinline__ KW1 load(const uint64_t *src) { return {src[0]}; }
};

template <> struct KOps<KW2> {
  static constexpr int WORDS = 2;
  __device__ static __forceinline__ uint64_t hmask(int k) { return (k >= 64) ? ~0ull : ((1ull << (2 * k - 64)) - 1); }
  __device__ static __forceinline__ KW2 shr(KW2 x, int s) {  /* 0 < s < 128 */
    if (s >= 64) return {x.hi >> (s - 64), 0};
    return {(x.lo >> s) | (x.hi << (64 - s)), x.hi >> s};
  }
  __device__ static __forceinline__ KW2 rc(KW2 x, int k) {
    KW2 y{rev_pairs(~x.hi), rev_pairs(~x.lo)};
    return shr(y, 128 - 2 * k);
  }
  __device__ static __forceinline__ bool lt(KW2 a, KW2 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
  __device__ static __forceinline__ bool le(KW2 a, KW2 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }
  __device__ static __forceinline__ bool eq(KW2 a, KW2 b) { return a.hi == b.hi && a.lo == b.lo; }
  __device__ static __forceinline__ uint64_t hash(KW2 a) { return mix64(a.lo ^ mix64(a.hi + 0x9e3779b97f4a7c15ull)); }
  /* (KW2_HC below is the same constant: kw2_lo inverts this hash for a given high word) */
  __device__ static __forceinline__ KW2 append(KW2 x, unsigned c, int k) {
    return {(x.lo << 2) | c, ((x.hi << 2) | (x.lo >> 62)) & hmask(k)};
  }
  __device__ static __forceinline__ KW2 prepend(unsigned c, KW2 x, int k) {
    KW2 y{(x.lo >> 2) | (x.hi << 62), x.hi >> 2};
    int pos = 2 * (k - 1);
    if (pos >= 64) y.hi |= (uint64_t)c << (pos - 64); else y.lo |= (uint64_t)c << pos;
    return y;
  }
  __device__ static __forceinline__ unsigned first(KW2 x, int k) {
    int pos = 2 * (k - 1);
    return (unsigned)((pos >= 64) ? (x.hi >> (pos - 64)) : (x.lo >> pos)) & 3u;
  }
  __device__ static __forceinline__ unsigned last(KW2 x) { return (unsigned)x.lo & 3u; }
  __device__ static __forceinline__ KW2 head_km1(KW2 x) { return shr(x, 2); }
  __device__ static __forceinline__ KW2 tail_km1(KW2 x, int k) {
    int b = 2 * (k - 1);  /* >= 62 */
    if (b >= 64) return {x.lo, x.hi & ((b - 64 == 0) ? 0ull : ((1ull << (b - 64)) - 1))};
    return {x.lo & ((1ull << b) - 1), 0};
  }
  __device__ static __forceinline__ KW2 extract(const uint64_t *w, int i, int k) {
    int q = i >> 5, r = i & 31;
    uint64_t a = w[q], b = w[q + 1], c = w[q + 2];
    KW2 x;
    if (r) { x.hi = (a << (2 * r)) | (b >> (64 - 2 * r)); x.lo = (b << (2 * r)) | (c >> (64 - 2 * r)); }
    else { x.hi = a; x.lo = b; }
    return shr(x, 128 - 2 * k);
  }
  __device__ static __forceinline__ unsigned base_lsb(KW2 x, int i) {
    return (unsigned)((i < 32) ? (x.lo >> (2 * i)) : (x.hi >> (2 * (i - 32)))) & 3u;
  }
  __device__ static __forceinline__ void store(uint64_t *dst, KW2 x) { dst[0] = x.lo; dst[1] = x.hi; }
  __device__ static __forceinline__ KW2 load(const uint64_t *src) { return {src[0], src[1]}; }
};

/* The (k-1)-mer rc-palindrome tests of kmer_traits.hpp:56-65 for odd k (for even k a
 * (k-1)-mer of DNA cannot be its own reverse complement). */
template <class KT>
__device__ __forceinline__ bool km1_high_palindrome(KT x, int k) {
  if ((k & 1) == 0) return false;
  KT h = KOps<KT>::head_km1(x);
  return KOps<KT>::eq(h, KOps<KT>::rc(h, k - 1));
}
template <class KT>
__device__ __forceinline__ bool km1_low_palindrome(KT x, int k) {
  if ((k & 1) == 0) return false;
  KT l = KOps<KT>::tail_km1(x, k);
  return KOps<KT>::eq(l, KOps<KT>::rc(l, k - 1));
}
/* kmer_traits::is_rc_palindrome (kmer_traits.hpp:68-71) */
template <class KT>
__device__ __forceinline__ bool k_palindrome(KT x, int k) {
  if (k & 1) return false;
  return KOps<KT>::eq(x, KOps<KT>::rc(x, k));
}

/* ---------------------------------------------------------------- table layout
 * The table is 2^pbits partitions of `region` slots; a key probes linearly inside its
 * partition.  For k <= 31 the position comes from a bijective mix of the 62-bit k-mer
 * (so an 8-byte record can carry the k-mer as mixed bits: partition bits implicit).  For
 * k > 31 it comes from H = mix64(lo ^ mix64(hi + c)), which for a given high word is a
 * bijection of the low word: a 16-byte record carries the high word and H without its top
 * (bucket) bits, and the low word is mix64_inv(H) ^ mix64(hi + c). */
constexpr uint64_t M62 = (1ull << 62) - 1;
constexpr uint64_t BJ_C1 = 0x3C79AC492BA7B653ull & M62;   /* odd */
constexpr uint64_t BJ_C2 = 0x1C69B3F74AC4AE35ull & M62;   /* odd */
__host__ __device__ constexpr uint64_t inv_odd64(uint64_t c) {
  /* inverse of an odd number modulo 2^64 by Newton iteration (also an inverse mod 2^62) */
  uint64_t x = c;
  for (int i = 0; i < 6; ++i) x *= 2 - c * x;
  return x;
}
constexpr uint64_t BJ_I1 = inv_odd64(BJ_C1), BJ_I2 = inv_odd64(BJ_C2);

__host__ __device__ __forceinline__ uint64_t bj_fwd(uint64_t x) {   /* 62-bit -> 62-bit bijection */
  x ^= x >> 31; x = (x * BJ_C1) & M62;
  x ^= x >> 29; x = (x * BJ_C2) & M62;
  x ^= x >> 32;
  return x;
}
__host__ __device__ __forceinline__ uint64_t xs_inv(uint64_t y, int s) {  /* inverse of y = x ^ (x >> s) */
  uint64_t x = y;
  for (int t = s; t < 62; t += s) x = y ^ (x >> s);
  return x;
}
__host__ __device__ __forceinline__ uint64_t bj_inv(uint64_t h) {
  uint64_t x = xs_inv(h, 32);
  x = (x * BJ_I2) & M62;
  x = xs_inv(x, 29);
  x = (x * BJ_I1) & M62;
  return xs_inv(x, 31);
}

/* inverse of mix64: each step of splitmix64's finaliser undone in reverse order */
__host__ __device__ __forceinline__ uint64_t xs_inv64(uint64_t y, int s) {  /* inverse of y = x ^ (x >> s) */
  uint64_t x = y;
  for (int t = s; t < 64; t += s) x = y ^ (x >> s);
  return x;
}
constexpr uint64_t MIX_I1 = inv_odd64(0xbf58476d1ce4e5b9ull), MIX_I2 = inv_odd64(0x94d049bb133111ebull);
__host__ __device__ __forceinline__ uint64_t mix64_inv(uint64_t x) {
  x = xs_inv64(x, 31); x *= MIX_I2;
  x = xs_inv64(x, 27); x *= MIX_I1;
  return xs_inv64(x, 30);
}
constexpr uint64_t KW2_HC = 0x9e3779b97f4a7c15ull;   /* the high word's offset in KOps<KW2>::hash */
/* the low word of a 128-bit key from its high word and its hash */
__host__ __device__ __forceinline__ uint64_t kw2_lo(uint64_t hi, uint64_t h) { return mix64_inv(h) ^ mix64(hi + KW2_HC); }

struct TableGeom {
  uint64_t nslots;   /* region << pbits */
  uint64_t region;
  int pbits;
  uint64_t base;     /* first slot: a sample's table in a batch of samples starts here (0 otherwise) */
};

/* The table stores a key derived from the canonical k-mer, so that counting records never
 * need inverting and the key itself gives the position: for k <= 31 the 62-bit mix
 * bj_fwd(k-mer); for k > 31 the pair (H, high word), H = KOps<KW2>::hash(k-mer) in the low word
 * (the high word keeps the k-mer's, whose two top bits stay free for the slot marks). */
__device__ __forceinline__ KW1 table_key(KW1 x) { return {bj_fwd(x.v)}; }
__device__ __forceinline__ KW2 table_key(KW2 x) { return {KOps<KW2>::hash(x), x.hi}; }
__device__ __forceinline__ KW1 key_kmer(KW1 t) { return {bj_inv(t.v)}; }
__device__ __forceinline__ KW2 key_kmer(KW2 t) { return {kw2_lo(t.hi, t.lo), t.hi}; }

/* home slot of a table key */
__device__ __forceinline__ uint64_t table_home(const TableGeom &g, KW1 t) {
  const uint64_t h = t.v;
  const uint64_t q = g.pbits ? (h >> (62 - g.pbits)) : 0;
  return g.base + q * g.region + __umul64hi(h << (2 + g.pbits), g.region);
}
__device__ __forceinline__ uint64_t table_home(const TableGeom &g, KW2 t) {
  const uint64_t h = t.lo;   /* the table key's low word is the hash */
  if (!g.pbits) return g.base + __umul64hi(h, g.region);
  return g.base + (h >> (64 - g.pbits)) * g.region + __umul64hi(h << g.pbits, g.region);
}
/* linear probing inside one partition */
struct Probe {
  uint64_t i, lo, hi;
  /* part_lo: the first slot of the partition if the caller knows it (saves a division) */
  __device__ __forceinline__ Probe(const TableGeom &g, uint64_t start, uint64_t part_lo = ~0ull) : i(start) {
    lo = part_lo != ~0ull ? part_lo : (g.pbits ? g.base + ((start - g.base) / g.region) * g.region : g.base);
    hi = lo + g.region;
  }
  __device__ __forceinline__ void next() { if (++i == hi) i = lo; }
};

/* ---------------------------------------------------------------- table slots */
template <class KT> struct Slot;

template <> struct Slot<KW1> {
  static constexpr int U64 = 4;       /* slot size in uint64 words */
  static constexpr int ENTRIES = 6;
  static constexpr int KEYW = 1;      /* key words */
};
template <> struct Slot<KW2> {
  static constexpr int U64 = 8;
  static constexpr int ENTRIES = 12;
  static constexpr int KEYW = 2;
};

/* biedge code <-> (in, out): 0 = no base, 1..4 = A C G T */
__device__ __forceinline__ unsigned biedge_code(unsigned in5, unsigned out5) { return in5 * 5u + out5 + 1u; }
__device__ __forceinline__ unsigned code_in5(unsigned code) { return (code - 1u) / 5u; }
__device__ __forceinline__ unsigned code_out5(unsigned code) { return (code - 1u) % 5u; }
/* DNA16 byte of a code: in base in the high nibble, out base in the low nibble */
__device__ __forceinline__ uint8_t code_biedge(unsigned code) {
  unsigned i = code_in5(code), o = code_out5(code);
  return (uint8_t)(((i ? (1u << (i - 1)) : 0u) << 4) | (o ? (1u << (o - 1)) : 0u));
}

/* entry words */
constexpr uint32_t E_BIG = 1u;
constexpr int E_CODE_SHIFT = 1;
constexpr int E_COUNT_SHIFT = 6;
constexpr uint32_t E_COUNT_BIG = 1u << 26;  /* stands for any count >= 2^24 where only a cap matters */
__device__ __forceinline__ unsigned entry_code(uint32_t e) { return (e >> E_CODE_SHIFT) & 31u; }
__device__ __forceinline__ uint32_t entry_count(uint32_t e) {
  return (e & E_BIG) ? E_COUNT_BIG : (e >> E_COUNT_SHIFT);
}

/* a whole slot in 32-byte loads */
template <int SU>
__device__ __forceinline__ void ld_slot(const uint64_t *slot, uint64_t *raw) {
  #pragma unroll
  for (int q = 0; q < SU; q += 4)
    asm volatile("ld.relaxed.gpu.global.v4.u64 {%0, %1, %2, %3}, [%4];"
                 : "=l"(raw[q]), "=l"(raw[q + 1]), "=l"(raw[q + 2]), "=l"(raw[q + 3])
                 : "l"(slot + q) : "memory");
}

/* slot key states */
__device__ __forceinline__ bool key_is_empty(KW1 k) { return k.v == KEY_EMPTY; }
__device__ __forceinline__ bool key_is_empty(KW2 k) { return k.hi == KEY_EMPTY && k.lo == KEY_EMPTY; }
__device__ __forceinline__ bool key_matches(KW1 k, KW1 want, bool cont) { return k.v == (want.v | (cont ? KEY_CONT : 0)); }
__device__ __forceinline__ bool key_matches(KW2 k, KW2 want, bool cont) {
  return k.lo == want.lo && k.hi == (want.hi | (cont ? KEY_CONT : 0));
}
__device__ __forceinline__ bool key_dead(KW1 k) { return (k.v & KEY_DEAD_BIT) != 0; }
__device__ __forceinline__ bool key_dead(KW2 k) { return (k.hi & KEY_DEAD_BIT) != 0; }
__device__ __forceinline__ bool key_cont(KW1 k) { return (k.v & KEY_CONT) != 0; }
__device__ __forceinline__ bool key_cont(KW2 k) { return (k.hi & KEY_CONT) != 0; }

/* After the filter a graph node's key carries KEY_NODE -- the continuation bit, free by then
 * because the filter folds every continuation slot into its k-mer's first slot -- and a k-mer
 * the filter dropped keeps its bare key, so dropping one costs no write.  Homes are always
 * computed from the bare key. */
constexpr uint64_t KEY_NODE = KEY_CONT;
__device__ __forceinline__ bool key_is_node(KW1 k) { return (k.v & (KEY_DEAD_BIT | KEY_NODE)) == KEY_NODE; }
__device__ __forceinline__ bool key_is_node(KW2 k) { return (k.hi & (KEY_DEAD_BIT | KEY_NODE)) == KEY_NODE; }
__device__ __forceinline__ KW1 node_key(KW1 k) { return {k.v & ~KEY_NODE}; }
__device__ __forceinline__ KW2 node_key(KW2 k) { return {k.lo, k.hi & ~KEY_NODE}; }
__device__ __forceinline__ KW1 as_node(KW1 k) { return {k.v | KEY_NODE}; }
__device__ __forceinline__ KW2 as_node(KW2 k) { return {k.lo, k.hi | KEY_NODE}; }

}  // namespace bg
