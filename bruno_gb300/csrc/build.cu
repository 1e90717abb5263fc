/*
 * build.cu -- FASTQ -> k-mer table -> graph nodes.
 *
 *  k_tile_stats / k_index_lines   FASTQ record split (4-line records, trailing blank lines
 *                                 ignored), one pass over the bytes each.
 *  k_hll                          HyperLogLog estimate of distinct canonical k-mers, used to
 *                                 size the table.
 *  k_count                        debruijn_kmer_simple_biedge_parser + lex_less +
 *                                 compute_biedge_freqencies: one warp per read packs the
 *                                 read to 2-bit words with ballots, every lane then cuts its
 *                                 k-mers out of the packed words, canonicalises them with the
 *                                 biedge and counts the pair in the k-mer's table slot.
 *  k_filter                       local_insert_by_freqencies: per k-mer, the (k+1)-mer sums,
 *                                 the per-entry flags, the compaction and the node update,
 *                                 all in registers; the node replaces the counts in place.
 *                                 IsBranchPoint / IsChainNode are decided in the same pass.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <mutex>

#include "table_plan.h"
#include "internal.cuh"

namespace bg {

namespace {

constexpr int TILE = 65536;          /* bytes per FASTQ tile */
constexpr int TPB = 256;

__device__ __forceinline__ int base_code(unsigned char c) {
  /* A/a 0, C/c 1, G/g 2, T/t 3, anything else (N, IUPAC, ...) -1 */
  switch (c | 0x20) {
    case 'a': return 0;
    case 'c': return 1;
    case 'g': return 2;
    case 't': return 3;
    default: return -1;
  }
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(~0u, v, o);
  return v;
}

/* block-wide exclusive prefix sum of one value per thread (blockDim.x == TPB); every
 * thread also receives the block total */
__device__ __forceinline__ uint32_t block_exscan(uint32_t v, uint32_t &total) {
  __shared__ uint32_t ws[TPB / 32 + 1];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(~0u, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int i = 0; i < TPB / 32; ++i) { uint32_t t = ws[i]; ws[i] = run; run += t; }
    ws[TPB / 32] = run;
  }
  __syncthreads();
  const uint32_t r = ws[w] + x - v;
  total = ws[TPB / 32];
  __syncthreads();
  return r;
}

/* ============================================================ FASTQ splitting */

/* per 4 bytes: 0x80 in every byte of w equal to that byte of c4, 0 elsewhere.  x = w ^ c4 is
 * zero exactly in those bytes; (x & 0x7F) + 0x7F keeps a byte's top bit clear only when its low
 * seven bits are zero and never carries into the next byte, and or-ing x itself in rules out
 * 0x80. */
__device__ __forceinline__ uint32_t bytes_eq(uint32_t w, uint32_t c4) {
  const uint32_t x = w ^ c4;
  return ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x | 0x7F7F7F7Fu);
}

/* 16 bytes at p (16-byte aligned if `aligned`, bounds-checked against n) as 4 words; a byte at
 * or past n reads as a carriage return, which the line scans skip as whitespace */
__device__ __forceinline__ uint4 load16(const unsigned char *buf, uint64_t p, uint64_t n, bool aligned) {
  if (aligned && p + 16 <= n) return *(const uint4 *)(buf + p);
  uint32_t w[4] = {0, 0, 0, 0};
  for (int i = 0; i < 16; ++i)
    w[i >> 2] |= (uint32_t)(p + i < n ? buf[p + i] : (unsigned char)'\r') << (8 * (i & 3));
  return make_uint4(w[0], w[1], w[2], w[3]);
}

/* newline count and last non-whitespace byte of each tile (16 bytes per thread-load) */
__global__ void __launch_bounds__(TPB, 8) k_tile_stats(const unsigned char *buf, uint64_t n, uint64_t *tile_cnt,
                                                     DevCounters *ctr, bool aligned) {
  const uint64_t t0 = (uint64_t)blockIdx.x * TILE;
  const uint64_t t1 = (n < t0 + TILE ? n : t0 + TILE);
  const uint32_t tl = (uint32_t)(t1 - t0);   /* the tile's bytes; offsets below are in the tile */
  /* newlines counted per byte lane of one word: a thread reads TILE / TPB bytes, so no lane
   * passes 255 */
  static_assert(TILE / TPB / 4 <= 255, "newline lane counts must fit a byte");
  uint32_t lanes = 0;
  uint32_t last_word = 0, last_keep = 0;   /* the thread's last word holding non-whitespace */
  /* four 16-byte loads in flight per thread, then their bytes */
  for (uint32_t o0 = 16u * threadIdx.x; o0 < tl; o0 += 64u * TPB) {
    uint4 v[4];
    #pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t o = o0 + 16u * TPB * u;
      v[u] = o < tl ? load16(buf, t0 + o, t1, aligned) : make_uint4(0u, 0u, 0u, 0u);
    }
    #pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t o = o0 + 16u * TPB * u;
      if (o >= tl) continue;
      const uint32_t w[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
      #pragma unroll
      for (int q = 0; q < 4; ++q) {
        /* bytes past the tile's end read as carriage returns: neither counted nor kept */
        const uint32_t nl = bytes_eq(w[q], 0x0A0A0A0Au), cr = bytes_eq(w[q], 0x0D0D0D0Du);
        lanes += nl >> 7;
        const uint32_t keep = ~(nl | cr) & 0x80808080u;
        /* a thread visits its bytes in increasing order, so its last hit is its largest */
        if (keep) { last_word = o + 4u * q; last_keep = keep; }
      }
    }
  }
  const uint32_t cnt = (lanes & 0xFFu) + ((lanes >> 8) & 0xFFu) + ((lanes >> 16) & 0xFFu) + (lanes >> 24);
  long long lastnw = last_keep ? (long long)(t0 + last_word + ((31 - __clz(last_keep)) >> 3)) : -1ll;
  __shared__ unsigned long long sc[TPB / 32];
  __shared__ long long sl[TPB / 32];
  const unsigned long long wcnt = warp_sum((unsigned long long)cnt);
  for (int o = 16; o > 0; o >>= 1) lastnw = max(lastnw, __shfl_down_sync(~0u, lastnw, o));
  if ((threadIdx.x & 31) == 0) { sc[threadIdx.x >> 5] = wcnt; sl[threadIdx.x >> 5] = lastnw; }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long c = 0; long long l = -1;
    for (int i = 0; i < TPB / 32; ++i) { c += sc[i]; l = max(l, sl[i]); }
    tile_cnt[blockIdx.x] = c;
    if (l >= 0) atomicMax(&ctr->last_nonws, l);
  }
}

/* Assigns a global line number to every newline and records each read's sequence span.
 * Line j ends at the j-th newline; records are lines 4r..4r+3 (header, sequence, '+',
 * quality).  Newlines after the last non-blank byte are trailing and ignored. */
__global__ void __launch_bounds__(TPB) k_index_lines(const unsigned char *buf, uint64_t n, const uint64_t *tile_base,
                                                      uint64_t *rstart, uint64_t *rend, uint64_t rbase,
                                                      uint64_t rcap, DevCounters *ctr, bool aligned) {
  const uint64_t t0 = (uint64_t)blockIdx.x * TILE;
  const uint64_t t1 = (n < t0 + TILE ? n : t0 + TILE);
  const long long E = ctr->last_nonws + 1;  /* effective end (exclusive) */
  uint64_t base = tile_base[blockIdx.x];
  unsigned long long nl_eff = 0;  /* newlines ending lines before E, max over this thread */
  if (blockIdx.x == 0 && threadIdx.x == 0 && E > 0 && buf[0] != '@') atomicMin(&ctr->bad_line, 0ull);
  /* stripes of TPB*64 bytes, 64 consecutive bytes per thread (four 16-byte loads in flight),
   * in byte order: one block scan per stripe */
  for (uint64_t s0 = t0; s0 < t1; s0 += (uint64_t)TPB * 64) {
    const uint64_t g0 = s0 + (uint64_t)threadIdx.x * 64;
    uint64_t m = 0;
    uint4 v[4];
    #pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint64_t p = g0 + 16ull * u;
      v[u] = p < t1 ? load16(buf, p, t1, aligned) : make_uint4(0u, 0u, 0u, 0u);
    }
    #pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t w[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
      #pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t nl = bytes_eq(w[q], 0x0A0A0A0Au) >> 7;   /* bit 8b per newline byte b */
        /* bits 0, 8, 16, 24 times 1 + 2^7 + 2^14 + 2^21 land on bits 21..24, and no two of the
         * sixteen products share a bit, so nothing carries into them */
        m |= (uint64_t)(((nl * 0x00204081u) >> 21) & 0xFu) << (16 * u + 4 * q);
      }
    }
    uint32_t total;
    const uint32_t rank = block_exscan((uint32_t)__popcll(m), total);
    uint64_t j = base + rank;
    while (m) {
      int i = __ffsll((long long)m) - 1;
      m &= m - 1;
      const uint64_t p = g0 + i;
      if ((long long)p < E) {
        const uint64_t ln = j;  /* this newline ends line ln */
        nl_eff = ln + 1;
        const uint64_t r = ln >> 2;
        const unsigned role = (unsigned)(ln & 3);
        if (role == 0 && rbase + r < rcap) rstart[rbase + r] = (uint64_t)(buf + p + 1);
        if (role == 1 && rbase + r < rcap) {
          uint64_t e = p;
          if (e > 0 && buf[e - 1] == '\r') --e;
          rend[rbase + r] = (uint64_t)(buf + e);
        }
        /* the first byte of line ln+1 */
        const unsigned nrole = (unsigned)((ln + 1) & 3);
        if (nrole == 0 || nrole == 2) {
          unsigned char c = ((long long)(p + 1) < E) ? buf[p + 1] : 0;
          if (c != (nrole == 0 ? '@' : '+')) atomicMin(&ctr->bad_line, (unsigned long long)(ln + 1));
        }
      }
      ++j;
    }
    base += total;
  }
  __shared__ unsigned long long snl[TPB / 32];
  for (int o = 16; o > 0; o >>= 1) nl_eff = max(nl_eff, __shfl_down_sync(~0u, nl_eff, o));
  if ((threadIdx.x & 31) == 0) snl[threadIdx.x >> 5] = nl_eff;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = 0;
    for (int i = 0; i < TPB / 32; ++i) m = max(m, snl[i]);
    if (m) atomicMax(&ctr->n_newlines_eff, m);
  }
}

/* ============================================================ k-mer extraction */

/* Per-warp staging of one chunk of a read as 2-bit words.  Chunk c covers k-mer start
 * positions [1024c, 1024c + 1024); word wi holds bases [1024c - 32 + 32wi, +32). */
constexpr int CHUNK_POS = 1024;
constexpr int CHUNK_WORDS = 40;  /* (32 + 1024 + 63 + 1) / 32 rounded up, plus 3 spare */

struct ReadView {
  const unsigned char *s;
  uint32_t L;
};

/* Loads the bases of chunk [p0, pend) plus flanks into words[]; returns true if any of
 * those bases is not A/C/G/T (the read must then be dropped). */
__device__ __forceinline__ bool stage_chunk(const ReadView &rv, uint32_t p0, uint32_t pend, int k, uint64_t *words,
                                            int lane) {
  bool bad = false;
  const long long c0 = (long long)p0 - 32;
  const long long cend = ((long long)rv.L < (long long)pend + k + 1) ? (long long)rv.L : (long long)pend + k + 1;
  const int nw = (int)((cend - c0 + 31) >> 5);
  for (int wi = 0; wi < nw; ++wi) {
    const long long c = c0 + 32 * wi + lane;
    unsigned code = 0;
    if (c >= 0 && c < (long long)rv.L) {
      const int bc = base_code(rv.s[c]);
      bad |= bc < 0;
      code = (unsigned)bc & 3u;
    }
    const unsigned m0 = __ballot_sync(~0u, code & 1u), m1 = __ballot_sync(~0u, code & 2u);
    if (lane == 0) {
      /* interleave: base i -> bits (62-2i, 63-2i), high bit from m1 */
      uint64_t z = 0;
      uint64_t a = m0, b = m1;
      a = (a | (a << 16)) & 0x0000FFFF0000FFFFull; a = (a | (a << 8)) & 0x00FF00FF00FF00FFull;
      a = (a | (a << 4)) & 0x0F0F0F0F0F0F0F0Full; a = (a | (a << 2)) & 0x3333333333333333ull;
      a = (a | (a << 1)) & 0x5555555555555555ull;
      b = (b | (b << 16)) & 0x0000FFFF0000FFFFull; b = (b | (b << 8)) & 0x00FF00FF00FF00FFull;
      b = (b | (b << 4)) & 0x0F0F0F0F0F0F0F0Full; b = (b | (b << 2)) & 0x3333333333333333ull;
      b = (b | (b << 1)) & 0x5555555555555555ull;
      z = (a << 1) | b;   /* bit 2i+1 = m0_i, bit 2i = m1_i */
      words[wi] = __brevll(z);
    }
  }
  if (lane < 3) words[nw + lane] = 0;
  __syncwarp();
  return __any_sync(~0u, bad);
}

__device__ __forceinline__ unsigned base_at(const uint64_t *w, int i) {
  return (unsigned)(w[i >> 5] >> (62 - 2 * (i & 31))) & 3u;
}

/* The k-mers of read positions [pc, e) of a staged chunk, cut into 32 contiguous runs
 * (one per lane).  Each lane extracts its first k-mer and its reverse complement once,
 * then rolls both one base at a time: fwd' = fwd.c, rc' = comp(c).rc without its last
 * base.  fn(valid, canonical k-mer, biedge code) is called in lock-step by the whole warp,
 * valid == false for lanes whose run is over. */
template <class KT, class F>
__device__ __forceinline__ void for_each_kmer_run(const uint64_t *words, uint32_t pc, uint32_t e, uint32_t p0,
                                                  uint32_t L, int k, int lane, F &&fn) {
  const uint32_t n = e - pc, r = (n + 31) >> 5;
  const uint32_t s = pc + lane * r, send = min(e, s + r);
  KT fwd{}, rev{};
  unsigned prev = 0;  /* base before the current k-mer */
  if (s < send) {
    const int lp = (int)(s - p0 + 32);
    fwd = KOps<KT>::extract(words, lp, k);
    rev = KOps<KT>::rc(fwd, k);
    prev = s > 0 ? base_at(words, lp - 1) : 0u;
  }
  for (uint32_t j = 0; j < r; ++j) {
    const uint32_t p = s + j;
    const bool valid = p < send;
    KT x{};
    unsigned code = 0, nb = 0;
    if (valid) {
      const bool has_out = p + k < L;
      nb = has_out ? base_at(words, (int)(p - p0 + 32) + k) : 0u;
      unsigned in5 = p > 0 ? prev + 1u : 0u, out5 = has_out ? nb + 1u : 0u;
      /* lex_less: keep if fwd < rc(fwd), else flip and reverse-complement the biedge */
      if (KOps<KT>::lt(fwd, rev)) {
        x = fwd;
      } else {
        x = rev;
        const unsigned ni = out5 ? 5u - out5 : 0u, no = in5 ? 5u - in5 : 0u;
        in5 = ni; out5 = no;
      }
      code = biedge_code(in5, out5);
    }
    fn(valid, x, code);
    if (valid) {
      prev = KOps<KT>::first(fwd, k);
      fwd = KOps<KT>::append(fwd, nb, k);
      rev = KOps<KT>::prepend(3u - nb, rev, k);
    }
  }
}

/* ============================================================ distinct estimate */

constexpr int HLL_P = 12;
constexpr int HLL_M = 1 << HLL_P;

template <class KT>
__global__ void __launch_bounds__(TPB) k_hll(const uint64_t *rstart, const uint64_t *rend, uint64_t nreads, int k,
                                              uint8_t *partial) {
  __shared__ uint64_t sw[TPB / 32][CHUNK_WORDS];
  __shared__ unsigned int reg[HLL_M];
  for (int i = threadIdx.x; i < HLL_M; i += TPB) reg[i] = 0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t *words = sw[warp];
  for (uint64_t r = (uint64_t)blockIdx.x * (TPB / 32) + warp; r < nreads; r += (uint64_t)gridDim.x * (TPB / 32)) {
    ReadView rv{(const unsigned char *)rstart[r], (uint32_t)(rend[r] - rstart[r])};
    if (rv.L < (uint32_t)k + 2) continue;
    const uint32_t npos = rv.L - k + 1;
    const bool one_chunk = npos <= CHUNK_POS;
    if (!one_chunk) {
      bool bad = false;
      for (uint32_t i = lane; i < rv.L; i += 32) bad |= base_code(rv.s[i]) < 0;
      if (__any_sync(~0u, bad)) continue;
    }
    for (uint32_t p0 = 0; p0 < npos; p0 += CHUNK_POS) {
      const uint32_t pend = min(npos, p0 + CHUNK_POS);
      __syncwarp();
      if (stage_chunk(rv, p0, pend, k, words, lane) && one_chunk) break;
      for_each_kmer_run<KT>(words, p0, pend, p0, rv.L, k, lane, [&](bool valid, KT x, unsigned) {
        if (!valid) return;
        const uint64_t h = KOps<KT>::hash(x);
        const unsigned idx = (unsigned)(h >> (64 - HLL_P));
        const unsigned rho = (unsigned)__clzll((h << HLL_P) | (1ull << (HLL_P - 1))) + 1u;
        if (rho > reg[idx]) atomicMax(&reg[idx], rho);
      });
    }
  }
  __syncthreads();
  uint8_t *dst = partial + (uint64_t)blockIdx.x * HLL_M;
  for (int i = threadIdx.x; i < HLL_M; i += TPB) dst[i] = (uint8_t)reg[i];
}

__global__ void k_hll_merge(const uint8_t *partial, int nblocks, DevCounters *ctr) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < HLL_M; i += gridDim.x * blockDim.x) {
    unsigned m = 0;
    for (int b = 0; b < nblocks; ++b) m = max(m, (unsigned)partial[(uint64_t)b * HLL_M + i]);
    ctr->hll[i] = m;
  }
}

/* ============================================================ counting */

struct CountArgs {
  const uint64_t *rstart, *rend;
  uint64_t nreads;
  int k;
  uint64_t *table;
  TableGeom g;
  uint32_t max_probe;
  DevCounters *ctr;
};



/* One more occurrence of the entry whose word lives at `key` (its address), in the exact
 * side table of counts past 2^24.  Every such entry needs 2^24 occurrences, so at most
 * n_instances / 2^24 of them exist: the table cannot fill below 2^34 instances. */
__device__ __forceinline__ void big_add(DevCounters *ctr, unsigned long long key) {
  unsigned h = (unsigned)mix64(key) & (BIG_SLOTS - 1);
  for (int p = 0; p < BIG_SLOTS; ++p, h = (h + 1) & (BIG_SLOTS - 1)) {
    const unsigned long long prev = atomicCAS(&ctr->big_key[h], 0ull, key);
    if (prev == 0ull) atomicAdd(&ctr->n_big, 1ull);
    if (prev == 0ull || prev == key) { atomicAdd(&ctr->big_cnt[h], 1ull); return; }
  }
  atomicOr(&ctr->err, (unsigned long long)DERR_INVARIANT);
}
__device__ __forceinline__ unsigned long long big_get(const DevCounters *ctr, unsigned long long key) {
  unsigned h = (unsigned)mix64(key) & (BIG_SLOTS - 1);
  for (int p = 0; p < BIG_SLOTS; ++p, h = (h + 1) & (BIG_SLOTS - 1)) {
    const unsigned long long k = ctr->big_key[h];
    if (k == key) return ctr->big_cnt[h];
    if (k == 0ull) return 0;
  }
  return 0;
}

/* after counting: every side-table entry resolved to (table key, biedge code, exact count) */
template <class KT>
__global__ void k_big_resolve(const uint64_t *table, const DevCounters *ctr, BigRes *out,
                              unsigned long long *n_out) {
  constexpr int SU = Slot<KT>::U64, KWD = Slot<KT>::KEYW;
  for (int h = threadIdx.x; h < BIG_SLOTS; h += blockDim.x) {
    const unsigned long long key = ctr->big_key[h];
    if (key == 0ull) continue;
    const uint64_t off = (uint64_t)(key - (unsigned long long)(uintptr_t)table);   /* bytes into the table */
    const uint64_t *slot = table + (off / (SU * 8)) * SU;
    const uint32_t w = *(const uint32_t *)(uintptr_t)key;
    BigRes r;
    r.k0 = slot[0];
    r.k1 = KWD == 2 ? slot[1] : 0ull;
    if (KWD == 1) r.k0 &= ~KEY_CONT; else r.k1 &= ~KEY_CONT;
    r.code = entry_code(w);
    r.pad = 0;
    r.count = (unsigned long long)(w >> E_COUNT_SHIFT) + ctr->big_cnt[h];
    out[atomicAdd(n_out, 1ull)] = r;
  }
}

/* One count into the entry words e[0..n) of a slot whose current contents were read into
 * `seen`.  Returns true when counted, false when every entry holds another biedge (slot
 * full).  A free entry is claimed with CAS; a stale free entry (claimed since the read)
 * shows up as a failed CAS returning the claimer's word.  Increments are fire-and-forget
 * while the count seen is below 2^24; from there on the entry word keeps its count (at most
 * 2^24 plus the increments in flight, far below the 26-bit field's limit), carries E_BIG, and
 * every further occurrence is counted exactly in the side table, so that the raw (k+2)-mer
 * counts stay exact to 32 bits like the reference's uint32 K2FreqType. */
template <int NE>
__device__ __forceinline__ bool count_in_entries(uint32_t *e, const uint32_t *seen, unsigned code,
                                                 unsigned long long &claims, DevCounters *ctr) {
  #pragma unroll
  for (int i = 0; i < NE; ++i) {
    uint32_t w = seen[i];
    if (w == 0) {
      const uint32_t nw = (code << E_CODE_SHIFT) | (1u << E_COUNT_SHIFT);
      const uint32_t old = atomicCAS(e + i, 0u, nw);
      if (old == 0) { ++claims; return true; }
      w = old;
    }
    if (entry_code(w) == code) {
      if ((w >> E_COUNT_SHIFT) < (1u << 24) && !(w & E_BIG)) {
        atomicAdd(e + i, 1u << E_COUNT_SHIFT);          /* result unused: a reduction */
      } else {
        if (!(w & E_BIG)) atomicOr(e + i, E_BIG);
        big_add(ctr, (unsigned long long)(uintptr_t)(e + i));
      }
      return true;
    }
  }
  return false;
}

/* 128-bit CAS on global memory (KW2 keys: lo, hi with the slot marks in hi) */
__device__ __forceinline__ unsigned long long cas128(uint64_t *addr, uint64_t cmp_lo, uint64_t cmp_hi, uint64_t new_lo,
                                                     uint64_t new_hi, uint64_t &old_hi) {
  unsigned long long olo, ohi;
  asm volatile(
      "{\n\t.reg .b128 d, b, c;\n\t"
      "mov.b128 b, {%2, %3};\n\t"
      "mov.b128 c, {%4, %5};\n\t"
      "atom.global.cas.b128 d, [%6], b, c;\n\t"
      "mov.b128 {%0, %1}, d;\n\t}"
      : "=l"(olo), "=l"(ohi)
      : "l"(cmp_lo), "l"(cmp_hi), "l"(new_lo), "l"(new_hi), "l"(addr)
      : "memory");
  old_hi = ohi;
  return olo;
}

/* claims a KW2 key (both words in one 128-bit CAS) */
__device__ __forceinline__ bool key_claim(KW2, uint64_t *slot, KW2 want, bool cont, KW2 &seen, bool &was_empty) {
  const uint64_t nhi = want.hi | (cont ? KEY_CONT : 0);
  uint64_t ohi;
  const uint64_t olo = cas128(slot, KEY_EMPTY, KEY_EMPTY, want.lo, nhi, ohi);
  was_empty = (olo == KEY_EMPTY && ohi == KEY_EMPTY);
  seen = was_empty ? KW2{want.lo, nhi} : KW2{olo, ohi};
  return was_empty;
}

/* Counts one canonical (k-mer, biedge code) occurrence whose first probe slot `i` was
 * already read into raw[].  Returns false if the probe limit was reached. */
template <class KT>
__device__ __forceinline__ bool table_count(uint64_t *table, const TableGeom &g, uint32_t max_probe, KT x,
                                            unsigned code, uint64_t home, uint64_t *raw,
                                            unsigned long long &slot_claims, unsigned long long &entry_claims,
                                            DevCounters *ctr, uint64_t part_lo = ~0ull) {
  constexpr int SU = Slot<KT>::U64, NE = Slot<KT>::ENTRIES, KWD = Slot<KT>::KEYW;
  bool seen_primary = false;
  Probe pr(g, home, part_lo);
  for (uint32_t probe = 0; probe < max_probe; ++probe, pr.next()) {
    uint64_t *slot = table + pr.i * SU;
    if (probe) ld_slot<SU>(slot, raw);
    KT key = KOps<KT>::load(raw);
    uint32_t seen[NE];
    #pragma unroll
    for (int q = 0; q < NE; ++q) seen[q] = (uint32_t)(raw[KWD + q / 2] >> (32 * (q & 1)));
    if (key_is_empty(key)) {
      if constexpr (KWD == 1) {
        /* claim the key and its first entry together: one 128-bit CAS of (key, entries 0-1)
         * from (EMPTY, 0) -- the entries of an unclaimed slot are always zero */
        const uint64_t nk = ((const uint64_t *)&x)[0] | (seen_primary ? KEY_CONT : 0);
        const uint64_t ne0 = (uint64_t)((code << E_CODE_SHIFT) | (1u << E_COUNT_SHIFT));
        uint64_t ohi;
        const uint64_t olo = cas128(slot, KEY_EMPTY, 0ull, nk, ne0, ohi);
        if (olo == KEY_EMPTY && ohi == 0) { ++slot_claims; ++entry_claims; return true; }
        ((uint64_t *)&key)[0] = olo;          /* claimed meanwhile: count against what is there */
        seen[0] = (uint32_t)ohi;
        seen[1] = (uint32_t)(ohi >> 32);
      } else {
        bool was_empty;
        key_claim(KT{}, slot, x, seen_primary, key, was_empty);
        if (was_empty) ++slot_claims;
      }
    }
    if (key_matches(key, x, seen_primary)) {
      seen_primary = true;
      if (count_in_entries<NE>((uint32_t *)(slot + KWD), seen, code, entry_claims, ctr)) return true;
    }
  }
  return false;
}

/* the canonical (k-mer, biedge code) at read position p of a staged chunk */
template <class KT>
__device__ __forceinline__ void kmer_at(const uint64_t *words, uint32_t p, uint32_t p0, uint32_t L, int k, KT &x,
                                        unsigned &code) {
  const int lp = (int)(p - p0 + 32);
  x = KOps<KT>::extract(words, lp, k);
  /* biedge in DNA: base before and after the k-mer in the read (0 = read end) */
  unsigned in5 = (p > 0) ? base_at(words, lp - 1) + 1u : 0u;
  unsigned out5 = (p + k < L) ? base_at(words, lp + k) + 1u : 0u;
  /* lex_less: keep if x < rc(x), else flip the k-mer and reverse-complement the biedge
   * (in' = comp(out), out' = comp(in); comp of a DNA code c is 3-c) */
  KT y = KOps<KT>::rc(x, k);
  if (!KOps<KT>::lt(x, y)) {
    x = y;
    const unsigned ni = out5 ? 5u - out5 : 0u, no = in5 ? 5u - in5 : 0u;
    in5 = ni; out5 = no;
  }
  code = biedge_code(in5, out5);
}

template <class KT>
__global__ void __launch_bounds__(TPB, 4) k_count(CountArgs a) {
  constexpr int SU = Slot<KT>::U64;
  __shared__ uint64_t sw[TPB / 32][CHUNK_WORDS];
  __shared__ unsigned long long s_inst, s_used, s_slots, s_entries;
  __shared__ int s_full;
  if (threadIdx.x == 0) { s_inst = s_used = s_slots = s_entries = 0; s_full = 0; }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = a.k;
  uint64_t *words = sw[warp];
  unsigned long long inst = 0, used = 0, slots = 0, entries = 0;
  bool full = false;
  for (uint64_t r = (uint64_t)blockIdx.x * (TPB / 32) + warp; r < a.nreads; r += (uint64_t)gridDim.x * (TPB / 32)) {
    ReadView rv{(const unsigned char *)a.rstart[r], (uint32_t)(a.rend[r] - a.rstart[r])};
    if (rv.L < (uint32_t)k + 2) continue;          /* shorter than the k+2 window */
    const uint32_t npos = rv.L - k + 1;
    const bool one_chunk = npos <= CHUNK_POS;
    if (!one_chunk) {                               /* long read: N filter first */
      bool bad = false;
      for (uint32_t i = lane; i < rv.L; i += 32) bad |= base_code(rv.s[i]) < 0;
      if (__any_sync(~0u, bad)) continue;
    }
    for (uint32_t p0 = 0; p0 < npos; p0 += CHUNK_POS) {
      const uint32_t pend = min(npos, p0 + CHUNK_POS);
      __syncwarp();
      if (stage_chunk(rv, p0, pend, k, words, lane) && one_chunk) break;   /* reads with N are dropped */
      if (p0 == 0) used += (lane == 0);
      /* two k-mers per lane in flight: both first-probe slots are read before either is used */
      for (uint32_t pb = p0; pb < pend; pb += 64) {
        const uint32_t pa = pb + lane, pc = pb + 32 + lane;
        KT xa{}, xc{};
        unsigned ca = 0, cc = 0;
        uint64_t ia = 0, ic = 0, ra[SU], rc[SU];
        if (pa < pend) {
          kmer_at<KT>(words, pa, p0, rv.L, k, xa, ca);
          xa = table_key(xa);
          ia = table_home(a.g, xa);
          ld_slot<SU>(a.table + ia * SU, ra);
        }
        if (pc < pend) {
          kmer_at<KT>(words, pc, p0, rv.L, k, xc, cc);
          xc = table_key(xc);
          ic = table_home(a.g, xc);
          ld_slot<SU>(a.table + ic * SU, rc);
        }
        if (pa < pend) {
          ++inst;
          if (!table_count<KT>(a.table, a.g, a.max_probe, xa, ca, ia, ra, slots, entries, a.ctr)) full = true;
        }
        if (pc < pend) {
          ++inst;
          if (!table_count<KT>(a.table, a.g, a.max_probe, xc, cc, ic, rc, slots, entries, a.ctr)) full = true;
        }
      }
    }
  }
  inst = warp_sum(inst); used = warp_sum(used); slots = warp_sum(slots); entries = warp_sum(entries);
  if (lane == 0) {
    atomicAdd(&s_inst, inst); atomicAdd(&s_used, used); atomicAdd(&s_slots, slots); atomicAdd(&s_entries, entries);
  }
  if (full) s_full = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&a.ctr->n_instances, s_inst); atomicAdd(&a.ctr->n_reads_used, s_used);
    atomicAdd(&a.ctr->n_slots_claimed, s_slots); atomicAdd(&a.ctr->n_entries, s_entries);
    if (s_full) atomicOr(&a.ctr->err, (unsigned long long)DERR_TABLE_FULL);
  }
}

/* ============================================================ partitioned counting
 * k <= 31.  Phase A (k_extract) turns every read into canonical (k-mer, biedge) instances
 * and writes each as one 8-byte record [low 54 bits of bj_fwd(k-mer) | biedge code:5]
 * into one of 256 hash buckets (the bucket is the top 8 bits of the mix); the block queues
 * its records by bucket in shared memory first, so every bucket grows by contiguous runs.
 * The distinct-count estimate rides along.  Phase B (k_insert) then fills the table one
 * partition at a time -- a partition is one or more buckets and a contiguous slot region
 * small enough to stay in L2 -- so the random slot traffic of counting stays on chip. */
constexpr int NBUCKET_BITS = 8, NBUCKET = 1 << NBUCKET_BITS;
constexpr int LOW_BITS = 62 - NBUCKET_BITS;          /* 54 */
__global__ void __launch_bounds__(TPB) k_kmer_upper(const uint64_t *rstart, const uint64_t *rend, uint64_t nreads,
                                                     int k, DevCounters *ctr) {
  unsigned long long n = 0;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nreads; r += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t L = rend[r] - rstart[r];
    if (L >= (uint64_t)k + 2) n += L - k + 1;
  }
  n = warp_sum(n);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(&ctr->n_upper, n);
}

/* Phase A runs one thread per read: each thread validates its read (any base that is not
 * A/C/G/T, either case, drops the read), then rolls the forward k-mer and its reverse
 * complement through the read one base at a time, so every k-mer costs a handful of
 * integer operations.  Records go to per-bucket shared-memory queues; after every round of
 * XROUND records per thread the block appends each queue to its bucket with one atomic. */
constexpr int XTPB = 512;                  /* threads per block */
constexpr int XROUND = 8;                  /* records per thread between two flushes */
constexpr int XQ = 32;                     /* queue capacity per bucket (mean fill 16) */

struct ExtractSmem {
  uint64_t q[NBUCKET][XQ];
  unsigned int hll[HLL_M];
  unsigned int cnt[NBUCKET];
  unsigned long long base[NBUCKET];   /* this flush: first `rem` records from base, the rest from base2 */
  unsigned long long base2[NBUCKET];
  unsigned int rem[NBUCKET];
  unsigned long long cpos[NBUCKET], cend[NBUCKET];   /* the block's current chunk of each bucket */
  int overflow;
};

/* bytes of one read's sequence through aligned 8-byte loads; no load goes past the word
 * that holds the last base, so nothing outside the read's own line is touched beyond its
 * last word */
struct SeqCursor {
  const uint64_t *w, *wlast;
  uint64_t cur, nxt;
  int left;
  __device__ __forceinline__ void init(const unsigned char *s, const unsigned char *e) {
    const uint64_t *w0 = (const uint64_t *)((uintptr_t)s & ~(uintptr_t)7);
    wlast = (const uint64_t *)((uintptr_t)(e - 1) & ~(uintptr_t)7);
    const int off = (int)((uintptr_t)s & 7);
    cur = __ldg(w0) >> (8 * off);
    left = 8 - off;
    w = w0 + 1;
    nxt = w <= wlast ? __ldg(w) : 0ull;
  }
  __device__ __forceinline__ unsigned next() {
    if (left == 0) {
      cur = nxt; left = 8; ++w;
      nxt = w <= wlast ? __ldg(w) : 0ull;
    }
    const unsigned b = (unsigned)cur & 0xFFu;
    cur >>= 8; --left;
    return b;
  }
};

/* true if every byte of [s, e) is A, C, G or T in either case */
__device__ __forceinline__ bool seq_valid(const unsigned char *s, const unsigned char *e) {
  const uintptr_t a0 = (uintptr_t)s & ~(uintptr_t)7, a1 = (uintptr_t)e;
  bool ok = true;
  for (uintptr_t a = a0; a < a1 && ok; a += 8) {
    const uint64_t x = __ldg((const uint64_t *)a) | 0x2020202020202020ull;
    /* bytes of this word that belong to the read */
    const int lo = a < (uintptr_t)s ? (int)((uintptr_t)s - a) : 0;
    const int hi = a + 8 > a1 ? (int)(a1 - a) : 8;
    const uint64_t in = (hi == 8 ? ~0ull : ((1ull << (8 * hi)) - 1)) & (~0ull << (8 * lo));
    uint32_t v[2];
    #pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t y = (uint32_t)(x >> (32 * h));
      v[h] = __vcmpeq4(y, 0x61616161u) | __vcmpeq4(y, 0x63636363u) | __vcmpeq4(y, 0x67676767u) |
             __vcmpeq4(y, 0x74747474u);
    }
    const uint64_t good = (uint64_t)v[0] | ((uint64_t)v[1] << 32);
    ok = (good & in) == in;
  }
  return ok;
}

/* ------------------------------------------------ the (k+1)-mer edge filter
 * The blocked driver's build_index_thresholded (compact_debruijn_graph_block_construct.cpp:
 * 417-470): compute_edge_frequency (debruijn_biedge_filters.hpp:128-177) counts every
 * canonical (k+1)-mer of the N-filtered reads at least k+1 long in a saturating uint16
 * counter and erases those outside [lo, hi); transform_biedges_by_frequency (:331-423)
 * clears every biedge edge whose (k+1)-mer is gone and filter_isolated_nodes (:66-75) drops
 * pairs left without edges; the rest are inserted unthresholded.  The (k+1)-mers (k <= 31,
 * so at most 64 bits) live in an open-addressing table of (key, count) slots keyed by the
 * canonical (k+1)-mer itself: all ones and all ones but the lowest bit are never canonical
 * (their reverse complements are smaller), so they mark empty and erased slots. */
constexpr uint64_t K1_EMPTY = ~0ull, K1_TOMB = ~1ull;

struct K1Roll {   /* forward and reverse-complement (k+1)-mer of a read, base by base */
  uint64_t fw = 0, rv = 0, mask;
  int top;
  __device__ __forceinline__ explicit K1Roll(int k1) : mask(k1 == 32 ? ~0ull : ((1ull << (2 * k1)) - 1)), top(2 * k1 - 2) {}
  __device__ __forceinline__ uint64_t push(unsigned c) {   /* the canonical (k+1)-mer ending here */
    fw = ((fw << 2) | c) & mask;
    rv = (rv >> 2) | ((uint64_t)(3u - c) << top);
    return fw < rv ? fw : rv;
  }
};

__device__ __forceinline__ uint64_t k1_home(uint64_t x, uint64_t nslots) { return __umul64hi(mix64(x), nslots); }

/* true if the (k+1)-mer x is in the table (erased slots are stepped over) */
__device__ __forceinline__ bool k1_exists(const uint64_t *tab, uint64_t nslots, uint64_t x) {
  uint64_t i = k1_home(x, nslots);
  for (uint64_t p = 0; p < nslots; ++p) {
    const uint64_t key = __ldg(tab + 2 * i);
    if (key == x) return true;
    if (key == K1_EMPTY) return false;
    if (++i == nslots) i = 0;
  }
  return false;
}

/* distinct (k+1)-mer estimate: HyperLogLog registers per block */
__global__ void __launch_bounds__(TPB) k_k1_hll(const uint64_t *rstart, const uint64_t *rend, uint64_t nreads, int k,
                                                 uint8_t *partial) {
  __shared__ unsigned int reg[HLL_M];
  for (int i = threadIdx.x; i < HLL_M; i += TPB) reg[i] = 0;
  __syncthreads();
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nreads; r += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned char *s = (const unsigned char *)rstart[r], *e = (const unsigned char *)rend[r];
    const uint32_t L = (uint32_t)(e - s);
    if (L < (uint32_t)k + 1 || !seq_valid(s, e)) continue;
    SeqCursor sc;
    sc.init(s, e);
    K1Roll roll(k + 1);
    for (uint32_t i = 0; i < L; ++i) {
      const unsigned byte = sc.next();
      const uint64_t x = roll.push(((byte >> 1) ^ (byte >> 2)) & 3u);
      if (i < (uint32_t)k) continue;
      const uint64_t h = mix64(x);
      const unsigned idx = (unsigned)(h >> (64 - HLL_P));
      const unsigned rho = (unsigned)__clzll((h << HLL_P) | (1ull << (HLL_P - 1))) + 1u;
      if (rho > reg[idx]) atomicMax(&reg[idx], rho);
    }
  }
  __syncthreads();
  uint8_t *dst = partial + (uint64_t)blockIdx.x * HLL_M;
  for (int i = threadIdx.x; i < HLL_M; i += TPB) dst[i] = (uint8_t)reg[i];
}

/* count every (k+1)-mer; a probe run longer than max_probe reports a full table */
__global__ void __launch_bounds__(TPB) k_k1_count(const uint64_t *rstart, const uint64_t *rend, uint64_t nreads, int k,
                                                   uint64_t *tab, uint64_t nslots, uint32_t max_probe,
                                                   DevCounters *ctr) {
  bool full = false;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nreads; r += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned char *s = (const unsigned char *)rstart[r], *e = (const unsigned char *)rend[r];
    const uint32_t L = (uint32_t)(e - s);
    if (L < (uint32_t)k + 1 || !seq_valid(s, e)) continue;
    SeqCursor sc;
    sc.init(s, e);
    K1Roll roll(k + 1);
    for (uint32_t i = 0; i < L; ++i) {
      const unsigned byte = sc.next();
      const uint64_t x = roll.push(((byte >> 1) ^ (byte >> 2)) & 3u);
      if (i < (uint32_t)k) continue;
      uint64_t j = k1_home(x, nslots);
      bool done = false;
      for (uint32_t p = 0; p < max_probe && !done; ++p) {
        unsigned long long *slot = (unsigned long long *)(tab + 2 * j);
        unsigned long long key = *(volatile unsigned long long *)slot;
        if (key == K1_EMPTY) key = atomicCAS(slot, K1_EMPTY, (unsigned long long)x);
        if (key == K1_EMPTY || key == x) { atomicAdd(slot + 1, 1ull); done = true; }
        else if (++j == nslots) j = 0;
      }
      full |= !done;
    }
  }
  if (full) atomicOr(&ctr->err, (unsigned long long)DERR_TABLE_FULL);
}

__global__ void k_k1_init(uint64_t *tab, uint64_t nslots) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 2 * nslots; i += (uint64_t)gridDim.x * blockDim.x)
    tab[i] = (i & 1) ? 0ull : K1_EMPTY;
}

/* erase the (k+1)-mers whose saturated count lies outside [lo, hi) */
__global__ void __launch_bounds__(TPB) k_k1_threshold(uint64_t *tab, uint64_t nslots, uint64_t lo, uint64_t hi) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += (uint64_t)gridDim.x * blockDim.x) {
    if (tab[2 * i] == K1_EMPTY) continue;
    const uint64_t c = min(tab[2 * i + 1], (uint64_t)0xFFFFu);
    if (c < lo || c >= hi) tab[2 * i] = K1_TOMB;
  }
}

/* The same (k+1)-mer table for k > 31: (k+1)-mers of 33..64 bases as 128-bit keys (KW2 packing)
 * in 32-byte slots [lo, hi, count, 0].  Both words all ones mark an empty slot and (all ones
 * but the lowest bit, all ones) an erased one: neither is canonical (at 64 bases their reverse
 * complements are smaller; below, the high word has bits past the k-mer). */
constexpr uint64_t K1W_TOMB_LO = ~1ull;

struct K1Roll2 {   /* forward and reverse-complement (k+1)-mer of a read, 128-bit */
  KW2 fw{0, 0}, rv{0, 0};
  int k1;
  __device__ __forceinline__ explicit K1Roll2(int k1_) : k1(k1_) {}
  __device__ __forceinline__ KW2 push(unsigned c) {   /* the canonical (k+1)-mer ending here */
    fw = KOps<KW2>::append(fw, c, k1);
    rv = KOps<KW2>::prepend(3u - c, rv, k1);
    return KOps<KW2>::lt(fw, rv) ? fw : rv;
  }
};

__device__ __forceinline__ uint64_t k1w_home(KW2 x, uint64_t nslots) { return __umul64hi(KOps<KW2>::hash(x), nslots); }

/* true if the 128-bit (k+1)-mer x is in the table (erased slots are stepped over) */
__device__ __forceinline__ bool k1w_exists(const uint64_t *tab, uint64_t nslots, KW2 x) {
  uint64_t i = k1w_home(x, nslots);
  for (uint64_t p = 0; p < nslots; ++p) {
    const ulonglong2 key = __ldg(reinterpret_cast<const ulonglong2 *>(tab + 4 * i));
    if (key.x == x.lo && key.y == x.hi) return true;
    if (key.x == KEY_EMPTY && key.y == KEY_EMPTY) return false;
    if (++i == nslots) i = 0;
  }
  return false;
}

__global__ void __launch_bounds__(TPB) k_k1w_hll(const uint64_t *rstart, const uint64_t *rend, uint64_t nreads, int k,
                                                  uint8_t *partial) {
  __shared__ unsigned int reg[HLL_M];
  for (int i = threadIdx.x; i < HLL_M; i += TPB) reg[i] = 0;
  __syncthreads();
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nreads; r += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned char *s = (const unsigned char *)rstart[r], *e = (const unsigned char *)rend[r];
    const uint32_t L = (uint32_t)(e - s);
    if (L < (uint32_t)k + 1 || !seq_valid(s, e)) continue;
    SeqCursor sc;
    sc.init(s, e);
    K1Roll2 roll(k + 1);
    for (uint32_t i = 0; i < L; ++i) {
      const unsigned byte = sc.next();
      const KW2 x = roll.push(((byte >> 1) ^ (byte >> 2)) & 3u);
      if (i < (uint32_t)k) continue;
      const uint64_t h = KOps<KW2>::hash(x);
      const unsigned idx = (unsigned)(h >> (64 - HLL_P));
      const unsigned rho = (unsigned)__clzll((h << HLL_P) | (1ull << (HLL_P - 1))) + 1u;
      if (rho > reg[idx]) atomicMax(&reg[idx], rho);
    }
  }
  __syncthreads();
  uint8_t *dst = partial + (uint64_t)blockIdx.x * HLL_M;
  for (int i = threadIdx.x; i < HLL_M; i += TPB) dst[i] = (uint8_t)reg[i];
}

__global__ void __launch_bounds__(TPB) k_k1w_count(const uint64_t *rstart, const uint64_t *rend, uint64_t nreads, int k,
                                                    uint64_t *tab, uint64_t nslots, uint32_t max_probe,
                                                    DevCounters *ctr) {
  bool full = false;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nreads; r += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned char *s = (const unsigned char *)rstart[r], *e = (const unsigned char *)rend[r];
    const uint32_t L = (uint32_t)(e - s);
    if (L < (uint32_t)k + 1 || !seq_valid(s, e)) continue;
    SeqCursor sc;
    sc.init(s, e);
    K1Roll2 roll(k + 1);
    for (uint32_t i = 0; i < L; ++i) {
      const unsigned byte = sc.next();
      const KW2 x = roll.push(((byte >> 1) ^ (byte >> 2)) & 3u);
      if (i < (uint32_t)k) continue;
      uint64_t j = k1w_home(x, nslots);
      bool done = false;
      for (uint32_t p = 0; p < max_probe && !done; ++p) {
        uint64_t *slot = tab + 4 * j;
        /* one 16-byte load: a key is claimed by one 128-bit CAS, so it is seen whole or empty */
        uint64_t klo, khi;
        asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(klo), "=l"(khi) : "l"(slot) : "memory");
        if (klo == KEY_EMPTY && khi == KEY_EMPTY) klo = cas128(slot, KEY_EMPTY, KEY_EMPTY, x.lo, x.hi, khi);
        if ((klo == KEY_EMPTY && khi == KEY_EMPTY) || (klo == x.lo && khi == x.hi)) {
          atomicAdd((unsigned long long *)(slot + 2), 1ull);
          done = true;
        } else if (++j == nslots) {
          j = 0;
        }
      }
      full |= !done;
    }
  }
  if (full) atomicOr(&ctr->err, (unsigned long long)DERR_TABLE_FULL);
}

__global__ void k_k1w_init(uint64_t *tab, uint64_t nslots) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 4 * nslots; i += (uint64_t)gridDim.x * blockDim.x)
    tab[i] = (i & 3) < 2 ? KEY_EMPTY : 0ull;
}

/* erase the 128-bit (k+1)-mers whose saturated count lies outside [lo, hi) */
__global__ void __launch_bounds__(TPB) k_k1w_threshold(uint64_t *tab, uint64_t nslots, uint64_t lo, uint64_t hi) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += (uint64_t)gridDim.x * blockDim.x) {
    if (tab[4 * i] == KEY_EMPTY && tab[4 * i + 1] == KEY_EMPTY) continue;
    const uint64_t c = min(tab[4 * i + 2], (uint64_t)0xFFFFu);
    if (c < lo || c >= hi) { tab[4 * i] = K1W_TOMB_LO; tab[4 * i + 1] = KEY_EMPTY; }
  }
}

/* EF: the (k+1)-mer edge filter above -- each edge whose (k+1)-mer is not in k1tab is cleared
 * and a pair without edges is not emitted; a read's (k+1)-mer at each position is looked up
 * once, as the out edge of one k-mer and the in edge of the next */
template <bool EF>
__global__ void __launch_bounds__(XTPB, 2) k_extract(const uint64_t *rstart, const uint64_t *rend, uint64_t nreads,
                                                      int k, uint64_t *records, uint64_t cap,
                                                      unsigned long long *bucket_cnt, uint8_t *hll_partial,
                                                      const uint64_t *k1tab, uint64_t k1slots, uint32_t chunk,
                                                      DevCounters *ctr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ExtractSmem &S = *reinterpret_cast<ExtractSmem *>(smem_raw);
  const int tid = threadIdx.x;
  for (int i = tid; i < HLL_M; i += XTPB) S.hll[i] = 0;
  for (int i = tid; i < NBUCKET; i += XTPB) { S.cnt[i] = 0; S.cpos[i] = 0; S.cend[i] = 0; }
  if (tid == 0) S.overflow = 0;
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * XTPB;
  const uint64_t kmask = (k == 32) ? ~0ull : ((1ull << (2 * k)) - 1);
  const int top = 2 * k - 2;
  uint64_t r = (uint64_t)blockIdx.x * XTPB + tid;
  unsigned long long inst = 0, used = 0;
  SeqCursor sc;
  uint32_t L = 0, i = 0;
  uint64_t fwd = 0, rev = 0;
  unsigned left = 0;
  /* advance to the next usable read of this thread */
  auto next_read = [&]() -> bool {
    for (; r < nreads; r += stride) {
      const unsigned char *s = (const unsigned char *)rstart[r], *e = (const unsigned char *)rend[r];
      const uint32_t len = (uint32_t)(e - s);
      if (len < (uint32_t)k + 2 || !seq_valid(s, e)) continue;
      ++used;
      sc.init(s, e);
      L = len; i = 0; fwd = 0; rev = 0; left = 0;
      return true;
    }
    return false;
  };
  auto emit = [&](unsigned in5, unsigned out5) {
    uint64_t x = fwd;
    if (!(fwd < rev)) {   /* lex_less: flip the k-mer and reverse-complement the biedge */
      x = rev;
      const unsigned ni = out5 ? 5u - out5 : 0u, no = in5 ? 5u - in5 : 0u;
      in5 = ni; out5 = no;
    }
    const uint64_t h = bj_fwd(x);
    const unsigned bucket = (unsigned)(h >> LOW_BITS);
    const uint64_t rec = ((h & ((1ull << LOW_BITS) - 1)) << 5) | biedge_code(in5, out5);
    const unsigned idx = (unsigned)(h >> (62 - HLL_P));
    const unsigned rho = (unsigned)__clzll((h << (2 + HLL_P)) | (1ull << (1 + HLL_P))) + 1u;
    if (rho > S.hll[idx]) atomicMax(&S.hll[idx], rho);
    ++inst;
    if (EF && in5 == 0 && out5 == 0) return;   /* filter_isolated_nodes */
    const unsigned pos = atomicAdd(&S.cnt[bucket], 1u);
    if (pos < (unsigned)XQ) {
      S.q[bucket][pos] = rec;
    } else {   /* queue full this round: append straight to the bucket */
      const unsigned long long o = atomicAdd(&bucket_cnt[bucket], 1ull);
      if (o < cap) records[(uint64_t)bucket * cap + o] = rec;
      else S.overflow = 1;
    }
  };
  bool ef_in_ok = false;   /* EF: the previous position's (k+1)-mer was kept */
  bool active = next_read();
  for (;;) {
    int emitted = 0;
    while (active && emitted < XROUND) {
      const unsigned byte = sc.next();
      const unsigned c = ((byte >> 1) ^ (byte >> 2)) & 3u;   /* A0 C1 G2 T3, either case */
      if (i >= (uint32_t)k) {   /* the k-mer ending before base i, its out-base is base i */
        unsigned in5 = i > (uint32_t)k ? left + 1u : 0u, out5 = c + 1u;
        if (EF) {
          const uint64_t f1 = (fwd << 2) | c, r1 = ((uint64_t)(3u - c) << (2 * k)) | rev;
          const bool out_ok = k1_exists(k1tab, k1slots, f1 < r1 ? f1 : r1);
          if (!ef_in_ok) in5 = 0;
          if (!out_ok) out5 = 0;
          ef_in_ok = out_ok;
        }
        emit(in5, out5);
        ++emitted;
      }
      left = (unsigned)(fwd >> top) & 3u;
      fwd = ((fwd << 2) | c) & kmask;
      rev = (rev >> 2) | ((uint64_t)(3u - c) << top);
      if (++i == L) {   /* the last k-mer has no out-base */
        emit(EF && !ef_in_ok ? 0u : left + 1u, 0u);
        ++emitted;
        r += stride;
        active = next_read();
      }
    }
    __syncthreads();
    /* each block fills chunks of `chunk` records per bucket, claimed with one atomic each, so
     * most flushes need no global atomic; a chunk's unused tail is zeroed at the end (0 is no
     * record: a biedge code is never 0) */
    if (tid < NBUCKET) {
      const unsigned f = min(S.cnt[tid], (unsigned)XQ);
      if (f) {
        const unsigned long long p = S.cpos[tid], avail = S.cend[tid] - p;
        S.base[tid] = p;
        if (avail >= f) {
          S.rem[tid] = f;
          S.cpos[tid] = p + f;
        } else {
          const unsigned long long need = f - avail, ch = max(need, (unsigned long long)chunk);
          const unsigned long long old = atomicAdd(&bucket_cnt[tid], ch);
          if (old + ch > cap) S.overflow = 1;
          const unsigned long long nb = (unsigned long long)tid * cap + old;
          S.rem[tid] = (unsigned)avail;
          S.base2[tid] = nb;
          S.cpos[tid] = nb + need;
          S.cend[tid] = nb + ch;
        }
      }
    }
    __syncthreads();
    for (int x = tid; x < NBUCKET * XQ; x += XTPB) {
      const int b = x / XQ, j = x % XQ;
      if ((unsigned)j < min(S.cnt[b], (unsigned)XQ)) {
        const unsigned long long dst = (unsigned)j < S.rem[b] ? S.base[b] + j : S.base2[b] + (j - S.rem[b]);
        if (dst < (unsigned long long)(b + 1) * cap) records[dst] = S.q[b][j];
      }
    }
    __syncthreads();
    if (tid < NBUCKET) S.cnt[tid] = 0;
    if (!__syncthreads_or(active)) break;
  }
  /* the unused tails of the block's chunks hold no records */
  for (int b = tid >> 5; b < NBUCKET; b += XTPB / 32) {
    const unsigned long long e = min(S.cend[b], (unsigned long long)(b + 1) * cap);
    for (unsigned long long p = S.cpos[b] + (tid & 31); p < e; p += 32) records[p] = 0ull;
  }
  inst = warp_sum(inst); used = warp_sum(used);
  if ((tid & 31) == 0) {
    if (inst) atomicAdd(&ctr->n_instances, inst);
    if (used) atomicAdd(&ctr->n_reads_used, used);
  }
  if (tid == 0 && S.overflow) atomicOr(&ctr->err, (unsigned long long)DERR_TABLE_FULL);
  uint8_t *dst = hll_partial + (uint64_t)blockIdx.x * HLL_M;
  for (int x = tid; x < HLL_M; x += XTPB) dst[x] = (uint8_t)S.hll[x];
}

/* ------------------------------------------------ extraction by samples
 * k_extract_s is k_extract (one thread per read, per-bucket queues in shared memory, chunk
 * claims) over work items of one sample's reads: every sample has buckets of its own (the
 * batched form counts many samples at once; the plain build is one sample).  A block takes a
 * contiguous range of items, so it changes sample rarely; when it does, it zeroes the unused
 * tails of its chunks and folds its HyperLogLog registers into the sample's.  The estimate is
 * fed with the k-mers whose mix has its HLL_SAMPLE low bits zero (1 in 8; scaled back). */
constexpr int HLL_SAMPLE = 3;

/* bucket b of sample s holds records[rec_base + b * cap, + cap); chunk = records a block claims at once */
struct XSample { unsigned long long rec_base, cap; unsigned int chunk, pad; };
/* reads [a, b) of sample s */
struct XItem { unsigned long long a, b; unsigned int s, pad; };

/* Records of the extraction, per key width.  k <= 31: 8 bytes, [low 54 bits of bj_fwd(k-mer) |
 * biedge code:5], the bucket being the mix's top 8 bits.  k > 31: 16 bytes, x = (H << 8) | code
 * with H = KOps<KW2>::hash(k-mer) (the bucket is H's top 8 bits) and y = the k-mer's high word,
 * from which the low word follows (kw2_lo).  A zero record is no record (codes are never 0). */
template <class KT> struct XRec;
template <> struct XRec<KW1> {
  using T = uint64_t;
  static constexpr int ROUND = 8, Q = 32;   /* records a thread between flushes, queue per bucket */
  __device__ static __forceinline__ T zero() { return 0ull; }
  __device__ static __forceinline__ bool none(T r) { return r == 0ull; }
  /* the record of k-mer x with biedge code; its bucket; the HyperLogLog sample (if any) */
  __device__ static __forceinline__ T make(KW1 x, unsigned code, unsigned &bucket, bool &sampled, unsigned &idx,
                                           unsigned &rho) {
    const uint64_t h = bj_fwd(x.v);
    bucket = (unsigned)(h >> LOW_BITS);
    sampled = (h & ((1u << HLL_SAMPLE) - 1)) == 0;
    idx = (unsigned)(h >> (62 - HLL_P));
    rho = (unsigned)__clzll((h << (2 + HLL_P)) | (1ull << (1 + HLL_P))) + 1u;
    return ((h & ((1ull << LOW_BITS) - 1)) << 5) | code;
  }
};
template <> struct XRec<KW2> {
  using T = ulonglong2;
  static constexpr int ROUND = 4, Q = 16;   /* twice the bytes a record: half the queue */
  __device__ static __forceinline__ T zero() { return make_ulonglong2(0ull, 0ull); }
  __device__ static __forceinline__ bool none(T r) { return r.x == 0ull; }
  __device__ static __forceinline__ T make(KW2 x, unsigned code, unsigned &bucket, bool &sampled, unsigned &idx,
                                           unsigned &rho) {
    const uint64_t h = KOps<KW2>::hash(x);
    bucket = (unsigned)(h >> 56);
    sampled = (h & ((1u << HLL_SAMPLE) - 1)) == 0;
    idx = (unsigned)(h >> (64 - HLL_P));
    rho = (unsigned)__clzll((h << HLL_P) | (1ull << (HLL_P - 1))) + 1u;
    return make_ulonglong2((h << 8) | code, x.hi);
  }
};

template <class KT>
struct ExtractSmemT {
  typename XRec<KT>::T q[NBUCKET][XRec<KT>::Q];
  unsigned int hll[HLL_M];
  unsigned int cnt[NBUCKET];
  unsigned long long base[NBUCKET];   /* this flush: first `rem` records from base, the rest from base2 */
  unsigned long long base2[NBUCKET];
  unsigned int rem[NBUCKET];
  unsigned long long cpos[NBUCKET], cend[NBUCKET];   /* the block's current chunk of each bucket */
  int overflow;
};

/* the forward k-mer and its reverse complement, rolled base by base */
template <class KT> struct Roll;
template <> struct Roll<KW1> {
  uint64_t fwd, rev, kmask;
  int top;
  __device__ __forceinline__ explicit Roll(int k) : fwd(0), rev(0), kmask((1ull << (2 * k)) - 1), top(2 * k - 2) {}
  __device__ __forceinline__ void reset() { fwd = 0; rev = 0; }
  __device__ __forceinline__ unsigned first() const { return (unsigned)(fwd >> top) & 3u; }
  __device__ __forceinline__ void push(unsigned c) {
    fwd = ((fwd << 2) | c) & kmask;
    rev = (rev >> 2) | ((uint64_t)(3u - c) << top);
  }
  __device__ __forceinline__ bool fwd_canonical() const { return fwd < rev; }
  __device__ __forceinline__ KW1 f() const { return {fwd}; }
  __device__ __forceinline__ KW1 r() const { return {rev}; }
};
template <> struct Roll<KW2> {
  KW2 fwd, rev;
  int k;
  __device__ __forceinline__ explicit Roll(int k_) : fwd{0, 0}, rev{0, 0}, k(k_) {}
  __device__ __forceinline__ void reset() { fwd = {0, 0}; rev = {0, 0}; }
  __device__ __forceinline__ unsigned first() const { return KOps<KW2>::first(fwd, k); }
  __device__ __forceinline__ void push(unsigned c) {
    fwd = KOps<KW2>::append(fwd, c, k);
    rev = KOps<KW2>::prepend(3u - c, rev, k);
  }
  __device__ __forceinline__ bool fwd_canonical() const { return KOps<KW2>::lt(fwd, rev); }
  __device__ __forceinline__ KW2 f() const { return fwd; }
  __device__ __forceinline__ KW2 r() const { return rev; }
};

/* the block's open chunks of sample xs closed (tails zeroed) and its registers folded into the
 * sample's (every thread of the block calls it) */
template <class KT>
__device__ __forceinline__ void xs_close(ExtractSmemT<KT> &S, const XSample &xs, typename XRec<KT>::T *records,
                                         unsigned int *hreg) {
  const int tid = threadIdx.x;
  __syncthreads();
  for (int b = tid >> 5; b < NBUCKET; b += XTPB / 32) {
    const unsigned long long e = min(S.cend[b], xs.rec_base + (unsigned long long)(b + 1) * xs.cap);
    for (unsigned long long p = S.cpos[b] + (tid & 31); p < e; p += 32) records[p] = XRec<KT>::zero();
  }
  for (int i = tid; i < HLL_M; i += XTPB) {
    if (S.hll[i]) atomicMax(&hreg[i], S.hll[i]);
    S.hll[i] = 0;
  }
  __syncthreads();
  for (int b = tid; b < NBUCKET; b += XTPB) { S.cpos[b] = 0; S.cend[b] = 0; }
  __syncthreads();
}

/* EF (k > 31 only): the (k+1)-mer edge filter of the blocked driver, as k_extract<true> applies
 * it for k <= 31 -- an edge whose (k+1)-mer is not in the 128-bit table k1tab is cleared, and a
 * pair left without edges is counted as an instance but not emitted (filter_isolated_nodes) */
template <class KT, bool EF = false>
__global__ void __launch_bounds__(XTPB, 2) k_extract_s(const uint64_t *rstart, const uint64_t *rend, uint64_t r0,
                                                        uint64_t r1, const XItem *items, uint64_t n_items,
                                                        uint32_t item_reads, int k, const XSample *xsamp,
                                                        typename XRec<KT>::T *records, unsigned long long *bucket_cnt,
                                                        unsigned int *hll, unsigned long long *s_inst,
                                                        unsigned long long *s_used, const uint64_t *k1tab,
                                                        uint64_t k1slots, DevCounters *ctr) {
  static_assert(!EF || sizeof(KT) == 16, "k <= 31 filters edges in k_extract<true>");
  using R = XRec<KT>;
  constexpr int XQT = R::Q, XROUNDT = R::ROUND;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ExtractSmemT<KT> &S = *reinterpret_cast<ExtractSmemT<KT> *>(smem_raw);
  const int tid = threadIdx.x;
  for (int i = tid; i < HLL_M; i += XTPB) S.hll[i] = 0;
  for (int i = tid; i < NBUCKET; i += XTPB) { S.cnt[i] = 0; S.cpos[i] = 0; S.cend[i] = 0; }
  if (tid == 0) S.overflow = 0;
  __syncthreads();
  const uint64_t nit = items ? n_items : (r1 - r0 + item_reads - 1) / item_reads;
  /* block b takes items [b * nit / grid, (b + 1) * nit / grid): every block gets the floor or
   * the ceiling of the mean, so the one wave of blocks ends together */
  const uint64_t it0 = (uint64_t)blockIdx.x * nit / gridDim.x, it1 = ((uint64_t)blockIdx.x + 1) * nit / gridDim.x;
  unsigned cur_s = ~0u;
  XSample xs{};
  unsigned long long inst_all = 0, used_all = 0;
  for (uint64_t it = it0; it < it1; ++it) {
    uint64_t a, b;
    unsigned smp;
    if (items) { a = items[it].a; b = items[it].b; smp = items[it].s; }
    else { a = r0 + it * item_reads; b = min(r1, a + item_reads); smp = 0; }
    if (smp != cur_s) {
      if (cur_s != ~0u) xs_close<KT>(S, xs, records, hll + (uint64_t)cur_s * HLL_M);
      cur_s = smp;
      xs = xsamp[smp];
    }
    uint64_t r = a + tid;
    unsigned long long inst = 0, used = 0;
    SeqCursor sc;
    uint32_t L = 0, i = 0;
    Roll<KT> roll(k);
    unsigned left = 0;
    /* advance to the next usable read of this thread in the item */
    auto next_read = [&]() -> bool {
      for (; r < b; r += XTPB) {
        const unsigned char *sp = (const unsigned char *)rstart[r], *ep = (const unsigned char *)rend[r];
        const uint32_t len = (uint32_t)(ep - sp);
        if (len < (uint32_t)k + 2 || !seq_valid(sp, ep)) continue;
        ++used;
        sc.init(sp, ep);
        L = len; i = 0; roll.reset(); left = 0;
        return true;
      }
      return false;
    };
    /* the record of the k-mer in the roll with edges (in5, out5): canonical form, mix, bucket */
    auto make_rec = [&](unsigned in5, unsigned out5, unsigned &bucket) -> typename R::T {
      KT x = roll.f();
      if (!roll.fwd_canonical()) {   /* lex_less: flip the k-mer and reverse-complement the biedge */
        x = roll.r();
        const unsigned ni = out5 ? 5u - out5 : 0u, no = in5 ? 5u - in5 : 0u;
        in5 = ni; out5 = no;
      }
      unsigned idx, rho;
      bool sampled;
      const typename R::T rec = R::make(x, biedge_code(in5, out5), bucket, sampled, idx, rho);
      if (sampled && rho > S.hll[idx]) atomicMax(&S.hll[idx], rho);
      ++inst;
      return rec;
    };
    auto enqueue = [&](const typename R::T &rec, unsigned bucket) {
      const unsigned pos = atomicAdd(&S.cnt[bucket], 1u);
      if (pos < (unsigned)XQT) {
        S.q[bucket][pos] = rec;
      } else {   /* queue full this round: append straight to the bucket */
        const unsigned long long o = atomicAdd(&bucket_cnt[(uint64_t)cur_s * NBUCKET + bucket], 1ull);
        if (o < xs.cap) records[xs.rec_base + (uint64_t)bucket * xs.cap + o] = rec;
        else S.overflow = 1;
      }
    };
    auto emit = [&](unsigned in5, unsigned out5) {
      unsigned bucket;
      const typename R::T rec = make_rec(in5, out5, bucket);
      if (EF && in5 == 0 && out5 == 0) return;   /* filter_isolated_nodes */
      enqueue(rec, bucket);
    };
    bool ef_in_ok = false;   /* EF: the previous position's (k+1)-mer was kept */
    bool active = next_read();
    for (;;) {
      int emitted = 0;
      while (active && emitted < XROUNDT) {
        if (!EF && sizeof(KT) == 8 && i > (uint32_t)k && i + 2 < L && emitted + 2 <= XROUNDT) {
          /* two interior k-mers a turn: both records are made before either is queued, so
           * their mixes interleave (64-bit keys only: with 128-bit keys the second record's
           * registers spill and the turn measured slower) */
          const unsigned b1 = sc.next(), b2 = sc.next();
          const unsigned c1 = ((b1 >> 1) ^ (b1 >> 2)) & 3u, c2 = ((b2 >> 1) ^ (b2 >> 2)) & 3u;
          unsigned bk1, bk2;
          const typename R::T rec1 = make_rec(left + 1u, c1 + 1u, bk1);
          left = roll.first();
          roll.push(c1);
          const typename R::T rec2 = make_rec(left + 1u, c2 + 1u, bk2);
          left = roll.first();
          roll.push(c2);
          i += 2;
          enqueue(rec1, bk1);
          enqueue(rec2, bk2);
          emitted += 2;
          continue;
        }
        const unsigned byte = sc.next();
        const unsigned c = ((byte >> 1) ^ (byte >> 2)) & 3u;   /* A0 C1 G2 T3, either case */
        if (i >= (uint32_t)k) {   /* the k-mer ending before base i, its out-base is base i */
          unsigned in5 = i > (uint32_t)k ? left + 1u : 0u, out5 = c + 1u;
          if constexpr (EF) {   /* the (k+1)-mer k-mer + c, canonical, against the table */
            const KW2 f1 = KOps<KW2>::append(roll.f(), c, k + 1);
            KW2 q1 = roll.r();
            const uint64_t b = (uint64_t)(3u - c);
            if (2 * k >= 64) q1.hi |= b << (2 * k - 64); else q1.lo |= b << (2 * k);
            const bool out_ok = k1w_exists(k1tab, k1slots, KOps<KW2>::lt(f1, q1) ? f1 : q1);
            if (!ef_in_ok) in5 = 0;
            if (!out_ok) out5 = 0;
            ef_in_ok = out_ok;
          }
          emit(in5, out5);
          ++emitted;
        }
        left = roll.first();
        roll.push(c);
        if (++i == L) {   /* the last k-mer has no out-base */
          emit(EF && !ef_in_ok ? 0u : left + 1u, 0u);
          ++emitted;
          r += XTPB;
          active = next_read();
        }
      }
      __syncthreads();
      /* each block fills chunks of `chunk` records per bucket, claimed with one atomic each, so
       * most flushes need no global atomic; a chunk's unused tail is zeroed when the block
       * leaves the sample (0 is no record: a biedge code is never 0) */
      if (tid < NBUCKET) {
        const unsigned f = min(S.cnt[tid], (unsigned)XQT);
        if (f) {
          const unsigned long long p = S.cpos[tid], avail = S.cend[tid] - p;
          S.base[tid] = p;
          if (avail >= f) {
            S.rem[tid] = f;
            S.cpos[tid] = p + f;
          } else {
            const unsigned long long need = f - avail, ch = max(need, (unsigned long long)xs.chunk);
            const unsigned long long old = atomicAdd(&bucket_cnt[(uint64_t)cur_s * NBUCKET + tid], ch);
            if (old + ch > xs.cap) S.overflow = 1;
            const unsigned long long nb = xs.rec_base + (unsigned long long)tid * xs.cap + old;
            S.rem[tid] = (unsigned)avail;
            S.base2[tid] = nb;
            S.cpos[tid] = nb + need;
            S.cend[tid] = nb + ch;
          }
        }
      }
      __syncthreads();
      for (int x = tid; x < NBUCKET * XQT; x += XTPB) {
        const int bk = x / XQT, j = x % XQT;
        if ((unsigned)j < min(S.cnt[bk], (unsigned)XQT)) {
          const unsigned long long dst = (unsigned)j < S.rem[bk] ? S.base[bk] + j : S.base2[bk] + (j - S.rem[bk]);
          if (dst < xs.rec_base + (unsigned long long)(bk + 1) * xs.cap) records[dst] = S.q[bk][j];
        }
      }
      __syncthreads();
      if (tid < NBUCKET) S.cnt[tid] = 0;
      if (!__syncthreads_or(active)) break;
    }
    inst = warp_sum(inst); used = warp_sum(used);
    if ((tid & 31) == 0) {
      inst_all += inst; used_all += used;
      if (s_inst && inst) atomicAdd(&s_inst[smp], inst);
      if (s_used && used) atomicAdd(&s_used[smp], used);
    }
  }
  if (cur_s != ~0u) xs_close<KT>(S, xs, records, hll + (uint64_t)cur_s * HLL_M);
  if ((tid & 31) == 0) {
    if (inst_all) atomicAdd(&ctr->n_instances, inst_all);
    if (used_all) atomicAdd(&ctr->n_reads_used, used_all);
  }
  if (tid == 0 && S.overflow) atomicOr(&ctr->err, (unsigned long long)DERR_TABLE_FULL);
}

/* per-sample distinct estimate inputs: sum of 2^-register and the number of zero registers
 * (one block per sample; the host finishes the HyperLogLog estimate) */
__global__ void k_hll_sums(const unsigned int *hll, double *sum, unsigned int *zeros) {
  __shared__ double ss[256];
  __shared__ unsigned int zz[256];
  const unsigned int *reg = hll + (uint64_t)blockIdx.x * HLL_M;
  double t = 0;
  unsigned z = 0;
  for (int i = threadIdx.x; i < HLL_M; i += blockDim.x) { t += ldexp(1.0, -(int)reg[i]); z += reg[i] == 0; }
  ss[threadIdx.x] = t; zz[threadIdx.x] = z;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) { ss[threadIdx.x] += ss[threadIdx.x + o]; zz[threadIdx.x] += zz[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { sum[blockIdx.x] = ss[0]; zeros[blockIdx.x] = zz[0]; }
}

/* one table partition: keys EMPTY, entries 0 (stays in L2 for the inserts that follow) */
template <class KT>
__global__ void k_part_init(uint64_t *table, uint64_t first_slot, uint64_t nslots) {
  constexpr int SU = Slot<KT>::U64, KWD = Slot<KT>::KEYW;
  uint64_t *t = table + first_slot * SU;
  const uint64_t nw = nslots * SU;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += (uint64_t)gridDim.x * blockDim.x)
    t[i] = ((int)(i % SU) < KWD) ? KEY_EMPTY : 0ull;
}

/* Phase B: the records of the buckets of partition q (blockIdx.y picks the bucket); two
 * records in flight per thread (their slot reads are issued before either is used) and
 * the next two already loading */
constexpr int INS_BATCH = 2;
__global__ void __launch_bounds__(TPB) k_insert(const uint64_t *records, const unsigned long long *bucket_cnt,
                                                 uint64_t cap, int bucket0, uint64_t *table, TableGeom g,
                                                 uint32_t max_probe, DevCounters *ctr) {
  constexpr int SU = Slot<KW1>::U64;
  const int b = bucket0 + (int)blockIdx.y;
  const uint64_t n = min((unsigned long long)cap, bucket_cnt[b]);
  const uint64_t *rb = records + (uint64_t)b * cap;
  /* every record of bucket b lives in partition q = b >> (8 - pbits) */
  const uint64_t lo = (uint64_t)(b >> (NBUCKET_BITS - g.pbits)) * g.region;
  unsigned long long slots = 0, entries = 0;
  bool full = false;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  /* the next batch of records is loaded while this one is counted */
  uint64_t nxt[INS_BATCH];
  #pragma unroll
  for (int q = 0; q < INS_BATCH; ++q) {
    const uint64_t j = i + q * stride;
    nxt[q] = j < n ? __ldcs(rb + j) : 0ull;   /* 0: no record (past the end, or a chunk tail) */
  }
  for (; i < n; i += INS_BATCH * stride) {
    uint64_t rec[INS_BATCH], home[INS_BATCH], raw[INS_BATCH][SU];
    #pragma unroll
    for (int q = 0; q < INS_BATCH; ++q) {
      rec[q] = nxt[q];
      const uint64_t j = i + (INS_BATCH + q) * stride;
      nxt[q] = j < n ? __ldcs(rb + j) : 0ull;
    }
    #pragma unroll
    for (int q = 0; q < INS_BATCH; ++q) {
      if (rec[q] == 0ull) continue;
      const uint64_t h = ((uint64_t)b << LOW_BITS) | (rec[q] >> 5);
      home[q] = lo + __umul64hi(h << (2 + g.pbits), g.region);
      ld_slot<SU>(table + home[q] * SU, raw[q]);
    }
    #pragma unroll
    for (int q = 0; q < INS_BATCH; ++q) {
      if (rec[q] == 0ull) continue;
      const uint64_t h = ((uint64_t)b << LOW_BITS) | (rec[q] >> 5);
      if (!table_count<KW1>(table, g, max_probe, KW1{h}, (unsigned)(rec[q] & 31), home[q], raw[q], slots, entries,
                            ctr, lo))
        full = true;
    }
  }
  slots = warp_sum(slots); entries = warp_sum(entries);
  if ((threadIdx.x & 31) == 0) {
    if (slots) atomicAdd(&ctr->n_slots_claimed, slots);
    if (entries) atomicAdd(&ctr->n_entries, entries);
  }
  if (full) atomicOr(&ctr->err, (unsigned long long)DERR_TABLE_FULL);
}

struct FilterArgs {
  uint32_t *chain_list, *branch_list;   /* slot indices of chain / branch nodes */
  uint64_t list_cap;
  uint64_t *table;
  uint64_t nslots;
  TableGeom g;
  int k;
  uint64_t t[6];
  int thresholding;
  uint32_t max_probe;
  uint64_t *f_keys; uint8_t *f_edges; uint32_t *f_counts; uint64_t f_cap;
  const BigRes *big; uint64_t n_big;   /* entries counted past 2^24, for exact filtered counts */
  const SGeom *sg; uint32_t S;         /* a batch of S samples (S = 1: the plain build) */
  unsigned long long *s_tally;         /* per-sample tallies (batch only) */
  const uint32_t *cand; uint64_t n_cand; /* the slots the count listed (NULL: every slot) */
  DevCounters *ctr;
};

/* per-thread k_del[] histogram in registers: 16-bit bins, four to a word (every update is
 * an unrolled select, so nothing is indexed at run time); `n` counts the updates so the
 * owner can drain the bins before one could wrap */
struct FlagHist {
  uint64_t p[4];
  uint32_t n;
  __device__ __forceinline__ void clear() {
    #pragma unroll
    for (int i = 0; i < 4; ++i) p[i] = 0;
    n = 0;
  }
  __device__ __forceinline__ void add(unsigned f) {
    const uint64_t inc = 1ull << (16 * (f & 3u));
    #pragma unroll
    for (int i = 0; i < 4; ++i) p[i] += ((f >> 2) == (unsigned)i) ? inc : 0ull;
    ++n;
  }
  __device__ __forceinline__ unsigned long long get(int f) const { return (p[f >> 2] >> (16 * (f & 3))) & 0xFFFFull; }
  static constexpr uint32_t DRAIN = 60000;   /* drain at or above this many updates */
};

struct FilterTally {
  unsigned long long nodes = 0, branch = 0, chain = 0;
  FlagHist hist;
  int kind = 0;          /* the last k-mer: 0 not a node, 1 chain node, 2 branch node */
  uint32_t sample = 0;   /* the sample of the k-mer being filtered (batch) */
};

/* v[c] for a run-time c in 0..3, as selects */
__device__ __forceinline__ uint32_t pick4(const uint32_t *v, unsigned c) {
  return c == 0 ? v[0] : c == 1 ? v[1] : c == 2 ? v[2] : v[3];
}

/* local_insert_by_freqencies (debruijn_graph_map.hpp:1258-1623) for one k-mer block: the
 * entry words w[0..ne) of the k-mer, all in registers when CAP is the slot capacity.
 * Writes the node (compact_multi_biedge counts, flags) over the slot, or a tombstone. */
/* Quick drop: a (k+1)-mer count is at most the k-mer's total, so when the total is below
 * the (k+1)-mer lower bound every entry gets flags 2 and 1 (debruijn_graph_map.hpp:
 * 1423-1448) and none is kept.  Tallies the flags exactly as the full pass would, writes
 * the tombstone and returns true; false when the k-mer needs the full pass. */
template <class KT, int CAP>
__device__ __forceinline__ bool filter_quick(uint64_t *s, const uint32_t *w, int ne, const FilterArgs &a,
                                             FilterTally &t) {
  if (!a.thresholding) return false;
  const uint32_t cmax32 = 0xFFFFu;
  uint32_t kf = 0;
  #pragma unroll
  for (int q = 0; q < CAP; ++q) {
    if (q >= ne) break;
    kf += entry_count(w[q]);
  }
  kf = min(cmax32, kf);
  if (kf >= a.t[2]) return false;
  const unsigned fk = 3u | ((kf < a.t[0] || kf >= a.t[1]) ? 8u : 0u);
  #pragma unroll
  for (int q = 0; q < CAP; ++q) {
    if (q >= ne) break;
    const uint32_t c16 = min(cmax32, entry_count(w[q]));
    t.hist.add(fk | ((c16 < a.t[4] || c16 >= a.t[5]) ? 4u : 0u));
  }
  return true;   /* the slot keeps its bare key: not a node */
}

template <class KT, int CAP, bool QUICK = true>
__device__ __forceinline__ void filter_kmer(uint64_t *s, uint64_t slot_index, KT tkey, const uint32_t *w, int ne,
                                            const FilterArgs &a, FilterTally &t) {
  constexpr int KWD = Slot<KT>::KEYW;
  const int k = a.k;
  if (QUICK && filter_quick<KT, CAP>(s, w, ne, a, t)) return;
  const KT key = key_kmer(tkey);   /* the canonical k-mer */
  /* step 4: per-block sums (:1460-1507) */
  const bool kpal = k_palindrome(key, k);
  const bool high = km1_high_palindrome(key, k), low = km1_low_palindrome(key, k);
  const unsigned first = KOps<KT>::first(key, k), last = KOps<KT>::last(key);
  const bool oddk = (k & 1) != 0;
  /* sums fit 32 bits: at most 25 entries of at most 2^26 each */
  uint32_t k_f = 0, k1in[4] = {0, 0, 0, 0}, k1out[4] = {0, 0, 0, 0};
  #pragma unroll
  for (int q = 0; q < CAP; ++q) {
    if (q >= ne) break;
    const uint32_t c = entry_count(w[q]);
    const unsigned code = entry_code(w[q]);
    const unsigned in5 = code_in5(code), out5 = code_out5(code);
    k_f += c;
    if (in5) {
      const unsigned ch = in5 - 1;
      const bool split = oddk && last == 3u - ch && high && !kpal;
      const uint32_t v = split ? ((c + 1) >> 1) : c;
      #pragma unroll
      for (int cc = 0; cc < 4; ++cc) k1in[cc] += (ch == (unsigned)cc) ? v : 0u;
    }
    if (out5) {
      const unsigned ch = out5 - 1;
      const bool split = oddk && first == 3u - ch && low && !kpal;
      const uint32_t v = split ? ((c + 1) >> 1) : c;
      #pragma unroll
      for (int cc = 0; cc < 4; ++cc) k1out[cc] += (ch == (unsigned)cc) ? v : 0u;
    }
  }
  /* caps at FreqType max (:1401-1407) */
  const uint32_t cmax32 = 0xFFFFu;
  k_f = min(cmax32, k_f);
  #pragma unroll
  for (int c = 0; c < 4; ++c) { k1in[c] = min(cmax32, k1in[c]); k1out[c] = min(cmax32, k1out[c]); }
  /* step 5: flags (:1410-1448), step 6: trim (:1563-1594), step 7: node update (:256-285);
   * node sums fit 32 bits (at most 25 entries of at most 65535) */
  uint32_t nc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  bool any = false;
  #pragma unroll
  for (int q = 0; q < CAP; ++q) {
    if (q >= ne) break;
    const uint32_t cnt = entry_count(w[q]);
    const uint32_t cnt16 = min(cmax32, cnt);
    const unsigned code = entry_code(w[q]);
    unsigned in5 = code_in5(code), out5 = code_out5(code);
    unsigned f = 0;
    if (a.thresholding) {
      if (cnt16 < a.t[4] || cnt16 >= a.t[5]) f |= 4;
      if (k_f < a.t[0] || k_f >= a.t[1]) f |= 8;
      uint64_t k1 = in5 ? (uint64_t)pick4(k1in, in5 - 1) : a.t[3];
      if (k1 < a.t[2] || k1 >= a.t[3]) f |= 2;
      k1 = out5 ? (uint64_t)pick4(k1out, out5 - 1) : a.t[3];
      if (k1 < a.t[2] || k1 >= a.t[3]) f |= 1;
    }
    t.hist.add(f);
    if (f >= 3) continue;
    if (f == 1) out5 = 0;
    if (f == 2) in5 = 0;
    any = true;
    #pragma unroll
    for (int c = 0; c < 4; ++c) {
      nc[c] += (out5 == (unsigned)c + 1) ? cnt16 : 0u;
      nc[4 + c] += (in5 == (unsigned)c + 1) ? cnt16 : 0u;
    }
    nc[8] += cnt16;
    if (a.f_keys) {
      unsigned long long o = atomicAdd(&a.ctr->n_filtered, 1ull);
      if (o < a.f_cap) {
        KOps<KT>::store(a.f_keys + o * KWD, key);
        a.f_edges[o] = code_biedge(biedge_code(in5, out5));
        uint32_t exact = cnt;
        if (w[q] & E_BIG)   /* counted past 2^24: the exact count, to 32 bits like the reference's */
          for (uint64_t b = 0; b < a.n_big; ++b)
            if (a.big[b].code == code && a.big[b].k0 == ((const uint64_t *)&tkey)[0] &&
                (KWD == 1 || a.big[b].k1 == ((const uint64_t *)&tkey)[KWD - 1]))
              exact = (uint32_t)a.big[b].count;
        a.f_counts[o] = exact;
      }
    }
  }
  if (!any) return;  /* no kept entry: the k-mer never enters the graph (its key stays bare) */
  uint16_t c16[9];
  #pragma unroll
  for (int q = 0; q < 9; ++q) c16[q] = (uint16_t)min(cmax32, nc[q]);
  /* IsBranchPoint / IsChainNode (debruijn_graph_filters.hpp:57-220) */
  unsigned din = 0, dout = 0;
  bool k1pal = false;
  #pragma unroll
  for (int c = 0; c < 4; ++c) {
    dout += c16[c] > 0;
    din += c16[4 + c] > 0;
    if (oddk && c16[c] > 0 && low && (first == 3u - c || first == (unsigned)c)) k1pal = true;
    if (oddk && c16[4 + c] > 0 && high && (last == 3u - c || last == (unsigned)c)) k1pal = true;
  }
  const bool is_branch = din >= 2 || dout >= 2 || kpal || k1pal;
  const uint32_t flags = (is_branch ? NF_BRANCH : NF_CHAIN) | (t.sample << NF_SAMPLE_SHIFT);
  ++t.nodes; t.branch += is_branch; t.chain += !is_branch;
  /* chain nodes get their chain index (slot aux) when the block flushes its node list */
  t.kind = is_branch ? 2 : 1;
  uint64_t *pw = s + KWD;
  pw[0] = (uint64_t)c16[0] | ((uint64_t)c16[1] << 16) | ((uint64_t)c16[2] << 32) | ((uint64_t)c16[3] << 48);
  pw[1] = (uint64_t)c16[4] | ((uint64_t)c16[5] << 16) | ((uint64_t)c16[6] << 32) | ((uint64_t)c16[7] << 48);
  pw[2] = (uint64_t)c16[8] | ((uint64_t)flags << 16) | (0xFFFFFFFFull << 32);
  KOps<KT>::store(s, as_node(tkey));   /* the key we hold, marked: no reload of the slot */
}

/* A k-mer with more biedges than one slot holds: gather the entries of its continuation
 * slots (further along its probe run, tombstoned as they are folded in) and filter them
 * together.  Rare, so kept out of line to leave the common path its registers. */
template <class KT>
__device__ __noinline__ void filter_wide_global(uint64_t *s, uint64_t i, KT key, const uint32_t *w,
                                                const FilterArgs &a, FilterTally &t) {
  constexpr int SU = Slot<KT>::U64, NE = Slot<KT>::ENTRIES, KWD = Slot<KT>::KEYW;
  uint32_t all[25];
  int ne = NE;
  for (int q = 0; q < NE; ++q) all[q] = w[q];
  Probe pr(a.S > 1 ? a.sg[t.sample].g : a.g, i);   /* inside the k-mer's own partition */
  for (uint32_t probe = 1; probe < a.max_probe; ++probe) {
    pr.next();
    uint64_t *s2 = a.table + pr.i * SU;
    const KT k2 = KOps<KT>::load(s2);
    if (key_is_empty(k2)) break;
    if (!key_matches(k2, key, true)) continue;
    const uint32_t *e2 = (const uint32_t *)(s2 + KWD);
    for (int q = 0; q < NE && ne < 25; ++q) {
      if (e2[q] == 0) break;
      all[ne++] = e2[q];
    }
    if (KWD == 1) s2[0] = KEY_TOMB; else { s2[0] = KEY_TOMB; s2[1] = KEY_TOMB; }
  }
  filter_kmer<KT, 25>(s, i, key, all, ne, a, t);
}

/* ------------------------------------------- shared-memory counting of small partitions
 * When the table is cut into 2^pbits partitions (pbits >= 8) of at most PART_SLOTS slots, a
 * partition fits in one CTA's shared memory.  k_split first splits every bucket into its
 * 2^(pbits-8) partitions (bucket b = partitions [b << s, (b+1) << s), picked by the next s
 * bits of the mix); k_count_local then gives each partition to one CTA, which counts the
 * partition's records into shared memory with shared-memory atomics and writes the finished
 * slot region to the table once, in coalesced 16-byte stores. */
constexpr int PART_SLOTS = 3072;           /* 96 KB of slots: the largest region */
constexpr int PTPB = 512;                  /* k_count_local threads unless cfg.count_threads says otherwise */
/* the tunables of the shared-memory count: the largest partition region (which bounds every
 * probe run; cfg.part_slots, 256..3072) and the counting block's threads (cfg.count_threads) */
uint64_t part_slots(const Ctx *c) {
  const int v = c->cfg.part_slots;
  return v <= 0 ? (uint64_t)PART_SLOTS : (uint64_t)std::max(256, std::min(PART_SLOTS, v));
}
int count_threads(const Ctx *c) {
  const int v = c->cfg.count_threads;
  return (v == 256 || v == 512 || v == 1024) ? v : PTPB;
}
/* a counting block for partitions of at most `region` slots: about one thread per two slots
 * (small samples' partitions hold a few hundred records), at least 128, at most the configured
 * block */
int count_threads_for(const Ctx *c, uint64_t region) {
  int t = 128;
  while (t < count_threads(c) && (uint64_t)t * 2 < region) t *= 2;
  return t;
}
constexpr int MAX_SPLIT_BITS = 10;
constexpr int SPLIT_ROUND = 16;            /* records per thread per round */
constexpr int SPLIT_REC = XTPB * SPLIT_ROUND;   /* 8192 records a round */

struct SplitSmem {
  uint64_t buf[SPLIT_REC];                        /* the round's records, ordered by partition */
  unsigned int cnt[1 << MAX_SPLIT_BITS];          /* records per partition this round */
  unsigned int start[1 << MAX_SPLIT_BITS];        /* their first position in buf */
  unsigned long long base[1 << MAX_SPLIT_BITS];   /* their first position in the output */
  unsigned int wsum[XTPB / 32];
  unsigned int wsum_total;
  int overflow;
};

/* A bucket of sample s -> its 2^sbits partitions (sbits = the sample's partition bits - 8): work
 * items are pieces [lo, hi) of one bucket, and a block moves its items in rounds of SPLIT_REC
 * records, a counting sort each: the records stay in registers while a shared-memory histogram
 * gives each its rank in its partition, a block scan turns the histogram into offsets, one
 * reservation per partition and round claims the output run, and the records, scattered into
 * partition order in shared memory, go out in one coalesced pass. */
struct SplitItem { unsigned long long lo, hi; unsigned int gb, pad; };   /* gb = sample * 256 + bucket */

__global__ void __launch_bounds__(XTPB, 2) k_split(const uint64_t *records, const XSample *xs, const SGeom *sg,
                                                 const SplitItem *items, uint64_t n_items, uint64_t *out,
                                                 unsigned long long *sub_cnt, DevCounters *ctr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SplitSmem &S = *reinterpret_cast<SplitSmem *>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int i = tid; i < (1 << MAX_SPLIT_BITS); i += XTPB) S.cnt[i] = 0;   /* every round re-zeroes what it used */
  if (tid == 0) S.overflow = 0;
  __syncthreads();
  for (uint64_t it = blockIdx.x; it < n_items; it += gridDim.x) {
    const SplitItem item = items[it];
    const unsigned smp = item.gb >> NBUCKET_BITS, b = item.gb & (NBUCKET - 1);
    const XSample X = xs[smp];
    const SGeom G = sg[smp];
    const int sbits = G.g.pbits - NBUCKET_BITS, nq = 1 << sbits;
    const uint64_t *rb = records + X.rec_base + (uint64_t)b * X.cap;
    const int shift = 5 + LOW_BITS - sbits;
    /* a round's records: every load of the round is in flight before the first use, and each
     * round after the first is loaded while the round before it is written out */
    uint64_t recs[SPLIT_ROUND];
    #pragma unroll
    for (int j = 0; j < SPLIT_ROUND; ++j) {
      const uint64_t i = item.lo + (uint64_t)j * XTPB + tid;
      recs[j] = i < item.hi ? __ldcs(rb + i) : 0ull;
    }
    for (uint64_t r0 = item.lo; r0 < item.hi; r0 += SPLIT_REC) {
      uint32_t pos[SPLIT_ROUND];    /* partition << 16 | rank in it; ~0 past the end */
      #pragma unroll
      for (int j = 0; j < SPLIT_ROUND; ++j) {
        const uint64_t i = r0 + (uint64_t)j * XTPB + tid;
        pos[j] = ~0u;
        if (i < item.hi && recs[j] != 0ull) {   /* 0: an unused chunk tail */
          const unsigned sq = (unsigned)(recs[j] >> shift) & (unsigned)(nq - 1);
          pos[j] = (sq << 16) | atomicAdd(&S.cnt[sq], 1u);
        }
      }
      __syncthreads();
      /* exclusive scan of the histogram (two partitions a thread) and the reservations */
      const int q0 = 2 * tid;
      const unsigned c0 = q0 < nq ? S.cnt[q0] : 0u, c1 = q0 + 1 < nq ? S.cnt[q0 + 1] : 0u;
      if (q0 < nq) S.cnt[q0] = 0;
      if (q0 + 1 < nq) S.cnt[q0 + 1] = 0;
      const unsigned v = c0 + c1;
      unsigned x = v;
      #pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(~0u, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) S.wsum[wid] = x;
      __syncthreads();
      if (wid == 0) {
        const unsigned w = lane < XTPB / 32 ? S.wsum[lane] : 0u;
        unsigned z = w;
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned y = __shfl_up_sync(~0u, z, o);
          if (lane >= o) z += y;
        }
        if (lane < XTPB / 32) S.wsum[lane] = z - w;
        if (lane == XTPB / 32 - 1) S.wsum_total = z;
      }
      __syncthreads();
      const unsigned ex = S.wsum[wid] + x - v;
      #pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int q = q0 + h;
        const unsigned c = h ? c1 : c0;
        if (q < nq) {
          S.start[q] = h ? ex + c0 : ex;
          if (c) {
            const uint64_t j = ((uint64_t)b << sbits) | (unsigned)q;   /* the sample's partition */
            const unsigned long long old = atomicAdd(&sub_cnt[G.pbase + j], (unsigned long long)c);
            if (old + c > G.cap2) S.overflow = 1;
            S.base[q] = G.rec2_base + j * G.cap2 + old;
          }
        }
      }
      __syncthreads();
      #pragma unroll
      for (int j = 0; j < SPLIT_ROUND; ++j)
        if (pos[j] != ~0u) S.buf[S.start[pos[j] >> 16] + (pos[j] & 0xFFFFu)] = recs[j];
      __syncthreads();
      if (r0 + SPLIT_REC < item.hi) {
        #pragma unroll
        for (int j = 0; j < SPLIT_ROUND; ++j) {
          const uint64_t i = r0 + SPLIT_REC + (uint64_t)j * XTPB + tid;
          recs[j] = i < item.hi ? __ldcs(rb + i) : 0ull;
        }
      }
      const unsigned nr = S.wsum_total;   /* the round's records, holes left out */
      for (unsigned y = tid; y < nr; y += XTPB) {
        const uint64_t rec = S.buf[y];
        const unsigned q = (unsigned)(rec >> shift) & (unsigned)(nq - 1);
        const uint64_t j = ((uint64_t)b << sbits) | q;
        const unsigned long long dst = S.base[q] + (y - S.start[q]);
        if (dst < G.rec2_base + (j + 1) * G.cap2) out[dst] = rec;
      }
      __syncthreads();   /* the next round writes buf, start and base */
    }
  }
  if (tid == 0 && S.overflow) atomicOr(&ctr->err, (unsigned long long)DERR_TABLE_FULL);
}

__device__ __forceinline__ uint64_t sm_cas128(uint32_t a, uint64_t cmp_lo, uint64_t cmp_hi, uint64_t new_lo,
                                              uint64_t new_hi, uint64_t &old_hi) {
  uint64_t olo, ohi;
  asm volatile(
      "{\n\t.reg .b128 d, b, c;\n\t"
      "mov.b128 b, {%2, %3};\n\t"
      "mov.b128 c, {%4, %5};\n\t"
      "atom.shared.cas.b128 d, [%6], b, c;\n\t"
      "mov.b128 {%0, %1}, d;\n\t}"
      : "=l"(olo), "=l"(ohi)
      : "l"(cmp_lo), "l"(cmp_hi), "l"(new_lo), "l"(new_hi), "r"(a)
      : "memory");
  old_hi = ohi;
  return olo;
}


/* one step of count_in_entries on entry word e (snapshot w): claim it if empty, count if it
 * holds the code; true when the record is counted */
__device__ __forceinline__ bool sm_entry_step(uint32_t *e, uint32_t w, unsigned code, unsigned long long &claims) {
  if (w == 0) {
    const uint32_t old = atomicCAS(e, 0u, (code << E_CODE_SHIFT) | (1u << E_COUNT_SHIFT));
    if (old == 0) { ++claims; return true; }
    w = old;
  }
  if (entry_code(w) == code) {
    atomicAdd(e, 1u << E_COUNT_SHIFT);   /* a partition counted here holds fewer than 2^24 records */
    return true;
  }
  return false;
}

/* count_in_entries over a slot's NE entry words in shared memory, reading them 16 bytes (four
 * entries) at a time, and a group only when the entries before it did not settle the record
 * (most k-mers hold one or two edges); `first` are the words already read */
template <int NE, int FIRST>
__device__ __forceinline__ bool sm_count_entries_lazy(uint32_t *e, uint32_t e_addr, const uint32_t *first,
                                                      unsigned code, unsigned long long &claims) {
  #pragma unroll
  for (int i = 0; i < FIRST; ++i)
    if (sm_entry_step(e + i, first[i], code, claims)) return true;
  #pragma unroll
  for (int g = FIRST; g < NE; g += 4) {
    uint64_t w0, w1;
    asm volatile("ld.volatile.shared.v2.u64 {%0, %1}, [%2];" : "=l"(w0), "=l"(w1) : "r"(e_addr + 4u * g) : "memory");
    const uint32_t s[4] = {(uint32_t)w0, (uint32_t)(w0 >> 32), (uint32_t)w1, (uint32_t)(w1 >> 32)};
    #pragma unroll
    for (int i = 0; i < 4; ++i)
      if (g + i < NE && sm_entry_step(e + g + i, s[i], code, claims)) return true;
  }
  return false;
}

/* one record into the partition held in shared memory; false if the region is full */
__device__ __forceinline__ bool sm_count(uint64_t *sm, uint32_t sm_base, uint32_t region, uint64_t h, unsigned code,
                                         uint32_t home, unsigned long long &slot_claims,
                                         unsigned long long &entry_claims) {
  bool seen_primary = false;
  uint32_t j = home;
  for (uint32_t probe = 0; probe < region; ++probe) {
    const uint32_t a = sm_base + j * 32u;
    uint64_t key, w01;   /* the key and entries 0-1; entries 2-5 only if these do not settle it */
    asm volatile("ld.volatile.shared.v2.u64 {%0, %1}, [%2];" : "=l"(key), "=l"(w01) : "r"(a) : "memory");
    const uint64_t want = h | (seen_primary ? KEY_CONT : 0);
    if (key == KEY_EMPTY) {
      const uint64_t ne0 = (uint64_t)((code << E_CODE_SHIFT) | (1u << E_COUNT_SHIFT));
      uint64_t ohi;
      const uint64_t olo = sm_cas128(a, KEY_EMPTY, 0ull, want, ne0, ohi);
      if (olo == KEY_EMPTY && ohi == 0) { ++slot_claims; ++entry_claims; return true; }
      key = olo;
      w01 = ohi;
    }
    if (key == want) {
      seen_primary = true;
      const uint32_t first[2] = {(uint32_t)w01, (uint32_t)(w01 >> 32)};
      if (sm_count_entries_lazy<6, 2>((uint32_t *)(sm + (uint64_t)j * 4 + 1), a + 8u, first, code, entry_claims))
        return true;
    }
    j = (j + 1 == region) ? 0u : j + 1;
  }
  return false;
}

/* The counting kernel's share of the filter, for thresholded builds: a k-mer that the filter's
 * quick rule drops (its total below the (k+1)-mer lower bound: every entry gets flags 1 and 2 and
 * the slot keeps its bare key; filter_quick) is tallied here and left as it is; every other
 * k-mer's first slot is listed, and the filter then reads only the listed slots. */
struct CandArgs {
  uint32_t *cand;                      /* NULL: no listing */
  uint64_t cap;
  unsigned long long *n_cand, *quick_hist;
  uint64_t t[6];
};

/* One CTA per partition (blockIdx.x counts the partitions of all samples): clear the slots, count
 * the partition's records into them, write the region back.  Partition j of sample s holds the
 * records whose mix has j in its top pbits bits: the bucket (top 8) and the split bits. */
/* the partitions of one launch of k_count_local, as runs of whole samples: the sample whose
 * partitions start at global partition pbase is the launch's partitions [run, run + 2^pbits) */
struct ClassRun { uint32_t run, pbase; };

__global__ void __launch_bounds__(1024) k_count_local(const uint64_t *recs, const unsigned long long *rec_cnt,
                                                       const SGeom *sg, uint32_t nsamples, const ClassRun *cls,
                                                       uint32_t ncls, uint64_t *table, unsigned long long *s_tally,
                                                       CandArgs ca, DevCounters *ctr) {
  extern __shared__ __align__(16) uint64_t sm[];
  /* cls: a batch launches its partitions by region size (each launch with the shared memory its
   * largest region needs), as runs of samples; NULL = partition blockIdx.x */
  uint32_t part = blockIdx.x;
  if (cls) {
    uint32_t lo = 0, hi = ncls;
    while (hi - lo > 1) { const uint32_t m = (lo + hi) >> 1; if (__ldg(&cls[m].run) <= blockIdx.x) lo = m; else hi = m; }
    const ClassRun r = cls[lo];
    part = r.pbase + (blockIdx.x - r.run);
  }
  const uint32_t smp = sample_of_part(sg, nsamples, part);
  const SGeom G = sg[smp];
  const uint64_t j = part - G.pbase;
  const int sbits = G.g.pbits - NBUCKET_BITS;
  const uint32_t region = (uint32_t)G.g.region;
  const int tid = threadIdx.x;
  const uint32_t nt = blockDim.x;   /* the block shape is a tunable (cfg.count_threads) */
  for (uint32_t w = tid; w < region * 4u; w += nt) sm[w] = (w & 3u) == 0 ? KEY_EMPTY : 0ull;
  __syncthreads();
  const uint32_t sm_base = (uint32_t)__cvta_generic_to_shared(sm);
  const uint64_t n = min((unsigned long long)G.cap2, rec_cnt[part]);
  const uint64_t *rp = recs + G.rec2_base + j * G.cap2;
  const uint64_t bucket_hi = (j >> sbits) << LOW_BITS;   /* bucket bits of the mix */
  unsigned long long slots = 0, entries = 0;
  bool full = false;
  uint64_t nxt = tid < n ? __ldcs(rp + tid) : 0ull;
  for (uint64_t i = tid; i < n; i += nt) {
    const uint64_t rec = nxt;
    nxt = i + nt < n ? __ldcs(rp + i + nt) : 0ull;
    if (rec == 0ull) continue;   /* an unused chunk tail, when the buckets are the partitions */
    const uint64_t h = bucket_hi | (rec >> 5);
    const uint32_t home = (uint32_t)__umul64hi(h << (2 + G.g.pbits), G.g.region);
    if (!sm_count(sm, sm_base, region, h, (unsigned)(rec & 31), home, slots, entries)) full = true;
  }
  __syncthreads();
  ulonglong2 *dst = reinterpret_cast<ulonglong2 *>(table + (G.g.base + j * G.g.region) * 4);
  const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(sm);
  for (uint32_t v = tid; v < region * 2u; v += nt) dst[v] = src[v];
  slots = warp_sum(slots); entries = warp_sum(entries);
  if ((tid & 31) == 0) {   /* reductions without a returned value: nothing waits on them */
    if (slots) atomicAdd(&ctr->n_slots_claimed, slots);
    if (entries) {
      atomicAdd(&ctr->n_entries, entries);
      if (s_tally) atomicAdd(&s_tally[(uint64_t)smp * T_NUM + T_ENTRIES], entries);
    }
  }
  if (ca.cand) {
    /* the region is written back: each slot's key word now holds its place in the block's list
     * (~0: not listed), so the listing needs no shared memory of its own */
    __shared__ unsigned int s_nc, s_qh[4];
    __shared__ unsigned long long s_base;
    if (tid < 4) s_qh[tid] = 0;
    if (tid == 0) s_nc = 0;
    __syncthreads();
    /* a quick drop's entries get flags 3 | 8 (k-mer total outside the k bounds) | 4 (entry count
     * outside the k+2 bounds): four possible values, tallied as 16-bit fields of one word (at
     * most 12 slots of 6 entries a thread, so no field can wrap) */
    uint64_t qh = 0;
    const int lane = tid & 31;
    for (uint32_t q0 = 0; q0 < region; q0 += nt) {
      const uint32_t q = q0 + tid;
      bool listed = false;
      if (q < region) {
        const uint64_t key = sm[q * 4];
        if (key != KEY_EMPTY && !(key & KEY_CONT)) {   /* a continuation belongs to its first slot */
          /* entries fill in order: the first empty one ends them (most slots hold one or two) */
          const uint32_t *ew = reinterpret_cast<const uint32_t *>(sm + q * 4 + 1);
          int ne = 0;
          uint32_t kf = 0;
          while (ne < 6 && ew[ne] != 0) kf += entry_count(ew[ne++]);
          kf = min(0xFFFFu, kf);
          listed = ne == 6 || kf >= ca.t[2];
          if (!listed) {
            const uint32_t kout = (kf < ca.t[0] || kf >= ca.t[1]) ? 2u : 0u;
            for (int e = 0; e < ne; ++e) {
              const uint32_t c16 = min(0xFFFFu, entry_count(ew[e]));
              qh += 1ull << (16 * (kout | ((c16 < ca.t[4] || c16 >= ca.t[5]) ? 1u : 0u)));
            }
          }
        }
      }
      const unsigned m = __ballot_sync(~0u, listed);   /* the loop bound is the same for every lane */
      unsigned base = 0;
      if (m && lane == __ffs(m) - 1) base = atomicAdd(&s_nc, (unsigned)__popc(m));
      if (m) base = __shfl_sync(~0u, base, __ffs(m) - 1);
      if (q < region) sm[q * 4] = listed ? (uint64_t)(base + __popc(m & ((1u << lane) - 1))) : ~0ull;
    }
    #pragma unroll
    for (int f = 0; f < 4; ++f) {
      const unsigned long long h = warp_sum((qh >> (16 * f)) & 0xFFFFull);
      if (lane == 0 && h) atomicAdd(&s_qh[f], (unsigned)h);
    }
    __syncthreads();
    if (tid == 0) s_base = s_nc ? atomicAdd(ca.n_cand, (unsigned long long)s_nc) : 0;
    if (tid < 4 && s_qh[tid]) atomicAdd(&ca.quick_hist[3 + 4 * tid], (unsigned long long)s_qh[tid]);
    __syncthreads();
    const uint64_t slot0 = G.g.base + j * G.g.region;
    for (uint32_t q = tid; q < region; q += nt) {
      const uint64_t o = sm[q * 4];
      if (o != ~0ull && s_base + o < ca.cap) ca.cand[s_base + o] = (uint32_t)(slot0 + q);
    }
  }
  if (full) atomicOr(&ctr->err, (unsigned long long)DERR_TABLE_FULL);
}

/* ------------------------------------------------ partitioned count, k > 31
 * The 16-byte records (XRec<KW2>) of the 256 hash buckets are scattered straight into the
 * table: partition j's records go to the memory of its own slot region (room for four records
 * a 64-byte slot), and k_count_local2 reads them into shared memory before it writes the
 * counted region over them, so the records need no second buffer. */
constexpr int MAX_SPLIT_BITS2 = 16;

/* The scatter split (k > 31 always; k <= 31 when a table needs more partitions than k_split's
 * shared-memory counting sort handles): every record goes straight to the memory of its own
 * partition's slot region, four records a slot.  Warps take 32-record runs in order; the runs of
 * a window of `win` buckets (a power of two) are interleaved round robin over its buckets, so
 * that the atomics in flight spread over at least 8192 partition cursors (a bucket of a small
 * table has few partitions, and all warps queueing on them measured 8 times slower), while the
 * scattered stores stay inside as small a share of the table as that allows (at large k one
 * bucket: spreading them over two buckets' 0.85 GB measured 1.2 times slower, over the whole
 * 109 GB table 2.4 times).  Each thread keeps SPLIT2_U records in flight.  A bucket's runs are
 * counted up to a power of two (2^lg_runs; the padding runs are empty), so that a run's bucket
 * and place come from shifts, not from 64-bit divisions. */
template <class KT> struct ScatterRec;
template <> struct ScatterRec<KW1> {   /* [low 54 bits of the mix | code:5] */
  using T = uint64_t;
  __device__ static __forceinline__ bool none(T r) { return r == 0ull; }
  __device__ static __forceinline__ uint64_t sub(T r, int sbits) { return sbits ? (r >> (5 + LOW_BITS - sbits)) : 0ull; }
};
template <> struct ScatterRec<KW2> {   /* x = (H << 8) | code, y = high word */
  using T = ulonglong2;
  __device__ static __forceinline__ bool none(T r) { return r.x == 0ull; }
  __device__ static __forceinline__ uint64_t sub(T r, int sbits) { return sbits ? (r.x >> (64 - sbits)) : 0ull; }
};
constexpr int SPLIT2_U = 4;
template <class KT>
__global__ void __launch_bounds__(TPB) k_split_scatter(const typename ScatterRec<KT>::T *records,
                                                        const unsigned long long *bucket_cnt, uint64_t cap,
                                                        int lg_runs, int lg_win, TableGeom g, uint64_t *table,
                                                        unsigned long long *sub_cnt, DevCounters *ctr) {
  using R = ScatterRec<KT>;
  using T = typename R::T;
  constexpr int SU = Slot<KT>::U64;
  const int sbits = g.pbits - NBUCKET_BITS;
  const uint64_t room = 4 * g.region;
  const int lane = threadIdx.x & 31;
  const uint64_t nwarps = (uint64_t)gridDim.x * (TPB / 32);
  const uint64_t total = (uint64_t)NBUCKET << lg_runs;
  const int lg_per_win = lg_runs + lg_win;
  const uint64_t win_mask = (1ull << lg_win) - 1, per_win_mask = (1ull << lg_per_win) - 1;
  bool over = false;
  for (uint64_t g0 = (uint64_t)blockIdx.x * (TPB / 32) + (threadIdx.x >> 5); g0 < total; g0 += nwarps * SPLIT2_U) {
    T r[SPLIT2_U];
    unsigned bk[SPLIT2_U];
    #pragma unroll
    for (int u = 0; u < SPLIT2_U; ++u) {
      const uint64_t run = g0 + (uint64_t)u * nwarps;
      const uint64_t w = run >> lg_per_win, rr = run & per_win_mask;
      bk[u] = (unsigned)((w << lg_win) + (rr & win_mask));
      const uint64_t i = ((rr >> lg_win) << 5) + lane;
      r[u] = T{};
      if (run < total && i < min((unsigned long long)cap, bucket_cnt[bk[u]])) r[u] = __ldcs(records + (uint64_t)bk[u] * cap + i);
    }
    unsigned long long o[SPLIT2_U];
    uint64_t j[SPLIT2_U];
    #pragma unroll
    for (int u = 0; u < SPLIT2_U; ++u) {
      if (R::none(r[u])) continue;   /* past the bucket's end, or an unused chunk tail */
      /* the partition: the bucket, then the mix bits right below it */
      j[u] = ((uint64_t)bk[u] << sbits) | R::sub(r[u], sbits);
      o[u] = atomicAdd(&sub_cnt[j[u]], 1ull);
    }
    #pragma unroll
    for (int u = 0; u < SPLIT2_U; ++u) {
      if (R::none(r[u])) continue;
      if (o[u] < room) __stcs(reinterpret_cast<T *>(table + (g.base + j[u] * g.region) * SU) + o[u], r[u]);
      else over = true;
    }
  }
  if (over) atomicOr(&ctr->err, (unsigned long long)DERR_TABLE_FULL);
}

using bruno_table_plan::scatter_lg_runs;
using bruno_table_plan::scatter_lg_window;

/* The scatter split bucket after bucket, for tables whose window is one bucket (large tables):
 * grid row y is bucket y, its blocks stride over the bucket's records, one record a thread
 * (measured 60 ms at large k against 70-73 for the windowed form above run on one bucket) */
template <class KT>
__global__ void __launch_bounds__(TPB) k_split_scatter_rows(const typename ScatterRec<KT>::T *records,
                                                             const unsigned long long *bucket_cnt, uint64_t cap,
                                                             TableGeom g, uint64_t *table, unsigned long long *sub_cnt,
                                                             DevCounters *ctr) {
  using R = ScatterRec<KT>;
  using T = typename R::T;
  constexpr int SU = Slot<KT>::U64;
  const int sbits = g.pbits - NBUCKET_BITS;
  const uint64_t room = 4 * g.region;
  const unsigned b = blockIdx.y;
  const uint64_t n = min((unsigned long long)cap, bucket_cnt[b]);
  const T *rb = records + (uint64_t)b * cap;
  bool over = false;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const T r = __ldcs(rb + i);
    if (R::none(r)) continue;   /* an unused chunk tail */
    const uint64_t j = ((uint64_t)b << sbits) | R::sub(r, sbits);
    const unsigned long long o = atomicAdd(&sub_cnt[j], 1ull);
    if (o < room) __stcs(reinterpret_cast<T *>(table + (g.base + j * g.region) * SU) + o, r);
    else over = true;
  }
  if (over) atomicOr(&ctr->err, (unsigned long long)DERR_TABLE_FULL);
}

int num_sms();
/* the scatter split's launch: bucket after bucket when the window is one bucket, else windows */
template <class KT>
void launch_scatter(const typename ScatterRec<KT>::T *records, const unsigned long long *bucket_cnt, uint64_t cap,
                    int pbits, TableGeom g, uint64_t *table, unsigned long long *sub_cnt, DevCounters *ctr,
                    cudaStream_t s);
/* blocks of the scatter split: one resident wave (no more than its warps' runs need) */
template <class KT>
unsigned scatter_blocks(int lg_runs) {
  static const int occ = [] {
    int o = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_split_scatter<KT>, TPB, 0) == cudaSuccess && o > 0 ? o
                                                                                                                : 4;
  }();
  const uint64_t runs = (uint64_t)NBUCKET << lg_runs, per_block = (TPB / 32) * SPLIT2_U;
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)num_sms() * occ, (runs + per_block - 1) / per_block));
}

template <class KT>
void launch_scatter(const typename ScatterRec<KT>::T *records, const unsigned long long *bucket_cnt, uint64_t cap,
                    int pbits, TableGeom g, uint64_t *table, unsigned long long *sub_cnt, DevCounters *ctr,
                    cudaStream_t s) {
  const int lg_win = scatter_lg_window(pbits);
  if (lg_win == 0) {
    const unsigned gx = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)num_sms() * 8, (cap + TPB - 1) / TPB));
    k_split_scatter_rows<KT><<<dim3(gx, NBUCKET), TPB, 0, s>>>(records, bucket_cnt, cap, g, table, sub_cnt, ctr);
  } else {
    const int lg_runs = scatter_lg_runs(cap);
    k_split_scatter<KT><<<scatter_blocks<KT>(lg_runs), TPB, 0, s>>>(records, bucket_cnt, cap, lg_runs, lg_win, g, table,
                                                                    sub_cnt, ctr);
  }
}

/* one record into a 64-byte slot region in shared memory (key 2 words, 12 entry words);
 * false if the region is full */
__device__ __forceinline__ bool sm_count2(uint64_t *sm, uint32_t sm_base, uint32_t region, uint64_t lo, uint64_t hi,
                                          unsigned code, uint32_t home, unsigned long long &slot_claims,
                                          unsigned long long &entry_claims) {
  bool seen_primary = false;
  uint32_t j = home;
  for (uint32_t probe = 0; probe < region; ++probe) {
    const uint32_t a = sm_base + j * 64u;
    uint64_t k0, k1;
    asm volatile("ld.volatile.shared.v2.u64 {%0, %1}, [%2];" : "=l"(k0), "=l"(k1) : "r"(a) : "memory");
    const uint64_t whi = hi | (seen_primary ? KEY_CONT : 0);
    if (k0 == KEY_EMPTY && k1 == KEY_EMPTY) {
      uint64_t ohi;
      const uint64_t olo = sm_cas128(a, KEY_EMPTY, KEY_EMPTY, lo, whi, ohi);
      if (olo == KEY_EMPTY && ohi == KEY_EMPTY) { ++slot_claims; k0 = lo; k1 = whi; }
      else { k0 = olo; k1 = ohi; }
    }
    if (k0 == lo && k1 == whi) {   /* the entries, four at a time as far as they are needed */
      seen_primary = true;
      if (sm_count_entries_lazy<12, 0>((uint32_t *)(sm + (uint64_t)j * 8 + 2), a + 16u, nullptr, code, entry_claims))
        return true;
    }
    j = (j + 1 == region) ? 0u : j + 1;
  }
  return false;
}

/* One CTA per partition j: clear its slots in shared memory, count its records (read from the
 * region's own memory, where k_split_scatter put them), write the region back over them; with
 * thresholds, list the slots the filter must read, as k_count_local does.  512 threads a CTA,
 * bounded to 40 registers so that three CTAs share an SM. */
constexpr int PTPB2 = 512;
__global__ void __launch_bounds__(PTPB2, 3) k_count_local2(const unsigned long long *sub_cnt, TableGeom g, uint64_t *table,
                                                        CandArgs ca, DevCounters *ctr) {
  extern __shared__ __align__(16) uint64_t sm[];
  const uint64_t j = blockIdx.x;
  const int sbits = g.pbits - NBUCKET_BITS;
  const uint32_t region = (uint32_t)g.region;
  const int tid = threadIdx.x;
  const uint32_t nt = blockDim.x;
  for (uint32_t w = tid; w < region * 8u; w += nt) sm[w] = (w & 7u) < 2 ? KEY_EMPTY : 0ull;
  __syncthreads();
  const uint32_t sm_base = (uint32_t)__cvta_generic_to_shared(sm);
  uint64_t *reg = table + (g.base + j * g.region) * 8;
  const uint64_t n = min((unsigned long long)(4 * g.region), sub_cnt[j]);
  const ulonglong2 *rp = reinterpret_cast<const ulonglong2 *>(reg);
  const uint64_t bucket_hi = (j >> sbits) << 56;   /* the bucket: the hash's top 8 bits */
  unsigned long long slots = 0, entries = 0;
  bool full = false;
  ulonglong2 nxt = tid < n ? __ldcs(rp + tid) : make_ulonglong2(0ull, 0ull);
  for (uint64_t i = tid; i < n; i += nt) {
    const ulonglong2 r = nxt;
    nxt = i + nt < n ? __ldcs(rp + i + nt) : make_ulonglong2(0ull, 0ull);
    const uint64_t h = bucket_hi | (r.x >> 8);   /* the table key is (h, high word) */
    const uint32_t home = (uint32_t)__umul64hi(h << g.pbits, g.region);
    if (!sm_count2(sm, sm_base, region, h, r.y, (unsigned)(r.x & 31u), home, slots, entries)) full = true;
  }
  __syncthreads();   /* every record is read: the region's memory is free for the slots */
  ulonglong2 *dst = reinterpret_cast<ulonglong2 *>(reg);
  const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(sm);
  for (uint32_t v = tid; v < region * 4u; v += nt) dst[v] = src[v];
  slots = warp_sum(slots); entries = warp_sum(entries);
  if ((tid & 31) == 0) {
    if (slots) atomicAdd(&ctr->n_slots_claimed, slots);
    if (entries) atomicAdd(&ctr->n_entries, entries);
  }
  if (ca.cand) {   /* as in k_count_local, with 12 entries a slot */
    __shared__ unsigned int s_nc, s_qh[4];
    __shared__ unsigned long long s_base;
    if (tid < 4) s_qh[tid] = 0;
    if (tid == 0) s_nc = 0;
    __syncthreads();
    uint64_t qh = 0;
    const int lane = tid & 31;
    for (uint32_t q0 = 0; q0 < region; q0 += nt) {
      const uint32_t q = q0 + tid;
      bool listed = false;
      if (q < region) {
        const uint64_t k0 = sm[q * 8], k1 = sm[q * 8 + 1];
        if (!(k0 == KEY_EMPTY && k1 == KEY_EMPTY) && !(k1 & KEY_CONT)) {
          /* entries fill in order: the first empty one ends them (most slots hold one or two) */
          const uint32_t *ew = reinterpret_cast<const uint32_t *>(sm + q * 8 + 2);
          int ne = 0;
          uint32_t kf = 0;
          while (ne < 12 && ew[ne] != 0) kf += entry_count(ew[ne++]);
          kf = min(0xFFFFu, kf);
          listed = ne == 12 || kf >= ca.t[2];
          if (!listed) {
            const uint32_t kout = (kf < ca.t[0] || kf >= ca.t[1]) ? 2u : 0u;
            for (int e = 0; e < ne; ++e) {
              const uint32_t c16 = min(0xFFFFu, entry_count(ew[e]));
              qh += 1ull << (16 * (kout | ((c16 < ca.t[4] || c16 >= ca.t[5]) ? 1u : 0u)));
            }
          }
        }
      }
      const unsigned m = __ballot_sync(~0u, listed);   /* the loop bound is the same for every lane */
      unsigned base = 0;
      if (m && lane == __ffs(m) - 1) base = atomicAdd(&s_nc, (unsigned)__popc(m));
      if (m) base = __shfl_sync(~0u, base, __ffs(m) - 1);
      if (q < region) sm[q * 8] = listed ? (uint64_t)(base + __popc(m & ((1u << lane) - 1))) : ~0ull;
    }
    #pragma unroll
    for (int f = 0; f < 4; ++f) {
      const unsigned long long h = warp_sum((qh >> (16 * f)) & 0xFFFFull);
      if (lane == 0 && h) atomicAdd(&s_qh[f], (unsigned)h);
    }
    __syncthreads();
    if (tid == 0) s_base = s_nc ? atomicAdd(ca.n_cand, (unsigned long long)s_nc) : 0;
    if (tid < 4 && s_qh[tid]) atomicAdd(&ca.quick_hist[3 + 4 * tid], (unsigned long long)s_qh[tid]);
    __syncthreads();
    const uint64_t slot0 = g.base + j * g.region;
    for (uint32_t q = tid; q < region; q += nt) {
      const uint64_t o = sm[q * 8];
      if (o != ~0ull && s_base + o < ca.cap) ca.cand[s_base + o] = (uint32_t)(slot0 + q);
    }
  }
  if (full) atomicOr(&ctr->err, (unsigned long long)DERR_TABLE_FULL);
}

/* table initialisation: every key word EMPTY, every entry 0; written as one flat word
 * array so that every warp store is 256 contiguous bytes */
template <class KT>
__global__ void k_table_init(uint64_t *table, uint64_t nslots) {
  constexpr int SU = Slot<KT>::U64, KWD = Slot<KT>::KEYW;
  const uint64_t nw = nslots * SU;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += (uint64_t)gridDim.x * blockDim.x)
    table[i] = ((int)(i % SU) < KWD) ? KEY_EMPTY : 0ull;
}

/* ============================================================ raw (k+2)-mer dump */
template <class KT>
__global__ void __launch_bounds__(TPB) k_dump_k2(const uint64_t *table, uint64_t nslots, uint64_t *keys, uint8_t *edges,
                                                  uint32_t *counts, uint64_t cap, DevCounters *ctr) {
  constexpr int SU = Slot<KT>::U64, NE = Slot<KT>::ENTRIES, KWD = Slot<KT>::KEYW;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t *s = table + i * SU;
    KT key = KOps<KT>::load(s);
    if (key_dead(key)) continue;
    ((uint64_t *)&key)[KWD - 1] &= ~KEY_CONT;  /* continuation slots belong to the same k-mer */
    key = key_kmer(key);
    const uint32_t *e = (const uint32_t *)(s + KWD);
    for (int j = 0; j < NE; ++j) {
      if (e[j] == 0) continue;
      unsigned long long o = atomicAdd(&ctr->n_k2_dump, 1ull);
      if (o < cap) {
        KOps<KT>::store(keys + o * KWD, key);
        edges[o] = code_biedge(entry_code(e[j]));
        /* past 2^24 the exact count is the word's plus the side table's, kept to 32 bits as the
         * reference's uint32 counter keeps it */
        counts[o] = (e[j] & E_BIG) ? (uint32_t)((e[j] >> E_COUNT_SHIFT) + big_get(ctr, (unsigned long long)(uintptr_t)(e + j)))
                                   : entry_count(e[j]);
      }
    }
  }
}

/* ============================================================ filter + insert */

/* The filter over the whole table, for counts that did not filter as they went.  A block
 * takes chunks of FCHUNK slots: pass 1 quick-drops what it can and lists the k-mers that need
 * the full filter, pass 2 runs those with every lane busy and lists the nodes, and each chunk
 * appends its chain / branch node lists with one reservation each. */
constexpr int FCHUNK = TPB * 8;
template <class KT>
__global__ void __launch_bounds__(TPB) k_filter(FilterArgs a) {
  constexpr int SU = Slot<KT>::U64, NE = Slot<KT>::ENTRIES, KWD = Slot<KT>::KEYW;
  __shared__ unsigned long long s_hist[16], s_nodes;
  __shared__ uint16_t s_cand[FCHUNK];
  __shared__ uint32_t s_chain[FCHUNK], s_branch[FCHUNK];
  __shared__ uint32_t s_nc, s_nb, s_ncand;
  __shared__ unsigned long long s_base_c, s_base_b;
  const int tid = threadIdx.x, lane = tid & 31;
  if (tid < 16) s_hist[tid] = 0;
  if (tid == 0) s_nodes = 0;
  FilterTally t;
  t.hist.clear();
  const uint64_t limit = a.cand ? a.n_cand : a.nslots;   /* chunks of listed slots, or of slots */
  for (uint64_t c0 = (uint64_t)blockIdx.x * FCHUNK; c0 < limit; c0 += (uint64_t)gridDim.x * FCHUNK) {
    if (tid == 0) { s_nc = 0; s_nb = 0; s_ncand = 0; }
    /* a batch: the chunk's slots belong to sample s0 up to `bound` and to s0 + 1 after it (a
     * sample has at least 256 partitions of 64 slots, more than a chunk) */
    uint32_t s0 = 0;
    uint64_t bound = ~0ull;
    if (a.S > 1 && !a.cand) {
      s0 = sample_of_slot(a.sg, a.S, c0);
      if (s0 + 1 < a.S) bound = a.sg[s0 + 1].g.base;
    }
    __syncthreads();
    if (t.hist.n >= FlagHist::DRAIN) {   /* drain the 16-bit bins long before they could wrap */
      #pragma unroll
      for (int f = 0; f < 16; ++f)
        if (t.hist.get(f)) atomicAdd(&s_hist[f], t.hist.get(f));
      t.hist.clear();
    }
    /* pass 1 (listed slots all go to pass 2) */
    if (a.cand) {
      const uint32_t nchunk = (uint32_t)min((uint64_t)FCHUNK, limit - c0);
      for (uint32_t x = tid; x < nchunk; x += TPB) s_cand[x] = (uint16_t)x;
      if (tid == 0) s_ncand = nchunk;
    }
    #pragma unroll 2
    for (int r = 0; r < (a.cand ? 0 : FCHUNK / TPB); ++r) {
      const uint32_t off = (uint32_t)(r * TPB + tid);
      const uint64_t i = c0 + off;
      bool full_pass = false;
      if (i < a.nslots) {
        uint64_t *s = a.table + i * SU;
        uint64_t raw[SU];
        ld_slot<SU>(s, raw);
        const KT key = KOps<KT>::load(raw);
        if (!key_dead(key) && !key_cont(key)) {
          uint32_t w[NE];
          int ne = 0;
          #pragma unroll
          for (int q = 0; q < NE; ++q) {
            w[q] = (uint32_t)(raw[KWD + q / 2] >> (32 * (q & 1)));
            ne += w[q] != 0;
          }
          full_pass = ne == NE || !filter_quick<KT, NE>(s, w, ne, a, t);
        }
      }
      const unsigned m = __ballot_sync(~0u, full_pass);
      if (m) {
        const int leader = __ffs(m) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(&s_ncand, (unsigned)__popc(m));
        base = __shfl_sync(~0u, base, leader);
        if (full_pass) s_cand[base + __popc(m & ((1u << lane) - 1))] = (uint16_t)off;
      }
    }
    __syncthreads();
    /* pass 2 */
    const unsigned ncand = s_ncand;
    for (unsigned x = tid; x < ncand; x += TPB) {
      const uint64_t i = a.cand ? (uint64_t)a.cand[c0 + s_cand[x]] : c0 + s_cand[x];
      uint64_t *s = a.table + i * SU;
      uint64_t raw[SU];
      ld_slot<SU>(s, raw);
      const KT key = KOps<KT>::load(raw);
      uint32_t w[NE];
      int ne = 0;
      #pragma unroll
      for (int q = 0; q < NE; ++q) {
        w[q] = (uint32_t)(raw[KWD + q / 2] >> (32 * (q & 1)));
        ne += w[q] != 0;
      }
      t.kind = 0;
      t.sample = a.cand && a.S > 1 ? sample_of_slot(a.sg, a.S, i) : (i < bound ? s0 : s0 + 1);
      if (ne < NE) filter_kmer<KT, NE, false>(s, i, key, w, ne, a, t);
      else filter_wide_global<KT>(s, i, key, w, a, t);   /* continuation slots */
      if (t.kind == 1) s_chain[atomicAdd(&s_nc, 1u)] = (uint32_t)i;
      if (t.kind == 2) s_branch[atomicAdd(&s_nb, 1u)] = (uint32_t)i;
    }
    __syncthreads();
    if (tid == 0) {
      s_base_c = s_nc ? atomicAdd(&a.ctr->n_chain, (unsigned long long)s_nc) : 0;
      s_base_b = s_nb ? atomicAdd(&a.ctr->n_branch, (unsigned long long)s_nb) : 0;
    }
    __syncthreads();
    for (unsigned x = tid; x < s_nc; x += TPB) {
      const unsigned long long o = s_base_c + x;
      const uint32_t sl = s_chain[x];
      if (o < a.list_cap) {
        a.chain_list[o] = sl;
        uint64_t *pw = a.table + (uint64_t)sl * SU + KWD;
        pw[2] = (pw[2] & 0xFFFFFFFFull) | (o << 32);   /* chain index */
      }
    }
    for (unsigned x = tid; x < s_nb; x += TPB)
      if (s_base_b + x < a.list_cap) a.branch_list[s_base_b + x] = s_branch[x];
    if (a.s_tally && a.cand) {   /* per-sample node tallies of listed slots: each node's own sample */
      for (int list = 0; list < 2; ++list) {
        const unsigned cnt = list ? s_nb : s_nc;
        const uint32_t *sl = list ? s_branch : s_chain;
        for (unsigned x0 = 0; x0 < cnt; x0 += TPB) {   /* the same bound for every thread */
          const unsigned x = x0 + tid;
          const uint32_t smp = x < cnt ? sample_of_slot(a.sg, a.S, sl[x]) : ~0u;
          const unsigned peers = __match_any_sync(~0u, smp);
          if (x < cnt && lane == __ffs(peers) - 1)
            atomicAdd(&a.s_tally[(uint64_t)smp * T_NUM + (list ? T_BRANCH : T_CHAIN)],
                      (unsigned long long)__popc(peers));
        }
      }
    } else if (a.s_tally) {   /* per-sample node tallies: the chunk's nodes past `bound` are s0 + 1's */
      unsigned hc = 0, hb = 0;
      for (unsigned x = tid; x < s_nc; x += TPB) hc += s_chain[x] >= bound;
      for (unsigned x = tid; x < s_nb; x += TPB) hb += s_branch[x] >= bound;
      hc = (unsigned)warp_sum(hc); hb = (unsigned)warp_sum(hb);
      if (lane == 0 && hc) atomicAdd(&a.s_tally[(uint64_t)(s0 + 1) * T_NUM + T_CHAIN], (unsigned long long)hc);
      if (lane == 0 && hb) atomicAdd(&a.s_tally[(uint64_t)(s0 + 1) * T_NUM + T_BRANCH], (unsigned long long)hb);
      if (tid == 0 && s_nc) atomicAdd(&a.s_tally[(uint64_t)s0 * T_NUM + T_CHAIN], (unsigned long long)s_nc);
      if (tid == 0 && s_nb) atomicAdd(&a.s_tally[(uint64_t)s0 * T_NUM + T_BRANCH], (unsigned long long)s_nb);
      /* s0 got every node of the chunk: take back those past `bound` */
      if (lane == 0 && hc) atomicAdd(&a.s_tally[(uint64_t)s0 * T_NUM + T_CHAIN], (unsigned long long)(0 - (unsigned long long)hc));
      if (lane == 0 && hb) atomicAdd(&a.s_tally[(uint64_t)s0 * T_NUM + T_BRANCH], (unsigned long long)(0 - (unsigned long long)hb));
    }
    __syncthreads();   /* every thread has read s_nc / s_nb before the next chunk resets them */
  }
  unsigned long long nodes = warp_sum(t.nodes);
  if (lane == 0) atomicAdd(&s_nodes, nodes);
  #pragma unroll
  for (int f = 0; f < 16; ++f) {
    unsigned long long h = warp_sum(t.hist.get(f));
    if (lane == 0 && h) atomicAdd(&s_hist[f], h);
  }
  __syncthreads();
  if (tid < 16 && s_hist[tid]) atomicAdd(&a.ctr->flag_hist[tid], s_hist[tid]);
  if (tid == 0) atomicAdd(&a.ctr->n_nodes, s_nodes);
}

/* live graph nodes -> arrays */
template <class KT>
__global__ void __launch_bounds__(TPB) k_dump_nodes(const uint64_t *table, uint64_t nslots, uint64_t *keys,
                                                     uint16_t *counts, uint8_t *flags, uint64_t cap,
                                                     unsigned long long *n) {
  constexpr int SU = Slot<KT>::U64, KWD = Slot<KT>::KEYW;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t *s = table + i * SU;
    KT key = KOps<KT>::load(s);
    if (!key_is_node(key)) continue;
    unsigned long long o = atomicAdd(n, 1ull);
    if (o >= cap) continue;
    KOps<KT>::store(keys + o * KWD, key_kmer(node_key(key)));
    const uint64_t *pw = s + KWD;
    for (int q = 0; q < 4; ++q) {
      counts[o * 9 + q] = (uint16_t)(pw[0] >> (16 * q));
      counts[o * 9 + 4 + q] = (uint16_t)(pw[1] >> (16 * q));
    }
    counts[o * 9 + 8] = (uint16_t)pw[2];
    if (flags) flags[o] = (uint8_t)((pw[2] >> 16) & (NF_BRANCH | NF_CHAIN));
  }
}

/* ============================================================ scan */
__global__ void __launch_bounds__(1024) k_scan_single(const uint64_t *in, uint64_t *out, uint64_t n,
                                                       unsigned long long *total) {
  __shared__ uint64_t part[1024];
  const uint64_t per = (n + 1023) / 1024;
  const uint64_t b = threadIdx.x * per, e = min(n, b + per);
  uint64_t s = 0;
  for (uint64_t i = b; i < e; ++i) s += in[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    uint64_t v = (threadIdx.x >= (unsigned)o) ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint64_t run = part[threadIdx.x] - s;
  for (uint64_t i = b; i < e; ++i) { uint64_t v = in[i]; out[i] = run; run += v; }
  if (threadIdx.x == 1023 && total) *total = part[1023];
}

int num_sms() {
  /* function-local statics below are initialised once, thread-safely (contexts may run on
   * several host threads) */
  static const int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  return sms;
}

template <class KT>
bruno_status count_typed(Ctx *c);
template <class KT>
bruno_status filter_typed(Ctx *c, const uint64_t *thr);

/* The multi-block scan: block b owns elements [b * chunk, (b + 1) * chunk).  Pass 1 sums each
 * block's elements, the single-block scan turns the sums into block offsets, pass 2 scans each
 * block's elements from its offset.  Every access is a coalesced run: a thread takes SCAN_V
 * consecutive elements of a tile of SCAN_TPB * SCAN_V. */
constexpr int SCAN_TPB = 1024, SCAN_V = 4;
constexpr uint64_t SCAN_TILE = (uint64_t)SCAN_TPB * SCAN_V;

__device__ __forceinline__ uint64_t block_sum_u64(uint64_t v, uint64_t *warp_part) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) warp_part[wid] = v;
  __syncthreads();
  uint64_t t = lane < (int)(blockDim.x >> 5) ? warp_part[lane] : 0;
  t = warp_sum(t);
  __syncthreads();   /* warp_part is reused by the caller's next call */
  return t;
}

__global__ void __launch_bounds__(SCAN_TPB) k_scan_reduce(const uint64_t *in, uint64_t n, uint64_t chunk,
                                                           uint64_t *block_sum) {
  __shared__ uint64_t wp[32];
  const uint64_t b0 = (uint64_t)blockIdx.x * chunk, b1 = min(n, b0 + chunk);
  uint64_t s = 0;
  for (uint64_t i = b0 + threadIdx.x; i < b1; i += SCAN_TPB) s += in[i];
  s = block_sum_u64(s, wp);
  if (threadIdx.x == 0) block_sum[blockIdx.x] = s;
}

__global__ void __launch_bounds__(SCAN_TPB) k_scan_apply(const uint64_t *in, uint64_t *out, uint64_t n, uint64_t chunk,
                                                          const uint64_t *block_off) {
  __shared__ uint64_t wp[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t b0 = (uint64_t)blockIdx.x * chunk, b1 = min(n, b0 + chunk);
  uint64_t carry = block_off[blockIdx.x];
  for (uint64_t t0 = b0; t0 < b1; t0 += SCAN_TILE) {
    const uint64_t i0 = t0 + (uint64_t)threadIdx.x * SCAN_V;
    uint64_t v[SCAN_V], sum = 0;
    #pragma unroll
    for (int q = 0; q < SCAN_V; ++q) {
      v[q] = i0 + q < b1 ? in[i0 + q] : 0;
      sum += v[q];
    }
    /* exclusive scan of the threads' sums: warp shuffles, then the warps' totals */
    uint64_t inc = sum;
    #pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t y = __shfl_up_sync(~0u, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) wp[wid] = inc;
    __syncthreads();
    if (wid == 0) {
      uint64_t w = lane < (SCAN_TPB >> 5) ? wp[lane] : 0;
      #pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(~0u, w, o);
        if (lane >= o) w += y;
      }
      wp[lane] = w;   /* inclusive totals of warps 0..lane */
    }
    __syncthreads();
    uint64_t run = carry + (wid ? wp[wid - 1] : 0) + inc - sum;
    const uint64_t tile_total = wp[(SCAN_TPB >> 5) - 1];
    #pragma unroll
    for (int q = 0; q < SCAN_V; ++q) {
      if (i0 + q < b1) out[i0 + q] = run;
      run += v[q];
    }
    carry += tile_total;
    __syncthreads();   /* wp is rewritten by the next tile */
  }
}

}  // namespace

int scan_u64(const uint64_t *in, uint64_t *out, uint64_t n, unsigned long long *total_dev, cudaStream_t s,
             uint64_t *scratch) {
  const uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles <= 2 || !scratch) {
    k_scan_single<<<1, 1024, 0, s>>>(in, out, n, total_dev);
    return 1;
  }
  /* blocks of a whole number of tiles, at most 1024 of them (the offsets' scan is one block) */
  const uint64_t nb_max = std::min<uint64_t>(1024, (uint64_t)num_sms() * 2);
  const uint64_t tiles_per = (tiles + nb_max - 1) / nb_max;
  const uint64_t chunk = tiles_per * SCAN_TILE;
  const unsigned nb = (unsigned)((n + chunk - 1) / chunk);
  k_scan_reduce<<<nb, SCAN_TPB, 0, s>>>(in, n, chunk, scratch);
  k_scan_single<<<1, 1024, 0, s>>>(scratch, scratch, nb, total_dev);
  k_scan_apply<<<nb, SCAN_TPB, 0, s>>>(in, out, n, chunk, scratch);
  return 3;
}

bruno_status scan_ctx(Ctx *c, const uint64_t *in, uint64_t *out, uint64_t n, unsigned long long *total_dev) {
  bruno_status st = ensure(c, c->scan_tmp, 1024 * 8);
  if (st != BRUNO_OK) return st;
  c->launches += scan_u64(in, out, n, total_dev, c->stream, (uint64_t *)c->scan_tmp.p);
  return BRUNO_OK;
}

/* ------------------------------------------------------------ read index */
bruno_status batch_segment(Ctx *c, size_t si, uint64_t r0, uint64_t r1);
namespace {
bruno_status extract_begin(Ctx *c, uint64_t upper, int max_blocks);
void extract_reads(Ctx *c, uint64_t r0, uint64_t r1);
int wx_blocks(uint64_t nr);
}  // namespace

/* Indexes every FASTQ segment.  A segment copied from the host in pieces (load_fastq) is
 * indexed as soon as its piece has landed, and on the partitioned path its reads are extracted
 * right away, so parsing and extraction run under the remaining copies. */
bruno_status run_index_reads(Ctx *c) {
  bruno_status st;
  /* first pass: sizes for every segment */
  uint64_t total_tiles = 0, total_bytes = 0;
  for (auto &sg : c->segs) {
    total_tiles = std::max<uint64_t>(total_tiles, (sg.n + TILE - 1) / TILE);
    total_bytes += sg.n;
  }
  if ((st = ensure(c, c->tile_cnt, std::max<uint64_t>(1, total_tiles) * 8)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->tile_base, std::max<uint64_t>(1, total_tiles) * 8)) != BRUNO_OK) return st;
  bool piped = false;
  for (auto &sg : c->segs) piped |= sg.ev >= 0;
  c->pre_extracted = piped && c->S == 1 && c->W == 1 && !c->cfg.edge_filter && c->force_direct_count != 1;
  const bool batch_hook = piped && c->S > 1 && c->batch_piped;   /* a batch extracts group by group */
  cudaMemsetAsync(c->dctr, 0, offsetof(DevCounters, hll), c->stream);
  if (c->pre_extracted) {
    /* every record holds its sequence and an equally long quality line, so the k-mer
     * positions of all reads are at most half the bytes */
    int blocks = 0;   /* one launch a segment, bounded as extract_reads bounds it (8 bytes a read at least) */
    for (auto &sg : c->segs) blocks += wx_blocks(sg.n / 8 + 1);
    if ((st = extract_begin(c, total_bytes / 2 + 1, std::max(1, blocks))) != BRUNO_OK) return st;
    cudaEventRecord(c->kev[0], c->stream);
  }
  /* the read arrays need the record count first; newline counts give an upper bound */
  uint64_t rcap = 0;
  for (size_t si = 0; si < c->segs.size(); ++si) {
    const Segment &sg = c->segs[si];
    if (sg.n == 0) continue;
    if (sg.ev >= 0) cudaStreamWaitEvent(c->stream, c->seg_ev[sg.ev], 0);
    const uint64_t tiles = (sg.n + TILE - 1) / TILE;
    cudaMemsetAsync(&c->dctr->n_newlines_eff, 0, 8, c->stream);   /* the extraction's tallies stay */
    long long neg = -1;
    unsigned long long nb = ~0ull;
    cudaMemcpyAsync(&c->dctr->last_nonws, &neg, sizeof(neg), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(&c->dctr->bad_line, &nb, sizeof(nb), cudaMemcpyHostToDevice, c->stream);
    c->launches += 2;   /* k_tile_stats, k_index_lines; the scan counts its own */
    const bool aligned = ((uintptr_t)sg.ptr & 15) == 0;
    k_tile_stats<<<(unsigned)tiles, TPB, 0, c->stream>>>((const unsigned char *)sg.ptr, sg.n, (uint64_t *)c->tile_cnt.p,
                                                          c->dctr, aligned);
    if ((st = scan_ctx(c, (const uint64_t *)c->tile_cnt.p, (uint64_t *)c->tile_base.p, tiles, &c->dctr->n_records)) !=
        BRUNO_OK)
      return st;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    /* n_records temporarily holds the total newline count: records <= newlines / 4 + 1 */
    uint64_t upper = c->hctr->n_records / 4 + 1;
    /* grow keeping the spans of earlier files; pieces of one input grow once, for all pieces
     * at the first piece's records per byte */
    if ((c->pre_extracted || batch_hook) && si == 0 && sg.n > 0)
      upper = std::max<uint64_t>(upper, (uint64_t)((double)upper * (double)total_bytes / (double)sg.n * 1.05) + 1);
    if ((st = ensure(c, c->rstart, (rcap + upper) * 8, true)) != BRUNO_OK) return st;
    if ((st = ensure(c, c->rend, (rcap + upper) * 8, true)) != BRUNO_OK) return st;
    k_index_lines<<<(unsigned)tiles, TPB, 0, c->stream>>>((const unsigned char *)sg.ptr, sg.n,
                                                           (const uint64_t *)c->tile_base.p, (uint64_t *)c->rstart.p,
                                                           (uint64_t *)c->rend.p, rcap, rcap + upper, c->dctr,
                                                           aligned);
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    const DevCounters &h = *c->hctr;
    if (h.last_nonws < 0) continue;  /* empty or blank file */
    const uint64_t lines = h.n_newlines_eff + 1;
    if (h.bad_line != ~0ull || (lines & 3) != 0)
      return set_err(c, BRUNO_ERR_BAD_INPUT, "malformed FASTQ in file " + std::to_string(si) + " near line " +
                                                 std::to_string(h.bad_line != ~0ull ? h.bad_line : lines));
    if (c->pre_extracted) extract_reads(c, rcap, rcap + lines / 4);
    if (batch_hook && (st = batch_segment(c, si, rcap, rcap + lines / 4)) != BRUNO_OK) return st;
    rcap += lines / 4;
  }
  c->n_reads = rcap;
  return BRUNO_OK;
}

/* ------------------------------------------------------------ counting */
namespace {
double hll_estimate(const unsigned int *reg) {
  double sum = 0; int zeros = 0;
  for (int i = 0; i < HLL_M; ++i) { sum += std::ldexp(1.0, -(int)reg[i]); zeros += reg[i] == 0; }
  const double m = HLL_M, alpha = 0.7213 / (1.0 + 1.079 / m);
  double est = alpha * m * m / sum;
  if (est <= 2.5 * m && zeros > 0) est = m * std::log(m / zeros);
  return est;
}

/* k_hll_sums writes each sample's zero-register count as a 32-bit word after the sums */
unsigned zeros_word(const void *p) {
  unsigned z;
  std::memcpy(&z, p, sizeof z);
  return z;
}

/* the HyperLogLog estimate of the k-mers sampled into it (1 in 2^HLL_SAMPLE), scaled back to all */
double hll_sampled_estimate(double sum, unsigned zeros) {
  const double m = HLL_M, alpha = 0.7213 / (1.0 + 1.079 / m);
  double est = alpha * m * m / sum;
  if (est <= 2.5 * m && zeros > 0) est = m * std::log(m / zeros);
  return est * (double)(1u << HLL_SAMPLE);
}

/* node and chain lists hold 32-bit slot indices: a table is at most 2^32 - 1 slots (137 GB of
 * 32-byte slots, 275 GB of 64-byte ones) */
bruno_status table_room(Ctx *c, uint64_t slots) {
  if (slots < (1ull << 32)) return BRUNO_OK;
  return set_err(c, BRUNO_ERR_TABLE_FULL, "k-mer table would need 2^32 slots or more");
}

uint64_t slots_for(const Ctx *c, double distinct) {
  const double load = c->cfg.max_load > 0 ? c->cfg.max_load : 0.5;
  /* a k-mer with more than one slot's worth of biedges takes continuation slots */
  return (uint64_t)(distinct * 1.04 / load) + 1024;
}

/* the direct count: every instance probes the whole table (k > 31, or a degenerate input
 * whose instances crowd one hash bucket) */
template <class KT>
bruno_status count_direct(Ctx *c) {
  bruno_status st;
  const int sms = num_sms();
  const uint64_t nreads = c->n_reads;
  uint64_t slots = c->cfg.table_slots;
  cudaEventRecord(c->kev[0], c->stream);
  if (slots == 0) {
    const int hb = std::max(1, std::min<int>(sms * 8, (int)((nreads + 7) / 8)));
    if ((st = ensure(c, c->blk_cnt, (size_t)hb * HLL_M)) != BRUNO_OK) return st;
    k_hll<KT><<<hb, TPB, 0, c->stream>>>((const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, nreads, c->cfg.k,
                                         (uint8_t *)c->blk_cnt.p);
    k_hll_merge<<<HLL_M / 256, 256, 0, c->stream>>>((const uint8_t *)c->blk_cnt.p, hb, c->dctr);
    c->launches += 2;
    if ((st = sync_counters(c, true)) != BRUNO_OK) return st;
    slots = slots_for(c, hll_estimate(c->hctr->hll));
  }
  for (int attempt = 0; attempt < 4; ++attempt) {
    const size_t bytes = slots * Slot<KT>::U64 * 8;
    if ((st = table_room(c, slots)) != BRUNO_OK) return st;
    if ((st = ensure(c, c->table, bytes)) != BRUNO_OK) return st;
    c->nslots = slots;
    c->geom = TableGeom{slots, slots, 0};
    cudaEventRecord(c->kev[1], c->stream);
    k_table_init<KT><<<sms * 8, TPB, 0, c->stream>>>((uint64_t *)c->table.p, slots);
    cudaMemsetAsync(c->dctr, 0, offsetof(DevCounters, hll), c->stream);
    cudaMemsetAsync(c->dctr->big_key, 0, sizeof(c->dctr->big_key) + sizeof(c->dctr->big_cnt), c->stream);
    cudaMemsetAsync(&c->dctr->n_big, 0, 8, c->stream);
    cudaEventRecord(c->kev[2], c->stream);
    CountArgs a{(const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, nreads, c->cfg.k, (uint64_t *)c->table.p,
                c->geom, 4096u, c->dctr};
    const int grid = std::max(1, std::min<int>(sms * 8, (int)((nreads + 7) / 8)));
    k_count<KT><<<grid, TPB, 0, c->stream>>>(a);
    cudaEventRecord(c->kev[3], c->stream);
    c->launches += 2;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    if (!(c->hctr->err & DERR_TABLE_FULL)) {
      float ms[3] = {0, 0, 0};
      cudaEventElapsedTime(&ms[0], c->kev[0], c->kev[1]);
      cudaEventElapsedTime(&ms[1], c->kev[1], c->kev[2]);
      cudaEventElapsedTime(&ms[2], c->kev[2], c->kev[3]);
      for (int q = 0; q < 3; ++q) c->phase_ms[6 + q] = ms[q];
      c->n_instances = c->hctr->n_instances;
      c->n_reads_used = c->hctr->n_reads_used;
      c->n_entries = c->hctr->n_entries;
      c->n_slots_claimed = c->hctr->n_slots_claimed;
      return BRUNO_OK;
    }
    slots *= 2;  /* the estimate was too low: grow and count again */
  }
  return set_err(c, BRUNO_ERR_TABLE_FULL, "k-mer table full after regrowth");
}

/* the partitioned count (k <= 31); returns with used = false if a bucket overflowed */
/* Extraction into the hash buckets, in one launch over all reads or in one launch per FASTQ
 * segment as segments arrive: `upper` bounds the k-mer positions of all launches together and
 * `max_blocks` their blocks together; every block claims bucket chunks of its own, so chunk
 * tails waste at most max_blocks * chunk records a bucket, kept within half the margin. */
bruno_status extract_begin(Ctx *c, uint64_t upper, int max_blocks) {
  bruno_status st;
  const uint64_t cap = upper / NBUCKET + upper / (NBUCKET * 12) + 4096;  /* hashing spreads buckets within ~0.1% */
  if ((st = ensure(c, c->records, (size_t)NBUCKET * cap * 8)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->bucket_cnt, NBUCKET * 8)) != BRUNO_OK) return st;
  cudaMemsetAsync(c->bucket_cnt.p, 0, NBUCKET * 8, c->stream);
  if ((st = ensure(c, c->blk_cnt, (size_t)max_blocks * HLL_M)) != BRUNO_OK) return st;
  static const bool attr = [] {
    cudaFuncSetAttribute(k_extract<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ExtractSmem));
    return true;
  }();
  (void)attr;
  const uint64_t margin = cap - upper / NBUCKET;
  c->xcap = cap;
  c->xchunk = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(512, margin / (2ull * max_blocks)));
  c->xblk = 0;
  c->xblk_max = max_blocks;
  /* the bucket layout of the one sample (the split reads it too) */
  if ((st = ensure(c, c->xsamp, sizeof(XSample))) != BRUNO_OK) return st;
  const XSample xs{0ull, cap, c->xchunk, 0u};
  if ((st = cuda_check(c, cudaMemcpyAsync(c->xsamp.p, &xs, sizeof(xs), cudaMemcpyHostToDevice, c->stream),
                       "extraction layout")) != BRUNO_OK)
    return st;
  if (!c->cfg.edge_filter) {   /* the extraction by samples and its HyperLogLog */
    static const bool sattr = [] {
      cudaFuncSetAttribute(k_extract_s<KW1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(ExtractSmemT<KW1>));
      return true;
    }();
    (void)sattr;
    if ((st = ensure(c, c->hllreg, HLL_M * 4)) != BRUNO_OK) return st;
    cudaMemsetAsync(c->hllreg.p, 0, HLL_M * 4, c->stream);
  }
  return BRUNO_OK;
}

/* The shared-memory count of every partition of every sample (sg: per sample its table
 * geometry and first partition; caps: its bucket capacity).  Buckets are split into their
 * partitions first unless the one sample has no split bits (its buckets are the partitions).
 * ok = false when a skewed input overflowed a partition's split capacity or an entry could pass
 * 2^24 occurrences in shared memory: nothing was counted and the caller falls back. */
bruno_status split_and_count(Ctx *c, std::vector<SGeom> &sg, const std::vector<uint64_t> &caps, bool &ok,
                             unsigned long long *s_tally) {
  bruno_status st;
  ok = false;
  const uint32_t S = (uint32_t)sg.size();
  bool split = S > 1;
  for (uint32_t q = 0; q < S; ++q) split |= sg[q].g.pbits > NBUCKET_BITS;
  uint64_t r2 = 0, cap2_max = 0, region_max = 0;
  for (uint32_t q = 0; q < S; ++q) {
    const int sbits = sg[q].g.pbits - NBUCKET_BITS;
    sg[q].rec2_base = split ? r2 : 0;
    sg[q].cap2 = split ? (caps[q] >> sbits) + (caps[q] >> sbits) / 8 + 1024 : caps[q];
    r2 += (uint64_t)sg[q].cap2 << sg[q].g.pbits;
    cap2_max = std::max(cap2_max, sg[q].cap2);
    region_max = std::max<uint64_t>(region_max, sg[q].g.region);
  }
  if (cap2_max >= (1ull << 24)) return BRUNO_OK;   /* counts could pass 2^24 in shared memory */
  const uint64_t nparts = sg.back().pbase + (1ull << sg.back().g.pbits);
  if ((st = ensure(c, c->sgeom, S * sizeof(SGeom))) != BRUNO_OK) return st;
  if ((st = cuda_check(c, cudaMemcpyAsync(c->sgeom.p, sg.data(), S * sizeof(SGeom), cudaMemcpyHostToDevice, c->stream),
                       "sample geometry")) != BRUNO_OK)
    return st;
  const uint64_t *recs = (const uint64_t *)c->records.p;
  const unsigned long long *cnts = (const unsigned long long *)c->bucket_cnt.p;
  cudaEventRecord(c->kev[4], c->stream);
  if (split) {
    if ((st = ensure(c, c->records2, (size_t)(r2 * 8))) != BRUNO_OK) return st;
    if ((st = ensure(c, c->sub_cnt, (size_t)(nparts * 8))) != BRUNO_OK) return st;
    cudaMemsetAsync(c->sub_cnt.p, 0, nparts * 8, c->stream);
    /* items: pieces of every bucket, from the bucket counts */
    std::vector<unsigned long long> bc((size_t)S * NBUCKET);
    if ((st = cuda_check(c, cudaMemcpyAsync(bc.data(), c->bucket_cnt.p, bc.size() * 8, cudaMemcpyDeviceToHost,
                                            c->stream), "bucket counts")) != BRUNO_OK)
      return st;
    if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "bucket counts")) != BRUNO_OK) return st;
    constexpr uint64_t PIECE = 16ull * SPLIT_REC;
    std::vector<SplitItem> items;
    for (uint32_t gb = 0; gb < S * NBUCKET; ++gb) {
      const uint64_t n = std::min<uint64_t>(caps[gb / NBUCKET], bc[gb]);
      for (uint64_t lo = 0; lo < n; lo += PIECE) items.push_back(SplitItem{lo, std::min(n, lo + PIECE), gb, 0u});
    }
    if (!items.empty()) {
      if ((st = ensure(c, c->split_items, items.size() * sizeof(SplitItem))) != BRUNO_OK) return st;
      if ((st = cuda_check(c, cudaMemcpyAsync(c->split_items.p, items.data(), items.size() * sizeof(SplitItem),
                                              cudaMemcpyHostToDevice, c->stream), "split items")) != BRUNO_OK)
        return st;
      const int grid = (int)std::min<uint64_t>(items.size(), (uint64_t)num_sms() * 2);
      k_split<<<grid, XTPB, sizeof(SplitSmem), c->stream>>>((const uint64_t *)c->records.p,
                                                             (const XSample *)c->xsamp.p, (const SGeom *)c->sgeom.p,
                                                             (const SplitItem *)c->split_items.p, items.size(),
                                                             (uint64_t *)c->records2.p,
                                                             (unsigned long long *)c->sub_cnt.p, c->dctr);
      c->launches += 1;
    }
    cudaEventRecord(c->kev[4], c->stream);
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    if (c->hctr->err & DERR_TABLE_FULL) {   /* a skewed bucket: the caller falls back */
      cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
      return BRUNO_OK;
    }
    recs = (const uint64_t *)c->records2.p;
    cnts = (const unsigned long long *)c->sub_cnt.p;
  }
  /* thresholded builds: the count lists the slots the filter must read (at most one per slot) */
  CandArgs ca{};
  const uint64_t nslots_all = sg.back().g.base + sg.back().g.nslots;
  if (c->cfg.thresholding && !c->cfg.edge_filter && nslots_all < (1ull << 32)) {
    if ((st = ensure(c, c->cand, nslots_all * 4)) != BRUNO_OK) return st;
    ca.cand = (uint32_t *)c->cand.p;
    ca.cap = nslots_all;
    ca.n_cand = &c->dctr->n_cand;
    ca.quick_hist = c->dctr->quick_hist;
    for (int i = 0; i < 6; ++i) ca.t[i] = c->cfg.thresh[i];
    cudaMemsetAsync(&c->dctr->n_cand, 0, sizeof(c->dctr->n_cand) + sizeof(c->dctr->quick_hist), c->stream);
  }
  if (S == 1) {
    k_count_local<<<(unsigned)nparts, count_threads_for(c, region_max), (unsigned)(region_max * 32), c->stream>>>(
        recs, cnts, (const SGeom *)c->sgeom.p, S, nullptr, 0, (uint64_t *)c->table.p, s_tally, ca, c->dctr);
    c->launches += 1;
  } else {
    /* partitions grouped by region size: a launch per class, with shared memory for its largest
     * region (classes a factor of about 1.5 apart, so no region reserves much more than it uses) */
    constexpr int NCL = bruno_table_plan::REGION_CLASSES;
    std::vector<ClassRun> runs;
    std::vector<size_t> at{0};
    std::vector<uint64_t> rmax, nparts_cl;
    for (int cl = 0; cl < NCL; ++cl) {
      uint64_t m = 0, n = 0;
      for (uint32_t q = 0; q < S; ++q) {
        const uint64_t r = sg[q].g.region;
        if (bruno_table_plan::region_class(r) != cl) continue;
        runs.push_back(ClassRun{(uint32_t)n, (uint32_t)sg[q].pbase});
        n += 1ull << sg[q].g.pbits;
        m = std::max(m, r);
      }
      at.push_back(runs.size());
      rmax.push_back(m);
      nparts_cl.push_back(n);
    }
    if ((st = ensure(c, c->grp_tmp, runs.size() * sizeof(ClassRun) + 16)) != BRUNO_OK) return st;
    if ((st = cuda_check(c, cudaMemcpyAsync(c->grp_tmp.p, runs.data(), runs.size() * sizeof(ClassRun),
                                            cudaMemcpyHostToDevice, c->stream), "partition classes")) != BRUNO_OK)
      return st;
    for (int cl = 0; cl < NCL; ++cl) {
      if (!nparts_cl[cl]) continue;
      k_count_local<<<(unsigned)nparts_cl[cl], count_threads_for(c, rmax[cl]), (unsigned)(rmax[cl] * 32),
                      c->stream>>>(
          recs, cnts, (const SGeom *)c->sgeom.p, S, (const ClassRun *)c->grp_tmp.p + at[cl],
          (uint32_t)(at[cl + 1] - at[cl]), (uint64_t *)c->table.p, s_tally, ca, c->dctr);
      c->launches += 1;
    }
  }
  if ((st = cuda_check(c, cudaGetLastError(), "k_count_local")) != BRUNO_OK) return st;
  c->have_cand = ca.cand != nullptr;   /* valid once the caller sees no overflow */
  ok = true;
  return BRUNO_OK;
}

/* k <= 31 with more partitions than k_split handles: the bucket records scattered into their
 * partitions' table regions (k_split_scatter), then k_count_local reads each partition's records
 * from its own region (the sample's record base 0 and capacity four records a slot, in units of
 * slots' words) before it writes the counted region over them */
bruno_status scatter_and_count(Ctx *c, uint64_t cap) {
  bruno_status st;
  const int pb = c->geom.pbits;
  const uint64_t region = c->geom.region;
  if ((st = ensure(c, c->sub_cnt, (size_t)8 << pb)) != BRUNO_OK) return st;
  cudaMemsetAsync(c->sub_cnt.p, 0, (size_t)8 << pb, c->stream);
  const SGeom sg{c->geom, 0, 0, 4 * region};
  if ((st = ensure(c, c->sgeom, sizeof(SGeom))) != BRUNO_OK) return st;
  cudaMemcpyAsync(c->sgeom.p, &sg, sizeof(SGeom), cudaMemcpyHostToDevice, c->stream);
  CandArgs ca{};
  if (c->cfg.thresholding && !c->cfg.edge_filter) {
    if ((st = ensure(c, c->cand, c->nslots * 4)) != BRUNO_OK) return st;
    ca.cand = (uint32_t *)c->cand.p;
    ca.cap = c->nslots;
    ca.n_cand = &c->dctr->n_cand;
    ca.quick_hist = c->dctr->quick_hist;
    for (int i = 0; i < 6; ++i) ca.t[i] = c->cfg.thresh[i];
    cudaMemsetAsync(&c->dctr->n_cand, 0, sizeof(c->dctr->n_cand) + sizeof(c->dctr->quick_hist), c->stream);
  }
  launch_scatter<KW1>((const uint64_t *)c->records.p, (const unsigned long long *)c->bucket_cnt.p, cap, pb, c->geom,
                      (uint64_t *)c->table.p, (unsigned long long *)c->sub_cnt.p, c->dctr, c->stream);
  cudaEventRecord(c->kev[4], c->stream);
  k_count_local<<<(unsigned)(1ull << pb), count_threads_for(c, region), (unsigned)(region * 32), c->stream>>>(
      (const uint64_t *)c->table.p, (const unsigned long long *)c->sub_cnt.p, (const SGeom *)c->sgeom.p, 1, nullptr, 0,
      (uint64_t *)c->table.p, nullptr, ca, c->dctr);
  c->launches += 2;
  c->have_cand = ca.cand != nullptr;
  return cuda_check(c, cudaGetLastError(), "k_count_local");
}

/* after a counting pass without overflow: the listed slots and the quick drops' tallies */
void take_candidates(Ctx *c) {
  if (!c->have_cand) return;
  c->n_cand = c->hctr->n_cand;
  for (int f = 0; f < 16; ++f) c->quick_hist[f] = c->hctr->quick_hist[f];
}

/* blocks of one extraction launch over nr reads (at most 2 per SM, at least one item of WX_ITEM
 * reads each) */
constexpr uint32_t WX_ITEM = XTPB;   /* one read a thread: fine enough to even out the blocks */
int wx_blocks(uint64_t nr) {
  return (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)num_sms() * 2, (nr + WX_ITEM - 1) / WX_ITEM));
}

/* one extraction launch over reads [r0, r1) */
void extract_reads(Ctx *c, uint64_t r0, uint64_t r1) {
  const uint64_t nr = r1 - r0;
  if (nr == 0) return;
  if (!c->cfg.edge_filter) {
    const int eb = std::max(1, std::min(wx_blocks(nr), c->xblk_max - c->xblk));
    k_extract_s<KW1><<<eb, XTPB, sizeof(ExtractSmemT<KW1>), c->stream>>>(
        (const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, r0, r1, nullptr, 0, WX_ITEM, c->cfg.k,
        (const XSample *)c->xsamp.p, (uint64_t *)c->records.p, (unsigned long long *)c->bucket_cnt.p,
        (unsigned int *)c->hllreg.p, nullptr, nullptr, nullptr, 0, c->dctr);
    c->xblk += eb;
    c->launches += 1;
    return;
  }
  const int eb = std::max(1, std::min<int>({num_sms() * 2, (int)((nr + XTPB - 1) / XTPB), c->xblk_max - c->xblk}));
  const uint64_t *rs = (const uint64_t *)c->rstart.p + r0, *re = (const uint64_t *)c->rend.p + r0;
  uint8_t *part = (uint8_t *)c->blk_cnt.p + (uint64_t)c->xblk * HLL_M;
  /* the (k+1)-mer edge filter's extraction (the rest goes by samples, above) */
  k_extract<true><<<eb, XTPB, sizeof(ExtractSmem), c->stream>>>(
      rs, re, nr, c->cfg.k, (uint64_t *)c->records.p, c->xcap, (unsigned long long *)c->bucket_cnt.p, part,
      (const uint64_t *)c->k1tab.p, c->k1slots, c->xchunk, c->dctr);
  c->xblk += eb;
  c->launches += 1;
}

bruno_status count_partitioned(Ctx *c, bool &used) {
  bruno_status st;
  used = false;
  const int sms = num_sms();
  const uint64_t nreads = c->n_reads;
  if (!c->pre_extracted) {   /* the read index ran alone: one extraction launch over all reads */
    cudaMemsetAsync(c->dctr, 0, offsetof(DevCounters, hll), c->stream);
    k_kmer_upper<<<sms * 4, TPB, 0, c->stream>>>((const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, nreads,
                                                 c->cfg.k, c->dctr);
    c->launches += 1;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    if ((st = extract_begin(c, c->hctr->n_upper, c->cfg.edge_filter ? sms * 2 : wx_blocks(nreads))) != BRUNO_OK)
      return st;
    cudaEventRecord(c->kev[0], c->stream);
    extract_reads(c, 0, nreads);
  }
  const uint64_t cap = c->xcap;
  double distinct = 0;
  if (c->cfg.edge_filter) {
    k_hll_merge<<<HLL_M / 256, 256, 0, c->stream>>>((const uint8_t *)c->blk_cnt.p, c->xblk, c->dctr);
    c->launches += 1;
    cudaEventRecord(c->kev[1], c->stream);
    if ((st = sync_counters(c, true)) != BRUNO_OK) return st;
    distinct = hll_estimate(c->hctr->hll);
  } else {
    if ((st = ensure(c, c->hsum, 16)) != BRUNO_OK) return st;
    k_hll_sums<<<1, 256, 0, c->stream>>>((const unsigned int *)c->hllreg.p, (double *)c->hsum.p,
                                         (unsigned int *)((double *)c->hsum.p + 1));
    c->launches += 1;
    cudaEventRecord(c->kev[1], c->stream);
    double hs[2] = {0, 0};
    cudaMemcpyAsync(hs, c->hsum.p, 16, cudaMemcpyDeviceToHost, c->stream);
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    distinct = hll_sampled_estimate(hs[0], zeros_word(&hs[1]));
  }
  if (c->hctr->err & DERR_TABLE_FULL) return BRUNO_OK;   /* a bucket overflowed: count directly */
  c->n_instances = c->hctr->n_instances;
  c->n_reads_used = c->hctr->n_reads_used;
  uint64_t slots = c->cfg.table_slots ? c->cfg.table_slots : slots_for(c, distinct);
  static const bool part_attr = [] {
    cudaFuncSetAttribute(k_count_local, cudaFuncAttributeMaxDynamicSharedMemorySize, PART_SLOTS * 32);
    cudaFuncSetAttribute(k_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SplitSmem));
    return true;
  }();
  (void)part_attr;
  for (int attempt = 0; attempt < 4; ++attempt) {
    /* shared-memory path: 2^pb partitions (pb >= 8) small enough for one CTA's shared memory;
     * past k_split's 8 + MAX_SPLIT_BITS bits the records are scattered into the table instead */
    const bruno_table_plan::Plan plan = bruno_table_plan::partitions(slots, part_slots(c), MAX_SPLIT_BITS2);
    const int pb = plan.pbits;
    const uint64_t region_c = plan.region;
    bool counted = false, counted_local = false;
    cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
    cudaMemsetAsync(&c->dctr->n_slots_claimed, 0, 16, c->stream);
    cudaMemsetAsync(c->dctr->big_key, 0, sizeof(c->dctr->big_key) + sizeof(c->dctr->big_cnt), c->stream);
    cudaMemsetAsync(&c->dctr->n_big, 0, 8, c->stream);
    if (region_c <= part_slots(c) && c->force_direct_count != 2) {
      c->geom = TableGeom{region_c << pb, region_c, pb, 0};
      c->nslots = c->geom.nslots;
      if ((st = table_room(c, c->nslots)) != BRUNO_OK) return st;
      if ((st = ensure(c, c->table, c->nslots * 32)) != BRUNO_OK) return st;
      cudaEventRecord(c->kev[2], c->stream);
      bool ok = false;
      if (pb <= NBUCKET_BITS + MAX_SPLIT_BITS) {
        std::vector<SGeom> sg{SGeom{c->geom, 0, 0, 0}};
        if ((st = split_and_count(c, sg, std::vector<uint64_t>{cap}, ok, nullptr)) != BRUNO_OK) return st;
      } else if ((st = scatter_and_count(c, cap)) != BRUNO_OK) {
        return st;
      } else {
        ok = true;
      }
      if (ok) {
        cudaEventRecord(c->kev[3], c->stream);
        counted = counted_local = true;
      }
    }
    if (!counted) {
      /* L2 path: partitions of at most ~48 MB (a whole number of buckets) filled one at a time */
      const double bytes = (double)slots * 32.0;
      int pt = 0;
      while (pt < NBUCKET_BITS && bytes / (double)(1ull << pt) > 48.0 * 1024 * 1024) ++pt;
      const uint64_t region = std::max<uint64_t>(64, (slots + (1ull << pt) - 1) >> pt);
      c->geom = TableGeom{region << pt, region, pt, 0};
      c->nslots = c->geom.nslots;
      if ((st = table_room(c, c->nslots)) != BRUNO_OK) return st;
      if ((st = ensure(c, c->table, c->nslots * 32)) != BRUNO_OK) return st;
      cudaEventRecord(c->kev[2], c->stream);
      const int G = 1 << (NBUCKET_BITS - pt);
      static const int ins_occ = [] {   /* resident k_insert blocks per SM: one full wave per partition */
        int o = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_insert, TPB, 0) == cudaSuccess && o > 0 ? o : 4;
      }();
      const int gx = std::max(1, (sms * ins_occ + G - 1) / G);
      for (int q = 0; q < (1 << pt); ++q) {
        k_part_init<KW1><<<sms * 2, TPB, 0, c->stream>>>((uint64_t *)c->table.p, (uint64_t)q * region, region);
        k_insert<<<dim3(gx, G), TPB, 0, c->stream>>>((const uint64_t *)c->records.p,
                                                      (const unsigned long long *)c->bucket_cnt.p, cap, q * G,
                                                      (uint64_t *)c->table.p, c->geom, 4096u, c->dctr);
      }
      c->launches += 2 << pt;
      cudaEventRecord(c->kev[3], c->stream);
    }
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    if (!(c->hctr->err & DERR_TABLE_FULL)) {
      float ms[3] = {0, 0, 0};
      cudaEventElapsedTime(&ms[0], c->kev[0], c->kev[1]);   /* phase A (extract + estimate) */
      cudaEventElapsedTime(&ms[2], c->kev[2], c->kev[3]);   /* phase B (split + count, or init + insert) */
      c->phase_ms[6] = ms[0];
      c->phase_ms[7] = 0;
      c->phase_ms[8] = ms[2];
      c->phase_ms[9] = 0;
      if (counted_local) {   /* the split alone; phase B minus the split is k_count_local */
        float sp = 0;
        cudaEventElapsedTime(&sp, c->kev[2], c->kev[4]);
        c->phase_ms[9] = sp;
      }
      c->n_entries = c->hctr->n_entries;
      c->n_slots_claimed = c->hctr->n_slots_claimed;
      if (counted_local) take_candidates(c);
      else c->have_cand = false;
      used = true;
      return BRUNO_OK;
    }
    slots = std::max<uint64_t>(slots, c->nslots) * 2;   /* grow from the size actually used */
  }
  return set_err(c, BRUNO_ERR_TABLE_FULL, "k-mer table full after regrowth");
}

/* The partitioned count for k > 31: exact k-mer positions size 256 buckets of 16-byte records,
 * one extraction fills them (with the distinct estimate), and per attempt the records are
 * scattered into the table's partitions and counted in shared memory.  used = false sends the
 * caller to the direct count: a bucket overflowed, or a partition got more records than its
 * region holds at every size tried (a heavily skewed input). */
bruno_status count_partitioned_w2(Ctx *c, bool &used) {
  bruno_status st;
  used = false;
  const int sms = num_sms();
  const uint64_t nreads = c->n_reads;
  cudaMemsetAsync(c->dctr, 0, offsetof(DevCounters, hll), c->stream);
  k_kmer_upper<<<sms * 4, TPB, 0, c->stream>>>((const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, nreads,
                                               c->cfg.k, c->dctr);
  c->launches += 1;
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  const uint64_t upper = c->hctr->n_upper;
  const uint64_t cap = upper / NBUCKET + upper / (NBUCKET * 12) + 4096;
  if ((st = ensure(c, c->records, (size_t)NBUCKET * cap * 16)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->bucket_cnt, NBUCKET * 8)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->xsamp, sizeof(XSample))) != BRUNO_OK) return st;
  if ((st = ensure(c, c->hllreg, HLL_M * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->hsum, 16)) != BRUNO_OK) return st;
  cudaMemsetAsync(c->bucket_cnt.p, 0, NBUCKET * 8, c->stream);
  cudaMemsetAsync(c->hllreg.p, 0, HLL_M * 4, c->stream);
  const int eb = wx_blocks(nreads);
  const uint64_t margin = cap - upper / NBUCKET;   /* every block may hold an open chunk of every bucket */
  const XSample xs{0ull, cap, (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(512, margin / (2ull * eb))), 0u};
  cudaMemcpyAsync(c->xsamp.p, &xs, sizeof(xs), cudaMemcpyHostToDevice, c->stream);
  static const bool attr = [] {
    cudaFuncSetAttribute(k_extract_s<KW2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(ExtractSmemT<KW2>));
    cudaFuncSetAttribute(k_extract_s<KW2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(ExtractSmemT<KW2>));
    cudaFuncSetAttribute(k_count_local2, cudaFuncAttributeMaxDynamicSharedMemorySize, PART_SLOTS / 2 * 64);
    return true;
  }();
  (void)attr;
  cudaEventRecord(c->kev[0], c->stream);
  if (c->cfg.edge_filter)   /* the blocked driver's (k+1)-mer filter, table built by build_k1w_table */
    k_extract_s<KW2, true><<<eb, XTPB, sizeof(ExtractSmemT<KW2>), c->stream>>>(
        (const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, 0, nreads, nullptr, 0, WX_ITEM, c->cfg.k,
        (const XSample *)c->xsamp.p, (ulonglong2 *)c->records.p, (unsigned long long *)c->bucket_cnt.p,
        (unsigned int *)c->hllreg.p, nullptr, nullptr, (const uint64_t *)c->k1tab.p, c->k1slots, c->dctr);
  else
    k_extract_s<KW2><<<eb, XTPB, sizeof(ExtractSmemT<KW2>), c->stream>>>(
        (const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, 0, nreads, nullptr, 0, WX_ITEM, c->cfg.k,
        (const XSample *)c->xsamp.p, (ulonglong2 *)c->records.p, (unsigned long long *)c->bucket_cnt.p,
        (unsigned int *)c->hllreg.p, nullptr, nullptr, nullptr, 0, c->dctr);
  k_hll_sums<<<1, 256, 0, c->stream>>>((const unsigned int *)c->hllreg.p, (double *)c->hsum.p,
                                       (unsigned int *)((double *)c->hsum.p + 1));
  c->launches += 2;
  cudaEventRecord(c->kev[1], c->stream);
  double hs[2] = {0, 0};
  cudaMemcpyAsync(hs, c->hsum.p, 16, cudaMemcpyDeviceToHost, c->stream);
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  if (c->hctr->err & DERR_TABLE_FULL) {   /* a bucket overflowed: count directly */
    cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
    return BRUNO_OK;
  }
  c->n_instances = c->hctr->n_instances;
  c->n_reads_used = c->hctr->n_reads_used;
  uint64_t slots = c->cfg.table_slots ? c->cfg.table_slots
                                      : slots_for(c, hll_sampled_estimate(hs[0], zeros_word(&hs[1])));
  const uint64_t pmax = part_slots(c) / 2;   /* 64-byte slots: half as many in the same shared memory */
  for (int attempt = 0; attempt < 4; ++attempt) {
    const bruno_table_plan::Plan plan = bruno_table_plan::partitions(slots, pmax, MAX_SPLIT_BITS2);
    const int pb = plan.pbits;
    const uint64_t region = plan.region;
    if (!plan.fits) return BRUNO_OK;
    c->geom = TableGeom{region << pb, region, pb, 0};
    c->nslots = c->geom.nslots;
    if ((st = table_room(c, c->nslots)) != BRUNO_OK) return st;
    if ((st = ensure(c, c->table, c->nslots * 64)) != BRUNO_OK) return st;
    if ((st = ensure(c, c->sub_cnt, (size_t)8 << pb)) != BRUNO_OK) return st;
    cudaMemsetAsync(c->sub_cnt.p, 0, (size_t)8 << pb, c->stream);
    cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
    cudaMemsetAsync(&c->dctr->n_slots_claimed, 0, 16, c->stream);
    cudaMemsetAsync(&c->dctr->n_big, 0, 8, c->stream);
    CandArgs ca{};
    if (c->cfg.thresholding && !c->cfg.edge_filter) {   /* the edge filter's insert is unthresholded */
      if ((st = ensure(c, c->cand, c->nslots * 4)) != BRUNO_OK) return st;
      ca.cand = (uint32_t *)c->cand.p;
      ca.cap = c->nslots;
      ca.n_cand = &c->dctr->n_cand;
      ca.quick_hist = c->dctr->quick_hist;
      for (int i = 0; i < 6; ++i) ca.t[i] = c->cfg.thresh[i];
      cudaMemsetAsync(&c->dctr->n_cand, 0, sizeof(c->dctr->n_cand) + sizeof(c->dctr->quick_hist), c->stream);
    }
    cudaEventRecord(c->kev[2], c->stream);
    launch_scatter<KW2>((const ulonglong2 *)c->records.p, (const unsigned long long *)c->bucket_cnt.p, cap, pb,
                        c->geom, (uint64_t *)c->table.p, (unsigned long long *)c->sub_cnt.p, c->dctr, c->stream);
    cudaEventRecord(c->kev[4], c->stream);
    k_count_local2<<<(unsigned)(1ull << pb), PTPB2, (unsigned)(region * 64), c->stream>>>(
        (const unsigned long long *)c->sub_cnt.p, c->geom, (uint64_t *)c->table.p, ca, c->dctr);
    c->launches += 2;
    cudaEventRecord(c->kev[3], c->stream);
    if ((st = cuda_check(c, cudaGetLastError(), "k_count_local2")) != BRUNO_OK) return st;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    if (!(c->hctr->err & DERR_TABLE_FULL)) {
      float ms[3] = {0, 0, 0};
      cudaEventElapsedTime(&ms[0], c->kev[0], c->kev[1]);
      cudaEventElapsedTime(&ms[1], c->kev[2], c->kev[4]);
      cudaEventElapsedTime(&ms[2], c->kev[2], c->kev[3]);
      c->phase_ms[6] = ms[0];
      c->phase_ms[7] = 0;
      c->phase_ms[8] = ms[2];
      c->phase_ms[9] = ms[1];
      c->n_entries = c->hctr->n_entries;
      c->n_slots_claimed = c->hctr->n_slots_claimed;
      c->have_cand = ca.cand != nullptr;
      take_candidates(c);
      used = true;
      return BRUNO_OK;
    }
    /* a partition's records overflowed its region, or its slots filled: larger regions, and
     * the records scattered again from the buckets */
    slots = std::max<uint64_t>(slots, c->nslots) * 2;
  }
  cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
  return BRUNO_OK;
}

/* compute_edge_frequency: the (k+1)-mer table, sized from its own distinct estimate and
 * regrown if a probe run overflows, then thresholded */
bruno_status build_k1_table(Ctx *c) {
  bruno_status st;
  const int sms = num_sms();
  const uint64_t nreads = c->n_reads;
  const int hb = std::max(1, std::min<int>(sms * 4, (int)((nreads + TPB - 1) / TPB)));
  if ((st = ensure(c, c->blk_cnt, (size_t)hb * HLL_M)) != BRUNO_OK) return st;
  k_k1_hll<<<hb, TPB, 0, c->stream>>>((const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, nreads, c->cfg.k,
                                      (uint8_t *)c->blk_cnt.p);
  k_hll_merge<<<HLL_M / 256, 256, 0, c->stream>>>((const uint8_t *)c->blk_cnt.p, hb, c->dctr);
  c->launches += 2;
  if ((st = sync_counters(c, true)) != BRUNO_OK) return st;
  uint64_t slots = (uint64_t)(hll_estimate(c->hctr->hll) * 2.2) + 1024;
  const int gb = std::max(1, std::min<int>(sms * 8, (int)((nreads + TPB - 1) / TPB)));
  for (int attempt = 0; attempt < 4; ++attempt, slots *= 2) {
    if ((st = ensure(c, c->k1tab, slots * 16)) != BRUNO_OK) return st;
    c->k1slots = slots;
    k_k1_init<<<sms * 8, TPB, 0, c->stream>>>((uint64_t *)c->k1tab.p, slots);
    cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
    k_k1_count<<<gb, TPB, 0, c->stream>>>((const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, nreads, c->cfg.k,
                                          (uint64_t *)c->k1tab.p, slots, 4096u, c->dctr);
    c->launches += 2;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    if (c->hctr->err & DERR_TABLE_FULL) continue;
    const uint64_t lo = c->cfg.thresh[2], hi = c->cfg.thresh[3];
    if (lo > 0 || hi < 65536) {
      k_k1_threshold<<<sms * 8, TPB, 0, c->stream>>>((uint64_t *)c->k1tab.p, slots, lo, hi);
      c->launches += 1;
    }
    return BRUNO_OK;
  }
  return set_err(c, BRUNO_ERR_TABLE_FULL, "(k+1)-mer table full after regrowth");
}

/* build_k1_table for k > 31: (k+1)-mers of 33..64 bases, 32-byte slots */
bruno_status build_k1w_table(Ctx *c) {
  bruno_status st;
  const int sms = num_sms();
  const uint64_t nreads = c->n_reads;
  const int hb = std::max(1, std::min<int>(sms * 4, (int)((nreads + TPB - 1) / TPB)));
  if ((st = ensure(c, c->blk_cnt, (size_t)hb * HLL_M)) != BRUNO_OK) return st;
  k_k1w_hll<<<hb, TPB, 0, c->stream>>>((const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, nreads, c->cfg.k,
                                       (uint8_t *)c->blk_cnt.p);
  k_hll_merge<<<HLL_M / 256, 256, 0, c->stream>>>((const uint8_t *)c->blk_cnt.p, hb, c->dctr);
  c->launches += 2;
  if ((st = sync_counters(c, true)) != BRUNO_OK) return st;
  uint64_t slots = (uint64_t)(hll_estimate(c->hctr->hll) * 2.2) + 1024;
  const int gb = std::max(1, std::min<int>(sms * 8, (int)((nreads + TPB - 1) / TPB)));
  for (int attempt = 0; attempt < 4; ++attempt, slots *= 2) {
    if ((st = ensure(c, c->k1tab, slots * 32)) != BRUNO_OK) return st;
    c->k1slots = slots;
    k_k1w_init<<<sms * 8, TPB, 0, c->stream>>>((uint64_t *)c->k1tab.p, slots);
    cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
    k_k1w_count<<<gb, TPB, 0, c->stream>>>((const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, nreads,
                                           c->cfg.k, (uint64_t *)c->k1tab.p, slots, 4096u, c->dctr);
    c->launches += 2;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    if (c->hctr->err & DERR_TABLE_FULL) continue;
    const uint64_t lo = c->cfg.thresh[2], hi = c->cfg.thresh[3];
    if (lo > 0 || hi < 65536) {
      k_k1w_threshold<<<sms * 8, TPB, 0, c->stream>>>((uint64_t *)c->k1tab.p, slots, lo, hi);
      c->launches += 1;
    }
    return BRUNO_OK;
  }
  return set_err(c, BRUNO_ERR_TABLE_FULL, "(k+1)-mer table full after regrowth");
}

template <class KT>
bruno_status count_paths(Ctx *c) {
  if (c->cfg.edge_filter && sizeof(KT) == 16) {   /* k > 31: the 128-bit (k+1)-mer table, partitioned count */
    bruno_status st = build_k1w_table(c);
    if (st != BRUNO_OK) return st;
    bool used = false;
    if ((st = count_partitioned_w2(c, used)) != BRUNO_OK) return st;
    return used ? BRUNO_OK : set_err(c, BRUNO_ERR_TABLE_FULL, "a partition overflowed under the (k+1)-mer filter");
  }
  if (c->cfg.edge_filter) {   /* the (k+1)-mer filter works on the partitioned path (k <= 31) */
    bruno_status st = build_k1_table(c);
    if (st != BRUNO_OK) return st;
    bool used = false;
    if ((st = count_partitioned(c, used)) != BRUNO_OK) return st;
    return used ? BRUNO_OK : set_err(c, BRUNO_ERR_TABLE_FULL, "a hash bucket overflowed under the (k+1)-mer filter");
  }
  if (sizeof(KT) == 8 && c->force_direct_count != 1) {
    bool used = false;
    bruno_status st = count_partitioned(c, used);
    if (st != BRUNO_OK || used) return st;
  }
  if (sizeof(KT) == 16 && c->force_direct_count == 0) {
    bool used = false;
    bruno_status st = count_partitioned_w2(c, used);
    if (st != BRUNO_OK || used) return st;
  }
  c->have_cand = false;   /* whatever a partitioned attempt listed is stale */
  return count_direct<KT>(c);
}

/* counting, then the entries counted past 2^24 (if any) resolved for the filter */
template <class KT>
bruno_status count_typed(Ctx *c) {
  c->have_cand = false;
  bruno_status st = count_paths<KT>(c);
  if (st != BRUNO_OK) return st;
  c->n_big = c->hctr->n_big;
  if (c->n_big == 0) return BRUNO_OK;
  if ((st = ensure(c, c->bigres, BIG_SLOTS * sizeof(BigRes))) != BRUNO_OK) return st;
  cudaMemsetAsync(&c->dctr->n_big_res, 0, 8, c->stream);
  k_big_resolve<KT><<<1, 1024, 0, c->stream>>>((const uint64_t *)c->table.p, c->dctr, (BigRes *)c->bigres.p,
                                               &c->dctr->n_big_res);
  c->launches += 1;
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  c->n_big = std::min<uint64_t>(c->hctr->n_big_res, BIG_SLOTS);
  return BRUNO_OK;
}

template <class KT>
bruno_status dump_k2_typed(Ctx *c) {
  bruno_status st;
  const uint64_t n = c->n_entries;
  if ((st = ensure(c, c->k2_keys, std::max<uint64_t>(1, n) * 8 * Slot<KT>::KEYW)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->k2_edges, std::max<uint64_t>(1, n))) != BRUNO_OK) return st;
  if ((st = ensure(c, c->k2_counts, std::max<uint64_t>(1, n) * 4)) != BRUNO_OK) return st;
  cudaMemsetAsync(&c->dctr->n_k2_dump, 0, 8, c->stream);
  c->launches += 1;
  k_dump_k2<KT><<<num_sms() * 8, TPB, 0, c->stream>>>((const uint64_t *)c->table.p, c->nslots, (uint64_t *)c->k2_keys.p,
                                                       (uint8_t *)c->k2_edges.p, (uint32_t *)c->k2_counts.p, n, c->dctr);
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  c->n_k2 = std::min<uint64_t>(n, c->hctr->n_k2_dump);
  c->k2_dumped = true;
  return BRUNO_OK;
}

template <class KT>
bruno_status filter_typed(Ctx *c, const uint64_t *thr) {
  bruno_status st;
  FilterArgs a{};
  a.table = (uint64_t *)c->table.p;
  a.nslots = c->nslots;
  a.g = c->geom;
  a.k = c->cfg.k;
  for (int i = 0; i < 6; ++i) a.t[i] = thr[i];
  a.thresholding = c->cfg.thresholding && !c->cfg.edge_filter;   /* the (k+1)-mer path inserts unthresholded */
  a.max_probe = 4096u;
  a.ctr = c->dctr;
  /* every node is a chain or a branch node: lists sized by the claimed slots */
  const uint64_t cap = std::max<uint64_t>(1, c->n_slots_claimed);
  if ((st = ensure(c, c->chain_list, cap * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->branch_list, cap * 4)) != BRUNO_OK) return st;
  a.chain_list = (uint32_t *)c->chain_list.p;
  a.branch_list = (uint32_t *)c->branch_list.p;
  a.list_cap = cap;
  a.big = (const BigRes *)c->bigres.p;
  a.n_big = c->n_big;
  a.S = c->S;
  a.sg = (const SGeom *)c->sgeom.p;
  a.s_tally = c->S > 1 ? (unsigned long long *)c->s_tally.p : nullptr;
  if (c->cfg.keep_filtered) {
    const uint64_t n = std::max<uint64_t>(1, c->n_entries);
    if ((st = ensure(c, c->f_keys, n * 8 * Slot<KT>::KEYW)) != BRUNO_OK) return st;
    if ((st = ensure(c, c->f_edges, n)) != BRUNO_OK) return st;
    if ((st = ensure(c, c->f_counts, n * 4)) != BRUNO_OK) return st;
    a.f_keys = (uint64_t *)c->f_keys.p; a.f_edges = (uint8_t *)c->f_edges.p; a.f_counts = (uint32_t *)c->f_counts.p;
    a.f_cap = n;
  }
  /* the count listed the slots that need the full filter (same thresholds): read only those,
   * and add the quick drops the count tallied */
  /* (at most one listed slot a slot: a count past the table's slots would mean a lost list) */
  const bool use_cand = c->have_cand && c->n_cand <= c->nslots && a.thresholding &&
                        std::equal(thr, thr + 6, c->cfg.thresh);
  if (use_cand) {
    a.cand = (const uint32_t *)c->cand.p;
    a.n_cand = c->n_cand;
  }
  cudaMemsetAsync(c->dctr, 0, offsetof(DevCounters, hll), c->stream);
  const uint64_t chunks = ((use_cand ? c->n_cand : c->nslots) + FCHUNK - 1) / FCHUNK;
  k_filter<KT><<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)num_sms() * 8, chunks)), TPB, 0,
                 c->stream>>>(a);
  c->launches += 1;
  c->have_cand = false;   /* the listed slots are nodes or tombstones now */
  c->filter_read = use_cand ? c->n_cand : c->nslots;
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  const DevCounters &h = *c->hctr;
  c->n_nodes = h.n_nodes; c->n_branch = h.n_branch; c->n_chain = h.n_chain;
  c->n_filtered = std::min<uint64_t>(h.n_filtered, a.f_cap);
  for (int f = 0; f < 16; ++f) c->flag_hist[f] = h.flag_hist[f] + (use_cand ? c->quick_hist[f] : 0);
  return BRUNO_OK;
}
}  // namespace

namespace {
/* first read of each sample: the first read whose sequence starts at or after the sample's
 * first byte (reads are indexed in byte order) */
__global__ void k_sample_first_read(const uint64_t *rstart, uint64_t nreads, const uint64_t *samp_addr, uint32_t n,
                                    uint64_t *r0) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const uint64_t a = samp_addr[q];
    uint64_t lo = 0, hi = nreads;
    while (lo < hi) { const uint64_t m = (lo + hi) >> 1; if (rstart[m] < a) lo = m + 1; else hi = m; }
    r0[q] = lo;
  }
}

}  // namespace

/* The batched form's count: S samples, concatenated in one device copy, each counted into
 * partitions of its own in one pass of every counting kernel (the plain path's kernels; the
 * plain build is a batch of one).  Needs k <= 31 and the shared-memory partitions. */
namespace {
/* The first read of each sample q in [q0, q1), among reads [r0, r1) (every read before r0 lies
 * before sample q0, every read of these samples before r1); out gets q1 - q0 + 1 values, the
 * last r1. */
bruno_status first_reads(Ctx *c, uint32_t q0, uint32_t q1, uint64_t r0, uint64_t r1, std::vector<uint64_t> &out) {
  bruno_status st;
  const uint32_t n = q1 - q0;
  out.assign(n + 1, r1);
  if (n == 0) return BRUNO_OK;
  std::vector<uint64_t> addr(n);
  const uint64_t base = (uint64_t)(uintptr_t)c->seg_bufs[0].p;
  for (uint32_t q = 0; q < n; ++q) addr[q] = base + c->samp_off[q0 + q];
  if ((st = ensure(c, c->fr_tmp, (size_t)n * 16)) != BRUNO_OK) return st;
  uint64_t *d = (uint64_t *)c->fr_tmp.p;
  cudaMemcpyAsync(d, addr.data(), (size_t)n * 8, cudaMemcpyHostToDevice, c->stream);
  k_sample_first_read<<<(n + 255) / 256, 256, 0, c->stream>>>((const uint64_t *)c->rstart.p + r0, r1 - r0, d, n, d + n);
  c->launches += 1;
  cudaMemcpyAsync(out.data(), d + n, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream);
  if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "sample reads")) != BRUNO_OK) return st;
  for (uint32_t q = 0; q < n; ++q) out[q] += r0;
  return BRUNO_OK;
}

/* One extraction launch over samples [q0, q1) whose first reads are f (q1 - q0 + 1 values):
 * work items of WX_ITEM reads of one sample, each sample's records into its own buckets. */
bruno_status extract_samples(Ctx *c, uint32_t q0, uint32_t q1, const std::vector<uint64_t> &f) {
  bruno_status st;
  std::vector<XItem> items;
  std::vector<uint64_t> items_of(q1 - q0, 0);
  for (uint32_t q = q0; q < q1; ++q)
    for (uint64_t a = f[q - q0]; a < f[q - q0 + 1]; a += WX_ITEM) {
      items.push_back(XItem{a, std::min<uint64_t>(f[q - q0 + 1], a + WX_ITEM), q, 0u});
      ++items_of[q - q0];
    }
  if (items.empty()) return BRUNO_OK;
  const int eb = wx_blocks(f.back() - f.front());
  const uint64_t per = std::max<uint64_t>(1, items.size() / eb);   /* the fewest items a block takes */
  std::vector<XSample> xs(q1 - q0);
  for (uint32_t q = q0; q < q1; ++q) {
    const uint64_t upper = (c->samp_off[q + 1] - c->samp_off[q]) / 2 + 1;   /* k-mer positions <= bytes / 2 */
    const uint64_t touching = (items_of[q - q0] + per - 1) / per + 1;   /* blocks whose chunks can hold its records */
    const uint64_t margin = c->x_cap[q] - upper / NBUCKET;
    xs[q - q0] = XSample{c->x_base[q], c->x_cap[q],
                         (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(512, margin / (2 * touching))), 0u};
  }
  if ((st = ensure(c, c->xitems, items.size() * sizeof(XItem))) != BRUNO_OK) return st;
  cudaMemcpyAsync((XSample *)c->xsamp.p + q0, xs.data(), xs.size() * sizeof(XSample), cudaMemcpyHostToDevice,
                  c->stream);
  cudaMemcpyAsync(c->xitems.p, items.data(), items.size() * sizeof(XItem), cudaMemcpyHostToDevice, c->stream);
  k_extract_s<KW1><<<eb, XTPB, sizeof(ExtractSmemT<KW1>), c->stream>>>(
      (const uint64_t *)c->rstart.p, (const uint64_t *)c->rend.p, 0, 0, (const XItem *)c->xitems.p, items.size(),
      WX_ITEM, c->cfg.k, (const XSample *)c->xsamp.p, (uint64_t *)c->records.p,
      (unsigned long long *)c->bucket_cnt.p, (unsigned int *)c->hllreg.p, (unsigned long long *)c->s_inst.p,
      (unsigned long long *)c->s_used.p, nullptr, 0, c->dctr);
  c->launches += 1;
  return cuda_check(c, cudaGetLastError(), "k_extract_s");
}
}  // namespace

/* the read index's hook for a batch copied in groups: segment si (reads [r0, r1)) has landed */
bruno_status batch_segment(Ctx *c, size_t si, uint64_t r0, uint64_t r1) {
  std::vector<uint64_t> f;
  const uint32_t q0 = c->seg_samp[si], q1 = c->seg_samp[si + 1];
  bruno_status st = first_reads(c, q0, q1, r0, r1, f);
  return st != BRUNO_OK ? st : extract_samples(c, q0, q1, f);
}

/* The batched form's count: S samples, concatenated in one device copy, each counted into
 * partitions of its own in one pass of every counting kernel (the plain path's kernels; the
 * plain build is a batch of one).  Needs k <= 31 and the shared-memory partitions. */
bruno_status run_count_samples(Ctx *c) {
  bruno_status st;
  c->have_cand = false;
  const uint32_t S = c->S;
  const int sms = num_sms();
  /* per sample its buckets: capacities from its bytes, so they are known before any read is */
  c->x_cap.assign(S, 0);
  c->x_base.assign(S, 0);
  std::vector<uint64_t> caps(S);
  uint64_t rec_total = 0;
  for (uint32_t q = 0; q < S; ++q) {
    const uint64_t upper = (c->samp_off[q + 1] - c->samp_off[q]) / 2 + 1;   /* k-mer positions <= bytes / 2 */
    caps[q] = c->x_cap[q] = upper / NBUCKET + upper / (NBUCKET * 12) + 4096;
    c->x_base[q] = rec_total;
    rec_total += caps[q] * NBUCKET;
  }
  if ((st = ensure(c, c->records, rec_total * 8)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->bucket_cnt, (size_t)S * NBUCKET * 8)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->xsamp, S * sizeof(XSample))) != BRUNO_OK) return st;
  if ((st = ensure(c, c->hllreg, (size_t)S * HLL_M * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->s_inst, (size_t)S * 8)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->s_used, (size_t)S * 8)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->s_tally, (size_t)S * T_NUM * 8)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->hsum, (size_t)S * 16)) != BRUNO_OK) return st;
  cudaMemsetAsync(c->bucket_cnt.p, 0, (size_t)S * NBUCKET * 8, c->stream);
  cudaMemsetAsync(c->hllreg.p, 0, (size_t)S * HLL_M * 4, c->stream);
  cudaMemsetAsync(c->s_inst.p, 0, (size_t)S * 8, c->stream);
  cudaMemsetAsync(c->s_used.p, 0, (size_t)S * 8, c->stream);
  cudaMemsetAsync(c->s_tally.p, 0, (size_t)S * T_NUM * 8, c->stream);
  static const bool wattr = [] {
    cudaFuncSetAttribute(k_extract_s<KW1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(ExtractSmemT<KW1>));
    cudaFuncSetAttribute(k_count_local, cudaFuncAttributeMaxDynamicSharedMemorySize, PART_SLOTS * 32);
    cudaFuncSetAttribute(k_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SplitSmem));
    return true;
  }();
  (void)wattr;
  /* the read index (its counters reset first); a batch copied in groups extracts each group
   * as it lands (batch_segment), otherwise one launch over every sample follows */
  if (c->batch_piped) cudaEventRecord(c->kev[0], c->stream);
  if ((st = run_index_reads(c)) != BRUNO_OK) return st;
  const uint64_t nreads = c->n_reads;
  if ((st = first_reads(c, 0, S, 0, nreads, c->samp_r0)) != BRUNO_OK) return st;
  if (!c->batch_piped) {
    cudaEventRecord(c->kev[0], c->stream);
    if ((st = extract_samples(c, 0, S, c->samp_r0)) != BRUNO_OK) return st;
  }
  k_hll_sums<<<S, 256, 0, c->stream>>>((const unsigned int *)c->hllreg.p, (double *)c->hsum.p,
                                       (unsigned int *)((double *)c->hsum.p + S));
  c->launches += 1;
  cudaEventRecord(c->kev[1], c->stream);
  std::vector<double> hs(2 * S);
  cudaMemcpyAsync(hs.data(), c->hsum.p, (size_t)S * 16, cudaMemcpyDeviceToHost, c->stream);
  c->h_inst.assign(S, 0);
  c->h_used.assign(S, 0);
  cudaMemcpyAsync(c->h_inst.data(), c->s_inst.p, (size_t)S * 8, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(c->h_used.data(), c->s_used.p, (size_t)S * 8, cudaMemcpyDeviceToHost, c->stream);
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  if (c->hctr->err & DERR_TABLE_FULL)
    return set_err(c, BRUNO_ERR_TABLE_FULL, "batch: a sample's hash bucket overflowed (a skewed sample)");
  c->n_instances = c->hctr->n_instances;
  c->n_reads_used = c->hctr->n_reads_used;
  std::vector<uint64_t> slots(S);
  const unsigned char *zeros = (const unsigned char *)(hs.data() + S);   /* S 32-bit words after the sums */
  for (uint32_t q = 0; q < S; ++q) slots[q] = slots_for(c, hll_sampled_estimate(hs[q], zeros_word(zeros + 4 * q)));
  for (int attempt = 0; attempt < 4; ++attempt) {
    std::vector<SGeom> sg(S);
    uint64_t base = 0, pbase = 0;
    for (uint32_t q = 0; q < S; ++q) {
      const bruno_table_plan::Plan plan = bruno_table_plan::partitions(slots[q], part_slots(c), MAX_SPLIT_BITS);
      const int pb = plan.pbits;
      const uint64_t region = plan.region;
      if (!plan.fits)
        return set_err(c, BRUNO_ERR_ARG, "batch: sample " + std::to_string(q) + " is too large for one batch");
      sg[q].g = TableGeom{region << pb, region, pb, base};
      sg[q].pbase = pbase;
      base += region << pb;
      pbase += 1ull << pb;
    }
    c->nslots = base;
    c->geom = TableGeom{base, sg[0].g.region, sg[0].g.pbits, 0};
    if ((st = table_room(c, c->nslots)) != BRUNO_OK) return st;
    if ((st = ensure(c, c->table, c->nslots * 32)) != BRUNO_OK) return st;
    cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
    cudaMemsetAsync(&c->dctr->n_slots_claimed, 0, 16, c->stream);
    cudaMemsetAsync(c->s_tally.p, 0, (size_t)S * T_NUM * 8, c->stream);
    cudaEventRecord(c->kev[2], c->stream);
    bool ok = false;
    if ((st = split_and_count(c, sg, caps, ok, (unsigned long long *)c->s_tally.p)) != BRUNO_OK) return st;
    if (!ok) return set_err(c, BRUNO_ERR_TABLE_FULL, "batch: a partition of a skewed sample overflowed");
    cudaEventRecord(c->kev[3], c->stream);
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    if (!(c->hctr->err & DERR_TABLE_FULL)) {
      c->h_sgeom = sg;
      c->n_entries = c->hctr->n_entries;
      c->n_slots_claimed = c->hctr->n_slots_claimed;
      c->n_big = 0;
      take_candidates(c);
      float ms[3] = {0, 0, 0};
      cudaEventElapsedTime(&ms[0], c->kev[0], c->kev[1]);
      cudaEventElapsedTime(&ms[1], c->kev[2], c->kev[4]);
      cudaEventElapsedTime(&ms[2], c->kev[2], c->kev[3]);
      c->phase_ms[6] = ms[0];
      c->phase_ms[7] = 0;
      c->phase_ms[8] = ms[2];
      c->phase_ms[9] = ms[1];
      return BRUNO_OK;
    }
    for (auto &x : slots) x *= 2;   /* an estimate was too low: every sample grows, all count again */
  }
  return set_err(c, BRUNO_ERR_TABLE_FULL, "batch: k-mer table full after regrowth");
}

bruno_status run_count(Ctx *c) { return c->W == 1 ? count_typed<KW1>(c) : count_typed<KW2>(c); }
bruno_status run_dump_k2(Ctx *c) { return c->W == 1 ? dump_k2_typed<KW1>(c) : dump_k2_typed<KW2>(c); }
bruno_status run_filter(Ctx *c, const uint64_t *thresh) {
  return c->W == 1 ? filter_typed<KW1>(c, thresh) : filter_typed<KW2>(c, thresh);
}

bruno_status run_copy_nodes(Ctx *c, uint64_t *keys, uint16_t *counts, uint8_t *flags, size_t cap, size_t *n) {
  return run_copy_nodes_range(c, 0, c->nslots, c->n_nodes, keys, counts, flags, cap, n);
}

bruno_status run_copy_nodes_range(Ctx *c, uint64_t base, uint64_t nslots, uint64_t nnodes, uint64_t *keys,
                                  uint16_t *counts, uint8_t *flags, size_t cap, size_t *n) {
  bruno_status st;
  *n = nnodes;
  if (!keys && !counts && !flags) return BRUNO_OK;
  if (cap < nnodes) return set_err(c, BRUNO_ERR_CAPACITY, "node buffers too small");
  const uint64_t nn = std::max<uint64_t>(1, nnodes);
  Buf dk, dc, df;
  if ((st = ensure(c, dk, nn * 8 * c->W)) != BRUNO_OK) return st;
  if ((st = ensure(c, dc, nn * 18)) != BRUNO_OK) return st;
  if ((st = ensure(c, df, nn)) != BRUNO_OK) return st;
  cudaMemsetAsync(&c->dctr->n_k2_dump, 0, 8, c->stream);
  if (c->W == 1)
    k_dump_nodes<KW1><<<num_sms() * 8, TPB, 0, c->stream>>>((const uint64_t *)c->table.p + base * Slot<KW1>::U64, nslots,
                                                            (uint64_t *)dk.p, (uint16_t *)dc.p, (uint8_t *)df.p, nn,
                                                            &c->dctr->n_k2_dump);
  else
    k_dump_nodes<KW2><<<num_sms() * 8, TPB, 0, c->stream>>>((const uint64_t *)c->table.p + base * Slot<KW2>::U64, nslots,
                                                            (uint64_t *)dk.p, (uint16_t *)dc.p, (uint8_t *)df.p, nn,
                                                            &c->dctr->n_k2_dump);
  bruno_status r = BRUNO_OK;
  if (keys) r = cuda_check(c, cudaMemcpyAsync(keys, dk.p, nnodes * 8 * c->W, cudaMemcpyDeviceToHost, c->stream), "copy");
  if (r == BRUNO_OK && counts)
    r = cuda_check(c, cudaMemcpyAsync(counts, dc.p, nnodes * 18, cudaMemcpyDeviceToHost, c->stream), "copy");
  if (r == BRUNO_OK && flags)
    r = cuda_check(c, cudaMemcpyAsync(flags, df.p, nnodes, cudaMemcpyDeviceToHost, c->stream), "copy");
  if (r == BRUNO_OK) r = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  cudaFreeAsync(dk.p, c->stream); cudaFreeAsync(dc.p, c->stream); cudaFreeAsync(df.p, c->stream);
  return r;
}

/* ================================================================ allocation-free counting
 * bruno_count_biedges_noalloc counts (k-mer, biedge) pairs that the caller already holds in
 * device memory and allocates nothing: its hash table lives in the fixed file-scope array
 * below, whose address is looked up once per device.  Layout of the array: a 64 KiB header
 * holding a DevCounters (the call uses err, n_slots_claimed, n_entries and n_k2_dump), then
 * the table slots, 32 B each for k <= 31 and 64 B for k <= 63.  Each call sizes its table to
 * max(256, 2n) slots, so the load stays at or below one half and an empty slot always exists
 * (a pair adds at most one slot). */
constexpr size_t NOALLOC_BYTES = BRUNO_NOALLOC_SCRATCH_BYTES;
constexpr size_t NOALLOC_HDR = 64u << 10;
static_assert(sizeof(DevCounters) <= NOALLOC_HDR, "scratch header too small");
static_assert(BRUNO_NOALLOC_MAX_PAIRS_K31 == (NOALLOC_BYTES - NOALLOC_HDR) / 32 / 2, "K31 limit");
static_assert(BRUNO_NOALLOC_MAX_PAIRS_K63 == (NOALLOC_BYTES - NOALLOC_HDR) / 64 / 2, "K63 limit");
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

namespace {
/* DNA16 nibble -> 0 (none), 1..4 (A C G T); 5 for anything else */
__device__ __forceinline__ unsigned dna16_to5(unsigned nib) {
  return nib == 0 ? 0u : nib == 1 ? 1u : nib == 2 ? 2u : nib == 4 ? 3u : nib == 8 ? 4u : 5u;
}

/* the table insert of the direct counting path, fed from a pair array instead of reads */
template <class KT>
__global__ void __launch_bounds__(TPB) k_count_pairs(const uint64_t *kmers, const uint8_t *edges, uint64_t n, int k,
                                                      uint64_t *table, TableGeom g, uint32_t max_probe,
                                                      DevCounters *ctr) {
  constexpr int SU = Slot<KT>::U64, KWD = Slot<KT>::KEYW;
  /* bits above 2k in the most significant word must be clear */
  const int top_bits = KWD == 1 ? 2 * k : 2 * k - 64;
  const uint64_t top_mask = top_bits >= 64 ? 0ull : ~0ull << top_bits;
  unsigned long long slots = 0, entries = 0;
  bool bad = false, full = false;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const KT x = KOps<KT>::load(kmers + i * KWD);
    const unsigned e = edges[i];
    const unsigned in5 = dna16_to5(e >> 4), out5 = dna16_to5(e & 15u);
    if (in5 > 4 || out5 > 4 || (((const uint64_t *)&x)[KWD - 1] & top_mask)) { bad = true; continue; }
    const KT key = table_key(x);
    const uint64_t home = table_home(g, key);
    uint64_t raw[SU];
    ld_slot<SU>(table + home * SU, raw);
    if (!table_count<KT>(table, g, max_probe, key, biedge_code(in5, out5), home, raw, slots, entries, ctr)) full = true;
  }
  slots = warp_sum(slots); entries = warp_sum(entries);
  if ((threadIdx.x & 31) == 0) {
    if (slots) atomicAdd(&ctr->n_slots_claimed, slots);
    if (entries) atomicAdd(&ctr->n_entries, entries);
  }
  if (bad) atomicOr(&ctr->err, (unsigned long long)DERR_BAD_INPUT);
  if (full) atomicOr(&ctr->err, (unsigned long long)DERR_TABLE_FULL);
}

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_base[NOALLOC_MAX_DEVICES];   /* device address of the array, per device */

/* once per device, with that device current: the array's device address */
bruno_status noalloc_setup(int device, unsigned char **base) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_base[device]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return BRUNO_ERR_CUDA;
    g_noalloc_base[device] = (unsigned char *)p;
  }
  *base = g_noalloc_base[device];
  return BRUNO_OK;
}

template <class KT>
bruno_status count_pairs_noalloc(unsigned char *base, int k, const uint64_t *kmers, const uint8_t *edges, uint64_t n,
                                 uint64_t *out_kmers, uint8_t *out_edges, uint32_t *out_counts, size_t out_cap,
                                 size_t *n_out, cudaStream_t stream) {
  constexpr int SU = Slot<KT>::U64;
  DevCounters *ctr = (DevCounters *)base;
  uint64_t *table = (uint64_t *)(base + NOALLOC_HDR);
  const uint64_t nslots = std::max<uint64_t>(256, 2 * n);
  const TableGeom g{nslots, nslots, 0};
  const int sms = num_sms();
  /* what must start at zero: the counters; the slots used get EMPTY keys and zero entries */
  if (cudaMemsetAsync(ctr, 0, offsetof(DevCounters, flag_hist), stream) != cudaSuccess) return BRUNO_ERR_CUDA;
  k_table_init<KT><<<(unsigned)std::min<uint64_t>((nslots * SU + TPB - 1) / TPB, (uint64_t)sms * 8), TPB, 0, stream>>>(
      table, nslots);
  if (n)
    k_count_pairs<KT><<<(unsigned)std::min<uint64_t>((n + TPB - 1) / TPB, (uint64_t)sms * 8), TPB, 0, stream>>>(
        kmers, edges, n, k, table, g, (uint32_t)nslots, ctr);
  const bool dump = out_kmers || out_edges || out_counts;
  if (dump)
    k_dump_k2<KT><<<(unsigned)std::min<uint64_t>((nslots + TPB - 1) / TPB, (uint64_t)sms * 8), TPB, 0, stream>>>(
        table, nslots, out_kmers, out_edges, out_counts, out_cap, ctr);
  if (cudaGetLastError() != cudaSuccess) return BRUNO_ERR_CUDA;
  DevCounters h;
  if (cudaMemcpyAsync(&h, ctr, offsetof(DevCounters, flag_hist), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return BRUNO_ERR_CUDA;
  if (h.err & DERR_BAD_INPUT) return BRUNO_ERR_BAD_INPUT;
  if (h.err & DERR_TABLE_FULL) return BRUNO_ERR_TABLE_FULL;
  *n_out = dump ? h.n_k2_dump : h.n_entries;
  if (dump && h.n_k2_dump > out_cap) return BRUNO_ERR_CAPACITY;
  return BRUNO_OK;
}
}  // namespace

bruno_status count_biedges_noalloc(int32_t device, int32_t k, const uint64_t *kmers, const uint8_t *edges, size_t n,
                                   uint64_t *out_kmers, uint8_t *out_edges, uint32_t *out_counts, size_t out_cap,
                                   size_t *n_out, void *stream) {
  if (!n_out || k < 3 || k > 63 || (n && (!kmers || !edges))) return BRUNO_ERR_ARG;
  const bool dump = out_kmers || out_edges || out_counts;
  if (dump && (!out_kmers || !out_edges || !out_counts)) return BRUNO_ERR_ARG;
  *n_out = 0;
  if (n > (k <= 31 ? (size_t)BRUNO_NOALLOC_MAX_PAIRS_K31 : (size_t)BRUNO_NOALLOC_MAX_PAIRS_K63))
    return BRUNO_ERR_CAPACITY;
  int ndev = 0, prev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || cudaGetDevice(&prev) != cudaSuccess) return BRUNO_ERR_CUDA;
  if (device < 0 || device >= ndev || device >= NOALLOC_MAX_DEVICES) return BRUNO_ERR_ARG;
  if (device != prev && cudaSetDevice(device) != cudaSuccess) return BRUNO_ERR_CUDA;
  unsigned char *base = nullptr;
  bruno_status st = noalloc_setup(device, &base);
  if (st == BRUNO_OK)
    st = k <= 31 ? count_pairs_noalloc<KW1>(base, k, kmers, edges, n, out_kmers, out_edges, out_counts, out_cap,
                                            n_out, (cudaStream_t)stream)
                 : count_pairs_noalloc<KW2>(base, k, kmers, edges, n, out_kmers, out_edges, out_counts, out_cap,
                                            n_out, (cudaStream_t)stream);
  if (device != prev) cudaSetDevice(prev);
  return st;
}

}  // namespace bg

extern "C" bruno_status bruno_count_biedges_noalloc(int32_t device, int32_t k, const uint64_t *kmers,
                                                    const uint8_t *edges, size_t n, uint64_t *out_kmers,
                                                    uint8_t *out_edges, uint32_t *out_counts, size_t out_cap,
                                                    size_t *n_out, void *stream) {
  return bg::count_biedges_noalloc(device, k, kmers, edges, n, out_kmers, out_edges, out_counts, out_cap, n_out,
                                   stream);
}
