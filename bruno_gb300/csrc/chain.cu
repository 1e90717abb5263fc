/*
 * chain.cu -- graph nodes -> chain map -> list ranking -> compacted chains.
 *
 *  k_chain_init          to_simple_biedge (debruijn_chain_node.hpp:83-111) for every chain
 *                        node the filter listed: neighbours are resolved once to chain
 *                        indices (+ strand flip), so ranking never hashes k-mers again
 *  k_termini             setup_chain_termini (debruijn_chain_graph.hpp:485-596) with
 *                        terminus_update (debruijn_chain_operations.hpp:57-93)
 *  k_lr_*                list_rank_min_update / list_rank (debruijn_chain_graph.hpp:793-1310):
 *                        round-synchronous pointer jumping with the reference's update rule
 *                        chain_update (debruijn_chain_operations.hpp:107-256).  Updates that
 *                        meet at one (node, side) in a round are reduced to the one with the
 *                        largest (distance, terminal mark); for the reference's chains this
 *                        equals applying them one after another in any order.
 *  k_separate            separate_cycles(iterations) and separate_isolated (:670-777)
 *  k_fast_*              the same ranking in O(M) when the chain map is mutually consistent
 *                        (ruling set: walks between rulers, pointer jumping over rulers, a
 *                        second walk that writes every node's final state)
 *  k_ranked / k_fill     to_listranked_chain_node (debruijn_chain_operations.hpp:260-309) and
 *                        to_compressed_chains (debruijn_chain_graph.hpp:1778-1856): every
 *                        chain is one head node with distance 0 plus one base per node, so
 *                        the sequence is scattered straight to its offset, no sort.
 *  k_gen_*               the same emission for chain maps whose pointers are not mutually
 *                        consistent: groups by representative, distance histograms, ranks
 *  k_chain_summary       to_summarized_chains (debruijn_chain_graph.hpp:1876-2005), on demand
 *  k_chain_freq /        compute_freq_map and print_chain_frequencies
 *  k_chain_edges         (compact_dbg_stats.hpp:783-816, 879-1065), on demand: the chain
 *                        ends' edge counts and each chain's node-frequency summary
 */
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.cuh"

namespace bg {

namespace {

constexpr int TPB = 256;
constexpr uint32_t DM = 0x7FFFFFFFu;    /* dist_mask (debruijn_chain_node.hpp:53) */
constexpr uint32_t TM = 0x80000000u;    /* term_mask */
constexpr uint32_t NONE32 = 0xFFFFFFFFu;

__device__ __forceinline__ bool ptcn(uint32_t x) { return (x ^ TM) > TM; }       /* points_to_chain_node */
__device__ __forceinline__ bool term(uint32_t x) { return (x & DM) == 0; }       /* is_chain_terminal */

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(~0u, v, o);
  return v;
}

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

/* warp-aggregated append: returns this lane's slot in `list` (valid lanes only) */
__device__ __forceinline__ unsigned long long warp_append(bool want, unsigned long long *counter) {
  const unsigned m = __ballot_sync(~0u, want);
  if (!m) return 0;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(m));
  base = __shfl_sync(~0u, base, leader);
  return base + __popc(m & ((1u << lane) - 1));
}

/* block-aggregated append: one atomic on `counter` per block and call (all threads of the
 * block must call it together); returns this thread's slot if `want` */
__device__ __forceinline__ unsigned long long block_append(bool want, unsigned long long *counter) {
  __shared__ unsigned long long s_base;
  uint32_t total;
  const uint32_t r = block_exscan(want ? 1u : 0u, total);
  if (threadIdx.x == 0) s_base = total ? atomicAdd(counter, (unsigned long long)total) : 0ull;
  __syncthreads();
  const unsigned long long b = s_base;
  __syncthreads();   /* everyone has read s_base before a next call writes it */
  return b + r;
}

template <class KT>
__device__ __forceinline__ uint32_t slot_flags(const uint64_t *s) {
  return (uint32_t)(s[Slot<KT>::KEYW + 2] >> 16) & 0xFFFFu;
}
template <class KT>
__device__ __forceinline__ uint32_t slot_aux(const uint64_t *s) {
  return (uint32_t)(s[Slot<KT>::KEYW + 2] >> 32);
}

/* slot index of a live node with canonical key x, -1 if absent */
template <class KT>
__device__ __forceinline__ long long table_find(const uint64_t *table, const TableGeom &g, uint32_t max_probe,
                                                KT kmer) {
  constexpr int SU = Slot<KT>::U64;
  const KT bare = table_key(kmer), x = as_node(bare);
  Probe pr(g, table_home(g, bare));
  for (uint32_t p = 0; p < max_probe; ++p, pr.next()) {
    const uint64_t *s = table + pr.i * SU;
    KT key = KOps<KT>::load(s);
    if (KOps<KT>::eq(key, x)) return (long long)pr.i;
    if (Slot<KT>::KEYW == 1 ? (((uint64_t *)&key)[0] == KEY_EMPTY) : (((uint64_t *)&key)[1] == KEY_EMPTY && ((uint64_t *)&key)[0] == KEY_EMPTY))
      return -1;
  }
  return -1;
}

/* Two lookups in lockstep: both first probes are in flight together, and each probe reads
 * the whole slot (key, counters, flags, aux) in 32-byte loads.  found = slot index or -1. */
template <class KT>
__device__ __forceinline__ void table_find2(const uint64_t *table, const TableGeom &g, uint32_t max_probe,
                                            const KT *want, const bool *has, long long *found,
                                            uint64_t (*raw)[Slot<KT>::U64]) {
  constexpr int SU = Slot<KT>::U64;
  KT x[2];
  uint64_t pos[2], lo[2], hi[2];
  bool done[2];
  #pragma unroll
  for (int q = 0; q < 2; ++q) {
    found[q] = -1;
    done[q] = !has[q];
    const KT bare = table_key(want[q]);
    x[q] = as_node(bare);
    const Probe pr(g, table_home(g, bare));
    pos[q] = pr.i; lo[q] = pr.lo; hi[q] = pr.hi;
  }
  for (uint32_t p = 0; p < max_probe && !(done[0] && done[1]); ++p) {
    #pragma unroll
    for (int q = 0; q < 2; ++q)
      if (!done[q]) ld_slot<SU>(table + pos[q] * SU, raw[q]);
    #pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (done[q]) continue;
      const KT key = KOps<KT>::load(raw[q]);
      if (KOps<KT>::eq(key, x[q])) { found[q] = (long long)pos[q]; done[q] = true; }
      else if (key_is_empty(key)) done[q] = true;
      else if (++pos[q] == hi[q]) pos[q] = lo[q];
    }
  }
}

/* ================================================================ chain init */
/* chain index i (listed by the filter, which also stored i in the slot) -> its k-mer, its
 * chain-map record and its edge byte; one read of its own slot gives key and counters */
template <class KT>
__global__ void __launch_bounds__(TPB) k_chain_init(const uint64_t *table, uint64_t nslots, TableGeom g0,
                                                     const SGeom *sg, uint32_t nsamples, int k,
                                                     const uint32_t *chain_list, uint64_t M, uint64_t *ckey,
                                                     ChainState *cs, uint8_t *cedge, uint32_t *csample,
                                                     uint32_t max_probe, DevCounters *ctr) {
  constexpr int SU = Slot<KT>::U64, KWD = Slot<KT>::KEYW;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t sl = chain_list[i];
    if (sl >= nslots) {   /* a list entry that was never written: report, never dereference */
      atomicOr(&ctr->err, (unsigned long long)DERR_INVARIANT);
      sl = 0;
    }
    uint64_t own[SU];
    ld_slot<SU>(table + sl * SU, own);
    TableGeom g = g0;
    if (nsamples > 1) {   /* a batch: the node's sample (in its flags) has its own partitions */
      const uint32_t smp = (uint32_t)(own[KWD + 2] >> (16 + NF_SAMPLE_SHIFT)) & (MAX_SAMPLES - 1);
      g = sg[smp < nsamples ? smp : 0].g;
      csample[i] = smp;
    }
    const KT K = key_kmer(node_key(KOps<KT>::load(own)));
    KOps<KT>::store(ckey + i * KWD, K);
    const uint64_t *pw = own + KWD;
    int inc = -1, outc = -1;
    for (int c = 0; c < 4; ++c) {
      if ((pw[0] >> (16 * c)) & 0xFFFFu) outc = c;
      if ((pw[1] >> (16 * c)) & 0xFFFFu) inc = c;
    }
    /* in neighbour nextReverseFromChar(c), out neighbour nextFromChar(c), canonical */
    KT want[2];
    bool has[2] = {inc >= 0, outc >= 0}, flip[2] = {false, false};
    #pragma unroll
    for (int q = 0; q < 2; ++q) {
      const KT n = q == 0 ? KOps<KT>::prepend((unsigned)max(inc, 0), K, k) : KOps<KT>::append(K, (unsigned)max(outc, 0), k);
      const KT y = KOps<KT>::rc(n, k);
      flip[q] = !KOps<KT>::lt(n, y);
      want[q] = flip[q] ? y : n;
    }
    long long found[2];
    uint64_t raw[2][SU];
    table_find2<KT>(table, g, max_probe, want, has, found, raw);
    ChainState st;
    st.pad = 0;
    #pragma unroll
    for (int q = 0; q < 2; ++q) {
      uint64_t P;
      uint32_t D;
      if (!has[q]) {
        P = PF_BLANK; D = TM;
      } else {
        const uint32_t fl = (uint32_t)(raw[q][KWD + 2] >> 16) & 0xFFFFu, aux = (uint32_t)(raw[q][KWD + 2] >> 32);
        if (found[q] >= 0 && (fl & NF_CHAIN) && aux < M) P = (uint64_t)aux | (flip[q] ? PF_FLIP : 0);
        else P = PF_EXT | (q ? PF_EXTOUT : 0) | i;
        D = 1;
      }
      if (q == 0) { st.inP = P; st.inD = D; } else { st.outP = P; st.outD = D; }
    }
    cs[i] = st;
    cedge[i] = (uint8_t)((inc >= 0 ? (4 | inc) : 0) | (outc >= 0 ? (32 | (outc << 3)) : 0));
  }
}

/* neighbours of branch nodes get their facing side set to branch_neighbor (0) */
template <class KT>
__global__ void __launch_bounds__(TPB) k_termini(const uint64_t *table, TableGeom g0, const SGeom *sg,
                                                  uint32_t nsamples, int k, ChainState *cs, uint64_t M,
                                                  uint32_t max_probe, const uint32_t *branch_list, uint64_t nb) {
  constexpr int SU = Slot<KT>::U64, KWD = Slot<KT>::KEYW;
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nb; q += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t *s = table + (uint64_t)branch_list[q] * SU;
    const KT K = key_kmer(node_key(KOps<KT>::load(s)));
    const uint64_t *pw = s + KWD;
    TableGeom g = g0;
    if (nsamples > 1) {
      const uint32_t smp = (uint32_t)(pw[2] >> (16 + NF_SAMPLE_SHIFT)) & (MAX_SAMPLES - 1);
      g = sg[smp < nsamples ? smp : 0].g;
    }
    for (int c = 0; c < 4; ++c) {
      if ((pw[0] >> (16 * c)) & 0xFFFFu) {  /* out neighbour receives (branch, IN) */
        KT n = KOps<KT>::append(K, (unsigned)c, k), y = KOps<KT>::rc(n, k);
        const bool flip = !KOps<KT>::lt(n, y);
        const long long j = table_find<KT>(table, g, max_probe, flip ? y : n);
        if (j >= 0 && (slot_flags<KT>(table + j * SU) & NF_CHAIN)) {
          const uint32_t idx = slot_aux<KT>(table + j * SU);
          if (idx < M) { if (flip) cs[idx].outD = 0; else cs[idx].inD = 0; }
        }
      }
      if ((pw[1] >> (16 * c)) & 0xFFFFu) {  /* in neighbour receives (branch, OUT) */
        KT n = KOps<KT>::prepend((unsigned)c, K, k), y = KOps<KT>::rc(n, k);
        const bool flip = !KOps<KT>::lt(n, y);
        const long long j = table_find<KT>(table, g, max_probe, flip ? y : n);
        if (j >= 0 && (slot_flags<KT>(table + j * SU) & NF_CHAIN)) {
          const uint32_t idx = slot_aux<KT>(table + j * SU);
          if (idx < M) { if (flip) cs[idx].inD = 0; else cs[idx].outD = 0; }
        }
      }
    }
  }
}

/* ================================================================ list ranking */
struct Upd { uint32_t t; int side; uint64_t P; uint32_t D; };  /* side 0 = in, 1 = out */

/* The updates node x sends this round (debruijn_chain_graph.hpp:1107-1142 for min_update,
 * :857-895 otherwise), already put on the target's canonical strand as lex_less does
 * (debruijn_chain_operations.hpp:500-504).  Targets outside the chain map are dropped. */
__device__ __forceinline__ int make_updates(uint32_t x, const ChainState &st, int min_update, Upd u[2]) {
  int n = 0;
  const uint32_t l = st.inD, r = st.outD, dist = (l & DM) + (r & DM);
  const bool send_l = min_update ? ptcn(l) : !term(l);
  const bool send_r = min_update ? ptcn(r) : !term(r);
  if (send_l && !(st.inP & (PF_EXT | PF_BLANK))) {
    uint64_t P = term(r) ? (uint64_t)x : st.outP;
    int side = 1;  /* OUT */
    if (st.inP & PF_FLIP) { P ^= PF_FLIP; side = 0; }
    u[n++] = {(uint32_t)st.inP, side, P, ptcn(r) ? dist : (dist | TM)};
  }
  if (send_r && !(st.outP & (PF_EXT | PF_BLANK))) {
    uint64_t P = term(l) ? (uint64_t)x : st.inP;
    int side = 0;  /* IN */
    if (st.outP & PF_FLIP) { P ^= PF_FLIP; side = 1; }
    u[n++] = {(uint32_t)st.outP, side, P, ptcn(l) ? dist : (dist | TM)};
  }
  return n;
}
__device__ __forceinline__ unsigned long long upd_key(uint32_t x, uint32_t D) {
  const uint64_t rank = ((uint64_t)(D & DM) << 1) | (D >> 31);
  return (rank << 32) | x;
}

__global__ void __launch_bounds__(TPB) k_lr_init(const ChainState *cs, uint64_t M, uint32_t *unf, unsigned long long *n) {
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < M; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    bool u = false;
    if (i < M) u = ptcn(cs[i].inD) || ptcn(cs[i].outD);
    const unsigned long long o = warp_append(u, n);
    if (u) unf[o] = (uint32_t)i;
  }
}

__global__ void __launch_bounds__(TPB) k_lr_propose(const ChainState *cs, const uint32_t *unf, uint64_t nu, int min_update,
                                                     unsigned long long *pend, DevCounters *ctr) {
  unsigned long long multi = 0;
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nu; q += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t x = unf[q];
    const ChainState st = cs[x];
    Upd u[2];
    const int n = make_updates(x, st, min_update, u);
    for (int j = 0; j < n; ++j) {
      const unsigned long long old = atomicMax(&pend[2ull * u[j].t + u[j].side], upd_key(x, u[j].D));
      multi += old != 0;
    }
  }
  multi = warp_sum(multi);
  if ((threadIdx.x & 31) == 0 && multi) atomicAdd(&ctr->lr_multi, multi);
}

__global__ void __launch_bounds__(TPB) k_lr_commit(const ChainState *cs, const uint32_t *unf, uint64_t nu, int min_update,
                                                    unsigned long long *pend, Payload *pay) {
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nu; q += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t x = unf[q];
    const ChainState st = cs[x];
    Upd u[2];
    const int n = make_updates(x, st, min_update, u);
    for (int j = 0; j < n; ++j) {
      const uint64_t slot = 2ull * u[j].t + u[j].side;
      if (pend[slot] != upd_key(x, u[j].D)) continue;   /* another update won this side */
      const uint32_t tD = u[j].side ? cs[u[j].t].outD : cs[u[j].t].inD;
      if (ptcn(tD)) pay[slot] = Payload{u[j].P, u[j].D, 0};
      else pend[slot] = 0;                                /* chain_update ignores it */
    }
  }
}

__global__ void __launch_bounds__(TPB) k_lr_apply(ChainState *cs, const uint32_t *unf, uint64_t nu,
                                                   unsigned long long *pend, const Payload *pay, uint32_t maxd,
                                                   uint32_t *next, DevCounters *ctr) {
  unsigned long long applied = 0, cycles = 0;
  for (uint64_t q0 = (uint64_t)blockIdx.x * blockDim.x; q0 < nu; q0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t q = q0 + threadIdx.x;
    bool keep = false;
    uint32_t x = 0;
    if (q < nu) {
      x = unf[q];
      ChainState st = cs[x];
      bool dirty = false;
      for (int side = 0; side < 2; ++side) {
        const uint64_t slot = 2ull * x + side;
        if (!pend[slot]) continue;
        const Payload pl = pay[slot];
        pend[slot] = 0;
        uint32_t &D = side ? st.outD : st.inD;
        uint64_t &P = side ? st.outP : st.inP;
        const uint32_t d = pl.D & DM;
        if (ptcn(D)) {      /* chain_update: farther target replaces, equal distance re-marks */
          if (d > D) P = pl.P;
          if (d >= D) { D = pl.D; ++applied; dirty = true; }
        }
      }
      if (dirty) cs[x] = st;
      keep = ptcn(st.inD) || ptcn(st.outD);
      cycles += keep && (st.inD & DM) == maxd && (st.outD & DM) == maxd;
    }
    const unsigned long long o = warp_append(keep, &ctr->lr_remaining);
    if (keep) next[o] = x;
  }
  applied = warp_sum(applied); cycles = warp_sum(cycles);
  if ((threadIdx.x & 31) == 0) {
    if (applied) atomicAdd(&ctr->lr_applied, applied);
    if (cycles) atomicAdd(&ctr->lr_cycles, cycles);
  }
}

/* ================================================================ O(M) ranking
 * For chain maps whose pointers are mutually consistent (every chain-pointing side of a
 * node is answered by the facing side of its target), the chain map is a union of simple
 * paths and cycles and the reference's round-synchronous rule has a closed form: a side
 * at distance a > 0 from its path's end is marked in round floor(log2 a) and ends as
 * (that end node, a | term_mask); terminal sides never change; cycle nodes never finish
 * and their distances are 2^rounds when the loop stops; the loop runs
 * floor(log2(n_max - 1)) + 1 rounds for the longest path (1 if only cycles remain);
 * separate_cycles then removes exactly the cycle nodes.  list_rank and
 * list_rank_min_update reach the same state on such maps.  So the ranks are computed with
 * a ruling set: rulers (every path end plus a hashed 1/32 sample) walk to their
 * neighbouring rulers, the ruler lists are ranked by pointer jumping, and every node adds
 * its offset to its ruler's ranks. */
constexpr uint32_t RULER_SAMPLE = 32;
struct Jump { uint32_t t; uint32_t fd; uint64_t d; }; /* ruler ordinal; flip | done << 1; distance */

__device__ __forceinline__ bool side_terminal(uint32_t D) { return (D & DM) == 0; }
__device__ __forceinline__ uint64_t side_ptr(const ChainState &s, int side) { return side ? s.outP : s.inP; }
__device__ __forceinline__ uint32_t side_dist(const ChainState &s, int side) { return side ? s.outD : s.inD; }

/* Ruler selection and the local half of the consistency check (every non-terminal side is a
 * chain pointer at distance 1).  A ruler's ordinal goes into its ChainState's spare word
 * (NONE32 for other nodes), so a walk learns that it reached a ruler from the same 32-byte
 * read that gives it the next pointer.  The other half -- every chain pointer is answered by
 * the facing side of its target -- is checked by the first walk for every node it passes and
 * by the marking pass for the nodes no walk reaches. */
__global__ void __launch_bounds__(TPB) k_fast_check(ChainState *cs, uint64_t M, uint32_t *rnode, DevCounters *ctr) {
  unsigned long long bad = 0;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < M; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t v = i0 + threadIdx.x;
    bool ruler = false;
    if (v < M) {
      const ChainState st = cs[v];
      bool term_side = false;
      for (int s = 0; s < 2; ++s) {
        const uint32_t D = side_dist(st, s);
        if (side_terminal(D)) { term_side = true; continue; }
        if (D != 1 || (side_ptr(st, s) & (PF_EXT | PF_BLANK))) ++bad;
      }
      ruler = term_side || (mix64(v * 0x9e3779b97f4a7c15ull + 0x632be59bd9b4e019ull) % RULER_SAMPLE) == 0;
    }
    const unsigned long long o = block_append(ruler, &ctr->lr_remaining);
    if (v < M) cs[v].pad = ruler ? o : (uint64_t)NONE32;
    if (ruler) rnode[o] = (uint32_t)v;
  }
  bad = warp_sum(bad);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(&ctr->lr_multi, bad);
}

/* the facing side of a chain pointer's target answers it: distance 1, a chain pointer back
 * to the source with the same flip */
__device__ __forceinline__ bool answers(const ChainState &t, int facing, uint32_t src, uint32_t f) {
  const uint64_t back = side_ptr(t, facing);
  return side_dist(t, facing) == 1 && !(back & (PF_EXT | PF_BLANK)) && (uint32_t)back == src &&
         (((back & PF_FLIP) ? 1u : 0u) == f);
}

/* Walk 1: every non-terminal ruler side walks to the next ruler and records (that ruler,
 * flip parity, gap) -- the first pointer-jumping link.  A terminal side is a finished link
 * to itself.  One read per step, which also checks that the node stepped to points back; the
 * grid is one resident wave, so each thread walks several sides and the geometric walk
 * lengths average out. */
__global__ void __launch_bounds__(TPB) k_fast_walk(const ChainState *cs, const uint32_t *rnode, uint64_t R, uint64_t M,
                                                    Jump *E0, uint64_t *place, DevCounters *ctr) {
  unsigned long long bad = 0;
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 2 * R; q += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t ord = (uint32_t)(q >> 1), r = rnode[ord];
    const int s0 = (int)(q & 1);
    ChainState st = cs[r];
    if (side_terminal(side_dist(st, s0))) { E0[q] = Jump{ord, 2u, 0}; continue; }
    uint32_t flip = 0, cur = r;
    int dir = s0;
    Jump out{ord, 0u, 0};   /* unreachable in a consistent map: every walk meets a ruler */
    for (uint64_t dist = 1; dist <= M; ++dist) {
      const uint64_t P = side_ptr(st, dir);
      if (side_dist(st, dir) != 1 || (P & (PF_EXT | PF_BLANK))) { ++bad; break; }
      const uint32_t f = (P & PF_FLIP) ? 1u : 0u, nxt = (uint32_t)P;
      flip ^= f;
      dir = f ? 1 - dir : dir;   /* travel direction in the next node's frame */
      st = cs[nxt];
      if (!answers(st, 1 - dir, cur, f)) { ++bad; break; }
      cur = nxt;
      if ((uint32_t)st.pad != NONE32) { out = Jump{(uint32_t)st.pad, flip, dist}; break; }
      /* the node's place on the segment, in the slot of the direction this walk crosses it */
      if (place) place[2ull * nxt + dir] = ((uint64_t)q << 32) | (dist << 1) | flip;
    }
    E0[q] = out;
  }
  bad = warp_sum(bad);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(&ctr->lr_multi, bad);
}

__global__ void __launch_bounds__(TPB) k_fast_jump(const Jump *E, Jump *F, uint64_t R, DevCounters *ctr) {
  unsigned long long undone = 0;
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 2 * R; q += (uint64_t)gridDim.x * blockDim.x) {
    Jump e = E[q];
    if (!(e.fd & 2u)) {
      const int s = (int)(q & 1);
      const uint32_t f = e.fd & 1u;
      const Jump n = E[2ull * e.t + (f ? 1 - s : s)];   /* continue in the same travel direction */
      const uint64_t sum = e.d + n.d;   /* saturate: only ruler cycles keep growing */
      e = Jump{n.t, (f ^ (n.fd & 1u)) | (n.fd & 2u), sum > 0xFFFFFFFFFFFFull ? 0xFFFFFFFFFFFFull : sum};
    }
    undone += !(e.fd & 2u);
    F[q] = e;
  }
  undone = warp_sum(undone);
  __shared__ unsigned long long s_undone;
  if (threadIdx.x == 0) s_undone = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0 && undone) atomicAdd(&s_undone, undone);
  __syncthreads();
  if (threadIdx.x == 0 && s_undone) atomicAdd(&ctr->lr_applied, s_undone);
}

/* final state of one side: the path end in that direction, its flip, the distance */
__device__ __forceinline__ void fast_side(const uint32_t *rnode, const Jump &e, uint32_t flip, uint64_t d,
                                          uint64_t &P, uint32_t &D) {
  P = (uint64_t)rnode[e.t] | (((flip ^ (e.fd & 1u)) != 0) ? PF_FLIP : 0ull);
  D = (uint32_t)d | TM;
}

/* rulers on paths: both non-terminal sides point at their path ends */
__global__ void __launch_bounds__(TPB) k_fast_rulers(const ChainState *cs, ChainState *cs2, const uint32_t *rnode,
                                                      uint64_t R, const Jump *E) {
  for (uint64_t a = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; a < R; a += (uint64_t)gridDim.x * blockDim.x) {
    const Jump e0 = E[2 * a], e1 = E[2 * a + 1];
    if (!(e0.fd & 2u) || !(e1.fd & 2u)) continue;   /* a ruler cycle: left for the cycle pass */
    const uint32_t v = rnode[a];
    ChainState st = cs[v];
    if (!side_terminal(st.inD)) fast_side(rnode, e0, 0, e0.d, st.inP, st.inD);
    if (!side_terminal(st.outD)) fast_side(rnode, e1, 0, e1.d, st.outP, st.outD);
    cs2[v] = st;
  }
}

/* Walk 2: each segment between two rulers on a path is walked once more, from its end with
 * the smaller ordinal (from side 1 when both ends are the same ruler), and every node on it
 * gets its final state: the side facing the walk's start leads past the start ruler to the
 * end E[start side'] and the other side past the far ruler to E[start side].  The walk reads
 * the chain map and writes the final states into a second array, so no step waits behind a
 * store to the array it reads. */
__global__ void __launch_bounds__(TPB) k_fast_fill(const ChainState *cs, ChainState *cs2, const uint32_t *rnode,
                                                    uint64_t R, const Jump *E0, const Jump *E) {
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 2 * R; q += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t ord = (uint32_t)(q >> 1);
    const int s0 = (int)(q & 1);
    const Jump link = E0[q];
    if (link.fd & 2u) continue;                                   /* terminal side */
    if (!(link.t > ord || (link.t == ord && s0 == 1))) continue;  /* walked from the other end */
    const Jump ef = E[q], eb = E[q ^ 1];
    if (!(ef.fd & 2u) || !(eb.fd & 2u)) continue;                 /* a ruler cycle */
    const uint64_t Pb_t = rnode[eb.t], Pf_t = rnode[ef.t];
    ChainState st = cs[rnode[ord]];
    uint32_t flip = 0;
    int dir = s0;
    for (uint64_t j = 1; j < link.d; ++j) {
      const uint64_t P = side_ptr(st, dir);
      const uint32_t v = (uint32_t)P;
      const uint32_t f = (P & PF_FLIP) ? 1u : 0u;
      flip ^= f;
      dir = f ? 1 - dir : dir;
      st = cs[v];
      ChainState w;
      w.pad = st.pad;
      /* side 1-dir faces the walk's start ruler, side dir leads on to the far ruler */
      const uint64_t Pb = Pb_t | (((flip ^ (eb.fd & 1u)) != 0) ? PF_FLIP : 0ull);
      const uint64_t Pf = Pf_t | (((flip ^ (ef.fd & 1u)) != 0) ? PF_FLIP : 0ull);
      const uint32_t Db = (uint32_t)(j + eb.d) | TM, Df = (uint32_t)(ef.d - j) | TM;
      if (dir) { w.inP = Pb; w.inD = Db; w.outP = Pf; w.outD = Df; }
      else { w.outP = Pb; w.outD = Db; w.inP = Pf; w.inD = Df; }
      cs2[v] = w;
    }
  }
}

/* The final states in one pass over the nodes (rank_fill = 1): a node between two rulers has
 * its place recorded by both walkers of its segment (walker, steps from its ruler, flip so
 * far), in the slot of the direction each crossed it; either record gives the state k_fast_fill
 * would write (the two walkers' path ends and distances are the same ones, seen from the two
 * sides).  Rulers, nodes on ruler cycles and nodes on cycles without a ruler are left as they
 * are, as k_fast_fill leaves them. */
__global__ void __launch_bounds__(TPB) k_fast_place(const ChainState *cs, ChainState *cs2, const uint32_t *rnode,
                                                     uint64_t M, const Jump *E, const uint64_t *place) {
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < M; v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t p0 = place[2 * v], p1 = place[2 * v + 1];
    if (p0 == ~0ull && p1 == ~0ull) continue;
    const int dir = p0 != ~0ull ? 0 : 1;
    const uint64_t p = dir ? p1 : p0;
    const uint64_t q = p >> 32, j = (p >> 1) & 0x7FFFFFFFull;
    const uint32_t flip = (uint32_t)(p & 1u);
    const Jump ef = E[q], eb = E[q ^ 1];
    if (!(ef.fd & 2u) || !(eb.fd & 2u)) continue;                 /* a ruler cycle */
    ChainState w;
    w.pad = cs[v].pad;
    const uint64_t Pb = (uint64_t)rnode[eb.t] | (((flip ^ (eb.fd & 1u)) != 0) ? PF_FLIP : 0ull);
    const uint64_t Pf = (uint64_t)rnode[ef.t] | (((flip ^ (ef.fd & 1u)) != 0) ? PF_FLIP : 0ull);
    const uint32_t Db = (uint32_t)(j + eb.d) | TM, Df = (uint32_t)(ef.d - j) | TM;
    if (dir) { w.inP = Pb; w.inD = Db; w.outP = Pf; w.outD = Df; }
    else { w.outP = Pb; w.outD = Db; w.inP = Pf; w.inD = Df; }
    cs2[v] = w;
  }
}

/* removed[] (1 = cycle: the node got no final state, 2 = isolated: both sides terminal), the
 * counts, and the longest path in nodes.  cs2 starts as all ones, which no final state is. */
constexpr uint32_t CS2_UNSET = 0xFFFFFFFFu;
__global__ void __launch_bounds__(TPB) k_fast_mark(const ChainState *cs, const ChainState *cs2, uint64_t M,
                                                    uint8_t *removed, unsigned long long *nmax,
                                                    const uint32_t *csample, unsigned long long *s_tally,
                                                    DevCounters *ctr) {
  unsigned long long ncy = 0, niso = 0, mx = 0, bad = 0;
  const int lane = threadIdx.x & 31;
  for (uint64_t v0 = (uint64_t)blockIdx.x * blockDim.x; v0 < M; v0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t v = v0 + threadIdx.x;
    uint32_t cyc_v = 0, iso_v = 0, mx_v = 0;
    if (v < M) {
      const ChainState st = cs2[v];
      const bool cyc = st.inD == CS2_UNSET;
      uint8_t r = 0;
      if (cyc) {
        r = 1; cyc_v = 1;
        /* no walk reached this node: check its pointers here (consistent only on a cycle) */
        const ChainState o = cs[v];
        for (int s = 0; s < 2; ++s) {
          const uint32_t D = side_dist(o, s);
          const uint64_t P = side_ptr(o, s);
          if (side_terminal(D)) continue;
          if (D != 1 || (P & (PF_EXT | PF_BLANK))) { ++bad; continue; }
          const uint32_t f = (P & PF_FLIP) ? 1u : 0u;
          if (!answers(cs[(uint32_t)P], f ? s : 1 - s, (uint32_t)v, f)) ++bad;
        }
      } else {
        mx_v = 1u + (st.inD & DM) + (st.outD & DM);
        if (st.inD == TM && st.outD == TM) { r = 2; iso_v = 1; }
      }
      removed[v] = r;
      ncy += cyc_v; niso += iso_v; mx = max(mx, (unsigned long long)mx_v);
    }
    if (s_tally) {   /* a batch: the same tallies per sample, summed over the lanes of one sample */
      const uint32_t smp = v < M ? csample[v] : ~0u;
      const unsigned peers = __match_any_sync(~0u, smp);
      const uint32_t sc = __reduce_add_sync(peers, cyc_v), si = __reduce_add_sync(peers, iso_v);
      const uint32_t sm = __reduce_max_sync(peers, mx_v);
      if (v < M && lane == __ffs(peers) - 1) {
        if (sc) atomicAdd(&s_tally[(uint64_t)smp * T_NUM + T_CYCLE], (unsigned long long)sc);
        if (si) atomicAdd(&s_tally[(uint64_t)smp * T_NUM + T_ISOLATED], (unsigned long long)si);
        if (sm) atomicMax(&s_tally[(uint64_t)smp * T_NUM + T_NMAX], (unsigned long long)sm);
      }
    }
  }
  ncy = warp_sum(ncy); niso = warp_sum(niso); bad = warp_sum(bad);
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_down_sync(~0u, mx, o));
  /* one global atomic per counter and block: per-warp ones on the same words serialised */
  __shared__ unsigned long long s_ncy, s_niso, s_bad, s_mx;
  if (threadIdx.x == 0) { s_ncy = 0; s_niso = 0; s_bad = 0; s_mx = 0; }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    if (bad) atomicAdd(&s_bad, bad);
    if (ncy) atomicAdd(&s_ncy, ncy);
    if (niso) atomicAdd(&s_niso, niso);
    if (mx) atomicMax(&s_mx, mx);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_bad) atomicAdd(&ctr->lr_multi, s_bad);
    if (s_ncy) atomicAdd(&ctr->n_cycle, s_ncy);
    if (s_niso) atomicAdd(&ctr->n_isolated, s_niso);
    if (s_mx) atomicMax(nmax, s_mx);
  }
}

/* separate_cycles(iterations) when anything is unfinished, then separate_isolated */
__global__ void __launch_bounds__(TPB) k_separate(const ChainState *cs, uint64_t M, int any_unfinished, uint32_t maxd,
                                                   uint8_t *removed, DevCounters *ctr) {
  unsigned long long ncy = 0, niso = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (uint64_t)gridDim.x * blockDim.x) {
    const ChainState st = cs[i];
    uint8_t r = 0;
    if (any_unfinished && (st.inD & DM) == maxd && (st.outD & DM) == maxd) { r = 1; ++ncy; }
    else if (st.inD == TM && st.outD == TM) { r = 2; ++niso; }
    removed[i] = r;
  }
  ncy = warp_sum(ncy); niso = warp_sum(niso);
  if ((threadIdx.x & 31) == 0) {
    if (ncy) atomicAdd(&ctr->n_cycle, ncy);
    if (niso) atomicAdd(&ctr->n_isolated, niso);
  }
}

/* ================================================================ emission */
template <class KT>
__device__ __forceinline__ KT ptr_kmer(uint64_t P, const uint64_t *ckey, const uint8_t *cedge, int k) {
  constexpr int KWD = KOps<KT>::WORDS;
  const uint32_t o = (uint32_t)P;
  KT base = KOps<KT>::load(ckey + (uint64_t)o * KWD);
  if (P & PF_EXT) {
    const uint8_t e = cedge[o];
    base = (P & PF_EXTOUT) ? KOps<KT>::append(base, (e >> 3) & 3u, k) : KOps<KT>::prepend(e & 3u, base, k);
  }
  return (P & PF_FLIP) ? KOps<KT>::rc(base, k) : base;
}

struct EmitArgs {
  const uint64_t *ckey;
  const uint8_t *cedge;
  const ChainState *cs;
  const uint8_t *removed;
  uint64_t M;
  int k;
  uint64_t *rK, *rrep;
  int32_t *rdist;
  uint32_t *rep_idx;   /* per chain node: chain index of its representative, NONE32 if external */
  int32_t *dist_of;    /* per chain node: rank distance */
  uint32_t *head_of;   /* per chain node: chain ordinal if it is a head */
  uint32_t *heads;     /* per chain ordinal: head node */
  uint64_t *head_len;  /* per chain ordinal: k - 1 + nodes */
  uint64_t *ch_rep;
  const uint32_t *csample;   /* a batch: per chain node its sample; then per listranked node and */
  uint32_t *r_samp, *h_samp; /* per chain (head) their sample */
  DevCounters *ctr;
};

template <class KT>
__global__ void __launch_bounds__(TPB) k_ranked(EmitArgs a) {
  constexpr int KWD = KOps<KT>::WORDS;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < a.M; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    const bool live = i < a.M && a.removed[i] == 0;
    KT K{}, rep{};
    int32_t dist = 0;
    bool head = false;
    if (live) {
      const ChainState st = a.cs[i];
      const KT key = KOps<KT>::load(a.ckey + i * KWD);
      const KT L = term(st.inD) ? key : ptr_kmer<KT>(st.inP, a.ckey, a.cedge, a.k);
      const KT R = KOps<KT>::rc(term(st.outD) ? key : ptr_kmer<KT>(st.outP, a.ckey, a.cedge, a.k), a.k);
      const bool sense = KOps<KT>::le(L, R);
      K = sense ? key : KOps<KT>::rc(key, a.k);
      rep = sense ? L : R;
      dist = (int32_t)(sense ? (st.inD & DM) : (st.outD & DM));
      const uint32_t sd = sense ? st.inD : st.outD;
      const uint64_t sp = sense ? st.inP : st.outP;
      a.rep_idx[i] = term(sd) ? (uint32_t)i : ((sp & (PF_EXT | PF_BLANK)) ? NONE32 : (uint32_t)sp);
      a.dist_of[i] = dist;
      head = dist == 0;
    }
    const unsigned long long o = block_append(live, &a.ctr->n_ranked);
    if (live) {
      KOps<KT>::store(a.rK + o * KWD, K);
      KOps<KT>::store(a.rrep + o * KWD, rep);
      a.rdist[o] = dist;
      if (a.csample) a.r_samp[o] = a.csample[i];
    }
    const unsigned long long h = warp_append(head, &a.ctr->n_heads);
    if (i < a.M) a.head_of[i] = head ? (uint32_t)h : NONE32;
    if (head) {
      const ChainState st = a.cs[i];
      a.heads[h] = (uint32_t)i;
      a.head_len[h] = (uint64_t)(a.k - 1) + (st.inD & DM) + (st.outD & DM) + 1;
      KOps<KT>::store(a.ch_rep + h * KWD, rep);
      if (a.csample) a.h_samp[h] = a.csample[i];
    }
  }
}

template <class KT>
__global__ void __launch_bounds__(TPB) k_fill(EmitArgs a, const uint64_t *ch_off, char *chars) {
  constexpr int KWD = KOps<KT>::WORDS;
  const char ACGT[4] = {'A', 'C', 'G', 'T'};
  bool bad = false;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.M; i += (uint64_t)gridDim.x * blockDim.x) {
    if (a.removed[i]) continue;
    const uint32_t ri = a.rep_idx[i];
    const uint32_t h = (ri == NONE32) ? NONE32 : a.head_of[ri];
    if (h == NONE32) { bad = true; continue; }
    const uint64_t off = ch_off[h], len = ch_off[h + 1] - off;
    const int32_t d = a.dist_of[i];
    const ChainState st = a.cs[i];
    const KT key = KOps<KT>::load(a.ckey + i * KWD);
    const KT L = term(st.inD) ? key : ptr_kmer<KT>(st.inP, a.ckey, a.cedge, a.k);
    const KT R = KOps<KT>::rc(term(st.outD) ? key : ptr_kmer<KT>(st.outP, a.ckey, a.cedge, a.k), a.k);
    const bool sense = KOps<KT>::le(L, R);
    const KT K = sense ? key : KOps<KT>::rc(key, a.k);
    if (d == 0) {   /* the representative itself: all k bases */
      for (int q = 0; q < a.k; ++q) chars[off + q] = ACGT[KOps<KT>::base_lsb(K, a.k - 1 - q)];
    } else {        /* one base per node: the last base of K on the representative's strand */
      const uint64_t pos = (uint64_t)(a.k - 1) + (uint64_t)d;
      if (pos >= len) { bad = true; continue; }
      chars[off + pos] = ACGT[KOps<KT>::last(K)];
    }
  }
  if (bad) atomicOr(&a.ctr->err, (unsigned long long)DERR_UNCLEAN_CHAINS);
}

/* every chain position was written: no character stayed zero (the buffer starts zeroed).
 * With every write inside its chain (k_fill checks that), the positions are then covered, and
 * they are covered once exactly when the live nodes are as many as the positions -- one per
 * chain for the representative's k bases plus one per further base -- which the host checks:
 * n_ranked == n_chain_chars - n_chains * (k - 1). */
__global__ void k_check_chains(const char *chars, uint64_t nchars, DevCounters *ctr) {
  bool bad = false;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nchars; i += (uint64_t)gridDim.x * blockDim.x)
    if (chars[i] == 0) bad = true;
  if (__any_sync(~0u, bad) && (threadIdx.x & 31) == 0) atomicOr(&ctr->err, (unsigned long long)DERR_UNCLEAN_CHAINS);
}

/* ================================================================ general emission
 * When the chain pointers are not mutually consistent (a filter with separate k and k+2 bounds
 * can trim an edge on one side only), a representative can be a k-mer outside the chain map,
 * a group can hold no distance-0 node, and several chains can share one representative.
 * to_compressed_chains (debruijn_chain_graph.hpp:1778-1856) still groups the listranked nodes
 * by representative, orders each group by (|distance|, K) (chain_rep_less,
 * debruijn_chain_operations.hpp:332-340) and prints the representative for a distance-0 node
 * and K's last base for every other one (print_chain_as_fasta, :359-384).  These kernels do
 * the same without a sort: group ids (the heads' groups first, then a hash on the
 * representative k-mer), a histogram per group over distances whose scans give every
 * (group, distance) bucket its character offset, and a rank by K inside a bucket. */
constexpr uint32_t GID_OWNER = 0x80000000u;   /* gid holds the index of the group's first node */

template <class KT>
__device__ __forceinline__ void node_ranked(const EmitArgs &a, uint64_t i, KT &K, KT &rep, int32_t &dist) {
  constexpr int KWD = KOps<KT>::WORDS;
  const ChainState st = a.cs[i];
  const KT key = KOps<KT>::load(a.ckey + i * KWD);
  const KT L = term(st.inD) ? key : ptr_kmer<KT>(st.inP, a.ckey, a.cedge, a.k);
  const KT R = KOps<KT>::rc(term(st.outD) ? key : ptr_kmer<KT>(st.outP, a.ckey, a.cedge, a.k), a.k);
  const bool sense = KOps<KT>::le(L, R);
  K = sense ? key : KOps<KT>::rc(key, a.k);
  rep = sense ? L : R;
  dist = (int32_t)(sense ? (st.inD & DM) : (st.outD & DM));
}

/* group of every live node: its head's group when the head's representative is its own,
 * otherwise the first node that claimed its representative in the hash table */
template <class KT>
__global__ void __launch_bounds__(TPB) k_gen_group(EmitArgs a, const uint64_t *ch_rep, uint32_t *gid, uint32_t *gtab,
                                                    uint64_t tmask) {
  constexpr int KWD = KOps<KT>::WORDS;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.M; i += (uint64_t)gridDim.x * blockDim.x) {
    if (a.removed[i]) continue;
    KT K, rep;
    int32_t d;
    node_ranked<KT>(a, i, K, rep, d);
    const uint32_t t = a.rep_idx[i];
    const uint32_t h = t == NONE32 ? NONE32 : a.head_of[t];
    if (h != NONE32 && KOps<KT>::eq(KOps<KT>::load(ch_rep + (uint64_t)h * KWD), rep)) { gid[i] = h; continue; }
    uint64_t s = KOps<KT>::hash(rep) & tmask;
    uint32_t owner = (uint32_t)i;
    for (uint64_t p = 0; p <= tmask; ++p, s = (s + 1) & tmask) {
      uint32_t o = gtab[s];
      if (o == 0) {
        o = atomicCAS(gtab + s, 0u, (uint32_t)i + 1);
        if (o == 0) break;                     /* claimed: this node owns the group */
      }
      KT Ko, repo;
      int32_t dd;
      node_ranked<KT>(a, o - 1, Ko, repo, dd);
      if (KOps<KT>::eq(repo, rep)) { owner = o - 1; break; }
    }
    gid[i] = GID_OWNER | owner;
  }
}

/* owners take the next group ids (after the heads' groups) and write their representative */
template <class KT>
__global__ void __launch_bounds__(TPB) k_gen_owner(EmitArgs a, uint32_t *gid, uint32_t *own_gid, uint64_t base,
                                                    uint64_t *ch_rep, unsigned long long *n_new) {
  constexpr int KWD = KOps<KT>::WORDS;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < a.M; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    const bool own = i < a.M && a.removed[i] == 0 && gid[i] == (GID_OWNER | (uint32_t)i);
    const unsigned long long o = warp_append(own, n_new);
    if (!own) continue;
    own_gid[i] = (uint32_t)(base + o);
    KT K, rep;
    int32_t d;
    node_ranked<KT>(a, i, K, rep, d);
    KOps<KT>::store(ch_rep + (base + o) * KWD, rep);
  }
}

/* final group ids; the largest distance of every group */
__global__ void __launch_bounds__(TPB) k_gen_resolve(const uint8_t *removed, const int32_t *dist_of, uint64_t M,
                                                      uint32_t *gid, const uint32_t *own_gid, uint32_t *gmax) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (uint64_t)gridDim.x * blockDim.x) {
    if (removed[i]) continue;
    uint32_t g = gid[i];
    if (g & GID_OWNER) g = own_gid[g & ~GID_OWNER];
    gid[i] = g;
    atomicMax(gmax + g, (uint32_t)abs(dist_of[i]));
  }
}

__global__ void k_gen_binlen(const uint32_t *gmax, uint64_t G, uint64_t *hlen) {
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < G; g += (uint64_t)gridDim.x * blockDim.x)
    hlen[g] = (uint64_t)gmax[g] + 1;
}

/* (group, distance) bins: node counts and character counts (k for distance 0, else 1) */
__global__ void __launch_bounds__(TPB) k_gen_hist(const uint8_t *removed, const int32_t *dist_of, uint64_t M, int k,
                                                   const uint32_t *gid, const uint64_t *hoff, uint64_t *ncnt,
                                                   uint64_t *wcnt) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (uint64_t)gridDim.x * blockDim.x) {
    if (removed[i]) continue;
    const uint32_t d = (uint32_t)abs(dist_of[i]);
    const uint64_t x = hoff[gid[i]] + d;
    atomicAdd((unsigned long long *)(ncnt + x), 1ull);
    atomicAdd((unsigned long long *)(wcnt + x), d == 0 ? (unsigned long long)k : 1ull);
  }
}

__global__ void __launch_bounds__(TPB) k_gen_place(const uint8_t *removed, const int32_t *dist_of, uint64_t M,
                                                    const uint32_t *gid, const uint64_t *hoff, const uint64_t *noff,
                                                    uint32_t *cur, uint32_t *members) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (uint64_t)gridDim.x * blockDim.x) {
    if (removed[i]) continue;
    const uint64_t x = hoff[gid[i]] + (uint32_t)abs(dist_of[i]);
    members[noff[x] + atomicAdd(cur + x, 1u)] = (uint32_t)i;
  }
}

/* every node's characters: its bin's offset plus its rank by K among the bin's nodes */
template <class KT>
__global__ void __launch_bounds__(TPB) k_gen_fill(EmitArgs a, const uint32_t *gid, const uint64_t *hoff,
                                                   const uint64_t *noff, const uint64_t *woff, const uint32_t *members,
                                                   char *chars) {
  const char ACGT[4] = {'A', 'C', 'G', 'T'};
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.M; i += (uint64_t)gridDim.x * blockDim.x) {
    if (a.removed[i]) continue;
    KT K, rep;
    int32_t d;
    node_ranked<KT>(a, i, K, rep, d);
    const uint32_t ad = (uint32_t)abs(d);
    const uint64_t x = hoff[gid[i]] + ad;
    uint64_t rank = 0;
    for (uint64_t q = noff[x]; q < noff[x + 1]; ++q) {
      const uint32_t j = members[q];
      if (j == (uint32_t)i) continue;
      KT Kj, rj;
      int32_t dj;
      node_ranked<KT>(a, j, Kj, rj, dj);
      if (KOps<KT>::lt(Kj, K)) ++rank;
    }
    if (ad == 0) {
      const uint64_t pos = woff[x] + rank * (uint64_t)a.k;
      for (int q = 0; q < a.k; ++q) chars[pos + q] = ACGT[KOps<KT>::base_lsb(rep, a.k - 1 - q)];
    } else {
      chars[woff[x] + rank] = ACGT[KOps<KT>::last(K)];
    }
  }
}

__global__ void k_gen_offsets(const uint64_t *hoff, const uint64_t *woff, uint64_t G, uint64_t total,
                              uint64_t *ch_off) {
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g <= G; g += (uint64_t)gridDim.x * blockDim.x)
    ch_off[g] = g < G ? woff[hoff[g]] : total;
}

/* ================================================================ chain summaries
 * to_summarized_chains (debruijn_chain_graph.hpp:1876-2005) on a consistent chain map: every
 * chain's head (distance 0, its representative) is the 5' terminus and the node its far side
 * points to (itself for a one-node chain) the 3' terminus; read on the representative's
 * strand they give (prev at 5', 5', 3', next at 3', distance, 5' flag, 3' flag) as
 * make_summarized_chain and transform::reverse_complement build them
 * (debruijn_chain_node.hpp:201-268).  A missing neighbour reads as the all-A Kmer(). */
template <class KT>
__device__ __forceinline__ KT side_kmer(uint64_t P, const EmitArgs &a) {
  return (P & PF_BLANK) ? KT{} : ptr_kmer<KT>(P, a.ckey, a.cedge, a.k);
}

template <class KT>
__global__ void __launch_bounds__(TPB) k_chain_summary(EmitArgs a, const uint32_t *heads, uint64_t nh, uint64_t *kmers,
                                                        uint32_t *dist, uint8_t *flags, DevCounters *ctr) {
  constexpr int KWD = KOps<KT>::WORDS;
  bool bad = false;
  for (uint64_t h = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t H = heads[h];
    if (H >= a.M) { bad = true; continue; }
    const ChainState st = a.cs[H];
    const KT key = KOps<KT>::load(a.ckey + (uint64_t)H * KWD);
    const KT L = term(st.inD) ? key : ptr_kmer<KT>(st.inP, a.ckey, a.cedge, a.k);
    const KT R = KOps<KT>::rc(term(st.outD) ? key : ptr_kmer<KT>(st.outP, a.ckey, a.cedge, a.k), a.k);
    const bool sense = KOps<KT>::le(L, R);
    const KT rep = sense ? L : R;
    const uint64_t P5 = sense ? st.inP : st.outP, Pf = sense ? st.outP : st.inP;
    const uint32_t D5 = sense ? st.inD : st.outD, Df = sense ? st.outD : st.inD;
    const KT s5 = side_kmer<KT>(P5, a);
    const KT prev = sense ? s5 : KOps<KT>::rc(s5, a.k);
    ChainState tt = st;
    KT keyT = key;
    bool senseT = sense;
    if (!term(Df)) {   /* the far side points to the 3' terminus */
      const uint32_t T = (uint32_t)Pf;
      if ((Pf & (PF_EXT | PF_BLANK)) || T >= a.M) { bad = true; continue; }
      tt = a.cs[T];
      keyT = KOps<KT>::load(a.ckey + (uint64_t)T * KWD);
      const KT LT = term(tt.inD) ? keyT : ptr_kmer<KT>(tt.inP, a.ckey, a.cedge, a.k);
      const KT RT = KOps<KT>::rc(term(tt.outD) ? keyT : ptr_kmer<KT>(tt.outP, a.ckey, a.cedge, a.k), a.k);
      senseT = KOps<KT>::le(LT, RT);
      if (!KOps<KT>::eq(senseT ? LT : RT, rep)) { bad = true; continue; }
    }
    const uint64_t P3 = senseT ? tt.outP : tt.inP;
    const uint32_t D3 = senseT ? tt.outD : tt.inD;
    if (!term(D3)) { bad = true; continue; }
    const KT s3 = side_kmer<KT>(P3, a);
    const KT next = senseT ? s3 : KOps<KT>::rc(s3, a.k);
    const KT K3 = senseT ? keyT : KOps<KT>::rc(keyT, a.k);
    uint64_t *o = kmers + h * 4 * KWD;
    KOps<KT>::store(o, prev);
    KOps<KT>::store(o + KWD, rep);
    KOps<KT>::store(o + 2 * KWD, K3);
    KOps<KT>::store(o + 3 * KWD, next);
    dist[h] = (st.inD & DM) + (st.outD & DM);
    flags[2 * h] = D5 == TM ? 0 : 1;
    flags[2 * h + 1] = D3 == TM ? 0 : 1;
  }
  if (bad) atomicOr(&ctr->err, (unsigned long long)DERR_UNCLEAN_CHAINS);
}

/* ================================================================ chain end edges */
/* compute_freq_map (compact_dbg_stats.hpp:783-816) per chain-map node: every listranked node
 * adds its self frequency (count, sum, min, max; freq_summary, debruijn_chain_operations.hpp:
 * 447-459) under the canonical k-mer of its representative.  That k-mer is the chain-map node
 * rep_idx names; a representative reached through an external pointer is looked up in the
 * table, and one that is no chain node is dropped, since only chain-map nodes' summaries are
 * ever read. */
template <class KT>
__global__ void __launch_bounds__(TPB) k_chain_freq(EmitArgs a, const uint64_t *table, TableGeom g, uint32_t max_probe,
                                                     const uint32_t *chain_list, unsigned long long *sum,
                                                     uint32_t *cnt, uint32_t *mn, uint32_t *mx) {
  constexpr int SU = Slot<KT>::U64, KWD = KOps<KT>::WORDS;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.M; i += (uint64_t)gridDim.x * blockDim.x) {
    if (a.removed[i]) continue;
    uint32_t t = a.rep_idx[i];
    if (t == NONE32) {
      const ChainState st = a.cs[i];
      const KT key = KOps<KT>::load(a.ckey + i * KWD);
      const KT L = term(st.inD) ? key : ptr_kmer<KT>(st.inP, a.ckey, a.cedge, a.k);
      const KT R = KOps<KT>::rc(term(st.outD) ? key : ptr_kmer<KT>(st.outP, a.ckey, a.cedge, a.k), a.k);
      const KT rep = KOps<KT>::le(L, R) ? L : R, y = KOps<KT>::rc(rep, a.k);
      const long long j = table_find<KT>(table, g, max_probe, KOps<KT>::le(rep, y) ? rep : y);
      if (j < 0 || !(slot_flags<KT>(table + j * SU) & NF_CHAIN)) continue;
      t = slot_aux<KT>(table + j * SU);
      if (t >= a.M) continue;
    }
    const uint32_t f = (uint32_t)(table[(uint64_t)chain_list[i] * SU + KWD + 2] & 0xFFFFu);
    atomicAdd(&sum[t], (unsigned long long)f);
    atomicAdd(&cnt[t], 1u);
    atomicMin(&mn[t], f);
    atomicMax(&mx[t], f);
  }
}

/* print_chain_frequencies (compact_dbg_stats.hpp:879-1065): one record per chain-map node that
 * IsCanonicalTerminusOrIsolated (debruijn_chain_filters.hpp:125-147) accepts.  L and R are the
 * chain's ends on one strand (:947-962); L's in-edges (A C G T) come from the canonical k-mer's
 * in-counters, or its out-counters T G C A when L is not canonical, and R's out-edges the other
 * way round (:973-1007); the summary is the one of canonical(L), which is this node, with the
 * mean (float)sum / (float)count truncated to the count type (:1009-1013).  An R that is not a
 * graph node (only in chains whose pointers are not mutually consistent) gets zero counts. */
template <class KT>
__global__ void __launch_bounds__(TPB) k_chain_edges(EmitArgs a, const uint64_t *table, TableGeom g, uint32_t max_probe,
                                                      const uint32_t *chain_list, const unsigned long long *sum,
                                                      const uint32_t *cnt, const uint32_t *mn, const uint32_t *mx,
                                                      uint64_t *ends, uint16_t *freqs, unsigned long long *n_out) {
  constexpr int SU = Slot<KT>::U64, KWD = KOps<KT>::WORDS;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < a.M; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    bool sel = false;
    KT L{}, R{};
    if (i < a.M && a.removed[i] == 0) {
      const ChainState st = a.cs[i];
      const KT K = KOps<KT>::load(a.ckey + i * KWD);
      const bool ti = term(st.inD), to = term(st.outD);
      if (ti && to) {
        sel = true; L = K; R = K;
      } else if (ti) {
        const KT o = ptr_kmer<KT>(st.outP, a.ckey, a.cedge, a.k);
        sel = KOps<KT>::le(K, KOps<KT>::rc(o, a.k)); L = K; R = o;
      } else if (to) {
        const KT in = ptr_kmer<KT>(st.inP, a.ckey, a.cedge, a.k), rk = KOps<KT>::rc(K, a.k);
        sel = KOps<KT>::lt(rk, in); L = rk; R = KOps<KT>::rc(in, a.k);
      }
    }
    const unsigned long long o = warp_append(sel, n_out);
    if (!sel) continue;
    uint16_t f[11];
    const uint64_t *pl = table + (uint64_t)chain_list[i] * SU + KWD;   /* canonical(L) is this node */
    const bool lc = KOps<KT>::le(L, KOps<KT>::rc(L, a.k));
    for (int b = 0; b < 4; ++b) f[b] = lc ? (uint16_t)(pl[1] >> (16 * b)) : (uint16_t)(pl[0] >> (16 * (3 - b)));
    const KT yR = KOps<KT>::rc(R, a.k);
    const bool rcn = KOps<KT>::le(R, yR);
    const long long j = table_find<KT>(table, g, max_probe, rcn ? R : yR);
    for (int b = 0; b < 4; ++b) {
      if (j < 0) { f[4 + b] = 0; continue; }
      const uint64_t *pr = table + (uint64_t)j * SU + KWD;
      f[4 + b] = rcn ? (uint16_t)(pr[0] >> (16 * b)) : (uint16_t)(pr[1] >> (16 * (3 - b)));
    }
    const uint32_t c = cnt[i];
    f[8] = c ? (uint16_t)__float2uint_rz(__fdiv_rn(__ull2float_rn(sum[i]), __ull2float_rn((unsigned long long)c))) : 0;
    f[9] = c ? (uint16_t)mn[i] : 0;
    f[10] = c ? (uint16_t)mx[i] : 0;
    KOps<KT>::store(ends + o * 2 * KWD, L);
    KOps<KT>::store(ends + o * 2 * KWD + KWD, R);
    for (int q = 0; q < 11; ++q) freqs[o * 11 + q] = f[q];
  }
}

int sms_count() {
  static const int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  return sms;
}

template <class KT>
bruno_status extract_typed(Ctx *c) {
  bruno_status st;
  const uint64_t M = c->n_chain, Mb = std::max<uint64_t>(1, M);
  const int KWD = Slot<KT>::KEYW;
  if ((st = ensure(c, c->ckey, Mb * 8 * KWD)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->cedge, Mb)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->cstate, Mb * sizeof(ChainState))) != BRUNO_OK) return st;
  const int sms = sms_count();
  cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
  if (c->S > 1 && (st = ensure(c, c->csample, Mb * 4)) != BRUNO_OK) return st;
  k_chain_init<KT><<<sms * 8, TPB, 0, c->stream>>>((const uint64_t *)c->table.p, c->nslots, c->geom,
                                                   (const SGeom *)c->sgeom.p, c->S, c->cfg.k,
                                                   (const uint32_t *)c->chain_list.p, M, (uint64_t *)c->ckey.p,
                                                   (ChainState *)c->cstate.p, (uint8_t *)c->cedge.p,
                                                   (uint32_t *)c->csample.p, 4096u, c->dctr);
  if (c->n_branch)
    k_termini<KT><<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>(sms * 8, (c->n_branch + TPB - 1) / TPB)), TPB, 0,
                    c->stream>>>((const uint64_t *)c->table.p, c->geom, (const SGeom *)c->sgeom.p, c->S, c->cfg.k,
                                 (ChainState *)c->cstate.p, M, 4096u, (const uint32_t *)c->branch_list.p, c->n_branch);
  c->launches += 2;
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  if (c->hctr->err & DERR_INVARIANT) return set_err(c, BRUNO_ERR_INVARIANT, "chain list incomplete");
  return BRUNO_OK;
}

/* the general emission over every live node (run when the scatter's check failed) */
template <class KT>
bruno_status general_emission(Ctx *c, EmitArgs a) {
  bruno_status st;
  const uint64_t M = c->n_chain, Mb = std::max<uint64_t>(1, M);
  const int sms = sms_count();
  uint64_t T = 64;
  while (T < 2 * Mb) T <<= 1;
  Buf bgid, bown, btab, bgmax, bhoff, bn, bw, bcur, bmem;
  auto release = [&] {
    for (Buf *b : {&bgid, &bown, &btab, &bgmax, &bhoff, &bn, &bw, &bcur, &bmem})
      if (b->p) cudaFreeAsync(b->p, c->stream);
  };
  if ((st = ensure(c, bgid, Mb * 4)) != BRUNO_OK || (st = ensure(c, bown, Mb * 4)) != BRUNO_OK ||
      (st = ensure(c, btab, T * 4)) != BRUNO_OK || (st = ensure(c, bgmax, Mb * 4)) != BRUNO_OK) {
    release();
    return st;
  }
  uint32_t *gid = (uint32_t *)bgid.p, *own = (uint32_t *)bown.p, *gmax = (uint32_t *)bgmax.p;
  const int32_t *dist_of = a.dist_of;
  cudaMemsetAsync(btab.p, 0, T * 4, c->stream);
  cudaMemsetAsync(gmax, 0, Mb * 4, c->stream);
  cudaMemsetAsync(&c->dctr->n_groups, 0, 16, c->stream);
  k_gen_group<KT><<<sms * 8, TPB, 0, c->stream>>>(a, (const uint64_t *)c->ch_rep.p, gid, (uint32_t *)btab.p, T - 1);
  k_gen_owner<KT><<<sms * 8, TPB, 0, c->stream>>>(a, gid, own, c->n_heads, (uint64_t *)c->ch_rep.p,
                                                  &c->dctr->n_groups);
  k_gen_resolve<<<sms * 8, TPB, 0, c->stream>>>(a.removed, dist_of, M, gid, own, gmax);
  c->launches += 3;
  if ((st = sync_counters(c)) != BRUNO_OK) { release(); return st; }
  const uint64_t G = c->n_heads + c->hctr->n_groups;
  if ((st = ensure(c, bhoff, (G + 1) * 8)) != BRUNO_OK) { release(); return st; }
  uint64_t *hoff = (uint64_t *)bhoff.p;
  cudaMemsetAsync(hoff + G, 0, 8, c->stream);
  k_gen_binlen<<<sms * 2, TPB, 0, c->stream>>>(gmax, G, hoff);
  c->launches += 1;
  if ((st = scan_ctx(c, hoff, hoff, G + 1, &c->dctr->n_hist)) != BRUNO_OK) { release(); return st; }
  if ((st = sync_counters(c)) != BRUNO_OK) { release(); return st; }
  const uint64_t H = c->hctr->n_hist;
  if ((st = ensure(c, bn, (H + 1) * 8)) != BRUNO_OK || (st = ensure(c, bw, (H + 1) * 8)) != BRUNO_OK ||
      (st = ensure(c, bcur, std::max<uint64_t>(1, H) * 4)) != BRUNO_OK || (st = ensure(c, bmem, Mb * 4)) != BRUNO_OK) {
    release();
    return st;
  }
  uint64_t *noff = (uint64_t *)bn.p, *woff = (uint64_t *)bw.p;
  cudaMemsetAsync(noff, 0, (H + 1) * 8, c->stream);
  cudaMemsetAsync(woff, 0, (H + 1) * 8, c->stream);
  cudaMemsetAsync(bcur.p, 0, std::max<uint64_t>(1, H) * 4, c->stream);
  k_gen_hist<<<sms * 8, TPB, 0, c->stream>>>(a.removed, dist_of, M, c->cfg.k, gid, hoff, noff, woff);
  if ((st = scan_ctx(c, noff, noff, H + 1, nullptr)) != BRUNO_OK ||
      (st = scan_ctx(c, woff, woff, H + 1, &c->dctr->n_chain_chars)) != BRUNO_OK) {
    release();
    return st;
  }
  k_gen_place<<<sms * 8, TPB, 0, c->stream>>>(a.removed, dist_of, M, gid, hoff, noff, (uint32_t *)bcur.p,
                                              (uint32_t *)bmem.p);
  c->launches += 2;   /* k_gen_hist, k_gen_place */
  if ((st = sync_counters(c)) != BRUNO_OK) { release(); return st; }
  const uint64_t total = c->hctr->n_chain_chars;
  if ((st = ensure(c, c->ch_chars, std::max<uint64_t>(1, total))) != BRUNO_OK) { release(); return st; }
  k_gen_fill<KT><<<sms * 8, TPB, 0, c->stream>>>(a, gid, hoff, noff, woff, (const uint32_t *)bmem.p,
                                                 (char *)c->ch_chars.p);
  k_gen_offsets<<<sms * 2, TPB, 0, c->stream>>>(hoff, woff, G, total, (uint64_t *)c->head_off.p);
  c->launches += 2;
  st = sync_counters(c);
  release();
  if (st != BRUNO_OK) return st;
  c->n_heads = G;
  c->n_chain_chars = total;
  c->chains_clean = true;
  c->general_emission = true;
  return BRUNO_OK;
}

/* ================================================================ batch grouping
 * A batch's listranked nodes and chains are grouped by sample (a counting sort on the sample
 * of each), so that each sample's results are one contiguous range; the order inside a sample
 * is arbitrary, as the table order is in the plain build. */
__global__ void __launch_bounds__(TPB) k_samp_hist(const uint32_t *samp, uint64_t n, unsigned long long *hist) {
  const int lane = threadIdx.x & 31;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    const uint32_t s = i < n ? samp[i] : ~0u;
    const unsigned peers = __match_any_sync(~0u, s);
    if (i < n && lane == __ffs(peers) - 1) atomicAdd(&hist[s], (unsigned long long)__popc(peers));
  }
}

/* a place in its sample's range for every lane: the lanes of one warp with the same sample take
 * consecutive places with one atomic on the sample's cursor (neighbouring elements mostly share
 * a sample, and per-element atomics on one cursor serialise) */
__device__ __forceinline__ unsigned long long group_place(uint32_t s, bool valid, unsigned long long *cursor) {
  const int lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(~0u, valid ? s : ~0u);
  const int leader = __ffs(peers) - 1;
  unsigned long long base = 0;
  if (valid && lane == leader) base = atomicAdd(&cursor[s], (unsigned long long)__popc(peers));
  base = __shfl_sync(~0u, base, leader);
  return base + __popc(peers & ((1u << lane) - 1));
}

/* listranked nodes to their sample's range (cursor: the range starts, advanced as they fill) */
template <class KT>
__global__ void __launch_bounds__(TPB) k_group_ranked(const uint32_t *samp, uint64_t n, unsigned long long *cursor,
                                                       const uint64_t *K, const uint64_t *rep, const int32_t *dist,
                                                       uint64_t *K2, uint64_t *rep2, int32_t *dist2) {
  constexpr int KWD = KOps<KT>::WORDS;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    const bool valid = i < n;
    const unsigned long long o = group_place(valid ? samp[i] : 0u, valid, cursor);
    if (!valid) continue;
    KOps<KT>::store(K2 + o * KWD, KOps<KT>::load(K + i * KWD));
    KOps<KT>::store(rep2 + o * KWD, KOps<KT>::load(rep + i * KWD));
    dist2[o] = dist[i];
  }
}

/* chains (heads) to their sample's range; head_of follows its head to the new ordinal */
template <class KT>
__global__ void __launch_bounds__(TPB) k_group_heads(const uint32_t *samp, uint64_t nh, unsigned long long *cursor,
                                                      const uint32_t *heads, const uint64_t *len, const uint64_t *rep,
                                                      uint32_t *heads2, uint64_t *len2, uint64_t *rep2,
                                                      uint32_t *head_of) {
  constexpr int KWD = KOps<KT>::WORDS;
  for (uint64_t h0 = (uint64_t)blockIdx.x * blockDim.x; h0 < nh; h0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t h = h0 + threadIdx.x;
    const bool valid = h < nh;
    const unsigned long long o = group_place(valid ? samp[h] : 0u, valid, cursor);
    if (!valid) continue;
    heads2[o] = heads[h];
    len2[o] = len[h];
    KOps<KT>::store(rep2 + o * KWD, KOps<KT>::load(rep + h * KWD));
    head_of[heads[h]] = (uint32_t)o;
  }
}

/* the counting sort's ranges: per sample the count, and the exclusive scan as start (host) */
bruno_status sample_ranges(Ctx *c, const uint32_t *samp, uint64_t n, std::vector<uint64_t> &start,
                           unsigned long long **cursor) {
  bruno_status st;
  const uint32_t S = c->S;
  if ((st = ensure(c, c->grp_tmp, (size_t)S * 8)) != BRUNO_OK) return st;
  cudaMemsetAsync(c->grp_tmp.p, 0, (size_t)S * 8, c->stream);
  if (n)
    k_samp_hist<<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms_count() * 8, (n + TPB - 1) / TPB)), TPB,
                  0, c->stream>>>(samp, n, (unsigned long long *)c->grp_tmp.p);
  std::vector<unsigned long long> hist(S);
  st = cuda_check(c, cudaMemcpyAsync(hist.data(), c->grp_tmp.p, (size_t)S * 8, cudaMemcpyDeviceToHost, c->stream), "hist");
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamSynchronize(c->stream), "hist");
  if (st != BRUNO_OK) return st;
  start.assign(S + 1, 0);
  for (uint32_t q = 0; q < S; ++q) start[q + 1] = start[q] + hist[q];
  st = cuda_check(c, cudaMemcpyAsync(c->grp_tmp.p, start.data(), (size_t)S * 8, cudaMemcpyHostToDevice, c->stream),
                  "cursors");
  *cursor = (unsigned long long *)c->grp_tmp.p;
  c->launches += 1;
  return st;
}

/* both groupings, between k_ranked and the chain offsets */
template <class KT>
bruno_status group_by_sample(Ctx *c) {
  bruno_status st;
  const uint64_t n = c->n_ranked, nh = c->n_heads, nb = std::max<uint64_t>(1, n), hb = std::max<uint64_t>(1, nh);
  const int KWD = KOps<KT>::WORDS;
  const unsigned g = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms_count() * 8, (n + TPB - 1) / TPB));
  unsigned long long *cursor = nullptr;
  /* listranked nodes */
  if ((st = sample_ranges(c, (const uint32_t *)c->r_samp.p, n, c->h_rank0, &cursor)) != BRUNO_OK) return st;
  Buf K2, R2, D2;
  if ((st = ensure(c, K2, nb * 8 * KWD)) != BRUNO_OK) return st;
  if ((st = ensure(c, R2, nb * 8 * KWD)) != BRUNO_OK) return st;
  if ((st = ensure(c, D2, nb * 4)) != BRUNO_OK) return st;
  if (n)
    k_group_ranked<KT><<<g, TPB, 0, c->stream>>>((const uint32_t *)c->r_samp.p, n, cursor, (const uint64_t *)c->r_K.p,
                                                 (const uint64_t *)c->r_rep.p, (const int32_t *)c->r_dist.p,
                                                 (uint64_t *)K2.p, (uint64_t *)R2.p, (int32_t *)D2.p);
  std::swap(c->r_K, K2); std::swap(c->r_rep, R2); std::swap(c->r_dist, D2);
  cudaFreeAsync(K2.p, c->stream); cudaFreeAsync(R2.p, c->stream); cudaFreeAsync(D2.p, c->stream);
  /* chains */
  if ((st = sample_ranges(c, (const uint32_t *)c->h_samp.p, nh, c->h_head0, &cursor)) != BRUNO_OK) return st;
  Buf H2, L2, P2;
  if ((st = ensure(c, H2, hb * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, L2, (hb + 1) * 8)) != BRUNO_OK) return st;
  if ((st = ensure(c, P2, hb * 8 * KWD)) != BRUNO_OK) return st;
  const unsigned gh = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms_count() * 8, (nh + TPB - 1) / TPB));
  if (nh)
    k_group_heads<KT><<<gh, TPB, 0, c->stream>>>((const uint32_t *)c->h_samp.p, nh, cursor, (const uint32_t *)c->heads.p,
                                                 (const uint64_t *)c->head_len.p, (const uint64_t *)c->ch_rep.p,
                                                 (uint32_t *)H2.p, (uint64_t *)L2.p, (uint64_t *)P2.p,
                                                 (uint32_t *)c->head_of.p);
  std::swap(c->heads, H2); std::swap(c->head_len, L2); std::swap(c->ch_rep, P2);
  cudaFreeAsync(H2.p, c->stream); cudaFreeAsync(L2.p, c->stream); cudaFreeAsync(P2.p, c->stream);
  c->launches += 2;
  return BRUNO_OK;
}

template <class KT>
bruno_status compress_typed(Ctx *c) {
  bruno_status st;
  const uint64_t M = c->n_chain, Mb = std::max<uint64_t>(1, M);
  const int KWD = Slot<KT>::KEYW;
  if ((st = ensure(c, c->r_K, Mb * 8 * KWD)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->r_rep, Mb * 8 * KWD)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->r_dist, Mb * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->rep_idx, Mb * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->head_of, Mb * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->heads, Mb * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->head_len, (Mb + 1) * 8)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->head_off, (Mb + 1) * 8)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->ch_rep, Mb * 8 * KWD)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->pay, Mb * 8)) != BRUNO_OK) return st;   /* reused: dist_of */
  cudaMemsetAsync(&c->dctr->n_ranked, 0, 8, c->stream);
  cudaMemsetAsync(&c->dctr->n_heads, 0, 8, c->stream);
  cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
  EmitArgs a{};
  a.ckey = (const uint64_t *)c->ckey.p; a.cedge = (const uint8_t *)c->cedge.p; a.cs = (const ChainState *)c->cstate.p;
  a.removed = (const uint8_t *)c->removed.p; a.M = M; a.k = c->cfg.k;
  a.rK = (uint64_t *)c->r_K.p; a.rrep = (uint64_t *)c->r_rep.p; a.rdist = (int32_t *)c->r_dist.p;
  a.rep_idx = (uint32_t *)c->rep_idx.p; a.dist_of = (int32_t *)c->pay.p; a.head_of = (uint32_t *)c->head_of.p;
  a.heads = (uint32_t *)c->heads.p; a.head_len = (uint64_t *)c->head_len.p; a.ch_rep = (uint64_t *)c->ch_rep.p;
  a.ctr = c->dctr;
  if (c->S > 1) {   /* a batch: the sample of every listranked node and chain */
    if ((st = ensure(c, c->r_samp, Mb * 4)) != BRUNO_OK) return st;
    if ((st = ensure(c, c->h_samp, Mb * 4)) != BRUNO_OK) return st;
    a.csample = (const uint32_t *)c->csample.p;
    a.r_samp = (uint32_t *)c->r_samp.p;
    a.h_samp = (uint32_t *)c->h_samp.p;
  }
  const int sms = sms_count();
  k_ranked<KT><<<sms * 8, TPB, 0, c->stream>>>(a);
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  c->n_ranked = c->hctr->n_ranked;
  c->n_heads = c->hctr->n_heads;
  const uint64_t nh = c->n_heads;
  if (c->S > 1) {
    if ((st = group_by_sample<KT>(c)) != BRUNO_OK) return st;
    a.rK = (uint64_t *)c->r_K.p; a.rrep = (uint64_t *)c->r_rep.p; a.rdist = (int32_t *)c->r_dist.p;
    a.heads = (uint32_t *)c->heads.p; a.head_len = (uint64_t *)c->head_len.p; a.ch_rep = (uint64_t *)c->ch_rep.p;
  }
  /* offsets: exclusive scan of per-chain lengths, total into n_chain_chars */
  cudaMemsetAsync((uint64_t *)c->head_len.p + nh, 0, 8, c->stream);
  if ((st = scan_ctx(c, (const uint64_t *)c->head_len.p, (uint64_t *)c->head_off.p, nh + 1,
                     &c->dctr->n_chain_chars)) != BRUNO_OK)
    return st;
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  c->n_chain_chars = c->hctr->n_chain_chars;
  if ((st = ensure(c, c->ch_chars, std::max<uint64_t>(1, c->n_chain_chars))) != BRUNO_OK) return st;
  cudaMemsetAsync(c->ch_chars.p, 0, c->n_chain_chars, c->stream);
  k_fill<KT><<<sms * 8, TPB, 0, c->stream>>>(a, (const uint64_t *)c->head_off.p, (char *)c->ch_chars.p);
  c->launches += 3;  /* k_ranked, k_fill, k_check_chains (the scan counts its own) */
  k_check_chains<<<sms * 4, TPB, 0, c->stream>>>((const char *)c->ch_chars.p, c->n_chain_chars, c->dctr);
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  c->chains_clean = !(c->hctr->err & DERR_UNCLEAN_CHAINS) &&
                    c->n_ranked + nh * (uint64_t)(c->cfg.k - 1) == c->n_chain_chars;
  if (!c->chains_clean) return general_emission<KT>(c, a);
  return BRUNO_OK;
}

template <class KT>
bruno_status chain_summaries_typed(Ctx *c) {
  bruno_status st;
  if (c->general_emission)
    return set_err(c, BRUNO_ERR_INVARIANT,
                   "chain summaries need mutually consistent chain pointers (the reference's pairing of "
                   "termini is order-dependent otherwise)");
  const uint64_t nh = c->n_heads, nb = std::max<uint64_t>(1, nh);
  const int KWD = Slot<KT>::KEYW;
  if ((st = ensure(c, c->s_kmers, nb * 4 * 8 * KWD)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->s_dist, nb * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->s_flags, nb * 2)) != BRUNO_OK) return st;
  cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
  EmitArgs a{};
  a.ckey = (const uint64_t *)c->ckey.p; a.cedge = (const uint8_t *)c->cedge.p; a.cs = (const ChainState *)c->cstate.p;
  a.removed = (const uint8_t *)c->removed.p; a.M = c->n_chain; a.k = c->cfg.k;
  const int sms = sms_count();
  k_chain_summary<KT><<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>(sms * 8, (nh + TPB - 1) / TPB)), TPB, 0,
                        c->stream>>>(a, (const uint32_t *)c->heads.p, nh, (uint64_t *)c->s_kmers.p,
                                     (uint32_t *)c->s_dist.p, (uint8_t *)c->s_flags.p, c->dctr);
  c->launches += 1;
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  if (c->hctr->err & DERR_UNCLEAN_CHAINS)
    return set_err(c, BRUNO_ERR_INVARIANT, "a chain's termini do not pair up");
  c->n_summaries = nh;
  c->summaries_done = true;
  return BRUNO_OK;
}

template <class KT>
bruno_status chain_edges_typed(Ctx *c) {
  bruno_status st;
  const uint64_t M = c->n_chain, Mb = std::max<uint64_t>(1, M);
  const int KWD = Slot<KT>::KEYW;
  if ((st = ensure(c, c->e_ends, Mb * 2 * 8 * KWD)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->e_freqs, Mb * 11 * 2)) != BRUNO_OK) return st;
  Buf acc;   /* per chain-map node: sum (u64), then count, min, max (u32) */
  if ((st = ensure(c, acc, Mb * 20)) != BRUNO_OK) return st;
  unsigned long long *sum = (unsigned long long *)acc.p;
  uint32_t *cnt = (uint32_t *)(sum + Mb), *mn = cnt + Mb, *mx = mn + Mb;
  cudaMemsetAsync(sum, 0, Mb * 12, c->stream);   /* sum and count */
  cudaMemsetAsync(mn, 0xFF, Mb * 4, c->stream);
  cudaMemsetAsync(mx, 0, Mb * 4, c->stream);
  cudaMemsetAsync(&c->dctr->n_chain_edges, 0, 8, c->stream);
  EmitArgs a{};
  a.ckey = (const uint64_t *)c->ckey.p; a.cedge = (const uint8_t *)c->cedge.p; a.cs = (const ChainState *)c->cstate.p;
  a.removed = (const uint8_t *)c->removed.p; a.M = M; a.k = c->cfg.k;
  a.rep_idx = (uint32_t *)c->rep_idx.p;
  const int sms = sms_count();
  const uint64_t *table = (const uint64_t *)c->table.p;
  const uint32_t *cl = (const uint32_t *)c->chain_list.p;
  k_chain_freq<KT><<<sms * 8, TPB, 0, c->stream>>>(a, table, c->geom, 4096u, cl, sum, cnt, mn, mx);
  k_chain_edges<KT><<<sms * 8, TPB, 0, c->stream>>>(a, table, c->geom, 4096u, cl, sum, cnt, mn, mx,
                                                    (uint64_t *)c->e_ends.p, (uint16_t *)c->e_freqs.p,
                                                    &c->dctr->n_chain_edges);
  c->launches += 2;
  st = sync_counters(c);
  cudaFreeAsync(acc.p, c->stream);
  if (st != BRUNO_OK) return st;
  c->n_chain_edges = c->hctr->n_chain_edges;
  c->chain_edges_done = true;
  return BRUNO_OK;
}


/* ================================================================ graph cleaning
 * clean_deadend_and_bubbles_naive (compact_dbg_clean.hpp:575-890) on the device, one rank:
 * dead ends and bubbles are read off summaries weighted by the node table, their low-frequency
 * end edges are erased on both nodes, edge-less nodes leave the graph, the nodes are classified
 * again and the chain map is rebuilt and ranked, until no dead end or bubble is left. */

/* summarized_chain<K, uint16> (debruijn_chain_node.hpp:174): prev at 5', 5' terminus (the
 * chain representative), 3' terminus, next at 3', distance between the termini, the 5' and 3'
 * end-edge frequencies; plus the chain node the record was made from */
template <class KT>
struct FSum { KT k0, k1, k2, k3; uint32_t len; uint16_t f5, f6; uint32_t node, pad; };

/* an erase query or a found edge: k-mer (low word first) and a DNA16 biedge */
struct EraseQ { uint64_t w[2]; uint32_t edge, pad; };

/* the bubble grouping table: chains with one 5' branch k-mer (key + 1; 0 = empty) */
struct BubbleEnt { unsigned long long key; unsigned int cnt; unsigned int idx[8]; unsigned int pad; };

template <class KT>
__device__ __forceinline__ int kcmp(KT a, KT b) { return KOps<KT>::lt(a, b) ? -1 : (KOps<KT>::eq(a, b) ? 0 : 1); }

/* the summaries' order: the reference's sort keys (5' terminus, next at 3'), then the rest of
 * the record, as the oracle breaks the reference's ties */
template <class KT>
__device__ __forceinline__ int sum_cmp(const FSum<KT> &a, const FSum<KT> &b) {
  int c;
  if ((c = kcmp(a.k1, b.k1)) != 0) return c;
  if ((c = kcmp(a.k3, b.k3)) != 0) return c;
  if ((c = kcmp(a.k0, b.k0)) != 0) return c;
  if ((c = kcmp(a.k2, b.k2)) != 0) return c;
  if (a.f5 != b.f5) return a.f5 < b.f5 ? -1 : 1;
  if (a.f6 != b.f6) return a.f6 < b.f6 ? -1 : 1;
  return 0;
}

/* the bubbles' order: (5' branch, 3' branch, length), then the termini */
template <class KT>
__device__ __forceinline__ bool bubble_less(const FSum<KT> &a, const FSum<KT> &b) {
  int c;
  if ((c = kcmp(a.k0, b.k0)) != 0) return c < 0;
  if ((c = kcmp(a.k3, b.k3)) != 0) return c < 0;
  if (a.len != b.len) return a.len < b.len;
  if ((c = kcmp(a.k1, b.k1)) != 0) return c < 0;
  return kcmp(a.k2, b.k2) < 0;
}

__device__ __forceinline__ uint16_t count_at(uint64_t w, unsigned c) { return (uint16_t)(w >> (16 * c)); }
/* get_{in,out}_edge_total_frequency (debruijn_graph_node.hpp:299-313): saturating sum */
__device__ __forceinline__ uint16_t total_of(uint64_t w) {
  uint32_t t = 0;
  #pragma unroll
  for (unsigned c = 0; c < 4; ++c) t = min(0xFFFFu, t + count_at(w, c));
  return (uint16_t)t;
}
__device__ __forceinline__ bool single16(unsigned n) { return n != 0 && (n & (n - 1)) == 0; }
__device__ __forceinline__ unsigned rc_biedge16(unsigned e) { return (comp16(e & 0xFu) << 4) | comp16((e >> 4) & 0xFu); }

template <class KT>
__device__ __forceinline__ void canon_edge(KT &x, unsigned &e, int k) {   /* lex_less on (k-mer, biedge) */
  const KT y = KOps<KT>::rc(x, k);
  if (!KOps<KT>::lt(x, y)) { x = y; e = rc_biedge16(e); }
}

/* zero the counts that the single-character nibbles of e name, on the node of canonical x */
template <class KT>
__device__ __forceinline__ void zero_edges(uint64_t *table, const TableGeom &g, KT x, unsigned e) {
  constexpr int SU = Slot<KT>::U64, KWD = Slot<KT>::KEYW;
  const long long s = table_find<KT>(table, g, 4096u, x);
  if (s < 0) return;
  unsigned long long *pw = (unsigned long long *)(table + (uint64_t)s * SU + KWD);
  const unsigned out = e & 0xFu, in = (e >> 4) & 0xFu;
  if (single16(out)) atomicAnd(&pw[0], ~(0xFFFFull << (16 * (__ffs(out) - 1))));
  if (single16(in)) atomicAnd(&pw[1], ~(0xFFFFull << (16 * (__ffs(in) - 1))));
}

template <class KT>
__device__ __forceinline__ void clear_node(uint64_t *slot) {   /* the slot stops being a graph node */
  atomicAnd((unsigned long long *)&slot[Slot<KT>::KEYW - 1], ~(unsigned long long)KEY_NODE);
}

/* erase_nodes(get_cycle_node_kmers()) (debruijn_graph_map.hpp:833-836, 811-827): every cycle
 * node leaves the graph and its neighbours lose the edges back to it (get_remote_edges, :440-471) */
template <class KT>
__global__ void __launch_bounds__(TPB) k_cl_cycles(const uint64_t *ckey, const uint8_t *removed, uint64_t M,
                                                    uint64_t *table, TableGeom g, int k) {
  constexpr int KWD = KOps<KT>::WORDS, SU = Slot<KT>::U64;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (uint64_t)gridDim.x * blockDim.x) {
    if (removed[i] != 1) continue;
    const KT K = KOps<KT>::load(ckey + i * KWD);
    const long long s = table_find<KT>(table, g, 4096u, K);
    if (s < 0) continue;
    uint64_t *slot = table + (uint64_t)s * SU;
    const uint64_t out = slot[KWD], in = slot[KWD + 1];
    for (unsigned c = 0; c < 4; ++c) {
      if (count_at(out, c)) {   /* K.c: its in-edge from K's first base */
        KT y = KOps<KT>::append(K, c, k);
        unsigned e = (1u << KOps<KT>::first(K, k)) << 4;
        canon_edge(y, e, k);
        zero_edges<KT>(table, g, y, e);
      }
      if (count_at(in, c)) {    /* c.K: its out-edge to K's last base */
        KT y = KOps<KT>::prepend(c, K, k);
        unsigned e = 1u << KOps<KT>::last(K);
        canon_edge(y, e, k);
        zero_edges<KT>(table, g, y, e);
      }
    }
    clear_node<KT>(slot);
  }
}

/* idx.erase_if(IsIsolated) (debruijn_graph_filters.hpp:163-172): nodes without an edge leave
 * the graph; counts the nodes and branch nodes that stay */
template <class KT>
__global__ void __launch_bounds__(TPB) k_cl_isolated(uint64_t *table, uint64_t nslots, DevCounters *ctr) {
  constexpr int KWD = Slot<KT>::KEYW, SU = Slot<KT>::U64;
  unsigned long long live = 0, br = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t *s = table + i * SU;
    if (!key_is_node(KOps<KT>::load(s))) continue;
    if (s[KWD] == 0 && s[KWD + 1] == 0) { clear_node<KT>(s); continue; }
    ++live;
    br += (slot_flags<KT>(s) & NF_BRANCH) ? 1 : 0;
  }
  live = warp_sum(live); br = warp_sum(br);
  if ((threadIdx.x & 31) == 0) {
    if (live) atomicAdd(&ctr->cl_live, live);
    if (br) atomicAdd(&ctr->cl_live_branch, br);
  }
}

/* IsBranchPoint / IsChainNode again for every node (the filter's rule, debruijn_graph_filters.hpp
 * :57-220), with the chain and branch lists and each chain node's index rebuilt */
template <class KT>
__global__ void __launch_bounds__(TPB) k_cl_classify(uint64_t *table, uint64_t nslots, int k, uint32_t *chain_list,
                                                      uint32_t *branch_list, uint64_t cap, DevCounters *ctr) {
  constexpr int KWD = Slot<KT>::KEYW, SU = Slot<KT>::U64;
  bool over = false;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < nslots; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    uint64_t *s = table + (i < nslots ? i : 0) * SU;
    const bool node = i < nslots && key_is_node(KOps<KT>::load(s));
    bool branch = false;
    if (node) {
      const KT key = key_kmer(node_key(KOps<KT>::load(s)));
      const bool kpal = k_palindrome(key, k);
      const bool high = km1_high_palindrome(key, k), low = km1_low_palindrome(key, k);
      const unsigned first = KOps<KT>::first(key, k), last = KOps<KT>::last(key);
      const bool oddk = (k & 1) != 0;
      unsigned din = 0, dout = 0;
      bool k1pal = false;
      #pragma unroll
      for (unsigned c = 0; c < 4; ++c) {
        const bool o = count_at(s[KWD], c) > 0, n = count_at(s[KWD + 1], c) > 0;
        dout += o; din += n;
        if (oddk && o && low && (first == 3u - c || first == c)) k1pal = true;
        if (oddk && n && high && (last == 3u - c || last == c)) k1pal = true;
      }
      branch = din >= 2 || dout >= 2 || kpal || k1pal;
    }
    const unsigned long long oc = block_append(node && !branch, &ctr->n_chain);
    const unsigned long long ob = block_append(node && branch, &ctr->n_branch);
    if (node) {
      const unsigned long long o = branch ? ob : oc;
      if (o >= cap) { over = true; continue; }
      const uint64_t aux = branch ? 0xFFFFFFFFull : o;
      s[KWD + 2] = (s[KWD + 2] & 0xFFFFull) | ((uint64_t)(branch ? NF_BRANCH : NF_CHAIN) << 16) | (aux << 32);
      (branch ? branch_list : chain_list)[o] = (uint32_t)i;
    }
  }
  if (over) atomicOr(&ctr->err, (unsigned long long)DERR_INVARIANT);
}

/* to_summarized_chains(dbg) (debruijn_chain_graph.hpp:2044-2105), first half: one record per
 * chain end (IsTerminusOrIsolated), oriented so that the 5' terminus is the representative,
 * with the end node's total in- or out-edge frequency.  tslot: record index per chain node. */
template <class KT>
__global__ void __launch_bounds__(TPB) k_cl_termini(EmitArgs a, const uint64_t *table, TableGeom g, FSum<KT> *trec,
                                                     uint32_t *tslot, DevCounters *ctr) {
  constexpr int KWD = KOps<KT>::WORDS, SU = Slot<KT>::U64;
  unsigned long long nz = 0;
  bool bad = false, missing = false;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < a.M; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    bool want = false;
    FSum<KT> r{};
    if (i < a.M && a.removed[i] == 0) {
      const ChainState st = a.cs[i];
      const bool t5 = term(st.inD), t3 = term(st.outD);
      if (t5 || t3) {
        want = true;
        const KT K = KOps<KT>::load(a.ckey + i * KWD);
        const KT inK = side_kmer<KT>(st.inP, a), outK = side_kmer<KT>(st.outP, a);
        uint16_t fin = 0, fout = 0;
        const long long s = table_find<KT>(table, g, 4096u, K);
        if (s < 0) missing = true;
        else { fout = total_of(table[(uint64_t)s * SU + KWD]); fin = total_of(table[(uint64_t)s * SU + KWD + 1]); }
        const KT Z{};
        r.len = (st.inD & DM) + (st.outD & DM);
        r.node = (uint32_t)i;
        if (t5 && t3) {   /* unit or isolated chain */
          r.k0 = inK; r.k1 = K; r.k2 = K; r.k3 = outK; r.f5 = fin; r.f6 = fout;
        } else if (t5) {
          const KT o = KOps<KT>::rc(outK, a.k);
          if (KOps<KT>::lt(K, o)) { r.k0 = inK; r.k1 = K; r.k2 = outK; r.k3 = Z; r.f5 = fin; }
          else if (KOps<KT>::lt(o, K)) { r.k0 = Z; r.k1 = o; r.k2 = KOps<KT>::rc(K, a.k); r.k3 = KOps<KT>::rc(inK, a.k); r.f6 = fin; }
          else bad = true;   /* the reference throws: a palindrome or a mobius strip */
        } else {
          const KT o = KOps<KT>::rc(K, a.k);
          if (KOps<KT>::lt(inK, o)) { r.k0 = Z; r.k1 = inK; r.k2 = K; r.k3 = outK; r.f6 = fout; }
          else if (KOps<KT>::lt(o, inK)) { r.k0 = KOps<KT>::rc(outK, a.k); r.k1 = o; r.k2 = KOps<KT>::rc(inK, a.k); r.k3 = Z; r.f5 = fout; }
          else bad = true;
        }
        nz += KOps<KT>::eq(r.k1, Z) ? 0 : 1;
      }
    }
    const unsigned long long o = block_append(want, &ctr->cl_term);
    if (want) { trec[o] = r; tslot[i] = (uint32_t)o; }
  }
  nz = warp_sum(nz);
  if ((threadIdx.x & 31) == 0 && nz) atomicAdd(&ctr->cl_nonzero, nz);
  if (bad) atomicOr(&ctr->err, (unsigned long long)DERR_UNCLEAN_CHAINS);
  if (missing) atomicOr(&ctr->err, (unsigned long long)DERR_INVARIANT);
}

/* second half (:2107-2128): sorted by (5' terminus, next at 3'), a unit chain's record is kept
 * and the two ends of a chain merge (merge_summarized_chains, debruijn_chain_node.hpp:176-197:
 * the later record in that order keeps its fields unless the earlier one has the larger end
 * frequency).  Each end finds its partner through its ranked pointer; the later one emits.  On
 * one rank the shifts deliver value-initialised records: a first record on the all-A k-mer is
 * also emitted alone, and a last one on it is dropped. */
template <class KT>
__global__ void __launch_bounds__(TPB) k_cl_pair(EmitArgs a, const FSum<KT> *trec, const uint32_t *tslot, uint64_t nt,
                                                  FSum<KT> *sums, DevCounters *ctr) {
  const bool all_polya = *(volatile unsigned long long *)&ctr->cl_nonzero == 0;
  bool bad = false;
  for (uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x; t0 < nt; t0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t t = t0 + threadIdx.x;
    bool emit = false;
    FSum<KT> m{};
    if (t < nt) {
      const FSum<KT> r = trec[t];
      const bool polya = KOps<KT>::eq(r.k1, KT{});
      if (r.len == 0) {
        m = r;
        emit = !(polya && all_polya);
      } else {
        const ChainState st = a.cs[r.node];
        const uint64_t P = term(st.inD) ? st.outP : st.inP;
        const uint32_t j = (uint32_t)P;
        if ((P & (PF_EXT | PF_BLANK)) || j >= a.M || j == r.node || a.removed[j] != 0 ||
            !(term(a.cs[j].inD) || term(a.cs[j].outD))) {
          bad = true;
        } else {
          const FSum<KT> q = trec[tslot[j]];
          if (q.node != j || q.len != r.len || !KOps<KT>::eq(q.k1, r.k1) || !KOps<KT>::eq(q.k2, r.k2)) {
            bad = true;
          } else {
            const int c = sum_cmp<KT>(r, q);
            if (c > 0 || (c == 0 && r.node > j)) {
              m = r;
              if (m.f5 < q.f5) { m.k0 = q.k0; m.f5 = q.f5; }
              if (m.f6 < q.f6) { m.k3 = q.k3; m.f6 = q.f6; }
              emit = !(polya && all_polya);
            } else if (polya) {
              m = r;
              emit = true;
            }
          }
        }
      }
    }
    const unsigned long long o = block_append(emit, &ctr->cl_sum);
    if (emit) sums[o] = m;
  }
  if (bad) atomicOr(&ctr->err, (unsigned long long)DERR_UNCLEAN_CHAINS);
}

template <class KT>
__device__ __forceinline__ void put_query(EraseQ *q, unsigned long long o, KT x, unsigned e) {
  EraseQ v{};
  KOps<KT>::store(v.w, x);
  v.edge = e;
  q[o] = v;
}

/* find_deadends (debruijn_topo_operations.hpp:146-175) with deadend_filter
 * (compact_dbg_clean.hpp:63-80) and the end edges to sever (:619-640): the 5' branch's
 * out-edge to the 5' terminus, the 3' branch's in-edge from the 3' terminus; and the chains
 * with both ends on branches (find_normal_chains, :251-272), put on the strand where the 5'
 * branch is not above the reverse complement of the 3' branch (find_bubbles, :310-316) */
template <class KT>
__global__ void __launch_bounds__(TPB) k_cl_select(const FSum<KT> *sums, uint64_t ns, int k, uint32_t min_freq,
                                                    uint32_t max_len, EraseQ *q, FSum<KT> *norm, DevCounters *ctr) {
  unsigned long long nd = 0;
  for (uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x; t0 < ns; t0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t t = t0 + threadIdx.x;
    FSum<KT> r{};
    if (t < ns) r = sums[t];
    const bool valid = t < ns;
    const bool dead = valid && r.len < max_len && r.f5 < min_freq && r.f6 < min_freq && ((r.f5 == 0) != (r.f6 == 0));
    const bool d5 = dead && r.f5 > 0, d3 = dead && r.f6 > 0;
    const bool normal = valid && r.len > 0 && r.f5 > 0 && r.f6 > 0;
    nd += dead ? 1 : 0;
    unsigned long long o = block_append(d5, &ctr->cl_q);
    if (d5) put_query<KT>(q, o, r.k0, 1u << KOps<KT>::last(r.k1));
    o = block_append(d3, &ctr->cl_q);
    if (d3) put_query<KT>(q, o, r.k3, (1u << KOps<KT>::first(r.k2, k)) << 4);
    if (normal && KOps<KT>::lt(KOps<KT>::rc(r.k3, k), r.k0)) {   /* transform::reverse_complement(summary) */
      FSum<KT> x = r;
      x.k0 = KOps<KT>::rc(r.k3, k); x.k1 = KOps<KT>::rc(r.k2, k);
      x.k2 = KOps<KT>::rc(r.k1, k); x.k3 = KOps<KT>::rc(r.k0, k);
      x.f5 = r.f6; x.f6 = r.f5;
      r = x;
    }
    o = block_append(normal, &ctr->cl_norm);
    if (normal) norm[o] = r;
  }
  nd = warp_sum(nd);
  if ((threadIdx.x & 31) == 0 && nd) atomicAdd(&ctr->cl_dead, nd);
}

__device__ __forceinline__ unsigned long long bubble_key(KW1 x) { return x.v + 1; }   /* k-mers fit 62 bits */
__device__ __forceinline__ unsigned long long bubble_key(KW2 x) {
  return (mix64(x.lo ^ mix64(x.hi + 0x9e3779b97f4a7c15ull)) >> 1) + 1;
}

/* chains grouped by their 5' branch k-mer (at most four leave one k-mer's out side; eight
 * places allow for hash collisions of 128-bit k-mers, told apart in k_cl_bubbles) */
template <class KT>
__global__ void __launch_bounds__(TPB) k_cl_group(const FSum<KT> *norm, uint64_t nn, BubbleEnt *tab, uint64_t hcap,
                                                   DevCounters *ctr) {
  bool over = false;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = bubble_key(norm[i].k0);
    uint64_t h = mix64(key) & (hcap - 1);
    bool placed = false;
    for (uint64_t p = 0; p < hcap && !placed; ++p, h = (h + 1) & (hcap - 1)) {
      const unsigned long long prev = atomicCAS(&tab[h].key, 0ull, key);
      if (prev != 0ull && prev != key) continue;
      const unsigned int c = atomicAdd(&tab[h].cnt, 1u);
      if (c < 8) tab[h].idx[c] = (unsigned int)i; else over = true;
      placed = true;
    }
    if (!placed) over = true;
  }
  if (over) atomicOr(&ctr->err, (unsigned long long)DERR_INVARIANT);
}

/* find_bubbles' scan (:348-392) per group: sorted by (5' branch, 3' branch, length), every run
 * of two or more chains between the same two branches whose neighbours pass bubble_filter
 * (compact_dbg_clean.hpp:84-112: lengths within one, an end edge below min_freq) gives both
 * end edges of each of its chains to sever (:687-699) */
template <class KT>
__global__ void __launch_bounds__(TPB) k_cl_bubbles(const FSum<KT> *norm, const BubbleEnt *tab, uint64_t hcap, int k,
                                                     uint32_t min_freq, EraseQ *q, DevCounters *ctr) {
  bool over = false;
  unsigned long long nb = 0;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < hcap; e += (uint64_t)gridDim.x * blockDim.x) {
    if (tab[e].key == 0ull) continue;
    const unsigned int n = tab[e].cnt;
    if (n > 8) { over = true; continue; }
    if (n < 2) continue;
    unsigned int m[8];
    for (unsigned int x = 0; x < n; ++x) m[x] = tab[e].idx[x];
    for (unsigned int x = 1; x < n; ++x)   /* insertion sort, at most eight */
      for (unsigned int y = x; y > 0 && bubble_less<KT>(norm[m[y]], norm[m[y - 1]]); --y) {
        const unsigned int t = m[y]; m[y] = m[y - 1]; m[y - 1] = t;
      }
    unsigned int first = 0, x = 1;
    for (; x <= n; ++x) {
      bool same = false;
      if (x < n) {
        const FSum<KT> &l = norm[m[x - 1]], &r = norm[m[x]];
        const uint32_t d = l.len > r.len ? l.len - r.len : r.len - l.len;
        same = KOps<KT>::eq(l.k0, r.k0) && KOps<KT>::eq(l.k3, r.k3) && d <= 1 &&
               (l.f5 < min_freq || l.f6 < min_freq || r.f5 < min_freq || r.f6 < min_freq);
      }
      if (same) continue;
      if (x - first > 1) {
        const unsigned long long o = atomicAdd(&ctr->cl_q, 2ull * (x - first));
        for (unsigned int y = first; y < x; ++y) {
          const FSum<KT> &c = norm[m[y]];
          put_query<KT>(q, o + 2ull * (y - first), c.k0, 1u << KOps<KT>::last(c.k1));
          put_query<KT>(q, o + 2ull * (y - first) + 1, c.k3, (1u << KOps<KT>::first(c.k2, k)) << 4);
        }
        nb += x - first;
      }
      first = x;
    }
  }
  if (nb) atomicAdd(&ctr->cl_bub, nb);
  if (over) atomicOr(&ctr->err, (unsigned long long)DERR_INVARIANT);
}

/* erase_edges(query, edge_freq_filter) (debruijn_graph_map.hpp:770-775), first step
 * (find_edges with the predicate, :615-660): per query on the canonical strand, the nibbles
 * whose edge exists with a count below min_freq (compact_multi_biedge::select) */
template <class KT>
__global__ void __launch_bounds__(TPB) k_cl_find(const EraseQ *q, uint64_t q0, uint64_t q1, const uint64_t *table,
                                                  TableGeom g, int k, uint32_t min_freq, EraseQ *found,
                                                  DevCounters *ctr) {
  constexpr int KWD = Slot<KT>::KEYW, SU = Slot<KT>::U64;
  for (uint64_t t0 = q0 + (uint64_t)blockIdx.x * blockDim.x; t0 < q1; t0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t t = t0 + threadIdx.x;
    bool want = false;
    KT x{};
    unsigned e = 0;
    if (t < q1) {
      x = KOps<KT>::load(q[t].w);
      e = q[t].edge;
      canon_edge(x, e, k);
      const long long s = table_find<KT>(table, g, 4096u, x);
      if (s >= 0) {
        const uint64_t *pw = table + (uint64_t)s * SU + KWD;
        const unsigned in = (e >> 4) & 0xFu, out = e & 0xFu;
        if (single16(in)) {
          const uint16_t v = count_at(pw[1], __ffs(in) - 1);
          if (!(v > 0 && v < min_freq)) e &= 0x0Fu;
        }
        if (single16(out)) {
          const uint16_t v = count_at(pw[0], __ffs(out) - 1);
          if (!(v > 0 && v < min_freq)) e &= 0xF0u;
        }
        want = e != 0;
      }
    }
    const unsigned long long o = block_append(want, &ctr->cl_found);
    if (want) put_query<KT>(found, o, x, e);
  }
}

/* second step (erase_edges_internal, :737-747): the edges found and, on the neighbours, the
 * same edges seen from there (get_remote_edges for simple biedges, :475-510) */
template <class KT>
__global__ void __launch_bounds__(TPB) k_cl_erase(const EraseQ *f, uint64_t nf, uint64_t *table, TableGeom g, int k) {
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += (uint64_t)gridDim.x * blockDim.x) {
    const KT x = KOps<KT>::load(f[t].w);
    const unsigned e = f[t].edge, in = (e >> 4) & 0xFu, out = e & 0xFu;
    zero_edges<KT>(table, g, x, e);
    if (single16(in)) {
      KT y = KOps<KT>::prepend((unsigned)(__ffs(in) - 1), x, k);
      unsigned r = 1u << KOps<KT>::last(x);
      canon_edge(y, r, k);
      zero_edges<KT>(table, g, y, r);
    }
    if (single16(out)) {
      KT y = KOps<KT>::append(x, (unsigned)(__ffs(out) - 1), k);
      unsigned r = (1u << KOps<KT>::first(x, k)) << 4;
      canon_edge(y, r, k);
      zero_edges<KT>(table, g, y, r);
    }
  }
}

/* ================================================================ graph and chain queries
 * The graph and chain-map operations the reference driver calls between the phases:
 * debruijn_graph::find_if / erase_if (debruijn_graph.hpp:188-252) with the node predicates of
 * bliss::debruijn::filter::graph, debruijn_graph_map::erase_nodes (debruijn_graph_map.hpp:
 * 833-836: the nodes and, on their neighbours, the edges back to them), and
 * debruijn_chain_graph::find_if (debruijn_chain_graph.hpp:306-311) with the chain predicates of
 * bliss::debruijn::filter::chain, get_cycle_node_kmers and get_isolated (:440-470). */

/* the node predicates (debruijn_graph_filters.hpp:38-220), on a node's canonical k-mer and its
 * out / in count words; the (k+1)-mer palindrome test is is_k1_k1pair_rc_palindrome
 * (kmer_traits.hpp:108-125) over the present edges */
template <class KT>
__device__ __forceinline__ bool node_matches(int f, KT key, uint64_t out, uint64_t in, int k) {
  const bool kpal = k_palindrome(key, k), oddk = (k & 1) != 0;
  const bool high = oddk && km1_high_palindrome(key, k), low = oddk && km1_low_palindrome(key, k);
  const unsigned first = KOps<KT>::first(key, k), last = KOps<KT>::last(key);
  unsigned din = 0, dout = 0;
  bool k1pal = false;
  #pragma unroll
  for (unsigned c = 0; c < 4; ++c) {
    const bool o = count_at(out, c) > 0, n = count_at(in, c) > 0;
    dout += o; din += n;
    if (o && low && (first == 3u - c || first == c)) k1pal = true;
    if (n && high && (last == 3u - c || last == c)) k1pal = true;
  }
  switch (f) {
    case BRUNO_NODES_ALL: return true;
    case BRUNO_IS_K_PALINDROME: return kpal;
    case BRUNO_IS_KPLUS1_PALINDROME: return k1pal;
    case BRUNO_IS_BRANCH_POINT: return din >= 2 || dout >= 2 || kpal || k1pal;
    case BRUNO_IS_ISOLATED_NODE: return din == 0 && dout == 0;
    case BRUNO_IS_CHAIN_INTERNAL_NODE: return din == 1 && dout == 1 && !kpal && !k1pal;
    case BRUNO_IS_CHAIN_NODE: return din < 2 && dout < 2 && !kpal && !k1pal;
    default: return false;
  }
}

/* find_if(pred) over the node table: (k-mer, counts[9], flags) of every matching node, flags
 * evaluated on the current counts; erase (erase_if) instead clears the matching nodes */
template <class KT>
__global__ void __launch_bounds__(TPB) k_node_query(uint64_t *table, uint64_t nslots, int k, int f, bool erase,
                                                     uint64_t *keys, uint16_t *counts, uint8_t *flags, uint64_t cap,
                                                     DevCounters *ctr) {
  constexpr int KWD = Slot<KT>::KEYW, SU = Slot<KT>::U64;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < nslots; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    uint64_t *s = table + (i < nslots ? i : 0) * SU;
    bool hit = false;
    KT key{};
    if (i < nslots && key_is_node(KOps<KT>::load(s))) {
      key = key_kmer(node_key(KOps<KT>::load(s)));
      hit = node_matches<KT>(f, key, s[KWD], s[KWD + 1], k);
    }
    const unsigned long long o = block_append(hit, &ctr->n_k2_dump);
    if (!hit) continue;
    if (erase) { clear_node<KT>(s); continue; }
    if (o >= cap) continue;
    if (keys) KOps<KT>::store(keys + o * KWD, key);
    if (counts)
      for (int q = 0; q < 4; ++q) {
        counts[o * 9 + q] = count_at(s[KWD], (unsigned)q);
        counts[o * 9 + 4 + q] = count_at(s[KWD + 1], (unsigned)q);
      }
    if (counts) counts[o * 9 + 8] = (uint16_t)s[KWD + 2];
    if (flags)
      flags[o] = (uint8_t)((node_matches<KT>(BRUNO_IS_BRANCH_POINT, key, s[KWD], s[KWD + 1], k) ? NF_BRANCH : 0u) |
                           (node_matches<KT>(BRUNO_IS_CHAIN_NODE, key, s[KWD], s[KWD + 1], k) ? NF_CHAIN : 0u));
  }
}

/* erase_nodes(query) (debruijn_graph_map.hpp:833-836, erase_nodes_and_edges :811-827): each
 * queried k-mer (either strand) that is a node leaves the graph, and its neighbours lose the
 * edges back to it (get_remote_edges, :440-471).  A node erased here has no edge left on a
 * surviving neighbour whatever the order of the threads: only a neighbour erased in the same
 * call can clear an edge of the node before its thread reads it. */
template <class KT>
__global__ void __launch_bounds__(TPB) k_erase_nodes(const uint64_t *q, uint64_t n, uint64_t *table, TableGeom g,
                                                      int k) {
  constexpr int KWD = KOps<KT>::WORDS, SW = Slot<KT>::KEYW, SU = Slot<KT>::U64;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    KT K = KOps<KT>::load(q + i * KWD);
    const KT R = KOps<KT>::rc(K, k);
    if (!KOps<KT>::lt(K, R)) K = R;
    const long long sl = table_find<KT>(table, g, 4096u, K);
    if (sl < 0) continue;
    uint64_t *slot = table + (uint64_t)sl * SU;
    const uint64_t out = slot[SW], in = slot[SW + 1];
    for (unsigned c = 0; c < 4; ++c) {
      if (count_at(out, c)) {   /* K.c: its in-edge from K's first base */
        KT y = KOps<KT>::append(K, c, k);
        unsigned e = (1u << KOps<KT>::first(K, k)) << 4;
        canon_edge(y, e, k);
        zero_edges<KT>(table, g, y, e);
      }
      if (count_at(in, c)) {    /* c.K: its out-edge to K's last base */
        KT y = KOps<KT>::prepend(c, K, k);
        unsigned e = 1u << KOps<KT>::last(K);
        canon_edge(y, e, k);
        zero_edges<KT>(table, g, y, e);
      }
    }
    clear_node<KT>(slot);
  }
}

/* live nodes after an erasure, with the classification of each stored again from its counts
 * (the filter's IsBranchPoint / IsChainNode), so that the node copy-out stays current */
template <class KT>
__global__ void __launch_bounds__(TPB) k_node_recount(uint64_t *table, uint64_t nslots, int k, DevCounters *ctr) {
  constexpr int KWD = Slot<KT>::KEYW, SU = Slot<KT>::U64;
  unsigned long long live = 0, br = 0, ch = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t *s = table + i * SU;
    if (!key_is_node(KOps<KT>::load(s))) continue;
    const KT key = key_kmer(node_key(KOps<KT>::load(s)));
    const bool b = node_matches<KT>(BRUNO_IS_BRANCH_POINT, key, s[KWD], s[KWD + 1], k);
    const bool cn = node_matches<KT>(BRUNO_IS_CHAIN_NODE, key, s[KWD], s[KWD + 1], k);
    const uint64_t fl = (b ? NF_BRANCH : 0u) | (cn ? NF_CHAIN : 0u);
    s[KWD + 2] = (s[KWD + 2] & ~(0xFFFFull << 16)) | (fl << 16);
    ++live; br += b; ch += cn;
  }
  live = warp_sum(live); br = warp_sum(br); ch = warp_sum(ch);
  if ((threadIdx.x & 31) == 0) {
    if (live) atomicAdd(&ctr->n_nodes, live);
    if (br) atomicAdd(&ctr->n_branch, br);
    if (ch) atomicAdd(&ctr->n_chain, ch);
  }
}

/* the chain predicates (debruijn_chain_filters.hpp:37-186) on a chain-map record */
template <class KT>
__device__ __forceinline__ bool chain_matches(int f, KT K, KT inK, KT outK, uint32_t inD, uint32_t outD, int k) {
  const bool ti = term(inD), to = term(outD);
  switch (f) {
    case BRUNO_CHAIN_ALL: return true;
    case BRUNO_CHAIN_IS_UNIT_LENGTH: return ti && to;
    case BRUNO_CHAIN_IS_ISOLATED: return inD == TM && outD == TM;
    case BRUNO_CHAIN_IS_TERMINUS: return ti != to;
    case BRUNO_CHAIN_IS_INTERNAL: return (inD & DM) > 0 && (outD & DM) > 0;
    case BRUNO_CHAIN_IS_TERMINUS_OR_ISOLATED: return ti || to;
    case BRUNO_CHAIN_IS_CANONICAL_TERMINUS:
    case BRUNO_CHAIN_IS_CANONICAL_TERMINUS_OR_ISOLATED:
      if (ti && to) return f == BRUNO_CHAIN_IS_CANONICAL_TERMINUS_OR_ISOLATED;
      if (ti) return KOps<KT>::le(K, KOps<KT>::rc(outK, k));
      if (to) return KOps<KT>::lt(KOps<KT>::rc(K, k), inK);
      return false;
    case BRUNO_CHAIN_POINTS_TO_TERMINI: return !ptcn(inD) && !ptcn(outD);
    case BRUNO_CHAIN_POINTS_TO_INTERNAL_NODE: return ptcn(inD) || ptcn(outD);
    default: return false;
  }
}

/* chain-map records (K, inK, outK, inD, outD) of the nodes whose removed[] mark is `which`
 * (0: in the chain map, 1: cycle nodes, 2: isolated nodes) that match f */
template <class KT>
__global__ void __launch_bounds__(TPB) k_chain_query(EmitArgs a, int f, uint8_t which, uint64_t *kmers, uint64_t *inK,
                                                      uint64_t *outK, uint32_t *inD, uint32_t *outD, uint64_t cap) {
  constexpr int KWD = KOps<KT>::WORDS;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < a.M; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    bool hit = false;
    KT K{}, L{}, R{};
    ChainState st{};
    if (i < a.M && (a.removed ? a.removed[i] : 0) == which) {
      st = a.cs[i];
      K = KOps<KT>::load(a.ckey + i * KWD);
      L = side_kmer<KT>(st.inP, a);
      R = side_kmer<KT>(st.outP, a);
      hit = chain_matches<KT>(f, K, L, R, st.inD, st.outD, a.k);
    }
    const unsigned long long o = block_append(hit, &a.ctr->n_k2_dump);
    if (!hit || o >= cap) continue;
    if (kmers) KOps<KT>::store(kmers + o * KWD, K);
    if (inK) KOps<KT>::store(inK + o * KWD, L);
    if (outK) KOps<KT>::store(outK + o * KWD, R);
    if (inD) inD[o] = st.inD;
    if (outD) outD[o] = st.outD;
  }
}

/* check_index (test/common/compact_dbg_stats.hpp:45-119): every neighbour k-mer that a node's
 * edges name (get_out_neighbors / get_in_neighbors, canonical) must be a node, and every node
 * with an edge must be named by some node; also counted: edges whose neighbour lacks the edge
 * back, and the in x out edge-count histogram of print_compact_multi_biedge_histogram
 * (debruijn_stats.hpp:39-74).  `ref` gets one bit per table slot named as a neighbour. */
struct IndexCheck { unsigned long long query, absent, unreferenced, unanswered, hist[25]; };

template <class KT>
__device__ __forceinline__ bool has_edge(const uint64_t *table, long long sl, unsigned e) {
  constexpr int KWD = Slot<KT>::KEYW, SU = Slot<KT>::U64;
  const uint64_t *pw = table + (uint64_t)sl * SU + KWD;
  const unsigned out = e & 0xFu, in = (e >> 4) & 0xFu;
  if (single16(out) && !count_at(pw[0], __ffs(out) - 1)) return false;
  if (single16(in) && !count_at(pw[1], __ffs(in) - 1)) return false;
  return true;
}

template <class KT>
__global__ void __launch_bounds__(TPB) k_check_refs(const uint64_t *table, uint64_t nslots, TableGeom g, int k,
                                                     uint32_t *ref, IndexCheck *out) {
  constexpr int KWD = Slot<KT>::KEYW, SU = Slot<KT>::U64;
  __shared__ unsigned long long s_hist[25];
  for (int i = threadIdx.x; i < 25; i += blockDim.x) s_hist[i] = 0;
  __syncthreads();
  unsigned long long q = 0, absent = 0, unanswered = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t *s = table + i * SU;
    if (!key_is_node(KOps<KT>::load(s))) continue;
    const KT K = key_kmer(node_key(KOps<KT>::load(s)));
    const uint64_t ow = s[KWD], iw = s[KWD + 1];
    unsigned din = 0, dout = 0;
    for (unsigned c = 0; c < 4; ++c) {
      for (int side = 0; side < 2; ++side) {
        if (!count_at(side ? iw : ow, c)) continue;
        ++q;
        side ? ++din : ++dout;
        /* the neighbour and the edge it should have back: K.c has an in edge from first(K);
         * c.K has an out edge to last(K) */
        KT y = side ? KOps<KT>::prepend(c, K, k) : KOps<KT>::append(K, c, k);
        unsigned e = side ? (1u << KOps<KT>::last(K)) : ((1u << KOps<KT>::first(K, k)) << 4);
        canon_edge(y, e, k);
        const long long sl = table_find<KT>(table, g, 4096u, y);
        if (sl < 0) { ++absent; continue; }
        atomicOr(&ref[(uint64_t)sl >> 5], 1u << ((uint64_t)sl & 31));
        if (!has_edge<KT>(table, sl, e)) ++unanswered;
      }
    }
    atomicAdd(&s_hist[din * 5 + dout], 1ull);
  }
  q = warp_sum(q); absent = warp_sum(absent); unanswered = warp_sum(unanswered);
  if ((threadIdx.x & 31) == 0) {
    if (q) atomicAdd(&out->query, q);
    if (absent) atomicAdd(&out->absent, absent);
    if (unanswered) atomicAdd(&out->unanswered, unanswered);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 25; i += blockDim.x)
    if (s_hist[i]) atomicAdd(&out->hist[i], s_hist[i]);
}

/* the second check: nodes with an edge that no node named */
template <class KT>
__global__ void __launch_bounds__(TPB) k_check_unreferenced(const uint64_t *table, uint64_t nslots,
                                                             const uint32_t *ref, IndexCheck *out) {
  constexpr int KWD = Slot<KT>::KEYW, SU = Slot<KT>::U64;
  unsigned long long n = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t *s = table + i * SU;
    if (!key_is_node(KOps<KT>::load(s))) continue;
    if (s[KWD] == 0 && s[KWD + 1] == 0) continue;   /* IsIsolated: erased before the check */
    if (!(ref[i >> 5] & (1u << (i & 31)))) ++n;
  }
  n = warp_sum(n);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(&out->unreferenced, n);
}

template <class KT>
bruno_status check_index_typed(Ctx *c, bruno_index_check *o) {
  bruno_status st;
  Buf ref, res;
  const uint64_t words = (c->nslots + 31) / 32 + 1;
  if ((st = ensure(c, ref, words * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, res, sizeof(IndexCheck))) != BRUNO_OK) return st;
  cudaMemsetAsync(ref.p, 0, words * 4, c->stream);
  cudaMemsetAsync(res.p, 0, sizeof(IndexCheck), c->stream);
  k_check_refs<KT><<<sms_count() * 8, TPB, 0, c->stream>>>((const uint64_t *)c->table.p, c->nslots, c->geom, c->cfg.k,
                                                          (uint32_t *)ref.p, (IndexCheck *)res.p);
  k_check_unreferenced<KT><<<sms_count() * 8, TPB, 0, c->stream>>>((const uint64_t *)c->table.p, c->nslots,
                                                                  (const uint32_t *)ref.p, (IndexCheck *)res.p);
  c->launches += 2;
  IndexCheck h{};
  st = cuda_check(c, cudaMemcpyAsync(&h, res.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream), "copy");
  if (st == BRUNO_OK) st = cuda_check(c, cudaStreamSynchronize(c->stream), "check_index");
  cudaFreeAsync(ref.p, c->stream);
  cudaFreeAsync(res.p, c->stream);
  if (st != BRUNO_OK) return st;
  o->n_query = h.query; o->n_absent = h.absent; o->n_unreferenced = h.unreferenced; o->n_unanswered = h.unanswered;
  for (int i = 0; i < 25; ++i) o->edge_hist[i] = h.hist[i];
  return BRUNO_OK;
}

template <class KT>
bruno_status node_query_typed(Ctx *c, int f, bool erase, uint64_t *keys, uint16_t *counts, uint8_t *flags, size_t cap,
                              size_t *n) {
  bruno_status st;
  const bool copy = !erase && (keys || counts || flags);
  const uint64_t nb = std::max<uint64_t>(1, c->n_nodes);
  Buf dk, dc, df;
  if (copy) {
    if ((st = ensure(c, dk, nb * 8 * c->W)) != BRUNO_OK) return st;
    if ((st = ensure(c, dc, nb * 18)) != BRUNO_OK) return st;
    if ((st = ensure(c, df, nb)) != BRUNO_OK) return st;
  }
  cudaMemsetAsync(&c->dctr->n_k2_dump, 0, 8, c->stream);
  k_node_query<KT><<<sms_count() * 8, TPB, 0, c->stream>>>((uint64_t *)c->table.p, c->nslots, c->cfg.k, f, erase,
                                                          (uint64_t *)dk.p, (uint16_t *)dc.p, (uint8_t *)df.p,
                                                          copy ? nb : 0, c->dctr);
  c->launches += 1;
  bruno_status r = sync_counters(c);
  const uint64_t hits = c->hctr->n_k2_dump;
  if (n) *n = hits;
  if (r == BRUNO_OK && copy) {
    if (cap < hits) r = set_err(c, BRUNO_ERR_CAPACITY, "find_if buffers too small");
    if (r == BRUNO_OK && keys) r = cuda_check(c, cudaMemcpyAsync(keys, dk.p, hits * 8 * c->W, cudaMemcpyDeviceToHost, c->stream), "copy");
    if (r == BRUNO_OK && counts) r = cuda_check(c, cudaMemcpyAsync(counts, dc.p, hits * 18, cudaMemcpyDeviceToHost, c->stream), "copy");
    if (r == BRUNO_OK && flags) r = cuda_check(c, cudaMemcpyAsync(flags, df.p, hits, cudaMemcpyDeviceToHost, c->stream), "copy");
    if (r == BRUNO_OK) r = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  }
  if (copy) { cudaFreeAsync(dk.p, c->stream); cudaFreeAsync(dc.p, c->stream); cudaFreeAsync(df.p, c->stream); }
  return r;
}

template <class KT>
bruno_status node_recount_typed(Ctx *c) {
  cudaMemsetAsync(&c->dctr->n_nodes, 0, 8, c->stream);
  cudaMemsetAsync(&c->dctr->n_branch, 0, 8, c->stream);
  cudaMemsetAsync(&c->dctr->n_chain, 0, 8, c->stream);
  k_node_recount<KT><<<sms_count() * 8, TPB, 0, c->stream>>>((uint64_t *)c->table.p, c->nslots, c->cfg.k, c->dctr);
  c->launches += 1;
  bruno_status st = sync_counters(c);
  if (st != BRUNO_OK) return st;
  c->n_nodes = c->hctr->n_nodes;
  c->n_branch = c->hctr->n_branch;
  c->chain_edges_done = false;   /* the chain ends' edge counts come from the node table */
  return BRUNO_OK;
}

template <class KT>
bruno_status erase_nodes_typed(Ctx *c, const uint64_t *kmers, size_t n) {
  bruno_status st;
  if (n) {
    Buf dq;
    if ((st = ensure(c, dq, n * 8 * c->W)) != BRUNO_OK) return st;
    if ((st = cuda_check(c, cudaMemcpyAsync(dq.p, kmers, n * 8 * c->W, cudaMemcpyHostToDevice, c->stream), "copy")) !=
        BRUNO_OK)
      return st;
    const int g = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms_count() * 8, (n + TPB - 1) / TPB));
    k_erase_nodes<KT><<<g, TPB, 0, c->stream>>>((const uint64_t *)dq.p, n, (uint64_t *)c->table.p, c->geom, c->cfg.k);
    c->launches += 1;
    cudaFreeAsync(dq.p, c->stream);
  }
  return node_recount_typed<KT>(c);
}

template <class KT>
bruno_status chain_query_typed(Ctx *c, int f, int which, uint64_t *kmers, uint64_t *inK, uint64_t *outK, uint32_t *inD,
                               uint32_t *outD, size_t cap, size_t *n) {
  bruno_status st;
  const uint64_t M = c->n_chain, Mb = std::max<uint64_t>(1, M);
  const bool copy = kmers || inK || outK || inD || outD;
  Buf b0, b1, b2, b3, b4;
  if (copy) {
    if ((st = ensure(c, b0, Mb * 8 * c->W)) != BRUNO_OK) return st;
    if ((st = ensure(c, b1, Mb * 8 * c->W)) != BRUNO_OK) return st;
    if ((st = ensure(c, b2, Mb * 8 * c->W)) != BRUNO_OK) return st;
    if ((st = ensure(c, b3, Mb * 4)) != BRUNO_OK) return st;
    if ((st = ensure(c, b4, Mb * 4)) != BRUNO_OK) return st;
  }
  EmitArgs a{};
  a.ckey = (const uint64_t *)c->ckey.p; a.cedge = (const uint8_t *)c->cedge.p; a.cs = (const ChainState *)c->cstate.p;
  a.removed = c->stage >= 5 ? (const uint8_t *)c->removed.p : nullptr;
  a.M = M; a.k = c->cfg.k; a.ctr = c->dctr;
  cudaMemsetAsync(&c->dctr->n_k2_dump, 0, 8, c->stream);
  if (M)
    k_chain_query<KT><<<sms_count() * 8, TPB, 0, c->stream>>>(a, f, (uint8_t)which, (uint64_t *)b0.p, (uint64_t *)b1.p,
                                                             (uint64_t *)b2.p, (uint32_t *)b3.p, (uint32_t *)b4.p,
                                                             copy ? Mb : 0);
  c->launches += 1;
  bruno_status r = sync_counters(c);
  const uint64_t hits = c->hctr->n_k2_dump;
  if (n) *n = hits;
  if (r == BRUNO_OK && copy) {
    if (cap < hits) r = set_err(c, BRUNO_ERR_CAPACITY, "chain find_if buffers too small");
    const size_t kb = hits * 8 * c->W;
    if (r == BRUNO_OK && kmers) r = cuda_check(c, cudaMemcpyAsync(kmers, b0.p, kb, cudaMemcpyDeviceToHost, c->stream), "copy");
    if (r == BRUNO_OK && inK) r = cuda_check(c, cudaMemcpyAsync(inK, b1.p, kb, cudaMemcpyDeviceToHost, c->stream), "copy");
    if (r == BRUNO_OK && outK) r = cuda_check(c, cudaMemcpyAsync(outK, b2.p, kb, cudaMemcpyDeviceToHost, c->stream), "copy");
    if (r == BRUNO_OK && inD) r = cuda_check(c, cudaMemcpyAsync(inD, b3.p, hits * 4, cudaMemcpyDeviceToHost, c->stream), "copy");
    if (r == BRUNO_OK && outD) r = cuda_check(c, cudaMemcpyAsync(outD, b4.p, hits * 4, cudaMemcpyDeviceToHost, c->stream), "copy");
    if (r == BRUNO_OK) r = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  }
  if (copy) {
    cudaFreeAsync(b0.p, c->stream); cudaFreeAsync(b1.p, c->stream); cudaFreeAsync(b2.p, c->stream);
    cudaFreeAsync(b3.p, c->stream); cudaFreeAsync(b4.p, c->stream);
  }
  return r;
}

template <class KT>
bruno_status clean_typed(Ctx *c, uint64_t *rounds, uint64_t *deadends, uint64_t *bubbles, uint64_t *edges,
                         int32_t *status) {
  bruno_status st;
  const int sms = sms_count(), k = c->cfg.k;
  const uint32_t min_freq = (uint32_t)(c->thr_used[2] + 1);     /* edge_freq_filter(threshes[2] + 1) */
  const uint32_t max_len = 2u * (uint32_t)k - 1u;               /* deadend_filter(2 * k - 1, ...) */
  uint64_t *table = (uint64_t *)c->table.p;
  const int KWD = Slot<KT>::KEYW;
  *rounds = *deadends = *bubbles = *edges = 0;
  *status = 0;
  auto isolated = [&]() -> bruno_status {
    cudaMemsetAsync(&c->dctr->cl_live, 0, 16, c->stream);
    k_cl_isolated<KT><<<sms * 8, TPB, 0, c->stream>>>(table, c->nslots, c->dctr);
    c->launches += 1;
    bruno_status s2 = sync_counters(c);
    if (s2 != BRUNO_OK) return s2;
    c->n_nodes = c->hctr->cl_live;
    c->n_branch = c->hctr->cl_live_branch;
    return BRUNO_OK;
  };
  auto cycles = [&]() -> bruno_status {
    if (c->n_cycle && c->n_chain)
      k_cl_cycles<KT><<<sms * 8, TPB, 0, c->stream>>>((const uint64_t *)c->ckey.p, (const uint8_t *)c->removed.p,
                                                      c->n_chain, table, c->geom, k);
    c->launches += 1;
    return isolated();
  };
  /* the driver takes cycle nodes and then edge-less nodes out right after the first ranking
   * (compact_dbg_freq_construct_clean.cpp:599-604) */
  if ((st = cycles()) != BRUNO_OK) return st;
  for (uint64_t iter = 0;; ++iter) {
    const uint64_t M = c->n_chain, Mb = std::max<uint64_t>(1, M);
    if ((st = ensure(c, c->cl_trec, Mb * sizeof(FSum<KT>))) != BRUNO_OK) return st;
    if ((st = ensure(c, c->cl_tslot, Mb * 4)) != BRUNO_OK) return st;
    EmitArgs a{};
    a.ckey = (const uint64_t *)c->ckey.p; a.cedge = (const uint8_t *)c->cedge.p; a.cs = (const ChainState *)c->cstate.p;
    a.removed = (const uint8_t *)c->removed.p; a.M = M; a.k = k;
    FSum<KT> *trec = (FSum<KT> *)c->cl_trec.p;
    cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
    cudaMemsetAsync(&c->dctr->cl_term, 0, 8 * 8, c->stream);   /* cl_term .. cl_bub */
    if (M) k_cl_termini<KT><<<sms * 8, TPB, 0, c->stream>>>(a, table, c->geom, trec, (uint32_t *)c->cl_tslot.p, c->dctr);
    c->launches += 1;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    const uint64_t nt = c->hctr->cl_term, ntb = std::max<uint64_t>(1, nt);
    if ((st = ensure(c, c->cl_sums, ntb * sizeof(FSum<KT>))) != BRUNO_OK) return st;
    if ((st = ensure(c, c->cl_norm, ntb * sizeof(FSum<KT>))) != BRUNO_OK) return st;
    if ((st = ensure(c, c->cl_q, 4 * ntb * sizeof(EraseQ))) != BRUNO_OK) return st;
    if ((st = ensure(c, c->cl_found, 4 * ntb * sizeof(EraseQ))) != BRUNO_OK) return st;
    FSum<KT> *sums = (FSum<KT> *)c->cl_sums.p, *norm = (FSum<KT> *)c->cl_norm.p;
    EraseQ *q = (EraseQ *)c->cl_q.p, *found = (EraseQ *)c->cl_found.p;
    const int gt = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * 8, (nt + TPB - 1) / TPB));
    if (nt) k_cl_pair<KT><<<gt, TPB, 0, c->stream>>>(a, trec, (const uint32_t *)c->cl_tslot.p, nt, sums, c->dctr);
    c->launches += 1;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    if (c->hctr->err & DERR_INVARIANT) return set_err(c, BRUNO_ERR_INVARIANT, "cleaning: a chain end has no node");
    if (c->hctr->err & DERR_UNCLEAN_CHAINS) {
      *status = 2;
      return set_err(c, BRUNO_ERR_INVARIANT, "cleaning needs mutually consistent chain pointers");
    }
    const uint64_t ns = c->hctr->cl_sum;
    if (ns) k_cl_select<KT><<<gt, TPB, 0, c->stream>>>(sums, ns, k, min_freq, max_len, q, norm, c->dctr);
    c->launches += 1;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    const uint64_t nq_dead = c->hctr->cl_q, nn = c->hctr->cl_norm, n_dead = c->hctr->cl_dead;
    uint64_t hcap = 64;
    while (hcap < 2 * nn) hcap <<= 1;
    if ((st = ensure(c, c->cl_htab, hcap * sizeof(BubbleEnt))) != BRUNO_OK) return st;
    BubbleEnt *tab = (BubbleEnt *)c->cl_htab.p;
    cudaMemsetAsync(tab, 0, hcap * sizeof(BubbleEnt), c->stream);
    const int gn = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * 8, (nn + TPB - 1) / TPB));
    const int gh = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * 8, (hcap + TPB - 1) / TPB));
    if (nn) {
      k_cl_group<KT><<<gn, TPB, 0, c->stream>>>(norm, nn, tab, hcap, c->dctr);
      k_cl_bubbles<KT><<<gh, TPB, 0, c->stream>>>(norm, tab, hcap, k, min_freq, q, c->dctr);
    }
    c->launches += 2;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    if (c->hctr->err & DERR_INVARIANT) return set_err(c, BRUNO_ERR_INVARIANT, "cleaning: bubble grouping overflowed");
    const uint64_t nq = c->hctr->cl_q, n_bub = c->hctr->cl_bub;
    if (n_dead == 0 && n_bub == 0) break;
    *deadends += n_dead;
    *bubbles += n_bub;
    /* dead ends first, then bubbles, each followed by the removal of edge-less nodes */
    uint64_t erased = 0;
    const uint64_t ranges[2][2] = {{0, nq_dead}, {nq_dead, nq}};
    for (int b = 0; b < 2; ++b) {
      const uint64_t q0 = ranges[b][0], q1 = ranges[b][1];
      cudaMemsetAsync(&c->dctr->cl_found, 0, 8, c->stream);
      const int gq = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * 8, (q1 - q0 + TPB - 1) / TPB));
      if (q1 > q0) k_cl_find<KT><<<gq, TPB, 0, c->stream>>>(q, q0, q1, table, c->geom, k, min_freq, found, c->dctr);
      c->launches += 1;
      if ((st = sync_counters(c)) != BRUNO_OK) return st;
      const uint64_t nf = c->hctr->cl_found;
      const int gf = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * 8, (nf + TPB - 1) / TPB));
      if (nf) k_cl_erase<KT><<<gf, TPB, 0, c->stream>>>(found, nf, table, c->geom, k);
      c->launches += 1;
      erased += nf;
      if ((st = isolated()) != BRUNO_OK) return st;
    }
    *edges += erased;
    ++*rounds;
    if (erased == 0) { *status = 1; break; }   /* the reference would find the same again, forever */
    /* recompaction: classify, rebuild the chain map, rank, take cycles and edge-less nodes out */
    const uint64_t cap = std::max<uint64_t>(1, c->n_slots_claimed);
    cudaMemsetAsync(&c->dctr->n_chain, 0, 8, c->stream);
    cudaMemsetAsync(&c->dctr->n_branch, 0, 8, c->stream);
    cudaMemsetAsync(&c->dctr->err, 0, 8, c->stream);
    k_cl_classify<KT><<<sms * 8, TPB, 0, c->stream>>>(table, c->nslots, k, (uint32_t *)c->chain_list.p,
                                                      (uint32_t *)c->branch_list.p, cap, c->dctr);
    c->launches += 1;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    if (c->hctr->err & DERR_INVARIANT) return set_err(c, BRUNO_ERR_INVARIANT, "cleaning: node lists overflowed");
    c->n_chain = c->hctr->n_chain;
    c->n_branch = c->hctr->n_branch;
    c->n_nodes = c->n_chain + c->n_branch;
    if ((st = extract_typed<KT>(c)) != BRUNO_OK) return st;
    if ((st = run_list_rank(c, c->cfg.min_update)) != BRUNO_OK) return st;
    if ((st = cycles()) != BRUNO_OK) return st;
    (void)iter;
  }
  (void)KWD;
  /* the cleaned graph, compacted; on-demand outputs are rebuilt from it */
  c->general_emission = false;
  c->chain_edges_done = false;
  c->summaries_done = false;
  return compress_typed<KT>(c);
}

}  // namespace

bruno_status run_extract_chains(Ctx *c) { return c->W == 1 ? extract_typed<KW1>(c) : extract_typed<KW2>(c); }

/* The ruling-set ranking; returns false (and changes nothing) if the chain map is not
 * mutually consistent, in which case the round-synchronous path runs. */
static bruno_status fast_list_rank(Ctx *c, bool &used) {
  bruno_status st;
  used = false;
  const uint64_t M = c->n_chain, Mb = std::max<uint64_t>(1, M);
  if (M >= (1ull << 30)) return BRUNO_OK;
  const int sms = sms_count();
  ChainState *cs = (ChainState *)c->cstate.p;
  if ((st = ensure(c, c->unf1, Mb * 4)) != BRUNO_OK) return st;        /* rnode */
  if ((st = ensure(c, c->removed, Mb)) != BRUNO_OK) return st;
  uint32_t *rnode = (uint32_t *)c->unf1.p;
  cudaMemsetAsync(&c->dctr->lr_applied, 0, 32, c->stream);   /* applied, remaining, cycles, multi */
  k_fast_check<<<sms * 8, TPB, 0, c->stream>>>(cs, M, rnode, c->dctr);
  c->launches += 1;
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  if (c->hctr->lr_multi != 0) return BRUNO_OK;                /* inconsistent pointers */
  const uint64_t R = c->hctr->lr_remaining, Rb = std::max<uint64_t>(1, R);
  if ((st = ensure(c, c->pay, Rb * 2 * sizeof(Jump) * 3)) != BRUNO_OK) return st;
  Jump *E0 = (Jump *)c->pay.p, *E = E0 + 2 * Rb, *F = E + 2 * Rb;
  static const int walk_occ = [] {   /* resident walk blocks per SM: the walks run as one wave */
    int o = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_fast_walk, TPB, 0) == cudaSuccess && o > 0 ? o : 4;
  }();
  const int gw = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * walk_occ, (2 * R + TPB - 1) / TPB));
  uint64_t *place = nullptr;
  Buf place_buf;
  struct FreeOnExit {   /* the places go back to the pool on every way out */
    Buf &b; cudaStream_t s;
    ~FreeOnExit() { if (b.p) cudaFreeAsync(b.p, s); }
  } place_guard{place_buf, c->stream};
  if (c->cfg.rank_fill == 1) {   /* two 8-byte places per node, all ones = not on a walked segment */
    if ((st = ensure(c, place_buf, Mb * 16)) != BRUNO_OK) return st;
    place = (uint64_t *)place_buf.p;
    cudaMemsetAsync(place, 0xFF, M * 16, c->stream);
  }
  k_fast_walk<<<gw, TPB, 0, c->stream>>>(cs, rnode, R, M, E0, place, c->dctr);
  c->launches += 1;
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  if (c->hctr->lr_multi != 0) return BRUNO_OK;                /* a pointer not answered by its target */
  const Jump *src = E0;
  uint64_t prev = ~0ull;
  for (int round = 0; round < 64; ++round) {
    cudaMemsetAsync(&c->dctr->lr_applied, 0, 8, c->stream);
    k_fast_jump<<<gw, TPB, 0, c->stream>>>(src, E, R, c->dctr);
    c->launches += 1;
    src = E;
    std::swap(E, F);
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    const uint64_t undone = c->hctr->lr_applied;
    if (undone == 0 || undone == prev) break;   /* only ruler cycles keep sides undone */
    prev = undone;
  }
  /* final states go to a second chain-state array (all ones = unset), which then becomes
   * the chain map; a node left unset is a cycle node, whose state nothing reads again */
  if ((st = ensure(c, c->cstate2, Mb * sizeof(ChainState))) != BRUNO_OK) return st;
  ChainState *cs2 = (ChainState *)c->cstate2.p;
  cudaMemsetAsync(cs2, 0xFF, M * sizeof(ChainState), c->stream);
  if (place) {
    k_fast_place<<<sms * 8, TPB, 0, c->stream>>>(cs, cs2, rnode, M, src, place);
  } else {
    k_fast_fill<<<gw, TPB, 0, c->stream>>>(cs, cs2, rnode, R, E0, src);
  }
  k_fast_rulers<<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * 8, (R + TPB - 1) / TPB)), TPB, 0,
                  c->stream>>>(cs, cs2, rnode, R, src);
  cudaMemsetAsync(&c->dctr->n_cycle, 0, 16, c->stream);
  cudaMemsetAsync(&c->dctr->n_heads, 0, 8, c->stream);        /* longest path, in nodes */
  k_fast_mark<<<sms * 8, TPB, 0, c->stream>>>(cs, cs2, M, (uint8_t *)c->removed.p, &c->dctr->n_heads,
                                               c->S > 1 ? (const uint32_t *)c->csample.p : nullptr,
                                               c->S > 1 ? (unsigned long long *)c->s_tally.p : nullptr, c->dctr);
  c->launches += 3;
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  if (c->hctr->lr_multi != 0) return BRUNO_OK;   /* an unreached node is not on a consistent cycle */
  std::swap(c->cstate, c->cstate2);              /* the final states become the chain map */
  c->n_cycle = c->hctr->n_cycle;
  c->n_isolated = c->hctr->n_isolated;
  const uint64_t nmax = c->hctr->n_heads;
  uint64_t it = 0;
  if (nmax >= 2) { uint64_t x = nmax - 1; while (x >>= 1) ++it; ++it; }  /* floor(log2(nmax-1)) + 1 */
  else if (c->n_cycle > 0) it = 1;
  c->iterations = it;
  c->multi = 0;
  used = true;
  return BRUNO_OK;
}

bruno_status run_list_rank(Ctx *c, int min_update) {
  bruno_status st;
  c->fast_ranked = false;
  if (!c->exact_ranking) {
    bool used = false;
    if ((st = fast_list_rank(c, used)) != BRUNO_OK) return st;
    c->fast_ranked = used;
    if (used) return BRUNO_OK;
  }
  const uint64_t M = c->n_chain, Mb = std::max<uint64_t>(1, M);
  if ((st = ensure(c, c->unf0, Mb * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->unf1, Mb * 4)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->pend, Mb * 16)) != BRUNO_OK) return st;
  if ((st = ensure(c, c->pay, Mb * 2 * sizeof(Payload))) != BRUNO_OK) return st;
  if ((st = ensure(c, c->removed, Mb)) != BRUNO_OK) return st;
  cudaMemsetAsync(c->pend.p, 0, Mb * 16, c->stream);
  cudaMemsetAsync(&c->dctr->lr_remaining, 0, 8, c->stream);
  cudaMemsetAsync(&c->dctr->lr_multi, 0, 8, c->stream);
  const int sms = sms_count();
  ChainState *cs = (ChainState *)c->cstate.p;
  uint32_t *cur = (uint32_t *)c->unf0.p, *nxt = (uint32_t *)c->unf1.p;
  k_lr_init<<<sms * 8, TPB, 0, c->stream>>>(cs, M, cur, &c->dctr->lr_remaining);
  c->launches += 2;  /* k_lr_init, k_separate */
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  uint64_t remaining = c->hctr->lr_remaining;
  bool all_compacted = remaining == 0;
  uint64_t iterations = 0;
  while (!all_compacted) {
    const int g = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * 8, (remaining + TPB - 1) / TPB));
    k_lr_propose<<<g, TPB, 0, c->stream>>>(cs, cur, remaining, min_update, (unsigned long long *)c->pend.p, c->dctr);
    k_lr_commit<<<g, TPB, 0, c->stream>>>(cs, cur, remaining, min_update, (unsigned long long *)c->pend.p,
                                          (Payload *)c->pay.p);
    cudaMemsetAsync(&c->dctr->lr_applied, 0, 24, c->stream);  /* applied, remaining, cycles */
    const uint32_t maxd = 1u << (iterations + 1);
    k_lr_apply<<<g, TPB, 0, c->stream>>>(cs, cur, remaining, (unsigned long long *)c->pend.p, (const Payload *)c->pay.p,
                                         maxd, nxt, c->dctr);
    c->launches += 3;
    if ((st = sync_counters(c)) != BRUNO_OK) return st;
    const uint64_t applied = c->hctr->lr_applied, cycles = c->hctr->lr_cycles;
    remaining = c->hctr->lr_remaining;
    std::swap(cur, nxt);
    ++iterations;
    if (iterations >= 30) all_compacted = true;
    else all_compacted = applied == 0 || cycles == remaining;
  }
  c->iterations = iterations;
  c->multi = c->hctr->lr_multi;
  cudaMemsetAsync(&c->dctr->n_cycle, 0, 16, c->stream);
  k_separate<<<sms * 8, TPB, 0, c->stream>>>(cs, M, remaining > 0 ? 1 : 0, (uint32_t)(1u << iterations),
                                             (uint8_t *)c->removed.p, c->dctr);
  if ((st = sync_counters(c)) != BRUNO_OK) return st;
  c->n_cycle = c->hctr->n_cycle;
  c->n_isolated = c->hctr->n_isolated;
  return BRUNO_OK;
}

bruno_status run_compress(Ctx *c) { return c->W == 1 ? compress_typed<KW1>(c) : compress_typed<KW2>(c); }

bruno_status run_chain_edges(Ctx *c) { return c->W == 1 ? chain_edges_typed<KW1>(c) : chain_edges_typed<KW2>(c); }
bruno_status run_chain_summaries(Ctx *c) {
  return c->W == 1 ? chain_summaries_typed<KW1>(c) : chain_summaries_typed<KW2>(c);
}

bruno_status run_node_query(Ctx *c, int filter, bool erase, uint64_t *keys, uint16_t *counts, uint8_t *flags,
                            size_t cap, size_t *n) {
  bruno_status st = c->W == 1 ? node_query_typed<KW1>(c, filter, erase, keys, counts, flags, cap, n)
                              : node_query_typed<KW2>(c, filter, erase, keys, counts, flags, cap, n);
  if (st != BRUNO_OK || !erase) return st;
  return c->W == 1 ? node_recount_typed<KW1>(c) : node_recount_typed<KW2>(c);
}
bruno_status run_check_index(Ctx *c, bruno_index_check *out) {
  return c->W == 1 ? check_index_typed<KW1>(c, out) : check_index_typed<KW2>(c, out);
}
bruno_status run_erase_nodes(Ctx *c, const uint64_t *kmers, size_t n) {
  return c->W == 1 ? erase_nodes_typed<KW1>(c, kmers, n) : erase_nodes_typed<KW2>(c, kmers, n);
}
bruno_status run_chain_query(Ctx *c, int filter, int which, uint64_t *kmers, uint64_t *inK, uint64_t *outK,
                             uint32_t *inD, uint32_t *outD, size_t cap, size_t *n) {
  return c->W == 1 ? chain_query_typed<KW1>(c, filter, which, kmers, inK, outK, inD, outD, cap, n)
                   : chain_query_typed<KW2>(c, filter, which, kmers, inK, outK, inD, outD, cap, n);
}
bruno_status run_clean(Ctx *c, uint64_t *rounds, uint64_t *deadends, uint64_t *bubbles, uint64_t *edges,
                       int32_t *status) {
  return c->W == 1 ? clean_typed<KW1>(c, rounds, deadends, bubbles, edges, status)
                   : clean_typed<KW2>(c, rounds, deadends, bubbles, edges, status);
}

}  // namespace bg
