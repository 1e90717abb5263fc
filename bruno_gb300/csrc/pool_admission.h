/*
 * pool_admission.h -- the admission rule of the build pool (pool.cu), as pure host functions
 * over the pool's per-worker tallies, so that it is tested on its own.
 *
 * A worker keeps its context's buffers between requests, so per worker the pool tracks the
 * largest estimate it has run (`held`) and whether it is running one (`busy`).  A request goes
 * to free worker w while the sum over workers -- w counted at the larger of what it holds and
 * the request's estimate -- stays within the budget, or when no other worker is busy (a request
 * larger than the budget then runs alone).  A request that ran out of memory beside others once
 * (`solo`) waits until no other worker is busy, and while it runs (`solo_running`) no other
 * request is admitted, so that it really runs alone.
 */
#ifndef BRUNO_POOL_ADMISSION_H_
#define BRUNO_POOL_ADMISSION_H_

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace bruno_pool_rules {

/* device memory a build of an n-byte FASTQ may hold: 20 bytes a FASTQ byte plus 64 MiB */
inline uint64_t estimate(size_t n) { return 20ull * n + (64ull << 20); }

/* may worker w take a request of estimate `est` now? */
inline bool admits(const std::vector<uint64_t> &held, const std::vector<bool> &busy, uint64_t budget, int w,
                   uint64_t est, bool solo, bool solo_running = false) {
  if (solo_running) return false;
  uint64_t sum = 0;
  bool others_busy = false;
  for (size_t i = 0; i < held.size(); ++i) {
    sum += (int)i == w ? std::max(held[i], est) : held[i];
    if ((int)i != w && busy[i]) others_busy = true;
  }
  if (solo) return !others_busy;
  return sum <= budget || !others_busy;
}

/* should idle worker w free its buffers so that the queue head (estimate est) fits?  Only
 * when no free worker could take it as things stand. */
inline bool should_trim(const std::vector<uint64_t> &held, const std::vector<bool> &busy, uint64_t budget, int w,
                        uint64_t est, bool solo, bool solo_running = false) {
  if (solo_running || busy[w] || held[w] == 0) return false;
  for (size_t i = 0; i < held.size(); ++i)
    if (!busy[i] && admits(held, busy, budget, (int)i, est, solo)) return false;
  return true;
}

}  // namespace bruno_pool_rules

#endif /* BRUNO_POOL_ADMISSION_H_ */
