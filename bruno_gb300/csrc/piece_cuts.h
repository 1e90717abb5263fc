/*
 * piece_cuts.h -- where a host FASTQ buffer is cut for the piecewise host-to-device copy of
 * bruno_load_fastq.  Host code only (no CUDA), so that it is tested on its own.
 */
#ifndef BRUNO_PIECE_CUTS_H_
#define BRUNO_PIECE_CUTS_H_

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

/* Record starts that cut a host FASTQ buffer into pieces of about `piece` bytes; {0} alone when
 * the buffer is under two pieces.  A cut is the start of a line that begins with '@' and whose
 * second-next line begins with '+': a quality line may begin with '@' as well, but two lines
 * after a quality line comes a sequence, which holds no '+'.  A target with no such line in the
 * MiB after it gets no cut. */
inline std::vector<uint64_t> piece_cuts(const char *buf, uint64_t n, uint64_t piece) {
  std::vector<uint64_t> cuts{0};
  if (piece == 0 || n < 2 * piece) return cuts;
  auto line_end = [&](uint64_t from) -> uint64_t {   /* the newline ending the line at `from`, or n */
    if (from >= n) return n;
    const void *e = std::memchr(buf + from, '\n', n - from);
    return e ? (uint64_t)((const char *)e - buf) : n;
  };
  for (uint64_t target = piece; target + piece / 2 < n; target += piece) {
    const uint64_t limit = std::min<uint64_t>(n, target + (1ull << 20));
    for (uint64_t q = line_end(target) + 1; q < limit; q = line_end(q) + 1) {
      if (buf[q] != '@' || q <= cuts.back()) continue;
      const uint64_t e1 = line_end(q);
      if (e1 >= n) break;
      const uint64_t e2 = line_end(e1 + 1);
      if (e2 + 1 < n && buf[e2 + 1] == '+') { cuts.push_back(q); break; }
    }
  }
  return cuts;
}

#endif /* BRUNO_PIECE_CUTS_H_ */
