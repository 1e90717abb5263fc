/*
 * table_plan.h -- how the k-mer table is cut into shared-memory partitions and how the
 * counting work is laid over them, as pure host functions so that the rules are tested on
 * their own.
 *
 * A table of `slots` slots is 2^pbits partitions of `region` slots (pbits >= 8: the 256 hash
 * buckets, then split bits).  The plan takes the fewest partitions whose region fits one CTA's
 * shared memory (`max_region` slots), with at least 64 slots a region.  The records of a table
 * with more split bits than k_split's counting sort handles are scattered straight into the
 * table regions; that scatter interleaves as many buckets as give 8192 partition cursors (one
 * bucket for large tables), and counts each bucket's 32-record runs up to a power of two so
 * that a run's bucket and place come from shifts.  A batch launches its partitions by region
 * size, in classes a factor of about 1.5 apart.
 */
#ifndef BRUNO_TABLE_PLAN_H_
#define BRUNO_TABLE_PLAN_H_

#include <algorithm>
#include <cstdint>

namespace bruno_table_plan {

constexpr int BUCKET_BITS = 8;

struct Plan {
  int pbits;        /* log2 of the partitions */
  uint64_t region;  /* slots a partition */
  bool fits;        /* region <= max_region (false: even 8 + max_split bits leave it larger) */
};

inline Plan partitions(uint64_t slots, uint64_t max_region, int max_split) {
  int pb = BUCKET_BITS;
  while (pb < BUCKET_BITS + max_split && (slots + (1ull << pb) - 1) >> pb > max_region) ++pb;
  const uint64_t region = std::max<uint64_t>(64, (slots + (1ull << pb) - 1) >> pb);
  return Plan{pb, region, region <= max_region};
}

/* log2 of the buckets the scatter split interleaves: enough for 8192 partition cursors */
inline int scatter_lg_window(int pbits) {
  int lg = 0;
  while (lg < BUCKET_BITS && (1ull << (lg + pbits - BUCKET_BITS)) < 8192) ++lg;
  return lg;
}

/* log2 of a bucket's 32-record runs, counted up to a power of two (cap records a bucket) */
inline int scatter_lg_runs(uint64_t cap) {
  int lg = 0;
  while ((1ull << lg) * 32 < cap) ++lg;
  return lg;
}

/* the batch's region classes: class c holds the regions in (bound[c - 1], bound[c]] */
constexpr int REGION_CLASSES = 10;
inline uint64_t region_class_bound(int c) {
  static const uint64_t bound[REGION_CLASSES] = {128, 192, 256, 384, 512, 768, 1024, 1536, 2048, ~0ull};
  return bound[c];
}
inline int region_class(uint64_t region) {
  int c = 0;
  while (region > region_class_bound(c)) ++c;
  return c;
}

}  // namespace bruno_table_plan

#endif  // BRUNO_TABLE_PLAN_H_
