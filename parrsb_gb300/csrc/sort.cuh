// sort.cuh -- segmented stable LSD radix sort of (uint64 key, int payload).
#pragma once
#include "common.cuh"

namespace prsb {

typedef unsigned long long u64;
typedef unsigned int u32;

// Workspace reused across calls (grown on demand).
struct SortWs {
  DBuf<u64> ktmp;
  DBuf<int> vtmp;
  DBuf<u32> counts;     // [256][ntiles]
  DBuf<u32> totals;     // [256]
  DBuf<u32> hist_all;   // [npass][256]
};

// Sort pairs (keys[i], vals[i]), i < n, stably by (seg_of_val[vals[i]], key).
// seg_of_val may be null (one segment); nseg is the number of segments
// (segment ids must lie in [0, nseg)).  On return *keys / *vals point at the
// sorted arrays, which are either the inputs or the workspace buffers (the
// pointers are swapped with ws buffers as needed; the caller's DBufs are
// swapped correspondingly).
void seg_sort_pairs(DBuf<u64> &keys, DBuf<int> &vals, ll n,
                    const int *seg_of_val, ll nseg, SortWs &ws);

}  // namespace prsb
